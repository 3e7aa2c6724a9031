/* fma_probe_main.c -- test infrastructure: drives probe_reduced_sum (built
 * with the reference's flags) on random pairs and reports which float64
 * accumulation it reproduces: "separate" (total + t*t, two roundings) or
 * "fused" (fma(t, t, total)).  Built with -ffp-contract=off so that both
 * references are computed exactly as written. */
#include <math.h>
#include <stdio.h>
#include <stdint.h>

typedef double (*component_fn)(const double *data, long index);
double probe_reduced_sum(const double *a, const double *b, long n_dim, component_fn get);

static double get_component(const double *data, long index) { return data[index]; }

static uint64_t state = 88172645463325252ull;
static double next_unit(void) {
    state ^= state << 13;
    state ^= state >> 7;
    state ^= state << 17;
    return (double)(state >> 11) * (1.0 / 9007199254740992.0);
}

int main(void) {
    long differ = 0, sep = 0, fus = 0;
    for (int t = 0; t < 200000; ++t) {
        double a[3], b[3];
        for (int k = 0; k < 3; ++k) {
            a[k] = next_unit();
            b[k] = next_unit();
        }
        double s_sep = 0, s_fus = 0;
        for (int k = 0; k < 3; ++k) {
            double d = a[k] - b[k];
            double sq = d * d;
            s_sep = s_sep + sq;
            s_fus = fma(d, d, s_fus);
        }
        double r = probe_reduced_sum(a, b, 3, get_component);
        if (s_sep != s_fus) {
            ++differ;
            sep += r == s_sep;
            fus += r == s_fus;
        }
    }
    const char *mode = differ == 0 ? "undecided" : sep == differ ? "separate" : fus == differ ? "fused" : "mixed";
    printf("%s %ld %ld %ld\n", mode, differ, sep, fus);
    return 0;
}
