// fma_probe_sum.cpp -- test infrastructure: the distance loop of
// MetricExtEuclideanReduced._calc_distance (src/cnnclustering/_types.pyx:
// 2253-2267) in the shape Cython gives it -- `total += cpow(a - b, 2)` with
// the components fetched through an opaque call (the reference reads them
// through InputDataExtInterface._get_component, a vtable call).  It is
// compiled with the reference's own build flags (oracle/fma_probe.py) to
// learn whether that build fuses the multiply-add on this host.
#include <cmath>

typedef double (*component_fn)(const double *data, long index);

extern "C" double probe_reduced_sum(const double *a, const double *b, long n_dim, component_fn get) {
    double total = 0;
    for (long i = 0; i < n_dim; ++i) {
        double x = get(a, i);
        double y = get(b, i);
        total += pow(x - y, 2);
    }
    return total;
}
