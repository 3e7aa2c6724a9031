/*
 * cnn_oracle.c -- CPU restatement of the CommonNN fit path of cnnclustering 0.5.0.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle that the CUDA library is
 * checked against.  Only the tests, the smoke check and the CPU-baseline legs
 * of bench.py load it.  The library never links, calls or falls back to it.
 *
 * Every function restates one reference function; the citation names the
 * reference file and lines (paths relative to the reference project root).
 *
 *   oracle_sqdist            MetricExtEuclideanReduced._calc_distance
 *                              src/cnnclustering/_types.pyx:2253-2267
 *                            (the Euclidean metric is sqrt of the same sum,
 *                              src/cnnclustering/_types.pyx:2173-2187)
 *   oracle_in_radius         NeighboursGetterExtBruteForce._get predicate
 *                              src/cnnclustering/_types.pyx:1692-1710
 *   oracle_neighbour_counts/ brute-force neighbourhoods, one row per point in
 *   oracle_neighbour_fill      index order, self included (is_selfcounting,
 *                              src/cnnclustering/_types.pyx:1676-1678)
 *   oracle_check_sorted      SimilarityCheckerExtScreensorted._check
 *                              src/cnnclustering/_types.pyx:2654-2706
 *   oracle_fit_bfs_csr       FitterExtBFS._fit over precomputed sorted lists
 *                              src/cnnclustering/_fit.pyx:408-491 with
 *                              NeighboursGetterExtLookup._get :1806-1817,
 *                              NeighboursExtVector._enough :1408-1411 and
 *                              QueueExtFIFOQueue :2802-2819
 *   oracle_fit_bfs_points    FitterExtBFS._fit with the default "coordinates"
 *                              recipe (brute-force getter, recomputed per
 *                              query), src/cnnclustering/recipes.py:318-328
 *
 * Floating point.  The reference sums (a-b)^2 over the dimensions in order,
 * starting from 0.0, and compares with pow(r, 2) (_types.pyx:2286-2287).
 * GCC folds pow(x, 2.0) into x*x.  Whether `total + t*t` is contracted into
 * one fused multiply-add depends on the target the reference was compiled
 * for (x86-64 baseline: two roundings; aarch64 default -ffp-contract=fast:
 * one rounding).  Both are offered as `fpmode` (0 = separate multiply and
 * add, 1 = fused).  This file is compiled with -ffp-contract=off so the
 * compiler does not change the chosen mode.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <pthread.h>

#define ORACLE_METRIC_EUCLIDEAN_REDUCED 0
#define ORACLE_METRIC_EUCLIDEAN 1

/* _types.pyx:2253-2267: total = 0; for i in dims: total += (a - b)^2 */
double oracle_sqdist(const double *xa, const double *xb, int32_t d, int fpmode)
{
    double total = 0.0;
    for (int32_t k = 0; k < d; ++k) {
        double t = xa[k] - xb[k];
        if (fpmode) {
            total = fma(t, t, total);
        } else {
            double sq = t * t;
            total = total + sq;
        }
    }
    return total;
}

/* The brute-force getter keeps i when distance <= radius_cutoff
 * (_types.pyx:1709).  radius_cutoff is the value after
 * Metric.adjust_radius: r*r for the reduced metric (_types.pyx:2286-2287),
 * r itself for the Euclidean metric (_types.pyx:2189-2190). */
static inline int oracle_in_radius(const double *xa, const double *xb, int32_t d,
                                   double radius_cutoff, int metric, int fpmode)
{
    double s = oracle_sqdist(xa, xb, d, fpmode);
    if (metric == ORACLE_METRIC_EUCLIDEAN) s = sqrt(s);
    return s <= radius_cutoff;
}

/* ------------------------------------------------------------------ */
/* Neighbourhoods (brute force, rows in parallel over host threads).   */
/* ------------------------------------------------------------------ */

typedef struct {
    const double *x;
    int64_t n;
    int32_t d;
    double radius_cutoff;
    int metric;
    int fpmode;
    int64_t row_begin, row_end;
    int64_t *counts;         /* count pass */
    const int64_t *offsets;  /* fill pass */
    int32_t *indices;
} nb_job;

static void *nb_count_worker(void *arg)
{
    nb_job *j = (nb_job *)arg;
    for (int64_t p = j->row_begin; p < j->row_end; ++p) {
        const double *xp = j->x + p * j->d;
        int64_t c = 0;
        for (int64_t i = 0; i < j->n; ++i)
            c += oracle_in_radius(xp, j->x + i * j->d, j->d, j->radius_cutoff, j->metric, j->fpmode);
        j->counts[p] = c;
    }
    return NULL;
}

static void *nb_fill_worker(void *arg)
{
    nb_job *j = (nb_job *)arg;
    for (int64_t p = j->row_begin; p < j->row_end; ++p) {
        const double *xp = j->x + p * j->d;
        int64_t w = j->offsets[p];
        for (int64_t i = 0; i < j->n; ++i)
            if (oracle_in_radius(xp, j->x + i * j->d, j->d, j->radius_cutoff, j->metric, j->fpmode))
                j->indices[w++] = (int32_t)i;
    }
    return NULL;
}

static int run_rows(void *(*fn)(void *), nb_job *tmpl, int nthreads)
{
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    if (tmpl->n < (int64_t)nthreads) nthreads = tmpl->n > 0 ? (int)tmpl->n : 1;
    nb_job jobs[256];
    pthread_t th[256];
    /* interleave rows in blocks so dense and sparse regions spread out */
    int64_t chunk = (tmpl->n + nthreads - 1) / nthreads;
    for (int t = 0; t < nthreads; ++t) {
        jobs[t] = *tmpl;
        jobs[t].row_begin = (int64_t)t * chunk;
        jobs[t].row_end = jobs[t].row_begin + chunk;
        if (jobs[t].row_end > tmpl->n) jobs[t].row_end = tmpl->n;
        if (jobs[t].row_begin > tmpl->n) jobs[t].row_begin = tmpl->n;
    }
    for (int t = 1; t < nthreads; ++t)
        if (pthread_create(&th[t], NULL, fn, &jobs[t]) != 0) return -1;
    fn(&jobs[0]);
    for (int t = 1; t < nthreads; ++t) pthread_join(th[t], NULL);
    return 0;
}

/* counts[p] = |N(p)| (self included). */
int oracle_neighbour_counts(const double *x, int64_t n, int32_t d, double radius_cutoff,
                            int metric, int fpmode, int nthreads, int64_t *counts)
{
    nb_job t = {x, n, d, radius_cutoff, metric, fpmode, 0, n, counts, NULL, NULL};
    return run_rows(nb_count_worker, &t, nthreads);
}

/* indices[offsets[p] .. offsets[p+1]) = N(p) in ascending index order. */
int oracle_neighbour_fill(const double *x, int64_t n, int32_t d, double radius_cutoff,
                          int metric, int fpmode, int nthreads, const int64_t *offsets,
                          int32_t *indices)
{
    nb_job t = {x, n, d, radius_cutoff, metric, fpmode, 0, n, NULL, offsets, indices};
    return run_rows(nb_fill_worker, &t, nthreads);
}

/* One query row by brute force (_types.pyx:1692-1710 for a single index):
 * writes the ascending indices i with predicate(query, x_i) into out and
 * returns their number. */
int64_t oracle_neighbour_row(const double *x, int64_t n, int32_t d, const double *query,
                             double radius_cutoff, int metric, int fpmode, int32_t *out)
{
    int64_t c = 0;
    for (int64_t i = 0; i < n; ++i)
        if (oracle_in_radius(query, x + i * d, d, radius_cutoff, metric, fpmode)) out[c++] = (int32_t)i;
    return c;
}

/* ------------------------------------------------------------------ */
/* Similarity check: two-pointer merge with early exit.                */
/* ------------------------------------------------------------------ */

/* _types.pyx:2654-2706.  Returns 1 when the sorted lists share at least
 * `c` members; c == 0 is always true; an empty list is false. */
int oracle_check_sorted(const int32_t *a, int64_t na, const int32_t *b, int64_t nb, int64_t c)
{
    if (c == 0) return 1;
    if (na == 0 || nb == 0) return 0;
    int64_t ia = 0, ib = 0, common = 0;
    int32_t ma = a[0], mb = b[0];
    for (;;) {
        if (ma == mb) {
            common += 1;
            if (common == c) return 1;
            ia += 1; ib += 1;
            if (ia == na || ib == nb) break;
            ma = a[ia]; mb = b[ib];
            continue;
        }
        if (ma < mb) {
            ia += 1;
            if (ia == na) break;
            ma = a[ia];
            continue;
        }
        ib += 1;
        if (ib == nb) break;
        mb = b[ib];
    }
    return 0;
}

/* Full count without early exit (SimilarityCheckerExtScreensorted._get,
 * _types.pyx:2708-2753). */
int64_t oracle_count_common_sorted(const int32_t *a, int64_t na, const int32_t *b, int64_t nb)
{
    int64_t ia = 0, ib = 0, common = 0;
    while (ia < na && ib < nb) {
        if (a[ia] == b[ib]) { ++common; ++ia; ++ib; }
        else if (a[ia] < b[ib]) ++ia;
        else ++ib;
    }
    return common;
}

/* ------------------------------------------------------------------ */
/* BFS fitter (_fit.pyx:408-491).                                      */
/* ------------------------------------------------------------------ */

/* Fixed-capacity FIFO ring (the queue never holds more than n members,
 * since a member is pushed only once: it is marked consider=0 first). */
typedef struct { int64_t *buf; int64_t cap, head, tail, size; } fifo;

static void fifo_push(fifo *q, int64_t v) { q->buf[q->tail] = v; q->tail = (q->tail + 1) % q->cap; q->size++; }
static int64_t fifo_pop(fifo *q) { int64_t v = q->buf[q->head]; q->head = (q->head + 1) % q->cap; q->size--; return v; }

/* FitterExtBFS._fit with NeighboursGetterExtLookup(is_sorted=True) over a
 * CSR (offsets int64[n+1], indices int32[nnz], rows ascending),
 * NeighboursExtVector containers, SimilarityCheckerExtScreensorted and the
 * FIFO queue.  labels/consider are updated in place exactly as the
 * reference does (_fit.pyx:428-491).  Returns the number of similarity
 * checks executed, or -1 on allocation failure. */
int64_t oracle_fit_bfs_csr(const int64_t *offsets, const int32_t *indices, int64_t n,
                           int64_t similarity_cutoff, int64_t n_member_cutoff,
                           int64_t current_start, uint8_t *consider, int64_t *labels)
{
    fifo q;
    q.cap = n > 0 ? n : 1;
    q.buf = (int64_t *)malloc(sizeof(int64_t) * (size_t)q.cap);
    if (!q.buf) return -1;
    q.head = q.tail = q.size = 0;
    int64_t current = current_start, n_checks = 0;

    for (int64_t init_point = 0; init_point < n; ++init_point) {
        if (consider[init_point] == 0) continue;
        consider[init_point] = 0;
        int64_t pa = init_point;
        int64_t na = offsets[pa + 1] - offsets[pa];
        if (!(na > n_member_cutoff)) continue;          /* _enough: strict > */
        labels[init_point] = current;
        for (;;) {
            const int32_t *la = indices + offsets[pa];
            for (int64_t mi = 0; mi < na; ++mi) {
                int64_t member = la[mi];
                if (consider[member] == 0) continue;
                int64_t nb = offsets[member + 1] - offsets[member];
                if (!(nb > n_member_cutoff)) { consider[member] = 0; continue; }
                n_checks++;
                if (oracle_check_sorted(la, na, indices + offsets[member], nb, similarity_cutoff)) {
                    consider[member] = 0;
                    labels[member] = current;
                    fifo_push(&q, member);
                }
            }
            if (q.size == 0) break;
            pa = fifo_pop(&q);
            na = offsets[pa + 1] - offsets[pa];
        }
        current += 1;
    }
    free(q.buf);
    return n_checks;
}

/* The same fitter with the default "coordinates" recipe: every neighbour
 * query is a brute-force scan over all points (_types.pyx:1692-1710), as
 * the reference does it.  O(n^2 d) per fit.  Neighbour lists come out in
 * index order, so the screensorted merge gives the same boolean as the
 * reference's default switch/unordered-set check (_types.pyx:2580-2610):
 * both count |N(a) & N(b)| and stop at the cutoff. */
int64_t oracle_fit_bfs_points(const double *x, int64_t n, int32_t d, double radius_cutoff,
                              int metric, int fpmode, int64_t similarity_cutoff,
                              int64_t n_member_cutoff, int64_t current_start,
                              uint8_t *consider, int64_t *labels)
{
    int32_t *na_buf = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
    int32_t *nb_buf = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
    fifo q;
    q.cap = n > 0 ? n : 1;
    q.buf = (int64_t *)malloc(sizeof(int64_t) * (size_t)q.cap);
    if (!na_buf || !nb_buf || !q.buf) { free(na_buf); free(nb_buf); free(q.buf); return -1; }
    q.head = q.tail = q.size = 0;
    int64_t current = current_start, n_checks = 0;

#define GET_ROW(point, buf, cnt)                                                        \
    do {                                                                                \
        const double *xp_ = x + (int64_t)(point) * d;                                  \
        cnt = 0;                                                                        \
        for (int64_t i_ = 0; i_ < n; ++i_)                                              \
            if (oracle_in_radius(xp_, x + i_ * d, d, radius_cutoff, metric, fpmode))    \
                buf[cnt++] = (int32_t)i_;                                               \
    } while (0)

    for (int64_t init_point = 0; init_point < n; ++init_point) {
        if (consider[init_point] == 0) continue;
        consider[init_point] = 0;
        int64_t na, nb;
        GET_ROW(init_point, na_buf, na);
        if (!(na > n_member_cutoff)) continue;
        labels[init_point] = current;
        for (;;) {
            for (int64_t mi = 0; mi < na; ++mi) {
                int64_t member = na_buf[mi];
                if (consider[member] == 0) continue;
                GET_ROW(member, nb_buf, nb);
                if (!(nb > n_member_cutoff)) { consider[member] = 0; continue; }
                n_checks++;
                if (oracle_check_sorted(na_buf, na, nb_buf, nb, similarity_cutoff)) {
                    consider[member] = 0;
                    labels[member] = current;
                    fifo_push(&q, member);
                }
            }
            if (q.size == 0) break;
            int64_t point = fifo_pop(&q);
            GET_ROW(point, na_buf, na);
        }
        current += 1;
    }
#undef GET_ROW
    free(na_buf); free(nb_buf); free(q.buf);
    return n_checks;
}

/* ------------------------------------------------------------------ */
/* Grid-accelerated neighbourhoods for d <= 3 (same predicate).        */
/* ------------------------------------------------------------------ */
/* The neighbour SET is defined by the predicate alone, so enumerating
 * candidates from a cell grid instead of all points changes nothing as
 * long as every pair that can pass the predicate lies in adjacent cells.
 * Cells have edge h = R (1 + 1e-6), R the search radius; a pair that
 * passes has |dx_k| <= R (1 + ~d 2^-52) < h in every dimension, so its
 * cell indices differ by at most one.  Rows are sorted before they are
 * written.  Used to make oracle neighbourhoods cheap at 10^5-10^6 points;
 * tests check it against the brute-force restatement above. */

typedef struct { uint64_t key; int32_t idx; } grid_entry;

static int cmp_grid_entry(const void *a, const void *b)
{
    const grid_entry *x = (const grid_entry *)a, *y = (const grid_entry *)b;
    if (x->key != y->key) return x->key < y->key ? -1 : 1;
    return (x->idx > y->idx) - (x->idx < y->idx);
}

static int cmp_i32(const void *a, const void *b)
{
    int32_t x = *(const int32_t *)a, y = *(const int32_t *)b;
    return (x > y) - (x < y);
}

typedef struct {
    const double *x; int64_t n; int32_t d; double radius_cutoff; int metric; int fpmode;
    const grid_entry *sorted; double lo[3]; double h; int64_t gdim[3];
    int64_t row_begin, row_end; int64_t *counts; const int64_t *offsets; int32_t *indices;
} grid_job;

static inline uint64_t grid_key(int64_t c0, int64_t c1, int64_t c2)
{
    return ((uint64_t)c0 << 42) | ((uint64_t)c1 << 21) | (uint64_t)c2;
}

static inline int64_t grid_cell(double v, double lo, double h, int64_t g)
{
    int64_t c = (int64_t)floor((v - lo) / h);
    if (c < 0) c = 0;
    if (c >= g) c = g - 1;
    return c;
}

static int64_t lower_bound_key(const grid_entry *s, int64_t n, uint64_t key)
{
    int64_t lo = 0, hi = n;
    while (lo < hi) {
        int64_t mid = lo + (hi - lo) / 2;
        if (s[mid].key < key) lo = mid + 1; else hi = mid;
    }
    return lo;
}

static void *grid_worker(void *arg)
{
    grid_job *j = (grid_job *)arg;
    int32_t *tmp = (int32_t *)malloc(sizeof(int32_t) * (size_t)(j->n > 0 ? j->n : 1));
    if (!tmp) return (void *)1;
    for (int64_t p = j->row_begin; p < j->row_end; ++p) {
        const double *xp = j->x + p * j->d;
        int64_t c[3] = {0, 0, 0};
        for (int k = 0; k < j->d; ++k) c[k] = grid_cell(xp[k], j->lo[k], j->h, j->gdim[k]);
        int64_t cnt = 0;
        for (int64_t a = c[0] - 1; a <= c[0] + 1; ++a) {
            if (a < 0 || a >= j->gdim[0]) continue;
            for (int64_t b = c[1] - 1; b <= c[1] + 1; ++b) {
                if (b < 0 || b >= j->gdim[1]) continue;
                for (int64_t e = c[2] - 1; e <= c[2] + 1; ++e) {
                    if (e < 0 || e >= j->gdim[2]) continue;
                    uint64_t key = grid_key(a, b, e);
                    int64_t s = lower_bound_key(j->sorted, j->n, key);
                    for (; s < j->n && j->sorted[s].key == key; ++s) {
                        int32_t i = j->sorted[s].idx;
                        if (oracle_in_radius(xp, j->x + (int64_t)i * j->d, j->d, j->radius_cutoff, j->metric, j->fpmode))
                            tmp[cnt++] = i;
                    }
                }
            }
        }
        if (j->counts) {
            j->counts[p] = cnt;
        } else {
            qsort(tmp, (size_t)cnt, sizeof(int32_t), cmp_i32);
            memcpy(j->indices + j->offsets[p], tmp, sizeof(int32_t) * (size_t)cnt);
        }
    }
    free(tmp);
    return NULL;
}

/* Returns 0 on success, 1 if the grid cannot be used (caller falls back to
 * brute force), -1 on allocation failure. */
static int grid_run(const double *x, int64_t n, int32_t d, double radius_cutoff, int metric,
                    int fpmode, int nthreads, int64_t *counts, const int64_t *offsets, int32_t *indices)
{
    if (d < 1 || d > 3 || n < 1) return 1;
    double R = metric == ORACLE_METRIC_EUCLIDEAN ? radius_cutoff : sqrt(radius_cutoff);
    if (!(R > 0) || !isfinite(R)) return 1;
    double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    for (int k = 0; k < d; ++k) { lo[k] = x[k]; hi[k] = x[k]; }
    for (int64_t p = 0; p < n; ++p)
        for (int k = 0; k < d; ++k) {
            double v = x[p * d + k];
            if (!isfinite(v)) return 1;
            if (v < lo[k]) lo[k] = v;
            if (v > hi[k]) hi[k] = v;
        }
    double h = R * (1.0 + 1e-6);
    int64_t gdim[3] = {1, 1, 1};
    for (int k = 0; k < d; ++k) {
        double g = floor((hi[k] - lo[k]) / h) + 1.0;
        if (g > (double)(1 << 20)) return 1;
        gdim[k] = (int64_t)g;
    }
    grid_entry *sorted = (grid_entry *)malloc(sizeof(grid_entry) * (size_t)n);
    if (!sorted) return -1;
    for (int64_t p = 0; p < n; ++p) {
        int64_t c[3] = {0, 0, 0};
        for (int k = 0; k < d; ++k) c[k] = grid_cell(x[p * d + k], lo[k], h, gdim[k]);
        sorted[p].key = grid_key(c[0], c[1], c[2]);
        sorted[p].idx = (int32_t)p;
    }
    qsort(sorted, (size_t)n, sizeof(grid_entry), cmp_grid_entry);

    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    if (n < nthreads) nthreads = (int)n;
    grid_job jobs[256];
    pthread_t th[256];
    int64_t chunk = (n + nthreads - 1) / nthreads;
    for (int t = 0; t < nthreads; ++t) {
        grid_job g = {x, n, d, radius_cutoff, metric, fpmode, sorted, {lo[0], lo[1], lo[2]}, h,
                      {gdim[0], gdim[1], gdim[2]}, 0, 0, counts, offsets, indices};
        g.row_begin = (int64_t)t * chunk;
        g.row_end = g.row_begin + chunk > n ? n : g.row_begin + chunk;
        if (g.row_begin > n) g.row_begin = n;
        jobs[t] = g;
    }
    int rc = 0;
    for (int t = 1; t < nthreads; ++t)
        if (pthread_create(&th[t], NULL, grid_worker, &jobs[t]) != 0) rc = -1;
    if (grid_worker(&jobs[0]) != NULL) rc = -1;
    for (int t = 1; t < nthreads; ++t) {
        void *r = NULL;
        pthread_join(th[t], &r);
        if (r != NULL) rc = -1;
    }
    free(sorted);
    return rc;
}

int oracle_neighbour_counts_grid(const double *x, int64_t n, int32_t d, double radius_cutoff,
                                 int metric, int fpmode, int nthreads, int64_t *counts)
{
    int rc = grid_run(x, n, d, radius_cutoff, metric, fpmode, nthreads, counts, NULL, NULL);
    if (rc == 1) return oracle_neighbour_counts(x, n, d, radius_cutoff, metric, fpmode, nthreads, counts);
    return rc;
}

int oracle_neighbour_fill_grid(const double *x, int64_t n, int32_t d, double radius_cutoff,
                               int metric, int fpmode, int nthreads, const int64_t *offsets,
                               int32_t *indices)
{
    int rc = grid_run(x, n, d, radius_cutoff, metric, fpmode, nthreads, NULL, offsets, indices);
    if (rc == 1) return oracle_neighbour_fill(x, n, d, radius_cutoff, metric, fpmode, nthreads, offsets, indices);
    return rc;
}

/* ------------------------------------------------------------------ */
/* Periodic metric: MetricExtEuclideanPeriodicReduced._calc_distance   */
/* (_types.pyx:2303-2325): per dimension d = |a - b|; when bound > 0,  */
/* d = fmod(d, bound) and d = bound - d if d > bound / 2; total += d^2 */
/* (separate or fused, like the plain metric).                         */
/* ------------------------------------------------------------------ */
double oracle_periodic_sqdist(const double *xa, const double *xb, int32_t d, const double *bounds, int fpmode)
{
    double total = 0.0;
    for (int32_t k = 0; k < d; ++k) {
        double t = fabs(xa[k] - xb[k]);
        const double bound = bounds[k];
        if (bound > 0) {
            t = fmod(t, bound);
            if (t > bound / 2) t = bound - t;
        }
        total = fpmode == 1 ? fma(t, t, total) : total + t * t;
    }
    return total;
}

/* Row of `query` among the n points under the periodic metric (ascending). */
int64_t oracle_periodic_row(const double *x, int64_t n, int32_t d, const double *bounds, const double *query,
                            double radius_cutoff, int fpmode, int32_t *out)
{
    int64_t c = 0;
    for (int64_t i = 0; i < n; ++i)
        if (oracle_periodic_sqdist(query, x + i * d, d, bounds, fpmode) <= radius_cutoff) out[c++] = (int32_t)i;
    return c;
}
