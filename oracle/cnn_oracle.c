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
 *   oracle_pivot_run/_take   the same rows with an exact pivot prune
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
/* Brute force with an exact pivot prune (high dimension, many points) */
/* ------------------------------------------------------------------ */
/* The predicate of oracle_neighbour_counts/fill, evaluated on fewer pairs.
 * Shortcuts that cannot change a row:
 *  - the float64 sum only grows (every term is >= 0 and rounding is
 *    monotone), so a partial sum above the cutoff already means "out";
 *  - triangle inequality, groups: points are grouped by their nearest of P
 *    group pivots; with rad(G) the largest distance of a member of G to its
 *    pivot g, no pair of G x H is closer than dist(g, h) - rad(G) - rad(H),
 *    so group pairs above the radius are skipped;
 *  - triangle inequality, pairs: with D(i, q) the distance to each of Q
 *    bound pivots, |D(i,q) - D(p,q)| <= dist(i, p) skips single pairs.
 * Every bound carries a relative margin of 1e-6, far above the rounding of
 * the pivot distances and of the reference's own sum.  One pass: rows are
 * gathered per thread, sorted ascending and handed out by
 * oracle_pivot_take.  Finite coordinates only (-2: use the plain scan). */

enum { kBoundPivots = 8 };

typedef struct { int32_t *buf; int64_t len, cap; } pv_buf;

typedef struct {
    const double *x;
    int64_t n;
    int32_t d, P, Q;
    double radius_cutoff, exit_above, reach;
    int metric, fpmode;
    int32_t *grp;      /* [n] group of each point (point order) */
    double *od;        /* [n] distance to its group pivot (point order) */
    double *bq;        /* [n][Q] distances to the bound pivots, group order */
    double *xs;        /* [n][d] coordinates, group order */
    int32_t *idx;      /* group order -> point index */
    int64_t *gstart;   /* [P + 1] */
    double *rad;       /* [P] */
    double *pp;        /* [P][P] pivot-pivot distances */
    int64_t *row_len;  /* [n] by point index */
    int64_t *row_start;/* [n] start in the writing thread's buffer */
    int32_t *row_tid;  /* [n] the writing thread */
    int phase;         /* 0: groups and bounds per point, 1: pivot pairs, 2: rows */
    int64_t next, total, block;
    pthread_mutex_t mu;
    int failed;
} pv_state;

static pv_state *g_pivot;  /* the result of the last oracle_pivot_run */
static pv_buf *g_pivot_bufs;
static int g_pivot_nbufs;

/* The reference predicate, stopped as soon as the growing sum passes
 * exit_above (past it the final sum cannot be within the cutoff). */
static inline int in_radius_early(const double *xa, const double *xb, int32_t d, double radius_cutoff,
                                  double exit_above, int metric, int fpmode)
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
        if (total > exit_above) return 0;
    }
    if (metric == ORACLE_METRIC_EUCLIDEAN) total = sqrt(total);
    return total <= radius_cutoff;
}

static double plain_dist(const double *a, const double *b, int32_t d)
{
    double t = 0;
    for (int32_t k = 0; k < d; ++k) t += (a[k] - b[k]) * (a[k] - b[k]);
    return sqrt(t);
}

static int pv_push(pv_buf *b, int32_t v)
{
    if (b->len == b->cap) {
        int64_t cap = b->cap ? 2 * b->cap : 1 << 20;
        int32_t *nb = (int32_t *)realloc(b->buf, sizeof(int32_t) * (size_t)cap);
        if (!nb) return -1;
        b->buf = nb;
        b->cap = cap;
    }
    b->buf[b->len++] = v;
    return 0;
}

typedef struct { pv_state *S; pv_buf *out; int32_t tid; } pv_arg;

static int pv_rows_of_group(pv_state *S, int64_t G, pv_buf *out, int32_t tid, int32_t *near)
{
    const int32_t P = S->P, Q = S->Q, d = S->d;
    const double reach = S->reach * (1.0 + 1e-6);
    int32_t nh = 0;
    for (int32_t H = 0; H < P; ++H) {
        if (S->gstart[H] == S->gstart[H + 1]) continue;
        const double gap = S->pp[G * P + H] - S->rad[G] - S->rad[H];
        if (gap > reach + 1e-6 * (S->pp[G * P + H] + S->rad[G] + S->rad[H])) continue;
        near[nh++] = H;
    }
    for (int64_t a = S->gstart[G]; a < S->gstart[G + 1]; ++a) {
        const double *xp = S->xs + a * d, *dp = S->bq + a * Q;
        const int64_t begin = out->len;
        for (int32_t h = 0; h < nh; ++h) {
            const int32_t H = near[h];
            for (int64_t b = S->gstart[H]; b < S->gstart[H + 1]; ++b) {
                const double *db = S->bq + b * Q;
                int pruned = 0;
                for (int32_t q = 0; q < Q && !pruned; ++q)
                    pruned = fabs(db[q] - dp[q]) > reach + 1e-6 * (db[q] + dp[q]);
                if (pruned) continue;
                if (in_radius_early(xp, S->xs + b * d, d, S->radius_cutoff, S->exit_above, S->metric, S->fpmode))
                    if (pv_push(out, S->idx[b]) != 0) return -1;
            }
        }
        const int32_t p = S->idx[a];
        qsort(out->buf + begin, (size_t)(out->len - begin), sizeof(int32_t), cmp_i32);
        S->row_len[p] = out->len - begin;
        S->row_start[p] = begin;
        S->row_tid[p] = tid;
    }
    return 0;
}

static void *pv_worker(void *arg)
{
    pv_arg *A = (pv_arg *)arg;
    pv_state *S = A->S;
    const int32_t P = S->P, Q = S->Q, d = S->d;
    int32_t *near = S->phase == 2 ? (int32_t *)malloc(sizeof(int32_t) * (size_t)P) : NULL;
    if (S->phase == 2 && !near) { S->failed = 1; return NULL; }
    const int64_t gstep = S->n / P, qstep = S->n / Q;
    for (;;) {
        pthread_mutex_lock(&S->mu);
        const int64_t b = S->next;
        S->next += S->block;
        pthread_mutex_unlock(&S->mu);
        if (b >= S->total) break;
        const int64_t e = b + S->block < S->total ? b + S->block : S->total;
        for (int64_t i = b; i < e; ++i) {
            if (S->phase == 0) {  /* point i: nearest group pivot */
                int32_t best = 0;
                double bd = INFINITY;
                for (int32_t v = 0; v < P; ++v) {
                    const double dv = plain_dist(S->x + i * d, S->x + (int64_t)v * gstep * d, d);
                    if (dv < bd) { bd = dv; best = v; }
                }
                S->grp[i] = best;
                S->od[i] = bd;
            } else if (S->phase == 1) {  /* pivot row i: distances to the other pivots */
                for (int32_t v = 0; v < P; ++v)
                    S->pp[i * P + v] = plain_dist(S->x + i * gstep * d, S->x + (int64_t)v * gstep * d, d);
            } else if (S->phase == 3) {  /* group-order point i: bound-pivot distances */
                for (int32_t q = 0; q < Q; ++q)
                    S->bq[i * Q + q] = plain_dist(S->xs + i * d, S->x + (int64_t)q * qstep * d, d);
            } else {
                if (pv_rows_of_group(S, i, A->out, A->tid, near) != 0) { S->failed = 1; free(near); return NULL; }
            }
        }
    }
    free(near);
    return NULL;
}

static int pv_phase(pv_state *S, int phase, int64_t total, int64_t block, pv_arg *args, int nthreads)
{
    pthread_t th[256];
    S->phase = phase;
    S->next = 0;
    S->total = total;
    S->block = block;
    int started = 1;
    for (int t = 1; t < nthreads; ++t, ++started)
        if (pthread_create(&th[t], NULL, pv_worker, &args[t]) != 0) break;
    pv_worker(&args[0]);
    for (int t = 1; t < started; ++t) pthread_join(th[t], NULL);
    return S->failed ? -1 : 0;
}

static void pivot_free(void)
{
    if (g_pivot) {
        pv_state *S = g_pivot;
        free(S->grp); free(S->od); free(S->bq); free(S->xs); free(S->idx); free(S->gstart); free(S->rad);
        free(S->pp); free(S->row_len); free(S->row_start); free(S->row_tid);
        free(S);
        g_pivot = NULL;
    }
    for (int t = 0; t < g_pivot_nbufs; ++t) free(g_pivot_bufs[t].buf);
    free(g_pivot_bufs);
    g_pivot_bufs = NULL;
    g_pivot_nbufs = 0;
}

/* Rows of every point; returns the total number of pairs (rows kept for
 * oracle_pivot_take), -1 on allocation failure, -2 for non-finite input. */
int64_t oracle_pivot_run(const double *x, int64_t n, int32_t d, double radius_cutoff, int metric, int fpmode,
                         int nthreads)
{
    pivot_free();
    for (int64_t e = 0; e < n * d; ++e)
        if (!isfinite(x[e])) return -2;
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    pv_state *S = (pv_state *)calloc(1, sizeof(pv_state));
    if (!S) return -1;
    g_pivot = S;
    S->x = x; S->n = n; S->d = d; S->radius_cutoff = radius_cutoff; S->metric = metric; S->fpmode = fpmode;
    S->P = n >= 1024 * 64 ? 1024 : (int32_t)(n / 64 > 1 ? n / 64 : 1);
    S->Q = S->P < kBoundPivots ? S->P : kBoundPivots;
    const int32_t P = S->P, Q = S->Q;
    const int ok_radius = radius_cutoff >= 0 && isfinite(radius_cutoff);
    S->reach = !ok_radius ? INFINITY : metric == ORACLE_METRIC_EUCLIDEAN ? radius_cutoff : sqrt(radius_cutoff);
    S->exit_above = !ok_radius ? INFINITY
                    : metric == ORACLE_METRIC_EUCLIDEAN ? radius_cutoff * radius_cutoff * (1.0 + 1e-9) + 1e-300
                                                        : radius_cutoff;
    const size_t nn = (size_t)(n > 0 ? n : 1);
    S->grp = (int32_t *)malloc(sizeof(int32_t) * nn);
    S->od = (double *)malloc(sizeof(double) * nn);
    S->bq = (double *)malloc(sizeof(double) * nn * Q);
    S->xs = (double *)malloc(sizeof(double) * nn * d);
    S->idx = (int32_t *)malloc(sizeof(int32_t) * nn);
    S->gstart = (int64_t *)calloc((size_t)P + 1, sizeof(int64_t));
    S->rad = (double *)calloc((size_t)P, sizeof(double));
    S->pp = (double *)malloc(sizeof(double) * (size_t)P * P);
    S->row_len = (int64_t *)calloc(nn, sizeof(int64_t));
    S->row_start = (int64_t *)calloc(nn, sizeof(int64_t));
    S->row_tid = (int32_t *)calloc(nn, sizeof(int32_t));
    g_pivot_bufs = (pv_buf *)calloc((size_t)nthreads, sizeof(pv_buf));
    pv_arg *args = (pv_arg *)calloc((size_t)nthreads, sizeof(pv_arg));
    if (!S->grp || !S->od || !S->bq || !S->xs || !S->idx || !S->gstart || !S->rad || !S->pp || !S->row_len ||
        !S->row_start || !S->row_tid || !g_pivot_bufs || !args) {
        free(args);
        pivot_free();
        return -1;
    }
    g_pivot_nbufs = nthreads;
    for (int t = 0; t < nthreads; ++t) { args[t].S = S; args[t].out = &g_pivot_bufs[t]; args[t].tid = t; }
    pthread_mutex_init(&S->mu, NULL);
    int rc = n == 0 ? 0 : pv_phase(S, 0, n, 256, args, nthreads);
    if (rc == 0 && n > 0) rc = pv_phase(S, 1, P, 8, args, nthreads);
    if (rc == 0 && n > 0) {
        /* group order: counting sort by group, index order inside a group */
        for (int64_t i = 0; i < n; ++i) S->gstart[S->grp[i] + 1]++;
        for (int32_t v = 0; v < P; ++v) S->gstart[v + 1] += S->gstart[v];
        int64_t *cur = (int64_t *)malloc(sizeof(int64_t) * (size_t)P);
        if (!cur) {
            rc = -1;
        } else {
            memcpy(cur, S->gstart, sizeof(int64_t) * (size_t)P);
            for (int64_t i = 0; i < n; ++i) {
                const int32_t G = S->grp[i];
                const int64_t a = cur[G]++;
                S->idx[a] = (int32_t)i;
                memcpy(S->xs + a * d, x + i * d, sizeof(double) * (size_t)d);
                if (S->od[i] > S->rad[G]) S->rad[G] = S->od[i];
            }
            free(cur);
            rc = pv_phase(S, 3, n, 256, args, nthreads);
        }
    }
    if (rc == 0 && n > 0) rc = pv_phase(S, 2, P, 1, args, nthreads);
    free(args);
    pthread_mutex_destroy(&S->mu);
    if (rc != 0) { pivot_free(); return -1; }
    int64_t total = 0;
    for (int64_t p = 0; p < n; ++p) total += S->row_len[p];
    return total;
}

/* The rows of the last oracle_pivot_run as CSR (offsets int64[n+1],
 * indices int32[total]); frees them. */
int oracle_pivot_take(int64_t *offsets, int32_t *indices)
{
    if (!g_pivot) return -1;
    const pv_state *S = g_pivot;
    offsets[0] = 0;
    for (int64_t p = 0; p < S->n; ++p) {
        offsets[p + 1] = offsets[p] + S->row_len[p];
        if (S->row_len[p])
            memcpy(indices + offsets[p], g_pivot_bufs[S->row_tid[p]].buf + S->row_start[p],
                   sizeof(int32_t) * (size_t)S->row_len[p]);
    }
    pivot_free();
    return 0;
}

void oracle_pivot_free(void) { pivot_free(); }

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
