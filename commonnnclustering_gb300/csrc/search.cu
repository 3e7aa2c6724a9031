// search.cu -- radius neighbour search producing sorted CSR neighbourhoods.
//
// Reference: NeighboursGetterExtBruteForce._get (src/cnnclustering/
// _types.pyx:1692-1710) keeps every i with distance(p, i) <= radius_cutoff,
// distance from MetricExtEuclideanReduced._calc_distance (:2253-2267):
// a float64 sum of (a-b)^2 over dimensions 0..d-1 starting from 0.0.  The
// neighbour SET is fixed by that predicate; the kernels here only change
// which pairs are looked at and how cheaply obvious ones are decided:
//
//  * Cell grid (d <= 3).  Points are bucketed into cubic cells of edge
//    h >= R (R = search radius) and ordered by cell id (x fastest; inside
//    a cell, in the order of an atomic counter -- any order will do).  A
//    point's candidates are the 3x3x3 cells around its own; for a fixed
//    (dy, dz) the three x-cells are contiguous, so candidates form 9 runs of
//    consecutive internal indices, visited in increasing order.  Rows come
//    out ascending in internal index without any sort.
//  * Tiled all-pairs (any d).  Candidate tiles of 32 points are staged in
//    shared memory; each warp tests its query against the tile.
//
// Every candidate is first tested in float32 on coordinates shifted to the
// bounding-box minimum.  A host-computed error bound gives a band around
// the cutoff; only pairs inside it are recomputed in float64 with exactly
// the reference's operation order (explicit __dsub_rn/__dmul_rn/__dadd_rn
// or __fma_rn, so the compiler cannot re-contract them).  Outside the band
// the float32 decision is provably the float64 one.
//
// Internal index space: the grid path stores the graph in cell order
// (perm: internal -> point index).  Intersections and connected
// components are invariant under that relabelling; export to point order
// happens only on request (cnn_get_neighbours).
#include <limits.h>
#include <math.h>

#include <algorithm>
#include <vector>

#include "common.cuh"

namespace cnn {

namespace {

struct SearchParams {
    double rc;        // radius_cutoff as the getter compares it
    int metric;       // cnn_metric
    int fpmode;       // cnn_fpmode
    float thr_in;     // sf <= thr_in  -> neighbour
    float thr_out;    // sf >  thr_out -> not a neighbour; else float64
    const double *bd = nullptr;  // periodic metric: box length per dimension (<= 0: not periodic)
    const float *bf = nullptr;   // the same in float32
    // wrapped cell grid: float32 box length and half length per dimension
    // (0 and +inf for dimensions that do not wrap)
    float wl[3] = {0.f, 0.f, 0.f};
    float whalf[3] = {INFINITY, INFINITY, INFINITY};
};

// Minimum-image difference of the periodic metric, reference order
// (MetricExtEuclideanPeriodicReduced._calc_distance, _types.pyx:2303-2325):
// d = |a - b|; if bound > 0: d = fmod(d, bound), d = bound - d if d > bound / 2.
__device__ __forceinline__ double periodic_diff(double a, double b, double bound) {
    double t = fabs(__dsub_rn(a, b));
    if (bound > 0.0) {
        t = fmod(t, bound);
        if (t > bound / 2.0) t = __dsub_rn(bound, t);
    }
    return t;
}

__device__ __forceinline__ float periodic_diff_f(float a, float b, float bound) {
    float t = fabsf(a - b);
    if (bound > 0.f) {
        t = fmodf(t, bound);
        if (t > 0.5f * bound) t = bound - t;
    }
    return t;
}

// Exact float64 predicate in the reference's operation order.
__device__ __forceinline__ bool exact_in_radius(const double *__restrict__ xa, const double *__restrict__ xb,
                                                int d, const SearchParams &sp) {
    double s = 0.0;
    if (sp.bd) {
        for (int k = 0; k < d; ++k) {
            const double t = periodic_diff(xa[k], xb[k], sp.bd[k]);
            s = sp.fpmode == CNN_FP_FUSED ? __fma_rn(t, t, s) : __dadd_rn(s, __dmul_rn(t, t));
        }
        return s <= sp.rc;
    }
    if (sp.fpmode == CNN_FP_FUSED) {
        for (int k = 0; k < d; ++k) {
            double t = __dsub_rn(xa[k], xb[k]);
            s = __fma_rn(t, t, s);
        }
    } else {
        for (int k = 0; k < d; ++k) {
            double t = __dsub_rn(xa[k], xb[k]);
            s = __dadd_rn(s, __dmul_rn(t, t));
        }
    }
    if (sp.metric == CNN_METRIC_EUCLIDEAN) s = __dsqrt_rn(s);
    return s <= sp.rc;
}

constexpr int kMaxGridDim = 3;

// ctx->counters (unsigned long long): [0] pairs decided in float64,
// [1] candidates (mask form, all-pairs search), [2..3] cnn_set_neighbours
// validation, [4..8] the fit, [10..14] the tensor-core search, [15] sweep
// buckets, [16..19] neighbour pairs of the rows the list search left in
// their slots (four addresses against atomic contention)
constexpr int kCounterSlots = 24, kSlotPairsAt = 16;
// public cell-grid builds leave the list search's rows in their slots (0: CSR at once)
#ifndef CNN_SLOT_ROWS
#define CNN_SLOT_ROWS 1
#endif

// General-d extents: per dimension min/max of finite rows (for the float32
// error bound of the all-pairs path).  part: [blocks][2*d + 1].
__global__ void extent_partial_kernel(const double *__restrict__ x, int64_t n, int d,
                                      double *__restrict__ part) {
    // one block per (dimension chunk): thread-strided over rows, dimension k
    const int k = blockIdx.y;
    double lo = INFINITY, hi = -INFINITY, bad = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double v = x[i * d + k];
        if (!isfinite(v)) { bad += 1; continue; }
        lo = fmin(lo, v);
        hi = fmax(hi, v);
    }
    __shared__ double s[3][256];
    s[0][threadIdx.x] = lo; s[1][threadIdx.x] = hi; s[2][threadIdx.x] = bad;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            s[0][threadIdx.x] = fmin(s[0][threadIdx.x], s[0][threadIdx.x + w]);
            s[1][threadIdx.x] = fmax(s[1][threadIdx.x], s[1][threadIdx.x + w]);
            s[2][threadIdx.x] += s[2][threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        double *o = part + ((int64_t)blockIdx.x * d + k) * 3;
        o[0] = s[0][0]; o[1] = s[1][0]; o[2] = s[2][0];
    }
}

// ---- grid construction (GridGeom: common.cuh) -------------------------------

// floor((v - lo) / h) with the quotient taken as a product by the rounded
// reciprocal: still monotone in v, and two values less than R apart land in
// cells at most one apart (h exceeds R by a relative 1e-6, far above the
// few ulps of relative rounding on (v - lo) / h for grids of <= 64M cells)
__device__ __forceinline__ int32_t cell_coord(double v, double lo, double inv_h, int32_t g) {
    double c = floor(__dmul_rn(__dsub_rn(v, lo), inv_h));
    if (!(c >= 0.0)) c = 0.0;
    if (c > (double)(g - 1)) c = (double)(g - 1);
    return (int32_t)c;
}

// A coordinate of a wrapping dimension mapped into the box [0, L): the
// minimum-image difference of two points equals the cyclic distance of
// their mapped coordinates (up to a few ulps of max(|x|, L)).
__device__ __forceinline__ double wrap_coord(double v, double L) { return v - L * floor(v / L); }

// Cell coordinate of dimension k (wrapping or not), clamped to the grid.
__device__ __forceinline__ int32_t cell_coord_k(double v, const GridGeom &geo, int k) {
    if ((geo.wrap >> k) & 1) {
        double c = floor(wrap_coord(v, geo.L[k]) * geo.inv_hk[k]);
        if (!(c >= 0.0)) c = 0.0;
        if (c > (double)(geo.g[k] - 1)) c = (double)(geo.g[k] - 1);
        return (int32_t)c;
    }
    return cell_coord(v, geo.lo[k], geo.inv_hk[k], geo.g[k]);
}

// cell of every point and its slot among the points of that cell (the
// order of the atomic increments: any order serves, rows are sorted by
// internal index whatever the order inside a cell)
__global__ void cell_assign_kernel(const double *__restrict__ x, int64_t n, int d, GridGeom geo,
                                   int32_t *__restrict__ cell_of, int32_t *__restrict__ slot,
                                   int32_t *__restrict__ cell_count) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        bool fin = true;
        for (int k = 0; k < d; ++k) fin = fin && isfinite(x[i * d + k]);
        int64_t id;
        if (!fin) {
            id = geo.ncells;
        } else {
            int32_t c[3] = {0, 0, 0};
            for (int k = 0; k < d; ++k) c[k] = cell_coord_k(x[i * d + k], geo, k);
            id = (int64_t)c[0] + (int64_t)geo.g[0] * ((int64_t)c[1] + (int64_t)geo.g[1] * c[2]);
        }
        cell_of[i] = (int32_t)id;
        slot[i] = atomicAdd(&cell_count[id], 1);
    }
}

// Internal order = cell order: point i goes to cell_start[cell] + slot;
// perm/inv map between the orders and xf4 holds the float32 coordinates
// relative to the grid origin in internal order.
__global__ void place_kernel(const int32_t *__restrict__ cell_of, const int32_t *__restrict__ slot,
                             const int64_t *__restrict__ cell_start, int64_t n, const double *__restrict__ x, int d,
                             GridGeom geo, int32_t *__restrict__ perm, int32_t *__restrict__ inv,
                             float4 *__restrict__ xf4) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t c = cell_of[i];
        const int32_t p = (int32_t)(cell_start[c] + slot[i]);
        perm[p] = (int32_t)i;
        inv[i] = p;
        float v[3] = {0.f, 0.f, 0.f};
        for (int k = 0; k < d; ++k)
            v[k] = (geo.wrap >> k) & 1 ? (float)wrap_coord(x[i * d + k], geo.L[k])
                                       : (float)__dsub_rn(x[i * d + k], geo.lo[k]);
        xf4[p] = make_float4(v[0], v[1], v[2], 0.f);
    }
}

// cell of every point in internal order (the mask form's row geometry)
__global__ void point_cell_kernel(const int32_t *__restrict__ cell_of, const int32_t *__restrict__ perm, int64_t n,
                                  int32_t *__restrict__ pcell) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x)
        pcell[p] = cell_of[perm[p]];
}

// ---- grid search -----------------------------------------------------------
// Float64 predicate on rows of the original-order coordinate array.
__device__ __forceinline__ bool exact_rows(const double *__restrict__ x, int d, int32_t ia, int32_t ib,
                                           const SearchParams &sp) {
    const double *xa = x + (int64_t)ia * d;
    const double *xb = x + (int64_t)ib * d;
    return exact_in_radius(xa, xb, d, sp);
}

// work items of kPer consecutive queries of one cell
template <int kPer>
__global__ void item_count_kernel(const int64_t *__restrict__ cell_start, int64_t ncells,
                                  int32_t *__restrict__ items_per_cell) {
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < ncells; c += (int64_t)gridDim.x * blockDim.x) {
        const int64_t q = cell_start[c + 1] - cell_start[c];
        items_per_cell[c] = (int32_t)((q + kPer - 1) / kPer);
    }
}

template <int kPer>
__global__ void item_fill_kernel(const int64_t *__restrict__ cell_start, int64_t ncells,
                                 const int64_t *__restrict__ item_off, int2 *__restrict__ items) {
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < ncells; c += (int64_t)gridDim.x * blockDim.x) {
        const int64_t b = item_off[c], e = item_off[c + 1];
        for (int64_t k = b; k < e; ++k)
            items[k] = make_int2((int32_t)c, (int32_t)(cell_start[c] + (k - b) * kPer));
    }
}

// Candidate count of a cell: the points of the (2 reach + 1)^3 cells around
// it (the same x-runs the search packs).
// The runs of the stencil row (y, z) around x-cell cx on a wrapped grid
// (reach 1): one run, or two where the three x-cells wrap around.
__device__ __forceinline__ int wrapped_x_runs(int32_t cx, int32_t g0, bool wrap_x, int32_t *a, int32_t *b) {
    if (wrap_x && cx == 0) {
        a[0] = 0; b[0] = 1; a[1] = g0 - 1; b[1] = g0 - 1;
        return 2;
    }
    if (wrap_x && cx == g0 - 1) {
        a[0] = g0 - 2; b[0] = g0 - 1; a[1] = 0; b[1] = 0;
        return 2;
    }
    a[0] = cx > 0 ? cx - 1 : 0;
    b[0] = cx + 1 < g0 ? cx + 1 : g0 - 1;
    return 1;
}

// neighbour row/plane index of c + dc, cyclic when the dimension wraps;
// -1 outside a grid that does not
__device__ __forceinline__ int32_t stencil_coord(int32_t c, int dc, int32_t g, bool wrap) {
    int32_t v = c + dc;
    if (wrap) return v < 0 ? v + g : (v >= g ? v - g : v);
    return v < 0 || v >= g ? -1 : v;
}

__device__ __forceinline__ int64_t cell_candidates(int64_t cid, const GridGeom &geo,
                                                   const int64_t *__restrict__ cell_start) {
    const int32_t cx = (int32_t)(cid % geo.g[0]);
    const int32_t cy = (int32_t)((cid / geo.g[0]) % geo.g[1]);
    const int32_t cz = (int32_t)(cid / ((int64_t)geo.g[0] * geo.g[1]));
    if (geo.wrap) {  // reach 1 (a wrapped grid is built with reach 1 only)
        int32_t a[2], b[2];
        const int nx = wrapped_x_runs(cx, geo.g[0], geo.wrap & 1, a, b);
        int64_t total = 0;
        for (int dz = -1; dz <= 1; ++dz) {
            const int32_t z = stencil_coord(cz, dz, geo.g[2], (geo.wrap >> 2) & 1);
            if (z < 0) continue;
            for (int dy = -1; dy <= 1; ++dy) {
                const int32_t y = stencil_coord(cy, dy, geo.g[1], (geo.wrap >> 1) & 1);
                if (y < 0) continue;
                const int64_t row = (int64_t)geo.g[0] * ((int64_t)y + (int64_t)geo.g[1] * z);
                for (int r = 0; r < nx; ++r) total += cell_start[row + b[r] + 1] - cell_start[row + a[r]];
            }
        }
        return total;
    }
    const int S = geo.reach;
    const int32_t xlo = cx > S - 1 ? cx - S : 0;
    const int32_t xhi = cx + S < geo.g[0] ? cx + S : geo.g[0] - 1;
    int64_t total = 0;
    for (int dz = -S; dz <= S; ++dz) {
        const int32_t z = cz + dz;
        if (z < 0 || z >= geo.g[2]) continue;
        for (int dy = -S; dy <= S; ++dy) {
            const int32_t y = cy + dy;
            if (y < 0 || y >= geo.g[1]) continue;
            const int64_t row = (int64_t)geo.g[0] * ((int64_t)y + (int64_t)geo.g[1] * z);
            const int64_t rs = cell_start[row + xlo], re = cell_start[row + xhi + 1];
            if (re > rs) total += re - rs;
        }
    }
    return total;
}

// slots of a cell = its points x its candidate count (upper bound of every
// row); kWords: its points x the 32-bit words of one mask row
template <bool kWords>
__global__ void cell_slots_kernel(const int64_t *__restrict__ cell_start, GridGeom geo,
                                  int64_t *__restrict__ slots) {
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < geo.ncells;
         c += (int64_t)gridDim.x * blockDim.x) {
        const int64_t q = cell_start[c + 1] - cell_start[c];
        const int64_t t = q > 0 ? cell_candidates(c, geo, cell_start) : 0;
        slots[c] = q * (kWords ? (t + 31) / 32 : t);
    }
}

// For rows left in their slots: end[a] = start[a] + len[a], and split[a] =
// the entries <= a of row a (rows ascending) by bisection, one thread per
// row -- the fit's walks over b > a start there (the compaction records the
// same when it makes the CSR).
__global__ void row_split_kernel(int64_t n, const int64_t *__restrict__ start, const int32_t *__restrict__ len,
                                 const int32_t *__restrict__ cols, int64_t *__restrict__ end,
                                 int32_t *__restrict__ split) {
    for (int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; a < n; a += (int64_t)gridDim.x * blockDim.x) {
        const int64_t s = start[a];
        const int32_t l = len[a];
        const int32_t *row = cols + s;
        int32_t lo = 0, hi = l;
        while (lo < hi) {
            const int32_t mid = (lo + hi) >> 1;
            if (row[mid] <= (int32_t)a) lo = mid + 1;
            else hi = mid;
        }
        end[a] = s + l;
        split[a] = lo;
    }
}

// Per cell its work items (kPer consecutive queries each) and its slots
// (points x candidate count, the upper bound of each row); the entries at
// ncells are the zero tails of the two exclusive scans.
template <int kPer>
__global__ void cell_units_kernel(const int64_t *__restrict__ cell_start, GridGeom geo, int32_t *__restrict__ items,
                                  int64_t *__restrict__ slots) {
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < geo.ncells;
         c += (int64_t)gridDim.x * blockDim.x) {
        const int64_t q = cell_start[c + 1] - cell_start[c];
        items[c] = (int32_t)((q + kPer - 1) / kPer);
        slots[c] = q > 0 ? q * cell_candidates(c, geo, cell_start) : 0;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        items[geo.ncells] = 0;
        slots[geo.ncells] = 0;
    }
}

// rows from their slots to the CSR (one warp per row); split[q] = the
// entries <= q of row q (rows are ascending), so the fit's walks over the
// entries > q start there
__global__ void compact_rows_kernel(int64_t n, const int64_t *__restrict__ qslot, const int32_t *__restrict__ slot_cols,
                                    const int64_t *__restrict__ row_off, int32_t *__restrict__ cols,
                                    int32_t *__restrict__ split) {
    const int lane = threadIdx.x & 31;
    const int64_t warp0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t q = warp0; q < n; q += nwarps) {
        const int64_t src = qslot[q], dst = row_off[q], len = row_off[q + 1] - dst;
        int32_t le = 0;
        for (int64_t e0 = 0; e0 < len; e0 += 128) {  // four independent loads in flight per lane
            int32_t v[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int64_t e = e0 + j * 32 + lane;
                v[j] = e < len ? slot_cols[src + e] : INT32_MAX;
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int64_t e = e0 + j * 32 + lane;
                if (e < len) cols[dst + e] = v[j];
                le += __popc(__ballot_sync(0xffffffffu, v[j] <= (int32_t)q));
            }
        }
        if (lane == 0) split[q] = le;
    }
}

// kMode: kCount writes deg; kFill writes the rows at row_off; kSlots writes
// each query's row into its slot (slot_base[cell] + rank in cell x the
// cell's candidate count, an upper bound of the row), its length to deg
// and the slot start to qslot -- one pass instead of count + fill when the
// slots fit in memory; kMask writes each query's row as bits, one 32-bit
// word (the step's ballot) per 32 candidates, at mbase[cell] + rank in cell
// x the words of the cell's rows, and its length to deg.
constexpr int kCount = 0, kFill = 1, kSlots = 2, kMask = 3;

// ---- warp-granular grid search ---------------------------------------------
// Work unit = (cell, up to kUnitQueries consecutive queries of that cell), one
// warp each, no block-wide staging: the warp reads its cell's candidate runs
// ((2 reach + 1)^2 (y,z) neighbours, each 2 reach + 1 x-cells long and
// contiguous in internal order) straight from xf4, 32 candidates at a time
// over the runs' concatenation, and tests each against its queries held in
// registers.
// Sparse cells (most cells hold a few points) cost one warp, not a block;
// the warps of a block work on neighbouring units and share candidates
// through L1.  Concatenated run order = ascending internal index, so every
// query's hits come out sorted.
#ifndef CNN_UNIT_QUERIES
#define CNN_UNIT_QUERIES 4
#endif
constexpr int kUnitQueries = CNN_UNIT_QUERIES;
constexpr int kUnitWarps = 8;
constexpr int kMaxRuns = 25;  // (2 * reach + 1)^2 runs of a cell's stencil, reach <= 2
#ifndef CNN_UNIT_SUB
#define CNN_UNIT_SUB 1  // two steps per iteration measured slower (register pressure)
#endif
constexpr int kUnitSub = CNN_UNIT_SUB;  // 32-candidate steps per loop iteration

#ifndef CNN_UNIT_MIN_BLOCKS
#define CNN_UNIT_MIN_BLOCKS 4  // 64 registers: four blocks of eight warps per SM
#endif

// kWrap: a wrapped grid (periodic metric, reach 1): up to 18 runs (a 3-cell
// x-run splits in two where it wraps), sorted by start so that the
// concatenation stays ascending, and minimum-image float32 differences.
template <int kMode, bool kWrap = false>
__global__ void __launch_bounds__(kUnitWarps * 32, CNN_UNIT_MIN_BLOCKS) grid_unit_kernel(
    const int2 *__restrict__ units, int64_t nunits, const double *__restrict__ x, int d, GridGeom geo,
    SearchParams sp, const int32_t *__restrict__ perm, const int64_t *__restrict__ cell_start,
    const float4 *__restrict__ xf4, int32_t *__restrict__ deg, const int64_t *__restrict__ row_off,
    int32_t *__restrict__ cols, unsigned long long *__restrict__ counters, int64_t *__restrict__ qslot) {
    __shared__ int32_t s_rs[kUnitWarps][kMaxRuns];
    __shared__ int32_t s_cum[kUnitWarps][kMaxRuns + 1];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int64_t u = (int64_t)blockIdx.x * kUnitWarps + wid;
    if (u >= nunits) return;  // whole warps only: nothing below syncs the block
    const int2 unit = units[u];
    const int32_t cid = unit.x;
    const int64_t q0 = unit.y;
    const int64_t cs = cell_start[cid], qend = cell_start[cid + 1];
    // run r = lane (r < nruns): (dz, dy) = (r / W - S, r % W - S); empty when outside the grid
    const int S = geo.reach, Wd = 2 * S + 1;
    const int nruns = kWrap ? 18 : Wd * Wd;
    int32_t rs = 0, len = 0;
    if (kWrap) {
        // lanes 0..8 hold the (dz, dy) rows' runs, two where x wraps; every
        // non-empty run goes to its rank by start (runs are disjoint), the
        // rest of the 18 slots are empty
        int32_t a0 = 0, l0 = 0, a1 = 0, l1 = 0;
        if (lane < 9) {
            const int32_t cx = cid % geo.g[0];
            const int32_t cy = (cid / geo.g[0]) % geo.g[1];
            const int32_t cz = cid / (geo.g[0] * geo.g[1]);
            const int32_t z = stencil_coord(cz, lane / 3 - 1, geo.g[2], (geo.wrap >> 2) & 1);
            const int32_t y = stencil_coord(cy, lane % 3 - 1, geo.g[1], (geo.wrap >> 1) & 1);
            if (z >= 0 && y >= 0) {
                int32_t xa[2], xb[2];
                const int nx = wrapped_x_runs(cx, geo.g[0], geo.wrap & 1, xa, xb);
                const int64_t row = (int64_t)geo.g[0] * ((int64_t)y + (int64_t)geo.g[1] * z);
                a0 = (int32_t)cell_start[row + xa[0]];
                l0 = (int32_t)(cell_start[row + xb[0] + 1] - a0);
                if (nx > 1) {
                    a1 = (int32_t)cell_start[row + xa[1]];
                    l1 = (int32_t)(cell_start[row + xb[1] + 1] - a1);
                }
            }
        }
        const int32_t k0 = l0 > 0 ? a0 : INT_MAX, k1 = l1 > 0 ? a1 : INT_MAX;
        int r0 = 0, r1 = 0;
#pragma unroll
        for (int j = 0; j < 9; ++j) {
            const int32_t o0 = __shfl_sync(0xffffffffu, k0, j), o1 = __shfl_sync(0xffffffffu, k1, j);
            r0 += (o0 < k0) + (o1 < k0);
            r1 += (o0 < k1) + (o1 < k1);
        }
        if (lane < 18) {
            s_rs[wid][lane] = 0;
            s_cum[wid][lane + 1] = 0;  // lengths, in rank order, until the scan below
        }
        __syncwarp();
        if (lane < 9 && l0 > 0) {
            s_rs[wid][r0] = a0;
            s_cum[wid][r0 + 1] = l0;
        }
        if (lane < 9 && l1 > 0) {
            s_rs[wid][r1] = a1;
            s_cum[wid][r1 + 1] = l1;
        }
        __syncwarp();
        if (lane < 18) {
            rs = s_rs[wid][lane];
            len = s_cum[wid][lane + 1];
        }
        __syncwarp();
    } else if (lane < nruns) {
        const int32_t cx = cid % geo.g[0];
        const int32_t cy = (cid / geo.g[0]) % geo.g[1];
        const int32_t cz = cid / (geo.g[0] * geo.g[1]);
        const int32_t z = cz + lane / Wd - S, y = cy + lane % Wd - S;
        if (z >= 0 && z < geo.g[2] && y >= 0 && y < geo.g[1]) {
            const int32_t xlo = cx > S - 1 ? cx - S : 0;
            const int32_t xhi = cx + S < geo.g[0] ? cx + S : geo.g[0] - 1;
            const int64_t row = (int64_t)geo.g[0] * ((int64_t)y + (int64_t)geo.g[1] * z);
            const int64_t b = cell_start[row + xlo], e = cell_start[row + xhi + 1];
            rs = (int32_t)b;
            len = e > b ? (int32_t)(e - b) : 0;
        }
    }
    int32_t inc = len;  // inclusive prefix over the runs
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int32_t v = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += v;
    }
    if (lane < nruns) {
        s_rs[wid][lane] = rs;
        s_cum[wid][lane + 1] = inc;
    }
    if (lane == 0) s_cum[wid][0] = 0;
    const int32_t total = __shfl_sync(0xffffffffu, inc, nruns - 1);
    __syncwarp();

    // query k: internal index (-1: none), coordinates, and for kFill/kSlots
    // its row in cols (kCount: a per-lane count)
    int32_t qi[kUnitQueries];
    float qx[kUnitQueries], qy[kUnitQueries], qz[kUnitQueries];
    int32_t *rowp[kUnitQueries];
    int32_t cnt[kUnitQueries];
    const int64_t row_len = kMode == kMask ? (int64_t)((total + 31) >> 5) : (int64_t)total;  // slot of one row
    const int64_t slot0 = (kMode == kSlots || kMode == kMask) ? row_off[cid] + (q0 - cs) * row_len : 0;
#pragma unroll
    for (int k = 0; k < kUnitQueries; ++k) {
        const int64_t qk = q0 + k;
        const bool ok = qk < qend;
        const float4 f = ok ? xf4[qk] : make_float4(INFINITY, INFINITY, INFINITY, 0.f);
        qx[k] = f.x;
        qy[k] = f.y;
        qz[k] = f.z;
        qi[k] = ok ? (int32_t)qk : -1;
        const int64_t w = kMode == kFill ? (ok ? row_off[qk] : 0) : slot0 + k * row_len;
        rowp[k] = kMode == kCount ? nullptr : cols + w;
        if (kMode == kSlots && ok && lane == 0) qslot[qk] = w;
        cnt[k] = 0;
    }
    const unsigned lt = (1u << lane) - 1u;
    unsigned long long n_exact = 0;
    // kUnitSub steps of 32 candidates per iteration (lane's candidates t and
    // t + 32, ...).  Each step's lane keeps its run: t in [.., hi) of the
    // concatenation maps to j = base + t; t only grows, so the run index only
    // moves forward (empty runs skipped)
    int r[kUnitSub];
    int32_t hi[kUnitSub], base[kUnitSub];
#pragma unroll
    for (int u = 0; u < kUnitSub; ++u) {
        r[u] = 0;
        hi[u] = s_cum[wid][1];
        base[u] = s_rs[wid][0];
    }
    for (int32_t t0 = lane; t0 - lane < total; t0 += 32 * kUnitSub) {
        int32_t j[kUnitSub];
        bool in[kUnitSub][kUnitQueries], amb[kUnitSub][kUnitQueries];
        bool any_amb = false;
#pragma unroll
        for (int u = 0; u < kUnitSub; ++u) {
            const int32_t t = t0 + 32 * u;
            while (t >= hi[u] && r[u] < nruns - 1) {
                ++r[u];
                base[u] = s_rs[wid][r[u]] - hi[u];
                hi[u] = s_cum[wid][r[u] + 1];
            }
            j[u] = base[u] + t;
            const float4 cf = t < total ? xf4[j[u]] : make_float4(INFINITY, INFINITY, INFINITY, 0.f);  // +inf never matches
#pragma unroll
            for (int k = 0; k < kUnitQueries; ++k) {
                float ex = qx[k] - cf.x, ey = qy[k] - cf.y, ez = qz[k] - cf.z;
                if (kWrap) {  // minimum image of wrapped coordinates (both in [0, L))
                    ex = fabsf(ex);
                    ey = fabsf(ey);
                    ez = fabsf(ez);
                    if (ex > sp.whalf[0]) ex = sp.wl[0] - ex;
                    if (ey > sp.whalf[1]) ey = sp.wl[1] - ey;
                    if (ez > sp.whalf[2]) ez = sp.wl[2] - ez;
                }
                const float sf = fmaf(ez, ez, fmaf(ey, ey, ex * ex));
                in[u][k] = sf <= sp.thr_in;
                amb[u][k] = !in[u][k] && sf <= sp.thr_out;
                any_amb |= amb[u][k];
            }
        }
        if (__any_sync(0xffffffffu, any_amb)) {  // rare: decide those pairs in float64
#pragma unroll
            for (int u = 0; u < kUnitSub; ++u)
#pragma unroll
                for (int k = 0; k < kUnitQueries; ++k) {
                    if (amb[u][k]) {
                        in[u][k] = exact_rows(x, d, perm[qi[k]], perm[j[u]], sp);
                        ++n_exact;
                    }
                }
        }
#pragma unroll
        for (int k = 0; k < kUnitQueries; ++k) {
#pragma unroll
            for (int u = 0; u < kUnitSub; ++u) {  // step u's candidates follow step u - 1's
                if (kMode == kMask) {
                    const unsigned hit = __ballot_sync(0xffffffffu, in[u][k]);
                    if (lane == k && qi[k] >= 0) rowp[k][((t0 - lane) >> 5) + u] = (int32_t)hit;
                    cnt[k] += __popc(hit);
                } else if (kMode != kCount) {
                    const unsigned hit = __ballot_sync(0xffffffffu, in[u][k]);
                    if (in[u][k]) rowp[k][cnt[k] + __popc(hit & lt)] = j[u];
                    cnt[k] += __popc(hit);
                } else {
                    cnt[k] += in[u][k];  // per-lane count, summed over the warp at the end
                }
            }
        }
    }
    if (kMode != kFill) {
        if (kMode == kCount) {
#pragma unroll
            for (int k = 0; k < kUnitQueries; ++k)
                for (int o = 16; o > 0; o >>= 1) cnt[k] += __shfl_down_sync(0xffffffffu, cnt[k], o);
        }
        if (lane == 0) {
            unsigned long long pairs = 0;
#pragma unroll
            for (int k = 0; k < kUnitQueries; ++k)
                if (qi[k] >= 0) {
                    deg[qi[k]] = cnt[k];
                    pairs += (unsigned long long)cnt[k];
                }
            if (kMode == kSlots) atomicAdd(&counters[kSlotPairsAt + (u & 3)], pairs);  // the pair count, unread
        }
        for (int o = 16; o > 0; o >>= 1) n_exact += __shfl_down_sync(0xffffffffu, n_exact, o);
        if (lane == 0 && n_exact) atomicAdd(&counters[0], n_exact);
        if (kMode == kMask && lane == 0) {  // candidate pairs looked at (statistics)
            unsigned long long q = 0;
#pragma unroll
            for (int k = 0; k < kUnitQueries; ++k) q += qi[k] >= 0 ? 1 : 0;
            atomicAdd(&counters[1], q * (unsigned long long)total);
        }
    }
}

// ---- tiled all-pairs search (any d) -----------------------------------------
constexpr int kTileWarps = 8;
constexpr int kTileCand = 32;

template <bool kFill>
__global__ void __launch_bounds__(kTileWarps * 32) tile_search_kernel(
    const double *__restrict__ x, const float *__restrict__ xf, int d, int64_t n, SearchParams sp,
    int32_t *__restrict__ deg, const int64_t *__restrict__ row_off, int32_t *__restrict__ cols,
    unsigned long long *__restrict__ counters) {
    extern __shared__ float smem[];
    const int ds = d + 1;                      // odd stride: conflict-free rows
    float *cand = smem;                        // [kTileCand][ds]
    float *qry = smem + kTileCand * ds;        // [kTileWarps][ds]
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int64_t p = (int64_t)blockIdx.x * kTileWarps + wid;
    const bool active = p < n;
    for (int k = lane; k < d; k += 32) qry[wid * ds + k] = active ? xf[p * d + k] : 0.f;
    const unsigned lt = (1u << lane) - 1u;
    int64_t w = (kFill && active) ? row_off[p] : 0;
    int64_t cnt = 0;
    unsigned long long n_exact = 0;
    for (int64_t j0 = 0; j0 < n; j0 += kTileCand) {
        __syncthreads();
        for (int e = threadIdx.x; e < kTileCand * d; e += blockDim.x) {
            int r = e / d, k = e - r * d;
            int64_t j = j0 + r;
            cand[r * ds + k] = j < n ? xf[j * d + k] : 0.f;
        }
        __syncthreads();
        const int64_t j = j0 + lane;
        bool in = false;
        if (active && j < n) {
            float sf = 0.f;
            const float *cr = cand + lane * ds;
            const float *qr = qry + wid * ds;
            if (sp.bf) {
                for (int k = 0; k < d; ++k) {
                    const float t = periodic_diff_f(qr[k], cr[k], sp.bf[k]);
                    sf = fmaf(t, t, sf);
                }
            } else {
                for (int k = 0; k < d; ++k) {
                    float t = qr[k] - cr[k];
                    sf = fmaf(t, t, sf);
                }
            }
            if (sf <= sp.thr_in) {
                in = true;
            } else if (!(sf > sp.thr_out)) {   // also catches NaN (non-finite candidate)
                in = exact_in_radius(x + p * d, x + j * d, d, sp);
                ++n_exact;
            }
        }
        const unsigned hit = __ballot_sync(0xffffffffu, in);
        if (kFill && in) cols[w + cnt + __popc(hit & lt)] = (int32_t)j;
        cnt += __popc(hit);
    }
    if (!kFill) {
        if (active && lane == 0) deg[p] = (int32_t)cnt;
        for (int o = 16; o > 0; o >>= 1) n_exact += __shfl_down_sync(0xffffffffu, n_exact, o);
        if (lane == 0 && n_exact) atomicAdd(&counters[0], n_exact);
        if (threadIdx.x == 0 && blockIdx.x == 0) atomicAdd(&counters[1], (unsigned long long)n * (unsigned long long)n);
    }
}

// Rows of other points against this set on this set's cell grid
// (NeighboursGetterExtBruteForce._get_other, src/cnnclustering/_types.pyx:
// 1712-1731, for n_dim <= 3): the other points are binned into the same
// cells (clamped to the grid: a point outside it has its neighbours, if
// any, in the boundary cells); one warp per (cell, up to kUnitQueries other
// points of that cell) scans the cell's stencil runs of this set's xf4 as
// grid_unit_kernel does.  kCount: row lengths; kFill: keys (other point
// index, this set's point index) for a radix sort into ascending rows.
template <bool kFill>
__global__ void __launch_bounds__(kUnitWarps * 32, CNN_UNIT_MIN_BLOCKS) cross_unit_kernel(
    const int2 *__restrict__ units, int64_t nunits, const double *__restrict__ xq, const double *__restrict__ x, int d,
    GridGeom geo, SearchParams sp, const int32_t *__restrict__ qperm, const int64_t *__restrict__ qcell_start,
    const float4 *__restrict__ qxf4, const int32_t *__restrict__ perm, const int64_t *__restrict__ cell_start,
    const float4 *__restrict__ xf4, int bits_n, int32_t *__restrict__ qdeg, const int64_t *__restrict__ qrow_off,
    uint64_t *__restrict__ keys, unsigned long long *__restrict__ counters) {
    __shared__ int32_t s_rs[kUnitWarps][kMaxRuns];
    __shared__ int32_t s_cum[kUnitWarps][kMaxRuns + 1];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int64_t u = (int64_t)blockIdx.x * kUnitWarps + wid;
    if (u >= nunits) return;  // whole warps only
    const int2 unit = units[u];
    const int32_t cid = unit.x;
    const int64_t q0 = unit.y, qend = qcell_start[cid + 1];
    const int S = geo.reach, Wd = 2 * S + 1, nruns = Wd * Wd;
    int32_t rs = 0, len = 0;
    if (lane < nruns) {
        const int32_t cx = cid % geo.g[0];
        const int32_t cy = (cid / geo.g[0]) % geo.g[1];
        const int32_t cz = cid / (geo.g[0] * geo.g[1]);
        const int32_t z = cz + lane / Wd - S, y = cy + lane % Wd - S;
        if (z >= 0 && z < geo.g[2] && y >= 0 && y < geo.g[1]) {
            const int32_t xlo = cx > S - 1 ? cx - S : 0;
            const int32_t xhi = cx + S < geo.g[0] ? cx + S : geo.g[0] - 1;
            const int64_t row = (int64_t)geo.g[0] * ((int64_t)y + (int64_t)geo.g[1] * z);
            const int64_t b = cell_start[row + xlo], e = cell_start[row + xhi + 1];
            rs = (int32_t)b;
            len = e > b ? (int32_t)(e - b) : 0;
        }
    }
    int32_t inc = len;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int32_t v = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += v;
    }
    if (lane < nruns) {
        s_rs[wid][lane] = rs;
        s_cum[wid][lane + 1] = inc;
    }
    if (lane == 0) s_cum[wid][0] = 0;
    const int32_t total = __shfl_sync(0xffffffffu, inc, nruns - 1);
    __syncwarp();

    int32_t qi[kUnitQueries];
    float qx[kUnitQueries], qy[kUnitQueries], qz[kUnitQueries];
    int64_t w[kUnitQueries];
    uint64_t qkey[kUnitQueries];
    int32_t cnt[kUnitQueries];
#pragma unroll
    for (int k = 0; k < kUnitQueries; ++k) {
        const int64_t qk = q0 + k;
        const bool ok = qk < qend;
        const float4 f = ok ? qxf4[qk] : make_float4(INFINITY, INFINITY, INFINITY, 0.f);
        qx[k] = f.x;
        qy[k] = f.y;
        qz[k] = f.z;
        qi[k] = ok ? qperm[qk] : -1;  // the other point's index
        w[k] = kFill && ok ? qrow_off[qk] : 0;
        qkey[k] = ok ? (uint64_t)(uint32_t)qi[k] << bits_n : 0;
        cnt[k] = 0;
    }
    const unsigned lt = (1u << lane) - 1u;
    unsigned long long n_exact = 0;
    int r = 0;
    int32_t hi = s_cum[wid][1], base = s_rs[wid][0];
    for (int32_t t = lane; t - lane < total; t += 32) {
        while (t >= hi && r < nruns - 1) {
            ++r;
            base = s_rs[wid][r] - hi;
            hi = s_cum[wid][r + 1];
        }
        const int32_t j = base + t;
        const float4 cf = t < total ? xf4[j] : make_float4(INFINITY, INFINITY, INFINITY, 0.f);
        bool in[kUnitQueries], amb[kUnitQueries];
        bool any_amb = false;
#pragma unroll
        for (int k = 0; k < kUnitQueries; ++k) {
            const float ex = qx[k] - cf.x, ey = qy[k] - cf.y, ez = qz[k] - cf.z;
            const float sf = fmaf(ez, ez, fmaf(ey, ey, ex * ex));
            in[k] = sf <= sp.thr_in;
            amb[k] = !in[k] && sf <= sp.thr_out && t < total && qi[k] >= 0;
            any_amb |= amb[k];
        }
        if (__any_sync(0xffffffffu, any_amb)) {
#pragma unroll
            for (int k = 0; k < kUnitQueries; ++k)
                if (amb[k]) {
                    in[k] = exact_in_radius(xq + (int64_t)qi[k] * d, x + (int64_t)perm[j] * d, d, sp);
                    ++n_exact;
                }
        }
#pragma unroll
        for (int k = 0; k < kUnitQueries; ++k) {
            const unsigned hit = __ballot_sync(0xffffffffu, in[k]);
            if (kFill && in[k]) keys[w[k] + cnt[k] + __popc(hit & lt)] = qkey[k] | (uint64_t)(uint32_t)perm[j];
            cnt[k] += __popc(hit);
        }
    }
    if (!kFill && lane == 0) {
#pragma unroll
        for (int k = 0; k < kUnitQueries; ++k)
            if (q0 + k < qend) qdeg[q0 + k] = cnt[k];
    }
    if (!kFill) {
        for (int o = 16; o > 0; o >>= 1) n_exact += __shfl_down_sync(0xffffffffu, n_exact, o);
        if (lane == 0 && n_exact) atomicAdd(&counters[0], n_exact);
    }
}

// Rows of other points (queries) against this set (candidates): the same
// float32 test with the float64 band, candidates in ascending index order.
// (NeighboursGetterExtBruteForce._get_other, src/cnnclustering/_types.pyx:1712-1731.)
template <bool kFill>
__global__ void __launch_bounds__(kTileWarps * 32) cross_tile_kernel(
    const double *__restrict__ xq, const float *__restrict__ xqf, int64_t m, const double *__restrict__ x,
    const float *__restrict__ xf, int64_t n, int d, SearchParams sp, int32_t *__restrict__ deg,
    const int64_t *__restrict__ row_off, int32_t *__restrict__ cols) {
    extern __shared__ float smem[];
    const int ds = d + 1;
    float *cand = smem;
    float *qry = smem + kTileCand * ds;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int64_t p = (int64_t)blockIdx.x * kTileWarps + wid;
    const bool active = p < m;
    for (int k = lane; k < d; k += 32) qry[wid * ds + k] = active ? xqf[p * d + k] : 0.f;
    const unsigned lt = (1u << lane) - 1u;
    int64_t w = (kFill && active) ? row_off[p] : 0;
    int64_t cnt = 0;
    for (int64_t j0 = 0; j0 < n; j0 += kTileCand) {
        __syncthreads();
        for (int e = threadIdx.x; e < kTileCand * d; e += blockDim.x) {
            const int r = e / d, k = e - r * d;
            const int64_t j = j0 + r;
            cand[r * ds + k] = j < n ? xf[j * d + k] : 0.f;
        }
        __syncthreads();
        const int64_t j = j0 + lane;
        bool in = false;
        if (active && j < n) {
            float sf = 0.f;
            const float *cr = cand + lane * ds;
            const float *qr = qry + wid * ds;
            for (int k = 0; k < d; ++k) {
                const float t = qr[k] - cr[k];
                sf = fmaf(t, t, sf);
            }
            if (sf <= sp.thr_in) in = true;
            else if (!(sf > sp.thr_out)) in = exact_in_radius(xq + p * d, x + j * d, d, sp);
        }
        const unsigned hit = __ballot_sync(0xffffffffu, in);
        if (kFill && in) cols[w + cnt + __popc(hit & lt)] = (int32_t)j;
        cnt += __popc(hit);
    }
    if (!kFill && active && lane == 0) deg[p] = (int32_t)cnt;
}

// Precomputed distances: row i keeps every j with distance(i, j) <= rc,
// ascending (NeighboursGetterExtBruteForce._get over
// MetricExtPrecomputed / DistanceGetterExtLookup, _types.pyx:1692-1710,
// 2108-2127, 2019-2037).  Linear layout: the upper triangle by rows,
// distance(a, b) for a < b at a (n - 1) - (a^2 - a) / 2 + b - a - 1, and 0
// on the diagonal (_types.pyx:1127-1143).  One warp per row.
template <bool kFill>
__global__ void distance_rows_kernel(const double *__restrict__ dist, int layout, int64_t n, double rc,
                                     int32_t *__restrict__ deg, const int64_t *__restrict__ row_off,
                                     int32_t *__restrict__ cols) {
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    const int64_t warp0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t i = warp0; i < n; i += nwarps) {
        int64_t w = kFill ? row_off[i] : 0;
        int64_t cnt = 0;
        const int64_t base_i = i * (n - 1) - (i * i - i) / 2;  // start of i's block (j > i)
        for (int64_t j0 = 0; j0 < n; j0 += 32) {
            const int64_t j = j0 + lane;
            bool in = false;
            if (j < n) {
                double v;
                if (layout == CNN_DIST_SQUARE) {
                    v = dist[i * n + j];
                } else if (j == i) {
                    v = 0.0;
                } else if (j > i) {
                    v = dist[base_i + j - i - 1];
                } else {
                    v = dist[j * (n - 1) - (j * j - j) / 2 + i - j - 1];
                }
                in = v <= rc;
            }
            const unsigned hit = __ballot_sync(0xffffffffu, in);
            if (kFill && in) cols[w + cnt + __popc(hit & lt)] = (int32_t)j;
            cnt += __popc(hit);
        }
        if (!kFill && lane == 0) deg[i] = (int32_t)cnt;
    }
}

__global__ void to_f32_kernel(const double *__restrict__ x, int64_t n, int d, const double *__restrict__ lo,
                              float *__restrict__ xf) {
    const int64_t total = n * d;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        int k = (int)(e % d);
        double v = x[e];
        xf[e] = isfinite(v) ? (float)__dsub_rn(v, lo[k]) : __int_as_float(0x7fc00000);
    }
}

__global__ void set_last_zero_kernel(int32_t *deg, int64_t n) { deg[n] = 0; }

// ---- export / import ----------------------------------------------------------
__global__ void export_keys_kernel(const int64_t *__restrict__ row_off, const int32_t *__restrict__ cols,
                                   const int32_t *__restrict__ perm, int64_t n, int bits_n,
                                   uint64_t *__restrict__ keys) {
    const int lane = threadIdx.x & 31;
    const int64_t p = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    if (p >= n) return;
    const uint64_t r = (uint64_t)(uint32_t)perm[p] << bits_n;
    for (int64_t e = row_off[p] + lane; e < row_off[p + 1]; e += 32)
        keys[e] = r | (uint64_t)(uint32_t)perm[cols[e]];
}

__global__ void keys_to_cols_kernel(const uint64_t *__restrict__ keys, int64_t nnz, int bits_n,
                                    int32_t *__restrict__ cols) {
    const uint64_t mask = (1ull << bits_n) - 1;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nnz; e += (int64_t)gridDim.x * blockDim.x)
        cols[e] = (int32_t)(keys[e] & mask);
}

__global__ void deg_by_point_kernel(const int32_t *__restrict__ deg, const int32_t *__restrict__ inv, int64_t n,
                                    int64_t *__restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = deg[inv[i]];
    if (blockIdx.x == 0 && threadIdx.x == 0) out[n] = 0;
}

__global__ void import_keys_kernel(const int64_t *__restrict__ off, const int32_t *__restrict__ idx, int64_t n,
                                   int bits_n, uint64_t *__restrict__ keys, int32_t *__restrict__ deg,
                                   unsigned long long *__restrict__ bad) {
    const int lane = threadIdx.x & 31;
    const int64_t p = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    if (p >= n) return;
    const int64_t s = off[p], e = off[p + 1];
    if (lane == 0) deg[p] = (int32_t)(e - s);
    for (int64_t k = s + lane; k < e; k += 32) {
        int32_t c = idx[k];
        if (c < 0 || (int64_t)c >= n) { atomicAdd(bad, 1ull); c = 0; }
        keys[k] = ((uint64_t)p << bits_n) | (uint64_t)(uint32_t)c;
    }
}

__global__ void check_offsets_kernel(const int64_t *__restrict__ off, int64_t n, unsigned long long *bad) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
        int64_t len = off[p + 1] - off[p];
        if (len < 0 || len > 0x7fffffff) atomicAdd(bad, 1ull);
    }
}

int bits_for(int64_t n) {
    int b = 1;
    while (b < 62 && (int64_t(1) << b) < n) ++b;
    return b;
}

// Float32 prefilter thresholds.  ext[k] = max |x_k - lo_k| over finite
// points.  For a pair with true squared distance D <= 4 R^2 the float32
// value sf differs from D by at most err (derivation in the comments);
// sf <= rc2 - err - margin then implies the float64 s <= rc2 and
// sf > rc2 + err + margin implies s > rc2.  Pairs with D > 4 R^2 have
// sf > rc2 + err + margin whenever the per-coordinate error is below
// R/1000, which is required for the filter to be used at all.
bool filter_thresholds(const std::vector<double> &ext, double R, double rc2, float *thr_in,
                       float *thr_out, double *band, const std::vector<double> *bounds = nullptr) {
    const double u32 = ldexp(1.0, -24), u64 = ldexp(1.0, -53);
    const int d = (int)ext.size();
    double emax = 0;
    for (double e : ext) emax = std::max(emax, e);
    if (!(R > 1e-30) || !(R < 1e30) || !isfinite(emax)) return false;
    // conversion error of one coordinate: rounding of (x - lo) in float64,
    // then to float32
    double err = 0;
    for (int k = 0; k < d; ++k) {
        double delta = ext[k] * (u32 + 2 * u64);
        if (delta > 1e-3 * R) return false;
        // |dx - D_k| <= 2 delta + u32 (|D_k| + 2 delta) with |D_k| <= 2R
        double eta = 2 * delta + u32 * (2 * R + 2 * delta);
        const double L = bounds ? (*bounds)[k] : 0.0;
        if (L > 0) {
            // minimum image: |a - b| (float32, up to the extent), then fmod
            // (exact) and bound - d.  The image map is 1-Lipschitz in the
            // difference and moves by at most (E/L + 1)|L_f - L| with the
            // float32 bound; the final subtraction rounds once more, and
            // the float64 reference rounds its own difference.
            eta = 2 * delta + u32 * (ext[k] + 2 * delta) + u32 * (ext[k] + L) + u32 * L * (1 + u32) +
                  4 * u64 * (ext[k] + L);
            if (eta > 1e-3 * R) return false;
        }
        err += eta * (4 * R + eta);
    }
    // rounding of the float32 squares and sum (fma chain): gamma_{d+1}
    double gam = (d + 2) * u32 / (1 - (d + 2) * u32);
    err += gam * (4 * R * R) * 1.0 + gam * err;
    // float64 result vs exact sum, and the sqrt-metric boundary: a few ulps
    double margin = 8 * (d + 2) * u64 * rc2 + 1e-300;
    double b = 2 * (err + margin);          // safety factor 2
    if (!(b < 0.25 * rc2)) return false;
    double tin = rc2 - b, tout = rc2 + b;
    float fin = (float)tin, fout = (float)tout;
    if ((double)fin > tin) fin = nextafterf(fin, -INFINITY);
    if ((double)fout < tout) fout = nextafterf(fout, INFINITY);
    if (!(fin > 0.f)) fin = -1.f;  // never "certainly in" by float32
    *thr_in = fin;
    *thr_out = fout;
    *band = b;
    return true;
}

}  // namespace

// ---------------------------------------------------------------------------
cnn_status build_neighbours_impl(cnn_context *ctx, double radius_cutoff, int metric, int fpmode, int form) {
    const int64_t n = ctx->n;
    const int d = ctx->d;
    cudaStream_t st = ctx->stream;
    ctx->have_graph = false;
    ctx->grid_geo_valid = false;
    ctx->graph_mask = false;
    ctx->csr_valid = true;
    ctx->tune_pending = false;
    ctx->split_valid = false;
    ctx->graph_slots = false;
    ctx->nnz_pending = false;
    ++ctx->graph_generation;
    ctx->stats = cnn_stats{};
    stages_reset(ctx, 0, cnn_context::kSlots - 1);
    ctx->search_stats_pending = false;
    ctx->fit_stats_pending = false;
    ctx->stats.n_points = n;
    CNN_TRY(ctx->ensure(ctx->counters, kCounterSlots * sizeof(unsigned long long)));
    CNN_CUDA(ctx, cudaMemsetAsync(ctx->counters.ptr, 0, kCounterSlots * sizeof(unsigned long long), st));
    CNN_TRY(ctx->ensure(ctx->deg, sizeof(int32_t) * (size_t)(n + 1)));
    CNN_TRY(ctx->ensure(ctx->row_off, sizeof(int64_t) * (size_t)(n + 1)));
    CNN_TRY(ctx->ensure(ctx->perm, sizeof(int32_t) * (size_t)(n > 0 ? n : 1)));
    CNN_TRY(ctx->ensure(ctx->inv, sizeof(int32_t) * (size_t)(n > 0 ? n : 1)));

    SearchParams sp;
    sp.rc = radius_cutoff;
    sp.metric = metric;
    sp.fpmode = fpmode;
    sp.thr_in = -1.f;
    sp.thr_out = INFINITY;

    if (n == 0) {
        CNN_CUDA(ctx, cudaMemsetAsync(ctx->row_off.ptr, 0, sizeof(int64_t), st));
        ctx->nnz = 0;
        ctx->identity_perm = true;
        ctx->have_graph = true;
        return CNN_OK;
    }

    if (metric == CNN_METRIC_PRECOMPUTED) {
        if (!ctx->dist_set) return ctx->fail(CNN_ERR_STATE, "precomputed metric: call cnn_set_distances first");
        int32_t *deg = ctx->deg.as<int32_t>();
        int64_t *row_off = ctx->row_off.as<int64_t>();
        CNN_TRY(iota_i32(ctx, ctx->perm.as<int32_t>(), n));
        CNN_TRY(iota_i32(ctx, ctx->inv.as<int32_t>(), n));
        const unsigned blocks = std::min<unsigned>(grid_for(n * 32, 256), ctx->sm_count * 16u);
        stage_begin(ctx, 2);
        distance_rows_kernel<false><<<blocks, 256, 0, st>>>(ctx->dist, ctx->dist_layout, n, radius_cutoff, deg, nullptr,
                                                            nullptr);
        CNN_LAUNCH_CHECK(ctx);
        stage_end(ctx, 2);
        set_last_zero_kernel<<<1, 1, 0, st>>>(deg, n);
        CNN_LAUNCH_CHECK(ctx);
        CNN_TRY(scan_exclusive_i32_to_i64(ctx, deg, row_off, n + 1));
        int64_t nnz = 0;
        CNN_CUDA(ctx, cudaMemcpyAsync(&nnz, row_off + n, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
        CNN_CUDA(ctx, cudaStreamSynchronize(st));
        CNN_TRY(ctx->ensure(ctx->cols, sizeof(int32_t) * (size_t)(nnz > 0 ? nnz : 1)));
        stage_begin(ctx, 4);
        distance_rows_kernel<true><<<blocks, 256, 0, st>>>(ctx->dist, ctx->dist_layout, n, radius_cutoff, nullptr,
                                                           row_off, ctx->cols.as<int32_t>());
        CNN_LAUNCH_CHECK(ctx);
        stage_end(ctx, 4);
        CNN_CUDA(ctx, cudaStreamSynchronize(st));
        ctx->identity_perm = true;
        ctx->stats.search_kind = 4;
        ctx->stats.n_candidates = n * n;
        ctx->stats.n_nonzero = nnz;
        ctx->nnz = nnz;
        ctx->have_graph = true;
        return CNN_OK;
    }
    if (!ctx->x) return ctx->fail(CNN_ERR_STATE, "no points: call cnn_set_points first");

    // search radius R in coordinate units.  A NaN or negative cutoff admits
    // no pair; +inf admits every pair whose distance is not NaN, which only
    // the all-pairs search with every pair decided in float64 can express.
    double R = metric == CNN_METRIC_EUCLIDEAN ? radius_cutoff : sqrt(radius_cutoff);
    const bool radius_ok = radius_cutoff >= 0.0 && isfinite(radius_cutoff);
    const bool radius_inf = radius_cutoff == INFINITY;
    const bool periodic = metric == CNN_METRIC_EUCLIDEAN_PERIODIC_REDUCED;
    if (periodic) {
        // minimum-image distances: the all-pairs search with the periodic
        // float32 test and float64 recheck
        if ((int)ctx->periodic_bounds.size() != d)
            return ctx->fail(CNN_ERR_INVALID_ARG, "periodic metric: call cnn_set_periodic_bounds with n_dim bounds");
        CNN_TRY(ctx->ensure(ctx->bounds_dev, (sizeof(double) + sizeof(float)) * (size_t)d + 64));
        std::vector<float> bf(d);
        for (int k = 0; k < d; ++k) bf[k] = (float)ctx->periodic_bounds[k];
        double *bd_dev = ctx->bounds_dev.as<double>();
        float *bf_dev = reinterpret_cast<float *>(bd_dev + d);
        CNN_CUDA(ctx, cudaMemcpyAsync(bd_dev, ctx->periodic_bounds.data(), sizeof(double) * d, cudaMemcpyHostToDevice,
                                      st));
        CNN_CUDA(ctx, cudaMemcpyAsync(bf_dev, bf.data(), sizeof(float) * d, cudaMemcpyHostToDevice, st));
        CNN_CUDA(ctx, cudaStreamSynchronize(st));  // bf leaves scope
        sp.bd = bd_dev;
        sp.bf = bf_dev;
    }

    const bool all_pairs = ctx->search_pref == CNN_SEARCH_ALL_PAIRS;
    if (d >= 16 && radius_ok && !periodic && !all_pairs) {
        // tensor-core Gram search; declines (used = false) for non-finite
        // data or when the float64 band would hold too many pairs
        bool used = false;
        stage_begin(ctx, 2);
        CNN_TRY(gram_search_impl(ctx, radius_cutoff, metric, fpmode, &used));
        stage_end(ctx, 2);
        if (used) {  // the graph in the search's internal order (perm / inv set by it)
            ctx->stats.search_kind = 3;
            ctx->stats.n_nonzero = ctx->nnz;
            CNN_CUDA(ctx, cudaStreamSynchronize(st));
            ctx->have_graph = true;
            return CNN_OK;
        }
        CNN_CUDA(ctx, cudaMemsetAsync(ctx->counters.ptr, 0, kCounterSlots * sizeof(unsigned long long), st));
        ctx->stats = cnn_stats{};
    stages_reset(ctx, 0, cnn_context::kSlots - 1);
        ctx->stats.n_points = n;
    }

    stage_begin(ctx, 0);
    // ---- extents of finite points
    std::vector<double> lo(d), hi(d);
    int64_t n_bad = 0;
    {
        const int blocks = (int)std::min<int64_t>(128, (n + 255) / 256);
        CNN_TRY(ctx->ensure(ctx->scratch_a, sizeof(double) * (size_t)blocks * (size_t)d * 3 + 64));
        extent_partial_kernel<<<dim3(blocks, d), 256, 0, st>>>(ctx->x, n, d, ctx->scratch_a.as<double>());
        CNN_LAUNCH_CHECK(ctx);
        std::vector<double> part((size_t)blocks * d * 3);
        CNN_TRY(read_back(ctx, part.data(), ctx->scratch_a.ptr, sizeof(double) * part.size()));
        for (int k = 0; k < d; ++k) { lo[k] = INFINITY; hi[k] = -INFINITY; }
        double bad0 = 0;
        for (int b = 0; b < blocks; ++b)
            for (int k = 0; k < d; ++k) {
                const double *o = &part[((size_t)b * d + k) * 3];
                lo[k] = std::min(lo[k], o[0]);
                hi[k] = std::max(hi[k], o[1]);
                if (k == 0) bad0 += o[2];
            }
        n_bad = (int64_t)bad0;  // rows with a non-finite first coordinate (diagnostic)
        for (int k = 0; k < d; ++k)
            if (!(lo[k] <= hi[k])) { lo[k] = 0; hi[k] = 0; }  // no finite point
    }
    (void)n_bad;
    stage_end(ctx, 0);

    std::vector<double> ext(d);
    for (int k = 0; k < d; ++k) ext[k] = std::max(std::fabs(hi[k] - lo[k]), 0.0);
    for (int k = 0; k < 3; ++k) ctx->grid_extent[k] = k < d ? ext[k] : 0.0;
    // periodic dimensions: the float32 values are either x - lo (all-pairs
    // search) or x mapped into [0, L) (wrapped grid; mapping error a few
    // ulps of max |x|): the bound takes the larger magnitude of the two
    std::vector<double> ext_f = ext;
    if (periodic)
        for (int k = 0; k < d; ++k) {
            const double L = ctx->periodic_bounds[k];
            if (L > 0)
                ext_f[k] = std::max(ext[k], L + ldexp(std::max(std::fabs(lo[k]), std::fabs(hi[k])), -28));
        }
    double band = 0;
    bool filt = false;
    if (radius_ok && (metric == CNN_METRIC_EUCLIDEAN_REDUCED || metric == CNN_METRIC_EUCLIDEAN || periodic)) {
        const double rc2 = metric == CNN_METRIC_EUCLIDEAN ? radius_cutoff * radius_cutoff : radius_cutoff;
        filt = filter_thresholds(ext_f, R, rc2, &sp.thr_in, &sp.thr_out, &band,
                                 periodic ? &ctx->periodic_bounds : nullptr);
    }
    if (!radius_ok && !radius_inf) {
        // nothing satisfies `s <= NaN`; a negative cutoff admits nothing
        sp.thr_in = -1.f;
        sp.thr_out = -1.f;  // everything is "certainly out"
        filt = true;
    }
    ctx->stats.filter_enabled = filt ? 1 : 0;
    ctx->stats.filter_band = band;

    // ---- choose the search
    GridGeom geo{};
    bool use_grid = d <= 3 && radius_ok && R > 0 && isfinite(R) && !all_pairs;
    if (use_grid && periodic) {
        // a wrapped grid (reach 1): every periodic dimension's mapping into
        // [0, L) must be exact to far below the 1e-6 R by which cells exceed
        // R, and each needs at least 3 cells (checked below)
        for (int k = 0; k < d; ++k) {
            const double L = ctx->periodic_bounds[k];
            if (L > 0 && (!(L < 1e30) || !(ldexp(std::max(std::fabs(lo[k]), std::fabs(hi[k])) + L, -50) < 1e-7 * R)))
                use_grid = false;
        }
    }
    if (use_grid) {
        // cells of edge h >= R / reach: a qualifying pair lies at most `reach`
        // cells apart in every dimension; reach 2 scans (5/2)^3 = 15.6 R^3
        // around a point instead of 27 R^3 (fewer candidates per neighbour)
        geo.reach = periodic ? 1 : ctx->grid_reach;
        double h = R / geo.reach * (1.0 + 1e-6);
        auto wraps = [&](int k) { return periodic && k < d && ctx->periodic_bounds[k] > 0; };
        // cells cost 12 bytes each (count + start); allow up to 64 per point
        // (at most 64M) so sparse sets in large boxes keep cells of edge ~R
        const double max_cells = std::max<double>(std::min<double>(64.0 * (double)n, 67108864.0), 4096.0);
        for (int attempt = 0; attempt < 200; ++attempt) {
            double cells = 1;
            for (int k = 0; k < 3; ++k) {
                // a wrapping dimension: floor(L / h) cells of edge L / g >= h
                double g = k >= d ? 1.0 : wraps(k) ? floor(ctx->periodic_bounds[k] / h) : floor(ext[k] / h) + 1.0;
                geo.g[k] = (int32_t)std::max(1.0, std::min(g, 2.0e9));
                cells *= std::max(g, 1.0);
            }
            if (cells <= max_cells && cells < 2.0e9) break;
            h *= 1.25;
        }
        geo.h = h;
        geo.inv_h = 1.0 / h;
        for (int k = 0; k < 3; ++k) {
            geo.lo[k] = k < d && !wraps(k) ? lo[k] : 0.0;
            geo.inv_hk[k] = geo.inv_h;
            if (wraps(k)) {
                geo.wrap |= 1 << k;
                geo.L[k] = ctx->periodic_bounds[k];
                geo.inv_hk[k] = (double)geo.g[k] / geo.L[k];
                sp.wl[k] = (float)geo.L[k];
                sp.whalf[k] = 0.5f * sp.wl[k];
                if (geo.g[k] < 3) use_grid = false;  // a 3-cell stencil would meet a cell twice
            }
        }
        geo.ncells = (int64_t)geo.g[0] * geo.g[1] * geo.g[2];
        if (geo.ncells >= 0x7ffffff0LL) use_grid = false;
    }
    ctx->stats.search_kind = use_grid ? 1 : 2;
    ctx->grid_geo = geo;
    ctx->grid_geo_valid = use_grid;

    int32_t *deg = ctx->deg.as<int32_t>();
    int64_t *row_off = ctx->row_off.as<int64_t>();
    int64_t grid_items = 0;
    int64_t n_candidates = -1;  // pairs looked at (grid path: from the slot sizes)
    bool use_slots = false;
    // Which form the cell-grid graph takes: lists (the merge intersection),
    // masks (the bitset intersection), or -- the first time a workload
    // profile is seen under CNN_INTERSECT_AUTO -- both, so that the first fit
    // can time the two and the tuner keep the faster (tuner.cu).
    const int pref = form == kFormLists ? CNN_INTERSECT_MERGE
                     : form == kFormMasks ? CNN_INTERSECT_BITSET
                                          : ctx->intersect_pref;
    // the mask form reads rows through 3 x 3 x 3 stencils: cells of reach 1 only
    bool use_mask = use_grid && pref == CNN_INTERSECT_BITSET && geo.reach == 1 && !geo.wrap;
    bool use_lists = !use_mask;
    bool calibrate = false;
    unsigned long long *counters = ctx->counters.as<unsigned long long>();

    if (use_grid) {
        stage_begin(ctx, 1);
        CNN_TRY(ctx->ensure(ctx->cell_of, sizeof(int32_t) * (size_t)n));
        CNN_TRY(ctx->ensure(ctx->cell_start, sizeof(int64_t) * (size_t)(geo.ncells + 2)));
        CNN_TRY(ctx->ensure(ctx->scratch_b, sizeof(int32_t) * (size_t)(geo.ncells + 2)));
        CNN_TRY(ctx->ensure(ctx->scratch_a, sizeof(int32_t) * (size_t)n));
        CNN_TRY(ctx->ensure(ctx->xf4, sizeof(float4) * (size_t)n));
        int32_t *cell_count = ctx->scratch_b.as<int32_t>();
        CNN_CUDA(ctx, cudaMemsetAsync(cell_count, 0, sizeof(int32_t) * (size_t)(geo.ncells + 2), st));
        const unsigned gb = std::min<unsigned>(grid_for(n, 256), ctx->sm_count * 16u);
        int32_t *slot = ctx->scratch_a.as<int32_t>();
        cell_assign_kernel<<<gb, 256, 0, st>>>(ctx->x, n, d, geo, ctx->cell_of.as<int32_t>(), slot, cell_count);
        CNN_LAUNCH_CHECK(ctx);
        CNN_TRY(scan_exclusive_i32_to_i64(ctx, cell_count, ctx->cell_start.as<int64_t>(), geo.ncells + 2));
        place_kernel<<<gb, 256, 0, st>>>(ctx->cell_of.as<int32_t>(), slot, ctx->cell_start.as<int64_t>(), n, ctx->x, d,
                                         geo, ctx->perm.as<int32_t>(), ctx->inv.as<int32_t>(),
                                         ctx->xf4.as<float4>());
        CNN_LAUNCH_CHECK(ctx);

        // work items: (cell, first query) for every kUnitQueries queries of a
        // cell; slots: every row's upper bound (its cell's candidate count),
        // and for the mask form every row's words
        CNN_TRY(ctx->ensure(ctx->io_a, sizeof(int32_t) * (size_t)(geo.ncells + 1)));
        CNN_TRY(ctx->ensure(ctx->io_b, sizeof(int64_t) * (size_t)(geo.ncells + 3)));  // + the slot and word totals
        CNN_TRY(ctx->ensure(ctx->grid_slot_base, sizeof(int64_t) * (size_t)(geo.ncells + 2)));
        int64_t *slot_base = ctx->grid_slot_base.as<int64_t>();
        CNN_TRY(ctx->ensure(ctx->scratch_c, sizeof(int64_t) * (size_t)(geo.ncells + 2)));
        const unsigned cgrid = std::min<unsigned>(grid_for(geo.ncells, 256), ctx->sm_count * 16u);
        cell_units_kernel<kUnitQueries><<<cgrid, 256, 0, st>>>(ctx->cell_start.as<int64_t>(), geo,
                                                               ctx->io_a.as<int32_t>(), ctx->scratch_c.as<int64_t>());
        CNN_LAUNCH_CHECK(ctx);
        CNN_TRY(scan_exclusive_i32_to_i64(ctx, ctx->io_a.as<int32_t>(), ctx->io_b.as<int64_t>(), geo.ncells + 1));
        CNN_TRY(scan_exclusive_i64(ctx, ctx->scratch_c.as<int64_t>(), slot_base, geo.ncells + 1));
        int64_t hcounts[3] = {0, 0, 0};  // work items, candidate slots, mask words
        CNN_CUDA(ctx, cudaMemcpyAsync(ctx->io_b.as<int64_t>() + geo.ncells + 1, slot_base + geo.ncells,
                                      sizeof(int64_t), cudaMemcpyDeviceToDevice, st));  // both totals side by side
        CNN_TRY(read_back(ctx, hcounts, ctx->io_b.as<int64_t>() + geo.ncells, 2 * sizeof(int64_t)));
        const int64_t nitems = hcounts[0];
        if (pref == CNN_INTERSECT_AUTO && geo.reach == 1 && !geo.wrap) {
            int choice = CNN_INTERSECT_AUTO;
            ctx->tune_key = tuner_key(ctx, n, hcounts[1]);
            if (tuner_lookup(ctx->tune_key, &choice)) {
                use_mask = choice == CNN_INTERSECT_BITSET;
                use_lists = !use_mask;
            } else {
                calibrate = use_mask = use_lists = true;  // the first fit times both forms
            }
        }
        int64_t *word_base = nullptr;
        if (use_mask) {
            // the mask form: every point's cell, every row's words
            CNN_TRY(ctx->ensure(ctx->pcell, sizeof(int32_t) * (size_t)n));
            point_cell_kernel<<<gb, 256, 0, st>>>(ctx->cell_of.as<int32_t>(), ctx->perm.as<int32_t>(), n,
                                                  ctx->pcell.as<int32_t>());
            CNN_LAUNCH_CHECK(ctx);
            CNN_TRY(ctx->ensure(ctx->mbase, sizeof(int64_t) * (size_t)(geo.ncells + 2)));
            word_base = ctx->mbase.as<int64_t>();
            cell_slots_kernel<true><<<cgrid, 256, 0, st>>>(ctx->cell_start.as<int64_t>(), geo,
                                                           ctx->scratch_c.as<int64_t>());
            CNN_LAUNCH_CHECK(ctx);
            CNN_TRY(scan_exclusive_i64(ctx, ctx->scratch_c.as<int64_t>(), word_base, geo.ncells + 1));
            CNN_TRY(read_back(ctx, &hcounts[2], word_base + geo.ncells, sizeof(int64_t)));
        }
        // one pass into slots when they take at most 4 GiB, else count + fill
        use_slots = use_lists && hcounts[1] <= (int64_t(1) << 30);
        if (use_mask) {
            // + 2 words: a row's last word may be read together with the next one
            CNN_TRY(ctx->ensure(ctx->masks, sizeof(uint32_t) * (size_t)(hcounts[2] + 2)));
            CNN_CUDA(ctx, cudaMemsetAsync(ctx->masks.as<uint32_t>() + hcounts[2], 0, 2 * sizeof(uint32_t), st));
        }
        if (use_slots) {
            CNN_TRY(ctx->ensure(ctx->grid_slot_cols, sizeof(int32_t) * (size_t)(hcounts[1] > 0 ? hcounts[1] : 1)));
            CNN_TRY(ctx->ensure(ctx->grid_qslot, sizeof(int64_t) * (size_t)n));
        }
        CNN_TRY(ctx->ensure(ctx->io_c, sizeof(int2) * (size_t)(nitems > 0 ? nitems : 1)));
        item_fill_kernel<kUnitQueries><<<std::min<unsigned>(grid_for(geo.ncells, 256), ctx->sm_count * 16u), 256, 0, st>>>(
            ctx->cell_start.as<int64_t>(), geo.ncells, ctx->io_b.as<int64_t>(), ctx->io_c.as<int2>());
        CNN_LAUNCH_CHECK(ctx);
        grid_items = nitems;
        stage_end(ctx, 1);

        stage_begin(ctx, 2);
        // deg[n] = 0 as well: the tail of the row-offset scan
        CNN_CUDA(ctx, cudaMemsetAsync(deg, 0, sizeof(int32_t) * (size_t)(n + 1), st));
        if (calibrate) CNN_CUDA(ctx, cudaEventRecord(ctx->tune_ev[0], st));
        if (nitems > 0 && use_mask) {
            grid_unit_kernel<kMask><<<(unsigned)((nitems + kUnitWarps - 1) / kUnitWarps), kUnitWarps * 32, 0, st>>>(
                ctx->io_c.as<int2>(), nitems, ctx->x, d, geo, sp, ctx->perm.as<int32_t>(),
                ctx->cell_start.as<int64_t>(), ctx->xf4.as<float4>(), deg, word_base,
                reinterpret_cast<int32_t *>(ctx->masks.as<uint32_t>()), counters, nullptr);
            CNN_LAUNCH_CHECK(ctx);
        }
        if (calibrate) {
            // the list search as well: the same rows and lengths, counted once
            CNN_CUDA(ctx, cudaEventRecord(ctx->tune_ev[1], st));
            CNN_CUDA(ctx, cudaMemsetAsync(counters, 0, 2 * sizeof(unsigned long long), st));
        }
        if (!use_lists) {
            // masks only
        } else if (nitems > 0 && use_slots) {
            (geo.wrap ? grid_unit_kernel<kSlots, true> : grid_unit_kernel<kSlots, false>)<<<(unsigned)((nitems + kUnitWarps - 1) / kUnitWarps), kUnitWarps * 32, 0, st>>>(
                ctx->io_c.as<int2>(), nitems, ctx->x, d, geo, sp, ctx->perm.as<int32_t>(),
                ctx->cell_start.as<int64_t>(), ctx->xf4.as<float4>(), deg, slot_base,
                ctx->grid_slot_cols.as<int32_t>(), counters, ctx->grid_qslot.as<int64_t>());
            CNN_LAUNCH_CHECK(ctx);
        } else if (nitems > 0) {
            (geo.wrap ? grid_unit_kernel<kCount, true> : grid_unit_kernel<kCount, false>)<<<(unsigned)((nitems + kUnitWarps - 1) / kUnitWarps), kUnitWarps * 32, 0, st>>>(
                ctx->io_c.as<int2>(), nitems, ctx->x, d, geo, sp, ctx->perm.as<int32_t>(),
                ctx->cell_start.as<int64_t>(), ctx->xf4.as<float4>(), deg, nullptr, nullptr, counters, nullptr);
            CNN_LAUNCH_CHECK(ctx);
        }
        if (calibrate) CNN_CUDA(ctx, cudaEventRecord(ctx->tune_ev[2], st));
        n_candidates = hcounts[1];  // every query against its cell's candidate runs
        stage_end(ctx, 2);
        ctx->identity_perm = false;
    } else {
        stage_begin(ctx, 1);
        CNN_TRY(iota_i32(ctx, ctx->perm.as<int32_t>(), n));
        CNN_TRY(iota_i32(ctx, ctx->inv.as<int32_t>(), n));
        CNN_TRY(ctx->ensure(ctx->scratch_b, sizeof(float) * (size_t)n * d));
        CNN_TRY(ctx->ensure(ctx->scratch_a, sizeof(double) * (size_t)d + 64));
        CNN_CUDA(ctx, cudaMemcpyAsync(ctx->scratch_a.ptr, lo.data(), sizeof(double) * d, cudaMemcpyHostToDevice, st));
        const unsigned gb = std::min<unsigned>(grid_for(n * d, 256), ctx->sm_count * 16u);
        to_f32_kernel<<<gb, 256, 0, st>>>(ctx->x, n, d, ctx->scratch_a.as<double>(), ctx->scratch_b.as<float>());
        CNN_LAUNCH_CHECK(ctx);
        stage_end(ctx, 1);
        if (d > 1024) return ctx->fail(CNN_ERR_UNSUPPORTED, "n_dim > 1024 is not supported");
        const size_t smem = sizeof(float) * (size_t)(kTileCand + kTileWarps) * (d + 1);
        CNN_TRY(allow_dynamic_smem(ctx, (const void *)tile_search_kernel<false>, smem));
        CNN_TRY(allow_dynamic_smem(ctx, (const void *)tile_search_kernel<true>, smem));
        stage_begin(ctx, 2);
        const unsigned gq = grid_for(n, kTileWarps);
        tile_search_kernel<false><<<gq, kTileWarps * 32, smem, st>>>(ctx->x, ctx->scratch_b.as<float>(), d, n, sp, deg,
                                                                      nullptr, nullptr, counters);
        CNN_LAUNCH_CHECK(ctx);
        stage_end(ctx, 2);
        ctx->identity_perm = true;
    }

    // Rows left in their slots (a public build on the list search): the
    // offsets, the read-back of the pair count and the compaction wait until
    // something asks for the CSR (ensure_csr); the fit walks the slots.
    const bool slot_form = CNN_SLOT_ROWS && form == kFormPref && use_grid && use_slots && !use_mask && !calibrate &&
                           grid_items > 0 && ctx->host_stats != nullptr;
    if (slot_form) {
        ctx->graph_slots = true;
        ctx->csr_valid = false;
        ctx->slot_total = n_candidates;
        stage_begin(ctx, 4);
        CNN_TRY(ctx->ensure(ctx->split, sizeof(int32_t) * (size_t)n));
        CNN_TRY(ctx->ensure(ctx->grid_qend, sizeof(int64_t) * (size_t)n));
        row_split_kernel<<<std::min<unsigned>(grid_for(n, 256), ctx->sm_count * 16u), 256, 0, st>>>(
            n, ctx->grid_qslot.as<int64_t>(), deg, ctx->grid_slot_cols.as<int32_t>(), ctx->grid_qend.as<int64_t>(),
            ctx->split.as<int32_t>());
        CNN_LAUNCH_CHECK(ctx);
        stage_end(ctx, 4);
        ctx->split_valid = true;
        // the pair count, summed by the search, comes back with the statistics
        CNN_CUDA(ctx, cudaMemcpyAsync(ctx->host_stats, counters, 2 * sizeof(unsigned long long),
                                      cudaMemcpyDeviceToHost, st));
        CNN_CUDA(ctx, cudaMemcpyAsync(ctx->host_stats + 10, counters + kSlotPairsAt, 4 * sizeof(unsigned long long),
                                      cudaMemcpyDeviceToHost, st));
        ctx->pending_candidates = n_candidates;
        ctx->search_stats_pending = true;
        ctx->nnz_pending = true;
        ctx->nnz = -1;  // unknown until resolve_nnz
        ctx->identity_perm = false;
        ctx->have_graph = true;
        return CNN_OK;
    }

    // ---- offsets
    stage_begin(ctx, 3);
    if (!use_grid) {  // the grid path cleared deg[n] with deg
        set_last_zero_kernel<<<1, 1, 0, st>>>(deg, n);
        CNN_LAUNCH_CHECK(ctx);
    }
    CNN_TRY(scan_exclusive_i32_to_i64(ctx, deg, row_off, n + 1));
    int64_t nnz = 0;
    CNN_TRY(read_back(ctx, &nnz, row_off + n, sizeof(int64_t)));
    stage_end(ctx, 3);
    if (use_lists) CNN_TRY(ctx->ensure(ctx->cols, sizeof(int32_t) * (size_t)(nnz > 0 ? nnz : 1)));

    stage_begin(ctx, 4);
    if (use_mask) {
        // the masks are the graph; lists are made from them on request
        ctx->graph_mask = true;
        ctx->csr_valid = false;
        ctx->mask_geo = geo;
    }
    if (calibrate) CNN_CUDA(ctx, cudaEventRecord(ctx->tune_ev[3], st));
    if (use_grid && use_lists) {
        if (grid_items > 0 && use_slots) {
            CNN_TRY(ctx->ensure(ctx->split, sizeof(int32_t) * (size_t)n));
            compact_rows_kernel<<<std::min<unsigned>(grid_for(n * 32, 256), ctx->sm_count * 16u), 256, 0, st>>>(
                n, ctx->grid_qslot.as<int64_t>(), ctx->grid_slot_cols.as<int32_t>(), row_off,
                ctx->cols.as<int32_t>(), ctx->split.as<int32_t>());
            CNN_LAUNCH_CHECK(ctx);
            ctx->split_valid = true;
        } else if (grid_items > 0) {
            (geo.wrap ? grid_unit_kernel<kFill, true> : grid_unit_kernel<kFill, false>)<<<(unsigned)((grid_items + kUnitWarps - 1) / kUnitWarps), kUnitWarps * 32, 0, st>>>(
                ctx->io_c.as<int2>(), grid_items, ctx->x, d, geo, sp, ctx->perm.as<int32_t>(),
                ctx->cell_start.as<int64_t>(), ctx->xf4.as<float4>(), deg, row_off, ctx->cols.as<int32_t>(), counters,
                nullptr);
            CNN_LAUNCH_CHECK(ctx);
        }
        ctx->csr_valid = true;
    } else if (!use_grid) {
        const size_t smem = sizeof(float) * (size_t)(kTileCand + kTileWarps) * (d + 1);
        tile_search_kernel<true><<<grid_for(n, kTileWarps), kTileWarps * 32, smem, st>>>(
            ctx->x, ctx->scratch_b.as<float>(), d, n, sp, deg, row_off, ctx->cols.as<int32_t>(), counters);
        CNN_LAUNCH_CHECK(ctx);
    }
    stage_end(ctx, 4);
    if (calibrate) {
        // search times of the two forms (the list form includes its compaction)
        CNN_CUDA(ctx, cudaEventRecord(ctx->tune_ev[4], st));
        CNN_CUDA(ctx, cudaEventSynchronize(ctx->tune_ev[4]));
        float m01 = 0.f, m12 = 0.f, m34 = 0.f;
        CNN_CUDA(ctx, cudaEventElapsedTime(&m01, ctx->tune_ev[0], ctx->tune_ev[1]));
        CNN_CUDA(ctx, cudaEventElapsedTime(&m12, ctx->tune_ev[1], ctx->tune_ev[2]));
        CNN_CUDA(ctx, cudaEventElapsedTime(&m34, ctx->tune_ev[3], ctx->tune_ev[4]));
        ctx->tune_ms_mask = m01;
        ctx->tune_ms_lists = m12 + m34;
        ctx->tune_pending = true;
    }

    if (ctx->host_stats) {  // read by cnn_get_stats
        CNN_CUDA(ctx, cudaMemcpyAsync(ctx->host_stats, counters, 2 * sizeof(unsigned long long),
                                      cudaMemcpyDeviceToHost, st));
        ctx->pending_candidates = n_candidates;
        ctx->search_stats_pending = true;
    } else {
        unsigned long long hc[2] = {0, 0};
        CNN_CUDA(ctx, cudaMemcpyAsync(hc, counters, sizeof(hc), cudaMemcpyDeviceToHost, st));
        CNN_CUDA(ctx, cudaStreamSynchronize(st));
        ctx->stats.n_exact = (int64_t)hc[0];
        ctx->stats.n_candidates = n_candidates >= 0 ? n_candidates : (int64_t)hc[1];
    }
    ctx->stats.n_nonzero = nnz;
    ctx->nnz = nnz;
    ctx->have_graph = true;
    return CNN_OK;
}

// The pair count of a graph left in its slots, read back (a stream sync).
cnn_status resolve_nnz(cnn_context *ctx) {
    if (!ctx->nnz_pending) return CNN_OK;
    CNN_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    const unsigned long long *h = ctx->host_stats + 10;
    ctx->nnz = (int64_t)(h[0] + h[1] + h[2] + h[3]);
    ctx->stats.n_nonzero = ctx->nnz;
    ctx->nnz_pending = false;
    return CNN_OK;
}

// The CSR of a graph left in its slots: the offsets from the row lengths
// (deg[n] is 0 since the search), then the compaction with split points.
cnn_status ensure_csr(cnn_context *ctx) {
    if (!ctx->have_graph || !ctx->graph_slots || ctx->csr_valid) return CNN_OK;
    CNN_TRY(resolve_nnz(ctx));
    const int64_t n = ctx->n;
    cudaStream_t st = ctx->stream;
    int64_t *row_off = ctx->row_off.as<int64_t>();
    CNN_TRY(scan_exclusive_i32_to_i64(ctx, ctx->deg.as<int32_t>(), row_off, n + 1));
    CNN_TRY(ctx->ensure(ctx->cols, sizeof(int32_t) * (size_t)(ctx->nnz > 0 ? ctx->nnz : 1)));
    CNN_TRY(ctx->ensure(ctx->split, sizeof(int32_t) * (size_t)(n > 0 ? n : 1)));
    compact_rows_kernel<<<std::min<unsigned>(grid_for(n * 32, 256), ctx->sm_count * 16u), 256, 0, st>>>(
        n, ctx->grid_qslot.as<int64_t>(), ctx->grid_slot_cols.as<int32_t>(), row_off, ctx->cols.as<int32_t>(),
        ctx->split.as<int32_t>());
    CNN_LAUNCH_CHECK(ctx);
    ctx->csr_valid = true;
    ctx->split_valid = true;
    return CNN_OK;
}

cnn_status ensure_lists(cnn_context *ctx) {
    if (!ctx->have_graph || !ctx->graph_mask || ctx->csr_valid) return CNN_OK;
    CNN_TRY(ctx->ensure(ctx->cols, sizeof(int32_t) * (size_t)(ctx->nnz > 0 ? ctx->nnz : 1)));
    CNN_TRY(masks_to_lists(ctx));
    ctx->csr_valid = true;
    return CNN_OK;
}

// Graph as CSR in point-index order (device output buffers).
cnn_status export_neighbours_impl(cnn_context *ctx, int64_t *offsets_dev, int32_t *indices_dev) {
    CNN_TRY(ensure_lists(ctx));
    CNN_TRY(ensure_csr(ctx));
    const int64_t n = ctx->n, nnz = ctx->nnz;
    cudaStream_t st = ctx->stream;
    if (ctx->identity_perm) {
        CNN_CUDA(ctx, cudaMemcpyAsync(offsets_dev, ctx->row_off.ptr, sizeof(int64_t) * (size_t)(n + 1),
                                      cudaMemcpyDeviceToDevice, st));
        if (nnz > 0)
            CNN_CUDA(ctx, cudaMemcpyAsync(indices_dev, ctx->cols.ptr, sizeof(int32_t) * (size_t)nnz,
                                          cudaMemcpyDeviceToDevice, st));
        return CNN_OK;
    }
    CNN_TRY(ctx->ensure(ctx->scratch_a, sizeof(int64_t) * (size_t)(n + 1)));
    deg_by_point_kernel<<<std::min<unsigned>(grid_for(n + 1, 256), 4096u), 256, 0, st>>>(
        ctx->deg.as<int32_t>(), ctx->inv.as<int32_t>(), n, ctx->scratch_a.as<int64_t>());
    CNN_LAUNCH_CHECK(ctx);
    CNN_TRY(scan_exclusive_i64(ctx, ctx->scratch_a.as<int64_t>(), offsets_dev, n + 1));
    if (nnz == 0) return CNN_OK;
    const int bits_n = bits_for(n);
    CNN_TRY(ctx->ensure(ctx->scratch_b, sizeof(uint64_t) * (size_t)nnz));
    uint64_t *keys = ctx->scratch_b.as<uint64_t>();
    export_keys_kernel<<<grid_for(n * 32, 256), 256, 0, st>>>(ctx->row_off.as<int64_t>(), ctx->cols.as<int32_t>(),
                                                              ctx->perm.as<int32_t>(), n, bits_n, keys);
    CNN_LAUNCH_CHECK(ctx);
    uint64_t *sorted = keys;
    CNN_TRY(radix_sort_u64(ctx, keys, nnz, 2 * bits_n, 0, &sorted));
    keys_to_cols_kernel<<<std::min<unsigned>(grid_for(nnz, 256), ctx->sm_count * 32u), 256, 0, st>>>(sorted, nnz, bits_n,
                                                                                             indices_dev);
    CNN_LAUNCH_CHECK(ctx);
    return CNN_OK;
}

// Neighbour rows of m other points (float64, device) against the current
// points: offsets (m+1, int64) and ascending point indices.  Float32
// coordinates relative to the lowest finite coordinate of both sets; the
// float64 band decides the rest.
cnn_status cross_neighbours_impl(cnn_context *ctx, const double *xq, int64_t m, double radius_cutoff, int metric,
                                 int fpmode, cnn::DevBuf &off_buf, cnn::DevBuf &cols_buf, int64_t *nnz_out) {
    const int64_t n = ctx->n;
    const int d = ctx->d;
    cudaStream_t st = ctx->stream;
    CNN_TRY(ctx->ensure(off_buf, sizeof(int64_t) * (size_t)(m + 1)));
    int64_t *off = off_buf.as<int64_t>();
    *nnz_out = 0;
    if (m == 0) {
        CNN_CUDA(ctx, cudaMemsetAsync(off, 0, sizeof(int64_t), st));
        return CNN_OK;
    }
    SearchParams sp;
    sp.rc = radius_cutoff;
    sp.metric = metric;
    sp.fpmode = fpmode;
    sp.thr_in = -1.f;
    sp.thr_out = INFINITY;
    const bool radius_ok = radius_cutoff >= 0.0 && isfinite(radius_cutoff);
    std::vector<double> lo(d, INFINITY), hi(d, -INFINITY);
    for (int set = 0; set < 2; ++set) {
        const double *src = set == 0 ? ctx->x : xq;
        const int64_t cnt = set == 0 ? n : m;
        if (cnt == 0) continue;
        const int blocks = (int)std::min<int64_t>(256, (cnt + 255) / 256);
        CNN_TRY(ctx->ensure(ctx->scratch_a, sizeof(double) * (size_t)blocks * (size_t)d * 3 + 64));
        extent_partial_kernel<<<dim3(blocks, d), 256, 0, st>>>(src, cnt, d, ctx->scratch_a.as<double>());
        CNN_LAUNCH_CHECK(ctx);
        std::vector<double> part((size_t)blocks * d * 3);
        CNN_CUDA(ctx, cudaMemcpyAsync(part.data(), ctx->scratch_a.ptr, sizeof(double) * part.size(),
                                      cudaMemcpyDeviceToHost, st));
        CNN_CUDA(ctx, cudaStreamSynchronize(st));
        for (int b = 0; b < blocks; ++b)
            for (int k = 0; k < d; ++k) {
                lo[k] = std::min(lo[k], part[((size_t)b * d + k) * 3]);
                hi[k] = std::max(hi[k], part[((size_t)b * d + k) * 3 + 1]);
            }
    }
    std::vector<double> ext(d);
    for (int k = 0; k < d; ++k) {
        if (!(lo[k] <= hi[k])) lo[k] = hi[k] = 0.0;
        ext[k] = hi[k] - lo[k];
    }
    if (radius_ok) {
        const double R = metric == CNN_METRIC_EUCLIDEAN ? radius_cutoff : sqrt(radius_cutoff);
        const double rc2 = metric == CNN_METRIC_EUCLIDEAN ? radius_cutoff * radius_cutoff : radius_cutoff;
        double band = 0;
        if (!filter_thresholds(ext, R, rc2, &sp.thr_in, &sp.thr_out, &band)) {
            sp.thr_in = -1.f;
            sp.thr_out = INFINITY;  // every pair in float64
        }
    } else if (radius_cutoff != INFINITY) {
        sp.thr_in = -1.f;
        sp.thr_out = -1.f;  // a NaN or negative cutoff admits nothing
    }
    // this set's cell grid, when its graph was built on one for a radius at
    // least this large (the other points are binned into the same cells)
    const GridGeom &geo = ctx->grid_geo;
    const double R = metric == CNN_METRIC_EUCLIDEAN ? radius_cutoff : sqrt(radius_cutoff);
    if (ctx->have_graph && ctx->grid_geo_valid && !geo.wrap && d <= 3 && radius_ok && R > 0 &&
        (metric == CNN_METRIC_EUCLIDEAN_REDUCED || metric == CNN_METRIC_EUCLIDEAN) &&
        geo.h * geo.reach >= R * (1.0 + 1e-6) && n > 0) {
        // float32 values relative to the grid origin: the bound takes the
        // largest magnitude either set reaches
        std::vector<double> ext_g(d);
        for (int k = 0; k < d; ++k) ext_g[k] = std::max(std::fabs(hi[k] - geo.lo[k]), std::fabs(lo[k] - geo.lo[k]));
        const double rc2 = metric == CNN_METRIC_EUCLIDEAN ? radius_cutoff * radius_cutoff : radius_cutoff;
        double band = 0;
        if (!filter_thresholds(ext_g, R, rc2, &sp.thr_in, &sp.thr_out, &band)) {
            sp.thr_in = -1.f;
            sp.thr_out = INFINITY;  // every candidate pair in float64
        }
        const int64_t ncells = geo.ncells;
        CNN_TRY(ctx->ensure(ctx->cross_cell_of, sizeof(int32_t) * (size_t)m));
        CNN_TRY(ctx->ensure(ctx->cross_slot, sizeof(int32_t) * (size_t)m));
        CNN_TRY(ctx->ensure(ctx->cross_count, sizeof(int32_t) * (size_t)(ncells + 2)));
        CNN_TRY(ctx->ensure(ctx->cross_start, sizeof(int64_t) * (size_t)(ncells + 2)));
        CNN_TRY(ctx->ensure(ctx->cross_perm, sizeof(int32_t) * (size_t)m));
        CNN_TRY(ctx->ensure(ctx->cross_inv, sizeof(int32_t) * (size_t)m));
        CNN_TRY(ctx->ensure(ctx->cross_xf4, sizeof(float4) * (size_t)m));
        int32_t *qcount = ctx->cross_count.as<int32_t>();
        int64_t *qstart = ctx->cross_start.as<int64_t>();
        CNN_CUDA(ctx, cudaMemsetAsync(qcount, 0, sizeof(int32_t) * (size_t)(ncells + 2), st));
        const unsigned gb = std::min<unsigned>(grid_for(m, 256), ctx->sm_count * 16u);
        cell_assign_kernel<<<gb, 256, 0, st>>>(xq, m, d, geo, ctx->cross_cell_of.as<int32_t>(),
                                               ctx->cross_slot.as<int32_t>(), qcount);
        CNN_LAUNCH_CHECK(ctx);
        CNN_TRY(scan_exclusive_i32_to_i64(ctx, qcount, qstart, ncells + 2));
        place_kernel<<<gb, 256, 0, st>>>(ctx->cross_cell_of.as<int32_t>(), ctx->cross_slot.as<int32_t>(), qstart, m, xq,
                                         d, geo, ctx->cross_perm.as<int32_t>(), ctx->cross_inv.as<int32_t>(),
                                         ctx->cross_xf4.as<float4>());
        CNN_LAUNCH_CHECK(ctx);
        // units: (cell, up to kUnitQueries other points); the bucket of
        // non-finite points (cell ncells) has no neighbours
        CNN_TRY(ctx->ensure(ctx->cross_units_n, sizeof(int32_t) * (size_t)(ncells + 1)));
        CNN_TRY(ctx->ensure(ctx->cross_units_off, sizeof(int64_t) * (size_t)(ncells + 1)));
        const unsigned cg = std::min<unsigned>(grid_for(ncells, 256), ctx->sm_count * 16u);
        item_count_kernel<kUnitQueries><<<cg, 256, 0, st>>>(qstart, ncells, ctx->cross_units_n.as<int32_t>());
        CNN_LAUNCH_CHECK(ctx);
        CNN_CUDA(ctx, cudaMemsetAsync(ctx->cross_units_n.as<int32_t>() + ncells, 0, sizeof(int32_t), st));
        CNN_TRY(scan_exclusive_i32_to_i64(ctx, ctx->cross_units_n.as<int32_t>(), ctx->cross_units_off.as<int64_t>(),
                                          ncells + 1));
        int64_t nunits = 0;
        CNN_TRY(read_back(ctx, &nunits, ctx->cross_units_off.as<int64_t>() + ncells, sizeof(int64_t)));
        CNN_TRY(ctx->ensure(ctx->cross_units, sizeof(int2) * (size_t)(nunits > 0 ? nunits : 1)));
        if (nunits > 0) {
            item_fill_kernel<kUnitQueries><<<cg, 256, 0, st>>>(qstart, ncells, ctx->cross_units_off.as<int64_t>(),
                                                               ctx->cross_units.as<int2>());
            CNN_LAUNCH_CHECK(ctx);
        }
        // row lengths (in binned order), offsets, keys, sort, rows
        CNN_TRY(ctx->ensure(ctx->cross_deg, sizeof(int32_t) * (size_t)(m + 1)));
        CNN_TRY(ctx->ensure(ctx->cross_row_off, sizeof(int64_t) * (size_t)(m + 1)));
        int32_t *qdeg = ctx->cross_deg.as<int32_t>();
        CNN_CUDA(ctx, cudaMemsetAsync(qdeg, 0, sizeof(int32_t) * (size_t)(m + 1), st));
        unsigned long long *counters = ctx->counters.as<unsigned long long>();
        const int bits_n = bits_for(n);
        const unsigned ug = (unsigned)((nunits + kUnitWarps - 1) / kUnitWarps);
        if (nunits > 0) {
            cross_unit_kernel<false><<<ug, kUnitWarps * 32, 0, st>>>(
                ctx->cross_units.as<int2>(), nunits, xq, ctx->x, d, geo, sp, ctx->cross_perm.as<int32_t>(), qstart,
                ctx->cross_xf4.as<float4>(), ctx->perm.as<int32_t>(), ctx->cell_start.as<int64_t>(),
                ctx->xf4.as<float4>(), bits_n, qdeg, nullptr, nullptr, counters);
            CNN_LAUNCH_CHECK(ctx);
        }
        CNN_TRY(scan_exclusive_i32_to_i64(ctx, qdeg, ctx->cross_row_off.as<int64_t>(), m + 1));
        int64_t nnz = 0;
        CNN_TRY(read_back(ctx, &nnz, ctx->cross_row_off.as<int64_t>() + m, sizeof(int64_t)));
        // offsets in the other points' order
        CNN_TRY(ctx->ensure(ctx->scratch_a, sizeof(int64_t) * (size_t)(m + 1)));
        deg_by_point_kernel<<<std::min<unsigned>(grid_for(m + 1, 256), 4096u), 256, 0, st>>>(
            qdeg, ctx->cross_inv.as<int32_t>(), m, ctx->scratch_a.as<int64_t>());
        CNN_LAUNCH_CHECK(ctx);
        CNN_TRY(scan_exclusive_i64(ctx, ctx->scratch_a.as<int64_t>(), off, m + 1));
        CNN_TRY(ctx->ensure(cols_buf, sizeof(int32_t) * (size_t)(nnz > 0 ? nnz : 1)));
        if (nnz > 0) {
            CNN_TRY(ctx->ensure(ctx->cross_keys, sizeof(uint64_t) * (size_t)nnz));
            uint64_t *keys = ctx->cross_keys.as<uint64_t>();
            cross_unit_kernel<true><<<ug, kUnitWarps * 32, 0, st>>>(
                ctx->cross_units.as<int2>(), nunits, xq, ctx->x, d, geo, sp, ctx->cross_perm.as<int32_t>(), qstart,
                ctx->cross_xf4.as<float4>(), ctx->perm.as<int32_t>(), ctx->cell_start.as<int64_t>(),
                ctx->xf4.as<float4>(), bits_n, nullptr, ctx->cross_row_off.as<int64_t>(), keys, counters);
            CNN_LAUNCH_CHECK(ctx);
            uint64_t *sorted = keys;
            CNN_TRY(radix_sort_u64(ctx, keys, nnz, bits_n + bits_for(m), 0, &sorted));
            keys_to_cols_kernel<<<std::min<unsigned>(grid_for(nnz, 256), ctx->sm_count * 32u), 256, 0, st>>>(
                sorted, nnz, bits_n, cols_buf.as<int32_t>());
            CNN_LAUNCH_CHECK(ctx);
        }
        *nnz_out = nnz;
        return CNN_OK;
    }
    if (d > 1024) return ctx->fail(CNN_ERR_UNSUPPORTED, "n_dim > 1024 is not supported");
    CNN_TRY(ctx->ensure(ctx->scratch_a, sizeof(double) * (size_t)d + 64));
    CNN_TRY(ctx->ensure(ctx->scratch_b, sizeof(float) * (size_t)(n + m) * d + 64));
    CNN_CUDA(ctx, cudaMemcpyAsync(ctx->scratch_a.ptr, lo.data(), sizeof(double) * d, cudaMemcpyHostToDevice, st));
    float *xf = ctx->scratch_b.as<float>();
    float *xqf = xf + (size_t)n * d;
    if (n > 0) {
        to_f32_kernel<<<std::min<unsigned>(grid_for(n * d, 256), ctx->sm_count * 16u), 256, 0, st>>>(
            ctx->x, n, d, ctx->scratch_a.as<double>(), xf);
        CNN_LAUNCH_CHECK(ctx);
    }
    to_f32_kernel<<<std::min<unsigned>(grid_for(m * d, 256), ctx->sm_count * 16u), 256, 0, st>>>(
        xq, m, d, ctx->scratch_a.as<double>(), xqf);
    CNN_LAUNCH_CHECK(ctx);
    const size_t smem = sizeof(float) * (size_t)(kTileCand + kTileWarps) * (d + 1);
    CNN_TRY(allow_dynamic_smem(ctx, (const void *)cross_tile_kernel<false>, smem));
    CNN_TRY(allow_dynamic_smem(ctx, (const void *)cross_tile_kernel<true>, smem));
    CNN_TRY(ctx->ensure(ctx->io_a, sizeof(int32_t) * (size_t)(m + 1)));
    int32_t *deg = ctx->io_a.as<int32_t>();
    const unsigned gq = grid_for(m, kTileWarps);
    cross_tile_kernel<false><<<gq, kTileWarps * 32, smem, st>>>(xq, xqf, m, ctx->x, xf, n, d, sp, deg, nullptr,
                                                                 nullptr);
    CNN_LAUNCH_CHECK(ctx);
    CNN_CUDA(ctx, cudaMemsetAsync(deg + m, 0, sizeof(int32_t), st));
    CNN_TRY(scan_exclusive_i32_to_i64(ctx, deg, off, m + 1));
    int64_t nnz = 0;
    CNN_CUDA(ctx, cudaMemcpyAsync(&nnz, off + m, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    CNN_CUDA(ctx, cudaStreamSynchronize(st));
    CNN_TRY(ctx->ensure(cols_buf, sizeof(int32_t) * (size_t)(nnz > 0 ? nnz : 1)));
    cross_tile_kernel<true><<<gq, kTileWarps * 32, smem, st>>>(xq, xqf, m, ctx->x, xf, n, d, sp, nullptr, off,
                                                                cols_buf.as<int32_t>());
    CNN_LAUNCH_CHECK(ctx);
    *nnz_out = nnz;
    return CNN_OK;
}

// Precomputed neighbourhoods: rows sorted on the device, identity order.
cnn_status set_neighbours_impl(cnn_context *ctx, const int64_t *offsets_dev, const int32_t *indices_dev,
                               int64_t n) {
    cudaStream_t st = ctx->stream;
    ctx->have_graph = false;
    ctx->graph_mask = false;
    ctx->csr_valid = true;
    ctx->graph_slots = false;
    ctx->nnz_pending = false;
    ctx->tune_pending = false;
    ctx->split_valid = false;
    ++ctx->graph_generation;
    ctx->stats = cnn_stats{};
    stages_reset(ctx, 0, cnn_context::kSlots - 1);
    ctx->search_stats_pending = false;
    ctx->fit_stats_pending = false;
    ctx->stats.n_points = n;
    ctx->n = n;
    ctx->d = 0;
    ctx->x = nullptr;
    ctx->dist = nullptr;
    ctx->dist_set = false;
    CNN_TRY(ctx->ensure(ctx->counters, kCounterSlots * sizeof(unsigned long long)));
    CNN_CUDA(ctx, cudaMemsetAsync(ctx->counters.ptr, 0, kCounterSlots * sizeof(unsigned long long), st));
    CNN_TRY(ctx->ensure(ctx->deg, sizeof(int32_t) * (size_t)(n + 1)));
    CNN_TRY(ctx->ensure(ctx->row_off, sizeof(int64_t) * (size_t)(n + 1)));
    CNN_TRY(ctx->ensure(ctx->perm, sizeof(int32_t) * (size_t)(n > 0 ? n : 1)));
    CNN_TRY(ctx->ensure(ctx->inv, sizeof(int32_t) * (size_t)(n > 0 ? n : 1)));
    int64_t first = 0, nnz = 0;
    CNN_CUDA(ctx, cudaMemcpyAsync(&first, offsets_dev, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    CNN_CUDA(ctx, cudaMemcpyAsync(&nnz, offsets_dev + n, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    CNN_CUDA(ctx, cudaStreamSynchronize(st));
    if (first != 0 || nnz < 0) return ctx->fail(CNN_ERR_INVALID_ARG, "offsets must start at 0 and not decrease");
    unsigned long long *counters = ctx->counters.as<unsigned long long>();
    check_offsets_kernel<<<std::min<unsigned>(grid_for(n, 256), 4096u), 256, 0, st>>>(offsets_dev, n, counters + 2);
    CNN_LAUNCH_CHECK(ctx);
    unsigned long long bad = 0;
    CNN_CUDA(ctx, cudaMemcpyAsync(&bad, counters + 2, sizeof(bad), cudaMemcpyDeviceToHost, st));
    CNN_CUDA(ctx, cudaStreamSynchronize(st));
    if (bad) return ctx->fail(CNN_ERR_INVALID_ARG, "offsets must not decrease");
    CNN_TRY(iota_i32(ctx, ctx->perm.as<int32_t>(), n));
    CNN_TRY(iota_i32(ctx, ctx->inv.as<int32_t>(), n));
    CNN_CUDA(ctx, cudaMemcpyAsync(ctx->row_off.ptr, offsets_dev, sizeof(int64_t) * (size_t)(n + 1),
                                  cudaMemcpyDeviceToDevice, st));
    CNN_TRY(ctx->ensure(ctx->cols, sizeof(int32_t) * (size_t)(nnz > 0 ? nnz : 1)));
    if (n > 0) {
        const int bits_n = bits_for(n);
        CNN_TRY(ctx->ensure(ctx->scratch_b, sizeof(uint64_t) * (size_t)(nnz > 0 ? nnz : 1)));
        uint64_t *keys = ctx->scratch_b.as<uint64_t>();
        import_keys_kernel<<<grid_for(n * 32, 256), 256, 0, st>>>(offsets_dev, indices_dev, n, bits_n, keys,
                                                                  ctx->deg.as<int32_t>(), counters + 3);
        CNN_LAUNCH_CHECK(ctx);
        CNN_CUDA(ctx, cudaMemcpyAsync(&bad, counters + 3, sizeof(bad), cudaMemcpyDeviceToHost, st));
        CNN_CUDA(ctx, cudaStreamSynchronize(st));
        if (bad) return ctx->fail(CNN_ERR_INVALID_ARG, "neighbour index out of range");
        if (nnz > 0) {
            uint64_t *sorted = keys;
            CNN_TRY(radix_sort_u64(ctx, keys, nnz, 2 * bits_n, 0, &sorted));
            keys_to_cols_kernel<<<std::min<unsigned>(grid_for(nnz, 256), ctx->sm_count * 32u), 256, 0, st>>>(
                sorted, nnz, bits_n, ctx->cols.as<int32_t>());
            CNN_LAUNCH_CHECK(ctx);
        }
    }
    ctx->nnz = nnz;
    ctx->identity_perm = true;
    ctx->have_graph = true;
    ctx->stats.n_nonzero = nnz;
    ctx->stats.search_kind = 0;
    return CNN_OK;
}

}  // namespace cnn
