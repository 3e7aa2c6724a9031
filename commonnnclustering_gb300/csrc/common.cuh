// common.cuh -- shared device helpers and the context definition.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <string>
#include <vector>

#include "cnngpu.h"

namespace cnn {

constexpr int kWarp = 32;

// ---------------------------------------------------------------------------
// Status plumbing: every CUDA call goes through CNN_CUDA, which records the
// message on the context and returns CNN_ERR_CUDA (or CNN_ERR_OOM).
// ---------------------------------------------------------------------------
struct Error {
    cnn_status status;
    std::string msg;
};

#define CNN_CUDA(ctx, expr)                                                             \
    do {                                                                                \
        cudaError_t e_ = (expr);                                                        \
        if (e_ != cudaSuccess) {                                                        \
            (void)cudaGetLastError();                                                   \
            return (ctx)->fail(e_ == cudaErrorMemoryAllocation ? CNN_ERR_OOM : CNN_ERR_CUDA, \
                               std::string(#expr) + ": " + cudaGetErrorString(e_));     \
        }                                                                               \
    } while (0)

#define CNN_TRY(expr)                       \
    do {                                    \
        cnn_status s_ = (expr);             \
        if (s_ != CNN_OK) return s_;        \
    } while (0)

// Called after every kernel launch: checks the launch and counts it.
#define CNN_LAUNCH_CHECK(ctx)             \
    do {                                  \
        ++(ctx)->n_launches;              \
        CNN_CUDA(ctx, cudaGetLastError()); \
    } while (0)

// A grow-only device buffer.  Memory is returned only when the context is
// destroyed, so repeated fits of the same size allocate nothing.
struct DevBuf {
    void *ptr = nullptr;
    size_t cap = 0;
    template <typename T> T *as() const { return static_cast<T *>(ptr); }
};

// Cell grid of the d <= 3 search: cubic cells of edge h >= R, internal
// order = points grouped by cell id (x fastest).
struct GridGeom {
    double lo[3];
    double h;
    double inv_h;      // 1 / h, rounded: cell coordinates are a monotone function of x
    int32_t g[3];      // cells per dimension (1 for unused dimensions)
    int64_t ncells;    // g0*g1*g2; bucket ncells holds non-finite points
    int32_t reach;     // neighbours lie at most `reach` cells apart (h >= R / reach)
    // periodic metric: bit k of `wrap` = dimension k wraps around its box
    // length L[k]; its coordinates are binned as x - L floor(x / L) into
    // g[k] >= 3 cells of edge L / g[k] >= h, neighbouring cyclically
    int32_t wrap;
    double L[3];
    double inv_hk[3];  // cell coordinate = floor(v * inv_hk[k]) (v = x - lo, or the wrapped x)
};

// The cell-grid neighbour graph as bit masks (fit_mask.cu): a point of cell
// c owns ceil(T_c / 32) words, one bit per candidate of the cell's candidate
// sequence (the 9 runs of its 3 x 3 x 3 stencil, ascending), set for a
// neighbour.  Kernel argument.
struct MaskGraph {
    const int64_t *cell_start;  // [ncells + 2] first internal index of each cell
    const int32_t *pcell;       // [n] internal index -> cell
    const int64_t *mbase;       // [ncells + 1] word offset of each cell's first row
    const uint32_t *masks;      // the rows (+ one padding word at the end)
    int32_t g0, g1, g2;         // cells per dimension
};

// Stage timer: CUDA events on the context stream.
struct StageTimer {
    cudaEvent_t a = nullptr, b = nullptr;
};

}  // namespace cnn

// The context behind the opaque cnn_context handle.
struct cnn_context {
    int device = 0;
    unsigned sm_count = 1;  // multiprocessors of `device` (cudaDevAttrMultiProcessorCount), sizes persistent grids
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    bool timing = false;
    int poison = -1;  // >= 0: fill every new workspace allocation with this byte (CNN_DEBUG_POISON)
    int64_t wait_limit_ns = 0;  // > 0: limit of the bounded waits in the kernels (cnn_set_wait_limit)
    int search_pref = CNN_SEARCH_AUTO;  // cnn_set_search
    int grid_reach = 1;  // cell edge R / grid_reach (CNN_GRID_REACH=1|2 at creation)
    // CUDA-graph capture of the sweep's fits (sweep.cu).  While capturing,
    // a buffer that has to grow gets new memory and the old block is kept
    // (captured work refers to it) until the graph has run.
    bool sweep_graphs = true;  // CNN_SWEEP_GRAPH=0 at creation: plain launches
    bool capturing = false;
    std::vector<void *> deferred_free;
    // the last sweep's instantiated graph: a sweep of the same shape updates
    // its parameters (cudaGraphExecUpdate) instead of instantiating anew
    cudaGraphExec_t sweep_exec = nullptr;
    // device bytes the workspace holds, and an optional limit on them (a
    // served job's reservation): a growth past mem_cap fails with
    // CNN_ERR_OOM before cudaMalloc and sets cap_hit
    std::atomic<int64_t> mem_held{0};  // read by a server's dispatcher while the slot runs
    int64_t mem_cap = 0;                // 0: no limit
    bool cap_hit = false;
    int64_t cap_need = 0;               // the holding the refused growth asked for
    int64_t n_launches = 0;
    std::string last_error;
    cnn_stats stats{};
    // Counters of the last search and fit, copied back without a sync into
    // pinned memory and read by cnn_get_stats (which syncs the stream).
    unsigned long long *host_stats = nullptr;  // [0] exact, [1] candidates, [4..6] fit, [8] clusters, [10..13] pairs
    // pinned bounce buffer for the small read-backs the host waits on
    static constexpr size_t kHostSmall = 64 << 10;
    void *host_small = nullptr;
    bool search_stats_pending = false;
    bool fit_stats_pending = false;
    int64_t pending_candidates = -1;  // >= 0: known on the host
    const int64_t *counted_labels = nullptr;  // labels whose counts the last fit left in flag
    bool graph_slots = false;  // the list search's rows left in their slots (grid_qslot, grid_qend, deg, grid_slot_cols)
    bool nnz_pending = false;  // nnz of such a graph not read back yet (host_stats[10..13])
    int64_t slot_total = 0;    // their slots' total size, a bound of nnz

    // points (original order, row-major float64)
    int64_t n = 0;
    int32_t d = 0;
    const double *x = nullptr;  // device pointer (borrowed or owned copy)
    cnn::DevBuf x_own;
    cnn::DevBuf x_f32_stage;    // float32 input staged before widening

    // precomputed distances instead of points (cnn_set_distances)
    const double *dist = nullptr;  // device pointer (borrowed or owned copy)
    int dist_layout = 0;           // cnn_dist_layout
    bool dist_set = false;
    cnn::DevBuf dist_own;
    // box lengths of the periodic metric (cnn_set_periodic_bounds), host copy
    // and device copies (float64 then float32, per dimension)
    std::vector<double> periodic_bounds;
    cnn::DevBuf bounds_dev;

    // neighbour graph in internal (permuted) index space; graph_generation
    // changes with every replaced input or rebuilt graph (cnn_graph_generation)
    bool have_graph = false;
    int64_t graph_generation = 0;
    bool identity_perm = true;
    int64_t nnz = 0;
    cnn::DevBuf perm;     // int32[n]: internal -> point index
    cnn::DevBuf inv;      // int32[n]: point index -> internal
    cnn::DevBuf deg;      // int32[n]
    cnn::DevBuf row_off;  // int64[n+1]
    cnn::DevBuf cols;     // int32[nnz], ascending internal indices per row
    cnn::DevBuf split;    // int32[n]: entries <= p of row p (valid when split_valid)
    bool split_valid = false;
    cnn::DevBuf xf4;      // float4[n] permuted float32 coordinates (grid search)
    cnn::DevBuf cell_of;  // int32[n] cell id per point (original order)
    cnn::DevBuf cell_start;  // int32[ncells+2]
    // one-pass grid search: per-cell slot offsets, the rows in their slots,
    // each row's slot start
    cnn::DevBuf grid_slot_base, grid_slot_cols, grid_qslot, grid_qend;

    // extents (max - min of finite points) per dimension of the last grid search
    double grid_extent[3] = {0.0, 0.0, 0.0};

    // the graph in mask form (cell-grid searches of cnn_build_neighbours):
    // graph_mask = the masks hold the graph; csr_valid = row_off/cols hold it
    // too (built from the masks when a caller needs the lists)
    bool graph_mask = false;
    bool csr_valid = true;
    cnn::GridGeom mask_geo{};
    cnn::DevBuf pcell, mbase, masks;
    // intersection strategy of cnn_build_neighbours + cnn_fit
    // (cnn_set_intersection); under AUTO the tuner (tuner.cu) picks per
    // workload profile, timing both forms on the first fit of a new profile
    int intersect_pref = CNN_INTERSECT_AUTO;
    bool tune_pending = false;          // the graph is in both forms: the next fit times both
    uint64_t tune_key = 0;
    float tune_ms_mask = 0.f, tune_ms_lists = 0.f;  // search times of the two forms
    cudaEvent_t tune_ev[5] = {};
    cnn::DevBuf tune_consider, tune_labels;

    // batched (radius, cut) sweep: the largest-radius graph kept aside,
    // per-pair radius buckets, consider flags of the per-fit runs
    cnn::DevBuf sweep_bucket, sweep_row_off_max, sweep_cols_max, sweep_deg_max, sweep_consider, sweep_forest;
    cnn::DevBuf sweep_multi_deg, sweep_multi_off, sweep_multi_cols, sweep_multi_base;  // every smaller radius's graph
    cnn::DevBuf sweep_open_a, sweep_open_b, sweep_open_count;  // open pairs of the last fit, two lists

    // tensor-core (Gram) search for n_dim >= 16
    cnn::DevBuf gram_hi, gram_mid, gram_lo, gram_aux, gram_amb, gram_blocks, gram_tiles, gram_perm;
    cnn::DevBuf gram_masks, gram_tkeys, gram_low, gram_pad2c;  // tile hit masks, tile order, lower tiles, row map
    cnn::DevBuf gram_rowwork, gram_chunkcnt;                   // the row builder's work items and chunk counts

    // prediction: this set's graph in point order, the other points' rows
    cnn::DevBuf pred_off, pred_cols, pred_xoff, pred_xcols, pred_x, pred_set;
    // the cell grid of the last grid search (valid with the graph it built)
    // and the other points binned into it (cross rows on the grid)
    cnn::GridGeom grid_geo{};
    bool grid_geo_valid = false;
    cnn::DevBuf cross_cell_of, cross_slot, cross_count, cross_start, cross_perm, cross_inv, cross_xf4;
    cnn::DevBuf cross_units_n, cross_units_off, cross_units, cross_deg, cross_row_off, cross_keys;

    // fit work arrays
    cnn::DevBuf node;     // uint8[n]
    cnn::DevBuf parent;   // int32[n]
    cnn::DevBuf comp_min; // int32[n]
    cnn::DevBuf flag;     // int32[n+1]
    cnn::DevBuf counters; // unsigned long long[16]

    // staging for host<->device transfers and general scratch
    cnn::DevBuf stage_labels, stage_consider, stage_offsets, stage_indices, stage_misc;
    cnn::DevBuf io_a, io_b, io_c;
    cnn::DevBuf scratch_a, scratch_b, scratch_c, scratch_d, scan_tmp;

    // stage timing: events recorded on the stream, read in cnn_get_stats
    static constexpr int kSlots = 12;
    cudaEvent_t ev_begin[kSlots] = {};
    cudaEvent_t ev_end[kSlots] = {};
    bool slot_pending[kSlots] = {};

    cnn_status fail(cnn_status s, const std::string &msg) {
        last_error = msg;
        return s;
    }
    cnn_status ensure(cnn::DevBuf &b, size_t bytes) {
        if (bytes <= b.cap) return CNN_OK;
        size_t want = bytes < 256 ? 256 : bytes;
        want = (want + 255) & ~size_t(255);
        const int64_t after = mem_held.load() - (int64_t)b.cap + (int64_t)want;
        if (mem_cap > 0 && after > mem_cap) {
            cap_hit = true;
            cap_need = after;
            return fail(CNN_ERR_OOM, "workspace limit: " + std::to_string(after) + " bytes needed, " +
                                         std::to_string(mem_cap) + " allowed");
        }
        if (b.ptr) {
            mem_held -= (int64_t)b.cap;
            if (capturing) {
                deferred_free.push_back(b.ptr);  // freed after the captured graph has run
            } else {
                cudaError_t e = cudaStreamSynchronize(stream);
                if (e != cudaSuccess) return fail(CNN_ERR_CUDA, cudaGetErrorString(e));
                cudaFree(b.ptr);
            }
            b.ptr = nullptr;
            b.cap = 0;
        }
        cudaError_t e = cudaMalloc(&b.ptr, want);
        if (e != cudaSuccess) {
            (void)cudaGetLastError();
            b.ptr = nullptr;
            return fail(e == cudaErrorMemoryAllocation ? CNN_ERR_OOM : CNN_ERR_CUDA,
                        std::string("cudaMalloc(") + std::to_string(want) + "): " + cudaGetErrorString(e));
        }
        b.cap = want;
        mem_held += (int64_t)want;
        if (poison >= 0) {
            // debugging aid: stale workspace contents must never change a result
            e = cudaMemsetAsync(b.ptr, poison, want, stream);
            if (e != cudaSuccess) return fail(CNN_ERR_CUDA, cudaGetErrorString(e));
        }
        return CNN_OK;
    }
};

namespace cnn {

// ---- launchers implemented in the .cu files --------------------------------

// prims.cu
cnn_status scan_exclusive_i64(cnn_context *ctx, const int64_t *in, int64_t *out, int64_t n);
cnn_status scan_exclusive_i32_to_i64(cnn_context *ctx, const int32_t *in, int64_t *out, int64_t n);
// sorted: if given, receives the buffer holding the result (keys or scratch_c,
// valid until scratch_c is next used) and the final copy back is skipped;
// n_dev: the key count read on the device (at most n; grids sized for n)
cnn_status radix_sort_u64(cnn_context *ctx, uint64_t *keys, int64_t n, int bits, int first_bit = 0,
                          uint64_t **sorted = nullptr, const int64_t *n_dev = nullptr);
// Copies `bytes` from the device to `host` and waits (through the pinned
// bounce buffer when it fits, else a plain copy).
cnn_status read_back(cnn_context *ctx, void *host, const void *dev, size_t bytes);
// raises a kernel's dynamic shared-memory limit to at least `bytes` (never lowers it)
cnn_status allow_dynamic_smem(cnn_context *ctx, const void *kernel, size_t bytes);
cnn_status fill_i32(cnn_context *ctx, int32_t *p, int64_t n, int32_t v);
cnn_status iota_i32(cnn_context *ctx, int32_t *p, int64_t n);

// cnngpu.cu
// cnn_fit on device arrays (with the intersection tuner); the cluster count
// stays in scratch_a[n]
cnn_status fit_dispatch(cnn_context *ctx, int64_t similarity_cutoff, int64_t n_member_cutoff, int64_t current_start,
                        uint8_t *cons_dev, int64_t *lab_dev);
// Frees every workspace buffer of the context (after its stream is idle):
// the graph and the points are gone, mem_held is 0.
cnn_status release_workspace(cnn_context *ctx);

// search.cu
// form of a cell-grid graph: kFormLists (callers that walk the lists
// themselves), kFormPref (cnn_build_neighbours: the context's intersection
// strategy, tuned under AUTO), kFormMasks (the mask form, fit_mask.cu)
constexpr int kFormLists = 0, kFormPref = 1, kFormMasks = 2;
cnn_status build_neighbours_impl(cnn_context *ctx, double radius_cutoff, int metric, int fpmode,
                                 int form = kFormLists);
// row_off/cols of the current graph (materialised from the masks if needed)
cnn_status ensure_lists(cnn_context *ctx);
cnn_status ensure_csr(cnn_context *ctx);   // the CSR of a graph left in its slots
cnn_status resolve_nnz(cnn_context *ctx);  // its pair count (a stream sync)
cnn_status export_neighbours_impl(cnn_context *ctx, int64_t *offsets_dev, int32_t *indices_dev);
cnn_status set_neighbours_impl(cnn_context *ctx, const int64_t *offsets_dev,
                               const int32_t *indices_dev, int64_t n);

// rows of m other points (device float64 [m][d]) against the current points
cnn_status cross_neighbours_impl(cnn_context *ctx, const double *xq, int64_t m, double radius_cutoff, int metric,
                                 int fpmode, cnn::DevBuf &off_buf, cnn::DevBuf &cols_buf, int64_t *nnz_out);

// predict.cu: first-match labels for other points
cnn_status predict_impl(cnn_context *ctx, const double *xq, int64_t m, const int64_t *labels_dev,
                        const int64_t *clusters_sorted_dev, int64_t n_clusters, double radius_cutoff, int metric,
                        int fpmode, int64_t similarity_cutoff, int64_t n_member_cutoff, int64_t *other_labels_dev,
                        uint8_t *other_consider_dev);

// mst.cu: maximum spanning forest of the common-neighbour graph (Prim's
// order); edges in the order the reference's tree queue pops them
cnn_status mst_prim_impl(cnn_context *ctx, double radius_cutoff, int metric, int fpmode, std::vector<int64_t> *ea,
                         std::vector<int64_t> *eb, std::vector<int64_t> *ew);

// gram.cu: tensor-core search (n_dim >= 16); *used = false when it declined
cnn_status gram_search_impl(cnn_context *ctx, double radius_cutoff, int metric, int fpmode, bool *used);

// tuner.cu: per-process choice of the intersection strategy by workload
// profile (grid search: point count and candidates per point, device)
uint64_t tuner_key(const cnn_context *ctx, int64_t n, int64_t candidates);
bool tuner_lookup(uint64_t key, int *choice);
void tuner_store(uint64_t key, int choice);

// fit_mask.cu: cnn_fit over the mask form
cnn_status fit_mask_impl(cnn_context *ctx, int64_t similarity_cutoff, int64_t n_member_cutoff,
                         int64_t current_start, uint8_t *consider_dev, int64_t *labels_dev);
// lists from the masks: cols[row_off[p] ..] = the set bits of p's row, ascending
cnn_status masks_to_lists(cnn_context *ctx);
// full common-neighbour counts of the pairs (p, q > p) of the point-order
// lists off/cols, taken from the masks of the current graph
cnn_status mask_pair_weights(cnn_context *ctx, const int64_t *off, const int32_t *cols, int32_t *weight);

// fit.cu
// seed_a / seed_b (optional, internal order): per point a node of a finished
// fit on the same graph order whose components refine this fit's (-1: none)
cnn_status fit_impl(cnn_context *ctx, int64_t similarity_cutoff, int64_t n_member_cutoff,
                    int64_t current_start, uint8_t *consider_dev, int64_t *labels_dev,
                    const int32_t *seed_a = nullptr, const int32_t *seed_b = nullptr,
                    const int2 *edge_list = nullptr, const unsigned long long *edge_count = nullptr,
                    int2 *wl_buf = nullptr, int64_t wl_buf_cap = 0);
// edge_list (device, count on the device): the pairs (a, b > a) that can
// still cross -- those a finished fit refining this one left open.
// wl_buf (optional): the cross-pair worklist with room for wl_buf_cap pairs
// (at least the pairs a pass can emit: no overflow pass)
cnn_status open_pairs_impl(cnn_context *ctx, const int2 *in_list, const unsigned long long *in_count, int2 *out,
                           unsigned long long *out_count, int64_t cap);
// sort_by_size of the labels a fit from fresh labels just wrote (no host
// round trip; fit.cu)
// device_count: read the cluster count on the device only (graph capture);
// otherwise one read-back picks the path and sizes its launches
cnn_status sort_fresh_impl(cnn_context *ctx, int64_t *labels, int64_t n, int64_t member_cutoff,
                           int64_t max_clusters, bool device_count);
cnn_status sort_by_size_impl(cnn_context *ctx, int64_t *labels_dev, int64_t n,
                             int64_t member_cutoff, int64_t max_clusters);
cnn_status check_lists_impl(cnn_context *ctx, const int32_t *a, int64_t na, const int32_t *b,
                            int64_t nb, int64_t c, int32_t *result_dev);
// a fresh fit (labels 0, consider 1, current_start 1) and sort_by_size into labels_dev
cnn_status fit_and_sort_into(cnn_context *ctx, int64_t similarity_cutoff, int64_t n_member_cutoff,
                             int64_t sort_member_cutoff, int64_t max_clusters, int64_t *labels_dev,
                             const int32_t *seed_a = nullptr, const int32_t *seed_b = nullptr, bool sort = true,
                             const int2 *edge_list = nullptr, const unsigned long long *edge_count = nullptr,
                             int2 *wl_buf = nullptr, int64_t wl_buf_cap = 0);

// sweep.cu
cnn_status sweep_impl(cnn_context *ctx, const double *radius_cutoffs, int32_t n_radii,
                      const int64_t *similarity_cutoffs, const int64_t *n_member_cutoffs, int32_t n_cuts,
                      int metric, int fpmode, int64_t sort_member_cutoff, int64_t max_clusters,
                      int64_t *labels_dev, const int32_t *out_slot = nullptr, bool sort = true);
// out_slot (host, [n_radii][n_cuts]): output index of each pair in labels_dev, -1 = not wanted

// timing helpers (cnngpu.cu): events only, no synchronisation
void stage_begin(cnn_context *ctx, int slot);
void stage_end(cnn_context *ctx, int slot);
void stages_reset(cnn_context *ctx, int first, int last);  // slots first..last: not run yet

inline unsigned grid_for(int64_t n, int block) {
    int64_t g = (n + block - 1) / block;
    if (g < 1) g = 1;
    if (g > 0x7fffffff) g = 0x7fffffff;
    return (unsigned)g;
}

}  // namespace cnn
