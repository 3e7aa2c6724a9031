// predict.cu -- cluster labels for other points (first match).
//
// Reference: PredictorFirstmatch.predict (src/cnnclustering/_fit.pyx:
// 1235-1291).  For every other point p with consider[p] == 1: its
// neighbours N_o(p) among the clustered points (NeighboursGetter.get_other,
// _types.pyx:1712-1731, ascending index, p itself not counted); if
// |N_o(p)| > n_member_cutoff, the members i are visited in index order and
// the first one whose label is in the consider set, whose own neighbourhood
// N(i) (self included) has more than n_member_cutoff members, and for which
// |N_o(p) & N(i)| reaches similarity_cutoff (0: always, < 0: never) gives
// p its label and sets consider[p] = 0.
//
// GB300 form: this set's graph is built (and kept) in point order, the
// rows of the other points come from the float32/float64 cross search, and
// one warp per other point screens 32 members at a time (label and degree
// tests by lane) before checking the survivors in index order with the
// merge-path intersection of the fit.
#include <algorithm>
#include <vector>

#include "common.cuh"
#include "fit_kernels.cuh"

namespace cnn {

namespace {

__device__ __forceinline__ bool label_in_set(int64_t label, const int64_t *__restrict__ set, int64_t nset) {
    int64_t lo = 0, hi = nset;
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (set[mid] < label) lo = mid + 1;
        else hi = mid;
    }
    return lo < nset && set[lo] == label;
}

__global__ void __launch_bounds__(256) predict_kernel(int64_t m, const int64_t *__restrict__ xoff,
                                                      const int32_t *__restrict__ xcols,
                                                      const int64_t *__restrict__ off,
                                                      const int32_t *__restrict__ cols,
                                                      const int64_t *__restrict__ labels,
                                                      const int64_t *__restrict__ set, int64_t nset, int64_t sim,
                                                      int64_t nmem, int64_t *__restrict__ olabels,
                                                      uint8_t *__restrict__ oconsider) {
    __shared__ int32_t s_wide[8][kWideChunk];  // 256 threads: a slot per warp for the wide merge
    int32_t *sA = s_wide[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    const int64_t warp0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int32_t needed = sim > INT32_MAX ? INT32_MAX : (int32_t)sim;
    for (int64_t p = warp0; p < m; p += nwarps) {
        if (oconsider[p] == 0) continue;
        const int64_t s = xoff[p], e = xoff[p + 1];
        const int64_t la = e - s;
        if (!(la > nmem)) continue;
        const int32_t *A = xcols + s;
        bool found = false;
        for (int64_t k0 = s; k0 < e && !found; k0 += 32) {
            const int64_t k = k0 + lane;
            int32_t i = -1;
            int64_t lab = 0;
            bool cand = false;
            if (k < e) {
                i = xcols[k];
                lab = labels[i];
                cand = label_in_set(lab, set, nset) && (off[i + 1] - off[i]) > nmem;
            }
            unsigned mask = __ballot_sync(0xffffffffu, cand);
            while (mask) {
                const int src = __ffs(mask) - 1;
                mask &= mask - 1;
                const int32_t ii = __shfl_sync(0xffffffffu, i, src);
                bool ok;
                if (sim <= 0) {
                    ok = sim == 0;
                } else {
                    const int64_t bs = off[ii];
                    ok = warp_shares(A, (int32_t)la, cols + bs, (int32_t)(off[ii + 1] - bs), needed, lane, sA);
                }
                if (ok) {
                    const int64_t l = __shfl_sync(0xffffffffu, lab, src);
                    if (lane == 0) {
                        olabels[p] = l;
                        oconsider[p] = 0;
                    }
                    found = true;
                    break;
                }
            }
        }
    }
}

}  // namespace

cnn_status predict_impl(cnn_context *ctx, const double *xq, int64_t m, const int64_t *labels_dev,
                        const int64_t *clusters_sorted_dev, int64_t n_clusters, double radius_cutoff, int metric,
                        int fpmode, int64_t similarity_cutoff, int64_t n_member_cutoff, int64_t *other_labels_dev,
                        uint8_t *other_consider_dev) {
    cudaStream_t st = ctx->stream;
    const int64_t n = ctx->n;
    if (m == 0) return CNN_OK;
    if (n > INT32_MAX - 2 || m > INT32_MAX - 2) return ctx->fail(CNN_ERR_UNSUPPORTED, "more than 2^31-3 points");
    // this set's neighbourhoods at the same radius, in point order
    CNN_TRY(build_neighbours_impl(ctx, radius_cutoff, metric, fpmode));
    CNN_TRY(ctx->ensure(ctx->pred_off, sizeof(int64_t) * (size_t)(n + 1)));
    CNN_TRY(ctx->ensure(ctx->pred_cols, sizeof(int32_t) * (size_t)(ctx->nnz > 0 ? ctx->nnz : 1)));
    CNN_TRY(export_neighbours_impl(ctx, ctx->pred_off.as<int64_t>(), ctx->pred_cols.as<int32_t>()));
    // the other points' rows against this set
    int64_t xnnz = 0;
    // the reference's periodic metric measures other points without the
    // minimum image (MetricExtEuclideanPeriodicReduced._calc_distance_other,
    // _types.pyx:2327-2345, sums (a - b)^2): kept alike
    const int xmetric = metric == CNN_METRIC_EUCLIDEAN_PERIODIC_REDUCED ? CNN_METRIC_EUCLIDEAN_REDUCED : metric;
    CNN_TRY(cross_neighbours_impl(ctx, xq, m, radius_cutoff, xmetric, fpmode, ctx->pred_xoff, ctx->pred_xcols, &xnnz));
    const unsigned blocks = std::min<unsigned>(grid_for(m * 32, 256), ctx->sm_count * 16u);
    predict_kernel<<<blocks, 256, 0, st>>>(m, ctx->pred_xoff.as<int64_t>(), ctx->pred_xcols.as<int32_t>(),
                                           ctx->pred_off.as<int64_t>(), ctx->pred_cols.as<int32_t>(), labels_dev,
                                           clusters_sorted_dev, n_clusters, similarity_cutoff, n_member_cutoff,
                                           other_labels_dev, other_consider_dev);
    CNN_LAUNCH_CHECK(ctx);
    return CNN_OK;
}

}  // namespace cnn
