// mst.cu -- edge weights and the maximum spanning forest of the
// common-neighbour graph (HierarchicalFitterMSTPrim).
//
// Reference: HierarchicalFitterMSTPrim._fit (src/cnnclustering/_fit.pyx:
// 820-899).  Every neighbour pair (a, b) is weighted by the full count of
// common neighbours |N(a) & N(b)| (SimilarityCheckerExtScreensorted._get,
// _types.pyx:2708-2753; both lists include their own point).  Prim's
// algorithm then grows a maximum spanning forest: from every unvisited point
// in index order, edges to unvisited neighbours go into a max-heap keyed
// (-weight, (a, b)) (PriorityQueueMaxHeap, _types.pyx:2825-2851); popped
// edges to unvisited points join the tree, whose own heap is popped last.
//
// GB300 form: the weights -- the O(sum of |N(a)| + |N(b)|) part -- are
// computed for all pairs at once, one warp per point counting its pairs
// (b > a) with the warp merge, and mirrored to (b, a) by a binary search.
// Prim's heap loop runs in the library's host code on those weights, so
// that ties resolve exactly as the reference's heap resolves them.
#include <algorithm>
#include <climits>
#include <queue>
#include <vector>

#include "common.cuh"
#include "fit_kernels.cuh"

namespace cnn {

namespace {

// |A & B| for ascending, duplicate-free lists (the whole warp, every lane
// returns the count): 32-wide chunks, each lane finds its B value among the
// 32 A values with a shuffle binary search, the chunk with the smaller
// maximum is consumed.
__device__ __forceinline__ int32_t warp_count_common(const int32_t *__restrict__ A, int32_t la,
                                                     const int32_t *__restrict__ B, int32_t lb, int lane) {
    int32_t ia = 0, ib = 0, count = 0;
    while (ia < la && ib < lb) {
        const int32_t va = ia + lane < la ? __ldg(A + ia + lane) : INT_MAX;
        const int32_t vb = ib + lane < lb ? __ldg(B + ib + lane) : INT_MAX - 1;
        int pos = 0;
#pragma unroll
        for (int step = 16; step > 0; step >>= 1) {
            const int32_t probe = __shfl_sync(0xffffffffu, va, pos + step - 1);
            if (probe < vb) pos += step;
        }
        const bool found = __shfl_sync(0xffffffffu, va, pos) == vb;
        count += __popc(__ballot_sync(0xffffffffu, found));
        const int32_t amax = __shfl_sync(0xffffffffu, va, 31);
        const int32_t bmax = __shfl_sync(0xffffffffu, vb, 31);
        if (amax <= bmax) ia += 32;
        if (bmax <= amax) ib += 32;
    }
    return count;
}

// weight of every stored pair (a, b > a); one warp per point a
__global__ void __launch_bounds__(256) pair_weight_kernel(int64_t n, const int64_t *__restrict__ off,
                                                          const int32_t *__restrict__ cols,
                                                          int32_t *__restrict__ weight) {
    const int lane = threadIdx.x & 31;
    const int64_t warp0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t a = warp0; a < n; a += nwarps) {
        const int64_t s = off[a], e = off[a + 1];
        const int32_t la = (int32_t)(e - s);
        for (int64_t k = warp_upper_bound(cols, s, e, (int32_t)a, lane); k < e; ++k) {
            const int32_t b = cols[k];
            const int64_t bs = off[b];
            const int32_t w = warp_count_common(cols + s, la, cols + bs, (int32_t)(off[b + 1] - bs), lane);
            if (lane == 0) weight[k] = w;
        }
    }
}

// (b, a < b) takes the weight of (a, b): binary search of b in row a
__global__ void mirror_weight_kernel(int64_t n, const int64_t *__restrict__ off, const int32_t *__restrict__ cols,
                                     int32_t *__restrict__ weight) {
    const int lane = threadIdx.x & 31;
    const int64_t warp0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t b = warp0; b < n; b += nwarps) {
        const int64_t s = off[b], e = off[b + 1];
        for (int64_t k = s + lane; k < e; k += 32) {
            const int32_t a = cols[k];
            if (a >= b) continue;
            int64_t lo = off[a], hi = off[a + 1];
            while (lo < hi) {
                const int64_t mid = (lo + hi) >> 1;
                if (cols[mid] < (int32_t)b) lo = mid + 1;
                else hi = mid;
            }
            weight[k] = (lo < off[a + 1] && cols[lo] == (int32_t)b) ? weight[lo] : 0;
        }
    }
}

struct HeapEdge {
    int64_t w;
    int32_t a, b;
};

// max-heap order of (-weight, (a, b)) in a min-heap: larger weight first,
// then smaller a, then smaller b
struct HeapAfter {
    bool operator()(const HeapEdge &x, const HeapEdge &y) const {
        if (x.w != y.w) return x.w < y.w;
        if (x.a != y.a) return x.a > y.a;
        return x.b > y.b;
    }
};

}  // namespace

cnn_status mst_prim_impl(cnn_context *ctx, double radius_cutoff, int metric, int fpmode, std::vector<int64_t> *ea,
                         std::vector<int64_t> *eb, std::vector<int64_t> *ew) {
    cudaStream_t st = ctx->stream;
    const int64_t n = ctx->n;
    ea->clear();
    eb->clear();
    ew->clear();
    if (n == 0) return CNN_OK;
    // the cell grid keeps the graph as masks unless the merge strategy is
    // asked for: full counts (no early exit) are what the bitset path is for
    CNN_TRY(build_neighbours_impl(ctx, radius_cutoff, metric, fpmode,
                                  ctx->intersect_pref == CNN_INTERSECT_MERGE ? kFormLists : kFormMasks));
    const int64_t nnz = ctx->nnz;
    CNN_TRY(ctx->ensure(ctx->pred_off, sizeof(int64_t) * (size_t)(n + 1)));
    CNN_TRY(ctx->ensure(ctx->pred_cols, sizeof(int32_t) * (size_t)(nnz > 0 ? nnz : 1)));
    CNN_TRY(ctx->ensure(ctx->pred_xcols, sizeof(int32_t) * (size_t)(nnz > 0 ? nnz : 1)));
    CNN_TRY(export_neighbours_impl(ctx, ctx->pred_off.as<int64_t>(), ctx->pred_cols.as<int32_t>()));
    int32_t *weight = ctx->pred_xcols.as<int32_t>();
    const unsigned blocks = std::min<unsigned>(grid_for(n * 32, 256), ctx->sm_count * 16u);
    stage_begin(ctx, 10);
    if (ctx->graph_mask) {
        CNN_TRY(mask_pair_weights(ctx, ctx->pred_off.as<int64_t>(), ctx->pred_cols.as<int32_t>(), weight));
        ctx->stats.intersection = CNN_INTERSECT_BITSET;
    } else {
        pair_weight_kernel<<<blocks, 256, 0, st>>>(n, ctx->pred_off.as<int64_t>(), ctx->pred_cols.as<int32_t>(),
                                                   weight);
        CNN_LAUNCH_CHECK(ctx);
        ctx->stats.intersection = CNN_INTERSECT_MERGE;
    }
    stage_end(ctx, 10);
    mirror_weight_kernel<<<blocks, 256, 0, st>>>(n, ctx->pred_off.as<int64_t>(), ctx->pred_cols.as<int32_t>(), weight);
    CNN_LAUNCH_CHECK(ctx);
    std::vector<int64_t> off(n + 1);
    std::vector<int32_t> cols(nnz), w(nnz);
    CNN_CUDA(ctx, cudaMemcpyAsync(off.data(), ctx->pred_off.ptr, sizeof(int64_t) * (size_t)(n + 1),
                                  cudaMemcpyDeviceToHost, st));
    if (nnz > 0) {
        CNN_CUDA(ctx, cudaMemcpyAsync(cols.data(), ctx->pred_cols.ptr, sizeof(int32_t) * (size_t)nnz,
                                      cudaMemcpyDeviceToHost, st));
        CNN_CUDA(ctx, cudaMemcpyAsync(w.data(), weight, sizeof(int32_t) * (size_t)nnz, cudaMemcpyDeviceToHost, st));
    }
    CNN_CUDA(ctx, cudaStreamSynchronize(st));

    // Prim, exactly the reference's loop and heap order
    std::vector<uint8_t> visited((size_t)n, 0);
    std::priority_queue<HeapEdge, std::vector<HeapEdge>, HeapAfter> heap, tree;
    auto push_row = [&](int64_t p) {
        for (int64_t k = off[p]; k < off[p + 1]; ++k)
            if (!visited[cols[k]]) heap.push(HeapEdge{w[k], (int32_t)p, cols[k]});
    };
    for (int64_t point = 0; point < n; ++point) {
        if (visited[point]) continue;
        visited[point] = 1;
        push_row(point);
        while (!heap.empty()) {
            const HeapEdge top = heap.top();
            heap.pop();
            if (visited[top.b]) continue;
            visited[top.b] = 1;
            tree.push(top);
            push_row(top.b);
        }
    }
    ea->reserve(tree.size());
    eb->reserve(tree.size());
    ew->reserve(tree.size());
    while (!tree.empty()) {
        const HeapEdge e = tree.top();
        tree.pop();
        ea->push_back(e.a);
        eb->push_back(e.b);
        ew->push_back(e.w);
    }
    return CNN_OK;
}

}  // namespace cnn
