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

// The reference's heap order of (-weight, (a, b)): larger weight first,
// then smaller a, then smaller b.
inline bool edge_before(const HeapEdge &x, const HeapEdge &y) {
    if (x.w != y.w) return x.w > y.w;
    if (x.a != y.a) return x.a < y.a;
    return x.b < y.b;
}

// Prim's frontier as an indexed heap with one entry per point not yet in
// the tree: its best edge (w, a) from the tree, ordered by edge_before of
// (w, a, b).  The reference's lazy heap holds every pushed (a, b) and pops
// the first by the same order among those whose b is not in the tree; that
// entry is the first over b of b's best entry, so popping this heap visits
// the points and picks the tree edges exactly as the reference does, with
// at most n entries instead of one per pair.
class Frontier {
  public:
    explicit Frontier(int64_t n) : pos_((size_t)n, -1), key_((size_t)n) {}
    bool empty() const { return heap_.empty(); }
    // b's entry becomes (w, a) if that comes first by the heap order
    void offer(int32_t b, int64_t w, int32_t a) {
        const HeapEdge e{w, a, b};
        int64_t i = pos_[b];
        if (i < 0) {
            key_[b] = e;
            i = (int64_t)heap_.size();
            heap_.push_back(b);
            pos_[b] = i;
        } else if (edge_before(e, key_[b])) {
            key_[b] = e;
        } else {
            return;
        }
        up(i);
    }
    HeapEdge pop() {
        const int32_t b = heap_[0];
        const HeapEdge e = key_[b];
        pos_[b] = -2;  // in the tree
        const int32_t last = heap_.back();
        heap_.pop_back();
        if (!heap_.empty()) {
            heap_[0] = last;
            pos_[last] = 0;
            down(0);
        }
        return e;
    }

  private:
    bool before(int32_t x, int32_t y) const { return edge_before(key_[x], key_[y]); }
    void up(int64_t i) {
        const int32_t b = heap_[i];
        while (i > 0) {
            const int64_t p = (i - 1) >> 1;
            if (!before(b, heap_[p])) break;
            heap_[i] = heap_[p];
            pos_[heap_[i]] = i;
            i = p;
        }
        heap_[i] = b;
        pos_[b] = i;
    }
    void down(int64_t i) {
        const int32_t b = heap_[i];
        const int64_t m = (int64_t)heap_.size();
        for (;;) {
            int64_t c = 2 * i + 1;
            if (c >= m) break;
            if (c + 1 < m && before(heap_[c + 1], heap_[c])) ++c;
            if (!before(heap_[c], b)) break;
            heap_[i] = heap_[c];
            pos_[heap_[i]] = i;
            i = c;
        }
        heap_[i] = b;
        pos_[b] = i;
    }
    std::vector<int64_t> pos_;  // index in heap_, -1 never offered, -2 in the tree
    std::vector<HeapEdge> key_;
    std::vector<int32_t> heap_;
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

    // Prim, the reference's loop and heap order (Frontier); the tree edges
    // then leave in the tree queue's order, the same heap order
    std::vector<uint8_t> visited((size_t)n, 0);
    Frontier frontier(n);
    std::vector<HeapEdge> tree;
    tree.reserve((size_t)(n > 0 ? n - 1 : 0));
    auto offer_row = [&](int64_t p) {
        for (int64_t k = off[p]; k < off[p + 1]; ++k)
            if (!visited[cols[k]]) frontier.offer(cols[k], w[k], (int32_t)p);
    };
    for (int64_t point = 0; point < n; ++point) {
        if (visited[point]) continue;
        visited[point] = 1;
        offer_row(point);
        while (!frontier.empty()) {
            const HeapEdge top = frontier.pop();
            visited[top.b] = 1;
            tree.push_back(top);
            offer_row(top.b);
        }
    }
    std::sort(tree.begin(), tree.end(), edge_before);
    ea->reserve(tree.size());
    eb->reserve(tree.size());
    ew->reserve(tree.size());
    for (const HeapEdge &e : tree) {
        ea->push_back(e.a);
        eb->push_back(e.b);
        ew->push_back(e.w);
    }
    return CNN_OK;
}

}  // namespace cnn
