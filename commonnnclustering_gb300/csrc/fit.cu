// fit.cu -- cluster assignment on the neighbour graph.
//
// Reference: FitterExtBFS._fit (src/cnnclustering/_fit.pyx:408-491) grows
// clusters breadth-first.  A point is a node when it has more than
// n_member_cutoff neighbours (NeighboursExtVector._enough,
// _types.pyx:1408-1411, strict '>') and consider == 1.  From a node a, a
// neighbour b that is also a node joins a's cluster when the two lists
// share at least similarity_cutoff members
// (SimilarityCheckerExtScreensorted._check, _types.pyx:2654-2706: c == 0
// passes, otherwise count common members until c).  Because the neighbour
// relation of a metric is symmetric and the check is symmetric in (a, b),
// the set labelled by one BFS is exactly one connected component of the
// graph {nodes, accepted edges}, and labels are handed out in the order of
// each component's lowest point index (the BFS seeds are visited in index
// order and a seed is always the lowest unvisited node of its component).
//
// GB300 form:
//   1. node flags;
//   2. one warp per node a walks its neighbours b > a.  An edge is checked
//      only if find(a) != find(b) at that moment: edges inside an already
//      joined set cannot change the components, so skipping them is exact.
//      The check merges N(a) and N(b) 32 entries at a time (each lane looks
//      one member of N(b) up among 32 of N(a) by shuffles) and stops as soon
//      as the count reaches the cutoff or can no longer reach it.  Accepted
//      edges are joined with a lock-free union-find (CAS on roots, path
//      halving).  A hook pass checks three edges per node; a read-only pass
//      then lists the edges whose roots still differ and only those are
//      checked;
//   3. per component, the minimum point index; ranks of those minima give
//      the labels (current_start + rank), written in point order.
#include <climits>

#include <algorithm>
#include <type_traits>

#include "common.cuh"
#include "fit_kernels.cuh"

namespace cnn {

namespace {

// ---- cross-edge worklist ------------------------------------------------------
// row entries per lane per step of the pair filters: 4 for the cross filter
// every fit runs (rows of a few hundred entries b > a), 8 for the sweep's
// passes over long rows and flat edge lists
#ifndef CNN_FILTER_UNROLL
#define CNN_FILTER_UNROLL 4
#endif
#ifndef CNN_LIST_UNROLL
#define CNN_LIST_UNROLL 8
#endif
constexpr int kFilterUnroll = CNN_FILTER_UNROLL;
constexpr int kListUnroll = CNN_LIST_UNROLL;

// After the hook pass and a full compression, parent[] holds every node's
// root.  A read-only pass streams the graph and keeps only candidate edges
// (a, b > a, both nodes) whose roots differ; everything else is already
// joined.  The worklist is then checked edge by edge with the same lazy
// rule.  If it overflows its capacity, the full lazy pass runs instead.
template <bool kSlotRows>
__global__ void __launch_bounds__(256) cross_filter_kernel(int64_t n, const int64_t *__restrict__ row_start,
                                                           const int64_t *__restrict__ row_end,
                                                           const int32_t *__restrict__ cols,
                                                           const int32_t *__restrict__ parent,
                                                           int2 *__restrict__ wl,
                                                           unsigned long long *__restrict__ wl_count,
                                                           int64_t cap, const int32_t *__restrict__ split) {
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    const int64_t warp0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t a64 = warp0; a64 < n; a64 += nwarps) {
        const int32_t a = (int32_t)a64;
        // parent[a], the row bounds and split[a] in one round trip
        int64_t v = 0;
        if (lane == 0) v = parent[a];
        else if (lane < 3) v = (kSlotRows && lane == 2) ? row_end[a] : row_start[a + (kSlotRows ? 0 : lane - 1)];
        else if (lane == 3 && split) v = split[a];
        const int32_t pa = (int32_t)__shfl_sync(0xffffffffu, v, 0);
        if (pa < 0) continue;
        const int64_t s = __shfl_sync(0xffffffffu, v, 1), e = __shfl_sync(0xffffffffu, v, 2);
        const int64_t split_a = __shfl_sync(0xffffffffu, v, 3);
        // 32 kFilterUnroll entries per step, kFilterUnroll per lane: the column
        // loads, then the parent loads, are in flight together; one worklist
        // atomic per step
        for (int64_t k0 = split ? s + split_a : warp_upper_bound(cols, s, e, a, lane); k0 < e;
             k0 += kFilterUnroll * 32) {
            int32_t b[kFilterUnroll], pb[kFilterUnroll];
#pragma unroll
            for (int u = 0; u < kFilterUnroll; ++u) {
                const int64_t k = k0 + u * 32 + lane;
                b[u] = k < e ? cols[k] : -1;
            }
#pragma unroll
            for (int u = 0; u < kFilterUnroll; ++u) pb[u] = b[u] > a ? parent[b[u]] : -1;
            unsigned mask[kFilterUnroll];
            int total = 0;
#pragma unroll
            for (int u = 0; u < kFilterUnroll; ++u) {
                mask[u] = __ballot_sync(0xffffffffu, pb[u] >= 0 && pb[u] != pa);
                total += __popc(mask[u]);
            }
            if (!total) continue;
            unsigned long long base = 0;
            if (lane == 0) base = atomicAdd(wl_count, (unsigned long long)total);
            base = __shfl_sync(0xffffffffu, base, 0);
#pragma unroll
            for (int u = 0; u < kFilterUnroll; ++u) {
                const unsigned long long idx = base + __popc(mask[u] & lt);
                if (((mask[u] >> lane) & 1u) && idx < (unsigned long long)cap) wl[idx] = make_int2(a, b[u]);
                base += __popc(mask[u]);
            }
        }
    }
}

// The cross filter over an edge list (a, b > a) instead of the graph; the
// list's length is read on the device.
__global__ void __launch_bounds__(256) cross_filter_list_kernel(const int2 *__restrict__ edges,
                                                                const unsigned long long *__restrict__ count,
                                                                const int32_t *__restrict__ parent,
                                                                int2 *__restrict__ wl,
                                                                unsigned long long *__restrict__ wl_count,
                                                                int64_t cap) {
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    const int64_t total = (int64_t)*count;
    // each warp takes 32 kListUnroll consecutive edges per step, kListUnroll
    // per lane: the edge loads, then the parent loads, are in flight together
    const int64_t stride = (int64_t)gridDim.x * blockDim.x * kListUnroll;
    for (int64_t base = ((int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31)) * kListUnroll; base < total;
         base += stride) {
        int2 ed[kListUnroll];
#pragma unroll
        for (int u = 0; u < kListUnroll; ++u) {
            const int64_t e = base + u * 32 + lane;
            ed[u] = e < total ? edges[e] : make_int2(-1, -1);
        }
        int32_t pa[kListUnroll], pb[kListUnroll];
#pragma unroll
        for (int u = 0; u < kListUnroll; ++u) {
            pa[u] = ed[u].x >= 0 ? parent[ed[u].x] : -1;
            pb[u] = ed[u].x >= 0 ? parent[ed[u].y] : -1;
        }
        unsigned mask[kListUnroll];
        int n_cross = 0;
#pragma unroll
        for (int u = 0; u < kListUnroll; ++u) {
            mask[u] = __ballot_sync(0xffffffffu, pa[u] >= 0 && pb[u] >= 0 && pa[u] != pb[u]);
            n_cross += __popc(mask[u]);
        }
        if (!n_cross) continue;
        unsigned long long w = 0;
        if (lane == 0) w = atomicAdd(wl_count, (unsigned long long)n_cross);
        w = __shfl_sync(0xffffffffu, w, 0);
#pragma unroll
        for (int u = 0; u < kListUnroll; ++u) {
            const unsigned long long idx = w + __popc(mask[u] & lt);
            if (((mask[u] >> lane) & 1u) && idx < (unsigned long long)cap) wl[idx] = ed[u];
            w += __popc(mask[u]);
        }
    }
}

// Pairs (a, b > a) a finished fit leaves open for a fit it refines: all
// but those whose points are nodes with the same root (parent holds roots).
__device__ __forceinline__ bool pair_open(const uint8_t *__restrict__ node, const int32_t *__restrict__ parent,
                                          int32_t a, int32_t b) {
    return !(node[a] && node[b] && parent[a] == parent[b]);
}

__global__ void __launch_bounds__(256) open_pairs_csr_kernel(int64_t n, const int64_t *__restrict__ row_off,
                                                             const int32_t *__restrict__ cols,
                                                             const uint8_t *__restrict__ node,
                                                             const int32_t *__restrict__ parent,
                                                             int2 *__restrict__ out,
                                                             unsigned long long *__restrict__ out_count,
                                                             int64_t cap) {
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    const int64_t warp0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t a64 = warp0; a64 < n; a64 += nwarps) {
        const int32_t a = (int32_t)a64;
        const int64_t s = row_off[a], e = row_off[a + 1];
        // pair_open(a, b) with a's node flag and root read once per row
        const bool na = node[a] != 0;
        const int32_t ra = parent[a];
        for (int64_t k0 = warp_upper_bound(cols, s, e, a, lane); k0 < e; k0 += kListUnroll * 32) {
            int32_t b[kListUnroll];
#pragma unroll
            for (int u = 0; u < kListUnroll; ++u) {  // kListUnroll entries per lane in flight
                const int64_t k = k0 + u * 32 + lane;
                b[u] = k < e ? cols[k] : -1;
            }
            bool keep[kListUnroll];
#pragma unroll
            for (int u = 0; u < kListUnroll; ++u)
                keep[u] = b[u] > a && !(na && node[b[u]] && ra == parent[b[u]]);
            unsigned mask[kListUnroll];
            int total = 0;
#pragma unroll
            for (int u = 0; u < kListUnroll; ++u) {
                mask[u] = __ballot_sync(0xffffffffu, keep[u]);
                total += __popc(mask[u]);
            }
            if (!total) continue;
            unsigned long long w = 0;
            if (lane == 0) w = atomicAdd(out_count, (unsigned long long)total);
            w = __shfl_sync(0xffffffffu, w, 0);
#pragma unroll
            for (int u = 0; u < kListUnroll; ++u) {
                const unsigned long long idx = w + __popc(mask[u] & lt);
                if (keep[u] && idx < (unsigned long long)cap) out[idx] = make_int2(a, b[u]);
                w += __popc(mask[u]);
            }
        }
    }
}

__global__ void __launch_bounds__(256) open_pairs_list_kernel(const int2 *__restrict__ edges,
                                                              const unsigned long long *__restrict__ count,
                                                              const uint8_t *__restrict__ node,
                                                              const int32_t *__restrict__ parent,
                                                              int2 *__restrict__ out,
                                                              unsigned long long *__restrict__ out_count,
                                                              int64_t cap) {
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    const int64_t total = (int64_t)*count;
    // 32 kListUnroll consecutive edges per warp step, kListUnroll per lane in flight
    const int64_t stride = (int64_t)gridDim.x * blockDim.x * kListUnroll;
    for (int64_t base = ((int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31)) * kListUnroll; base < total;
         base += stride) {
        int2 ed[kListUnroll];
#pragma unroll
        for (int u = 0; u < kListUnroll; ++u) {
            const int64_t e = base + u * 32 + lane;
            ed[u] = e < total ? edges[e] : make_int2(-1, -1);
        }
        unsigned mask[kListUnroll];
        int n_keep = 0;
#pragma unroll
        for (int u = 0; u < kListUnroll; ++u) {
            mask[u] = __ballot_sync(0xffffffffu, ed[u].x >= 0 && pair_open(node, parent, ed[u].x, ed[u].y));
            n_keep += __popc(mask[u]);
        }
        if (!n_keep) continue;
        unsigned long long w = 0;
        if (lane == 0) w = atomicAdd(out_count, (unsigned long long)n_keep);
        w = __shfl_sync(0xffffffffu, w, 0);
#pragma unroll
        for (int u = 0; u < kListUnroll; ++u) {
            const unsigned long long idx = w + __popc(mask[u] & lt);
            if (((mask[u] >> lane) & 1u) && idx < (unsigned long long)cap) out[idx] = ed[u];
            w += __popc(mask[u]);
        }
    }
}

template <bool kSlotRows>
__global__ void __launch_bounds__(kCheckWarps * 32, CNN_CHECK_MIN_BLOCKS) edge_check_kernel(const int2 *__restrict__ wl,
                                                         const unsigned long long *__restrict__ wl_count,
                                                         int64_t cap, const int64_t *__restrict__ row_start,
                                                         const int64_t *__restrict__ row_end,
                                                         const int32_t *__restrict__ cols,
                                                         int32_t *__restrict__ parent, int32_t needed,
                                                         unsigned long long *__restrict__ counters) {
    __shared__ int32_t s_wide[kCheckWarps][kWideChunk];
    int32_t *sA = s_wide[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    const int64_t warp0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const unsigned long long total = *wl_count;
    if (total > (unsigned long long)cap) return;  // overflow: the full lazy pass runs instead
    const int64_t count = (int64_t)total;
    unsigned long long n_checks = 0, n_acc = 0;
    for (int64_t base = warp0 * 32; base < count; base += nwarps * 32) {
        const int64_t e = base + lane;
        const bool valid = e < count;
        int32_t a = -1, b = -1, ra = -1, rb = -1;
        if (valid) {
            const int2 ed = wl[e];
            a = ed.x;
            b = ed.y;
            ra = uf_find(parent, a);
            rb = uf_find(parent, b);
        }
        unsigned mask = __ballot_sync(0xffffffffu, valid && ra != rb);
        bool dirty = false;
        while (mask) {
            if (dirty) {
                const bool live = (mask >> lane) & 1u;
                if (live) {
                    ra = uf_find(parent, ra);
                    rb = uf_find(parent, rb);
                }
                mask = __ballot_sync(0xffffffffu, live && ra != rb);
                dirty = false;
                if (!mask) break;
            }
            const int src = __ffs(mask) - 1;
            mask &= mask - 1;
            const int32_t aa = __shfl_sync(0xffffffffu, a, src);
            const int32_t bb = __shfl_sync(0xffffffffu, b, src);
            bool ok;
            if (needed <= 0) {
                ok = needed == 0;
            } else {
                const int64_t as = row_start[aa], bs = row_start[bb];
                const int64_t ae = kSlotRows ? row_end[aa] : row_start[aa + 1];
                const int64_t be = kSlotRows ? row_end[bb] : row_start[bb + 1];
                ok = warp_shares(cols + as, (int32_t)(ae - as), cols + bs, (int32_t)(be - bs), needed, lane, sA);
                ++n_checks;
            }
            if (ok) {
                if (lane == 0) uf_unite(parent, aa, bb);
                __syncwarp();
                ++n_acc;
                dirty = true;
            }
        }
    }
    if (lane == 0 && n_checks) atomicAdd(&counters[5], n_checks);
    if (lane == 0 && n_acc) atomicAdd(&counters[6], n_acc);
}

// The full lazy pass, run only when the worklist overflowed.
template <bool kSlotRows>
__global__ void __launch_bounds__(kCheckWarps * 32) check_union_if_overflow_kernel(
    int64_t n, const int64_t *__restrict__ row_start, const int64_t *__restrict__ row_end,
    const int32_t *__restrict__ cols, int32_t *__restrict__ parent,
    int32_t needed, const unsigned long long *__restrict__ wl_count, int64_t cap,
    unsigned long long *__restrict__ counters) {
    if (*wl_count <= (unsigned long long)cap) return;
    // same body as the full pass of check_union_kernel
    check_union_body<kSlotRows>(n, row_start, row_end, cols, parent, needed, INT32_MAX, counters);
}

// ---- sort_by_size ---------------------------------------------------------
// Range and count of the nonzero labels: per block in shared memory, then
// one set of atomics per block.
__global__ void __launch_bounds__(256) label_range_kernel(const int64_t *__restrict__ labels, int64_t n,
                                                          long long *__restrict__ out) {
    __shared__ long long s_lo[8], s_hi[8];
    __shared__ unsigned long long s_nz[8];
    long long lo = LLONG_MAX, hi = LLONG_MIN;
    unsigned long long nz = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const long long v = labels[i];
        if (v == 0) continue;
        lo = v < lo ? v : lo;
        hi = v > hi ? v : hi;
        ++nz;
    }
    for (int o = 16; o > 0; o >>= 1) {
        long long l2 = __shfl_down_sync(0xffffffffu, lo, o);
        long long h2 = __shfl_down_sync(0xffffffffu, hi, o);
        nz += __shfl_down_sync(0xffffffffu, nz, o);
        lo = l2 < lo ? l2 : lo;
        hi = h2 > hi ? h2 : hi;
    }
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        s_lo[w] = lo;
        s_hi[w] = hi;
        s_nz[w] = nz;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < (int)(blockDim.x >> 5); ++k) {
            lo = s_lo[k] < lo ? s_lo[k] : lo;
            hi = s_hi[k] > hi ? s_hi[k] : hi;
            nz += s_nz[k];
        }
        if (nz) {
            atomicMin(&out[0], lo);
            atomicMax(&out[1], hi);
            atomicAdd((unsigned long long *)&out[2], nz);
        }
    }
}

__global__ void init_range_kernel(long long *out) {
    out[0] = LLONG_MAX;
    out[1] = LLONG_MIN;
    out[2] = 0;
}

__global__ void dense_id_kernel(const int64_t *__restrict__ labels, int64_t n, long long lo, int32_t *__restrict__ ids) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t v = labels[i];
        ids[i] = v == 0 ? -1 : (int32_t)(v - lo);
    }
}

// Sparse label values: order-preserving 64-bit keys (sign bit flipped).
__global__ void label_keys_kernel(const int64_t *__restrict__ labels, int64_t n, uint64_t *__restrict__ keys) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        keys[i] = (uint64_t)labels[i] ^ 0x8000000000000000ull;
}

__global__ void unique_flag_kernel(const uint64_t *__restrict__ keys, int64_t n, int32_t *__restrict__ flag) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        flag[i] = (i == 0 || keys[i] != keys[i - 1]) ? 1 : 0;
}

__global__ void unique_compact_kernel(const uint64_t *__restrict__ keys, const int32_t *__restrict__ flag,
                                      const int64_t *__restrict__ pos, int64_t n, uint64_t *__restrict__ uniq) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        if (flag[i]) uniq[pos[i]] = keys[i];
}

__global__ void sparse_id_kernel(const int64_t *__restrict__ labels, int64_t n, const uint64_t *__restrict__ uniq,
                                 int64_t nu, int32_t *__restrict__ ids) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t v = labels[i];
        if (v == 0) { ids[i] = -1; continue; }
        const uint64_t key = (uint64_t)v ^ 0x8000000000000000ull;
        int64_t lo = 0, hi = nu;
        while (lo < hi) {
            int64_t mid = (lo + hi) >> 1;
            if (uniq[mid] < key) lo = mid + 1; else hi = mid;
        }
        ids[i] = (int32_t)lo;
    }
}

__global__ void count_first_kernel(const int32_t *__restrict__ ids, int64_t n, int32_t *__restrict__ cnt,
                                   int32_t *__restrict__ first) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t id = ids[i];
        if (id < 0) continue;
        atomicAdd(&cnt[id], 1);
        atomicMin(&first[id], (int32_t)i);
    }
}

__global__ void cluster_flag_kernel(const int32_t *__restrict__ cnt, int64_t r, int32_t *__restrict__ flag) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < r; i += (int64_t)gridDim.x * blockDim.x)
        flag[i] = cnt[i] > 0 ? 1 : 0;
    if (blockIdx.x == 0 && threadIdx.x == 0) flag[r] = 0;
}

// key = (n - size) << bits_n | first: ascending key = size descending, then
// first occurrence ascending (Counter.most_common's order).
__global__ void cluster_key_kernel(const int32_t *__restrict__ cnt, const int32_t *__restrict__ first,
                                   const int64_t *__restrict__ pos, int64_t r, int64_t n, int bits_n,
                                   uint64_t *__restrict__ keys) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < r; i += (int64_t)gridDim.x * blockDim.x) {
        if (cnt[i] <= 0) continue;
        keys[pos[i]] = ((uint64_t)(n - cnt[i]) << bits_n) | (uint64_t)first[i];
    }
}

__global__ void new_label_kernel(const uint64_t *__restrict__ keys, int64_t k, int64_t n, int bits_n,
                                 const int32_t *__restrict__ ids, int64_t member_cutoff, int64_t max_clusters,
                                 int64_t *__restrict__ newlab) {
    const uint64_t mask = (1ull << bits_n) - 1;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < k; q += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t key = keys[q];
        const int64_t first = (int64_t)(key & mask);
        const int64_t size = n - (int64_t)(key >> bits_n);
        const int64_t rank = q + 1;  // cluster_count in the reference loop
        newlab[ids[first]] = (rank > max_clusters) ? 0 : (size >= member_cutoff ? rank : 0);
    }
}

// ---- sort_by_size for label ranges of up to kOrderSmall values -------------
// One pass counts sizes and first occurrences per label value (lo..lo+r-1);
// one kernel ranks the clusters by (size descending, first occurrence
// ascending) and writes the new label of every value; one pass applies it.
// The ranking block holds all r keys in shared memory (8 bytes each), so r
// is bounded by the shared memory of a block.
constexpr int kOrderSmall = 24576;
constexpr int kOrderThreads = 1024;

__global__ void init_count_first_kernel(int32_t *__restrict__ cnt, int32_t *__restrict__ first, int64_t r) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < r; i += (int64_t)gridDim.x * blockDim.x) {
        cnt[i] = 0;
        first[i] = INT32_MAX;
    }
}

// Points in label order are often runs of one value: lanes with the same
// value add their count with one atomic.
__global__ void count_first_dense_kernel(const int64_t *__restrict__ labels, int64_t n, int64_t lo,
                                         int32_t *__restrict__ cnt, int32_t *__restrict__ first) {
    const int lane = threadIdx.x & 31;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < n; base += stride) {
        const int64_t i = base + lane;
        const int64_t v = i < n ? labels[i] : 0;
        const int32_t id = v == 0 ? -1 : (int32_t)(v - lo);
        const unsigned peers = __match_any_sync(0xffffffffu, id);
        if (id >= 0 && lane == __ffs(peers) - 1) {
            atomicAdd(&cnt[id], __popc(peers));
            atomicMin(&first[id], (int32_t)i);  // the lowest lane holds the lowest index of its peers
        }
    }
}

// New label of every value: its rank among the used values' keys (size
// descending, first occurrence ascending; distinct per value).  Every block
// holds all keys in shared memory; each warp ranks its values in turn, the
// lanes striding over the keys.
__global__ void __launch_bounds__(kOrderThreads) order_small_kernel(
    const int32_t *__restrict__ cnt, const int32_t *__restrict__ first, int r, int per_block, int64_t n, int bits_n,
    int64_t member_cutoff, int64_t max_clusters, int64_t *__restrict__ newlab) {
    extern __shared__ uint64_t s_keys[];  // [r]
    __shared__ int s_k;
    if (threadIdx.x == 0) s_k = 0;
    __syncthreads();
    int local = 0;
    for (int i = threadIdx.x; i < r; i += blockDim.x) {
        const bool used = cnt[i] > 0;
        s_keys[i] = used ? (((uint64_t)(n - cnt[i]) << bits_n) | (uint64_t)first[i]) : ~0ull;
        local += used;
    }
    for (int o = 16; o > 0; o >>= 1) local += __shfl_down_sync(0xffffffffu, local, o);
    if ((threadIdx.x & 31) == 0 && local) atomicAdd(&s_k, local);
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const int v_end = min(r, (int)(blockIdx.x + 1) * per_block);
    for (int i = (int)blockIdx.x * per_block + warp; i < v_end; i += nwarps) {
        const uint64_t key = s_keys[i];
        int below = 0;
        for (int j = lane; j < r; j += 32) below += s_keys[j] < key;
        below = __reduce_add_sync(0xffffffffu, below);
        if (lane != 0) continue;
        if (key == ~0ull) {  // value not used
            newlab[i] = 0;
            continue;
        }
        const int64_t maxc = max_clusters < 0 ? s_k : max_clusters;
        const int64_t rank = below + 1;  // cluster_count in the reference loop
        newlab[i] = rank > maxc ? 0 : ((int64_t)cnt[i] >= member_cutoff ? rank : 0);
    }
}

__global__ void apply_dense_kernel(int64_t *__restrict__ labels, int64_t n, int64_t lo,
                                   const int64_t *__restrict__ newlab) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t v = labels[i];
        if (v != 0) labels[i] = newlab[v - lo];
    }
}

// ---- sort_by_size of fresh labels, without a host round trip --------------
// After a fit from fresh labels (all 0, current_start 1) the clusters are
// 1..k in order of their lowest point index, so the first occurrence order
// is the label order and k is known on the device (the fit's rank total).
// Sizes are counted per label; keys (n - size, label - 1) of labels 1..k are
// radix-sorted on the size bits only (the label bits are ascending already);
// key q gives its label the new label q + 1, or 0 past max_clusters or
// below member_cutoff -- the same rule as new_label_kernel.
// Up to kFreshSmemBins labels (the count read on the device) each block
// counts in shared memory and adds its nonzero bins once; more labels go to
// global atomics directly.  Either way warps first merge equal labels.
constexpr int kFreshSmemBins = 2048;

__global__ void __launch_bounds__(256) fresh_count_kernel(const int64_t *__restrict__ labels, int64_t n,
                                                          const int64_t *__restrict__ k_dev,
                                                          int32_t *__restrict__ cnt) {
    __shared__ int32_t s_cnt[kFreshSmemBins];
    const int64_t k = *k_dev < n ? *k_dev : n;
    const bool local = k <= kFreshSmemBins;  // block-uniform
    if (local) {
        for (int i = threadIdx.x; i < (int)k; i += blockDim.x) s_cnt[i] = 0;
        __syncthreads();
    }
    const int lane = threadIdx.x & 31;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < n; base += stride) {
        const int64_t i = base + lane;
        const int64_t v = i < n ? labels[i] : 0;
        const unsigned peers = __match_any_sync(0xffffffffu, v);
        if (v > 0 && v <= k && lane == __ffs(peers) - 1) {
            if (local) atomicAdd(&s_cnt[v - 1], __popc(peers));
            else atomicAdd(&cnt[v - 1], __popc(peers));
        }
    }
    if (local) {
        __syncthreads();
        for (int i = threadIdx.x; i < (int)k; i += blockDim.x)
            if (s_cnt[i]) atomicAdd(&cnt[i], s_cnt[i]);
    }
}

// Up to kOrderSmall labels: every block holds all keys in shared memory and
// its warps rank a slice of the labels (as order_small_kernel does); the
// count k_big for the radix path is k when k is larger, else 0.
__global__ void __launch_bounds__(kOrderThreads) fresh_order_small_kernel(
    const int32_t *__restrict__ cnt, const int64_t *__restrict__ k_dev, int64_t n, int bits_n, int64_t member_cutoff,
    int64_t max_clusters, int64_t *__restrict__ newlab, int64_t *__restrict__ k_big) {
    extern __shared__ uint64_t s_keys[];  // [min(n, kOrderSmall)]
    const int64_t k = *k_dev < n ? *k_dev : n;
    if (blockIdx.x == 0 && threadIdx.x == 0) *k_big = k > kOrderSmall ? k : 0;
    if (k > kOrderSmall || k <= 0) return;
    const int kk = (int)k;
    const int per_block = (kk + (int)gridDim.x - 1) / (int)gridDim.x;
    const int v0 = (int)blockIdx.x * per_block;
    if (v0 >= kk) return;  // block-uniform
    for (int i = threadIdx.x; i < kk; i += blockDim.x) s_keys[i] = ((uint64_t)(n - cnt[i]) << bits_n) | (uint64_t)i;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const int v_end = min(kk, v0 + per_block);
    const int64_t maxc = max_clusters < 0 ? k : max_clusters;
    for (int i = v0 + warp; i < v_end; i += nwarps) {
        const uint64_t key = s_keys[i];
        int below = 0;
        for (int j = lane; j < kk; j += 32) below += s_keys[j] < key;
        below = __reduce_add_sync(0xffffffffu, below);
        if (lane != 0) continue;
        const int64_t rank = below + 1;
        newlab[i] = rank > maxc ? 0 : ((int64_t)cnt[i] >= member_cutoff ? rank : 0);
    }
}

__global__ void fresh_keys_kernel(const int32_t *__restrict__ cnt, const int64_t *__restrict__ k_dev, int64_t n,
                                  int bits_n, uint64_t *__restrict__ keys) {
    const int64_t k = *k_dev < n ? *k_dev : n;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < k; q += (int64_t)gridDim.x * blockDim.x)
        keys[q] = ((uint64_t)(n - cnt[q]) << bits_n) | (uint64_t)q;
}

__global__ void fresh_new_label_kernel(const uint64_t *__restrict__ keys, const int64_t *__restrict__ k_dev, int64_t n,
                                       int bits_n, int64_t member_cutoff, int64_t max_clusters,
                                       int64_t *__restrict__ newlab) {
    const int64_t k = *k_dev < n ? *k_dev : n;
    const int64_t maxc = max_clusters < 0 ? k : max_clusters;
    const uint64_t mask = (1ull << bits_n) - 1;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < k; q += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t key = keys[q];
        const int64_t size = n - (int64_t)(key >> bits_n);
        const int64_t rank = q + 1;
        newlab[key & mask] = (rank > maxc) ? 0 : (size >= member_cutoff ? rank : 0);
    }
}

__global__ void apply_label_kernel(int64_t *__restrict__ labels, const int32_t *__restrict__ ids, int64_t n,
                                   const int64_t *__restrict__ newlab) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t id = ids[i];
        labels[i] = id < 0 ? 0 : newlab[id];
    }
}

__global__ void check_lists_kernel(const int32_t *__restrict__ a, int64_t na, const int32_t *__restrict__ b,
                                   int64_t nb, int64_t c, int32_t *__restrict__ result) {
    const int lane = threadIdx.x & 31;
    int32_t r;
    if (c == 0) r = 1;
    else if (na == 0 || nb == 0 || c < 0) r = 0;
    else if (c > na || c > nb) r = 0;
    else r = warp_shares_at_least(a, (int32_t)na, b, (int32_t)nb, (int32_t)c, lane) ? 1 : 0;
    if (lane == 0) *result = r;
}

unsigned blocks_for(const cnn_context *ctx, int64_t n) { return std::min<unsigned>(grid_for(n, 256), ctx->sm_count * 16u); }

}  // namespace

int bits_for_fit(int64_t n) {
    int b = 1;
    while (b < 62 && (int64_t(1) << b) < n) ++b;
    return b;
}

// Seeds (batched sweep): join every node p with seed[p] (a node, or -1) of
// a finished fit whose components refine this fit's components.
__global__ void seed_union_kernel(int64_t n, const uint8_t *__restrict__ node, int32_t *__restrict__ parent,
                                  const int32_t *__restrict__ seed_a, const int32_t *__restrict__ seed_b) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
        if (!node[p]) continue;
        const int32_t a = seed_a ? seed_a[p] : -1, b = seed_b ? seed_b[p] : -1;
        if (a >= 0 && a != p && node[a]) uf_unite(parent, (int32_t)p, a);
        if (b >= 0 && b != p && node[b]) uf_unite(parent, (int32_t)p, b);
    }
}

cnn_status fit_impl(cnn_context *ctx, int64_t similarity_cutoff, int64_t n_member_cutoff, int64_t current_start,
                    uint8_t *consider_dev, int64_t *labels_dev, const int32_t *seed_a, const int32_t *seed_b,
                    const int2 *edge_list, const unsigned long long *edge_count, int2 *wl_buf,
                    int64_t wl_buf_cap) {
    ctx->counted_labels = nullptr;  // set by the label stage
    stages_reset(ctx, 5, 8);           // nodes, check, labels, sort: this fit's own
    if (!ctx->have_graph) return ctx->fail(CNN_ERR_STATE, "no neighbour graph: call cnn_build_neighbours first");
    CNN_TRY(ensure_lists(ctx));
    const int64_t n = ctx->n;
    cudaStream_t st = ctx->stream;
    ctx->fit_stats_pending = false;
    if (n == 0) return CNN_OK;
    // no list is longer than 2^31-1; any negative cutoff rejects every pair
    if (similarity_cutoff > INT32_MAX) similarity_cutoff = INT32_MAX;
    if (similarity_cutoff < -1) similarity_cutoff = -1;
    CNN_TRY(ctx->ensure(ctx->node, (size_t)n));
    CNN_TRY(ctx->ensure(ctx->parent, sizeof(int32_t) * (size_t)n));
    CNN_TRY(ctx->ensure(ctx->comp_min, sizeof(int32_t) * (size_t)n));
    CNN_TRY(ctx->ensure(ctx->flag, sizeof(int32_t) * (size_t)(2 * n + 1)));  // + the component sizes
    CNN_TRY(ctx->ensure(ctx->scratch_a, sizeof(int64_t) * (size_t)(n + 1)));
    unsigned long long *counters = ctx->counters.as<unsigned long long>();
    CNN_CUDA(ctx, cudaMemsetAsync(counters + 4, 0, 5 * sizeof(unsigned long long), st));
    uint8_t *node = ctx->node.as<uint8_t>();
    int32_t *parent = ctx->parent.as<int32_t>();
    int32_t *comp_min = ctx->comp_min.as<int32_t>();
    const int32_t *perm = ctx->perm.as<int32_t>();

    stage_begin(ctx, 5);
    node_kernel<<<blocks_for(ctx, n), 256, 0, st>>>(ctx->deg.as<int32_t>(), perm, consider_dev, n, n_member_cutoff,
                                               node, parent, comp_min, counters);
    CNN_LAUNCH_CHECK(ctx);
    if (seed_a || seed_b) {
        seed_union_kernel<<<blocks_for(ctx, n), 256, 0, st>>>(n, node, parent, seed_a, seed_b);
        CNN_LAUNCH_CHECK(ctx);
    }
    stage_end(ctx, 5);

    stage_begin(ctx, 6);
    // persistent warps: exactly the blocks that are resident at once, so
    // that no block (and the nodes it strides over) waits for a second wave
    auto resident = [&](const void *kernel, int threads, size_t smem) -> unsigned {
        int per_sm = 0, sms = 0, dev = 0;
        cudaGetDevice(&dev);
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem) != cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
            (void)cudaGetLastError();
            per_sm = 8;
            sms = (int)ctx->sm_count;
        }
        return std::min<unsigned>(grid_for(n, kCheckWarps), (unsigned)std::max(1, per_sm * sms));
    };
    // rows ascending: the entries > a start at split[a] when the search recorded it
    const int32_t *split = ctx->split_valid ? ctx->split.as<int32_t>() : nullptr;
    // the rows: the CSR, or the slots the search left them in (no CSR asked for yet)
    const bool slots = ctx->graph_slots && !ctx->csr_valid;
    const RowView g = slots ? RowView{ctx->grid_qslot.as<int64_t>(), ctx->grid_qend.as<int64_t>(),
                                      ctx->grid_slot_cols.as<int32_t>()}
                            : csr_view(ctx->row_off.as<int64_t>(), ctx->cols.as<int32_t>());
    // worklist capacity: a list-fed filter (pairs a finished fit left open)
    // holds more cross pairs than the graph-fed one after its hook pass;
    // overflow falls back to the full lazy pass (measured on the 1M-point
    // sweep: nnz/4 for lists, nnz/16 for the graph).  Rows in their slots:
    // the pair count is not read back yet; a quarter of the slot total (the
    // stencil candidates, about five per pair) stands in for it.
    const int64_t pairs = slots ? ctx->slot_total / 4 : ctx->nnz;
    int64_t wl_cap = std::max<int64_t>(int64_t(1) << 20, pairs / (edge_list ? 4 : 16));
    int2 *wl = nullptr;
    if (wl_buf && wl_buf_cap > 0) {  // the caller's room: every pair the filter can emit
        wl = wl_buf;
        wl_cap = wl_buf_cap;
    } else {
        CNN_TRY(ctx->ensure(ctx->io_c, sizeof(int2) * (size_t)wl_cap));
        wl = ctx->io_c.as<int2>();
    }
    unsigned long long *wl_count = counters + 8;
    // hook: every node checks its first kHookEdges candidate edges; compress;
    // then the cross-root pairs only, where pairs inside joined sets cost one
    // load -- with the kernels of the rows' form
    auto check_stage = [&](auto slot_rows) -> cnn_status {
        constexpr bool kS = decltype(slot_rows)::value;
        const unsigned check_blocks = resident((const void *)check_union_kernel<kS>, kCheckWarps * 32, 0);
        check_union_kernel<kS><<<check_blocks, kCheckWarps * 32, 0, st>>>(
            n, g.start, g.end, g.cols, parent, (int32_t)similarity_cutoff, kHookEdges, counters, seed_a, seed_b,
            split);
        CNN_LAUNCH_CHECK(ctx);
        root_store_kernel<<<blocks_for(ctx, n), 256, 0, st>>>(n, node, parent);
        CNN_LAUNCH_CHECK(ctx);
        // cross edges between the hooked sets -> worklist -> checks
        CNN_CUDA(ctx, cudaMemsetAsync(wl_count, 0, sizeof(unsigned long long), st));
        if (edge_list) {
            // only pairs a finished fit that refines this one left open can cross
            cross_filter_list_kernel<<<ctx->sm_count * 16u, 256, 0, st>>>(edge_list, edge_count, parent, wl,
                                                                 wl_count, wl_cap);
        } else {
            cross_filter_kernel<kS><<<resident((const void *)cross_filter_kernel<kS>, 256, 0), 256, 0, st>>>(
                n, g.start, g.end, g.cols, parent, wl, wl_count, wl_cap, split);
        }
        CNN_LAUNCH_CHECK(ctx);
        edge_check_kernel<kS><<<resident((const void *)edge_check_kernel<kS>, kCheckWarps * 32, 0),
                                kCheckWarps * 32, 0, st>>>(wl, wl_count, wl_cap, g.start, g.end, g.cols, parent,
                                                           (int32_t)similarity_cutoff, counters);
        CNN_LAUNCH_CHECK(ctx);
        check_union_if_overflow_kernel<kS><<<check_blocks, kCheckWarps * 32, 0, st>>>(
            n, g.start, g.end, g.cols, parent, (int32_t)similarity_cutoff, wl_count, wl_cap, counters);
        CNN_LAUNCH_CHECK(ctx);
        return CNN_OK;
    };
    CNN_TRY(slots ? check_stage(std::true_type{}) : check_stage(std::false_type{}));
    stage_end(ctx, 6);

    stage_begin(ctx, 7);
    // flag[0..n] for the cluster ranks, then (fresh labels) comp_size[0..n):
    // the component sizes, which become the label counts sort_by_size reads
    // (in flag, once the ranks are scanned)
    int32_t *flag = ctx->flag.as<int32_t>();
    int64_t *rank = ctx->scratch_a.as<int64_t>();
    const bool count = current_start == 1;
    int32_t *comp_size = count ? flag + (n + 1) : nullptr;
    CNN_CUDA(ctx, cudaMemsetAsync(flag, 0, sizeof(int32_t) * (size_t)(count ? 2 * n + 1 : n + 1), st));
    root_min_kernel<<<blocks_for(ctx, n), 256, 0, st>>>(n, node, parent, perm, comp_min, comp_size);
    CNN_LAUNCH_CHECK(ctx);
    root_store_kernel<<<blocks_for(ctx, n), 256, 0, st>>>(n, node, parent);
    CNN_LAUNCH_CHECK(ctx);
    min_flag_kernel<<<blocks_for(ctx, n), 256, 0, st>>>(n, node, parent, comp_min, flag);
    CNN_LAUNCH_CHECK(ctx);
    CNN_TRY(scan_exclusive_i32_to_i64(ctx, flag, rank, n + 1));
    label_kernel<<<blocks_for(ctx, n), 256, 0, st>>>(n, node, parent, comp_min, perm, rank, current_start, labels_dev,
                                                     comp_size, count ? flag : nullptr);
    CNN_LAUNCH_CHECK(ctx);
    ctx->counted_labels = count ? labels_dev : nullptr;
    // every point with consider == 1 is visited by the reference loop and
    // left at consider == 0; points already at 0 stay 0
    CNN_CUDA(ctx, cudaMemsetAsync(consider_dev, 0, (size_t)n, st));
    stage_end(ctx, 7);

    if (ctx->host_stats) {  // read by cnn_get_stats
        CNN_CUDA(ctx, cudaMemcpyAsync(ctx->host_stats + 4, counters + 4, 3 * sizeof(unsigned long long),
                                      cudaMemcpyDeviceToHost, st));
        CNN_CUDA(ctx, cudaMemcpyAsync(ctx->host_stats + 8, rank + n, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
        ctx->fit_stats_pending = true;
        return CNN_OK;
    }
    unsigned long long hc[4] = {0, 0, 0, 0};
    int64_t k = 0;
    CNN_CUDA(ctx, cudaMemcpyAsync(hc, counters + 4, sizeof(hc), cudaMemcpyDeviceToHost, st));
    CNN_CUDA(ctx, cudaMemcpyAsync(&k, rank + n, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    CNN_CUDA(ctx, cudaStreamSynchronize(st));
    ctx->stats.n_nodes = (int64_t)hc[0];
    ctx->stats.n_checks = (int64_t)hc[1];
    ctx->stats.n_accepted = (int64_t)hc[2];
    ctx->stats.n_clusters = k;
    return CNN_OK;
}

cnn_status sort_by_size_impl(cnn_context *ctx, int64_t *labels, int64_t n, int64_t member_cutoff,
                             int64_t max_clusters) {
    cudaStream_t st = ctx->stream;
    if (n <= 0) return CNN_OK;
    if (n > INT32_MAX) return ctx->fail(CNN_ERR_UNSUPPORTED, "more than 2^31-1 labels");
    stage_begin(ctx, 8);
    CNN_TRY(ctx->ensure(ctx->io_c, 4 * sizeof(long long)));
    long long *range = ctx->io_c.as<long long>();
    init_range_kernel<<<1, 1, 0, st>>>(range);
    CNN_LAUNCH_CHECK(ctx);
    label_range_kernel<<<blocks_for(ctx, n), 256, 0, st>>>(labels, n, range);
    CNN_LAUNCH_CHECK(ctx);
    long long hr[3];
    CNN_CUDA(ctx, cudaMemcpyAsync(hr, range, sizeof(hr), cudaMemcpyDeviceToHost, st));
    CNN_CUDA(ctx, cudaStreamSynchronize(st));
    if (hr[2] == 0) {  // only noise
        stage_end(ctx, 8);
        return CNN_OK;
    }
    const long long lo = hr[0], hi = hr[1];
    if ((double)hi - (double)lo + 1.0 <= (double)kOrderSmall) {
        // few label values: count, order in one block, apply (no further sync)
        const int r = (int)(hi - lo + 1);
        CNN_TRY(ctx->ensure(ctx->scratch_b, sizeof(int32_t) * (size_t)(2 * r) + sizeof(int64_t) * (size_t)r + 64));
        int32_t *cnt = ctx->scratch_b.as<int32_t>();
        int32_t *first = cnt + r;
        int64_t *newlab = reinterpret_cast<int64_t *>((reinterpret_cast<uintptr_t>(first + r) + 15) & ~uintptr_t(15));
        init_count_first_kernel<<<blocks_for(ctx, r), 256, 0, st>>>(cnt, first, r);
        CNN_LAUNCH_CHECK(ctx);
        count_first_dense_kernel<<<blocks_for(ctx, n), 256, 0, st>>>(labels, n, lo, cnt, first);
        CNN_LAUNCH_CHECK(ctx);
        const size_t keys_smem = sizeof(uint64_t) * (size_t)r;
        CNN_TRY(allow_dynamic_smem(ctx, (const void *)order_small_kernel, keys_smem));
        // values per block: at least one per warp, about two blocks per SM
        const int per_sm2 = (int)((r + 2 * ctx->sm_count - 1) / (2 * ctx->sm_count));
        const int per_block = std::max(kOrderThreads / 32, (per_sm2 + 31) / 32 * 32);
        order_small_kernel<<<(unsigned)((r + per_block - 1) / per_block), kOrderThreads, keys_smem, st>>>(
            cnt, first, r, per_block, n, bits_for_fit(n), member_cutoff, max_clusters, newlab);
        CNN_LAUNCH_CHECK(ctx);
        apply_dense_kernel<<<blocks_for(ctx, n), 256, 0, st>>>(labels, n, lo, newlab);
        CNN_LAUNCH_CHECK(ctx);
        stage_end(ctx, 8);
        return CNN_OK;
    }
    CNN_TRY(ctx->ensure(ctx->io_a, sizeof(int32_t) * (size_t)n));
    int32_t *ids = ctx->io_a.as<int32_t>();
    // dense id space when the label values are compact enough
    const double span = (double)hi - (double)lo + 1.0;
    int64_t r;
    if (span <= 4.0 * (double)n + 1024.0) {
        r = (int64_t)(hi - lo + 1);
        dense_id_kernel<<<blocks_for(ctx, n), 256, 0, st>>>(labels, n, lo, ids);
        CNN_LAUNCH_CHECK(ctx);
    } else {
        CNN_TRY(ctx->ensure(ctx->io_b, sizeof(uint64_t) * (size_t)n * 2 + 64));
        uint64_t *keys = ctx->io_b.as<uint64_t>();
        uint64_t *uniq = keys + n;
        CNN_TRY(ctx->ensure(ctx->flag, sizeof(int32_t) * (size_t)(n + 1)));
        CNN_TRY(ctx->ensure(ctx->scratch_a, sizeof(int64_t) * (size_t)(n + 1)));
        label_keys_kernel<<<blocks_for(ctx, n), 256, 0, st>>>(labels, n, keys);
        CNN_LAUNCH_CHECK(ctx);
        CNN_TRY(radix_sort_u64(ctx, keys, n, 64));
        int32_t *flag = ctx->flag.as<int32_t>();
        int64_t *pos = ctx->scratch_a.as<int64_t>();
        unique_flag_kernel<<<blocks_for(ctx, n), 256, 0, st>>>(keys, n, flag);
        CNN_LAUNCH_CHECK(ctx);
        CNN_CUDA(ctx, cudaMemsetAsync(flag + n, 0, sizeof(int32_t), st));
        CNN_TRY(scan_exclusive_i32_to_i64(ctx, flag, pos, n + 1));
        unique_compact_kernel<<<blocks_for(ctx, n), 256, 0, st>>>(keys, flag, pos, n, uniq);
        CNN_LAUNCH_CHECK(ctx);
        int64_t nu = 0;
        CNN_CUDA(ctx, cudaMemcpyAsync(&nu, pos + n, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
        CNN_CUDA(ctx, cudaStreamSynchronize(st));
        sparse_id_kernel<<<blocks_for(ctx, n), 256, 0, st>>>(labels, n, uniq, nu, ids);
        CNN_LAUNCH_CHECK(ctx);
        r = nu;
    }
    // per id: size and first occurrence
    CNN_TRY(ctx->ensure(ctx->scratch_b, sizeof(int32_t) * (size_t)(2 * r + 2)));
    int32_t *cnt = ctx->scratch_b.as<int32_t>();
    int32_t *first = cnt + r;
    CNN_CUDA(ctx, cudaMemsetAsync(cnt, 0, sizeof(int32_t) * (size_t)r, st));
    CNN_TRY(fill_i32(ctx, first, r, INT32_MAX));
    count_first_kernel<<<blocks_for(ctx, n), 256, 0, st>>>(ids, n, cnt, first);
    CNN_LAUNCH_CHECK(ctx);
    CNN_TRY(ctx->ensure(ctx->scratch_d, sizeof(int32_t) * (size_t)(r + 1) + sizeof(int64_t) * (size_t)(r + 1) + 64));
    int32_t *cflag = ctx->scratch_d.as<int32_t>();
    int64_t *cpos = reinterpret_cast<int64_t *>((reinterpret_cast<uintptr_t>(cflag + r + 1) + 15) & ~uintptr_t(15));
    cluster_flag_kernel<<<blocks_for(ctx, r + 1), 256, 0, st>>>(cnt, r, cflag);
    CNN_LAUNCH_CHECK(ctx);
    CNN_TRY(scan_exclusive_i32_to_i64(ctx, cflag, cpos, r + 1));
    int64_t k = 0;
    CNN_CUDA(ctx, cudaMemcpyAsync(&k, cpos + r, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    CNN_CUDA(ctx, cudaStreamSynchronize(st));
    const int bits_n = bits_for_fit(n);
    CNN_TRY(ctx->ensure(ctx->io_b, sizeof(uint64_t) * (size_t)(k + 1) + sizeof(int64_t) * (size_t)(r + 1) + 64));
    uint64_t *ckeys = ctx->io_b.as<uint64_t>();
    int64_t *newlab = reinterpret_cast<int64_t *>(ckeys + k + 1);
    cluster_key_kernel<<<blocks_for(ctx, r), 256, 0, st>>>(cnt, first, cpos, r, n, bits_n, ckeys);
    CNN_LAUNCH_CHECK(ctx);
    CNN_TRY(radix_sort_u64(ctx, ckeys, k, bits_n + bits_for_fit(n + 1)));
    const int64_t maxc = max_clusters < 0 ? k : max_clusters;
    new_label_kernel<<<blocks_for(ctx, k), 256, 0, st>>>(ckeys, k, n, bits_n, ids, member_cutoff, maxc, newlab);
    CNN_LAUNCH_CHECK(ctx);
    apply_label_kernel<<<blocks_for(ctx, n), 256, 0, st>>>(labels, ids, n, newlab);
    CNN_LAUNCH_CHECK(ctx);
    stage_end(ctx, 8);
    return CNN_OK;
}

// sort_by_size_impl for the labels of a fit from fresh labels that has just
// run on this context (its rank total, the cluster count, is still in
// scratch_a[n]): the same result, and the same work enqueued whatever the
// labels hold, so that a sequence of fits can be captured as a CUDA graph.
cnn_status sort_fresh_impl(cnn_context *ctx, int64_t *labels, int64_t n, int64_t member_cutoff,
                           int64_t max_clusters, bool device_count) {
    cudaStream_t st = ctx->stream;
    if (n <= 0) return CNN_OK;
    if (n > INT32_MAX) return ctx->fail(CNN_ERR_UNSUPPORTED, "more than 2^31-1 labels");
    stage_begin(ctx, 8);
    const int64_t *k_dev = ctx->scratch_a.as<int64_t>() + n;
    const int bits_n = bits_for_fit(n);
    CNN_TRY(ctx->ensure(ctx->flag, sizeof(int32_t) * (size_t)(n + 1)));
    CNN_TRY(ctx->ensure(ctx->io_b, sizeof(uint64_t) * (size_t)(n + 1) + 64));
    CNN_TRY(ctx->ensure(ctx->scratch_b, sizeof(int64_t) * (size_t)n + 64));
    int32_t *cnt = ctx->flag.as<int32_t>();
    uint64_t *keys = ctx->io_b.as<uint64_t>();
    // the fit that wrote these labels left their counts in cnt (its label stage)
    const bool counted = ctx->counted_labels == labels;
    ctx->counted_labels = nullptr;
    int64_t *k_big = reinterpret_cast<int64_t *>(keys + n);  // k when above kOrderSmall, else 0
    int64_t *newlab = ctx->scratch_b.as<int64_t>();
    // outside a graph capture one read of the cluster count picks the path
    // and sizes its launches (no idle launches of the other path)
    int64_t k_host = -1;
    if (!device_count) {
        CNN_TRY(read_back(ctx, &k_host, k_dev, sizeof(int64_t)));
        if (k_host <= 0) {
            stage_end(ctx, 8);
            return CNN_OK;  // only noise
        }
    }
    if (!counted) {
        CNN_CUDA(ctx, cudaMemsetAsync(cnt, 0, sizeof(int32_t) * (size_t)(k_host >= 0 ? k_host : n), st));
        fresh_count_kernel<<<std::min<unsigned>(blocks_for(ctx, n), 2 * ctx->sm_count), 256, 0, st>>>(labels, n,
                                                                                                k_dev, cnt);
        CNN_LAUNCH_CHECK(ctx);
    }
    if (k_host >= 0 && k_host <= kOrderSmall) {
        const size_t smem = sizeof(uint64_t) * (size_t)k_host;
        CNN_TRY(allow_dynamic_smem(ctx, (const void *)fresh_order_small_kernel, smem));
        const unsigned blocks = (unsigned)std::min<int64_t>(2 * (int64_t)ctx->sm_count, (k_host + 31) / 32);
        fresh_order_small_kernel<<<blocks, kOrderThreads, smem, st>>>(cnt, k_dev, n, bits_n, member_cutoff,
                                                                      max_clusters, newlab, k_big);
        CNN_LAUNCH_CHECK(ctx);
        apply_dense_kernel<<<blocks_for(ctx, n), 256, 0, st>>>(labels, n, 1, newlab);
        CNN_LAUNCH_CHECK(ctx);
        stage_end(ctx, 8);
        return CNN_OK;
    }
    if (k_host > kOrderSmall) {  // the radix path with the count known here
        CNN_CUDA(ctx, cudaMemcpyAsync(k_big, k_dev, sizeof(int64_t), cudaMemcpyDeviceToDevice, st));
        fresh_keys_kernel<<<blocks_for(ctx, k_host), 256, 0, st>>>(cnt, k_big, n, bits_n, keys);
        CNN_LAUNCH_CHECK(ctx);
        uint64_t *sorted = keys;
        CNN_TRY(radix_sort_u64(ctx, keys, k_host, bits_n + bits_for_fit(n + 1), bits_n, &sorted));
        fresh_new_label_kernel<<<blocks_for(ctx, k_host), 256, 0, st>>>(sorted, k_big, n, bits_n, member_cutoff,
                                                                       max_clusters, newlab);
        CNN_LAUNCH_CHECK(ctx);
        apply_dense_kernel<<<blocks_for(ctx, n), 256, 0, st>>>(labels, n, 1, newlab);
        CNN_LAUNCH_CHECK(ctx);
        stage_end(ctx, 8);
        return CNN_OK;
    }
    // device count (a graph capture): at most kOrderSmall labels ranked in
    // shared memory, more by a radix sort -- both enqueued, each does
    // nothing when the other applies
    const size_t keys_smem = sizeof(uint64_t) * (size_t)std::min<int64_t>(n, kOrderSmall);
    CNN_TRY(allow_dynamic_smem(ctx, (const void *)fresh_order_small_kernel, keys_smem));
    fresh_order_small_kernel<<<2 * ctx->sm_count, kOrderThreads, keys_smem, st>>>(
        cnt, k_dev, n, bits_n, member_cutoff, max_clusters, newlab, k_big);
    CNN_LAUNCH_CHECK(ctx);
    fresh_keys_kernel<<<blocks_for(ctx, n), 256, 0, st>>>(cnt, k_big, n, bits_n, keys);
    CNN_LAUNCH_CHECK(ctx);
    uint64_t *sorted = keys;
    CNN_TRY(radix_sort_u64(ctx, keys, n, bits_n + bits_for_fit(n + 1), bits_n, &sorted, k_big));
    fresh_new_label_kernel<<<blocks_for(ctx, n), 256, 0, st>>>(sorted, k_big, n, bits_n, member_cutoff, max_clusters,
                                                              newlab);
    CNN_LAUNCH_CHECK(ctx);
    apply_dense_kernel<<<blocks_for(ctx, n), 256, 0, st>>>(labels, n, 1, newlab);
    CNN_LAUNCH_CHECK(ctx);
    stage_end(ctx, 8);
    return CNN_OK;
}

// What Clustering.fit does around the fitter for fresh labels
// (src/cnnclustering/cluster.pyx:316-364): labels 0, consider 1,
// current_start 1, the fit, then sort_by_size.
cnn_status fit_and_sort_into(cnn_context *ctx, int64_t similarity_cutoff, int64_t n_member_cutoff,
                             int64_t sort_member_cutoff, int64_t max_clusters, int64_t *labels_dev,
                             const int32_t *seed_a, const int32_t *seed_b, bool sort, const int2 *edge_list,
                             const unsigned long long *edge_count, int2 *wl_buf, int64_t wl_buf_cap) {
    const int64_t n = ctx->n;
    cudaStream_t st = ctx->stream;
    if (n == 0) return CNN_OK;
    CNN_TRY(ctx->ensure(ctx->sweep_consider, (size_t)n));
    CNN_CUDA(ctx, cudaMemsetAsync(labels_dev, 0, sizeof(int64_t) * (size_t)n, st));
    CNN_CUDA(ctx, cudaMemsetAsync(ctx->sweep_consider.ptr, 1, (size_t)n, st));
    CNN_TRY(fit_impl(ctx, similarity_cutoff, n_member_cutoff, 1, ctx->sweep_consider.as<uint8_t>(), labels_dev,
                     seed_a, seed_b, edge_list, edge_count, wl_buf, wl_buf_cap));
    return sort ? sort_fresh_impl(ctx, labels_dev, n, sort_member_cutoff, max_clusters, true) : CNN_OK;
}

// The pairs the last fit left open, from the graph (in_list null) or from
// the list that fit used; out_count is a device counter.
cnn_status open_pairs_impl(cnn_context *ctx, const int2 *in_list, const unsigned long long *in_count, int2 *out,
                           unsigned long long *out_count, int64_t cap) {
    CNN_TRY(ensure_lists(ctx));
    cudaStream_t st = ctx->stream;
    const int64_t n = ctx->n;
    CNN_CUDA(ctx, cudaMemsetAsync(out_count, 0, sizeof(unsigned long long), st));
    if (n == 0) return CNN_OK;
    if (in_list) {
        open_pairs_list_kernel<<<ctx->sm_count * 16u, 256, 0, st>>>(in_list, in_count, ctx->node.as<uint8_t>(),
                                                            ctx->parent.as<int32_t>(), out, out_count, cap);
    } else {
        open_pairs_csr_kernel<<<std::min<unsigned>(grid_for(n * 32, 256), ctx->sm_count * 16u), 256, 0, st>>>(
            n, ctx->row_off.as<int64_t>(), ctx->cols.as<int32_t>(), ctx->node.as<uint8_t>(),
            ctx->parent.as<int32_t>(), out, out_count, cap);
    }
    CNN_LAUNCH_CHECK(ctx);
    return CNN_OK;
}

cnn_status check_lists_impl(cnn_context *ctx, const int32_t *a, int64_t na, const int32_t *b, int64_t nb,
                            int64_t c, int32_t *result_dev) {
    if (na > INT32_MAX || nb > INT32_MAX) return ctx->fail(CNN_ERR_UNSUPPORTED, "list longer than 2^31-1");
    check_lists_kernel<<<1, 32, 0, ctx->stream>>>(a, na, b, nb, c, result_dev);
    CNN_LAUNCH_CHECK(ctx);
    return CNN_OK;
}

}  // namespace cnn
