// fit_kernels.cuh -- device code of the fit (union-find, similarity check,
// node flags, labelling), shared by fit.cu and noalloc.cu.  See fit.cu for
// the algorithm and its relation to the reference's FitterExtBFS.
#pragma once

#include <climits>

#include "common.cuh"

namespace cnn {
namespace {

constexpr int kCheckWarps = 8;

// The neighbour rows a fit walks: row a is cols[start[a] .. end[a]).  CSR:
// start = offsets, end = offsets + 1; rows left in the slots the cell-grid
// search wrote them to: their starts and ends.  The kernels take the three
// pointers as separate __restrict__ parameters (a struct parameter costs
// the hook pass registers) and a kSlotRows flag: false reads a row's end as
// the next row's start.
struct RowView {
    const int64_t *start;
    const int64_t *end;
    const int32_t *cols;
};

inline RowView csr_view(const int64_t *off, const int32_t *cols) { return RowView{off, off + 1, cols}; }

// candidate edges each node checks in the hook pass
#ifndef CNN_HOOK_EDGES
#define CNN_HOOK_EDGES 3
#endif
constexpr int32_t kHookEdges = CNN_HOOK_EDGES;

__device__ __forceinline__ int32_t uf_find(int32_t *parent, int32_t x) {
    int32_t cur = x;
    int32_t next = *(volatile int32_t *)&parent[cur];
    while (next != cur) {
        int32_t nn = *(volatile int32_t *)&parent[next];
        if (nn != next) *(volatile int32_t *)&parent[cur] = nn;  // path halving
        cur = next;
        next = nn;
    }
    return cur;
}

// Join the sets of a and b; the smaller root index becomes the root.
// Lock-free: a failed CAS means another thread changed that root first.
__device__ __forceinline__ void uf_unite(int32_t *parent, int32_t a, int32_t b) {
    for (;;) {
        a = uf_find(parent, a);
        b = uf_find(parent, b);
        if (a == b) return;
        if (a > b) { int32_t t = a; a = b; b = t; }
        if (atomicCAS(&parent[b], b, a) == b) return;
    }
}

// Warp-cooperative merge-path count: does |A & B| reach `needed` (> 0)?
// A and B ascending, duplicate-free, values < 2^31 - 2.  Each step loads
// one 32-wide chunk of each list (coalesced), every lane finds its B value
// among the 32 A values with a 5-step shuffle binary search, and the chunk
// with the smaller maximum is consumed (no pair can match across it).
// Stops at `needed` matches, or when the rest cannot reach it.
__device__ __forceinline__ bool warp_shares_at_least(const int32_t *__restrict__ A, int32_t la,
                                                     const int32_t *__restrict__ B, int32_t lb, int32_t needed,
                                                     int lane) {
    if (la < needed || lb < needed) return false;
    int32_t ia = 0, ib = 0, count = 0;
    while (ia < la && ib < lb) {
        const int32_t va = ia + lane < la ? __ldg(A + ia + lane) : INT_MAX;      // padding never matches:
        const int32_t vb = ib + lane < lb ? __ldg(B + ib + lane) : INT_MAX - 1;  // A pads differ from B pads
        int pos = 0;
#pragma unroll
        for (int step = 16; step > 0; step >>= 1) {
            const int32_t probe = __shfl_sync(0xffffffffu, va, pos + step - 1);
            if (probe < vb) pos += step;
        }
        const bool found = __shfl_sync(0xffffffffu, va, pos) == vb;
        count += __popc(__ballot_sync(0xffffffffu, found));
        if (count >= needed) return true;
        const int32_t amax = __shfl_sync(0xffffffffu, va, 31);
        const int32_t bmax = __shfl_sync(0xffffffffu, vb, 31);
        if (amax <= bmax) ia += 32;
        if (bmax <= amax) ib += 32;
        const int32_t rest = min(la - ia, lb - ib);
        if (count + (rest > 0 ? rest : 0) < needed) return false;
    }
    return false;
}

// The same count for two long lists, 128 entries of each per step: A's
// chunk goes to the warp's shared-memory slot sA (128 entries), B's stays
// in registers (4 per lane), and each lane looks its 4 values up in A's
// chunk by binary search.  Both chunks load together, so a list pair costs
// a quarter of the dependent round trips of the 32-wide merge -- what a
// rejected pair of long rows (scanned to the end) is bound by.
constexpr int kWideChunk = 128;

__device__ __forceinline__ bool warp_shares_at_least_wide(const int32_t *__restrict__ A, int32_t la,
                                                          const int32_t *__restrict__ B, int32_t lb, int32_t needed,
                                                          int lane, int32_t *sA) {
    if (la < needed || lb < needed) return false;
    int32_t ia = 0, ib = 0, count = 0;
    while (ia < la && ib < lb) {
        int32_t av[4], bv[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int32_t i = ia + j * 32 + lane, k = ib + j * 32 + lane;
            av[j] = i < la ? __ldg(A + i) : INT_MAX;      // padding never matches:
            bv[j] = k < lb ? __ldg(B + k) : INT_MAX - 1;  // A pads differ from B pads
        }
        __syncwarp();  // the previous step's lookups are done
#pragma unroll
        for (int j = 0; j < 4; ++j) sA[j * 32 + lane] = av[j];
        __syncwarp();
        const int32_t amax = sA[kWideChunk - 1];
        const int32_t bmax = __shfl_sync(0xffffffffu, bv[3], 31);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            int pos = 0;  // entries of the chunk below bv[j]
#pragma unroll
            for (int step = kWideChunk / 2; step > 0; step >>= 1)
                if (sA[pos + step - 1] < bv[j]) pos += step;
            const bool found = pos < kWideChunk && sA[pos] == bv[j];
            count += __popc(__ballot_sync(0xffffffffu, found));
        }
        if (count >= needed) return true;
        if (amax <= bmax) ia += kWideChunk;
        if (bmax <= amax) ib += kWideChunk;
        const int32_t rest = min(la - ia, lb - ib);
        if (count + (rest > 0 ? rest : 0) < needed) return false;
    }
    return false;
}

// Either merge, by the lengths: the wide one as soon as one list is at least
// kWideMin long (a short row against a long one is walked 128 at a time).
#ifndef CNN_WIDE_MIN
#define CNN_WIDE_MIN 128
#endif
constexpr int kWideMin = CNN_WIDE_MIN;

__device__ __forceinline__ bool warp_shares(const int32_t *__restrict__ A, int32_t la, const int32_t *__restrict__ B,
                                            int32_t lb, int32_t needed, int lane, int32_t *sA) {
    return (la >= kWideMin || lb >= kWideMin) ? warp_shares_at_least_wide(A, la, B, lb, needed, lane, sA)
                                              : warp_shares_at_least(A, la, B, lb, needed, lane);
}

// Persistent check kernels: nodes are dealt to warps in contiguous chunks
// (CNN_CHECK_CHUNKED=0 strides them), so that warps working at the same time
// sit in different regions of the (cell-ordered) graph and rarely race on
// one root, while each warp's own nodes share roots it has just resolved.
// Seeded fits stride: their open nodes are few and clustered.
#ifndef CNN_CHECK_CHUNKED
#define CNN_CHECK_CHUNKED 1
#endif
// minimum resident blocks per SM asked of the compiler for the check kernels
// (latency-bound: more resident warps keep more union-find chains in flight)
#ifndef CNN_CHECK_MIN_BLOCKS
#define CNN_CHECK_MIN_BLOCKS 7
#endif

__global__ void node_kernel(const int32_t *__restrict__ deg, const int32_t *__restrict__ perm,
                            const uint8_t *__restrict__ consider, int64_t n, int64_t n_member_cutoff,
                            uint8_t *__restrict__ node, int32_t *__restrict__ parent,
                            int32_t *__restrict__ comp_min, unsigned long long *__restrict__ counters) {
    unsigned long long local = 0;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
        const bool is_node = (int64_t)deg[p] > n_member_cutoff && consider[perm[p]] != 0;
        node[p] = is_node ? 1 : 0;
        parent[p] = is_node ? (int32_t)p : -1;  // -1: not a node (never joined)
        comp_min[p] = INT_MAX;
        local += is_node;
    }
    for (int o = 16; o > 0; o >>= 1) local += __shfl_down_sync(0xffffffffu, local, o);
    if ((threadIdx.x & 31) == 0 && local) atomicAdd(&counters[4], local);
}

// Index of the first entry > v in the ascending run cols[s, e), found by the
// whole warp with 32-way probing (every lane returns the same value).
// Invariant: entries before lo are <= v, entries from hi on are > v.
__device__ __forceinline__ int64_t warp_upper_bound(const int32_t *__restrict__ cols, int64_t s, int64_t e, int32_t v,
                                                    int lane) {
    int64_t lo = s, hi = e;
    while (hi - lo > 32) {
        const int64_t step = (hi - lo + 31) / 32;
        const int64_t p = lo + (int64_t)lane * step;
        const int c = __popc(__ballot_sync(0xffffffffu, p < hi && cols[p] <= v));  // a prefix of the probes
        if (c == 0) return lo;
        const int64_t nlo = lo + (int64_t)(c - 1) * step + 1;
        hi = min(hi, lo + (int64_t)c * step);
        lo = nlo;
    }
    const int64_t p = lo + lane;
    return lo + __popc(__ballot_sync(0xffffffffu, p < hi && cols[p] <= v));
}

// Persistent warps over nodes.  For node a, candidate edges (a, b) with
// b > a and b a node (parent[b] >= 0) are taken 32 at a time; their roots
// are resolved in parallel (one lane each) and re-resolved only after this
// warp joined something: a stale "different" only costs an extra check,
// never a wrong skip.  max_edges bounds the candidate edges one node
// examines (the hook pass uses 3).  Rows are ascending, so the walk starts
// at the first entry > a: split[a] (the number of entries <= a, when the
// search recorded it) or a warp-wide binary search.  Nodes with
// skip_a[a] >= 0 or skip_b[a] >= 0 (already joined by seeds) are left to
// the cross-edge pass.
template <bool kSlotRows>
__device__ __forceinline__ void check_union_body(
    int64_t n, const int64_t *__restrict__ row_start, const int64_t *__restrict__ row_end,
    const int32_t *__restrict__ cols, int32_t *__restrict__ parent, int32_t needed, int32_t max_edges,
    unsigned long long *__restrict__ counters, const int32_t *__restrict__ skip_a = nullptr,
    const int32_t *__restrict__ skip_b = nullptr, const int32_t *__restrict__ split = nullptr) {
    __shared__ int32_t s_wide[kCheckWarps][kWideChunk];
    int32_t *sA = s_wide[(threadIdx.x >> 5) % kCheckWarps];
    const int lane = threadIdx.x & 31;
    const int64_t warp0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    unsigned long long n_checks = 0, n_acc = 0;
    // contiguous chunks, or a stride when most nodes skip (seeded fits: the
    // few open nodes cluster in space and would load a few warps only)
    const bool chunked = CNN_CHECK_CHUNKED && !skip_a && !skip_b;
    const int64_t per = chunked ? (n + nwarps - 1) / nwarps : 1;
    const int64_t a_begin = chunked ? warp0 * per : warp0;
    const int64_t a_end = chunked ? min(n, (warp0 + 1) * per) : n;
    const int64_t a_step = chunked ? 1 : nwarps;
    for (int64_t a64 = a_begin; a64 < a_end; a64 += a_step) {
        const int32_t a = (int32_t)a64;
        // parent[a], the row bounds and split[a] in one round trip (lanes 0..3)
        int64_t v = 0;
        if (lane == 0) v = *(volatile int32_t *)&parent[a];
        else if (lane < 3) v = (kSlotRows && lane == 2) ? row_end[a] : row_start[a + (kSlotRows ? 0 : lane - 1)];
        else if (lane == 3 && split) v = split[a];
        const int32_t pa = (int32_t)__shfl_sync(0xffffffffu, v, 0);
        if (pa < 0) continue;  // not a node
        if ((skip_a && skip_a[a] >= 0) || (skip_b && skip_b[a] >= 0)) continue;
        const int64_t s = __shfl_sync(0xffffffffu, v, 1), e = __shfl_sync(0xffffffffu, v, 2);
        const int64_t split_a = __shfl_sync(0xffffffffu, v, 3);
        const int32_t la = (int32_t)(e - s);
        const int32_t *A = cols + s;
        // ra (and rx once set) are roots observed to hold a: equal roots mean
        // one set, since sets only merge; a stale "different" costs a check
        int32_t ra = -1, rx = -1;
        bool dirty = true;
        int32_t seen = 0;
        for (int64_t k0 = split ? s + split_a : warp_upper_bound(cols, s, e, a, lane); k0 < e && seen < max_edges;
             k0 += 32) {
            const int64_t k = k0 + lane;
            int32_t b = -1, pb = -1;
            if (k < e) {
                b = cols[k];
                if (b > a) pb = *(volatile int32_t *)&parent[b];
            }
            bool cand = pb >= 0;
            unsigned cmask = __ballot_sync(0xffffffffu, cand);
            if (!cmask) continue;
            if (seen + __popc(cmask) > max_edges) {  // keep only the first edges
                const int keep = max_edges - seen;
                unsigned m = cmask, kept = 0;
                for (int i = 0; i < keep; ++i) { kept |= m & (0u - m); m &= m - 1; }
                cmask = kept;
                cand = (cmask >> lane) & 1u;
            }
            seen += __popc(cmask);
            if (dirty) {
                ra = (ra < 0 && pa == a) ? a : uf_find(parent, ra < 0 ? pa : a);  // parent pointers only rise
                rx = -1;
                dirty = false;
            }
            int32_t rb = cand ? uf_find(parent, pb) : -1;
            unsigned mask = __ballot_sync(0xffffffffu, cand && rb != ra && rb != rx);
            while (mask) {
                if (dirty) {
                    ra = uf_find(parent, a);
                    rx = -1;
                    const bool live = (mask >> lane) & 1u;
                    if (live) rb = uf_find(parent, rb);
                    mask = __ballot_sync(0xffffffffu, live && rb != ra);
                    dirty = false;
                    if (!mask) break;
                }
                const int src = __ffs(mask) - 1;
                mask &= mask - 1;
                const int32_t bb = __shfl_sync(0xffffffffu, b, src);
                bool ok;
                if (needed <= 0) {
                    ok = needed == 0;
                } else {
                    const int64_t bs = row_start[bb];
                    const int32_t lb = (int32_t)((kSlotRows ? row_end[bb] : row_start[bb + 1]) - bs);
                    ok = warp_shares(A, la, cols + bs, lb, needed, lane, sA);
                    ++n_checks;
                }
                if (ok) {
                    // link the two observed roots directly (larger under
                    // smaller, as uf_unite does); if the larger one is no
                    // longer a root, take the general path and re-resolve
                    const int32_t rbb = __shfl_sync(0xffffffffu, rb, src);
                    const int32_t lo = min(ra, rbb), hi = max(ra, rbb);
                    int direct = 0;
                    if (lane == 0) {
                        direct = atomicCAS(&parent[hi], hi, lo) == hi;
                        if (!direct) uf_unite(parent, a, bb);
                    }
                    direct = __shfl_sync(0xffffffffu, direct, 0);
                    ++n_acc;
                    if (direct) {
                        ra = lo;
                        rx = hi;
                        mask = __ballot_sync(0xffffffffu, ((mask >> lane) & 1u) && rb != ra && rb != rx);
                    } else {
                        dirty = true;
                    }
                }
            }
        }
    }
    if (lane == 0 && n_checks) atomicAdd(&counters[5], n_checks);
    if (lane == 0 && n_acc) atomicAdd(&counters[6], n_acc);
}

template <bool kSlotRows>
__global__ void __launch_bounds__(kCheckWarps * 32, CNN_CHECK_MIN_BLOCKS) check_union_kernel(
    int64_t n, const int64_t *__restrict__ row_start, const int64_t *__restrict__ row_end,
    const int32_t *__restrict__ cols, int32_t *__restrict__ parent, int32_t needed, int32_t max_edges,
    unsigned long long *__restrict__ counters, const int32_t *__restrict__ skip_a,
    const int32_t *__restrict__ skip_b, const int32_t *__restrict__ split = nullptr) {
    check_union_body<kSlotRows>(n, row_start, row_end, cols, parent, needed, max_edges, counters, skip_a, skip_b,
                                split);
}

// Full path compression and per-component minimum point index.
// Neighbouring internal indices mostly share a root: lanes with the same
// root combine their minimum first and issue one atomic.
// comp_size (optional): the nodes of each component, counted the same way.
__global__ void root_min_kernel(int64_t n, const uint8_t *__restrict__ node, int32_t *__restrict__ parent,
                                const int32_t *__restrict__ perm, int32_t *__restrict__ comp_min,
                                int32_t *__restrict__ comp_size = nullptr) {
    const int lane = threadIdx.x & 31;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < n; base += stride) {
        const int64_t p = base + lane;
        const bool is_node = p < n && node[p];
        const int32_t r = is_node ? uf_find(parent, (int32_t)p) : -1;
        int32_t v = is_node ? perm[p] : INT_MAX;
        const unsigned peers = __match_any_sync(0xffffffffu, r);
        v = __reduce_min_sync(peers, v);
        if (is_node && lane == __ffs(peers) - 1) {
            atomicMin(&comp_min[r], v);
            if (comp_size) atomicAdd(&comp_size[r], __popc(peers));
        }
    }
}

// Every node's parent becomes its root.  The walk writes nothing: with
// path halving, another thread could store a not-yet-root ancestor into a
// slot after its owner stored the root; here each slot is written once, by
// its owner, with the root (no unions run at this point).
__global__ void root_store_kernel(int64_t n, const uint8_t *__restrict__ node, int32_t *__restrict__ parent) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
        if (!node[p]) continue;
        int32_t r = (int32_t)p, next = *(volatile int32_t *)&parent[r];
        while (next != r) {
            r = next;
            next = *(volatile int32_t *)&parent[r];
        }
        parent[p] = r;
    }
}

__global__ void min_flag_kernel(int64_t n, const uint8_t *__restrict__ node, const int32_t *__restrict__ parent,
                                const int32_t *__restrict__ comp_min, int32_t *__restrict__ flag) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
        if (!node[p]) continue;
        if (parent[p] == (int32_t)p) flag[comp_min[p]] = 1;
    }
}

// label_cnt (optional): at each root, the size of its component as the count
// of label current_start + rank (entry rank), what sort_by_size counts.
__global__ void label_kernel(int64_t n, const uint8_t *__restrict__ node, const int32_t *__restrict__ parent,
                             const int32_t *__restrict__ comp_min, const int32_t *__restrict__ perm,
                             const int64_t *__restrict__ rank, int64_t current_start, int64_t *__restrict__ labels,
                             const int32_t *__restrict__ comp_size = nullptr, int32_t *__restrict__ label_cnt = nullptr) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
        if (!node[p]) continue;
        const int32_t r = parent[p];
        const int64_t lab = rank[comp_min[r]];
        labels[perm[p]] = current_start + lab;
        if (label_cnt && r == (int32_t)p) label_cnt[lab] = comp_size[p];
    }
}

}  // namespace
}  // namespace cnn
