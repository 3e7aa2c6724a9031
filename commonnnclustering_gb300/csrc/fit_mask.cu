// fit_mask.cu -- the fit over the cell-grid neighbour graph in mask form.
//
// Graph form.  The cell-grid search (search.cu) tests every point of a cell
// against the same candidate sequence: the 9 runs of consecutive internal
// indices its 3 x 3 x 3 stencil covers, concatenated in ascending order.
// The mask form stores, per point, one bit per candidate (set = neighbour):
// ceil(T_c / 32) words for a cell with T_c candidates, written straight
// from the search's per-step ballots.  A row costs T_c / 8 bytes instead of
// 4 bytes per neighbour (200,000 x 3 at mean degree 215: 29 MB instead of
// 172 MB, small enough to stay in L2 through the fit).
//
// The fit is fit.cu's (FitterExtBFS._fit, src/cnnclustering/_fit.pyx:
// 408-491, as connected components of the accepted edges: a lazy lock-free
// union-find with a hook pass, a cross-edge worklist, the full pass as the
// worklist's overflow guard, then the same labelling).  What changes is how
// a row is read:
//   * the entries b > a of a's row are the set bits after a's own bit (the
//     candidate sequence is ascending and a sits in its own run 4), mapped
//     back to internal indices through the cell's run table;
//   * |N(a) & N(b)| (SimilarityCheckerExtScreensorted._check,
//     src/cnnclustering/_types.pyx:2654-2706, without the early exit) is a
//     popcount of AND-ed bit ranges: a's run over grid row (y, z) and b's run
//     over the same grid row are intervals of consecutive internal indices,
//     so their overlap is one interval, at bit offsets off_a and off_b of
//     the two rows; the count is the sum over the (at most 9) grid rows the
//     two stencils share of popc(bits_a[off_a + i] & bits_b[off_b + i]), 32
//     bits at a time (funnel shifts) spread over the warp's lanes.
#include <climits>

#include <algorithm>

#include "common.cuh"
#include "fit_kernels.cuh"

namespace cnn {
namespace {

// resident blocks per SM asked of the compiler for the mask check kernels
// (fewer than the list kernels': their walk keeps more state per thread)
#ifndef CNN_MASK_MIN_BLOCKS
#define CNN_MASK_MIN_BLOCKS 5
#endif

// Run table of one row's candidate sequence, per warp in shared memory.
struct RunTable {
    int32_t rs[9];    // first internal index of each run
    int32_t len[9];   // its length (0: outside the grid, or no points)
    int32_t cum[10];  // exclusive prefix of len; cum[9] = T_c
    int32_t cy, cz;   // the cell's grid row
    int32_t self_t;   // the row owner's own bit
    int32_t words;    // words of the row
    int64_t base;     // word offset of the row
};

// Overlap segments of two rows, per warp in shared memory.
struct SegTable {
    int32_t first[9];  // first chunk of each segment (exclusive prefix of the chunk counts)
    int32_t off_a[9], off_b[9], len[9];
};

// The run table of `point`'s row (the whole warp; the same geometry as the
// search's grid_unit_kernel, so the same candidate order).
__device__ __forceinline__ void load_runs(const MaskGraph &G, int32_t point, RunTable &rt, int lane) {
    const int32_t c = G.pcell[point];
    const int32_t cx = c % G.g0, cy = (c / G.g0) % G.g1, cz = c / (G.g0 * G.g1);
    int32_t rs = 0, len = 0;
    int64_t aux = 0;
    if (lane < 9) {
        const int32_t z = cz + lane / 3 - 1, y = cy + lane % 3 - 1;
        if (z >= 0 && z < G.g2 && y >= 0 && y < G.g1) {
            const int32_t xlo = cx > 0 ? cx - 1 : 0;
            const int32_t xhi = cx + 1 < G.g0 ? cx + 1 : G.g0 - 1;
            const int64_t row = (int64_t)G.g0 * ((int64_t)y + (int64_t)G.g1 * z);
            const int64_t b = G.cell_start[row + xlo], e = G.cell_start[row + xhi + 1];
            rs = (int32_t)b;
            len = e > b ? (int32_t)(e - b) : 0;
        }
    } else if (lane == 9) {
        aux = G.cell_start[c];
    } else if (lane == 10) {
        aux = G.mbase[c];
    }
    int32_t inc = len;
#pragma unroll
    for (int o = 1; o < 16; o <<= 1) {
        const int32_t v = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += v;
    }
    const int64_t cell_first = __shfl_sync(0xffffffffu, aux, 9);
    const int64_t mbase = __shfl_sync(0xffffffffu, aux, 10);
    const int32_t total = __shfl_sync(0xffffffffu, inc, 8);
    const int32_t rs4 = __shfl_sync(0xffffffffu, rs, 4);
    const int32_t cum4 = __shfl_sync(0xffffffffu, inc - len, 4);
    __syncwarp();
    if (lane < 9) {
        rt.rs[lane] = rs;
        rt.len[lane] = len;
        rt.cum[lane] = inc - len;
    }
    if (lane == 0) {
        const int32_t words = (total + 31) >> 5;
        rt.cum[9] = total;
        rt.cy = cy;
        rt.cz = cz;
        rt.words = words;
        rt.base = mbase + ((int64_t)point - cell_first) * (int64_t)words;
        rt.self_t = cum4 + (point - rs4);
    }
    __syncwarp();
}

// internal index of candidate t of a row
__device__ __forceinline__ int32_t cand_index(const RunTable &rt, int32_t t) {
    int r = 0;
#pragma unroll
    for (int k = 1; k < 9; ++k) r += t >= rt.cum[k] ? 1 : 0;
    return rt.rs[r] + (t - rt.cum[r]);
}

// 32 bits of a row starting at bit `bit` (the next word is read too: every
// row is followed by another row or by the padding words)
__device__ __forceinline__ uint32_t bits32_at(const uint32_t *__restrict__ row, int32_t bit) {
    const int32_t i = bit >> 5;
    const uint32_t lo = row[i], hi = row[i + 1];
    return __funnelshift_r(lo, hi, (uint32_t)(bit & 31));
}

// |N(a) & N(b)| for the rows of run tables ra and rb (the whole warp; every
// lane returns the count).
__device__ __forceinline__ int32_t mask_common(const MaskGraph &G, const RunTable &ra, const RunTable &rb,
                                               SegTable &sg, int lane) {
    int32_t seg_len = 0, off_a = 0, off_b = 0;
    if (lane < 9 && ra.len[lane] > 0) {
        const int32_t ya = ra.cy + lane % 3 - 1, za = ra.cz + lane / 3 - 1;
        const int32_t dy = ya - rb.cy, dz = za - rb.cz;
        if (dy >= -1 && dy <= 1 && dz >= -1 && dz <= 1) {
            const int r2 = (dz + 1) * 3 + (dy + 1);
            const int32_t lo = max(ra.rs[lane], rb.rs[r2]);
            const int32_t hi = min(ra.rs[lane] + ra.len[lane], rb.rs[r2] + rb.len[r2]);
            if (hi > lo) {
                seg_len = hi - lo;
                off_a = ra.cum[lane] + (lo - ra.rs[lane]);
                off_b = rb.cum[r2] + (lo - rb.rs[r2]);
            }
        }
    }
    const int32_t chunks = (seg_len + 31) >> 5;
    int32_t inc = chunks;
#pragma unroll
    for (int o = 1; o < 16; o <<= 1) {
        const int32_t v = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += v;
    }
    const int32_t total = __shfl_sync(0xffffffffu, inc, 8);
    __syncwarp();
    if (lane < 9) {
        sg.first[lane] = inc - chunks;
        sg.off_a[lane] = off_a;
        sg.off_b[lane] = off_b;
        sg.len[lane] = seg_len;
    }
    __syncwarp();
    const uint32_t *row_a = G.masks + ra.base, *row_b = G.masks + rb.base;
    int32_t count = 0;
    for (int32_t i = lane; i < total; i += 32) {
        // the segment of chunk i: the last one starting at or before it (the
        // starts do not decrease, and the last such segment is not empty)
        int s = 0;
#pragma unroll
        for (int k = 1; k < 9; ++k) s += i >= sg.first[k] ? 1 : 0;
        const int32_t m = i - sg.first[s];
        const int32_t left = sg.len[s] - 32 * m;
        const uint32_t keep = left >= 32 ? 0xffffffffu : ((1u << left) - 1u);
        const uint32_t wa = bits32_at(row_a, sg.off_a[s] + 32 * m);
        const uint32_t wb = bits32_at(row_b, sg.off_b[s] + 32 * m);
        count += __popc(wa & wb & keep);
    }
    count = __reduce_add_sync(0xffffffffu, count);
    __syncwarp();
    return count;
}

// the similarity decision of fit.cu's checks: needed <= 0 -> needed == 0
__device__ __forceinline__ bool mask_check(const MaskGraph &G, const RunTable &ra, const RunTable &rb, SegTable &sg,
                                           int32_t needed, int lane) {
    if (needed <= 0) return needed == 0;
    return mask_common(G, ra, rb, sg, lane) >= needed;
}

// The k-th (0-based) set bit of w.
__device__ __forceinline__ int32_t nth_set_bit(uint32_t w, int32_t k) {
    int32_t pos = 0;
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) {
        const int32_t c = __popc(w & ((1u << s) - 1u));
        if (k >= c) {
            k -= c;
            w >>= s;
            pos += s;
        }
    }
    return pos;
}

// Walks the set bits of a row at candidate positions >= t_from, 32 at a time
// in ascending order: after next(), lane l holds the l-th of them (valid
// when l < count) as an internal index.
struct BitWalk {
    int32_t w0;       // first word of the current window of 32 words
    uint32_t word;    // this lane's word of the window
    int32_t excl;     // set bits of the window before this lane's word
    int32_t win_tot;  // set bits in the window
    int32_t taken;    // of them already handed out
};

__device__ __forceinline__ void walk_window(const MaskGraph &G, const RunTable &rt, int32_t t_from, BitWalk &bw,
                                            int lane) {
    const int32_t w = bw.w0 + lane;
    uint32_t word = w < rt.words ? G.masks[rt.base + w] : 0u;
    if (w == (t_from >> 5)) word &= 0xffffffffu << (t_from & 31);
    if (w < (t_from >> 5)) word = 0u;
    const int32_t c = __popc(word);
    int32_t inc = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int32_t v = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += v;
    }
    bw.word = word;
    bw.excl = inc - c;
    bw.win_tot = __shfl_sync(0xffffffffu, inc, 31);
    bw.taken = 0;
}

// Next up to 32 set bits; returns how many (0: the row is done).
__device__ __forceinline__ int32_t walk_next(const MaskGraph &G, const RunTable &rt, int32_t t_from, BitWalk &bw,
                                             int lane, int32_t *j_out) {
    while (bw.taken >= bw.win_tot) {
        bw.w0 += 32;
        if (bw.w0 >= rt.words) return 0;
        walk_window(G, rt, t_from, bw, lane);
    }
    const int32_t r = bw.taken + lane;  // rank inside the window
    const int32_t count = min(32, bw.win_tot - bw.taken);
    // the lane whose word holds rank r: the last lane with excl <= r
    int32_t L = 0;
#pragma unroll
    for (int step = 16; step > 0; step >>= 1) {
        const int32_t e = __shfl_sync(0xffffffffu, bw.excl, min(L + step, 31));
        if (L + step <= 31 && e <= r) L += step;
    }
    const uint32_t wl = __shfl_sync(0xffffffffu, bw.word, L);
    const int32_t el = __shfl_sync(0xffffffffu, bw.excl, L);
    int32_t j = -1;
    if (lane < count) {
        const int32_t t = 32 * (bw.w0 + L) + nth_set_bit(wl, r - el);
        j = cand_index(rt, t);
    }
    bw.taken += count;
    *j_out = j;
    return count;
}

__device__ __forceinline__ void walk_begin(const MaskGraph &G, const RunTable &rt, int32_t t_from, BitWalk &bw,
                                           int lane) {
    bw.w0 = t_from >> 5;
    if (bw.w0 >= rt.words) {
        bw.win_tot = bw.taken = 0;
        return;
    }
    walk_window(G, rt, t_from, bw, lane);
}

// ---- hook pass / full lazy pass over the masks ---------------------------
// check_union_body of fit_kernels.cuh with the rows read from the masks:
// persistent warps over nodes (contiguous chunks), candidate edges (a, b > a)
// with b a node, checked only while the roots observed differ; max_edges
// bounds the candidate edges a node examines (the hook pass takes 3).
__global__ void __launch_bounds__(kCheckWarps * 32, CNN_MASK_MIN_BLOCKS) mask_check_union_kernel(
    int64_t n, MaskGraph G, int32_t *__restrict__ parent, int32_t needed, int32_t max_edges,
    unsigned long long *__restrict__ counters) {
    __shared__ RunTable s_ra[kCheckWarps], s_rb[kCheckWarps];
    __shared__ SegTable s_sg[kCheckWarps];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    RunTable &RA = s_ra[wid];
    RunTable &RB = s_rb[wid];
    SegTable &SG = s_sg[wid];
    const int64_t warp0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    unsigned long long n_checks = 0, n_acc = 0;
    const int64_t per = (n + nwarps - 1) / nwarps;
    const int64_t a_end = min(n, (warp0 + 1) * per);
    for (int64_t a64 = warp0 * per; a64 < a_end; ++a64) {
        const int32_t a = (int32_t)a64;
        const int32_t pa = *(volatile int32_t *)&parent[a];
        if (pa < 0) continue;  // not a node
        load_runs(G, a, RA, lane);
        const int32_t t_from = RA.self_t + 1;
        BitWalk bw;
        walk_begin(G, RA, t_from, bw, lane);
        int32_t ra = -1, rx = -1;
        bool dirty = true;
        int32_t seen = 0;
        int32_t b;
        int32_t got;
        while (seen < max_edges && (got = walk_next(G, RA, t_from, bw, lane, &b)) > 0) {
            const int32_t pb = lane < got ? *(volatile int32_t *)&parent[b] : -1;
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
                    load_runs(G, bb, RB, lane);
                    ok = mask_check(G, RA, RB, SG, needed, lane);
                    ++n_checks;
                }
                if (ok) {
                    // link the two observed roots directly (larger under
                    // smaller); if the larger one is no longer a root, take
                    // the general path and re-resolve
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

// Cross edges after the hook pass and a full compression (parent holds
// roots): every (a, b > a), both nodes, whose roots differ -> worklist.
__global__ void __launch_bounds__(256) mask_cross_filter_kernel(int64_t n, MaskGraph G,
                                                                const int32_t *__restrict__ parent,
                                                                int2 *__restrict__ wl,
                                                                unsigned long long *__restrict__ wl_count,
                                                                int64_t cap) {
    __shared__ RunTable s_ra[8];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    RunTable &RA = s_ra[wid];
    const unsigned lt = (1u << lane) - 1u;
    const int64_t warp0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t a64 = warp0; a64 < n; a64 += nwarps) {
        const int32_t a = (int32_t)a64;
        const int32_t pa = parent[a];
        if (pa < 0) continue;
        load_runs(G, a, RA, lane);
        const int32_t t_from = RA.self_t + 1;
        BitWalk bw;
        walk_begin(G, RA, t_from, bw, lane);
        int32_t b, got;
        while ((got = walk_next(G, RA, t_from, bw, lane, &b)) > 0) {
            const int32_t pb = lane < got ? parent[b] : -1;
            const bool cross = pb >= 0 && pb != pa;
            const unsigned mask = __ballot_sync(0xffffffffu, cross);
            if (!mask) continue;
            unsigned long long base = 0;
            if (lane == 0) base = atomicAdd(wl_count, (unsigned long long)__popc(mask));
            base = __shfl_sync(0xffffffffu, base, 0);
            const unsigned long long idx = base + __popc(mask & lt);
            if (cross && idx < (unsigned long long)cap) wl[idx] = make_int2(a, b);
        }
    }
}

// The worklist's edges, each checked while the roots differ.
__global__ void __launch_bounds__(kCheckWarps * 32, CNN_MASK_MIN_BLOCKS) mask_edge_check_kernel(
    const int2 *__restrict__ wl, const unsigned long long *__restrict__ wl_count, int64_t cap, MaskGraph G,
    int32_t *__restrict__ parent, int32_t needed, unsigned long long *__restrict__ counters) {
    __shared__ RunTable s_ra[kCheckWarps], s_rb[kCheckWarps];
    __shared__ SegTable s_sg[kCheckWarps];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    RunTable &RA = s_ra[wid];
    RunTable &RB = s_rb[wid];
    SegTable &SG = s_sg[wid];
    const int64_t warp0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const unsigned long long total = *wl_count;
    if (total > (unsigned long long)cap) return;  // overflow: the full lazy pass runs instead
    const int64_t count = (int64_t)total;
    unsigned long long n_checks = 0, n_acc = 0;
    int32_t loaded_a = -1;  // whose run table RA holds (edges of one row come together)
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
                if (aa != loaded_a) {
                    load_runs(G, aa, RA, lane);
                    loaded_a = aa;
                }
                load_runs(G, bb, RB, lane);
                ok = mask_check(G, RA, RB, SG, needed, lane);
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
__global__ void __launch_bounds__(kCheckWarps * 32) mask_overflow_kernel(int64_t n, MaskGraph G,
                                                                         int32_t *__restrict__ parent, int32_t needed,
                                                                         const unsigned long long *__restrict__ wl_count,
                                                                         int64_t cap,
                                                                         unsigned long long *__restrict__ counters) {
    if (*wl_count <= (unsigned long long)cap) return;
    // the body of mask_check_union_kernel with every edge of every node
    __shared__ RunTable s_ra[kCheckWarps], s_rb[kCheckWarps];
    __shared__ SegTable s_sg[kCheckWarps];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    RunTable &RA = s_ra[wid];
    RunTable &RB = s_rb[wid];
    SegTable &SG = s_sg[wid];
    const int64_t warp0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    unsigned long long n_checks = 0, n_acc = 0;
    for (int64_t a64 = warp0; a64 < n; a64 += nwarps) {
        const int32_t a = (int32_t)a64;
        if (*(volatile int32_t *)&parent[a] < 0) continue;
        load_runs(G, a, RA, lane);
        const int32_t t_from = RA.self_t + 1;
        BitWalk bw;
        walk_begin(G, RA, t_from, bw, lane);
        int32_t b, got;
        while ((got = walk_next(G, RA, t_from, bw, lane, &b)) > 0) {
            const int32_t pb = lane < got ? *(volatile int32_t *)&parent[b] : -1;
            unsigned mask = __ballot_sync(0xffffffffu, pb >= 0);
            while (mask) {
                const int src = __ffs(mask) - 1;
                mask &= mask - 1;
                const int32_t bb = __shfl_sync(0xffffffffu, b, src);
                int32_t same = 0;
                if (lane == 0) same = uf_find(parent, a) == uf_find(parent, bb);
                same = __shfl_sync(0xffffffffu, same, 0);
                if (same) continue;
                bool ok;
                if (needed <= 0) {
                    ok = needed == 0;
                } else {
                    load_runs(G, bb, RB, lane);
                    ok = mask_check(G, RA, RB, SG, needed, lane);
                    ++n_checks;
                }
                if (ok) {
                    if (lane == 0) uf_unite(parent, a, bb);
                    __syncwarp();
                    ++n_acc;
                }
            }
        }
    }
    if (lane == 0 && n_checks) atomicAdd(&counters[5], n_checks);
    if (lane == 0 && n_acc) atomicAdd(&counters[6], n_acc);
}

// Lists from the masks: row p's set bits, ascending, at cols[row_off[p]..].
__global__ void __launch_bounds__(256) masks_to_lists_kernel(int64_t n, MaskGraph G,
                                                             const int64_t *__restrict__ row_off,
                                                             int32_t *__restrict__ cols) {
    __shared__ RunTable s_ra[8];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    RunTable &RA = s_ra[wid];
    const int64_t warp0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t p64 = warp0; p64 < n; p64 += nwarps) {
        const int32_t p = (int32_t)p64;
        if (row_off[p + 1] == row_off[p]) continue;  // empty row (a non-finite point)
        load_runs(G, p, RA, lane);
        BitWalk bw;
        walk_begin(G, RA, 0, bw, lane);
        int64_t w = row_off[p];
        int32_t j, got;
        while ((got = walk_next(G, RA, 0, bw, lane, &j)) > 0) {
            if (lane < got) cols[w + lane] = j;
            w += got;
        }
    }
}

// Full common-neighbour count of every pair (p, q > p) of the point-order
// lists (off, cols), from the masks (one warp per point p; inv maps point
// index -> internal index).  The MST fitter's weights
// (SimilarityCheckerExtScreensorted._get, src/cnnclustering/_types.pyx:
// 2708-2753: the whole intersection, no early exit).
__global__ void __launch_bounds__(256) mask_pair_weight_kernel(int64_t n, MaskGraph G,
                                                               const int32_t *__restrict__ inv,
                                                               const int64_t *__restrict__ off,
                                                               const int32_t *__restrict__ cols,
                                                               int32_t *__restrict__ weight) {
    __shared__ RunTable s_ra[8], s_rb[8];
    __shared__ SegTable s_sg[8];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    RunTable &RA = s_ra[wid];
    RunTable &RB = s_rb[wid];
    SegTable &SG = s_sg[wid];
    const int64_t warp0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t p = warp0; p < n; p += nwarps) {
        const int64_t s = off[p], e = off[p + 1];
        const int64_t k0 = warp_upper_bound(cols, s, e, (int32_t)p, lane);
        if (k0 >= e) continue;
        load_runs(G, inv[p], RA, lane);
        for (int64_t k = k0; k < e; ++k) {
            load_runs(G, inv[cols[k]], RB, lane);
            const int32_t w = mask_common(G, RA, RB, SG, lane);
            if (lane == 0) weight[k] = w;
        }
    }
}

MaskGraph mask_graph(const cnn_context *ctx) {
    MaskGraph G;
    G.cell_start = ctx->cell_start.as<int64_t>();
    G.pcell = ctx->pcell.as<int32_t>();
    G.mbase = ctx->mbase.as<int64_t>();
    G.masks = ctx->masks.as<uint32_t>();
    G.g0 = ctx->mask_geo.g[0];
    G.g1 = ctx->mask_geo.g[1];
    G.g2 = ctx->mask_geo.g[2];
    return G;
}

unsigned resident_blocks(cnn_context *ctx, const void *kernel, int threads, int64_t want) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, 0) != cudaSuccess || per_sm < 1) {
        (void)cudaGetLastError();
        per_sm = 1;
    }
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)per_sm * ctx->sm_count));
}

}  // namespace

cnn_status mask_pair_weights(cnn_context *ctx, const int64_t *off, const int32_t *cols, int32_t *weight) {
    const int64_t n = ctx->n;
    if (!ctx->graph_mask) return ctx->fail(CNN_ERR_STATE, "no neighbour graph in mask form");
    if (n == 0) return CNN_OK;
    mask_pair_weight_kernel<<<std::min<unsigned>(grid_for(n * 32, 256), ctx->sm_count * 16u), 256, 0, ctx->stream>>>(
        n, mask_graph(ctx), ctx->inv.as<int32_t>(), off, cols, weight);
    CNN_LAUNCH_CHECK(ctx);
    return CNN_OK;
}

cnn_status masks_to_lists(cnn_context *ctx) {
    const int64_t n = ctx->n;
    if (n == 0 || ctx->nnz == 0) return CNN_OK;
    masks_to_lists_kernel<<<std::min<unsigned>(grid_for(n * 32, 256), ctx->sm_count * 16u), 256, 0, ctx->stream>>>(
        n, mask_graph(ctx), ctx->row_off.as<int64_t>(), ctx->cols.as<int32_t>());
    CNN_LAUNCH_CHECK(ctx);
    return CNN_OK;
}

cnn_status fit_mask_impl(cnn_context *ctx, int64_t similarity_cutoff, int64_t n_member_cutoff, int64_t current_start,
                         uint8_t *consider_dev, int64_t *labels_dev) {
    ctx->counted_labels = nullptr;  // this fit leaves no label counts
    stages_reset(ctx, 5, 8);
    if (!ctx->have_graph || !ctx->graph_mask) return ctx->fail(CNN_ERR_STATE, "no neighbour graph in mask form");
    const int64_t n = ctx->n;
    cudaStream_t st = ctx->stream;
    ctx->fit_stats_pending = false;
    if (n == 0) return CNN_OK;
    if (similarity_cutoff > INT32_MAX) similarity_cutoff = INT32_MAX;
    if (similarity_cutoff < -1) similarity_cutoff = -1;
    CNN_TRY(ctx->ensure(ctx->node, (size_t)n));
    CNN_TRY(ctx->ensure(ctx->parent, sizeof(int32_t) * (size_t)n));
    CNN_TRY(ctx->ensure(ctx->comp_min, sizeof(int32_t) * (size_t)n));
    CNN_TRY(ctx->ensure(ctx->flag, sizeof(int32_t) * (size_t)(n + 1)));
    CNN_TRY(ctx->ensure(ctx->scratch_a, sizeof(int64_t) * (size_t)(n + 1)));
    unsigned long long *counters = ctx->counters.as<unsigned long long>();
    CNN_CUDA(ctx, cudaMemsetAsync(counters + 4, 0, 5 * sizeof(unsigned long long), st));
    uint8_t *node = ctx->node.as<uint8_t>();
    int32_t *parent = ctx->parent.as<int32_t>();
    int32_t *comp_min = ctx->comp_min.as<int32_t>();
    const int32_t *perm = ctx->perm.as<int32_t>();
    const MaskGraph G = mask_graph(ctx);
    const unsigned small = std::min<unsigned>(grid_for(n, 256), ctx->sm_count * 16u);
    const int32_t needed = (int32_t)similarity_cutoff;

    stage_begin(ctx, 5);
    node_kernel<<<small, 256, 0, st>>>(ctx->deg.as<int32_t>(), perm, consider_dev, n, n_member_cutoff, node, parent,
                                       comp_min, counters);
    CNN_LAUNCH_CHECK(ctx);
    stage_end(ctx, 5);

    stage_begin(ctx, 6);
    const unsigned check_blocks =
        resident_blocks(ctx, (const void *)mask_check_union_kernel, kCheckWarps * 32, grid_for(n, kCheckWarps));
    mask_check_union_kernel<<<check_blocks, kCheckWarps * 32, 0, st>>>(n, G, parent, needed, kHookEdges, counters);
    CNN_LAUNCH_CHECK(ctx);
    root_store_kernel<<<small, 256, 0, st>>>(n, node, parent);
    CNN_LAUNCH_CHECK(ctx);
    const int64_t wl_cap = std::max<int64_t>(int64_t(1) << 20, ctx->nnz / 16);
    CNN_TRY(ctx->ensure(ctx->io_c, sizeof(int2) * (size_t)wl_cap));
    unsigned long long *wl_count = counters + 8;
    CNN_CUDA(ctx, cudaMemsetAsync(wl_count, 0, sizeof(unsigned long long), st));
    mask_cross_filter_kernel<<<resident_blocks(ctx, (const void *)mask_cross_filter_kernel, 256,
                                               grid_for(n * 32, 256)),
                               256, 0, st>>>(n, G, parent, ctx->io_c.as<int2>(), wl_count, wl_cap);
    CNN_LAUNCH_CHECK(ctx);
    mask_edge_check_kernel<<<resident_blocks(ctx, (const void *)mask_edge_check_kernel, kCheckWarps * 32,
                                             grid_for(n, kCheckWarps)),
                             kCheckWarps * 32, 0, st>>>(ctx->io_c.as<int2>(), wl_count, wl_cap, G, parent, needed,
                                                        counters);
    CNN_LAUNCH_CHECK(ctx);
    mask_overflow_kernel<<<check_blocks, kCheckWarps * 32, 0, st>>>(n, G, parent, needed, wl_count, wl_cap, counters);
    CNN_LAUNCH_CHECK(ctx);
    stage_end(ctx, 6);

    stage_begin(ctx, 7);
    int32_t *flag = ctx->flag.as<int32_t>();
    int64_t *rank = ctx->scratch_a.as<int64_t>();
    CNN_CUDA(ctx, cudaMemsetAsync(flag, 0, sizeof(int32_t) * (size_t)(n + 1), st));
    root_min_kernel<<<small, 256, 0, st>>>(n, node, parent, perm, comp_min);
    CNN_LAUNCH_CHECK(ctx);
    root_store_kernel<<<small, 256, 0, st>>>(n, node, parent);
    CNN_LAUNCH_CHECK(ctx);
    min_flag_kernel<<<small, 256, 0, st>>>(n, node, parent, comp_min, flag);
    CNN_LAUNCH_CHECK(ctx);
    CNN_TRY(scan_exclusive_i32_to_i64(ctx, flag, rank, n + 1));
    label_kernel<<<small, 256, 0, st>>>(n, node, parent, comp_min, perm, rank, current_start, labels_dev);
    CNN_LAUNCH_CHECK(ctx);
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

}  // namespace cnn
