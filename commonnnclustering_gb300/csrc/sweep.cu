// sweep.cu -- batched fits over many (radius, cnn_cutoff) pairs.
//
// Reference caller: HierarchicalFitterRepeat (src/cnnclustering/
// _fit.pyx:1014-1187) refits all points from scratch for every
// (radius_cutoff, cnn_cutoff) step (:1131-1141), each fit recomputing every
// neighbourhood.  Here the neighbour search runs once, at the largest
// radius: every stored pair (p, j) gets the index of the smallest radius
// whose cutoff admits it ("bucket").  Because the float64 distance does not
// depend on the radius, the neighbourhood at radius k is exactly the pairs
// with bucket <= k -- a stable filter of the index-sorted r_max rows, so the
// filtered rows stay sorted.  Each radius's graph is materialised once and
// fitted for every cut; every fit and sort is the same code cnn_fit and
// cnn_sort_by_size run, so each result equals a separate fit.
#include <math.h>
#include <stdlib.h>

#include <algorithm>
#include <chrono>
#include <vector>

#include "common.cuh"

namespace cnn {

namespace {

constexpr int kMaxRadii = 16;
#ifndef CNN_BUCKET_UNROLL
#define CNN_BUCKET_UNROLL 4
#endif
constexpr int kBucketUnroll = CNN_BUCKET_UNROLL;  // row entries per lane per step of the per-row passes
#ifndef CNN_BUCKET_MIN_BLOCKS
#define CNN_BUCKET_MIN_BLOCKS 4  // 64 registers (a few bytes spilled) for four blocks per SM
#endif

struct Ladder {
    int32_t k;                  // number of radii
    double rc[kMaxRadii];       // cutoffs as compared (ascending)
    float thr_in[kMaxRadii];    // float32 sure-in thresholds on squared distance
    float thr_out[kMaxRadii];   // float32 sure-out thresholds
    int32_t metric, fpmode;
};

__device__ __forceinline__ double exact_s(const double *__restrict__ x, int d, int32_t a, int32_t b, int fpmode) {
    const double *xa = x + (int64_t)a * d, *xb = x + (int64_t)b * d;
    double s = 0.0;
    if (fpmode == CNN_FP_FUSED) {
        for (int k = 0; k < d; ++k) {
            const double t = __dsub_rn(xa[k], xb[k]);
            s = __fma_rn(t, t, s);
        }
    } else {
        for (int k = 0; k < d; ++k) {
            const double t = __dsub_rn(xa[k], xb[k]);
            s = __dadd_rn(s, __dmul_rn(t, t));
        }
    }
    return s;
}

// One warp per row of the r_max graph (internal order): bucket of each pair.
// With deg_all, the same pass counts each row's pairs of every radius below
// the largest (bucket <= k) into deg_all[k * (n + 1) + p] (entry n: 0).
// The ladder sits in shared memory (lanes index it by their own radius) and
// every lane counts its pairs per bucket in its own shared-memory column.
// In-band pairs wait in a per-warp queue and are decided in float64 32 at a
// time, one per lane: decided where they are found, each would stall its
// whole warp on a dependent gather (about one 32-entry step in two holds one
// on a wide box, where the float32 bands are wide).
constexpr int kBandQueue = 64;

__global__ void __launch_bounds__(256, CNN_BUCKET_MIN_BLOCKS) bucket_kernel(const double *__restrict__ x, int d, int64_t n,
                                                     const int32_t *__restrict__ perm,
                                                     const float4 *__restrict__ xf4,
                                                     const int64_t *__restrict__ row_off,
                                                     const int32_t *__restrict__ cols, Ladder lad,
                                                     uint8_t *__restrict__ bucket,
                                                     unsigned long long *__restrict__ n_exact, int kf,
                                                     int32_t *__restrict__ deg_all) {
    __shared__ float s_in[kMaxRadii], s_out[kMaxRadii];
    __shared__ double s_rc[kMaxRadii];
    __shared__ int32_t s_cnt[8][kMaxRadii][32];  // [warp][bucket][lane]
    __shared__ int64_t s_qe[8][kBandQueue];       // queued in-band pairs: entry,
    __shared__ int32_t s_qj[8][kBandQueue];       // other point (internal index),
    __shared__ int32_t s_qk[8][kBandQueue];       // lowest possible bucket
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned lt = (1u << lane) - 1u;
    if (threadIdx.x < kMaxRadii) {
        s_in[threadIdx.x] = threadIdx.x < lad.k ? lad.thr_in[threadIdx.x] : INFINITY;
        s_out[threadIdx.x] = threadIdx.x < lad.k ? lad.thr_out[threadIdx.x] : INFINITY;
        s_rc[threadIdx.x] = threadIdx.x < lad.k ? lad.rc[threadIdx.x] : INFINITY;
    }
#pragma unroll
    for (int b = 0; b < kMaxRadii; ++b) s_cnt[w][b][lane] = 0;
    __syncthreads();
    const int64_t p = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    if (deg_all && p == 0 && lane < kf) deg_all[(int64_t)lane * (n + 1) + n] = 0;
    if (p >= n) return;  // whole warps (nothing below syncs the block)
    const float4 q = xf4[p];
    const int32_t ip = perm[p];
    unsigned long long ex = 0;
    const int kl = lad.k - 1;
    const int64_t e_end = row_off[p + 1];
    int qn = 0;  // queued pairs (warp-uniform)
    // lanes < count decide queue entries [0, count) in float64
    auto decide = [&](int count) {
        __syncwarp();
        if (lane < count) {
            const int64_t e = s_qe[w][lane];
            double s = exact_s(x, d, ip, perm[s_qj[w][lane]], lad.fpmode);
            if (lad.metric == CNN_METRIC_EUCLIDEAN) s = __dsqrt_rn(s);
            int b = lad.k - 1;
            for (int kk = s_qk[w][lane]; kk < lad.k; ++kk)
                if (s <= s_rc[kk]) {
                    b = kk;
                    break;
                }
            bucket[e] = (uint8_t)b;
            ++s_cnt[w][b][lane];
            ++ex;
        }
        __syncwarp();
    };
    // 32 kBucketUnroll entries per step, kBucketUnroll per lane: their column
    // loads, then their coordinate gathers, are in flight together
    for (int64_t e0 = row_off[p]; e0 < e_end; e0 += kBucketUnroll * 32) {
        int32_t jv[kBucketUnroll];
        float4 cv[kBucketUnroll];
#pragma unroll
        for (int u = 0; u < kBucketUnroll; ++u) {
            const int64_t e = e0 + u * 32 + lane;
            jv[u] = e < e_end ? cols[e] : -1;
        }
#pragma unroll
        for (int u = 0; u < kBucketUnroll; ++u) cv[u] = jv[u] >= 0 ? xf4[jv[u]] : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int u = 0; u < kBucketUnroll; ++u) {
            const bool valid = jv[u] >= 0;
            const int64_t e = e0 + u * 32 + lane;
            const float dx = q.x - cv[u].x, dy = q.y - cv[u].y, dz = q.z - cv[u].z;
            const float sf = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
            // radii that are certainly too small (the thresholds ascend)
            int k = 0;
#pragma unroll
            for (int kk = 0; kk < kMaxRadii - 1; ++kk) k += (kk < kl) & (sf > s_out[kk]);
            const bool band = valid && !(sf <= s_in[k]);  // inside the band of radius k
            const unsigned bm = __ballot_sync(0xffffffffu, band);
            if (band) {  // queue it (qn <= 31 here, so the queue has room for 32)
                const int slot = qn + __popc(bm & lt);
                s_qe[w][slot] = e;
                s_qj[w][slot] = jv[u];
                s_qk[w][slot] = k;
            } else if (valid) {
                bucket[e] = (uint8_t)k;
                ++s_cnt[w][k][lane];
            }
            qn += __popc(bm);
            if (qn >= 32) {
                decide(32);
                if (lane < qn - 32) {  // move the rest (fewer than 32) to the front
                    s_qe[w][lane] = s_qe[w][lane + 32];
                    s_qj[w][lane] = s_qj[w][lane + 32];
                    s_qk[w][lane] = s_qk[w][lane + 32];
                }
                qn -= 32;
            }
        }
    }
    if (qn > 0) decide(qn);
    if (deg_all) {
        __syncwarp();
        int32_t run = 0;  // this lane's pairs of buckets <= k
        for (int k = 0; k < kf; ++k) {
            run += s_cnt[w][k][lane];
            const int32_t t = __reduce_add_sync(0xffffffffu, run);
            if (lane == 0) deg_all[(int64_t)k * (n + 1) + p] = t;
        }
    }
    for (int o = 16; o > 0; o >>= 1) ex += __shfl_down_sync(0xffffffffu, ex, o);
    if (lane == 0 && ex) atomicAdd(n_exact, ex);
}

__global__ void filter_count_kernel(int64_t n, const int64_t *__restrict__ row_off, const uint8_t *__restrict__ bucket,
                                    int k, int32_t *__restrict__ deg) {
    const int lane = threadIdx.x & 31;
    const int64_t p = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    if (p >= n) return;
    int32_t c = 0;
    for (int64_t e = row_off[p] + lane; e < row_off[p + 1]; e += 32) c += bucket[e] <= k;
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    if (lane == 0) deg[p] = c;
}

__global__ void filter_fill_kernel(int64_t n, const int64_t *__restrict__ row_off, const int32_t *__restrict__ cols,
                                   const uint8_t *__restrict__ bucket, int k, const int64_t *__restrict__ out_off,
                                   int32_t *__restrict__ out_cols) {
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    const int64_t p = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    if (p >= n) return;
    int64_t w = out_off[p];
    for (int64_t e0 = row_off[p]; e0 < row_off[p + 1]; e0 += 32) {
        const int64_t e = e0 + lane;
        const bool keep = e < row_off[p + 1] && bucket[e] <= k;
        const unsigned m = __ballot_sync(0xffffffffu, keep);
        if (keep) out_cols[w + __popc(m & lt)] = cols[e];
        w += __popc(m);
    }
}

// Every radius below the largest at once: bucket_kernel counts, per row, the
// pairs of each radius (bucket <= k); one pass writes each radius's filtered
// rows (stable, so still sorted).  Radius k's arrays sit at k * (n + 1) in
// deg_all / off_all and at base[k] in cols_all.
constexpr int kMaxFiltered = kMaxRadii - 1;

__global__ void __launch_bounds__(256) multi_fill_kernel(int64_t n, const int64_t *__restrict__ row_off,
                                                         const int32_t *__restrict__ cols,
                                                         const uint8_t *__restrict__ bucket, int kf,
                                                         const int64_t *__restrict__ off_all,
                                                         const int64_t *__restrict__ base,
                                                         int32_t *__restrict__ cols_all) {
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    const int64_t warp0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t p = warp0; p < n; p += nwarps) {
        int64_t w[kMaxFiltered];
#pragma unroll
        for (int k = 0; k < kMaxFiltered; ++k) w[k] = k < kf ? base[k] + off_all[(int64_t)k * (n + 1) + p] : 0;
        const int64_t e1 = row_off[p + 1];
        for (int64_t e0 = row_off[p]; e0 < e1; e0 += kBucketUnroll * 32) {
            int bv[kBucketUnroll];
            int32_t cv[kBucketUnroll];
#pragma unroll
            for (int u = 0; u < kBucketUnroll; ++u) {  // four entries per lane in flight
                const int64_t e = e0 + u * 32 + lane;
                const bool valid = e < e1;
                bv[u] = valid ? bucket[e] : 255;
                cv[u] = valid ? cols[e] : 0;
            }
#pragma unroll
            for (int u = 0; u < kBucketUnroll; ++u) {  // in entry order: the rows stay sorted
#pragma unroll
                for (int k = 0; k < kMaxFiltered; ++k) {
                    if (k >= kf) break;
                    const bool keep = bv[u] <= k;
                    const unsigned m = __ballot_sync(0xffffffffu, keep);
                    if (keep) cols_all[w[k] + __popc(m & lt)] = cv[u];
                    w[k] += __popc(m);
                }
            }
        }
    }
}

__global__ void set_zero_tail_kernel(int32_t *deg, int64_t n) { deg[n] = 0; }

bool ladder_thresholds(const std::vector<double> &ext, const std::vector<double> &rcs, int metric, Ladder *lad) {
    // float32 bands per radius: the same bound as the single-radius search,
    // evaluated at the largest radius (it only grows with R)
    const double u32 = ldexp(1.0, -24), u64 = ldexp(1.0, -53);
    const int d = (int)ext.size();
    const double rmax = metric == CNN_METRIC_EUCLIDEAN ? rcs.back() : sqrt(rcs.back());
    double err = 0;
    for (int k = 0; k < d; ++k) {
        const double delta = ext[k] * (u32 + 2 * u64);
        if (delta > 1e-3 * rmax) return false;
        const double eta = 2 * delta + u32 * (2 * rmax + 2 * delta);
        err += eta * (4 * rmax + eta);
    }
    const double gam = (d + 2) * u32 / (1 - (d + 2) * u32);
    err += gam * 4 * rmax * rmax + gam * err;
    for (size_t i = 0; i < rcs.size(); ++i) {
        const double rc2 = metric == CNN_METRIC_EUCLIDEAN ? rcs[i] * rcs[i] : rcs[i];
        const double b = 2 * (err + 8 * (d + 2) * u64 * rc2 + 1e-300);
        float fin = (float)(rc2 - b), fout = (float)(rc2 + b);
        if ((double)fin > rc2 - b) fin = nextafterf(fin, -INFINITY);
        if ((double)fout < rc2 + b) fout = nextafterf(fout, INFINITY);
        lad->thr_in[i] = fin > 0.f ? fin : -1.f;
        lad->thr_out[i] = fout;
        lad->rc[i] = rcs[i];
    }
    return true;
}

// Runs `body` -- host logic that only enqueues work on the context stream --
// as one CUDA graph: captured (relaxed mode: buffers may still grow, see
// cnn_context::ensure), instantiated and launched.  With `keep`, the
// instantiated graph stays with the context and the next call whose graph
// has the same shape only updates its parameters (no new instantiation or
// upload).  Where the stream cannot be captured or capture fails, nothing
// captured has run and `body` runs again with plain launches; it must
// therefore be repeatable from the same host state.
template <class F>
cnn_status run_as_graph(cnn_context *ctx, bool keep, F &&body) {
    cudaStream_t st = ctx->stream;
    if (!ctx->sweep_graphs || st == nullptr || st == cudaStreamLegacy || st == cudaStreamPerThread) return body();
    const auto t0 = std::chrono::steady_clock::now();
    const bool timing = ctx->timing;
    if (cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed) != cudaSuccess) {
        (void)cudaGetLastError();
        return body();
    }
    ctx->capturing = true;
    ctx->timing = false;  // stage events are not recorded inside a graph
    const int64_t launches0 = ctx->n_launches;
    const cnn_status s = body();
    cudaGraph_t graph = nullptr;
    const cudaError_t e = cudaStreamEndCapture(st, &graph);
    ctx->capturing = false;
    ctx->timing = timing;
    cudaGraphExec_t exec = nullptr;
    size_t nodes = 0;
    bool ok = s == CNN_OK && e == cudaSuccess && graph != nullptr &&
              cudaGraphGetNodes(graph, nullptr, &nodes) == cudaSuccess;
    if (ok && keep && ctx->sweep_exec) {
        cudaGraphExecUpdateResultInfo info{};
        if (cudaGraphExecUpdate(ctx->sweep_exec, graph, &info) == cudaSuccess) {
            exec = ctx->sweep_exec;  // same shape: parameters updated in place
        } else {
            (void)cudaGetLastError();
            cudaGraphExecDestroy(ctx->sweep_exec);
        }
        ctx->sweep_exec = nullptr;
    }
    if (ok && !exec) ok = cudaGraphInstantiate(&exec, graph, 0) == cudaSuccess;
    if (graph) cudaGraphDestroy(graph);
    if (!ok) {
        (void)cudaGetLastError();
        if (exec) cudaGraphExecDestroy(exec);
        for (void *p : ctx->deferred_free) cudaFree(p);  // nothing captured has run
        ctx->deferred_free.clear();
        ctx->n_launches = launches0;
        return body();
    }
    const cudaError_t le = cudaGraphLaunch(exec, st);
    if (keep && le == cudaSuccess) ctx->sweep_exec = exec;
    else cudaGraphExecDestroy(exec);  // released once the launch completes
    ctx->stats.graphs += 1;
    ctx->stats.graph_nodes += (int64_t)nodes;
    ctx->stats.ms_graph_build +=
        std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (le != cudaSuccess) {
        (void)cudaGetLastError();
        return ctx->fail(CNN_ERR_CUDA, std::string("cudaGraphLaunch: ") + cudaGetErrorString(le));
    }
    if (!ctx->deferred_free.empty()) {  // the blocks replaced during capture
        CNN_CUDA(ctx, cudaStreamSynchronize(st));
        for (void *p : ctx->deferred_free) cudaFree(p);
        ctx->deferred_free.clear();
    }
    return CNN_OK;
}

}  // namespace

cnn_status sweep_impl(cnn_context *ctx, const double *rcs_in, int32_t n_radii, const int64_t *sim_cut,
                      const int64_t *member_cut, int32_t n_cuts, int metric, int fpmode, int64_t sort_member_cutoff,
                      int64_t max_clusters, int64_t *labels_dev, const int32_t *out_slot, bool sort) {
    const int64_t n = ctx->n;
    const int d = ctx->d;
    cudaStream_t st = ctx->stream;
    std::vector<double> rcs(rcs_in, rcs_in + n_radii);
    for (int i = 1; i < n_radii; ++i)
        if (!(rcs[i] >= rcs[i - 1])) return ctx->fail(CNN_ERR_INVALID_ARG, "radius cutoffs must be ascending");
    // output slot of (radius k, cut j); -1: not wanted
    auto slot = [&](int32_t k, int j) -> int64_t {
        return out_slot ? (int64_t)out_slot[(int64_t)k * n_cuts + j] : (int64_t)k * n_cuts + j;
    };

    // Components only grow along the (radius, cut) lattice: a pair accepted
    // at (r, sim, nmem) is accepted at any (r' >= r, 0 <= sim' <= sim,
    // nmem' <= nmem) -- neighbourhoods, degrees and intersections only grow.
    // So each fit starts from the finished components of up to two fits that
    // refine it (the same cut at the last radius it ran at, and the closest
    // stricter cut at this radius); the lazy check then skips every pair
    // already joined.  The result is the same partition (the seeds only join
    // points the fit itself would join), so labels equal a separate fit's.
    std::vector<int> order(n_cuts);
    for (int j = 0; j < n_cuts; ++j) order[j] = j;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        return sim_cut[a] != sim_cut[b] ? sim_cut[a] > sim_cut[b] : member_cut[a] > member_cut[b];
    });
    auto refines = [&](int i, int j) {  // fit i's components refine fit j's (same radius or smaller)
        return sim_cut[j] >= 0 && sim_cut[i] >= sim_cut[j] && member_cut[i] >= member_cut[j];
    };
    CNN_TRY(ctx->ensure(ctx->sweep_forest, sizeof(int32_t) * (size_t)n * (size_t)n_cuts + 256));
    int32_t *forest = ctx->sweep_forest.as<int32_t>();
    std::vector<char> have(n_cuts, 0);  // slot j: cut j at the last radius it ran at
    // Within a radius the graph is fixed, so a fit only needs to look at the
    // pairs the fit it starts from left open (not both in one component):
    // the pairs inside its components are inside this fit's components too.
    // Those open pairs are kept as a list (two alternating buffers) while
    // fits follow each other at one radius.
    auto fit_cuts = [&](int32_t k, bool same_order_as_previous) -> cnn_status {
        if (!same_order_as_previous) std::fill(have.begin(), have.end(), 0);
        std::vector<int> todo;
        for (int t = 0; t < n_cuts; ++t)
            if (slot(k, order[t]) >= 0) todo.push_back(order[t]);
        const int64_t half = ctx->nnz / 2 + 1;
        const bool lists = todo.size() > 1 && n > 0 && half * (int64_t)(2 * sizeof(int2)) <= (int64_t(24) << 30);
        int2 *cur = nullptr, *nxt = nullptr;
        unsigned long long *ccur = nullptr, *cnxt = nullptr;
        if (lists) {
            CNN_TRY(ctx->ensure(ctx->sweep_open_a, sizeof(int2) * (size_t)half));
            CNN_TRY(ctx->ensure(ctx->sweep_open_b, sizeof(int2) * (size_t)half));
            CNN_TRY(ctx->ensure(ctx->sweep_open_count, 2 * sizeof(unsigned long long)));
            cur = ctx->sweep_open_a.as<int2>();
            nxt = ctx->sweep_open_b.as<int2>();
            ccur = ctx->sweep_open_count.as<unsigned long long>();
            cnxt = ccur + 1;
        }
        std::vector<int> done_here;
        int last = -1;            // the cut fitted last at this radius
        bool list_valid = false;  // cur holds the pairs `last` left open
        for (size_t t = 0; t < todo.size(); ++t) {
            const int j = todo[t];
            const int64_t out = slot(k, j);
            int best = -1;
            for (int i : done_here)
                if (refines(i, j) && (best < 0 || sim_cut[i] < sim_cut[best] ||
                                      (sim_cut[i] == sim_cut[best] && member_cut[i] < member_cut[best])))
                    best = i;
            const int32_t *sa = have[j] && sim_cut[j] >= 0 ? forest + (size_t)j * n : nullptr;
            const int32_t *sb = best >= 0 ? forest + (size_t)best * n : nullptr;
            const bool use_list = lists && list_valid && best == last;
            // the next open-pairs list is written after the fit: its buffer
            // (room for every pair b > a) holds this fit's cross-pair worklist
            CNN_TRY(fit_and_sort_into(ctx, sim_cut[j], member_cut[j], sort_member_cutoff, max_clusters,
                                      labels_dev + out * n, sa, sb, sort, use_list ? cur : nullptr,
                                      use_list ? ccur : nullptr, lists ? nxt : nullptr, lists ? half : 0));
            // after the fit the union-find array holds every node's root (-1 elsewhere)
            if (n > 0)
                CNN_CUDA(ctx, cudaMemcpyAsync(forest + (size_t)j * n, ctx->parent.ptr, sizeof(int32_t) * (size_t)n,
                                              cudaMemcpyDeviceToDevice, st));
            if (lists && t + 1 < todo.size()) {
                CNN_TRY(open_pairs_impl(ctx, use_list ? cur : nullptr, use_list ? ccur : nullptr, nxt, cnxt, half));
                std::swap(cur, nxt);
                std::swap(ccur, cnxt);
                list_valid = true;
            }
            have[j] = 1;
            done_here.push_back(j);
            last = j;
        }
        return CNN_OK;
    };

    // The fits of one or more radii as one CUDA graph: every fit, its sort
    // and the open-pair lists between fits enqueue the same work whatever
    // the data (counts stay on the device), so the host logic of fit_cuts
    // runs once at capture; a fallback repeats it from the same state.
    ctx->stats.graphs = 0;
    ctx->stats.graph_nodes = 0;
    ctx->stats.ms_graph_build = 0.f;
    auto fits_as_graph = [&](bool keep, auto &&fits) -> cnn_status {
        const std::vector<char> have0 = have;
        return run_as_graph(ctx, keep, [&]() -> cnn_status {
            have = have0;
            return fits();
        });
    };

    // one search, at the largest radius (the same search cnn_build_neighbours runs)
    CNN_TRY(build_neighbours_impl(ctx, rcs.back(), metric, fpmode));
    ctx->split_valid = false;  // the fits below see other graphs in the same arrays
    const int64_t nnz = ctx->nnz;
    Ladder lad{};
    lad.k = n_radii;
    lad.metric = metric;
    lad.fpmode = fpmode;
    // the radius buckets use plain differences: not for the periodic metric
    const bool ladder = ctx->stats.search_kind == 1 && n_radii > 1 && n > 0 &&
                        metric != CNN_METRIC_EUCLIDEAN_PERIODIC_REDUCED &&
                        ladder_thresholds(std::vector<double>(ctx->grid_extent, ctx->grid_extent + d), rcs, metric,
                                          &lad);
    if (!ladder) {
        // no cell-grid graph to filter (all-pairs or tensor-core search):
        // search every radius on its own, smallest first
        bool prev_identity = false;
        for (int32_t k = 0; k < n_radii; ++k) {
            if (k < n_radii - 1) CNN_TRY(build_neighbours_impl(ctx, rcs[k], metric, fpmode));
            else if (n_radii > 1) CNN_TRY(build_neighbours_impl(ctx, rcs.back(), metric, fpmode));
            // seeds across radii need the same internal order (identity here)
            const bool same = prev_identity && ctx->identity_perm;
            CNN_TRY(fits_as_graph(false, [&] { return fit_cuts(k, same); }));
            prev_identity = ctx->identity_perm;
        }
        return CNN_OK;
    }

    // buckets of the largest-radius graph, then keep it aside
    CNN_TRY(ctx->ensure(ctx->sweep_bucket, (size_t)(nnz > 0 ? nnz : 1)));
    uint8_t *bucket = ctx->sweep_bucket.as<uint8_t>();
    unsigned long long *counters = ctx->counters.as<unsigned long long>();
    const int kf = n_radii - 1;  // radii below the largest
    int32_t *deg_all = nullptr;  // their row lengths, counted with the buckets
    if (kf > 0 && n > 0) {
        CNN_TRY(ctx->ensure(ctx->sweep_multi_deg, sizeof(int32_t) * (size_t)kf * (size_t)(n + 1)));
        deg_all = ctx->sweep_multi_deg.as<int32_t>();
    }
    bucket_kernel<<<grid_for(n * 32, 256), 256, 0, st>>>(ctx->x, d, n, ctx->perm.as<int32_t>(), ctx->xf4.as<float4>(),
                                                          ctx->row_off.as<int64_t>(), ctx->cols.as<int32_t>(), lad,
                                                          bucket, counters + 15, kf, deg_all);
    CNN_LAUNCH_CHECK(ctx);
    std::swap(ctx->row_off, ctx->sweep_row_off_max);
    std::swap(ctx->cols, ctx->sweep_cols_max);
    std::swap(ctx->deg, ctx->sweep_deg_max);
    const int64_t *off_max = ctx->sweep_row_off_max.as<int64_t>();
    const int32_t *cols_max = ctx->sweep_cols_max.as<int32_t>();
    CNN_TRY(ctx->ensure(ctx->row_off, sizeof(int64_t) * (size_t)(n + 1)));
    CNN_TRY(ctx->ensure(ctx->deg, sizeof(int32_t) * (size_t)(n + 1)));

    // every smaller radius's graph in two passes, when they fit in the budget
    if (kf > 0 && n > 0) {
        CNN_TRY(ctx->ensure(ctx->sweep_multi_off, sizeof(int64_t) * (size_t)kf * (size_t)(n + 1)));
        int64_t *off_all = ctx->sweep_multi_off.as<int64_t>();
        const unsigned mgrid = std::min<unsigned>(grid_for((n + 1) * 32, 256), ctx->sm_count * 16u);
        for (int32_t k = 0; k < kf; ++k)
            CNN_TRY(scan_exclusive_i32_to_i64(ctx, deg_all + (size_t)k * (n + 1), off_all + (size_t)k * (n + 1), n + 1));
        std::vector<int64_t> nnz_k(kf), base(kf + 1, 0);
        for (int32_t k = 0; k < kf; ++k)
            CNN_CUDA(ctx, cudaMemcpyAsync(&nnz_k[k], off_all + (size_t)k * (n + 1) + n, sizeof(int64_t),
                                          cudaMemcpyDeviceToHost, st));
        CNN_CUDA(ctx, cudaStreamSynchronize(st));
        for (int32_t k = 0; k < kf; ++k) base[k + 1] = base[k] + nnz_k[k];
        // CNN_SWEEP_GRAPH_BUDGET (bytes) overrides the 48 GiB the graphs may take together
        int64_t budget = int64_t(48) << 30;
        if (const char *b = getenv("CNN_SWEEP_GRAPH_BUDGET")) budget = atoll(b);
        if (base[kf] * (int64_t)sizeof(int32_t) <= budget) {
            CNN_TRY(ctx->ensure(ctx->sweep_multi_cols, sizeof(int32_t) * (size_t)(base[kf] > 0 ? base[kf] : 1)));
            CNN_TRY(ctx->ensure(ctx->sweep_multi_base, sizeof(int64_t) * (size_t)(kf + 1)));
            CNN_CUDA(ctx, cudaMemcpyAsync(ctx->sweep_multi_base.ptr, base.data(), sizeof(int64_t) * (size_t)(kf + 1),
                                          cudaMemcpyHostToDevice, st));
            multi_fill_kernel<<<mgrid, 256, 0, st>>>(n, off_max, cols_max, bucket, kf, off_all,
                                                     ctx->sweep_multi_base.as<int64_t>(),
                                                     ctx->sweep_multi_cols.as<int32_t>());
            CNN_LAUNCH_CHECK(ctx);
            // the fits of radius k see views of its arrays as the graph, the
            // largest radius the kept graph itself; all 64 fits, one graph
            const cnn::DevBuf own_off = ctx->row_off, own_cols = ctx->cols, own_deg = ctx->deg;
            const cnn::DevBuf max_off = ctx->sweep_row_off_max, max_cols = ctx->sweep_cols_max,
                              max_deg = ctx->sweep_deg_max;
            auto all_fits = [&]() -> cnn_status {
                cnn_status fs = CNN_OK;
                for (int32_t k = 0; k < kf && fs == CNN_OK; ++k) {
                    ctx->row_off = cnn::DevBuf{off_all + (size_t)k * (n + 1), sizeof(int64_t) * (size_t)(n + 1)};
                    ctx->deg = cnn::DevBuf{deg_all + (size_t)k * (n + 1), sizeof(int32_t) * (size_t)(n + 1)};
                    ctx->cols = cnn::DevBuf{ctx->sweep_multi_cols.as<int32_t>() + base[k],
                                            sizeof(int32_t) * (size_t)(nnz_k[k] > 0 ? nnz_k[k] : 1)};
                    ctx->nnz = nnz_k[k];
                    fs = fit_cuts(k, true);
                }
                if (fs == CNN_OK) {
                    ctx->row_off = max_off;
                    ctx->cols = max_cols;
                    ctx->deg = max_deg;
                    ctx->nnz = nnz;
                    fs = fit_cuts(kf, true);
                }
                ctx->row_off = own_off;
                ctx->cols = own_cols;
                ctx->deg = own_deg;
                return fs;
            };
            CNN_TRY(fits_as_graph(true, all_fits));
            // the context keeps the largest-radius graph
            std::swap(ctx->row_off, ctx->sweep_row_off_max);
            std::swap(ctx->cols, ctx->sweep_cols_max);
            std::swap(ctx->deg, ctx->sweep_deg_max);
            ctx->nnz = nnz;
            return CNN_OK;
        }
    }
    for (int32_t k = 0; k < n_radii; ++k) {
        int64_t nnz_k = nnz;
        if (k < n_radii - 1) {
            filter_count_kernel<<<grid_for(n * 32, 256), 256, 0, st>>>(n, off_max, bucket, k, ctx->deg.as<int32_t>());
            CNN_LAUNCH_CHECK(ctx);
            set_zero_tail_kernel<<<1, 1, 0, st>>>(ctx->deg.as<int32_t>(), n);
            CNN_LAUNCH_CHECK(ctx);
            CNN_TRY(scan_exclusive_i32_to_i64(ctx, ctx->deg.as<int32_t>(), ctx->row_off.as<int64_t>(), n + 1));
            CNN_CUDA(ctx, cudaMemcpyAsync(&nnz_k, ctx->row_off.as<int64_t>() + n, sizeof(int64_t),
                                          cudaMemcpyDeviceToHost, st));
            CNN_CUDA(ctx, cudaStreamSynchronize(st));
            CNN_TRY(ctx->ensure(ctx->cols, sizeof(int32_t) * (size_t)(nnz_k > 0 ? nnz_k : 1)));
            filter_fill_kernel<<<grid_for(n * 32, 256), 256, 0, st>>>(n, off_max, cols_max, bucket, k,
                                                                       ctx->row_off.as<int64_t>(),
                                                                       ctx->cols.as<int32_t>());
            CNN_LAUNCH_CHECK(ctx);
        } else {
            // the largest radius is the kept graph itself
            std::swap(ctx->row_off, ctx->sweep_row_off_max);
            std::swap(ctx->cols, ctx->sweep_cols_max);
            std::swap(ctx->deg, ctx->sweep_deg_max);
        }
        ctx->nnz = nnz_k;
        // every radius keeps the largest-radius internal order
        CNN_TRY(fits_as_graph(false, [&] { return fit_cuts(k, true); }));
    }
    return CNN_OK;
}

}  // namespace cnn
