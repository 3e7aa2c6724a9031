// gram.cu -- radius neighbour search for n_dim >= 16 on the tensor cores.
//
// Squared distances come from the Gram matrix: d2(i,j) = |x_i|^2 + |x_j|^2
// - 2 x_i.x_j, on mean-centred coordinates.  x_i.x_j is computed on the 5th
// generation tensor cores (tcgen05.mma, kind::f16) from a BF16 split of
// every coordinate, x = hi + lo with hi = bf16(x), lo = bf16(x - hi):
// x.y ~ hi.hi + hi.lo + lo.hi (three MMAs per 16-wide K slice), FP32
// accumulation in tensor memory.  Per tile (128 x 128 pairs) a rigorous
// error bound gives a band around the cutoff: pairs below it are
// neighbours, pairs above are not, pairs inside are recomputed in float64
// with the reference's exact operation order (the only float64 step).
//
// Kernel structure (one persistent CTA per SM, 10 warps):
//   warp 0  TMA producer: hi/lo tiles of the row block I and the column
//           block J (cp.async.bulk.tensor, 128-byte swizzle) into a 2-stage
//           shared-memory ring, completion counted on an mbarrier;
//   warp 1  allocates 256 TMEM columns (two 128-column accumulators) and
//           issues the MMAs from one thread; tcgen05.commit frees the
//           shared stage and publishes the accumulator;
//   warps 2-9  epilogue, two per TMEM lane quadrant: each thread owns one
//           tile row (its TMEM lane) and 64 of the columns, loads 32
//           columns at a time with tcgen05.ld, compares, and appends hits /
//           band pairs to global lists.
// Only tiles with J >= I are computed; off-diagonal hits are emitted in
// both directions.  Every wait is bounded (globaltimer): on timeout the
// kernel records an error, stops issuing work and frees its TMEM.
#include <cuda.h>
#include <cuda_bf16.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "common.cuh"

namespace cnn {

namespace {

constexpr int kTM = 128;              // tile rows (M) = tile columns (N)
constexpr int kKB = 64;               // K block: 64 bf16 = 128 bytes per row
constexpr int kStages = 2;
constexpr int kTileBytes = kTM * kKB * 2;          // 16 KB: one operand tile
constexpr int kStageBytes = 4 * kTileBytes;         // A_hi, A_lo, B_hi, B_lo
constexpr int kGramThreads = 320;  // warp 0 TMA, warp 1 MMA, warps 2-9 epilogue
constexpr uint32_t kTmemCols = 256;
constexpr unsigned long long kWaitNs = 2000000000ull;  // 2 s per wait

struct GramArgs {
    int64_t n;
    int32_t nkb;        // K blocks of 64
    int32_t nblk;       // row blocks of 128
    int64_t ntiles;     // tiles in the list
    const int2 *tiles;  // (I, J >= I) block pairs that can hold a neighbour pair
    float rc2;          // squared radius the float32 value is compared with
    float coef;         // band = coef * maxnorm_I * maxnorm_J + slack
    float slack_coef;   // float32 epilogue rounding: slack_coef * (maxn2_I + maxn2_J)
    float min_band;
    const float *norm2;     // |x'_i|^2 (float)
    const float *blk_norm;  // max |x'_i| per row block
    const float *blk_norm2; // max |x'_i|^2 per row block
    uint64_t *keys;         // (row << 32 | col) of neighbours
    unsigned long long *nkeys;
    int64_t key_cap;
    uint64_t *amb;          // band pairs; bit 63 = emit both directions
    float *amb_d2;          // their float32 squared distance
    unsigned long long *namb;
    int64_t amb_cap;
    int *status;            // nonzero on a timed-out wait
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ uint64_t globaltimer() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait on an mbarrier phase.  Returns false on timeout or when
// another warp has already given up (abort flag in shared memory).
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, volatile int *abort_flag) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = globaltimer();
    for (;;) {
        if (mbar_try_wait(bar, parity)) return true;
        if (*abort_flag) return false;
        if (globaltimer() - t0 > kWaitNs) return false;
        __nanosleep(32);  // back off: waiting warps leave issue slots and shared-memory bandwidth
    }
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int c0, int c1, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            smem_u32(dst)),
        "l"((uint64_t)map), "r"(c0), "r"(c1), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor: K-major operand, 128-byte swizzle, rows
// of 128 bytes, 8-row groups 1024 bytes apart.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)1u << 16;             // leading byte offset (not used with 128-byte swizzle)
    d |= (uint64_t)(1024u >> 4) << 32;   // stride byte offset
    d |= (uint64_t)1u << 46;             // descriptor version
    d |= (uint64_t)2u << 61;             // 128-byte swizzle
    return d;
}

// Instruction descriptor, kind::f16: BF16 A and B (K-major), FP32 D, M = N = 128.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kTM >> 3) << 17) |
                            ((uint32_t)(kTM >> 4) << 24);

__device__ __forceinline__ void umma(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void umma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&v)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
          "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
          "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]),
          "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]),
          "=r"(v[30]), "=r"(v[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

struct EpilogueTile {
    int64_t gi;
    bool row_ok, diag;
    float ni, thr_in, thr_out;
    int32_t J;
};

__device__ __forceinline__ void tmem_ld32_async(uint32_t taddr, uint32_t (&v)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
          "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
          "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]),
          "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]),
          "=r"(v[30]), "=r"(v[31])
        : "r"(taddr));
}

// Waits for the outstanding tcgen05.ld; the registers are listed as
// operands so no use of them can be scheduled before the wait.
__device__ __forceinline__ void tmem_wait_ld(uint32_t (&v)[32]) {
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(v[0]), "+r"(v[1]), "+r"(v[2]), "+r"(v[3]), "+r"(v[4]), "+r"(v[5]), "+r"(v[6]), "+r"(v[7]),
                   "+r"(v[8]), "+r"(v[9]), "+r"(v[10]), "+r"(v[11]), "+r"(v[12]), "+r"(v[13]), "+r"(v[14]),
                   "+r"(v[15]), "+r"(v[16]), "+r"(v[17]), "+r"(v[18]), "+r"(v[19]), "+r"(v[20]), "+r"(v[21]),
                   "+r"(v[22]), "+r"(v[23]), "+r"(v[24]), "+r"(v[25]), "+r"(v[26]), "+r"(v[27]), "+r"(v[28]),
                   "+r"(v[29]), "+r"(v[30]), "+r"(v[31])
                 :
                 : "memory");
}

// Emission for a 32-column chunk with at least one neighbour or band pair
// somewhere in the warp: one warp-wide atomic per output list reserves the
// slots, then each thread writes its pairs.  Fully unrolled so the
// accumulator registers are never indexed dynamically.
__device__ __forceinline__ void epilogue_emit_masks(const GramArgs &args, const EpilogueTile &et,
                                                    const uint32_t (&v)[32], const float *norms, int col0, int lane,
                                                    uint32_t in_mask, uint32_t amb_mask) {
    const int per_hit = et.diag ? 1 : 2;
    const int my_keys = __popc(in_mask) * per_hit, my_amb = __popc(amb_mask);
    int inc_k = my_keys, inc_a = my_amb;
    for (int o = 1; o < 32; o <<= 1) {
        const int uk = __shfl_up_sync(0xffffffffu, inc_k, o);
        const int ua = __shfl_up_sync(0xffffffffu, inc_a, o);
        if (lane >= o) {
            inc_k += uk;
            inc_a += ua;
        }
    }
    const int tot_k = __shfl_sync(0xffffffffu, inc_k, 31), tot_a = __shfl_sync(0xffffffffu, inc_a, 31);
    unsigned long long base_k = 0, base_a = 0;
    if (lane == 31) {
        if (tot_k) base_k = atomicAdd(args.nkeys, (unsigned long long)tot_k);
        if (tot_a) base_a = atomicAdd(args.namb, (unsigned long long)tot_a);
    }
    unsigned long long wk = __shfl_sync(0xffffffffu, base_k, 31) + (unsigned long long)(inc_k - my_keys);
    unsigned long long wa = __shfl_sync(0xffffffffu, base_a, 31) + (unsigned long long)(inc_a - my_amb);
    if (!(in_mask | amb_mask)) return;
    const uint64_t gi = (uint64_t)et.gi;
#pragma unroll
    for (int jj = 0; jj < 32; ++jj) {
        const uint64_t gj = (uint64_t)et.J * kTM + (uint64_t)(col0 + jj);
        if ((in_mask >> jj) & 1u) {
            if (wk < (unsigned long long)args.key_cap) args.keys[wk] = (gi << 32) | gj;
            ++wk;
            if (!et.diag) {
                if (wk < (unsigned long long)args.key_cap) args.keys[wk] = (gj << 32) | gi;
                ++wk;
            }
        }
        if ((amb_mask >> jj) & 1u) {
            if (wa < (unsigned long long)args.amb_cap) {
                args.amb[wa] = (gi << 32) | gj | (et.diag ? 0ull : (1ull << 63));
                args.amb_d2[wa] = fmaf(-2.f, __uint_as_float(v[jj]), et.ni + norms[jj]);
            }
            ++wa;
        }
    }
}

__global__ void __launch_bounds__(kGramThreads, 1) gram_search_kernel(const __grid_constant__ CUtensorMap map_hi,
                                                                      const __grid_constant__ CUtensorMap map_lo,
                                                                      GramArgs args) {
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    // 1024-byte alignment for the swizzled tiles
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    __shared__ __align__(8) uint64_t full_bar[kStages];
    __shared__ __align__(8) uint64_t empty_bar[kStages];
    __shared__ __align__(8) uint64_t accf_bar[2];
    __shared__ __align__(8) uint64_t acce_bar[2];
    __shared__ __align__(8) uint64_t done_bar;
    __shared__ uint32_t tmem_base_sh;
    __shared__ int abort_sh;
    __shared__ float s_colnorm[8][64];  // per epilogue warp: its 64 column norms

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // contiguous range of tiles for this CTA
    const int64_t per = (args.ntiles + gridDim.x - 1) / gridDim.x;
    const int64_t t_begin = (int64_t)blockIdx.x * per;
    const int64_t t_end = min(args.ntiles, t_begin + per);
    const int64_t my_tiles = t_end > t_begin ? t_end - t_begin : 0;

    if (threadIdx.x == 0) {
        abort_sh = 0;
        for (int s = 0; s < kStages; ++s) {
            mbar_init(&full_bar[s], 1);
            mbar_init(&empty_bar[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&accf_bar[b], 1);
            mbar_init(&acce_bar[b], 8);  // one arrival per epilogue warp
        }
        mbar_init(&done_bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base_sh)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tmem_base = tmem_base_sh;
    volatile int *abort_flag = &abort_sh;

    if (warp == 0) {
        // ---------------- TMA producer ----------------
        if (lane == 0 && my_tiles > 0) {
            int64_t it = 0;  // (tile, k block) iterations
            bool ok = true;
            for (int64_t t = t_begin; t < t_end && ok; ++t) {
                const int2 tile = args.tiles[t];
                const int32_t I = tile.x, J = tile.y;
                for (int32_t kb = 0; kb < args.nkb; ++kb, ++it) {
                    const int s = (int)(it % kStages);
                    const uint32_t ph = (uint32_t)((it / kStages) & 1);
                    if (!mbar_wait(&empty_bar[s], ph ^ 1u, abort_flag)) { ok = false; break; }
                    uint8_t *st = smem + s * kStageBytes;
                    mbar_expect_tx(&full_bar[s], kStageBytes);
                    tma_load_2d(st + 0 * kTileBytes, &map_hi, kb * kKB, I * kTM, &full_bar[s]);
                    tma_load_2d(st + 1 * kTileBytes, &map_lo, kb * kKB, I * kTM, &full_bar[s]);
                    tma_load_2d(st + 2 * kTileBytes, &map_hi, kb * kKB, J * kTM, &full_bar[s]);
                    tma_load_2d(st + 3 * kTileBytes, &map_lo, kb * kKB, J * kTM, &full_bar[s]);
                }
            }
            if (!ok) {
                atomicExch(args.status, 1);
                *abort_flag = 1;
            }
            // drain: every issued stage must have landed before the CTA exits
            const int64_t issued = it;
            for (int64_t k = issued > kStages ? issued - kStages : 0; k < issued; ++k)
                mbar_wait(&full_bar[(int)(k % kStages)], (uint32_t)((k / kStages) & 1), abort_flag);
        }
    } else if (warp == 1) {
        // ---------------- MMA issuer ----------------
        if (lane == 0 && my_tiles > 0) {
            int64_t it = 0;
            bool ok = true;
            for (int64_t tl = 0; tl < my_tiles && ok; ++tl) {
                const int b = (int)(tl & 1);
                const uint32_t acc_ph = (uint32_t)((tl >> 1) & 1);
                if (!mbar_wait(&acce_bar[b], acc_ph ^ 1u, abort_flag)) { ok = false; break; }
                fence_after_sync();
                const uint32_t d_tmem = tmem_base + (uint32_t)(b * kTM);
                for (int32_t kb = 0; kb < args.nkb; ++kb, ++it) {
                    const int s = (int)(it % kStages);
                    const uint32_t ph = (uint32_t)((it / kStages) & 1);
                    if (!mbar_wait(&full_bar[s], ph, abort_flag)) { ok = false; break; }
                    fence_after_sync();
                    const uint32_t st = smem_u32(smem + s * kStageBytes);
#pragma unroll
                    for (int kk = 0; kk < kKB / 16; ++kk) {
                        const uint32_t koff = (uint32_t)kk * 32u;  // 16 bf16 = 32 bytes along K
                        const uint64_t a_hi = smem_desc(st + 0 * kTileBytes + koff);
                        const uint64_t a_lo = smem_desc(st + 1 * kTileBytes + koff);
                        const uint64_t b_hi = smem_desc(st + 2 * kTileBytes + koff);
                        const uint64_t b_lo = smem_desc(st + 3 * kTileBytes + koff);
                        umma(d_tmem, a_hi, b_hi, (kb > 0 || kk > 0) ? 1u : 0u);
                        umma(d_tmem, a_hi, b_lo, 1u);
                        umma(d_tmem, a_lo, b_hi, 1u);
                    }
                    umma_commit(&empty_bar[s]);  // stage free once these MMAs are done
                }
                if (ok) umma_commit(&accf_bar[b]);  // accumulator b complete
            }
            if (!ok) {
                atomicExch(args.status, 2);
                *abort_flag = 1;
            }
            // every MMA this thread issued has finished before TMEM is freed
            umma_commit(&done_bar);
            const uint64_t t0 = globaltimer();
            while (!mbar_try_wait(&done_bar, 0) && globaltimer() - t0 < kWaitNs) {
            }
        }
    } else {
        // ---------------- epilogue (warps 2..9) ----------------
        // two warps per TMEM lane quadrant (so each scheduler has two to
        // alternate between), each owning 64 of the tile's 128 columns
        const int quad = warp & 3;            // TMEM lanes 32*quad .. 32*quad+31
        const int half = (warp - 2) >> 2;     // columns 64*half .. 64*half+63
        const int row_in_tile = quad * 32 + lane;
        float *my_norms = s_colnorm[warp - 2];
        for (int64_t tl = 0; tl < my_tiles; ++tl) {
            const int2 tile = args.tiles[t_begin + tl];
            const int32_t I = tile.x, J = tile.y;
            const int b = (int)(tl & 1);
            const uint32_t acc_ph = (uint32_t)((tl >> 1) & 1);
            if (!mbar_wait(&accf_bar[b], acc_ph, abort_flag)) {
                atomicExch(args.status, 3);
                *abort_flag = 1;
                break;
            }
            fence_after_sync();
            EpilogueTile et;
            et.gi = (int64_t)I * kTM + row_in_tile;
            et.row_ok = et.gi < args.n;
            et.ni = et.row_ok ? args.norm2[et.gi] : 0.f;
            const float band = fmaxf(args.coef * args.blk_norm[I] * args.blk_norm[J] +
                                         args.slack_coef * (args.blk_norm2[I] + args.blk_norm2[J]),
                                     args.min_band);
            et.thr_in = args.rc2 - band;
            et.thr_out = args.rc2 + band;
            et.diag = I == J;
            et.J = J;
            // this warp's 64 column norms, read back as shared broadcasts
            for (int h = 0; h < 2; ++h) {
                const int64_t gj = (int64_t)J * kTM + half * 64 + h * 32 + lane;
                my_norms[h * 32 + lane] = gj < args.n ? args.norm2[gj] : INFINITY;
            }
            __syncwarp();
            const uint32_t taddr =
                tmem_base + ((uint32_t)(quad * 32) << 16) + (uint32_t)(b * kTM + half * 64);
#pragma unroll 1
            for (int c = 0; c < 2; ++c) {
                uint32_t v[32];
                tmem_ld32_async(taddr + (uint32_t)(c * 32), v);
                tmem_wait_ld(v);
                uint32_t in_mask = 0, amb_mask = 0;
#pragma unroll
                for (int jj = 0; jj < 32; ++jj) {
                    const float d2 = fmaf(-2.f, __uint_as_float(v[jj]), et.ni + my_norms[c * 32 + jj]);
                    const bool in = d2 <= et.thr_in;
                    in_mask |= (uint32_t)in << jj;
                    amb_mask |= (uint32_t)(!in && d2 <= et.thr_out) << jj;
                }
                if (!et.row_ok) {
                    in_mask = 0;
                    amb_mask = 0;
                }
                if (__any_sync(0xffffffffu, (in_mask | amb_mask) != 0))
                    epilogue_emit_masks(args, et, v, my_norms + c * 32, half * 64 + c * 32, lane, in_mask,
                                        amb_mask);
            }
            __syncwarp();
            fence_before_sync();
            __syncwarp();
            if (lane == 0) mbar_arrive(&acce_bar[b]);
        }
    }

    fence_before_sync();
    __syncthreads();
    if (warp == 1) {
        fence_after_sync();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base), "r"(kTmemCols)
                     : "memory");
    }
}

// ---- preparation: centring, BF16 split, norms ------------------------------------
__global__ void column_sum_kernel(const double *__restrict__ x, int64_t n, int d, double *__restrict__ sum) {
    const int k = blockIdx.y;
    double s = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double v = x[i * d + k];
        if (isfinite(v)) s += v;
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(&sum[k], s);
}

// One warp per point (internal order i = perm position): split x - mean into
// hi/lo bf16 (K padded with zeros to dp), float32 squared norm, per-block max
// norm (as ordered int bits).
__global__ void gram_prep_kernel(const double *__restrict__ x, int64_t n, int d, int dp,
                                 const double *__restrict__ sum, const int32_t *__restrict__ perm,
                                 __nv_bfloat16 *__restrict__ hi, __nv_bfloat16 *__restrict__ lo,
                                 float *__restrict__ norm2, unsigned *__restrict__ blk_norm_bits,
                                 unsigned *__restrict__ blk_norm2_bits, int *__restrict__ nonfinite) {
    const int lane = threadIdx.x & 31;
    const int64_t i = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    if (i >= n) return;
    const int64_t src = perm[i];
    double s2 = 0;
    bool fin = true;
    for (int k = lane; k < dp; k += 32) {
        float h = 0.f, l = 0.f;
        if (k < d) {
            const double v = x[src * d + k];
            fin = fin && isfinite(v);
            const double c = v - sum[k] / (double)n;
            const float cf = (float)c;
            const __nv_bfloat16 hb = __float2bfloat16_rn(cf);
            h = __bfloat162float(hb);
            l = __bfloat162float(__float2bfloat16_rn((float)(c - (double)h)));
            s2 += c * c;
        }
        hi[i * dp + k] = __float2bfloat16_rn(h);
        lo[i * dp + k] = __float2bfloat16_rn(l);
    }
    for (int o = 16; o > 0; o >>= 1) s2 += __shfl_down_sync(0xffffffffu, s2, o);
    fin = __all_sync(0xffffffffu, fin);
    if (lane == 0) {
        const float n2 = fin ? (float)s2 : INFINITY;
        norm2[i] = n2;
        if (!fin) atomicExch(nonfinite, 1);
        const float nrm = sqrtf(fin ? (float)s2 : 0.f) * (1.f + 1e-6f);
        atomicMax(&blk_norm_bits[i / kTM], __float_as_uint(nrm));
        atomicMax(&blk_norm2_bits[i / kTM], __float_as_uint(fin ? (float)s2 * (1.f + 1e-6f) : 0.f));
    }
}

// ---- tile pruning ---------------------------------------------------------------
// Points are grouped by their nearest pivot (float32, centred coordinates;
// any grouping gives the same result, compact groups let more tiles go).
// One warp per point, lane k holding coordinates k, k+32, k+64, k+96
// (n_dim <= 128); pivots staged in shared memory.
__global__ void pivot_assign_kernel(const double *__restrict__ x, int64_t n, int d, const double *__restrict__ sum,
                                    int32_t n_pivots, int bits_n, uint64_t *__restrict__ keys) {
    extern __shared__ float s_piv[];  // [n_pivots][d]
    const int64_t stride = n / n_pivots;
    for (int e = threadIdx.x; e < n_pivots * d; e += blockDim.x) {
        const int kp = e / d, k = e - kp * d;
        s_piv[e] = (float)(x[(int64_t)kp * stride * d + k] - sum[k] / (double)n);
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int64_t w0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t i = w0; i < n; i += nw) {
        float xc[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const int k = lane + 32 * c;
            xc[c] = k < d ? (float)(x[i * d + k] - sum[k] / (double)n) : 0.f;
        }
        float best = INFINITY;
        int32_t bi = 0;
        for (int kp = 0; kp < n_pivots; ++kp) {
            const float *pv = s_piv + kp * d;
            float acc = 0.f;
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const int k = lane + 32 * c;
                if (k < d) {
                    const float t = xc[c] - pv[k];
                    acc = fmaf(t, t, acc);
                }
            }
            for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
            if (acc < best) {
                best = acc;
                bi = kp;
            }
        }
        if (lane == 0) keys[i] = ((uint64_t)(uint32_t)bi << bits_n) | (uint64_t)i;
    }
}

__global__ void perm_from_keys_kernel(const uint64_t *__restrict__ keys, int64_t n, int bits_n,
                                      int32_t *__restrict__ perm) {
    const uint64_t mask = (1ull << bits_n) - 1;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x)
        perm[p] = (int32_t)(keys[p] & mask);
}

// Per row block (internal order): centroid and radius of its points.
// Float32 values rounded outward enough for the pruning test below.
__global__ void block_bounds_kernel(const double *__restrict__ x, int64_t n, int d, const double *__restrict__ sum,
                                    const int32_t *__restrict__ perm, float *__restrict__ centroid,
                                    float *__restrict__ radius) {
    __shared__ double s_c[128];
    __shared__ double s_r[256];
    const int64_t I = blockIdx.x;
    const int64_t r0 = I * kTM, r1 = min(n, r0 + kTM);
    const int rows = (int)(r1 - r0);
    for (int k = threadIdx.x; k < d; k += blockDim.x) {
        double c = 0;
        for (int r = 0; r < rows; ++r) c += x[(int64_t)perm[r0 + r] * d + k] - sum[k] / (double)n;
        s_c[k] = c / rows;
        centroid[I * d + k] = (float)s_c[k];
    }
    __syncthreads();
    double m = 0;
    for (int r = threadIdx.x; r < rows; r += blockDim.x) {
        double s = 0;
        const int64_t src = perm[r0 + r];
        for (int k = 0; k < d; ++k) {
            // distance to the float32 centroid actually used in the test
            const double t = (x[src * d + k] - sum[k] / (double)n) - (double)(float)s_c[k];
            s += t * t;
        }
        m = fmax(m, s);
    }
    s_r[threadIdx.x] = m;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) s_r[threadIdx.x] = fmax(s_r[threadIdx.x], s_r[threadIdx.x + w]);
        __syncthreads();
    }
    if (threadIdx.x == 0) radius[I] = (float)(sqrt(s_r[0]) * (1.0 + 1e-6) + 1e-30);
}

// Can blocks I and J (J >= I) hold a pair within R?  |c_I - c_J| - rho_I -
// rho_J > R means every pair is farther than R (triangle inequality); the
// margin covers the float32 evaluation of the centroid distance.
__device__ __forceinline__ bool blocks_may_touch(const float *__restrict__ centroid, const float *__restrict__ radius,
                                                 int d, int64_t I, int64_t J, float R) {
    if (I == J) return true;
    const float *a = centroid + I * d, *b = centroid + J * d;
    float s = 0.f, na = 0.f, nb = 0.f;
    for (int k = 0; k < d; ++k) {
        const float t = a[k] - b[k];
        s = fmaf(t, t, s);
        na = fmaf(a[k], a[k], na);
        nb = fmaf(b[k], b[k], nb);
    }
    const float margin = 1e-5f * (sqrtf(na) + sqrtf(nb) + radius[I] + radius[J] + R);
    return sqrtf(s) - radius[I] - radius[J] <= R + margin;
}

// Row I of the tile triangle: count (pass 1) or write (pass 2) its kept J.
template <bool kWrite>
__global__ void tile_list_kernel(const float *__restrict__ centroid, const float *__restrict__ radius, int d,
                                 int64_t nblk, float R, int32_t *__restrict__ row_count,
                                 const int64_t *__restrict__ row_off, int2 *__restrict__ tiles) {
    __shared__ int32_t s_cnt;
    const int64_t I = blockIdx.x;
    if (threadIdx.x == 0) s_cnt = 0;
    __syncthreads();
    for (int64_t J = I + threadIdx.x; J < nblk; J += blockDim.x) {
        if (blocks_may_touch(centroid, radius, d, I, J, R)) {
            const int32_t k = atomicAdd(&s_cnt, 1);
            if (kWrite) tiles[row_off[I] + k] = make_int2((int32_t)I, (int32_t)J);
        }
    }
    __syncthreads();
    if (!kWrite && threadIdx.x == 0) row_count[I] = s_cnt;
}

// internal indices -> point indices in the key lists (bit 63 kept)
__global__ void map_keys_kernel(uint64_t *__restrict__ keys, const unsigned long long *__restrict__ count,
                                int64_t cap, const int32_t *__restrict__ perm) {
    const int64_t nk = min((int64_t)*count, cap);
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nk; e += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t k = keys[e];
        const uint64_t flag = k & (1ull << 63);
        const uint64_t a = (k >> 32) & 0x7fffffffull, b = k & 0xffffffffull;
        keys[e] = flag | ((uint64_t)(uint32_t)perm[a] << 32) | (uint64_t)(uint32_t)perm[b];
    }
}

// Band pairs in float64, reference order; hits appended to the key list.
__global__ void gram_recheck_kernel(const double *__restrict__ x, int d, const uint64_t *__restrict__ amb,
                                    const unsigned long long *__restrict__ namb, int64_t amb_cap, double rc,
                                    int metric, int fpmode, uint64_t *__restrict__ keys,
                                    unsigned long long *__restrict__ nkeys, int64_t key_cap,
                                    const float *__restrict__ amb_d2, unsigned *__restrict__ max_err_bits) {
    const int64_t total = min((int64_t)*namb, amb_cap);
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t a = amb[e];
        const bool both = (a >> 63) & 1ull;
        const int64_t i = (int64_t)((a >> 32) & 0x7fffffffull), j = (int64_t)(a & 0xffffffffull);
        double s = 0.0;
        const double *xa = x + i * d, *xb = x + j * d;
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
        const double sv = metric == CNN_METRIC_EUCLIDEAN ? __dsqrt_rn(s) : s;
        if (sv <= rc) {
            const unsigned long long w = atomicAdd(nkeys, both ? 2ull : 1ull);
            if (w < (unsigned long long)key_cap) keys[w] = ((uint64_t)i << 32) | (uint64_t)j;
            if (both && w + 1 < (unsigned long long)key_cap) keys[w + 1] = ((uint64_t)j << 32) | (uint64_t)i;
        }
        const float err = fabsf((float)(s - (double)amb_d2[e]));
        atomicMax(max_err_bits, __float_as_uint(err));
    }
}

__global__ void keys_rows_kernel(const uint64_t *__restrict__ keys, int64_t nk, int32_t *__restrict__ deg,
                                 int32_t *__restrict__ cols) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nk; e += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t k = keys[e];
        atomicAdd(&deg[(int64_t)(k >> 32)], 1);
        cols[e] = (int32_t)(k & 0xffffffffull);
    }
}

typedef CUresult (*PFN_encodeTiled)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                    const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                    CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

PFN_encodeTiled get_encode_fn() {
    static PFN_encodeTiled fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPoint("cuTensorMapEncodeTiled", &p, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_encodeTiled>(p);
        (void)cudaGetLastError();
    }
    return fn;
}

bool make_map(CUtensorMap *map, void *base, int64_t rows, int dp) {
    PFN_encodeTiled enc = get_encode_fn();
    if (!enc) return false;
    const cuuint64_t dims[2] = {(cuuint64_t)dp, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)dp * 2};
    const cuuint32_t box[2] = {(cuuint32_t)kKB, (cuuint32_t)kTM};
    const cuuint32_t estr[2] = {1, 1};
    return enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

// Error bound on |acc - x'.y'| relative to |x'||y'|: the split leaves at most
// 2^-16 |x_k| per coordinate and drops lo.lo (<= 2^-16 |x_k||y_k|): about
// 3.1 * 2^-16 overall; FP32 accumulation of 3*dp exact products adds at most
// (3 dp + 8) 2^-23.  d2 uses 2*acc, so the band coefficient doubles both.
// Taken with a safety factor of 2.
double gram_band_coef(int dp) { return 2.0 * 2.0 * (3.2 * ldexp(1.0, -16) + (3.0 * dp + 8.0) * ldexp(1.0, -23)); }

cnn_status gram_search_impl(cnn_context *ctx, double radius_cutoff, int metric, int fpmode, bool *used) {
    *used = false;
    const int64_t n = ctx->n;
    const int d = ctx->d;
    cudaStream_t st = ctx->stream;
    if (n < 1 || d < 16 || n >= (int64_t(1) << 31) - 256) return CNN_OK;
    if (!(radius_cutoff >= 0.0) || !isfinite(radius_cutoff)) return CNN_OK;
    if (!get_encode_fn()) return CNN_OK;
    int dev = 0, major = 0, minor = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
    cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
    (void)cudaGetLastError();
    if (major != 10 || minor != 3) return CNN_OK;  // tcgen05 code is built for sm_103a only

    const int dp = (d + kKB - 1) / kKB * kKB;
    const int nkb = dp / kKB;
    const int64_t nblk = (n + kTM - 1) / kTM;
    const double rc2 = metric == CNN_METRIC_EUCLIDEAN ? radius_cutoff * radius_cutoff : radius_cutoff;

    // buffers: hi, lo (bf16 n x dp), norm2 (n), block norms, counters
    CNN_TRY(ctx->ensure(ctx->gram_hi, sizeof(__nv_bfloat16) * (size_t)n * dp));
    CNN_TRY(ctx->ensure(ctx->gram_lo, sizeof(__nv_bfloat16) * (size_t)n * dp));
    CNN_TRY(ctx->ensure(ctx->gram_aux, sizeof(float) * (size_t)(n + 2 * nblk + 64) + sizeof(double) * (size_t)d + 256));
    float *norm2 = ctx->gram_aux.as<float>();
    unsigned *blk_norm_bits = reinterpret_cast<unsigned *>(norm2 + n);
    unsigned *blk_norm2_bits = blk_norm_bits + nblk;
    double *colsum = reinterpret_cast<double *>(
        (reinterpret_cast<uintptr_t>(blk_norm2_bits + nblk + 16) + 15) & ~uintptr_t(15));
    unsigned long long *counters = ctx->counters.as<unsigned long long>();
    unsigned long long *nkeys = counters + 10, *namb = counters + 11;
    int *status = reinterpret_cast<int *>(counters + 12);
    int *nonfinite = reinterpret_cast<int *>(counters + 13);
    unsigned *max_err_bits = reinterpret_cast<unsigned *>(counters + 14);
    CNN_CUDA(ctx, cudaMemsetAsync(counters + 10, 0, 4 * sizeof(unsigned long long), st));
    CNN_CUDA(ctx, cudaMemsetAsync(blk_norm_bits, 0, sizeof(unsigned) * 2 * (size_t)nblk, st));
    CNN_CUDA(ctx, cudaMemsetAsync(colsum, 0, sizeof(double) * d, st));
    {
        const int blocks = (int)std::min<int64_t>(256, (n + 255) / 256);
        column_sum_kernel<<<dim3(blocks, d), 256, 0, st>>>(ctx->x, n, d, colsum);
        CNN_LAUNCH_CHECK(ctx);
    }
    // internal order: points grouped by nearest pivot, so that 128-point
    // blocks are compact and far-apart block pairs can be skipped
    const int bits_n = [&] { int b = 1; while (b < 62 && (int64_t(1) << b) < n) ++b; return b; }();
    const bool prune = d <= 128 && n >= 8 * kTM;
    int32_t *perm = ctx->perm.as<int32_t>();
    if (prune) {
        const int n_pivots = (int)std::max<int64_t>(1, std::min<int64_t>({512, n / 1024, 98304 / (4 * d)}));
        CNN_TRY(ctx->ensure(ctx->scratch_a, sizeof(uint64_t) * (size_t)n));
        uint64_t *pkeys = ctx->scratch_a.as<uint64_t>();
        const size_t psmem = sizeof(float) * (size_t)n_pivots * d;
        CNN_CUDA(ctx, cudaFuncSetAttribute(pivot_assign_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)psmem));
        pivot_assign_kernel<<<152 * 4, 256, psmem, st>>>(ctx->x, n, d, colsum, n_pivots, bits_n, pkeys);
        CNN_LAUNCH_CHECK(ctx);
        int pb = 1;
        while ((1 << pb) < n_pivots) ++pb;
        CNN_TRY(radix_sort_u64(ctx, pkeys, n, bits_n + pb));
        perm_from_keys_kernel<<<std::min<unsigned>(grid_for(n, 256), 4096u), 256, 0, st>>>(pkeys, n, bits_n, perm);
        CNN_LAUNCH_CHECK(ctx);
    } else {
        CNN_TRY(iota_i32(ctx, perm, n));
    }
    gram_prep_kernel<<<grid_for(n * 32, 256), 256, 0, st>>>(ctx->x, n, d, dp, colsum, perm,
                                                            ctx->gram_hi.as<__nv_bfloat16>(),
                                                            ctx->gram_lo.as<__nv_bfloat16>(), norm2, blk_norm_bits,
                                                            blk_norm2_bits, nonfinite);
    CNN_LAUNCH_CHECK(ctx);
    int h_nonfinite = 0;
    CNN_CUDA(ctx, cudaMemcpyAsync(&h_nonfinite, nonfinite, sizeof(int), cudaMemcpyDeviceToHost, st));
    CNN_CUDA(ctx, cudaStreamSynchronize(st));
    if (h_nonfinite) return CNN_OK;  // non-finite coordinates: the all-pairs path handles them

    // the list of block pairs (I, J >= I) that can hold a pair within R
    const double Rsearch = (metric == CNN_METRIC_EUCLIDEAN ? radius_cutoff : sqrt(radius_cutoff)) * (1.0 + 1e-6);
    CNN_TRY(ctx->ensure(ctx->gram_blocks, sizeof(float) * (size_t)nblk * (d + 1) +
                                              (sizeof(int32_t) + sizeof(int64_t)) * (size_t)(nblk + 1) + 256));
    float *centroid = ctx->gram_blocks.as<float>();
    float *bradius = centroid + nblk * d;
    int32_t *row_count = reinterpret_cast<int32_t *>(bradius + nblk);
    int64_t *row_off = reinterpret_cast<int64_t *>(
        (reinterpret_cast<uintptr_t>(row_count + nblk + 1) + 15) & ~uintptr_t(15));
    const float Rf = prune ? (float)Rsearch : INFINITY;
    if (prune) {
        block_bounds_kernel<<<(unsigned)nblk, 256, 0, st>>>(ctx->x, n, d, colsum, perm, centroid, bradius);
        CNN_LAUNCH_CHECK(ctx);
    } else {
        CNN_CUDA(ctx, cudaMemsetAsync(centroid, 0, sizeof(float) * (size_t)nblk * (d + 1), st));
    }
    tile_list_kernel<false><<<(unsigned)nblk, 256, 0, st>>>(centroid, bradius, d, nblk, Rf, row_count, nullptr,
                                                             nullptr);
    CNN_LAUNCH_CHECK(ctx);
    CNN_CUDA(ctx, cudaMemsetAsync(row_count + nblk, 0, sizeof(int32_t), st));
    CNN_TRY(scan_exclusive_i32_to_i64(ctx, row_count, row_off, nblk + 1));
    int64_t ntiles = 0;
    CNN_CUDA(ctx, cudaMemcpyAsync(&ntiles, row_off + nblk, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    CNN_CUDA(ctx, cudaStreamSynchronize(st));
    CNN_TRY(ctx->ensure(ctx->gram_tiles, sizeof(int2) * (size_t)(ntiles > 0 ? ntiles : 1)));
    tile_list_kernel<true><<<(unsigned)nblk, 256, 0, st>>>(centroid, bradius, d, nblk, Rf, nullptr, row_off,
                                                            ctx->gram_tiles.as<int2>());
    CNN_LAUNCH_CHECK(ctx);

    CUtensorMap map_hi, map_lo;
    if (!make_map(&map_hi, ctx->gram_hi.ptr, n, dp) || !make_map(&map_lo, ctx->gram_lo.ptr, n, dp))
        return CNN_OK;

    const double coef = gram_band_coef(dp);
    GramArgs a{};
    a.n = n;
    a.nkb = nkb;
    a.nblk = (int32_t)nblk;
    a.ntiles = ntiles;
    a.tiles = ctx->gram_tiles.as<int2>();
    a.rc2 = (float)rc2;
    a.coef = (float)coef;
    a.slack_coef = (float)(8.0 * ldexp(1.0, -24));  // float32 rounding of |x|^2, |y|^2 and the fma
    a.min_band = (float)(1e-3 * rc2);
    a.norm2 = norm2;
    a.blk_norm = reinterpret_cast<const float *>(blk_norm_bits);
    a.blk_norm2 = reinterpret_cast<const float *>(blk_norm2_bits);
    a.status = status;
    // the float32 threshold must itself be an upper/lower bound of rc2
    int64_t key_cap = std::max<int64_t>(ctx->gram_key_hint, std::min<int64_t>(n * 256, int64_t(1) << 31));
    const int64_t amb_cap = std::max<int64_t>(int64_t(1) << 22, n * 64);
    const int sms = 152;
    int dev_sms = 0;
    cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, dev);
    const int grid = (int)std::min<int64_t>(ntiles, dev_sms > 0 ? dev_sms : sms);
    const size_t smem = (size_t)kStages * kStageBytes + 1024;
    CNN_CUDA(ctx, cudaFuncSetAttribute(gram_search_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    for (int attempt = 0; attempt < 2; ++attempt) {
        CNN_TRY(ctx->ensure(ctx->gram_keys, sizeof(uint64_t) * (size_t)key_cap));
        CNN_TRY(ctx->ensure(ctx->gram_amb, (sizeof(uint64_t) + sizeof(float)) * (size_t)amb_cap));
        a.keys = ctx->gram_keys.as<uint64_t>();
        a.key_cap = key_cap;
        a.amb = ctx->gram_amb.as<uint64_t>();
        a.amb_d2 = reinterpret_cast<float *>(a.amb + amb_cap);
        a.amb_cap = amb_cap;
        a.nkeys = nkeys;
        a.namb = namb;
        CNN_CUDA(ctx, cudaMemsetAsync(counters + 10, 0, 3 * sizeof(unsigned long long), st));
        CNN_CUDA(ctx, cudaMemsetAsync(max_err_bits, 0, sizeof(unsigned), st));
        stage_begin(ctx, 9);
        gram_search_kernel<<<grid, kGramThreads, smem, st>>>(map_hi, map_lo, a);
        CNN_LAUNCH_CHECK(ctx);
        stage_end(ctx, 9);
        // internal indices -> point indices (before the recheck appends more keys)
        map_keys_kernel<<<152u * 8u, 256, 0, st>>>(a.keys, nkeys, key_cap, perm);
        CNN_LAUNCH_CHECK(ctx);
        map_keys_kernel<<<152u * 8u, 256, 0, st>>>(a.amb, namb, amb_cap, perm);
        CNN_LAUNCH_CHECK(ctx);
        gram_recheck_kernel<<<std::min<unsigned>(grid_for(amb_cap, 256), 152u * 8u), 256, 0, st>>>(
            ctx->x, d, a.amb, namb, amb_cap, radius_cutoff, metric, fpmode, a.keys, nkeys, key_cap, a.amb_d2,
            max_err_bits);
        CNN_LAUNCH_CHECK(ctx);
        unsigned long long hc[3];
        CNN_CUDA(ctx, cudaMemcpyAsync(hc, counters + 10, sizeof(hc), cudaMemcpyDeviceToHost, st));
        CNN_CUDA(ctx, cudaStreamSynchronize(st));
        int h_status = (int)(hc[2] & 0xffffffffull);
        if (h_status != 0) return ctx->fail(CNN_ERR_TIMEOUT, "tensor-core distance kernel timed out on a barrier");
        if ((int64_t)hc[1] > amb_cap) return CNN_OK;  // too many band pairs: the all-pairs path decides
        if ((int64_t)hc[0] <= key_cap) {
            const int64_t nk = (int64_t)hc[0];
            ctx->gram_key_hint = nk + nk / 8 + 1024;
            ctx->stats.n_exact = (int64_t)hc[1];
            unsigned me = 0;
            CNN_CUDA(ctx, cudaMemcpy(&me, max_err_bits, sizeof(unsigned), cudaMemcpyDeviceToHost));
            float mef;
            memcpy(&mef, &me, sizeof(float));
            ctx->stats.max_abs_err = mef;
            ctx->stats.n_candidates = ntiles * kTM * kTM;
            ctx->stats.filter_band = std::max(coef, 0.0);
            ctx->stats.filter_enabled = 1;
            // CSR: sort keys by (row, col), rows from the high half
            CNN_TRY(radix_sort_u64(ctx, a.keys, nk, 32 + bits_n));
            CNN_TRY(ctx->ensure(ctx->cols, sizeof(int32_t) * (size_t)(nk > 0 ? nk : 1)));
            int32_t *deg = ctx->deg.as<int32_t>();
            CNN_CUDA(ctx, cudaMemsetAsync(deg, 0, sizeof(int32_t) * (size_t)(n + 1), st));
            keys_rows_kernel<<<std::min<unsigned>(grid_for(nk, 256), 152u * 16u), 256, 0, st>>>(
                a.keys, nk, deg, ctx->cols.as<int32_t>());
            CNN_LAUNCH_CHECK(ctx);
            CNN_TRY(scan_exclusive_i32_to_i64(ctx, deg, ctx->row_off.as<int64_t>(), n + 1));
            ctx->nnz = nk;
            *used = true;
            return CNN_OK;
        }
        key_cap = (int64_t)hc[0] + 1024;  // exact size now known: run once more
    }
    return CNN_OK;
}

}  // namespace cnn
