// gram.cu -- radius neighbour search for n_dim >= 16 on the tensor cores.
//
// Squared distances come from the Gram matrix: d2(i,j) = |x_i|^2 + |x_j|^2
// - 2 x_i.x_j, on mean-centred coordinates.  x_i.x_j is computed on the 5th
// generation tensor cores (tcgen05.mma, kind::f16) from a BF16 split of
// every coordinate, x = hi + mid + lo with hi = bf16(x), mid = bf16(x - hi),
// lo = bf16(x - hi - mid): x.y ~ hi.hi + (hi.mid + mid.hi + hi.lo + lo.hi +
// mid.mid) (six MMAs per 16-wide K slice), FP32 accumulation in tensor
// memory, hi.hi and the small cross terms in separate accumulators so that
// the accumulation error scales with dp, not 6 dp.  Per tile (128 x 128 pairs) a rigorous
// error bound gives a band around the cutoff: pairs below it are
// neighbours, pairs above are not, pairs inside are recomputed in float64
// with the reference's exact operation order (the only float64 step).
//
// Kernel structure (one persistent CTA per SM, 10 warps):
//   warp 0  TMA producer: hi/mid/lo tiles of the row block I and the column
//           block J (cp.async.bulk.tensor, 128-byte swizzle) into a 2-stage
//           shared-memory ring, completion counted on an mbarrier;
//   warp 1  allocates 512 TMEM columns (two buffers, each a 128-column hi.hi
//           accumulator and a 128-column cross-term accumulator) and issues
//           the MMAs from one thread; tcgen05.commit frees the shared stage
//           and publishes the accumulator;
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

// Upper bound of the pivot groups that order the rows for tile pruning.  The
// pivots are every (n / groups)-th point: too few of them leave natural
// clusters without a pivot and the blocks loose; each costs n x d FMAs.
constexpr int64_t kMaxGroups = 256;

constexpr int kTM = 128;              // tile rows (M) = tile columns (N)
constexpr int kMaskWords = kTM * kTM / 32;  // a tile's hit mask: row r, column c = word r * 4 + c / 32, bit c % 32
constexpr int kKB = 64;               // K block: 64 bf16 = 128 bytes per row
constexpr int kStages = 2;
constexpr int kTileBytes = kTM * kKB * 2;          // 16 KB: one operand tile
constexpr int kSplits = 3;                          // x = hi + mid + lo (bf16 each)
constexpr int kStageBytes = 2 * kSplits * kTileBytes;  // A_hi, A_mid, A_lo, B_hi, B_mid, B_lo: 96 KB
constexpr int kGramThreads = 320;  // warp 0 TMA, warp 1 MMA, warps 2-9 epilogue
constexpr uint32_t kAccCols = 256;   // per accumulator buffer: hi.hi (128 columns), then the cross terms (128)
constexpr uint32_t kTmemCols = 512;  // two buffers
constexpr unsigned long long kWaitNs = 2000000000ull;   // default limit of a pipeline wait (2 s)
constexpr unsigned long long kDrainNs = 2000000000ull;  // limit of the drains before exit (copies, MMAs)

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
    uint32_t *masks;        // per listed tile: 128 rows x 4 words, bit = neighbour (kMaskWords per tile)
    uint64_t *amb;          // band pairs (padded row << 32 | padded col); bit 63: off-diagonal tile
    float *amb_d2;          // their float32 squared distance
    unsigned long long *namb;
    int64_t amb_cap;
    int *status;            // nonzero on a timed-out wait
    unsigned long long wait_ns;  // limit of every pipeline wait (nanoseconds)
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

// Bounded wait on an mbarrier phase.  Returns false after limit_ns or when
// another warp has already given up (abort flag in shared memory).
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, volatile int *abort_flag,
                                          unsigned long long limit_ns) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = globaltimer();
    for (;;) {
        if (mbar_try_wait(bar, parity)) return true;
        if (*abort_flag) return false;
        if (globaltimer() - t0 > limit_ns) return false;
        __nanosleep(32);  // back off: waiting warps leave issue slots and shared-memory bandwidth
    }
}

// Wait for a phase that is certain to complete (copies already issued), also
// after an abort: the CTA may not exit while a copy still writes its shared
// memory.  Bounded by kDrainNs all the same.
__device__ __forceinline__ void mbar_drain(uint64_t *bar, uint32_t parity) {
    const uint64_t t0 = globaltimer();
    while (!mbar_try_wait(bar, parity) && globaltimer() - t0 < kDrainNs) __nanosleep(32);
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

// Band pairs of a 32-column chunk with at least one somewhere in the warp:
// one warp-wide atomic reserves the slots, then each thread writes its own,
// visiting only the set bits of its mask.  A band pair's accumulator value
// is picked from the 32 registers with an unrolled select, so the registers
// are never indexed dynamically (which would move them to local memory).
// Neighbours need no list: the chunk's hit bits go to the tile mask.
__device__ __forceinline__ void epilogue_emit_band(const GramArgs &args, const EpilogueTile &et,
                                                   const uint32_t (&v)[32], const float *norms, int col0, int lane,
                                                   uint32_t amb_mask) {
    const int my_amb = __popc(amb_mask);
    int inc_a = my_amb;
    for (int o = 1; o < 32; o <<= 1) {
        const int ua = __shfl_up_sync(0xffffffffu, inc_a, o);
        if (lane >= o) inc_a += ua;
    }
    const int tot_a = __shfl_sync(0xffffffffu, inc_a, 31);
    unsigned long long base_a = 0;
    if (lane == 31 && tot_a) base_a = atomicAdd(args.namb, (unsigned long long)tot_a);
    unsigned long long wa = __shfl_sync(0xffffffffu, base_a, 31) + (unsigned long long)(inc_a - my_amb);
    const uint64_t gi = (uint64_t)et.gi;
    const uint64_t gj0 = (uint64_t)et.J * kTM + (uint64_t)col0;
    const unsigned long long acap = (unsigned long long)args.amb_cap;
    for (uint32_t m = amb_mask; m; m &= m - 1) {
        const int jj = __ffs(m) - 1;
        uint32_t acc = 0;
#pragma unroll
        for (int u = 0; u < 32; ++u) acc = u == jj ? v[u] : acc;
        if (wa < acap) {
            args.amb[wa] = (gi << 32) | (gj0 + (uint64_t)jj) | (et.diag ? 0ull : (1ull << 63));
            args.amb_d2[wa] = fmaf(-2.f, __uint_as_float(acc), et.ni + norms[jj]);
        }
        ++wa;
    }
}

__global__ void __launch_bounds__(kGramThreads, 1) gram_search_kernel(const __grid_constant__ CUtensorMap map_hi,
                                                                      const __grid_constant__ CUtensorMap map_mid,
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
                    if (!mbar_wait(&empty_bar[s], ph ^ 1u, abort_flag, args.wait_ns)) { ok = false; break; }
                    uint8_t *st = smem + s * kStageBytes;
                    mbar_expect_tx(&full_bar[s], kStageBytes);
                    tma_load_2d(st + 0 * kTileBytes, &map_hi, kb * kKB, I * kTM, &full_bar[s]);
                    tma_load_2d(st + 1 * kTileBytes, &map_mid, kb * kKB, I * kTM, &full_bar[s]);
                    tma_load_2d(st + 2 * kTileBytes, &map_lo, kb * kKB, I * kTM, &full_bar[s]);
                    tma_load_2d(st + 3 * kTileBytes, &map_hi, kb * kKB, J * kTM, &full_bar[s]);
                    tma_load_2d(st + 4 * kTileBytes, &map_mid, kb * kKB, J * kTM, &full_bar[s]);
                    tma_load_2d(st + 5 * kTileBytes, &map_lo, kb * kKB, J * kTM, &full_bar[s]);
                }
            }
            if (!ok) {
                atomicExch(args.status, 1);
                *abort_flag = 1;
            }
            // drain: every issued stage must have landed before the CTA exits
            // (not abortable: the copies complete whatever the other warps do)
            const int64_t issued = it;
            for (int64_t k = issued > kStages ? issued - kStages : 0; k < issued; ++k)
                mbar_drain(&full_bar[(int)(k % kStages)], (uint32_t)((k / kStages) & 1));
        }
    } else if (warp == 1) {
        // ---------------- MMA issuer ----------------
        if (lane == 0 && my_tiles > 0) {
            int64_t it = 0;
            bool ok = true;
            for (int64_t tl = 0; tl < my_tiles && ok; ++tl) {
                const int b = (int)(tl & 1);
                const uint32_t acc_ph = (uint32_t)((tl >> 1) & 1);
                if (!mbar_wait(&acce_bar[b], acc_ph ^ 1u, abort_flag, args.wait_ns)) { ok = false; break; }
                fence_after_sync();
                const uint32_t d_hh = tmem_base + (uint32_t)(b * kAccCols);  // hi.hi
                const uint32_t d_x = d_hh + (uint32_t)kTM;                      // cross terms
                for (int32_t kb = 0; kb < args.nkb; ++kb, ++it) {
                    const int s = (int)(it % kStages);
                    const uint32_t ph = (uint32_t)((it / kStages) & 1);
                    if (!mbar_wait(&full_bar[s], ph, abort_flag, args.wait_ns)) { ok = false; break; }
                    fence_after_sync();
                    const uint32_t st = smem_u32(smem + s * kStageBytes);
#pragma unroll
                    for (int kk = 0; kk < kKB / 16; ++kk) {
                        const uint32_t koff = (uint32_t)kk * 32u;  // 16 bf16 = 32 bytes along K
                        const uint64_t a_h = smem_desc(st + 0 * kTileBytes + koff);
                        const uint64_t a_m = smem_desc(st + 1 * kTileBytes + koff);
                        const uint64_t a_l = smem_desc(st + 2 * kTileBytes + koff);
                        const uint64_t b_h = smem_desc(st + 3 * kTileBytes + koff);
                        const uint64_t b_m = smem_desc(st + 4 * kTileBytes + koff);
                        const uint64_t b_l = smem_desc(st + 5 * kTileBytes + koff);
                        const uint32_t acc = (kb > 0 || kk > 0) ? 1u : 0u;
                        umma(d_hh, a_h, b_h, acc);
                        umma(d_x, a_h, b_m, acc);
                        umma(d_x, a_m, b_h, 1u);
                        umma(d_x, a_h, b_l, 1u);
                        umma(d_x, a_l, b_h, 1u);
                        umma(d_x, a_m, b_m, 1u);
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
            mbar_drain(&done_bar, 0);
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
            if (!mbar_wait(&accf_bar[b], acc_ph, abort_flag, args.wait_ns)) {
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
                tmem_base + ((uint32_t)(quad * 32) << 16) + (uint32_t)(b * kAccCols + half * 64);
#pragma unroll 1
            for (int c = 0; c < 2; ++c) {
                uint32_t v[32], vx[32];
                tmem_ld32_async(taddr + (uint32_t)(c * 32), v);         // hi.hi
                tmem_ld32_async(taddr + (uint32_t)(kTM + c * 32), vx);  // cross terms
                tmem_wait_ld(v);
                tmem_wait_ld(vx);
#pragma unroll
                for (int jj = 0; jj < 32; ++jj) v[jj] = __float_as_uint(__uint_as_float(v[jj]) + __uint_as_float(vx[jj]));
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
                // every word of every listed tile's mask is written here
                args.masks[(size_t)(t_begin + tl) * kMaskWords + row_in_tile * 4 + half * 2 + c] = in_mask;
                if (__any_sync(0xffffffffu, amb_mask != 0))
                    epilogue_emit_band(args, et, v, my_norms + c * 32, half * 64 + c * 32, lane, amb_mask);
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
// Column sums of the finite coordinates; *nonfinite set if any coordinate is
// not.  The array is read flat and coalesced: the block size is a multiple of
// n_dim and so is the grid stride, so every thread stays on one column
// (threadIdx.x % n_dim); the block adds its threads' sums per column.
__global__ void column_sum_kernel(const double *__restrict__ x, int64_t n, int d, double *__restrict__ sum,
                                  int *__restrict__ nonfinite) {
    extern __shared__ double s_part[];  // [blockDim.x]
    const int64_t total = n * d;
    double acc = 0;
    bool fin = true;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        const double v = x[e];
        if (isfinite(v)) acc += v;
        else fin = false;
    }
    s_part[threadIdx.x] = acc;
    // block-wide (the block size need not be a multiple of 32); also the barrier for s_part
    if (__syncthreads_or(!fin) && threadIdx.x == 0) atomicExch(nonfinite, 1);
    for (int k = threadIdx.x; k < d; k += blockDim.x) {
        double t = 0;
        for (int i = k; i < (int)blockDim.x; i += d) t += s_part[i];
        atomicAdd(&sum[k], t);
    }
}

__global__ void column_mean_kernel(double *__restrict__ sum, int d, int64_t n) {
    for (int k = threadIdx.x; k < d; k += blockDim.x) sum[k] = sum[k] / (double)n;
}

// One warp per row of the padded internal order (perm[i] = point index, -1
// for an empty row): split x - mean into hi/lo bf16 (K padded with zeros to
// dp), float32 squared norm (+inf for an empty row), per-block max norm (as
// ordered int bits).  All coordinates are finite here.
// Three-way bf16 split of a centred coordinate c, in float32: cf = (float)c
// is within 2^-24 |c|; hi = bf16(cf) and the residuals cf - hi and
// (cf - hi) - mid are exact in float32 (each operand pair within a factor
// of 2), so hi + mid + lo misses cf by the last bf16 rounding only,
// 2^-9 |(cf - hi) - mid| <= 2^-27 |cf|.  One float64 operation per
// coordinate remains (the centring); GB300's float64 rate is low.
__device__ __forceinline__ void split3(double c, __nv_bfloat16 &bh, __nv_bfloat16 &bm, __nv_bfloat16 &bl) {
    const float cf = (float)c;
    bh = __float2bfloat16_rn(cf);
    const float r1 = cf - __bfloat162float(bh);
    bm = __float2bfloat16_rn(r1);
    const float r2 = r1 - __bfloat162float(bm);
    bl = __float2bfloat16_rn(r2);
}

__global__ void gram_prep_kernel(const double *__restrict__ x, int64_t n_rows, int64_t n, int d, int dp,
                                 const double *__restrict__ mean, const int32_t *__restrict__ perm,
                                 __nv_bfloat16 *__restrict__ hi, __nv_bfloat16 *__restrict__ mid,
                                 __nv_bfloat16 *__restrict__ lo, float *__restrict__ norm2,
                                 unsigned *__restrict__ blk_norm_bits, unsigned *__restrict__ blk_norm2_bits) {
    const int lane = threadIdx.x & 31;
    const int64_t i = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    if (i >= n_rows) return;
    const int64_t src = perm[i];
    double s2 = 0;
    for (int k = lane; k < dp; k += 32) {
        __nv_bfloat16 bh = __float2bfloat16_rn(0.f), bm = bh, bl = bh;
        if (k < d && src >= 0) {
            const double c = x[src * d + k] - mean[k];
            split3(c, bh, bm, bl);
            s2 = fma(c, c, s2);
        }
        hi[i * dp + k] = bh;
        mid[i * dp + k] = bm;
        lo[i * dp + k] = bl;
    }
    for (int o = 16; o > 0; o >>= 1) s2 += __shfl_down_sync(0xffffffffu, s2, o);
    if (lane == 0) {
        if (src < 0) {
            norm2[i] = INFINITY;
        } else {
            norm2[i] = (float)s2;
            const float nrm = sqrtf((float)s2) * (1.f + 1e-6f);
            atomicMax(&blk_norm_bits[i / kTM], __float_as_uint(nrm));
            atomicMax(&blk_norm2_bits[i / kTM], __float_as_uint((float)s2 * (1.f + 1e-6f)));
        }
    }
}

// One block per 128-row block of the padded internal order: every row split
// as in gram_prep_kernel (float64 centring, exact residuals), its float32
// norm, the block's norm maxima, and -- for the tile pruning -- the block's
// float32 centroid (stored transposed, [d][nblk]) and a radius that bounds the distance of every point of
// the block to it: the float32 evaluation from the float32 coordinates,
// inflated by its rounding ((d + 8) 2^-23 relative) and by the conversion
// of the coordinates (2^-24 of the largest norm, taken twice).
constexpr int kPrepWarps = 16;

__global__ void __launch_bounds__(kPrepWarps * 32) gram_prep_bounds_kernel(
    const double *__restrict__ x, int64_t n_rows, int d, int dp, const double *__restrict__ mean,
    const int32_t *__restrict__ perm, __nv_bfloat16 *__restrict__ hi, __nv_bfloat16 *__restrict__ mid,
    __nv_bfloat16 *__restrict__ lo, float *__restrict__ norm2, unsigned *__restrict__ blk_norm_bits,
    unsigned *__restrict__ blk_norm2_bits, int bounds, int64_t nblk, float *__restrict__ centroid_t,
    float *__restrict__ radius) {
    extern __shared__ float s_cf[];  // [kTM][d + 1] float32 coordinates, then [d] centroid
    __shared__ float s_max[kPrepWarps][2];
    __shared__ int s_used[kPrepWarps];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int ld = d + 1;
    float *s_cent = s_cf + kTM * ld;
    const int64_t I = blockIdx.x;
    float wmax = 0.f, wmax2 = 0.f;
    int used = 0;
    for (int r = w; r < kTM; r += kPrepWarps) {
        const int64_t i = I * kTM + r;
        const int64_t src = i < n_rows ? perm[i] : -1;
        double s2 = 0;
        for (int k = lane; k < dp; k += 32) {
            __nv_bfloat16 bh = __float2bfloat16_rn(0.f), bm = bh, bl = bh;
            float cf = 0.f;
            if (k < d && src >= 0) {
                const double c = x[src * d + k] - mean[k];
                split3(c, bh, bm, bl);
                s2 = fma(c, c, s2);
                cf = (float)c;
            }
            if (i < n_rows) {
                hi[i * dp + k] = bh;
                mid[i * dp + k] = bm;
                lo[i * dp + k] = bl;
            }
            if (k < d) s_cf[r * ld + k] = cf;
        }
        for (int o = 16; o > 0; o >>= 1) s2 += __shfl_down_sync(0xffffffffu, s2, o);
        if (lane == 0) {
            if (i < n_rows) norm2[i] = src < 0 ? INFINITY : (float)s2;
            if (src >= 0) {
                wmax = fmaxf(wmax, sqrtf((float)s2) * (1.f + 1e-6f));
                wmax2 = fmaxf(wmax2, (float)s2 * (1.f + 1e-6f));
                ++used;
            }
        }
        if (lane == 0 && src < 0) s_cf[r * ld + d] = -1.f;  // marks an empty row
        else if (lane == 0) s_cf[r * ld + d] = 1.f;
    }
    if (lane == 0) {
        s_max[w][0] = wmax;
        s_max[w][1] = wmax2;
        s_used[w] = used;
    }
    __syncthreads();
    float bmax = 0.f, bmax2 = 0.f;
    int rows = 0;
    for (int k = 0; k < kPrepWarps; ++k) {
        bmax = fmaxf(bmax, s_max[k][0]);
        bmax2 = fmaxf(bmax2, s_max[k][1]);
        rows += s_used[k];
    }
    if (threadIdx.x == 0) {
        blk_norm_bits[I] = __float_as_uint(bmax);
        blk_norm2_bits[I] = __float_as_uint(bmax2);
    }
    if (!bounds) return;
    // centroid of the block's points (any reference point serves)
    for (int k = threadIdx.x; k < d; k += blockDim.x) {
        float c = 0.f;
        for (int r = 0; r < kTM; ++r)
            if (s_cf[r * ld + d] > 0.f) c += s_cf[r * ld + k];
        c = rows > 0 ? c / (float)rows : 0.f;
        s_cent[k] = c;
        centroid_t[(int64_t)k * nblk + I] = c;
    }
    __syncthreads();
    float m = 0.f;
    for (int r = threadIdx.x; r < kTM; r += blockDim.x) {
        if (!(s_cf[r * ld + d] > 0.f)) continue;
        float s = 0.f;
        for (int k = 0; k < d; ++k) {
            const float t = s_cf[r * ld + k] - s_cent[k];
            s = fmaf(t, t, s);
        }
        m = fmaxf(m, s);
    }
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, o));
    __syncthreads();
    if (lane == 0) s_max[w][0] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < kPrepWarps; ++k) m = fmaxf(m, s_max[k][0]);
        const float rel = 1.f + (float)(d + 8) * 0x1p-23f;
        radius[I] = sqrtf(m) * rel + 0x1p-22f * bmax + 1e-30f;
    }
}

// ---- tile pruning ---------------------------------------------------------------
// Points are grouped by their nearest pivot (centred coordinates; any
// grouping gives the same result, compact groups let more tiles go) and
// every group starts on a 128-row block boundary, so that no block mixes two
// groups.  Rows left over at a group's end are empty (no point, infinite
// norm): they never produce a pair.
//
// The score |p|^2 - 2 x.p ranks pivots like |x - p|^2.  Its products run on
// the tensor cores in bf16 (a grouping heuristic needs no more): one warp
// takes 16 points at a time as the A operand of mma.sync m16n8k16 (fp32
// accumulation), the pivots sit in shared memory as the B operand (rows of
// K = n_dim rounded up to 16, padded by 4 words so the fragment loads hit
// distinct banks), 8 pivots per MMA column block.  Each thread keeps the best
// pivot of its two rows over its two columns; the quad then agrees on the
// minimum (lowest index on ties).
__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t *>(&v);
}

__device__ __forceinline__ void mma_bf16_16816(float (&c)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

constexpr int kPivotMaxK = 128;  // n_dim of the pruned path

__global__ void __launch_bounds__(256) pivot_assign_kernel(const double *__restrict__ x, int64_t n, int d,
                                                           const double *__restrict__ mean, int32_t n_pivots,
                                                           int bits_n, uint64_t *__restrict__ keys) {
    extern __shared__ uint32_t s_piv[];  // [pad8(n_pivots)][ldw] bf16 pairs, then |p|^2 per pivot
    const int dk = (d + 15) & ~15, ldw = dk / 2 + 4, ksteps = dk / 16;
    const int np8 = (n_pivots + 7) & ~7;
    float *s_pn = reinterpret_cast<float *>(s_piv + (size_t)np8 * ldw);
    const int64_t stride = n / n_pivots;
    for (int e = threadIdx.x; e < np8 * (dk / 2); e += blockDim.x) {
        const int kp = e / (dk / 2), k = 2 * (e - kp * (dk / 2));
        float v0 = 0.f, v1 = 0.f;
        if (kp < n_pivots) {
            const double *row = x + (int64_t)kp * stride * d;
            if (k < d) v0 = (float)(row[k] - mean[k]);
            if (k + 1 < d) v1 = (float)(row[k + 1] - mean[k + 1]);
        }
        s_piv[kp * ldw + k / 2] = pack_bf16x2(v0, v1);
    }
    __syncthreads();
    for (int kp = threadIdx.x; kp < np8; kp += blockDim.x) {
        float s2 = 0.f;  // of the bf16 values the products use
        for (int w = 0; w < dk / 2; ++w) {
            const __nv_bfloat162 v = *reinterpret_cast<const __nv_bfloat162 *>(&s_piv[kp * ldw + w]);
            const float2 f = __bfloat1622float2(v);
            s2 = fmaf(f.x, f.x, fmaf(f.y, f.y, s2));
        }
        s_pn[kp] = kp < n_pivots ? s2 : INFINITY;
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, g = lane >> 2, tig = lane & 3;
    const int64_t warp0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t row0 = warp0 * 16; row0 < n; row0 += nwarps * 16) {
        const int64_t ra = row0 + g, rb = row0 + g + 8;
        auto val = [&](int64_t r, int k) -> float {
            return (r < n && k < d) ? (float)(x[r * d + k] - mean[k]) : 0.f;
        };
        uint32_t a[kPivotMaxK / 16][4];
#pragma unroll
        for (int ks = 0; ks < kPivotMaxK / 16; ++ks) {
            if (ks < ksteps) {
                const int k0 = ks * 16 + tig * 2;
                a[ks][0] = pack_bf16x2(val(ra, k0), val(ra, k0 + 1));
                a[ks][1] = pack_bf16x2(val(rb, k0), val(rb, k0 + 1));
                a[ks][2] = pack_bf16x2(val(ra, k0 + 8), val(ra, k0 + 9));
                a[ks][3] = pack_bf16x2(val(rb, k0 + 8), val(rb, k0 + 9));
            }
        }
        float best_a = INFINITY, best_b = INFINITY;
        int32_t bi_a = 0, bi_b = 0;
        for (int nt = 0; nt < np8; nt += 8) {
            float c[4] = {0.f, 0.f, 0.f, 0.f};
            const uint32_t *prow = s_piv + (size_t)(nt + g) * ldw;
#pragma unroll
            for (int ks = 0; ks < kPivotMaxK / 16; ++ks)
                if (ks < ksteps) mma_bf16_16816(c, a[ks], prow[ks * 8 + tig], prow[ks * 8 + 4 + tig]);
            const int p0 = nt + tig * 2;
            const float s0 = s_pn[p0] - 2.f * c[0], s1 = s_pn[p0 + 1] - 2.f * c[1];
            const float s2 = s_pn[p0] - 2.f * c[2], s3 = s_pn[p0 + 1] - 2.f * c[3];
            if (s0 < best_a) { best_a = s0; bi_a = p0; }
            if (s1 < best_a) { best_a = s1; bi_a = p0 + 1; }
            if (s2 < best_b) { best_b = s2; bi_b = p0; }
            if (s3 < best_b) { best_b = s3; bi_b = p0 + 1; }
        }
#pragma unroll
        for (int o = 1; o <= 2; o <<= 1) {
            const float oa = __shfl_xor_sync(0xffffffffu, best_a, o), ob = __shfl_xor_sync(0xffffffffu, best_b, o);
            const int32_t ia = __shfl_xor_sync(0xffffffffu, bi_a, o), ib = __shfl_xor_sync(0xffffffffu, bi_b, o);
            if (oa < best_a || (oa == best_a && ia < bi_a)) { best_a = oa; bi_a = ia; }
            if (ob < best_b || (ob == best_b && ib < bi_b)) { best_b = ob; bi_b = ib; }
        }
        if (tig == 0) {
            if (ra < n) keys[ra] = ((uint64_t)(uint32_t)bi_a << bits_n) | (uint64_t)ra;
            if (rb < n) keys[rb] = ((uint64_t)(uint32_t)bi_b << bits_n) | (uint64_t)rb;
        }
    }
}

// Group sizes from the pivot keys (any order).
__global__ void group_count_kernel(const uint64_t *__restrict__ keys, int64_t n, int bits_n, int32_t n_groups,
                                   int32_t *__restrict__ count) {
    extern __shared__ int32_t s_cnt[];
    for (int g = threadIdx.x; g < n_groups; g += blockDim.x) s_cnt[g] = 0;
    __syncthreads();
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x)
        atomicAdd(&s_cnt[(int)(keys[p] >> bits_n)], 1);
    __syncthreads();
    for (int g = threadIdx.x; g < n_groups; g += blockDim.x)
        if (s_cnt[g]) atomicAdd(&count[g], s_cnt[g]);
}

// Start of every group among the sorted keys and in the padded row order
// (groups rounded up to whole 128-row blocks); [n_groups] holds the totals.
__global__ void group_layout_kernel(const int32_t *__restrict__ count, int32_t n_groups, int64_t *__restrict__ start,
                                    int64_t *__restrict__ pstart) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    int64_t s = 0, ps = 0;
    for (int g = 0; g < n_groups; ++g) {
        start[g] = s;
        pstart[g] = ps;
        s += count[g];
        ps += (count[g] + kTM - 1) / kTM * kTM;
    }
    start[n_groups] = s;
    pstart[n_groups] = ps;
}

// Padded row -> point index (rows not written stay -1).
__global__ void padded_perm_kernel(const uint64_t *__restrict__ keys, int64_t n, int bits_n,
                                   const int64_t *__restrict__ start, const int64_t *__restrict__ pstart,
                                   int32_t *__restrict__ perm) {
    const uint64_t mask = (1ull << bits_n) - 1;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t k = keys[p];
        const int g = (int)(k >> bits_n);
        perm[pstart[g] + (p - start[g])] = (int32_t)(k & mask);
    }
}

// Can blocks I and J (J >= I) hold a pair within R?  |c_I - c_J| - rho_I -
// rho_J > R means every pair is farther than R (triangle inequality); the
// margin covers the float32 evaluation of the centroid distance.
//
// kListRows consecutive rows I per CTA and kListCols columns J (grid y):
// the row centroids sit in shared memory, the column centroids are read
// from the transposed array [d][nblk] (coalesced), once for all rows.  Pass
// 1 counts the kept J per row, pass 2 writes them (order within a row is
// arbitrary).
constexpr int kListRows = 8;

constexpr int kListCols = 1024;  // column blocks J per CTA (grid y)

template <bool kWrite>
__global__ void __launch_bounds__(256) tile_list_kernel(const float *__restrict__ centroid_t,
                                                        const float *__restrict__ radius, int d, int64_t nblk,
                                                        float R, int32_t *__restrict__ row_count,
                                                        const int64_t *__restrict__ row_off,
                                                        int32_t *__restrict__ cursor, int2 *__restrict__ tiles) {
    __shared__ float s_a[kListRows][128];
    __shared__ float s_na[kListRows], s_ra[kListRows];
    __shared__ int32_t s_cnt[kListRows];
    const int64_t I0 = (int64_t)blockIdx.x * kListRows;
    const int rows = (int)min((int64_t)kListRows, nblk - I0);
    const int64_t J0 = max(I0, (int64_t)blockIdx.y * kListCols);
    const int64_t J1 = min(nblk, (int64_t)(blockIdx.y + 1) * kListCols);
    if (J0 >= J1) return;  // the whole CTA: nothing of this column range is at or right of the diagonal
    const bool keep_all = !(R < INFINITY);  // no pruning (centroids unused; n_dim may exceed 128)
    for (int e = threadIdx.x; e < kListRows * d && !keep_all; e += blockDim.x) {
        const int r = e / d, k = e - r * d;
        s_a[r][k] = r < rows ? centroid_t[(int64_t)k * nblk + I0 + r] : 0.f;
    }
    if (threadIdx.x < kListRows) {
        s_cnt[threadIdx.x] = 0;
        s_ra[threadIdx.x] = threadIdx.x < rows ? radius[I0 + threadIdx.x] : 0.f;
    }
    __syncthreads();
    if (threadIdx.x < kListRows && !keep_all) {
        float na = 0.f;
        for (int k = 0; k < d; ++k) na = fmaf(s_a[threadIdx.x][k], s_a[threadIdx.x][k], na);
        s_na[threadIdx.x] = sqrtf(na);
    }
    __syncthreads();
    for (int64_t J = J0 + threadIdx.x; J < J1; J += blockDim.x) {
        float s[kListRows];
#pragma unroll
        for (int r = 0; r < kListRows; ++r) s[r] = 0.f;
        float nb = 0.f;
        for (int k = 0; k < d && !keep_all; ++k) {
            const float bk = centroid_t[(int64_t)k * nblk + J];  // consecutive J: coalesced
            nb = fmaf(bk, bk, nb);
#pragma unroll
            for (int r = 0; r < kListRows; ++r) {
                const float t = s_a[r][k] - bk;
                s[r] = fmaf(t, t, s[r]);
            }
        }
        const float rb = keep_all ? 0.f : radius[J];
        nb = sqrtf(nb);
#pragma unroll
        for (int r = 0; r < kListRows; ++r) {
            const int64_t I = I0 + r;
            if (r >= rows || J < I) continue;
            const float margin = 1e-5f * (s_na[r] + nb + s_ra[r] + rb + R);
            const bool touch = keep_all || J == I || sqrtf(s[r]) - s_ra[r] - rb <= R + margin;
            if (touch) {
                if (kWrite) tiles[row_off[I] + atomicAdd(&cursor[I], 1)] = make_int2((int32_t)I, (int32_t)J);
                else atomicAdd(&s_cnt[r], 1);
            }
        }
    }
    __syncthreads();
    if (!kWrite && threadIdx.x < rows && s_cnt[threadIdx.x]) atomicAdd(&row_count[I0 + threadIdx.x], s_cnt[threadIdx.x]);
}

// Tile list -> sort keys (I, J) of every tile, and (J, I) of the tiles
// below the diagonal's mirror (J > I), counted per column block J.
__global__ void tile_keys_kernel(const int2 *__restrict__ tiles, int64_t ntiles, uint64_t *__restrict__ keys,
                                 uint64_t *__restrict__ ckeys, unsigned long long *__restrict__ nlow,
                                 int32_t *__restrict__ col_count) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < ntiles; t += (int64_t)gridDim.x * blockDim.x) {
        const int2 tl = tiles[t];
        keys[t] = ((uint64_t)(uint32_t)tl.x << 32) | (uint32_t)tl.y;
        if (tl.y > tl.x) {
            ckeys[atomicAdd(nlow, 1ull)] = ((uint64_t)(uint32_t)tl.y << 32) | (uint32_t)tl.x;
            atomicAdd(&col_count[tl.y], 1);
        }
    }
}

__global__ void tiles_from_keys_kernel(const uint64_t *__restrict__ keys, int64_t ntiles, int2 *__restrict__ tiles) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < ntiles; t += (int64_t)gridDim.x * blockDim.x)
        tiles[t] = make_int2((int32_t)(keys[t] >> 32), (int32_t)(keys[t] & 0xffffffffull));
}

// Index of tile (I, J) in the list (sorted by I, then J; every listed pair
// has J >= I); -1 when not listed.
__device__ __forceinline__ int64_t find_tile(const int2 *__restrict__ tiles, const int64_t *__restrict__ tile_off,
                                             int32_t I, int32_t J) {
    int64_t lo = tile_off[I], hi = tile_off[I + 1];
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (tiles[mid].y < J) lo = mid + 1;
        else hi = mid;
    }
    return lo < tile_off[I + 1] && tiles[lo].y == J ? lo : -1;
}

// Padded rows -> compact internal index (rows of points in padded order,
// padding rows removed): the neighbour graph is kept in this order, so a
// tile's columns come out ascending with no sort.
__global__ void real_flag_kernel(const int32_t *__restrict__ perm, int64_t n_rows, int32_t *__restrict__ flag) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p <= n_rows; p += (int64_t)gridDim.x * blockDim.x)
        flag[p] = p < n_rows && perm[p] >= 0 ? 1 : 0;
}

__global__ void compact_order_kernel(const int32_t *__restrict__ perm_pad, const int64_t *__restrict__ pos,
                                     int64_t n_rows, int32_t *__restrict__ pad2c, int32_t *__restrict__ perm,
                                     int32_t *__restrict__ inv) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n_rows; p += (int64_t)gridDim.x * blockDim.x) {
        const int32_t pt = perm_pad[p];
        if (pt < 0) {
            pad2c[p] = -1;
            continue;
        }
        const int32_t c = (int32_t)pos[p];
        pad2c[p] = c;
        perm[c] = pt;
        inv[pt] = c;
    }
}

// Band pairs in float64, reference order; a pair within the radius sets
// its bit in the mask of its tile.  One thread per pair keeps the
// sequential sum of the reference; each warp stages its 32 pairs' rows in
// shared memory kRecheckDims coordinates at a time, so the global loads are
// 64-byte runs instead of 32 scattered words per instruction.  The largest
// error is reduced once per warp.
constexpr int kRecheckWarps = 8;
constexpr int kRecheckDims = 8;

__global__ void __launch_bounds__(kRecheckWarps * 32) gram_recheck_kernel(
    const double *__restrict__ x, int d, const uint64_t *__restrict__ amb, const unsigned long long *__restrict__ namb,
    int64_t amb_cap, double rc, int metric, int fpmode, const int32_t *__restrict__ perm_pad,
    const int2 *__restrict__ tiles, const int64_t *__restrict__ tile_off, uint32_t *__restrict__ masks,
    const float *__restrict__ amb_d2, unsigned *__restrict__ max_err_bits) {
    __shared__ double s_a[kRecheckWarps][32][kRecheckDims + 1];
    __shared__ double s_b[kRecheckWarps][32][kRecheckDims + 1];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t total = min((int64_t)*namb, amb_cap);
    float max_err = 0.f;
    for (int64_t base = ((int64_t)blockIdx.x * kRecheckWarps + w) * 32; base < total;
         base += (int64_t)gridDim.x * kRecheckWarps * 32) {
        const int64_t e = base + lane;
        const bool valid = e < total;
        const uint64_t a = valid ? amb[e] : 0ull;
        const int64_t pi = (int64_t)((a >> 32) & 0x7fffffffull), pj = (int64_t)(a & 0xffffffffull);  // padded rows
        const int64_t i = valid ? perm_pad[pi] : 0, j = valid ? perm_pad[pj] : 0;                    // points
        double s = 0.0;
        for (int k0 = 0; k0 < d; k0 += kRecheckDims) {
            // element m*32 + lane of the warp's 32 x kRecheckDims block: row r, coordinate c
#pragma unroll
            for (int m = 0; m < kRecheckDims; ++m) {
                const int idx = m * 32 + lane;
                const int r = idx / kRecheckDims, c = idx % kRecheckDims;
                const int64_t ri = __shfl_sync(0xffffffffu, i, r), rj = __shfl_sync(0xffffffffu, j, r);
                const bool rv = __shfl_sync(0xffffffffu, valid, r);
                const int k = k0 + c;
                s_a[w][r][c] = rv && k < d ? x[ri * d + k] : 0.0;
                s_b[w][r][c] = rv && k < d ? x[rj * d + k] : 0.0;
            }
            __syncwarp();
            const int kn = min(kRecheckDims, d - k0);
            if (fpmode == CNN_FP_FUSED) {
                for (int c = 0; c < kn; ++c) {
                    const double t = __dsub_rn(s_a[w][lane][c], s_b[w][lane][c]);
                    s = __fma_rn(t, t, s);
                }
            } else {
                for (int c = 0; c < kn; ++c) {
                    const double t = __dsub_rn(s_a[w][lane][c], s_b[w][lane][c]);
                    s = __dadd_rn(s, __dmul_rn(t, t));
                }
            }
            __syncwarp();
        }
        const double sv = metric == CNN_METRIC_EUCLIDEAN ? __dsqrt_rn(s) : s;
        if (valid && sv <= rc) {
            const int64_t t = find_tile(tiles, tile_off, (int32_t)(pi / kTM), (int32_t)(pj / kTM));
            if (t >= 0)  // always: the pair came from that tile
                atomicOr(&masks[t * kMaskWords + (pi % kTM) * 4 + (pj % kTM) / 32], 1u << (pj % 32));
        }
        if (valid) max_err = fmaxf(max_err, fabsf((float)(s - (double)amb_d2[e])));
    }
    for (int o = 16; o > 0; o >>= 1) max_err = fmaxf(max_err, __shfl_xor_sync(0xffffffffu, max_err, o));
    if (lane == 0 && max_err > 0.f) atomicMax(max_err_bits, __float_as_uint(max_err));
}

// Rows of the neighbour graph from the tile masks, in the compact internal
// order.  Row block B's columns come from a sequence of tiles: first the
// tiles (J', B) with J' < B (ascending J', columns of their masks,
// transposed in the warp), then the tiles (B, J), J >= B (ascending J, rows
// of their masks).  The sequence is cut
// into chunks of kRowChunk tiles, and every (row block, 32-row quadrant,
// chunk) is one warp's work (lane = row), so that row blocks with many
// tiles spread over many warps.  The count pass stores each (chunk, row)
// count and adds it to the row's degree; the fill pass starts each chunk of
// a row after the chunks before it.
constexpr int kRowChunk = 8;

// 32 x 32 bit transpose across a warp: lane r holds row r (bit c = column
// c); afterwards lane c holds column c (bit r = row r).  Five butterfly
// stages swap the off-diagonal blocks of size 16, 8, 4, 2, 1.
__device__ __forceinline__ uint32_t transpose32(uint32_t x, int lane) {
    const uint32_t m16 = 0x0000ffffu, m8 = 0x00ff00ffu, m4 = 0x0f0f0f0fu, m2 = 0x33333333u, m1 = 0x55555555u;
#define CNN_T32_STAGE(S, M)                                               \
    {                                                                     \
        const uint32_t y = __shfl_xor_sync(0xffffffffu, x, S);            \
        x = (lane & S) ? ((x & ~M) | ((y >> S) & M)) : ((x & M) | ((y & M) << S)); \
    }
    CNN_T32_STAGE(16, m16)
    CNN_T32_STAGE(8, m8)
    CNN_T32_STAGE(4, m4)
    CNN_T32_STAGE(2, m2)
    CNN_T32_STAGE(1, m1)
#undef CNN_T32_STAGE
    return x;
}

// the lower tiles' list indices (sorted keys (B << 32 | J') -> tile of (J', B))
__global__ void lower_tiles_kernel(const uint64_t *__restrict__ lkeys, const unsigned long long *__restrict__ nlow,
                                   const int2 *__restrict__ tiles, const int64_t *__restrict__ tile_off,
                                   int64_t *__restrict__ ltile) {
    const int64_t m = (int64_t)*nlow;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < m; e += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t k = lkeys[e];
        ltile[e] = find_tile(tiles, tile_off, (int32_t)(k & 0xffffffffull), (int32_t)(k >> 32));
    }
}

// chunks of every row block's tile sequence
__global__ void row_chunks_kernel(int64_t nblk, const int64_t *__restrict__ tile_off,
                                  const int64_t *__restrict__ low_off, int32_t *__restrict__ nchunk) {
    for (int64_t B = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; B <= nblk; B += (int64_t)gridDim.x * blockDim.x) {
        if (B == nblk) {
            nchunk[B] = 0;
            continue;
        }
        const int64_t L = (low_off[B + 1] - low_off[B]) + (tile_off[B + 1] - tile_off[B]);
        nchunk[B] = (int32_t)((L + kRowChunk - 1) / kRowChunk);
    }
}

template <bool kFill>
__global__ void __launch_bounds__(256) gram_rows_kernel(
    int64_t nblk, int64_t nwork, const int64_t *__restrict__ chunk_base, const int2 *__restrict__ tiles,
    const int64_t *__restrict__ tile_off, const int64_t *__restrict__ ltile, const int64_t *__restrict__ low_off,
    const uint32_t *__restrict__ masks, const int32_t *__restrict__ pad2c, int32_t *__restrict__ chunk_cnt,
    int32_t *__restrict__ deg, const int64_t *__restrict__ row_off, int32_t *__restrict__ cols) {
    const int lane = threadIdx.x & 31;
    const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    if (gw >= nwork) return;
    // the row block: 4 * chunk_base[B] <= gw < 4 * chunk_base[B + 1]
    int64_t lo = 0, hi = nblk;
    while (hi - lo > 1) {
        const int64_t mid = (lo + hi) >> 1;
        if (4 * chunk_base[mid] <= gw) lo = mid;
        else hi = mid;
    }
    const int32_t B = (int32_t)lo;
    const int64_t nch = chunk_base[B + 1] - chunk_base[B];
    const int64_t r = gw - 4 * chunk_base[B];
    const int q = (int)(r / nch);
    const int64_t k = r - (int64_t)q * nch;
    const int lr = q * 32 + lane;
    const int32_t me = pad2c[(int64_t)B * kTM + lr];  // -1: a padding row (never a neighbour)
    const int64_t item0 = 4 * chunk_base[B] + (int64_t)q * nch;  // chunk 0 of this (block, quadrant)
    int64_t w = 0;
    if (kFill && me >= 0) {
        w = row_off[me];
        for (int64_t kk = 0; kk < k; ++kk) w += chunk_cnt[(item0 + kk) * 32 + lane];
    }
    const int64_t nlow = low_off[B + 1] - low_off[B];
    const int64_t L = nlow + (tile_off[B + 1] - tile_off[B]);
    const int64_t s1 = min(L, (k + 1) * kRowChunk);
    int32_t cnt = 0;
    for (int64_t sidx = k * kRowChunk; sidx < s1; ++sidx) {
        // tile (J', B), J' < B: column lr of its mask, transposed in the
        // warp from word q of its rows; tile (B, J), J >= B: row lr of its
        // mask.  Either way 128 bits over the other block's rows.
        int64_t t;
        int32_t J;
        uint32_t words[4];
        if (sidx < nlow) {
            t = ltile[low_off[B] + sidx];
            if (t < 0) continue;  // not reached: every lower entry is a listed tile (warp-uniform)
            J = tiles[t].x;
            const uint32_t *mt = masks + t * kMaskWords;
#pragma unroll
            for (int g = 0; g < 4; ++g) words[g] = transpose32(mt[(g * 32 + lane) * 4 + q], lane);
        } else {
            t = tile_off[B] + (sidx - nlow);
            J = tiles[t].y;
            const uint4 rw = *reinterpret_cast<const uint4 *>(masks + t * kMaskWords + lr * 4);
            words[0] = rw.x;
            words[1] = rw.y;
            words[2] = rw.z;
            words[3] = rw.w;
        }
        {
#pragma unroll
            for (int g = 0; g < 4; ++g) {
                if (!kFill) {
                    cnt += __popc(words[g]);
                    continue;
                }
                for (uint32_t m = words[g]; m; m &= m - 1) {
                    if (me >= 0) cols[w + cnt] = pad2c[(int64_t)J * kTM + g * 32 + __ffs(m) - 1];
                    ++cnt;
                }
            }
        }
    }
    if (!kFill) {
        chunk_cnt[(item0 + k) * 32 + lane] = cnt;
        if (me >= 0 && cnt) atomicAdd(&deg[me], cnt);
    }
}

typedef CUresult (*PFN_encodeTiled)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                    const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                    CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// looked up once per process (thread-safe initialisation of the static)
PFN_encodeTiled get_encode_fn() {
    static const PFN_encodeTiled fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        PFN_encodeTiled f = nullptr;
        if (cudaGetDriverEntryPoint("cuTensorMapEncodeTiled", &p, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            f = reinterpret_cast<PFN_encodeTiled>(p);
        (void)cudaGetLastError();
        return f;
    }();
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

// Error bound on |acc - x'.y'| relative to |x'||y'| (Cauchy-Schwarz on the
// per-coordinate bounds): the three-way split (split3) leaves at most
// (1 + 2^-3) 2^-24 |x_k| per coordinate, so the residuals of both operands
// add at most 2.25 * 2^-24 |x_k||y_k|, and the dropped mid.lo, lo.mid,
// lo.lo at most 2^-26 |x_k||y_k|: below 2.5 * 2^-24, counted as 6 * 2^-24.  FP32
// accumulation of the dp exact hi.hi products adds (dp + 8) 2^-23; the
// cross-term accumulator (5 dp products, each below 2^-7 |x_k||y_k|) adds
// (5 dp + 8) 2^-29, and summing the two accumulators 2 * 2^-24.  d2 uses
// 2 * acc, so the band coefficient doubles the total; taken with a safety
// factor of 2.
double gram_band_coef(int dp) {
    const double rel = 6.0 * ldexp(1.0, -24) + (dp + 8.0) * ldexp(1.0, -23) + (5.0 * dp + 8.0) * ldexp(1.0, -29) +
                       2.0 * ldexp(1.0, -24);
    return 2.0 * 2.0 * rel;
}

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
    const double rc2 = metric == CNN_METRIC_EUCLIDEAN ? radius_cutoff * radius_cutoff : radius_cutoff;
    unsigned long long *counters = ctx->counters.as<unsigned long long>();
    unsigned long long *nkeys = counters + 10, *namb = counters + 11;
    int *status = reinterpret_cast<int *>(counters + 12);
    int *nonfinite = reinterpret_cast<int *>(counters + 13);
    unsigned *max_err_bits = reinterpret_cast<unsigned *>(counters + 14);
    CNN_CUDA(ctx, cudaMemsetAsync(counters + 10, 0, 4 * sizeof(unsigned long long), st));

    // column sums (the centring) and the non-finite check
    CNN_TRY(ctx->ensure(ctx->scratch_b, sizeof(double) * (size_t)d + 3 * sizeof(int64_t) * 1024 + 4096));
    double *colsum = ctx->scratch_b.as<double>();
    int32_t *gcount = reinterpret_cast<int32_t *>(colsum + d);
    int64_t *gstart = reinterpret_cast<int64_t *>(
        (reinterpret_cast<uintptr_t>(gcount + 1024) + 15) & ~uintptr_t(15));
    int64_t *gpstart = gstart + 1024;
    CNN_CUDA(ctx, cudaMemsetAsync(colsum, 0, sizeof(double) * d, st));
    {
        // block = a multiple of n_dim (at most 1024 threads); grid stride a multiple too
        const int per = std::max(1, 256 / d), threads = d * per;
        if (threads > 1024) return CNN_OK;  // n_dim > 1024: the all-pairs path takes it
        const int blocks = (int)std::min<int64_t>((int64_t)ctx->sm_count * 4, (n * d + threads - 1) / threads);
        column_sum_kernel<<<blocks, threads, sizeof(double) * threads, st>>>(ctx->x, n, d, colsum, nonfinite);
        CNN_LAUNCH_CHECK(ctx);
        column_mean_kernel<<<1, 128, 0, st>>>(colsum, d, n);  // colsum holds the column means from here
        CNN_LAUNCH_CHECK(ctx);
    }
    // internal order: points grouped by nearest pivot, every group starting
    // on a block boundary, so that 128-row blocks are compact and far-apart
    // block pairs can be skipped
    const int bits_n = [&] { int b = 1; while (b < 62 && (int64_t(1) << b) < n) ++b; return b; }();
    const bool prune = d <= 128 && n >= 8 * kTM;
    int n_groups = 1;
    if (prune) {
        n_groups = (int)std::max<int64_t>(1, std::min<int64_t>({kMaxGroups, n / 1024, 98304 / (4 * ((d + 3) / 4 * 4))}));
        CNN_TRY(ctx->ensure(ctx->scratch_a, sizeof(uint64_t) * (size_t)n));
        uint64_t *pkeys = ctx->scratch_a.as<uint64_t>();
        const int dk = (d + 15) & ~15, np8 = (n_groups + 7) & ~7;
        const size_t psmem = sizeof(uint32_t) * (size_t)np8 * (dk / 2 + 4) + sizeof(float) * (size_t)np8;
        CNN_TRY(allow_dynamic_smem(ctx, (const void *)pivot_assign_kernel, psmem));
        pivot_assign_kernel<<<ctx->sm_count * 4u, 256, psmem, st>>>(ctx->x, n, d, colsum, n_groups, bits_n, pkeys);
        CNN_LAUNCH_CHECK(ctx);
        int pb = 1;
        while ((1 << pb) < n_groups) ++pb;
        CNN_TRY(radix_sort_u64(ctx, pkeys, n, bits_n + pb, bits_n));  // built in point order
        CNN_CUDA(ctx, cudaMemsetAsync(gcount, 0, sizeof(int32_t) * n_groups, st));
        group_count_kernel<<<std::min<unsigned>(grid_for(n, 256), ctx->sm_count * 2u), 256, sizeof(int32_t) * n_groups, st>>>(
            pkeys, n, bits_n, n_groups, gcount);
        CNN_LAUNCH_CHECK(ctx);
        group_layout_kernel<<<1, 32, 0, st>>>(gcount, n_groups, gstart, gpstart);
        CNN_LAUNCH_CHECK(ctx);
    }
    int64_t h_rows = n;
    int h_nonfinite = 0;
    if (prune) CNN_CUDA(ctx, cudaMemcpyAsync(&h_rows, gpstart + n_groups, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    CNN_CUDA(ctx, cudaMemcpyAsync(&h_nonfinite, nonfinite, sizeof(int), cudaMemcpyDeviceToHost, st));
    CNN_CUDA(ctx, cudaStreamSynchronize(st));
    if (h_nonfinite) return CNN_OK;  // non-finite coordinates: the all-pairs path handles them
    const int64_t n_rows = h_rows;   // padded internal rows (n without pruning)
    if (n_rows >= (int64_t(1) << 31) - 256) return CNN_OK;
    const int64_t nblk = (n_rows + kTM - 1) / kTM;

    CNN_TRY(ctx->ensure(ctx->gram_perm, sizeof(int32_t) * (size_t)n_rows));
    int32_t *perm = ctx->gram_perm.as<int32_t>();
    if (prune) {
        CNN_TRY(fill_i32(ctx, perm, n_rows, -1));
        padded_perm_kernel<<<std::min<unsigned>(grid_for(n, 256), 4096u), 256, 0, st>>>(
            ctx->scratch_a.as<uint64_t>(), n, bits_n, gstart, gpstart, perm);
        CNN_LAUNCH_CHECK(ctx);
    } else {
        CNN_TRY(iota_i32(ctx, perm, n));
    }

    // hi, lo (bf16 n_rows x dp), norm2 (n_rows), block norms
    CNN_TRY(ctx->ensure(ctx->gram_hi, sizeof(__nv_bfloat16) * (size_t)n_rows * dp));
    CNN_TRY(ctx->ensure(ctx->gram_mid, sizeof(__nv_bfloat16) * (size_t)n_rows * dp));
    CNN_TRY(ctx->ensure(ctx->gram_lo, sizeof(__nv_bfloat16) * (size_t)n_rows * dp));
    CNN_TRY(ctx->ensure(ctx->gram_aux, sizeof(float) * (size_t)(n_rows + 2 * nblk + 64)));
    float *norm2 = ctx->gram_aux.as<float>();
    unsigned *blk_norm_bits = reinterpret_cast<unsigned *>(norm2 + n_rows);
    unsigned *blk_norm2_bits = blk_norm_bits + nblk;
    // the list of block pairs (I, J >= I) that can hold a pair within R
    const double Rsearch = (metric == CNN_METRIC_EUCLIDEAN ? radius_cutoff : sqrt(radius_cutoff)) * (1.0 + 1e-6);
    CNN_TRY(ctx->ensure(ctx->gram_blocks, sizeof(float) * (size_t)nblk * (d + 1) +
                                              (2 * sizeof(int32_t) + sizeof(int64_t)) * (size_t)(nblk + 1) + 256));
    float *centroid = ctx->gram_blocks.as<float>();  // transposed: [d][nblk]
    float *bradius = centroid + nblk * d;
    int32_t *row_count = reinterpret_cast<int32_t *>(bradius + nblk);
    int32_t *row_cursor = row_count + nblk + 1;
    int64_t *row_off = reinterpret_cast<int64_t *>(
        (reinterpret_cast<uintptr_t>(row_cursor + nblk + 1) + 15) & ~uintptr_t(15));
    const float Rf = prune ? (float)Rsearch : INFINITY;
    if (prune) {  // n_dim <= 128: the block's coordinates fit in shared memory
        const size_t psmem = sizeof(float) * ((size_t)kTM * (d + 1) + d);
        CNN_TRY(allow_dynamic_smem(ctx, (const void *)gram_prep_bounds_kernel, psmem));
        gram_prep_bounds_kernel<<<(unsigned)nblk, kPrepWarps * 32, psmem, st>>>(
            ctx->x, n_rows, d, dp, colsum, perm, ctx->gram_hi.as<__nv_bfloat16>(), ctx->gram_mid.as<__nv_bfloat16>(),
            ctx->gram_lo.as<__nv_bfloat16>(), norm2, blk_norm_bits, blk_norm2_bits, 1, nblk, centroid, bradius);
        CNN_LAUNCH_CHECK(ctx);
    } else {
        CNN_CUDA(ctx, cudaMemsetAsync(blk_norm_bits, 0, sizeof(unsigned) * 2 * (size_t)nblk, st));
        gram_prep_kernel<<<grid_for(n_rows * 32, 256), 256, 0, st>>>(
            ctx->x, n_rows, n, d, dp, colsum, perm, ctx->gram_hi.as<__nv_bfloat16>(),
            ctx->gram_mid.as<__nv_bfloat16>(), ctx->gram_lo.as<__nv_bfloat16>(), norm2, blk_norm_bits,
            blk_norm2_bits);
        CNN_LAUNCH_CHECK(ctx);
        CNN_CUDA(ctx, cudaMemsetAsync(centroid, 0, sizeof(float) * (size_t)nblk * (d + 1), st));
    }
    const dim3 lgrid((unsigned)((nblk + kListRows - 1) / kListRows), (unsigned)((nblk + kListCols - 1) / kListCols));
    CNN_CUDA(ctx, cudaMemsetAsync(row_count, 0, sizeof(int32_t) * 2 * (size_t)(nblk + 1), st));  // counts, cursors
    tile_list_kernel<false><<<lgrid, 256, 0, st>>>(centroid, bradius, d, nblk, Rf, row_count, nullptr, nullptr,
                                                   nullptr);
    CNN_LAUNCH_CHECK(ctx);
    CNN_TRY(scan_exclusive_i32_to_i64(ctx, row_count, row_off, nblk + 1));
    int64_t ntiles = 0;
    CNN_CUDA(ctx, cudaMemcpyAsync(&ntiles, row_off + nblk, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    CNN_CUDA(ctx, cudaStreamSynchronize(st));
    // a 2 KB hit mask per listed tile: decline past 64 GiB of them
    if (ntiles > (int64_t(64) << 30) / (int64_t)(kMaskWords * sizeof(uint32_t))) return CNN_OK;
    CNN_TRY(ctx->ensure(ctx->gram_tiles, sizeof(int2) * (size_t)(ntiles > 0 ? ntiles : 1)));
    int2 *tiles = ctx->gram_tiles.as<int2>();
    tile_list_kernel<true><<<lgrid, 256, 0, st>>>(centroid, bradius, d, nblk, Rf, nullptr, row_off, row_cursor,
                                                  tiles);
    CNN_LAUNCH_CHECK(ctx);
    // the list sorted by (I, J); the tiles (J', I) with J' < I by column
    // block I, then J' (the lower half of every row's columns)
    const int bits_blk = [&] { int b = 1; while (b < 31 && (int64_t(1) << b) <= nblk) ++b; return b; }();
    CNN_TRY(ctx->ensure(ctx->gram_tkeys, sizeof(uint64_t) * (size_t)(2 * ntiles + 2)));
    CNN_TRY(ctx->ensure(ctx->gram_low, (sizeof(int32_t) + sizeof(int64_t)) * (size_t)(nblk + 1) + 64));
    uint64_t *tkeys = ctx->gram_tkeys.as<uint64_t>();
    uint64_t *lkeys = tkeys + ntiles;
    int32_t *low_count = ctx->gram_low.as<int32_t>();
    int64_t *low_off = reinterpret_cast<int64_t *>(
        (reinterpret_cast<uintptr_t>(low_count + nblk + 1) + 15) & ~uintptr_t(15));
    unsigned long long *nlow = counters + 10;
    CNN_CUDA(ctx, cudaMemsetAsync(low_count, 0, sizeof(int32_t) * (size_t)(nblk + 1), st));
    CNN_CUDA(ctx, cudaMemsetAsync(nlow, 0, sizeof(unsigned long long), st));
    const unsigned tg = std::min<unsigned>(grid_for(ntiles, 256), ctx->sm_count * 8u);
    tile_keys_kernel<<<tg, 256, 0, st>>>(tiles, ntiles, tkeys, lkeys, nlow, low_count);
    CNN_LAUNCH_CHECK(ctx);
    CNN_TRY(radix_sort_u64(ctx, tkeys, ntiles, 32 + bits_blk));
    tiles_from_keys_kernel<<<tg, 256, 0, st>>>(tkeys, ntiles, tiles);
    CNN_LAUNCH_CHECK(ctx);
    CNN_TRY(scan_exclusive_i32_to_i64(ctx, low_count, low_off, nblk + 1));
    // the count of lower tiles stays on the device (at most ntiles)
    CNN_TRY(radix_sort_u64(ctx, lkeys, ntiles, 32 + bits_blk, 0, nullptr, reinterpret_cast<const int64_t *>(nlow)));

    CUtensorMap map_hi, map_mid, map_lo;
    if (!make_map(&map_hi, ctx->gram_hi.ptr, n_rows, dp) || !make_map(&map_mid, ctx->gram_mid.ptr, n_rows, dp) ||
        !make_map(&map_lo, ctx->gram_lo.ptr, n_rows, dp))
        return CNN_OK;

    const double coef = gram_band_coef(dp);
    GramArgs a{};
    a.n = n_rows;
    a.nkb = nkb;
    a.nblk = (int32_t)nblk;
    a.ntiles = ntiles;
    a.tiles = tiles;
    a.rc2 = (float)rc2;
    a.coef = (float)coef;
    a.slack_coef = (float)(8.0 * ldexp(1.0, -24));  // float32 rounding of |x|^2, |y|^2 and the fma
    a.min_band = (float)(1e-6 * rc2);  // float32 rounding of rc2 and of rc2 -/+ band
    a.norm2 = norm2;
    a.blk_norm = reinterpret_cast<const float *>(blk_norm_bits);
    a.blk_norm2 = reinterpret_cast<const float *>(blk_norm2_bits);
    a.status = status;
    a.wait_ns = ctx->wait_limit_ns > 0 ? (unsigned long long)ctx->wait_limit_ns : kWaitNs;
    const int64_t amb_cap = std::max<int64_t>(int64_t(1) << 22, n * 64);
    const int sms = (int)ctx->sm_count;
    int dev_sms = 0;
    cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, dev);
    const int grid = (int)std::min<int64_t>(ntiles, dev_sms > 0 ? dev_sms : sms);
    const size_t smem = (size_t)kStages * kStageBytes + 1024;
    CNN_TRY(allow_dynamic_smem(ctx, (const void *)gram_search_kernel, smem));
    CNN_TRY(ctx->ensure(ctx->gram_masks, sizeof(uint32_t) * (size_t)kMaskWords * (size_t)ntiles));
    CNN_TRY(ctx->ensure(ctx->gram_amb, (sizeof(uint64_t) + sizeof(float)) * (size_t)amb_cap));
    a.masks = ctx->gram_masks.as<uint32_t>();
    a.amb = ctx->gram_amb.as<uint64_t>();
    a.amb_d2 = reinterpret_cast<float *>(a.amb + amb_cap);
    a.amb_cap = amb_cap;
    a.namb = namb;
    CNN_CUDA(ctx, cudaMemsetAsync(counters + 11, 0, 2 * sizeof(unsigned long long), st));
    CNN_CUDA(ctx, cudaMemsetAsync(max_err_bits, 0, sizeof(unsigned), st));
    stage_begin(ctx, 9);
    gram_search_kernel<<<grid, kGramThreads, smem, st>>>(map_hi, map_mid, map_lo, a);
    CNN_LAUNCH_CHECK(ctx);
    stage_end(ctx, 9);
    gram_recheck_kernel<<<ctx->sm_count * 8u, kRecheckWarps * 32, 0, st>>>(
        ctx->x, d, a.amb, namb, amb_cap, radius_cutoff, metric, fpmode, perm, tiles, row_off, a.masks, a.amb_d2,
        max_err_bits);
    CNN_LAUNCH_CHECK(ctx);
    unsigned long long hc[3];
    CNN_CUDA(ctx, cudaMemcpyAsync(hc, counters + 10, sizeof(hc), cudaMemcpyDeviceToHost, st));
    CNN_CUDA(ctx, cudaStreamSynchronize(st));
    const int h_status = (int)(hc[2] & 0xffffffffull);
    if (h_status != 0) return ctx->fail(CNN_ERR_TIMEOUT, "tensor-core distance kernel timed out on a barrier");
    if ((int64_t)hc[1] > amb_cap) return CNN_OK;  // too many band pairs: the all-pairs path decides
    ctx->stats.n_exact = (int64_t)hc[1];
    unsigned me = 0;
    CNN_CUDA(ctx, cudaMemcpyAsync(&me, max_err_bits, sizeof(unsigned), cudaMemcpyDeviceToHost, st));

    // the compact internal order (padded rows without padding) and the
    // rows from the masks
    CNN_TRY(ctx->ensure(ctx->gram_pad2c, sizeof(int32_t) * (size_t)(nblk * kTM + 1)));
    CNN_TRY(ctx->ensure(ctx->scratch_c, sizeof(int64_t) * (size_t)(n_rows + 1) + sizeof(int32_t) * (size_t)(n_rows + 1) + 64));
    int32_t *pad2c = ctx->gram_pad2c.as<int32_t>();
    int64_t *pos = ctx->scratch_c.as<int64_t>();
    int32_t *rflag = reinterpret_cast<int32_t *>(pos + n_rows + 1);
    CNN_TRY(fill_i32(ctx, pad2c, nblk * kTM, -1));
    real_flag_kernel<<<std::min<unsigned>(grid_for(n_rows + 1, 256), ctx->sm_count * 16u), 256, 0, st>>>(perm, n_rows,
                                                                                                    rflag);
    CNN_LAUNCH_CHECK(ctx);
    CNN_TRY(scan_exclusive_i32_to_i64(ctx, rflag, pos, n_rows + 1));
    compact_order_kernel<<<std::min<unsigned>(grid_for(n_rows, 256), ctx->sm_count * 16u), 256, 0, st>>>(
        perm, pos, n_rows, pad2c, ctx->perm.as<int32_t>(), ctx->inv.as<int32_t>());
    CNN_LAUNCH_CHECK(ctx);
    // work items of the row builder: (row block, quadrant, chunk of tiles)
    CNN_TRY(ctx->ensure(ctx->gram_rowwork, sizeof(int64_t) * (size_t)(ntiles + nblk + 2) +
                                               sizeof(int32_t) * (size_t)(nblk + 1) + 64));
    int64_t *ltile = ctx->gram_rowwork.as<int64_t>();
    int64_t *chunk_base = ltile + ntiles;
    int32_t *nchunk = reinterpret_cast<int32_t *>(chunk_base + nblk + 2);
    lower_tiles_kernel<<<tg, 256, 0, st>>>(lkeys, nlow, tiles, row_off, ltile);
    CNN_LAUNCH_CHECK(ctx);
    row_chunks_kernel<<<std::min<unsigned>(grid_for(nblk + 1, 256), ctx->sm_count * 8u), 256, 0, st>>>(
        nblk, row_off, low_off, nchunk);
    CNN_LAUNCH_CHECK(ctx);
    CNN_TRY(scan_exclusive_i32_to_i64(ctx, nchunk, chunk_base, nblk + 1));
    int64_t nchunks = 0;
    CNN_TRY(read_back(ctx, &nchunks, chunk_base + nblk, sizeof(int64_t)));
    const int64_t nwork = 4 * nchunks;
    CNN_TRY(ctx->ensure(ctx->gram_chunkcnt, sizeof(int32_t) * 32 * (size_t)(nwork > 0 ? nwork : 1)));
    int32_t *deg = ctx->deg.as<int32_t>();
    int64_t *row_off_csr = ctx->row_off.as<int64_t>();
    CNN_CUDA(ctx, cudaMemsetAsync(deg, 0, sizeof(int32_t) * (size_t)(n + 1), st));
    const unsigned rg = (unsigned)((nwork * 32 + 255) / 256);
    if (nwork > 0) {
        gram_rows_kernel<false><<<rg, 256, 0, st>>>(nblk, nwork, chunk_base, tiles, row_off, ltile, low_off, a.masks,
                                                    pad2c, ctx->gram_chunkcnt.as<int32_t>(), deg, nullptr, nullptr);
        CNN_LAUNCH_CHECK(ctx);
    }
    CNN_TRY(scan_exclusive_i32_to_i64(ctx, deg, row_off_csr, n + 1));
    int64_t nk = 0;
    CNN_TRY(read_back(ctx, &nk, row_off_csr + n, sizeof(int64_t)));
    CNN_TRY(ctx->ensure(ctx->cols, sizeof(int32_t) * (size_t)(nk > 0 ? nk : 1)));
    if (nwork > 0) {
        gram_rows_kernel<true><<<rg, 256, 0, st>>>(nblk, nwork, chunk_base, tiles, row_off, ltile, low_off, a.masks,
                                                   pad2c, ctx->gram_chunkcnt.as<int32_t>(), nullptr, row_off_csr,
                                                   ctx->cols.as<int32_t>());
        CNN_LAUNCH_CHECK(ctx);
    }
    float mef;
    memcpy(&mef, &me, sizeof(float));
    ctx->stats.max_abs_err = mef;
    ctx->stats.n_candidates = ntiles * kTM * kTM;
    ctx->stats.filter_band = std::max(coef, 0.0);
    ctx->stats.filter_enabled = 1;
    ctx->nnz = nk;
    ctx->identity_perm = !prune;  // without pruning the rows are the points in order
    *used = true;
    return CNN_OK;
}

}  // namespace cnn
