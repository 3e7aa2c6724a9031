// prims.cu -- device-wide primitives: exclusive scan and LSD radix sort.
//
// Both are plain HBM-streaming kernels: a tile of 2048 elements per block
// (256 threads x 8), staged through shared memory so that every global
// access is coalesced.
#include <string.h>

#include <map>
#include <mutex>
#include <utility>

#include "common.cuh"

namespace cnn {

namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;
constexpr int64_t kScanSumMax = 1024;  // blocks up to which a scan takes two launches

__device__ __forceinline__ int64_t warp_incl_scan(int64_t v) {
    int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int64_t u = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += u;
    }
    return v;
}

// Exclusive scan of the 2048-element tile held in s[].  Each thread owns 8
// consecutive elements.
__device__ __forceinline__ void block_scan_tile(int64_t *s) {
    __shared__ int64_t warp_tot[kScanThreads / 32];
    const int t = threadIdx.x;
    int64_t local[kScanItems];
    int64_t sum = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        local[i] = s[t * kScanItems + i];
        sum += local[i];
    }
    int64_t incl = warp_incl_scan(sum);
    if ((t & 31) == 31) warp_tot[t >> 5] = incl;
    __syncthreads();
    if (t < 32) {
        int64_t w = t < kScanThreads / 32 ? warp_tot[t] : 0;
        int64_t wi = warp_incl_scan(w);
        if (t < kScanThreads / 32) warp_tot[t] = wi - w;
    }
    __syncthreads();
    int64_t run = warp_tot[t >> 5] + incl - sum;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        s[t * kScanItems + i] = run;
        run += local[i];
    }
    __syncthreads();
}

template <typename TIn>
__global__ void __launch_bounds__(kScanThreads) scan_reduce_kernel(const TIn *__restrict__ in, int64_t n,
                                                                   int64_t *__restrict__ partial) {
    __shared__ int64_t red[kScanThreads / 32];
    const int64_t base = (int64_t)blockIdx.x * kScanTile;
    int64_t sum = 0;
    for (int i = threadIdx.x; i < kScanTile; i += kScanThreads) {
        int64_t g = base + i;
        if (g < n) sum += (int64_t)in[g];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = sum;
    __syncthreads();
    if (threadIdx.x == 0) {
        int64_t t = 0;
        for (int w = 0; w < kScanThreads / 32; ++w) t += red[w];
        partial[blockIdx.x] = t;
    }
}

// kSum: offs holds the blocks' unscanned sums and each block adds up those
// before it (a few KB from L2 for at most kScanSumMax blocks) -- one launch
// fewer than scanning the sums first.
template <typename TIn, bool kSum = false>
__global__ void __launch_bounds__(kScanThreads) scan_apply_kernel(const TIn *__restrict__ in, int64_t n,
                                                                  const int64_t *__restrict__ offs,
                                                                  int64_t *__restrict__ out) {
    __shared__ int64_t s[kScanTile];
    __shared__ int64_t s_off[kScanThreads / 32];
    const int64_t base = (int64_t)blockIdx.x * kScanTile;
    int64_t before = 0;
    if (kSum)
        for (int i = threadIdx.x; i < (int)blockIdx.x; i += kScanThreads) before += offs[i];
    for (int i = threadIdx.x; i < kScanTile; i += kScanThreads) {
        int64_t g = base + i;
        s[i] = g < n ? (int64_t)in[g] : 0;
    }
    if (kSum) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) before += __shfl_down_sync(0xffffffffu, before, o);
        if ((threadIdx.x & 31) == 0) s_off[threadIdx.x >> 5] = before;
    }
    __syncthreads();
    block_scan_tile(s);  // synchronises the block, so s_off is complete
    int64_t off = 0;
    if (kSum) {
#pragma unroll
        for (int w = 0; w < kScanThreads / 32; ++w) off += s_off[w];
    } else if (offs) {
        off = offs[blockIdx.x];
    }
    for (int i = threadIdx.x; i < kScanTile; i += kScanThreads) {
        int64_t g = base + i;
        if (g < n) out[g] = s[i] + off;
    }
}

template <typename TIn>
cnn_status scan_impl(cnn_context *ctx, const TIn *in, int64_t *out, int64_t n, size_t tmp_off) {
    if (n <= 0) return CNN_OK;
    const int64_t nb = (n + kScanTile - 1) / kScanTile;
    if (nb == 1) {
        scan_apply_kernel<TIn><<<1, kScanThreads, 0, ctx->stream>>>(in, n, nullptr, out);
        CNN_LAUNCH_CHECK(ctx);
        return CNN_OK;
    }
    // partial sums of this level live in scan_tmp at tmp_off; the next
    // level follows them.
    size_t need = tmp_off + sizeof(int64_t) * (size_t)(2 * nb + 64);
    if (need > ctx->scan_tmp.cap) return ctx->fail(CNN_ERR_STATE, "scan temp too small");
    int64_t *partial = reinterpret_cast<int64_t *>(static_cast<char *>(ctx->scan_tmp.ptr) + tmp_off);
    int64_t *partial_scan = partial + nb;
    scan_reduce_kernel<TIn><<<(unsigned)nb, kScanThreads, 0, ctx->stream>>>(in, n, partial);
    CNN_LAUNCH_CHECK(ctx);
    if (nb <= kScanSumMax) {  // every block adds up the sums before it
        scan_apply_kernel<TIn, true><<<(unsigned)nb, kScanThreads, 0, ctx->stream>>>(in, n, partial, out);
        CNN_LAUNCH_CHECK(ctx);
        return CNN_OK;
    }
    size_t next_off = tmp_off + sizeof(int64_t) * (size_t)(2 * nb);
    next_off = (next_off + 255) & ~size_t(255);
    CNN_TRY(scan_impl<int64_t>(ctx, partial, partial_scan, nb, next_off));
    scan_apply_kernel<TIn><<<(unsigned)nb, kScanThreads, 0, ctx->stream>>>(in, n, partial_scan, out);
    CNN_LAUNCH_CHECK(ctx);
    return CNN_OK;
}

size_t scan_tmp_bytes(int64_t n) {
    size_t total = 0;
    int64_t m = n;
    while (m > kScanTile) {
        int64_t nb = (m + kScanTile - 1) / kScanTile;
        total += sizeof(int64_t) * (size_t)(2 * nb) + 256;
        m = nb;
    }
    return total + 4096;
}

// ---------------------------------------------------------------------------
// LSD radix sort of uint64 keys, 8 bits per pass.
// ---------------------------------------------------------------------------
constexpr int kRadixThreads = 256;
constexpr int kRadixItems = 8;
constexpr int kRadixTile = kRadixThreads * kRadixItems;  // 2048
constexpr int kRadixWarps = kRadixThreads / 32;

// n_dev (optional): the key count on the device, at most n (grids are sized
// for n; tiles past the count hold no keys)
__device__ __forceinline__ int64_t key_count(int64_t n, const int64_t *n_dev) {
    if (!n_dev) return n;
    const int64_t m = *n_dev;
    return m < 0 ? 0 : (m < n ? m : n);
}

__global__ void __launch_bounds__(kRadixThreads) radix_hist_kernel(const uint64_t *__restrict__ keys, int64_t n_max,
                                                                   const int64_t *__restrict__ n_dev, int shift,
                                                                   int64_t ntiles, int32_t *__restrict__ hist) {
    const int64_t n = key_count(n_max, n_dev);
    __shared__ int32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * kRadixTile;
    for (int i = threadIdx.x; i < kRadixTile; i += kRadixThreads) {
        int64_t g = base + i;
        if (g < n) atomicAdd(&h[(keys[g] >> shift) & 0xff], 1);
    }
    __syncthreads();
    hist[(int64_t)threadIdx.x * ntiles + blockIdx.x] = h[threadIdx.x];
}

// Stable scatter of one tile: keys are ranked by digit within the tile
// (warp match_any ranks + per-warp digit counts), placed in digit order in
// shared memory, then written out so that consecutive threads write
// consecutive addresses of each digit's run (coalesced stores).
__global__ void __launch_bounds__(kRadixThreads, 2) radix_scatter_kernel(const uint64_t *__restrict__ keys,
                                                                      uint64_t *__restrict__ out, int64_t n_max,
                                                                      const int64_t *__restrict__ n_dev, int shift,
                                                                      int64_t ntiles,
                                                                      const int64_t *__restrict__ goff) {
    const int64_t n = key_count(n_max, n_dev);
    __shared__ int32_t wcount[kRadixWarps][256];
    __shared__ int64_t tile_off[256];
    __shared__ int32_t digit_start[257];
    __shared__ uint64_t staged[kRadixTile];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < kRadixWarps * 256; i += kRadixThreads) (&wcount[0][0])[i] = 0;
    tile_off[threadIdx.x] = goff[(int64_t)threadIdx.x * ntiles + blockIdx.x];
    __syncthreads();
    const int64_t tile0 = (int64_t)blockIdx.x * kRadixTile;
    const int64_t base = tile0 + (int64_t)w * (kRadixItems * 32);
    const unsigned lt = (1u << lane) - 1u;
    uint64_t k[kRadixItems];
    int32_t rank[kRadixItems];
    int32_t dig[kRadixItems];
#pragma unroll
    for (int it = 0; it < kRadixItems; ++it) {
        int64_t g = base + it * 32 + lane;
        bool valid = g < n;
        k[it] = valid ? keys[g] : 0;
        int d = valid ? (int)((k[it] >> shift) & 0xff) : (0x100 | lane);
        unsigned peers = __match_any_sync(0xffffffffu, d);
        int before = __popc(peers & lt);
        int cnt = valid ? wcount[w][d] : 0;
        __syncwarp();
        if (valid && before == 0) wcount[w][d] = cnt + __popc(peers);
        __syncwarp();
        rank[it] = cnt + before;
        dig[it] = valid ? d : -1;
    }
    __syncthreads();
    int32_t digit_total;
    {
        const int t = threadIdx.x;  // one digit per thread: offsets of the warps within the digit
        int32_t run = 0;
#pragma unroll
        for (int ww = 0; ww < kRadixWarps; ++ww) {
            int32_t c = wcount[ww][t];
            wcount[ww][t] = run;
            run += c;
        }
        digit_total = run;
    }
    // exclusive scan of the digit totals (256 threads, one digit each)
    {
        __shared__ int32_t scan_buf[256];
        scan_buf[threadIdx.x] = digit_total;
        __syncthreads();
        for (int o = 1; o < 256; o <<= 1) {
            const int32_t v = threadIdx.x >= o ? scan_buf[threadIdx.x - o] : 0;
            __syncthreads();
            scan_buf[threadIdx.x] += v;
            __syncthreads();
        }
        digit_start[threadIdx.x] = scan_buf[threadIdx.x] - digit_total;
        if (threadIdx.x == 255) digit_start[256] = scan_buf[255];
    }
    __syncthreads();
#pragma unroll
    for (int it = 0; it < kRadixItems; ++it)
        if (dig[it] >= 0) staged[digit_start[dig[it]] + wcount[w][dig[it]] + rank[it]] = k[it];
    __syncthreads();
    const int valid_in_tile = digit_start[256];
    for (int i = threadIdx.x; i < valid_in_tile; i += kRadixThreads) {
        const uint64_t key = staged[i];
        const int d = (int)((key >> shift) & 0xff);
        out[tile_off[d] + (i - digit_start[d])] = key;
    }
}

__global__ void fill_i32_kernel(int32_t *p, int64_t n, int32_t v) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        p[i] = v;
}

__global__ void iota_i32_kernel(int32_t *p, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        p[i] = (int32_t)i;
}

}  // namespace

cnn_status scan_exclusive_i64(cnn_context *ctx, const int64_t *in, int64_t *out, int64_t n) {
    CNN_TRY(ctx->ensure(ctx->scan_tmp, scan_tmp_bytes(n)));
    return scan_impl<int64_t>(ctx, in, out, n, 0);
}

cnn_status scan_exclusive_i32_to_i64(cnn_context *ctx, const int32_t *in, int64_t *out, int64_t n) {
    CNN_TRY(ctx->ensure(ctx->scan_tmp, scan_tmp_bytes(n)));
    return scan_impl<int32_t>(ctx, in, out, n, 0);
}

// Up to kSmallSort keys: one block, bitonic sort in shared memory.
constexpr int kSmallSort = 4096;

__global__ void __launch_bounds__(1024) small_sort_kernel(uint64_t *__restrict__ keys, int n_max,
                                                          const int64_t *__restrict__ n_dev) {
    const int n = (int)key_count(n_max, n_dev);
    __shared__ uint64_t s[kSmallSort];
    int m = 1;
    while (m < n) m <<= 1;
    for (int i = threadIdx.x; i < m; i += blockDim.x) s[i] = i < n ? keys[i] : ~0ull;
    __syncthreads();
    for (int k = 2; k <= m; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < m; i += blockDim.x) {
                const int p = i ^ j;
                if (p > i) {
                    const uint64_t a = s[i], b = s[p];
                    const bool up = (i & k) == 0;
                    if ((a > b) == up) {
                        s[i] = b;
                        s[p] = a;
                    }
                }
            }
            __syncthreads();
        }
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) keys[i] = s[i];
}

// Sorts keys[0..n) ascending by their bits [first_bit, bits) (higher bits
// must be zero; bits below first_bit must already be in ascending order
// within equal higher bits, which the stable passes keep -- e.g. an index
// in the low bits of keys built in index order).  Uses scratch_c/scratch_d
// and the scan temp.
// n_dev (optional): the key count is read on the device (at most n), so the
// sort enqueues the same work whatever the count -- no host round trip.
cnn_status radix_sort_u64(cnn_context *ctx, uint64_t *keys, int64_t n, int bits, int first_bit, uint64_t **sorted,
                          const int64_t *n_dev) {
    if (sorted) *sorted = keys;
    if (n <= 1) return CNN_OK;
    if (bits < 1) bits = 1;
    if (bits > 64) bits = 64;
    if (n <= kSmallSort) {  // every key distinct or not, a full sort gives the same order
        small_sort_kernel<<<1, 1024, 0, ctx->stream>>>(keys, (int)n, n_dev);
        CNN_LAUNCH_CHECK(ctx);
        return CNN_OK;
    }
    first_bit = first_bit < 0 ? 0 : (first_bit / 8) * 8;
    const int64_t ntiles = (n + kRadixTile - 1) / kRadixTile;
    const int64_t nh = 256 * ntiles;
    CNN_TRY(ctx->ensure(ctx->scratch_c, sizeof(uint64_t) * (size_t)n));
    CNN_TRY(ctx->ensure(ctx->scratch_d, (sizeof(int32_t) + sizeof(int64_t)) * (size_t)nh + 256));
    CNN_TRY(ctx->ensure(ctx->scan_tmp, scan_tmp_bytes(nh)));
    int32_t *hist = ctx->scratch_d.as<int32_t>();
    int64_t *goff = reinterpret_cast<int64_t *>(
        (reinterpret_cast<uintptr_t>(hist + nh) + 15) & ~uintptr_t(15));
    uint64_t *a = keys, *b = ctx->scratch_c.as<uint64_t>();
    const int passes = (bits - first_bit + 7) / 8;
    for (int p = 0; p < passes; ++p) {
        const int shift = first_bit + p * 8;
        radix_hist_kernel<<<(unsigned)ntiles, kRadixThreads, 0, ctx->stream>>>(a, n, n_dev, shift, ntiles, hist);
        CNN_LAUNCH_CHECK(ctx);
        CNN_TRY(scan_impl<int32_t>(ctx, hist, goff, nh, 0));
        radix_scatter_kernel<<<(unsigned)ntiles, kRadixThreads, 0, ctx->stream>>>(a, b, n, n_dev, shift, ntiles,
                                                                                 goff);
        CNN_LAUNCH_CHECK(ctx);
        uint64_t *t = a; a = b; b = t;
    }
    if (sorted) {
        *sorted = a;  // the caller reads the result where the last pass left it
    } else if (a != keys) {
        CNN_CUDA(ctx, cudaMemcpyAsync(keys, a, sizeof(uint64_t) * (size_t)n, cudaMemcpyDeviceToDevice, ctx->stream));
    }
    return CNN_OK;
}

cnn_status read_back(cnn_context *ctx, void *host, const void *dev, size_t bytes) {
    if (bytes == 0) return CNN_OK;
    if (ctx->host_small && bytes <= cnn_context::kHostSmall) {
        CNN_CUDA(ctx, cudaMemcpyAsync(ctx->host_small, dev, bytes, cudaMemcpyDeviceToHost, ctx->stream));
        CNN_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        memcpy(host, ctx->host_small, bytes);
        return CNN_OK;
    }
    CNN_CUDA(ctx, cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    CNN_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return CNN_OK;
}

// The dynamic shared-memory limit is a property of the kernel on a device,
// shared by every thread and context of the process: it is only ever raised
// (under a lock), so a launch sized under a limit set earlier stays valid
// while another thread raises it for a bigger launch of the same kernel.
cnn_status allow_dynamic_smem(cnn_context *ctx, const void *kernel, size_t bytes) {
    static std::mutex mu;
    static std::map<std::pair<int, const void *>, size_t> limit;
    std::lock_guard<std::mutex> lock(mu);
    size_t &cur = limit[std::make_pair(ctx->device, kernel)];
    if (bytes <= cur) return CNN_OK;
    CNN_CUDA(ctx, cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    cur = bytes;
    return CNN_OK;
}

cnn_status fill_i32(cnn_context *ctx, int32_t *p, int64_t n, int32_t v) {
    if (n <= 0) return CNN_OK;
    fill_i32_kernel<<<grid_for(n, 256) > 4096 ? 4096 : grid_for(n, 256), 256, 0, ctx->stream>>>(p, n, v);
    CNN_LAUNCH_CHECK(ctx);
    return CNN_OK;
}

cnn_status iota_i32(cnn_context *ctx, int32_t *p, int64_t n) {
    if (n <= 0) return CNN_OK;
    iota_i32_kernel<<<grid_for(n, 256) > 4096 ? 4096 : grid_for(n, 256), 256, 0, ctx->stream>>>(p, n);
    CNN_LAUNCH_CHECK(ctx);
    return CNN_OK;
}

}  // namespace cnn
