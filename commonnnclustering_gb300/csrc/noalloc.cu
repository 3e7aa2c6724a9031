// noalloc.cu -- cnn_fit_csr_noalloc: the CommonNN fit over a caller-provided
// neighbour graph without any device memory allocation.
//
// Who needs it: callers that may not allocate device memory once they are
// running.  A serving loop that fixes its memory budget at start-up, a
// plug-in living inside a framework whose caching allocator has already
// reserved the free memory, or a latency-critical loop that must not pay for
// (or be stalled by) cudaMalloc/cudaFree -- both can synchronise the whole
// device.  Such a caller owns the inputs and outputs; everything else the fit
// needs lives in one fixed scratch block below.
//
// Scratch: a file-scope __device__ array sized for kNoAllocMaxPoints points
// (about 1.9 MB).  Every GPU that loads this library holds it until the
// process exits.  All calls share it and it keeps the contents of the last
// call, so each call re-initialises everything it reads before reading it;
// calls whose GPU work overlaps (two streams, two host threads) race on it.
//
// Host code cannot pass the array's name to a kernel: on the host that name
// is a stand-in, not a device address.  The device address is taken once per
// device with cudaGetSymbolAddress, with that device current, by the first
// call on that device (so the first call on a device should come before any
// stream capture), and passed to the kernels as a pointer.
#include <mutex>

#include "common.cuh"
#include "fit_kernels.cuh"

namespace cnn {
namespace {

constexpr int64_t kNoAllocMaxPoints = CNN_NOALLOC_MAX_POINTS;

struct NoAllocScratch {
    int64_t rank[kNoAllocMaxPoints + 1];
    int32_t deg[kNoAllocMaxPoints];
    int32_t perm[kNoAllocMaxPoints];
    int32_t parent[kNoAllocMaxPoints];
    int32_t comp_min[kNoAllocMaxPoints];
    int32_t flag[kNoAllocMaxPoints + 1];
    uint8_t node[kNoAllocMaxPoints];
    unsigned long long counters[16];
};

static __device__ __align__(256) NoAllocScratch g_fit_scratch;

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
NoAllocScratch *g_scratch_addr[kMaxDevices] = {};

// Device address of the scratch block on the current device (set-up on the
// first call per device).
cnn_status scratch_for_current_device(NoAllocScratch **out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        (void)cudaGetLastError();
        return CNN_ERR_CUDA;
    }
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_addr[dev]) {
        void *ptr = nullptr;
        if (cudaGetSymbolAddress(&ptr, g_fit_scratch) != cudaSuccess || !ptr) {
            (void)cudaGetLastError();
            return CNN_ERR_CUDA;
        }
        g_scratch_addr[dev] = static_cast<NoAllocScratch *>(ptr);
    }
    *out = g_scratch_addr[dev];
    return CNN_OK;
}

// Per-point set-up: degree from the offsets, identity order, zeroed flags
// and counters (the scratch keeps the previous call's values).
__global__ void noalloc_prepare_kernel(const int64_t *__restrict__ offsets, int64_t n, NoAllocScratch *sc) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p <= n; p += (int64_t)gridDim.x * blockDim.x) {
        sc->flag[p] = 0;
        if (p < n) {
            sc->deg[p] = (int32_t)(offsets[p + 1] - offsets[p]);
            sc->perm[p] = (int32_t)p;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x < 16) sc->counters[threadIdx.x] = 0;
}

// Exclusive scan of flag[0..m) into rank[0..m) by one block (m <= 65,537).
__global__ void __launch_bounds__(1024) noalloc_scan_kernel(const int32_t *__restrict__ in, int64_t *__restrict__ out,
                                                            int64_t m) {
    __shared__ int64_t warp_sum[32];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    const int64_t per = (m + blockDim.x - 1) / blockDim.x;
    const int64_t b = t * per, e = b + per < m ? b + per : m;
    int64_t local = 0;
    for (int64_t i = b; i < e; ++i) local += in[i];
    int64_t incl = local;
    for (int o = 1; o < 32; o <<= 1) {
        const int64_t u = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += u;
    }
    if (lane == 31) warp_sum[w] = incl;
    __syncthreads();
    if (w == 0) {
        const int64_t v = lane < (int)(blockDim.x >> 5) ? warp_sum[lane] : 0;
        int64_t vi = v;
        for (int o = 1; o < 32; o <<= 1) {
            const int64_t u = __shfl_up_sync(0xffffffffu, vi, o);
            if (lane >= o) vi += u;
        }
        if (lane < (int)(blockDim.x >> 5)) warp_sum[lane] = vi - v;
    }
    __syncthreads();
    int64_t run = warp_sum[w] + incl - local;
    for (int64_t i = b; i < e; ++i) {
        out[i] = run;
        run += in[i];
    }
}

unsigned nblocks(int64_t n) { return std::min<unsigned>(grid_for(n, 256), 152u * 4u); }

}  // namespace
}  // namespace cnn

using namespace cnn;

extern "C" CNN_API cnn_status cnn_fit_csr_noalloc(const int64_t *offsets, const int32_t *indices, int64_t n_points,
                                                  int64_t similarity_cutoff, int64_t n_member_cutoff,
                                                  int64_t current_start, uint8_t *consider, int64_t *labels,
                                                  void *stream) {
    if (n_points < 0 || n_points > kNoAllocMaxPoints) return CNN_ERR_INVALID_ARG;
    if (n_points == 0) return CNN_OK;
    if (!offsets || !indices || !consider || !labels) return CNN_ERR_INVALID_ARG;
    NoAllocScratch *sc = nullptr;
    CNN_TRY(scratch_for_current_device(&sc));
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int64_t n = n_points;
    if (similarity_cutoff > INT32_MAX) similarity_cutoff = INT32_MAX;
    if (similarity_cutoff < -1) similarity_cutoff = -1;
    unsigned long long *counters = sc->counters;

    noalloc_prepare_kernel<<<nblocks(n + 1), 256, 0, st>>>(offsets, n, sc);
    node_kernel<<<nblocks(n), 256, 0, st>>>(sc->deg, sc->perm, consider, n, n_member_cutoff, sc->node, sc->parent,
                                            sc->comp_min, counters);
    const unsigned check_blocks = std::min<unsigned>(grid_for(n, kCheckWarps), 152u * CNN_CHECK_MIN_BLOCKS);
    check_union_kernel<<<check_blocks, kCheckWarps * 32, 0, st>>>(n, offsets, indices, sc->parent,
                                                                   (int32_t)similarity_cutoff, 2, counters, nullptr, nullptr);
    root_store_kernel<<<nblocks(n), 256, 0, st>>>(n, sc->node, sc->parent);
    check_union_kernel<<<check_blocks, kCheckWarps * 32, 0, st>>>(n, offsets, indices, sc->parent,
                                                                   (int32_t)similarity_cutoff, INT32_MAX, counters, nullptr,
                                                                   nullptr);
    root_min_kernel<<<nblocks(n), 256, 0, st>>>(n, sc->node, sc->parent, sc->perm, sc->comp_min);
    root_store_kernel<<<nblocks(n), 256, 0, st>>>(n, sc->node, sc->parent);
    min_flag_kernel<<<nblocks(n), 256, 0, st>>>(n, sc->node, sc->parent, sc->comp_min, sc->flag);
    noalloc_scan_kernel<<<1, 1024, 0, st>>>(sc->flag, sc->rank, n + 1);
    label_kernel<<<nblocks(n), 256, 0, st>>>(n, sc->node, sc->parent, sc->comp_min, sc->perm, sc->rank,
                                             current_start, labels);
    if (cudaGetLastError() != cudaSuccess) return CNN_ERR_CUDA;
    if (cudaMemsetAsync(consider, 0, (size_t)n, st) != cudaSuccess) {
        (void)cudaGetLastError();
        return CNN_ERR_CUDA;
    }
    return CNN_OK;
}
