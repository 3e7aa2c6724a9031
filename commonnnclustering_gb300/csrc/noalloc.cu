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
// stream capture), and passed to the kernels as a pointer.  The cached
// address belongs to the device's primary context: after cudaDeviceReset the
// entry point must not be called again in that process.
//
// The graph is checked on the device before the fit reads it: offsets must
// start at 0 and not decrease, no row may hold more than n_points entries,
// and every row must be strictly ascending with indices in [0, n_points).  A
// graph that fails the check is not fitted: labels and consider are left
// exactly as they were (a valid call always leaves every consider entry 0).
#include <algorithm>
#include <mutex>

#include "common.cuh"
#include "fit_kernels.cuh"

namespace cnn {
namespace {

constexpr int64_t kNoAllocMaxPoints = CNN_NOALLOC_MAX_POINTS;
constexpr int kBadGraph = 15;  // counters slot: entries that failed the graph check

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

// What the first call on a device looks up: the scratch block's device
// address and the launch sizes of the fit kernels on that device.
struct DeviceSetup {
    NoAllocScratch *scratch = nullptr;
    unsigned small_blocks = 0;  // grid of the per-point kernels
    unsigned check_blocks = 0;  // resident blocks of the check kernel
};

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
DeviceSetup g_setup[kMaxDevices];

cnn_status setup_for_current_device(DeviceSetup *out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        (void)cudaGetLastError();
        return CNN_ERR_CUDA;
    }
    std::lock_guard<std::mutex> lock(g_setup_mu);
    DeviceSetup &s = g_setup[dev];
    if (!s.scratch) {
        void *ptr = nullptr;
        int sms = 0, per_sm = 0;
        if (cudaGetSymbolAddress(&ptr, g_fit_scratch) != cudaSuccess || !ptr ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1 ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, check_union_kernel<false>, kCheckWarps * 32, 0) !=
                cudaSuccess) {
            (void)cudaGetLastError();
            return CNN_ERR_CUDA;
        }
        s.small_blocks = (unsigned)sms * 4u;
        s.check_blocks = (unsigned)sms * (unsigned)std::max(1, per_sm);
        s.scratch = static_cast<NoAllocScratch *>(ptr);
    }
    *out = s;
    return CNN_OK;
}

// Per-point set-up: degree from the offsets, identity order, zeroed flags
// and counters (the scratch keeps the previous call's values).
__global__ void noalloc_prepare_kernel(const int64_t *__restrict__ offsets, int64_t n, NoAllocScratch *sc) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p <= n; p += (int64_t)gridDim.x * blockDim.x) {
        sc->flag[p] = 0;
        if (p < n) {
            const int64_t len = offsets[p + 1] - offsets[p];
            sc->deg[p] = (int32_t)(len < 0 ? 0 : len > n ? n : len);  // a bad row is rejected below
            sc->perm[p] = (int32_t)p;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x < 16) sc->counters[threadIdx.x] = 0;
}

// Offsets check (after the counters are zeroed): start at 0, every row holds
// 0..n entries.  Then offsets never decrease, so every row lies inside the
// offsets[n] entries the caller's indices array holds.
__global__ void noalloc_offsets_kernel(const int64_t *__restrict__ offsets, int64_t n, NoAllocScratch *sc) {
    unsigned long long bad = 0;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p <= n; p += (int64_t)gridDim.x * blockDim.x) {
        if (p < n) {
            const int64_t len = offsets[p + 1] - offsets[p];
            bad += (len < 0 || len > n) ? 1 : 0;
        } else {
            bad += offsets[0] != 0 ? 1 : 0;
        }
    }
    for (int o = 16; o > 0; o >>= 1) bad += __shfl_down_sync(0xffffffffu, bad, o);
    if ((threadIdx.x & 31) == 0 && bad) atomicAdd(&sc->counters[kBadGraph], bad);
}

// Row check, one warp per row, only when the offsets passed: indices in
// [0, n), strictly ascending.  Counts every bad entry into
// counters[kBadGraph].
__global__ void noalloc_rows_kernel(const int64_t *__restrict__ offsets, const int32_t *__restrict__ indices,
                                    int64_t n, NoAllocScratch *sc) {
    if (sc->counters[kBadGraph] != 0) return;  // offsets bad: the rows cannot be walked safely
    const int lane = threadIdx.x & 31;
    const int64_t warp0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    unsigned long long bad = 0;
    for (int64_t p = warp0; p < n; p += nwarps) {
        const int64_t s = offsets[p], e = offsets[p + 1];
        for (int64_t k = s + lane; k < e; k += 32) {
            const int32_t c = indices[k];
            const bool ok = c >= 0 && (int64_t)c < n && (k == s || indices[k - 1] < c);
            bad += ok ? 0 : 1;
        }
    }
    for (int o = 16; o > 0; o >>= 1) bad += __shfl_down_sync(0xffffffffu, bad, o);
    if (lane == 0 && bad) atomicAdd(&sc->counters[kBadGraph], bad);
}

// After node_kernel: a rejected graph has no nodes, so no later kernel reads
// its rows, writes a label or touches the union-find.
__global__ void noalloc_gate_kernel(int64_t n, NoAllocScratch *sc) {
    if (sc->counters[kBadGraph] == 0) return;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
        sc->node[p] = 0;
        sc->parent[p] = -1;
    }
}

// consider = 0 for every point (the reference's loop visits them all),
// unless the graph was rejected.
__global__ void noalloc_consider_kernel(int64_t n, const NoAllocScratch *sc, uint8_t *__restrict__ consider) {
    if (sc->counters[kBadGraph] != 0) return;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x)
        consider[p] = 0;
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

}  // namespace
}  // namespace cnn

using namespace cnn;

// Checked after every launch: a launch error stops the call (kernels queued
// before it still run).
#define NOALLOC_LAUNCHED()                                       \
    do {                                                         \
        if (cudaGetLastError() != cudaSuccess) return CNN_ERR_CUDA; \
    } while (0)

extern "C" CNN_API cnn_status cnn_fit_csr_noalloc(const int64_t *offsets, const int32_t *indices, int64_t n_points,
                                                  int64_t similarity_cutoff, int64_t n_member_cutoff,
                                                  int64_t current_start, uint8_t *consider, int64_t *labels,
                                                  void *stream) {
    if (n_points < 0 || n_points > kNoAllocMaxPoints) return CNN_ERR_INVALID_ARG;
    if (n_points == 0) return CNN_OK;
    if (!offsets || !indices || !consider || !labels) return CNN_ERR_INVALID_ARG;
    // an error the caller left pending is theirs: report it, clear nothing
    if (cudaPeekAtLastError() != cudaSuccess) return CNN_ERR_CUDA;
    DeviceSetup su;
    CNN_TRY(setup_for_current_device(&su));
    NoAllocScratch *sc = su.scratch;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int64_t n = n_points;
    if (similarity_cutoff > INT32_MAX) similarity_cutoff = INT32_MAX;
    if (similarity_cutoff < -1) similarity_cutoff = -1;
    unsigned long long *counters = sc->counters;
    const unsigned pb = std::min<unsigned>(grid_for(n + 1, 256), su.small_blocks);
    const unsigned cb = std::min<unsigned>(grid_for(n, kCheckWarps), su.check_blocks);

    noalloc_prepare_kernel<<<pb, 256, 0, st>>>(offsets, n, sc);
    NOALLOC_LAUNCHED();
    noalloc_offsets_kernel<<<pb, 256, 0, st>>>(offsets, n, sc);
    NOALLOC_LAUNCHED();
    noalloc_rows_kernel<<<std::min<unsigned>(grid_for(n * 32, 256), su.small_blocks), 256, 0, st>>>(offsets, indices,
                                                                                                   n, sc);
    NOALLOC_LAUNCHED();
    node_kernel<<<pb, 256, 0, st>>>(sc->deg, sc->perm, consider, n, n_member_cutoff, sc->node, sc->parent,
                                    sc->comp_min, counters);
    NOALLOC_LAUNCHED();
    noalloc_gate_kernel<<<pb, 256, 0, st>>>(n, sc);
    NOALLOC_LAUNCHED();
    check_union_kernel<false><<<cb, kCheckWarps * 32, 0, st>>>(n, offsets, offsets + 1, indices, sc->parent,
                                                        (int32_t)similarity_cutoff, kHookEdges, counters, nullptr,
                                                        nullptr);
    NOALLOC_LAUNCHED();
    root_store_kernel<<<pb, 256, 0, st>>>(n, sc->node, sc->parent);
    NOALLOC_LAUNCHED();
    check_union_kernel<false><<<cb, kCheckWarps * 32, 0, st>>>(n, offsets, offsets + 1, indices, sc->parent,
                                                        (int32_t)similarity_cutoff, INT32_MAX, counters, nullptr,
                                                        nullptr);
    NOALLOC_LAUNCHED();
    root_min_kernel<<<pb, 256, 0, st>>>(n, sc->node, sc->parent, sc->perm, sc->comp_min);
    NOALLOC_LAUNCHED();
    root_store_kernel<<<pb, 256, 0, st>>>(n, sc->node, sc->parent);
    NOALLOC_LAUNCHED();
    min_flag_kernel<<<pb, 256, 0, st>>>(n, sc->node, sc->parent, sc->comp_min, sc->flag);
    NOALLOC_LAUNCHED();
    noalloc_scan_kernel<<<1, 1024, 0, st>>>(sc->flag, sc->rank, n + 1);
    NOALLOC_LAUNCHED();
    label_kernel<<<pb, 256, 0, st>>>(n, sc->node, sc->parent, sc->comp_min, sc->perm, sc->rank, current_start,
                                     labels);
    NOALLOC_LAUNCHED();
    noalloc_consider_kernel<<<pb, 256, 0, st>>>(n, sc, consider);
    NOALLOC_LAUNCHED();
    return CNN_OK;
}
