// cnngpu.cu -- the C ABI: context lifetime, argument checks, host<->device
// staging, and dispatch to the kernels in search.cu / fit.cu / prims.cu.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <new>
#include <utility>
#include <vector>

#include "common.cuh"

namespace cnn {

void stage_begin(cnn_context *ctx, int slot) {
    if (!ctx->timing || slot < 0 || slot >= cnn_context::kSlots) return;
    cudaEventRecord(ctx->ev_begin[slot], ctx->stream);
}

void stage_end(cnn_context *ctx, int slot) {
    if (!ctx->timing || slot < 0 || slot >= cnn_context::kSlots) return;
    cudaEventRecord(ctx->ev_end[slot], ctx->stream);
    ctx->slot_pending[slot] = true;
}

// the cnn_stats field each stage slot's events time
static float *stage_field(cnn_context *ctx, int slot) {
    float *f[cnn_context::kSlots] = {
        &ctx->stats.ms_bbox, &ctx->stats.ms_cells, &ctx->stats.ms_count, &ctx->stats.ms_scan,
        &ctx->stats.ms_fill, &ctx->stats.ms_nodes, &ctx->stats.ms_check, &ctx->stats.ms_label,
        &ctx->stats.ms_sort, &ctx->stats.ms_gram, &ctx->stats.ms_weights, nullptr};
    return slot >= 0 && slot < cnn_context::kSlots ? f[slot] : nullptr;
}

void stages_reset(cnn_context *ctx, int first, int last) {
    for (int i = first; i <= last && i < cnn_context::kSlots; ++i) {
        ctx->slot_pending[i] = false;  // a stage this call skips reports 0, not an older time
        if (float *f = stage_field(ctx, i)) *f = 0.f;
    }
}

namespace {

__global__ void widen_f32_kernel(const float *__restrict__ in, int64_t total, double *__restrict__ out) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x)
        out[e] = (double)in[e];
}

bool metric_known(int metric) {
    return metric == CNN_METRIC_EUCLIDEAN_REDUCED || metric == CNN_METRIC_EUCLIDEAN ||
           metric == CNN_METRIC_PRECOMPUTED || metric == CNN_METRIC_EUCLIDEAN_PERIODIC_REDUCED;
}

// The metric needs points (or, precomputed, distances) on the context.
cnn_status check_source(cnn_context *ctx, int metric) {
    if (metric == CNN_METRIC_PRECOMPUTED) {
        if (!ctx->dist_set) return ctx->fail(CNN_ERR_STATE, "no distances: call cnn_set_distances first");
        return CNN_OK;
    }
    if (ctx->d < 1) return ctx->fail(CNN_ERR_STATE, "no points: call cnn_set_points first");
    return CNN_OK;
}

cnn_status check_ctx(cnn_context *ctx) {
    if (!ctx) return CNN_ERR_INVALID_ARG;
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return ctx->fail(CNN_ERR_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
    return CNN_OK;
}

// Copy a host array into a staging buffer or pass a device pointer through.
template <typename T>
cnn_status stage_in(cnn_context *ctx, cnn::DevBuf &buf, const T *src, int64_t count, cnn_memspace mem,
                    const T **dev_out) {
    if (mem == CNN_MEM_DEVICE) {
        *dev_out = src;
        return CNN_OK;
    }
    CNN_TRY(ctx->ensure(buf, sizeof(T) * (size_t)(count > 0 ? count : 1)));
    if (count > 0)
        CNN_CUDA(ctx, cudaMemcpyAsync(buf.ptr, src, sizeof(T) * (size_t)count, cudaMemcpyHostToDevice, ctx->stream));
    *dev_out = buf.as<T>();
    return CNN_OK;
}

}  // namespace
}  // namespace cnn

using namespace cnn;

namespace cnn {
namespace {

std::vector<DevBuf *> workspace_buffers(cnn_context *ctx) {
    return {&ctx->x_own, &ctx->x_f32_stage, &ctx->perm, &ctx->inv, &ctx->deg, &ctx->row_off,
                           &ctx->cols, &ctx->xf4, &ctx->cell_of, &ctx->cell_start, &ctx->grid_slot_base,
                           &ctx->grid_slot_cols, &ctx->grid_qslot, &ctx->grid_qend, &ctx->node, &ctx->parent,
                           &ctx->comp_min, &ctx->flag, &ctx->counters, &ctx->stage_labels, &ctx->gram_hi, &ctx->gram_mid,
                           &ctx->gram_lo, &ctx->gram_aux, &ctx->gram_masks, &ctx->gram_tkeys, &ctx->gram_low, &ctx->gram_pad2c, &ctx->gram_rowwork, &ctx->gram_chunkcnt, &ctx->gram_amb,
                           &ctx->gram_blocks, &ctx->gram_tiles, &ctx->gram_perm, &ctx->pred_off, &ctx->pred_cols,
                           &ctx->pred_xoff, &ctx->pred_xcols, &ctx->pred_x, &ctx->pred_set,
                           &ctx->sweep_bucket, &ctx->sweep_row_off_max, &ctx->sweep_cols_max,
                           &ctx->sweep_deg_max, &ctx->sweep_consider, &ctx->sweep_forest, &ctx->sweep_open_a,
                           &ctx->sweep_multi_deg, &ctx->sweep_multi_off, &ctx->sweep_multi_cols, &ctx->sweep_multi_base,
                           &ctx->sweep_open_b, &ctx->sweep_open_count,
                           &ctx->stage_consider, &ctx->stage_offsets, &ctx->stage_indices, &ctx->stage_misc,
                           &ctx->pcell, &ctx->mbase, &ctx->masks, &ctx->dist_own, &ctx->bounds_dev,
                           &ctx->tune_consider, &ctx->tune_labels, &ctx->split,
                           &ctx->io_a, &ctx->io_b, &ctx->io_c, &ctx->scratch_a, &ctx->scratch_b,
                           &ctx->scratch_c, &ctx->scratch_d, &ctx->scan_tmp,
                           &ctx->cross_cell_of, &ctx->cross_slot, &ctx->cross_count, &ctx->cross_start,
                           &ctx->cross_perm, &ctx->cross_inv, &ctx->cross_xf4, &ctx->cross_units_n,
                           &ctx->cross_units_off, &ctx->cross_units, &ctx->cross_deg, &ctx->cross_row_off,
                           &ctx->cross_keys};
}

}  // namespace

cnn_status release_workspace(cnn_context *ctx) {
    CNN_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (DevBuf *b : workspace_buffers(ctx)) {
        if (b->ptr) cudaFree(b->ptr);
        *b = DevBuf{};
    }
    for (void *p : ctx->deferred_free) cudaFree(p);
    ctx->deferred_free.clear();
    if (ctx->sweep_exec) {
        cudaGraphExecDestroy(ctx->sweep_exec);
        ctx->sweep_exec = nullptr;
    }
    ctx->mem_held = 0;
    ctx->have_graph = false;
    ctx->graph_mask = false;
    ctx->csr_valid = true;
    ctx->graph_slots = false;
    ctx->nnz_pending = false;
    ctx->split_valid = false;
    ctx->tune_pending = false;
    ++ctx->graph_generation;
    ctx->x = nullptr;
    ctx->n = 0;
    ctx->d = 0;
    ctx->dist = nullptr;
    ctx->dist_set = false;
    return CNN_OK;
}

// The fit of cnn_fit on device arrays: the strategy of the graph's form,
// or -- the first fit of a new workload profile under CNN_INTERSECT_AUTO --
// both strategies from the same labels and consider, timed, the faster kept
// by the tuner.  Either way the cluster count is left in scratch_a[n].
cnn_status fit_dispatch(cnn_context *ctx, int64_t similarity_cutoff, int64_t n_member_cutoff, int64_t current_start,
                        uint8_t *cons_dev, int64_t *lab_dev) {
    const int64_t n = ctx->n;
    ctx->stats.tuned = 0;
    ctx->stats.tune_ms_merge = ctx->stats.tune_ms_bitset = 0.f;
    if (ctx->tune_pending && n > 0) {
        // the graph is in both forms: fit it both ways from the same labels
        // and consider, timed, and keep the faster strategy for this profile
        cudaStream_t st = ctx->stream;
        CNN_TRY(ctx->ensure(ctx->tune_consider, (size_t)n));
        CNN_TRY(ctx->ensure(ctx->tune_labels, sizeof(int64_t) * (size_t)n));
        CNN_CUDA(ctx, cudaMemcpyAsync(ctx->tune_consider.ptr, cons_dev, (size_t)n, cudaMemcpyDeviceToDevice, st));
        CNN_CUDA(ctx, cudaMemcpyAsync(ctx->tune_labels.ptr, lab_dev, sizeof(int64_t) * (size_t)n,
                                      cudaMemcpyDeviceToDevice, st));
        CNN_CUDA(ctx, cudaEventRecord(ctx->tune_ev[0], st));
        CNN_TRY(fit_mask_impl(ctx, similarity_cutoff, n_member_cutoff, current_start, cons_dev, lab_dev));
        CNN_CUDA(ctx, cudaEventRecord(ctx->tune_ev[1], st));
        CNN_CUDA(ctx, cudaMemcpyAsync(cons_dev, ctx->tune_consider.ptr, (size_t)n, cudaMemcpyDeviceToDevice, st));
        CNN_CUDA(ctx, cudaMemcpyAsync(lab_dev, ctx->tune_labels.ptr, sizeof(int64_t) * (size_t)n,
                                      cudaMemcpyDeviceToDevice, st));
        CNN_CUDA(ctx, cudaEventRecord(ctx->tune_ev[2], st));
        CNN_TRY(fit_impl(ctx, similarity_cutoff, n_member_cutoff, current_start, cons_dev, lab_dev));
        CNN_CUDA(ctx, cudaEventRecord(ctx->tune_ev[3], st));
        CNN_CUDA(ctx, cudaEventSynchronize(ctx->tune_ev[3]));
        float fm = 0.f, fl = 0.f;
        CNN_CUDA(ctx, cudaEventElapsedTime(&fm, ctx->tune_ev[0], ctx->tune_ev[1]));
        CNN_CUDA(ctx, cudaEventElapsedTime(&fl, ctx->tune_ev[2], ctx->tune_ev[3]));
        const float bitset = ctx->tune_ms_mask + fm, merge = ctx->tune_ms_lists + fl;
        const int choice = bitset < merge ? CNN_INTERSECT_BITSET : CNN_INTERSECT_MERGE;
        tuner_store(ctx->tune_key, choice);
        ctx->tune_pending = false;
        ctx->graph_mask = choice == CNN_INTERSECT_BITSET;  // both forms stay valid for this graph
        ctx->stats.tuned = 1;
        ctx->stats.tune_ms_merge = merge;
        ctx->stats.tune_ms_bitset = bitset;
        ctx->stats.intersection = choice;
    } else if (ctx->graph_mask) {
        CNN_TRY(fit_mask_impl(ctx, similarity_cutoff, n_member_cutoff, current_start, cons_dev, lab_dev));
        ctx->stats.intersection = CNN_INTERSECT_BITSET;
    } else {
        CNN_TRY(fit_impl(ctx, similarity_cutoff, n_member_cutoff, current_start, cons_dev, lab_dev));
        ctx->stats.intersection = CNN_INTERSECT_MERGE;
    }
    return CNN_OK;
}

}  // namespace cnn

extern "C" {

CNN_API int cnn_abi_version(void) { return CNN_ABI_VERSION; }

CNN_API cnn_status cnn_create(cnn_context **out, int device, void *stream) {
    if (!out) return CNN_ERR_INVALID_ARG;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count) {
        (void)cudaGetLastError();
        return CNN_ERR_CUDA;
    }
    cnn_context *ctx = new (std::nothrow) cnn_context();
    if (!ctx) return CNN_ERR_OOM;
    ctx->device = device;
    if (const char *pz = getenv("CNN_DEBUG_POISON")) ctx->poison = atoi(pz) & 0xff;
    if (const char *gr = getenv("CNN_GRID_REACH")) ctx->grid_reach = atoi(gr) == 2 ? 2 : 1;
    if (const char *sg = getenv("CNN_SWEEP_GRAPH")) ctx->sweep_graphs = atoi(sg) != 0;
    int sms = 0;
    if (cudaSetDevice(device) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || sms < 1) {
        (void)cudaGetLastError();
        delete ctx;
        return CNN_ERR_CUDA;
    }
    ctx->sm_count = (unsigned)sms;
    if (stream) {
        ctx->stream = static_cast<cudaStream_t>(stream);
    } else {
        if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
            delete ctx;
            return CNN_ERR_CUDA;
        }
        ctx->own_stream = true;
    }
    for (int i = 0; i < cnn_context::kSlots; ++i) {
        if (cudaEventCreate(&ctx->ev_begin[i]) != cudaSuccess || cudaEventCreate(&ctx->ev_end[i]) != cudaSuccess) {
            (void)cudaGetLastError();
            cnn_destroy(ctx);
            return CNN_ERR_CUDA;
        }
    }
    for (cudaEvent_t &e : ctx->tune_ev) {
        if (cudaEventCreate(&e) != cudaSuccess) {
            (void)cudaGetLastError();
            cnn_destroy(ctx);
            return CNN_ERR_CUDA;
        }
    }
    if (cudaMallocHost(&ctx->host_stats, 16 * sizeof(unsigned long long)) != cudaSuccess) {
        (void)cudaGetLastError();
        ctx->host_stats = nullptr;  // statistics are then read back with a sync
    }
    if (cudaMallocHost(&ctx->host_small, cnn_context::kHostSmall) != cudaSuccess) {
        (void)cudaGetLastError();
        ctx->host_small = nullptr;  // read-backs then go to pageable memory
    }
    *out = ctx;
    return CNN_OK;
}

CNN_API cnn_status cnn_destroy(cnn_context *ctx) {
    if (!ctx) return CNN_OK;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    for (cnn::DevBuf *b : cnn::workspace_buffers(ctx))
        if (b->ptr) cudaFree(b->ptr);
    for (void *p : ctx->deferred_free) cudaFree(p);
    if (ctx->sweep_exec) cudaGraphExecDestroy(ctx->sweep_exec);
    for (int i = 0; i < cnn_context::kSlots; ++i) {
        if (ctx->ev_begin[i]) cudaEventDestroy(ctx->ev_begin[i]);
        if (ctx->ev_end[i]) cudaEventDestroy(ctx->ev_end[i]);
    }
    for (cudaEvent_t e : ctx->tune_ev)
        if (e) cudaEventDestroy(e);
    if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
    if (ctx->host_stats) cudaFreeHost(ctx->host_stats);
    if (ctx->host_small) cudaFreeHost(ctx->host_small);
    (void)cudaGetLastError();
    delete ctx;
    return CNN_OK;
}

CNN_API cnn_status cnn_set_stream(cnn_context *ctx, void *stream) {
    CNN_TRY(check_ctx(ctx));
    CNN_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (ctx->own_stream) {
        cudaStreamDestroy(ctx->stream);
        ctx->own_stream = false;
    }
    if (stream) {
        ctx->stream = static_cast<cudaStream_t>(stream);
    } else {
        CNN_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
        ctx->own_stream = true;
    }
    return CNN_OK;
}

CNN_API const char *cnn_last_error(const cnn_context *ctx) {
    if (!ctx) return "null context";
    return ctx->last_error.c_str();
}

CNN_API cnn_status cnn_set_timing(cnn_context *ctx, int enabled) {
    if (!ctx) return CNN_ERR_INVALID_ARG;
    ctx->timing = enabled != 0;
    for (int i = 0; i < cnn_context::kSlots; ++i) ctx->slot_pending[i] = false;
    return CNN_OK;
}

CNN_API cnn_status cnn_set_wait_limit(cnn_context *ctx, int64_t limit_ns) {
    if (!ctx) return CNN_ERR_INVALID_ARG;
    ctx->wait_limit_ns = limit_ns > 0 ? limit_ns : 0;
    return CNN_OK;
}

CNN_API cnn_status cnn_set_intersection(cnn_context *ctx, cnn_intersection intersection) {
    if (!ctx) return CNN_ERR_INVALID_ARG;
    if (intersection < CNN_INTERSECT_AUTO || intersection > CNN_INTERSECT_BITSET)
        return ctx->fail(CNN_ERR_INVALID_ARG, "bad intersection strategy");
    ctx->intersect_pref = intersection;
    return CNN_OK;
}

CNN_API cnn_status cnn_set_search(cnn_context *ctx, cnn_search search) {
    if (!ctx) return CNN_ERR_INVALID_ARG;
    if (search < CNN_SEARCH_AUTO || search > CNN_SEARCH_TENSOR) return ctx->fail(CNN_ERR_INVALID_ARG, "bad search");
    ctx->search_pref = search;
    return CNN_OK;
}

CNN_API cnn_status cnn_get_stats(const cnn_context *cctx, cnn_stats *out) {
    cnn_context *ctx = const_cast<cnn_context *>(cctx);
    if (!ctx || !out) return CNN_ERR_INVALID_ARG;
    CNN_TRY(check_ctx(ctx));
    CNN_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (int i = 0; i < cnn_context::kSlots; ++i) {
        float *field = stage_field(ctx, i);
        if (!ctx->slot_pending[i] || !field) continue;
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, ctx->ev_begin[i], ctx->ev_end[i]) == cudaSuccess) *field = ms;
        (void)cudaGetLastError();
    }
    CNN_TRY(resolve_nnz(ctx));  // the stream is idle: no wait
    if (ctx->search_stats_pending) {
        ctx->stats.n_exact = (int64_t)ctx->host_stats[0];
        ctx->stats.n_candidates = ctx->pending_candidates >= 0 ? ctx->pending_candidates : (int64_t)ctx->host_stats[1];
        ctx->search_stats_pending = false;
    }
    if (ctx->fit_stats_pending) {
        ctx->stats.n_nodes = (int64_t)ctx->host_stats[4];
        ctx->stats.n_checks = (int64_t)ctx->host_stats[5];
        ctx->stats.n_accepted = (int64_t)ctx->host_stats[6];
        ctx->stats.n_clusters = (int64_t)ctx->host_stats[8];
        ctx->fit_stats_pending = false;
    }
    ctx->stats.n_launches = ctx->n_launches;
    *out = ctx->stats;
    return CNN_OK;
}

CNN_API cnn_status cnn_set_points(cnn_context *ctx, const void *points, cnn_dtype dtype, int64_t n_points,
                                  int32_t n_dim, cnn_memspace mem) {
    CNN_TRY(check_ctx(ctx));
    if (n_points < 0 || n_points > INT32_MAX - 1 || n_dim < 1 || (n_points > 0 && !points))
        return ctx->fail(CNN_ERR_INVALID_ARG, "n_points must be in [0, 2^31-2], n_dim >= 1");
    if (dtype != CNN_DTYPE_F64 && dtype != CNN_DTYPE_F32) return ctx->fail(CNN_ERR_INVALID_ARG, "bad dtype");
    if (mem != CNN_MEM_HOST && mem != CNN_MEM_DEVICE) return ctx->fail(CNN_ERR_INVALID_ARG, "bad memspace");
    ctx->have_graph = false;
    ++ctx->graph_generation;
    ctx->dist = nullptr;
    ctx->dist_set = false;
    ctx->n = n_points;
    ctx->d = n_dim;
    const int64_t total = n_points * n_dim;
    if (dtype == CNN_DTYPE_F64) {
        if (mem == CNN_MEM_DEVICE) {
            ctx->x = static_cast<const double *>(points);
        } else {
            CNN_TRY(ctx->ensure(ctx->x_own, sizeof(double) * (size_t)(total > 0 ? total : 1)));
            if (total > 0)
                CNN_CUDA(ctx, cudaMemcpyAsync(ctx->x_own.ptr, points, sizeof(double) * (size_t)total,
                                              cudaMemcpyHostToDevice, ctx->stream));
            ctx->x = ctx->x_own.as<double>();
        }
    } else {
        const float *src = static_cast<const float *>(points);
        if (mem == CNN_MEM_HOST) {
            CNN_TRY(ctx->ensure(ctx->x_f32_stage, sizeof(float) * (size_t)(total > 0 ? total : 1)));
            if (total > 0)
                CNN_CUDA(ctx, cudaMemcpyAsync(ctx->x_f32_stage.ptr, points, sizeof(float) * (size_t)total,
                                              cudaMemcpyHostToDevice, ctx->stream));
            src = ctx->x_f32_stage.as<float>();
        }
        CNN_TRY(ctx->ensure(ctx->x_own, sizeof(double) * (size_t)(total > 0 ? total : 1)));
        if (total > 0) {
            widen_f32_kernel<<<grid_for(total, 256) > 4096 ? 4096 : grid_for(total, 256), 256, 0, ctx->stream>>>(
                src, total, ctx->x_own.as<double>());
            CNN_LAUNCH_CHECK(ctx);
        }
        ctx->x = ctx->x_own.as<double>();
    }
    return CNN_OK;
}

CNN_API cnn_status cnn_set_distances(cnn_context *ctx, const double *distances, cnn_dist_layout layout,
                                     int64_t n_points, cnn_memspace mem) {
    CNN_TRY(check_ctx(ctx));
    if (n_points < 0 || n_points > INT32_MAX - 1) return ctx->fail(CNN_ERR_INVALID_ARG, "n_points out of range");
    if (layout != CNN_DIST_SQUARE && layout != CNN_DIST_LINEAR) return ctx->fail(CNN_ERR_INVALID_ARG, "bad layout");
    if (mem != CNN_MEM_HOST && mem != CNN_MEM_DEVICE) return ctx->fail(CNN_ERR_INVALID_ARG, "bad memspace");
    const int64_t count = layout == CNN_DIST_SQUARE ? n_points * n_points : n_points * (n_points - 1) / 2;
    if (count > 0 && !distances) return ctx->fail(CNN_ERR_INVALID_ARG, "distances missing");
    ctx->have_graph = false;
    ++ctx->graph_generation;
    ctx->x = nullptr;
    ctx->d = 0;
    ctx->n = n_points;
    ctx->dist_layout = layout;
    if (mem == CNN_MEM_DEVICE || count == 0) {
        ctx->dist = distances;
    } else {
        CNN_TRY(ctx->ensure(ctx->dist_own, sizeof(double) * (size_t)count));
        CNN_CUDA(ctx, cudaMemcpyAsync(ctx->dist_own.ptr, distances, sizeof(double) * (size_t)count,
                                      cudaMemcpyHostToDevice, ctx->stream));
        ctx->dist = ctx->dist_own.as<double>();
    }
    ctx->dist_set = true;
    CNN_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return CNN_OK;
}

CNN_API cnn_status cnn_set_periodic_bounds(cnn_context *ctx, const double *bounds, int32_t n_dim) {
    CNN_TRY(check_ctx(ctx));
    if (n_dim < 0 || (n_dim > 0 && !bounds)) return ctx->fail(CNN_ERR_INVALID_ARG, "bad bounds");
    ctx->periodic_bounds.assign(bounds, bounds + n_dim);
    return CNN_OK;
}

CNN_API cnn_status cnn_build_neighbours(cnn_context *ctx, double radius_cutoff, cnn_metric metric,
                                        cnn_fpmode fpmode) {
    CNN_TRY(check_ctx(ctx));
    if (!metric_known(metric)) return ctx->fail(CNN_ERR_INVALID_ARG, "unknown metric");
    if (fpmode != CNN_FP_SEPARATE && fpmode != CNN_FP_FUSED) return ctx->fail(CNN_ERR_INVALID_ARG, "unknown fpmode");
    CNN_TRY(check_source(ctx, metric));
    return build_neighbours_impl(ctx, radius_cutoff, metric, fpmode, kFormPref);
}

CNN_API cnn_status cnn_set_neighbours(cnn_context *ctx, const int64_t *offsets, const int32_t *indices,
                                      int64_t n_points, cnn_memspace mem) {
    CNN_TRY(check_ctx(ctx));
    if (n_points < 0 || n_points > INT32_MAX - 1 || !offsets)
        return ctx->fail(CNN_ERR_INVALID_ARG, "n_points must be in [0, 2^31-2] and offsets given");
    int64_t nnz = 0;
    if (mem == CNN_MEM_HOST) {
        nnz = offsets[n_points];
        if (offsets[0] != 0 || nnz < 0) return ctx->fail(CNN_ERR_INVALID_ARG, "offsets must start at 0");
        if (nnz > 0 && !indices) return ctx->fail(CNN_ERR_INVALID_ARG, "indices missing");
    }
    const int64_t *off_dev = nullptr;
    const int32_t *idx_dev = nullptr;
    CNN_TRY(stage_in<int64_t>(ctx, ctx->stage_offsets, offsets, n_points + 1, mem, &off_dev));
    CNN_TRY(stage_in<int32_t>(ctx, ctx->stage_indices, indices, nnz, mem, &idx_dev));
    return set_neighbours_impl(ctx, off_dev, idx_dev, n_points);
}

CNN_API cnn_status cnn_neighbour_count(cnn_context *ctx, int64_t *nnz) {
    CNN_TRY(check_ctx(ctx));
    if (!nnz) return ctx->fail(CNN_ERR_INVALID_ARG, "null output");
    if (!ctx->have_graph) return ctx->fail(CNN_ERR_STATE, "no neighbour graph");
    CNN_TRY(resolve_nnz(ctx));
    *nnz = ctx->nnz;
    return CNN_OK;
}

CNN_API cnn_status cnn_get_neighbours(cnn_context *ctx, int64_t *offsets, int32_t *indices, cnn_memspace mem) {
    CNN_TRY(check_ctx(ctx));
    if (!ctx->have_graph) return ctx->fail(CNN_ERR_STATE, "no neighbour graph");
    CNN_TRY(ensure_csr(ctx));
    if (!offsets || (ctx->nnz > 0 && !indices)) return ctx->fail(CNN_ERR_INVALID_ARG, "null output");
    const int64_t n = ctx->n, nnz = ctx->nnz;
    int64_t *off_dev = offsets;
    int32_t *idx_dev = indices;
    if (mem == CNN_MEM_HOST) {
        CNN_TRY(ctx->ensure(ctx->stage_offsets, sizeof(int64_t) * (size_t)(n + 1)));
        CNN_TRY(ctx->ensure(ctx->stage_indices, sizeof(int32_t) * (size_t)(nnz > 0 ? nnz : 1)));
        off_dev = ctx->stage_offsets.as<int64_t>();
        idx_dev = ctx->stage_indices.as<int32_t>();
    }
    CNN_TRY(export_neighbours_impl(ctx, off_dev, idx_dev));
    if (mem == CNN_MEM_HOST) {
        CNN_CUDA(ctx, cudaMemcpyAsync(offsets, off_dev, sizeof(int64_t) * (size_t)(n + 1), cudaMemcpyDeviceToHost,
                                      ctx->stream));
        if (nnz > 0)
            CNN_CUDA(ctx, cudaMemcpyAsync(indices, idx_dev, sizeof(int32_t) * (size_t)nnz, cudaMemcpyDeviceToHost,
                                          ctx->stream));
    }
    CNN_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return CNN_OK;
}

CNN_API cnn_status cnn_fit(cnn_context *ctx, int64_t similarity_cutoff, int64_t n_member_cutoff,
                           int64_t current_start, uint8_t *consider, int64_t *labels, int64_t n_points,
                           cnn_memspace mem) {
    CNN_TRY(check_ctx(ctx));
    if (!ctx->have_graph) return ctx->fail(CNN_ERR_STATE, "no neighbour graph: build or set neighbours first");
    const int64_t n = ctx->n;
    if (n_points != n)
        return ctx->fail(CNN_ERR_INVALID_ARG, "labels/consider hold " + std::to_string(n_points) +
                                                  " points, the neighbour graph " + std::to_string(n));
    if (mem != CNN_MEM_HOST && mem != CNN_MEM_DEVICE) return ctx->fail(CNN_ERR_INVALID_ARG, "bad memspace");
    if (n > 0 && (!consider || !labels)) return ctx->fail(CNN_ERR_INVALID_ARG, "consider and labels are required");
    uint8_t *cons_dev = consider;
    int64_t *lab_dev = labels;
    if (mem == CNN_MEM_HOST) {
        const uint8_t *c_in = nullptr;
        const int64_t *l_in = nullptr;
        CNN_TRY(stage_in<uint8_t>(ctx, ctx->stage_consider, consider, n, mem, &c_in));
        CNN_TRY(stage_in<int64_t>(ctx, ctx->stage_labels, labels, n, mem, &l_in));
        cons_dev = const_cast<uint8_t *>(c_in);
        lab_dev = const_cast<int64_t *>(l_in);
    }
    CNN_TRY(cnn::fit_dispatch(ctx, similarity_cutoff, n_member_cutoff, current_start, cons_dev, lab_dev));
    if (mem == CNN_MEM_HOST && n > 0) {
        CNN_CUDA(ctx, cudaMemcpyAsync(labels, lab_dev, sizeof(int64_t) * (size_t)n, cudaMemcpyDeviceToHost, ctx->stream));
        CNN_CUDA(ctx, cudaMemcpyAsync(consider, cons_dev, (size_t)n, cudaMemcpyDeviceToHost, ctx->stream));
        CNN_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    }
    return CNN_OK;
}

CNN_API cnn_status cnn_fit_fresh(cnn_context *ctx, int64_t similarity_cutoff, int64_t n_member_cutoff, int32_t sort,
                                 int64_t member_cutoff, int64_t max_clusters, int64_t *labels, uint8_t *consider,
                                 int64_t n_points, cnn_memspace mem) {
    CNN_TRY(check_ctx(ctx));
    if (!ctx->have_graph) return ctx->fail(CNN_ERR_STATE, "no neighbour graph: build or set neighbours first");
    const int64_t n = ctx->n;
    if (n_points != n)
        return ctx->fail(CNN_ERR_INVALID_ARG, "labels hold " + std::to_string(n_points) +
                                                  " points, the neighbour graph " + std::to_string(n));
    if (mem != CNN_MEM_HOST && mem != CNN_MEM_DEVICE) return ctx->fail(CNN_ERR_INVALID_ARG, "bad memspace");
    if (n > 0 && !labels) return ctx->fail(CNN_ERR_INVALID_ARG, "labels are required");
    if (n > INT32_MAX) return ctx->fail(CNN_ERR_UNSUPPORTED, "more than 2^31-1 labels");
    if (n == 0) return CNN_OK;
    cudaStream_t st = ctx->stream;
    // fresh labels and consider flags are made on the device: nothing is copied in
    int64_t *lab_dev = labels;
    if (mem == CNN_MEM_HOST) {
        CNN_TRY(ctx->ensure(ctx->stage_labels, sizeof(int64_t) * (size_t)n));
        lab_dev = ctx->stage_labels.as<int64_t>();
    }
    uint8_t *cons_dev = consider;
    if (mem == CNN_MEM_HOST || !consider) {
        CNN_TRY(ctx->ensure(ctx->stage_consider, (size_t)n));
        cons_dev = ctx->stage_consider.as<uint8_t>();
    }
    CNN_CUDA(ctx, cudaMemsetAsync(lab_dev, 0, sizeof(int64_t) * (size_t)n, st));
    CNN_CUDA(ctx, cudaMemsetAsync(cons_dev, 1, (size_t)n, st));
    CNN_TRY(cnn::fit_dispatch(ctx, similarity_cutoff, n_member_cutoff, 1, cons_dev, lab_dev));
    if (sort) CNN_TRY(cnn::sort_fresh_impl(ctx, lab_dev, n, member_cutoff, max_clusters, ctx->capturing));
    if (mem == CNN_MEM_HOST) {
        CNN_CUDA(ctx, cudaMemcpyAsync(labels, lab_dev, sizeof(int64_t) * (size_t)n, cudaMemcpyDeviceToHost, st));
        CNN_CUDA(ctx, cudaStreamSynchronize(st));
        if (consider) memset(consider, 0, (size_t)n);  // the fit visits every point
    }
    return CNN_OK;
}

CNN_API cnn_status cnn_graph_generation(const cnn_context *ctx, int64_t *generation) {
    if (!ctx || !generation) return CNN_ERR_INVALID_ARG;
    *generation = ctx->graph_generation;
    return CNN_OK;
}

CNN_API cnn_status cnn_sort_by_size(cnn_context *ctx, int64_t *labels, int64_t n, int64_t member_cutoff,
                                    int64_t max_clusters, cnn_memspace mem) {
    CNN_TRY(check_ctx(ctx));
    if (n < 0 || (n > 0 && !labels)) return ctx->fail(CNN_ERR_INVALID_ARG, "bad labels");
    int64_t *lab_dev = labels;
    if (mem == CNN_MEM_HOST) {
        const int64_t *l_in = nullptr;
        CNN_TRY(stage_in<int64_t>(ctx, ctx->stage_labels, labels, n, mem, &l_in));
        lab_dev = const_cast<int64_t *>(l_in);
    }
    CNN_TRY(sort_by_size_impl(ctx, lab_dev, n, member_cutoff, max_clusters));
    if (mem == CNN_MEM_HOST && n > 0) {
        CNN_CUDA(ctx, cudaMemcpyAsync(labels, lab_dev, sizeof(int64_t) * (size_t)n, cudaMemcpyDeviceToHost, ctx->stream));
        CNN_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    }
    return CNN_OK;
}

CNN_API cnn_status cnn_sweep(cnn_context *ctx, const double *radius_cutoffs, int32_t n_radii,
                             const int64_t *similarity_cutoffs, const int64_t *n_member_cutoffs, int32_t n_cuts,
                             cnn_metric metric, cnn_fpmode fpmode, int64_t member_cutoff, int64_t max_clusters,
                             int64_t *labels_out, cnn_memspace mem) {
    CNN_TRY(check_ctx(ctx));
    if (n_radii < 1 || n_radii > 16 || n_cuts < 1 || !radius_cutoffs || !similarity_cutoffs || !n_member_cutoffs ||
        !labels_out)
        return ctx->fail(CNN_ERR_INVALID_ARG, "need 1..16 radii, >= 1 cut and all arrays");
    if (!metric_known(metric)) return ctx->fail(CNN_ERR_INVALID_ARG, "unknown metric");
    CNN_TRY(check_source(ctx, metric));
    if (fpmode != CNN_FP_SEPARATE && fpmode != CNN_FP_FUSED) return ctx->fail(CNN_ERR_INVALID_ARG, "unknown fpmode");
    const int64_t total = (int64_t)n_radii * n_cuts * ctx->n;
    int64_t *lab_dev = labels_out;
    if (mem == CNN_MEM_HOST) {
        CNN_TRY(ctx->ensure(ctx->stage_labels, sizeof(int64_t) * (size_t)(total > 0 ? total : 1)));
        lab_dev = ctx->stage_labels.as<int64_t>();
    }
    CNN_TRY(sweep_impl(ctx, radius_cutoffs, n_radii, similarity_cutoffs, n_member_cutoffs, n_cuts, metric, fpmode,
                       member_cutoff, max_clusters, lab_dev));
    if (mem == CNN_MEM_HOST && total > 0)
        CNN_CUDA(ctx, cudaMemcpyAsync(labels_out, lab_dev, sizeof(int64_t) * (size_t)total, cudaMemcpyDeviceToHost,
                                      ctx->stream));
    CNN_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return CNN_OK;
}

CNN_API cnn_status cnn_sweep_pairs(cnn_context *ctx, const double *radius_cutoffs,
                                   const int64_t *similarity_cutoffs, const int64_t *n_member_cutoffs,
                                   int32_t n_steps, cnn_metric metric, cnn_fpmode fpmode, int32_t sort,
                                   int64_t member_cutoff, int64_t max_clusters, int64_t *labels_out,
                                   cnn_memspace mem) {
    CNN_TRY(check_ctx(ctx));
    if (n_steps < 1 || !radius_cutoffs || !similarity_cutoffs || !n_member_cutoffs || !labels_out)
        return ctx->fail(CNN_ERR_INVALID_ARG, "need >= 1 step and all arrays");
    if (!metric_known(metric)) return ctx->fail(CNN_ERR_INVALID_ARG, "unknown metric");
    CNN_TRY(check_source(ctx, metric));
    if (fpmode != CNN_FP_SEPARATE && fpmode != CNN_FP_FUSED) return ctx->fail(CNN_ERR_INVALID_ARG, "unknown fpmode");
    for (int32_t i = 0; i < n_steps; ++i)
        if (std::isnan(radius_cutoffs[i])) return ctx->fail(CNN_ERR_INVALID_ARG, "NaN radius cutoff");
    const int64_t n = ctx->n;
    const int64_t total = (int64_t)n_steps * n;
    int64_t *lab_dev = labels_out;
    if (mem == CNN_MEM_HOST) {
        CNN_TRY(ctx->ensure(ctx->stage_labels, sizeof(int64_t) * (size_t)(total > 0 ? total : 1)));
        lab_dev = ctx->stage_labels.as<int64_t>();
    }
    // distinct radii (ascending) and distinct cuts; the first step of every
    // distinct (radius, cut) pair is fitted, repeats are copied
    std::vector<double> radii(radius_cutoffs, radius_cutoffs + n_steps);
    std::sort(radii.begin(), radii.end());
    radii.erase(std::unique(radii.begin(), radii.end()), radii.end());
    std::vector<std::pair<int64_t, int64_t>> cuts;
    for (int32_t i = 0; i < n_steps; ++i) cuts.emplace_back(similarity_cutoffs[i], n_member_cutoffs[i]);
    std::sort(cuts.begin(), cuts.end());
    cuts.erase(std::unique(cuts.begin(), cuts.end()), cuts.end());
    const int32_t nr = (int32_t)radii.size(), nc = (int32_t)cuts.size();
    std::vector<int32_t> first(static_cast<size_t>(nr) * nc, -1);
    std::vector<int32_t> step_pair(n_steps);
    for (int32_t i = 0; i < n_steps; ++i) {
        const int32_t k = (int32_t)(std::lower_bound(radii.begin(), radii.end(), radius_cutoffs[i]) - radii.begin());
        const int32_t j = (int32_t)(std::lower_bound(cuts.begin(), cuts.end(),
                                                     std::make_pair(similarity_cutoffs[i], n_member_cutoffs[i])) -
                                    cuts.begin());
        step_pair[i] = k * nc + j;
        if (first[step_pair[i]] < 0) first[step_pair[i]] = i;
    }
    std::vector<int64_t> sim(nc), mem_cut(nc);
    for (int32_t j = 0; j < nc; ++j) {
        sim[j] = cuts[j].first;
        mem_cut[j] = cuts[j].second;
    }
    // at most 16 radii share one largest-radius search
    for (int32_t k0 = 0; k0 < nr; k0 += 16) {
        const int32_t kn = std::min<int32_t>(16, nr - k0);
        CNN_TRY(sweep_impl(ctx, radii.data() + k0, kn, sim.data(), mem_cut.data(), nc, metric, fpmode, member_cutoff,
                           max_clusters, lab_dev, first.data() + (size_t)k0 * nc, sort != 0));
    }
    for (int32_t i = 0; i < n_steps; ++i)
        if (first[step_pair[i]] != i && n > 0)
            CNN_CUDA(ctx, cudaMemcpyAsync(lab_dev + (int64_t)i * n, lab_dev + (int64_t)first[step_pair[i]] * n,
                                          sizeof(int64_t) * (size_t)n, cudaMemcpyDeviceToDevice, ctx->stream));
    if (mem == CNN_MEM_HOST && total > 0)
        CNN_CUDA(ctx, cudaMemcpyAsync(labels_out, lab_dev, sizeof(int64_t) * (size_t)total, cudaMemcpyDeviceToHost,
                                      ctx->stream));
    CNN_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return CNN_OK;
}

CNN_API cnn_status cnn_predict(cnn_context *ctx, const void *other_points, cnn_dtype dtype, int64_t n_other,
                               int32_t n_dim, const int64_t *labels, const int64_t *clusters, int64_t n_clusters,
                               double radius_cutoff, cnn_metric metric, cnn_fpmode fpmode, int64_t similarity_cutoff,
                               int64_t n_member_cutoff, int64_t *other_labels, uint8_t *other_consider,
                               cnn_memspace mem) {
    CNN_TRY(check_ctx(ctx));
    if (ctx->d < 1 || !ctx->x) return ctx->fail(CNN_ERR_STATE, "no points: call cnn_set_points first");
    if (n_dim != ctx->d) return ctx->fail(CNN_ERR_INVALID_ARG, "other points must have the same n_dim");
    if (n_other < 0 || n_other > INT32_MAX - 2 || n_clusters < 0) return ctx->fail(CNN_ERR_INVALID_ARG, "bad sizes");
    if (n_other > 0 && (!other_points || !other_labels || !other_consider))
        return ctx->fail(CNN_ERR_INVALID_ARG, "other points, labels and consider are required");
    if (ctx->n > 0 && !labels) return ctx->fail(CNN_ERR_INVALID_ARG, "labels of the clustered points are required");
    if (n_clusters > 0 && !clusters) return ctx->fail(CNN_ERR_INVALID_ARG, "clusters missing");
    if (dtype != CNN_DTYPE_F64 && dtype != CNN_DTYPE_F32) return ctx->fail(CNN_ERR_INVALID_ARG, "bad dtype");
    if (metric == CNN_METRIC_PRECOMPUTED)
        return ctx->fail(CNN_ERR_UNSUPPORTED, "prediction needs coordinates, not precomputed distances");
    if (!metric_known(metric)) return ctx->fail(CNN_ERR_INVALID_ARG, "unknown metric");
    if (fpmode != CNN_FP_SEPARATE && fpmode != CNN_FP_FUSED) return ctx->fail(CNN_ERR_INVALID_ARG, "unknown fpmode");
    if (mem != CNN_MEM_HOST && mem != CNN_MEM_DEVICE) return ctx->fail(CNN_ERR_INVALID_ARG, "bad memspace");
    cudaStream_t st = ctx->stream;
    const int64_t n = ctx->n, m = n_other, total = m * n_dim;
    // other points as float64 on the device
    const double *xq = nullptr;
    if (dtype == CNN_DTYPE_F64 && mem == CNN_MEM_DEVICE) {
        xq = static_cast<const double *>(other_points);
    } else {
        CNN_TRY(ctx->ensure(ctx->pred_x, sizeof(double) * (size_t)(total > 0 ? total : 1)));
        if (dtype == CNN_DTYPE_F64) {
            if (total > 0)
                CNN_CUDA(ctx, cudaMemcpyAsync(ctx->pred_x.ptr, other_points, sizeof(double) * (size_t)total,
                                              cudaMemcpyHostToDevice, st));
        } else {
            const float *src = static_cast<const float *>(other_points);
            if (mem == CNN_MEM_HOST) {
                CNN_TRY(ctx->ensure(ctx->stage_indices, sizeof(float) * (size_t)(total > 0 ? total : 1)));
                if (total > 0)
                    CNN_CUDA(ctx, cudaMemcpyAsync(ctx->stage_indices.ptr, other_points, sizeof(float) * (size_t)total,
                                                  cudaMemcpyHostToDevice, st));
                src = ctx->stage_indices.as<float>();
            }
            if (total > 0) {
                widen_f32_kernel<<<grid_for(total, 256) > 4096 ? 4096 : grid_for(total, 256), 256, 0, st>>>(
                    src, total, ctx->pred_x.as<double>());
                CNN_LAUNCH_CHECK(ctx);
            }
        }
        xq = ctx->pred_x.as<double>();
    }
    // clustered labels, the consider set (sorted, distinct), the other labels and flags
    const int64_t *lab_dev = labels;
    if (mem == CNN_MEM_HOST) CNN_TRY(stage_in<int64_t>(ctx, ctx->stage_labels, labels, n, mem, &lab_dev));
    std::vector<int64_t> set(static_cast<size_t>(n_clusters));
    if (n_clusters > 0) {
        if (mem == CNN_MEM_HOST) {
            memcpy(set.data(), clusters, sizeof(int64_t) * (size_t)n_clusters);
        } else {
            CNN_CUDA(ctx, cudaMemcpyAsync(set.data(), clusters, sizeof(int64_t) * (size_t)n_clusters,
                                          cudaMemcpyDeviceToHost, st));
            CNN_CUDA(ctx, cudaStreamSynchronize(st));
        }
    }
    std::sort(set.begin(), set.end());
    set.erase(std::unique(set.begin(), set.end()), set.end());
    CNN_TRY(ctx->ensure(ctx->pred_set, sizeof(int64_t) * (set.size() + 1)));
    if (!set.empty())
        CNN_CUDA(ctx, cudaMemcpyAsync(ctx->pred_set.ptr, set.data(), sizeof(int64_t) * set.size(),
                                      cudaMemcpyHostToDevice, st));
    int64_t *olab = other_labels;
    uint8_t *ocons = other_consider;
    if (mem == CNN_MEM_HOST) {
        const int64_t *l_in = nullptr;
        const uint8_t *c_in = nullptr;
        CNN_TRY(stage_in<int64_t>(ctx, ctx->stage_offsets, other_labels, m, mem, &l_in));
        CNN_TRY(stage_in<uint8_t>(ctx, ctx->stage_consider, other_consider, m, mem, &c_in));
        olab = const_cast<int64_t *>(l_in);
        ocons = const_cast<uint8_t *>(c_in);
    }
    CNN_TRY(predict_impl(ctx, xq, m, lab_dev, ctx->pred_set.as<int64_t>(), (int64_t)set.size(), radius_cutoff,
                         metric, fpmode, similarity_cutoff, n_member_cutoff, olab, ocons));
    if (mem == CNN_MEM_HOST && m > 0) {
        CNN_CUDA(ctx, cudaMemcpyAsync(other_labels, olab, sizeof(int64_t) * (size_t)m, cudaMemcpyDeviceToHost, st));
        CNN_CUDA(ctx, cudaMemcpyAsync(other_consider, ocons, (size_t)m, cudaMemcpyDeviceToHost, st));
    }
    CNN_CUDA(ctx, cudaStreamSynchronize(st));
    return CNN_OK;
}

CNN_API cnn_status cnn_mst_prim(cnn_context *ctx, double radius_cutoff, cnn_metric metric, cnn_fpmode fpmode,
                                int64_t *edges_a, int64_t *edges_b, int64_t *weights, int64_t capacity,
                                int64_t *n_edges) {
    CNN_TRY(check_ctx(ctx));
    if (!n_edges) return ctx->fail(CNN_ERR_INVALID_ARG, "n_edges missing");
    if (!metric_known(metric)) return ctx->fail(CNN_ERR_INVALID_ARG, "unknown metric");
    if (fpmode != CNN_FP_SEPARATE && fpmode != CNN_FP_FUSED) return ctx->fail(CNN_ERR_INVALID_ARG, "unknown fpmode");
    CNN_TRY(check_source(ctx, metric));
    std::vector<int64_t> a, b, w;
    CNN_TRY(mst_prim_impl(ctx, radius_cutoff, metric, fpmode, &a, &b, &w));
    *n_edges = (int64_t)a.size();
    if ((int64_t)a.size() > capacity || (!a.empty() && (!edges_a || !edges_b || !weights)))
        return ctx->fail(CNN_ERR_INVALID_ARG, "edge arrays too small (n_points - 1 always suffice)");
    if (!a.empty()) {
        memcpy(edges_a, a.data(), sizeof(int64_t) * a.size());
        memcpy(edges_b, b.data(), sizeof(int64_t) * b.size());
        memcpy(weights, w.data(), sizeof(int64_t) * w.size());
    }
    return CNN_OK;
}

CNN_API cnn_status cnn_check_lists(cnn_context *ctx, const int32_t *a, int64_t na, const int32_t *b, int64_t nb,
                                   int64_t c, int32_t *result, cnn_memspace mem) {
    CNN_TRY(check_ctx(ctx));
    if (na < 0 || nb < 0 || !result || (na > 0 && !a) || (nb > 0 && !b))
        return ctx->fail(CNN_ERR_INVALID_ARG, "bad lists");
    const int32_t *a_dev = a, *b_dev = b;
    int32_t *r_dev = result;
    if (mem == CNN_MEM_HOST) {
        CNN_TRY(stage_in<int32_t>(ctx, ctx->stage_offsets, a, na, mem, &a_dev));
        CNN_TRY(stage_in<int32_t>(ctx, ctx->stage_indices, b, nb, mem, &b_dev));
        CNN_TRY(ctx->ensure(ctx->stage_misc, 64));
        r_dev = ctx->stage_misc.as<int32_t>();
    }
    CNN_TRY(check_lists_impl(ctx, a_dev, na, b_dev, nb, c, r_dev));
    if (mem == CNN_MEM_HOST)
        CNN_CUDA(ctx, cudaMemcpyAsync(result, r_dev, sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
    CNN_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return CNN_OK;
}

}  // extern "C"
