// tuner.cu -- the intersection strategy of cell-grid fits, chosen by
// measurement.
//
// Both strategies give the same labels; which is faster depends on the
// workload: sorted lists with an early-exit merge read little per check
// when rows are short and checks stop early, masks (one bit per stencil
// candidate) are cheaper to build and shrink the graph when rows are long.
// Under CNN_INTERSECT_AUTO the first fit of a workload profile builds the
// graph in both forms and fits it both ways (cnn_fit), timing search + fit
// of each with CUDA events; the faster is kept for the profile and later
// graphs of that profile are built in that form only.  The profile is the
// device (its multiprocessor count), the point count and the candidate
// pairs per point of the cell grid, each on a log2 scale.  The choices live
// for the process and are shared by its contexts.
#include <math.h>

#include <map>
#include <mutex>

#include "common.cuh"

namespace cnn {

namespace {
std::mutex g_tune_mu;
std::map<uint64_t, int> g_tune_choice;

uint64_t log2_bucket(double v) { return v < 1.0 ? 0 : (uint64_t)floor(log2(v) * 2.0); }  // half-octave steps
}  // namespace

uint64_t tuner_key(const cnn_context *ctx, int64_t n, int64_t candidates) {
    const double per_point = n > 0 ? (double)candidates / (double)n : 0.0;
    return ((uint64_t)ctx->sm_count << 40) | (log2_bucket((double)n) << 20) | log2_bucket(per_point);
}

bool tuner_lookup(uint64_t key, int *choice) {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    auto it = g_tune_choice.find(key);
    if (it == g_tune_choice.end()) return false;
    *choice = it->second;
    return true;
}

void tuner_store(uint64_t key, int choice) {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tune_choice[key] = choice;
}

}  // namespace cnn
