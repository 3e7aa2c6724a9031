// server.cu -- a served stream of clustering jobs with continuous batching,
// behind the C ABI (cnn_server_*, cnn_submit, cnn_poll, cnn_wait).
//
// One context per slot (own stream, grow-only workspace kept between jobs)
// and one host worker thread per slot.  A job is one Clustering.fit of a
// point set (src/cnnclustering/cluster.pyx:256-392 with fresh labels:
// make_parameters already applied by the caller, search, fit from
// current_start 1, sort_by_size), so its labels do not depend on what else
// runs.  Jobs start oldest first as slots free up; a job that does not fit
// the memory budget yet is passed by later jobs that do (backfill) until it
// has been passed kMaxPassed times, after which nothing passes it.
//
// Device memory is bounded for real, not by estimates: every running slot
// holds a reservation and its context may not grow past it (the limit is
// checked before cudaMalloc, cnn_context::ensure); an idle slot keeps its
// workspace and counts with what it holds.  Reservations plus idle holdings
// never exceed the budget -- idle workspaces are released when a waiting
// job needs the room -- so neither do the bytes the slots hold.
//
// A job's reservation is what its slot already holds plus its own need: an
// estimate scaled by what jobs of its kind (d <= 3, d < 16, d >= 16) were
// seen to need beyond their estimates.  A job that outgrows its reservation
// stops at the refused allocation and is queued again at the front with at
// least twice the need (and at least what was asked for); once that reaches
// the whole budget it runs alone, and fails with CNN_ERR_OOM only if the
// whole budget is too small.
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "common.cuh"

namespace {

constexpr int kMaxPassed = 64;

struct JobRec {
    cnn_job job{};
    cnn_job_state state = CNN_JOB_QUEUED;
    cnn_status result = CNN_OK;
    double t_submit = 0, t_start = 0, t_done = 0;
    int32_t slot = -1;
    int32_t attempts = 0;
    int32_t passed = 0;     // times a later job started before it
    bool whole = false;     // needs the whole budget: runs alone
    int64_t estimate = 0;   // the caller's hint or estimate_bytes
    int64_t floor = 0;      // need at least this (after outgrowing a reservation)
    int kind = 0;           // 0: d <= 3, 1: d < 16, 2: d >= 16
    int64_t reserved = 0;
    std::string error;
};

// Device bytes of one fit of n x d points (upper estimate at mean degree
// 300): points, the neighbour graph and its search buffers, fit arrays.
int64_t estimate_bytes(int64_t n, int32_t d) {
    const int64_t pts = n * d * 8 + n * d * 4;
    int64_t graph = (int64_t)((double)n * 300.0 * 4 * 1.25) + n * 48;
    const int64_t work = n * 64 + (16 << 20);
    if (d >= 16) {
        const int64_t dp = (d + 63) / 64 * 64;
        graph += n * dp * 4 + n * 256 * 8 + n * 64 * 12;
    } else if (d > 3) {
        graph += n * d * 4;
    } else {
        graph += n * 32 + std::min<int64_t>(64 * n, int64_t(1) << 26) * 12;
    }
    return pts + graph + work;
}

}  // namespace

struct cnn_server {
    int device = 0;
    int64_t budget = 0;
    std::vector<cnn_context *> ctx;
    std::vector<std::thread> workers;
    std::vector<int64_t> slot_job;       // job id running on the slot, -1: idle
    std::vector<int64_t> slot_reserved;  // reservation of the running job
    std::mutex mu;
    std::condition_variable cv_slot;  // workers: a job was assigned, or stop
    std::condition_variable cv_done;  // waiters: a job finished
    std::deque<int64_t> queue;
    std::unordered_map<int64_t, JobRec> jobs;
    int64_t next_id = 1;
    bool stopping = false;
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
    cnn_server_stats st{};
    double scale[3] = {1.0, 1.0, 1.0};  // need / estimate seen per kind of job

    double now() const {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }

    // bytes counted against the budget: reservations of running slots,
    // holdings of idle ones
    int64_t committed_locked() const {
        int64_t c = 0;
        for (size_t s = 0; s < ctx.size(); ++s) c += slot_job[s] >= 0 ? slot_reserved[s] : ctx[s]->mem_held.load();
        return c;
    }

    int64_t held_locked() const {
        int64_t h = 0;
        for (cnn_context *c : ctx) h += c->mem_held.load();
        return h;
    }

    // The job's own need: the estimate scaled by what its kind of job was
    // seen to need, at least its floor, at most the budget.
    int64_t need_of(const JobRec &j) const {
        if (j.whole) return budget;
        const double scaled = (double)j.estimate * scale[j.kind] * 1.1;
        const int64_t need = std::max<int64_t>(j.floor, scaled > 9e18 ? INT64_MAX : (int64_t)scaled);
        return std::min(need, budget);
    }

    // Starts every queued job that fits (oldest first, then backfill).  A
    // job fits when its reservation plus the running jobs' reservations is
    // within the budget; idle slots' workspaces are released (largest
    // first) as far as needed to make the room real.  The job goes to the
    // idle slot whose workspace it can reuse (the largest holding within its
    // reservation), else the one holding least, released first.
    void admit_locked() {
        while (!stopping && !queue.empty()) {
            int64_t running_reserved = 0;
            int running = 0;
            std::vector<int> idles;
            for (size_t s = 0; s < ctx.size(); ++s) {
                if (slot_job[s] >= 0) {
                    running_reserved += slot_reserved[s];
                    ++running;
                } else {
                    idles.push_back((int)s);
                }
            }
            if (idles.empty()) return;
            size_t qi = 0;
            int64_t need = 0;
            bool found = false;
            for (; qi < queue.size(); ++qi) {
                JobRec &j = jobs[queue[qi]];
                need = need_of(j);
                const bool ok = j.whole ? running == 0 : need + running_reserved <= budget;
                if (ok) {
                    found = true;
                    break;
                }
                if (j.whole || j.passed >= kMaxPassed) break;  // nothing passes it: it waits at the head
            }
            if (!found) return;
            // the slot: the one holding most whose holding still fits beside
            // the need (its workspace is reused), else the one holding least,
            // released first
            int slot = -1;
            int64_t idle_all = 0;
            for (int s : idles) idle_all += ctx[s]->mem_held;
            for (int s : idles) {
                const int64_t h = ctx[s]->mem_held;
                if (h + need + running_reserved <= budget && (slot < 0 || h > ctx[slot]->mem_held)) slot = s;
            }
            if (slot < 0) {
                for (int s : idles)
                    if (slot < 0 || ctx[s]->mem_held < ctx[slot]->mem_held) slot = s;
                cnn::release_workspace(ctx[slot]);
                ++st.released;
            }
            (void)idle_all;
            const int64_t reserve = ctx[slot]->mem_held + need;
            int64_t idle_held = 0;
            for (int s : idles)
                if (s != slot) idle_held += ctx[s]->mem_held;
            if (reserve + running_reserved + idle_held > budget) {
                std::sort(idles.begin(), idles.end(),
                          [&](int a, int b) { return ctx[a]->mem_held > ctx[b]->mem_held; });
                for (int s : idles) {
                    if (reserve + running_reserved + idle_held <= budget) break;
                    if (s == slot || ctx[s]->mem_held == 0) continue;
                    idle_held -= ctx[s]->mem_held;
                    cnn::release_workspace(ctx[s]);
                    ++st.released;
                }
            }
            for (size_t pj = 0; pj < qi; ++pj) ++jobs[queue[pj]].passed;
            const int64_t id = queue[qi];
            queue.erase(queue.begin() + (int64_t)qi);
            JobRec &j = jobs[id];
            j.state = CNN_JOB_RUNNING;
            j.slot = slot;
            j.reserved = reserve;
            j.t_start = now();
            ++j.attempts;
            slot_job[slot] = id;
            slot_reserved[slot] = reserve;
            st.max_running = std::max<int32_t>(st.max_running, running + 1);
            cv_slot.notify_all();
        }
    }

    void run_slot(int s) {
        cnn_context *c = ctx[s];
        for (;;) {
            int64_t id;
            cnn_job job;
            int64_t reserve;
            {
                std::unique_lock<std::mutex> lk(mu);
                cv_slot.wait(lk, [&] { return stopping || slot_job[s] >= 0; });
                if (slot_job[s] < 0) return;  // stopping and idle
                id = slot_job[s];
                job = jobs[id].job;
                reserve = slot_reserved[s];
            }
            cnn_status r = CNN_OK;
            const int64_t held0 = c->mem_held.load();
            c->mem_cap = reserve;  // the slot's holding plus the job's need (admit_locked)
            c->cap_hit = false;
            const int64_t n = job.n_points;
            if (r == CNN_OK) r = cnn_set_points(c, job.points, job.dtype, n, job.n_dim, CNN_MEM_HOST);
            if (r == CNN_OK) r = cnn_build_neighbours(c, job.radius_cutoff, job.metric, job.fpmode);
            // fresh labels, the fit and sort_by_size in one call: only the labels come back
            if (r == CNN_OK)
                r = cnn_fit_fresh(c, job.similarity_cutoff, job.n_member_cutoff, job.member_cutoff >= 0 ? 1 : 0,
                                  job.member_cutoff, job.max_clusters, job.labels, nullptr, n, CNN_MEM_HOST);
            const bool outgrew = r == CNN_ERR_OOM && c->cap_hit;
            const std::string err = r == CNN_OK ? std::string() : std::string(cnn_last_error(c));
            // what the job added to the slot's holding (a lower bound of its
            // need when it was refused)
            const int64_t grew = (outgrew ? c->cap_need : c->mem_held.load()) - held0;
            if (outgrew) cnn::release_workspace(c);  // a partial graph is of no use to the next job
            c->mem_cap = 0;
            {
                std::lock_guard<std::mutex> lk(mu);
                JobRec &rec = jobs[id];
                slot_job[s] = -1;
                slot_reserved[s] = 0;
                st.peak_held_bytes = std::max(st.peak_held_bytes, held_locked());
                // learn how far estimates of this kind fall short (exact only
                // from an empty slot: a reused workspace hides part of the need)
                if (held0 == 0 && rec.estimate > 0 && grew > 0)
                    scale[rec.kind] = std::max(scale[rec.kind], (double)grew / (double)rec.estimate);
                if (outgrew && !rec.whole) {  // again, first in line, with a larger need
                    const int64_t prev = reserve - held0;
                    rec.floor = std::max<int64_t>(2 * prev, grew + grew / 4);
                    rec.whole = rec.floor >= budget;
                    rec.state = CNN_JOB_QUEUED;
                    rec.slot = -1;
                    ++st.requeued;
                    queue.push_front(id);
                } else {
                    rec.state = CNN_JOB_DONE;
                    rec.result = r;
                    rec.error = err;
                    rec.t_done = now();
                    ++st.done;
                    if (r != CNN_OK) ++st.failed;
                    cv_done.notify_all();
                }
                admit_locked();
            }
        }
    }
};

namespace {

void fill_info(const JobRec &j, cnn_job_info *info) {
    if (!info) return;
    info->state = j.state;
    info->result = j.result;
    info->slot = j.slot;
    info->attempts = j.attempts;
    info->reserved_bytes = j.reserved;
    info->t_submit = j.t_submit;
    info->t_start = j.t_start;
    info->t_done = j.t_done;
}

}  // namespace

extern "C" {

CNN_API cnn_status cnn_server_create(cnn_server **out, int device, int32_t n_slots, int64_t budget_bytes) {
    if (!out || n_slots < 1 || n_slots > 256 || budget_bytes <= 0) return CNN_ERR_INVALID_ARG;
    *out = nullptr;
    cnn_server *srv = new (std::nothrow) cnn_server();
    if (!srv) return CNN_ERR_OOM;
    srv->device = device;
    srv->budget = budget_bytes;
    srv->st.budget_bytes = budget_bytes;
    for (int s = 0; s < n_slots; ++s) {
        cnn_context *c = nullptr;
        const cnn_status r = cnn_create(&c, device, nullptr);
        if (r != CNN_OK) {
            for (cnn_context *o : srv->ctx) cnn_destroy(o);
            delete srv;
            return r;
        }
        srv->ctx.push_back(c);
    }
    srv->slot_job.assign((size_t)n_slots, -1);
    srv->slot_reserved.assign((size_t)n_slots, 0);
    for (int s = 0; s < n_slots; ++s) srv->workers.emplace_back([srv, s] {
        cudaSetDevice(srv->device);
        srv->run_slot(s);
    });
    *out = srv;
    return CNN_OK;
}

CNN_API cnn_status cnn_server_destroy(cnn_server *srv) {
    if (!srv) return CNN_OK;
    {
        std::unique_lock<std::mutex> lk(srv->mu);
        // the jobs already submitted run to the end
        srv->cv_done.wait(lk, [&] {
            if (!srv->queue.empty()) return false;
            for (int64_t j : srv->slot_job)
                if (j >= 0) return false;
            return true;
        });
        srv->stopping = true;
        srv->cv_slot.notify_all();
    }
    for (std::thread &t : srv->workers) t.join();
    for (cnn_context *c : srv->ctx) cnn_destroy(c);
    delete srv;
    return CNN_OK;
}

CNN_API cnn_status cnn_submit(cnn_server *srv, const cnn_job *job, int64_t *job_id) {
    if (!srv || !job || !job_id) return CNN_ERR_INVALID_ARG;
    if (job->n_points < 0 || job->n_points > INT32_MAX - 1 || job->n_dim < 1 ||
        (job->n_points > 0 && (!job->points || !job->labels)) ||
        (job->dtype != CNN_DTYPE_F64 && job->dtype != CNN_DTYPE_F32) ||
        (job->fpmode != CNN_FP_SEPARATE && job->fpmode != CNN_FP_FUSED) ||
        (job->metric != CNN_METRIC_EUCLIDEAN_REDUCED && job->metric != CNN_METRIC_EUCLIDEAN))
        return CNN_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(srv->mu);
    if (srv->stopping) return CNN_ERR_STATE;
    const int64_t id = srv->next_id++;
    JobRec &rec = srv->jobs[id];
    rec.job = *job;
    rec.t_submit = srv->now();
    rec.estimate = job->reserve_bytes > 0 ? job->reserve_bytes : estimate_bytes(job->n_points, job->n_dim);
    rec.kind = job->n_dim <= 3 ? 0 : job->n_dim < 16 ? 1 : 2;
    srv->queue.push_back(id);
    ++srv->st.submitted;
    srv->admit_locked();
    *job_id = id;
    return CNN_OK;
}

CNN_API cnn_status cnn_poll(cnn_server *srv, int64_t job_id, cnn_job_info *info) {
    if (!srv || !info) return CNN_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(srv->mu);
    auto it = srv->jobs.find(job_id);
    if (it == srv->jobs.end()) return CNN_ERR_INVALID_ARG;
    fill_info(it->second, info);
    return CNN_OK;
}

CNN_API cnn_status cnn_wait(cnn_server *srv, int64_t job_id, int64_t timeout_ns, cnn_job_info *info) {
    if (!srv) return CNN_ERR_INVALID_ARG;
    std::unique_lock<std::mutex> lk(srv->mu);
    if (srv->jobs.find(job_id) == srv->jobs.end()) return CNN_ERR_INVALID_ARG;
    // done, or released by another thread meanwhile (then the id is gone)
    auto done = [&] {
        auto it = srv->jobs.find(job_id);
        return it == srv->jobs.end() || it->second.state == CNN_JOB_DONE;
    };
    const bool finished = timeout_ns < 0 ? (srv->cv_done.wait(lk, done), true)
                                         : srv->cv_done.wait_for(lk, std::chrono::nanoseconds(timeout_ns), done);
    auto it = srv->jobs.find(job_id);
    if (it == srv->jobs.end()) return CNN_ERR_INVALID_ARG;
    fill_info(it->second, info);
    return finished ? CNN_OK : CNN_ERR_TIMEOUT;
}

CNN_API cnn_status cnn_job_error(cnn_server *srv, int64_t job_id, char *buf, int64_t size) {
    if (!srv || !buf || size < 1) return CNN_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(srv->mu);
    auto it = srv->jobs.find(job_id);
    if (it == srv->jobs.end()) return CNN_ERR_INVALID_ARG;
    const std::string &e = it->second.error;
    const size_t k = std::min<size_t>(e.size(), (size_t)size - 1);
    memcpy(buf, e.data(), k);
    buf[k] = '\0';
    return CNN_OK;
}

CNN_API cnn_status cnn_job_release(cnn_server *srv, int64_t job_id) {
    if (!srv) return CNN_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(srv->mu);
    auto it = srv->jobs.find(job_id);
    if (it == srv->jobs.end()) return CNN_ERR_INVALID_ARG;
    if (it->second.state != CNN_JOB_DONE) return CNN_ERR_STATE;
    srv->jobs.erase(it);
    srv->cv_done.notify_all();  // a waiter on this id returns
    return CNN_OK;
}

CNN_API cnn_status cnn_server_get_stats(cnn_server *srv, cnn_server_stats *out) {
    if (!srv || !out) return CNN_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(srv->mu);
    *out = srv->st;
    int32_t running = 0;
    for (int64_t j : srv->slot_job) running += j >= 0;
    out->running = running;
    out->queued = (int32_t)srv->queue.size();
    out->committed_bytes = srv->committed_locked();
    out->held_bytes = srv->held_locked();
    out->peak_held_bytes = std::max(out->peak_held_bytes, out->held_bytes);
    return CNN_OK;
}

}  // extern "C"
