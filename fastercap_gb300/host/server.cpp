// Extraction server: continuous admission of solve jobs onto one GPU.
//
// Jobs wait in arrival order. A free slot takes the head job as soon as the
// sum of admitted footprints plus the head's stays within the budget (or no
// job is running, so a job larger than the budget still runs, alone). Each
// slot is a host thread with its own CUDA stream; device memory is
// stream-ordered, so admitted jobs never synchronise one another and their
// kernels overlap on the GPU. A job owns its problem (links, coefficients,
// Krylov basis) from admission to result and shares nothing with other jobs,
// so its result is the same alone and in any mix.
#include <stdint.h>
#include <string.h>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/fastercap_gb300.h"
#include "handles.hpp"

namespace {

double now_ms() {
    using namespace std::chrono;
    return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

struct Job {
    int64_t id = 0;
    // file jobs: the slot builds the model from the input file first
    bool from_file = false;
    std::string path;
    fcg_build_options bopt;
    fcg_model *model = nullptr;  // built by the slot, freed with the job's problem
    double build_ms = 0;
    bool admitted = false;  // footprint counted in the server's in_use
    fcg_model_arrays a;
    int precision = FCG_PREC_MIXED;
    fcg_solve_options opt;
    int n_cond = 0;
    int state = FCG_JOB_QUEUED;
    int status = FCG_NORMAL_END;
    std::string error;
    std::vector<double> cap;
    std::vector<int> iters;
    int slot = -1;
    int64_t footprint = 0, device_bytes = 0;
    double t_submit = 0, t_start = 0, t_end = 0;
    double fill_ms = 0, solve_ms = 0;
    int iterations_max = 0;
    int64_t launches = 0;
    bool cancel = false;
    fcg::DeviceProblem *prob = nullptr;  // while running (guarded by the server mutex)
};

}  // namespace

struct fcg_server {
    fcg::DeviceContext *ctx = nullptr;
    int slots = 4;
    int64_t budget = 0, in_use = 0, peak_in_use = 0;
    int iterations_hint = 64;
    int running = 0, max_running = 0;
    int solving = 0;  // running jobs whose footprint is counted in in_use
    int64_t next_id = 1, submitted = 0, completed = 0;
    bool stop = false;
    std::mutex mu;
    std::condition_variable cv_admit, cv_done;
    std::deque<Job *> queue;
    std::unordered_map<int64_t, Job *> jobs;
    std::vector<std::thread> workers;
    std::vector<void *> streams;
};

// The head job takes a free slot once its footprint fits next to the
// footprints already admitted (or nothing holds memory). A file job's
// footprint is known only after its model is built: it takes the slot at
// once, builds, and then waits in run_job for the same memory rule.
static bool can_admit(const fcg_server *s) {
    if (s->queue.empty()) return false;
    const Job *j = s->queue.front();
    return j->from_file || s->solving == 0 || s->in_use + j->footprint <= s->budget;
}

static int count_conductors(const fcg_model_arrays &a) {
    int n = 0;
    for (int32_t c = 0; c < a.n_conductors; c++) n += (a.cond_is_diel && a.cond_is_diel[c]) ? 0 : 1;
    return n;
}

// build a file job's model on the server's GPU (mesh refinement and link
// construction on the device), then wait until its footprint may be admitted
static int build_file_job(fcg_server *s, Job *j) {
    double t0 = now_ms();
    char ebuf[512] = {0};
    int r = fcg::model_build_device_links(s->ctx, j->path.c_str(), &j->bopt, &j->model, ebuf, sizeof ebuf);
    j->build_ms = now_ms() - t0;
    if (r != FCG_NORMAL_END) {
        j->error = ebuf[0] ? std::string(ebuf) : fcg::get_error();
        return r;
    }
    fcg_model_arrays_get(j->model, &j->a);
    j->n_cond = count_conductors(j->a);
    j->footprint = fcg::problem_estimate_bytes(j->a, j->precision, j->n_cond, s->iterations_hint);
    std::unique_lock<std::mutex> lk(s->mu);
    s->cv_admit.wait(lk, [&] { return j->cancel || s->solving == 0 || s->in_use + j->footprint <= s->budget; });
    if (j->cancel) {
        j->footprint = 0;
        j->error = "job cancelled before its solve";
        return FCG_USER_BREAK;
    }
    s->in_use += j->footprint;
    s->peak_in_use = std::max(s->peak_in_use, s->in_use);
    s->solving++;
    j->admitted = true;
    return FCG_NORMAL_END;
}

static void run_job(fcg_server *s, Job *j, void *stream) {
    fcg::DeviceProblem *p = nullptr;
    int r = FCG_NORMAL_END;
    if (j->from_file) r = build_file_job(s, j);
    if (r == FCG_NORMAL_END) r = fcg::problem_create(*s->ctx, j->a, j->precision, stream, &p);
    // a job solves once: measuring launch shapes would not pay
    if (r == FCG_NORMAL_END) fcg::problem_set_tuning(p, false);
    if (r == FCG_NORMAL_END) {
        std::lock_guard<std::mutex> lk(s->mu);
        j->prob = p;
        if (j->cancel) fcg::problem_cancel(p);
    }
    if (r == FCG_NORMAL_END) r = fcg::problem_fill(p);
    if (r == FCG_NORMAL_END) {
        j->cap.assign((size_t)j->n_cond * j->n_cond, 0.0);
        j->iters.assign(j->n_cond, 0);
        r = fcg::problem_solve(p, j->opt, j->cap.data(), j->iters.data());
    }
    if (p) {
        fcg::SolveTimings t = fcg::problem_timings(p);
        j->fill_ms = t.fill_ms;
        j->solve_ms = t.solve_ms;
        j->iterations_max = t.iterations_max;
        j->launches = t.launches;
        j->device_bytes = fcg::problem_device_bytes(p);
        {
            std::lock_guard<std::mutex> lk(s->mu);
            j->prob = nullptr;
        }
        fcg::problem_destroy(p);
    }
    if (j->model) {
        fcg_model_free(j->model);
        j->model = nullptr;
    }
    j->status = r;
    if (r != FCG_NORMAL_END && j->error.empty()) j->error = fcg::get_error();
}

static void worker(fcg_server *s, int slot) {
    for (;;) {
        Job *j = nullptr;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv_admit.wait(lk, [&] { return s->stop || can_admit(s); });
            if (s->stop) return;
            j = s->queue.front();
            s->queue.pop_front();
            if (!j->from_file) {
                s->in_use += j->footprint;
                s->peak_in_use = std::max(s->peak_in_use, s->in_use);
                s->solving++;
                j->admitted = true;
            }
            s->running++;
            s->max_running = std::max(s->max_running, s->running);
            j->state = FCG_JOB_RUNNING;
            j->slot = slot;
            j->t_start = now_ms();
        }
        run_job(s, j, s->streams[slot]);
        {
            std::lock_guard<std::mutex> lk(s->mu);
            // a file job that failed or was cancelled while building holds no memory
            if (j->admitted) {
                s->in_use -= j->footprint;
                s->solving--;
            }
            s->running--;
            s->completed++;
            j->t_end = now_ms();
            j->state = FCG_JOB_DONE;
        }
        // memory freed: the head job may fit now
        s->cv_admit.notify_all();
        s->cv_done.notify_all();
    }
}

static void fill_info(const Job *j, fcg_job_info *info) {
    if (!info) return;
    memset(info, 0, sizeof(*info));
    info->state = j->state;
    info->status = j->status;
    info->n_cond = j->n_cond;
    info->iterations_max = j->iterations_max;
    info->slot = j->slot;
    info->footprint_bytes = j->footprint;
    info->device_bytes = j->device_bytes;
    double end = j->t_end > 0 ? j->t_end : now_ms();
    info->queue_ms = (j->t_start > 0 ? j->t_start : end) - j->t_submit;
    info->run_ms = j->t_start > 0 ? end - j->t_start : 0.0;
    info->fill_ms = j->fill_ms;
    info->solve_ms = j->solve_ms;
    info->kernel_launches = j->launches;
    info->build_ms = j->build_ms;
    info->n_panels = j->a.n_panels;
    info->n_links = j->a.n_links;
}

extern "C" {

int fcg_server_create(fcg_context *ctx, const fcg_server_config *cfg, fcg_server **out) {
    if (!ctx || !out) return FCG_GENERIC_ERROR;
    *out = nullptr;
    fcg_server *s = new fcg_server();
    s->ctx = ctx->dev;
    s->ctx->refs.fetch_add(1);
    s->slots = (cfg && cfg->slots > 0) ? cfg->slots : 4;
    s->budget = (cfg && cfg->memory_budget > 0) ? cfg->memory_budget : (int64_t)(0.8 * (double)s->ctx->free_bytes);
    s->iterations_hint = (cfg && cfg->iterations_hint > 0) ? cfg->iterations_hint : 64;
    for (int i = 0; i < s->slots; i++) {
        void *st = fcg::stream_create(s->ctx->device);
        if (!st) {
            for (void *q : s->streams) fcg::stream_destroy(s->ctx->device, q);
            fcg::context_unref(s->ctx);
            delete s;
            fcg::set_error("cannot create the server's streams");
            return FCG_DEVICE_ERROR;
        }
        s->streams.push_back(st);
    }
    for (int i = 0; i < s->slots; i++) s->workers.emplace_back(worker, s, i);
    *out = s;
    return FCG_NORMAL_END;
}

void fcg_server_destroy(fcg_server *s) {
    if (!s) return;
    {
        std::unique_lock<std::mutex> lk(s->mu);
        for (Job *j : s->queue) {
            j->state = FCG_JOB_CANCELLED;
            j->status = FCG_USER_BREAK;
        }
        s->queue.clear();
        // running jobs finish; then the workers leave
        s->cv_done.wait(lk, [&] { return s->running == 0; });
        s->stop = true;
    }
    s->cv_admit.notify_all();
    s->cv_done.notify_all();
    for (std::thread &t : s->workers) t.join();
    for (void *q : s->streams) fcg::stream_destroy(s->ctx->device, q);
    for (auto &kv : s->jobs) delete kv.second;
    fcg::context_unref(s->ctx);
    delete s;
}

static Job *new_job(int precision, const fcg_solve_options *opt) {
    if (precision != FCG_PREC_FP64 && precision != FCG_PREC_MIXED) {
        fcg::set_error("unknown precision");
        return nullptr;
    }
    Job *j = new Job();
    memset(&j->a, 0, sizeof j->a);
    j->precision = precision;
    j->opt.tol = 0.01;
    j->opt.precond = FCG_PRECOND_JACOBI;
    j->opt.max_iter = 0;
    j->opt.rhs_width = 0;
    j->opt.precond_dim = 0;
    j->opt.refine = 0;
    if (opt) j->opt = *opt;
    return j;
}

static int enqueue(fcg_server *s, Job *j, int64_t *job) {
    j->t_submit = now_ms();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->stop) {
            delete j;
            fcg::set_error("server is shutting down");
            return FCG_GENERIC_ERROR;
        }
        j->id = s->next_id++;
        s->jobs[j->id] = j;
        s->queue.push_back(j);
        s->submitted++;
        *job = j->id;
    }
    s->cv_admit.notify_one();
    return FCG_NORMAL_END;
}

int fcg_server_submit(fcg_server *s, const fcg_model_arrays *a, int precision, const fcg_solve_options *opt, int64_t *job) {
    if (!s || !a || !job) return FCG_GENERIC_ERROR;
    Job *j = new_job(precision, opt);
    if (!j) return FCG_GENERIC_ERROR;
    j->a = *a;
    j->n_cond = count_conductors(*a);
    j->footprint = fcg::problem_estimate_bytes(*a, precision, j->n_cond, s->iterations_hint);
    return enqueue(s, j, job);
}

int fcg_server_submit_file(fcg_server *s, const char *path, const fcg_build_options *bopt, int precision,
                           const fcg_solve_options *opt, int64_t *job) {
    if (!s || !path || !job) return FCG_GENERIC_ERROR;
    Job *j = new_job(precision, opt);
    if (!j) return FCG_GENERIC_ERROR;
    j->from_file = true;
    j->path = path;
    j->bopt.mesh_eps = 0.1;
    j->bopt.eps_ratio = 1.0;
    j->bopt.mesh_curv = 3.0;
    j->bopt.verbose = 0;
    if (bopt) j->bopt = *bopt;
    return enqueue(s, j, job);
}

int fcg_server_wait(fcg_server *s, int64_t job, fcg_job_info *info) {
    if (!s) return FCG_GENERIC_ERROR;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->jobs.find(job);
    if (it == s->jobs.end()) {
        fcg::set_error("unknown job");
        return FCG_GENERIC_ERROR;
    }
    Job *j = it->second;
    s->cv_done.wait(lk, [&] { return j->state == FCG_JOB_DONE || j->state == FCG_JOB_CANCELLED; });
    fill_info(j, info);
    return FCG_NORMAL_END;
}

int fcg_server_poll(fcg_server *s, int64_t job, fcg_job_info *info) {
    if (!s) return FCG_GENERIC_ERROR;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->jobs.find(job);
    if (it == s->jobs.end()) {
        fcg::set_error("unknown job");
        return FCG_GENERIC_ERROR;
    }
    fill_info(it->second, info);
    return FCG_NORMAL_END;
}

int fcg_server_result(fcg_server *s, int64_t job, double *cap, int *iterations, fcg_job_info *info) {
    if (!s) return FCG_GENERIC_ERROR;
    Job *j = nullptr;
    {
        std::unique_lock<std::mutex> lk(s->mu);
        auto it = s->jobs.find(job);
        if (it == s->jobs.end()) {
            fcg::set_error("unknown job");
            return FCG_GENERIC_ERROR;
        }
        j = it->second;
        s->cv_done.wait(lk, [&] { return j->state == FCG_JOB_DONE || j->state == FCG_JOB_CANCELLED; });
        s->jobs.erase(it);
    }
    fill_info(j, info);
    int status = j->status;
    if (status == FCG_NORMAL_END || status == FCG_NOT_CONVERGED) {
        if (cap && !j->cap.empty()) memcpy(cap, j->cap.data(), j->cap.size() * sizeof(double));
        if (iterations && !j->iters.empty()) memcpy(iterations, j->iters.data(), j->iters.size() * sizeof(int));
    } else if (!j->error.empty()) {
        fcg::set_error(j->error);
    }
    delete j;
    return status;
}

int fcg_server_cancel(fcg_server *s, int64_t job) {
    if (!s) return FCG_GENERIC_ERROR;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        auto it = s->jobs.find(job);
        if (it == s->jobs.end()) {
            fcg::set_error("unknown job");
            return FCG_GENERIC_ERROR;
        }
        Job *j = it->second;
        if (j->state == FCG_JOB_QUEUED) {
            for (auto q = s->queue.begin(); q != s->queue.end(); ++q)
                if (*q == j) {
                    s->queue.erase(q);
                    break;
                }
            j->state = FCG_JOB_CANCELLED;
            j->status = FCG_USER_BREAK;
            j->error = "job cancelled before it ran";
            j->t_end = now_ms();
        } else if (j->state == FCG_JOB_RUNNING) {
            j->cancel = true;
            if (j->prob) fcg::problem_cancel(j->prob);
        }
    }
    s->cv_done.notify_all();
    s->cv_admit.notify_all();
    return FCG_NORMAL_END;
}

int fcg_server_get_stats(fcg_server *s, fcg_server_stats *st) {
    if (!s || !st) return FCG_GENERIC_ERROR;
    std::lock_guard<std::mutex> lk(s->mu);
    st->slots = s->slots;
    st->running = s->running;
    st->queued = (int)s->queue.size();
    st->max_running = s->max_running;
    st->budget = s->budget;
    st->in_use = s->in_use;
    st->peak_in_use = s->peak_in_use;
    st->submitted = s->submitted;
    st->completed = s->completed;
    return FCG_NORMAL_END;
}

}  // extern "C"
