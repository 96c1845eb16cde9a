// iso_server.cu -- device-resident request loop with continuous batching.
//
// A fixed pool of workers, each owning an engine context (its own CUDA stream
// and device arena), takes ISM requests from a queue: first in, first out, or
// (ISO_SERVE_SHORTEST_FIRST) the smallest work estimate first, with a bound on
// how long the oldest request may be passed over; a request smaller than one
// already running then goes to a high-priority stream.  Requests run
// concurrently on the device as workers free up.  Device memory is admitted
// against a budget: a request first runs its surface count pass (volume plus
// small buffers), which fixes its exact need; the worker then waits until
//   sum over running workers of max(reserved, held) + sum over idle arenas
//   + this request's need <= budget,
// trimming idle workers' arenas to make room.  Waiting requests are admitted
// in submission order, and a request whose need alone exceeds the budget is
// refused with ISO_ERR_NOMEM, so the loop cannot deadlock.  Results do not
// depend on what else runs: each request's kernels read only its own buffers.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <string>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "iso_internal.cuh"

namespace {

using Clock = std::chrono::steady_clock;

struct Job {
    iso_request req;
    double cost = 0;  // work estimate: samples x isovalues x (isovalues + 64)
    int64_t ticket = 0;
    int status = ISO_OK;
    std::string error;
    int32_t m = 0;
    iso_timing timing{};
    Clock::time_point t_submit, t_start, t_admit, t_end;
    bool done = false;
};

enum class WState { Idle, Counting, Waiting, Running };

struct Worker {
    iso_ctx *ctx = nullptr;
    cudaStream_t normal = nullptr;  // the context's own stream
    cudaStream_t urgent = nullptr;  // a high-priority stream for requests smaller than a running one
    double cost = 0;                // estimate of the running request (0: none)
    std::thread thread;
    WState state = WState::Idle;
    size_t held = 0;      // arena bytes physically allocated
    size_t reserved = 0;  // admitted need of the running request
    int64_t ticket = -1;
};

}  // namespace

struct iso_server {
    int device = 0;
    size_t budget = 0;
    int policy = ISO_SERVE_FIFO;
    double max_wait_ms = 0;
    std::vector<Worker> workers;
    std::mutex mu;
    std::condition_variable cv_queue, cv_mem, cv_done;
    std::deque<Job *> queue;
    std::unordered_map<int64_t, Job *> jobs;
    int64_t next_ticket = 1;
    bool stop = false;
    std::vector<double> latencies_ms;
    int64_t completed = 0, failed = 0;
    size_t peak_bytes = 0;

    size_t others_bytes(size_t self) const
    {
        size_t total = 0;
        for (size_t w = 0; w < workers.size(); ++w) {
            if (w == self) continue;
            const Worker &k = workers[w];
            total += k.state == WState::Running ? std::max(k.reserved, k.held) : k.held;
        }
        return total;
    }
    // the earliest waiting ticket goes first
    bool earliest_waiter(size_t self) const
    {
        for (size_t w = 0; w < workers.size(); ++w)
            if (w != self && workers[w].state == WState::Waiting && workers[w].ticket < workers[self].ticket) return false;
        return true;
    }
};

namespace {

struct AdmitCtx {
    iso_server *s;
    size_t self;
};

int admit_cb(void *user, size_t need)
{
    AdmitCtx *a = static_cast<AdmitCtx *>(user);
    iso_server *s = a->s;
    std::unique_lock<std::mutex> lock(s->mu);
    Worker &me = s->workers[a->self];
    if (need > s->budget) return 1;
    me.state = WState::Waiting;
    s->cv_mem.notify_all();  // the earliest waiter may have been waiting on this worker
    for (;;) {
        if (s->earliest_waiter(a->self)) {
            auto fits = [&] { return s->others_bytes(a->self) + std::max(need, me.held) <= s->budget; };
            if (!fits()) {
                // free memory lazily, cheapest first: idle arenas, then the
                // arenas of requests waiting behind this one (blocked here, so
                // their streams are idle; their staged surface buffers stay),
                // then this request's own leftovers from earlier requests
                for (size_t w = 0; w < s->workers.size() && !fits(); ++w) {
                    Worker &k = s->workers[w];
                    if (w != a->self && k.state == WState::Idle && k.held > 0) {
                        iso_ctx_release(k.ctx);
                        k.held = 0;
                    }
                }
                for (size_t w = 0; w < s->workers.size() && !fits(); ++w) {
                    Worker &k = s->workers[w];
                    if (w != a->self && k.state == WState::Waiting && k.held > 0) {
                        iso_ctx_release_except_surfaces(k.ctx);
                        k.held = iso_ctx_device_bytes(k.ctx);
                    }
                }
                if (!fits()) {
                    iso_ctx_release_except_surfaces(me.ctx);
                    me.held = iso_ctx_device_bytes(me.ctx);
                }
            }
            if (fits()) break;
            // nothing left that will free memory: refuse instead of waiting
            bool pending = false;
            for (size_t w = 0; w < s->workers.size(); ++w)
                if (w != a->self && (s->workers[w].state == WState::Running || s->workers[w].state == WState::Counting))
                    pending = true;
            if (!pending) {
                me.state = WState::Counting;
                return 1;
            }
        }
        s->cv_mem.wait(lock);
    }
    me.state = WState::Running;
    me.reserved = need;
    const size_t total = s->others_bytes(a->self) + std::max(need, me.held);
    s->peak_bytes = std::max(s->peak_bytes, total);
    return 0;
}

void worker_loop(iso_server *s, size_t self)
{
    Worker &me = s->workers[self];
    cudaSetDevice(s->device);
    AdmitCtx actx{s, self};
    for (;;) {
        Job *job = nullptr;
        {
            std::unique_lock<std::mutex> lock(s->mu);
            s->cv_queue.wait(lock, [&] { return s->stop || !s->queue.empty(); });
            if (s->stop && s->queue.empty()) return;
            // FIFO, or the smallest estimate first unless the oldest request
            // has waited longer than max_wait_ms
            auto pick = s->queue.begin();
            if (s->policy == ISO_SERVE_SHORTEST_FIRST) {
                const double waited =
                    std::chrono::duration<double, std::milli>(Clock::now() - (*pick)->t_submit).count();
                if (waited <= s->max_wait_ms)
                    for (auto it = s->queue.begin(); it != s->queue.end(); ++it)
                        if ((*it)->cost < (*pick)->cost) pick = it;
            }
            job = *pick;
            s->queue.erase(pick);
            // a request smaller than one already on the device runs on the
            // high-priority stream, so that its blocks are scheduled first
            bool urgent = false;
            if (s->policy == ISO_SERVE_SHORTEST_FIRST)
                for (size_t w = 0; w < s->workers.size(); ++w)
                    if (w != self && s->workers[w].cost > job->cost) urgent = true;
            me.ctx->stream = urgent && me.urgent ? me.urgent : me.normal;
            me.cost = job->cost;
            me.state = WState::Counting;
            me.ticket = job->ticket;
            job->t_start = Clock::now();
        }
        me.ctx->admit = admit_cb;
        me.ctx->admit_user = &actx;
        const iso_request &r = job->req;
        int rc = iso_ism(me.ctx, r.volume, r.X, r.Y, r.Z, r.isovalues, r.n, &r.opts, r.ism_out, r.field_ids_out,
                         &job->m, nullptr, &job->timing);
        std::string err = rc == ISO_OK ? "" : iso_last_error();
        me.ctx->admit = nullptr;
        {
            std::lock_guard<std::mutex> lock(s->mu);
            job->status = rc;
            job->error = err;
            job->t_end = Clock::now();
            job->done = true;
            if (r.m_out) *r.m_out = job->m;
            me.held = iso_ctx_device_bytes(me.ctx);
            me.reserved = 0;
            me.cost = 0;
            me.ctx->stream = me.normal;
            me.state = WState::Idle;
            me.ticket = -1;
            if (rc == ISO_OK) {
                ++s->completed;
                s->latencies_ms.push_back(std::chrono::duration<double, std::milli>(job->t_end - job->t_submit).count());
            } else {
                ++s->failed;
            }
        }
        s->cv_mem.notify_all();
        s->cv_done.notify_all();
    }
}


}  // namespace

extern "C" int iso_server_create(int device, int slots, size_t hbm_budget_bytes, iso_server **out)
{
    iso_clear_error();
    if (!out || slots < 1 || slots > 64 || hbm_budget_bytes == 0) return iso_fail(ISO_ERR_ARG, "iso_server_create: bad argument");
    iso_server *s = new iso_server();
    s->device = device;
    s->budget = hbm_budget_bytes;
    s->workers.resize(slots);
    for (int w = 0; w < slots; ++w) {
        int rc = iso_ctx_create(device, &s->workers[w].ctx);
        if (rc != ISO_OK) {
            for (int k = 0; k < w; ++k) iso_ctx_destroy(s->workers[k].ctx);
            delete s;
            return rc;
        }
    }
    int lo = 0, hi = 0;
    cudaSetDevice(device);
    if (cudaDeviceGetStreamPriorityRange(&lo, &hi) != cudaSuccess) cudaGetLastError();
    for (int w = 0; w < slots; ++w) {
        Worker &k = s->workers[w];
        k.normal = k.ctx->stream;
        if (cudaStreamCreateWithPriority(&k.urgent, cudaStreamNonBlocking, hi) != cudaSuccess) {
            cudaGetLastError();
            k.urgent = nullptr;
        }
    }
    for (int w = 0; w < slots; ++w) s->workers[w].thread = std::thread(worker_loop, s, (size_t)w);
    *out = s;
    return ISO_OK;
}

extern "C" int iso_server_set_policy(iso_server *s, int policy, double max_wait_ms)
{
    iso_clear_error();
    if (!s || (policy != ISO_SERVE_FIFO && policy != ISO_SERVE_SHORTEST_FIRST) || !(max_wait_ms >= 0))
        return iso_fail(ISO_ERR_ARG, "iso_server_set_policy: bad argument");
    std::lock_guard<std::mutex> lock(s->mu);
    s->policy = policy;
    s->max_wait_ms = max_wait_ms;
    return ISO_OK;
}

extern "C" int iso_server_set_limit(iso_server *s, int which, int64_t value)
{
    iso_clear_error();
    if (!s) return iso_fail(ISO_ERR_ARG, "iso_server_set_limit: bad argument");
    std::lock_guard<std::mutex> lock(s->mu);
    // a worker reads its context's settings while it runs a request: only an
    // idle server takes new ones
    bool busy = !s->queue.empty();
    for (const Worker &k : s->workers) busy = busy || k.state != WState::Idle;
    if (busy) return iso_fail(ISO_ERR_ARG, "iso_server_set_limit: requests are queued or running");
    for (Worker &k : s->workers) {
        const int rc = iso_ctx_set_limit(k.ctx, which, value);
        if (rc != ISO_OK) return rc;
    }
    return ISO_OK;
}

extern "C" int iso_server_submit(iso_server *s, const iso_request *req, int64_t *ticket)
{
    iso_clear_error();
    if (!s || !req || !ticket || !req->volume || !req->isovalues || !req->ism_out || !req->field_ids_out)
        return iso_fail(ISO_ERR_ARG, "iso_server_submit: bad argument");
    Job *job = new Job();
    job->req = *req;
    {
        const double ds = req->opts.df_downscale > 0 ? req->opts.df_downscale : 1;
        const double F = (double)req->X * req->Y * req->Z / (ds * ds * ds);
        job->cost = F * req->n * (req->n + 64.0);
    }
    job->t_submit = Clock::now();
    {
        std::lock_guard<std::mutex> lock(s->mu);
        job->ticket = s->next_ticket++;
        s->jobs[job->ticket] = job;
        s->queue.push_back(job);
        *ticket = job->ticket;
    }
    s->cv_queue.notify_one();
    return ISO_OK;
}

extern "C" int iso_server_wait(iso_server *s, int64_t ticket, iso_request_result *result)
{
    iso_clear_error();
    if (!s) return iso_fail(ISO_ERR_ARG, "iso_server_wait: NULL server");
    std::unique_lock<std::mutex> lock(s->mu);
    auto it = s->jobs.find(ticket);
    if (it == s->jobs.end()) return iso_fail(ISO_ERR_ARG, "iso_server_wait: unknown ticket %lld", (long long)ticket);
    Job *job = it->second;
    s->cv_done.wait(lock, [&] { return job->done; });
    if (result) {
        result->status = job->status;
        result->m = job->m;
        result->latency_ms = std::chrono::duration<double, std::milli>(job->t_end - job->t_submit).count();
        result->queue_ms = std::chrono::duration<double, std::milli>(job->t_start - job->t_submit).count();
        result->timing = job->timing;
    }
    int status = job->status;
    std::string err = job->error;
    s->jobs.erase(it);
    delete job;
    if (status != ISO_OK) return iso_fail(status, "%s", err.c_str());
    return ISO_OK;
}

extern "C" int iso_server_get_stats(iso_server *s, iso_server_stats *out)
{
    if (!s || !out) return iso_fail(ISO_ERR_ARG, "iso_server_get_stats: bad argument");
    std::lock_guard<std::mutex> lock(s->mu);
    std::vector<double> l = s->latencies_ms;
    std::sort(l.begin(), l.end());
    auto pct = [&](double p) {
        if (l.empty()) return 0.0;
        size_t i = (size_t)std::min<double>((double)l.size() - 1, std::ceil(p * l.size()) - 1);
        return l[i];
    };
    out->completed = s->completed;
    out->failed = s->failed;
    out->p50_ms = pct(0.50);
    out->p99_ms = pct(0.99);
    out->peak_device_bytes = s->peak_bytes;
    size_t held = 0;
    for (auto &w : s->workers) held += w.held;
    out->held_device_bytes = held;
    return ISO_OK;
}

extern "C" void iso_server_destroy(iso_server *s)
{
    if (!s) return;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        s->stop = true;
    }
    s->cv_queue.notify_all();
    for (auto &w : s->workers)
        if (w.thread.joinable()) w.thread.join();
    for (auto &w : s->workers) {
        if (w.ctx) w.ctx->stream = w.normal;
        iso_ctx_destroy(w.ctx);
        if (w.urgent) cudaStreamDestroy(w.urgent);
    }
    for (auto &kv : s->jobs) delete kv.second;
    delete s;
}
