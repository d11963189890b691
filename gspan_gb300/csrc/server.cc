// Serving loop: mining requests (graph, min_support, k) accepted as they
// arrive and run while others are on the GPU.  No counterpart in the
// reference, which mines one graph per process run.
//
//  * Graphs are uploaded once (gspan_server_add_graph) and stay resident.
//  * `slots` worker threads each own a context (its own CUDA stream), so
//    admitted jobs overlap on the device; a job is the same gspan_mine call it
//    would be alone, so its result is the same.
//  * Admission is first come, first served: the job at the head of the queue
//    starts when a slot is free and its predicted working bytes fit the
//    server's device budget next to the jobs already running (or when nothing
//    else runs).  A job that still runs out of device memory next to others
//    goes back to the head of the queue and then runs alone.
#include "miner.h"

#include <chrono>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>

namespace {

using Clock = std::chrono::steady_clock;

struct Job {
    int64_t id = 0;
    int32_t graph = 0, k = 0, min_support = 0;
    double predicted = 0;        // bytes
    bool alone = false;          // retry after running out of memory beside others
    Clock::time_point submitted, started, finished;
    bool done = false;
    gspan_status status = GSPAN_OK;
    std::string error;
    std::vector<std::vector<gspan_pattern_edge>> codes;
    std::vector<int32_t> supports;
    gspan_stats stats{};
};

}  // namespace

struct gspan_server {
    int device = 0;
    double budget = 0;           // device bytes admitted jobs may be predicted to use
    gspan_ctx* owner = nullptr;  // uploads graphs
    std::vector<gspan_graph*> graphs;
    std::vector<gspan_ctx*> ctxs;
    std::vector<std::thread> workers;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Job*> queue;
    std::unordered_map<int64_t, std::unique_ptr<Job>> jobs;
    int64_t next_id = 1;
    int running = 0;
    double in_use = 0;
    bool stop = false;
};

namespace {

// Working memory a job is expected to need beside its resident graph: the
// first extension level's tables and the mask-path arrays, per level.  A
// coarse model; the out-of-memory retry keeps admission safe when it is low.
double predict_bytes(const gs::DevGraph& g, int k)
{
    const double per_level = 64.0 * g.n + 48.0 * g.m;
    return per_level * std::max(1, k - 1);
}

bool admissible(const gspan_server* s, const Job* j)
{
    if (s->running == 0) return true;
    if (j->alone) return false;
    return s->in_use + j->predicted <= s->budget;
}

void worker(gspan_server* s, gspan_ctx* ctx)
{
    for (;;) {
        Job* job = nullptr;
        const gspan_graph* graph = nullptr;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv_work.wait(lk, [&] { return s->stop || (!s->queue.empty() && admissible(s, s->queue.front())); });
            if (s->stop) return;
            job = s->queue.front();
            s->queue.pop_front();
            ++s->running;
            s->in_use += job->predicted;
            job->started = Clock::now();
            graph = s->graphs[job->graph];   // under the lock: add_graph may grow the vector
        }
        job->codes.clear();
        job->supports.clear();
        gspan_stats st{};
        auto collect = [](void* user, const gspan_pattern_edge* c, int32_t len, int32_t sup) {
            Job* jb = static_cast<Job*>(user);
            jb->codes.emplace_back(c, c + len);
            jb->supports.push_back(sup);
            return 0;
        };
        const gspan_status rc = gspan_mine(ctx, graph, job->k, job->min_support, collect, job, &st);
        {
            std::lock_guard<std::mutex> lk(s->mu);
            --s->running;
            s->in_use -= job->predicted;
            if (rc == GSPAN_ERR_NOMEM && !job->alone) {
                job->alone = true;            // retry with the device to itself
                s->queue.push_front(job);
            } else {
                job->status = rc;
                job->error = rc == GSPAN_OK ? std::string() : std::string(gspan_last_error(ctx));
                job->stats = st;
                job->finished = Clock::now();
                job->done = true;
                s->cv_done.notify_all();
            }
        }
        s->cv_work.notify_all();
    }
}

}  // namespace

extern "C" {

gspan_status gspan_server_create(int32_t device, int32_t slots, double budget_bytes, gspan_server** out)
{
    if (!out || slots < 1 || slots > 64) return GSPAN_ERR_INVALID;
    *out = nullptr;
    gspan_opts o;
    gspan_opts_default(&o);
    o.device = device;
    std::unique_ptr<gspan_server> s(new (std::nothrow) gspan_server());
    if (!s) return GSPAN_ERR_NOMEM;
    s->device = device;
    gspan_status rc = gspan_ctx_create(&o, &s->owner);
    if (rc != GSPAN_OK) return rc;
    size_t free_b = 0, total_b = 0;
    cudaSetDevice(device);
    cudaMemGetInfo(&free_b, &total_b);
    s->budget = budget_bytes > 0 ? budget_bytes : 0.6 * (double)free_b;
    // Each slot's mask-path arrays share the budget.
    o.mem_fraction = std::min(0.4, 0.6 / slots);
    for (int32_t i = 0; i < slots; ++i) {
        gspan_ctx* c = nullptr;
        rc = gspan_ctx_create(&o, &c);
        if (rc != GSPAN_OK) {
            for (gspan_ctx* x : s->ctxs) gspan_ctx_destroy(x);
            gspan_ctx_destroy(s->owner);
            return rc;
        }
        s->ctxs.push_back(c);
    }
    gspan_server* raw = s.release();
    for (gspan_ctx* c : raw->ctxs) raw->workers.emplace_back(worker, raw, c);
    *out = raw;
    return GSPAN_OK;
}

void gspan_server_destroy(gspan_server* s)
{
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    for (auto& t : s->workers) t.join();
    for (gspan_ctx* c : s->ctxs) gspan_ctx_destroy(c);
    for (gspan_graph* g : s->graphs) gspan_graph_free(s->owner, g);
    gspan_ctx_destroy(s->owner);
    delete s;
}

gspan_status gspan_server_add_graph(gspan_server* s, int32_t nr_nodes, int32_t nr_edges, const int32_t* offsets,
                                    const int32_t* vlabels, const gspan_edge* edges, int32_t* graph_id)
{
    if (!s || !graph_id) return GSPAN_ERR_INVALID;
    gspan_graph* g = nullptr;
    std::lock_guard<std::mutex> lk(s->mu);   // the owner context is not shared between threads
    const gspan_status rc = gspan_graph_upload(s->owner, nr_nodes, nr_edges, offsets, vlabels, edges, &g);
    if (rc != GSPAN_OK) return rc;
    s->graphs.push_back(g);
    *graph_id = (int32_t)s->graphs.size() - 1;
    return GSPAN_OK;
}

gspan_status gspan_server_submit(gspan_server* s, int32_t graph_id, int32_t k, int32_t min_support, int64_t* job_id)
{
    if (!s || !job_id) return GSPAN_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    if (graph_id < 0 || graph_id >= (int32_t)s->graphs.size()) return GSPAN_ERR_INVALID;
    std::unique_ptr<Job> j(new (std::nothrow) Job());
    if (!j) return GSPAN_ERR_NOMEM;
    j->id = s->next_id++;
    j->graph = graph_id;
    j->k = k;
    j->min_support = min_support;
    j->predicted = predict_bytes(s->graphs[graph_id]->g, k);
    j->submitted = Clock::now();
    *job_id = j->id;
    s->queue.push_back(j.get());
    s->jobs.emplace(j->id, std::move(j));
    s->cv_work.notify_all();
    return GSPAN_OK;
}

gspan_status gspan_server_wait(gspan_server* s, int64_t job_id, gspan_emit_fn emit, void* user,
                               gspan_job_info* info)
{
    if (!s) return GSPAN_ERR_INVALID;
    std::unique_ptr<Job> job;
    {
        std::unique_lock<std::mutex> lk(s->mu);
        auto it = s->jobs.find(job_id);
        if (it == s->jobs.end()) return GSPAN_ERR_INVALID;
        Job* j = it->second.get();
        s->cv_done.wait(lk, [&] { return j->done; });
        job = std::move(it->second);
        s->jobs.erase(it);
    }
    if (info) {
        info->status = job->status;
        info->queued_ms = std::chrono::duration<double, std::milli>(job->started - job->submitted).count();
        info->run_ms = std::chrono::duration<double, std::milli>(job->finished - job->started).count();
        info->latency_ms = std::chrono::duration<double, std::milli>(job->finished - job->submitted).count();
        info->predicted_bytes = job->predicted;
        info->retried_alone = job->alone ? 1 : 0;
        info->stats = job->stats;
    }
    if (job->status == GSPAN_OK && emit)
        for (size_t i = 0; i < job->codes.size(); ++i)
            if (emit(user, job->codes[i].data(), (int32_t)job->codes[i].size(), job->supports[i]) != 0)
                return GSPAN_ERR_ABORTED;
    return job->status;
}

}  // extern "C"
