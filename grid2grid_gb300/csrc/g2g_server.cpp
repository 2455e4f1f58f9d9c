// Serving loop: continuous batching of transforms of device-resident
// layouts (the g2g_server_* entry points of include/grid2grid_gb300.h).
//
//  submit      plans the request (plan cache keyed by a 128-bit hash of the
//              descriptors, dtype and op) and queues it.
//  dispatcher  one thread: while a launch slot is free, takes every queued
//              request that fits the HBM budget (FIFO, up to
//              max_batch_requests) and issues them as ONE launch of the
//              persistent gather-scatter (g2g_plans_execute) on the next of
//              several streams; a host callback queued behind the launch
//              marks its requests complete, releases their budget and wakes
//              the dispatcher. Launches on different streams overlap.
//  replay      an open-loop driver: submits requests at given arrival times
//              from a native thread (accurate at tens of kHz).
//
// No device-side waits are involved: all waiting is on the host.
#include "g2g_host.hpp"

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <list>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

namespace {

int64_t now_ns() {
    return std::chrono::duration_cast<std::chrono::nanoseconds>(
               std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

struct Req {
    g2g_plan *plan = nullptr;
    int *refs = nullptr; // the plan's cache reference count
    int64_t bytes = 0;   // m*n*sizeof(T)
    int64_t charge = 0;  // bytes held against the budget
    g2g_request_times t{};
    bool done = false;
};

struct CacheEntry {
    g2g_plan *plan = nullptr;
    int64_t bytes = 0;
    int refs = 0; // queued or in-flight requests using the plan
    std::list<g2g::Sig>::iterator lru;
};

struct Launch;

} // namespace

struct g2g_server {
    g2g_server_config cfg{};
    int device = 0;
    std::mutex mu;
    std::condition_variable cv_dispatch, cv_done;
    std::deque<uint64_t> pending;
    std::unordered_map<uint64_t, Req> reqs;
    uint64_t next_ticket = 1;
    int64_t inflight_bytes = 0;
    int inflight_launches = 0;
    std::vector<cudaStream_t> streams;
    int next_stream = 0;
    std::unordered_map<g2g::Sig, CacheEntry, g2g::SigHash> cache;
    std::list<g2g::Sig> lru; // most recent at front
    std::thread dispatcher;
    bool stop = false;
    g2g_server_stats stats{};
};

namespace {

struct Launch {
    g2g_server *srv;
    std::vector<uint64_t> tickets;
    int64_t charge;
};

void CUDART_CB on_launch_done(void *arg) {
    Launch *L = (Launch *)arg;
    g2g_server *s = L->srv;
    const int64_t t = now_ns();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        for (uint64_t tk : L->tickets) {
            auto it = s->reqs.find(tk);
            if (it == s->reqs.end())
                continue;
            Req &r = it->second;
            r.t.complete_ns = t;
            r.done = true;
            s->stats.completed++;
            s->stats.bytes_completed += r.bytes;
            if (r.refs)
                --*r.refs;
        }
        s->inflight_bytes -= L->charge;
        s->inflight_launches--;
    }
    s->cv_dispatch.notify_all();
    s->cv_done.notify_all();
    delete L;
}

void dispatch_loop(g2g_server *s) {
    cudaSetDevice(s->device);
    const int64_t budget = s->cfg.hbm_budget_bytes;
    std::unique_lock<std::mutex> lk(s->mu);
    for (;;) {
        s->cv_dispatch.wait(lk, [&] {
            if (s->stop && s->pending.empty())
                return true;
            if (s->pending.empty() || s->inflight_launches >= s->cfg.max_launches_in_flight)
                return false;
            const Req &head = s->reqs[s->pending.front()];
            return s->inflight_bytes + head.charge <= budget;
        });
        if (s->stop && s->pending.empty())
            break;
        Launch *L = new Launch{s, {}, 0};
        std::vector<g2g_plan *> plans;
        while (!s->pending.empty() && (int)plans.size() < s->cfg.max_batch_requests) {
            Req &r = s->reqs[s->pending.front()];
            if (s->inflight_bytes + L->charge + r.charge > budget)
                break;
            L->charge += r.charge;
            L->tickets.push_back(s->pending.front());
            plans.push_back(r.plan);
            s->pending.pop_front();
        }
        s->inflight_bytes += L->charge;
        s->inflight_launches++;
        s->stats.launches++;
        s->stats.inflight_bytes_peak = std::max(s->stats.inflight_bytes_peak, s->inflight_bytes);
        cudaStream_t st = s->streams[s->next_stream];
        s->next_stream = (s->next_stream + 1) % (int)s->streams.size();
        // record launch data while the requests are certainly alive: once the
        // launch is issued its callback may complete them at any time
        const int64_t t_launch = now_ns();
        for (uint64_t tk : L->tickets) {
            Req &r = s->reqs[tk];
            r.t.launch_ns = t_launch;
            r.t.batch_size = (int32_t)L->tickets.size();
        }
        lk.unlock();
        g2g_status rc = g2g_plans_execute((int32_t)plans.size(), plans.data(), st);
        cudaError_t ce = cudaSuccess;
        if (rc == G2G_SUCCESS)
            ce = cudaLaunchHostFunc(st, on_launch_done, L);
        if (rc != G2G_SUCCESS || ce != cudaSuccess) {
            // nothing will call back: finish the requests here with the error
            {
                std::lock_guard<std::mutex> g(s->mu);
                for (uint64_t tk : L->tickets)
                    s->reqs[tk].t.status = rc != G2G_SUCCESS ? rc : G2G_ERROR_CUDA;
            }
            on_launch_done(L);
        }
        lk.lock();
    }
}

// Plans (or finds) the request's plan and takes a reference on it (released
// when the request completes); the caller holds no lock. Cache entries are
// node-stable and never erased while referenced, so *refs stays valid.
g2g_status plan_for(g2g_server *s, const g2g_layout_desc *init, const g2g_layout_desc *fin,
                    g2g_dtype dtype, const g2g_op *op, g2g_plan **plan, int64_t *bytes,
                    int **refs) {
    g2g::Sig sig;
    g2g::add_layout(sig, init);
    g2g::add_layout(sig, fin);
    sig.add(dtype);
    g2g_op o;
    std::memset(&o, 0, sizeof(o));
    o.trans = 'N';
    o.alpha[0] = 1.0;
    if (op) {
        o.trans = op->trans;
        o.alpha[0] = op->alpha[0];
        o.alpha[1] = op->alpha[1];
        o.beta[0] = op->beta[0];
        o.beta[1] = op->beta[1];
    }
    sig.add(o.trans);
    sig.add(o.alpha);
    sig.add(o.beta);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        auto it = s->cache.find(sig);
        if (it != s->cache.end()) {
            it->second.refs++;
            s->lru.erase(it->second.lru);
            s->lru.push_front(sig);
            it->second.lru = s->lru.begin();
            s->stats.plan_cache_hits++;
            *plan = it->second.plan;
            *bytes = it->second.bytes;
            *refs = &it->second.refs;
            return G2G_SUCCESS;
        }
    }
    g2g_plan *p = nullptr;
    g2g_status st = g2g_plan_create(init, fin, dtype, &o, nullptr, &p);
    if (st != G2G_SUCCESS)
        return st;
    const int64_t b = g2g::plan_bytes_moved(p);
    std::vector<g2g_plan *> evicted;
    int *r = nullptr;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        auto it = s->cache.find(sig);
        if (it != s->cache.end()) { // planned concurrently by another thread
            evicted.push_back(p);
            it->second.refs++;
            p = it->second.plan;
            r = &it->second.refs;
        } else {
            s->lru.push_front(sig);
            CacheEntry ce;
            ce.plan = p;
            ce.bytes = b;
            ce.refs = 1;
            ce.lru = s->lru.begin();
            r = &s->cache.emplace(sig, ce).first->second.refs;
            s->stats.plan_cache_misses++;
            // evict least recently used plans no request holds
            auto li = s->lru.end();
            while ((int)s->cache.size() > s->cfg.plan_cache_entries && li != s->lru.begin()) {
                --li;
                auto ci = s->cache.find(*li);
                if (ci != s->cache.end() && ci->second.refs == 0) {
                    evicted.push_back(ci->second.plan);
                    s->cache.erase(ci);
                    li = s->lru.erase(li);
                }
            }
        }
    }
    for (g2g_plan *e : evicted)
        g2g_plan_destroy(e); // stream-ordered: waits for its last launch
    *plan = p;
    *bytes = b;
    *refs = r;
    return G2G_SUCCESS;
}

// Queues a planned request that holds one reference on its plan.
g2g_status enqueue(g2g_server *s, g2g_plan *plan, int *refs, int64_t bytes, uint64_t *ticket) {
    const int64_t charge = 2 * bytes; // source + destination
    if (charge > s->cfg.hbm_budget_bytes) {
        std::lock_guard<std::mutex> lk(s->mu);
        if (refs)
            --*refs;
        return g2g::fail(G2G_ERROR_BUDGET,
                         "request of %lld bytes exceeds the server's HBM budget of %lld",
                         (long long)charge, (long long)s->cfg.hbm_budget_bytes);
    }
    {
        std::lock_guard<std::mutex> lk(s->mu);
        const uint64_t tk = s->next_ticket++;
        Req r;
        r.plan = plan;
        r.refs = refs;
        r.bytes = bytes;
        r.charge = charge;
        r.t.submit_ns = now_ns();
        r.t.bytes = bytes;
        s->reqs.emplace(tk, r);
        s->pending.push_back(tk);
        s->stats.submitted++;
        *ticket = tk;
    }
    s->cv_dispatch.notify_one();
    return G2G_SUCCESS;
}

} // namespace

extern "C" {

g2g_status g2g_server_create(const g2g_server_config *config, g2g_server **out) {
    if (!out)
        return g2g::fail(G2G_ERROR_INVALID_ARGUMENT, "server output pointer is NULL");
    *out = nullptr;
    g2g_server *s = new g2g_server();
    if (config)
        s->cfg = *config;
    if (s->cfg.hbm_budget_bytes <= 0)
        s->cfg.hbm_budget_bytes = 120ll * 1000 * 1000 * 1000;
    if (s->cfg.max_launches_in_flight <= 0)
        s->cfg.max_launches_in_flight = 3;
    if (s->cfg.max_batch_requests <= 0 || s->cfg.max_batch_requests > 256)
        s->cfg.max_batch_requests = 256;
    if (s->cfg.plan_cache_entries <= 0)
        s->cfg.plan_cache_entries = 4096;
    cudaError_t e = cudaGetDevice(&s->device);
    // every kernel instance a batch can select is loaded now, not by the
    // first request that needs it (a lazily loaded module costs milliseconds)
    if (e == cudaSuccess)
        e = g2g::preload_scatter_kernels();
    for (int k = 0; e == cudaSuccess && k < s->cfg.max_launches_in_flight; ++k) {
        cudaStream_t st;
        e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
        if (e == cudaSuccess)
            s->streams.push_back(st);
    }
    if (e != cudaSuccess) {
        for (cudaStream_t st : s->streams)
            cudaStreamDestroy(st);
        delete s;
        return g2g::fail(G2G_ERROR_CUDA, "server: %s", cudaGetErrorString(e));
    }
    s->dispatcher = std::thread(dispatch_loop, s);
    *out = s;
    return G2G_SUCCESS;
}

g2g_status g2g_server_submit(g2g_server *s, const g2g_layout_desc *initial,
                             const g2g_layout_desc *final_, g2g_dtype dtype, const g2g_op *op,
                             uint64_t *ticket) {
    if (!s || !ticket)
        return g2g::fail(G2G_ERROR_INVALID_ARGUMENT, "server or ticket is NULL");
    g2g_plan *plan = nullptr;
    int64_t bytes = 0;
    int *refs = nullptr;
    g2g_status st = plan_for(s, initial, final_, dtype, op, &plan, &bytes, &refs);
    if (st != G2G_SUCCESS)
        return st;
    return enqueue(s, plan, refs, bytes, ticket);
}

g2g_status g2g_server_wait(g2g_server *s, uint64_t ticket, int64_t timeout_us,
                           g2g_request_times *times) {
    if (!s)
        return g2g::fail(G2G_ERROR_INVALID_ARGUMENT, "server is NULL");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end())
        return g2g::fail(G2G_ERROR_INVALID_ARGUMENT, "unknown ticket %llu",
                         (unsigned long long)ticket);
    auto ready = [&] { return s->reqs[ticket].done; };
    if (timeout_us < 0)
        s->cv_done.wait(lk, ready);
    else if (!s->cv_done.wait_for(lk, std::chrono::microseconds(timeout_us), ready))
        return G2G_ERROR_NOT_READY;
    Req r = s->reqs[ticket];
    s->reqs.erase(ticket);
    if (times)
        *times = r.t;
    if (r.t.status != G2G_SUCCESS)
        return g2g::fail((g2g_status)r.t.status, "request %llu failed",
                         (unsigned long long)ticket);
    return G2G_SUCCESS;
}

g2g_status g2g_server_replay(g2g_server *s, int32_t n_pairs, const g2g_layout_desc *initials,
                             const g2g_layout_desc *finals, const g2g_dtype *dtypes,
                             const g2g_op *ops, int64_t n_requests, const int32_t *pair_index,
                             const double *arrival_s, g2g_request_times *times) {
    if (!s || n_pairs < 1 || !initials || !finals || !dtypes || n_requests < 0 ||
        (n_requests > 0 && (!pair_index || !arrival_s || !times)))
        return g2g::fail(G2G_ERROR_INVALID_ARGUMENT, "replay: bad arguments");
    for (int64_t k = 0; k < n_requests; ++k)
        if (pair_index[k] < 0 || pair_index[k] >= n_pairs)
            return g2g::fail(G2G_ERROR_INVALID_ARGUMENT, "replay: pair index out of range");
    // plan every pair up front (cache), so submissions cost no planning
    std::vector<g2g_plan *> plans(n_pairs);
    std::vector<int64_t> bytes(n_pairs);
    std::vector<int *> refs(n_pairs);
    for (int k = 0; k < n_pairs; ++k) {
        g2g_status st = plan_for(s, &initials[k], &finals[k], dtypes[k], ops ? &ops[k] : nullptr,
                                 &plans[k], &bytes[k], &refs[k]);
        if (st != G2G_SUCCESS) {
            std::lock_guard<std::mutex> lk(s->mu);
            for (int j = 0; j < k; ++j)
                --*refs[j];
            return st;
        }
    }
    std::vector<uint64_t> tickets((size_t)n_requests, 0);
    std::vector<int32_t> rejected((size_t)n_requests, 0);
    const int64_t t0 = now_ns();
    for (int64_t k = 0; k < n_requests; ++k) {
        const int64_t target = t0 + (int64_t)(arrival_s[k] * 1e9);
        for (;;) { // sleep coarsely, then spin to the arrival time
            const int64_t left = target - now_ns();
            if (left <= 0)
                break;
            if (left > 200000)
                std::this_thread::sleep_for(std::chrono::nanoseconds(left - 100000));
        }
        const int p = pair_index[k];
        {
            std::lock_guard<std::mutex> lk(s->mu);
            ++*refs[p];
        }
        g2g_status st = enqueue(s, plans[p], refs[p], bytes[p], &tickets[k]);
        if (st != G2G_SUCCESS)
            rejected[k] = st;
    }
    g2g_status result = G2G_SUCCESS;
    for (int64_t k = 0; k < n_requests; ++k) {
        std::memset(&times[k], 0, sizeof(times[k]));
        if (rejected[k]) {
            times[k].status = rejected[k];
            times[k].bytes = bytes[pair_index[k]];
            continue;
        }
        g2g_status st = g2g_server_wait(s, tickets[k], -1, &times[k]);
        if (st != G2G_SUCCESS && result == G2G_SUCCESS)
            result = st;
    }
    // drop the references replay took when planning
    {
        std::lock_guard<std::mutex> lk(s->mu);
        for (int k = 0; k < n_pairs; ++k)
            --*refs[k];
    }
    return result;
}

g2g_status g2g_server_get_stats(const g2g_server *s, g2g_server_stats *stats) {
    if (!s || !stats)
        return g2g::fail(G2G_ERROR_INVALID_ARGUMENT, "server or stats is NULL");
    g2g_server *m = const_cast<g2g_server *>(s);
    std::lock_guard<std::mutex> lk(m->mu);
    *stats = m->stats;
    stats->plan_cache_hits = m->stats.plan_cache_hits;
    return G2G_SUCCESS;
}

g2g_status g2g_server_destroy(g2g_server *s) {
    if (!s)
        return G2G_SUCCESS;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_dispatch.notify_all();
    if (s->dispatcher.joinable())
        s->dispatcher.join();
    cudaSetDevice(s->device);
    for (cudaStream_t st : s->streams)
        cudaStreamSynchronize(st); // callbacks of the last launches have run
    for (auto &ce : s->cache)
        g2g_plan_destroy(ce.second.plan);
    for (cudaStream_t st : s->streams)
        cudaStreamDestroy(st);
    delete s;
    return G2G_SUCCESS;
}

} // extern "C"
