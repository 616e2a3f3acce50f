// Request server: independent surface solves of different meshes,
// wavenumbers and source counts run concurrently on one GPU.
//
// Each worker thread drives one solver handle at a time, and every handle has
// its own non-blocking CUDA stream, so the assembly and Krylov kernels of
// different requests overlap on the device.  A request is admitted when a
// worker is free and its estimated device footprint fits the HBM budget next
// to everything already resident (requests in flight and cached systems);
// idle cached systems are evicted, least recently used first, to make room.
// The queue is served in arrival order, except that a request that does not
// fit yet is passed over by later ones that do; once passed over
// 4 x slots times it blocks the requests behind it, so it cannot starve.
//
// Assembled systems are keyed by a 64-bit hash of the geometry (nodes,
// elements, boundary condition, CHIEF points) and the wavenumber; a request
// whose key matches an idle cached system reuses its A and rebuilds only
// B = p_inc - beta for its own sources.  Two requests with the same key never
// run at once: the second waits for the first to release the system.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "bem_common.h"
#include "solver.h"

namespace bem {
namespace {

using Clock = std::chrono::steady_clock;

inline uint64_t splitmix(uint64_t x) {
    x += 0x9e3779b97f4a7c15ull;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
    return x ^ (x >> 31);
}

uint64_t hash_bytes(uint64_t h, const void *p, size_t n) {
    const unsigned char *c = static_cast<const unsigned char *>(p);
    size_t i = 0;
    for (; i + 8 <= n; i += 8) {
        uint64_t v;
        std::memcpy(&v, c + i, 8);
        h = splitmix(h ^ v);
    }
    uint64_t v = 0;
    std::memcpy(&v, c + i, n - i);
    return splitmix(h ^ v ^ (uint64_t)n);
}

double ms_between(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

struct Request {
    long long ticket = 0;
    std::vector<double> pnts, bc, chief;
    std::vector<int> elems;
    std::vector<bem_source_t> srcs;
    int N = 0, E = 0, M = 0, S = 0, method = BEM_SOLVE_GMRES_REFINED;
    double k = 0.0;
    uint64_t key = 0;
    size_t est = 0;
    int passed_over = 0;
    Clock::time_point t_submit, t_start, t_end;
    bool done = false;
    int status = BEM_SUCCESS;
    std::string error;
    bem_solve_info_t info{};
    bool cache_hit = false;
    std::vector<double> x;   // N x S c128, column-major, ld = N
};

struct Entry {
    uint64_t key = 0;
    std::unique_ptr<bem_solver_s> solver;
    size_t bytes = 0;          // counted against the budget
    bool busy = false, assembled = false;
    Clock::time_point last_use;
};

}  // namespace
}  // namespace bem

using namespace bem;

struct bem_server_s {
    bem_server_options_t opt{};
    int device = 0;
    size_t budget = 0;

    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<std::shared_ptr<Request>> queue;
    std::unordered_map<long long, std::shared_ptr<Request>> reqs;
    std::map<uint64_t, std::shared_ptr<Entry>> cache;
    size_t resident = 0, peak = 0;
    int in_flight = 0, max_in_flight = 0;
    long long next_ticket = 1;
    long long submitted = 0, completed = 0, failed = 0, solves = 0, hits = 0, evictions = 0;
    std::vector<double> latencies;
    bool stop = false;
    std::vector<std::thread> workers;

    void worker();
    // Under mu: the next admissible request and the entry it runs on, or
    // false.  Systems evicted to make room are moved to `evicted`.
    bool pick(std::shared_ptr<Request> &req, std::shared_ptr<Entry> &ent,
              std::vector<std::unique_ptr<bem_solver_s>> &evicted);
    bool evict_one(uint64_t keep, std::vector<std::unique_ptr<bem_solver_s>> &evicted);
    void finish(const std::shared_ptr<Request> &req, int status, const std::string &err);
};

bool bem_server_s::evict_one(uint64_t keep, std::vector<std::unique_ptr<bem_solver_s>> &evicted) {
    auto victim = cache.end();
    for (auto it = cache.begin(); it != cache.end(); ++it) {
        if (it->second->busy || it->first == keep) continue;
        if (victim == cache.end() || it->second->last_use < victim->second->last_use) victim = it;
    }
    if (victim == cache.end()) return false;
    resident -= std::min(resident, victim->second->bytes);
    if (victim->second->solver) evicted.push_back(std::move(victim->second->solver));
    cache.erase(victim);
    evictions++;
    return true;
}

void bem_server_s::finish(const std::shared_ptr<Request> &req, int status, const std::string &err) {
    req->status = status;
    req->error = err;
    req->t_end = Clock::now();
    req->done = true;
    if (status == BEM_SUCCESS || status == BEM_ERR_NOT_CONVERGED) {
        completed++;
        solves += req->S;
        latencies.push_back(ms_between(req->t_submit, req->t_end));
    } else {
        failed++;
    }
}

bool bem_server_s::pick(std::shared_ptr<Request> &req, std::shared_ptr<Entry> &ent,
                        std::vector<std::unique_ptr<bem_solver_s>> &evicted) {
    std::vector<Request *> skipped;
    for (auto qi = queue.begin(); qi != queue.end(); ++qi) {
        const std::shared_ptr<Request> r = *qi;
        auto ce = cache.find(r->key);
        bool fits = false;
        size_t need = 0;
        if (ce == cache.end() || !ce->second->busy) {
            const size_t have = ce != cache.end() ? ce->second->bytes : 0;
            need = r->est > have ? r->est - have : 0;
            size_t idle = 0;   // bytes of cached systems that eviction could free
            for (auto &kv : cache)
                if (!kv.second->busy && kv.first != r->key) idle += kv.second->bytes;
            if (resident + need <= budget) {
                fits = true;
            } else if (resident - std::min(resident, idle) + need <= budget) {
                while (resident + need > budget && evict_one(r->key, evicted)) {}
                fits = resident + need <= budget;
            } else if (in_flight == 0 && (r->est > budget || resident - std::min(resident, idle + have) == 0)) {
                // Nothing running and even an empty device would not hold it.
                finish(r, BEM_ERR_TOO_LARGE,
                       "request needs " + std::to_string(r->est) + " device bytes, budget is " +
                           std::to_string(budget));
                queue.erase(qi);
                cv_done.notify_all();
                return pick(req, ent, evicted);
            }
        }
        if (!fits) {
            // a request passed over too often holds back the ones behind it
            if (r->passed_over >= 4 * std::max(1, opt.slots)) return false;
            skipped.push_back(r.get());
            continue;
        }
        for (Request *p : skipped) p->passed_over++;
        if (ce == cache.end()) {
            auto e = std::make_shared<Entry>();
            e->key = r->key;
            ce = cache.emplace(r->key, e).first;
        }
        ent = ce->second;
        ent->busy = true;
        ent->bytes += need;
        resident += need;
        peak = std::max(peak, resident);
        in_flight++;
        max_in_flight = std::max(max_in_flight, in_flight);
        req = r;
        queue.erase(qi);
        return true;
    }
    return false;
}

void bem_server_s::worker() {
    cudaSetDevice(device);
    for (;;) {
        std::shared_ptr<Request> req;
        std::shared_ptr<Entry> ent;
        std::vector<std::unique_ptr<bem_solver_s>> evicted;
        {
            std::unique_lock<std::mutex> lk(mu);
            cv_work.wait(lk, [&] { return (stop && queue.empty()) || pick(req, ent, evicted); });
            if (!req) {
                evicted.clear();
                return;
            }
            req->t_start = Clock::now();
        }
        evicted.clear();   // frees the evicted systems' device memory before this request allocates
        int status = BEM_SUCCESS;
        std::string err;
        try {
            if (!ent->solver) {
                ent->solver.reset(new bem_solver_s());
                ent->solver->opt = opt.solver;
            }
            bem_solver_s &sv = *ent->solver;
            if (!ent->assembled) {
                sv.set_geometry(req->pnts.data(), req->N, req->elems.data(), req->E,
                                req->bc.empty() ? nullptr : req->bc.data(),
                                req->chief.empty() ? nullptr : req->chief.data(), req->M);
                sv.set_sources(req->srcs.data(), req->S);
                sv.assemble(req->k, BEM_PREC_C64);
                ent->assembled = true;
            } else {
                sv.set_sources(req->srcs.data(), req->S);   // A reused, B rebuilt
                req->cache_hit = true;
            }
            sv.solve(req->method, &req->info);
            req->x.resize((size_t)2 * req->N * req->S);
            sv.get_solution(req->x.data(), req->N, BEM_PREC_C128);
            if (!req->info.converged) status = BEM_ERR_NOT_CONVERGED;
        } catch (const bem::Error &e) {
            status = e.status;
            err = e.what();
        } catch (const std::bad_alloc &) {
            status = BEM_ERR_NOMEM;
            err = "host out of memory";
        } catch (const std::exception &e) {
            status = BEM_FAILURE;
            err = e.what();
        }
        std::unique_ptr<bem_solver_s> drop;
        {
            std::lock_guard<std::mutex> lk(mu);
            in_flight--;
            ent->busy = false;
            ent->last_use = Clock::now();
            const bool keep = ent->assembled && status != BEM_FAILURE && status != BEM_ERR_CUDA &&
                              status != BEM_ERR_NOMEM && opt.cache_systems > 0;
            if (keep) {
                // true up the reservation to what the handle really holds
                const size_t actual = ent->solver->device_bytes();
                resident = resident - std::min(resident, ent->bytes) + actual;
                ent->bytes = actual;
                peak = std::max(peak, resident);
            } else {
                resident -= std::min(resident, ent->bytes);
                drop = std::move(ent->solver);
                cache.erase(ent->key);
            }
            if (req->cache_hit && status == BEM_SUCCESS) hits++;
            finish(req, status, err);
        }
        drop.reset();
        {
            std::lock_guard<std::mutex> lk(mu);
            int idle = 0;
            for (auto &kv : cache) idle += kv.second->busy ? 0 : 1;
            while (idle > opt.cache_systems && evict_one(0, evicted)) idle--;
        }
        evicted.clear();
        cv_done.notify_all();
        cv_work.notify_all();
    }
}

extern "C" {

int bem_server_options_default(bem_server_options_t *o) {
    if (!o) return BEM_ERR_INVALID_ARG;
    o->slots = 4;
    o->hbm_budget_bytes = 0.0;
    o->cache_systems = 8;
    o->block_min_sources = 4;
    return bem_options_default(&o->solver);
}

int bem_server_create(const bem_server_options_t *o, bem_server_t *out) {
    BEM_API_BEGIN
    BEM_CHECK_ARG(o && out, "null argument");
    BEM_CHECK_ARG(o->slots >= 1 && o->slots <= 64, "slots must be in [1, 64]");
    BEM_CHECK_ARG(o->hbm_budget_bytes >= 0 && o->cache_systems >= 0 && o->block_min_sources >= 1,
                  "bad server options");
    validate_options(o->solver);
    int dev = 0;
    CUDA_TRY(cudaGetDevice(&dev));
    size_t free_b = 0, total_b = 0;
    CUDA_TRY(cudaMemGetInfo(&free_b, &total_b));
    std::unique_ptr<bem_server_s> s(new bem_server_s());
    s->opt = *o;
    s->device = dev;
    s->budget = o->hbm_budget_bytes > 0 ? (size_t)o->hbm_budget_bytes : (size_t)(0.85 * (double)free_b);
    for (int i = 0; i < o->slots; i++) s->workers.emplace_back(&bem_server_s::worker, s.get());
    *out = s.release();
    BEM_API_END
}

int bem_server_destroy(bem_server_t s) {
    if (!s) return BEM_SUCCESS;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    for (auto &t : s->workers) t.join();
    int cur = -1;
    cudaGetDevice(&cur);
    cudaSetDevice(s->device);
    s->cache.clear();
    if (cur >= 0) cudaSetDevice(cur);
    delete s;
    return BEM_SUCCESS;
}

int bem_server_submit(bem_server_t s, const bem_request_t *r, long long *ticket) {
    BEM_API_BEGIN
    BEM_CHECK_ARG(s && r && ticket, "null argument");
    BEM_CHECK_ARG(r->pnts && r->elems && r->num_pnts > 0 && r->num_elems > 0, "empty geometry");
    BEM_CHECK_ARG(r->num_chief >= 0 && (r->num_chief == 0 || r->chief), "bad CHIEF points");
    BEM_CHECK_ARG(r->srcs && r->num_srcs >= 1 && r->num_srcs <= 65535, "need 1 to 65535 sources");
    BEM_CHECK_ARG(std::isfinite(r->k) && r->k > 0, "wavenumber must be positive");
    for (long long i = 0; i < 3LL * r->num_elems; i++)
        BEM_CHECK_ARG(r->elems[i] >= 0 && r->elems[i] < r->num_pnts, "element node index out of range");
    for (int i = 0; i < r->num_srcs; i++)
        BEM_CHECK_ARG(r->srcs[i].kind == BEM_SRC_POINT || r->srcs[i].kind == BEM_SRC_PLANE, "bad source kind");
    if (r->bc)
        for (int e = 0; e < r->num_elems; e++)
            BEM_CHECK_ARG(r->bc[6 * e + 2] != 0.0 || r->bc[6 * e + 3] != 0.0, "cb must be nonzero");
    auto q = std::make_shared<Request>();
    q->N = r->num_pnts;
    q->E = r->num_elems;
    q->M = r->num_chief;
    q->S = r->num_srcs;
    q->k = r->k;
    q->pnts.assign(r->pnts, r->pnts + 3 * (size_t)q->N);
    q->elems.assign(r->elems, r->elems + 3 * (size_t)q->E);
    if (r->bc) q->bc.assign(r->bc, r->bc + 6 * (size_t)q->E);
    if (q->M) q->chief.assign(r->chief, r->chief + 3 * (size_t)q->M);
    q->srcs.assign(r->srcs, r->srcs + q->S);
    uint64_t h = 0x6a09e667f3bcc908ull;
    h = hash_bytes(h, q->pnts.data(), sizeof(double) * q->pnts.size());
    h = hash_bytes(h, q->elems.data(), sizeof(int) * q->elems.size());
    h = hash_bytes(h, q->bc.data(), sizeof(double) * q->bc.size());
    h = hash_bytes(h, q->chief.data(), sizeof(double) * q->chief.size());
    h = hash_bytes(h, &q->k, sizeof(double));
    q->key = h ? h : 1;
    q->method = q->S >= s->opt.block_min_sources ? BEM_SOLVE_BLOCK_GMRES : BEM_SOLVE_GMRES_REFINED;
    q->est = bem_solver_s::estimate_bytes(q->N, q->E, q->M, q->S, q->method, s->opt.solver);
    q->t_submit = Clock::now();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        BEM_CHECK_ARG(!s->stop, "server is shutting down");
        q->ticket = s->next_ticket++;
        s->reqs[q->ticket] = q;
        s->queue.push_back(q);
        s->submitted++;
        *ticket = q->ticket;
    }
    s->cv_work.notify_all();
    BEM_API_END
}

int bem_server_wait(bem_server_t s, long long ticket, double timeout_s, void *x, int ldx,
                    bem_request_result_t *res) {
    int status = BEM_SUCCESS;
    BEM_API_BEGIN
    BEM_CHECK_ARG(s, "null server");
    std::shared_ptr<Request> q;
    {
        std::unique_lock<std::mutex> lk(s->mu);
        auto it = s->reqs.find(ticket);
        BEM_CHECK_ARG(it != s->reqs.end(), "unknown or already collected ticket");
        q = it->second;
        BEM_CHECK_ARG(!x || ldx >= q->N, "ldx must be >= the number of nodes");
        auto ready = [&] { return q->done; };
        if (timeout_s < 0) {
            s->cv_done.wait(lk, ready);
        } else if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), ready)) {
            BEM_FAIL(BEM_ERR_TIMEOUT, "request still running");
        }
        s->reqs.erase(it);
    }
    if (x && !q->x.empty())
        for (int c = 0; c < q->S; c++)
            std::memcpy(static_cast<double *>(x) + 2 * (size_t)c * ldx, q->x.data() + 2 * (size_t)c * q->N,
                        sizeof(double) * 2 * q->N);
    if (res) {
        res->status = q->status;
        res->method = q->method;
        res->iterations = q->info.iterations;
        res->refinements = q->info.refinements;
        res->converged = q->info.converged;
        res->rel_residual = q->info.rel_residual;
        res->queue_ms = q->t_start.time_since_epoch().count() ? ms_between(q->t_submit, q->t_start) : 0.0;
        res->service_ms = q->t_start.time_since_epoch().count() ? ms_between(q->t_start, q->t_end) : 0.0;
        res->latency_ms = ms_between(q->t_submit, q->t_end);
        res->cache_hit = q->cache_hit ? 1 : 0;
        res->device_bytes = (double)q->est;
        res->num_pnts = q->N;
        res->num_srcs = q->S;
    }
    status = q->status;
    if (status != BEM_SUCCESS) g_last_error = q->error;
    if (status != BEM_SUCCESS) return status;
    BEM_API_END
}

int bem_server_stats(bem_server_t s, bem_server_stats_t *st) {
    BEM_API_BEGIN
    BEM_CHECK_ARG(s && st, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    std::memset(st, 0, sizeof(*st));
    st->submitted = s->submitted;
    st->completed = s->completed;
    st->failed = s->failed;
    st->solves = s->solves;
    st->cache_hits = s->hits;
    st->evictions = s->evictions;
    st->resident_bytes = (double)s->resident;
    st->peak_bytes = (double)s->peak;
    st->max_in_flight = s->max_in_flight;
    if (!s->latencies.empty()) {
        std::vector<double> l = s->latencies;
        std::sort(l.begin(), l.end());
        auto pct = [&](double p) {
            // nearest-rank percentile
            size_t i = (size_t)std::ceil(p / 100.0 * (double)l.size());
            return l[std::min(l.size(), std::max<size_t>(i, 1)) - 1];
        };
        st->p50_ms = pct(50.0);
        st->p99_ms = pct(99.0);
        st->max_ms = l.back();
        double sum = 0;
        for (double v : l) sum += v;
        st->mean_ms = sum / (double)l.size();
    }
    BEM_API_END
}

int bem_server_reset_stats(bem_server_t s) {
    BEM_API_BEGIN
    BEM_CHECK_ARG(s, "null server");
    std::lock_guard<std::mutex> lk(s->mu);
    s->submitted = s->completed = s->failed = s->solves = s->hits = s->evictions = 0;
    s->latencies.clear();
    s->peak = s->resident;
    s->max_in_flight = s->in_flight;
    BEM_API_END
}

}  // extern "C"
