// Serving loop: builds and lookup batches of different sizes arrive at any
// time from any host thread; DAGs stay resident in HBM under a byte budget.
//
// The reference has no serving layer (its app precomputes one shadow and
// evaluates it every frame, src/main.cpp:236-268).  Here a worker thread
// owns the context and runs continuous batching:
//   * every pass it first retires finished lookup launches (event polling),
//     then launches ALL pending lookups whose DAG is resident as one
//     segmented multi-DAG kernel on the lookup stream (each request reads
//     its points and writes its bits where they lie), then builds the
//     pending maps as one batch (one plan, one graph launch) on the build
//     stream -- so lookups keep running on the device while a build runs,
//     and requests that arrive meanwhile join the next launch;
//   * a lookup waits while a build of its key is queued or running, and
//     fails (CPVS_ERR_INVALID_ARG) for a key that is neither resident nor
//     being built;
//   * residency: least-recently-used DAGs that no in-flight lookup pins are
//     evicted while the resident bytes exceed the budget; a build whose DAG
//     alone exceeds the budget fails with CPVS_ERR_BUDGET.
// Every request's answer is the one the plain API gives for it alone.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <list>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "objects.h"

using cpvs::fail;

namespace {

using Clock = std::chrono::steady_clock;

enum Kind { kBuild = 0, kLookup = 1 };
enum State { kQueued = 0, kRunning = 1, kDone = 2 };

struct Request {
    uint64_t ticket = 0;
    Kind kind = kBuild;
    uint64_t key = 0;
    const float* depth = nullptr;  // build
    uint32_t n = 0;
    const float* xyz = nullptr;  // lookup
    uint64_t count = 0;
    uint32_t* bits = nullptr;
    std::atomic<int> state{kQueued};  // kQueued -> kRunning (worker) | kDone (cancel); kRunning -> kDone
    bool claim() {  // worker: take a queued request; false when it was cancelled
        int q = kQueued;
        return state.compare_exchange_strong(q, kRunning);
    }
    cpvs_status status = CPVS_OK;
    std::string error;
    Clock::time_point t_submit, t_done;
};
using Req = std::shared_ptr<Request>;

struct Resident {
    cpvs_shadow* sh = nullptr;
    uint64_t bytes = 0;
    uint64_t last_use = 0;  // LRU tick
    int pins = 0;           // in-flight lookups reading it
};

struct InFlight {
    cudaEvent_t done = nullptr;
    std::vector<Req> reqs;
    std::vector<uint64_t> keys;         // pinned
    std::vector<cpvs_shadow*> retired;  // replaced while pinned: destroyed when this retires
    void* scratch = nullptr;            // segment + DAG tables
    uint64_t scratch_bytes = 0;
};

double pct(std::vector<double> v, double p) {
    if (v.empty()) return 0.0;
    std::sort(v.begin(), v.end());
    const size_t i = (size_t)std::min<double>(v.size() - 1, std::max(0.0, p * (v.size() - 1) + 0.5));
    return v[i];
}

}  // namespace

struct cpvs_server {
    cpvs_ctx* ctx = nullptr;
    cpvs_server_config cfg{};
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Req> queue;
    std::unordered_map<uint64_t, Req> tickets;
    uint64_t next_ticket = 1;
    bool stop = false;
    std::thread worker;
    // worker-thread state
    cudaStream_t s_build = nullptr, s_lookup = nullptr;
    std::unordered_map<uint64_t, Resident> resident;
    uint64_t resident_bytes = 0;
    uint64_t tick = 0;
    std::deque<InFlight> inflight;
    // statistics (under mu)
    std::vector<double> lat[2];
    uint64_t done_count[2] = {0, 0}, failed = 0, cancelled = 0, evictions = 0;
    uint64_t stat_resident_dags = 0, stat_resident_bytes = 0;

    void complete(const Req& r, cpvs_status st, const std::string& msg) {
        std::lock_guard<std::mutex> lock(mu);
        r->status = st;
        r->error = msg;
        r->t_done = Clock::now();
        r->state = kDone;
        if (st == CPVS_OK) {
            lat[r->kind].push_back(std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count());
            done_count[r->kind]++;
        } else if (st == CPVS_ERR_CANCELLED) {
            cancelled++;
        } else {
            failed++;
        }
        cv_done.notify_all();
    }

    void evict_to(uint64_t target) {
        while (resident_bytes > target) {
            auto victim = resident.end();
            for (auto it = resident.begin(); it != resident.end(); ++it)
                if (it->second.pins == 0 && (victim == resident.end() || it->second.last_use < victim->second.last_use))
                    victim = it;
            if (victim == resident.end()) return;  // everything pinned
            resident_bytes -= victim->second.bytes;
            cpvs_shadow_destroy(victim->second.sh);
            resident.erase(victim);
            std::lock_guard<std::mutex> lock(mu);
            evictions++;
        }
    }

    void retire_finished(bool wait_all) {
        while (!inflight.empty()) {
            InFlight& f = inflight.front();
            if (wait_all) cudaEventSynchronize(f.done);
            const cudaError_t q = cudaEventQuery(f.done);
            if (q == cudaErrorNotReady) return;
            const cpvs_status st = (q == cudaSuccess) ? CPVS_OK : CPVS_ERR_DEVICE;
            const std::string msg = (q == cudaSuccess) ? "" : cudaGetErrorString(q);
            cudaGetLastError();
            for (uint64_t k : f.keys) {
                auto it = resident.find(k);
                if (it != resident.end()) it->second.pins--;
            }
            for (cpvs_shadow* sh : f.retired) cpvs_shadow_destroy(sh);
            if (f.scratch) ctx->c.release(f.scratch, f.scratch_bytes, false, s_lookup);
            cudaEventDestroy(f.done);
            for (const Req& r : f.reqs) complete(r, st, msg);
            inflight.pop_front();
        }
    }

    // One segmented launch for every runnable lookup.
    void launch_lookups(std::vector<Req>& pending, const std::unordered_map<uint64_t, int>& building) {
        std::vector<Req> run, keep;
        for (const Req& r : pending) {
            if (r->state.load() == kDone) continue;  // cancelled while waiting here
            if (resident.count(r->key)) {
                if (run.size() < cfg.max_batch_lookups && r->claim()) run.push_back(r);
                else if (r->state.load() == kQueued) keep.push_back(r);
            } else if (building.count(r->key)) {
                keep.push_back(r);
            } else if (r->claim()) {
                complete(r, CPVS_ERR_INVALID_ARG, "lookup: key " + std::to_string(r->key) + " is not resident");
            }
        }
        pending.swap(keep);
        if (run.empty()) return;
        // device tables: distinct DAGs, then one segment per request
        std::vector<cpvs::MultiDag> dags;
        std::unordered_map<uint64_t, uint32_t> dag_of;
        std::vector<cpvs::LookupSegment> segs;
        uint64_t words = 0;
        InFlight f;
        for (const Req& r : run) {
            auto [it, fresh] = dag_of.try_emplace(r->key, (uint32_t)dags.size());
            if (fresh) {
                Resident& res = resident[r->key];
                dags.push_back(cpvs::MultiDag{res.sh->dag, (uint32_t)res.sh->words, res.sh->num_levels,
                                              res.sh->leafmasks ? 1u : 0u, 0u});
                res.pins++;
                res.last_use = ++tick;
                f.keys.push_back(r->key);
            }
            const float* q = static_cast<const float*>(cpvs::host_accessible(ctx->c, r->xyz));
            uint32_t* b = static_cast<uint32_t*>(cpvs::host_accessible(ctx->c, r->bits));
            if (!q || !b) {
                // the server reads points and writes bits in place
                complete(r, CPVS_ERR_INVALID_ARG, "lookup: host buffers must be GPU-accessible (pinned, or any "
                                                  "host memory on hosts where the GPU reads pageable memory)");
                continue;
            }
            segs.push_back(cpvs::LookupSegment{q, b, words, r->count, it->second, 0u});
            words += (r->count + 31) / 32;
            f.reqs.push_back(r);
        }
        if (f.reqs.empty()) {
            for (uint64_t k : f.keys) resident[k].pins--;
            return;
        }
        const uint64_t db = dags.size() * sizeof(cpvs::MultiDag), sb = segs.size() * sizeof(cpvs::LookupSegment);
        f.scratch_bytes = db + sb + 256;
        cpvs_status st = ctx->c.alloc(&f.scratch, f.scratch_bytes, false, s_lookup);
        cudaError_t e = cudaSuccess;
        char* base = static_cast<char*>(f.scratch);
        if (st == CPVS_OK) {
            e = cudaMemcpyAsync(base, dags.data(), db, cudaMemcpyHostToDevice, s_lookup);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(base + ((db + 255) & ~(uint64_t)255), segs.data(), sb, cudaMemcpyHostToDevice, s_lookup);
            if (e == cudaSuccess)
                st = cpvs::launch_segment_lookup(reinterpret_cast<const cpvs::MultiDag*>(base), (uint32_t)dags.size(),
                                                 reinterpret_cast<const cpvs::LookupSegment*>(base + ((db + 255) & ~(uint64_t)255)),
                                                 (uint32_t)segs.size(), words, s_lookup, &ctx->c.timing);
        }
        if (st == CPVS_OK && e == cudaSuccess) e = cudaEventCreateWithFlags(&f.done, cudaEventDisableTiming);
        if (st == CPVS_OK && e == cudaSuccess) e = cudaEventRecord(f.done, s_lookup);
        if (st != CPVS_OK || e != cudaSuccess) {
            const std::string msg = e != cudaSuccess ? cudaGetErrorString(e) : cpvs_last_error();
            cudaGetLastError();
            for (uint64_t k : f.keys) resident[k].pins--;
            if (f.scratch) ctx->c.release(f.scratch, f.scratch_bytes, false, s_lookup);
            if (f.done) cudaEventDestroy(f.done);
            for (const Req& r : f.reqs) complete(r, st != CPVS_OK ? st : CPVS_ERR_DEVICE, msg);
            return;
        }
        inflight.push_back(std::move(f));
    }

    // The pending builds as one batch.
    void run_builds(std::vector<Req>& builds) {
        if (builds.empty()) return;
        std::vector<Req> batch, rest;
        for (const Req& r : builds) {
            if (r->state.load() == kDone) continue;  // cancelled while waiting here
            if (batch.size() < cfg.max_batch_builds && r->claim()) batch.push_back(r);
            else if (r->state.load() == kQueued) rest.push_back(r);
        }
        builds.swap(rest);
        if (batch.empty()) return;
        // admission: room for the new DAGs (estimated at n^2/4 bytes each)
        uint64_t estimate = 0;
        for (const Req& r : batch) estimate += (uint64_t)r->n * r->n / 4;
        if (cfg.budget_bytes) evict_to(cfg.budget_bytes > estimate ? cfg.budget_bytes - estimate : 0);
        std::vector<cpvs_hierarchy*> hs;
        std::vector<Req> ok;
        for (const Req& r : batch) {
            cpvs_hierarchy* h = nullptr;
            cpvs_status st = cpvs_hierarchy_create(ctx, r->depth, r->n, 0, s_build, &h);
            if (st != CPVS_OK) {
                complete(r, st, cpvs_last_error());
                continue;
            }
            hs.push_back(h);
            ok.push_back(r);
        }
        if (ok.empty()) return;
        std::vector<cpvs_build_job> jobs(ok.size());
        for (size_t i = 0; i < ok.size(); ++i) jobs[i] = cpvs_build_job{(uint32_t)i, 0u, 1u};
        std::vector<cpvs_shadow*> out(ok.size(), nullptr);
        cpvs_status st = cpvs_shadow_create_batch(ctx, hs.data(), (uint32_t)hs.size(), jobs.data(),
                                                  (uint32_t)jobs.size(), cfg.flags, s_build, out.data());
        const std::string msg = st == CPVS_OK ? "" : cpvs_last_error();
        for (cpvs_hierarchy* h : hs) cpvs_hierarchy_destroy(h);
        if (st != CPVS_OK) {
            for (const Req& r : ok) complete(r, st, msg);
            return;
        }
        // the lookup stream must see the new DAGs: order it after the build
        cudaEvent_t built = nullptr;
        if (cudaEventCreateWithFlags(&built, cudaEventDisableTiming) == cudaSuccess) {
            cudaEventRecord(built, s_build);
            cudaStreamWaitEvent(s_lookup, built, 0);
            cudaEventDestroy(built);
        }
        for (size_t i = 0; i < ok.size(); ++i) {
            const Req& r = ok[i];
            const uint64_t bytes = out[i]->words * 4;
            if (cfg.budget_bytes && bytes > cfg.budget_bytes) {
                cpvs_shadow_destroy(out[i]);
                complete(r, CPVS_ERR_BUDGET, "build: the DAG alone exceeds the server's budget");
                continue;
            }
            auto it = resident.find(r->key);
            if (it != resident.end()) {
                // replaced: a pinned old DAG dies with the launch that reads it
                resident_bytes -= it->second.bytes;
                if (it->second.pins) {
                    for (InFlight& fl : inflight)
                        if (std::find(fl.keys.begin(), fl.keys.end(), r->key) != fl.keys.end()) {
                            fl.retired.push_back(it->second.sh);
                            fl.keys.erase(std::find(fl.keys.begin(), fl.keys.end(), r->key));
                            break;
                        }
                } else {
                    cpvs_shadow_destroy(it->second.sh);
                }
                resident.erase(it);
            }
            Resident res;
            res.sh = out[i];
            res.bytes = bytes;
            res.last_use = ++tick;
            resident[r->key] = res;
            resident_bytes += bytes;
            complete(r, CPVS_OK, "");
        }
        if (cfg.budget_bytes) evict_to(cfg.budget_bytes);
    }

    void loop() {
        cudaSetDevice(ctx->c.device);
        std::vector<Req> lookups, builds;
        for (;;) {
            {
                std::unique_lock<std::mutex> lock(mu);
                const bool busy = !inflight.empty() || !lookups.empty() || !builds.empty();
                if (busy)
                    cv_work.wait_for(lock, std::chrono::microseconds(50), [&] { return stop || !queue.empty(); });
                else
                    cv_work.wait(lock, [&] { return stop || !queue.empty(); });
                while (!queue.empty()) {
                    Req r = queue.front();
                    queue.pop_front();
                    if (r->state == kDone) continue;  // cancelled while queued
                    (r->kind == kBuild ? builds : lookups).push_back(r);
                }
                if (stop) break;
            }
            retire_finished(false);
            std::unordered_map<uint64_t, int> building;
            for (const Req& r : builds) building[r->key]++;
            launch_lookups(lookups, building);
            run_builds(builds);
            {
                std::lock_guard<std::mutex> lock(mu);
                stat_resident_dags = resident.size();
                stat_resident_bytes = resident_bytes;
            }
        }
        // shutdown: finish what runs, cancel what waits
        retire_finished(true);
        for (const Req& r : lookups)
            if (r->claim()) complete(r, CPVS_ERR_CANCELLED, "server stopped");
        for (const Req& r : builds)
            if (r->claim()) complete(r, CPVS_ERR_CANCELLED, "server stopped");
        for (auto& kv : resident) cpvs_shadow_destroy(kv.second.sh);
        resident.clear();
        cudaStreamSynchronize(s_build);
        cudaStreamSynchronize(s_lookup);
    }
};

extern "C" {

cpvs_status cpvs_server_create(cpvs_ctx* ctx, const cpvs_server_config* cfg, cpvs_server** out) {
    if (!ctx || !out) return fail(CPVS_ERR_INVALID_ARG, "server_create: null argument");
    *out = nullptr;
    CPVS_CUDA(cudaSetDevice(ctx->c.device));
    auto* s = new cpvs_server;
    s->ctx = ctx;
    if (cfg) s->cfg = *cfg;
    if (!s->cfg.max_batch_builds) s->cfg.max_batch_builds = 16;
    if (!s->cfg.max_batch_lookups) s->cfg.max_batch_lookups = 256;
    if (cudaStreamCreateWithFlags(&s->s_build, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&s->s_lookup, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        if (s->s_build) cudaStreamDestroy(s->s_build);
        delete s;
        return fail(CPVS_ERR_DEVICE, "server_create: stream creation failed");
    }
    s->worker = std::thread([s] { s->loop(); });
    *out = s;
    return CPVS_OK;
}

void cpvs_server_destroy(cpvs_server* s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        s->stop = true;
        for (Req& r : s->queue) {
            int q = kQueued;
            if (r->state.compare_exchange_strong(q, kDone)) {
                r->status = CPVS_ERR_CANCELLED;
                r->error = "server stopped";
                r->t_done = Clock::now();
                s->cancelled++;
            }
        }
        s->queue.clear();
        s->cv_done.notify_all();
    }
    s->cv_work.notify_all();
    if (s->worker.joinable()) s->worker.join();
    cudaSetDevice(s->ctx->c.device);
    cudaStreamDestroy(s->s_build);
    cudaStreamDestroy(s->s_lookup);
    delete s;
}

static cpvs_status submit(cpvs_server* s, const Req& r, uint64_t* ticket) {
    std::lock_guard<std::mutex> lock(s->mu);
    if (s->stop) return fail(CPVS_ERR_CANCELLED, "server stopped");
    r->ticket = s->next_ticket++;
    r->t_submit = Clock::now();
    s->tickets[r->ticket] = r;
    s->queue.push_back(r);
    if (ticket) *ticket = r->ticket;
    s->cv_work.notify_one();
    return CPVS_OK;
}

cpvs_status cpvs_server_submit_build(cpvs_server* s, uint64_t key, const float* depth, uint32_t n, uint64_t* ticket) {
    if (!s || !depth) return fail(CPVS_ERR_INVALID_ARG, "submit_build: null argument");
    if (n < 8 || n > 65536 || (n & (n - 1))) return fail(CPVS_ERR_INVALID_ARG, "submit_build: bad map size");
    auto r = std::make_shared<Request>();
    r->kind = kBuild;
    r->key = key;
    r->depth = depth;
    r->n = n;
    return submit(s, r, ticket);
}

cpvs_status cpvs_server_submit_lookup(cpvs_server* s, uint64_t key, const float* xyz, uint64_t n, uint32_t* bits_out,
                                      uint64_t* ticket) {
    if (!s || (n && (!xyz || !bits_out))) return fail(CPVS_ERR_INVALID_ARG, "submit_lookup: null argument");
    auto r = std::make_shared<Request>();
    r->kind = kLookup;
    r->key = key;
    r->xyz = xyz;
    r->count = n;
    r->bits = bits_out;
    return submit(s, r, ticket);
}

cpvs_status cpvs_server_wait(cpvs_server* s, uint64_t ticket, int64_t timeout_us, double* latency_ms) {
    if (!s) return fail(CPVS_ERR_INVALID_ARG, "server_wait: null server");
    std::unique_lock<std::mutex> lock(s->mu);
    auto it = s->tickets.find(ticket);
    if (it == s->tickets.end()) return fail(CPVS_ERR_INVALID_ARG, "server_wait: unknown ticket");
    Req r = it->second;
    auto ready = [&] { return r->state.load() == kDone; };
    if (timeout_us < 0)
        s->cv_done.wait(lock, ready);
    else if (!s->cv_done.wait_for(lock, std::chrono::microseconds(timeout_us), ready))
        return fail(CPVS_ERR_TIMEOUT, "server_wait: not done yet");
    s->tickets.erase(ticket);
    if (latency_ms) *latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
    if (r->status != CPVS_OK) return fail(r->status, r->error);
    return CPVS_OK;
}

cpvs_status cpvs_server_cancel(cpvs_server* s, uint64_t ticket) {
    if (!s) return fail(CPVS_ERR_INVALID_ARG, "server_cancel: null server");
    std::lock_guard<std::mutex> lock(s->mu);
    auto it = s->tickets.find(ticket);
    if (it == s->tickets.end()) return fail(CPVS_ERR_INVALID_ARG, "server_cancel: unknown ticket");
    Request& r = *it->second;
    r.status = CPVS_ERR_CANCELLED;  // only read once the state says done
    r.error = "cancelled";
    r.t_done = Clock::now();
    int q = kQueued;
    if (!r.state.compare_exchange_strong(q, kDone)) {
        r.status = CPVS_OK;
        r.error.clear();
        return fail(CPVS_ERR_INVALID_ARG, "server_cancel: already running or done");
    }
    s->cancelled++;
    s->cv_done.notify_all();
    return CPVS_OK;
}

cpvs_status cpvs_server_get_stats(cpvs_server* s, cpvs_server_stats* out) {
    if (!s || !out) return fail(CPVS_ERR_INVALID_ARG, "server_stats: null argument");
    std::lock_guard<std::mutex> lock(s->mu);
    out->builds_done = s->done_count[kBuild];
    out->lookups_done = s->done_count[kLookup];
    out->failed = s->failed;
    out->cancelled = s->cancelled;
    out->evictions = s->evictions;
    out->resident_dags = s->stat_resident_dags;
    out->resident_bytes = s->stat_resident_bytes;
    out->queued = s->queue.size();
    out->build_p50_ms = pct(s->lat[kBuild], 0.50);
    out->build_p99_ms = pct(s->lat[kBuild], 0.99);
    out->lookup_p50_ms = pct(s->lat[kLookup], 0.50);
    out->lookup_p99_ms = pct(s->lat[kLookup], 0.99);
    return CPVS_OK;
}

}  // extern "C"
