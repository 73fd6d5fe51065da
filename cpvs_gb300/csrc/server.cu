// Serving loop: builds and lookup batches of different sizes arrive at any
// time from any host thread; DAGs stay resident in HBM under a byte budget.
//
// The reference has no serving layer (its app precomputes one shadow and
// evaluates it every frame, src/main.cpp:236-268).  Here two threads share
// the device:
//   * the dispatcher takes submissions, launches ALL pending lookups whose
//     DAG is resident as one segmented multi-DAG kernel on the lookup stream
//     (each request reads its points and writes its bits where they lie; the
//     launch tables go through a ring of pinned/device slots owned by the
//     server) and retires finished launches by event polling.  It never
//     waits for a build, so lookups keep flowing while one runs;
//   * the builder owns the context: it builds the pending maps of one side
//     as one batch (one plan, one graph launch) on the build stream, makes
//     the lookup stream wait for the new DAGs, publishes them, and evicts
//     least-recently-used DAGs that no in-flight lookup pins while the
//     resident bytes exceed the budget (a DAG alone above the budget fails
//     with CPVS_ERR_BUDGET).
// Order: every build of a key gets the next generation of that key; a lookup
// needs the generation that was current when it was submitted (or a newer
// one).  It waits while that build is pending and fails
// (CPVS_ERR_INVALID_ARG) once the build has failed, was cancelled, or its
// DAG was evicted, and for a key that was never built.  Every request's
// answer is the one the plain API gives for it alone.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
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
constexpr uint32_t kRingSlots = 32;  // lookup launches in flight at most

struct Request {
    uint64_t ticket = 0;
    Kind kind = kBuild;
    uint64_t key = 0;
    uint64_t gen = 0;              // build: its generation; lookup: the one it needs
    const float* depth = nullptr;  // build
    uint32_t n = 0;
    const float* xyz = nullptr;  // lookup
    uint64_t count = 0;
    uint32_t* bits = nullptr;
    std::atomic<int> state{kQueued};  // kQueued -> kRunning (a server thread) | kDone (cancel); kRunning -> kDone
    bool claim() {  // take a queued request; false when it was cancelled
        int q = kQueued;
        return state.compare_exchange_strong(q, kRunning);
    }
    cpvs_status status = CPVS_OK;
    std::string error;
    Clock::time_point t_submit, t_done;
};
using Req = std::shared_ptr<Request>;

// A resident DAG.  In-flight lookups pin it; one that is replaced or evicted
// while pinned is destroyed by the builder once the last pin goes.
struct Entry {
    cpvs_shadow* sh = nullptr;
    uint64_t bytes = 0;
    uint64_t gen = 0;
    uint64_t last_use = 0;  // LRU tick
    int pins = 0;
    bool dropped = false;  // no longer resident
};
using EntryP = std::shared_ptr<Entry>;

struct InFlight {
    cudaEvent_t done = nullptr;
    std::vector<Req> reqs;
    std::vector<EntryP> pinned;
};

double pct(std::vector<double> v, double p) {
    if (v.empty()) return 0.0;
    std::sort(v.begin(), v.end());
    const size_t i = (size_t)std::min<double>(v.size() - 1, std::max(0.0, p * (v.size() - 1) + 0.5));
    return v[i];
}

uint64_t align256(uint64_t x) { return (x + 255) & ~(uint64_t)255; }

}  // namespace

struct cpvs_server {
    cpvs_ctx* ctx = nullptr;
    cpvs_server_config cfg{};
    std::mutex mu;  // everything below that is not marked as one thread's own
    std::condition_variable cv_work, cv_build, cv_done;
    std::deque<Req> queue;
    std::unordered_map<uint64_t, Req> tickets;
    uint64_t next_ticket = 1;
    bool stop = false;
    bool wake = false;  // a build finished: waiting lookups may now run or fail
    std::thread dispatcher, builder;
    std::vector<Req> builds_pending;
    std::unordered_map<uint64_t, EntryP> resident;
    uint64_t resident_bytes = 0, tick = 0;
    uint64_t dag_bytes_seen[17] = {0};  // largest DAG built so far per log2 map side (admission estimate)
    std::unordered_map<uint64_t, uint64_t> gen_submitted, gen_done;
    std::vector<cpvs_shadow*> graveyard;  // unpinned after being dropped: the builder destroys them
    std::vector<double> lat[2];
    uint64_t done_count[2] = {0, 0}, failed = 0, cancelled = 0, evictions = 0;
    // streams and the lookup table ring (allocated before the threads start)
    cudaStream_t s_build = nullptr, s_lookup = nullptr;
    uint64_t slot_bytes = 0, dag_table_bytes = 0;
    char* ring_dev = nullptr;
    char* ring_host = nullptr;
    uint64_t ring_bytes = 0;
    // dispatcher's own
    std::vector<Req> lookups_pending;
    std::deque<InFlight> inflight;
    uint32_t ring_next = 0;

    // ------------------------------------------------------------ common
    void complete_locked(const Req& r, cpvs_status st, const std::string& msg) {
        r->status = st;
        r->error = msg;
        r->t_done = Clock::now();
        r->state = kDone;
        if (r->kind == kBuild) {
            uint64_t& g = gen_done[r->key];
            g = std::max(g, r->gen);
            wake = true;
        }
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
    void complete(const Req& r, cpvs_status st, const std::string& msg) {
        {
            std::lock_guard<std::mutex> lock(mu);
            complete_locked(r, st, msg);
        }
        if (r->kind == kBuild) cv_work.notify_one();
    }
    // Takes `e` out of the resident set; returns its shadow when it can be
    // destroyed now (unpinned), else leaves that to the last unpin.
    cpvs_shadow* drop_locked(const EntryP& e) {
        e->dropped = true;
        resident_bytes -= e->bytes;
        return e->pins == 0 ? e->sh : nullptr;
    }
    void unpin_locked(const EntryP& e) {
        if (--e->pins == 0 && e->dropped) {
            graveyard.push_back(e->sh);
            cv_build.notify_one();
        }
    }

    // -------------------------------------------------------- dispatcher
    void retire_finished(bool wait_front) {
        while (!inflight.empty()) {
            InFlight& f = inflight.front();
            if (wait_front) {
                cudaEventSynchronize(f.done);
                wait_front = false;
            }
            const cudaError_t q = cudaEventQuery(f.done);
            if (q == cudaErrorNotReady) return;
            const cpvs_status st = (q == cudaSuccess) ? CPVS_OK : CPVS_ERR_DEVICE;
            const std::string msg = (q == cudaSuccess) ? "" : cudaGetErrorString(q);
            cudaGetLastError();
            cudaEventDestroy(f.done);
            {
                std::lock_guard<std::mutex> lock(mu);
                for (const EntryP& e : f.pinned) unpin_locked(e);
                for (const Req& r : f.reqs) complete_locked(r, st, msg);
            }
            inflight.pop_front();
        }
    }

    // One segmented launch for every runnable lookup (up to max_batch_lookups).
    void launch_lookups() {
        cpvs::NvtxRange range("cpvs server: lookup launch");
        if (lookups_pending.empty()) return;
        if (inflight.size() >= kRingSlots) retire_finished(true);  // frees the oldest slot
        std::vector<Req> run, keep;
        std::vector<EntryP> run_entry;
        std::vector<std::pair<Req, std::string>> rejected;
        {
            std::lock_guard<std::mutex> lock(mu);
            for (const Req& r : lookups_pending) {
                if (r->state.load() == kDone) continue;  // cancelled while waiting here
                auto it = resident.find(r->key);
                if (it != resident.end() && it->second->gen >= r->gen) {
                    if (run.size() < cfg.max_batch_lookups && r->claim()) {
                        run.push_back(r);
                        run_entry.push_back(it->second);
                        it->second->pins++;
                        it->second->last_use = ++tick;
                    } else if (r->state.load() == kQueued) {
                        keep.push_back(r);
                    }
                    continue;
                }
                auto gd = gen_done.find(r->key);
                const uint64_t done = gd == gen_done.end() ? 0 : gd->second;
                if (done >= r->gen) {
                    if (r->claim()) {
                        const char* why = r->gen == 0 ? " was never built" : " is not resident (evicted, failed or cancelled)";
                        rejected.emplace_back(r, "lookup: key " + std::to_string(r->key) + why);
                    }
                } else {
                    keep.push_back(r);  // its build is pending
                }
            }
        }
        lookups_pending.swap(keep);
        for (auto& [r, msg] : rejected) complete(r, CPVS_ERR_INVALID_ARG, msg);
        if (run.empty()) return;
        // launch tables in this slot: distinct DAGs, then one segment per request
        const uint32_t slot = ring_next;
        char* hbase = ring_host + (uint64_t)slot * slot_bytes;
        char* dbase = ring_dev + (uint64_t)slot * slot_bytes;
        auto* hdags = reinterpret_cast<cpvs::MultiDag*>(hbase);
        auto* hsegs = reinterpret_cast<cpvs::LookupSegment*>(hbase + dag_table_bytes);
        std::unordered_map<const Entry*, uint32_t> dag_of;
        uint32_t ndags = 0, nsegs = 0;
        uint64_t words = 0;
        InFlight f;
        std::vector<std::pair<Req, std::string>> bad;
        for (size_t i = 0; i < run.size(); ++i) {
            const Req& r = run[i];
            const Entry* e = run_entry[i].get();
            const float* q = static_cast<const float*>(cpvs::host_accessible(ctx->c, r->xyz));
            uint32_t* b = static_cast<uint32_t*>(cpvs::host_accessible(ctx->c, r->bits));
            if (!q || !b) {
                // the server reads points and writes bits in place
                bad.emplace_back(r, "lookup: host buffers must be GPU-accessible (pinned, or any host memory on "
                                    "hosts where the GPU reads pageable memory)");
                continue;
            }
            auto [it, fresh] = dag_of.try_emplace(e, ndags);
            if (fresh) hdags[ndags++] = cpvs::shadow_table_entry(e->sh);
            hsegs[nsegs++] = cpvs::LookupSegment{q, b, words, r->count, it->second, 0u};
            words += (r->count + 31) / 32;
            f.reqs.push_back(r);
        }
        f.pinned = std::move(run_entry);
        cudaError_t e = cudaSuccess;
        cpvs_status st = CPVS_OK;
        if (!f.reqs.empty() && words == 0) {
            // only empty requests: nothing to launch
            std::lock_guard<std::mutex> lock(mu);
            for (const EntryP& p : f.pinned) unpin_locked(p);
            for (const Req& r : f.reqs) complete_locked(r, CPVS_OK, "");
            f.reqs.clear();
            f.pinned.clear();
        }
        if (!f.reqs.empty()) {
            e = cudaMemcpyAsync(dbase, hbase, dag_table_bytes + (uint64_t)nsegs * sizeof(cpvs::LookupSegment),
                                cudaMemcpyHostToDevice, s_lookup);
            if (e == cudaSuccess)
                st = cpvs::launch_segment_lookup(reinterpret_cast<const cpvs::MultiDag*>(dbase), ndags,
                                                 reinterpret_cast<const cpvs::LookupSegment*>(dbase + dag_table_bytes),
                                                 nsegs, words, s_lookup, nullptr);
            if (st == CPVS_OK && e == cudaSuccess) e = cudaEventCreateWithFlags(&f.done, cudaEventDisableTiming);
            if (st == CPVS_OK && e == cudaSuccess) e = cudaEventRecord(f.done, s_lookup);
        }
        if (!f.reqs.empty() && (st != CPVS_OK || e != cudaSuccess)) {
            const std::string msg = e != cudaSuccess ? cudaGetErrorString(e) : cpvs_last_error();
            cudaGetLastError();
            if (f.done) cudaEventDestroy(f.done);
            // the slot's copy may still be pending: wait before its reuse
            cudaStreamSynchronize(s_lookup);
            std::lock_guard<std::mutex> lock(mu);
            for (const EntryP& p : f.pinned) unpin_locked(p);
            for (const Req& r : f.reqs) complete_locked(r, st != CPVS_OK ? st : CPVS_ERR_DEVICE, msg);
            f.reqs.clear();
            f.pinned.clear();
        }
        if (!f.reqs.empty()) {
            inflight.push_back(std::move(f));
            ring_next = (ring_next + 1) % kRingSlots;
        } else if (!f.pinned.empty()) {
            std::lock_guard<std::mutex> lock(mu);
            for (const EntryP& p : f.pinned) unpin_locked(p);
        }
        for (auto& [r, msg] : bad) complete(r, CPVS_ERR_INVALID_ARG, msg);
    }

    void dispatch_loop() {
        cudaSetDevice(ctx->c.device);
        for (;;) {
            {
                std::unique_lock<std::mutex> lock(mu);
                // sleep only when no launch is in flight; waiting lookups are
                // woken by the builder
                if (inflight.empty())
                    cv_work.wait(lock, [&] { return stop || !queue.empty() || wake; });
                wake = false;
                bool new_builds = false;
                while (!queue.empty()) {
                    Req r = queue.front();
                    queue.pop_front();
                    if (r->state == kDone) continue;  // cancelled while queued
                    if (r->kind == kBuild) {
                        builds_pending.push_back(r);
                        new_builds = true;
                    } else {
                        lookups_pending.push_back(r);
                    }
                }
                if (new_builds) cv_build.notify_one();
                if (stop) break;
            }
            retire_finished(false);
            launch_lookups();
            if (!inflight.empty()) std::this_thread::yield();
        }
        // shutdown: finish what runs, cancel what waits
        while (!inflight.empty()) retire_finished(true);
        for (const Req& r : lookups_pending)
            if (r->claim()) complete(r, CPVS_ERR_CANCELLED, "server stopped");
        lookups_pending.clear();
    }

    // ----------------------------------------------------------- builder
    // Evicts unpinned least-recently-used DAGs until the resident bytes are
    // at most `target`; returns the shadows to destroy.
    std::vector<cpvs_shadow*> evict_locked(uint64_t target) {
        std::vector<cpvs_shadow*> out;
        while (resident_bytes > target) {
            auto victim = resident.end();
            for (auto it = resident.begin(); it != resident.end(); ++it)
                if (it->second->pins == 0 &&
                    (victim == resident.end() || it->second->last_use < victim->second->last_use))
                    victim = it;
            if (victim == resident.end()) break;  // everything pinned
            if (cpvs_shadow* sh = drop_locked(victim->second)) out.push_back(sh);
            resident.erase(victim);
            evictions++;
        }
        return out;
    }

    void build_batch(std::vector<Req>& batch) {
        cpvs::NvtxRange range("cpvs server: build batch");
        // admission: room for the new DAGs, each estimated at the largest
        // DAG built so far from a map of its side (n^2/4 bytes before any)
        if (cfg.budget_bytes) {
            uint64_t estimate = 0;
            for (const Req& r : batch) {
                const uint64_t seen = dag_bytes_seen[cpvs::log2_u32(r->n)];
                estimate += seen ? seen : (uint64_t)r->n * r->n / 4;
            }
            std::vector<cpvs_shadow*> dead;
            {
                std::lock_guard<std::mutex> lock(mu);
                dead = evict_locked(cfg.budget_bytes > estimate ? cfg.budget_bytes - estimate : 0);
            }
            for (cpvs_shadow* sh : dead) cpvs_shadow_destroy(sh);
        }
        std::vector<cpvs_hierarchy*> hs;
        std::vector<Req> ok;
        // each request keeps its map until it completes, so the pyramids'
        // reads of the maps are waited for once, after the batch build
        std::vector<cudaEvent_t> reads;
        for (const Req& r : batch) {
            cpvs_hierarchy* h = nullptr;
            cudaEvent_t read = nullptr;
            const cpvs_status st =
                cpvs::hierarchy_create_for_build(ctx, r->depth, r->n, 0, cfg.flags, s_build, &h, &read);
            if (st != CPVS_OK) {
                complete(r, st, cpvs_last_error());
                continue;
            }
            if (read) reads.push_back(read);
            hs.push_back(h);
            ok.push_back(r);
        }
        if (ok.empty()) return;
        std::vector<cpvs_build_job> jobs(ok.size());
        for (size_t i = 0; i < ok.size(); ++i) jobs[i] = cpvs_build_job{(uint32_t)i, 0u, 1u};
        std::vector<cpvs_shadow*> out(ok.size(), nullptr);
        const cpvs_status st = cpvs_shadow_create_batch(ctx, hs.data(), (uint32_t)hs.size(), jobs.data(),
                                                        (uint32_t)jobs.size(), cfg.flags, s_build, out.data());
        const std::string msg = st == CPVS_OK ? "" : cpvs_last_error();
        for (cudaEvent_t e : reads) {
            cudaEventSynchronize(e);
            cudaEventDestroy(e);
        }
        for (cpvs_hierarchy* h : hs) cpvs_hierarchy_destroy(h);
        if (st != CPVS_OK) {
            for (const Req& r : ok) complete(r, st, msg);
            return;
        }
        // their lookup top grids, then: lookups launched after the DAGs are
        // published run after all of it
        for (cpvs_shadow* sh : out) cpvs::shadow_ensure_top(sh, s_build, 1);
        cudaEvent_t built = nullptr;
        if (cudaEventCreateWithFlags(&built, cudaEventDisableTiming) == cudaSuccess) {
            cudaEventRecord(built, s_build);
            cudaStreamWaitEvent(s_lookup, built, 0);
            cudaEventDestroy(built);
        }
        std::vector<cpvs_shadow*> dead;
        {
            std::lock_guard<std::mutex> lock(mu);
            for (size_t i = 0; i < ok.size(); ++i) {
                const Req& r = ok[i];
                const uint64_t bytes = out[i]->words * 4;
                uint64_t& seen = dag_bytes_seen[cpvs::log2_u32(r->n)];
                if (bytes > seen) seen = bytes;
                if (cfg.budget_bytes && bytes > cfg.budget_bytes) {
                    dead.push_back(out[i]);
                    complete_locked(r, CPVS_ERR_BUDGET, "build: the DAG alone exceeds the server's budget");
                    continue;
                }
                auto it = resident.find(r->key);
                if (it != resident.end()) {
                    if (cpvs_shadow* sh = drop_locked(it->second)) dead.push_back(sh);
                    resident.erase(it);
                }
                auto e = std::make_shared<Entry>();
                e->sh = out[i];
                e->bytes = bytes;
                e->gen = r->gen;
                e->last_use = ++tick;
                resident[r->key] = e;
                resident_bytes += bytes;
                complete_locked(r, CPVS_OK, "");
            }
            if (cfg.budget_bytes) {
                std::vector<cpvs_shadow*> more = evict_locked(cfg.budget_bytes);
                dead.insert(dead.end(), more.begin(), more.end());
            }
        }
        cv_work.notify_one();
        for (cpvs_shadow* sh : dead) cpvs_shadow_destroy(sh);
    }

    void build_loop() {
        cudaSetDevice(ctx->c.device);
        for (;;) {
            std::vector<Req> batch;
            std::vector<cpvs_shadow*> dead;
            bool quit = false;
            {
                std::unique_lock<std::mutex> lock(mu);
                cv_build.wait(lock, [&] { return stop || !builds_pending.empty() || !graveyard.empty(); });
                dead.swap(graveyard);
                if (stop) {
                    quit = true;
                } else {
                    // one batch: the oldest pending build's map side, oldest first
                    std::vector<Req> rest;
                    uint32_t side = 0;
                    for (const Req& r : builds_pending) {
                        if (r->state.load() == kDone) continue;  // cancelled while pending
                        if (!side) side = r->n;
                        if (r->n == side && batch.size() < cfg.max_batch_builds && r->claim())
                            batch.push_back(r);
                        else if (r->state.load() == kQueued)
                            rest.push_back(r);
                    }
                    builds_pending.swap(rest);
                }
            }
            for (cpvs_shadow* sh : dead) cpvs_shadow_destroy(sh);
            if (quit) break;
            if (!batch.empty()) build_batch(batch);
        }
        std::vector<Req> left;
        {
            std::lock_guard<std::mutex> lock(mu);
            left.swap(builds_pending);
        }
        for (const Req& r : left)
            if (r->claim()) complete(r, CPVS_ERR_CANCELLED, "server stopped");
    }
};

extern "C" {

cpvs_status cpvs_server_create(cpvs_ctx* ctx, const cpvs_server_config* cfg, cpvs_server** out) {
    if (!ctx || !out) return fail(CPVS_ERR_INVALID_ARG, "server_create: null argument");
    *out = nullptr;
    CPVS_CUDA(cudaSetDevice(ctx->c.device));
    auto s = std::make_unique<cpvs_server>();
    s->ctx = ctx;
    // the server's builds keep the default launch shapes (or those the
    // context's options fix): timing candidates would stall the loop
    ctx->c.tune_builds = false;
    if (cfg) s->cfg = *cfg;
    if (!s->cfg.max_batch_builds) s->cfg.max_batch_builds = 16;
    if (!s->cfg.max_batch_lookups) s->cfg.max_batch_lookups = 256;
    if (s->cfg.max_batch_lookups > 65536) return fail(CPVS_ERR_INVALID_ARG, "server_create: max_batch_lookups > 65536");
    const uint64_t m = s->cfg.max_batch_lookups;
    s->dag_table_bytes = align256(m * sizeof(cpvs::MultiDag));
    s->slot_bytes = align256(s->dag_table_bytes + m * sizeof(cpvs::LookupSegment));
    s->ring_bytes = s->slot_bytes * kRingSlots;
    auto undo = [&](const char* what) {
        cudaGetLastError();
        if (s->ring_host) cudaFreeHost(s->ring_host);
        if (s->ring_dev) s->ctx->c.release(s->ring_dev, s->ring_bytes, true, nullptr);
        if (s->s_build) cudaStreamDestroy(s->s_build);
        if (s->s_lookup) cudaStreamDestroy(s->s_lookup);
        return fail(CPVS_ERR_DEVICE, std::string("server_create: ") + what);
    };
    // lookups are short and latency-bound: their CTAs go ahead of waiting
    // build CTAs
    int prio_low = 0, prio_high = 0;
    cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high);
    if (cudaStreamCreateWithPriority(&s->s_build, cudaStreamNonBlocking, prio_low) != cudaSuccess ||
        cudaStreamCreateWithPriority(&s->s_lookup, cudaStreamNonBlocking, prio_high) != cudaSuccess)
        return undo("stream creation failed");
    if (cudaMallocHost(&s->ring_host, s->ring_bytes) != cudaSuccess) return undo("pinned ring allocation failed");
    {
        void* p = nullptr;
        const cpvs_status st = ctx->c.alloc(&p, s->ring_bytes, true, s->s_lookup);
        if (st != CPVS_OK) {
            const std::string msg = cpvs_last_error();
            undo("ring allocation failed");
            return fail(st, msg);
        }
        s->ring_dev = static_cast<char*>(p);
    }
    cpvs_server* raw = s.release();
    raw->dispatcher = std::thread([raw] { raw->dispatch_loop(); });
    raw->builder = std::thread([raw] { raw->build_loop(); });
    *out = raw;
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
    s->cv_build.notify_all();
    if (s->dispatcher.joinable()) s->dispatcher.join();
    if (s->builder.joinable()) s->builder.join();
    cudaSetDevice(s->ctx->c.device);
    cudaStreamSynchronize(s->s_build);
    cudaStreamSynchronize(s->s_lookup);
    for (auto& kv : s->resident) cpvs_shadow_destroy(kv.second->sh);
    s->resident.clear();
    for (cpvs_shadow* sh : s->graveyard) cpvs_shadow_destroy(sh);
    s->graveyard.clear();
    s->ctx->c.release(s->ring_dev, s->ring_bytes, true, nullptr);
    cudaFreeHost(s->ring_host);
    cudaStreamDestroy(s->s_build);
    cudaStreamDestroy(s->s_lookup);
    delete s;
}

static cpvs_status submit(cpvs_server* s, const Req& r, uint64_t* ticket) {
    {
        std::lock_guard<std::mutex> lock(s->mu);
        if (s->stop) return fail(CPVS_ERR_CANCELLED, "server stopped");
        r->ticket = s->next_ticket++;
        r->t_submit = Clock::now();
        if (r->kind == kBuild) {
            r->gen = ++s->gen_submitted[r->key];
        } else {
            auto it = s->gen_submitted.find(r->key);
            r->gen = it == s->gen_submitted.end() ? 0 : it->second;
        }
        s->tickets[r->ticket] = r;
        s->queue.push_back(r);
        if (ticket) *ticket = r->ticket;
    }
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
    {
        std::lock_guard<std::mutex> lock(s->mu);
        auto it = s->tickets.find(ticket);
        if (it == s->tickets.end()) return fail(CPVS_ERR_INVALID_ARG, "server_cancel: unknown ticket");
        const Req r = it->second;
        int q = kQueued;
        if (!r->state.compare_exchange_strong(q, kRunning))
            return fail(CPVS_ERR_INVALID_ARG, "server_cancel: already running or done");
        s->complete_locked(r, CPVS_ERR_CANCELLED, "cancelled");
    }
    s->cv_work.notify_one();  // lookups waiting on a cancelled build now fail
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
    out->resident_dags = s->resident.size();
    out->resident_bytes = s->resident_bytes;
    out->queued = s->queue.size() + s->builds_pending.size();
    out->build_p50_ms = pct(s->lat[kBuild], 0.50);
    out->build_p99_ms = pct(s->lat[kBuild], 0.99);
    out->lookup_p50_ms = pct(s->lat[kLookup], 0.50);
    out->lookup_p99_ms = pct(s->lat[kLookup], 0.99);
    return CPVS_OK;
}

}  // extern "C"
