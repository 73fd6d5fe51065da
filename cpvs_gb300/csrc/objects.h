// Handle types behind the C ABI, shared by the translation units that
// implement it (capi.cu, server.cu).
#pragma once

#include <vector>

#include "common.cuh"

struct cpvs_ctx {
    cpvs::Ctx c;
};

// Every object with device memory records `last_use` on the stream of each
// call that enqueues work on it; its memory is freed after that event.
struct DeviceObject {
    cudaEvent_t last_use = nullptr;
    DeviceObject() { cudaEventCreateWithFlags(&last_use, cudaEventDisableTiming); }
    ~DeviceObject() {
        if (last_use) cudaEventDestroy(last_use);
    }
    void touch(cudaStream_t st) const { cudaEventRecord(last_use, st); }
};

struct cpvs_hierarchy : DeviceObject {
    cpvs_ctx* ctx = nullptr;
    uint32_t n = 0;
    float* depth = nullptr;    // device n*n
    bool owns_depth = true;    // false when borrowed from the caller
    float2* levels = nullptr;  // device pyramid
    int first_level = 1;       // lowest pyramid level stored (a build's temporary hierarchy may skip some)
    uint64_t bytes = 0;
};

// Device block holding the DAGs of one build (one or many jobs back to
// back, followed by kDagPad zeroed words).  Shared by the shadows (and the
// grid) that point into it; freed when the last of them lets go, after every
// holder's last use.
struct DagBlock {
    cpvs_ctx* ctx = nullptr;
    uint32_t* base = nullptr;
    uint64_t bytes = 0;
    int refs = 0;
};

inline void block_unref(DagBlock* b, cudaEvent_t last_use) {
    if (!b) return;
    cpvs::Ctx& c = b->ctx->c;
    if (last_use) cudaStreamWaitEvent(c.free_stream, last_use, 0);  // the free waits for every holder
    if (--b->refs == 0) {
        c.release(b->base, b->bytes, true, nullptr, nullptr);
        delete b;
    }
}

struct cpvs_shadow : DeviceObject {
    cpvs_ctx* ctx = nullptr;
    DagBlock* block = nullptr;
    uint32_t* dag = nullptr;   // inside block; at least kDagPad readable words follow it
    uint64_t words = 0;
    uint32_t* top = nullptr;   // dense top index for lookups, built on the first lookup
    uint64_t top_bytes = 0;
    int top_depth = 0;         // levels below the root that `top` resolves
    uint32_t num_levels = 0;
    bool leafmasks = false;
    uint32_t root_mask = 0;
    std::vector<uint64_t> tree, uniq;
    const cpvs_grid* owner = nullptr;  // the grid whose cell holds it (and destroys it)
};

struct cpvs_grid : DeviceObject {
    cpvs_ctx* ctx = nullptr;
    uint32_t length = 0;
    std::vector<cpvs_shadow*> cells;
    DagBlock* block = nullptr;  // the combined DAG
    uint32_t* dag = nullptr;
    uint64_t words = 0;
    uint32_t* cell_words = nullptr;
    uint32_t dag_levels = 0;
    bool leafmasks = false;
    bool finalized = false;
    uint32_t filter_size = 1;  // PCF footprint of evaluate
    uint32_t* gtop = nullptr;  // grid top index, built on the first lookup
    uint64_t gtop_bytes = 0;   // ~0: none (too small, or its allocation failed)
    int gtop_depth = 0;
};


namespace cpvs {
// The address under which the GPU reads host memory `p` in place, or null.
void* host_accessible(const Ctx& c, const void* p);
// Builds the shadow's lookup top grid if it has none yet (stream-ordered,
// on the context's thread).
void shadow_ensure_top(const cpvs_shadow* s, cudaStream_t st, uint32_t max_factor);
// The shadow as an entry of a multi-DAG lookup table (with its top grid).
MultiDag shadow_table_entry(const cpvs_shadow* s);
// A hierarchy that only feeds builds with the given flags (destroyed after
// them): with leafmasks, pyramid levels 1 and 2 are not stored.  With
// `host_read`, a host map read in place is not waited for: the event
// recorded after the read is returned, and the caller waits for it before
// its own caller may reuse the map.
cpvs_status hierarchy_create_for_build(cpvs_ctx* ctx, const float* depth, uint32_t n, uint32_t flags,
                                       uint32_t build_flags, void* stream, cpvs_hierarchy** out,
                                       cudaEvent_t* host_read = nullptr);
}  // namespace cpvs
