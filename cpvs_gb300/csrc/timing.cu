// Per-kernel CUDA-event timing of a context (off unless enabled): an event
// pair on the launching stream around each launch, resolved on demand.
#include "common.cuh"

namespace cpvs {

const char* kernel_name(int id) {
    static const char* names[K_COUNT] = {
        "k_pyramid64",      "k_level_bounds", "k_expand_count", "k_expand",      "k_leaf_columns",
        "k_classify_bottom", "table_clear",    "k_leaf_resolve", "k_dedup_insert", "k_dedup_resolve",
        "k_merge_scan",      "k_dedup_remap",  "k_layout",       "k_emit_all",     "k_lookup",
        "k_grid_lookup",     "k_raster",       "k_multi_lookup", "k_grid_evaluate", "k_shade",
        "k_leaf_classes", "k_top_index"};
    return (id >= 0 && id < K_COUNT) ? names[id] : "";
}

cudaEvent_t Timing::get() {
    if (!free_events.empty()) {
        cudaEvent_t e = free_events.back();
        free_events.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

void Timing::collect() {
    for (const Pending& p : pending) {
        float t = 0.f;
        if (cudaEventSynchronize(p.b) == cudaSuccess && cudaEventElapsedTime(&t, p.a, p.b) == cudaSuccess) {
            ms[p.id] += t;
            launches[p.id] += 1;
        }
        cudaGetLastError();
        free_events.push_back(p.a);
        free_events.push_back(p.b);
    }
    pending.clear();
}

void Timing::reset() {
    collect();
    for (int i = 0; i < K_COUNT; ++i) {
        ms[i] = 0.0;
        launches[i] = 0;
    }
}

Timing::~Timing() {
    for (const Pending& p : pending) {
        cudaEventDestroy(p.a);
        cudaEventDestroy(p.b);
    }
    for (cudaEvent_t e : free_events) cudaEventDestroy(e);
}

KernelTimer::KernelTimer(Timing* timing, int kid, cudaStream_t s) : t(timing), id(kid), st(s) {
    if (t && t->on) {
        a = t->get();
        cudaEventRecord(a, st);
    }
}

KernelTimer::~KernelTimer() {
    if (a) {
        cudaEvent_t b = t->get();
        cudaEventRecord(b, st);
        t->pending.push_back(Timing::Pending{id, a, b});
    }
}

}  // namespace cpvs
