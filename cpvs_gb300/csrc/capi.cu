// C ABI of the library (include/cpvs.h): handles, validation, memory budget,
// host <-> device staging.  All compute is in pyramid.cu, build.cu,
// lookup.cu, raster.cu and shade.cu; nothing here computes a result on the
// host.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <functional>
#include <string>
#include <vector>

#include "common.cuh"

namespace cpvs {

static thread_local std::string g_last_error;

cpvs_status fail(cpvs_status s, const std::string& msg) {
    g_last_error = msg;
    return s;
}

cpvs_status cuda_fail(cudaError_t e, const char* what) {
    const cpvs_status s = (e == cudaErrorMemoryAllocation) ? CPVS_ERR_OOM : CPVS_ERR_DEVICE;
    cudaGetLastError();  // clear a non-sticky error
    return fail(s, std::string(what) + ": " + cudaGetErrorString(e));
}

cpvs_status Ctx::alloc(void** p, uint64_t bytes, bool persistent, cudaStream_t st) {
    *p = nullptr;
    if (budget && in_use + scratch + bytes > budget)
        return fail(CPVS_ERR_BUDGET, "allocation of " + std::to_string(bytes) + " bytes exceeds the context budget");
    cudaError_t e = cudaMallocFromPoolAsync(p, bytes, pool, st);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMallocFromPoolAsync");
    if (persistent)
        in_use += bytes;
    else
        scratch += bytes;
    return CPVS_OK;
}

void Ctx::release(void* p, uint64_t bytes, bool persistent, cudaStream_t st, cudaEvent_t last_use) {
    if (persistent) {
        if (p) {
            if (last_use) cudaStreamWaitEvent(free_stream, last_use, 0);
            cudaFreeAsync(p, free_stream);
        }
        in_use -= std::min(in_use, bytes);
    } else {
        if (p) cudaFreeAsync(p, st);
        scratch -= std::min(scratch, bytes);
    }
}

}  // namespace cpvs

using cpvs::fail;

namespace cpvs {
// The address under which the GPU reads host memory `p` in place, or null:
// pinned / registered memory through its mapped address, and, where the GPU
// walks the host page tables (Grace-class hosts), any host pointer.
void* host_accessible(const Ctx& c, const void* p) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type == cudaMemoryTypeHost && a.devicePointer) return a.devicePointer;
    if (a.type == cudaMemoryTypeUnregistered && c.pageable_access) return const_cast<void*>(p);
    return nullptr;
}

}  // namespace cpvs
using cpvs::host_accessible;

#include "objects.h"

namespace {

bool is_pow2(uint64_t v) { return v && !(v & (v - 1)); }

cpvs_status set_device(const cpvs_ctx* ctx) {
    cudaError_t e = cudaSetDevice(ctx->c.device);
    if (e != cudaSuccess) return cpvs::cuda_fail(e, "cudaSetDevice");
    return CPVS_OK;
}

// A hierarchy needs a square power-of-two map (src/MinMaxHierarchy.cpp:12-14);
// a DAG needs numLevels > 3, i.e. n >= 8 (src/CompressedShadow.cpp:46).
cpvs_status check_map_size(uint32_t n, uint32_t min_n) {
    if (!is_pow2(n) || n < min_n || n > 65536)
        return fail(CPVS_ERR_INVALID_ARG, "map side must be a power of two in [" + std::to_string(min_n) +
                                              ", 65536], got " + std::to_string(n));
    return CPVS_OK;
}

// Device view of a host or device input: used in place when the GPU can read
// it, else copied to scratch (`owned` then tells to free it).
cpvs_status stage_in(cpvs::Ctx& c, const void* src, uint64_t bytes, uint32_t flags, cudaStream_t st, void** dev,
                     bool* owned) {
    if (flags & CPVS_IO_DEVICE) {
        *dev = const_cast<void*>(src);
        *owned = false;
        return CPVS_OK;
    }
    if (void* in_place = host_accessible(c, src)) {
        *dev = in_place;
        *owned = false;
        return CPVS_OK;
    }
    cpvs_status r = c.alloc(dev, std::max<uint64_t>(bytes, 4), false, st);
    if (r != CPVS_OK) return r;
    *owned = true;
    if (bytes) CPVS_CUDA(cudaMemcpyAsync(*dev, src, bytes, cudaMemcpyHostToDevice, st));
    return CPVS_OK;
}

// Host or device input of `qbytes` and output of `obytes` around one launch:
// host buffers are read / written in place where the GPU can reach them,
// else staged through stream-ordered scratch.  Host output is complete on
// return.
cpvs_status io_common(cpvs_ctx* ctx, const void* in, uint64_t qbytes, void* out, uint64_t obytes, uint32_t flags,
                      cudaStream_t st, const std::function<cpvs_status(const void*, void*)>& run) {
    cpvs_status r = set_device(ctx);
    if (r != CPVS_OK) return r;
    cpvs::Ctx& c = ctx->c;
    void* q = nullptr;
    bool qowned = false;
    r = stage_in(c, in, qbytes, flags, st, &q, &qowned);
    if (r != CPVS_OK) return r;
    void* o = out;
    bool oowned = false, host_out = false;
    if (!(flags & CPVS_IO_DEVICE)) {
        host_out = true;
        o = host_accessible(c, out);
        if (!o) {
            r = c.alloc(&o, obytes, false, st);
            if (r != CPVS_OK) {
                if (qowned) c.release(q, qbytes, false, st);
                return r;
            }
            oowned = true;
        }
    }
    r = run(q, o);
    if (r == CPVS_OK && host_out) {
        cudaError_t e = oowned ? cudaMemcpyAsync(out, o, obytes, cudaMemcpyDeviceToHost, st) : cudaSuccess;
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) r = cpvs::cuda_fail(e, "lookup read-back");
    }
    if (qowned) c.release(q, std::max<uint64_t>(qbytes, 4), false, st);
    if (oowned) c.release(o, obytes, false, st);
    return r;
}

cpvs_status lookup_common(cpvs_ctx* ctx, const void* xyz, uint64_t n, uint32_t* bits_out, uint32_t flags,
                          cudaStream_t st, const std::function<cpvs_status(const void*, uint32_t*)>& run) {
    if (!xyz && n) return fail(CPVS_ERR_INVALID_ARG, "lookup: null input");
    if (!bits_out && n) return fail(CPVS_ERR_INVALID_ARG, "lookup: null output");
    if (n == 0) return CPVS_OK;
    if (n >= (1ull << 40)) return fail(CPVS_ERR_INVALID_ARG, "lookup: batch too large");
    return io_common(ctx, xyz, n * 12, bits_out, (n + 31) / 32 * 4, flags, st,
                     [&](const void* q, void* o) { return run(q, static_cast<uint32_t*>(o)); });
}

// Builds `jobs` in one batch and wraps each job's DAG in a shadow; all of
// them share one device block.  `total` receives the block's DAG words.
cpvs_status build_into_shadows(cpvs_ctx* ctx, const std::vector<cpvs::SourceSpec>& src,
                               const std::vector<cpvs::JobSpec>& jobs, bool leaf, cudaStream_t st, DagBlock** block_out,
                               std::vector<cpvs_shadow*>& out, std::vector<uint64_t>* offsets = nullptr,
                               uint64_t* total = nullptr) {
    cpvs::BuildOutput bo;
    cpvs_status r = cpvs::build_dags(ctx->c, src, jobs, leaf, st, bo);
    if (r != CPVS_OK) {
        if (bo.dag) {
            cudaStreamSynchronize(st);
            ctx->c.release(bo.dag, (bo.dag_words + cpvs::kDagPad) * 4, true, nullptr);
        }
        return r;
    }
    auto* b = new DagBlock{ctx, bo.dag, (bo.dag_words + cpvs::kDagPad) * 4, 0};
    for (size_t j = 0; j < jobs.size(); ++j) {
        auto* s = new cpvs_shadow;
        s->ctx = ctx;
        s->block = b;
        b->refs++;
        s->dag = bo.dag + bo.job_offset[j];
        s->words = bo.job_words[j];
        s->num_levels = (uint32_t)cpvs::log2_u32(src[jobs[j].source].n) + 1;
        s->leafmasks = leaf;
        s->root_mask = bo.root_mask[j];
        s->tree = bo.tree_nodes[j];
        s->uniq = bo.unique_nodes[j];
        s->touch(st);
        out.push_back(s);
    }
    if (offsets) *offsets = bo.job_offset;
    if (total) *total = bo.dag_words;
    *block_out = b;
    return CPVS_OK;
}

// The shadow's top index, built on its first lookup (stream-ordered), at
// most max_factor times the DAG's size: a lookup of its own affords 8x (one
// more level resolved by one load), a server that keeps many DAGs resident
// under a budget 1x.
constexpr uint32_t kTopFactor = 8;
void ensure_top(const cpvs_shadow* cs, cudaStream_t st, uint32_t max_factor = kTopFactor) {
    cpvs_shadow* s = const_cast<cpvs_shadow*>(cs);
    if (s->top || s->top_bytes == ~0ull) return;
    const int depth = cpvs::top_index_depth(s->num_levels, s->leafmasks, s->words, max_factor);
    cpvs::KernelTimer kt(&s->ctx->c.timing, cpvs::K_TOP_INDEX, st);
    if (depth <= 0 || s->ctx->c.alloc((void**)&s->top, uint64_t(4) << (3 * depth), true, st) != CPVS_OK ||
        cpvs::launch_top_index(s->dag, s->words, depth, s->top, st) != CPVS_OK) {
        if (s->top) s->ctx->c.release(s->top, uint64_t(4) << (3 * depth), true, st);
        s->top = nullptr;
        s->top_bytes = ~0ull;  // look up without it
        cudaGetLastError();
        return;
    }
    s->top_bytes = uint64_t(4) << (3 * depth);
    s->top_depth = depth;
}

}  // namespace

namespace cpvs {
void shadow_ensure_top(const cpvs_shadow* s, cudaStream_t st, uint32_t max_factor) { ensure_top(s, st, max_factor); }

MultiDag shadow_table_entry(const cpvs_shadow* s) {
    return MultiDag{s->dag, (uint32_t)s->words, s->num_levels, s->leafmasks ? 1u : 0u,
                    s->top ? (uint32_t)s->top_depth : 0u, s->top};
}
}  // namespace cpvs

namespace {

// Queries per thread for a lookup on `s`: the context's fixed choice, or the
// tuned one for this DAG depth and input kind (tuned on the first batch that
// needs it).  Points read in place from host memory cross the host link with
// its latency, which favours more queries in flight per thread than points
// in device memory do, so the two kinds are tuned apart.
int lookup_qpt(const cpvs_shadow* s, const void* q, bool ndc, bool host_in, uint64_t n, uint32_t* bits,
               cudaStream_t st) {
    cpvs::Ctx& c = s->ctx->c;
    if (c.lookup_qpt) return c.lookup_qpt;
    int& t = c.lookup_qpt_tuned[s->num_levels % CPVS_MAX_LEVELS][ndc ? 1 : 0][host_in ? 1 : 0];
    if (!t)
        t = cpvs::tune_lookup(s->dag, s->words, s->num_levels, s->leafmasks, s->top, s->top_depth, q, ndc, n, bits, st);
    return t;
}

}  // namespace

extern "C" {

const char* cpvs_status_string(cpvs_status s) {
    switch (s) {
        case CPVS_OK: return "ok";
        case CPVS_ERR_INVALID_ARG: return "invalid argument";
        case CPVS_ERR_OOM: return "out of device memory";
        case CPVS_ERR_TIMEOUT: return "timed out";
        case CPVS_ERR_DEVICE: return "CUDA device error";
        case CPVS_ERR_UNIMPLEMENTED: return "unimplemented";
        case CPVS_ERR_BUDGET: return "memory budget exceeded";
        case CPVS_ERR_CANCELLED: return "cancelled";
        case CPVS_ERR_CAPACITY: return "output buffer too small";
    }
    return "unknown status";
}

const char* cpvs_last_error(void) { return cpvs::g_last_error.c_str(); }
int cpvs_abi_version(void) { return CPVS_ABI_VERSION; }

cpvs_status cpvs_ctx_create(int device, cpvs_ctx** out) {
    if (!out) return fail(CPVS_ERR_INVALID_ARG, "ctx_create: null out");
    *out = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) {
        cudaGetLastError();
        return fail(CPVS_ERR_DEVICE, "no CUDA device available");
    }
    if (device < 0 || device >= count) return fail(CPVS_ERR_INVALID_ARG, "ctx_create: bad device index");
    CPVS_CUDA(cudaSetDevice(device));
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device;
    cudaMemPool_t pool = nullptr;
    CPVS_CUDA(cudaMemPoolCreate(&pool, &props));
    uint64_t keep = ~0ull;  // freed blocks stay in the pool: never returned to the CUDA driver
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    cudaStream_t fs = nullptr;
    cudaError_t e2 = cudaStreamCreateWithFlags(&fs, cudaStreamNonBlocking);
    if (e2 != cudaSuccess) {
        cudaMemPoolDestroy(pool);
        return cpvs::cuda_fail(e2, "cudaStreamCreateWithFlags");
    }
    auto* c = new cpvs_ctx;
    c->c.device = device;
    c->c.pool = pool;
    c->c.free_stream = fs;
    cudaDeviceGetAttribute(&c->c.num_sms, cudaDevAttrMultiProcessorCount, device);
    int pageable = 0;
    cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, device);
    c->c.pageable_access = pageable != 0;
    *out = c;
    return CPVS_OK;
}

// Objects created from the context must be destroyed first.
void cpvs_ctx_destroy(cpvs_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->c.device);
    cudaDeviceSynchronize();
    cpvs::destroy_plans(ctx->c);
    cudaDeviceSynchronize();
    if (ctx->c.capture_stream) cudaStreamDestroy(ctx->c.capture_stream);
    if (ctx->c.capture_rank_stream) cudaStreamDestroy(ctx->c.capture_rank_stream);
    cudaStreamDestroy(ctx->c.free_stream);
    cudaMemPoolDestroy(ctx->c.pool);
    delete ctx;
}

cpvs_status cpvs_ctx_set_budget(cpvs_ctx* ctx, uint64_t bytes) {
    if (!ctx) return fail(CPVS_ERR_INVALID_ARG, "null ctx");
    ctx->c.budget = bytes;
    return CPVS_OK;
}

uint64_t cpvs_ctx_bytes_in_use(const cpvs_ctx* ctx) { return ctx ? ctx->c.in_use + ctx->c.scratch : 0; }

cpvs_status cpvs_ctx_set_option(cpvs_ctx* ctx, cpvs_option key, int64_t value) {
    if (!ctx) return fail(CPVS_ERR_INVALID_ARG, "null ctx");
    switch (key) {
        case CPVS_OPT_LOOKUP_QUERIES_PER_THREAD:
            if (value != 0 && value != 1 && value != 2 && value != 4)
                return fail(CPVS_ERR_INVALID_ARG, "lookup queries per thread must be 0 (tuned), 1, 2 or 4");
            ctx->c.lookup_qpt = (int)value;
            return CPVS_OK;
        case CPVS_OPT_BUILD_CLUSTER_CAP:
            if (value != 0 && value != 2048 && value != 4096 && value != 8192 && value != 16384)
                return fail(CPVS_ERR_INVALID_ARG, "build cluster cap must be 0 (tuned), 2048, 4096, 8192 or 16384");
            ctx->c.build_cluster_cap = (int)value;
            return CPVS_OK;
        case CPVS_OPT_BUILD_INSERT_WAVES:
            if (value < 0 || value > 2) return fail(CPVS_ERR_INVALID_ARG, "build insert waves must be 0 (tuned), 1 or 2");
            ctx->c.build_insert_waves = (int)value;
            return CPVS_OK;
    }
    return fail(CPVS_ERR_INVALID_ARG, "unknown option");
}

cpvs_status cpvs_ctx_last_build(const cpvs_ctx* ctx, cpvs_build_report* out) {
    if (!ctx || !out) return fail(CPVS_ERR_INVALID_ARG, "last_build: null argument");
    const auto& b = ctx->c.last_build;
    *out = cpvs_build_report{b.error_word, b.replans, b.cluster_cap, b.insert_waves, b.tuned, b.tuning_ms};
    return CPVS_OK;
}

int64_t cpvs_ctx_get_option(const cpvs_ctx* ctx, cpvs_option key) {
    if (!ctx) return -1;
    switch (key) {
        case CPVS_OPT_LOOKUP_QUERIES_PER_THREAD: return ctx->c.lookup_qpt;
        case CPVS_OPT_BUILD_CLUSTER_CAP: return ctx->c.build_cluster_cap;
        case CPVS_OPT_BUILD_INSERT_WAVES: return ctx->c.build_insert_waves;
    }
    return -1;
}

cpvs_status cpvs_ctx_enable_timing(cpvs_ctx* ctx, int on) {
    if (!ctx) return fail(CPVS_ERR_INVALID_ARG, "null ctx");
    cudaSetDevice(ctx->c.device);
    ctx->c.timing.on = on != 0;
    ctx->c.timing.reset();
    return CPVS_OK;
}

cpvs_status cpvs_ctx_kernel_times(cpvs_ctx* ctx, double* total_ms, uint64_t* launches, uint32_t capacity,
                                  uint32_t* count) {
    if (!ctx) return fail(CPVS_ERR_INVALID_ARG, "null ctx");
    if (count) *count = cpvs::K_COUNT;
    cudaSetDevice(ctx->c.device);
    ctx->c.timing.collect();
    for (uint32_t i = 0; i < capacity && i < (uint32_t)cpvs::K_COUNT; ++i) {
        if (total_ms) total_ms[i] = ctx->c.timing.ms[i];
        if (launches) launches[i] = ctx->c.timing.launches[i];
    }
    return CPVS_OK;
}

const char* cpvs_kernel_name(uint32_t id) { return cpvs::kernel_name((int)id); }

// ------------------------------------------------------------- hierarchy
namespace {
// `first_level`: the lowest pyramid level stored (1 for a hierarchy handed to
// the caller).  A host map that the GPU reads in place must not change
// before the pyramid has read it: the call waits for that read, unless
// `host_read` is given, which then receives an event recorded after the read
// (null when nothing reads host memory); the caller waits for it before it
// returns to its own caller.
cpvs_status hierarchy_create(cpvs_ctx* ctx, const float* depth, uint32_t n, uint32_t flags, void* stream,
                             int first_level, cpvs_hierarchy** out, cudaEvent_t* host_read = nullptr) {
    if (host_read) *host_read = nullptr;
    if (!ctx || !depth || !out) return fail(CPVS_ERR_INVALID_ARG, "hierarchy_create: null argument");
    *out = nullptr;
    cpvs_status r = check_map_size(n, 2);
    if (r != CPVS_OK) return r;
    r = set_device(ctx);
    if (r != CPVS_OK) return r;
    cudaStream_t st = (cudaStream_t)stream;
    cpvs::Ctx& c = ctx->c;
    const uint64_t dbytes = (uint64_t)n * n * 4;
    const uint64_t lbytes = cpvs::pyramid_bytes(n);
    auto* h = new cpvs_hierarchy;
    h->ctx = ctx;
    h->n = n;
    h->first_level = first_level;
    const bool borrow = (flags & CPVS_IO_DEVICE) && (flags & CPVS_FLAG_BORROW_INPUT);
    if (borrow) {
        h->depth = const_cast<float*>(depth);
        h->owns_depth = false;
    } else {
        r = c.alloc((void**)&h->depth, dbytes, true, st);
        if (r == CPVS_OK) h->bytes += dbytes;
    }
    if (r == CPVS_OK) {
        r = c.alloc((void**)&h->levels, lbytes, true, st);
        if (r == CPVS_OK) h->bytes += lbytes;
    }
    // a host map the GPU reads in place is copied by the pyramid kernel as
    // it reduces it (one pass over the host link); any other host map is
    // uploaded first
    const float* in_place = (!(flags & CPVS_IO_DEVICE) && r == CPVS_OK)
                                ? static_cast<const float*>(cpvs::host_accessible(c, depth))
                                : nullptr;
    if (r == CPVS_OK && !borrow && !in_place) {
        cudaError_t e = cudaMemcpyAsync(h->depth, depth, dbytes,
                                        (flags & CPVS_IO_DEVICE) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) r = cpvs::cuda_fail(e, "hierarchy upload");
    }
    if (r == CPVS_OK) {
        if (in_place) {
            r = cpvs::launch_pyramid(in_place, n, h->levels, st, &c.timing, h->depth, first_level,
                                     cpvs::pyramid_nan_flag(h->levels, n));
            // the caller may reuse its buffer on return: wait for the read
            // (or hand the wait to the caller)
            if (r == CPVS_OK && host_read) {
                cudaError_t e = cudaEventCreateWithFlags(host_read, cudaEventDisableTiming);
                if (e == cudaSuccess) e = cudaEventRecord(*host_read, st);
                if (e != cudaSuccess) r = cpvs::cuda_fail(e, "hierarchy read of the host map");
            }
            if (r != CPVS_OK || !host_read) {
                const cudaError_t e = cudaStreamSynchronize(st);
                if (e != cudaSuccess && r == CPVS_OK) r = cpvs::cuda_fail(e, "hierarchy read of the host map");
            }
        } else {
            r = cpvs::launch_pyramid(h->depth, n, h->levels, st, &c.timing, nullptr, first_level,
                                     cpvs::pyramid_nan_flag(h->levels, n));
        }
    }
    h->touch(st);
    if (r != CPVS_OK) {
        if (host_read && *host_read) {
            cudaEventDestroy(*host_read);
            *host_read = nullptr;
        }
        cpvs_hierarchy_destroy(h);
        return r;
    }
    *out = h;
    return CPVS_OK;
}
}  // namespace

cpvs_status cpvs_hierarchy_create(cpvs_ctx* ctx, const float* depth, uint32_t n, uint32_t flags, void* stream,
                                  cpvs_hierarchy** out) {
    return hierarchy_create(ctx, depth, n, flags, stream, 1, out);
}

cpvs_status cpvs_hierarchy_create_batch(cpvs_ctx* ctx, const float* const* depths, const uint32_t* sides,
                                        uint32_t count, uint32_t flags, void* stream, cpvs_hierarchy** out) {
    if (!ctx || (count && (!depths || !sides || !out)))
        return fail(CPVS_ERR_INVALID_ARG, "hierarchy_create_batch: null argument");
    for (uint32_t i = 0; i < count; ++i) out[i] = nullptr;
    for (uint32_t i = 0; i < count; ++i) {
        if (!depths[i]) return fail(CPVS_ERR_INVALID_ARG, "hierarchy_create_batch: null map " + std::to_string(i));
        cpvs_status r = check_map_size(sides[i], 2);
        if (r != CPVS_OK) return r;
    }
    cpvs_status r = set_device(ctx);
    if (r != CPVS_OK || count == 0) return r;
    cudaStream_t st = (cudaStream_t)stream;
    cpvs::Ctx& c = ctx->c;
    const bool dev = (flags & CPVS_IO_DEVICE) != 0, borrow = dev && (flags & CPVS_FLAG_BORROW_INPUT);
    std::vector<cpvs_hierarchy*> hs;
    std::vector<cpvs::PyramidMap> maps;
    hs.reserve(count);
    maps.reserve(count);
    for (uint32_t i = 0; i < count && r == CPVS_OK; ++i) {
        const uint32_t n = sides[i];
        auto* h = new cpvs_hierarchy;
        h->ctx = ctx;
        h->n = n;
        h->first_level = 1;
        hs.push_back(h);
        const uint64_t dbytes = (uint64_t)n * n * 4, lbytes = cpvs::pyramid_bytes(n);
        if (borrow) {
            h->depth = const_cast<float*>(depths[i]);
            h->owns_depth = false;
        } else {
            r = c.alloc((void**)&h->depth, dbytes, true, st);
            if (r == CPVS_OK) {
                h->bytes += dbytes;
                const cudaError_t e = cudaMemcpyAsync(h->depth, depths[i], dbytes,
                                                      dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st);
                if (e != cudaSuccess) r = cpvs::cuda_fail(e, "hierarchy_create_batch: map upload");
            }
        }
        if (r == CPVS_OK) r = c.alloc((void**)&h->levels, lbytes, true, st);
        if (r == CPVS_OK) {
            h->bytes += lbytes;
            maps.push_back(cpvs::PyramidMap{h->depth, n, h->levels, 1, cpvs::pyramid_nan_flag(h->levels, n)});
        }
    }
    if (r == CPVS_OK) r = cpvs::launch_pyramid_batch(maps, st, &c.timing);
    for (cpvs_hierarchy* h : hs) h->touch(st);
    // host maps were copied from the caller's buffers: done before return
    if (!dev || r != CPVS_OK) {
        const cudaError_t e = cudaStreamSynchronize(st);
        if (e != cudaSuccess && r == CPVS_OK) r = cpvs::cuda_fail(e, "hierarchy_create_batch");
    }
    if (r != CPVS_OK) {
        for (cpvs_hierarchy* h : hs) cpvs_hierarchy_destroy(h);
        return r;
    }
    for (uint32_t i = 0; i < count; ++i) out[i] = hs[i];
    return CPVS_OK;
}


void cpvs_hierarchy_destroy(cpvs_hierarchy* h) {
    if (!h) return;
    cpvs::Ctx& c = h->ctx->c;
    cudaSetDevice(c.device);
    if (h->depth && h->owns_depth) c.release(h->depth, (uint64_t)h->n * h->n * 4, true, nullptr, h->last_use);
    if (h->levels) c.release(h->levels, cpvs::pyramid_bytes(h->n), true, nullptr, h->last_use);
    delete h;
}

uint32_t cpvs_hierarchy_num_levels(const cpvs_hierarchy* h) { return h ? (uint32_t)cpvs::log2_u32(h->n) + 1 : 0; }
uint32_t cpvs_hierarchy_size(const cpvs_hierarchy* h) { return h ? h->n : 0; }

cpvs_status cpvs_hierarchy_level(const cpvs_hierarchy* h, uint32_t level, float* host_out, uint64_t capacity,
                                 void* stream) {
    if (!h || !host_out) return fail(CPVS_ERR_INVALID_ARG, "hierarchy_level: null argument");
    const uint32_t nl = cpvs_hierarchy_num_levels(h);
    if ((int)level < h->first_level || level >= nl)
        return fail(CPVS_ERR_INVALID_ARG, "hierarchy_level: level out of range");
    const uint64_t s = h->n >> level;
    if (capacity < 2 * s * s) return fail(CPVS_ERR_CAPACITY, "hierarchy_level: buffer too small");
    cpvs_status r = set_device(h->ctx);
    if (r != CPVS_OK) return r;
    cudaStream_t st = (cudaStream_t)stream;
    CPVS_CUDA(cudaMemcpyAsync(host_out, h->levels + cpvs::pyramid_level_offset(h->n, (int)level), 2 * s * s * 4,
                              cudaMemcpyDeviceToHost, st));
    h->touch(st);
    CPVS_CUDA(cudaStreamSynchronize(st));
    return CPVS_OK;
}

// ---------------------------------------------------------------- raster
cpvs_status cpvs_raster_depth(cpvs_ctx* ctx, const float* boxes, uint32_t num_boxes, const float* spheres,
                              uint32_t num_spheres, float plane, uint32_t n, uint32_t x0, uint32_t y0, uint32_t w,
                              uint32_t h, float* depth_out, uint32_t flags, void* stream) {
    if (!ctx || !depth_out || (num_boxes && !boxes) || (num_spheres && !spheres))
        return fail(CPVS_ERR_INVALID_ARG, "raster_depth: null argument");
    if (!is_pow2(n) || n > 65536 || (uint64_t)x0 + w > n || (uint64_t)y0 + h > n)
        return fail(CPVS_ERR_INVALID_ARG, "raster_depth: window must lie inside a power-of-two map of side <= 65536");
    cpvs_status r = set_device(ctx);
    if (r != CPVS_OK) return r;
    cudaStream_t st = (cudaStream_t)stream;
    cpvs::Ctx& c = ctx->c;
    const uint64_t bb = (uint64_t)num_boxes * 5 * 4, sb = (uint64_t)num_spheres * 4 * 4;
    const uint64_t ob = (uint64_t)w * h * 4;
    void *db = nullptr, *ds = nullptr;
    bool ob_own = false, os_own = false;
    r = stage_in(c, boxes, bb, flags, st, &db, &ob_own);
    if (r == CPVS_OK) r = stage_in(c, spheres, sb, flags, st, &ds, &os_own);
    float* out = depth_out;
    bool out_own = false;
    if (r == CPVS_OK && !(flags & CPVS_IO_DEVICE)) {
        out = static_cast<float*>(host_accessible(c, depth_out));
        if (!out) {
            r = c.alloc((void**)&out, std::max<uint64_t>(ob, 4), false, st);
            out_own = r == CPVS_OK;
        }
    }
    if (r == CPVS_OK)
        r = cpvs::launch_raster(static_cast<const float*>(db), num_boxes, static_cast<const float*>(ds), num_spheres,
                                plane, n, x0, y0, w, h, out, st, &c.timing);
    if (r == CPVS_OK && !(flags & CPVS_IO_DEVICE)) {
        cudaError_t e = out_own ? cudaMemcpyAsync(depth_out, out, ob, cudaMemcpyDeviceToHost, st) : cudaSuccess;
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) r = cpvs::cuda_fail(e, "raster read-back");
    }
    if (ob_own) c.release(db, std::max<uint64_t>(bb, 4), false, st);
    if (os_own) c.release(ds, std::max<uint64_t>(sb, 4), false, st);
    if (out_own) c.release(out, std::max<uint64_t>(ob, 4), false, st);
    return r;
}

cpvs_status cpvs_raster_triangles(cpvs_ctx* ctx, const float* tris, uint32_t num_tris, float plane, uint32_t n,
                                  uint32_t x0, uint32_t y0, uint32_t w, uint32_t h, float* depth_out, uint32_t flags,
                                  void* stream) {
    if (!ctx || !depth_out || (num_tris && !tris)) return fail(CPVS_ERR_INVALID_ARG, "raster_triangles: null argument");
    if (!is_pow2(n) || n > 65536 || (uint64_t)x0 + w > n || (uint64_t)y0 + h > n)
        return fail(CPVS_ERR_INVALID_ARG, "raster_triangles: window must lie inside a power-of-two map of side <= 65536");
    cpvs_status r = set_device(ctx);
    if (r != CPVS_OK) return r;
    cudaStream_t st = (cudaStream_t)stream;
    cpvs::Ctx& c = ctx->c;
    const uint64_t tb = (uint64_t)num_tris * 9 * 4, ob = (uint64_t)w * h * 4;
    void* dt = nullptr;
    bool dt_own = false;
    r = stage_in(c, tris, tb, flags, st, &dt, &dt_own);
    float* out = depth_out;
    bool out_own = false;
    if (r == CPVS_OK && !(flags & CPVS_IO_DEVICE)) {
        out = static_cast<float*>(host_accessible(c, depth_out));
        if (!out) {
            r = c.alloc((void**)&out, std::max<uint64_t>(ob, 4), false, st);
            out_own = r == CPVS_OK;
        }
    }
    if (r == CPVS_OK)
        r = cpvs::launch_raster_triangles(c, static_cast<const float*>(dt), num_tris, plane, n, x0, y0, w, h, out, st);
    if (r == CPVS_OK && !(flags & CPVS_IO_DEVICE)) {
        cudaError_t e = out_own ? cudaMemcpyAsync(depth_out, out, ob, cudaMemcpyDeviceToHost, st) : cudaSuccess;
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) r = cpvs::cuda_fail(e, "raster_triangles read-back");
    } else if (r == CPVS_OK && dt_own) {
        cudaStreamSynchronize(st);
    }
    if (dt_own) c.release(dt, std::max<uint64_t>(tb, 4), false, st);
    if (out_own) c.release(out, std::max<uint64_t>(ob, 4), false, st);
    return r;
}

// ---------------------------------------------------------------- shadow
cpvs_status cpvs_shadow_create(cpvs_ctx* ctx, const cpvs_hierarchy* h, uint32_t z_tile_index, uint32_t z_tile_num,
                               uint32_t flags, void* stream, cpvs_shadow** out) {
    if (!ctx || !h || !out) return fail(CPVS_ERR_INVALID_ARG, "shadow_create: null argument");
    *out = nullptr;
    cpvs_status r0 = check_map_size(h->n, 8);
    if (r0 != CPVS_OK) return r0;
    if (z_tile_num == 0 || z_tile_index >= z_tile_num)
        return fail(CPVS_ERR_INVALID_ARG, "shadow_create: need z_tile_index < z_tile_num");
    // every voxel's z and its centre z+0.5 must be exact in float32, as the
    // classification computes them (src/CompressedShadowUtil.cpp:36-40,
    // src/CompressedShadowUtil.h:51-57)
    if ((uint64_t)h->n * z_tile_num > (1ull << 23))
        return fail(CPVS_ERR_INVALID_ARG, "shadow_create: n * z_tile_num must not exceed 2^23");
    cpvs_status r = set_device(ctx);
    if (r != CPVS_OK) return r;
    const uint32_t nl = (uint32_t)cpvs::log2_u32(h->n) + 1;
    const bool leaf = (flags & CPVS_FLAG_LEAFMASKS) && (nl - 3 >= 2);
    std::vector<cpvs::SourceSpec> src{{h->depth, h->levels, h->n, cpvs::pyramid_nan_flag(h->levels, h->n)}};
    std::vector<cpvs::JobSpec> jobs{{0, z_tile_index, z_tile_num}};
    DagBlock* block = nullptr;
    std::vector<cpvs_shadow*> shadows;
    r = build_into_shadows(ctx, src, jobs, leaf, (cudaStream_t)stream, &block, shadows);
    h->touch((cudaStream_t)stream);
    if (r != CPVS_OK) return r;
    *out = shadows[0];
    return CPVS_OK;
}

cpvs_status cpvs_shadow_create_batch(cpvs_ctx* ctx, const cpvs_hierarchy* const* sources, uint32_t num_sources,
                                     const cpvs_build_job* jobs, uint32_t num_jobs, uint32_t flags, void* stream,
                                     cpvs_shadow** out) {
    if (!ctx || !sources || !jobs || !out) return fail(CPVS_ERR_INVALID_ARG, "create_batch: null argument");
    for (uint32_t j = 0; j < num_jobs; ++j) out[j] = nullptr;
    if (num_jobs == 0) return CPVS_OK;
    std::vector<cpvs::SourceSpec> src(num_sources);
    for (uint32_t i = 0; i < num_sources; ++i) {
        if (!sources[i]) return fail(CPVS_ERR_INVALID_ARG, "create_batch: null hierarchy");
        cpvs_status r = check_map_size(sources[i]->n, 8);
        if (r != CPVS_OK) return r;
        src[i] = cpvs::SourceSpec{sources[i]->depth, sources[i]->levels, sources[i]->n,
                                  cpvs::pyramid_nan_flag(sources[i]->levels, sources[i]->n)};
    }
    // jobs grouped by leafmask mode (maps below 16^2 cannot use leafmasks)
    std::vector<cpvs::JobSpec> group[2];
    std::vector<uint32_t> index[2];
    for (uint32_t j = 0; j < num_jobs; ++j) {
        const cpvs_build_job& jb = jobs[j];
        if (jb.source >= num_sources) return fail(CPVS_ERR_INVALID_ARG, "create_batch: job source out of range");
        if (jb.z_tile_num == 0 || jb.z_tile_index >= jb.z_tile_num)
            return fail(CPVS_ERR_INVALID_ARG, "create_batch: need z_tile_index < z_tile_num");
        if ((uint64_t)src[jb.source].n * jb.z_tile_num > (1ull << 23))
            return fail(CPVS_ERR_INVALID_ARG, "create_batch: n * z_tile_num must not exceed 2^23");
        const uint32_t nl = (uint32_t)cpvs::log2_u32(src[jb.source].n) + 1;
        const int g = ((flags & CPVS_FLAG_LEAFMASKS) && nl - 3 >= 2) ? 1 : 0;
        group[g].push_back(cpvs::JobSpec{jb.source, jb.z_tile_index, jb.z_tile_num});
        index[g].push_back(j);
    }
    cpvs_status r = set_device(ctx);
    if (r != CPVS_OK) return r;
    for (int g = 0; g < 2 && r == CPVS_OK; ++g) {
        if (group[g].empty()) continue;
        DagBlock* block = nullptr;
        std::vector<cpvs_shadow*> shadows;
        r = build_into_shadows(ctx, src, group[g], g == 1, (cudaStream_t)stream, &block, shadows);
        for (size_t k = 0; k < shadows.size(); ++k) out[index[g][k]] = shadows[k];
    }
    for (uint32_t i = 0; i < num_sources; ++i) sources[i]->touch((cudaStream_t)stream);
    if (r != CPVS_OK) {
        for (uint32_t j = 0; j < num_jobs; ++j) {
            cpvs_shadow_destroy(out[j]);
            out[j] = nullptr;
        }
    }
    return r;
}

cpvs_status cpvs_shadow_create_from_depth(cpvs_ctx* ctx, const float* depth, uint32_t n, uint32_t z_tile_index,
                                          uint32_t z_tile_num, uint32_t flags, void* stream, cpvs_shadow** out) {
    if (out) *out = nullptr;
    cpvs_status r = check_map_size(n, 8);
    if (r != CPVS_OK) return r;
    // The temporary hierarchy is gone before this call returns, so a device
    // map can be read in place.
    // A host map read in place is waited for once, at the end: the build is
    // queued behind the pyramid instead of after a host round trip.
    cpvs_hierarchy* h = nullptr;
    cudaEvent_t host_read = nullptr;
    r = cpvs::hierarchy_create_for_build(ctx, depth, n, flags | CPVS_FLAG_BORROW_INPUT, flags, stream, &h, &host_read);
    if (r != CPVS_OK) return r;
    r = cpvs_shadow_create(ctx, h, z_tile_index, z_tile_num, flags, stream, out);
    cpvs_hierarchy_destroy(h);
    if (host_read) {
        const cudaError_t e = cudaEventSynchronize(host_read);
        cudaEventDestroy(host_read);
        if (e != cudaSuccess && r == CPVS_OK) {
            cpvs_shadow_destroy(*out);
            *out = nullptr;
            r = cpvs::cuda_fail(e, "hierarchy read of the host map");
        }
    }
    return r;
}

void cpvs_shadow_destroy(cpvs_shadow* s) {
    if (!s) return;
    cudaSetDevice(s->ctx->c.device);
    if (s->top) s->ctx->c.release(s->top, s->top_bytes, true, nullptr, s->last_use);
    block_unref(s->block, s->last_use);
    delete s;
}

uint32_t cpvs_shadow_num_levels(const cpvs_shadow* s) { return s ? s->num_levels : 0; }
int cpvs_shadow_uses_leafmasks(const cpvs_shadow* s) { return s && s->leafmasks ? 1 : 0; }

cpvs_visibility cpvs_shadow_total_visibility(const cpvs_shadow* s) {
    if (!s) return CPVS_PARTIAL;
    if (s->root_mask == 0x5555u) return CPVS_VISIBLE;
    if (s->root_mask == 0u) return CPVS_SHADOW;
    return CPVS_PARTIAL;
}

uint64_t cpvs_shadow_dag_size(const cpvs_shadow* s) { return s ? s->words : 0; }
const uint32_t* cpvs_shadow_device_dag(const cpvs_shadow* s) { return s ? s->dag : nullptr; }

cpvs_status cpvs_shadow_dag_words(const cpvs_shadow* s, uint32_t* host_out, uint64_t capacity, uint64_t* n_out,
                                  void* stream) {
    if (!s) return fail(CPVS_ERR_INVALID_ARG, "dag_words: null shadow");
    if (n_out) *n_out = s->words;
    if (!host_out) return CPVS_OK;
    if (capacity < s->words) return fail(CPVS_ERR_CAPACITY, "dag_words: buffer too small");
    cpvs_status r = set_device(s->ctx);
    if (r != CPVS_OK) return r;
    cudaStream_t st = (cudaStream_t)stream;
    CPVS_CUDA(cudaMemcpyAsync(host_out, s->dag, s->words * 4, cudaMemcpyDeviceToHost, st));
    s->touch(st);
    CPVS_CUDA(cudaStreamSynchronize(st));
    return CPVS_OK;
}

cpvs_status cpvs_shadow_level_counts(const cpvs_shadow* s, uint64_t* tree, uint64_t* unique, uint32_t capacity) {
    if (!s) return fail(CPVS_ERR_INVALID_ARG, "level_counts: null shadow");
    if (capacity < s->num_levels) return fail(CPVS_ERR_CAPACITY, "level_counts: capacity below numLevels");
    for (uint32_t L = 0; L < s->num_levels; ++L) {
        if (tree) tree[L] = L < s->tree.size() ? s->tree[L] : 0;
        if (unique) unique[L] = L < s->uniq.size() ? s->uniq[L] : 0;
    }
    return CPVS_OK;
}

cpvs_status cpvs_shadow_lookup_ndc(const cpvs_shadow* s, const float* xyz, uint64_t n, uint32_t* bits_out,
                                   uint32_t flags, void* stream) {
    if (!s) return fail(CPVS_ERR_INVALID_ARG, "lookup_ndc: null shadow");
    cpvs::NvtxRange range("cpvs lookup");
    cudaStream_t st = (cudaStream_t)stream;
    return lookup_common(s->ctx, xyz, n, bits_out, flags, st, [&](const void* q, uint32_t* bits) {
        ensure_top(s, st);
        cpvs_status r =
            cpvs::launch_lookup(s->dag, s->words, s->num_levels, s->leafmasks, s->top, s->top_depth, q, true, n, bits,
                                st, &s->ctx->c.timing, lookup_qpt(s, q, true, q == xyz && !(flags & CPVS_IO_DEVICE), n,
                                                                  bits, st));
        s->touch(st);
        return r;
    });
}

cpvs_status cpvs_shadow_lookup_voxel(const cpvs_shadow* s, const int32_t* xyz, uint64_t n, uint32_t* bits_out,
                                     uint32_t flags, void* stream) {
    if (!s) return fail(CPVS_ERR_INVALID_ARG, "lookup_voxel: null shadow");
    cpvs::NvtxRange range("cpvs lookup");
    cudaStream_t st = (cudaStream_t)stream;
    return lookup_common(s->ctx, xyz, n, bits_out, flags, st, [&](const void* q, uint32_t* bits) {
        ensure_top(s, st);
        cpvs_status r =
            cpvs::launch_lookup(s->dag, s->words, s->num_levels, s->leafmasks, s->top, s->top_depth, q, false, n,
                                bits, st, &s->ctx->c.timing,
                                lookup_qpt(s, q, false, q == xyz && !(flags & CPVS_IO_DEVICE), n, bits, st));
        s->touch(st);
        return r;
    });
}

cpvs_status cpvs_lookup_ndc_multi(const cpvs_shadow* const* shadows, uint32_t num_shadows, const uint32_t* dag_index,
                                  const float* xyz, uint64_t n, uint32_t* bits_out, uint32_t flags, void* stream) {
    if (!shadows || num_shadows == 0) return fail(CPVS_ERR_INVALID_ARG, "lookup_multi: no shadows");
    if (n && !dag_index) return fail(CPVS_ERR_INVALID_ARG, "lookup_multi: null dag_index");
    cpvs_ctx* ctx = shadows[0] ? shadows[0]->ctx : nullptr;
    for (uint32_t i = 0; i < num_shadows; ++i)
        if (!shadows[i] || shadows[i]->ctx != ctx)
            return fail(CPVS_ERR_INVALID_ARG, "lookup_multi: shadows must share one context");
    cudaStream_t st = (cudaStream_t)stream;
    cpvs_status r = set_device(ctx);
    if (r != CPVS_OK) return r;
    std::vector<cpvs::MultiDag> table(num_shadows);
    for (uint32_t i = 0; i < num_shadows; ++i) {
        ensure_top(shadows[i], st);
        table[i] = cpvs::shadow_table_entry(shadows[i]);
    }
    cpvs::Ctx& c = ctx->c;
    cpvs::MultiDag* dtab = nullptr;
    const uint64_t tb = num_shadows * sizeof(cpvs::MultiDag);
    r = c.alloc((void**)&dtab, tb, false, st);
    if (r != CPVS_OK) return r;
    CPVS_CUDA(cudaMemcpyAsync(dtab, table.data(), tb, cudaMemcpyHostToDevice, st));
    void* ids = nullptr;
    bool ids_own = false;
    r = stage_in(c, dag_index, n * 4, flags, st, &ids, &ids_own);
    if (r == CPVS_OK)
        r = lookup_common(ctx, xyz, n, bits_out, flags, st, [&](const void* q, uint32_t* bits) {
            return cpvs::launch_multi_lookup(dtab, num_shadows, static_cast<const uint32_t*>(ids),
                                             static_cast<const float*>(q), n, bits, st, &c.timing);
        });
    for (uint32_t i = 0; i < num_shadows; ++i) shadows[i]->touch(st);
    if (ids_own) c.release(ids, std::max<uint64_t>(n * 4, 4), false, st);
    c.release(dtab, tb, false, st);
    return r;
}

// ------------------------------------------------------------------ grid
cpvs_status cpvs_grid_create(cpvs_ctx* ctx, uint32_t length, cpvs_grid** out) {
    if (!ctx || !out) return fail(CPVS_ERR_INVALID_ARG, "grid_create: null argument");
    *out = nullptr;
    if (!is_pow2(length) || length > 256) return fail(CPVS_ERR_INVALID_ARG, "grid length must be a power of two <= 256");
    auto* g = new cpvs_grid;
    g->ctx = ctx;
    g->length = length;
    g->cells.assign((size_t)length * length * length, nullptr);
    *out = g;
    return CPVS_OK;
}

static void grid_release_device(cpvs_grid* g) {
    cpvs::Ctx& c = g->ctx->c;
    if (g->gtop) c.release(g->gtop, g->gtop_bytes, true, nullptr, g->last_use);
    g->gtop = nullptr;
    g->gtop_bytes = 0;
    g->gtop_depth = 0;
    block_unref(g->block, g->last_use);
    if (g->cell_words) c.release(g->cell_words, g->cells.size() * 4, true, nullptr, g->last_use);
    g->block = nullptr;
    g->dag = nullptr;
    g->cell_words = nullptr;
    g->finalized = false;
}

void cpvs_grid_destroy(cpvs_grid* g) {
    if (!g) return;
    cudaSetDevice(g->ctx->c.device);
    for (auto* s : g->cells) cpvs_shadow_destroy(s);
    grid_release_device(g);
    delete g;
}

uint32_t cpvs_grid_length(const cpvs_grid* g) { return g ? g->length : 0; }

cpvs_status cpvs_grid_set(cpvs_grid* g, uint32_t x, uint32_t y, uint32_t z, cpvs_shadow* s) {
    if (!g) return fail(CPVS_ERR_INVALID_ARG, "grid_set: null grid");
    if (x >= g->length || y >= g->length || z >= g->length) return fail(CPVS_ERR_INVALID_ARG, "grid_set: cell out of range");
    const size_t i = ((size_t)z * g->length + y) * g->length + x;
    // a cell owns its shadow: a shadow that a cell already holds (this
    // grid's other cells or another grid's) would be destroyed twice
    if (s && s->owner && !(s->owner == g && g->cells[i] == s))
        return fail(CPVS_ERR_INVALID_ARG, "grid_set: the shadow already belongs to a grid cell");
    if (g->cells[i] && g->cells[i] != s) cpvs_shadow_destroy(g->cells[i]);
    g->cells[i] = s;
    if (s) s->owner = g;
    return CPVS_OK;
}

const cpvs_shadow* cpvs_grid_get(const cpvs_grid* g, uint32_t x, uint32_t y, uint32_t z) {
    if (!g || x >= g->length || y >= g->length || z >= g->length) return nullptr;
    return g->cells[((size_t)z * g->length + y) * g->length + x];
}

cpvs_status cpvs_grid_finalize(cpvs_grid* g, int release_cells, void* stream) {
    if (!g) return fail(CPVS_ERR_INVALID_ARG, "grid_finalize: null grid");
    cpvs_status r = set_device(g->ctx);
    if (r != CPVS_OK) return r;
    cudaStream_t st = (cudaStream_t)stream;
    uint64_t total = 0;
    uint32_t nl = 0;
    bool leaf = false;
    std::vector<uint32_t> cellw(g->cells.size());
    for (size_t i = 0; i < g->cells.size(); ++i) {
        const cpvs_shadow* s = g->cells[i];
        if (!s) return fail(CPVS_ERR_INVALID_ARG, "grid_finalize: cell " + std::to_string(i) + " is empty");
        if (i == 0) {
            nl = s->num_levels;
            leaf = s->leafmasks;
        } else if (s->num_levels != nl || s->leafmasks != leaf) {
            return fail(CPVS_ERR_INVALID_ARG, "grid_finalize: cells differ in numLevels or leafmask mode");
        }
        // createTopLevelGrid (src/CompressedShadowContainer.cpp:71-91), with
        // the sentinel values the shader tests (shader/traverse.cs:85-88)
        if (s->root_mask == 0u)
            cellw[i] = 0xFFFFFFFFu;
        else if (s->root_mask == 0x5555u)
            cellw[i] = 0xFFFFFFFEu;
        else
            cellw[i] = (uint32_t)total;
        total += s->words;
        if (total >= 0xFFFFFFFEull) return fail(CPVS_ERR_BUDGET, "grid_finalize: combined DAG exceeds 2^32-2 words");
    }
    grid_release_device(g);
    cpvs::Ctx& c = g->ctx->c;
    uint32_t* dag = nullptr;
    r = c.alloc((void**)&dag, (total + cpvs::kDagPad) * 4, true, st);
    if (r != CPVS_OK) return r;
    g->block = new DagBlock{g->ctx, dag, (total + cpvs::kDagPad) * 4, 1};
    g->dag = dag;
    g->words = total;
    CPVS_CUDA(cudaMemsetAsync(g->dag + total, 0, cpvs::kDagPad * 4, st));
    r = c.alloc((void**)&g->cell_words, g->cells.size() * 4, true, st);
    if (r != CPVS_OK) {
        grid_release_device(g);
        return r;
    }
    uint64_t off = 0;
    for (const cpvs_shadow* s : g->cells) {
        CPVS_CUDA(cudaMemcpyAsync(g->dag + off, s->dag, s->words * 4, cudaMemcpyDeviceToDevice, st));
        s->touch(st);
        off += s->words;
    }
    CPVS_CUDA(cudaMemcpyAsync(g->cell_words, cellw.data(), cellw.size() * 4, cudaMemcpyHostToDevice, st));
    g->touch(st);
    CPVS_CUDA(cudaStreamSynchronize(st));
    g->words = total;
    g->dag_levels = nl;
    g->leafmasks = leaf;
    g->finalized = true;
    if (release_cells) {
        for (auto*& s : g->cells) {
            cpvs_shadow_destroy(s);
            s = nullptr;
        }
    }
    return CPVS_OK;
}

cpvs_status cpvs_grid_build(cpvs_grid* g, const cpvs_hierarchy* const* xy_tiles, uint32_t flags, void* stream) {
    if (!g || !xy_tiles) return fail(CPVS_ERR_INVALID_ARG, "grid_build: null argument");
    const uint32_t L = g->length;
    std::vector<cpvs::SourceSpec> src(L * L);
    for (uint32_t i = 0; i < L * L; ++i) {
        const cpvs_hierarchy* h = xy_tiles[i];
        if (!h) return fail(CPVS_ERR_INVALID_ARG, "grid_build: null tile hierarchy");
        if (h->n != xy_tiles[0]->n) return fail(CPVS_ERR_INVALID_ARG, "grid_build: tiles differ in size");
        cpvs_status r = check_map_size(h->n, 8);
        if (r != CPVS_OK) return r;
        src[i] = cpvs::SourceSpec{h->depth, h->levels, h->n, cpvs::pyramid_nan_flag(h->levels, h->n)};
    }
    if ((uint64_t)src[0].n * L > (1ull << 23)) return fail(CPVS_ERR_INVALID_ARG, "grid_build: n * length must not exceed 2^23");
    cpvs_status r = set_device(g->ctx);
    if (r != CPVS_OK) return r;
    cudaStream_t st = (cudaStream_t)stream;
    // cell (x,y,z) = z-tile z of xy tile (x,y), jobs in cell order z*L^2+y*L+x
    // (src/DeferredRenderer.cpp:150-187, src/CompressedShadowContainer.h:34-39)
    std::vector<cpvs::JobSpec> jobs;
    jobs.reserve((size_t)L * L * L);
    for (uint32_t z = 0; z < L; ++z)
        for (uint32_t y = 0; y < L; ++y)
            for (uint32_t x = 0; x < L; ++x) jobs.push_back(cpvs::JobSpec{y * L + x, z, L});
    const uint32_t nl = (uint32_t)cpvs::log2_u32(src[0].n) + 1;
    const bool leaf = (flags & CPVS_FLAG_LEAFMASKS) && (nl - 3 >= 2);
    DagBlock* block = nullptr;
    std::vector<cpvs_shadow*> shadows;
    std::vector<uint64_t> offsets;
    uint64_t total = 0;
    r = build_into_shadows(g->ctx, src, jobs, leaf, st, &block, shadows, &offsets, &total);
    for (uint32_t i = 0; i < L * L; ++i) xy_tiles[i]->touch(st);
    if (r != CPVS_OK) return r;
    if (total >= 0xFFFFFFFEull) {
        for (auto* sh : shadows) cpvs_shadow_destroy(sh);
        return fail(CPVS_ERR_BUDGET, "grid_build: combined DAG exceeds 2^32-2 words");
    }
    std::vector<uint32_t> cellw(jobs.size());
    for (size_t i = 0; i < jobs.size(); ++i) {
        const uint32_t m = shadows[i]->root_mask;
        cellw[i] = (m == 0u) ? 0xFFFFFFFFu : (m == 0x5555u ? 0xFFFFFFFEu : (uint32_t)offsets[i]);
    }
    // the new cell words are allocated before the old cells go, so that a
    // failed build leaves the grid (and every handle to its cells) as it was
    uint32_t* cell_words = nullptr;
    r = g->ctx->c.alloc((void**)&cell_words, g->cells.size() * 4, true, st);
    if (r != CPVS_OK) {
        for (auto* sh : shadows) cpvs_shadow_destroy(sh);
        return r;
    }
    for (auto*& c : g->cells) {
        cpvs_shadow_destroy(c);
        c = nullptr;
    }
    grid_release_device(g);
    g->cell_words = cell_words;
    CPVS_CUDA(cudaMemcpyAsync(g->cell_words, cellw.data(), cellw.size() * 4, cudaMemcpyHostToDevice, st));
    g->block = block;
    block->refs++;
    g->dag = block->base;
    g->words = total;
    for (size_t i = 0; i < jobs.size(); ++i) {
        g->cells[i] = shadows[i];
        shadows[i]->owner = g;
    }
    g->dag_levels = nl;
    g->leafmasks = leaf;
    g->finalized = true;
    g->touch(st);
    CPVS_CUDA(cudaStreamSynchronize(st));  // the host staging above leaves scope
    return CPVS_OK;
}

uint64_t cpvs_grid_dag_size(const cpvs_grid* g) { return g && g->finalized ? g->words : 0; }

cpvs_status cpvs_grid_words(const cpvs_grid* g, uint32_t* dag_out, uint64_t dag_capacity, uint32_t* cells_out,
                            uint64_t cells_capacity, void* stream) {
    if (!g || !g->finalized) return fail(CPVS_ERR_INVALID_ARG, "grid_words: grid not finalized");
    cpvs_status r = set_device(g->ctx);
    if (r != CPVS_OK) return r;
    cudaStream_t st = (cudaStream_t)stream;
    if (dag_out) {
        if (dag_capacity < g->words) return fail(CPVS_ERR_CAPACITY, "grid_words: DAG buffer too small");
        CPVS_CUDA(cudaMemcpyAsync(dag_out, g->dag, g->words * 4, cudaMemcpyDeviceToHost, st));
    }
    if (cells_out) {
        if (cells_capacity < g->cells.size()) return fail(CPVS_ERR_CAPACITY, "grid_words: cell buffer too small");
        CPVS_CUDA(cudaMemcpyAsync(cells_out, g->cell_words, g->cells.size() * 4, cudaMemcpyDeviceToHost, st));
    }
    g->touch(st);
    CPVS_CUDA(cudaStreamSynchronize(st));
    return CPVS_OK;
}

// The grid's top index, built on its first lookup (stream-ordered).
static void ensure_grid_top(const cpvs_grid* cg, cudaStream_t st) {
    cpvs_grid* g = const_cast<cpvs_grid*>(cg);
    if (g->gtop || g->gtop_bytes == ~0ull) return;
    const int depth = cpvs::grid_top_depth(g->length, g->dag_levels, g->leafmasks, g->words);
    const uint64_t bytes = uint64_t(4) << (3 * (cpvs::log2_u32(g->length) + depth));
    if (depth <= 0 || g->ctx->c.alloc((void**)&g->gtop, bytes, true, st) != CPVS_OK ||
        cpvs::launch_grid_top_index(g->dag, g->words, g->cell_words, g->length, g->dag_levels, depth, g->gtop, st) !=
            CPVS_OK) {
        if (g->gtop) g->ctx->c.release(g->gtop, bytes, true, st);
        g->gtop = nullptr;
        g->gtop_bytes = ~0ull;  // look up without it
        cudaGetLastError();
        return;
    }
    g->gtop_bytes = bytes;
    g->gtop_depth = depth;
}

cpvs_status cpvs_grid_lookup_ndc(const cpvs_grid* g, const float* xyz, uint64_t n, uint32_t* bits_out, uint32_t flags,
                                 void* stream) {
    if (!g || !g->finalized) return fail(CPVS_ERR_INVALID_ARG, "grid_lookup_ndc: grid not finalized");
    cudaStream_t st = (cudaStream_t)stream;
    return lookup_common(g->ctx, xyz, n, bits_out, flags, st, [&](const void* q, uint32_t* bits) {
        ensure_grid_top(g, st);
        cpvs_status r = cpvs::launch_grid_lookup(g->dag, g->words, g->cell_words, g->length, g->dag_levels,
                                                 g->leafmasks, g->gtop, g->gtop_depth, static_cast<const float*>(q), n,
                                                 bits, st, &g->ctx->c.timing);
        g->touch(st);
        return r;
    });
}

cpvs_status cpvs_grid_set_filter_size(cpvs_grid* g, uint32_t filter_size) {
    if (!g) return fail(CPVS_ERR_INVALID_ARG, "grid_set_filter_size: null grid");
    if (filter_size > 32) return fail(CPVS_ERR_INVALID_ARG, "grid_set_filter_size: filter size above 32");
    g->filter_size = filter_size ? filter_size : 1;
    return CPVS_OK;
}

cpvs_status cpvs_grid_evaluate(const cpvs_grid* g, const float* positions, uint32_t width, uint32_t height,
                               uint32_t floats_per_pixel, const float* light_view_proj, uint32_t flags, void* out,
                               void* stream) {
    if (!g || !g->finalized) return fail(CPVS_ERR_INVALID_ARG, "grid_evaluate: grid not finalized");
    if (!light_view_proj) return fail(CPVS_ERR_INVALID_ARG, "grid_evaluate: null matrix");
    if (floats_per_pixel < 3) return fail(CPVS_ERR_INVALID_ARG, "grid_evaluate: fewer than 3 floats per pixel");
    const uint64_t n = (uint64_t)width * height;
    if (n == 0) return CPVS_OK;
    if (!positions || !out) return fail(CPVS_ERR_INVALID_ARG, "grid_evaluate: null buffer");
    if (n >= (1ull << 40)) return fail(CPVS_ERR_INVALID_ARG, "grid_evaluate: image too large");
    const bool u8 = (flags & CPVS_EVAL_U8) != 0;
    if (!u8 && g->filter_size > 1)
        return fail(CPVS_ERR_INVALID_ARG, "grid_evaluate: a filter size above 1 needs CPVS_EVAL_U8 output");
    cudaStream_t st = (cudaStream_t)stream;
    const uint64_t obytes = u8 ? n : (n + 31) / 32 * 4;
    return io_common(g->ctx, positions, n * floats_per_pixel * 4, out, obytes, flags, st,
                     [&](const void* q, void* o) {
                         ensure_grid_top(g, st);
                         cpvs_status r = cpvs::launch_grid_evaluate(
                             g->dag, g->words, g->cell_words, g->length, g->dag_levels, g->leafmasks, g->gtop,
                             g->gtop_depth, static_cast<const float*>(q), floats_per_pixel, n, light_view_proj,
                             g->filter_size, u8, o, st, &g->ctx->c.timing);
                         g->touch(st);
                         return r;
                     });
}

cpvs_status cpvs_shade(cpvs_ctx* ctx, uint32_t width, uint32_t height, const float* normals, uint32_t normal_floats,
                       const float* albedo, const uint8_t* visibilities, const float* positions,
                       uint32_t position_floats, const float* shadow_map, uint32_t shadow_map_side,
                       const float* light_view_proj, const float* light_direction, float* rgba_out, void* stream) {
    if (!ctx) return fail(CPVS_ERR_INVALID_ARG, "shade: null context");
    if (!light_direction) return fail(CPVS_ERR_INVALID_ARG, "shade: null light direction");
    for (int k = 0; k < 3; ++k)
        if (!std::isfinite(light_direction[k])) return fail(CPVS_ERR_INVALID_ARG, "shade: light direction not finite");
    if (light_direction[0] == 0.f && light_direction[1] == 0.f && light_direction[2] == 0.f)
        return fail(CPVS_ERR_INVALID_ARG, "shade: zero light direction");
    const uint64_t n = (uint64_t)width * height;
    if (n == 0) return CPVS_OK;
    if (normal_floats < 3) return fail(CPVS_ERR_INVALID_ARG, "shade: fewer than 3 floats per normal");
    const bool map_test = visibilities == nullptr;
    if (map_test) {
        if (position_floats < 3) return fail(CPVS_ERR_INVALID_ARG, "shade: fewer than 3 floats per position");
        if (!light_view_proj) return fail(CPVS_ERR_INVALID_ARG, "shade: null matrix for the shadow-map test");
        if (shadow_map_side == 0 || shadow_map_side > (1u << 16))
            return fail(CPVS_ERR_INVALID_ARG, "shade: shadow map side outside [1, 65536]");
    }
    cpvs_status r = set_device(ctx);
    if (r != CPVS_OK) return r;
    const cpvs::Ctx& c = ctx->c;
    // every pixel buffer must be one the GPU reads (or writes) in place
    auto view = [&](const void* p) -> void* {
        if (!p) return nullptr;
        cudaPointerAttributes a{};
        if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) return const_cast<void*>(p);
        return host_accessible(c, p);
    };
    const float* nrm = static_cast<const float*>(view(normals));
    const float* alb = static_cast<const float*>(view(albedo));
    float* out = static_cast<float*>(view(rgba_out));
    if (!nrm || !alb || !out) return fail(CPVS_ERR_INVALID_ARG, "shade: a buffer the GPU cannot reach (or null)");
    const uint8_t* vis = nullptr;
    const float *pos = nullptr, *sm = nullptr;
    if (map_test) {
        pos = static_cast<const float*>(view(positions));
        sm = static_cast<const float*>(view(shadow_map));
        if (!pos || !sm) return fail(CPVS_ERR_INVALID_ARG, "shade: a buffer the GPU cannot reach (or null)");
    } else {
        vis = static_cast<const uint8_t*>(view(visibilities));
        if (!vis) return fail(CPVS_ERR_INVALID_ARG, "shade: a buffer the GPU cannot reach");
    }
    return cpvs::launch_shade(n, nrm, normal_floats, alb, vis, pos, position_floats, sm, shadow_map_side,
                              light_view_proj, light_direction, out, (cudaStream_t)stream, &ctx->c.timing);
}

}  // extern "C"
namespace cpvs {
// With leafmasks a build reads pyramid levels 3 and up only (the leaves read
// the map itself): levels 1 and 2, the bulk of the pyramid, are reduced on
// chip but never stored.
cpvs_status hierarchy_create_for_build(cpvs_ctx* ctx, const float* depth, uint32_t n, uint32_t flags,
                                       uint32_t build_flags, void* stream, cpvs_hierarchy** out,
                                       cudaEvent_t* host_read) {
    const uint32_t nl = (uint32_t)log2_u32(n) + 1;
    const bool leaf = (build_flags & CPVS_FLAG_LEAFMASKS) && n >= 2 && (nl - 3 >= 2);
    return hierarchy_create(ctx, depth, n, flags, stream, leaf ? 3 : 1, out, host_read);
}
}  // namespace cpvs
