// Host-side interfaces shared by the library's translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "../../include/cpvs.h"

#define CPVS_MAX_LEVELS 18

namespace cpvs {
// Every resident DAG buffer carries this many zeroed words past its last
// word, so a node's mask and child slots can be read once its offset is
// known to lie inside the DAG.
constexpr uint64_t kDagPad = 16;
// Levels below the root replaced by the dense top index in lookups.
constexpr int kTopIndexDepth = 8;  // levels below the root resolved by the lookup's top grid, at most
}  // namespace cpvs

namespace cpvs {

// Records `msg` as this thread's last error and returns `s`.
cpvs_status fail(cpvs_status s, const std::string& msg);
cpvs_status cuda_fail(cudaError_t e, const char* what);

#define CPVS_CUDA(call)                                          \
    do {                                                         \
        cudaError_t e_ = (call);                                 \
        if (e_ != cudaSuccess) return ::cpvs::cuda_fail(e_, #call); \
    } while (0)

// ------------------------------------------------------------- pyramid
// Float2 offset of pyramid level L (L >= 1) in the packed level array of an
// n x n map: levels 1..log2(n) of (n>>l)^2 (min,max) pairs back to back.
inline uint64_t pyramid_level_offset(uint32_t n, int L) {
    uint64_t o = 0;
    for (int l = 1; l < L; ++l) o += (uint64_t)(n >> l) * (n >> l);
    return o;
}
inline uint64_t pyramid_texels(uint32_t n) {
    uint64_t o = 0;
    for (uint32_t s = n >> 1; s >= 1; s >>= 1) o += (uint64_t)s * s;
    return o;
}
// Device bytes of a pyramid: its texels plus 16 bytes, so that reads
// rounded up to 16-byte chunks stay inside the allocation, plus 16 bytes
// that hold the map's NaN flag.
inline uint64_t pyramid_bytes(uint32_t n) { return pyramid_texels(n) * 8 + 32; }
// The word after a pyramid's padding: nonzero when its map holds a NaN
// (set by launch_pyramid when it is given the word).
inline uint32_t* pyramid_nan_flag(float2* levels, uint32_t n) {
    return reinterpret_cast<uint32_t*>(reinterpret_cast<char*>(levels) + pyramid_texels(n) * 8 + 16);
}
inline int log2_u32(uint32_t n) {
    int l = 0;
    while ((1u << l) < n) ++l;
    return l;
}

// Builds levels 1..log2(n) of the min-max pyramid of `depth` into `levels`.
struct Timing;
// `depth_copy` (optional): the map is also copied there while it is read.
// Levels below `store_from` are reduced but not stored (the first pass must
// still store its last level, which the next pass reads: store_from <= 3).
// `nan_flag` (optional): zeroed, then set when the map holds a NaN.
cpvs_status launch_pyramid(const float* depth, uint32_t n, float2* levels, cudaStream_t st, Timing* timing = nullptr,
                           float* depth_copy = nullptr, int store_from = 1, uint32_t* nan_flag = nullptr);
// Many device maps' pyramids at once: pass k of every map in one launch
// (up to three launches per 256 maps, plus one that zeroes the NaN flags).
struct PyramidMap {
    const float* depth;  // device, n x n
    uint32_t n;
    float2* levels;
    int store_from;
    uint32_t* nan_flag;
};
cpvs_status launch_pyramid_batch(const std::vector<PyramidMap>& maps, cudaStream_t st, Timing* timing = nullptr);

// One z-tile of a source map whose per-level node bounds are wanted.
struct BoundJob {
    uint32_t z_idx, z_num;
    uint32_t out_row;  // row of `bounds` to accumulate into
};
// bounds[row * CPVS_MAX_LEVELS + (L-1)] += number of partial cells of the
// job's z range at pyramid level L, for L in [lmin, numLevels-2]: an upper
// bound on the SVO node count at level L-1.
cpvs_status launch_level_bounds(const float2* levels, uint32_t n, int lmin, const BoundJob* jobs_dev, int njobs,
                                unsigned long long* bounds, cudaStream_t st);

// Depth map of a plane plus boxes (cx,cy,hx,hy,top) and spheres
// (cx,cy,r,depth), window [x0,x0+w) x [y0,y0+h) of an n x n map (device
// pointers).
struct Ctx;
// Depth map of triangles (9 floats each) over a plane; bins into tiles
// first (one host synchronisation to size the bins).
cpvs_status launch_raster_triangles(Ctx& c, const float* tris, uint32_t ntris, float plane, uint32_t n, uint32_t x0,
                                    uint32_t y0, uint32_t w, uint32_t h, float* out, cudaStream_t st);
cpvs_status launch_raster(const float* boxes, uint32_t nb, const float* spheres, uint32_t ns, float plane, uint32_t n,
                          uint32_t x0, uint32_t y0, uint32_t w, uint32_t h, float* out, cudaStream_t st,
                          Timing* timing = nullptr);

// --------------------------------------------------------------- build
struct SourceSpec {
    const float* depth;    // device, n*n
    const float2* levels;  // device pyramid (levels 1..log2 n)
    uint32_t n;
    const uint32_t* nan_flag;  // device word, nonzero if the map holds a NaN (null: unknown)
};
struct JobSpec {
    uint32_t source;
    uint32_t z_idx, z_num;
};
struct BuildOutput {
    uint32_t* dag = nullptr;          // device, all jobs concatenated (cudaMalloc'd, caller owns)
    uint64_t dag_words = 0;
    std::vector<uint64_t> job_offset;  // word offset of each job's DAG in `dag`
    std::vector<uint64_t> job_words;
    std::vector<uint32_t> root_mask;
    std::vector<std::vector<uint64_t>> tree_nodes, unique_nodes;  // [job][level]
    bool leafmasks = false;
};
struct Ctx;
// Builds the DAGs of `jobs` (all with the same leafmask mode).
cpvs_status build_dags(Ctx& ctx, const std::vector<SourceSpec>& sources, const std::vector<JobSpec>& jobs,
                       bool leafmasks, cudaStream_t st, BuildOutput& out);
void destroy_plans(Ctx& ctx);

// -------------------------------------------------------------- lookup
// Depth of the top index of a DAG (0: none), its 8^depth words at most
// max_factor times the DAG's size (at least 64 KiB), and its build.
int top_index_depth(uint32_t num_levels, bool leafmasks, uint64_t words, uint32_t max_factor);
cpvs_status launch_top_index(const uint32_t* dag, uint64_t words, int depth, uint32_t* out, cudaStream_t st);
// `top` may be null (no top index).
// One resident DAG in a multi-DAG lookup table.
struct MultiDag {
    const uint32_t* dag;
    uint32_t words;
    uint32_t num_levels;
    uint32_t leafmasks;
    uint32_t top_depth;   // levels resolved by `top` (0: no top grid)
    const uint32_t* top;  // the DAG's top grid, or null
};
cpvs_status launch_multi_lookup(const MultiDag* dags, uint32_t ndags, const uint32_t* ids, const float* xyz, uint64_t n,
                                uint32_t* bits, cudaStream_t st, Timing* timing = nullptr);
// One request of a segmented lookup: n points at xyz, ceil(n/32) words of
// bits, output words [word_start, ...) of the launch, against dags[dag].
struct LookupSegment {
    const float* xyz;
    uint32_t* bits;
    uint64_t word_start;
    uint64_t n;
    uint32_t dag;
    uint32_t pad;
};
cpvs_status launch_segment_lookup(const MultiDag* dags, uint32_t ndags, const LookupSegment* segs, uint32_t nsegs,
                                  uint64_t total_words, cudaStream_t st, Timing* timing = nullptr);
// Times queries_per_thread = 1, 2, 4 on up to 2^24 of the queries, in four
// chunks spread over the batch (writing their bits), and returns the fastest.
int tune_lookup(const uint32_t* dag, uint64_t words, uint32_t num_levels, bool leafmasks, const uint32_t* top,
                int top_depth, const void* xyz, bool ndc, uint64_t n, uint32_t* bits, cudaStream_t st);
// `queries_per_thread` (1, 2 or 4): independent descents each thread carries.
cpvs_status launch_lookup(const uint32_t* dag, uint64_t words, uint32_t num_levels, bool leafmasks,
                          const uint32_t* top, int top_depth, const void* xyz, bool ndc, uint64_t n, uint32_t* bits,
                          cudaStream_t st, Timing* timing = nullptr, int queries_per_thread = 4);
// World-space evaluation over a grid: n pixels of `fpp` floats (xyz first),
// column-major 4x4 light view-projection, PCF footprint `filter`; output one
// byte per pixel (u8) or one bit per pixel.
// Grid top index: depth (levels of every cell DAG it resolves; 0: none) and
// build into (length * 2^depth)^3 words.
int grid_top_depth(uint32_t length, uint32_t dag_levels, bool leafmasks, uint64_t words);
cpvs_status launch_grid_top_index(const uint32_t* dag, uint64_t words, const uint32_t* cells, uint32_t length,
                                  uint32_t dag_levels, int depth, uint32_t* out, cudaStream_t st);
cpvs_status launch_grid_evaluate(const uint32_t* dag, uint64_t words, const uint32_t* cells, uint32_t length,
                                 uint32_t dag_levels, bool leafmasks, const uint32_t* gtop, int gdepth,
                                 const float* positions, uint32_t fpp, uint64_t n, const float* light_view_proj,
                                 uint32_t filter, bool u8, void* out, cudaStream_t st, Timing* timing = nullptr);
cpvs_status launch_grid_lookup(const uint32_t* dag, uint64_t words, const uint32_t* cells, uint32_t length,
                               uint32_t dag_levels, bool leafmasks, const uint32_t* gtop, int gdepth, const float* xyz,
                               uint64_t n, uint32_t* bits, cudaStream_t st, Timing* timing = nullptr);
// Deferred shading of n pixels (device buffers; visibilities null selects
// the shadow-map test on positions, shadow_map and light_view_proj).
cpvs_status launch_shade(uint64_t n, const float* normals, uint32_t normal_floats, const float* albedo,
                         const uint8_t* visibilities, const float* positions, uint32_t position_floats,
                         const float* shadow_map, uint32_t shadow_map_side, const float* light_view_proj,
                         const float* light_direction, float* out, cudaStream_t st, Timing* timing = nullptr);

// ------------------------------------------------------------ timing
// Kernels timed (when a context's timing is on) with a CUDA event pair on
// the launching stream around every launch; kernel_name() gives the kernel
// (or, for K_EXPAND_WRITE and K_SCAN, the kernels) each id times.
enum KernelId : int {
    K_PYRAMID = 0,
    K_LEVEL_BOUNDS,
    K_EXPAND_COUNT,
    K_EXPAND_WRITE,
    K_LEAF_COLUMNS,
    K_CLASSIFY_BOTTOM,
    K_TABLE_CLEAR,
    K_LEAF_RESOLVE,
    K_INSERT_INNER,
    K_RESOLVE,
    K_SCAN,
    K_REMAP,
    K_LAYOUT,
    K_EMIT,
    K_LOOKUP,
    K_GRID_LOOKUP,
    K_RASTER,
    K_MULTI_LOOKUP,
    K_EVALUATE,
    K_SHADE,
    K_LEAF_CLASSES,
    K_TOP_INDEX,
    K_COUNT
};
const char* kernel_name(int id);

struct Timing {
    bool on = false;
    std::vector<cudaEvent_t> free_events;
    struct Pending {
        int id;
        cudaEvent_t a, b;
    };
    std::vector<Pending> pending;
    double ms[K_COUNT] = {0};
    uint64_t launches[K_COUNT] = {0};
    cudaEvent_t get();
    void collect();  // waits for pending events and accumulates
    void reset();
    ~Timing();
};

// An NVTX range over its scope (host phases of builds, lookups and the
// server's batches, for a timeline profiler; a no-op without one).
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

// Records an event pair around the launches in its scope.
struct KernelTimer {
    Timing* t;
    int id;
    cudaStream_t st;
    cudaEvent_t a = nullptr;
    KernelTimer(Timing* timing, int kid, cudaStream_t s);
    ~KernelTimer();
};

// ----------------------------------------------------------------- ctx
struct Ctx {
    Timing timing;
    int device = 0;
    int num_sms = 0;
    int cluster_blocks = -1;  // blocks per cluster of the small-level build kernels (-1: not probed yet)
    bool pageable_access = false;  // the GPU reads pageable host memory in place
    // lookup queries per thread: fixed by cpvs_ctx_set_option, else tuned
    // once per (DAG levels, NDC or voxel input)
    int lookup_qpt = 0;
    int lookup_qpt_tuned[CPVS_MAX_LEVELS][2][2] = {};  // [levels][ndc][points in host memory]
    // build launch shapes fixed by cpvs_ctx_set_option (0: timed per plan on
    // its first build): the largest level the cluster kernels take, and the
    // inner-level insert's grid in resident waves
    int build_cluster_cap = 0;
    int build_insert_waves = 0;
    bool tune_builds = true;  // a server's context does not time candidates inside its loop
    // what the last build did (cpvs_ctx_last_build)
    struct BuildReport {
        uint32_t error_word = 0, replans = 0, cluster_cap = 0, insert_waves = 0, tuned = 0;
        float tuning_ms = 0.f;
    } last_build;
    uint64_t budget = 0;   // 0 = unlimited
    uint64_t in_use = 0;   // persistent bytes (hierarchies, DAGs, grids)
    uint64_t scratch = 0;  // stream-ordered build / staging scratch
    // All device memory comes from this context's stream-ordered pool, which
    // keeps freed blocks for reuse (no cudaMalloc / cudaFree in steady state).
    cudaMemPool_t pool = nullptr;
    // Stream on which persistent blocks are freed, after their last use.
    cudaStream_t free_stream = nullptr;
    // Allocation on stream `st`, with budget accounting.
    cpvs_status alloc(void** p, uint64_t bytes, bool persistent, cudaStream_t st);
    // Scratch: freed in the order of `st`.  Persistent: freed once
    // `last_use` (the last event recorded after work on the block) is reached.
    void release(void* p, uint64_t bytes, bool persistent, cudaStream_t st, cudaEvent_t last_use = nullptr);
    // Cached build plans (scratch + captured launch sequence per batch shape)
    // and the stream their launch sequences are captured on.
    struct PlanCache* plans = nullptr;
    cudaStream_t capture_stream = nullptr;
    cudaStream_t capture_rank_stream = nullptr;  // the ranking passes' branch of a captured build
};

}  // namespace cpvs
