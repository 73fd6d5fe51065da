/*
 * cpvs.h -- C ABI of the GB300 precomputed-voxelized-shadow library.
 *
 * Builds the sparse-voxel DAG of a shadow volume ("compressed shadow") from a
 * float32 depth map on the GPU and answers batched visibility lookups for
 * light-space points.  Every entry point returns a cpvs_status; the library
 * never falls back to the CPU: without a usable CUDA device every call that
 * needs one returns CPVS_ERR_DEVICE.
 *
 * Conventions
 *   - All sizes are in elements unless named *_bytes.
 *   - `stream` is a cudaStream_t passed as void* (NULL = the legacy default
 *     stream).  Calls are stream-ordered; calls that return host data
 *     synchronise that stream before returning.
 *   - Pointers are host memory unless the call's flags say CPVS_IO_DEVICE
 *     (cpvs_shade, which has no flags, takes any buffer the GPU can reach).
 *     A plain pointer carries no size: each buffer must hold the elements
 *     its call documents, and a CPVS_IO_DEVICE pointer must be device memory
 *     of the context's device, which the call uses as given.  (The Python
 *     front end checks its arrays, and the C++ classes their images, before
 *     they call.)
 *   - Handles are immutable after creation and may be read from several host
 *     threads; a cpvs_ctx must not be used by two host threads at once.
 *   - Visibility classes follow the reference's NodeVisibility
 *     (src/CompressedShadow.h:22-26): SHADOW 0, VISIBLE 1, PARTIAL 2.
 *     Lookup results are bit-packed: bit (i % 32) of word (i / 32) is 1 when
 *     point i is lit (VISIBLE) and 0 when it is in shadow.
 */
#ifndef CPVS_H
#define CPVS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CPVS_ABI_VERSION 1

#if defined(__GNUC__)
#define CPVS_API __attribute__((visibility("default")))
#else
#define CPVS_API
#endif

typedef enum cpvs_status {
    CPVS_OK = 0,
    CPVS_ERR_INVALID_ARG = 1,  /* a size, flag or pointer the call cannot accept */
    CPVS_ERR_OOM = 2,          /* device allocation failed */
    CPVS_ERR_TIMEOUT = 3,      /* a bounded wait ended first: cpvs_server_wait's timeout */
    CPVS_ERR_DEVICE = 4,       /* CUDA error, or no usable device */
    CPVS_ERR_UNIMPLEMENTED = 5,
    CPVS_ERR_BUDGET = 6,       /* request exceeds the context's memory budget */
    CPVS_ERR_CANCELLED = 7,    /* request cancelled before it ran */
    CPVS_ERR_CAPACITY = 8      /* a caller-provided buffer is too small */
} cpvs_status;

typedef enum cpvs_visibility {
    CPVS_SHADOW = 0,
    CPVS_VISIBLE = 1,
    CPVS_PARTIAL = 2
} cpvs_visibility;

/* Build flags. */
#define CPVS_FLAG_LEAFMASKS 0x1u     /* 64-bit leafmasks for the last 3 levels
                                        (the reference's #define LEAFMASKS,
                                        src/CompressedShadow.cpp:16-27); used only
                                        when numLevels-3 >= 2, as there */
#define CPVS_IO_DEVICE 0x100u        /* input/output pointers are device memory */
#define CPVS_FLAG_BORROW_INPUT 0x200u  /* with CPVS_IO_DEVICE: a hierarchy reads the
                                          caller's depth map in place instead of
                                          copying it; the caller keeps it alive and
                                          unchanged until the hierarchy is destroyed */

typedef struct cpvs_ctx cpvs_ctx;
typedef struct cpvs_hierarchy cpvs_hierarchy;
typedef struct cpvs_shadow cpvs_shadow;
typedef struct cpvs_grid cpvs_grid;

/* ---- context ---------------------------------------------------------- */

/* Opens the library on CUDA device `device`.  Replaces the GL context the
 * reference renders and dispatches through (src/cpvs.h, src/ShaderProgram.*). */
CPVS_API cpvs_status cpvs_ctx_create(int device, cpvs_ctx** out);
CPVS_API void cpvs_ctx_destroy(cpvs_ctx* ctx);
/* Upper bound on device bytes this context may hold in build scratch plus
 * resident DAGs; 0 = unlimited.  Builds that would exceed it fail with
 * CPVS_ERR_BUDGET. */
CPVS_API cpvs_status cpvs_ctx_set_budget(cpvs_ctx* ctx, uint64_t bytes);
CPVS_API uint64_t cpvs_ctx_bytes_in_use(const cpvs_ctx* ctx);
/* Tunable launch shapes; 0 (the default) = timed by the library.
 * CPVS_OPT_LOOKUP_QUERIES_PER_THREAD: independent descents each lookup
 * thread carries (1, 2 or 4); tuned per DAG depth by timing the three on the
 * first lookup batch of that depth.
 * CPVS_OPT_BUILD_CLUSTER_CAP: the largest level (planned nodes) that the
 * small-level cluster kernels take (2048, 4096, 8192 or 16384); larger
 * levels run in the multi-block kernels.
 * CPVS_OPT_BUILD_INSERT_WAVES: grid of the inner-level merge insert, in
 * waves of resident blocks (1 or 2).
 * The two build shapes are tuned per build plan (one per batch shape) by
 * timing every pair on the plan's first build; setting either fixes both
 * (the other at its default: 8192, 1).  The DAG does not depend on them. */
typedef enum cpvs_option {
    CPVS_OPT_LOOKUP_QUERIES_PER_THREAD = 1,
    CPVS_OPT_BUILD_CLUSTER_CAP = 2,
    CPVS_OPT_BUILD_INSERT_WAVES = 3
} cpvs_option;
CPVS_API cpvs_status cpvs_ctx_set_option(cpvs_ctx* ctx, cpvs_option key, int64_t value);
CPVS_API int64_t cpvs_ctx_get_option(const cpvs_ctx* ctx, cpvs_option key);
/* What the context's last successful build did: the internal-check word of
 * its final pass (always 0: any other bit fails the build), the plan
 * re-growths it needed (a level or hash table outgrew the plan), the launch
 * shapes it ran with, and whether it timed the candidate shapes (a plan's
 * first build) and for how long.  No counterpart in the reference. */
typedef struct cpvs_build_report {
    uint32_t error_word;
    uint32_t replans;
    uint32_t cluster_cap;
    uint32_t insert_waves;
    uint32_t tuned;
    float tuning_ms;
} cpvs_build_report;
CPVS_API cpvs_status cpvs_ctx_last_build(const cpvs_ctx* ctx, cpvs_build_report* out);

/* Per-kernel CUDA-event timing (off by default).  When on, every kernel the
 * context launches is bracketed by an event pair on its stream;
 * cpvs_ctx_kernel_times waits for those events and returns, per kernel id
 * (0 .. count-1, names from cpvs_kernel_name), the summed milliseconds and
 * the launch count since timing was enabled. */
CPVS_API cpvs_status cpvs_ctx_enable_timing(cpvs_ctx* ctx, int on);
CPVS_API cpvs_status cpvs_ctx_kernel_times(cpvs_ctx* ctx, double* total_ms, uint64_t* launches, uint32_t capacity,
                                           uint32_t* count);
CPVS_API const char* cpvs_kernel_name(uint32_t id);
CPVS_API const char* cpvs_status_string(cpvs_status s);
/* Message of the last failed call on this host thread ("" if none). */
CPVS_API const char* cpvs_last_error(void);
CPVS_API int cpvs_abi_version(void);

/* ---- min-max hierarchy ------------------------------------------------ */

/* Device min-max pyramid of an n x n depth map (n a power of two, 2 <= n <=
 * 65536; building a DAG from it needs n >= 8).  Replaces MinMaxHierarchy(const ImageF&)
 * (src/MinMaxHierarchy.h:23, src/MinMaxHierarchy.cpp:9-27).  `depth` is
 * row-major n*n float32, host memory unless flags has CPVS_IO_DEVICE.  The
 * depth map is copied; the caller's buffer may be reused on return. */
CPVS_API cpvs_status cpvs_hierarchy_create(cpvs_ctx* ctx, const float* depth, uint32_t n, uint32_t flags, void* stream,
                                  cpvs_hierarchy** out);
/* `count` hierarchies at once, map i of side sides[i] (sides may differ):
 * the same pyramids as cpvs_hierarchy_create per map, from one launch per
 * pyramid pass over every map's tiles (at most three per 256 maps) instead
 * of up to three per map -- the many-lights case, where the maps' own
 * launches dominate small maps.  flags: CPVS_IO_DEVICE (maps in device
 * memory), CPVS_FLAG_BORROW_INPUT with it (read in place; the maps must
 * outlive the hierarchies).  On failure no hierarchy is returned. */
CPVS_API cpvs_status cpvs_hierarchy_create_batch(cpvs_ctx* ctx, const float* const* depths, const uint32_t* sides,
                                                 uint32_t count, uint32_t flags, void* stream, cpvs_hierarchy** out);
CPVS_API void cpvs_hierarchy_destroy(cpvs_hierarchy* h);
/* numLevels including the depth map itself (MinMaxHierarchy::getNumLevels,
 * src/MinMaxHierarchy.h:60-62). */
CPVS_API uint32_t cpvs_hierarchy_num_levels(const cpvs_hierarchy* h);
CPVS_API uint32_t cpvs_hierarchy_size(const cpvs_hierarchy* h);
/* Copies level `level` (1 <= level < numLevels) to host memory as
 * (n>>level)^2 interleaved (min,max) float pairs, row-major
 * (MinMaxHierarchy::getMin/getMax, src/MinMaxHierarchy.h:31-55).
 * `capacity` is in floats. */
CPVS_API cpvs_status cpvs_hierarchy_level(const cpvs_hierarchy* h, uint32_t level, float* host_out, uint64_t capacity,
                                 void* stream);

/* ---- depth-map producer ----------------------------------------------- */

/* Rasterises the window [x0,x0+w) x [y0,y0+h) of an n x n depth map (n a
 * power of two): a ground plane at depth `plane`, min-combined with
 * axis-aligned boxes (num_boxes x {cx, cy, half-width, half-height, top
 * depth}) and spheres (num_spheres x {cx, cy, radius, centre depth}), in map
 * coordinates [0,1].  Pixel (x,y) samples its centre ((x+0.5)/n, (y+0.5)/n);
 * a box covers the centres in [c-h, c+h]; a sphere contributes
 * depth - sqrt(r^2 - rho^2) where rho^2 < r^2.  Writes w*h float32,
 * row-major.  Replaces the reference's GL shadow pass and read-back
 * (src/DeferredRenderer.cpp:110-148, src/ShadowMap.cpp:23-30) for the
 * synthetic scenes the benchmarks use.  Primitive arrays and the output are
 * host memory unless flags has CPVS_IO_DEVICE. */
CPVS_API cpvs_status cpvs_raster_depth(cpvs_ctx* ctx, const float* boxes, uint32_t num_boxes, const float* spheres,
                                       uint32_t num_spheres, float plane, uint32_t n, uint32_t x0, uint32_t y0,
                                       uint32_t w, uint32_t h, float* depth_out, uint32_t flags, void* stream);

/* Rasterises triangles over a ground plane at depth `plane` into the window
 * [x0,x0+w) x [y0,y0+h) of an n x n depth map (the reference renders meshes
 * into its shadow map under the light, src/DeferredRenderer.cpp:110-148,
 * shader/create_sm.vert:10-17).  `tris` holds num_tris x 9 floats
 * (x0,y0,d0, x1,y1,d1, x2,y2,d2): vertex positions in map coordinates [0,1]
 * and their depths.  A triangle covers pixel centre p = ((x+0.5)/n, (y+0.5)/n)
 * when p lies in its bounding box and the edge functions
 * e0 = (x2-x1)(py-y1) - (y2-y1)(px-x1), e1 = (x0-x2)(py-y2) - (y0-y2)(px-x2),
 * e2 = (x1-x0)(py-y0) - (y1-y0)(px-x0) all have the sign of
 * area = (e0+e1)+e2 != 0 (zero included, either winding); its depth there is
 * ((e0 d0 + e1 d1) + e2 d2) / area -- float32, round to nearest, no
 * contraction, in that order -- and each pixel keeps the minimum (NaN
 * propagates).  Buffers are host memory unless flags has CPVS_IO_DEVICE. */
CPVS_API cpvs_status cpvs_raster_triangles(cpvs_ctx* ctx, const float* tris, uint32_t num_tris, float plane,
                                           uint32_t n, uint32_t x0, uint32_t y0, uint32_t w, uint32_t h,
                                           float* depth_out, uint32_t flags, void* stream);

/* ---- compressed shadow (one DAG) ------------------------------------- */

/* Builds the DAG of z-tile `z_tile_index` of `z_tile_num` from a hierarchy.
 * Replaces CompressedShadow::create(const MinMaxHierarchy&, uint zTileIndex,
 * uint zTileNum) (src/CompressedShadow.h:48-49, src/CompressedShadow.cpp:49-59):
 * the SVO classification, subtree merge and pointer compression all run on
 * the device and the DAG stays resident there.  The DAG words equal the
 * reference's getDAG() whenever the reference's own build is defined. */
CPVS_API cpvs_status cpvs_shadow_create(cpvs_ctx* ctx, const cpvs_hierarchy* h, uint32_t z_tile_index, uint32_t z_tile_num,
                               uint32_t flags, void* stream, cpvs_shadow** out);
/* One DAG of a batch: z-tile `z_tile_index` of `z_tile_num` of hierarchy
 * `source`. */
typedef struct cpvs_build_job {
    uint32_t source;
    uint32_t z_tile_index;
    uint32_t z_tile_num;
} cpvs_build_job;

/* Builds many DAGs in one batch: z-tiles of one map (the reference's
 * createShadowTiles thread per z-tile, src/DeferredRenderer.cpp:150-163) or
 * independent lights of different sizes.  All jobs run through the same
 * device launches; each gets its own shadow handle in out[j] (the handles
 * share one device block, freed when the last of them is destroyed).  The
 * DAG of every job equals the one cpvs_shadow_create would build. */
CPVS_API cpvs_status cpvs_shadow_create_batch(cpvs_ctx* ctx, const cpvs_hierarchy* const* sources,
                                              uint32_t num_sources, const cpvs_build_job* jobs, uint32_t num_jobs,
                                              uint32_t flags, void* stream, cpvs_shadow** out);

/* Depth map straight to DAG: hierarchy + create in one call.  Replaces
 * CompressedShadow::create(const ShadowMap*, ...) (src/CompressedShadow.h:55-56),
 * whose GL read-back becomes a host or device float32 buffer. */
CPVS_API cpvs_status cpvs_shadow_create_from_depth(cpvs_ctx* ctx, const float* depth, uint32_t n, uint32_t z_tile_index,
                                          uint32_t z_tile_num, uint32_t flags, void* stream, cpvs_shadow** out);
CPVS_API void cpvs_shadow_destroy(cpvs_shadow* s);
/* CompressedShadow::getNumLevels (src/CompressedShadow.h:71-73). */
CPVS_API uint32_t cpvs_shadow_num_levels(const cpvs_shadow* s);
/* 1 if the DAG uses 64-bit leafmasks. */
CPVS_API int cpvs_shadow_uses_leafmasks(const cpvs_shadow* s);
/* CompressedShadow::getTotalVisibility (src/CompressedShadow.cpp:66-72);
 * CPVS_PARTIAL ("descend to know") for a null shadow. */
CPVS_API cpvs_visibility cpvs_shadow_total_visibility(const cpvs_shadow* s);
/* Number of 32-bit words in the DAG. */
CPVS_API uint64_t cpvs_shadow_dag_size(const cpvs_shadow* s);
/* Copies the DAG words to host memory: CompressedShadow::getDAG()
 * (src/CompressedShadow.h:75-77).  `capacity` is in words; `n_out` receives
 * the DAG size (may be NULL). */
CPVS_API cpvs_status cpvs_shadow_dag_words(const cpvs_shadow* s, uint32_t* host_out, uint64_t capacity, uint64_t* n_out,
                                  void* stream);
/* Device address of the resident DAG words (valid until destroy). */
CPVS_API const uint32_t* cpvs_shadow_device_dag(const cpvs_shadow* s);
/* Per-level node counts of the last build: `tree` before the subtree merge,
 * `unique` after it; index = level (0 .. numLevels-1). */
CPVS_API cpvs_status cpvs_shadow_level_counts(const cpvs_shadow* s, uint64_t* tree, uint64_t* unique, uint32_t capacity);

/* Visibility of n light-space points in NDC ([-1,1]^3), xyz interleaved
 * float32.  Replaces CompressedShadow::traverse(const vec3, bool)
 * (src/CompressedShadow.h:64, src/CompressedShadow.cpp:404-463) and the
 * per-pixel descent of shader/traverse.cs:75-133; the NDC is quantised with
 * the reference's float32 order (src/CompressedShadowUtil.h:70-75).
 * `bits_out` holds ceil(n/32) words. */
CPVS_API cpvs_status cpvs_shadow_lookup_ndc(const cpvs_shadow* s, const float* xyz, uint64_t n, uint32_t* bits_out,
                                   uint32_t flags, void* stream);
/* Same, for integer voxel coordinates (the path getPathFromNDC yields),
 * xyz interleaved int32. */
CPVS_API cpvs_status cpvs_shadow_lookup_voxel(const cpvs_shadow* s, const int32_t* xyz, uint64_t n, uint32_t* bits_out,
                                     uint32_t flags, void* stream);

/* ---- allocation-free build ------------------------------------------- */

/* Builds one shadow DAG without allocating any device memory.  No
 * counterpart in the reference: it exists for callers that may not allocate,
 * e.g. a render loop that must not stall on cudaMalloc/cudaFree (both can
 * synchronise the device) or a plugin inside a host application that owns
 * all GPU memory.  All scratch lives in a fixed 8 MiB array compiled into
 * this library, which every GPU that loads the library holds until the
 * process exits; maps are limited to n <= 256 with CPVS_FLAG_LEAFMASKS and
 * n <= 64 without (power of two, >= 8); other flag bits are rejected
 * (CPVS_ERR_INVALID_ARG).  `depth` is a device n*n float32 map; the DAG
 * (the same words cpvs_shadow_create_from_depth builds) is written to the
 * device buffer `dag_out` of `dag_capacity` words, and `*dag_words`
 * receives its size (also when the buffer is too small: CPVS_ERR_CAPACITY).
 * The calling thread's current device is used; every call looks up the
 * array's device address there.  The first call on a device may load this
 * library's GPU code (CUDA loads modules lazily), which places the array in
 * device memory and can synchronise: make one warm-up call at start-up,
 * outside render loops and before any stream capture.  All calls share the
 * one array: calls whose work overlaps on the GPU (other streams or host
 * threads) race and must be serialised by the caller.  Returns after the
 * build has finished. */
CPVS_API cpvs_status cpvs_shadow_build_noalloc(const float* depth, uint32_t n, uint32_t z_tile_index,
                                               uint32_t z_tile_num, uint32_t flags, uint32_t* dag_out,
                                               uint64_t dag_capacity, uint64_t* dag_words, void* stream);

/* Visibility of n NDC points against many resident DAGs at once: point i
 * descends shadows[dag_index[i]] (an index outside the table answers
 * shadow).  One launch serves lookups spread over many lights or requests;
 * each answer equals cpvs_shadow_lookup_ndc on that shadow alone.  All
 * shadows must come from one context. */
CPVS_API cpvs_status cpvs_lookup_ndc_multi(const cpvs_shadow* const* shadows, uint32_t num_shadows,
                                           const uint32_t* dag_index, const float* xyz, uint64_t n,
                                           uint32_t* bits_out, uint32_t flags, void* stream);

/* ---- top-level grid (container) -------------------------------------- */

/* A cubic length^3 grid of DAGs (length a power of two).  Replaces
 * CompressedShadowContainer (src/CompressedShadowContainer.h:21-73). */
CPVS_API cpvs_status cpvs_grid_create(cpvs_ctx* ctx, uint32_t length, cpvs_grid** out);
CPVS_API void cpvs_grid_destroy(cpvs_grid* g);
CPVS_API uint32_t cpvs_grid_length(const cpvs_grid* g);
/* CompressedShadowContainer::set (src/CompressedShadowContainer.h:34-39):
 * cell (x,y,z) takes ownership of `s` (destroys any previous DAG there);
 * the grid destroys it, so the caller must not, and must not use `s` after
 * the grid is destroyed.  A shadow that a cell already holds (of this grid or
 * another) is refused with CPVS_ERR_INVALID_ARG. */
CPVS_API cpvs_status cpvs_grid_set(cpvs_grid* g, uint32_t x, uint32_t y, uint32_t z, cpvs_shadow* s);
/* CompressedShadowContainer::get: the DAG at (x,y,z), or NULL. */
CPVS_API const cpvs_shadow* cpvs_grid_get(const cpvs_grid* g, uint32_t x, uint32_t y, uint32_t z);
/* copyToGPU/moveToGPU (src/CompressedShadowContainer.cpp:31-91): concatenates
 * the DAGs in cell order z*L^2+y*L+x and writes the top-level grid, one word
 * per cell: the cell DAG's start offset, or 0xFFFFFFFF / 0xFFFFFFFE for a
 * uniformly shadowed / lit cell.  All cells must be set and share numLevels.
 * With `release_cells` the per-cell DAGs are freed afterwards (moveToGPU). */
CPVS_API cpvs_status cpvs_grid_finalize(cpvs_grid* g, int release_cells, void* stream);
/* Builds every cell of the grid in one batch and finalizes it: cell
 * (x,y,z) is z-tile z of length of the xy tile hierarchy xy_tiles[y*length+x]
 * (the reference's tiled precompute, src/DeferredRenderer.cpp:150-187, and
 * copyToGPU).  xy_tiles holds exactly length^2 handles (the call has no count
 * to check it against).  Replaces any cells set before, once the build has
 * succeeded; tiles must share one size. */
CPVS_API cpvs_status cpvs_grid_build(cpvs_grid* g, const cpvs_hierarchy* const* xy_tiles, uint32_t flags,
                                     void* stream);
/* Size in words of the concatenated DAG, and its copy (after finalize). */
CPVS_API uint64_t cpvs_grid_dag_size(const cpvs_grid* g);
CPVS_API cpvs_status cpvs_grid_words(const cpvs_grid* g, uint32_t* dag_out, uint64_t dag_capacity, uint32_t* cells_out,
                            uint64_t cells_capacity, void* stream);
/* Grid lookup of n NDC points (shader/traverse.cs:41-133): the point is
 * quantised at resolution 2^(dag_levels+grid_levels-1), routed to its cell
 * and descended there.  Points outside the grid are lit. */
CPVS_API cpvs_status cpvs_grid_lookup_ndc(const cpvs_grid* g, const float* xyz, uint64_t n, uint32_t* bits_out,
                                 uint32_t flags, void* stream);

/* ---- serving ---------------------------------------------------------- */

/* Saving and loading built DAGs (no reference counterpart: the reference
 * keeps DAGs in memory only, getDAG() in src/CompressedShadow.h:71-77).
 * The format, little-endian: a 48-byte header -- magic "CPVSDAG\0", u32
 * version 1, u32 kind (0 shadow, 1 grid), u32 numLevels, u32 flags (bit 0
 * leafmasks), u32 grid length (1 for a shadow), u32 0, u64 DAG words, u64
 * FNV-1a-64 checksum of all bytes after the header -- then for a shadow its
 * per-level tree and unique node counts (2 x numLevels u64) and the DAG
 * words, for a grid its length^3 cell words and the combined DAG words.
 * serialize: with buf == NULL only *size is set; else the image is written
 * to the host buffer (CPVS_ERR_CAPACITY when capacity < *size).
 * deserialize: checks magic, version, sizes, checksum and cell offsets
 * (CPVS_ERR_INVALID_ARG) and uploads the DAG; a loaded grid is finalized and
 * has no cell shadows (cpvs_grid_get returns NULL). */
CPVS_API cpvs_status cpvs_shadow_serialize(const cpvs_shadow* s, void* buf, uint64_t capacity, uint64_t* size,
                                           void* stream);
CPVS_API cpvs_status cpvs_shadow_deserialize(cpvs_ctx* ctx, const void* buf, uint64_t size, void* stream,
                                             cpvs_shadow** out);
CPVS_API cpvs_status cpvs_grid_serialize(const cpvs_grid* g, void* buf, uint64_t capacity, uint64_t* size,
                                         void* stream);
CPVS_API cpvs_status cpvs_grid_deserialize(cpvs_ctx* ctx, const void* buf, uint64_t size, void* stream,
                                           cpvs_grid** out);

/* Output of cpvs_grid_evaluate: one byte per pixel instead of one bit. */
#define CPVS_EVAL_U8 0x400u

/* CompressedShadowContainer::setFilterSize (src/CompressedShadowContainer.h:70-73):
 * the width (= height) of the percentage-closer filter footprint of
 * cpvs_grid_evaluate, 1 (default) .. 32.  The reference passes it to its
 * shader but never uses it (shader/traverse.cs:16-17); here it filters. */
CPVS_API cpvs_status cpvs_grid_set_filter_size(cpvs_grid* g, uint32_t filter_size);
/* CompressedShadowContainer::evaluate (src/CompressedShadowContainer.cpp:93-124,
 * shader/traverse.cs:134-148) on buffers instead of textures: `positions`
 * is a row-major width x height image of `floats_per_pixel` (>= 3) floats
 * per pixel whose first three are the world-space position (an rgba32f
 * G-buffer has 4; the 4th is ignored, as the shader reads .xyz).  Each
 * position goes through `light_view_proj` (16 floats, column-major as
 * glm::value_ptr gives them) as c = M * (x, y, z, 1) in float32 without
 * contraction, in the order ((m[r]*x + m[4+r]*y) + m[8+r]*z) + m[12+r];
 * ndc = c.xyz / c.w; then the grid lookup of cpvs_grid_lookup_ndc.  Output:
 * with CPVS_EVAL_U8 one byte per pixel -- 255 lit / 0 shadowed (what the
 * shader's r8 image stores), or with a filter size f > 1 round(255 * lit / f^2)
 * over the f x f texel footprint (offsets -(f-1)/2 .. f/2 in x and y around
 * the quantised path, same depth voxel) -- else one bit per pixel
 * (ceil(width*height/32) words; filter size 1 only).  Host or device
 * buffers as for lookups (CPVS_IO_DEVICE). */
CPVS_API cpvs_status cpvs_grid_evaluate(const cpvs_grid* g, const float* positions, uint32_t width, uint32_t height,
                                        uint32_t floats_per_pixel, const float* light_view_proj, uint32_t flags,
                                        void* out, void* stream);

/* Deferred shading of one frame (shader/shade.frag:34-56, drawn by
 * DeferredRenderer::doAllShading, src/DeferredRenderer.cpp:319-348) on
 * buffers instead of G-buffer textures.  All pixel buffers are row-major
 * width x height images the GPU can read (device memory, or host memory the
 * GPU reaches in place); `rgba_out` receives 4 floats per pixel.
 *   normals:  `normal_floats` (>= 3) floats per pixel, xyz first.
 *   albedo:   4 floats per pixel (the diffuse buffer's rgba).
 *   visibilities: cpvs_grid_evaluate's CPVS_EVAL_U8 output (renderShadow != 0:
 *     vis = byte / 255); or NULL for the shader's shadow-map branch
 *     (renderShadow == 0): `positions` (`position_floats` >= 3 per pixel) go
 *     through `light_view_proj` as in cpvs_grid_evaluate, s = c.xyz / c.w *
 *     0.5 + 0.5, and vis = 0 when the `shadow_map_side`^2 float depth map
 *     `shadow_map` at texel (floor(s.x * side), floor(s.y * side)) is below
 *     s.z, else 1 (nearest filtering; outside the map the border depth 1.0,
 *     src/ShadowMap.cpp:3-9).
 *   light_direction: 3 host floats (normalised here; not all zero).
 * colour = ((0.15 + max(0, dot(N, L)) * vis) * albedo.rgb, albedo.a), every
 * float operation one IEEE round-to-nearest step in the order written, no
 * contraction.  Stream-ordered; returns after the launch. */
CPVS_API cpvs_status cpvs_shade(cpvs_ctx* ctx, uint32_t width, uint32_t height, const float* normals,
                                uint32_t normal_floats, const float* albedo, const uint8_t* visibilities,
                                const float* positions, uint32_t position_floats, const float* shadow_map,
                                uint32_t shadow_map_side, const float* light_view_proj, const float* light_direction,
                                float* rgba_out, void* stream);

/* A request loop that takes builds and lookup batches of any size from any
 * host thread, keeps the built DAGs resident in HBM under a byte budget
 * (least recently used first out), and batches continuously: a dispatcher
 * thread sends all lookups whose DAG is resident as one multi-DAG launch on
 * a lookup stream and never waits for a build; a builder thread builds the
 * pending maps of one side as one batch on a build stream.  The two overlap
 * on the device, and requests that arrive meanwhile join the next launch.  Every
 * answer equals what the plain calls give for that request alone.  The
 * reference has no serving layer; its app builds once and evaluates every
 * frame (src/main.cpp:236-268).  The server takes over `ctx`: do not use the
 * context elsewhere while the server lives. */
typedef struct cpvs_server cpvs_server;

typedef struct cpvs_server_config {
    uint64_t budget_bytes;       /* resident DAG bytes; 0 = unlimited */
    uint32_t max_batch_builds;   /* builds per batch; 0 = 16 */
    uint32_t max_batch_lookups;  /* lookup requests per launch; 0 = 256 */
    uint32_t flags;              /* build flags (CPVS_FLAG_LEAFMASKS) */
} cpvs_server_config;

typedef struct cpvs_server_stats {
    uint64_t builds_done, lookups_done, failed, cancelled, evictions;
    uint64_t resident_dags, resident_bytes, queued;
    double build_p50_ms, build_p99_ms;   /* submit -> done */
    double lookup_p50_ms, lookup_p99_ms;
} cpvs_server_stats;

/* The server takes over `ctx`.  Its builds keep the default launch shapes
 * or those fixed by the context's options (the build tuner does not run
 * inside the serving loop).  Admission by bytes: before a batch of builds,
 * least-recently-used unpinned DAGs are evicted until the batch fits the
 * budget, each new DAG estimated at the largest DAG the server has built
 * from a map of its side (n^2/4 bytes before the first). */
CPVS_API cpvs_status cpvs_server_create(cpvs_ctx* ctx, const cpvs_server_config* cfg, cpvs_server** out);
/* Cancels queued requests, finishes running ones, frees the resident DAGs. */
CPVS_API void cpvs_server_destroy(cpvs_server* s);
/* Builds the n x n host depth map into the resident DAG `key` (replacing any
 * DAG of that key).  `depth` must stay valid until the ticket completes. */
CPVS_API cpvs_status cpvs_server_submit_build(cpvs_server* s, uint64_t key, const float* depth, uint32_t n,
                                              uint64_t* ticket);
/* Looks up n NDC points (xyz interleaved) in the DAG of `key` built by the
 * latest build of `key` submitted before this call (or a later one): waits
 * while that build is pending; fails with CPVS_ERR_INVALID_ARG if it failed,
 * was cancelled or its DAG was evicted, or if `key` was never built.  Bits are written to `bits_out` (ceil(n/32) words).  Both
 * buffers must stay valid until the ticket completes and be readable by the
 * GPU in place (pinned memory; any host memory on hosts where the GPU reads
 * pageable memory). */
CPVS_API cpvs_status cpvs_server_submit_lookup(cpvs_server* s, uint64_t key, const float* xyz, uint64_t n,
                                               uint32_t* bits_out, uint64_t* ticket);
/* Waits up to timeout_us (< 0: forever) for a ticket; returns its result
 * (CPVS_ERR_TIMEOUT if it is not done yet) and its submit-to-done latency.
 * A ticket is reported once. */
CPVS_API cpvs_status cpvs_server_wait(cpvs_server* s, uint64_t ticket, int64_t timeout_us, double* latency_ms);
/* Cancels a ticket that has not started (CPVS_ERR_CANCELLED is then its result). */
CPVS_API cpvs_status cpvs_server_cancel(cpvs_server* s, uint64_t ticket);
CPVS_API cpvs_status cpvs_server_get_stats(cpvs_server* s, cpvs_server_stats* out);

#ifdef __cplusplus
}
#endif

#endif /* CPVS_H */
