// On-disk format of built DAGs: save a shadow or a finalized grid, load it
// back into HBM without rebuilding.  The reference keeps DAGs only in memory
// (getDAG(), src/CompressedShadow.h:71-77; the grid and combined buffer of
// src/CompressedShadowContainer.cpp:52-91); this is checkpoint / resume for
// serving.
//
// Layout (little-endian, every field naturally aligned):
//   0  char[8]  magic "CPVSDAG\0"
//   8  u32      version (1)
//  12  u32      kind: 0 shadow, 1 grid
//  16  u32      numLevels of the DAG (of every cell's DAG for a grid)
//  20  u32      flags: bit 0 leafmasks
//  24  u32      grid side length (1 for a shadow)
//  28  u32      reserved (0)
//  32  u64      DAG words
//  40  u64      FNV-1a 64 checksum of every byte after the header
//  48  shadow: u64 tree[numLevels], u64 unique[numLevels] (per-level node
//              counts before and after the merge), then u32 dag[words]
//      grid:   u32 cells[length^3] (DAG start offset, or 0xFFFFFFFF /
//              0xFFFFFFFE for a uniformly shadowed / lit cell), then
//              u32 dag[words] (the combined DAG)
// Loading checks the magic, version, sizes, the checksum, and that every
// cell offset lies inside the DAG; the lookups bounds-check every node read,
// so a DAG that passes these checks cannot make them read outside it.
#include <cstring>
#include <string>
#include <vector>

#include "objects.h"

using cpvs::fail;

namespace {

constexpr char kMagic[8] = {'C', 'P', 'V', 'S', 'D', 'A', 'G', '\0'};
constexpr uint32_t kVersion = 1, kKindShadow = 0, kKindGrid = 1;
constexpr uint64_t kHeader = 48;

struct Header {
    char magic[8];
    uint32_t version, kind, num_levels, flags, length, reserved;
    uint64_t words, checksum;
};
static_assert(sizeof(Header) == kHeader, "header layout");

uint64_t fnv1a(const unsigned char* p, uint64_t n, uint64_t h = 0xcbf29ce484222325ull) {
    for (uint64_t i = 0; i < n; ++i) {
        h ^= p[i];
        h *= 0x100000001b3ull;
    }
    return h;
}

bool little_endian() {
    const uint32_t one = 1;
    unsigned char b;
    std::memcpy(&b, &one, 1);
    return b == 1;
}

cpvs_status use_device(const cpvs_ctx* ctx) {
    const cudaError_t e = cudaSetDevice(ctx->c.device);
    if (e != cudaSuccess) return cpvs::cuda_fail(e, "cudaSetDevice");
    return CPVS_OK;
}

uint64_t shadow_bytes(uint32_t num_levels, uint64_t words) { return kHeader + 16ull * num_levels + 4 * words; }
uint64_t grid_bytes(uint32_t length, uint64_t words) {
    return kHeader + 4ull * length * length * length + 4 * words;
}

cpvs_status read_header(const void* buf, uint64_t size, uint32_t kind, Header& h) {
    if (!little_endian()) return fail(CPVS_ERR_UNIMPLEMENTED, "deserialize: big-endian hosts are not supported");
    if (!buf || size < kHeader) return fail(CPVS_ERR_INVALID_ARG, "deserialize: buffer shorter than the header");
    std::memcpy(&h, buf, kHeader);
    if (std::memcmp(h.magic, kMagic, 8) != 0) return fail(CPVS_ERR_INVALID_ARG, "deserialize: not a cpvs DAG file");
    if (h.version != kVersion)
        return fail(CPVS_ERR_INVALID_ARG, "deserialize: unsupported version " + std::to_string(h.version));
    if (h.kind != kind)
        return fail(CPVS_ERR_INVALID_ARG, kind == kKindShadow ? "deserialize: file holds a grid, not a shadow"
                                                              : "deserialize: file holds a shadow, not a grid");
    if (h.num_levels < 2 || h.num_levels > 17 || (h.flags & ~1u) || h.reserved)
        return fail(CPVS_ERR_INVALID_ARG, "deserialize: bad header fields");
    if ((h.flags & 1u) && h.num_levels < 5)
        return fail(CPVS_ERR_INVALID_ARG, "deserialize: leafmasks need numLevels >= 5");
    if (h.words == 0 || h.words >= 0xFFFFFFFEull) return fail(CPVS_ERR_INVALID_ARG, "deserialize: bad DAG size");
    const uint64_t want = kind == kKindShadow ? shadow_bytes(h.num_levels, h.words) : grid_bytes(h.length, h.words);
    if (kind == kKindGrid && (h.length == 0 || h.length > 256 || (h.length & (h.length - 1))))
        return fail(CPVS_ERR_INVALID_ARG, "deserialize: bad grid length");
    if (kind == kKindShadow && h.length != 1) return fail(CPVS_ERR_INVALID_ARG, "deserialize: bad header fields");
    if (size < want) return fail(CPVS_ERR_INVALID_ARG, "deserialize: buffer truncated");
    const auto* p = static_cast<const unsigned char*>(buf);
    if (fnv1a(p + kHeader, want - kHeader) != h.checksum)
        return fail(CPVS_ERR_INVALID_ARG, "deserialize: checksum mismatch");
    return CPVS_OK;
}

// Copies `words` DAG words from host memory into a new device block (with
// its zeroed tail) on `st`; the caller synchronizes.
cpvs_status upload_dag(cpvs_ctx* ctx, const unsigned char* src, uint64_t words, cudaStream_t st, DagBlock** out) {
    uint32_t* dag = nullptr;
    const uint64_t bytes = (words + cpvs::kDagPad) * 4;
    cpvs_status r = ctx->c.alloc((void**)&dag, bytes, true, st);
    if (r != CPVS_OK) return r;
    cudaError_t e = cudaMemcpyAsync(dag, src, words * 4, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(dag + words, 0, cpvs::kDagPad * 4, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // the source is the caller's buffer
    if (e != cudaSuccess) {
        ctx->c.release(dag, bytes, true, nullptr);
        return cpvs::cuda_fail(e, "deserialize upload");
    }
    *out = new DagBlock{ctx, dag, bytes, 1};
    return CPVS_OK;
}

}  // namespace

extern "C" {

cpvs_status cpvs_shadow_serialize(const cpvs_shadow* s, void* buf, uint64_t capacity, uint64_t* size, void* stream) {
    if (!s) return fail(CPVS_ERR_INVALID_ARG, "shadow_serialize: null shadow");
    if (!little_endian()) return fail(CPVS_ERR_UNIMPLEMENTED, "serialize: big-endian hosts are not supported");
    const uint64_t need = shadow_bytes(s->num_levels, s->words);
    if (size) *size = need;
    if (!buf) return CPVS_OK;
    if (capacity < need) return fail(CPVS_ERR_CAPACITY, "shadow_serialize: buffer too small");
    cpvs_status r = use_device(s->ctx);
    if (r != CPVS_OK) return r;
    auto* p = static_cast<unsigned char*>(buf);
    std::vector<uint64_t> counts(2ull * s->num_levels, 0);
    for (uint32_t L = 0; L < s->num_levels; ++L) {
        counts[L] = L < s->tree.size() ? s->tree[L] : 0;
        counts[s->num_levels + L] = L < s->uniq.size() ? s->uniq[L] : 0;
    }
    std::memcpy(p + kHeader, counts.data(), counts.size() * 8);
    cudaStream_t st = (cudaStream_t)stream;
    CPVS_CUDA(cudaMemcpyAsync(p + kHeader + counts.size() * 8, s->dag, s->words * 4, cudaMemcpyDeviceToHost, st));
    s->touch(st);
    CPVS_CUDA(cudaStreamSynchronize(st));
    Header h{};
    std::memcpy(h.magic, kMagic, 8);
    h.version = kVersion;
    h.kind = kKindShadow;
    h.num_levels = s->num_levels;
    h.flags = s->leafmasks ? 1u : 0u;
    h.length = 1;
    h.words = s->words;
    h.checksum = fnv1a(p + kHeader, need - kHeader);
    std::memcpy(p, &h, kHeader);
    return CPVS_OK;
}

cpvs_status cpvs_shadow_deserialize(cpvs_ctx* ctx, const void* buf, uint64_t size, void* stream, cpvs_shadow** out) {
    if (!ctx || !out) return fail(CPVS_ERR_INVALID_ARG, "shadow_deserialize: null argument");
    *out = nullptr;
    Header h{};
    cpvs_status r = read_header(buf, size, kKindShadow, h);
    if (r != CPVS_OK) return r;
    if ((r = use_device(ctx)) != CPVS_OK) return r;
    const auto* p = static_cast<const unsigned char*>(buf);
    const uint64_t nc = 2ull * h.num_levels;
    std::vector<uint64_t> counts(nc);
    std::memcpy(counts.data(), p + kHeader, nc * 8);
    const unsigned char* words = p + kHeader + nc * 8;
    uint32_t root = 0;
    std::memcpy(&root, words, 4);
    DagBlock* b = nullptr;
    if ((r = upload_dag(ctx, words, h.words, (cudaStream_t)stream, &b)) != CPVS_OK) return r;
    auto* s = new cpvs_shadow;
    s->ctx = ctx;
    s->block = b;
    s->dag = b->base;
    s->words = h.words;
    s->num_levels = h.num_levels;
    s->leafmasks = (h.flags & 1u) != 0;
    s->root_mask = root;
    s->tree.assign(counts.begin(), counts.begin() + h.num_levels);
    s->uniq.assign(counts.begin() + h.num_levels, counts.end());
    *out = s;
    return CPVS_OK;
}

cpvs_status cpvs_grid_serialize(const cpvs_grid* g, void* buf, uint64_t capacity, uint64_t* size, void* stream) {
    if (!g || !g->finalized) return fail(CPVS_ERR_INVALID_ARG, "grid_serialize: grid not finalized");
    if (!little_endian()) return fail(CPVS_ERR_UNIMPLEMENTED, "serialize: big-endian hosts are not supported");
    const uint64_t ncell = (uint64_t)g->length * g->length * g->length;
    const uint64_t need = grid_bytes(g->length, g->words);
    if (size) *size = need;
    if (!buf) return CPVS_OK;
    if (capacity < need) return fail(CPVS_ERR_CAPACITY, "grid_serialize: buffer too small");
    cpvs_status r = use_device(g->ctx);
    if (r != CPVS_OK) return r;
    auto* p = static_cast<unsigned char*>(buf);
    cudaStream_t st = (cudaStream_t)stream;
    CPVS_CUDA(cudaMemcpyAsync(p + kHeader, g->cell_words, ncell * 4, cudaMemcpyDeviceToHost, st));
    CPVS_CUDA(cudaMemcpyAsync(p + kHeader + ncell * 4, g->dag, g->words * 4, cudaMemcpyDeviceToHost, st));
    g->touch(st);
    CPVS_CUDA(cudaStreamSynchronize(st));
    Header h{};
    std::memcpy(h.magic, kMagic, 8);
    h.version = kVersion;
    h.kind = kKindGrid;
    h.num_levels = g->dag_levels;
    h.flags = g->leafmasks ? 1u : 0u;
    h.length = g->length;
    h.words = g->words;
    h.checksum = fnv1a(p + kHeader, need - kHeader);
    std::memcpy(p, &h, kHeader);
    return CPVS_OK;
}

cpvs_status cpvs_grid_deserialize(cpvs_ctx* ctx, const void* buf, uint64_t size, void* stream, cpvs_grid** out) {
    if (!ctx || !out) return fail(CPVS_ERR_INVALID_ARG, "grid_deserialize: null argument");
    *out = nullptr;
    Header h{};
    cpvs_status r = read_header(buf, size, kKindGrid, h);
    if (r != CPVS_OK) return r;
    const auto* p = static_cast<const unsigned char*>(buf);
    const uint64_t ncell = (uint64_t)h.length * h.length * h.length;
    std::vector<uint32_t> cells(ncell);
    std::memcpy(cells.data(), p + kHeader, ncell * 4);
    for (uint32_t c : cells)
        if (c < 0xFFFFFFFEu && c >= h.words) return fail(CPVS_ERR_INVALID_ARG, "grid_deserialize: cell offset outside the DAG");
    if ((r = use_device(ctx)) != CPVS_OK) return r;
    cudaStream_t st = (cudaStream_t)stream;
    DagBlock* b = nullptr;
    if ((r = upload_dag(ctx, p + kHeader + ncell * 4, h.words, st, &b)) != CPVS_OK) return r;
    uint32_t* cw = nullptr;
    r = ctx->c.alloc((void**)&cw, ncell * 4, true, st);
    cudaError_t e = cudaSuccess;
    if (r == CPVS_OK) e = cudaMemcpyAsync(cw, cells.data(), ncell * 4, cudaMemcpyHostToDevice, st);
    if (r == CPVS_OK && e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (r != CPVS_OK || e != cudaSuccess) {
        if (cw) ctx->c.release(cw, ncell * 4, true, nullptr);
        block_unref(b, nullptr);
        return r != CPVS_OK ? r : cpvs::cuda_fail(e, "grid_deserialize upload");
    }
    auto* g = new cpvs_grid;
    g->ctx = ctx;
    g->length = h.length;
    g->cells.assign(ncell, nullptr);  // the cells' own shadows are not stored
    g->block = b;
    g->dag = b->base;
    g->words = h.words;
    g->cell_words = cw;
    g->dag_levels = h.num_levels;
    g->leafmasks = (h.flags & 1u) != 0;
    g->finalized = true;
    *out = g;
    return CPVS_OK;
}

}  // extern "C"
