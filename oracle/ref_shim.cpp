/*
 * extern "C" shim over the reference's own CPU shadow build and lookup.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is compiled together with the
 * reference's unmodified sources (src/CompressedShadow.cpp,
 * src/CompressedShadowUtil.cpp, src/MinMaxHierarchy.cpp, read in place from
 * the reference checkout) into oracle/_ref/libcpvs_ref.so by oracle/Makefile.
 * It is used to pin the C++ restatement (oracle/cpvs_oracle.cpp) and to write
 * the golden fixtures under tests/golden/.  Nothing in the product links it.
 */
#include "CompressedShadow.h"
#include "CompressedShadowUtil.h"
#include "MinMaxHierarchy.h"
#include "ShadowMap.h"

#include <cstdint>
#include <cstring>
#include <vector>

/* CompressedShadow::create(const ShadowMap*) references the GL read-back
 * (src/ShadowMap.cpp:23-30).  The oracle never takes that path; an empty
 * image keeps the link closed without GL. */
ImageF ShadowMap::createImageF() const { return ImageF(0, 0, 1); }

namespace {
ImageF makeImage(const float* depth, uint32_t n) {
    ImageF img(n, n, 1);
    img.setAll(depth);
    return img;
}
struct RefShadow {
    std::unique_ptr<CompressedShadow> cs;
};
}  // namespace

extern "C" {

/* MinMaxHierarchy(const ImageF&).getNumLevels()  (src/MinMaxHierarchy.h:60-62) */
int ref_num_levels(const float* depth, uint32_t n) {
    MinMaxHierarchy mm(makeImage(depth, n));
    return mm.getNumLevels();
}

/* All pyramid levels 1..numLevels-1, each (n>>L)^2 texels of (min,max),
 * written back to back in level order.  Returns numLevels. */
int ref_pyramid(const float* depth, uint32_t n, float* out) {
    MinMaxHierarchy mm(makeImage(depth, n));
    const int levels = mm.getNumLevels();
    size_t o = 0;
    for (int L = 1; L < levels; ++L) {
        const uint32_t s = n >> L;
        for (uint32_t y = 0; y < s; ++y)
            for (uint32_t x = 0; x < s; ++x) {
                out[o++] = mm.getMin(L, x, y);
                out[o++] = mm.getMax(L, x, y);
            }
    }
    return levels;
}

/* cs::createChildmask on the pyramid of `depth`, with the depth scale of
 * zTileNum z-tiles (src/CompressedShadowUtil.cpp:10-54). */
uint32_t ref_create_childmask(const float* depth, uint32_t n, uint32_t level, int x, int y, int z,
                              uint32_t zTileNum) {
    MinMaxHierarchy mm(makeImage(depth, n));
    cs::setDepthOffset(zTileNum);
    uint32_t m = cs::createChildmask(mm, level, ivec3(x, y, z));
    cs::setDepthOffset(1);
    return m;
}

/* CompressedShadow::create(minMax, zTileIndex, zTileNum) (src/CompressedShadow.cpp:49-59). */
void* ref_create(const float* depth, uint32_t n, uint32_t zTileIndex, uint32_t zTileNum) {
    MinMaxHierarchy mm(makeImage(depth, n));
    auto* h = new RefShadow;
    h->cs = CompressedShadow::create(mm, zTileIndex, zTileNum);
    return h;
}

void ref_free(void* h) { delete static_cast<RefShadow*>(h); }

size_t ref_dag_size(void* h) { return static_cast<RefShadow*>(h)->cs->getDAG().size(); }

void ref_dag_copy(void* h, uint32_t* out) {
    const auto& d = static_cast<RefShadow*>(h)->cs->getDAG();
    if (!d.empty()) std::memcpy(out, d.data(), d.size() * sizeof(uint32_t));
}

uint32_t ref_dag_num_levels(void* h) { return static_cast<RefShadow*>(h)->cs->getNumLevels(); }

int ref_total_visibility(void* h) { return static_cast<RefShadow*>(h)->cs->getTotalVisibility(); }

/* CompressedShadow::traverse(ndc, tryLeafmasks) over n points (xyz interleaved). */
void ref_traverse_ndc(void* h, const float* xyz, uint64_t n, int tryLeafmasks, uint8_t* out) {
    CompressedShadow& cs = *static_cast<RefShadow*>(h)->cs;
    for (uint64_t i = 0; i < n; ++i)
        out[i] = (uint8_t)cs.traverse(vec3(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]), tryLeafmasks != 0);
}

/* cs::mergeLevel over `numWords` words of equal-size nodes
 * (src/CompressedShadowUtil.h:154-182).  Writes the merged level to `out`
 * (numWords words, zero padded), the old->new level-relative offset of each
 * node to `mapping` (one entry per node) and returns the unique count. */
uint32_t ref_merge_level(const uint32_t* words, uint32_t numWords, uint32_t nodeSize, uint32_t* out,
                         uint32_t* mapping) {
    std::vector<uint32_t> in(words, words + numWords), res(numWords, 0);
    uint32_t left = 0;
    auto m = cs::mergeLevel(in.begin(), in.end(), res.begin(), nodeSize, &left);
    std::memcpy(out, res.data(), numWords * sizeof(uint32_t));
    for (uint32_t i = 0; i < numWords / nodeSize; ++i) mapping[i] = m[i * nodeSize];
    return left;
}

/* The container's grid_levels = (uint)log8(#cells) (src/CompressedShadowContainer.cpp:42),
 * with the reference's own log8 (src/cpvs.h:64-66). */
uint32_t ref_grid_levels(uint32_t numCells) { return (uint32_t)log8((double)numCells); }

}  // extern "C"
