/* Header-only C++ classes over the C ABI (cpvs.h) with the reference's names
 * and call shapes, so code written against the reference's
 * CompressedShadow / MinMaxHierarchy / CompressedShadowContainer / ImageF
 * (src/CompressedShadow.h:20-125, src/MinMaxHierarchy.h:18-72,
 * src/CompressedShadowContainer.h:18-95, src/Image.h:9-69) compiles against
 * it.  The GL parts are replaced by buffers: create(const ShadowMap*) by
 * create(const ImageF&), evaluate's textures by a position image in host
 * memory and a byte per pixel out.  Differences a caller can see:
 *   - DAGs live on the GPU; getDAG() reads them back once and caches them;
 *   - traverse(position, tryLeafmasks) answers one point by a GPU lookup
 *     (batch with lookup() instead).  tryLeafmasks must match the DAG's
 *     leafmask mode: a mismatch (which the reference answers by reading leaf
 *     nodes as inner nodes, src/CompressedShadow.cpp:408-430) throws
 *     cpvs::Error with CPVS_ERR_INVALID_ARG;
 *   - errors throw cpvs::Error (the reference asserts).
 * By default the classes are also declared in the global namespace, like
 * the reference's; define CPVS_NO_GLOBAL_NAMES to keep them in cpvs::.
 * With CPVS_USE_GLM, vec3 and mat4 are glm's. */
#pragma once

#include <cstdint>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "cpvs.h"

#ifdef CPVS_USE_GLM
#include <glm/glm.hpp>
#include <glm/gtc/type_ptr.hpp>
#endif

namespace cpvs {

using uint = unsigned int;

#ifdef CPVS_USE_GLM
using vec3 = glm::vec3;
using mat4 = glm::mat4;
inline const float* mat4_data(const mat4& m) { return glm::value_ptr(m); }
#else
/* Minimal stand-ins for glm::vec3 / glm::mat4 (column-major). */
struct vec3 {
    float x = 0, y = 0, z = 0;
    vec3() = default;
    vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    explicit vec3(float s) : x(s), y(s), z(s) {}
};
inline vec3 operator*(vec3 v, float s) { return vec3(v.x * s, v.y * s, v.z * s); }
inline vec3 operator+(vec3 v, float s) { return vec3(v.x + s, v.y + s, v.z + s); }
inline vec3 operator+(vec3 a, vec3 b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
struct mat4 {
    float m[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};  // m[4*col + row]
};
inline const float* mat4_data(const mat4& m) { return m.m; }
#endif

class Error : public std::runtime_error {
public:
    Error(cpvs_status s, const std::string& msg) : std::runtime_error(msg), status(s) {}
    cpvs_status status;
};

inline void check(cpvs_status s) {
    if (s != CPVS_OK) throw Error(s, std::string(cpvs_status_string(s)) + ": " + cpvs_last_error());
}

/* The context every object below uses unless given one: device 0, opened
 * on first use, closed at exit. */
class Context {
public:
    explicit Context(int device = 0) { check(cpvs_ctx_create(device, &ctx_)); }
    ~Context() { cpvs_ctx_destroy(ctx_); }
    Context(const Context&) = delete;
    Context& operator=(const Context&) = delete;
    cpvs_ctx* get() const { return ctx_; }
    static Context& shared() {
        static Context c(0);
        return c;
    }

private:
    cpvs_ctx* ctx_ = nullptr;
};

/* 2-D host image, element (x,y,c) at (y*W+x)*C+c (src/Image.h:9-69). */
template <typename T>
class Image {
public:
    Image(size_t width, size_t height, size_t numChannels)
        : m_width(width), m_height(height), m_numChannels(numChannels), m_values(width * height * numChannels) {}
    void setAll(const T* ptr) { m_values.assign(ptr, ptr + m_width * m_height * m_numChannels); }
    void setAll(const std::vector<T>& v) { m_values.assign(v.begin(), v.end()); }
    T get(size_t x, size_t y, size_t c) const { return m_values[(y * m_width + x) * m_numChannels + c]; }
    void set(size_t x, size_t y, size_t c, T v) { m_values[(y * m_width + x) * m_numChannels + c] = v; }
    size_t getWidth() const { return m_width; }
    size_t getHeight() const { return m_height; }
    size_t getNumChannels() const { return m_numChannels; }
    const T* data() const { return m_values.data(); }
    T* data() { return m_values.data(); }

private:
    size_t m_width, m_height, m_numChannels;
    std::vector<T> m_values;
};
using ImageF = Image<float>;

/* MinMaxHierarchy(const ImageF&): the pyramid is built on the GPU; getMin /
 * getMax read its levels back on first use. */
class MinMaxHierarchy {
public:
    explicit MinMaxHierarchy(const ImageF& orig, Context& ctx = Context::shared()) : m_ctx(&ctx) {
        if (orig.getWidth() != orig.getHeight() || orig.getNumChannels() != 1)
            throw Error(CPVS_ERR_INVALID_ARG, "MinMaxHierarchy: the image must be square with one channel");
        m_depth.assign(orig.data(), orig.data() + orig.getWidth() * orig.getHeight());
        check(cpvs_hierarchy_create(ctx.get(), m_depth.data(), (uint32_t)orig.getWidth(), 0, nullptr, &m_h));
    }
    ~MinMaxHierarchy() { cpvs_hierarchy_destroy(m_h); }
    MinMaxHierarchy(const MinMaxHierarchy&) = delete;
    MinMaxHierarchy& operator=(const MinMaxHierarchy&) = delete;

    /* One hierarchy per map (cpvs_hierarchy_create_batch): every map's
     * pyramid in one launch per pass, the many-lights case.  Each image is
     * square with one channel; sides may differ. */
    static std::vector<std::unique_ptr<MinMaxHierarchy>> createBatch(const std::vector<const ImageF*>& maps,
                                                                     Context& ctx = Context::shared()) {
        std::vector<const float*> depths;
        std::vector<uint32_t> sides;
        for (const ImageF* m : maps) {
            if (!m || m->getWidth() != m->getHeight() || m->getNumChannels() != 1)
                throw Error(CPVS_ERR_INVALID_ARG,
                            "MinMaxHierarchy::createBatch: every image must be square with one channel");
            depths.push_back(m->data());
            sides.push_back((uint32_t)m->getWidth());
        }
        std::vector<std::unique_ptr<MinMaxHierarchy>> out;
        if (maps.empty()) return out;
        std::vector<cpvs_hierarchy*> hs(maps.size(), nullptr);
        check(cpvs_hierarchy_create_batch(ctx.get(), depths.data(), sides.data(), (uint32_t)maps.size(), 0, nullptr,
                                          hs.data()));
        size_t i = 0;
        try {
            out.reserve(maps.size());
            for (; i < maps.size(); ++i) out.emplace_back(new MinMaxHierarchy(hs[i], *maps[i], ctx));
        } catch (...) {
            for (; i < maps.size(); ++i) cpvs_hierarchy_destroy(hs[i]);
            throw;
        }
        return out;
    }

    float getMin(size_t level, size_t x, size_t y) const { return texel(level, x, y, 0); }
    float getMax(size_t level, size_t x, size_t y) const { return texel(level, x, y, 1); }
    int getNumLevels() const { return (int)cpvs_hierarchy_num_levels(m_h); }

    const cpvs_hierarchy* handle() const { return m_h; }
    Context& context() const { return *m_ctx; }

private:
    /* Takes ownership of h, built from orig, once constructed (createBatch
     * destroys h if this throws); the copy of orig answers level 0. */
    MinMaxHierarchy(cpvs_hierarchy* h, const ImageF& orig, Context& ctx) : m_ctx(&ctx), m_h(h) {
        m_depth.assign(orig.data(), orig.data() + orig.getWidth() * orig.getHeight());
    }
    float texel(size_t level, size_t x, size_t y, int channel) const {
        const uint32_t n = cpvs_hierarchy_size(m_h);
        if (level == 0) return m_depth[y * n + x];
        if (m_levels.empty()) m_levels.resize(getNumLevels());
        std::vector<float>& L = m_levels[level];
        const uint64_t side = n >> level;
        if (L.empty()) {
            L.resize(2 * side * side);
            check(cpvs_hierarchy_level(m_h, (uint32_t)level, L.data(), L.size(), nullptr));
        }
        return L[2 * (y * side + x) + channel];
    }
    Context* m_ctx;
    cpvs_hierarchy* m_h = nullptr;
    std::vector<float> m_depth;
    mutable std::vector<std::vector<float>> m_levels;
};

class CompressedShadowContainer;

/* CompressedShadow: one resident DAG. */
class CompressedShadow {
public:
    enum NodeVisibility { SHADOW = CPVS_SHADOW, VISIBLE = CPVS_VISIBLE, PARTIAL = CPVS_PARTIAL };

    static std::unique_ptr<CompressedShadow> create(const MinMaxHierarchy& minMax, uint zTileIndex = 0,
                                                    uint zTileNum = 1, bool leafmasks = true) {
        cpvs_shadow* s = nullptr;
        check(cpvs_shadow_create(minMax.context().get(), minMax.handle(), zTileIndex, zTileNum,
                                 leafmasks ? CPVS_FLAG_LEAFMASKS : 0u, nullptr, &s));
        return std::unique_ptr<CompressedShadow>(new CompressedShadow(s));
    }
    /* Replaces create(const ShadowMap*, ...): straight from a depth image. */
    static std::unique_ptr<CompressedShadow> create(const ImageF& depth, uint zTileIndex = 0, uint zTileNum = 1,
                                                    bool leafmasks = true, Context& ctx = Context::shared()) {
        if (depth.getWidth() != depth.getHeight() || depth.getNumChannels() != 1)
            throw Error(CPVS_ERR_INVALID_ARG, "CompressedShadow::create: the image must be square with one channel");
        cpvs_shadow* s = nullptr;
        check(cpvs_shadow_create_from_depth(ctx.get(), depth.data(), (uint32_t)depth.getWidth(), zTileIndex,
                                            zTileNum, leafmasks ? CPVS_FLAG_LEAFMASKS : 0u, nullptr, &s));
        return std::unique_ptr<CompressedShadow>(new CompressedShadow(s));
    }
    /* Many DAGs in one batch (cpvs_shadow_create_batch): DAG j is z-tile
     * jobs[j].z_tile_index of jobs[j].z_tile_num of sources[jobs[j].source],
     * equal to what create() builds for it.  The sources share one context. */
    static std::vector<std::unique_ptr<CompressedShadow>> createBatch(
        const std::vector<const MinMaxHierarchy*>& sources, const std::vector<cpvs_build_job>& jobs,
        bool leafmasks = true) {
        std::vector<std::unique_ptr<CompressedShadow>> out;
        if (jobs.empty()) return out;
        if (sources.empty()) throw Error(CPVS_ERR_INVALID_ARG, "CompressedShadow::createBatch: no sources");
        std::vector<const cpvs_hierarchy*> hs;
        for (const MinMaxHierarchy* m : sources) {
            if (!m) throw Error(CPVS_ERR_INVALID_ARG, "CompressedShadow::createBatch: null source");
            if (&m->context() != &sources[0]->context())
                throw Error(CPVS_ERR_INVALID_ARG, "CompressedShadow::createBatch: sources differ in context");
            hs.push_back(m->handle());
        }
        std::vector<cpvs_shadow*> s(jobs.size(), nullptr);
        check(cpvs_shadow_create_batch(sources[0]->context().get(), hs.data(), (uint32_t)hs.size(), jobs.data(),
                                       (uint32_t)jobs.size(), leafmasks ? CPVS_FLAG_LEAFMASKS : 0u, nullptr,
                                       s.data()));
        size_t j = 0;
        try {
            out.reserve(jobs.size());
            for (; j < jobs.size(); ++j) out.emplace_back(new CompressedShadow(s[j]));
        } catch (...) {
            for (; j < jobs.size(); ++j) cpvs_shadow_destroy(s[j]);
            throw;
        }
        return out;
    }
    ~CompressedShadow() {
        if (m_owned) cpvs_shadow_destroy(m_s);
    }
    CompressedShadow(const CompressedShadow&) = delete;
    CompressedShadow& operator=(const CompressedShadow&) = delete;

    NodeVisibility traverse(const vec3 position, bool tryLeafmasks = true) {
        if (tryLeafmasks != (cpvs_shadow_uses_leafmasks(m_s) == 1))
            throw Error(CPVS_ERR_INVALID_ARG, "CompressedShadow::traverse: tryLeafmasks must match the DAG's leafmask mode");
        const float p[3] = {position.x, position.y, position.z};
        uint32_t bits = 0;
        check(cpvs_shadow_lookup_ndc(m_s, p, 1, &bits, 0, nullptr));
        return (bits & 1u) ? VISIBLE : SHADOW;
    }
    /* n NDC points (xyz interleaved) -> ceil(n/32) words of bits (1 = lit). */
    void lookup(const float* xyz, uint64_t n, uint32_t* bits) const {
        check(cpvs_shadow_lookup_ndc(m_s, xyz, n, bits, 0, nullptr));
    }
    NodeVisibility getTotalVisibility() const { return (NodeVisibility)cpvs_shadow_total_visibility(m_s); }
    uint getNumLevels() const { return cpvs_shadow_num_levels(m_s); }
    const std::vector<uint>& getDAG() const {
        if (m_dag.empty()) {
            uint64_t n = cpvs_shadow_dag_size(m_s);
            m_dag.resize(n);
            check(cpvs_shadow_dag_words(m_s, m_dag.data(), n, &n, nullptr));
        }
        return m_dag;
    }
    const cpvs_shadow* handle() const { return m_s; }

private:
    friend class CompressedShadowContainer;
    explicit CompressedShadow(cpvs_shadow* s) : m_s(s) {}
    cpvs_shadow* m_s = nullptr;
    bool m_owned = true;  // false once a container holds the DAG
    mutable std::vector<uint> m_dag;
};

/* CompressedShadowContainer: a cubic grid of DAGs, evaluated on the GPU. */
class CompressedShadowContainer {
public:
    explicit CompressedShadowContainer(uint length, Context& ctx = Context::shared()) : m_length(length) {
        check(cpvs_grid_create(ctx.get(), length, &m_g));
        m_data.resize((size_t)length * length * length);
    }
    explicit CompressedShadowContainer(std::unique_ptr<CompressedShadow> shadow, Context& ctx = Context::shared())
        : CompressedShadowContainer(1, ctx) {
        set(std::move(shadow), 0, 0, 0);
    }
    ~CompressedShadowContainer() {
        m_data.clear();
        cpvs_grid_destroy(m_g);
    }
    CompressedShadowContainer(const CompressedShadowContainer&) = delete;
    CompressedShadowContainer& operator=(const CompressedShadowContainer&) = delete;

    void set(std::unique_ptr<CompressedShadow> shadow, uint x, uint y, uint z) {
        if (!shadow) throw Error(CPVS_ERR_INVALID_ARG, "CompressedShadowContainer::set: null shadow");
        check(cpvs_grid_set(m_g, x, y, z, shadow->m_s));
        shadow->m_owned = false;  // the grid cell owns the DAG now
        m_data[((size_t)z * m_length + y) * m_length + x] = std::move(shadow);
    }
    const CompressedShadow* get(uint x, uint y, uint z) const {
        return m_data[((size_t)z * m_length + y) * m_length + x].get();
    }
    /* Drops the host-side handles; get() then returns NULL. */
    void freeOnCPU() {
        for (auto& p : m_data) p.reset();
    }
    /* Builds every cell in one batch and finalizes the grid (cpvs_grid_build):
     * cell (x,y,z) is z-tile z of length of xyTiles[y*length+x], tiles of one
     * size.  It replaces the cells set before, so get() returns NULL for every
     * cell afterwards, as after moveToGPU().  A build refused by its checks or
     * short of memory leaves the cells as they were. */
    void build(const std::vector<const MinMaxHierarchy*>& xyTiles, bool leafmasks = true) {
        if (xyTiles.size() != (size_t)m_length * m_length)
            throw Error(CPVS_ERR_INVALID_ARG, "CompressedShadowContainer::build: needs length^2 xy tiles");
        std::vector<const cpvs_hierarchy*> hs;
        for (const MinMaxHierarchy* m : xyTiles) {
            if (!m) throw Error(CPVS_ERR_INVALID_ARG, "CompressedShadowContainer::build: null tile");
            hs.push_back(m->handle());
        }
        check(cpvs_grid_build(m_g, hs.data(), leafmasks ? CPVS_FLAG_LEAFMASKS : 0u, nullptr));
        freeOnCPU();  // the grid destroyed the cells' previous DAGs
    }
    void copyToGPU() { check(cpvs_grid_finalize(m_g, 0, nullptr)); }
    void moveToGPU() {
        check(cpvs_grid_finalize(m_g, 1, nullptr));
        freeOnCPU();
    }
    void setFilterSize(uint size) { check(cpvs_grid_set_filter_size(m_g, size)); }

    /* evaluate(positionsWS, lightViewProj, visibilities) on host buffers:
     * `positions` is width x height pixels of `floatsPerPixel` floats (xyz
     * first), `visibilities` one byte per pixel (255 lit, 0 shadowed, or the
     * filtered fraction). */
    void evaluate(const float* positions, uint width, uint height, uint floatsPerPixel, const mat4& lightViewProj,
                  uint8_t* visibilities) const {
        check(cpvs_grid_evaluate(m_g, positions, width, height, floatsPerPixel, mat4_data(lightViewProj),
                                 CPVS_EVAL_U8, visibilities, nullptr));
    }
    void evaluate(const ImageF& positions, const mat4& lightViewProj, Image<uint8_t>& visibilities) const {
        if (visibilities.getWidth() != positions.getWidth() || visibilities.getHeight() != positions.getHeight() ||
            visibilities.getNumChannels() != 1)
            throw Error(CPVS_ERR_INVALID_ARG,
                        "CompressedShadowContainer::evaluate: visibilities must have the positions' size, one channel");
        evaluate(positions.data(), (uint)positions.getWidth(), (uint)positions.getHeight(),
                 (uint)positions.getNumChannels(), lightViewProj, visibilities.data());
    }
    /* n NDC points -> bits, routed through the grid. */
    void lookup(const float* xyz, uint64_t n, uint32_t* bits) const {
        check(cpvs_grid_lookup_ndc(m_g, xyz, n, bits, 0, nullptr));
    }
    const cpvs_grid* handle() const { return m_g; }

private:
    uint m_length;
    cpvs_grid* m_g = nullptr;
    std::vector<std::unique_ptr<CompressedShadow>> m_data;
};

}  // namespace cpvs

#ifndef CPVS_NO_GLOBAL_NAMES
using cpvs::CompressedShadow;
using cpvs::CompressedShadowContainer;
using cpvs::ImageF;
using cpvs::MinMaxHierarchy;
#ifndef CPVS_USE_GLM
using cpvs::mat4;
using cpvs::vec3;
#endif
#endif
