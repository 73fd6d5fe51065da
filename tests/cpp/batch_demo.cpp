// Uses the batched forms of include/cpvs.hpp: MinMaxHierarchy::createBatch
// over lights of different sizes, CompressedShadow::createBatch over whole
// maps and a z-tile, and CompressedShadowContainer::build over the xy tiles
// of a grid (the tiled precompute of src/DeferredRenderer.cpp:150-187 in one
// call).  Inputs and outputs are raw files so that the test driving it can
// compare every DAG with the oracle's.
//
//   batch_demo <k> <side_0> ... <side_k-1> <maps.f32> <length> <tile_side> <tiles.f32> <out-prefix>
//
// maps.f32 holds the k maps back to back, tiles.f32 the length^2 xy tiles in
// the order y*length+x.  Writes <out>.dag<j> per job (job j < k: map j whole;
// job k: z-tile 1 of 2 of map 0), <out>.meta, <out>.grid and <out>.cells.
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "cpvs.hpp"

static std::vector<float> read_floats(const char* path, size_t count) {
    std::vector<float> v(count);
    std::ifstream f(path, std::ios::binary);
    f.read(reinterpret_cast<char*>(v.data()), (std::streamsize)(count * sizeof(float)));
    if (!f) {
        std::cerr << "cannot read " << path << "\n";
        std::exit(2);
    }
    return v;
}

template <typename T>
static void write_file(const std::string& path, const T* p, size_t count) {
    std::ofstream f(path, std::ios::binary);
    f.write(reinterpret_cast<const char*>(p), (std::streamsize)(count * sizeof(T)));
}

int main(int argc, char** argv) {
    if (argc < 2) {
        std::cerr << "usage: batch_demo k side... maps length tile_side tiles out-prefix\n";
        return 2;
    }
    const size_t k = std::strtoul(argv[1], nullptr, 10);
    if (k == 0 || (size_t)argc != 7 + k) {
        std::cerr << "usage: batch_demo k side... maps length tile_side tiles out-prefix\n";
        return 2;
    }
    std::vector<size_t> sides;
    size_t total = 0;
    for (size_t i = 0; i < k; ++i) {
        sides.push_back(std::strtoul(argv[2 + i], nullptr, 10));
        total += sides.back() * sides.back();
    }
    const char* maps_path = argv[2 + k];
    const uint32_t L = (uint32_t)std::strtoul(argv[3 + k], nullptr, 10);
    const size_t tn = std::strtoul(argv[4 + k], nullptr, 10);
    const char* tiles_path = argv[5 + k];
    const std::string out = argv[6 + k];
    try {
        // the lights: one hierarchy each, every pyramid pass in one launch
        const std::vector<float> all = read_floats(maps_path, total);
        std::vector<ImageF> maps;
        size_t off = 0;
        for (size_t s : sides) {
            maps.emplace_back(s, s, 1);
            maps.back().setAll(all.data() + off);
            off += s * s;
        }
        std::vector<const ImageF*> mp;
        for (const ImageF& m : maps) mp.push_back(&m);
        auto hs = MinMaxHierarchy::createBatch(mp);

        std::ofstream meta(out + ".meta");
        meta.precision(9);  // float32 round-trips through 9 significant digits
        for (auto& h : hs) meta << h->getNumLevels() << " " << h->getMin(1, 0, 0) << " " << h->getMax(1, 0, 0) << " ";
        meta << "\n";

        // every light whole, plus the upper z-tile of the first, in one batch
        std::vector<const MinMaxHierarchy*> src;
        std::vector<cpvs_build_job> jobs;
        for (uint32_t i = 0; i < (uint32_t)k; ++i) {
            src.push_back(hs[i].get());
            jobs.push_back(cpvs_build_job{i, 0, 1});
        }
        jobs.push_back(cpvs_build_job{0, 1, 2});
        auto shadows = CompressedShadow::createBatch(src, jobs);
        for (size_t j = 0; j < shadows.size(); ++j) {
            const std::vector<unsigned>& dag = shadows[j]->getDAG();
            write_file(out + ".dag" + std::to_string(j), dag.data(), dag.size());
        }

        // the grid: its xy tiles' hierarchies in one batch, then every cell
        const std::vector<float> tall = read_floats(tiles_path, (size_t)L * L * tn * tn);
        std::vector<ImageF> tiles;
        for (size_t t = 0; t < (size_t)L * L; ++t) {
            tiles.emplace_back(tn, tn, 1);
            tiles.back().setAll(tall.data() + t * tn * tn);
        }
        std::vector<const ImageF*> tp;
        for (const ImageF& t : tiles) tp.push_back(&t);
        auto th = MinMaxHierarchy::createBatch(tp);
        std::vector<const MinMaxHierarchy*> tiles_h;
        for (auto& h : th) tiles_h.push_back(h.get());

        CompressedShadowContainer grid(L);
        grid.set(CompressedShadow::create(*th[0]), 0, 0, 0);  // replaced by the build
        grid.build(tiles_h);
        const bool released = grid.get(0, 0, 0) == nullptr;
        const uint64_t words = cpvs_grid_dag_size(grid.handle());

        // a build with the wrong number of tiles is refused and changes nothing
        bool refused = false;
        try {
            grid.build(std::vector<const MinMaxHierarchy*>(1, tiles_h[0]));
        } catch (const cpvs::Error& e) {
            refused = e.status == CPVS_ERR_INVALID_ARG;
        }
        const bool kept = cpvs_grid_dag_size(grid.handle()) == words;

        std::vector<uint32_t> dag(words), cells((size_t)L * L * L);
        cpvs::check(cpvs_grid_words(grid.handle(), dag.data(), dag.size(), cells.data(), cells.size(), nullptr));
        write_file(out + ".grid", dag.data(), dag.size());
        write_file(out + ".cells", cells.data(), cells.size());
        meta << (int)released << " " << (int)refused << " " << (int)kept << "\n";
    } catch (const std::exception& e) {
        std::cerr << e.what() << "\n";
        return 1;
    }
    return 0;
}
