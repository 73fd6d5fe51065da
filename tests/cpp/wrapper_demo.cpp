// Uses include/cpvs.hpp the way code written against the reference's classes
// does (the call shapes of test/CompressedShadowTest.cpp and of
// src/DeferredRenderer.cpp:150-235 / :333): build a hierarchy from an image,
// create a shadow, traverse points, read the DAG, wrap it in a container and
// evaluate world-space positions.  Inputs and outputs are raw files so that
// the test driving it can compare every answer with the oracle.
//
//   wrapper_demo <n> <depth.f32> <npts> <points.f32> <w> <h> <positions.f32> <matrix.f32> <filter> <out-prefix>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <vector>

#include "cpvs.hpp"

template <typename T>
static std::vector<T> read_file(const char* path, size_t count) {
    std::vector<T> v(count);
    std::ifstream f(path, std::ios::binary);
    f.read(reinterpret_cast<char*>(v.data()), (std::streamsize)(count * sizeof(T)));
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
    if (argc != 11) {
        std::cerr << "usage: wrapper_demo n depth npts points w h positions matrix filter out-prefix\n";
        return 2;
    }
    const size_t n = std::strtoul(argv[1], nullptr, 10);
    const size_t npts = std::strtoul(argv[3], nullptr, 10);
    const uint32_t w = (uint32_t)std::strtoul(argv[5], nullptr, 10), h = (uint32_t)std::strtoul(argv[6], nullptr, 10);
    const uint32_t filter = (uint32_t)std::strtoul(argv[9], nullptr, 10);
    const std::string out = argv[10];
    try {
        ImageF img(n, n, 1);
        img.setAll(read_file<float>(argv[2], n * n));
        MinMaxHierarchy mm(img);
        auto cs = CompressedShadow::create(mm);

        // getDAG / getNumLevels / getTotalVisibility
        const std::vector<unsigned>& dag = cs->getDAG();
        write_file(out + ".dag", dag.data(), dag.size());
        std::ofstream meta(out + ".meta");
        meta.precision(9);  // float32 round-trips through 9 significant digits
        meta << cs->getNumLevels() << " " << (int)cs->getTotalVisibility() << " " << mm.getNumLevels() << " "
             << mm.getMin(1, 0, 0) << " " << mm.getMax(1, 0, 0) << " " << mm.getMin(0, 1, 0) << "\n";

        // traverse, one point at a time, like the reference's unit tests
        const std::vector<float> pts = read_file<float>(argv[4], 3 * npts);
        std::vector<uint8_t> trav(npts);
        for (size_t i = 0; i < npts; ++i)
            trav[i] = (uint8_t)cs->traverse(vec3(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]));
        write_file(out + ".trav", trav.data(), trav.size());
        // tryLeafmasks that does not match the DAG's mode is refused, not misread
        if (n >= 16) {
            bool refused = false;
            try {
                cs->traverse(vec3(0.f, 0.f, 0.f), false);
            } catch (const cpvs::Error& e) {
                refused = e.status == CPVS_ERR_INVALID_ARG;
            }
            if (!refused) return 5;
        }

        // the container path: copyToGPU, setFilterSize, evaluate
        CompressedShadowContainer container(std::move(cs));
        container.copyToGPU();
        container.setFilterSize(filter);
        ImageF positions(w, h, 4);
        positions.setAll(read_file<float>(argv[7], (size_t)w * h * 4));
        mat4 m;
        const std::vector<float> mv = read_file<float>(argv[8], 16);
        float* md = const_cast<float*>(cpvs::mat4_data(m));  // column-major, as glm::value_ptr
        for (int k = 0; k < 16; ++k) md[k] = mv[k];
        cpvs::Image<uint8_t> vis(w, h, 1);
        container.evaluate(positions, m, vis);
        write_file(out + ".eval", vis.data(), (size_t)w * h);
        if (container.get(0, 0, 0) == nullptr) return 3;
        container.moveToGPU();
        if (container.get(0, 0, 0) != nullptr) return 4;
    } catch (const cpvs::Error& e) {
        std::cerr << "cpvs error " << e.status << ": " << e.what() << "\n";
        return 1;
    }
    return 0;
}
