// Test driver for include/hpdbscan.h, written the way an upstream user calls the
// HPDBSCAN class:  cluster_demo <points.f32> <n> <d> <eps> <minPts> <labels.i64>
//                  cluster_demo --h5 <file.h5> <dataset> <eps> <minPts> <labels.i64>
//                  cluster_demo --io-roundtrip <in.h5> <dataset> <out.h5>
//                  cluster_demo --io-cluster <in.h5> <dataset> <eps> <minPts> <out.h5>
//                  cluster_demo --bad-eps
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "hpdbscan.h"

int main(int argc, char** argv) {
    if (argc == 2 && std::string(argv[1]) == "--bad-eps") {
        try {
            HPDBSCAN h(-1.0f, 5);
        } catch (const std::invalid_argument& e) {
            std::cout << "invalid_argument: " << e.what() << std::endl;
            return 0;
        }
        return 1;
    }
    if (argc == 5 && std::string(argv[1]) == "--io-roundtrip") {
        // IO::read_hdf5 -> Dataset, then labels derived from the shape through IO::write_hdf5
        try {
            Dataset ds = IO::read_hdf5(argv[2], argv[3]);
            std::cout << "shape " << ds.m_shape[0] << " " << ds.m_shape[1] << " type " << ds.m_type << std::endl;
            Clusters c(static_cast<std::size_t>(ds.m_chunk[0]));
            for (std::size_t i = 0; i < c.size(); ++i) c[i] = static_cast<Cluster>(i % 7) - 3;
            IO::write_hdf5(argv[4], "CLUSTERS", c);
        } catch (const std::invalid_argument& e) {
            std::cout << "invalid_argument: " << e.what() << std::endl;
        }
        return 0;
    }
    if (argc == 7 && std::string(argv[1]) == "--io-cluster") {
        HPDBSCAN h(static_cast<float>(std::atof(argv[4])), static_cast<size_t>(std::atol(argv[5])));
        Dataset ds = IO::read_hdf5(argv[2], argv[3]);
        Clusters c = h.cluster<float>(ds, 0);
        IO::write_hdf5(argv[6], "CLUSTERS", c);
        try {
            h.cluster<double>(ds);
        } catch (const std::invalid_argument& e) {
            std::cout << "invalid_argument: " << e.what() << std::endl;
        }
        return 0;
    }
    if (argc == 7 && std::string(argv[1]) == "--h5") {
        HPDBSCAN h(static_cast<float>(std::atof(argv[4])), static_cast<size_t>(std::atol(argv[5])));
        Clusters c;
        try {
            c = h.cluster(std::string(argv[2]), std::string(argv[3]));
        } catch (const std::invalid_argument& e) {
            std::cout << "invalid_argument: " << e.what() << std::endl;
            return 0;
        } catch (const std::runtime_error& e) {
            std::cout << "runtime_error: " << e.what() << std::endl;
            return 0;
        }
        std::FILE* o = std::fopen(argv[6], "wb");
        std::vector<int64_t> out(c.begin(), c.end());
        std::fwrite(out.data(), sizeof(int64_t), out.size(), o);
        std::fclose(o);
        return 0;
    }
    if (argc != 7) return 2;
    const int n = std::atoi(argv[2]), d = std::atoi(argv[3]);
    std::vector<float> pts(static_cast<size_t>(n) * d);
    std::FILE* f = std::fopen(argv[1], "rb");
    if (!f || std::fread(pts.data(), sizeof(float), pts.size(), f) != pts.size()) return 3;
    std::fclose(f);
    HPDBSCAN h(static_cast<float>(std::atof(argv[4])), static_cast<size_t>(std::atol(argv[5])));
    Clusters c = h.cluster(pts.data(), n, d);
    std::FILE* o = std::fopen(argv[6], "wb");
    std::vector<int64_t> out(c.begin(), c.end());
    std::fwrite(out.data(), sizeof(int64_t), out.size(), o);
    std::fclose(o);
    try {
        h.cluster(std::string("/nonexistent/data.h5"), std::string("DATA"));
    } catch (const std::invalid_argument& e) {
        std::cout << "file: " << e.what() << std::endl;
    }
    return 0;
}
