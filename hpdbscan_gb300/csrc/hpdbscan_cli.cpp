// hpdbscan command line tool with the flags of the upstream CLI (src/cli.cpp:42-52):
//
//   hpdbscan [-h] [-m minPoints=2] [-e epsilon=0.1] [-t threads] [-i input=data.h5]
//            [-o output=data.h5] [--input-dataset DATA] [--output-dataset CLUSTERS]
//
// Clusters the 2-D dataset of the input file on the GPU and writes the int64 labels
// (input order) to the output file, printing the phase report and summary of the
// upstream WITH_OUTPUT build (include/hpdbscan.h:213-285, 360-469,
// include/spatial_index.h:548-602).  Like upstream, errors go to stderr and the exit
// code is always 0.
//
// Files are HDF5 (read and written by the library's own implementation of the format,
// hpd_h5_read / hpd_h5_write; the labels become a 1-D int64 dataset added to the
// output file, which may be the input file, as upstream).  A file name ending in .npy
// is a NumPy array instead (2-D C-order array in; 1-D int64 labels out) and the
// dataset flag is ignored for it.
#include <cctype>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iomanip>
#include <iostream>
#include <map>
#include <set>
#include <stdexcept>
#include <string>
#include <vector>

#include "hpdbscan_gb300.h"

namespace {

struct Npy {
    int dtype = -1;
    std::vector<int64_t> shape;
    std::vector<char> data;
};

int dtype_of_descr(const std::string& descr) {
    static const std::map<std::string, int> m = {
        {"<f4", HPD_F32}, {"<f8", HPD_F64}, {"|i1", HPD_I8}, {"<i2", HPD_I16}, {"<i4", HPD_I32}, {"<i8", HPD_I64},
        {"|u1", HPD_U8}, {"<u2", HPD_U16}, {"<u4", HPD_U32}, {"<u8", HPD_U64}, {"i1", HPD_I8}, {"u1", HPD_U8}};
    auto it = m.find(descr);
    return it == m.end() ? -1 : it->second;
}

size_t dtype_size(int dtype) {
    switch (dtype) {
        case HPD_I8: case HPD_U8: return 1;
        case HPD_I16: case HPD_U16: return 2;
        case HPD_F32: case HPD_I32: case HPD_U32: return 4;
        default: return 8;
    }
}

std::string field(const std::string& header, const std::string& key) {
    const size_t k = header.find("'" + key + "'");
    if (k == std::string::npos) return "";
    size_t v = header.find(':', k);
    if (v == std::string::npos) return "";
    ++v;
    while (v < header.size() && std::isspace((unsigned char)header[v])) ++v;
    size_t e = v;
    if (header[v] == '\'') {
        e = header.find('\'', v + 1);
        return header.substr(v + 1, e - v - 1);
    }
    if (header[v] == '(') {
        e = header.find(')', v);
        return header.substr(v + 1, e - v - 1);
    }
    while (e < header.size() && header[e] != ',' && header[e] != '}') ++e;
    return header.substr(v, e - v);
}

Npy read_npy(const std::string& path) {
    std::FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) throw std::invalid_argument("Could not open " + path);
    unsigned char magic[8];
    if (std::fread(magic, 1, 8, f) != 8 || std::memcmp(magic, "\x93NUMPY", 6) != 0) {
        std::fclose(f);
        throw std::invalid_argument("Could not open " + path + " (not a .npy file)");
    }
    uint32_t hlen = 0;
    if (magic[6] == 1) {
        unsigned char b[2];
        if (std::fread(b, 1, 2, f) != 2) { std::fclose(f); throw std::runtime_error("Failed to read data"); }
        hlen = b[0] | (b[1] << 8);
    } else {
        unsigned char b[4];
        if (std::fread(b, 1, 4, f) != 4) { std::fclose(f); throw std::runtime_error("Failed to read data"); }
        hlen = b[0] | (b[1] << 8) | (b[2] << 16) | ((uint32_t)b[3] << 24);
    }
    std::string header(hlen, ' ');
    if (std::fread(&header[0], 1, hlen, f) != hlen) { std::fclose(f); throw std::runtime_error("Failed to read data"); }
    Npy out;
    out.dtype = dtype_of_descr(field(header, "descr"));
    if (out.dtype < 0) { std::fclose(f); throw std::invalid_argument("Unsupported data set type"); }
    if (field(header, "fortran_order").find("True") != std::string::npos) {
        std::fclose(f);
        throw std::invalid_argument("Data in dataset " + path + " should be a C-order matrix");
    }
    const std::string sh = field(header, "shape");
    size_t pos = 0;
    while (pos < sh.size()) {
        while (pos < sh.size() && !std::isdigit((unsigned char)sh[pos])) ++pos;
        if (pos >= sh.size()) break;
        size_t e = pos;
        while (e < sh.size() && std::isdigit((unsigned char)sh[e])) ++e;
        out.shape.push_back(std::stoll(sh.substr(pos, e - pos)));
        pos = e;
    }
    if (out.shape.size() != 2) {
        std::fclose(f);
        throw std::invalid_argument("Data in dataset " + path + " should be a matrix");
    }
    const size_t bytes = (size_t)out.shape[0] * out.shape[1] * dtype_size(out.dtype);
    out.data.resize(bytes);
    if (bytes && std::fread(out.data.data(), 1, bytes, f) != bytes) {
        std::fclose(f);
        throw std::runtime_error("Failed to read data");
    }
    std::fclose(f);
    return out;
}

void write_npy(const std::string& path, const std::vector<int64_t>& labels) {
    std::string header = "{'descr': '<i8', 'fortran_order': False, 'shape': (" + std::to_string(labels.size()) + ",), }";
    const size_t total = 10 + header.size() + 1;
    header += std::string((64 - total % 64) % 64, ' ') + "\n";
    std::FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) throw std::invalid_argument("Could not open " + path);
    const unsigned char pre[8] = {0x93, 'N', 'U', 'M', 'P', 'Y', 1, 0};
    const uint16_t hl = (uint16_t)header.size();
    const unsigned char hb[2] = {(unsigned char)(hl & 0xff), (unsigned char)(hl >> 8)};
    bool ok = std::fwrite(pre, 1, 8, f) == 8 && std::fwrite(hb, 1, 2, f) == 2 &&
              std::fwrite(header.data(), 1, header.size(), f) == header.size() &&
              std::fwrite(labels.data(), sizeof(int64_t), labels.size(), f) == labels.size();
    std::fclose(f);
    if (!ok) throw std::runtime_error("Failed to write data, target data set is probably of wrong size or type");
}

bool is_npy(const std::string& path) {
    return path.size() >= 4 && path.compare(path.size() - 4, 4, ".npy") == 0;
}

// The input as the reference reads it: HDF5 dataset (or .npy array), element type kept.
Npy read_input(const std::string& path, const std::string& dataset) {
    if (is_npy(path)) return read_npy(path);
    void* buf = nullptr;
    int64_t n = 0;
    int32_t d = 0, dtype = 0;
    const int rc = hpd_h5_read(path.c_str(), dataset.c_str(), &buf, &n, &d, &dtype);
    if (rc == HPD_ERR_INVALID || rc == HPD_ERR_UNSUPPORTED) throw std::invalid_argument(hpd_last_error());
    if (rc != HPD_OK) throw std::runtime_error(hpd_last_error());
    Npy out;
    out.dtype = dtype;
    out.shape = {n, d};
    const char* p = static_cast<const char*>(buf);
    out.data.assign(p, p + (size_t)n * (size_t)d * dtype_size(dtype));
    hpd_h5_free(buf);
    return out;
}

void write_output(const std::string& path, const std::string& dataset, const std::vector<int64_t>& labels) {
    if (is_npy(path)) return write_npy(path, labels);
    const int rc = hpd_h5_write(path.c_str(), dataset.c_str(), labels.data(), (int64_t)labels.size());
    if (rc == HPD_ERR_INVALID || rc == HPD_ERR_UNSUPPORTED) throw std::invalid_argument(hpd_last_error());
    if (rc != HPD_OK) throw std::runtime_error(hpd_last_error());
}

void usage() {
    std::cout << "Highly parallel DBSCAN clustering algorithm (GB300)\n"
              << "Usage:\n  hpdbscan [OPTION...]\n\n"
              << "  -h, --help                this help message\n"
              << "  -m, --minPoints arg       density threshold (default: 2)\n"
              << "  -e, --epsilon arg         spatial search radius (default: 0.1)\n"
              << "  -t, --threads arg         utilized threads (accepted; the work runs on the GPU)\n"
              << "  -i, --input arg           input file (default: data.h5)\n"
              << "  -o, --output arg          output file (default: data.h5)\n"
              << "      --input-dataset arg   input dataset name (default: DATA)\n"
              << "      --output-dataset arg  output dataset name (default: CLUSTERS)\n"
              << "\nFiles are HDF5; a name ending in .npy is a NumPy array (2-D points in, 1-D int64 labels out).\n";
}

}  // namespace

int main(int argc, char** argv) {
    size_t min_points = 2;
    float epsilon = 0.1f;
    int threads = 0;
    std::string input = "data.h5", output = "data.h5", in_ds = "DATA", out_ds = "CLUSTERS";
    try {
        for (int i = 1; i < argc; ++i) {
            std::string a = argv[i];
            std::string val;
            const size_t eq = a.find('=');
            if (a.rfind("--", 0) == 0 && eq != std::string::npos) {
                val = a.substr(eq + 1);
                a = a.substr(0, eq);
            }
            auto next = [&]() -> std::string {
                if (!val.empty()) return val;
                if (i + 1 >= argc) throw std::invalid_argument("Option '" + a + "' is missing an argument");
                return argv[++i];
            };
            if (a == "-h" || a == "--help") { usage(); return 0; }
            else if (a == "-m" || a == "--minPoints") min_points = std::stoull(next());
            else if (a == "-e" || a == "--epsilon") epsilon = std::stof(next());
            else if (a == "-t" || a == "--threads") threads = std::stoi(next());
            else if (a == "-i" || a == "--input") input = next();
            else if (a == "-o" || a == "--output") output = next();
            else if (a == "--input-dataset") in_ds = next();
            else if (a == "--output-dataset") out_ds = next();
            else throw std::invalid_argument("Option '" + a + "' does not exist");
        }
    } catch (const std::exception& e) {
        std::cerr << "Could not parse command line:" << std::endl << e.what() << std::endl;
        return 0;
    }
    (void)threads;

    std::vector<int64_t> labels;
    hpd_handle* h = nullptr;
    const auto t0 = std::chrono::steady_clock::now();
    try {
        if (hpd_create(epsilon, min_points, &h) != HPD_OK) throw std::invalid_argument(hpd_last_error());
        Npy data = read_input(input, in_ds);
        labels.resize((size_t)data.shape[0]);
        std::cout << std::fixed << std::setw(11) << std::setprecision(6) << std::setfill(' ');
        const int rc = hpd_cluster(h, data.data.data(), data.shape[0], (int32_t)data.shape[1], data.dtype, threads,
                                   labels.data());
        if (rc != HPD_OK) throw std::invalid_argument(hpd_last_error());
        hpd_stats st;
        hpd_get_stats(h, &st);
        auto s = [](double ms) { return ms / 1000.0; };
        // the upstream phases (hpdbscan.h:376-458, spatial_index.h:549-602) from the engine's:
        //   dimensions  per-dimension extent, grid and dimension order
        //   cells       cell id of every point + cell table (upstream: ids + histogram index)
        //   sorting     stable radix sort by cell id + gather of the coordinates
        //   DBSCAN      core test, connectivity, borders and their tie-break
        //   rules       every core resolved to its cluster root (upstream: apply_rules)
        //   order       labels scattered back to input order
        std::cout << "Computing cell space" << std::endl
                  << "\tComputing dimensions...[OK] in " << s(st.extent_ms) << std::endl
                  << "\tComputing cells...     [OK] in " << s(st.cell_ids_ms + st.cell_table_ms) << std::endl
                  << "\tSorting points...      [OK] in " << s(st.cells_sort_ms - st.cell_ids_ms) << std::endl
                  << "Clustering..." << std::endl
                  << "\tDBSCAN...              [OK] in "
                  << s(st.core_ms + st.union_ms - st.rules_ms + st.border_ms + st.tie_ms) << std::endl
                  << "\tAppyling rules...      [OK] in " << s(st.rules_ms) << std::endl
                  << "\tRecovering order...    [OK] in " << s(st.finalize_ms) << std::endl;
        std::set<int64_t> unique;
        size_t cluster_points = 0, noise_points = 0, core_points = 0;
        for (int64_t v : labels) {
            unique.insert(v < 0 ? -v : v);
            if (v == 0) ++noise_points; else ++cluster_points;
            if (v < 0) ++core_points;
        }
        std::cout << "Summary..." << std::endl
                  << "\tClusters:       " << (noise_points ? unique.size() - 1 : unique.size()) << std::endl
                  << "\tCluster points: " << cluster_points << std::endl
                  << "\tNoise points:   " << noise_points << std::endl
                  << "\tCore points:    " << core_points << std::endl
                  << "Total time: "
                  << std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count() << std::endl;
    } catch (const std::exception& e) {
        std::cerr << e.what() << std::endl;
        hpd_destroy(h);
        return 0;
    }
    hpd_destroy(h);
    try {
        write_output(output, out_ds, labels);
    } catch (const std::exception& e) {
        std::cerr << e.what() << std::endl;
    }
    return 0;
}
