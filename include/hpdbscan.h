/*
 * hpdbscan.h -- source-compatible C++ interface of the GB300 DBSCAN engine.
 *
 * Mirrors the public class of upstream include/hpdbscan.h (HPDBSCAN, lines 42-487):
 *   HPDBSCAN(float epsilon, size_t min_points)                          (:288-298)
 *   Clusters cluster(const std::string& path, const std::string& dataset[, int threads])
 *                                                                       (:300-356)
 *   template <typename T> Clusters cluster(T* data, int dim0, int dim1[, int threads])
 *                                                                       (:475-486)
 * with Clusters = std::vector<ptrdiff_t> (upstream include/constants.h:25-26), labels
 * in input order (0 noise, -k core of cluster k, +k border of cluster k) and the same
 * exceptions: std::invalid_argument for bad arguments, std::runtime_error otherwise.
 * The ten element types of the upstream explicit instantiations (src/hpdbscan.cpp:19-30)
 * are accepted; `threads` is accepted and unused (the work runs on the current GPU).
 *
 *   template <typename T> Clusters cluster(Dataset& dataset[, int threads])   (:358-473)
 * and the upstream data container and file helpers:
 *   struct Dataset  (include/dataset.h:25-59)   m_shape, m_chunk, m_offset, m_type, m_p
 *   class IO        (include/io.h:33-197)       read_hdf5(path, name), write_hdf5(path, name, clusters)
 *
 * Header-only over the C ABI (hpdbscan_gb300.h); link with -lhpdbscan_gb300 -lcudart.
 * The file overloads and IO read and write HDF5 with the library's own implementation
 * of the format (hpd_h5_read / hpd_h5_write, no libhdf5) and dispatch on the element
 * type as upstream.  Dataset::m_type holds the element type as an hpd_dtype value
 * (upstream: an HDF5 type id), since no libhdf5 types are involved; define
 * HPDBSCAN_GB300_NO_IO to leave Dataset and IO out.
 */
#ifndef HPDBSCAN_GB300_CXX_H
#define HPDBSCAN_GB300_CXX_H

#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "hpdbscan_gb300.h"

#ifndef HPDBSCAN_GB300_NO_CLUSTER_TYPES
using Cluster = std::ptrdiff_t;
using Clusters = std::vector<Cluster>;
#endif

namespace hpdbscan_gb300_detail {

template <typename T> struct dtype_of;
template <> struct dtype_of<float> { static const int value = HPD_F32; };
template <> struct dtype_of<double> { static const int value = HPD_F64; };
template <> struct dtype_of<int8_t> { static const int value = HPD_I8; };
template <> struct dtype_of<int16_t> { static const int value = HPD_I16; };
template <> struct dtype_of<int32_t> { static const int value = HPD_I32; };
template <> struct dtype_of<int64_t> { static const int value = HPD_I64; };
template <> struct dtype_of<uint8_t> { static const int value = HPD_U8; };
template <> struct dtype_of<uint16_t> { static const int value = HPD_U16; };
template <> struct dtype_of<uint32_t> { static const int value = HPD_U32; };
template <> struct dtype_of<uint64_t> { static const int value = HPD_U64; };

inline void raise(int status) {
    if (status == HPD_OK) return;
    const std::string msg = hpd_last_error();
    if (status == HPD_ERR_INVALID || status == HPD_ERR_UNSUPPORTED) throw std::invalid_argument(msg);
    throw std::runtime_error(msg);
}

inline std::size_t dtype_size(int dtype) {
    switch (dtype) {
        case HPD_I8: case HPD_U8: return 1;
        case HPD_I16: case HPD_U16: return 2;
        case HPD_F32: case HPD_I32: case HPD_U32: return 4;
        default: return 8;
    }
}

}  // namespace hpdbscan_gb300_detail

#ifndef HPDBSCAN_GB300_NO_IO
/* Points of one process: an m_shape[0] x m_shape[1] row-major array of element type
 * m_type (an hpd_dtype); m_chunk and m_offset describe the part held here, which is
 * the whole array on one GPU (upstream splits it across MPI ranks). */
struct Dataset {
    unsigned long long m_shape[2];
    unsigned long long m_chunk[2];
    unsigned long long m_offset[2];
    int m_type;
    void* m_p;

    Dataset(const unsigned long long shape[2], int type) : m_type(type), m_p(nullptr) {
        for (int k = 0; k < 2; ++k) {
            m_shape[k] = m_chunk[k] = shape[k];
            m_offset[k] = 0;
        }
        const std::size_t bytes = static_cast<std::size_t>(shape[0] * shape[1]) * hpdbscan_gb300_detail::dtype_size(type);
        m_p = std::malloc(bytes ? bytes : 1);
        if (!m_p) throw std::runtime_error("Dataset: out of host memory");
    }
    template <typename T>
    Dataset(T* data, const unsigned long long shape[2], int type) : Dataset(shape, type) {
        std::copy(data, data + shape[0] * shape[1], static_cast<T*>(m_p));
    }
    Dataset(Dataset&& other) noexcept : m_type(other.m_type), m_p(other.m_p) {
        for (int k = 0; k < 2; ++k) {
            m_shape[k] = other.m_shape[k];
            m_chunk[k] = other.m_chunk[k];
            m_offset[k] = other.m_offset[k];
        }
        other.m_p = nullptr;
    }
    Dataset(const Dataset&) = delete;
    Dataset& operator=(const Dataset&) = delete;
    ~Dataset() { std::free(m_p); }
};

class IO {
public:
    /* The 2-D dataset `dataset_name` of the HDF5 file `path`, in its own element type. */
    static Dataset read_hdf5(const std::string& path, const std::string& dataset_name) {
        void* data = nullptr;
        int64_t n = 0;
        int32_t d = 0, dtype = 0;
        hpdbscan_gb300_detail::raise(hpd_h5_read(path.c_str(), dataset_name.c_str(), &data, &n, &d, &dtype));
        const unsigned long long shape[2] = {static_cast<unsigned long long>(n), static_cast<unsigned long long>(d)};
        Dataset ds(shape, dtype);
        const std::size_t bytes = static_cast<std::size_t>(n) * static_cast<std::size_t>(d) *
                                  hpdbscan_gb300_detail::dtype_size(dtype);
        if (bytes) std::memcpy(ds.m_p, data, bytes);
        hpd_h5_free(data);
        return ds;
    }
    /* The labels as the 1-D int64 dataset `dataset_name` of `path` (created as needed). */
    static void write_hdf5(const std::string& path, const std::string& dataset_name, Clusters& clusters) {
        std::vector<int64_t> labels(clusters.begin(), clusters.end());
        hpdbscan_gb300_detail::raise(hpd_h5_write(path.c_str(), dataset_name.c_str(), labels.data(),
                                                  static_cast<int64_t>(labels.size())));
    }
};
#endif

class HPDBSCAN {
    hpd_handle* m_handle;

public:
    HPDBSCAN(float epsilon, std::size_t min_points) : m_handle(nullptr) {
        hpdbscan_gb300_detail::raise(hpd_create(epsilon, static_cast<uint64_t>(min_points), &m_handle));
    }
    ~HPDBSCAN() { hpd_destroy(m_handle); }
    HPDBSCAN(const HPDBSCAN&) = delete;
    HPDBSCAN& operator=(const HPDBSCAN&) = delete;
    HPDBSCAN(HPDBSCAN&& other) noexcept : m_handle(other.m_handle) { other.m_handle = nullptr; }

    Clusters cluster(const std::string& path, const std::string& dataset) { return cluster(path, dataset, 0); }

    Clusters cluster(const std::string& path, const std::string& dataset, int threads) {
        void* data = nullptr;
        int64_t n = 0;
        int32_t d = 0, dtype = 0;
        hpdbscan_gb300_detail::raise(hpd_h5_read(path.c_str(), dataset.c_str(), &data, &n, &d, &dtype));
        std::vector<int64_t> labels(static_cast<std::size_t>(n));
        const int status = hpd_cluster(m_handle, data, n, d, dtype, threads, labels.data());
        hpd_h5_free(data);
        hpdbscan_gb300_detail::raise(status);
        return Clusters(labels.begin(), labels.end());
    }

    template <typename T>
    Clusters cluster(T* data, int dim0, int dim1, int threads) {
        if (dim0 < 0) throw std::invalid_argument("number of points must not be negative");
        std::vector<int64_t> labels(static_cast<std::size_t>(dim0));
        hpdbscan_gb300_detail::raise(hpd_cluster(m_handle, data, dim0, dim1, hpdbscan_gb300_detail::dtype_of<T>::value,
                                                 threads, labels.data()));
        return Clusters(labels.begin(), labels.end());
    }

    template <typename T>
    Clusters cluster(T* data, int dim0, int dim1) {
        return cluster(data, dim0, dim1, 0);
    }

#ifndef HPDBSCAN_GB300_NO_IO
    /* the points of a Dataset, read as element type T (as upstream, T must match it) */
    template <typename T>
    Clusters cluster(Dataset& dataset, int threads) {
        if (dataset.m_type != hpdbscan_gb300_detail::dtype_of<T>::value)
            throw std::invalid_argument("Dataset element type differs from the requested one");
        if (dataset.m_chunk[0] > 0x7ffffffeull || dataset.m_chunk[1] > 0x7fffffffull)
            throw std::invalid_argument("number of points must be in [0, 2^31 - 2]");
        return cluster(static_cast<T*>(dataset.m_p), static_cast<int>(dataset.m_chunk[0]),
                       static_cast<int>(dataset.m_chunk[1]), threads);
    }

    template <typename T>
    Clusters cluster(Dataset& dataset) {
        return cluster<T>(dataset, 0);
    }
#endif

    /* the arithmetic of the reference build to match (see hpdbscan_gb300.h) */
    void set_arith(int cell_mode, int dist_mode) {
        hpdbscan_gb300_detail::raise(hpd_set_arith(m_handle, cell_mode, dist_mode));
    }

    /* HPD_TIE_EXACT (default) or HPD_TIE_SMALLEST_ID (see hpdbscan_gb300.h) */
    void set_tie_break(int mode) {
        hpdbscan_gb300_detail::raise(hpd_set_tie_break(m_handle, mode));
    }
};

#endif
