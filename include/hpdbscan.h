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
 * Header-only over the C ABI (hpdbscan_gb300.h); link with -lhpdbscan_gb300 -lcudart.
 * The file overloads read the HDF5 dataset with the library's own HDF5 reader
 * (hpd_h5_read, no libhdf5) and dispatch on its element type as upstream; the
 * upstream `cluster<T>(Dataset&, int)` overload is not provided (Dataset is the
 * upstream's libhdf5-backed container).
 */
#ifndef HPDBSCAN_GB300_CXX_H
#define HPDBSCAN_GB300_CXX_H

#include <cstddef>
#include <cstdint>
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

}  // namespace hpdbscan_gb300_detail

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
