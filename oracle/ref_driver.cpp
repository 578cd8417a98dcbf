/*
 * C entry points around the UPSTREAM HPDBSCAN headers, compiled unmodified from
 * the reference checkout by oracle/Makefile into oracle/_ref/libhpdref.so.
 *
 * Test infrastructure only: the parity tests and the CPU-baseline leg of the
 * benchmark load this library as the reference implementation; nothing in the
 * product links it.
 *
 *   hpdref_cluster  -> HPDBSCAN(eps, min_points).cluster<T>(T*, n, d, threads)
 *                      (upstream include/hpdbscan.h:288-298, 475-481)
 *   hpdref_index    -> SpatialIndex<T>(dataset, eps): the cell id and the original
 *                      index of every point in sorted order
 *                      (upstream include/spatial_index.h:528-628)
 *
 * SpatialIndex keeps its cell ids and order private; they are read through member
 * pointers formed in explicit template instantiations (where access checking does
 * not apply), so the upstream headers compile exactly as upstream ships them.
 */
#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <iomanip>
#include <iostream>
#include <limits>
#include <map>
#include <numeric>
#include <omp.h>
#include <parallel/algorithm>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "hdf5.h"

#include "hpdbscan.h"

/* member-pointer access to SpatialIndex<T> internals (see header comment) */
template <typename Tag, typename Tag::type M>
struct HpdSteal {
    friend typename Tag::type hpd_get(Tag) { return M; }
};
#define HPD_MEMBER_TAG(NAME, T, MTYPE, MEMBER)                                   \
    struct NAME {                                                                \
        typedef MTYPE SpatialIndex<T>::*type;                                    \
        friend type hpd_get(NAME);                                               \
    };                                                                           \
    template struct HpdSteal<NAME, &SpatialIndex<T>::MEMBER>;
#define HPD_TAGS(T, SUFFIX)                                                      \
    HPD_MEMBER_TAG(CellsTag_##SUFFIX, T, Cells, m_cells)                         \
    HPD_MEMBER_TAG(OrderTag_##SUFFIX, T, std::vector<size_t>, m_initial_order)   \
    HPD_MEMBER_TAG(DimsTag_##SUFFIX, T, std::vector<size_t>, m_cell_dimensions)  \
    HPD_MEMBER_TAG(SwapTag_##SUFFIX, T, std::vector<size_t>, m_swapped_dimensions) \
    template <> struct Tags<T> {                                                 \
        typedef CellsTag_##SUFFIX cells; typedef OrderTag_##SUFFIX order;        \
        typedef DimsTag_##SUFFIX dims; typedef SwapTag_##SUFFIX swap;            \
    };
template <typename T> struct Tags;
HPD_TAGS(float, f32)
HPD_TAGS(double, f64)
HPD_TAGS(int8_t, i8)
HPD_TAGS(int16_t, i16)
HPD_TAGS(int32_t, i32)
HPD_TAGS(int64_t, i64)
HPD_TAGS(uint8_t, u8)
HPD_TAGS(uint16_t, u16)
HPD_TAGS(uint32_t, u32)
HPD_TAGS(uint64_t, u64)

namespace {
thread_local std::string g_error;

template <typename T>
int run_cluster(const void* data, int n, int d, float eps, size_t min_points, int threads, int64_t* out) {
    HPDBSCAN h(eps, min_points);
    Clusters c = h.cluster<T>(const_cast<T*>(static_cast<const T*>(data)), n, d, threads);
    std::copy(c.begin(), c.end(), out);
    return 0;
}

template <typename T>
int run_index(const void* data, int n, int d, float eps, int64_t* cells, int64_t* order, int64_t* dims) {
    hsize_t shape[2] = {static_cast<hsize_t>(n), static_cast<hsize_t>(d)};
    Dataset ds(const_cast<T*>(static_cast<const T*>(data)), shape, HDF5_Types<T>::map());
    SpatialIndex<T> index(ds, eps);
    const Cells& c = index.*hpd_get(typename Tags<T>::cells());
    const std::vector<size_t>& o = index.*hpd_get(typename Tags<T>::order());
    const std::vector<size_t>& cd = index.*hpd_get(typename Tags<T>::dims());
    const std::vector<size_t>& sw = index.*hpd_get(typename Tags<T>::swap());
    for (int i = 0; i < n; ++i) {
        cells[i] = static_cast<int64_t>(c[i]);
        order[i] = static_cast<int64_t>(o[i]);
    }
    for (int k = 0; k < d; ++k) {
        dims[k] = static_cast<int64_t>(cd[k]);
        dims[d + k] = static_cast<int64_t>(sw[k]);
    }
    return 0;
}
}  // namespace

/* dtype codes shared with the product's C ABI (include/hpdbscan_gb300.h) */
#define HPDREF_DISPATCH(dtype, FN, ...)                                   \
    switch (dtype) {                                                      \
        case 0: return FN<float>(__VA_ARGS__);                            \
        case 1: return FN<double>(__VA_ARGS__);                           \
        case 2: return FN<int8_t>(__VA_ARGS__);                           \
        case 3: return FN<int16_t>(__VA_ARGS__);                          \
        case 4: return FN<int32_t>(__VA_ARGS__);                          \
        case 5: return FN<int64_t>(__VA_ARGS__);                          \
        case 6: return FN<uint8_t>(__VA_ARGS__);                          \
        case 7: return FN<uint16_t>(__VA_ARGS__);                         \
        case 8: return FN<uint32_t>(__VA_ARGS__);                         \
        case 9: return FN<uint64_t>(__VA_ARGS__);                         \
        default: g_error = "unsupported dtype"; return 2;                 \
    }

extern "C" {

const char* hpdref_last_error(void) { return g_error.c_str(); }

int hpdref_cluster(const void* data, int n, int d, int dtype, float eps, uint64_t min_points, int threads,
                   int64_t* out) {
    try {
        HPDREF_DISPATCH(dtype, run_cluster, data, n, d, eps, static_cast<size_t>(min_points), threads, out);
    } catch (const std::invalid_argument& e) {
        g_error = e.what();
        return 1;
    } catch (const std::exception& e) {
        g_error = e.what();
        return 3;
    }
}

int hpdref_index(const void* data, int n, int d, int dtype, float eps, int64_t* cells, int64_t* order,
                 int64_t* dims) {
    try {
        HPDREF_DISPATCH(dtype, run_index, data, n, d, eps, cells, order, dims);
    } catch (const std::exception& e) {
        g_error = e.what();
        return 3;
    }
}

int hpdref_max_threads(void) { return omp_get_max_threads(); }

}  // extern "C"
