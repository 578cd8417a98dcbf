/*
 * Minimal stand-in for <hdf5.h>, written for this project so that the upstream
 * HPDBSCAN headers compile without libhdf5 (which is not installed on the build
 * hosts).  Only the in-memory clustering path is usable through it:
 *
 *   - the type ids H5T_NATIVE_* and H5Tcopy / H5Tget_precision / H5Tclose are
 *     real enough for Dataset(T*, shape, type) (upstream include/dataset.h:32-43);
 *   - every file, dataset and dataspace call fails (returns -1), so the
 *     HPDBSCAN::cluster(path, dataset) overloads throw their "Could not open"
 *     errors instead of touching the disk.
 *
 * This header is test infrastructure for the oracle build only.
 */
#ifndef HPD_REF_SHIM_HDF5_H
#define HPD_REF_SHIM_HDF5_H

#include <cstddef>
#include <cstdint>

typedef int64_t hid_t;
typedef unsigned long long hsize_t;
typedef int herr_t;

typedef enum { H5T_NO_CLASS = -1, H5T_INTEGER = 0, H5T_FLOAT = 1 } H5T_class_t;
typedef enum { H5T_SGN_ERROR = -1, H5T_SGN_NONE = 0, H5T_SGN_2 = 1 } H5T_sign_t;
typedef enum { H5T_DIR_DEFAULT = 0 } H5T_direction_t;
typedef enum { H5S_SELECT_SET = 0 } H5S_seloper_t;

/* type ids: low byte = precision in bits / 8, bit 8 = signed, bit 9 = float */
#define HPD_SHIM_TYPE(bytes, is_signed, is_float) \
    ((hid_t)((bytes) | ((is_signed) << 8) | ((is_float) << 9) | (1 << 12)))
#define H5T_NATIVE_UCHAR  HPD_SHIM_TYPE(1, 0, 0)
#define H5T_NATIVE_USHORT HPD_SHIM_TYPE(2, 0, 0)
#define H5T_NATIVE_UINT   HPD_SHIM_TYPE(4, 0, 0)
#define H5T_NATIVE_ULONG  HPD_SHIM_TYPE(8, 0, 0)
#define H5T_NATIVE_SCHAR  HPD_SHIM_TYPE(1, 1, 0)
#define H5T_NATIVE_SHORT  HPD_SHIM_TYPE(2, 1, 0)
#define H5T_NATIVE_INT    HPD_SHIM_TYPE(4, 1, 0)
#define H5T_NATIVE_LONG   HPD_SHIM_TYPE(8, 1, 0)
#define H5T_NATIVE_FLOAT  HPD_SHIM_TYPE(4, 1, 1)
#define H5T_NATIVE_DOUBLE HPD_SHIM_TYPE(8, 1, 1)

#define H5E_DEFAULT    ((hid_t)0)
#define H5P_DEFAULT    ((hid_t)0)
#define H5F_ACC_RDONLY 0u
#define H5F_ACC_RDWR   1u
#define H5F_ACC_EXCL   2u

static inline hid_t  H5Tcopy(hid_t t) { return t; }
static inline herr_t H5Tclose(hid_t) { return 0; }
static inline size_t H5Tget_precision(hid_t t) { return (size_t)(t & 0xff) * 8u; }
static inline H5T_class_t H5Tget_class(hid_t t) { return (t & (1 << 9)) ? H5T_FLOAT : H5T_INTEGER; }
static inline H5T_sign_t  H5Tget_sign(hid_t t) { return (t & (1 << 8)) ? H5T_SGN_2 : H5T_SGN_NONE; }
static inline hid_t  H5Tget_native_type(hid_t t, H5T_direction_t) { return t; }

static inline herr_t H5Eget_auto(hid_t, herr_t (**f)(hid_t, void*), void** d) { *f = nullptr; *d = nullptr; return 0; }
static inline herr_t H5Eset_auto(hid_t, herr_t (*)(hid_t, void*), void*) { return 0; }

static inline hid_t  H5Fopen(const char*, unsigned, hid_t) { return -1; }
static inline hid_t  H5Fcreate(const char*, unsigned, hid_t, hid_t) { return -1; }
static inline herr_t H5Fclose(hid_t) { return -1; }
static inline hid_t  H5Dopen1(hid_t, const char*) { return -1; }
static inline hid_t  H5Dcreate1(hid_t, const char*, hid_t, hid_t, hid_t) { return -1; }
static inline hid_t  H5Dget_type(hid_t) { return -1; }
static inline hid_t  H5Dget_space(hid_t) { return -1; }
static inline herr_t H5Dread(hid_t, hid_t, hid_t, hid_t, hid_t, void*) { return -1; }
static inline herr_t H5Dwrite(hid_t, hid_t, hid_t, hid_t, hid_t, const void*) { return -1; }
static inline herr_t H5Dclose(hid_t) { return -1; }
static inline hid_t  H5Screate_simple(int, const hsize_t*, const hsize_t*) { return -1; }
static inline int    H5Sget_simple_extent_ndims(hid_t) { return -1; }
static inline int    H5Sget_simple_extent_dims(hid_t, hsize_t*, hsize_t*) { return -1; }
static inline herr_t H5Sselect_hyperslab(hid_t, H5S_seloper_t, const hsize_t*, const hsize_t*, const hsize_t*, const hsize_t*) { return -1; }
static inline herr_t H5Sclose(hid_t) { return -1; }

#endif
