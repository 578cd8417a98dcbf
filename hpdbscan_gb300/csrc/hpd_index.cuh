// Grid-index kernels: per-dimension extent, cell id per point, gather of the
// points into cell order, the cell table and the work items of the query kernels.
// Reference: spatial_index.h:92-216 (SpatialIndex constructor path).
#pragma once

#include <cfloat>
#include <climits>
#include <cstdint>
#include <type_traits>

#include "hpd_common.cuh"

namespace hpd {

// --------------------------------------------------------------- element traits
// F: the floating type of (x - min) / eps in the reference expression
// (double for double points, float for everything else: the integer difference is
// converted to float because eps is a float).
template <typename T> struct Elem;
template <> struct Elem<float> {
    using F = float;
    static constexpr bool kFloat = true;
    __host__ __device__ static float lowest_for_max() { return FLT_MIN; }  // numeric_limits<float>::min()
    __host__ __device__ static float highest() { return FLT_MAX; }
    __host__ __device__ static float lowest() { return -FLT_MAX; }
};
template <> struct Elem<double> {
    using F = double;
    static constexpr bool kFloat = true;
    __host__ __device__ static double lowest_for_max() { return DBL_MIN; }
    __host__ __device__ static double highest() { return DBL_MAX; }
    __host__ __device__ static double lowest() { return -DBL_MAX; }
};
// Integer element types: numeric_limits<T>::min() is the most negative value (0 for
// unsigned), so the reference's max initialiser is simply the type's minimum.
#define HPD_INT_ELEM(T, LO, HI)                                                  \
    template <> struct Elem<T> {                                                 \
        using F = float;                                                         \
        static constexpr bool kFloat = false;                                    \
        __host__ __device__ static T lowest_for_max() { return LO; }            \
        __host__ __device__ static T highest() { return HI; }                   \
        __host__ __device__ static T lowest() { return LO; }                    \
    };
HPD_INT_ELEM(int8_t, INT8_MIN, INT8_MAX)
HPD_INT_ELEM(int16_t, INT16_MIN, INT16_MAX)
HPD_INT_ELEM(int32_t, INT32_MIN, INT32_MAX)
HPD_INT_ELEM(int64_t, INT64_MIN, INT64_MAX)
HPD_INT_ELEM(uint8_t, 0, UINT8_MAX)
HPD_INT_ELEM(uint16_t, 0, UINT16_MAX)
HPD_INT_ELEM(uint32_t, 0, UINT32_MAX)
HPD_INT_ELEM(uint64_t, 0, UINT64_MAX)
#undef HPD_INT_ELEM

// (x - mn) as the reference evaluates it, in the float type F: for integer T the
// difference is taken in the promoted type (int below 32 bits, else T itself, which
// wraps) and converted to float with round-to-nearest.
template <typename T>
__host__ __device__ __forceinline__ typename Elem<T>::F diff_f(T x, T mn) {
#ifdef __CUDA_ARCH__
    if constexpr (Elem<T>::kFloat) return sub_(x, mn);
#else
    if constexpr (Elem<T>::kFloat) return x - mn;  // host code is compiled without contraction or fast-math
#endif
    else if constexpr (sizeof(T) < 4) return (float)((int)x - (int)mn);
    else if constexpr (std::is_signed<T>::value && sizeof(T) == 4) return (float)(int32_t)((uint32_t)x - (uint32_t)mn);
    else if constexpr (std::is_signed<T>::value) return (float)(int64_t)((uint64_t)x - (uint64_t)mn);
    else return (float)(T)(x - mn);
}

// EPS2 = (T)(float)(eps * eps) (hpdbscan.h:53, then the region query's T parameter)
// as GCC compiles the float -> integer conversion for the reference's target.  The
// conversions are spelled out, so that the result does not depend on the compiler
// of this library.  x86-64 (cvttss2si): a 32-bit result for types below 32 bits and
// for int32, a 64-bit result for uint32 and int64, GCC's two-step sequence around
// 2^63 for uint64; out of range gives the "integer indefinite" 0x80...0.  aarch64
// (fcvtzs / fcvtzu into a 32-bit register up to 32 bits, a 64-bit one above): saturate.
struct Eps2Conv {
    static int64_t x86_32(float f) {
        return (f > -2147483649.0f && f < 2147483648.0f) ? (int64_t)(int32_t)f : (int64_t)INT32_MIN;
    }
    static int64_t x86_64(float f) {
        return (f >= -9223372036854775808.0f && f < 9223372036854775808.0f) ? (int64_t)f : INT64_MIN;
    }
    static uint64_t x86_u64(float f) {
        if (f < 9223372036854775808.0f) return (uint64_t)x86_64(f);
        return (uint64_t)x86_64(f - 9223372036854775808.0f) ^ 0x8000000000000000ull;
    }
    static int64_t sat_s32(float f) {
        if (f != f) return 0;
        if (f >= 2147483648.0f) return INT32_MAX;
        if (f <= -2147483648.0f) return INT32_MIN;
        return (int64_t)(int32_t)f;
    }
    static uint64_t sat_u32(float f) {
        if (f != f || f <= -1.0f) return 0;
        if (f >= 4294967296.0f) return UINT32_MAX;
        return (uint64_t)(uint32_t)f;
    }
    static int64_t sat_s64(float f) {
        if (f != f) return 0;
        if (f >= 9223372036854775808.0f) return INT64_MAX;
        if (f <= -9223372036854775808.0f) return INT64_MIN;
        return (int64_t)f;
    }
    static uint64_t sat_u64(float f) {
        if (f != f || f <= -1.0f) return 0;
        if (f >= 18446744073709551616.0f) return UINT64_MAX;
        return (uint64_t)f;
    }
};

template <typename T>
inline T eps2_of(float eps, bool aarch64) {
    const float e2 = eps * eps;
    if constexpr (Elem<T>::kFloat) {
        return (T)e2;
    } else if constexpr (std::is_signed<T>::value) {
        if constexpr (sizeof(T) <= 4) return (T)(aarch64 ? Eps2Conv::sat_s32(e2) : Eps2Conv::x86_32(e2));
        else return (T)(aarch64 ? Eps2Conv::sat_s64(e2) : Eps2Conv::x86_64(e2));
    } else {
        if constexpr (sizeof(T) < 4) return (T)(aarch64 ? (int64_t)Eps2Conv::sat_u32(e2) : Eps2Conv::x86_32(e2));
        else if constexpr (sizeof(T) == 4) return (T)(aarch64 ? (int64_t)Eps2Conv::sat_u32(e2) : Eps2Conv::x86_64(e2));
        else return (T)(aarch64 ? Eps2Conv::sat_u64(e2) : Eps2Conv::x86_u64(e2));
    }
}

template <typename T>
__device__ __forceinline__ bool nonfinite(T c) {
    if constexpr (Elem<T>::kFloat) return !isfinite(c);
    else return false;
}

// floor((x - mn) / eps) with the reference's rounding, as an unsigned cell index.
template <typename T>
__device__ __forceinline__ unsigned long long cell_coord(T x, T mn, typename Elem<T>::F eps, typename Elem<T>::F recip,
                                                         int cell_mode) {
    using F = typename Elem<T>::F;
    F df = diff_f<T>(x, mn);
    F q;
    if (cell_mode == HPD_CELL_RECIP) {
        if (sizeof(F) == 4) q = (F)__fmul_rn((float)df, (float)recip);
        else q = (F)__dmul_rn((double)df, (double)recip);
    } else {
        if (sizeof(F) == 4) q = (F)__fdiv_rn((float)df, (float)eps);
        else q = (F)__ddiv_rn((double)df, (double)eps);
    }
    if (sizeof(F) == 4) return (unsigned long long)floorf((float)q);
    return (unsigned long long)floor((double)q);
}

// ---------------------------------------------------------------- min / max
// Threads of a block are laid out so that thread t always reads dimension t % d:
// the block size and the grid stride are multiples of d.
template <typename T>
__global__ void k_minmax_partial(const T* __restrict__ data, int64_t count, int d, T* __restrict__ pmin,
                                 T* __restrict__ pmax, int* __restrict__ bad) {
    extern __shared__ unsigned char smem_raw[];
    T* smin = reinterpret_cast<T*>(smem_raw);
    T* smax = smin + blockDim.x;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    T mn = Elem<T>::highest(), mx = Elem<T>::lowest();
    bool bad_value = false;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < count; e += stride) {
        T c = data[e];
        if (nonfinite(c)) bad_value = true;
        if (c < mn) mn = c;
        if (mx < c) mx = c;
    }
    if (bad_value) atomicExch(bad, 1);
    smin[threadIdx.x] = mn;
    smax[threadIdx.x] = mx;
    __syncthreads();
    if (threadIdx.x < (unsigned)d) {
        for (int t = threadIdx.x + d; t < (int)blockDim.x; t += d) {
            if (smin[t] < mn) mn = smin[t];
            if (mx < smax[t]) mx = smax[t];
        }
        pmin[(int64_t)blockIdx.x * d + threadIdx.x] = mn;
        pmax[(int64_t)blockIdx.x * d + threadIdx.x] = mx;
    }
}

template <typename T>
__global__ void __launch_bounds__(256) k_minmax_final(const T* __restrict__ pmin, const T* __restrict__ pmax, int nblocks,
                                                      int d, T* __restrict__ out /* [2d]: mins, maxs */) {
    // one block of 256 threads: every thread folds a strided share of the partial
    // results of each dimension, then a tree in shared memory (min / max are exact)
    __shared__ T smn[256], smx[256];
    for (int k = 0; k < d; ++k) {
        T mn = Elem<T>::highest(), mx = Elem<T>::lowest();
        for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
            const T a = pmin[(int64_t)b * d + k], c = pmax[(int64_t)b * d + k];
            if (a < mn) mn = a;
            if (mx < c) mx = c;
        }
        smn[threadIdx.x] = mn;
        smx[threadIdx.x] = mx;
        __syncthreads();
        for (int h = blockDim.x / 2; h > 0; h >>= 1) {
            if ((int)threadIdx.x < h) {
                if (smn[threadIdx.x + h] < smn[threadIdx.x]) smn[threadIdx.x] = smn[threadIdx.x + h];
                if (smx[threadIdx.x] < smx[threadIdx.x + h]) smx[threadIdx.x] = smx[threadIdx.x + h];
            }
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            out[k] = smn[0];
            out[d + k] = smx[0];
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------- cell ids
struct CellParams {
    Grid g;
    unsigned long long mins_raw[kMaxDims];  // per original dimension: the bytes of the T minimum
    double eps;
    double recip;
    int cell_mode;
};

template <typename T, typename K>
__global__ void k_cell_keys(const T* __restrict__ data, int64_t n, CellParams cp, K* __restrict__ keys,
                            int32_t* __restrict__ idx) {
    using F = typename Elem<T>::F;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int d = cp.g.d;
    const T* p = data + i * d;
    unsigned long long key = 0;
    for (int s = 0; s < d; ++s) {
        const int k = cp.g.swapped[s];
        T mn;
        memcpy(&mn, &cp.mins_raw[k], sizeof(T));
        key += cell_coord<T>(p[k], mn, (F)cp.eps, (F)cp.recip, cp.cell_mode) * cp.g.stride[s];
    }
    keys[i] = (K)key;
    idx[i] = (int32_t)i;
}

// sorted coordinates, one plane per dimension: coords[k * n + i] = data[perm[i] * d + k]
template <typename T>
__global__ void k_gather(const T* __restrict__ data, int64_t n, int d, const int32_t* __restrict__ perm,
                         T* __restrict__ coords) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int64_t src = (int64_t)perm[i] * d;
    for (int k = 0; k < d; ++k) coords[(int64_t)k * n + i] = data[src + k];
}

// ------------------------------------------------------------- cell table
template <typename K>
__global__ void k_cell_flags(const K* __restrict__ keys, int64_t n, uint32_t* __restrict__ flag) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    flag[i] = (i == 0 || keys[i] != keys[i - 1]) ? 1u : 0u;
}

// rank[i] = exclusive scan of flags; writes cell start / key and the per-point cell rank
template <typename K>
__global__ void k_cell_table(const K* __restrict__ keys, int64_t n, const uint32_t* __restrict__ flag,
                             uint32_t* __restrict__ rank, int32_t* __restrict__ cell_start,
                             unsigned long long* __restrict__ cell_key, int32_t* __restrict__ dense,
                             uint32_t* __restrict__ ccoord, Grid g) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t f = flag[i];
    const uint32_t r = rank[i] + f - 1u;  // inclusive rank - 1
    rank[i] = r;
    if (f) {
        cell_start[r] = (int32_t)i;
        cell_key[r] = (unsigned long long)keys[i];
        if (dense) dense[(unsigned long long)keys[i]] = (int32_t)r;
        const unsigned long long key = (unsigned long long)keys[i];
        for (int s = 0; s < g.d; ++s)  // grid coordinate along each swapped dimension
            ccoord[(size_t)s * n + r] = (uint32_t)((key / g.stride[s]) % g.dims[g.swapped[s]]);
    }
    if (i == n - 1) cell_start[r + 1] = (int32_t)n;
}

// Work items of the query kernels: chunks of up to 32 consecutive points of one
// cell.  item_flag[i] = 1 where a chunk starts.
// Also records the largest cell population in *max_cell (one atomic per warp).
static __global__ void k_item_flags(const uint32_t* __restrict__ cellrank, const int32_t* __restrict__ cell_start, int64_t n,
                             uint32_t* __restrict__ item_flag, uint32_t* __restrict__ max_cell) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t v = 0;
    if (i < n) {
        const uint32_t c = cellrank[i];
        const int32_t s = cell_start[c];
        item_flag[i] = ((i - s) & 31) == 0 ? 1u : 0u;
        if (s == (int32_t)i) v = (uint32_t)(cell_start[c + 1] - s);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    // the maximum settles early, so most warps only read it (no contended atomic)
    if ((threadIdx.x & 31) == 0 && v && v > *(volatile uint32_t*)max_cell) atomicMax(max_cell, v);
}

static __global__ void k_item_write(const uint32_t* __restrict__ item_flag, const uint32_t* __restrict__ item_pos,
                             const uint32_t* __restrict__ cellrank, int64_t n, int2* __restrict__ items) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (item_flag[i]) items[item_pos[i]] = make_int2((int)cellrank[i], (int)i);
}

}  // namespace hpd
