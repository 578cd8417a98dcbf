// Shared definitions for the GB300 DBSCAN engine: index types, the arithmetic of
// the reference (cell coordinates and squared distances, bit for bit) and small
// device helpers.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/hpdbscan_gb300.h"

namespace hpd {

constexpr int kWarp = 32;
constexpr int kMaxDims = 16;

// Status codes returned through the C ABI.
enum Status : int {
    kOk = HPD_OK,
    kInvalid = HPD_ERR_INVALID,
    kUnsupported = HPD_ERR_UNSUPPORTED,
    kRuntime = HPD_ERR_RUNTIME,
    kGrid = HPD_ERR_GRID,
    kNoMem = HPD_ERR_NOMEM,
    kCuda = HPD_ERR_CUDA,
    kTimeout = HPD_ERR_TIMEOUT,
};

// Grid geometry shared by every kernel of one clustering call.  Cell ids are
// linearised over the "swapped" dimension order of the reference
// (spatial_index.h:133-165): dimension swapped[0] varies fastest.
struct Grid {
    int d;
    int swapped[kMaxDims];           // dimension order, fewest cells first
    unsigned long long dims[kMaxDims];   // cells per dimension, indexed by original dim
    unsigned long long stride[kMaxDims]; // stride of position s of the swapped order
    unsigned long long total;        // product of dims
};

// ------------------------------------------------------------------ distances
// Summation orders of sum_k (p_k - q_k)^2, each reproducing one compilation of the
// reference's loop (spatial_index.h:751-754) exactly.  All operations are
// explicitly rounded intrinsics, so nvcc never contracts or reassociates them.
enum DistMode : int {
    kDistGccX86 = HPD_DIST_GCC_X86,
    kDistSeq = HPD_DIST_SEQ,
    kDistSeqFma = HPD_DIST_SEQ_FMA,
    kDistGccArm = HPD_DIST_GCC_AARCH64
};

__device__ __forceinline__ float sq_(float t) { return __fmul_rn(t, t); }
__device__ __forceinline__ double sq_(double t) { return __dmul_rn(t, t); }
__device__ __forceinline__ float sub_(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double sub_(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float add_(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float fma_(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fma_(double a, double b, double c) { return __fma_rn(a, b, c); }

// t[k] = p_k - q_k already formed; returns the squared distance in mode M for a
// float/double element type with `lanes` = 4 (float) or 2 (double) partial sums
// in the GCC x86-64 order.
template <typename F, int M, int D>
__device__ __forceinline__ F fold_sq(const F* t, int d) {
    const int n = D > 0 ? D : d;
    if (M == kDistGccArm) {
        // GCC -Ofast on aarch64 (NEON): float from 4 dimensions and double from 2 on,
        // lanes (4 / 2) accumulate dimensions k = j (mod lanes) with fused
        // multiply-adds, are folded pairwise ((l0 + l1) + (l2 + l3), or l0 + l1), and
        // the remaining dimensions are added with fused multiply-adds; below that, a
        // fused running sum.
        constexpr int L = sizeof(F) == 4 ? 4 : 2;
        const int nv = n >= L ? (n & ~(L - 1)) : 0;
        F s = 0;
        int j = 0;
        if (nv) {
            F l[L];
#pragma unroll
            for (int k = 0; k < L; ++k) l[k] = sq_(t[k]);
#pragma unroll
            for (int jj = L; jj < (D > 0 ? D : kMaxDims); jj += L) {
                if (jj + L - 1 >= (D > 0 ? D : kMaxDims) || jj >= nv) break;
#pragma unroll
                for (int k = 0; k < L; ++k) l[k] = fma_(t[jj + k], t[jj + k], l[k]);
            }
            if constexpr (L == 4) s = add_(add_(l[0], l[1]), add_(l[2], l[3]));
            else s = add_(l[0], l[1]);
            j = nv;
        } else {
            s = sq_(t[0]);
            j = 1;
        }
#pragma unroll
        for (int k = 1; k < (D > 0 ? D : kMaxDims); ++k) {
            if (k < j) continue;
            if (k >= n) break;
            s = fma_(t[k], t[k], s);
        }
        return s;
    } else if (M == kDistSeq || (M == kDistGccX86 && n <= 3)) {
        F off = sq_(t[0]);
#pragma unroll
        for (int k = 1; k < (D > 0 ? D : kMaxDims); ++k) {
            if (D <= 0 && k >= n) break;
            off = add_(off, sq_(t[k]));
        }
        return off;
    } else if (M == kDistSeqFma) {
        F off = sq_(t[0]);
#pragma unroll
        for (int k = 1; k < (D > 0 ? D : kMaxDims); ++k) {
            if (D <= 0 && k >= n) break;
            off = fma_(t[k], t[k], off);
        }
        return off;
    } else if (sizeof(F) == 4) {
        // 4 lanes over the first n & ~3 dims, folded (l0 + l2), (l1 + l3), summed
        // l13 + l02; a 2-wide step adds the next two squares to the folded pair;
        // an odd last dimension is added on its own.
        const int nv = n & ~3;
        F l0 = 0, l1 = 0, l2 = 0, l3 = 0;
#pragma unroll
        for (int j = 0; j < (D > 0 ? D : kMaxDims); j += 4) {
            if (j + 3 >= (D > 0 ? D : kMaxDims) || j >= nv) break;
            l0 = add_(l0, sq_(t[j]));
            l1 = add_(l1, sq_(t[j + 1]));
            l2 = add_(l2, sq_(t[j + 2]));
            l3 = add_(l3, sq_(t[j + 3]));
        }
        F e0 = add_(l0, l2), e1 = add_(l1, l3);
        F s = add_(e1, e0);
        const int rem = n - nv;
        if (rem == 0) return s;
        int j = nv;
        if (rem >= 2) {
            e0 = add_(e0, sq_(t[j]));
            e1 = add_(e1, sq_(t[j + 1]));
            s = add_(e1, e0);
            j += 2;
            if (!(rem & 1)) return s;
        }
        return add_(s, sq_(t[j]));
    } else {
        // double: 2 lanes over the first n & ~1 dims, summed l1 + l0, odd tail added
        const int nv = n & ~1;
        F l0 = 0, l1 = 0;
#pragma unroll
        for (int j = 0; j < (D > 0 ? D : kMaxDims); j += 2) {
            if (j + 1 >= (D > 0 ? D : kMaxDims) || j >= nv) break;
            l0 = add_(l0, sq_(t[j]));
            l1 = add_(l1, sq_(t[j + 1]));
        }
        F s = add_(l1, l0);
        if (n & 1) s = add_(s, sq_(t[n - 1]));
        return s;
    }
}

// ----------------------------------------------------------- misc helpers
__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }

template <typename T>
__device__ __forceinline__ T ld_volatile(const T* p) { return *(const volatile T*)p; }

}  // namespace hpd
