// Small shared kernels and the grow-only device arena.
#include "hpd_internal.h"

namespace hpd {

__global__ void k_iota(int* p, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = i;
}

__global__ void k_fill_int(int* p, int n, int v) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = v;
}

cudaError_t Arena::reserve(size_t bytes) {
    if (bytes <= cap) return cudaSuccess;
    if (fixed) return cudaErrorMemoryAllocation;
    if (fail_next) {  // injected failure: nothing is freed or allocated
        fail_next = false;
        return cudaErrorMemoryAllocation;
    }
    if (ptr) {
        cudaError_t e = cudaFree(ptr);
        ptr = nullptr;
        cap = 0;
        if (e != cudaSuccess) return e;
    }
    size_t want = bytes + bytes / 8;  // headroom so that slightly larger calls reuse the block
    cudaError_t e = cudaMalloc(&ptr, want);
    if (e != cudaSuccess) {
        ptr = nullptr;
        cudaGetLastError();  // clear the sticky-free allocation error
        return e;
    }
    cap = want;
    return cudaSuccess;
}

Arena::~Arena() {
    if (ptr && !fixed) cudaFree(ptr);
}

}  // namespace hpd
