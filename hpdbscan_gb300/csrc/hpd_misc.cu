// Small shared kernels and the grow-only device arena.
#include <algorithm>
#include <mutex>
#include <vector>

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

namespace {
std::mutex g_tuning_mu;
std::vector<hpd_tuning_entry> g_tuning_table;
}  // namespace

hpd_tuning resolve_tuning(const hpd_tuning& own, int64_t n, int d) {
    hpd_tuning t = own;
    {
        std::lock_guard<std::mutex> lock(g_tuning_mu);
        for (const auto& e : g_tuning_table) {
            if (n <= e.max_points && (e.dims == 0 || e.dims == d)) {
                if (!t.sparse_queries) t.sparse_queries = e.tuning.sparse_queries;
                if (!t.dense_min_points) t.dense_min_points = e.tuning.dense_min_points;
                if (!t.greedy_tiles) t.greedy_tiles = e.tuning.greedy_tiles;
                break;
            }
        }
    }
    const bool large = n > kLargeInputPoints && d >= 3;
    if (!t.sparse_queries) t.sparse_queries = large ? kLargeSparseQueries : kDefaultSparseQueries;
    if (!t.dense_min_points) t.dense_min_points = large ? kLargeDenseMinPoints : kDefaultDenseMinPoints;
    if (!t.greedy_tiles) t.greedy_tiles = large ? kLargeGreedyTiles : kDefaultGreedyTiles;
    t.sparse_queries = std::min(std::max(t.sparse_queries, 0), 32);
    t.dense_min_points = std::max(t.dense_min_points, 32);
    t.greedy_tiles = std::max(t.greedy_tiles, 1);
    return t;
}

int set_tuning_table(const hpd_tuning_entry* entries, int32_t n_entries) {
    if (n_entries < 0 || n_entries > 64 || (n_entries > 0 && !entries)) return HPD_ERR_INVALID;
    std::lock_guard<std::mutex> lock(g_tuning_mu);
    g_tuning_table.assign(entries, entries + n_entries);
    return HPD_OK;
}

Arena::~Arena() {
    if (ptr && !fixed) cudaFree(ptr);
}

}  // namespace hpd
