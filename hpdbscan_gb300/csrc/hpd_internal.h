// Internal interfaces between the translation units of the engine.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "hpd_common.cuh"

namespace hpd {

// Sets the message of hpd_last_error() for this thread (the C ABI's error channel).
void set_last_error(const std::string& msg);

// ------------------------------------------------------------ scan / sort
int64_t scan_scratch_elems(int64_t n);
template <typename T>
void exclusive_scan(const T* in, T* out, int64_t n, T* scratch, T* total, cudaStream_t s, int* launches);

int64_t radix_counts_elems(int64_t n);
// Sorts (keys, vals) by the low `bits` bits of the keys, stably.  Returns 1 when
// the result ended up in (keys_alt, vals_alt), 0 when in (keys, vals).
template <typename K>
int radix_sort_pairs(K* keys, int32_t* vals, K* keys_alt, int32_t* vals_alt, int64_t n, int bits, uint32_t* counts,
                     uint32_t* scan_scratch, cudaStream_t s, int* launches);

// ------------------------------------------------------------ device arena
// Grow-only device buffers owned by one handle: after the first call of a given
// size no further cudaMalloc happens on that handle.
struct Arena {
    void* ptr = nullptr;
    size_t cap = 0;
    size_t used = 0;
    bool fixed = false;  // wraps memory it does not own: never allocates or frees
    bool fail_next = false;  // test hook: the next reserve that must allocate fails instead
    cudaError_t reserve(size_t bytes);
    void reset() { used = 0; }
    // Hands out the next 256-byte aligned block; the caller reserves enough for all
    // its blocks (size + 256 each) and checks overflowed() once after the last take.
    template <typename T>
    T* take(size_t count) {
        size_t off = (used + 255) & ~size_t(255);
        used = off + count * sizeof(T);
        return reinterpret_cast<T*>(static_cast<char*>(ptr) + off);
    }
    bool overflowed() const { return used > cap; }
    ~Arena();
};

struct Timers {
    cudaEvent_t ev[12] = {};
    bool ok = false;
};

constexpr int kDefaultTiePassLimit = 1 << 20;  // far beyond any real input (tens of passes)

struct Request {
    const void* d_data;  // row-major n x d of the element type, device memory
    int64_t n;
    int d;
    float eps;
    uint64_t min_points;
    int cell_mode;
    int dist_mode;
    int tie_mode = 0;    // 0: exact reference tie-break; 1: smallest cluster id
    int64_t* d_labels;   // device, input order
    cudaStream_t stream;
    bool no_dense = false;  // look cells up by binary search only (no grid-sized table)
    int tie_pass_limit = kDefaultTiePassLimit;  // relaxation passes before HPD_ERR_TIMEOUT
    bool count_pairs = false;  // diagnostic pass: count the core test's distance evaluations
    hpd_tuning tuning = {0, 0, 0};  // 0 fields: the size-class table, then the defaults
};

// Built-in tuning, and the table of hpd_set_tuning_table, resolved for one request.
constexpr int kDefaultSparseQueries = 8;
constexpr int kDefaultDenseMinPoints = 128;
constexpr int kDefaultGreedyTiles = 6;
// Above the largest size class of the tuned table (10^6 points), for three or more
// dimensions, measured on the 10M-point 3-D workload on GB300: 12.4 ms per clustering
// against 13.3 ms with the values above (labels do not depend on them).  The 50M-point
// 2-D skewed workload was slower with them (core test 28.5 -> 31.2 ms) and keeps the
// values above.
constexpr int64_t kLargeInputPoints = 1000000;
constexpr int kLargeSparseQueries = 16;
constexpr int kLargeDenseMinPoints = 64;
constexpr int kLargeGreedyTiles = 12;
hpd_tuning resolve_tuning(const hpd_tuning& own, int64_t n, int d);
int set_tuning_table(const hpd_tuning_entry* entries, int32_t n_entries);

struct RunInfo {
    int64_t n_cells = 0, n_core = 0, n_ambiguous = 0, tie_iterations = 0, core_pairs = 0;
    int launches = 0;
    float ms[7] = {0, 0, 0, 0, 0, 0, 0};  // total, index, core, union, border, tie-break, finalize
    float index_ms[3] = {0, 0, 0};          // extent, cell ids + sort, cell table
    float cell_ids_ms = 0;                  // part of index_ms[1]: the cell id kernel
    float rules_ms = 0;                     // part of ms[3]: resolving every core to its root
};

// Runs the whole pipeline for element type T.  Returns a Status and fills `err`.
template <typename T>
int run_pipeline(const Request& rq, Arena& small, Arena& main, Timers* timers, RunInfo& info, std::string& err);
template <typename T, bool WIDE>
int run_pipeline_dims(const Request& rq, Arena& small, Arena& main, Timers* timers, RunInfo& info, std::string& err);

}  // namespace hpd
