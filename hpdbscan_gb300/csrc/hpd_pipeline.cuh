// Host orchestration of one clustering call for element type T: every phase runs
// on the request's stream; the host reads back only the extent (2d values), the
// cell / work-item counts and the ambiguous-border count.
#pragma once

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>
#include <string>

#include "hpd_index.cuh"
#include "hpd_internal.h"
#include "hpd_query.cuh"
#include "hpd_core.cuh"
#include "hpd_union.cuh"
#include "hpd_dense.cuh"
#include "hpd_border.cuh"
#include "hpd_tie.cuh"

namespace hpd {

#define HPD_CU(call)                                                              \
    do {                                                                          \
        cudaError_t e_ = (call);                                                  \
        if (e_ != cudaSuccess) {                                                  \
            err = std::string(#call) + ": " + cudaGetErrorString(e_);             \
            return e_ == cudaErrorMemoryAllocation ? kNoMem : kCuda;              \
        }                                                                         \
    } while (0)

__global__ void k_iota(int* p, int n);
__global__ void k_fill_int(int* p, int n, int v);


inline unsigned blocks_for(int64_t n, int threads) { return (unsigned)((n + threads - 1) / threads); }

// Dispatch over (distance mode, compile-time dimensionality).  For d <= 3 the
// GCC x86-64 order equals the sequential order.
#define HPD_QUERY_DISPATCH(KERNEL, T, mode, d, grid, block, smem, stream, ...)                                 \
    do {                                                                                                     \
        if constexpr (WIDE) {                                                                                \
            if constexpr (!Elem<T>::kFloat) KERNEL<T, kDistSeq, -1><<<grid, block, smem, stream>>>(__VA_ARGS__); \
            else if ((mode) == kDistSeqFma) KERNEL<T, kDistSeqFma, -1><<<grid, block, smem, stream>>>(__VA_ARGS__); \
            else if ((mode) == kDistSeq) KERNEL<T, kDistSeq, -1><<<grid, block, smem, stream>>>(__VA_ARGS__); \
            else if ((mode) == kDistGccArm) KERNEL<T, kDistGccArm, -1><<<grid, block, smem, stream>>>(__VA_ARGS__); \
            else KERNEL<T, kDistGccX86, -1><<<grid, block, smem, stream>>>(__VA_ARGS__); \
        } else if constexpr (!Elem<T>::kFloat) {                                                             \
            /* integer sums wrap, so every summation order gives the same result */                          \
            if ((d) == 2) KERNEL<T, kDistSeq, 2><<<grid, block, smem, stream>>>(__VA_ARGS__);                \
            else if ((d) == 3) KERNEL<T, kDistSeq, 3><<<grid, block, smem, stream>>>(__VA_ARGS__);           \
            else KERNEL<T, kDistSeq, 0><<<grid, block, smem, stream>>>(__VA_ARGS__);                         \
        } else if ((d) == 2) {                                                                               \
            /* aarch64: float below 4 dims is the fused running sum; double d = 2 equals the plain sum */   \
            if ((mode) == kDistSeqFma || ((mode) == kDistGccArm && sizeof(T) == 4))                          \
                KERNEL<T, kDistSeqFma, 2><<<grid, block, smem, stream>>>(__VA_ARGS__);                    \
            else KERNEL<T, kDistSeq, 2><<<grid, block, smem, stream>>>(__VA_ARGS__);                         \
        } else if ((d) == 3) {                                                                               \
            if ((mode) == kDistSeqFma || ((mode) == kDistGccArm && sizeof(T) == 4))                          \
                KERNEL<T, kDistSeqFma, 3><<<grid, block, smem, stream>>>(__VA_ARGS__);                    \
            else if ((mode) == kDistGccArm) KERNEL<T, kDistGccArm, 0><<<grid, block, smem, stream>>>(__VA_ARGS__); \
            else KERNEL<T, kDistSeq, 3><<<grid, block, smem, stream>>>(__VA_ARGS__);                         \
        } else {                                                                                             \
            if ((mode) == kDistSeqFma) KERNEL<T, kDistSeqFma, 0><<<grid, block, smem, stream>>>(__VA_ARGS__); \
            else if ((mode) == kDistSeq) KERNEL<T, kDistSeq, 0><<<grid, block, smem, stream>>>(__VA_ARGS__);  \
            else if ((mode) == kDistGccArm) KERNEL<T, kDistGccArm, 0><<<grid, block, smem, stream>>>(__VA_ARGS__); \
            else KERNEL<T, kDistGccX86, 0><<<grid, block, smem, stream>>>(__VA_ARGS__);                      \
        }                                                                                                    \
    } while (0)

// Same, for kernels with a trailing bool template parameter B.  (Both expect the
// pipeline's WIDE template parameter in scope.)
#define HPD_QUERY_DISPATCH_B(KERNEL, B, T, mode, d, grid, block, smem, stream, ...)                                 \
    do {                                                                                                     \
        if constexpr (WIDE) {                                                                                \
            if constexpr (!Elem<T>::kFloat) KERNEL<T, kDistSeq, -1, B><<<grid, block, smem, stream>>>(__VA_ARGS__); \
            else if ((mode) == kDistSeqFma) KERNEL<T, kDistSeqFma, -1, B><<<grid, block, smem, stream>>>(__VA_ARGS__); \
            else if ((mode) == kDistSeq) KERNEL<T, kDistSeq, -1, B><<<grid, block, smem, stream>>>(__VA_ARGS__); \
            else if ((mode) == kDistGccArm) KERNEL<T, kDistGccArm, -1, B><<<grid, block, smem, stream>>>(__VA_ARGS__); \
            else KERNEL<T, kDistGccX86, -1, B><<<grid, block, smem, stream>>>(__VA_ARGS__); \
        } else if constexpr (!Elem<T>::kFloat) {                                                             \
            /* integer sums wrap, so every summation order gives the same result */                          \
            if ((d) == 2) KERNEL<T, kDistSeq, 2, B><<<grid, block, smem, stream>>>(__VA_ARGS__);                \
            else if ((d) == 3) KERNEL<T, kDistSeq, 3, B><<<grid, block, smem, stream>>>(__VA_ARGS__);           \
            else KERNEL<T, kDistSeq, 0, B><<<grid, block, smem, stream>>>(__VA_ARGS__);                         \
        } else if ((d) == 2) {                                                                               \
            /* aarch64: float below 4 dims is the fused running sum; double d = 2 equals the plain sum */   \
            if ((mode) == kDistSeqFma || ((mode) == kDistGccArm && sizeof(T) == 4))                          \
                KERNEL<T, kDistSeqFma, 2, B><<<grid, block, smem, stream>>>(__VA_ARGS__);                    \
            else KERNEL<T, kDistSeq, 2, B><<<grid, block, smem, stream>>>(__VA_ARGS__);                         \
        } else if ((d) == 3) {                                                                               \
            if ((mode) == kDistSeqFma || ((mode) == kDistGccArm && sizeof(T) == 4))                          \
                KERNEL<T, kDistSeqFma, 3, B><<<grid, block, smem, stream>>>(__VA_ARGS__);                    \
            else if ((mode) == kDistGccArm) KERNEL<T, kDistGccArm, 0, B><<<grid, block, smem, stream>>>(__VA_ARGS__); \
            else KERNEL<T, kDistSeq, 3, B><<<grid, block, smem, stream>>>(__VA_ARGS__);                         \
        } else {                                                                                             \
            if ((mode) == kDistSeqFma) KERNEL<T, kDistSeqFma, 0, B><<<grid, block, smem, stream>>>(__VA_ARGS__); \
            else if ((mode) == kDistSeq) KERNEL<T, kDistSeq, 0, B><<<grid, block, smem, stream>>>(__VA_ARGS__);  \
            else if ((mode) == kDistGccArm) KERNEL<T, kDistGccArm, 0, B><<<grid, block, smem, stream>>>(__VA_ARGS__); \
            else KERNEL<T, kDistGccX86, 0, B><<<grid, block, smem, stream>>>(__VA_ARGS__);                      \
        }                                                                                                    \
    } while (0)

constexpr int kFineMinPoints = 65536;  // a largest cell this big selects the finer sub-cell split
constexpr int kJumpPasses = 3;          // relaxation passes followed by a pointer-jumping sweep

template <typename T, typename K, bool WIDE>
int run_pipeline_k(const Request& rq, Arena& main, Timers* tm, RunInfo& info, std::string& err, const Grid& g,
                   const T* mins, bool dense_ok);

// WIDE: the grid has more than kStencilDirectDims dimensions; its query kernels are
// compiled separately (dimension template -1), in their own translation units.
template <typename T, bool WIDE>
int run_pipeline_dims(const Request& rq, Arena& small, Arena& main, Timers* tm, RunInfo& info, std::string& err) {
    using F = typename Elem<T>::F;
    const int64_t n = rq.n;
    const int d = rq.d;
    cudaStream_t s = rq.stream;
    info = RunInfo();
    if (tm && tm->ok) HPD_CU(cudaEventRecord(tm->ev[0], s));

    // ---- extent (spatial_index.h:99-122)
    const int64_t count = n * d;
    const int tpb = (256 / d) * d;
    int nblk = (int)std::min<int64_t>(1184, (count + tpb - 1) / tpb);
    if (nblk < 1) nblk = 1;
    HPD_CU(small.reserve(2 * (size_t)nblk * d * sizeof(T) + 2 * d * sizeof(T) + 1024));
    small.reset();
    T* pmin = small.take<T>((size_t)nblk * d);
    T* pmax = small.take<T>((size_t)nblk * d);
    T* ext = small.take<T>(2 * d);
    int* bad = small.take<int>(1);
    if (small.overflowed()) {
        err = "internal error: device buffer plan exceeds its reservation";
        return kRuntime;
    }
    HPD_CU(cudaMemsetAsync(bad, 0, sizeof(int), s));
    k_minmax_partial<T><<<nblk, tpb, 2 * tpb * sizeof(T), s>>>(static_cast<const T*>(rq.d_data), count, d, pmin, pmax, bad);
    k_minmax_final<T><<<1, 256, 0, s>>>(pmin, pmax, nblk, d, ext);
    info.launches += 2;
    if (tm && tm->ok) HPD_CU(cudaEventRecord(tm->ev[7], s));
    T h_ext[2 * kMaxDims];
    int h_bad = 0;
    HPD_CU(cudaMemcpyAsync(h_ext, ext, 2 * d * sizeof(T), cudaMemcpyDeviceToHost, s));
    HPD_CU(cudaMemcpyAsync(&h_bad, bad, sizeof(int), cudaMemcpyDeviceToHost, s));
    HPD_CU(cudaStreamSynchronize(s));
    if (h_bad) {
        err = "data contains non-finite coordinates";
        return kInvalid;
    }

    // ---- grid geometry (spatial_index.h:124-142), host arithmetic in F
    Grid g;
    memset(&g, 0, sizeof g);
    g.d = d;
    T mins[kMaxDims];
    const F epsf = (F)rq.eps;
    const F recip = (F)1 / epsf;
    unsigned long long total = 1;
    for (int k = 0; k < d; ++k) {
        mins[k] = h_ext[k];
        const T dmax = h_ext[d + k];
        const T mx = (Elem<T>::lowest_for_max() < dmax) ? dmax : Elem<T>::lowest_for_max();
        const F diff = diff_f<T>(mx, mins[k]);
        const F q = rq.cell_mode == HPD_CELL_RECIP ? diff * recip : diff / epsf;
        const F c = std::ceil(q);
        if (!(c >= 0) || c > (F)4.0e18) {
            err = "cell grid too large in dimension " + std::to_string(k);
            return kGrid;
        }
        g.dims[k] = (unsigned long long)c + 1;
        if (total > ~0ull / g.dims[k]) {
            err = "cell grid does not fit 64-bit cell ids";
            return kGrid;
        }
        total *= g.dims[k];
    }
    for (int k = 0; k < d; ++k) g.swapped[k] = k;
    for (int a = 1; a < d; ++a) {  // stable: std::sort on <= 16 elements is an insertion sort
        int v = g.swapped[a], b = a - 1;
        while (b >= 0 && g.dims[v] < g.dims[g.swapped[b]]) { g.swapped[b + 1] = g.swapped[b]; --b; }
        g.swapped[b + 1] = v;
    }
    unsigned long long acc = 1;
    for (int s2 = 0; s2 < d; ++s2) {
        g.stride[s2] = acc;
        acc *= g.dims[g.swapped[s2]];
    }
    g.total = total;
    const bool dense_ok = !rq.no_dense && total <= (1ull << 31) && total <= std::max<unsigned long long>(1ull << 26, 8ull * (unsigned long long)n);
    if (total <= (1ull << 32))
        return run_pipeline_k<T, uint32_t, WIDE>(rq, main, tm, info, err, g, mins, dense_ok);
    return run_pipeline_k<T, unsigned long long, WIDE>(rq, main, tm, info, err, g, mins, dense_ok);
}

template <typename T, typename K, bool WIDE>
int run_pipeline_k(const Request& rq, Arena& main, Timers* tm, RunInfo& info, std::string& err, const Grid& g,
                   const T* mins, bool dense_ok) {
    using F = typename Elem<T>::F;
    const int n = (int)rq.n;
    const int d = rq.d;
    cudaStream_t s = rq.stream;
    const bool timed = tm && tm->ok;
    const hpd_tuning tune = resolve_tuning(rq.tuning, rq.n, rq.d);
    int bits = 0;
    while (bits < 64 && ((g.total - 1) >> bits) != 0) ++bits;

    const int64_t ncounts = radix_counts_elems(n);
    const int64_t nscan = scan_scratch_elems(std::max<int64_t>(ncounts, n));
    size_t need = 0;
    need += 2 * (size_t)n * sizeof(K) + 2 * (size_t)n * 4;          // keys, vals (+ alternates)
    need += (size_t)n * d * sizeof(T);                               // sorted coordinate planes
    need += 4 * (size_t)n * 4;                                       // flag, rank, item flag, item pos
    need += ((size_t)n + 1) * 4 + (size_t)n * 8;                     // cell start, cell key
    need += dense_ok ? (size_t)g.total * 4 : 0;                      // dense cell lookup
    need += (size_t)d * n * 4;                                       // cell grid coordinates
    need += (size_t)n * 8;                                           // items
    need += (size_t)n + 6 * (size_t)n * 4;                           // core, tmax, tlow, parent, broot, lm1, amb
    need += (size_t)n * 4 + (size_t)n;                               // cell rep, cell flags
    need += 9 * (size_t)n * 4;                                       // dirty / schedule stamps, dirty list, work lists, cell / item min, item flags
    // dense cells: sub-cells per dimension (0: path off), see k_dense_assign
    int dense_k = 0;
    // (squared distances near the float subnormal range would void the rounding margins)
    if (Elem<T>::kFloat && d <= 4 && (double)rq.eps * (double)rq.eps >= 1e-30) {
        double err = 0;
        for (int k = 0; k < d; ++k)
            err = std::max(err, (std::fabs((double)mins[k]) + (double)g.dims[k] * (double)rq.eps) * std::ldexp(1.0, -20));
        for (int kk = 2; kk <= 3 && !dense_k; ++kk) {
            int groups = 1;
            for (int k = 0; k < d; ++k) groups *= kk;
            if (groups <= kDenseMaxGroups && std::sqrt((double)d) * ((double)rq.eps / kk + 4 * err) <= 0.95 * (double)rq.eps)
                dense_k = kk;
        }
    }
    // a grid whose largest cell holds >= kFineMinPoints points splits dense cells finer
    // (decided once the cell table exists); the tables are sized for either split
    const int fine_k = dense_k == 0 ? 0 : std::max(dense_k, d == 1 ? 32 : d == 2 ? 8 : d == 3 ? 4 : 3);
    int dense_groups = 1, groups_cap = 1;
    for (int k = 0; k < d; ++k) {
        dense_groups *= std::max(dense_k, 1);
        groups_cap *= std::max(fine_k, 1);
    }
    const int64_t dense_max = (int64_t)n / tune.dense_min_points + 1;
    need += 3 * (size_t)n * 4 + (size_t)dense_max * (3 * groups_cap + 2) * 4;  // dense-cell tables
    need += dense_k ? (size_t)dense_max * groups_cap * 2 * d * sizeof(T) : 0;   // sub-cell boxes
    need += dense_k ? (size_t)n * d * sizeof(T) : 0;                 // dense cells' coordinates by sub-cell
    need += (size_t)n * 4;                                           // second ambiguous list
    const int chunk_cap = n / 4 + 1024;
    need += (size_t)chunk_cap * 16;                                  // tie-break chunk tasks
    need += (size_t)ncounts * 4 + (size_t)nscan * 8 + 256;           // radix counts, scan scratch, totals, flags
    need += 64 * 256;                                                // alignment of up to 64 blocks
    HPD_CU(main.reserve(need));
    main.reset();
    K* keys = main.take<K>(n);
    K* keys_alt = main.take<K>(n);
    int32_t* vals = main.take<int32_t>(n);
    int32_t* vals_alt = main.take<int32_t>(n);
    T* coords = main.take<T>((size_t)n * d);
    uint32_t* flag = main.take<uint32_t>(n);
    uint32_t* rank = main.take<uint32_t>(n);
    uint32_t* iflag = main.take<uint32_t>(n);
    uint32_t* ipos = main.take<uint32_t>(n);
    int32_t* cell_start = main.take<int32_t>((size_t)n + 1);
    unsigned long long* cell_key = main.take<unsigned long long>(n);
    int32_t* dense = dense_ok ? main.take<int32_t>(g.total) : nullptr;
    uint32_t* ccoord = main.take<uint32_t>((size_t)d * n);
    int2* items = main.take<int2>(n);
    uint8_t* core = main.take<uint8_t>(n);
    int* tmax = main.take<int>(n);
    int* tlow = main.take<int>(n);
    int* parent = main.take<int>(n);
    int* broot = main.take<int>(n);
    int* lm1 = main.take<int>(n);
    int* amb = main.take<int>(n);
    int* amb2 = main.take<int>(n);
    int* cell_rep = main.take<int>(n);
    uint8_t* cell_flags = main.take<uint8_t>(n);
    int* dirty_gen = main.take<int>(n);
    int* sched_gen = main.take<int>(n);
    int* dlist = main.take<int>(n);
    int* wl0 = main.take<int>(n);
    int* wl1 = main.take<int>(n);
    int* cell_min_l = main.take<int>(n);
    int* item_min_l = main.take<int>(n);
    uint32_t* item_flag = main.take<uint32_t>(n);
    int* dense_id = main.take<int>(n);
    int* dense_cells = main.take<int>(dense_max);
    int* dense_grp = main.take<int>((size_t)dense_max * (groups_cap + 1));
    int* dense_rep = main.take<int>((size_t)dense_max * groups_cap);
    int* dense_cur = main.take<int>((size_t)dense_max * groups_cap);
    int* dense_sec = main.take<int>(n);
    int* dense_gidx = main.take<int>(n);
    T* dense_box = main.take<T>(dense_k ? (size_t)dense_max * groups_cap * 2 * d : 0);
    T* dense_coords = main.take<T>(dense_k ? (size_t)n * d : 0);
    uint32_t* item_pos = main.take<uint32_t>(n);
    int4* chunks = main.take<int4>(chunk_cap);
    uint32_t* counts = main.take<uint32_t>(ncounts);
    uint32_t* scan32 = main.take<uint32_t>(2 * nscan);
    uint32_t* totals = main.take<uint32_t>(4);   // cells, items, largest cell
    int* flags_dev = main.take<int>(32);          // list counters, [6] cores, [8..11] trace, [12] dense cells,
                                                  // [13..15] range-check record, [16..17] pair count,
                                                  // [18] tie-break chunk tasks
    if (main.overflowed()) {
        err = "internal error: device buffer plan exceeds its reservation";
        return kRuntime;
    }
    int* guard = flags_dev + 13;
    HPD_CU(cudaMemsetAsync(flags_dev, 0, 32 * sizeof(int), s));

    // ---- cell ids (spatial_index.h:144-165)
    CellParams cp;
    memset(&cp, 0, sizeof cp);
    cp.g = g;
    for (int k = 0; k < d; ++k) memcpy(&cp.mins_raw[k], &mins[k], sizeof(T));
    cp.eps = (double)(F)rq.eps;
    cp.recip = (double)((F)1 / (F)rq.eps);
    cp.cell_mode = rq.cell_mode;
    const T* data = static_cast<const T*>(rq.d_data);
    k_cell_keys<T, K><<<blocks_for(n, 256), 256, 0, s>>>(data, n, cp, keys, vals);
    info.launches += 1;
    if (timed) HPD_CU(cudaEventRecord(tm->ev[9], s));

    // ---- stable sort by cell id (spatial_index.h:184-216)
    K* skeys = keys;
    int32_t* perm = vals;
    if (bits > 0) {
        const int alt = radix_sort_pairs<K>(keys, vals, keys_alt, vals_alt, n, bits, counts, scan32, s, &info.launches);
        if (alt) { skeys = keys_alt; perm = vals_alt; }
    }
    k_gather<T><<<blocks_for(n, 256), 256, 0, s>>>(data, n, d, perm, coords);
    if (timed) HPD_CU(cudaEventRecord(tm->ev[8], s));

    // ---- cell table (spatial_index.h:167-182) and work items
    if (dense) HPD_CU(cudaMemsetAsync(dense, 0xff, (size_t)g.total * 4, s));
    k_cell_flags<K><<<blocks_for(n, 256), 256, 0, s>>>(skeys, n, flag);
    exclusive_scan<uint32_t>(flag, rank, n, scan32, totals + 0, s, &info.launches);
    k_cell_table<K><<<blocks_for(n, 256), 256, 0, s>>>(skeys, n, flag, rank, cell_start, cell_key, dense, ccoord, g);
    HPD_CU(cudaMemsetAsync(totals + 2, 0, sizeof(uint32_t), s));
    k_item_flags<<<blocks_for(n, 256), 256, 0, s>>>(rank, cell_start, n, iflag, totals + 2);
    exclusive_scan<uint32_t>(iflag, ipos, n, scan32, totals + 1, s, &info.launches);
    k_item_write<<<blocks_for(n, 256), 256, 0, s>>>(iflag, ipos, rank, n, items);
    info.launches += 5;
    uint32_t h_tot[3];
    HPD_CU(cudaMemcpyAsync(h_tot, totals, 3 * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    HPD_CU(cudaStreamSynchronize(s));
    const int m = (int)h_tot[0];
    const int n_items = (int)h_tot[1];
    if (dense_k > 0 && h_tot[2] >= (uint32_t)kFineMinPoints) {
        dense_k = fine_k;
        dense_groups = groups_cap;
    }
    // cells of >= kPruneMinPoints points get sub-cell boxes and the pruned query paths
    const bool prune = dense_k > 0 && h_tot[2] >= (uint32_t)kPruneMinPoints;
    info.n_cells = m;
    if (timed) HPD_CU(cudaEventRecord(tm->ev[1], s));

    QueryArgs<T> a;
    memset(&a, 0, sizeof a);
    a.coords = coords;
    a.n = n;
    a.g = g;
    a.ct.start = cell_start;
    a.ct.key = cell_key;
    a.ct.dense = dense;
    a.ct.m = m;
    a.ct.ccoord = ccoord;
    a.ct.pitch = n;
    a.ct.guard = guard;
    a.guard = guard;
    a.eps2 = eps2_of<T>(rq.eps, rq.dist_mode == HPD_DIST_GCC_AARCH64);  // const float EPS2 = eps * eps (hpdbscan.h:53), as T
    a.items = items;
    a.n_items = n_items;
    a.min_points = (int)std::min<uint64_t>(rq.min_points, (uint64_t)n + 1);
    a.core = core;
    a.parent = parent;
    a.broot = broot;
    a.amb = amb;
    a.n_amb = flags_dev + 0;
    a.tmax = tmax;
    a.tlow = tlow;
    a.lm1 = lm1;
    a.changed = flags_dev + 1;
    a.cellrank = rank;
    a.cell_rep = cell_rep;
    a.cell_flags = cell_flags;
    a.sparse_queries = tune.sparse_queries;
    a.greedy_tiles = tune.greedy_tiles;
    const int mode = rq.dist_mode;
    const unsigned qgrid = blocks_for(n_items, 4);
    const size_t qsmem = 4 * ((size_t)tile_stride(d) * 32 * sizeof(T) + 32 * sizeof(int));

    // ---- dense cells: sub-cells (certified cliques) for the core test and the unions
    HPD_CU(cudaMemsetAsync(cell_flags, kCellUniform, m, s));
    DenseArgs da;
    memset(&da, 0, sizeof da);
    if (dense_k > 0) {
        da.k = dense_k;
        da.groups = 1;
        for (int k = 0; k < d; ++k) da.groups *= dense_k;
        da.min_points = tune.dense_min_points;
        da.scale = (double)dense_k / (double)rq.eps;
        for (int k = 0; k < d; ++k) da.mins_d[k] = (double)mins[k];
        da.dense_id = dense_id;
        da.cells = dense_cells;
        da.n_dense = flags_dev + 12;
        da.grp = dense_grp;
        da.grp_rep = dense_rep;
        da.sec = dense_sec;
        da.gidx = dense_gidx;
        da.box = dense_box;
        da.coords = dense_coords;
        da.cur = dense_cur;
        da.boxes = prune ? 1 : 0;
        HPD_CU(cudaMemsetAsync(da.n_dense, 0, sizeof(int), s));
        k_dense_list<<<blocks_for(m, 256), 256, 0, s>>>(cell_start, m, da);
        k_dense_init<T><<<blocks_for(dense_max * da.groups, 256), 256, 0, s>>>(a, da);
        k_dense_assign<T><<<blocks_for(n, 256), 256, 0, s>>>(a, da);
        k_dense_offsets<T><<<blocks_for(dense_max, 4), 128, 0, s>>>(a, da);
        k_dense_scatter<T><<<blocks_for(n, 256), 256, 0, s>>>(a, da);
        if (prune) k_mark_near_big<T, WIDE ? -1 : 0><<<blocks_for(dense_max, 4), 128, 0, s>>>(a, da);
        a.dense_id = dense_id;
        a.dense_grp = dense_grp;
        a.dense_gidx = dense_gidx;
        a.dense_groups = da.groups;
        a.dense_sec = dense_sec;
        a.dense_box = dense_box;
        a.dense_coords = dense_coords;
        a.dense_rep = dense_rep;
        info.launches += prune ? 6 : 5;
    }

    // ---- core test (hpdbscan.h:72-78)
    if (rq.min_points <= 1) {
        HPD_CU(cudaMemsetAsync(core, 1, n, s));
    } else if (rq.min_points > (uint64_t)n) {
        HPD_CU(cudaMemsetAsync(core, 0, n, s));
    } else {
        if (rq.count_pairs) {
            // diagnostic pass: the same core test, counting its distance evaluations
            a.pair_count = reinterpret_cast<unsigned long long*>(flags_dev + 16);
            if (prune) HPD_QUERY_DISPATCH_B(k_core, kCorePrune | kCoreCount, T, mode, d, qgrid, 128, qsmem, s, a);
            HPD_QUERY_DISPATCH_B(k_core, kCoreCount, T, mode, d, qgrid, 128, qsmem, s, a);
        } else {
            if (prune) HPD_QUERY_DISPATCH_B(k_core, kCorePrune, T, mode, d, qgrid, 128, qsmem, s, a);
            HPD_QUERY_DISPATCH_B(k_core, 0, T, mode, d, qgrid, 128, qsmem, s, a);
        }
        info.launches += prune ? 2 : 1;
    }
    if (timed) HPD_CU(cudaEventRecord(tm->ev[2], s));

    // ---- core-core connectivity
    k_iota<<<blocks_for(n, 256), 256, 0, s>>>(parent, n);
    if (dense_k > 0) {
        k_dense_rep<T><<<blocks_for(n, 256), 256, 0, s>>>(a, da);
        k_dense_link<T><<<blocks_for(n, 256), 256, 0, s>>>(a, da);
        HPD_QUERY_DISPATCH(k_dense_pairs, T, mode, d, blocks_for(dense_max, 4), 128, 0, s, a, da);
        info.launches += 3;
    }
    HPD_QUERY_DISPATCH(k_union_small_cells, T, mode, d, blocks_for(m, 4), 128, qsmem, s, a);
    HPD_QUERY_DISPATCH(k_union_intra, T, mode, d, qgrid, 128, qsmem, s, a);
    info.launches += 1;
    k_fill_int<<<blocks_for(m, 256), 256, 0, s>>>(cell_rep, m, kNoCore);
    k_cell_rep<<<blocks_for(n, 256), 256, 0, s>>>(core, parent, rank, n, cell_rep);
    k_cell_uniform<<<blocks_for(n, 256), 256, 0, s>>>(core, parent, rank, n, cell_rep, cell_flags);
    HPD_QUERY_DISPATCH(k_union_cells, T, mode, d, blocks_for(m, 4), 128, 0, s, a);
    HPD_QUERY_DISPATCH(k_union_cross, T, mode, d, qgrid, 128, qsmem, s, a);
    if (timed) HPD_CU(cudaEventRecord(tm->ev[10], s));
    k_compress<<<blocks_for(n, 256), 256, 0, s>>>(parent, core, n, flags_dev + 6);
    info.launches += 8;
    if (timed) HPD_CU(cudaEventRecord(tm->ev[3], s));

    // ---- borders
    HPD_CU(cudaMemsetAsync(flags_dev, 0, 6 * sizeof(int), s));
    if (prune) {
        HPD_QUERY_DISPATCH_B(k_border, true, T, mode, d, qgrid, 128, qsmem, s, a);
        info.launches += 1;
    }
    HPD_QUERY_DISPATCH_B(k_border, false, T, mode, d, qgrid, 128, qsmem, s, a);
    info.launches += 1;
    int h_counts[7];  // [0] ambiguous borders, [6] cores
    HPD_CU(cudaMemcpyAsync(h_counts, flags_dev, sizeof h_counts, cudaMemcpyDeviceToHost, s));
    HPD_CU(cudaStreamSynchronize(s));
    const int h_amb = h_counts[0];
    info.n_ambiguous = h_amb;
    info.n_core = h_counts[6];
    if (timed) HPD_CU(cudaEventRecord(tm->ev[4], s));

    // ---- tie-break for borders next to several clusters
    if (h_amb > 0 && rq.tie_mode != 0) {
        a.amb = amb;
        a.n_amb = flags_dev + 0;
        HPD_QUERY_DISPATCH(k_tie_min_root, T, mode, d, blocks_for(h_amb, 4), 128, 0, s, a);
        info.launches += 1;
    } else if (h_amb > 0) {
        const bool trace = getenv("HPD_TIE_TRACE") != nullptr;
        unsigned long long* tcount = reinterpret_cast<unsigned long long*>(flags_dev + 8);
        a.trace_counts = trace ? tcount : nullptr;
        k_tie_init<<<blocks_for(n, 256), 256, 0, s>>>(core, lm1, n);
        HPD_CU(cudaMemsetAsync(dirty_gen, 0, (size_t)m * sizeof(int), s));
        HPD_CU(cudaMemsetAsync(sched_gen, 0, (size_t)m * sizeof(int), s));
        info.launches += 1;
        a.dirty_gen = dirty_gen;
        a.sched_gen = sched_gen;
        a.dlist = dlist;
        a.n_dlist = flags_dev + 1;
        a.ipos = ipos;
        a.cell_min_l = cell_min_l;
        a.item_min_l = item_min_l;
        a.item_flag = item_flag;
        a.ticket = flags_dev + 5;
        a.chunks = chunks;
        a.n_chunks = flags_dev + 18;
        a.chunk_cap = chunk_cap;
        HPD_CU(cudaMemsetAsync(item_flag, 0, (size_t)n_items * sizeof(uint32_t), s));
        a.gen = 0;
        // ping-pong lists of undecided borders (amb, amb2) and of work items (wl0, wl1)
        int* lists[2] = {amb, amb2};
        int* counts[2] = {flags_dev + 0, flags_dev + 2};
        int* wls[2] = {wl0, wl1};
        int* wcounts[2] = {flags_dev + 3, flags_dev + 4};
        int cur = 0, wcur = 0;
        const int kPassesPerCheck = 4;
        const unsigned list_grid = 152 * 16;
        int h_left = h_amb;
        // the work items holding an unsettled core, in increasing order, into (wl, *wn)
        auto list_items = [&](int by_value, int* wl, int* wn) -> int {
            k_tie_list_flags<T><<<blocks_for(n, 256), 256, 0, s>>>(a, by_value);
            exclusive_scan<uint32_t>(item_flag, item_pos, n_items, scan32, reinterpret_cast<uint32_t*>(wn), s,
                                     &info.launches);
            k_tie_compact<<<blocks_for(n_items, 256), 256, 0, s>>>(item_flag, item_pos, n_items, wl, guard);
            info.launches += 2;
            return kOk;
        };
        // round 0 decides with positions as bounds, round 1 with greedy-descent bounds
        for (int round = 0; round < 2 && h_left > 0; ++round) {
            a.amb = lists[cur];
            a.n_amb = counts[cur];
            a.amb_out = lists[cur ^ 1];
            a.n_amb_out = counts[cur ^ 1];
            HPD_CU(cudaMemsetAsync(a.n_amb_out, 0, sizeof(int), s));
            HPD_QUERY_DISPATCH(k_tie_decide, T, mode, d, blocks_for(h_left, 4), 128, 0, s, a, 0);
            cur ^= 1;
            HPD_CU(cudaMemcpyAsync(&h_left, counts[cur], sizeof(int), cudaMemcpyDeviceToHost, s));
            HPD_CU(cudaStreamSynchronize(s));
            info.launches += 1;
            if (trace) fprintf(stderr, "[hpd tie] round %d undecided %d\n", round, h_left);
            if (h_left == 0) break;
            a.amb = lists[cur];
            a.n_amb = counts[cur];
            HPD_CU(cudaMemsetAsync(tmax, 0xff, (size_t)n * sizeof(int), s));
            HPD_CU(cudaMemsetAsync(tlow, 0x7f, (size_t)n * sizeof(int), s));  // 0x7f7f7f7f: no threshold yet
            HPD_QUERY_DISPATCH(k_tie_mark, T, mode, d, blocks_for(h_left, 4), 128, 0, s, a);
            info.launches += 1;
            if (round == 0 && d <= 5) {
                // descend from the listed items only (about a tenth of all items)
                list_items(0, wls[0], wcounts[0]);
                a.wlist = wls[0];
                a.n_wlist = wcounts[0];
                HPD_CU(cudaMemsetAsync(a.ticket, 0, sizeof(int), s));
                HPD_QUERY_DISPATCH(k_tie_greedy, T, mode, d, list_grid, 128, qsmem, s, a);
                k_tie_jump<T><<<blocks_for(n, 256), 256, 0, s>>>(a);
                k_tie_jump<T><<<blocks_for(n, 256), 256, 0, s>>>(a);
                info.launches += 3;
            } else {
                break;
            }
        }
        // relaxation passes until every border is decided or the values are exact; the
        // first pass takes the items holding an unsettled core, later passes the items
        // next to cells whose values dropped
        if (h_left > 0) {
            k_fill_int<<<blocks_for(m, 256), 256, 0, s>>>(cell_min_l, m, INT_MAX);
            k_fill_int<<<blocks_for(n_items, 256), 256, 0, s>>>(item_min_l, n_items, INT_MAX);
            k_tie_cell_min<T><<<blocks_for(n, 256), 256, 0, s>>>(a);
            info.launches += 2;
            list_items(1, wls[0], wcounts[0]);
        }
        int pass = 0;
        bool converged = false;
        while (h_left > 0 && !converged) {
            // after the first round the values change slowly: decide every 8 passes
            const int per_check = pass < kPassesPerCheck ? kPassesPerCheck : 2 * kPassesPerCheck;
            for (int k = 0; k < per_check; ++k) {
                if (pass >= rq.tie_pass_limit) {
                    err = "border tie-break did not converge";
                    return kTimeout;
                }
                ++pass;
                a.gen = pass;
                a.wlist = wls[wcur];
                a.n_wlist = wcounts[wcur];
                a.wlist_out = wls[wcur ^ 1];
                a.n_wlist_out = wcounts[wcur ^ 1];
                HPD_CU(cudaMemsetAsync(a.n_dlist, 0, sizeof(int), s));
                HPD_CU(cudaMemsetAsync(a.ticket, 0, sizeof(int), s));
                if (trace) HPD_CU(cudaMemsetAsync(tcount, 0, 2 * sizeof(unsigned long long), s));
                HPD_CU(cudaMemsetAsync(a.n_chunks, 0, sizeof(int), s));
                HPD_QUERY_DISPATCH(k_tie_edge_list, T, mode, d, list_grid, 128, qsmem, s, a);
                HPD_CU(cudaMemsetAsync(a.ticket, 0, sizeof(int), s));
                HPD_QUERY_DISPATCH(k_tie_edge_chunks, T, mode, d, list_grid, 128, qsmem, s, a);
                info.launches += 1;
                // pointer jumping speeds up the early passes; in the tail few values change
                // and the edge passes alone reach the same (exact) fixpoint
                if (pass <= kJumpPasses) k_tie_jump<T><<<blocks_for(n, 256), 256, 0, s>>>(a);
                HPD_CU(cudaMemsetAsync(a.n_wlist_out, 0, sizeof(int), s));
                HPD_QUERY_DISPATCH(k_tie_schedule, T, mode, d, list_grid, 128, 0, s, a);
                info.launches += 3;
                if (trace) {
                    unsigned long long tc[2];
                    int wn = 0;
                    // the engine's stream does not synchronise with the legacy default stream
                    HPD_CU(cudaMemcpyAsync(tc, tcount, sizeof tc, cudaMemcpyDeviceToHost, s));
                    HPD_CU(cudaMemcpyAsync(&wn, a.n_wlist, sizeof(int), cudaMemcpyDeviceToHost, s));
                    HPD_CU(cudaStreamSynchronize(s));
                    fprintf(stderr, "[hpd tie] pass %d items %d active lanes %llu tiles %llu\n", pass,
                            pass == 1 ? n_items : wn, tc[0], tc[1]);
                }
                wcur ^= 1;
            }
            int h_work = 0;
            HPD_CU(cudaMemcpyAsync(&h_work, wcounts[wcur], sizeof(int), cudaMemcpyDeviceToHost, s));
            HPD_CU(cudaStreamSynchronize(s));
            converged = h_work == 0;
            a.amb = lists[cur];
            a.n_amb = counts[cur];
            a.amb_out = lists[cur ^ 1];
            a.n_amb_out = counts[cur ^ 1];
            HPD_CU(cudaMemsetAsync(a.n_amb_out, 0, sizeof(int), s));
            HPD_QUERY_DISPATCH(k_tie_decide, T, mode, d, blocks_for(h_left, 4), 128, 0, s, a, converged ? 1 : 0);
            cur ^= 1;
            HPD_CU(cudaMemcpyAsync(&h_left, counts[cur], sizeof(int), cudaMemcpyDeviceToHost, s));
            HPD_CU(cudaStreamSynchronize(s));
            info.launches += 1;
            if (trace) fprintf(stderr, "[hpd tie] pass %d work %d undecided %d\n", pass, h_work, h_left);
            if (h_left > 0 && !converged) {
                // only the components next to the borders still undecided need values
                a.amb = lists[cur];
                a.n_amb = counts[cur];
                HPD_CU(cudaMemsetAsync(tmax, 0xff, (size_t)n * sizeof(int), s));
                HPD_CU(cudaMemsetAsync(tlow, 0x7f, (size_t)n * sizeof(int), s));
                HPD_QUERY_DISPATCH(k_tie_mark, T, mode, d, blocks_for(h_left, 4), 128, 0, s, a);
                info.launches += 1;
            }
        }
        info.tie_iterations = pass;
    }
    if (timed) HPD_CU(cudaEventRecord(tm->ev[5], s));

    // ---- labels in input order
    k_finalize<<<blocks_for(n, 256), 256, 0, s>>>(core, parent, broot, perm, n, rq.d_labels);
    info.launches += 1;
    if (timed) HPD_CU(cudaEventRecord(tm->ev[6], s));
    int h_guard[3] = {0, 0, 0};
    HPD_CU(cudaMemcpyAsync(h_guard, guard, sizeof h_guard, cudaMemcpyDeviceToHost, s));
    HPD_CU(cudaGetLastError());
    HPD_CU(cudaStreamSynchronize(s));
    if (rq.count_pairs) {
        unsigned long long pairs = 0;
        HPD_CU(cudaMemcpyAsync(&pairs, flags_dev + 16, sizeof pairs, cudaMemcpyDeviceToHost, s));
        HPD_CU(cudaStreamSynchronize(s));
        info.core_pairs = (int64_t)pairs;
    }
    if (h_guard[0]) {
        err = "internal error: device index out of range (check " + std::to_string(h_guard[1]) + ", index " +
              std::to_string(h_guard[2]) + ", " + std::to_string(h_guard[0]) + " times)";
        return kRuntime;
    }
    if (timed) {
        float ms = 0;
        cudaEventElapsedTime(&ms, tm->ev[0], tm->ev[6]); info.ms[0] = ms;
        for (int k = 1; k <= 6; ++k) {
            cudaEventElapsedTime(&ms, tm->ev[k - 1], tm->ev[k]);
            info.ms[k] = ms;
        }
        cudaEventElapsedTime(&ms, tm->ev[0], tm->ev[7]); info.index_ms[0] = ms;
        cudaEventElapsedTime(&ms, tm->ev[7], tm->ev[8]); info.index_ms[1] = ms;
        cudaEventElapsedTime(&ms, tm->ev[8], tm->ev[1]); info.index_ms[2] = ms;
        cudaEventElapsedTime(&ms, tm->ev[7], tm->ev[9]); info.cell_ids_ms = ms;
        cudaEventElapsedTime(&ms, tm->ev[10], tm->ev[3]); info.rules_ms = ms;
    }
    return kOk;
}

template <typename T>
int run_pipeline(const Request& rq, Arena& small, Arena& main, Timers* tm, RunInfo& info, std::string& err) {
    return rq.d > kStencilDirectDims ? run_pipeline_dims<T, true>(rq, small, main, tm, info, err)
                                     : run_pipeline_dims<T, false>(rq, small, main, tm, info, err);
}

}  // namespace hpd
