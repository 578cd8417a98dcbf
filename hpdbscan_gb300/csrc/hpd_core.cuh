// Core test: neighbour counts with an early exit at minPoints.
#pragma once

#include "hpd_query.cuh"

namespace hpd {

// ---------------------------------------------------------------- core test
// |N_eps(p)| >= minPoints, self included, with an early exit once every query of
// the warp has reached minPoints (hpdbscan.h:74-78).
template <typename T>
__device__ __forceinline__ T shfl_val(T v, int src) {
    if constexpr (sizeof(T) < 4) return (T)__shfl_sync(0xffffffffu, (int)v, src);
    else return __shfl_sync(0xffffffffu, v, src);
}

constexpr int kMaxRanges = 32;     // neighbour ranges kept in shared memory (3^d <= 32: d <= 3)

// F: bit 0 (kCorePrune) selects the cells next to big dense cells, bit 1
// (kCoreCount) counts the distance evaluations into a.pair_count (diagnostic pass).
constexpr int kCorePrune = 1, kCoreCount = 2;

template <typename T, int M, int D, int F>
__global__ void __launch_bounds__(128) k_core(QueryArgs<T> a) {
    constexpr bool PRUNE = (F & kCorePrune) != 0;
    constexpr bool COUNT = (F & kCoreCount) != 0;
    unsigned long long evals = 0;
    auto flush_evals = [&]() {
        if constexpr (COUNT) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) evals += __shfl_xor_sync(0xffffffffu, evals, o);
            if (lane_id() == 0) atomicAdd(a.pair_count, evals);
        }
    };
    __shared__ int2 s_rng[4][kMaxRanges];
    __shared__ int s_pre[4][32];
    const int w = threadIdx.x >> 5;
    const int item = blockIdx.x * 4 + w;
    if (item >= a.n_items) return;
    const int2 it = a.items[item];
    const int r = it.x;
    // cells next to a big dense cell are handled by the PRUNE instantiation
    if (((a.cell_flags[r] & kCellNearBig) != 0) != PRUNE) return;
    const Tile<T> tile = warp_tile<T>(a.g.d);
    const int pend = min(it.y + 32, a.ct.start[r + 1]);
    const int p = it.y + (int)lane_id();
    const bool active = p < pend;
    T q[D > 0 ? D : kMaxDims];
    load_query<T, D>(a, p, active, q);
    int count = 0;
    const int limit = a.min_points;
    if (a.dense_id) {
        // a point of a dense cell whose sub-cell holds >= minPoints points has that many
        // neighbours within eps already (sub-cells are certified cliques)
        const int id = a.dense_id[r];
        if (id >= 0 && active) {
            const int g = a.dense_gidx[p];
            const int* grp = a.dense_grp + (size_t)id * (a.dense_groups + 1);
            if (grp[g + 1] - grp[g] >= limit) count = limit;
        }
        if (__all_sync(0xffffffffu, !active || count >= limit)) {
            if (active) a.core[p] = 1;
            flush_evals();
            return;
        }
    }
    int S = 1;
    for (int sd = 0; sd < a.g.d; ++sd) S *= 3;
    if (!PRUNE && pend - it.y <= a.sparse_queries && S <= kMaxRanges) {
        // few queries: the candidates of all neighbour cells form one flat list; each
        // lane loads one candidate and tests every open query against it (a ballot
        // counts the hits per query), so a candidate is loaded once for the item
        int nr = 0;
        visit_stencil<D>(a.g, a.ct, r, 0, [&](int cr, bool) {
            if (lane_id() == 0) s_rng[w][nr] = make_int2(a.ct.start[cr], a.ct.start[cr + 1]);
            ++nr;
            return true;
        });
        __syncwarp();
        const int lane = (int)lane_id();
        const int sz = lane < nr ? s_rng[w][lane].y - s_rng[w][lane].x : 0;
        int incl = sz;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        const int total = __shfl_sync(0xffffffffu, incl, 31);
        s_pre[w][lane] = incl - sz;  // first flat index of range `lane`
        __syncwarp();
        const int nq = pend - it.y;
        int hits = 0;  // lane i < nq: hits of query i
        unsigned open = __ballot_sync(0xffffffffu, lane < nq);
        for (int t0 = 0; t0 < total && open; t0 += 32) {
            const int t = t0 + lane;
            const bool valid = t < total;
            T c[D > 0 ? D : kMaxDims];
            if (valid) {
                int lo = 0, hi = nr - 1;  // last range starting at or before t
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (s_pre[w][mid] <= t) lo = mid; else hi = mid - 1;
                }
                const int j = s_rng[w][lo].x + (t - s_pre[w][lo]);
#pragma unroll
                for (int k = 0; k < (D > 0 ? D : kMaxDims); ++k) {
                    if (D <= 0 && k >= a.g.d) break;
                    c[k] = a.coords[(size_t)k * a.n + j];
                }
            }
            for (int src = 0; src < nq; ++src) {
                if (!((open >> src) & 1u)) continue;
                T qq[D > 0 ? D : kMaxDims];
#pragma unroll
                for (int k = 0; k < (D > 0 ? D : kMaxDims); ++k) {
                    if (D <= 0 && k >= a.g.d) break;
                    qq[k] = shfl_val(q[k], src);
                }
                const bool hit = valid && within_vals<T, M, D>(a, qq, c);
                if constexpr (COUNT) evals += valid ? 1 : 0;
                const int h = __popc(__ballot_sync(0xffffffffu, hit));
                if (lane == src) hits += h;
            }
            open = __ballot_sync(0xffffffffu, lane < nq && hits < limit);
        }
        if (lane < nq) a.core[it.y + lane] = hits >= limit ? 1 : 0;
        flush_evals();
        return;
    }
    auto aux_of = [](int) { return 0; };
    auto pair = [&](int, int u, int) {
        if constexpr (COUNT) evals += active ? 1 : 0;
        if (active && within<T, M, D>(a, q, tile, u)) ++count;
    };
    auto done = [&]() { return __all_sync(0xffffffffu, !active || count >= limit); };
    visit_stencil<D>(a.g, a.ct, r, 0, [&](int cr, bool) {
        if constexpr (PRUNE) {
            if (pruned_cell(a, cr)) {
                // a sub-cell wholly within eps adds its population without a scan; only
                // sub-cells crossing the eps sphere are streamed, for the lanes they cross
                const int* grp = a.dense_grp + (size_t)a.dense_id[cr] * (a.dense_groups + 1);
                int cur = kBoxFar;
                auto visit_group = [&](int g, int cls) -> bool {
                    cur = cls;
                    if (cls == kBoxIn) count += grp[g + 1] - grp[g];
                    return __any_sync(0xffffffffu, cls == kBoxEdge);
                };
                auto pair_edge = [&](int, int u, int) {
                    if constexpr (COUNT) evals += (active && cur == kBoxEdge) ? 1 : 0;
                    if (cur == kBoxEdge && within<T, M, D>(a, q, tile, u)) ++count;
                };
                return !scan_dense<T, D>(a, tile, cr, q, active && count < limit, visit_group, aux_of, pair_edge,
                                         done);
            }
        }
        return !scan_range(a, tile, a.ct.start[cr], a.ct.start[cr + 1], aux_of, pair, done);
    });
    if (active) a.core[p] = count >= limit ? 1 : 0;
    flush_evals();
}

}  // namespace hpd
