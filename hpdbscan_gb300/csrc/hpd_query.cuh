// Query kernels: neighbour counts (core test), core-core connectivity, border
// assignment, the border tie-break and the final labels.
//
// Work decomposition: one warp per work item, an item being up to 32 consecutive
// points of one cell (the "queries", one per lane).  The warp enumerates the
// 3^d neighbour cells of the item's cell once (reference get_neighbors,
// spatial_index.h:682-737), streams each neighbour cell's points through shared
// memory in tiles of 32 (coalesced loads from the cell-sorted coordinate planes)
// and every lane tests its query against the tile (reference region_query,
// spatial_index.h:739-768), in the reference's own arithmetic.
#pragma once

#include <climits>
#include <type_traits>

#include "hpd_common.cuh"
#include "hpd_index.cuh"

namespace hpd {

// Range check of an index read from device tables: an index outside [0, bound) is
// recorded in guard[0..2] (count, tag, index) and the access is skipped, so that a
// corrupted table ends the call with an error status instead of a memory fault.
enum GuardTag : int {
    kGuardStencilKey = 1, kGuardStencilCell, kGuardItem, kGuardRoot, kGuardDirtyCell, kGuardDirtyList,
    kGuardAmbiguous, kGuardLabel, kGuardCellRank, kGuardItemIndex, kGuardList, kGuardCount
};
__device__ __forceinline__ bool in_range(int* guard, long long i, long long bound, int tag) {
    if (i >= 0 && i < bound) return true;
    if (guard && atomicAdd(guard, 1) == 0) {
        guard[1] = tag;
        guard[2] = (int)i;
    }
    return false;
}

struct CellTable {
    const int32_t* start;              // [m + 1] first sorted position of each cell
    const unsigned long long* key;     // [m] cell id
    const int32_t* dense;              // [grid total] cell rank or -1; nullptr -> binary search
    const uint32_t* ccoord;            // [d][pitch] grid coordinate of each cell, swapped order
    int m;
    int pitch;
    int* guard;                        // range-check record (see in_range)
};

__device__ __forceinline__ int find_cell(const CellTable& ct, unsigned long long key) {
    if (ct.dense) return ct.dense[key];
    int lo = 0, hi = ct.m;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (ct.key[mid] < key) lo = mid + 1; else hi = mid;
    }
    return (lo < ct.m && ct.key[lo] == key) ? lo : -1;
}

// Warp-aggregated atomics: the lanes of a warp that target the same address combine
// their values first, so that cells of millions of points cost one atomic per warp
// rather than one per point.  Every lane of the warp must call; lanes with ok false
// take no part in the update.
__device__ __forceinline__ void agg_atomic_min(int* base, int idx, int v, bool ok) {
    const unsigned peers = __match_any_sync(0xffffffffu, ok ? idx : -1);
    if (!ok) return;
    const int m = __reduce_min_sync(peers, v);
    if ((int)lane_id() == __ffs(peers) - 1) atomicMin(base + idx, m);
}
__device__ __forceinline__ void agg_atomic_add(int* base, int idx, bool ok) {
    const unsigned peers = __match_any_sync(0xffffffffu, ok ? idx : -1);
    if (ok && (int)lane_id() == __ffs(peers) - 1) atomicAdd(base + idx, __popc(peers));
}
// slot of the lane among its peers: the leader reserves popc(peers) slots at base[idx]
__device__ __forceinline__ int agg_reserve(int* base, int idx, bool ok) {
    const unsigned peers = __match_any_sync(0xffffffffu, ok ? idx : -1);
    const int leader = __ffs(peers) - 1;
    int b = 0;
    if (ok && (int)lane_id() == leader) b = atomicAdd(base + idx, __popc(peers));
    b = __shfl_sync(0xffffffffu, b, leader);
    return b + __popc(peers & ((1u << lane_id()) - 1u));
}

// Visits the non-empty cells of the 3^d block around cell r (sel: 0 all, 1 only
// smaller cell ids, 2 only larger cell ids), the item's own cell first (or last
// when own_last), calling fn(cell_rank, is_own) warp-uniformly; fn returns false
// to stop the visit.
struct KeepAll {
    __device__ __forceinline__ bool operator()(int) const { return true; }
};

template <class Fn, class Keep = KeepAll>
__device__ __forceinline__ void visit_stencil(const Grid& g, const CellTable& ct, int r, int sel, Fn&& fn,
                                              bool own_last = false, Keep keep = Keep()) {
    if (!own_last && !fn(r, true)) return;
    const unsigned lane = lane_id();
    const unsigned long long key = ct.key[r];
    unsigned long long coord[kMaxDims];
    for (int s = 0; s < g.d; ++s) coord[s] = ct.ccoord[(size_t)s * ct.pitch + r];
    int S = 1;
    for (int s = 0; s < g.d; ++s) S *= 3;
    const int center = (S - 1) / 2;
    for (int b = 0; b < S; b += 32) {
        const int o = b + (int)lane;
        int nr = -1;
        if (o < S && o != center) {
            int rest = o;
            bool ok = true;
            unsigned long long nk = key;
            for (int s = 0; s < g.d; ++s) {
                const int dig = rest % 3;
                rest /= 3;
                if (dig == 0) {
                    if (coord[s] == 0) ok = false; else nk -= g.stride[s];
                } else if (dig == 2) {
                    if (coord[s] + 1 >= g.dims[g.swapped[s]]) ok = false; else nk += g.stride[s];
                }
            }
            if (ok && (sel == 0 || (sel == 1 ? nk < key : nk > key))) {
                nr = (ct.dense && !in_range(ct.guard, (long long)nk, (long long)g.total, kGuardStencilKey))
                         ? -1 : find_cell(ct, nk);
                if (nr >= 0 && !in_range(ct.guard, nr, ct.m, kGuardStencilCell)) nr = -1;
            }
            // the per-cell filter runs on all lanes at once, hiding its load latency
            if (nr >= 0 && !keep(nr)) nr = -1;
        }
        unsigned mask = __ballot_sync(0xffffffffu, nr >= 0);
        while (mask) {
            const int src = __ffs(mask) - 1;
            mask &= mask - 1;
            const int cr = __shfl_sync(0xffffffffu, nr, src);
            if (!fn(cr, false)) return;
        }
    }
    if (own_last) fn(r, true);
}

// Union-find over sorted point positions; roots are component minima.
__device__ __forceinline__ int uf_find(int* parent, int x) {
    for (;;) {
        const int p = ld_volatile(parent + x);
        if (p == x) return x;
        const int gp = ld_volatile(parent + p);
        if (gp != p) parent[x] = gp;
        x = p;
    }
}
__device__ __forceinline__ void uf_union(int* parent, int a, int b) {
    for (;;) {
        a = uf_find(parent, a);
        b = uf_find(parent, b);
        if (a == b) return;
        if (a < b) { const int t = a; a = b; b = t; }
        if (atomicCAS(parent + a, a, b) == a) return;
    }
}

template <typename T>
struct QueryArgs {
    const T* coords;      // d planes of n
    int n;
    Grid g;
    CellTable ct;
    T eps2;
    const int2* items;    // (cell rank, first point)
    int n_items;
    int min_points;       // clamped to n + 1
    uint8_t* core;
    int* parent;          // union-find; after compression: component root of every core
    int* broot;           // border: root of the assigned cluster, -1 noise
    int* amb;             // ambiguous border points
    int* n_amb;
    int* tmax;            // per root: highest position of a core next to an undecided border
    int* tlow;            // per root: a value below it decides every undecided border of the component
                          // (-1: component not involved); only positions <= tmax matter
    int* lm1;             // tie-break value L - 1 (see k_tie_edge)
    int* changed;
    const uint32_t* cellrank;  // cell rank of every sorted point
    int* cell_rep;        // smallest core root of the cell after the in-cell unions, kNoCore if none
    uint8_t* cell_flags;  // kCellUniform: every core of the cell has root cell_rep
    // tie-break frontier: a cell is dirty in pass g when a value in it dropped in pass g
    int* dirty_gen;       // last pass that dirtied the cell
    int* sched_gen;       // last pass whose work list holds the cell's items
    int gen;              // current pass
    int* dlist;           // cells dirtied in the current pass
    int* n_dlist;
    const int* wlist;     // work items of the current pass
    const int* n_wlist;
    int* wlist_out;       // work items of the next pass
    int* n_wlist_out;
    const uint32_t* ipos; // item index of each chunk-start point
    int* cell_min_l;      // per cell: smallest lm1 among its cores (kept current as values drop)
    int* item_min_l;      // per work item (32-point chunk): the same, one level finer
    uint32_t* item_flag;  // items scheduled for the next pass
    int* ticket;          // next work-list entry to take
    unsigned long long* trace_counts;  // diagnostics (nullptr: off): [0] active lanes, [1] tiles scanned
    int* guard;           // range-check record (see in_range)
    const int* dense_id;  // per cell: >= 0 when the dense-cell kernels connect its cores
    const int* dense_grp; // [dense][groups + 1] sub-cell starts (see DenseArgs)
    const int* dense_gidx;  // per point of a dense cell: its sub-cell
    int dense_groups;
    const int* dense_sec; // points of dense cells grouped by sub-cell (positions)
    const T* dense_box;   // [dense][groups][2][d] bounding box of each sub-cell's points
    const int* dense_rep; // [dense][groups] smallest core of each sub-cell (INT_MAX: none), after the core test
    const T* dense_coords;  // [d][n] coordinates of dense cells' points in dense_sec order
    int* amb_out;         // undecided ambiguous borders after a decision round
    int* n_amb_out;
};

// Per-warp tile in shared memory: d planes of 32 coordinates plus one aux word.
// Per-warp tile in shared memory: 32 candidates, each padded to tile_stride(d)
// coordinates (2 or 4 for d <= 4, so that one vector load fetches a candidate),
// plus one aux word per candidate.
__host__ __device__ __forceinline__ int tile_stride(int d) { return d <= 2 ? 2 : (d <= 4 ? 4 : d); }

// cell summaries (cell_rep, cell_flags)
constexpr int kNoCore = INT_MAX;
constexpr uint8_t kCellUniform = 1;
constexpr uint8_t kCellNearBig = 2;  // a cell of the 3^d block holds >= kPruneMinPoints points (dense path)

template <typename T>
struct Tile {
    T* c;      // [32][tile_stride(d)]
    int* aux;  // [32]
};

// tmax of the component of a cell's representative core (range-checked)
template <typename T>
__device__ __forceinline__ int tmax_of(const QueryArgs<T>& a, int rep_c) {
    if (!in_range(a.guard, rep_c, a.n, kGuardRoot)) return INT_MAX;
    const int root = a.parent[rep_c];
    return in_range(a.guard, root, a.n, kGuardRoot) ? a.tmax[root] : INT_MAX;
}

template <typename T>
__device__ __forceinline__ Tile<T> warp_tile(int d) {
    extern __shared__ __align__(16) unsigned char smem_q[];
    const int w = threadIdx.x >> 5;
    const size_t per = (size_t)tile_stride(d) * 32 * sizeof(T) + 32 * sizeof(int);
    unsigned char* base = smem_q + per * w;
    Tile<T> t;
    t.c = reinterpret_cast<T*>(base);
    t.aux = reinterpret_cast<int*>(base + (size_t)tile_stride(d) * 32 * sizeof(T));
    return t;
}

// Streams candidates [cs, ce) through the tile; pair(q, u, aux) runs per lane for
// every candidate q (tile slot u); returns true when done() holds for the warp.
template <typename T, class Aux, class Pair, class Done>
__device__ __forceinline__ bool scan_range(const QueryArgs<T>& a, const Tile<T>& tile, int cs, int ce, Aux&& aux_of,
                                           Pair&& pair, Done&& done) {
    const int d = a.g.d;
    const int S = tile_stride(d);
    const unsigned lane = lane_id();
    for (int t0 = cs; t0 < ce; t0 += 32) {
        const int j = t0 + (int)lane;
        if (j < ce) {
            for (int k = 0; k < d; ++k) tile.c[lane * S + k] = a.coords[(size_t)k * a.n + j];
            tile.aux[lane] = aux_of(j);
        }
        __syncwarp();
        const int cnt = min(32, ce - t0);
        for (int u = 0; u < cnt; ++u) pair(t0 + u, u, tile.aux[u]);
        __syncwarp();
        if (done()) return true;
    }
    return false;
}

// Where a query lies relative to a sub-cell's bounding box: kBoxFar when every point
// of the box is farther than eps, kBoxIn when every point is within eps, else
// kBoxEdge.  The tests leave a 1e-4 relative margin on the squared distance; they run
// in the element type (float or double), whose rounding (~1e-6 relative for float)
// stays far inside that margin, so the verdict holds for the reference's own sum.
constexpr int kBoxFar = 0, kBoxIn = 1, kBoxEdge = 2;
template <typename T>
using BoxReal = typename std::conditional<Elem<T>::kFloat, T, double>::type;
template <typename T, int D>
__device__ __forceinline__ int box_class(const T* q, const T* box, int d, BoxReal<T> eps2) {
    using R = BoxReal<T>;
    R lo2 = 0, hi2 = 0;
#pragma unroll
    for (int k = 0; k < (D > 0 ? D : kMaxDims); ++k) {
        if (D == 0 && k >= d) break;
        const R lo = (R)box[k], hi = (R)box[d + k], x = (R)q[k];
        const R dn = x < lo ? lo - x : (x > hi ? x - hi : R(0));
        const R df = x - lo > hi - x ? x - lo : hi - x;
        lo2 += dn * dn;
        hi2 += df * df;
    }
    if (lo2 > eps2 * R(1.0001)) return kBoxFar;
    return hi2 <= eps2 * R(0.9999) ? kBoxIn : kBoxEdge;
}

// Dense cells with at least this many points are visited sub-cell by sub-cell with the
// box tests above; smaller ones are cheaper to stream whole.
constexpr int kPruneMinPoints = 8192;
template <typename T>
__device__ __forceinline__ bool pruned_cell(const QueryArgs<T>& a, int cr) {
    return a.dense_id && a.dense_id[cr] >= 0 && a.ct.start[cr + 1] - a.ct.start[cr] >= kPruneMinPoints;
}

// Visits dense cell cr sub-cell by sub-cell: visit_group(g, cls) receives each lane's
// box verdict for sub-cell g (kBoxFar for inactive lanes), may account for the whole
// sub-cell, and returns whether the warp must stream its points through the tile
// (warp-uniform).  pair(q, u, aux) gets the candidate's position q; returns true when
// done() holds for the warp.
template <typename T, int D, class Visit, class Aux, class Pair, class Done>
__device__ __forceinline__ bool scan_dense(const QueryArgs<T>& a, const Tile<T>& tile, int cr, const T* q, bool active,
                                           Visit&& visit_group, Aux&& aux_of, Pair&& pair, Done&& done) {
    const int d = a.g.d;
    const int S = tile_stride(d);
    const unsigned lane = lane_id();
    const int id = a.dense_id[cr];
    const int s0 = a.ct.start[cr];
    const int* grp = a.dense_grp + (size_t)id * (a.dense_groups + 1);
    const T* box = a.dense_box + (size_t)id * a.dense_groups * 2 * d;
    const int* idx = a.dense_sec + s0;
    for (int g = 0; g < a.dense_groups; ++g) {
        const int gs = grp[g], ge = grp[g + 1];
        if (gs == ge) continue;
        const int cls = active ? box_class<T, D>(q, box + (size_t)g * 2 * d, d, (BoxReal<T>)a.eps2) : kBoxFar;
        if (visit_group(g, cls)) {
            for (int t0 = gs; t0 < ge; t0 += 32) {
                const int t = t0 + (int)lane;
                int j = -1;
                if (t < ge) {
                    j = idx[t];
                    for (int k = 0; k < d; ++k) tile.c[lane * S + k] = a.dense_coords[(size_t)k * a.n + s0 + t];
                    tile.aux[lane] = aux_of(j);
                }
                __syncwarp();
                const int cnt = min(32, ge - t0);
                for (int u = 0; u < cnt; ++u) pair(__shfl_sync(0xffffffffu, j, u), u, tile.aux[u]);
                __syncwarp();
                if (done()) return true;
            }
        }
        if (done()) return true;
    }
    return false;
}

// Like scan_range for union-find work, with the expensive per-candidate lookup done
// lazily: each lane first tests its query against the tile's core candidates
// (test(q, u)), and aux_of runs only for candidates that some lane hit (one lane per
// candidate); on_hit(q, u, aux) then runs per lane for its own hits.
template <typename T, class Test, class Aux, class OnHit, class Done>
__device__ __forceinline__ bool scan_range_hits(const QueryArgs<T>& a, const Tile<T>& tile, int cs, int ce, Test&& test,
                                                Aux&& aux_of, OnHit&& on_hit, Done&& done) {
    const int d = a.g.d;
    const int S = tile_stride(d);
    const unsigned lane = lane_id();
    for (int t0 = cs; t0 < ce; t0 += 32) {
        const int j = t0 + (int)lane;
        bool is_core = false;
        if (j < ce) {
            for (int k = 0; k < d; ++k) tile.c[lane * S + k] = a.coords[(size_t)k * a.n + j];
            is_core = a.core[j] != 0;
        }
        const unsigned cores = __ballot_sync(0xffffffffu, is_core);
        __syncwarp();
        unsigned mine = 0;
        for (unsigned m = cores; m; m &= m - 1) {
            const int u = __ffs(m) - 1;
            if (test(t0 + u, u)) mine |= 1u << u;
        }
        const unsigned hit = __reduce_or_sync(0xffffffffu, mine);
        if (hit) {
            if ((hit >> lane) & 1u) tile.aux[lane] = aux_of(j);
            __syncwarp();
            for (; mine; mine &= mine - 1) {
                const int u = __ffs(mine) - 1;
                on_hit(t0 + u, u, tile.aux[u]);
            }
        }
        __syncwarp();
        if (done()) return true;
    }
    return false;
}

// candidate u of the tile into c[] (vector loads for d = 2..4)
template <typename T, int D>
__device__ __forceinline__ void tile_load(const Tile<T>& tile, int u, int d, T* c) {
    if constexpr (!Elem<T>::kFloat) {
        const int S = tile_stride(d);
#pragma unroll
        for (int k = 0; k < (D > 0 ? D : kMaxDims); ++k) {
            if (D == 0 && k >= d) break;
            c[k] = tile.c[u * S + k];
        }
    } else if (D == 2) {
        if (sizeof(T) == 4) { const float2 v = reinterpret_cast<const float2*>(tile.c)[u]; c[0] = (T)v.x; c[1] = (T)v.y; }
        else { const double2 v = reinterpret_cast<const double2*>(tile.c)[u]; c[0] = (T)v.x; c[1] = (T)v.y; }
    } else if (D == 3 || D == 4) {
        if (sizeof(T) == 4) {
            const float4 v = reinterpret_cast<const float4*>(tile.c)[u];
            c[0] = (T)v.x; c[1] = (T)v.y; c[2] = (T)v.z;
            if (D == 4) c[3] = (T)v.w;
        } else {
            const double2 v0 = reinterpret_cast<const double2*>(tile.c)[2 * u];
            const double2 v1 = reinterpret_cast<const double2*>(tile.c)[2 * u + 1];
            c[0] = (T)v0.x; c[1] = (T)v0.y; c[2] = (T)v1.x;
            if (D == 4) c[3] = (T)v1.y;
        }
    } else {
        const int S = tile_stride(d);
#pragma unroll
        for (int k = 0; k < kMaxDims; ++k) {
            if (k >= d) break;
            c[k] = tile.c[u * S + k];
        }
    }
}

// Integer element types: `T distance = p - q; offset += distance * distance`
// (spatial_index.h:751-754) wraps at every store into T, so the result is the sum of
// the wrapped squares modulo 2^bits(T), read back as T, in any summation order.
template <typename T, int D>
__device__ __forceinline__ bool int_within(const T* p, const T* q, int d, T eps2) {
    unsigned long long acc = 0;
#pragma unroll
    for (int k = 0; k < (D > 0 ? D : kMaxDims); ++k) {
        if (D == 0 && k >= d) break;
        const T t = (T)((unsigned long long)p[k] - (unsigned long long)q[k]);
        const unsigned long long w = (unsigned long long)(long long)t;
        acc += w * w;
    }
    return (T)acc <= eps2;
}

// squared distance between q[] and c[] in the reference's arithmetic, <= eps2
template <typename T, int M, int D>
__device__ __forceinline__ bool within_vals(const QueryArgs<T>& a, const T* q, const T* c) {
    if constexpr (!Elem<T>::kFloat) {
        return int_within<T, D>(q, c, a.g.d, a.eps2);
    } else {
        T t[D > 0 ? D : kMaxDims];
#pragma unroll
        for (int k = 0; k < (D > 0 ? D : kMaxDims); ++k) {
            if (D == 0 && k >= a.g.d) break;
            t[k] = sub_(q[k], c[k]);
        }
        return fold_sq<T, M, D>(t, a.g.d) <= a.eps2;
    }
}

// squared distance from the lane's query (q[]) to tile slot u, compared with eps2
template <typename T, int M, int D>
__device__ __forceinline__ bool within(const QueryArgs<T>& a, const T* q, const Tile<T>& tile, int u) {
    T c[D > 0 ? (D < 4 ? 4 : D) : kMaxDims];
    tile_load<T, D>(tile, u, a.g.d, c);
    if constexpr (!Elem<T>::kFloat) {
        return int_within<T, D>(q, c, a.g.d, a.eps2);
    } else {
        T t[D > 0 ? D : kMaxDims];
#pragma unroll
        for (int k = 0; k < (D > 0 ? D : kMaxDims); ++k) {
            if (D == 0 && k >= a.g.d) break;
            t[k] = sub_(q[k], c[k]);
        }
        return fold_sq<T, M, D>(t, a.g.d) <= a.eps2;
    }
}

template <typename T, int D>
__device__ __forceinline__ void load_query(const QueryArgs<T>& a, int p, bool active, T* q) {
#pragma unroll
    for (int k = 0; k < (D > 0 ? D : kMaxDims); ++k) {
        if (D == 0 && k >= a.g.d) break;
        q[k] = active ? a.coords[(size_t)k * a.n + p] : T(0);
    }
}

// ---------------------------------------------------------------- core test
// |N_eps(p)| >= minPoints, self included, with an early exit once every query of
// the warp has reached minPoints (hpdbscan.h:74-78).
template <typename T>
__device__ __forceinline__ T shfl_val(T v, int src) {
    if constexpr (sizeof(T) < 4) return (T)__shfl_sync(0xffffffffu, (int)v, src);
    else return __shfl_sync(0xffffffffu, v, src);
}

constexpr int kSparseQueries = 8;  // items with at most this many points use candidate lanes
constexpr int kMaxRanges = 32;     // neighbour ranges kept in shared memory (3^d <= 32: d <= 3)

template <typename T, int M, int D, bool PRUNE>
__global__ void __launch_bounds__(128) k_core(QueryArgs<T> a) {
    __shared__ int2 s_rng[4][kMaxRanges];
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
            return;
        }
    }
    int S = 1;
    for (int sd = 0; sd < a.g.d; ++sd) S *= 3;
    if (!PRUNE && pend - it.y <= kSparseQueries && S <= kMaxRanges) {
        // few queries: the whole warp tests consecutive candidates of one query at a
        // time (a ballot counts the hits), instead of leaving most lanes idle
        int nr = 0;
        visit_stencil(a.g, a.ct, r, 0, [&](int cr, bool) {
            if (lane_id() == 0) s_rng[w][nr] = make_int2(a.ct.start[cr], a.ct.start[cr + 1]);
            ++nr;
            return true;
        });
        __syncwarp();
        for (int src = 0; src < pend - it.y; ++src) {
            T qq[D > 0 ? D : kMaxDims];
#pragma unroll
            for (int k = 0; k < (D > 0 ? D : kMaxDims); ++k) {
                if (D == 0 && k >= a.g.d) break;
                qq[k] = shfl_val(q[k], src);
            }
            int hits = 0;
            for (int ri = 0; ri < nr && hits < limit; ++ri) {
                const int ce = s_rng[w][ri].y;
                for (int j0 = s_rng[w][ri].x; j0 < ce && hits < limit; j0 += 32) {
                    const int j = j0 + (int)lane_id();
                    bool hit = false;
                    if (j < ce) {
                        T c[D > 0 ? D : kMaxDims];
#pragma unroll
                        for (int k = 0; k < (D > 0 ? D : kMaxDims); ++k) {
                            if (D == 0 && k >= a.g.d) break;
                            c[k] = a.coords[(size_t)k * a.n + j];
                        }
                        hit = within_vals<T, M, D>(a, qq, c);
                    }
                    hits += __popc(__ballot_sync(0xffffffffu, hit));
                }
            }
            if (lane_id() == 0) a.core[it.y + src] = hits >= limit ? 1 : 0;
        }
        return;
    }
    auto aux_of = [](int) { return 0; };
    auto pair = [&](int, int u, int) {
        if (active && within<T, M, D>(a, q, tile, u)) ++count;
    };
    auto done = [&]() { return __all_sync(0xffffffffu, !active || count >= limit); };
    visit_stencil(a.g, a.ct, r, 0, [&](int cr, bool) {
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
                    if (cur == kBoxEdge && within<T, M, D>(a, q, tile, u)) ++count;
                };
                return !scan_dense<T, D>(a, tile, cr, q, active && count < limit, visit_group, aux_of, pair_edge,
                                         done);
            }
        }
        return !scan_range(a, tile, a.ct.start[cr], a.ct.start[cr + 1], aux_of, pair, done);
    });
    if (active) a.core[p] = count >= limit ? 1 : 0;
}

// ---------------------------------------------------- core-core connectivity
// Every core-core eps edge (q < p) is united.  Pass 1 unites the pairs inside each
// cell; then every cell gets a summary (the smallest component root among its
// cores, and whether all its cores share it); pass 2 unites pairs across cells
// and skips, without loading a single coordinate, a neighbour cell that holds no
// core or whose cores are already in the query cell's component.  Within a tile,
// candidates already in the query's component are skipped without a distance test.

template <typename T, int M, int D>
__global__ void __launch_bounds__(128) k_union_intra(QueryArgs<T> a) {
    const int item = blockIdx.x * 4 + (threadIdx.x >> 5);
    if (item >= a.n_items) return;
    const int2 it = a.items[item];
    const int r = it.x;
    if (a.dense_id && a.dense_id[r] >= 0) return;  // connected by the dense-cell kernels
    const int pend = min(it.y + 32, a.ct.start[r + 1]);
    const int p = it.y + (int)lane_id();
    const bool active = p < pend && a.core[p];
    if (!__any_sync(0xffffffffu, active)) return;
    const Tile<T> tile = warp_tile<T>(a.g.d);
    T q[D > 0 ? D : kMaxDims];
    load_query<T, D>(a, p, active, q);
    int myroot = active ? uf_find(a.parent, p) : -1;
    auto test = [&](int qi, int u) { return active && qi < p && within<T, M, D>(a, q, tile, u); };
    auto aux_of = [&](int j) { return uf_find(a.parent, j); };
    auto on_hit = [&](int qi, int, int rep) {
        if (rep == myroot) return;
        uf_union(a.parent, p, qi);
        myroot = uf_find(a.parent, p);
    };
    auto never = []() { return false; };
    scan_range_hits(a, tile, a.ct.start[r], pend, test, aux_of, on_hit, never);
}

static __global__ void k_cell_rep(const uint8_t* core, int* parent, const uint32_t* cellrank, int n, int* cell_rep) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool ok = i < n && core[i];
    agg_atomic_min(cell_rep, ok ? (int)cellrank[i] : 0, ok ? uf_find(parent, i) : 0, ok);
}

static __global__ void k_cell_uniform(const uint8_t* core, int* parent, const uint32_t* cellrank, int n,
                                      const int* cell_rep, uint8_t* cell_flags) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && core[i]) {
        const uint32_t c = cellrank[i];
        // every writer clears the same bit of a byte whose other bits no longer change
        if (uf_find(parent, i) != cell_rep[c]) cell_flags[c] &= (uint8_t)~kCellUniform;
    }
}

// ------------------------------------------------------ dense cells
// A cell holding many points is split into k^d sub-cells of side eps / k, with k
// chosen on the host so that the diagonal of a sub-cell, widened by the rounding
// slack of the cell computation, is at most 0.95 eps: any two points of one sub-cell
// are then within eps under the reference's arithmetic (the computed squared
// distance stays ~10 % below EPS2), so the cores of a sub-cell form a clique and are
// united as a star.  Sub-cells of one cell are then connected pairwise by a
// first-hit scan unless already in one component.  Connectivity is exactly that of
// the core-core eps graph inside the cell, at O(points) cost instead of O(points^2).
struct DenseArgs {
    int k;                  // sub-cells per dimension
    int groups;             // k^d
    int min_points;         // cells with at least this many points take this path
    double scale;           // k / eps
    double mins_d[kMaxDims];
    int* dense_id;          // per cell: index in the dense list or -1
    int* cells;             // dense list: cell rank
    int* n_dense;
    int* grp;               // [dense][groups + 1] start of each sub-cell in sec (relative to the cell)
    int* grp_rep;           // [dense][groups] smallest core of each sub-cell (INT_MAX: none)
    int* sec;               // points of dense cells grouped by sub-cell (same range as the cell)
    int* gidx;              // per point of a dense cell: its sub-cell
    void* box;              // [dense][groups][2][d] element-type bounding box of each sub-cell
    void* coords;           // [d][n] coordinates of dense cells' points in sec order
    int* cur;               // [dense][groups] scatter cursors
    int boxes;              // build boxes and the coordinate copy (a cell holds >= kPruneMinPoints)
};

static __global__ void k_dense_list(const int32_t* cell_start, int m, DenseArgs da) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= m) return;
    if (cell_start[c + 1] - cell_start[c] >= da.min_points) {
        const int id = atomicAdd(da.n_dense, 1);
        da.dense_id[c] = id;
        da.cells[id] = c;
    } else {
        da.dense_id[c] = -1;
    }
}

// Order-preserving unsigned encoding of a floating value (larger value, larger code),
// so that integer atomics can take minima and maxima of coordinates.
template <typename T> struct OrdKey;
template <> struct OrdKey<float> {
    using U = unsigned;
    __device__ static U enc(float v) {
        const unsigned u = __float_as_uint(v);
        return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
    }
    __device__ static float dec(U u) { return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u); }
};
template <> struct OrdKey<double> {
    using U = unsigned long long;
    __device__ static U enc(double v) {
        const unsigned long long u = (unsigned long long)__double_as_longlong(v);
        return (u >> 63) ? ~u : (u | (1ull << 63));
    }
    __device__ static double dec(U u) { return __longlong_as_double((long long)((u >> 63) ? (u & ~(1ull << 63)) : ~u)); }
};

constexpr int kDenseMaxGroups = 81;  // k^d for the sub-cell splits used (<= 81)

// Sub-cell construction for all dense cells at once, parallel over points (a cell of
// millions of points is spread over the whole GPU):
//   k_dense_init     per (dense cell, sub-cell): count 0, no core, empty box
//   k_dense_assign   per point of a dense cell: its sub-cell, the count, the box
//   k_dense_offsets  per dense cell: counts -> start offsets, boxes decoded
//   k_dense_scatter  per point: its slot in sec and its coordinates in sec order
template <typename T>
__global__ void k_dense_init(QueryArgs<T> a, DenseArgs da) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)*da.n_dense * da.groups) return;
    const int64_t id = t / da.groups, g = t - id * da.groups;
    da.grp[id * (da.groups + 1) + g] = 0;
    if (g == 0) da.grp[id * (da.groups + 1) + da.groups] = 0;
    da.grp_rep[t] = INT_MAX;
    if constexpr (Elem<T>::kFloat) {
        if (!da.boxes) return;
        using U = typename OrdKey<T>::U;
        U* box = static_cast<U*>(da.box) + (size_t)t * 2 * a.g.d;
        for (int k = 0; k < a.g.d; ++k) {
            box[k] = ~U(0);
            box[a.g.d + k] = U(0);
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(256) k_dense_assign(QueryArgs<T> a, DenseArgs da) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int d = a.g.d;
    bool ok = i < a.n;
    int c = 0, id = -1, g = 0;
    if (ok) {
        c = (int)a.cellrank[i];
        id = da.dense_id[c];
        ok = id >= 0;
    }
    if (ok) {
        int mul = 1;
        for (int sd = 0; sd < d; ++sd) {
            const int j = a.g.swapped[sd];
            const double v = ((double)a.coords[(size_t)j * a.n + i] - da.mins_d[j]) * da.scale;
            long long sub = (long long)floor(v) - (long long)da.k * (long long)a.ct.ccoord[(size_t)sd * a.ct.pitch + c];
            sub = sub < 0 ? 0 : (sub >= da.k ? da.k - 1 : sub);
            g += (int)sub * mul;
            mul *= da.k;
        }
        da.gidx[i] = g;
    }
    agg_atomic_add(da.grp, ok ? id * (da.groups + 1) + g : 0, ok);
    if (!da.boxes) return;
    if constexpr (Elem<T>::kFloat) {
        using U = typename OrdKey<T>::U;
        U* box = static_cast<U*>(da.box) + ((size_t)(ok ? id : 0) * da.groups + g) * 2 * d;
        const unsigned peers = __match_any_sync(0xffffffffu, ok ? id * da.groups + g : -1);
        const bool leader = (int)lane_id() == __ffs(peers) - 1;
        for (int k = 0; k < d; ++k) {
            const U kv = ok ? OrdKey<T>::enc(a.coords[(size_t)k * a.n + i]) : U(0);
            if constexpr (sizeof(U) == 4) {
                if (ok) {
                    const U lo = __reduce_min_sync(peers, kv), hi = __reduce_max_sync(peers, kv);
                    if (leader) {
                        atomicMin(box + k, lo);
                        atomicMax(box + d + k, hi);
                    }
                }
            } else if (ok) {
                atomicMin(box + k, kv);
                atomicMax(box + d + k, kv);
            }
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(128) k_dense_offsets(QueryArgs<T> a, DenseArgs da) {
    const int id = blockIdx.x * 4 + (threadIdx.x >> 5);
    if (id >= *da.n_dense) return;
    const int lane = (int)lane_id();
    int* grp = da.grp + (size_t)id * (da.groups + 1);
    int run = 0;
    for (int g0 = 0; g0 < da.groups; g0 += 32) {
        const int g = g0 + lane;
        const int v = g < da.groups ? grp[g] : 0;
        int inc = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += y;
        }
        if (g < da.groups) {
            grp[g] = run + inc - v;
            da.cur[(size_t)id * da.groups + g] = run + inc - v;
        }
        run += __shfl_sync(0xffffffffu, inc, 31);
    }
    if (lane == 0) grp[da.groups] = run;
    if (!da.boxes) return;
    if constexpr (Elem<T>::kFloat) {
        using U = typename OrdKey<T>::U;
        const size_t nb = (size_t)da.groups * 2 * a.g.d;
        U* key = static_cast<U*>(da.box) + (size_t)id * nb;
        T* val = static_cast<T*>(da.box) + (size_t)id * nb;
        for (size_t t = lane; t < nb; t += 32) val[t] = OrdKey<T>::dec(key[t]);
    }
}

template <typename T>
__global__ void __launch_bounds__(256) k_dense_scatter(QueryArgs<T> a, DenseArgs da) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool ok = i < a.n;
    int c = 0, id = -1;
    if (ok) {
        c = (int)a.cellrank[i];
        id = da.dense_id[c];
        ok = id >= 0;
    }
    const int g = ok ? da.gidx[i] : 0;
    const int slot = agg_reserve(da.cur, ok ? id * da.groups + g : 0, ok);
    if (ok) {
        const int s0 = a.ct.start[c];
        da.sec[s0 + slot] = (int)i;
        if (da.boxes) {
            T* dc = static_cast<T*>(da.coords);
            for (int k = 0; k < a.g.d; ++k) dc[(size_t)k * a.n + s0 + slot] = a.coords[(size_t)k * a.n + i];
        }
    }
}

// Stars over the sub-cell cliques (after the core test, before any other union): the
// smallest core of every sub-cell (k_dense_rep) becomes the parent of the others
// (k_dense_link).  Parallel over points.
template <typename T>
__global__ void __launch_bounds__(256) k_dense_rep(QueryArgs<T> a, DenseArgs da) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool ok = i < a.n && a.core[i];
    int id = -1;
    if (ok) {
        id = da.dense_id[a.cellrank[i]];
        ok = id >= 0;
    }
    agg_atomic_min(da.grp_rep, ok ? id * da.groups + da.gidx[i] : 0, (int)i, ok);
}

template <typename T>
__global__ void __launch_bounds__(256) k_dense_link(QueryArgs<T> a, DenseArgs da) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n || !a.core[i]) return;
    const int id = da.dense_id[a.cellrank[i]];
    if (id < 0) return;
    const int r = da.grp_rep[(size_t)id * da.groups + da.gidx[i]];
    if (r != (int)i) a.parent[i] = r;
}

// warp per dense cell: a cell with >= kPruneMinPoints points flags every cell of its
// 3^d block (itself included) with kCellNearBig.  Every writer sets the same bit of a
// byte whose other bit no longer changes, so the unsynchronised updates agree.
template <typename T>
__global__ void __launch_bounds__(128) k_mark_near_big(QueryArgs<T> a, DenseArgs da) {
    const int id = blockIdx.x * 4 + (threadIdx.x >> 5);
    if (id >= *da.n_dense) return;
    const int c = da.cells[id];
    if (a.ct.start[c + 1] - a.ct.start[c] < kPruneMinPoints) return;
    visit_stencil(a.g, a.ct, c, 0, [&](int cr, bool) {
        if (lane_id() == 0) a.cell_flags[cr] |= kCellNearBig;
        return true;
    });
}

__device__ __forceinline__ bool same_component(int* parent, int x, int y);

// squared distance between two sub-cell boxes exceeds eps^2 (with the box-test margin)
template <typename T>
__device__ __forceinline__ bool boxes_apart(const T* b1, const T* b2, int d, BoxReal<T> eps2) {
    using R = BoxReal<T>;
    R s2 = 0;
    for (int k = 0; k < d; ++k) {
        R gap = (R)b2[k] - (R)b1[d + k];
        const R g2 = (R)b1[k] - (R)b2[d + k];
        gap = gap > g2 ? gap : g2;
        if (gap > R(0)) s2 += gap * gap;
    }
    return s2 > eps2 * R(1.0001);
}

// warp per dense cell: connect its sub-cells pairwise.  Sub-cell pairs whose boxes are
// farther apart than eps, or already in one component, are skipped; otherwise the
// lanes take 32 cores of the first sub-cell at a time (those within reach of the
// second sub-cell's box) and stream the second sub-cell's cores past them until one
// core-core eps pair is found, which is united.
template <typename T, int M, int D>
__global__ void __launch_bounds__(128) k_dense_pairs(QueryArgs<T> a, DenseArgs da) {
    const int id = blockIdx.x * 4 + (threadIdx.x >> 5);
    if (id >= *da.n_dense) return;
    const unsigned lane = lane_id();
    const int d = a.g.d;
    const int c = da.cells[id];
    const int s0 = a.ct.start[c];
    const int* grp = da.grp + (size_t)id * (da.groups + 1);
    const int* rep = da.grp_rep + (size_t)id * da.groups;
    const T* box = a.dense_box + (size_t)id * da.groups * 2 * d;
    const BoxReal<T> eps2 = (BoxReal<T>)a.eps2;
    for (int g1 = 0; g1 < da.groups; ++g1) {
        if (rep[g1] == INT_MAX) continue;
        for (int g2 = g1 + 1; g2 < da.groups; ++g2) {
            if (rep[g2] == INT_MAX) continue;
            if (da.boxes && boxes_apart(box + (size_t)g1 * 2 * d, box + (size_t)g2 * 2 * d, d, eps2)) continue;
            if (same_component(a.parent, rep[g1], rep[g2])) continue;
            bool joined = false;
            for (int x0 = grp[g1]; x0 < grp[g1 + 1] && !joined; x0 += 32) {
                const int x = x0 + (int)lane;
                int pa = -1;
                T qa[D > 0 ? D : kMaxDims];
                if (x < grp[g1 + 1]) {
                    pa = da.sec[s0 + x];
#pragma unroll
                    for (int k = 0; k < (D > 0 ? D : kMaxDims); ++k) {
                        if (D == 0 && k >= d) break;
                        qa[k] = a.coords[(size_t)k * a.n + pa];
                    }
                    if (!a.core[pa] || (da.boxes && box_class<T, D>(qa, box + (size_t)g2 * 2 * d, d, eps2) == kBoxFar))
                        pa = -1;
                }
                if (!__any_sync(0xffffffffu, pa >= 0)) continue;
                for (int y0 = grp[g2]; y0 < grp[g2 + 1] && !joined; y0 += 32) {
                    const int y = y0 + (int)lane;
                    int pb = -1;
                    T cb[D > 0 ? D : kMaxDims];
                    if (y < grp[g2 + 1]) {
                        const int j = da.sec[s0 + y];
                        pb = a.core[j] ? j : -1;
#pragma unroll
                        for (int k = 0; k < (D > 0 ? D : kMaxDims); ++k) {
                            if (D == 0 && k >= d) break;
                            cb[k] = a.coords[(size_t)k * a.n + j];
                        }
                    }
                    unsigned cand = __ballot_sync(0xffffffffu, pb >= 0);
                    while (cand && !joined) {
                        const int u = __ffs(cand) - 1;
                        cand &= cand - 1;
                        T cu[D > 0 ? D : kMaxDims];
#pragma unroll
                        for (int k = 0; k < (D > 0 ? D : kMaxDims); ++k) {
                            if (D == 0 && k >= d) break;
                            cu[k] = shfl_val(cb[k], u);
                        }
                        const unsigned hit = __ballot_sync(0xffffffffu, pa >= 0 && within_vals<T, M, D>(a, qa, cu));
                        if (hit) {
                            const int src = __ffs(hit) - 1;
                            const int xa = __shfl_sync(0xffffffffu, pa, src);
                            const int yb = __shfl_sync(0xffffffffu, pb, u);
                            if (lane == 0) uf_union(a.parent, xa, yb);
                            __syncwarp();
                            joined = true;
                        }
                    }
                }
            }
        }
    }
}

// warp-uniform "same component" test of two cores (lane 0 decides)
__device__ __forceinline__ bool same_component(int* parent, int x, int y) {
    int same = 0;
    if (lane_id() == 0) same = uf_find(parent, x) == uf_find(parent, y);
    return __shfl_sync(0xffffffffu, same, 0) != 0;
}

template <typename T, int M, int D>
__global__ void __launch_bounds__(128) k_union_cross(QueryArgs<T> a) {
    const int item = blockIdx.x * 4 + (threadIdx.x >> 5);
    if (item >= a.n_items) return;
    const int2 it = a.items[item];
    const int r = it.x;
    const int pend = min(it.y + 32, a.ct.start[r + 1]);
    const int p = it.y + (int)lane_id();
    const bool active = p < pend && a.core[p];
    if (!__any_sync(0xffffffffu, active)) return;
    const Tile<T> tile = warp_tile<T>(a.g.d);
    T q[D > 0 ? D : kMaxDims];
    load_query<T, D>(a, p, active, q);
    int myroot = active ? uf_find(a.parent, p) : -1;
    const bool uni_r = (a.cell_flags[r] & kCellUniform) != 0;
    const int rep_r = a.cell_rep[r];
    auto test = [&](int, int u) { return active && within<T, M, D>(a, q, tile, u); };
    auto aux_of = [&](int j) { return uf_find(a.parent, j); };
    auto on_hit = [&](int qi, int, int rep) {
        if (rep == myroot) return;
        uf_union(a.parent, p, qi);
        myroot = uf_find(a.parent, p);
    };
    (void)rep_r;
    // pairs of single-component cells are joined by k_union_cells
    visit_stencil(a.g, a.ct, r, 1, [&](int cr, bool own) {
        if (own) return true;
        auto never = []() { return false; };
        scan_range_hits(a, tile, a.ct.start[cr], a.ct.start[cr + 1], test, aux_of, on_hit, never);
        return true;
    }, false, [&](int cr) { return a.cell_rep[cr] != kNoCore && !(uni_r && (a.cell_flags[cr] & kCellUniform)); });
}

// Cross-cell unions between single-component cells, one warp per cell: for each
// lower neighbour cell that is also single-component and not yet in the same
// component, the lanes take 32 cores of the cell at a time and stream the
// neighbour's cores past them until one core-core eps pair is found, which joins the
// two components (a single pair suffices).
template <typename T, int M, int D>
__global__ void __launch_bounds__(128) k_union_cells(QueryArgs<T> a) {
    const int c = blockIdx.x * 4 + (threadIdx.x >> 5);
    if (c >= a.ct.m) return;
    const int rep_c = a.cell_rep[c];
    if (rep_c == kNoCore || !(a.cell_flags[c] & kCellUniform)) return;
    const unsigned lane = lane_id();
    const int d = a.g.d;
    const int cs = a.ct.start[c], ce = a.ct.start[c + 1];
    visit_stencil(a.g, a.ct, c, 1, [&](int cr, bool own) {
        if (own) return true;
        const int rep_n = a.cell_rep[cr];
        if (same_component(a.parent, rep_c, rep_n)) return true;
        const int ns = a.ct.start[cr], ne = a.ct.start[cr + 1];
        bool joined = false;
        for (int x0 = cs; x0 < ce && !joined; x0 += 32) {
            const int x = x0 + (int)lane;
            const bool ca = x < ce && a.core[x];
            if (!__any_sync(0xffffffffu, ca)) continue;
            T qa[D > 0 ? D : kMaxDims];
            load_query<T, D>(a, x, ca, qa);
            for (int y0 = ns; y0 < ne && !joined; y0 += 32) {
                const int y = y0 + (int)lane;
                const bool cb = y < ne && a.core[y];
                T vb[D > 0 ? D : kMaxDims];
                load_query<T, D>(a, y, cb, vb);
                unsigned cand = __ballot_sync(0xffffffffu, cb);
                while (cand) {
                    const int u = __ffs(cand) - 1;
                    cand &= cand - 1;
                    T cu[D > 0 ? D : kMaxDims];
#pragma unroll
                    for (int k = 0; k < (D > 0 ? D : kMaxDims); ++k) {
                        if (D == 0 && k >= d) break;
                        cu[k] = shfl_val(vb[k], u);
                    }
                    const unsigned hit = __ballot_sync(0xffffffffu, ca && within_vals<T, M, D>(a, qa, cu));
                    if (hit) {
                        const int xa = x0 + __ffs(hit) - 1;
                        if (lane == 0) uf_union(a.parent, xa, y0 + u);
                        __syncwarp();
                        joined = true;
                        break;
                    }
                }
            }
        }
        return true;
    }, false, [&](int cr) { return a.cell_rep[cr] != kNoCore && (a.cell_flags[cr] & kCellUniform); });
}

// Every core points at its component root; counts the cores (one atomic per warp).
// The walk to the root only reads, so the only value ever written is a root: a
// path-halving find here could overwrite another thread's root with a stale
// grandparent and leave a core pointing below its root.
static __global__ void k_compress(int* parent, const uint8_t* core, int n, int* n_core) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool c = i < n && core[i];
    if (c) {
        int x = i;
        for (;;) {  // parents strictly decrease along the walk, so it ends
            const int up = ld_volatile(parent + x);
            if (up == x) break;
            x = up;
        }
        parent[i] = x;
    }
    const unsigned m = __ballot_sync(0xffffffffu, c);
    if (lane_id() == 0 && m) atomicAdd(n_core, __popc(m));
}

// ---------------------------------------------------------- border assignment
// A non-core point with core neighbours of a single component joins it; with
// several it is recorded as ambiguous for the tie-break.  Cells without cores,
// and single-component cells of the component already found, are skipped.
template <typename T, int M, int D, bool PRUNE>
__global__ void __launch_bounds__(128) k_border(QueryArgs<T> a) {
    const int item = blockIdx.x * 4 + (threadIdx.x >> 5);
    if (item >= a.n_items) return;
    const int2 it = a.items[item];
    const int r = it.x;
    // cells next to a big dense cell are handled by the PRUNE instantiation
    if (((a.cell_flags[r] & kCellNearBig) != 0) != PRUNE) return;
    const int pend = min(it.y + 32, a.ct.start[r + 1]);
    const int p = it.y + (int)lane_id();
    const bool active = p < pend && !a.core[p];
    if (!__any_sync(0xffffffffu, active)) return;
    const Tile<T> tile = warp_tile<T>(a.g.d);
    T q[D > 0 ? D : kMaxDims];
    load_query<T, D>(a, p, active, q);
    int r1 = -1;
    bool multi = false;
    auto aux_of = [&](int j) { return a.core[j] ? a.parent[j] : -1; };
    auto hit = [&](int rep) {  // a core of component rep lies within eps
        if (r1 < 0) r1 = rep;
        else if (rep != r1) { multi = true; r1 = min(r1, rep); }
    };
    auto pair = [&](int, int u, int rep) {
        if (!active || multi || rep < 0 || rep == r1) return;
        if (within<T, M, D>(a, q, tile, u)) hit(rep);
    };
    auto done = [&]() { return __all_sync(0xffffffffu, !active || multi); };
    visit_stencil(a.g, a.ct, r, 0, [&](int cr, bool) {
        const int rep_c = a.cell_rep[cr];
        if (rep_c == kNoCore) return true;
        const bool dense = PRUNE && pruned_cell(a, cr);
        // sub-cells are cliques, so the cores of one sub-cell share a component: a
        // sub-cell wholly within eps that holds a core is a hit without a scan
        const int* grep = dense ? a.dense_rep + (size_t)a.dense_id[cr] * a.dense_groups : nullptr;
        auto visit_group = [&](int g, int cls) -> bool {
            const int rc = grep[g];
            if (rc == INT_MAX) return false;  // no core in the sub-cell
            if (cls == kBoxIn && !multi) hit(a.parent[rc]);
            return __any_sync(0xffffffffu, cls == kBoxEdge && !multi);
        };
        if (a.cell_flags[cr] & kCellUniform) {
            // every core of the cell is in component root_c: once each lane holds it
            // (or two clusters), the rest of the cell changes nothing
            const int root_c = a.parent[rep_c];
            auto cell_done = [&]() { return __all_sync(0xffffffffu, !active || multi || r1 == root_c); };
            if (cell_done()) return true;
            if constexpr (PRUNE) {
                if (dense) scan_dense<T, D>(a, tile, cr, q, active && !multi, visit_group, aux_of, pair, cell_done);
                else scan_range(a, tile, a.ct.start[cr], a.ct.start[cr + 1], aux_of, pair, cell_done);
            } else {
                scan_range(a, tile, a.ct.start[cr], a.ct.start[cr + 1], aux_of, pair, cell_done);
            }
            return !done();
        }
        if constexpr (PRUNE) {
            if (dense) return !scan_dense<T, D>(a, tile, cr, q, active && !multi, visit_group, aux_of, pair, done);
        }
        return !scan_range(a, tile, a.ct.start[cr], a.ct.start[cr + 1], aux_of, pair, done);
    }, false, [&](int cr) { return a.cell_rep[cr] != kNoCore; });
    if (active) {
        a.broot[p] = r1;
        if (multi) a.amb[atomicAdd(a.n_amb, 1)] = p;
    }
}

// ------------------------------------------------------------------ tie-break
// The single-threaded reference labels a border point with the component of the
// core neighbour q whose provisional label L(q) is smallest, where
//   L(p) = min(p + 1, min{ L(q) : q < p, q a core eps-neighbour of p })
// (hpdbscan.h:72-92: a core takes the smallest label among its already labelled
// core neighbours and every border keeps the minimum label offered to it).
// L(p) - 1 is therefore the smallest position reachable from p along core edges
// of strictly decreasing position.  It is computed on the components that touch
// an ambiguous border by monotone relaxation over decreasing edges plus pointer
// jumping (L(p) - 1 is itself reachable from p, so L(L(p) - 1) may be taken),
// iterated until an edge pass changes nothing.

// Candidate-parallel scan of the full stencil around one point (warp-uniform).
template <typename T, int M, int D, class Hit>
__device__ __forceinline__ void scan_point(const QueryArgs<T>& a, int p, Hit&& hit) {
    const unsigned lane = lane_id();
    T q[D > 0 ? D : kMaxDims];
#pragma unroll
    for (int k = 0; k < (D > 0 ? D : kMaxDims); ++k) {
        if (D == 0 && k >= a.g.d) break;
        q[k] = a.coords[(size_t)k * a.n + p];
    }
    // the cell of p: binary search on cell starts
    int lo = 0, hi = a.ct.m;
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (a.ct.start[mid] <= p) lo = mid; else hi = mid;
    }
    visit_stencil(a.g, a.ct, lo, 0, [&](int cr, bool) {
        const int ce = a.ct.start[cr + 1];
        for (int j = a.ct.start[cr] + (int)lane; j < ce; j += 32) {
            if (!a.core[j]) continue;
            T c[D > 0 ? D : kMaxDims];
#pragma unroll
            for (int k = 0; k < (D > 0 ? D : kMaxDims); ++k) {
                if (D == 0 && k >= a.g.d) break;
                c[k] = a.coords[(size_t)k * a.n + j];
            }
            bool in;
            if constexpr (!Elem<T>::kFloat) {
                in = int_within<T, D>(q, c, a.g.d, a.eps2);
            } else {
                T t[D > 0 ? D : kMaxDims];
#pragma unroll
                for (int k = 0; k < (D > 0 ? D : kMaxDims); ++k) {
                    if (D == 0 && k >= a.g.d) break;
                    t[k] = sub_(q[k], c[k]);
                }
                in = fold_sq<T, M, D>(t, a.g.d) <= a.eps2;
            }
            if (in) hit(j);
        }
        return true;
    });
}

template <typename T, int M, int D>
__global__ void __launch_bounds__(128) k_tie_mark(QueryArgs<T> a) {
    const int w = blockIdx.x * 4 + (threadIdx.x >> 5);
    if (w >= *a.n_amb) return;
    const int b = a.amb[w];
    if (!in_range(a.guard, b, a.n, kGuardAmbiguous)) return;
    // r1 < r2: the two smallest roots next to b
    int r1 = INT_MAX, r2 = INT_MAX;
    scan_point<T, M, D>(a, b, [&](int j) {
        const int x = a.parent[j];
        if (!in_range(a.guard, x, a.n, kGuardRoot)) return;
        atomicMax(a.tmax + x, j);
        if (x < r1) {
            r2 = r1;
            r1 = x;
        } else if (x != r1 && x < r2) {
            r2 = x;
        }
    });
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const int b1 = __shfl_xor_sync(0xffffffffu, r1, o), b2 = __shfl_xor_sync(0xffffffffu, r2, o);
        const int n1 = min(r1, b1);
        const int n2 = r1 == b1 ? min(r2, b2) : (r1 < b1 ? min(r2, b1) : min(b2, r1));
        r1 = n1;
        r2 = n2;
    }
    // The component of r1 wins b as soon as one of its cores next to b holds a value
    // below r2 (every other value is at least r2), so its values need no improvement
    // below r2; every other component's values must be exact (threshold root + 1).
    scan_point<T, M, D>(a, b, [&](int j) {
        const int x = a.parent[j];
        if (in_range(a.guard, x, a.n, kGuardRoot)) atomicMin(a.tlow + x, x == r1 ? r2 : x + 1);
    });
}

// Smallest-id tie-break: an ambiguous border takes the smallest root (cluster id)
// among all its core eps-neighbours (k_border stops at the second cluster found).
template <typename T, int M, int D>
__global__ void __launch_bounds__(128) k_tie_min_root(QueryArgs<T> a) {
    const int w = blockIdx.x * 4 + (threadIdx.x >> 5);
    if (w >= *a.n_amb) return;
    const int p = a.amb[w];
    if (!in_range(a.guard, p, a.n, kGuardAmbiguous)) return;
    scan_point<T, M, D>(a, p, [&](int j) { atomicMin(a.broot + p, a.parent[j]); });
}

static __global__ void k_tie_init(const uint8_t* core, int* lm1, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) lm1[i] = core[i] ? i : INT_MAX;
}

template <typename T>
__device__ __forceinline__ void mark_dirty_cell(const QueryArgs<T>& a, int c) {
    if (!in_range(a.guard, c, a.ct.m, kGuardDirtyCell)) return;
    if (atomicMax(a.dirty_gen + c, a.gen) < a.gen) {
        const int k = atomicAdd(a.n_dlist, 1);
        if (in_range(a.guard, k, a.ct.m, kGuardDirtyList)) a.dlist[k] = c;
    }
}

// One relaxation pass over decreasing core edges for one work item.  Only
// candidates in cells dirtied since the previous pass are rescanned: for every
// other candidate q the query already holds L(p) <= L(q) from an earlier pass.
// Lower cells are scanned first and the result is published at once; the own
// cell is then rescanned until no lane of the warp improves, so that chains of
// improvements inside one chunk settle within this pass.
template <typename T, int M, int D>
__device__ __forceinline__ void tie_edge_item(const QueryArgs<T>& a, int item) {
    if (!in_range(a.guard, item, a.n_items, kGuardItem)) return;
    const int2 it = a.items[item];
    const int r = it.x;
    if (!in_range(a.guard, r, a.ct.m, kGuardCellRank) || !in_range(a.guard, it.y, a.n, kGuardItem)) return;
    const int pend = min(it.y + 32, a.ct.start[r + 1]);
    const int p = it.y + (int)lane_id();
    bool active = p < pend && a.core[p];
    const int root = active ? a.parent[p] : INT_MIN;
    if (active && !in_range(a.guard, root, a.n, kGuardRoot)) active = false;
    // a core whose value is below its component's threshold (at least root + 1: the
    // root is the smallest value possible) needs no further improvement
    int tl = INT_MIN;
    if (active) {
        tl = a.tlow[root];
        active = p <= a.tmax[root] && ld_volatile(a.lm1 + p) >= tl;
    }
    if (!__any_sync(0xffffffffu, active)) return;
    if (a.trace_counts) {
        const unsigned am = __ballot_sync(0xffffffffu, active);  // every lane takes part
        if (lane_id() == 0) atomicAdd(a.trace_counts, (unsigned long long)__popc(am));
    }
    const Tile<T> tile = warp_tile<T>(a.g.d);
    T q[D > 0 ? D : kMaxDims];
    load_query<T, D>(a, p, active, q);
    const int start_l = active ? ld_volatile(a.lm1 + p) : INT_MAX;
    int myl = start_l;
    int published = start_l;
    const int since = a.gen - 1;
    auto aux_of = [&](int j) { return a.core[j] ? ld_volatile(a.lm1 + j) : INT_MAX; };
    auto pair = [&](int qi, int u, int lq) {
        if (!active || lq >= myl || qi >= p) return;
        if (within<T, M, D>(a, q, tile, u)) myl = lq;
    };
    auto publish = [&]() {
        const bool better = active && myl < published;
        if (better) {
            atomicMin(a.lm1 + p, myl);
            atomicMin(a.cell_min_l + r, myl);
            atomicMin(a.item_min_l + item, myl);
            published = myl;
        }
        return better;
    };
    auto never = []() { return false; };
    // a lane is finished once its value is below its component's threshold
    auto settled = [&]() { return __all_sync(0xffffffffu, !active || myl < tl); };
    // tiles are aligned with the 32-point chunks of a cell, so each tile is one work
    // item; a tile whose smallest value cannot improve any lane is skipped unread
    auto scan_pruned = [&](int cr, int cs, int ce, int worst) {
        const int first_item = (int)a.ipos[a.ct.start[cr]];
        for (int t0 = cs; t0 < ce; t0 += 32) {
            const int ti = first_item + ((t0 - a.ct.start[cr]) >> 5);
            if (!in_range(a.guard, ti, a.n_items, kGuardItemIndex)) return false;
            if (ld_volatile(a.item_min_l + ti) >= worst) continue;
            if (a.trace_counts && lane_id() == 0) atomicAdd(a.trace_counts + 1, 1ull);
            if (scan_range(a, tile, t0, min(t0 + 32, ce), aux_of, pair, settled)) return true;
        }
        return false;
    };
    const bool own_dirty = ld_volatile(a.dirty_gen + r) >= since;
    int worst0 = active ? myl : INT_MIN;  // largest lane value at the start: a cell must beat it
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) worst0 = max(worst0, __shfl_xor_sync(0xffffffffu, worst0, o));
    visit_stencil(a.g, a.ct, r, 1, [&](int cr, bool own) {
        if (own) {
            // own cell: the lower chunks once, then the warp's own chunk until no
            // lane improves (at most one round per lane), publishing every round
            const bool improved = publish();
            if (!own_dirty && !__any_sync(0xffffffffu, improved)) return true;
            if (!settled()) {
                int worst = (active && myl >= tl) ? myl : INT_MIN;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) worst = max(worst, __shfl_xor_sync(0xffffffffu, worst, o));
                scan_pruned(r, a.ct.start[r], it.y, worst);
            }
            bool again = !settled();
            for (int round = 0; again && round < 33; ++round) {
                publish();
                scan_range(a, tile, it.y, pend, aux_of, pair, never);
                again = __any_sync(0xffffffffu, active && myl < published);
            }
            publish();
            return true;
        }
        if (ld_volatile(a.dirty_gen + cr) < since) return true;
        const int rep_c = a.cell_rep[cr];
        if (rep_c == kNoCore) return true;
        if ((a.cell_flags[cr] & kCellUniform) && tmax_of(a, rep_c) < a.ct.start[cr]) return true;
        // no core of that cell holds a value below any lane's: nothing to gain
        if (settled()) return true;
        int worst = (active && myl >= tl) ? myl : INT_MIN;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) worst = max(worst, __shfl_xor_sync(0xffffffffu, worst, o));
        if (ld_volatile(a.cell_min_l + cr) >= worst) return true;
        scan_pruned(cr, a.ct.start[cr], a.ct.start[cr + 1], worst);
        return true;
    }, /*own_last=*/true, [&](int cr) {
        if (ld_volatile(a.dirty_gen + cr) < since) return false;
        const int rep_c = a.cell_rep[cr];
        if (rep_c == kNoCore) return false;
        if ((a.cell_flags[cr] & kCellUniform) && tmax_of(a, rep_c) < a.ct.start[cr]) return false;
        return ld_volatile(a.cell_min_l + cr) < worst0;
    });
    if (__any_sync(0xffffffffu, active && myl < start_l) && lane_id() == 0) mark_dirty_cell(a, r);
}

template <typename T, int M, int D>
__global__ void __launch_bounds__(128) k_tie_edge(QueryArgs<T> a) {
    const int item = blockIdx.x * 4 + (threadIdx.x >> 5);
    if (item >= a.n_items) return;
    tie_edge_item<T, M, D>(a, item);
}

// Same pass over a work list (sorted by item, so lower positions go first), by a
// fixed grid of warps that take the next item from a shared ticket.
template <typename T, int M, int D>
__global__ void __launch_bounds__(128) k_tie_edge_list(QueryArgs<T> a) {
    int cnt = *a.n_wlist;
    if (!in_range(a.guard, cnt, (long long)a.n_items + 1, kGuardCount)) cnt = 0;
    for (;;) {
        int wi = 0;
        if (lane_id() == 0) wi = atomicAdd(a.ticket, 1);
        wi = __shfl_sync(0xffffffffu, wi, 0);
        if (wi >= cnt) return;
        tie_edge_item<T, M, D>(a, a.wlist[wi]);
    }
}

// Pointer jumping: L(p) - 1 is reachable from p, so L(p) may take L(L(p) - 1).
template <typename T>
__global__ void k_tie_jump(QueryArgs<T> a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    int l = ld_volatile(a.lm1 + i);
    if (l == INT_MAX || l == i) return;
    const int l0 = l;
    for (;;) {  // strictly decreasing, so at most n steps
        if (!in_range(a.guard, l, a.n, kGuardLabel)) return;
        const int ll = ld_volatile(a.lm1 + l);
        if (ll >= l) break;
        l = ll;
    }
    if (l < l0) {
        atomicMin(a.lm1 + i, l);
        const int c = (int)a.cellrank[i];
        if (!in_range(a.guard, c, a.ct.m, kGuardCellRank)) return;
        atomicMin(a.cell_min_l + c, l);
        const int s0 = a.ct.start[c];
        const int ti = (int)a.ipos[s0] + ((i - s0) >> 5);
        if (!in_range(a.guard, ti, a.n_items, kGuardItemIndex)) return;
        atomicMin(a.item_min_l + ti, l);
        if (a.gen > 0) mark_dirty_cell(a, c);
    }
}

// per-cell minimum of the current values of its cores
template <typename T>
__global__ void k_tie_cell_min(QueryArgs<T> a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    bool ok = i < a.n && a.core[i];
    const int c = ok ? (int)a.cellrank[i] : 0;
    if (ok && !in_range(a.guard, c, a.ct.m, kGuardCellRank)) ok = false;
    const int v = ok ? a.lm1[i] : 0;
    agg_atomic_min(a.cell_min_l, c, v, ok);
    int ti = 0;
    if (ok) {
        const int s0 = a.ct.start[c];
        ti = (int)a.ipos[s0] + ((i - s0) >> 5);
        if (!in_range(a.guard, ti, a.n_items, kGuardItemIndex)) ok = false;
    }
    agg_atomic_min(a.item_min_l, ti, v, ok);
}

// Next pass's work: the items of every cell whose lower stencil or own cell was
// dirtied in this pass are flagged (warp per dirty cell); k_tie_compact then lists the
// flagged items in increasing order.
template <typename T>
__global__ void __launch_bounds__(128) k_tie_schedule(QueryArgs<T> a) {
    const int nw = gridDim.x * 4;
    int cnt = *a.n_dlist;
    if (!in_range(a.guard, cnt, (long long)a.ct.m + 1, kGuardCount)) cnt = 0;
    const unsigned lane = lane_id();
    for (int w = blockIdx.x * 4 + (threadIdx.x >> 5); w < cnt; w += nw) {
        const int c = a.dlist[w];
        if (!in_range(a.guard, c, a.ct.m, kGuardDirtyCell)) continue;
        visit_stencil(a.g, a.ct, c, 2, [&](int cr, bool) {
            const int rep_c = a.cell_rep[cr];
            if (rep_c == kNoCore) return true;
            if ((a.cell_flags[cr] & kCellUniform) && tmax_of(a, rep_c) < a.ct.start[cr]) return true;
            int fresh = 0;
            if (lane == 0) fresh = atomicMax(a.sched_gen + cr, a.gen) < a.gen;
            if (!__shfl_sync(0xffffffffu, fresh, 0)) return true;
            const int s0 = a.ct.start[cr];
            const int nit = (a.ct.start[cr + 1] - s0 + 31) >> 5;
            const int first = (int)a.ipos[s0];
            for (int k = (int)lane; k < nit; k += 32)
                if (in_range(a.guard, first + k, a.n_items, kGuardItemIndex)) a.item_flag[first + k] = 1u;
            return true;
        }, false, [&](int cr) {
            const int rep_c = a.cell_rep[cr];
            if (rep_c == kNoCore) return false;
            return !((a.cell_flags[cr] & kCellUniform) && tmax_of(a, rep_c) < a.ct.start[cr]);
        });
    }
}

// Lists the flagged items in increasing order (pos = exclusive scan of the flags)
// and clears the flags for the next pass.
static __global__ void k_tie_compact(uint32_t* item_flag, const uint32_t* pos, int n_items, int* wlist, int* guard) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n_items && item_flag[i]) {
        if (in_range(guard, pos[i], n_items, kGuardList)) wlist[pos[i]] = i;
        item_flag[i] = 0u;
    }
}

// Greedy descent step: g(p) = some core eps-neighbour below p (p itself if none).
// Any decreasing core edge leads to a position reachable from p, so following g
// from p (pointer jumping) ends at an upper bound of L(p) - 1, equal to the
// component root whenever the descent reaches it.  Each lane stops at its first hit.
template <typename T, int M, int D>
__global__ void __launch_bounds__(128) k_tie_greedy(QueryArgs<T> a) {
    const int item = blockIdx.x * 4 + (threadIdx.x >> 5);
    if (item >= a.n_items) return;
    const int2 it = a.items[item];
    const int r = it.x;
    const int pend = min(it.y + 32, a.ct.start[r + 1]);
    const int p = it.y + (int)lane_id();
    bool active = p < pend && a.core[p];
    if (active) {
        // positions below the component's threshold are settled already (value p)
        const int root = a.parent[p];
        active = p <= a.tmax[root] && p >= a.tlow[root];
    }
    if (!__any_sync(0xffffffffu, active)) return;
    const Tile<T> tile = warp_tile<T>(a.g.d);
    T q[D > 0 ? D : kMaxDims];
    load_query<T, D>(a, p, active, q);
    int g = active ? p : INT_MAX;
    bool found = !active;
    auto aux_of = [&](int j) { return (int)a.core[j]; };
    auto pair = [&](int qi, int u, int is_core) {
        if (found || !is_core || qi >= p) return;
        if (within<T, M, D>(a, q, tile, u)) { g = qi; found = true; }
    };
    auto done = [&]() { return __all_sync(0xffffffffu, found); };
    // lower positions of the own cell first (most pairs inside a cell are within eps),
    // then the lower face across the most significant dimension, then the rest
    bool all = scan_range(a, tile, a.ct.start[r], pend, aux_of, pair, done);
    const int top = a.g.d - 1;
    const unsigned long long key = a.ct.key[r];
    int face = -1;
    if (!all && a.ct.ccoord[(size_t)top * a.ct.pitch + r] > 0) face = find_cell(a.ct, key - a.g.stride[top]);
    if (face >= 0 && a.cell_rep[face] != kNoCore)
        all = scan_range(a, tile, a.ct.start[face], a.ct.start[face + 1], aux_of, pair, done);
    if (!all) {
        visit_stencil(a.g, a.ct, r, 1, [&](int cr, bool own) {
            if (own || cr == face || a.cell_rep[cr] == kNoCore) return true;
            return !scan_range(a, tile, a.ct.start[cr], a.ct.start[cr + 1], aux_of, pair, done);
        });
    }
    if (active) a.lm1[p] = g;
}

// Decides the ambiguous borders of the list (a.amb, *a.n_amb) that current bounds
// settle: lm1[q] is an upper bound of L(q) - 1 and the component root a lower
// bound, so the component holding the smallest upper bound wins as soon as that
// bound is below the root of every other adjacent component.  With `final` the
// values are exact and every border is decided.  Undecided borders are appended to
// (a.amb_out, *a.n_amb_out).
template <typename T, int M, int D>
__global__ void __launch_bounds__(128) k_tie_decide(QueryArgs<T> a, int final_pass) {
    const int w = blockIdx.x * 4 + (threadIdx.x >> 5);
    if (w >= *a.n_amb) return;
    const int b = a.amb[w];
    if (!in_range(a.guard, b, a.n, kGuardAmbiguous)) return;
    unsigned long long best = ~0ull;  // (upper bound of L - 1) << 32 | root
    scan_point<T, M, D>(a, b, [&](int j) {
        const unsigned long long v = ((unsigned long long)(unsigned)ld_volatile(a.lm1 + j) << 32) | (unsigned)a.parent[j];
        if (v < best) best = v;
    });
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long y = __shfl_xor_sync(0xffffffffu, best, o);
        if (y < best) best = y;
    }
    const int root_best = (int)(best & 0xffffffffu);
    const int ub = (int)(best >> 32);
    int other = INT_MAX;  // smallest root of the other adjacent components
    scan_point<T, M, D>(a, b, [&](int j) {
        const int rj = a.parent[j];
        if (rj != root_best && rj < other) other = rj;
    });
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) other = min(other, __shfl_xor_sync(0xffffffffu, other, o));
    if (lane_id() == 0) {
        if (final_pass || ub < other) a.broot[b] = root_best;
        else a.amb_out[atomicAdd(a.n_amb_out, 1)] = b;
    }
}

// ------------------------------------------------------------------- labels
// Signed labels (constants.h:36-37, hpdbscan.h:198-211): core -(root+1), border
// +(root+1), noise 0; scattered back to input order (spatial_index.h:852-872).
static __global__ void k_finalize(const uint8_t* core, const int* parent, const int* broot, const int32_t* perm, int n,
                           int64_t* labels) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int64_t lab;
    if (core[i]) lab = -(int64_t)parent[i] - 1;
    else lab = broot[i] >= 0 ? (int64_t)broot[i] + 1 : 0;
    labels[perm[i]] = lab;
}

}  // namespace hpd
