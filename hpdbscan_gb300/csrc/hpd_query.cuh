// Shared machinery of the query kernels (core test hpd_core.cuh, connectivity
// hpd_union.cuh, dense cells hpd_dense.cuh, borders and labels hpd_border.cuh,
// tie-break hpd_tie.cuh): the cell table and stencil walk, the kernel arguments, the
// candidate tiles and scans, the distance tests in the reference's arithmetic, the
// sub-cell box tests and the range guards.
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

// First cell rank whose key is at least `key` (m if none).
__device__ __forceinline__ int lower_cell(const CellTable& ct, unsigned long long key) {
    int lo = 0, hi = ct.m;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (ct.key[mid] < key) lo = mid + 1; else hi = mid;
    }
    return lo;
}

constexpr int kStencilDirectDims = 5;  // up to 3^5 offsets: every offset is enumerated

// The neighbour visit past kStencilDirectDims dimensions.  3^d offsets (43M at d =
// 16) would dwarf the occupied cells.  The block's neighbours have keys within
// [key - reach_lo, key + reach_hi] (stride s exceeds the reach of all lower
// positions), so the visit walks the cheaper of (a) the offsets that stay inside the
// grid, looked up one by one (mixed radix, dimension 0 fastest), and (b) the occupied
// cells of that key range, tested coordinate by coordinate.  Both hand out the same
// cells in the same ascending-key order as the direct enumeration.  wide_plan picks
// the walk, wide_cell gives a lane its candidate.
struct WidePlan {
    long long count;  // steps of the walk
    int first;        // range walk: first cell rank; -1: offset walk
};

__device__ __forceinline__ WidePlan wide_plan(const Grid& g, const CellTable& ct, int r, int sel) {
    const unsigned long long key = ct.key[r];
    long long valid = 1;
    unsigned long long reach_lo = 0, reach_hi = 0;
    for (int s = 0; s < g.d; ++s) {
        const unsigned long long c = ct.ccoord[(size_t)s * ct.pitch + r];
        const bool lo = c > 0, hi = c + 1 < g.dims[g.swapped[s]];
        valid *= 1 + (int)lo + (int)hi;
        if (lo) reach_lo += g.stride[s];
        if (hi) reach_hi += g.stride[s];
    }
    const unsigned long long klo = sel == 2 ? key + 1 : key - reach_lo;
    const unsigned long long khi = sel == 1 ? key - 1 : key + reach_hi;
    const int first = (sel == 1 && reach_lo == 0) ? r : lower_cell(ct, klo);
    const int last = (sel == 2 && reach_hi == 0) ? r : lower_cell(ct, khi + 1);  // one past the range
    if ((long long)(last - first) <= valid) return WidePlan{last > first ? last - first : 0, first};
    return WidePlan{valid, -1};
}

// Cell of step `step` of the walk (-1: not a neighbour, the own cell, or filtered by sel).
__device__ __forceinline__ int wide_cell(const Grid& g, const CellTable& ct, int r, int sel, WidePlan plan,
                                      long long step) {
    if (step >= plan.count) return -1;
    if (plan.first >= 0) {
        const int cr = plan.first + (int)step;
        if (cr == r) return -1;
        for (int s = 0; s < g.d; ++s) {
            const unsigned long long c = ct.ccoord[(size_t)s * ct.pitch + cr];
            const unsigned long long o = ct.ccoord[(size_t)s * ct.pitch + r];
            if (c + 1 < o || c > o + 1) return -1;
        }
        return cr;
    }
    const unsigned long long key = ct.key[r];
    long long rest = step;
    bool own = true;
    unsigned long long nk = key;
    for (int s = 0; s < g.d; ++s) {
        const unsigned long long c = ct.ccoord[(size_t)s * ct.pitch + r];
        const bool lo = c > 0, hi = c + 1 < g.dims[g.swapped[s]];
        const int n_dig = 1 + (int)lo + (int)hi;
        const int dig = (int)(rest % n_dig) + (lo ? 0 : 1);  // 0: -1, 1: same, 2: +1
        rest /= n_dig;
        if (dig == 0) nk -= g.stride[s];
        if (dig == 2) nk += g.stride[s];
        own = own && dig == 1;
    }
    if (own || (sel == 1 && nk >= key) || (sel == 2 && nk <= key)) return -1;
    if (ct.dense && !in_range(ct.guard, (long long)nk, (long long)g.total, kGuardStencilKey)) return -1;
    const int nr = find_cell(ct, nk);
    return (nr >= 0 && in_range(ct.guard, nr, ct.m, kGuardStencilCell)) ? nr : -1;
}

// DS: the caller's compiled dimension count: 2 or 3, 0 for other counts up to
// kStencilDirectDims (direct enumeration), -1 for counts past it (the wide walk; the
// pipeline compiles its kernels separately for those).
template <int DS = 0, class Fn, class Keep = KeepAll>
__device__ __forceinline__ void visit_stencil(const Grid& g, const CellTable& ct, int r, int sel, Fn&& fn,
                                              bool own_last = false, Keep keep = Keep()) {
    if (!own_last && !fn(r, true)) return;
    const unsigned lane = lane_id();
    if constexpr (DS < 0) {
        const WidePlan plan = wide_plan(g, ct, r, sel);
        for (long long b = 0; b < plan.count; b += 32) {
            int nr = wide_cell(g, ct, r, sel, plan, b + (long long)lane);
            if (nr >= 0 && !keep(nr)) nr = -1;
            unsigned mask = __ballot_sync(0xffffffffu, nr >= 0);
            while (mask) {
                const int src = __ffs(mask) - 1;
                mask &= mask - 1;
                const int cr = __shfl_sync(0xffffffffu, nr, src);
                if (!fn(cr, false)) return;
            }
        }
        if (own_last) fn(r, true);
        return;
    }
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
    unsigned long long* pair_count;  // diagnostic pass: distance evaluations of the core test
    int sparse_queries;   // work items of at most this many points take the core test's flat path
    int greedy_tiles;     // candidate tiles a work item of the greedy descent scans at most
    int4* chunks;         // tie-break chunk tasks (item, cell, first, end position) of a pass
    int* n_chunks;
    int chunk_cap;
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
        if (D <= 0 && k >= d) break;
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
            if (D <= 0 && k >= d) break;
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
        if (D <= 0 && k >= d) break;
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
            if (D <= 0 && k >= a.g.d) break;
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
            if (D <= 0 && k >= a.g.d) break;
            t[k] = sub_(q[k], c[k]);
        }
        return fold_sq<T, M, D>(t, a.g.d) <= a.eps2;
    }
}

template <typename T, int D>
__device__ __forceinline__ void load_query(const QueryArgs<T>& a, int p, bool active, T* q) {
#pragma unroll
    for (int k = 0; k < (D > 0 ? D : kMaxDims); ++k) {
        if (D <= 0 && k >= a.g.d) break;
        q[k] = active ? a.coords[(size_t)k * a.n + p] : T(0);
    }
}

}  // namespace hpd
