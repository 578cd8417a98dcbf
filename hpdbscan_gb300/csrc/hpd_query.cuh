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

#include "hpd_common.cuh"

namespace hpd {

struct CellTable {
    const int32_t* start;              // [m + 1] first sorted position of each cell
    const unsigned long long* key;     // [m] cell id
    const int32_t* dense;              // [grid total] cell rank or -1; nullptr -> binary search
    int m;
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

// Visits the item's own cell first, then the other non-empty cells of the 3^d
// block around it (only those with a smaller cell id when lower_only), calling
// fn(cell_rank, is_own) warp-uniformly; fn returns false to stop the visit.
template <class Fn>
__device__ __forceinline__ void visit_stencil(const Grid& g, const CellTable& ct, int r, bool lower_only, Fn&& fn) {
    if (!fn(r, true)) return;
    const unsigned lane = lane_id();
    const unsigned long long key = ct.key[r];
    unsigned long long coord[kMaxDims];
    for (int s = 0; s < g.d; ++s) coord[s] = (key / g.stride[s]) % g.dims[g.swapped[s]];
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
            if (ok && (!lower_only || nk < key)) nr = find_cell(ct, nk);
        }
        unsigned mask = __ballot_sync(0xffffffffu, nr >= 0);
        while (mask) {
            const int src = __ffs(mask) - 1;
            mask &= mask - 1;
            const int cr = __shfl_sync(0xffffffffu, nr, src);
            if (!fn(cr, false)) return;
        }
    }
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
    uint8_t* relevant;    // per root: component touches an ambiguous border
    int* lm1;             // tie-break value L - 1 (see k_tie_edge)
    int* changed;
};

// Per-warp tile in shared memory: d planes of 32 coordinates plus one aux word.
template <typename T>
struct Tile {
    T* c;    // [d][32]
    int* aux;  // [32]
};

template <typename T>
__device__ __forceinline__ Tile<T> warp_tile(int d) {
    extern __shared__ __align__(16) unsigned char smem_q[];
    const int w = threadIdx.x >> 5;
    const size_t per = (size_t)d * 32 * sizeof(T) + 32 * sizeof(int);
    unsigned char* base = smem_q + per * w;
    Tile<T> t;
    t.c = reinterpret_cast<T*>(base);
    t.aux = reinterpret_cast<int*>(base + (size_t)d * 32 * sizeof(T));
    return t;
}

// Streams candidates [cs, ce) through the tile; pair(q, u, aux) runs per lane for
// every candidate q (tile slot u); returns true when done() holds for the warp.
template <typename T, class Aux, class Pair, class Done>
__device__ __forceinline__ bool scan_range(const QueryArgs<T>& a, const Tile<T>& tile, int cs, int ce, Aux&& aux_of,
                                           Pair&& pair, Done&& done) {
    const int d = a.g.d;
    const unsigned lane = lane_id();
    for (int t0 = cs; t0 < ce; t0 += 32) {
        const int j = t0 + (int)lane;
        if (j < ce) {
            for (int k = 0; k < d; ++k) tile.c[k * 32 + lane] = a.coords[(size_t)k * a.n + j];
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

// squared distance from the lane's query (q[]) to tile slot u, compared with eps2
template <typename T, int M, int D>
__device__ __forceinline__ bool within(const QueryArgs<T>& a, const T* q, const Tile<T>& tile, int u) {
    T t[D > 0 ? D : kMaxDims];
#pragma unroll
    for (int k = 0; k < (D > 0 ? D : kMaxDims); ++k) {
        if (D == 0 && k >= a.g.d) break;
        t[k] = sub_(q[k], tile.c[k * 32 + u]);
    }
    return fold_sq<T, M, D>(t, a.g.d) <= a.eps2;
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
template <typename T, int M, int D>
__global__ void __launch_bounds__(128) k_core(QueryArgs<T> a) {
    const int item = blockIdx.x * 4 + (threadIdx.x >> 5);
    if (item >= a.n_items) return;
    const Tile<T> tile = warp_tile<T>(a.g.d);
    const int2 it = a.items[item];
    const int r = it.x;
    const int pend = min(it.y + 32, a.ct.start[r + 1]);
    const int p = it.y + (int)lane_id();
    const bool active = p < pend;
    T q[D > 0 ? D : kMaxDims];
    load_query<T, D>(a, p, active, q);
    int count = 0;
    const int limit = a.min_points;
    auto aux_of = [](int) { return 0; };
    auto pair = [&](int, int u, int) {
        if (active && count < limit && within<T, M, D>(a, q, tile, u)) ++count;
    };
    auto done = [&]() { return __all_sync(0xffffffffu, !active || count >= limit); };
    visit_stencil(a.g, a.ct, r, false, [&](int cr, bool) {
        return !scan_range(a, tile, a.ct.start[cr], a.ct.start[cr + 1], aux_of, pair, done);
    });
    if (active) a.core[p] = count >= limit ? 1 : 0;
}

// ---------------------------------------------------- core-core connectivity
// Every core-core eps edge (q < p) is united; candidates already in the query's
// component are skipped without a distance test.
template <typename T, int M, int D>
__global__ void __launch_bounds__(128) k_union(QueryArgs<T> a) {
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
    auto aux_of = [&](int j) { return a.core[j] ? uf_find(a.parent, j) : -1; };
    auto pair = [&](int qi, int u, int rep) {
        if (!active || rep < 0 || rep == myroot || qi >= p) return;
        if (within<T, M, D>(a, q, tile, u)) {
            uf_union(a.parent, p, qi);
            myroot = uf_find(a.parent, p);
        }
    };
    auto never = []() { return false; };
    visit_stencil(a.g, a.ct, r, true, [&](int cr, bool own) {
        const int ce = own ? pend : a.ct.start[cr + 1];
        scan_range(a, tile, a.ct.start[cr], ce, aux_of, pair, never);
        return true;
    });
}

static __global__ void k_compress(int* parent, const uint8_t* core, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && core[i]) parent[i] = uf_find(parent, i);
}

// ---------------------------------------------------------- border assignment
// A non-core point with core neighbours of a single component joins it; with
// several it is recorded as ambiguous for the tie-break.
template <typename T, int M, int D>
__global__ void __launch_bounds__(128) k_border(QueryArgs<T> a) {
    const int item = blockIdx.x * 4 + (threadIdx.x >> 5);
    if (item >= a.n_items) return;
    const int2 it = a.items[item];
    const int r = it.x;
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
    auto pair = [&](int, int u, int rep) {
        if (!active || multi || rep < 0 || rep == r1) return;
        if (within<T, M, D>(a, q, tile, u)) {
            if (r1 < 0) r1 = rep;
            else { multi = true; r1 = min(r1, rep); }
        }
    };
    auto done = [&]() { return __all_sync(0xffffffffu, !active || multi); };
    visit_stencil(a.g, a.ct, r, false, [&](int cr, bool) {
        return !scan_range(a, tile, a.ct.start[cr], a.ct.start[cr + 1], aux_of, pair, done);
    });
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
    visit_stencil(a.g, a.ct, lo, false, [&](int cr, bool) {
        const int ce = a.ct.start[cr + 1];
        for (int j = a.ct.start[cr] + (int)lane; j < ce; j += 32) {
            if (!a.core[j]) continue;
            T t[D > 0 ? D : kMaxDims];
#pragma unroll
            for (int k = 0; k < (D > 0 ? D : kMaxDims); ++k) {
                if (D == 0 && k >= a.g.d) break;
                t[k] = sub_(q[k], a.coords[(size_t)k * a.n + j]);
            }
            if (fold_sq<T, M, D>(t, a.g.d) <= a.eps2) hit(j);
        }
        return true;
    });
}

template <typename T, int M, int D>
__global__ void __launch_bounds__(128) k_tie_mark(QueryArgs<T> a) {
    const int w = blockIdx.x * 4 + (threadIdx.x >> 5);
    if (w >= *a.n_amb) return;
    scan_point<T, M, D>(a, a.amb[w], [&](int j) { a.relevant[a.parent[j]] = 1; });
}

static __global__ void k_tie_init(const uint8_t* core, const int* parent, const uint8_t* relevant, int* lm1, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) lm1[i] = (core[i] && relevant[parent[i]]) ? i : INT_MAX;
}

template <typename T, int M, int D>
__global__ void __launch_bounds__(128) k_tie_edge(QueryArgs<T> a) {
    const int item = blockIdx.x * 4 + (threadIdx.x >> 5);
    if (item >= a.n_items) return;
    const int2 it = a.items[item];
    const int r = it.x;
    const int pend = min(it.y + 32, a.ct.start[r + 1]);
    const int p = it.y + (int)lane_id();
    bool active = p < pend && a.core[p];
    if (active) active = a.relevant[a.parent[p]] != 0;
    if (!__any_sync(0xffffffffu, active)) return;
    const Tile<T> tile = warp_tile<T>(a.g.d);
    T q[D > 0 ? D : kMaxDims];
    load_query<T, D>(a, p, active, q);
    const int start_l = active ? ld_volatile(a.lm1 + p) : INT_MAX;
    int myl = start_l;
    auto aux_of = [&](int j) { return a.core[j] ? ld_volatile(a.lm1 + j) : INT_MAX; };
    auto pair = [&](int qi, int u, int lq) {
        if (!active || lq >= myl || qi >= p) return;
        if (within<T, M, D>(a, q, tile, u)) myl = lq;
    };
    auto never = []() { return false; };
    visit_stencil(a.g, a.ct, r, true, [&](int cr, bool own) {
        const int ce = own ? pend : a.ct.start[cr + 1];
        scan_range(a, tile, a.ct.start[cr], ce, aux_of, pair, never);
        return true;
    });
    if (active && myl < start_l) {
        atomicMin(a.lm1 + p, myl);
        *a.changed = 1;
    }
}

static __global__ void k_tie_jump(int* lm1, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int l = ld_volatile(lm1 + i);
    if (l == INT_MAX || l == i) return;
    const int l0 = l;
    for (;;) {  // strictly decreasing, so at most n steps
        const int ll = ld_volatile(lm1 + l);
        if (ll >= l) break;
        l = ll;
    }
    if (l < l0) atomicMin(lm1 + i, l);
}

template <typename T, int M, int D>
__global__ void __launch_bounds__(128) k_tie_resolve(QueryArgs<T> a) {
    const int w = blockIdx.x * 4 + (threadIdx.x >> 5);
    if (w >= *a.n_amb) return;
    const int b = a.amb[w];
    unsigned long long best = ~0ull;  // (L - 1) << 32 | root
    scan_point<T, M, D>(a, b, [&](int j) {
        const unsigned long long v = ((unsigned long long)(unsigned)a.lm1[j] << 32) | (unsigned)a.parent[j];
        if (v < best) best = v;
    });
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long y = __shfl_xor_sync(0xffffffffu, best, o);
        if (y < best) best = y;
    }
    if (lane_id() == 0) a.broot[b] = (int)(best & 0xffffffffu);
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
