// Core-core connectivity: union-find over the cores' eps graph.
#pragma once

#include "hpd_query.cuh"

namespace hpd {

// ---------------------------------------------------- core-core connectivity
// Every core-core eps edge (q < p) is united.  Pass 1 unites the pairs inside each
// cell; then every cell gets a summary (the smallest component root among its
// cores, and whether all its cores share it); pass 2 unites pairs across cells
// and skips, without loading a single coordinate, a neighbour cell that holds no
// core or whose cores are already in the query cell's component.  Within a tile,
// candidates already in the query's component are skipped without a distance test.

constexpr int kSmallCell = 128;  // cells up to this size are united in shared memory (k_union_small_cells)

// Pairs inside one cell of at most kSmallCell points, one warp per cell: a union-find
// over the cell's points in shared memory (roots are the smallest local index), then
// every core's global parent is set to its local root, a core of the same component
// at a lower position.  No global atomics.
template <typename T, int M, int D>
__global__ void __launch_bounds__(128) k_union_small_cells(QueryArgs<T> a) {
    __shared__ int s_lp[4][kSmallCell];
    const int w = threadIdx.x >> 5;
    const int c = blockIdx.x * 4 + w;
    if (c >= a.ct.m) return;
    const int cs = a.ct.start[c];
    const int size = a.ct.start[c + 1] - cs;
    if (size < 2 || size > kSmallCell) return;
    if (a.dense_id && a.dense_id[c] >= 0) return;  // connected by the dense-cell kernels
    const unsigned lane = lane_id();
    volatile int* lp = s_lp[w];
    for (int k = (int)lane; k < size; k += 32) lp[k] = k;
    __syncwarp();
    auto find = [&](int x) {
        for (;;) {
            const int px = lp[x];
            if (px == x) return x;
            const int gx = lp[px];
            if (gx != px) lp[x] = gx;  // path halving
            x = px;
        }
    };
    auto unite = [&](int x, int y) {
        for (;;) {
            x = find(x);
            y = find(y);
            if (x == y) return;
            if (x < y) { const int t = x; x = y; y = t; }
            if (atomicCAS((int*)&lp[x], x, y) == x) return;
        }
    };
    const Tile<T> tile = warp_tile<T>(a.g.d);
    for (int i0 = 0; i0 < size; i0 += 32) {
        const int li = i0 + (int)lane;
        const int p = cs + li;
        const bool active = li < size && a.core[p];
        T q[D > 0 ? D : kMaxDims];
        load_query<T, D>(a, p, active, q);
        auto aux_of = [&](int j) { return (int)a.core[j]; };
        auto pair = [&](int qi, int u, int is_core) {
            if (active && is_core && qi < p && within<T, M, D>(a, q, tile, u)) unite(li, qi - cs);
        };
        auto never = []() { return false; };
        scan_range(a, tile, cs, min(cs + i0 + 32, cs + size), aux_of, pair, never);
    }
    __syncwarp();
    for (int k = (int)lane; k < size; k += 32)
        if (a.core[cs + k]) a.parent[cs + k] = cs + find(k);
}

// Pairs inside the cells larger than kSmallCell that the dense-cell kernels do not
// connect, one warp per work item.
template <typename T, int M, int D>
__global__ void __launch_bounds__(128) k_union_intra(QueryArgs<T> a) {
    const int item = blockIdx.x * 4 + (threadIdx.x >> 5);
    if (item >= a.n_items) return;
    const int2 it = a.items[item];
    const int r = it.x;
    if (a.dense_id && a.dense_id[r] >= 0) return;  // connected by the dense-cell kernels
    if (a.ct.start[r + 1] - a.ct.start[r] <= kSmallCell) return;  // k_union_small_cells
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
    visit_stencil<D>(a.g, a.ct, r, 1, [&](int cr, bool own) {
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
    visit_stencil<D>(a.g, a.ct, c, 1, [&](int cr, bool own) {
        if (own) return true;
        const int rep_n = a.cell_rep[cr];
        if (same_component(a.parent, rep_c, rep_n)) return true;  // joined since the filter ran
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
                        if (D <= 0 && k >= d) break;
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
    }, false, [&](int cr) {
        // one neighbour per lane: single-component neighbours not yet in this component
        const int rep_n = a.cell_rep[cr];
        return rep_n != kNoCore && (a.cell_flags[cr] & kCellUniform) && uf_find(a.parent, rep_c) != uf_find(a.parent, rep_n);
    });
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

}  // namespace hpd
