// Dense cells: certified sub-cell cliques, their tables and boxes.
#pragma once

#include "hpd_query.cuh"
#include "hpd_union.cuh"

namespace hpd {

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
template <typename T, int DS>
__global__ void __launch_bounds__(128) k_mark_near_big(QueryArgs<T> a, DenseArgs da) {
    const int id = blockIdx.x * 4 + (threadIdx.x >> 5);
    if (id >= *da.n_dense) return;
    const int c = da.cells[id];
    if (a.ct.start[c + 1] - a.ct.start[c] < kPruneMinPoints) return;
    visit_stencil<DS>(a.g, a.ct, c, 0, [&](int cr, bool) {
        if (lane_id() == 0) a.cell_flags[cr] |= kCellNearBig;
        return true;
    });
}



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
                        if (D <= 0 && k >= d) break;
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
                            if (D <= 0 && k >= d) break;
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
                            if (D <= 0 && k >= d) break;
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

}  // namespace hpd
