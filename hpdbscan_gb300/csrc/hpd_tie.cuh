// Border tie-break: the single-threaded reference's choice among adjacent clusters.
#pragma once

#include "hpd_query.cuh"

namespace hpd {

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
        if (D <= 0 && k >= a.g.d) break;
        q[k] = a.coords[(size_t)k * a.n + p];
    }
    // the cell of p: binary search on cell starts
    int lo = 0, hi = a.ct.m;
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (a.ct.start[mid] <= p) lo = mid; else hi = mid;
    }
    visit_stencil<D>(a.g, a.ct, lo, 0, [&](int cr, bool) {
        const int ce = a.ct.start[cr + 1];
        for (int j = a.ct.start[cr] + (int)lane; j < ce; j += 32) {
            if (!a.core[j]) continue;
            T c[D > 0 ? D : kMaxDims];
#pragma unroll
            for (int k = 0; k < (D > 0 ? D : kMaxDims); ++k) {
                if (D <= 0 && k >= a.g.d) break;
                c[k] = a.coords[(size_t)k * a.n + j];
            }
            bool in;
            if constexpr (!Elem<T>::kFloat) {
                in = int_within<T, D>(q, c, a.g.d, a.eps2);
            } else {
                T t[D > 0 ? D : kMaxDims];
#pragma unroll
                for (int k = 0; k < (D > 0 ? D : kMaxDims); ++k) {
                    if (D <= 0 && k >= a.g.d) break;
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

constexpr int kInlineTiles = 4;  // tiles a work item scans of one range before handing the rest off
constexpr int kChunkTiles = 16;  // tiles per chunk task (one check of their minima)

// Scans the tiles of [c0, c1) (a range of cell cr, tiles aligned with its 32-point
// work items) whose item minimum is below `worst`, 32 tiles per check of the minima:
// scan(t0, t1) per surviving tile, in order.  Stops after `budget` scanned tiles and
// returns the first position not examined (c1 when done), or -1 when scan says stop.
template <typename T, class Scan>
__device__ __forceinline__ int scan_live_tiles(const QueryArgs<T>& a, int cr, int c0, int c1, int worst, int budget,
                                               Scan&& scan) {
    const int cs = a.ct.start[cr];
    const int first = (int)a.ipos[cs];
    int scanned = 0;
    for (int base = c0; base < c1; base += 32 * 32) {
        const int t = base + 32 * (int)lane_id();
        bool live = false;
        if (t < c1) {
            const int ti = first + ((t - cs) >> 5);
            live = in_range(a.guard, ti, a.n_items, kGuardItemIndex) && ld_volatile(a.item_min_l + ti) < worst;
        }
        unsigned mask = __ballot_sync(0xffffffffu, live);
        while (mask) {
            const int u = __ffs(mask) - 1;
            mask &= mask - 1;
            const int t0 = base + 32 * u;
            if (scanned == budget) return t0;
            ++scanned;
            if (scan(t0, min(t0 + 32, c1))) return -1;
        }
    }
    return c1;
}

// Hands [t0, ce) of cell cr, scanned for `item`, to chunk tasks of kChunkTiles tiles
// (warp-uniform; false when the queue is full, and the caller scans on itself).
template <typename T>
__device__ __forceinline__ bool push_chunks(const QueryArgs<T>& a, int item, int cr, int t0, int ce) {
    const int span = 32 * kChunkTiles;
    const int nt = (ce - t0 + span - 1) / span;
    int k = 0;
    if (lane_id() == 0) k = atomicAdd(a.n_chunks, nt);
    k = __shfl_sync(0xffffffffu, k, 0);
    if (k + nt > a.chunk_cap) {
        // the queue is full: the slots of [k, k + nt) below the cap become no-op tasks,
        // so that the chunk kernel reads no unwritten slot, and the caller scans on
        for (int i = (int)lane_id(); i < nt && k + i < a.chunk_cap; i += 32) a.chunks[k + i] = make_int4(-1, 0, 0, 0);
        return false;
    }
    for (int i = (int)lane_id(); i < nt; i += 32)
        a.chunks[k + i] = make_int4(item, cr, t0 + i * span, min(t0 + (i + 1) * span, ce));
    return true;
}

// One relaxation pass over decreasing core edges for one work item.  Only
// candidates in cells dirtied since the previous pass are rescanned: for every
// other candidate q the query already holds L(p) <= L(q) from an earlier pass.
// Lower cells are scanned first and the result is published at once; the own
// chunk is then closed in registers (each lane offers its value to the higher
// lanes within eps, in position order), so that chains of improvements inside one
// chunk settle within this pass.
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
    // Long scans (cells of hundreds of points) would keep one warp busy while the rest
    // of the grid idles: after kInlineTiles tiles the rest of the range is handed to
    // chunk tasks (k_tie_edge_chunks), whose results are published by atomicMin like
    // this item's own.
    auto scan_pruned = [&](int cr, int cs, int ce, int worst) {
        auto scan = [&](int t0, int t1) {
            if (a.trace_counts && lane_id() == 0) atomicAdd(a.trace_counts + 1, 1ull);
            return scan_range(a, tile, t0, t1, aux_of, pair, settled);
        };
        int rest = scan_live_tiles(a, cr, cs, ce, worst, a.chunks ? kInlineTiles : INT_MAX, scan);
        while (rest >= 0 && rest < ce) {
            if (push_chunks(a, item, cr, rest, ce)) return false;
            rest = scan_live_tiles(a, cr, rest, ce, worst, INT_MAX, scan);  // queue full: on our own
        }
        return rest < 0;
    };
    const bool own_dirty = ld_volatile(a.dirty_gen + r) >= since;
    int worst0 = active ? myl : INT_MIN;  // largest lane value at the start: a cell must beat it
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) worst0 = max(worst0, __shfl_xor_sync(0xffffffffu, worst0, o));
    visit_stencil<D>(a.g, a.ct, r, 1, [&](int cr, bool own) {
        if (own) {
            // own cell: the lower chunks once, then the warp's own chunk: every lane
            // offers its value to the higher lanes of the chunk within eps; taking the
            // lanes in position order closes the chunk in one pass, in registers
            const bool improved = publish();
            if (!own_dirty && !__any_sync(0xffffffffu, improved)) return true;
            if (!settled()) {
                int worst = (active && myl >= tl) ? myl : INT_MIN;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) worst = max(worst, __shfl_xor_sync(0xffffffffu, worst, o));
                scan_pruned(r, a.ct.start[r], it.y, worst);
            }
            if (!settled()) {
                unsigned lower = 0;  // cores of the chunk below this lane within eps
                auto aux_core = [&](int j) { return (int)a.core[j]; };
                auto mark = [&](int qi, int u, int is_core) {
                    if (active && is_core && qi < p && within<T, M, D>(a, q, tile, u)) lower |= 1u << u;
                };
                scan_range(a, tile, it.y, pend, aux_core, mark, never);
                int offer = (p < pend && a.core[p]) ? (active ? myl : ld_volatile(a.lm1 + p)) : INT_MAX;
                const int cnt = pend - it.y;
                for (int j = 0; j < cnt; ++j) {
                    const int vj = __shfl_sync(0xffffffffu, offer, j);
                    if (((lower >> j) & 1u) && vj < myl) myl = vj;
                    if (active) offer = myl;
                }
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

// One chunk task: the lanes of a work item against the tiles [t0, t1) of cell cr, as
// in tie_edge_item; improvements are published by atomicMin and dirty the item's cell.
template <typename T, int M, int D>
__device__ __forceinline__ void tie_edge_chunk(const QueryArgs<T>& a, int4 task) {
    const int item = task.x, cr = task.y;
    if (item < 0) return;  // no-op slot of a push that found the queue full
    if (!in_range(a.guard, item, a.n_items, kGuardItem) || !in_range(a.guard, cr, a.ct.m, kGuardCellRank)) return;
    const int2 it = a.items[item];
    const int r = it.x;
    if (!in_range(a.guard, r, a.ct.m, kGuardCellRank) || !in_range(a.guard, it.y, a.n, kGuardItem)) return;
    const int pend = min(it.y + 32, a.ct.start[r + 1]);
    const int p = it.y + (int)lane_id();
    bool active = p < pend && a.core[p];
    const int root = active ? a.parent[p] : INT_MIN;
    if (active && !in_range(a.guard, root, a.n, kGuardRoot)) active = false;
    int tl = INT_MIN;
    if (active) {
        tl = a.tlow[root];
        active = p <= a.tmax[root] && ld_volatile(a.lm1 + p) >= tl;
    }
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
    auto settled = [&]() { return __all_sync(0xffffffffu, !active || myl < tl); };
    int worst = (active && myl >= tl) ? myl : INT_MIN;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) worst = max(worst, __shfl_xor_sync(0xffffffffu, worst, o));
    scan_live_tiles(a, cr, task.z, task.w, worst, INT_MAX,
                    [&](int t0, int t1) { return scan_range(a, tile, t0, t1, aux_of, pair, settled); });
    const bool better = active && myl < start_l;
    if (better) {
        atomicMin(a.lm1 + p, myl);
        atomicMin(a.cell_min_l + r, myl);
        atomicMin(a.item_min_l + item, myl);
    }
    if (__any_sync(0xffffffffu, better) && lane_id() == 0) mark_dirty_cell(a, r);
}

// The chunk tasks of a pass, by a fixed grid of warps taking the next task by ticket.
template <typename T, int M, int D>
__global__ void __launch_bounds__(128) k_tie_edge_chunks(QueryArgs<T> a) {
    int cnt = *a.n_chunks;  // may exceed chunk_cap after a full queue: slots stop there
    if (cnt > a.chunk_cap) cnt = a.chunk_cap;
    if (cnt < 0) cnt = 0;
    for (;;) {
        int wi = 0;
        if (lane_id() == 0) wi = atomicAdd(a.ticket, 1);
        wi = __shfl_sync(0xffffffffu, wi, 0);
        if (wi >= cnt) return;
        tie_edge_chunk<T, M, D>(a, a.chunks[wi]);
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
// dirtied in this pass are appended to the next work list (warp per dirty cell).
template <typename T, int M, int D>
__global__ void __launch_bounds__(128) k_tie_schedule(QueryArgs<T> a) {
    const int nw = gridDim.x * 4;
    int cnt = *a.n_dlist;
    if (!in_range(a.guard, cnt, (long long)a.ct.m + 1, kGuardCount)) cnt = 0;
    const unsigned lane = lane_id();
    for (int w = blockIdx.x * 4 + (threadIdx.x >> 5); w < cnt; w += nw) {
        const int c = a.dlist[w];
        if (!in_range(a.guard, c, a.ct.m, kGuardDirtyCell)) continue;
        // a cell is relevant when it holds a core of a component below its highest core
        // next to an undecided border; the first warp to claim it in this pass lists it
        auto claim = [&](int cr) {
            const int rep_c = a.cell_rep[cr];
            if (rep_c == kNoCore) return false;
            if ((a.cell_flags[cr] & kCellUniform) && tmax_of(a, rep_c) < a.ct.start[cr]) return false;
            return atomicMax(a.sched_gen + cr, a.gen) < a.gen;
        };
        visit_stencil<D>(a.g, a.ct, c, 2, [&](int cr, bool own) {
            if (own) {  // the stencil filter (claim, one neighbour per lane) skips the own cell
                int fresh = 0;
                if (lane == 0) fresh = claim(cr);
                if (!__shfl_sync(0xffffffffu, fresh, 0)) return true;
            }
            const int s0 = a.ct.start[cr];
            const int nit = (a.ct.start[cr + 1] - s0 + 31) >> 5;
            const int first = (int)a.ipos[s0];
            // append each item once per pass (the stamp gen + 2 marks it listed); the order
            // of the list does not matter for the relaxation
            const unsigned stamp = (unsigned)a.gen + 2u;
            for (int k0 = 0; k0 < nit; k0 += 32) {
                const int k = k0 + (int)lane;
                const bool add = k < nit && in_range(a.guard, first + k, a.n_items, kGuardItemIndex) &&
                                 atomicExch(a.item_flag + first + k, stamp) != stamp;
                const unsigned m = __ballot_sync(0xffffffffu, add);
                int base = 0;
                if (lane == 0 && m) base = atomicAdd(a.n_wlist_out, __popc(m));
                base = __shfl_sync(0xffffffffu, base, 0);
                if (add) {
                    const int slot = base + __popc(m & ((1u << lane) - 1u));
                    if (in_range(a.guard, slot, a.n_items, kGuardList)) a.wlist_out[slot] = first + k;
                }
            }
            return true;
        }, false, claim);
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
__device__ __forceinline__ void tie_greedy_item(const QueryArgs<T>& a, int item) {
    if (!in_range(a.guard, item, a.n_items, kGuardItem)) return;
    const int2 it = a.items[item];
    const int r = it.x;
    const int pend = min(it.y + 32, a.ct.start[r + 1]);
    const int p = it.y + (int)lane_id();
    bool active = p < pend && a.core[p];
    if (active) {
        // positions below the component's threshold are settled already (value p)
        const int root = a.parent[p];
        active = in_range(a.guard, root, a.n, kGuardRoot) && p <= a.tmax[root] && p >= a.tlow[root];
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
    // the descent is a bound, not a result: a warp stops after a.greedy_tiles tiles, and a
    // lane without a hit by then keeps its own position (values only need to be reachable)
    int tiles = 0;
    auto done = [&]() { return ++tiles >= a.greedy_tiles || __all_sync(0xffffffffu, found); };
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
        visit_stencil<D>(a.g, a.ct, r, 1, [&](int cr, bool own) {
            if (own || cr == face || a.cell_rep[cr] == kNoCore) return true;
            return !scan_range(a, tile, a.ct.start[cr], a.ct.start[cr + 1], aux_of, pair, done);
        });
    }
    if (active) a.lm1[p] = g;
}

// Greedy descent over the listed work items, by a fixed grid of warps taking the next
// list entry from a shared ticket.
template <typename T, int M, int D>
__global__ void __launch_bounds__(128) k_tie_greedy(QueryArgs<T> a) {
    int cnt = *a.n_wlist;
    if (!in_range(a.guard, cnt, (long long)a.n_items + 1, kGuardCount)) cnt = 0;
    for (;;) {
        int wi = 0;
        if (lane_id() == 0) wi = atomicAdd(a.ticket, 1);
        wi = __shfl_sync(0xffffffffu, wi, 0);
        if (wi >= cnt) return;
        tie_greedy_item<T, M, D>(a, a.wlist[wi]);
    }
}

// Flags the work items holding a core of a component next to an undecided border,
// at or below the component's highest such core (tmax), that is not settled yet:
// its position (by_value 0, before the descent) or its value (by_value 1) is at
// least the component's threshold.  k_tie_compact lists the flagged items in order.
template <typename T>
__global__ void k_tie_list_flags(QueryArgs<T> a, int by_value) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.n || !a.core[p]) return;
    const int root = a.parent[p];
    if (!in_range(a.guard, root, a.n, kGuardRoot) || p > a.tmax[root]) return;
    if ((by_value ? ld_volatile(a.lm1 + p) : p) < a.tlow[root]) return;
    const int c = (int)a.cellrank[p];
    if (!in_range(a.guard, c, a.ct.m, kGuardCellRank)) return;
    const int s0 = a.ct.start[c];
    const int ti = (int)a.ipos[s0] + ((p - s0) >> 5);
    if (in_range(a.guard, ti, a.n_items, kGuardItemIndex)) a.item_flag[ti] = 1u;
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
        if (best == ~0ull) {
            // an ambiguous border has core neighbours of two components by construction
            in_range(a.guard, -1, a.n, kGuardAmbiguous);
        } else if (final_pass || ub < other) {
            a.broot[b] = root_best;
        } else {
            const int k = atomicAdd(a.n_amb_out, 1);
            if (in_range(a.guard, k, a.n, kGuardList)) a.amb_out[k] = b;
        }
    }
}

}  // namespace hpd
