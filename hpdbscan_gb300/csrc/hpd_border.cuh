// Border assignment and the final labels.
#pragma once

#include "hpd_query.cuh"

namespace hpd {

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
    visit_stencil<D>(a.g, a.ct, r, 0, [&](int cr, bool) {
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
        if (multi) {
            const int k = atomicAdd(a.n_amb, 1);
            if (in_range(a.guard, k, a.n, kGuardList)) a.amb[k] = p;
        }
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
