/*
 * CPU restatement of the HPDBSCAN single-node clustering path (the oracle).
 *
 * TEST INFRASTRUCTURE ONLY.  The parity tests, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py call it as the checker; the product never links it.
 *
 * It restates, in plain C, the algorithm of upstream include/spatial_index.h and
 * include/hpdbscan.h (line references beside each step in hpd_oracle.c):
 * grid index with cell side eps, stable sort by cell, per-point region query over
 * the 3^d neighbour cells, core test, label propagation with equivalence rules,
 * rule resolution and un-permutation back to input order.
 *
 * threads == 1 gives the deterministic single-thread semantics that the GPU path
 * reproduces bit for bit; threads > 1 runs the same loop the way the reference
 * parallelises it (OpenMP, dynamic chunks of 32 points, CAS-min labels), whose
 * border labels may vary from run to run exactly like the reference's own.
 */
#ifndef HPD_ORACLE_H
#define HPD_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* element types, same codes as the product's C ABI */
enum {
    HPDO_F32 = 0, HPDO_F64 = 1,
    HPDO_I8 = 2, HPDO_I16 = 3, HPDO_I32 = 4, HPDO_I64 = 5,
    HPDO_U8 = 6, HPDO_U16 = 7, HPDO_U32 = 8, HPDO_U64 = 9
};

/* How (x - min) / eps is evaluated for cell coordinates and cell counts. */
enum {
    HPDO_CELL_RECIP = 0, /* (x - min) * (1 / eps): what GCC -Ofast emits (reciprocal math) */
    HPDO_CELL_DIV = 1    /* (x - min) / eps: strict IEEE division (-O2) */
};

/* Summation order of the squared distance sum_k (p_k - q_k)^2. */
enum {
    HPDO_DIST_GCC_X86 = 0, /* GCC -Ofast on x86-64/SSE2: lane-strided partial sums, unfused */
    HPDO_DIST_SEQ = 1,     /* strictly sequential, every product and sum rounded */
    HPDO_DIST_SEQ_FMA = 2, /* strictly sequential, off = fma(t, t, off) */
    HPDO_DIST_GCC_AARCH64 = 3 /* GCC -Ofast on aarch64/NEON: fused lane sums, pairwise fold,
                               * fused tail; saturating float -> integer conversions */
};

int hpd_oracle_cluster(const void* data, int64_t n, int32_t d, int32_t dtype, float eps,
                       uint64_t min_points, int32_t threads, int32_t cell_mode, int32_t dist_mode,
                       int64_t* labels, int64_t* sorted_order, uint64_t* sorted_cells);

const char* hpd_oracle_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
