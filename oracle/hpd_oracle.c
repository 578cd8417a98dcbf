/*
 * CPU restatement of the HPDBSCAN single-node clustering path (the oracle).
 * TEST INFRASTRUCTURE ONLY -- see hpd_oracle.h.  Compiled with -ffp-contract=off
 * so that each arithmetic step below is rounded exactly as written.
 *
 * Upstream references (paths within the HPDBSCAN project):
 *   min / max per dimension        include/spatial_index.h:99-122, init :531-532
 *   cells per dimension            include/spatial_index.h:124-131
 *   dimension order                include/spatial_index.h:133-142
 *   cell id per point              include/spatial_index.h:144-165
 *   cell index + stable sort       include/spatial_index.h:167-216
 *   neighbour cells                include/spatial_index.h:682-737
 *   region query                   include/spatial_index.h:739-768
 *   label propagation              include/hpdbscan.h:51-101, include/atomic.h:20-36
 *   equivalence rules              include/rules.h:54-71, include/hpdbscan.h:198-211
 *   un-permute                     include/spatial_index.h:852-872
 *   label constants                include/constants.h:36-37
 */
#include "hpd_oracle.h"

#include <float.h>
#include <math.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define NOT_VISITED INT64_MAX
#define NOISE (INT64_MAX - 1)
#define MAX_DIMS 16

static _Thread_local char g_err[256];
const char* hpd_oracle_last_error(void) { return g_err; }
static int fail(int code, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
    return code;
}

/* ---------------------------------------------------------------- helpers */

/* stable LSD radix sort of (key, value) pairs, 8-bit digits, `bytes` key bytes */
static void radix_sort_pairs(uint64_t* key, int64_t* val, int64_t n, int bytes) {
    uint64_t* k2 = (uint64_t*)malloc((size_t)(n > 0 ? n : 1) * sizeof(uint64_t));
    int64_t* v2 = (int64_t*)malloc((size_t)(n > 0 ? n : 1) * sizeof(int64_t));
    for (int b = 0; b < bytes; ++b) {
        int64_t cnt[257] = {0};
        const int sh = 8 * b;
        for (int64_t i = 0; i < n; ++i) cnt[((key[i] >> sh) & 255u) + 1]++;
        for (int j = 0; j < 256; ++j) cnt[j + 1] += cnt[j];
        for (int64_t i = 0; i < n; ++i) {
            int64_t dst = cnt[(key[i] >> sh) & 255u]++;
            k2[dst] = key[i];
            v2[dst] = val[i];
        }
        memcpy(key, k2, (size_t)n * sizeof(uint64_t));
        memcpy(val, v2, (size_t)n * sizeof(int64_t));
    }
    free(k2);
    free(v2);
}

/* first index with keys[i] == k, or -1 (keys sorted ascending, unique) */
static int64_t find_cell(const uint64_t* keys, int64_t m, uint64_t k) {
    int64_t lo = 0, hi = m;
    while (lo < hi) {
        int64_t mid = lo + (hi - lo) / 2;
        if (keys[mid] < k) lo = mid + 1; else hi = mid;
    }
    return (lo < m && keys[lo] == k) ? lo : -1;
}

/* Lock-free union by minimum over cluster labels.  The upstream Rules map
 * (rules.h:54-71) keeps every label pointing at a smaller one and resolves a
 * label by following the chain (hpdbscan.h:198-211); the chain of any label ends
 * at the smallest label of its equivalence class.  This structure maintains the
 * same classes and returns the same smallest member. */
static int64_t uf_find(int64_t* parent, int64_t x) {
    for (;;) {
        int64_t p = __atomic_load_n(&parent[x], __ATOMIC_RELAXED);
        if (p == x) return x;
        int64_t gp = __atomic_load_n(&parent[p], __ATOMIC_RELAXED);
        if (gp != p) __atomic_compare_exchange_n(&parent[x], &p, gp, 0, __ATOMIC_RELAXED, __ATOMIC_RELAXED);
        x = gp;
    }
}
static void uf_union(int64_t* parent, int64_t a, int64_t b) {
    for (;;) {
        a = uf_find(parent, a);
        b = uf_find(parent, b);
        if (a == b) return;
        if (a < b) { int64_t t = a; a = b; b = t; }
        int64_t expect = a;
        if (__atomic_compare_exchange_n(&parent[a], &expect, b, 0, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) return;
    }
}

/* atomic_min on int64 labels (atomic.h:20-36) */
static void label_min(int64_t* addr, int64_t v) {
    int64_t cur = __atomic_load_n(addr, __ATOMIC_RELAXED);
    while (v < cur) {
        if (__atomic_compare_exchange_n(addr, &cur, v, 0, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) return;
    }
}

/* -------------------------------------------------- squared distance, floats */

static float dist2_f32(const float* p, const float* q, int d, int mode) {
    if (mode == HPDO_DIST_GCC_AARCH64) {
        /* GCC -Ofast, aarch64 NEON: below 4 dimensions a fused running sum; else 4
         * lanes accumulate dimensions k = j (mod 4) with fused multiply-adds over the
         * first d & ~3 dimensions, are folded pairwise as (l0 + l1) + (l2 + l3), and
         * the remaining dimensions are added with fused multiply-adds. */
        int nv = d >= 4 ? (d & ~3) : 0, j = 0;
        float s = 0.0f;
        if (nv) {
            float l[4] = {0.0f, 0.0f, 0.0f, 0.0f};
            for (; j < nv; j += 4)
                for (int k = 0; k < 4; ++k) { float t = p[j + k] - q[j + k]; l[k] = fmaf(t, t, l[k]); }
            s = (l[0] + l[1]) + (l[2] + l[3]);
        }
        for (; j < d; ++j) { float t = p[j] - q[j]; s = fmaf(t, t, s); }
        return s;
    }
    if (mode == HPDO_DIST_SEQ) {
        float off = 0.0f;
        for (int k = 0; k < d; ++k) { float t = p[k] - q[k]; float s = t * t; off = off + s; }
        return off;
    }
    if (mode == HPDO_DIST_SEQ_FMA) {
        float off = 0.0f;
        for (int k = 0; k < d; ++k) { float t = p[k] - q[k]; off = fmaf(t, t, off); }
        return off;
    }
    /* GCC -Ofast, x86-64 SSE2: 4 lanes accumulate dimensions k = j (mod 4) over the
     * first d & ~3 dimensions, lanes are folded as (l0 + l2) + (l1 + l3); a 2-wide
     * step then adds the next two squares to the folded pair and sums the pair; an
     * odd last dimension is added on its own.  For d <= 3 this is the sequential sum. */
    int nv = d >= 4 ? (d & ~3) : 0, j = 0;
    float l0 = 0.0f, l1 = 0.0f, l2 = 0.0f, l3 = 0.0f;
    for (; j < nv; j += 4) {
        float t0 = p[j] - q[j], t1 = p[j + 1] - q[j + 1], t2 = p[j + 2] - q[j + 2], t3 = p[j + 3] - q[j + 3];
        float s0 = t0 * t0, s1 = t1 * t1, s2 = t2 * t2, s3 = t3 * t3;
        l0 = l0 + s0; l1 = l1 + s1; l2 = l2 + s2; l3 = l3 + s3;
    }
    float e0 = l0 + l2, e1 = l1 + l3;
    float s = nv ? e1 + e0 : 0.0f;
    int rem = d - nv;
    if (rem == 0) return s;
    if (rem >= 2) {
        float t0 = p[j] - q[j], t1 = p[j + 1] - q[j + 1];
        float s0 = t0 * t0, s1 = t1 * t1;
        if (!nv) { e0 = 0.0f; e1 = 0.0f; }
        e0 = e0 + s0; e1 = e1 + s1;
        s = e1 + e0;
        j += 2;
        if (!(rem & 1)) return s;
    }
    float t = p[j] - q[j];
    float sq = t * t;
    return s + sq;
}

static double dist2_f64(const double* p, const double* q, int d, int mode) {
    if (mode == HPDO_DIST_GCC_AARCH64) {
        /* GCC -Ofast, aarch64 NEON: from 2 dimensions on, 2 lanes accumulate even / odd
         * dimensions with fused multiply-adds, summed l0 + l1; an odd last dimension is
         * added with a fused multiply-add. */
        int nv = d >= 2 ? (d & ~1) : 0, j = 0;
        double s = 0.0;
        if (nv) {
            double l0 = 0.0, l1 = 0.0;
            for (; j < nv; j += 2) {
                double t0 = p[j] - q[j], t1 = p[j + 1] - q[j + 1];
                l0 = fma(t0, t0, l0);
                l1 = fma(t1, t1, l1);
            }
            s = l0 + l1;
        }
        for (; j < d; ++j) { double t = p[j] - q[j]; s = fma(t, t, s); }
        return s;
    }
    if (mode == HPDO_DIST_SEQ) {
        double off = 0.0;
        for (int k = 0; k < d; ++k) { double t = p[k] - q[k]; double s = t * t; off = off + s; }
        return off;
    }
    if (mode == HPDO_DIST_SEQ_FMA) {
        double off = 0.0;
        for (int k = 0; k < d; ++k) { double t = p[k] - q[k]; off = fma(t, t, off); }
        return off;
    }
    /* GCC -Ofast, x86-64 SSE2: 2 lanes accumulate even / odd dimensions over the
     * first d & ~1 dimensions, folded as l1 + l0; an odd last dimension is added. */
    if (d == 1) { double t = p[0] - q[0]; return t * t; }
    int nv = d & ~1, j = 0;
    double l0 = 0.0, l1 = 0.0;
    for (; j < nv; j += 2) {
        double t0 = p[j] - q[j], t1 = p[j + 1] - q[j + 1];
        double s0 = t0 * t0, s1 = t1 * t1;
        l0 = l0 + s0; l1 = l1 + s1;
    }
    double s = nv ? l1 + l0 : 0.0;
    if (d & 1) { double t = p[j] - q[j]; double sq = t * t; s = s + sq; }
    return s;
}

/* --------------------------------------------- per-type index construction */

/* Index built for one element type: everything downstream is type-independent
 * except the distance test, which goes through a callback. */
typedef struct {
    int64_t n;
    int d;
    uint64_t* cell;      /* [n] cell id in sorted order */
    int64_t* order;      /* [n] original index in sorted order */
    uint64_t* keys;      /* [m] unique cell ids ascending */
    int64_t* start;      /* [m + 1] first sorted position of each cell */
    int64_t m;
    uint64_t dims[MAX_DIMS];   /* cells per dimension */
    int swapped[MAX_DIMS];     /* dimension order, fewest cells first */
    void* sorted;              /* [n * d] points in sorted order */
} Index;

/* EPS2 = (T)(float)(eps * eps) (hpdbscan.h:53, then region_query's T parameter) as GCC
 * compiles the float -> integer conversion for the target.  x86-64: cvttss2si with a
 * 32-bit result for types below 32 bits and for int32, a 64-bit result for uint32 and
 * int64, and GCC's two-step sequence around 2^63 for uint64; a value out of range gives
 * the "integer indefinite" 0x80...0.  aarch64: fcvtzs / fcvtzu into a 32-bit register
 * for types up to 32 bits, a 64-bit one for the 64-bit types; both saturate. */
static int64_t cvt_x86_32(float f) {
    return (f > -2147483649.0f && f < 2147483648.0f) ? (int64_t)(int32_t)f : (int64_t)INT32_MIN;
}
static int64_t cvt_x86_64(float f) {
    return (f >= -9223372036854775808.0f && f < 9223372036854775808.0f) ? (int64_t)f : INT64_MIN;
}
static uint64_t cvt_x86_u64(float f) {
    if (f < 9223372036854775808.0f) return (uint64_t)cvt_x86_64(f);
    return (uint64_t)cvt_x86_64(f - 9223372036854775808.0f) ^ 0x8000000000000000ull;
}
static int64_t sat_s32(float f) {
    if (f != f) return 0;
    if (f >= 2147483648.0f) return INT32_MAX;
    if (f <= -2147483648.0f) return INT32_MIN;
    return (int64_t)(int32_t)f;
}
static uint64_t sat_u32(float f) {
    if (f != f || f <= -1.0f) return 0;
    if (f >= 4294967296.0f) return UINT32_MAX;
    return (uint64_t)(uint32_t)f;
}
static int64_t sat_s64(float f) {
    if (f != f) return 0;
    if (f >= 9223372036854775808.0f) return INT64_MAX;
    if (f <= -9223372036854775808.0f) return INT64_MIN;
    return (int64_t)f;
}
static uint64_t sat_u64(float f) {
    if (f != f || f <= -1.0f) return 0;
    if (f >= 18446744073709551616.0f) return UINT64_MAX;
    return (uint64_t)f;
}

typedef int (*within_fn)(const void* pts, int d, int64_t a, int64_t b, const void* eps2, int mode);

static int within_f32(const void* pts, int d, int64_t a, int64_t b, const void* eps2, int mode) {
    const float* P = (const float*)pts;
    return dist2_f32(P + a * d, P + b * d, d, mode) <= *(const float*)eps2;
}
static int within_f64(const void* pts, int d, int64_t a, int64_t b, const void* eps2, int mode) {
    const double* P = (const double*)pts;
    return dist2_f64(P + a * d, P + b * d, d, mode) <= *(const double*)eps2;
}

/* Integer element types: `T distance = p - q; offset += distance * distance`
 * (spatial_index.h:751-754) wraps modulo 2^bits(T) at every store into T, so the
 * sum equals the modulo-2^bits sum of the wrapped squares in any order. */
#define DEFINE_WITHIN_INT(T, SUF)                                                        \
    static int within_##SUF(const void* pts, int d, int64_t a, int64_t b, const void* eps2, int mode) { \
        (void)mode;                                                                      \
        const T* P = (const T*)pts;                                                      \
        const T* p = P + a * d;                                                          \
        const T* q = P + b * d;                                                          \
        uint64_t acc = 0;                                                                \
        for (int k = 0; k < d; ++k) {                                                    \
            T t = (T)((uint64_t)p[k] - (uint64_t)q[k]);                                  \
            acc += (uint64_t)(int64_t)t * (uint64_t)(int64_t)t;                           \
        }                                                                                \
        T off = (T)acc;                                                                  \
        return off <= *(const T*)eps2;                                                   \
    }
DEFINE_WITHIN_INT(int8_t, i8)
DEFINE_WITHIN_INT(int16_t, i16)
DEFINE_WITHIN_INT(int32_t, i32)
DEFINE_WITHIN_INT(int64_t, i64)
DEFINE_WITHIN_INT(uint8_t, u8)
DEFINE_WITHIN_INT(uint16_t, u16)
DEFINE_WITHIN_INT(uint32_t, u32)
DEFINE_WITHIN_INT(uint64_t, u64)

/* (x - min) as the upstream expression evaluates it, converted to the float type
 * F of the division: F is double for double points and float otherwise.  For
 * integer T the difference is taken in the promoted integer type (int for types
 * narrower than int, else T itself, wrapping) and then converted. */
#define DIFF_FLOAT(T, x, mn) (FLOATOF_##T)((PROMO_##T)(x) - (PROMO_##T)(mn))
#define FLOATOF_float float
#define FLOATOF_double double
#define FLOATOF_int8_t float
#define FLOATOF_int16_t float
#define FLOATOF_int32_t float
#define FLOATOF_int64_t float
#define FLOATOF_uint8_t float
#define FLOATOF_uint16_t float
#define FLOATOF_uint32_t float
#define FLOATOF_uint64_t float
#define PROMO_float float
#define PROMO_double double
#define PROMO_int8_t int32_t
#define PROMO_int16_t int32_t
#define PROMO_int32_t uint32_t /* int - int wraps like uint32 on the targets of interest */
#define PROMO_int64_t uint64_t
#define PROMO_uint8_t int32_t
#define PROMO_uint16_t int32_t
#define PROMO_uint32_t uint32_t
#define PROMO_uint64_t uint64_t
/* signed 32/64-bit differences are converted from their wrapped signed value */
#define SIGNED_FIX_int32_t(v) ((float)(int32_t)(v))
#define SIGNED_FIX_int64_t(v) ((float)(int64_t)(v))

#define DEFINE_INDEX(T, SUF, TMAX_INIT, TMAX_INIT_FOR_MAX, DIFFEXPR)                    \
    static int build_index_##SUF(const T* data, int64_t n, int d, float eps, int cell_mode, \
                                 int threads, Index* ix) {                               \
        typedef FLOATOF_##T F;                                                           \
        T mins[MAX_DIMS], maxs[MAX_DIMS];                                                \
        /* spatial_index.h:531-532: min starts at max(T), max at numeric_limits<T>::min() */ \
        for (int k = 0; k < d; ++k) { mins[k] = TMAX_INIT; maxs[k] = TMAX_INIT_FOR_MAX; } \
        for (int64_t i = 0; i < n; ++i) {                                                \
            for (int k = 0; k < d; ++k) {                                                \
                T c = data[i * d + k];                                                   \
                if (NONFINITE_##SUF(c)) return fail(1, "non-finite coordinate at point %lld", (long long)i); \
                if (c < mins[k]) mins[k] = c;      /* std::min(m, c) */                  \
                if (maxs[k] < c) maxs[k] = c;      /* std::max(m, c) */                  \
            }                                                                            \
        }                                                                                \
        const F recip = (F)1 / (F)eps;                                                   \
        uint64_t total = 1;                                                              \
        for (int k = 0; k < d; ++k) {                                                    \
            F diff = DIFFEXPR(T, maxs[k], mins[k]);                                      \
            F q = cell_mode == HPDO_CELL_RECIP ? diff * recip : diff / (F)eps;          \
            F c = ceil(q);                                                               \
            if (!(c >= 0) || c > (F)4.0e18) return fail(4, "cell grid too large or non-finite extent in dimension %d", k); \
            ix->dims[k] = (uint64_t)c + 1;                                               \
            if (ix->dims[k] != 0 && total > UINT64_MAX / ix->dims[k]) return fail(4, "cell grid overflows 64 bits"); \
            total *= ix->dims[k];                                                        \
        }                                                                                \
        /* spatial_index.h:133-142: stable order by ascending cell count (d <= 16) */   \
        for (int k = 0; k < d; ++k) ix->swapped[k] = k;                                  \
        for (int a = 1; a < d; ++a) {                                                    \
            int v = ix->swapped[a], b = a - 1;                                           \
            while (b >= 0 && ix->dims[v] < ix->dims[ix->swapped[b]]) { ix->swapped[b + 1] = ix->swapped[b]; --b; } \
            ix->swapped[b + 1] = v;                                                      \
        }                                                                                \
        uint64_t* cell = (uint64_t*)malloc((size_t)(n ? n : 1) * sizeof(uint64_t));     \
        int64_t* order = (int64_t*)malloc((size_t)(n ? n : 1) * sizeof(int64_t));       \
        _Pragma("omp parallel for num_threads(threads) schedule(static)")                \
        for (int64_t i = 0; i < n; ++i) {                                                \
            uint64_t id = 0, acc = 1;                                                    \
            for (int s = 0; s < d; ++s) {                                                \
                int k = ix->swapped[s];                                                  \
                F diff = DIFFEXPR(T, data[i * d + k], mins[k]);                          \
                F q = cell_mode == HPDO_CELL_RECIP ? diff * recip : diff / (F)eps;      \
                uint64_t idx = (uint64_t)floor(q);                                       \
                id += idx * acc;                                                         \
                acc *= ix->dims[k];                                                      \
            }                                                                            \
            cell[i] = id;                                                                \
            order[i] = i;                                                                \
        }                                                                                \
        int bytes = 0;                                                                   \
        while (bytes < 8 && (total - 1) >> (8 * bytes)) ++bytes;                         \
        radix_sort_pairs(cell, order, n, bytes);                                         \
        T* sorted = (T*)malloc((size_t)(n ? n : 1) * d * sizeof(T));                     \
        for (int64_t i = 0; i < n; ++i)                                                  \
            memcpy(sorted + i * d, data + order[i] * d, (size_t)d * sizeof(T));          \
        int64_t m = 0;                                                                   \
        for (int64_t i = 0; i < n; ++i) if (i == 0 || cell[i] != cell[i - 1]) ++m;       \
        ix->keys = (uint64_t*)malloc((size_t)(m ? m : 1) * sizeof(uint64_t));           \
        ix->start = (int64_t*)malloc((size_t)(m + 1) * sizeof(int64_t));                 \
        m = 0;                                                                           \
        for (int64_t i = 0; i < n; ++i)                                                  \
            if (i == 0 || cell[i] != cell[i - 1]) { ix->keys[m] = cell[i]; ix->start[m] = i; ++m; } \
        ix->start[m] = n;                                                                \
        ix->m = m; ix->n = n; ix->d = d;                                                 \
        ix->cell = cell; ix->order = order; ix->sorted = sorted;                         \
        return 0;                                                                        \
    }

#define NONFINITE_f32(c) (!isfinite(c))
#define NONFINITE_f64(c) (!isfinite(c))
#define NONFINITE_i8(c) 0
#define NONFINITE_i16(c) 0
#define NONFINITE_i32(c) 0
#define NONFINITE_i64(c) 0
#define NONFINITE_u8(c) 0
#define NONFINITE_u16(c) 0
#define NONFINITE_u32(c) 0
#define NONFINITE_u64(c) 0
#define DIFF_PLAIN(T, x, mn) DIFF_FLOAT(T, x, mn)
#define DIFF_S32(T, x, mn) SIGNED_FIX_int32_t((uint32_t)(x) - (uint32_t)(mn))
#define DIFF_S64(T, x, mn) SIGNED_FIX_int64_t((uint64_t)(x) - (uint64_t)(mn))

DEFINE_INDEX(float, f32, FLT_MAX, FLT_MIN, DIFF_PLAIN)
DEFINE_INDEX(double, f64, DBL_MAX, DBL_MIN, DIFF_PLAIN)
DEFINE_INDEX(int8_t, i8, INT8_MAX, INT8_MIN, DIFF_PLAIN)
DEFINE_INDEX(int16_t, i16, INT16_MAX, INT16_MIN, DIFF_PLAIN)
DEFINE_INDEX(int32_t, i32, INT32_MAX, INT32_MIN, DIFF_S32)
DEFINE_INDEX(int64_t, i64, INT64_MAX, INT64_MIN, DIFF_S64)
DEFINE_INDEX(uint8_t, u8, UINT8_MAX, 0, DIFF_PLAIN)
DEFINE_INDEX(uint16_t, u16, UINT16_MAX, 0, DIFF_PLAIN)
DEFINE_INDEX(uint32_t, u32, UINT32_MAX, 0, DIFF_PLAIN)
DEFINE_INDEX(uint64_t, u64, UINT64_MAX, 0, DIFF_PLAIN)

static void free_index(Index* ix) {
    free(ix->cell); free(ix->order); free(ix->keys); free(ix->start); free(ix->sorted);
}

/* Neighbour cell ranges of one cell: the 3^d block around it, clipped to the grid
 * (spatial_index.h:682-737).  Writes (start, count) of the non-empty ones and
 * returns the total number of candidate points. */
static int64_t neighbour_ranges(const Index* ix, int64_t cell_pos, int64_t* rs, int64_t* rc, int* nr) {
    const int d = ix->d;
    uint64_t key = ix->keys[cell_pos];
    uint64_t coord[MAX_DIMS], stride[MAX_DIMS];
    uint64_t acc = 1, rest = key;
    for (int s = 0; s < d; ++s) {
        uint64_t dim = ix->dims[ix->swapped[s]];
        stride[s] = acc;
        coord[s] = rest % dim;
        rest /= dim;
        acc *= dim;
    }
    int64_t total = 0;
    int count = 0;
    int off[MAX_DIMS];
    for (int s = 0; s < d; ++s) off[s] = -1;
    for (;;) {
        int ok = 1;
        uint64_t nk = key;
        for (int s = 0; s < d && ok; ++s) {
            uint64_t dim = ix->dims[ix->swapped[s]];
            if (off[s] < 0) { if (coord[s] == 0) ok = 0; else nk -= stride[s]; }
            else if (off[s] > 0) { if (coord[s] + 1 >= dim) ok = 0; else nk += stride[s]; }
        }
        if (ok) {
            int64_t pos = (nk == key) ? cell_pos : find_cell(ix->keys, ix->m, nk);
            if (pos >= 0) {
                rs[count] = ix->start[pos];
                rc[count] = ix->start[pos + 1] - ix->start[pos];
                total += rc[count];
                ++count;
            }
        }
        int s = 0;
        while (s < d && off[s] == 1) { off[s] = -1; ++s; }
        if (s == d) break;
        ++off[s];
    }
    *nr = count;
    return total;
}

/* ------------------------------------------------------------ the DBSCAN loop */

static int run_dbscan(const Index* ix, within_fn within, const void* eps2, int dist_mode,
                      uint64_t min_points, int threads, int64_t* clusters, int64_t* parent) {
    const int64_t n = ix->n;
    const int d = ix->d;
    int64_t max_ranges = 1;
    for (int s = 0; s < d; ++s) max_ranges *= 3;
    int err = 0;

    for (int64_t i = 0; i < n; ++i) clusters[i] = NOT_VISITED;
    for (int64_t i = 0; i <= n + 1; ++i) parent[i] = i;

#pragma omp parallel num_threads(threads)
    {
        int64_t* rs = (int64_t*)malloc((size_t)max_ranges * sizeof(int64_t));
        int64_t* rc = (int64_t*)malloc((size_t)max_ranges * sizeof(int64_t));
        int64_t cap = 1024, na = 0;
        int64_t* area = (int64_t*)malloc((size_t)cap * sizeof(int64_t));
        int64_t prev_cell = -1, candidates = 0;
        int nr = 0;
        if (!rs || !rc || !area) err = 1;

        /* hpdbscan.h:62: dynamic schedule, chunks of 32 points */
#pragma omp for schedule(dynamic, 32)
        for (int64_t p = 0; p < n; ++p) {
            if (err) continue;
            /* position of p's cell in the cell table */
            int64_t cpos = find_cell(ix->keys, ix->m, ix->cell[p]);
            if (cpos != prev_cell) {
                candidates = neighbour_ranges(ix, cpos, rs, rc, &nr);
                prev_cell = cpos;
            }
            na = 0;
            int64_t label = NOISE;
            if ((uint64_t)candidates >= min_points) {
                /* region query (spatial_index.h:739-768) */
                label = p + 1;
                for (int r = 0; r < nr; ++r) {
                    for (int64_t q = rs[r]; q < rs[r] + rc[r]; ++q) {
                        if (!within(ix->sorted, d, p, q, eps2, dist_mode)) continue;
                        int64_t lq = __atomic_load_n(&clusters[q], __ATOMIC_RELAXED);
                        if (na == cap) {
                            cap *= 2;
                            int64_t* grown = (int64_t*)realloc(area, (size_t)cap * sizeof(int64_t));
                            if (!grown) { err = 1; break; }
                            area = grown;
                        }
                        area[na++] = q;
                        if (lq != NOT_VISITED && lq < 0 && -lq < label) label = -lq;
                    }
                }
            }
            if ((uint64_t)na >= min_points) {
                /* core point: hpdbscan.h:78-93 */
                label_min(&clusters[p], -label);
                for (int64_t a = 0; a < na; ++a) {
                    int64_t o = area[a];
                    int64_t lo = __atomic_load_n(&clusters[o], __ATOMIC_RELAXED);
                    if (lo < 0) {
                        int64_t other = -lo;
                        if (other != label) uf_union(parent, other, label);
                    }
                    label_min(&clusters[o], label);
                }
            } else if (__atomic_load_n(&clusters[p], __ATOMIC_RELAXED) == NOT_VISITED) {
                label_min(&clusters[p], NOISE);
            }
        }
        free(rs);
        free(rc);
        free(area);
    }
    if (err) return fail(5, "out of host memory");

    /* apply_rules (hpdbscan.h:198-211): noise -> 0, every label -> its class minimum */
#pragma omp parallel for num_threads(threads) schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        int64_t c = clusters[i];
        int core = c < 0;
        int64_t v = core ? -c : c;
        if (v == NOISE) v = 0;
        else if (v != NOT_VISITED) v = uf_find(parent, v);
        clusters[i] = core ? -v : v;
    }
    return 0;
}

/* ------------------------------------------------------------------ entry */

int hpd_oracle_cluster(const void* data, int64_t n, int32_t d, int32_t dtype, float eps,
                       uint64_t min_points, int32_t threads, int32_t cell_mode, int32_t dist_mode,
                       int64_t* labels, int64_t* sorted_order, uint64_t* sorted_cells) {
    g_err[0] = 0;
    if (!(eps > 0.0f)) return fail(1, "epsilon needs to be positive");
    if (n < 0 || d < 1 || d > MAX_DIMS) return fail(1, "unsupported shape (n=%lld, d=%d)", (long long)n, d);
    if (threads < 1) threads = 1;
    if (n == 0) return 0;
    Index ix;
    memset(&ix, 0, sizeof ix);
    int rc = 0;
    const float eps2f = eps * eps; /* hpdbscan.h:53 */
    const int arm = dist_mode == HPDO_DIST_GCC_AARCH64;
    union { float f; double g; int8_t i8; int16_t i16; int32_t i32; int64_t i64;
            uint8_t u8; uint16_t u16; uint32_t u32; uint64_t u64; } e2;
    within_fn within = NULL;
    switch (dtype) {
        case HPDO_F32: rc = build_index_f32((const float*)data, n, d, eps, cell_mode, threads, &ix); e2.f = eps2f; within = within_f32; break;
        case HPDO_F64: rc = build_index_f64((const double*)data, n, d, eps, cell_mode, threads, &ix); e2.g = (double)eps2f; within = within_f64; break;
        case HPDO_I8:  rc = build_index_i8((const int8_t*)data, n, d, eps, cell_mode, threads, &ix); e2.i8 = (int8_t)(arm ? sat_s32(eps2f) : cvt_x86_32(eps2f)); within = within_i8; break;
        case HPDO_I16: rc = build_index_i16((const int16_t*)data, n, d, eps, cell_mode, threads, &ix); e2.i16 = (int16_t)(arm ? sat_s32(eps2f) : cvt_x86_32(eps2f)); within = within_i16; break;
        case HPDO_I32: rc = build_index_i32((const int32_t*)data, n, d, eps, cell_mode, threads, &ix); e2.i32 = (int32_t)(arm ? sat_s32(eps2f) : cvt_x86_32(eps2f)); within = within_i32; break;
        case HPDO_I64: rc = build_index_i64((const int64_t*)data, n, d, eps, cell_mode, threads, &ix); e2.i64 = arm ? sat_s64(eps2f) : cvt_x86_64(eps2f); within = within_i64; break;
        case HPDO_U8:  rc = build_index_u8((const uint8_t*)data, n, d, eps, cell_mode, threads, &ix); e2.u8 = (uint8_t)(arm ? (int64_t)sat_u32(eps2f) : cvt_x86_32(eps2f)); within = within_u8; break;
        case HPDO_U16: rc = build_index_u16((const uint16_t*)data, n, d, eps, cell_mode, threads, &ix); e2.u16 = (uint16_t)(arm ? (int64_t)sat_u32(eps2f) : cvt_x86_32(eps2f)); within = within_u16; break;
        case HPDO_U32: rc = build_index_u32((const uint32_t*)data, n, d, eps, cell_mode, threads, &ix); e2.u32 = (uint32_t)(arm ? (int64_t)sat_u32(eps2f) : cvt_x86_64(eps2f)); within = within_u32; break;
        case HPDO_U64: rc = build_index_u64((const uint64_t*)data, n, d, eps, cell_mode, threads, &ix); e2.u64 = arm ? sat_u64(eps2f) : cvt_x86_u64(eps2f); within = within_u64; break;
        default: return fail(2, "unsupported dtype %d", dtype);
    }
    if (rc) return rc;
    int64_t* clusters = (int64_t*)malloc((size_t)n * sizeof(int64_t));
    int64_t* parent = (int64_t*)malloc((size_t)(n + 2) * sizeof(int64_t));
    if (!clusters || !parent) { free(clusters); free(parent); free_index(&ix); return fail(5, "out of host memory"); }
    rc = run_dbscan(&ix, within, &e2, dist_mode, min_points, threads, clusters, parent);
    if (!rc) {
        /* recover_initial_order (spatial_index.h:852-872) */
        for (int64_t i = 0; i < n; ++i) labels[ix.order[i]] = clusters[i];
        if (sorted_order) memcpy(sorted_order, ix.order, (size_t)n * sizeof(int64_t));
        if (sorted_cells) memcpy(sorted_cells, ix.cell, (size_t)n * sizeof(uint64_t));
    }
    free(clusters);
    free(parent);
    free_index(&ix);
    return rc;
}
