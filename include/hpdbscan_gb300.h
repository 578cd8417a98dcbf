/*
 * hpdbscan_gb300 -- C ABI of the GB300 DBSCAN engine.
 *
 * A drop-in for the single-node clustering path of HPDBSCAN: same inputs
 * (an n x d row-major array of one of ten element types, epsilon, minPoints),
 * same output (one int64 label per point in input order: 0 noise, -k core point of
 * cluster k, +k border point of cluster k, k = 1 + the position of the cluster's
 * first core point in cell-sorted order) and the same errors.  Plain pointers and
 * sizes only; every entry point returns an hpd_status and leaves a message for
 * hpd_last_error() on failure.
 *
 * Upstream interfaces replaced (paths within the HPDBSCAN project):
 *   hpd_create / hpd_destroy    HPDBSCAN::HPDBSCAN(float epsilon, size_t min_points)
 *                               include/hpdbscan.h:288-298
 *   hpd_cluster                 HPDBSCAN::cluster<T>(T* data, int dim0, int dim1, int threads)
 *                               include/hpdbscan.h:475-486 (explicit instantiations
 *                               src/hpdbscan.cpp:19-30), Python cluster(ndarray)
 *                               swig/hpdbscan.i:27-34
 *   hpd_cluster_device          the same computation on buffers already in device memory
 *                               (no upstream counterpart; the host entry point uses it)
 *   hpd_h5_read / hpd_h5_write  IO::read_hdf5 / IO::write_hdf5 (include/io.h:35-197)
 *                               with the element-type dispatch of HPDBSCAN::cluster(path,
 *                               dataset, threads) (include/hpdbscan.h:300-356)
 *   hpd_last_error             the what() of the std::invalid_argument / runtime_error
 *                               the upstream class throws (hpdbscan.h:296,327,340,350,354)
 */
#ifndef HPDBSCAN_GB300_H
#define HPDBSCAN_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  HPD_ERR_INVALID corresponds to upstream std::invalid_argument,
 * HPD_ERR_RUNTIME to std::runtime_error; the others are engine conditions. */
typedef enum {
    HPD_OK = 0,
    HPD_ERR_INVALID = 1,     /* bad epsilon, shape, non-finite coordinate, missing file/dataset */
    HPD_ERR_UNSUPPORTED = 2, /* unsupported element type / precision / dimensionality */
    HPD_ERR_RUNTIME = 3,     /* read/write failure */
    HPD_ERR_GRID = 4,        /* cell grid does not fit 64-bit cell ids */
    HPD_ERR_NOMEM = 5,       /* device or host allocation failed */
    HPD_ERR_CUDA = 6,        /* CUDA runtime error */
    HPD_ERR_TIMEOUT = 7      /* a bounded device loop hit its iteration limit */
} hpd_status;

/* Element types: the ten upstream instantiations (src/hpdbscan.cpp:19-30). */
typedef enum {
    HPD_F32 = 0, HPD_F64 = 1,
    HPD_I8 = 2, HPD_I16 = 3, HPD_I32 = 4, HPD_I64 = 5,
    HPD_U8 = 6, HPD_U16 = 7, HPD_U32 = 8, HPD_U64 = 9
} hpd_dtype;

/* Arithmetic of the reference build being matched.  Upstream computes cell
 * coordinates as floor((x - min) / eps) (spatial_index.h:156) and squared distances
 * by a running sum (spatial_index.h:751-754); its CMake flags (-Ofast) let the
 * compiler turn the division into a multiply by 1/eps and reassociate the sum.
 * The defaults reproduce GCC -Ofast on x86-64: reciprocal cell coordinates and
 * the SSE2 partial-sum order.  HPD_DIST_GCC_AARCH64 reproduces GCC -Ofast on aarch64
 * (NEON lanes accumulated with fused multiply-adds, folded pairwise, fused tail); for
 * the integer element types the distance modes differ only in how EPS2 = (T)(float)
 * (eps * eps) converts an out-of-range value: x86-64 gives 0x80...0, aarch64 saturates. */
typedef enum { HPD_CELL_RECIP = 0, HPD_CELL_DIV = 1 } hpd_cell_mode;
typedef enum { HPD_DIST_GCC_X86 = 0, HPD_DIST_SEQ = 1, HPD_DIST_SEQ_FMA = 2, HPD_DIST_GCC_AARCH64 = 3 } hpd_dist_mode;

typedef struct hpd_handle hpd_handle;

/* Phase timings of the last call on a handle, in milliseconds of device time. */
typedef struct {
    double total_ms;
    double index_ms;    /* min/max, cell ids, radix sort, gather, cell table */
    double core_ms;     /* neighbour counts with early exit at minPoints */
    double union_ms;    /* core-core connectivity */
    double border_ms;   /* border assignment */
    double tie_ms;      /* tie-break for borders next to several clusters */
    double finalize_ms; /* labels + un-permute */
    int64_t n_cells;    /* non-empty cells */
    int64_t n_core;
    int64_t n_ambiguous; /* border points adjacent to >= 2 clusters */
    int64_t tie_iterations;
    int64_t kernel_launches;
    double extent_ms;      /* part of index_ms: per-dimension min / max */
    double cells_sort_ms;  /* part of index_ms: cell ids, radix sort, gather */
    double cell_table_ms;  /* part of index_ms: cell table and work items */
    double cell_ids_ms;    /* part of cells_sort_ms: the cell id of every point */
    double rules_ms;       /* part of union_ms: every core resolved to its cluster root */
    int64_t core_pairs;    /* distance evaluations of the core test (HPD_DIAG_COUNT_PAIRS only) */
} hpd_stats;

/* HPDBSCAN(epsilon, min_points): fails with HPD_ERR_INVALID and the upstream
 * message "epsilon needs to be positive" when epsilon <= 0. */
int hpd_create(float epsilon, uint64_t min_points, hpd_handle** out);
void hpd_destroy(hpd_handle* h);

int hpd_set_arith(hpd_handle* h, int cell_mode, int dist_mode);

/* Labels of border points next to two or more clusters.  HPD_TIE_EXACT (default)
 * gives the label the single-thread reference gives (the smallest provisional label
 * offered while its loop runs, hpdbscan.h:72-92), which needs a relaxation over
 * the provisional labels of the cores.  HPD_TIE_SMALLEST_ID skips it and gives such a
 * border the smallest cluster id among its core neighbours: a valid DBSCAN result
 * (the multi-threaded reference may give either), and cores, noise and every other
 * border keep their exact labels.  No counterpart in the reference. */
typedef enum { HPD_TIE_EXACT = 0, HPD_TIE_SMALLEST_ID = 1 } hpd_tie_mode;
int hpd_set_tie_break(hpd_handle* h, int mode);

/* Bound of the exact tie-break (no counterpart in the reference): it relaxes the
 * reference's provisional labels pass by pass until no value changes; a call that
 * would need more than `passes` passes gives up with HPD_ERR_TIMEOUT and the handle
 * stays usable.  0 restores the default (2^20 passes). */
int hpd_set_tie_pass_limit(hpd_handle* h, int32_t passes);

/* Diagnostics (no counterpart in the reference).  HPD_DIAG_COUNT_PAIRS: the core test
 * counts the distance evaluations it performs into hpd_stats.core_pairs (slower; for
 * measurement runs only).  0 turns diagnostics off. */
typedef enum { HPD_DIAG_COUNT_PAIRS = 1 } hpd_diag;
int hpd_set_diagnostics(hpd_handle* h, int32_t flags);

/* Tuning of the engine's work decomposition (no counterpart in the reference; labels
 * do not depend on it).  0 in a field keeps the built-in default.
 *   sparse_queries    work items of at most this many points test their queries against
 *                     one flat candidate list of the neighbour cells (default 8, max 32);
 *   dense_min_points  cells with at least this many points are connected through
 *                     certified sub-cells (default 128, min 32);
 *   greedy_tiles      candidate tiles a work item of the tie-break's greedy descent
 *                     scans at most (default 6). */
typedef struct {
    int32_t sparse_queries;
    int32_t dense_min_points;
    int32_t greedy_tiles;
} hpd_tuning;
int hpd_set_tuning(hpd_handle* h, const hpd_tuning* tuning);

/* A process-wide table of tunings by size class, consulted by every call whose handle
 * (or batch / served job) has no tuning of its own: the first entry with
 * n <= max_points and d == dims applies (dims 0 matches any d).  Written by the
 * autotuner (hpdbscan_gb300/tune.py); n_entries 0 clears it.  At most 64 entries. */
typedef struct {
    int64_t max_points;
    int32_t dims;
    hpd_tuning tuning;
} hpd_tuning_entry;
int hpd_set_tuning_table(const hpd_tuning_entry* entries, int32_t n_entries);

/* Test hook (no counterpart in the reference) for the next call on the handle:
 * HPD_INJECT_FAIL_ALLOC makes the first device allocation the call needs fail without
 * being attempted, so the call returns HPD_ERR_NOMEM. */
typedef enum { HPD_INJECT_FAIL_ALLOC = 1 } hpd_inject;
int hpd_debug_inject(hpd_handle* h, int32_t what);

/* Labels for n points of d coordinates (row-major, host memory) into labels[n]
 * (host memory), in input order.  `threads` is accepted for interface parity and
 * unused: the work runs on the current CUDA device. */
int hpd_cluster(hpd_handle* h, const void* data, int64_t n, int32_t d, int32_t dtype, int32_t threads,
                int64_t* labels);

/* Same, with data and labels in device memory, ordered on `stream`
 * (a cudaStream_t; NULL = the handle's own stream).  Returns after the labels
 * are written (the call synchronises the stream). */
int hpd_cluster_device(hpd_handle* h, const void* d_data, int64_t n, int32_t d, int32_t dtype,
                       int64_t* d_labels, void* stream);

int hpd_get_stats(const hpd_handle* h, hpd_stats* out);

/* ------------------------------------------------------------ batches, serving
 * No counterpart in the reference (its jobs run one at a time): many independent
 * clustering jobs on one GPU.  A job names host buffers; it stays owned by the caller
 * and must stay valid until the job completes. */
typedef struct {
    const void* data;      /* host, n x d row-major */
    int64_t n;
    int32_t d;
    int32_t dtype;         /* HPD_F32 or HPD_F64 */
    float epsilon;
    uint64_t min_points;
    int32_t cell_mode;     /* hpd_cell_mode, 0 = default */
    int32_t dist_mode;     /* hpd_dist_mode, 0 = default */
    int64_t* labels;       /* host, n: written in input order */
    int32_t status;        /* out: hpd_status of the job, -1 while pending */
    double queue_ms;       /* out: submission to start */
    double run_ms;         /* out: start to labels on the host */
    double deadline_ms;    /* in: a job still waiting for a worker this long after its
                            * submission completes with HPD_ERR_TIMEOUT without running;
                            * 0 = no deadline */
} hpd_job;

/* Runs every job of the array on the current GPU with n_workers concurrent streams
 * (0 = 8), largest jobs first.  Returns HPD_OK when all jobs succeeded; each job's own
 * status is in jobs[i].status. */
int hpd_cluster_batch(hpd_job* jobs, int64_t n_jobs, int32_t n_workers);

/* A serving loop on the current GPU: n_workers threads, each with its own CUDA stream
 * and device buffers (sized up front for reserve_points points of reserve_dims
 * dimensions), take submitted jobs in arrival order; a job is admitted when the device
 * bytes of the jobs in flight plus its own stay within hbm_budget_bytes (a job is
 * always admitted onto an idle server), and starts as soon as a worker is free, so jobs
 * that arrive while others run overlap with them on the device. */
typedef struct hpd_server hpd_server;
int hpd_server_create(int32_t n_workers, uint64_t hbm_budget_bytes, int64_t reserve_points, int32_t reserve_dims,
                      hpd_server** out);
int hpd_server_submit(hpd_server* s, hpd_job* job, int64_t* ticket);
int hpd_server_poll(hpd_server* s, int64_t ticket, int32_t* done);
/* Blocks until the job is done, forgets the ticket and returns the job's status. */
int hpd_server_wait(hpd_server* s, int64_t ticket);
/* Finishes the jobs already submitted, then stops the workers. */
void hpd_server_destroy(hpd_server* s);
const char* hpd_server_last_error(void);

/* No counterpart in the reference.  Clustering for callers that cannot call
 * cudaMalloc (a fixed device-memory budget, a framework that owns all device
 * allocations): same computation and labels as hpd_cluster_device, but every
 * intermediate buffer lives in one file-scope device array of 16 MiB that the
 * library keeps on each GPU that loads it until the process exits.  Nothing is
 * allocated: no cudaMalloc / cudaFree and no handle.
 *   - at most 32768 points (any d <= 16, float32 or float64); larger inputs fail with
 *     HPD_ERR_INVALID;
 *   - data, labels and stream as for hpd_cluster_device (NULL stream = the legacy
 *     default stream); the call reads counts back and synchronises that stream
 *     before it returns, after the labels are written;
 *   - each call looks up the array's device address on the current device
 *     (cudaGetSymbolAddress, which allocates nothing), so the address stays right
 *     after cudaDeviceReset;
 *   - every call uses the same array, which keeps the last call's contents: calls that
 *     overlap on the GPU (from two host threads or two streams) race;
 *   - errors are reported by hpd_noalloc_last_error(). */
int hpd_cluster_device_noalloc(float epsilon, uint64_t min_points, int32_t cell_mode, int32_t dist_mode,
                               const void* d_data, int64_t n, int32_t d, int32_t dtype, int64_t* d_labels,
                               void* stream);
const char* hpd_noalloc_last_error(void);

/* HDF5 files (the reference's IO::read_hdf5 / IO::write_hdf5, include/io.h:35-197),
 * read and written by the library's own implementation of the HDF5 file format (no
 * libhdf5): superblock versions 0-3, symbol-table and compact link groups, fixed-point
 * and IEEE floating-point data of either byte order, compact / contiguous / chunked
 * (unfiltered) storage.
 *
 * hpd_h5_read: the 2-D dataset `dataset` (a path of groups separated by '/') of the
 * file `path`, row-major in its own element type, in a buffer the library allocates
 * (release it with hpd_h5_free); *n rows (points), *d columns, *dtype the hpd_dtype of
 * the reference's dispatch (include/hpdbscan.h:309-355).  Errors: HPD_ERR_INVALID
 * "Could not open <path>" / "Could not open dataset <name>" / "Data in dataset <name>
 * should be a matrix"; HPD_ERR_UNSUPPORTED "Unsupported signed integer precision" and
 * the other element-type messages; HPD_ERR_RUNTIME "Failed to read data" (a broken
 * file, or compressed storage, with the reason in parentheses).
 *
 * hpd_h5_write: n int64 labels as the dataset `dataset` of the file `path` like the
 * reference: the file is created if it does not exist; a dataset of that name is
 * created as 1-D int64, or an existing one receives the labels (its first n elements
 * for a 1-D dataset, else all of exactly n elements; integer targets saturate,
 * floating-point targets round).  Errors: HPD_ERR_INVALID "Could not open <path>" /
 * "Could not open dataset <name>"; HPD_ERR_RUNTIME "Failed to write data, target data
 * set is probably of wrong size or type". */
int hpd_h5_read(const char* path, const char* dataset, void** data, int64_t* n, int32_t* d, int32_t* dtype);
void hpd_h5_free(void* data);
int hpd_h5_write(const char* path, const char* dataset, const int64_t* labels, int64_t n);

/* Message of the last failed call on this thread ("" if none). */
const char* hpd_last_error(void);

/* Version string of the engine. */
const char* hpd_version(void);

#ifdef __cplusplus
}
#endif
#endif
