// C ABI of the engine (include/hpdbscan_gb300.h): handles, argument checks with
// the upstream error messages, host<->device staging and dtype dispatch.
#include <cuda_runtime.h>

#include <climits>
#include <cstring>
#include <new>
#include <string>

#include "hpd_internal.h"

using namespace hpd;

struct hpd_handle {
    float eps;
    uint64_t min_points;
    int cell_mode = HPD_CELL_RECIP;
    int dist_mode = HPD_DIST_GCC_X86;
    int tie_mode = HPD_TIE_EXACT;
    int tie_pass_limit = kDefaultTiePassLimit;
    int diag = 0;    // hpd_diag bits
    hpd_tuning tuning = {0, 0, 0};
    int inject = 0;  // hpd_inject bits for the next call
    int device = 0;
    cudaStream_t stream = nullptr;
    Arena small, main, in_buf, out_buf;
    Timers timers;
    RunInfo last;
};

namespace {
thread_local std::string g_error;

int fail(int code, const std::string& msg) {
    g_error = msg;
    return code;
}

size_t dtype_size(int dtype) {
    switch (dtype) {
        case HPD_F32: return 4;
        case HPD_F64: return 8;
        case HPD_I8: case HPD_U8: return 1;
        case HPD_I16: case HPD_U16: return 2;
        case HPD_I32: case HPD_U32: return 4;
        case HPD_I64: case HPD_U64: return 8;
        default: return 0;
    }
}

int check_shape(int64_t n, int32_t d, int32_t dtype) {
    if (dtype_size(dtype) == 0) return fail(HPD_ERR_UNSUPPORTED, "Unsupported data set type");
    if (n < 0 || n > INT_MAX - 1) return fail(HPD_ERR_INVALID, "number of points must be in [0, 2^31 - 2]");
    if (d < 1) return fail(HPD_ERR_INVALID, "data must have at least one dimension");
    if (d > kMaxDims) return fail(HPD_ERR_UNSUPPORTED, "at most 16 dimensions are supported");
    return HPD_OK;
}

int run(hpd_handle* h, const void* d_data, int64_t n, int32_t d, int32_t dtype, int64_t* d_labels, cudaStream_t s) {
    Request rq;
    rq.d_data = d_data;
    rq.n = n;
    rq.d = d;
    rq.eps = h->eps;
    rq.min_points = h->min_points;
    rq.cell_mode = h->cell_mode;
    rq.dist_mode = h->dist_mode;
    rq.tie_mode = h->tie_mode;
    rq.d_labels = d_labels;
    rq.stream = s;
    rq.tie_pass_limit = h->tie_pass_limit;
    rq.count_pairs = (h->diag & HPD_DIAG_COUNT_PAIRS) != 0;
    rq.tuning = h->tuning;
    std::string err;
    int rc;
    switch (dtype) {
        case HPD_F32: rc = run_pipeline<float>(rq, h->small, h->main, &h->timers, h->last, err); break;
        case HPD_F64: rc = run_pipeline<double>(rq, h->small, h->main, &h->timers, h->last, err); break;
        case HPD_I8: rc = run_pipeline<int8_t>(rq, h->small, h->main, &h->timers, h->last, err); break;
        case HPD_I16: rc = run_pipeline<int16_t>(rq, h->small, h->main, &h->timers, h->last, err); break;
        case HPD_I32: rc = run_pipeline<int32_t>(rq, h->small, h->main, &h->timers, h->last, err); break;
        case HPD_I64: rc = run_pipeline<int64_t>(rq, h->small, h->main, &h->timers, h->last, err); break;
        case HPD_U8: rc = run_pipeline<uint8_t>(rq, h->small, h->main, &h->timers, h->last, err); break;
        case HPD_U16: rc = run_pipeline<uint16_t>(rq, h->small, h->main, &h->timers, h->last, err); break;
        case HPD_U32: rc = run_pipeline<uint32_t>(rq, h->small, h->main, &h->timers, h->last, err); break;
        case HPD_U64: rc = run_pipeline<uint64_t>(rq, h->small, h->main, &h->timers, h->last, err); break;
        default: return fail(HPD_ERR_UNSUPPORTED, "element type not supported by this build");
    }
    if (rc != HPD_OK) return fail(rc, err);
    return HPD_OK;
}
// the injected allocation failure hits the first arena of the call that must grow
void arm_alloc_failure(hpd_handle* h) {
    if (!(h->inject & HPD_INJECT_FAIL_ALLOC)) return;
    h->inject &= ~HPD_INJECT_FAIL_ALLOC;
    h->in_buf.fail_next = h->out_buf.fail_next = h->small.fail_next = h->main.fail_next = true;
}
void disarm_alloc_failure(hpd_handle* h) {
    h->in_buf.fail_next = h->out_buf.fail_next = h->small.fail_next = h->main.fail_next = false;
}
}  // namespace

void hpd::set_last_error(const std::string& msg) { g_error = msg; }

extern "C" {

const char* hpd_last_error(void) { return g_error.c_str(); }

const char* hpd_version(void) { return "hpdbscan_gb300 0.1 (sm_103a)"; }

int hpd_create(float epsilon, uint64_t min_points, hpd_handle** out) {
    if (!out) return fail(HPD_ERR_INVALID, "null output handle");
    *out = nullptr;
    if (!(epsilon > 0.0f)) return fail(HPD_ERR_INVALID, "epsilon needs to be positive");
    hpd_handle* h = new (std::nothrow) hpd_handle();
    if (!h) return fail(HPD_ERR_NOMEM, "out of host memory");
    h->eps = epsilon;
    h->min_points = min_points;
    if (cudaGetDevice(&h->device) != cudaSuccess) {
        cudaGetLastError();
        delete h;
        return fail(HPD_ERR_CUDA, "no CUDA device available");
    }
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        delete h;
        return fail(HPD_ERR_CUDA, "cudaStreamCreate failed");
    }
    h->timers.ok = true;
    for (auto& e : h->timers.ev)
        if (cudaEventCreate(&e) != cudaSuccess) h->timers.ok = false;
    *out = h;
    return HPD_OK;
}

void hpd_destroy(hpd_handle* h) {
    if (!h) return;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    for (auto& e : h->timers.ev)
        if (e) cudaEventDestroy(e);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
}

int hpd_set_arith(hpd_handle* h, int cell_mode, int dist_mode) {
    if (!h) return fail(HPD_ERR_INVALID, "null handle");
    if (cell_mode != HPD_CELL_RECIP && cell_mode != HPD_CELL_DIV) return fail(HPD_ERR_INVALID, "bad cell mode");
    if (dist_mode < HPD_DIST_GCC_X86 || dist_mode > HPD_DIST_GCC_AARCH64) return fail(HPD_ERR_INVALID, "bad distance mode");
    h->cell_mode = cell_mode;
    h->dist_mode = dist_mode;
    return HPD_OK;
}

int hpd_set_tie_break(hpd_handle* h, int mode) {
    if (!h) return fail(HPD_ERR_INVALID, "null handle");
    if (mode != HPD_TIE_EXACT && mode != HPD_TIE_SMALLEST_ID) return fail(HPD_ERR_INVALID, "bad tie-break mode");
    h->tie_mode = mode;
    return HPD_OK;
}

int hpd_set_tie_pass_limit(hpd_handle* h, int32_t passes) {
    if (!h) return fail(HPD_ERR_INVALID, "null handle");
    if (passes < 0) return fail(HPD_ERR_INVALID, "pass limit must be >= 0");
    h->tie_pass_limit = passes == 0 ? kDefaultTiePassLimit : passes;
    return HPD_OK;
}

int hpd_set_tuning(hpd_handle* h, const hpd_tuning* tuning) {
    if (!h) return fail(HPD_ERR_INVALID, "null handle");
    if (!tuning) {
        h->tuning = hpd_tuning{0, 0, 0};
        return HPD_OK;
    }
    if (tuning->sparse_queries < 0 || tuning->sparse_queries > 32 || tuning->dense_min_points < 0 ||
        (tuning->dense_min_points > 0 && tuning->dense_min_points < 32) || tuning->greedy_tiles < 0)
        return fail(HPD_ERR_INVALID, "tuning out of range");
    h->tuning = *tuning;
    return HPD_OK;
}

int hpd_set_tuning_table(const hpd_tuning_entry* entries, int32_t n_entries) {
    if (set_tuning_table(entries, n_entries) != HPD_OK)
        return fail(HPD_ERR_INVALID, "tuning table: at most 64 entries, non-null when not empty");
    return HPD_OK;
}

int hpd_set_diagnostics(hpd_handle* h, int32_t flags) {
    if (!h) return fail(HPD_ERR_INVALID, "null handle");
    if (flags & ~HPD_DIAG_COUNT_PAIRS) return fail(HPD_ERR_INVALID, "bad diagnostics flags");
    h->diag = flags;
    return HPD_OK;
}

int hpd_debug_inject(hpd_handle* h, int32_t what) {
    if (!h) return fail(HPD_ERR_INVALID, "null handle");
    if (what & ~HPD_INJECT_FAIL_ALLOC) return fail(HPD_ERR_INVALID, "bad injection");
    h->inject |= what;
    return HPD_OK;
}

int hpd_cluster_device(hpd_handle* h, const void* d_data, int64_t n, int32_t d, int32_t dtype, int64_t* d_labels,
                       void* stream) {
    if (!h) return fail(HPD_ERR_INVALID, "null handle");
    int rc = check_shape(n, d, dtype);
    if (rc) return rc;
    if (n == 0) return HPD_OK;
    if (!d_data || !d_labels) return fail(HPD_ERR_INVALID, "null data or label pointer");
    if (cudaSetDevice(h->device) != cudaSuccess) return fail(HPD_ERR_CUDA, "cudaSetDevice failed");
    cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : h->stream;
    arm_alloc_failure(h);
    rc = run(h, d_data, n, d, dtype, d_labels, s);
    disarm_alloc_failure(h);
    return rc;
}

int hpd_cluster(hpd_handle* h, const void* data, int64_t n, int32_t d, int32_t dtype, int32_t threads,
                int64_t* labels) {
    (void)threads;
    if (!h) return fail(HPD_ERR_INVALID, "null handle");
    int rc = check_shape(n, d, dtype);
    if (rc) return rc;
    if (n == 0) return HPD_OK;
    if (!data || !labels) return fail(HPD_ERR_INVALID, "null data or label pointer");
    if (cudaSetDevice(h->device) != cudaSuccess) return fail(HPD_ERR_CUDA, "cudaSetDevice failed");
    const size_t in_bytes = (size_t)n * d * dtype_size(dtype);
    const size_t out_bytes = (size_t)n * sizeof(int64_t);
    arm_alloc_failure(h);
    cudaError_t e = h->in_buf.reserve(in_bytes);
    if (e == cudaSuccess) e = h->out_buf.reserve(out_bytes);
    if (e != cudaSuccess) {
        disarm_alloc_failure(h);
        return fail(e == cudaErrorMemoryAllocation ? HPD_ERR_NOMEM : HPD_ERR_CUDA, cudaGetErrorString(e));
    }
    // the caller's array is only read: the upstream class works on a copy (dataset.h:37-43)
    e = cudaMemcpyAsync(h->in_buf.ptr, data, in_bytes, cudaMemcpyHostToDevice, h->stream);
    if (e != cudaSuccess) return fail(HPD_ERR_CUDA, cudaGetErrorString(e));
    rc = run(h, h->in_buf.ptr, n, d, dtype, static_cast<int64_t*>(h->out_buf.ptr), h->stream);
    disarm_alloc_failure(h);
    if (rc) return rc;
    e = cudaMemcpyAsync(labels, h->out_buf.ptr, out_bytes, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return fail(HPD_ERR_CUDA, cudaGetErrorString(e));
    return HPD_OK;
}

int hpd_get_stats(const hpd_handle* h, hpd_stats* out) {
    if (!h || !out) return fail(HPD_ERR_INVALID, "null argument");
    memset(out, 0, sizeof *out);
    out->total_ms = h->last.ms[0];
    out->index_ms = h->last.ms[1];
    out->core_ms = h->last.ms[2];
    out->union_ms = h->last.ms[3];
    out->border_ms = h->last.ms[4];
    out->tie_ms = h->last.ms[5];
    out->finalize_ms = h->last.ms[6];
    out->extent_ms = h->last.index_ms[0];
    out->cells_sort_ms = h->last.index_ms[1];
    out->cell_table_ms = h->last.index_ms[2];
    out->cell_ids_ms = h->last.cell_ids_ms;
    out->rules_ms = h->last.rules_ms;
    out->core_pairs = h->last.core_pairs;
    out->n_cells = h->last.n_cells;
    out->n_core = h->last.n_core;
    out->n_ambiguous = h->last.n_ambiguous;
    out->tie_iterations = h->last.tie_iterations;
    out->kernel_launches = h->last.launches;
    return HPD_OK;
}

}  // extern "C"
