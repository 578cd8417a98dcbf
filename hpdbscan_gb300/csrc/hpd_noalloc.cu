// Clustering entry point that allocates nothing, for callers that cannot call
// cudaMalloc (for example code running under a fixed device-memory budget or inside
// a framework that owns every allocation).  Its scratch is a file-scope device array
// of kNoAllocScratchBytes, held by every GPU that loads the library until the
// process exits; it serves inputs of at most kNoAllocMaxPoints points.
#include <cuda_runtime.h>

#include <climits>
#include <string>

#include "hpd_internal.h"

namespace {

constexpr int64_t kNoAllocMaxPoints = 32768;
constexpr size_t kNoAllocSmallBytes = size_t(1) << 20;   // extent reduction partials
constexpr size_t kNoAllocScratchBytes = size_t(16) << 20; // enough for 32768 points, d <= 16, doubles
__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}

// Device address of the scratch array on the current device.  In host code the
// array's name is only a host-side stand-in, so the address is looked up with the
// device current.  The lookup runs on every call (it allocates nothing): an address
// kept from an earlier call would go stale after cudaDeviceReset or under another
// context on the same device, and kernels would then write through it.
int scratch_address(void** out) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
        cudaGetLastError();
        return fail(HPD_ERR_CUDA, std::string("cudaGetSymbolAddress failed: ") + cudaGetErrorString(e));
    }
    *out = p;
    return HPD_OK;
}

}  // namespace

extern "C" {

const char* hpd_noalloc_last_error(void) { return g_err.c_str(); }

int hpd_cluster_device_noalloc(float epsilon, uint64_t min_points, int32_t cell_mode, int32_t dist_mode,
                               const void* d_data, int64_t n, int32_t d, int32_t dtype, int64_t* d_labels,
                               void* stream) {
    using namespace hpd;
    if (!(epsilon > 0.0f)) return fail(HPD_ERR_INVALID, "epsilon needs to be positive");
    if (dtype != HPD_F32 && dtype != HPD_F64) return fail(HPD_ERR_UNSUPPORTED, "element type not supported by this build");
    if (n < 0 || d < 1) return fail(HPD_ERR_INVALID, "bad shape");
    if (d > kMaxDims) return fail(HPD_ERR_UNSUPPORTED, "at most 16 dimensions are supported");
    if (n > kNoAllocMaxPoints)
        return fail(HPD_ERR_INVALID, "the no-allocation entry point takes at most 32768 points (got " +
                                         std::to_string(n) + ")");
    if (cell_mode != HPD_CELL_RECIP && cell_mode != HPD_CELL_DIV) return fail(HPD_ERR_INVALID, "bad cell mode");
    if (dist_mode < HPD_DIST_GCC_X86 || dist_mode > HPD_DIST_GCC_AARCH64) return fail(HPD_ERR_INVALID, "bad distance mode");
    if (n == 0) return HPD_OK;
    if (!d_data || !d_labels) return fail(HPD_ERR_INVALID, "null data or label pointer");
    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess) {
        cudaGetLastError();
        return fail(HPD_ERR_CUDA, "no usable CUDA device");
    }
    void* base = nullptr;
    int rc = scratch_address(&base);
    if (rc) return rc;

    // two arenas over the static array; they never allocate or free
    Arena small, main;
    small.fixed = main.fixed = true;
    small.ptr = base;
    small.cap = kNoAllocSmallBytes;
    main.ptr = static_cast<unsigned char*>(base) + kNoAllocSmallBytes;
    main.cap = kNoAllocScratchBytes - kNoAllocSmallBytes;

    Request rq;
    rq.d_data = d_data;
    rq.n = n;
    rq.d = d;
    rq.eps = epsilon;
    rq.min_points = min_points;
    rq.cell_mode = cell_mode;
    rq.dist_mode = dist_mode;
    rq.d_labels = d_labels;
    rq.stream = static_cast<cudaStream_t>(stream);
    rq.no_dense = true;
    // the built-in tuning, never the process-wide table: the scratch budget is sized for it
    rq.tuning = hpd_tuning{kDefaultSparseQueries, kDefaultDenseMinPoints, kDefaultGreedyTiles};
    RunInfo info;
    std::string err;
    rc = dtype == HPD_F32 ? run_pipeline<float>(rq, small, main, nullptr, info, err)
                          : run_pipeline<double>(rq, small, main, nullptr, info, err);
    if (rc != HPD_OK) return fail(rc, err);
    return HPD_OK;
}

}  // extern "C"
