// Batched and served clustering: a pool of worker threads, each with its own CUDA
// stream and grow-only device arenas, runs independent clustering jobs concurrently
// on one GPU.  Jobs are admitted in arrival order while the device bytes of the jobs
// in flight stay within the server's budget; a job starts as soon as a worker and
// budget are free (continuous batching), so small jobs overlap on the device instead of
// leaving it idle between the host round trips of one pipeline.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "hpd_internal.h"

using namespace hpd;

namespace {

using Clock = std::chrono::steady_clock;

thread_local std::string g_err;
int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}

size_t elem_size(int dtype) {
    switch (dtype) {
        case HPD_F32: return 4;
        case HPD_F64: return 8;
        default: return 0;
    }
}

// Upper bound of the device bytes one job holds while it runs: input, labels and the
// pipeline's buffers (about 200 bytes per point plus the coordinate copies), plus the
// largest grid-sized lookup table the pipeline may build (2^26 cells of 4 bytes).
uint64_t job_bytes(const hpd_job& j) {
    const uint64_t n = (uint64_t)j.n, d = (uint64_t)j.d, es = elem_size(j.dtype);
    return n * (2 * d * es + 8 + d * 4 + 240) + (uint64_t(1) << 28);
}

struct Entry {
    hpd_job* job = nullptr;
    uint64_t bytes = 0;
    bool done = false;
    Clock::time_point submit, start, end;
};

struct WorkerState {
    cudaStream_t stream = nullptr;
    Arena small, main, in, out;
    RunInfo info;
};

}  // namespace

struct hpd_server {
    int device = 0;
    uint64_t budget = 0;
    uint64_t in_flight = 0;
    int64_t next_ticket = 1;
    bool stop = false;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<int64_t> queue;
    std::unordered_map<int64_t, Entry> entries;
    std::vector<std::thread> threads;
    std::vector<WorkerState*> states;
    uint64_t completed = 0;

    void worker(WorkerState* ws, int64_t reserve_points, int reserve_dims);
};

namespace {

int run_job(WorkerState& ws, hpd_job& j) {
    const size_t es = elem_size(j.dtype);
    const size_t in_bytes = (size_t)j.n * j.d * es, out_bytes = (size_t)j.n * sizeof(int64_t);
    cudaError_t e = ws.in.reserve(in_bytes);
    if (e == cudaSuccess) e = ws.out.reserve(out_bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return e == cudaErrorMemoryAllocation ? HPD_ERR_NOMEM : HPD_ERR_CUDA;
    }
    e = cudaMemcpyAsync(ws.in.ptr, j.data, in_bytes, cudaMemcpyHostToDevice, ws.stream);
    if (e != cudaSuccess) return HPD_ERR_CUDA;
    Request rq;
    rq.d_data = ws.in.ptr;
    rq.n = j.n;
    rq.d = j.d;
    rq.eps = j.epsilon;
    rq.min_points = j.min_points;
    rq.cell_mode = j.cell_mode;
    rq.dist_mode = j.dist_mode;
    rq.d_labels = static_cast<int64_t*>(ws.out.ptr);
    rq.stream = ws.stream;
    std::string err;
    int rc = j.dtype == HPD_F32 ? run_pipeline<float>(rq, ws.small, ws.main, nullptr, ws.info, err)
                                : run_pipeline<double>(rq, ws.small, ws.main, nullptr, ws.info, err);
    if (rc != HPD_OK) return rc;
    e = cudaMemcpyAsync(j.labels, ws.out.ptr, out_bytes, cudaMemcpyDeviceToHost, ws.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ws.stream);
    return e == cudaSuccess ? HPD_OK : HPD_ERR_CUDA;
}

int validate(const hpd_job* j) {
    if (!j) return fail(HPD_ERR_INVALID, "null job");
    if (!(j->deadline_ms >= 0)) return fail(HPD_ERR_INVALID, "deadline must be >= 0");
    if (j->cell_mode != HPD_CELL_RECIP && j->cell_mode != HPD_CELL_DIV) return fail(HPD_ERR_INVALID, "bad cell mode");
    if (j->dist_mode < HPD_DIST_GCC_X86 || j->dist_mode > HPD_DIST_GCC_AARCH64)
        return fail(HPD_ERR_INVALID, "bad distance mode");
    if (!(j->epsilon > 0.0f)) return fail(HPD_ERR_INVALID, "epsilon needs to be positive");
    if (elem_size(j->dtype) == 0) return fail(HPD_ERR_UNSUPPORTED, "element type not supported by this build");
    if (j->n < 0 || j->n > INT32_MAX - 1 || j->d < 1) return fail(HPD_ERR_INVALID, "bad shape");
    if (j->d > kMaxDims) return fail(HPD_ERR_UNSUPPORTED, "at most 16 dimensions are supported");
    if (j->n > 0 && (!j->data || !j->labels)) return fail(HPD_ERR_INVALID, "null data or label pointer");
    return HPD_OK;
}

double ms_between(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

}  // namespace

void hpd_server::worker(WorkerState* ws, int64_t reserve_points, int reserve_dims) {
    cudaSetDevice(device);
    cudaStreamCreateWithFlags(&ws->stream, cudaStreamNonBlocking);
    if (reserve_points > 0) {
        // size the buffers once for the largest expected job so that serving never allocates
        hpd_job probe{};
        probe.n = reserve_points;
        probe.d = reserve_dims;
        probe.dtype = HPD_F32;
        ws->in.reserve((size_t)reserve_points * reserve_dims * 8);
        ws->out.reserve((size_t)reserve_points * 8);
        ws->main.reserve((size_t)(job_bytes(probe) - (uint64_t(1) << 28)) + (size_t(1) << 28));
        ws->small.reserve(size_t(1) << 20);
        cudaGetLastError();
    }
    for (;;) {
        int64_t ticket = 0;
        hpd_job* job = nullptr;
        bool late = false;
        {
            std::unique_lock<std::mutex> lock(mu);
            // a job past its deadline leaves the queue at once, without budget
            auto expired = [&](const Entry& en) {
                return en.job->deadline_ms > 0 && ms_between(en.submit, Clock::now()) > en.job->deadline_ms;
            };
            cv_work.wait_for(lock, std::chrono::milliseconds(5), [&] {
                if (stop) return true;
                if (queue.empty()) return false;
                const Entry& head = entries[queue.front()];
                return in_flight == 0 || in_flight + head.bytes <= budget || expired(head);
            });
            if (stop && queue.empty()) break;
            if (queue.empty()) continue;
            ticket = queue.front();
            Entry& en = entries[ticket];
            late = expired(en);
            if (!late && !(in_flight == 0 || in_flight + en.bytes <= budget)) continue;
            queue.pop_front();
            if (!late) in_flight += en.bytes;
            en.start = Clock::now();
            job = en.job;
        }
        const int rc = late ? HPD_ERR_TIMEOUT : (job->n > 0 ? run_job(*ws, *job) : HPD_OK);
        {
            std::lock_guard<std::mutex> lock(mu);
            Entry& en = entries[ticket];
            en.end = Clock::now();
            en.done = true;
            if (!late) in_flight -= en.bytes;
            job->status = rc;
            job->queue_ms = ms_between(en.submit, en.start);
            job->run_ms = ms_between(en.start, en.end);
            ++completed;
        }
        cv_done.notify_all();
        cv_work.notify_all();
    }
    cudaStreamDestroy(ws->stream);
}

extern "C" {

const char* hpd_server_last_error(void) { return g_err.c_str(); }

int hpd_server_create(int32_t n_workers, uint64_t hbm_budget_bytes, int64_t reserve_points, int32_t reserve_dims,
                      hpd_server** out) {
    if (!out) return fail(HPD_ERR_INVALID, "null output");
    *out = nullptr;
    if (n_workers < 1 || n_workers > 256) return fail(HPD_ERR_INVALID, "n_workers must be in [1, 256]");
    hpd_server* s = new hpd_server();
    if (cudaGetDevice(&s->device) != cudaSuccess) {
        cudaGetLastError();
        delete s;
        return fail(HPD_ERR_CUDA, "no CUDA device available");
    }
    s->budget = hbm_budget_bytes;
    for (int i = 0; i < n_workers; ++i) {
        WorkerState* ws = new WorkerState();
        s->states.push_back(ws);
        s->threads.emplace_back(&hpd_server::worker, s, ws, reserve_points, reserve_dims < 1 ? 3 : reserve_dims);
    }
    *out = s;
    return HPD_OK;
}

int hpd_server_submit(hpd_server* s, hpd_job* job, int64_t* ticket) {
    if (!s || !ticket) return fail(HPD_ERR_INVALID, "null argument");
    int rc = validate(job);
    if (rc) {
        if (job) job->status = rc;
        return rc;
    }
    {
        std::lock_guard<std::mutex> lock(s->mu);
        const int64_t t = s->next_ticket++;
        Entry& en = s->entries[t];
        en.job = job;
        en.bytes = job_bytes(*job);
        en.submit = Clock::now();
        job->status = -1;
        s->queue.push_back(t);
        *ticket = t;
    }
    s->cv_work.notify_one();
    return HPD_OK;
}

int hpd_server_poll(hpd_server* s, int64_t ticket, int32_t* done) {
    if (!s || !done) return fail(HPD_ERR_INVALID, "null argument");
    std::lock_guard<std::mutex> lock(s->mu);
    auto it = s->entries.find(ticket);
    if (it == s->entries.end()) return fail(HPD_ERR_INVALID, "unknown ticket");
    *done = it->second.done ? 1 : 0;
    return HPD_OK;
}

int hpd_server_wait(hpd_server* s, int64_t ticket) {
    if (!s) return fail(HPD_ERR_INVALID, "null argument");
    std::unique_lock<std::mutex> lock(s->mu);
    auto it = s->entries.find(ticket);
    if (it == s->entries.end()) return fail(HPD_ERR_INVALID, "unknown ticket");
    s->cv_done.wait(lock, [&] { return it->second.done; });
    const int status = it->second.job->status;
    s->entries.erase(it);
    return status;
}

void hpd_server_destroy(hpd_server* s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    for (auto& t : s->threads) t.join();
    for (auto* ws : s->states) delete ws;
    delete s;
}

int hpd_cluster_batch(hpd_job* jobs, int64_t n_jobs, int32_t n_workers) {
    if (n_jobs < 0 || (n_jobs > 0 && !jobs)) return fail(HPD_ERR_INVALID, "bad job array");
    for (int64_t i = 0; i < n_jobs; ++i) {
        const int rc = validate(&jobs[i]);
        if (rc) {
            jobs[i].status = rc;
            return rc;
        }
    }
    if (n_jobs == 0) return HPD_OK;
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
        cudaGetLastError();
        return fail(HPD_ERR_CUDA, "cudaMemGetInfo failed");
    }
    // largest jobs first, so that the tail of the batch is made of short jobs
    std::vector<int64_t> order(n_jobs);
    for (int64_t i = 0; i < n_jobs; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return jobs[a].n > jobs[b].n; });
    int64_t max_n = jobs[order[0]].n;
    int max_d = 1;
    for (int64_t i = 0; i < n_jobs; ++i) max_d = std::max(max_d, (int)jobs[i].d);
    hpd_server* s = nullptr;
    int rc = hpd_server_create(n_workers < 1 ? 8 : n_workers, (uint64_t)(free_b * 0.8), max_n, max_d, &s);
    if (rc) return rc;
    std::vector<int64_t> tickets(n_jobs);
    for (int64_t k = 0; k < n_jobs; ++k) hpd_server_submit(s, &jobs[order[k]], &tickets[k]);
    int first_err = HPD_OK;
    for (int64_t k = 0; k < n_jobs; ++k) {
        const int st = hpd_server_wait(s, tickets[k]);
        if (st != HPD_OK && first_err == HPD_OK) first_err = st;
    }
    hpd_server_destroy(s);
    if (first_err) return fail(first_err, "one or more jobs failed (see their status)");
    return HPD_OK;
}

}  // extern "C"
