// Device-wide exclusive scan and stable LSD radix sort of (cell id, point index)
// pairs.  The sort replaces the reference's sequential counting sort by cell
// (spatial_index.h:184-216): sorting the pairs stably by cell id, with the point
// indices starting in input order, gives the same (cell id, input index) order.
#include "hpd_internal.h"

namespace hpd {

namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;
constexpr int kScanTile = kScanThreads * kScanItems;  // 4096

template <typename T>
__device__ __forceinline__ T block_exclusive_sum(T v, T* s_warp, T* total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    T inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
    }
    if (lane == 31) s_warp[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        T w = lane < (int)(blockDim.x >> 5) ? s_warp[lane] : T(0);
        T wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            T y = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += y;
        }
        if (lane < (int)(blockDim.x >> 5)) s_warp[lane] = wi - w;
        if (lane == 31) *total = wi;
    }
    __syncthreads();
    T r = s_warp[warp] + inc - v;
    __syncthreads();
    return r;
}

template <typename T>
__global__ void __launch_bounds__(kScanThreads) k_scan_reduce(const T* __restrict__ in, int64_t n, T* __restrict__ sums) {
    __shared__ T s_warp[32];
    __shared__ T s_total;
    const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
    T acc = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i)
        if (base + i < n) acc += in[base + i];
    block_exclusive_sum(acc, s_warp, &s_total);
    if (threadIdx.x == 0) sums[blockIdx.x] = s_total;
}

// Exclusive scan of the block sums by one block; writes the grand total.
template <typename T>
__global__ void __launch_bounds__(1024) k_scan_top(T* __restrict__ sums, int64_t nb, T* __restrict__ total) {
    __shared__ T s_warp[32];
    __shared__ T s_total;
    const int64_t per = (nb + blockDim.x - 1) / blockDim.x;
    const int64_t lo = (int64_t)threadIdx.x * per;
    T acc = 0;
    for (int64_t i = lo; i < lo + per && i < nb; ++i) acc += sums[i];
    T run = block_exclusive_sum(acc, s_warp, &s_total);
    for (int64_t i = lo; i < lo + per && i < nb; ++i) {
        T v = sums[i];
        sums[i] = run;
        run += v;
    }
    if (threadIdx.x == 0 && total) *total = s_total;
}

template <typename T>
__global__ void __launch_bounds__(kScanThreads) k_scan_apply(const T* __restrict__ in, int64_t n, const T* __restrict__ sums,
                                                             T* __restrict__ out) {
    __shared__ T s_warp[32];
    __shared__ T s_total;
    const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
    T v[kScanItems];
    T acc = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        v[i] = base + i < n ? in[base + i] : T(0);
        acc += v[i];
    }
    T run = block_exclusive_sum(acc, s_warp, &s_total) + sums[blockIdx.x];
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        if (base + i < n) out[base + i] = run;
        run += v[i];
    }
}

// ------------------------------------------------------------------ radix sort
constexpr int kSortThreads = 256;
constexpr int kSortWarps = kSortThreads / 32;
constexpr int kSortItems = 16;  // per thread
constexpr int kSortTile = kSortThreads * kSortItems;  // 4096
constexpr int kRadix = 256;

template <typename K>
__global__ void __launch_bounds__(kSortThreads) k_radix_upsweep(const K* __restrict__ keys, int64_t n, int shift,
                                                                uint32_t* __restrict__ counts, int nb) {
    __shared__ uint32_t hist[kRadix];
    hist[threadIdx.x] = 0;
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * kSortTile;
#pragma unroll 4
    for (int i = 0; i < kSortItems; ++i) {
        int64_t idx = base + (int64_t)i * kSortThreads + threadIdx.x;
        if (idx < n) atomicAdd(&hist[(uint32_t)(keys[idx] >> shift) & (kRadix - 1)], 1u);
    }
    __syncthreads();
    counts[(int64_t)threadIdx.x * nb + blockIdx.x] = hist[threadIdx.x];
}

// Stable scatter: warp w ranks items [w*512, (w+1)*512) of the tile in 16 rounds of
// 32 consecutive items; ranks within a round come from __match_any_sync, ranks
// across rounds from per-warp digit counters, ranks across warps from a prefix
// over the warps' counters.  Item order within each digit is therefore preserved.
// Each item keeps only its packed (digit, rank); the block then lists its items in
// digit order in shared memory and writes them out in that order, so that the items
// of one digit go to consecutive addresses (coalesced runs) instead of one scattered
// store per item.
template <typename K>
__global__ void __launch_bounds__(kSortThreads) k_radix_downsweep(const K* __restrict__ keys_in, const int32_t* __restrict__ vals_in,
                                                                  K* __restrict__ keys_out, int32_t* __restrict__ vals_out, int64_t n,
                                                                  int shift, const uint32_t* __restrict__ offsets, int nb) {
    __shared__ uint32_t wcnt[kSortWarps][kRadix];
    __shared__ uint32_t s_off[kRadix];    // global start of each digit for this tile
    __shared__ uint32_t s_start[kRadix];  // tile-local start of each digit
    __shared__ uint16_t s_item[kSortTile];  // tile-local item of each tile-local position
    __shared__ uint32_t s_warp[32];
    __shared__ uint32_t s_total;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < kSortWarps * kRadix; i += kSortThreads) (&wcnt[0][0])[i] = 0;
    s_off[threadIdx.x] = offsets[(int64_t)threadIdx.x * nb + blockIdx.x];
    __syncthreads();
    const int64_t tile0 = (int64_t)blockIdx.x * kSortTile;
    const int wbase = warp * (kSortItems * 32);
    const unsigned lt_mask = (1u << lane) - 1u;
    uint32_t dr[kSortItems];  // digit << 16 | rank within the warp's items of that digit
#pragma unroll
    for (int i = 0; i < kSortItems; ++i) {
        const int64_t idx = tile0 + wbase + i * 32 + lane;
        const bool ok = idx < n;
        const uint32_t dig = ok ? ((uint32_t)(keys_in[idx] >> shift) & (kRadix - 1)) : 0x10000u + lane;
        const unsigned peers = __match_any_sync(0xffffffffu, dig);
        uint32_t before = 0;
        if (ok) before = wcnt[warp][dig];
        __syncwarp();
        if (ok && (31 - __clz(peers)) == lane) wcnt[warp][dig] = before + __popc(peers);
        __syncwarp();
        dr[i] = ok ? (dig << 16) | (before + __popc(peers & lt_mask)) : 0xffffffffu;
    }
    __syncthreads();
    {
        // per digit (one per thread): the warps' counts become offsets within the
        // digit, and the digit's tile-local start is the prefix over the digits
        uint32_t run = 0;
#pragma unroll
        for (int w = 0; w < kSortWarps; ++w) {
            const uint32_t c = wcnt[w][threadIdx.x];
            wcnt[w][threadIdx.x] = run;
            run += c;
        }
        const int dlane = threadIdx.x & 31, dwarp = threadIdx.x >> 5;
        uint32_t inc = run;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
            if (dlane >= o) inc += y;
        }
        if (dlane == 31) s_warp[dwarp] = inc;
        __syncthreads();
        if (dwarp == 0) {
            const uint32_t wv = dlane < kSortWarps ? s_warp[dlane] : 0u;
            uint32_t wi = wv;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, wi, o);
                if (dlane >= o) wi += y;
            }
            if (dlane < kSortWarps) s_warp[dlane] = wi - wv;
            if (dlane == 31) s_total = wi;
        }
        __syncthreads();
        s_start[threadIdx.x] = s_warp[dwarp] + inc - run;
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < kSortItems; ++i) {
        if (dr[i] == 0xffffffffu) continue;
        const uint32_t dig = dr[i] >> 16;
        const uint32_t lp = s_start[dig] + wcnt[warp][dig] + (dr[i] & 0xffffu);
        s_item[lp] = (uint16_t)(wbase + i * 32 + lane);
    }
    __syncthreads();
    const int cnt = (int)s_total;
    for (int j = threadIdx.x; j < cnt; j += kSortThreads) {
        const int64_t src = tile0 + s_item[j];
        const K key = keys_in[src];
        const uint32_t dig = (uint32_t)(key >> shift) & (kRadix - 1);
        const int64_t pos = (int64_t)s_off[dig] + (j - (int)s_start[dig]);
        keys_out[pos] = key;
        vals_out[pos] = vals_in[src];
    }
}

}  // namespace

int64_t scan_scratch_elems(int64_t n) { return (n + kScanTile - 1) / kScanTile + 1; }

template <typename T>
void exclusive_scan(const T* in, T* out, int64_t n, T* scratch, T* total, cudaStream_t s, int* launches) {
    if (n <= 0) return;
    const int64_t nb = (n + kScanTile - 1) / kScanTile;
    k_scan_reduce<T><<<(unsigned)nb, kScanThreads, 0, s>>>(in, n, scratch);
    k_scan_top<T><<<1, 1024, 0, s>>>(scratch, nb, total);
    k_scan_apply<T><<<(unsigned)nb, kScanThreads, 0, s>>>(in, n, scratch, out);
    if (launches) *launches += 3;
}
template void exclusive_scan<uint32_t>(const uint32_t*, uint32_t*, int64_t, uint32_t*, uint32_t*, cudaStream_t, int*);
template void exclusive_scan<int64_t>(const int64_t*, int64_t*, int64_t, int64_t*, int64_t*, cudaStream_t, int*);

int64_t radix_counts_elems(int64_t n) { return (int64_t)kRadix * ((n + kSortTile - 1) / kSortTile); }

template <typename K>
int radix_sort_pairs(K* keys, int32_t* vals, K* keys_alt, int32_t* vals_alt, int64_t n, int bits, uint32_t* counts,
                     uint32_t* scan_scratch, cudaStream_t s, int* launches) {
    const int nb = (int)((n + kSortTile - 1) / kSortTile);
    const int64_t nc = (int64_t)kRadix * nb;
    int flips = 0;
    for (int shift = 0; shift < bits; shift += 8) {
        K* kin = (flips & 1) ? keys_alt : keys;
        K* kout = (flips & 1) ? keys : keys_alt;
        int32_t* vin = (flips & 1) ? vals_alt : vals;
        int32_t* vout = (flips & 1) ? vals : vals_alt;
        k_radix_upsweep<K><<<nb, kSortThreads, 0, s>>>(kin, n, shift, counts, nb);
        exclusive_scan<uint32_t>(counts, counts, nc, scan_scratch, nullptr, s, launches);
        k_radix_downsweep<K><<<nb, kSortThreads, 0, s>>>(kin, vin, kout, vout, n, shift, counts, nb);
        if (launches) *launches += 2;
        ++flips;
    }
    return flips & 1;  // 1: result is in the alternate buffers
}
template int radix_sort_pairs<uint32_t>(uint32_t*, int32_t*, uint32_t*, int32_t*, int64_t, int, uint32_t*, uint32_t*,
                                        cudaStream_t, int*);
template int radix_sort_pairs<unsigned long long>(unsigned long long*, int32_t*, unsigned long long*, int32_t*, int64_t, int,
                                                  uint32_t*, uint32_t*, cudaStream_t, int*);

}  // namespace hpd
