// Device-wide exclusive scan and stable LSD radix sort (8-bit digits).
//
// Scan: reduce -> scan of block totals -> scan with offsets (three launches).
// Radix sort pass: (1) per-tile digit histogram, (2) exclusive scan of the
// digit-major histogram table, (3) per-tile stable ranking with
// __match_any_sync (warp multisplit), staging in shared memory and coalesced
// scatter.  Keys are stable across passes, so sorting (key, value) pairs
// whose values arrive in ascending order gives ascending values per key.
#include "common.cuh"
#include "sort.cuh"

namespace tdt {

constexpr int kScanBlock = 512;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanBlock * kScanItems;

template <class T>
__device__ __forceinline__ T block_excl_scan(T v, T* s_warp, T* total) {
    const unsigned lane = lane_id();
    const int w = threadIdx.x / kWarp;
    T incl = warp_incl_scan(v);
    if (lane == 31) s_warp[w] = incl;
    __syncthreads();
    if (w == 0) {
        T x = (lane < blockDim.x / kWarp) ? s_warp[lane] : T(0);
        T xi = warp_incl_scan(x);
        if (lane < blockDim.x / kWarp) s_warp[lane] = xi - x;
        if (lane == 31) s_warp[32] = xi;
    }
    __syncthreads();
    T res = s_warp[w] + incl - v;
    if (total) *total = s_warp[32];
    __syncthreads();
    return res;
}

template <class TI, class TO>
__global__ void __launch_bounds__(kScanBlock) scan_reduce_kernel(const TI* __restrict__ in, int64_t n,
                                                                 TO* __restrict__ partial) {
    __shared__ TO s_warp[33];
    int64_t base = (int64_t)blockIdx.x * kScanTile;
    TO sum = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        int64_t i = base + (int64_t)k * kScanBlock + threadIdx.x;
        if (i < n) sum += (TO)in[i];
    }
    TO tot;
    block_excl_scan<TO>(sum, s_warp, &tot);
    if (threadIdx.x == 0) partial[blockIdx.x] = tot;
}

template <class TO>
__global__ void __launch_bounds__(kScanBlock) scan_partials_kernel(TO* partial, int64_t nb) {
    __shared__ TO s_warp[33];
    TO carry = 0;
    for (int64_t b0 = 0; b0 < nb; b0 += kScanBlock) {
        int64_t i = b0 + threadIdx.x;
        TO v = i < nb ? partial[i] : TO(0);
        TO tot;
        TO ex = block_excl_scan<TO>(v, s_warp, &tot);
        if (i < nb) partial[i] = carry + ex;
        carry += tot;
    }
}

template <class TI, class TO>
__global__ void __launch_bounds__(kScanBlock) scan_final_kernel(const TI* __restrict__ in, int64_t n,
                                                                const TO* __restrict__ partial,
                                                                TO* __restrict__ out, TO* total_out) {
    __shared__ TO s_warp[33];
    const int64_t base = (int64_t)blockIdx.x * kScanTile;
    // blocked arrangement: thread t owns items base + t*kScanItems ...
    TO v[kScanItems];
    TO sum = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        int64_t i = base + (int64_t)threadIdx.x * kScanItems + k;
        v[k] = i < n ? (TO)in[i] : TO(0);
        sum += v[k];
    }
    TO tot;
    TO run = partial[blockIdx.x] + block_excl_scan<TO>(sum, s_warp, &tot);
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        int64_t i = base + (int64_t)threadIdx.x * kScanItems + k;
        if (i < n) out[i] = run;
        run += v[k];
    }
    if (total_out && blockIdx.x == gridDim.x - 1 && threadIdx.x == kScanBlock - 1) *total_out = run;
}

size_t scan_scratch_bytes(int64_t n) {
    int64_t nb = (n + kScanTile - 1) / kScanTile;
    return (size_t)(nb + 1) * 8 + 256;
}

// out[i] = sum(in[0..i)), and *total_out (device, may be null) = sum(in).
// `in` and `out` may alias.
template <class TI, class TO>
int exclusive_scan(const TI* in, TO* out, int64_t n, TO* total_out, void* scratch, cudaStream_t st) {
    if (n <= 0) {
        if (total_out) TDT_CUDA(cudaMemsetAsync(total_out, 0, sizeof(TO), st));
        return TDT_OK;
    }
    int64_t nb = (n + kScanTile - 1) / kScanTile;
    TO* partial = reinterpret_cast<TO*>(scratch);
    scan_reduce_kernel<TI, TO><<<(unsigned)nb, kScanBlock, 0, st>>>(in, n, partial);
    TDT_LAUNCH_CHECK("scan_reduce");
    scan_partials_kernel<TO><<<1, kScanBlock, 0, st>>>(partial, nb);
    TDT_LAUNCH_CHECK("scan_partials");
    scan_final_kernel<TI, TO><<<(unsigned)nb, kScanBlock, 0, st>>>(in, n, partial, out, total_out);
    TDT_LAUNCH_CHECK("scan_final");
    return TDT_OK;
}

template int exclusive_scan<int32_t, int64_t>(const int32_t*, int64_t*, int64_t, int64_t*, void*, cudaStream_t);
template int exclusive_scan<int64_t, int64_t>(const int64_t*, int64_t*, int64_t, int64_t*, void*, cudaStream_t);
template int exclusive_scan<uint32_t, uint32_t>(const uint32_t*, uint32_t*, int64_t, uint32_t*, void*,
                                                cudaStream_t);
template int exclusive_scan<int32_t, int32_t>(const int32_t*, int32_t*, int64_t, int32_t*, void*, cudaStream_t);

// ------------------------------------------------------------------ radix sort
constexpr int kSortBlock = 256;
constexpr int kSortWarps = kSortBlock / kWarp;
constexpr int kRadix = 256;
// keys per thread: the staging tile (keys + values) stays within 48 KB static smem
template <class K>
struct SortCfg {
    static constexpr int items = sizeof(K) == 8 ? 8 : 16;
    static constexpr int tile = kSortBlock * items;  // 2048 (64-bit) or 4096 (32-bit) keys
};

template <class K>
__global__ void __launch_bounds__(kSortBlock) radix_hist_kernel(const K* __restrict__ keys, int64_t n,
                                                                int shift, uint32_t* __restrict__ hist,
                                                                int64_t ntiles) {
    __shared__ uint32_t s_h[kRadix];
    for (int i = threadIdx.x; i < kRadix; i += kSortBlock) s_h[i] = 0;
    __syncthreads();
    constexpr int kSortItems = SortCfg<K>::items;
    const int64_t base = (int64_t)blockIdx.x * SortCfg<K>::tile;
#pragma unroll 4
    for (int k = 0; k < kSortItems; k++) {
        int64_t i = base + (int64_t)k * kSortBlock + threadIdx.x;
        if (i < n) atomicAdd(&s_h[(unsigned)((keys[i] >> shift) & 0xff)], 1u);
    }
    __syncthreads();
    for (int d = threadIdx.x; d < kRadix; d += kSortBlock) hist[(int64_t)d * ntiles + blockIdx.x] = s_h[d];
}

template <class K, bool kHasVals>
__global__ void __launch_bounds__(kSortBlock) radix_scatter_kernel(
    const K* __restrict__ keys_in, const uint32_t* __restrict__ vals_in, K* __restrict__ keys_out,
    uint32_t* __restrict__ vals_out, int64_t n, int shift, const uint32_t* __restrict__ hist_scan,
    int64_t ntiles) {
    constexpr int kSortItems = SortCfg<K>::items;
    constexpr int kSortTile = SortCfg<K>::tile;
    __shared__ uint32_t s_wcnt[kSortWarps][kRadix];
    __shared__ uint32_t s_tile_start[kRadix];
    __shared__ uint32_t s_warp_tmp[33];
    __shared__ K s_keys[kSortTile];
    __shared__ uint32_t s_vals[kHasVals ? kSortTile : 1];
    const int w = threadIdx.x / kWarp;
    const unsigned lane = lane_id();
    for (int i = lane; i < kRadix; i += kWarp) s_wcnt[w][i] = 0;
    __syncwarp();
    const int64_t base = (int64_t)blockIdx.x * kSortTile;
    // warp w owns the contiguous sub-tile [w*kSortItems*32, (w+1)*kSortItems*32)
    K key[kSortItems];
    uint32_t val[kSortItems];
    uint32_t rank[kSortItems];
#pragma unroll
    for (int it = 0; it < kSortItems; it++) {
        const int64_t i = base + (int64_t)w * (kSortItems * kWarp) + it * kWarp + lane;
        const bool ok = i < n;
        key[it] = ok ? keys_in[i] : K(0);
        if (kHasVals) val[it] = ok ? vals_in[i] : 0u;
        const unsigned d = ok ? (unsigned)((key[it] >> shift) & 0xff) : (unsigned)kRadix;
        const unsigned peers = __match_any_sync(kFull, d);
        const unsigned leader = __ffs(peers) - 1;
        uint32_t pre = 0;
        if (ok) pre = s_wcnt[w][d];
        __syncwarp();
        if (ok && lane == leader) s_wcnt[w][d] = pre + __popc(peers);
        __syncwarp();
        rank[it] = ok ? pre + __popc(peers & lanemask_lt()) : 0xffffffffu;
    }
    __syncthreads();
    // per digit: exclusive offsets across warps, then across digits
    uint32_t tile_cnt = 0;
    if (threadIdx.x < kRadix) {
        const int d = threadIdx.x;
        uint32_t run = 0;
#pragma unroll
        for (int ww = 0; ww < kSortWarps; ww++) {
            uint32_t c = s_wcnt[ww][d];
            s_wcnt[ww][d] = run;
            run += c;
        }
        tile_cnt = run;
    }
    uint32_t tot;
    uint32_t start = block_excl_scan<uint32_t>(tile_cnt, s_warp_tmp, &tot);
    if (threadIdx.x < kRadix) s_tile_start[threadIdx.x] = start;
    __syncthreads();
#pragma unroll
    for (int it = 0; it < kSortItems; it++) {
        if (rank[it] != 0xffffffffu) {
            const unsigned d = (unsigned)((key[it] >> shift) & 0xff);
            const uint32_t p = s_tile_start[d] + s_wcnt[w][d] + rank[it];
            s_keys[p] = key[it];
            if (kHasVals) s_vals[p] = val[it];
        }
    }
    __syncthreads();
    const int64_t tile_n = min((int64_t)kSortTile, n - base);
    for (int i = threadIdx.x; i < tile_n; i += kSortBlock) {
        const K k = s_keys[i];
        const unsigned d = (unsigned)((k >> shift) & 0xff);
        const int64_t g = (int64_t)hist_scan[(int64_t)d * ntiles + blockIdx.x] + (i - s_tile_start[d]);
        keys_out[g] = k;
        if (kHasVals) vals_out[g] = s_vals[i];
    }
}

size_t radix_sort_scratch_bytes(int64_t n) {
    int64_t ntiles = (n + SortCfg<uint32_t>::tile - 1) / SortCfg<uint32_t>::tile;
    int64_t ntiles64 = (n + SortCfg<uint64_t>::tile - 1) / SortCfg<uint64_t>::tile;
    if (ntiles64 > ntiles) ntiles = ntiles64;
    int64_t hn = ntiles * kRadix;
    return (size_t)hn * 4 + scan_scratch_bytes(hn) + 512;
}

// Stable sort of (keys, vals) by key bits [begin_bit, end_bit).  Ping-pongs
// between (keys, vals) and (keys_alt, vals_alt); the result ends in the pair
// returned through *result_in_alt.  vals may be null (keys only).
template <class K>
int radix_sort_pairs(K* keys, uint32_t* vals, K* keys_alt, uint32_t* vals_alt, int64_t n,
                     int begin_bit, int end_bit, void* scratch, bool* result_in_alt, cudaStream_t st) {
    *result_in_alt = false;
    if (n <= 1) return TDT_OK;
    TDT_CHECK_ARG(n < (int64_t)UINT32_MAX, "radix sort of %lld keys exceeds 32-bit ranks", (long long)n);
    const int64_t ntiles = (n + SortCfg<K>::tile - 1) / SortCfg<K>::tile;
    const int64_t hn = ntiles * kRadix;
    uint32_t* hist = reinterpret_cast<uint32_t*>(scratch);
    void* scan_ws = reinterpret_cast<char*>(scratch) + ((hn * 4 + 255) / 256) * 256;
    K* src_k = keys;
    uint32_t* src_v = vals;
    K* dst_k = keys_alt;
    uint32_t* dst_v = vals_alt;
    bool alt = false;
    for (int shift = begin_bit; shift < end_bit; shift += 8) {
        radix_hist_kernel<K><<<(unsigned)ntiles, kSortBlock, 0, st>>>(src_k, n, shift, hist, ntiles);
        TDT_LAUNCH_CHECK("radix_hist");
        int rc = exclusive_scan<uint32_t, uint32_t>(hist, hist, hn, nullptr, scan_ws, st);
        if (rc) return rc;
        if (vals)
            radix_scatter_kernel<K, true><<<(unsigned)ntiles, kSortBlock, 0, st>>>(
                src_k, src_v, dst_k, dst_v, n, shift, hist, ntiles);
        else
            radix_scatter_kernel<K, false><<<(unsigned)ntiles, kSortBlock, 0, st>>>(
                src_k, nullptr, dst_k, nullptr, n, shift, hist, ntiles);
        TDT_LAUNCH_CHECK("radix_scatter");
        K* tk = src_k; src_k = dst_k; dst_k = tk;
        uint32_t* tv = src_v; src_v = dst_v; dst_v = tv;
        alt = !alt;
    }
    *result_in_alt = alt;
    return TDT_OK;
}

template int radix_sort_pairs<uint32_t>(uint32_t*, uint32_t*, uint32_t*, uint32_t*, int64_t, int, int, void*,
                                        bool*, cudaStream_t);
template int radix_sort_pairs<uint64_t>(uint64_t*, uint32_t*, uint64_t*, uint32_t*, int64_t, int, int, void*,
                                        bool*, cudaStream_t);

}  // namespace tdt
