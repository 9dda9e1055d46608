// Seeded synthetic graph generators (edge lists, before preprocessing).
//
// All draws come from a counter-based stream: draw j of seed s is
// splitmix64(splitmix64(s) + j), so the host (numpy) and device versions of a
// generator produce the same edges.
#include <stdint.h>
#include <string.h>

#include <vector>

#include "common.cuh"

namespace tdt {

__host__ __device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

// R-MAT: draw i picks `scale` quadrants; quadrant draw b uses stream index
// i*scale + b and compares its top 53 bits with thresholds
// ta = floor(a*2^53), tab = floor((a+b)*2^53), tabc = floor((a+b+c)*2^53).
__global__ void rmat_kernel(int scale, int64_t m, uint64_t key, uint64_t ta, uint64_t tab, uint64_t tabc,
                            int32_t* __restrict__ src, int32_t* __restrict__ dst) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        uint32_t s = 0, d = 0;
        for (int b = 0; b < scale; b++) {
            const uint64_t r = splitmix64(key + (uint64_t)i * (uint64_t)scale + (uint64_t)b) >> 11;
            const uint32_t bs = r >= tab;                       // quadrants c, d: source bit 1
            const uint32_t bd = (r >= ta && r < tab) || r >= tabc;  // quadrants b, d: target bit 1
            s = (s << 1) | bs;
            d = (d << 1) | bd;
        }
        src[i] = (int32_t)s;
        dst[i] = (int32_t)d;
    }
}

// Chung-Lu: draw i takes stream values 2i and 2i+1 modulo the total integer
// weight and maps each to the first vertex whose cumulative weight exceeds it
// (cum: inclusive prefix sums of the per-vertex integer weights, n entries).
__global__ void chung_lu_kernel(int64_t n, int64_t m, uint64_t key, const uint64_t* __restrict__ cum,
                                uint64_t total, int32_t* __restrict__ src, int32_t* __restrict__ dst) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        int32_t out[2];
        for (int k = 0; k < 2; k++) {
            const uint64_t r = splitmix64(key + 2ull * (uint64_t)i + (uint64_t)k) % total;
            int64_t lo = 0, hi = n;  // first index with cum > r
            while (lo < hi) {
                const int64_t mid = (lo + hi) >> 1;
                if (__ldg(cum + mid) > r) hi = mid; else lo = mid + 1;
            }
            out[k] = (int32_t)(lo < n ? lo : n - 1);
        }
        src[i] = out[0];
        dst[i] = out[1];
    }
}

}  // namespace tdt

using namespace tdt;
#define API extern "C" __attribute__((visibility("default")))

API uint64_t tdt_splitmix64(uint64_t x) { return splitmix64(x); }

// R-MAT edge list on the device (src/dst int32[m]).
API int tdt_gen_rmat(int32_t scale, int64_t m, uint64_t seed, uint64_t ta, uint64_t tab, uint64_t tabc,
                     int32_t* src, int32_t* dst, tdt_stream_t stream) {
    TDT_CHECK_ARG(scale >= 1 && scale <= 31, "scale %d out of range", scale);
    TDT_CHECK_ARG(m >= 0, "negative edge count");
    if (m == 0) return TDT_OK;
    TDT_CHECK_ARG(src && dst, "null pointer");
    DeviceInfo di;
    int rc = device_info(&di);
    if (rc) return rc;
    rmat_kernel<<<grid_for(m, 256, di.sms, 16), 256, 0, (cudaStream_t)stream>>>(scale, m, splitmix64(seed), ta, tab,
                                                                             tabc, src, dst);
    TDT_LAUNCH_CHECK("rmat");
    return TDT_OK;
}

// Chung-Lu edge list on the device (src/dst int32[m]) from the cumulative
// integer weights cum (device, uint64[n], strictly positive weights).
API int tdt_gen_chung_lu(int64_t n, int64_t m, uint64_t seed, const uint64_t* cum, uint64_t total, int32_t* src,
                         int32_t* dst, tdt_stream_t stream) {
    TDT_CHECK_ARG(n >= 1 && n <= (int64_t)INT32_MAX, "n %lld out of range", (long long)n);
    TDT_CHECK_ARG(m >= 0, "negative edge count");
    TDT_CHECK_ARG(total >= 1, "total weight must be positive");
    if (m == 0) return TDT_OK;
    TDT_CHECK_ARG(src && dst && cum, "null pointer");
    DeviceInfo di;
    int rc = device_info(&di);
    if (rc) return rc;
    chung_lu_kernel<<<grid_for(m, 256, di.sms, 16), 256, 0, (cudaStream_t)stream>>>(n, m, splitmix64(seed), cum,
                                                                                 total, src, dst);
    TDT_LAUNCH_CHECK("chung_lu");
    return TDT_OK;
}

// Barabasi-Albert preferential attachment (host).  Start: a star on m+1
// vertices (centre 0); each new vertex t = m+1 .. n-1 attaches to m distinct
// existing vertices drawn uniformly from the list of edge endpoints so far
// (probability proportional to degree), redrawing duplicates.  Writes
// (m + (n-m-1)*m) edges into src/dst (capacity `cap`); returns the count, or
// -1 when cap is too small or the arguments are invalid.
API int64_t tdt_gen_ba(int64_t n, int32_t m, uint64_t seed, int32_t* src, int32_t* dst, int64_t cap) {
    if (m < 1 || n < (int64_t)m + 1 || !src || !dst) return -1;
    const int64_t total = (int64_t)m + (n - m - 1) * (int64_t)m;
    if (cap < total) return -1;
    std::vector<int32_t> rep;
    rep.reserve((size_t)(2 * total));
    int64_t k = 0;
    for (int32_t v = 1; v <= m; v++) {
        src[k] = 0;
        dst[k] = v;
        k++;
        rep.push_back(0);
        rep.push_back(v);
    }
    const uint64_t key = splitmix64(seed);
    uint64_t ctr = 0;
    std::vector<int32_t> targets((size_t)m);
    for (int64_t t = m + 1; t < n; t++) {
        int got = 0;
        while (got < m) {
            const uint64_t r = splitmix64(key + ctr++);
            const int32_t c = rep[(size_t)(r % (uint64_t)rep.size())];
            bool dup = false;
            for (int j = 0; j < got; j++) dup |= targets[(size_t)j] == c;
            if (!dup) targets[(size_t)got++] = c;
        }
        for (int j = 0; j < m; j++) {
            src[k] = (int32_t)t;
            dst[k] = targets[(size_t)j];
            k++;
            rep.push_back(targets[(size_t)j]);
            rep.push_back((int32_t)t);
        }
    }
    return k;
}
