// Shared device/host helpers for the GB300 truss-decomposition library.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>

#include "../../include/tdt_gb300.h"

namespace tdt {

constexpr int kWarp = 32;
constexpr unsigned kFull = 0xffffffffu;

// Per-thread last error detail for tdt_last_error().
void set_error(const char* fmt, ...);
int cuda_status(cudaError_t e, const char* what);

#define TDT_CHECK_ARG(cond, ...)                      \
    do {                                              \
        if (!(cond)) {                                \
            ::tdt::set_error(__VA_ARGS__);            \
            return TDT_ERR_INVALID;                   \
        }                                             \
    } while (0)

#define TDT_CUDA(call)                                                   \
    do {                                                                 \
        cudaError_t e__ = (call);                                        \
        if (e__ != cudaSuccess) return ::tdt::cuda_status(e__, #call);   \
    } while (0)

// Every kernel launch of the library is followed by TDT_LAUNCH_CHECK, which
// also counts it (tdt_launch_count()).
void note_launch();
#define TDT_LAUNCH_CHECK(what)            \
    do {                                  \
        ::tdt::note_launch();             \
        TDT_CUDA(cudaPeekAtLastError());  \
    } while (0)

// Number of SMs and resident-block limits of the current device (cached per device).
struct DeviceInfo {
    int device;
    int sms;
    int max_smem_optin;
    int cc_major, cc_minor;
};
int device_info(DeviceInfo* out);

// Grid-stride launch size: a multiple of the SM count.
inline unsigned grid_for(int64_t work_items, int block, int sms, int per_sm = 8) {
    int64_t want = (work_items + block - 1) / block;
    int64_t cap = (int64_t)sms * per_sm;
    if (want < 1) want = 1;
    return (unsigned)(want < cap ? want : cap);
}

// ------------------------------------------------------------------ device
__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }
__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}
__device__ __forceinline__ uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ int ld_volatile_i32(const int* p) {
    return *(const volatile int*)p;
}

template <class T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
    return v;
}
template <class T>
__device__ __forceinline__ T warp_min(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        T w = __shfl_xor_sync(kFull, v, o);
        v = w < v ? w : v;
    }
    return v;
}
// Inclusive warp scan.
template <class T>
__device__ __forceinline__ T warp_incl_scan(T v) {
    unsigned lane = lane_id();
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T w = __shfl_up_sync(kFull, v, o);
        if (lane >= (unsigned)o) v += w;
    }
    return v;
}

// Lower-bound search of `key` in the sorted range cols[lo, hi); returns the
// position of key or -1.
template <class Off>
__device__ __forceinline__ Off find_sorted(const int32_t* __restrict__ cols, Off lo, Off hi,
                                           int32_t key) {
    Off end = hi;
    while (lo < hi) {
        Off mid = lo + ((hi - lo) >> 1);
        if (__ldg(cols + mid) < key)
            lo = mid + 1;
        else
            hi = mid;
    }
    return (lo < end && __ldg(cols + lo) == key) ? lo : (Off)-1;
}

// ------------------------------------------------------------------ grid barrier
// Control block shared by the persistent kernels (device memory, zeroed by the
// host before a launch).  One 64-bit arrival counter that only grows: barrier
// k of a launch is complete when it reaches k x nblocks, so the last block to
// arrive releases the others with its own increment (no reset, no second
// word to publish).  Bit 63 of the same word aborts the run: a waiter sees it
// in the value it polls and an arriving block in the value its increment
// returns, with no extra load on the barrier's path.
struct GridCtl {
    unsigned long long arrive;
    unsigned pad0[62];
    int pad1;
    int status;
    unsigned pad2[30];
};
static_assert(sizeof(GridCtl) == 384, "control block layout");

constexpr unsigned long long kGridAbortBit = 1ull << 63;

__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

// Makes every block leave at its next grid barrier (and any block waiting at
// one now).
__device__ __forceinline__ void grid_abort(GridCtl* ctl) { atomicOr(&ctl->arrive, kGridAbortBit); }

// Wait limit of one grid barrier.  A barrier that does not complete within it
// sets GridCtl::status = TDT_ERR_TIMEOUT and every block leaves its loop.
constexpr uint64_t kBarrierTimeoutNs = 20ull * 1000ull * 1000ull * 1000ull;

// Barrier over all blocks of a cooperative launch.  Returns false when the
// run is being aborted (timeout or an error elsewhere).
__device__ __forceinline__ bool grid_barrier(GridCtl* ctl, unsigned nblocks,
                                             uint64_t limit_ns = kBarrierTimeoutNs) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        __threadfence();  // the block's writes before its arrival
        const unsigned long long old = atomicAdd(&ctl->arrive, 1ull);
        if (old & kGridAbortBit) {
            ok = 0;
        } else {
            const unsigned long long target = (old / nblocks + 1) * nblocks;
            if (old + 1 != target) {
                // one load per spin; the clock every 32 spins, and a short
                // sleep once the wait is long
                const uint64_t t0 = globaltimer_ns();
                unsigned spins = 0;
                for (;;) {
                    const unsigned long long v = ld_acquire_u64(&ctl->arrive);
                    if (v & kGridAbortBit) {
                        ok = 0;
                        break;
                    }
                    if (v >= target) break;
                    if ((++spins & 31u) == 0) {
                        if (globaltimer_ns() - t0 > limit_ns) {
                            atomicMax(&ctl->status, (int)TDT_ERR_TIMEOUT);
                            grid_abort(ctl);
                            ok = 0;
                            break;
                        }
                        if (spins > 4096) __nanosleep(200);
                    }
                }
            }
        }
        __threadfence();  // the other blocks' writes before this block's next reads
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

}  // namespace tdt
