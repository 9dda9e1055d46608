// Per-edge support (triangle count per edge) over the degree-oriented CSR.
//
// Replaces checkElementsTwoPtr / checkElementsTwoPtrTile (kernel.cu:28-141),
// which give every edge (u,v) one thread that merges N+(u) and N+(v) and adds
// +1 to (u,w), +1 to (v,w) and +count to (u,v) for every common w.
//
// Here the unit of work is the source vertex u of the triangle u<v<w:
//   * N+(u) is staged once in shared memory (warp slice for d+(u) <= kWarpCap,
//     the whole block's buffer for larger rows; rows beyond the block buffer
//     are searched in place);
//   * the warp walks the flattened list of all (v, w) with v in N+(u) and
//     w in N+(v), 32 consecutive entries per step (coalesced loads of N+(v)),
//     and looks each w up in N+(u) by binary search (restricted to the
//     entries after v when the orientation is by vertex id);
//   * hits on the edges (u,v) and (u,w) go to shared-memory counters that are
//     flushed once per row; only the (v,w) hit is a global atomic.
// The counts are exactly the reference's (each triangle is found once, from
// its (source, middle) edge), so the output is bit-identical for any n_cut.
#include "common.cuh"

namespace tdt {

constexpr int kSupBlock = 512;                 // 16 warps
constexpr int kSupWarps = kSupBlock / kWarp;
constexpr int kWarpCap = 256;                  // light rows: d+(u) <= kWarpCap
constexpr int kVertexBatch = 8;                // vertices per dynamic grab
// dynamic shared memory of the support kernel
constexpr int kSupSmemBytes = 96 * 1024;
constexpr int kHeavyCap = (kSupSmemBytes - 1024) / 8;  // entries of N+(u) kept in smem

// Row ranges are clamped to [0, ne] so a malformed row_ptr cannot move an
// access outside cols/out.
template <class Off>
struct OutRows {
    const Off* rp;
    int32_t stride;  // row_ptr entries per vertex (n_cut)
    const int32_t* cols;
    int64_t nv;      // vertices
    int64_t ne;      // edges
    __device__ __forceinline__ Off clamp(Off x) const { return x < 0 ? Off(0) : (x > (Off)ne ? (Off)ne : x); }
    __device__ __forceinline__ Off begin(int64_t v) const { return clamp(__ldg(rp + v * stride)); }
    __device__ __forceinline__ Off end(int64_t v) const {
        Off b = begin(v), e = clamp(__ldg(rp + v * stride + stride));
        return e < b ? b : e;
    }
};

struct SupCtl {
    unsigned long long heavy_next;
    unsigned long long light_next;
};

// Binary search of key in s[lo, hi) (shared or global, generic address).
__device__ __forceinline__ int bsearch_i32(const int32_t* s, int lo, int hi, int32_t key) {
    int end = hi;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (s[mid] < key) lo = mid + 1; else hi = mid;
    }
    return (lo < end && s[lo] == key) ? lo : -1;
}

// One warp processes the v-batches vb = first, first+step, ... of row u.
// su: N+(u) (d entries), cnt: per-position counters for the edges (u, su[i]).
// kIdOrdered: every edge goes from a lower to a higher vertex id (the
// reference's rank orientation), so w lies after v in N+(u) and the last v has
// no partner; without it (any acyclic orientation) all of N+(u) is searched.
template <bool kIdOrdered, class Off>
__device__ __forceinline__ void wedge_walk(const OutRows<Off>& G, int32_t* __restrict__ out,
                                           const int32_t* su, int32_t* cnt, int d, int first,
                                           int step, int32_t* s_excl, Off* s_bv) {
    const unsigned lane = lane_id();
    const int32_t umax = su[d - 1];
    const int vend = kIdOrdered ? d - 1 : d;
    for (int vb = first; vb < vend; vb += step) {
        const int i = vb + (int)lane;
        int32_t len = 0;
        Off bv = 0;
        if (i < vend) {
            int32_t v = su[i];
            if (v >= 0 && v < G.nv) {
                bv = G.begin(v);
                len = (int32_t)(G.end(v) - bv);
            }
        }
        int32_t incl = warp_incl_scan(len);
        int32_t total = __shfl_sync(kFull, incl, 31);
        s_excl[lane] = incl - len;
        s_bv[lane] = bv;
        __syncwarp();
        for (int32_t t = lane; t < total; t += kWarp) {
            // owner lane o: last o with s_excl[o] <= t
            int lo = 0, hi = 31;
            while (lo < hi) {
                int mid = (lo + hi + 1) >> 1;
                if (s_excl[mid] <= t) lo = mid; else hi = mid - 1;
            }
            const int o = lo;
            const Off pos = s_bv[o] + (t - s_excl[o]);
            const int32_t w = __ldg(G.cols + pos);
            if (w > umax) continue;
            const int p = bsearch_i32(su, kIdOrdered ? vb + o + 1 : 0, d, w);
            if (p >= 0) {
                atomicAdd(cnt + p, 1);
                atomicAdd(cnt + vb + o, 1);
                atomicAdd(out + pos, 1);
            }
        }
        __syncwarp();
    }
}

constexpr int kHeavyChunk = 256;  // vertices scanned per phase-1 grab

// ctl != nullptr: dynamic scheduling through its counters (zeroed by the
// caller); ctl == nullptr: static round-robin scheduling (no scratch at all).
template <bool kIdOrdered, class Off>
__global__ void __launch_bounds__(kSupBlock) support_kernel(OutRows<Off> G, int64_t nv,
                                                            int32_t* __restrict__ out, SupCtl* ctl,
                                                            const int* gate) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int32_t s_excl[kSupWarps][kWarp];
    __shared__ Off s_bv[kSupWarps][kWarp];
    __shared__ int32_t s_list[kHeavyChunk];
    __shared__ int s_n;
    __shared__ long long s_chunk;
    const int wib = threadIdx.x / kWarp;
    const unsigned lane = lane_id();
    const long long nchunks = (nv + kHeavyChunk - 1) / kHeavyChunk;
    if (gate && *(volatile const int*)gate != 0) return;  // input rejected by validation

    // ---- phase 1: rows with d+(u) > kWarpCap, one block per row
    for (long long it = 0;; it++) {
        if (threadIdx.x == 0) {
            s_chunk = ctl ? (long long)atomicAdd(&ctl->heavy_next, 1ull) : blockIdx.x + it * gridDim.x;
            s_n = 0;
        }
        __syncthreads();
        const long long c = s_chunk;
        if (c >= nchunks) break;
        for (int k = threadIdx.x; k < kHeavyChunk; k += kSupBlock) {
            const long long u = c * kHeavyChunk + k;
            if (u < nv && G.end(u) - G.begin(u) > kWarpCap) s_list[atomicAdd(&s_n, 1)] = (int32_t)u;
        }
        __syncthreads();
        const int nh = s_n;
        for (int h = 0; h < nh; h++) {
            const long long u = s_list[h];
            const Off bu = G.begin(u);
            const int d = (int)(G.end(u) - bu);
            const bool in_smem = d <= kHeavyCap;
            int32_t* su_s = reinterpret_cast<int32_t*>(smem);
            int32_t* cnt_s = su_s + kHeavyCap;
            const int32_t* su = in_smem ? su_s : (G.cols + bu);
            int32_t* cnt = in_smem ? cnt_s : (out + bu);
            if (in_smem) {
                for (int i = threadIdx.x; i < d; i += kSupBlock) {
                    su_s[i] = __ldg(G.cols + bu + i);
                    cnt_s[i] = 0;
                }
            }
            __syncthreads();
            wedge_walk<kIdOrdered>(G, out, su, cnt, d, wib * kWarp, kSupBlock, s_excl[wib], s_bv[wib]);
            __syncthreads();
            if (in_smem) {
                for (int i = threadIdx.x; i < d; i += kSupBlock)
                    if (cnt_s[i]) atomicAdd(out + bu + i, cnt_s[i]);
            }
            __syncthreads();
        }
    }

    // ---- phase 2: rows with 2 <= d+(u) <= kWarpCap, one warp per row, taken
    // in batches from the top ids (highest degree rank) down
    int32_t* su = reinterpret_cast<int32_t*>(smem) + wib * (2 * kWarpCap);
    int32_t* cnt = su + kWarpCap;
    const long long gw = (long long)blockIdx.x * kSupWarps + wib;
    const long long nw = (long long)gridDim.x * kSupWarps;
    for (long long it = 0;; it++) {
        unsigned long long b = 0;
        if (ctl) {
            if (lane == 0) b = atomicAdd(&ctl->light_next, (unsigned long long)kVertexBatch);
            b = __shfl_sync(kFull, b, 0);
        } else {
            b = (unsigned long long)((gw + it * nw) * kVertexBatch);
        }
        if ((long long)b >= nv) break;
        for (int q = 0; q < kVertexBatch; q++) {
            const long long uu = nv - 1 - ((long long)b + q);
            if (uu < 0) break;
            const Off bu = G.begin(uu);
            const int d = (int)(G.end(uu) - bu);
            if (d < 2 || d > kWarpCap) continue;
            for (int i = lane; i < d; i += kWarp) {
                su[i] = __ldg(G.cols + bu + i);
                cnt[i] = 0;
            }
            __syncwarp();
            wedge_walk<kIdOrdered>(G, out, su, cnt, d, 0, kWarp, s_excl[wib], s_bv[wib]);
            for (int i = lane; i < d; i += kWarp)
                if (cnt[i]) atomicAdd(out + bu + i, cnt[i]);
            __syncwarp();
        }
    }
}

// Launches the support pass (accumulates into out).  ctl_ws: 256 bytes of
// device scratch for dynamic scheduling, or null for the scratch-free static
// schedule.
template <bool kIdOrdered, class Off>
int launch_support(const Off* rp, int32_t stride, const int32_t* cols, int64_t nv, int64_t ne, int32_t* out,
                   void* ctl_ws, const int* gate, cudaStream_t st) {
    if (nv <= 0) return TDT_OK;
    DeviceInfo di;
    int rc = device_info(&di);
    if (rc) return rc;
    // set on every call: cheap, and valid for whichever device is current
    TDT_CUDA(cudaFuncSetAttribute(support_kernel<kIdOrdered, Off>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, kSupSmemBytes));
    SupCtl* ctl = reinterpret_cast<SupCtl*>(ctl_ws);
    if (ctl) TDT_CUDA(cudaMemsetAsync(ctl, 0, sizeof(SupCtl), st));
    OutRows<Off> G{rp, stride, cols, nv, ne};
    int blocks_per_sm = 0;
    TDT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, support_kernel<kIdOrdered, Off>,
                                                           kSupBlock, kSupSmemBytes));
    if (blocks_per_sm < 1) blocks_per_sm = 1;
    support_kernel<kIdOrdered, Off><<<di.sms * blocks_per_sm, kSupBlock, kSupSmemBytes, st>>>(G, nv, out, ctl,
                                                                                          gate);
    TDT_LAUNCH_CHECK("support");
    return TDT_OK;
}

size_t support_ctl_bytes() { return 256; }

// Whole-path support pass: int64 row offsets, id-ordered orientation.
int launch_support_i64(const int64_t* rp, const int32_t* cols, int64_t nv, int64_t ne, int32_t* out, void* ctl,
                       const int* gate, cudaStream_t st) {
    return launch_support<true, int64_t>(rp, 1, cols, nv, ne, out, ctl, gate, st);
}

template int launch_support<false, int32_t>(const int32_t*, int32_t, const int32_t*, int64_t, int64_t,
                                            int32_t*, void*, const int*, cudaStream_t);
template int launch_support<true, int64_t>(const int64_t*, int32_t, const int32_t*, int64_t, int64_t, int32_t*,
                                           void*, const int*, cudaStream_t);

}  // namespace tdt
