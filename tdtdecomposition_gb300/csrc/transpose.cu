// Role-C entries of the per-edge triangle lists, by transposing role-A lists.
//
// The listing pass writes every triangle's role-A entry (in the list of its
// (source, middle) edge) and role-B entry (in the list of its (source, sink)
// edge); both edges belong to the source row, so those writes stay inside one
// row's list region.  The role-C entry belongs to the (middle, sink) edge of
// another row; written from the source row it would be a random 8-byte store
// per triangle (a DRAM read-modify-write of a 32-byte sector each).
//
// Here each middle vertex v collects its own role-C entries: for every
// in-edge (u, v) (from the in-adjacency), the role-A list of (u, v) holds
// (eB = (u,w), eC = (v,w)) for each triangle (u, v, w), and the role-C entry of
// eC is (e_uv, eB).  All of v's stores land in v's list region; the slot
// counters live in shared memory.  The in-edges' lists are one flat index
// space walked 32 entries per step (the same owner reduction as the support
// pass).  Every store is bounds-checked against the role-C count of its edge,
// and every counter must end at that count (else TDT_ERR_CAPACITY).
//
// Work units: rows with at most 32 in-edges and d+(v) <= kTrLightCap get one
// warp; other rows one block (in-edges in groups of 512); rows with d+(v) >
// kTrHeavyCap keep their counters in global memory.
#include "common.cuh"

namespace tdt {

constexpr int kTrBlock = 512;
constexpr int kTrWarps = kTrBlock / kWarp;
constexpr int kTrMinBlocks = 3;
constexpr int kTrSmemBytes = 64 * 1024;
constexpr int kTrSlice = kTrSmemBytes / kTrWarps;   // 4 KB per warp for light rows
constexpr int kTrLightCap = 192;
constexpr int kTrGroup = kTrBlock;                  // in-edges per heavy group
constexpr int kTrHeavyChunk = 16;
constexpr int kTrBatch = 8;
// per-row entry: slot base (8 B), counter (4 B), limit (4 B)
constexpr int kTrEntryBytes = 16;
// light slice: rows | group S[32] VI[32] BV[32]
static_assert(kTrEntryBytes * kTrLightCap + 16 * kWarp <= kTrSlice, "light slice");
// heavy buffer: rows | group S[512] VI[512] BV[512]
constexpr int kTrHvGroup = kTrSmemBytes - 16 * kTrGroup;
constexpr int kTrHeavyCap = kTrHvGroup / kTrEntryBytes;

struct TrArgs {
    const int64_t* rp;        // out-CSR row offsets
    const int64_t* cp;        // in-adjacency offsets
    const int32_t* in_eid;    // in-adjacency edge ids
    const int64_t* off;       // list offsets
    const int32_t* cA;
    const int32_t* cB;
    const int32_t* cC;
    int2* lists;
    int32_t* gcnt;            // global counters (zeroed) for rows beyond kTrHeavyCap
    int* status;
    const int* gate;          // non-zero: skip
    int64_t nv, ne;
};

struct TrCtl {
    unsigned long long heavy_next;
    unsigned long long light_next;
};

struct TrRow {
    int64_t rbeg;             // first edge of row v
    int d;                    // d+(v)
    bool packed;              // counters in shared memory
    int64_t* base;
    int32_t* cnt;
    int32_t* lim;
};

__device__ __forceinline__ TrRow tr_stage(const TrArgs& A, int64_t rbeg, int d, bool packed, unsigned char* buf,
                                          int cap, int tid, int nthr) {
    TrRow R;
    R.rbeg = rbeg;
    R.d = d;
    R.packed = packed;
    R.base = reinterpret_cast<int64_t*>(buf);
    R.cnt = reinterpret_cast<int32_t*>(buf + 8 * cap);
    R.lim = R.cnt + cap;
    if (packed) {
        for (int j = tid; j < d; j += nthr) {
            const int64_t e = rbeg + j;
            R.base[j] = __ldg(A.off + e) + __ldg(A.cA + e) + __ldg(A.cB + e);
            R.cnt[j] = 0;
            R.lim[j] = __ldg(A.cC + e);
        }
    }
    return R;
}

__device__ __forceinline__ void tr_fail(const TrArgs& A) {
    if (A.status) atomicMax(A.status, (int)TDT_ERR_CAPACITY);
}

// Walk in-edge list entries [w0, w1) of a group (S: strictly increasing starts
// of the non-empty role-A lists, BV their list positions, VI their edge ids).
__device__ __forceinline__ void tr_walk(const TrArgs& A, const TrRow& R, const int32_t* S, const int32_t* VI,
                                        const int64_t* BV, int n, int w0, int w1, int o0) {
    const unsigned lane = lane_id();
    const unsigned le = lanemask_lt() | (1u << lane);
    int ob = o0;
    for (int base = w0; base < w1; base += kWarp) {
        const int k = ob + 1 + (int)lane;
        const int32_t B = k < n ? S[k] : INT32_MAX;
        const unsigned bit = ((unsigned)(B - base) < (unsigned)kWarp) ? (1u << (B - base)) : 0u;
        const unsigned mk = __reduce_or_sync(kFull, bit);
        const int nb = __popc(mk);
        const int32_t Bn = __shfl_sync(kFull, B, nb);
        const int t = base + (int)lane;
        if (t < w1) {
            const int o = ob + __popc(mk & le);
            const int2 ent = __ldcg(A.lists + BV[o] + (t - S[o]));  // (eB, eC) of a role-A entry
            const int64_t j = (int64_t)ent.y - R.rbeg;
            if (j < 0 || j >= R.d) {
                tr_fail(A);
            } else if (R.packed) {
                const int c = atomicAdd(R.cnt + j, 1);
                if (c < R.lim[j]) A.lists[R.base[j] + c] = make_int2(VI[o], ent.x);
                else tr_fail(A);
            } else {
                const int64_t e = ent.y;
                const int c = atomicAdd(A.gcnt + e, 1);
                if (c < __ldg(A.cC + e))
                    A.lists[__ldg(A.off + e) + __ldg(A.cA + e) + __ldg(A.cB + e) + c] = make_int2(VI[o], ent.x);
                else
                    tr_fail(A);
            }
        }
        ob += nb + (Bn == base + kWarp ? 1 : 0);
    }
}

__device__ __forceinline__ void tr_flush(const TrArgs& A, const TrRow& R, int tid, int nthr) {
    for (int j = tid; j < R.d; j += nthr) {
        const int64_t e = R.rbeg + j;
        const int c = R.packed ? R.cnt[j] : A.gcnt[e];
        if (c != __ldg(A.cC + e)) tr_fail(A);
    }
}

__global__ void __launch_bounds__(kTrBlock, kTrMinBlocks) transpose_kernel(TrArgs A, TrCtl* ctl) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int32_t s_list[kTrHeavyChunk];
    __shared__ int32_t s_wsum[2][kTrWarps + 1];
    __shared__ int s_n;
    __shared__ long long s_chunk;
    if (A.gate && *(volatile const int*)A.gate != 0) return;
    const int wib = threadIdx.x / kWarp;
    const unsigned lane = lane_id();
    const int64_t nv = A.nv;
    const long long nchunks = (nv + kTrHeavyChunk - 1) / kTrHeavyChunk;

    // ---- phase 1: rows with more than 32 in-edges or d+(v) > kTrLightCap
    {
        int32_t* g_S = reinterpret_cast<int32_t*>(smem + kTrHvGroup);
        int32_t* g_VI = g_S + kTrGroup;
        int64_t* g_BV = reinterpret_cast<int64_t*>(g_VI + kTrGroup);
        for (;;) {
            if (threadIdx.x == 0) {
                s_chunk = (long long)atomicAdd(&ctl->heavy_next, 1ull);
                s_n = 0;
            }
            __syncthreads();
            const long long c = s_chunk;
            if (c >= nchunks) break;
            for (int k = threadIdx.x; k < kTrHeavyChunk; k += kTrBlock) {
                const long long v = c * kTrHeavyChunk + k;
                if (v < nv) {
                    const int64_t d = __ldg(A.rp + v + 1) - __ldg(A.rp + v);
                    const int64_t din = __ldg(A.cp + v + 1) - __ldg(A.cp + v);
                    if (d > 0 && din > 0 && (din > kWarp || d > kTrLightCap)) s_list[atomicAdd(&s_n, 1)] = (int32_t)v;
                }
            }
            __syncthreads();
            const int nh = s_n;
            __syncthreads();
            for (int h = 0; h < nh; h++) {
                const long long v = s_list[h];
                const int64_t rbeg = __ldg(A.rp + v);
                const int d = (int)(__ldg(A.rp + v + 1) - rbeg);
                const int64_t k0 = __ldg(A.cp + v), k1 = __ldg(A.cp + v + 1);
                TrRow R = tr_stage(A, rbeg, d, d <= kTrHeavyCap, smem, kTrHeavyCap, threadIdx.x, kTrBlock);
                __syncthreads();
                for (int64_t g0 = k0; g0 < k1; g0 += kTrGroup) {
                    const int64_t k = g0 + threadIdx.x;
                    int32_t len = 0, eid = 0;
                    int64_t bv = 0;
                    if (k < k1) {
                        eid = __ldg(A.in_eid + k);
                        if (eid >= 0 && eid < A.ne) {
                            len = __ldg(A.cA + eid);
                            bv = __ldg(A.off + eid);
                        }
                    }
                    const unsigned nem = __ballot_sync(kFull, len > 0);
                    const int32_t incl = warp_incl_scan(len);
                    if (lane == 31) {
                        s_wsum[0][wib] = incl;
                        s_wsum[1][wib] = __popc(nem);
                    }
                    __syncthreads();
                    if (wib == 0) {
                        const int32_t x = (int)lane < kTrWarps ? s_wsum[0][lane] : 0;
                        const int32_t y = (int)lane < kTrWarps ? s_wsum[1][lane] : 0;
                        const int32_t xi = warp_incl_scan(x), yi = warp_incl_scan(y);
                        if ((int)lane < kTrWarps) {
                            s_wsum[0][lane] = xi - x;
                            s_wsum[1][lane] = yi - y;
                        }
                        if ((int)lane == kTrWarps - 1) {
                            s_wsum[0][kTrWarps] = xi;
                            s_wsum[1][kTrWarps] = yi;
                        }
                    }
                    __syncthreads();
                    if (len > 0) {
                        const int ci = s_wsum[1][wib] + __popc(nem & lanemask_lt());
                        g_S[ci] = s_wsum[0][wib] + incl - len;
                        g_VI[ci] = eid;
                        g_BV[ci] = bv;
                    }
                    const int total = s_wsum[0][kTrWarps];
                    const int n = s_wsum[1][kTrWarps];
                    __syncthreads();
                    const int share = ((total + kTrBlock - 1) / kTrBlock) * kWarp;
                    const int w0 = wib * share;
                    const int w1 = w0 + share < total ? w0 + share : total;
                    if (w0 < w1) {
                        int o0 = 0;
                        if (lane == 0) {
                            int lo = 0, hi = n - 1;
                            while (lo < hi) {
                                const int mid = (lo + hi + 1) >> 1;
                                if (g_S[mid] <= w0) lo = mid; else hi = mid - 1;
                            }
                            o0 = lo;
                        }
                        o0 = __shfl_sync(kFull, o0, 0);
                        tr_walk(A, R, g_S, g_VI, g_BV, n, w0, w1, o0);
                    }
                    __syncthreads();
                }
                tr_flush(A, R, threadIdx.x, kTrBlock);
                __syncthreads();
            }
        }
    }

    // ---- phase 2: rows with 1..32 in-edges and 1 <= d+(v) <= kTrLightCap, one warp per row
    unsigned char* sl = smem + wib * kTrSlice;
    int32_t* l_S = reinterpret_cast<int32_t*>(sl + kTrEntryBytes * kTrLightCap);
    int32_t* l_VI = l_S + kWarp;
    int64_t* l_BV = reinterpret_cast<int64_t*>(l_VI + kWarp);
    for (;;) {
        unsigned long long b = 0;
        if (lane == 0) b = atomicAdd(&ctl->light_next, (unsigned long long)kTrBatch);
        b = __shfl_sync(kFull, b, 0);
        if ((long long)b >= nv) break;
        for (int q = 0; q < kTrBatch; q++) {
            const long long v = (long long)b + q;
            if (v >= nv) break;
            const int64_t rbeg = __ldg(A.rp + v);
            const int d = (int)(__ldg(A.rp + v + 1) - rbeg);
            const int64_t k0 = __ldg(A.cp + v), k1 = __ldg(A.cp + v + 1);
            if (d <= 0 || k1 <= k0 || k1 - k0 > kWarp || d > kTrLightCap) continue;
            TrRow R = tr_stage(A, rbeg, d, true, sl, kTrLightCap, lane, kWarp);
            const int64_t k = k0 + lane;
            int32_t len = 0, eid = 0;
            int64_t bv = 0;
            if (k < k1) {
                eid = __ldg(A.in_eid + k);
                if (eid >= 0 && eid < A.ne) {
                    len = __ldg(A.cA + eid);
                    bv = __ldg(A.off + eid);
                }
            }
            const unsigned nem = __ballot_sync(kFull, len > 0);
            const int32_t incl = warp_incl_scan(len);
            const int total = __shfl_sync(kFull, incl, 31);
            if (len > 0) {
                const int ci = __popc(nem & lanemask_lt());
                l_S[ci] = incl - len;
                l_VI[ci] = eid;
                l_BV[ci] = bv;
            }
            __syncwarp();
            if (total > 0) tr_walk(A, R, l_S, l_VI, l_BV, __popc(nem), 0, total, 0);
            __syncwarp();
            tr_flush(A, R, lane, kWarp);
            __syncwarp();
        }
    }
}

// Role-C entries of every list (skipped on the device when *gate != 0).  gcnt:
// int32[E] scratch, ctl: 16 bytes of scratch; both zeroed here.
int launch_list_transpose(const int64_t* rp, const int64_t* cp, const int32_t* in_eid, int64_t nv, int64_t ne,
                          const int64_t* off, const int32_t* cA, const int32_t* cB, const int32_t* cC, int2* lists,
                          int32_t* gcnt, void* ctl, const int* gate, int* status, cudaStream_t st) {
    if (nv <= 0 || ne <= 0) return TDT_OK;
    DeviceInfo di;
    int rc = device_info(&di);
    if (rc) return rc;
    TDT_CUDA(cudaMemsetAsync(gcnt, 0, 4 * (size_t)ne, st));
    TDT_CUDA(cudaMemsetAsync(ctl, 0, sizeof(TrCtl), st));
    TDT_CUDA(cudaFuncSetAttribute(transpose_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kTrSmemBytes));
    TDT_CUDA(cudaFuncSetAttribute(transpose_kernel, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
    int per_sm = 0;
    TDT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, transpose_kernel, kTrBlock, kTrSmemBytes));
    if (per_sm < 1) per_sm = 1;
    TrArgs A{rp, cp, in_eid, off, cA, cB, cC, lists, gcnt, status, gate, nv, ne};
    transpose_kernel<<<di.sms * per_sm, kTrBlock, kTrSmemBytes, st>>>(A, reinterpret_cast<TrCtl*>(ctl));
    TDT_LAUNCH_CHECK("list_transpose");
    return TDT_OK;
}

}  // namespace tdt
