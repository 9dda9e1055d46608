// Per-edge support (triangle count per edge) and per-edge triangle lists over
// the degree-oriented CSR.
//
// Replaces checkElementsTwoPtr / checkElementsTwoPtrTile (kernel.cu:28-141),
// which give every edge (u,v) one thread that merges N+(u) and N+(v) and adds
// +1 to (u,w), +1 to (v,w) and +count to (u,v) for every common w.
//
// Here the unit of work is the source vertex u of the triangle (u, v, w)
// (u -> v, u -> w, v -> w):
//   * N+(u) is staged once in shared memory (warp slice for d+(u) <= kWarpCap,
//     the whole block's buffer for larger rows; rows beyond the block buffer
//     are searched in place);
//   * the warp walks the flattened list of all (v, w) with v in N+(u) and
//     w in N+(v), 32 consecutive entries per step (coalesced loads of N+(v)),
//     and looks each w up in N+(u) by binary search (restricted to the
//     entries after v when the orientation is by vertex id);
//   * hits on (u,v) and (u,w) go to shared-memory counters flushed once per
//     row; only the (v,w) hit is a global atomic.
// Each triangle is found exactly once, from its (source, middle) edge, so the
// counts are the reference's for any n_cut.
//
// Modes:
//   kSupAccum  output[e] += support (the drop-in operator);
//   kSupRoles  role counts: cA[e] triangles where e is (source,middle),
//              cB[e] where e is (source,sink), cC[e] where e is (middle,sink);
//   kSupList   per-edge triangle lists: the entry of edge e in triangle
//              (eA, eB, eC) holds the two other edges; e's list occupies
//              [off[e], off[e+1]) with its role-A entries first, then role B,
//              then role C.  Slots of roles A and B come from per-row cursors
//              in shared memory, role C from a global cursor.
#include "common.cuh"

namespace tdt {

constexpr int kSupBlock = 512;                 // 16 warps
constexpr int kSupWarps = kSupBlock / kWarp;
constexpr int kVertexBatch = 8;                // vertices per dynamic grab
// 48 KB of dynamic shared memory per block: with ~6 KB static, four blocks
// (64 warps, full occupancy at <= 32 registers) fit the SM's 228 KB
constexpr int kSupSmemBytes = 48 * 1024;
constexpr int kHeavyChunk = 16;                // vertices scanned per phase-1 grab

enum SupMode { kSupAccum = 0, kSupRoles = 1, kSupList = 2 };

// shared-memory bytes per staged row entry (light rows: row + counters; heavy
// rows add the pair-space prefix (4 B) and the out-list start of each v (8 B))
template <int M>
struct RowBytes {
    static constexpr int value = M == kSupAccum ? 8 : (M == kSupRoles ? 12 : 20);
};
template <int M>
struct HeavyCap {
    static constexpr int value = (kSupSmemBytes - 1024) / (RowBytes<M>::value + 12);
};
// light rows (d+(u) <= WarpCap) get one warp and a per-warp shared slice
template <int M>
struct WarpCap {
    static constexpr int value = M == kSupList ? 128 : 256;
};
static_assert(RowBytes<kSupList>::value * WarpCap<kSupList>::value * kSupWarps <= kSupSmemBytes, "list slices");
static_assert(RowBytes<kSupRoles>::value * WarpCap<kSupRoles>::value * kSupWarps <= kSupSmemBytes, "role slices");

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

struct SupArgs {
    int32_t* out;                   // kSupAccum
    int32_t* cA;                    // kSupRoles outputs (cC by global atomics)
    int32_t* cB;
    int32_t* cC;
    const int64_t* off;             // kSupList: list offsets int64[E+1]
    const int32_t* cA_in;           // kSupList: role-A counts (role-B base = off + cA)
    const int32_t* cB_in;           // kSupList: role-B counts (end-of-row check)
    unsigned long long* curA_g;     // kSupList: global cursors for rows beyond the smem cap
    unsigned long long* curB_g;
    unsigned long long* curC;       // kSupList: role-C cursors, start at off + cA + cB
    int2* lists;
    const int* gate;                // non-zero: skip the pass
    int* status;                    // kSupList: set when a row's slots do not end where counted
    int warp_cap;                   // rows with d+ <= warp_cap go to one warp (<= kWarpCap)
    int heavy_cap;                  // heavier rows staged in smem up to this size (<= the mode's cap)
};

// Test hook: lower the light/heavy thresholds so small graphs drive every path
// (0 restores the defaults).
static int g_warp_cap = 0, g_heavy_cap = 0;
void set_support_caps(int warp_cap, int heavy_cap) {
    g_warp_cap = warp_cap;
    g_heavy_cap = heavy_cap;
}

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

// Per-row state of one staged row (shared memory or, beyond the cap, global).
template <int M>
struct RowState {
    const int32_t* su;            // N+(u)
    int32_t* cnt0;                // accum: counters; roles: role A counters
    int32_t* cnt1;                // roles: role B counters
    unsigned long long* curA;     // list: slot cursors of (u, su[i]) as role A
    unsigned long long* curB;     // list: slot cursors as role B
    int64_t bu;                   // position of the row's first edge
};

// One triangle (u, v = su[i], w = su[p]) with (v,w) at position pos.
template <int M>
__device__ __forceinline__ void on_triangle(const RowState<M>& R, const SupArgs& A, int i, int p, int64_t pos) {
    if (M == kSupAccum) {
        atomicAdd(R.cnt0 + p, 1);
        atomicAdd(R.cnt0 + i, 1);
        atomicAdd(A.out + pos, 1);
    } else if (M == kSupRoles) {
        atomicAdd(R.cnt0 + i, 1);
        atomicAdd(R.cnt1 + p, 1);
        atomicAdd(A.cC + pos, 1);
    } else {
        const int32_t eA = (int32_t)(R.bu + i), eB = (int32_t)(R.bu + p), eC = (int32_t)pos;
        const unsigned long long sA = atomicAdd(R.curA + i, 1ull);
        const unsigned long long sB = atomicAdd(R.curB + p, 1ull);
        const unsigned long long sC = atomicAdd(A.curC + pos, 1ull);
        A.lists[sA] = make_int2(eB, eC);
        A.lists[sB] = make_int2(eA, eC);
        A.lists[sC] = make_int2(eA, eB);
    }
}

// One warp processes the v-batches vb = first, first+step, ... of row u.
// kIdOrdered: every edge goes from a lower to a higher vertex id (the
// reference's rank orientation), so w lies after v in N+(u) and the last v has
// no partner; without it (any acyclic orientation) all of N+(u) is searched.
template <int M, bool kIdOrdered, class Off>
__device__ __forceinline__ void wedge_walk(const OutRows<Off>& G, const SupArgs& A, const RowState<M>& R, int d,
                                           int first, int step, int32_t* s_excl, Off* s_bv) {
    const unsigned lane = lane_id();
    const int32_t* su = R.su;
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
            if (p >= 0) on_triangle<M>(R, A, vb + o, p, (int64_t)pos);
        }
        __syncwarp();
    }
}

// Stage row u (d entries at bu) into buf; rows that do not fit use global arrays.
template <int M, class Off>
__device__ __forceinline__ RowState<M> stage_row(const OutRows<Off>& G, const SupArgs& A, unsigned char* buf,
                                                 int cap, bool in_smem, Off bu, int d, int tid, int nthr) {
    RowState<M> R;
    R.bu = bu;
    R.cnt0 = R.cnt1 = nullptr;
    R.curA = R.curB = nullptr;
    if (!in_smem) {
        R.su = G.cols + bu;
        if (M == kSupAccum) R.cnt0 = A.out + bu;
        if (M == kSupRoles) { R.cnt0 = A.cA + bu; R.cnt1 = A.cB + bu; }
        if (M == kSupList) { R.curA = A.curA_g + bu; R.curB = A.curB_g + bu; }
        return R;
    }
    int32_t* su = reinterpret_cast<int32_t*>(buf);
    R.su = su;
    if (M == kSupList) {
        unsigned long long* ca = reinterpret_cast<unsigned long long*>(buf + ((4 * cap + 15) & ~15));
        unsigned long long* cb = ca + cap;
        R.curA = ca;
        R.curB = cb;
        for (int i = tid; i < d; i += nthr) {
            su[i] = __ldg(G.cols + bu + i);
            const unsigned long long o = (unsigned long long)__ldg(A.off + bu + i);
            ca[i] = o;
            cb[i] = o + (unsigned long long)__ldg(A.cA_in + bu + i);
        }
    } else {
        int32_t* c0 = su + cap;
        int32_t* c1 = c0 + cap;
        R.cnt0 = c0;
        R.cnt1 = c1;
        for (int i = tid; i < d; i += nthr) {
            su[i] = __ldg(G.cols + bu + i);
            c0[i] = 0;
            if (M == kSupRoles) c1[i] = 0;
        }
    }
    return R;
}

// Heavy rows in shared memory: the row's (v, w) pair space is flattened with
// a block-wide prefix over d+(v) so every thread gets an equal share of the
// pairs (a row's pairs can be far more than 32 lanes x d).
template <int M, bool kIdOrdered, class Off>
__device__ __forceinline__ void heavy_flat_walk(const OutRows<Off>& G, const SupArgs& A, const RowState<M>& R, int d,
                                                int32_t* pre, Off* bv, int32_t* s_wsum) {
    const int tid = threadIdx.x;
    const unsigned lane = lane_id();
    const int wib = tid / kWarp;
    const int32_t* su = R.su;
    const int vend = kIdOrdered ? d - 1 : d;
    // pre[i] = sum of d+(su[j]) for j < i, for i in [0, vend]
    int32_t carry = 0;
    for (int base = 0; base < vend; base += kSupBlock) {
        const int i = base + tid;
        int32_t len = 0;
        Off b = 0;
        if (i < vend) {
            const int32_t v = su[i];
            if (v >= 0 && v < G.nv) {
                b = G.begin(v);
                len = (int32_t)(G.end(v) - b);
            }
            bv[i] = b;
        }
        int32_t incl = warp_incl_scan(len);
        if (lane == 31) s_wsum[wib] = incl;
        __syncthreads();
        if (wib == 0) {
            int32_t x = s_wsum[lane < kSupWarps ? lane : 0];
            if (lane >= kSupWarps) x = 0;
            const int32_t xi = warp_incl_scan(x);
            if (lane < kSupWarps) s_wsum[lane] = xi - x;
            if (lane == kSupWarps - 1) s_wsum[kSupWarps] = xi;
        }
        __syncthreads();
        if (i < vend) pre[i] = carry + s_wsum[wib] + incl - len;
        carry += s_wsum[kSupWarps];
        __syncthreads();
    }
    if (tid == 0) pre[vend] = carry;
    __syncthreads();
    const int32_t total = carry;
    const int32_t umax = su[d - 1];
    for (int32_t t = tid; t < total; t += kSupBlock) {
        int lo = 0, hi = vend - 1;  // last i with pre[i] <= t
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (pre[mid] <= t) lo = mid; else hi = mid - 1;
        }
        const Off pos = bv[lo] + (t - pre[lo]);
        const int32_t w = __ldg(G.cols + pos);
        if (w > umax) continue;
        const int p = bsearch_i32(su, kIdOrdered ? lo + 1 : 0, d, w);
        if (p >= 0) on_triangle<M>(R, A, lo, p, (int64_t)pos);
    }
}

template <int M>
__device__ __forceinline__ void flush_row(const RowState<M>& R, const SupArgs& A, bool in_smem, int d, int tid,
                                          int nthr) {
    if (M == kSupList) {
        // every role-A / role-B cursor of the row must have reached the end of
        // its segment: the listing pass found exactly the triangles counted
        for (int i = tid; i < d; i += nthr) {
            const unsigned long long o = (unsigned long long)__ldg(A.off + R.bu + i);
            const unsigned long long a = o + (unsigned long long)__ldg(A.cA_in + R.bu + i);
            const unsigned long long b = a + (unsigned long long)__ldg(A.cB_in + R.bu + i);
            if ((R.curA[i] != a || R.curB[i] != b) && A.status) atomicMax(A.status, (int)TDT_ERR_CAPACITY);
        }
        return;
    }
    if (!in_smem) return;
    if (M == kSupAccum) {
        for (int i = tid; i < d; i += nthr)
            if (R.cnt0[i]) atomicAdd(A.out + R.bu + i, R.cnt0[i]);
    } else if (M == kSupRoles) {
        // role A/B counts of row u's edges come only from row u: plain stores
        for (int i = tid; i < d; i += nthr) {
            A.cA[R.bu + i] = R.cnt0[i];
            A.cB[R.bu + i] = R.cnt1[i];
        }
    }
}

// ctl != nullptr: dynamic scheduling through its counters (zeroed by the
// caller); ctl == nullptr: static round-robin scheduling (no scratch at all).
template <int M, bool kIdOrdered, class Off>
__global__ void __launch_bounds__(kSupBlock) support_kernel(OutRows<Off> G, SupArgs A, SupCtl* ctl) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int32_t s_excl[kSupWarps][kWarp];
    __shared__ Off s_bv[kSupWarps][kWarp];
    __shared__ int32_t s_list[kHeavyChunk];
    __shared__ int32_t s_wsum[kSupWarps + 1];
    __shared__ int s_n;
    __shared__ long long s_chunk;
    const int wib = threadIdx.x / kWarp;
    const unsigned lane = lane_id();
    const int64_t nv = G.nv;
    const long long nchunks = (nv + kHeavyChunk - 1) / kHeavyChunk;
    if (A.gate && *(volatile const int*)A.gate != 0) return;
    constexpr int kHeavy = HeavyCap<M>::value;
    const int warp_cap = A.warp_cap;
    const int heavy_cap = A.heavy_cap;

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
            if (u < nv && G.end(u) - G.begin(u) > warp_cap) s_list[atomicAdd(&s_n, 1)] = (int32_t)u;
        }
        __syncthreads();
        const int nh = s_n;
        __syncthreads();  // every thread has read s_n before thread 0 resets it
        for (int h = 0; h < nh; h++) {
            const long long u = s_list[h];
            const Off bu = G.begin(u);
            const int d = (int)(G.end(u) - bu);
            const bool in_smem = d <= heavy_cap;
            RowState<M> R = stage_row<M>(G, A, smem, kHeavy, in_smem, bu, d, threadIdx.x, kSupBlock);
            __syncthreads();
            if (in_smem) {
                // prefix and out-list starts live after the row buffers
                unsigned char* tail = smem + ((size_t)RowBytes<M>::value * kHeavy + 15) / 16 * 16;
                Off* bvv = reinterpret_cast<Off*>(tail);
                int32_t* pre = reinterpret_cast<int32_t*>(bvv + kHeavy);
                heavy_flat_walk<M, kIdOrdered>(G, A, R, d, pre, bvv, s_wsum);
            } else {
                wedge_walk<M, kIdOrdered>(G, A, R, d, wib * kWarp, kSupBlock, s_excl[wib], s_bv[wib]);
            }
            __syncthreads();
            flush_row<M>(R, A, in_smem, d, threadIdx.x, kSupBlock);
            __syncthreads();
        }
    }

    // ---- phase 2: rows with 2 <= d+(u) <= kWarpCap, one warp per row, taken
    // in batches from the top ids (highest degree rank) down
    unsigned char* wbuf = smem + wib * (RowBytes<M>::value * WarpCap<M>::value);
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
            if (d < 2 || d > warp_cap) continue;
            RowState<M> R = stage_row<M>(G, A, wbuf, WarpCap<M>::value, true, bu, d, lane, kWarp);
            __syncwarp();
            wedge_walk<M, kIdOrdered>(G, A, R, d, 0, kWarp, s_excl[wib], s_bv[wib]);
            __syncwarp();
            flush_row<M>(R, A, true, d, lane, kWarp);
            __syncwarp();
        }
    }
}

template <int M, bool kIdOrdered, class Off>
static int launch_mode(const OutRows<Off>& G, const SupArgs& A, SupCtl* ctl, cudaStream_t st) {
    DeviceInfo di;
    int rc = device_info(&di);
    if (rc) return rc;
    SupArgs A2 = A;
    A2.warp_cap = (g_warp_cap > 0 && g_warp_cap < WarpCap<M>::value) ? g_warp_cap : WarpCap<M>::value;
    A2.heavy_cap = (g_heavy_cap > 0 && g_heavy_cap < HeavyCap<M>::value) ? g_heavy_cap : HeavyCap<M>::value;
    auto kern = support_kernel<M, kIdOrdered, Off>;
    TDT_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, kSupSmemBytes));
    TDT_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
    if (ctl) TDT_CUDA(cudaMemsetAsync(ctl, 0, sizeof(SupCtl), st));
    int blocks_per_sm = 0;
    TDT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, kern, kSupBlock, kSupSmemBytes));
    if (blocks_per_sm < 1) blocks_per_sm = 1;
    kern<<<di.sms * blocks_per_sm, kSupBlock, kSupSmemBytes, st>>>(G, A2, ctl);
    TDT_LAUNCH_CHECK("support");
    return TDT_OK;
}

// Drop-in support operator: accumulates into out; static schedule, no scratch.
int launch_support_accum_i32(const int32_t* rp, int32_t stride, const int32_t* cols, int64_t nv, int64_t ne,
                             int32_t* out, cudaStream_t st) {
    if (nv <= 0) return TDT_OK;
    OutRows<int32_t> G{rp, stride, cols, nv, ne};
    SupArgs A{};
    A.out = out;
    return launch_mode<kSupAccum, false, int32_t>(G, A, nullptr, st);
}

// Whole-path pass 1: role counts.  cA/cB are stored per row, cC accumulated by
// atomics, so all three are zeroed first.
int launch_support_roles(const int64_t* rp, const int32_t* cols, int64_t nv, int64_t ne, int32_t* cA, int32_t* cB,
                         int32_t* cC, void* ctl, const int* gate, cudaStream_t st) {
    TDT_CUDA(cudaMemsetAsync(cA, 0, 4 * (size_t)ne, st));
    TDT_CUDA(cudaMemsetAsync(cB, 0, 4 * (size_t)ne, st));
    TDT_CUDA(cudaMemsetAsync(cC, 0, 4 * (size_t)ne, st));
    if (nv <= 0) return TDT_OK;
    OutRows<int64_t> G{rp, 1, cols, nv, ne};
    SupArgs A{};
    A.cA = cA;
    A.cB = cB;
    A.cC = cC;
    A.gate = gate;
    return launch_mode<kSupRoles, true, int64_t>(G, A, reinterpret_cast<SupCtl*>(ctl), st);
}

// Whole-path pass 2: triangle lists (skipped on the device when *gate != 0).
int launch_support_list(const int64_t* rp, const int32_t* cols, int64_t nv, int64_t ne, const int64_t* off,
                        const int32_t* cA, const int32_t* cB, unsigned long long* curA_g, unsigned long long* curB_g,
                        unsigned long long* curC, int2* lists, void* ctl, const int* gate, int* status,
                        cudaStream_t st) {
    if (nv <= 0) return TDT_OK;
    OutRows<int64_t> G{rp, 1, cols, nv, ne};
    SupArgs A{};
    A.off = off;
    A.cA_in = cA;
    A.cB_in = cB;
    A.curA_g = curA_g;
    A.curB_g = curB_g;
    A.curC = curC;
    A.lists = lists;
    A.gate = gate;
    A.status = status;
    return launch_mode<kSupList, true, int64_t>(G, A, reinterpret_cast<SupCtl*>(ctl), st);
}

size_t support_ctl_bytes() { return 256; }

}  // namespace tdt
