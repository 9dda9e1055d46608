// Role-C entries of the per-edge triangle lists, by transposing role-A lists.
//
// The listing pass writes every triangle's role-A entry (in the list of its
// (source, middle) edge) and role-B entry (in the list of its (source, sink)
// edge); both edges belong to the source row, so those writes stay inside one
// row's list region.  The role-C entry belongs to the (middle, sink) edge of
// another row; written from the source row it would be a random 8-byte store
// per triangle (a DRAM read-modify-write of a 32-byte sector each).
//
// Here the role-C entries are produced in middle-vertex order: the
// in-adjacency lists every edge (u, v) grouped by v, and the role-A list of
// (u, v) holds (eB = (u,w), eC = (v,w)) for each triangle (u, v, w); the
// role-C entry of eC is (e_uv, eB).  Walking the in-adjacency in order, the
// stores of consecutive in-edges land in the list region of the same vertex v.
// The in-adjacency is cut into groups of 512 in-edges (one per thread),
// whatever the vertex boundaries, so a vertex with a huge in-degree spreads
// over many blocks; the role-A lists of a group are one flat index space that
// the block's warps split evenly and walk 32 entries per step (the same owner
// reduction as the support pass).  Slots come from one 64-bit cursor per edge
// (start of its role-C segment); every store is checked against the end of
// the lists (one bound for the kernel instead of a random load of the edge's
// own end per entry), and check_kernel verifies afterwards that every cursor
// ended exactly at its edge's list end (else TDT_ERR_CAPACITY, and the lists
// are not used).
// The in-edges of a group have consecutive target vertices, whose out-edges
// (the edges that receive the group's role-C entries) are one contiguous edge
// range.  For the vertices whose in-edges all lie inside the group, the
// cursors of up to kTrSmemCur of those out-edges are copied to shared memory
// at the start of the group, advanced there, and written back at its end: no
// other group touches them.  Only the entries of the group's first and last
// vertices (shared with the neighbouring groups) and of very long out-edge
// ranges take the global atomic.
//
// Keyed groups: when all out-edges of the group's target vertices (one
// contiguous edge range, up to kTrKeys of them) fit a shared-memory table,
// the group's entries are taken in chunks of kTrChunk; each entry's rank
// among the chunk's entries of the same (middle, sink) edge comes from a
// shared-memory counter, one global cursor atomic per distinct edge of the
// chunk reserves that edge's run of slots, and the run's stores land side
// by side.  A hub vertex (many in-edges, few out-edges) gives long runs: its
// role-C entries cost a fraction of a global atomic each.
#include "common.cuh"

namespace tdt {

constexpr int kTrBlock = 512;
constexpr int kTrWarps = kTrBlock / kWarp;
#ifndef TDT_TR_MINB
#define TDT_TR_MINB 3
#endif
constexpr int kTrMinBlocks = TDT_TR_MINB;
constexpr int kTrSmemCur = 3072;   // out-edge cursors a group keeps in shared memory (24 KB)
#ifndef TDT_TR_KEYED
#define TDT_TR_KEYED 1
#endif
constexpr int kTrKeys = TDT_TR_KEYED ? kTrSmemCur : 0;  // out-edges of a keyed group (bases reuse s_cur)
#ifndef TDT_TR_CHUNK_PER
#define TDT_TR_CHUNK_PER 4
#endif
constexpr int kTrChunkPer = TDT_TR_CHUNK_PER;                           // entries per thread per keyed chunk (counts stay below 2^16)
constexpr int kTrChunk = kTrBlock * kTrChunkPer;
static_assert(kTrChunk < 65536 && kTrSmemCur <= 65536 && kTrSmemCur % 2 == 0,
              "16-bit per-edge counters and touched-edge indices");

struct TrArgs {
    const int64_t* cp;                  // in-adjacency offsets (cp[V] = E)
    const int64_t* rp;                  // out-adjacency offsets (rp[V] = E)
    const int32_t* cols;                // out-adjacency targets
    const int32_t* in_eid;              // in-adjacency edge ids
    const int64_t* off;                 // list offsets
    const int32_t* cA;
    unsigned long long* cur;            // role-C cursors, start at off + cA + cB
    int2* lists;
    int* status;
    const int* gate;                    // non-zero: skip
    int64_t ne;
    int64_t nv;
};

__device__ __forceinline__ void tr_fail(const TrArgs& A) {
    if (A.status) atomicMax(A.status, (int)TDT_ERR_CAPACITY);
}

// Index of the list holding flat position p: the last i < n with S[i] <= p.
__device__ __forceinline__ int tr_owner(const int32_t* S, int n, int p) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (S[mid] <= p) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// A keyed group (see the top of the file): every thread of the block calls
// it; the group's role-A lists are S/VI/BV (n lists, total entries) and its
// role-C targets the out-edges [rbase, rbase + nkeys).  hist is all zero on
// entry and on return.
__device__ __forceinline__ void keyed_group(const TrArgs& A, const int32_t* S, const int32_t* VI, const int64_t* BV,
                                            int n, int total, long long rbase, int nkeys, unsigned long long cap,
                                            unsigned* hist, uint16_t* touch, int* ntouch,
                                            unsigned long long* base) {
    const int wib = threadIdx.x / kWarp;
    const unsigned lane = lane_id();
    const unsigned le = lanemask_lt() | (1u << lane);
    for (int cs = 0; cs < total; cs += kTrChunk) {
        const int ce = cs + kTrChunk < total ? cs + kTrChunk : total;
        const int p0 = cs + wib * (kTrChunkPer * kWarp);
        int key[kTrChunkPer], vi[kTrChunkPer];
        unsigned rank[kTrChunkPer];
        int32_t eb[kTrChunkPer];
#pragma unroll
        for (int h = 0; h < kTrChunkPer; h++) key[h] = -1;
        if (p0 < ce) {
            int ob = 0;
            if (lane == 0) ob = tr_owner(S, n, p0);
            ob = __shfl_sync(kFull, ob, 0);
            int2 ent[kTrChunkPer];
            int o[kTrChunkPer];
#pragma unroll
            for (int h = 0; h < kTrChunkPer; h++) {
                const int wb = p0 + h * kWarp;
                // list starts inside (wb, wb + 32): each is > wb, at most 31 fit
                const int kk = ob + 1 + (int)lane;
                const int32_t B = kk < n ? S[kk] : INT32_MAX;
                const unsigned bit = ((unsigned)(B - wb) < (unsigned)kWarp) ? (1u << (B - wb)) : 0u;
                const unsigned mk = __reduce_or_sync(kFull, bit);
                const int nb = __popc(mk);
                const int32_t Bn = __shfl_sync(kFull, B, nb);
                o[h] = ob + __popc(mk & le);
                ent[h] = make_int2(0, -1);
                if (wb + (int)lane < ce) ent[h] = __ldcg(A.lists + BV[o[h]] + (wb + (int)lane - S[o[h]]));  // (eB, eC)
                ob += nb + (Bn == wb + kWarp ? 1 : 0);
            }
#pragma unroll
            for (int h = 0; h < kTrChunkPer; h++) {
                if (p0 + h * kWarp + (int)lane >= ce) continue;
                const long long kk = (long long)ent[h].y - rbase;
                if (kk < 0 || kk >= nkeys) {
                    tr_fail(A);
                    continue;
                }
                key[h] = (int)kk;
                eb[h] = ent[h].x;
                vi[h] = VI[o[h]];
                const unsigned sh = (unsigned)(key[h] & 1) * 16u;
                rank[h] = (atomicAdd(hist + (key[h] >> 1), 1u << sh) >> sh) & 0xffffu;
                if (rank[h] == 0u) touch[atomicAdd(ntouch, 1)] = (uint16_t)key[h];
            }
        }
        __syncthreads();
        // one cursor atomic per edge the chunk touched; its counter cleared
        const int nt = *ntouch;
        for (int i = threadIdx.x; i < nt; i += kTrBlock) {
            const int kk = touch[i];
            const unsigned sh = (unsigned)(kk & 1) * 16u;
            const unsigned c = (hist[kk >> 1] >> sh) & 0xffffu;
            base[kk] = atomicAdd(A.cur + rbase + kk, (unsigned long long)c);
        }
        __syncthreads();
        for (int i = threadIdx.x; i < nt; i += kTrBlock) hist[touch[i] >> 1] = 0u;
        if (threadIdx.x == 0) *ntouch = 0;
#pragma unroll
        for (int h = 0; h < kTrChunkPer; h++) {
            if (key[h] < 0) continue;
            const unsigned long long slot = base[key[h]] + rank[h];
            if (slot < cap) A.lists[slot] = make_int2(vi[h], eb[h]);
            else tr_fail(A);
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kTrBlock, kTrMinBlocks) transpose_kernel(TrArgs A, unsigned long long* next) {
    __shared__ int32_t s_S[kTrBlock];
    __shared__ int32_t s_VI[kTrBlock];
    __shared__ int64_t s_BV[kTrBlock];
    __shared__ int32_t s_wsum[2][kTrWarps + 1];
    __shared__ long long s_group;
    __shared__ unsigned long long s_cur[kTrSmemCur];
    __shared__ long long s_lo, s_hi;  // out-edges [s_lo, s_hi) have their cursors in s_cur
    // keyed groups: per-edge counters of a chunk (two 16-bit counters a word),
    // the edges the chunk touched, their count; the run bases go to s_cur
    __shared__ unsigned s_hist[kTrSmemCur / 2];
    __shared__ uint16_t s_touch[kTrChunk];
    __shared__ int s_ntouch;
    __shared__ long long s_rbase;
    __shared__ int s_nkeys;   // > 0: keyed group over out-edges [s_rbase, s_rbase + s_nkeys)
    if (A.gate && *(volatile const int*)A.gate != 0) return;
    const int wib = threadIdx.x / kWarp;
    const unsigned lane = lane_id();
    const unsigned le = lanemask_lt() | (1u << lane);
    const int64_t ne = A.ne;
    const long long ngroups = (ne + kTrBlock - 1) / kTrBlock;
    // stores stay inside the lists; tr_check_kernel then requires every
    // cursor to end exactly at its own list end
    const unsigned long long cap = (unsigned long long)__ldg(A.off + ne);
    for (int j = threadIdx.x; j < kTrSmemCur / 2; j += kTrBlock) s_hist[j] = 0u;
    if (threadIdx.x == 0) s_ntouch = 0;
    for (;;) {
        if (threadIdx.x == 0) s_group = (long long)atomicAdd(next, 1ull);
        __syncthreads();
        const long long grp = s_group;
        if (grp >= ngroups) break;
        // the vertices whose in-edges all lie in [k0, k1), and their out-edges
        if (threadIdx.x == 0) {
            const int64_t k0 = grp * kTrBlock, k1 = k0 + kTrBlock < ne ? k0 + kTrBlock : ne;
            long long lo = 0, hi = 0;
            int nkeys = 0;
            long long rbase = 0;
            const int32_t e0 = __ldg(A.in_eid + k0), e1 = __ldg(A.in_eid + k1 - 1);
            if (e0 >= 0 && e0 < ne && e1 >= 0 && e1 < ne) {
                int32_t va = __ldg(A.cols + e0), vb = __ldg(A.cols + e1);
                if (va >= 0 && vb >= va && vb < A.nv) {
                    rbase = __ldg(A.rp + va);
                    const long long r1 = __ldg(A.rp + vb + 1);
                    if (r1 > rbase && r1 - rbase <= kTrKeys) nkeys = (int)(r1 - rbase);
                }
                if (__ldg(A.cp + va) < k0) va++;          // shares its in-edges with the group before
                if (__ldg(A.cp + vb + 1) > k1) vb--;      // ... with the group after
                if (va <= vb) {
                    lo = __ldg(A.rp + va);
                    hi = __ldg(A.rp + vb + 1);
                    if (hi - lo > kTrSmemCur) hi = lo + kTrSmemCur;
                }
            }
            if (nkeys > 0) lo = hi = 0;  // s_cur holds the run bases instead
            s_lo = lo;
            s_hi = hi;
            s_rbase = rbase;
            s_nkeys = nkeys;
        }
        __syncthreads();
        const long long clo = s_lo, chi = s_hi;
        for (long long j = threadIdx.x; j < chi - clo; j += kTrBlock) s_cur[j] = A.cur[clo + j];
        // this thread's in-edge and the length / position of its role-A list
        const int64_t k = grp * kTrBlock + threadIdx.x;
        int32_t len = 0, eid = 0;
        int64_t bv = 0;
        if (k < ne) {
            eid = __ldg(A.in_eid + k);
            if (eid >= 0 && eid < ne) {
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
            s_S[ci] = s_wsum[0][wib] + incl - len;
            s_VI[ci] = eid;
            s_BV[ci] = bv;
        }
        const int total = s_wsum[0][kTrWarps];
        const int n = s_wsum[1][kTrWarps];
        const int nkeys = s_nkeys;
        const long long rbase = s_rbase;
        __syncthreads();
        if (nkeys > 0) {
            keyed_group(A, s_S, s_VI, s_BV, n, total, rbase, nkeys, cap, s_hist, s_touch, &s_ntouch, s_cur);
            continue;  // keyed_group ends with a barrier; s_cur holds no cursors
        }
        // equal shares of the group's entries, whole steps of 32
        const int share = ((total + kTrBlock - 1) / kTrBlock) * kWarp;
        const int w0 = wib * share;
        const int w1 = w0 + share < total ? w0 + share : total;
        if (w0 < w1) {
            int ob = 0;
            if (lane == 0) {
                int lo = 0, hi = n - 1;  // last entry with S <= w0
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (s_S[mid] <= w0) lo = mid; else hi = mid - 1;
                }
                ob = lo;
            }
            ob = __shfl_sync(kFull, ob, 0);
            for (int base = w0; base < w1; base += kWarp) {
                // list starts inside (base, base + 32): each is > base, at most 31 fit
                const int kk = ob + 1 + (int)lane;
                const int32_t B = kk < n ? s_S[kk] : INT32_MAX;
                const unsigned bit = ((unsigned)(B - base) < (unsigned)kWarp) ? (1u << (B - base)) : 0u;
                const unsigned mk = __reduce_or_sync(kFull, bit);
                const int nb = __popc(mk);
                const int32_t Bn = __shfl_sync(kFull, B, nb);
                const int t = base + (int)lane;
                if (t < w1) {
                    const int o = ob + __popc(mk & le);
                    const int2 ent = __ldcg(A.lists + s_BV[o] + (t - s_S[o]));  // (eB, eC)
                    const int32_t eC = ent.y;
                    if (eC < 0 || eC >= ne) {
                        tr_fail(A);
                    } else {
                        const unsigned long long slot = (eC >= clo && eC < chi)
                                                            ? atomicAdd(s_cur + (eC - clo), 1ull)
                                                            : atomicAdd(A.cur + eC, 1ull);
                        if (slot < cap) A.lists[slot] = make_int2(s_VI[o], ent.x);
                        else tr_fail(A);
                    }
                }
                ob += nb + (Bn == base + kWarp ? 1 : 0);
            }
        }
        __syncthreads();  // the group arrays are rewritten next
        for (long long j = threadIdx.x; j < chi - clo; j += kTrBlock) A.cur[clo + j] = s_cur[j];
    }
}

__global__ void tr_init_kernel(const int64_t* __restrict__ off, const int32_t* __restrict__ cA,
                               const int32_t* __restrict__ cB, int64_t E, unsigned long long* __restrict__ cur,
                               const int* gate) {
    if (gate && *(volatile const int*)gate != 0) return;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x)
        cur[e] = (unsigned long long)(off[e] + cA[e] + cB[e]);
}

// Every role-C cursor must end at the end of its edge's list.
__global__ void tr_check_kernel(const int64_t* __restrict__ off, int64_t E,
                                const unsigned long long* __restrict__ cur, const int* gate, int* status) {
    if (gate && *(volatile const int*)gate != 0) return;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x)
        if (cur[e] != (unsigned long long)off[e + 1]) atomicMax(status, (int)TDT_ERR_CAPACITY);
}

// Role-C entries of every list (skipped on the device when *gate != 0).  cur:
// uint64[E] scratch; next: 8 bytes of scratch.
int launch_list_transpose(const int64_t* cp, const int64_t* rp, const int32_t* cols, const int32_t* in_eid,
                          int64_t nv, int64_t ne, const int64_t* off,
                          const int32_t* cA, const int32_t* cB, int2* lists, unsigned long long* cur, void* next,
                          const int* gate, int* status, cudaStream_t st) {
    if (nv <= 0 || ne <= 0) return TDT_OK;
    DeviceInfo di;
    int rc = device_info(&di);
    if (rc) return rc;
    const unsigned g_e = grid_for(ne, 256, di.sms, 8);
    tr_init_kernel<<<g_e, 256, 0, st>>>(off, cA, cB, ne, cur, gate);
    TDT_LAUNCH_CHECK("list_transpose_init");
    TDT_CUDA(cudaMemsetAsync(next, 0, sizeof(unsigned long long), st));
    int per_sm = 0;
    TDT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, transpose_kernel, kTrBlock, 0));
    if (per_sm < 1) per_sm = 1;
    TrArgs A{cp, rp, cols, in_eid, off, cA, cur, lists, status, gate, ne, nv};
    transpose_kernel<<<di.sms * per_sm, kTrBlock, 0, st>>>(A, reinterpret_cast<unsigned long long*>(next));
    TDT_LAUNCH_CHECK("list_transpose");
    tr_check_kernel<<<g_e, 256, 0, st>>>(off, ne, cur, gate, status);
    TDT_LAUNCH_CHECK("list_transpose_check");
    return TDT_OK;
}

}  // namespace tdt
