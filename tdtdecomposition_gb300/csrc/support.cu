// Per-edge support (triangle count per edge) and per-edge triangle lists over
// the degree-oriented CSR.
//
// Replaces checkElementsTwoPtr / checkElementsTwoPtrTile (kernel.cu:28-141),
// which give every edge (u,v) one thread that merges N+(u) and N+(v) and adds
// +1 to (u,w), +1 to (v,w) and +count to (u,v) for every common w.
//
// Here the unit of work is the source vertex u of the triangle (u, v, w)
// (u -> v, u -> w, v -> w):
//   * N+(u) is staged once in shared memory (one warp for d+(u) <= warp_cap,
//     a whole block for larger rows; rows beyond the block buffer are searched
//     in place), with a bitmap of its hashed vertex ids;
//   * the wedges (v, w), v in N+(u), w in N+(v), form one flat index space
//     (the out-lists of a group of v's back to back: 32 v's for a warp, 512 for
//     a block).  A warp walks it 32 consecutive wedges per step (coalesced
//     loads of N+(v)); the owner v of each lane's wedge comes from one
//     OR-reduction of the group boundaries inside the step, not a search;
//   * w is tested against the bitmap; most wedges close no triangle and stop
//     there.  Candidates go to a per-warp queue in shared memory and are
//     resolved 32 at a time by binary search in N+(u) (full warps instead of a
//     few active lanes);
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
//              then role C.  This pass writes roles A and B (slots from the
//              row's counters in shared memory; both edges are in the source
//              row, so the stores stay in that row's list region); role C is
//              filled afterwards from the role-A lists (transpose.cu).
//   kSupStage  one walk for counts and lists: the role counts of kSupRoles,
//              and every triangle's role-A and role-B entries written into a
//              staging region per edge whose size is an upper bound known
//              before the walk (role A of (u,v), v = N+(u)[i]: at most
//              min(d+(u)-i-1, d+(v)); role B of (u,w), w = N+(u)[p]: at most
//              min(p, d-(w)-1)); a compaction pass then packs them into the
//              final lists.  Saves the second walk of kSupList.
#include "common.cuh"

namespace tdt {

constexpr int kSupBlock = 512;                 // 16 warps
constexpr int kSupWarps = kSupBlock / kWarp;
#ifndef TDT_SUP_MINB
#define TDT_SUP_MINB 3
#endif
constexpr int kSupMinBlocks = TDT_SUP_MINB;    // resident blocks per SM (3: registers <= 42)
constexpr int kSupSmemBytes = 64 * 1024;       // dynamic shared memory per block
constexpr int kVertexBatch = 2;                // light vertices per grab below the top quarter of ids
constexpr int kHeavyChunk = 16;                // vertices scanned per heavy grab
constexpr int kQueue = 64;                     // candidate queue entries per warp

// Light rows: one warp, a 4 KB slice of the block buffer:
//   su[256] | cnt[256] | group S[32] VI[32] BV[32] | bitmap 8192 bits | queue
constexpr int kWarpCap = 256;
constexpr int kSliceBytes = kSupSmemBytes / kSupWarps;
constexpr int kLightBmLog2 = 13;
constexpr int kSlSu = 0;
constexpr int kSlCnt = kSlSu + 4 * kWarpCap;
constexpr int kSlS = kSlCnt + 4 * kWarpCap;
constexpr int kSlVI = kSlS + 4 * kWarp;
constexpr int kSlBV = kSlVI + 4 * kWarp;
constexpr int kSlBm = kSlBV + 8 * kWarp;
constexpr int kSlQ = kSlBm + (1 << kLightBmLog2) / 8;
static_assert(kSlQ + 8 * kQueue <= kSliceBytes, "light slice");
// a push adds up to 32 candidates to a queue holding up to 31 (it is drained
// to below 32 after every push)
static_assert(kQueue >= 2 * kWarp, "candidate queue");
// the vectorised walk keeps a group as int4 {SC, BV, HI, VI} over S|VI|BV|HI
static_assert(kSlS % 16 == 0 && kSlVI == kSlS + 4 * kWarp && kSlBV == kSlVI + 4 * kWarp && kSlBm >= kSlS + 16 * kWarp,
              "light group layout");

// Heavy rows: one block, the whole buffer:
//   su[H] | cnt[H] | group S[512] VI[512] BV[512] | bitmap 2^16 bits | queues
// Rows longer than H are searched in place (su and counters in global memory)
// with a 2^18-bit bitmap over the su/cnt area.
constexpr int kSeg = kSupBlock;                // v's per heavy group (one per thread)
constexpr int kHeavyBmLog2 = 16;
constexpr int kHugeBmLog2 = 18;
constexpr int kHvQueues = kSupSmemBytes - kSupWarps * 8 * kQueue;
constexpr int kHvBm = kHvQueues - (1 << kHeavyBmLog2) / 8;
constexpr int kHvBV = kHvBm - 8 * kSeg;
constexpr int kHvVI = kHvBV - 4 * kSeg;
constexpr int kHvS = kHvVI - 4 * kSeg;
constexpr int kHeavyCap = kHvS / 8;            // su + cnt, 8 bytes per entry
static_assert(kHeavyCap >= 4096, "heavy cap");
static_assert(kHvS % 16 == 0 && kHvVI == kHvS + 4 * kSeg && kHvBV == kHvVI + 4 * kSeg && kHvBm >= kHvS + 16 * kSeg,
              "heavy group layout");
static_assert((1 << kHugeBmLog2) / 8 <= kHvS, "in-place bitmap");
static_assert(kHeavyCap < 65536, "packed 16-bit role counters");

enum SupMode { kSupAccum = 0, kSupRoles = 1, kSupList = 2, kSupStage = 3 };

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
    unsigned long long* curA_g;     // kSupList / kSupStage: global cursors for rows searched in place
    unsigned long long* curB_g;
    int2* lists;                    // kSupList: final lists; kSupStage: one past the end of the
                                    // staging area, which is indexed backwards (slot s at lists[-1-s])
    const int64_t* soff;            // kSupStage: staging offsets int64[E+1]
    const int32_t* bnd;             // kSupStage: role-A bound per edge (role-B region follows it)
    unsigned long long stage_cap;   // kSupStage: slots the staging area holds; no store at or past it
    const int* gate;                // non-zero: skip the pass
    int* status;                    // kSupList: set when a row's slots do not end where counted
    int bulk;                       // stage heavy rows by a bulk copy (needs kVec and a status word)
    int warp_cap;                   // rows with d+ <= warp_cap go to one warp (<= kWarpCap)
    int heavy_cap;                  // heavier rows staged in smem up to this size (<= kHeavyCap)
};

// Test hook: lower the light/heavy thresholds so small graphs drive every path
// (0 restores the defaults).
static int g_warp_cap = 0, g_heavy_cap = 0;
// Test hook: 0 forces the scalar wedge walk (the vectorised one is the default).
static int g_vec_walk = 1;
void set_vector_walk(int on) { g_vec_walk = on != 0; }
// Heavy rows staged by a bulk copy (1) or plain loads (0, the default).
static int g_bulk_stage = 0;
void set_bulk_staging(int on) { g_bulk_stage = on != 0; }
void set_support_caps(int warp_cap, int heavy_cap) {
    g_warp_cap = warp_cap;
    g_heavy_cap = heavy_cap;
}

struct SupCtl {
    unsigned long long heavy_next;
    unsigned long long light_next;
};

#ifndef TDT_BM_LOWBITS
#define TDT_BM_LOWBITS 1
#endif
// Bitmap index of vertex id w: its low bits (ids are degree ranks, and a
// row's out-neighbours cluster among the high ranks, so consecutive ids land
// on distinct bits), or a multiplicative hash.
__device__ __forceinline__ uint32_t bm_hash(int32_t w, int log2bits) {
    if (TDT_BM_LOWBITS) return (uint32_t)w & ((1u << log2bits) - 1u);
    return ((uint32_t)w * 0x9E3779B1u) >> (32 - log2bits);
}

// Binary search of key in s[lo, hi) (shared or global, generic address).
__device__ __forceinline__ int bsearch_i32(const int32_t* s, int lo, int hi, int32_t key) {
    int end = hi;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (s[mid] < key) lo = mid + 1; else hi = mid;
    }
    return (lo < end && s[lo] == key) ? lo : -1;
}

// One staged row.  packed: counters in shared memory, one 32-bit word per
// entry (accum: count; roles/list: role-A count in the low half, role-B count
// in the high half); otherwise the global per-edge arrays.
struct RowState {
    const int32_t* su;            // N+(u)
    uint32_t* cnt;
    const uint32_t* bm;           // bitmap of hashed N+(u)
    int bm_log2;
    int d;
    int32_t umax;                 // largest id in N+(u)
    bool packed;
    int64_t bu;                   // position of the row's first edge
};

// One triangle (u, v = su[i], w = su[p]) with (v,w) at position pos.
template <int M>
__device__ __forceinline__ void on_triangle(const RowState& R, const SupArgs& A, int i, int p, int64_t pos) {
    if (M == kSupAccum) {
        if (R.packed) {
            atomicAdd(R.cnt + i, 1u);
            atomicAdd(R.cnt + p, 1u);
        } else {
            atomicAdd(A.out + R.bu + i, 1);
            atomicAdd(A.out + R.bu + p, 1);
        }
        atomicAdd(A.out + pos, 1);
    } else if (M == kSupRoles) {
        if (R.packed) {
            atomicAdd(R.cnt + i, 1u);
            atomicAdd(R.cnt + p, 1u << 16);
        } else {
            atomicAdd(A.cA + R.bu + i, 1);
            atomicAdd(A.cB + R.bu + p, 1);
        }
        atomicAdd(A.cC + pos, 1);
    } else if (M == kSupStage) {
        const int32_t eA = (int32_t)(R.bu + i), eB = (int32_t)(R.bu + p), eC = (int32_t)pos;
        unsigned long long sA, sB;
        if (R.packed) {
            const uint32_t a = atomicAdd(R.cnt + i, 1u) & 0xffffu;
            const uint32_t b = atomicAdd(R.cnt + p, 1u << 16) >> 16;
            sA = (unsigned long long)__ldg(A.soff + eA) + a;
            sB = (unsigned long long)__ldg(A.soff + eB) + (unsigned long long)__ldg(A.bnd + eB) + b;
        } else {
            sA = atomicAdd(A.curA_g + eA, 1ull);
            sB = atomicAdd(A.curB_g + eB, 1ull);
        }
        // a count past its bound is caught per row in flush_row; this check
        // only keeps every store inside the staging area
        if (sA < A.stage_cap) A.lists[-1 - (long long)sA] = make_int2(eB, eC);
        if (sB < A.stage_cap) A.lists[-1 - (long long)sB] = make_int2(eA, eC);
        atomicAdd(A.cC + pos, 1);
    } else {
        const int32_t eA = (int32_t)(R.bu + i), eB = (int32_t)(R.bu + p), eC = (int32_t)pos;
        unsigned long long sA, sB;
        if (R.packed) {
            const uint32_t a = atomicAdd(R.cnt + i, 1u) & 0xffffu;
            const uint32_t b = atomicAdd(R.cnt + p, 1u << 16) >> 16;
            sA = (unsigned long long)__ldg(A.off + eA) + a;
            sB = (unsigned long long)__ldg(A.off + eB) + (unsigned long long)__ldg(A.cA_in + eB) + b;
        } else {
            sA = atomicAdd(A.curA_g + eA, 1ull);
            sB = atomicAdd(A.curB_g + eB, 1ull);
        }
        A.lists[sA] = make_int2(eB, eC);
        A.lists[sB] = make_int2(eA, eC);
    }
}

// Per-warp candidate queue: wedge position (the (v,w) edge) and v's index i.
struct WarpQueue {
    int32_t* pos;
    int32_t* vi;
    int n;                        // warp-uniform fill
};

// Resolve queue entries [0, cnt) (cnt <= 32), one per lane.
template <int M, bool kIdOrdered, class Off>
__device__ __forceinline__ void resolve(const OutRows<Off>& G, const SupArgs& A, const RowState& R,
                                        const WarpQueue& Q, int cnt) {
    const unsigned lane = lane_id();
    if ((int)lane < cnt) {
        const int32_t pos = Q.pos[lane];
        const int i = Q.vi[lane];
        const int32_t w = __ldg(G.cols + pos);
        const int p = bsearch_i32(R.su, kIdOrdered ? i + 1 : 0, R.d, w);
        if (p >= 0) on_triangle<M>(R, A, i, p, (int64_t)pos);
    }
}

// Positions in cols are int32: edge ids are int32 throughout (the whole-path
// calls reject E >= 2^31 and the drop-in operators take int32 row_ptr).
//
// Walk wedges [w0, w1) of a group: S[0..n) are the strictly increasing starts
// of the group's non-empty out-lists in the flat wedge space, BV their
// positions in cols, VI the index of their v in N+(u).  w0 is a multiple of
// 32 and o0 the group entry that holds wedge w0.
template <int M, bool kIdOrdered, class Off>
__device__ __forceinline__ void walk_group(const OutRows<Off>& G, const SupArgs& A, const RowState& R,
                                           const int32_t* S, const int32_t* VI, const int32_t* BV, int n, int w0, int w1,
                                           int o0, WarpQueue& Q) {
    const unsigned lane = lane_id();
    const unsigned lt = lanemask_lt();
    int ob = o0;
    for (int base = w0; base < w1; base += kWarp) {
        // group starts inside (base, base + 32): each is > base, and at most 31 fit
        const int k = ob + 1 + (int)lane;
        const int32_t B = k < n ? S[k] : INT32_MAX;
        const unsigned bit = ((unsigned)(B - base) < (unsigned)kWarp) ? (1u << (B - base)) : 0u;
        const unsigned mk = __reduce_or_sync(kFull, bit);
        const int nb = __popc(mk);
        const int32_t Bn = __shfl_sync(kFull, B, nb);
        const int t = base + (int)lane;
        bool cand = false;
        int32_t pos32 = 0;
        int vi = 0;
        if (t < w1) {
            const int o = ob + __popc(mk & (lt | (1u << lane)));
            const int32_t pos = BV[o] + (t - S[o]);
            const int32_t w = __ldg(G.cols + pos);
            if (w <= R.umax) {
                const uint32_t h = bm_hash(w, R.bm_log2);
                cand = (R.bm[h >> 5] >> (h & 31)) & 1u;
            }
            pos32 = (int32_t)pos;
            vi = VI[o];
        }
        ob += nb + (Bn == base + kWarp ? 1 : 0);
        const unsigned cm = __ballot_sync(kFull, cand);
        if (cm) {
            if (cand) {
                const int at = Q.n + __popc(cm & lt);
                Q.pos[at] = pos32;
                Q.vi[at] = vi;
            }
            Q.n += __popc(cm);
            if (Q.n >= kWarp) {
                __syncwarp();
                resolve<M, kIdOrdered>(G, A, R, Q, kWarp);
                __syncwarp();
                const int rest = Q.n - kWarp;
                int32_t p2 = 0, v2 = 0;
                if ((int)lane < rest) {
                    p2 = Q.pos[kWarp + lane];
                    v2 = Q.vi[kWarp + lane];
                }
                __syncwarp();
                if ((int)lane < rest) {
                    Q.pos[lane] = p2;
                    Q.vi[lane] = v2;
                }
                __syncwarp();
                Q.n = rest;
            }
        }
    }
}

// The same walk over 16-byte chunks of cols, four wedges per lane and step:
// each out-list N+(v) = cols[BV[k], HI[k]) is widened to the aligned chunks
// that hold it, so a chunk belongs to one v and comes with one int4 load; the
// widened ends are masked by [BV[k], HI[k]).  SC[0..n) are the strictly
// increasing chunk starts of the group's lists in the flat chunk space, c0 a
// multiple of 32 and o0 the group entry that holds chunk c0.  The group is
// one int4 per list, GE[k] = {SC[k], BV[k], HI[k], VI[k]}: a lane reads its
// list's entry with one shared-memory load.  One owner
// reduction serves 128 wedges instead of 32.  cols must be 16-byte aligned
// (a 16-byte chunk never crosses a page, so the widened reads stay mapped).
template <int M, bool kIdOrdered, class Off>
__device__ __forceinline__ void walk_group_vec(const OutRows<Off>& G, const SupArgs& A, const RowState& R,
                                               const int4* GE, int n, int c0, int c1, int o0, WarpQueue& Q) {
    const unsigned lane = lane_id();
    const unsigned lt = lanemask_lt();
    const int4* __restrict__ cols4 = reinterpret_cast<const int4*>(G.cols);
    int ob = o0;
    for (int base = c0; base < c1; base += kWarp) {
        const int k = ob + 1 + (int)lane;
        const int32_t B = k < n ? GE[k].x : INT32_MAX;
        const unsigned bit = ((unsigned)(B - base) < (unsigned)kWarp) ? (1u << (B - base)) : 0u;
        const unsigned mk = __reduce_or_sync(kFull, bit);
        const int nb = __popc(mk);
        const int32_t Bn = __shfl_sync(kFull, B, nb);
        const int c = base + (int)lane;
        unsigned cm = 0;
        int32_t p0 = 0;
        int vi = 0;
        if (c < c1) {
            const int o = ob + __popc(mk & (lt | (1u << lane)));
            const int4 ge = GE[o];
            const int32_t lo = ge.y, hi = ge.z;
            p0 = ((lo >> 2) + (c - ge.x)) << 2;
            const int4 w4 = __ldg(cols4 + (p0 >> 2));
            const int32_t wq[4] = {w4.x, w4.y, w4.z, w4.w};
            // the chunk's entries inside [lo, hi): a mask, once per chunk
            unsigned vm = 0xFu;
            if (p0 < lo) vm &= 0xFu << (lo - p0);
            if (p0 + 4 > hi) vm &= 0xFu >> (p0 + 4 - hi);
            // every entry is tested (a hashed index stays inside the bitmap)
            // and the mask applied after
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int32_t w = wq[q];
                const uint32_t h = bm_hash(w, R.bm_log2);
                const unsigned hit = (R.bm[h >> 5] >> (h & 31)) & (w <= R.umax ? 1u : 0u);
                cm |= hit << q;
            }
            cm &= vm;
            vi = ge.w;
        }
        ob += nb + (Bn == base + kWarp ? 1 : 0);
        if (__any_sync(kFull, cm != 0)) {
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const bool cand = (cm >> q) & 1u;
                const unsigned m = __ballot_sync(kFull, cand);
                if (m == 0) continue;
                if (cand) {
                    const int at = Q.n + __popc(m & lt);
                    Q.pos[at] = p0 + q;
                    Q.vi[at] = vi;
                }
                Q.n += __popc(m);
                if (Q.n >= kWarp) {
                    __syncwarp();
                    resolve<M, kIdOrdered>(G, A, R, Q, kWarp);
                    __syncwarp();
                    const int rest = Q.n - kWarp;
                    int32_t p2 = 0, v2 = 0;
                    if ((int)lane < rest) {
                        p2 = Q.pos[kWarp + lane];
                        v2 = Q.vi[kWarp + lane];
                    }
                    __syncwarp();
                    if ((int)lane < rest) {
                        Q.pos[lane] = p2;
                        Q.vi[lane] = v2;
                    }
                    __syncwarp();
                    Q.n = rest;
                }
            }
        }
    }
}

template <int M, bool kIdOrdered, class Off>
__device__ __forceinline__ void drain(const OutRows<Off>& G, const SupArgs& A, const RowState& R, WarpQueue& Q) {
    __syncwarp();
    if (Q.n > 0) resolve<M, kIdOrdered>(G, A, R, Q, Q.n);
    __syncwarp();
    Q.n = 0;
}

// Stage row u (d entries at bu).  in_smem: su and packed counters in the
// given buffers; otherwise the global arrays.  The bitmap (2^bm_log2 bits) is
// cleared and filled; block_sync selects block- or warp-wide synchronisation.
template <int M, class Off>
__device__ __forceinline__ RowState stage_row(const OutRows<Off>& G, const SupArgs& A, int32_t* su_buf,
                                              uint32_t* cnt_buf, uint32_t* bm, int bm_log2, bool in_smem, Off bu,
                                              int d, int tid, int nthr, bool block_sync) {
    RowState R;
    R.bu = bu;
    R.d = d;
    R.bm = bm;
    R.bm_log2 = bm_log2;
    R.packed = in_smem;
    for (int i = tid; i < (1 << bm_log2) / 32; i += nthr) bm[i] = 0u;
    if (block_sync) __syncthreads(); else __syncwarp();
    if (in_smem) {
        R.su = su_buf;
        R.cnt = cnt_buf;
        for (int i = tid; i < d; i += nthr) {
            const int32_t w = __ldg(G.cols + bu + i);
            su_buf[i] = w;
            cnt_buf[i] = 0u;
            const uint32_t h = bm_hash(w, bm_log2);
            atomicOr(bm + (h >> 5), 1u << (h & 31));
        }
    } else {
        R.su = G.cols + bu;
        R.cnt = nullptr;
        for (int i = tid; i < d; i += nthr) {
            const uint32_t h = bm_hash(__ldg(G.cols + bu + i), bm_log2);
            atomicOr(bm + (h >> 5), 1u << (h & 31));
        }
    }
    R.umax = d > 0 ? __ldg(G.cols + bu + d - 1) : INT32_MIN;
    return R;
}

// ---- heavy rows staged by one bulk copy (TMA, cp.async.bulk) ----------------
// A heavy row's middle part (the 16-byte aligned span of cols[bu, bu+d)) is
// copied into shared memory by one bulk copy that thread 0 issues and an
// mbarrier tracks; meanwhile the block clears the bitmap and counters and
// loads the ragged ends with plain loads.  The row buffer starts (bu mod 4)
// entries into its area so that su[i] and cols[bu + i] share their address
// mod 16 (the copy needs 16-byte aligned source and destination and a size in
// whole 16 bytes).  The wait is bounded: past kBulkWaitNs the block records
// TDT_ERR_TIMEOUT (the run's result is then rejected) and goes on.
// Off by default (tdt_set_bulk_staging): at R-MAT scale 22 the support phase
// took 65.1 ms with it against 63.7 ms with plain loads (the copy has to land
// before the bitmap is built, where plain loads overlap the two), a tie at
// scale 20.
constexpr uint64_t kBulkWaitNs = 2000000000ull;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Thread 0: order the block's earlier accesses of the buffer (made visible to
// it by the preceding __syncthreads) before the async proxy's writes, then
// expect `bytes` on the barrier and start the copy.
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned phase) {
    unsigned done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(phase)
        : "memory");
    return done != 0;
}

// Thread 0: wait for the copy of phase `phase` (bounded); true when it landed.
__device__ __noinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned phase) {
    const uint64_t t0 = globaltimer_ns();
    for (unsigned it = 1;; it++) {
        if (mbar_try_wait(bar, phase)) return true;
        if ((it & 63u) == 0 && globaltimer_ns() - t0 > kBulkWaitNs) return false;
    }
}

// Stage heavy row u (d entries at bu, d + 3 <= kHeavyCap) by a bulk copy;
// the same RowState as stage_row's in-shared-memory case.  Called by the
// whole block right after a __syncthreads.
template <int M, class Off>
__device__ __forceinline__ RowState stage_row_bulk(const OutRows<Off>& G, const SupArgs& A, int32_t* su_area,
                                                   uint32_t* cnt_buf, uint32_t* bm, int bm_log2, Off bu, int d,
                                                   uint64_t* bar, unsigned& phase) {
    RowState R;
    int32_t* su = su_area + (int)(bu & 3);
    const Off a0 = (bu + 3) & ~(Off)3, a1 = (bu + d) & ~(Off)3;
    const bool bulk = a1 > a0;
    if (threadIdx.x == 0 && bulk) bulk_copy_g2s(su + (a0 - bu), G.cols + a0, 4u * (unsigned)(a1 - a0), bar);
    for (int i = threadIdx.x; i < (1 << bm_log2) / 32; i += kSupBlock) bm[i] = 0u;
    for (int i = threadIdx.x; i < d; i += kSupBlock) {
        cnt_buf[i] = 0u;
        if (!bulk || i < (int)(a0 - bu) || i >= (int)(a1 - bu)) su[i] = __ldg(G.cols + bu + i);
    }
    if (threadIdx.x == 0 && bulk) {
        if (!mbar_wait_bounded(bar, phase) && A.status) atomicMax(A.status, (int)TDT_ERR_TIMEOUT);
        phase ^= 1u;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < d; i += kSupBlock) {
        const uint32_t h = bm_hash(su[i], bm_log2);
        atomicOr(bm + (h >> 5), 1u << (h & 31));
    }
    R.bu = bu;
    R.d = d;
    R.bm = bm;
    R.bm_log2 = bm_log2;
    R.packed = true;
    R.su = su;
    R.cnt = cnt_buf;
    R.umax = d > 0 ? __ldg(G.cols + bu + d - 1) : INT32_MIN;
    return R;
}

template <int M>
__device__ __forceinline__ void flush_row(const RowState& R, const SupArgs& A, int tid, int nthr) {
    const int d = R.d;
    if (M == kSupList) {
        // every role-A / role-B counter of the row must have reached its count:
        // the listing pass found exactly the triangles the support pass counted
        for (int i = tid; i < d; i += nthr) {
            const int64_t e = R.bu + i;
            const uint32_t ca = (uint32_t)__ldg(A.cA_in + e), cb = (uint32_t)__ldg(A.cB_in + e);
            bool bad;
            if (R.packed) {
                const uint32_t c = R.cnt[i];
                bad = (c & 0xffffu) != ca || (c >> 16) != cb;
            } else {
                const unsigned long long o = (unsigned long long)__ldg(A.off + e);
                bad = A.curA_g[e] != o + ca || A.curB_g[e] != o + ca + cb;
            }
            if (bad && A.status) atomicMax(A.status, (int)TDT_ERR_CAPACITY);
        }
        return;
    }
    if (M == kSupStage) {
        // role counts from the row's counters (or its cursors), each within
        // its staging bound
        for (int i = tid; i < d; i += nthr) {
            const int64_t e = R.bu + i;
            const unsigned long long o = (unsigned long long)__ldg(A.soff + e);
            const unsigned long long bA = (unsigned long long)__ldg(A.bnd + e);
            const unsigned long long bB = (unsigned long long)__ldg(A.soff + e + 1) - o - bA;
            unsigned long long ca, cb;
            if (R.packed) {
                const uint32_t c = R.cnt[i];
                ca = c & 0xffffu;
                cb = c >> 16;
            } else {
                ca = A.curA_g[e] - o;
                cb = A.curB_g[e] - o - bA;
            }
            A.cA[e] = (int32_t)ca;
            A.cB[e] = (int32_t)cb;
            if ((ca > bA || cb > bB) && A.status) atomicMax(A.status, (int)TDT_ERR_CAPACITY);
        }
        return;
    }
    if (!R.packed) return;
    if (M == kSupAccum) {
        for (int i = tid; i < d; i += nthr)
            if (R.cnt[i]) atomicAdd(A.out + R.bu + i, (int32_t)R.cnt[i]);
    } else {
        // role A/B counts of row u's edges come only from row u: plain stores
        for (int i = tid; i < d; i += nthr) {
            const uint32_t c = R.cnt[i];
            A.cA[R.bu + i] = (int32_t)(c & 0xffffu);
            A.cB[R.bu + i] = (int32_t)(c >> 16);
        }
    }
}

// ctl != nullptr: dynamic scheduling through its counters (zeroed by the
// caller); ctl == nullptr: static round-robin scheduling (no scratch at all).
// kVec: the wedge walk loads 16-byte chunks of cols (walk_group_vec).
template <int M, bool kIdOrdered, bool kVec, class Off>
__global__ void __launch_bounds__(kSupBlock, kSupMinBlocks) support_kernel(OutRows<Off> G, SupArgs A, SupCtl* ctl) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int32_t s_list[kHeavyChunk];
    __shared__ int32_t s_wsum[2][kSupWarps + 1];
    __shared__ int s_n;
    __shared__ long long s_chunk;
    __shared__ __align__(8) uint64_t s_bar;  // bulk copies of heavy rows
    const int wib = threadIdx.x / kWarp;
    const unsigned lane = lane_id();
    const int64_t nv = G.nv;
    const long long nchunks = (nv + kHeavyChunk - 1) / kHeavyChunk;
    if (A.gate && *(volatile const int*)A.gate != 0) return;
    const int warp_cap = A.warp_cap;
    const int heavy_cap = A.heavy_cap;

    // ---- phase 1: rows with d+(u) > warp_cap, one block per row
    {
        // bulk staging needs 16-byte aligned columns (kVec) and a status word
        // for a wait that runs out
        const bool bulk_ok = kVec && A.bulk && A.status != nullptr;
        unsigned phase = 0;
        if (threadIdx.x == 0 && bulk_ok) mbar_init(&s_bar, 1);  // first used after the next __syncthreads
        int32_t* h_su = reinterpret_cast<int32_t*>(smem);
        uint32_t* h_cnt = reinterpret_cast<uint32_t*>(smem + 4 * kHeavyCap);
        int32_t* g_S = reinterpret_cast<int32_t*>(smem + kHvS);
        int32_t* g_VI = reinterpret_cast<int32_t*>(smem + kHvVI);
        int32_t* g_BV = reinterpret_cast<int32_t*>(smem + kHvBV);
        int32_t* g_HI = g_BV + kSeg;  // list ends (the vectorised walk)
        int4* g_GE = reinterpret_cast<int4*>(smem + kHvS);  // the vectorised walk's layout of the same area
        WarpQueue Q;
        Q.pos = reinterpret_cast<int32_t*>(smem + kHvQueues + wib * 8 * kQueue);
        Q.vi = Q.pos + kQueue;
        Q.n = 0;
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
                uint32_t* bm = in_smem ? reinterpret_cast<uint32_t*>(smem + kHvBm) : reinterpret_cast<uint32_t*>(smem);
                RowState R = (bulk_ok && in_smem && d + 3 <= kHeavyCap)
                                 ? stage_row_bulk<M>(G, A, h_su, h_cnt, bm, kHeavyBmLog2, bu, d, &s_bar, phase)
                                 : stage_row<M>(G, A, h_su, h_cnt, bm, in_smem ? kHeavyBmLog2 : kHugeBmLog2, in_smem,
                                                bu, d, threadIdx.x, kSupBlock, true);
                __syncthreads();
                const int vend = kIdOrdered ? d - 1 : d;
                for (int g0 = 0; g0 < vend; g0 += kSeg) {
                    // group: v's g0 .. g0+511, one per thread
                    const int i = g0 + threadIdx.x;
                    int32_t len = 0;
                    int32_t bv = 0;
                    if (i < vend) {
                        const int32_t v = R.su[i];
                        if (v >= 0 && v < nv) {
                            bv = (int32_t)G.begin(v);
                            len = (int32_t)(G.end(v) - bv);
                        }
                    }
                    // work units of the walk: wedges, or 16-byte chunks of cols
                    const int32_t units = kVec ? (len > 0 ? ((bv + len + 3) >> 2) - (bv >> 2) : 0) : len;
                    const unsigned nem = __ballot_sync(kFull, len > 0);
                    const int32_t incl = warp_incl_scan(units);
                    if (lane == 31) {
                        s_wsum[0][wib] = incl;
                        s_wsum[1][wib] = __popc(nem);
                    }
                    __syncthreads();
                    if (wib == 0) {
                        const int32_t x = (int)lane < kSupWarps ? s_wsum[0][lane] : 0;
                        const int32_t y = (int)lane < kSupWarps ? s_wsum[1][lane] : 0;
                        const int32_t xi = warp_incl_scan(x), yi = warp_incl_scan(y);
                        if ((int)lane < kSupWarps) {
                            s_wsum[0][lane] = xi - x;
                            s_wsum[1][lane] = yi - y;
                        }
                        if ((int)lane == kSupWarps - 1) {
                            s_wsum[0][kSupWarps] = xi;
                            s_wsum[1][kSupWarps] = yi;
                        }
                    }
                    __syncthreads();
                    if (len > 0) {
                        const int ci = s_wsum[1][wib] + __popc(nem & lanemask_lt());
                        if (kVec) {
                            g_GE[ci] = make_int4(s_wsum[0][wib] + incl - units, bv, bv + len, i);
                        } else {
                            g_S[ci] = s_wsum[0][wib] + incl - units;
                            g_VI[ci] = i;
                            g_BV[ci] = bv;
                            g_HI[ci] = bv + len;
                        }
                    }
                    const int total = s_wsum[0][kSupWarps];
                    const int n = s_wsum[1][kSupWarps];
                    __syncthreads();
                    // equal shares of the group's wedges, in whole steps of 32
                    const int share = ((total + kSupBlock - 1) / kSupBlock) * kWarp;
                    const int w0 = wib * share;
                    const int w1 = w0 + share < total ? w0 + share : total;
                    if (w0 < w1) {
                        int o0 = 0;
                        if (lane == 0) {
                            int lo = 0, hi = n - 1;  // last entry with S <= w0
                            while (lo < hi) {
                                const int mid = (lo + hi + 1) >> 1;
                                if ((kVec ? g_GE[mid].x : g_S[mid]) <= w0) lo = mid; else hi = mid - 1;
                            }
                            o0 = lo;
                        }
                        o0 = __shfl_sync(kFull, o0, 0);
                        if (kVec) walk_group_vec<M, kIdOrdered>(G, A, R, g_GE, n, w0, w1, o0, Q);
                        else walk_group<M, kIdOrdered>(G, A, R, g_S, g_VI, g_BV, n, w0, w1, o0, Q);
                    }
                    __syncthreads();  // the group arrays are rewritten next
                }
                drain<M, kIdOrdered>(G, A, R, Q);
                __syncthreads();
                flush_row<M>(R, A, threadIdx.x, kSupBlock);
                __syncthreads();
            }
        }
    }

    // ---- phase 2: rows with 2 <= d+(u) <= warp_cap, one warp per row, taken
    // in batches from the top ids (highest degree rank) down
    unsigned char* sl = smem + wib * kSliceBytes;
    int32_t* l_su = reinterpret_cast<int32_t*>(sl + kSlSu);
    uint32_t* l_cnt = reinterpret_cast<uint32_t*>(sl + kSlCnt);
    int32_t* l_S = reinterpret_cast<int32_t*>(sl + kSlS);
    int32_t* l_VI = reinterpret_cast<int32_t*>(sl + kSlVI);
    int32_t* l_BV = reinterpret_cast<int32_t*>(sl + kSlBV);
    int32_t* l_HI = l_BV + kWarp;  // list ends (the vectorised walk)
    int4* l_GE = reinterpret_cast<int4*>(sl + kSlS);  // the vectorised walk's layout of the same area
    uint32_t* l_bm = reinterpret_cast<uint32_t*>(sl + kSlBm);
    WarpQueue Q;
    Q.pos = reinterpret_cast<int32_t*>(sl + kSlQ);
    Q.vi = Q.pos + kQueue;
    Q.n = 0;
    const long long gw = (long long)blockIdx.x * kSupWarps + wib;
    const long long nw = (long long)gridDim.x * kSupWarps;
    // rows are taken from the top id down: the top quarter of the ids (the
    // rows whose out-neighbours have the longest lists) one row per grab, the
    // rest kVertexBatch rows per grab, so no warp is left with a long batch
    // while the others idle
    const unsigned long long t1 = ((unsigned long long)nv + 3) / 4;
    for (long long it = 0;; it++) {
        unsigned long long t = 0;
        if (ctl) {
            if (lane == 0) t = atomicAdd(&ctl->light_next, 1ull);
            t = __shfl_sync(kFull, t, 0);
        } else {
            t = (unsigned long long)(gw + it * nw);
        }
        const unsigned long long b = t < t1 ? t : t1 + (t - t1) * kVertexBatch;
        const int nq = t < t1 ? 1 : kVertexBatch;
        if ((long long)b >= nv) break;
        for (int q = 0; q < nq; q++) {
            const long long uu = nv - 1 - ((long long)b + q);
            if (uu < 0) break;
            const Off bu = G.begin(uu);
            const int d = (int)(G.end(uu) - bu);
            if (d < 2 || d > warp_cap) continue;
            RowState R = stage_row<M>(G, A, l_su, l_cnt, l_bm, kLightBmLog2, true, bu, d, lane, kWarp, false);
            __syncwarp();
            const int vend = kIdOrdered ? d - 1 : d;
            for (int vb = 0; vb < vend; vb += kWarp) {
                const int i = vb + (int)lane;
                int32_t len = 0;
                int32_t bv = 0;
                if (i < vend) {
                    const int32_t v = l_su[i];
                    if (v >= 0 && v < nv) {
                        bv = (int32_t)G.begin(v);
                        len = (int32_t)(G.end(v) - bv);
                    }
                }
                const int32_t units = kVec ? (len > 0 ? ((bv + len + 3) >> 2) - (bv >> 2) : 0) : len;
                const unsigned nem = __ballot_sync(kFull, len > 0);
                const int32_t incl = warp_incl_scan(units);
                const int total = __shfl_sync(kFull, incl, 31);
                if (len > 0) {
                    const int ci = __popc(nem & lanemask_lt());
                    if (kVec) {
                        l_GE[ci] = make_int4(incl - units, bv, bv + len, i);
                    } else {
                        l_S[ci] = incl - units;
                        l_VI[ci] = i;
                        l_BV[ci] = bv;
                        l_HI[ci] = bv + len;
                    }
                }
                __syncwarp();
                if (total > 0) {
                    if (kVec) walk_group_vec<M, kIdOrdered>(G, A, R, l_GE, __popc(nem), 0, total, 0, Q);
                    else walk_group<M, kIdOrdered>(G, A, R, l_S, l_VI, l_BV, __popc(nem), 0, total, 0, Q);
                }
                __syncwarp();
            }
            drain<M, kIdOrdered>(G, A, R, Q);
            flush_row<M>(R, A, lane, kWarp);
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
    A2.warp_cap = (g_warp_cap > 0 && g_warp_cap < kWarpCap) ? g_warp_cap : kWarpCap;
    A2.heavy_cap = (g_heavy_cap > 0 && g_heavy_cap < kHeavyCap) ? g_heavy_cap : kHeavyCap;
    A2.bulk = g_bulk_stage;
    // the vectorised walk needs 16-byte aligned columns (chunk positions stay
    // below 2^31 under 2^30 edges)
    const bool vec = g_vec_walk && ((uintptr_t)G.cols & 15u) == 0 && G.ne < (1ll << 30);
    auto kern = vec ? support_kernel<M, kIdOrdered, true, Off> : support_kernel<M, kIdOrdered, false, Off>;
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

// Whole-path count-only walk: role counts.  cA/cB are stored per row (by
// atomics for rows searched in place), cC accumulated by atomics: the caller
// zeroes all three first.
int launch_support_roles(const int64_t* rp, const int32_t* cols, int64_t nv, int64_t ne, int32_t* cA, int32_t* cB,
                         int32_t* cC, void* ctl, const int* gate, int* status, cudaStream_t st) {
    if (nv <= 0) return TDT_OK;
    OutRows<int64_t> G{rp, 1, cols, nv, ne};
    SupArgs A{};
    A.cA = cA;
    A.cB = cB;
    A.cC = cC;
    A.gate = gate;
    A.status = status;
    return launch_mode<kSupRoles, true, int64_t>(G, A, reinterpret_cast<SupCtl*>(ctl), st);
}

// Whole-path pass 2: triangle lists (skipped on the device when *gate != 0).
int launch_support_list(const int64_t* rp, const int32_t* cols, int64_t nv, int64_t ne, const int64_t* off,
                        const int32_t* cA, const int32_t* cB, unsigned long long* curA_g, unsigned long long* curB_g,
                        int2* lists, void* ctl, const int* gate, int* status, cudaStream_t st) {
    if (nv <= 0) return TDT_OK;
    OutRows<int64_t> G{rp, 1, cols, nv, ne};
    SupArgs A{};
    A.off = off;
    A.cA_in = cA;
    A.cB_in = cB;
    A.curA_g = curA_g;
    A.curB_g = curB_g;
    A.lists = lists;
    A.gate = gate;
    A.status = status;
    return launch_mode<kSupList, true, int64_t>(G, A, reinterpret_cast<SupCtl*>(ctl), st);
}

// Whole-path one-walk pass: role counts (cA, cB stored per row, cC by
// atomics: the caller zeroes cC first) and the role-A/B entries of every
// triangle in the staging regions (skipped on the device when *gate != 0).
int launch_support_stage(const int64_t* rp, const int32_t* cols, int64_t nv, int64_t ne, const int64_t* soff,
                         const int32_t* bnd, int32_t* cA, int32_t* cB, int32_t* cC, unsigned long long* curA_g,
                         unsigned long long* curB_g, int2* stage_end, unsigned long long stage_slots, void* ctl,
                         const int* gate, int* status, cudaStream_t st) {
    if (nv <= 0) return TDT_OK;
    OutRows<int64_t> G{rp, 1, cols, nv, ne};
    SupArgs A{};
    A.cA = cA;
    A.cB = cB;
    A.cC = cC;
    A.soff = soff;
    A.bnd = bnd;
    A.curA_g = curA_g;
    A.curB_g = curB_g;
    A.lists = stage_end;
    A.gate = gate;
    A.status = status;
    A.stage_cap = stage_slots;
    return launch_mode<kSupStage, true, int64_t>(G, A, reinterpret_cast<SupCtl*>(ctl), st);
}

size_t support_ctl_bytes() { return 256; }

}  // namespace tdt
