// Device-resident truss decomposition and k-truss search.
//
// Replaces the `--cuda` flow's Python peel loop (singlegpu_truss.py:67-158:
// ~12 torch launches and ~6 host syncs per sub-round, each O(E)) by ONE
// persistent cooperative kernel that runs every sub-round and level on the
// device, separated by a bounded grid barrier.
//
// Per sub-round r at level l, F_r = edges peeled in r (rnd[e] == r):
//   * every e in F_r enumerates its triangles from the endpoint x of lower
//     degree: the candidates are x's out- and in-neighbours w; the third edge
//     between w and the other endpoint y is found by binary search in the
//     sorted out-list of min(w, y) (ids are degree ranks, so that list is
//     short);
//   * a triangle (e, f, g) whose edges were all alive at the start of r is
//     destroyed; f and g outside F_r lose one support each; when f (or g) is
//     also in F_r only the member with the smaller index decrements the third
//     edge; when all three are in F_r nothing is decremented;
//   * an edge whose support drops from l+1 to l joins F_{r+1}.
// When F_{r+1} is empty, the level advances to the minimum support of the
// alive edges and F_{r+1} = alive edges with that support.
// This yields exactly the reference's sub-round sets (singlegpu_truss.py:
// 99-152 with sub_AllAffectedSupport_tilenot, kernel.cu:492-547): each
// non-peeled edge loses one support per destroyed triangle, and an edge
// joins the next sub-round exactly when its support reaches <= l; so
// truss[e] = level + 2 and the reference's e_truss order (sub-rounds in
// order, ascending edge index within a sub-round) are reproduced exactly.
//
// Work in a sub-round is a flat candidate space: each queued edge owns
// deg(x) consecutive candidate slots (reserved with one packed 64-bit atomic
// per warp: item count in the high bits, candidate count in the low bits, so
// item order equals slot order), and every lane of the grid takes one slot
// per step.  Hub edges therefore spread over all SMs instead of one thread.
// With per-edge triangle lists (listed mode) a slot is one list entry: the
// two partner edges, whose states come from 4-bit round codes held in L2.
#include "common.cuh"
#include "sort.cuh"

namespace tdt {

#ifndef TDT_PEEL_BLOCK
#define TDT_PEEL_BLOCK 512
#endif
constexpr int kPeelBlock = TDT_PEEL_BLOCK;
constexpr int kPeelWarps = kPeelBlock / kWarp;
constexpr int kItemBits = 28;
constexpr int kCandBits = 36;
constexpr unsigned long long kCandMask = (1ull << kCandBits) - 1ull;
// Wall-clock budget of one persistent peel launch; past it the run stops with
// TDT_ERR_TIMEOUT instead of holding the GPU.
constexpr uint64_t kPeelDeadlineNs = 120ull * 1000ull * 1000ull * 1000ull;

struct PeelCtl {
    GridCtl g;
    // round r's counters live at r & 3: round r reads slot r, appends to r+1,
    // sets the dead bits of round r-1's edges, and the top of round r clears r+2
    unsigned long long q[4];      // packed (items << kCandBits | candidates) per round slot
    unsigned long long fe[4];     // frontier edges per round slot (queued or not)
    unsigned long long cnt[3];     // survivors written by level change t, at t % 3
    unsigned long long pfe[3];     // edges queued by level-change pass k, at k % 3
    int mgt[3];                    // minimum support found by level-change pass k, at k % 3
    int dmin[2];                   // minimum decrement result above the level during level L_t, at t & 1
    long long passes;              // level-change passes run (diagnostic)
    int listed;                   // 1: per-edge triangle lists were built (they fit the workspace)
    int list_skip;                // gate of the role-C transpose (no lists)
    int rewalk_skip;              // gate of the second walk (lists written by kSupList)
    int compact_skip;             // gate of the staging compaction (lists from the one-walk pass)
    int stage_skip;               // gate of the one-walk pass (kSupStage)
    int roles_skip;               // gate of the count-only walk (kSupRoles)
    int pad0[2];
    long long rounds;
    long long triangles;
    unsigned long long alive;
    // block 0's time (ns) in candidate processing, grid-barrier waits after
    // processing, and level transitions; diagnostic only
    unsigned long long t_proc, t_wait, t_trans, t_total;
    unsigned long long grab[4];    // slot cursor of search-mode sub-round r, at r & 3
};

struct PeelArgs {
    const int64_t* rp;
    const int32_t* cols;
    const int32_t* rows;
    const int64_t* cp;
    const int32_t* in_src;
    const int32_t* in_eid;
    int32_t* live;        // support of each edge, decremented as its triangles are destroyed
    int32_t* rnd;         // sub-round that peeled each edge (-1: alive)
    int32_t* round_level;
    // queue of round r in buffer r % 3: round r reads r, appends r+1, and the
    // items of round r-1 stay intact for the dead bits set during round r
    int4* qi[3];
    long long* qb[3];
    int32_t* alive[2];    // compacted alive-edge lists (level transitions)
    // bit e set: edge e was peeled in a sub-round before the current one (a
    // filter in L2 before the state checks, used only in builds without the
    // round codes; a bit not set yet only costs the check it would have saved)
    unsigned* dead;
    // round code of edge e in the 4 bits at (e & 7) * 4 of word e >> 3 (the
    // listed peel's partner-state check; see code_round)
    unsigned* code;
    const int64_t* off;   // listed mode: list offsets int64[E+1]
    const int2* lists;    // listed mode: partner edge pairs
    int64_t V, E, round_cap;
    int32_t mode;         // 0: full decomposition, 1: fixed-level peel (k-truss search)
    int32_t fixed_level;
    unsigned long long deadline_ns;  // wall-clock budget of the launch
    unsigned long long fixed_item_cap, fixed_cand_cap;  // k-truss collection batch limits
    long long dyn_min_slots;      // search mode: sub-rounds of at least this many slots take dynamic ranges
    PeelCtl* ctl;
};

__device__ __forceinline__ void set_status(PeelCtl* c, int s) {
    atomicMax(&c->g.status, s);
    grid_abort(&c->g);
}

__device__ __forceinline__ unsigned long long ld_cg_u64(const unsigned long long* p) {
    return __ldcg(p);
}

// Round codes: 4 bits per edge, 32 MB at 64 M edges, so they stay in L2.
// 0xF: never marked (alive); 0-3: marked for sub-round y, stored as y & 3;
// bit 3 set: peeled and done.  A code is set once, when its edge is marked
// (0xF -> y & 3, one atomicAnd), and turned dead during sub-round y + 1 with
// the dead bits of that round's items (atomicOr 0x8).  An edge marked without
// an item (no triangle left to enumerate) is dead at once: each of its
// triangles is already destroyed by a partner peeled before it.  Hence, in
// sub-round r (a grid barrier after every sub-round), a code reads 0xF
// alive, r & 3 peeling in r, (r + 1) & 3 marked for r + 1, and anything else
// peeled before r (an edge of r - 1 may still carry (r + 3) & 3).
constexpr unsigned kCodeAlive = 0xFu, kCodeDead = 0x8u;

__device__ __forceinline__ void code_mark(unsigned* code, int32_t e, unsigned c) {
    atomicAnd(code + (e >> 3), ~((kCodeAlive ^ c) << ((unsigned)(e & 7) * 4u)));
}

// The sub-round stamp of edge e read from its code word in sub-round r: -1
// alive, r or r + 1, or -2 for peeled before r.
__device__ __forceinline__ int32_t code_round(unsigned word, int32_t e, int r) {
    const unsigned c = (word >> ((unsigned)(e & 7) * 4u)) & 15u;
    if (c == kCodeAlive) return -1;
    if (c == ((unsigned)r & 3u)) return r;
    if (c == ((unsigned)(r + 1) & 3u)) return r + 1;
    return -2;
}

// Queue item of edge e (listed: e's list offset and length; search: the
// lower-degree endpoint x, the other endpoint y, x's out-degree dxo and the
// candidate count dx).  Returns false when e has nothing to enumerate.
template <bool Listed>
__device__ __forceinline__ bool make_item(const PeelArgs& A, bool want, int32_t cur_sup, int32_t e, int4& it,
                                          long long& dx) {
    it = make_int4(e, 0, 0, 0);
    dx = 0;
    if (!want || cur_sup <= 0) return false;
    if (Listed) {
        // the edge's original triangles; the item carries the list offset
        const long long o = __ldg(A.off + e);
        dx = __ldg(A.off + e + 1) - o;
        it.y = (int32_t)(unsigned)(o & 0xffffffffll);
        it.z = (int32_t)(o >> 32);
        return dx > 0;
    }
    const int32_t u = __ldg(A.rows + e), v = __ldg(A.cols + e);
    const long long duo = __ldg(A.rp + u + 1) - __ldg(A.rp + u);
    const long long du = duo + __ldg(A.cp + u + 1) - __ldg(A.cp + u);
    const long long dvo = __ldg(A.rp + v + 1) - __ldg(A.rp + v);
    const long long dv = dvo + __ldg(A.cp + v + 1) - __ldg(A.cp + v);
    if (du <= dv) { it.y = u; it.z = v; dx = du; it.w = (int32_t)duo; }
    else { it.y = v; it.z = u; dx = dv; it.w = (int32_t)dvo; }
    return dx > 1;
}

// Reserve n items and tot candidate slots of the round in `slot` (lane 0's
// atomic, broadcast); sets TDT_ERR_CAPACITY past the queue limits.
__device__ __forceinline__ unsigned long long reserve_items(const PeelArgs& A, int slot, int n, long long tot) {
    unsigned long long old = 0;
    if (lane_id() == 0) {
        old = atomicAdd(&A.ctl->q[slot], ((unsigned long long)n << kCandBits) + (unsigned long long)tot);
        const unsigned long long it0 = old >> kCandBits, c0 = old & kCandMask;
        if (it0 + n >= (1ull << kItemBits) || c0 + tot >= (1ull << kCandBits) || (long long)(it0 + n) > A.E)
            set_status(A.ctl, TDT_ERR_CAPACITY);
    }
    return __shfl_sync(kFull, old, 0);
}

// Appends of the listed sub-rounds and of the level changes are staged per
// warp in shared memory (edge ids only, 256 bytes a warp, so the carveout
// leaves L1 its room) and queued in batches: one queue atomic (and one
// frontier-count atomic) per flush instead of two per warp step that marks an
// edge, which keeps the reservation's round trip and the contention on the
// round's counters out of most steps.  The items are built at the flush.  The
// queue order of items changes nothing: a sub-round is a set.
#ifndef TDT_APPEND_BUF
#define TDT_APPEND_BUF 64
#endif
constexpr int kAppBuf = TDT_APPEND_BUF;  // entries per warp; a flush leaves room for one 64-edge append
static_assert(kAppBuf >= 64 && kAppBuf % 32 == 0, "append buffer");

struct AppendBuf {
    int32_t* e;                  // this warp's staged edges (shared memory)
    int n;                       // staged edges (warp-uniform)
    unsigned long long nfront;   // edges marked since the last flush (warp-uniform)
};

// Queue the staged edges: their items are built here (kAppBuf / 32 per lane),
// reserved with one atomic and written.
template <bool Listed>
__device__ __forceinline__ void append_flush(const PeelArgs& A, int slot, int buf, AppendBuf& B,
                                             unsigned long long* nfront) {
    const unsigned lane = lane_id();
    __syncwarp();
    if (B.nfront) {
        if (lane == 0) atomicAdd(nfront, B.nfront);
        B.nfront = 0;
    }
    if (B.n > 0) {
        constexpr int kPer = kAppBuf / kWarp;
        int4 it[kPer];
        long long dx[kPer];
        bool q[kPer];
        int nq = 0;
        long long sum = 0;
#pragma unroll
        for (int k = 0; k < kPer; k++) {
            const int i = (int)lane * kPer + k;
            q[k] = i < B.n && make_item<Listed>(A, true, 1, B.e[i], it[k], dx[k]);
            if (q[k]) {
                nq++;
                sum += dx[k];
            }
        }
        const int nincl = warp_incl_scan(nq);
        const int ntot = __shfl_sync(kFull, nincl, 31);
        const long long cincl = warp_incl_scan(sum);
        const long long ctot = __shfl_sync(kFull, cincl, 31);
        if (ntot > 0) {
            const unsigned long long old = reserve_items(A, slot, ntot, ctot);
            long long idx = (long long)(old >> kCandBits) + nincl - nq;
            long long cc = (long long)(old & kCandMask) + cincl - sum;
#pragma unroll
            for (int k = 0; k < kPer; k++) {
                if (q[k]) {
                    if (idx < A.E) {
                        A.qi[buf][idx] = it[k];
                        A.qb[buf][idx] = cc;
                    }
                    idx++;
                    cc += dx[k];
                }
            }
        }
        B.n = 0;
    }
    __syncwarp();
}

// The same as a call (the level-change passes: several call sites, rare flushes).
template <bool Listed>
__device__ __noinline__ void append_flush_call(const PeelArgs& A, int slot, int buf, AppendBuf& B,
                                               unsigned long long* nfront) {
    append_flush<Listed>(A, slot, buf, B, nfront);
}

// Stage up to two edges per lane (f, g of one triangle) for the round in
// `slot`; cur_sup (the level, warp-uniform) <= 0 queues no item.
template <bool Listed>
__device__ __forceinline__ void warp_append2_staged(const PeelArgs& A, int slot, int buf, bool wf, int32_t f,
                                                    bool wg, int32_t g, int32_t cur_sup, AppendBuf& B,
                                                    unsigned long long* nfront) {
    const unsigned mf = __ballot_sync(kFull, wf), mg = __ballot_sync(kFull, wg);
    if ((mf | mg) == 0) return;
    B.nfront += (unsigned long long)(__popc(mf) + __popc(mg));
    if (cur_sup <= 0) return;
    const int nq = (wf ? 1 : 0) + (wg ? 1 : 0);
    const int nincl = warp_incl_scan(nq);
    const int ntot = __shfl_sync(kFull, nincl, 31);
    if (B.n + ntot > kAppBuf) append_flush<Listed>(A, slot, buf, B, nfront);
    int p = B.n + nincl - nq;
    if (wf) B.e[p++] = f;
    if (wg) B.e[p] = g;
    B.n += ntot;
}

// Queue up to two edges per lane directly, with one reservation per warp step
// (the search-mode sub-rounds: their steps are long and append rarely, and the
// staging state would stay live across the binary searches).
template <bool Listed>
__device__ __forceinline__ void warp_append2_direct(const PeelArgs& A, int slot, int buf, bool wf, int32_t f,
                                                    bool wg, int32_t g, int32_t cur_sup,
                                                    unsigned long long* nfront) {
    const unsigned lane = lane_id();
    const unsigned mf = __ballot_sync(kFull, wf), mg = __ballot_sync(kFull, wg);
    if ((mf | mg) == 0) return;
    if (lane == 0) atomicAdd(nfront, (unsigned long long)(__popc(mf) + __popc(mg)));
    int4 itf, itg;
    long long dxf, dxg;
    const bool qf = make_item<Listed>(A, wf, cur_sup, f, itf, dxf);
    const bool qg = make_item<Listed>(A, wg, cur_sup, g, itg, dxg);
    const int nq = (qf ? 1 : 0) + (qg ? 1 : 0);
    if (__ballot_sync(kFull, nq > 0) == 0) return;
    const long long c = (qf ? dxf : 0) + (qg ? dxg : 0);
    const int nincl = warp_incl_scan(nq);
    const long long cincl = warp_incl_scan(c);
    const int ntot = __shfl_sync(kFull, nincl, 31);
    const long long ctot = __shfl_sync(kFull, cincl, 31);
    const unsigned long long old = reserve_items(A, slot, ntot, ctot);
    long long idx = (long long)(old >> kCandBits) + nincl - nq;
    long long cc = (long long)(old & kCandMask) + cincl - c;
    if (qf) {
        if (idx < A.E) {
            A.qi[buf][idx] = itf;
            A.qb[buf][idx] = cc;
        }
        idx++;
        cc += dxf;
    }
    if (qg && idx < A.E) {
        A.qi[buf][idx] = itg;
        A.qb[buf][idx] = cc;
    }
}

// Stage the edges flagged by `want` (one per lane) for the round in `slot`.
// cur_sup is the edge's support at marking time (0 => no alive triangle).
__device__ __forceinline__ void warp_append_staged(const PeelArgs& A, bool listed, int slot, int buf, bool want,
                                                   int32_t e, int32_t cur_sup, AppendBuf& B,
                                                   unsigned long long* nfront) {
    const unsigned mf = __ballot_sync(kFull, want);
    if (mf == 0) return;
    B.nfront += (unsigned long long)__popc(mf);
    const bool st = want && cur_sup > 0;
    const unsigned m = __ballot_sync(kFull, st);
    if (m == 0) return;
    const int ntot = __popc(m);
    if (B.n + ntot > kAppBuf) {
        if (listed) append_flush_call<true>(A, slot, buf, B, nfront);
        else append_flush_call<false>(A, slot, buf, B, nfront);
    }
    if (st) B.e[B.n + __popc(m & lanemask_lt())] = e;
    B.n += ntot;
}

// Level changes (decomposition mode).  Level change t starts level L_t =
// min support over the alive edges and queues F = alive edges with support
// L_t.  The alive edges live in a compacted list (list t&1 is the input of
// change t, all edge ids at t = 0).
//
// One streaming pass usually suffices: a lower bound g of L_t is known before
// the pass (0 at t = 0; afterwards the minimum support above L_{t-1} seen at
// change t-1, lowered by every decrement result above L_{t-1} during level
// L_{t-1}).  The pass compacts the survivors into list (t+1)&1, queues the
// alive edges with support == g, and takes the minimum support above g.  If
// anything was queued, L_t = g.  Otherwise L_t = that minimum, and one more
// pass over the compacted list queues its frontier (3 of 307 level changes
// at R-MAT scale 22; a side list of the supports just above g, written by
// every first pass for that case, cost the level changes 3 ms there).  Every
// pass k ends with a grid barrier and writes its minimum and queued count to
// slot k % 3 of mgt / pfe; the block-0 thread that clears slot (k+1) % 3 at
// the start of pass k clears a slot that every block finished reading before
// the barrier of pass k-1.

// Fold a per-lane minimum into *dst: one atomic per warp, skipped when *dst
// is already no larger (a plain read keeps ten thousand warps from
// serialising on one address).
__device__ __forceinline__ void fold_min(int* dst, int32_t v) {
    v = warp_min(v);
    if (lane_id() == 0 && v != INT32_MAX && v < *(volatile int*)dst) atomicMin(dst, v);
}

__device__ __forceinline__ void pass_min(const PeelArgs& A, int np, int32_t v) { fold_min(&A.ctl->mgt[np % 3], v); }

// Level-change passes stream the alive list in steps of kStep x 32 entries per
// warp: the gathers of a step are in flight together and the step reserves its
// output ranges with one atomic each.
#ifndef TDT_DYN_CHUNK
#define TDT_DYN_CHUNK 256
#endif
#ifndef TDT_DYN_MIN_LOG2
#define TDT_DYN_MIN_LOG2 20
#endif
constexpr long long kDynChunk = TDT_DYN_CHUNK;  // 0: static ranges in search mode too
constexpr int kDynMinLog2 = TDT_DYN_MIN_LOG2;
static_assert(kDynChunk % 64 == 0, "dynamic ranges are whole 64-slot steps");
// An edge already marked for sub-round r+1 (support <= l) is not decremented
// again: its support no longer decides anything (it is peeled next sub-round,
// and its truss number is the level).
#ifndef TDT_SKIP_MARKED
#define TDT_SKIP_MARKED 1
#endif
constexpr bool kSkipMarked = TDT_SKIP_MARKED != 0;
// The 1-bit dead-edge filter before the edge-state loads of a slot.
#ifndef TDT_DEAD_FILTER
#define TDT_DEAD_FILTER 1
#endif
constexpr bool kDeadFilter = TDT_DEAD_FILTER != 0;

// The decrement results of a peel step are used one step later, after the
// next step's loads are in flight (0: used at once).
#ifndef TDT_PEEL_DEFER
#define TDT_PEEL_DEFER 1
#endif
constexpr bool kPeelDefer = TDT_PEEL_DEFER != 0;

// The listed peel reads its partners' round codes instead of the dead bits
// and the edge states (0: dead bits, then edge states).
#ifndef TDT_PEEL_CODES
#define TDT_PEEL_CODES 1
#endif
constexpr bool kPeelCodes = TDT_PEEL_CODES != 0;

#ifndef TDT_PEEL_STEP
#define TDT_PEEL_STEP 8
#endif
constexpr int kStep = TDT_PEEL_STEP;

__device__ __forceinline__ void pass_start(const PeelArgs& A, int np) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        A.ctl->mgt[(np + 1) % 3] = INT32_MAX;
        A.ctl->pfe[(np + 1) % 3] = 0;
        A.ctl->passes++;
    }
}

__device__ __forceinline__ bool level_transition(const PeelArgs& A, bool listed, int r_next, int t, int& np,
                                              int32_t* l_out, int32_t* app_e) {
    const unsigned lane = lane_id();
    const long long gw = (long long)blockIdx.x * kPeelWarps + threadIdx.x / kWarp;
    const long long nw = (long long)gridDim.x * kPeelWarps;
    const int p = t & 1;
    const bool first = t == 0;
    const int32_t* cur = A.alive[p];
    int32_t* nxt = A.alive[p ^ 1];
    const long long ncur = first ? A.E : (long long)__ldcg(&A.ctl->cnt[(t + 2) % 3]);
    int32_t g = 0;
    if (!first) {
        const int32_t a = *(volatile int*)&A.ctl->mgt[(np + 2) % 3];
        const int32_t b = *(volatile int*)&A.ctl->dmin[(t + 1) & 1];
        g = a < b ? a : b;
    }
    const int slot = r_next & 3, buf = r_next % 3;
    AppendBuf B{app_e + (threadIdx.x / kWarp) * kAppBuf, 0, 0ull};
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        A.ctl->cnt[(t + 1) % 3] = 0;
        A.ctl->dmin[t & 1] = INT32_MAX;
    }
    pass_start(A, np);
    // pass 1: compact, queue support == g, minimum above g.  Blocks take
    // tiles of kPeelWarps x kStep x 32 entries; each tile reserves its
    // survivor range with one atomic.
    {
        __shared__ int s_tk[kPeelWarps];
        __shared__ unsigned long long s_base;
        constexpr long long kTile = (long long)kPeelWarps * kStep * kWarp;
        const int wib = threadIdx.x / kWarp;
        int32_t mloc = INT32_MAX;
        unsigned long long* ocnt = &A.ctl->cnt[t % 3];
        const unsigned lt = lanemask_lt();
        for (long long tb = (long long)blockIdx.x * kTile; tb < ncur; tb += (long long)gridDim.x * kTile) {
            const long long base = tb + (long long)wib * (kStep * kWarp);
            int32_t e[kStep], sv[kStep];
            bool keep[kStep];
#pragma unroll
            for (int u = 0; u < kStep; u++) {
                const long long i = base + u * kWarp + lane;
                e[u] = 0;
                if (i < ncur) e[u] = first ? (int32_t)i : __ldcg(cur + i);
            }
#pragma unroll
            for (int u = 0; u < kStep; u++) {
                const long long i = base + u * kWarp + lane;
                keep[u] = false;
                sv[u] = 0;
                if (i < ncur) {
                    // alive = never marked (its round code, in L2); the
                    // support is a 4-byte gather
                    const unsigned cw = __ldcg(A.code + (e[u] >> 3));
                    sv[u] = __ldcg(A.live + e[u]);
                    keep[u] = ((cw >> ((unsigned)(e[u] & 7) * 4u)) & 15u) == kCodeAlive;
                }
            }
            unsigned km[kStep];
            int nk = 0;
#pragma unroll
            for (int u = 0; u < kStep; u++) {
                km[u] = __ballot_sync(kFull, keep[u]);
                nk += __popc(km[u]);
                if (keep[u] && sv[u] > g) mloc = sv[u] < mloc ? sv[u] : mloc;
            }
            if (lane == 0) s_tk[wib] = nk;
            __syncthreads();
            if (wib == 0) {
                const int a = lane < kPeelWarps ? s_tk[lane] : 0;
                const int ai = warp_incl_scan(a);
                if (lane == kPeelWarps - 1) s_base = ai ? atomicAdd(ocnt, (unsigned long long)ai) : 0ull;
                if (lane < kPeelWarps) s_tk[lane] = ai - a;
            }
            __syncthreads();
            unsigned long long ok = s_base + (unsigned long long)s_tk[wib];
#pragma unroll
            for (int u = 0; u < kStep; u++) {
                if (keep[u]) nxt[ok + __popc(km[u] & lt)] = e[u];
                ok += __popc(km[u]);
                const bool want = keep[u] && sv[u] == g;
                if (want) {
                    A.rnd[e[u]] = r_next;
                    code_mark(A.code, e[u], sv[u] > 0 ? ((unsigned)r_next & 3u) : kCodeDead);
                }
                warp_append_staged(A, listed, slot, buf, want, e[u], sv[u], B, &A.ctl->pfe[np % 3]);
            }
            __syncthreads();  // s_tk / s_base are reused by the next tile
        }
        if (listed) append_flush_call<true>(A, slot, buf, B, &A.ctl->pfe[np % 3]);
        else append_flush_call<false>(A, slot, buf, B, &A.ctl->pfe[np % 3]);
        pass_min(A, np, mloc);
    }
    np++;
    if (!grid_barrier(&A.ctl->g, gridDim.x)) return false;
    if (ld_cg_u64(&A.ctl->pfe[(np + 2) % 3]) > 0) {
        *l_out = g;
        return true;
    }
    const int32_t m = *(volatile int*)&A.ctl->mgt[(np + 2) % 3];
    if (m == INT32_MAX) return false;  // no edge is alive
    *l_out = m;
    pass_start(A, np);
    int32_t mloc = INT32_MAX;
    {
        // pass 2: one more pass over the compacted list
        const long long n2 = (long long)__ldcg(&A.ctl->cnt[t % 3]);
        for (long long base = gw * kWarp; base < n2; base += nw * kWarp) {
            const long long i = base + lane;
            int32_t e = 0, sv = INT32_MAX;
            if (i < n2) {
                e = __ldcg(nxt + i);
                sv = __ldcg(A.live + e);
            }
            const bool want = i < n2 && sv == m;
            if (!want && sv > m) mloc = sv < mloc ? sv : mloc;
            if (want) {
                A.rnd[e] = r_next;
                code_mark(A.code, e, sv > 0 ? ((unsigned)r_next & 3u) : kCodeDead);
            }
            warp_append_staged(A, listed, slot, buf, want, e, sv, B, &A.ctl->pfe[np % 3]);
        }
    }
    if (listed) append_flush_call<true>(A, slot, buf, B, &A.ctl->pfe[np % 3]);
    else append_flush_call<false>(A, slot, buf, B, &A.ctl->pfe[np % 3]);
    pass_min(A, np, mloc);
    np++;
    return grid_barrier(&A.ctl->g, gridDim.x);
}

// k-truss search (fixed level l): the frontier is every alive edge with
// support <= l, collected in batches.  A collection pass queues such edges
// while the round's queue stays under fixed_item_cap items and fixed_cand_cap
// candidate slots (by default far below the packed counter's limits, which
// leaves room for warps that read the count before others added to it);
// edges left out stay alive and are taken by the next pass, which runs
// whenever a sub-round queues nothing.  The k-truss does not depend on how the
// peel is split into rounds, so the batches change no result; they keep the
// rounds of graphs whose low-support edges outnumber the queue within it.
constexpr unsigned long long kFixedItemCap = 1ull << 27;
constexpr unsigned long long kFixedCandCap = 1ull << 35;

__device__ __forceinline__ void warp_append_capped(const PeelArgs& A, bool listed, int slot, int buf, bool want,
                                                   int32_t e,
                                                   int32_t s, int r_next, unsigned long long* nfront) {
    const unsigned lane = lane_id();
    if (__ballot_sync(kFull, want) == 0) return;
    int4 it;
    long long dx;
    const bool q = listed ? make_item<true>(A, want, s, e, it, dx) : make_item<false>(A, want, s, e, it, dx);
    const unsigned m = __ballot_sync(kFull, q);
    const long long c = q ? dx : 0;
    const long long incl = warp_incl_scan(c);
    const long long tot = __shfl_sync(kFull, incl, 31);
    const int n = __popc(m);
    int ok = 1;
    unsigned long long old = 0;
    if (lane == 0 && n > 0) {
        const unsigned long long cur = ld_cg_u64(&A.ctl->q[slot]);
        // a batch always takes something (an empty queue accepts any warp)
        if (cur != 0 && ((cur >> kCandBits) + (unsigned long long)n > A.fixed_item_cap ||
                         (cur & kCandMask) + (unsigned long long)tot > A.fixed_cand_cap)) {
            ok = 0;
        } else {
            old = atomicAdd(&A.ctl->q[slot], ((unsigned long long)n << kCandBits) + (unsigned long long)tot);
            const unsigned long long it0 = old >> kCandBits, c0 = old & kCandMask;
            if (it0 + n >= (1ull << kItemBits) || c0 + tot >= (1ull << kCandBits) || (long long)(it0 + n) > A.E)
                set_status(A.ctl, TDT_ERR_CAPACITY);
        }
    }
    ok = __shfl_sync(kFull, ok, 0);
    old = __shfl_sync(kFull, old, 0);
    // edges without candidates use no queue space and are always taken
    const bool acc = want && (!q || ok);
    if (acc) {
        A.rnd[e] = r_next;
        code_mark(A.code, e, q ? ((unsigned)r_next & 3u) : kCodeDead);
    }
    const unsigned ma = __ballot_sync(kFull, acc);
    if (lane == 0 && ma) atomicAdd(nfront, (unsigned long long)__popc(ma));
    if (q && ok) {
        const long long idx = (long long)(old >> kCandBits) + __popc(m & lanemask_lt());
        if (idx < A.E) {
            A.qi[buf][idx] = it;
            A.qb[buf][idx] = (long long)(old & kCandMask) + incl - c;
        }
    }
}

// One collection pass for sub-round r_next; true when it took an edge.
__device__ bool fixed_collect(const PeelArgs& A, bool listed, int32_t l, int r_next, int& np) {
    const unsigned lane = lane_id();
    const int64_t nthreads = (int64_t)gridDim.x * blockDim.x;
    const int slot = r_next & 3, buf = r_next % 3;
    pass_start(A, np);
    for (int64_t base = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) & ~31ll; base < A.E;
         base += nthreads) {
        const int64_t e = base + lane;
        bool want = false;
        int32_t s = 0;
        if (e < A.E) {
            const unsigned cw = __ldcg(A.code + (e >> 3));
            s = __ldcg(A.live + e);
            want = ((cw >> ((unsigned)(e & 7) * 4u)) & 15u) == kCodeAlive && s <= l;
        }
        warp_append_capped(A, listed, slot, buf, want, (int32_t)e, s, r_next, &A.ctl->pfe[np % 3]);
    }
    np++;
    if (!grid_barrier(&A.ctl->g, gridDim.x)) return false;
    return ld_cg_u64(&A.ctl->pfe[(np + 2) % 3]) > 0;
}

// Item windows: slot cb lies in item i0 (first slot base0); items i0+1.. start
// at strictly increasing slots, all > cb, so at most 31 start inside
// (cb, cb+32).  One OR-reduction gives every lane the item of slot cb+lane.
struct Window {
    int k;              // this lane's item is i0 + k
    long long base_l;   // first slot of that item
    long long i0n;      // item of slot cb+32
    long long base0n;   // its first slot
    long long nsn;      // first slot of item i0n + 1 (-1: not among the loaded starts)
    bool starts_next;   // item i0n starts at cb+32 (no lane of this window holds it)
};

__device__ __forceinline__ Window locate(const long long* __restrict__ qb, long long N, long long i0,
                                         long long base0, long long cb, unsigned le) {
    const unsigned lane = lane_id();
    const long long B = (i0 + 1 + lane < N) ? __ldcg(qb + i0 + 1 + lane) : LLONG_MAX;
    const unsigned bit = (B - cb < kWarp) ? (1u << (unsigned)(B - cb)) : 0u;
    const unsigned mk = __reduce_or_sync(kFull, bit);
    Window w;
    w.k = __popc(mk & le);
    const long long Bk = __shfl_sync(kFull, B, (w.k + 31) & 31);
    w.base_l = w.k == 0 ? base0 : Bk;
    const int nb = __popc(mk);
    const long long Bn = __shfl_sync(kFull, B, nb);
    const long long Bl = __shfl_sync(kFull, B, (nb + 31) & 31);
    const long long B2 = __shfl_sync(kFull, B, (nb + 1) & 31);
    w.starts_next = Bn == cb + kWarp;
    if (w.starts_next) {
        w.i0n = i0 + nb + 1;
        w.base0n = Bn;
        w.nsn = nb + 1 < kWarp ? B2 : -1;
    } else {
        w.i0n = i0 + nb;
        w.base0n = nb > 0 ? Bl : base0;
        w.nsn = nb < kWarp ? Bn : -1;
    }
    return w;
}

// The items of one window [cb, cb + 32) of a warp's range: this lane's item
// record and first slot.  The warp keeps its current item i0 (holding slot
// cb, or ending just before it when item i0 + 1 starts at cb; locate handles
// both), that item's first slot, the first slot of the next item (nst, -1 when
// unknown) and the item's record (rec, valid when rv): a window that lies
// wholly in item i0 -- most windows, since most slots belong to long lists --
// needs no load at all; otherwise one locate step and one record load per
// lane, which also refresh the state.
__device__ __forceinline__ void window_items(const long long* __restrict__ qb, const int4* __restrict__ qi,
                                             long long N, long long cb, bool valid, unsigned le, long long& i0,
                                             long long& base0, long long& nst, int4& rec, bool& rv, int4& it,
                                             long long& base_l) {
    if (nst >= cb + kWarp) {
        if (!rv) {
            rec = __ldcg(qi + i0);
            rv = true;
        }
        it = rec;
        base_l = base0;
        return;
    }
    const Window w = locate(qb, N, i0, base0, cb, le);
    it = make_int4(0, 0, 0, 0);
    if (valid) it = __ldcg(qi + i0 + w.k);
    base_l = w.base_l;
    // lane 31 holds item i0n unless that item starts at cb + 32 (or lane 31
    // lies past the range)
    const bool v31 = (__ballot_sync(kFull, valid) >> 31) != 0u;
    rec.x = __shfl_sync(kFull, it.x, 31);
    rec.y = __shfl_sync(kFull, it.y, 31);
    rec.z = __shfl_sync(kFull, it.z, 31);
    rec.w = __shfl_sync(kFull, it.w, 31);
    rv = v31 && !w.starts_next;
    i0 = w.i0n;
    base0 = w.base0n;
    nst = w.nsn;
}

// The other two edges (f, g) of slot tl of item it; false when the slot is
// not a triangle (search mode only).
template <bool Listed>
__device__ __forceinline__ bool slot_edges(const PeelArgs& A, const int4& it, long long tl, int r, int32_t& f,
                                           int32_t& g) {
    if (Listed) {
        const long long lo = (long long)(unsigned)it.y | ((long long)it.z << 32);
        const int2 fg = __ldg(A.lists + lo + tl);
        f = fg.x;
        g = fg.y;
        return true;
    }
    const int32_t x = it.y, y = it.z, dxo = it.w;
    int32_t w;
    if (tl < dxo) {
        f = (int32_t)(__ldg(A.rp + x) + tl);
        w = __ldg(A.cols + f);
    } else {
        const int64_t kk = __ldg(A.cp + x) + (tl - dxo);
        w = __ldg(A.in_src + kk);
        f = __ldg(A.in_eid + kk);
    }
    if (w == y) return false;
    if (kPeelCodes) {
        // no search when (x,w) was peeled before this round, or peels in it
        // too with the smaller index: then the other edge of the triangle is
        // decremented from (x,w)'s own slot, not from this one
        const int32_t cf = code_round(__ldcg(A.code + (f >> 3)), f, r);
        if (cf == -2 || (cf == r && it.x > f)) return false;
    } else if (kDeadFilter && ((A.dead[f >> 5] >> (f & 31)) & 1u)) {
        return false;  // (x,w) peeled before this round
    }
    const int64_t gg = (w < y) ? find_sorted<int64_t>(A.cols, __ldg(A.rp + w), __ldg(A.rp + w + 1), y)
                               : find_sorted<int64_t>(A.cols, __ldg(A.rp + y), __ldg(A.rp + y + 1), w);
    g = (int32_t)gg;
    return gg >= 0;
}

// The decrements of one peel step: the four edges and the supports before
// their decrements (INT32_MIN: no decrement).  An edge whose support fell to
// l is marked for sub-round r+1 and queued; a larger result lowers the bound
// dm of the next level.
#ifndef TDT_PEEL_WIN
#define TDT_PEEL_WIN 2
#endif
constexpr int kWin = TDT_PEEL_WIN;  // 32-slot windows per peel step
struct Pending {
    int32_t e[2 * kWin];
    int32_t o[2 * kWin];
};

template <bool Listed>
__device__ __forceinline__ void settle(const PeelArgs& A, const Pending& P, int r, int32_t l, int nslot, int nbuf,
                                       AppendBuf& B, int32_t& dm) {
    bool w[2 * kWin];
    // queued with an item when the level is above 0 (an edge without
    // triangles never appears in a list, so its code is never read)
    const unsigned cm = l > 0 ? ((unsigned)(r + 1) & 3u) : kCodeDead;
#pragma unroll
    for (int j = 0; j < 2 * kWin; j++) {
        w[j] = P.o[j] == l + 1;
        if (P.o[j] > l + 1) dm = P.o[j] - 1 < dm ? P.o[j] - 1 : dm;
        if (w[j]) {
            A.rnd[P.e[j]] = r + 1;
            code_mark(A.code, P.e[j], cm);
        }
    }
#pragma unroll
    for (int h = 0; h < kWin; h++) {
        if (Listed)
            warp_append2_staged<Listed>(A, nslot, nbuf, w[2 * h], P.e[2 * h], w[2 * h + 1], P.e[2 * h + 1], l, B,
                                        &A.ctl->fe[nslot]);
        else
            warp_append2_direct<Listed>(A, nslot, nbuf, w[2 * h], P.e[2 * h], w[2 * h + 1], P.e[2 * h + 1], l,
                                        &A.ctl->fe[nslot]);
    }
}

// One sub-round: warps gwarp = 0..nwarps-1 share the candidate slots of round r.
// The smallest decrement result above l is folded into *dmin (the lower bound
// of the next level).  Each step covers two 32-slot windows whose loads and
// decrements are in flight together.  Inlined into the persistent loop (with
// the level changes): the kernel arguments are a __grid_constant__ parameter,
// so no call passes a local copy of them, and no call frame is saved around
// every sub-round.
template <bool Listed>
__device__ __forceinline__ void process_round(const PeelArgs& A, int r, int32_t l, long long gwarp, long long nwarps,
                                           int* dmin, int32_t* app_e) {
    const unsigned lane = lane_id();
    const unsigned le = lanemask_lt() | (1u << lane);
    int32_t dm = INT32_MAX;
    const int slot = r & 3, buf = r % 3;
    const int nslot = (r + 1) & 3, nbuf = (r + 1) % 3;
    const int wib = threadIdx.x / kWarp;
    AppendBuf B{app_e + wib * kAppBuf, 0, 0ull};
    const unsigned long long packed = ld_cg_u64(&A.ctl->q[slot]);
    const long long N = (long long)(packed >> kCandBits);
    const long long T = (long long)(packed & kCandMask);
    const long long* __restrict__ qb = A.qb[buf];
    const int4* __restrict__ qi = A.qi[buf];
    // the edges of round r-1 are dead from this round on: their round codes
    // turn dead (needed by round r+2, where (r-1) & 3 would read "marked for
    // the next round"), or, without the codes, their dead bits are set (a bit
    // read before it is set only sends that triangle to the state check)
    if ((kPeelCodes || kDeadFilter) && r > 0) {
        long long nprev = (long long)(ld_cg_u64(&A.ctl->q[(r - 1) & 3]) >> kCandBits);
        if (nprev > A.E) nprev = A.E;
        const int4* __restrict__ qp = A.qi[(r - 1) % 3];
        for (long long i = gwarp * kWarp + lane; i < nprev; i += nwarps * kWarp) {
            const int32_t e = __ldcg(&qp[i].x);
            if (kPeelCodes) atomicOr(A.code + (e >> 3), kCodeDead << ((unsigned)(e & 7) * 4u));
            else atomicOr(A.dead + (e >> 5), 1u << (e & 31));
        }
    }
    // listed mode: each warp owns a contiguous range of candidate slots (a
    // multiple of 64).  Search mode with many slots: warps take ranges of
    // kDynChunk slots from a shared cursor (the binary search of a slot costs
    // from one load to twenty, so equal ranges finish far apart).
    const bool dyn = !Listed && kDynChunk > 0 && T >= A.dyn_min_slots;
    constexpr long long kStepSlots = (long long)kWin * kWarp;
    const long long per_warp = (((T + nwarps - 1) / nwarps) + kStepSlots - 1) / kStepSlots * kStepSlots;
    long long cb0 = gwarp * per_warp;
    long long cb1 = cb0 + per_warp < T ? cb0 + per_warp : T;
    if (!dyn && cb0 >= cb1) return;
    Pending P;
#pragma unroll
    for (int j = 0; j < 2 * kWin; j++) {
        P.e[j] = 0;
        P.o[j] = INT32_MIN;
    }
    for (;;) {
    if (dyn) {
        unsigned long long c = 0;
        if (lane == 0) c = atomicAdd(&A.ctl->grab[slot], (unsigned long long)kDynChunk);
        cb0 = (long long)__shfl_sync(kFull, c, 0);
        if (cb0 >= T) break;
        cb1 = cb0 + kDynChunk < T ? cb0 + kDynChunk : T;
    }
    // item of slot cb0 = last i with qb[i] <= cb0: a 32-way search, each step
    // one load per lane (log32 N dependent loads instead of log2 N)
    long long i0 = 0;
    {
        long long lo = 0, hi = N;  // answer in [lo, hi)
        while (hi - lo > 1) {
            const long long step = (hi - lo + kWarp - 1) / kWarp;
            const long long p = lo + (long long)lane * step;
            const bool le_ = p < hi && __ldcg(qb + p) <= cb0;
            const unsigned m = __ballot_sync(kFull, le_);
            const int j = 31 - __clz(m);  // qb[lo] <= cb0 always holds, so m != 0
            lo += (long long)j * step;
            hi = lo + step < hi ? lo + step : hi;
        }
        i0 = lo;
    }
    long long base0 = __ldcg(qb + i0);
    long long nst = i0 + 1 < N ? __ldcg(qb + i0 + 1) : LLONG_MAX;
    int4 rec = __ldcg(qi + i0);
    bool rv = true;
    for (long long cb = cb0; cb < cb1; cb += kStepSlots) {
        int4 it[kWin];
        long long bl[kWin];
        bool v[kWin];
#pragma unroll
        for (int h = 0; h < kWin; h++) {
            const long long cbh = cb + h * kWarp;
            it[h] = make_int4(0, 0, 0, 0);
            bl[h] = 0;
            v[h] = cbh + lane < cb1;
            if (cbh < cb1) window_items(qb, qi, N, cbh, v[h], le, i0, base0, nst, rec, rv, it[h], bl[h]);
        }
        int32_t f[kWin], g[kWin];
        bool tr[kWin];
#pragma unroll
        for (int h = 0; h < kWin; h++) {
            f[h] = 0;
            g[h] = 0;
            tr[h] = false;
            if (v[h]) tr[h] = slot_edges<Listed>(A, it[h], cb + h * kWarp + lane - bl[h], r, f[h], g[h]);
        }
        int32_t rf[kWin], rg[kWin];
#pragma unroll
        for (int h = 0; h < kWin; h++) rf[h] = rg[h] = -2;
        if (kPeelCodes) {
            // the partners' round codes (L2): dead, alive, peeling now, marked
            unsigned x[kWin], y[kWin];
#pragma unroll
            for (int h = 0; h < kWin; h++) {
                x[h] = y[h] = 0;
                if (tr[h]) {
                    x[h] = __ldcg(A.code + (f[h] >> 3));
                    y[h] = __ldcg(A.code + (g[h] >> 3));
                }
            }
            // the previous step's decrement results, while these loads are in flight
            if (kPeelDefer) settle<Listed>(A, P, r, l, nslot, nbuf, B, dm);
#pragma unroll
            for (int h = 0; h < kWin; h++) {
                if (tr[h]) {
                    rf[h] = code_round(x[h], f[h], r);
                    rg[h] = code_round(y[h], g[h], r);
                }
            }
        } else {
            // dead-bit filter: a triangle with an edge peeled before round r is gone
            if (kDeadFilter) {
                unsigned x[kWin], y[kWin];
#pragma unroll
                for (int h = 0; h < kWin; h++) {
                    x[h] = y[h] = 0;
                    if (tr[h]) {
                        x[h] = A.dead[f[h] >> 5];
                        y[h] = A.dead[g[h] >> 5];
                    }
                }
#pragma unroll
                for (int h = 0; h < kWin; h++)
                    if (tr[h] && (((x[h] >> (f[h] & 31)) | (y[h] >> (g[h] & 31))) & 1u)) tr[h] = false;
            }
#pragma unroll
            for (int h = 0; h < kWin; h++) {
                if (tr[h]) {
                    rf[h] = __ldcg(A.rnd + f[h]);
                    rg[h] = __ldcg(A.rnd + g[h]);
                }
            }
            // the previous step's decrement results, while these loads are in flight
            if (kPeelDefer) settle<Listed>(A, P, r, l, nslot, nbuf, B, dm);
        }
        // a triangle is alive when both other edges are alive or peel in r or r+1;
        // which of f, g this lane decrements: the ownership rules above
        bool df[kWin], dg[kWin];
#pragma unroll
        for (int h = 0; h < kWin; h++) {
            df[h] = dg[h] = false;
            if (tr[h] && (rf[h] == -1 || rf[h] >= r) && (rg[h] == -1 || rg[h] >= r)) {
                const bool ff = rf[h] == r, fg = rg[h] == r;
                df[h] = !ff && (!fg || it[h].x < g[h]) && (!kSkipMarked || rf[h] != r + 1);
                dg[h] = !fg && (!ff || it[h].x < f[h]) && (!kSkipMarked || rg[h] != r + 1);
            }
        }
        // issue all decrements; their results are used by the next step
#pragma unroll
        for (int h = 0; h < kWin; h++) {
            P.e[2 * h] = f[h];
            P.e[2 * h + 1] = g[h];
        }
#pragma unroll
        for (int h = 0; h < kWin; h++) {
            P.o[2 * h] = df[h] ? atomicSub(A.live + f[h], 1) : INT32_MIN;
            P.o[2 * h + 1] = dg[h] ? atomicSub(A.live + g[h], 1) : INT32_MIN;
        }
        if (!kPeelDefer) {
            settle<Listed>(A, P, r, l, nslot, nbuf, B, dm);
#pragma unroll
            for (int j = 0; j < 2 * kWin; j++) P.o[j] = INT32_MIN;
        }
    }
    if (!dyn) break;
    }
    if (kPeelDefer) settle<Listed>(A, P, r, l, nslot, nbuf, B, dm);
    if (Listed) append_flush<Listed>(A, nslot, nbuf, B, &A.ctl->fe[nslot]);
    fold_min(dmin, dm);
}

#ifndef TDT_PEEL_MINB
#define TDT_PEEL_MINB 2
#endif
// A is a __grid_constant__ parameter: the helpers take it by reference and
// read its fields from the parameter bank instead of a local copy.
__global__ void __launch_bounds__(kPeelBlock, TDT_PEEL_MINB) peel_kernel(const __grid_constant__ PeelArgs A) {
    __shared__ int32_t s_app_e[kPeelWarps * kAppBuf];  // per-warp append staging
    const bool listed = A.lists != nullptr && *(volatile int*)&A.ctl->listed != 0;
    const int wib = threadIdx.x / kWarp;
    const int64_t gwarp = (int64_t)blockIdx.x * kPeelWarps + wib;
    const int64_t nwarps = (int64_t)gridDim.x * kPeelWarps;
    const bool master = blockIdx.x == 0 && threadIdx.x == 0;

    if (*(volatile int*)&A.ctl->g.status != 0) return;  // invalid input was detected
    const uint64_t t_start = globaltimer_ns();
    int r = 0;
    int32_t l = 0;
    int ntrans = 0, np = 0;
    bool ok;
    if (A.mode == 0) {
        ok = level_transition(A, listed, 0, ntrans++, np, &l, s_app_e);
    } else {
        l = A.fixed_level;
        ok = fixed_collect(A, listed, l, 0, np);
    }
    if (!ok) {
        if (master) A.ctl->rounds = 0;
        return;
    }
    uint64_t t_mark = globaltimer_ns();
    for (;;) {
        if (master) {
            A.round_level[r] = l;
            A.ctl->q[(r + 2) & 3] = 0;
            A.ctl->fe[(r + 2) & 3] = 0;
            A.ctl->grab[(r + 2) & 3] = 0;
            if (globaltimer_ns() - t_start > A.deadline_ns) set_status(A.ctl, TDT_ERR_TIMEOUT);
        }
        // level L_t (t = ntrans - 1) folds its decrement results into dmin[t & 1]
        if (listed) process_round<true>(A, r, l, gwarp, nwarps, &A.ctl->dmin[(ntrans + 1) & 1], s_app_e);
        else process_round<false>(A, r, l, gwarp, nwarps, &A.ctl->dmin[(ntrans + 1) & 1], s_app_e);
        __syncthreads();
        const uint64_t t_p = globaltimer_ns();
        if (!grid_barrier(&A.ctl->g, gridDim.x)) return;
        const uint64_t t_b = globaltimer_ns();
        if (master) {
            A.ctl->t_proc += t_p - t_mark;
            A.ctl->t_wait += t_b - t_p;
        }
        if (r + 2 >= A.round_cap) {
            if (master) set_status(A.ctl, TDT_ERR_CAPACITY);
            return;
        }
        // fe[(r+1) & 3] is only written by sub-round r (level changes count
        // into pfe), and cleared again at the top of sub-round r+3
        if (ld_cg_u64(&A.ctl->fe[(r + 1) & 3]) == 0) {
            if (A.mode != 0) {
                // k-truss search: the next batch of low-support edges, if any
                if (!fixed_collect(A, listed, l, r + 1, np)) break;
                t_mark = globaltimer_ns();
                r++;
                continue;
            }
            int32_t nl;
            const bool more = level_transition(A, listed, r + 1, ntrans++, np, &nl, s_app_e);
            if (master) A.ctl->t_trans += globaltimer_ns() - t_b;
            if (!more) break;
            l = nl;
        }
        t_mark = globaltimer_ns();
        r++;
    }
    if (master) {
        A.ctl->rounds = r + 1;
        A.ctl->t_total = globaltimer_ns() - t_start;
    }
}

// ------------------------------------------------------------------ setup / output kernels
__global__ void rows_from_rp_kernel(const int64_t* __restrict__ rp, int64_t V, int32_t* __restrict__ rows) {
    const unsigned lane = lane_id();
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t u = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; u < V; u += nw) {
        const int64_t b = rp[u], e = rp[u + 1];
        for (int64_t i = b + lane; i < e; i += kWarp) rows[i] = (int32_t)u;
    }
}

// Input validation, before any kernel indexes through the graph:
// row_ptr[0] == 0, row_ptr[V] == E, non-decreasing; rows[e] is the row that
// owns position e; u < v < V; columns strictly increasing within a row.
__global__ void validate_kernel(const int64_t* __restrict__ rp, const int32_t* __restrict__ rows,
                                const int32_t* __restrict__ cols, int64_t E, int64_t V, PeelCtl* ctl) {
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t nth = (int64_t)gridDim.x * blockDim.x;
    if (tid == 0 && (rp[0] != 0 || rp[V] != E)) atomicMax(&ctl->g.status, (int)TDT_ERR_INVALID);
    for (int64_t u = tid; u < V; u += nth)
        if (rp[u] > rp[u + 1]) atomicMax(&ctl->g.status, (int)TDT_ERR_INVALID);
    for (int64_t e = tid; e < E; e += nth) {
        const int32_t u = rows[e], v = cols[e];
        if (u < 0 || u >= V || v >= V || u >= v) {
            atomicMax(&ctl->g.status, (int)TDT_ERR_NOT_ORIENTED);
            continue;
        }
        const int64_t b = rp[u], en = rp[u + 1];
        if (e < b || e >= en) {
            atomicMax(&ctl->g.status, (int)TDT_ERR_INVALID);
            continue;
        }
        if (e + 1 < en && cols[e + 1] <= v) atomicMax(&ctl->g.status, (int)TDT_ERR_INVALID);
    }
}

__global__ void indeg_kernel(const int32_t* __restrict__ rows, const int32_t* __restrict__ cols, int64_t E,
                             int64_t V, int32_t* __restrict__ indeg, const PeelCtl* ctl) {
    if (*(volatile const int*)&ctl->g.status != 0) return;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < E;
         e += (int64_t)gridDim.x * blockDim.x)
        atomicAdd(indeg + cols[e], 1);
}

__global__ void csc_fill_kernel(const int32_t* __restrict__ rows, const int32_t* __restrict__ cols, int64_t E,
                                int64_t V, const int64_t* __restrict__ cp, int32_t* __restrict__ cursor,
                                int32_t* __restrict__ in_src, int32_t* __restrict__ in_eid, const PeelCtl* ctl) {
    if (*(volatile const int*)&ctl->g.status != 0) return;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < E;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int32_t u = rows[e], v = cols[e];
        const int64_t pos = cp[v] + atomicAdd(cursor + v, 1);
        in_src[pos] = u;
        in_eid[pos] = (int32_t)e;
    }
}

// sup = cA + cB + cC (the role counts of the support pass), edge state =
// {sup, alive}, triangle total.
__global__ void init_state_kernel(const int32_t* __restrict__ cA, const int32_t* __restrict__ cB,
                                  const int32_t* __restrict__ cC, int32_t* __restrict__ sup,
                                  int32_t* __restrict__ live, int32_t* __restrict__ rnd, int64_t E,
                                  PeelCtl* ctl) {
    __shared__ long long s_part[32];
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        for (int i = 0; i < 3; i++) ctl->mgt[i] = INT32_MAX;
        ctl->dmin[0] = INT32_MAX;
        ctl->dmin[1] = INT32_MAX;
    }
    long long acc = 0;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < E;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int32_t s = cA[e] + cB[e] + cC[e];
        sup[e] = s;
        live[e] = s;
        rnd[e] = -1;
        acc += s;
    }
    acc = warp_sum(acc);
    if (lane_id() == 0) s_part[threadIdx.x / kWarp] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        long long b = 0;
        for (int i = 0; i < (int)(blockDim.x / kWarp); i++) b += s_part[i];
        atomicAdd((unsigned long long*)&ctl->triangles, (unsigned long long)b);
    }
}

// Staging bounds of the one-walk pass, per edge e = (u, v) at position i of
// row u: role A (triangles (u, v, w)) at most min(d+(u) - i - 1, d+(v)) --
// w lies in N+(u) after v and in N+(v); role B (triangles (u, x, v), x in
// N+(u) before v and in N-(v) \ {u}) at most min(i, d-(v) - 1).  bnd[e] =
// the role-A bound, sz[e] = both (the staging region of e).
__global__ void stage_bounds_kernel(const int32_t* __restrict__ rows, const int32_t* __restrict__ cols,
                                    const int64_t* __restrict__ rp, const int64_t* __restrict__ cp, int64_t E,
                                    int32_t* __restrict__ bnd, int32_t* __restrict__ sz, const PeelCtl* ctl) {
    if (*(volatile const int*)&ctl->g.status != 0) return;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < E;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int32_t u = rows[e], v = cols[e];
        const int64_t bu = rp[u];
        const int64_t i = e - bu, du = rp[u + 1] - bu;
        const int64_t dv = rp[v + 1] - rp[v], inv = cp[v + 1] - cp[v];
        const int64_t a = du - i - 1 < dv ? du - i - 1 : dv;
        const int64_t b = i < inv - 1 ? i : inv - 1;
        const int64_t aa = a < 0 ? 0 : a, bb = b < 0 ? 0 : b;
        bnd[e] = (int32_t)aa;
        sz[e] = (int32_t)(aa + bb);  // < 2^31: the one-walk pass is only chosen for V < 2^30
    }
}

// Count-only walk or one walk with staging: the one walk when the staging
// regions (8 bytes x soff[E]) fit the list tail.
__global__ void stage_decide_kernel(const int64_t* __restrict__ soff, int64_t E, int64_t V,
                                    unsigned long long tail_bytes, int want_lists, PeelCtl* ctl) {
    const int ok0 = ctl->g.status == 0;
    const int st = ok0 && want_lists && V < (1ll << 30) && 8ull * (unsigned long long)soff[E] <= tail_bytes;
    ctl->stage_skip = !st;
    ctl->roles_skip = !ok0 || st;
}

// Global cursors of the one walk's staging slots (used by rows searched in
// place): role A at soff[e], role B at soff[e] + bnd[e].
__global__ void stage_cursor_kernel(const int64_t* __restrict__ soff, const int32_t* __restrict__ bnd, int64_t E,
                                    unsigned long long* __restrict__ curA, unsigned long long* __restrict__ curB,
                                    const PeelCtl* ctl) {
    if (*(volatile const int*)&ctl->stage_skip) return;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < E;
         e += (int64_t)gridDim.x * blockDim.x) {
        const unsigned long long o = (unsigned long long)soff[e];
        curA[e] = o;
        curB[e] = o + (unsigned long long)bnd[e];
    }
}

// Lists fit when 8 bytes x (3T = off[E]) fit the workspace tail.  After the
// one walk they are packed from the staging area (which sits at the end of
// the tail) when both fit side by side; otherwise, when the lists alone fit,
// the second walk writes them; otherwise the peel searches.
__global__ void list_decide_kernel(const int64_t* __restrict__ off, const int64_t* __restrict__ soff, int64_t E,
                                   unsigned long long tail_bytes, int want_lists, PeelCtl* ctl) {
    const unsigned long long need = 8ull * (unsigned long long)off[E];
    const int ok0 = want_lists && ctl->g.status == 0;
    const int staged = !ctl->stage_skip;
    const unsigned long long stage = staged ? 8ull * (unsigned long long)soff[E] : 0ull;
    const int compact = ok0 && staged && need <= tail_bytes - stage;
    const int rewalk = ok0 && !compact && need <= tail_bytes;
    ctl->listed = compact || rewalk;
    ctl->list_skip = !(compact || rewalk);
    ctl->compact_skip = !compact;
    ctl->rewalk_skip = !rewalk;
}

// Pack the role-A / role-B entries of every edge from its staging region
// (slot s at stage_end[-1-s]) into its final list: role A at off[e], role B
// at off[e] + cA[e].  A warp takes 32 edges at a time: their entries form one
// flat index space (lane-held exclusive starts S), each lane finds the edge
// of its entry by a 5-step search over S (shuffles), and four 32-entry
// windows are copied per step so four loads per lane are in flight.
#ifndef TDT_CMP_WIN
#define TDT_CMP_WIN 4
#endif
#ifndef TDT_CMP_MINB
#define TDT_CMP_MINB 6
#endif
constexpr int kCmpBlock = 256;
__global__ void __launch_bounds__(kCmpBlock, TDT_CMP_MINB)
stage_compact_kernel(const int64_t* __restrict__ soff, const int32_t* __restrict__ bnd,
                                     const int32_t* __restrict__ cA, const int32_t* __restrict__ cB,
                                     const int64_t* __restrict__ off, const int2* __restrict__ stage_end,
                                     int2* __restrict__ lists, int64_t E, const PeelCtl* ctl) {
    if (*(volatile const int*)&ctl->compact_skip) return;
    const unsigned lane = lane_id();
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    constexpr int kWin = TDT_CMP_WIN;
    for (int64_t base = (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * kWarp; base < E;
         base += nw * kWarp) {
        const int64_t e = base + lane;
        int64_t so = 0, o = 0;
        int32_t b = 0, na = 0, n = 0;
        if (e < E) {
            so = soff[e];
            b = bnd[e];
            na = cA[e];
            n = na + cB[e];
            o = off[e];
        }
        const int32_t incl = warp_incl_scan(n);
        const int32_t total = __shfl_sync(kFull, incl, 31);
        const int32_t S = incl - n;  // first flat entry of this lane's edge
        for (int32_t tb = 0; tb < total; tb += kWin * kWarp) {
            int2 v[kWin];
            int64_t dst[kWin];
#pragma unroll
            for (int w = 0; w < kWin; w++) {
                const int32_t t = tb + w * kWarp + (int)lane;
                // last lane k with S_k <= t (S is non-decreasing, S_0 = 0)
                int k = 0;
#pragma unroll
                for (int step = 16; step > 0; step >>= 1) {
                    const int32_t Sc = __shfl_sync(kFull, S, k + step);
                    if (Sc <= t) k += step;
                }
                const int32_t Sk = __shfl_sync(kFull, S, k), ak = __shfl_sync(kFull, na, k),
                              bk = __shfl_sync(kFull, b, k);
                const int64_t sk = __shfl_sync(kFull, so, k), ok = __shfl_sync(kFull, o, k);
                const int32_t loc = t - Sk;
                dst[w] = -1;
                if (t < total) {
                    const int64_t src = sk + (loc < ak ? loc : bk + (loc - ak));
                    v[w] = __ldcs(stage_end - 1 - src);
                    dst[w] = ok + loc;
                }
            }
#pragma unroll
            for (int w = 0; w < kWin; w++)
                if (dst[w] >= 0) lists[dst[w]] = v[w];
        }
    }
}

// Global slot cursors of the second walk (used by rows listed in place):
// role A at off[e], role B at off[e] + cA[e].
__global__ void list_cursor_kernel(const int64_t* __restrict__ off, const int32_t* __restrict__ cA, int64_t E,
                                   unsigned long long* __restrict__ curA, unsigned long long* __restrict__ curB,
                                   const PeelCtl* ctl) {
    if (*(volatile const int*)&ctl->rewalk_skip) return;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < E;
         e += (int64_t)gridDim.x * blockDim.x) {
        const unsigned long long o = (unsigned long long)off[e];
        curA[e] = o;
        curB[e] = o + cA[e];
    }
}

__global__ void truss_out_kernel(const int32_t* __restrict__ rnd, const int32_t* __restrict__ round_level,
                                 int64_t E, int32_t* __restrict__ truss, uint32_t* __restrict__ keys,
                                 uint32_t* __restrict__ vals, PeelCtl* ctl) {
    if (ctl->g.status != 0) return;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < E;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int32_t r = rnd[e];
        if (r < 0) {  // every edge is peeled when the run completes
            atomicMax((int*)&ctl->g.status, (int)TDT_ERR_CAPACITY);
            continue;
        }
        if (truss) truss[e] = round_level[r] + 2;
        keys[e] = (uint32_t)r;
        vals[e] = (uint32_t)e;
    }
}

// Number of sorted positions whose round has level <= lv (levels are
// non-decreasing in round order).
__device__ __forceinline__ int64_t count_level_le(const uint32_t* keys, int64_t E, const int32_t* round_level,
                                                  int32_t lv) {
    int64_t lo = 0, hi = E;
    while (lo < hi) {
        int64_t mid = (lo + hi) >> 1;
        if (round_level[keys[mid]] <= lv) lo = mid + 1; else hi = mid;
    }
    return lo;
}

__global__ void ptr_etruss_kernel(const uint32_t* __restrict__ keys, const uint32_t* __restrict__ vals, int64_t E,
                                  const int32_t* __restrict__ round_level, int32_t* __restrict__ ptr_truss,
                                  int64_t ptr_cap, int32_t* __restrict__ e_truss, PeelCtl* ctl,
                                  int64_t* __restrict__ stats) {
    if (*(volatile int*)&ctl->g.status != 0) return;
    const long long rounds = ctl->rounds;
    const int32_t L = rounds > 0 ? round_level[rounds - 1] : 0;
    const int64_t n0 = rounds > 0 ? count_level_le(keys, E, round_level, 0) : E;
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t nth = (int64_t)gridDim.x * blockDim.x;
    if (ptr_truss) {
        if ((int64_t)L + 1 > ptr_cap) {
            if (tid == 0) atomicMax(&ctl->g.status, (int)TDT_ERR_CAPACITY);
        } else {
            for (int64_t i = tid; i <= L; i += nth)
                ptr_truss[i] = (int32_t)((i == 0 ? n0 : count_level_le(keys, E, round_level, (int32_t)i)) - n0);
        }
    }
    if (e_truss)
        for (int64_t p = n0 + tid; p < E; p += nth) e_truss[p - n0] = (int32_t)vals[p];
    if (tid == 0) {
        stats[TDT_STAT_KMAX] = (long long)L + 2;
        stats[TDT_STAT_NPTR] = (long long)L + 1;
        stats[TDT_STAT_ROUNDS] = rounds;
        stats[TDT_STAT_TRIANGLES] = ctl->triangles / 3;
        stats[TDT_STAT_NETRUSS] = E - n0;
    }
}

__global__ void ktruss_out_kernel(const int32_t* __restrict__ rnd, int64_t E, uint8_t* __restrict__ in_k,
                                  PeelCtl* ctl) {
    __shared__ unsigned long long s_part[32];
    unsigned long long acc = 0;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < E;
         e += (int64_t)gridDim.x * blockDim.x) {
        const uint8_t a = rnd[e] == -1;
        in_k[e] = a;
        acc += a;
    }
    acc = warp_sum(acc);
    if (lane_id() == 0) s_part[threadIdx.x / kWarp] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long b = 0;
        for (int i = 0; i < (int)(blockDim.x / kWarp); i++) b += s_part[i];
        atomicAdd(&ctl->alive, b);
    }
}

__global__ void stats_final_kernel(PeelCtl* ctl, int64_t* stats, int mode) {
    stats[TDT_STAT_STATUS] = ctl->g.status;
    stats[TDT_STAT_LISTED] = ctl->listed ? (ctl->compact_skip ? 1 : 2) : 0;
    if (mode != 0) {
        stats[TDT_STAT_ALIVE] = (long long)ctl->alive;
        stats[TDT_STAT_ROUNDS] = ctl->rounds;
        stats[TDT_STAT_TRIANGLES] = ctl->triangles / 3;
    }
}

// ------------------------------------------------------------------ host side
void prof_mark(int phase, cudaStream_t st);

// Test hook: wall-clock budget of the next peel launches (<= 0: the default).
static long long g_peel_deadline_ns = 0;
void set_peel_deadline(long long ns) { g_peel_deadline_ns = ns; }

// Test hook: lower the k-truss collection batch limits (<= 0: the defaults).
static long long g_dyn_min_slots = 0;

// Block 0's clock of the last persistent peel run in this workspace (the
// control block sits at its start): processing, grid-barrier waits after
// processing, level changes, and the whole kernel, in ns.
int peel_clock(const void* ws, long long* ns, cudaStream_t st) {
    TDT_CHECK_ARG(ws != nullptr && ns != nullptr, "null pointer");
    const PeelCtl* ctl = reinterpret_cast<const PeelCtl*>(ws);
    unsigned long long t[4];
    TDT_CUDA(cudaMemcpyAsync(t, &ctl->t_proc, sizeof(t), cudaMemcpyDeviceToHost, st));
    TDT_CUDA(cudaStreamSynchronize(st));
    for (int i = 0; i < 4; i++) ns[i] = (long long)t[i];
    return TDT_OK;
}
void set_peel_dyn_min(long long slots) { g_dyn_min_slots = slots; }
// Peel grid in half-SM units (0: the size heuristic below); the autotuner's
// launch-shape dimension.
static int g_peel_half_sms = 0;
void set_peel_grid(int half_sms) { g_peel_half_sms = half_sms > 0 ? half_sms : 0; }
static long long g_fixed_item_cap = 0, g_fixed_cand_cap = 0;
void set_fixed_caps(long long items, long long cands) {
    g_fixed_item_cap = items;
    g_fixed_cand_cap = cands;
}

// A grid barrier that one block never reaches: the others wait limit_ns, then
// leave with TDT_ERR_TIMEOUT in ctl->status (the test of the bounded waits).
__global__ void barrier_probe_kernel(GridCtl* ctl, unsigned long long limit_ns) {
    if (blockIdx.x == 0) return;
    grid_barrier(ctl, gridDim.x, limit_ns);
}

int test_barrier_timeout(void* ws, long long limit_ns, cudaStream_t st) {
    TDT_CHECK_ARG(ws != nullptr, "null workspace");
    TDT_CHECK_ARG(limit_ns >= 1000000ll && limit_ns <= 2000000000ll, "limit %lld ns outside [1 ms, 2 s]",
                  limit_ns);
    GridCtl* ctl = reinterpret_cast<GridCtl*>(ws);
    TDT_CUDA(cudaMemsetAsync(ctl, 0, sizeof(GridCtl), st));
    barrier_probe_kernel<<<8, 32, 0, st>>>(ctl, (unsigned long long)limit_ns);
    TDT_LAUNCH_CHECK("barrier_probe");
    int status = 0;
    TDT_CUDA(cudaMemcpyAsync(&status, &ctl->status, sizeof(int), cudaMemcpyDeviceToHost, st));
    TDT_CUDA(cudaStreamSynchronize(st));
    return status;
}

int launch_support_roles(const int64_t* rp, const int32_t* cols, int64_t nv, int64_t ne, int32_t* cA, int32_t* cB,
                         int32_t* cC, void* ctl, const int* gate, int* status, cudaStream_t st);
int launch_support_list(const int64_t* rp, const int32_t* cols, int64_t nv, int64_t ne, const int64_t* off,
                        const int32_t* cA, const int32_t* cB, unsigned long long* curA_g,
                        unsigned long long* curB_g, int2* lists, void* ctl, const int* gate, int* status,
                        cudaStream_t st);
int launch_support_stage(const int64_t* rp, const int32_t* cols, int64_t nv, int64_t ne, const int64_t* soff,
                         const int32_t* bnd, int32_t* cA, int32_t* cB, int32_t* cC, unsigned long long* curA_g,
                         unsigned long long* curB_g, int2* stage_end, unsigned long long stage_slots, void* ctl,
                         const int* gate, int* status, cudaStream_t st);
int launch_list_transpose(const int64_t* cp, const int64_t* rp, const int32_t* cols, const int32_t* in_eid,
                          int64_t nv, int64_t ne, const int64_t* off,
                          const int32_t* cA, const int32_t* cB, int2* lists, unsigned long long* cur, void* next,
                          const int* gate, int* status, cudaStream_t st);

namespace {
struct Carver {
    char* base;
    size_t off = 0;
    size_t cap;
    void* take(size_t bytes) {
        off = (off + 255) & ~(size_t)255;
        void* p = base ? base + off : nullptr;
        off += bytes;
        return p;
    }
};

struct Layout {
    PeelCtl* ctl;
    void* sup_ctl;
    int32_t* rows_d;
    int32_t* indeg;
    int64_t* cp;
    int32_t* in_src;
    int32_t* in_eid;
    int32_t* sup;
    int32_t* live;
    int32_t* rnd;
    int32_t* round_level;
    int4* qi[3];
    long long* qb[3];
    int64_t* off;
    int64_t* soff;
    int32_t* bnd;
    int32_t* alive[2];
    unsigned* dead;
    unsigned* code;
    void* scan_ws;
    void* sort_ws;
    size_t total;
};

Layout carve(void* ws, int64_t V, int64_t E) {
    Carver c{reinterpret_cast<char*>(ws)};
    Layout L;
    const size_t e = (size_t)(E > 0 ? E : 1), v = (size_t)(V > 0 ? V : 1);
    L.ctl = (PeelCtl*)c.take(4096);
    L.sup_ctl = c.take(256);
    L.rows_d = (int32_t*)c.take(4 * e);
    L.indeg = (int32_t*)c.take(4 * v);
    L.cp = (int64_t*)c.take(8 * (v + 1));
    L.in_src = (int32_t*)c.take(4 * e);
    L.in_eid = (int32_t*)c.take(4 * e);
    L.sup = (int32_t*)c.take(4 * e);
    L.live = (int32_t*)c.take(4 * e);
    L.rnd = (int32_t*)c.take(4 * e);
    L.round_level = (int32_t*)c.take(4 * (e + 2));
    for (int b = 0; b < 3; b++) {
        L.qi[b] = (int4*)c.take(16 * e);
        L.qb[b] = (long long*)c.take(8 * e);
    }
    L.off = (int64_t*)c.take(8 * (e + 1));
    L.soff = (int64_t*)c.take(8 * (e + 1));
    L.bnd = (int32_t*)c.take(4 * e);
    L.alive[0] = (int32_t*)c.take(4 * e);
    L.alive[1] = (int32_t*)c.take(4 * e);
    L.dead = (unsigned*)c.take(4 * (e / 32 + 1));
    L.code = (unsigned*)c.take(4 * (e / 8 + 1));
    size_t scan_b = scan_scratch_bytes((int64_t)(e > v ? e : v) + 1);
    L.scan_ws = c.take(scan_b);
    L.sort_ws = c.take(radix_sort_scratch_bytes((int64_t)e));
    L.total = c.off + 256;
    return L;
}
}  // namespace

size_t decompose_workspace_bytes(int64_t V, int64_t E) {
    // the e_truss sort reuses the queue buffers for its keys/values
    return carve(nullptr, V, E).total;
}

// mode 0: decomposition; 1: k-truss search at level fixed_level; 2: support / triangle count only.
int run_peel(int mode, const int32_t* rows, const int32_t* cols, const int64_t* rp, int64_t V, int64_t E,
             int32_t fixed_level, int32_t* truss, int32_t* e_truss, int32_t* ptr_truss, int64_t ptr_cap,
             uint8_t* in_k, int32_t* support_out, int64_t* stats, void* ws, size_t ws_bytes, cudaStream_t st) {
    TDT_CHECK_ARG(V >= 0 && E >= 0, "negative graph size");
    TDT_CHECK_ARG(E < (int64_t)INT32_MAX, "num_edges %lld exceeds int32 edge ids", (long long)E);
    TDT_CHECK_ARG(V < (int64_t)INT32_MAX, "num_vertices %lld exceeds int32 vertex ids", (long long)V);
    TDT_CHECK_ARG(stats != nullptr, "stats is required");
    TDT_CHECK_ARG(E == 0 || (cols && rp), "null graph pointer");
    const size_t need = decompose_workspace_bytes(V, E);
    if (ws_bytes < need || ws == nullptr) {
        set_error("workspace of %zu bytes < required %zu", ws_bytes, need);
        return TDT_ERR_WORKSPACE;
    }
    DeviceInfo di;
    int rc = device_info(&di);
    if (rc) return rc;
    Layout L = carve(ws, V, E);
    TDT_CUDA(cudaMemsetAsync(L.ctl, 0, 4096, st));
    TDT_CUDA(cudaMemsetAsync(stats, 0, sizeof(int64_t) * TDT_STAT_COUNT, st));
    if (E == 0) {
        if (mode == 0) {
            if (ptr_truss && ptr_cap >= 1) TDT_CUDA(cudaMemsetAsync(ptr_truss, 0, 4, st));
            int64_t h[TDT_STAT_COUNT] = {0, 2, 1, 0, 0, 0, 0, 0};
            if (ptr_truss && ptr_cap < 1) h[0] = TDT_ERR_CAPACITY;
            TDT_CUDA(cudaMemcpyAsync(stats, h, sizeof(h), cudaMemcpyHostToDevice, st));
            TDT_CUDA(cudaStreamSynchronize(st));
        }
        return TDT_OK;
    }
    const int tb = 256;
    const unsigned g_e = grid_for(E, tb, di.sms, 8);
    const int32_t* rows_use = rows;
    if (!rows_use) {
        rows_from_rp_kernel<<<grid_for(V * 32, tb, di.sms, 8), tb, 0, st>>>(rp, V, L.rows_d);
        TDT_LAUNCH_CHECK("rows_from_rp");
        rows_use = L.rows_d;
    }
    validate_kernel<<<g_e, tb, 0, st>>>(rp, rows_use, cols, E, V, L.ctl);
    TDT_LAUNCH_CHECK("validate");
    // cA, cB, cC (role counts) live in the first queue buffer until the peel starts
    int32_t* cA = reinterpret_cast<int32_t*>(L.qi[0]);
    int32_t* cB = cA + E;
    int32_t* cC = cB + E;
    prof_mark(0, st);
    TDT_CUDA(cudaMemsetAsync(cA, 0, 12 * (size_t)E, st));
    if (mode == 2) {
        // triangle count: the count-only walk (skipped on the device when
        // validation failed)
        rc = launch_support_roles(rp, cols, V, E, cA, cB, cC, L.sup_ctl, &L.ctl->g.status, &L.ctl->g.status, st);
        if (rc) return rc;
        init_state_kernel<<<g_e, tb, 0, st>>>(cA, cB, cC, L.sup, L.live, L.rnd, E, L.ctl);
        TDT_LAUNCH_CHECK("init_state");
        prof_mark(1, st);
        if (support_out) TDT_CUDA(cudaMemcpyAsync(support_out, L.sup, 4 * (size_t)E, cudaMemcpyDeviceToDevice, st));
        stats_final_kernel<<<1, 1, 0, st>>>(L.ctl, stats, 1);
        TDT_LAUNCH_CHECK("stats_final");
        for (int ph = 2; ph <= 4; ph++) prof_mark(ph, st);
        return TDT_OK;
    }
    // The list tail: final lists grow from its start, the one walk's staging
    // area (indexed backwards) ends at its end.
    const size_t list_base = (need + 255) & ~(size_t)255;
    const unsigned long long tail = ws_bytes > list_base ? (unsigned long long)(ws_bytes - list_base) : 0ull;
    int2* lists = reinterpret_cast<int2*>(reinterpret_cast<char*>(ws) + list_base);
    const unsigned long long stage_slots = tail / 8;
    int2* stage_end = lists + stage_slots;
    // in-adjacency (CSC) of the oriented graph: staging bounds, role-C
    // transpose, and the peel without lists
    TDT_CUDA(cudaMemsetAsync(L.indeg, 0, 4 * (size_t)V, st));
    indeg_kernel<<<g_e, tb, 0, st>>>(rows_use, cols, E, V, L.indeg, L.ctl);
    TDT_LAUNCH_CHECK("indeg");
    rc = exclusive_scan<int32_t, int64_t>(L.indeg, L.cp, V, L.cp + V, L.scan_ws, st);
    if (rc) return rc;
    TDT_CUDA(cudaMemsetAsync(L.indeg, 0, 4 * (size_t)V, st));
    csc_fill_kernel<<<g_e, tb, 0, st>>>(rows_use, cols, E, V, L.cp, L.indeg, L.in_src, L.in_eid, L.ctl);
    TDT_LAUNCH_CHECK("csc_fill");
    // staging regions of the one walk (L.sup holds their sizes until
    // init_state overwrites it), and the choice of walk
    stage_bounds_kernel<<<g_e, tb, 0, st>>>(rows_use, cols, rp, L.cp, E, L.bnd, L.sup, L.ctl);
    TDT_LAUNCH_CHECK("stage_bounds");
    rc = exclusive_scan<int32_t, int64_t>(L.sup, L.soff, E, L.soff + E, L.scan_ws, st);
    if (rc) return rc;
    stage_decide_kernel<<<1, 1, 0, st>>>(L.soff, E, V, tail, tail > 0, L.ctl);
    TDT_LAUNCH_CHECK("stage_decide");
    unsigned long long* curA = reinterpret_cast<unsigned long long*>(L.qb[0]);
    unsigned long long* curB = reinterpret_cast<unsigned long long*>(L.qb[1]);
    stage_cursor_kernel<<<g_e, tb, 0, st>>>(L.soff, L.bnd, E, curA, curB, L.ctl);
    TDT_LAUNCH_CHECK("stage_cursor");
    // the walk: counts and staged role-A/B entries, or counts only (each
    // launch returns at once when its gate is set)
    rc = launch_support_stage(rp, cols, V, E, L.soff, L.bnd, cA, cB, cC, curA, curB, stage_end, stage_slots,
                              L.sup_ctl, &L.ctl->stage_skip, &L.ctl->g.status, st);
    if (rc) return rc;
    rc = launch_support_roles(rp, cols, V, E, cA, cB, cC, L.sup_ctl, &L.ctl->roles_skip, &L.ctl->g.status, st);
    if (rc) return rc;
    init_state_kernel<<<g_e, tb, 0, st>>>(cA, cB, cC, L.sup, L.live, L.rnd, E, L.ctl);
    TDT_LAUNCH_CHECK("init_state");
    prof_mark(1, st);
    // per-edge triangle lists in the workspace tail when 24 T bytes fit
    rc = exclusive_scan<int32_t, int64_t>(L.sup, L.off, E, L.off + E, L.scan_ws, st);
    if (rc) return rc;
    list_decide_kernel<<<1, 1, 0, st>>>(L.off, L.soff, E, tail, tail > 0, L.ctl);
    TDT_LAUNCH_CHECK("list_decide");
    {
        // one wave of resident blocks (the loop is grid-strided)
        int occ_c = 0;
        TDT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_c, stage_compact_kernel, kCmpBlock, 0));
        if (occ_c < 1) occ_c = 1;
        const unsigned g_c = grid_for(E * 32, kCmpBlock, di.sms, occ_c);
        stage_compact_kernel<<<g_c, kCmpBlock, 0, st>>>(L.soff, L.bnd, cA, cB, L.off, stage_end, lists, E, L.ctl);
    }
    TDT_LAUNCH_CHECK("stage_compact");
    // second walk, when the lists fit but not beside the staging area
    list_cursor_kernel<<<g_e, tb, 0, st>>>(L.off, cA, E, curA, curB, L.ctl);
    TDT_LAUNCH_CHECK("list_cursor");
    rc = launch_support_list(rp, cols, V, E, L.off, cA, cB, curA, curB, lists, L.sup_ctl, &L.ctl->rewalk_skip,
                             &L.ctl->g.status, st);
    if (rc) return rc;
    // role C of every list, from the role-A lists of each vertex's in-edges
    rc = launch_list_transpose(L.cp, rp, cols, L.in_eid, V, E, L.off, cA, cB, lists,
                               reinterpret_cast<unsigned long long*>(L.qi[1]), L.sup_ctl, &L.ctl->list_skip,
                               &L.ctl->g.status, st);
    if (rc) return rc;
    prof_mark(2, st);

    // persistent peel
    int occ = 0;
    TDT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, peel_kernel, kPeelBlock, 0));
    if (occ < 1) {
        set_error("peel kernel cannot be resident");
        return TDT_ERR_UNSUPPORTED;
    }
    PeelArgs A;
    A.rp = rp; A.cols = cols; A.rows = rows_use; A.cp = L.cp; A.in_src = L.in_src; A.in_eid = L.in_eid;
    A.live = L.live; A.rnd = L.rnd; A.round_level = L.round_level;
    for (int b = 0; b < 3; b++) {
        A.qi[b] = L.qi[b];
        A.qb[b] = L.qb[b];
    }
    A.dead = L.dead;
    TDT_CUDA(cudaMemsetAsync(L.dead, 0, 4 * (size_t)(E / 32 + 1), st));
    A.code = L.code;
    TDT_CUDA(cudaMemsetAsync(L.code, 0xff, 4 * (size_t)(E / 8 + 1), st));
    A.off = L.off; A.lists = lists;
    A.alive[0] = L.alive[0]; A.alive[1] = L.alive[1];
    A.V = V; A.E = E; A.round_cap = E + 2;
    A.mode = mode == 0 ? 0 : 1;
    A.fixed_level = fixed_level;
    A.deadline_ns = g_peel_deadline_ns > 0 ? (unsigned long long)g_peel_deadline_ns : kPeelDeadlineNs;
    A.dyn_min_slots = g_dyn_min_slots > 0 ? g_dyn_min_slots : (1ll << kDynMinLog2);
    A.fixed_item_cap = g_fixed_item_cap > 0 && (unsigned long long)g_fixed_item_cap < kFixedItemCap
                           ? (unsigned long long)g_fixed_item_cap : kFixedItemCap;
    A.fixed_cand_cap = g_fixed_cand_cap > 0 && (unsigned long long)g_fixed_cand_cap < kFixedCandCap
                           ? (unsigned long long)g_fixed_cand_cap : kFixedCandCap;
    A.ctl = L.ctl;
    if (di.sms * occ > 4096) occ = 4096 / di.sms;
    // Smaller graphs peel their lists faster on fewer blocks: the sub-rounds
    // are short, so the grid barrier and the idle warps cost more than the
    // parallelism gives (R-MAT scale 10-18 measured 4-15 % faster on one block
    // per SM, scales 10-14 on one per two SMs; scale 20 and up fastest on
    // all).  The search peel (no list tail) keeps every block: its slots are
    // binary searches, and scale 18 ran 22 % slower on half the blocks.
    int nblk = di.sms * occ;
    if (tail > 0 && E < (1ll << 18)) nblk = (di.sms + 1) / 2;
    else if (tail > 0 && E < (1ll << 22)) nblk = di.sms;
    if (g_peel_half_sms > 0) nblk = (g_peel_half_sms * di.sms + 1) / 2;
    if (nblk > di.sms * occ) nblk = di.sms * occ;
    dim3 grid(nblk), block(kPeelBlock);
    void* args[] = {&A};
    TDT_CUDA(cudaLaunchCooperativeKernel((void*)peel_kernel, grid, block, args, 0, st));
    note_launch();
    prof_mark(3, st);

    if (mode == 0) {
        // outputs: truss numbers, then e_truss / ptr_truss from a stable sort by round
        uint32_t* keys = reinterpret_cast<uint32_t*>(L.qi[0]);
        uint32_t* vals = keys + E;
        uint32_t* keys_alt = reinterpret_cast<uint32_t*>(L.qi[1]);
        uint32_t* vals_alt = keys_alt + E;
        truss_out_kernel<<<g_e, tb, 0, st>>>(L.rnd, L.round_level, E, truss, keys, vals, L.ctl);
        TDT_LAUNCH_CHECK("truss_out");
        const uint32_t* sk = keys;
        const uint32_t* sv = vals;
        int bits = 8;
        while (bits < 32 && ((int64_t)1 << bits) < E + 2) bits += 8;
        bool in_alt = false;
        rc = radix_sort_pairs<uint32_t>(keys, vals, keys_alt, vals_alt, E, 0, bits, L.sort_ws, &in_alt, st);
        if (rc) return rc;
        if (in_alt) { sk = keys_alt; sv = vals_alt; }
        ptr_etruss_kernel<<<g_e, tb, 0, st>>>(sk, sv, E, L.round_level, ptr_truss, ptr_cap, e_truss, L.ctl,
                                               stats);
        TDT_LAUNCH_CHECK("ptr_etruss");
        stats_final_kernel<<<1, 1, 0, st>>>(L.ctl, stats, 0);
        TDT_LAUNCH_CHECK("stats_final");
    } else {
        ktruss_out_kernel<<<g_e, tb, 0, st>>>(L.rnd, E, in_k, L.ctl);
        TDT_LAUNCH_CHECK("ktruss_out");
        stats_final_kernel<<<1, 1, 0, st>>>(L.ctl, stats, 1);
        TDT_LAUNCH_CHECK("stats_final");
    }
    prof_mark(4, st);
    return TDT_OK;
}

}  // namespace tdt
