// The reference's research-variant operators (outside the --cuda flow):
//   segment_isinis_m / segment_isinmm  (kernel.cu:687-737, :1555-1607): per row,
//       flag the positions of the values two sorted rows share;
//   sub_suppport_affect                 (kernel.cu:739-805): support update
//       from precomputed triangle partners;
//   peeling_undirect(_tile), peeling_direct_{oo,ii,oi}(_tile)
//                                       (kernel.cu:808-1551): peel update of
//       the triangles of the current edges, the third vertex found in two
//       sorted lists of the edge's endpoints.
//
// The peel family: for a current edge e = (u, v) (u = rows[e], v = columns[e]),
// the third vertex w of a triangle appears in one list of u and one of v:
//   UND  symmetric adjacency of u and of v (columns_g, edge ids edges_id_nbr);
//   OO   out-lists of u and v (edge id = position);
//   II   in-lists of u and v (r_edges: edge ids grouped by head, sorted by
//        tail; re_ptr their offsets);
//   OI   out-list of u and in-list of v.
// For every shared w with both other edges alive (e_mask), the edges not in
// the current set (in_curr) are decremented; with one of them current, a rule
// per variant decides who decrements so each destroyed triangle counts once.
// An edge whose decrement takes its support from l to l-1 is marked in n_mark
// (the wrappers pass the level + 1 as l, myhpu_extension.cpp:330 etc.).
// Tiled forms split every list into n_cut column tiles (ptr[v * n_cut + k]).
//
// Every operator here pairs two lists the way the reference's two-pointer
// merge does.  One warp takes one pair (edge x tile, or row).  It first checks
// that both lists are strictly increasing (isinis_m: ignoring its -1 holes,
// with every other value >= 0).  For such lists the merge pairs exactly the
// equal values, so the warp hashes the shorter list into shared memory
// (value -> position) and streams the longer one against it.  Otherwise one
// lane runs the reference's merge walk itself, so the outcome is the
// reference's on any input.  Decrements are exact atomics: supports and n_mark
// do not depend on thread order.  List positions and edge ids are
// bounds-checked; an out-of-range id takes part in no triangle.
#include "common.cuh"

namespace tdt {

namespace {

constexpr int kRBlock = 256;
constexpr int kRWarps = kRBlock / kWarp;
constexpr int kRSlots = 256;   // hash slots per warp
constexpr int kRChunk = 128;   // keys hashed per pass
constexpr int32_t kREmpty = INT32_MIN;

__device__ __forceinline__ unsigned rhash(int32_t k) { return ((uint32_t)k * 0x9E3779B1u) >> 24; }

// ------------------------------------------------------------------ list pairing
// A list source S gives key(i) for a position i of its array.

// True on every lane when [b, e) of s is strictly increasing (skip_neg1: the
// -1 entries are left out and every other entry must be >= 0) and holds no
// INT32_MIN.  Called by all 32 lanes.
template <class S>
__device__ bool warp_increasing(const S& s, int64_t b, int64_t e, bool skip_neg1, unsigned lane) {
    bool ok = true, has_prev = false;
    int32_t prev = 0;
    for (int64_t c = b; c < e; c += kWarp) {
        const int64_t i = c + lane;
        const bool valid = i < e;
        const int32_t k = valid ? s.key(i) : 0;
        if (valid && (k == kREmpty || (skip_neg1 && k < -1))) ok = false;
        const bool real = valid && !(skip_neg1 && k == -1);
        const unsigned rm = __ballot_sync(kFull, real);
        const unsigned below = rm & lanemask_lt();
        const int32_t pk = __shfl_sync(kFull, k, below ? 31 - __clz(below) : 0);
        if (real) {
            if (below) {
                if (!(pk < k)) ok = false;
            } else if (has_prev && !(prev < k)) {
                ok = false;
            }
        }
        if (rm) {
            prev = __shfl_sync(kFull, k, 31 - __clz(rm));
            has_prev = true;
        }
    }
    return __all_sync(kFull, ok);
}

// Hash pairing of two strictly increasing lists: on_match(short_pos, long_pos)
// for every value both hold (skip_neg1: -1 excepted).  Called by all lanes.
template <class SS, class SL, class F>
__device__ void warp_hash_pairs(const SS& S, int64_t sb, int64_t se, const SL& L, int64_t lb, int64_t le,
                                bool skip_neg1, int32_t* hkey, int32_t* hpos, unsigned lane, F&& on_match) {
    for (int64_t c = sb; c < se; c += kRChunk) {
        const int64_t ce = c + kRChunk < se ? c + kRChunk : se;
        for (int i = lane; i < kRSlots; i += kWarp) hkey[i] = kREmpty;
        __syncwarp();
        for (int64_t i = c + lane; i < ce; i += kWarp) {
            const int32_t key = S.key(i);
            if (skip_neg1 && key == -1) continue;
            unsigned h = rhash(key);
            for (int probe = 0; probe < kRSlots; probe++) {
                if (atomicCAS(&hkey[h], kREmpty, key) == kREmpty) {
                    hpos[h] = (int32_t)(i - c);
                    break;
                }
                h = (h + 1) & (kRSlots - 1);
            }
        }
        __syncwarp();
        for (int64_t i = lb + lane; i < le; i += kWarp) {
            const int32_t key = L.key(i);
            if (skip_neg1 && key == -1) continue;
            unsigned h = rhash(key);
            for (int probe = 0; probe < kRSlots; probe++) {
                const int32_t kk = hkey[h];
                if (kk == kREmpty) break;
                if (kk == key) {
                    on_match(c + hpos[h], i);
                    break;
                }
                h = (h + 1) & (kRSlots - 1);
            }
        }
        __syncwarp();
    }
}

// The reference's two-pointer walk (e.g. kernel.cu:822-857), run by one lane.
template <class SA, class SB, class F>
__device__ void lane_merge(const SA& A, int64_t i, int64_t ie, const SB& B, int64_t j, int64_t je, bool skip_neg1,
                           F&& on_match) {
    while (i < ie && j < je) {
        const int32_t x = A.key(i), y = B.key(j);
        if (x == y && !(skip_neg1 && x == -1)) {
            on_match(i, j);
            i++;
            j++;
        } else if (x < y) {
            i++;
        } else {
            j++;
        }
    }
}

// Pair list A [ab, ae) with list B [bb, be): on_match(posA, posB) for the
// pairs the reference's merge would match.  Called by all lanes.
template <class SA, class SB, class F>
__device__ void warp_pairs(const SA& A, int64_t ab, int64_t ae, const SB& B, int64_t bb, int64_t be, bool skip_neg1,
                           int32_t* hkey, int32_t* hpos, unsigned lane, F&& on_match) {
    if (ae <= ab || be <= bb) return;
    if (warp_increasing(A, ab, ae, skip_neg1, lane) && warp_increasing(B, bb, be, skip_neg1, lane)) {
        if (ae - ab <= be - bb) {
            warp_hash_pairs(A, ab, ae, B, bb, be, skip_neg1, hkey, hpos, lane, on_match);
        } else {
            warp_hash_pairs(B, bb, be, A, ab, ae, skip_neg1, hkey, hpos, lane,
                            [&](int64_t pb, int64_t pa) { on_match(pa, pb); });
        }
    } else {
        if (lane == 0) lane_merge(A, ab, ae, B, bb, be, skip_neg1, on_match);
        __syncwarp();
    }
}

// ------------------------------------------------------------------ peel updates
enum ListKind { kOut = 0, kIn = 1, kUnd = 2 };
enum Variant { kVarUnd = 0, kVarOO = 1, kVarII = 2, kVarOI = 3 };

struct PeelOpArgs {
    const int32_t* e_curr;
    int64_t n_curr;
    const int32_t* rows;
    const int32_t* columns;
    int64_t E;                    // rows/columns/support/e_mask/n_mark/in_curr length
    const int32_t* row_ptr;       // out-list offsets (tiled), or the symmetric adjacency's
    int64_t row_ptr_len;
    const int32_t* r_edges;       // in-lists
    const int32_t* re_ptr;
    int64_t re_ptr_len;
    int64_t r_len;
    const int32_t* columns_g;     // symmetric adjacency
    const int32_t* edges_id_nbr;
    int64_t g_len;
    int32_t* support;
    const uint8_t* e_mask;
    uint8_t* n_mark;
    const uint8_t* in_curr;
    int32_t l;                    // level + 1: a decrement from l marks the edge
    int32_t n_cut;
};

// Third-vertex keys and edge ids of one list kind.
template <int K>
struct EdgeList {
    const PeelOpArgs* A;
    __device__ __forceinline__ int32_t id(int64_t i) const {
        if (K == kOut) return (int32_t)i;
        if (K == kIn) return __ldg(A->r_edges + i);
        return __ldg(A->edges_id_nbr + i);
    }
    __device__ __forceinline__ int32_t key(int64_t i) const {
        if (K == kOut) return __ldg(A->columns + i);
        if (K == kUnd) return __ldg(A->columns_g + i);
        const int32_t x = __ldg(A->r_edges + i);
        return (x >= 0 && x < A->E) ? __ldg(A->rows + x) : kREmpty;
    }
};

template <int K>
__device__ __forceinline__ void list_range(const PeelOpArgs& A, int32_t v, int k, int64_t& b, int64_t& e) {
    const int32_t* ptr = K == kIn ? A.re_ptr : A.row_ptr;
    const int64_t plen = K == kIn ? A.re_ptr_len : A.row_ptr_len;
    const int64_t cap = K == kOut ? A.E : (K == kIn ? A.r_len : A.g_len);
    const int64_t j = (int64_t)v * A.n_cut + k;
    b = e = 0;
    if (v < 0 || j + 1 >= plen) return;
    int64_t x = __ldg(ptr + j), y = __ldg(ptr + j + 1);
    x = x < 0 ? 0 : (x > cap ? cap : x);
    y = y < x ? x : (y > cap ? cap : y);
    b = x;
    e = y;
}

__device__ __forceinline__ void dec_mark(const PeelOpArgs& A, int32_t x) {
    if (atomicSub(A.support + x, 1) == A.l) A.n_mark[x] = 1;
}

template <int V>
__device__ __forceinline__ void on_shared(const PeelOpArgs& A, int32_t e, int32_t e2, int32_t e3) {
    if (e2 < 0 || e2 >= A.E || e3 < 0 || e3 >= A.E) return;
    if (!A.e_mask[e2] || !A.e_mask[e3]) return;
    const bool f2 = A.in_curr[e2], f3 = A.in_curr[e3];
    if (!f2 && !f3) {
        dec_mark(A, e2);
        dec_mark(A, e3);
    } else if (!f2 && f3) {
        if (V == kVarOO || V == kVarOI || (V == kVarUnd && e < e3)) dec_mark(A, e2);
    } else if (f2 && !f3) {
        if (V == kVarOO || (V == kVarUnd && e < e2)) dec_mark(A, e3);
    }
}

template <int V>
__global__ void __launch_bounds__(kRBlock) peel_op_kernel(const __grid_constant__ PeelOpArgs A) {
    constexpr int KA = V == kVarII ? kIn : (V == kVarUnd ? kUnd : kOut);
    constexpr int KB = V == kVarOO ? kOut : (V == kVarUnd ? kUnd : kIn);
    __shared__ int32_t s_key[kRWarps][kRSlots];
    __shared__ int32_t s_pos[kRWarps][kRSlots];
    const int wib = threadIdx.x / kWarp;
    const unsigned lane = lane_id();
    const EdgeList<KA> LA{&A};
    const EdgeList<KB> LB{&A};
    const int64_t units = A.n_curr * A.n_cut;
    const int64_t nw = (int64_t)gridDim.x * kRWarps;
    for (int64_t w = (int64_t)blockIdx.x * kRWarps + wib; w < units; w += nw) {
        const int64_t j = w / A.n_cut;
        const int k = (int)(w % A.n_cut);
        const int32_t e = __ldg(A.e_curr + j);
        if (e < 0 || e >= A.E) continue;
        int64_t ab, ae, bb, be;
        list_range<KA>(A, __ldg(A.rows + e), k, ab, ae);
        list_range<KB>(A, __ldg(A.columns + e), k, bb, be);
        warp_pairs(LA, ab, ae, LB, bb, be, false, s_key[wib], s_pos[wib], lane,
                   [&](int64_t pa, int64_t pb) { on_shared<V>(A, e, LA.id(pa), LB.id(pb)); });
    }
}

// ------------------------------------------------------------------ row-wise match masks
struct PlainList {
    const int32_t* v;
    __device__ __forceinline__ int32_t key(int64_t i) const { return __ldg(v + i); }
};

// segment_isinis_m (skip_neg1) / segment_isinmm: row r of a against row r of b.
__global__ void __launch_bounds__(kRBlock) isin_mask_kernel(const int32_t* a_cols, int64_t a_len, const int32_t* a_rp,
                                                            const int32_t* b_cols, int64_t b_len, const int32_t* b_rp,
                                                            int64_t rows, uint8_t* m1, uint8_t* m2,
                                                            int skip_neg1) {
    __shared__ int32_t s_key[kRWarps][kRSlots];
    __shared__ int32_t s_pos[kRWarps][kRSlots];
    const int wib = threadIdx.x / kWarp;
    const unsigned lane = lane_id();
    const PlainList A{a_cols}, B{b_cols};
    const int64_t nw = (int64_t)gridDim.x * kRWarps;
    for (int64_t r = (int64_t)blockIdx.x * kRWarps + wib; r < rows; r += nw) {
        int64_t ab = __ldg(a_rp + r), ae = __ldg(a_rp + r + 1), bb = __ldg(b_rp + r), be = __ldg(b_rp + r + 1);
        ab = ab < 0 ? 0 : (ab > a_len ? a_len : ab);
        ae = ae < ab ? ab : (ae > a_len ? a_len : ae);
        bb = bb < 0 ? 0 : (bb > b_len ? b_len : bb);
        be = be < bb ? bb : (be > b_len ? b_len : be);
        warp_pairs(A, ab, ae, B, bb, be, skip_neg1 != 0, s_key[wib], s_pos[wib], lane,
                   [&](int64_t pa, int64_t pb) {
                       m1[pa] = 1;
                       m2[pb] = 1;
                   });
    }
}

// sub_suppport_affect: triangle (e_curr_rep[i], left[i], right[i]) with the
// other two edges' flags mask1/mask2 (set: that edge takes part).
__global__ void support_affect_kernel(const int32_t* left, const int32_t* right, const int32_t* cur, int64_t n,
                                      int32_t* support, int64_t E, const uint8_t* m1, const uint8_t* m2,
                                      uint8_t* affect) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t a = left[i], b = right[i], c = cur[i];
        const bool sa = m1[i], sb = m2[i];
        const bool da = sa && (sb || c < b), db = sb && (sa || c < a);
        if (da && a >= 0 && a < E) {
            atomicSub(support + a, 1);
            affect[a] = 1;
        }
        if (db && b >= 0 && b < E) {
            atomicSub(support + b, 1);
            affect[b] = 1;
        }
    }
}

}  // namespace

static int launch_peel_op(int variant, const PeelOpArgs& A, cudaStream_t st) {
    TDT_CHECK_ARG(A.n_curr >= 0 && A.E >= 0, "negative size");
    TDT_CHECK_ARG(A.n_cut >= 1, "n_cut must be >= 1");
    TDT_CHECK_ARG(A.n_curr == 0 || (A.e_curr && A.rows && A.columns && A.support && A.e_mask && A.n_mark &&
                                    A.in_curr),
                  "null pointer");
    TDT_CHECK_ARG(A.n_curr <= INT64_MAX / 32 / A.n_cut, "e_curr too long");
    if (A.n_curr == 0) return TDT_OK;
    DeviceInfo di;
    int rc = device_info(&di);
    if (rc) return rc;
    const unsigned grid = grid_for(A.n_curr * A.n_cut * kWarp, kRBlock, di.sms, 16);
    switch (variant) {
        case kVarUnd: peel_op_kernel<kVarUnd><<<grid, kRBlock, 0, st>>>(A); break;
        case kVarOO: peel_op_kernel<kVarOO><<<grid, kRBlock, 0, st>>>(A); break;
        case kVarII: peel_op_kernel<kVarII><<<grid, kRBlock, 0, st>>>(A); break;
        default: peel_op_kernel<kVarOI><<<grid, kRBlock, 0, st>>>(A); break;
    }
    TDT_LAUNCH_CHECK("peel_op");
    return TDT_OK;
}

static int launch_isin_mask(const int32_t* a, int64_t a_len, const int32_t* a_rp, const int32_t* b, int64_t b_len,
                            const int32_t* b_rp, int64_t rows, uint8_t* m1, uint8_t* m2, int skip_neg1,
                            cudaStream_t st) {
    TDT_CHECK_ARG(rows >= 0 && a_len >= 0 && b_len >= 0, "negative size");
    if (rows == 0) return TDT_OK;
    TDT_CHECK_ARG(a_rp && b_rp && (a_len == 0 || (a && m1)) && (b_len == 0 || (b && m2)), "null pointer");
    DeviceInfo di;
    int rc = device_info(&di);
    if (rc) return rc;
    isin_mask_kernel<<<grid_for(rows * kWarp, kRBlock, di.sms, 16), kRBlock, 0, st>>>(a, a_len, a_rp, b, b_len, b_rp,
                                                                                       rows, m1, m2, skip_neg1);
    TDT_LAUNCH_CHECK("isin_mask");
    return TDT_OK;
}

}  // namespace tdt

using namespace tdt;
#define API extern "C" __attribute__((visibility("default")))

API int tdt_segment_isinis_m(const int32_t* a_columns, int64_t a_len, const int32_t* a_row_ptr,
                             const int32_t* b_columns, int64_t b_len, const int32_t* b_row_ptr, int64_t num_rows,
                             uint8_t* mask1, uint8_t* mask2, tdt_stream_t stream) {
    return launch_isin_mask(a_columns, a_len, a_row_ptr, b_columns, b_len, b_row_ptr, num_rows, mask1, mask2, 1,
                            (cudaStream_t)stream);
}

API int tdt_segment_isinmm(const int32_t* u_clos, int64_t u_len, const int32_t* v_clos, int64_t v_len,
                           const int32_t* uptr, const int32_t* vptr, int64_t num_rows, uint8_t* u_mask,
                           uint8_t* v_mask, tdt_stream_t stream) {
    return launch_isin_mask(u_clos, u_len, uptr, v_clos, v_len, vptr, num_rows, u_mask, v_mask, 0,
                            (cudaStream_t)stream);
}

API int tdt_sub_suppport_affect(const int32_t* left_nbr, const int32_t* right_nbr, const int32_t* e_curr_rep,
                                int64_t num_triangles, int32_t* support, int64_t num_edges, const uint8_t* mask1,
                                const uint8_t* mask2, uint8_t* e_affect_mask, int32_t l, tdt_stream_t stream) {
    (void)l;  // the reference passes it on and does not use it
    TDT_CHECK_ARG(num_triangles >= 0 && num_edges >= 0, "negative size");
    if (num_triangles == 0) return TDT_OK;
    TDT_CHECK_ARG(left_nbr && right_nbr && e_curr_rep && support && mask1 && mask2 && e_affect_mask,
                  "null pointer");
    DeviceInfo di;
    int rc = device_info(&di);
    if (rc) return rc;
    support_affect_kernel<<<grid_for(num_triangles, 256, di.sms, 16), 256, 0, (cudaStream_t)stream>>>(
        left_nbr, right_nbr, e_curr_rep, num_triangles, support, num_edges, mask1, mask2, e_affect_mask);
    TDT_LAUNCH_CHECK("support_affect");
    return TDT_OK;
}

static PeelOpArgs peel_args(const int32_t* e_curr, int64_t n_curr, const int32_t* rows, const int32_t* columns,
                            int64_t num_edges, int32_t* support, const uint8_t* e_mask, uint8_t* n_mark,
                            const uint8_t* in_curr, int32_t l, int32_t n_cut) {
    PeelOpArgs A{};
    A.e_curr = e_curr;
    A.n_curr = n_curr;
    A.rows = rows;
    A.columns = columns;
    A.E = num_edges;
    A.support = support;
    A.e_mask = e_mask;
    A.n_mark = n_mark;
    A.in_curr = in_curr;
    A.l = l + 1;  // the reference's op hands l + 1 to its kernel
    A.n_cut = n_cut;
    return A;
}

API int tdt_peeling_undirect_tile(const int32_t* e_curr, int64_t n_curr, const int32_t* rows, const int32_t* columns,
                                  const int32_t* columns_g, const int32_t* row_ptr, int64_t row_ptr_len,
                                  const int32_t* edges_id_nbr, int64_t g_len, int32_t* support,
                                  const uint8_t* e_mask, uint8_t* n_mark, const uint8_t* in_curr, int32_t l,
                                  int32_t n_cut, int64_t num_edges, tdt_stream_t stream) {
    PeelOpArgs A = peel_args(e_curr, n_curr, rows, columns, num_edges, support, e_mask, n_mark, in_curr, l, n_cut);
    TDT_CHECK_ARG(n_curr == 0 || (columns_g && row_ptr && edges_id_nbr), "null pointer");
    A.columns_g = columns_g;
    A.edges_id_nbr = edges_id_nbr;
    A.g_len = g_len;
    A.row_ptr = row_ptr;
    A.row_ptr_len = row_ptr_len;
    return launch_peel_op(kVarUnd, A, (cudaStream_t)stream);
}
API int tdt_peeling_undirect(const int32_t* e_curr, int64_t n_curr, const int32_t* rows, const int32_t* columns,
                             const int32_t* columns_g, const int32_t* row_ptr, int64_t row_ptr_len,
                             const int32_t* edges_id_nbr, int64_t g_len, int32_t* support, const uint8_t* e_mask,
                             uint8_t* n_mark, const uint8_t* in_curr, int32_t l, int64_t num_edges,
                             tdt_stream_t stream) {
    return tdt_peeling_undirect_tile(e_curr, n_curr, rows, columns, columns_g, row_ptr, row_ptr_len, edges_id_nbr,
                                     g_len, support, e_mask, n_mark, in_curr, l, 1, num_edges, stream);
}

API int tdt_peeling_direct_tile_oo(const int32_t* e_curr, int64_t n_curr, const int32_t* rows,
                                   const int32_t* columns, const int32_t* row_ptr, int64_t row_ptr_len,
                                   int32_t* support, const uint8_t* e_mask, uint8_t* n_mark, const uint8_t* in_curr,
                                   int32_t l, int32_t n_cut, int64_t num_edges, tdt_stream_t stream) {
    PeelOpArgs A = peel_args(e_curr, n_curr, rows, columns, num_edges, support, e_mask, n_mark, in_curr, l, n_cut);
    TDT_CHECK_ARG(n_curr == 0 || row_ptr, "null pointer");
    A.row_ptr = row_ptr;
    A.row_ptr_len = row_ptr_len;
    return launch_peel_op(kVarOO, A, (cudaStream_t)stream);
}
API int tdt_peeling_direct_oo(const int32_t* e_curr, int64_t n_curr, const int32_t* rows, const int32_t* columns,
                              const int32_t* row_ptr, int64_t row_ptr_len, int32_t* support, const uint8_t* e_mask,
                              uint8_t* n_mark, const uint8_t* in_curr, int32_t l, int64_t num_edges,
                              tdt_stream_t stream) {
    return tdt_peeling_direct_tile_oo(e_curr, n_curr, rows, columns, row_ptr, row_ptr_len, support, e_mask, n_mark,
                                      in_curr, l, 1, num_edges, stream);
}

API int tdt_peeling_direct_tile_ii(const int32_t* e_curr, int64_t n_curr, const int32_t* rows,
                                   const int32_t* columns, const int32_t* r_edges, const int32_t* re_ptr,
                                   int64_t re_ptr_len, int32_t* support, const uint8_t* e_mask, uint8_t* n_mark,
                                   const uint8_t* in_curr, int32_t l, int32_t n_cut, int64_t num_edges,
                                   tdt_stream_t stream) {
    PeelOpArgs A = peel_args(e_curr, n_curr, rows, columns, num_edges, support, e_mask, n_mark, in_curr, l, n_cut);
    TDT_CHECK_ARG(n_curr == 0 || (r_edges && re_ptr), "null pointer");
    A.r_edges = r_edges;
    A.r_len = num_edges;
    A.re_ptr = re_ptr;
    A.re_ptr_len = re_ptr_len;
    return launch_peel_op(kVarII, A, (cudaStream_t)stream);
}
API int tdt_peeling_direct_ii(const int32_t* e_curr, int64_t n_curr, const int32_t* rows, const int32_t* columns,
                              const int32_t* r_edges, const int32_t* re_ptr, int64_t re_ptr_len, int32_t* support,
                              const uint8_t* e_mask, uint8_t* n_mark, const uint8_t* in_curr, int32_t l,
                              int64_t num_edges, tdt_stream_t stream) {
    return tdt_peeling_direct_tile_ii(e_curr, n_curr, rows, columns, r_edges, re_ptr, re_ptr_len, support, e_mask,
                                      n_mark, in_curr, l, 1, num_edges, stream);
}

API int tdt_peeling_direct_tile_oi(const int32_t* e_curr, int64_t n_curr, const int32_t* rows,
                                   const int32_t* columns, const int32_t* row_ptr, int64_t row_ptr_len,
                                   const int32_t* r_edges, const int32_t* re_ptr, int64_t re_ptr_len,
                                   int32_t* support, const uint8_t* e_mask, uint8_t* n_mark, const uint8_t* in_curr,
                                   int32_t l, int32_t n_cut, int64_t num_edges, tdt_stream_t stream) {
    PeelOpArgs A = peel_args(e_curr, n_curr, rows, columns, num_edges, support, e_mask, n_mark, in_curr, l, n_cut);
    TDT_CHECK_ARG(n_curr == 0 || (row_ptr && r_edges && re_ptr), "null pointer");
    A.row_ptr = row_ptr;
    A.row_ptr_len = row_ptr_len;
    A.r_edges = r_edges;
    A.r_len = num_edges;
    A.re_ptr = re_ptr;
    A.re_ptr_len = re_ptr_len;
    return launch_peel_op(kVarOI, A, (cudaStream_t)stream);
}
API int tdt_peeling_direct_oi(const int32_t* e_curr, int64_t n_curr, const int32_t* rows, const int32_t* columns,
                              const int32_t* row_ptr, int64_t row_ptr_len, const int32_t* r_edges,
                              const int32_t* re_ptr, int64_t re_ptr_len, int32_t* support, const uint8_t* e_mask,
                              uint8_t* n_mark, const uint8_t* in_curr, int32_t l, int64_t num_edges,
                              tdt_stream_t stream) {
    return tdt_peeling_direct_tile_oi(e_curr, n_curr, rows, columns, row_ptr, row_ptr_len, r_edges, re_ptr,
                                      re_ptr_len, support, e_mask, n_mark, in_curr, l, 1, num_edges, stream);
}
