// Drop-in `trusstensor` operators (myhpu_extension.cpp:572-593) for sm_103a.
//
// The reference runs one thread per (edge, tile) and walks a two-pointer merge
// of the two out-lists with scalar loads (kernel.cu:28-685).  Here one warp
// owns one edge: the shorter of the two out-lists is hashed into a per-warp
// shared-memory table (128 keys per pass) and the longer list is streamed
// through it with coalesced loads, 32 columns per step.  Matching on column
// values instead of merging keeps the operators exact on lists that carry the
// reference's -1 sentinels (peeled edges are overwritten with -1 in place,
// singlegpu_truss.py:118), where a binary search would not be.
//
// Tiling (n_cut): tile j of vertex v is [row_ptr[v*n_cut+j], row_ptr[v*n_cut+j+1])
// and tiles partition a row by column value (csr_to_tilingcsr,
// singlegpu_truss.py:160-169), so the union over tiles of the per-tile
// intersections is the intersection of the whole rows; each warp intersects
// whole rows [row_ptr[v*n_cut], row_ptr[v*n_cut+n_cut]).
#include "common.cuh"

namespace tdt {

constexpr int kHashSlots = 256;   // per warp, power of two
constexpr int kHashChunk = 128;   // keys per pass (load factor 1/2)
constexpr int kOpsBlock = 256;    // 8 warps
constexpr int32_t kEmpty = INT32_MIN;

__device__ __forceinline__ unsigned hash_slot(int32_t key) {
    return ((unsigned)key * 2654435761u) >> (32 - 8);  // 8 = log2(kHashSlots)
}

// Intersects cols[a0,a1) and cols[b0,b1) (sorted apart from -1 holes) and calls
// on_match(pa, pb) for every pair of positions holding the same column >= 0.
// All 32 lanes must call it together.
template <class F>
__device__ __forceinline__ void warp_intersect_hash(const int32_t* __restrict__ cols, int64_t a0,
                                                    int64_t a1, int64_t b0, int64_t b1,
                                                    int32_t* hkey, int32_t* hpos, F&& on_match) {
    const unsigned lane = lane_id();
    const int64_t la = a1 - a0, lb = b1 - b0;
    if (la <= 0 || lb <= 0) return;
    const bool a_short = la <= lb;
    const int64_t s0 = a_short ? a0 : b0, s1 = a_short ? a1 : b1;
    const int64_t l0 = a_short ? b0 : a0, l1 = a_short ? b1 : a1;
    for (int64_t c = s0; c < s1; c += kHashChunk) {
        const int64_t ce = min(c + (int64_t)kHashChunk, s1);
        for (int i = lane; i < kHashSlots; i += kWarp) hkey[i] = kEmpty;
        __syncwarp();
        for (int64_t i = c + lane; i < ce; i += kWarp) {
            int32_t key = __ldg(cols + i);
            if (key < 0) continue;
            unsigned h = hash_slot(key);
            for (int probe = 0; probe < kHashSlots; probe++) {
                int32_t old = atomicCAS(&hkey[h], kEmpty, key);
                if (old == kEmpty) { hpos[h] = (int32_t)(i - c); break; }
                h = (h + 1) & (kHashSlots - 1);
            }
        }
        __syncwarp();
        for (int64_t j = l0 + lane; j < l1; j += kWarp) {
            int32_t x = __ldg(cols + j);
            if (x < 0) continue;
            unsigned h = hash_slot(x);
            for (int probe = 0; probe < kHashSlots; probe++) {
                int32_t k = hkey[h];
                if (k == kEmpty) break;
                if (k == x) {
                    int64_t sp = c + hpos[h];
                    if (a_short) on_match(sp, j); else on_match(j, sp);
                    break;
                }
                h = (h + 1) & (kHashSlots - 1);
            }
        }
        __syncwarp();
    }
}

// Row ranges are clamped to [0, n_edges] so a malformed row_ptr cannot move an
// access outside the per-edge arrays.
struct RowView {
    const int32_t* rp;
    int32_t n_cut;
    int64_t nrows;    // vertices = (row_ptr_len - 1) / n_cut
    int64_t n_edges;
    __device__ __forceinline__ bool valid(int32_t v) const { return v >= 0 && v < nrows; }
    __device__ __forceinline__ int64_t clamp(int64_t x) const { return x < 0 ? 0 : (x > n_edges ? n_edges : x); }
    __device__ __forceinline__ int64_t begin(int32_t v) const { return clamp(__ldg(rp + (int64_t)v * n_cut)); }
    __device__ __forceinline__ int64_t end(int32_t v) const {
        int64_t b = begin(v), e = clamp(__ldg(rp + (int64_t)v * n_cut + n_cut));
        return e < b ? b : e;
    }
};

// ------------------------------------------------------------------ segment_add
// kernel.cu:5-26: one thread per row.
__global__ void segment_add_kernel(const int32_t* __restrict__ vals, const int32_t* __restrict__ ptr,
                                   int32_t* __restrict__ out, int64_t nrows, int64_t nvals) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nrows;
         r += (int64_t)gridDim.x * blockDim.x) {
        int32_t s = __ldg(ptr + r), e = __ldg(ptr + r + 1);
        if (nvals >= 0) {  // clamp to the values array when its length is known
            s = s < 0 ? 0 : (s > nvals ? (int32_t)nvals : s);
            e = e < 0 ? 0 : (e > nvals ? (int32_t)nvals : e);
        }
        if (s < e) {
            int32_t sum = 0;
            for (int32_t i = s; i < e; i++) sum += __ldg(vals + i);
            out[r] = sum;
        }
    }
}

// ------------------------------------------------------------------ peel-update operators
enum AffectMode { kAffectDeleted = 0, kAffectNot = 1, kAffectNotWin = 2 };

struct AffectArgs {
    const int32_t* e_affect;
    int64_t n_affect;
    const int32_t* rows;
    const int32_t* cols;
    RowView rv;
    const uint8_t* mark;
    int32_t l;
    uint8_t* n_mark;
    int32_t* out;
    int32_t windows_high;
    uint8_t* in_win;
    int32_t* buff_index;
    int32_t* buf_size;
};

// kernel.cu:144-191/:407-456 (kAffectDeleted), :220-273/:492-547 (kAffectNot),
// :302-370/:578-648 (kAffectNotWin).  One warp per affected edge.
template <int MODE>
__global__ void __launch_bounds__(kOpsBlock) affect_kernel(AffectArgs A) {
    __shared__ int32_t s_key[kOpsBlock / kWarp][kHashSlots];
    __shared__ int32_t s_pos[kOpsBlock / kWarp][kHashSlots];
    const int wib = threadIdx.x / kWarp;
    const unsigned lane = lane_id();
    const int64_t nw = (int64_t)gridDim.x * (kOpsBlock / kWarp);
    for (int64_t i = blockIdx.x * (int64_t)(kOpsBlock / kWarp) + wib; i < A.n_affect; i += nw) {
        const int64_t e = __ldg(A.e_affect + i);
        if (e < 0 || e >= A.rv.n_edges) continue;
        const int32_t u = __ldg(A.rows + e), v = __ldg(A.cols + e);
        if (!A.rv.valid(u) || !A.rv.valid(v)) continue;  // a sentinel edge has no triangles
        const bool me = A.mark[e] != 0;
        int32_t count = 0;
        warp_intersect_hash(A.cols, A.rv.begin(v), A.rv.end(v), A.rv.begin(u), A.rv.end(u),
                            s_key[wib], s_pos[wib], [&](int64_t pa, int64_t pb) {
            const bool ma = A.mark[pa] != 0, mb = A.mark[pb] != 0;
            if (MODE == kAffectDeleted) {
                if (me || ma || mb) {
                    if (*(volatile int32_t*)(A.out + pa) > A.l) { atomicSub(A.out + pa, 1); A.n_mark[pa] = 1; }
                    if (*(volatile int32_t*)(A.out + pb) > A.l) { atomicSub(A.out + pb, 1); A.n_mark[pb] = 1; }
                    if (!me) count++;
                }
            } else {
                if (!(me && ma && mb)) {
                    const int64_t wedge[2] = {pa, pb};
#pragma unroll
                    for (int q = 0; q < 2; q++) {
                        const int64_t x = wedge[q];
                        if (*(volatile int32_t*)(A.out + x) > A.l) {
                            int32_t t = atomicSub(A.out + x, 1);
                            if (t - 1 == A.l) A.n_mark[x] = 1;
                            if (MODE == kAffectNotWin && t == A.windows_high) {
                                A.in_win[x] = 1;
                                const int32_t slot = atomicAdd(A.buf_size, 1);
                                if (slot >= 0 && slot < A.rv.n_edges) A.buff_index[slot] = (int32_t)x;
                            }
                        }
                    }
                    if (me) count++;
                }
            }
        });
        count = warp_sum(count);
        if (lane == 0 && count > 0) {
            if (MODE == kAffectDeleted) {
                atomicSub(A.out + e, count);
                A.n_mark[e] = 1;
            } else {
                int32_t t = atomicSub(A.out + e, count);
                if (t - count <= A.l) A.n_mark[e] = 1;
                if (MODE == kAffectNotWin && t - count < A.windows_high && t >= A.windows_high) {
                    A.in_win[e] = 1;
                    const int32_t slot = atomicAdd(A.buf_size, 1);
                    if (slot >= 0 && slot < A.rv.n_edges) A.buff_index[slot] = (int32_t)e;
                }
            }
        }
    }
}

// ------------------------------------------------------------------ k-truss search operators
struct EdgeOpArgs {
    const int32_t* rows;
    const int32_t* cols;
    RowView rv;
    int64_t n_edges;
    int32_t k;
    const uint8_t* mark;
    int32_t* out;
};

// ktruss_cuda.py:121-200: support saturating at k.
__global__ void __launch_bounds__(kOpsBlock) support_k_kernel(EdgeOpArgs A) {
    __shared__ int32_t s_key[kOpsBlock / kWarp][kHashSlots];
    __shared__ int32_t s_pos[kOpsBlock / kWarp][kHashSlots];
    const int wib = threadIdx.x / kWarp;
    const unsigned lane = lane_id();
    const int64_t nw = (int64_t)gridDim.x * (kOpsBlock / kWarp);
    for (int64_t i = blockIdx.x * (int64_t)(kOpsBlock / kWarp) + wib; i < A.n_edges; i += nw) {
        const int32_t u = __ldg(A.rows + i), v = __ldg(A.cols + i);
        if (!A.rv.valid(u) || !A.rv.valid(v)) continue;
        int32_t count = 0;
        warp_intersect_hash(A.cols, A.rv.begin(v), A.rv.end(v), A.rv.begin(u), A.rv.end(u),
                            s_key[wib], s_pos[wib], [&](int64_t pa, int64_t pb) {
            if (*(volatile int32_t*)(A.out + pa) < A.k) atomicAdd(A.out + pa, 1);
            if (*(volatile int32_t*)(A.out + pb) < A.k) atomicAdd(A.out + pb, 1);
            count++;
        });
        count = warp_sum(count);
        if (lane == 0 && count > 0 && *(volatile int32_t*)(A.out + i) < A.k) atomicAdd(A.out + i, count);
    }
}

// ktruss_cuda.py:201-286: unconditional decrements on an extracted subgraph.
__global__ void __launch_bounds__(kOpsBlock) sub_affect_kernel(EdgeOpArgs A) {
    __shared__ int32_t s_key[kOpsBlock / kWarp][kHashSlots];
    __shared__ int32_t s_pos[kOpsBlock / kWarp][kHashSlots];
    const int wib = threadIdx.x / kWarp;
    const unsigned lane = lane_id();
    const int64_t nw = (int64_t)gridDim.x * (kOpsBlock / kWarp);
    for (int64_t i = blockIdx.x * (int64_t)(kOpsBlock / kWarp) + wib; i < A.n_edges; i += nw) {
        const int32_t u = __ldg(A.rows + i), v = __ldg(A.cols + i);
        if (!A.rv.valid(u) || !A.rv.valid(v)) continue;
        const bool mi = A.mark[i] != 0;
        int32_t count = 0;
        warp_intersect_hash(A.cols, A.rv.begin(v), A.rv.end(v), A.rv.begin(u), A.rv.end(u),
                            s_key[wib], s_pos[wib], [&](int64_t pa, int64_t pb) {
            const bool ma = A.mark[pa] != 0, mb = A.mark[pb] != 0;
            if (mi || ma || mb) {
                if (!ma) atomicSub(A.out + pa, 1);
                if (!mb) atomicSub(A.out + pb, 1);
                if (!mi) count++;
            }
        });
        count = warp_sum(count);
        if (lane == 0 && count > 0) atomicSub(A.out + i, count);
    }
}

// ------------------------------------------------------------------ host launchers
static int ops_grid(int64_t warps_needed) {
    DeviceInfo di;
    if (device_info(&di) != TDT_OK) return -1;
    int64_t blocks = (warps_needed + (kOpsBlock / kWarp) - 1) / (kOpsBlock / kWarp);
    int64_t cap = (int64_t)di.sms * 8;
    if (blocks < 1) blocks = 1;
    return (int)(blocks < cap ? blocks : cap);
}

static int check_rowptr(int64_t row_ptr_len, int32_t n_cut) {
    TDT_CHECK_ARG(n_cut >= 1, "n_cut must be >= 1 (got %d)", n_cut);
    TDT_CHECK_ARG(row_ptr_len >= 1 && (row_ptr_len - 1) % n_cut == 0,
                  "row_ptr length %lld is not V*n_cut+1 for n_cut=%d", (long long)row_ptr_len, n_cut);
    return TDT_OK;
}

int launch_segment_add(const int32_t* vals, const int32_t* ptr, int32_t* out, int64_t nrows, int64_t nvals,
                       cudaStream_t st) {
    TDT_CHECK_ARG(nrows >= 0, "num_rows < 0");
    if (nrows == 0) return TDT_OK;
    TDT_CHECK_ARG(vals && ptr && out, "null pointer");
    DeviceInfo di;
    int rc = device_info(&di);
    if (rc) return rc;
    segment_add_kernel<<<grid_for(nrows, 256, di.sms, 16), 256, 0, st>>>(vals, ptr, out, nrows, nvals);
    TDT_LAUNCH_CHECK("segment_add");
    return TDT_OK;
}

int launch_affect(int mode, const int32_t* e_affect, int64_t n_affect, const int32_t* rows,
                  const int32_t* cols, const int32_t* rp, int64_t row_ptr_len, int32_t n_cut,
                  const uint8_t* mark, int32_t l, uint8_t* n_mark, int32_t* out, int32_t windows_high,
                  uint8_t* in_win, int32_t* buff_index, int32_t* buf_size, int64_t n_edges,
                  cudaStream_t st) {
    int rc = check_rowptr(row_ptr_len, n_cut);
    if (rc) return rc;
    TDT_CHECK_ARG(n_affect >= 0 && n_edges >= 0, "negative size");
    if (n_affect == 0) return TDT_OK;
    TDT_CHECK_ARG(e_affect && rows && cols && rp && mark && n_mark && out, "null pointer");
    if (mode == kAffectNotWin) TDT_CHECK_ARG(in_win && buff_index && buf_size, "null window buffer");
    AffectArgs A{e_affect, n_affect, rows, cols, RowView{rp, n_cut, (row_ptr_len - 1) / n_cut, n_edges},
                 mark, l, n_mark, out, windows_high, in_win, buff_index, buf_size};
    int g = ops_grid(n_affect);
    if (g < 0) return TDT_ERR_CUDA;
    switch (mode) {
        case kAffectDeleted: affect_kernel<kAffectDeleted><<<g, kOpsBlock, 0, st>>>(A); break;
        case kAffectNot: affect_kernel<kAffectNot><<<g, kOpsBlock, 0, st>>>(A); break;
        default: affect_kernel<kAffectNotWin><<<g, kOpsBlock, 0, st>>>(A); break;
    }
    TDT_LAUNCH_CHECK("affect");
    return TDT_OK;
}

int launch_support_k(const int32_t* rows, const int32_t* cols, const int32_t* rp, int64_t row_ptr_len,
                     int32_t n_cut, int32_t k, int32_t* out, int64_t n_edges, cudaStream_t st) {
    int rc = check_rowptr(row_ptr_len, n_cut);
    if (rc) return rc;
    TDT_CHECK_ARG(n_edges >= 0, "negative size");
    if (n_edges == 0) return TDT_OK;
    TDT_CHECK_ARG(rows && cols && rp && out, "null pointer");
    EdgeOpArgs A{rows, cols, RowView{rp, n_cut, (row_ptr_len - 1) / n_cut, n_edges}, n_edges, k, nullptr, out};
    int g = ops_grid(n_edges);
    if (g < 0) return TDT_ERR_CUDA;
    support_k_kernel<<<g, kOpsBlock, 0, st>>>(A);
    TDT_LAUNCH_CHECK("support_k");
    return TDT_OK;
}

int launch_sub_affect(const int32_t* rows, const int32_t* cols, const int32_t* rp, int64_t row_ptr_len,
                      int32_t n_cut, const uint8_t* mark, int32_t* out, int64_t n_edges,
                      cudaStream_t st) {
    int rc = check_rowptr(row_ptr_len, n_cut);
    if (rc) return rc;
    TDT_CHECK_ARG(n_edges >= 0, "negative size");
    if (n_edges == 0) return TDT_OK;
    TDT_CHECK_ARG(rows && cols && rp && mark && out, "null pointer");
    EdgeOpArgs A{rows, cols, RowView{rp, n_cut, (row_ptr_len - 1) / n_cut, n_edges}, n_edges, 0, mark, out};
    int g = ops_grid(n_edges);
    if (g < 0) return TDT_ERR_CUDA;
    sub_affect_kernel<<<g, kOpsBlock, 0, st>>>(A);
    TDT_LAUNCH_CHECK("sub_affect");
    return TDT_OK;
}

}  // namespace tdt
