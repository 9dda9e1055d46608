// Graph preprocessing on the device: raw edge list -> degree-oriented CSRCOO.
//
// Restates read_prepro_save (singlegpu_truss.py:172-178):
//   Graph.read_edgelist (src/type/Graph_Truss.py:177-213): drop self-loops
//     (:188), dedup unordered pairs (:200-202), rank vertices by degree
//     (:209-211; the reference's numpy argsort is unstable, here ties go to
//     the smaller id, and an optional vertex group ranks first so a batch of
//     graphs keeps contiguous rank ranges);
//   CSRCOO.edge_list_to_Graph (src/type/CSRCOO.py:128-162) + counter_sort
//     (:169-177): relabel by rank, orient low->high, CSR sorted by (row, col).
//
// Pipeline (every size that varies is read on the device, so there is no
// host synchronisation between the steps):
//   1. key = (min << B) | max per draw (self-loops -> sentinel), radix sort
//   2. keep the first of each run of equal keys (scan + scatter) -> E_out
//   3. degrees by atomics; present vertices -> (group, degree, id) keys
//   4. radix sort the vertex keys -> rank of every id, vertices[rank]
//   5. relabel + orient each edge -> (lo << B2) | hi, radix sort
//   6. rows / cols, row counts -> scan -> row_ptr
#include "common.cuh"
#include "sort.cuh"

namespace tdt {

static int bits_for(uint64_t x) {  // bits needed to hold values < x (x >= 1)
    int b = 0;
    while (b < 64 && (x - 1) >> b) b++;
    return b < 1 ? 1 : b;
}

__global__ void pp_edge_keys(const int32_t* __restrict__ src, const int32_t* __restrict__ dst, int64_t m,
                             int64_t num_ids, int B, uint64_t sentinel, uint64_t* __restrict__ keys, int* status) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t a = src[i], b = dst[i];
        if (a < 0 || b < 0 || a >= num_ids || b >= num_ids) {
            atomicMax(status, (int)TDT_ERR_INVALID);
            keys[i] = sentinel;
            continue;
        }
        if (a == b) { keys[i] = sentinel; continue; }
        const uint64_t lo = (uint64_t)(a < b ? a : b), hi = (uint64_t)(a < b ? b : a);
        keys[i] = (lo << B) | hi;
    }
}

// first-of-run flags of the sorted keys (sentinels excluded)
__global__ void pp_unique_flags(const uint64_t* __restrict__ keys, int64_t m, uint64_t sentinel,
                                uint32_t* __restrict__ flags) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t k = keys[i];
        flags[i] = (k != sentinel && (i == 0 || keys[i - 1] != k)) ? 1u : 0u;
    }
}

__global__ void pp_unique_scatter(const uint64_t* __restrict__ keys, const uint32_t* __restrict__ flags,
                                  const uint32_t* __restrict__ pos, int64_t m, int B, uint64_t* __restrict__ ukeys,
                                  int32_t* __restrict__ deg) {
    const uint64_t mask = (1ull << B) - 1;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        if (!flags[i]) continue;
        const uint64_t k = keys[i];
        ukeys[pos[i]] = k;
        atomicAdd(deg + (k >> B), 1);
        atomicAdd(deg + (k & mask), 1);
    }
}

// vertex keys: present ids -> (group, degree, id); absent ids -> sentinel
__global__ void pp_vertex_keys(const int32_t* __restrict__ deg, const int32_t* __restrict__ group, int64_t num_ids,
                               int B, int D, uint64_t* __restrict__ vkeys) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < num_ids;
         v += (int64_t)gridDim.x * blockDim.x) {
        const int32_t d = deg[v];
        if (d == 0) { vkeys[v] = ~0ull; continue; }
        const uint64_t g = group ? (uint64_t)group[v] : 0ull;
        vkeys[v] = (g << (B + D)) | ((uint64_t)d << B) | (uint64_t)v;
    }
}

// sorted vertex keys -> rank[id], vertices[rank]; V_out = number of present ids
__global__ void pp_ranks(const uint64_t* __restrict__ vkeys, int64_t num_ids, int B, int32_t* __restrict__ rank,
                         int32_t* __restrict__ vertices, unsigned long long* __restrict__ vcount) {
    const uint64_t mask = (1ull << B) - 1;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < num_ids;
         p += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t k = vkeys[p];
        if (k == ~0ull) continue;
        const int32_t id = (int32_t)(k & mask);
        rank[id] = (int32_t)p;
        vertices[p] = id;
        atomicAdd(vcount, 1ull);
    }
}

// relabel the unique edges (positions >= E_out become sentinels)
__global__ void pp_relabel(const uint64_t* __restrict__ ukeys, const uint32_t* __restrict__ e_out, int64_t m, int B,
                           int B2, const int32_t* __restrict__ rank, uint64_t* __restrict__ keys2) {
    const uint64_t mask = (1ull << B) - 1;
    const int64_t eo = (int64_t)*e_out;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        if (i >= eo) { keys2[i] = ~0ull; continue; }
        const uint64_t k = ukeys[i];
        const uint64_t a = (uint64_t)rank[k >> B], b = (uint64_t)rank[k & mask];
        keys2[i] = ((a < b ? a : b) << B2) | (a < b ? b : a);
    }
}

__global__ void pp_emit(const uint64_t* __restrict__ keys2, const uint32_t* __restrict__ e_out, int B2,
                        int32_t* __restrict__ rows, int32_t* __restrict__ cols, int32_t* __restrict__ rowcnt) {
    const uint64_t mask = (1ull << B2) - 1;
    const int64_t eo = (int64_t)*e_out;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < eo; i += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t k = keys2[i];
        const int32_t r = (int32_t)(k >> B2);
        rows[i] = r;
        cols[i] = (int32_t)(k & mask);
        atomicAdd(rowcnt + r, 1);
    }
}

__global__ void pp_counts(const uint32_t* __restrict__ e_out, const unsigned long long* __restrict__ vcount,
                          const int* __restrict__ status, int64_t* __restrict__ counts) {
    counts[0] = (int64_t)*e_out;
    counts[1] = (int64_t)*vcount;
    counts[2] = *status;
}

namespace {
struct PpLayout {
    uint64_t* k0;
    uint64_t* k1;
    uint32_t* flags;
    uint32_t* pos;      // +1 entry: total
    int32_t* deg;
    int32_t* rank;
    uint64_t* v0;
    uint64_t* v1;
    int32_t* rowcnt;
    unsigned long long* vcount;
    int* status;
    void* scan_ws;
    void* sort_ws;
    size_t total;
};

PpLayout pp_carve(void* ws, int64_t m, int64_t n) {
    char* base = reinterpret_cast<char*>(ws);
    size_t off = 0;
    auto take = [&](size_t bytes) -> void* {
        off = (off + 255) & ~(size_t)255;
        void* p = base ? base + off : nullptr;
        off += bytes;
        return p;
    };
    const size_t M = (size_t)(m > 0 ? m : 1), N = (size_t)(n > 0 ? n : 1);
    PpLayout L;
    L.k0 = (uint64_t*)take(8 * M);
    L.k1 = (uint64_t*)take(8 * M);
    L.flags = (uint32_t*)take(4 * M);
    L.pos = (uint32_t*)take(4 * (M + 1));
    L.deg = (int32_t*)take(4 * N);
    L.rank = (int32_t*)take(4 * N);
    L.v0 = (uint64_t*)take(8 * N);
    L.v1 = (uint64_t*)take(8 * N);
    L.rowcnt = (int32_t*)take(4 * N);
    L.vcount = (unsigned long long*)take(256);
    L.status = (int*)take(256);
    L.scan_ws = take(scan_scratch_bytes((int64_t)(M > N ? M : N) + 1));
    L.sort_ws = take(radix_sort_scratch_bytes((int64_t)(M > N ? M : N)));
    L.total = off + 256;
    return L;
}
}  // namespace

size_t preprocess_workspace_bytes(int64_t m, int64_t n) { return pp_carve(nullptr, m, n).total; }

int run_preprocess(const int32_t* src, const int32_t* dst, int64_t m, int64_t num_ids, const int32_t* group,
                   int32_t num_groups, int32_t* rows, int32_t* cols, int64_t* row_ptr, int32_t* vertices,
                   int64_t* counts, void* ws, size_t ws_bytes, cudaStream_t st) {
    TDT_CHECK_ARG(m >= 0 && num_ids >= 0, "negative size");
    TDT_CHECK_ARG(m < (int64_t)UINT32_MAX - 1, "too many edges for one preprocessing call");
    TDT_CHECK_ARG(num_ids < (int64_t)INT32_MAX, "vertex ids must fit int32");
    TDT_CHECK_ARG(counts && row_ptr, "null output");
    TDT_CHECK_ARG(m == 0 || (src && dst && rows && cols), "null edge pointer");
    TDT_CHECK_ARG(num_ids == 0 || vertices, "null vertices");
    const size_t need = preprocess_workspace_bytes(m, num_ids);
    if (!ws || ws_bytes < need) {
        set_error("preprocess workspace of %zu bytes < required %zu", ws_bytes, need);
        return TDT_ERR_WORKSPACE;
    }
    DeviceInfo di;
    int rc = device_info(&di);
    if (rc) return rc;
    PpLayout L = pp_carve(ws, m, num_ids);
    TDT_CUDA(cudaMemsetAsync(L.status, 0, 256, st));
    TDT_CUDA(cudaMemsetAsync(L.vcount, 0, 256, st));
    TDT_CUDA(cudaMemsetAsync(row_ptr, 0, 8 * (size_t)(num_ids + 1), st));
    if (m == 0 || num_ids == 0) {
        TDT_CUDA(cudaMemsetAsync(counts, 0, 3 * sizeof(int64_t), st));
        return TDT_OK;
    }
    const int B = bits_for((uint64_t)num_ids);
    const int D = bits_for((uint64_t)num_ids + 1);  // degrees < num_ids in a simple graph
    const int GB = group ? bits_for((uint64_t)(num_groups > 0 ? num_groups : 1)) : 0;
    TDT_CHECK_ARG(2 * B + 1 <= 64 && B + D + GB + 1 <= 64, "id/degree/group bits (%d/%d/%d) exceed 64", B, D, GB);
    const uint64_t sentinel = (1ull << (2 * B)) - 1;
    const int tb = 256;
    const unsigned g_m = grid_for(m, tb, di.sms, 16), g_n = grid_for(num_ids, tb, di.sms, 16);
    // 1. edge keys, sorted
    pp_edge_keys<<<g_m, tb, 0, st>>>(src, dst, m, num_ids, B, sentinel, L.k0, L.status);
    TDT_LAUNCH_CHECK("pp_edge_keys");
    bool alt = false;
    rc = radix_sort_pairs<uint64_t>(L.k0, nullptr, L.k1, nullptr, m, 0, 2 * B, L.sort_ws, &alt, st);
    if (rc) return rc;
    uint64_t* sk = alt ? L.k1 : L.k0;
    uint64_t* uk = alt ? L.k0 : L.k1;
    // 2. dedup
    pp_unique_flags<<<g_m, tb, 0, st>>>(sk, m, sentinel, L.flags);
    TDT_LAUNCH_CHECK("pp_unique_flags");
    rc = exclusive_scan<uint32_t, uint32_t>(L.flags, L.pos, m, L.pos + m, L.scan_ws, st);
    if (rc) return rc;
    TDT_CUDA(cudaMemsetAsync(L.deg, 0, 4 * (size_t)num_ids, st));
    pp_unique_scatter<<<g_m, tb, 0, st>>>(sk, L.flags, L.pos, m, B, uk, L.deg);
    TDT_LAUNCH_CHECK("pp_unique_scatter");
    const uint32_t* e_out = L.pos + m;
    // 3-4. rank vertices by (group, degree, id)
    pp_vertex_keys<<<g_n, tb, 0, st>>>(L.deg, group, num_ids, B, D, L.v0);
    TDT_LAUNCH_CHECK("pp_vertex_keys");
    // absent ids carry ~0, which stays above every key on the low GB+D+B+1 bits
    rc = radix_sort_pairs<uint64_t>(L.v0, nullptr, L.v1, nullptr, num_ids, 0, GB + D + B + 1, L.sort_ws, &alt, st);
    if (rc) return rc;
    const uint64_t* svk = alt ? L.v1 : L.v0;
    pp_ranks<<<g_n, tb, 0, st>>>(svk, num_ids, B, L.rank, vertices, L.vcount);
    TDT_LAUNCH_CHECK("pp_ranks");
    // 5. relabel + orient, sort by (row, col)
    uint64_t* k2 = sk;  // the sorted draw keys are no longer needed
    pp_relabel<<<g_m, tb, 0, st>>>(uk, e_out, m, B, B, L.rank, k2);
    TDT_LAUNCH_CHECK("pp_relabel");
    rc = radix_sort_pairs<uint64_t>(k2, nullptr, uk, nullptr, m, 0, 2 * B + 1, L.sort_ws, &alt, st);
    if (rc) return rc;
    const uint64_t* sk2 = alt ? uk : k2;
    // 6. CSRCOO
    TDT_CUDA(cudaMemsetAsync(L.rowcnt, 0, 4 * (size_t)num_ids, st));
    pp_emit<<<g_m, tb, 0, st>>>(sk2, e_out, B, rows, cols, L.rowcnt);
    TDT_LAUNCH_CHECK("pp_emit");
    rc = exclusive_scan<int32_t, int64_t>(L.rowcnt, row_ptr, num_ids, row_ptr + num_ids, L.scan_ws, st);
    if (rc) return rc;
    pp_counts<<<1, 1, 0, st>>>(e_out, L.vcount, L.status, counts);
    TDT_LAUNCH_CHECK("pp_counts");
    return TDT_OK;
}

}  // namespace tdt

extern "C" __attribute__((visibility("default"))) size_t tdt_preprocess_workspace_bytes(int64_t num_draws,
                                                                                       int64_t num_ids) {
    return tdt::preprocess_workspace_bytes(num_draws, num_ids);
}

extern "C" __attribute__((visibility("default"))) int tdt_preprocess(
    const int32_t* src, const int32_t* dst, int64_t num_draws, int64_t num_ids, const int32_t* vertex_group,
    int32_t num_groups, int32_t* rows, int32_t* cols, int64_t* row_ptr, int32_t* vertices, int64_t* counts,
    void* workspace, size_t workspace_bytes, tdt_stream_t stream) {
    return tdt::run_preprocess(src, dst, num_draws, num_ids, vertex_group, num_groups, rows, cols, row_ptr, vertices,
                               counts, workspace, workspace_bytes, (cudaStream_t)stream);
}
