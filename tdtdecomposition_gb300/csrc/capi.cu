// extern "C" entry points of libtdt_gb300.so (declared in include/tdt_gb300.h).
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <atomic>
#include <mutex>

#include <nvtx3/nvToolsExt.h>

#include "common.cuh"

namespace tdt {

static thread_local char g_err[512];
static unsigned long long g_launches = 0;

void note_launch() { __atomic_fetch_add(&g_launches, 1ull, __ATOMIC_RELAXED); }

// Phase timing of the whole-path calls (CUDA events on the launching stream).
constexpr int kPhases = 5;
struct PhaseRec {
    cudaEvent_t ev[kPhases];
};
static PhaseRec* g_prof = nullptr;
static int g_prof_cap = 0, g_prof_n = 0, g_prof_on = 0;

// NVTX ranges of the phases on the calling thread (no-ops unless a profiler
// is attached).  A call that ended early between two marks leaves its range
// open; the next call's start closes it.
static thread_local int t_nvtx_depth = 0;
static const char* const kPhaseNames[4] = {"tdt support", "tdt listing", "tdt peel", "tdt outputs"};
static void nvtx_mark(int phase) {
    if (phase == 0) {
        for (; t_nvtx_depth > 0; t_nvtx_depth--) nvtxRangePop();
    } else if (t_nvtx_depth > 0) {
        nvtxRangePop();
        t_nvtx_depth--;
    }
    if (phase >= 0 && phase < 4) {
        nvtxRangePushA(kPhaseNames[phase]);
        t_nvtx_depth++;
    }
}

// Called by run_peel: phase 0 = start, 1 = after the support pass, 2 = after
// the listing pass, 3 = after the peel, 4 = end.
void prof_mark(int phase, cudaStream_t st) {
    nvtx_mark(phase);
    if (!g_prof_on) return;
    if (phase == 0) {
        if (g_prof_n >= g_prof_cap) return;
        g_prof_n++;
    }
    if (g_prof_n == 0 || g_prof_n > g_prof_cap) return;
    cudaEventRecord(g_prof[g_prof_n - 1].ev[phase], st);
}

void set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

int cuda_status(cudaError_t e, const char* what) {
    set_error("%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? TDT_ERR_WORKSPACE : TDT_ERR_CUDA;
}

// Per-device attributes, cached.  Calls come from several host threads (the
// server ingests on one and decomposes on another): a cache entry is
// published with a release store of its flag after it is written, and read
// only after an acquire load of the flag sees it.
int device_info(DeviceInfo* out) {
    static DeviceInfo cache[64];
    static std::atomic<bool> have[64];
    int dev = 0;
    TDT_CUDA(cudaGetDevice(&dev));
    if (dev >= 0 && dev < 64 && have[dev].load(std::memory_order_acquire)) {
        *out = cache[dev];
        return TDT_OK;
    }
    DeviceInfo di;
    di.device = dev;
    TDT_CUDA(cudaDeviceGetAttribute(&di.sms, cudaDevAttrMultiProcessorCount, dev));
    TDT_CUDA(cudaDeviceGetAttribute(&di.max_smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    TDT_CUDA(cudaDeviceGetAttribute(&di.cc_major, cudaDevAttrComputeCapabilityMajor, dev));
    TDT_CUDA(cudaDeviceGetAttribute(&di.cc_minor, cudaDevAttrComputeCapabilityMinor, dev));
    if (di.cc_major != 10 || di.cc_minor != 3) {
        set_error("device %d is sm_%d%d; this library is built for sm_103a (GB300) only", dev, di.cc_major,
                  di.cc_minor);
        return TDT_ERR_UNSUPPORTED;
    }
    if (dev >= 0 && dev < 64 && !have[dev].load(std::memory_order_acquire)) {
        static std::mutex m;
        std::lock_guard<std::mutex> lk(m);
        if (!have[dev].load(std::memory_order_relaxed)) {
            cache[dev] = di;
            have[dev].store(true, std::memory_order_release);
        }
    }
    *out = di;
    return TDT_OK;
}

// ops.cu
int launch_segment_add(const int32_t*, const int32_t*, int32_t*, int64_t, int64_t, cudaStream_t);
int launch_affect(int mode, const int32_t*, int64_t, const int32_t*, const int32_t*, const int32_t*, int64_t,
                  int32_t, const uint8_t*, int32_t, uint8_t*, int32_t*, int32_t, uint8_t*, int32_t*, int32_t*,
                  int64_t, cudaStream_t);
int launch_support_k(const int32_t*, const int32_t*, const int32_t*, int64_t, int32_t, int32_t, int32_t*, int64_t,
                     cudaStream_t);
int launch_sub_affect(const int32_t*, const int32_t*, const int32_t*, int64_t, int32_t, const uint8_t*, int32_t*,
                      int64_t, cudaStream_t);
// peel.cu
size_t decompose_workspace_bytes(int64_t V, int64_t E);
int run_peel(int mode, const int32_t* rows, const int32_t* cols, const int64_t* rp, int64_t V, int64_t E,
             int32_t fixed_level, int32_t* truss, int32_t* e_truss, int32_t* ptr_truss, int64_t ptr_cap,
             uint8_t* in_k, int32_t* support_out, int64_t* stats, void* ws, size_t ws_bytes, cudaStream_t st);

void set_support_caps(int warp_cap, int heavy_cap);
void set_vector_walk(int on);
void set_bulk_staging(int on);
void set_peel_grid(int half_sms);
void set_peel_deadline(long long ns);
void set_fixed_caps(long long items, long long cands);
void set_peel_dyn_min(long long slots);
int peel_clock(const void* ws, long long* ns, cudaStream_t st);
int test_barrier_timeout(void* ws, long long limit_ns, cudaStream_t st);
int launch_support_accum_i32(const int32_t* rp, int32_t stride, const int32_t* cols, int64_t nv, int64_t ne,
                             int32_t* out, cudaStream_t st);

// The drop-in support op takes no workspace (as in the reference), so it runs
// the support kernel with its scratch-free static schedule.
static int op_support(const int32_t* a_rows, const int32_t* cols, const int32_t* rp, int64_t rp_len, int32_t n_cut,
                      int32_t* out, int64_t n_edges, cudaStream_t st) {
    TDT_CHECK_ARG(n_cut >= 1, "n_cut must be >= 1 (got %d)", n_cut);
    TDT_CHECK_ARG(rp_len >= 1 && (rp_len - 1) % n_cut == 0, "row_ptr length %lld is not V*n_cut+1",
                  (long long)rp_len);
    TDT_CHECK_ARG(n_edges >= 0, "negative size");
    if (n_edges == 0) return TDT_OK;
    TDT_CHECK_ARG(a_rows && cols && rp && out, "null pointer");
    return launch_support_accum_i32(rp, n_cut, cols, (rp_len - 1) / n_cut, n_edges, out, st);
}

}  // namespace tdt

using namespace tdt;

#define API extern "C" __attribute__((visibility("default")))

API const char* tdt_status_string(int s) {
    switch (s) {
        case TDT_OK: return "ok";
        case TDT_ERR_INVALID: return "invalid argument";
        case TDT_ERR_CUDA: return "CUDA error";
        case TDT_ERR_WORKSPACE: return "workspace too small";
        case TDT_ERR_TIMEOUT: return "device wait timed out";
        case TDT_ERR_CAPACITY: return "output capacity exceeded";
        case TDT_ERR_UNSUPPORTED: return "unsupported device or configuration";
        case TDT_ERR_NOT_ORIENTED: return "graph is not oriented low->high (rows[i] < cols[i])";
        default: return "unknown status";
    }
}
API const char* tdt_last_error(void) { return g_err; }
API unsigned long long tdt_launch_count(void) { return __atomic_load_n(&g_launches, __ATOMIC_RELAXED); }

API void tdt_set_support_caps(int warp_cap, int heavy_cap) { set_support_caps(warp_cap, heavy_cap); }
API void tdt_set_vector_walk(int on) { set_vector_walk(on); }
API void tdt_set_bulk_staging(int on) { set_bulk_staging(on); }
API void tdt_set_peel_grid(int half_sms) { set_peel_grid(half_sms); }
API void tdt_set_peel_deadline_ns(long long ns) { set_peel_deadline(ns); }
API void tdt_set_ktruss_batch_caps(long long items, long long cands) { set_fixed_caps(items, cands); }
API void tdt_set_peel_dynamic_min(long long slots) { set_peel_dyn_min(slots); }
API int tdt_peel_clock(const void* workspace, long long* ns, cudaStream_t stream) {
    return peel_clock(workspace, ns, stream);
}
API int tdt_test_barrier_timeout(void* workspace, long long limit_ns, cudaStream_t stream) {
    return test_barrier_timeout(workspace, limit_ns, stream);
}

API int tdt_profile_start(int max_calls) {
    TDT_CHECK_ARG(max_calls > 0 && max_calls <= 4096, "max_calls out of range");
    if (g_prof_cap < max_calls) {
        PhaseRec* p = new PhaseRec[max_calls];
        for (int i = 0; i < max_calls; i++)
            for (int k = 0; k < kPhases; k++) TDT_CUDA(cudaEventCreate(&p[i].ev[k]));
        if (g_prof) {
            for (int i = 0; i < g_prof_cap; i++)
                for (int k = 0; k < kPhases; k++) cudaEventDestroy(g_prof[i].ev[k]);
            delete[] g_prof;
        }
        g_prof = p;
        g_prof_cap = max_calls;
    }
    g_prof_n = 0;
    g_prof_on = 1;
    return TDT_OK;
}

API int tdt_profile_stop(float* ms_phase, int* ncalls) {
    g_prof_on = 0;
    float acc[kPhases - 1] = {0, 0, 0, 0};
    for (int i = 0; i < g_prof_n; i++) {
        TDT_CUDA(cudaEventSynchronize(g_prof[i].ev[kPhases - 1]));
        for (int k = 0; k + 1 < kPhases; k++) {
            float x;
            TDT_CUDA(cudaEventElapsedTime(&x, g_prof[i].ev[k], g_prof[i].ev[k + 1]));
            acc[k] += x;
        }
    }
    if (ms_phase)
        for (int k = 0; k + 1 < kPhases; k++) ms_phase[k] = acc[k];
    if (ncalls) *ncalls = g_prof_n;
    return TDT_OK;
}
API int tdt_version(void) { return 100; }

API int tdt_segment_add(const int32_t* col_indices, int64_t num_values, const int32_t* col_ptr, int32_t* output,
                        int64_t num_rows, tdt_stream_t stream) {
    TDT_CHECK_ARG(num_values >= 0, "num_values < 0");
    return launch_segment_add(col_indices, col_ptr, output, num_rows, num_values, (cudaStream_t)stream);
}

API int tdt_segment_isin2(const int32_t* a_rows, const int32_t* b_col_indices, const int32_t* b_row_ptr,
                          int64_t row_ptr_len, int32_t* output, int64_t num_edges, tdt_stream_t stream) {
    return op_support(a_rows, b_col_indices, b_row_ptr, row_ptr_len, 1, output, num_edges, (cudaStream_t)stream);
}

API int tdt_segment_isin2tile(const int32_t* a_rows, const int32_t* b_col_indices, const int32_t* b_row_ptr,
                              int64_t row_ptr_len, int32_t n_cut, int32_t* output, int64_t num_edges,
                              tdt_stream_t stream) {
    return op_support(a_rows, b_col_indices, b_row_ptr, row_ptr_len, n_cut, output, num_edges,
                      (cudaStream_t)stream);
}

enum { kModeDeleted = 0, kModeNot = 1, kModeNotWin = 2 };

API int tdt_sub_all_affected_support(const int32_t* e_affect, int64_t num_affect, const int32_t* a_rows,
                                     const int32_t* b_col_indices, const int32_t* b_row_ptr, int64_t row_ptr_len,
                                     const uint8_t* mark, int32_t l, uint8_t* n_mark, int32_t* output,
                                     int64_t num_edges, tdt_stream_t stream) {
    return launch_affect(kModeDeleted, e_affect, num_affect, a_rows, b_col_indices, b_row_ptr, row_ptr_len, 1, mark,
                         l, n_mark, output, 0, nullptr, nullptr, nullptr, num_edges, (cudaStream_t)stream);
}
API int tdt_sub_all_affected_support_tile(const int32_t* e_affect, int64_t num_affect, const int32_t* a_rows,
                                          const int32_t* b_col_indices, const int32_t* b_row_ptr,
                                          int64_t row_ptr_len, int32_t n_cut, const uint8_t* mark, int32_t l,
                                          uint8_t* n_mark, int32_t* output, int64_t num_edges,
                                          tdt_stream_t stream) {
    return launch_affect(kModeDeleted, e_affect, num_affect, a_rows, b_col_indices, b_row_ptr, row_ptr_len, n_cut,
                         mark, l, n_mark, output, 0, nullptr, nullptr, nullptr, num_edges, (cudaStream_t)stream);
}
API int tdt_sub_all_affected_support_not(const int32_t* e_affect, int64_t num_affect, const int32_t* a_rows,
                                         const int32_t* b_col_indices, const int32_t* b_row_ptr,
                                         int64_t row_ptr_len, const uint8_t* mark, int32_t l, uint8_t* n_mark,
                                         int32_t* output, int64_t num_edges, tdt_stream_t stream) {
    return launch_affect(kModeNot, e_affect, num_affect, a_rows, b_col_indices, b_row_ptr, row_ptr_len, 1, mark, l,
                         n_mark, output, 0, nullptr, nullptr, nullptr, num_edges, (cudaStream_t)stream);
}
API int tdt_sub_all_affected_support_tilenot(const int32_t* e_affect, int64_t num_affect, const int32_t* a_rows,
                                             const int32_t* b_col_indices, const int32_t* b_row_ptr,
                                             int64_t row_ptr_len, int32_t n_cut, const uint8_t* mark, int32_t l,
                                             uint8_t* n_mark, int32_t* output, int64_t num_edges,
                                             tdt_stream_t stream) {
    return launch_affect(kModeNot, e_affect, num_affect, a_rows, b_col_indices, b_row_ptr, row_ptr_len, n_cut, mark,
                         l, n_mark, output, 0, nullptr, nullptr, nullptr, num_edges, (cudaStream_t)stream);
}
API int tdt_sub_all_affected_support_notwin(const int32_t* e_affect, int64_t num_affect, const int32_t* a_rows,
                                            const int32_t* b_col_indices, const int32_t* b_row_ptr,
                                            int64_t row_ptr_len, const uint8_t* mark, int32_t l, uint8_t* n_mark,
                                            int32_t* output, int32_t windows_high, uint8_t* in_windows_mask,
                                            int32_t* buff_index, int32_t* buf_size, int64_t num_edges,
                                            tdt_stream_t stream) {
    return launch_affect(kModeNotWin, e_affect, num_affect, a_rows, b_col_indices, b_row_ptr, row_ptr_len, 1, mark,
                         l, n_mark, output, windows_high, in_windows_mask, buff_index, buf_size, num_edges,
                         (cudaStream_t)stream);
}
API int tdt_sub_all_affected_support_tilenotwin(const int32_t* e_affect, int64_t num_affect, const int32_t* a_rows,
                                                const int32_t* b_col_indices, const int32_t* b_row_ptr,
                                                int64_t row_ptr_len, int32_t n_cut, const uint8_t* mark, int32_t l,
                                                uint8_t* n_mark, int32_t* output, int32_t windows_high,
                                                uint8_t* in_windows_mask, int32_t* buff_index, int32_t* buf_size,
                                                int64_t num_edges, tdt_stream_t stream) {
    return launch_affect(kModeNotWin, e_affect, num_affect, a_rows, b_col_indices, b_row_ptr, row_ptr_len, n_cut,
                         mark, l, n_mark, output, windows_high, in_windows_mask, buff_index, buf_size, num_edges,
                         (cudaStream_t)stream);
}

API int tdt_segment_isin2_k(const int32_t* a_rows, const int32_t* b_col_indices, const int32_t* b_row_ptr,
                            int64_t row_ptr_len, int32_t k, int32_t* output, int64_t num_edges,
                            tdt_stream_t stream) {
    return launch_support_k(a_rows, b_col_indices, b_row_ptr, row_ptr_len, 1, k, output, num_edges,
                            (cudaStream_t)stream);
}
API int tdt_segment_isin2tile_k(const int32_t* a_rows, const int32_t* b_col_indices, const int32_t* b_row_ptr,
                                int64_t row_ptr_len, int32_t n_cut, int32_t k, int32_t* output, int64_t num_edges,
                                tdt_stream_t stream) {
    return launch_support_k(a_rows, b_col_indices, b_row_ptr, row_ptr_len, n_cut, k, output, num_edges,
                            (cudaStream_t)stream);
}
API int tdt_sub_affected_support(const int32_t* sub_rows, const int32_t* sub_columns, const int32_t* sub_row_ptr,
                                 int64_t row_ptr_len, const uint8_t* mark, int32_t* sub_support, int64_t num_edges,
                                 tdt_stream_t stream) {
    return launch_sub_affect(sub_rows, sub_columns, sub_row_ptr, row_ptr_len, 1, mark, sub_support, num_edges,
                             (cudaStream_t)stream);
}
API int tdt_sub_affected_support_tile(const int32_t* sub_rows, const int32_t* sub_columns,
                                      const int32_t* sub_row_ptr, int64_t row_ptr_len, int32_t n_cut,
                                      const uint8_t* mark, int32_t* sub_support, int64_t num_edges,
                                      tdt_stream_t stream) {
    return launch_sub_affect(sub_rows, sub_columns, sub_row_ptr, row_ptr_len, n_cut, mark, sub_support, num_edges,
                             (cudaStream_t)stream);
}

API size_t tdt_decompose_workspace_bytes(int64_t num_vertices, int64_t num_edges) {
    return decompose_workspace_bytes(num_vertices, num_edges);
}

API int tdt_truss_decompose(const int32_t* rows, const int32_t* cols, const int64_t* row_ptr, int64_t num_vertices,
                            int64_t num_edges, int32_t* truss, int32_t* e_truss, int32_t* ptr_truss,
                            int64_t ptr_truss_cap, int64_t* stats, void* workspace, size_t workspace_bytes,
                            tdt_stream_t stream) {
    return run_peel(0, rows, cols, row_ptr, num_vertices, num_edges, 0, truss, e_truss, ptr_truss, ptr_truss_cap,
                    nullptr, nullptr, stats, workspace, workspace_bytes, (cudaStream_t)stream);
}

API int tdt_triangle_count(const int32_t* cols, const int64_t* row_ptr, int64_t num_vertices, int64_t num_edges,
                           int32_t* support, int64_t* stats, void* workspace, size_t workspace_bytes,
                           tdt_stream_t stream) {
    return run_peel(2, nullptr, cols, row_ptr, num_vertices, num_edges, 0, nullptr, nullptr, nullptr, 0, nullptr,
                    support, stats, workspace, workspace_bytes, (cudaStream_t)stream);
}

API int tdt_ktruss_search(const int32_t* rows, const int32_t* cols, const int64_t* row_ptr, int64_t num_vertices,
                          int64_t num_edges, int32_t k, uint8_t* in_ktruss, int64_t* stats, void* workspace,
                          size_t workspace_bytes, tdt_stream_t stream) {
    TDT_CHECK_ARG(in_ktruss != nullptr || num_edges == 0, "in_ktruss is required");
    // k-truss: every edge in >= k-2 triangles of the remaining graph; peel at
    // level k-3 (support <= k-3) until no edge is left below it.
    return run_peel(1, rows, cols, row_ptr, num_vertices, num_edges, k - 3, nullptr, nullptr, nullptr, 0, in_ktruss,
                    nullptr, stats, workspace, workspace_bytes, (cudaStream_t)stream);
}
