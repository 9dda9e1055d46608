// Triangle count (per-edge support + total) that allocates no device memory.
//
// Who needs it: callers that cannot call cudaMalloc at the point where they
// want the count -- code that runs while another component owns the device
// allocator (a framework's caching pool, a fixed memory budget carved out up
// front), or latency-critical paths where a cudaMalloc/cudaFree would stall
// the device.  They still provide the graph and the output buffers; the
// scratch the count needs lives in a fixed array inside this library instead
// of a caller-provided workspace.
//
// The scratch is a file-scope __device__ array of kNoAllocScratchBytes.  Every
// GPU that loads the library keeps that array until the process exits.  It
// bounds the graphs this entry point accepts: at most kNoAllocMaxVertices
// vertices and kNoAllocMaxEdges edges; larger graphs are rejected with
// TDT_ERR_INVALID and a message, and should use tdt_triangle_count with a
// workspace.
#include <mutex>

#include "common.cuh"

namespace tdt {

size_t decompose_workspace_bytes(int64_t V, int64_t E);
int run_peel(int mode, const int32_t* rows, const int32_t* cols, const int64_t* rp, int64_t V, int64_t E,
             int32_t fixed_level, int32_t* truss, int32_t* e_truss, int32_t* ptr_truss, int64_t ptr_cap,
             uint8_t* in_k, int32_t* support_out, int64_t* stats, void* ws, size_t ws_bytes, cudaStream_t st);

constexpr int64_t kNoAllocMaxVertices = 1 << 18;
constexpr int64_t kNoAllocMaxEdges = 1 << 18;
// 40 MiB: holds the workspace of kNoAllocMaxVertices vertices and
// kNoAllocMaxEdges edges (35.2 MiB); the first call checks that it does.
constexpr size_t kNoAllocScratchBytes = 40ull << 20;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Host code cannot use g_noalloc_scratch as an address (on the host the name
// only stands for the symbol), so each device's address is looked up once,
// with that device current, and cached.  A cudaDeviceReset by the caller
// unloads the module and makes the cached address stale: this entry point
// must not be used across a cudaDeviceReset.
static std::mutex g_noalloc_mu;
static void* g_noalloc_addr[64] = {nullptr};

static int noalloc_scratch(void** out) {
    int dev = 0;
    TDT_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) {
        set_error("device ordinal %d out of range for the no-allocation scratch table", dev);
        return TDT_ERR_UNSUPPORTED;
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
        const size_t at_limit = decompose_workspace_bytes(kNoAllocMaxVertices, kNoAllocMaxEdges);
        if (at_limit > kNoAllocScratchBytes) {
            set_error("tdt_triangle_count_noalloc: the workspace of its size limit (%zu bytes) exceeds the static "
                      "scratch (%zu bytes)", at_limit, kNoAllocScratchBytes);
            return TDT_ERR_UNSUPPORTED;
        }
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_status(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
        g_noalloc_addr[dev] = p;
    }
    *out = g_noalloc_addr[dev];
    return TDT_OK;
}

}  // namespace tdt

using namespace tdt;

extern "C" __attribute__((visibility("default"))) int tdt_triangle_count_noalloc(
    const int32_t* cols, const int64_t* row_ptr, int64_t num_vertices, int64_t num_edges, int32_t* support,
    int64_t* stats, tdt_stream_t stream) {
    if (num_vertices < 0 || num_edges < 0 || num_vertices > kNoAllocMaxVertices || num_edges > kNoAllocMaxEdges) {
        set_error("tdt_triangle_count_noalloc accepts at most %lld vertices and %lld edges (got %lld, %lld); "
                  "use tdt_triangle_count with a workspace for larger graphs",
                  (long long)kNoAllocMaxVertices, (long long)kNoAllocMaxEdges, (long long)num_vertices,
                  (long long)num_edges);
        return TDT_ERR_INVALID;
    }
    const size_t need = decompose_workspace_bytes(num_vertices, num_edges);
    if (need > kNoAllocScratchBytes) {
        set_error("tdt_triangle_count_noalloc: graph needs %zu scratch bytes, the static scratch holds %zu", need,
                  kNoAllocScratchBytes);
        return TDT_ERR_INVALID;
    }
    void* scratch = nullptr;
    int rc = noalloc_scratch(&scratch);
    if (rc) return rc;
    // run_peel re-initialises every scratch word it reads (control block,
    // role counters, stats) on the stream before use, so a call does not see
    // the previous call's contents.
    return run_peel(2, nullptr, cols, row_ptr, num_vertices, num_edges, 0, nullptr, nullptr, nullptr, 0, nullptr,
                    support, stats, scratch, kNoAllocScratchBytes, (cudaStream_t)stream);
}
