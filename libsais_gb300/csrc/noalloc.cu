// noalloc.cu -- suffix array of a device-resident text without allocating
// any memory.
//
// Some callers cannot call cudaMalloc.  A plugin that runs inside a host
// application whose caching allocator owns all of the device's memory (a
// deep-learning framework, a database engine) must not allocate behind that
// allocator's back: cudaMalloc can fail for want of free memory the
// allocator is holding, and it can synchronise the whole device, stalling
// the host's other streams.  Latency-critical callers avoid it for the same
// reason.  For them this file provides gsais_sa_device_noalloc, which runs
// the same prefix-doubling suffix sort as gsais_sa_device but takes all of
// its device scratch from one file-scope __device__ array of fixed size, so
// the call itself allocates nothing (no cudaMalloc/cudaFree, no pinned host
// memory, no library routine that allocates).
//
// Limits and sharing rules:
//   * texts of at most kNoAllocMaxN = 65,536 symbols; longer texts get -1;
//   * the scratch array (kNoAllocScratchBytes = 6 MiB) is reserved on every
//     GPU that loads this library, for as long as the library stays loaded;
//   * every call uses the same array and the array keeps the previous call's
//     contents; the sort clears everything that must start at zero;
//   * calls whose work overlaps on one GPU race on the array.  Each CUDA
//     context has its own copy of it, so separate processes never share it;
//     within one process a host mutex admits one call at a time and every
//     call returns only after the work it queued on `stream` has finished
//     (an error return first drains `stream`), so calls made one after
//     another, from any thread, do not overlap;
//   * the first call on each device looks up the array's device address with
//     cudaGetSymbolAddress (with that device current) and keeps it.
#include <cstring>
#include <mutex>

#include "device_util.cuh"
#include "engine.h"
#include "libsais_gb300.h"
#include "suffix_sort.cuh"

using namespace gsais;

namespace {

constexpr uint64_t kNoAllocMaxN = 65536;
constexpr size_t kNoAllocScratchBytes = (size_t)6 << 20;
constexpr int kMaxDevices = 64;

// The only device memory the entry point uses.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Host-side read-back buffers (ordinary static storage, no allocation).
alignas(16) static uint32_t g_host_small[kHostSmallWords];
alignas(16) static uint32_t g_host_hist[8 * 256];
static uint32_t g_host_flag[4];

std::mutex g_noalloc_mu;
void *g_scratch_addr[kMaxDevices] = {nullptr};

// Device address of the scratch array for the current device, looked up once.
void *scratch_for(int dev)
{
    if (dev < 0 || dev >= kMaxDevices) return nullptr;
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        g_scratch_addr[dev] = p;
    }
    return g_scratch_addr[dev];
}

// Error return: no kernel of this call may still use the shared array once
// the mutex is released, so the stream is drained first (its own error, if
// any, is cleared; the call fails either way).
int64_t fail_drained(cudaStream_t st)
{
    cudaGetLastError();
    cudaStreamSynchronize(st);
    cudaGetLastError();
    return -2;
}

}  // namespace

extern "C" int64_t gsais_sa_device_noalloc(const void *T, int32_t symbytes, int64_t n, int32_t gsa, void *SA,
                                           void *stream)
{
    if (!T || !SA || n < 0 || (symbytes != 1 && symbytes != 2)) return -1;
    if ((uint64_t)n > kNoAllocMaxN) return -1;   // beyond the fixed scratch size
    if (n == 0) return 0;
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return -2;
    }
    char *base = static_cast<char *>(scratch_for(dev));
    if (!base) return -2;
    const size_t need = sort_workspace_bytes((uint64_t)n, symbytes);
    if (need + 256 > kNoAllocScratchBytes) return -1;
    cudaStream_t st = static_cast<cudaStream_t>(stream);

    // error word and validity flag at the front, the sort workspace after them
    uint32_t *d_err = reinterpret_cast<uint32_t *>(base);
    SortWorkspace ws;
    sort_workspace_carve(ws, base + 256, (uint64_t)n, symbytes, g_host_small, g_host_hist);
    ws.sa = static_cast<uint32_t *>(SA);
    if (cudaMemsetAsync(d_err, 0, 8, st) != cudaSuccess) return fail_drained(st);
    if (gsa) {
        bool valid = true;
        if (gsa_validate(T, symbytes, (uint64_t)n, d_err + 1, g_host_flag, st, &valid) != cudaSuccess)
            return fail_drained(st);
        if (!valid) return -1;
    }
    SortOptions opt;
    if (suffix_sort(T, symbytes, (uint64_t)n, gsa != 0, ws, opt, d_err, st, nullptr) != cudaSuccess)
        return fail_drained(st);
    return 0;
}
