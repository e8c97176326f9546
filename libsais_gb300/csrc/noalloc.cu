// noalloc.cu -- suffix array of a device-resident text without allocating
// any memory.
//
// Some callers cannot call cudaMalloc: code that runs while a CUDA graph is
// being captured, code inside a framework whose caching allocator owns all
// device memory, and real-time paths where an allocation may block.  For
// them this file provides gsais_sa_device_noalloc, which runs the same
// prefix-doubling suffix sort as gsais_sa_device but takes all of its
// scratch from one file-scope __device__ array of fixed size, so the call
// itself allocates nothing (no cudaMalloc/cudaFree, no pinned host memory).
//
// Limits and sharing rules:
//   * texts of at most kNoAllocMaxN = 65,536 symbols; longer texts get -1;
//   * the scratch array (kNoAllocScratchBytes = 6 MiB) is reserved on every
//     GPU that loads this library, for as long as the library stays loaded;
//   * every call uses the same array and the array keeps the previous call's
//     contents; the sort clears everything that must start at zero;
//   * calls are serialised on the host by a mutex, but calls that overlap on
//     the GPU (for example from two processes sharing the module, or a
//     caller that replays captured work concurrently) race on the array;
//   * the first call on each device looks up the array's device address with
//     cudaGetSymbolAddress; make that first call before any stream capture.
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
    if (cudaMemsetAsync(d_err, 0, 8, st) != cudaSuccess) {
        cudaGetLastError();
        return -2;
    }
    if (gsa) {
        bool valid = true;
        if (gsa_validate(T, symbytes, (uint64_t)n, d_err + 1, g_host_flag, st, &valid) != cudaSuccess) {
            cudaGetLastError();
            return -2;
        }
        if (!valid) return -1;
    }
    SortOptions opt;
    if (suffix_sort(T, symbytes, (uint64_t)n, gsa != 0, ws, opt, d_err, st, nullptr) != cudaSuccess) {
        cudaGetLastError();
        return -2;
    }
    return 0;
}
