// engine.h -- internal C++ interface between the CUDA translation units.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include <atomic>
#include <vector>

#include "tuning.h"

namespace gsais {

// Number of kernels this library has launched (all contexts).
extern std::atomic<uint64_t> g_launches;
#define GSAIS_COUNTED(launch) do { launch; ::gsais::g_launches.fetch_add(1, std::memory_order_relaxed); } while (0)

// Optional per-kernel timing: CUDA events recorded on the launching stream
// around each launch of the instrumented kernels, resolved after the stream
// synchronises.  `bytes` is the algorithmic traffic of the launch.
enum KernelKind {
    KK_RADIX_PASS = 0, KK_TILE_COUNTS, KK_UPSWEEP, KK_SEED, KK_ROUND_KEYS, KK_SUMMARY, KK_ASSIGN, KK_SMALL, KK_PAIRS,
    KK_UNBWT, KK_HIST, KK_PERM, KK_CLASSIFY, KK_MEDIUM, KK_BWT, KK_FEW, KK_COUNT
};

struct KernelProfiler {
    bool enabled = false;
    struct Rec { int kind; cudaEvent_t a, b; uint64_t bytes; };
    std::vector<Rec> pending;
    std::vector<cudaEvent_t> pool;
    double ms[KK_COUNT] = {0};
    uint64_t launches[KK_COUNT] = {0};
    uint64_t bytes[KK_COUNT] = {0};

    cudaEvent_t get();
    // returns the start event to pair with end(); nullptr when disabled
    cudaEvent_t begin(cudaStream_t st);
    void end(int kind, cudaEvent_t a, cudaStream_t st, uint64_t bytes);
    // algorithmic bytes known only after the launch (device-side counts)
    void add_bytes(int kind, uint64_t b)
    {
        if (enabled) bytes[kind] += b;
    }
    void flush();   // call after the stream has synchronised
    void reset();
    ~KernelProfiler();
};

// Small device-to-host read on stream st (a multiple of 4 bytes).  Into
// pinned memory it is a one-block kernel storing over the host link, so it
// does not queue behind a large copy that occupies the copy engine (an early
// SA copy); into other host memory it is a cudaMemcpyAsync.
cudaError_t read_back(void *h_dst, const void *d_src, size_t bytes, cudaStream_t st);

// ---------------------------------------------------------------- radix sort
// LSD radix sort of (key, value) pairs: 8-bit digits, one upsweep histogram
// pass for all digits, then per digit a tile-count pass, a scan of the counts
// over tiles and one scatter pass.  Digits on which every key agrees are
// skipped.
struct RadixScratch {
    uint32_t *hist = nullptr;      // [8][256] digit histograms
    uint32_t *bases = nullptr;     // [8][256] exclusive bucket starts
    uint64_t *status = nullptr;    // per (tile, digit): 32-bit count + 32-bit offset
    uint32_t *counters = nullptr;  // [8] spare counters
    size_t status_words = 0;
    uint32_t *h_hist = nullptr;    // pinned host copy of hist
    KernelProfiler *prof = nullptr;
    int items32 = 24;              // keys per thread of a digit pass, 32-bit keys (16, 20, 24, 28)
    int items64 = 16;              // the same for 64-bit keys (12, 16, 20)
};

size_t radix_status_words(uint64_t n);
// Whether a digit-pass instance with `items` keys per thread is compiled for
// keys of key_bytes (4 or 8) bytes.
bool radix_items_supported(int key_bytes, int items);

// Sorts keys[0]/vals[0] by key bits [0, end_bit).  keys[1]/vals[1] are the
// alternate buffers.  On success returns 0 and sets *which to the buffer
// index holding the result; returns a CUDA error code otherwise.
// hist_ready: rs.hist already holds the digit histograms of keys[0] (the
// producer accumulated them), so the upsweep read is skipped.
cudaError_t radix_sort_pairs(uint64_t *keys[2], uint32_t *vals[2], uint64_t n, int end_bit,
                             RadixScratch &rs, uint32_t *d_err, cudaStream_t st, int *which,
                             int *passes_run, bool hist_ready = false);
// implicit_vals: vals[0] is not read; value i is n - 1 - i (seed keys written
// in reverse text order carry their suffix index implicitly).
cudaError_t radix_sort_pairs32(uint32_t *keys[2], uint32_t *vals[2], uint64_t n, int end_bit,
                               RadixScratch &rs, uint32_t *d_err, cudaStream_t st, int *which,
                               int *passes_run, bool hist_ready = false, bool implicit_vals = false);
// Stable partition of (uint32 key, value) pairs by key bits [begin_bit, end_bit).
cudaError_t radix_partition32(uint32_t *keys[2], uint32_t *vals[2], uint64_t n, int begin_bit, int end_bit,
                              RadixScratch &rs, uint32_t *d_err, cudaStream_t st, int *which);

// Test hook: limit (ns) of an extra bounded wait that every full radix tile
// makes on a barrier nothing arrives on (0 = off); set on the current device.
cudaError_t set_test_stall_wait(uint64_t limit_ns);

// --------------------------------------------------------------- statistics
struct SortStats {
    int rounds = 0;                // doubling rounds after the seed sort
    int seed_symbols = 0;          // symbols packed per seed key
    int seed_bits = 0;             // bits per symbol code
    uint64_t active_total = 0;     // sum of active suffixes over rounds
    uint64_t large_total = 0;      // sum over rounds of suffixes in groups sorted by the radix path
    uint64_t pairs_direct = 0;     // tied pairs ordered by direct comparison
    uint64_t early_patch = 0;      // SA slots written to the host after an early SA copy
    int radix_passes = 0;          // non-trivial digit passes over all sorts
    Tuning tuning;                 // the tuning the sort ran with
    int few_rounds = 0;            // rounds whose large groups took the few-others path
};

}  // namespace gsais
