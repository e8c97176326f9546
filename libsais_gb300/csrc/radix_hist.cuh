// radix_hist.cuh -- digit histograms of radix-sort keys, accumulated by the
// kernels that produce the keys (so the sort needs no separate upsweep read).
#pragma once
#include <cstdint>

#include "device_util.cuh"

namespace gsais {

constexpr int kMaxRadixPasses = 8;

__device__ __forceinline__ uint32_t radix_digit(uint64_t key, int p, int end_bit)
{
    const int bits = end_bit - 8 * p < 8 ? end_bit - 8 * p : 8;
    return (uint32_t)(key >> (8 * p)) & ((1u << bits) - 1u);
}

// Adds the digits of `key` (for passes [0, passes)) to the CTA table sh.
// Whole warps must call it together; lanes with ok == false add nothing.
// A warp whose 32 digits agree adds 32 with a single shared atomic.
__device__ __forceinline__ void radix_hist_add(uint32_t (*sh)[256], uint64_t key, bool ok, int passes, int end_bit)
{
    const bool full = __all_sync(GSAIS_FULL_MASK, ok);
    const int lane = threadIdx.x & 31;
    for (int p = 0; p < passes; ++p) {
        const uint32_t d = radix_digit(key, p, end_bit);
        if (full && __reduce_min_sync(GSAIS_FULL_MASK, d) == __reduce_max_sync(GSAIS_FULL_MASK, d)) {
            if (lane == 0) atomicAdd(&sh[p][d], 32u);
        } else if (ok) {
            atomicAdd(&sh[p][d], 1u);
        }
    }
}

__device__ __forceinline__ void radix_hist_zero(uint32_t (*sh)[256], int passes)
{
    for (int i = threadIdx.x; i < passes * 256; i += blockDim.x) (&sh[0][0])[i] = 0;
}

// Adds the CTA table to the global histograms (call after a __syncthreads).
__device__ __forceinline__ void radix_hist_flush(uint32_t (*sh)[256], int passes, uint32_t *hist)
{
    for (int i = threadIdx.x; i < passes * 256; i += blockDim.x) {
        const uint32_t v = (&sh[0][0])[i];
        if (v) atomicAdd(&hist[i], v);
    }
}

}  // namespace gsais
