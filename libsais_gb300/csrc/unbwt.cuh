// unbwt.cuh -- inverse BWT (internal).
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "engine.h"

namespace gsais {

inline size_t align_up_to(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Rows that are multiples of this are the splitters of the parallel walk.
uint64_t unbwt_gap(uint64_t n);

// Device scratch bytes of unbwt_run for n symbols.
size_t unbwt_workspace_bytes(uint64_t n);

// Text of n symbols (symbytes 1 or 2) from its BWT d_U in libsais_bwt layout
// and the primary index p (1 <= p <= n) into d_out (may not alias d_U).
// h_hist: pinned host words for the radix histograms.
cudaError_t unbwt_run(const void *d_U, int symbytes, uint64_t n, uint64_t p, void *d_out, void *scratch,
                      uint32_t *h_hist, KernelProfiler *prof, uint32_t *d_err, cudaStream_t st);

}  // namespace gsais
