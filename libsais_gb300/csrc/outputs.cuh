// outputs.cuh -- kernels that derive BWT / auxiliary indexes / PLCP / LCP
// from a finished suffix array (internal).  `err` is the context's device
// error word: out-of-range indexes raise GSAIS_ERR_BOUNDS there.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace gsais {

// U[0] = T[n-1]; U[k] = T[SA[row]-1] with the primary row skipped
// (libsais src/libsais.c:7111-7118).  isa1 = rank array (ISA + 1).
// err == nullptr: rows whose SA entry is out of range are skipped silently
// (an early BWT, whose unresolved rows are rewritten later).
// With pack_bits 2 or 4 the symbols are read from the packed code text
// (positions p at bits [(p % per)*pack_bits, ...) of word p / per) and mapped
// back through decode[], which keeps the gather inside L2 for DNA-like texts.
struct PackedText {
    const uint8_t *packed = nullptr;
    int pack_bits = 0;
    uint16_t decode[16] = {0};
};
cudaError_t bwt_gather(const void *d_T, int symbytes, const uint32_t *d_SA, const uint32_t *d_isa1, uint64_t n,
                       void *d_U, const PackedText &pk, uint32_t *err, cudaStream_t st);

// U[k] for the BWT rows whose SA slots are marked in row_bits ((n + 31) / 32
// words), with the final primary row isa1[0] - 1: repairs a BWT taken while
// those slots were unresolved.  U may be the device's address of pinned
// host memory.
cudaError_t bwt_patch(const void *d_T, int symbytes, const uint32_t *d_SA, const uint32_t *d_isa1, uint64_t n,
                      const uint32_t *row_bits, void *U, const PackedText &pk, uint32_t *err, cudaStream_t st);

// I[t] = ISA[t*r] + 1 for t = 0..(n-1)/r, as int32 (idx_bytes 4) or int64 (8).
cudaError_t aux_sample(const uint32_t *d_isa1, uint64_t n, uint64_t r, void *d_I, int idx_bytes, cudaStream_t st);

// int64 <-> uint32 index conversion (narrowing checks 0 <= v < n).
cudaError_t widen_u32_to_i64(const uint32_t *src, int64_t *dst, uint64_t n, cudaStream_t st);
cudaError_t narrow_i64_to_u32(const int64_t *src, uint32_t *dst, uint64_t n, uint32_t *err, cudaStream_t st);

// PLCP of (T, SA) into d_PLCP (uint32), using d_sparse (plcp_sparse_words(n)
// words) as scratch.  gsa stops at separators (src/libsais.c:8215-8238).
// h_hist (65536 host words, may be null): read-back buffer for the symbol
// histogram; with it, 8- and 16-bit texts of at most 16 symbols are packed
// into 2- or 4-bit codes first and the comparisons read the packed text.
size_t plcp_sparse_words(uint64_t n);
cudaError_t plcp_build(const void *d_T, int symbytes, const uint32_t *d_SA, uint64_t n, bool gsa, uint32_t *d_PLCP,
                       uint32_t *d_sparse, uint32_t *h_hist, uint32_t *err, cudaStream_t st);

// d_map (eight words) = the 256-bit map of the byte values that occur in T.
cudaError_t byte_presence(const uint8_t *d_T, uint64_t n, uint32_t *d_map, cudaStream_t st);

// Integer alphabets (int32 or int64 symbols, tbytes 4 or 8): d_out[0] = the
// largest value, d_out[1] = 1 if some value lies outside [0, k).
cudaError_t int_alphabet_scan(const void *d_T, int tbytes, uint64_t n, int64_t k, unsigned long long *d_out,
                              cudaStream_t st);
// Integer symbols copied to obytes-wide unsigned symbols (values already checked to fit).
cudaError_t int_narrow(const void *d_T, int tbytes, uint64_t n, void *d_out, int obytes, cudaStream_t st);

// LCP[i] = PLCP[SA[i]].  scratch: lcp_scratch_words(n) words (0 for texts
// whose PLCP array stays in L2; a null scratch takes the direct gather).
size_t lcp_scratch_words(uint64_t n);
cudaError_t lcp_gather(const uint32_t *d_PLCP, const uint32_t *d_SA, uint32_t *d_LCP, uint64_t n, uint32_t *scratch,
                       uint32_t *err, cudaStream_t st);

}  // namespace gsais
