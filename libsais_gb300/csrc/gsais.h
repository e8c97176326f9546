/*
 * gsais.h -- C-ABI between the libsais-compatible C shim (api.c) and the CUDA
 * engine (engine.cu).  Plain pointers and sizes only.
 *
 * Return convention of the gsais_run_* calls: >= 0 on success (the BWT calls
 * return the primary index), -1 for invalid input detected on the device
 * (a malformed generalized-suffix-array text), -2 for any CUDA or allocation
 * failure -- the same codes libsais uses (src/libsais.c:6930-6932).
 */
#ifndef GSAIS_H
#define GSAIS_H 1

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gsais_ctx gsais_ctx;

gsais_ctx *gsais_ctx_create(void);
void gsais_ctx_destroy(gsais_ctx *ctx);

/* Process-wide context used by the context-less libsais calls; guarded by a
 * mutex inside the gsais_run_* calls when `shared` is set. */
gsais_ctx *gsais_default_ctx(void);

/* SA (sa_bytes 4 or 8) and symbol frequencies (freq_bytes 4 or 8, may be
 * NULL) of a host text of n symbols (symbytes 1 or 2). */
int64_t gsais_run_sa(gsais_ctx *ctx, const void *T, int symbytes, int64_t n, int gsa, void *SA, int sa_bytes,
                     void *freq, int freq_bytes);

/* SA of an integer string (tbytes 4: int32, 8: int64 symbols) over [0, k)
 * (libsais_int, libsais64_long).  -1 if a symbol lies outside [0, k); -2 if a
 * symbol is wider than 32 bits. */
int64_t gsais_run_sa_int(gsais_ctx *ctx, const void *T, int tbytes, int64_t n, int64_t k, void *SA, int sa_bytes);

/* BWT into U (libsais_bwt layout).  r > 0 also writes I[t] = ISA[t*r] + 1
 * (idx_bytes wide) and returns 0 instead of the primary index.  SA (may be
 * NULL) additionally receives the suffix array. */
int64_t gsais_run_bwt(gsais_ctx *ctx, const void *T, int symbytes, int64_t n, void *U, void *freq, int freq_bytes,
                      int64_t r, void *I, int idx_bytes, void *SA, int sa_bytes);

/* Text from its BWT T (libsais_bwt layout, symbytes 1 or 2) and primary
 * index (1..n) into U (libsais_unbwt).  -1 for a primary index outside 1..n,
 * -2 for device failures or a T that is not the BWT of any text with that
 * primary index. */
int64_t gsais_run_unbwt(gsais_ctx *ctx, const void *T, int symbytes, int64_t n, int64_t primary, void *U);

/* PLCP of (T, SA) into PLCP (idx_bytes wide). */
int64_t gsais_run_plcp(gsais_ctx *ctx, const void *T, int symbytes, const void *SA, void *PLCP, int idx_bytes,
                       int64_t n, int gsa);

/* LCP[i] = PLCP[SA[i]] (idx_bytes wide). */
int64_t gsais_run_lcp(gsais_ctx *ctx, const void *PLCP, const void *SA, void *LCP, int idx_bytes, int64_t n);

/* SA + BWT of `count` small jobs sorted together (one batched sort), each job
 * k with its own host buffers: text T[k] of n[k] symbols (symbytes 1 or 2),
 * SA[k] (int32) and U[k].  result[k] receives the primary index.  Returns 0,
 * -1 for invalid arguments, -2 on device failure.  At most 32000 jobs. */
int64_t gsais_batch_jobs(gsais_ctx *ctx, int32_t symbytes, int32_t count, const void *const *T, const int64_t *n,
                         int32_t *const *SA, void *const *U, int64_t *result);

/* Device workspace currently held by ctx (bytes). */
int64_t gsais_ctx_workspace_bytes(gsais_ctx *ctx);

#ifdef __cplusplus
}
#endif

#endif
