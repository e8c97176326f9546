/*
 * api.c -- the libsais 2.10.4 construction API on top of the GB300 engine.
 *
 * Each entry point repeats the reference's argument checks and n <= 1 special
 * cases on the host (src/libsais.c:7018-7322 and :8363-8517,
 * src/libsais64.c:7058-7230 and :8302-8338, src/libsais16.c:6995-7230 and
 * :8064-8100), then hands the text to the CUDA engine through gsais.h.  The
 * context-less calls use the engine's process-wide context; the _ctx calls
 * use the caller's context; `threads` only has its sign checked.
 */
#include <stddef.h>
#include <stdint.h>
#include <string.h>

#include "../../include/libsais.h"
#include "../../include/libsais16.h"
#include "../../include/libsais64.h"
#include "../../include/libsais16x64.h"
#include "gsais.h"

/* ------------------------------------------------------------ helpers */

static void freq_reset(void *freq, int symbytes, int freq_bytes)
{
    if (freq) memset(freq, 0, (size_t)(symbytes == 1 ? 256 : 65536) * (size_t)freq_bytes);
}

static unsigned sym_at(const void *T, int symbytes, int64_t i)
{
    return symbytes == 1 ? ((const uint8_t *)T)[i] : ((const uint16_t *)T)[i];
}

static void freq_bump(void *freq, int freq_bytes, unsigned c)
{
    if (!freq) return;
    if (freq_bytes == 8) ((int64_t *)freq)[c]++;
    else ((int32_t *)freq)[c]++;
}

static void put_index(void *A, int bytes, int64_t i, int64_t v)
{
    if (bytes == 8) ((int64_t *)A)[i] = v;
    else ((int32_t *)A)[i] = (int32_t)v;
}

static int64_t get_index(const void *A, int bytes, int64_t i)
{
    return bytes == 8 ? ((const int64_t *)A)[i] : (int64_t)((const int32_t *)A)[i];
}

/* SA / GSA: (src/libsais.c:7018 libsais, :7034 libsais_gsa) */
static int64_t do_sa(gsais_ctx *ctx, const void *T, int symbytes, void *SA, int idx_bytes, int64_t n, int64_t fs,
                     void *freq, int gsa)
{
    if (T == NULL || SA == NULL || n < 0 || fs < 0) return -1;
    if (gsa && n > 0 && sym_at(T, symbytes, n - 1) != 0) return -1;
    if (n <= 1) {
        freq_reset(freq, symbytes, idx_bytes);
        if (n == 1) {
            put_index(SA, idx_bytes, 0, 0);
            freq_bump(freq, idx_bytes, sym_at(T, symbytes, 0));
        }
        return 0;
    }
    return gsais_run_sa(ctx, T, symbytes, n, gsa, SA, idx_bytes, freq, idx_bytes);
}

/* BWT / BWT-aux: (src/libsais.c:7097 libsais_bwt, :7123 libsais_bwt_aux) */
static int64_t do_bwt(gsais_ctx *ctx, const void *T, int symbytes, void *U, void *A, int idx_bytes, int64_t n,
                      int64_t fs, void *freq, int64_t r, void *I, int aux)
{
    if (T == NULL || U == NULL || A == NULL || n < 0 || fs < 0) return -1;
    if (aux && (r < 2 || (r & (r - 1)) != 0 || I == NULL)) return -1;
    if (n <= 1) {
        freq_reset(freq, symbytes, idx_bytes);
        if (n == 1) {
            if (symbytes == 1) ((uint8_t *)U)[0] = ((const uint8_t *)T)[0];
            else ((uint16_t *)U)[0] = ((const uint16_t *)T)[0];
            freq_bump(freq, idx_bytes, sym_at(T, symbytes, 0));
        }
        if (aux) {
            put_index(I, idx_bytes, 0, n);
            return 0;
        }
        return n;
    }
    return gsais_run_bwt(ctx, T, symbytes, n, U, freq, idx_bytes, aux ? r : 0, aux ? I : NULL, idx_bytes, NULL, 4);
}

/* PLCP: (src/libsais.c:8363 libsais_plcp, :8381 libsais_plcp_gsa) */
static int64_t do_plcp(const void *T, int symbytes, const void *SA, void *PLCP, int idx_bytes, int64_t n, int gsa)
{
    if (T == NULL || SA == NULL || PLCP == NULL || n < 0) return -1;
    if (gsa && n > 0 && sym_at(T, symbytes, n - 1) != 0) return -1;
    if (n <= 1) {
        if (n == 1) put_index(PLCP, idx_bytes, 0, 0);
        return 0;
    }
    return gsais_run_plcp(gsais_default_ctx(), T, symbytes, SA, PLCP, idx_bytes, n, gsa);
}

/* LCP: (src/libsais.c:8417 libsais_lcp) */
static int64_t do_lcp(const void *PLCP, const void *SA, void *LCP, int idx_bytes, int64_t n)
{
    if (PLCP == NULL || SA == NULL || LCP == NULL || n < 0) return -1;
    if (n <= 1) {
        if (n == 1) put_index(LCP, idx_bytes, 0, get_index(PLCP, idx_bytes, get_index(SA, idx_bytes, 0)));
        return 0;
    }
    return gsais_run_lcp(gsais_default_ctx(), PLCP, SA, LCP, idx_bytes, n);
}

/* SA of an integer string: (src/libsais.c:7050 libsais_int, src/libsais64.c:7118 libsais64_long) */
static int64_t do_sa_int(const void *T, int tbytes, void *SA, int idx_bytes, int64_t n, int64_t k, int64_t fs)
{
    if (T == NULL || SA == NULL || n < 0 || fs < 0) return -1;
    if (n <= 1) {
        if (n == 1) put_index(SA, idx_bytes, 0, 0);
        return 0;
    }
    return gsais_run_sa_int(gsais_default_ctx(), T, tbytes, n, k, SA, idx_bytes);
}

/* Inverse BWT: (src/libsais.c:8040 libsais_unbwt_aux; libsais_unbwt is r = n, I = &i, :8030) */
static int64_t do_unbwt(gsais_ctx *ctx, const void *T, int symbytes, void *U, const void *A, int64_t n, int64_t r,
                        const void *I, int idx_bytes)
{
    if (T == NULL || U == NULL || A == NULL || n < 0 || ((r != n) && ((r < 2) || ((r & (r - 1)) != 0))) ||
        I == NULL)
        return -1;
    if (n <= 1) {
        if (get_index(I, idx_bytes, 0) != n) return -1;
        if (n == 1) {
            if (symbytes == 1) ((uint8_t *)U)[0] = ((const uint8_t *)T)[0];
            else ((uint16_t *)U)[0] = ((const uint16_t *)T)[0];
        }
        return 0;
    }
    for (int64_t t = 0; t <= (n - 1) / r; ++t) {
        const int64_t v = get_index(I, idx_bytes, t);
        if (v <= 0 || v > n) return -1;
    }
    if (ctx == NULL) return -2;
    return gsais_run_unbwt(ctx, T, symbytes, n, get_index(I, idx_bytes, 0), U);
}

#define DEF_CTX gsais_default_ctx()
#define USE_CTX(c) ((gsais_ctx *)(uintptr_t)(c))

/* ----------------------------------------------------- libsais.h (8-bit) */

void *libsais_create_ctx(void) { return gsais_ctx_create(); }

void *libsais_create_ctx_omp(int32_t threads) { return threads < 0 ? NULL : gsais_ctx_create(); }

void libsais_free_ctx(void *ctx) { gsais_ctx_destroy((gsais_ctx *)ctx); }

int32_t libsais(const uint8_t *T, int32_t *SA, int32_t n, int32_t fs, int32_t *freq)
{
    return (int32_t)do_sa(DEF_CTX, T, 1, SA, 4, n, fs, freq, 0);
}

int32_t libsais_gsa(const uint8_t *T, int32_t *SA, int32_t n, int32_t fs, int32_t *freq)
{
    return (int32_t)do_sa(DEF_CTX, T, 1, SA, 4, n, fs, freq, 1);
}

int32_t libsais_ctx(const void *ctx, const uint8_t *T, int32_t *SA, int32_t n, int32_t fs, int32_t *freq)
{
    if (ctx == NULL) return -1;
    return (int32_t)do_sa(USE_CTX(ctx), T, 1, SA, 4, n, fs, freq, 0);
}

int32_t libsais_gsa_ctx(const void *ctx, const uint8_t *T, int32_t *SA, int32_t n, int32_t fs, int32_t *freq)
{
    if (ctx == NULL) return -1;
    return (int32_t)do_sa(USE_CTX(ctx), T, 1, SA, 4, n, fs, freq, 1);
}

int32_t libsais_omp(const uint8_t *T, int32_t *SA, int32_t n, int32_t fs, int32_t *freq, int32_t threads)
{
    if (threads < 0) return -1;
    return (int32_t)do_sa(DEF_CTX, T, 1, SA, 4, n, fs, freq, 0);
}

int32_t libsais_gsa_omp(const uint8_t *T, int32_t *SA, int32_t n, int32_t fs, int32_t *freq, int32_t threads)
{
    if (threads < 0) return -1;
    return (int32_t)do_sa(DEF_CTX, T, 1, SA, 4, n, fs, freq, 1);
}

int32_t libsais_bwt(const uint8_t *T, uint8_t *U, int32_t *A, int32_t n, int32_t fs, int32_t *freq)
{
    return (int32_t)do_bwt(DEF_CTX, T, 1, U, A, 4, n, fs, freq, 0, NULL, 0);
}

int32_t libsais_bwt_aux(const uint8_t *T, uint8_t *U, int32_t *A, int32_t n, int32_t fs, int32_t *freq, int32_t r,
                        int32_t *I)
{
    return (int32_t)do_bwt(DEF_CTX, T, 1, U, A, 4, n, fs, freq, r, I, 1);
}

int32_t libsais_bwt_ctx(const void *ctx, const uint8_t *T, uint8_t *U, int32_t *A, int32_t n, int32_t fs,
                        int32_t *freq)
{
    if (ctx == NULL) return -1;
    return (int32_t)do_bwt(USE_CTX(ctx), T, 1, U, A, 4, n, fs, freq, 0, NULL, 0);
}

int32_t libsais_bwt_aux_ctx(const void *ctx, const uint8_t *T, uint8_t *U, int32_t *A, int32_t n, int32_t fs,
                            int32_t *freq, int32_t r, int32_t *I)
{
    if (ctx == NULL) return -1;
    return (int32_t)do_bwt(USE_CTX(ctx), T, 1, U, A, 4, n, fs, freq, r, I, 1);
}

int32_t libsais_bwt_omp(const uint8_t *T, uint8_t *U, int32_t *A, int32_t n, int32_t fs, int32_t *freq,
                        int32_t threads)
{
    if (threads < 0) return -1;
    return (int32_t)do_bwt(DEF_CTX, T, 1, U, A, 4, n, fs, freq, 0, NULL, 0);
}

int32_t libsais_bwt_aux_omp(const uint8_t *T, uint8_t *U, int32_t *A, int32_t n, int32_t fs, int32_t *freq, int32_t r,
                            int32_t *I, int32_t threads)
{
    if (threads < 0) return -1;
    return (int32_t)do_bwt(DEF_CTX, T, 1, U, A, 4, n, fs, freq, r, I, 1);
}

int32_t libsais_plcp(const uint8_t *T, const int32_t *SA, int32_t *PLCP, int32_t n)
{
    return (int32_t)do_plcp(T, 1, SA, PLCP, 4, n, 0);
}

int32_t libsais_plcp_gsa(const uint8_t *T, const int32_t *SA, int32_t *PLCP, int32_t n)
{
    return (int32_t)do_plcp(T, 1, SA, PLCP, 4, n, 1);
}

int32_t libsais_lcp(const int32_t *PLCP, const int32_t *SA, int32_t *LCP, int32_t n)
{
    return (int32_t)do_lcp(PLCP, SA, LCP, 4, n);
}

int32_t libsais_plcp_omp(const uint8_t *T, const int32_t *SA, int32_t *PLCP, int32_t n, int32_t threads)
{
    if (threads < 0) return -1;
    return (int32_t)do_plcp(T, 1, SA, PLCP, 4, n, 0);
}

int32_t libsais_plcp_gsa_omp(const uint8_t *T, const int32_t *SA, int32_t *PLCP, int32_t n, int32_t threads)
{
    if (threads < 0) return -1;
    return (int32_t)do_plcp(T, 1, SA, PLCP, 4, n, 1);
}

int32_t libsais_lcp_omp(const int32_t *PLCP, const int32_t *SA, int32_t *LCP, int32_t n, int32_t threads)
{
    if (threads < 0) return -1;
    return (int32_t)do_lcp(PLCP, SA, LCP, 4, n);
}

/* ---------------------------------------------------- libsais64.h (8-bit) */

int64_t libsais64(const uint8_t *T, int64_t *SA, int64_t n, int64_t fs, int64_t *freq)
{
    return do_sa(DEF_CTX, T, 1, SA, 8, n, fs, freq, 0);
}

int64_t libsais64_gsa(const uint8_t *T, int64_t *SA, int64_t n, int64_t fs, int64_t *freq)
{
    return do_sa(DEF_CTX, T, 1, SA, 8, n, fs, freq, 1);
}

int64_t libsais64_omp(const uint8_t *T, int64_t *SA, int64_t n, int64_t fs, int64_t *freq, int64_t threads)
{
    if (threads < 0) return -1;
    return do_sa(DEF_CTX, T, 1, SA, 8, n, fs, freq, 0);
}

int64_t libsais64_gsa_omp(const uint8_t *T, int64_t *SA, int64_t n, int64_t fs, int64_t *freq, int64_t threads)
{
    if (threads < 0) return -1;
    return do_sa(DEF_CTX, T, 1, SA, 8, n, fs, freq, 1);
}

int64_t libsais64_bwt(const uint8_t *T, uint8_t *U, int64_t *A, int64_t n, int64_t fs, int64_t *freq)
{
    return do_bwt(DEF_CTX, T, 1, U, A, 8, n, fs, freq, 0, NULL, 0);
}

int64_t libsais64_bwt_aux(const uint8_t *T, uint8_t *U, int64_t *A, int64_t n, int64_t fs, int64_t *freq, int64_t r,
                          int64_t *I)
{
    return do_bwt(DEF_CTX, T, 1, U, A, 8, n, fs, freq, r, I, 1);
}

int64_t libsais64_bwt_omp(const uint8_t *T, uint8_t *U, int64_t *A, int64_t n, int64_t fs, int64_t *freq,
                          int64_t threads)
{
    if (threads < 0) return -1;
    return do_bwt(DEF_CTX, T, 1, U, A, 8, n, fs, freq, 0, NULL, 0);
}

int64_t libsais64_bwt_aux_omp(const uint8_t *T, uint8_t *U, int64_t *A, int64_t n, int64_t fs, int64_t *freq,
                              int64_t r, int64_t *I, int64_t threads)
{
    if (threads < 0) return -1;
    return do_bwt(DEF_CTX, T, 1, U, A, 8, n, fs, freq, r, I, 1);
}

int64_t libsais64_plcp(const uint8_t *T, const int64_t *SA, int64_t *PLCP, int64_t n)
{
    return do_plcp(T, 1, SA, PLCP, 8, n, 0);
}

int64_t libsais64_plcp_gsa(const uint8_t *T, const int64_t *SA, int64_t *PLCP, int64_t n)
{
    return do_plcp(T, 1, SA, PLCP, 8, n, 1);
}

int64_t libsais64_lcp(const int64_t *PLCP, const int64_t *SA, int64_t *LCP, int64_t n)
{
    return do_lcp(PLCP, SA, LCP, 8, n);
}

int64_t libsais64_plcp_omp(const uint8_t *T, const int64_t *SA, int64_t *PLCP, int64_t n, int64_t threads)
{
    if (threads < 0) return -1;
    return do_plcp(T, 1, SA, PLCP, 8, n, 0);
}

int64_t libsais64_plcp_gsa_omp(const uint8_t *T, const int64_t *SA, int64_t *PLCP, int64_t n, int64_t threads)
{
    if (threads < 0) return -1;
    return do_plcp(T, 1, SA, PLCP, 8, n, 1);
}

int64_t libsais64_lcp_omp(const int64_t *PLCP, const int64_t *SA, int64_t *LCP, int64_t n, int64_t threads)
{
    if (threads < 0) return -1;
    return do_lcp(PLCP, SA, LCP, 8, n);
}

/* ---------------------------------------------------- libsais16.h (16-bit) */

void *libsais16_create_ctx(void) { return gsais_ctx_create(); }

void *libsais16_create_ctx_omp(int32_t threads) { return threads < 0 ? NULL : gsais_ctx_create(); }

void libsais16_free_ctx(void *ctx) { gsais_ctx_destroy((gsais_ctx *)ctx); }

int32_t libsais16(const uint16_t *T, int32_t *SA, int32_t n, int32_t fs, int32_t *freq)
{
    return (int32_t)do_sa(DEF_CTX, T, 2, SA, 4, n, fs, freq, 0);
}

int32_t libsais16_gsa(const uint16_t *T, int32_t *SA, int32_t n, int32_t fs, int32_t *freq)
{
    return (int32_t)do_sa(DEF_CTX, T, 2, SA, 4, n, fs, freq, 1);
}

int32_t libsais16_ctx(const void *ctx, const uint16_t *T, int32_t *SA, int32_t n, int32_t fs, int32_t *freq)
{
    if (ctx == NULL) return -1;
    return (int32_t)do_sa(USE_CTX(ctx), T, 2, SA, 4, n, fs, freq, 0);
}

int32_t libsais16_gsa_ctx(const void *ctx, const uint16_t *T, int32_t *SA, int32_t n, int32_t fs, int32_t *freq)
{
    if (ctx == NULL) return -1;
    return (int32_t)do_sa(USE_CTX(ctx), T, 2, SA, 4, n, fs, freq, 1);
}

int32_t libsais16_omp(const uint16_t *T, int32_t *SA, int32_t n, int32_t fs, int32_t *freq, int32_t threads)
{
    if (threads < 0) return -1;
    return (int32_t)do_sa(DEF_CTX, T, 2, SA, 4, n, fs, freq, 0);
}

int32_t libsais16_gsa_omp(const uint16_t *T, int32_t *SA, int32_t n, int32_t fs, int32_t *freq, int32_t threads)
{
    if (threads < 0) return -1;
    return (int32_t)do_sa(DEF_CTX, T, 2, SA, 4, n, fs, freq, 1);
}

int32_t libsais16_bwt(const uint16_t *T, uint16_t *U, int32_t *A, int32_t n, int32_t fs, int32_t *freq)
{
    return (int32_t)do_bwt(DEF_CTX, T, 2, U, A, 4, n, fs, freq, 0, NULL, 0);
}

int32_t libsais16_bwt_aux(const uint16_t *T, uint16_t *U, int32_t *A, int32_t n, int32_t fs, int32_t *freq, int32_t r,
                          int32_t *I)
{
    return (int32_t)do_bwt(DEF_CTX, T, 2, U, A, 4, n, fs, freq, r, I, 1);
}

int32_t libsais16_bwt_ctx(const void *ctx, const uint16_t *T, uint16_t *U, int32_t *A, int32_t n, int32_t fs,
                          int32_t *freq)
{
    if (ctx == NULL) return -1;
    return (int32_t)do_bwt(USE_CTX(ctx), T, 2, U, A, 4, n, fs, freq, 0, NULL, 0);
}

int32_t libsais16_bwt_aux_ctx(const void *ctx, const uint16_t *T, uint16_t *U, int32_t *A, int32_t n, int32_t fs,
                              int32_t *freq, int32_t r, int32_t *I)
{
    if (ctx == NULL) return -1;
    return (int32_t)do_bwt(USE_CTX(ctx), T, 2, U, A, 4, n, fs, freq, r, I, 1);
}

int32_t libsais16_bwt_omp(const uint16_t *T, uint16_t *U, int32_t *A, int32_t n, int32_t fs, int32_t *freq,
                          int32_t threads)
{
    if (threads < 0) return -1;
    return (int32_t)do_bwt(DEF_CTX, T, 2, U, A, 4, n, fs, freq, 0, NULL, 0);
}

int32_t libsais16_bwt_aux_omp(const uint16_t *T, uint16_t *U, int32_t *A, int32_t n, int32_t fs, int32_t *freq,
                              int32_t r, int32_t *I, int32_t threads)
{
    if (threads < 0) return -1;
    return (int32_t)do_bwt(DEF_CTX, T, 2, U, A, 4, n, fs, freq, r, I, 1);
}

int32_t libsais16_plcp(const uint16_t *T, const int32_t *SA, int32_t *PLCP, int32_t n)
{
    return (int32_t)do_plcp(T, 2, SA, PLCP, 4, n, 0);
}

int32_t libsais16_plcp_gsa(const uint16_t *T, const int32_t *SA, int32_t *PLCP, int32_t n)
{
    return (int32_t)do_plcp(T, 2, SA, PLCP, 4, n, 1);
}

int32_t libsais16_lcp(const int32_t *PLCP, const int32_t *SA, int32_t *LCP, int32_t n)
{
    return (int32_t)do_lcp(PLCP, SA, LCP, 4, n);
}

int32_t libsais16_plcp_omp(const uint16_t *T, const int32_t *SA, int32_t *PLCP, int32_t n, int32_t threads)
{
    if (threads < 0) return -1;
    return (int32_t)do_plcp(T, 2, SA, PLCP, 4, n, 0);
}

int32_t libsais16_plcp_gsa_omp(const uint16_t *T, const int32_t *SA, int32_t *PLCP, int32_t n, int32_t threads)
{
    if (threads < 0) return -1;
    return (int32_t)do_plcp(T, 2, SA, PLCP, 4, n, 1);
}

int32_t libsais16_lcp_omp(const int32_t *PLCP, const int32_t *SA, int32_t *LCP, int32_t n, int32_t threads)
{
    if (threads < 0) return -1;
    return (int32_t)do_lcp(PLCP, SA, LCP, 4, n);
}

/* ------------------------------------ integer alphabets (libsais.h, libsais16.h, libsais64.h) */

int32_t libsais_int(int32_t *T, int32_t *SA, int32_t n, int32_t k, int32_t fs)
{
    return (int32_t)do_sa_int(T, 4, SA, 4, n, k, fs);
}

int32_t libsais_int_omp(int32_t *T, int32_t *SA, int32_t n, int32_t k, int32_t fs, int32_t threads)
{
    if (threads < 0) return -1;
    return (int32_t)do_sa_int(T, 4, SA, 4, n, k, fs);
}

int32_t libsais16_int(int32_t *T, int32_t *SA, int32_t n, int32_t k, int32_t fs)
{
    return (int32_t)do_sa_int(T, 4, SA, 4, n, k, fs);
}

int32_t libsais16_int_omp(int32_t *T, int32_t *SA, int32_t n, int32_t k, int32_t fs, int32_t threads)
{
    if (threads < 0) return -1;
    return (int32_t)do_sa_int(T, 4, SA, 4, n, k, fs);
}

int64_t libsais64_long(int64_t *T, int64_t *SA, int64_t n, int64_t k, int64_t fs)
{
    return do_sa_int(T, 8, SA, 8, n, k, fs);
}

int64_t libsais64_long_omp(int64_t *T, int64_t *SA, int64_t n, int64_t k, int64_t fs, int64_t threads)
{
    if (threads < 0) return -1;
    return do_sa_int(T, 8, SA, 8, n, k, fs);
}

/* (src/libsais.c:8399 libsais_plcp_int) */
int32_t libsais_plcp_int(const int32_t *T, const int32_t *SA, int32_t *PLCP, int32_t n)
{
    if (T == NULL || SA == NULL || PLCP == NULL || n < 0) return -1;
    if (n <= 1) {
        if (n == 1) PLCP[0] = 0;
        return 0;
    }
    return (int32_t)gsais_run_plcp(gsais_default_ctx(), T, 4, SA, PLCP, 4, n, 0);
}

int32_t libsais_plcp_int_omp(const int32_t *T, const int32_t *SA, int32_t *PLCP, int32_t n, int32_t threads)
{
    if (threads < 0) return -1;
    return libsais_plcp_int(T, SA, PLCP, n);
}

/* ----------------------------------------------------- inverse BWT, 8-bit */

void *libsais_unbwt_create_ctx(void) { return gsais_ctx_create(); }

void *libsais_unbwt_create_ctx_omp(int32_t threads) { return threads < 0 ? NULL : gsais_ctx_create(); }

void libsais_unbwt_free_ctx(void *ctx) { gsais_ctx_destroy((gsais_ctx *)ctx); }

int32_t libsais_unbwt(const uint8_t *T, uint8_t *U, int32_t *A, int32_t n, const int32_t *freq, int32_t i)
{
    (void)freq;
    return (int32_t)do_unbwt(DEF_CTX, T, 1, U, A, n, n, &i, 4);
}

int32_t libsais_unbwt_ctx(const void *ctx, const uint8_t *T, uint8_t *U, int32_t *A, int32_t n, const int32_t *freq,
                          int32_t i)
{
    (void)freq;
    return (int32_t)do_unbwt(USE_CTX(ctx), T, 1, U, A, n, n, &i, 4);
}

int32_t libsais_unbwt_aux(const uint8_t *T, uint8_t *U, int32_t *A, int32_t n, const int32_t *freq, int32_t r,
                          const int32_t *I)
{
    (void)freq;
    return (int32_t)do_unbwt(DEF_CTX, T, 1, U, A, n, r, I, 4);
}

int32_t libsais_unbwt_aux_ctx(const void *ctx, const uint8_t *T, uint8_t *U, int32_t *A, int32_t n,
                              const int32_t *freq, int32_t r, const int32_t *I)
{
    (void)freq;
    return (int32_t)do_unbwt(USE_CTX(ctx), T, 1, U, A, n, r, I, 4);
}

int32_t libsais_unbwt_omp(const uint8_t *T, uint8_t *U, int32_t *A, int32_t n, const int32_t *freq, int32_t i,
                          int32_t threads)
{
    if (threads < 0) return -1;
    return libsais_unbwt(T, U, A, n, freq, i);
}

int32_t libsais_unbwt_aux_omp(const uint8_t *T, uint8_t *U, int32_t *A, int32_t n, const int32_t *freq, int32_t r,
                              const int32_t *I, int32_t threads)
{
    if (threads < 0) return -1;
    return libsais_unbwt_aux(T, U, A, n, freq, r, I);
}

/* ---------------------------------------------------- inverse BWT, 16-bit */

void *libsais16_unbwt_create_ctx(void) { return gsais_ctx_create(); }

void *libsais16_unbwt_create_ctx_omp(int32_t threads) { return threads < 0 ? NULL : gsais_ctx_create(); }

void libsais16_unbwt_free_ctx(void *ctx) { gsais_ctx_destroy((gsais_ctx *)ctx); }

int32_t libsais16_unbwt(const uint16_t *T, uint16_t *U, int32_t *A, int32_t n, const int32_t *freq, int32_t i)
{
    (void)freq;
    return (int32_t)do_unbwt(DEF_CTX, T, 2, U, A, n, n, &i, 4);
}

int32_t libsais16_unbwt_ctx(const void *ctx, const uint16_t *T, uint16_t *U, int32_t *A, int32_t n,
                            const int32_t *freq, int32_t i)
{
    (void)freq;
    return (int32_t)do_unbwt(USE_CTX(ctx), T, 2, U, A, n, n, &i, 4);
}

int32_t libsais16_unbwt_aux(const uint16_t *T, uint16_t *U, int32_t *A, int32_t n, const int32_t *freq, int32_t r,
                            const int32_t *I)
{
    (void)freq;
    return (int32_t)do_unbwt(DEF_CTX, T, 2, U, A, n, r, I, 4);
}

int32_t libsais16_unbwt_aux_ctx(const void *ctx, const uint16_t *T, uint16_t *U, int32_t *A, int32_t n,
                                const int32_t *freq, int32_t r, const int32_t *I)
{
    (void)freq;
    return (int32_t)do_unbwt(USE_CTX(ctx), T, 2, U, A, n, r, I, 4);
}

int32_t libsais16_unbwt_omp(const uint16_t *T, uint16_t *U, int32_t *A, int32_t n, const int32_t *freq, int32_t i,
                            int32_t threads)
{
    if (threads < 0) return -1;
    return libsais16_unbwt(T, U, A, n, freq, i);
}

int32_t libsais16_unbwt_aux_omp(const uint16_t *T, uint16_t *U, int32_t *A, int32_t n, const int32_t *freq,
                                int32_t r, const int32_t *I, int32_t threads)
{
    if (threads < 0) return -1;
    return libsais16_unbwt_aux(T, U, A, n, freq, r, I);
}

/* ---------------------------------------------- inverse BWT, 64-bit indexes */

int64_t libsais64_unbwt(const uint8_t *T, uint8_t *U, int64_t *A, int64_t n, const int64_t *freq, int64_t i)
{
    (void)freq;
    return do_unbwt(DEF_CTX, T, 1, U, A, n, n, &i, 8);
}

int64_t libsais64_unbwt_aux(const uint8_t *T, uint8_t *U, int64_t *A, int64_t n, const int64_t *freq, int64_t r,
                            const int64_t *I)
{
    (void)freq;
    return do_unbwt(DEF_CTX, T, 1, U, A, n, r, I, 8);
}

int64_t libsais64_unbwt_omp(const uint8_t *T, uint8_t *U, int64_t *A, int64_t n, const int64_t *freq, int64_t i,
                            int64_t threads)
{
    if (threads < 0) return -1;
    return libsais64_unbwt(T, U, A, n, freq, i);
}

int64_t libsais64_unbwt_aux_omp(const uint8_t *T, uint8_t *U, int64_t *A, int64_t n, const int64_t *freq, int64_t r,
                                const int64_t *I, int64_t threads)
{
    if (threads < 0) return -1;
    return libsais64_unbwt_aux(T, U, A, n, freq, r, I);
}

/* ---------------------------- libsais16x64.h: 16-bit symbols, 64-bit indexes
 * (src/libsais16x64.c:7036-7230 and :7789-8100 delegate to the 16-bit code
 * and widen the results; here the engine writes int64 directly) */

int64_t libsais16x64(const uint16_t *T, int64_t *SA, int64_t n, int64_t fs, int64_t *freq)
{
    return do_sa(DEF_CTX, T, 2, SA, 8, n, fs, freq, 0);
}

int64_t libsais16x64_gsa(const uint16_t *T, int64_t *SA, int64_t n, int64_t fs, int64_t *freq)
{
    return do_sa(DEF_CTX, T, 2, SA, 8, n, fs, freq, 1);
}

int64_t libsais16x64_long(int64_t *T, int64_t *SA, int64_t n, int64_t k, int64_t fs)
{
    return do_sa_int(T, 8, SA, 8, n, k, fs);
}

int64_t libsais16x64_omp(const uint16_t *T, int64_t *SA, int64_t n, int64_t fs, int64_t *freq, int64_t threads)
{
    if (threads < 0) return -1;
    return libsais16x64(T, SA, n, fs, freq);
}

int64_t libsais16x64_gsa_omp(const uint16_t *T, int64_t *SA, int64_t n, int64_t fs, int64_t *freq, int64_t threads)
{
    if (threads < 0) return -1;
    return libsais16x64_gsa(T, SA, n, fs, freq);
}

int64_t libsais16x64_long_omp(int64_t *T, int64_t *SA, int64_t n, int64_t k, int64_t fs, int64_t threads)
{
    if (threads < 0) return -1;
    return libsais16x64_long(T, SA, n, k, fs);
}

int64_t libsais16x64_bwt(const uint16_t *T, uint16_t *U, int64_t *A, int64_t n, int64_t fs, int64_t *freq)
{
    return do_bwt(DEF_CTX, T, 2, U, A, 8, n, fs, freq, 0, NULL, 0);
}

int64_t libsais16x64_bwt_aux(const uint16_t *T, uint16_t *U, int64_t *A, int64_t n, int64_t fs, int64_t *freq,
                             int64_t r, int64_t *I)
{
    return do_bwt(DEF_CTX, T, 2, U, A, 8, n, fs, freq, r, I, 1);
}

int64_t libsais16x64_bwt_omp(const uint16_t *T, uint16_t *U, int64_t *A, int64_t n, int64_t fs, int64_t *freq,
                             int64_t threads)
{
    if (threads < 0) return -1;
    return libsais16x64_bwt(T, U, A, n, fs, freq);
}

int64_t libsais16x64_bwt_aux_omp(const uint16_t *T, uint16_t *U, int64_t *A, int64_t n, int64_t fs, int64_t *freq,
                                 int64_t r, int64_t *I, int64_t threads)
{
    if (threads < 0) return -1;
    return libsais16x64_bwt_aux(T, U, A, n, fs, freq, r, I);
}

int64_t libsais16x64_unbwt(const uint16_t *T, uint16_t *U, int64_t *A, int64_t n, const int64_t *freq, int64_t i)
{
    (void)freq;
    return do_unbwt(DEF_CTX, T, 2, U, A, n, n, &i, 8);
}

int64_t libsais16x64_unbwt_aux(const uint16_t *T, uint16_t *U, int64_t *A, int64_t n, const int64_t *freq,
                               int64_t r, const int64_t *I)
{
    (void)freq;
    return do_unbwt(DEF_CTX, T, 2, U, A, n, r, I, 8);
}

int64_t libsais16x64_unbwt_omp(const uint16_t *T, uint16_t *U, int64_t *A, int64_t n, const int64_t *freq, int64_t i,
                               int64_t threads)
{
    if (threads < 0) return -1;
    return libsais16x64_unbwt(T, U, A, n, freq, i);
}

int64_t libsais16x64_unbwt_aux_omp(const uint16_t *T, uint16_t *U, int64_t *A, int64_t n, const int64_t *freq,
                                   int64_t r, const int64_t *I, int64_t threads)
{
    if (threads < 0) return -1;
    return libsais16x64_unbwt_aux(T, U, A, n, freq, r, I);
}

int64_t libsais16x64_plcp(const uint16_t *T, const int64_t *SA, int64_t *PLCP, int64_t n)
{
    return do_plcp(T, 2, SA, PLCP, 8, n, 0);
}

int64_t libsais16x64_plcp_gsa(const uint16_t *T, const int64_t *SA, int64_t *PLCP, int64_t n)
{
    return do_plcp(T, 2, SA, PLCP, 8, n, 1);
}

int64_t libsais16x64_lcp(const int64_t *PLCP, const int64_t *SA, int64_t *LCP, int64_t n)
{
    return do_lcp(PLCP, SA, LCP, 8, n);
}

int64_t libsais16x64_plcp_omp(const uint16_t *T, const int64_t *SA, int64_t *PLCP, int64_t n, int64_t threads)
{
    if (threads < 0) return -1;
    return libsais16x64_plcp(T, SA, PLCP, n);
}

int64_t libsais16x64_plcp_gsa_omp(const uint16_t *T, const int64_t *SA, int64_t *PLCP, int64_t n, int64_t threads)
{
    if (threads < 0) return -1;
    return libsais16x64_plcp_gsa(T, SA, PLCP, n);
}

int64_t libsais16x64_lcp_omp(const int64_t *PLCP, const int64_t *SA, int64_t *LCP, int64_t n, int64_t threads)
{
    if (threads < 0) return -1;
    return libsais16x64_lcp(PLCP, SA, LCP, n);
}
