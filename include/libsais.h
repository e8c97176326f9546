/*--

libsais_gb300 -- drop-in replacement for the construction entry points of
libsais 2.10.4 (include/libsais.h of the reference), computed on an NVIDIA
GB300 GPU.  Signatures, argument meaning and return codes are the
reference's; each declaration cites the reference line it replaces.

Return codes: 0 (or the BWT primary index) on success, -1 for invalid
arguments, -2 for allocation or device failures.  Texts must have fewer than
2^32 symbols.  The `threads` argument of the _omp variants is validated
(negative -> -1) and otherwise ignored: the GPU sets its own parallelism.
`fs` is validated and otherwise ignored: the GPU never needs extra SA space.
The temporary array `A` of the BWT calls is not written.

Integer alphabets (libsais_int): symbols must lie in [0, k) (-1 otherwise);
T is not modified.  The inverse BWT ignores `freq` and does not write `A`;
the libsais_unbwt_*_ctx functions take any context from libsais_create_ctx
or libsais_unbwt_create_ctx.

--*/

#ifndef LIBSAIS_H
#define LIBSAIS_H 1

#define LIBSAIS_VERSION_MAJOR   2
#define LIBSAIS_VERSION_MINOR   10
#define LIBSAIS_VERSION_PATCH   4
#define LIBSAIS_VERSION_STRING  "2.10.4"

#ifndef LIBSAIS_API
    #define LIBSAIS_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

    #include <stdint.h>

    /* Context owning a CUDA stream and a device workspace that grows to the
       largest call made with it; one thread at a time.  (ref include/libsais.h:57) */
    LIBSAIS_API void * libsais_create_ctx(void);
    /* (ref include/libsais.h:66) threads >= 0 accepted; NULL if threads < 0. */
    LIBSAIS_API void * libsais_create_ctx_omp(int32_t threads);
    /* (ref include/libsais.h:73) ctx may be NULL. */
    LIBSAIS_API void libsais_free_ctx(void * ctx);

    /* Suffix array of T[0..n-1]; freq[0..255] optional.  (ref include/libsais.h:84) */
    LIBSAIS_API int32_t libsais(const uint8_t * T, int32_t * SA, int32_t n, int32_t fs, int32_t * freq);
    /* Generalized suffix array; 0 separates strings, T[n-1] must be 0.  (ref include/libsais.h:95) */
    LIBSAIS_API int32_t libsais_gsa(const uint8_t * T, int32_t * SA, int32_t n, int32_t fs, int32_t * freq);
    /* (ref include/libsais.h:119) */
    LIBSAIS_API int32_t libsais_ctx(const void * ctx, const uint8_t * T, int32_t * SA, int32_t n, int32_t fs, int32_t * freq);
    /* Suffix array of an integer string over [0, k).  (ref include/libsais.h:107) */
    LIBSAIS_API int32_t libsais_int(int32_t * T, int32_t * SA, int32_t n, int32_t k, int32_t fs);
    /* (ref include/libsais.h:131) */
    LIBSAIS_API int32_t libsais_gsa_ctx(const void * ctx, const uint8_t * T, int32_t * SA, int32_t n, int32_t fs, int32_t * freq);
    /* (ref include/libsais.h:144) */
    LIBSAIS_API int32_t libsais_omp(const uint8_t * T, int32_t * SA, int32_t n, int32_t fs, int32_t * freq, int32_t threads);
    /* (ref include/libsais.h:156) */
    LIBSAIS_API int32_t libsais_gsa_omp(const uint8_t * T, int32_t * SA, int32_t n, int32_t fs, int32_t * freq, int32_t threads);
    /* (ref include/libsais.h:169) */
    LIBSAIS_API int32_t libsais_int_omp(int32_t * T, int32_t * SA, int32_t n, int32_t k, int32_t fs, int32_t threads);

    /* BWT of T into U (U may be T); returns the primary index.  (ref include/libsais.h:182) */
    LIBSAIS_API int32_t libsais_bwt(const uint8_t * T, uint8_t * U, int32_t * A, int32_t n, int32_t fs, int32_t * freq);
    /* BWT plus I[t] = ISA[t*r] + 1, r a power of two >= 2; returns 0.  (ref include/libsais.h:196) */
    LIBSAIS_API int32_t libsais_bwt_aux(const uint8_t * T, uint8_t * U, int32_t * A, int32_t n, int32_t fs, int32_t * freq, int32_t r, int32_t * I);
    /* (ref include/libsais.h:209) */
    LIBSAIS_API int32_t libsais_bwt_ctx(const void * ctx, const uint8_t * T, uint8_t * U, int32_t * A, int32_t n, int32_t fs, int32_t * freq);
    /* (ref include/libsais.h:224) */
    LIBSAIS_API int32_t libsais_bwt_aux_ctx(const void * ctx, const uint8_t * T, uint8_t * U, int32_t * A, int32_t n, int32_t fs, int32_t * freq, int32_t r, int32_t * I);
    /* (ref include/libsais.h:238) */
    LIBSAIS_API int32_t libsais_bwt_omp(const uint8_t * T, uint8_t * U, int32_t * A, int32_t n, int32_t fs, int32_t * freq, int32_t threads);
    /* (ref include/libsais.h:253) */
    LIBSAIS_API int32_t libsais_bwt_aux_omp(const uint8_t * T, uint8_t * U, int32_t * A, int32_t n, int32_t fs, int32_t * freq, int32_t r, int32_t * I, int32_t threads);

    /* Inverse BWT context (a regular context).  (ref include/libsais.h:261) */
    LIBSAIS_API void * libsais_unbwt_create_ctx(void);
    /* (ref include/libsais.h:270) */
    LIBSAIS_API void * libsais_unbwt_create_ctx_omp(int32_t threads);
    /* (ref include/libsais.h:277) */
    LIBSAIS_API void libsais_unbwt_free_ctx(void * ctx);
    /* Original string from its BWT T and primary index i; U may be T.  (ref include/libsais.h:289) */
    LIBSAIS_API int32_t libsais_unbwt(const uint8_t * T, uint8_t * U, int32_t * A, int32_t n, const int32_t * freq, int32_t i);
    /* (ref include/libsais.h:302) */
    LIBSAIS_API int32_t libsais_unbwt_ctx(const void * ctx, const uint8_t * T, uint8_t * U, int32_t * A, int32_t n, const int32_t * freq, int32_t i);
    /* With the auxiliary indexes of libsais_bwt_aux (I[0] is the primary index).  (ref include/libsais.h:315) */
    LIBSAIS_API int32_t libsais_unbwt_aux(const uint8_t * T, uint8_t * U, int32_t * A, int32_t n, const int32_t * freq, int32_t r, const int32_t * I);
    /* (ref include/libsais.h:329) */
    LIBSAIS_API int32_t libsais_unbwt_aux_ctx(const void * ctx, const uint8_t * T, uint8_t * U, int32_t * A, int32_t n, const int32_t * freq, int32_t r, const int32_t * I);
    /* (ref include/libsais.h:343) */
    LIBSAIS_API int32_t libsais_unbwt_omp(const uint8_t * T, uint8_t * U, int32_t * A, int32_t n, const int32_t * freq, int32_t i, int32_t threads);
    /* (ref include/libsais.h:357) */
    LIBSAIS_API int32_t libsais_unbwt_aux_omp(const uint8_t * T, uint8_t * U, int32_t * A, int32_t n, const int32_t * freq, int32_t r, const int32_t * I, int32_t threads);

    /* Permuted LCP from T and SA.  (ref include/libsais.h:368) */
    LIBSAIS_API int32_t libsais_plcp(const uint8_t * T, const int32_t * SA, int32_t * PLCP, int32_t n);
    /* Permuted LCP of a generalized SA; never extends across a 0.  (ref include/libsais.h:378) */
    LIBSAIS_API int32_t libsais_plcp_gsa(const uint8_t * T, const int32_t * SA, int32_t * PLCP, int32_t n);
    /* Permuted LCP of an integer string.  (ref include/libsais.h:388) */
    LIBSAIS_API int32_t libsais_plcp_int(const int32_t * T, const int32_t * SA, int32_t * PLCP, int32_t n);
    /* LCP[i] = PLCP[SA[i]]; LCP may be SA.  (ref include/libsais.h:398) */
    LIBSAIS_API int32_t libsais_lcp(const int32_t * PLCP, const int32_t * SA, int32_t * LCP, int32_t n);
    /* (ref include/libsais.h:410) */
    LIBSAIS_API int32_t libsais_plcp_omp(const uint8_t * T, const int32_t * SA, int32_t * PLCP, int32_t n, int32_t threads);
    /* (ref include/libsais.h:421) */
    LIBSAIS_API int32_t libsais_plcp_gsa_omp(const uint8_t * T, const int32_t * SA, int32_t * PLCP, int32_t n, int32_t threads);
    /* (ref include/libsais.h:432) */
    LIBSAIS_API int32_t libsais_plcp_int_omp(const int32_t * T, const int32_t * SA, int32_t * PLCP, int32_t n, int32_t threads);
    /* (ref include/libsais.h:443) */
    LIBSAIS_API int32_t libsais_lcp_omp(const int32_t * PLCP, const int32_t * SA, int32_t * LCP, int32_t n, int32_t threads);

#ifdef __cplusplus
}
#endif

#endif
