/*--

libsais_gb300 -- drop-in replacement for the construction entry points of
libsais 2.10.4's 16-bit interface (include/libsais16.h of the reference),
computed on an NVIDIA GB300 GPU.  Same signatures and return codes; symbols
are uint16_t and freq has 65536 entries.  `threads` and `fs` are validated
and otherwise ignored; `A` is not written.

libsais16_int takes an integer string with symbols in [0, k) (-1 otherwise).
The inverse BWT ignores `freq` and does not write `A`.

--*/

#ifndef LIBSAIS16_H
#define LIBSAIS16_H 1

#define LIBSAIS16_VERSION_MAJOR   2
#define LIBSAIS16_VERSION_MINOR   10
#define LIBSAIS16_VERSION_PATCH   4
#define LIBSAIS16_VERSION_STRING  "2.10.4"

#ifndef LIBSAIS16_API
    #define LIBSAIS16_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

    #include <stdint.h>

    /* (ref include/libsais16.h:57) */
    LIBSAIS16_API void * libsais16_create_ctx(void);
    /* (ref include/libsais16.h:66) */
    LIBSAIS16_API void * libsais16_create_ctx_omp(int32_t threads);
    /* (ref include/libsais16.h:73) */
    LIBSAIS16_API void libsais16_free_ctx(void * ctx);

    /* (ref include/libsais16.h:84) */
    LIBSAIS16_API int32_t libsais16(const uint16_t * T, int32_t * SA, int32_t n, int32_t fs, int32_t * freq);
    /* (ref include/libsais16.h:95) */
    LIBSAIS16_API int32_t libsais16_gsa(const uint16_t * T, int32_t * SA, int32_t n, int32_t fs, int32_t * freq);
    /* (ref include/libsais16.h:119) */
    LIBSAIS16_API int32_t libsais16_ctx(const void * ctx, const uint16_t * T, int32_t * SA, int32_t n, int32_t fs, int32_t * freq);
    /* (ref include/libsais16.h:131) */
    LIBSAIS16_API int32_t libsais16_gsa_ctx(const void * ctx, const uint16_t * T, int32_t * SA, int32_t n, int32_t fs, int32_t * freq);
    /* (ref include/libsais16.h:144) */
    LIBSAIS16_API int32_t libsais16_omp(const uint16_t * T, int32_t * SA, int32_t n, int32_t fs, int32_t * freq, int32_t threads);
    /* (ref include/libsais16.h:156) */
    LIBSAIS16_API int32_t libsais16_gsa_omp(const uint16_t * T, int32_t * SA, int32_t n, int32_t fs, int32_t * freq, int32_t threads);
    /* (ref include/libsais16.h:107) */
    LIBSAIS16_API int32_t libsais16_int(int32_t * T, int32_t * SA, int32_t n, int32_t k, int32_t fs);
    /* (ref include/libsais16.h:169) */
    LIBSAIS16_API int32_t libsais16_int_omp(int32_t * T, int32_t * SA, int32_t n, int32_t k, int32_t fs, int32_t threads);

    /* (ref include/libsais16.h:182) */
    LIBSAIS16_API int32_t libsais16_bwt(const uint16_t * T, uint16_t * U, int32_t * A, int32_t n, int32_t fs, int32_t * freq);
    /* (ref include/libsais16.h:196) */
    LIBSAIS16_API int32_t libsais16_bwt_aux(const uint16_t * T, uint16_t * U, int32_t * A, int32_t n, int32_t fs, int32_t * freq, int32_t r, int32_t * I);
    /* (ref include/libsais16.h:209) */
    LIBSAIS16_API int32_t libsais16_bwt_ctx(const void * ctx, const uint16_t * T, uint16_t * U, int32_t * A, int32_t n, int32_t fs, int32_t * freq);
    /* (ref include/libsais16.h:224) */
    LIBSAIS16_API int32_t libsais16_bwt_aux_ctx(const void * ctx, const uint16_t * T, uint16_t * U, int32_t * A, int32_t n, int32_t fs, int32_t * freq, int32_t r, int32_t * I);
    /* (ref include/libsais16.h:238) */
    LIBSAIS16_API int32_t libsais16_bwt_omp(const uint16_t * T, uint16_t * U, int32_t * A, int32_t n, int32_t fs, int32_t * freq, int32_t threads);
    /* (ref include/libsais16.h:253) */
    LIBSAIS16_API int32_t libsais16_bwt_aux_omp(const uint16_t * T, uint16_t * U, int32_t * A, int32_t n, int32_t fs, int32_t * freq, int32_t r, int32_t * I, int32_t threads);

    /* (ref include/libsais16.h:261) */
    LIBSAIS16_API void * libsais16_unbwt_create_ctx(void);
    /* (ref include/libsais16.h:270) */
    LIBSAIS16_API void * libsais16_unbwt_create_ctx_omp(int32_t threads);
    /* (ref include/libsais16.h:277) */
    LIBSAIS16_API void libsais16_unbwt_free_ctx(void * ctx);
    /* (ref include/libsais16.h:289) */
    LIBSAIS16_API int32_t libsais16_unbwt(const uint16_t * T, uint16_t * U, int32_t * A, int32_t n, const int32_t * freq, int32_t i);
    /* (ref include/libsais16.h:302) */
    LIBSAIS16_API int32_t libsais16_unbwt_ctx(const void * ctx, const uint16_t * T, uint16_t * U, int32_t * A, int32_t n, const int32_t * freq, int32_t i);
    /* (ref include/libsais16.h:315) */
    LIBSAIS16_API int32_t libsais16_unbwt_aux(const uint16_t * T, uint16_t * U, int32_t * A, int32_t n, const int32_t * freq, int32_t r, const int32_t * I);
    /* (ref include/libsais16.h:329) */
    LIBSAIS16_API int32_t libsais16_unbwt_aux_ctx(const void * ctx, const uint16_t * T, uint16_t * U, int32_t * A, int32_t n, const int32_t * freq, int32_t r, const int32_t * I);
    /* (ref include/libsais16.h:343) */
    LIBSAIS16_API int32_t libsais16_unbwt_omp(const uint16_t * T, uint16_t * U, int32_t * A, int32_t n, const int32_t * freq, int32_t i, int32_t threads);
    /* (ref include/libsais16.h:357) */
    LIBSAIS16_API int32_t libsais16_unbwt_aux_omp(const uint16_t * T, uint16_t * U, int32_t * A, int32_t n, const int32_t * freq, int32_t r, const int32_t * I, int32_t threads);

    /* (ref include/libsais16.h:368) */
    LIBSAIS16_API int32_t libsais16_plcp(const uint16_t * T, const int32_t * SA, int32_t * PLCP, int32_t n);
    /* (ref include/libsais16.h:378) */
    LIBSAIS16_API int32_t libsais16_plcp_gsa(const uint16_t * T, const int32_t * SA, int32_t * PLCP, int32_t n);
    /* (ref include/libsais16.h:388) */
    LIBSAIS16_API int32_t libsais16_lcp(const int32_t * PLCP, const int32_t * SA, int32_t * LCP, int32_t n);
    /* (ref include/libsais16.h:400) */
    LIBSAIS16_API int32_t libsais16_plcp_omp(const uint16_t * T, const int32_t * SA, int32_t * PLCP, int32_t n, int32_t threads);
    /* (ref include/libsais16.h:411) */
    LIBSAIS16_API int32_t libsais16_plcp_gsa_omp(const uint16_t * T, const int32_t * SA, int32_t * PLCP, int32_t n, int32_t threads);
    /* (ref include/libsais16.h:422) */
    LIBSAIS16_API int32_t libsais16_lcp_omp(const int32_t * PLCP, const int32_t * SA, int32_t * LCP, int32_t n, int32_t threads);

#ifdef __cplusplus
}
#endif

#endif
