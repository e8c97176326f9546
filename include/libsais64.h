/*--

libsais_gb300 -- drop-in replacement for the construction entry points of
libsais 2.10.4's 64-bit interface (include/libsais64.h of the reference),
computed on an NVIDIA GB300 GPU.  Same signatures and return codes; indices
are int64.  Texts must have fewer than 2^32 symbols (the GPU ranks with
32-bit indices and widens on output); longer texts return -2.
`threads` and `fs` are validated and otherwise ignored; `A` is not written.

libsais64_long takes an integer string with symbols in [0, k) (-1 otherwise)
whose symbols fit 32 bits (-2 otherwise).  The inverse BWT ignores `freq`
and does not write `A`.

--*/

#ifndef LIBSAIS64_H
#define LIBSAIS64_H 1

#define LIBSAIS64_VERSION_MAJOR   2
#define LIBSAIS64_VERSION_MINOR   10
#define LIBSAIS64_VERSION_PATCH   4
#define LIBSAIS64_VERSION_STRING  "2.10.4"

#ifndef LIBSAIS64_API
    #define LIBSAIS64_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

    #include <stdint.h>

    /* (ref include/libsais64.h:61) */
    LIBSAIS64_API int64_t libsais64(const uint8_t * T, int64_t * SA, int64_t n, int64_t fs, int64_t * freq);
    /* (ref include/libsais64.h:72) */
    LIBSAIS64_API int64_t libsais64_gsa(const uint8_t * T, int64_t * SA, int64_t n, int64_t fs, int64_t * freq);
    /* (ref include/libsais64.h:97) */
    LIBSAIS64_API int64_t libsais64_omp(const uint8_t * T, int64_t * SA, int64_t n, int64_t fs, int64_t * freq, int64_t threads);
    /* (ref include/libsais64.h:109) */
    LIBSAIS64_API int64_t libsais64_gsa_omp(const uint8_t * T, int64_t * SA, int64_t n, int64_t fs, int64_t * freq, int64_t threads);
    /* Suffix array of an integer string over [0, k).  (ref include/libsais64.h:84) */
    LIBSAIS64_API int64_t libsais64_long(int64_t * T, int64_t * SA, int64_t n, int64_t k, int64_t fs);
    /* (ref include/libsais64.h:122) */
    LIBSAIS64_API int64_t libsais64_long_omp(int64_t * T, int64_t * SA, int64_t n, int64_t k, int64_t fs, int64_t threads);
    /* (ref include/libsais64.h:135) */
    LIBSAIS64_API int64_t libsais64_bwt(const uint8_t * T, uint8_t * U, int64_t * A, int64_t n, int64_t fs, int64_t * freq);
    /* (ref include/libsais64.h:149) */
    LIBSAIS64_API int64_t libsais64_bwt_aux(const uint8_t * T, uint8_t * U, int64_t * A, int64_t n, int64_t fs, int64_t * freq, int64_t r, int64_t * I);
    /* (ref include/libsais64.h:163) */
    LIBSAIS64_API int64_t libsais64_bwt_omp(const uint8_t * T, uint8_t * U, int64_t * A, int64_t n, int64_t fs, int64_t * freq, int64_t threads);
    /* (ref include/libsais64.h:178) */
    LIBSAIS64_API int64_t libsais64_bwt_aux_omp(const uint8_t * T, uint8_t * U, int64_t * A, int64_t n, int64_t fs, int64_t * freq, int64_t r, int64_t * I, int64_t threads);
    /* (ref include/libsais64.h:191) */
    LIBSAIS64_API int64_t libsais64_unbwt(const uint8_t * T, uint8_t * U, int64_t * A, int64_t n, const int64_t * freq, int64_t i);
    /* (ref include/libsais64.h:204) */
    LIBSAIS64_API int64_t libsais64_unbwt_aux(const uint8_t * T, uint8_t * U, int64_t * A, int64_t n, const int64_t * freq, int64_t r, const int64_t * I);
    /* (ref include/libsais64.h:218) */
    LIBSAIS64_API int64_t libsais64_unbwt_omp(const uint8_t * T, uint8_t * U, int64_t * A, int64_t n, const int64_t * freq, int64_t i, int64_t threads);
    /* (ref include/libsais64.h:232) */
    LIBSAIS64_API int64_t libsais64_unbwt_aux_omp(const uint8_t * T, uint8_t * U, int64_t * A, int64_t n, const int64_t * freq, int64_t r, const int64_t * I, int64_t threads);
    /* (ref include/libsais64.h:243) */
    LIBSAIS64_API int64_t libsais64_plcp(const uint8_t * T, const int64_t * SA, int64_t * PLCP, int64_t n);
    /* (ref include/libsais64.h:253) */
    LIBSAIS64_API int64_t libsais64_plcp_gsa(const uint8_t * T, const int64_t * SA, int64_t * PLCP, int64_t n);
    /* (ref include/libsais64.h:263) */
    LIBSAIS64_API int64_t libsais64_lcp(const int64_t * PLCP, const int64_t * SA, int64_t * LCP, int64_t n);
    /* (ref include/libsais64.h:275) */
    LIBSAIS64_API int64_t libsais64_plcp_omp(const uint8_t * T, const int64_t * SA, int64_t * PLCP, int64_t n, int64_t threads);
    /* (ref include/libsais64.h:286) */
    LIBSAIS64_API int64_t libsais64_plcp_gsa_omp(const uint8_t * T, const int64_t * SA, int64_t * PLCP, int64_t n, int64_t threads);
    /* (ref include/libsais64.h:297) */
    LIBSAIS64_API int64_t libsais64_lcp_omp(const int64_t * PLCP, const int64_t * SA, int64_t * LCP, int64_t n, int64_t threads);

#ifdef __cplusplus
}
#endif

#endif
