/*--

libsais_gb300 -- drop-in replacement for libsais 2.10.4's 16-bit / 64-bit
interface (include/libsais16x64.h of the reference), computed on an NVIDIA
GB300 GPU.  Symbols are uint16_t (freq has 65536 entries), indices int64.
Texts must have fewer than 2^32 symbols (-2 otherwise).  `threads` and `fs`
are validated and otherwise ignored; `A` is not written; the inverse BWT
ignores `freq`.  libsais16x64_long takes an integer string with symbols in
[0, k) (-1 otherwise) that fit 32 bits (-2 otherwise).

--*/

#ifndef LIBSAIS16X64_H
#define LIBSAIS16X64_H 1

#define LIBSAIS16X64_VERSION_MAJOR   2
#define LIBSAIS16X64_VERSION_MINOR   10
#define LIBSAIS16X64_VERSION_PATCH   4
#define LIBSAIS16X64_VERSION_STRING  "2.10.4"

#ifndef LIBSAIS16X64_API
    #define LIBSAIS16X64_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

    #include <stdint.h>

    /* (ref include/libsais16x64.h:61) */
    LIBSAIS16X64_API int64_t libsais16x64(const uint16_t * T, int64_t * SA, int64_t n, int64_t fs, int64_t * freq);
    /* (ref include/libsais16x64.h:72) */
    LIBSAIS16X64_API int64_t libsais16x64_gsa(const uint16_t * T, int64_t * SA, int64_t n, int64_t fs, int64_t * freq);
    /* (ref include/libsais16x64.h:84) */
    LIBSAIS16X64_API int64_t libsais16x64_long(int64_t * T, int64_t * SA, int64_t n, int64_t k, int64_t fs);
    /* (ref include/libsais16x64.h:97) */
    LIBSAIS16X64_API int64_t libsais16x64_omp(const uint16_t * T, int64_t * SA, int64_t n, int64_t fs, int64_t * freq, int64_t threads);
    /* (ref include/libsais16x64.h:109) */
    LIBSAIS16X64_API int64_t libsais16x64_gsa_omp(const uint16_t * T, int64_t * SA, int64_t n, int64_t fs, int64_t * freq, int64_t threads);
    /* (ref include/libsais16x64.h:122) */
    LIBSAIS16X64_API int64_t libsais16x64_long_omp(int64_t * T, int64_t * SA, int64_t n, int64_t k, int64_t fs, int64_t threads);

    /* (ref include/libsais16x64.h:135) */
    LIBSAIS16X64_API int64_t libsais16x64_bwt(const uint16_t * T, uint16_t * U, int64_t * A, int64_t n, int64_t fs, int64_t * freq);
    /* (ref include/libsais16x64.h:149) */
    LIBSAIS16X64_API int64_t libsais16x64_bwt_aux(const uint16_t * T, uint16_t * U, int64_t * A, int64_t n, int64_t fs, int64_t * freq, int64_t r, int64_t * I);
    /* (ref include/libsais16x64.h:163) */
    LIBSAIS16X64_API int64_t libsais16x64_bwt_omp(const uint16_t * T, uint16_t * U, int64_t * A, int64_t n, int64_t fs, int64_t * freq, int64_t threads);
    /* (ref include/libsais16x64.h:178) */
    LIBSAIS16X64_API int64_t libsais16x64_bwt_aux_omp(const uint16_t * T, uint16_t * U, int64_t * A, int64_t n, int64_t fs, int64_t * freq, int64_t r, int64_t * I, int64_t threads);

    /* (ref include/libsais16x64.h:191) */
    LIBSAIS16X64_API int64_t libsais16x64_unbwt(const uint16_t * T, uint16_t * U, int64_t * A, int64_t n, const int64_t * freq, int64_t i);
    /* (ref include/libsais16x64.h:204) */
    LIBSAIS16X64_API int64_t libsais16x64_unbwt_aux(const uint16_t * T, uint16_t * U, int64_t * A, int64_t n, const int64_t * freq, int64_t r, const int64_t * I);
    /* (ref include/libsais16x64.h:218) */
    LIBSAIS16X64_API int64_t libsais16x64_unbwt_omp(const uint16_t * T, uint16_t * U, int64_t * A, int64_t n, const int64_t * freq, int64_t i, int64_t threads);
    /* (ref include/libsais16x64.h:232) */
    LIBSAIS16X64_API int64_t libsais16x64_unbwt_aux_omp(const uint16_t * T, uint16_t * U, int64_t * A, int64_t n, const int64_t * freq, int64_t r, const int64_t * I, int64_t threads);

    /* (ref include/libsais16x64.h:243) */
    LIBSAIS16X64_API int64_t libsais16x64_plcp(const uint16_t * T, const int64_t * SA, int64_t * PLCP, int64_t n);
    /* (ref include/libsais16x64.h:253) */
    LIBSAIS16X64_API int64_t libsais16x64_plcp_gsa(const uint16_t * T, const int64_t * SA, int64_t * PLCP, int64_t n);
    /* (ref include/libsais16x64.h:263) */
    LIBSAIS16X64_API int64_t libsais16x64_lcp(const int64_t * PLCP, const int64_t * SA, int64_t * LCP, int64_t n);
    /* (ref include/libsais16x64.h:275) */
    LIBSAIS16X64_API int64_t libsais16x64_plcp_omp(const uint16_t * T, const int64_t * SA, int64_t * PLCP, int64_t n, int64_t threads);
    /* (ref include/libsais16x64.h:286) */
    LIBSAIS16X64_API int64_t libsais16x64_plcp_gsa_omp(const uint16_t * T, const int64_t * SA, int64_t * PLCP, int64_t n, int64_t threads);
    /* (ref include/libsais16x64.h:297) */
    LIBSAIS16X64_API int64_t libsais16x64_lcp_omp(const int64_t * PLCP, const int64_t * SA, int64_t * LCP, int64_t n, int64_t threads);

#ifdef __cplusplus
}
#endif

#endif
