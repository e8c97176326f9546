/*
 * oracle.c -- CPU restatement of libsais's construction outputs.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the libsais_gb300 product links, loads
 * or calls this file; only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg use it, as the checker.
 *
 * What it restates (reference = libsais 2.10.4):
 *   - suffix array order: lexicographic, a proper prefix sorts first
 *     (libsais src/libsais.c:7018 `libsais`, :6879 `libsais_main_8u`).  The
 *     algorithm is the same family as the reference (SA-IS induced sorting,
 *     Nong/Zhang/Chan 2009), written here from the published description
 *     with an implicit end sentinel and one recursion over LMS names.
 *   - generalized suffix array (src/libsais.c:7034 `libsais_gsa`): every 0 is
 *     a separator; two suffixes that reach a separator at the same offset are
 *     ordered by position.  Restated by mapping the j-th separator to the
 *     unique symbol j (all below the real symbols) and sorting that string.
 *     Validity rule of src/libsais.c:6886-6889: T[0] != 0, no "00" pair.
 *   - BWT with primary index (src/libsais.c:7097-7121, bwt copy :6960):
 *     U[0] = T[n-1]; rows with SA[i] != 0 emit T[SA[i]-1] in order into
 *     U[1..n-1]; return value = 1 + row of suffix 0.
 *   - auxiliary BWT indexes (src/libsais.c:7123 `libsais_bwt_aux`):
 *     I[t] = 1 + ISA[t*r].
 *   - PLCP via the Phi array (src/libsais.c:8116 `compute_phi`, :8167
 *     `compute_plcp`, GSA variant :8215 `compute_plcp_gsa`) and LCP by
 *     gather (src/libsais.c:8311 `compute_lcp`).
 *   - symbol frequencies (src/libsais.c:1398-1427: freq[c] = count of c).
 *   - PLCP of an integer string (src/libsais.c:8399 `libsais_plcp_int`,
 *     :8263 `compute_plcp_int`): symbytes 4.
 *   - inverse BWT (src/libsais.c:8030 `libsais_unbwt`): the text from U and
 *     the primary index by the LF mapping, restated from the textbook
 *     definition (not the reference's bigram decoder).
 *
 * Indices are int64 throughout so one code path serves the 32- and 64-bit
 * APIs; callers narrow.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef int64_t idx_t;

/* ---------------------------------------------------------------- SA-IS */

static void bucket_bounds(const int32_t *T, idx_t n, idx_t k, idx_t *bkt, int end)
{
    memset(bkt, 0, (size_t)k * sizeof(idx_t));
    for (idx_t i = 0; i < n; i++) bkt[T[i]]++;
    idx_t sum = 0;
    for (idx_t c = 0; c < k; c++) {
        sum += bkt[c];
        bkt[c] = end ? sum : sum - bkt[c];
    }
}

#define IS_LMS(ty, i) ((i) > 0 && (ty)[(i)] && !(ty)[(i) - 1])

/* L-type then S-type induction pass.  ty[i] = 1 for S-type. */
static void induce(const int32_t *T, idx_t *SA, idx_t n, idx_t k, const uint8_t *ty, idx_t *bkt)
{
    bucket_bounds(T, n, k, bkt, 0);
    /* the last suffix is L-type and directly follows the virtual sentinel */
    SA[bkt[T[n - 1]]++] = n - 1;
    for (idx_t i = 0; i < n; i++) {
        idx_t p = SA[i];
        if (p > 0 && !ty[p - 1]) SA[bkt[T[p - 1]]++] = p - 1;
    }
    bucket_bounds(T, n, k, bkt, 1);
    for (idx_t i = n - 1; i >= 0; i--) {
        idx_t p = SA[i];
        if (p > 0 && ty[p - 1]) SA[--bkt[T[p - 1]]] = p - 1;
    }
}

static int lms_equal(const int32_t *T, const uint8_t *ty, idx_t n, idx_t a, idx_t b)
{
    if (a < 0 || b < 0) return 0;
    for (idx_t d = 0;; d++) {
        if (a + d == n || b + d == n) return 0;
        if (T[a + d] != T[b + d] || ty[a + d] != ty[b + d]) return 0;
        if (d > 0) {
            int la = IS_LMS(ty, a + d), lb = IS_LMS(ty, b + d);
            if (la && lb) return 1;
            if (la != lb) return 0;
        }
    }
}

/* SA of T[0..n) over the alphabet [0, k).  Returns 0, or -2 on allocation failure. */
static int sais_int(const int32_t *T, idx_t *SA, idx_t n, idx_t k)
{
    if (n <= 0) return 0;
    if (n == 1) { SA[0] = 0; return 0; }

    uint8_t *ty = (uint8_t *)malloc((size_t)n);
    idx_t *bkt = (idx_t *)malloc((size_t)k * sizeof(idx_t));
    if (!ty || !bkt) { free(ty); free(bkt); return -2; }

    ty[n - 1] = 0;
    for (idx_t i = n - 2; i >= 0; i--)
        ty[i] = (T[i] < T[i + 1]) || (T[i] == T[i + 1] && ty[i + 1]);

    /* stage 1: sort LMS substrings */
    for (idx_t i = 0; i < n; i++) SA[i] = -1;
    bucket_bounds(T, n, k, bkt, 1);
    for (idx_t i = 1; i < n; i++)
        if (IS_LMS(ty, i)) SA[--bkt[T[i]]] = i;
    induce(T, SA, n, k, ty, bkt);

    idx_t m = 0;
    for (idx_t i = 0; i < n; i++)
        if (IS_LMS(ty, SA[i])) SA[m++] = SA[i];

    /* name LMS substrings; names go to SA[m + p/2] */
    for (idx_t i = m; i < n; i++) SA[i] = -1;
    idx_t names = 0, prev = -1;
    for (idx_t i = 0; i < m; i++) {
        idx_t p = SA[i];
        if (!lms_equal(T, ty, n, p, prev)) { names++; prev = p; }
        SA[m + p / 2] = names - 1;
    }

    int32_t *s1 = (int32_t *)malloc((size_t)(m ? m : 1) * sizeof(int32_t));
    idx_t *sa1 = (idx_t *)malloc((size_t)(m ? m : 1) * sizeof(idx_t));
    idx_t *lms = (idx_t *)malloc((size_t)(m ? m : 1) * sizeof(idx_t));
    if (!s1 || !sa1 || !lms) { free(s1); free(sa1); free(lms); free(ty); free(bkt); return -2; }

    idx_t j = 0;
    for (idx_t i = m; i < n; i++)
        if (SA[i] >= 0) s1[j++] = (int32_t)SA[i];

    /* stage 2: order of the reduced string */
    int rc = 0;
    if (names < m) rc = sais_int(s1, sa1, m, names);
    else for (idx_t i = 0; i < m; i++) sa1[s1[i]] = i;

    if (rc == 0) {
        j = 0;
        for (idx_t i = 1; i < n; i++)
            if (IS_LMS(ty, i)) lms[j++] = i;

        /* stage 3: place sorted LMS suffixes at bucket ends and induce */
        for (idx_t i = 0; i < n; i++) SA[i] = -1;
        bucket_bounds(T, n, k, bkt, 1);
        for (idx_t i = m - 1; i >= 0; i--) {
            idx_t p = lms[sa1[i]];
            SA[--bkt[T[p]]] = p;
        }
        induce(T, SA, n, k, ty, bkt);
    }

    free(s1); free(sa1); free(lms); free(ty); free(bkt);
    return rc;
}

/* ------------------------------------------------------------ exported */

/* GSA validity (src/libsais.c:6886-6889 plus the T[n-1] == 0 API check). */
int oracle_gsa_valid(const void *T, int symbytes, idx_t n)
{
    if (n <= 0) return 1;
    #define SYM(i) (symbytes == 1 ? (int32_t)((const uint8_t *)T)[i] : (int32_t)((const uint16_t *)T)[i])
    if (SYM(n - 1) != 0) return 0;
    if (n == 1) return 1;
    if (SYM(0) == 0) return 0;
    for (idx_t i = 1; i < n; i++)
        if (SYM(i) == 0 && SYM(i - 1) == 0) return 0;
    return 1;
    #undef SYM
}

/*
 * Suffix array of an 8-bit (symbytes = 1) or 16-bit (symbytes = 2) text.
 * gsa != 0 sorts as a generalized suffix array (0 = separator).
 * Returns 0, -1 (invalid GSA input) or -2.
 */
int oracle_sa(const void *T, int symbytes, idx_t *SA, idx_t n, int gsa)
{
    if (n <= 0) return 0;
    if (gsa && !oracle_gsa_valid(T, symbytes, n)) return -1;
    int32_t *t = (int32_t *)malloc((size_t)n * sizeof(int32_t));
    if (!t) return -2;
    idx_t k = symbytes == 1 ? 256 : 65536;
    if (!gsa) {
        for (idx_t i = 0; i < n; i++)
            t[i] = symbytes == 1 ? ((const uint8_t *)T)[i] : ((const uint16_t *)T)[i];
    } else {
        idx_t seps = 0;
        for (idx_t i = 0; i < n; i++) {
            int32_t c = symbytes == 1 ? ((const uint8_t *)T)[i] : ((const uint16_t *)T)[i];
            if (c == 0) seps++;
        }
        idx_t s = 0;
        for (idx_t i = 0; i < n; i++) {
            int32_t c = symbytes == 1 ? ((const uint8_t *)T)[i] : ((const uint16_t *)T)[i];
            t[i] = c == 0 ? (int32_t)(s++) : (int32_t)(seps - 1 + c);
        }
        k = seps - 1 + k;
    }
    int rc = sais_int(t, SA, n, k);
    free(t);
    return rc;
}

/* Suffix array of an integer string over [0, k). */
int oracle_sa_int(const int32_t *T, idx_t *SA, idx_t n, idx_t k)
{
    return sais_int(T, SA, n, k);
}

/* freq[c] = number of occurrences of c (256 or 65536 entries). */
void oracle_freq(const void *T, int symbytes, idx_t n, idx_t *freq)
{
    idx_t k = symbytes == 1 ? 256 : 65536;
    memset(freq, 0, (size_t)k * sizeof(idx_t));
    for (idx_t i = 0; i < n; i++)
        freq[symbytes == 1 ? ((const uint8_t *)T)[i] : ((const uint16_t *)T)[i]]++;
}

/*
 * BWT from a suffix array with libsais_bwt's layout (src/libsais.c:7111-7118).
 * U receives n symbols of width symbytes.  Returns the primary index.
 * If r > 0, I[t] = 1 + ISA[t*r] for t = 0..(n-1)/r (libsais_bwt_aux).
 */
idx_t oracle_bwt(const void *T, int symbytes, const idx_t *SA, idx_t n, void *U, idx_t r, idx_t *I)
{
    if (n <= 0) return 0;
    idx_t i0 = -1;
    for (idx_t i = 0; i < n; i++) if (SA[i] == 0) { i0 = i; break; }
    #define GET(p) (symbytes == 1 ? (uint32_t)((const uint8_t *)T)[p] : (uint32_t)((const uint16_t *)T)[p])
    #define PUT(p, v) do { if (symbytes == 1) ((uint8_t *)U)[p] = (uint8_t)(v); else ((uint16_t *)U)[p] = (uint16_t)(v); } while (0)
    uint32_t first = GET(n - 1);
    idx_t k = 1;
    for (idx_t i = 0; i < n; i++) {
        if (i == i0) continue;
        PUT(k, GET(SA[i] - 1));
        k++;
    }
    PUT(0, first);
    #undef GET
    #undef PUT
    if (r > 0 && I) {
        for (idx_t i = 0; i < n; i++)
            if ((SA[i] & (r - 1)) == 0) I[SA[i] / r] = i + 1;
    }
    return i0 + 1;
}

/*
 * PLCP by the Phi method (src/libsais.c:8116-8190; GSA stop rule :8215-8238).
 * Phi[SA[0]] = n, Phi[SA[i]] = SA[i-1]; then Kasai's carried length.
 */
void oracle_plcp(const void *T, int symbytes, const idx_t *SA, idx_t *PLCP, idx_t n, int gsa)
{
    if (n <= 0) return;
    idx_t k = n;
    for (idx_t i = 0; i < n; i++) { PLCP[SA[i]] = k; k = SA[i]; }
    #define SYM(p) (symbytes == 1 ? (int32_t)((const uint8_t *)T)[p] : \
                    symbytes == 2 ? (int32_t)((const uint16_t *)T)[p] : ((const int32_t *)T)[p])
    idx_t l = 0;
    for (idx_t i = 0; i < n; i++) {
        idx_t j = PLCP[i];
        if (!gsa) {
            idx_t m = n - (i > j ? i : j);
            while (l < m && SYM(i + l) == SYM(j + l)) l++;
        } else {
            while (i + l < n && j + l < n && SYM(i + l) > 0 && SYM(i + l) == SYM(j + l)) l++;
        }
        PLCP[i] = l;
        l -= (l != 0);
    }
    #undef SYM
}

/*
 * Inverse BWT.  Rows 0..n of the BWT matrix: row 0 is the empty suffix, row
 * p (the primary index) has the sentinel as last symbol and is absent from U:
 * L[r] = U[r] for r < p, U[r - 1] for r > p.  LF(r) = C[L[r]] + (occurrences
 * of L[r] in L[0..r)), with C counting the sentinel.  Walking from row 0
 * yields the text backwards: T[n-1-j] = L[LF^j(0)].
 */
int oracle_unbwt(const void *U, int symbytes, idx_t n, idx_t p, void *T)
{
    if (n <= 0) return 0;
    if (p < 1 || p > n) return -1;
    const idx_t k = symbytes == 1 ? 256 : 65536;
    idx_t *C = calloc((size_t)k + 1, sizeof(idx_t));
    idx_t *occ = calloc((size_t)k, sizeof(idx_t));
    idx_t *lf = malloc((size_t)(n + 1) * sizeof(idx_t));
    if (!C || !occ || !lf) { free(C); free(occ); free(lf); return -2; }
    #define LSYM(r) (symbytes == 1 ? (idx_t)((const uint8_t *)U)[(r) < p ? (r) : (r) - 1] \
                                   : (idx_t)((const uint16_t *)U)[(r) < p ? (r) : (r) - 1])
    for (idx_t r = 0; r <= n; r++) if (r != p) C[LSYM(r) + 1]++;
    C[0] = 1;   /* the sentinel row sorts first */
    for (idx_t c = 1; c <= k; c++) C[c] += C[c - 1];
    for (idx_t r = 0; r <= n; r++) {
        if (r == p) { lf[r] = 0; continue; }
        const idx_t c = LSYM(r);
        lf[r] = C[c] + occ[c]++;
    }
    idx_t r = 0;
    for (idx_t j = 0; j < n; j++) {
        const idx_t c = LSYM(r);
        if (symbytes == 1) ((uint8_t *)T)[n - 1 - j] = (uint8_t)c;
        else ((uint16_t *)T)[n - 1 - j] = (uint16_t)c;
        r = lf[r];
        if (r == p && j + 1 < n) { free(C); free(occ); free(lf); return -1; }
    }
    #undef LSYM
    free(C); free(occ); free(lf);
    return 0;
}

/* LCP[i] = PLCP[SA[i]] (src/libsais.c:8311). */
void oracle_lcp(const idx_t *PLCP, const idx_t *SA, idx_t *LCP, idx_t n)
{
    for (idx_t i = 0; i < n; i++) LCP[i] = PLCP[SA[i]];
}

/*
 * Linear-time check that SA is the (generalized) suffix array of T
 * (permutation + neighbour rule with the inverse array).  Returns 1 if valid.
 */
int oracle_check_sa(const void *T, int symbytes, const idx_t *SA, idx_t n, int gsa)
{
    if (n <= 0) return 1;
    /* inverse ranks stored as rank + 1 (0 = unset / the end of the text), in
       32 bits when they fit so very long texts stay within host memory */
    const int narrow = n < 0xFFFFFFFFll;
    void *isa = calloc((size_t)(n + 1), narrow ? sizeof(uint32_t) : sizeof(idx_t));
    if (!isa) return -2;
    #define ISA_GET(p) (narrow ? (idx_t)((uint32_t *)isa)[p] : ((idx_t *)isa)[p])
    #define ISA_SET(p, v) do { if (narrow) ((uint32_t *)isa)[p] = (uint32_t)(v); else ((idx_t *)isa)[p] = (v); } while (0)
    for (idx_t i = 0; i < n; i++) {
        if (SA[i] < 0 || SA[i] >= n || ISA_GET(SA[i]) != 0) { free(isa); return 0; }
        ISA_SET(SA[i], i + 1);
    }
    #define SYM(p) (symbytes == 1 ? (int64_t)((const uint8_t *)T)[p] : (int64_t)((const uint16_t *)T)[p])
    int ok = 1;
    for (idx_t i = 1; i < n && ok; i++) {
        idx_t a = SA[i - 1], b = SA[i];
        int64_t ca = SYM(a), cb = SYM(b);
        if (ca < cb) continue;
        if (ca > cb) { ok = 0; break; }
        if (gsa && ca == 0) { ok = a < b; continue; }
        /* equal symbol: compare the following suffixes by rank (end = smallest) */
        if (ISA_GET(a + 1) >= ISA_GET(b + 1)) ok = 0;
    }
    #undef SYM
    #undef ISA_GET
    #undef ISA_SET
    free(isa);
    return ok;
}
