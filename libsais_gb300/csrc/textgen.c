/*
 * textgen.c -- seeded synthetic texts for the suffix-sorting workloads.
 *
 * The public corpora that libsais's Benchmarks.md times (E.coli, chr22, cere,
 * the Pizza&Chili DNA files, ...) are not available here, so every workload
 * uses seeded synthetic inputs with the same shapes: DNA-like texts over
 * {A,C,G,T}, repetitive genome-like texts, degenerate stress texts, short-read
 * sets for the generalized suffix array and Zipf-distributed 16-bit texts.
 *
 * RNG: xoshiro256** seeded through SplitMix64, so a (generator, seed) pair
 * gives the same bytes on every machine.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct { uint64_t s[4]; } rng_t;

static uint64_t splitmix64(uint64_t *x)
{
    uint64_t z = (*x += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static void rng_seed(rng_t *r, uint64_t seed)
{
    uint64_t x = seed;
    for (int i = 0; i < 4; i++) r->s[i] = splitmix64(&x);
}

static inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

static inline uint64_t rng_next(rng_t *r)
{
    uint64_t *s = r->s;
    uint64_t result = rotl(s[1] * 5, 7) * 9;
    uint64_t t = s[1] << 17;
    s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3];
    s[2] ^= t; s[3] = rotl(s[3], 45);
    return result;
}

/* uniform double in [0, 1) */
static inline double rng_unit(rng_t *r) { return (double)(rng_next(r) >> 11) * (1.0 / 9007199254740992.0); }

/* uniform integer in [0, k) */
static inline uint64_t rng_below(rng_t *r, uint64_t k) { return k ? (uint64_t)(rng_unit(r) * (double)k) % k : 0; }

static const uint8_t DNA[4] = {'A', 'C', 'G', 'T'};

/* i.i.d. symbols drawn uniformly from alphabet[0..k). */
void tg_iid_u8(uint8_t *out, uint64_t n, const uint8_t *alphabet, int k, uint64_t seed)
{
    rng_t r; rng_seed(&r, seed);
    for (uint64_t i = 0; i < n; i++) out[i] = alphabet[rng_below(&r, (uint64_t)k)];
}

/* i.i.d. ACGT with a given fraction of 'N' (byte 78). */
void tg_dna_with_n(uint8_t *out, uint64_t n, double n_frac, uint64_t seed)
{
    rng_t r; rng_seed(&r, seed);
    for (uint64_t i = 0; i < n; i++)
        out[i] = rng_unit(&r) < n_frac ? (uint8_t)'N' : DNA[rng_next(&r) >> 62];
}

void tg_constant(uint8_t *out, uint64_t n, uint8_t c) { memset(out, c, n); }

void tg_periodic(uint8_t *out, uint64_t n, const uint8_t *pattern, uint64_t plen)
{
    for (uint64_t i = 0; i < n; i++) out[i] = pattern[i % plen];
}

/*
 * Order-2 Markov DNA.  Stationary vector with the given GC content
 * (P(C) = P(G) = gc/2, P(A) = P(T) = (1-gc)/2); each of the 16 two-base
 * contexts draws its row as stationary x (1 +- 20% seeded jitter), renormalised.
 */
static void markov2_fill(rng_t *r, uint8_t *out, uint64_t n, double gc)
{
    double stat[4] = {(1.0 - gc) / 2, gc / 2, gc / 2, (1.0 - gc) / 2};
    double cdf[16][4];
    for (int c = 0; c < 16; c++) {
        double row[4], sum = 0;
        for (int b = 0; b < 4; b++) { row[b] = stat[b] * (0.8 + 0.4 * rng_unit(r)); sum += row[b]; }
        double acc = 0;
        for (int b = 0; b < 4; b++) { acc += row[b] / sum; cdf[c][b] = acc; }
        cdf[c][3] = 1.0;
    }
    int ctx = (int)(rng_next(r) >> 60);
    for (uint64_t i = 0; i < n; i++) {
        double u = rng_unit(r);
        int b = 0;
        while (b < 3 && u >= cdf[ctx][b]) b++;
        out[i] = DNA[b];
        ctx = ((ctx << 2) | b) & 15;
    }
}

void tg_markov2_dna(uint8_t *out, uint64_t n, double gc, uint64_t seed)
{
    rng_t r; rng_seed(&r, seed);
    markov2_fill(&r, out, n, gc);
}

static inline uint8_t substitute(rng_t *r, uint8_t c)
{
    uint8_t d;
    do { d = DNA[rng_next(r) >> 62]; } while (d == c);
    return d;
}

/*
 * Repetitive genome-like text: order-2 Markov DNA (GC 0.41), then about
 * dup_frac of the positions overwritten by copies of earlier segments
 * (lengths log-uniform over [1 KiB, 1 MiB], 0.1% substitutions), then tandem
 * repeats (period U{2..64}, copies U{10..500}) covering about tandem_frac.
 */
void tg_genome_like(uint8_t *out, uint64_t n, double dup_frac, double tandem_frac, uint64_t seed)
{
    rng_t r; rng_seed(&r, seed);
    markov2_fill(&r, out, n, 0.41);

    uint64_t budget = (uint64_t)(dup_frac * (double)n), done = 0;
    const double lo = log(1024.0), hi = log(1048576.0);
    while (done < budget && n > 4096) {
        uint64_t len = (uint64_t)exp(lo + (hi - lo) * rng_unit(&r));
        if (len > n / 4) len = n / 4;
        if (len < 16) break;
        uint64_t dst = len + rng_below(&r, n - 2 * len);       /* dst >= len, dst + len <= n */
        uint64_t src = rng_below(&r, dst - len + 1);            /* src + len <= dst: an earlier segment */
        memmove(out + dst, out + src, len);
        for (uint64_t i = 0; i < len; i++)
            if (rng_unit(&r) < 0.001) out[dst + i] = substitute(&r, out[dst + i]);
        done += len;
    }

    budget = (uint64_t)(tandem_frac * (double)n); done = 0;
    while (done < budget && n > 65536) {
        uint64_t period = 2 + rng_below(&r, 63);
        uint64_t copies = 10 + rng_below(&r, 491);
        uint64_t len = period * copies;
        uint64_t dst = rng_below(&r, n - len);
        uint8_t unit[64];
        for (uint64_t i = 0; i < period; i++) unit[i] = DNA[rng_next(&r) >> 62];
        for (uint64_t i = 0; i < len; i++) out[dst + i] = unit[i % period];
        done += len;
    }
}

/* Lengths log-uniform over [lo, hi] (inclusive), rounded to integers. */
void tg_loguniform_lengths(uint64_t *out, uint64_t count, double lo, double hi, uint64_t seed)
{
    rng_t r; rng_seed(&r, seed);
    double a = log(lo), b = log(hi);
    for (uint64_t i = 0; i < count; i++) {
        uint64_t v = (uint64_t)llround(exp(a + (b - a) * rng_unit(&r)));
        if (v < (uint64_t)lo) v = (uint64_t)lo;
        if (v > (uint64_t)hi) v = (uint64_t)hi;
        out[i] = v;
    }
}

/*
 * Short-read set for the generalized suffix array: a random ACGT reference of
 * ref_len bases, then nreads reads of length round(N(150, 20)) clipped to
 * [50, 300] from uniform start positions with 1% substitutions, each followed
 * by byte 0.  Writes at most cap bytes; returns the total length written.
 */
uint64_t tg_reads_gsa(uint8_t *out, uint64_t cap, uint64_t nreads, uint64_t ref_len, uint64_t seed)
{
    rng_t r; rng_seed(&r, seed);
    uint8_t *ref = (uint8_t *)malloc(ref_len ? ref_len : 1);
    if (!ref) return 0;
    for (uint64_t i = 0; i < ref_len; i++) ref[i] = DNA[rng_next(&r) >> 62];
    uint64_t pos = 0;
    for (uint64_t k = 0; k < nreads; k++) {
        double u1 = rng_unit(&r), u2 = rng_unit(&r);
        double z = sqrt(-2.0 * log(u1 > 1e-300 ? u1 : 1e-300)) * cos(6.283185307179586 * u2);
        long len = lround(150.0 + 20.0 * z);
        if (len < 50) len = 50;
        if (len > 300) len = 300;
        if ((uint64_t)len > ref_len) len = (long)ref_len;
        if (pos + (uint64_t)len + 1 > cap) break;
        uint64_t start = rng_below(&r, ref_len - (uint64_t)len + 1);
        for (long i = 0; i < len; i++) {
            uint8_t c = ref[start + (uint64_t)i];
            out[pos++] = rng_unit(&r) < 0.01 ? substitute(&r, c) : c;
        }
        out[pos++] = 0;
    }
    free(ref);
    return pos;
}

/* 16-bit text, Zipf(s) over symbols 1..kmax (rank 1 most frequent). */
int tg_zipf_u16(uint16_t *out, uint64_t n, double s, uint32_t kmax, uint64_t seed)
{
    rng_t r; rng_seed(&r, seed);
    double *cdf = (double *)malloc((size_t)kmax * sizeof(double));
    if (!cdf) return -1;
    double acc = 0;
    for (uint32_t k = 0; k < kmax; k++) { acc += 1.0 / pow((double)(k + 1), s); cdf[k] = acc; }
    for (uint32_t k = 0; k < kmax; k++) cdf[k] /= acc;
    /* a fixed seeded permutation decouples symbol value from frequency rank */
    uint16_t *perm = (uint16_t *)malloc((size_t)kmax * sizeof(uint16_t));
    if (!perm) { free(cdf); return -1; }
    for (uint32_t k = 0; k < kmax; k++) perm[k] = (uint16_t)(k + 1);
    for (uint32_t k = kmax - 1; k > 0; k--) {
        uint32_t j = (uint32_t)rng_below(&r, (uint64_t)k + 1);
        uint16_t t = perm[k]; perm[k] = perm[j]; perm[j] = t;
    }
    for (uint64_t i = 0; i < n; i++) {
        double u = rng_unit(&r);
        uint32_t lo = 0, hi = kmax - 1;
        while (lo < hi) { uint32_t mid = (lo + hi) >> 1; if (cdf[mid] < u) lo = mid + 1; else hi = mid; }
        out[i] = perm[lo];
    }
    free(perm); free(cdf);
    return 0;
}

/* Poisson arrival times (seconds) at the given rate. */
void tg_poisson_arrivals(double *out, uint64_t count, double rate, uint64_t seed)
{
    rng_t r; rng_seed(&r, seed);
    double t = 0;
    for (uint64_t i = 0; i < count; i++) {
        double u = rng_unit(&r);
        t += -log(1.0 - u) / rate;
        out[i] = t;
    }
}

/* uniform double stream, for host-side choices that must be seeded */
void tg_uniform(double *out, uint64_t count, uint64_t seed)
{
    rng_t r; rng_seed(&r, seed);
    for (uint64_t i = 0; i < count; i++) out[i] = rng_unit(&r);
}
