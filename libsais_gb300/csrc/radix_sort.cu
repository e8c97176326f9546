// radix_sort.cu -- LSD radix sort of (key, uint32 value) pairs with 32- or
// 64-bit keys, hand-written for sm_103a.
//
// One digit pass (8-bit digits, 256 buckets) is reduce-then-scan over tiles:
//   * k_tile_counts: digit counts of every tile (one read of the keys);
//   * k_tile_offsets: per digit, an exclusive scan over the tiles plus the
//     digit's bucket base gives every tile its global write offset per digit;
//   * k_radix_pass: full tiles are staged into shared memory with two TMA bulk
//     copies (keys, values) completing on one mbarrier; each warp ranks its
//     keys in input order (stable) with eight ballots per key (lanes holding
//     the same digit) and a per-warp shared digit counter; keys and values are
//     re-ordered by digit inside the tile and each digit run is written
//     contiguously at its offset.
// No CTA waits on another (no look-back chain): on a GB300 the extra read of
// the keys costs less than the L2 round trips a decoupled look-back spends.
// The global digit histograms of all passes come from one upsweep over the
// keys, or are accumulated by the producer of the keys.
// This replaces the bucket/induction passes of libsais's SA-IS
// (src/libsais.c:1586-1660 radix_sort_lms_suffixes, :4034 induce_partial_order)
// as the ordering primitive of the prefix-doubling suffix sort.
#include "device_util.cuh"
#include "engine.h"
#include "radix_hist.cuh"

namespace gsais {

namespace {

constexpr int kHistCopies = 4;

}  // namespace

// Test hook (gsais_test_stall_radix_wait): when non-zero, every full tile of
// k_radix_pass, after its staging copies have landed, also waits on a second
// mbarrier that nothing arrives on, giving up after this many nanoseconds.
// The give-up path is the one a real staging timeout takes: the error bit is
// raised (the call returns -2) and the tile is staged again with plain loads.
__device__ uint64_t g_test_stall_wait_ns = 0;

namespace {

// Histograms of every digit pass in one read of the keys (used when the
// producer of the keys did not accumulate them).  Counters are replicated
// kHistCopies times (by warp) to spread shared-atomic traffic.
// Bytes per key: sizeof(K) read.
template <typename K>
__global__ void __launch_bounds__(256) k_upsweep(const K *__restrict__ keys, uint64_t n, int passes, int begin_bit,
                                                 int end_bit, uint32_t *__restrict__ hist)
{
    __shared__ uint32_t sh[kHistCopies][8][256];
    for (int c = 0; c < kHistCopies; ++c) radix_hist_zero(sh[c], 8);
    __syncthreads();
    const int copy = (threadIdx.x >> 5) & (kHistCopies - 1);
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t n_round = (n + 31) & ~31ull;   // whole warps iterate together
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_round; i += stride) {
        const bool ok = i < n;
        radix_hist_add(sh[copy], ok ? ((uint64_t)keys[i] >> begin_bit) : 0, ok, passes, end_bit - begin_bit);
    }
    __syncthreads();
    for (int c = 1; c < kHistCopies; ++c)
        for (int i = threadIdx.x; i < passes * 256; i += blockDim.x) (&sh[0][0][0])[i] += (&sh[c][0][0])[i];
    __syncthreads();
    radix_hist_flush(sh[0], passes, hist);
}

// Exclusive bucket starts per pass: bases[p][d] = sum_{e<d} hist[p][e].
__global__ void __launch_bounds__(256) k_bucket_bases(const uint32_t *__restrict__ hist, uint32_t *__restrict__ bases)
{
    __shared__ uint32_t wbuf[9];
    const int p = blockIdx.x;
    uint32_t total;
    const uint32_t v = hist[p * 256 + threadIdx.x];
    const uint32_t e = block_exclusive_sum<uint32_t, 256>(v, wbuf, total);
    bases[p * 256 + threadIdx.x] = e;
}

// Tile shape of a digit pass: 256 threads (one per digit in the scans) x
// ITEMS keys.  The items per thread are a tuning parameter (RadixScratch);
// the instances compiled here are the candidates the autotuner searches.
template <typename K, int ITEMS>
struct PassShape {
    static constexpr int kThreads = 256, kItems = ITEMS;
    // registers: keys, values and ranks of ITEMS items stay in registers
    static constexpr int kMinBlocks = (ITEMS * (sizeof(K) / 4 + 1) <= 48) ? 3 : 2;
};

template <typename K, int ITEMS>
__host__ __device__ constexpr int pass_tile()
{
    return PassShape<K, ITEMS>::kThreads * ITEMS;
}

// staged keys + values of one tile; values are re-ordered in place (they are
// held in registers while the tile is ranked)
template <typename K, int ITEMS>
__host__ __device__ constexpr size_t pass_smem()
{
    return (size_t)pass_tile<K, ITEMS>() * (sizeof(K) + sizeof(uint32_t));
}

// Per-tile digit counts of one pass, digit-major: counts[d * tiles + t].
// Bytes per key: sizeof(K) read.
template <typename K, int ITEMS>
__global__ void __launch_bounds__(256) k_tile_counts(const K *__restrict__ keys, uint64_t n, int shift, uint32_t mask,
                                                     uint32_t *__restrict__ counts, uint32_t tiles)
{
    constexpr int TILE = pass_tile<K, ITEMS>();
    constexpr int PER_VEC = 16 / sizeof(K);
    static_assert(TILE % (256 * PER_VEC) == 0, "tile is a whole number of 16-byte vectors per thread");
    __shared__ uint32_t h[8][256];
    const int tid = threadIdx.x, warp = tid >> 5;
    for (int i = tid; i < 8 * 256; i += 256) (&h[0][0])[i] = 0;
    __syncthreads();
    const uint64_t base = (uint64_t)blockIdx.x * TILE;
    if (base + TILE <= n && (reinterpret_cast<uintptr_t>(keys) & 15) == 0) {
        const uint4 *k4 = reinterpret_cast<const uint4 *>(keys + base);
#pragma unroll
        for (int q = 0; q < TILE / (256 * PER_VEC); ++q) {
            const uint4 v = k4[q * 256 + tid];
            const K *kv = reinterpret_cast<const K *>(&v);
#pragma unroll
            for (int j = 0; j < PER_VEC; ++j) atomicAdd(&h[warp][(uint32_t)(kv[j] >> shift) & mask], 1u);
        }
    } else {
        for (uint64_t i = base + tid; i < n && i < base + TILE; i += 256)
            atomicAdd(&h[warp][(uint32_t)(keys[i] >> shift) & mask], 1u);
    }
    __syncthreads();
    uint32_t c = 0;
#pragma unroll
    for (int w = 0; w < 8; ++w) c += h[w][tid];
    counts[(uint64_t)tid * tiles + blockIdx.x] = c;
}

// One CTA per digit: offs[d * tiles + t] = bucket base of d + count of d in
// tiles before t.
__global__ void __launch_bounds__(1024) k_tile_offsets(const uint32_t *__restrict__ counts, uint32_t tiles,
                                                       const uint32_t *__restrict__ bases, uint32_t *__restrict__ offs)
{
    __shared__ uint32_t wbuf[33];
    const uint32_t d = blockIdx.x;
    const uint32_t *c = counts + (uint64_t)d * tiles;
    uint32_t *o = offs + (uint64_t)d * tiles;
    uint32_t run = bases[d];
    for (uint32_t b0 = 0; b0 < tiles; b0 += 1024 * 4) {
        uint32_t v[4], s = 0;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const uint32_t i = b0 + threadIdx.x * 4 + j;
            v[j] = i < tiles ? c[i] : 0u;
            s += v[j];
        }
        uint32_t total;
        uint32_t a = run + block_exclusive_sum<uint32_t, 1024>(s, wbuf, total);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const uint32_t i = b0 + threadIdx.x * 4 + j;
            if (i < tiles) o[i] = a;
            a += v[j];
        }
        run += total;
        __syncthreads();
    }
}

// Digit pass of one tile (tile = blockIdx.x): stage, rank stably, re-order by
// digit in shared memory, write each digit run to its global offset.
// vin == nullptr: the values are implicit, value(i) = n - 1 - i (the suffix
// indexes of seed keys written in reverse text order), so only keys are read.
template <typename K, int ITEMS>
__global__ void __launch_bounds__(PassShape<K, ITEMS>::kThreads, PassShape<K, ITEMS>::kMinBlocks)
    k_radix_pass(const K *__restrict__ kin, const uint32_t *__restrict__ vin, K *__restrict__ kout,
                 uint32_t *__restrict__ vout, uint64_t n, int shift, uint32_t mask,
                 const uint32_t *__restrict__ offs, uint32_t tiles, uint32_t *err)
{
    constexpr int THREADS = PassShape<K, ITEMS>::kThreads;
    static_assert(THREADS == 256, "one thread per digit");
    constexpr int TILE = THREADS * ITEMS;
    constexpr int WARPS = THREADS / 32;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    K *s_keys = reinterpret_cast<K *>(smem_raw);
    uint32_t *s_vals = reinterpret_cast<uint32_t *>(smem_raw + (size_t)TILE * sizeof(K));
    __shared__ uint32_t s_whist[WARPS][256];
    __shared__ uint32_t s_lstart[256];
    __shared__ uint32_t s_gbase[256];
    __shared__ uint32_t s_scan[WARPS + 1];
    __shared__ __align__(8) uint64_t s_bar;
    __shared__ __align__(8) uint64_t s_never;   // test hook only: no thread arrives on it

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t tile = blockIdx.x;
    const uint64_t base = (uint64_t)tile * TILE;
    const uint32_t valid = (uint32_t)((n - base) < (uint64_t)TILE ? (n - base) : (uint64_t)TILE);
    const bool full = valid == TILE;
    const uint64_t stall_ns = full ? g_test_stall_wait_ns : 0;
    const bool implicit = vin == nullptr;
    if (tid == 0 && full) {
        mbar_init(&s_bar, 1);
        if (stall_ns) mbar_init(&s_never, 1);
        mbar_arrive_expect_tx(&s_bar, TILE * (uint32_t)(sizeof(K) + (implicit ? 0 : sizeof(uint32_t))));
        bulk_copy_g2s(s_keys, kin + base, TILE * sizeof(K), &s_bar);
        if (!implicit) bulk_copy_g2s(s_vals, vin + base, TILE * sizeof(uint32_t), &s_bar);
    }
    for (int i = tid; i < WARPS * 256; i += THREADS) (&s_whist[0][0])[i] = 0;
    const uint32_t gofs = offs[(uint64_t)tid * tiles + tile];
    __syncthreads();
    bool staged = true;
    if (full) {
        bool landed = mbar_wait_bounded(&s_bar, 0, err);
        staged = landed;
        if (landed && stall_ns) staged = mbar_wait_bounded_ns(&s_never, 0, err, stall_ns);
        // A wait that gave up has raised the error bit (the call will return
        // -2).  The tile is then staged again with plain loads, so the pass
        // still writes a permutation of its input and no later kernel reads
        // stale entries as indexes; copies still in flight get one more
        // bounded wait first (they write the same bytes).
        staged = __syncthreads_and(staged);
        if (!staged && !landed) mbar_wait_bounded(&s_bar, 0, err);
    }
    if (!full || !staged) {
        for (uint32_t i = tid; i < valid; i += THREADS) {
            s_keys[i] = kin[base + i];
            if (!implicit) s_vals[i] = vin[base + i];
        }
        __syncthreads();
    }
    const uint32_t vbase = (uint32_t)(n - 1 - base);   // implicit value of entry base + i: vbase - i

    // ---- rank inside each warp, in input order (stable).  Lanes with equal
    // digits are found with eight ballots; the lowest such lane advances the
    // warp's counter for that digit after every lane has read it.
    // The implicit-value pass is the first pass that moves entries: its input
    // order only matters among equal keys, which the doubling rounds order
    // later, except for the suffixes shorter than a seed (the first slots,
    // in tile 0), whose padded keys tie with longer suffixes and must stay
    // first.  So its other tiles rank by shared-memory atomics (unstable).
    K kr[ITEMS];
    uint32_t vr[ITEMS];
    uint16_t rk[ITEMS];
    const int wbase = warp * ITEMS * 32;
    if (full && implicit && tile != 0) {
#pragma unroll
        for (int k = 0; k < ITEMS; ++k) {
            const int idx = wbase + k * 32 + lane;
            const K key = s_keys[idx];
            kr[k] = key;
            vr[k] = vbase - (uint32_t)idx;
            const uint32_t d = (uint32_t)(key >> shift) & mask;
            rk[k] = (uint16_t)atomicAdd(&s_whist[warp][d], 1u);
        }
    } else if (full) {
#pragma unroll
        for (int k = 0; k < ITEMS; ++k) {
            const int idx = wbase + k * 32 + lane;
            const K key = s_keys[idx];
            kr[k] = key;
            vr[k] = implicit ? vbase - (uint32_t)idx : s_vals[idx];
            const uint32_t d = (uint32_t)(key >> shift) & mask;
            uint32_t peers = GSAIS_FULL_MASK;
#pragma unroll
            for (int b = 0; b < 8; ++b) {
                const uint32_t bit = (d >> b) & 1u;
                peers &= __ballot_sync(GSAIS_FULL_MASK, bit) ^ (bit - 1u);
            }
            const uint32_t before = __popc(peers & lanemask_lt());
            const uint32_t old = s_whist[warp][d];
            __syncwarp();
            if (before == 0) s_whist[warp][d] = old + __popc(peers);
            __syncwarp();
            rk[k] = (uint16_t)(old + before);
        }
    } else {
#pragma unroll
        for (int k = 0; k < ITEMS; ++k) {
            const int idx = wbase + k * 32 + lane;
            const bool ok = (uint32_t)idx < valid;
            const K key = ok ? s_keys[idx] : K(0);
            kr[k] = key;
            vr[k] = ok ? (implicit ? vbase - (uint32_t)idx : s_vals[idx]) : 0u;
            const uint32_t d = ok ? ((uint32_t)(key >> shift) & mask) : 256u;
            const uint32_t peers = __match_any_sync(GSAIS_FULL_MASK, d);
            const uint32_t before = __popc(peers & lanemask_lt());
            uint32_t old = 0;
            if (ok && before == 0) old = atomicAdd(&s_whist[warp][d], (uint32_t)__popc(peers));
            old = __shfl_sync(GSAIS_FULL_MASK, old, __ffs(peers) - 1);
            rk[k] = (uint16_t)(old + before);
        }
    }
    __syncthreads();

    // ---- per-digit counts: exclusive over warps, then over the tile
    const uint32_t digit = tid;
    uint32_t count = 0;
#pragma unroll
    for (int w = 0; w < WARPS; ++w) {
        const uint32_t c = s_whist[w][digit];
        s_whist[w][digit] = count;
        count += c;
    }
    uint32_t total;
    const uint32_t lstart = block_exclusive_sum<uint32_t, THREADS>(count, s_scan, total);
    s_lstart[digit] = lstart;
    s_gbase[digit] = gofs - lstart;
    __syncthreads();

    // ---- re-order by digit inside the tile (all staged reads are done)
#pragma unroll
    for (int k = 0; k < ITEMS; ++k) {
        const int idx = wbase + k * 32 + lane;
        if (full || (uint32_t)idx < valid) {
            const uint32_t d = (uint32_t)(kr[k] >> shift) & mask;
            const uint32_t p = s_lstart[d] + s_whist[warp][d] + rk[k];
            s_keys[p] = kr[k];
            s_vals[p] = vr[k];
        }
    }
    __syncthreads();

    // ---- write digit runs to their global positions
    bool bad = false;
#pragma unroll
    for (int k = 0; k < ITEMS; ++k) {
        const uint32_t i = k * THREADS + tid;
        if (full || i < valid) {
            const K key = s_keys[i];
            const uint32_t d = (uint32_t)(key >> shift) & mask;
            const uint32_t o = s_gbase[d] + i;
            const bool ok = (uint64_t)o < n;
            bad |= !ok;
            if (ok) {
                kout[o] = key;
                vout[o] = s_vals[i];
            }
        }
    }
    if (bad) atomicOr(err, GSAIS_ERR_BOUNDS);
}

// vals[i] = n - 1 - i: the implicit values, materialised when no digit pass
// ran (every key alike).
__global__ void __launch_bounds__(256) k_fill_implicit(uint32_t *__restrict__ vals, uint64_t n)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        vals[i] = (uint32_t)(n - 1 - i);
}

__global__ void __launch_bounds__(256) k_read_back(uint32_t *__restrict__ dst, const uint32_t *__restrict__ src,
                                                   uint32_t words)
{
    for (uint32_t i = threadIdx.x; i < words; i += blockDim.x) dst[i] = src[i];
}

int sm_count()
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms > 0 ? sms : 1;
}

template <typename K, int ITEMS>
cudaError_t pass_attr()
{
    // cudaFuncSetAttribute applies to the current device; remember per device
    static bool done[64] = {false};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev >= 0 && dev < 64 && done[dev]) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(k_radix_pass<K, ITEMS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)pass_smem<K, ITEMS>());
    if (e == cudaSuccess && dev >= 0 && dev < 64) done[dev] = true;
    return e;
}

// One digit pass (tile counts, tile offsets, scatter) with ITEMS keys per thread.
template <typename K, int ITEMS>
cudaError_t run_pass(K *kin, const uint32_t *vin, K *kout, uint32_t *vout, uint64_t n, int shift, uint32_t mask,
                     const uint32_t *bases, uint32_t *counts, uint64_t status_words, RadixScratch &rs,
                     uint32_t *d_err, cudaStream_t st, bool implicit)
{
    constexpr int TILE = pass_tile<K, ITEMS>();
    const uint64_t tiles = (n + TILE - 1) / TILE;
    if (tiles * 256 * 2 > status_words * 2) return cudaErrorInvalidValue;   // counts + offsets
    cudaError_t e;
    if ((e = pass_attr<K, ITEMS>()) != cudaSuccess) return e;
    uint32_t *offs = counts + tiles * 256;
    cudaEvent_t ev0 = rs.prof ? rs.prof->begin(st) : nullptr;
    GSAIS_COUNTED((k_tile_counts<K, ITEMS><<<(unsigned)tiles, 256, 0, st>>>(kin, n, shift, mask, counts,
                                                                             (uint32_t)tiles)));
    GSAIS_COUNTED((k_tile_offsets<<<256, 1024, 0, st>>>(counts, (uint32_t)tiles, bases, offs)));
    if (ev0) rs.prof->end(KK_TILE_COUNTS, ev0, st, n * sizeof(K));
    cudaEvent_t ev1 = rs.prof ? rs.prof->begin(st) : nullptr;
    GSAIS_COUNTED((k_radix_pass<K, ITEMS><<<(unsigned)tiles, 256, pass_smem<K, ITEMS>(), st>>>(
        kin, implicit ? nullptr : vin, kout, vout, n, shift, mask, offs, (uint32_t)tiles, d_err)));
    // algorithmic bytes: every (key, value) pair read once and written once
    // (an implicit value is only written)
    if (ev1) rs.prof->end(KK_RADIX_PASS, ev1, st, n * (2 * sizeof(K) + (implicit ? 1 : 2) * sizeof(uint32_t)));
    return cudaGetLastError();
}

// Items per thread of the compiled pass instances, per key width.
bool items_supported(int key_bytes, int items)
{
    if (key_bytes == 4) return items == 16 || items == 20 || items == 24 || items == 28;
    return items == 12 || items == 16 || items == 20;
}

template <typename K>
cudaError_t run_pass_items(int items, K *kin, const uint32_t *vin, K *kout, uint32_t *vout, uint64_t n, int shift,
                           uint32_t mask, const uint32_t *bases, uint32_t *counts, uint64_t status_words,
                           RadixScratch &rs, uint32_t *d_err, cudaStream_t st, bool implicit)
{
#define GSAIS_PASS(I) \
    return run_pass<K, I>(kin, vin, kout, vout, n, shift, mask, bases, counts, status_words, rs, d_err, st, implicit)
    if constexpr (sizeof(K) == 4) {
        switch (items) {
        case 16: GSAIS_PASS(16);
        case 20: GSAIS_PASS(20);
        case 28: GSAIS_PASS(28);
        default: GSAIS_PASS(24);
        }
    } else {
        switch (items) {
        case 12: GSAIS_PASS(12);
        case 20: GSAIS_PASS(20);
        default: GSAIS_PASS(16);
        }
    }
#undef GSAIS_PASS
}

template <typename K>
cudaError_t sort_impl(K *keys[2], uint32_t *vals[2], uint64_t n, int begin_bit, int end_bit, RadixScratch &rs,
                      uint32_t *d_err, cudaStream_t st, int *which, int *passes_run, bool hist_ready,
                      bool implicit_vals = false)
{
    *which = 0;
    if (passes_run) *passes_run = 0;
    if (n <= 1 || end_bit <= begin_bit) {
        if (implicit_vals && n)
            GSAIS_COUNTED((k_fill_implicit<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(vals[0], n)));
        return cudaGetLastError();
    }
    const int passes = (end_bit - begin_bit + 7) / 8;
    cudaError_t e;
    if (!hist_ready) {
        if ((e = cudaMemsetAsync(rs.hist, 0, (size_t)passes * 256 * sizeof(uint32_t), st)) != cudaSuccess) return e;
        const uint64_t want = (n + 255) / 256;
        const uint64_t cap = (uint64_t)sm_count() * 8;
        const int grid = (int)(want < 1 ? 1 : (want < cap ? want : cap));
        cudaEvent_t ev = rs.prof ? rs.prof->begin(st) : nullptr;
        GSAIS_COUNTED((k_upsweep<K><<<grid, 256, 0, st>>>(keys[0], n, passes, begin_bit, end_bit, rs.hist)));
        if (ev) rs.prof->end(KK_UPSWEEP, ev, st, n * sizeof(K));
    }
    GSAIS_COUNTED((k_bucket_bases<<<passes, 256, 0, st>>>(rs.hist, rs.bases)));
    if ((e = read_back(rs.h_hist, rs.hist, (size_t)passes * 256 * sizeof(uint32_t), st)) != cudaSuccess) return e;
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;

    const int items = sizeof(K) == 4 ? rs.items32 : rs.items64;
    uint32_t *counts = reinterpret_cast<uint32_t *>(rs.status);
    int cur = 0, ran = 0;
    for (int p = 0; p < passes; ++p) {
        bool trivial = false;
        for (int d = 0; d < 256; ++d)
            if (rs.h_hist[p * 256 + d] == n) { trivial = true; break; }
        if (trivial) continue;
        const int shift = begin_bit + 8 * p;
        const int bits = end_bit - shift < 8 ? end_bit - shift : 8;
        const uint32_t mask = (1u << bits) - 1u;
        if ((e = run_pass_items<K>(items, keys[cur], vals[cur], keys[cur ^ 1], vals[cur ^ 1], n, shift, mask,
                                   rs.bases + p * 256, counts, rs.status_words, rs, d_err, st,
                                   implicit_vals && ran == 0)) != cudaSuccess)
            return e;
        cur ^= 1;
        ++ran;
    }
    if (implicit_vals && ran == 0)
        GSAIS_COUNTED((k_fill_implicit<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(vals[0], n)));
    *which = cur;
    if (passes_run) *passes_run = ran;
    return cudaGetLastError();
}

}  // namespace

cudaError_t set_test_stall_wait(uint64_t limit_ns)
{
    return cudaMemcpyToSymbol(g_test_stall_wait_ns, &limit_ns, sizeof(limit_ns));
}

cudaError_t read_back(void *h_dst, const void *d_src, size_t bytes, cudaStream_t st)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, h_dst) != cudaSuccess) {
        cudaGetLastError();
        a.type = cudaMemoryTypeUnregistered;
    }
    if (a.type != cudaMemoryTypeHost || !a.devicePointer || (bytes & 3) ||
        (reinterpret_cast<uintptr_t>(d_src) & 3) || (reinterpret_cast<uintptr_t>(h_dst) & 3))
        return cudaMemcpyAsync(h_dst, d_src, bytes, cudaMemcpyDeviceToHost, st);
    GSAIS_COUNTED((k_read_back<<<1, 256, 0, st>>>(static_cast<uint32_t *>(a.devicePointer),
                                                 static_cast<const uint32_t *>(d_src), (uint32_t)(bytes / 4))));
    return cudaGetLastError();
}

size_t radix_status_words(uint64_t n)
{
    // per (tile, digit): one 32-bit count and one 32-bit offset; sized for the
    // smallest pass tile of either key width (64-bit keys, 12 items)
    constexpr uint64_t TILE = (uint64_t)pass_tile<uint64_t, 12>();
    const uint64_t tiles = (n + TILE - 1) / TILE;
    return (size_t)(tiles ? tiles : 1) * 256;
}

bool radix_items_supported(int key_bytes, int items) { return items_supported(key_bytes, items); }

cudaError_t radix_sort_pairs(uint64_t *keys[2], uint32_t *vals[2], uint64_t n, int end_bit, RadixScratch &rs,
                             uint32_t *d_err, cudaStream_t st, int *which, int *passes_run, bool hist_ready)
{
    return sort_impl<uint64_t>(keys, vals, n, 0, end_bit, rs, d_err, st, which, passes_run, hist_ready);
}

cudaError_t radix_sort_pairs32(uint32_t *keys[2], uint32_t *vals[2], uint64_t n, int end_bit, RadixScratch &rs,
                               uint32_t *d_err, cudaStream_t st, int *which, int *passes_run, bool hist_ready,
                               bool implicit_vals)
{
    return sort_impl<uint32_t>(keys, vals, n, 0, end_bit, rs, d_err, st, which, passes_run, hist_ready,
                               implicit_vals);
}

cudaError_t radix_partition32(uint32_t *keys[2], uint32_t *vals[2], uint64_t n, int begin_bit, int end_bit,
                              RadixScratch &rs, uint32_t *d_err, cudaStream_t st, int *which)
{
    return sort_impl<uint32_t>(keys, vals, n, begin_bit, end_bit, rs, d_err, st, which, nullptr, false);
}

std::atomic<uint64_t> g_launches{0};

cudaEvent_t KernelProfiler::get()
{
    if (!pool.empty()) {
        cudaEvent_t e = pool.back();
        pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
    return e;
}

cudaEvent_t KernelProfiler::begin(cudaStream_t st)
{
    if (!enabled) return nullptr;
    cudaEvent_t a = get();
    if (a) cudaEventRecord(a, st);
    return a;
}

void KernelProfiler::end(int kind, cudaEvent_t a, cudaStream_t st, uint64_t b)
{
    if (!enabled || !a) return;
    cudaEvent_t e = get();
    if (!e) return;
    cudaEventRecord(e, st);
    pending.push_back({kind, a, e, b});
}

void KernelProfiler::flush()
{
    for (auto &r : pending) {
        float t = 0.f;
        if (cudaEventElapsedTime(&t, r.a, r.b) == cudaSuccess) {
            ms[r.kind] += t;
            launches[r.kind] += 1;
            bytes[r.kind] += r.bytes;
        }
        pool.push_back(r.a);
        pool.push_back(r.b);
    }
    pending.clear();
}

void KernelProfiler::reset()
{
    flush();
    for (int k = 0; k < KK_COUNT; ++k) { ms[k] = 0; launches[k] = 0; bytes[k] = 0; }
}

KernelProfiler::~KernelProfiler()
{
    for (auto &r : pending) { pool.push_back(r.a); pool.push_back(r.b); }
    for (auto e : pool) cudaEventDestroy(e);
}

}  // namespace gsais
