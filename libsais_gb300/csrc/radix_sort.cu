// radix_sort.cu -- onesweep LSD radix sort of (key, uint32 value) pairs with
// 32- or 64-bit keys, hand-written for sm_103a.
//
// Layout of one digit pass (8-bit digits, 256 buckets):
//   * a CTA takes the next tile ticket (atomic counter, so tiles start in
//     ticket order and the look-back below always makes progress);
//   * full tiles are staged into shared memory with two TMA bulk copies
//     (keys, values) completing on one mbarrier; the ragged last tile uses
//     guarded loads;
//   * each warp ranks its keys with __match_any_sync over the digit and a
//     per-warp shared-memory digit histogram, in input order (stable);
//   * per-digit tile counts are published to a decoupled look-back array and
//     the exclusive prefix over earlier tiles is gathered with bounded spins;
//   * keys (from registers) and values (shared -> shared) are re-ordered by
//     digit inside the tile and written out, so each digit run of the tile
//     lands contiguously in global memory.
// The histograms of all digit passes come from one upsweep over the keys.
// This replaces the bucket/induction passes of libsais's SA-IS
// (src/libsais.c:1586-1660 radix_sort_lms_suffixes, :4034 induce_partial_order)
// as the ordering primitive of the prefix-doubling suffix sort.
#include "device_util.cuh"
#include "engine.h"
#include "radix_hist.cuh"

namespace gsais {

namespace {

constexpr uint64_t kFlagAggregate = 1ull << 62;
constexpr uint64_t kFlagPrefix = 2ull << 62;
constexpr uint64_t kValueMask = (1ull << 62) - 1;
constexpr int kHistCopies = 4;

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

__device__ __forceinline__ uint32_t lookback_exclusive(uint64_t *status, uint32_t tile, uint32_t digit,
                                                       uint32_t count, uint32_t *err)
{
    uint64_t *mine = status + (uint64_t)tile * 256 + digit;
    if (tile == 0) {
        st_relaxed_gpu(mine, kFlagPrefix | count);
        return 0;
    }
    st_relaxed_gpu(mine, kFlagAggregate | count);
    uint64_t excl = 0;
    int64_t u = (int64_t)tile - 1;
    uint32_t spins = 0;
    uint64_t t0 = 0;
    while (u >= 0) {
        const uint64_t s = ld_relaxed_gpu(status + (uint64_t)u * 256 + digit);
        const uint64_t f = s & ~kValueMask;
        if (f == 0) {
            if (spins == 0) t0 = global_ns();
            if (++spins > GSAIS_SPIN_LIMIT || ((spins & 255) == 0 && global_ns() - t0 > GSAIS_SPIN_NS)) {
                atomicOr(err, GSAIS_ERR_LOOKBACK_SPIN);
                break;
            }
            __nanosleep(32);
            continue;
        }
        excl += s & kValueMask;
        if (f == kFlagPrefix) break;
        --u;
    }
    st_relaxed_gpu(mine, kFlagPrefix | (excl + count));
    return (uint32_t)excl;
}

template <typename K>
struct OnesweepShape;
template <>
struct OnesweepShape<uint64_t> {
    static constexpr int kThreads = 256, kItems = 16, kMinBlocks = 3;
};
template <>
struct OnesweepShape<uint32_t> {
    static constexpr int kThreads = 256, kItems = 16, kMinBlocks = 4;
};

template <typename K>
constexpr size_t onesweep_smem()
{
    return (size_t)OnesweepShape<K>::kThreads * OnesweepShape<K>::kItems * (sizeof(K) + 2 * sizeof(uint32_t));
}

template <typename K>
__global__ void __launch_bounds__(OnesweepShape<K>::kThreads, OnesweepShape<K>::kMinBlocks)
    k_onesweep(const K *__restrict__ kin, const uint32_t *__restrict__ vin, K *__restrict__ kout,
               uint32_t *__restrict__ vout, uint64_t n, int shift, uint32_t mask, const uint32_t *__restrict__ bases,
               uint64_t *status, uint32_t *counter, uint32_t *err)
{
    constexpr int THREADS = OnesweepShape<K>::kThreads;
    constexpr int ITEMS = OnesweepShape<K>::kItems;
    static_assert(THREADS == 256, "one thread per digit");
    constexpr int TILE = THREADS * ITEMS;
    constexpr int WARPS = THREADS / 32;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    K *s_keys = reinterpret_cast<K *>(smem_raw);                                       // staged, then sorted
    uint32_t *s_vin = reinterpret_cast<uint32_t *>(smem_raw + (size_t)TILE * sizeof(K));   // staged values
    uint32_t *s_vout = s_vin + TILE;                                                    // sorted values
    __shared__ uint32_t s_whist[WARPS][256];
    __shared__ uint32_t s_lstart[256];
    __shared__ uint32_t s_gbase[256];
    __shared__ uint32_t s_scan[WARPS + 1];
    __shared__ __align__(8) uint64_t s_bar;
    __shared__ uint32_t s_tile;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

    if (tid == 0) {
        const uint32_t t = atomicAdd(counter, 1u);
        s_tile = t;
        const uint64_t b = (uint64_t)t * TILE;
        if (b + TILE <= n) {
            mbar_init(&s_bar, 1);
            mbar_arrive_expect_tx(&s_bar, TILE * (uint32_t)(sizeof(K) + sizeof(uint32_t)));
            bulk_copy_g2s(s_keys, kin + b, TILE * sizeof(K), &s_bar);
            bulk_copy_g2s(s_vin, vin + b, TILE * sizeof(uint32_t), &s_bar);
        }
    }
    for (int i = tid; i < WARPS * 256; i += THREADS) (&s_whist[0][0])[i] = 0;
    __syncthreads();

    const uint32_t tile = s_tile;
    const uint64_t base = (uint64_t)tile * TILE;
    const uint32_t valid = (uint32_t)((n - base) < (uint64_t)TILE ? (n - base) : (uint64_t)TILE);
    if (valid == TILE) {
        mbar_wait_bounded(&s_bar, 0, err);
    } else {
        for (uint32_t i = tid; i < valid; i += THREADS) {
            s_keys[i] = kin[base + i];
            s_vin[i] = vin[base + i];
        }
        __syncthreads();
    }

    // ---- rank keys inside each warp, in input order (stable)
    K kr[ITEMS];
    uint16_t rk[ITEMS];
    const int wbase = warp * ITEMS * 32;
#pragma unroll
    for (int k = 0; k < ITEMS; ++k) {
        const int idx = wbase + k * 32 + lane;
        const bool ok = (uint32_t)idx < valid;
        const K key = ok ? s_keys[idx] : K(0);
        kr[k] = key;
        const uint32_t d = ok ? (uint32_t)((key >> shift) & mask) : 256u;
        const uint32_t peers = __match_any_sync(GSAIS_FULL_MASK, d);
        const uint32_t before = __popc(peers & lanemask_lt());
        // the lowest lane of each digit group bumps the warp's counter once;
        // successive items of a warp hit the shared atomic unit in program
        // order, so ranks stay in input order (stable)
        uint32_t old = 0;
        if (ok && before == 0) old = atomicAdd(&s_whist[warp][d], (uint32_t)__popc(peers));
        old = __shfl_sync(GSAIS_FULL_MASK, old, __ffs(peers) - 1);
        rk[k] = (uint16_t)(old + before);
    }
    __syncthreads();

    // ---- per-digit counts: exclusive over warps, then across tiles
    const uint32_t digit = tid;
    uint32_t count = 0;
#pragma unroll
    for (int w = 0; w < WARPS; ++w) {
        const uint32_t c = s_whist[w][digit];
        s_whist[w][digit] = count;
        count += c;
    }
    const uint32_t excl = lookback_exclusive(status, tile, digit, count, err);
    uint32_t total;
    const uint32_t lstart = block_exclusive_sum<uint32_t, THREADS>(count, s_scan, total);
    s_lstart[digit] = lstart;
    s_gbase[digit] = bases[digit] + excl - lstart;
    __syncthreads();

    // ---- reorder by digit inside the tile (keys from registers, values shared -> shared)
#pragma unroll
    for (int k = 0; k < ITEMS; ++k) {
        const int idx = wbase + k * 32 + lane;
        if ((uint32_t)idx < valid) {
            const uint32_t d = (uint32_t)((kr[k] >> shift) & mask);
            const uint32_t p = s_lstart[d] + s_whist[warp][d] + rk[k];
            s_keys[p] = kr[k];
            s_vout[p] = s_vin[idx];
        }
    }
    __syncthreads();

    // ---- write digit runs to their global positions
    for (uint32_t i = tid; i < valid; i += THREADS) {
        const K key = s_keys[i];
        const uint32_t d = (uint32_t)((key >> shift) & mask);
        const uint32_t o = s_gbase[d] + i;
        if ((uint64_t)o < n) {
            kout[o] = key;
            vout[o] = s_vout[i];
        } else {
            atomicOr(err, GSAIS_ERR_BOUNDS);
        }
    }
}

int sm_count()
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms > 0 ? sms : 1;
}

template <typename K>
cudaError_t onesweep_attr()
{
    // cudaFuncSetAttribute applies to the current device; remember per device
    static bool done[64] = {false};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev >= 0 && dev < 64 && done[dev]) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(k_onesweep<K>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)onesweep_smem<K>());
    if (e == cudaSuccess && dev >= 0 && dev < 64) done[dev] = true;
    return e;
}

template <typename K>
cudaError_t sort_impl(K *keys[2], uint32_t *vals[2], uint64_t n, int begin_bit, int end_bit, RadixScratch &rs,
                      uint32_t *d_err, cudaStream_t st, int *which, int *passes_run, bool hist_ready)
{
    *which = 0;
    if (passes_run) *passes_run = 0;
    if (n <= 1 || end_bit <= begin_bit) return cudaSuccess;
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
    if ((e = cudaMemcpyAsync(rs.h_hist, rs.hist, (size_t)passes * 256 * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                             st)) != cudaSuccess)
        return e;
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
    if ((e = onesweep_attr<K>()) != cudaSuccess) return e;

    constexpr int TILE = OnesweepShape<K>::kThreads * OnesweepShape<K>::kItems;
    const uint64_t tiles = (n + TILE - 1) / TILE;
    int cur = 0, ran = 0;
    for (int p = 0; p < passes; ++p) {
        bool trivial = false;
        for (int d = 0; d < 256; ++d)
            if (rs.h_hist[p * 256 + d] == n) { trivial = true; break; }
        if (trivial) continue;
        if ((e = cudaMemsetAsync(rs.status, 0, (size_t)tiles * 256 * sizeof(uint64_t), st)) != cudaSuccess) return e;
        if ((e = cudaMemsetAsync(rs.counters + p, 0, sizeof(uint32_t), st)) != cudaSuccess) return e;
        const int bits = end_bit - begin_bit - 8 * p < 8 ? end_bit - begin_bit - 8 * p : 8;
        const uint32_t mask = (1u << bits) - 1u;
        cudaEvent_t ev1 = rs.prof ? rs.prof->begin(st) : nullptr;
        GSAIS_COUNTED((k_onesweep<K><<<(unsigned)tiles, OnesweepShape<K>::kThreads, onesweep_smem<K>(), st>>>(
            keys[cur], vals[cur], keys[cur ^ 1], vals[cur ^ 1], n, begin_bit + 8 * p, mask, rs.bases + p * 256, rs.status,
            rs.counters + p, d_err)));
        // algorithmic bytes: every (key, value) pair read once and written once
        if (ev1) rs.prof->end(KK_ONESWEEP, ev1, st, 2 * n * (sizeof(K) + sizeof(uint32_t)));
        cur ^= 1;
        ++ran;
    }
    *which = cur;
    if (passes_run) *passes_run = ran;
    return cudaGetLastError();
}

}  // namespace

size_t radix_status_words(uint64_t n)
{
    constexpr int TILE = 4096;   // the smallest onesweep tile of either key width
    const uint64_t tiles = (n + TILE - 1) / TILE;
    return (size_t)(tiles ? tiles : 1) * 256;
}

cudaError_t radix_sort_pairs(uint64_t *keys[2], uint32_t *vals[2], uint64_t n, int end_bit, RadixScratch &rs,
                             uint32_t *d_err, cudaStream_t st, int *which, int *passes_run, bool hist_ready)
{
    return sort_impl<uint64_t>(keys, vals, n, 0, end_bit, rs, d_err, st, which, passes_run, hist_ready);
}

cudaError_t radix_sort_pairs32(uint32_t *keys[2], uint32_t *vals[2], uint64_t n, int end_bit, RadixScratch &rs,
                               uint32_t *d_err, cudaStream_t st, int *which, int *passes_run, bool hist_ready)
{
    return sort_impl<uint32_t>(keys, vals, n, 0, end_bit, rs, d_err, st, which, passes_run, hist_ready);
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
