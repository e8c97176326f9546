// radix_sort.cu -- onesweep LSD radix sort of (uint64 key, uint32 value)
// pairs, hand-written for sm_103a.
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
//   * keys/values are re-ordered by digit in shared memory and written out,
//     so each digit run of the tile is written contiguously.
// The histograms for all digit passes come from one upsweep over the keys.
// This replaces the bucket/induction passes of libsais's SA-IS
// (src/libsais.c:1586-1660 radix_sort_lms_suffixes, :4034 induce_partial_order)
// as the ordering primitive of the prefix-doubling suffix sort.
#include "device_util.cuh"
#include "engine.h"

namespace gsais {

namespace {

constexpr uint64_t kFlagAggregate = 1ull << 62;
constexpr uint64_t kFlagPrefix = 2ull << 62;
constexpr uint64_t kValueMask = (1ull << 62) - 1;

// Histogram of every 8-bit digit of every key, `passes` digits per key.
__global__ void __launch_bounds__(256) k_upsweep(const uint64_t *__restrict__ keys, uint64_t n, int passes,
                                                 int end_bit, uint32_t *__restrict__ hist)
{
    __shared__ uint32_t sh[8][256];
    for (int i = threadIdx.x; i < 8 * 256; i += blockDim.x) (&sh[0][0])[i] = 0;
    __syncthreads();
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    // whole warps iterate together so __match_any_sync sees full masks
    const uint64_t n_round = (n + 31) & ~31ull;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_round; i += stride) {
        const bool ok = i < n;
        const uint64_t k = ok ? keys[i] : 0;
        for (int p = 0; p < passes; ++p) {
            const int bits = end_bit - 8 * p < 8 ? end_bit - 8 * p : 8;
            const uint32_t d = ok ? (uint32_t)((k >> (8 * p)) & ((1u << bits) - 1u)) : 256u;
            const uint32_t peers = __match_any_sync(GSAIS_FULL_MASK, d);
            if (ok && (peers & lanemask_lt()) == 0) atomicAdd(&sh[p][d], (uint32_t)__popc(peers));
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < passes * 256; i += blockDim.x) {
        const uint32_t v = (&sh[0][0])[i];
        if (v) atomicAdd(&hist[i], v);
    }
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

template <int THREADS, int ITEMS>
__global__ void __launch_bounds__(THREADS, 2)
    k_onesweep(const uint64_t *__restrict__ kin, const uint32_t *__restrict__ vin, uint64_t *__restrict__ kout,
               uint32_t *__restrict__ vout, uint64_t n, int shift, uint32_t mask, const uint32_t *__restrict__ bases,
               uint64_t *status, uint32_t *counter, uint32_t *err)
{
    static_assert(THREADS == 256, "one thread per digit");
    constexpr int TILE = THREADS * ITEMS;
    constexpr int WARPS = THREADS / 32;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    uint64_t *s_keys = reinterpret_cast<uint64_t *>(smem_raw);
    uint32_t *s_vals = reinterpret_cast<uint32_t *>(smem_raw + (size_t)TILE * sizeof(uint64_t));
    __shared__ uint16_t s_whist[WARPS][256];
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
            mbar_arrive_expect_tx(&s_bar, TILE * (uint32_t)(sizeof(uint64_t) + sizeof(uint32_t)));
            bulk_copy_g2s(s_keys, kin + b, TILE * sizeof(uint64_t), &s_bar);
            bulk_copy_g2s(s_vals, vin + b, TILE * sizeof(uint32_t), &s_bar);
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
            s_vals[i] = vin[base + i];
        }
        __syncthreads();
    }

    // ---- rank keys inside each warp, in input order (stable)
    uint64_t kr[ITEMS];
    uint16_t rk[ITEMS];
    const int wbase = warp * ITEMS * 32;
#pragma unroll
    for (int k = 0; k < ITEMS; ++k) {
        const int idx = wbase + k * 32 + lane;
        const bool ok = (uint32_t)idx < valid;
        const uint64_t key = ok ? s_keys[idx] : 0ull;
        kr[k] = key;
        const uint32_t d = ok ? (uint32_t)((key >> shift) & mask) : 256u;
        const uint32_t peers = __match_any_sync(GSAIS_FULL_MASK, d);
        const uint32_t before = __popc(peers & lanemask_lt());
        uint32_t cnt = 0;
        if (ok) cnt = s_whist[warp][d];
        __syncwarp();
        if (ok && before == 0) s_whist[warp][d] = (uint16_t)(cnt + __popc(peers));
        __syncwarp();
        rk[k] = (uint16_t)(cnt + before);
    }
    __syncthreads();

    // ---- per-digit counts: exclusive over warps, then across tiles
    const uint32_t digit = tid;
    uint32_t count = 0;
#pragma unroll
    for (int w = 0; w < WARPS; ++w) {
        const uint32_t c = s_whist[w][digit];
        s_whist[w][digit] = (uint16_t)count;
        count += c;
    }
    const uint32_t excl = lookback_exclusive(status, tile, digit, count, err);
    uint32_t total;
    const uint32_t lstart = block_exclusive_sum<uint32_t, THREADS>(count, s_scan, total);
    s_lstart[digit] = lstart;
    s_gbase[digit] = bases[digit] + excl - lstart;

    uint32_t vr[ITEMS];
#pragma unroll
    for (int k = 0; k < ITEMS; ++k) {
        const int idx = wbase + k * 32 + lane;
        vr[k] = (uint32_t)idx < valid ? s_vals[idx] : 0u;
    }
    __syncthreads();

    // ---- reorder by digit inside the tile
#pragma unroll
    for (int k = 0; k < ITEMS; ++k) {
        const int idx = wbase + k * 32 + lane;
        if ((uint32_t)idx < valid) {
            const uint32_t d = (uint32_t)((kr[k] >> shift) & mask);
            const uint32_t p = s_lstart[d] + s_whist[warp][d] + rk[k];
            s_keys[p] = kr[k];
            s_vals[p] = vr[k];
        }
    }
    __syncthreads();

    // ---- write digit runs to their global positions
    for (uint32_t i = tid; i < valid; i += THREADS) {
        const uint64_t key = s_keys[i];
        const uint32_t d = (uint32_t)((key >> shift) & mask);
        const uint32_t o = s_gbase[d] + i;
        if ((uint64_t)o < n) {
            kout[o] = key;
            vout[o] = s_vals[i];
        } else {
            atomicOr(err, GSAIS_ERR_BOUNDS);
        }
    }
}

}  // namespace

size_t radix_status_words(uint64_t n)
{
    const uint64_t tiles = (n + kRadixTile - 1) / kRadixTile;
    return (size_t)(tiles ? tiles : 1) * 256;
}

cudaError_t radix_sort_pairs(uint64_t *keys[2], uint32_t *vals[2], uint64_t n, int end_bit, RadixScratch &rs,
                             uint32_t *d_err, cudaStream_t st, int *which, int *passes_run)
{
    *which = 0;
    if (passes_run) *passes_run = 0;
    if (n <= 1 || end_bit <= 0) return cudaSuccess;
    const int passes = (end_bit + 7) / 8;
    cudaError_t e;
    if ((e = cudaMemsetAsync(rs.hist, 0, (size_t)passes * 256 * sizeof(uint32_t), st)) != cudaSuccess) return e;

    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    uint64_t want = (n + 255) / 256;
    int grid = (int)(want < (uint64_t)sms * 8 ? want : (uint64_t)sms * 8);
    if (grid < 1) grid = 1;
    cudaEvent_t ev = rs.prof ? rs.prof->begin(st) : nullptr;
    GSAIS_COUNTED((k_upsweep<<<grid, 256, 0, st>>>(keys[0], n, passes, end_bit, rs.hist)));
    if (ev) rs.prof->end(KK_UPSWEEP, ev, st, n * sizeof(uint64_t));
    GSAIS_COUNTED((k_bucket_bases<<<passes, 256, 0, st>>>(rs.hist, rs.bases)));
    if ((e = cudaMemcpyAsync(rs.h_hist, rs.hist, (size_t)passes * 256 * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                             st)) != cudaSuccess)
        return e;
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;

    constexpr size_t smem = (size_t)kRadixTile * (sizeof(uint64_t) + sizeof(uint32_t));
    static bool attr_set = false;
    if (!attr_set) {
        e = cudaFuncSetAttribute(k_onesweep<kRadixThreads, kRadixItems>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem);
        if (e != cudaSuccess) return e;
        attr_set = true;
    }

    const uint64_t tiles = (n + kRadixTile - 1) / kRadixTile;
    int cur = 0, ran = 0;
    for (int p = 0; p < passes; ++p) {
        bool trivial = false;
        for (int d = 0; d < 256; ++d)
            if (rs.h_hist[p * 256 + d] == n) { trivial = true; break; }
        if (trivial) continue;
        if ((e = cudaMemsetAsync(rs.status, 0, (size_t)tiles * 256 * sizeof(uint64_t), st)) != cudaSuccess) return e;
        if ((e = cudaMemsetAsync(rs.counters + p, 0, sizeof(uint32_t), st)) != cudaSuccess) return e;
        const int bits = end_bit - 8 * p < 8 ? end_bit - 8 * p : 8;
        const uint32_t mask = (1u << bits) - 1u;
        cudaEvent_t ev1 = rs.prof ? rs.prof->begin(st) : nullptr;
        GSAIS_COUNTED((k_onesweep<kRadixThreads, kRadixItems><<<(unsigned)tiles, kRadixThreads, smem, st>>>(
            keys[cur], vals[cur], keys[cur ^ 1], vals[cur ^ 1], n, 8 * p, mask, rs.bases + p * 256, rs.status,
            rs.counters + p, d_err)));
        // algorithmic bytes: every (key, value) pair read once and written once
        if (ev1) rs.prof->end(KK_ONESWEEP, ev1, st, 2 * n * (sizeof(uint64_t) + sizeof(uint32_t)));
        cur ^= 1;
        ++ran;
    }
    *which = cur;
    if (passes_run) *passes_run = ran;
    return cudaGetLastError();
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
