// suffix_sort.cu -- GPU prefix doubling for suffix arrays (sm_103a).
//
// Replaces libsais's SA-IS pipeline (src/libsais.c:6879-6923 libsais_main_8u:
// LMS gathering, induced sorting and the recursion of :6668
// libsais_main_32s_recursion) with prefix doubling whose output is the same
// suffix array:
//
//   seed   Every symbol present is mapped to a dense code (ceil(log2 sigma)
//          bits), and K = floor(64 / bits) codes of T[i..i+K) are packed into
//          one 64-bit key (positions past the end pack as 0).  A stable radix
//          sort of the keys gives the K-prefix order.  Texts shorter than K
//          at the end of T ("tails") would tie with longer suffixes whose
//          next symbols are the smallest code; they are emitted in reverse
//          text order so the stable sort places the shorter suffix first,
//          and a suffix of length < K is always its own group.  For the
//          generalized suffix array the key stops after the first 0 and a
//          suffix containing a separator in its window is its own group,
//          ordered by position (the GSA tie rule of src/libsais.c:3022,
//          :5472).
//   round  rank[i] = 1 + SA position of the start of i's group (rank[n] = 0
//          is the end-of-text sentinel).  Only suffixes in groups of size >= 2
//          are "active".  Each round sorts the active suffixes by
//          (dense group id, rank[i + h]), splits groups where the key
//          changes, writes final SA entries for new singletons, updates ranks
//          and compacts the singletons out; h doubles each round.
//
// Every kernel is memory-bound integer work; the per-element algorithmic
// traffic is given beside each kernel.
#include <cstring>

#include "device_util.cuh"
#include "engine.h"
#include "suffix_sort.cuh"

namespace gsais {

namespace {

constexpr int kAssignThreads = 256;
constexpr int kAssignWarps = kAssignThreads / 32;
constexpr int kAssignPerLane = 8;
constexpr int kAssignTile = kAssignThreads * kAssignPerLane;   // 2048
constexpr int kSeedTile = 2048;

inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// ------------------------------------------------------------- histogram
// Bytes: n (T read).  The text may start at any byte; the unaligned head
// and the ragged tail are counted by block 0.
__global__ void __launch_bounds__(256) k_hist_u8(const uint8_t *__restrict__ T, uint64_t n, uint32_t *__restrict__ hist)
{
    __shared__ uint32_t sh[256];
    sh[threadIdx.x] = 0;
    __syncthreads();
    uint64_t head = (4 - ((uintptr_t)T & 3)) & 3;
    if (head > n) head = n;
    const uint64_t words = (n - head) / 4;
    const uint64_t words_round = (words + 31) & ~31ull;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint32_t *W = reinterpret_cast<const uint32_t *>(T + head);
    for (uint64_t w = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; w < words_round; w += stride) {
        const bool ok = w < words;
        const uint32_t v = ok ? W[w] : 0u;
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const uint32_t d = ok ? ((v >> (8 * b)) & 255u) : 256u;
            const uint32_t peers = __match_any_sync(GSAIS_FULL_MASK, d);
            if (ok && (peers & lanemask_lt()) == 0) atomicAdd(&sh[d], (uint32_t)__popc(peers));
        }
    }
    if (blockIdx.x == 0) {
        const uint64_t tail0 = head + words * 4;
        if (threadIdx.x < head) atomicAdd(&sh[T[threadIdx.x]], 1u);
        if (tail0 + threadIdx.x < n && threadIdx.x < 4) atomicAdd(&sh[T[tail0 + threadIdx.x]], 1u);
    }
    __syncthreads();
    if (sh[threadIdx.x]) atomicAdd(&hist[threadIdx.x], sh[threadIdx.x]);
}

// Bytes: 2n (T read).
__global__ void __launch_bounds__(256) k_hist_u16(const uint16_t *__restrict__ T, uint64_t n, uint32_t *__restrict__ hist)
{
    const uint64_t n_round = (n + 31) & ~31ull;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_round; i += stride) {
        const bool ok = i < n;
        const uint32_t d = ok ? (uint32_t)T[i] : 65536u;
        const uint32_t peers = __match_any_sync(GSAIS_FULL_MASK, d);
        if (ok && (peers & lanemask_lt()) == 0) atomicAdd(&hist[d], (uint32_t)__popc(peers));
    }
}

// ------------------------------------------------------------------ seed
// Bytes per suffix: T 1-2 (staged), key 8 + value 4 written.
template <typename Sym>
__global__ void __launch_bounds__(256) k_seed(const Sym *__restrict__ T, uint64_t n, const uint16_t *__restrict__ codes,
                                              int bits, int K, int gsa, uint64_t *__restrict__ keys,
                                              uint32_t *__restrict__ vals)
{
    __shared__ uint16_t sc[kSeedTile + 64];
    const uint64_t base = (uint64_t)blockIdx.x * kSeedTile;
    for (int q = threadIdx.x; q < kSeedTile + K - 1; q += blockDim.x) {
        const uint64_t p = base + q;
        sc[q] = p < n ? codes[T[p]] : (uint16_t)0;
    }
    __syncthreads();
    for (int r = threadIdx.x; r < kSeedTile; r += blockDim.x) {
        const uint64_t i = base + r;
        if (i >= n) break;
        uint64_t key = 0;
        bool term = false;
        for (int q = 0; q < K; ++q) {
            const uint32_t c = term ? 0u : (uint32_t)sc[r + q];
            key = (key << bits) | c;
            if (gsa && c == 0) term = true;
        }
        const uint64_t j = gsa ? i : n - 1 - i;
        keys[j] = key;
        vals[j] = (uint32_t)i;
    }
}

// ------------------------------------------------------------ round keys
// Bytes per active suffix: index 4 + group 4 read, rank gather 4, key 8 written.
__global__ void __launch_bounds__(256) k_round_keys(const uint32_t *__restrict__ act_i,
                                                    const uint32_t *__restrict__ act_gid,
                                                    const uint32_t *__restrict__ rank, uint64_t h, uint64_t N,
                                                    uint64_t n, int b2, uint64_t *__restrict__ keys,
                                                    uint32_t *__restrict__ err)
{
    const uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= N) return;
    const uint64_t i = act_i[j];
    // an active suffix has length >= h, so i + h <= n (rank[n] is the sentinel)
    uint32_t r2 = 0;
    if (i + h <= n) r2 = rank[i + h];
    else atomicOr(err, GSAIS_ERR_BOUNDS);
    keys[j] = ((uint64_t)act_gid[j] << b2) | (uint64_t)r2;
}

// --------------------------------------------------- head / assign tiles
enum { MODE_INIT_PLAIN = 0, MODE_INIT_GSA = 1, MODE_ROUND = 2 };

struct TileArgs {
    const uint64_t *keys;
    const uint32_t *vals;
    const uint32_t *pos;     // nullptr: identity (the seed round)
    uint64_t N;              // entries in this round
    uint64_t n;              // text length
    uint32_t K;              // seed symbols per key
    uint64_t zlo, zhi;       // zero-field masks of the packed seed codes
};

__device__ __forceinline__ bool has_zero_field(uint64_t x, uint64_t lo, uint64_t hi)
{
    return ((x - lo) & ~x & hi) != 0;
}

// Stage keys/vals[base-1 .. base+valid] into shared memory (one halo entry
// on each side) and return the number of valid entries.
__device__ __forceinline__ uint32_t stage_tile(const TileArgs &a, uint64_t base, uint64_t *s_keys, uint32_t *s_vals,
                                               bool need_vals)
{
    const uint32_t valid = (uint32_t)((a.N - base) < (uint64_t)kAssignTile ? (a.N - base) : (uint64_t)kAssignTile);
    for (int x = threadIdx.x; x < (int)valid + 2; x += blockDim.x) {
        const int64_t j = (int64_t)base + x - 1;
        const bool in = j >= 0 && (uint64_t)j < a.N;
        s_keys[x] = in ? a.keys[j] : 0ull;
        if (need_vals) s_vals[x] = in ? a.vals[j] : 0u;
    }
    __syncthreads();
    return valid;
}

// Head test for global entry j = base + l - 1 (l indexes the staged arrays).
template <int MODE>
__device__ __forceinline__ bool head_at(const TileArgs &a, uint64_t base, int l, const uint64_t *s_keys,
                                        const uint32_t *s_vals)
{
    const uint64_t j = base + (uint64_t)l - 1;
    if (j == 0 || j >= a.N) return true;
    const uint64_t k = s_keys[l], kp = s_keys[l - 1];
    if (k != kp) return true;
    if (MODE == MODE_INIT_PLAIN) {
        const uint64_t v = s_vals[l], vp = s_vals[l - 1];
        const uint64_t lc = a.n - v < a.K ? a.n - v : a.K;
        const uint64_t lcp = a.n - vp < a.K ? a.n - vp : a.K;
        return lc != lcp;
    } else if (MODE == MODE_INIT_GSA) {
        return has_zero_field(k, a.zlo, a.zhi);   // k == kp here
    }
    return false;
}

struct ElemFlags {
    uint32_t hv;    // 1 + SA position if the entry starts a group, else 0
    uint32_t kept;  // 1 if the entry stays active
    uint32_t kh;    // 1 if the entry starts a group that stays active
    bool single;
};

template <int MODE>
__device__ __forceinline__ ElemFlags elem_flags(const TileArgs &a, uint64_t base, int x, const uint64_t *s_keys,
                                                const uint32_t *s_vals, uint32_t pos)
{
    ElemFlags f;
    const bool head = head_at<MODE>(a, base, x + 1, s_keys, s_vals);
    const bool last = head_at<MODE>(a, base, x + 2, s_keys, s_vals);
    f.single = head && last;
    f.hv = head ? pos + 1 : 0u;
    f.kept = f.single ? 0u : 1u;
    f.kh = (head && !f.single) ? 1u : 0u;
    return f;
}

// Per-tile reduction: max group-start value, kept entries, kept groups.
// Bytes per entry: key 8 (+ value 4 and pos 4 when used).
template <int MODE>
__global__ void __launch_bounds__(kAssignThreads) k_tile_summary(TileArgs a, uint32_t *__restrict__ info)
{
    __shared__ uint64_t s_keys[kAssignTile + 2];
    __shared__ uint32_t s_vals[kAssignTile + 2];
    __shared__ uint32_t s_red[3][kAssignWarps];
    const uint64_t base = (uint64_t)blockIdx.x * kAssignTile;
    const uint32_t valid = stage_tile(a, base, s_keys, s_vals, MODE == MODE_INIT_PLAIN);
    uint32_t mx = 0, kept = 0, kh = 0;
    for (int x = threadIdx.x; x < (int)valid; x += blockDim.x) {
        const uint64_t j = base + x;
        const uint32_t pos = a.pos ? a.pos[j] : (uint32_t)j;
        const ElemFlags f = elem_flags<MODE>(a, base, x, s_keys, s_vals, pos);
        mx = f.hv > mx ? f.hv : mx;
        kept += f.kept;
        kh += f.kh;
    }
    for (int o = 16; o > 0; o >>= 1) {
        const uint32_t m2 = __shfl_down_sync(GSAIS_FULL_MASK, mx, o);
        mx = m2 > mx ? m2 : mx;
        kept += __shfl_down_sync(GSAIS_FULL_MASK, kept, o);
        kh += __shfl_down_sync(GSAIS_FULL_MASK, kh, o);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) { s_red[0][warp] = mx; s_red[1][warp] = kept; s_red[2][warp] = kh; }
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t M = 0, A = 0, B = 0;
        for (int w = 0; w < kAssignWarps; ++w) {
            M = s_red[0][w] > M ? s_red[0][w] : M;
            A += s_red[1][w];
            B += s_red[2][w];
        }
        info[3 * blockIdx.x + 0] = M;
        info[3 * blockIdx.x + 1] = A;
        info[3 * blockIdx.x + 2] = B;
    }
}

// Exclusive scan of the tile summaries (single CTA): carry[t] = (max, sum, sum)
// over tiles < t; totals[0] = kept entries, totals[1] = kept groups.
__global__ void __launch_bounds__(1024) k_tile_scan(const uint32_t *__restrict__ info, uint32_t *__restrict__ carry,
                                                    uint64_t tiles, uint32_t *__restrict__ totals)
{
    __shared__ uint32_t wb[3][33];
    uint32_t cm = 0, ck = 0, ch = 0;
    for (uint64_t c0 = 0; c0 < tiles; c0 += 1024) {
        const uint64_t t = c0 + threadIdx.x;
        const bool ok = t < tiles;
        const uint32_t m = ok ? info[3 * t + 0] : 0u;
        const uint32_t k = ok ? info[3 * t + 1] : 0u;
        const uint32_t h = ok ? info[3 * t + 2] : 0u;
        uint32_t tk, th;
        const uint32_t em = block_exclusive_max<uint32_t, 1024>(m, wb[0]);
        const uint32_t ek = block_exclusive_sum<uint32_t, 1024>(k, wb[1], tk);
        const uint32_t eh = block_exclusive_sum<uint32_t, 1024>(h, wb[2], th);
        if (ok) {
            carry[3 * t + 0] = em > cm ? em : cm;
            carry[3 * t + 1] = ck + ek;
            carry[3 * t + 2] = ch + eh;
        }
        // block max of this chunk: the last thread's inclusive value
        __shared__ uint32_t s_lastmax;
        if (threadIdx.x == 1023) s_lastmax = em > m ? em : m;
        __syncthreads();
        cm = s_lastmax > cm ? s_lastmax : cm;
        ck += tk;
        ch += th;
        __syncthreads();
    }
    if (threadIdx.x == 0) { totals[0] = ck; totals[1] = ch; }
}

// Assign new ranks, emit singletons, compact the survivors.
// Bytes per entry: key 8 + value 4 + pos 4 read; rank scatter 4; SA 4 for
// singletons or 12 (index, pos, group) for survivors.
template <int MODE>
__global__ void __launch_bounds__(kAssignThreads)
    k_assign(TileArgs a, const uint32_t *__restrict__ carry, uint32_t *__restrict__ rank, uint32_t *__restrict__ sa,
             uint32_t *__restrict__ out_i, uint32_t *__restrict__ out_pos, uint32_t *__restrict__ out_gid)
{
    __shared__ uint64_t s_keys[kAssignTile + 2];
    __shared__ uint32_t s_vals[kAssignTile + 2];
    __shared__ uint32_t s_w[3][kAssignWarps];
    const uint64_t base = (uint64_t)blockIdx.x * kAssignTile;
    const uint32_t valid = stage_tile(a, base, s_keys, s_vals, true);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;

    uint32_t hv_inc[kAssignPerLane], k_exc[kAssignPerLane], h_inc[kAssignPerLane], posv[kAssignPerLane];
    bool single[kAssignPerLane];
    uint32_t run_m = 0, run_k = 0, run_h = 0;
#pragma unroll
    for (int q = 0; q < kAssignPerLane; ++q) {
        const int x = warp * 256 + q * 32 + lane;
        const bool ok = x < (int)valid;
        ElemFlags f = {0u, 0u, 0u, false};
        uint32_t pos = 0;
        if (ok) {
            const uint64_t j = base + x;
            pos = a.pos ? a.pos[j] : (uint32_t)j;
            f = elem_flags<MODE>(a, base, x, s_keys, s_vals, pos);
        }
        posv[q] = pos;
        single[q] = f.single;
        uint32_t m = warp_inclusive_max(f.hv);
        m = m > run_m ? m : run_m;
        const uint32_t ki = warp_inclusive_sum(f.kept);
        const uint32_t hi = warp_inclusive_sum(f.kh);
        hv_inc[q] = m;
        k_exc[q] = run_k + ki - f.kept;
        h_inc[q] = run_h + hi;
        run_m = __shfl_sync(GSAIS_FULL_MASK, m, 31);
        run_k += __shfl_sync(GSAIS_FULL_MASK, ki, 31);
        run_h += __shfl_sync(GSAIS_FULL_MASK, hi, 31);
    }
    if (lane == 0) { s_w[0][warp] = run_m; s_w[1][warp] = run_k; s_w[2][warp] = run_h; }
    __syncthreads();
    uint32_t wm = carry[3 * blockIdx.x + 0], wk = carry[3 * blockIdx.x + 1], wh = carry[3 * blockIdx.x + 2];
    for (int w = 0; w < warp; ++w) {
        wm = s_w[0][w] > wm ? s_w[0][w] : wm;
        wk += s_w[1][w];
        wh += s_w[2][w];
    }
#pragma unroll
    for (int q = 0; q < kAssignPerLane; ++q) {
        const int x = warp * 256 + q * 32 + lane;
        if (x >= (int)valid) continue;
        const uint32_t v = s_vals[x + 1];
        const uint32_t r = hv_inc[q] > wm ? hv_inc[q] : wm;
        rank[v] = r;
        if (single[q]) {
            sa[posv[q]] = v;
        } else {
            const uint32_t c = wk + k_exc[q];
            out_i[c] = v;
            out_pos[c] = posv[q];
            out_gid[c] = wh + h_inc[q] - 1;
        }
    }
}

// GSA validity: T[n-1] == 0, T[0] != 0, no two adjacent zeros.
template <typename Sym>
__global__ void k_gsa_check(const Sym *__restrict__ T, uint64_t n, uint32_t *__restrict__ flag)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const bool bad = (i == n - 1 && T[i] != 0) || (i == 0 && n > 1 && T[0] == 0) ||
                         (i + 1 < n && T[i] == 0 && T[i + 1] == 0);
        if (bad) atomicOr(flag, 1u);
    }
}

}  // namespace

size_t sort_workspace_bytes(uint64_t n, int symbytes)
{
    (void)symbytes;
    const size_t A = 256;
    const uint64_t tiles = (n + kAssignTile - 1) / kAssignTile + 1;
    size_t s = 0;
    s += align_up((n + 1) * 4, A);                 // rank
    s += align_up(n * 4, A);                       // sa
    s += 2 * align_up(n * 8, A);                   // keys
    s += 2 * align_up(n * 4, A);                   // vals
    s += 2 * align_up(n * 4, A);                   // pos
    s += 2 * align_up(n * 4, A);                   // gid
    s += 2 * align_up(tiles * 12, A);              // tile info + carry
    s += align_up(16 * 4, A);                      // totals
    s += align_up(65536 * 4, A);                   // hist
    s += align_up(65536 * 2, A);                   // codes
    s += 2 * align_up(8 * 256 * 4, A);             // radix hist + bases
    s += align_up(8 * 4, A);                       // radix counters
    s += align_up(radix_status_words(n) * 8, A);   // look-back words
    return s;
}

void sort_workspace_carve(SortWorkspace &ws, void *base, uint64_t n, int symbytes, uint32_t *h_small,
                          uint32_t *h_hist)
{
    (void)symbytes;
    const size_t A = 256;
    const uint64_t tiles = (n + kAssignTile - 1) / kAssignTile + 1;
    char *p = static_cast<char *>(base);
    auto take = [&](size_t bytes) { char *r = p; p += align_up(bytes, A); return r; };
    ws.rank = reinterpret_cast<uint32_t *>(take((n + 1) * 4));
    ws.sa = reinterpret_cast<uint32_t *>(take(n * 4));
    for (int i = 0; i < 2; ++i) ws.keys[i] = reinterpret_cast<uint64_t *>(take(n * 8));
    for (int i = 0; i < 2; ++i) ws.vals[i] = reinterpret_cast<uint32_t *>(take(n * 4));
    for (int i = 0; i < 2; ++i) ws.pos[i] = reinterpret_cast<uint32_t *>(take(n * 4));
    for (int i = 0; i < 2; ++i) ws.gid[i] = reinterpret_cast<uint32_t *>(take(n * 4));
    ws.tile_info = reinterpret_cast<uint32_t *>(take(tiles * 12));
    ws.tile_carry = reinterpret_cast<uint32_t *>(take(tiles * 12));
    ws.totals = reinterpret_cast<uint32_t *>(take(16 * 4));
    ws.hist = reinterpret_cast<uint32_t *>(take(65536 * 4));
    ws.codes = reinterpret_cast<uint16_t *>(take(65536 * 2));
    ws.radix.hist = reinterpret_cast<uint32_t *>(take(8 * 256 * 4));
    ws.radix.bases = reinterpret_cast<uint32_t *>(take(8 * 256 * 4));
    ws.radix.counters = reinterpret_cast<uint32_t *>(take(8 * 4));
    ws.radix.status_words = radix_status_words(n);
    ws.radix.status = reinterpret_cast<uint64_t *>(take(ws.radix.status_words * 8));
    ws.radix.h_hist = h_hist;
    ws.h_small = h_small;
}

static int grid_for(uint64_t items, int per_block)
{
    const uint64_t g = (items + per_block - 1) / per_block;
    return (int)(g ? g : 1);
}

static int stream_grid(uint64_t items, int threads)
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const uint64_t want = (items + threads - 1) / threads;
    const uint64_t cap = (uint64_t)sms * 8;
    return (int)(want < 1 ? 1 : (want < cap ? want : cap));
}

template <int MODE>
static cudaError_t run_assign(const TileArgs &a, SortWorkspace &ws, uint32_t *out_i, uint32_t *out_pos,
                              uint32_t *out_gid, cudaStream_t st, uint32_t *kept, uint32_t *groups)
{
    const uint64_t tiles = (a.N + kAssignTile - 1) / kAssignTile;
    KernelProfiler *prof = ws.radix.prof;
    cudaEvent_t ev = prof ? prof->begin(st) : nullptr;
    GSAIS_COUNTED((k_tile_summary<MODE><<<(unsigned)tiles, kAssignThreads, 0, st>>>(a, ws.tile_info)));
    if (ev) prof->end(KK_SUMMARY, ev, st, a.N * (MODE == MODE_ROUND ? 12 : 16));
    GSAIS_COUNTED((k_tile_scan<<<1, 1024, 0, st>>>(ws.tile_info, ws.tile_carry, tiles, ws.totals)));
    ev = prof ? prof->begin(st) : nullptr;
    GSAIS_COUNTED((k_assign<MODE><<<(unsigned)tiles, kAssignThreads, 0, st>>>(a, ws.tile_carry, ws.rank, ws.sa, out_i,
                                                                                out_pos, out_gid)));
    // algorithmic bytes: key 8 + value 4 + slot 4 read, rank 4 scattered, and
    // 4 (SA) or 12 (survivor lists) written -- counted as 28 per entry
    if (ev) prof->end(KK_ASSIGN, ev, st, a.N * 28);
    cudaError_t e = cudaMemcpyAsync(ws.h_small, ws.totals, 2 * sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess) return e;
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
    *kept = ws.h_small[0];
    *groups = ws.h_small[1];
    return cudaGetLastError();
}

cudaError_t suffix_sort(const void *d_T, int symbytes, uint64_t n, bool gsa, SortWorkspace &ws,
                        const SortOptions &opt, uint32_t *d_err, cudaStream_t st, SortStats *stats)
{
    cudaError_t e;
    SortStats local;
    SortStats &S = stats ? *stats : local;
    S = SortStats();
    if (n == 0) return cudaSuccess;

    // ---- symbol histogram -> dense codes
    const int nsym = symbytes == 1 ? 256 : 65536;
    uint32_t *h_hist = ws.h_small + 16;
    uint16_t *h_codes = reinterpret_cast<uint16_t *>(ws.h_small + 16 + 65536);
    if ((e = symbol_histogram(d_T, symbytes, n, ws.hist, h_hist, st)) != cudaSuccess) return e;
    uint32_t sigma = 0;
    for (int c = 0; c < nsym; ++c) {
        h_codes[c] = (uint16_t)sigma;
        if (h_hist[c]) ++sigma;
    }
    int bits = gsais_bits_for(sigma > 1 ? sigma - 1 : 1);
    int K = opt.seed_key_bits / bits;
    if (K < 1) K = 1;
    if (K > 64) K = 64;
    S.seed_symbols = K;
    S.seed_bits = bits;
    if ((e = cudaMemcpyAsync(ws.codes, h_codes, (size_t)nsym * 2, cudaMemcpyHostToDevice, st)) != cudaSuccess)
        return e;
    if ((e = cudaMemsetAsync(ws.rank + n, 0, sizeof(uint32_t), st)) != cudaSuccess) return e;

    // ---- seed keys and the K-prefix sort
    const unsigned seed_grid = (unsigned)grid_for(n, kSeedTile);
    cudaEvent_t ev_seed = ws.radix.prof ? ws.radix.prof->begin(st) : nullptr;
    if (symbytes == 1)
        GSAIS_COUNTED((k_seed<uint8_t><<<seed_grid, 256, 0, st>>>(static_cast<const uint8_t *>(d_T), n, ws.codes, bits, K, gsa ? 1 : 0,
                                                   ws.keys[0], ws.vals[0])));
    else
        GSAIS_COUNTED((k_seed<uint16_t><<<seed_grid, 256, 0, st>>>(static_cast<const uint16_t *>(d_T), n, ws.codes, bits, K,
                                                    gsa ? 1 : 0, ws.keys[0], ws.vals[0])));
    if (ev_seed) ws.radix.prof->end(KK_SEED, ev_seed, st, n * (symbytes + 12));
    int w = 0, ran = 0;
    {
        uint64_t *kk[2] = {ws.keys[0], ws.keys[1]};
        uint32_t *vv[2] = {ws.vals[0], ws.vals[1]};
        if ((e = radix_sort_pairs(kk, vv, n, K * bits, ws.radix, d_err, st, &w, &ran)) != cudaSuccess) return e;
        S.radix_passes += ran;
    }

    TileArgs a;
    a.keys = ws.keys[w];
    a.vals = ws.vals[w];
    a.pos = nullptr;
    a.N = n;
    a.n = n;
    a.K = (uint32_t)K;
    a.zlo = 0;
    for (int q = 0; q < K; ++q) a.zlo |= 1ull << (q * bits);
    a.zhi = a.zlo << (bits - 1);
    uint32_t kept = 0, groups = 0;
    int av = w ^ 1, pg = 0;
    if (gsa)
        e = run_assign<MODE_INIT_GSA>(a, ws, ws.vals[av], ws.pos[pg], ws.gid[pg], st, &kept, &groups);
    else
        e = run_assign<MODE_INIT_PLAIN>(a, ws, ws.vals[av], ws.pos[pg], ws.gid[pg], st, &kept, &groups);
    if (e != cudaSuccess) return e;

    // ---- doubling rounds over the active suffixes
    const int b2 = gsais_bits_for(n);
    uint64_t h = (uint64_t)K;
    while (kept > 0) {
        if (++S.rounds > 64) {
            uint32_t flag = GSAIS_ERR_ROUNDS;
            cudaMemcpyAsync(d_err, &flag, 4, cudaMemcpyHostToDevice, st);
            cudaStreamSynchronize(st);
            return cudaErrorUnknown;
        }
        S.active_total += kept;
        const uint64_t N = kept;
        const int gb = gsais_bits_for(groups > 1 ? groups - 1 : 0);
        cudaEvent_t ev_rk = ws.radix.prof ? ws.radix.prof->begin(st) : nullptr;
        GSAIS_COUNTED((k_round_keys<<<grid_for(N, 256), 256, 0, st>>>(ws.vals[av], ws.gid[pg], ws.rank, h, N, n, b2, ws.keys[0],
                                                        d_err)));
        if (ev_rk) ws.radix.prof->end(KK_ROUND_KEYS, ev_rk, st, N * 24);
        uint64_t *kk[2] = {ws.keys[0], ws.keys[1]};
        uint32_t *vv[2] = {ws.vals[av], ws.vals[av ^ 1]};
        int which = 0;
        if ((e = radix_sort_pairs(kk, vv, N, b2 + gb, ws.radix, d_err, st, &which, &ran)) != cudaSuccess) return e;
        S.radix_passes += ran;
        const int sv = which == 0 ? av : (av ^ 1);   // vals buffer holding the sorted values
        TileArgs r;
        r.keys = kk[which];
        r.vals = ws.vals[sv];
        r.pos = ws.pos[pg];
        r.N = N;
        r.n = n;
        r.K = (uint32_t)K;
        r.zlo = r.zhi = 0;
        if ((e = run_assign<MODE_ROUND>(r, ws, ws.vals[sv ^ 1], ws.pos[pg ^ 1], ws.gid[pg ^ 1], st, &kept, &groups)) !=
            cudaSuccess)
            return e;
        av = sv ^ 1;
        pg ^= 1;
        h *= 2;
    }
    uint32_t herr = 0;
    if ((e = cudaMemcpyAsync(ws.h_small, d_err, 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
    herr = ws.h_small[0];
    if (ws.radix.prof) ws.radix.prof->flush();
    return herr ? cudaErrorUnknown : cudaSuccess;
}

cudaError_t symbol_histogram(const void *d_T, int symbytes, uint64_t n, uint32_t *d_hist, uint32_t *h_hist,
                             cudaStream_t st)
{
    cudaError_t e;
    const int nsym = symbytes == 1 ? 256 : 65536;
    if ((e = cudaMemsetAsync(d_hist, 0, (size_t)nsym * 4, st)) != cudaSuccess) return e;
    if (n > 0) {
        if (symbytes == 1)
            GSAIS_COUNTED((k_hist_u8<<<stream_grid(n / 4 + 1, 256), 256, 0, st>>>(static_cast<const uint8_t *>(d_T), n, d_hist)));
        else
            GSAIS_COUNTED((k_hist_u16<<<stream_grid(n, 256), 256, 0, st>>>(static_cast<const uint16_t *>(d_T), n, d_hist)));
    }
    if ((e = cudaMemcpyAsync(h_hist, d_hist, (size_t)nsym * 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
    return cudaGetLastError();
}

cudaError_t gsa_validate(const void *d_T, int symbytes, uint64_t n, uint32_t *d_flag, uint32_t *h_flag,
                         cudaStream_t st, bool *valid)
{
    cudaError_t e;
    if ((e = cudaMemsetAsync(d_flag, 0, 4, st)) != cudaSuccess) return e;
    if (symbytes == 1)
        GSAIS_COUNTED((k_gsa_check<uint8_t><<<stream_grid(n, 256), 256, 0, st>>>(static_cast<const uint8_t *>(d_T), n, d_flag)));
    else
        GSAIS_COUNTED((k_gsa_check<uint16_t><<<stream_grid(n, 256), 256, 0, st>>>(static_cast<const uint16_t *>(d_T), n, d_flag)));
    if ((e = cudaMemcpyAsync(h_flag, d_flag, 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
    *valid = (*h_flag == 0);
    return cudaGetLastError();
}

}  // namespace gsais
