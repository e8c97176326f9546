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
#include "outputs.cuh"
#include "radix_hist.cuh"
#include "suffix_sort.cuh"

#include <type_traits>

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

// Seed keys for 2- and 4-bit codes with 32-bit keys (plain texts): the tile's
// codes are packed most-significant-first into shared words, so the key of
// position x (the K = 32 / B codes from x) is one funnel shift of two words.
// Also writes the packed text (least-significant-first, the layout the BWT
// gather and the pair comparison read) and digit 0's histogram.
// The suffix index is not written: key slot j holds suffix n - 1 - j, which
// the first radix pass computes instead of reading a value array.
// Bytes per suffix: T s read, key 4 written (+ B/8 packed).
template <typename Sym, int B>
__global__ void __launch_bounds__(256) k_seed_packed(const Sym *__restrict__ T, uint64_t n,
                                                     const uint16_t *__restrict__ codes, uint32_t *__restrict__ keys,
                                                     uint32_t *__restrict__ vals, int end_bit,
                                                     uint32_t *__restrict__ hist, uint8_t *__restrict__ packed)
{
    static_assert(B == 2 || B == 4, "2- or 4-bit codes");
    constexpr int PER = kSeedTile / 256;   // 8 codes per thread
    constexpr int CPW = 32 / B;            // codes per word
    constexpr int WORDS = kSeedTile / CPW; // words of the tile, plus one halo word
    __shared__ uint32_t w[WORDS + 1];
    __shared__ uint32_t sh[1][256];
    radix_hist_zero(sh, 1);
    const uint64_t tiles = (n + kSeedTile - 1) / kSeedTile;
    const int tid = threadIdx.x, lane = tid & 31;
    for (uint64_t t = blockIdx.x; t < tiles; t += gridDim.x) {
        const uint64_t base = t * kSeedTile;
        // codes of positions base + PER * tid .. + PER (past the end: 0)
        uint32_t c[PER];
#pragma unroll
        for (int r = 0; r < PER; ++r) {
            const uint64_t p = base + (uint64_t)tid * PER + r;
            c[r] = p < n ? codes[T[p]] : 0u;
        }
        // packed text, least significant first
        uint32_t lsb = 0, msb = 0;
#pragma unroll
        for (int r = 0; r < PER; ++r) {
            lsb |= c[r] << (B * r);
            msb = (msb << B) | c[r];
        }
        if (B == 2) reinterpret_cast<uint16_t *>(packed)[(base / PER) + tid] = (uint16_t)lsb;
        else reinterpret_cast<uint32_t *>(packed)[(base / PER) + tid] = lsb;
        __syncthreads();   // the previous tile's keys are read
        if (B == 4) {
            w[tid] = msb;
        } else {
            const uint32_t lo = __shfl_down_sync(GSAIS_FULL_MASK, msb, 1);
            if ((lane & 1) == 0) w[tid >> 1] = (msb << 16) | lo;
        }
        if (tid == 0) {   // halo word: the CPW codes after the tile
            uint32_t h = 0;
            for (int q = 0; q < CPW; ++q) {
                const uint64_t p = base + kSeedTile + q;
                h = (h << B) | (p < n ? (uint32_t)codes[T[p]] : 0u);
            }
            w[WORDS] = h;
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < PER; ++r) {
            const int x = tid + 256 * r;
            const int i = x / CPW, s = (x % CPW) * B;
            const uint32_t key = __funnelshift_l(w[i + 1], w[i], s);
            const uint64_t p = base + (uint64_t)x;
            const bool ok = p < n;
            if (ok) keys[n - 1 - p] = key;   // reverse text order: shorter suffixes first; the
                                             // value (suffix index p) is implicit in the slot
            radix_hist_add(sh, (uint64_t)key, ok, 1, end_bit);
        }
    }
    __syncthreads();
    radix_hist_flush(sh, 1, hist);
}

// ------------------------------------------------------------------ seed
// Packed K-symbol prefix of every suffix.  Each thread builds the keys of 8
// consecutive positions: the highest one from its K codes, the others by
// sliding the window one symbol left (key(i) = code(T[i]) on top of
// key(i+1) >> bits; a separator zeroes the rest for the GSA).  Keys are
// staged in shared memory and written out coalesced, in reverse text order
// for plain texts (see the tail rule above).
// The same pass accumulates the digit histograms of the keys for the radix
// sort and, for small alphabets (codes of <= 4 bits), writes the text as
// packed codes (pack_bits 2 or 4) for the BWT gather.
// Bytes per suffix: T s read (staged), key sizeof(KeyT) + value 4 written
// (+ pack_bits/8 for the packed text).
template <typename Sym, typename KeyT>
__global__ void __launch_bounds__(256) k_seed(const Sym *__restrict__ T, uint64_t n, const uint16_t *__restrict__ codes,
                                              int bits, int K, int gsa, KeyT *__restrict__ keys,
                                              uint32_t *__restrict__ vals, int passes, int end_bit,
                                              uint32_t *__restrict__ hist, int pack_bits,
                                              uint8_t *__restrict__ packed)
{
    constexpr int PER = kSeedTile / 256;
    // 32-bit symbols (integer alphabets) are their own codes; 8/16-bit
    // symbols go through the dense code table
    constexpr bool RAW = sizeof(Sym) == 4;
    using CodeT = typename std::conditional<RAW, uint32_t, uint16_t>::type;
    __shared__ CodeT sc[kSeedTile + 64];
    __shared__ KeyT sk[kSeedTile];
    __shared__ uint32_t sh[kMaxRadixPasses][256];
    radix_hist_zero(sh, passes);
    const uint64_t tiles = (n + kSeedTile - 1) / kSeedTile;
    const int r0 = threadIdx.x * PER;
    const int top = (K - 1) * bits;
    for (uint64_t t = blockIdx.x; t < tiles; t += gridDim.x) {
        const uint64_t base = t * kSeedTile;
        __syncthreads();   // previous tile's sk/sc reads are done
        for (int q = threadIdx.x; q < kSeedTile + K - 1; q += blockDim.x) {
            const uint64_t p = base + q;
            sc[q] = p < n ? (RAW ? (CodeT)T[p] : (CodeT)codes[T[p]]) : (CodeT)0;
        }
        __syncthreads();
        KeyT key = 0;
        {
            bool term = false;
            for (int q = 0; q < K; ++q) {
                const KeyT c = term ? KeyT(0) : (KeyT)sc[r0 + PER - 1 + q];
                key = (KeyT)((key << bits) | c);
                if (gsa && c == 0) term = true;
            }
        }
        sk[r0 + PER - 1] = key;
#pragma unroll
        for (int r = PER - 2; r >= 0; --r) {
            const KeyT c = (KeyT)sc[r0 + r];
            key = (gsa && c == 0) ? KeyT(0) : (KeyT)((c << top) | (key >> bits));
            sk[r0 + r] = key;
        }
        if (pack_bits == 2) {
            uint32_t w = 0;
#pragma unroll
            for (int r = 0; r < PER; ++r) w |= (uint32_t)(sc[r0 + r] & 3u) << (2 * r);
            reinterpret_cast<uint16_t *>(packed)[(base + r0) / PER] = (uint16_t)w;
        } else if (pack_bits == 4) {
            uint32_t w = 0;
#pragma unroll
            for (int r = 0; r < PER; ++r) w |= (uint32_t)(sc[r0 + r] & 15u) << (4 * r);
            reinterpret_cast<uint32_t *>(packed)[(base + r0) / PER] = w;
        }
        __syncthreads();
        for (int r = threadIdx.x; r < kSeedTile; r += blockDim.x) {
            const uint64_t i = base + r;
            const bool ok = i < n;
            const KeyT k = sk[r];
            if (ok) {
                const uint64_t j = gsa ? i : n - 1 - i;
                keys[j] = k;
                vals[j] = (uint32_t)i;
            }
            radix_hist_add(sh, (uint64_t)k, ok, passes, end_bit);
        }
    }
    __syncthreads();
    radix_hist_flush(sh, passes, hist);
}

// --------------------------------------------------- head / assign tiles
enum { MODE_INIT_PLAIN = 0, MODE_INIT_GSA = 1, MODE_ROUND = 2 };

struct TileArgs {
    const uint64_t *keys;
    const uint32_t *keys32;  // non-null: 32-bit keys (the seed round with short seeds)
    const uint32_t *vals;
    const uint32_t *pos;     // nullptr: identity (the seed round)
    uint32_t *rank_out;      // non-null: new ranks go here by list position (scattered later)
    uint32_t *pairs;         // non-null (seed round, plain texts): groups of exactly two leave
    unsigned long long *pair_count;   //   the list; their first slot is appended here
    uint32_t *slot0;         // non-null (seed round): receives 1 + the slot of suffix 0
    uint64_t N;              // entries in this round
    uint64_t n;              // text length
    uint32_t K;              // seed symbols per key
    uint64_t zlo, zhi;       // zero-field masks of the packed seed codes
};

__device__ __forceinline__ bool has_zero_field(uint64_t x, uint64_t lo, uint64_t hi)
{
    return ((x - lo) & ~x & hi) != 0;
}

// ---- group heads as bits.  Word w of `heads` holds the head flags of list
// entries [32w, 32w + 32); entries past N read as heads.  A head is an entry
// whose key differs from the previous entry's (the seed round also splits
// equal keys of different tail lengths, and for the GSA keys that hold a
// separator; these mirror libsais's implicit sentinel and separator order).
// The per-entry flags of the assign follow from three words with shifts:
//   single     h(j) & h(j+1)
//   pair first h(j) & !h(j+1) & h(j+2)    (seed round, plain texts)
//   pair other !h(j) & h(j-1) & h(j+1)
//   kept       !(single | pair),  kept head = h(j) & kept.
constexpr int kAssignWordsPerTile = kAssignTile / 32;

template <int MODE>
__device__ __forceinline__ uint64_t list_key(const TileArgs &a, uint64_t j)
{
    return a.keys32 ? (uint64_t)a.keys32[j] : a.keys[j];
}

// One warp per word: keys of 32 entries, the previous entry's through a
// shuffle; each warp takes four words per step with all loads issued first.
// (Suffixes shorter than K, whose padded keys may tie with longer ones, get
// their heads from k_tail_heads.)  Bytes per entry: key 4 or 8.
template <int MODE>
__global__ void __launch_bounds__(256) k_heads(TileArgs a, uint32_t *__restrict__ heads)
{
    constexpr int WPS = 4;   // words per warp per step
    const uint64_t words = (a.N + 31) / 32;
    const int lane = threadIdx.x & 31;
    const uint64_t nw = (uint64_t)gridDim.x * (blockDim.x / 32) * WPS;
    for (uint64_t w0 = ((uint64_t)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5)) * WPS; w0 < words; w0 += nw) {
        uint64_t k[WPS], kp0[WPS];
#pragma unroll
        for (int u = 0; u < WPS; ++u) {
            const uint64_t j = (w0 + u) * 32 + lane;
            const bool in = j < a.N;
            k[u] = in ? list_key<MODE>(a, j) : 0ull;
            const bool first = lane == 0 && j > 0 && in;   // lane 0 loads its predecessor
            kp0[u] = first ? list_key<MODE>(a, j - 1) : 0ull;
        }
#pragma unroll
        for (int u = 0; u < WPS; ++u) {
            const uint64_t w = w0 + u;
            const uint64_t j = w * 32 + lane;
            const bool in = j < a.N;
            uint64_t kp = __shfl_up_sync(GSAIS_FULL_MASK, k[u], 1);
            if (lane == 0) kp = kp0[u];
            bool head = !in || j == 0 || k[u] != kp;
            if (!head && MODE == MODE_INIT_GSA) {
                head = has_zero_field(k[u], a.zlo, a.zhi);
            }
            const uint32_t bits = __ballot_sync(GSAIS_FULL_MASK, head);
            if (lane == 0 && w < words) heads[w] = bits;
        }
    }
}

// Seed round of a plain text: a suffix shorter than K (position n - K + 1
// .. n - 1) pads its key with code 0, so the key can tie with a longer
// suffix's.  Such a suffix is its own group (lengths differ) and its entry
// comes first among its key's (the seed list is in reverse text order and
// the sort is stable), shortest first: the head bits of its entry and of the
// entry after it are set.  One thread per short suffix: its key from the
// text, the first entry of that key by binary search over the sorted keys,
// plus the shorter suffixes with the same key.
template <typename Sym>
__global__ void __launch_bounds__(64) k_tail_heads(const Sym *__restrict__ T, uint64_t n,
                                                   const uint16_t *__restrict__ codes, int bits, TileArgs a,
                                                   uint32_t *__restrict__ heads)
{
    __shared__ uint64_t sk[64];
    const int t = threadIdx.x;   // suffix length t + 1
    const int K = (int)a.K;
    const bool act = t < K - 1 && (uint64_t)t < n;
    uint64_t key = 0;
    if (act) {
        const uint64_t p = n - 1 - t;
        for (int q = 0; q < K; ++q) {
            const uint64_t c = p + q < n ? (sizeof(Sym) == 4 ? (uint64_t)T[p + q] : (uint64_t)codes[T[p + q]]) : 0ull;
            key = (key << bits) | c;
        }
    }
    sk[t] = key;
    __syncthreads();
    if (!act) return;
    uint64_t e = 0;
    for (int u = 0; u < t; ++u) e += sk[u] == key;
    uint64_t lo = 0, hi = a.N;
    while (lo < hi) {
        const uint64_t mid = lo + (hi - lo) / 2;
        if (list_key<MODE_INIT_PLAIN>(a, mid) < key) lo = mid + 1;
        else hi = mid;
    }
    e += lo;
    if (e < a.N) atomicOr(&heads[e >> 5], 1u << (e & 31));
    if (e + 1 < a.N) atomicOr(&heads[(e + 1) >> 5], 1u << ((e + 1) & 31));
}

struct TailSource {   // the text of a plain seed round, for k_tail_heads
    const void *T = nullptr;
    int symbytes = 1;
    const uint16_t *codes = nullptr;
    int bits = 0;
};

struct RowFlags {
    uint32_t head, single, pair, first, kept, kh;   // bit l: entry 32 r + l of the row
};

// Flags of the 32 entries of word r from words r - 1, r, r + 1, r + 2 of the
// heads (words outside [0, words) read as all heads).
__device__ __forceinline__ RowFlags row_flags(const uint32_t *__restrict__ heads, uint64_t r, uint64_t words,
                                              bool pairs)
{
    const uint32_t W = r < words ? heads[r] : ~0u;
    const uint32_t Wp = (r > 0 && r - 1 < words) ? heads[r - 1] : ~0u;
    const uint32_t Wn = r + 1 < words ? heads[r + 1] : ~0u;
    const uint32_t N1 = (W >> 1) | (Wn << 31);
    const uint32_t N2 = (W >> 2) | (Wn << 30);
    const uint32_t P1 = (W << 1) | (Wp >> 31);
    RowFlags f;
    f.head = W;
    f.single = W & N1;
    f.first = pairs ? (W & ~N1 & N2) : 0u;
    f.pair = pairs ? (f.first | (~W & P1 & N1)) : 0u;
    f.kept = ~(f.single | f.pair);
    f.kh = W & f.kept;
    return f;
}

// Per-tile reduction over the head bits: (value of the tile's last head, kept
// entries, kept groups, two-member groups taken out).  One warp per tile,
// two words per lane.
template <int MODE>
__global__ void __launch_bounds__(256) k_tile_summary(TileArgs a, const uint32_t *__restrict__ heads,
                                                      uint32_t *__restrict__ info)
{
    const uint64_t tiles = (a.N + kAssignTile - 1) / kAssignTile;
    const uint64_t words = (a.N + 31) / 32;
    const int lane = threadIdx.x & 31;
    const bool pairs = MODE == MODE_INIT_PLAIN && a.pairs;
    const uint64_t t = (uint64_t)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
    if (t >= tiles) return;
    uint32_t kept = 0, kh = 0, np = 0;
    int64_t last = -1;   // list index of the last head
#pragma unroll
    for (int e = 0; e < 2; ++e) {
        const uint64_t r = t * kAssignWordsPerTile + 2 * lane + e;
        if (r >= words) continue;
        const RowFlags f = row_flags(heads, r, words, pairs);
        const uint64_t j0 = r * 32;
        const uint32_t valid = a.N - j0 >= 32 ? ~0u : ((1u << (a.N - j0)) - 1u);
        kept += __popc(f.kept & valid);
        kh += __popc(f.kh & valid);
        np += __popc(f.first & valid);
        if (f.head & valid) last = (int64_t)(j0 + 31 - __clz(f.head & valid));
    }
    for (int o = 16; o > 0; o >>= 1) {
        kept += __shfl_down_sync(GSAIS_FULL_MASK, kept, o);
        kh += __shfl_down_sync(GSAIS_FULL_MASK, kh, o);
        np += __shfl_down_sync(GSAIS_FULL_MASK, np, o);
        const int64_t l2 = __shfl_down_sync(GSAIS_FULL_MASK, last, o);
        if (l2 > last) last = l2;
    }
    if (lane == 0) {
        uint32_t M = 0;
        if (last >= 0) M = 1 + (a.pos ? a.pos[last] : (uint32_t)last);
        info[4 * t + 0] = M;
        info[4 * t + 1] = kept;
        info[4 * t + 2] = kh;
        info[4 * t + 3] = np;
    }
}


// Exclusive scan of the tile summaries (single CTA): carry[t] = (max, sum,
// sum, sum) over tiles < t; totals[0] = kept entries, totals[1] = kept
// groups; *pair_total (nullable) = two-member groups taken out.
// `base` (nullable) = (groups << 32 | entries) already emitted by the
// small-group path of the same round; survivors and groups follow them.
__global__ void __launch_bounds__(1024) k_tile_scan(const uint32_t *__restrict__ info, uint32_t *__restrict__ carry,
                                                    uint64_t tiles, uint32_t *__restrict__ totals,
                                                    const unsigned long long *__restrict__ base,
                                                    unsigned long long *__restrict__ pair_total)
{
    // each thread scans 32 consecutive tiles sequentially; one block scan per
    // 32768 tiles combines the threads
    constexpr int PT = 32;
    __shared__ uint32_t wb[4][33];
    const uint4 *in4 = reinterpret_cast<const uint4 *>(info);
    uint4 *out4 = reinterpret_cast<uint4 *>(carry);
    const unsigned long long b0 = base ? *base : 0ull;
    uint32_t cm = 0, ck = (uint32_t)b0, ch = (uint32_t)(b0 >> 32), cp = 0;
    for (uint64_t c0 = 0; c0 < tiles; c0 += 1024 * PT) {
        const uint64_t t0 = c0 + (uint64_t)threadIdx.x * PT;
        uint32_t m = 0, k = 0, h = 0, p = 0;
        for (int i = 0; i < PT; ++i) {
            if (t0 + i >= tiles) break;
            const uint4 x = in4[t0 + i];
            m = lastnz(m, x.x);
            k += x.y;
            h += x.z;
            p += x.w;
        }
        uint32_t tk, th, tm, tp;
        const uint32_t em = block_exclusive_lastnz<1024>(m, wb[0], tm);
        const uint32_t ek = block_exclusive_sum<uint32_t, 1024>(k, wb[1], tk);
        const uint32_t eh = block_exclusive_sum<uint32_t, 1024>(h, wb[2], th);
        const uint32_t ep = block_exclusive_sum<uint32_t, 1024>(p, wb[3], tp);
        uint32_t rm = lastnz(cm, em), rk = ck + ek, rh = ch + eh, rp = cp + ep;
        for (int i = 0; i < PT; ++i) {
            if (t0 + i >= tiles) break;
            const uint4 x = in4[t0 + i];
            out4[t0 + i] = make_uint4(rm, rk, rh, rp);
            rm = lastnz(rm, x.x);
            rk += x.y;
            rh += x.z;
            rp += x.w;
        }
        cm = lastnz(cm, tm);
        ck += tk;
        ch += th;
        cp += tp;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        totals[0] = ck;
        totals[1] = ch;
        if (pair_total) *pair_total = cp;
    }
}

// The same scan over many CTAs (the seed round has up to 2^21 assign tiles, a
// long sequential pass for one CTA): k_scan_up reduces kScanSpan tiles per
// CTA, k_scan_top scans those aggregates from the base (one CTA), k_scan_down
// rescans each CTA's tiles from its aggregate's prefix.  agg holds the
// aggregates, then their prefixes.
constexpr int kScanThreads = 256, kScanPer = 8, kScanSpan = kScanThreads * kScanPer;

__device__ __forceinline__ void scan_load(const uint4 *in4, uint64_t tiles, uint64_t t0, uint4 (&x)[kScanPer],
                                          uint32_t &m, uint32_t &k, uint32_t &h, uint32_t &p)
{
    m = k = h = p = 0;
#pragma unroll
    for (int i = 0; i < kScanPer; ++i) {
        x[i] = t0 + i < tiles ? in4[t0 + i] : make_uint4(0, 0, 0, 0);
        m = lastnz(m, x[i].x);
        k += x[i].y;
        h += x[i].z;
        p += x[i].w;
    }
}

__global__ void __launch_bounds__(kScanThreads) k_scan_up(const uint32_t *__restrict__ info, uint64_t tiles,
                                                          uint4 *__restrict__ agg)
{
    __shared__ uint32_t wb[4][kScanThreads / 32 + 1];
    const uint64_t t0 = (uint64_t)blockIdx.x * kScanSpan + (uint64_t)threadIdx.x * kScanPer;
    uint4 x[kScanPer];
    uint32_t m, k, h, p, tm, tk, th, tp;
    scan_load(reinterpret_cast<const uint4 *>(info), tiles, t0, x, m, k, h, p);
    block_exclusive_lastnz<kScanThreads>(m, wb[0], tm);
    block_exclusive_sum<uint32_t, kScanThreads>(k, wb[1], tk);
    block_exclusive_sum<uint32_t, kScanThreads>(h, wb[2], th);
    block_exclusive_sum<uint32_t, kScanThreads>(p, wb[3], tp);
    if (threadIdx.x == 0) agg[blockIdx.x] = make_uint4(tm, tk, th, tp);
}

__global__ void __launch_bounds__(1024) k_scan_top(uint4 *__restrict__ agg, uint32_t blocks,
                                                   uint32_t *__restrict__ totals,
                                                   const unsigned long long *__restrict__ base,
                                                   unsigned long long *__restrict__ pair_total)
{
    __shared__ uint32_t wb[4][33];
    const unsigned long long b0 = base ? *base : 0ull;
    uint32_t cm = 0, ck = (uint32_t)b0, ch = (uint32_t)(b0 >> 32), cp = 0;
    for (uint32_t c0 = 0; c0 < blocks; c0 += 1024) {
        const uint32_t i = c0 + threadIdx.x;
        const uint4 x = i < blocks ? agg[i] : make_uint4(0, 0, 0, 0);
        uint32_t tm, tk, th, tp;
        const uint32_t em = block_exclusive_lastnz<1024>(x.x, wb[0], tm);
        const uint32_t ek = block_exclusive_sum<uint32_t, 1024>(x.y, wb[1], tk);
        const uint32_t eh = block_exclusive_sum<uint32_t, 1024>(x.z, wb[2], th);
        const uint32_t ep = block_exclusive_sum<uint32_t, 1024>(x.w, wb[3], tp);
        if (i < blocks) agg[blocks + i] = make_uint4(lastnz(cm, em), ck + ek, ch + eh, cp + ep);
        cm = lastnz(cm, tm);
        ck += tk;
        ch += th;
        cp += tp;
    }
    if (threadIdx.x == 0) {
        totals[0] = ck;
        totals[1] = ch;
        if (pair_total) *pair_total = cp;
    }
}

__global__ void __launch_bounds__(kScanThreads) k_scan_down(const uint32_t *__restrict__ info, uint64_t tiles,
                                                            const uint4 *__restrict__ prefix,
                                                            uint32_t *__restrict__ carry)
{
    __shared__ uint32_t wb[4][kScanThreads / 32 + 1];
    const uint64_t t0 = (uint64_t)blockIdx.x * kScanSpan + (uint64_t)threadIdx.x * kScanPer;
    uint4 x[kScanPer];
    uint32_t m, k, h, p, tm, tk, th, tp;
    scan_load(reinterpret_cast<const uint4 *>(info), tiles, t0, x, m, k, h, p);
    const uint32_t em = block_exclusive_lastnz<kScanThreads>(m, wb[0], tm);
    const uint32_t ek = block_exclusive_sum<uint32_t, kScanThreads>(k, wb[1], tk);
    const uint32_t eh = block_exclusive_sum<uint32_t, kScanThreads>(h, wb[2], th);
    const uint32_t ep = block_exclusive_sum<uint32_t, kScanThreads>(p, wb[3], tp);
    const uint4 b = prefix[blockIdx.x];
    uint32_t rm = lastnz(b.x, em), rk = b.y + ek, rh = b.z + eh, rp = b.w + ep;
    uint4 *out4 = reinterpret_cast<uint4 *>(carry);
#pragma unroll
    for (int i = 0; i < kScanPer; ++i) {
        if (t0 + i >= tiles) break;
        out4[t0 + i] = make_uint4(rm, rk, rh, rp);
        rm = lastnz(rm, x[i].x);
        rk += x[i].y;
        rh += x[i].z;
        rp += x[i].w;
    }
}

// Assign new ranks, emit singletons, compact the survivors.  Flags come from
// the head bits (one word per 32 entries, rows aligned to words), values and
// slots are read in place; nothing is staged.
// Bytes per entry: value 4 (+ slot 4 in the rounds) and 1/8 head bit read;
// rank 4; SA 4 for singletons or 12 (index, slot, group) for survivors.
template <int MODE>
__global__ void __launch_bounds__(kAssignThreads, 3)
    k_assign(TileArgs a, const uint32_t *__restrict__ carry, const uint32_t *__restrict__ heads,
             uint32_t *__restrict__ rank, uint32_t *__restrict__ sa, uint32_t *__restrict__ out_i,
             uint32_t *__restrict__ out_pos, uint32_t *__restrict__ out_gid, uint32_t *__restrict__ gstart_out)
{
    __shared__ uint32_t s_w[4][kAssignWarps];
    const uint64_t base = (uint64_t)blockIdx.x * kAssignTile;
    const uint64_t words = (a.N + 31) / 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const bool pairs = MODE == MODE_INIT_PLAIN && a.pairs;
    const uint32_t le = lanemask_lt() | (1u << lane);

    uint32_t hv_inc[kAssignPerLane], k_exc[kAssignPerLane], h_inc[kAssignPerLane];
    uint32_t vv[kAssignPerLane], pv[kAssignPerLane];
    RowFlags rf[kAssignPerLane];
    uint32_t run_m = 0, run_k = 0, run_h = 0, run_p = 0;
#pragma unroll
    for (int q = 0; q < kAssignPerLane; ++q) {
        const uint64_t j = base + (uint64_t)(warp * 256 + q * 32 + lane);
        const bool ok = j < a.N;
        vv[q] = ok ? a.vals[j] : 0u;
        pv[q] = ok ? (a.pos ? a.pos[j] : (uint32_t)j) : 0u;
    }
#pragma unroll
    for (int q = 0; q < kAssignPerLane; ++q) {
        const uint64_t r = base / 32 + (uint64_t)(warp * 8 + q);
        const uint64_t j0 = r * 32;
        const uint32_t valid = j0 >= a.N ? 0u : (a.N - j0 >= 32 ? ~0u : ((1u << (a.N - j0)) - 1u));
        RowFlags f = row_flags(heads, r, words, pairs);
        f.head &= valid;
        f.kept &= valid;
        f.kh &= valid;
        f.first &= valid;
        rf[q] = f;
        run_p += (uint32_t)__popc(f.first);
        // the last head at or before this lane gives the group start
        const uint32_t hm = f.head & le;
        const uint32_t src = hm ? 31u - (uint32_t)__clz(hm) : (uint32_t)lane;
        uint32_t m = __shfl_sync(GSAIS_FULL_MASK, pv[q] + 1, src);
        m = hm ? m : run_m;
        const uint32_t kbit = (f.kept >> lane) & 1u;
        hv_inc[q] = m;
        k_exc[q] = run_k + (uint32_t)__popc(f.kept & le) - kbit;
        h_inc[q] = run_h + (uint32_t)__popc(f.kh & le);
        run_m = __shfl_sync(GSAIS_FULL_MASK, m, 31);
        run_k += (uint32_t)__popc(f.kept);
        run_h += (uint32_t)__popc(f.kh);
    }
    if (lane == 0) { s_w[0][warp] = run_m; s_w[1][warp] = run_k; s_w[2][warp] = run_h; s_w[3][warp] = run_p; }
    __syncthreads();

    uint32_t wm = carry[4 * blockIdx.x + 0], wk = carry[4 * blockIdx.x + 1], wh = carry[4 * blockIdx.x + 2];
    for (int w = 0; w < warp; ++w) {
        wm = lastnz(wm, s_w[0][w]);
        wk += s_w[1][w];
        wh += s_w[2][w];
    }
#pragma unroll
    for (int q = 0; q < kAssignPerLane; ++q) {
        const uint64_t x = (uint64_t)(warp * 256 + q * 32 + lane);
        if (base + x >= a.N) continue;
        const uint32_t v = vv[q];
        const uint32_t r = lastnz(wm, hv_inc[q]);
        if (a.rank_out) a.rank_out[base + x] = r;
        else rank[v] = r;
        if (MODE != MODE_ROUND && v == 0 && a.slot0) *a.slot0 = (uint32_t)(base + x) + 1;
        const uint32_t bit = 1u << lane;
        if ((rf[q].single | rf[q].pair) & bit) {
            sa[pv[q]] = v;   // a single, or a pair's two members in either order until k_pair_compare
        } else {
            const uint32_t c = wk + k_exc[q];
            out_i[c] = v;
            out_pos[c] = pv[q];
            const uint32_t g = wh + h_inc[q] - 1;
            out_gid[c] = g;
            if (rf[q].kh & bit) gstart_out[g] = c;
        }
    }
    if (pairs) {
        uint32_t b = carry[4 * blockIdx.x + 3];   // pair-list slots of earlier tiles
        for (int w = 0; w < warp; ++w) b += s_w[3][w];
#pragma unroll
        for (int q = 0; q < kAssignPerLane; ++q) {
            const uint32_t m = rf[q].first;
            if ((m >> lane) & 1u) a.pairs[b + __popc(m & lanemask_lt())] = pv[q];
            b += (uint32_t)__popc(m);
        }
    }
}

// ------------------------------------------------- rounds: small / large
// Groups of at most kSmallMax suffixes are split inside one warp (no global
// sort); larger groups go through the global radix sort keyed by
// (dense large-group id, rank[i + h]).
constexpr uint32_t kSmallMax = 32;      // <= this: split inside one warp
constexpr uint32_t kMediumMax = 4096;   // <= this: sorted and split inside one CTA
constexpr uint32_t kMediumSmall = 512;   // <= this: the 128-thread CTA tier
constexpr uint32_t kNoLarge = 0xFFFFFFFFu;
constexpr uint32_t kMedium = 0xFFFFFFFEu;

// Per group: size from the group table.  Medium groups are listed for the
// CTA path; large groups get an id and a slot range in the large list from
// one combined counter, so ids and ranges are in the same order.
// Bytes per group: 8 read, 4-8 written.
// medium_small <= kMediumSmall and medium_max <= kMediumMax are the tuned
// cut-overs (the capacities of the two CTA tiers are the compiled maxima).
__global__ void __launch_bounds__(256) k_classify(const uint32_t *__restrict__ gstart, uint64_t G, uint64_t N,
                                                  uint32_t *__restrict__ lid, uint32_t *__restrict__ loff,
                                                  unsigned long long *__restrict__ lcount,
                                                  uint32_t *__restrict__ mlist, unsigned long long *__restrict__ mcount,
                                                  uint32_t *__restrict__ mlist2,
                                                  unsigned long long *__restrict__ mcount2, uint32_t medium_small,
                                                  uint32_t medium_max, uint32_t *__restrict__ lstart,
                                                  uint32_t *__restrict__ small_tiles)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g < G; g += stride) {
        const uint64_t s = gstart[g];
        const uint64_t e = g + 1 < G ? gstart[g + 1] : N;
        const uint64_t size = e - s;
        if (size > medium_max) {
            const unsigned long long old = atomicAdd(lcount, (1ull << 32) | size);
            lid[g] = (uint32_t)(old >> 32);
            loff[g] = (uint32_t)old;
            lstart[old >> 32] = (uint32_t)old;   // large id -> first slot in the large list
        } else if (size > medium_small) {
            lid[g] = kMedium;   // count in the low half, members in the high half
            mlist2[(uint32_t)atomicAdd(mcount2, (size << 32) | 1ull)] = (uint32_t)g;
        } else if (size > kSmallMax) {
            lid[g] = kMedium;
            mlist[(uint32_t)atomicAdd(mcount, (size << 32) | 1ull)] = (uint32_t)g;
        } else {
            lid[g] = kNoLarge;
            small_tiles[s >> 8] = 1u;   // k_small_groups walks the 256-entry tiles marked here
        }
    }
}

// The marked tiles, as a list (any order) with its length in *count.
__global__ void __launch_bounds__(256) k_collect_tiles(uint32_t *__restrict__ flags, uint64_t tiles,
                                                       uint32_t *__restrict__ list,
                                                       unsigned long long *__restrict__ count)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t t_round = (tiles + 31) & ~31ull;
    for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < t_round; t += stride) {
        const bool f = t < tiles && flags[t] != 0;
        const uint32_t m = __ballot_sync(GSAIS_FULL_MASK, f);
        if (!m) continue;
        const int lead = __ffs(m) - 1;
        unsigned long long base = 0;
        if ((int)(threadIdx.x & 31) == lead) base = atomicAdd(count, (unsigned long long)__popc(m));
        base = __shfl_sync(GSAIS_FULL_MASK, base, lead);
        if (f) list[base + __popc(m & lanemask_lt())] = (uint32_t)t;
    }
}

// ---- large groups with few differing members.  In a round, the members of
// a large group are ordered by r = rank[i + h].  On repetitive texts (runs,
// tandem repeats) almost all members of such a group carry the same r: the
// group's copy one period on.  Then only the few others are radix-sorted and
// the majority is placed as one run between the others below and above it,
// which gives the same list (up to order inside runs of equal keys) that the
// full sort of the group would.  The large list holds group L's members at
// [lstart[L], lstart[L+1]) with keys (L << b2) | r.
constexpr int kFewTile = 2048;               // entries per CTA (256 threads x 8)
constexpr int kFewSpan = 64;                 // large groups a tile may aggregate in shared memory

// Words of the few-others scratch: five per-group arrays (lstart, candidate,
// below, above, others before the group) and two per-tile arrays.  Large
// groups have more than 64 members, so there are at most n / 64 of them.
uint64_t few_group_words(uint64_t n) { return n / 64 + 64; }
uint64_t few_tile_words(uint64_t n) { return n / kFewTile + 64; }
size_t few_scratch_bytes(uint64_t n) { return (size_t)(5 * few_group_words(n) + 2 * few_tile_words(n)) * 4; }
// Flags and list of the small-group tiles of a round (256 entries each).
uint64_t sg_tile_words(uint64_t n) { return 2 * ((n + 255) / 256 + 64); }

// One warp per large group: the most frequent r among 32 members sampled
// evenly over the group.
__global__ void __launch_bounds__(256) k_large_cand(const uint64_t *__restrict__ lkeys,
                                                    const uint32_t *__restrict__ lstart, uint64_t LG, int b2,
                                                    uint32_t *__restrict__ cand)
{
    const uint64_t L = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (L >= LG) return;
    const int lane = threadIdx.x & 31;
    const uint64_t s = lstart[L], e = lstart[L + 1];
    const uint64_t mask = (1ull << b2) - 1;
    const uint32_t v = (uint32_t)(lkeys[s + (e - s) * (uint64_t)lane / 32] & mask);
    const uint32_t peers = __match_any_sync(GSAIS_FULL_MASK, v);
    uint32_t best = (uint32_t)__popc(peers) << 5 | (31u - (uint32_t)lane);   // ties: lowest lane
    for (int o = 16; o > 0; o >>= 1) {
        const uint32_t y = __shfl_xor_sync(GSAIS_FULL_MASK, best, o);
        best = y > best ? y : best;
    }
    const int src = 31 - (int)(best & 31u);
    const uint32_t c = __shfl_sync(GSAIS_FULL_MASK, v, src);
    if (lane == 0) cand[L] = c;
}

// Per tile: the number of members that differ from their group's candidate
// (tile_other[tile]); per group the numbers below and above it (less[L],
// greater[L]), aggregated in shared memory over the groups a tile spans.
// Bytes per entry: key 8 read.
__global__ void __launch_bounds__(256) k_large_count(const uint64_t *__restrict__ lkeys, uint64_t NL, uint64_t LG,
                                                     int b2, const uint32_t *__restrict__ cand,
                                                     uint32_t *__restrict__ less, uint32_t *__restrict__ greater,
                                                     uint32_t *__restrict__ tile_other, uint32_t *__restrict__ err)
{
    __shared__ uint32_t s_lo[kFewSpan], s_hi[kFewSpan];
    __shared__ uint32_t s_tot;
    const uint64_t t0 = (uint64_t)blockIdx.x * kFewTile;
    const uint64_t mask = (1ull << b2) - 1;
    const uint64_t L0 = lkeys[t0] >> b2;
    if (threadIdx.x < kFewSpan) {
        s_lo[threadIdx.x] = 0;
        s_hi[threadIdx.x] = 0;
    }
    if (threadIdx.x == 0) s_tot = 0;
    __syncthreads();
    uint32_t mine = 0;
    for (int k = 0; k < kFewTile / 256; ++k) {
        const uint64_t d = t0 + (uint64_t)k * 256 + threadIdx.x;
        if (d >= NL) break;
        const uint64_t key = lkeys[d];
        const uint64_t L = key >> b2;
        if (L >= LG) {
            atomicOr(err, GSAIS_ERR_BOUNDS);
            continue;
        }
        const uint32_t r = (uint32_t)(key & mask), c = cand[L];
        if (r == c) continue;
        ++mine;
        const uint64_t x = L - L0;
        if (x < (uint64_t)kFewSpan) {
            atomicAdd(r < c ? &s_lo[x] : &s_hi[x], 1u);
        } else {
            atomicAdd(r < c ? &less[L] : &greater[L], 1u);
        }
    }
    for (int o = 16; o > 0; o >>= 1) mine += __shfl_xor_sync(GSAIS_FULL_MASK, mine, o);
    if ((threadIdx.x & 31) == 0 && mine) atomicAdd(&s_tot, mine);
    __syncthreads();
    if (threadIdx.x < kFewSpan) {
        const uint64_t L = L0 + threadIdx.x;   // counts exist only for L < LG
        if (s_lo[threadIdx.x]) atomicAdd(&less[L], s_lo[threadIdx.x]);
        if (s_hi[threadIdx.x]) atomicAdd(&greater[L], s_hi[threadIdx.x]);
    }
    if (threadIdx.x == 0) tile_other[blockIdx.x] = s_tot;
}

// Exclusive prefix sums of count values (a[i], plus b[i] when b is given)
// into out[0..count], out[count] = total, by one CTA.
__global__ void __launch_bounds__(1024) k_scan_counts(const uint32_t *__restrict__ a, const uint32_t *__restrict__ b,
                                                      uint64_t count, uint32_t *__restrict__ out)
{
    __shared__ uint32_t wbuf[33];
    uint32_t run = 0;
    const uint64_t per = (count + 1023) / 1024;
    for (uint64_t base = 0; base < count; base += 1024 * 4) {
        uint32_t v[4], sum = 0;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const uint64_t i = base + (uint64_t)threadIdx.x * 4 + q;
            v[q] = i < count ? a[i] + (b ? b[i] : 0u) : 0u;
            sum += v[q];
        }
        uint32_t total;
        uint32_t x = run + block_exclusive_sum<uint32_t, 1024>(sum, wbuf, total);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const uint64_t i = base + (uint64_t)threadIdx.x * 4 + q;
            if (i < count) out[i] = x;
            x += v[q];
        }
        run += total;
    }
    (void)per;
    if (threadIdx.x == 0) out[count] = run;
}

// Places the majority members of each group at lstart[L] + less[L] + their
// index among the group's majority (list order), and appends the others, in
// list order, to the others list at their global index.  O(d) (others before
// d) = tile_off[tile] + the others before d inside the tile; the group's
// others before its start = ocum[L].  Bytes per entry: key 8 + value 4 read,
// 12 written.
__global__ void __launch_bounds__(256) k_large_place(const uint64_t *__restrict__ lkeys,
                                                     const uint32_t *__restrict__ lvals, uint64_t NL, uint64_t LG,
                                                     int b2,
                                                     const uint32_t *__restrict__ cand,
                                                     const uint32_t *__restrict__ lstart,
                                                     const uint32_t *__restrict__ less,
                                                     const uint32_t *__restrict__ ocum,
                                                     const uint32_t *__restrict__ tile_off,
                                                     uint64_t *__restrict__ out_keys, uint32_t *__restrict__ out_vals,
                                                     uint64_t *__restrict__ okeys, uint32_t *__restrict__ ovals,
                                                     uint32_t *__restrict__ err)
{
    __shared__ uint32_t s_w[8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint64_t t0 = (uint64_t)blockIdx.x * kFewTile;
    const uint64_t mask = (1ull << b2) - 1;
    // warp w handles the 256 entries [t0 + 256 w, ...), eight rows of 32
    uint64_t key[8];
    uint32_t val[8], oth = 0;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const uint64_t d = t0 + (uint64_t)warp * 256 + q * 32 + lane;
        const bool ok = d < NL && (lkeys[d] >> b2) < LG;   // k_large_count flags keys of no large group
        key[q] = ok ? lkeys[d] : 0ull;
        val[q] = ok ? lvals[d] : 0u;
        const bool o = ok && (uint32_t)(key[q] & mask) != cand[key[q] >> b2];
        if (!ok) key[q] = ~0ull;   // marks an entry to skip
        oth |= (uint32_t)o << q;
    }
    uint32_t wtot = 0;
#pragma unroll
    for (int q = 0; q < 8; ++q) wtot += (uint32_t)__popc(__ballot_sync(GSAIS_FULL_MASK, (oth >> q) & 1u));
    if (lane == 0) s_w[warp] = wtot;
    __syncthreads();
    uint32_t before = tile_off[blockIdx.x];
    for (int w = 0; w < warp; ++w) before += s_w[w];
    bool bad = false;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const uint64_t d = t0 + (uint64_t)warp * 256 + q * 32 + lane;
        const uint32_t ball = __ballot_sync(GSAIS_FULL_MASK, (oth >> q) & 1u);
        const uint32_t Od = before + (uint32_t)__popc(ball & lanemask_lt());
        before += (uint32_t)__popc(ball);
        if (d >= NL || key[q] == ~0ull) continue;
        const uint64_t L = key[q] >> b2;
        if ((oth >> q) & 1u) {
            okeys[Od] = key[q];
            ovals[Od] = val[q];
        } else {
            const uint64_t dest = (uint64_t)less[L] + d - Od + ocum[L];
            if (dest < lstart[L] || dest >= lstart[L + 1]) {
                bad = true;
                continue;
            }
            out_keys[dest] = key[q];
            out_vals[dest] = val[q];
        }
    }
    if (bad) atomicOr(err, GSAIS_ERR_BOUNDS);
}

// The sorted others into their groups: below the majority run when r < c,
// above it otherwise.  Bytes per other: 12 read, 12 written.
__global__ void __launch_bounds__(256) k_others_place(const uint64_t *__restrict__ okeys,
                                                      const uint32_t *__restrict__ ovals, uint64_t O, int b2,
                                                      const uint32_t *__restrict__ lstart,
                                                      const uint32_t *__restrict__ less,
                                                      const uint32_t *__restrict__ greater,
                                                      const uint32_t *__restrict__ ocum, uint64_t LG,
                                                      uint64_t *__restrict__ out_keys, uint32_t *__restrict__ out_vals,
                                                      uint32_t *__restrict__ err)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; q < O; q += stride) {
        const uint64_t key = okeys[q];
        const uint64_t L = key >> b2;
        if (L >= LG) {
            atomicOr(err, GSAIS_ERR_BOUNDS);
            continue;
        }
        const uint64_t s = lstart[L], size = lstart[L + 1] - s;
        const uint64_t t = q - ocum[L];
        const uint64_t lo = less[L], hi = greater[L];
        const uint64_t M = size - lo - hi;
        const uint64_t dest = s + (t < lo ? t : M + t);
        if (t >= lo + hi || dest >= s + size) {
            atomicOr(err, GSAIS_ERR_BOUNDS);
            continue;
        }
        out_keys[dest] = key;
        out_vals[dest] = ovals[q];
    }
}

__global__ void k_set_word(uint32_t *__restrict__ p, uint32_t v) { *p = v; }

// Bitonic sort of THREADS * R keys held R to a thread (thread t holds
// positions t*R .. t*R+R-1), stages k <= pw only (pw a power of two; the
// positions >= pw are never touched).  A compare-exchange partner t ^ j is
// in the same thread for j < R, in another lane of the warp for
// j < 32 * R (shuffles) and in another warp otherwise (shared memory).
template <int THREADS, int R>
__device__ __forceinline__ void block_bitonic(uint64_t (&v)[R], uint64_t *__restrict__ sm, uint32_t pw)
{
    const uint32_t base = threadIdx.x * R;
    for (uint32_t k = 2; k <= pw; k <<= 1) {
        for (uint32_t j = k >> 1; j >= (uint32_t)R; j >>= 1) {
            if (j >= 32u * R) {
#pragma unroll
                for (int r = 0; r < R; ++r) sm[base + r] = v[r];
                __syncthreads();
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    const uint32_t t = base + r;
                    const uint64_t b = sm[t ^ j];
                    const bool lo = ((t & j) == 0) == ((t & k) == 0);
                    v[r] = lo ? (v[r] < b ? v[r] : b) : (v[r] > b ? v[r] : b);
                }
                __syncthreads();
            } else {
                const int lx = (int)(j / R);
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    const uint32_t t = base + r;
                    const uint64_t b = __shfl_xor_sync(GSAIS_FULL_MASK, v[r], lx);
                    const bool lo = ((t & j) == 0) == ((t & k) == 0);
                    v[r] = lo ? (v[r] < b ? v[r] : b) : (v[r] > b ? v[r] : b);
                }
            }
        }
#pragma unroll
        for (int jj = R / 2; jj > 0; jj >>= 1) {
            if ((uint32_t)jj < k) {
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    if (r & jj) continue;
                    const bool asc = ((base + r) & k) == 0;
                    const uint64_t a = v[r], b = v[r | jj];
                    const uint64_t mn = a < b ? a : b, mx = a < b ? b : a;
                    v[r] = asc ? mn : mx;
                    v[r | jj] = asc ? mx : mn;
                }
            }
        }
    }
}

// Splits the medium groups (kSmallMax < size <= MAXN), one group per CTA
// iteration (two tiers: 128 threads for groups of at most kMediumSmall, 256
// for the rest): keys (rank[i+h] << 12 | member) are bitonic-sorted in
// registers (block_bitonic); a member's new slot is the group's first slot plus its
// sorted position, its rank 1 + the first slot of its run of equal keys; a
// run of one is final; survivors are appended behind the same atomic
// (groups, entries) reservation as the warp path.
// Bytes per suffix: r2 4 + index 4 read, rank scatter 4, SA 4 or survivors 12.
template <int THREADS, uint32_t MAXN>
__global__ void __launch_bounds__(THREADS) k_medium_groups(const uint32_t *__restrict__ mlist,
                                                       const unsigned long long *__restrict__ mcount,
                                                       const uint32_t *__restrict__ gstart, uint64_t G, uint64_t N,
                                                       const uint32_t *__restrict__ act_i,
                                                       const uint32_t *__restrict__ act_pos,
                                                       const uint32_t *__restrict__ r2, uint32_t *__restrict__ rank,
                                                       uint32_t *__restrict__ sa, uint32_t *__restrict__ out_i,
                                                       uint32_t *__restrict__ out_pos, uint32_t *__restrict__ out_gid,
                                                       uint32_t *__restrict__ gstart_out,
                                                       unsigned long long *__restrict__ counter)
{
    constexpr int R = (int)(MAXN / THREADS);
    static_assert(R * THREADS == (int)MAXN && (R & (R - 1)) == 0, "MAXN = THREADS * power of two");
    constexpr uint32_t kFewOthers = 128;   // one warp's register sort
    __shared__ uint64_t key[MAXN];
    __shared__ uint64_t few[kFewOthers];
    __shared__ uint32_t wb[2][THREADS / 32 + 1];
    __shared__ unsigned long long s_base;
    __shared__ uint32_t s_lt;
    const uint32_t M = (uint32_t)*mcount;
    const int tid = threadIdx.x;
    for (uint32_t m = blockIdx.x; m < M; m += gridDim.x) {
        const uint32_t g = mlist[m];
        const uint64_t s = gstart[g];
        const uint64_t e = (uint64_t)g + 1 < G ? gstart[g + 1] : N;
        const uint32_t size = (uint32_t)(e - s);
        const uint32_t P = act_pos[s];
        uint32_t pw = 64;
        while (pw < size) pw <<= 1;
        const uint32_t r0 = r2[s];
        bool same = true;
        uint64_t v[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const uint32_t t = tid * R + r;
            const uint32_t rt = t < size ? r2[s + t] : r0;
            same &= rt == r0;
            v[r] = t < size ? (((uint64_t)rt << 12) | t) : ~0ull;
        }
        if (__syncthreads_and(same)) {
            // No member differs at this depth (copies of one long repeat):
            // the group survives whole, in member order, and its ranks
            // (1 + its first slot) stay as they are.
            if (tid == 0) s_base = atomicAdd(counter, (1ull << 32) | size);
            __syncthreads();
            const uint32_t base_e = (uint32_t)s_base, gid = (uint32_t)(s_base >> 32);
            for (uint32_t t = tid; t < size; t += THREADS) {
                out_i[base_e + t] = act_i[s + t];
                out_pos[base_e + t] = P + t;
                out_gid[base_e + t] = gid;
            }
            if (tid == 0) gstart_out[gid] = base_e;
            // s_base is next written after the next group's __syncthreads_and,
            // which every thread reaches only after reading it here
            continue;
        }
        // Mostly one value (a run of periodic repeats loses a few members a
        // round): the D members whose r2 differs from the middle member's are
        // sorted by warp 0 when D <= kFewOthers, and the others form one run,
        // in member order, between the smaller and the larger ones; the
        // result equals the full sort of the keys.
        const uint32_t c = r2[s + size / 2];
        uint32_t nb = 0;
#pragma unroll
        for (int r = 0; r < R; ++r) nb += tid * R + r < size && (uint32_t)(v[r] >> 12) != c;
        uint32_t D;
        const uint32_t nb_ex = block_exclusive_sum<uint32_t, THREADS>(nb, wb[1], D);
        if (D <= kFewOthers) {
            uint32_t o = nb_ex;
#pragma unroll
            for (int r = 0; r < R; ++r)
                if (tid * R + r < size && (uint32_t)(v[r] >> 12) != c) few[o++] = v[r];
            __syncthreads();
            if (tid < 32) {
                uint32_t pd = 2;
                while (pd < D) pd <<= 1;
                uint64_t w[4];
#pragma unroll
                for (int r = 0; r < 4; ++r) w[r] = (uint32_t)(tid * 4 + r) < D ? few[tid * 4 + r] : ~0ull;
                block_bitonic<32, 4>(w, nullptr, pd);   // pd <= 128: every partner is in this warp
                uint32_t lt = 0;
                const uint32_t B = size - D;
#pragma unroll
                for (int r = 0; r < 4; ++r) {
                    const uint32_t x = tid * 4 + r;
                    const uint32_t rw = (uint32_t)(w[r] >> 12);
                    lt += __popc(__ballot_sync(GSAIS_FULL_MASK, x < D && rw < c));
                    if (x < D) key[x + (rw > c ? B : 0u)] = w[r];
                }
                if (tid == 0) s_lt = lt;
            }
            __syncthreads();
            uint32_t b = s_lt + tid * R - nb_ex;   // slot of this thread's first member of the run
#pragma unroll
            for (int r = 0; r < R; ++r)
                if (tid * R + r < size && (uint32_t)(v[r] >> 12) == c) key[b++] = v[r];
        } else {
            block_bitonic<THREADS, R>(v, key, pw);
#pragma unroll
            for (int r = 0; r < R; ++r) key[tid * R + r] = v[r];
        }
        __syncthreads();
        // blocked ranges of sorted positions per thread
        const uint32_t C = (size + THREADS - 1) / THREADS;
        const uint32_t k0 = tid * C, k1 = k0 + C < size ? k0 + C : size;
        uint32_t lastv = 0, surv = 0, sheads = 0;
        for (uint32_t k = k0; k < k1; ++k) {
            const uint64_t rk = key[k] >> 12;
            const bool head = k == 0 || (key[k - 1] >> 12) != rk;
            const bool last = k + 1 == size || (key[k + 1] >> 12) != rk;
            if (head) lastv = k + 1;
            if (!(head && last)) {
                ++surv;
                sheads += head;
            }
        }
        uint32_t tot_sh, tot_l;
        const uint32_t ex_last = block_exclusive_lastnz<THREADS>(lastv, wb[0], tot_l);
        // survivors and survivor heads (each <= 4096) in the two halves of one word
        const uint32_t ex_sh = block_exclusive_sum<uint32_t, THREADS>(surv | sheads << 16, wb[1], tot_sh);
        const uint32_t ex_surv = ex_sh & 0xFFFFu, ex_head = ex_sh >> 16;
        const uint32_t tot_s = tot_sh & 0xFFFFu, tot_h = tot_sh >> 16;
        if (tid == 0) s_base = tot_s ? atomicAdd(counter, ((unsigned long long)tot_h << 32) | tot_s) : 0ull;
        __syncthreads();
        const uint32_t base_e = (uint32_t)s_base, base_g = (uint32_t)(s_base >> 32);
        uint32_t run = ex_last, cs = ex_surv, ch = ex_head;
        for (uint32_t k = k0; k < k1; ++k) {
            const uint64_t kv = key[k];
            const uint64_t rk = kv >> 12;
            const bool head = k == 0 || (key[k - 1] >> 12) != rk;
            const bool last = k + 1 == size || (key[k + 1] >> 12) != rk;
            if (head) run = k + 1;
            const uint32_t i = act_i[s + (kv & 4095u)];
            rank[i] = 1 + P + (run - 1);
            if (head && last) {
                sa[P + k] = i;
            } else {
                ch += head;
                const uint32_t gid = base_g + ch - 1;
                const uint32_t c = base_e + cs++;
                out_i[c] = i;
                out_pos[c] = P + k;
                out_gid[c] = gid;
                if (head) gstart_out[gid] = c;
            }
        }
        __syncthreads();   // key[] is reused by the next group
    }
}

// Gathers rank[i + h] of every active suffix (before any rank of this round
// changes).  Entries of small groups keep it in r2[]; entries of large groups
// are copied to the large list with key (large id << b2 | rank), and the
// key's digit histograms are accumulated for the radix sort.
// Bytes per active suffix: index 4 + slot 4 + group 4 read, rank gather 4,
// group table 8 read; 4 (r2) or 16 (large list) written.
__global__ void __launch_bounds__(256) k_round_r2(const uint32_t *__restrict__ act_i,
                                                  const uint32_t *__restrict__ act_pos,
                                                  const uint32_t *__restrict__ act_gid,
                                                  const uint32_t *__restrict__ gstart, const uint32_t *__restrict__ lid,
                                                  const uint32_t *__restrict__ loff, const uint32_t *__restrict__ rank,
                                                  uint64_t h, uint64_t N, uint64_t n, int b2, uint32_t *__restrict__ r2o,
                                                  uint64_t *__restrict__ lkeys, uint32_t *__restrict__ lvals,
                                                  uint32_t *__restrict__ lpos, uint32_t *__restrict__ err, int passes,
                                                  int end_bit, uint32_t *__restrict__ hist)
{
    __shared__ uint32_t sh[kMaxRadixPasses][256];
    radix_hist_zero(sh, passes);
    __syncthreads();
    // B entries per thread per step: the list loads, then the dependent
    // gathers (rank[i+h], the group's class), then the writes
    constexpr int B = 4;
    const uint64_t span = (uint64_t)gridDim.x * blockDim.x * B;
    const uint64_t N_round = (N + 31) & ~31ull;   // whole warps iterate together
    for (uint64_t j0 = (uint64_t)blockIdx.x * blockDim.x * B + threadIdx.x; j0 < N_round; j0 += span) {
        uint32_t iv[B], gv[B], r2v[B], Lv[B];
#pragma unroll
        for (int b = 0; b < B; ++b) {
            const uint64_t j = j0 + (uint64_t)b * blockDim.x;
            iv[b] = j < N ? act_i[j] : 0u;
            gv[b] = j < N ? act_gid[j] : 0u;
        }
#pragma unroll
        for (int b = 0; b < B; ++b) {
            const uint64_t j = j0 + (uint64_t)b * blockDim.x;
            // an active suffix has length >= h, so i + h <= n (rank[n] is the sentinel)
            const bool ok = j < N && (uint64_t)iv[b] + h <= n;
            r2v[b] = ok ? rank[iv[b] + h] : 0u;
            Lv[b] = j < N ? lid[gv[b]] : kNoLarge;
            if (j < N && !ok) atomicOr(err, GSAIS_ERR_BOUNDS);
        }
#pragma unroll
        for (int b = 0; b < B; ++b) {
            const uint64_t j = j0 + (uint64_t)b * blockDim.x;
            bool large = false;
            uint64_t key = 0;
            if (j < N) {
                const uint32_t g = gv[b], L = Lv[b];
                if (L >= kMedium) {   // small or medium group: keep rank[i+h] by list position
                    r2o[j] = r2v[b];
                } else {
                    large = true;
                    const uint64_t d = (uint64_t)loff[g] + (j - gstart[g]);
                    key = ((uint64_t)L << b2) | r2v[b];
                    lkeys[d] = key;
                    lvals[d] = iv[b];
                    lpos[d] = act_pos[j];
                }
            }
            radix_hist_add(sh, key, large, passes, end_bit);
        }
    }
    __syncthreads();
    radix_hist_flush(sh, passes, hist);
}

// Splits the small groups.  A warp takes a window of 32 list positions and
// owns the groups that start in it (with their members: at most 63
// entries, two per lane).  For each owned suffix, counting over its group's
// members gives lt (members with smaller rank[i+h]), eq and its new slot;
// rank = 1 + first slot of its new subgroup; a subgroup of one is final
// (SA[slot] = i); survivors are written in slot order behind one atomic
// reservation per CTA of (groups, entries), which keeps group ids increasing
// with list position.  Bytes per suffix: 16 read, rank scatter 4, SA 4 or
// survivors 12-16 written.
// Ranks inside the owned groups of a 64-entry warp window (entry o = e * 32 +
// lane holds the values of offset o) by a bitonic sort of the keys
// (group start, r2, offset) -- unique, so the order is total -- with the
// entries of groups the warp does not own sorted past the end.  In sorted
// order a group's members are contiguous and ordered by (r2, offset), so
// before = position - group start, lt = start of the run of equal r2 -
// group start and eq = the run's length; they go back to their entries
// through shared memory (s: 3 x 64 words of this warp).  About 21 exchange
// stages, against maxsz steps of all-pairs comparison: used for warps whose
// largest owned group has more than kSmallSortMin members.
constexpr int kSmallSortMin = 16;

__device__ __forceinline__ void window_rank_sort(const bool (&own)[2], const int (&gs)[2], uint32_t r0, uint32_t r1,
                                                 uint32_t (&lt)[2], uint32_t (&eq)[2], uint32_t (&before)[2],
                                                 uint32_t *s)
{
    const int lane = threadIdx.x & 31;
    uint64_t k[2];
    k[0] = own[0] ? ((uint64_t)gs[0] << 38) | ((uint64_t)r0 << 6) | (uint64_t)lane : ~0ull;
    k[1] = own[1] ? ((uint64_t)gs[1] << 38) | ((uint64_t)r1 << 6) | (uint64_t)(32 + lane) : ~0ull;
#pragma unroll
    for (int kk = 2; kk <= 64; kk <<= 1) {
#pragma unroll
        for (int j = kk >> 1; j > 0; j >>= 1) {
            if (j == 32) {   // kk == 64: entries lane and 32 + lane, ascending
                const uint64_t a = k[0] < k[1] ? k[0] : k[1], b = k[0] < k[1] ? k[1] : k[0];
                k[0] = a;
                k[1] = b;
            } else {
#pragma unroll
                for (int e = 0; e < 2; ++e) {
                    const uint64_t o = __shfl_xor_sync(GSAIS_FULL_MASK, k[e], j);
                    const bool asc = ((e * 32 + lane) & kk) == 0;
                    const bool lower = (lane & j) == 0;
                    const bool take_min = lower == asc;
                    k[e] = take_min ? (o < k[e] ? o : k[e]) : (o > k[e] ? o : k[e]);
                }
            }
        }
    }
    // boundaries in sorted order: group heads, heads of runs of equal r2, the valid range
    const uint64_t p0 = __shfl_up_sync(GSAIS_FULL_MASK, k[0], 1);
    uint64_t p1 = __shfl_up_sync(GSAIS_FULL_MASK, k[1], 1);
    const uint64_t last0 = __shfl_sync(GSAIS_FULL_MASK, k[0], 31);
    if (lane == 0) p1 = last0;
    const bool v0 = k[0] != ~0ull, v1 = k[1] != ~0ull;
    const bool gh0 = v0 && (lane == 0 || (p0 >> 38) != (k[0] >> 38));
    const bool gh1 = v1 && (p1 >> 38) != (k[1] >> 38);
    const bool vh0 = v0 && (lane == 0 || (p0 >> 6) != (k[0] >> 6));
    const bool vh1 = v1 && (p1 >> 6) != (k[1] >> 6);
    const uint64_t GH = (uint64_t)__ballot_sync(GSAIS_FULL_MASK, gh0) | ((uint64_t)__ballot_sync(GSAIS_FULL_MASK, gh1) << 32);
    const uint64_t VH = (uint64_t)__ballot_sync(GSAIS_FULL_MASK, vh0) | ((uint64_t)__ballot_sync(GSAIS_FULL_MASK, vh1) << 32);
    const uint64_t INV = ~((uint64_t)__ballot_sync(GSAIS_FULL_MASK, v0) | ((uint64_t)__ballot_sync(GSAIS_FULL_MASK, v1) << 32));
#pragma unroll
    for (int e = 0; e < 2; ++e) {
        if (!(e ? v1 : v0)) continue;
        const int p = e * 32 + lane;
        const uint64_t upto = p == 63 ? ~0ull : ((2ull << p) - 1);
        const int g0 = 63 - __clzll((long long)(GH & upto));
        const int vs = 63 - __clzll((long long)(VH & upto));
        const uint64_t above = (VH | INV) & ~upto;
        const int ve = above ? __ffsll((long long)above) - 1 : 64;
        const uint32_t o = (uint32_t)(k[e] & 63);
        s[o] = (uint32_t)(vs - g0);
        s[64 + o] = (uint32_t)(ve - vs);
        s[128 + o] = (uint32_t)(p - g0);
    }
    __syncwarp();
#pragma unroll
    for (int e = 0; e < 2; ++e) {
        if (!own[e]) continue;
        const int o = e * 32 + lane;
        lt[e] = s[o];
        eq[e] = s[64 + o];
        before[e] = s[128 + o];
    }
    __syncwarp();
}

__global__ void __launch_bounds__(256) k_small_groups(const uint32_t *__restrict__ act_i,
                                                      const uint32_t *__restrict__ act_pos,
                                                      const uint32_t *__restrict__ act_gid,
                                                      const uint32_t *__restrict__ r2, uint64_t N,
                                                      uint32_t *__restrict__ rank, uint32_t *__restrict__ sa,
                                                      uint32_t *__restrict__ out_i, uint32_t *__restrict__ out_pos,
                                                      uint32_t *__restrict__ out_gid,
                                                      uint32_t *__restrict__ gstart_out,
                                                      unsigned long long *__restrict__ counter,
                                                      uint32_t *__restrict__ pairs,
                                                      unsigned long long *__restrict__ pair_count,
                                                      const uint32_t *__restrict__ tile_list,
                                                      const unsigned long long *__restrict__ tile_count)
{
    constexpr int WARPS = 8;
    __shared__ uint32_t s_we[WARPS], s_wg[WARPS];
    __shared__ unsigned long long s_base;
    __shared__ uint32_t s_rk[WARPS][3 * 64];   // window_rank_sort results by window offset
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // a resident grid walks the 256-entry tiles in which a small group starts
    // (listed by k_classify / k_collect_tiles); a tile whose warps own no
    // group is skipped whole
    const uint64_t tiles = *tile_count;
    for (uint64_t ti = blockIdx.x; ti < tiles; ti += gridDim.x) {
    const uint64_t tile = tile_list[ti];
    const uint64_t wb = (tile * WARPS + warp) * 32;
    const uint64_t j0 = wb + lane, j1 = wb + 32 + lane;
    const bool v0 = j0 < N, v1 = j1 < N;
    const uint32_t g0 = v0 ? act_gid[j0] : 0xFFFFFFFFu;
    const uint32_t g1 = v1 ? act_gid[j1] : 0xFFFFFFFEu;
    uint32_t pg0 = __shfl_up_sync(GSAIS_FULL_MASK, g0, 1);
    uint32_t pg1 = __shfl_up_sync(GSAIS_FULL_MASK, g1, 1);
    const uint32_t g0_last = __shfl_sync(GSAIS_FULL_MASK, g0, 31);
    if (lane == 0) {
        pg0 = (wb > 0 && wb - 1 < N) ? act_gid[wb - 1] : ~g0;
        pg1 = g0_last;
    }
    const bool head0 = v0 && (j0 == 0 || g0 != pg0);
    const bool head1 = v1 && g1 != pg1;
    const uint64_t H = (uint64_t)__ballot_sync(GSAIS_FULL_MASK, head0) |
                       ((uint64_t)__ballot_sync(GSAIS_FULL_MASK, head1) << 32);

    // group [gs, ge) (window offsets) of offset o; gs = -1 if it started before the window
    auto group_of = [&](int o, int &gs, int &ge) {
        const uint64_t upto = o == 63 ? ~0ull : ((2ull << o) - 1);
        const uint64_t m = H & upto;
        gs = m ? 63 - __clzll((long long)m) : -1;
        const uint64_t above = H & ~upto;
        ge = above ? __ffsll((long long)above) - 1 : 64;
    };
    int gs[2], ge[2];
    group_of(lane, gs[0], ge[0]);
    group_of(32 + lane, gs[1], ge[1]);
    bool own[2];
    for (int e = 0; e < 2; ++e) {
        const uint64_t j = e ? j1 : j0;
        bool ok = (e ? v1 : v0) && gs[e] >= 0 && gs[e] < 32;
        if (ok) {
            const uint64_t start = wb + gs[e];
            const uint64_t end = (ge[e] == 64 || wb + ge[e] > N) ? N : wb + ge[e];
            // a group reaching the window end may continue: it is large then
            const bool open = ge[e] == 64 && wb + 64 < N;
            ok = !open && end - start <= kSmallMax;
        }
        (void)j;
        own[e] = ok;
    }
    if (!__syncthreads_or(own[0] || own[1])) continue;   // the same decision in every thread
    const uint32_t rr0 = own[0] ? r2[j0] : 0u, rr1 = own[1] ? r2[j1] : 0u;
    const uint32_t p0 = own[0] ? act_pos[j0] : 0u, p1 = own[1] ? act_pos[j1] : 0u;
    const uint32_t i0 = own[0] ? act_i[j0] : 0u, i1 = own[1] ? act_i[j1] : 0u;

    // group end inside the window (the list may end before offset 64);
    // the widest owned group of the warp bounds the member loops
    int gend[2];
    int sz_me = 0;
    for (int e = 0; e < 2; ++e) {
        gend[e] = (ge[e] == 64 || wb + ge[e] > N) ? (int)(N - wb < 64 ? N - wb : 64) : ge[e];
        if (own[e]) {
            const int sz = gend[e] - gs[e];
            sz_me = sz > sz_me ? sz : sz_me;
        }
    }
    const int maxsz = (int)__reduce_max_sync(GSAIS_FULL_MASK, (uint32_t)sz_me);

    uint32_t lt[2] = {0, 0}, eq[2] = {0, 0}, before[2] = {0, 0};
    const uint32_t myr[2] = {rr0, rr1};
    if (maxsz > kSmallSortMin) window_rank_sort(own, gs, rr0, rr1, lt, eq, before, s_rk[warp]);
    else
    for (int t = 0; t < maxsz; ++t) {
        for (int e = 0; e < 2; ++e) {
            const int src = (gs[e] < 0 ? 0 : gs[e]) + t;
            const uint32_t a = __shfl_sync(GSAIS_FULL_MASK, rr0, src & 31);
            const uint32_t b = __shfl_sync(GSAIS_FULL_MASK, rr1, src & 31);
            const uint32_t rt = src >= 32 ? b : a;
            const int o = e ? 32 + lane : lane;
            if (own[e] && src < gend[e]) {
                lt[e] += rt < myr[e];
                eq[e] += rt == myr[e];
                before[e] += (rt < myr[e]) || (rt == myr[e] && src < o);
            }
        }
    }
    // the group's first slot is the slot of its first member (offset gs < 32)
    uint32_t P[2];
    for (int e = 0; e < 2; ++e) P[e] = __shfl_sync(GSAIS_FULL_MASK, p0, (gs[e] < 0 ? 0 : gs[e]) & 31);

    bool surv[2], hsub[2];
    for (int e = 0; e < 2; ++e) {
        surv[e] = false;
        hsub[e] = false;
        if (!own[e]) continue;
        const uint32_t idx = e ? i1 : i0;
        const uint32_t sub = P[e] + lt[e];
        rank[idx] = 1 + sub;
        if (eq[e] == 1) {
            sa[sub] = idx;
        } else {
            surv[e] = true;
            hsub[e] = before[e] == lt[e];
        }
    }
    // A tied pair (a group of exactly two members with equal r2) leaves the
    // doubling: its members go to sa[P], sa[P + 1] in either order and the
    // slot P to the pair list, to be ordered by comparing the two suffixes
    // directly (k_pair_compare).  The first member of an owned group always
    // sits at offset gs < 32, i.e. in the first half of the window.
    if (pairs) {
        const uint32_t nx0 = __shfl_sync(GSAIS_FULL_MASK, i0, (lane + 1) & 31);
        const uint32_t nx1 = __shfl_sync(GSAIS_FULL_MASK, i1, (lane + 1) & 31);
        bool lead = false;
        for (int e = 0; e < 2; ++e) {
            if (own[e] && gend[e] - gs[e] == 2 && eq[e] == 2) {
                surv[e] = false;
                hsub[e] = false;
                if (e == 0 && gs[0] == lane) lead = true;
            }
        }
        const uint32_t m = __ballot_sync(GSAIS_FULL_MASK, lead);
        if (m) {
            uint32_t b = 0;
            if (lane == 0) b = (uint32_t)atomicAdd(pair_count, (unsigned long long)__popc(m));
            b = __shfl_sync(GSAIS_FULL_MASK, b, 0);
            if (lead) {
                sa[P[0]] = i0;
                sa[P[0] + 1] = lane < 31 ? nx0 : nx1;
                pairs[b + __popc(m & lanemask_lt())] = P[0];
            }
        }
    }
    const uint64_t S = (uint64_t)__ballot_sync(GSAIS_FULL_MASK, surv[0]) |
                       ((uint64_t)__ballot_sync(GSAIS_FULL_MASK, surv[1]) << 32);
    const uint64_t HS = (uint64_t)__ballot_sync(GSAIS_FULL_MASK, hsub[0]) |
                        ((uint64_t)__ballot_sync(GSAIS_FULL_MASK, hsub[1]) << 32);

    // survivors / subgroup heads of my group ordered before me
    uint32_t sb[2] = {0, 0}, hb[2] = {0, 0};
    const uint32_t bf0 = before[0], bf1 = before[1];
    for (int t = 0; t < maxsz; ++t) {
        for (int e = 0; e < 2; ++e) {
            const int src = (gs[e] < 0 ? 0 : gs[e]) + t;
            const uint32_t ra = __shfl_sync(GSAIS_FULL_MASK, rr0, src & 31);
            const uint32_t rb = __shfl_sync(GSAIS_FULL_MASK, rr1, src & 31);
            const uint32_t ba = __shfl_sync(GSAIS_FULL_MASK, bf0, src & 31);
            const uint32_t bb = __shfl_sync(GSAIS_FULL_MASK, bf1, src & 31);
            const uint32_t rt = src >= 32 ? rb : ra;
            const uint32_t bt = src >= 32 ? bb : ba;
            if (surv[e] && src < gend[e]) {
                const bool st = (S >> src) & 1ull, ht = (HS >> src) & 1ull;
                sb[e] += st && bt < before[e];
                hb[e] += ht && rt < myr[e];
            }
        }
    }
    // per-warp totals -> one reservation per CTA
    if (lane == 0) {
        s_we[warp] = (uint32_t)__popcll((long long)S);
        s_wg[warp] = (uint32_t)__popcll((long long)HS);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t te = 0, tg = 0;
        for (int w = 0; w < WARPS; ++w) {
            const uint32_t a = s_we[w], b = s_wg[w];
            s_we[w] = te;
            s_wg[w] = tg;
            te += a;
            tg += b;
        }
        s_base = (te | tg) ? atomicAdd(counter, ((unsigned long long)tg << 32) | te) : 0ull;
    }
    __syncthreads();
    const uint32_t base_e = (uint32_t)s_base + s_we[warp];
    const uint32_t base_g = (uint32_t)(s_base >> 32) + s_wg[warp];
    for (int e = 0; e < 2; ++e) {
        if (!surv[e]) continue;
        const uint64_t below = (1ull << gs[e]) - 1;   // offsets of earlier groups in the window
        const uint32_t c = base_e + (uint32_t)__popcll((long long)(S & below)) + sb[e];
        const uint32_t g = base_g + (uint32_t)__popcll((long long)(HS & below)) + hb[e];
        out_i[c] = e ? i1 : i0;
        out_pos[c] = P[e] + before[e];
        out_gid[c] = g;
        if (hsub[e]) gstart_out[g] = c;
    }
    __syncthreads();   // s_we, s_wg and s_base are reused by the next tile
    }
}

// ------------------------------------------------------ batched strings
// Many independent strings are sorted together: string s of the
// concatenation occupies [offs[s], offs[s+1]) and, in rank coordinates, the
// slots [offs[s] + s, offs[s+1] + s) followed by one gap slot whose rank is
// 0 (its end-of-string sentinel).  Symbol codes are shifted by one so the
// gap's code 0 ends a seed window: a suffix shorter than K packs zeros after
// its last symbol and therefore sorts before every longer suffix with the
// same symbols (libsais's implicit sentinel).  The string id sits in the
// high bits of the seed key, so groups never span two strings and the
// sorted rows come out grouped by string.

// Largest s with offs[s] <= p (offs has count + 1 entries, offs[count] = n).
__device__ __forceinline__ uint32_t string_of(const uint64_t *__restrict__ offs, uint32_t count, uint64_t p)
{
    uint32_t lo = 0, hi = count;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (offs[mid] <= p) lo = mid;
        else hi = mid;
    }
    return lo;
}

// Bytes per suffix: T s read (windows overlap in L1), key 8 + value 4 written.
template <typename Sym>
__global__ void __launch_bounds__(256) k_seed_batch(const Sym *__restrict__ T, uint64_t n,
                                                    const uint64_t *__restrict__ offs, uint32_t count,
                                                    const uint16_t *__restrict__ codes, int bits, int K,
                                                    uint64_t *__restrict__ keys, uint32_t *__restrict__ vals,
                                                    int passes, int end_bit, uint32_t *__restrict__ hist)
{
    __shared__ uint32_t sh[kMaxRadixPasses][256];
    radix_hist_zero(sh, passes);
    __syncthreads();
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t n_round = (n + 31) & ~31ull;
    for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n_round; p += stride) {
        const bool ok = p < n;
        uint64_t key = 0;
        if (ok) {
            const uint32_t s = string_of(offs, count, p);
            const uint64_t e = offs[s + 1];
            for (int q = 0; q < K; ++q) {
                const uint64_t c = p + q < e ? (uint64_t)codes[T[p + q]] : 0ull;
                key = (key << bits) | c;
            }
            key |= (uint64_t)s << (K * bits);
            keys[p] = key;
            vals[p] = (uint32_t)(p + s);
        }
        radix_hist_add(sh, key, ok, passes, end_bit);
    }
    __syncthreads();
    radix_hist_flush(sh, passes, hist);
}

// Per-string outputs from the batched rows: SA relative to the string start,
// BWT in libsais_bwt's layout and the primary index of every string.
// Bytes per row: SA 4 read + 4 gathered, T 1 gathered; SA 4 + U 1 written.
template <typename Sym>
__global__ void __launch_bounds__(256) k_batch_outputs(const uint32_t *__restrict__ SA, const uint32_t *__restrict__ isa1,
                                                       const Sym *__restrict__ T, uint64_t n,
                                                       const uint64_t *__restrict__ offs, uint32_t count,
                                                       int32_t *__restrict__ sa_out, Sym *__restrict__ U,
                                                       int32_t *__restrict__ primary, uint32_t *__restrict__ err)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride) {
        const uint32_t s = string_of(offs, count, r);
        const uint64_t base = offs[s], len = offs[s + 1] - base, gs = base + s;
        const uint64_t k = r - base;
        const uint64_t g = SA[r];
        if (g < gs || g >= gs + len) {
            atomicOr(err, GSAIS_ERR_BOUNDS);
            continue;
        }
        sa_out[r] = (int32_t)(g - gs);
        const uint64_t i0 = (uint64_t)isa1[gs] - 1 - base;   // row of the string's suffix 0
        if (k == 0) {
            U[r] = T[base + len - 1];
            primary[s] = (int32_t)(i0 + 1);
        } else {
            const uint64_t row = k <= i0 ? k - 1 : k;
            const uint64_t p = (uint64_t)SA[base + row] - gs;
            if (p == 0 || p >= len) {
                atomicOr(err, GSAIS_ERR_BOUNDS);
                continue;
            }
            U[r] = T[base + p - 1];
        }
    }
}

// rank[pos[j]] = r[j] for a list partitioned by the high bits of pos, so
// the writes of each stretch land in one L2-resident window of rank[] and
// reach DRAM as whole sectors.  Bytes per entry: 8 read, 4 written.
__global__ void __launch_bounds__(256) k_scatter_ranks(const uint32_t *__restrict__ pos,
                                                       const uint32_t *__restrict__ r, uint64_t N, uint64_t nr,
                                                       uint32_t *__restrict__ rank, uint32_t *__restrict__ err)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < N; j += stride) {
        const uint32_t p = pos[j];
        if (p >= nr) {
            atomicOr(err, GSAIS_ERR_BOUNDS);
            continue;
        }
        rank[p] = r[j];
    }
}


// Packed dense codes of the text: PB bits per symbol, symbol j at bits
// PB * (j % (64 / PB)) of 64-bit word j / (64 / PB).
struct PackedWords {
    const uint64_t *w;
    uint64_t nwords;   // readable words (indexes are clamped to the last one)
};


// Orders the tied pairs (two-member groups of the seed round, and tied pairs
// found by k_small_groups) by comparing the two suffixes directly on the
// packed codes, from offset `skip` (a prefix both are known to share) on:
// the first differing code decides, and when one suffix ends inside the
// common part the shorter one is smaller (the implicit sentinel of libsais,
// src/libsais.c:7018).  One lane per pair; a step aligns 4 * kPairBlocks
// 32-bit words per side with word selects and funnel shifts from aligned
// 16-byte blocks, and loads the blocks the following step needs.  A lane
// whose pair is done idles until a quarter of its warp is idle; those lanes
// then take their next pairs together from a global cursor, so the refill
// code runs rarely and work stays balanced.  A pair still equal after
// `limit` more symbols goes back to the active list as a two-member group.
constexpr int kPairBlocks = 2;   // 16-byte blocks per side per step (3 and 4 measured no faster)

struct PairSide {
    uint4 prev;               // block holding the window's first word
    uint4 next[kPairBlocks];  // the blocks after it, loaded one step ahead
    uint32_t q;               // next block to load
    uint32_t d;               // word offset of the window inside the first block
    int sh;                   // bit offset of the window inside its first word
};

// The 4 * kPairBlocks words of the window (aligned with word selects and
// funnel shifts); loads the blocks of the following step.
__device__ __forceinline__ void pair_window(const uint4 *__restrict__ W4, uint32_t last4, PairSide &s,
                                            uint32_t out[4 * kPairBlocks])
{
    constexpr int NW = 4 + 4 * kPairBlocks;
    uint32_t w[NW];
    w[0] = s.prev.x;
    w[1] = s.prev.y;
    w[2] = s.prev.z;
    w[3] = s.prev.w;
#pragma unroll
    for (int b = 0; b < kPairBlocks; ++b) {
        w[4 + 4 * b] = s.next[b].x;
        w[5 + 4 * b] = s.next[b].y;
        w[6 + 4 * b] = s.next[b].z;
        w[7 + 4 * b] = s.next[b].w;
    }
    s.prev = s.next[kPairBlocks - 1];
#pragma unroll
    for (int b = 0; b < kPairBlocks; ++b) {
        const uint32_t q = s.q + b;
        s.next[b] = W4[q < last4 ? q : last4];   // prefetch for the following step
    }
    s.q += kPairBlocks;
    uint32_t u[NW - 2], e[NW - 3];
#pragma unroll
    for (int i = 0; i < NW - 2; ++i) u[i] = (s.d & 2) ? w[i + 2] : w[i];
#pragma unroll
    for (int i = 0; i < NW - 3; ++i) e[i] = (s.d & 1) ? u[i + 1] : u[i];
#pragma unroll
    for (int i = 0; i < 4 * kPairBlocks; ++i) out[i] = __funnelshift_r(e[i], e[i + 1], s.sh);
}

template <int PB>
__global__ void __launch_bounds__(256) k_pair_compare(const uint32_t *__restrict__ pairs,
                                                      const unsigned long long *__restrict__ pair_count,
                                                      unsigned long long *__restrict__ cursor, PackedWords pw,
                                                      uint64_t n, uint64_t skip, uint32_t limit,
                                                      uint32_t *__restrict__ sa, uint32_t *__restrict__ rank,
                                                      uint32_t *__restrict__ list_pos,
                                                      uint32_t *__restrict__ list_rank,
                                                      uint32_t *__restrict__ slot0,
                                                      uint32_t *__restrict__ out_i, uint32_t *__restrict__ out_pos,
                                                      uint32_t *__restrict__ out_gid,
                                                      uint32_t *__restrict__ gstart_out,
                                                      unsigned long long *__restrict__ counter,
                                                      uint32_t *__restrict__ err)
{
    constexpr uint32_t SPW = 32 / PB;   // symbols per 32-bit word
    constexpr uint32_t STEP = 4 * kPairBlocks * SPW;
    constexpr uint32_t CM = (1u << PB) - 1;
    const uint64_t count = *pair_count;
    const uint4 *W4 = reinterpret_cast<const uint4 *>(pw.w);
    const uint32_t last4 = (uint32_t)(pw.nwords / 2 - 1);
    const int lane = threadIdx.x & 31;

    bool live = false, finished = false, at_end = false;
    uint32_t P = 0, a = 0, b = 0, rem = 0;   // rem: symbols left before `stop`
    PairSide A{}, B{};
    auto init_side = [&](PairSide &s, uint64_t x) {
        const uint64_t q = x / SPW;   // word holding symbol x
        s.d = (uint32_t)(q & 3);
        s.sh = (int)(x % SPW) * PB;
        const uint32_t q4 = (uint32_t)(q >> 2);
        s.prev = W4[q4 < last4 ? q4 : last4];
#pragma unroll
        for (int b = 0; b < kPairBlocks; ++b) s.next[b] = W4[q4 + 1 + b < last4 ? q4 + 1 + b : last4];
        s.q = q4 + 1 + kPairBlocks;
    };
    while (true) {
        const uint32_t busy = __ballot_sync(GSAIS_FULL_MASK, live);
        const uint32_t needy = __ballot_sync(GSAIS_FULL_MASK, !live && !finished);
        if (busy == 0 && needy == 0) break;
        if (needy && (busy == 0 || __popc(needy) >= 8)) {
            unsigned long long base = 0;
            if (lane == __ffs(needy) - 1) base = atomicAdd(cursor, (unsigned long long)__popc(needy));
            base = __shfl_sync(GSAIS_FULL_MASK, base, __ffs(needy) - 1);
            if (!live && !finished) {
                const uint64_t jj = base + __popc(needy & lanemask_lt());
                if (jj >= count) {
                    finished = true;
                } else {
                    P = pairs[jj];
                    const bool okp = (uint64_t)P + 1 < n;
                    a = okp ? sa[P] : 0u;
                    b = okp ? sa[P + 1] : 0u;
                    if (okp && a < n && b < n && a != b) {
                        const uint64_t la = n - a, lb = n - b;
                        const uint64_t minlen = la < lb ? la : lb;
                        const uint64_t stop = minlen < skip + limit ? minlen : skip + limit;
                        at_end = stop == minlen;
                        rem = (uint32_t)(stop - skip);
                        init_side(A, a + skip);
                        init_side(B, b + skip);
                        live = true;
                    } else {
                        atomicOr(err, GSAIS_ERR_BOUNDS);
                    }
                }
            }
            continue;
        }
        if (!live) continue;
        int res = 0;   // -1: a smaller, 1: b smaller, 2: equal up to `limit`, 0: go on
        const int end_res = at_end ? ((n - a) < (n - b) ? -1 : 1) : 2;
        if (rem == 0) {
            res = end_res;
        } else {
            uint32_t va[4 * kPairBlocks], vb[4 * kPairBlocks];
            pair_window(W4, last4, A, va);
            pair_window(W4, last4, B, vb);
            uint32_t x = 0, wa = 0, wb = 0, wi = 4 * kPairBlocks;
#pragma unroll
            for (int i = 4 * kPairBlocks - 1; i >= 0; --i) {
                const uint32_t xi = va[i] ^ vb[i];
                if (xi) { x = xi; wa = va[i]; wb = vb[i]; wi = i; }
            }
            if (x) {
                const uint32_t bit = (uint32_t)__ffs(x) - 1;
                const uint32_t sym = wi * SPW + bit / PB;
                if (sym < rem) {
                    const int f = (int)(bit / PB * PB);
                    res = ((wa >> f) & CM) < ((wb >> f) & CM) ? -1 : 1;
                } else {
                    res = end_res;
                }
            } else if (rem <= STEP) {
                res = end_res;
            } else {
                rem -= STEP;
            }
        }
        if (res == 0) continue;
        if (res != 2) {
            const uint32_t lo = res < 0 ? a : b, hi = res < 0 ? b : a;
            sa[P] = lo;
            sa[P + 1] = hi;
            if (slot0 && (lo == 0 || hi == 0)) *slot0 = P + (lo == 0 ? 1u : 2u);
            if (list_rank) {   // seed ranks not scattered yet: order the pair in the SA-order list
                list_pos[P] = lo;
                list_pos[P + 1] = hi;
                list_rank[P + 1] = P + 2;
            } else {
                rank[lo] = P + 1;
                rank[hi] = P + 2;
            }
        } else {
            const unsigned long long r = atomicAdd(counter, (1ull << 32) | 2ull);
            const uint32_t cc = (uint32_t)r, g = (uint32_t)(r >> 32);
            out_i[cc] = a;
            out_i[cc + 1] = b;
            out_pos[cc] = P;
            out_pos[cc + 1] = P + 1;
            out_gid[cc] = g;
            out_gid[cc + 1] = g;
            gstart_out[g] = cc;
        }
        live = false;
    }
}

// ---- inverse permutation of the seed round: rank[pos[j]] = r[j] where pos
// is a permutation of [0, N).  Two unstable partitions by the high bits of
// pos (8 bits, then 8 more) leave every 2^shift2 consecutive positions in one
// contiguous bucket of exactly that many entries; one CTA then scatters its
// bucket into a shared-memory window and writes the window out coalesced.
// Each level reads and writes 8 bytes per entry; the window pass reads 8 and
// writes 4.  No random access reaches DRAM or L2.
constexpr int kPermItems = 16;
constexpr int kPermThreads = 512;
constexpr int kPermTile = kPermThreads * kPermItems;   // 8192: runs of ~32 entries per digit
constexpr size_t kPermSmem = (size_t)2 * kPermTile * sizeof(uint32_t);

__global__ void k_perm_cursors(uint32_t *__restrict__ cursor, uint32_t count, int shift, uint64_t N)
{
    const uint32_t d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d < count) {
        const uint64_t s = (uint64_t)d << shift;
        cursor[d] = (uint32_t)(s < N ? s : N);
    }
}

// One partition level.  digit(p) = p >> shift; a tile's digits lie in
// [lbase, lbase + RANGE) where lbase = (p0 >> lshift) << (lshift - shift) for
// the tile's first position p0 (lshift = 0: lbase = 0).  Entries land at
// cursor[digit]++ (order inside a digit is not kept: the scatter after the
// last level does not need it).  PHI: the value of entry j is not read from
// in_r but is in_pos[j - 1] (N for j = 0), the Phi array of a suffix array
// (libsais src/libsais.c:8116 compute_phi: Phi[SA[j]] = SA[j-1]).
template <int RANGE, bool PHI = false>
__global__ void __launch_bounds__(kPermThreads) k_perm_partition(const uint32_t *__restrict__ in_pos,
                                                                 const uint32_t *__restrict__ in_r, uint64_t N,
                                                                 int shift, int lshift,
                                                                 uint32_t *__restrict__ cursor, uint32_t ncursor,
                                                                 uint32_t *__restrict__ out_pos,
                                                                 uint32_t *__restrict__ out_r,
                                                                 uint32_t *__restrict__ err)
{
    constexpr int THREADS = kPermThreads;
    constexpr int PER = (RANGE + THREADS - 1) / THREADS;   // digits per thread in the scan
    extern __shared__ uint32_t s_dyn[];
    uint32_t *s_pos = s_dyn, *s_r = s_dyn + kPermTile;
    __shared__ uint32_t s_cnt[RANGE], s_lstart[RANGE], s_g[RANGE];
    __shared__ uint32_t s_scan[THREADS / 32 + 1];
    const int tid = threadIdx.x;
    const uint64_t t0 = (uint64_t)blockIdx.x * kPermTile;
    const uint32_t valid = (uint32_t)(N - t0 < (uint64_t)kPermTile ? N - t0 : (uint64_t)kPermTile);
    for (int i = tid; i < RANGE; i += THREADS) s_cnt[i] = 0;
    const uint32_t lbase = lshift ? ((in_pos[t0] >> lshift) << (lshift - shift)) : 0u;
    __syncthreads();
    uint32_t p[kPermItems], r[kPermItems];
    uint16_t slot[kPermItems];
    bool bad = false;
    // all loads of the tile first, then the shared-memory slot counters
#pragma unroll
    for (int k = 0; k < kPermItems; ++k) {
        const uint32_t i = k * THREADS + tid;
        p[k] = i < valid ? in_pos[t0 + i] : 0xFFFFFFFFu;
        if (PHI)
            r[k] = i < valid ? (t0 + i ? in_pos[t0 + i - 1] : (uint32_t)N) : 0u;
        else
            r[k] = i < valid ? in_r[t0 + i] : 0u;
    }
#pragma unroll
    for (int k = 0; k < kPermItems; ++k) {
        if (p[k] != 0xFFFFFFFFu) {
            const uint32_t ld = (p[k] >> shift) - lbase;
            if (ld < RANGE && (uint64_t)lbase + ld < ncursor) {
                slot[k] = (uint16_t)atomicAdd(&s_cnt[ld], 1u);
            } else {
                bad = true;
                p[k] = 0xFFFFFFFFu;
            }
        }
    }
    __syncthreads();
    // exclusive scan of the digit counts; reserve each digit's run globally
    uint32_t c[PER], sum = 0;
#pragma unroll
    for (int q = 0; q < PER; ++q) {
        const uint32_t ld = tid * PER + q;
        c[q] = ld < RANGE ? s_cnt[ld] : 0u;
        sum += c[q];
    }
    uint32_t total;
    uint32_t a = block_exclusive_sum<uint32_t, THREADS>(sum, s_scan, total);
#pragma unroll
    for (int q = 0; q < PER; ++q) {
        const uint32_t ld = tid * PER + q;
        if (ld < RANGE) {   // c[q] > 0 only for digits whose cursor exists
            s_lstart[ld] = a;
            s_g[ld] = c[q] ? atomicAdd(&cursor[lbase + ld], c[q]) : 0u;
        }
        a += c[q];
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kPermItems; ++k) {
        if (p[k] != 0xFFFFFFFFu) {
            const uint32_t ld = (p[k] >> shift) - lbase;
            const uint32_t o = s_lstart[ld] + slot[k];
            s_pos[o] = p[k];
            s_r[o] = r[k];
        }
    }
    __syncthreads();
    const uint32_t kept = total;
    for (uint32_t i = tid; i < kept; i += THREADS) {
        const uint32_t q = s_pos[i];
        const uint32_t ld = (q >> shift) - lbase;
        const uint64_t o = (uint64_t)s_g[ld] + (i - s_lstart[ld]);
        if (o < N) {
            out_pos[o] = q;
            out_r[o] = s_r[i];
        } else {
            bad = true;
        }
    }
    if (bad) atomicOr(err, GSAIS_ERR_BOUNDS);
}

// Bucket b holds exactly the positions [b << shift, (b + 1) << shift).
__global__ void __launch_bounds__(256) k_perm_window(const uint32_t *__restrict__ pos, const uint32_t *__restrict__ r,
                                                     uint64_t N, int shift, uint32_t *__restrict__ rank,
                                                     uint32_t *__restrict__ err)
{
    extern __shared__ uint32_t s_win[];
    const uint64_t w0 = (uint64_t)blockIdx.x << shift;
    const uint32_t W = (uint32_t)(N - w0 < (1ull << shift) ? N - w0 : (1ull << shift));
    bool bad = false;
    for (uint32_t i = threadIdx.x; i < W; i += 256) {
        const uint32_t q = pos[w0 + i];
        const uint64_t x = (uint64_t)q - w0;
        if (q >= w0 && x < W) s_win[x] = r[w0 + i];
        else bad = true;
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < W; i += 256) rank[w0 + i] = s_win[i];
    if (bad) atomicOr(err, GSAIS_ERR_BOUNDS);
}

// Window pass of the Phi permutation: like k_perm_window, but `out` may be
// the same buffer as `r` (each CTA reads its whole window before writing it).
__global__ void __launch_bounds__(256) k_phi_window(const uint32_t *__restrict__ pos, const uint32_t *r, uint64_t N,
                                                    int shift, uint32_t *out, uint32_t *__restrict__ err)
{
    extern __shared__ uint32_t s_win[];
    const uint64_t w0 = (uint64_t)blockIdx.x << shift;
    const uint32_t W = (uint32_t)(N - w0 < (1ull << shift) ? N - w0 : (1ull << shift));
    bool bad = false;
    for (uint32_t i = threadIdx.x; i < W; i += 256) {
        const uint32_t q = pos[w0 + i];
        const uint64_t x = (uint64_t)q - w0;
        if (q >= w0 && x < W) s_win[x] = r[w0 + i];
        else bad = true;
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < W; i += 256) out[w0 + i] = s_win[i];
    if (bad) atomicOr(err, GSAIS_ERR_BOUNDS);
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
    s += 4 * align_up((n / 2 + 2) * 4, A);         // gstart x2, lid, loff (at most n/2 groups are active)
    s += 3 * align_up(n * 4, A);                   // large list: values x2, slots
    s += align_up(8 * 8, A);                       // round counters
    s += 2 * align_up(tiles * 16, A);              // tile info + carry
    s += align_up((2 * (tiles / kScanSpan) + 4) * 16, A);   // tile-scan aggregates + their prefixes
    s += align_up((tiles * kAssignTile / 32 + 2) * 4, A);   // head bits of the assign tiles
    s += align_up(16 * 4, A);                      // totals
    s += align_up(65536 * 4, A);                   // hist
    s += align_up(65536 * 2, A);                   // codes
    s += align_up((n + kSeedTile - 1) / kSeedTile * (kSeedTile / 2) + 16, A);   // packed codes (<= 4 bits each)
    s += 2 * align_up(8 * 256 * 4, A);             // radix hist + bases
    s += align_up(8 * 4, A);                       // radix counters
    s += align_up(radix_status_words(n) * 8, A);   // radix tile counts + offsets
    s += align_up(few_scratch_bytes(n), A);         // large groups with few differing members
    s += align_up(sg_tile_words(n) * 4, A);         // small-group tiles of a round
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
    for (int i = 0; i < 2; ++i) ws.gstart[i] = reinterpret_cast<uint32_t *>(take((n / 2 + 2) * 4));
    ws.lid = reinterpret_cast<uint32_t *>(take((n / 2 + 2) * 4));
    ws.loff = reinterpret_cast<uint32_t *>(take((n / 2 + 2) * 4));
    for (int i = 0; i < 2; ++i) ws.lvals[i] = reinterpret_cast<uint32_t *>(take(n * 4));
    ws.lpos = reinterpret_cast<uint32_t *>(take(n * 4));
    ws.counters = reinterpret_cast<unsigned long long *>(take(8 * 8));
    ws.slot0 = reinterpret_cast<uint32_t *>(ws.counters + 7);
    ws.tile_info = reinterpret_cast<uint32_t *>(take(tiles * 16));
    ws.tile_carry = reinterpret_cast<uint32_t *>(take(tiles * 16));
    ws.tile_agg = reinterpret_cast<uint32_t *>(take((2 * (tiles / kScanSpan) + 4) * 16));
    ws.heads = reinterpret_cast<uint32_t *>(take((tiles * kAssignTile / 32 + 2) * 4));
    ws.totals = reinterpret_cast<uint32_t *>(take(16 * 4));
    ws.hist = reinterpret_cast<uint32_t *>(take(65536 * 4));
    ws.codes = reinterpret_cast<uint16_t *>(take(65536 * 2));
    ws.packed = reinterpret_cast<uint8_t *>(take((n + kSeedTile - 1) / kSeedTile * (kSeedTile / 2) + 16));
    ws.pack_bits = 0;
    ws.radix.hist = reinterpret_cast<uint32_t *>(take(8 * 256 * 4));
    ws.radix.bases = reinterpret_cast<uint32_t *>(take(8 * 256 * 4));
    ws.radix.counters = reinterpret_cast<uint32_t *>(take(8 * 4));
    ws.radix.status_words = radix_status_words(n);
    ws.radix.status = reinterpret_cast<uint64_t *>(take(ws.radix.status_words * 8));
    ws.few = reinterpret_cast<uint32_t *>(take(few_scratch_bytes(n)));
    ws.sg_tiles = reinterpret_cast<uint32_t *>(take(sg_tile_words(n) * 4));
    ws.n_cap = n;
    ws.radix.h_hist = h_hist;
    ws.h_small = h_small;
}

static int grid_for(uint64_t items, int per_block)
{
    const uint64_t g = (items + per_block - 1) / per_block;
    return (int)(g ? g : 1);
}

// Sets the bit of every listed SA slot.  Bytes per slot: 4 read, one L2 atomic.
__global__ void __launch_bounds__(256) k_mark_slots(const uint32_t *__restrict__ slots, uint64_t m, uint64_t n,
                                                    uint32_t *__restrict__ bits)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < m; j += stride) {
        const uint64_t s = slots[j];
        if (s < n) atomicOr(&bits[s >> 5], 1u << (s & 31));
    }
}

// host[slot] = sa[slot] for the marked slots, in address order: each warp
// reads 32 bitmap words at once and takes the non-zero ones in turn, a lane
// per slot of the word, so a run of marked slots leaves as one coalesced
// write over the host link.  Bytes: n / 8 read, 8 per marked slot.
__global__ void __launch_bounds__(256) k_sa_patch(const uint32_t *__restrict__ bits, uint64_t words,
                                                  const uint32_t *__restrict__ sa, uint64_t n,
                                                  int32_t *__restrict__ host)
{
    const int lane = threadIdx.x & 31;
    const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x >> 5);
    for (uint64_t base = ((uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 32; base < words;
         base += warps * 32) {
        const uint32_t m = base + lane < words ? bits[base + lane] : 0u;
        uint32_t nz = __ballot_sync(GSAIS_FULL_MASK, m != 0);
        while (nz) {
            const int l = __ffs(nz) - 1;
            nz &= nz - 1;
            const uint32_t mw = __shfl_sync(GSAIS_FULL_MASK, m, l);
            const uint64_t slot = (base + (uint64_t)l) * 32 + (uint64_t)lane;
            if (((mw >> lane) & 1u) && slot < n) host[slot] = (int32_t)sa[slot];
        }
    }
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

// Grid of one full wave of resident CTAs, capped at `items`.
template <typename Kernel>
static unsigned resident_grid(Kernel kernel, int threads, uint64_t items)
{
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, threads, 0);
    const uint64_t cap = (uint64_t)sms * (per > 0 ? per : 1);
    return (unsigned)(items < cap ? (items ? items : 1) : cap);
}

template <int MODE>
static cudaError_t run_assign(const TileArgs &a, SortWorkspace &ws, uint32_t *out_i, uint32_t *out_pos,
                              uint32_t *out_gid, uint32_t *gstart_out, const unsigned long long *base,
                              cudaStream_t st, uint32_t *kept, uint32_t *groups, const TailSource *tails = nullptr)
{
    const uint64_t tiles = (a.N + kAssignTile - 1) / kAssignTile;
    KernelProfiler *prof = ws.radix.prof;
    cudaEvent_t ev = prof ? prof->begin(st) : nullptr;
    const uint64_t words = (a.N + 31) / 32;
    const uint64_t hsteps = (words + 31) / 32;   // 8 warps x 4 words per block step
    GSAIS_COUNTED((k_heads<MODE><<<(unsigned)(hsteps < (1u << 16) ? (hsteps ? hsteps : 1) : (1u << 16)), 256, 0, st>>>(
        a, ws.heads)));
    if (MODE == MODE_INIT_PLAIN && tails && tails->T && a.K > 1) {
        if (tails->symbytes == 1)
            GSAIS_COUNTED((k_tail_heads<uint8_t><<<1, 64, 0, st>>>(static_cast<const uint8_t *>(tails->T), a.n,
                                                                 tails->codes, tails->bits, a, ws.heads)));
        else if (tails->symbytes == 2)
            GSAIS_COUNTED((k_tail_heads<uint16_t><<<1, 64, 0, st>>>(static_cast<const uint16_t *>(tails->T), a.n,
                                                                  tails->codes, tails->bits, a, ws.heads)));
        else
            GSAIS_COUNTED((k_tail_heads<uint32_t><<<1, 64, 0, st>>>(static_cast<const uint32_t *>(tails->T), a.n,
                                                                  tails->codes, tails->bits, a, ws.heads)));
    }
    GSAIS_COUNTED((k_tile_summary<MODE><<<(unsigned)((tiles + 7) / 8), 256, 0, st>>>(a, ws.heads, ws.tile_info)));
    if (ev) prof->end(KK_SUMMARY, ev, st, a.N * (MODE == MODE_ROUND ? 12 : 16));
    ev = prof ? prof->begin(st) : nullptr;   // the tile scan is timed with the assign
    if (tiles <= 4 * (uint64_t)kScanSpan) {
        GSAIS_COUNTED((k_tile_scan<<<1, 1024, 0, st>>>(ws.tile_info, ws.tile_carry, tiles, ws.totals, base,
                                                       a.pairs ? a.pair_count : nullptr)));
    } else {
        const uint32_t blocks = (uint32_t)((tiles + kScanSpan - 1) / kScanSpan);
        uint4 *agg = reinterpret_cast<uint4 *>(ws.tile_agg);
        GSAIS_COUNTED((k_scan_up<<<blocks, kScanThreads, 0, st>>>(ws.tile_info, tiles, agg)));
        GSAIS_COUNTED((k_scan_top<<<1, 1024, 0, st>>>(agg, blocks, ws.totals, base,
                                                      a.pairs ? a.pair_count : nullptr)));
        GSAIS_COUNTED((k_scan_down<<<blocks, kScanThreads, 0, st>>>(ws.tile_info, tiles, agg + blocks,
                                                                    ws.tile_carry)));
    }
    GSAIS_COUNTED((k_assign<MODE><<<(unsigned)tiles, kAssignThreads, 0, st>>>(
        a, ws.tile_carry, ws.heads, ws.rank, ws.sa, out_i, out_pos, out_gid, gstart_out)));
    // algorithmic bytes: key 8 + value 4 + slot 4 read, rank 4 scattered, and
    // 4 (SA) or 12 (survivor lists) written -- counted as 28 per entry
    if (ev) prof->end(KK_ASSIGN, ev, st, a.N * 28);
    cudaError_t e = read_back(ws.h_small, ws.totals, 2 * sizeof(uint32_t), st);
    if (e != cudaSuccess) return e;
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
    *kept = ws.h_small[0];
    *groups = ws.h_small[1];
    return cudaGetLastError();
}

// Seed round: for a large rank domain the new ranks are written by list
// position and then moved to text order without random writes into a rank
// array larger than L2.  When the list is a permutation of [0, nr) the
// three-level partition + shared-memory window scatter is used; otherwise
// (gapped batch coordinates) a stable radix partition by the top 8 position
// bits followed by a scatter inside L2-resident windows.
static bool use_two_level_ranks(uint64_t nr) { return nr >= (1ull << 23); }

static cudaError_t scatter_seed_ranks_impl(SortWorkspace &ws, uint32_t *sorted_pos, uint32_t *ranks, uint64_t N,
                                           uint64_t nr, uint32_t *d_err, cudaStream_t st);

// Timed as one kernel family: two partitions (16 bytes per entry each) and
// the window pass (12), or the radix partition and the windowed scatter.
static cudaError_t scatter_seed_ranks(SortWorkspace &ws, uint32_t *sorted_pos, uint32_t *ranks, uint64_t N,
                                      uint64_t nr, uint32_t *d_err, cudaStream_t st)
{
    KernelProfiler *prof = ws.radix.prof;
    cudaEvent_t ev = prof ? prof->begin(st) : nullptr;
    const cudaError_t e = scatter_seed_ranks_impl(ws, sorted_pos, ranks, N, nr, d_err, st);
    if (ev) prof->end(KK_PERM, ev, st, N * 44);
    return e;
}

static cudaError_t scatter_seed_ranks_impl(SortWorkspace &ws, uint32_t *sorted_pos, uint32_t *ranks, uint64_t N,
                                           uint64_t nr, uint32_t *d_err, cudaStream_t st)
{
    cudaError_t e;
    const int b = gsais_bits_for(nr - 1);
    const int shift1 = b - 8, shift2 = b - 16;
    if (N == nr && b >= 23 && shift2 <= 15) {
        // level 1: by bits [shift1, b) into lvals; level 2: by bits [shift2, b) back
        uint32_t *cur = reinterpret_cast<uint32_t *>(ws.radix.status);
        const uint64_t tiles = (N + kPermTile - 1) / kPermTile;
        const uint32_t n1 = (uint32_t)(((N - 1) >> shift1) + 1), n2 = (uint32_t)(((N - 1) >> shift2) + 1);
        if ((uint64_t)n1 + n2 > ws.radix.status_words * 2) return cudaErrorInvalidValue;
        GSAIS_COUNTED((k_perm_cursors<<<(n1 + 255) / 256, 256, 0, st>>>(cur, n1, shift1, N)));
        GSAIS_COUNTED((k_perm_cursors<<<(n2 + 255) / 256, 256, 0, st>>>(cur + n1, n2, shift2, N)));
        static bool attr_done[64] = {false};   // dynamic shared memory above 48 KB, per device
        int dev = 0;
        cudaGetDevice(&dev);
        if (dev < 0 || dev >= 64 || !attr_done[dev]) {
            if ((e = cudaFuncSetAttribute(k_perm_partition<256>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)kPermSmem)) != cudaSuccess ||
                (e = cudaFuncSetAttribute(k_perm_partition<512>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)kPermSmem)) != cudaSuccess)
                return e;
            if (dev >= 0 && dev < 64) attr_done[dev] = true;
        }
        GSAIS_COUNTED((k_perm_partition<256><<<(unsigned)tiles, kPermThreads, kPermSmem, st>>>(
            sorted_pos, ranks, N, shift1, 0, cur, n1, ws.lvals[0], ws.lvals[1], d_err)));
        GSAIS_COUNTED((k_perm_partition<512><<<(unsigned)tiles, kPermThreads, kPermSmem, st>>>(
            ws.lvals[0], ws.lvals[1], N, shift2, shift1, cur + n1, n2, sorted_pos, ranks, d_err)));
        const size_t smem = (size_t)4 << shift2;
        if (smem > 48 * 1024 &&
            (e = cudaFuncSetAttribute(k_perm_window, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) !=
                cudaSuccess)
            return e;
        GSAIS_COUNTED((k_perm_window<<<n2, 256, smem, st>>>(sorted_pos, ranks, N, shift2, ws.rank, d_err)));
        return cudaGetLastError();
    }
    const int bb = gsais_bits_for(nr);
    uint32_t *kk[2] = {sorted_pos, ws.lvals[0]};
    uint32_t *vv[2] = {ranks, ws.lvals[1]};
    int which = 0;
    e = radix_partition32(kk, vv, N, bb > 8 ? bb - 8 : 0, bb, ws.radix, d_err, st, &which);
    if (e != cudaSuccess) return e;
    GSAIS_COUNTED((k_scatter_ranks<<<stream_grid(N, 256), 256, 0, st>>>(kk[which], vv[which], N, nr, ws.rank,
                                                                        d_err)));
    return cudaGetLastError();
}

// Phi[SA[j]] = SA[j-1] (Phi[SA[0]] = N) for a suffix array SA of N entries,
// by two position partitions and a shared-memory window pass, so that no
// random write reaches DRAM.  Scratch: phi_scratch_words(N) words.
bool phi_partitioned(uint64_t N)
{
    if (N < (1ull << 23)) return false;
    const int b = gsais_bits_for(N - 1);
    return b - 16 <= 15;
}

// Cursor words: 256 for the first level, and for the second level every
// index a tile can name (digits below 256 << 8 plus a 512-digit range), so
// that even entries of a malformed SA stay inside the scratch.
constexpr size_t kPhiCursorWords = 256 + (256 << 8) + 512;

size_t phi_scratch_words(uint64_t N)
{
    if (!phi_partitioned(N)) return 0;
    return (size_t)3 * ((N + 63) / 64 * 64) + kPhiCursorWords;
}

cudaError_t phi_permute(const uint32_t *SA, uint64_t N, uint32_t *phi, uint32_t *scratch, uint32_t *d_err,
                        cudaStream_t st)
{
    cudaError_t e;
    const int b = gsais_bits_for(N - 1);
    const int shift1 = b - 8, shift2 = b - 16;
    const uint64_t Np = (N + 63) / 64 * 64;
    uint32_t *X = scratch, *Y = scratch + Np, *Z = scratch + 2 * Np, *cur = scratch + 3 * Np;
    const uint64_t tiles = (N + kPermTile - 1) / kPermTile;
    const uint32_t n2 = (uint32_t)(((N - 1) >> shift2) + 1);
    // level-1 cursors at cur[0, 256), level-2 cursors from cur + 256
    GSAIS_COUNTED((k_perm_cursors<<<1, 256, 0, st>>>(cur, 256, shift1, N)));
    GSAIS_COUNTED((k_perm_cursors<<<(unsigned)((kPhiCursorWords - 256 + 255) / 256), 256, 0, st>>>(
        cur + 256, (uint32_t)(kPhiCursorWords - 256), shift2, N)));
    static bool attr_done[64] = {false};   // dynamic shared memory above 48 KB, per device
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64 || !attr_done[dev]) {
        if ((e = cudaFuncSetAttribute(k_perm_partition<256, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)kPermSmem)) != cudaSuccess ||
            (e = cudaFuncSetAttribute(k_perm_partition<512>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)kPermSmem)) != cudaSuccess)
            return e;
        if (dev >= 0 && dev < 64) attr_done[dev] = true;
    }
    GSAIS_COUNTED((k_perm_partition<256, true><<<(unsigned)tiles, kPermThreads, kPermSmem, st>>>(
        SA, nullptr, N, shift1, 0, cur, 256u, X, Y, d_err)));
    GSAIS_COUNTED((k_perm_partition<512><<<(unsigned)tiles, kPermThreads, kPermSmem, st>>>(
        X, Y, N, shift2, shift1, cur + 256, (uint32_t)(kPhiCursorWords - 256), Z, phi, d_err)));
    const size_t smem = (size_t)4 << shift2;
    if (smem > 48 * 1024 &&
        (e = cudaFuncSetAttribute(k_phi_window, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) !=
            cudaSuccess)
        return e;
    GSAIS_COUNTED((k_phi_window<<<n2, 256, smem, st>>>(Z, phi, N, shift2, phi, d_err)));
    return cudaGetLastError();
}

// Doubling rounds over the kept groups of the seed round until every suffix
// is final.  nr = length of the rank domain (rank[nr] is the sentinel).
// Tied pairs are ordered by direct comparison when the packed codes of the
// text are available (single text, at most 16 symbols).
struct PairSource {
    int pack_bits = 0;   // 0: no direct comparison
    PackedWords words{nullptr, 0};
    uint64_t n = 0;
};
constexpr uint32_t kPairLimit = 1u << 16;   // symbols compared beyond the shared prefix

// Orders the pairs listed in `pairs` (count in counters[3], cursor
// counters[4]); members share `skip` symbols.  Unresolved pairs are appended
// to the out lists behind the reservation counter counters[0].
// list_pos/list_rank (seed round with two-level ranks): the SA-order list of
// (position, rank) not yet scattered into rank[]; the pair's order goes there.
static cudaError_t run_pair_compare(SortWorkspace &ws, const PairSource &ps, const uint32_t *pairs, uint64_t max_pairs,
                                    uint64_t skip, uint32_t *out_i, uint32_t *out_pos, uint32_t *out_gid,
                                    uint32_t *gstart_out, uint32_t *d_err, cudaStream_t st,
                                    uint32_t *list_pos = nullptr, uint32_t *list_rank = nullptr,
                                    uint32_t *slot0 = nullptr)
{
    unsigned long long *pair_count = ws.counters + 3;
    cudaEvent_t ev_pc = ws.radix.prof ? ws.radix.prof->begin(st) : nullptr;
    const unsigned grid = (unsigned)stream_grid(max_pairs, 256);
    if (ps.pack_bits == 2)
        GSAIS_COUNTED((k_pair_compare<2><<<grid, 256, 0, st>>>(pairs, pair_count, ws.counters + 4, ps.words, ps.n,
                                                              skip, kPairLimit, ws.sa, ws.rank, list_pos, list_rank,
                                                              slot0, out_i, out_pos, out_gid, gstart_out, ws.counters, d_err)));
    else
        GSAIS_COUNTED((k_pair_compare<4><<<grid, 256, 0, st>>>(pairs, pair_count, ws.counters + 4, ps.words, ps.n,
                                                              skip, kPairLimit, ws.sa, ws.rank, list_pos, list_rank,
                                                              slot0, out_i, out_pos, out_gid, gstart_out, ws.counters, d_err)));
    if (ev_pc) ws.radix.prof->end(KK_PAIRS, ev_pc, st, 0);
    return cudaGetLastError();
}

// The large groups of a round (NL members in LG groups, large list in
// keys[0] / lvals[0]): if at most a quarter of the members differ from their
// group's candidate value, sorts only those and places the majority runs,
// leaving the sorted list in keys[1] / lvals[1] (*few = true).  The others
// and their sort use the active list's buffers, which the round has consumed.
static cudaError_t large_few_others(SortWorkspace &ws, uint64_t NL, uint64_t LG, int b2, int end_bit, uint64_t N,
                                    int av, int pg, uint32_t *d_err, cudaStream_t st, SortStats &S, bool *few)
{
    cudaError_t e;
    *few = false;
    const uint64_t GW = few_group_words(ws.n_cap), TW = few_tile_words(ws.n_cap);
    // the others and their sort live in halves of the active list's buffers
    if (LG + 1 > GW || N < 4096) return cudaSuccess;
    uint32_t *lstart = ws.few, *cand = lstart + GW, *less = cand + GW, *greater = less + GW, *ocum = greater + GW;
    uint32_t *tile_other = ocum + GW, *tile_off = tile_other + TW;
    const uint64_t ftiles = (NL + kFewTile - 1) / kFewTile;
    if (ftiles + 1 > TW) return cudaSuccess;
    KernelProfiler *prof = ws.radix.prof;
    cudaEvent_t ev = prof ? prof->begin(st) : nullptr;
    GSAIS_COUNTED((k_set_word<<<1, 1, 0, st>>>(lstart + LG, (uint32_t)NL)));
    if ((e = cudaMemsetAsync(less, 0, LG * 4, st)) != cudaSuccess ||
        (e = cudaMemsetAsync(greater, 0, LG * 4, st)) != cudaSuccess)
        return e;
    GSAIS_COUNTED((k_large_cand<<<(unsigned)((LG * 32 + 255) / 256), 256, 0, st>>>(ws.keys[0], lstart, LG, b2, cand)));
    GSAIS_COUNTED((k_large_count<<<(unsigned)ftiles, 256, 0, st>>>(ws.keys[0], NL, LG, b2, cand, less, greater,
                                                                  tile_other, d_err)));
    GSAIS_COUNTED((k_scan_counts<<<1, 1024, 0, st>>>(tile_other, nullptr, ftiles, tile_off)));
    if ((e = read_back(ws.h_small, tile_off + ftiles, 4, st)) != cudaSuccess) return e;
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
    const uint64_t O = ws.h_small[0];
    if (ev) prof->end(KK_FEW, ev, st, NL * 8);
    if (O > NL / 4) return cudaSuccess;
    *few = true;
    ev = prof ? prof->begin(st) : nullptr;
    GSAIS_COUNTED((k_scan_counts<<<1, 1024, 0, st>>>(less, greater, LG, ocum)));
    const uint64_t half = (N / 2 + 63) & ~63ull;
    uint64_t *ok[2] = {reinterpret_cast<uint64_t *>(ws.pos[pg]), reinterpret_cast<uint64_t *>(ws.gid[pg])};
    uint32_t *ov[2] = {ws.vals[av], ws.vals[av] + half};
    GSAIS_COUNTED((k_large_place<<<(unsigned)ftiles, 256, 0, st>>>(ws.keys[0], ws.lvals[0], NL, LG, b2, cand, lstart,
                                                                  less,
                                                                  ocum, tile_off, ws.keys[1], ws.lvals[1], ok[0],
                                                                  ov[0], d_err)));
    if (ev) prof->end(KK_FEW, ev, st, NL * 24);
    if (O > 0) {
        int which = 0, ran = 0;
        if ((e = radix_sort_pairs(ok, ov, O, end_bit, ws.radix, d_err, st, &which, &ran, false)) != cudaSuccess)
            return e;
        S.radix_passes += ran;
        GSAIS_COUNTED((k_others_place<<<stream_grid(O, 256), 256, 0, st>>>(ok[which], ov[which], O, b2, lstart, less,
                                                                          greater, ocum, LG, ws.keys[1], ws.lvals[1],
                                                                          d_err)));
    }
    S.few_rounds += 1;
    return cudaGetLastError();
}

static cudaError_t run_rounds(SortWorkspace &ws, uint64_t nr, int K, uint32_t kept, uint32_t groups, int av, int pg,
                              uint32_t *d_err, cudaStream_t st, SortStats &S, const PairSource &ps, const Tuning &tn)
{
    const uint32_t medium_small = (uint32_t)(tn.medium_small < (int)kMediumSmall ? tn.medium_small : kMediumSmall);
    const uint32_t medium_max = (uint32_t)(tn.medium_max < (int)kMediumMax ? tn.medium_max : kMediumMax);
    // the large groups of the previous round took the few-others path: this
    // round's keys skip the digit histograms (a full sort counts its own)
    bool few_last = false;
    cudaError_t e;
    int ran = 0;
    const int b2 = gsais_bits_for(nr);
    uint64_t h = (uint64_t)K;
    while (kept > 0) {
        if (++S.rounds > 64) {
            uint32_t flag = GSAIS_ERR_ROUNDS;
            cudaMemcpyAsync(d_err, &flag, 4, cudaMemcpyHostToDevice, st);
            cudaStreamSynchronize(st);
            return cudaErrorUnknown;
        }
        S.active_total += kept;
        const uint64_t N = kept, G = groups;
        const int gb = gsais_bits_for(G > 1 ? G - 1 : 0);
        const int end_bit = b2 + gb;   // large ids < G: unused top digits are skipped by the sort
        const int passes = (end_bit + 7) / 8;
        uint32_t *act_i = ws.vals[av], *act_pos = ws.pos[pg], *act_gid = ws.gid[pg];
        uint32_t *out_i = ws.vals[av ^ 1], *out_pos = ws.pos[pg ^ 1], *out_gid = ws.gid[pg ^ 1];
        uint32_t *r2 = reinterpret_cast<uint32_t *>(ws.keys[1]);   // consumed before the large sort reuses keys[1]
        // counters: [0] small+medium output, [1] large list, [2] medium groups (<= kMediumSmall),
        // [3] tied pairs, [4] next tied pair to compare, [5] medium groups (> kMediumSmall)
        if ((e = cudaMemsetAsync(ws.counters, 0, 6 * sizeof(unsigned long long), st)) != cudaSuccess) return e;
        uint32_t *pairs = ps.pack_bits ? r2 + N : nullptr;   // after r2 in keys[1]: N/2 slots at most
        if ((e = cudaMemsetAsync(ws.radix.hist, 0, (size_t)passes * 256 * 4, st)) != cudaSuccess) return e;
        // the 256-entry tiles in which a small group starts: flags, then their list
        const uint64_t sg_tiles = (N + 255) / 256;
        uint32_t *tile_flags = ws.sg_tiles, *tile_list = ws.sg_tiles + sg_tile_words(ws.n_cap) / 2;
        if ((e = cudaMemsetAsync(tile_flags, 0, sg_tiles * 4, st)) != cudaSuccess ||
            (e = cudaMemsetAsync(ws.counters + 6, 0, sizeof(unsigned long long), st)) != cudaSuccess)
            return e;
        uint32_t *mlist = ws.lvals[1];   // free until the large sort's first pass
        uint32_t *mlist2 = ws.lvals[1] + N / 2;   // medium groups have > 32 members: N / 33 of each at most
        cudaEvent_t ev_cl = ws.radix.prof ? ws.radix.prof->begin(st) : nullptr;
        GSAIS_COUNTED((k_classify<<<stream_grid(G, 256), 256, 0, st>>>(ws.gstart[pg], G, N, ws.lid, ws.loff,
                                                                      ws.counters + 1, mlist, ws.counters + 2, mlist2,
                                                                      ws.counters + 5, medium_small, medium_max,
                                                                      ws.few, tile_flags)));
        if (ev_cl) ws.radix.prof->end(KK_CLASSIFY, ev_cl, st, G * 12);   // group table 8 read, class 4 written
        cudaEvent_t ev_rk = ws.radix.prof ? ws.radix.prof->begin(st) : nullptr;
        const int hist_passes = (tn.large_few_others && few_last) ? 0 : passes;
        GSAIS_COUNTED((k_round_r2<<<stream_grid(N, 256), 256, 0, st>>>(
            act_i, act_pos, act_gid, ws.gstart[pg], ws.lid, ws.loff, ws.rank, h, N, nr, b2, r2, ws.keys[0],
            ws.lvals[0], ws.lpos, d_err, hist_passes, end_bit, ws.radix.hist)));
        if (ev_rk) ws.radix.prof->end(KK_ROUND_KEYS, ev_rk, st, N * 28);
        cudaEvent_t ev_sm = ws.radix.prof ? ws.radix.prof->begin(st) : nullptr;
        GSAIS_COUNTED((k_collect_tiles<<<stream_grid(sg_tiles, 256), 256, 0, st>>>(tile_flags, sg_tiles, tile_list,
                                                                                   ws.counters + 6)));
        GSAIS_COUNTED((k_small_groups<<<resident_grid(k_small_groups, 256, sg_tiles), 256, 0, st>>>(
            act_i, act_pos, act_gid, r2, N, ws.rank, ws.sa, out_i, out_pos, out_gid, ws.gstart[pg ^ 1],
            ws.counters, pairs, ws.counters + 3, tile_list, ws.counters + 6)));
        if (ev_sm) ws.radix.prof->end(KK_SMALL, ev_sm, st, N * 32);
        // medium groups: one wave of resident CTAs, each looping over the
        // groups (their count is on the device)
        const uint64_t mg_max = G < N / (kSmallMax + 1) ? G : N / (kSmallMax + 1);
        cudaEvent_t ev_md = ws.radix.prof ? ws.radix.prof->begin(st) : nullptr;
        GSAIS_COUNTED((k_medium_groups<128, kMediumSmall>
                       <<<resident_grid(k_medium_groups<128, kMediumSmall>, 128, mg_max), 128, 0, st>>>(
            mlist, ws.counters + 2, ws.gstart[pg], G, N, act_i, act_pos, r2, ws.rank, ws.sa, out_i, out_pos, out_gid,
            ws.gstart[pg ^ 1], ws.counters)));
        GSAIS_COUNTED((k_medium_groups<256, kMediumMax>
                       <<<resident_grid(k_medium_groups<256, kMediumMax>, 256, mg_max), 256, 0, st>>>(
            mlist2, ws.counters + 5, ws.gstart[pg], G, N, act_i, act_pos, r2, ws.rank, ws.sa, out_i, out_pos, out_gid,
            ws.gstart[pg ^ 1], ws.counters)));
        if (ev_md) ws.radix.prof->end(KK_MEDIUM, ev_md, st, 0);   // bytes added once the member counts are read
        // members of a tied pair share 2h symbols: h by their group, h more by equal r2
        if (pairs && (e = run_pair_compare(ws, ps, pairs, N / 2, 2 * h, out_i, out_pos, out_gid, ws.gstart[pg ^ 1],
                                           d_err, st)) != cudaSuccess)
            return e;
        if ((e = read_back(ws.h_small, ws.counters, 6 * sizeof(unsigned long long), st)) != cudaSuccess) return e;
        if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
        const unsigned long long *hc = reinterpret_cast<const unsigned long long *>(ws.h_small);
        const unsigned long long small_tot = hc[0];
        const unsigned long long large_tot = hc[1];
        S.pairs_direct += hc[3];
        if (ws.radix.prof) {
            // medium members: r2 4 + index 4 + slot 4 read, rank 4 + SA or survivors 8 written
            ws.radix.prof->add_bytes(KK_MEDIUM, ((hc[2] >> 32) + (hc[5] >> 32)) * 24);
            // tied pairs: two slots and two indexes read, two ranks and two SA entries written
            ws.radix.prof->add_bytes(KK_PAIRS, hc[3] * 24);
        }
        const uint64_t NL = (uint32_t)large_tot;
        if (NL == 0) {
            kept = (uint32_t)small_tot;
            groups = (uint32_t)(small_tot >> 32);
        } else {
            const uint64_t LG = large_tot >> 32;
            const uint64_t* sorted_keys = nullptr;
            const uint32_t* sorted_vals = nullptr;
            bool few = false;
            if (tn.large_few_others && LG > 0) {
                if ((e = large_few_others(ws, NL, LG, b2, end_bit, N, av, pg, d_err, st, S, &few)) != cudaSuccess)
                    return e;
                if (few) {
                    sorted_keys = ws.keys[1];
                    sorted_vals = ws.lvals[1];
                }
            }
            few_last = few;
            if (!few) {
                uint64_t *kk[2] = {ws.keys[0], ws.keys[1]};
                uint32_t *vv[2] = {ws.lvals[0], ws.lvals[1]};
                int which = 0;
                if ((e = radix_sort_pairs(kk, vv, NL, end_bit, ws.radix, d_err, st, &which, &ran,
                                          hist_passes > 0)) != cudaSuccess)
                    return e;
                S.radix_passes += ran;
                sorted_keys = kk[which];
                sorted_vals = vv[which];
            }
            S.large_total += NL;
            TileArgs r;
            r.keys = sorted_keys;
            r.keys32 = nullptr;
            r.vals = sorted_vals;
            r.pos = ws.lpos;
            r.rank_out = nullptr;
            r.pairs = nullptr;
            r.pair_count = nullptr;
            r.slot0 = nullptr;
            r.N = NL;
            r.n = nr;
            r.K = (uint32_t)K;
            r.zlo = r.zhi = 0;
            if ((e = run_assign<MODE_ROUND>(r, ws, out_i, out_pos, out_gid, ws.gstart[pg ^ 1], ws.counters, st, &kept,
                                            &groups)) != cudaSuccess)
                return e;
        }
        int sv = av;
        av = sv ^ 1;
        pg ^= 1;
        h *= 2;
    }
    return cudaSuccess;
}

// Digit histograms of the seed keys from one histogram.  When a digit holds
// d = 8 / bits whole codes, digit p of the key of suffix i is the d-gram of
// codes starting at i + K - d (p + 1), so its histogram is the d-gram
// histogram over the positions [s_p, n + s_p), s_p = K - d (p + 1).  The
// seed kernel accumulates digit 0 only; digit p's histogram is digit 0's
// plus the d*p grams at positions [s_p, s_0) and minus the d*p grams at
// [n + s_p, n + s_0), which lie past the end of the text and are 0 (codes
// past the end are 0, as in the keys).  `head` holds the codes of positions
// [0, K).
static void seed_hist_from_grams(uint32_t *hist, int passes, int bits, int K, const uint16_t *head)
{
    const int d = 8 / bits;
    const int s0 = K - d;
    for (int p = 1; p < passes; ++p) {
        const int sp = K - d * (p + 1);
        uint32_t *h = hist + 256 * p;
        for (int v = 0; v < 256; ++v) h[v] = hist[v];
        for (int j = sp; j < s0; ++j) {
            uint32_t v = 0;
            for (int q = 0; q < d; ++q) v = (v << bits) | head[j + q];
            h[v] += 1;
        }
        h[0] -= (uint32_t)(s0 - sp);
    }
}

cudaError_t suffix_sort(const void *d_T, int symbytes, uint64_t n, bool gsa, SortWorkspace &ws,
                        const SortOptions &opt, uint32_t *d_err, cudaStream_t st, SortStats *stats)
{
    cudaError_t e;
    SortStats local;
    SortStats &S = stats ? *stats : local;
    S = SortStats();
    if (n == 0) return cudaSuccess;

    // ---- symbol histogram -> dense codes (32-bit integer symbols are their own
    // codes: bits = bits(opt.raw_max))
    const bool raw = symbytes == 4;
    const int nsym = symbytes == 1 ? 256 : 65536;
    uint32_t *h_hist = ws.h_small + 16;
    uint16_t *h_codes = reinterpret_cast<uint16_t *>(ws.h_small + 16 + 65536);
    int bits;
    if (raw) {
        bits = gsais_bits_for(opt.raw_max > 1 ? opt.raw_max : 1);
    } else {
        if (opt.hist_ready) {
            if ((e = cudaMemcpyAsync(h_hist, ws.hist, (size_t)nsym * 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
                (e = cudaStreamSynchronize(st)) != cudaSuccess)
                return e;
        } else if (opt.presence_only && symbytes == 1) {
            // the codes only need which bytes occur: h_hist[c] = 1 for those
            cudaEvent_t ev_h = ws.radix.prof ? ws.radix.prof->begin(st) : nullptr;
            uint32_t *h_map = h_hist + 256;
            if ((e = byte_presence(static_cast<const uint8_t *>(d_T), n, ws.hist, st)) != cudaSuccess ||
                (e = read_back(h_map, ws.hist, 8 * sizeof(uint32_t), st)) != cudaSuccess ||
                (e = cudaStreamSynchronize(st)) != cudaSuccess)
                return e;
            if (ev_h) ws.radix.prof->end(KK_HIST, ev_h, st, n);
            for (int c = 0; c < 256; ++c) h_hist[c] = (h_map[c >> 5] >> (c & 31)) & 1u;
        } else {
            cudaEvent_t ev_h = ws.radix.prof ? ws.radix.prof->begin(st) : nullptr;
            if ((e = symbol_histogram(d_T, symbytes, n, ws.hist, h_hist, st)) != cudaSuccess) return e;
            if (ev_h) ws.radix.prof->end(KK_HIST, ev_h, st, n * symbytes);
        }
        uint32_t sigma = 0;
        for (int c = 0; c < nsym; ++c) {
            h_codes[c] = (uint16_t)sigma;
            if (h_hist[c]) ++sigma;
        }
        bits = gsais_bits_for(sigma > 1 ? sigma - 1 : 1);
    }
    const Tuning tn = opt.tuning_set ? opt.tuning : tuning_lookup(n, bits);
    ws.radix.items32 = tn.radix_items32;
    ws.radix.items64 = tn.radix_items64;
    S.tuning = tn;
    // 3- and 4-bit codes: a 32-bit key holds 10 or 8 symbols, so on read sets
    // and small alphabets most suffixes stay in large seed groups; 64-bit keys
    // cost four more digit passes and save doubling rounds (GSA of 2^20 reads:
    // 41.9 vs 51.6 ms).  2-bit codes (16 symbols) and wide alphabets keep 32.
    const int key_bits = opt.seed_key_bits ? opt.seed_key_bits : ((bits == 3 || bits == 4) ? 64 : 32);
    int K = (key_bits <= 32 ? 32 : 64) / bits;
    if (K < 2 && bits <= 32) K = 64 / bits;   // wide symbols: at least two per key
    if (K < 1) K = 1;
    if (K > 64) K = 64;
    S.seed_symbols = K;
    S.seed_bits = bits;
    if (!raw &&
        (e = cudaMemcpyAsync(ws.codes, h_codes, (size_t)nsym * 2, cudaMemcpyHostToDevice, st)) != cudaSuccess)
        return e;
    if ((e = cudaMemsetAsync(ws.rank + n, 0, sizeof(uint32_t), st)) != cudaSuccess) return e;

    // ---- seed keys (+ digit histograms, + packed codes) and the K-prefix sort
    const int seed_end = K * bits;
    const int seed_passes = (seed_end + 7) / 8;
    const bool narrow = seed_end <= 32;   // 32-bit seed keys: less sort traffic
    ws.pack_bits = (gsa || raw) ? 0 : (bits <= 2 ? 2 : (bits <= 4 ? 4 : 0));
    for (int c = 0, code = 0; !raw && c < nsym && code < 16; ++c)
        if (h_hist[c]) ws.decode[code++] = (uint16_t)c;
    const unsigned seed_grid = (unsigned)stream_grid((n + kSeedTile - 1) / kSeedTile * 256, 256);
    // digits made of whole codes (plain texts, bits 1, 2, 4, 8): the seed
    // kernel builds digit 0's histogram, the others follow on the host
    const bool grams = !gsa && !raw && 8 % bits == 0 && seed_end % 8 == 0 && K <= 64 && n >= (uint64_t)(2 * K + 16);
    const int hist_passes = grams ? 1 : seed_passes;
    uint32_t *k32[2] = {reinterpret_cast<uint32_t *>(ws.keys[0]), reinterpret_cast<uint32_t *>(ws.keys[1])};
    if ((e = cudaMemsetAsync(ws.radix.hist, 0, (size_t)seed_passes * 256 * 4, st)) != cudaSuccess) return e;
    cudaEvent_t ev_seed = ws.radix.prof ? ws.radix.prof->begin(st) : nullptr;
    const bool fast_seed = grams && narrow && (bits == 2 || bits == 4) && ws.pack_bits == bits;
    if (fast_seed) {
        if (symbytes == 1 && bits == 2)
            GSAIS_COUNTED((k_seed_packed<uint8_t, 2><<<seed_grid, 256, 0, st>>>(
                static_cast<const uint8_t *>(d_T), n, ws.codes, k32[0], ws.vals[0], seed_end, ws.radix.hist, ws.packed)));
        else if (symbytes == 1)
            GSAIS_COUNTED((k_seed_packed<uint8_t, 4><<<seed_grid, 256, 0, st>>>(
                static_cast<const uint8_t *>(d_T), n, ws.codes, k32[0], ws.vals[0], seed_end, ws.radix.hist, ws.packed)));
        else if (bits == 2)
            GSAIS_COUNTED((k_seed_packed<uint16_t, 2><<<seed_grid, 256, 0, st>>>(
                static_cast<const uint16_t *>(d_T), n, ws.codes, k32[0], ws.vals[0], seed_end, ws.radix.hist,
                ws.packed)));
        else
            GSAIS_COUNTED((k_seed_packed<uint16_t, 4><<<seed_grid, 256, 0, st>>>(
                static_cast<const uint16_t *>(d_T), n, ws.codes, k32[0], ws.vals[0], seed_end, ws.radix.hist,
                ws.packed)));
    } else if (symbytes == 1) {
        const uint8_t *T8 = static_cast<const uint8_t *>(d_T);
        if (narrow)
            GSAIS_COUNTED((k_seed<uint8_t, uint32_t><<<seed_grid, 256, 0, st>>>(
                T8, n, ws.codes, bits, K, gsa ? 1 : 0, k32[0], ws.vals[0], hist_passes, seed_end, ws.radix.hist,
                ws.pack_bits, ws.packed)));
        else
            GSAIS_COUNTED((k_seed<uint8_t, uint64_t><<<seed_grid, 256, 0, st>>>(
                T8, n, ws.codes, bits, K, gsa ? 1 : 0, ws.keys[0], ws.vals[0], hist_passes, seed_end, ws.radix.hist,
                ws.pack_bits, ws.packed)));
    } else if (raw) {
        const uint32_t *T32 = static_cast<const uint32_t *>(d_T);
        if (narrow)
            GSAIS_COUNTED((k_seed<uint32_t, uint32_t><<<seed_grid, 256, 0, st>>>(
                T32, n, ws.codes, bits, K, 0, k32[0], ws.vals[0], hist_passes, seed_end, ws.radix.hist, 0,
                ws.packed)));
        else
            GSAIS_COUNTED((k_seed<uint32_t, uint64_t><<<seed_grid, 256, 0, st>>>(
                T32, n, ws.codes, bits, K, 0, ws.keys[0], ws.vals[0], hist_passes, seed_end, ws.radix.hist, 0,
                ws.packed)));
    } else {
        const uint16_t *T16 = static_cast<const uint16_t *>(d_T);
        if (narrow)
            GSAIS_COUNTED((k_seed<uint16_t, uint32_t><<<seed_grid, 256, 0, st>>>(
                T16, n, ws.codes, bits, K, gsa ? 1 : 0, k32[0], ws.vals[0], hist_passes, seed_end, ws.radix.hist,
                ws.pack_bits, ws.packed)));
        else
            GSAIS_COUNTED((k_seed<uint16_t, uint64_t><<<seed_grid, 256, 0, st>>>(
                T16, n, ws.codes, bits, K, gsa ? 1 : 0, ws.keys[0], ws.vals[0], hist_passes, seed_end, ws.radix.hist,
                ws.pack_bits, ws.packed)));
    }
    if (ev_seed)
        ws.radix.prof->end(KK_SEED, ev_seed, st,
                           fast_seed ? n * (symbytes + 4) + n * bits / 8 : n * (symbytes + (narrow ? 8 : 12)));
    if (grams) {
        uint32_t *h_hist0 = ws.radix.h_hist;
        uint8_t *h_edge = reinterpret_cast<uint8_t *>(ws.h_small + 16 + 65536 + 32768);
        if ((e = cudaMemcpyAsync(h_hist0, ws.radix.hist, 256 * 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
        if ((e = cudaMemcpyAsync(h_edge, d_T, (size_t)K * symbytes, cudaMemcpyDeviceToHost, st)) != cudaSuccess)
            return e;
        if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
        uint16_t head[64];
        for (int q = 0; q < K; ++q)
            head[q] = h_codes[symbytes == 1 ? h_edge[q] : reinterpret_cast<const uint16_t *>(h_edge)[q]];
        seed_hist_from_grams(h_hist0, seed_passes, bits, K, head);
        if ((e = cudaMemcpyAsync(ws.radix.hist, h_hist0, (size_t)seed_passes * 256 * 4, cudaMemcpyHostToDevice, st)) !=
            cudaSuccess)
            return e;
    }
    int w = 0, ran = 0;
    {
        uint32_t *vv[2] = {ws.vals[0], ws.vals[1]};
        if (narrow) {
            if ((e = radix_sort_pairs32(k32, vv, n, seed_end, ws.radix, d_err, st, &w, &ran, true, fast_seed)) !=
                cudaSuccess)
                return e;
        } else {
            uint64_t *kk[2] = {ws.keys[0], ws.keys[1]};
            if ((e = radix_sort_pairs(kk, vv, n, seed_end, ws.radix, d_err, st, &w, &ran, true)) != cudaSuccess)
                return e;
        }
        S.radix_passes += ran;
    }

    TileArgs a;
    a.keys = ws.keys[w];
    a.keys32 = narrow ? k32[w] : nullptr;
    a.vals = ws.vals[w];
    a.pos = nullptr;
    a.rank_out = nullptr;
    a.pairs = nullptr;
    a.pair_count = nullptr;
    a.slot0 = ws.slot0;
    a.N = n;
    a.n = n;
    a.K = (uint32_t)K;
    a.zlo = 0;
    for (int q = 0; q < K; ++q) a.zlo |= 1ull << (q * bits);
    a.zhi = a.zlo << (bits - 1);
    uint32_t kept = 0, groups = 0;
    int av = w ^ 1, pg = 0;
    if (use_two_level_ranks(n)) a.rank_out = reinterpret_cast<uint32_t *>(ws.keys[w ^ 1]);
    PairSource ps;
    if (ws.pack_bits == 2 || ws.pack_bits == 4) {
        ps.pack_bits = ws.pack_bits;
        ps.words.w = reinterpret_cast<const uint64_t *>(ws.packed);
        ps.words.nwords = (n + kSeedTile - 1) / kSeedTile * (uint64_t)kSeedTile * ws.pack_bits / 64;
        ps.n = n;
    }
    if (!gsa && ps.pack_bits) {
        // groups of exactly two leave the seed round for direct comparison;
        // their slots go after the ranks in keys[w ^ 1] (at most n / 2)
        a.pairs = reinterpret_cast<uint32_t *>(ws.keys[w ^ 1]) + n;
        a.pair_count = ws.counters + 3;
        if ((e = cudaMemsetAsync(ws.counters, 0, 5 * sizeof(unsigned long long), st)) != cudaSuccess) return e;
    }
    if (gsa)
        e = run_assign<MODE_INIT_GSA>(a, ws, ws.vals[av], ws.pos[pg], ws.gid[pg], ws.gstart[pg], nullptr, st, &kept,
                                      &groups);
    else {
        TailSource tails;   // suffixes shorter than K get their heads from the text
        tails.T = d_T;
        tails.symbytes = symbytes;
        tails.codes = ws.codes;
        tails.bits = bits;
        e = run_assign<MODE_INIT_PLAIN>(a, ws, ws.vals[av], ws.pos[pg], ws.gid[pg], ws.gstart[pg], nullptr, st,
                                        &kept, &groups, &tails);
    }
    if (e != cudaSuccess) return e;
    if (a.pairs) {
        // order the pairs (they share the K seed symbols); unresolved ones are
        // appended behind the survivors.  With two-level ranks the order goes
        // into the SA-order list the rank scatter below reads.
        unsigned long long *h = reinterpret_cast<unsigned long long *>(ws.h_small + 8);
        h[0] = ((unsigned long long)groups << 32) | kept;
        if ((e = cudaMemcpyAsync(ws.counters, h, sizeof(unsigned long long), cudaMemcpyHostToDevice, st)) !=
            cudaSuccess)
            return e;
        if ((e = run_pair_compare(ws, ps, a.pairs, n / 2, (uint64_t)K, ws.vals[av], ws.pos[pg], ws.gid[pg],
                                  ws.gstart[pg], d_err, st, a.rank_out ? ws.vals[w] : nullptr, a.rank_out,
                                  ws.slot0)) != cudaSuccess)
            return e;
        unsigned long long *hc = reinterpret_cast<unsigned long long *>(ws.h_small);
        if ((e = cudaMemcpyAsync(hc, ws.counters, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st)) !=
            cudaSuccess)
            return e;
        if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
        kept = (uint32_t)hc[0];
        groups = (uint32_t)(hc[0] >> 32);
        S.pairs_direct += hc[3];
        if (ws.radix.prof) ws.radix.prof->add_bytes(KK_PAIRS, hc[3] * 24);
    }

    // ---- SA leaves for the host while the rank scatter and the rounds run
    // (the slots the rounds write are patched afterwards)
    if (opt.early && (opt.early->host || opt.early->on_start) && kept > 0 && kept <= opt.early->patch_cap) {
        EarlySaCopy &ec = *opt.early;
        if ((e = cudaMemsetAsync(ec.bits, 0, (n + 31) / 32 * 4, st)) != cudaSuccess) return e;
        GSAIS_COUNTED((k_mark_slots<<<stream_grid(kept, 256), 256, 0, st>>>(ws.pos[pg], kept, n, ec.bits)));
        if ((e = cudaEventRecord(ec.ready, st)) != cudaSuccess) return e;
        if (ec.host) {
            if ((e = cudaStreamWaitEvent(ec.stream, ec.ready, 0)) != cudaSuccess) return e;
            if ((e = cudaMemcpyAsync(ec.host, ws.sa, n * 4, cudaMemcpyDeviceToHost, ec.stream)) != cudaSuccess)
                return e;
            if ((e = cudaEventRecord(ec.copied, ec.stream)) != cudaSuccess) return e;
        }
        ec.patch_n = kept;
        ec.started = true;
        S.early_patch = kept;
        if (ec.on_start && (e = ec.on_start(st)) != cudaSuccess) return e;
    }
    if (a.rank_out && (e = scatter_seed_ranks(ws, ws.vals[w], a.rank_out, n, n, d_err, st)) != cudaSuccess) return e;

    // ---- doubling rounds over the active suffixes
    if ((e = run_rounds(ws, n, K, kept, groups, av, pg, d_err, st, S, ps, tn)) != cudaSuccess) return e;
    uint32_t herr = 0;
    if ((e = read_back(ws.h_small, d_err, 4, st)) != cudaSuccess) return e;
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
    herr = ws.h_small[0];
    if (ws.radix.prof) ws.radix.prof->flush();
    return herr ? cudaErrorUnknown : cudaSuccess;
}

cudaError_t early_sa_patch(const EarlySaCopy &ec, const uint32_t *d_sa, uint64_t n, cudaStream_t st)
{
    if (!ec.started || ec.patch_n == 0) return cudaSuccess;
    cudaError_t e = cudaStreamWaitEvent(st, ec.copied, 0);
    if (e != cudaSuccess) return e;
    const uint64_t words = (n + 31) / 32;
    GSAIS_COUNTED((k_sa_patch<<<stream_grid(words, 256), 256, 0, st>>>(ec.bits, words, d_sa, n, ec.host_dev)));
    return cudaGetLastError();
}

cudaError_t symbol_histogram_part(const void *d_part, int symbytes, uint64_t len, uint32_t *d_hist, cudaStream_t st)
{
    if (len == 0) return cudaSuccess;
    if (symbytes == 1)
        GSAIS_COUNTED((k_hist_u8<<<stream_grid(len / 4 + 1, 256), 256, 0, st>>>(static_cast<const uint8_t *>(d_part),
                                                                                len, d_hist)));
    else
        GSAIS_COUNTED((k_hist_u16<<<stream_grid(len, 256), 256, 0, st>>>(static_cast<const uint16_t *>(d_part), len,
                                                                          d_hist)));
    return cudaGetLastError();
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

namespace gsais {

size_t batch_workspace_bytes(uint64_t n, uint32_t count) { return sort_workspace_bytes(n + count, 1); }

cudaError_t batch_suffix_sort(const void *d_T, int symbytes, uint64_t n, const uint64_t *d_offs, uint32_t count,
                              SortWorkspace &ws, uint32_t *d_err, cudaStream_t st, SortStats *stats,
                              const Tuning *tuning)
{
    cudaError_t e;
    SortStats local;
    SortStats &S = stats ? *stats : local;
    S = SortStats();
    if (n == 0) return cudaSuccess;
    const uint64_t nr = n + count;   // rank domain: every string followed by its gap slot

    uint32_t *h_hist = ws.h_small + 16;
    uint16_t *h_codes = reinterpret_cast<uint16_t *>(ws.h_small + 16 + 65536);
    const int nsym = symbytes == 1 ? 256 : 65536;
    if ((e = symbol_histogram(d_T, symbytes, n, ws.hist, h_hist, st)) != cudaSuccess) return e;
    uint32_t sigma = 0;
    for (int c = 0; c < nsym; ++c) {
        if (h_hist[c]) ++sigma;
        h_codes[c] = h_hist[c] ? (uint16_t)sigma : (uint16_t)0;   // codes 1..sigma; 0 = end of string
    }
    const int bits = gsais_bits_for(sigma);
    const Tuning tn = tuning ? *tuning : tuning_lookup(n, bits);
    ws.radix.items32 = tn.radix_items32;
    ws.radix.items64 = tn.radix_items64;
    S.tuning = tn;
    const int sid_bits = gsais_bits_for(count > 1 ? count - 1 : 0);
    int K = (64 - sid_bits) / bits;
    if (K < 1) K = 1;
    S.seed_symbols = K;
    S.seed_bits = bits;
    ws.pack_bits = 0;
    if ((e = cudaMemcpyAsync(ws.codes, h_codes, (size_t)nsym * 2, cudaMemcpyHostToDevice, st)) != cudaSuccess)
        return e;
    if ((e = cudaMemsetAsync(ws.rank, 0, (nr + 1) * sizeof(uint32_t), st)) != cudaSuccess) return e;

    const int seed_end = K * bits + sid_bits;
    const int seed_passes = (seed_end + 7) / 8;
    if ((e = cudaMemsetAsync(ws.radix.hist, 0, (size_t)seed_passes * 256 * 4, st)) != cudaSuccess) return e;
    cudaEvent_t ev_seed = ws.radix.prof ? ws.radix.prof->begin(st) : nullptr;
    if (symbytes == 1)
        GSAIS_COUNTED((k_seed_batch<uint8_t><<<stream_grid(n, 256), 256, 0, st>>>(
            static_cast<const uint8_t *>(d_T), n, d_offs, count, ws.codes, bits, K, ws.keys[0], ws.vals[0],
            seed_passes, seed_end, ws.radix.hist)));
    else
        GSAIS_COUNTED((k_seed_batch<uint16_t><<<stream_grid(n, 256), 256, 0, st>>>(
            static_cast<const uint16_t *>(d_T), n, d_offs, count, ws.codes, bits, K, ws.keys[0], ws.vals[0],
            seed_passes, seed_end, ws.radix.hist)));
    if (ev_seed) ws.radix.prof->end(KK_SEED, ev_seed, st, n * 13);
    int w = 0, ran = 0;
    {
        uint64_t *kk[2] = {ws.keys[0], ws.keys[1]};
        uint32_t *vv[2] = {ws.vals[0], ws.vals[1]};
        if ((e = radix_sort_pairs(kk, vv, n, seed_end, ws.radix, d_err, st, &w, &ran, true)) != cudaSuccess) return e;
        S.radix_passes += ran;
    }
    // seed-round groups: equal (string, K-window); windows that reach the gap are unique
    TileArgs a;
    a.keys = ws.keys[w];
    a.keys32 = nullptr;
    a.vals = ws.vals[w];
    a.pos = nullptr;
    a.rank_out = nullptr;
    a.pairs = nullptr;
    a.pair_count = nullptr;
    a.slot0 = nullptr;
    a.N = n;
    a.n = nr;
    a.K = (uint32_t)K;
    a.zlo = a.zhi = 0;
    uint32_t kept = 0, groups = 0;
    const int av = w ^ 1, pg = 0;
    if (use_two_level_ranks(nr)) a.rank_out = reinterpret_cast<uint32_t *>(ws.keys[w ^ 1]);
    if ((e = run_assign<MODE_ROUND>(a, ws, ws.vals[av], ws.pos[pg], ws.gid[pg], ws.gstart[pg], nullptr, st, &kept,
                                    &groups)) != cudaSuccess)
        return e;
    if (a.rank_out && (e = scatter_seed_ranks(ws, ws.vals[w], a.rank_out, n, nr, d_err, st)) != cudaSuccess)
        return e;
    if ((e = run_rounds(ws, nr, K, kept, groups, av, pg, d_err, st, S, PairSource(), tn)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(ws.h_small, d_err, 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
    if (ws.radix.prof) ws.radix.prof->flush();
    return ws.h_small[0] ? cudaErrorUnknown : cudaSuccess;
}

cudaError_t batch_outputs(const SortWorkspace &ws, const void *d_T, int symbytes, uint64_t n, const uint64_t *d_offs,
                          uint32_t count, int32_t *d_sa, void *d_U, int32_t *d_primary, uint32_t *d_err,
                          cudaStream_t st)
{
    cudaError_t e;
    if ((e = cudaMemsetAsync(d_primary, 0, (size_t)count * sizeof(int32_t), st)) != cudaSuccess) return e;
    if (n == 0) return cudaSuccess;
    if (symbytes == 1)
        GSAIS_COUNTED((k_batch_outputs<uint8_t><<<stream_grid(n, 256), 256, 0, st>>>(
            ws.sa, ws.rank, static_cast<const uint8_t *>(d_T), n, d_offs, count, d_sa, static_cast<uint8_t *>(d_U),
            d_primary, d_err)));
    else
        GSAIS_COUNTED((k_batch_outputs<uint16_t><<<stream_grid(n, 256), 256, 0, st>>>(
            ws.sa, ws.rank, static_cast<const uint16_t *>(d_T), n, d_offs, count, d_sa,
            static_cast<uint16_t *>(d_U), d_primary, d_err)));
    return cudaGetLastError();
}

}  // namespace gsais
