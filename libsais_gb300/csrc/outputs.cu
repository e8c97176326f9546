// outputs.cu -- BWT gather, auxiliary ISA samples, Phi-array PLCP and the
// LCP permute, for sm_103a.  All are HBM-bound gathers/scatters.
//
// Every index read from an array (SA entries, Phi entries) is checked against
// n before it is used as an address; a bad index raises GSAIS_ERR_BOUNDS in
// the context's error word and the access is skipped, so a malformed caller
// array becomes a -2 return instead of a device fault.
#include <cstring>
#include <type_traits>
#include <vector>

#include "device_util.cuh"
#include "engine.h"
#include "outputs.cuh"
#include "suffix_sort.cuh"

namespace gsais {

namespace {

int sm_count()
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms > 0 ? sms : 1;
}

int grid_for(uint64_t items, int threads)
{
    const uint64_t want = (items + threads - 1) / threads;
    const uint64_t cap = (uint64_t)sm_count() * 16;
    return (int)(want < 1 ? 1 : (want < cap ? want : cap));
}

// Bytes per row: SA 4 read, T symbol gathered, U symbol written
// (libsais src/libsais.c:4777/:5396 write T[p-1] during the final induction).
template <typename Sym>
__global__ void __launch_bounds__(256) k_bwt(const Sym *__restrict__ T, const uint32_t *__restrict__ SA, uint64_t n,
                                             const uint32_t *__restrict__ isa1, Sym *__restrict__ U, PackedText pk,
                                             uint32_t *__restrict__ err)
{
    constexpr int B = 8;   // rows per thread per step: all SA loads, then all gathers
    __shared__ Sym dec[16];
    if (threadIdx.x < 16) dec[threadIdx.x] = (Sym)pk.decode[threadIdx.x];
    __syncthreads();
    const uint64_t i0 = (uint64_t)isa1[0] - 1;   // SA row of suffix 0
    const uint64_t span = (uint64_t)gridDim.x * blockDim.x * B;
    for (uint64_t k0 = (uint64_t)blockIdx.x * blockDim.x * B + threadIdx.x; k0 < n; k0 += span) {
        uint32_t p[B];
#pragma unroll
        for (int j = 0; j < B; ++j) {
            const uint64_t k = k0 + (uint64_t)j * blockDim.x;
            const uint64_t row = k <= i0 ? k - 1 : k;
            p[j] = (k > 0 && k < n && row < n) ? SA[row] : 0u;
        }
#pragma unroll
        for (int j = 0; j < B; ++j) {
            const uint64_t k = k0 + (uint64_t)j * blockDim.x;
            if (k >= n) break;
            if (k == 0) {
                U[0] = T[n - 1];
                continue;
            }
            const uint64_t q = p[j];
            if (q == 0 || q > n) {
                if (err) atomicOr(err, GSAIS_ERR_BOUNDS);
                continue;
            }
            if (pk.pack_bits == 2) {
                const uint32_t w = reinterpret_cast<const uint16_t *>(pk.packed)[(q - 1) >> 3];
                U[k] = dec[(w >> (2 * ((q - 1) & 7))) & 3u];
            } else if (pk.pack_bits == 4) {
                const uint32_t w = reinterpret_cast<const uint32_t *>(pk.packed)[(q - 1) >> 3];
                U[k] = dec[(w >> (4 * ((q - 1) & 7))) & 15u];
            } else {
                U[k] = T[q - 1];
            }
        }
    }
}

// BWT rows of the marked SA slots: the rows of slots still unresolved when
// an early BWT was taken (their U positions are the same under the
// provisional and the final primary row, as every row between the two lies
// in suffix 0's group, which is marked).  Address order, a warp per bitmap
// word, so runs of rows leave as coalesced writes when U is host memory.
// Bytes: n / 8 read; per marked row SA 4 read, symbol gathered, 1-2 written.
template <typename Sym>
__global__ void __launch_bounds__(256) k_bwt_patch(const uint32_t *__restrict__ bits, uint64_t words,
                                                   const Sym *__restrict__ T, const uint32_t *__restrict__ SA,
                                                   uint64_t n, const uint32_t *__restrict__ isa1,
                                                   Sym *__restrict__ U, PackedText pk, uint32_t *__restrict__ err)
{
    __shared__ Sym dec[16];
    if (threadIdx.x < 16) dec[threadIdx.x] = (Sym)pk.decode[threadIdx.x];
    __syncthreads();
    const uint64_t i0 = (uint64_t)isa1[0] - 1;
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
            const uint64_t s = (base + (uint64_t)l) * 32 + (uint64_t)lane;
            if (!((mw >> lane) & 1u) || s >= n || s == i0) continue;
            const uint64_t k = s < i0 ? s + 1 : s;
            const uint64_t q = SA[s];
            if (q == 0 || q > n) {
                atomicOr(err, GSAIS_ERR_BOUNDS);
                continue;
            }
            if (pk.pack_bits == 2) {
                const uint32_t w = reinterpret_cast<const uint16_t *>(pk.packed)[(q - 1) >> 3];
                U[k] = dec[(w >> (2 * ((q - 1) & 7))) & 3u];
            } else if (pk.pack_bits == 4) {
                const uint32_t w = reinterpret_cast<const uint32_t *>(pk.packed)[(q - 1) >> 3];
                U[k] = dec[(w >> (4 * ((q - 1) & 7))) & 15u];
            } else {
                U[k] = T[q - 1];
            }
        }
    }
}

template <typename I>
__global__ void __launch_bounds__(256) k_aux(const uint32_t *__restrict__ isa1, uint64_t n, uint64_t r, I *__restrict__ out)
{
    const uint64_t cnt = (n - 1) / r + 1;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < cnt; t += stride) out[t] = (I)isa1[t * r];
}

__global__ void __launch_bounds__(256) k_widen(const uint32_t *__restrict__ s, int64_t *__restrict__ d, uint64_t n)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) d[i] = (int64_t)s[i];
}

__global__ void __launch_bounds__(256) k_narrow(const int64_t *__restrict__ s, uint32_t *__restrict__ d, uint64_t n,
                                                uint32_t *__restrict__ err)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const int64_t v = s[i];
        if (v < 0 || (uint64_t)v >= n) atomicOr(err, GSAIS_ERR_BOUNDS);
        d[i] = (uint32_t)v;
    }
}

// Integer alphabets: the largest value and whether any value lies outside
// [0, k) (libsais_int, src/libsais.c:7050; libsais64_long, src/libsais64.c:7118).
// out[0] = max (as uint64), out[1] = 1 if a value is out of range.
template <typename I>
__global__ void __launch_bounds__(256) k_int_scan(const I *__restrict__ T, uint64_t n, int64_t k,
                                                  unsigned long long *__restrict__ out)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    unsigned long long mx = 0;
    bool bad = false;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const int64_t v = (int64_t)T[i];
        bad |= v < 0 || v >= k;
        if (v > 0 && (unsigned long long)v > mx) mx = (unsigned long long)v;
    }
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long y = __shfl_down_sync(GSAIS_FULL_MASK, mx, o);
        if (y > mx) mx = y;
    }
    const bool anybad = __any_sync(GSAIS_FULL_MASK, bad);
    if ((threadIdx.x & 31) == 0) {
        if (mx) atomicMax(&out[0], mx);
        if (anybad) atomicOr(&out[1], 1ull);
    }
}

// Integer symbols narrowed to 16 or 32 bits (the caller checked the range).
template <typename I, typename O>
__global__ void __launch_bounds__(256) k_int_narrow(const I *__restrict__ T, uint64_t n, O *__restrict__ out)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) out[i] = (O)T[i];
}

// Phi[SA[j]] = SA[j-1], Phi[SA[0]] = n (src/libsais.c:8116 compute_phi), by
// a direct scatter (texts too small for the position partitions).
// Bytes per row: SA 4 + 4 read, Phi 4 scattered.
__global__ void __launch_bounds__(256) k_phi(const uint32_t *__restrict__ SA, uint64_t n, uint32_t *__restrict__ phi,
                                             uint32_t *__restrict__ err)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += stride) {
        const uint64_t s = SA[j];
        if (s >= n) {
            atomicOr(err, GSAIS_ERR_BOUNDS);
            continue;
        }
        phi[s] = j ? SA[j - 1] : (uint32_t)n;
    }
}

// ---- symbol comparison on 64-bit windows of the text.  A window at symbol p
// holds the symbols p, p+1, ... least significant first, SB bits each:
//   PB = 0: the raw text (SB = 8 * sizeof(Sym)), read as aligned 64-bit words
//           (a window at any byte offset is two words and a funnel shift; a
//           word not wholly inside the text is assembled byte by byte, bytes
//           past the end reading as 0);
//   PB = 2 or 4: the text as dense codes of PB bits (plcp_build packs it when
//           the alphabet has at most 16 symbols), two 64-bit words and a
//           funnel shift; the packed array ends with two zero words.
// Every caller clamps lengths to the text, so the contents past the end do
// not matter.
struct TextWords {
    const uint8_t *T;         // the raw text
    uint64_t nbytes;          // its length in bytes
    uint32_t mis;             // T's offset past the previous 8-byte boundary
    const uint64_t *packed;   // PB > 0: the packed codes
};

template <typename Sym, int PB>
struct SymBits {
    static constexpr int value = PB ? PB : 8 * (int)sizeof(Sym);
};

__device__ __forceinline__ uint64_t load8(const TextWords &tw, uint64_t off)
{
    const uint64_t a = off + tw.mis;
    const uint64_t w = a >> 3;
    const uint32_t sh = (uint32_t)(a & 7) * 8;
    const uint64_t end = tw.mis + tw.nbytes;   // in aligned coordinates
    if (w * 8 >= tw.mis && (w + 2) * 8 <= end) {
        const uint64_t *W = reinterpret_cast<const uint64_t *>(tw.T - tw.mis);
        const uint64_t lo = __ldg(W + w);
        if (sh == 0) return lo;
        const uint64_t hi = __ldg(W + w + 1);
        return (lo >> sh) | (hi << (64 - sh));
    }
    uint64_t v = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k)
        if (off + k < tw.nbytes) v |= (uint64_t)tw.T[off + k] << (8 * k);
    return v;
}

template <typename Sym, int PB>
__device__ __forceinline__ uint64_t window(const TextWords &tw, uint64_t p)
{
    if (PB == 0) return load8(tw, p * sizeof(Sym));
    const uint64_t bit = p * PB;
    const uint64_t w = bit >> 6;
    const uint32_t sh = (uint32_t)(bit & 63);
    const uint64_t lo = __ldg(tw.packed + w);
    if (sh == 0) return lo;
    return (lo >> sh) | (__ldg(tw.packed + w + 1) << (64 - sh));
}

// Equal leading symbols of two windows of SB-bit symbols; GSA also stops at a
// 0 symbol (code 0 when packed: the separator is the smallest symbol) of x.
template <int SB, bool GSA>
__device__ __forceinline__ uint32_t eq_symbols(uint64_t x, uint64_t y)
{
    uint64_t stop = x ^ y;
    if (GSA) {
        // lowest flagged field = the first 0 field (borrows only run upwards)
        constexpr uint64_t lo = SB == 2 ? 0x5555555555555555ull
                              : SB == 4 ? 0x1111111111111111ull
                              : SB == 8 ? 0x0101010101010101ull
                                        : 0x0001000100010001ull;
        stop |= (x - lo) & ~x & (lo << (SB - 1));
    }
    const uint32_t bit = stop ? (uint32_t)(__ffsll((long long)stop) - 1) : 64u;
    return bit / SB;
}

// First mismatch offset >= l of the suffixes at p and q, at most m (one
// thread, one 64-bit window per step).  Plain texts: m = n - max(p, q)
// (src/libsais.c:8177); GSA also stops at a separator (:8215-8238).
template <typename Sym, bool GSA, int PB>
__device__ __forceinline__ uint64_t extend_thread(const TextWords &tw, uint64_t p, uint64_t q, uint64_t l, uint64_t m)
{
    constexpr int SB = SymBits<Sym, PB>::value, PER = 64 / SB;
    while (l < m) {
        const uint32_t c = eq_symbols<SB, GSA>(window<Sym, PB>(tw, p + l), window<Sym, PB>(tw, q + l));
        l += c;
        if (c < (uint32_t)PER) break;
    }
    return l < m ? l : m;
}

// Equal leading symbols of two consecutive windows at symbol offset o
// (capped at m - o; 0 if o >= m).
template <typename Sym, bool GSA, int PB>
__device__ __forceinline__ uint32_t lane_window(const TextWords &tw, uint64_t p, uint64_t q, uint64_t o, uint64_t m)
{
    constexpr int SB = SymBits<Sym, PB>::value, HALF = 64 / SB;
    if (o >= m) return 0;
    uint32_t c = eq_symbols<SB, GSA>(window<Sym, PB>(tw, p + o), window<Sym, PB>(tw, q + o));
    if (c == (uint32_t)HALF)
        c += eq_symbols<SB, GSA>(window<Sym, PB>(tw, p + o + HALF), window<Sym, PB>(tw, q + o + HALF));
    return (uint64_t)c > m - o ? (uint32_t)(m - o) : c;
}

// PLCP of the first chunk start (position 0) from scratch, by every CTA of the
// grid: CTA g compares blocks g, g + grid, ... of two windows per thread and
// lowers sparse[0] to the first mismatch it finds; a block that starts at or
// beyond the value already found is skipped.  sparse[0] holds m (or 0) on entry.
template <typename Sym, bool GSA, int PB>
__global__ void __launch_bounds__(256) k_plcp_first(TextWords tw, uint64_t n, const uint32_t *__restrict__ phi,
                                                    uint32_t *sparse)
{
    constexpr int PER = 2 * 64 / SymBits<Sym, PB>::value;
    constexpr uint64_t BLK = 256 * PER;
    const uint64_t b = phi[0];
    if (b >= n) return;   // suffix 0 is first in SA (or a bad entry): PLCP 0
    const uint64_t m = n - b;   // a = 0 < b
    __shared__ unsigned long long s_min;
    __shared__ uint32_t s_cur;
    for (uint64_t g = blockIdx.x;; g += gridDim.x) {
        const uint64_t o0 = g * BLK;
        if (threadIdx.x == 0) {
            s_cur = *reinterpret_cast<volatile uint32_t *>(sparse);
            s_min = ~0ull;
        }
        __syncthreads();
        if (o0 >= m || o0 >= s_cur) break;   // the same decision in every thread
        const uint64_t o = o0 + (uint64_t)threadIdx.x * PER;
        const uint32_t c = lane_window<Sym, GSA, PB>(tw, 0, b, o, m);
        if (c < (uint32_t)PER) atomicMin(&s_min, (unsigned long long)(o + c));
        __syncthreads();
        if (threadIdx.x == 0 && s_min != ~0ull) atomicMin(sparse, (uint32_t)(s_min < m ? s_min : m));
        __syncthreads();
    }
}

__global__ void k_plcp_first_init(const uint32_t *__restrict__ phi, uint64_t n, uint32_t *__restrict__ sparse,
                                  uint32_t *__restrict__ level_counts, int levels, uint32_t *__restrict__ err)
{
    const uint64_t b = phi[0];
    if (b > n) atomicOr(err, GSAIS_ERR_BOUNDS);
    sparse[0] = b >= n ? 0u : (uint32_t)(n - b);
    for (int k = 0; k < levels; ++k) level_counts[k] = 0;
}

// One level of exact PLCP values at chunk starts: chunk k = (2w+1)*half takes
// its lower bound from chunk k - half (PLCP[i+d] >= PLCP[i] - d).  A thread
// per chunk start extends one window per step for at most kLevelSteps steps
// (the bound is tight for most starts); starts still matching go to the
// long list for k_plcp_long.
constexpr int kLevelSteps = 16;

template <typename Sym, bool GSA, int PB>
__global__ void __launch_bounds__(256) k_plcp_level(TextWords tw, uint64_t n, const uint32_t *__restrict__ phi,
                                                    uint32_t chunk, uint64_t nchunks, uint64_t half,
                                                    uint32_t *__restrict__ sparse, uint2 *__restrict__ long_list,
                                                    uint32_t *__restrict__ long_count, uint32_t *__restrict__ err)
{
    constexpr int SB = SymBits<Sym, PB>::value, PER = 64 / SB;
    const uint64_t w = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t k = (2 * w + 1) * half;
    if (k >= nchunks) return;
    const uint64_t a = k * chunk;
    uint64_t b = phi[a];
    if (b > n) {
        atomicOr(err, GSAIS_ERR_BOUNDS);
        b = n;
    }
    uint64_t l = 0;
    bool done = true;
    if (b != n) {
        const uint64_t kp = k - half;
        const uint64_t d = a - kp * chunk;
        const uint64_t lp = sparse[kp];
        const uint64_t m = n - (a > b ? a : b);
        l = lp > d ? lp - d : 0;
        if (l > m) l = m;
        done = false;
        for (int it = 0; it < kLevelSteps; ++it) {
            if (l >= m) {
                l = m;
                done = true;
                break;
            }
            const uint32_t c = eq_symbols<SB, GSA>(window<Sym, PB>(tw, a + l), window<Sym, PB>(tw, b + l));
            l += c;
            if (c < (uint32_t)PER) {
                if (l > m) l = m;
                done = true;
                break;
            }
        }
    }
    if (done) {
        sparse[k] = (uint32_t)l;
    } else {
        const uint32_t slot = atomicAdd(long_count, 1u);
        long_list[slot] = make_uint2((uint32_t)k, (uint32_t)l);
    }
}

// The same level with a warp per chunk start, for the levels whose bounds come
// from far away (half * chunk symbols back: the bound is loose and the start
// extends by about its whole PLCP value): lane j compares two windows at
// l + j * (two windows), so a step covers 32 x 2 windows and most starts
// finish in one step instead of a chain of dependent window reads.  Starts
// still matching after kLevelWarpSteps steps go to the long list.
constexpr int kLevelWarpSteps = 4;

template <typename Sym, bool GSA, int PB>
__global__ void __launch_bounds__(256) k_plcp_level_warp(TextWords tw, uint64_t n, const uint32_t *__restrict__ phi,
                                                         uint32_t chunk, uint64_t nchunks, uint64_t half,
                                                         uint32_t *__restrict__ sparse,
                                                         uint2 *__restrict__ long_list,
                                                         uint32_t *__restrict__ long_count,
                                                         uint32_t *__restrict__ err)
{
    constexpr int PER2 = 2 * 64 / SymBits<Sym, PB>::value;
    const int lane = threadIdx.x & 31;
    const uint64_t w = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t k = (2 * w + 1) * half;
    if (k >= nchunks) return;   // the same for the whole warp
    const uint64_t a = k * chunk;
    uint64_t b = phi[a];
    if (b > n) {
        if (lane == 0) atomicOr(err, GSAIS_ERR_BOUNDS);
        b = n;
    }
    uint64_t l = 0;
    bool done = true;
    if (b != n) {
        const uint64_t kp = k - half;
        const uint64_t d = a - kp * chunk;
        const uint64_t lp = sparse[kp];
        const uint64_t m = n - (a > b ? a : b);
        l = lp > d ? lp - d : 0;
        if (l > m) l = m;
        done = false;
        for (int it = 0; it < kLevelWarpSteps; ++it) {
            // lane_window is 0 at or past m, so the first such lane ends the scan at m
            const uint64_t o = l + (uint64_t)lane * PER2;
            const uint32_t c = lane_window<Sym, GSA, PB>(tw, a, b, o, m);
            const uint32_t stop = __ballot_sync(GSAIS_FULL_MASK, c < (uint32_t)PER2);
            if (stop) {
                const int f = __ffs(stop) - 1;
                l += (uint64_t)f * PER2 + __shfl_sync(GSAIS_FULL_MASK, c, f);
                if (l > m) l = m;
                done = true;
                break;
            }
            l += 32ull * PER2;
        }
    }
    if (lane == 0) {
        if (done) {
            sparse[k] = (uint32_t)l;
        } else {
            const uint32_t slot = atomicAdd(long_count, 1u);
            long_list[slot] = make_uint2((uint32_t)k, (uint32_t)l);
        }
    }
}

// The long extensions of one level: a CTA per listed start, 256 threads x two
// windows per step.
template <typename Sym, bool GSA, int PB>
__global__ void __launch_bounds__(256) k_plcp_long(TextWords tw, uint64_t n, const uint32_t *__restrict__ phi,
                                                   uint32_t chunk, uint32_t *__restrict__ sparse,
                                                   const uint2 *__restrict__ long_list,
                                                   const uint32_t *__restrict__ long_count)
{
    constexpr int PER = 2 * 64 / SymBits<Sym, PB>::value;
    __shared__ unsigned long long s_min;
    const uint32_t count = *long_count;
    for (uint32_t j = blockIdx.x; j < count; j += gridDim.x) {
        const uint2 e = long_list[j];
        const uint64_t a = (uint64_t)e.x * chunk;
        const uint64_t b = phi[a];   // listed by k_plcp_level only when b < n
        const uint64_t m = b < n ? n - (a > b ? a : b) : 0;
        uint64_t l = e.y < m ? e.y : m;
        while (l < m) {
            if (threadIdx.x == 0) s_min = ~0ull;
            __syncthreads();
            const uint64_t o = l + (uint64_t)threadIdx.x * PER;
            const uint32_t c = lane_window<Sym, GSA, PB>(tw, a, b, o, m);
            if (c < (uint32_t)PER) atomicMin(&s_min, (unsigned long long)(o + c));
            __syncthreads();
            const unsigned long long r = s_min;
            __syncthreads();
            if (r != ~0ull) {
                l = r < m ? r : m;
                break;
            }
            l += 256 * PER;
        }
        if (threadIdx.x == 0) sparse[e.x] = (uint32_t)(l < m ? l : m);
    }
}

// Kasai's carried length inside each chunk of kPlcpChunk positions, starting
// from the exact value at the chunk start (src/libsais.c:8167 compute_plcp
// restarts at block starts too).  A CTA stages the Phi values of its chunks
// in shared memory with coalesced streaming loads (evict-first, so they do
// not push the packed text out of L2), each thread walks its chunk -- one
// dependent chain of text reads, so the short chunk keeps the shared memory
// per chain small and many chains in flight -- and the PLCP values leave
// coalesced, streamed as well.
constexpr uint32_t kPlcpChunk = 32;
constexpr int kKasaiThreads = 128;
constexpr int kKasaiStride = kPlcpChunk + 1;   // padded rows: no bank conflicts

template <typename Sym, bool GSA, int PB>
__global__ void __launch_bounds__(kKasaiThreads) k_plcp_kasai(TextWords tw, uint64_t n, uint64_t nchunks,
                                                              const uint32_t *__restrict__ sparse,
                                                              const uint32_t *__restrict__ phi,
                                                              uint32_t *__restrict__ plcp, uint32_t *__restrict__ err)
{
    __shared__ uint32_t s[kKasaiThreads * kKasaiStride];
    const uint64_t tile0 = (uint64_t)blockIdx.x * kKasaiThreads * kPlcpChunk;
    for (uint32_t e = threadIdx.x; e < kKasaiThreads * kPlcpChunk; e += kKasaiThreads) {
        const uint64_t x = tile0 + e;
        if (x < n) s[(e / kPlcpChunk) * kKasaiStride + (e % kPlcpChunk)] = __ldcs(phi + x);
    }
    __syncthreads();
    const uint64_t k = (uint64_t)blockIdx.x * kKasaiThreads + threadIdx.x;
    bool bad = false;
    if (k < nchunks) {
        uint32_t *row = s + threadIdx.x * kKasaiStride;
        const uint64_t a = k * kPlcpChunk;
        const uint64_t e = a + kPlcpChunk < n ? a + kPlcpChunk : n;
        constexpr int SB = SymBits<Sym, PB>::value, PER = 64 / SB;
        uint64_t l = sparse[k];
        row[0] = (uint32_t)l;
        // Each step also loads the next step's two windows, at the guess
        // g = (this step's starting length) - 1: the next step starts at
        // (this step's final length) - 1 >= g, and when this step extends by
        // d < PER symbols the guessed windows still cover that start.  So a
        // chain keeps two text reads in flight instead of one.
        // A guess reaching past the text end is neither loaded nor used (the
        // step's own start length is below it then).
        uint64_t b = a + 1 < e ? row[1] : n;
        uint64_t g = l ? l - 1 : 0;
        uint64_t wa = 0, wb = 0;
        bool have = a + 1 < e && b < n && a + 1 + g < n && b + g < n;
        if (have) {
            wa = window<Sym, PB>(tw, a + 1 + g);
            wb = window<Sym, PB>(tw, b + g);
        }
        for (uint64_t x = a + 1; x < e; ++x) {
            if (b > n) {
                bad = true;
                b = n;
            }
            const uint64_t bn = x + 1 < e ? row[x + 1 - a] : n;
            if (b == n) {
                l = 0;
                // next step starts from 0
                const uint64_t g1 = 0;
                uint64_t wa1 = 0, wb1 = 0;
                const bool have1 = bn < n && x + 1 < n;
                if (have1) {
                    wa1 = window<Sym, PB>(tw, x + 1);
                    wb1 = window<Sym, PB>(tw, bn);
                }
                row[x - a] = 0;
                b = bn, g = g1, wa = wa1, wb = wb1, have = have1;
                continue;
            }
            uint64_t ls = l ? l - 1 : 0;
            const uint64_t m = n - (x > b ? x : b);
            if (ls > m) ls = m;
            // the next step's windows, guessed from this step's start
            const uint64_t g1 = ls ? ls - 1 : 0;
            uint64_t wa1 = 0, wb1 = 0;
            const bool have1 = bn < n && x + 1 + g1 < n && bn + g1 < n;
            if (have1) {
                wa1 = window<Sym, PB>(tw, x + 1 + g1);
                wb1 = window<Sym, PB>(tw, bn + g1);
            }
            // this step: the guessed windows start d = ls - g symbols early
            // (ls >= g unless the text end cut ls below the guess)
            const uint64_t d = ls - g;
            bool done = false;
            if (have && ls >= g && d < (uint64_t)PER) {
                const int sh = (int)d * SB;
                const uint32_t c0 = eq_symbols<SB, GSA>(wa >> sh, wb >> sh);
                const uint32_t avail = (uint32_t)(PER - d);
                if (c0 < avail) {
                    l = ls + c0;
                    done = true;
                } else {
                    ls += avail;
                }
            }
            if (!done) l = extend_thread<Sym, GSA, PB>(tw, x, b, ls < m ? ls : m, m);
            if (l > m) l = m;
            row[x - a] = (uint32_t)l;
            b = bn, g = g1, wa = wa1, wb = wb1, have = have1;
        }
    }
    if (bad) atomicOr(err, GSAIS_ERR_BOUNDS);
    __syncthreads();
    for (uint32_t e = threadIdx.x; e < kKasaiThreads * kPlcpChunk; e += kKasaiThreads) {
        const uint64_t x = tile0 + e;
        if (x < n) __stcs(plcp + x, s[(e / kPlcpChunk) * kKasaiStride + (e % kPlcpChunk)]);
    }
}

// LCP[i] = PLCP[SA[i]] (src/libsais.c:8311 compute_lcp).  Bytes: 12 per row.
// Eight rows per thread per step: all SA loads, then all eight gathers in
// flight, then the stores.
__global__ void __launch_bounds__(256) k_lcp(const uint32_t *__restrict__ plcp, const uint32_t *__restrict__ SA,
                                             uint32_t *__restrict__ lcp, uint64_t n, uint32_t *__restrict__ err)
{
    constexpr int B = 8;
    const uint64_t span = (uint64_t)gridDim.x * blockDim.x * B;
    bool bad = false;
    for (uint64_t i0 = (uint64_t)blockIdx.x * blockDim.x * B + threadIdx.x; i0 < n; i0 += span) {
        uint32_t s[B], v[B];
#pragma unroll
        for (int j = 0; j < B; ++j) {
            const uint64_t i = i0 + (uint64_t)j * blockDim.x;
            s[j] = i < n ? SA[i] : 0u;
        }
#pragma unroll
        for (int j = 0; j < B; ++j) {
            const uint64_t i = i0 + (uint64_t)j * blockDim.x;
            const bool ok = i < n && s[j] < n;
            bad |= i < n && !ok;
            v[j] = ok ? __ldg(plcp + s[j]) : 0u;
        }
#pragma unroll
        for (int j = 0; j < B; ++j) {
            const uint64_t i = i0 + (uint64_t)j * blockDim.x;
            if (i < n) lcp[i] = v[j];
        }
    }
    if (bad) atomicOr(err, GSAIS_ERR_BOUNDS);
}

// ---- LCP[i] = PLCP[SA[i]] for PLCP arrays much larger than L2.  A direct
// gather (k_lcp) pulls a 64-byte DRAM burst per 4-byte entry.  Instead the
// rows go through buckets of 2^shift consecutive positions (kLcpBuckets
// buckets):
//   k_lcp_partition  tiles of kLcpTile consecutive rows; a tile reserves one
//                    run per bucket (atomic cursor, the bucket's first free
//                    slot), writes its rows' positions there and keeps, per
//                    row, its place in the tile's bucket order (16 bits) and,
//                    per (tile, bucket), the run's first slot and its start
//                    in the tile's order;
//   k_lcp_fetch      in place over the bucketed positions, in order: pos[k]
//                    becomes PLCP[pos[k]]; the CTAs in flight work inside one
//                    or two buckets, so the PLCP window of 2^shift entries
//                    stays in L2 and DRAM reads it once;
//   k_lcp_place      each tile copies its runs of values into shared memory
//                    and writes LCP[i] = value at the row's place.
// Bytes per row: SA 4 read, pos 4 + place 2 written; pos 4 + PLCP 4 read,
// val 4 written; place 2 + val 4 read, LCP 4 written = 32 (and 4 per tile
// and bucket of run records).
constexpr int kLcpBucketBits = 8;
constexpr int kLcpBuckets = 1 << kLcpBucketBits;
constexpr int kLcpThreads = 512;
constexpr int kLcpItems = 16;
constexpr int kLcpTile = kLcpThreads * kLcpItems;   // 8192 rows: runs of ~32 entries per bucket
constexpr uint16_t kLcpNoPlace = 0xFFFF;

// Below 2^26 rows the PLCP array is at most twice L2 and the direct gather
// is faster (2^25 random rows: 0.36 ms direct, 0.47 ms bucketed).
bool lcp_partitioned(uint64_t n) { return n >= (1ull << 26); }

int lcp_shift(uint64_t n)
{
    int b = 0;
    while (b < 40 && (1ull << b) < n) ++b;   // positions < n <= 2^b
    return b > kLcpBucketBits ? b - kLcpBucketBits : 0;
}

__global__ void k_lcp_cursors(uint32_t *__restrict__ cursor, int shift, uint64_t n)
{
    const uint32_t b = threadIdx.x;
    if (b < kLcpBuckets) {
        const uint64_t s = (uint64_t)b << shift;
        cursor[b] = (uint32_t)(s < n ? s : n);
    }
}

// runs[t][0][d] = first slot of bucket d's run, runs[t][1][d] = its start in
// the tile's bucket order.
__global__ void __launch_bounds__(kLcpThreads) k_lcp_partition(const uint32_t *__restrict__ SA, uint64_t n, int shift,
                                                               uint32_t *__restrict__ cursor,
                                                               uint32_t *__restrict__ runs,
                                                               uint32_t *__restrict__ pos,
                                                               uint16_t *__restrict__ place,
                                                               uint32_t *__restrict__ err)
{
    __shared__ uint32_t s_cnt[kLcpBuckets], s_start[kLcpBuckets], s_g[kLcpBuckets];
    __shared__ uint32_t s_scan[kLcpThreads / 32 + 1];
    __shared__ uint32_t s_pos[kLcpTile];
    const uint64_t t0 = (uint64_t)blockIdx.x * kLcpTile;
    for (int d = threadIdx.x; d < kLcpBuckets; d += kLcpThreads) s_cnt[d] = 0;
    uint32_t q[kLcpItems];
    uint16_t slot[kLcpItems];
    bool bad = false;
#pragma unroll
    for (int k = 0; k < kLcpItems; ++k) {
        const uint64_t i = t0 + (uint64_t)k * kLcpThreads + threadIdx.x;
        q[k] = i < n ? __ldcs(SA + i) : 0xFFFFFFFFu;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kLcpItems; ++k) {
        const uint64_t i = t0 + (uint64_t)k * kLcpThreads + threadIdx.x;
        if (i < n && q[k] >= n) bad = true;
        if (q[k] < n) slot[k] = (uint16_t)atomicAdd(&s_cnt[q[k] >> shift], 1u);
    }
    __syncthreads();
    const uint32_t c = threadIdx.x < kLcpBuckets ? s_cnt[threadIdx.x] : 0u;
    uint32_t total;
    const uint32_t st = block_exclusive_sum<uint32_t, kLcpThreads>(c, s_scan, total);
    if (threadIdx.x < kLcpBuckets) {
        const uint32_t d = threadIdx.x;
        const uint32_t g = c ? atomicAdd(&cursor[d], c) : 0u;
        s_start[d] = st;
        s_g[d] = g;
        uint32_t *r = runs + (uint64_t)blockIdx.x * 2 * kLcpBuckets;
        r[d] = g;
        r[kLcpBuckets + d] = st;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kLcpItems; ++k) {
        const uint64_t i = t0 + (uint64_t)k * kLcpThreads + threadIdx.x;
        if (i >= n) continue;
        uint16_t pl = kLcpNoPlace;
        if (q[k] < n) {
            const uint32_t loc = s_start[q[k] >> shift] + slot[k];
            s_pos[loc] = q[k];
            pl = (uint16_t)loc;
        }
        __stcs(place + i, pl);
    }
    __syncthreads();
    for (uint32_t e = threadIdx.x; e < total; e += kLcpThreads) {
        const uint32_t p = s_pos[e], d = p >> shift;
        const uint64_t o = (uint64_t)s_g[d] + (e - s_start[d]);
        // a suffix array fills every bucket exactly; a run past its bucket
        // means repeated positions
        const uint64_t end = ((uint64_t)d + 1) << shift;
        if (o < n && o < end) pos[o] = p;
        else bad = true;
    }
    if (bad) atomicOr(err, GSAIS_ERR_BOUNDS);
}

// In place: v[k] = PLCP[v[k]], eight entries per thread in flight.
__global__ void __launch_bounds__(256) k_lcp_fetch(const uint32_t *__restrict__ plcp, uint32_t *__restrict__ v,
                                                   uint64_t n, uint32_t *__restrict__ err)
{
    constexpr int B = 8;
    const uint64_t span = (uint64_t)gridDim.x * blockDim.x * B;
    bool bad = false;
    for (uint64_t k0 = (uint64_t)blockIdx.x * blockDim.x * B + threadIdx.x; k0 < n; k0 += span) {
        uint32_t s[B], x[B];
#pragma unroll
        for (int j = 0; j < B; ++j) {
            const uint64_t k = k0 + (uint64_t)j * blockDim.x;
            s[j] = k < n ? __ldcs(v + k) : 0u;
        }
#pragma unroll
        for (int j = 0; j < B; ++j) {
            const uint64_t k = k0 + (uint64_t)j * blockDim.x;
            const bool ok = k < n && s[j] < n;
            bad |= k < n && !ok;
            x[j] = ok ? __ldg(plcp + s[j]) : 0u;
        }
#pragma unroll
        for (int j = 0; j < B; ++j) {
            const uint64_t k = k0 + (uint64_t)j * blockDim.x;
            if (k < n) __stcs(v + k, x[j]);
        }
    }
    if (bad) atomicOr(err, GSAIS_ERR_BOUNDS);
}

// LCP may be the SA buffer (this pass does not read SA).
__global__ void __launch_bounds__(kLcpThreads) k_lcp_place(uint64_t n, const uint32_t *__restrict__ runs,
                                                           const uint16_t *__restrict__ place,
                                                           const uint32_t *__restrict__ val, uint32_t *lcp)
{
    __shared__ uint32_t s_g[kLcpBuckets], s_start[kLcpBuckets + 1];
    __shared__ uint32_t s_val[kLcpTile];
    const uint64_t t0 = (uint64_t)blockIdx.x * kLcpTile;
    const uint32_t rows = (uint32_t)(n - t0 < (uint64_t)kLcpTile ? n - t0 : (uint64_t)kLcpTile);
    const uint32_t *r = runs + (uint64_t)blockIdx.x * 2 * kLcpBuckets;
    for (int d = threadIdx.x; d < kLcpBuckets; d += kLcpThreads) {
        s_g[d] = r[d];
        s_start[d] = r[kLcpBuckets + d];
    }
    if (threadIdx.x == 0) s_start[kLcpBuckets] = rows;
    __syncthreads();
    // every value of the tile in flight at once: entry e of the tile's bucket
    // order belongs to the last bucket whose run starts at or before e
    uint32_t v[kLcpItems];
#pragma unroll
    for (int k = 0; k < kLcpItems; ++k) {
        const uint32_t e = (uint32_t)k * kLcpThreads + threadIdx.x;
        v[k] = 0u;
        if (e < rows) {
            uint32_t lo = 0;
#pragma unroll
            for (int step = kLcpBuckets / 2; step > 0; step >>= 1)
                if (s_start[lo + step] <= e) lo += step;
            const uint64_t o = (uint64_t)s_g[lo] + (e - s_start[lo]);
            if (o < n) v[k] = __ldcs(val + o);
        }
    }
#pragma unroll
    for (int k = 0; k < kLcpItems; ++k) s_val[k * kLcpThreads + threadIdx.x] = v[k];
    __syncthreads();
#pragma unroll 4
    for (int k = 0; k < kLcpItems; ++k) {
        const uint64_t i = t0 + (uint64_t)k * kLcpThreads + threadIdx.x;
        if (i >= n) continue;
        const uint16_t pl = __ldcs(place + i);
        __stcs(lcp + i, pl < rows ? s_val[pl] : 0u);
    }
}

// The text as dense codes of B bits, least significant first, one 64-bit
// word per thread step; words past the text (the two padding words) are 0.
// Bytes per symbol: sizeof(Sym) read (+ a code-table lookup), B/8 written.
template <typename Sym, int B>
__global__ void __launch_bounds__(256) k_pack_codes(const Sym *__restrict__ T, uint64_t n,
                                                    const uint16_t *__restrict__ codes, uint64_t *__restrict__ packed,
                                                    uint64_t words)
{
    constexpr int SPW = 64 / B;
    // 8-bit texts: the code table in shared memory and the word's SPW bytes in
    // 16-byte loads (a warp reads 32 x SPW contiguous bytes)
    constexpr bool BYTES = sizeof(Sym) == 1;
    __shared__ uint8_t s_codes[BYTES ? 256 : 1];
    if (BYTES) {
        for (int c = threadIdx.x; c < 256; c += blockDim.x) s_codes[c] = (uint8_t)codes[c];
        __syncthreads();
    }
    const bool vec = BYTES && (reinterpret_cast<uintptr_t>(T) & 15) == 0;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t w = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; w < words; w += stride) {
        uint64_t v = 0;
        const uint64_t p0 = w * SPW;
        if (vec && p0 + SPW <= n) {
            const uint4 *src = reinterpret_cast<const uint4 *>(reinterpret_cast<const uint8_t *>(T) + p0);
#pragma unroll
            for (int q = 0; q < SPW / 16; ++q) {
                const uint4 x = __ldcs(src + q);
                const uint32_t xs[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
                for (int j = 0; j < 16; ++j)
                    v |= (uint64_t)s_codes[(xs[j >> 2] >> (8 * (j & 3))) & 255u] << ((q * 16 + j) * B);
            }
        } else {
#pragma unroll 8
            for (int k = 0; k < SPW; ++k) {
                const uint64_t p = p0 + k;
                if (p < n) v |= (uint64_t)(BYTES ? s_codes[(uint32_t)T[p]] : __ldg(codes + T[p])) << (k * B);
            }
        }
        packed[w] = v;
    }
}

// Scratch of plcp_run, in words: chunk-start values, the long list (two words
// per entry, at most one entry per chunk start of a level), per-level long
// counts, the Phi partitions' scratch, and the packed text with its symbol
// histogram and code table.
constexpr int kMaxLevels = 40;

uint64_t plcp_chunks(uint64_t n) { return (n + kPlcpChunk - 1) / kPlcpChunk; }

struct PlcpLayout {
    size_t o_long, o_counts, o_phi, o_phiarr, o_hist, o_codes, o_packed, total;
};

PlcpLayout plcp_scratch_layout(uint64_t n)
{
    PlcpLayout L;
    const uint64_t nc = plcp_chunks(n);
    size_t w = (nc + 2 + 63) / 64 * 64;   // sparse
    L.o_long = w;
    w += 2 * ((nc / 2 + 2 + 31) / 32 * 32);
    L.o_counts = w;
    w += 64;
    L.o_phi = w;
    w += (phi_scratch_words(n) + 63) / 64 * 64;
    L.o_phiarr = w;   // Phi itself
    w += (n + 63) / 64 * 64;
    L.o_hist = w;
    w += 65536;
    L.o_codes = w;
    w += 32768;   // 65536 16-bit codes
    L.o_packed = w;
    w += 2 * ((n + 15) / 16 + 2) + 64;   // 4-bit codes at most, as 64-bit words + 2 padding words
    L.total = w;
    return L;
}

template <typename Sym, bool GSA, int PB>
cudaError_t plcp_run(const Sym *T, const uint32_t *SA, uint64_t n, uint32_t *plcp, uint32_t *scratch, uint32_t *err,
                     cudaStream_t st)
{
    const PlcpLayout L = plcp_scratch_layout(n);
    uint32_t *sparse = scratch;
    uint2 *long_list = reinterpret_cast<uint2 *>(scratch + L.o_long);
    uint32_t *counts = scratch + L.o_counts;
    uint32_t *phi = scratch + L.o_phiarr;
    if (phi_partitioned(n)) {
        cudaError_t e = phi_permute(SA, n, phi, scratch + L.o_phi, err, st);
        if (e != cudaSuccess) return e;
    } else {
        GSAIS_COUNTED((k_phi<<<grid_for(n, 256), 256, 0, st>>>(SA, n, phi, err)));
    }
    TextWords tw;
    tw.T = reinterpret_cast<const uint8_t *>(T);
    tw.nbytes = n * sizeof(Sym);
    tw.mis = (uint32_t)(reinterpret_cast<uintptr_t>(T) & 7);
    tw.packed = reinterpret_cast<const uint64_t *>(scratch + L.o_packed);
    const uint64_t nchunks = plcp_chunks(n);
    uint64_t top = 1;
    int levels = 0;
    while (top < nchunks) {
        top <<= 1;
        ++levels;
    }
    if (levels > kMaxLevels) return cudaErrorInvalidValue;
    // level 0: chunk 0 from scratch, by the whole grid
    GSAIS_COUNTED((k_plcp_first_init<<<1, 1, 0, st>>>(phi, n, sparse, counts, levels, err)));
    GSAIS_COUNTED((k_plcp_first<Sym, GSA, PB><<<sm_count() * 4, 256, 0, st>>>(tw, n, phi, sparse)));
    int level = 0;
    for (uint64_t half = top >> 1; half >= 1; half >>= 1, ++level) {
        const uint64_t count = nchunks > half ? (nchunks - half + 2 * half - 1) / (2 * half) : 0;
        if (count == 0) continue;
        if (half * kPlcpChunk > 256) {   // loose bounds: a warp per start
            const unsigned blocks = (unsigned)((count + 7) / 8);
            GSAIS_COUNTED((k_plcp_level_warp<Sym, GSA, PB><<<blocks, 256, 0, st>>>(
                tw, n, phi, kPlcpChunk, nchunks, half, sparse, long_list, counts + level, err)));
        } else {
            const unsigned blocks = (unsigned)((count + 255) / 256);
            GSAIS_COUNTED((k_plcp_level<Sym, GSA, PB><<<blocks, 256, 0, st>>>(
                tw, n, phi, kPlcpChunk, nchunks, half, sparse, long_list, counts + level, err)));
        }
        // the long list is empty at most levels and holds thousands of starts
        // at the last ones: a grid-stride loop over it, CTAs that find no
        // entry exit at once
        const uint64_t lcap = (uint64_t)sm_count() * 8;
        const unsigned lg = (unsigned)(count < lcap ? count : lcap);
        GSAIS_COUNTED((k_plcp_long<Sym, GSA, PB><<<lg, 256, 0, st>>>(tw, n, phi, kPlcpChunk, sparse, long_list,
                                                                     counts + level)));
    }
    GSAIS_COUNTED((k_plcp_kasai<Sym, GSA, PB><<<(unsigned)((nchunks + kKasaiThreads - 1) / kKasaiThreads),
                                                kKasaiThreads, 0, st>>>(tw, n, nchunks, sparse, phi, plcp, err)));
    return cudaGetLastError();
}

// Which byte values occur in an 8-bit text: bit c of the 256-bit map (eight
// words).  Each thread keeps one 32-symbol block of the map in a register (the
// block of the last symbol it met outside it): texts of a few symbols in one
// block (DNA) never leave it, other symbols go to the CTA's map by a
// shared-memory atomicOr; a block does one atomicOr per word at the end.
// Bytes per symbol: 1 read.
__global__ void __launch_bounds__(256) k_presence_u8(const uint8_t *__restrict__ T, uint64_t n,
                                                     uint32_t *__restrict__ present)
{
    __shared__ uint32_t sm[8];
    if (threadIdx.x < 8) sm[threadIdx.x] = 0;
    __syncthreads();
    uint32_t cur_q = 0, cur_m = 0;
    auto add = [&](uint32_t c) {
        const uint32_t q = c >> 5, bit = 1u << (c & 31);
        if (q == cur_q) {
            cur_m |= bit;
        } else {
            if (cur_m) atomicOr(&sm[cur_q], cur_m);
            cur_q = q;
            cur_m = bit;
        }
    };
    const uint64_t head = (16 - (reinterpret_cast<uintptr_t>(T) & 15)) & 15;
    const uint64_t h = head < n ? head : n;
    const uint64_t vecs = (n - h) / 16;
    const uint4 *V = reinterpret_cast<const uint4 *>(T + h);
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; v < vecs; v += stride) {
        const uint4 w = __ldcs(V + v);
        const uint32_t words[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
        for (int q = 0; q < 4; ++q)
#pragma unroll
            for (int b = 0; b < 4; ++b) add((words[q] >> (8 * b)) & 255u);
    }
    if (blockIdx.x == 0 && threadIdx.x < 32) {   // the unaligned head and the tail
        for (uint64_t i = threadIdx.x; i < h; i += 32) add(T[i]);
        for (uint64_t i = h + vecs * 16 + threadIdx.x; i < n; i += 32) add(T[i]);
    }
    if (cur_m) atomicOr(&sm[cur_q], cur_m);
    __syncthreads();
    if (threadIdx.x < 8 && sm[threadIdx.x]) atomicOr(&present[threadIdx.x], sm[threadIdx.x]);
}

// Packs an 8- or 16-bit text into dense 2- or 4-bit codes when its alphabet
// has at most 16 symbols (the random text reads of the PLCP kernels then hit
// a quarter or half of the bytes, which stays in L2 for texts up to ~2^29
// symbols).  Returns the code width (0: not packed).  Synchronises st.
template <typename Sym>
cudaError_t pack_for_plcp(const Sym *T, uint64_t n, uint32_t *scratch, uint32_t *h_hist, cudaStream_t st, int *bits)
{
    *bits = 0;
    if (!h_hist || n < (1u << 16)) return cudaSuccess;   // small texts: the raw text is cache-resident anyway
    const PlcpLayout L = plcp_scratch_layout(n);
    const int nsym = sizeof(Sym) == 1 ? 256 : 65536;
    cudaError_t e;
    if (sizeof(Sym) == 1) {
        // only which symbols occur matters here: a 256-bit presence map
        uint32_t *d_map = scratch + L.o_hist;
        if ((e = cudaMemsetAsync(d_map, 0, 32, st)) != cudaSuccess) return e;
        GSAIS_COUNTED((k_presence_u8<<<grid_for(n / 16 + 1, 256), 256, 0, st>>>(
            reinterpret_cast<const uint8_t *>(T), n, d_map)));
        if ((e = cudaMemcpyAsync(h_hist, d_map, 32, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
            (e = cudaStreamSynchronize(st)) != cudaSuccess)
            return e;
        uint32_t map[8];
        std::memcpy(map, h_hist, 32);
        for (int c = 0; c < 256; ++c) h_hist[c] = (map[c >> 5] >> (c & 31)) & 1u;
    } else if ((e = symbol_histogram(T, (int)sizeof(Sym), n, scratch + L.o_hist, h_hist, st)) != cudaSuccess) {
        return e;
    }
    std::vector<uint16_t> codes(nsym, 0);
    uint32_t sigma = 0;
    for (int c = 0; c < nsym; ++c) {
        codes[c] = (uint16_t)sigma;
        if (h_hist[c]) ++sigma;
    }
    if (sigma > 16) return cudaSuccess;
    const int B = sigma <= 4 ? 2 : 4;
    uint16_t *d_codes = reinterpret_cast<uint16_t *>(scratch + L.o_codes);
    if ((e = cudaMemcpyAsync(d_codes, codes.data(), (size_t)nsym * 2, cudaMemcpyHostToDevice, st)) != cudaSuccess)
        return e;
    uint64_t *packed = reinterpret_cast<uint64_t *>(scratch + L.o_packed);
    const uint64_t words = (n * B + 63) / 64 + 2;
    if (B == 2)
        GSAIS_COUNTED((k_pack_codes<Sym, 2><<<grid_for(words, 256), 256, 0, st>>>(T, n, d_codes, packed, words)));
    else
        GSAIS_COUNTED((k_pack_codes<Sym, 4><<<grid_for(words, 256), 256, 0, st>>>(T, n, d_codes, packed, words)));
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;   // codes (pageable) are copied
    *bits = B;
    return cudaGetLastError();
}

template <typename Sym, bool GSA>
cudaError_t plcp_dispatch(const Sym *T, const uint32_t *SA, uint64_t n, uint32_t *plcp, uint32_t *scratch,
                          uint32_t *h_hist, uint32_t *err, cudaStream_t st)
{
    int bits = 0;
    cudaError_t e = pack_for_plcp(T, n, scratch, h_hist, st, &bits);
    if (e != cudaSuccess) return e;
    if (bits == 2) return plcp_run<Sym, GSA, 2>(T, SA, n, plcp, scratch, err, st);
    if (bits == 4) return plcp_run<Sym, GSA, 4>(T, SA, n, plcp, scratch, err, st);
    return plcp_run<Sym, GSA, 0>(T, SA, n, plcp, scratch, err, st);
}

}  // namespace

cudaError_t bwt_gather(const void *d_T, int symbytes, const uint32_t *d_SA, const uint32_t *d_isa1, uint64_t n,
                       void *d_U, const PackedText &pk, uint32_t *err, cudaStream_t st)
{
    if (n == 0) return cudaSuccess;
    if (symbytes == 1)
        GSAIS_COUNTED((k_bwt<uint8_t><<<grid_for((n + 7) / 8, 256), 256, 0, st>>>(
            static_cast<const uint8_t *>(d_T), d_SA, n, d_isa1, static_cast<uint8_t *>(d_U), pk, err)));
    else
        GSAIS_COUNTED((k_bwt<uint16_t><<<grid_for((n + 7) / 8, 256), 256, 0, st>>>(
            static_cast<const uint16_t *>(d_T), d_SA, n, d_isa1, static_cast<uint16_t *>(d_U), pk, err)));
    return cudaGetLastError();
}

cudaError_t bwt_patch(const void *d_T, int symbytes, const uint32_t *d_SA, const uint32_t *d_isa1, uint64_t n,
                      const uint32_t *row_bits, void *U, const PackedText &pk, uint32_t *err, cudaStream_t st)
{
    const uint64_t words = (n + 31) / 32;
    if (words == 0) return cudaSuccess;
    if (symbytes == 1)
        GSAIS_COUNTED((k_bwt_patch<uint8_t><<<grid_for(words, 256), 256, 0, st>>>(
            row_bits, words, static_cast<const uint8_t *>(d_T), d_SA, n, d_isa1, static_cast<uint8_t *>(U), pk,
            err)));
    else
        GSAIS_COUNTED((k_bwt_patch<uint16_t><<<grid_for(words, 256), 256, 0, st>>>(
            row_bits, words, static_cast<const uint16_t *>(d_T), d_SA, n, d_isa1, static_cast<uint16_t *>(U), pk,
            err)));
    return cudaGetLastError();
}

cudaError_t aux_sample(const uint32_t *d_isa1, uint64_t n, uint64_t r, void *d_I, int idx_bytes, cudaStream_t st)
{
    if (n == 0 || r == 0) return cudaSuccess;
    const uint64_t cnt = (n - 1) / r + 1;
    if (idx_bytes == 4)
        GSAIS_COUNTED((k_aux<int32_t><<<grid_for(cnt, 256), 256, 0, st>>>(d_isa1, n, r, static_cast<int32_t *>(d_I))));
    else
        GSAIS_COUNTED((k_aux<int64_t><<<grid_for(cnt, 256), 256, 0, st>>>(d_isa1, n, r, static_cast<int64_t *>(d_I))));
    return cudaGetLastError();
}

cudaError_t widen_u32_to_i64(const uint32_t *src, int64_t *dst, uint64_t n, cudaStream_t st)
{
    if (n == 0) return cudaSuccess;
    GSAIS_COUNTED((k_widen<<<grid_for(n, 256), 256, 0, st>>>(src, dst, n)));
    return cudaGetLastError();
}

cudaError_t narrow_i64_to_u32(const int64_t *src, uint32_t *dst, uint64_t n, uint32_t *err, cudaStream_t st)
{
    if (n == 0) return cudaSuccess;
    GSAIS_COUNTED((k_narrow<<<grid_for(n, 256), 256, 0, st>>>(src, dst, n, err)));
    return cudaGetLastError();
}

size_t plcp_sparse_words(uint64_t n) { return plcp_scratch_layout(n).total; }

cudaError_t plcp_build(const void *d_T, int symbytes, const uint32_t *d_SA, uint64_t n, bool gsa, uint32_t *d_PLCP,
                       uint32_t *d_sparse, uint32_t *h_hist, uint32_t *err, cudaStream_t st)
{
    if (n == 0) return cudaSuccess;
    if (symbytes == 4) {   // integer symbols (libsais_plcp_int, src/libsais.c:8399): plain stop rule
        const uint32_t *T = static_cast<const uint32_t *>(d_T);
        return plcp_run<uint32_t, false, 0>(T, d_SA, n, d_PLCP, d_sparse, err, st);
    }
    if (symbytes == 1) {
        const uint8_t *T = static_cast<const uint8_t *>(d_T);
        return gsa ? plcp_dispatch<uint8_t, true>(T, d_SA, n, d_PLCP, d_sparse, h_hist, err, st)
                   : plcp_dispatch<uint8_t, false>(T, d_SA, n, d_PLCP, d_sparse, h_hist, err, st);
    }
    const uint16_t *T = static_cast<const uint16_t *>(d_T);
    return gsa ? plcp_dispatch<uint16_t, true>(T, d_SA, n, d_PLCP, d_sparse, h_hist, err, st)
               : plcp_dispatch<uint16_t, false>(T, d_SA, n, d_PLCP, d_sparse, h_hist, err, st);
}

cudaError_t byte_presence(const uint8_t *d_T, uint64_t n, uint32_t *d_map, cudaStream_t st)
{
    cudaError_t e = cudaMemsetAsync(d_map, 0, 8 * sizeof(uint32_t), st);
    if (e != cudaSuccess || n == 0) return e;
    GSAIS_COUNTED((k_presence_u8<<<grid_for(n / 16 + 1, 256), 256, 0, st>>>(d_T, n, d_map)));
    return cudaGetLastError();
}

cudaError_t int_alphabet_scan(const void *d_T, int tbytes, uint64_t n, int64_t k, unsigned long long *d_out,
                              cudaStream_t st)
{
    cudaError_t e = cudaMemsetAsync(d_out, 0, 2 * sizeof(unsigned long long), st);
    if (e != cudaSuccess || n == 0) return e;
    if (tbytes == 4)
        GSAIS_COUNTED((k_int_scan<int32_t><<<grid_for(n, 256), 256, 0, st>>>(static_cast<const int32_t *>(d_T), n, k,
                                                                           d_out)));
    else
        GSAIS_COUNTED((k_int_scan<int64_t><<<grid_for(n, 256), 256, 0, st>>>(static_cast<const int64_t *>(d_T), n, k,
                                                                           d_out)));
    return cudaGetLastError();
}

cudaError_t int_narrow(const void *d_T, int tbytes, uint64_t n, void *d_out, int obytes, cudaStream_t st)
{
    if (n == 0) return cudaSuccess;
    const int g = grid_for(n, 256);
    if (tbytes == 4 && obytes == 2)
        GSAIS_COUNTED((k_int_narrow<int32_t, uint16_t><<<g, 256, 0, st>>>(static_cast<const int32_t *>(d_T), n,
                                                                           static_cast<uint16_t *>(d_out))));
    else if (tbytes == 8 && obytes == 2)
        GSAIS_COUNTED((k_int_narrow<int64_t, uint16_t><<<g, 256, 0, st>>>(static_cast<const int64_t *>(d_T), n,
                                                                           static_cast<uint16_t *>(d_out))));
    else if (tbytes == 8 && obytes == 4)
        GSAIS_COUNTED((k_int_narrow<int64_t, uint32_t><<<g, 256, 0, st>>>(static_cast<const int64_t *>(d_T), n,
                                                                           static_cast<uint32_t *>(d_out))));
    else
        return cudaErrorInvalidValue;
    return cudaGetLastError();
}

size_t lcp_scratch_words(uint64_t n)
{
    if (!lcp_partitioned(n)) return 0;
    const uint64_t tiles = (n + kLcpTile - 1) / kLcpTile;
    const uint64_t np = (n + 63) / 64 * 64;
    return (size_t)(np + np / 2 + tiles * 2 * kLcpBuckets + kLcpBuckets);
}

cudaError_t lcp_gather(const uint32_t *d_PLCP, const uint32_t *d_SA, uint32_t *d_LCP, uint64_t n, uint32_t *scratch,
                       uint32_t *err, cudaStream_t st)
{
    if (n == 0) return cudaSuccess;
    if (!lcp_partitioned(n) || !scratch) {
        GSAIS_COUNTED((k_lcp<<<grid_for(n, 256), 256, 0, st>>>(d_PLCP, d_SA, d_LCP, n, err)));
        return cudaGetLastError();
    }
    const int shift = lcp_shift(n);
    const uint64_t tiles = (n + kLcpTile - 1) / kLcpTile;
    const uint64_t np = (n + 63) / 64 * 64;
    uint32_t *pos = scratch;
    uint16_t *place = reinterpret_cast<uint16_t *>(scratch + np);
    uint32_t *runs = scratch + np + np / 2, *cursor = runs + tiles * 2 * kLcpBuckets;
    GSAIS_COUNTED((k_lcp_cursors<<<1, kLcpBuckets, 0, st>>>(cursor, shift, n)));
    GSAIS_COUNTED((k_lcp_partition<<<(unsigned)tiles, kLcpThreads, 0, st>>>(d_SA, n, shift, cursor, runs, pos, place,
                                                                           err)));
    GSAIS_COUNTED((k_lcp_fetch<<<grid_for(n, 256), 256, 0, st>>>(d_PLCP, pos, n, err)));
    GSAIS_COUNTED((k_lcp_place<<<(unsigned)tiles, kLcpThreads, 0, st>>>(n, runs, place, pos, d_LCP)));
    return cudaGetLastError();
}

}  // namespace gsais
