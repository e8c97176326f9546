// outputs.cu -- BWT gather, auxiliary ISA samples, Phi-array PLCP and the
// LCP permute, for sm_103a.  All are HBM-bound gathers/scatters.
//
// Every index read from an array (SA entries, Phi entries) is checked against
// n before it is used as an address; a bad index raises GSAIS_ERR_BOUNDS in
// the context's error word and the access is skipped, so a malformed caller
// array becomes a -2 return instead of a device fault.
#include "device_util.cuh"
#include "engine.h"
#include "outputs.cuh"

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

// Phi[SA[j]] = SA[j-1], Phi[SA[0]] = n (src/libsais.c:8116 compute_phi).
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

// Length of the common prefix of suffixes a and b, known to be >= l0,
// extended by one warp 32 symbols per step.  Plain texts stop at the text
// end (src/libsais.c:8177: m = n - max(i, k)); GSA stops at a separator.
template <typename Sym, bool GSA>
__device__ __forceinline__ uint64_t warp_extend(const Sym *__restrict__ T, uint64_t n, uint64_t a, uint64_t b,
                                                uint64_t l0)
{
    const int lane = threadIdx.x & 31;
    const uint64_t m = n - (a > b ? a : b);
    if (l0 > m) l0 = m;
    for (;;) {
        const uint64_t x = l0 + lane;
        bool match;
        if (!GSA) {
            match = x < m && T[a + x] == T[b + x];
        } else {
            match = x < m && T[a + x] != 0 && T[a + x] == T[b + x];
        }
        const uint32_t bad = __ballot_sync(GSAIS_FULL_MASK, !match);
        if (bad) return l0 + (uint64_t)(__ffs(bad) - 1);
        l0 += 32;
    }
}

// One level of exact PLCP values at chunk starts: chunk k = (2w+1)*half
// takes its lower bound from chunk k - half (PLCP[i+d] >= PLCP[i] - d).
template <typename Sym, bool GSA>
__global__ void __launch_bounds__(256) k_plcp_level(const Sym *__restrict__ T, uint64_t n,
                                                    const uint32_t *__restrict__ phi, uint32_t chunk,
                                                    uint64_t nchunks, uint64_t half, uint32_t *__restrict__ sparse,
                                                    uint32_t *__restrict__ err)
{
    const uint64_t w = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t k = half == 0 ? w : (2 * w + 1) * half;
    if (k >= nchunks || (half == 0 && k > 0)) return;
    const uint64_t a = k * chunk;
    uint64_t b = phi[a];
    if (b > n) {
        if ((threadIdx.x & 31) == 0) atomicOr(err, GSAIS_ERR_BOUNDS);
        b = n;
    }
    uint64_t l = 0;
    if (b != n) {
        uint64_t lb = 0;
        if (half != 0) {
            const uint64_t kp = k - half;
            const uint64_t d = a - kp * chunk;
            const uint64_t lp = sparse[kp];
            lb = lp > d ? lp - d : 0;
        }
        l = warp_extend<Sym, GSA>(T, n, a, b, lb);
    }
    if ((threadIdx.x & 31) == 0) sparse[k] = (uint32_t)l;
}

// Kasai's carried length inside each chunk, starting from the exact value at
// the chunk start (src/libsais.c:8167 compute_plcp restarts at block starts
// too).  Phi is read and overwritten by PLCP in place.
template <typename Sym, bool GSA>
__global__ void __launch_bounds__(256) k_plcp_chunks(const Sym *__restrict__ T, uint64_t n, uint32_t chunk,
                                                     uint64_t nchunks, const uint32_t *__restrict__ sparse,
                                                     uint32_t *__restrict__ plcp, uint32_t *__restrict__ err)
{
    const uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nchunks) return;
    const uint64_t a = k * chunk;
    const uint64_t e = a + chunk < n ? a + chunk : n;
    uint64_t l = sparse[k];
    plcp[a] = (uint32_t)l;
    for (uint64_t x = a + 1; x < e; ++x) {
        uint64_t b = plcp[x];
        if (b > n) {
            atomicOr(err, GSAIS_ERR_BOUNDS);
            b = n;
        }
        if (b == n) {
            l = 0;
        } else {
            l = l ? l - 1 : 0;
            const uint64_t m = n - (x > b ? x : b);
            if (l > m) l = m;
            if (!GSA) {
                while (l < m && T[x + l] == T[b + l]) ++l;
            } else {
                while (l < m && T[x + l] != 0 && T[x + l] == T[b + l]) ++l;
            }
        }
        plcp[x] = (uint32_t)l;
    }
}

// LCP[i] = PLCP[SA[i]] (src/libsais.c:8311 compute_lcp).  Bytes: 12 per row.
__global__ void __launch_bounds__(256) k_lcp(const uint32_t *__restrict__ plcp, const uint32_t *__restrict__ SA,
                                             uint32_t *__restrict__ lcp, uint64_t n, uint32_t *__restrict__ err)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const uint64_t s = SA[i];
        if (s >= n) {
            atomicOr(err, GSAIS_ERR_BOUNDS);
            continue;
        }
        lcp[i] = plcp[s];
    }
}

constexpr uint32_t kPlcpChunk = 64;

template <typename Sym, bool GSA>
cudaError_t plcp_run(const Sym *T, const uint32_t *SA, uint64_t n, uint32_t *plcp, uint32_t *sparse, uint32_t *err,
                     cudaStream_t st)
{
    GSAIS_COUNTED((k_phi<<<grid_for(n, 256), 256, 0, st>>>(SA, n, plcp, err)));
    const uint64_t nchunks = (n + kPlcpChunk - 1) / kPlcpChunk;
    // level 0: chunk 0 from scratch
    GSAIS_COUNTED((k_plcp_level<Sym, GSA><<<1, 32, 0, st>>>(T, n, plcp, kPlcpChunk, nchunks, 0, sparse, err)));
    uint64_t top = 1;
    while (top < nchunks) top <<= 1;
    for (uint64_t half = top >> 1; half >= 1; half >>= 1) {
        const uint64_t count = nchunks > half ? (nchunks - half + 2 * half - 1) / (2 * half) : 0;
        if (count == 0) continue;
        const uint64_t threads = count * 32;
        const unsigned blocks = (unsigned)((threads + 255) / 256);
        GSAIS_COUNTED(
            (k_plcp_level<Sym, GSA><<<blocks, 256, 0, st>>>(T, n, plcp, kPlcpChunk, nchunks, half, sparse, err)));
    }
    GSAIS_COUNTED((k_plcp_chunks<Sym, GSA><<<(unsigned)((nchunks + 255) / 256), 256, 0, st>>>(
        T, n, kPlcpChunk, nchunks, sparse, plcp, err)));
    return cudaGetLastError();
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

size_t plcp_sparse_words(uint64_t n) { return (size_t)((n + kPlcpChunk - 1) / kPlcpChunk + 1); }

cudaError_t plcp_build(const void *d_T, int symbytes, const uint32_t *d_SA, uint64_t n, bool gsa, uint32_t *d_PLCP,
                       uint32_t *d_sparse, uint32_t *err, cudaStream_t st)
{
    if (n == 0) return cudaSuccess;
    if (symbytes == 4) {   // integer symbols (libsais_plcp_int, src/libsais.c:8399): plain stop rule
        const uint32_t *T = static_cast<const uint32_t *>(d_T);
        return plcp_run<uint32_t, false>(T, d_SA, n, d_PLCP, d_sparse, err, st);
    }
    if (symbytes == 1) {
        const uint8_t *T = static_cast<const uint8_t *>(d_T);
        return gsa ? plcp_run<uint8_t, true>(T, d_SA, n, d_PLCP, d_sparse, err, st)
                   : plcp_run<uint8_t, false>(T, d_SA, n, d_PLCP, d_sparse, err, st);
    }
    const uint16_t *T = static_cast<const uint16_t *>(d_T);
    return gsa ? plcp_run<uint16_t, true>(T, d_SA, n, d_PLCP, d_sparse, err, st)
               : plcp_run<uint16_t, false>(T, d_SA, n, d_PLCP, d_sparse, err, st);
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

cudaError_t lcp_gather(const uint32_t *d_PLCP, const uint32_t *d_SA, uint32_t *d_LCP, uint64_t n, uint32_t *err,
                       cudaStream_t st)
{
    if (n == 0) return cudaSuccess;
    GSAIS_COUNTED((k_lcp<<<grid_for(n, 256), 256, 0, st>>>(d_PLCP, d_SA, d_LCP, n, err)));
    return cudaGetLastError();
}

}  // namespace gsais
