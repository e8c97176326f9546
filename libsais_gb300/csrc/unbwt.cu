// unbwt.cu -- inverse Burrows-Wheeler transform on the GPU (libsais_unbwt*,
// src/libsais.c:7326-8112 of the reference, which decodes with a bigram
// LF table on the CPU).
//
// Rows of the BWT matrix are numbered 0..n: row 0 is the empty suffix, row r
// >= 1 the suffix SA[r-1].  U (the libsais_bwt output) is the last column
// with the primary row p (the row of suffix 0, whose last symbol is the
// sentinel) left out: U[k] sits in row k for k < p and row k + 1 for k >= p.
//
//   1. One stable radix pass over (U[k], row) orders the rows by their last
//      symbol: the q-th row of that order (q >= 1; q = 0 is the sentinel row
//      p) is Psi(q), the row of the suffix one position further in the text,
//      and the symbol F(q) is the first symbol of row q.  Psi and F are packed
//      into one 64-bit word per row, so a step of the walk below reads one
//      sector.
//   2. The text is the walk T[i] = F(Psi^i(p)), i = 0..n-1.  Rows that are
//      multiples of `gap`, and p, are splitters; every splitter walks (in
//      parallel) to the next splitter and records the step count.
//   3. Pointer jumping over the splitter list gives each splitter its distance
//      to row 0 (the end of the text), i.e. the text position of its suffix.
//   4. Every splitter walks again and writes its stretch of the text.
// Walks are bounded by n + 1 steps; a malformed input (a row that is not on
// p's cycle) raises the error word instead of looping.
#include "device_util.cuh"
#include "engine.h"
#include "unbwt.cuh"

namespace gsais {

namespace {

int unbwt_grid(uint64_t items)
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const uint64_t want = (items + 255) / 256;
    const uint64_t cap = (uint64_t)(sms > 0 ? sms : 1) * 8;
    return (int)(want < 1 ? 1 : (want < cap ? want : cap));
}

template <typename Sym>
__global__ void __launch_bounds__(256) k_unbwt_keys(const Sym *__restrict__ U, uint64_t n, uint64_t p,
                                                    uint32_t *__restrict__ keys, uint32_t *__restrict__ rows)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride) {
        keys[k] = U[k];
        rows[k] = (uint32_t)(k < p ? k : k + 1);
    }
}

// PF[q] = Psi(q) | F(q) << 32; PF[0] = p (the sentinel row, F unused).
__global__ void __launch_bounds__(256) k_unbwt_pack(const uint32_t *__restrict__ keys,
                                                    const uint32_t *__restrict__ rows, uint64_t n, uint64_t p,
                                                    uint64_t *__restrict__ PF)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; q <= n; q += stride)
        PF[q] = q == 0 ? p : ((uint64_t)rows[q - 1] | ((uint64_t)keys[q - 1] << 32));
}

struct Splitters {
    uint64_t gap;   // rows that are multiples of gap are splitters ...
    uint64_t m0;    // ... with ids row / gap, 0 <= id < m0
    uint64_t p;     // the primary row; id m0 when p is not a multiple of gap
    uint64_t m;     // splitter count
    __device__ __forceinline__ uint64_t row_of(uint64_t s) const { return s < m0 ? s * gap : p; }
    __device__ __forceinline__ bool is_splitter(uint64_t row) const { return row % gap == 0 || row == p; }
    __device__ __forceinline__ uint64_t id_of(uint64_t row) const { return row % gap == 0 ? row / gap : m0; }
};

// Walk from every splitter to the next one: next[s], len[s] (the number of
// text symbols the stretch covers).  Row 0 (the end of the text) is the
// terminal: next = itself, len = 0.
__global__ void __launch_bounds__(256) k_unbwt_walk(const uint64_t *__restrict__ PF, uint64_t n, Splitters sp,
                                                    uint32_t *__restrict__ next, uint32_t *__restrict__ len,
                                                    uint32_t *__restrict__ err)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; s < sp.m; s += stride) {
        uint64_t row = sp.row_of(s);
        if (row == 0) {
            next[s] = 0;
            len[s] = 0;
            continue;
        }
        uint64_t cnt = 0;
        do {
            row = (uint32_t)PF[row];
            ++cnt;
        } while (!sp.is_splitter(row) && row <= n && cnt <= n);
        if (row > n || cnt > n) {
            atomicOr(err, GSAIS_ERR_BOUNDS);
            next[s] = 0;
            len[s] = 0;
            continue;
        }
        next[s] = (uint32_t)sp.id_of(row);
        len[s] = (uint32_t)cnt;
    }
}

// One pointer-jumping step: D'[s] = D[s] + D[N[s]], N'[s] = N[N[s]].
__global__ void __launch_bounds__(256) k_unbwt_jump(const uint32_t *__restrict__ N, const uint32_t *__restrict__ D,
                                                    uint64_t m, uint32_t *__restrict__ N2, uint32_t *__restrict__ D2)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; s < m; s += stride) {
        const uint32_t t = N[s];
        N2[s] = N[t];
        D2[s] = D[s] + D[t];
    }
}

// Every splitter writes its stretch: the suffix of row_of(s) is text position
// n - dist[s].  A splitter not on p's cycle (next != terminal), or a
// stretch outside the text, raises the error word.
template <typename Sym>
__global__ void __launch_bounds__(256) k_unbwt_emit(const uint64_t *__restrict__ PF, uint64_t n, Splitters sp,
                                                    const uint32_t *__restrict__ N, const uint32_t *__restrict__ dist,
                                                    const uint32_t *__restrict__ len, Sym *__restrict__ out,
                                                    uint32_t *__restrict__ err)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; s < sp.m; s += stride) {
        uint64_t row = sp.row_of(s);
        if (row == 0) continue;
        const uint64_t d = dist[s], l = len[s];
        if (N[s] != 0 || d > n || d < l || (row == sp.p && d != n)) {
            atomicOr(err, GSAIS_ERR_BOUNDS);
            continue;
        }
        uint64_t i = n - d;
        for (uint64_t j = 0; j < l; ++j) {
            const uint64_t w = PF[row];
            out[i + j] = (Sym)(w >> 32);
            row = (uint32_t)w;
            if (row > n) {
                atomicOr(err, GSAIS_ERR_BOUNDS);
                break;
            }
        }
    }
}

}  // namespace

size_t unbwt_workspace_bytes(uint64_t n)
{
    const size_t A = 256;
    const uint64_t m = n / unbwt_gap(n) + 2;
    size_t s = 0;
    s += 4 * align_up_to(n * 4, A);             // keys x2, rows x2
    s += align_up_to((n + 1) * 8, A);           // PF
    s += 6 * align_up_to(m * 4, A);             // next/dist x2, len, spare
    s += 2 * align_up_to(8 * 256 * 4, A);       // radix hist + bases
    s += align_up_to(8 * 4, A);                 // radix counters
    s += align_up_to(radix_status_words(n) * 8, A);
    return s;
}

uint64_t unbwt_gap(uint64_t n) { return n >= (1ull << 24) ? 64 : (n >= (1ull << 16) ? 32 : 8); }

cudaError_t unbwt_run(const void *d_U, int symbytes, uint64_t n, uint64_t p, void *d_out, void *scratch,
                      uint32_t *h_hist, KernelProfiler *prof, uint32_t *d_err, cudaStream_t st)
{
    if (n == 0) return cudaSuccess;
    const size_t A = 256;
    char *c = static_cast<char *>(scratch);
    auto take = [&](size_t bytes) {
        char *r = c;
        c += align_up_to(bytes, A);
        return r;
    };
    uint32_t *keys[2], *rows[2];
    for (int i = 0; i < 2; ++i) keys[i] = reinterpret_cast<uint32_t *>(take(n * 4));
    for (int i = 0; i < 2; ++i) rows[i] = reinterpret_cast<uint32_t *>(take(n * 4));
    uint64_t *PF = reinterpret_cast<uint64_t *>(take((n + 1) * 8));
    Splitters sp;
    sp.gap = unbwt_gap(n);
    sp.m0 = n / sp.gap + 1;
    sp.p = p;
    sp.m = sp.m0 + (p % sp.gap ? 1 : 0);
    const uint64_t mcap = n / sp.gap + 2;
    uint32_t *N[2], *D[2];
    N[0] = reinterpret_cast<uint32_t *>(take(mcap * 4));
    N[1] = reinterpret_cast<uint32_t *>(take(mcap * 4));
    D[0] = reinterpret_cast<uint32_t *>(take(mcap * 4));
    D[1] = reinterpret_cast<uint32_t *>(take(mcap * 4));
    uint32_t *len = reinterpret_cast<uint32_t *>(take(mcap * 4));
    take(mcap * 4);
    RadixScratch rs;
    rs.hist = reinterpret_cast<uint32_t *>(take(8 * 256 * 4));
    rs.bases = reinterpret_cast<uint32_t *>(take(8 * 256 * 4));
    rs.counters = reinterpret_cast<uint32_t *>(take(8 * 4));
    rs.status_words = radix_status_words(n);
    rs.status = reinterpret_cast<uint64_t *>(take(rs.status_words * 8));
    rs.h_hist = h_hist;
    rs.prof = prof;

    cudaEvent_t ev = prof ? prof->begin(st) : nullptr;
    const int g = unbwt_grid(n);
    if (symbytes == 1)
        GSAIS_COUNTED((k_unbwt_keys<uint8_t><<<g, 256, 0, st>>>(static_cast<const uint8_t *>(d_U), n, p, keys[0],
                                                                 rows[0])));
    else
        GSAIS_COUNTED((k_unbwt_keys<uint16_t><<<g, 256, 0, st>>>(static_cast<const uint16_t *>(d_U), n, p, keys[0],
                                                                  rows[0])));
    int which = 0, ran = 0;
    cudaError_t e = radix_sort_pairs32(keys, rows, n, 8 * symbytes, rs, d_err, st, &which, &ran, false);
    if (e != cudaSuccess) return e;
    GSAIS_COUNTED((k_unbwt_pack<<<unbwt_grid(n + 1), 256, 0, st>>>(keys[which], rows[which], n, p, PF)));
    const int gm = unbwt_grid(sp.m);
    GSAIS_COUNTED((k_unbwt_walk<<<gm, 256, 0, st>>>(PF, n, sp, N[0], len, d_err)));
    if ((e = cudaMemcpyAsync(D[0], len, sp.m * 4, cudaMemcpyDeviceToDevice, st)) != cudaSuccess) return e;
    int cur = 0;
    for (uint64_t span = 1; span < sp.m; span <<= 1) {
        GSAIS_COUNTED((k_unbwt_jump<<<gm, 256, 0, st>>>(N[cur], D[cur], sp.m, N[cur ^ 1], D[cur ^ 1])));
        cur ^= 1;
    }
    if (symbytes == 1)
        GSAIS_COUNTED((k_unbwt_emit<uint8_t><<<gm, 256, 0, st>>>(PF, n, sp, N[cur], D[cur], len,
                                                                  static_cast<uint8_t *>(d_out), d_err)));
    else
        GSAIS_COUNTED((k_unbwt_emit<uint16_t><<<gm, 256, 0, st>>>(PF, n, sp, N[cur], D[cur], len,
                                                                   static_cast<uint16_t *>(d_out), d_err)));
    // bytes: BWT read, text written (the walks' random reads are not counted)
    if (ev) prof->end(KK_UNBWT, ev, st, 2 * n * symbytes);
    return cudaGetLastError();
}

}  // namespace gsais
