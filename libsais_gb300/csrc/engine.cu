// engine.cu -- device contexts, workspace arena and the C-ABI entry points
// that the libsais-compatible shim (api.c) and direct device users call.
//
// A context maps libsais's LIBSAIS_CONTEXT (src/libsais.c:63-99, 176-266:
// buckets + per-thread state reused across calls) onto GPU resources: one
// CUDA stream, one device workspace arena that grows to the high-water mark
// of the calls made on it, pinned host scratch for small read-backs, and a
// device error word for bounded spin-waits.  The context-less libsais calls
// share one process-wide context behind its mutex.
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "device_util.cuh"
#include "engine.h"
#include "gsais.h"
#include "libsais_gb300.h"
#include "outputs.cuh"
#include "unbwt.cuh"
#include "suffix_sort.cuh"

using namespace gsais;

struct gsais_ctx {
    std::mutex mu;
    bool ready = false;
    int device = -1;
    cudaStream_t stream = nullptr;
    cudaStream_t copy_stream = nullptr;   // device->host copies that overlap later kernels
    cudaStream_t side_stream = nullptr;   // early BWT and SA patch, beside the sort and the copies
    cudaEvent_t early_ev = nullptr;       // SA may leave for the host (EarlySaCopy)
    cudaEvent_t copied_ev = nullptr;      // the early SA copy has landed
    cudaEvent_t bwt_ev = nullptr;         // the early BWT is done
    cudaEvent_t upload_ev = nullptr;      // a chunk of the text has arrived
    void *arena = nullptr;
    size_t arena_bytes = 0;
    uint32_t *d_misc = nullptr;   // [0] error word, [1] validity flag
    uint32_t *h_small = nullptr;  // pinned: 16 + 65536 hist words + 65536 u16 codes
    uint32_t *h_hist = nullptr;   // pinned: radix histograms
    SortOptions opt;
    SortStats stats;
    KernelProfiler prof;
};

namespace {

constexpr size_t kAlign = 256;
constexpr size_t kSmallWords = kHostSmallWords;
constexpr uint64_t kMaxN = 0xFFFFFFFFull;   // 32-bit internal indices

inline size_t align_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev)
    {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (dev >= 0 && dev != prev) cudaSetDevice(dev);
    }
    ~DeviceGuard()
    {
        int cur = -1;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
    }
};

bool ctx_init(gsais_ctx *c)
{
    if (c->ready) return true;
    if (cudaGetDevice(&c->device) != cudaSuccess) return false;
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) return false;
    if (cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking) != cudaSuccess) return false;
    if (cudaStreamCreateWithFlags(&c->side_stream, cudaStreamNonBlocking) != cudaSuccess) return false;
    if (cudaEventCreateWithFlags(&c->early_ev, cudaEventDisableTiming) != cudaSuccess) return false;
    if (cudaEventCreateWithFlags(&c->copied_ev, cudaEventDisableTiming) != cudaSuccess) return false;
    if (cudaEventCreateWithFlags(&c->bwt_ev, cudaEventDisableTiming) != cudaSuccess) return false;
    if (cudaEventCreateWithFlags(&c->upload_ev, cudaEventDisableTiming) != cudaSuccess) return false;
    if (cudaMalloc(&c->d_misc, 64) != cudaSuccess) return false;
    if (cudaMemset(c->d_misc, 0, 64) != cudaSuccess) return false;
    if (cudaMallocHost(&c->h_small, kSmallWords * sizeof(uint32_t)) != cudaSuccess) return false;
    if (cudaMallocHost(&c->h_hist, 8 * 256 * sizeof(uint32_t)) != cudaSuccess) return false;
    c->ready = true;
    return true;
}

// Test hook: the next g_fail_allocs workspace allocations fail as if the
// device were out of memory (gsais_test_fail_allocations).
std::atomic<int32_t> g_fail_allocs{0};

bool ensure_arena(gsais_ctx *c, size_t bytes)
{
    if (c->arena_bytes >= bytes) return true;
    for (int32_t k = g_fail_allocs.load(); k > 0;)
        if (g_fail_allocs.compare_exchange_weak(k, k - 1)) return false;
    if (c->arena) {
        cudaFree(c->arena);
        c->arena = nullptr;
        c->arena_bytes = 0;
    }
    const size_t want = (bytes + ((size_t)2 << 20) - 1) / ((size_t)2 << 20) * ((size_t)2 << 20);
    if (cudaMalloc(&c->arena, want) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    c->arena_bytes = want;
    return true;
}

struct Carver {
    char *p;
    explicit Carver(void *base) : p(static_cast<char *>(base)) {}
    template <typename T>
    T *take(size_t count)
    {
        T *r = reinterpret_cast<T *>(p);
        p += align_up(count * sizeof(T));
        return r;
    }
};

// Clears the device error word; returns false on CUDA failure.
bool clear_err(gsais_ctx *c, cudaStream_t st) { return cudaMemsetAsync(c->d_misc, 0, 8, st) == cudaSuccess; }

// Synchronises the stream and turns a raised device error word into an error.
cudaError_t sync_checked(gsais_ctx *c, cudaStream_t st)
{
    cudaError_t e = cudaMemcpyAsync(c->h_small + 8, c->d_misc, 4, cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess) return e;
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
    return c->h_small[8] ? cudaErrorUnknown : cudaSuccess;
}

void emit_freq(const uint32_t *h_hist, int symbytes, void *freq, int freq_bytes)
{
    if (!freq) return;
    const int k = symbytes == 1 ? 256 : 65536;
    if (freq_bytes == 8) {
        int64_t *f = static_cast<int64_t *>(freq);
        for (int c = 0; c < k; ++c) f[c] = h_hist[c];
    } else {
        int32_t *f = static_cast<int32_t *>(freq);
        for (int c = 0; c < k; ++c) f[c] = (int32_t)h_hist[c];
    }
}

gsais_ctx *resolve(void *ctx) { return ctx ? static_cast<gsais_ctx *>(ctx) : gsais_default_ctx(); }

int64_t fail(cudaError_t)
{
    cudaGetLastError();   // clear a non-sticky error so the context stays usable
    return -2;
}

#define GS_TRY(expr)                                         \
    do {                                                     \
        cudaError_t _e = (expr);                             \
        if (_e != cudaSuccess) return fail(_e);              \
    } while (0)

// The device's address of a pinned (page-locked) host buffer, or nullptr.
void *pinned_view(void *p)
{
    cudaPointerAttributes a;
    if (!p || cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

// Slots an early SA copy may patch: at most n / 8 (more would make the
// patch cost a sizable part of the copy it saves).
inline uint64_t early_patch_cap(uint64_t n) { return n / 8; }

// Sets up an early copy of the int32 SA into the caller's pinned buffer,
// when it is one; the patch list comes from the arena (taken before the
// sort workspace).
bool early_setup(gsais_ctx *c, EarlySaCopy &ec, void *SA, int sa_bytes, uint64_t n, Carver &cv)
{
    if (sa_bytes != 4 || !SA) return false;
    void *dev = pinned_view(SA);
    if (!dev) return false;
    ec.host = static_cast<int32_t *>(SA);
    ec.host_dev = static_cast<int32_t *>(dev);
    ec.stream = c->copy_stream;
    ec.ready = c->early_ev;
    ec.copied = c->copied_ev;
    ec.patch_cap = early_patch_cap(n);
    ec.bits = cv.take<uint32_t>((n + 31) / 32);
    return true;
}

inline size_t early_bytes(void *SA, int sa_bytes, uint64_t n)
{
    return sa_bytes == 4 && pinned_view(SA) ? align_up((n + 31) / 32 * 4) : 0;
}

// A BWT-only call (no SA wanted) into a pinned U: the early point copies no
// SA, but the BWT is gathered and leaves while the rounds run, and the slots
// the rounds still write are recorded for the patch of their BWT rows.
bool early_setup_bwt_only(gsais_ctx *c, EarlySaCopy &ec, uint64_t n, Carver &cv)
{
    ec.host = nullptr;
    ec.host_dev = nullptr;
    ec.stream = c->copy_stream;
    ec.ready = c->early_ev;
    ec.copied = c->copied_ev;
    ec.patch_cap = early_patch_cap(n);
    ec.bits = cv.take<uint32_t>((n + 31) / 32);
    return true;
}

// Waits for a stream when it goes out of scope.
struct StreamJoin {
    cudaStream_t s;
    ~StreamJoin()
    {
        if (s) cudaStreamSynchronize(s);
    }
};

PackedText packed_of(const SortWorkspace &ws)
{
    PackedText pk;
    pk.packed = ws.packed;
    pk.pack_bits = ws.pack_bits;
    for (int c = 0; c < 16; ++c) pk.decode[c] = ws.decode[c];
    return pk;
}

// Workspace for one suffix sort carved after `extra` bytes of call buffers.
struct SortPlan {
    size_t sort_bytes;
    size_t total;
};

SortPlan plan_sort(uint64_t n, int symbytes, size_t extra)
{
    SortPlan p;
    p.sort_bytes = sort_workspace_bytes(n, symbytes);
    p.total = extra + p.sort_bytes;
    return p;
}

// Sort a device text already placed in the arena.  `sa_override` (nullable)
// receives SA directly when the caller wants uint32 output in its own buffer.
// Uploads the text on st in chunks, the symbol histogram following each
// chunk on xs, so the histogram costs no time of its own; small texts (and
// other symbol widths) go in one copy and the sort counts them itself.
// *hist_ready: ws.hist holds the histogram (pass it to run_sort).
cudaError_t upload_text(gsais_ctx *c, void *d_T, const void *T, int symbytes, uint64_t n, SortWorkspace &ws,
                        cudaStream_t st, cudaStream_t xs, bool *hist_ready)
{
    *hist_ready = false;
    if (n < (1ull << 24) || (symbytes != 1 && symbytes != 2))
        return cudaMemcpyAsync(d_T, T, n * symbytes, cudaMemcpyHostToDevice, st);
    cudaError_t e;
    if ((e = cudaMemsetAsync(ws.hist, 0, (size_t)(symbytes == 1 ? 256 : 65536) * 4, xs)) != cudaSuccess) return e;
    const uint64_t chunk = 1ull << 25;   // symbols per copy
    for (uint64_t off = 0; off < n; off += chunk) {
        const uint64_t len = n - off < chunk ? n - off : chunk;
        char *dst = static_cast<char *>(d_T) + off * symbytes;
        if ((e = cudaMemcpyAsync(dst, static_cast<const char *>(T) + off * symbytes, len * symbytes,
                                 cudaMemcpyHostToDevice, st)) != cudaSuccess ||
            (e = cudaEventRecord(c->upload_ev, st)) != cudaSuccess ||
            (e = cudaStreamWaitEvent(xs, c->upload_ev, 0)) != cudaSuccess ||
            (e = symbol_histogram_part(dst, symbytes, len, ws.hist, xs)) != cudaSuccess)
            return e;
    }
    if ((e = cudaEventRecord(c->upload_ev, xs)) != cudaSuccess || (e = cudaStreamWaitEvent(st, c->upload_ev, 0)) !=
                                                                       cudaSuccess)
        return e;
    *hist_ready = true;
    return cudaSuccess;
}

// counts: the caller returns symbol counts (freq); without them an 8-bit
// text's codes come from a presence map.
int64_t run_sort(gsais_ctx *c, const void *d_T, int symbytes, uint64_t n, bool gsa, SortWorkspace &ws,
                 cudaStream_t st, uint32_t raw_max = 0, EarlySaCopy *early = nullptr, bool hist_ready = false,
                 bool counts = true)
{
    if (gsa) {
        bool valid = true;
        GS_TRY(gsa_validate(d_T, symbytes, n, c->d_misc + 1, c->h_small, st, &valid));
        if (!valid) return -1;
    }
    ws.radix.prof = &c->prof;
    SortOptions opt = c->opt;
    opt.raw_max = raw_max;
    opt.early = early;
    opt.hist_ready = hist_ready;
    opt.presence_only = !counts;
    GS_TRY(suffix_sort(d_T, symbytes, n, gsa, ws, opt, c->d_misc, st, &c->stats));
    return 0;
}

}  // namespace

// ------------------------------------------------------------------ C ABI
extern "C" {

gsais_ctx *gsais_ctx_create(void)
{
    gsais_ctx *c = new (std::nothrow) gsais_ctx();
    return c;
}

void gsais_ctx_destroy(gsais_ctx *c)
{
    if (!c) return;
    if (c->ready) {
        DeviceGuard g(c->device);
        if (c->stream) cudaStreamSynchronize(c->stream);
        if (c->copy_stream) cudaStreamSynchronize(c->copy_stream);
        if (c->side_stream) cudaStreamSynchronize(c->side_stream);
        if (c->arena) cudaFree(c->arena);
        if (c->d_misc) cudaFree(c->d_misc);
        if (c->h_small) cudaFreeHost(c->h_small);
        if (c->h_hist) cudaFreeHost(c->h_hist);
        if (c->stream) cudaStreamDestroy(c->stream);
        if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
        if (c->side_stream) cudaStreamDestroy(c->side_stream);
        if (c->early_ev) cudaEventDestroy(c->early_ev);
        if (c->copied_ev) cudaEventDestroy(c->copied_ev);
        if (c->bwt_ev) cudaEventDestroy(c->bwt_ev);
        if (c->upload_ev) cudaEventDestroy(c->upload_ev);
    }
    delete c;
}

gsais_ctx *gsais_default_ctx(void)
{
    static gsais_ctx *g = new gsais_ctx();
    return g;
}

int64_t gsais_run_sa(gsais_ctx *c, const void *T, int symbytes, int64_t n_, int gsa, void *SA, int sa_bytes,
                     void *freq, int freq_bytes)
{
    if (!c) return -2;
    std::lock_guard<std::mutex> lock(c->mu);
    const uint64_t n = (uint64_t)n_;
    if (n > kMaxN) return -2;
    if (!ctx_init(c)) return fail(cudaErrorUnknown);
    DeviceGuard g(c->device);
    cudaStream_t st = c->stream;
    const size_t tb = align_up(n * symbytes);
    const size_t wide = sa_bytes == 8 ? align_up(n * 8) : 0;
    const SortPlan plan = plan_sort(n, symbytes, tb + wide + early_bytes(SA, sa_bytes, n));
    if (!ensure_arena(c, plan.total)) return -2;
    Carver cv(c->arena);
    uint8_t *d_T = cv.take<uint8_t>(n * symbytes);
    int64_t *d_wide = sa_bytes == 8 ? cv.take<int64_t>(n) : nullptr;
    EarlySaCopy ec;
    const bool early = early_setup(c, ec, SA, sa_bytes, n, cv);
    SortWorkspace ws;
    sort_workspace_carve(ws, cv.p, n, symbytes, c->h_small, c->h_hist);
    if (!clear_err(c, st)) return fail(cudaErrorUnknown);
    cudaStream_t cs = c->copy_stream, xs = c->side_stream;
    StreamJoin join{cs}, join_x{xs};   // no write into the caller's buffers outlives the call
    bool hist_ready = false;
    GS_TRY(upload_text(c, d_T, T, symbytes, n, ws, st, xs, &hist_ready));
    const int64_t rc = run_sort(c, d_T, symbytes, n, gsa != 0, ws, st, 0, early ? &ec : nullptr, hist_ready);
    if (rc == -1) {
        // libsais fills freq before rejecting a malformed GSA text (src/libsais.c:6883-6889)
        GS_TRY(symbol_histogram(d_T, symbytes, n, ws.hist, c->h_small + 16, st));
        emit_freq(c->h_small + 16, symbytes, freq, freq_bytes);
        return -1;
    }
    if (rc != 0) return rc;
    if (sa_bytes == 8) {
        GS_TRY(widen_u32_to_i64(ws.sa, d_wide, n, st));
        GS_TRY(cudaMemcpyAsync(SA, d_wide, n * 8, cudaMemcpyDeviceToHost, st));
    } else if (ec.started) {
        GS_TRY(early_sa_patch(ec, ws.sa, n, xs));   // the sort is done: run_sort synchronised st
    } else {
        GS_TRY(cudaMemcpyAsync(SA, ws.sa, n * 4, cudaMemcpyDeviceToHost, st));
    }
    const cudaError_t ce = cudaStreamSynchronize(cs), xe = cudaStreamSynchronize(xs);
    GS_TRY(sync_checked(c, st));
    GS_TRY(ce);
    GS_TRY(xe);
    emit_freq(c->h_small + 16, symbytes, freq, freq_bytes);
    return 0;
}

int64_t gsais_run_sa_int(gsais_ctx *c, const void *T, int tbytes, int64_t n_, int64_t k, void *SA, int sa_bytes)
{
    if (!c || (tbytes != 4 && tbytes != 8)) return -2;
    std::lock_guard<std::mutex> lock(c->mu);
    const uint64_t n = (uint64_t)n_;
    if (n > kMaxN) return -2;
    if (!ctx_init(c)) return fail(cudaErrorUnknown);
    DeviceGuard g(c->device);
    cudaStream_t st = c->stream;
    const size_t extra = align_up(n * tbytes) + align_up(n * 4) + (sa_bytes == 8 ? align_up(n * 8) : 0) + kAlign;
    const SortPlan plan = plan_sort(n, 4, extra);
    if (!ensure_arena(c, plan.total)) return -2;
    Carver cv(c->arena);
    uint8_t *d_T = cv.take<uint8_t>(n * tbytes);
    uint8_t *d_N = cv.take<uint8_t>(n * 4);   // symbols narrowed to 16 or 32 bits
    int64_t *d_wide = sa_bytes == 8 ? cv.take<int64_t>(n) : nullptr;
    unsigned long long *d_scan = cv.take<unsigned long long>(2);
    SortWorkspace ws;
    sort_workspace_carve(ws, cv.p, n, 4, c->h_small, c->h_hist);
    if (!clear_err(c, st)) return fail(cudaErrorUnknown);
    GS_TRY(cudaMemcpyAsync(d_T, T, n * tbytes, cudaMemcpyHostToDevice, st));
    GS_TRY(int_alphabet_scan(d_T, tbytes, n, k, d_scan, st));
    unsigned long long *h_scan = reinterpret_cast<unsigned long long *>(c->h_small + 2);
    GS_TRY(cudaMemcpyAsync(h_scan, d_scan, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    GS_TRY(cudaStreamSynchronize(st));
    if (h_scan[1]) return -1;   // a symbol outside [0, k)
    const unsigned long long mx = h_scan[0];
    if (mx > 0xFFFFFFFFull) return -2;   // symbols wider than 32 bits are not supported
    int64_t rc;
    if (mx < 65536) {
        // small alphabets take the 16-bit path (dense codes, packed text)
        GS_TRY(int_narrow(d_T, tbytes, n, d_N, 2, st));
        rc = run_sort(c, d_N, 2, n, false, ws, st);
    } else {
        const void *src = d_T;   // non-negative int32 symbols are uint32 symbols
        if (tbytes == 8) {
            GS_TRY(int_narrow(d_T, 8, n, d_N, 4, st));
            src = d_N;
        }
        rc = run_sort(c, src, 4, n, false, ws, st, (uint32_t)mx);
    }
    if (rc != 0) return rc;
    if (sa_bytes == 8) {
        GS_TRY(widen_u32_to_i64(ws.sa, d_wide, n, st));
        GS_TRY(cudaMemcpyAsync(SA, d_wide, n * 8, cudaMemcpyDeviceToHost, st));
    } else {
        GS_TRY(cudaMemcpyAsync(SA, ws.sa, n * 4, cudaMemcpyDeviceToHost, st));
    }
    GS_TRY(sync_checked(c, st));
    return 0;
}

int64_t gsais_run_bwt(gsais_ctx *c, const void *T, int symbytes, int64_t n_, void *U, void *freq, int freq_bytes,
                      int64_t r, void *I, int idx_bytes, void *SA, int sa_bytes)
{
    if (!c) return -2;
    std::lock_guard<std::mutex> lock(c->mu);
    const uint64_t n = (uint64_t)n_;
    if (n > kMaxN) return -2;
    if (!ctx_init(c)) return fail(cudaErrorUnknown);
    DeviceGuard g(c->device);
    cudaStream_t st = c->stream;
    const uint64_t icount = r > 0 ? (n - 1) / (uint64_t)r + 1 : 0;
    void *U_pin = pinned_view(U);
    const bool bwt_only_early = !SA && U_pin;
    const size_t extra = align_up(n * symbytes) * 2 + (r > 0 ? align_up(icount * idx_bytes) : 0) +
                         (SA && sa_bytes == 8 ? align_up(n * 8) : 0) + early_bytes(SA, sa_bytes, n) +
                         (bwt_only_early ? align_up((n + 31) / 32 * 4) : 0);
    const SortPlan plan = plan_sort(n, symbytes, extra);
    if (!ensure_arena(c, plan.total)) return -2;
    Carver cv(c->arena);
    uint8_t *d_T = cv.take<uint8_t>(n * symbytes);
    uint8_t *d_U = cv.take<uint8_t>(n * symbytes);
    void *d_I = r > 0 ? (void *)cv.take<uint8_t>(icount * idx_bytes) : nullptr;
    int64_t *d_wide = (SA && sa_bytes == 8) ? cv.take<int64_t>(n) : nullptr;
    EarlySaCopy ec;
    const bool early = bwt_only_early ? early_setup_bwt_only(c, ec, n, cv) : early_setup(c, ec, SA, sa_bytes, n, cv);
    void *U_dev = early ? U_pin : nullptr;   // an early BWT needs U pinned too
    SortWorkspace ws;
    sort_workspace_carve(ws, cv.p, n, symbytes, c->h_small, c->h_hist);
    if (!clear_err(c, st)) return fail(cudaErrorUnknown);
    cudaStream_t cs = c->copy_stream, xs = c->side_stream;
    StreamJoin join{cs}, join_x{xs};   // no write into the caller's buffers outlives the call
    bool hist_ready = false;
    GS_TRY(upload_text(c, d_T, T, symbytes, n, ws, st, xs, &hist_ready));
    // With SA copied early and U pinned, the BWT is also taken early: at that
    // point SA is final except the recorded slots, whose BWT rows are
    // rewritten after the sort.  The gather runs on the side stream beside
    // the rest of the sort; U leaves right behind SA on the copy stream.
    bool early_u = false;
    if (U_dev)
        ec.on_start = [&](cudaStream_t) -> cudaError_t {
            // unresolved slots may hold anything yet: no bounds error for them
            cudaError_t e = cudaStreamWaitEvent(xs, ec.ready, 0);
            if (e == cudaSuccess)
                e = bwt_gather(d_T, symbytes, ws.sa, ws.slot0, n, d_U, packed_of(ws), nullptr, xs);
            if (e == cudaSuccess) e = cudaEventRecord(c->bwt_ev, xs);
            if (e == cudaSuccess) e = cudaStreamWaitEvent(cs, c->bwt_ev, 0);
            if (e == cudaSuccess) e = cudaMemcpyAsync(U, d_U, n * symbytes, cudaMemcpyDeviceToHost, cs);
            early_u = e == cudaSuccess;
            return e;
        };
    const int64_t rc = run_sort(c, d_T, symbytes, n, false, ws, st, 0, early ? &ec : nullptr, hist_ready);
    if (rc != 0) return rc;
    // the sort has completed (run_sort synchronises st): SA leaves on the copy
    // stream (or, copied early, gets its late slots) while the BWT gather,
    // which only reads SA, runs on st
    if (SA) {
        if (sa_bytes == 8) {
            GS_TRY(widen_u32_to_i64(ws.sa, d_wide, n, cs));
            GS_TRY(cudaMemcpyAsync(SA, d_wide, n * 8, cudaMemcpyDeviceToHost, cs));
        } else if (ec.started) {
            GS_TRY(early_sa_patch(ec, ws.sa, n, xs));
        } else {
            GS_TRY(cudaMemcpyAsync(SA, ws.sa, n * 4, cudaMemcpyDeviceToHost, cs));
        }
    }
    if (early_u) {
        // the unresolved rows, written into the host copy behind it on the copy
        // stream (the SA patch runs beside it on the side stream)
        GS_TRY(bwt_patch(d_T, symbytes, ws.sa, ws.rank, n, ec.bits, U_dev, packed_of(ws), c->d_misc, cs));
    } else {
        GS_TRY(bwt_gather(d_T, symbytes, ws.sa, ws.rank, n, d_U, packed_of(ws), c->d_misc, st));
        GS_TRY(cudaMemcpyAsync(U, d_U, n * symbytes, cudaMemcpyDeviceToHost, st));
    }
    if (r > 0) GS_TRY(aux_sample(ws.rank, n, (uint64_t)r, d_I, idx_bytes, st));
    GS_TRY(cudaMemcpyAsync(c->h_small, ws.rank, 4, cudaMemcpyDeviceToHost, st));
    if (r > 0) GS_TRY(cudaMemcpyAsync(I, d_I, icount * idx_bytes, cudaMemcpyDeviceToHost, st));
    const cudaError_t ce = cudaStreamSynchronize(cs), xe = cudaStreamSynchronize(xs);
    GS_TRY(sync_checked(c, st));
    GS_TRY(ce);
    GS_TRY(xe);
    const int64_t prim = (int64_t)c->h_small[0];   // ISA[0] + 1
    emit_freq(c->h_small + 16, symbytes, freq, freq_bytes);
    return r > 0 ? 0 : prim;
}

int64_t gsais_run_unbwt(gsais_ctx *c, const void *T, int symbytes, int64_t n_, int64_t primary, void *U)
{
    if (!c) return -2;
    std::lock_guard<std::mutex> lock(c->mu);
    const uint64_t n = (uint64_t)n_;
    if (n > kMaxN - 1 || primary < 1 || (uint64_t)primary > n) return n > kMaxN - 1 ? -2 : -1;
    if (!ctx_init(c)) return fail(cudaErrorUnknown);
    DeviceGuard g(c->device);
    cudaStream_t st = c->stream;
    const size_t total = 2 * align_up(n * symbytes) + unbwt_workspace_bytes(n);
    if (!ensure_arena(c, total)) return -2;
    Carver cv(c->arena);
    uint8_t *d_in = cv.take<uint8_t>(n * symbytes);
    uint8_t *d_out = cv.take<uint8_t>(n * symbytes);
    if (!clear_err(c, st)) return fail(cudaErrorUnknown);
    GS_TRY(cudaMemcpyAsync(d_in, T, n * symbytes, cudaMemcpyHostToDevice, st));
    GS_TRY(unbwt_run(d_in, symbytes, n, (uint64_t)primary, d_out, cv.p, c->h_hist, &c->prof, c->d_misc, st));
    GS_TRY(cudaMemcpyAsync(U, d_out, n * symbytes, cudaMemcpyDeviceToHost, st));
    GS_TRY(sync_checked(c, st));
    c->prof.flush();
    return 0;
}

int64_t gsais_run_plcp(gsais_ctx *c, const void *T, int symbytes, const void *SA, void *PLCP, int idx_bytes,
                       int64_t n_, int gsa)
{
    if (!c) return -2;
    std::lock_guard<std::mutex> lock(c->mu);
    const uint64_t n = (uint64_t)n_;
    if (n > kMaxN) return -2;
    if (!ctx_init(c)) return fail(cudaErrorUnknown);
    DeviceGuard g(c->device);
    cudaStream_t st = c->stream;
    const size_t total = align_up(n * symbytes) + 2 * align_up(n * 4) + (idx_bytes == 8 ? align_up(n * 8) : 0) +
                         align_up(plcp_sparse_words(n) * 4);
    if (!ensure_arena(c, total)) return -2;
    Carver cv(c->arena);
    uint8_t *d_T = cv.take<uint8_t>(n * symbytes);
    uint32_t *d_SA = cv.take<uint32_t>(n);
    uint32_t *d_P = cv.take<uint32_t>(n);
    int64_t *d_wide = idx_bytes == 8 ? cv.take<int64_t>(n) : nullptr;
    uint32_t *d_sparse = cv.take<uint32_t>(plcp_sparse_words(n));
    if (!clear_err(c, st)) return fail(cudaErrorUnknown);
    GS_TRY(cudaMemcpyAsync(d_T, T, n * symbytes, cudaMemcpyHostToDevice, st));
    if (idx_bytes == 8) {
        GS_TRY(cudaMemcpyAsync(d_wide, SA, n * 8, cudaMemcpyHostToDevice, st));
        GS_TRY(narrow_i64_to_u32(d_wide, d_SA, n, c->d_misc, st));
    } else {
        GS_TRY(cudaMemcpyAsync(d_SA, SA, n * 4, cudaMemcpyHostToDevice, st));
    }
    GS_TRY(plcp_build(d_T, symbytes, d_SA, n, gsa != 0, d_P, d_sparse, c->h_small + 16, c->d_misc, st));
    if (idx_bytes == 8) {
        GS_TRY(widen_u32_to_i64(d_P, d_wide, n, st));
        GS_TRY(cudaMemcpyAsync(PLCP, d_wide, n * 8, cudaMemcpyDeviceToHost, st));
    } else {
        GS_TRY(cudaMemcpyAsync(PLCP, d_P, n * 4, cudaMemcpyDeviceToHost, st));
    }
    GS_TRY(sync_checked(c, st));
    return 0;
}

int64_t gsais_run_lcp(gsais_ctx *c, const void *PLCP, const void *SA, void *LCP, int idx_bytes, int64_t n_)
{
    if (!c) return -2;
    std::lock_guard<std::mutex> lock(c->mu);
    const uint64_t n = (uint64_t)n_;
    if (n > kMaxN) return -2;
    if (!ctx_init(c)) return fail(cudaErrorUnknown);
    DeviceGuard g(c->device);
    cudaStream_t st = c->stream;
    const size_t total = 3 * align_up(n * 4) + (idx_bytes == 8 ? align_up(n * 8) : 0) +
                         align_up(lcp_scratch_words(n) * 4);
    if (!ensure_arena(c, total)) return -2;
    Carver cv(c->arena);
    uint32_t *d_P = cv.take<uint32_t>(n);
    uint32_t *d_SA = cv.take<uint32_t>(n);
    uint32_t *d_L = cv.take<uint32_t>(n);
    int64_t *d_wide = idx_bytes == 8 ? cv.take<int64_t>(n) : nullptr;
    uint32_t *d_scratch = lcp_scratch_words(n) ? cv.take<uint32_t>(lcp_scratch_words(n)) : nullptr;
    if (!clear_err(c, st)) return fail(cudaErrorUnknown);
    if (idx_bytes == 8) {
        GS_TRY(cudaMemcpyAsync(d_wide, PLCP, n * 8, cudaMemcpyHostToDevice, st));
        GS_TRY(narrow_i64_to_u32(d_wide, d_P, n, c->d_misc, st));
        GS_TRY(cudaMemcpyAsync(d_wide, SA, n * 8, cudaMemcpyHostToDevice, st));
        GS_TRY(narrow_i64_to_u32(d_wide, d_SA, n, c->d_misc, st));
    } else {
        GS_TRY(cudaMemcpyAsync(d_P, PLCP, n * 4, cudaMemcpyHostToDevice, st));
        GS_TRY(cudaMemcpyAsync(d_SA, SA, n * 4, cudaMemcpyHostToDevice, st));
    }
    GS_TRY(lcp_gather(d_P, d_SA, d_L, n, d_scratch, c->d_misc, st));
    if (idx_bytes == 8) {
        GS_TRY(widen_u32_to_i64(d_L, d_wide, n, st));
        GS_TRY(cudaMemcpyAsync(LCP, d_wide, n * 8, cudaMemcpyDeviceToHost, st));
    } else {
        GS_TRY(cudaMemcpyAsync(LCP, d_L, n * 4, cudaMemcpyDeviceToHost, st));
    }
    GS_TRY(sync_checked(c, st));
    return 0;
}

// ------------------------------------------------ public extension entry points

int64_t gsais_sa_device(void *ctx, const void *T, int32_t symbytes, int64_t n_, int32_t gsa, void *SA,
                        int32_t sa_bytes, void *stream)
{
    gsais_ctx *c = resolve(ctx);
    if (!c || !T || !SA || n_ < 0 || (symbytes != 1 && symbytes != 2) || (sa_bytes != 4 && sa_bytes != 8)) return -1;
    std::lock_guard<std::mutex> lock(c->mu);
    const uint64_t n = (uint64_t)n_;
    if (n > kMaxN) return -2;
    if (n == 0) return 0;
    if (!ctx_init(c)) return fail(cudaErrorUnknown);
    DeviceGuard g(c->device);
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : c->stream;
    const SortPlan plan = plan_sort(n, symbytes, 0);
    if (!ensure_arena(c, plan.total)) return -2;
    SortWorkspace ws;
    sort_workspace_carve(ws, c->arena, n, symbytes, c->h_small, c->h_hist);
    if (sa_bytes == 4) ws.sa = static_cast<uint32_t *>(SA);
    if (!clear_err(c, st)) return fail(cudaErrorUnknown);
    const int64_t rc = run_sort(c, T, symbytes, n, gsa != 0, ws, st, 0, nullptr, false, false);
    if (rc != 0) return rc;
    if (sa_bytes == 8) GS_TRY(widen_u32_to_i64(ws.sa, static_cast<int64_t *>(SA), n, st));
    GS_TRY(sync_checked(c, st));
    return 0;
}

int64_t gsais_sa_bwt_device(void *ctx, const void *T, int32_t symbytes, int64_t n_, void *SA, int32_t sa_bytes,
                            void *U, void *stream)
{
    gsais_ctx *c = resolve(ctx);
    if (!c || !T || !U || n_ < 0 || (symbytes != 1 && symbytes != 2) || (SA && sa_bytes != 4 && sa_bytes != 8))
        return -1;
    std::lock_guard<std::mutex> lock(c->mu);
    const uint64_t n = (uint64_t)n_;
    if (n > kMaxN) return -2;
    if (n == 0) return 0;
    if (!ctx_init(c)) return fail(cudaErrorUnknown);
    DeviceGuard g(c->device);
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : c->stream;
    const SortPlan plan = plan_sort(n, symbytes, 0);
    if (!ensure_arena(c, plan.total)) return -2;
    SortWorkspace ws;
    sort_workspace_carve(ws, c->arena, n, symbytes, c->h_small, c->h_hist);
    if (SA && sa_bytes == 4) ws.sa = static_cast<uint32_t *>(SA);
    if (!clear_err(c, st)) return fail(cudaErrorUnknown);
    const int64_t rc = run_sort(c, T, symbytes, n, false, ws, st, 0, nullptr, false, false);
    if (rc != 0) return rc;
    cudaEvent_t ev_bwt = c->prof.begin(st);
    GS_TRY(bwt_gather(T, symbytes, ws.sa, ws.rank, n, U, packed_of(ws), c->d_misc, st));
    if (ev_bwt) c->prof.end(KK_BWT, ev_bwt, st, n * (4 + 2 * (uint64_t)symbytes));   // SA read, T gathered, U written
    if (SA && sa_bytes == 8) GS_TRY(widen_u32_to_i64(ws.sa, static_cast<int64_t *>(SA), n, st));
    GS_TRY(cudaMemcpyAsync(c->h_small, ws.rank, 4, cudaMemcpyDeviceToHost, st));
    GS_TRY(sync_checked(c, st));
    c->prof.flush();
    return (int64_t)c->h_small[0];
}

int64_t gsais_plcp_device(void *ctx, const void *T, int32_t symbytes, const void *SA, void *PLCP, int32_t idx_bytes,
                          int64_t n_, int32_t gsa, void *stream)
{
    gsais_ctx *c = resolve(ctx);
    if (!c || !T || !SA || !PLCP || n_ < 0 || (symbytes != 1 && symbytes != 2) || (idx_bytes != 4 && idx_bytes != 8))
        return -1;
    std::lock_guard<std::mutex> lock(c->mu);
    const uint64_t n = (uint64_t)n_;
    if (n > kMaxN) return -2;
    if (n == 0) return 0;
    if (!ctx_init(c)) return fail(cudaErrorUnknown);
    DeviceGuard g(c->device);
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : c->stream;
    const size_t total = (idx_bytes == 8 ? 2 * align_up(n * 4) : 0) + align_up(plcp_sparse_words(n) * 4);
    if (!ensure_arena(c, total)) return -2;
    if (!clear_err(c, st)) return fail(cudaErrorUnknown);
    Carver cv(c->arena);
    const uint32_t *d_SA = static_cast<const uint32_t *>(SA);
    uint32_t *d_P = static_cast<uint32_t *>(PLCP);
    if (idx_bytes == 8) {
        uint32_t *sa32 = cv.take<uint32_t>(n);
        d_P = cv.take<uint32_t>(n);
        GS_TRY(narrow_i64_to_u32(static_cast<const int64_t *>(SA), sa32, n, c->d_misc, st));
        d_SA = sa32;
    }
    uint32_t *d_sparse = cv.take<uint32_t>(plcp_sparse_words(n));
    GS_TRY(plcp_build(T, symbytes, d_SA, n, gsa != 0, d_P, d_sparse, c->h_small + 16, c->d_misc, st));
    if (idx_bytes == 8) GS_TRY(widen_u32_to_i64(d_P, static_cast<int64_t *>(PLCP), n, st));
    GS_TRY(sync_checked(c, st));
    return 0;
}

int64_t gsais_lcp_device(void *ctx, const void *PLCP, const void *SA, void *LCP, int32_t idx_bytes, int64_t n_,
                         void *stream)
{
    gsais_ctx *c = resolve(ctx);
    if (!c || !PLCP || !SA || !LCP || n_ < 0 || (idx_bytes != 4 && idx_bytes != 8)) return -1;
    std::lock_guard<std::mutex> lock(c->mu);
    const uint64_t n = (uint64_t)n_;
    if (n > kMaxN) return -2;
    if (n == 0) return 0;
    if (!ctx_init(c)) return fail(cudaErrorUnknown);
    DeviceGuard g(c->device);
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : c->stream;
    if (!clear_err(c, st)) return fail(cudaErrorUnknown);
    const size_t sw = lcp_scratch_words(n);
    if (idx_bytes == 4) {
        if (sw && !ensure_arena(c, align_up(sw * 4))) return -2;
        uint32_t *scratch = sw ? Carver(c->arena).take<uint32_t>(sw) : nullptr;
        GS_TRY(lcp_gather(static_cast<const uint32_t *>(PLCP), static_cast<const uint32_t *>(SA),
                          static_cast<uint32_t *>(LCP), n, scratch, c->d_misc, st));
    } else {
        if (!ensure_arena(c, 3 * align_up(n * 4) + align_up(sw * 4))) return -2;
        Carver cv(c->arena);
        uint32_t *p = cv.take<uint32_t>(n), *s = cv.take<uint32_t>(n), *l = cv.take<uint32_t>(n);
        uint32_t *scratch = sw ? cv.take<uint32_t>(sw) : nullptr;
        GS_TRY(narrow_i64_to_u32(static_cast<const int64_t *>(PLCP), p, n, c->d_misc, st));
        GS_TRY(narrow_i64_to_u32(static_cast<const int64_t *>(SA), s, n, c->d_misc, st));
        GS_TRY(lcp_gather(p, s, l, n, scratch, c->d_misc, st));
        GS_TRY(widen_u32_to_i64(l, static_cast<int64_t *>(LCP), n, st));
    }
    GS_TRY(sync_checked(c, st));
    return 0;
}

int64_t gsais_sa_bwt(void *ctx, const void *T, int32_t symbytes, int64_t n, void *SA, int32_t sa_bytes, void *U,
                     void *freq, int32_t freq_bytes)
{
    gsais_ctx *c = resolve(ctx);
    if (!c || !T || !SA || !U || n < 0 || (symbytes != 1 && symbytes != 2) || (sa_bytes != 4 && sa_bytes != 8))
        return -1;
    if (n <= 1) {
        if (freq) std::memset(freq, 0, (size_t)(symbytes == 1 ? 256 : 65536) * freq_bytes);
        if (n == 1) {
            if (sa_bytes == 8) static_cast<int64_t *>(SA)[0] = 0;
            else static_cast<int32_t *>(SA)[0] = 0;
            const uint32_t sym = symbytes == 1 ? static_cast<const uint8_t *>(T)[0] : static_cast<const uint16_t *>(T)[0];
            if (symbytes == 1) static_cast<uint8_t *>(U)[0] = (uint8_t)sym;
            else static_cast<uint16_t *>(U)[0] = (uint16_t)sym;
            if (freq) {
                if (freq_bytes == 8) static_cast<int64_t *>(freq)[sym] = 1;
                else static_cast<int32_t *>(freq)[sym] = 1;
            }
        }
        return n;
    }
    return gsais_run_bwt(c, T, symbytes, n, U, freq, freq_bytes, 0, nullptr, 4, SA, sa_bytes);
}

static int64_t batch_run(gsais_ctx *c, const void *d_T, int symbytes, int64_t n_, const uint64_t *d_offs,
                         int32_t count, int32_t *d_SA, void *d_U, int32_t *d_primary, cudaStream_t st,
                         size_t extra_front)
{
    const uint64_t n = (uint64_t)n_;
    SortWorkspace ws;
    Carver cv(static_cast<char *>(c->arena) + extra_front);
    sort_workspace_carve(ws, cv.p, n + (uint64_t)count, symbytes, c->h_small, c->h_hist);
    ws.radix.prof = &c->prof;
    if (!clear_err(c, st)) return fail(cudaErrorUnknown);
    GS_TRY(batch_suffix_sort(d_T, symbytes, n, d_offs, (uint32_t)count, ws, c->d_misc, st, &c->stats,
                             c->opt.tuning_set ? &c->opt.tuning : nullptr));
    GS_TRY(batch_outputs(ws, d_T, symbytes, n, d_offs, (uint32_t)count, d_SA, d_U, d_primary, c->d_misc, st));
    GS_TRY(sync_checked(c, st));
    return 0;
}

int64_t gsais_batch_sa_bwt_sym_device(void *ctx, const void *T, int32_t symbytes, int64_t n, const int64_t *offsets,
                                      int32_t count, int32_t *SA, void *U, int32_t *primary, void *stream)
{
    gsais_ctx *c = resolve(ctx);
    if (!c || !T || !offsets || !SA || !U || !primary || n < 0 || count <= 0 || (symbytes != 1 && symbytes != 2))
        return -1;
    std::lock_guard<std::mutex> lock(c->mu);
    if ((uint64_t)n + (uint64_t)count > kMaxN) return -2;
    if (!ctx_init(c)) return fail(cudaErrorUnknown);
    DeviceGuard g(c->device);
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : c->stream;
    if (!ensure_arena(c, batch_workspace_bytes((uint64_t)n, (uint32_t)count))) return -2;
    return batch_run(c, T, symbytes, n, reinterpret_cast<const uint64_t *>(offsets), count, SA, U, primary, st, 0);
}

int64_t gsais_batch_sa_bwt_device(void *ctx, const void *T, int64_t n, const int64_t *offsets, int32_t count,
                                  int32_t *SA, uint8_t *U, int32_t *primary, void *stream)
{
    return gsais_batch_sa_bwt_sym_device(ctx, T, 1, n, offsets, count, SA, U, primary, stream);
}

int64_t gsais_batch_jobs(gsais_ctx *c, int32_t symbytes, int32_t count, const void *const *T, const int64_t *n,
                         int32_t *const *SA, void *const *U, int64_t *result)
{
    if (!c || !T || !n || !SA || !U || !result || count <= 0 || (symbytes != 1 && symbytes != 2)) return -1;
    uint64_t total = 0;
    for (int32_t k = 0; k < count; ++k) {
        if (!T[k] || !SA[k] || !U[k] || n[k] < 1) return -1;
        total += (uint64_t)n[k];
    }
    std::lock_guard<std::mutex> lock(c->mu);
    if (total + (uint64_t)count > kMaxN) return -2;
    if (!ctx_init(c)) return fail(cudaErrorUnknown);
    DeviceGuard g(c->device);
    cudaStream_t st = c->stream;
    const size_t sb = (size_t)symbytes;
    const size_t front = align_up(total * sb) + align_up((size_t)(count + 1) * 8) + align_up(total * 4) +
                         align_up(total * sb) + align_up((size_t)count * 4);
    if (!ensure_arena(c, front + batch_workspace_bytes(total, (uint32_t)count))) return -2;
    Carver cv(c->arena);
    uint8_t *d_T = cv.take<uint8_t>(total * sb);
    uint64_t *d_offs = cv.take<uint64_t>(count + 1);
    int32_t *d_SA = cv.take<int32_t>(total);
    uint8_t *d_U = cv.take<uint8_t>(total * sb);
    int32_t *d_P = cv.take<int32_t>(count);
    // the offsets stay in host memory of their own (the sort reuses the
    // context's pinned scratch); the primary indexes come back through it
    // once the sort is done (at most 32000 jobs)
    if ((size_t)count > kSmallWords - 16) return -1;
    std::vector<uint64_t> h_offs((size_t)count + 1, 0);
    for (int32_t k = 0; k < count; ++k) h_offs[k + 1] = h_offs[k] + (uint64_t)n[k];
    // one copy per job straight from its buffer (DMA when the buffer is pinned)
    for (int32_t k = 0; k < count; ++k)
        GS_TRY(cudaMemcpyAsync(d_T + h_offs[k] * sb, T[k], (size_t)n[k] * sb, cudaMemcpyHostToDevice, st));
    GS_TRY(cudaMemcpyAsync(d_offs, h_offs.data(), (size_t)(count + 1) * 8, cudaMemcpyHostToDevice, st));
    const int64_t rc = batch_run(c, d_T, symbytes, (int64_t)total, d_offs, count, d_SA, d_U, d_P, st, front);
    if (rc != 0) return rc;
    int32_t *h_prim = reinterpret_cast<int32_t *>(c->h_small + 16);
    for (int32_t k = 0; k < count; ++k) {
        GS_TRY(cudaMemcpyAsync(SA[k], d_SA + h_offs[k], (size_t)n[k] * 4, cudaMemcpyDeviceToHost, st));
        GS_TRY(cudaMemcpyAsync(U[k], d_U + h_offs[k] * sb, (size_t)n[k] * sb, cudaMemcpyDeviceToHost, st));
    }
    GS_TRY(cudaMemcpyAsync(h_prim, d_P, (size_t)count * 4, cudaMemcpyDeviceToHost, st));
    GS_TRY(cudaStreamSynchronize(st));
    for (int32_t k = 0; k < count; ++k) result[k] = h_prim[k];
    return 0;
}

int64_t gsais_ctx_workspace_bytes(gsais_ctx *c)
{
    if (!c) return 0;
    std::lock_guard<std::mutex> lock(c->mu);
    return (int64_t)c->arena_bytes;
}

int64_t gsais_batch_sa_bwt(void *ctx, const void *T, const int64_t *offsets, int32_t count, int32_t *SA, uint8_t *U,
                           int32_t *primary)
{
    gsais_ctx *c = resolve(ctx);
    if (!c || !T || !offsets || !SA || !U || !primary || count <= 0) return -1;
    const int64_t n_ = offsets[count];
    if (n_ < 0 || offsets[0] != 0) return -1;
    for (int32_t s = 0; s < count; ++s)
        if (offsets[s + 1] < offsets[s]) return -1;
    std::lock_guard<std::mutex> lock(c->mu);
    const uint64_t n = (uint64_t)n_;
    if (n + (uint64_t)count > kMaxN) return -2;
    if (!ctx_init(c)) return fail(cudaErrorUnknown);
    DeviceGuard g(c->device);
    cudaStream_t st = c->stream;
    const size_t front = align_up(n) + align_up((count + 1) * 8) + align_up(n * 4) + align_up(n) +
                         align_up((size_t)count * 4);
    if (!ensure_arena(c, front + batch_workspace_bytes(n, (uint32_t)count))) return -2;
    Carver cv(c->arena);
    uint8_t *d_T = cv.take<uint8_t>(n);
    uint64_t *d_offs = cv.take<uint64_t>(count + 1);
    int32_t *d_SA = cv.take<int32_t>(n);
    uint8_t *d_U = cv.take<uint8_t>(n);
    int32_t *d_P = cv.take<int32_t>(count);
    GS_TRY(cudaMemcpyAsync(d_T, T, n, cudaMemcpyHostToDevice, st));
    GS_TRY(cudaMemcpyAsync(d_offs, offsets, (size_t)(count + 1) * 8, cudaMemcpyHostToDevice, st));
    const int64_t rc = batch_run(c, d_T, 1, n_, d_offs, count, d_SA, d_U, d_P, st, front);
    if (rc != 0) return rc;
    GS_TRY(cudaMemcpyAsync(SA, d_SA, n * 4, cudaMemcpyDeviceToHost, st));
    GS_TRY(cudaMemcpyAsync(U, d_U, n, cudaMemcpyDeviceToHost, st));
    GS_TRY(cudaMemcpyAsync(primary, d_P, (size_t)count * 4, cudaMemcpyDeviceToHost, st));
    GS_TRY(cudaStreamSynchronize(st));
    return 0;
}

int32_t gsais_last_stats(void *ctx, gsais_stats *out)
{
    gsais_ctx *c = resolve(ctx);
    if (!c || !out) return -1;
    std::lock_guard<std::mutex> lock(c->mu);
    out->rounds = c->stats.rounds;
    out->seed_symbols = c->stats.seed_symbols;
    out->seed_bits = c->stats.seed_bits;
    out->radix_passes = c->stats.radix_passes;
    out->active_total = (int64_t)c->stats.active_total;
    out->workspace_bytes = (int64_t)c->arena_bytes;
    out->large_total = (int64_t)c->stats.large_total;
    out->pairs_direct = (int64_t)c->stats.pairs_direct;
    out->early_patch = (int64_t)c->stats.early_patch;
    return 0;
}

int32_t gsais_set_seed_key_bits(void *ctx, int32_t bits)
{
    gsais_ctx *c = resolve(ctx);
    if (!c || (bits != 0 && bits != 32 && bits != 64)) return -1;
    std::lock_guard<std::mutex> lock(c->mu);
    const int32_t prev = c->opt.seed_key_bits;
    c->opt.seed_key_bits = bits;
    return prev;
}

int32_t gsais_set_tuning(void *ctx, const gsais_tuning *t)
{
    gsais_ctx *c = resolve(ctx);
    if (!c) return -1;
    std::lock_guard<std::mutex> lock(c->mu);
    if (!t) {
        c->opt.tuning_set = false;
        c->opt.tuning = Tuning();
        return 0;
    }
    Tuning tn;
    tn.digit_bits = t->digit_bits;
    tn.radix_items32 = t->radix_items32;
    tn.radix_items64 = t->radix_items64;
    tn.medium_small = t->medium_small;
    tn.medium_max = t->medium_max;
    tn.large_few_others = t->large_few_others;
    if (!tuning_valid(tn)) return -1;
    c->opt.tuning = tn;
    c->opt.tuning_set = true;
    return 0;
}

int32_t gsais_last_tuning(void *ctx, gsais_tuning *out)
{
    gsais_ctx *c = resolve(ctx);
    if (!c || !out) return -1;
    std::lock_guard<std::mutex> lock(c->mu);
    const Tuning &tn = c->stats.tuning;
    out->digit_bits = tn.digit_bits;
    out->radix_items32 = tn.radix_items32;
    out->radix_items64 = tn.radix_items64;
    out->medium_small = tn.medium_small;
    out->medium_max = tn.medium_max;
    out->large_few_others = tn.large_few_others;
    return 0;
}

int32_t gsais_load_tuning_cache(const char *path) { return tuning_load_cache(path); }

int32_t gsais_profile_enable(void *ctx, int32_t on)
{
    gsais_ctx *c = resolve(ctx);
    if (!c) return -1;
    std::lock_guard<std::mutex> lock(c->mu);
    const int32_t prev = c->prof.enabled ? 1 : 0;
    c->prof.enabled = on != 0;
    return prev;
}

int32_t gsais_profile_read(void *ctx, gsais_kernel_profile *out, int32_t max_kinds)
{
    gsais_ctx *c = resolve(ctx);
    if (!c || !out) return -1;
    std::lock_guard<std::mutex> lock(c->mu);
    static const char *names[KK_COUNT] = {"radix_pass",   "tile_counts", "upsweep",      "seed",
                                          "round_keys",   "tile_summary", "assign",      "small_groups",
                                          "pair_compare", "unbwt",        "histogram",   "rank_scatter",
                                          "classify",     "medium_groups", "bwt",         "large_few"};
    int k = 0;
    for (; k < KK_COUNT && k < max_kinds; ++k) {
        out[k].name = names[k];
        out[k].launches = (int64_t)c->prof.launches[k];
        out[k].total_ms = c->prof.ms[k];
        out[k].bytes = (int64_t)c->prof.bytes[k];
    }
    return k;
}

void gsais_profile_reset(void *ctx)
{
    gsais_ctx *c = resolve(ctx);
    if (!c) return;
    std::lock_guard<std::mutex> lock(c->mu);
    c->prof.reset();
}

int64_t gsais_launch_count(void) { return (int64_t)g_launches.load(); }

int32_t gsais_test_stall_radix_wait(int64_t limit_ns)
{
    if (limit_ns < 0 || limit_ns > 1000000000ll) return -1;
    if (set_test_stall_wait((uint64_t)limit_ns) != cudaSuccess) {
        cudaGetLastError();
        return -2;
    }
    return 0;
}

int32_t gsais_test_fail_allocations(int32_t count)
{
    if (count < 0) return -1;
    g_fail_allocs.store(count);
    return 0;
}

void gsais_release_workspace(void *ctx)
{
    gsais_ctx *c = resolve(ctx);
    if (!c) return;
    std::lock_guard<std::mutex> lock(c->mu);
    if (c->ready && c->arena) {
        DeviceGuard g(c->device);
        cudaStreamSynchronize(c->stream);
        cudaFree(c->arena);
        c->arena = nullptr;
        c->arena_bytes = 0;
    }
}

}  // extern "C"
