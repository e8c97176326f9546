// device_util.cuh -- small sm_103a helpers shared by the kernels: scoped
// relaxed loads/stores, mbarrier + TMA bulk copies,
// warp/block scans, and the bounded-spin error word.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#define GSAIS_WARP 32
#define GSAIS_FULL_MASK 0xffffffffu

// Device error bits written to the context's error word.
enum : uint32_t {
    GSAIS_ERR_LOOKBACK_SPIN = 1u << 0,   // a decoupled look-back wait ran past its limit
    GSAIS_ERR_MBARRIER_SPIN = 1u << 1,   // a TMA mbarrier wait ran past its limit
    GSAIS_ERR_ROUNDS        = 1u << 2,   // prefix doubling did not converge
    GSAIS_ERR_BOUNDS        = 1u << 3,   // an index check failed (debug guard)
};

// Upper bound on polling iterations of any spin-wait, and on its duration:
// a wait gives up after GSAIS_SPIN_LIMIT polls or GSAIS_SPIN_NS nanoseconds
// of %globaltimer, whichever comes first.
#define GSAIS_SPIN_LIMIT (1u << 24)
#define GSAIS_SPIN_NS (2000000000ull)

__device__ __forceinline__ uint64_t global_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ uint64_t ld_relaxed_gpu(const uint64_t *p)
{
    uint64_t v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_relaxed_gpu(uint64_t *p, uint64_t v)
{
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__device__ __forceinline__ uint32_t smem_addr(const void *p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

// One-dimensional TMA bulk copy global -> shared, completion counted on bar.
// dst, src 16-byte aligned; bytes a multiple of 16.
__device__ __forceinline__ void bulk_copy_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait on an mbarrier phase.  Returns false (and raises the error
// bit) if the phase did not complete within limit_ns nanoseconds (or
// GSAIS_SPIN_LIMIT polls).
__device__ __forceinline__ bool mbar_wait_bounded_ns(uint64_t *bar, uint32_t parity, uint32_t *err,
                                                     uint64_t limit_ns)
{
    const uint64_t t0 = global_ns();
    for (uint32_t it = 0; it < GSAIS_SPIN_LIMIT; ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((it & 255) == 255 && global_ns() - t0 > limit_ns) break;
    }
    atomicOr(err, GSAIS_ERR_MBARRIER_SPIN);
    return false;
}

__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, uint32_t *err)
{
    return mbar_wait_bounded_ns(bar, parity, err, GSAIS_SPIN_NS);
}

__device__ __forceinline__ uint32_t lanemask_lt()
{
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

template <typename T>
__device__ __forceinline__ T warp_inclusive_sum(T v)
{
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T u = __shfl_up_sync(GSAIS_FULL_MASK, v, o);
        if (lane >= o) v += u;
    }
    return v;
}

template <typename T>
__device__ __forceinline__ T warp_inclusive_max(T v)
{
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T u = __shfl_up_sync(GSAIS_FULL_MASK, v, o);
        if (lane >= o) v = v > u ? v : u;
    }
    return v;
}

// "Last non-zero" scans: the operator keeps the right operand when it is
// non-zero, else the left one (associative).  Used to carry the value of the
// most recent group head along a list whose groups are in any order.
__device__ __forceinline__ uint32_t lastnz(uint32_t a, uint32_t b) { return b ? b : a; }

__device__ __forceinline__ uint32_t warp_inclusive_lastnz(uint32_t v)
{
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t u = __shfl_up_sync(GSAIS_FULL_MASK, v, o);
        if (lane >= o) v = lastnz(u, v);
    }
    return v;
}

// Exclusive block-wide lastnz scan (identity 0); `warp_buf` >= blockDim.x/32.
template <int THREADS>
__device__ __forceinline__ uint32_t block_exclusive_lastnz(uint32_t v, uint32_t *warp_buf, uint32_t &total)
{
    constexpr int WARPS = THREADS / 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t inc = warp_inclusive_lastnz(v);
    uint32_t exc = __shfl_up_sync(GSAIS_FULL_MASK, inc, 1);
    if (lane == 0) exc = 0;
    if (lane == 31) warp_buf[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        const uint32_t w = lane < WARPS ? warp_buf[lane] : 0u;
        const uint32_t wi = warp_inclusive_lastnz(w);
        uint32_t we = __shfl_up_sync(GSAIS_FULL_MASK, wi, 1);
        if (lane == 0) we = 0;
        if (lane < WARPS) warp_buf[lane] = we;
        if (lane == WARPS - 1) warp_buf[WARPS] = wi;
    }
    __syncthreads();
    const uint32_t r = lastnz(warp_buf[warp], exc);
    total = warp_buf[WARPS];
    __syncthreads();
    return r;
}

// Exclusive block-wide sum; `warp_buf` holds at least blockDim.x/32 entries.
// Returns the exclusive prefix for the calling thread and the block total.
template <typename T, int THREADS>
__device__ __forceinline__ T block_exclusive_sum(T v, T *warp_buf, T &total)
{
    constexpr int WARPS = THREADS / 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    T inc = warp_inclusive_sum(v);
    if (lane == 31) warp_buf[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        T w = lane < WARPS ? warp_buf[lane] : T(0);
        T wi = warp_inclusive_sum(w);
        if (lane < WARPS) warp_buf[lane] = wi - w;
        if (lane == WARPS - 1) warp_buf[WARPS] = wi;
    }
    __syncthreads();
    T r = warp_buf[warp] + inc - v;
    total = warp_buf[WARPS];
    __syncthreads();
    return r;
}

// Exclusive block-wide max (identity 0).
template <typename T, int THREADS>
__device__ __forceinline__ T block_exclusive_max(T v, T *warp_buf)
{
    constexpr int WARPS = THREADS / 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    T inc = warp_inclusive_max(v);
    T exc = __shfl_up_sync(GSAIS_FULL_MASK, inc, 1);
    if (lane == 0) exc = T(0);
    if (lane == 31) warp_buf[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        T w = lane < WARPS ? warp_buf[lane] : T(0);
        T wi = warp_inclusive_max(w);
        T we = __shfl_up_sync(GSAIS_FULL_MASK, wi, 1);
        if (lane == 0) we = T(0);
        if (lane < WARPS) warp_buf[lane] = we;
    }
    __syncthreads();
    T p = warp_buf[warp];
    T r = p > exc ? p : exc;
    __syncthreads();
    return r;
}

static inline int gsais_bits_for(uint64_t x)
{
    int b = 0;
    while (x) { ++b; x >>= 1; }
    return b;
}
