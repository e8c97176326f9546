/*--

libsais_gb300 -- GB300 (sm_103a) suffix-array construction behind the libsais
API.  This header declares the entry points that have NO counterpart in the
reference libsais 2.10.4: device-resident variants for callers whose text
already lives in GPU memory, a combined SA + BWT call, and run statistics.
The reference-compatible entry points are declared in libsais.h,
libsais64.h and libsais16.h.

Conventions shared with libsais: return 0 (or the BWT primary index) on
success, -1 for invalid arguments, -2 for allocation or device failures.

--*/

#ifndef LIBSAIS_GB300_H
#define LIBSAIS_GB300_H 1

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

    /**
    * Suffix array of a text that already resides in device memory.
    * @param ctx A context from libsais_create_ctx (or NULL for the process-wide one).
    * @param T [0..n-1] Device pointer to the text (1- or 2-byte symbols).
    * @param symbytes 1 for uint8_t text, 2 for uint16_t text.
    * @param n The text length (must be < 2^32).
    * @param gsa Non-zero to build the generalized suffix array (0 separators, T[n-1] == 0).
    * @param SA [0..n-1] Device pointer receiving the suffix array (int32 or int64).
    * @param sa_bytes 4 for int32 SA, 8 for int64 SA.
    * @param stream cudaStream_t to run on (NULL: the context's stream).
    * @return 0 on success, -1 or -2 otherwise.
    */
    int64_t gsais_sa_device(void * ctx, const void * T, int32_t symbytes, int64_t n, int32_t gsa, void * SA, int32_t sa_bytes, void * stream);

    /**
    * Suffix array and BWT (libsais_bwt layout) of a device-resident text in one sort.
    * @param SA [0..n-1] Device pointer receiving the suffix array (may be NULL).
    * @param U [0..n-1] Device pointer receiving the BWT (must not alias T).
    * @return The primary index (as libsais_bwt returns it), or -1 / -2.
    */
    int64_t gsais_sa_bwt_device(void * ctx, const void * T, int32_t symbytes, int64_t n, void * SA, int32_t sa_bytes, void * U, void * stream);

    /**
    * PLCP of a device-resident text and suffix array.
    * @param idx_bytes Width of SA and PLCP entries (4 or 8).
    * @return 0 on success, -1 or -2 otherwise.
    */
    int64_t gsais_plcp_device(void * ctx, const void * T, int32_t symbytes, const void * SA, void * PLCP, int32_t idx_bytes, int64_t n, int32_t gsa, void * stream);

    /**
    * LCP[i] = PLCP[SA[i]] on device-resident arrays (idx_bytes 4 or 8; LCP must not alias PLCP).
    */
    int64_t gsais_lcp_device(void * ctx, const void * PLCP, const void * SA, void * LCP, int32_t idx_bytes, int64_t n, void * stream);

    /**
    * Suffix array and BWT of a host text with one sort (one H2D of T, D2H of SA and U).
    * @param SA [0..n-1] Output suffix array (int32 or int64 per sa_bytes).
    * @param U [0..n-1] Output BWT in libsais_bwt's layout (may be T).
    * @param freq Optional symbol frequencies (256 or 65536 entries, freq_bytes wide).
    * @return The primary index, or -1 / -2.
    */
    int64_t gsais_sa_bwt(void * ctx, const void * T, int32_t symbytes, int64_t n, void * SA, int32_t sa_bytes, void * U, void * freq, int32_t freq_bytes);

    /**
    * Suffix arrays and BWTs of many independent uint8 strings in one batched sort
    * (every doubling round is one set of launches for all strings; the string id
    * is packed into the high bits of the seed keys).  String s is
    * T[offsets[s] .. offsets[s+1]-1]; offsets has count + 1 entries, offsets[0] = 0.
    * Outputs use the same concatenated layout: SA[offsets[s] + k] is the k-th suffix
    * of string s (relative to its start), U[offsets[s] ..] its BWT in libsais_bwt's
    * layout, primary[s] its primary index (as libsais_bwt returns it; 0 for empty strings).
    * Host buffers.  Returns 0, -1 or -2.
    */
    int64_t gsais_batch_sa_bwt(void * ctx, const void * T, const int64_t * offsets, int32_t count, int32_t * SA, uint8_t * U, int32_t * primary);

    /** gsais_batch_sa_bwt on device buffers (n = offsets[count], given by the caller). */
    int64_t gsais_batch_sa_bwt_device(void * ctx, const void * T, int64_t n, const int64_t * offsets, int32_t count, int32_t * SA, uint8_t * U, int32_t * primary, void * stream);

    /**
    * gsais_batch_sa_bwt_device for strings of 8- or 16-bit symbols (symbytes 1 or 2; U has
    * the same symbol width as T).  Each string's SA and BWT equal libsais/libsais16 and
    * libsais_bwt/libsais16_bwt on it alone (src/libsais16.c:6995, :7074).
    */
    int64_t gsais_batch_sa_bwt_sym_device(void * ctx, const void * T, int32_t symbytes, int64_t n, const int64_t * offsets, int32_t count, int32_t * SA, void * U, int32_t * primary, void * stream);

    /**
    * SA+BWT request loop with continuous batching.  `workers` host threads each own a
    * CUDA stream and device workspace, so jobs taken by different workers overlap on
    * the GPU; a free worker takes the oldest queued job and, if it is a small 8-bit job
    * (n <= small_job_symbols), coalesces the small 8-bit jobs queued behind it (up to
    * max_batch) into one batched sort.  Each worker may hold budget/workers bytes of
    * device memory; a job needs about footprint_bytes_per_symbol * n bytes, and jobs
    * that do not fit a worker's share complete with -2.
    * @return an opaque server handle, or NULL.
    */
    void * gsais_server_create(int64_t hbm_budget_bytes, int32_t workers, int64_t small_job_symbols, int32_t max_batch);

    /**
    * Queues SA+BWT of T[0..n-1] (host memory, symbytes 1 or 2, n >= 2); SA (int32) and
    * U receive the outputs.  The buffers must stay valid until the job is waited for.
    * @return the job id (> 0), or -1 / -2.
    */
    int64_t gsais_server_submit(void * server, const void * T, int32_t symbytes, int64_t n, int32_t * SA, void * U);

    /**
    * Blocks until job `id` completes; stores its result (the BWT primary index, or -1 /
    * -2), the seconds it waited in the queue, its total latency and the number of jobs in
    * the batch it ran in.  Returns 0, or -1 for an unknown id.
    */
    int32_t gsais_server_wait(void * server, int64_t id, int64_t * result, double * queued_s, double * total_s, int32_t * batched);

    typedef struct gsais_server_stats
    {
        int64_t submitted, completed, rejected;
        int64_t batches;              /* coalesced launches of more than one job */
        int64_t batched_jobs;         /* jobs that ran in such batches */
        int64_t symbols_done;
        int64_t hbm_high_water_bytes; /* peak admitted footprint */
        int64_t hbm_budget_bytes;
        double busy_seconds;          /* first submit to last completion */
        double footprint_bytes_per_symbol;
    } gsais_server_stats;

    int32_t gsais_server_get_stats(void * server, gsais_server_stats * out);

    /** Drains the queue, stops the workers and frees their contexts. */
    void gsais_server_destroy(void * server);

    /** Statistics of the last suffix sort run on a context. */
    typedef struct gsais_stats
    {
        int32_t rounds;          /* prefix-doubling rounds after the seed sort */
        int32_t seed_symbols;    /* symbols packed into each seed key */
        int32_t seed_bits;       /* bits per dense symbol code */
        int32_t radix_passes;    /* digit passes actually run (all sorts) */
        int64_t active_total;    /* sum over rounds of still-unsorted suffixes */
        int64_t workspace_bytes; /* device workspace held by the context */
        int64_t large_total;     /* sum over rounds of suffixes sorted by the global radix path */
        int64_t pairs_direct;    /* tied suffix pairs ordered by direct comparison of their text */
        int64_t early_patch;     /* SA slots patched after SA left early for a pinned host buffer (0: no early copy) */
    } gsais_stats;

    int32_t gsais_last_stats(void * ctx, gsais_stats * out);

    /** Seed key width in bits used by later sorts on ctx: 32, 64, or 0 (the default: 64 when the
     *  text's codes take 3 or 4 bits, else 32); returns the previous setting, -1 for other values. */
    int32_t gsais_set_seed_key_bits(void * ctx, int32_t bits);

    /**
    * Tuning parameters of the suffix sort (no counterpart in the reference, which
    * has no tunables on this path).  digit_bits: radix digit width (8);
    * radix_items32 / radix_items64: keys per thread of a radix digit pass over 32-bit
    * (16, 20, 24, 28) and 64-bit (12, 16, 20) keys, the tile being 256 threads times
    * that; medium_small (64..512) and medium_max (medium_small..4096): unsorted groups
    * of up to medium_small members are split by a 128-thread CTA, up to medium_max by
    * a 256-thread CTA, larger ones by the global segmented radix sort;
    * large_few_others (0 or 1): a large group whose members mostly carry the same
    * rank of their suffix h on (runs, tandem repeats) sorts only the other members and
    * places the rest as one run.
    */
    typedef struct gsais_tuning
    {
        int32_t digit_bits;
        int32_t radix_items32;
        int32_t radix_items64;
        int32_t medium_small;
        int32_t medium_max;
        int32_t large_few_others;
    } gsais_tuning;

    /**
    * Fixes the tuning of later sorts on ctx (NULL: the process-wide context).  t == NULL
    * goes back to the autotuner cache (its entry for the GPU, the alphabet's code bits
    * and the nearest n bucket) or the built-in defaults.
    * @return 0, or -1 for values outside the ranges above.
    */
    int32_t gsais_set_tuning(void * ctx, const gsais_tuning * t);

    /** The tuning the last sort on ctx ran with. */
    int32_t gsais_last_tuning(void * ctx, gsais_tuning * out);

    /**
    * Loads the autotuner cache (the JSON file libsais_gb300.autotune writes; path NULL:
    * $GSAIS_TUNING_CACHE, which is also read on first use).  Sorts without a tuning of
    * their own take its entry for their GPU, code bits and nearest n bucket.
    * @return the number of entries loaded, or -1 if the file is missing or malformed.
    */
    int32_t gsais_load_tuning_cache(const char * path);

    /** Per-kernel timing record (CUDA events on the launching stream). */
    typedef struct gsais_kernel_profile
    {
        const char * name;       /* kernel family */
        int64_t launches;        /* timed launches */
        double total_ms;         /* summed device time */
        int64_t bytes;           /* summed algorithmic bytes (reads + writes) */
    } gsais_kernel_profile;

    /** Turns per-kernel timing on ctx on or off; returns the previous state. */
    int32_t gsais_profile_enable(void * ctx, int32_t on);

    /** Copies up to max_kinds records; returns how many were written. */
    int32_t gsais_profile_read(void * ctx, gsais_kernel_profile * out, int32_t max_kinds);

    /** Clears the accumulated timing records of ctx. */
    void gsais_profile_reset(void * ctx);

    /** Kernels launched by this library since the process started (all contexts). */
    int64_t gsais_launch_count(void);

    /** Releases the device workspace cached by ctx (NULL: the process-wide context). */
    void gsais_release_workspace(void * ctx);

    /**
    * Test hook for the bounded device waits (no counterpart in the reference).  With
    * limit_ns > 0, every full tile of the radix digit pass, after its staging copies
    * have landed, also waits on a barrier that nothing arrives on and gives up after
    * limit_ns nanoseconds: the wait's error bit is raised, the tile is staged again
    * with plain loads, and the sort returns -2 (src/libsais.c:6930-6932 uses -2 for
    * internal failures).  0 switches it off.  Applies to the current device.
    * @return 0, -1 for a limit outside [0, 1e9], -2 on a CUDA failure.
    */
    int32_t gsais_test_stall_radix_wait(int64_t limit_ns);

    /**
    * Test hook (no counterpart in the reference): the next `count` device workspace
    * allocations of any context fail as if the device were out of memory, so the
    * calls that need them return -2 as the reference does on a failed allocation
    * (src/libsais.c:6930-6932).  0 switches it off.
    * @return 0, or -1 for a negative count.
    */
    int32_t gsais_test_fail_allocations(int32_t count);

    /**
    * Suffix array of a device-resident text, allocating nothing.  No counterpart in
    * the reference libsais.  It serves callers that cannot call cudaMalloc: a plugin
    * running inside an application whose caching allocator owns the device's memory
    * (cudaMalloc there can fail on memory the allocator holds, and can synchronise
    * the device under the host's other streams), and latency-critical paths.  All
    * scratch comes from one fixed 6 MiB __device__ array that every GPU loading this
    * library reserves until the library is unloaded.  Calls share the array, which
    * keeps the previous call's contents (the sort clears what must start at zero),
    * and calls whose work overlaps on one GPU race on it; a host mutex admits one call
    * at a time and the call returns only after its work on `stream` has finished
    * (error returns drain `stream` first).  The first call on each device looks up
    * the array's device address (cudaGetSymbolAddress, that device current).
    * @param T [0..n-1] Device pointer to the text (symbytes 1 or 2).
    * @param n The text length, at most 65536 symbols (longer texts return -1).
    * @param gsa Non-zero for the generalized suffix array (0 separators, T[n-1] == 0).
    * @param SA [0..n-1] Device pointer receiving the int32 suffix array.
    * @param stream cudaStream_t to run on (NULL: the legacy default stream).
    * @return 0 on success, -1 for invalid arguments or n > 65536, -2 on device failure.
    */
    int64_t gsais_sa_device_noalloc(const void * T, int32_t symbytes, int64_t n, int32_t gsa, void * SA, void * stream);

#ifdef __cplusplus
}
#endif

#endif
