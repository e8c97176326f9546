// suffix_sort.cuh -- prefix-doubling suffix sorter (device side, internal).
#pragma once
#include <functional>
#include <cstdint>
#include <cuda_runtime.h>

#include "engine.h"

namespace gsais {

// Device buffers used by one suffix sort of a text of n symbols.
struct SortWorkspace {
    uint32_t *rank = nullptr;      // n + 1: 1 + SA position of the suffix's group start; rank[n] = 0
    uint32_t *sa = nullptr;        // n: the suffix array (output)
    uint64_t *keys[2] = {nullptr, nullptr};
    uint32_t *vals[2] = {nullptr, nullptr};
    uint32_t *pos[2] = {nullptr, nullptr};   // SA slot of each active entry
    uint32_t *gid[2] = {nullptr, nullptr};   // dense id of each active entry's group
    uint32_t *gstart[2] = {nullptr, nullptr};  // list index of each group's first entry
    uint32_t *lid = nullptr;                 // per group: id among the large groups, or none
    uint32_t *loff = nullptr;                // per group: first slot in the large list
    uint32_t *lvals[2] = {nullptr, nullptr};   // large list: suffix indexes (sort ping-pong)
    uint32_t *lpos = nullptr;                // large list: SA slot of each entry
    uint32_t *heads = nullptr;               // head bit of every entry of an assign (summary -> assign)
    unsigned long long *counters = nullptr;  // 8 round counters: output reservation (groups<<32 | entries),
                                             // large list, medium groups, tied pairs, pair cursor
    uint32_t *slot0 = nullptr;               // (in counters[7]) 1 + SA slot of suffix 0 after the seed round
    uint32_t *tile_info = nullptr;           // 3 words per assign tile
    uint32_t *tile_carry = nullptr;          // 3 words per assign tile
    uint32_t *tile_agg = nullptr;            // tile-scan aggregates of kScanSpan tiles, then their prefixes
    uint32_t *totals = nullptr;              // [4] kept entries, kept groups, ...
    uint32_t *hist = nullptr;                // symbol histogram (256 or 65536)
    uint16_t *codes = nullptr;               // dense symbol codes (256 or 65536)
    uint8_t *packed = nullptr;               // text as packed codes when they fit 2 or 4 bits
    int pack_bits = 0;                       // 0 (not packed), 2 or 4
    uint16_t decode[16] = {0};               // symbol of each code when packed
    uint32_t *few = nullptr;                 // scratch of the large groups with few differing members
    uint32_t *sg_tiles = nullptr;            // flags + list of a round's small-group tiles
    uint64_t n_cap = 0;                      // symbols the workspace was carved for
    RadixScratch radix;
    uint32_t *h_small = nullptr;             // pinned host scratch (kHostSmallWords words)
};

// Bytes of device memory SortWorkspace needs for n symbols of `symbytes`
// bytes (the text itself is not included).
size_t sort_workspace_bytes(uint64_t n, int symbytes);

// Carves a SortWorkspace out of `base` (which holds sort_workspace_bytes).
void sort_workspace_carve(SortWorkspace &ws, void *base, uint64_t n, int symbytes, uint32_t *h_small,
                          uint32_t *h_hist);

// Host scratch of a sort: 16 words of counters, a 65536-word symbol
// histogram, 65536 16-bit codes, and kHostEdgeWords words for the symbols at
// both ends of the text.
constexpr size_t kHostEdgeWords = 256;
constexpr size_t kHostSmallWords = 16 + 65536 + 32768 + kHostEdgeWords;

// Early device-to-host copy of an int32 suffix array into pinned host
// memory.  When the seed round (with its tied pairs) leaves at most
// patch_cap unresolved entries, the sort starts copying SA to `host` on
// `stream` before the doubling rounds and sets the bits of those entries'
// SA slots in `bits`; the rounds write only those slots, so once the sort is
// done early_sa_patch() writes their final values through `host_dev` (the
// device's address of the same buffer) and the copy of the whole array
// overlaps the rounds.  The patches go in address order, a warp per 32
// slots, so the unresolved slots' runs (their groups, adjacent groups
// merged) leave as coalesced writes: the host link takes scattered 4-byte
// writes at only a few billion a second.
struct EarlySaCopy {
    int32_t *host = nullptr;       // destination (the caller's pinned buffer); null: no SA copy,
                                   // only the slot bits and on_start (a BWT-only call)
    int32_t *host_dev = nullptr;   // the same buffer as the device addresses it
    cudaStream_t stream = nullptr;
    cudaEvent_t ready = nullptr;   // recorded on the sort's stream when the copy may start
    cudaEvent_t copied = nullptr;  // recorded on `stream` behind the bulk copy
    uint32_t *bits = nullptr;      // device: (n + 31) / 32 words, one bit per SA slot
    uint64_t patch_cap = 0;
    uint64_t patch_n = 0;          // out: slots recorded
    bool started = false;          // out: the bulk copy is queued on `stream`
    // Called once the bulk copy is queued (SA final except the recorded
    // slots; ws.slot0 holds 1 + the slot of suffix 0, provisional when that
    // slot is recorded); may queue more work on the sort's stream and on
    // `stream` (an early BWT and its copy).
    std::function<cudaError_t(cudaStream_t sort_stream)> on_start;
};

struct SortOptions {
    Tuning tuning;            // used when tuning_set; otherwise tuning_lookup(n, code bits)
    bool tuning_set = false;
    int seed_key_bits = 0;    // width of the packed seed prefix: 32, 64, or 0 (64 when the codes
                              // take 3 or 4 bits, whose 32-bit keys hold only 10 or 8 symbols)
    uint32_t raw_max = 0;     // 32-bit integer symbols: the largest symbol value
    EarlySaCopy *early = nullptr;
    bool hist_ready = false;  // ws.hist already holds the symbol histogram (symbol_histogram_part)
    bool presence_only = false;   // no caller wants the counts (freq): 8-bit texts take a presence map
};

// Queues on `st`, behind the bulk copy (ec.copied), the writes of the
// recorded slots' final values from d_sa into the host buffer.
cudaError_t early_sa_patch(const EarlySaCopy &ec, const uint32_t *d_sa, uint64_t n, cudaStream_t st);

// Suffix array of the device text d_T (n symbols of `symbytes` bytes).  gsa
// sorts as a generalized suffix array with 0 separators (the caller has
// validated the text).  On return ws.sa holds SA, ws.rank holds ISA + 1,
// ws.hist the symbol histogram and ws.h_small[16..] a host copy of it.  Returns a CUDA error (or cudaErrorUnknown
// when the device error word was raised).
cudaError_t suffix_sort(const void *d_T, int symbytes, uint64_t n, bool gsa, SortWorkspace &ws,
                        const SortOptions &opt, uint32_t *d_err, cudaStream_t st, SortStats *stats);

// Batched suffix arrays of `count` independent strings of 8- or 16-bit
// symbols (symbytes 1 or 2) concatenated in d_T (string s = [offs[s],
// offs[s+1]), offs on the device, offs[count] = n), all sorted in the same
// launches.  Workspace: batch_workspace_bytes.
// On return ws.sa holds the rows (rank coordinates) grouped by string.
size_t batch_workspace_bytes(uint64_t n, uint32_t count);
cudaError_t batch_suffix_sort(const void *d_T, int symbytes, uint64_t n, const uint64_t *d_offs, uint32_t count,
                              SortWorkspace &ws, uint32_t *d_err, cudaStream_t st, SortStats *stats,
                              const Tuning *tuning = nullptr);
// Per-string SA (relative to each string), BWT (libsais_bwt layout) and
// primary indexes from a finished batch_suffix_sort.
cudaError_t batch_outputs(const SortWorkspace &ws, const void *d_T, int symbytes, uint64_t n, const uint64_t *d_offs,
                          uint32_t count, int32_t *d_sa, void *d_U, int32_t *d_primary, uint32_t *d_err,
                          cudaStream_t st);

// Symbol histogram of a device text into d_hist and the pinned h_hist
// (256 or 65536 counts); synchronises the stream.
// Adds the symbols of a stretch of the text to d_hist (no zeroing, no
// read-back): lets the histogram follow the text's upload chunk by chunk.
cudaError_t symbol_histogram_part(const void *d_part, int symbytes, uint64_t len, uint32_t *d_hist, cudaStream_t st);
cudaError_t symbol_histogram(const void *d_T, int symbytes, uint64_t n, uint32_t *d_hist, uint32_t *h_hist,
                             cudaStream_t st);

// Phi[SA[j]] = SA[j-1], Phi[SA[0]] = N, for a suffix array of N entries
// (a permutation of [0, N)), through position partitions when
// phi_partitioned(N) (scratch: phi_scratch_words(N) words); the caller uses
// a direct scatter otherwise.
bool phi_partitioned(uint64_t N);
size_t phi_scratch_words(uint64_t N);
cudaError_t phi_permute(const uint32_t *SA, uint64_t N, uint32_t *phi, uint32_t *scratch, uint32_t *d_err,
                        cudaStream_t st);

// GSA validity of a device text: T[0] != 0, no two adjacent zeros,
// T[n-1] == 0.  Result through a pinned host word.
cudaError_t gsa_validate(const void *d_T, int symbytes, uint64_t n, uint32_t *d_flag, uint32_t *h_flag,
                         cudaStream_t st, bool *valid);

}  // namespace gsais
