// tuning.h -- tuning parameters of one suffix sort (internal).
#pragma once
#include <cstdint>

namespace gsais {

struct Tuning {
    int digit_bits = 8;        // radix digit width (the compiled passes rank 8-bit digits)
    int radix_items32 = 20;    // keys per thread of a digit pass over 32-bit keys: 16, 20, 24, 28
    int radix_items64 = 16;    // the same for 64-bit keys: 12, 16, 20
    int medium_small = 512;    // groups of 33..medium_small members: 128-thread CTA sort
    int medium_max = 4096;     // groups up to medium_max: 256-thread CTA sort; larger: global radix sort
    int large_few_others = 1;  // large groups whose members mostly share rank[i+h]: sort only the others
};

bool tuning_valid(const Tuning &t);

// The tuning for a sort of n symbols whose alphabet codes take `bits` bits on
// the current device: the autotuner cache entry with the nearest n bucket
// (loaded from $GSAIS_TUNING_CACHE on first use, or by tuning_load_cache),
// else the defaults.
Tuning tuning_lookup(uint64_t n, int bits);

// Replaces the cache with the entries of a JSON file (path, or
// $GSAIS_TUNING_CACHE when null).  Returns the number of entries, -1 on error.
int tuning_load_cache(const char *path);

}  // namespace gsais
