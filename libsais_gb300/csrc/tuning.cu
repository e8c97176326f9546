// tuning.cu -- the tuning parameters of the suffix sort and the cache the
// autotuner (libsais_gb300/autotune.py) writes.
//
// A tuning names, for one sort, the radix digit width, the keys per thread of
// a digit pass for 32- and 64-bit keys (the tile is 256 threads x that many
// keys), the group sizes at which the doubling rounds switch from the
// 128-thread CTA sort to the 256-thread CTA sort (medium_small) and from
// there to the global segmented radix sort (medium_max), and whether large
// groups whose members mostly share rank[i+h] sort only the others.  The cache is a JSON
// file of entries keyed by (GPU name, n bucket = ceil(log2 n), code bits of the
// alphabet); a sort without an explicit tuning takes the entry for its GPU
// and code bits with the nearest n bucket, else the built-in defaults.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "engine.h"
#include "libsais_gb300.h"
#include "tuning.h"

namespace gsais {

namespace {

struct CacheEntry {
    std::string gpu;
    int n_log2 = 0;
    int bits = 0;
    Tuning t;
};

std::mutex g_mu;
std::vector<CacheEntry> g_cache;
bool g_env_tried = false;
std::string g_dev_name[64];

// ---- a small reader for the cache's JSON: {"entries": [{"key": value, ...}, ...]}
// with string and integer values (other values are skipped).
struct Reader {
    const char *p, *e;
    void ws()
    {
        while (p < e && (*p == ' ' || *p == '\n' || *p == '\r' || *p == '\t')) ++p;
    }
    bool lit(char c)
    {
        ws();
        if (p < e && *p == c) {
            ++p;
            return true;
        }
        return false;
    }
    bool str(std::string &out)
    {
        ws();
        if (p >= e || *p != '"') return false;
        ++p;
        out.clear();
        while (p < e && *p != '"') {
            if (*p == '\\' && p + 1 < e) ++p;
            out.push_back(*p++);
        }
        if (p >= e) return false;
        ++p;
        return true;
    }
    // skips any value; numbers are returned in *num (when num != nullptr)
    bool value(std::string *s, double *num)
    {
        ws();
        if (p >= e) return false;
        if (*p == '"') {
            std::string tmp;
            if (!str(tmp)) return false;
            if (s) *s = tmp;
            return true;
        }
        if (*p == '{' || *p == '[') {
            const char open = *p, close = open == '{' ? '}' : ']';
            int depth = 0;
            bool in_str = false;
            for (; p < e; ++p) {
                if (in_str) {
                    if (*p == '\\') ++p;
                    else if (*p == '"') in_str = false;
                } else if (*p == '"') {
                    in_str = true;
                } else if (*p == open) {
                    ++depth;
                } else if (*p == close && --depth == 0) {
                    ++p;
                    return true;
                }
            }
            return false;
        }
        char *end = nullptr;
        const double v = std::strtod(p, &end);
        if (end != p) {
            if (num) *num = v;
            p = end;
            return true;
        }
        while (p < e && *p != ',' && *p != '}' && *p != ']') ++p;   // true / false / null
        return true;
    }
};

bool parse_entry(Reader &r, CacheEntry &ce)
{
    if (!r.lit('{')) return false;
    if (r.lit('}')) return true;
    for (;;) {
        std::string key, sval;
        double num = -1;
        if (!r.str(key) || !r.lit(':') || !r.value(&sval, &num)) return false;
        const int v = (int)num;
        if (key == "gpu") ce.gpu = sval;
        else if (key == "n_log2") ce.n_log2 = v;
        else if (key == "bits") ce.bits = v;
        else if (key == "digit_bits") ce.t.digit_bits = v;
        else if (key == "radix_items32") ce.t.radix_items32 = v;
        else if (key == "radix_items64") ce.t.radix_items64 = v;
        else if (key == "medium_small") ce.t.medium_small = v;
        else if (key == "medium_max") ce.t.medium_max = v;
        else if (key == "large_few_others") ce.t.large_few_others = v;
        if (r.lit(',')) continue;
        return r.lit('}');
    }
}

int load_file(const char *path, std::vector<CacheEntry> &out)
{
    FILE *f = std::fopen(path, "rb");
    if (!f) return -1;
    std::string text;
    char buf[4096];
    size_t got;
    while ((got = std::fread(buf, 1, sizeof buf, f)) > 0) text.append(buf, got);
    std::fclose(f);
    Reader r{text.data(), text.data() + text.size()};
    if (!r.lit('{')) return -1;
    for (;;) {
        std::string key;
        if (!r.str(key) || !r.lit(':')) return -1;
        if (key == "entries") {
            if (!r.lit('[')) return -1;
            if (!r.lit(']')) {
                for (;;) {
                    CacheEntry ce;
                    if (!parse_entry(r, ce)) return -1;
                    if (tuning_valid(ce.t) && !ce.gpu.empty()) out.push_back(ce);
                    if (r.lit(',')) continue;
                    if (!r.lit(']')) return -1;
                    break;
                }
            }
        } else if (!r.value(nullptr, nullptr)) {
            return -1;
        }
        if (r.lit(',')) continue;
        return r.lit('}') ? (int)out.size() : -1;
    }
}

const std::string &device_name(int dev)
{
    static const std::string none;
    if (dev < 0 || dev >= 64) return none;
    if (g_dev_name[dev].empty()) {
        cudaDeviceProp prop;
        if (cudaGetDeviceProperties(&prop, dev) == cudaSuccess) g_dev_name[dev] = prop.name;
        else cudaGetLastError();
    }
    return g_dev_name[dev];
}

int ceil_log2(uint64_t n)
{
    int b = 0;
    while (b < 63 && (1ull << b) < n) ++b;
    return b;
}

}  // namespace

bool tuning_valid(const Tuning &t)
{
    return t.digit_bits == 8 && radix_items_supported(4, t.radix_items32) &&
           radix_items_supported(8, t.radix_items64) && t.medium_small >= 64 && t.medium_small <= 512 &&
           t.medium_max >= t.medium_small && t.medium_max <= 4096 &&
           (t.large_few_others == 0 || t.large_few_others == 1);
}

Tuning tuning_lookup(uint64_t n, int bits)
{
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_env_tried) {
        g_env_tried = true;
        if (const char *path = std::getenv("GSAIS_TUNING_CACHE")) load_file(path, g_cache);
    }
    Tuning best;
    if (g_cache.empty()) return best;
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return best;
    }
    const std::string &name = device_name(dev);
    const int nb = ceil_log2(n);
    int dist = 1 << 30;
    for (const CacheEntry &ce : g_cache) {
        if (ce.gpu != name || ce.bits != bits) continue;
        const int d = ce.n_log2 > nb ? ce.n_log2 - nb : nb - ce.n_log2;
        if (d < dist) {
            dist = d;
            best = ce.t;
        }
    }
    return best;
}

int tuning_load_cache(const char *path)
{
    const char *p = path ? path : std::getenv("GSAIS_TUNING_CACHE");
    if (!p) return -1;
    std::vector<CacheEntry> fresh;
    const int k = load_file(p, fresh);
    if (k < 0) return -1;
    std::lock_guard<std::mutex> lock(g_mu);
    g_cache.swap(fresh);
    g_env_tried = true;
    return k;
}

}  // namespace gsais
