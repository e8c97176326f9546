"""Autotuner for the suffix sort's tuning parameters.

The search space is the set of kernel instances compiled into
lib/libsais_gb300.so (include/libsais_gb300.h, gsais_tuning):

* digit_bits     radix digit width (the digit passes rank 8-bit digits);
* radix_items32  keys per thread of a digit pass over 32-bit keys: 16, 20, 24, 28
                 (the tile is 256 threads x that many keys);
* radix_items64  the same for 64-bit keys: 12, 16, 20;
* medium_small   groups of 33..medium_small members are split by a 128-thread CTA;
* medium_max     groups up to medium_max by a 256-thread CTA, larger ones by the
                 global segmented radix sort (the cut-over from segmented radix
                 sort to per-group shared-memory sort);
* large_few_others  1: a large group whose members mostly share rank[i+h] sorts
                 only the other members (runs, tandem repeats); 0: always the
                 full segmented sort.

``tune(n, bits)`` times SA+BWT of a synthetic text of n symbols whose alphabet
codes take `bits` bits, on the current GPU, by coordinate descent from the
defaults (each parameter in turn over its candidates, the others held), and
keeps a configuration only if its SA, BWT and primary index are bit-identical
to those of the defaults.  The result is stored in a JSON cache keyed by
(GPU name, n bucket = ceil(log2 n), bits); the library reads that cache
(gsais_load_tuning_cache, or $GSAIS_TUNING_CACHE on first use) and every sort
without a tuning of its own takes the entry for its GPU and code bits with the
nearest n bucket.
"""
from __future__ import annotations

import json
import math
import os
import statistics

import numpy as np

from . import textgen

CANDIDATES = {
    "digit_bits": [8],
    "radix_items32": [16, 20, 24, 28],
    "radix_items64": [12, 16, 20],
    "medium_small": [128, 256, 512],
    "medium_max": [1024, 2048, 4096],
    "large_few_others": [1, 0],
}
DEFAULTS = {"digit_bits": 8, "radix_items32": 20, "radix_items64": 16, "medium_small": 512, "medium_max": 4096,
            "large_few_others": 1}


def default_cache_path() -> str:
    return os.environ.get("GSAIS_TUNING_CACHE") or os.path.join(os.path.expanduser("~"), ".cache", "libsais_gb300",
                                                                "tuning.json")


def n_bucket(n: int) -> int:
    return max(0, math.ceil(math.log2(max(n, 1))))


def workload(n: int, bits: int, seed: int = 11) -> np.ndarray:
    """A synthetic text of n symbols whose dense codes take `bits` bits: the
    repetitive genome-like DNA text for 2 bits, otherwise i.i.d. symbols over
    2^bits byte values (at most 256)."""
    if bits <= 2:
        return textgen.genome_like(n, seed=seed)
    k = min(1 << bits, 256)
    alphabet = np.arange(256 - k, 256, dtype=np.uint8)   # codes fill `bits` bits exactly
    return textgen.iid(n, alphabet=alphabet, seed=seed)


def read_cache(path: str) -> dict:
    try:
        with open(path) as f:
            data = json.load(f)
        if isinstance(data, dict) and isinstance(data.get("entries"), list):
            return data
    except (OSError, ValueError):
        pass
    return {"version": 1, "entries": []}


def write_cache(path: str, entry: dict) -> None:
    data = read_cache(path)
    key = (entry["gpu"], entry["n_log2"], entry["bits"])
    data["entries"] = [e for e in data["entries"] if (e.get("gpu"), e.get("n_log2"), e.get("bits")) != key]
    data["entries"].append(entry)
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def tune(n: int, bits: int = 2, steps: int = 3, text: np.ndarray | None = None, cache_path: str | None = None,
         write: bool = True, ctx=None) -> dict:
    """Tunes SA+BWT for (this GPU, n, bits) and returns the cache entry
    (written to the cache unless write=False).  `text` overrides the synthetic
    workload (its length is n).  Needs torch with CUDA."""
    import torch

    import libsais_gb300 as G

    T = text if text is not None else workload(n, bits)
    n = int(T.size)
    dT = torch.from_numpy(T).cuda()
    dSA = torch.empty(n, dtype=torch.int32, device="cuda")
    dU = torch.empty(n, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()

    def run(cfg):
        if G.set_tuning(cfg, ctx=ctx) != 0:
            raise ValueError(f"rejected tuning {cfg}")
        prim = G.sa_bwt_device(dT, dSA, dU, ctx=ctx, stream=stream)   # warm-up, and the output to compare
        if prim < 0:
            raise RuntimeError(f"sort failed with {cfg}: {prim}")
        out = (prim, dSA.clone(), dU.clone())
        times = []
        for _ in range(steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            G.sa_bwt_device(dT, dSA, dU, ctx=ctx, stream=stream)
            e1.record(stream)
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1))
        return statistics.median(times), out

    try:
        best = dict(DEFAULTS)
        best_ms, ref = run(best)
        default_ms = best_ms
        tried = 1
        for name, values in CANDIDATES.items():
            for v in values:
                if v == best[name]:
                    continue
                cfg = dict(best, **{name: v})
                if cfg["medium_max"] < cfg["medium_small"]:
                    continue
                ms, out = run(cfg)
                tried += 1
                same = out[0] == ref[0] and torch.equal(out[1], ref[1]) and torch.equal(out[2], ref[2])
                if not same:
                    raise RuntimeError(f"tuning {cfg} changed the output")
                if ms < best_ms * 0.99:
                    best, best_ms = cfg, ms
    finally:
        G.set_tuning(None, ctx=ctx)
    entry = dict(best)
    entry.update({"gpu": torch.cuda.get_device_name(), "n_log2": n_bucket(n), "bits": int(bits),
                  "ms": round(best_ms, 4), "default_ms": round(default_ms, 4), "configs_tried": tried,
                  "outputs_identical": True})
    if write:
        path = cache_path or default_cache_path()
        write_cache(path, entry)
        G.load_tuning_cache(path)
    return entry
