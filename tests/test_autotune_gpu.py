"""The autotuner and the tuning parameters it searches.

* Every candidate value of every tuning parameter (radix keys per thread for
  32- and 64-bit keys, the medium-group cut-overs) gives bit-exact SA, BWT and
  primary index against the oracle, on texts that reach each path: the
  genome-like text (32-bit seed keys), a period-7 text (groups larger than the
  medium cut-over go through the 64-bit segmented radix sort) and bytes.
* tune() writes a cache entry keyed by (GPU, n bucket, code bits) whose
  configuration reproduced the default output; the cache round-trips through
  the C loader, and a sort without a tuning of its own then runs with the
  cached entry.
"""
import json

import numpy as np
import pytest

import libsais_gb300 as G
from libsais_gb300 import autotune, textgen

pytestmark = pytest.mark.gpu


def texts():
    rng = np.random.default_rng(5)
    yield "genome", textgen.genome_like(150_000, seed=41)
    yield "period7", textgen.periodic(120_000)
    yield "bytes", rng.integers(0, 256, 100_000).astype(np.uint8)


@pytest.mark.parametrize("name", list(autotune.CANDIDATES))
def test_every_candidate_is_bit_exact(oracle, name):
    for label, T in texts():
        _, oSA = oracle.sa(T)
        p, oU, _ = oracle.bwt_from_sa(T, oSA)
        for v in autotune.CANDIDATES[name]:
            cfg = {name: v}
            if name == "medium_max":
                cfg["medium_small"] = min(v, 512)
            assert G.set_tuning(cfg) == 0
            try:
                prim, SA, U, _ = G.sa_bwt(T)
                used = G.last_tuning()
            finally:
                G.set_tuning(None)
            assert used[name] == v
            assert prim == p, (label, cfg)
            assert np.array_equal(SA.astype(np.int64), oSA), (label, cfg)
            assert np.array_equal(U, oU), (label, cfg)


def test_invalid_tuning_is_rejected():
    assert G.set_tuning({"digit_bits": 4}) == -1
    assert G.set_tuning({"radix_items32": 18}) == -1
    assert G.set_tuning({"medium_small": 512, "medium_max": 256}) == -1
    assert G.set_tuning(None) == 0


def test_tune_writes_and_applies_the_cache(tmp_path, oracle):
    path = str(tmp_path / "tuning.json")
    e2 = autotune.tune(1 << 20, bits=2, steps=2, cache_path=path)
    e8 = autotune.tune(1 << 18, bits=8, steps=2, cache_path=path)
    with open(path) as f:
        data = json.load(f)
    assert len(data["entries"]) == 2
    for e in (e2, e8):
        assert e["outputs_identical"] and e["configs_tried"] >= 2
    assert G.load_tuning_cache(path) == 2
    # a sort of a 2-bit text of the tuned bucket runs with the cached entry
    T = textgen.genome_like(1 << 20, seed=42)
    prim, SA, U, _ = G.sa_bwt(T)
    used = G.last_tuning()
    assert {k: used[k] for k in autotune.DEFAULTS} == {k: e2[k] for k in autotune.DEFAULTS}
    _, oSA = oracle.sa(T)
    assert np.array_equal(SA.astype(np.int64), oSA)
    # an empty cache brings the defaults back
    empty = str(tmp_path / "empty.json")
    with open(empty, "w") as f:
        json.dump({"version": 1, "entries": []}, f)
    assert G.load_tuning_cache(empty) == 0
    G.sa_bwt(T)
    assert {k: G.last_tuning()[k] for k in autotune.DEFAULTS} == autotune.DEFAULTS
