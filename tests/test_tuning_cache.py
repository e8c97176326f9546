"""The tuning cache's file format, read by the C library (no GPU needed):
entries with valid values are loaded, invalid ones skipped, malformed files
rejected with -1."""
import json

import libsais_gb300 as G
from libsais_gb300 import autotune


def test_cache_round_trip(tmp_path):
    path = str(tmp_path / "t.json")
    good = dict(autotune.DEFAULTS, gpu="NVIDIA GB300", n_log2=28, bits=2, ms=16.9)
    other = dict(good, radix_items32=16, n_log2=20)
    bad = dict(good, radix_items32=17, n_log2=24)   # no such instance: skipped when loaded
    autotune.write_cache(path, good)
    autotune.write_cache(path, other)
    autotune.write_cache(path, bad)
    with open(path) as f:
        entries = json.load(f)["entries"]
    assert len(entries) == 3
    assert G.load_tuning_cache(path) == 2
    autotune.write_cache(path, dict(good, radix_items32=28))   # same key: replaced
    assert len(autotune.read_cache(path)["entries"]) == 3


def test_malformed_cache_is_rejected(tmp_path):
    p = tmp_path / "bad.json"
    p.write_text('{"entries": [{"gpu": "x", "bits": 2,')
    assert G.load_tuning_cache(str(p)) == -1
    assert G.load_tuning_cache(str(tmp_path / "missing.json")) == -1
    p.write_text(json.dumps({"version": 1, "entries": []}))
    assert G.load_tuning_cache(str(p)) == 0
