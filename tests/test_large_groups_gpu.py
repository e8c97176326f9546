"""Large groups with few differing members (runs, tandem repeats, periodic
texts): with the few-others path on (the default) and off, SA, BWT and
primary index are bit-exact against the oracle.  The texts are long enough
for groups above the 4096-member cut-over, and mix runs of different
periods so that some rounds take the path and others the full sort."""
import numpy as np
import pytest

import libsais_gb300 as G
from libsais_gb300 import textgen

pytestmark = pytest.mark.gpu


def texts():
    rng = np.random.default_rng(17)
    yield "all_A", textgen.constant(60_000)
    yield "period7", textgen.periodic(90_000)
    yield "period2", np.tile(np.frombuffer(b"AC", dtype=np.uint8), 40_000)
    # runs of several periods separated by random DNA
    parts = []
    for p in (1, 3, 5, 11, 64):
        unit = rng.choice(np.frombuffer(b"ACGT", dtype=np.uint8), size=p)
        parts.append(np.tile(unit, 12_000 // p + 1)[:12_000])
        parts.append(rng.choice(np.frombuffer(b"ACGT", dtype=np.uint8), size=500))
    yield "mixed_runs", np.concatenate(parts)
    # a long copied block with point changes (pairs and large groups)
    base = rng.choice(np.frombuffer(b"ACGT", dtype=np.uint8), size=20_000)
    copies = np.tile(base, 5)
    copies[rng.integers(0, copies.size, 40)] = ord("G")
    yield "copies", copies
    yield "bytes_runs", np.repeat(rng.integers(0, 256, 300).astype(np.uint8), 250)


@pytest.mark.parametrize("few", [1, 0])
def test_large_groups_bit_exact(oracle, few):
    for label, T in texts():
        _, oSA = oracle.sa(T)
        p, oU, _ = oracle.bwt_from_sa(T, oSA)
        assert G.set_tuning({"large_few_others": few}) == 0
        try:
            prim, SA, U, _ = G.sa_bwt(T)
            rc, SA2, _ = G.libsais(T)
        finally:
            G.set_tuning(None)
        assert rc == 0
        assert np.array_equal(SA.astype(np.int64), oSA), label
        assert np.array_equal(SA2.astype(np.int64), oSA), label
        assert prim == p and np.array_equal(U, oU), label
