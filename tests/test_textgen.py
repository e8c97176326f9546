"""Seeded generators: deterministic, right shapes and value distributions."""
import numpy as np

from libsais_gb300 import textgen


def test_iid_deterministic():
    a = textgen.iid(10000, seed=1)
    b = textgen.iid(10000, seed=1)
    assert np.array_equal(a, b)
    assert set(np.unique(a)) == {65, 67, 71, 84}
    assert not np.array_equal(a, textgen.iid(10000, seed=2))


def test_genome_like_gc_and_repeats():
    t = textgen.genome_like(1 << 20, seed=2)
    assert set(np.unique(t)) <= {65, 67, 71, 84}
    gc = np.isin(t, [67, 71]).mean()
    assert 0.35 < gc < 0.47


def test_reads_gsa_valid():
    from oracle.oracle import Oracle
    r = textgen.reads_gsa(2000, ref_len=100000, seed=4)
    assert r[-1] == 0
    lens = np.diff(np.flatnonzero(r == 0), prepend=-1) - 1
    assert lens.min() >= 50 and lens.max() <= 300
    assert abs(lens.mean() - 150) < 5
    assert Oracle().gsa_valid(r)


def test_zipf_u16_range():
    z = textgen.zipf_u16(100000, seed=6)
    assert z.min() >= 1
    counts = np.bincount(z)
    assert counts.max() > 100 * np.median(counts[counts > 0])


def test_batch_strings():
    buf, offs = textgen.batch_strings(64, seed=3)
    lens = np.diff(offs)
    assert lens.min() >= 256 and lens.max() <= 4 << 20
    assert buf.size == offs[-1]
    assert 0.003 < (buf == 78).mean() < 0.02
