"""Batched path: many independent strings sorted together in one set of
launches per doubling round must give, for every string, exactly the SA,
BWT and primary index libsais gives for that string alone (oracle)."""
import numpy as np
import pytest

import libsais_gb300 as G
from libsais_gb300 import textgen

pytestmark = pytest.mark.gpu


def check_batch(oracle, T, offs):
    rc, SA, U, P = G.batch_sa_bwt(T, offs)
    assert rc == 0
    for s in range(offs.size - 1):
        a, b = int(offs[s]), int(offs[s + 1])
        t = T[a:b]
        if t.size == 0:
            assert P[s] == 0
            continue
        _, oSA = oracle.sa(t)
        p, oU, _, _ = oracle.libsais_bwt(t)
        assert np.array_equal(SA[a:b].astype(np.int64), oSA), s
        assert np.array_equal(U[a:b], oU), s
        assert P[s] == p, (s, P[s], p)


def test_batch_random_small(oracle):
    rng = np.random.default_rng(31)
    for trial in range(40):
        count = int(rng.integers(1, 120))
        lens = rng.integers(0, 600, count)
        lens[rng.random(count) < 0.1] = 1
        offs = np.zeros(count + 1, dtype=np.int64)
        offs[1:] = np.cumsum(lens)
        k = int(rng.integers(1, 5))
        base = 0 if trial % 3 == 0 else 65
        T = (rng.integers(0, k, int(offs[-1])) + base).astype(np.uint8)
        check_batch(oracle, T, offs)


def test_batch_repeats_across_strings(oracle):
    """Identical and periodic strings: groups must never span strings."""
    parts = [np.frombuffer(b"ACGTACGTAC" * 30, dtype=np.uint8)] * 5 + [np.full(700, 65, np.uint8)] * 4
    parts += [textgen.iid(1500, seed=s) for s in range(6)]
    lens = np.array([p.size for p in parts])
    offs = np.zeros(len(parts) + 1, dtype=np.int64)
    offs[1:] = np.cumsum(lens)
    check_batch(oracle, np.concatenate(parts), offs)


def test_batch_workload_shape(oracle):
    """The batched workload's generator (log-uniform lengths, ACGT + 1% N), scaled down."""
    T, offs = textgen.batch_strings(256, lo=256, hi=1 << 16, seed=3)
    check_batch(oracle, T, offs)


def test_batch_device_api(oracle):
    torch = pytest.importorskip("torch")
    T, offs = textgen.batch_strings(64, lo=256, hi=1 << 14, seed=7)
    n = int(offs[-1])
    dT = torch.from_numpy(T).cuda()
    dO = torch.from_numpy(offs).cuda()
    dSA = torch.empty(n, dtype=torch.int32, device="cuda")
    dU = torch.empty(n, dtype=torch.uint8, device="cuda")
    dP = torch.empty(offs.size - 1, dtype=torch.int32, device="cuda")
    assert G.batch_sa_bwt_device(dT, dO, dSA, dU, dP) == 0
    rc, SA, U, P = G.batch_sa_bwt(T, offs)
    assert np.array_equal(dSA.cpu().numpy(), SA)
    assert np.array_equal(dU.cpu().numpy(), U)
    assert np.array_equal(dP.cpu().numpy(), P)
