"""The CPU oracle against the reference's golden vectors, a brute-force
sorter, and (where the reference compiled here) the reference itself."""
import itertools
import os

import numpy as np
import pytest

from conftest import golden_cases, load_golden


def brute_sa(T, gsa=False):
    n = len(T)
    if not gsa:
        return np.array(sorted(range(n), key=lambda i: tuple(T[i:])), dtype=np.int64)
    # separators compare by position: the j-th 0 becomes -(count - j)
    seps = np.flatnonzero(T == 0)
    key = T.astype(np.int64)
    key[seps] = np.arange(len(seps)) - len(seps)
    return np.array(sorted(range(n), key=lambda i: tuple(key[i:])), dtype=np.int64)


@pytest.mark.parametrize("path", golden_cases(), ids=lambda p: os.path.basename(p)[:-4])
def test_oracle_matches_golden(oracle, path):
    g = load_golden(path)
    T, gsa = g["T"], bool(g["gsa"])
    rc, SA, freq = oracle.libsais(T, gsa=gsa)
    assert rc == 0
    assert np.array_equal(SA, g["SA"].astype(np.int64))
    assert np.array_equal(freq, g["freq"].astype(np.int64))
    if "U" in g:
        p, U, _, _ = oracle.libsais_bwt(T)
        assert p == int(g["primary"])
        assert np.array_equal(U, g["U"])
    if "I8" in g:
        a, _, I, _ = oracle.libsais_bwt(T, r=8)
        assert a == 0 and np.array_equal(I, g["I8"].astype(np.int64))
    P = oracle.plcp(T, SA, gsa=gsa)
    assert np.array_equal(P, g["PLCP"].astype(np.int64))
    assert np.array_equal(oracle.lcp(P, SA), g["LCP"].astype(np.int64))


def test_oracle_exhaustive_binary(oracle):
    """Every string over {A, C} up to length 12 against a brute-force sort."""
    for n in range(1, 13):
        for bits in itertools.product(b"AC", repeat=n):
            T = np.frombuffer(bytes(bits), dtype=np.uint8)
            rc, SA = oracle.sa(T)
            assert rc == 0
            assert np.array_equal(SA, brute_sa(T)), bytes(bits)


def test_oracle_random_small(oracle):
    rng = np.random.default_rng(7)
    for _ in range(1500):
        n = int(rng.integers(1, 50))
        k = int(rng.integers(1, 6))
        T = rng.integers(0, k, n).astype(np.uint8)
        assert np.array_equal(oracle.sa(T)[1], brute_sa(T))
        T16 = (rng.integers(0, k, n) * 9000).astype(np.uint16)
        assert np.array_equal(oracle.sa(T16)[1], brute_sa(T16))
        assert oracle.check_sa(T, oracle.sa(T)[1])


def test_oracle_gsa_rules(oracle):
    rng = np.random.default_rng(8)
    for _ in range(500):
        parts = []
        for _ in range(int(rng.integers(1, 6))):
            parts.append(rng.integers(1, 4, int(rng.integers(1, 8))).astype(np.uint8))
            parts.append(np.zeros(1, np.uint8))
        G = np.concatenate(parts)
        rc, SA = oracle.sa(G, gsa=True)
        assert rc == 0 and np.array_equal(SA, brute_sa(G, gsa=True))
        assert oracle.check_sa(G, SA, gsa=True)
    assert not oracle.gsa_valid(np.array([0, 1, 0], np.uint8))      # leading separator
    assert not oracle.gsa_valid(np.array([1, 0, 0], np.uint8))      # empty string
    assert not oracle.gsa_valid(np.array([1, 2], np.uint8))         # not terminated
    assert oracle.gsa_valid(np.array([1, 0, 2, 0], np.uint8))


def test_oracle_check_sa_rejects(oracle):
    T = np.frombuffer(b"mississippi", dtype=np.uint8)
    _, SA = oracle.sa(T)
    assert oracle.check_sa(T, SA)
    bad = SA.copy()
    bad[[2, 3]] = bad[[3, 2]]
    assert not oracle.check_sa(T, bad)


REF = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle", "_ref", "libsais_ref.so")


@pytest.mark.skipif(not os.path.exists(REF), reason="reference not compiled here")
def test_oracle_matches_reference_random():
    from oracle.oracle import Oracle, Reference
    O, R = Oracle(), Reference()
    rng = np.random.default_rng(9)
    for _ in range(400):
        n = int(rng.integers(2, 400))
        k = int(rng.integers(1, 5))
        T = (rng.integers(0, k, n) + 65).astype(np.uint8)
        rc, SA, freq = R.libsais(T)
        assert np.array_equal(O.sa(T)[1], SA.astype(np.int64))
        p, U, _, _ = R.libsais_bwt(T)
        po, Uo, _, _ = O.libsais_bwt(T)
        assert p == po and np.array_equal(U, Uo)
        _, P = R.plcp(T, SA)
        assert np.array_equal(O.plcp(T, SA), P.astype(np.int64))
    T = (rng.integers(0, 4, 1 << 20) + 65).astype(np.uint8)
    assert np.array_equal(O.sa(T)[1], R.libsais(T)[1].astype(np.int64))


def test_oracle_unbwt_round_trip(oracle):
    """Inverse BWT restatement: BWT -> text on random and structured texts,
    8- and 16-bit, including a primary index that is not a row of the text
    (the walk must notice)."""
    rng = np.random.default_rng(21)
    texts = [np.frombuffer(b"banana", np.uint8).copy(), np.full(50, 65, np.uint8),
             np.tile(np.frombuffer(b"ACGTACG", np.uint8), 30)]
    for _ in range(300):
        n = int(rng.integers(2, 300))
        k = int(rng.integers(1, 6))
        texts.append((rng.integers(0, k, n) + 65).astype(np.uint8))
    for _ in range(50):
        n = int(rng.integers(2, 300))
        texts.append(rng.integers(0, 70000 % 65536, n).astype(np.uint16))
    for T in texts:
        p, U, _, _ = oracle.libsais_bwt(T)
        rc, back = oracle.unbwt(U, p)
        assert rc == 0 and np.array_equal(back, T)
    assert oracle.unbwt(np.frombuffer(b"abc", np.uint8).copy(), 0)[0] == -1


def test_oracle_plcp_int(oracle):
    rng = np.random.default_rng(22)
    for _ in range(100):
        n = int(rng.integers(2, 200))
        k = int(rng.integers(1, 1 << 20))
        T = rng.integers(0, k, n).astype(np.int32)
        _, SA = oracle.sa_int(T, k)
        P = oracle.plcp(T, SA)
        SAi = [tuple(T[i:]) for i in SA]
        for j in range(n):
            prev = SA[j - 1] if j else None
            want = 0
            if prev is not None:
                a, b = T[SA[j]:], T[prev:]
                while want < min(len(a), len(b)) and a[want] == b[want]:
                    want += 1
            assert P[SA[j]] == want
        assert SAi == sorted(SAi)


@pytest.mark.skipif(not os.path.exists(REF), reason="reference not compiled here")
def test_oracle_new_families_match_reference():
    """libsais_int, libsais_plcp_int and libsais_unbwt/libsais16_unbwt of the
    compiled reference against the restatement."""
    from oracle.oracle import Oracle, Reference
    O, R = Oracle(), Reference()
    rng = np.random.default_rng(23)
    for _ in range(200):
        n = int(rng.integers(2, 500))
        k = int(rng.choice([2, 5, 300, 70000]))
        T = rng.integers(0, k, n).astype(np.int32)
        rc, SA = R.libsais_int(T, k)
        assert rc == 0 and np.array_equal(O.sa_int(T, k)[1], SA.astype(np.int64))
        rc, P = R.plcp_int(T, SA)
        assert rc == 0 and np.array_equal(O.plcp(T, SA), P.astype(np.int64))
    for _ in range(200):
        n = int(rng.integers(2, 500))
        sixteen = rng.random() < 0.3
        T = rng.integers(0, 40000 if sixteen else 4, n).astype(np.uint16 if sixteen else np.uint8)
        p, U, _, _ = O.libsais_bwt(T)
        rc, back = R.unbwt(U, p)
        assert rc == 0 and np.array_equal(back, T)
        assert np.array_equal(O.unbwt(U, p)[1], back)
