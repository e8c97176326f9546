"""Integer alphabets (libsais_int, libsais16_int, libsais64_long,
libsais16x64_long, libsais_plcp_int), the inverse BWT (libsais_unbwt and its
aux / 16-bit / 64-bit / context forms) and the 16-bit 64-bit-index family
(libsais16x64*), through the C-ABI against the oracle."""
import numpy as np
import pytest

import libsais_gb300 as G
from libsais_gb300 import textgen

pytestmark = pytest.mark.gpu


def int_texts(rng):
    out = []
    for k in (2, 5, 300, 65535, 65536, 70_000, 1 << 20, (1 << 31) - 1):
        for n in (2, 17, 1000, 40_000):
            T = rng.integers(0, k, n).astype(np.int64)
            if n >= 1000:
                a = int(rng.integers(0, n // 2))
                L = int(rng.integers(10, n // 4))
                T[n - L:] = T[a:a + L]          # a repeat, so groups survive the seed
            out.append((T, k))
    return out


def test_libsais_int_matches_oracle(oracle):
    rng = np.random.default_rng(31)
    for T, k in int_texts(rng):
        T32 = T.astype(np.int32)
        want = oracle.sa_int_any(T32)[1]
        rc, SA = G.libsais_int(T32, k)
        assert rc == 0 and np.array_equal(SA.astype(np.int64), want), (T.size, k)
        rc, SA = G.libsais_int(T32, k, threads=4)
        assert rc == 0 and np.array_equal(SA.astype(np.int64), want)
        rc, SA64 = G.libsais64_long(T, k)
        assert rc == 0 and np.array_equal(SA64, want)
        rc, SA64 = G.libsais64_long(T, k, name="libsais16x64_long")
        assert rc == 0 and np.array_equal(SA64, want)


def test_libsais_int_rejects_symbols_outside_the_alphabet():
    T = np.array([0, 3, 1, 2], np.int32)
    assert G.libsais_int(T, 3)[0] == -1          # 3 >= k
    T[1] = -1
    assert G.libsais_int(T, 5)[0] == -1          # negative
    big = np.array([1, 1 << 33, 2], np.int64)
    assert G.libsais64_long(big, 1 << 40)[0] == -2   # symbols wider than 32 bits


def test_libsais_plcp_int(oracle):
    rng = np.random.default_rng(32)
    for T, k in int_texts(rng):
        T32 = T.astype(np.int32)
        _, SA = G.libsais_int(T32, k)
        rc, P = G.libsais_plcp_int(T32, SA)
        assert rc == 0 and np.array_equal(P.astype(np.int64), oracle.plcp(T32, SA.astype(np.int64)))


def unbwt_texts(rng):
    out = [np.frombuffer(b"banana", np.uint8).copy(), np.full(3000, 65, np.uint8),
           np.tile(np.frombuffer(b"ACGTACG", np.uint8), 500), textgen.genome_like(1 << 20, seed=4),
           textgen.iid(1 << 18, seed=5), (rng.integers(0, 256, 100_000)).astype(np.uint8)]
    for _ in range(40):
        n = int(rng.integers(2, 5000))
        out.append((rng.integers(0, int(rng.integers(1, 5)), n) + 65).astype(np.uint8))
    return out


def test_unbwt_round_trip(oracle):
    rng = np.random.default_rng(33)
    for T in unbwt_texts(rng):
        p, U, _ = G.libsais_bwt(T)
        rc, back = G.libsais_unbwt(U, p)
        assert rc == 0 and np.array_equal(back, T), T.size
        rc, back = G.libsais_unbwt(U, p, threads=2)
        assert rc == 0 and np.array_equal(back, T)
        if T.size < 5000:
            assert np.array_equal(oracle.unbwt(U, p)[1], T)


def test_unbwt_aux_64bit_ctx_and_in_place():
    T = textgen.genome_like(300_000, seed=7)
    rc, U, I, _ = G.libsais_bwt_aux(T, 64)
    assert rc == 0
    rc, back = G.libsais_unbwt_aux(U, 64, I)
    assert rc == 0 and np.array_equal(back, T)
    p, U, _ = G.libsais_bwt(T)
    rc, back = G.libsais64_unbwt(U, p)
    assert rc == 0 and np.array_equal(back, T)
    rc, back = G.libsais64_unbwt_aux(U, T.size, np.array([p], np.int64))   # r = n: I[0] is the primary index
    assert rc == 0 and np.array_equal(back, T)
    ctx = G.Context()
    try:
        rc, back = G.libsais_unbwt(U, p, ctx=ctx)
        assert rc == 0 and np.array_equal(back, T)
    finally:
        ctx.close()
    W = U.copy()
    rc, back = G.libsais_unbwt(W, p, out=W)          # U may be T
    assert rc == 0 and np.array_equal(W, T)


def test_unbwt_16bit():
    T = textgen.zipf_u16(200_000, seed=8)
    rc, U, _ = G.libsais16_bwt(T)
    assert rc > 0
    rc2, back = G.libsais16_unbwt(U, rc)
    assert rc2 == 0 and np.array_equal(back, T)
    rc3, back = G.libsais16x64_unbwt(U, rc)
    assert rc3 == 0 and np.array_equal(back, T)


def test_unbwt_rejects_a_wrong_primary_index():
    T = textgen.iid(10_000, seed=9)
    p, U, _ = G.libsais_bwt(T)
    assert G.libsais_unbwt(U, 0)[0] == -1
    assert G.libsais_unbwt(U, T.size + 1)[0] == -1


def test_libsais16x64_family(oracle):
    rng = np.random.default_rng(34)
    for n in (2, 1000, 50_000):
        T = rng.integers(1, 600, n).astype(np.uint16)
        rc, SA, F = G.libsais16x64(T)
        orc, oSA, ofreq = oracle.libsais(T)
        assert rc == 0 and np.array_equal(SA, oSA) and np.array_equal(F, ofreq)
        p, oU, _, _ = oracle.libsais_bwt(T)
        rc, U, _ = G.libsais16x64_bwt(T)
        assert rc == p and np.array_equal(U, oU)
        rc, U, I, _ = G.libsais16x64_bwt(T, r=16)
        _, _, oI, _ = oracle.libsais_bwt(T, r=16)
        assert rc == 0 and np.array_equal(I, oI)
    Tg = np.concatenate([rng.integers(1, 9, 40), [0], rng.integers(1, 9, 30), [0]]).astype(np.uint16)
    rc, SA, _ = G.libsais16x64(Tg, gsa=True)
    assert rc == 0 and np.array_equal(SA, oracle.libsais(Tg, gsa=True)[1])
