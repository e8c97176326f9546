"""GPU parity: every construction entry point, called through the C-ABI, must
be bit-exact against the CPU oracle (itself pinned to the reference's golden
vectors) on the same inputs.  Integer outputs, so the tolerance is zero."""
import itertools
import os

import numpy as np
import pytest

import libsais_gb300 as G
from libsais_gb300 import textgen
from conftest import golden_cases, load_golden

pytestmark = pytest.mark.gpu


def check_all(oracle, T, gsa=False, plcp=True, r=8):
    """SA, freq, BWT/primary, aux I, PLCP, LCP against the oracle."""
    T = np.ascontiguousarray(T)
    sixteen = T.dtype == np.uint16
    ors, oSA, ofreq = oracle.libsais(T, gsa=gsa)
    if gsa:
        rc, SA, F = (G.libsais16_gsa if sixteen else G.libsais_gsa)(T)
    else:
        rc, SA, F = (G.libsais16 if sixteen else G.libsais)(T)
    assert rc == ors == 0
    assert np.array_equal(SA.astype(np.int64), oSA), "SA mismatch"
    assert np.array_equal(F.astype(np.int64), ofreq), "freq mismatch"
    if not gsa:
        p, oU, oI, _ = oracle.libsais_bwt(T)
        prim, U, _ = (G.libsais16_bwt if sixteen else G.libsais_bwt)(T)
        assert prim == p, "primary index mismatch"
        assert np.array_equal(U, oU), "BWT mismatch"
        if r:
            _, _, oI, _ = oracle.libsais_bwt(T, r=r)
            rc, Ua, I, _ = (G.libsais16_bwt_aux if sixteen else G.libsais_bwt_aux)(T, r)
            assert rc == 0 and np.array_equal(Ua, oU) and np.array_equal(I.astype(np.int64), oI)
    if plcp:
        oP = oracle.plcp(T, oSA, gsa=gsa)
        if sixteen:
            rc, P = (G.libsais16_plcp_gsa if gsa else G.libsais16_plcp)(T, SA)
        else:
            rc, P = (G.libsais_plcp_gsa if gsa else G.libsais_plcp)(T, SA)
        assert rc == 0 and np.array_equal(P.astype(np.int64), oP), "PLCP mismatch"
        rc, L = G.libsais_lcp(P, SA)
        assert rc == 0 and np.array_equal(L.astype(np.int64), oracle.lcp(oP, oSA)), "LCP mismatch"
    return SA


@pytest.mark.parametrize("path", golden_cases(), ids=lambda p: os.path.basename(p)[:-4])
def test_golden_vectors(path):
    g = load_golden(path)
    T, gsa = g["T"], bool(g["gsa"])
    sixteen = T.dtype == np.uint16
    f = (G.libsais16_gsa if gsa else G.libsais16) if sixteen else (G.libsais_gsa if gsa else G.libsais)
    rc, SA, F = f(T)
    assert rc == 0
    assert np.array_equal(SA, g["SA"]) and np.array_equal(F, g["freq"])
    if "U" in g:
        prim, U, _ = (G.libsais16_bwt if sixteen else G.libsais_bwt)(T)
        assert prim == int(g["primary"]) and np.array_equal(U, g["U"])
    if "I8" in g:
        rc, _, I, _ = G.libsais_bwt_aux(T, 8)
        assert rc == 0 and np.array_equal(I, g["I8"])
        rc, SA64, _ = G.libsais64(T)
        assert rc == 0 and np.array_equal(SA64, g["SA"].astype(np.int64))
    pf = (G.libsais16_plcp_gsa if gsa else G.libsais16_plcp) if sixteen else (G.libsais_plcp_gsa if gsa else G.libsais_plcp)
    rc, P = pf(T, SA)
    assert rc == 0 and np.array_equal(P, g["PLCP"])
    rc, L = G.libsais_lcp(P, SA)
    assert rc == 0 and np.array_equal(L, g["LCP"])


def test_exhaustive_binary_strings(oracle):
    """All strings over {A, C} of length 2..10 (SA and BWT)."""
    for n in range(2, 11):
        for bits in itertools.product(b"AC", repeat=n):
            T = np.frombuffer(bytes(bits), dtype=np.uint8)
            _, oSA = oracle.sa(T)
            rc, SA, _ = G.libsais(T)
            assert rc == 0 and np.array_equal(SA.astype(np.int64), oSA), bytes(bits)


def test_random_small(oracle):
    rng = np.random.default_rng(11)
    for trial in range(300):
        n = int(rng.integers(2, 300))
        k = int(rng.integers(1, 6))
        base = 0 if trial % 3 == 0 else 65
        T = (rng.integers(0, k, n) + base).astype(np.uint8)
        check_all(oracle, T, plcp=trial % 2 == 0, r=2 ** int(rng.integers(1, 5)))


def test_random_small_u16(oracle):
    rng = np.random.default_rng(12)
    for trial in range(120):
        n = int(rng.integers(2, 400))
        T = (rng.integers(0, int(rng.integers(1, 7)), n) * 9973).astype(np.uint16)
        check_all(oracle, T, plcp=True, r=4)


def test_runs_and_tandem_repeats(oracle):
    """Runs of the smallest symbol at the end and inside the text, and tandem
    repeats: groups of every size around the 32-suffix small/large cut-over,
    including the last group of the active list ending mid-window."""
    rng = np.random.default_rng(5)
    for trial in range(200):
        m = int(rng.integers(50, 5000))
        s = (rng.integers(0, 4, m) + 65).astype(np.uint8)
        s[-int(rng.integers(1, 30)):] = 65
        s[int(rng.integers(0, m // 2)):][:40] = 65
        rc, SA, _ = G.libsais(s)
        assert rc == 0 and np.array_equal(SA.astype(np.int64), oracle.sa(s)[1]), trial
    for trial in range(60):
        n = int(rng.integers(2000, 20000))
        t = (rng.integers(0, 4, n) + 65).astype(np.uint8)
        a = int(rng.integers(0, n // 2))
        L = int(rng.integers(50, n // 4))
        p = int(rng.integers(2, 40))
        t[a:a + L] = np.tile(t[a:a + p], L // p + 1)[:L]
        check_all(oracle, t, plcp=trial % 4 == 0, r=0)


def test_copied_segments_pairs(oracle):
    """Exact and near-exact copies: tied suffix pairs ordered by direct text
    comparison, including copies that run to the end of the text (one suffix
    ends inside the common part), copies longer than the comparison limit
    (the pair goes back to doubling), 4-bit packed codes (8 and 16 symbols,
    8- and 16-bit texts) and 2-bit codes."""
    rng = np.random.default_rng(17)
    cases = []
    for sigma, dtype in ((4, np.uint8), (8, np.uint8), (16, np.uint16), (3, np.uint16)):
        n = int(rng.integers(150_000, 300_000))
        t = rng.integers(0, sigma, n).astype(dtype) + (65 if dtype == np.uint8 else 1000)
        L = int(rng.integers(2_000, 20_000))
        a = int(rng.integers(0, n // 3))
        t[n - L:] = t[a:a + L]                             # copy reaching the end of the text
        b = int(rng.integers(n // 3, n // 2))
        t[b:b + 5_000] = t[a + 100:a + 5_100]               # copy inside the text
        t[b + int(rng.integers(10, 4_000))] = t[0]          # one substitution in it
        cases.append(t)
    n = 200_000
    t = (rng.integers(0, 4, n) + 65).astype(np.uint8)
    t[110_000:190_000] = t[10_000:90_000]                  # 80 000-symbol exact copy: past the limit
    cases.append(t)
    for t in cases:
        check_all(oracle, t, plcp=False, r=0)
        st = G.last_stats()
        assert st["pairs_direct"] > 0, st


def test_pinned_host_buffers_early_copy(oracle):
    """Host calls whose SA buffer is pinned: SA leaves for the host while the
    doubling rounds run and the slots the rounds write are patched afterwards
    (early_patch > 0 when that path ran).  SA, BWT and primary index must
    equal the oracle's, for libsais, the combined SA + BWT call and
    libsais_bwt (which returns no SA: with U pinned only the BWT is taken
    early); a periodic text leaves too many unresolved suffixes and takes the
    plain copy.  With U pinned, the BWT is taken at the same point and its
    unresolved rows rewritten later, including texts whose suffix 0 is still
    unresolved then (a tied pair, a group of three)."""
    torch = pytest.importorskip("torch")
    lib = G.load()
    rng = np.random.default_rng(23)
    dna = lambda m: (rng.integers(0, 4, m) + 65).astype(np.uint8)
    X = dna(5_000)
    Y = dna(3_000)
    # suffix 0 in a tied pair (X again at the end; Y three times keeps a
    # group for the rounds) and in a group of three
    pair0 = np.concatenate([X, dna(50_000), Y, dna(50_000), Y, dna(50_000), Y, dna(50_000), X])
    group0 = np.concatenate([X, dna(100_000), X, dna(100_000), X[:4_000]])
    cases = [(textgen.genome_like(1 << 20, seed=5), True),
             (textgen.genome_like(300_001, seed=6), True),
             (pair0, True), (group0, True),
             ((rng.integers(0, 256, 200_000)).astype(np.uint8), None),
             (np.frombuffer(b"abcab" * 40_000, dtype=np.uint8).copy(), False)]
    for T, expect_early in cases:
        n = T.size
        _, oSA, _ = oracle.libsais(T)
        p, oU, _, _ = oracle.libsais_bwt(T)
        hT = torch.from_numpy(T).pin_memory()
        for call in ("sa", "bwt", "sa_bwt"):
            hSA = torch.full((n,), -7, dtype=torch.int32).pin_memory()
            hU = torch.zeros(n, dtype=torch.uint8).pin_memory()
            if call == "sa":
                assert lib.libsais(hT.data_ptr(), hSA.data_ptr(), n, 0, None) == 0
            elif call == "bwt":
                assert lib.libsais_bwt(hT.data_ptr(), hU.data_ptr(), hSA.data_ptr(), n, 0, None) == p
            else:
                assert lib.gsais_sa_bwt(None, hT.data_ptr(), 1, n, hSA.data_ptr(), 4, hU.data_ptr(), None, 4) == p
            early = G.last_stats()["early_patch"]
            if expect_early is not None:
                assert (early > 0) == expect_early, (call, n, early)
            if call != "bwt":
                assert np.array_equal(hSA.numpy().astype(np.int64), oSA), (call, n)
            if call != "sa":
                assert np.array_equal(hU.numpy(), oU), (call, n)


def random_gsa(rng, count, maxlen, k):
    parts = []
    for _ in range(count):
        parts.append(rng.integers(1, k + 1, int(rng.integers(1, maxlen + 1))).astype(np.uint8))
        parts.append(np.zeros(1, np.uint8))
    return np.concatenate(parts)


def test_random_gsa(oracle):
    rng = np.random.default_rng(13)
    for trial in range(150):
        T = random_gsa(rng, int(rng.integers(1, 30)), int(rng.integers(1, 40)), int(rng.integers(1, 4)))
        check_all(oracle, T, gsa=True)


def test_gsa_invalid_inputs_fill_freq(oracle):
    for bad in ([0, 1, 2, 0], [1, 0, 0, 2, 0], [3, 1, 0, 0]):
        T = np.array(bad, np.uint8)
        rc, _, F = G.libsais_gsa(T)
        assert rc == -1
        if T[-1] == 0:   # past the host-side T[n-1] check, freq is filled as the reference does
            assert np.array_equal(F.astype(np.int64), oracle.freq(T))


@pytest.mark.parametrize("name,make", [
    ("dna_iid_1M", lambda: textgen.iid(1 << 20, seed=1)),
    ("genome_like_4M", lambda: textgen.genome_like(1 << 22, seed=2)),
    ("all_A_1M", lambda: textgen.constant(1 << 20)),
    ("period7_1M", lambda: textgen.periodic(1 << 20)),
    ("bytes_1M", lambda: np.random.default_rng(3).integers(0, 256, 1 << 20).astype(np.uint8)),
    ("zeros_256K", lambda: np.zeros(1 << 18, np.uint8)),
    ("binary_1M", lambda: np.random.default_rng(4).integers(0, 2, 1 << 20).astype(np.uint8)),
    ("dna_n_1M", lambda: textgen.dna_with_n(1 << 20, 0.01, seed=5)),
])
def test_medium_texts(oracle, name, make):
    check_all(oracle, make())


def test_medium_u16_zipf(oracle):
    check_all(oracle, textgen.zipf_u16(1 << 20, seed=6))


def test_medium_gsa_reads(oracle):
    check_all(oracle, textgen.reads_gsa(1 << 14, ref_len=200_000, seed=4), gsa=True)


def test_c1_workload(oracle):
    """The plain single-string workload at full size: n = 2^24 i.i.d. ACGT."""
    check_all(oracle, textgen.iid(1 << 24, seed=1), r=0)


def test_64bit_api(oracle):
    T = textgen.genome_like(1 << 20, seed=9)
    _, oSA = oracle.sa(T)
    rc, SA, F = G.libsais64(T)
    assert rc == 0 and SA.dtype == np.int64 and np.array_equal(SA, oSA)
    assert np.array_equal(F, oracle.freq(T))
    p, oU, _, _ = oracle.libsais_bwt(T)
    prim, U, _ = G.libsais64_bwt(T)
    assert prim == p and np.array_equal(U, oU)
    _, _, oI, _ = oracle.libsais_bwt(T, r=16)
    rc, _, I, _ = G.libsais64_bwt_aux(T, 16)
    assert rc == 0 and np.array_equal(I, oI)
    rc, P = G.libsais64_plcp(T, SA)
    oP = oracle.plcp(T, oSA)
    assert rc == 0 and np.array_equal(P, oP)
    rc, L = G.libsais64_lcp(P, SA)
    assert rc == 0 and np.array_equal(L, oracle.lcp(oP, oSA))
    G64 = textgen.reads_gsa(3000, ref_len=50_000, seed=10)
    rc, SAg, _ = G.libsais64_gsa(G64)
    assert rc == 0 and np.array_equal(SAg, oracle.sa(G64, gsa=True)[1])
    rc, Pg = G.libsais64_plcp_gsa(G64, SAg)
    assert rc == 0 and np.array_equal(Pg, oracle.plcp(G64, SAg, gsa=True))


def test_context_reuse_across_sizes(oracle):
    ctx = G.Context()
    try:
        for n, seed in ((1 << 18, 1), (1000, 2), (1 << 19, 3), (17, 4)):
            T = textgen.iid(n, seed=seed)
            rc, SA, _ = G.libsais(T, ctx=ctx)
            assert rc == 0 and np.array_equal(SA.astype(np.int64), oracle.sa(T)[1])
            p, U, _ = G.libsais_bwt(T, ctx=ctx)
            po, Uo, _, _ = oracle.libsais_bwt(T)
            assert p == po and np.array_equal(U, Uo)
    finally:
        ctx.close()


def test_bwt_in_place(oracle):
    """U may be T (include/libsais.h: 'can be T')."""
    T = textgen.iid(5000, seed=3)
    po, Uo, _, _ = oracle.libsais_bwt(T)
    buf = T.copy()
    rc, U, _, _ = G._bwt_call("libsais_bwt", buf, 4, U=buf)
    assert rc == po and np.array_equal(buf, Uo)


def test_lcp_may_alias_sa(oracle):
    T = textgen.iid(7000, seed=4)
    rc, SA, _ = G.libsais(T)
    rc, P = G.libsais_plcp(T, SA)
    expect = oracle.lcp(P.astype(np.int64), SA.astype(np.int64))
    buf = SA.copy()
    rc, L = G.libsais_lcp(P, buf, out=buf)
    assert rc == 0 and np.array_equal(buf.astype(np.int64), expect)


@pytest.mark.parametrize("n", [(1 << 24) + 12345, 1 << 26, (1 << 26) + 12345])
def test_lcp_partitioned_gather(n):
    """From 2^26 rows on, LCP[i] = PLCP[SA[i]] goes through position buckets
    (partition, in-place fetch, place); below, a direct gather.  Checked
    against plain indexing on any permutation and any PLCP values, in place
    over SA, for int64 arrays and through the host entry point."""
    torch = pytest.importorskip("torch")
    g = torch.Generator(device="cuda").manual_seed(n)
    dSA = torch.randperm(n, device="cuda", generator=g).to(torch.int32)
    dP = torch.randint(0, n, (n,), device="cuda", generator=g, dtype=torch.int32)   # PLCP values are < n
    expect = dP[dSA.long()]
    st = torch.cuda.current_stream()   # the inputs were made on this stream
    dL = torch.full_like(dSA, -1)
    assert G.lcp_device(dP, dSA, dL, stream=st) == 0
    assert torch.equal(dL, expect)
    buf = dSA.clone()
    assert G.lcp_device(dP, buf, buf, stream=st) == 0   # LCP may be the SA buffer
    assert torch.equal(buf, expect)
    dL64 = torch.empty(n, dtype=torch.int64, device="cuda")
    assert G.lcp_device(dP.long(), dSA.long(), dL64, stream=st) == 0
    assert torch.equal(dL64, expect.long())
    if n == (1 << 26) + 12345:
        rc, L = G.libsais_lcp(dP.cpu().numpy(), dSA.cpu().numpy())
        assert rc == 0 and np.array_equal(L, expect.cpu().numpy())


@pytest.mark.parametrize("key_bits", [32, 64, 0])
def test_seed_key_widths(oracle, key_bits):
    """32- and 64-bit seed keys and the automatic choice (64 bits for 3- and
    4-bit codes) give the same outputs: a DNA text with 1 % 'N' (5 symbols,
    3-bit codes), a repetitive 9-symbol text (4-bit codes) and a read set
    (GSA, the separator and ACGT: 3-bit codes)."""
    prev = G.set_seed_key_bits(key_bits)
    try:
        rng = np.random.default_rng(41)
        nine = (rng.integers(0, 9, 300_000) + 97).astype(np.uint8)
        nine[150_000:] = nine[:150_000]   # one long copy
        check_all(oracle, textgen.dna_with_n(1 << 19, seed=9), plcp=True, r=4)
        check_all(oracle, nine, plcp=False, r=0)
        reads = textgen.reads_gsa(4000, ref_len=100_000, seed=11)
        check_all(oracle, reads, gsa=True, plcp=True)
        assert G.last_stats()["seed_symbols"] == (10 if key_bits == 32 else 21)
    finally:
        G.set_seed_key_bits(prev)


def test_combined_sa_bwt(oracle):
    T = textgen.genome_like(1 << 20, seed=12)
    prim, SA, U, F = G.sa_bwt(T)
    p, oU, _, _ = oracle.libsais_bwt(T)
    assert prim == p and np.array_equal(U, oU)
    assert np.array_equal(SA.astype(np.int64), oracle.sa(T)[1])


def test_device_api(oracle):
    torch = pytest.importorskip("torch")
    T = textgen.genome_like(1 << 20, seed=13)
    dT = torch.from_numpy(T).cuda()
    dSA = torch.empty(T.size, dtype=torch.int32, device="cuda")
    dU = torch.empty(T.size, dtype=torch.uint8, device="cuda")
    prim = G.sa_bwt_device(dT, dSA, dU, stream=torch.cuda.current_stream())
    p, oU, _, _ = oracle.libsais_bwt(T)
    _, oSA = oracle.sa(T)
    assert prim == p
    assert np.array_equal(dU.cpu().numpy(), oU)
    assert np.array_equal(dSA.cpu().numpy().astype(np.int64), oSA)
    dSA64 = torch.empty(T.size, dtype=torch.int64, device="cuda")
    assert G.sa_device(dT, dSA64) == 0
    assert np.array_equal(dSA64.cpu().numpy(), oSA)
    dP = torch.empty_like(dSA)
    assert G.plcp_device(dT, dSA, dP) == 0
    oP = oracle.plcp(T, oSA)
    assert np.array_equal(dP.cpu().numpy().astype(np.int64), oP)
    dL = torch.empty_like(dSA)
    assert G.lcp_device(dP, dSA, dL) == 0
    assert np.array_equal(dL.cpu().numpy().astype(np.int64), oracle.lcp(oP, oSA))


def test_stats_reported():
    T = textgen.periodic(1 << 16)
    rc, _, _ = G.libsais(T)
    s = G.last_stats()
    assert rc == 0 and s["rounds"] >= 1 and s["seed_symbols"] >= 8 and s["workspace_bytes"] > 0
