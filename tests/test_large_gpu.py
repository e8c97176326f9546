"""Full-size checks of the workloads the benchmark is quoted on.

* The 2^28 genome-like text (the benchmark text): the SA passes the oracle's
  linear-time suffix-array check (permutation + inverse-rank neighbour rule),
  the BWT and primary index equal the ones derived from that SA, and PLCP and
  LCP equal the oracle's (Phi / Kasai, src/libsais.c:8116-8190, :8311-8338).
* The degenerate texts at n = 2^26 (all 'A', and period 7, the worst case for
  the number of doubling rounds): SA check, BWT + primary, PLCP, LCP.
* The batched workload in full: 4096 strings of log-uniform length
  256 B - 4 MiB (1.76 G symbols) sorted in one batched call; every string's SA
  passes the SA check and its BWT and primary index equal the oracle's.
* The 64-bit index path on a 3 GiB order-2 Markov ACGT text (n = 3 * 2^30 > 2^31):
  SA check + BWT from SA.

The 3 GiB case needs about 260 GB of device memory and ~60 GB of host memory
and is skipped where that is not available.
"""
import concurrent.futures as cf
import os

import numpy as np
import pytest

import libsais_gb300 as G
from libsais_gb300 import textgen

pytestmark = [pytest.mark.gpu, pytest.mark.slow]


def host_free_bytes():
    try:
        with open("/proc/meminfo") as f:
            for line in f:
                if line.startswith("MemAvailable:"):
                    return int(line.split()[1]) * 1024
    except OSError:
        pass
    return 0


def check_sa_bwt(oracle, T, dSA, dU, prim):
    SA = dSA.cpu().numpy().astype(np.int64, copy=False)
    assert oracle.check_sa(T, SA), "suffix array check failed"
    p, U, _ = oracle.bwt_from_sa(T, SA)
    assert prim == p
    assert np.array_equal(dU.cpu().numpy(), U)


def check_plcp_lcp(oracle, T, dT, dSA):
    torch = pytest.importorskip("torch")
    dP = torch.empty_like(dSA)
    dL = torch.empty_like(dSA)
    assert G.plcp_device(dT, dSA, dP) == 0
    assert G.lcp_device(dP, dSA, dL) == 0
    SA = dSA.cpu().numpy().astype(np.int64)
    oP = oracle.plcp(T, SA)
    assert np.array_equal(dP.cpu().numpy().astype(np.int64), oP), "PLCP differs from the oracle"
    assert np.array_equal(dL.cpu().numpy().astype(np.int64), oracle.lcp(oP, SA)), "LCP differs from the oracle"


def run_full(oracle, T):
    torch = pytest.importorskip("torch")
    dT = torch.from_numpy(T).cuda()
    dSA = torch.empty(T.size, dtype=torch.int32, device="cuda")
    dU = torch.empty(T.size, dtype=torch.uint8, device="cuda")
    prim = G.sa_bwt_device(dT, dSA, dU)
    assert prim > 0
    check_sa_bwt(oracle, T, dSA, dU, prim)
    check_plcp_lcp(oracle, T, dT, dSA)
    del dT, dSA, dU
    G.release_workspace()
    torch.cuda.empty_cache()


def test_genome_like_2_28(oracle):
    run_full(oracle, textgen.genome_like(1 << 28, seed=2))


@pytest.mark.parametrize("kind", ["all_A", "period7"])
def test_degenerate_2_26(oracle, kind):
    n = 1 << 26
    run_full(oracle, textgen.constant(n) if kind == "all_A" else textgen.periodic(n))


def test_batched_4096_strings_full(oracle):
    """Every string of the 4096-string batch, checked against the oracle."""
    torch = pytest.importorskip("torch")
    count = 4096
    T, offs = textgen.batch_strings(count, seed=3)
    n = int(offs[-1])
    dT = torch.from_numpy(T).cuda()
    dO = torch.from_numpy(offs).cuda()
    dSA = torch.empty(n, dtype=torch.int32, device="cuda")
    dU = torch.empty(n, dtype=torch.uint8, device="cuda")
    dP = torch.empty(count, dtype=torch.int32, device="cuda")
    assert G.batch_sa_bwt_device(dT, dO, dSA, dU, dP) == 0
    SA, U, P = dSA.cpu().numpy(), dU.cpu().numpy(), dP.cpu().numpy()
    del dT, dO, dSA, dU, dP
    G.release_workspace()
    torch.cuda.empty_cache()

    def check(s):
        a, b = int(offs[s]), int(offs[s + 1])
        t, sa = T[a:b], SA[a:b].astype(np.int64)
        if not oracle.check_sa(t, sa):
            return f"string {s}: SA check failed"
        p, u, _ = oracle.bwt_from_sa(t, sa)
        if p != int(P[s]) or not np.array_equal(u, U[a:b]):
            return f"string {s}: BWT or primary index differs"
        return None

    # the oracle's C calls release the GIL, so threads check strings in parallel
    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 1)) as ex:
        bad = [r for r in ex.map(check, range(count)) if r]
    assert not bad, bad[:5]


def test_libsais64_3gib(oracle):
    torch = pytest.importorskip("torch")
    n = 3 << 30
    free_dev, total_dev = torch.cuda.mem_get_info()
    if free_dev < 262e9 or host_free_bytes() < 60e9:
        pytest.skip("needs ~262 GB of free device memory and ~60 GB of host memory")
    G.release_workspace()
    torch.cuda.empty_cache()
    T = textgen.markov2_dna(n, seed=5)
    dT = torch.from_numpy(T).cuda()
    dSA = torch.empty(n, dtype=torch.int64, device="cuda")
    dU = torch.empty(n, dtype=torch.uint8, device="cuda")
    prim = G.sa_bwt_device(dT, dSA, dU)
    stats = G.last_stats()
    G.release_workspace()
    del dT
    torch.cuda.empty_cache()
    assert prim > 0, prim
    assert stats["seed_symbols"] == 16
    check_sa_bwt(oracle, T, dSA, dU, prim)
