"""Full-size property checks of the long-input workloads.

* The 64-bit index path on a 3 GiB order-2 Markov ACGT text (n = 3 * 2^30 > 2^31):
  the int64 SA must pass the oracle's linear-time suffix-array check
  (permutation + inverse-rank neighbour rule) and the BWT and primary index
  must equal the ones derived from that SA.
* The 2^28 genome-like text (the benchmark text): SA check + BWT from SA.

These need about 260 GB of device memory and ~50 GB of host memory; they are
skipped where that is not available.
"""
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


def test_genome_like_2_28(oracle):
    torch = pytest.importorskip("torch")
    T = textgen.genome_like(1 << 28, seed=2)
    dT = torch.from_numpy(T).cuda()
    dSA = torch.empty(T.size, dtype=torch.int32, device="cuda")
    dU = torch.empty(T.size, dtype=torch.uint8, device="cuda")
    prim = G.sa_bwt_device(dT, dSA, dU)
    assert prim > 0
    check_sa_bwt(oracle, T, dSA, dU, prim)


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
