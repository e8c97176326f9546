"""Failure paths, exercised without faulting the GPU.

* A bounded device wait that runs out: a test hook makes every full tile of
  the radix digit pass wait (after its staging copies have landed) on a
  barrier that nothing arrives on, with a 1 ms limit.  The wait gives up, the
  kernel raises its error bit and stages the tile again with plain loads, and
  the call returns -2 (the reference's code for an internal failure,
  src/libsais.c:6930-6932).  With the hook off, the next call on the same
  context succeeds and matches the oracle: the context stays usable.
* A failed workspace allocation (host-side hook in front of cudaMalloc): the
  call returns -2, and the next call allocates and succeeds.
"""
import numpy as np
import pytest

import libsais_gb300 as G
from libsais_gb300 import textgen

pytestmark = pytest.mark.gpu


def test_radix_wait_timeout_returns_minus_two_and_context_recovers(oracle):
    lib = G.load()
    T = textgen.genome_like(200_000, seed=31)   # many full radix tiles
    _, oSA = oracle.sa(T)
    try:
        assert lib.gsais_test_stall_radix_wait(1_000_000) == 0   # 1 ms
        rc, SA, _ = G.libsais(T)
        assert rc == -2
    finally:
        assert lib.gsais_test_stall_radix_wait(0) == 0
    rc, SA, _ = G.libsais(T)
    assert rc == 0
    assert np.array_equal(SA.astype(np.int64), oSA)


def test_stall_hook_rejects_out_of_range_limits():
    lib = G.load()
    assert lib.gsais_test_stall_radix_wait(-1) == -1
    assert lib.gsais_test_stall_radix_wait(2_000_000_000) == -1


def test_failed_allocation_returns_minus_two(oracle):
    lib = G.load()
    T = textgen.iid(50_000, seed=32)
    _, oSA = oracle.sa(T)
    G.release_workspace()   # the next call must allocate its workspace
    try:
        assert lib.gsais_test_fail_allocations(1) == 0
        rc, _, _ = G.libsais(T)
        assert rc == -2
        prim, _, _ = G.libsais_bwt(T)   # the hook is spent: this call allocates
        assert prim > 0
    finally:
        lib.gsais_test_fail_allocations(0)
    rc, SA, _ = G.libsais(T)
    assert rc == 0 and np.array_equal(SA.astype(np.int64), oSA)
