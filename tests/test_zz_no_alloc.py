"""The allocation-free entry point gsais_sa_device_noalloc.

It serves callers that cannot call cudaMalloc (CUDA graph capture, a
framework allocator that owns all device memory, latency-critical paths):
the suffix sort takes all of its scratch from a fixed 6 MiB __device__
array, for texts of at most 65,536 symbols.  This test calls it through the
C-ABI twice in a row on each input and compares its output with the existing
allocating entry point gsais_sa_device; suffix arrays are integers, so the
tolerance is zero.  The file name sorts last so that a run that stops at the
first failure has already run every other test.
"""
import numpy as np
import pytest

import libsais_gb300 as G
from libsais_gb300 import textgen

pytestmark = pytest.mark.gpu

MAX_N = 65536


def inputs():
    rng = np.random.default_rng(99)
    yield textgen.genome_like(MAX_N, seed=21), False
    yield textgen.periodic(50_000), False
    yield (rng.integers(0, 256, 40_000)).astype(np.uint8), False
    yield textgen.zipf_u16(30_000, seed=22), False
    yield textgen.reads_gsa(200, ref_len=20_000, seed=23)[:MAX_N], True
    yield np.frombuffer(b"banana", dtype=np.uint8).copy(), False


def test_no_alloc_matches_allocating_entry_point():
    torch = pytest.importorskip("torch")
    lib = G.load()
    stream = torch.cuda.current_stream()
    for T, gsa in inputs():
        if gsa:
            T = T[: int(np.flatnonzero(T == 0)[-1]) + 1]   # keep it 0-terminated
        n = T.size
        dT = torch.from_numpy(T.view(np.int16) if T.dtype == np.uint16 else T).cuda()
        expect = torch.empty(n, dtype=torch.int32, device="cuda")
        assert G.sa_device(dT, expect, gsa=gsa, stream=stream) == 0
        for _ in range(2):   # two calls in a row share the static scratch
            got = torch.full((n,), -7, dtype=torch.int32, device="cuda")
            rc = lib.gsais_sa_device_noalloc(dT.data_ptr(), T.itemsize, n, int(gsa), got.data_ptr(),
                                             stream.cuda_stream)
            torch.cuda.synchronize()
            assert rc == 0
            assert torch.equal(got, expect)


def test_no_alloc_rejects_oversized_text():
    torch = pytest.importorskip("torch")
    lib = G.load()
    dT = torch.zeros(MAX_N + 1, dtype=torch.uint8, device="cuda")
    dSA = torch.empty(MAX_N + 1, dtype=torch.int32, device="cuda")
    assert lib.gsais_sa_device_noalloc(dT.data_ptr(), 1, MAX_N + 1, 0, dSA.data_ptr(), None) == -1
