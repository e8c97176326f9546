"""The allocation-free entry point gsais_sa_device_noalloc.

It serves callers that cannot call cudaMalloc: a plugin running inside an
application whose caching allocator owns the device's memory (there
cudaMalloc can fail on memory that allocator holds, and can synchronise the
device under the application's other streams), and latency-critical paths.
The suffix sort takes all of its scratch from a fixed 6 MiB __device__ array,
for texts of at most 65,536 symbols.

The test calls it through the C-ABI twice in a row on each input and compares
its output with the existing allocating entry point gsais_sa_device; suffix
arrays are integers, so the tolerance is zero.  It also checks that a call
leaves the device's free memory unchanged (after a first call on the same
input has loaded the kernels it uses), that a malformed generalized text is
rejected with -1 and that an oversized text is rejected with -1.  The file
name sorts last so that a run that stops at the first failure has already
run every other test.
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


def device_text(torch, T):
    return torch.from_numpy(T.view(np.int16) if T.dtype == np.uint16 else T).cuda()


def test_no_alloc_matches_allocating_entry_point():
    torch = pytest.importorskip("torch")
    lib = G.load()
    stream = torch.cuda.current_stream()
    for T, gsa in inputs():
        if gsa:
            T = T[: int(np.flatnonzero(T == 0)[-1]) + 1]   # keep it 0-terminated
        n = T.size
        dT = device_text(torch, T)
        expect = torch.empty(n, dtype=torch.int32, device="cuda")
        assert G.sa_device(dT, expect, gsa=gsa, stream=stream) == 0
        outs = [torch.full((n,), -7, dtype=torch.int32, device="cuda") for _ in range(2)]
        torch.cuda.synchronize()
        for k, got in enumerate(outs):   # two calls in a row share the static scratch
            free0 = torch.cuda.mem_get_info()[0]
            rc = lib.gsais_sa_device_noalloc(dT.data_ptr(), T.itemsize, n, int(gsa), got.data_ptr(),
                                             stream.cuda_stream)
            torch.cuda.synchronize()
            assert rc == 0
            assert torch.equal(got, expect)
            if k == 1:   # the first call on this input may load kernels; the second allocates nothing
                assert torch.cuda.mem_get_info()[0] == free0, "the call allocated device memory"


def test_no_alloc_rejects_malformed_gsa_text():
    torch = pytest.importorskip("torch")
    lib = G.load()
    T = np.array([1, 0, 0, 2, 0], dtype=np.uint8)   # an empty string between two separators
    dT = device_text(torch, T)
    dSA = torch.empty(T.size, dtype=torch.int32, device="cuda")
    rc = lib.gsais_sa_device_noalloc(dT.data_ptr(), 1, T.size, 1, dSA.data_ptr(), None)
    torch.cuda.synchronize()
    assert rc == -1


def test_no_alloc_rejects_oversized_text():
    torch = pytest.importorskip("torch")
    lib = G.load()
    dT = torch.zeros(MAX_N + 1, dtype=torch.uint8, device="cuda")
    dSA = torch.empty(MAX_N + 1, dtype=torch.int32, device="cuda")
    assert lib.gsais_sa_device_noalloc(dT.data_ptr(), 1, MAX_N + 1, 0, dSA.data_ptr(), None) == -1
