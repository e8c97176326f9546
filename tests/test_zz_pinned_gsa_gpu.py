"""GSA construction into pinned host memory (the early SA copy of the
generalized suffix array), checked against the oracle through the C-ABI."""
import numpy as np
import pytest

import libsais_gb300 as G

pytestmark = pytest.mark.gpu


def test_pinned_gsa_early_copy(oracle):
    """libsais_gsa into a pinned SA buffer: the early copy and its patch on a
    0-separated set of byte strings, some of them repeated (their suffixes are
    what the doubling rounds still sort)."""
    torch = pytest.importorskip("torch")
    lib = G.load()
    rng = np.random.default_rng(29)
    strings = [rng.integers(1, 200, int(rng.integers(100, 800))).astype(np.uint8) for _ in range(2_000)]
    strings += [strings[int(i)] for i in rng.integers(0, len(strings), 60)]
    T = np.concatenate([np.append(s_, np.uint8(0)) for s_ in strings])
    n = T.size
    _, oSA, _ = oracle.libsais(T, gsa=True)
    hT = torch.from_numpy(T).pin_memory()
    hSA = torch.full((n,), -7, dtype=torch.int32).pin_memory()
    assert lib.libsais_gsa(hT.data_ptr(), hSA.data_ptr(), n, 0, None) == 0
    assert np.array_equal(hSA.numpy().astype(np.int64), oSA)
    # about 6 % of the suffixes (those of the repeated strings) are left for
    # the rounds, under the n / 8 limit of an early copy
    assert G.last_stats()["early_patch"] > 0
