"""Generate the golden vectors in this directory from the reference libsais.

The reference (libsais 2.10.4) ships no test vectors, so the vectors are made
by running the reference itself, compiled from its own sources by
``make -C oracle ref`` into ``oracle/_ref/libsais_ref.so``.  Run from the
repository root where the reference source tree is present:

    python tests/golden/make_golden.py

Each case is stored as ``<name>.npz`` with the input text and every output of
the reference's construction entry points on it.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.oracle import Reference, build  # noqa: E402


def cases():
    rng = np.random.default_rng(20251203)
    dna = np.frombuffer(b"ACGT", dtype=np.uint8)
    yield "dna_iid_4096", dna[rng.integers(0, 4, 4096)], False
    yield "binary_2000", rng.integers(0, 2, 2000).astype(np.uint8), False
    yield "bytes_3000", rng.integers(0, 256, 3000).astype(np.uint8), False
    yield "all_a_1500", np.full(1500, ord("A"), dtype=np.uint8), False
    yield "period7_2100", np.frombuffer((b"ACGTACG" * 300), dtype=np.uint8).copy(), False
    yield "zeros_700", np.zeros(700, dtype=np.uint8), False
    # tandem repeat inside random text, plus a long copy
    t = dna[rng.integers(0, 4, 6000)]
    t[1000:1600] = np.tile(t[1000:1013], 47)[:600]
    t[4000:4800] = t[200:1000]
    yield "repeats_6000", t, False
    yield "tiny_banana", np.frombuffer(b"banana", dtype=np.uint8).copy(), False
    # generalized suffix array: 0-separated reads
    parts = []
    for _ in range(40):
        L = int(rng.integers(5, 40))
        parts.append(dna[rng.integers(0, 4, L)])
        parts.append(np.zeros(1, dtype=np.uint8))
    parts[6] = parts[2].copy()   # duplicated read
    yield "gsa_reads_40", np.concatenate(parts), True
    # 16-bit texts
    yield "u16_zipfish_3000", (rng.zipf(1.3, 3000) % 65535 + 1).astype(np.uint16), False
    yield "u16_small_alpha_2500", (rng.integers(0, 3, 2500) * 20000).astype(np.uint16), False


def main():
    build(with_reference=True)
    R = Reference()
    for name, T, gsa in cases():
        out = {"T": T, "gsa": np.array(gsa)}
        rc, SA, freq = R.libsais(T, gsa=gsa)
        assert rc == 0, (name, rc)
        out["SA"], out["freq"] = SA, freq
        if not gsa:
            p, U, _, _ = R.libsais_bwt(T)
            out["U"], out["primary"] = U, np.array(p)
            if T.dtype == np.uint8:
                a, Ua, I, _ = R.libsais_bwt(T, r=8)
                assert a == 0 and np.array_equal(Ua, U)
                out["I8"] = I
                rc64, SA64, _ = R.libsais64(T)
                assert rc64 == 0 and np.array_equal(SA64, SA.astype(np.int64))
        rc, P = R.plcp(T, SA, gsa=gsa)
        assert rc == 0
        rc, L = R.lcp(P, SA)
        assert rc == 0
        out["PLCP"], out["LCP"] = P, L
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print("wrote", name, T.size)


if __name__ == "__main__":
    main()
