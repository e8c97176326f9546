"""Seeded synthetic texts for the suffix-sorting workloads (wraps lib/libtextgen.so).

The public corpora timed by libsais's Benchmarks.md are not available, so the
workloads use these generators with the same shapes and value distributions:
i.i.d. DNA, a repetitive genome-like text (order-2 Markov DNA with segmental
duplications and tandem repeats), degenerate texts, short-read sets for the
generalized suffix array and Zipf-distributed 16-bit texts.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from ._build import TEXTGEN_SO, build

_u64 = ctypes.c_uint64
_p = ctypes.c_void_p
_d = ctypes.c_double
_tg = None
_tg_path = None   # None: lib/libtextgen.so


def set_library(path=None) -> None:
    """Load the generators from another build of textgen.c (None: the package's
    lib/libtextgen.so).  The CPU-only reference timing uses the oracle's copy, so
    that it loads no library of this package."""
    global _tg, _tg_path
    _tg, _tg_path = None, path

ACGT = np.frombuffer(b"ACGT", dtype=np.uint8)


def _lib():
    global _tg
    if _tg is None:
        path = _tg_path or TEXTGEN_SO
        if _tg_path is None and not os.path.exists(TEXTGEN_SO):
            build()
        lib = ctypes.CDLL(path)
        lib.tg_iid_u8.argtypes = [_p, _u64, _p, ctypes.c_int, _u64]
        lib.tg_dna_with_n.argtypes = [_p, _u64, _d, _u64]
        lib.tg_constant.argtypes = [_p, _u64, ctypes.c_uint8]
        lib.tg_periodic.argtypes = [_p, _u64, _p, _u64]
        lib.tg_markov2_dna.argtypes = [_p, _u64, _d, _u64]
        lib.tg_genome_like.argtypes = [_p, _u64, _d, _d, _u64]
        lib.tg_loguniform_lengths.argtypes = [_p, _u64, _d, _d, _u64]
        lib.tg_reads_gsa.argtypes = [_p, _u64, _u64, _u64, _u64]
        lib.tg_reads_gsa.restype = _u64
        lib.tg_zipf_u16.argtypes = [_p, _u64, _d, ctypes.c_uint32, _u64]
        lib.tg_zipf_u16.restype = ctypes.c_int
        lib.tg_poisson_arrivals.argtypes = [_p, _u64, _d, _u64]
        lib.tg_uniform.argtypes = [_p, _u64, _u64]
        _tg = lib
    return _tg


def iid(n: int, alphabet=ACGT, seed: int = 1) -> np.ndarray:
    """i.i.d. symbols drawn uniformly from `alphabet` (bytes)."""
    a = np.ascontiguousarray(np.asarray(alphabet, dtype=np.uint8))
    out = np.empty(n, dtype=np.uint8)
    _lib().tg_iid_u8(out.ctypes.data, n, a.ctypes.data, a.size, seed)
    return out


def dna_with_n(n: int, n_frac: float = 0.01, seed: int = 3) -> np.ndarray:
    out = np.empty(n, dtype=np.uint8)
    _lib().tg_dna_with_n(out.ctypes.data, n, n_frac, seed)
    return out


def constant(n: int, c: int = ord("A")) -> np.ndarray:
    out = np.empty(n, dtype=np.uint8)
    _lib().tg_constant(out.ctypes.data, n, c)
    return out


def periodic(n: int, pattern: bytes = b"ACGTACG") -> np.ndarray:
    p = np.frombuffer(pattern, dtype=np.uint8).copy()
    out = np.empty(n, dtype=np.uint8)
    _lib().tg_periodic(out.ctypes.data, n, p.ctypes.data, p.size)
    return out


def markov2_dna(n: int, gc: float = 0.41, seed: int = 5) -> np.ndarray:
    out = np.empty(n, dtype=np.uint8)
    _lib().tg_markov2_dna(out.ctypes.data, n, gc, seed)
    return out


def genome_like(n: int, dup_frac: float = 0.05, tandem_frac: float = 0.01, seed: int = 2) -> np.ndarray:
    """Order-2 Markov DNA (GC 0.41) + segmental duplications + tandem repeats."""
    out = np.empty(n, dtype=np.uint8)
    _lib().tg_genome_like(out.ctypes.data, n, dup_frac, tandem_frac, seed)
    return out


def loguniform_lengths(count: int, lo: float, hi: float, seed: int) -> np.ndarray:
    out = np.empty(count, dtype=np.uint64)
    _lib().tg_loguniform_lengths(out.ctypes.data, count, lo, hi, seed)
    return out


def reads_gsa(nreads: int, ref_len: int = 4_000_000, seed: int = 4) -> np.ndarray:
    """0-terminated short reads (length ~ N(150, 20) clipped to [50, 300])."""
    cap = nreads * 302 + 16
    out = np.empty(cap, dtype=np.uint8)
    n = _lib().tg_reads_gsa(out.ctypes.data, cap, nreads, ref_len, seed)
    return out[:n].copy()


def zipf_u16(n: int, s: float = 1.1, kmax: int = 65535, seed: int = 6) -> np.ndarray:
    out = np.empty(n, dtype=np.uint16)
    if _lib().tg_zipf_u16(out.ctypes.data, n, s, kmax, seed) != 0:
        raise MemoryError("zipf table")
    return out


def poisson_arrivals(count: int, rate: float, seed: int) -> np.ndarray:
    out = np.empty(count, dtype=np.float64)
    _lib().tg_poisson_arrivals(out.ctypes.data, count, rate, seed)
    return out


def uniform(count: int, seed: int) -> np.ndarray:
    out = np.empty(count, dtype=np.float64)
    _lib().tg_uniform(out.ctypes.data, count, seed)
    return out


def batch_strings(count: int = 4096, lo: float = 256, hi: float = 4 << 20, n_frac: float = 0.01, seed: int = 3):
    """The batched workload: `count` strings, log-uniform lengths, ACGT with 1% 'N'."""
    lens = loguniform_lengths(count, lo, hi, seed)
    total = int(lens.sum())
    buf = dna_with_n(total, n_frac, seed + 1000)
    offs = np.zeros(count + 1, dtype=np.int64)
    offs[1:] = np.cumsum(lens.astype(np.int64))
    return buf, offs
