"""CPU oracle for libsais's construction outputs -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg may
import this module, and only as the checker; the libsais_gb300 product never
touches it.

Two back ends, same Python shapes:

* ``Oracle`` wraps ``liboracle.so``, the C restatement in ``oracle.c``
  (SA-IS written from the published algorithm; BWT, aux indexes, Phi-PLCP and
  LCP following libsais src/libsais.c:6960-7146 and :8116-8338).
* ``Reference`` wraps ``_ref/libsais_ref.so``, the reference library compiled
  from its own sources by ``make -C oracle ref`` (only where the reference
  source tree exists).

Each method mirrors one libsais entry point and returns numpy arrays plus the
entry point's integer return value.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libsais_ref.so")

_p = ctypes.c_void_p
_i64 = ctypes.c_int64
_i32 = ctypes.c_int32


ROOT = os.path.dirname(HERE)
STAGED_REF = os.path.join(ROOT, "baseline", "_ref")


def reference_dir() -> str:
    """Source tree the reference is compiled from: $LIBSAIS_REFERENCE_DIR, else
    the staged copy under baseline/_ref (made by ``make -C oracle stage``)."""
    return os.environ.get("LIBSAIS_REFERENCE_DIR") or STAGED_REF


def build(with_reference: bool = True) -> None:
    """Compile liboracle.so (and the reference, when its sources are present).

    Without $LIBSAIS_REFERENCE_DIR and without a staged copy, the Makefile's
    ``stage`` recipe is tried first; where no reference source tree exists it
    fails quietly and only liboracle.so is built."""
    targets = ["all"]
    ref_dir = reference_dir()
    if with_reference and not os.environ.get("LIBSAIS_REFERENCE_DIR") and \
            not os.path.isdir(os.path.join(ref_dir, "src")):
        subprocess.run(["make", "-s", "-C", HERE, "stage"], stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    if with_reference and os.path.isdir(os.path.join(ref_dir, "src")):
        targets.append("ref")
    jobs = str(max(4, min(8, os.cpu_count() or 4)))
    subprocess.run(["make", "-s", "-C", HERE, "-j" + jobs, f"REF={ref_dir}"] + targets, check=True)


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data if a is not None else 0


def _symbytes(T: np.ndarray) -> int:
    if T.dtype == np.uint8:
        return 1
    if T.dtype == np.uint16:
        return 2
    if T.dtype == np.int32:
        return 4
    raise TypeError("text must be uint8, uint16 or int32")


class Oracle:
    """The C restatement.  All index outputs are int64 arrays."""

    def __init__(self, path: str = ORACLE_SO):
        if not os.path.exists(path):
            build(with_reference=False)
        lib = ctypes.CDLL(path)
        lib.oracle_sa.argtypes = [_p, ctypes.c_int, _p, _i64, ctypes.c_int]
        lib.oracle_sa.restype = ctypes.c_int
        lib.oracle_sa_int.argtypes = [_p, _p, _i64, _i64]
        lib.oracle_sa_int.restype = ctypes.c_int
        lib.oracle_gsa_valid.argtypes = [_p, ctypes.c_int, _i64]
        lib.oracle_gsa_valid.restype = ctypes.c_int
        lib.oracle_freq.argtypes = [_p, ctypes.c_int, _i64, _p]
        lib.oracle_freq.restype = None
        lib.oracle_bwt.argtypes = [_p, ctypes.c_int, _p, _i64, _p, _i64, _p]
        lib.oracle_bwt.restype = _i64
        lib.oracle_plcp.argtypes = [_p, ctypes.c_int, _p, _p, _i64, ctypes.c_int]
        lib.oracle_plcp.restype = None
        lib.oracle_lcp.argtypes = [_p, _p, _p, _i64]
        lib.oracle_lcp.restype = None
        lib.oracle_check_sa.argtypes = [_p, ctypes.c_int, _p, _i64, ctypes.c_int]
        lib.oracle_check_sa.restype = ctypes.c_int
        lib.oracle_unbwt.argtypes = [_p, ctypes.c_int, _i64, _i64, _p]
        lib.oracle_unbwt.restype = ctypes.c_int
        self.lib = lib

    # -- primitives -----------------------------------------------------
    def sa(self, T: np.ndarray, gsa: bool = False):
        T = np.ascontiguousarray(T)
        n = T.size
        SA = np.empty(max(n, 1), dtype=np.int64)[:n]
        rc = self.lib.oracle_sa(_ptr(T), _symbytes(T), _ptr(SA), n, int(gsa))
        return rc, SA

    def sa_int(self, T: np.ndarray, k: int):
        T = np.ascontiguousarray(T, dtype=np.int32)
        SA = np.empty(max(T.size, 1), dtype=np.int64)[: T.size]
        rc = self.lib.oracle_sa_int(_ptr(T), _ptr(SA), T.size, k)
        return rc, SA

    def sa_int_any(self, T: np.ndarray):
        """SA of an integer string with arbitrary non-negative values: the values
        are first replaced by their ranks (same order, so the same SA)."""
        T = np.asarray(T)
        vals, codes = np.unique(T, return_inverse=True)
        return self.sa_int(codes.astype(np.int32), max(int(vals.size), 1))

    def gsa_valid(self, T: np.ndarray) -> bool:
        T = np.ascontiguousarray(T)
        return bool(self.lib.oracle_gsa_valid(_ptr(T), _symbytes(T), T.size))

    def freq(self, T: np.ndarray) -> np.ndarray:
        T = np.ascontiguousarray(T)
        f = np.zeros(256 if T.dtype == np.uint8 else 65536, dtype=np.int64)
        self.lib.oracle_freq(_ptr(T), _symbytes(T), T.size, _ptr(f))
        return f

    def bwt_from_sa(self, T: np.ndarray, SA: np.ndarray, r: int = 0):
        T = np.ascontiguousarray(T)
        SA = np.ascontiguousarray(SA, dtype=np.int64)
        n = T.size
        U = np.empty_like(T)
        I = np.zeros((n - 1) // r + 1 if (r and n) else 1, dtype=np.int64)
        primary = self.lib.oracle_bwt(_ptr(T), _symbytes(T), _ptr(SA), n, _ptr(U), r, _ptr(I) if r else 0)
        return int(primary), U, I

    def plcp(self, T: np.ndarray, SA: np.ndarray, gsa: bool = False) -> np.ndarray:
        T = np.ascontiguousarray(T)
        SA = np.ascontiguousarray(SA, dtype=np.int64)
        P = np.empty(max(T.size, 1), dtype=np.int64)[: T.size]
        self.lib.oracle_plcp(_ptr(T), _symbytes(T), _ptr(SA), _ptr(P), T.size, int(gsa))
        return P

    def unbwt(self, U: np.ndarray, primary: int):
        """(rc, T) from a BWT in libsais_bwt layout and its primary index."""
        U = np.ascontiguousarray(U)
        T = np.empty_like(U)
        rc = self.lib.oracle_unbwt(_ptr(U), _symbytes(U), U.size, primary, _ptr(T))
        return rc, T

    def lcp(self, PLCP: np.ndarray, SA: np.ndarray) -> np.ndarray:
        PLCP = np.ascontiguousarray(PLCP, dtype=np.int64)
        SA = np.ascontiguousarray(SA, dtype=np.int64)
        L = np.empty_like(SA)
        self.lib.oracle_lcp(_ptr(PLCP), _ptr(SA), _ptr(L), SA.size)
        return L

    def check_sa(self, T: np.ndarray, SA: np.ndarray, gsa: bool = False) -> bool:
        T = np.ascontiguousarray(T)
        SA = np.ascontiguousarray(SA, dtype=np.int64)
        return self.lib.oracle_check_sa(_ptr(T), _symbytes(T), _ptr(SA), T.size, int(gsa)) == 1

    # -- libsais-shaped compositions ---------------------------------------
    def libsais(self, T: np.ndarray, gsa: bool = False):
        """(rc, SA, freq) as libsais()/libsais_gsa()/libsais16() would return."""
        T = np.ascontiguousarray(T)
        if gsa and (T.size == 0 or T[-1] != 0):
            return -1, None, None
        if T.size <= 1:
            return 0, np.zeros(T.size, dtype=np.int64), self.freq(T)
        rc, SA = self.sa(T, gsa)
        return rc, SA, self.freq(T)

    def libsais_bwt(self, T: np.ndarray, r: int = 0):
        """(primary or rc, U, I, freq) as libsais_bwt()/libsais_bwt_aux() would return."""
        T = np.ascontiguousarray(T)
        n = T.size
        if n <= 1:
            I = np.array([n], dtype=np.int64)
            return (0 if r else n), T.copy(), I, self.freq(T)
        rc, SA = self.sa(T)
        if rc != 0:
            return rc, None, None, None
        primary, U, I = self.bwt_from_sa(T, SA, r)
        return (0 if r else primary), U, I, self.freq(T)


class Reference:
    """The reference libsais compiled from its own sources (oracle/_ref)."""

    def __init__(self, path: str = REF_SO):
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        lib = ctypes.CDLL(path)
        for name in ("libsais", "libsais_gsa"):
            f = getattr(lib, name)
            f.argtypes = [_p, _p, _i32, _i32, _p]
            f.restype = _i32
        for name in ("libsais_omp", "libsais_gsa_omp"):
            f = getattr(lib, name)
            f.argtypes = [_p, _p, _i32, _i32, _p, _i32]
            f.restype = _i32
        for name in ("libsais16", "libsais16_gsa"):
            f = getattr(lib, name)
            f.argtypes = [_p, _p, _i32, _i32, _p]
            f.restype = _i32
        for name in ("libsais64", "libsais64_gsa"):
            f = getattr(lib, name)
            f.argtypes = [_p, _p, _i64, _i64, _p]
            f.restype = _i64
        lib.libsais_bwt.argtypes = [_p, _p, _p, _i32, _i32, _p]
        lib.libsais_bwt.restype = _i32
        lib.libsais_bwt_omp.argtypes = [_p, _p, _p, _i32, _i32, _p, _i32]
        lib.libsais_bwt_omp.restype = _i32
        lib.libsais16_bwt.argtypes = [_p, _p, _p, _i32, _i32, _p]
        lib.libsais16_bwt.restype = _i32
        lib.libsais64_bwt.argtypes = [_p, _p, _p, _i64, _i64, _p]
        lib.libsais64_bwt.restype = _i64
        lib.libsais_bwt_aux.argtypes = [_p, _p, _p, _i32, _i32, _p, _i32, _p]
        lib.libsais_bwt_aux.restype = _i32
        for name in ("libsais_plcp", "libsais_plcp_gsa", "libsais16_plcp", "libsais16_plcp_gsa"):
            f = getattr(lib, name)
            f.argtypes = [_p, _p, _p, _i32]
            f.restype = _i32
        lib.libsais_lcp.argtypes = [_p, _p, _p, _i32]
        lib.libsais_lcp.restype = _i32
        for name in ("libsais64_plcp", "libsais64_plcp_gsa"):
            f = getattr(lib, name)
            f.argtypes = [_p, _p, _p, _i64]
            f.restype = _i64
        lib.libsais64_lcp.argtypes = [_p, _p, _p, _i64]
        lib.libsais64_lcp.restype = _i64
        lib.libsais_int.argtypes = [_p, _p, _i32, _i32, _i32]
        lib.libsais_int.restype = _i32
        lib.libsais_plcp_int.argtypes = [_p, _p, _p, _i32]
        lib.libsais_plcp_int.restype = _i32
        lib.libsais_unbwt.argtypes = [_p, _p, _p, _i32, _p, _i32]
        lib.libsais_unbwt.restype = _i32
        lib.libsais16_unbwt.argtypes = [_p, _p, _p, _i32, _p, _i32]
        lib.libsais16_unbwt.restype = _i32
        self.lib = lib

    def libsais_int(self, T: np.ndarray, k: int):
        """libsais_int on a copy of T (the reference permutes T while it works)."""
        T = np.array(T, dtype=np.int32)
        SA = np.empty(max(T.size, 1), dtype=np.int32)
        rc = self.lib.libsais_int(_ptr(T), _ptr(SA), T.size, k, 0)
        return int(rc), SA[: T.size]

    def plcp_int(self, T: np.ndarray, SA: np.ndarray):
        T = np.ascontiguousarray(T, dtype=np.int32)
        SA = np.ascontiguousarray(SA, dtype=np.int32)
        P = np.empty(max(T.size, 1), dtype=np.int32)
        rc = self.lib.libsais_plcp_int(_ptr(T), _ptr(SA), _ptr(P), T.size)
        return int(rc), P[: T.size]

    def unbwt(self, U: np.ndarray, primary: int):
        U = np.ascontiguousarray(U)
        n = U.size
        T = np.empty(max(n, 1), dtype=U.dtype)
        A = np.empty(n + 1, dtype=np.int32)
        f = self.lib.libsais16_unbwt if U.dtype == np.uint16 else self.lib.libsais_unbwt
        rc = f(_ptr(U), _ptr(T), _ptr(A), n, None, primary)
        return int(rc), T[:n]

    def libsais(self, T: np.ndarray, gsa: bool = False, threads: int = 1):
        T = np.ascontiguousarray(T)
        n = T.size
        SA = np.empty(max(n, 1), dtype=np.int32)
        if T.dtype == np.uint16:
            freq = np.zeros(65536, dtype=np.int32)
            f = self.lib.libsais16_gsa if gsa else self.lib.libsais16
            rc = f(_ptr(T), _ptr(SA), n, 0, _ptr(freq))
        else:
            freq = np.zeros(256, dtype=np.int32)
            if threads == 1:
                f = self.lib.libsais_gsa if gsa else self.lib.libsais
                rc = f(_ptr(T), _ptr(SA), n, 0, _ptr(freq))
            else:
                f = self.lib.libsais_gsa_omp if gsa else self.lib.libsais_omp
                rc = f(_ptr(T), _ptr(SA), n, 0, _ptr(freq), threads)
        return int(rc), SA[:n], freq

    def libsais64(self, T: np.ndarray, gsa: bool = False):
        T = np.ascontiguousarray(T, dtype=np.uint8)
        n = T.size
        SA = np.empty(max(n, 1), dtype=np.int64)
        freq = np.zeros(256, dtype=np.int64)
        f = self.lib.libsais64_gsa if gsa else self.lib.libsais64
        rc = f(_ptr(T), _ptr(SA), n, 0, _ptr(freq))
        return int(rc), SA[:n], freq

    def libsais_bwt(self, T: np.ndarray, r: int = 0, threads: int = 1):
        T = np.ascontiguousarray(T)
        n = T.size
        U = np.empty(max(n, 1), dtype=T.dtype)
        A = np.empty(max(n, 1), dtype=np.int32)
        if T.dtype == np.uint16:
            freq = np.zeros(65536, dtype=np.int32)
            rc = self.lib.libsais16_bwt(_ptr(T), _ptr(U), _ptr(A), n, 0, _ptr(freq))
            return int(rc), U[:n], None, freq
        freq = np.zeros(256, dtype=np.int32)
        if r:
            I = np.zeros((n - 1) // r + 1 if n else 1, dtype=np.int32)
            rc = self.lib.libsais_bwt_aux(_ptr(T), _ptr(U), _ptr(A), n, 0, _ptr(freq), r, _ptr(I))
            return int(rc), U[:n], I, freq
        if threads == 1:
            rc = self.lib.libsais_bwt(_ptr(T), _ptr(U), _ptr(A), n, 0, _ptr(freq))
        else:
            rc = self.lib.libsais_bwt_omp(_ptr(T), _ptr(U), _ptr(A), n, 0, _ptr(freq), threads)
        return int(rc), U[:n], None, freq

    def libsais64_bwt(self, T: np.ndarray):
        T = np.ascontiguousarray(T, dtype=np.uint8)
        n = T.size
        U = np.empty(max(n, 1), dtype=np.uint8)
        A = np.empty(max(n, 1), dtype=np.int64)
        freq = np.zeros(256, dtype=np.int64)
        rc = self.lib.libsais64_bwt(_ptr(T), _ptr(U), _ptr(A), n, 0, _ptr(freq))
        return int(rc), U[:n], freq

    def plcp(self, T: np.ndarray, SA: np.ndarray, gsa: bool = False):
        T = np.ascontiguousarray(T)
        n = T.size
        SA = np.ascontiguousarray(SA, dtype=np.int32)
        P = np.empty(max(n, 1), dtype=np.int32)
        if T.dtype == np.uint16:
            f = self.lib.libsais16_plcp_gsa if gsa else self.lib.libsais16_plcp
        else:
            f = self.lib.libsais_plcp_gsa if gsa else self.lib.libsais_plcp
        rc = f(_ptr(T), _ptr(SA), _ptr(P), n)
        return int(rc), P[:n]

    def lcp(self, PLCP: np.ndarray, SA: np.ndarray):
        PLCP = np.ascontiguousarray(PLCP, dtype=np.int32)
        SA = np.ascontiguousarray(SA, dtype=np.int32)
        L = np.empty(max(SA.size, 1), dtype=np.int32)
        rc = self.lib.libsais_lcp(_ptr(PLCP), _ptr(SA), _ptr(L), SA.size)
        return int(rc), L[: SA.size]
