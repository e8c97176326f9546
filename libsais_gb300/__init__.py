"""libsais_gb300 -- GB300 suffix-array construction behind the libsais C API.

The product is the shared library ``lib/libsais_gb300.so`` (CUDA kernels for
sm_103a + a C shim exporting libsais 2.10.4's construction entry points, see
``include/*.h``).  This module is a thin ctypes mirror of that C-ABI for
Python callers and tests: every function below calls exactly one exported C
symbol of the same name and returns what it returns, plus the output arrays.

There is no CPU fallback: if the shared library is missing or no GPU is
present, calls fail (``load()`` raises, or the C entry points return -2).
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from ._build import LIBDIR, MAIN_SO, TEXTGEN_SO, build

__all__ = [
    "load", "build", "Context",
    "libsais", "libsais_gsa", "libsais_omp", "libsais_bwt", "libsais_bwt_aux", "libsais_plcp", "libsais_plcp_gsa",
    "libsais_lcp", "libsais64", "libsais64_gsa", "libsais64_bwt", "libsais64_bwt_aux", "libsais64_plcp",
    "libsais64_plcp_gsa", "libsais64_lcp", "libsais16", "libsais16_gsa", "libsais16_bwt", "libsais16_bwt_aux",
    "libsais16_plcp", "libsais16_plcp_gsa", "libsais16_lcp", "sa_bwt", "sa_device", "sa_bwt_device",
    "plcp_device", "lcp_device", "last_stats", "set_seed_key_bits", "EXPORTED_SYMBOLS",
    "libsais_int", "libsais64_long", "libsais_plcp_int", "libsais_unbwt", "libsais_unbwt_aux", "libsais16_unbwt",
    "libsais16_unbwt_aux", "libsais64_unbwt", "libsais64_unbwt_aux", "libsais16x64", "libsais16x64_bwt",
    "libsais16x64_unbwt",
]

_p = ctypes.c_void_p
_i32 = ctypes.c_int32
_i64 = ctypes.c_int64

# name -> (restype, argtypes); the exact signatures of include/*.h
_SIGS = {
    "libsais_create_ctx": (_p, []),
    "libsais_create_ctx_omp": (_p, [_i32]),
    "libsais_free_ctx": (None, [_p]),
    "libsais": (_i32, [_p, _p, _i32, _i32, _p]),
    "libsais_gsa": (_i32, [_p, _p, _i32, _i32, _p]),
    "libsais_ctx": (_i32, [_p, _p, _p, _i32, _i32, _p]),
    "libsais_gsa_ctx": (_i32, [_p, _p, _p, _i32, _i32, _p]),
    "libsais_omp": (_i32, [_p, _p, _i32, _i32, _p, _i32]),
    "libsais_gsa_omp": (_i32, [_p, _p, _i32, _i32, _p, _i32]),
    "libsais_bwt": (_i32, [_p, _p, _p, _i32, _i32, _p]),
    "libsais_bwt_aux": (_i32, [_p, _p, _p, _i32, _i32, _p, _i32, _p]),
    "libsais_bwt_ctx": (_i32, [_p, _p, _p, _p, _i32, _i32, _p]),
    "libsais_bwt_aux_ctx": (_i32, [_p, _p, _p, _p, _i32, _i32, _p, _i32, _p]),
    "libsais_bwt_omp": (_i32, [_p, _p, _p, _i32, _i32, _p, _i32]),
    "libsais_bwt_aux_omp": (_i32, [_p, _p, _p, _i32, _i32, _p, _i32, _p, _i32]),
    "libsais_plcp": (_i32, [_p, _p, _p, _i32]),
    "libsais_plcp_gsa": (_i32, [_p, _p, _p, _i32]),
    "libsais_lcp": (_i32, [_p, _p, _p, _i32]),
    "libsais_plcp_omp": (_i32, [_p, _p, _p, _i32, _i32]),
    "libsais_plcp_gsa_omp": (_i32, [_p, _p, _p, _i32, _i32]),
    "libsais_lcp_omp": (_i32, [_p, _p, _p, _i32, _i32]),
    "libsais64": (_i64, [_p, _p, _i64, _i64, _p]),
    "libsais64_gsa": (_i64, [_p, _p, _i64, _i64, _p]),
    "libsais64_omp": (_i64, [_p, _p, _i64, _i64, _p, _i64]),
    "libsais64_gsa_omp": (_i64, [_p, _p, _i64, _i64, _p, _i64]),
    "libsais64_bwt": (_i64, [_p, _p, _p, _i64, _i64, _p]),
    "libsais64_bwt_aux": (_i64, [_p, _p, _p, _i64, _i64, _p, _i64, _p]),
    "libsais64_bwt_omp": (_i64, [_p, _p, _p, _i64, _i64, _p, _i64]),
    "libsais64_bwt_aux_omp": (_i64, [_p, _p, _p, _i64, _i64, _p, _i64, _p, _i64]),
    "libsais64_plcp": (_i64, [_p, _p, _p, _i64]),
    "libsais64_plcp_gsa": (_i64, [_p, _p, _p, _i64]),
    "libsais64_lcp": (_i64, [_p, _p, _p, _i64]),
    "libsais64_plcp_omp": (_i64, [_p, _p, _p, _i64, _i64]),
    "libsais64_plcp_gsa_omp": (_i64, [_p, _p, _p, _i64, _i64]),
    "libsais64_lcp_omp": (_i64, [_p, _p, _p, _i64, _i64]),
    "libsais16_create_ctx": (_p, []),
    "libsais16_create_ctx_omp": (_p, [_i32]),
    "libsais16_free_ctx": (None, [_p]),
    "libsais16": (_i32, [_p, _p, _i32, _i32, _p]),
    "libsais16_gsa": (_i32, [_p, _p, _i32, _i32, _p]),
    "libsais16_ctx": (_i32, [_p, _p, _p, _i32, _i32, _p]),
    "libsais16_gsa_ctx": (_i32, [_p, _p, _p, _i32, _i32, _p]),
    "libsais16_omp": (_i32, [_p, _p, _i32, _i32, _p, _i32]),
    "libsais16_gsa_omp": (_i32, [_p, _p, _i32, _i32, _p, _i32]),
    "libsais16_bwt": (_i32, [_p, _p, _p, _i32, _i32, _p]),
    "libsais16_bwt_aux": (_i32, [_p, _p, _p, _i32, _i32, _p, _i32, _p]),
    "libsais16_bwt_ctx": (_i32, [_p, _p, _p, _p, _i32, _i32, _p]),
    "libsais16_bwt_aux_ctx": (_i32, [_p, _p, _p, _p, _i32, _i32, _p, _i32, _p]),
    "libsais16_bwt_omp": (_i32, [_p, _p, _p, _i32, _i32, _p, _i32]),
    "libsais16_bwt_aux_omp": (_i32, [_p, _p, _p, _i32, _i32, _p, _i32, _p, _i32]),
    "libsais16_plcp": (_i32, [_p, _p, _p, _i32]),
    "libsais16_plcp_gsa": (_i32, [_p, _p, _p, _i32]),
    "libsais16_lcp": (_i32, [_p, _p, _p, _i32]),
    "libsais16_plcp_omp": (_i32, [_p, _p, _p, _i32, _i32]),
    "libsais16_plcp_gsa_omp": (_i32, [_p, _p, _p, _i32, _i32]),
    "libsais16_lcp_omp": (_i32, [_p, _p, _p, _i32, _i32]),
    "libsais_int": (_i32, [_p, _p, _i32, _i32, _i32]),
    "libsais_int_omp": (_i32, [_p, _p, _i32, _i32, _i32, _i32]),
    "libsais_plcp_int": (_i32, [_p, _p, _p, _i32]),
    "libsais_plcp_int_omp": (_i32, [_p, _p, _p, _i32, _i32]),
    "libsais16_int": (_i32, [_p, _p, _i32, _i32, _i32]),
    "libsais16_int_omp": (_i32, [_p, _p, _i32, _i32, _i32, _i32]),
    "libsais64_long": (_i64, [_p, _p, _i64, _i64, _i64]),
    "libsais64_long_omp": (_i64, [_p, _p, _i64, _i64, _i64, _i64]),
    "libsais_unbwt_create_ctx": (_p, []),
    "libsais_unbwt_create_ctx_omp": (_p, [_i32]),
    "libsais_unbwt_free_ctx": (None, [_p]),
    "libsais_unbwt": (_i32, [_p, _p, _p, _i32, _p, _i32]),
    "libsais_unbwt_ctx": (_i32, [_p, _p, _p, _p, _i32, _p, _i32]),
    "libsais_unbwt_aux": (_i32, [_p, _p, _p, _i32, _p, _i32, _p]),
    "libsais_unbwt_aux_ctx": (_i32, [_p, _p, _p, _p, _i32, _p, _i32, _p]),
    "libsais_unbwt_omp": (_i32, [_p, _p, _p, _i32, _p, _i32, _i32]),
    "libsais_unbwt_aux_omp": (_i32, [_p, _p, _p, _i32, _p, _i32, _p, _i32]),
    "libsais16_unbwt_create_ctx": (_p, []),
    "libsais16_unbwt_create_ctx_omp": (_p, [_i32]),
    "libsais16_unbwt_free_ctx": (None, [_p]),
    "libsais16_unbwt": (_i32, [_p, _p, _p, _i32, _p, _i32]),
    "libsais16_unbwt_ctx": (_i32, [_p, _p, _p, _p, _i32, _p, _i32]),
    "libsais16_unbwt_aux": (_i32, [_p, _p, _p, _i32, _p, _i32, _p]),
    "libsais16_unbwt_aux_ctx": (_i32, [_p, _p, _p, _p, _i32, _p, _i32, _p]),
    "libsais16_unbwt_omp": (_i32, [_p, _p, _p, _i32, _p, _i32, _i32]),
    "libsais16_unbwt_aux_omp": (_i32, [_p, _p, _p, _i32, _p, _i32, _p, _i32]),
    "libsais64_unbwt": (_i64, [_p, _p, _p, _i64, _p, _i64]),
    "libsais64_unbwt_aux": (_i64, [_p, _p, _p, _i64, _p, _i64, _p]),
    "libsais64_unbwt_omp": (_i64, [_p, _p, _p, _i64, _p, _i64, _i64]),
    "libsais64_unbwt_aux_omp": (_i64, [_p, _p, _p, _i64, _p, _i64, _p, _i64]),
    "libsais16x64": (_i64, [_p, _p, _i64, _i64, _p]),
    "libsais16x64_gsa": (_i64, [_p, _p, _i64, _i64, _p]),
    "libsais16x64_long": (_i64, [_p, _p, _i64, _i64, _i64]),
    "libsais16x64_omp": (_i64, [_p, _p, _i64, _i64, _p, _i64]),
    "libsais16x64_gsa_omp": (_i64, [_p, _p, _i64, _i64, _p, _i64]),
    "libsais16x64_long_omp": (_i64, [_p, _p, _i64, _i64, _i64, _i64]),
    "libsais16x64_bwt": (_i64, [_p, _p, _p, _i64, _i64, _p]),
    "libsais16x64_bwt_aux": (_i64, [_p, _p, _p, _i64, _i64, _p, _i64, _p]),
    "libsais16x64_bwt_omp": (_i64, [_p, _p, _p, _i64, _i64, _p, _i64]),
    "libsais16x64_bwt_aux_omp": (_i64, [_p, _p, _p, _i64, _i64, _p, _i64, _p, _i64]),
    "libsais16x64_unbwt": (_i64, [_p, _p, _p, _i64, _p, _i64]),
    "libsais16x64_unbwt_aux": (_i64, [_p, _p, _p, _i64, _p, _i64, _p]),
    "libsais16x64_unbwt_omp": (_i64, [_p, _p, _p, _i64, _p, _i64, _i64]),
    "libsais16x64_unbwt_aux_omp": (_i64, [_p, _p, _p, _i64, _p, _i64, _p, _i64]),
    "libsais16x64_plcp": (_i64, [_p, _p, _p, _i64]),
    "libsais16x64_plcp_gsa": (_i64, [_p, _p, _p, _i64]),
    "libsais16x64_lcp": (_i64, [_p, _p, _p, _i64]),
    "libsais16x64_plcp_omp": (_i64, [_p, _p, _p, _i64, _i64]),
    "libsais16x64_plcp_gsa_omp": (_i64, [_p, _p, _p, _i64, _i64]),
    "libsais16x64_lcp_omp": (_i64, [_p, _p, _p, _i64, _i64]),
    "gsais_sa_device": (_i64, [_p, _p, _i32, _i64, _i32, _p, _i32, _p]),
    "gsais_sa_bwt_device": (_i64, [_p, _p, _i32, _i64, _p, _i32, _p, _p]),
    "gsais_plcp_device": (_i64, [_p, _p, _i32, _p, _p, _i32, _i64, _i32, _p]),
    "gsais_lcp_device": (_i64, [_p, _p, _p, _p, _i32, _i64, _p]),
    "gsais_sa_bwt": (_i64, [_p, _p, _i32, _i64, _p, _i32, _p, _p, _i32]),
    "gsais_last_stats": (_i32, [_p, _p]),
    "gsais_set_seed_key_bits": (_i32, [_p, _i32]),
    "gsais_release_workspace": (None, [_p]),
    "gsais_profile_enable": (_i32, [_p, _i32]),
    "gsais_profile_read": (_i32, [_p, _p, _i32]),
    "gsais_profile_reset": (None, [_p]),
    "gsais_launch_count": (_i64, []),
    "gsais_sa_device_noalloc": (_i64, [_p, _i32, _i64, _i32, _p, _p]),
    "gsais_set_tuning": (_i32, [_p, _p]),
    "gsais_last_tuning": (_i32, [_p, _p]),
    "gsais_load_tuning_cache": (_i32, [ctypes.c_char_p]),
    "gsais_test_stall_radix_wait": (_i32, [_i64]),
    "gsais_test_fail_allocations": (_i32, [_i32]),
    "gsais_batch_sa_bwt": (_i64, [_p, _p, _p, _i32, _p, _p, _p]),
    "gsais_batch_sa_bwt_device": (_i64, [_p, _p, _i64, _p, _i32, _p, _p, _p, _p]),
    "gsais_batch_sa_bwt_sym_device": (_i64, [_p, _p, _i32, _i64, _p, _i32, _p, _p, _p, _p]),
    "gsais_server_create": (_p, [_i64, _i32, _i64, _i32]),
    "gsais_server_submit": (_i64, [_p, _p, _i32, _i64, _p, _p]),
    "gsais_server_wait": (_i32, [_p, _i64, _p, _p, _p, _p]),
    "gsais_server_get_stats": (_i32, [_p, _p]),
    "gsais_server_destroy": (None, [_p]),
}

EXPORTED_SYMBOLS = tuple(_SIGS)

_lib = None


class GsaisStats(ctypes.Structure):
    _fields_ = [("rounds", _i32), ("seed_symbols", _i32), ("seed_bits", _i32), ("radix_passes", _i32),
                ("active_total", _i64), ("workspace_bytes", _i64), ("large_total", _i64),
                ("pairs_direct", _i64), ("early_patch", _i64)]


class GsaisTuning(ctypes.Structure):
    _fields_ = [("digit_bits", _i32), ("radix_items32", _i32), ("radix_items64", _i32), ("medium_small", _i32),
                ("medium_max", _i32), ("large_few_others", _i32)]


TUNING_DEFAULTS = {"digit_bits": 8, "radix_items32": 20, "radix_items64": 16, "medium_small": 512,
                   "medium_max": 4096, "large_few_others": 1}


def set_tuning(tuning=None, ctx=None) -> int:
    """gsais_set_tuning: fix the sort's tuning on ctx (a dict of GsaisTuning
    fields, missing ones from TUNING_DEFAULTS), or None for cache/defaults."""
    lib = load()
    h = ctx.handle if ctx else None
    if tuning is None:
        return int(lib.gsais_set_tuning(h, None))
    t = GsaisTuning(**{**TUNING_DEFAULTS, **tuning})
    return int(lib.gsais_set_tuning(h, ctypes.byref(t)))


def last_tuning(ctx=None) -> dict:
    lib = load()
    t = GsaisTuning()
    lib.gsais_last_tuning(ctx.handle if ctx else None, ctypes.byref(t))
    return {k: getattr(t, k) for k, _ in GsaisTuning._fields_}


def load_tuning_cache(path=None) -> int:
    return int(load().gsais_load_tuning_cache(path.encode() if path else None))


class KernelProfile(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char_p), ("launches", _i64), ("total_ms", ctypes.c_double), ("bytes", _i64)]


def load(path: str = MAIN_SO):
    """Load the shared library (building it first if absent)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        build()
    lib = ctypes.CDLL(path)
    for name, (res, args) in _SIGS.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def _ptr(a) -> int:
    if a is None:
        return 0
    return a.ctypes.data


def _text(T):
    T = np.ascontiguousarray(T)
    if T.dtype not in (np.uint8, np.uint16):
        raise TypeError("text must be uint8 or uint16")
    return T


class Context:
    """libsais_create_ctx / libsais_free_ctx as a Python object."""

    def __init__(self, sixteen: bool = False):
        lib = load()
        self.handle = lib.libsais16_create_ctx() if sixteen else lib.libsais_create_ctx()
        if not self.handle:
            raise MemoryError("libsais_create_ctx failed")

    def close(self):
        if self.handle:
            load().libsais_free_ctx(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------------------ 32-bit index
def _sa_call(name, T, width, fs=0, freq=True, ctx=None, threads=None):
    lib = load()
    T = _text(T)
    n = T.size
    SA = np.zeros(max(n, 1) + fs, dtype=np.int32 if width == 4 else np.int64)
    F = np.zeros(256 if T.dtype == np.uint8 else 65536, dtype=SA.dtype) if freq else None
    f = getattr(lib, name)
    if ctx is not None:
        rc = f(ctx.handle, _ptr(T), _ptr(SA), n, fs, _ptr(F))
    elif threads is not None:
        rc = f(_ptr(T), _ptr(SA), n, fs, _ptr(F), threads)
    else:
        rc = f(_ptr(T), _ptr(SA), n, fs, _ptr(F))
    return int(rc), SA[:n], F


def libsais(T, fs=0, freq=True, ctx=None):
    return _sa_call("libsais_ctx" if ctx else "libsais", T, 4, fs, freq, ctx)


def libsais_omp(T, fs=0, freq=True, threads=0):
    return _sa_call("libsais_omp", T, 4, fs, freq, threads=threads)


def libsais_gsa(T, fs=0, freq=True, ctx=None):
    return _sa_call("libsais_gsa_ctx" if ctx else "libsais_gsa", T, 4, fs, freq, ctx)


def libsais16(T, fs=0, freq=True, ctx=None):
    return _sa_call("libsais16_ctx" if ctx else "libsais16", np.asarray(T, dtype=np.uint16), 4, fs, freq, ctx)


def libsais16_gsa(T, fs=0, freq=True, ctx=None):
    return _sa_call("libsais16_gsa_ctx" if ctx else "libsais16_gsa", np.asarray(T, dtype=np.uint16), 4, fs, freq,
                    ctx)


def libsais64(T, fs=0, freq=True):
    return _sa_call("libsais64", T, 8, fs, freq)


def libsais64_gsa(T, fs=0, freq=True):
    return _sa_call("libsais64_gsa", T, 8, fs, freq)


def _bwt_call(name, T, width, r=0, fs=0, freq=True, ctx=None, U=None):
    lib = load()
    T = _text(T)
    n = T.size
    if U is None:
        U = np.zeros(max(n, 1), dtype=T.dtype)
    A = np.zeros(max(n, 1) + fs, dtype=np.int32 if width == 4 else np.int64)
    F = np.zeros(256 if T.dtype == np.uint8 else 65536, dtype=A.dtype) if freq else None
    f = getattr(lib, name)
    args = [_ptr(T), _ptr(U), _ptr(A), n, fs, _ptr(F)]
    I = None
    if r:
        I = np.zeros((n - 1) // r + 1 if n else 1, dtype=A.dtype)
        args += [r, _ptr(I)]
    if ctx is not None:
        args = [ctx.handle] + args
    rc = f(*args)
    return int(rc), U[:n], I, F


def libsais_bwt(T, fs=0, freq=True, ctx=None):
    rc, U, _, F = _bwt_call("libsais_bwt_ctx" if ctx else "libsais_bwt", T, 4, 0, fs, freq, ctx)
    return rc, U, F


def libsais_bwt_aux(T, r, fs=0, freq=True, ctx=None):
    return _bwt_call("libsais_bwt_aux_ctx" if ctx else "libsais_bwt_aux", T, 4, r, fs, freq, ctx)


def libsais16_bwt(T, fs=0, freq=True, ctx=None):
    rc, U, _, F = _bwt_call("libsais16_bwt_ctx" if ctx else "libsais16_bwt", np.asarray(T, dtype=np.uint16), 4, 0, fs,
                            freq, ctx)
    return rc, U, F


def libsais16_bwt_aux(T, r, fs=0, freq=True, ctx=None):
    return _bwt_call("libsais16_bwt_aux_ctx" if ctx else "libsais16_bwt_aux", np.asarray(T, dtype=np.uint16), 4, r,
                     fs, freq, ctx)


def libsais64_bwt(T, fs=0, freq=True):
    rc, U, _, F = _bwt_call("libsais64_bwt", T, 8, 0, fs, freq)
    return rc, U, F


def libsais64_bwt_aux(T, r, fs=0, freq=True):
    return _bwt_call("libsais64_bwt_aux", T, 8, r, fs, freq)


# ------------------------------------------------------- integer alphabets
def libsais_int(T, k, fs=0, threads=None):
    """libsais_int (or libsais_int_omp): SA of an int32 string over [0, k)."""
    lib = load()
    T = np.ascontiguousarray(T, dtype=np.int32)
    SA = np.zeros(max(T.size, 1) + fs, dtype=np.int32)
    if threads is None:
        rc = lib.libsais_int(_ptr(T), _ptr(SA), T.size, k, fs)
    else:
        rc = lib.libsais_int_omp(_ptr(T), _ptr(SA), T.size, k, fs, threads)
    return int(rc), SA[: T.size]


def libsais64_long(T, k, fs=0, name="libsais64_long"):
    """libsais64_long (or libsais16x64_long): SA of an int64 string over [0, k)."""
    lib = load()
    T = np.ascontiguousarray(T, dtype=np.int64)
    SA = np.zeros(max(T.size, 1) + fs, dtype=np.int64)
    rc = getattr(lib, name)(_ptr(T), _ptr(SA), T.size, k, fs)
    return int(rc), SA[: T.size]


def libsais_plcp_int(T, SA):
    lib = load()
    T = np.ascontiguousarray(T, dtype=np.int32)
    SA = np.ascontiguousarray(SA, dtype=np.int32)
    P = np.zeros(max(T.size, 1), dtype=np.int32)
    rc = lib.libsais_plcp_int(_ptr(T), _ptr(SA), _ptr(P), T.size)
    return int(rc), P[: T.size]


# ------------------------------------------------------------- inverse BWT
def _unbwt_call(name, U, width, r, I, ctx=None, threads=None, out=None):
    lib = load()
    U = _text(U)
    n = U.size
    T = np.zeros(max(n, 1), dtype=U.dtype) if out is None else out
    A = np.zeros(n + 1, dtype=np.int32 if width == 4 else np.int64)
    f = getattr(lib, name)
    args = [_ptr(U), _ptr(T), _ptr(A), n, None]
    if r is None:
        args.append(I)   # the primary index
    else:
        I = np.ascontiguousarray(I, dtype=A.dtype)
        args += [r, _ptr(I)]
    if threads is not None:
        args.append(threads)
    if ctx is not None:
        args = [ctx.handle] + args
    rc = f(*args)
    return int(rc), T[:n]


def libsais_unbwt(U, primary, ctx=None, threads=None, out=None):
    name = "libsais_unbwt_ctx" if ctx else ("libsais_unbwt_omp" if threads is not None else "libsais_unbwt")
    return _unbwt_call(name, np.asarray(U, dtype=np.uint8), 4, None, primary, ctx, threads, out)


def libsais_unbwt_aux(U, r, I, ctx=None):
    return _unbwt_call("libsais_unbwt_aux_ctx" if ctx else "libsais_unbwt_aux", np.asarray(U, dtype=np.uint8), 4, r,
                       I, ctx)


def libsais16_unbwt(U, primary, ctx=None):
    return _unbwt_call("libsais16_unbwt_ctx" if ctx else "libsais16_unbwt", np.asarray(U, dtype=np.uint16), 4, None,
                       primary, ctx)


def libsais16_unbwt_aux(U, r, I):
    return _unbwt_call("libsais16_unbwt_aux", np.asarray(U, dtype=np.uint16), 4, r, I)


def libsais64_unbwt(U, primary):
    return _unbwt_call("libsais64_unbwt", np.asarray(U, dtype=np.uint8), 8, None, primary)


def libsais64_unbwt_aux(U, r, I):
    return _unbwt_call("libsais64_unbwt_aux", np.asarray(U, dtype=np.uint8), 8, r, I)


# ----------------------------------------------- 16-bit symbols, int64 index
def libsais16x64(T, fs=0, freq=True, gsa=False):
    return _sa_call("libsais16x64_gsa" if gsa else "libsais16x64", np.asarray(T, dtype=np.uint16), 8, fs, freq)


def libsais16x64_bwt(T, r=0, fs=0, freq=True):
    if r:
        return _bwt_call("libsais16x64_bwt_aux", np.asarray(T, dtype=np.uint16), 8, r, fs, freq)
    rc, U, _, F = _bwt_call("libsais16x64_bwt", np.asarray(T, dtype=np.uint16), 8, 0, fs, freq)
    return rc, U, F


def libsais16x64_unbwt(U, primary):
    return _unbwt_call("libsais16x64_unbwt", np.asarray(U, dtype=np.uint16), 8, None, primary)


def _plcp_call(name, T, SA, width):
    lib = load()
    T = _text(T)
    SA = np.ascontiguousarray(SA, dtype=np.int32 if width == 4 else np.int64)
    P = np.zeros(max(T.size, 1), dtype=SA.dtype)
    rc = getattr(lib, name)(_ptr(T), _ptr(SA), _ptr(P), T.size)
    return int(rc), P[: T.size]


def libsais_plcp(T, SA):
    return _plcp_call("libsais_plcp", T, SA, 4)


def libsais_plcp_gsa(T, SA):
    return _plcp_call("libsais_plcp_gsa", T, SA, 4)


def libsais16_plcp(T, SA):
    return _plcp_call("libsais16_plcp", np.asarray(T, dtype=np.uint16), SA, 4)


def libsais16_plcp_gsa(T, SA):
    return _plcp_call("libsais16_plcp_gsa", np.asarray(T, dtype=np.uint16), SA, 4)


def libsais64_plcp(T, SA):
    return _plcp_call("libsais64_plcp", T, SA, 8)


def libsais64_plcp_gsa(T, SA):
    return _plcp_call("libsais64_plcp_gsa", T, SA, 8)


def _lcp_call(name, PLCP, SA, width, out=None):
    lib = load()
    dt = np.int32 if width == 4 else np.int64
    PLCP = np.ascontiguousarray(PLCP, dtype=dt)
    SA = np.ascontiguousarray(SA, dtype=dt)
    L = out if out is not None else np.zeros(max(SA.size, 1), dtype=dt)
    rc = getattr(lib, name)(_ptr(PLCP), _ptr(SA), _ptr(L), SA.size)
    return int(rc), L[: SA.size]


def libsais_lcp(PLCP, SA, out=None):
    return _lcp_call("libsais_lcp", PLCP, SA, 4, out)


def libsais16_lcp(PLCP, SA, out=None):
    return _lcp_call("libsais16_lcp", PLCP, SA, 4, out)


def libsais64_lcp(PLCP, SA, out=None):
    return _lcp_call("libsais64_lcp", PLCP, SA, 8, out)


# ------------------------------------------------------------ extensions
def sa_bwt(T, width=4, freq=True, ctx=None):
    """SA and BWT of a host text with one sort: (primary or rc, SA, U, freq)."""
    lib = load()
    T = _text(T)
    n = T.size
    SA = np.zeros(max(n, 1), dtype=np.int32 if width == 4 else np.int64)
    U = np.zeros(max(n, 1), dtype=T.dtype)
    F = np.zeros(256 if T.dtype == np.uint8 else 65536, dtype=SA.dtype) if freq else None
    rc = lib.gsais_sa_bwt(ctx.handle if ctx else None, _ptr(T), T.itemsize, n, _ptr(SA), width, _ptr(U), _ptr(F),
                          width)
    return int(rc), SA[:n], U[:n], F


_CUDA_STREAM_LEGACY = 1   # cudaStreamLegacy


def _stream_handle(stream):
    """None: the context's own stream.  A torch stream (or a raw handle): that
    stream; torch's default stream has handle 0, which the C entry points
    read as "the context's stream", so it is passed as cudaStreamLegacy to
    keep the call ordered after the work already queued there."""
    if stream is None:
        return None
    h = getattr(stream, "cuda_stream", stream)
    return _CUDA_STREAM_LEGACY if h == 0 and hasattr(stream, "cuda_stream") else h


def sa_device(T, SA, gsa=False, ctx=None, stream=None):
    """Device-resident SA (torch tensors: T uint8/int16-as-uint16, SA int32/int64)."""
    lib = load()
    return int(lib.gsais_sa_device(ctx.handle if ctx else None, T.data_ptr(), T.element_size(), T.numel(), int(gsa),
                                   SA.data_ptr(), SA.element_size(), _stream_handle(stream)))


def sa_bwt_device(T, SA, U, ctx=None, stream=None):
    lib = load()
    return int(lib.gsais_sa_bwt_device(ctx.handle if ctx else None, T.data_ptr(), T.element_size(), T.numel(),
                                       SA.data_ptr() if SA is not None else None,
                                       SA.element_size() if SA is not None else 4, U.data_ptr(),
                                       _stream_handle(stream)))


def plcp_device(T, SA, PLCP, gsa=False, ctx=None, stream=None):
    lib = load()
    return int(lib.gsais_plcp_device(ctx.handle if ctx else None, T.data_ptr(), T.element_size(), SA.data_ptr(),
                                     PLCP.data_ptr(), SA.element_size(), T.numel(), int(gsa),
                                     _stream_handle(stream)))


def lcp_device(PLCP, SA, LCP, ctx=None, stream=None):
    lib = load()
    return int(lib.gsais_lcp_device(ctx.handle if ctx else None, PLCP.data_ptr(), SA.data_ptr(), LCP.data_ptr(),
                                    SA.element_size(), SA.numel(), _stream_handle(stream)))


def last_stats(ctx=None) -> dict:
    lib = load()
    s = GsaisStats()
    lib.gsais_last_stats(ctx.handle if ctx else None, ctypes.byref(s))
    return {k: getattr(s, k) for k, _ in GsaisStats._fields_}


def set_seed_key_bits(bits: int, ctx=None) -> int:
    return int(load().gsais_set_seed_key_bits(ctx.handle if ctx else None, bits))


def profile_enable(on: bool = True, ctx=None) -> bool:
    return bool(load().gsais_profile_enable(ctx.handle if ctx else None, int(on)))


def profile_reset(ctx=None) -> None:
    load().gsais_profile_reset(ctx.handle if ctx else None)


def profile_read(ctx=None) -> dict:
    """{kernel: {"launches", "total_ms", "bytes"}} accumulated while profiling was on."""
    recs = (KernelProfile * 16)()
    k = load().gsais_profile_read(ctx.handle if ctx else None, recs, 16)
    return {recs[i].name.decode(): {"launches": recs[i].launches, "total_ms": recs[i].total_ms,
                                     "bytes": recs[i].bytes} for i in range(max(k, 0))}


def launch_count() -> int:
    return int(load().gsais_launch_count())


def batch_sa_bwt(T, offsets, ctx=None):
    """Batched SA + BWT of the strings T[offsets[s]:offsets[s+1]] (host arrays).

    Returns (rc, SA, U, primary) in the concatenated layout."""
    lib = load()
    T = np.ascontiguousarray(T, dtype=np.uint8)
    offsets = np.ascontiguousarray(offsets, dtype=np.int64)
    count = offsets.size - 1
    n = int(offsets[-1])
    SA = np.zeros(max(n, 1), dtype=np.int32)
    U = np.zeros(max(n, 1), dtype=np.uint8)
    P = np.zeros(max(count, 1), dtype=np.int32)
    rc = lib.gsais_batch_sa_bwt(ctx.handle if ctx else None, _ptr(T), _ptr(offsets), count, _ptr(SA), _ptr(U),
                                _ptr(P))
    return int(rc), SA[:n], U[:n], P[:count]


def batch_sa_bwt_device(T, offsets, SA, U, primary, ctx=None, stream=None):
    """Device variant: torch tensors T (uint8), offsets (int64, count + 1), SA (int32), U (uint8), primary (int32)."""
    lib = load()
    count = offsets.numel() - 1
    return int(lib.gsais_batch_sa_bwt_device(ctx.handle if ctx else None, T.data_ptr(), T.numel(),
                                             offsets.data_ptr(), count, SA.data_ptr(), U.data_ptr(),
                                             primary.data_ptr(), _stream_handle(stream)))


def batch_sa_bwt_sym_device(T, offsets, SA, U, primary, symbytes=1, ctx=None, stream=None):
    """gsais_batch_sa_bwt_sym_device: T and U hold 8-bit (symbytes 1, uint8 tensors) or
    16-bit symbols (symbytes 2, int16 tensors viewed as uint16)."""
    lib = load()
    count = offsets.numel() - 1
    return int(lib.gsais_batch_sa_bwt_sym_device(ctx.handle if ctx else None, T.data_ptr(), symbytes, T.numel(),
                                                 offsets.data_ptr(), count, SA.data_ptr(), U.data_ptr(),
                                                 primary.data_ptr(), _stream_handle(stream)))


def release_workspace(ctx=None) -> None:
    """Free the device workspace cached by a context (the process-wide one by default)."""
    load().gsais_release_workspace(ctx.handle if ctx else None)


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", _i64), ("completed", _i64), ("rejected", _i64), ("batches", _i64),
                ("batched_jobs", _i64), ("symbols_done", _i64), ("hbm_high_water_bytes", _i64),
                ("hbm_budget_bytes", _i64), ("busy_seconds", ctypes.c_double),
                ("footprint_bytes_per_symbol", ctypes.c_double)]


class Server:
    """gsais_server_*: SA+BWT request loop with continuous batching."""

    def __init__(self, hbm_budget_bytes: int, workers: int = 2, small_job_symbols: int = 1 << 20,
                 max_batch: int = 256):
        self.lib = load()
        self.handle = self.lib.gsais_server_create(hbm_budget_bytes, workers, small_job_symbols, max_batch)
        if not self.handle:
            raise MemoryError("gsais_server_create failed")
        self._keep = {}

    def submit(self, T):
        T = _text(T)
        n = T.size
        SA = np.empty(n, dtype=np.int32)
        U = np.empty(n, dtype=T.dtype)
        jid = int(self.lib.gsais_server_submit(self.handle, _ptr(T), T.itemsize, n, _ptr(SA), _ptr(U)))
        if jid > 0:
            self._keep[jid] = (T, SA, U)
        return jid

    def submit_into(self, T, SA, U):
        """Submits T with caller-owned output arrays (SA int32 and U of T's dtype,
        at least T.size long; pinned host memory lets the copies run as DMA)."""
        T = _text(T)
        n = T.size
        if SA.dtype != np.int32 or SA.size < n or U.dtype != T.dtype or U.size < n:
            raise ValueError("SA must be int32 and U of the text's dtype, each at least n long")
        jid = int(self.lib.gsais_server_submit(self.handle, _ptr(T), T.itemsize, n, _ptr(SA), _ptr(U)))
        if jid > 0:
            self._keep[jid] = (T, SA[:n], U[:n])
        return jid

    def wait(self, jid: int):
        """(result, SA, U, queued_s, total_s, batched)"""
        res = ctypes.c_int64()
        q = ctypes.c_double()
        t = ctypes.c_double()
        b = ctypes.c_int32()
        rc = self.lib.gsais_server_wait(self.handle, jid, ctypes.byref(res), ctypes.byref(q), ctypes.byref(t),
                                        ctypes.byref(b))
        if rc != 0:
            raise KeyError(jid)
        T, SA, U = self._keep.pop(jid)
        return int(res.value), SA, U, q.value, t.value, b.value

    def stats(self) -> dict:
        s = ServerStats()
        self.lib.gsais_server_get_stats(self.handle, ctypes.byref(s))
        return {k: getattr(s, k) for k, _ in ServerStats._fields_}

    def close(self):
        if self.handle:
            self.lib.gsais_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
