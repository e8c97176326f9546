"""In-tree build of the libsais_gb300 shared libraries.

* ``lib/libsais_gb300.so`` -- CUDA kernels for sm_103a plus the libsais C API
  shim; exports the symbols declared in ``include/*.h``.
* ``lib/libtextgen.so``    -- seeded synthetic text generators (host C).

Each translation unit is compiled in parallel; a unit is rebuilt only when a
source or header is newer than its object file.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "lib")
OBJDIR = os.path.join(LIBDIR, "obj")
INCLUDE = os.path.join(ROOT, "include")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I" + CSRC, "-I" + INCLUDE]
CC_FLAGS = ["-O2", "-fPIC", "-std=c99", "-Wall", "-I" + CSRC, "-I" + INCLUDE]

MAIN_SO = os.path.join(LIBDIR, "libsais_gb300.so")
TEXTGEN_SO = os.path.join(LIBDIR, "libtextgen.so")


def _newest(paths):
    return max((os.path.getmtime(p) for p in paths if os.path.exists(p)), default=0.0)


def _headers():
    return glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(
        os.path.join(INCLUDE, "*.h"))


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r


def _compile(src: str, hdr_time: float, extra_flags=()):
    obj = os.path.join(OBJDIR, os.path.basename(src) + ".o")
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(src), hdr_time):
        return obj
    if src.endswith(".cu"):
        cmd = [NVCC] + NVCC_FLAGS + list(extra_flags) + ["-c", src, "-o", obj]
    else:
        cmd = ["gcc"] + CC_FLAGS + ["-c", src, "-o", obj]
    _run(cmd)
    return obj


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    """Compile every translation unit and link the shared libraries."""
    os.makedirs(OBJDIR, exist_ok=True)
    hdr_time = _newest(_headers())
    cu = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    cs = [os.path.join(CSRC, "api.c")]
    extra = ["-Xptxas", "-v"] if ptxas_info else []
    with cf.ThreadPoolExecutor(max_workers=max(4, len(cu) + len(cs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, hdr_time, extra), cu + cs))
    if not os.path.exists(MAIN_SO) or os.path.getmtime(MAIN_SO) < _newest(objs):
        tmp = MAIN_SO + ".tmp"
        _run([NVCC] + ARCH + ["-shared", "-o", tmp] + objs + ["-lpthread"])
        os.replace(tmp, MAIN_SO)
    tg = os.path.join(CSRC, "textgen.c")
    if not os.path.exists(TEXTGEN_SO) or os.path.getmtime(TEXTGEN_SO) < os.path.getmtime(tg):
        _run(["gcc", "-O2", "-fPIC", "-shared", "-std=c99", tg, "-o", TEXTGEN_SO, "-lm"])
    if verbose:
        print("built", MAIN_SO)
    return MAIN_SO


def clean() -> None:
    shutil.rmtree(LIBDIR, ignore_errors=True)


if __name__ == "__main__":
    build(verbose=True)
