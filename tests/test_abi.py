"""The C-ABI library: it builds, loads, exports every entry point the public
headers declare, and its host-side argument handling (reference checks and
n <= 1 cases, none of which reach the GPU) matches libsais."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")


def declared_symbols():
    names = set()
    for h in os.listdir(INCLUDE):
        src = open(os.path.join(INCLUDE, h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"\b(?:LIBSAIS(?:16|64)?_API\s+)?(?:void|int32_t|int64_t)\s*\*?\s*(\w+)\s*\(", src):
            names.add(m.group(1))
    return sorted(names)


def test_headers_declare_the_api():
    names = declared_symbols()
    for must in ("libsais", "libsais_bwt", "libsais_gsa", "libsais_plcp", "libsais_lcp", "libsais64", "libsais16",
                 "libsais_bwt_aux", "libsais_create_ctx", "gsais_sa_device"):
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    so = lib._name
    out = subprocess.run(["nm", "-D", "--defined-only", so], capture_output=True, text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = [s for s in declared_symbols() if s not in exported]
    assert not missing, missing
    for s in declared_symbols():
        assert hasattr(lib, s)


def test_python_mirror_covers_headers():
    import libsais_gb300
    assert set(declared_symbols()) <= set(libsais_gb300.EXPORTED_SYMBOLS)


def test_header_compiles_as_c():
    src = ("#include <libsais.h>\n#include <libsais64.h>\n#include <libsais16.h>\n#include <libsais16x64.h>\n"
           "#include <libsais_gb300.h>\nint main(void){return 0;}\n")
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", INCLUDE, "-x", "c", "-", "-o", "/dev/null"],
                       input=src, text=True, capture_output=True)
    assert r.returncode == 0, r.stderr


# ---- host-side paths (no GPU involved) -----------------------------------

def test_invalid_arguments_return_minus_one(lib):
    T = np.frombuffer(b"banana", dtype=np.uint8).copy()
    SA = np.zeros(6, np.int32)
    U = np.zeros(6, np.uint8)
    I = np.zeros(6, np.int32)
    p = lambda a: a.ctypes.data
    assert lib.libsais(None, p(SA), 6, 0, None) == -1
    assert lib.libsais(p(T), None, 6, 0, None) == -1
    assert lib.libsais(p(T), p(SA), -1, 0, None) == -1
    assert lib.libsais(p(T), p(SA), 6, -1, None) == -1
    assert lib.libsais_omp(p(T), p(SA), 6, 0, None, -1) == -1
    assert lib.libsais_ctx(None, p(T), p(SA), 6, 0, None) == -1
    assert lib.libsais_gsa(p(T), p(SA), 6, 0, None) == -1            # not 0-terminated
    assert lib.libsais_bwt(p(T), p(U), None, 6, 0, None) == -1
    assert lib.libsais_bwt_aux(p(T), p(U), p(SA), 6, 0, None, 3, p(I)) == -1    # r not a power of two
    assert lib.libsais_bwt_aux(p(T), p(U), p(SA), 6, 0, None, 1, p(I)) == -1    # r < 2
    assert lib.libsais_bwt_aux(p(T), p(U), p(SA), 6, 0, None, 4, None) == -1
    assert lib.libsais_plcp(p(T), None, p(SA), 6) == -1
    assert lib.libsais_plcp_gsa(p(T), p(SA), p(I), 6) == -1          # not 0-terminated
    assert lib.libsais_lcp(None, p(SA), p(I), 6) == -1
    assert lib.libsais64(None, None, 5, 0, None) == -1
    assert lib.libsais16(None, None, 5, 0, None) == -1
    assert lib.libsais_create_ctx_omp(-1) is None


def test_trivial_lengths(lib):
    p = lambda a: a.ctypes.data
    T = np.array([7], np.uint8)
    SA = np.full(2, 99, np.int32)
    F = np.full(256, 5, np.int32)
    assert lib.libsais(p(T), p(SA), 1, 0, p(F)) == 0
    assert SA[0] == 0 and F[7] == 1 and F.sum() == 1
    assert lib.libsais(p(T), p(SA), 0, 0, p(F)) == 0 and F.sum() == 0
    U = np.zeros(1, np.uint8)
    A = np.zeros(1, np.int32)
    assert lib.libsais_bwt(p(T), p(U), p(A), 1, 0, None) == 1 and U[0] == 7
    assert lib.libsais_bwt(p(T), p(U), p(A), 0, 0, None) == 0
    I = np.full(1, -5, np.int32)
    assert lib.libsais_bwt_aux(p(T), p(U), p(A), 1, 0, None, 4, p(I)) == 0 and I[0] == 1
    P = np.full(1, 9, np.int32)
    assert lib.libsais_plcp(p(T), p(SA), p(P), 1) == 0 and P[0] == 0
    L = np.full(1, 9, np.int32)
    P[0] = 3
    SA[0] = 0
    assert lib.libsais_lcp(p(P), p(SA), p(L), 1) == 0 and L[0] == 3
    G = np.array([0], np.uint8)
    assert lib.libsais_gsa(p(G), p(SA), 1, 0, None) == 0 and SA[0] == 0
    assert lib.libsais_gsa(p(T), p(SA), 1, 0, None) == -1
    S64 = np.full(1, 9, np.int64)
    F64 = np.zeros(256, np.int64)
    assert lib.libsais64(p(T), p(S64), 1, 0, p(F64)) == 0 and S64[0] == 0 and F64[7] == 1
    T16 = np.array([40000], np.uint16)
    F16 = np.zeros(65536, np.int32)
    assert lib.libsais16(p(T16), p(SA), 1, 0, p(F16)) == 0 and F16[40000] == 1


def test_contexts_create_and_free(lib):
    c = lib.libsais_create_ctx()
    assert c
    lib.libsais_free_ctx(c)
    lib.libsais_free_ctx(None)
    c16 = lib.libsais16_create_ctx_omp(0)
    assert c16
    lib.libsais16_free_ctx(c16)


def test_new_families_host_checks(lib):
    """Integer alphabets, inverse BWT and 16x64: the reference's argument checks
    and n <= 1 cases (src/libsais.c:7050, :8040, :8399; src/libsais64.c:7118,
    :8039; src/libsais16x64.c:7036, :7789), all answered on the host."""
    p = lambda a: a.ctypes.data
    Ti = np.array([3, 1, 2], np.int32)
    SA = np.full(4, 77, np.int32)
    assert lib.libsais_int(None, p(SA), 3, 4, 0) == -1
    assert lib.libsais_int(p(Ti), p(SA), -1, 4, 0) == -1
    assert lib.libsais_int(p(Ti), p(SA), 3, 4, -1) == -1
    assert lib.libsais_int_omp(p(Ti), p(SA), 3, 4, 0, -1) == -1
    assert lib.libsais_int(p(Ti), p(SA), 1, 4, 0) == 0 and SA[0] == 0
    assert lib.libsais16_int(p(Ti), p(SA), 0, 4, 0) == 0
    S64 = np.full(2, 5, np.int64)
    T64 = np.array([9], np.int64)
    assert lib.libsais64_long(p(T64), p(S64), 1, 10, 0) == 0 and S64[0] == 0
    assert lib.libsais64_long(p(T64), None, 1, 10, 0) == -1
    assert lib.libsais16x64_long_omp(p(T64), p(S64), 1, 10, 0, -2) == -1
    P = np.full(2, 9, np.int32)
    assert lib.libsais_plcp_int(p(Ti), p(SA), p(P), 1) == 0 and P[0] == 0
    assert lib.libsais_plcp_int(p(Ti), None, p(P), 3) == -1
    # inverse BWT
    U = np.array([65, 66, 67, 68], np.uint8)
    O = np.zeros(4, np.uint8)
    A = np.zeros(5, np.int32)
    I = np.array([2, 3], np.int32)
    assert lib.libsais_unbwt(p(U), p(O), None, 4, None, 1) == -1            # A NULL
    assert lib.libsais_unbwt(p(U), p(O), p(A), 4, None, 0) == -1            # primary <= 0
    assert lib.libsais_unbwt(p(U), p(O), p(A), 4, None, 5) == -1            # primary > n
    assert lib.libsais_unbwt_aux(p(U), p(O), p(A), 4, None, 3, p(I)) == -1  # r not a power of two
    assert lib.libsais_unbwt_aux(p(U), p(O), p(A), 4, None, 2, None) == -1
    bad = np.array([2, 0], np.int32)
    assert lib.libsais_unbwt_aux(p(U), p(O), p(A), 4, None, 2, p(bad)) == -1
    assert lib.libsais_unbwt_omp(p(U), p(O), p(A), 4, None, 1, -1) == -1
    assert lib.libsais_unbwt(p(U), p(O), p(A), 1, None, 1) == 0 and O[0] == 65
    assert lib.libsais_unbwt(p(U), p(O), p(A), 1, None, 0) == -1            # n = 1 needs primary 1
    assert lib.libsais_unbwt(p(U), p(O), p(A), 0, None, 0) == 0
    c = lib.libsais_unbwt_create_ctx()
    assert c
    assert lib.libsais_unbwt_ctx(c, p(U), p(O), p(A), 4, None, 7) == -1
    lib.libsais_unbwt_free_ctx(c)
    assert lib.libsais_unbwt_create_ctx_omp(-1) is None
    A64 = np.zeros(5, np.int64)
    assert lib.libsais64_unbwt(p(U), p(O), p(A64), 4, None, 9) == -1
    U16 = np.array([500], np.uint16)
    O16 = np.zeros(1, np.uint16)
    assert lib.libsais16x64_unbwt(p(U16), p(O16), p(A64), 1, None, 1) == 0 and O16[0] == 500
    S16 = np.full(1, 3, np.int64)
    F = np.zeros(65536, np.int64)
    assert lib.libsais16x64(p(U16), p(S16), 1, 0, p(F)) == 0 and S16[0] == 0 and F[500] == 1


def test_python_structs_match_the_header(tmp_path):
    """The ctypes mirrors of the header's structs have the C layout: every
    field's offset and the struct size, as gcc lays them out."""
    import libsais_gb300 as G
    mirrors = {"gsais_stats": G.GsaisStats, "gsais_kernel_profile": G.KernelProfile,
               "gsais_server_stats": G.ServerStats}
    lines = ["#include <stdio.h>", "#include <stddef.h>", "#include <libsais_gb300.h>", "int main(void){"]
    for cname, py in mirrors.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines.append("return 0;}")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    r = subprocess.run(["gcc", "-std=c99", "-I", INCLUDE, str(src), "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {tuple(l.split()[:2]): int(l.split()[2]) for l in out if l}
    for cname, py in mirrors.items():
        assert got[(cname, "size")] == ctypes.sizeof(py), cname
        for fname, _ in py._fields_:
            assert got[(cname, fname)] == getattr(py, fname).offset, (cname, fname)


def test_stream_handles_passed_to_the_c_entry_points():
    """None stays NULL (the context's own stream); a raw handle passes as is;
    a torch stream passes its handle, except torch's default stream (handle
    0), which the C entry points would read as "the context's stream": it
    goes as cudaStreamLegacy (1), so the call is ordered after the work
    already queued there."""
    import libsais_gb300 as G

    class FakeStream:
        def __init__(self, h):
            self.cuda_stream = h

    assert G._stream_handle(None) is None
    assert G._stream_handle(0x7F00) == 0x7F00
    assert G._stream_handle(FakeStream(0x5000)) == 0x5000
    assert G._stream_handle(FakeStream(0)) == 1
