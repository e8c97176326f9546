"""The CMake package: an application written against the reference's
exported target (`find_package(libsais)` + `target_link_libraries(app
libsais)`) configures, links the GPU build and runs its host-side calls."""
import os
import shutil
import subprocess
import textwrap

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_find_package_links_the_gpu_build(tmp_path, lib):
    cmake = shutil.which("cmake")
    if cmake is None:
        pytest.skip("cmake is not installed")
    (tmp_path / "CMakeLists.txt").write_text(textwrap.dedent(f"""
        cmake_minimum_required(VERSION 3.16)
        project(consumer C)
        find_package(libsais 2.10 CONFIG REQUIRED PATHS "{ROOT}/libsais_gb300/cmake" NO_DEFAULT_PATH)
        add_executable(app main.c)
        target_link_libraries(app PRIVATE libsais)
    """))
    (tmp_path / "main.c").write_text(textwrap.dedent("""
        #include <stdint.h>
        #include <libsais.h>
        #include <libsais64.h>
        #include <libsais16x64.h>
        int main(void) {
            const uint8_t t[1] = {'x'};
            int32_t sa[1] = {7};
            int32_t freq[256];
            if (libsais(t, sa, 1, 0, freq) != 0 || sa[0] != 0 || freq['x'] != 1) return 1;   /* n = 1: host only */
            if (libsais(0, sa, 5, 0, 0) != -1) return 2;
            uint8_t u[1]; int32_t a[2];
            if (libsais_unbwt(t, u, a, 1, 0, 1) != 0 || u[0] != 'x') return 3;
            int64_t sa64[1];
            if (libsais64(t, sa64, 1, 0, 0) != 0 || sa64[0] != 0) return 4;
            return LIBSAIS_VERSION_MAJOR == 2 ? 0 : 5;
        }
    """))
    build = tmp_path / "build"
    r = subprocess.run([cmake, "-S", str(tmp_path), "-B", str(build)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    r = subprocess.run([cmake, "--build", str(build)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    env = dict(os.environ, LD_LIBRARY_PATH=os.path.join(ROOT, "libsais_gb300", "lib"))
    r = subprocess.run([str(build / "app")], capture_output=True, text=True, env=env, timeout=120)
    assert r.returncode == 0, (r.returncode, r.stderr)


def test_version_file_rejects_other_major(tmp_path):
    cmake = shutil.which("cmake")
    if cmake is None:
        pytest.skip("cmake is not installed")
    (tmp_path / "CMakeLists.txt").write_text(textwrap.dedent(f"""
        cmake_minimum_required(VERSION 3.16)
        project(consumer NONE)
        find_package(libsais 3 CONFIG QUIET PATHS "{ROOT}/libsais_gb300/cmake" NO_DEFAULT_PATH)
        if(libsais_FOUND)
            message(FATAL_ERROR "major version 3 must not match")
        endif()
    """))
    r = subprocess.run([cmake, "-S", str(tmp_path), "-B", str(tmp_path / "b")], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
