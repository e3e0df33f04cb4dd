"""The reference's C++ class API (include/liblbswim/) on the GPU: the README
scenario written against the reference's classes (tests/cpp_driver.cpp) ends
with the same bits as the same scenario driven through the C ABI alone
(tests/c_driver.c)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "gpu-swimmers_gb300", "lbswim")
STEPS = 100


def _build(tmp_path, compiler, src, extra):
    exe = str(tmp_path / os.path.splitext(os.path.basename(src))[0])
    cmd = [compiler] + extra + [os.path.join(ROOT, "tests", src), "-o", exe,
                                "-I", os.path.join(ROOT, "include", "liblbswim"),
                                "-I", os.path.join(ROOT, "include"),
                                "-L", LIBDIR, "-l:_liblbswim.so", "-Wl,-rpath," + LIBDIR, "-lm"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def _run(exe, tmp_path):
    out = str(tmp_path / (os.path.basename(exe) + ".bin"))
    r = subprocess.run([exe, str(STEPS), out], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    return np.fromfile(out, dtype=np.float64)


def test_cpp_class_api_matches_c_abi(tmp_path):
    gcc, gxx = shutil.which("gcc"), shutil.which("g++")
    if gcc is None or gxx is None:
        pytest.skip("no C / C++ compiler")
    assert os.path.exists(os.path.join(LIBDIR, "_liblbswim.so"))
    from_cpp = _run(_build(tmp_path, gxx, "cpp_driver.cpp", ["-std=c++17", "-O2"]), tmp_path)
    from_c = _run(_build(tmp_path, gcc, "c_driver.c", ["-std=c99", "-O2"]), tmp_path)
    N = 16 ** 3
    assert from_cpp.size == from_c.size == 7 * N + 6
    assert np.array_equal(from_cpp, from_c)
    assert from_cpp[4 * N + 2] > 8.0  # the swimmer moved along +z
