"""The reference's C++ class API as include/liblbswim/ provides it.

* A C++ program written against the reference's classes (Lattice,
  LatticeData, SharedArray, SharedItem, CommonParams, SwimmerArray,
  TracerArray; tests/cpp_driver.cpp) compiles warning-free and links against
  the library.
* The reference's own Cython package -- its unchanged lb.pyx, shared.pyx,
  swimmers.pyx and tracers.pyx with their .pxd declarations (_lb.pxd,
  _shared.pxd, SwimmerArray.pxd, TracerArray.pxd) -- cythonizes, compiles
  against these headers, links against the library and imports (where the
  reference sources and Cython are present; nothing is written next to them).
No GPU is needed: nothing here creates a lattice.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
import sysconfig

import pytest

import build_ref

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "gpu-swimmers_gb300", "lbswim")
INC = [os.path.join(ROOT, "include", "liblbswim"), os.path.join(ROOT, "include")]


def _lib():
    lib = os.path.join(LIBDIR, "_liblbswim.so")
    if not os.path.exists(lib):
        sys.path.insert(0, os.path.join(ROOT, "gpu-swimmers_gb300"))
        import build
        build.build()
    return lib


def _link_args():
    _lib()
    return ["-L", LIBDIR, "-l:_liblbswim.so", "-Wl,-rpath," + LIBDIR]


def test_cpp_program_on_the_reference_classes_builds(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "cpp_driver")
    cmd = [gxx, "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror",
           os.path.join(ROOT, "tests", "cpp_driver.cpp"), "-o", exe]
    for d in INC:
        cmd += ["-I", d]
    r = subprocess.run(cmd + _link_args(), capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    # without a GPU the first allocation fails and is reported, not fatal
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2 and "usage" in r.stderr


def test_reference_cython_package_builds_on_these_headers(tmp_path):
    ref = build_ref.reference_root()
    if ref is None:
        pytest.skip("reference sources not present")
    pytest.importorskip("Cython")
    np = pytest.importorskip("numpy")
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no C++ compiler")
    src = os.path.join(ref, "lbswim")
    pkg = tmp_path / "pkg" / "lbswim"
    pkg.mkdir(parents=True)
    (pkg / "__init__.py").write_text("")
    ext = sysconfig.get_config_var("EXT_SUFFIX")
    inc = INC + [sysconfig.get_paths()["include"], np.get_include()]
    link = _link_args()

    def build(mod):
        cpp = str(tmp_path / (mod + ".cpp"))
        r = subprocess.run([sys.executable, "-m", "cython", "--cplus", "-2", "-I", src, "-o", cpp,
                            os.path.join(src, mod + ".pyx")], capture_output=True, text=True)
        if r.returncode != 0:
            return mod, "cython: " + r.stderr[-2000:]
        cmd = [gxx, "-shared", "-fPIC", "-O0", "-w", "-std=c++17", cpp,
               "-o", str(pkg / (mod + ext))]
        for d in inc:
            cmd += ["-I", d]
        r = subprocess.run(cmd + link, capture_output=True, text=True)
        return mod, (None if r.returncode == 0 else "g++: " + r.stderr[-2000:])

    mods = ["shared", "lb", "swimmers", "tracers"]
    with cf.ThreadPoolExecutor(max_workers=4) as ex:
        errs = {m: e for m, e in ex.map(build, mods) if e}
    assert not errs, errs
    probe = ("import sys; sys.path.insert(0, %r)\n"
             "from lbswim import shared, lb, swimmers, tracers\n"
             "assert lb.Lattice and lb.LBParams and lb.LatticeAddressing\n"
             "assert swimmers.CommonParams and swimmers.Array and tracers.Array\n"
             "assert shared.Array and shared.PrngArray\n"
             "print('ok')\n" % str(tmp_path / "pkg"))
    r = subprocess.run([sys.executable, "-c", probe], capture_output=True, text=True,
                       cwd=str(tmp_path), timeout=120)
    assert r.returncode == 0 and "ok" in r.stdout, r.stderr
