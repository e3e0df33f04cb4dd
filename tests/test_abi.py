"""The C ABI library loads and exports every entry point include/lbswim_c.h
declares; argument errors are reported without touching a GPU."""
import ctypes as C
import os
import re

import pytest

from helpers import ROOT

HEADER = os.path.join(ROOT, "include", "lbswim_c.h")


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"\b(lbswim_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "lbswim_lattice_create" in syms and "lbswim_system_step" in syms
    assert len(syms) >= 30


def test_library_exports_every_declared_symbol():
    from lbswim import _lib
    for name in declared_symbols():
        assert hasattr(_lib.lib, name), name


def test_argument_errors_without_gpu():
    from lbswim import _lib
    h = C.c_void_p()
    assert _lib.lib.lbswim_lattice_create(0, 4, 4, 0.8, 0.8, 0, C.byref(h)) == -1
    assert b"positive" in _lib.lib.lbswim_last_error()
    assert _lib.lib.lbswim_lattice_create(4, 4, 4, -0.6, 0.8, 0, C.byref(h)) == -1
    assert _lib.lib.lbswim_lattice_create(4, 4, 4, 0.8, 0.8, 9, C.byref(h)) == -1
    assert _lib.lib.lbswim_lattice_step(None) == -1
    assert _lib.lib.lbswim_swimmers_create(-1, None, C.byref(h)) == -1
    assert _lib.lib.lbswim_tracers_create(-5, C.byref(h)) == -1
    with pytest.raises(_lib.LbswimError):
        _lib.check(_lib.lib.lbswim_lattice_step(None))


def test_python_surface_mirrors_reference_modules():
    from lbswim import lb, shared, swimmers, tracers
    from lbswim.System import System
    for cls, names in ((lb.Lattice, ["Step", "CalcHydro", "InitFromHydro", "ZeroForce", "rho",
                                     "u", "force", "fOld", "fNew", "params", "addr",
                                     "time_step", "__reduce__", "__setstate__"]),
                       (swimmers.Array, ["AddForces", "Move", "H2D", "D2H", "r", "v", "n",
                                         "common", "__reduce__", "__setstate__"]),
                       (tracers.Array, ["AddForces", "Move", "H2D", "D2H", "r", "s", "v"]),
                       (System, ["AddThing", "Step"]),
                       (shared.Array, ["H2D", "D2H", "data"])):
        for n in names:
            assert hasattr(cls, n), (cls, n)
    cp = swimmers.CommonParams()
    cp.P = 1e-3
    cp.seed = 1234
    cp.rotational_advection_off = True
    assert cp.P == 1e-3 and cp.seed == 1234 and cp.rotational_advection_off is True
    import pickle
    cp2 = pickle.loads(pickle.dumps(cp))
    assert cp2.P == 1e-3 and cp2.seed == 1234


def test_c_program_builds_against_header_and_library(tmp_path):
    # tests/c_driver.c uses nothing but include/lbswim_c.h: it compiles as C99
    # and links against the library (its run is a GPU test)
    import shutil
    import subprocess
    from lbswim import _lib
    gcc = shutil.which("gcc") or shutil.which("cc")
    if gcc is None:
        pytest.skip("no C compiler")
    libdir = os.path.dirname(os.path.abspath(_lib.lib._name))
    exe = str(tmp_path / "c_driver")
    r = subprocess.run([gcc, "-std=c99", "-O2", "-Wall", "-Werror",
                        os.path.join(ROOT, "tests", "c_driver.c"),
                        "-I", os.path.join(ROOT, "include"), "-o", exe, "-L", libdir,
                        "-l:" + os.path.basename(_lib.lib._name), "-lm"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert os.path.exists(exe)


def test_lbparams_fill_matches_oracle_tables():
    # LatticeEigenSet of the C++ class API (d3q15.c:2-186) runs on the host
    import numpy as np
    import oracle as O
    from lbswim import _lib
    p = _lib.LBParamsStruct()
    p.tau_s, p.tau_b = 0.7, 1.3
    _lib.check(_lib.lib.lbswim_lbparams_fill(C.byref(p)))
    ref = O.params_dict(O.params(0.7, 1.3))
    assert (p.tau_s, p.tau_b) == (0.7, 1.3)
    for name in ("w", "xi", "ci", "Q", "complement", "norms", "mm", "mmi"):
        assert np.array_equal(np.ctypeslib.as_array(getattr(p, name)), ref[name]), name
