"""The C ABI on its own: a C program (tests/c_driver.c) built with gcc against
include/lbswim_c.h and the library runs the reference's README scenario with
single calls; the Python surface running the same scenario through System.Step
ends with the same bits."""
import os
import shutil
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "gpu-swimmers_gb300", "lbswim")
STEPS = 100


def _python_run(steps):
    from lbswim import lb, swimmers, tracers
    from lbswim.System import System
    tau = 0.25
    lat = lb.Lattice(16, 16, 16, tau, tau)
    lat.rho[:] = 1.0
    lat.rho.H2D()
    lat.u[:] = 0.0
    lat.u.H2D()
    lat.ZeroForce()
    system = System(lat)
    cp = swimmers.CommonParams()
    cp.P = 1e-3
    cp.l = 0.1
    cp.alpha = 0.01
    cp.mobility = (1.0 / 0.1 - 1.0 / 1.5) / (6.0 * np.pi * (tau / 3.0))
    cp.translational_advection_off = False
    cp.rotational_advection_off = False
    cp.seed = 1234
    sw = swimmers.Array(1, cp)
    sw.r[:] = 8
    sw.n[:] = [[0], [0], [1]]
    sw.v[:] = 0.0
    sw.H2D()
    system.AddThing(sw)
    tr = tracers.Array(16 ** 3)
    tr.r[:] = np.mgrid[:16, :16, :16].reshape(3, 16 ** 3)
    tr.v[:] = 0.0
    tr.H2D()
    system.AddThing(tr)
    lat.InitFromHydro()
    system.Step(steps)
    lat.rho.D2H()
    lat.u.D2H()
    sw.D2H()
    tr.D2H()
    return np.concatenate([lat.rho.data.reshape(-1), lat.u.data.reshape(-1),
                           sw.r.data.reshape(-1), sw.n.data.reshape(-1),
                           tr.r.data.reshape(-1)])


def test_c_program_matches_python_surface(tmp_path):
    gcc = shutil.which("gcc") or shutil.which("cc")
    if gcc is None:
        pytest.skip("no C compiler")
    lib = os.path.join(LIBDIR, "_liblbswim.so")
    assert os.path.exists(lib), "build the library first (gpu-swimmers_gb300/build.py)"
    exe = str(tmp_path / "c_driver")
    subprocess.run([gcc, "-std=c99", "-O2", "-Wall", "-Werror",
                    os.path.join(ROOT, "tests", "c_driver.c"),
                    "-I", os.path.join(ROOT, "include"), "-o", exe,
                    "-L", LIBDIR, "-l:_liblbswim.so", "-Wl,-rpath," + LIBDIR, "-lm"],
                   check=True, capture_output=True, text=True)
    out = str(tmp_path / "state.bin")
    r = subprocess.run([exe, str(STEPS), out], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    from_c = np.fromfile(out, dtype=np.float64)
    from_py = _python_run(STEPS)
    N = 16 ** 3
    assert from_c.size == from_py.size == N + 3 * N + 6 + 3 * N
    assert np.array_equal(from_c, from_py)
    # the swimmer moved along +z and mass stayed put
    sw_r = from_c[4 * N:4 * N + 3]
    assert sw_r[2] > 8.0
    assert abs(from_c[:N].sum() - N) < 1e-9
