"""Python surface behaviour on the GPU: README scenario, fields, pickle, errors."""
import pickle

import numpy as np
import pytest

import oracle as O
from gpu_harness import build_gpu, snapshot
from helpers import TOL_F64, rel_l2, rel_max

pytestmark = pytest.mark.gpu


def test_readme_example_runs_unchanged():
    from lbswim import lb, swimmers, tracers
    from lbswim.System import System
    tau = 0.25
    eta = tau / 3
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
    a = 0.1
    hydroRadius = 1.5
    cp.mobility = (1.0 / a - 1.0 / hydroRadius) / (6.0 * np.pi * eta)
    cp.translational_advection_off = False
    cp.rotational_advection_off = False
    cp.seed = 1234
    sw = swimmers.Array(1, cp)
    sw.r[:] = 8
    sw.n[:] = [[0], [0], [1]]
    sw.v[:] = 0.
    sw.H2D()
    system.AddThing(sw)
    tr = tracers.Array(16 ** 3)
    tr.r[:] = np.mgrid[:16, :16, :16].reshape(3, 16 ** 3)
    tr.v[:] = 0.
    tr.H2D()
    system.AddThing(tr)
    lat.InitFromHydro()
    traj = []
    while lat.time_step < 100:
        if lat.time_step % 10 == 0:
            sw.D2H()
            traj.append(sw.r[:, 0].copy())
        system.Step()
    assert lat.time_step == 100
    traj = np.array(traj)
    assert np.all(np.diff(traj[:, 2]) > 0)  # swims along +z
    assert lat.params.eta == pytest.approx(tau / 3)
    assert lat.addr.size == (16, 16, 16) and lat.addr.n == 4096
    assert lat.rho.shape == (1, 16, 16, 16) and lat.fOld.shape == (15, 16, 16, 16)


def test_params_tables_match_oracle():
    from lbswim import lb
    lat = lb.Lattice(4, 4, 4, 0.7, 0.9)
    P = lat.params
    ref = O.params_dict(O.params(0.7, 0.9))
    for k in ("w", "xi", "ci", "Q", "complement", "norms", "mm", "mmi"):
        assert np.array_equal(getattr(P, k), ref[k]), k
    assert P.cs2 == ref["cs2"] and P.tau_s == 0.7 and P.tau_b == 0.9


@pytest.mark.parametrize("precision,tol", [("f64", 0.0), ("f32", 1e-9), ("bf16", 2e-5),
                                           ("f16", 1e-6)])
def test_field_roundtrip(precision, tol):
    from lbswim import lb
    lat = lb.Lattice(10, 12, 14, 0.8, 0.8, precision=precision)
    rng = np.random.default_rng(0)
    w = lat.params.w.reshape(15, 1, 1, 1)
    f = w * (1.0 + 1e-3 * rng.standard_normal((15, 10, 12, 14)))
    lat.fOld[:] = f
    lat.fOld.H2D()
    lat.fOld[:] = 0
    lat.fOld.D2H()
    assert np.max(np.abs(lat.fOld.data - f)) <= tol
    for name in ("rho", "u", "force"):
        fld = getattr(lat, name)
        vals = rng.standard_normal(fld.shape)
        fld[:] = vals
        fld.H2D()
        fld[:] = 0
        fld.D2H()
        assert np.max(np.abs(fld.data - vals)) <= (0 if precision == "f64" else 1e-6)


def test_zero_force_then_read_is_zero():
    from lbswim import lb
    lat = lb.Lattice(8, 8, 8, 0.8, 0.8)
    lat.force[:] = 1.0
    lat.force.H2D()
    lat.ZeroForce()
    lat.force.D2H()
    assert np.all(lat.force.data == 0)


def test_pickle_resume_is_exact():
    case = O.random_case((12, 14, 16), 40, 100, seed=31, alpha=0.3)
    lat, sw, tr, system = build_gpu(case)
    system.Step(10)
    blob = pickle.dumps((lat, sw, tr))
    system.Step(15)
    end = snapshot(lat, sw, tr)
    lat2, sw2, tr2 = pickle.loads(blob)
    from lbswim.System import System
    s2 = System(lat2)
    s2.AddThing(sw2)
    s2.AddThing(tr2)
    # the reference pickles only fOld; rho/u are recomputed by the first step
    assert lat2.time_step == 10
    s2.Step(15)
    res = snapshot(lat2, sw2, tr2)
    for k in ("f", "rho", "u", "sw_r", "sw_n", "tr_r"):
        assert np.array_equal(res[k], end[k]), k


def test_invalid_field_raises():
    from lbswim import _lib, lb
    lat = lb.Lattice(4, 4, 4, 0.8, 0.8)
    buf = np.zeros(4 * 4 * 4)
    with pytest.raises(_lib.LbswimError):
        _lib.check(_lib.lib.lbswim_lattice_h2d(lat._h, 7, _lib.dptr(buf)))


def test_kernel_launch_counter_advances():
    from lbswim import _lib
    before = _lib.kernel_launches()
    case = O.random_case((8, 8, 8), 4, 10, seed=1)
    lat, sw, tr, system = build_gpu(case)
    system.Step(3)
    lat.synchronize()
    assert _lib.kernel_launches() - before >= 3 * 6


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_system_step_matches_single_calls_bitwise(precision):
    """lbswim_system_step moves tracers on their own stream; its results are
    those of the README's sequence of single calls, bit for bit."""
    case = O.random_case((24, 16, 32), 80, 700, seed=44, alpha=0.1, u_amp=0.01)
    lat1, sw1, tr1, system1 = build_gpu(case, precision)
    lat2, sw2, tr2, _ = build_gpu(case, precision)
    system1.Step(70)  # crosses a tracer re-binning
    for _ in range(70):
        lat2.ZeroForce()
        sw2.AddForces(lat2)
        lat2.Step()
        lat2.CalcHydro()
        sw2.Move(lat2)
        tr2.Move(lat2)
    a, b = snapshot(lat1, sw1, tr1), snapshot(lat2, sw2, tr2)
    for k in a:
        assert np.array_equal(a[k], b[k]), k


@pytest.mark.parametrize("precision", ["f32", "bf16"])
def test_system_steps_across_calls_match_single_calls(precision):
    # The swimmer move of a system step also records the next step's dipole
    # ends; the next System.Step takes them unless another call came in
    # between.  One Step per call with read-backs (which change nothing), then
    # the swimmer positions written back (same values) and P changed between
    # calls: the same bits as the README's single calls throughout.
    case = O.random_case((24, 16, 32), 80, 300, seed=45, alpha=0.1, u_amp=0.01)
    lat1, sw1, tr1, system1 = build_gpu(case, precision)
    lat2, sw2, tr2, _ = build_gpu(case, precision)

    def single(n):
        for _ in range(n):
            lat2.ZeroForce()
            sw2.AddForces(lat2)
            lat2.Step()
            lat2.CalcHydro()
            sw2.Move(lat2)
            tr2.Move(lat2)

    for _ in range(30):
        system1.Step()
        sw1.D2H()
        assert lat1.time_step > 0
    single(30)
    for sw in (sw1, sw2):
        sw.D2H()
        sw.H2D()
    for _ in range(10):
        system1.Step()
    single(10)
    for sw in (sw1, sw2):
        sw.common.P = 2e-3
    system1.Step(12)
    single(12)
    a, b = snapshot(lat1, sw1, tr1), snapshot(lat2, sw2, tr2)
    for k in a:
        assert np.array_equal(a[k], b[k]), k


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_empty_particle_arrays_leave_the_lattice_alone(precision):
    # a System holding a swimmer array and a tracer array of zero particles
    # (the reference allows SwimmerArray(0, ...) and TracerArray(0)) steps the
    # lattice exactly as ZeroForce, Step and CalcHydro alone do
    from lbswim import swimmers, tracers
    from lbswim.System import System
    case = O.random_case((12, 10, 14), 0, 0, seed=31, u_amp=0.01)
    lat1 = build_gpu(case, precision)[0]
    lat2 = build_gpu(case, precision)[0]
    sw0 = swimmers.Array(0, swimmers.CommonParams())
    tr0 = tracers.Array(0)
    system = System(lat1)
    system.AddThing(sw0)
    system.AddThing(tr0)
    system.Step(4)
    system.Step()
    for _ in range(5):
        lat2.ZeroForce()
        lat2.Step()
        lat2.CalcHydro()
    a, b = snapshot(lat1, sw0, tr0), snapshot(lat2, None, None)
    for k in b:
        assert np.array_equal(a[k], b[k]), k
    for k in ("sw_r", "sw_v", "sw_n", "tr_r", "tr_v", "tr_s"):
        assert a[k].shape == (3, 0), k
    assert lat1.time_step == lat2.time_step == 5


def test_particle_host_copies_are_pinned_and_round_trip():
    # swimmer and tracer host copies live in page-locked memory from
    # lbswim_host_alloc; they keep the FP64 values exactly through H2D/D2H
    import ctypes as C
    from lbswim import _lib, swimmers, tracers
    ptr = C.c_void_p()
    _lib.check(_lib.lib.lbswim_host_alloc(1 << 20, C.byref(ptr)))
    assert ptr.value
    _lib.check(_lib.lib.lbswim_host_free(ptr))
    _lib.check(_lib.lib.lbswim_host_free(None))
    rng = np.random.default_rng(5)
    sw = swimmers.Array(37, swimmers.CommonParams())
    tr = tracers.Array(53)
    vals = {}
    for arr, name in ((sw.r, "sw"), (tr.r, "tr")):
        v = rng.random(arr.data.shape) * 10.0
        arr[:] = v
        arr.H2D()
        arr[:] = 0.0
        arr.D2H()
        vals[name] = (v, arr.data.copy())
    for v, got in vals.values():
        assert np.array_equal(v, got)


def test_swimmer_read_back_of_chosen_fields():
    # lbswim_swimmers_d2h_all copies the fields whose buffers are given and
    # leaves the others alone
    from lbswim import _lib, swimmers
    sw = swimmers.Array(29, swimmers.CommonParams())
    rng = np.random.default_rng(9)
    vals = [rng.random((3, 29)) for _ in range(3)]
    for arr, v in zip((sw.r, sw.v, sw.n), vals):
        arr[:] = v
        arr.H2D()
    r = np.zeros(3 * 29)
    n = np.zeros(3 * 29)
    _lib.check(_lib.lib.lbswim_swimmers_d2h_all(sw._h, _lib.dptr(r), None, _lib.dptr(n)))
    assert np.array_equal(r, vals[0].reshape(-1)) and np.array_equal(n, vals[2].reshape(-1))


@pytest.mark.parametrize("precision", ["f32", "bf16"])
def test_blocked_distributions_on_ragged_sizes(precision):
    # reduced-precision distributions are stored in blocks of 32 sites; with
    # N = 7*9*11 (not a multiple of 32) fOld goes through H2D/D2H unchanged
    # (to the format's precision) and a step conserves mass
    from lbswim import lb
    lat = lb.Lattice(7, 9, 11, 0.8, 0.8, precision=precision)
    N = 7 * 9 * 11
    rng = np.random.default_rng(3)
    lat.rho[:] = (1.0 + 1e-3 * rng.random(N)).reshape(1, 7, 9, 11)
    lat.rho.H2D()
    lat.u[:] = 0.01 * rng.standard_normal((3, 7, 9, 11))
    lat.u.H2D()
    lat.InitFromHydro()
    lat.fOld.D2H()
    f0 = lat.fOld.data.copy()
    lat.fOld[:] = f0
    lat.fOld.H2D()
    lat.fOld[:] = 0.0
    lat.fOld.D2H()
    tol = 1e-7 if precision == "f32" else 1e-4
    assert np.max(np.abs(lat.fOld.data - f0)) <= tol * np.max(np.abs(f0))
    m0 = lat.conservation()[0]
    lat.ZeroForce()
    lat.Step()
    assert abs(lat.conservation()[0] - m0) <= 1e-6 * m0
