"""ctypes front end for the CPU oracle (TEST INFRASTRUCTURE ONLY).

Two libraries live behind this module:

* ``liborc``  -- oracle/lbswim_oracle.c, the project's CPU restatement of the
  reference's coupled step, built into oracle/_build/.
* ``libref``  -- the reference's own kernels built for the host by
  oracle/build_ref.py into oracle/_ref/ (only where the reference sources are
  present; never on a machine without them).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module.  The product library (gpu-swimmers_gb300/) never does.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
ORC_SO = os.path.join(BUILD_DIR, "liborc.so")
REF_SO = os.path.join(HERE, "_ref", "libref.so")

_D = C.POINTER(C.c_double)
_I3 = C.c_int * 3


def build(verbose=False):
    """Compile lbswim_oracle.c into oracle/_build/liborc.so."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    src = os.path.join(HERE, "lbswim_oracle.c")
    if os.path.exists(ORC_SO) and os.path.getmtime(ORC_SO) >= max(
            os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "lbswim_oracle.h"))):
        return ORC_SO
    cmd = ["gcc", "-O3", "-fPIC", "-shared", "-fopenmp", "-std=c11", "-ffp-contract=off",
           src, "-o", ORC_SO + ".tmp", "-lm"]
    subprocess.run(cmd, check=True, capture_output=not verbose)
    os.replace(ORC_SO + ".tmp", ORC_SO)
    return ORC_SO


class OrcParams(C.Structure):
    _fields_ = [("cs2", C.c_double), ("w", C.c_double * 15), ("xi", (C.c_double * 3) * 15),
                ("ci", (C.c_int * 3) * 15), ("Q", ((C.c_double * 3) * 3) * 15),
                ("complement", C.c_int * 15), ("norms", C.c_double * 15),
                ("mm", (C.c_double * 15) * 15), ("mmi", (C.c_double * 15) * 15),
                ("tau_s", C.c_double), ("tau_b", C.c_double)]


class OrcCommon(C.Structure):
    _fields_ = [("P", C.c_double), ("l", C.c_double), ("alpha", C.c_double),
                ("mobility", C.c_double), ("translational_advection_off", C.c_int),
                ("rotational_advection_off", C.c_int), ("seed", C.c_uint64)]


class OrcSystem(C.Structure):
    _fields_ = [("params", OrcParams), ("size", C.c_int * 3), ("f_old", _D), ("f_new", _D),
                ("rho", _D), ("u", _D), ("force", _D), ("nsw", C.c_int), ("common", OrcCommon),
                ("sw_step", C.c_uint64), ("sw_r", _D), ("sw_v", _D), ("sw_n", _D),
                ("ntr", C.c_int), ("tr_r", _D), ("tr_s", _D), ("tr_v", _D),
                ("time_step", C.c_int)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(ORC_SO)
        L.orc_peskin_delta.restype = C.c_double
        L.orc_peskin_delta.argtypes = [C.c_double]
        L.orc_rng_uniform.restype = C.c_float
        L.orc_rng_uniform.argtypes = [C.c_uint64, C.c_uint32, C.c_uint64]
        L.orc_rng_normal3.argtypes = [C.c_uint64, C.c_uint32, C.c_uint64, _D]
        L.orc_det_log.restype = C.c_double
        L.orc_det_log.argtypes = [C.c_double]
        L.orc_det_sincos2pi.argtypes = [C.c_double, C.POINTER(C.c_double),
                                        C.POINTER(C.c_double)]
        L.orc_philox4x32.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                     C.POINTER(C.c_uint32)]
        L.orc_eigenset.argtypes = [C.POINTER(OrcParams), C.c_double, C.c_double]
        L.orc_system_step.argtypes = [C.POINTER(OrcSystem), C.c_int]
        L.orc_init_from_hydro.argtypes = [C.POINTER(OrcParams), _I3, _D, _D, _D, C.c_int]
        L.orc_step.argtypes = [C.POINTER(OrcParams), _I3, _D, _D, _D]
        L.orc_calc_hydro.argtypes = [C.POINTER(OrcParams), _I3, _D, _D, _D, _D]
        L.orc_swimmers_add_forces.argtypes = [_I3, _D, C.c_int, C.POINTER(OrcCommon), _D, _D]
        L.orc_swimmers_move.argtypes = [_I3, _D, C.c_int, C.POINTER(OrcCommon), C.c_uint64,
                                        _D, _D, _D]
        L.orc_tracers_move.argtypes = [_I3, _D, C.c_int, _D, _D, _D]
        L.orc_interp_velocity.argtypes = [_I3, _D, _D, _D]
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_get_threads.restype = C.c_int
        _lib = L
    return _lib


def _p(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_D)


def params(tau_s, tau_b):
    P = OrcParams()
    lib().orc_eigenset(C.byref(P), tau_s, tau_b)
    return P


def params_dict(P):
    return {"cs2": P.cs2, "w": np.ctypeslib.as_array(P.w).copy(),
            "xi": np.ctypeslib.as_array(P.xi).copy(), "ci": np.ctypeslib.as_array(P.ci).copy(),
            "Q": np.ctypeslib.as_array(P.Q).copy(),
            "complement": np.ctypeslib.as_array(P.complement).copy(),
            "norms": np.ctypeslib.as_array(P.norms).copy(),
            "mm": np.ctypeslib.as_array(P.mm).copy(), "mmi": np.ctypeslib.as_array(P.mmi).copy(),
            "tau_s": P.tau_s, "tau_b": P.tau_b}


def peskin_delta(x):
    return lib().orc_peskin_delta(float(x))


def philox4x32(ctr, key):
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib().orc_philox4x32(c, k, o)
    return list(o)


def rng_uniform(seed, swimmer, step):
    return lib().orc_rng_uniform(seed, swimmer, step)


def rng_normal3(seed, swimmer, step):
    out = np.zeros(3)
    lib().orc_rng_normal3(seed, swimmer, step, _p(out))
    return out


def set_threads(n):
    lib().orc_set_threads(int(n))


def get_threads():
    return lib().orc_get_threads()


class System:
    """State of one coupled solve held in numpy arrays (FP64, element-slowest)."""

    def __init__(self, size, tau_s, tau_b, rho, u, swimmers=None, tracers=None, compat_sxz=True):
        nx, ny, nz = size
        N = nx * ny * nz
        self.size = tuple(size)
        self.N = N
        self.P = params(tau_s, tau_b)
        self.rho = np.ascontiguousarray(np.broadcast_to(rho, (N,)), dtype=np.float64).copy()
        self.u = np.ascontiguousarray(np.broadcast_to(u, (3, N)), dtype=np.float64).reshape(3 * N).copy()
        self.force = np.zeros(3 * N)
        self.f_a = np.zeros(15 * N)
        self.f_b = np.zeros(15 * N)
        lib().orc_init_from_hydro(C.byref(self.P), _I3(*size), _p(self.rho), _p(self.u),
                                  _p(self.f_a), int(bool(compat_sxz)))
        s = OrcSystem()
        s.params = self.P
        s.size = _I3(*size)
        s.f_old = _p(self.f_a)
        s.f_new = _p(self.f_b)
        s.rho = _p(self.rho)
        s.u = _p(self.u)
        s.force = _p(self.force)
        self.sw = None
        if swimmers is not None and swimmers["n"] > 0:
            n = swimmers["n"]
            self.sw = {k: np.ascontiguousarray(swimmers[k], dtype=np.float64).reshape(3 * n).copy()
                       for k in ("r", "v", "nvec")}
            c = OrcCommon()
            for k in ("P", "l", "alpha", "mobility"):
                setattr(c, k, float(swimmers[k]))
            c.translational_advection_off = int(bool(swimmers.get("translational_advection_off", False)))
            c.rotational_advection_off = int(bool(swimmers.get("rotational_advection_off", False)))
            c.seed = int(swimmers["seed"])
            s.nsw = n
            s.common = c
            s.sw_step = int(swimmers.get("step", 0))
            s.sw_r = _p(self.sw["r"])
            s.sw_v = _p(self.sw["v"])
            s.sw_n = _p(self.sw["nvec"])
        self.tr = None
        if tracers is not None and tracers["n"] > 0:
            n = tracers["n"]
            self.tr = {k: np.ascontiguousarray(tracers[k], dtype=np.float64).reshape(3 * n).copy()
                       for k in ("r", "v")}
            self.tr["s"] = np.ascontiguousarray(tracers.get("s", np.zeros(3 * n)),
                                                dtype=np.float64).reshape(3 * n).copy()
            s.ntr = n
            s.tr_r = _p(self.tr["r"])
            s.tr_s = _p(self.tr["s"])
            s.tr_v = _p(self.tr["v"])
        self.s = s

    def step(self, nsteps=1):
        lib().orc_system_step(C.byref(self.s), int(nsteps))

    @property
    def f(self):
        addr = C.cast(self.s.f_old, C.c_void_p).value
        return self.f_a if addr == self.f_a.ctypes.data else self.f_b

    @property
    def time_step(self):
        return self.s.time_step

    def snapshot(self):
        N = self.N
        out = {"rho": self.rho.copy(), "u": self.u.reshape(3, N).copy(),
               "force": self.force.reshape(3, N).copy(), "f": self.f.reshape(15, N).copy()}
        if self.sw is not None:
            n = self.s.nsw
            out.update({"sw_r": self.sw["r"].reshape(3, n).copy(),
                        "sw_v": self.sw["v"].reshape(3, n).copy(),
                        "sw_n": self.sw["nvec"].reshape(3, n).copy()})
        if self.tr is not None:
            n = self.s.ntr
            out.update({"tr_r": self.tr["r"].reshape(3, n).copy(),
                        "tr_v": self.tr["v"].reshape(3, n).copy(),
                        "tr_s": self.tr["s"].reshape(3, n).copy()})
        return out


# ---------------------------------------------------------------------------
# The reference's own kernels, host build (oracle/_ref/libref.so)
# ---------------------------------------------------------------------------
_ref = None


def ref_available():
    return os.path.exists(REF_SO)


def ref_lib():
    global _ref
    if _ref is None:
        L = C.CDLL(REF_SO)
        L.ref_lattice_new.restype = C.c_void_p
        L.ref_lattice_new.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double]
        L.ref_lattice_free.argtypes = [C.c_void_p]
        L.ref_lattice_host.restype = _D
        L.ref_lattice_host.argtypes = [C.c_void_p, C.c_int]
        L.ref_lattice_h2d.argtypes = [C.c_void_p, C.c_int]
        L.ref_lattice_d2h.argtypes = [C.c_void_p, C.c_int]
        L.ref_lattice_op.argtypes = [C.c_void_p, C.c_int]
        L.ref_lattice_time_step.argtypes = [C.c_void_p]
        L.ref_lattice_params.argtypes = [C.c_void_p, _D]
        L.ref_lbparams_size.restype = C.c_int
        L.ref_swimmers_new.restype = C.c_void_p
        L.ref_swimmers_new.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                       C.c_int, C.c_int, C.c_ulonglong]
        L.ref_swimmers_host.restype = _D
        L.ref_swimmers_host.argtypes = [C.c_void_p, C.c_int]
        for name in ("ref_swimmers_h2d", "ref_swimmers_d2h", "ref_tracers_h2d", "ref_tracers_d2h"):
            getattr(L, name).argtypes = [C.c_void_p]
        for name in ("ref_swimmers_add_forces", "ref_swimmers_move", "ref_tracers_move"):
            getattr(L, name).argtypes = [C.c_void_p, C.c_void_p]
        L.ref_tracers_new.restype = C.c_void_p
        L.ref_tracers_new.argtypes = [C.c_int]
        L.ref_tracers_host.restype = _D
        L.ref_tracers_host.argtypes = [C.c_void_p, C.c_int]
        L.ref_set_threads.argtypes = [C.c_int]
        _ref = L
    return _ref


class RefSystem:
    """The reference's classes driven in the order of its README / System.py."""

    def __init__(self, size, tau_s, tau_b, rho, u, swimmers=None, tracers=None, threads=1):
        L = ref_lib()
        L.ref_set_threads(int(threads))
        nx, ny, nz = size
        self.N = N = nx * ny * nz
        self.size = tuple(size)
        self.lat = L.ref_lattice_new(nx, ny, nz, tau_s, tau_b)
        self._view(0, N)[:] = np.broadcast_to(rho, (N,))
        L.ref_lattice_h2d(self.lat, 0)
        self._view(1, 3 * N)[:] = np.broadcast_to(u, (3, N)).reshape(3 * N)
        L.ref_lattice_h2d(self.lat, 1)
        L.ref_lattice_op(self.lat, 0)  # ZeroForce
        self.sw = None
        if swimmers is not None and swimmers["n"] > 0:
            n = swimmers["n"]
            self.sw = L.ref_swimmers_new(n, swimmers["P"], swimmers["l"], swimmers["alpha"],
                                         swimmers["mobility"],
                                         int(bool(swimmers.get("translational_advection_off", False))),
                                         int(bool(swimmers.get("rotational_advection_off", False))),
                                         int(swimmers["seed"]))
            self.nsw = n
            for k, which in (("r", 0), ("v", 1), ("nvec", 2)):
                np.ctypeslib.as_array(L.ref_swimmers_host(self.sw, which), (3 * n,))[:] = \
                    np.asarray(swimmers[k], dtype=np.float64).reshape(3 * n)
            L.ref_swimmers_h2d(self.sw)
        self.tr = None
        if tracers is not None and tracers["n"] > 0:
            n = tracers["n"]
            self.tr = L.ref_tracers_new(n)
            self.ntr = n
            np.ctypeslib.as_array(L.ref_tracers_host(self.tr, 0), (3 * n,))[:] = \
                np.asarray(tracers["r"], dtype=np.float64).reshape(3 * n)
            np.ctypeslib.as_array(L.ref_tracers_host(self.tr, 1), (3 * n,))[:] = 0.0
            np.ctypeslib.as_array(L.ref_tracers_host(self.tr, 2), (3 * n,))[:] = \
                np.asarray(tracers["v"], dtype=np.float64).reshape(3 * n)
            L.ref_tracers_h2d(self.tr)
        L.ref_lattice_op(self.lat, 3)  # InitFromHydro

    def _view(self, which, n):
        return np.ctypeslib.as_array(ref_lib().ref_lattice_host(self.lat, which), (n,))

    def step(self, nsteps=1):
        L = ref_lib()
        for _ in range(nsteps):
            L.ref_lattice_op(self.lat, 0)
            if self.sw is not None:
                L.ref_swimmers_add_forces(self.sw, self.lat)
            L.ref_lattice_op(self.lat, 1)
            L.ref_lattice_op(self.lat, 2)
            if self.sw is not None:
                L.ref_swimmers_move(self.sw, self.lat)
            if self.tr is not None:
                L.ref_tracers_move(self.tr, self.lat)

    @property
    def time_step(self):
        return ref_lib().ref_lattice_time_step(self.lat)

    def snapshot(self):
        L = ref_lib()
        N = self.N
        for which in range(4):
            L.ref_lattice_d2h(self.lat, which)
        out = {"rho": self._view(0, N).copy(), "u": self._view(1, 3 * N).reshape(3, N).copy(),
               "force": self._view(2, 3 * N).reshape(3, N).copy(),
               "f": self._view(3, 15 * N).reshape(15, N).copy()}
        if self.sw is not None:
            L.ref_swimmers_d2h(self.sw)
            n = self.nsw
            for k, which in (("sw_r", 0), ("sw_v", 1), ("sw_n", 2)):
                out[k] = np.ctypeslib.as_array(L.ref_swimmers_host(self.sw, which), (3 * n,)).reshape(3, n).copy()
        if self.tr is not None:
            L.ref_tracers_d2h(self.tr)
            n = self.ntr
            out["tr_r"] = np.ctypeslib.as_array(L.ref_tracers_host(self.tr, 0), (3 * n,)).reshape(3, n).copy()
            out["tr_v"] = np.ctypeslib.as_array(L.ref_tracers_host(self.tr, 2), (3 * n,)).reshape(3, n).copy()
        return out

    def params(self):
        L = ref_lib()
        nbytes = L.ref_lbparams_size()
        buf = (C.c_double * (nbytes // 8 + 1))()
        L.ref_lattice_params(self.lat, C.cast(buf, _D))
        P = OrcParams.from_buffer_copy(bytes(buf)[:C.sizeof(OrcParams)])
        return P


# ---------------------------------------------------------------------------
# Workload builders shared by tests, fixtures and the CPU baseline
# ---------------------------------------------------------------------------
def readme_case(n=16, tau=0.25):
    """The README example: 16^3, one swimmer at the centre, tracers on nodes."""
    eta = tau / 3.0
    a, hydro = 0.1, 1.5
    sw = {"n": 1, "P": 1e-3, "l": 0.1, "alpha": 0.01,
          "mobility": (1.0 / a - 1.0 / hydro) / (6.0 * np.pi * eta),
          "translational_advection_off": False, "rotational_advection_off": False,
          "seed": 1234, "r": np.full((3, 1), n / 2.0), "nvec": np.array([[0.0], [0.0], [1.0]]),
          "v": np.zeros((3, 1))}
    tr = {"n": n ** 3, "r": np.mgrid[:n, :n, :n].reshape(3, n ** 3).astype(np.float64),
          "v": np.zeros((3, n ** 3))}
    return {"size": (n, n, n), "tau_s": tau, "tau_b": tau, "rho": 1.0, "u": 0.0,
            "swimmers": sw, "tracers": tr}


def random_case(size, nsw, ntr, seed, tau_s=0.8, tau_b=0.8, u_amp=0.0, P=1e-3, l=0.5,
                alpha=0.01, rot_off=False, trans_off=False):
    """Seeded random case: rho = 1 + 1e-3 U[0,1), swimmers uniform in the box
    with orientations uniform on the sphere, tracers uniform in the box."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = size
    N = nx * ny * nz
    L = np.array(size, dtype=np.float64).reshape(3, 1)
    rho = 1.0 + 1e-3 * rng.random(N)
    u = u_amp * (rng.random((3, N)) - 0.5)
    eta = tau_s / 3.0
    nv = rng.standard_normal((3, nsw))
    nv /= np.linalg.norm(nv, axis=0, keepdims=True) if nsw else 1.0
    sw = {"n": nsw, "P": P, "l": l, "alpha": alpha,
          "mobility": (1.0 / 0.1 - 1.0 / 1.5) / (6.0 * np.pi * eta),
          "translational_advection_off": trans_off, "rotational_advection_off": rot_off,
          "seed": int(seed) * 7919 + 17, "r": rng.random((3, nsw)) * L, "nvec": nv,
          "v": np.zeros((3, nsw))}
    tr = {"n": ntr, "r": rng.random((3, ntr)) * L, "v": np.zeros((3, ntr))}
    return {"size": tuple(size), "tau_s": tau_s, "tau_b": tau_b, "rho": rho, "u": u,
            "swimmers": sw, "tracers": tr}


def make_system(case, compat_sxz=True):
    return System(case["size"], case["tau_s"], case["tau_b"], case["rho"], case["u"],
                  case.get("swimmers"), case.get("tracers"), compat_sxz=compat_sxz)


def make_ref_system(case, threads=1):
    return RefSystem(case["size"], case["tau_s"], case["tau_b"], case["rho"], case["u"],
                     case.get("swimmers"), case.get("tracers"), threads=threads)
