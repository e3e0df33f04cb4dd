"""Lattice-Boltzmann fluid (reference lbswim/lb.pyx, lbswim/_lb.pxd).

``Lattice(nx, ny, nz, tau_s, tau_b)`` is the reference's D3Q15 MRT fluid on a
periodic box.  The optional ``precision`` selects the device storage:
"f64" (default) is the reference's FP64 method; "f32", "bf16" and "f16" store
distributions as deviations from rest equilibrium and collide in FP32 with
one fused collide/stream/hydro kernel per step.
"""
import ctypes as C

import numpy as np

from . import _lib
from . import shared


class ArrayWrapper:
    """numpy view of a parameter table kept alive by its owner (lb.pyx:11-19)."""

    def __init__(self, owner):
        self.owner = owner

    def wrap(self, array):
        return array


class SharedLatticeArray:
    """A lattice field with shape (components, nx, ny, nz) (lb.pyx:21-46)."""

    def __init__(self, lat, sa):
        self.impl = sa
        nsites = lat.addr.n
        shape = (sa.view.size // nsites,) + lat.addr.size
        self.view = sa.view.reshape(shape)

    @property
    def data(self):
        return self.view

    def H2D(self):
        self.impl.H2D()

    def D2H(self):
        self.impl.D2H()

    def __getattr__(self, attr):
        if attr in ("impl", "view"):
            raise AttributeError(attr)
        return getattr(self.view, attr)

    def __getitem__(self, idx):
        return self.view[idx]

    def __setitem__(self, idx, val):
        self.view[idx] = val

    def __array__(self, dtype=None, copy=None):
        return np.asarray(self.view, dtype=dtype)


class LatticeAddressing:
    """Sizes and strides of the lattice (lb.pyx:48-55, Lattice.h:8-12)."""

    def __init__(self, s):
        self.impl = s

    @property
    def size(self):
        return tuple(self.impl.size)

    @property
    def strides(self):
        return tuple(self.impl.strides)

    @property
    def n(self):
        return int(self.impl.n)


class LBParams:
    """All parameters of the LB model; treat as read only (lb.pyx:57-137)."""

    def __init__(self, s, lat=None):
        self.impl = s
        self.lat = lat

    def _arr(self, name, dtype):
        return np.ctypeslib.as_array(getattr(self.impl, name)).astype(dtype, copy=False)

    @property
    def cs2(self):
        """Speed of sound, squared"""
        return self.impl.cs2

    @property
    def w(self):
        """Quadrature weights"""
        return self._arr("w", np.float64)

    @property
    def xi(self):
        """Velocities as doubles"""
        return self._arr("xi", np.float64)

    @property
    def ci(self):
        """Velocities as ints"""
        return self._arr("ci", np.intc)

    @property
    def Q(self):
        """Kinetic projector Q_i_ab = xi_i_a * xi_i_b - delta_ab cs^2"""
        return self._arr("Q", np.float64)

    @property
    def complement(self):
        return self._arr("complement", np.intc)

    @property
    def norms(self):
        """The modes' normalizers"""
        return self._arr("norms", np.float64)

    @property
    def mm(self):
        """Matrix of eigenvectors (they are the rows)"""
        return self._arr("mm", np.float64)

    @property
    def mmi(self):
        """Inverse matrix"""
        return self._arr("mmi", np.float64)

    @property
    def tau_s(self):
        """Shear relaxation time."""
        return self.impl.tau_s

    @property
    def eta(self):
        """Viscosity of the fluid"""
        return self.tau_s * self.cs2

    @property
    def tau_b(self):
        """Bulk relaxation time."""
        return self.impl.tau_b


class Lattice:
    """D3Q15 MRT lattice-Boltzmann fluid with periodic boundaries (lb.pyx:139-244)."""

    def __init__(self, nx, ny, nz, tau_s, tau_b, precision="f64"):
        if isinstance(precision, str):
            if precision.lower() not in _lib.PRECISIONS:
                raise ValueError("unknown precision %r" % (precision,))
            precision = _lib.PRECISIONS[precision.lower()]
        self._h = None
        h = C.c_void_p()
        _lib.check(_lib.lib.lbswim_lattice_create(int(nx), int(ny), int(nz), float(tau_s),
                                                  float(tau_b), int(precision), C.byref(h)))
        self._h = h
        self._precision = int(precision)
        self._params = None
        self._addr = None
        self._fields = {}

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            _lib.lib.lbswim_lattice_destroy(h)
            self._h = None

    # -- operations (lb.pyx:155-165) --
    def Step(self):
        _lib.check(_lib.lib.lbswim_lattice_step(self._h))

    def CalcHydro(self):
        _lib.check(_lib.lib.lbswim_lattice_calc_hydro(self._h))

    def InitFromHydro(self):
        _lib.check(_lib.lib.lbswim_lattice_init_from_hydro(self._h))

    def ZeroForce(self):
        _lib.check(_lib.lib.lbswim_lattice_zero_force(self._h))

    # -- extensions --
    @property
    def precision(self):
        return _lib.PRECISION_NAMES[self._precision]

    def set_compat(self, flags):
        _lib.check(_lib.lib.lbswim_lattice_set_compat(self._h, int(flags)))

    def set_stream(self, stream):
        """Launch this lattice's work (and that of particles moved with it) on a
        CUDA stream given as an integer handle; 0 is the default stream."""
        _lib.check(_lib.lib.lbswim_lattice_set_stream(self._h, C.c_void_p(int(stream))))

    def synchronize(self):
        _lib.check(_lib.lib.lbswim_lattice_synchronize(self._h))

    @property
    def rho0(self):
        """Reference density of the reduced-precision storage (0 for FP64)."""
        v = C.c_double()
        _lib.check(_lib.lib.lbswim_lattice_get_rho0(self._h, C.byref(v)))
        return v.value

    def init_random(self, seed, amplitude=1e-3):
        """rho = 1 + amplitude U[0, 1), u = 0 from a counter stream keyed by
        (seed, site), made on the device, then InitFromHydro."""
        _lib.check(_lib.lib.lbswim_lattice_init_random(self._h, int(seed), float(amplitude)))

    def set_tau(self, tau_s, tau_b):
        _lib.check(_lib.lib.lbswim_lattice_set_tau(self._h, float(tau_s), float(tau_b)))
        self._params = None

    def status(self, clear=False):
        """Sticky status bits the lattice's kernels and the particle moves on it
        set (_lib.STATUS_NONFINITE, STATUS_PARTICLE_OUTSIDE, STATUS_COPY_TIMEOUT);
        waits for the lattice's queued work; clear resets them."""
        out = C.c_uint()
        _lib.check(_lib.lib.lbswim_lattice_get_status(self._h, C.byref(out), int(bool(clear))))
        return out.value

    def conservation(self):
        """(mass, momentum x, y, z): sums of f and c f over the lattice in FP64,
        in a fixed order."""
        out = (C.c_double * 4)()
        _lib.check(_lib.lib.lbswim_lattice_conservation(self._h, out))
        return tuple(out)

    @property
    def tile(self):
        """Slab shape of the step kernel: 0 = 8 x 32 cross-section, 1 = 16 x 16."""
        t = C.c_int()
        _lib.check(_lib.lib.lbswim_lattice_get_tile(self._h, C.byref(t)))
        return t.value

    @tile.setter
    def tile(self, value):
        _lib.check(_lib.lib.lbswim_lattice_set_tile(self._h, int(value)))

    def join(self):
        """Order this lattice's stream after the tracer moves that System.Step
        leaves running on the tracers' own streams (no host wait)."""
        _lib.check(_lib.lib.lbswim_lattice_join(self._h))

    def set_timing(self, enable=True):
        """Bracket every LB step kernel of this lattice with CUDA events."""
        _lib.check(_lib.lib.lbswim_lattice_set_timing(self._h, int(bool(enable))))

    def read_timing(self):
        """(total device ms, launches) of the LB step kernel since the last read."""
        ms, n = C.c_double(), C.c_int()
        _lib.check(_lib.lib.lbswim_lattice_get_timing(self._h, C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def interp_velocity(self, r):
        """InterpVelocity (interp.cu:8-47) of the current u at points r[3, n]."""
        r = np.ascontiguousarray(np.asarray(r, dtype=np.float64).reshape(3, -1))
        v = np.zeros_like(r)
        _lib.check(_lib.lib.lbswim_lattice_interp_velocity(self._h, r.shape[1], _lib.dptr(r),
                                                           _lib.dptr(v)))
        return v

    def device_ptr(self, field):
        ptr, elem = C.c_void_p(), C.c_int()
        _lib.check(_lib.lib.lbswim_lattice_device_ptr(self._h, int(field), C.byref(ptr),
                                                      C.byref(elem)))
        return ptr.value, elem.value

    # -- state --
    @property
    def time_step(self):
        out = C.c_int()
        _lib.check(_lib.lib.lbswim_lattice_get_time_step(self._h, C.byref(out)))
        return out.value

    @property
    def addr(self):
        if self._addr is None:
            s = _lib.AddressingStruct()
            _lib.check(_lib.lib.lbswim_lattice_get_addressing(self._h, C.byref(s)))
            self._addr = LatticeAddressing(s)
        return self._addr

    @property
    def params(self):
        if self._params is None:
            s = _lib.LBParamsStruct()
            _lib.check(_lib.lib.lbswim_lattice_get_params(self._h, C.byref(s)))
            self._params = LBParams(s, self)
        return self._params

    def _field(self, which):
        f = self._fields.get(which)
        if f is None:
            n = self.addr.n * _lib.FIELD_COMPONENTS[which]
            h = self._h

            def h2d(buf, which=which):
                _lib.check(_lib.lib.lbswim_lattice_h2d(h, which, _lib.dptr(buf)))

            def d2h(buf, which=which):
                _lib.check(_lib.lib.lbswim_lattice_d2h(h, which, _lib.dptr(buf)))

            # rho, u and force (the fields a host loop reads and writes) keep
            # their host copy in page-locked memory up to 2 GB per field
            pinned = (which in (_lib.FIELD_RHO, _lib.FIELD_U, _lib.FIELD_FORCE)
                      and 8 * n <= (1 << 31))
            f = SharedLatticeArray(self, shared.Array(self, n, h2d, d2h, pinned=pinned))
            self._fields[which] = f
        return f

    @property
    def rho(self):
        return self._field(_lib.FIELD_RHO)

    @property
    def u(self):
        return self._field(_lib.FIELD_U)

    @property
    def force(self):
        return self._field(_lib.FIELD_FORCE)

    @property
    def fOld(self):
        return self._field(_lib.FIELD_FOLD)

    @property
    def fNew(self):
        return self._field(_lib.FIELD_FNEW)

    # -- pickle (lb.pyx:221-244): only time_step and fOld are saved --
    def __reduce__(self):
        size = self.addr.size
        p = self.params
        init_args = (size[0], size[1], size[2], p.tau_s, p.tau_b)
        if self._precision != _lib.F64:
            init_args = init_args + (self.precision,)
        self.fOld.D2H()
        return (self.__class__, init_args, (self.time_step, self.fOld.data.copy()))

    def __setstate__(self, data):
        ts, file_f_data = data
        _lib.check(_lib.lib.lbswim_lattice_set_time_step(self._h, int(ts)))
        my_f_data = self.fOld.data
        my_f_data[:] = file_f_data[:]
        self.fOld.H2D()
