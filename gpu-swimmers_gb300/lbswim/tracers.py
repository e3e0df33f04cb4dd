"""Passive tracers (reference lbswim/tracers.pyx, TracerArray.h)."""
import ctypes as C

from . import _lib
from . import shared


class Array:
    """An array of tracer particles advected by the fluid (tracers.pyx:5-57)."""

    def __init__(self, n):
        self._h = None
        h = C.c_void_p()
        _lib.check(_lib.lib.lbswim_tracers_create(int(n), C.byref(h)))
        self._h = h
        self.num = int(n)
        self._r = self._shared(_lib.TR_R)
        self._s = self._shared(_lib.TR_S)
        self._v = self._shared(_lib.TR_V)

    def _shared(self, which):
        h = self._h

        def h2d(buf):
            _lib.check(_lib.lib.lbswim_tracers_h2d(h, which, _lib.dptr(buf)))

        def d2h(buf):
            _lib.check(_lib.lib.lbswim_tracers_d2h(h, which, _lib.dptr(buf)))

        a = shared.Array(self, 3 * self.num, h2d, d2h, pinned=True)
        a.view = a.view.reshape(3, self.num)
        return a

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            _lib.lib.lbswim_tracers_destroy(h)
            self._h = None

    def AddForces(self, lat):
        """Tracers exert no force (tracers.pyx:20-21)."""

    def init_random(self, lat, seed):
        """Positions uniform in lat's box, s = v = 0, made on the device."""
        _lib.check(_lib.lib.lbswim_tracers_init_random(self._h, lat._h, int(seed)))

    def Move(self, lat):
        _lib.check(_lib.lib.lbswim_tracers_move(self._h, lat._h))

    def H2D(self):
        self._r.H2D()
        self._s.H2D()
        self._v.H2D()

    def D2H(self):
        self._r.D2H()
        self._s.D2H()
        self._v.D2H()

    @property
    def r(self):
        return self._r

    @property
    def s(self):
        return self._s

    @property
    def v(self):
        return self._v

    def __reduce__(self):
        self.D2H()
        return (Array, (self.num,), (self._r.data.copy(), self._s.data.copy(),
                                     self._v.data.copy()))

    def __setstate__(self, data):
        r, s, v = data
        self._r.data[:] = r[:]
        self._s.data[:] = s[:]
        self._v.data[:] = v[:]
        self.H2D()
