"""Run-and-tumble swimmers (reference lbswim/swimmers.pyx, SwimmerArray.h)."""
import ctypes as C

import numpy as np

from . import _lib
from . import shared

_FIELDS = ("P", "l", "alpha", "mobility", "translational_advection_off",
           "rotational_advection_off", "seed")


class CommonParams:
    """Parameters shared by all swimmers of an array (swimmers.pyx:5-92).

    A free-standing CommonParams only holds values.  The ``common`` of a
    swimmer Array is bound to it: setting a property there updates the array
    at once, like the reference's property setters that call H2D.
    """

    def __init__(self):
        object.__setattr__(self, "_s", _lib.CommonParamsStruct())
        object.__setattr__(self, "_owner", None)

    def _adopt(self, owner):
        object.__setattr__(self, "_owner", owner)
        _lib.check(_lib.lib.lbswim_swimmers_get_common(owner._h, C.byref(self._s)))

    def _push(self):
        if self._owner is not None:
            _lib.check(_lib.lib.lbswim_swimmers_set_common(self._owner._h, C.byref(self._s)))

    def __getattr__(self, name):
        if name in _FIELDS:
            v = getattr(self._s, name)
            return bool(v) if name.endswith("_off") else v
        raise AttributeError(name)

    def __setattr__(self, name, value):
        if name not in _FIELDS:
            raise AttributeError("CommonParams has no field %r" % (name,))
        if name.endswith("_off"):
            value = int(bool(value))
        elif name == "seed":
            value = int(value)
        else:
            value = float(value)
        setattr(self._s, name, value)
        self._push()

    def H2D(self):
        self._push()

    def D2H(self):
        if self._owner is not None:
            _lib.check(_lib.lib.lbswim_swimmers_get_common(self._owner._h, C.byref(self._s)))

    def __reduce__(self):
        return (CommonParams, (), {k: getattr(self, k) for k in _FIELDS})

    def __setstate__(self, params):
        for k in _FIELDS:
            setattr(self._s, k, params[k] if k != "seed" else int(params[k]))
        self._push()


class Array:
    """An array of swimmers (swimmers.pyx:94-155; SwimmerArray.cu)."""

    def __init__(self, n, cp):
        self._h = None
        h = C.c_void_p()
        _lib.check(_lib.lib.lbswim_swimmers_create(int(n), C.byref(cp._s), C.byref(h)))
        self._h = h
        self.num = int(n)
        self._r = self._shared(_lib.SW_R)
        self._v = self._shared(_lib.SW_V)
        self._n = self._shared(_lib.SW_N)
        self._common = CommonParams()
        self._common._adopt(self)
        self.prng = shared.PrngArray(self)
        # As the reference's constructor does (SwimmerArray.cu:24), pull the
        # freshly seeded stream state so a later H2D() pushes it back intact.
        self.prng.D2H()

    def _shared(self, which):
        h = self._h

        def h2d(buf):
            _lib.check(_lib.lib.lbswim_swimmers_h2d(h, which, _lib.dptr(buf)))

        def d2h(buf):
            _lib.check(_lib.lib.lbswim_swimmers_d2h(h, which, _lib.dptr(buf)))

        a = shared.Array(self, 3 * self.num, h2d, d2h, pinned=True)
        a.view = a.view.reshape(3, self.num)
        return a

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            _lib.lib.lbswim_swimmers_destroy(h)
            self._h = None

    def init_random(self, lat, seed):
        """Positions uniform in lat's box, orientations uniform on the sphere,
        v = 0, made on the device from (seed, swimmer)."""
        _lib.check(_lib.lib.lbswim_swimmers_init_random(self._h, lat._h, int(seed)))

    def AddForces(self, lat):
        _lib.check(_lib.lib.lbswim_swimmers_add_forces(self._h, lat._h))

    def Move(self, lat):
        _lib.check(_lib.lib.lbswim_swimmers_move(self._h, lat._h))

    def H2D(self):
        self._r.H2D()
        self._v.H2D()
        self._n.H2D()
        self.prng.H2D()

    def D2H(self):
        # r, v and n in one call (one wait for the device), then the stream state
        bufs = [a.view.reshape(-1) for a in (self._r, self._v, self._n)]
        _lib.check(_lib.lib.lbswim_swimmers_d2h_all(self._h, *[_lib.dptr(b) for b in bufs]))
        self.prng.D2H()

    @property
    def r(self):
        return self._r

    @property
    def v(self):
        return self._v

    @property
    def n(self):
        return self._n

    @property
    def common(self):
        return self._common

    # The reference pickles (r, v, n) and re-seeds on load, so a resumed run
    # diverges (swimmers.pyx:143-155).  The random-stream state is appended
    # here, which makes resume exact; a 3-item state is still accepted.
    def __reduce__(self):
        self.D2H()
        data = (self._r.data.copy(), self._v.data.copy(), self._n.data.copy(),
                self.prng.data.copy())
        return (Array, (self.num, self._common), data)

    def __setstate__(self, data):
        r, v, n = data[:3]
        self._r.data[:] = r[:]
        self._v.data[:] = v[:]
        self._n.data[:] = n[:]
        if len(data) > 3:
            self.prng.data[:] = np.asarray(data[3], dtype=np.uint64)
        else:
            self.prng.D2H()
        self.H2D()
