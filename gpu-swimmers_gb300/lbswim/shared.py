"""Host mirrors of device arrays (reference lbswim/shared.pyx:6-66).

A ``shared.Array`` owns a float64 numpy buffer, the host copy, and knows how to
copy it to and from one device field through the C ABI.  As in the
reference, numpy views of the host copy are handed out directly, and nothing
moves between host and device unless H2D() or D2H() is called.
"""
import numpy as np

from . import _lib


class Array:
    """Host copy of a device array (shared.pyx:6-35)."""

    def __init__(self, owner, size, h2d, d2h, pinned=False):
        """pinned: hold the host copy in page-locked memory (particle arrays,
        which are copied every step in typical loops)."""
        self.owner = owner
        self._h2d = h2d
        self._d2h = d2h
        self.view = None
        if pinned:
            try:
                self.view = _lib.pinned_zeros(size)
            except _lib.LbswimError:  # no page-locked memory left: pageable
                self.view = None
        if self.view is None:
            self.view = np.zeros(int(size), dtype=np.float64)

    def init(self, owner, sa):  # reference-style construction hook
        return self

    @property
    def data(self):
        return self.view

    def H2D(self):
        self._h2d(np.ascontiguousarray(self.view.reshape(-1)))

    def D2H(self):
        buf = self.view.reshape(-1)
        if buf.base is not None and not buf.flags.c_contiguous:
            raise RuntimeError("host view is not contiguous")
        self._d2h(buf)

    def __getattr__(self, attr):
        if attr in ("view", "owner", "_h2d", "_d2h"):
            raise AttributeError(attr)
        return getattr(self.view, attr)

    def __getitem__(self, idx):
        return self.view[idx]

    def __setitem__(self, idx, val):
        self.view[idx] = val

    def __len__(self):
        return len(self.view)

    def __array__(self, dtype=None, copy=None):
        return np.asarray(self.view, dtype=dtype)


class PrngArray:
    """Random-stream state of a swimmer array (shared.pyx:37-66).

    The reference stores one cuRAND XORWOW state per swimmer.  Here the stream
    is counter based, keyed by (seed, swimmer, move step), so the whole state
    is the seed and the next move step: ``data`` is a uint64 array [seed, step].
    """

    def __init__(self, swimmers):
        self.owner = swimmers
        self.view = np.zeros(2, dtype=np.uint64)

    @property
    def data(self):
        return self.view

    def D2H(self):
        seed, step = _lib.C.c_ulonglong(), _lib.C.c_ulonglong()
        _lib.check(_lib.lib.lbswim_swimmers_get_rng(self.owner._h, _lib.C.byref(seed),
                                                    _lib.C.byref(step)))
        self.view[:] = (seed.value, step.value)

    def H2D(self):
        _lib.check(_lib.lib.lbswim_swimmers_set_rng(self.owner._h, int(self.view[0]),
                                                    int(self.view[1])))

    def __getitem__(self, idx):
        return self.view[idx]

    def __setitem__(self, idx, val):
        self.view[idx] = val
