"""Batched ensembles of independent FP32 solves (no reference counterpart).

An Ensemble advances many (Lattice, swimmers.Array or None, tracers.Array or
None) members by the coupled step of System.Step -- ZeroForce, AddForces,
Step, CalcHydro, Move -- with a few batched launches per step replayed from a
CUDA graph.  Each member ends exactly where its own System.Step would have
taken it.  Members are ordinary objects of this package: set them up and read
them back with their usual methods.
"""
import ctypes as C

from . import _lib


class Ensemble:
    def __init__(self, members=()):
        h = C.c_void_p()
        _lib.check(_lib.lib.lbswim_ensemble_create(C.byref(h)))
        self._h = h
        self._members = []
        self.set_members(members)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and _lib.lib is not None:
            _lib.lib.lbswim_ensemble_destroy(h)
            self._h = None

    @property
    def members(self):
        return list(self._members)

    def set_members(self, members):
        """Replace the membership by a list of (lattice, swimmers or None,
        tracers or None); the objects must stay alive while they are members.
        A member's swimmer array holds at most 32767 swimmers (2047 when an
        axis of its lattice is shorter than 4 sites)."""
        members = [tuple(m) + (None,) * (3 - len(m)) for m in members]
        n = len(members)
        arr = C.c_void_p * max(n, 1)
        lat = arr(*[m[0]._h for m in members])
        sw = arr(*[(m[1]._h if m[1] is not None else None) for m in members])
        tr = arr(*[(m[2]._h if m[2] is not None else None) for m in members])
        _lib.check(_lib.lib.lbswim_ensemble_set_members(self._h, lat, sw, tr, n))
        self._members = members

    def Step(self, nsteps=1, limits=None):
        """nsteps batched steps; with `limits` (one int per member, in
        membership order) member m takes only the first limits[m] of them."""
        if limits is None:
            _lib.check(_lib.lib.lbswim_ensemble_step(self._h, int(nsteps)))
            return
        if len(limits) != len(self._members):
            raise ValueError("one limit per member")
        arr = (C.c_int * max(1, len(limits)))(*[int(x) for x in limits])
        _lib.check(_lib.lib.lbswim_ensemble_step_limited(self._h, int(nsteps), arr))

    def autotune(self):
        """Pick the faster slab shape per lattice shape (timed on scratch copies)."""
        _lib.check(_lib.lib.lbswim_ensemble_autotune(self._h))
