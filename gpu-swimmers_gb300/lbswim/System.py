"""Coupled step driver (reference lbswim/System.py:1-17).

``Step()`` runs ZeroForce, every thing's AddForces, Step, CalcHydro and every
thing's Move.  When all things are swimmer and tracer arrays of this package,
the whole sequence is one call into the library (lbswim_system_step), in the
same order; other objects are called one method at a time as in the reference.
"""
import ctypes as C

from . import _lib
from . import swimmers as _sw
from . import tracers as _tr


class System:
    def __init__(self, lat):
        self.lat = lat
        self.things = []

    def AddThing(self, th):
        self.things.append(th)

    def _native(self):
        sw = [t for t in self.things if type(t) is _sw.Array]
        tr = [t for t in self.things if type(t) is _tr.Array]
        if len(sw) + len(tr) != len(self.things):
            return None
        # AddForces of tracers is a no-op and swimmers move before tracers only
        # if they come first in the list; keep the reference's order exactly.
        seen_tracer = False
        for t in self.things:
            if type(t) is _tr.Array:
                seen_tracer = True
            elif seen_tracer:
                return None
        return sw, tr

    def Step(self, nsteps=1):
        native = self._native()
        if native is not None:
            sw, tr = native
            swa = (C.c_void_p * max(len(sw), 1))(*[t._h for t in sw])
            tra = (C.c_void_p * max(len(tr), 1))(*[t._h for t in tr])
            _lib.check(_lib.lib.lbswim_system_step(self.lat._h, swa, len(sw), tra, len(tr),
                                                   int(nsteps)))
            return
        for _ in range(int(nsteps)):
            self.lat.ZeroForce()
            for th in self.things:
                th.AddForces(self.lat)
            self.lat.Step()
            self.lat.CalcHydro()
            for th in self.things:
                th.Move(self.lat)
