"""Drive a seeded workload through the lbswim Python API (the drop-in surface)."""
import numpy as np

from lbswim import lb, swimmers, tracers
from lbswim.System import System


def build_gpu(case, precision="f64", compat=None):
    nx, ny, nz = case["size"]
    N = nx * ny * nz
    lat = lb.Lattice(nx, ny, nz, case["tau_s"], case["tau_b"], precision=precision)
    if compat is not None:
        lat.set_compat(compat)
    lat.rho[:] = np.broadcast_to(case["rho"], (N,)).reshape(1, nx, ny, nz)
    lat.rho.H2D()
    lat.u[:] = np.broadcast_to(case["u"], (3, N)).reshape(3, nx, ny, nz)
    lat.u.H2D()
    lat.ZeroForce()
    system = System(lat)
    sw = tr = None
    s = case.get("swimmers")
    if s is not None and s["n"] > 0:
        cp = swimmers.CommonParams()
        for k in ("P", "l", "alpha", "mobility", "translational_advection_off",
                  "rotational_advection_off", "seed"):
            setattr(cp, k, s.get(k, False) if k.endswith("_off") else s[k])
        sw = swimmers.Array(s["n"], cp)
        sw.r[:] = s["r"]
        sw.n[:] = s["nvec"]
        sw.v[:] = s["v"]
        sw.H2D()
        system.AddThing(sw)
    t = case.get("tracers")
    if t is not None and t["n"] > 0:
        tr = tracers.Array(t["n"])
        tr.r[:] = t["r"]
        tr.v[:] = t["v"]
        tr.s[:] = 0.0
        tr.H2D()
        system.AddThing(tr)
    lat.InitFromHydro()
    return lat, sw, tr, system


def snapshot(lat, sw, tr):
    N = lat.addr.n
    out = {}
    for name in ("rho", "u", "force", "fOld"):
        f = getattr(lat, name)
        f.D2H()
        out["f" if name == "fOld" else name] = f.data.reshape(-1, N).copy()
    out["rho"] = out["rho"][0]
    if sw is not None:
        sw.D2H()
        out.update(sw_r=sw.r.data.copy(), sw_v=sw.v.data.copy(), sw_n=sw.n.data.copy())
    if tr is not None:
        tr.D2H()
        out.update(tr_r=tr.r.data.copy(), tr_v=tr.v.data.copy(), tr_s=tr.s.data.copy())
    return out
