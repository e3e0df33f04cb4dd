"""Precision study of the reduced-precision distribution storage.

The same seeded coupled problem is advanced with FP64 distributions (the
reference's precision) and with FP32, BF16 and FP16 deviation storage (FP32
collision in all three); the fields and swimmer positions are then compared
with the FP64 run.  Default problem: a 384^3 lattice, tau = 0.8,
rho = 1 + 1e-3 U[0, 1), u = 0; 262,144 swimmers in 16 arrays, each array with
its own P drawn from [5e-4, 2e-3] and alpha from [0, 0.05] (the swimmer
parameters of the reference are common to an array), l = 0.5, orientations
uniform on the sphere; 1,048,576 tracers; 1000 steps.  Smaller sizes scale the
particle counts with the volume.

    python precision_study.py [--size 384] [--steps 1000] [--out result.json]
"""
import argparse
import json
import os
import sys
import time

import numpy as np

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "gpu-swimmers_gb300"))
from lbswim import lb, swimmers, tracers  # noqa: E402
from lbswim.System import System  # noqa: E402


def problem(size, nsw_total, ntr, arrays, seed=42):
    rng = np.random.default_rng(seed)
    N = size ** 3
    box = float(size)
    rho = 1.0 + 1e-3 * rng.random(N)
    groups = []
    per = nsw_total // arrays
    for a in range(arrays):
        n = per + (1 if a < nsw_total % arrays else 0)
        nv = rng.standard_normal((3, n))
        nv /= np.linalg.norm(nv, axis=0, keepdims=True)
        groups.append({"n": n, "P": float(rng.uniform(5e-4, 2e-3)),
                       "alpha": float(rng.uniform(0.0, 0.05)), "seed": 1000 + a,
                       "r": rng.random((3, n)) * box, "nvec": nv})
    return {"size": size, "tau": 0.8, "rho": rho, "swimmers": groups,
            "tracers": rng.random((3, ntr)) * box}


def run(prob, precision, steps):
    s = prob["size"]
    lat = lb.Lattice(s, s, s, prob["tau"], prob["tau"], precision=precision)
    lat.rho[:] = prob["rho"].reshape(1, s, s, s)
    lat.rho.H2D()
    lat.u[:] = 0.0
    lat.u.H2D()
    lat.InitFromHydro()
    system = System(lat)
    arrs = []
    mobility = (1.0 / 0.1 - 1.0 / 1.5) / (6.0 * np.pi * prob["tau"] / 3.0)
    for g in prob["swimmers"]:
        cp = swimmers.CommonParams()
        cp.P, cp.l, cp.alpha, cp.mobility, cp.seed = g["P"], 0.5, g["alpha"], mobility, g["seed"]
        sw = swimmers.Array(g["n"], cp)
        sw.r[:] = g["r"]
        sw.n[:] = g["nvec"]
        sw.v[:] = 0.0
        sw.H2D()
        system.AddThing(sw)
        arrs.append(sw)
    tr = tracers.Array(prob["tracers"].shape[1])
    tr.r[:] = prob["tracers"]
    tr.s[:] = 0.0
    tr.v[:] = 0.0
    tr.H2D()
    system.AddThing(tr)
    t0 = time.perf_counter()
    system.Step(steps)
    lat.synchronize()
    dt = time.perf_counter() - t0
    lat.rho.D2H()
    lat.u.D2H()
    rho = lat.rho.data.reshape(-1).copy()
    u = lat.u.data.reshape(3, -1).copy()
    pos = []
    for sw in arrs:
        sw.D2H()
        pos.append(sw.r.data.copy())
    tr.D2H()
    out = {"rho": rho, "u": u, "sw_r": np.concatenate(pos, axis=1), "tr_r": tr.r.data.copy(),
           "seconds": dt, "mass_momentum": lat.conservation()}
    del system, arrs, tr, lat
    return out


def periodic_max(a, b, size):
    d = (a - b + size / 2.0) % size - size / 2.0
    return float(np.abs(d).max())


def compare(ref, got, size):
    drho_ref = ref["rho"] - ref["rho"].mean()
    return {
        "rho_rel_l2": float(np.linalg.norm(got["rho"] - ref["rho"]) / np.linalg.norm(ref["rho"])),
        "rho_dev_rel_l2": float(np.linalg.norm(got["rho"] - ref["rho"]) / np.linalg.norm(drho_ref)),
        "u_rel_l2": float(np.linalg.norm(got["u"] - ref["u"]) / np.linalg.norm(ref["u"])),
        "swimmer_pos_max_err": periodic_max(got["sw_r"], ref["sw_r"], size),
        "tracer_pos_max_err": periodic_max(got["tr_r"], ref["tr_r"], size),
        "seconds": got["seconds"],
    }


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--size", type=int, default=384)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--arrays", type=int, default=16)
    ap.add_argument("--precisions", default="f32,bf16,f16")
    ap.add_argument("--out", default=None)
    a = ap.parse_args(argv)
    f = (a.size / 384.0) ** 3
    prob = problem(a.size, max(a.arrays, int(round(262144 * f))), max(1, int(round(1048576 * f))),
                   a.arrays)
    ref = run(prob, "f64", a.steps)
    result = {"size": a.size, "steps": a.steps, "swimmers": sum(g["n"] for g in prob["swimmers"]),
              "swimmer_arrays": a.arrays, "tracers": prob["tracers"].shape[1],
              "f64_seconds": ref["seconds"], "f64_mass_momentum": ref["mass_momentum"],
              "against_f64": {}}
    for p in a.precisions.split(","):
        got = run(prob, p, a.steps)
        result["against_f64"][p] = compare(ref, got, float(a.size))
        result["against_f64"][p]["mass_momentum"] = got["mass_momentum"]
    text = json.dumps(result, indent=1)
    if a.out:
        with open(a.out, "w") as fh:
            fh.write(text)
    print(text)
    return result


if __name__ == "__main__":
    main()
