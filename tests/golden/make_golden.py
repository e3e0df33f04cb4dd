"""Generate the golden fixtures in tests/golden/ from the reference itself.

The reference's own kernels (rupertnash/gpu-swimmers lbswim/liblbswim/*.cu)
are built for the host by oracle/build_ref.py and driven in the order of the
reference's README / System.py.  Each fixture stores, per snapshot step:

* SHA-256 digests of the full FP64 arrays (rho, u, force, f, particle state),
  which pin the oracle restatement bit for bit;
* the values at a fixed seeded subset of sites and particles, which the GPU
  tests compare against within tolerance.

Run from the repository root:  python tests/golden/make_golden.py
"""
import hashlib
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import build_ref  # noqa: E402
import oracle as O  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
SUBSET = 384


def cases():
    return {
        # README example (BASELINE config 0): 16^3, one swimmer, 4096 tracers.
        "c0_readme": (O.readme_case(), [1, 10, 100, 1000]),
        # Non-cubic lattice, non-zero initial u (exercises lb.cu:356), tumbles.
        "rand_small": (O.random_case((8, 12, 16), 20, 300, seed=5, u_amp=0.02, alpha=0.3,
                                     tau_s=0.7, tau_b=1.1), [1, 50]),
        # Translational advection off.
        "rand_trans_off": (O.random_case((12, 8, 10), 12, 200, seed=11, alpha=0.05,
                                         trans_off=True, tau_s=0.6, tau_b=0.9), [1, 25]),
        # Tiny ragged lattice: every stencil wraps.
        "ragged_tiny": (O.random_case((5, 7, 3), 6, 40, seed=23, u_amp=0.01, alpha=0.2,
                                      P=3e-3, l=0.3), [1, 30]),
        # 32^3 with the swimmer / tracer densities of the 256^3 configuration.
        "c1_density_32": (O.random_case((32, 32, 32), 128, 2048, seed=42), [1, 20]),
    }


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.float64).tobytes()).hexdigest()


def main():
    build_ref.build()
    for name, (case, snaps) in cases().items():
        ref = O.make_ref_system(case, threads=1)
        N = ref.N
        rng = np.random.default_rng(1000 + len(name))
        sites = np.sort(rng.choice(N, size=min(SUBSET, N), replace=False))
        nsw = case["swimmers"]["n"]
        ntr = case["tracers"]["n"]
        tsel = np.sort(rng.choice(ntr, size=min(SUBSET, ntr), replace=False))
        out = {"sites": sites, "tracers": tsel, "snaps": np.array(snaps)}
        done = 0
        for t in snaps:
            ref.step(t - done)
            done = t
            s = ref.snapshot()
            for key, arr in s.items():
                out["%s@%d#sha" % (key, t)] = np.array(digest(arr))
            out["rho@%d" % t] = s["rho"][sites]
            out["u@%d" % t] = s["u"][:, sites]
            out["force@%d" % t] = s["force"][:, sites]
            out["f@%d" % t] = s["f"][:, sites]
            if nsw:
                for key in ("sw_r", "sw_v", "sw_n"):
                    out["%s@%d" % (key, t)] = s[key]
            if ntr:
                for key in ("tr_r", "tr_v"):
                    out["%s@%d" % (key, t)] = s[key][:, tsel]
        path = os.path.join(OUT, name + ".npz")
        np.savez_compressed(path, **out)
        print("wrote", path, os.path.getsize(path))

    # Peskin delta and stencil interpolation known answers.
    L = O.ref_lib()
    L.ref_peskin_delta.restype = O.C.c_double
    L.ref_peskin_delta.argtypes = [O.C.c_double]
    xs = np.concatenate([np.linspace(-2.5, 2.5, 101), [-2.0, -1.0, 0.0, 1.0, 2.0, 1e-300,
                                                      0.5 - 1e-12, 1.0 - 1e-15, 1.999999999]])
    phi = np.array([L.ref_peskin_delta(float(x)) for x in xs])
    np.savez_compressed(os.path.join(OUT, "peskin.npz"), x=xs, phi=phi)
    print("wrote peskin.npz")


if __name__ == "__main__":
    main()
