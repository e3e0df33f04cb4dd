"""Shared helpers for the test suite (comparison metrics, golden loading)."""
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")

# FP64 parity tolerance: relative error of the reference's own implementation.
TOL_F64 = 1e-12


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))


def rel_l2_maxnorm(a, b):
    """RMS of a - b over max |b|: relative L2 of a field normalised by its
    largest magnitude, for fields such as u that are ~0 in places."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    mb = np.max(np.abs(b))
    return float(np.sqrt(np.mean((a - b) ** 2)) / (mb if mb > 0 else 1.0))


def rel_max(a, b):
    """max |a - b| / max |b| (for fields such as u that are ~0 in places)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    mb = np.max(np.abs(b))
    return float(np.max(np.abs(a - b)) / (mb if mb > 0 else 1.0))


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


GOLDEN_CASES = ["c0_readme", "rand_small", "rand_trans_off", "ragged_tiny", "c1_density_32"]


def golden_case(name):
    """Workload of a golden fixture, rebuilt from its recorded recipe."""
    import oracle as O
    table = {
        "c0_readme": lambda: O.readme_case(),
        "rand_small": lambda: O.random_case((8, 12, 16), 20, 300, seed=5, u_amp=0.02, alpha=0.3,
                                            tau_s=0.7, tau_b=1.1),
        "rand_trans_off": lambda: O.random_case((12, 8, 10), 12, 200, seed=11, alpha=0.05,
                                                trans_off=True, tau_s=0.6, tau_b=0.9),
        "ragged_tiny": lambda: O.random_case((5, 7, 3), 6, 40, seed=23, u_amp=0.01, alpha=0.2,
                                             P=3e-3, l=0.3),
        "c1_density_32": lambda: O.random_case((32, 32, 32), 128, 2048, seed=42),
    }
    return table[name]()
