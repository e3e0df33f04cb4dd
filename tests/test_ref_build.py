"""The reference's own kernels build for the host from their sources and the
oracle restatement agrees with them bit for bit on fresh seeded cases."""
import numpy as np
import pytest

import build_ref
import oracle as O

REF = build_ref.reference_root()
pytestmark = pytest.mark.skipif(REF is None, reason="reference sources not present")


@pytest.fixture(scope="module")
def ref_built():
    build_ref.build(REF, quiet=True)
    O._ref = None
    return True


@pytest.mark.parametrize("seed", [101, 202])
def test_oracle_bit_exact_vs_reference(ref_built, seed):
    rng = np.random.default_rng(seed)
    size = tuple(int(x) for x in rng.integers(3, 13, size=3))
    case = O.random_case(size, int(rng.integers(1, 9)), int(rng.integers(0, 60)), seed=seed,
                         u_amp=0.01, alpha=0.25, tau_s=float(rng.uniform(0.55, 1.4)),
                         tau_b=float(rng.uniform(0.55, 1.4)))
    a = O.make_system(case)
    b = O.make_ref_system(case)
    a.step(15)
    b.step(15)
    sa, sb = a.snapshot(), b.snapshot()
    for k in sb:
        assert np.array_equal(sa[k], sb[k]), k
