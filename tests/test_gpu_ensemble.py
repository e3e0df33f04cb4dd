"""Batched ensembles: each member ends where its own System.Step takes it.

The batched kernels run the same per-slab and per-block code as the
single-lattice path, so with the same slab shape the results agree bit for
bit; against FP64 one-at-a-time solves the FP32 velocity fields agree to the
stated 1e-5 relative L2.
"""
import numpy as np
import pytest

import oracle as O
from gpu_harness import build_gpu, snapshot
from helpers import rel_l2

pytestmark = pytest.mark.gpu

SPECS = [((16, 16, 16), 0, 64, 0.7, 1),
         ((24, 24, 24), 12, 300, 1.1, 2),
         ((32, 16, 48), 40, 0, 0.9, 3),
         ((20, 12, 40), 3, 150, 1.4, 4),
         ((9, 7, 5), 5, 30, 0.8, 5)]


def _case(size, nsw, ntr, tau, seed):
    return O.random_case(size, nsw, ntr, seed=seed, tau_s=tau, tau_b=tau, u_amp=0.01,
                         alpha=0.1, P=2e-3, l=0.4)


def _build(specs, precision="f32"):
    out = []
    for size, nsw, ntr, tau, seed in specs:
        out.append(build_gpu(_case(size, nsw, ntr, tau, seed), precision))
    return out


def _same(a, b):
    sa, sb = snapshot(*a[:3]), snapshot(*b[:3])
    for k in sa:
        assert np.array_equal(sa[k], sb[k]), k


def test_members_match_their_own_system_step():
    from lbswim.ensemble import Ensemble
    batched, alone = _build(SPECS), _build(SPECS)
    for b, a in zip(batched, alone):
        a[0].tile = b[0].tile
    ens = Ensemble([(lat, sw, tr) for lat, sw, tr, _ in batched])
    ens.Step(7)   # odd: the one-step graph too
    ens.Step(6)
    for a in alone:
        a[3].Step(13)
    for b, a in zip(batched, alone):
        assert b[0].time_step == a[0].time_step == 13
        _same(b, a)


def test_membership_changes_between_runs():
    from lbswim.ensemble import Ensemble
    batched, alone = _build(SPECS), _build(SPECS)
    for b, a in zip(batched, alone):
        a[0].tile = b[0].tile
    ens = Ensemble([(lat, sw, tr) for lat, sw, tr, _ in batched[:3]])
    ens.Step(4)
    ens.set_members([(lat, sw, tr) for lat, sw, tr, _ in batched[1:]])  # one leaves, two join
    ens.Step(5)
    steps = [4, 9, 9, 5, 5]
    for a, n in zip(alone, steps):
        a[3].Step(n)
    for b, a in zip(batched, alone):
        _same(b, a)


def test_autotuned_tiles_keep_results():
    from lbswim.ensemble import Ensemble
    batched = _build(SPECS[:3])
    ens = Ensemble([(lat, sw, tr) for lat, sw, tr, _ in batched])
    ens.autotune()
    alone = _build(SPECS[:3])
    for b, a in zip(batched, alone):
        assert b[0].tile in (0, 1)
        a[0].tile = b[0].tile
    ens.Step(8)
    for a in alone:
        a[3].Step(8)
    for b, a in zip(batched, alone):
        _same(b, a)


def test_fp32_ensemble_velocity_within_1e5_of_fp64():
    # members drawn from the batched-ensemble distribution (shapes 16^3 ..
    # 48x48x96, tau in [0.6, 1.5], up to 512 swimmers and 4096 tracers, fluid
    # at rest at the start): the batched FP32 solves against the same solves in
    # plain FP64 after 1000 steps, velocity-field relative L2 <= 1e-5
    from lbswim import serve
    from lbswim.ensemble import Ensemble
    from lbswim.System import System
    rng = np.random.default_rng(2024)
    specs = [serve.draw_spec(rng) for _ in range(6)]
    batched = [serve.build_solve(sp, "f32") for sp in specs]
    ens = Ensemble(batched)
    ens.Step(1000)
    for (lat32, _, _), sp in zip(batched, specs):
        lat, sw, tr = serve.build_solve(sp, "f64")
        system = System(lat)
        system.AddThing(sw)
        if tr is not None:
            system.AddThing(tr)
        system.Step(1000)
        lat.u.D2H()
        lat32.u.D2H()
        lat.rho.D2H()
        lat32.rho.D2H()
        assert lat32.time_step == lat.time_step == 1000
        assert rel_l2(lat32.u.data, lat.u.data) <= 1e-5, sp.shape
        assert rel_l2(lat32.rho.data, lat.rho.data) <= 1e-6, sp.shape


def test_fp32_ensemble_decaying_flow_within_1e5_of_fp64():
    # a random initial velocity decaying over 200 steps (its relative error
    # grows as the flow dies away): batched FP32 against FP64 one at a time
    from lbswim.ensemble import Ensemble
    specs = SPECS[:4]
    batched = _build(specs)
    ens = Ensemble([(lat, sw, tr) for lat, sw, tr, _ in batched])
    ens.Step(200)
    for b, spec in zip(batched, specs):
        ref = build_gpu(_case(*spec), "f64")
        ref[3].Step(200)
        gs, rs = snapshot(*b[:3]), snapshot(*ref[:3])
        assert rel_l2(gs["u"], rs["u"]) < 1e-5
        assert rel_l2(gs["rho"], rs["rho"]) < 1e-6


def test_member_swimmer_limit():
    # a member takes at most 32767 swimmers (2047 on a lattice with an axis
    # shorter than 4 sites): beyond that its force sums could leave the split form
    from lbswim import _lib, lb, swimmers
    from lbswim.ensemble import Ensemble
    ens = Ensemble()
    for size, ok, bad in (((8, 8, 8), 32767, 32768), ((3, 8, 8), 2047, 2048)):
        lat = lb.Lattice(*size, 0.8, 0.8, precision="f32")
        for n, fine in ((ok, True), (bad, False)):
            sw = swimmers.Array(n, swimmers.CommonParams())
            if fine:
                ens.set_members([(lat, sw)])
                ens.set_members([])
            else:
                with pytest.raises(_lib.LbswimError, match="32767 swimmers"):
                    ens.set_members([(lat, sw)])


def test_members_with_step_limits_stop_where_their_own_steps_end():
    # a run of 9 batched steps in which members take 9, 4, 0, 7 and 1 of them:
    # each ends exactly where its own System.Step of that many steps ends,
    # and one that took none is untouched
    from lbswim.ensemble import Ensemble
    batched, alone = _build(SPECS), _build(SPECS)
    for b, a in zip(batched, alone):
        a[0].tile = b[0].tile
    limits = [9, 4, 0, 7, 1]
    ens = Ensemble([(lat, sw, tr) for lat, sw, tr, _ in batched])
    ens.Step(9, limits=limits)
    ens.Step(3)  # then everyone goes on together
    for a, n in zip(alone, limits):
        a[3].Step(n + 3)
    for b, a, n in zip(batched, alone, limits):
        assert b[0].time_step == a[0].time_step == n + 3
        _same(b, a)
