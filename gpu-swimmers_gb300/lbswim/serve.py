"""Serving many independent solves on one GPU (no reference counterpart).

A solve is a lattice with its swimmers and tracers advanced a requested
number of coupled steps.  `Server` keeps a batched Ensemble of the solves in
flight: arrivals are admitted while their device memory fits an HBM budget,
every solve in flight advances in the same batched launches, and a solve
leaves the batch (its slot and memory freed) as soon as it has done its
steps; solves that arrive while others run join at the next chunk of steps.
`serve_one_at_a_time` is the plain counterpart: one solve at a time, in
arrival order, through System.Step.

Solves are drawn from the batched-ensemble distribution: lattice shapes from
16^3 to 48x48x96 (96^3 and 128^3 added for serving), tau uniform in
[0.6, 1.5], a swimmer count log-uniform in [1, 512] with P in [1e-4, 1e-3]
and alpha in [0, 0.05], orientations uniform on the sphere, and a tracer
count uniform in [0, 4096].  Initial density 1 + 1e-3 U[0, 1), velocity 0.
"""
import collections
import math
import time

import numpy as np

from . import _lib, lb, swimmers, tracers
from .ensemble import Ensemble
from .System import System

ENSEMBLE_SHAPES = [(16, 16, 16), (24, 24, 24), (32, 32, 32), (48, 48, 48), (64, 64, 64),
                   (32, 32, 64), (48, 48, 96)]
SERVING_SHAPES = ENSEMBLE_SHAPES + [(96, 96, 96), (128, 128, 128)]


class Spec:
    """One solve: lattice shape, relaxation time, particles and seeds."""

    def __init__(self, shape, tau, nsw, P, alpha, ntr, seed, steps=0, l=0.5):
        self.shape, self.tau, self.nsw, self.P, self.alpha = tuple(shape), tau, nsw, P, alpha
        self.ntr, self.seed, self.steps, self.l = ntr, seed, steps, l

    @property
    def sites(self):
        return self.shape[0] * self.shape[1] * self.shape[2]

    def device_bytes(self, precision="f32"):
        """Device memory of the solve: two f buffers, velocity buffers, force,
        slab buckets, dipole-end records and particles."""
        n = self.sites
        fb = {"f64": 8, "f32": 4}.get(precision, 2)
        per_site = 2 * 15 * fb + (56 if precision == "f64" else 2 * 16 + 12)
        slabs = math.ceil(self.shape[0] / 32) * math.ceil(self.shape[1] / 8) * \
            math.ceil(self.shape[2] / 32) + 64
        return n * per_site + slabs * 4096 + self.nsw * 300 + self.ntr * 200 + (1 << 16)


def draw_spec(rng, shapes=ENSEMBLE_SHAPES, steps_range=None):
    shape = shapes[rng.integers(len(shapes))]
    nsw = int(math.floor(math.exp(rng.uniform(0.0, math.log(512.0)))))
    steps = 0
    if steps_range:
        lo, hi = steps_range
        steps = int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))
    return Spec(shape, float(rng.uniform(0.6, 1.5)), max(1, min(512, nsw)),
                float(rng.uniform(1e-4, 1e-3)), float(rng.uniform(0.0, 0.05)),
                int(rng.integers(0, 4097)), int(rng.integers(1, 2**31)), steps)


def build_solve(spec, precision="f32", lattice=None):
    """Device objects of a solve, initialised on the device from its seed
    (rho = 1 + 1e-3 U[0, 1), u = 0, particles uniform in the box, swimmer
    orientations uniform on the sphere).  `lattice`, of the solve's shape and
    precision, is reused when given."""
    nx, ny, nz = spec.shape
    if lattice is None:
        lat = lb.Lattice(nx, ny, nz, spec.tau, spec.tau, precision=precision)
    else:
        lat = lattice
        lat.set_tau(spec.tau, spec.tau)
        _lib.check(_lib.lib.lbswim_lattice_set_time_step(lat._h, 0))
    lat.init_random(spec.seed)
    cp = swimmers.CommonParams()
    cp.P = spec.P
    cp.l = spec.l
    cp.alpha = spec.alpha
    cp.mobility = (1.0 / 0.1 - 1.0 / 1.5) / (6.0 * np.pi * spec.tau / 3.0)
    cp.seed = spec.seed
    sw = swimmers.Array(spec.nsw, cp)
    sw.init_random(lat, spec.seed)
    tr = None
    if spec.ntr > 0:
        tr = tracers.Array(spec.ntr)
        tr.init_random(lat, spec.seed + 1)
    return lat, sw, tr


def poisson_trace(rng, rate, duration, shapes=SERVING_SHAPES, steps_range=(100, 5000)):
    """Arrival times of a Poisson stream and the solve of each arrival."""
    t, out = 0.0, []
    while True:
        t += float(rng.exponential(1.0 / rate))
        if t >= duration:
            return out
        out.append((t, draw_spec(rng, shapes, steps_range)))


class _Job:
    def __init__(self, arrival, spec, objs, nbytes):
        self.arrival, self.spec, self.objs, self.bytes = arrival, spec, objs, nbytes
        self.remaining = spec.steps
        self.admitted = None


def spec_problem(spec):
    """Why a request cannot be served at all (None when it can): a malformed
    spec is rejected on arrival, before anything is allocated."""
    try:
        shape = tuple(int(x) for x in spec.shape)
        if len(shape) != 3 or min(shape) < 1 or shape[0] > 65535:
            return "bad lattice shape %r" % (spec.shape,)
        if not (math.isfinite(spec.tau) and spec.tau > -0.5):
            return "bad relaxation time %r" % (spec.tau,)
        if int(spec.steps) < 1:
            return "bad step count %r" % (spec.steps,)
        if not (0 <= int(spec.nsw) <= 32767 and 0 <= int(spec.ntr)):
            return "bad particle counts %r, %r" % (spec.nsw, spec.ntr)
        if int(spec.nsw) > 2047 and min(shape) < 4:
            return "too many swimmers for a lattice axis shorter than 4 sites"
        if not all(math.isfinite(v) for v in (spec.P, spec.alpha, spec.l)):
            return "non-finite swimmer parameters"
    except (TypeError, ValueError, AttributeError) as e:
        return "malformed request: %s" % e
    return None


def _is_alloc_failure(exc):
    return isinstance(exc, MemoryError) or (
        isinstance(exc, _lib.LbswimError) and exc.code == -3)


def read_result(objs):
    """The state a served solve returns to its client (read back to the host):
    the velocity field u [3, nx, ny, nz] and the swimmers' r, v, n [3, n] (as
    swimmers.Array.D2H gives them, swimmers.pyx:123-127) and the tracers' r,
    s, v."""
    lat, sw, tr = (tuple(objs) + (None, None))[:3]
    lat.u.D2H()
    out = {"u": lat.u.data.copy(), "time_step": lat.time_step}
    if sw is not None:
        sw.D2H()
        out.update(sw_r=sw.r.data.copy(), sw_v=sw.v.data.copy(), sw_n=sw.n.data.copy())
    if tr is not None:
        tr.D2H()
        out.update(tr_r=tr.r.data.copy(), tr_s=tr.s.data.copy(), tr_v=tr.v.data.copy())
    return out


class Server:
    """Continuous batching of solves under an HBM budget.

    A solve is admitted (in arrival order) while its device memory fits the
    budget and the sites in flight stay within `max_sites` (beyond the point
    where the GPU is full, more solves in the batch only lengthen every
    solve's time).  Lattices of finished solves are kept, per shape, for the
    next solve of that shape; kept lattices count against the budget and are
    released when a solve of another shape needs the memory.

    Faults stay with the request that caused them: a malformed request, or one
    that needs more device memory than the whole budget, is rejected with its
    reason; an allocation that fails when a solve is admitted frees the kept
    lattices and retries, and otherwise leaves the request waiting for memory
    (or rejects it when nothing else holds memory); a request can be
    cancelled while it waits or runs.  The serving loop goes on in every case.

    build: (spec, precision, lattice) -> (lattice, swimmers, tracers), and
    ensemble: the batched stepper, default the device ones (tests pass fakes).
    readback: each finished solve's state (read_result) is copied to the host
    before its latency is taken; True returns it with the solve's record, a
    callable receives (trace index, result) instead (a client hand-off that
    keeps nothing in the server)."""

    def __init__(self, budget_bytes, chunk=64, precision="f32", autotune=True,
                 max_sites=64 << 20, readback=False, build=None, ensemble=None):
        self.budget, self.chunk, self.precision = budget_bytes, chunk, precision
        self.autotune, self.max_sites, self.readback = autotune, max_sites, readback
        self.build = build or (lambda spec, prec, lattice=None:
                               build_solve(spec, prec, lattice=lattice))
        self.ens = ensemble if ensemble is not None else Ensemble()
        self.pool = collections.defaultdict(list)  # shape -> [(lattice, bytes)]

    def run(self, trace, duration, drain=False, keep=None, cancel=None):
        """Serve `trace` (list of (arrival seconds, Spec)) for `duration`
        seconds of wall time (or until done with drain).  Returns the latency
        (and, with readback, the result) of every finished solve, the rejected
        and cancelled requests, the site updates done and the wall time.
        `keep` (a set of trace indices) keeps those solves' objects; `cancel`
        maps trace indices to the time their client withdraws them."""
        t0 = time.perf_counter()
        pending = collections.deque((i, a, s) for i, (a, s) in enumerate(trace))
        cancel = dict(cancel or {})
        waiting, active, done, rejected, cancelled = collections.deque(), [], [], [], []
        used = sum(nb for lst in self.pool.values() for _, nb in lst)  # kept lattices
        sites_in_flight = 0
        updates = 0
        kept = {}
        members_changed = False

        def release_one():
            nonlocal used
            victims = [k for k, v in self.pool.items() if v]
            if not victims:
                return False
            _, vb = self.pool[victims[0]].pop()
            used -= vb
            return True

        def fits(spec):
            nb = spec.device_bytes(self.precision)
            if active and sites_in_flight + spec.sites > self.max_sites:
                return False
            if self.pool.get(spec.shape):
                return True  # a kept lattice of this shape
            while used + nb > self.budget:
                if not release_one():
                    return False
            return True

        def admit(spec):
            """Device objects of the solve, or None when the allocation failed
            even after the kept lattices were released."""
            nonlocal used
            if self.pool.get(spec.shape):
                lat, nb = self.pool[spec.shape].pop()
                return self.build(spec, self.precision, lat), nb
            nb = spec.device_bytes(self.precision)
            while True:
                try:
                    objs = self.build(spec, self.precision, None)
                except Exception as e:  # noqa: BLE001 -- only allocation failures are retried
                    if not _is_alloc_failure(e):
                        raise
                    if release_one():
                        continue
                    return None, nb
                used += nb
                return objs, nb

        while True:
            now = time.perf_counter() - t0
            if now >= duration and not (drain and (pending or waiting or active)):
                break
            while pending and pending[0][1] <= now:
                i, arrival, spec = pending.popleft()
                why = spec_problem(spec)
                if why is None and spec.device_bytes(self.precision) > self.budget:
                    why = "needs %d bytes of device memory, more than the budget %d" % (
                        spec.device_bytes(self.precision), self.budget)
                if why is not None:
                    rejected.append({"index": i, "reason": why})
                else:
                    waiting.append((i, arrival, spec))
            # withdrawn requests leave the trace, the queue or the batch
            due = {i for i, tc in cancel.items() if tc <= now} if cancel else ()
            if due:
                for i in due:
                    del cancel[i]
                for where, seq in (("before arrival", pending), ("queue", waiting)):
                    for item in seq:
                        if item[0] in due:
                            cancelled.append({"index": item[0], "where": where})
                pending = collections.deque(x for x in pending if x[0] not in due)
                waiting = collections.deque(x for x in waiting if x[0] not in due)
                gone = [j for j in active if j.index in due]
                if gone:
                    active = [j for j in active if j.index not in due]
                    for j in gone:
                        cancelled.append({"index": j.index, "where": "batch",
                                          "steps_done": j.spec.steps - j.remaining})
                        sites_in_flight -= j.spec.sites
                        self.pool[j.spec.shape].append((j.objs[0], j.bytes))
                    self.ens.set_members([j.objs for j in active])
                    members_changed = bool(active)
            # admission: in arrival order while the next solve fits
            while waiting and fits(waiting[0][2]):
                i, arrival, spec = waiting[0]
                objs, nb = admit(spec)
                if objs is None:
                    if not active:  # nothing else holds memory: it cannot run
                        waiting.popleft()
                        rejected.append({"index": i, "reason": "device allocation failed"})
                        continue
                    break  # wait for running solves to free memory
                waiting.popleft()
                job = _Job(arrival, spec, objs, nb)
                job.index = i
                job.admitted = time.perf_counter() - t0
                sites_in_flight += spec.sites
                active.append(job)
                members_changed = True
            if not active:
                if waiting and used == 0 and not fits(waiting[0][2]):
                    i, _, spec = waiting.popleft()
                    rejected.append({"index": i, "reason": "does not fit the HBM budget"})
                    continue
                nxt = pending[0][1] if pending else None
                if nxt is None and not waiting:
                    if drain:
                        break
                    time.sleep(max(0.0, min(duration - now, 0.01)))
                    continue
                if nxt is not None:
                    time.sleep(max(0.0, min(nxt - now, duration - now, 0.01)))
                continue
            if members_changed:
                self.ens.set_members([j.objs for j in active])
                if self.autotune:
                    self.ens.autotune()
                members_changed = False
            # a full chunk for the batch; a solve that needs fewer steps takes
            # only those and leaves at the chunk's end
            k = min(self.chunk, max(j.remaining for j in active))
            lim = [min(k, j.remaining) for j in active]
            self.ens.Step(k, limits=lim)
            for j, kj in zip(active, lim):
                j.remaining -= kj
                updates += j.spec.sites * kj
            finished = [j for j in active if j.remaining <= 0]
            if finished:
                active = [j for j in active if j.remaining > 0]
                results = {j.index: read_result(j.objs) for j in finished} if self.readback \
                    else {}
                t_fin = time.perf_counter() - t0
                for j in finished:
                    rec = {"index": j.index, "latency": t_fin - j.arrival,
                           "queue": j.admitted - j.arrival, "sites": j.spec.sites,
                           "steps": j.spec.steps}
                    if callable(self.readback):
                        self.readback(j.index, results[j.index])
                    elif self.readback:
                        rec["result"] = results[j.index]
                    done.append(rec)
                    sites_in_flight -= j.spec.sites
                    if keep is not None and j.index in keep:
                        kept[j.index] = j.objs
                        used -= j.bytes
                    else:
                        self.pool[j.spec.shape].append((j.objs[0], j.bytes))
                self.ens.set_members([j.objs for j in active])
        wall = time.perf_counter() - t0
        return {"done": done, "rejected": rejected, "cancelled": cancelled, "updates": updates,
                "wall": wall, "unfinished": len(active) + len(waiting) + len(pending),
                "kept": kept}


def serve_one_at_a_time(trace, duration, precision="f64", readback=None):
    """The plain counterpart: each solve in arrival order through System.Step;
    readback (a callable, as Server's) receives each finished solve's state
    before its latency is taken."""
    t0 = time.perf_counter()
    done, updates = [], 0
    unfinished = 0
    for i, (arrival, spec) in enumerate(trace):
        now = time.perf_counter() - t0
        if now >= duration:
            unfinished = len(trace) - i
            break
        if arrival > now:
            time.sleep(arrival - now)
        lat, sw, tr = build_solve(spec, precision)
        system = System(lat)
        system.AddThing(sw)
        if tr is not None:
            system.AddThing(tr)
        left = spec.steps
        while left > 0 and time.perf_counter() - t0 < duration:
            k = min(left, 64)
            system.Step(k)
            lat.synchronize()
            left -= k
            updates += spec.sites * k
        if left > 0:
            unfinished = len(trace) - i
            break
        if readback is not None:
            readback(i, read_result((lat, sw, tr)))
        done.append({"index": i, "latency": time.perf_counter() - t0 - arrival,
                     "sites": spec.sites, "steps": spec.steps})
    return {"done": done, "updates": updates, "wall": time.perf_counter() - t0,
            "unfinished": unfinished}


def summary(result):
    lat = sorted(d["latency"] for d in result["done"])

    def pct(p):
        if not lat:
            return None
        return lat[min(len(lat) - 1, int(math.ceil(p / 100.0 * len(lat))) - 1)]
    return {"completed": len(lat), "unfinished": result["unfinished"],
            "p50_s": pct(50), "p99_s": pct(99),
            "glups": result["updates"] / result["wall"] / 1e9, "wall_s": result["wall"]}
