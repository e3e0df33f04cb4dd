#!/usr/bin/env python3
"""Coupled-step benchmark: D3Q15 MRT LB + swimmers + tracers on one GB300.

Default workload: a 256^3 periodic lattice (tau_s = tau_b = 0.8,
rho = 1 + 1e-3 U[0,1), u = 0) with 65,536 run-and-tumble swimmers and
1,048,576 tracers at seeded uniform positions, FP32 deviation storage with
FP32 collision, advanced with the coupled step ZeroForce / AddForces / Step /
CalcHydro / Move.  A step is one coupled step of the whole lattice.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--precision f32|bf16|f16|f64] [--size S]

Prints one JSON line (rank 0).  `value` is device-resident throughput in
GLUPS (lattice-site updates per second); `e2e` is the same metric through the
public Python API with host buffers, the per-step swimmer read-back and the
initial upload inside the timed region.  `--impl reference` times the
reference's method (the FP64 CPU restatement in oracle/, all host threads) on
a bounded sample of the same workload.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "gpu-swimmers_gb300"))

METRIC = "coupled-step GLUPS & % HBM roofline; p50/p99 latency, batched vs plain FP64"
L2_BYTES = 129 * 1024 * 1024
# FP64 operations per site of the reference's DoStep (lb.cu:72-218), each add,
# multiply and divide counted once: the two dense 15x15 mode transforms (900),
# the relaxation of the stress modes with forcing (200), the two rates (4)
REF_DOSTEP_FLOP = 1104
# The step kernel's own CUDA events (the roofline's launch time) bracket every
# TIMING_EVERY-th step of the timed region: events around every launch cost
# the coupled step about 10 us (1.5%), around every 4th about 1 us.
TIMING_EVERY = 4


def workload(size, nsw, ntr, seed=42, tau=0.8, P=1e-3, l=0.5, alpha=0.01):
    """Seeded synthetic inputs: rho = 1 + 1e-3 U[0,1), u = 0, particles uniform in
    the box, swimmer orientations uniform on the sphere."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = size
    N = nx * ny * nz
    L = np.array(size, dtype=np.float64).reshape(3, 1)
    rho = 1.0 + 1e-3 * rng.random(N)
    nv = rng.standard_normal((3, nsw))
    if nsw:
        nv /= np.linalg.norm(nv, axis=0, keepdims=True)
    eta = tau / 3.0
    sw = {"n": nsw, "P": P, "l": l, "alpha": alpha,
          "mobility": (1.0 / 0.1 - 1.0 / 1.5) / (6.0 * np.pi * eta),
          "translational_advection_off": False, "rotational_advection_off": False,
          "seed": seed * 7919 + 17, "r": rng.random((3, nsw)) * L, "nvec": nv,
          "v": np.zeros((3, nsw))}
    tr = {"n": ntr, "r": rng.random((3, ntr)) * L, "v": np.zeros((3, ntr))}
    return {"size": tuple(size), "tau_s": tau, "tau_b": tau, "rho": rho, "u": 0.0,
            "swimmers": sw, "tracers": tr}


def scaled_counts(side, base_side=256, nsw=65536, ntr=1048576):
    f = (side / base_side) ** 3
    return max(1, int(round(nsw * f))), max(1, int(round(ntr * f)))


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)),
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(x, world):
    """The largest x over the ranks of the job (a timing is the slowest rank's)."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def emit(line, rank):
    """Rank 0 prints the job's one JSON line."""
    if rank == 0:
        print(json.dumps(line), flush=True)


def build_objects(case, precision):
    from lbswim import lb, swimmers, tracers
    from lbswim.System import System
    nx, ny, nz = case["size"]
    lat = lb.Lattice(nx, ny, nz, case["tau_s"], case["tau_b"], precision=precision)
    sw_d = case["swimmers"]
    cp = swimmers.CommonParams()
    for k in ("P", "l", "alpha", "mobility", "translational_advection_off",
              "rotational_advection_off", "seed"):
        setattr(cp, k, sw_d[k])
    sw = swimmers.Array(sw_d["n"], cp)
    tr = tracers.Array(case["tracers"]["n"])
    system = System(lat)
    system.AddThing(sw)
    system.AddThing(tr)
    return lat, sw, tr, system


def fill_host(case, lat, sw, tr):
    """Write the initial state into the objects' (page-locked) host copies."""
    nx, ny, nz = case["size"]
    N = nx * ny * nz
    lat.rho[:] = np.broadcast_to(case["rho"], (N,)).reshape(1, nx, ny, nz)
    lat.u[:] = np.broadcast_to(case["u"], (3 * N,)).reshape(3, nx, ny, nz)
    s = case["swimmers"]
    sw.r[:] = s["r"]
    sw.n[:] = s["nvec"]
    sw.v[:] = s["v"]
    t = case["tracers"]
    tr.r[:] = t["r"]
    tr.v[:] = t["v"]
    tr.s[:] = 0.0


def push(case, lat, sw, tr):
    """Host -> device copy of the whole initial state from the host copies, then
    InitFromHydro; returns the bytes copied."""
    lat.rho.H2D()
    lat.u.H2D()
    lat.ZeroForce()
    sw.H2D()
    tr.H2D()
    lat.InitFromHydro()
    N = int(np.prod(case["size"]))
    return 8 * N * 4 + 8 * 9 * case["swimmers"]["n"] + 16 + 8 * 9 * case["tracers"]["n"]


def upload(case, lat, sw, tr):
    """Host fill and host -> device copy of the whole initial state."""
    fill_host(case, lat, sw, tr)
    return push(case, lat, sw, tr)


def algorithmic_bytes(N, nsw, ntr, s_f, s_h):
    """Per step: f read + write, force read, rho + u write per site; r, n (or s)
    read + write and v write per particle."""
    lb_bytes = N * (30 * s_f + 3 * s_h + 4 * s_h)
    return lb_bytes, lb_bytes + 120 * nsw + 120 * ntr


def oracle_module():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build()
    O.set_threads(os.cpu_count())
    return O


def cpu_side(O, size, per_step_budget_s):
    """Largest lattice side <= size whose coupled FP64 oracle step (particles at
    the 256^3 workload's densities) fits per_step_budget_s, calibrated on 64^3."""
    nsw, ntr = scaled_counts(64)
    cal = O.make_system(workload((64, 64, 64), nsw, ntr))
    cal.step(1)
    t0 = time.perf_counter()
    cal.step(2)
    per_site = (time.perf_counter() - t0) / 2 / 64 ** 3
    return int(max(16, min(size, (per_step_budget_s / per_site) ** (1.0 / 3.0))))


def run_cpu_port(size, budget_s, min_steps=3):
    """Time the FP64 CPU restatement of the reference (all host threads) on the
    size^3 workload, or on the largest cube that fits the budget."""
    O = oracle_module()
    side = cpu_side(O, size, budget_s / (min_steps + 1))
    nsw, ntr = scaled_counts(side)
    case = workload((side, side, side), nsw, ntr)
    s = O.make_system(case)
    s.step(1)
    t0 = time.perf_counter()
    n = 0
    while n < min_steps or time.perf_counter() - t0 < budget_s:
        s.step(1)
        n += 1
    dt = time.perf_counter() - t0
    N = side ** 3
    return {"value": N * n / dt / 1e9, "unit": "GLUPS", "cores": O.get_threads(), "kind": "port",
            "sample": "%d^3 lattice, %d swimmers, %d tracers%s, %d coupled FP64 steps in %.1f s "
                      "after one untimed step, oracle/lbswim_oracle.c with OpenMP"
                      % (side, nsw, ntr, "" if side == size else
                         " (the %d^3 workload's densities)" % size, n, dt)}


def reference_arm(args, world, rank):
    if rank != 0:
        return
    O = oracle_module()
    threads = O.get_threads()
    # size the sample so the whole warm-up + timed run stays within about two
    # minutes (the full 256^3 workload takes ~0.4 s per step on 16 Grace cores)
    side = cpu_side(O, args.size, 120.0 / max(1, args.steps + args.warmup))
    nsw, ntr = scaled_counts(side)
    case = workload((side, side, side), nsw, ntr)
    s = O.make_system(case)
    s.step(args.warmup)
    t0 = time.perf_counter()
    s.step(args.steps)
    dt = time.perf_counter() - t0
    N = side ** 3
    value = N * args.steps / dt / 1e9
    sample = ("%d^3 lattice, %d swimmers, %d tracers%s, FP64, oracle/lbswim_oracle.c (the "
              "reference's method restated in C) on %d threads"
              % (side, nsw, ntr, "" if side == args.size else
                 " (the %d^3 workload's densities)" % args.size, threads))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "GLUPS",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config_dict(args, world, precision="f64", ours=False),
            "cpu_baseline": {"value": value, "unit": "GLUPS", "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": "GLUPS", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def config_dict(args, world, precision=None, ours=True):
    precision = precision or args.precision
    nsw, ntr = scaled_counts(args.size)
    cfg = {"workload": "coupled step, %d^3 D3Q15 MRT lattice, %d swimmers, %d tracers, %s "
                        "distributions" % (args.size, nsw, ntr, precision),
            "lattice": [args.size] * 3, "swimmers": nsw, "tracers": ntr, "tau": 0.8,
            "precision": precision, "parallelism": "replicas x%d" % world,
            "l2": "no flush: each step streams %.2f GB of distributions, larger than the "
                  "129 MB L2" % (2 * 15 * args.size ** 3 * {"f64": 8, "f32": 4}.get(
                      precision, 2) / 1e9)}
    if ours:
        cfg["streams"] = ("lattice on a highest-priority stream (lbswim_lattice_set_stream), "
                          "tracer moves on their own least-priority stream")
    return cfg


def load_traffic(precision, side):
    name = "step_push_f64" if precision == "f64" else "fused_step_%s" % precision
    path = os.path.join(ROOT, "profiles", "%s_traffic.json" % name)
    try:
        with open(path) as fh:
            rec = json.load(fh)
        # bytes per launch scale with the sites of the lattice
        return rec["dram_bytes_per_site"] * side ** 3
    except Exception:
        return None


def timed_steps(lat, system, steps, stream):
    """CUDA-event time (ms) of `steps` coupled steps on the lattice's stream and
    the LB step kernel's own event time (total ms, launches), the kernel timed
    on every TIMING_EVERY-th step."""
    import torch
    lat.read_timing()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for i in range(steps):
        lat.set_timing(i % TIMING_EVERY == 0)
        system.Step()
    lat.join()  # the last tracer moves run on the tracers' stream
    ev1.record(stream)
    torch.cuda.synchronize()
    lb_ms, lb_n = lat.read_timing()
    lat.set_timing(False)
    return ev0.elapsed_time(ev1), lb_ms, lb_n


def f64_arm(args, case, stream):
    """The reference's own method and precision (FP64 storage and arithmetic)
    on the same workload, device-resident, for the like-for-like ratio with the
    FP64 reference arm."""
    import torch
    N = int(np.prod(case["size"]))
    nsw, ntr = case["swimmers"]["n"], case["tracers"]["n"]
    lat, sw, tr, system = build_objects(case, "f64")
    lat.set_stream(stream.cuda_stream)
    upload(case, lat, sw, tr)
    for _ in range(3):
        system.Step()
    torch.cuda.synchronize()
    ms, lb_ms, lb_n = timed_steps(lat, system, args.f64_steps, stream)
    ms_step = ms / args.f64_steps
    peak, _ = measured_peak()
    kernel_s = lb_ms / max(lb_n, 1) / 1e3
    # k_step_push_f64 reads f and the force and writes f (rho, u come from the
    # separate CalcHydro kernel)
    kernel_bytes = N * (30 * 8 + 3 * 8)
    _, step_bytes = algorithmic_bytes(N, nsw, ntr, 8, 8)
    out = {"precision": "f64", "steps": args.f64_steps, "warmup": 3,
           "ms_per_step": ms_step, "glups": N / (ms_step / 1e3) / 1e9,
           "step_roofline": {"achieved": step_bytes / (ms_step / 1e3) / 1e9, "peak": peak,
                             "unit": "GB/s", "frac": step_bytes / (ms_step / 1e3) / 1e9 / peak,
                             "bytes_per_step": step_bytes},
           "kernel": {"name": "k_step_push_f64", "ms": kernel_s * 1e3,
                      "bytes_per_launch": kernel_bytes,
                      "hbm_frac": kernel_bytes / kernel_s / 1e9 / peak,
                      "ref_equiv_flop_per_site": REF_DOSTEP_FLOP,
                      "ref_equiv_tflops": REF_DOSTEP_FLOP * N / kernel_s / 1e12,
                      "bound": "fp64 pipe (the kernel's FP64 instructions, not HBM)"}}
    del system, sw, tr, lat
    return out


def our_arm(args, world, rank, local):
    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from lbswim import _lib
    side = args.size
    nsw, ntr = scaled_counts(side)
    case = workload((side, side, side), nsw, ntr, seed=42 + rank)
    N = side ** 3
    lat, sw, tr, system = build_objects(case, args.precision)
    # The lattice (and the particles moved with it) on a stream of the highest
    # priority: the step kernels are dispatched ahead of tracer blocks still
    # queued on the tracers' own least-priority stream, which fill the SMs the
    # step leaves idle.
    stream = torch.cuda.Stream(priority=-5)
    lat.set_stream(stream.cuda_stream)
    if args.bulk_copy:
        lat.set_compat(_lib.COMPAT_INIT_SXZ | _lib.COMPAT_BULK_COPY)
    upload(case, lat, sw, tr)

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    for _ in range(args.warmup):
        system.Step()
    barrier()
    lat.read_timing()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    launches0 = _lib.kernel_launches()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for i in range(args.steps):
        lat.set_timing(i % TIMING_EVERY == 0)
        system.Step()
    lat.join()  # the last tracer moves run on the tracers' stream
    ev1.record(stream)
    barrier()
    launches = _lib.kernel_launches() - launches0
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1)
    lb_ms, lb_n = lat.read_timing()
    lat.set_timing(False)
    ms = max_over_ranks(ms, world)
    ms_step = ms / args.steps
    value = N * args.steps * world / (ms / 1e3) / 1e9

    # End to end through the public API, from the page-locked host copies the
    # initial state was written into beforehand: upload of rho, u and the
    # particles, InitFromHydro, K steps each followed by the swimmer read-back
    # of the README loop, and the final read-back of rho and u.
    fill_host(case, lat, sw, tr)
    barrier()
    t0 = time.perf_counter()
    h2d = push(case, lat, sw, tr)
    lat.synchronize()
    t1 = time.perf_counter()
    d2h = 0
    for _ in range(args.steps):
        system.Step()
        sw.D2H()
        d2h += 8 * 9 * nsw + 16
    lat.synchronize()
    t2 = time.perf_counter()
    lat.rho.D2H()
    lat.u.D2H()
    d2h += 8 * 4 * N
    barrier()
    t3 = time.perf_counter()
    e2e_s = max_over_ranks(t3 - t0, world)
    e2e = {"value": N * args.steps * world / e2e_s / 1e9, "unit": "GLUPS",
           "h2d_bytes_per_step": int(h2d / args.steps), "d2h_bytes_per_step": int(d2h / args.steps),
           "api": "lbswim.System.Step() + swimmers.Array.D2H() per step (Python -> C ABI)",
           "steps": args.steps,
           "pieces_ms": {"upload_and_init": (t1 - t0) * 1e3, "steps_with_readback": (t2 - t1) * 1e3,
                         "final_readback": (t3 - t2) * 1e3},
           "host_fill": "outside the timed region (written into page-locked host copies first)"}

    s_f = {"f64": 8, "f32": 4}.get(args.precision, 2)
    s_h = 8 if args.precision == "f64" else 4
    lb_bytes, step_bytes = algorithmic_bytes(N, nsw, ntr, s_f, s_h)
    if args.precision == "f64":
        # k_step_push_f64 reads f and the force and writes f; rho and u come
        # from the separate CalcHydro kernel
        lb_bytes = N * (30 * s_f + 3 * s_h)
    peak, peak_kind = measured_peak()
    lb_avg_s = lb_ms / max(lb_n, 1) / 1e3
    achieved = lb_bytes / lb_avg_s / 1e9
    traffic = load_traffic(args.precision, side)
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic,
                "kernel": "k_fused_step" if args.precision != "f64" else "k_step_push_f64",
                "kernel_ms": lb_avg_s * 1e3, "bytes_per_launch": lb_bytes,
                "timed_launches": "%d of %d (every %d-th step of the timed region)"
                                  % (lb_n, args.steps, TIMING_EVERY),
                "peak_source": "%s (MEASURED_PEAKS.json hbm_gbs)" % peak_kind
                if peak_kind == "measured" else "fallback 6.8 TB/s"}
    step_ach = step_bytes / (ms_step / 1e3) / 1e9
    line = {"metric": METRIC, "value": value, "unit": "GLUPS", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32" if args.precision == "f32" else args.precision, "data": "synthetic",
            "config": config_dict(args, world), "clocks": clk, "e2e": e2e,
            "gpu_launches": int(launches), "roofline": roofline,
            "step_roofline": {"achieved": step_ach, "peak": peak, "unit": "GB/s",
                              "frac": step_ach / peak, "bytes_per_step": step_bytes}}
    if args.precision == "f64":
        # the FP64 ALU check, in the reference's operations per site;
        # k_step_push_f64 does the same step with the butterfly transform and
        # fused multiply-adds, so fewer FP64 instructions
        line["fp64"] = {"ref_equiv_flop_per_site": REF_DOSTEP_FLOP,
                        "ref_equiv_tflops": REF_DOSTEP_FLOP * N / lb_avg_s / 1e12,
                        "kernel": "k_step_push_f64"}
    del system, sw, tr, lat
    if args.precision != "f64" and args.f64_steps > 0:
        # the same workload in the reference's precision, beside the headline
        line["f64"] = f64_arm(args, case, stream)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = run_cpu_port(side, args.cpu_seconds)
    # the batched ensemble and the served stream, each against plain FP64
    # one solve at a time (every rank runs its own replica)
    if args.ens_members > 0:
        line["ensemble"] = ensemble_arm(args, world, rank)
    if args.serve_seconds > 0:
        line["serving"] = serving_arm(args, world, rank)
    emit(line, rank)
    if world > 1:
        torch.distributed.destroy_process_group()


def ensemble_arm(args, world=1, rank=0):
    """Batched ensemble of independent FP32 solves (shapes 16^3 .. 48x48x96,
    tau, swimmers and tracers drawn per solve) advanced together, against the
    same solves stepped one at a time in plain FP64 (stepping timed only).
    With several ranks the solves are shared out (lbswim.shard) and each rank
    runs its share; rates are the job's total site updates over the slowest
    rank's time."""
    import torch
    from lbswim import serve, shard
    from lbswim.ensemble import Ensemble
    from lbswim.System import System
    rng = np.random.default_rng(7)
    all_specs = [serve.draw_spec(rng) for _ in range(args.ens_members)]
    ranks = shard.assign(all_specs, world)
    specs = [sp for _, sp in shard.mine(all_specs, ranks, rank)]
    sites_all = sum(s.sites for s in all_specs)
    objs = [serve.build_solve(s, "f32") for s in specs]
    ens = Ensemble(objs)
    ens.autotune()
    tiles = [o[0].tile for o in objs]
    ens.Step(2)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ens.Step(args.ens_steps)
    torch.cuda.synchronize()
    dt = max_over_ranks(time.perf_counter() - t0, world)
    batched = sites_all * args.ens_steps / dt / 1e9
    del ens, objs
    # plain FP64, one solve at a time, the same solves
    f64_steps, f64_time = args.ens_f64_steps, 0.0
    for sp in specs:
        lat, sw, tr = serve.build_solve(sp, "f64")
        system = System(lat)
        system.AddThing(sw)
        if tr is not None:
            system.AddThing(tr)
        lat.synchronize()
        t0 = time.perf_counter()
        system.Step(f64_steps)
        lat.synchronize()
        f64_time += time.perf_counter() - t0
    f64_time = max_over_ranks(f64_time, world)
    plain = sites_all * f64_steps / f64_time / 1e9
    # FP32 (batched) against FP64 velocity fields after the full run
    chk = specs[:args.ens_check]
    cobjs = [serve.build_solve(sp, "f32") for sp in chk]
    cens = Ensemble(cobjs)
    cens.Step(args.ens_steps)
    err = 0.0
    for sp, (lat32, _, _) in zip(chk, cobjs):
        lat, sw, tr = serve.build_solve(sp, "f64")
        system = System(lat)
        system.AddThing(sw)
        if tr is not None:
            system.AddThing(tr)
        system.Step(args.ens_steps)
        lat.u.D2H()
        lat32.u.D2H()
        a, b = lat32.u.data.reshape(3, -1), lat.u.data.reshape(3, -1)
        err = max(err, float(np.linalg.norm(a - b) / np.linalg.norm(b)))
    err = max_over_ranks(err, world)
    return {"members": len(all_specs), "ranks": world, "sites": sites_all,
            "steps": args.ens_steps, "precision": "f32",
            "batched_glups": batched, "batched_s": dt,
            "plain_f64_glups": plain, "plain_f64_steps_timed": f64_steps,
            "speedup_vs_plain_f64": batched / plain,
            "u_rel_l2_vs_f64": err, "u_check_members": len(chk) * world,
            "tiles": {"8x32": tiles.count(0), "16x16": tiles.count(1)},
            "launches_per_step": 5, "graph": "two steps captured, replayed"}


def serving_arm(args, world=1, rank=0):
    """Poisson arrivals of solves (the ensemble distribution plus 96^3 and
    128^3, steps log-uniform in [100, 5000]) served by continuous batching
    under an HBM budget -- each finished solve's state (u, swimmers, tracers)
    read back to the host inside its latency -- at the BASELINE rate and at a
    lower rate where the queue stays short (service time), and the same
    BASELINE-rate trace served one solve at a time in plain FP64.  With
    several ranks each serves its share of every stream (lbswim.shard)."""
    import torch
    from lbswim import serve, shard
    free, _ = torch.cuda.mem_get_info()
    budget = int(0.6 * free)
    sink = lambda index, result: None  # noqa: E731 -- the client takes the result

    def served(rate, seconds, plain=False):
        trace = serve.poisson_trace(np.random.default_rng(11), rate, seconds)
        ranks = shard.assign_stream(trace, world)
        local = shard.mine(trace, ranks, rank)
        sub = [x for _, x in local]
        if plain:
            res = serve.serve_one_at_a_time(sub, seconds, "f64", readback=sink)
        else:
            srv = serve.Server(budget, chunk=64, readback=sink)
            res = srv.run(sub, seconds)
            res.pop("kept")
            del srv
        glob = [i for i, _ in local]
        for d in res["done"]:
            d["index"] = glob[d["index"]]
        merged = shard.merge_served(shard.gather_objects(res, world))
        out = serve.summary(merged)
        out["arrivals"] = len(trace)
        return out

    batched = served(args.serve_rate, args.serve_seconds)
    low = served(args.serve_rate_low, args.serve_seconds) if args.serve_rate_low > 0 else None
    plain_s = args.serve_plain_seconds or args.serve_seconds
    plain = served(args.serve_rate, plain_s, plain=True)
    return {"rate_per_s": args.serve_rate, "seconds": args.serve_seconds,
            "plain_seconds": plain_s, "ranks": world,
            "arrivals": batched["arrivals"], "hbm_budget_gb": budget / 1e9,
            "result_readback": "u, swimmer r/v/n and tracer r/s/v of every finished solve copied "
                               "to the host inside its latency",
            "batched_f32": batched,
            "batched_f32_low_rate": dict(low, rate_per_s=args.serve_rate_low) if low else None,
            "plain_f64": plain,
            "glups_ratio": (batched["glups"] / plain["glups"]) if plain["glups"] else None}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--precision", default="f32", choices=["f64", "f32", "bf16", "f16"])
    ap.add_argument("--size", type=int, default=256)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--bulk-copy", action="store_true",
                    help="step kernel with bulk-copied rows (LBSWIM_COMPAT_BULK_COPY; "
                         "comparison runs)")
    ap.add_argument("--cpu-seconds", type=float, default=10.0,
                    help="timed CPU work of the cpu_baseline leg")
    ap.add_argument("--f64-steps", type=int, default=20,
                    help="steps of the FP64 run of the same workload (0: skip)")
    ap.add_argument("--ens-members", type=int, default=512,
                    help="batched-ensemble members (0: skip the ensemble figures)")
    ap.add_argument("--ens-steps", type=int, default=1000)
    ap.add_argument("--ens-check", type=int, default=8,
                    help="members checked against FP64 after the full run")
    ap.add_argument("--ens-f64-steps", type=int, default=20,
                    help="steps per solve timed for the plain FP64 rate")
    ap.add_argument("--serve-seconds", type=float, default=20.0,
                    help="wall time of each served stream (0: skip)")
    ap.add_argument("--serve-rate", type=float, default=200.0)
    ap.add_argument("--serve-rate-low", type=float, default=50.0,
                    help="a second, lower arrival rate for service-time latencies (0: skip)")
    ap.add_argument("--serve-plain-seconds", type=float, default=0.0,
                    help="wall time of the plain FP64 stream (0: as --serve-seconds)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    world, rank, local = dist_setup()
    if args.impl == "reference":
        reference_arm(args, world, rank)
    else:
        our_arm(args, world, rank, local)


if __name__ == "__main__":
    main()
