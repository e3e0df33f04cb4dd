"""Independent solves shared out over GPUs, one process per GPU (no reference
counterpart: the reference runs one solve on one GPU).

Solves of a batched ensemble, or requests of a served stream, are
independent, so they are partitioned across the ranks of a job with no
communication on the data path: every rank computes the same assignment from
the same inputs, runs its own share on its own GPU (an Ensemble or a Server of
this package), and only the per-rank summaries travel, once, over the host
process group at the end (gloo or any torch.distributed backend).

The assignment is deterministic: longest work first, each solve to the rank
with the least work assigned so far (work = site updates, sites x steps,
scaled by the rank's relative HBM budget), ties to the lower rank.
"""
import heapq


def work_of(spec):
    """Site updates a solve asks for."""
    return int(spec.sites) * max(1, int(getattr(spec, "steps", 1) or 1))


def assign(specs, world, capacity=None):
    """Rank of each solve: LPT greedy over `world` ranks; `capacity` (one
    positive weight per rank, e.g. each GPU's free HBM) scales how much work a
    rank takes.  Identical on every rank for identical inputs."""
    if world < 1:
        raise ValueError("world must be >= 1")
    cap = [1.0] * world if capacity is None else [float(c) for c in capacity]
    if len(cap) != world or min(cap) <= 0:
        raise ValueError("one positive capacity per rank")
    order = sorted(range(len(specs)), key=lambda i: (-work_of(specs[i]), i))
    heap = [(0.0, r) for r in range(world)]
    out = [0] * len(specs)
    for i in order:
        load, r = heapq.heappop(heap)
        out[i] = r
        heapq.heappush(heap, (load + work_of(specs[i]) / cap[r], r))
    return out


def assign_stream(trace, world, capacity=None):
    """Rank of each request of an arrival trace [(time, spec)]: in arrival
    order, to the rank with the least outstanding work at that time (work
    assigned minus the work its GPU can have done since, at a rate
    proportional to its capacity); ties to the lower rank.  Depends on the
    trace only, so every rank computes the same split."""
    cap = [1.0] * world if capacity is None else [float(c) for c in capacity]
    backlog = [0.0] * world
    last = 0.0
    rate = 1e9  # nominal site updates per second per unit of capacity
    out = []
    for t, spec in trace:
        dt = max(0.0, t - last)
        last = max(last, t)
        backlog = [max(0.0, b - rate * c * dt) for b, c in zip(backlog, cap)]
        r = min(range(world), key=lambda k: (backlog[k] / cap[k], k))
        out.append(r)
        backlog[r] += work_of(spec)
    return out


def mine(items, ranks, rank):
    """The items (with their indices) assigned to `rank`."""
    return [(i, x) for i, (x, r) in enumerate(zip(items, ranks)) if r == rank]


def gather_objects(obj, world):
    """Every rank's `obj` (a small picklable summary), in rank order, over the
    default torch.distributed process group; [obj] when world == 1."""
    if world <= 1:
        return [obj]
    import torch.distributed as dist
    out = [None] * world
    dist.all_gather_object(out, obj)
    return out


def merge_served(parts):
    """One served-stream result from the ranks' results (trace indices are
    global): latencies of every finished request, rejections, cancellations,
    site updates summed, wall time the slowest rank's."""
    done, rejected, cancelled = [], [], []
    updates, wall, unfinished = 0, 0.0, 0
    for p in parts:
        done += p["done"]
        rejected += p.get("rejected", [])
        cancelled += p.get("cancelled", [])
        updates += p["updates"]
        wall = max(wall, p["wall"])
        unfinished += p["unfinished"]
    return {"done": done, "rejected": rejected, "cancelled": cancelled, "updates": updates,
            "wall": wall, "unfinished": unfinished}
