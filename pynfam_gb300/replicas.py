"""Replicas across the GPUs of one node.

Every (nucleus, operator, omega) point is independent -- the reference runs each
one as its own pnfam_main.x process -- so N GPUs run N independent copies of the
serving stream, one process per GPU, with no collective on the data path.  The
only communication is a barrier on each side of the timed region and the maximum
of the step times over the ranks: the job's time is its slowest replica, and the
job's rate is N times the points of one replica over that time.  A stream of many
nuclei is split instead with ``partition``: whole nuclei to ranks, by estimated work.
"""
from __future__ import annotations

import os


def env():
    """(world size, rank, local rank) from the launcher's environment."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def init(backend: str) -> int:
    """Join the process group when there is more than one rank; returns the world size."""
    world = env()[0]
    if world > 1:
        import torch.distributed as dist
        if not dist.is_initialized():
            dist.init_process_group(backend)
    return world


def barrier(device=None):
    import torch
    if device is not None and str(device).startswith("cuda"):
        torch.cuda.synchronize()
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.barrier()


def max_over_ranks(x: float, device="cpu") -> float:
    """The largest x over the ranks (x itself with one rank)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_replica: float, step_s: float, world: int) -> float:
    """Units per second of the whole job: every replica processed units_per_replica
    within step_s (the slowest replica's time)."""
    return world * units_per_replica / step_s


def partition(requests, world: int, cost=None, group=None):
    """Assign a stream's requests to ``world`` ranks without splitting a group: the
    requests of one ground state (``group(r)``, default ``r.key[0]`` or ``r.key``) stay on
    one GPU, which keeps that nucleus's contexts and pair tensors resident there and
    builds them once.  Groups are placed largest first on the rank with the least
    estimated work so far (``cost(r)``, default the request's number of points), ties to
    the lower rank, so every rank computes the same assignment without communicating.
    Returns one list of requests per rank, each in arrival order."""
    if cost is None:
        cost = lambda r: len(r.omegas)
    if group is None:
        group = lambda r: r.key[0] if isinstance(r.key, tuple) else r.key
    groups = {}
    for r in requests:
        groups.setdefault(group(r), []).append(r)
    order = sorted(groups, key=lambda g: (-sum(cost(r) for r in groups[g]), repr(g)))
    load = [0.0] * world
    out = [[] for _ in range(world)]
    for g in order:
        k = min(range(world), key=lambda i: (load[i], i))
        out[k] += groups[g]
        load[k] += sum(cost(r) for r in groups[g])
    for o in out:
        o.sort(key=lambda r: (r.arrival, r.rid))
    return out


def finish():
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        dist.destroy_process_group()
