"""The multi-GPU path is replicas only (independent points, no data-path
collective): two gloo ranks on the CPU check the barrier, the maximum of the
step times over the ranks and the job rate that bench.py reports."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _stream(n=14, seed=3):
    import numpy as np
    from pynfam_gb300.serve import Request
    rng = np.random.default_rng(seed)
    nuclei = [("S40", 8), ("Kr116", 12), ("Gd162", 16), ("Gd162", 20), ("S40", 20)]
    reqs = []
    for i in range(n):
        nuc = nuclei[int(rng.integers(len(nuclei)))]
        reqs.append(Request(i, (nuc, int(rng.integers(2))), np.zeros(int(rng.integers(10, 51)), dtype=complex),
                            float(i) * 0.1))
    return reqs


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    from pynfam_gb300 import replicas
    assert replicas.env() == (world, rank, rank)
    assert replicas.init("gloo") == world
    replicas.barrier()
    step = 1.5 + rank          # each replica's own step time
    slowest = replicas.max_over_ranks(step)
    # the rank's share of a many-nucleus stream, computed alone on every rank; the ranks'
    # request ids are gathered to check that they cover the stream once
    import torch
    import torch.distributed as dist
    mine = replicas.partition(_stream(), world)[rank]
    ids = torch.full((64,), -1, dtype=torch.int64)
    ids[:len(mine)] = torch.tensor([r.rid for r in mine], dtype=torch.int64)
    allids = [torch.empty_like(ids) for _ in range(world)]
    dist.all_gather(allids, ids)
    got = sorted(int(x) for t in allids for x in t.tolist() if x >= 0)
    out.put((rank, slowest, replicas.job_rate(120, slowest, world), got, sorted({r.key[0] for r in mine})))
    replicas.barrier()
    replicas.finish()


def test_two_replicas_take_the_slowest_step():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[0] for r in res] == [0, 1]
    for _, slowest, rate, got, _ in res:
        assert slowest == 2.5
        assert rate == pytest.approx(2 * 120 / 2.5)
        assert got == list(range(len(_stream())))     # every request on exactly one rank
    assert not set(res[0][4]) & set(res[1][4])       # no nucleus on two ranks


def test_single_process_is_its_own_job():
    from pynfam_gb300 import replicas
    assert replicas.max_over_ranks(3.0) == 3.0
    assert replicas.job_rate(128, 4.0, 1) == 32.0


def test_partition_keeps_nuclei_together_and_balances_work():
    from pynfam_gb300 import replicas
    reqs = _stream(40)
    for world in (1, 2, 3, 4):
        parts = replicas.partition(reqs, world)
        assert sorted(r.rid for p in parts for r in p) == list(range(len(reqs)))
        owner = {}
        for k, p in enumerate(parts):
            assert [r.arrival for r in p] == sorted(r.arrival for r in p)
            for r in p:
                assert owner.setdefault(r.key[0], k) == k
        loads = [sum(len(r.omegas) for r in p) for p in parts]
        groups = {}
        for r in reqs:
            groups[r.key[0]] = groups.get(r.key[0], 0) + len(r.omegas)
        # largest-first greedy: no rank exceeds the average by more than the largest group
        assert max(loads) <= sum(loads) / world + max(groups.values())
