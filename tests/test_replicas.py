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


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    from pynfam_gb300 import replicas
    assert replicas.env() == (world, rank, rank)
    assert replicas.init("gloo") == world
    replicas.barrier()
    step = 1.5 + rank          # each replica's own step time
    slowest = replicas.max_over_ranks(step)
    out.put((rank, slowest, replicas.job_rate(120, slowest, world)))
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
    assert [r for r, _, _ in res] == [0, 1]
    for _, slowest, rate in res:
        assert slowest == 2.5
        assert rate == pytest.approx(2 * 120 / 2.5)


def test_single_process_is_its_own_job():
    from pynfam_gb300 import replicas
    assert replicas.max_over_ranks(3.0) == 3.0
    assert replicas.job_rate(128, 4.0, 1) == 32.0
