"""Serving loop: continuous batching of FAM solve requests on one GPU.

The reference answers one (nucleus, operator, omega) point per pnfam_main.x
process and leaves scheduling to pynfam's task farm (pynfam/fortran/
pnfam_run.py, pynfam's MPI master/worker split).  Here a request is a list of
omega points for one (nucleus, operator) pair; the server keeps one engine
(pnfam_gpu_engine_*) per pair resident on the device, admits the points of
queued requests into free slots as earlier points retire, and steps all
engines together so that their work overlaps on the GPU.  Engines are created
while their estimated device memory fits the budget and released when their
queue is empty and another pair needs the memory.

Each engine steps at its own pace: ``launch`` only enqueues an evaluation, and the
loop takes an engine's results as soon as ``ready`` says they are there, admits new
points into its free slots and launches it again, so an engine with a few slow
points left is not held to the pace of a busy one, and the engines' work overlaps on
the GPU.  The scheduler only talks to objects with the Engine interface (``slots``,
``active``, ``admit``, ``launch``, ``ready``, ``finish``, ``close``), so it is tested
on the host with a fake engine.
"""
from __future__ import annotations

import collections
import time
from dataclasses import dataclass, field

import numpy as np


@dataclass
class Request:
    rid: int
    key: object                # (nucleus, operator) identifier known to the engine factory
    omegas: np.ndarray         # complex omega points
    arrival: float = 0.0       # seconds after the start of the run


@dataclass
class PointOutcome:
    rid: int
    index: int                 # position of the point in its request
    omega: complex
    S: np.ndarray
    iters: int
    si: float
    arrival: float
    admitted: float
    done: float

    @property
    def latency(self) -> float:
        return self.done - self.arrival


@dataclass
class ServeStats:
    points: int = 0
    converged: int = 0
    wall: float = 0.0
    steps: int = 0             # evaluations launched (all engines)
    peak_engines: int = 0
    peak_bytes: int = 0
    latencies: list = field(default_factory=list)

    def percentile(self, q):
        return float(np.percentile(self.latencies, q)) if self.latencies else float("nan")


def slot_bytes(nxy: int, broyden_m: int, mixed: bool, statistical: bool = False) -> int:
    """Device memory of one solve slot (the per-point buffers of pnfam_gpu.cu); the
    statistical FAM doubles the QP-state arrays (quadrants P and Q) and the scratch."""
    q = 2 if statistical else 1
    f64 = q * (4 + 4 + 16 + 4 + 4 + 2 * 4 * max(broyden_m, 1)) + 8 + 8   # state, vout, T, hqp, G, df+dv; rsp, hsp
    if mixed:
        f64 += 4 + 4 + 4 * 4                                     # anchor, its image; Broyden raw vectors
    f32 = (4 + 16 + 8 + 8 + 4) if mixed else 0
    return int(nxy) * (8 * f64 + 4 * f32)


class Server:
    """engine_factory(key, slots) -> Engine; engine_bytes(key, slots) -> int; poll: the
    wait (s) between looks at the engines in flight when none has finished."""

    def __init__(self, engine_factory, engine_bytes, slots: int, budget_bytes: int,
                 clock=time.perf_counter, sleep=time.sleep, poll: float = 5e-5):
        self.factory = engine_factory
        self.bytes = engine_bytes
        self.slots = int(slots)
        self.budget = int(budget_bytes)
        self.clock = clock
        self.sleep = sleep
        self.poll = float(poll)

    def run(self, requests):
        reqs = sorted(requests, key=lambda r: r.arrival)
        arrivals = collections.deque(reqs)
        queues = collections.OrderedDict()     # key -> deque of (rid, index, omega, arrival)
        engines = collections.OrderedDict()    # key -> engine
        used = {}                              # key -> bytes
        inflight = collections.OrderedDict()   # key -> engine with an evaluation in flight
        meta = {}                              # tag -> (rid, index, omega, arrival, admitted)
        outcomes = []
        stats = ServeStats(points=sum(len(r.omegas) for r in reqs))
        tag = 0
        t0 = self.clock()

        def collect(key):
            eng = inflight.pop(key)
            for res in eng.finish():
                rid, idx, w, arr, adm = meta.pop(res.tag)
                done = self.clock() - t0
                outcomes.append(PointOutcome(rid, idx, w, res.S, res.iters, res.si, arr, adm, done))

        while True:
            now = self.clock() - t0
            while arrivals and arrivals[0].arrival <= now:
                r = arrivals.popleft()
                q = queues.setdefault(r.key, collections.deque())
                for i, w in enumerate(np.atleast_1d(r.omegas)):
                    q.append((r.rid, i, complex(w), r.arrival))
            # every engine steps at its own pace: results of the evaluations that have
            # completed are taken as they come, without waiting for the other engines
            for key in [k for k, e in inflight.items() if e.ready()]:
                collect(key)
            # engines for queued keys, within the memory budget (idle engines make room)
            for key, q in queues.items():
                if not q or key in engines:
                    continue
                need = self.bytes(key, self.slots)
                for k2 in list(engines):
                    if sum(used.values()) + need <= self.budget:
                        break
                    if k2 not in inflight and engines[k2].active == 0 and not queues.get(k2):
                        engines.pop(k2).close()
                        used.pop(k2)
                if sum(used.values()) + need <= self.budget or not engines:
                    engines[key] = self.factory(key, self.slots)
                    used[key] = need
            stats.peak_engines = max(stats.peak_engines, len(engines))
            stats.peak_bytes = max(stats.peak_bytes, sum(used.values()))
            # admit into the free slots of the idle engines, and launch them
            for key, eng in engines.items():
                if key in inflight:
                    continue
                q = queues.get(key)
                free = eng.slots - eng.active
                if q and free > 0:
                    batch = [q.popleft() for _ in range(min(free, len(q)))]
                    tags = np.arange(tag, tag + len(batch), dtype=np.int64)
                    adm = self.clock() - t0
                    for t, b in zip(tags, batch):
                        meta[int(t)] = b + (adm,)
                    tag += len(batch)
                    n = eng.admit(np.array([b[2] for b in batch]), tags)
                    if n != len(batch):
                        raise RuntimeError(f"engine admitted {n} of {len(batch)} points")
                if eng.active > 0:
                    eng.launch()       # enqueues one evaluation and returns
                    inflight[key] = eng
                    stats.steps += 1
            if not inflight:
                if not arrivals and not any(queues.values()):
                    break
                if arrivals and not any(queues.values()):
                    self.sleep(max(0.0, arrivals[0].arrival - (self.clock() - t0)))
                continue
            if not any(e.ready() for e in inflight.values()):
                self.sleep(self.poll)   # nothing to take yet
        stats.wall = self.clock() - t0
        stats.converged = sum(1 for o in outcomes if o.iters >= 0)
        stats.latencies = [o.latency for o in outcomes]
        for eng in engines.values():
            eng.close()
        return outcomes, stats


def poisson_arrivals(n, rate, seed=0):
    """Arrival times (s) of n requests of a Poisson process with the given rate (1/s)."""
    rng = np.random.default_rng(seed)
    return np.cumsum(rng.exponential(1.0 / rate, size=n)) if rate > 0 else np.zeros(n)
