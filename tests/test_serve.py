"""Host-side tests of the serving scheduler (pynfam_gb300.serve) with a fake
engine: continuous batching refills retired slots, requests are not admitted
before they arrive, the device-memory budget limits the resident engines, and
every point's result is the one it gets alone."""
import numpy as np
import pytest

from pynfam_gb300.serve import Request, Server, poisson_arrivals, slot_bytes


class FakeClock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        return self.t

    def sleep(self, dt):
        self.t += max(dt, 0.0)


class Res:
    def __init__(self, tag, S, iters, si):
        self.tag, self.S, self.iters, self.si = tag, S, iters, si


def fake_result(key, w):
    """What the fake solver returns for a point: depends only on (key, omega)."""
    return np.array([np.sin(w.real) + 1j * np.cos(w.imag) + 0.01 * hash(key) % 7])


def fake_iters(w):
    return 3 + int(abs(w.real)) % 5


class FakeEngine:
    def __init__(self, key, slots, clock, log, dt=0.01):
        self.key, self.slots, self.clock, self.log, self.dt = key, slots, clock, log, dt
        self.pts = {}   # slot -> [tag, omega, remaining]
        self.closed = False
        self.launched = False
        log.append(("create", key, clock()))

    @property
    def active(self):
        return len(self.pts)

    def admit(self, omegas, tags):
        n = 0
        for w, t in zip(omegas, tags):
            free = [s for s in range(self.slots) if s not in self.pts]
            if not free:
                break
            self.pts[free[0]] = [int(t), complex(w), fake_iters(complex(w))]
            self.log.append(("admit", self.key, int(t), self.clock()))
            n += 1
        return n

    def launch(self):
        assert not self.launched and self.pts
        self.launched = True

    def ready(self):
        return True

    def finish(self):
        assert self.launched
        self.launched = False
        self.clock.t += self.dt
        out = []
        for s in list(self.pts):
            p = self.pts[s]
            p[2] -= 1
            if p[2] == 0:
                out.append(Res(p[0], fake_result(self.key, p[1]), fake_iters(p[1]), 1e-9))
                del self.pts[s]
        return out

    def close(self):
        self.closed = True
        self.log.append(("close", self.key, self.clock()))


def make_server(slots, budget, per_engine, clock, log):
    return Server(lambda key, n: FakeEngine(key, n, clock, log), lambda key, n: per_engine, slots, budget,
                  clock=clock, sleep=clock.sleep)


def test_every_point_gets_its_alone_result():
    clock, log = FakeClock(), []
    rng = np.random.default_rng(1)
    reqs = [Request(i, i % 3, rng.uniform(-10, 30, 7) + 0.5j, arrival=0.05 * i) for i in range(6)]
    out, st = make_server(4, 10, 1, clock, log).run(reqs)
    assert len(out) == sum(len(r.omegas) for r in reqs) == st.points
    for o in out:
        r = reqs[o.rid]
        assert o.omega == r.omegas[o.index]
        np.testing.assert_allclose(o.S, fake_result(r.key, complex(o.omega)))
        assert o.iters == fake_iters(complex(o.omega))
        assert o.arrival <= o.admitted <= o.done


def test_retired_slots_are_refilled():
    clock, log = FakeClock(), []
    w = np.array([0.5, 1.5, 2.5, 3.5, 4.5, 0.5, 1.5]) + 0.1j   # 3..7 iterations each
    out, st = make_server(2, 10, 1, clock, log).run([Request(0, 0, w)])
    iters = [fake_iters(complex(x)) for x in w]
    # two slots working in parallel: fewer steps than one point after another
    assert st.steps < sum(iters)
    assert st.steps >= sum(iters) / 2
    admits = [e for e in log if e[0] == "admit"]
    assert len(admits) == len(w)
    # later points are admitted only after earlier ones retire (never more than 2 in flight)
    assert max(sum(1 for a in admits if a[3] <= o.done) - sum(1 for p in out if p.done <= o.done)
               for o in out) <= 2


def test_points_are_not_admitted_before_arrival():
    clock, log = FakeClock(), []
    reqs = [Request(0, 0, np.array([1.0 + 0.1j]), arrival=0.0), Request(1, 0, np.array([2.0 + 0.1j]), arrival=1.0)]
    out, st = make_server(4, 10, 1, clock, log).run(reqs)
    by = {o.rid: o for o in out}
    assert by[1].admitted >= 1.0
    assert by[1].latency == pytest.approx(by[1].done - 1.0)
    assert st.percentile(50) > 0


def test_memory_budget_limits_resident_engines():
    clock, log = FakeClock(), []
    reqs = [Request(i, i, np.array([1.0, 2.0, 3.0]) + 0.1j) for i in range(3)]
    out, st = make_server(2, 10, 6, clock, log).run(reqs)   # one engine of 6 fits in 10
    assert st.peak_engines == 1 and st.peak_bytes <= 10
    assert len(out) == 9
    creates = [e for e in log if e[0] == "create"]
    closes = [e for e in log if e[0] == "close"]
    assert len(creates) == 3 and len(closes) == 3
    # an engine is closed before the next one is created
    order = [e[0] for e in log if e[0] in ("create", "close")]
    assert order == ["create", "close", "create", "close", "create", "close"]


def test_two_engines_are_resident_within_budget():
    clock, log = FakeClock(), []
    reqs = [Request(0, "a", np.array([4.5, 4.5]) + 0.1j), Request(1, "b", np.array([4.5, 4.5]) + 0.1j)]
    out, st = make_server(2, 10, 5, clock, log).run(reqs)
    assert st.peak_engines == 2
    assert st.steps == 2 * fake_iters(4.5 + 0.1j)   # evaluations launched, both engines
    assert len(out) == 4


class TimedEngine(FakeEngine):
    """An evaluation takes dt of (fake) device time after its launch: ready() is false
    until then, and finish() waits for it."""

    def launch(self):
        super().launch()
        self.t_launch = self.clock.t

    def ready(self):
        return not self.launched or self.clock.t >= self.t_launch + self.dt

    def finish(self):
        assert self.launched
        self.launched = False
        self.clock.t = max(self.clock.t, self.t_launch + self.dt)
        out = []
        for sl in list(self.pts):
            pt = self.pts[sl]
            pt[2] -= 1
            if pt[2] == 0:
                out.append(Res(pt[0], fake_result(self.key, pt[1]), fake_iters(pt[1]), 1e-9))
                del self.pts[sl]
        return out


def test_engines_step_at_their_own_pace():
    """A point on a fast engine is not held to the pace of a slow one."""
    clock, log = FakeClock(), []
    dts = {"slow": 1.0, "fast": 0.1}
    srv = Server(lambda key, n: TimedEngine(key, n, clock, log, dt=dts[key]), lambda key, n: 1, slots=2,
                 budget_bytes=10, clock=clock, sleep=clock.sleep, poll=0.01)
    w = np.array([2.0 + 0.1j])   # fake_iters = 5 evaluations
    out, st = srv.run([Request(0, "slow", w), Request(1, "fast", w)])
    by = {o.rid: o for o in out}
    assert by[1].done == pytest.approx(5 * 0.1, abs=0.05)
    assert by[0].done == pytest.approx(5 * 1.0, abs=0.05)
    assert by[1].iters == by[0].iters == 5


def test_slot_bytes_grow_with_history_and_precision():
    assert slot_bytes(1000, 50, True) > slot_bytes(1000, 50, False) > slot_bytes(1000, 5, False)
    assert slot_bytes(94482, 50, True) < 400e6
    # the statistical FAM (P, Q quadrants) doubles the QP-state arrays
    assert 1.9 < slot_bytes(1000, 50, False, True) / slot_bytes(1000, 50, False) < 2.0


def test_poisson_arrivals():
    a = poisson_arrivals(2000, 100.0, seed=3)
    assert np.all(np.diff(a) >= 0)
    assert 15.0 < a[-1] < 25.0
