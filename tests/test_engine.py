"""Continuous batching on the GPU (pnfam_gpu_engine_* through the C ABI).

1. An engine with fewer slots than points (slots refilled as points retire)
   gives every point the result and iteration count of the batch solve.
2. Serving a mix of requests of two nuclei/operators (two engines stepping
   together, overlapping on the GPU) gives every point its result alone,
   within the 1e-6 relative tolerance, for the FP64 and the mixed form.
3. Misuse is refused with an error code, not a crash.
"""
import numpy as np
import pytest

from golden_cases import case_for, golden

pytestmark = pytest.mark.gpu

REL = 1e-6


def _omegas(case, op):
    return np.array([complex(p["namelist"]["real_eqrpa"], p["namelist"]["imag_eqrpa"])
                     for p in golden(case)["operators"][op]])


def _kw(c):
    s = c.nml["solver"]
    return dict(max_iter=s["max_iter"], eps=s["convergence_epsilon"], broyden_m=s["broyden_history_size"],
                quench=c.quench)


def test_engine_refills_slots_and_matches_batch_solve():
    from pynfam_gb300.solver import GPUSolver
    c, _ = case_for("S40", "GT-K0", 0)
    w = _omegas("S40", "GT-K0")
    gpu = GPUSolver(c.hfb, c.couplings)
    gpu.set_operator(c.F, c.G)
    ref = gpu.solve(w, **_kw(c))
    eng = gpu.engine(7, **_kw(c))
    todo = list(range(len(w)))
    got = {}
    steps = 0
    while todo or eng.active:
        free = eng.slots - eng.active
        if todo and free:
            take, todo = todo[:free], todo[free:]
            assert eng.admit(w[take], take) == len(take)
        eng.launch()
        steps += 1
        for r in eng.finish():
            got[r.tag] = r
    eng.close()
    gpu.close()
    assert sorted(got) == list(range(len(w)))
    assert steps < int(np.sum(ref.iters)) / 3   # points overlapped in the slots
    # the same kernels, sums and Broyden steps per point whatever else is in flight
    worst = 0.0
    for i in range(len(w)):
        assert got[i].iters == ref.iters[i], (i, got[i].iters, ref.iters[i])
        want = ref.re_S[i] + 1j * ref.im_S[i]
        rel = np.max(np.abs(got[i].S - want)) / np.max(np.abs(want))
        worst = max(worst, rel)
        assert rel <= 1e-13, (i, rel)
    print(f"engine vs batch solve: {steps} steps, worst relative difference {worst:.1e}")


@pytest.mark.parametrize("precision", [0, 1])
def test_served_mix_matches_each_point_alone(precision):
    from pynfam_gb300.serve import Request, Server
    from pynfam_gb300.solver import GPUSolver
    pairs = {("S40", "GT-K0"): case_for("S40", "GT-K0", 0)[0], ("Kr116", "P-K0"): case_for("Kr116", "P-K0", 0)[0]}
    eps = 1e-7 if precision == 0 else 1e-9
    solvers = {}

    def factory(key, slots):
        c = pairs[key]
        g = GPUSolver(c.hfb, c.couplings)
        g.set_operator(c.F, c.G)
        solvers[key] = g
        kw = _kw(c)
        kw["eps"] = eps
        return g.engine(slots, precision=precision, **kw)

    rng = np.random.default_rng(5)
    reqs, rid = [], 0
    for key in pairs:
        w = _omegas(*key)
        for chunk in np.array_split(rng.permutation(len(w)), 3):
            reqs.append(Request(rid, key, w[chunk], arrival=0.0))
            rid += 1
    rng.shuffle(reqs)
    out, st = Server(factory, lambda key, n: 1, slots=6, budget_bytes=10).run(reqs)
    assert st.peak_engines == 2 and len(out) == sum(len(r.omegas) for r in reqs)
    by_req = {r.rid: r for r in reqs}
    for key, c in pairs.items():
        g = GPUSolver(c.hfb, c.couplings)
        g.set_operator(c.F, c.G)
        kw = _kw(c)
        kw["eps"] = eps
        mine = [o for o in out if by_req[o.rid].key == key]
        alone = g.solve(np.array([o.omega for o in mine]), precision=precision, **kw)
        g.close()
        scale = np.max(np.abs(alone.re_S[:, 0] + 1j * alone.im_S[:, 0]))
        for k, o in enumerate(mine):
            want = alone.re_S[k] + 1j * alone.im_S[k]
            assert o.iters >= 0 and alone.iters[k] >= 0
            for g_, w_ in zip(o.S, want):
                for a, b in ((g_.real, w_.real), (g_.imag, w_.imag)):
                    assert abs(a - b) <= REL * abs(b) + 1e-12 * scale, (key, k, a, b)
    for g in solvers.values():
        g.close()
    print(f"precision {precision}: {st.points} points, {st.steps} steps, p50 {st.percentile(50) * 1e3:.1f} ms, "
          f"p99 {st.percentile(99) * 1e3:.1f} ms")


def test_asynchronous_anchors_give_each_point_its_result():
    """Mixed form with asynchronous anchors (opts.reserved[5]): points whose FP64 anchor
    runs beside other points' FP32 increments are parked until it completes, while the
    engine keeps stepping the others.  Every point converges to the result of the
    synchronous batch solve within 1e-6 per Re/Im value of the strength and each cross
    term (both within 1e-9 of the same fixed point)."""
    from pynfam_gb300.solver import GPUSolver
    c, _ = case_for("S40", "RS1-K1", 0)
    w = _omegas("S40", "RS1-K1")
    gpu = GPUSolver(c.hfb, c.couplings)
    gpu.set_operator(c.F, c.G)
    kw = _kw(c)
    kw.update(eps=1e-9, precision=1, settle=8, max_iter=300)
    ref = gpu.solve(w, **kw)
    eng = gpu.engine(9, async_anchors=True, **kw)
    todo = list(range(len(w)))
    got = {}
    while todo or eng.active:
        free = eng.slots - eng.active
        if todo and free:
            take, todo = todo[:free], todo[free:]
            assert eng.admit(w[take], take) == len(take)
        eng.launch()
        for r in eng.finish():
            got[r.tag] = r
    prof, _ = gpu.last_profile()
    eng.close()
    gpu.close()
    assert sorted(got) == list(range(len(w)))
    scale = np.max(np.abs(ref.re_S[:, 0] + 1j * ref.im_S[:, 0]))
    for i in range(len(w)):
        assert got[i].iters >= 0 and ref.iters[i] >= 0, i
        want = ref.re_S[i] + 1j * ref.im_S[i]
        for g_, w_ in zip(got[i].S, want):
            for a, b in ((g_.real, w_.real), (g_.imag, w_.imag)):
                assert abs(a - b) <= REL * abs(b) + 1e-12 * scale, (i, a, b)
    assert prof["point_iterations_fp64"] > 0 and prof["point_iterations_fp32"] > 0


def test_engine_misuse_is_refused():
    from pynfam_gb300 import _lib
    from pynfam_gb300.solver import GPUSolver
    c, _ = case_for("S40", "GT-K0", 0)
    gpu = GPUSolver(c.hfb, c.couplings)
    gpu.set_operator(c.F, c.G)
    eng = gpu.engine(2, **_kw(c))
    with pytest.raises(_lib.PnfamGPUError) as ei:
        gpu.solve([c.omega], **_kw(c))          # buffers belong to the engine
    assert ei.value.code == 5
    with pytest.raises(_lib.PnfamGPUError):
        gpu.engine(2, **_kw(c))                 # one engine per context
    assert eng.admit(np.array([c.omega] * 3), [0, 1, 2]) == 2   # two free slots
    eng.launch()
    with pytest.raises(_lib.PnfamGPUError):
        eng.launch()                            # an evaluation is in flight
    eng.finish()
    gpu.close()                                 # context freed first: the engine is detached
    with pytest.raises(_lib.PnfamGPUError) as ei:
        eng.launch()
    assert ei.value.code == 5
    eng.close()


def test_autotuner_choices_are_reported_and_cached():
    """The first mixed-form engine of an operator tunes the pair-tensor GEMMs (the density
    task span, the point count from which the pair-tensor path is taken) from timed trial
    evaluations; a second context of the same operator takes the same choices from the
    process's cache without trials."""
    from pynfam_gb300.solver import GPUSolver
    c, _ = case_for("Gd162", "GT-K1", 0)
    kw = _kw(c)
    kw.update(precision=1, eps=1e-9)
    choices = []
    for _ in range(2):
        gpu = GPUSolver(c.hfb, c.couplings)
        gpu.set_operator(c.F, c.G)
        eng = gpu.engine(16, **kw)
        prof, _ = gpu.last_profile()
        choices.append((int(prof["tuned_density_kspan"]), int(prof["tuned_pair_min_points"]), prof["autotune_ms"]))
        eng.close()
        gpu.close()
    (k0, m0, t0), (k1, m1, t1) = choices
    assert k0 in (96, 192, 384, 768) and (m0 in (1, 2, 4, 8, 16) or m0 == 1 << 30)
    assert t0 > 0.0 and (k1, m1) == (k0, m0) and t1 == 0.0
    print(f"Gd162 GT-K1: density task span {k0} K chunks, pair-tensor path from {m0} points, tuning {t0:.0f} ms")
