"""The N_sh = 16 benchmark workload pinned to the CPU oracle.

tests/golden/nsh16_oracle.json holds the oracle's (oracle/fam_oracle.py) fixed
point at epsilon 1e-12 and first iterations for points of every operator of the
benchmark (tests/golden/make_nsh16_oracle.py).  The benchmark's accuracy
reference, tests/golden/bench_fixed_point_nsh16.json, is the GPU's FP64 form at
the same epsilon: here it is held to the oracle (1e-8 relative per Re/Im value),
and the GPU's first five iterations to the oracle's (1e-9).
"""
import json
import os

import numpy as np
import pytest

from golden_cases import GOLDEN

import bench

PIN = os.path.join(GOLDEN, "nsh16_oracle.json")


def _pins():
    with open(PIN) as fh:
        return json.load(fh)


def test_pins_are_for_the_benchmark_workload():
    d = _pins()
    assert d["signature"] == bench.signature()
    ops = {tuple(p["operator"]) for p in d["points"]}
    assert ops == set(bench.OPERATORS)
    # a point next to the real axis is among them (Re omega = -15 MeV end of the contour)
    assert any(p["index"] == bench.POINTS - 1 for p in d["points"])
    assert sum(p["iter_conv"] > 0 for p in d["points"]) >= 4


def test_benchmark_fixed_point_matches_oracle():
    fp = bench.load_fixed_point()
    assert fp is not None, "bench_fixed_point_nsh16.json is not for the benchmark workload"
    n = 0
    for p in _pins()["points"]:
        if p["iter_conv"] < 0:
            continue
        got = fp[tuple(p["operator"])]["S"][p["index"]]
        assert got is not None, p["operator"]
        want = np.array([complex(*x) for x in p["S"]])
        got = np.array([complex(*x) for x in got])
        assert got.shape == want.shape
        scale = abs(want[0])
        for g, w in zip(got, want):
            for a, b in ((g.real, w.real), (g.imag, w.imag)):
                assert abs(a - b) <= 1e-8 * abs(b) + 1e-12 * scale, (p["operator"], p["index"], a, b)
        n += 1
    assert n >= 4


@pytest.mark.gpu
def test_gpu_first_iterations_match_oracle_at_nsh16():
    """The FP64 form's first five iterations (si, Re S, Im S) at N_sh = 16 against the oracle."""
    from pynfam_gb300.solver import GPUSolver
    pins = _pins()["points"]
    cases, omegas = bench.workload()
    by_op = {op: c for op, c in zip(bench.OPERATORS, cases)}
    for p in pins:
        c = by_op[tuple(p["operator"])]
        gpu = GPUSolver(c.hfb, c.couplings)
        gpu.set_operator(c.F, c.G)
        s = c.nml["solver"]
        n = len(p["history"]) - 1
        r = gpu.solve([complex(*p["omega"])], max_iter=n, eps=1e-30, broyden_m=s["broyden_history_size"],
                      quench=c.quench, history=True)
        gpu.close()
        for it, si, re, im in p["history"]:
            g = r.hist[0, it]
            assert abs(g[0] - si) <= 1e-9 * max(abs(si), 1e-6), (p["operator"], it, g, si)
            assert abs(g[1] - re) <= 1e-9 * max(abs(re), 1e-6), (p["operator"], it, g, re)
            assert abs(g[2] - im) <= 1e-9 * max(abs(im), 1e-6), (p["operator"], it, g, im)
