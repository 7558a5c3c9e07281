"""Pins the CPU oracle to the reference's recorded FP64 pnfam_main output.

Each case rebuilds the ground state from the recorded .hel file, runs the
oracle for a recorded (operator, omega) point and compares the final strength
(and cross terms) with the recorded 19-digit values, plus the whole recorded
iteration table (si, Re S, Im S printed with 10 decimals).
"""
import numpy as np
import pytest

from golden_cases import case_for
from oracle.fam_oracle import FAMOracle

POINTS = [("S40", "GT-K0", 0), ("S40", "GT-K1", 7), ("S40", "F-K0", 3), ("S40", "P-K1", 12),
          ("S40", "RS0-K0", 20), ("S40", "RS2-K2", 5), ("Gd162", "GT-K1", 30), ("Kr116", "P-K0", 4)]

REL = 1e-6


def run(case, op, idx):
    c, pt = case_for(case, op, idx)
    s = c.nml["solver"]
    orc = FAMOracle(c.hfb, c.couplings, c.F, c.G, quench=c.quench)
    r = orc.solve(c.omega, max_iter=s["max_iter"], eps=s["convergence_epsilon"], broyden_m=s["broyden_history_size"])
    return c, pt, orc, r


@pytest.mark.parametrize("case,op,idx", POINTS)
def test_oracle_matches_recorded(case, op, idx):
    c, pt, orc, r = run(case, op, idx)
    assert r.iter_conv == pt["converged"]
    labels = ["Strength"] + orc.xlabels
    for k, lab in enumerate(labels):
        want = pt["result"][lab]
        for got, w in ((r.re_str[k], want[0]), (r.im_str[k], want[1])):
            assert abs(got - w) <= REL * abs(w) + 1e-13, (lab, got, w)
    # the recorded iteration table, 10 printed decimals
    for (it, flag, si, re, im), h in zip(pt["history"], r.history):
        assert it == h[0] and flag == h[1]
        assert abs(si - h[2]) < 1.5e-10 * max(1.0, abs(si)) + 6e-11
        assert abs(re - h[3]) < 6e-11 + 1e-9 * abs(re)
        assert abs(im - h[4]) < 6e-11 + 1e-9 * abs(im)


def _counts():
    from golden_cases import oracle_counts
    return oracle_counts()


def test_oracle_iteration_counts_match_recorded_runs():
    """The oracle stops at the recorded iteration on all but a handful of the 594
    recorded points; those few lie inside the window the GPU test allows for
    rounding-sensitive stopping steps (tests/golden/oracle_counts.json, made by
    tests/golden/make_oracle_counts.py)."""
    from golden_cases import count_window, golden
    d = _counts()
    total = same = 0
    for case, ops in d["counts"].items():
        for op, lst in ops.items():
            pts = golden(case)["operators"][op]
            assert len(lst) == len(pts)
            for p, o in zip(pts, lst):
                total += 1
                same += o[0] == p["converged"]
                want, slack = count_window(p, {"near": d["near"], "point": o})
                assert want >= 0 and abs(p["converged"] - want) <= slack
    assert total == 594 and same >= 580, (total, same)


@pytest.mark.parametrize("case,op,idx", [("S40", "GT-K0", 27), ("S40", "PS0-K0", 3), ("Kr116", "P-K0", 10)])
def test_oracle_counts_fixture_is_the_oracle(case, op, idx):
    _, pt, _, r = run(case, op, idx)
    assert _counts()["counts"][case][op][idx][0] == r.iter_conv
