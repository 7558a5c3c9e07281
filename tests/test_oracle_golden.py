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
