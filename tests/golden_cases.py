"""Helpers that turn the recorded reference runs (tests/golden/*.json) into
solver inputs.  Shared by the CPU oracle tests and the GPU parity tests."""
import functools
import json
import os

from pynfam_gb300.hfb_solution import load_hfb_solution
from pynfam_gb300.namelist import defaults, parse_namelist_text
from pynfam_gb300.pnfam_setup import setup_case

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@functools.lru_cache(maxsize=None)
def golden(case):
    with open(os.path.join(GOLDEN, f"{case}.json")) as fh:
        return json.load(fh)


@functools.lru_cache(maxsize=None)
def hfb(case):
    return load_hfb_solution(os.path.join(GOLDEN, f"{case}.hel"))


def namelist_for(case, point):
    g = golden(case)
    nml = defaults()
    nml["interaction"].update(parse_namelist_text(g["interaction"])["interaction"])
    p = point["namelist"]
    for k in ("operator_name", "operator_k", "beta_type", "compute_crossterms"):
        nml["ext_field"][k] = p[k]
    for k in ("two_body_current_mode", "two_body_current_usep", "two_body_current_lecs"):
        if k in p:
            nml["ext_field"][k] = p[k]
    if "fam_output_filename" in p:
        nml["general"]["fam_output_filename"] = p["fam_output_filename"]
    for k in ("max_iter", "convergence_epsilon", "broyden_history_size", "quench_residual_int"):
        nml["solver"][k] = p[k]
    nml["general"]["real_eqrpa"] = p["real_eqrpa"]
    nml["general"]["imag_eqrpa"] = p["imag_eqrpa"]
    return nml


def case_for(case, op, index=0):
    """Solver inputs of a recorded point; two-body-current cases read their
    cached finite-range fields from tests/golden/<case>/ and apply the
    constants of the reference revision that recorded them."""
    g = golden(case)
    pt = g["operators"][op][index]
    tbc_dir = os.path.join(GOLDEN, g["tbc_dir"]) if g.get("tbc_dir") else GOLDEN
    return setup_case(namelist_for(case, pt), None, hfb=hfb(case), tbc_dir=tbc_dir,
                      twobc_revision=g.get("revision") or None), pt


def recorded_values(point, labels):
    """Recorded (re, im) per output row, in solver order [Strength, cross terms...]."""
    res = point["result"]
    return [res[l] for l in labels]


@functools.lru_cache(maxsize=None)
def oracle_counts():
    """The oracle's convergence step and first near-threshold iteration of every
    recorded point (tests/golden/make_oracle_counts.py)."""
    with open(os.path.join(GOLDEN, "oracle_counts.json")) as fh:
        return json.load(fh)


def count_window(point, oracle):
    """(expected iteration count, allowance) of a recorded point.

    The FAM stops at the first iteration with si < eps (`pnfam_solver.f90:127`).  Two
    correct FP64 implementations stop at the same step where si falls through eps
    decisively; where si lingers within 5 eps of the threshold for several iterations
    before crossing it (¹⁶²Gd GT-K0 at omega = 2.746 + 0.1i: iterations 52 to 62 of
    the recorded run), rounding differences pick another iteration of that stretch.
    The expected count is the oracle's on the same inputs; the allowance is 2 plus
    the longer of the two near-threshold stretches (the recorded run's and the
    oracle's) beyond two iterations, plus the spread between the recorded run and the
    oracle themselves."""
    near = oracle["near"]
    eps = point["namelist"]["convergence_epsilon"]
    rec = point["converged"]
    orc_conv, orc_first = oracle["point"]
    rec_near = [h[0] for h in point["history"] if h[0] < rec and h[2] < near * eps]
    stretch = max(rec - rec_near[0] if rec_near else 0,
                  orc_conv - orc_first if orc_first is not None and orc_conv >= 0 else 0)
    return orc_conv, 2 + max(0, stretch - 2) + abs(rec - orc_conv)
