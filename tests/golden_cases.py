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
