"""Record the CPU oracle's convergence step for every recorded reference point.

``python tests/golden/make_oracle_counts.py [workers]`` runs the oracle
(oracle/fam_oracle.py) on every recorded (case, operator, omega) point of
tests/golden/<case>.json, with the namelist values of the run, and writes
tests/golden/oracle_counts.json:

    {case: {operator: [[iter_conv, first_near], ...]}}   (one pair per point)

``iter_conv`` is the oracle's iteration count (-1 if it did not converge) and
``first_near`` the first iteration at which the oracle's si came within 5 eps
of the threshold (None if never before convergence).

Why: the reference stops at the first iteration with si < eps
(pnfam_solver.f90:127).  Where si falls through eps decisively, two correct
FP64 implementations stop at the same step; where it lingers near eps, or
where the Broyden trajectory is sensitive enough that rounding differences
grow to the size of si itself, the stopping step moves by a few iterations
between implementations (the oracle and the recorded runs already differ
there).  The GPU parity test holds the device's count to the oracle's count
on the same inputs with an allowance that grows with that lingering.
"""
from __future__ import annotations

import json
import multiprocessing as mp
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
CASES = ("S40", "Gd162", "Kr116", "S40_2bc_fam", "S40_2bc_dme", "S40_2bc_ps0", "Gd162_2bc_p",
         "S40_2bc_p_dme", "S40_2bc_ps0_dme")
NEAR = 5.0   # "near the threshold": si < NEAR * eps


def _paths():
    for p in (ROOT, os.path.join(ROOT, "tests")):
        if p not in sys.path:
            sys.path.insert(0, p)


def one(job):
    _paths()
    from golden_cases import case_for
    from oracle.fam_oracle import FAMOracle
    case, op, idx = job
    c, pt = case_for(case, op, idx)
    s = c.nml["solver"]
    orc = FAMOracle(c.hfb, c.couplings, c.F, c.G, quench=c.quench)
    r = orc.solve(c.omega, max_iter=s["max_iter"], eps=s["convergence_epsilon"],
                  broyden_m=s["broyden_history_size"])
    eps = s["convergence_epsilon"]
    stop = r.iter_conv if r.iter_conv >= 0 else s["max_iter"] + 1
    near = [int(h[0]) for h in r.history if int(h[0]) < stop and float(h[2]) < NEAR * eps]
    return job, [int(r.iter_conv), near[0] if near else None]


def main(workers: int) -> None:
    _paths()
    from golden_cases import golden
    jobs = [(case, op, i) for case in CASES for op in sorted(golden(case)["operators"])
            for i in range(len(golden(case)["operators"][op]))]
    out = {case: {op: [None] * len(golden(case)["operators"][op]) for op in golden(case)["operators"]}
           for case in CASES}
    with mp.get_context("spawn").Pool(workers) as pool:
        for n, ((case, op, i), rec) in enumerate(pool.imap_unordered(one, jobs, chunksize=1)):
            out[case][op][i] = rec
            if n % 50 == 0:
                print(f"{n}/{len(jobs)}", flush=True)
    with open(os.path.join(HERE, "oracle_counts.json"), "w") as fh:
        json.dump({"near": NEAR, "counts": out}, fh, separators=(",", ":"))


if __name__ == "__main__":
    main(int(sys.argv[1]) if len(sys.argv) > 1 else os.cpu_count() or 1)
