"""Pin the N_sh = 16 benchmark workload to the CPU oracle.

``python tests/golden/make_nsh16_oracle.py [workers]`` runs the oracle
(oracle/fam_oracle.py, FP64 numpy restatement of the reference solver) on a few
points of the benchmark's workload (bench.py: the 162Gd ground state in the
N_sh = 16 basis, beta- GT K = 0, 1 and first-forbidden RS1 K = 0, 1, RS2 K = 2
with their cross terms, the 120-point CIRCLE contour), to epsilon 1e-12 with the
reference's Broyden settings, and writes tests/golden/nsh16_oracle.json:

    {"points": [{"operator": [name, K], "index": i, "omega": [re, im],
                 "iter_conv": n, "S": [[re, im], ...]  (strength, cross terms),
                 "history": [[it, si, Re S, Im S], ...]  (iterations 0-5)}]}

The chosen points are mid-contour points of every operator and the last contour
point (Re omega = -15 MeV, next to the real axis).  The benchmark's accuracy
reference (tests/golden/bench_fixed_point_nsh16.json, the GPU's FP64 form at
1e-12) is checked against these values on the CPU, and the GPU's first
iterations against the stored history, so the headline's reference is not the
GPU's own output alone.
"""
from __future__ import annotations

import json
import multiprocessing as mp
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
# (operator index in bench.OPERATORS, contour index)
PICKS = ((0, 60), (0, 119), (1, 30), (2, 90), (3, 45), (4, 100))
EPS = 1e-12
MAX_ITER = 600
HISTORY = 6


def _paths():
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)


def one(pick):
    _paths()
    import bench
    from oracle.fam_oracle import FAMOracle
    k, i = pick
    cases, omegas = bench.workload(bench.POINTS, (bench.OPERATORS[k],))
    c = cases[0]
    s = c.nml["solver"]
    orc = FAMOracle(c.hfb, c.couplings, c.F, c.G, quench=c.quench)
    w = complex(omegas[i])
    r = orc.solve(w, max_iter=MAX_ITER, eps=EPS, broyden_m=s["broyden_history_size"])
    return {"operator": list(bench.OPERATORS[k]), "index": i, "omega": [w.real, w.imag],
            "iter_conv": int(r.iter_conv),
            "S": [[float(a), float(b)] for a, b in zip(r.re_str, r.im_str)],
            "history": [[int(h[0]), float(h[2]), float(h[3]), float(h[4])] for h in r.history[:HISTORY]]}


def main(workers: int) -> None:
    _paths()
    import bench
    with mp.get_context("spawn").Pool(workers) as pool:
        pts = pool.map(one, PICKS, chunksize=1)
    for p in pts:
        print(p["operator"], p["index"], p["iter_conv"], p["S"][0], flush=True)
    with open(os.path.join(HERE, "nsh16_oracle.json"), "w") as fh:
        json.dump({"signature": bench.signature(), "epsilon": EPS, "points": pts}, fh, indent=1)


if __name__ == "__main__":
    main(int(sys.argv[1]) if len(sys.argv) > 1 else len(PICKS))
