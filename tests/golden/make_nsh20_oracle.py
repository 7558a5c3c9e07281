"""Oracle history of the large-basis stress configuration (N_sh = 20).

``python tests/golden/make_nsh20_oracle.py`` builds the synthetic Bogoliubov
ground state of the stress configuration (pynfam_gb300.synthetic.
bogoliubov_nucleus: seed 3, the full N_sh = 20 basis with Omega-only blocks, the
largest 231 states, on the recorded 162Gd mesh), sets up beta- GT K = 0 and K = 1
with the SkO' residual interaction, runs the CPU oracle (oracle/fam_oracle.py)
for four FAM iterations at one omega each and writes
tests/golden/nsh20_oracle.json:

    {"omega": [re, im], "operators": {"GT-K0": [[it, si, Re S, Im S], ...], ...}}

The GPU test of the configuration (tests/test_configs.py) compares the device's
first four iterations with these.
"""
from __future__ import annotations

import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OMEGA = complex(6.0, 0.5)
ITERS = 4
NSH = 20
SEED = 3


def main() -> None:
    for p in (ROOT, os.path.join(ROOT, "tests")):
        if p not in sys.path:
            sys.path.insert(0, p)
    from oracle.fam_oracle import FAMOracle
    from pynfam_gb300.synthetic import bogoliubov_nucleus
    from test_configs import _case
    hfb = bogoliubov_nucleus(os.path.join(HERE, "Gd162.hel"), NSH, seed=SEED, parity=False)
    out = {"omega": [OMEGA.real, OMEGA.imag], "nsh": NSH, "seed": SEED, "dqp": int(hfb.dqp),
           "max_block": int(max(hfb.db)), "operators": {}, "nxy": {}}
    for k in (0, 1):
        c = _case(hfb, k, 50, self_consistent=False)
        orc = FAMOracle(c.hfb, c.couplings, c.F, c.G, quench=c.quench)
        r = orc.solve(OMEGA, max_iter=ITERS, eps=1e-30, broyden_m=50)
        out["operators"][f"GT-K{k}"] = [[int(h[0]), float(h[2]), float(h[3]), float(h[4])] for h in r.history]
        out["nxy"][f"GT-K{k}"] = int(c.F.mat.nelem)
        print(k, out["operators"][f"GT-K{k}"], flush=True)
    with open(os.path.join(HERE, "nsh20_oracle.json"), "w") as fh:
        json.dump(out, fh, indent=1)


if __name__ == "__main__":
    main()
