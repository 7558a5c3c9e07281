"""Extract golden vectors from the reference's recorded pnfam_main runs.

Run once, in a checkout that has the reference repository next to it
(``python tests/golden/make_golden.py <reference-root>``).  For each recorded
case it copies the HFBTHO ``.hel`` ground state (the solver input) and writes
``<case>.json`` with, per operator and omega point, the namelist values the
point was run with and the reference's FP64 output: the iteration table
(si, Re S, Im S per iteration, 10 decimals) and the final 19-digit strength
and cross terms.  Only outputs of one-body runs (two_body_current_mode = 0)
are taken.
"""
from __future__ import annotations

import io
import json
import os
import re
import shutil
import sys
import tarfile

HERE = os.path.dirname(os.path.abspath(__file__))
# 40S in the N_sh = 8 basis (parity-split blocks up to 25, 165 states): the
# reference's recorded GT runs on it are empty
INPUT_ONLY = {"S40_nsh8": "S40_GT_2bc_reruntest/000000"}
CASES = {
    # case name -> directory (relative to <reference>/tests)
    "S40": "S40_GT_All/000000",
    "Gd162": "Gd162_GT_open/000000",
    "Kr116": "pynfam_test/000000",
}


def parse_dat(text: str) -> dict:
    out = {"history": [], "converged": None, "result": {}}
    for line in text.splitlines():
        m = re.match(r"#\s+(\d+)([NLB])\s+([-\d.Ee+]+)\s+([-\d.Ee+]+)\s+([-\d.Ee+]+)\s+([-\d.Ee+]+)", line)
        if m:
            out["history"].append([int(m.group(1)), m.group(2), float(m.group(3)), float(m.group(4)), float(m.group(5))])
            continue
        if "FAM iteration converged" in line:
            out["converged"] = int(re.search(r"after\s+(\d+)", line).group(1))
        elif "FAM iteration interrupted" in line:
            out["converged"] = -1
        if not line.startswith("#") and line.strip() and "Real" not in line:
            parts = line.split()
            if len(parts) == 3:
                out["result"][parts[0]] = [float(parts[1]), float(parts[2])]
    return out


def parse_in(text: str) -> dict:
    vals = {}
    for key in ("real_eqrpa", "imag_eqrpa", "operator_name", "operator_k", "beta_type", "compute_crossterms",
                "max_iter", "convergence_epsilon", "broyden_history_size", "quench_residual_int",
                "two_body_current_mode"):
        m = re.search(rf"^\s*{key}\s*=\s*(.+?)\s*$", text, re.M)
        if m:
            raw = m.group(1).strip()
            v = raw.strip("'\"")
            if raw[:1] in ("'", '"'):
                pass
            elif v in (".true.", "T"):
                v = True
            elif v in (".false.", "F"):
                v = False
            else:
                try:
                    v = int(v)
                except ValueError:
                    try:
                        v = float(v)
                    except ValueError:
                        pass
            vals[key] = v
    return vals


def main(ref_root: str):
    for case, rel in CASES.items():
        src = os.path.join(ref_root, "tests", rel)
        shutil.copyfile(os.path.join(src, "hfb_soln", "hfbtho_output.hel"), os.path.join(HERE, f"{case}.hel"))
        meta = os.path.join(src, "fam_soln", "fam_meta")
        ops = {}
        interaction = None
        for tname in sorted(os.listdir(meta)):
            if not tname.endswith(".tar"):
                continue
            label = tname[:-4]
            with tarfile.open(os.path.join(meta, tname)) as tf:
                pts = {}
                for mem in tf.getmembers():
                    if not mem.isfile():
                        continue
                    d, f = os.path.split(mem.name)
                    idx = os.path.basename(d)
                    data = tf.extractfile(mem).read().decode(errors="replace")
                    pts.setdefault(idx, {})[f.rsplit(".", 1)[1]] = data
            points = []
            for idx in sorted(pts):
                rec = pts[idx]
                if "in" not in rec or "dat" not in rec:
                    continue
                nml = parse_in(rec["in"])
                grp = re.search(r"&interaction(.*?)^\s*/", rec["in"], re.S | re.M).group(1)
                grp = "\n".join(l.strip() for l in grp.strip().splitlines())
                if interaction is None:
                    interaction = grp
                elif grp != interaction:
                    raise SystemExit(f"{case}: &interaction differs between points")
                if nml.get("two_body_current_mode", 0) != 0:
                    continue
                res = parse_dat(rec["dat"])
                if not res["result"]:
                    continue
                points.append({"index": idx, "namelist": nml, **res})
            if points:
                ops[label] = points
        with open(os.path.join(HERE, f"{case}.json"), "w") as fh:
            json.dump({"case": case, "source": f"tests/{rel}", "interaction": "&interaction\n" + interaction + "\n/\n",
                       "operators": ops}, fh, separators=(",", ":"))
        print(case, {k: len(v) for k, v in ops.items()})
    # ground states without recorded FAM outputs (their .dat files are empty): inputs
    # of the oracle-versus-GPU parity tests
    for case, rel in INPUT_ONLY.items():
        shutil.copyfile(os.path.join(ref_root, "tests", rel, "hfb_soln", "hfbtho_output.hel"),
                        os.path.join(HERE, f"{case}.hel"))
        print(case, "ground state only")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
