"""Extract golden vectors from the reference's recorded pnfam_main runs.

Run once, in a checkout that has the reference repository next to it
(``python tests/golden/make_golden.py <reference-root>``).  For each recorded
case it copies the HFBTHO ``.hel`` ground state (the solver input) and writes
``<case>.json`` with, per operator and omega point, the namelist values the
point was run with and the reference's FP64 output: the iteration table
(si, Re S, Im S per iteration, 10 decimals) and the final 19-digit strength
and cross terms.  The one-body cases take only one-body runs
(two_body_current_mode = 0); the two-body-current cases take the first points
of the listed operators, copy the cached finite-range fields (``.tbc``) they
read, and record the constants of the reference revision that produced them
(``revision``: the pair momentum and P-correction sign of the nuclear-matter
corrections, the DME forms), found by matching the recorded strengths.
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
HBARC = 197.3269718


def _p_1361():
    """sqrt(1.2)*1.361/2 fm^-1 evaluated in single precision."""
    import numpy as np
    return float(np.float32(np.float32(np.sqrt(np.float32(1.2))) * np.float32(1.361)) / np.float32(2.0))


# two-body-current cases: name -> (directory, operators, points per operator, revision, .tbc files)
TWO_BODY = {
    # GT full FAM (111100): one-body part with the Park sign + the cached finite-range field
    "S40_2bc_fam": ("S40_All_GT2bc/000000", ("GT-K0", "GT-K1"), 3, {}, ("GT-K0.tbc", "GT-K1.tbc")),
    # GT DME exchange (141100)
    "S40_2bc_dme": ("S40 closed tests/GT_S40_DME_updated/000000", ("GT-K0", "GT-K1"), 3, {}, ()),
    # PS0 nuclear matter at P = 250 MeV (111001); RS0 runs carry it in the RS0xPS0 cross term
    "S40_2bc_ps0": ("S40 closed tests/pynfam_test_S40_0-_2bcP250MeV/000000", ("PS0-K0", "RS0-K0"), 2,
                    {"pair_momentum": 250.0 / HBARC}, ()),
    # P nuclear matter (111010), pair momentum sqrt(1.2)*1.361/2 fm^-1, opposite sign
    "Gd162_2bc_p": ("Gd162 closed tests/1-_2bc/000000", ("P-K0", "P-K1", "R-K1"), 2,
                    {"pair_momentum": None, "p_sign": -1.0}, ()),
    # P DME, constant-density form (111020)
    "S40_2bc_p_dme": ("S40_P_2bc_constdensity/000000", ("P-K0",), 3, {"dme_vector_form": "constant_density"}, ()),
    # PS0 DME, earlier axial-charge form (111002)
    "S40_2bc_ps0_dme": ("S40 closed tests/0-_S40_DME_updated/000000", ("PS0-K0", "RS0-K0"), 2,
                        {"dme_axial_form": "earlier"}, ()),
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
                "two_body_current_mode", "two_body_current_usep", "two_body_current_lecs", "fam_output_filename"):
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
            elif "," in v:
                v = [float(x) for x in v.split(",") if x.strip()]
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


def read_points(meta, label_filter, one_body_only, limit=None):
    """Per operator tar in ``meta``: the recorded points (namelist + output)."""
    ops = {}
    interaction = None
    for tname in sorted(os.listdir(meta)):
        if not tname.endswith(".tar"):
            continue
        label = tname[:-4]
        if label_filter is not None and label not in label_filter:
            continue
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
                raise SystemExit(f"{meta}: &interaction differs between points")
            if one_body_only and nml.get("two_body_current_mode", 0) != 0:
                continue
            res = parse_dat(rec["dat"])
            if not res["result"]:
                continue
            points.append({"index": idx, "namelist": nml, **res})
            if limit and len(points) >= limit:
                break
        if points:
            ops[label] = points
    return ops, interaction


def main(ref_root: str):
    for case, (rel, labels, limit, revision, tbcs) in TWO_BODY.items():
        src = os.path.join(ref_root, "tests", rel)
        shutil.copyfile(os.path.join(src, "hfb_soln", "hfbtho_output.hel"), os.path.join(HERE, f"{case}.hel"))
        ops, interaction = read_points(os.path.join(src, "fam_soln", "fam_meta"), labels, False, limit)
        if tbcs:
            os.makedirs(os.path.join(HERE, case), exist_ok=True)
            for t in tbcs:
                shutil.copyfile(os.path.join(src, "hfb_soln", t), os.path.join(HERE, case, t))
        rev = {k: (_p_1361() if (k == "pair_momentum" and v is None) else v) for k, v in revision.items()}
        with open(os.path.join(HERE, f"{case}.json"), "w") as fh:
            json.dump({"case": case, "source": f"tests/{rel}", "interaction": "&interaction\n" + interaction + "\n/\n",
                       "revision": rev, "tbc_dir": case if tbcs else None, "operators": ops}, fh, separators=(",", ":"))
        print(case, {k: len(v) for k, v in ops.items()})
    for case, rel in CASES.items():
        src = os.path.join(ref_root, "tests", rel)
        shutil.copyfile(os.path.join(src, "hfb_soln", "hfbtho_output.hel"), os.path.join(HERE, f"{case}.hel"))
        ops, interaction = read_points(os.path.join(src, "fam_soln", "fam_meta"), None, True)
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
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <root of the reference checkout>")
    main(sys.argv[1])
