"""``contour_main`` drop-in: strength functions along an energy line, many operators.

The reference's second executable (contour_prog.f90, contour_setup.f90) reads
``pnfam_CONTOUR.dat`` (or the file named on the command line): ``&ctr_general``
(fam_mode, fam_input_filename), ``&ctr_extfield`` (operator_groups,
operator_active) and ``&str_parameters`` (energy_start, energy_step, nr_points,
half_width), takes everything else from the pnfam namelist, and solves
nr_points energies (Re E = energy_start + n * energy_step, n = 0, 1, ...;
Im E = half_width) for the operator of that namelist or, if groups are active,
for every operator of the active J-parity groups (0+: F; 1+: GT K=0,1; 0-: RS0, PS0; 1-: R, P, RS1 K=0,1;
2-: RS2 K=0,1,2, with the sign of K taken from operator_k).  Each point writes its
own ``<op><beta>K<k>_<i>.dat`` (when fam_output_filename is set) and each operator
a summary ``<op><beta>K<k>.out`` (convergence flag, Re E, strength and cross
terms).  The reference reads only the STR parameters, whatever fam_mode says;
so does this driver.

Here the ground state is rebuilt once and stays on the GPU, and all energies of
one operator are solved as one batch (pnfam_gpu_solve).
"""
from __future__ import annotations

import copy
import os
import sys
import time

from . import pnfam_main, txtoutput
from .namelist import NamelistError, parse_namelist_file, read_pnfam_namelist

GROUPS = ("0+", "1+", "0-", "1-", "2-")
# operators of each J-parity group with |K| (contour_setup.f90:167-216)
GROUP_OPS = {0: (("F", 0),), 1: (("GT", 0), ("GT", 1)), 2: (("RS0", 0), ("PS0", 0)),
             3: (("R", 0), ("R", 1), ("P", 0), ("P", 1), ("RS1", 0), ("RS1", 1)),
             4: (("RS2", 0), ("RS2", 1), ("RS2", 2))}


def ctr_defaults() -> dict:
    """init_ctr_namelist (contour_setup.f90:63-73)."""
    return {"fam_mode": "STR", "fam_input_filename": "pnfam_NAMELIST.dat",
            "operator_groups": list(GROUPS), "operator_active": [0, 0, 0, 0, 0],
            "energy_start": 0.0, "energy_step": 0.2, "nr_points": 5, "half_width": 0.5}


def read_contour_namelist(path: str) -> dict:
    try:
        given = parse_namelist_file(path)
    except OSError as e:
        raise NamelistError(f"problem reading contour namelist: {e}")
    c = ctr_defaults()
    for grp in ("ctr_general", "ctr_extfield", "str_parameters"):
        for k, v in given.get(grp, {}).items():
            if k not in c:
                raise NamelistError(f"problem reading contour namelist: unknown entry {grp}%{k}")
            if v is None:
                continue
            if isinstance(c[k], list):
                v = [x for x in (v if isinstance(v, list) else [v])]
                v = [d if x is None else x for x, d in zip(v + [None] * (len(c[k]) - len(v)), c[k])]
            elif isinstance(v, list):
                v = next((x for x in v if x is not None), None)
                if v is None:
                    continue
            c[k] = v
    return c


def _sign(a: int, b: int) -> int:
    """Fortran SIGN(a, b) for integers: |a| with the sign of b (b = 0 counts as +)."""
    return abs(a) if b >= 0 else -abs(a)


def operator_list(ctr: dict, op_name: str, op_k: int):
    """setup_operators (contour_setup.f90:160-216)."""
    active = [i for i, a in enumerate(ctr["operator_active"]) if int(a or 0) != 0]
    if not active:
        return [(op_name, int(op_k))]
    return [(name, _sign(k, int(op_k))) for i in active for name, k in GROUP_OPS[i]]


def energies(ctr: dict):
    """setup_energy_contour (contour_setup.f90:145-158)."""
    n = int(ctr["nr_points"])
    return [complex(float(ctr["energy_start"]) + i * float(ctr["energy_step"]), float(ctr["half_width"]))
            for i in range(n)]


def _summary(path, ctr_path, case, op, beta, k, half_width, rows):
    xl = [g.label for g in case.G]
    with open(path, "w") as fh:
        fh.write(f"# pnFAM code version: {txtoutput.VERSION}\n")
        fh.write("# pnFAM code commit:  \n")
        fh.write(f"# Contour input file name: {ctr_path}\n")
        fh.write(f"# Residual interaction: {case.couplings.name}\n")
        fh.write(f"# Operator: {op} with K = {k}\n")
        fh.write(f"# Gamma (half-width): {half_width:.4f}\n")
        fh.write("#\n")
        head = "#" + f"{'Conv':>5}" + f"{'Re(EQRPA)':>29}" + f"{'Re(Strength)':>34}" + f"{'Im(Strength)':>34}"
        head += "".join(f"{'Re(' + l + ')':>34}{'Im(' + l + ')':>34}" for l in xl)
        fh.write(head + "\n")
        for conv, w, re_S, im_S in rows:
            line = f"{conv:5d}{w.real:30.19f}" + "".join(f"{a:34.19E}{b:34.19E}" for a, b in zip(re_S, im_S))
            fh.write(line + "\n")


def run(ctr_path: str, cwd: str = ".", solver_factory=None) -> int:
    from .pnfam_setup import setup_case
    ctr = read_contour_namelist(os.path.join(cwd, ctr_path))
    base = read_pnfam_namelist(os.path.join(cwd, str(ctr["fam_input_filename"]).strip()))
    hfb = pnfam_main.load_ground_state(os.path.join(cwd, pnfam_main.HEL_NAME))
    ws = energies(ctr)
    e = base["ext_field"]
    beta = e["beta_type"]
    out_base = str(base["general"]["fam_output_filename"]).strip()
    gpu = None
    try:
        for op, k in operator_list(ctr, e["operator_name"], e["operator_k"]):
            nml = copy.deepcopy(base)
            nml["ext_field"]["operator_name"], nml["ext_field"]["operator_k"] = op, k
            case = setup_case(nml, None, hfb=hfb, tbc_dir=cwd)
            if gpu is None:
                gpu = (solver_factory or _gpu_solver)(case)
            gpu.set_operator(case.F, case.G)
            s = nml["solver"]
            t0 = time.perf_counter()
            res = gpu.solve(ws, history=True, max_iter=int(s["max_iter"]), eps=float(s["convergence_epsilon"]),
                            broyden_m=int(s["broyden_history_size"]), quench=case.quench)
            dt = (time.perf_counter() - t0) / max(len(ws), 1)
            rows = []
            for i, w in enumerate(ws):
                pn = copy.deepcopy(nml)
                pn["general"]["real_eqrpa"], pn["general"]["imag_eqrpa"] = w.real, w.imag
                name = f"{op}{beta}K{k}_{i:06d}" if out_base else ""
                pn["general"]["fam_output_filename"] = name
                log = txtoutput.Log(os.path.join(cwd, name + ".dat") if name else "",
                                    bool(pn["general"]["print_stdout"]) or not name)
                pcase = copy.copy(case)
                pcase.nml = pn
                txtoutput.header(log, pn, pcase, int(hfb.n00))
                pnfam_main.finish(pnfam_main.Point(pn, log, pcase), res, i, dt)
                it = int(res.iters[i])
                rows.append((1 if it > 0 else 0, w, res.re_S[i], res.im_S[i]))
            _summary(os.path.join(cwd, f"{op}{beta}K{k}.out"), ctr_path, case, op, beta, k,
                     float(ctr["half_width"]), rows)
    finally:
        if gpu is not None:
            gpu.close()
    return 0


def _gpu_solver(case):
    from .solver import GPUSolver
    return GPUSolver(case.hfb, case.couplings, occupations=case.hfb.occupations)


def main(argv=None) -> int:
    argv = sys.argv[1:] if argv is None else argv
    if len(argv) > 1:
        sys.stderr.write("More than one command-line argument! Aborting.\n")
        return 1
    try:
        return run(argv[0] if argv else "pnfam_CONTOUR.dat")
    except Exception as e:
        sys.stderr.write(f"ERROR: {type(e).__name__}: {e}\n")
        return 1


if __name__ == "__main__":
    sys.exit(main())
