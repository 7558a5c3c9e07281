"""``pnfam_main`` drop-in: one (operator, K, omega) point per process.

Usage (what pynfam's fortProcess runs, pynfam/fortran/pnfam_run.py:140-167):

    pnfam_main.x [namelist]        # default: pnfam_NAMELIST.dat

Reads the namelist (&general &ext_field &interaction &solver,
pnfam_setup.f90:232-268), ``hfbtho_output.hel`` and, for the finite-range
two-body-current modes, ``<fam_output_filename>.tbc`` from the working
directory, solves the point on the GPU and writes ``<fam_output_filename>.dat``
(pnfam_txtoutput.f90).  On any error it writes the message to the log and to
stderr, writes no result table and exits with status 1; pynfam treats
non-empty stderr or a missing result as a failed point.

The HFB reconstruction is cached per ``.hel`` content (directory from
$PNFAM_GB300_CACHE, default ~/.cache/pynfam_gb300; set it to "off" to
disable), so the points of one contour pay it once.
"""
from __future__ import annotations

import hashlib
import os
import pickle
import sys
import time

HEL_NAME = "hfbtho_output.hel"


def _cache_dir():
    d = os.environ.get("PNFAM_GB300_CACHE", os.path.join(os.path.expanduser("~"), ".cache", "pynfam_gb300"))
    return None if d.lower() == "off" else d


def load_ground_state(hel_path: str):
    from .hfb_solution import load_hfb_solution
    cdir = _cache_dir()
    key = None
    if cdir:
        with open(hel_path, "rb") as fh:
            # the tag changes whenever the cached HFBSolution gains fields
            key = hashlib.sha256(b"hfb-solution-3\0" + fh.read()).hexdigest()
        p = os.path.join(cdir, key + ".pkl")
        if os.path.exists(p):
            try:
                with open(p, "rb") as fh:
                    return pickle.load(fh)
            except Exception:
                pass
    hfb = load_hfb_solution(hel_path)
    if cdir and key:
        try:
            os.makedirs(cdir, exist_ok=True)
            tmp = os.path.join(cdir, f"{key}.{os.getpid()}.tmp")
            with open(tmp, "wb") as fh:
                pickle.dump(hfb, fh, protocol=pickle.HIGHEST_PROTOCOL)
            os.replace(tmp, os.path.join(cdir, key + ".pkl"))
        except OSError:
            pass
    return hfb


def main(argv=None) -> int:
    from . import txtoutput
    from .namelist import read_pnfam_namelist
    argv = sys.argv[1:] if argv is None else argv
    if len(argv) > 1:
        sys.stderr.write("More than one command-line argument! Aborting.\n")
        return 1
    nml_path = argv[0] if argv else "pnfam_NAMELIST.dat"
    log = None
    try:
        nml = read_pnfam_namelist(nml_path)
        g = nml["general"]
        name = str(g["fam_output_filename"]).strip()
        log = txtoutput.Log(name + ".dat" if name else "", bool(g["print_stdout"]) or not name)
        if int(g["use_fam_storage"]) != 0:
            log.write(" Note: use_fam_storage is not supported; running without restart storage")
        from .pnfam_setup import setup_case
        from .solver import GPUSolver
        hfb = load_ground_state(HEL_NAME)
        case = setup_case(nml, None, hfb=hfb)
        txtoutput.header(log, nml, case, int(hfb.n00))
        s = nml["solver"]
        gpu = GPUSolver(case.hfb, case.couplings, occupations=case.hfb.occupations)
        gpu.set_operator(case.F, case.G)
        t0 = time.perf_counter()
        res = gpu.solve([case.omega], max_iter=int(s["max_iter"]), eps=float(s["convergence_epsilon"]),
                        broyden_m=int(s["broyden_history_size"]), quench=case.quench, history=True)
        dt = time.perf_counter() - t0
        gpu.close()
        it_conv = int(res.iters[0])
        last = it_conv if it_conv >= 0 else int(s["max_iter"])
        hist = [tuple(res.hist[0, i]) for i in range(last + 1)]
        txtoutput.iterations(log, hist, it_conv, float(res.si[0]), [x.label for x in case.G])
        txtoutput.result(log, dt, case.omega, res.re_S[0], res.im_S[0], [x.label for x in case.G])
        log.close()
        return 0
    except Exception as e:  # the reference aborts with a message and no result table
        msg = f" ERROR: {type(e).__name__}: {e}"
        if log is not None:
            log.write(msg)
            log.close()
        sys.stderr.write(msg.strip() + "\n")
        return 1


if __name__ == "__main__":
    sys.exit(main())
