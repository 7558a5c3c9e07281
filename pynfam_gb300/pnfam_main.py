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
disable), so the points of one contour pay it once.  With
$PNFAM_GB300_SERVER naming the socket of a running point server
(``python -m pynfam_gb300.pointserver <socket>``), the point is handed to that
resident process, which batches the points of concurrent runs on the GPU; if
no server answers there, the point runs here.
"""
from __future__ import annotations

import hashlib
import os
import pickle
import sys
import threading
import time

from . import storage

HEL_NAME = "hfbtho_output.hel"


def _cache_dir():
    d = os.environ.get("PNFAM_GB300_CACHE", os.path.join(os.path.expanduser("~"), ".cache", "pynfam_gb300"))
    return None if d.lower() == "off" else d


_MEMO = {}                  # ground states rebuilt in this process, by .hel content
_MEMO_LOCK = threading.Lock()


# the modules whose code decides what a reconstruction produces: a change to any of
# them gives new cache keys, so a stale reconstruction is never loaded
_RECONSTRUCTION_SOURCES = ("hfb_solution.py", "hel.py", "interaction.py", "synthetic.py")


def _code_digest() -> bytes:
    h = hashlib.sha256(b"hfb-solution\0")
    here = os.path.dirname(os.path.abspath(__file__))
    for name in _RECONSTRUCTION_SOURCES:
        with open(os.path.join(here, name), "rb") as fh:
            h.update(name.encode() + b"\0" + fh.read())
    return h.digest()


def load_ground_state(hel_path: str):
    """The rebuilt ground state of a ``.hel`` file: from this process's memo, the
    on-disk cache or a fresh reconstruction (each by the file's content and the
    reconstruction code's own digest)."""
    with open(hel_path, "rb") as fh:
        key = hashlib.sha256(_code_digest() + fh.read()).hexdigest()
    with _MEMO_LOCK:   # one reconstruction per .hel content, even for concurrent callers
        if key not in _MEMO:
            _MEMO[key] = _load_uncached(hel_path, key)
        return _MEMO[key]


def _load_uncached(hel_path: str, key: str):
    from .hfb_solution import load_hfb_solution
    cdir = _cache_dir()
    hfb = None
    if cdir:
        p = os.path.join(cdir, key + ".pkl")
        if os.path.exists(p) and _private(cdir) and _private(p):
            try:
                with open(p, "rb") as fh:
                    hfb = pickle.load(fh)
            except Exception:
                hfb = None
    if hfb is None:
        hfb = load_hfb_solution(hel_path)
        if cdir:
            try:
                os.makedirs(cdir, mode=0o700, exist_ok=True)
                tmp = os.path.join(cdir, f"{key}.{os.getpid()}.{threading.get_ident()}.tmp")
                with open(tmp, "wb") as fh:
                    pickle.dump(hfb, fh, protocol=pickle.HIGHEST_PROTOCOL)
                os.replace(tmp, os.path.join(cdir, key + ".pkl"))
            except OSError:
                pass
    return hfb


def _private(path: str) -> bool:
    """True if ``path`` belongs to this user and nobody else can write to it: a cached
    reconstruction is unpickled only from such a file in such a directory."""
    try:
        st = os.stat(path)
    except OSError:
        return False
    return st.st_uid == os.getuid() and not (st.st_mode & 0o022)


class Point:
    """One pnfam_main run: its namelist, output log and solver inputs; with restart
    storage (``use_fam_storage`` != 0) the start vector read from
    ``<fam_output_filename>.bin`` (``restart``) and whether the final vector is
    stored there (``store``)."""

    def __init__(self, nml, log, case, restart=None, store="", nxy=0):
        self.nml, self.log, self.case = nml, log, case
        self.restart, self.store, self.nxy = restart, store, nxy

    @property
    def x0(self):
        return None if self.restart is None else self.restart.vector

    @property
    def done_at_start(self) -> bool:
        """The stored state already meets the stopping test: the reference stops at
        iteration 0 (pnfam_solver.f90:126-129) with the stored strengths."""
        return self.x0 is not None and self.restart.si < float(self.nml["solver"]["convergence_epsilon"])

    @property
    def solve_kwargs(self) -> dict:
        s = self.nml["solver"]
        return dict(max_iter=int(s["max_iter"]), eps=float(s["convergence_epsilon"]),
                    broyden_m=int(s["broyden_history_size"]), quench=self.case.quench)


def prepare(nml_path: str, cwd: str = ".", sink=None) -> Point:
    """Read the namelist and the ground state of the run directory ``cwd``, set up
    the operator and write the header of ``<fam_output_filename>.dat``.  ``sink``
    (a list) collects the lines the run would print instead of printing them."""
    from . import txtoutput
    from .namelist import read_pnfam_namelist
    from .pnfam_setup import setup_case
    log = None
    try:
        nml = read_pnfam_namelist(os.path.join(cwd, nml_path))
        g = nml["general"]
        name = str(g["fam_output_filename"]).strip()
        log = txtoutput.Log(os.path.join(cwd, name + ".dat") if name else "", bool(g["print_stdout"]) or not name,
                            sink=sink)
        hfb = load_ground_state(os.path.join(cwd, HEL_NAME))
        case = setup_case(nml, None, hfb=hfb, tbc_dir=cwd)
        txtoutput.main_header(log, nml, case)
        use = int(g["use_fam_storage"]) if name else 0
        path = storage.storage_path(nml, cwd)
        restart = None
        nxy = case.F.mat.nelem
        if use != 0:
            nq = 4 if hfb.occupations is not None else 2
            restart = storage.read_storage(path, case, nxy, 2 * nq * nxy, log)
        txtoutput.solver_header(log, nml, case, int(hfb.n00))
        return Point(nml, log, case, restart, path if use == -1 else "", nxy)
    except Exception as e:
        if log is not None:
            e.pnfam_log = log
        raise


def finish(pt: Point, res, index: int, seconds: float) -> None:
    """The iteration table and the result table of point ``index`` of ``res``."""
    from . import txtoutput
    s = pt.nml["solver"]
    it_conv = int(res.iters[index])
    last = it_conv if it_conv >= 0 else int(s["max_iter"])
    hist = [tuple(res.hist[index, i]) for i in range(last + 1)]
    if pt.restart is not None:
        # iteration 0 shows the stored si (1 when the file was not taken) and strength
        s0 = pt.restart.s0
        hist[0] = (pt.restart.si, s0[0].real if s0 is not None else 0.0, s0[0].imag if s0 is not None else 0.0)
    labels = [x.label for x in pt.case.G]
    txtoutput.iterations(pt.log, hist, it_conv, float(res.si[index]), labels)
    txtoutput.result(pt.log, seconds, pt.case.omega, res.re_S[index], res.im_S[index], labels)
    pt.log.close()
    if pt.store:
        storage.write_storage(pt.store, pt.case, pt.nxy, float(res.si[index]), res.re_S[index], res.im_S[index],
                              res.state[index])


def stored_result(pt: Point):
    """The result of a run whose stored state already meets the stopping test:
    converged at iteration 0 with the stored si, strengths and vector."""
    from .solver import SolveResult
    import numpy as np
    s0 = pt.restart.s0
    hist = np.full((1, 1, 3), np.nan)
    hist[0, 0] = (pt.restart.si, s0[0].real, s0[0].imag)
    return SolveResult(s0.real[None, :].copy(), s0.imag[None, :].copy(), np.zeros(1, dtype=np.int32),
                       np.array([pt.restart.si]), hist, 0.0, pt.x0[None, :].copy())


def fail(err: Exception, log=None) -> str:
    """The reference aborts with a message and no result table."""
    msg = f" ERROR: {type(err).__name__}: {err}"
    log = log or getattr(err, "pnfam_log", None)
    if log is not None:
        log.write(msg)
        log.close()
    return msg.strip() + "\n"


def main(argv=None) -> int:
    argv = sys.argv[1:] if argv is None else argv
    if len(argv) > 1:
        sys.stderr.write("More than one command-line argument! Aborting.\n")
        return 1
    nml_path = argv[0] if argv else "pnfam_NAMELIST.dat"
    server = os.environ.get("PNFAM_GB300_SERVER", "")
    if server:
        from .pointserver import submit
        rc = submit(server, os.getcwd(), nml_path)
        if rc is not None:
            return rc
    pt = None
    try:
        pt = prepare(nml_path)
        if pt.done_at_start:
            finish(pt, stored_result(pt), 0, 0.0)
            return 0
        from .solver import GPUSolver
        gpu = GPUSolver(pt.case.hfb, pt.case.couplings, occupations=pt.case.hfb.occupations)
        gpu.set_operator(pt.case.F, pt.case.G)
        t0 = time.perf_counter()
        x0 = None if pt.x0 is None else pt.x0[None, :]
        res = gpu.solve([pt.case.omega], history=True, x0=x0, return_state=bool(pt.store), **pt.solve_kwargs)
        dt = time.perf_counter() - t0
        gpu.close()
        finish(pt, res, 0, dt)
        return 0
    except Exception as e:
        sys.stderr.write(fail(e, pt.log if pt else None))
        return 1


if __name__ == "__main__":
    sys.exit(main())
