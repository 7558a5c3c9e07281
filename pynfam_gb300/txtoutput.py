"""The pnFAM text output (``<fam_output_filename>.dat``).

Layout follows pnfam_txtoutput.f90 and pnfam_logger.f90: every log line is a
comment starting with '#'; the iteration table (pnfam_solver.f90:107-113),
the convergence line (:212-218) and "Total CPU time = ... minutes"; then the
un-commented result table in ES34.19 (pnfam_txtoutput.f90:230-253).  pynfam's
parser (pynfam/outputs/pnfam_parser.py:44-132) reads "Version:", "Total CPU
time", "iteration converged"/"interrupted" and the Real/Imag table.
"""
from __future__ import annotations

import datetime
import sys

VERSION = "2.00-gb300"


class Log:
    """``sink``: a list that takes the printed lines instead of stdout (a run served
    by another process returns them to its caller)."""

    def __init__(self, path: str, to_stdout: bool, sink=None):
        self.fh = open(path, "w") if path else None
        self.to_stdout = to_stdout
        self.sink = sink

    def write(self, s: str = "", comment: bool = True):
        line = ("#" + s) if comment else (" " + s)
        line = line.rstrip()
        if self.fh:
            self.fh.write(line + "\n")
        if self.to_stdout:
            if self.sink is not None:
                self.sink.append(line)
            else:
                sys.stdout.write(line + "\n")

    def close(self):
        if self.fh:
            self.fh.close()
            self.fh = None


def _txtl(s, n):
    return f"{s:<{n}}"


def _txtr(s, n):
    return f"{s:>{n}}"


def header(log: Log, nml: dict, case, nshells: int):
    """The run header (print_main_header) and the solver and interaction details
    (log_header); a run with restart storage reports its read between the two."""
    main_header(log, nml, case)
    solver_header(log, nml, case, nshells)


def main_header(log: Log, nml: dict, case):
    g, e = nml["general"], nml["ext_field"]
    hfb = case.hfb
    Z, N = hfb.Z, hfb.N
    bm = e["beta_type"] == "-"
    zf, nf = (Z + 1, N - 1) if bm else (Z - 1, N + 1)
    now = datetime.datetime.now()
    w = 51
    log.write()
    log.write(" " + "=" * w)
    log.write(" " + _center("pnFAM", w))
    log.write(" " + _center("Charge-changing Finite Amplitude Method", w))
    log.write(" " + _center(f"Version: {VERSION}", w))
    log.write(" " + _center("GB300 (sm_103a) solver", w))
    log.write(" " + _center(f"Run date: {now.month}/{now.day}/{now.year} {now:%H:%M:%S}", w))
    log.write(" " + "=" * w)
    log.write(" " + _center(f"Operator: {e['operator_name']}{e['beta_type']} for K = {e['operator_k']}", w))
    log.write(" " + _center(f"Energy: ({g['real_eqrpa']:8.4f} {'+' if g['imag_eqrpa'] >= 0 else '-'} "
                            f"{abs(g['imag_eqrpa']):8.4f}i)", w))
    log.write(" " + _center(f"Parent nucleus: (N={N}, Z={Z})", w))
    log.write(" " + _center(f"Daughter nucleus: (N={nf}, Z={zf})", w))
    log.write(" " + "=" * w)
    log.write()


def solver_header(log: Log, nml: dict, case, nshells: int):
    g, e, s = nml["general"], nml["ext_field"], nml["solver"]
    hfb = case.hfb
    w = 51
    log.write(" " + "-" * w)
    log.write(" " + _center("pnFAM solver details", w))
    log.write(" " + "-" * w)
    log.write(f" Operator:                        {e['operator_name']}{e['beta_type']}  K={e['operator_k']:2d}")
    mode = int(e.get("two_body_current_mode", 0) or 0)
    log.write(f" Two-body current mode (use_p):   {mode} ({1 if e.get('two_body_current_usep') else 0})")
    if mode != 0:
        lecs = " ".join(f"{float(x):+8.4f}" for x in e["two_body_current_lecs"])
        log.write(f"   LECs (c3, c4, cd):             {lecs}")
    xt = ", ".join(x.label for x in case.G) if case.G else "None"
    log.write(f" Compute cross-terms:             {'Yes' if e['compute_crossterms'] else 'No'}")
    log.write(f"   Cross-terms computed:          {xt}")
    log.write(f" Re(EQRPA):                       {g['real_eqrpa']:10.4f} MeV")
    log.write(f" Im(EQRPA):                       {g['imag_eqrpa']:10.4f} MeV")
    log.write()
    log.write(f" Number shells:                   {nshells}")
    log.write(f" Basis size:                      {hfb.dqp}")
    log.write(f" Number matrix blocks:            {hfb.nb}")
    log.write(f" Non-trivial FAM matrix elements: {case.F.mat.nelem}")
    log.write()
    log.write(f" Maximum iterations:              {s['max_iter']}")
    log.write(f" Broyden history size:            {s['broyden_history_size']}")
    log.write(f" Broyden mixing factor:           0.70")
    log.write(f" Convergence limit:               {s['convergence_epsilon']:9.1E}")
    log.write()
    cp = case.couplings
    log.write(" " + "-" * w)
    log.write(" " + _center("pnFAM Interaction", w))
    log.write(" " + "-" * w)
    if cp.skip_residual_interaction:
        log.write(" Residual interaction:            None")
    else:
        log.write(f" Residual interaction:            {cp.name}")
        log.write(f" Crho[0] = {cp.cr0:15.9f};   Cs[0]   = {cp.cs0:15.9f}")
        log.write(f" Crho[r] = {cp.crr:15.9f};   Cs[r]   = {cp.csr:15.9f}")
        log.write(f" Cdr     = {cp.cdrho:15.9f};   Cds     = {cp.cds:15.9f}")
        log.write(f" Ctau    = {cp.ctau:15.9f};   Cj      = {cp.cj:15.9f}")
        log.write(f" CrdJ    = {cp.crdj:15.9f};   Csdj    = {cp.csdj:15.9f}")
        log.write(f" CtJ0    = {cp.ctj0:15.9f};   Cgs     = {cp.cgs:15.9f}")
        log.write(f" CtJ1    = {cp.ctj1:15.9f};   CT      = {cp.ct:15.9f}")
        log.write(f" CtJ2    = {cp.ctj2:15.9f};   CF      = {cp.cf:15.9f}")
        log.write(f" Cpr[0]  = {cp.cpair0:15.9f};   Cps[0]  = {cp.cspair0:15.9f}")
        log.write(f" Cpr[r]  = {cp.cpairr:15.9f};   Cps[r]  = {cp.cspairr:15.9f}")
    log.write()


def _center(s, w):
    return s.center(w).rstrip()


def iterations(log: Log, hist, iter_conv: int, si: float, xlabels, xhist=None):
    """hist: [(si, re, im)] for iterations 0..last; flags N, L, B as in the reference."""
    log.write(" " + "-" * 72)
    log.write(" " + "    i" + "               si" + "               Re(S)" + "               Im(S)" + "      Time")
    log.write(" " + "-" * 72)
    for it, (s_, re, im) in enumerate(hist):
        flag = "N" if it == 0 else ("L" if it == 1 else "B")
        log.write(f" {it:4d}{flag}  {s_:15.10f}  {re:18.10f}  {im:18.10f}  {0.0:8.3f}")
    log.write(" " + "-" * 72)
    n = len(hist) - 1
    if iter_conv >= 0:
        log.write(f"  *  FAM iteration converged after   {n:4d} steps.  si = {si:12.5E}")
    else:
        log.write(f"  *  FAM iteration interrupted after {n:4d} steps.  si = {si:12.5E}")
    log.write(" " + "-" * 72)


def result(log: Log, seconds: float, omega: complex, re_S, im_S, xlabels):
    log.write(f" Total CPU time = {seconds / 60.0:12.3E} minutes")
    log.write()
    log.write()
    log.write(" Result (Energy [MeV], strength and cross-terms [MeV^-1]):")
    log.write(" " + "-" * 78)
    log.write(" " + " " * 10 + _txtr("Real", 34) + _txtr("Imag", 34), comment=False)
    log.write(_txtl("Energy", 10) + f"{omega.real:34.19E}{omega.imag:34.19E}", comment=False)
    log.write(_txtl("Strength", 10) + f"{re_S[0]:34.19E}{im_S[0]:34.19E}", comment=False)
    for k, lab in enumerate(xlabels):
        log.write(_txtl(lab, 10) + f"{re_S[k + 1]:34.19E}{im_S[k + 1]:34.19E}", comment=False)
    log.write("", comment=False)
