"""Host-side mirror of the reference solver interface, on top of the C ABI.

``GPUSolver`` owns one device context per nucleus (pnfam_gpu_init), one
operator at a time (pnfam_gpu_set_operator) and solves batches of omega points
(pnfam_gpu_solve).  It mirrors the reference's pnfam_solve / init_pnfam_solver
/ ifam split (pnfam_solver.f90:32-221) with the per-process set-up hoisted out
of the per-point loop.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from .blockmatrix import BlockMatrix


@dataclass
class SolveResult:
    re_S: np.ndarray      # [P, 1 + n_xterms]
    im_S: np.ndarray
    iters: np.ndarray     # [P] iteration at convergence, -1 if interrupted
    si: np.ndarray        # [P]
    hist: np.ndarray = None  # [P, max_iter + 1, 3] (si, Re S, Im S), NaN after convergence
    seconds: float = 0.0
    state: np.ndarray = None  # [P, state_size] final Broyden vectors (solve(..., return_state=True))


def _flat_blocks(blocks) -> np.ndarray:
    parts = [np.asarray(b, dtype=np.float64).reshape(-1, order="F") for b in blocks]
    return np.ascontiguousarray(np.concatenate(parts)) if parts else np.zeros(0)


class GPUSolver:
    """One nucleus resident on the current CUDA device."""

    def __init__(self, hfb, couplings, occupations=None):
        """occupations: (f_p, f_n) quasiparticle occupations [dqp] of a finite-temperature
        or EFA-blocked ground state (pynfam_gb300.statistics), for the statistical FAM."""
        self.lib = _lib.load()
        self.hfb = hfb
        self.nb = int(hfb.nb)
        self._keep = []
        db = np.ascontiguousarray(hfb.db, dtype=np.int32)
        nup = np.ascontiguousarray(hfb.num_spin_up, dtype=np.int32)
        ns = np.ascontiguousarray(hfb.ns, dtype=np.int32)
        self._keep += [db, nup, ns]
        basis = _lib.Basis(self.nb, _lib.iptr(db), _lib.iptr(nup), _lib.iptr(ns), int(hfb.nghl))
        phi = np.ascontiguousarray(np.stack([hfb.wf, hfb.wfdr, hfb.wfdp, hfb.wfdz, hfb.wfd2_all]))
        Up, Vp, Un, Vn = (_flat_blocks(x) for x in (hfb.Up, hfb.Vp, hfb.Un, hfb.Vn))
        Ep = np.ascontiguousarray(hfb.Ep, dtype=np.float64)
        En = np.ascontiguousarray(hfb.En, dtype=np.float64)
        wd = np.ascontiguousarray(hfb.wdcori, dtype=np.float64)
        cpl = [np.ascontiguousarray(a, dtype=np.float64) for a in (couplings.crho, couplings.cs, couplings.cpair, couplings.cspair)]
        self._keep += [phi, Up, Vp, Un, Vn, Ep, En, wd] + cpl
        cp = _lib.Coupl(_lib.dptr(cpl[0]), _lib.dptr(cpl[1]), _lib.dptr(cpl[2]), _lib.dptr(cpl[3]),
                        (C.c_double * 12)(*couplings.scalars()))
        ctx = C.c_void_p()
        _lib.check(self.lib.pnfam_gpu_init(C.byref(basis), _lib.dptr(Ep), _lib.dptr(En), _lib.dptr(Up),
                                           _lib.dptr(Vp), _lib.dptr(Un), _lib.dptr(Vn), _lib.dptr(phi),
                                           _lib.dptr(wd), C.byref(cp), C.byref(ctx)))
        self.ctx = ctx
        self.nops = 1
        self.F = None
        if occupations is not None:
            self.set_occupations(*occupations)

    def set_occupations(self, fp=None, fn=None):
        """Statistical FAM with these occupations (None, None: zero temperature); the
        operator must be set afterwards."""
        if (fp is None) != (fn is None):
            raise ValueError("give both occupation arrays or neither")
        if fp is None:
            _lib.check(self.lib.pnfam_gpu_set_occupations(self.ctx, None, None))
            self.occupations = None
            return
        a = np.ascontiguousarray(fp, dtype=np.float64); b = np.ascontiguousarray(fn, dtype=np.float64)
        if a.shape != (int(self.hfb.dqp),) or b.shape != a.shape:
            raise ValueError("occupations must have dqp entries")
        _lib.check(self.lib.pnfam_gpu_set_occupations(self.ctx, _lib.dptr(a), _lib.dptr(b)))
        self.occupations = (a, b)
        self.F = None

    def set_operator(self, F, G=()):
        """F: ExternalField (or BlockMatrix + beta flag via F.beta_minus)."""
        mat = F.mat if hasattr(F, "mat") else F
        fcols = np.ascontiguousarray(mat.cols, dtype=np.int32)
        fsp = np.ascontiguousarray(mat.flatten(), dtype=np.float64)
        gs = [np.ascontiguousarray(g.mat.flatten(), dtype=np.float64) for g in G]
        arr = (C.POINTER(C.c_double) * max(1, len(gs)))(*[_lib.dptr(g) for g in gs]) if gs else None
        _lib.check(self.lib.pnfam_gpu_set_operator(self.ctx, 1 if F.beta_minus else 0, _lib.iptr(fcols),
                                                   _lib.dptr(fsp), len(gs), arr))
        self.nops = 1 + len(gs)
        self.F = F
        self.fcols = fcols

    @property
    def nxy(self) -> int:
        return int(self.lib.pnfam_gpu_nxy(self.ctx))

    @staticmethod
    def options(max_iter=300, eps=1e-7, broyden_m=50, quench=1.0, alpha_mix=None, timed=False, precision=0,
                switch_exp=0, live=False, settle=0, near_exp=0, async_anchors=False):
        if alpha_mix is None:
            from .pnfam_setup import ALPHA_MIX as alpha_mix
        o = _lib.SolverOpts()
        o.max_iter = int(max_iter); o.broyden_history_size = int(broyden_m)
        o.convergence_epsilon = float(eps); o.alpha_mix = float(alpha_mix)
        o.quench_residual_int = float(quench); o.precision = int(precision)
        o.reserved[0] = 1 if timed else 0
        o.reserved[1] = int(switch_exp)
        o.reserved[2] = 1 if live else 0
        o.reserved[3] = int(settle)
        o.reserved[4] = int(near_exp)
        o.reserved[5] = 1 if async_anchors else 0
        return o

    def engine(self, slots, owns_solver=False, **opts) -> "Engine":
        """Continuous-batching engine on this context (see Engine); with
        owns_solver, closing the engine also frees this context."""
        return Engine(self, slots, self.options(**opts), owns_solver)

    def solve(self, omegas, max_iter=300, eps=1e-7, broyden_m=50, quench=1.0, alpha_mix=None,
              history=False, timed=False, precision=0, switch_exp=0, settle=0, near_exp=0,
              x0=None, return_state=False) -> SolveResult:
        """precision 0: FP64 throughout (the reference's arithmetic and iteration
        trajectory).  precision 1: defect correction -- the field is evaluated in
        FP32 on the increment from an FP64 anchor; within 1000*eps of the anchor
        convergence is accepted on an FP32 increment evaluation, farther out an
        FP64 anchor evaluation is taken when si < 10**-switch_exp (default
        100*eps) or si stops falling.  settle = n > 0: convergence also waits until
        every strength value moved by at most 10**-n of itself in the last iteration;
        near_exp = n > 0: a point counts as near its anchor within 10**n * eps (default 1000).
        x0: [P, state_size] start vectors (the reference's restart storage; None: X = 0);
        return_state: also return the final vectors (SolveResult.state)."""
        import time
        w = np.atleast_1d(np.asarray(omegas, dtype=complex))
        P = len(w)
        wre = np.ascontiguousarray(w.real); wim = np.ascontiguousarray(w.imag)
        reS = np.zeros(P * self.nops); imS = np.zeros(P * self.nops)
        iters = np.zeros(P, dtype=np.int32); si = np.zeros(P)
        hist = np.full(P * (max_iter + 1) * 3, np.nan) if history else None
        o = self.options(max_iter, eps, broyden_m, quench, alpha_mix, timed, precision, switch_exp,
                         settle=settle, near_exp=near_exp)
        t0 = time.perf_counter()
        if x0 is None and not return_state:
            _lib.check(self.lib.pnfam_gpu_solve(self.ctx, P, _lib.dptr(wre), _lib.dptr(wim), C.byref(o),
                                                _lib.dptr(reS), _lib.dptr(imS), _lib.iptr(iters), _lib.dptr(si),
                                                _lib.dptr(hist) if hist is not None else None))
            xo = None
        else:
            n = self.state_size
            xs = None
            if x0 is not None:
                xs = np.ascontiguousarray(x0, dtype=np.float64).reshape(P, n)
            xo = np.zeros((P, n)) if return_state else None
            _lib.check(self.lib.pnfam_gpu_solve_state(
                self.ctx, P, _lib.dptr(wre), _lib.dptr(wim), C.byref(o), _lib.dptr(xs) if xs is not None else None,
                _lib.dptr(reS), _lib.dptr(imS), _lib.iptr(iters), _lib.dptr(si),
                _lib.dptr(hist) if hist is not None else None, _lib.dptr(xo) if xo is not None else None))
        dt = time.perf_counter() - t0
        return SolveResult(reS.reshape(P, self.nops), imS.reshape(P, self.nops), iters, si,
                           hist.reshape(P, max_iter + 1, 3) if hist is not None else None, dt, xo)

    @property
    def state_size(self) -> int:
        """Length of one point's state (Broyden) vector: 4 nxy, 8 nxy in the statistical FAM."""
        return int(self.lib.pnfam_gpu_state_size(self.ctx))

    def last_profile(self):
        """Per-stage device ms of the last solve (or of this context's engine so far);
        the *_fp32 entries are the FP32 evaluations of the mixed form."""
        ms = np.zeros(23); n = C.c_longlong()
        _lib.check(self.lib.pnfam_gpu_last_profile(self.ctx, _lib.dptr(ms), 23, C.byref(n)))
        names = ("k1_blockgemm", "density", "meanfield", "field_projection", "k2_blockgemm", "green", "broyden",
                 "strength", "total", "point_iterations_fp64", "point_iterations_fp32", "k1_blockgemm_fp32",
                 "density_fp32", "meanfield_fp32", "field_projection_fp32", "k2_blockgemm_fp32",
                 "live_density_launches", "live_density_ms", "live_projection_launches", "live_projection_ms",
                 "tuned_pair_min_points", "tuned_density_kspan", "autotune_ms")
        return dict(zip(names, ms.tolist())), int(n.value)

    def calc_hamiltonian(self, rho_pn, kp, rho_np, km, mixed=False):
        """Plugin seam: complex flat arrays (nxy) in the structures documented in
        include/pnfam_gpu.h; returns (h_pn, Delta+, h_np, Delta-) complex.
        mixed=True evaluates in FP32 with the tensor-core projection (the
        kernels of the mixed form's increment evaluations)."""
        n = self.nxy
        ins = []
        for a in (rho_pn, kp, rho_np, km):
            a = np.asarray(a, dtype=complex)
            ins += [np.ascontiguousarray(a.real), np.ascontiguousarray(a.imag)]
        outs = [np.zeros(n) for _ in range(8)]
        fn = self.lib.pnfam_gpu_calc_hamiltonian_mixed if mixed else self.lib.pnfam_gpu_calc_hamiltonian
        _lib.check(fn(self.ctx, *[_lib.dptr(x) for x in ins], *[_lib.dptr(x) for x in outs]))
        return tuple(outs[2 * k] + 1j * outs[2 * k + 1] for k in range(4))

    def close(self):
        if getattr(self, "ctx", None) is not None and self.ctx.value:
            self.lib.pnfam_gpu_free(self.ctx)
            self.ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass
class PointResult:
    tag: int
    S: np.ndarray         # [1 + n_xterms] complex strength and cross terms
    iters: int            # iteration at convergence, -1 if max_iter was reached
    si: float


class Engine:
    """Continuous batching on one context (pnfam_gpu_engine_*): ``slots`` omega
    points iterate together, each on its own counter; ``admit`` fills free
    slots, ``launch`` enqueues one iteration of every active slot (asynchronous,
    on the context's own stream, so engines of different contexts overlap on
    the GPU) and ``finish`` waits for it and returns the points that finished."""

    def __init__(self, solver: GPUSolver, slots: int, opts, owns_solver=False):
        self.solver = solver
        self.owns_solver = owns_solver
        self.lib = solver.lib
        self.slots = int(slots)
        self.nops = solver.nops
        eng = C.c_void_p()
        _lib.check(self.lib.pnfam_gpu_engine_create(solver.ctx, self.slots, C.byref(opts), C.byref(eng)))
        self.eng = eng
        n = self.slots
        self._tags = np.zeros(n, dtype=np.int64)
        self._re = np.zeros(n * self.nops); self._im = np.zeros(n * self.nops)
        self._it = np.zeros(n, dtype=np.int32); self._si = np.zeros(n)

    @property
    def active(self) -> int:
        return int(self.lib.pnfam_gpu_engine_active(self.eng))

    def admit(self, omegas, tags) -> int:
        w = np.atleast_1d(np.asarray(omegas, dtype=complex))
        wre = np.ascontiguousarray(w.real); wim = np.ascontiguousarray(w.imag)
        t = np.ascontiguousarray(tags, dtype=np.int64)
        k = int(self.lib.pnfam_gpu_engine_admit(self.eng, len(w), _lib.dptr(wre), _lib.dptr(wim),
                                                t.ctypes.data_as(C.POINTER(C.c_longlong))))
        if k < 0:
            _lib.check(-k)
        return k

    def launch(self):
        _lib.check(self.lib.pnfam_gpu_engine_launch(self.eng))

    def ready(self) -> bool:
        """True when finish() would not wait for the device."""
        r = int(self.lib.pnfam_gpu_engine_ready(self.eng))
        if r < 0:
            _lib.check(-r)
        return r == 1

    def finish(self):
        out = []
        while True:
            n = C.c_int()
            _lib.check(self.lib.pnfam_gpu_engine_finish(
                self.eng, self.slots, self._tags.ctypes.data_as(C.POINTER(C.c_longlong)), _lib.dptr(self._re),
                _lib.dptr(self._im), _lib.iptr(self._it), _lib.dptr(self._si), C.byref(n)))
            for k in range(n.value):
                S = self._re[k * self.nops:(k + 1) * self.nops] + 1j * self._im[k * self.nops:(k + 1) * self.nops]
                out.append(PointResult(int(self._tags[k]), S.copy(), int(self._it[k]), float(self._si[k])))
            if n.value < self.slots:
                return out

    def close(self):
        if getattr(self, "eng", None) is not None and self.eng.value:
            self.lib.pnfam_gpu_engine_free(self.eng)
            self.eng = C.c_void_p()
        if getattr(self, "owns_solver", False):
            self.solver.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
