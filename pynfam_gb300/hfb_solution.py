"""HFB ground state for pnFAM, rebuilt from an HFBTHO ``.hel`` file.

This is the input side of the solver (it runs once per nucleus, on the host, or
with the arithmetic of steps 1-4 on the GPU: ``hfb_device``).
It reproduces what the reference obtains by re-running HFBTHO for zero
iterations (pnfam: hfbtho_interface.f90:20-226 -> HFBTHO_DFT_SOLVER) and then
reshaping the result for the FAM (pnfam: hfbtho_solution.f90:137-459):

1. harmonic-oscillator basis functions on the Gauss-Hermite x Gauss-Laguerre
   mesh, with the square roots of the quadrature weights mixed in
   (hfbtho_solver.f90:3463-3671 ``gaupol``, :4237-4314 ``optHFBTHO``,
   :1215-1240 ``coordinateLST``);
2. the HFB matrix (h, Delta) of each Omega block from the mean and pairing
   fields stored in the file (hfbtho_solver.f90:5145-5366 ``gamdel``);
3. block diagonalisation of [[h-lambda, Delta], [Delta, -h+lambda]] inside the
   particle-number loop that re-adjusts the Fermi energy (hfbtho_solver.f90:
   1441-1972 ``hfbdiag``, :1977-2075 ``ALambda``), including the quasiparticle
   pairing window;
4. the local density rho(r) of the final solution (hfbtho_solver.f90:4318-4734
   ``DENSIT``), used for the density-dependent couplings;
5. explicit time-reversed partners (doubling of blocks, states, U, V, E), the
   spin-up-first ordering inside each block and the zeroing of quasiparticles
   above the pairing window (hfbtho_solution.f90:137-459).

All arrays are float64.  Mesh index ``ihil = ih + il*ngh`` (Hermite/z fastest),
as in HFBTHO.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from .hel import HelData, read_hel

CUTOFF_TOL = 1.0e-6  # hfbtho_variables.f90:253


class HFBReconstructionError(RuntimeError):
    pass


# ----------------------------------------------------------------------------
# 1. Basis functions on the mesh
# ----------------------------------------------------------------------------
def _hermite_functions(xh, wh, nzm):
    """qh[n, ih], qh1[n, ih] (gaupol, hfbtho_solver.f90:3489-3503)."""
    ngh = len(xh)
    qh = np.zeros((max(nzm, 1) + 1, ngh))
    qh1 = np.zeros_like(qh)
    w0 = np.pi ** (-0.25) * np.exp(-0.5 * xh * xh) * np.sqrt(wh)
    s2 = math.sqrt(2.0)
    qh[0] = w0
    qh[1] = s2 * w0 * xh
    qh1[0] = -w0 * xh
    qh1[1] = s2 * w0 * (1.0 - xh * xh)
    for n in range(2, nzm + 1):
        qh[n] = (s2 * xh * qh[n - 1] - math.sqrt(n - 1) * qh[n - 2]) / math.sqrt(n)
        qh1[n] = math.sqrt(2 * n) * qh[n - 1] - xh * qh[n]
    return qh, qh1


def _laguerre_functions(xl, wl, nrm, nlm):
    """ql[n, l, il], ql1[n, l, il] (gaupol, hfbtho_solver.f90:3510-3546)."""
    ngl = len(xl)
    nn = max(nrm, 1) + 1
    ql = np.zeros((nn, nlm + 1, ngl))
    ql1 = np.zeros_like(ql)
    wfi = [1.0 / math.sqrt(math.factorial(k)) for k in range(nlm + 3)]
    w00 = math.sqrt(2.0) * np.exp(-0.5 * xl)
    for l in range(nlm + 1):
        w0 = w00 * np.sqrt(0.5 * wl * xl ** l)
        ql[0, l] = wfi[l] * w0
        ql[1, l] = (l + 1 - xl) * wfi[l + 1] * w0
        ql1[0, l] = (l - xl) * wfi[l] * w0
        ql1[1, l] = (float(l * l + l) - xl * float(l + l + 3) + xl * xl) * wfi[l + 1] * w0
        for n in range(2, nrm + 1):
            dsq = math.sqrt(n) * math.sqrt(n + l)
            d1 = float(n + n + l - 1) - xl
            d2 = math.sqrt(n - 1) * math.sqrt(n - 1 + l)
            d3 = float(n + n + l) - xl
            d4 = 2.0 * dsq
            ql[n, l] = (d1 * ql[n - 1, l] - d2 * ql[n - 2, l]) / dsq
            ql1[n, l] = d3 * ql[n, l] - d4 * ql[n - 1, l]
    return ql, ql1


@dataclass
class MeshBasis:
    """HO basis (HFBTHO order, Omega>0 half) evaluated on the mesh."""
    qhla: np.ndarray   # [nt, nghl] wave function * sqrt(weight)
    fi1r: np.ndarray   # d/dr
    fi1z: np.ndarray   # d/dz
    fi2d: np.ndarray   # Laplacian (r,z part)
    y: np.ndarray      # 1/r on the mesh [nghl]
    z: np.ndarray      # z on the mesh [nghl]
    wdcori: np.ndarray # inverse of (quadrature weight x Jacobian)
    xlam: np.ndarray   # per block: Lambda of spin-up states (Omega-1/2)
    xlap: np.ndarray   # per block: Lambda of spin-down states (Omega+1/2)


def build_mesh_basis(h: HelData, device: bool = False) -> MeshBasis:
    """The basis on the mesh; ``device``: the functions by the GPU kernel."""
    if device:
        from . import hfb_device
        qhla, fi1r, fi1z, fi2d = hfb_device.basis_functions(h)
        return _mesh_basis_from(h, qhla, fi1r, fi1z, fi2d)
    ngh, ngl = h.ngh, h.ngl
    nzm, nrm, nlm = int(h.nz.max()), int(h.nr.max()), int(h.nl.max())
    qh, qh1 = _hermite_functions(h.xh, h.wh, nzm)
    ql, ql1 = _laguerre_functions(h.xl, h.wl, nrm, nlm)
    bz, bp = h.bz, h.bp
    xh = np.tile(h.xh, ngl)          # ihil = ih + il*ngh
    xl = np.repeat(h.xl, ngh)
    wh = np.tile(h.wh, ngl)
    wl = np.repeat(h.wl, ngh)
    ih = np.tile(np.arange(ngh), ngl)
    il = np.repeat(np.arange(ngl), ngh)
    v2 = 0.5 / xl
    v4 = v2 * v2
    y = 1.0 / (np.sqrt(xl) * bp)
    nt = len(h.nr)
    qhla = np.empty((nt, ngh * ngl)); fi1r = np.empty_like(qhla)
    fi1z = np.empty_like(qhla); fi2d = np.empty_like(qhla)
    for ja in range(nt):
        nza, nra, nla = int(h.nz[ja]), int(h.nr[ja]), int(h.nl[ja])
        qha = qh[nza, ih]; qla = ql[nra, nla, il]
        q = qha * qla
        qhl1a = qha * ql1[nra, nla, il] * v2
        qh1la = qh1[nza, ih] * qla
        qhla[ja] = q
        fi1r[ja] = (2.0 * np.sqrt(xl) / bp) * qhl1a
        fi1z[ja] = qh1la / bz
        cnzaa = nza + nza + 1
        cnraa = nra + nra + nla + 1
        fi2d[ja] = ((xh * xh - cnzaa) / (bz * bz)
                    + 4.0 * (0.25 - cnraa * v2 + nla * nla * v4) * xl / (bp * bp)) * q
    return _mesh_basis_from(h, qhla, fi1r, fi1z, fi2d)


def _mesh_basis_from(h: HelData, qhla, fi1r, fi1z, fi2d) -> MeshBasis:
    """MeshBasis of the basis functions with 1/r, z, the inverse weights and the
    blocks' Lambda values."""
    ngh, ngl = h.ngh, h.ngl
    bz, bp = h.bz, h.bp
    xh = np.tile(h.xh, ngl)
    xl = np.repeat(h.xl, ngh)
    wh = np.tile(h.wh, ngl)
    wl = np.repeat(h.wl, ngh)
    y = 1.0 / (np.sqrt(xl) * bp)
    wdcor = np.pi * wh * wl * bz * bp * bp
    # Lambda of the spin-up / spin-down members of each block, from Omega
    nb = len(h.ID)
    xlam = np.zeros(nb); xlap = np.zeros(nb)
    start = 0
    for ib in range(nb):
        two_omega = int(2 * h.nl[start] + h.ns[start])
        xlap[ib] = (two_omega + 1) // 2
        xlam[ib] = xlap[ib] - 1
        start += int(h.ID[ib])
    return MeshBasis(qhla, fi1r, fi1z, fi2d, y, bz * xh, 1.0 / wdcor, xlam, xlap)


# ----------------------------------------------------------------------------
# 2. HFB matrix from the fields (gamdel)
# ----------------------------------------------------------------------------
def hfb_matrices(h: HelData, mb: MeshBasis):
    """Per block: dict it -> (h_block, delta_block), full symmetric matrices.

    Restates gamdel (hfbtho_solver.f90:5190-5302) for one block at a time.  Every
    matrix element there is a mesh sum of products of two basis functions (or their
    derivatives) weighted by a field, so each group of terms is one GEMM
    (A w) B^T over the mesh: same-spin terms with the weights
    w1 = v + 2 Lyam vSFIZ + L^2y^2 (2 vd + vhb), w2 = 2 vd + vhb, w3 = vr +/- Ly vs
    (L = Lambda of the spin, +/- for up/down), and the spin-flip terms of
    J_{r phi}, J_{phi r}, J_{z phi} and nabla.J.  The reference fills n2 <= n1 and
    mirrors; the lower triangle is taken the same way here.
    """
    out = {"n": [], "p": []}
    start = 0
    y = mb.y
    for ib, nd in enumerate(h.ID):
        nd = int(nd)
        sl = slice(start, start + nd)
        ns = h.ns[sl]
        up = (ns > 0).astype(float)[:, None]
        dn = (ns < 0).astype(float)[:, None]
        q = mb.qhla[sl]; r1 = mb.fi1r[sl]; z1 = mb.fi1z[sl]; d2 = mb.fi2d[sl]
        xlam, xlap = mb.xlam[ib], mb.xlap[ib]
        xlamy = xlam * y; xlapy = xlap * y; xlampy = xlamy + xlapy
        xlamy2 = xlam * xlam * y * y; xlapy2 = xlap * xlap * y * y
        FU, FUR, FUZ, FUD2 = q * up, r1 * up, z1 * up, (d2 - xlamy2 * q) * up
        FD, FDR, FDZ, FDD2 = q * dn, r1 * dn, z1 * dn, (d2 - xlapy2 * q) * dn
        flip_du = (ns[:, None] < 0) & (ns[None, :] > 0)   # a down, b up
        flip_ud = (ns[:, None] > 0) & (ns[None, :] < 0)   # a up, b down

        def G(A, w, B):
            return (A * w) @ B.T

        def sym2(A, w, B):
            m = G(A, w, B)
            return m + m.T
        for t in ("n", "p"):
            f = h.fields[t]
            v, vd, vhb, vs, vr, vz = f["v"], f["vd"], f["vhb"], f["vs"], f["vr"], f["vz"]
            vsfiz, vsrfi, vsfir, vszfi = f["vSFIZ"], f["vSRFI"], f["vSFIR"], f["vSZFI"]
            w2 = 2.0 * vd + vhb
            hm = (G(FU, v + 2.0 * xlamy * vsfiz + xlamy2 * w2, FU) + G(FUR, w2, FUR) + G(FUZ, w2, FUZ)
                  + sym2(FU, vd, FUD2) + sym2(FUR, vr + xlamy * vs, FU) + sym2(FUZ, vz, FU))
            hm += (G(FD, v - 2.0 * xlapy * vsfiz + xlapy2 * w2, FD) + G(FDR, w2, FDR) + G(FDZ, w2, FDZ)
                   + sym2(FD, vd, FDD2) + sym2(FDR, vr - xlapy * vs, FD) + sym2(FDZ, vz, FD))
            dm = G(FU, f["dv"], FU) + G(FD, f["dv"], FD)
            # spin flip, a down / b up, and a up / b down
            du = (G(FDR, -vs, FUZ) + G(FDZ, vs, FUR) + G(FDZ, -xlamy * vs - vszfi, FU)
                  + G(FD, -xlapy * vs + vszfi, FUZ) + G(FDR, -vsrfi, FU) + G(FD, vsrfi, FUR)
                  + G(FD, xlampy * vsfir, FU))
            ud = (G(FUR, vs, FDZ) + G(FUZ, -vs, FDR) + G(FUZ, -xlapy * vs + vszfi, FD)
                  + G(FU, -xlamy * vs - vszfi, FDZ) + G(FUR, vsrfi, FD) + G(FU, -vsrfi, FDR)
                  + G(FU, xlampy * vsfir, FD))
            hm = np.where(flip_du, du, hm)
            hm = np.where(flip_ud, ud, hm)
            # the reference computes element (n1, n2<=n1) and uses it for both
            hm = np.tril(hm) + np.tril(hm, -1).T
            dm = np.tril(dm) + np.tril(dm, -1).T
            out[t].append((hm, dm))
        start += nd
    return out


# ----------------------------------------------------------------------------
# 3. Diagonalisation with the particle-number loop (hfbdiag + ALambda)
# ----------------------------------------------------------------------------
def _alambda(al, erhfb, drhfb, tz, cpv0_zero, temper=0.0):
    """Fermi energy from the BCS-like particle number (hfbtho_solver.f90:1977-2075);
    at temperature T each pairing-window state adds 2 (1 - 2 v^2) f with
    f = (1 - tanh(b / 2T)) / 2, b = sqrt((e - lambda)^2 + Delta^2).  Returns
    (lambda, f of the last particle-number evaluation, in pairing-window order)."""
    if cpv0_zero:
        if temper > 0.0:
            raise HFBReconstructionError("finite-temperature solutions without pairing are not supported")
        ntz = int(tz + 0.1) // 2
        d = np.sort(erhfb)
        if ntz < len(d):
            return 0.5 * (d[ntz - 1] + d[ntz]), None
        return d[ntz - 1] + 0.001, None
    thermal = temper > 1e-12
    fT = None
    xinf, xsup = -1000.0, 1000.0
    for lit in range(1, 501):
        y = erhfb - al
        a = y * y + drhfb ** 2
        b = np.sqrt(a)
        with np.errstate(divide="ignore", invalid="ignore"):
            vh = np.where(b > 0, 0.5 * (1.0 - y / b), 0.0)
            dvh = np.where(b > 0, 0.5 * drhfb ** 2 / (a * b), 0.0)
        vh = np.where(vh < 1e-12, 0.0, vh)
        vh = np.where((vh - 1.0) > 1e-12, 1.0, vh)
        if thermal:
            fT = 0.5 * (1.0 - np.tanh(0.5 * b / temper))
            with np.errstate(divide="ignore", invalid="ignore"):
                dfT = y / b / temper * fT * (1.0 - fT)
            sn = float(np.sum(2.0 * vh + 2.0 * (1.0 - 2.0 * vh) * fT))
            dez = float(np.sum(2.0 * (1.0 - 2.0 * fT) * dvh)) + float(np.sum(2.0 * (1.0 - 2.0 * vh) * dfT))
        else:
            sn = float(np.sum(2.0 * vh))
            dez = float(np.sum(2.0 * dvh))
        ez = sn - tz
        absez = abs(ez) / tz
        if ez < 0:
            xinf = max(xinf, al)
        else:
            xsup = min(xsup, al)
        if lit == 1:
            al = al - ez if absez <= 0.10 else al - 0.10 * math.copysign(1.0, ez)
        else:
            al = al - ez / (dez + 1e-20)
        if al < xinf or al > xsup:
            al = 0.5 * (xinf + xsup)
        if absez <= 1e-10:
            return al, fT
    return al, fT


@dataclass
class QPSolution:
    """Quasiparticles of one isospin, Omega>0 half, HFBTHO block order."""
    E: list        # per block: [nd] quasiparticle energies
    U: list        # per block: [nd, nd] (row = basis state, col = qp)
    V: list
    active: list   # per block: [nd] bool, below the pairing window
    ala: float
    fwin: list = None   # finite temperature: per block, f of the active quasiparticles (DENSIT)


def _eigh_host(mats):
    return [np.linalg.eigh(m) for m in mats]


def diagonalise(h: HelData, hd, it: str, tz: float, temper: float = 0.0, eigh=None) -> QPSolution:
    """hfbdiag(it, icanon) restricted to what pnFAM reads (no blocking); at
    temperature T the particle number of each pairing-window state is
    2 v^2 + 2 (1 - 2 v^2) f(E) (hfbtho_solver.f90:1750-1774)."""
    k = 0 if it == "n" else 1
    ala = float(h.ala[k])
    pwi = h.pwi
    cpv0_zero = (h.CpV0[k] == 0.0)
    sitest = min(0.10, h.si * 0.010)
    blocks = hd[it]
    eig = None
    norm_to_improve = True
    inner = -1
    sumnz = 1.0
    while norm_to_improve:
        inner += 1
        if abs(sumnz) < sitest or inner == 20:
            norm_to_improve = False
        al = ala
        erhfb, drhfb = [], []
        eig = []
        nsum = 0.0
        mats = []
        for (hm, dm) in blocks:
            nd = hm.shape[0]
            M = np.empty((2 * nd, 2 * nd))
            M[:nd, :nd] = hm - al * np.eye(nd)
            M[nd:, nd:] = -hm + al * np.eye(nd)
            M[nd:, :nd] = dm
            M[:nd, nd:] = dm
            mats.append(M)
        for (hm, dm), (w, vec) in zip(blocks, (eigh or _eigh_host)(mats)):
            nd = hm.shape[0]
            Eq = w[nd:]
            Ub = vec[:nd, nd:]
            Vb = vec[nd:, nd:]
            pn = np.sum(Vb * Vb, axis=0)
            ela = Eq * (1.0 - 2.0 * pn)
            enb = ela + al
            ekb = np.sqrt(np.abs(Eq * Eq - ela * ela))
            arg = 100.0 * (enb - pwi)
            with np.errstate(over="ignore"):
                expo = np.where(np.abs(arg) < math.log(np.finfo(float).max), np.exp(np.minimum(arg, 700.0)), np.inf)
            act = (enb <= pwi) | (np.abs(1.0 / (1.0 + expo)) > CUTOFF_TOL)
            erhfb.append(enb[act]); drhfb.append(ekb[act])
            if temper > 1e-12:
                fe = 0.5 * (1.0 - np.tanh(0.5 * Eq[act] / temper))
                nsum += float(np.sum(2.0 * pn[act] + 2.0 * (1.0 - 2.0 * pn[act]) * fe))
            else:
                nsum += float(np.sum(2.0 * pn[act]))
            eig.append((Eq, Ub, Vb, act))
        erhfb = np.concatenate(erhfb); drhfb = np.concatenate(drhfb)
        if len(erhfb) == 0:
            raise HFBReconstructionError("no states below the pairing window")
        sumnz = nsum - tz
        al, fwin = _alambda(al, erhfb, drhfb, tz, cpv0_zero, temper)
        final_ala = ala
        ala = al
    per_block = None
    if fwin is not None:
        # ALambda's occupations, in the pairing-window numbering, are what DENSIT reads
        counts = [int(np.sum(e[3])) for e in eig]
        per_block = np.split(fwin, np.cumsum(counts)[:-1])
    return QPSolution([e[0] for e in eig], [e[1] for e in eig], [e[2] for e in eig],
                      [e[3] for e in eig], final_ala, per_block)


def local_densities(h: HelData, mb: MeshBasis, qp: QPSolution, tz: float):
    """rho(r), tau(r) and the Laplacian of rho(r) of one isospin from the final
    quasiparticles: DENSIT without blocking (hfbtho_solver.f90:4318-4734).
    Per block and pairing-window quasiparticle k, with f_up/down = sum_i V_ik phi_i
    over the spin-up/down basis states and Lambda_up/down = Omega -/+ 1/2:
    rho ~ f_u^2 + f_d^2; tau ~ (Lambda_u y f_u)^2 + (Lambda_d y f_d)^2 + |grad f|^2;
    Laplacian ~ 2 (f_u Lap f_u + f_d Lap f_d + |grad f|^2).  At finite temperature
    every term is (1 - f_k) (its V form) + f_k (the same with U), f_k the thermal
    occupation of ALambda.  The sums are normalised to the particle number and
    freed of the quadrature weights."""
    nghl = h.ngh * h.ngl
    tro = np.zeros(nghl); ttau = np.zeros(nghl); tdro = np.zeros(nghl)
    y2 = mb.y * mb.y
    start = 0
    for ib, nd in enumerate(h.ID):
        nd = int(nd)
        ns = h.ns[start:start + nd]
        up, dn = ns > 0, ns < 0
        sl = slice(start, start + nd)
        xl2, xp2 = mb.xlam[ib] ** 2 * y2, mb.xlap[ib] ** 2 * y2
        thermal = qp.fwin is not None
        parts = [(qp.V[ib][:, qp.active[ib]], 1.0 - qp.fwin[ib] if thermal else None)]
        if thermal:
            parts.append((qp.U[ib][:, qp.active[ib]], qp.fwin[ib]))
        for W, wk in parts:
            Wu, Wd = W[up].T, W[dn].T

            def comp(a):
                a = a[sl]
                return Wu @ a[up], Wd @ a[dn]
            fu, fd = comp(mb.qhla)
            fur, fdr = comp(mb.fi1r)
            fuz, fdz = comp(mb.fi1z)
            fu2, fd2 = comp(mb.fi2d)
            kw = (lambda x: x) if wk is None else (lambda x: x * wk[:, None])
            tw = np.sum(kw(fur * fur + fdr * fdr + fuz * fuz + fdz * fdz), axis=0)
            tro += np.sum(kw(fu * fu + fd * fd), axis=0)
            ttau += np.sum(kw(xl2 * fu * fu + xp2 * fd * fd), axis=0) + tw
            tdro += np.sum(kw(fu * fu2 + fd * fd2), axis=0) + tw
        start += nd
    s = 2.0 * tro.sum()
    wgt = mb.wdcori * (2.0 * tz / s)
    return tro * wgt, ttau * wgt, tdro * (2.0 * wgt)


def local_density(h: HelData, mb: MeshBasis, qp: QPSolution, tz: float) -> np.ndarray:
    """rho(r) of one isospin from the final quasiparticles (DENSIT, T=0)."""
    return local_densities(h, mb, qp, tz)[0]


# ----------------------------------------------------------------------------
# 5. pnFAM view of the solution (TR doubling, spin sort, pairing window)
# ----------------------------------------------------------------------------
@dataclass
class HFBSolution:
    """The ground state in the layout the FAM kernels consume.

    Doubled basis of ``dqp`` states in ``nb`` blocks (blocks nb/2.. are the
    time-reversed partners of blocks 0..nb/2-1), spin-up states first inside
    every block.  U is block diagonal; V maps block i to its partner
    (i +- nb/2).  Block matrices are stored block by block, column-major inside
    a block (Fortran order), in block-row order.
    """
    Z: int
    N: int
    n00: int
    nb: int
    db: np.ndarray          # [nb]
    isstart: np.ndarray     # [nb] first state of each block (0-based)
    nr: np.ndarray
    nz: np.ndarray
    nl: np.ndarray
    ns: np.ndarray
    npar: np.ndarray
    num_spin_up: np.ndarray # [nb]
    nghl: int
    wf: np.ndarray          # [dqp, nghl]
    wfdr: np.ndarray
    wfdz: np.ndarray
    wfdp: np.ndarray        # y*nl*wf
    wfd2_all: np.ndarray    # wfd2 - y*nl*wfdp
    y: np.ndarray
    z: np.ndarray
    wdcori: np.ndarray
    Ep: np.ndarray          # [dqp]
    En: np.ndarray
    Up: list                # per block row: [db, db] (block-diagonal)
    Vp: list                # per block row i: [db_i, db_partner]
    Un: list
    Vn: list
    rho_n: np.ndarray       # [nghl] local densities (for couplings)
    rho_p: np.ndarray
    hel: HelData
    tau_n: np.ndarray = None    # [nghl] kinetic densities (two-body-current fields)
    tau_p: np.ndarray = None
    d2rho_n: np.ndarray = None  # [nghl] Laplacian of the densities
    d2rho_p: np.ndarray = None
    temperature: float = 0.0    # MeV; > 0: the statistical FAM with occupations fp, fn
    fp: np.ndarray = None       # [dqp] thermal quasiparticle occupations
    fn: np.ndarray = None

    @property
    def occupations(self):
        """(fp, fn) of a finite-temperature solution, None at T = 0."""
        return None if self.fp is None else (self.fp, self.fn)

    @property
    def dqp(self) -> int:
        return int(self.db.sum())

    def partner(self, ib: int) -> int:
        half = self.nb // 2
        return ib + half if ib < half else ib - half

    def density_matrices(self, it: str) -> list:
        """HFBTHO's oscillator-basis density matrix ``rk`` (twice rho) of isospin
        ``it`` ('n' or 'p') per HFBTHO block, in HFBTHO's state order
        (hfbdiag, hfbtho_solver.f90:1819-1856): rk = 2 sum_k V_ik V_jk over the
        pairing-window quasiparticles, at temperature T the sum of
        V (1 - f_k) V + U f_k U."""
        U, V = (self.Un, self.Vn) if it == "n" else (self.Up, self.Vp)
        f = self.occupations[1 if it == "n" else 0] if self.occupations is not None else None
        h = self.hel
        half = self.nb // 2
        out = []
        for ib in range(half):
            s0, d = int(self.isstart[ib]), int(self.db[ib])
            v = V[ib]
            if f is None:
                rk = 2.0 * (v @ v.T)
            else:
                fu = f[s0:s0 + d]
                pr = int(self.isstart[ib + half])
                fv = f[pr:pr + d]
                rk = 2.0 * ((v * (1.0 - fv)) @ v.T + (U[ib] * fu) @ U[ib].T)
            # undo the spin sort: sorted position i holds HFBTHO state perm[i]
            ns = np.asarray(h.ns[s0:s0 + d])
            perm = np.concatenate([np.nonzero(ns > 0)[0], np.nonzero(ns < 0)[0]])
            r = np.empty_like(rk)
            r[np.ix_(perm, perm)] = rk
            out.append(r)
        return out


def load_hfb_solution(path, device: bool = None) -> HFBSolution:
    """get_raw_hfb_solution (hfbtho_solution.f90:137-395) from a ``.hel`` file
    (a path, or an already decoded :class:`HelData`).  A finite-temperature
    solution is rebuilt with HFBTHO's thermal particle number and densities and
    carries the quasiparticle occupations of the statistical FAM.  ``device``: the
    basis functions, HFB matrices, eigensolves and densities on the GPU
    (``hfb_device``); default from PNFAM_GB300_HFB_DEVICE=1, else the host."""
    if device is None:
        import os
        device = os.environ.get("PNFAM_GB300_HFB_DEVICE", "0") == "1"
    h = path if isinstance(path, HelData) else read_hel(path)
    if int(h.N) % 2 or int(h.Z) % 2:
        # an odd nucleus is an HFBTHO solution with a blocked quasiparticle, whose
        # reconstruction (blocked hfbdiag/ALambda/DENSIT) this reader does not restate
        raise ValueError(f"the .hel ground state has N = {h.N}, Z = {h.Z}: rebuilding blocked odd-nucleus solutions "
                         "is not supported (pass EFA occupations from pynfam_gb300.statistics to GPUSolver to run "
                         "the statistical FAM on an even-even basis)")
    temper = h.temperature if h.set_temperature else 0.0
    if device:
        from . import hfb_device as dv
        mb = build_mesh_basis(h, device=True)
        hd = dv.hfb_matrices(h, mb)
        eigh, dens = dv.eigh_batch, dv.local_densities
    else:
        mb = build_mesh_basis(h)
        hd = hfb_matrices(h, mb)
        eigh, dens = None, None
    qpn = diagonalise(h, hd, "n", float(h.N), temper, eigh and dv.eigh_chain())
    qpp = diagonalise(h, hd, "p", float(h.Z), temper, eigh and dv.eigh_chain())
    hfb = assemble(h, mb, qpn, qpp, dens)
    if temper > 1e-12:
        # the statistical FAM's occupations from the final quasiparticle energies,
        # 0 above the pairing window (hfbtho_solution.f90:376-389, 426, 446)
        from .statistics import thermal_occupations
        hfb.temperature = temper
        hfb.fp, hfb.fn = thermal_occupations(hfb, temper)
    return hfb


def assemble(h: HelData, mb: MeshBasis, qpn: QPSolution, qpp: QPSolution, densities=None) -> HFBSolution:
    """The pnFAM view of Omega>0 quasiparticles (hfbtho_solution.f90:164-459): TR
    doubling, spin sort inside each block, pairing window."""
    dens = densities or local_densities
    rho_n, tau_n, d2rho_n = dens(h, mb, qpn, float(h.N))
    rho_p, tau_p, d2rho_p = dens(h, mb, qpp, float(h.Z))

    nbh = len(h.ID)
    nb = 2 * nbh
    db = np.concatenate([h.ID, h.ID]).astype(np.int64)
    nt = len(h.nr)
    nr = np.concatenate([h.nr, h.nr]); nz = np.concatenate([h.nz, h.nz])
    nl = np.concatenate([h.nl, -h.nl]); ns = np.concatenate([h.ns, -h.ns])
    npar = 1 + (h.nz + h.nl) % 2
    npar = np.concatenate([npar, npar])
    sign = np.where(h.ns < 0, -1.0, 1.0)[:, None]
    wf = np.concatenate([mb.qhla, sign * mb.qhla])
    wfdr = np.concatenate([mb.fi1r, sign * mb.fi1r])
    wfdz = np.concatenate([mb.fi1z, sign * mb.fi1z])
    wfd2 = np.concatenate([mb.fi2d, sign * mb.fi2d])

    isstart = np.concatenate([[0], np.cumsum(db)[:-1]]).astype(np.int64)
    # spin sort inside each (doubled) block
    new_order = np.empty(2 * nt, dtype=np.int64)
    num_up = np.zeros(nb, dtype=np.int64)
    for ib in range(nb):
        s0, d = isstart[ib], db[ib]
        idx = np.arange(s0, s0 + d)
        upi = idx[ns[idx] > 0]; dni = idx[ns[idx] < 0]
        num_up[ib] = len(upi)
        new_order[s0:s0 + d] = np.concatenate([upi, dni])
    nr, nz, nl, ns, npar = nr[new_order], nz[new_order], nl[new_order], ns[new_order], npar[new_order]
    wf, wfdr, wfdz, wfd2 = wf[new_order], wfdr[new_order], wfdz[new_order], wfd2[new_order]
    y = mb.y
    wfdp = y[None, :] * nl[:, None] * wf
    wfd2_all = wfd2 - y[None, :] * nl[:, None] * wfdp

    def doubled(qp: QPSolution):
        E = np.concatenate(qp.E + qp.E)
        act = np.concatenate(qp.active + qp.active)
        U = [u.copy() for u in qp.U] + [u.copy() for u in qp.U]
        V = [-v for v in qp.V] + [v.copy() for v in qp.V]
        # rows of U, V follow the spin sort of their block row
        for ib in range(nb):
            s0, d = isstart[ib], db[ib]
            perm = new_order[s0:s0 + d] - s0
            U[ib] = U[ib][perm]
            V[ib] = V[ib][perm]
        # erase quasiparticles above the pairing window (columns); the QP
        # columns of block row i live in block i for U and partner(i) for V
        for ib in range(nb):
            s0, d = isstart[ib], db[ib]
            a = act[s0:s0 + d]
            U[ib][:, ~a] = 0.0
            pr = ib + nbh if ib < nbh else ib - nbh
            V[pr][:, ~a] = 0.0
        E = np.where(act, E, 0.0)
        return E, U, V

    Ep, Up, Vp = doubled(qpp)
    En, Un, Vn = doubled(qpn)
    return HFBSolution(h.Z, h.N, h.n00, nb, db, isstart, nr, nz, nl, ns, npar, num_up,
                       h.ngh * h.ngl, wf, wfdr, wfdz, wfdp, wfd2_all, y, mb.z, mb.wdcori,
                       Ep, En, Up, Vp, Un, Vn, rho_n, rho_p, h, tau_n, tau_p, d2rho_n, d2rho_p)
