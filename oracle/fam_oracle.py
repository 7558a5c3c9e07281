"""CPU FP64 oracle for the pnFAM iteration -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this module, and only as the checker or the timed CPU
baseline.  The product path (pynfam_gb300 + its CUDA library) never calls it.

A numpy restatement of the reference's FAM solver, written to follow the
reference's structure closely so that each step can be checked line by line:

* quadrant ("bigblock") algebra with stored signs and transposes:
  pnfam_type_bbm.f90:217-576 (``triprod_bbm_quad`` :428-552, ``contract_bbm``
  :393-421) on top of ``triprod`` (pnfam_type_blockmatrix.f90:140-212);
* solver set-up: pnfam_solver.f90:226-460 (``init_pnfam_solver``) and the
  Green's function ``matrix_2qp`` :510-544;
* the iteration ``ifam``: pnfam_solver.f90:93-221;
* the residual-interaction field ``calc_hamiltonian``:
  pnfam_hamiltonian_blas.f90:51-74 (density :124-711, meanfield :717-1169,
  pairingfield :1175-1262);
* modified Broyden mixing: pnfam_broyden.f90:26-216.

Complex (Re, Im) pairs of the reference are held as complex128 arrays where
that reads the same; the Broyden vector is the reference's real layout.

Parity pinning: checked against the reference's recorded FP64 outputs of
``pnfam_main`` (tests/golden/), see tests/test_oracle_golden.py.
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass, field

import numpy as np

from pynfam_gb300.blockmatrix import BlockMatrix

PI = 3.141592653589793238462643


# -----------------------------------------------------------------------------
# block-level triple product (pnfam_type_blockmatrix.f90:140-212)
# -----------------------------------------------------------------------------
def _ic2r(m: BlockMatrix) -> np.ndarray:
    inv = np.full(len(m.cols), -1, dtype=np.int64)
    for i, c in enumerate(m.cols):
        if c >= 0:
            inv[c] = i
    return inv


def _op(t, m: BlockMatrix, i):
    """(next block index, block) of op(M) in block row i."""
    if t == "n":
        k = m.cols[i]
        return (k, m.blocks[i]) if k >= 0 else (-1, None)
    k = _ic2r(m)[i]
    return (k, m.blocks[k].T) if k >= 0 else (-1, None)


def triprod(ta, a, tb, b, tc, c, alpha, acc: dict):
    """acc[i] = (j, block) += alpha * op(A) op(B) op(C) for each block row i."""
    nb = len(a.cols)
    cols = np.full(nb, -1, dtype=np.int64)
    for i in range(nb):
        k, A = _op(ta, a, i)
        if k < 0:
            continue
        l, B = _op(tb, b, k)
        if l < 0:
            continue
        j, C = _op(tc, c, l)
        if j < 0:
            continue
        cols[i] = j
        prod = alpha * (A @ B @ C)
        if i in acc:
            jj, blk = acc[i]
            assert jj == j, "inconsistent block structure in triprod"
            acc[i] = (j, blk + prod)
        else:
            acc[i] = (j, prod)
    return cols


# -----------------------------------------------------------------------------
# bigblock matrices (pnfam_type_bbm.f90)
# -----------------------------------------------------------------------------
@dataclass
class BBM:
    q: dict = field(default_factory=lambda: {11: None, 12: None, 21: None, 22: None})
    s: dict = field(default_factory=lambda: {11: 1.0, 12: 1.0, 21: 1.0, 22: 1.0})
    t: dict = field(default_factory=lambda: {11: "n", 12: "n", 21: "n", 22: "n"})
    imag: bool = False

    def copy(self):
        return BBM(dict(self.q), dict(self.s), dict(self.t), self.imag)


def transpose_bbm(a: BBM) -> BBM:
    b = a.copy()
    b.q[12], b.q[21] = a.q[21], a.q[12]
    b.s[12], b.s[21] = a.s[21], a.s[12]
    b.t = {k: ("t" if v == "n" else "n") for k, v in a.t.items()}
    return b


_TERMS = {
    11: ((11, 11, 11), (12, 21, 11), (11, 12, 21), (12, 22, 21)),
    12: ((11, 11, 12), (12, 21, 12), (11, 12, 22), (12, 22, 22)),
    21: ((21, 11, 11), (22, 21, 11), (21, 12, 21), (22, 22, 21)),
    22: ((21, 11, 12), (22, 21, 12), (21, 12, 22), (22, 22, 22)),
}


def triprod_bbm_quad(ta, ain, tb, bin_, tc, cin, quad, sabc, tabc, nb, db) -> BlockMatrix:
    a, b, c = ain.copy(), bin_.copy(), cin.copy()
    s = sabc
    if ta == "t": a = transpose_bbm(a)
    if tb == "t": b = transpose_bbm(b)
    if tc == "t": c = transpose_bbm(c)
    if tabc == "t":
        a, c = c, a
        a, b, c = transpose_bbm(a), transpose_bbm(b), transpose_bbm(c)
        quad = {12: 21, 21: 12}.get(quad, quad)
    im = int(a.imag) + int(b.imag) + int(c.imag)
    if im >= 2:
        s = -s
    acc = {}
    cols = None
    for (qa, qb, qc) in _TERMS[quad]:
        if a.q[qa] is None or b.q[qb] is None or c.q[qc] is None:
            continue
        cols = triprod(a.t[qa], a.q[qa], b.t[qb], b.q[qb], c.t[qc], c.q[qc],
                       s * a.s[qa] * b.s[qb] * c.s[qc], acc)
    if cols is None:
        cols = np.full(nb, -1, dtype=np.int64)
    blocks = [None] * nb
    for i in range(nb):
        if cols[i] >= 0:
            blocks[i] = acc[i][1]
    return BlockMatrix(cols, blocks)


def triprod_bbm(ta, a, tb, b, tc, c, abc: BBM, nb, db) -> BBM:
    out = abc.copy()
    for quad in (11, 12, 21, 22):
        if abc.q[quad] is not None:
            out.q[quad] = triprod_bbm_quad(ta, a, tb, b, tc, c, quad, abc.s[quad], abc.t[quad], nb, db)
    return out


def contract_bbm(a: BBM, b: BBM) -> float:
    s = 0.0
    for quad in (11, 12, 21, 22):
        if a.q[quad] is not None and b.q[quad] is not None:
            s += float(np.dot(a.q[quad].flatten(), b.q[quad].flatten()))
    if int(a.imag) + int(b.imag) == 2:
        s = -s
    return s


# -----------------------------------------------------------------------------
# residual-interaction field (pnfam_hamiltonian_blas.f90)
# -----------------------------------------------------------------------------
class _Basis:
    """Mesh arrays of the doubled, spin-sorted basis as [nghl, dqp]."""

    def __init__(self, hfb):
        self.hfb = hfb
        self.P = [hfb.wf.T, hfb.wfdr.T, hfb.wfdp.T, hfb.wfdz.T, hfb.wfd2_all.T]
        self.ns = hfb.ns.astype(np.int64)
        self.nghl = hfb.nghl
        self.dqp = hfb.dqp


def _wfa_rho(basis: _Basis, re: BlockMatrix, im: BlockMatrix, nphi: int):
    """Sum_a phi_a rho_ab, per spin of a (density :184-238); complex."""
    h = basis.hfb
    out = {s: [np.zeros((basis.nghl, basis.dqp), dtype=complex) for _ in range(nphi)] for s in (1, -1)}
    for ix in range(h.nb):
        iy = re.cols[ix]
        if iy < 0:
            continue
        ia, ib = h.isstart[ix], h.isstart[iy]
        nup, d, dc = h.num_spin_up[ix], h.db[ix], h.db[iy]
        blk = re.blocks[ix] + 1j * im.blocks[ix]
        for p in range(nphi):
            ph = basis.P[p]
            if nup > 0:
                out[1][p][:, ib:ib + dc] = ph[:, ia:ia + nup] @ blk[:nup]
            if d - nup > 0:
                out[-1][p][:, ib:ib + dc] = ph[:, ia + nup:ia + d] @ blk[nup:]
    return out


def density(basis: _Basis, rerho, imrho, rek, imk, wdcori):
    """Local densities (complex) on the mesh; names as in the reference."""
    ns = basis.ns
    P0, P1, P2, P3 = basis.P[0], basis.P[1], basis.P[2], basis.P[3]
    w = _wfa_rho(basis, rerho, imrho, 4)
    up = ns > 0
    # same spin: wfa_rhoab(ns(b)); opposite: wfa_rhoab(-ns(b))
    S = [np.where(up[None, :], w[1][p], w[-1][p]) for p in range(4)]
    O = [np.where(up[None, :], w[-1][p], w[1][p]) for p in range(4)]
    nsf = ns.astype(float)[None, :]
    d = {}
    sm = lambda x: x.sum(axis=1)
    # diagonal in spin (:264-350)
    w0 = S[0] * P0
    d["rho"] = sm(w0)
    d["sz"] = sm(nsf * w0)
    a = (S[0] * P2 + S[2] * P0) / 2
    d["jp"] = sm(a)
    d["tjpz"] = sm(nsf * a)
    t = S[1] * P1 + S[2] * P2 + S[3] * P3
    d["tau"] = sm(t)
    d["tz"] = sm(nsf * t)
    a = (S[0] * P1 - S[1] * P0) / 2
    d["jr"] = 1j * sm(a)
    d["tjrz"] = 1j * sm(nsf * a)
    a = (S[0] * P3 - S[3] * P0) / 2
    d["jz"] = 1j * sm(a)
    d["tjzz"] = 1j * sm(nsf * a)
    d["gs"] = sm(nsf * (S[0] * P3 + S[3] * P0))
    d["fr"] = sm(nsf * (S[1] * P3 + S[3] * P1)) / 2
    d["fp"] = 1j * sm(nsf * (S[2] * P3 - S[3] * P2)) / 2
    d["fz"] = sm(nsf * S[3] * P3)
    # not diagonal in spin (:353-584); mdn: b is spin down (a up), mup: b up
    mdn = (~up)[None, :].astype(float)
    mup = up[None, :].astype(float)
    wo = O[0] * P0
    d["sr"] = sm(wo)
    d["sp"] = 1j * sm((mdn - mup) * wo)
    a1 = (O[2] * P0 + O[0] * P2) / 2
    d["tjpr"] = sm(a1)
    d["tjpp"] = 1j * sm((mdn - mup) * a1)
    d["gs"] = d["gs"] + sm((mdn - mup) * (O[0] * P2 - O[2] * P0)) + sm(O[0] * P1 + O[1] * P0)
    a3 = O[1] * P1 + O[2] * P2 + O[3] * P3
    d["tr"] = sm(a3)
    d["tp"] = 1j * sm((mdn - mup) * a3)
    a4 = (O[0] * P1 - O[1] * P0) / 2
    d["tjrr"] = 1j * sm(a4)
    d["tjrp"] = sm((mup - mdn) * a4)
    a5 = (O[0] * P3 - O[3] * P0) / 2
    d["tjzr"] = 1j * sm(a5)
    d["tjzp"] = sm((mup - mdn) * a5)
    fr_dn = O[1] * (P1 + 0.5 * P2) - 0.5 * O[2] * P1
    fr_up = O[1] * (P1 - 0.5 * P2) + 0.5 * O[2] * P1
    d["fr"] = d["fr"] + sm(mdn * fr_dn + mup * fr_up)
    fp_dn = O[2] * P2 + 0.5 * (O[2] * P1 - O[1] * P2)
    fp_up = -O[2] * P2 + 0.5 * (O[2] * P1 - O[1] * P2)
    d["fp"] = d["fp"] + 1j * sm(mdn * fp_dn + mup * fp_up)
    fz_dn = O[3] * (P1 + P2) + O[1] * P3 - O[2] * P3
    fz_up = O[3] * (P1 - P2) + O[1] * P3 + O[2] * P3
    d["fz"] = d["fz"] + sm(mdn * fz_dn + mup * fz_up) / 2
    # pairing densities (:596-675)
    k = _wfa_rho(basis, rek, imk, 1)
    Sk = np.where(up[None, :], k[1][0], k[-1][0])
    Ok = np.where(up[None, :], k[-1][0], k[1][0])
    wk = 2 * Ok * P0
    d["rb"] = -sm(nsf * wk)
    d["sbz"] = sm(wk)
    wk = 2 * Sk * P0
    d["sbr"] = sm((mdn - mup) * wk)
    d["sbp"] = -1j * sm(wk)
    for key in d:
        d[key] = d[key] * wdcori
    return d


def meanfield(basis: _Basis, ds, cp, re_cols, db, isstart, num_up):
    """h_ab from the densities (:717-1169), literal re/im transcription."""
    R = lambda x: x.real
    I = lambda x: x.imag
    C = lambda re, im: re + 1j * im
    crho, cs = cp.crho, cp.cs
    ctau, cj, ct, cdrho, cds, crdj, csdj = cp.ctau, cp.cj, cp.ct, cp.cdrho, cp.cds, cp.crdj, cp.csdj
    ctj0, ctj1, ctj2, cf, cgs = cp.ctj0, cp.ctj1, cp.ctj2, cp.cf, cp.cgs
    n = basis.nghl
    mf = {}
    z = lambda: np.zeros(n, dtype=complex)
    for sb in (-1, 1):
        for sa in (-1, 1):
            for ib in range(4):
                for ia in range(4):
                    mf[(ia, ib, sa, sb)] = z()
            mf[(0, 4, sa, sb)] = z(); mf[(4, 0, sa, sb)] = z()

    def add(key, sym, f):
        mf[key] = mf[key] + sym * f

    d = ds
    t0 = ctj0 * (d["tjrr"] + d["tjpp"] + d["tjzz"])
    t1a = ctj1 * (d["tjzr"] - d["tjrz"])
    t1b = ctj1 * (d["tjpz"] - d["tjzp"])
    t2a = ctj2 * (d["tjrz"] + d["tjzr"])
    t2b = ctj2 * (d["tjpz"] + d["tjzp"])

    mf[(0, 0, 1, 1)] = 2.0 * crho * d["rho"] + ctau * d["tau"]
    mf[(0, 0, -1, -1)] = mf[(0, 0, 1, 1)].copy()
    aux = 2.0 * cs * d["sz"] + ct * d["tz"] + cf * d["fz"]
    add((0, 0, 1, 1), 1, aux); add((0, 0, -1, -1), -1, aux)

    mf[(0, 1, 1, 1)] = -crdj * (d["tjpz"] - d["tjzp"])
    mf[(0, 1, -1, -1)] = mf[(0, 1, 1, 1)].copy()
    aux = -csdj * d["jp"]
    add((0, 1, 1, 1), 1, aux); add((0, 1, -1, -1), -1, aux)
    mf[(1, 0, 1, 1)] = mf[(0, 1, 1, 1)].copy()
    mf[(1, 0, -1, -1)] = mf[(0, 1, -1, -1)].copy()
    aux = C(-I(t1a) + 0.5 * I(t2a), R(t1a) - 0.5 * R(t2a))
    add((0, 1, 1, 1), 1, aux); add((0, 1, -1, -1), -1, aux)
    add((1, 0, 1, 1), -1, aux); add((1, 0, -1, -1), 1, aux)
    aux = C(cj * I(d["jr"]), -cj * R(d["jr"]))
    add((0, 1, 1, 1), 1, aux); add((0, 1, -1, -1), 1, aux)
    add((1, 0, 1, 1), -1, aux); add((1, 0, -1, -1), -1, aux)

    mf[(0, 2, 1, 1)] = cj * d["jp"]
    mf[(0, 2, -1, -1)] = mf[(0, 2, 1, 1)].copy()
    aux = t1b + 0.5 * t2b
    add((0, 2, 1, 1), 1, aux); add((0, 2, -1, -1), -1, aux)
    mf[(2, 0, 1, 1)] = mf[(0, 2, 1, 1)].copy()
    mf[(2, 0, -1, -1)] = mf[(0, 2, -1, -1)].copy()
    aux = C(-csdj * I(d["jr"]), csdj * R(d["jr"]))
    add((0, 2, 1, 1), 1, aux); add((0, 2, -1, -1), -1, aux)
    add((2, 0, 1, 1), -1, aux); add((2, 0, -1, -1), 1, aux)
    aux = C(crdj * I(d["tjzr"] - d["tjrz"]), -crdj * R(d["tjzr"] - d["tjrz"]))
    add((0, 2, 1, 1), 1, aux); add((0, 2, -1, -1), 1, aux)
    add((2, 0, 1, 1), -1, aux); add((2, 0, -1, -1), -1, aux)

    mf[(0, 3, 1, 1)] = -crdj * (d["tjrp"] - d["tjpr"])
    mf[(0, 3, -1, -1)] = mf[(0, 3, 1, 1)].copy()
    aux = 2.0 * cgs * d["gs"]
    add((0, 3, 1, 1), 1, aux); add((0, 3, -1, -1), -1, aux)
    mf[(3, 0, 1, 1)] = mf[(0, 3, 1, 1)].copy()
    mf[(3, 0, -1, -1)] = mf[(0, 3, -1, -1)].copy()
    trr, tpp, tzz = d["tjrr"], d["tjpp"], d["tjzz"]
    aux = C(I(t0) - ctj2 * (I(trr) + I(tpp) - 2.0 * I(tzz)) / 3.0,
            -R(t0) + ctj2 * (R(trr) + R(tpp) - 2.0 * R(tzz)) / 3.0)
    add((0, 3, 1, 1), 1, aux); add((0, 3, -1, -1), -1, aux)
    add((3, 0, 1, 1), -1, aux); add((3, 0, -1, -1), 1, aux)
    aux = C(cj * I(d["jz"]), -cj * R(d["jz"]))
    add((0, 3, 1, 1), 1, aux); add((0, 3, -1, -1), 1, aux)
    add((3, 0, 1, 1), -1, aux); add((3, 0, -1, -1), -1, aux)

    mf[(0, 4, 1, 1)] = 2.0 * cdrho * d["rho"]
    mf[(0, 4, -1, -1)] = mf[(0, 4, 1, 1)].copy()
    aux = 2.0 * cds * d["sz"]
    add((0, 4, 1, 1), 1, aux); add((0, 4, -1, -1), -1, aux)
    mf[(4, 0, 1, 1)] = mf[(0, 4, 1, 1)].copy()
    mf[(4, 0, -1, -1)] = mf[(0, 4, -1, -1)].copy()

    mf[(1, 2, 1, 1)] = csdj * d["sz"]
    mf[(1, 2, -1, -1)] = mf[(1, 2, 1, 1)].copy()
    aux = crdj * d["rho"]
    add((1, 2, 1, 1), 1, aux); add((1, 2, -1, -1), -1, aux)
    mf[(2, 1, 1, 1)] = mf[(1, 2, 1, 1)].copy()
    mf[(2, 1, -1, -1)] = mf[(1, 2, -1, -1)].copy()

    mf[(1, 3, 1, 1)] = 0.5 * cf * d["sr"]
    mf[(1, 3, -1, -1)] = -mf[(1, 3, 1, 1)]
    mf[(3, 1, 1, 1)] = mf[(1, 3, 1, 1)].copy()
    mf[(3, 1, -1, -1)] = mf[(1, 3, -1, -1)].copy()
    aux = C(-csdj * I(d["sp"]), csdj * R(d["sp"]))
    add((1, 3, 1, 1), 1, aux); add((1, 3, -1, -1), 1, aux)
    add((3, 1, 1, 1), -1, aux); add((3, 1, -1, -1), -1, aux)

    mf[(2, 3, 1, 1)] = -csdj * d["sr"]
    mf[(2, 3, -1, -1)] = mf[(2, 3, 1, 1)].copy()
    aux = C(0.5 * cf * I(d["sp"]), -0.5 * cf * R(d["sp"]))
    add((2, 3, 1, 1), 1, aux); add((2, 3, -1, -1), -1, aux)
    mf[(3, 2, 1, 1)] = mf[(2, 3, -1, -1)].copy()
    mf[(3, 2, -1, -1)] = mf[(2, 3, 1, 1)].copy()

    mf[(1, 1, 1, 1)] = (4.0 * cdrho + ctau) * d["rho"]
    mf[(1, 1, -1, -1)] = mf[(1, 1, 1, 1)].copy()
    aux = (4.0 * cds + ct) * d["sz"]
    add((1, 1, 1, 1), 1, aux); add((1, 1, -1, -1), -1, aux)
    mf[(2, 2, 1, 1)] = mf[(1, 1, 1, 1)].copy()
    mf[(2, 2, -1, -1)] = mf[(1, 1, -1, -1)].copy()
    mf[(3, 3, 1, 1)] = mf[(1, 1, 1, 1)].copy()
    mf[(3, 3, -1, -1)] = mf[(1, 1, -1, -1)].copy()
    aux = cf * d["sz"]
    add((3, 3, 1, 1), 1, aux); add((3, 3, -1, -1), -1, aux)

    # not diagonal in spin
    mf[(0, 0, 1, -1)] = 2.0 * cs * d["sr"] + ct * d["tr"] + cf * d["fr"]
    mf[(0, 0, -1, 1)] = mf[(0, 0, 1, -1)].copy()
    aux = C(2.0 * cs * I(d["sp"]) + ct * I(d["tp"]) + cf * I(d["fp"]),
            -2.0 * cs * R(d["sp"]) - ct * R(d["tp"]) - cf * R(d["fp"]))
    add((0, 0, 1, -1), 1, aux); add((0, 0, -1, 1), -1, aux)

    mf[(0, 1, 1, -1)] = 2.0 * cgs * d["gs"]
    mf[(0, 1, -1, 1)] = mf[(0, 1, 1, -1)].copy()
    aux = C(csdj * I(d["jz"]), -csdj * R(d["jz"]))
    add((0, 1, 1, -1), 1, aux); add((0, 1, -1, 1), -1, aux)
    mf[(1, 0, 1, -1)] = mf[(0, 1, 1, -1)].copy()
    mf[(1, 0, -1, 1)] = mf[(0, 1, -1, 1)].copy()
    mf[(0, 2, 1, -1)] = mf[(0, 1, 1, -1)].copy()
    mf[(2, 0, -1, 1)] = mf[(1, 0, -1, 1)].copy()
    mf[(2, 0, 1, -1)] = -mf[(0, 2, 1, -1)]
    mf[(0, 2, -1, 1)] = -mf[(2, 0, -1, 1)]
    aux = -ctj1 * (d["tjrp"] - d["tjpr"])
    for key, sg in (((0, 1, 1, -1), 1), ((0, 1, -1, 1), -1), ((1, 0, 1, -1), -1), ((1, 0, -1, 1), 1),
                    ((0, 2, 1, -1), 1), ((0, 2, -1, 1), 1), ((2, 0, 1, -1), 1), ((2, 0, -1, 1), 1)):
        add(key, sg, aux)
    aux = C(I(t0), -R(t0))
    for key, sg in (((0, 1, 1, -1), 1), ((0, 1, -1, 1), 1), ((1, 0, 1, -1), -1), ((1, 0, -1, 1), -1),
                    ((0, 2, 1, -1), 1), ((0, 2, -1, 1), -1), ((2, 0, 1, -1), 1), ((2, 0, -1, 1), -1)):
        add(key, sg, aux)
    aux = -0.5 * ctj2 * (d["tjrp"] + d["tjpr"])
    for key, sg in (((0, 1, 1, -1), 1), ((0, 1, -1, 1), -1), ((1, 0, 1, -1), -1), ((1, 0, -1, 1), 1),
                    ((0, 2, 1, -1), -1), ((0, 2, -1, 1), -1), ((2, 0, 1, -1), -1), ((2, 0, -1, 1), -1)):
        add(key, sg, aux)
    aux = C(-ctj2 * (-2.0 * I(trr) + I(tpp) + I(tzz)) / 3.0, ctj2 * (-2.0 * R(trr) + R(tpp) + R(tzz)) / 3.0)
    for key, sg in (((0, 1, 1, -1), 1), ((0, 1, -1, 1), 1), ((1, 0, 1, -1), -1), ((1, 0, -1, 1), -1)):
        add(key, sg, aux)
    aux = C(-ctj2 * (I(trr) - 2.0 * I(tpp) + I(tzz)) / 3.0, ctj2 * (R(trr) - 2.0 * R(tpp) + R(tzz)) / 3.0)
    for key, sg in (((0, 2, 1, -1), 1), ((0, 2, -1, 1), -1), ((2, 0, 1, -1), 1), ((2, 0, -1, 1), -1)):
        add(key, sg, aux)

    mf[(0, 3, 1, -1)] = csdj * d["jp"]
    mf[(0, 3, -1, 1)] = mf[(0, 3, 1, -1)].copy()
    aux = C(-csdj * I(d["jr"]), csdj * R(d["jr"]))
    add((0, 3, 1, -1), 1, aux); add((0, 3, -1, 1), -1, aux)
    mf[(3, 0, 1, -1)] = mf[(0, 3, 1, -1)].copy()
    mf[(3, 0, -1, 1)] = mf[(0, 3, -1, 1)].copy()
    aux = C(I(t1a) + 0.5 * I(t2a), -R(t1a) - 0.5 * R(t2a))
    for key, sg in (((0, 3, 1, -1), 1), ((0, 3, -1, 1), 1), ((3, 0, 1, -1), -1), ((3, 0, -1, 1), -1)):
        add(key, sg, aux)
    aux = t1b - 0.5 * t2b
    for key, sg in (((0, 3, 1, -1), 1), ((0, 3, -1, 1), -1), ((3, 0, 1, -1), -1), ((3, 0, -1, 1), 1)):
        add(key, sg, aux)

    mf[(0, 4, 1, -1)] = 2.0 * cds * d["sr"]
    mf[(0, 4, -1, 1)] = mf[(0, 4, 1, -1)].copy()
    aux = C(2.0 * cds * I(d["sp"]), -2.0 * cds * R(d["sp"]))
    add((0, 4, 1, -1), 1, aux); add((0, 4, -1, 1), -1, aux)
    mf[(4, 0, 1, -1)] = mf[(0, 4, 1, -1)].copy()
    mf[(4, 0, -1, 1)] = mf[(0, 4, -1, 1)].copy()

    mf[(1, 2, 1, -1)] = C(-0.5 * cf * I(d["sp"]), 0.5 * cf * R(d["sp"]))
    mf[(1, 2, -1, 1)] = mf[(1, 2, 1, -1)].copy()
    aux = 0.5 * cf * d["sr"]
    add((1, 2, 1, -1), 1, aux); add((1, 2, -1, 1), -1, aux)
    mf[(2, 1, 1, -1)] = -mf[(1, 2, 1, -1)]
    mf[(2, 1, -1, 1)] = -mf[(1, 2, -1, 1)]

    mf[(1, 3, 1, -1)] = 0.5 * cf * d["sz"]
    mf[(1, 3, -1, 1)] = mf[(1, 3, 1, -1)].copy()
    aux = crdj * d["rho"]
    add((1, 3, 1, -1), 1, aux); add((1, 3, -1, 1), -1, aux)
    mf[(3, 1, 1, -1)] = mf[(1, 3, -1, 1)].copy()
    mf[(3, 1, -1, 1)] = mf[(1, 3, 1, -1)].copy()
    mf[(3, 2, 1, -1)] = mf[(3, 1, 1, -1)].copy()
    mf[(2, 3, -1, 1)] = mf[(1, 3, -1, 1)].copy()
    mf[(2, 3, 1, -1)] = -mf[(1, 3, 1, -1)]
    mf[(3, 2, -1, 1)] = -mf[(3, 1, -1, 1)]

    mf[(3, 3, 1, -1)] = (ct + 4.0 * cds) * d["sr"]
    mf[(3, 3, -1, 1)] = mf[(3, 3, 1, -1)].copy()
    aux = C((ct + 4.0 * cds) * I(d["sp"]), -(ct + 4.0 * cds) * R(d["sp"]))
    add((3, 3, 1, -1), 1, aux); add((3, 3, -1, 1), -1, aux)
    mf[(1, 1, 1, -1)] = mf[(3, 3, 1, -1)].copy()
    mf[(1, 1, -1, 1)] = mf[(3, 3, -1, 1)].copy()
    aux = cf * d["sr"]
    add((1, 1, 1, -1), 1, aux); add((1, 1, -1, 1), 1, aux)
    mf[(2, 2, 1, -1)] = mf[(3, 3, 1, -1)].copy()
    mf[(2, 2, -1, 1)] = mf[(3, 3, -1, 1)].copy()
    aux = C(cf * I(d["sp"]), -cf * R(d["sp"]))
    add((2, 2, 1, -1), 1, aux); add((2, 2, -1, 1), -1, aux)

    # hpsi(iy, sa)[:, b] = sum_iz mf(iy, iz, sa, ns_b) * phi_iz(b)  (:1107-1127)
    ns = basis.ns
    hpsi = {}
    for sa in (1, -1):
        for iy in range(5):
            acc = np.zeros((n, basis.dqp), dtype=complex)
            for iz in range(5):
                ku = (iy, iz, sa, 1); kd = (iy, iz, sa, -1)
                if ku not in mf:
                    continue
                fb = np.where(ns[None, :] > 0, mf[ku][:, None], mf[kd][:, None])
                acc += fb * basis.P[iz]
            hpsi[(iy, sa)] = acc
    # h_ab = 2 sum_r phi_a hpsi  (:1132-1167)
    return _project(basis, hpsi, re_cols, db, isstart, num_up, 5)


def _project(basis, psi, cols, db, isstart, num_up, nphi):
    blocks = [None] * len(cols)
    for ix, iy in enumerate(cols):
        if iy < 0:
            continue
        ia, ib = isstart[ix], isstart[iy]
        nup, d, dc = num_up[ix], db[ix], db[iy]
        blk = np.zeros((d, dc), dtype=complex)
        for iz in range(nphi):
            ph = basis.P[iz]
            if nup > 0:
                blk[:nup] += 2.0 * ph[:, ia:ia + nup].T @ psi[(iz, 1)][:, ib:ib + dc]
            if d - nup > 0:
                blk[nup:] += 2.0 * ph[:, ia + nup:ia + d].T @ psi[(iz, -1)][:, ib:ib + dc]
        blocks[ix] = blk
    return blocks


def pairingfield(basis, ds, cp, cols, db, isstart, num_up):
    """Delta_ab from rho-breve and s-breve (:1175-1262)."""
    cpair, cspair = cp.cpair, cp.cspair
    rb, sbr, sbp, sbz = ds["rb"], ds["sbr"], ds["sbp"], ds["sbz"]
    aux_pp = cspair * (sbr - 1j * sbp)
    aux_mp = -cpair * rb - cspair * sbz
    aux_pm = cpair * rb - cspair * sbz
    aux_mm = cspair * (-sbr - 1j * sbp)
    up = basis.ns[None, :] > 0
    wf = basis.P[0]
    dpsi = {(0, 1): np.where(up, aux_pp[:, None], aux_pm[:, None]) * wf,
            (0, -1): np.where(up, aux_mp[:, None], aux_mm[:, None]) * wf}
    return _project(basis, dpsi, cols, db, isstart, num_up, 1)


def calc_hamiltonian(basis, cp, rho_pn, kp, rho_np, km, h_cols):
    """rho_* / k* are (re, im) BlockMatrix pairs; h_cols gives the output block
    structures: dict with keys 'h_pn', 'dp', 'h_np', 'dm'.  Returns complex blocks."""
    hfb = basis.hfb
    out = {}
    for tag, rho, kap, hk, dk in (("pn", rho_pn, kp, "h_pn", "dp"), ("np", rho_np, km, "h_np", "dm")):
        ds = density(basis, rho[0], rho[1], kap[0], kap[1], hfb.wdcori)
        out[hk] = meanfield(basis, ds, cp, h_cols[hk], hfb.db, hfb.isstart, hfb.num_spin_up)
        out[dk] = pairingfield(basis, ds, cp, h_cols[dk], hfb.db, hfb.isstart, hfb.num_spin_up)
    return out


# -----------------------------------------------------------------------------
# modified Broyden (pnfam_broyden.f90:117-216)
# -----------------------------------------------------------------------------
class Broyden:
    def __init__(self, n, m, alpha):
        self.n, self.m, self.alpha = n, m, alpha
        self.df = self.dv = None
        self.w0 = 0.01

    def step(self, vout, vin, it):
        """Returns (new vin, si, flag); vout/vin are float64 vectors."""
        M = self.m
        vout = vout - vin
        si = float(np.max(np.abs(vout))) if len(vout) else 0.0
        if M < 0:
            return vin + vout, si, "N"
        if M == 0 or it == 0:
            return vin + self.alpha * vout, si, "L"
        fdiv = lambda a, b: int(a / b)   # Fortran integer division truncates
        iter_used = min(it - 1, M)
        ipos = it - 1 - fdiv(it - 2, M) * M
        inext = it - fdiv(it - 1, M) * M
        if it == 1:
            self.w0 = 0.01
            self.df = np.zeros((self.n, M)); self.dv = np.zeros((self.n, M))
        else:
            p = ipos - 1
            self.df[:, p] = vout - self.df[:, p]
            self.dv[:, p] = vin - self.dv[:, p]
            normi = 1.0 / math.sqrt(np.linalg.norm(self.df[:, p]) ** 2)
            self.df[:, p] *= normi
            self.dv[:, p] *= normi
        beta = np.zeros((iter_used, iter_used))
        for i in range(iter_used):
            for j in range(i + 1, iter_used):
                beta[i, j] = float(np.dot(self.df[:, j], self.df[:, i]))
                beta[j, i] = beta[i, j]
            beta[i, i] = self.w0 * self.w0 + 1.0
        if iter_used:
            beta = np.linalg.inv(beta)
        work = np.array([float(np.dot(self.df[:, i], vout)) for i in range(iter_used)])
        curv = self.alpha * vout
        for i in range(iter_used):
            gamma = float(np.dot(beta[:, i], work))
            curv = curv - gamma * (self.dv[:, i] + self.alpha * self.df[:, i])
        self.df[:, inext - 1] = vout
        self.dv[:, inext - 1] = vin
        return vin + curv, si, "B"


# -----------------------------------------------------------------------------
# the solver (pnfam_solver.f90)
# -----------------------------------------------------------------------------
@dataclass
class OracleResult:
    re_str: np.ndarray          # [1 + nxterms]
    im_str: np.ndarray
    iter_conv: int              # -1 if not converged
    si: float
    history: list               # per iteration: (iter, flag, si, re_S, im_S)
    seconds: float
    X_re: np.ndarray = None
    Y_re: np.ndarray = None
    X_im: np.ndarray = None
    Y_im: np.ndarray = None
    vector: np.ndarray = None   # the final Broyden vector (what the restart storage keeps)


def _bm(m: BlockMatrix, sgn=1.0):
    return BlockMatrix(m.cols.copy(), [None if b is None else sgn * b for b in m.blocks])


class FAMOracle:
    """pnfam_solve for one (operator, omega) on a prepared HFB solution.

    ``occupations`` = (f_p, f_n), quasiparticle occupations [dqp] of the doubled
    basis, switches on the statistical FAM (finite temperature or EFA blocking,
    pnfam_solver.f90:248-254,425-458): the diagonal quadrants P (m11) and Q (m22)
    join X and Y, with Green's functions -1/(E1 - E2 -/+ w) and the occupation
    factors 1 - f1 - f2 (X, Y) and f2 - f1 (P, Q) applied after the Green's
    function; the Broyden vector is [Re X, Re Y, Im X, Im Y, Re P, Re Q, Im P, Im Q]
    (pnfam_broyden.f90:26-61)."""

    def __init__(self, hfb, couplings, F, G=(), quench=1.0, alpha_mix=float(np.float32(0.7)), occupations=None):
        # alpha_mix: pnfam_broyden.f90:20 sets 0.7 from a single-precision literal
        self.hfb, self.cp, self.quench, self.alpha = hfb, couplings, quench, alpha_mix
        nb, db = hfb.nb, hfb.db
        self.nb, self.db = nb, db
        self.bminus = F.beta_minus
        eye_cols = np.arange(nb)
        tr_cols = np.array([hfb.partner(i) for i in range(nb)])
        Un = BlockMatrix(eye_cols, list(hfb.Un)); Up = BlockMatrix(eye_cols, list(hfb.Up))
        Vn = BlockMatrix(tr_cols, list(hfb.Vn)); Vp = BlockMatrix(tr_cols, list(hfb.Vp))
        mk = lambda U, V: BBM(q={11: U, 12: V, 21: V, 22: U})
        self.Wn, self.Wp = mk(Un, Vn), mk(Up, Vp)
        self.W1, self.W2 = (self.Wp, self.Wn) if self.bminus else (self.Wn, self.Wp)
        self.E1, self.E2 = (hfb.Ep, hfb.En) if self.bminus else (hfb.En, hfb.Ep)
        self.stat = occupations is not None
        if self.stat:
            fp, fn = (np.asarray(x, dtype=np.float64) for x in occupations)
            self.f1, self.f2 = (fp, fn) if self.bminus else (fn, fp)
        self.quads = (12, 21, 11, 22) if self.stat else (12, 21)
        d = True if self.stat else None
        Fsp = BBM(q={11: F.mat, 12: None, 21: None, 22: None})
        qp = BBM(q={11: d, 12: True, 21: True, 22: d}, s={11: 1.0, 12: 1.0, 21: -1.0, 22: -1.0})
        self.Fqp = triprod_bbm("t", self.W1, "n", Fsp, "n", self.W2, qp, nb, db)
        self.Gqp = [triprod_bbm("t", self.W1, "n", BBM(q={11: g.mat, 12: None, 21: None, 22: None}),
                                "n", self.W2, qp, nb, db) for g in G]
        self.xlabels = [g.label for g in G]
        self.fmat = F.mat
        self.nxy = F.mat.nelem

    def _map2qp(self, quad, f):
        """f(i, j) on the blocks of Fqp quadrant ``quad`` (row/column states)."""
        m = self.Fqp.q[quad]
        st = self.hfb.isstart
        blocks = []
        for i, j in enumerate(m.cols):
            if j < 0:
                blocks.append(None); continue
            blocks.append(f(slice(st[i], st[i] + self.db[i]), slice(st[j], st[j] + self.db[j])))
        return blocks

    def _green(self, quad, ree, ime, c=1.0):
        """matrix_2qp(-1,+1,c,-1, ree, ime, E1, E2) on the block structure of quad."""
        return self._map2qp(quad, lambda r, k: -1.0 / (self.E1[r][:, None] + c * self.E2[k][None, :] + complex(ree, ime)))

    def _occupation(self, quad):
        """matrix_2qp(+1,-1,-1,+1, 1, 0) on X/Y and (+1,-1,+1,+1, 0, 0) on P/Q
        (pnfam_solver.f90:445-458)."""
        if quad in (12, 21):
            return self._map2qp(quad, lambda r, k: (-self.f1[r][:, None] - self.f2[k][None, :]) + 1.0)
        return self._map2qp(quad, lambda r, k: (-self.f1[r][:, None] + self.f2[k][None, :]) + 0.0)

    def solve(self, omega: complex, max_iter=300, eps=1e-7, broyden_m=50, keep_solution=False, x0=None,
              si0=1.0, s0=None):
        """x0: a start vector in the Broyden layout (the restart storage of pnfam_solve,
        pnfam_solver.f90:63-72), with the stored si0 and strengths s0 (complex, strength
        then cross terms) shown at iteration 0; the result's ``vector`` is the final one."""
        t0 = time.perf_counter()
        nb, db, hfb = self.nb, self.db, self.hfb
        quench = self.quench
        Fq = self.Fqp
        quads = self.quads
        # Green's functions X (12), Y (21) and, statistical, P (11), Q (22); complex
        Gf = {12: self._green(12, -omega.real, -omega.imag), 21: self._green(21, omega.real, omega.imag)}
        Tq = {}
        if self.stat:
            Gf[11] = self._green(11, -omega.real, -omega.imag, -1.0)
            Gf[22] = self._green(22, omega.real, omega.imag, -1.0)
            Tq = {q: self._occupation(q) for q in quads}
        cols = {q: Fq.q[q].cols for q in quads}
        colsX, colsY = cols[12], cols[21]
        nx = Fq.q[12].nelem
        R = {q: [None if c < 0 else np.zeros((db[i], db[c]), dtype=complex) for i, c in enumerate(cols[q])]
             for q in quads}
        if abs(quench) < 1e-10:
            broyden_m = -1
        bro = Broyden(len(quads) * 2 * nx, broyden_m, self.alpha)
        flat = lambda blks: np.concatenate([b.reshape(-1, order="F") for b in blks if b is not None])
        # Broyden layout: (quadrant pair, Re|Im) groups of pnfam_broyden.f90:47-60
        groups = [(12, 21)] + ([(11, 22)] if self.stat else [])

        def pack(Rd):
            parts = []
            for qa, qb in groups:
                fa, fb = flat(Rd[qa]), flat(Rd[qb])
                parts += [fa.real, fb.real, fa.imag, fb.imag]
            return np.concatenate(parts)

        def unpack(v):
            out = {q: [None if b is None else np.zeros(b.shape, dtype=complex) for b in R[q]] for q in quads}
            base = 0
            for qa, qb in groups:
                for q, off_re, off_im in ((qa, base, base + 2 * nx), (qb, base + nx, base + 3 * nx)):
                    p = 0
                    for b in out[q]:
                        if b is None:
                            continue
                        n = b.size
                        b[...] = (v[off_re + p:off_re + p + n] + 1j * v[off_im + p:off_im + p + n]).reshape(b.shape, order="F")
                        p += n
                base += 4 * nx
            return out

        vin = pack(R)
        si = 1.0
        flag = "N"
        nxt = len(self.Gqp)
        re_str = np.zeros(1 + nxt); im_str = np.zeros(1 + nxt)
        if x0 is not None:
            vin = np.array(x0, dtype=np.float64)
            R = unpack(vin)
            si = float(si0)
            if s0 is not None:
                re_str[:] = np.real(s0); im_str[:] = np.imag(s0)
        history = []
        iter_conv = -1
        # SP-basis structures of the H/rho quadrants
        h_cols = {"h_pn": self.fmat.cols, "h_np": self.fmat.cols, "dp": colsX, "dm": colsY}
        basis = _Basis(hfb)

        def contract(op, Rd):
            # contract_bbm (pnfam_type_bbm.f90:393-421): quadrants 11, 12, 21, 22 in order
            sr = si_ = 0.0
            for q in (11, 12, 21, 22):
                if q in Rd:
                    f = op.q[q].flatten(); x = flat(Rd[q])
                    sr = sr + float(np.dot(f, x.real)); si_ = si_ + float(np.dot(f, x.imag))
            return -sr / PI, -si_ / PI

        for it in range(0, max_iter + 1):
            history.append((it, flag, si, re_str[0], im_str[0], re_str[1:].copy(), im_str[1:].copy()))
            if si < eps:
                iter_conv = it
                break
            if it == max_iter:
                iter_conv = -1
                break
            if abs(quench) < 1e-10:
                H = {q: [None if b is None else np.zeros_like(b) for b in R[q]] for q in quads}
            else:
                H = self._residual(R, cols, h_cols, basis)
                H = {q: [None if b is None else quench * b for b in H[q]] for q in quads}
            Ro = {}
            for q in quads:
                Hq = [None if b is None else b + Fq.q[q].blocks[i] for i, b in enumerate(H[q])]
                Ro[q] = [None if b is None else Gf[q][i] * b for i, b in enumerate(Hq)]
                if self.stat:
                    Ro[q] = [None if b is None else Tq[q][i] * b for i, b in enumerate(Ro[q])]
            vout = pack(Ro)
            vin, si, flag = bro.step(vout, vin, it)
            R = unpack(vin)
            re_str[0], im_str[0] = contract(Fq, R)
            for k, g in enumerate(self.Gqp):
                re_str[1 + k], im_str[1 + k] = contract(g, R)
        res = OracleResult(re_str.copy(), im_str.copy(), iter_conv, si, history, time.perf_counter() - t0)
        res.vector = vin.copy()
        if keep_solution:
            fx = flat(R[12]); fy = flat(R[21])
            res.X_re, res.X_im, res.Y_re, res.Y_im = fx.real.copy(), fx.imag.copy(), fy.real.copy(), fy.imag.copy()
        return res

    def _residual(self, R, cols, h_cols, basis):
        """dH_qp (stored quadrants, complex) from dR_qp, via the SP basis."""
        nb, db = self.nb, self.db
        mkq = lambda q, part: BlockMatrix(cols[q], [None if b is None else getattr(b, part).copy() for b in R[q]])
        dRq = {}
        for part, im in (("real", False), ("imag", True)):
            dRq[part] = BBM(q={q: (mkq(q, part) if q in R else None) for q in (11, 12, 21, 22)},
                            s={11: 1.0, 12: 1.0, 21: -1.0, 22: -1.0}, imag=im)
        sp_re = BBM(q={11: True, 12: True, 21: True, 22: True}, s={11: 1.0, 12: -1.0, 21: 1.0, 22: -1.0},
                    t={11: "n", 12: "t", 21: "t", 22: "t"})
        sp_im = BBM(q={11: True, 12: True, 21: True, 22: True}, s={11: 1.0, 12: -1.0, 21: -1.0, 22: -1.0},
                    t={11: "n", 12: "t", 21: "t", 22: "t"}, imag=True)
        dRsp_re = triprod_bbm("n", self.W1, "n", dRq["real"], "t", self.W2, sp_re, nb, db)
        dRsp_im = triprod_bbm("n", self.W1, "n", dRq["imag"], "t", self.W2, sp_im, nb, db)
        out = calc_hamiltonian(basis, self.cp,
                               (dRsp_re.q[11], dRsp_im.q[11]), (dRsp_re.q[12], dRsp_im.q[12]),
                               (dRsp_re.q[22], dRsp_im.q[22]), (dRsp_re.q[21], dRsp_im.q[21]), h_cols)
        mk = lambda cols, blks, part: BlockMatrix(np.asarray(cols), [None if b is None else getattr(b, part).copy() for b in blks])
        Hre = BBM(q={11: mk(h_cols["h_pn"], out["h_pn"], "real"), 12: mk(h_cols["dp"], out["dp"], "real"),
                     21: mk(h_cols["dm"], out["dm"], "real"), 22: mk(h_cols["h_np"], out["h_np"], "real")},
                  s={11: 1.0, 12: 1.0, 21: -1.0, 22: -1.0}, t={11: "n", 12: "n", 21: "n", 22: "t"})
        Him = BBM(q={11: mk(h_cols["h_pn"], out["h_pn"], "imag"), 12: mk(h_cols["dp"], out["dp"], "imag"),
                     21: mk(h_cols["dm"], out["dm"], "imag"), 22: mk(h_cols["h_np"], out["h_np"], "imag")},
                  s={11: 1.0, 12: 1.0, 21: 1.0, 22: -1.0}, t={11: "n", 12: "n", 21: "n", 22: "t"}, imag=True)
        d = True if self.stat else None
        qp_re = BBM(q={11: d, 12: True, 21: True, 22: d}, s={11: 1.0, 12: 1.0, 21: -1.0, 22: -1.0})
        qp_im = BBM(q={11: d, 12: True, 21: True, 22: d}, s={11: 1.0, 12: 1.0, 21: -1.0, 22: -1.0}, imag=True)
        Hq_re = triprod_bbm("t", self.W1, "n", Hre, "n", self.W2, qp_re, nb, db)
        Hq_im = triprod_bbm("t", self.W1, "n", Him, "n", self.W2, qp_im, nb, db)
        return {q: [None if b is None else b + 1j * Hq_im.q[q].blocks[i] for i, b in enumerate(Hq_re.q[q].blocks)]
                for q in self.quads}
