"""One-body charge-changing external fields F_sp = <i|O_K|j>.

Follows pnfam_extfield.f90: ``init_external_field`` (:37-108), the operator
matrix elements of ``ext_field_operator`` (:110-627), the FAM block map
``init_fam_mapping`` (:763-841) and the cross-term operators of
``setup_crossterms`` (:883-949).  Two-body-current modes and the I-function
variants RI/RS0I/RS1I enter as a mesh weight on the bra wave function
(``extfield_2bc.operator_weight``); the GT two-body-current composition is in
``pnfam_setup``.

Cross terms follow the operator sets of the reference runs that produced the
recorded strength functions: rank-0 odd operators (RS0, PS0) get
{RS0, PS0}; R, P and RS1 get {R, RS1, P}.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .blockmatrix import BlockMatrix
from .extfield_2bc import LECs, operator_weight, gt_density_factor

EVEN_OPS = ("F", "GT")
ODD_OPS = ("RS0", "RS1", "RS2", "R", "P", "PS0", "RI", "RS0I", "RS1I")
RANK = {"F": 0, "RS0": 0, "PS0": 0, "RS0I": 0, "GT": 1, "R": 1, "P": 1, "RS1": 1, "RI": 1, "RS1I": 1, "RS2": 2}
# the I-function variants share the matrix elements of their base operator
_BASE = {"RI": "R", "RS0I": "RS0", "RS1I": "RS1"}


class ExtFieldError(RuntimeError):
    pass


@dataclass
class ExternalField:
    label: str
    k: int
    beta_minus: bool
    parity_even: bool
    rank: int
    mat: BlockMatrix = None


def init_fam_mapping(hfb, k: int, parity_even: bool) -> np.ndarray:
    """Block column of F for each block row: 2*Omega_1 - 2*Omega_2 = 2K and
    the parity rule; the first matching block is taken (extfield.f90:763-841)."""
    nb = hfb.nb
    st = hfb.isstart
    two_omega = 2 * hfb.nl[st] + hfb.ns[st]
    par = hfb.npar[st]
    pty_blocks = all(np.all(hfb.npar[st[i]:st[i] + hfb.db[i]] == par[i]) for i in range(nb))
    cols = np.full(nb, -1, dtype=np.int64)
    for i1 in range(nb):
        for i2 in range(nb):
            if two_omega[i1] - two_omega[i2] == 2 * k and \
                    (not pty_blocks or ((par[i1] == par[i2]) == parity_even)):
                cols[i1] = i2
                break
    if not np.any(cols >= 0):
        raise ExtFieldError("The K and parity are outside the model space.")
    return cols


def _element_block(label, K, hfb, i_rows, i_cols, weight=None):
    """Matrix elements of block (rows, cols), vectorised over the pair grid;
    ``weight`` (a mesh function) multiplies every integrand."""
    label = _BASE.get(label, label)
    wf1 = hfb.wf[i_rows]; wf2 = hfb.wf[i_cols]
    if weight is not None:
        wf1 = wf1 * weight[None, :]
    dr2 = hfb.wfdr[i_cols]; dz2 = hfb.wfdz[i_cols]
    l1 = hfb.nl[i_rows][:, None]; l2 = hfb.nl[i_cols][None, :]
    s1 = hfb.ns[i_rows][:, None]; s2 = hfb.ns[i_cols][None, :]
    y, z = hfb.y, hfb.z
    r = 1.0 / y
    dot = lambda a, b: a @ b.T
    ov = lambda: dot(wf1, wf2)
    zz = lambda: dot(wf1, wf2 * z)
    rr = lambda: dot(wf1, wf2 * r)
    same = (l1 == l2) & (s1 == s2)
    out = np.zeros((len(i_rows), len(i_cols)))
    sq2, sq3 = np.sqrt(2.0), np.sqrt(3.0)
    if label == "F":
        out = np.where(same, ov(), 0.0)
    elif label == "GT":
        if K == 0:
            out = np.where(same, s1 * ov(), 0.0)
        else:
            out = np.where((l1 == l2) & (s1 == s2 + 2 * K), -K * sq2 * ov(), 0.0)
    elif label == "R":
        if K == 0:
            out = np.where(same, zz(), 0.0)
        else:
            out = np.where((l1 == l2 + K) & (s1 == s2), -K / sq2 * rr(), 0.0)
    elif label == "P":
        if K == 0:
            out = np.where(same, -dot(wf1, dz2), 0.0)
        else:
            m = K / sq2 * (dot(wf1, dr2) - K * l2 * dot(wf1, wf2 * y))
            out = np.where((l1 == l2 + K) & (s1 == s2), m, 0.0)
    elif label == "RS0":
        c1 = (l1 == l2 + 1) & (s1 == s2 - 2)
        c2 = (l1 == l2 - 1) & (s1 == s2 + 2)
        out = np.where(same, -s1 * zz(), np.where(c1 | c2, -rr(), 0.0))
    elif label == "RS1":
        if K == 0:
            c1 = (l1 == l2 - 1) & (s1 == s2 + 2)
            c2 = (l1 == l2 + 1) & (s1 == s2 - 2)
            out = np.where(c1, np.sqrt(1.5) * rr(), np.where(c2, -np.sqrt(1.5) * rr(), 0.0))
        else:
            c1 = (l1 == l2) & (s1 == s2 + 2 * K)
            c2 = (l1 == l2 + K) & (s1 == s2)
            out = np.where(c1, sq3 * zz(), np.where(c2, -s1 * sq3 / 2.0 * rr(), 0.0))
    elif label == "RS2":
        if K == 0:
            c1 = (l1 == l2 + 1) & (s1 == s2 - 2)
            c2 = (l1 == l2 - 1) & (s1 == s2 + 2)
            out = np.where(same, s1 * sq2 * zz(), np.where(c1 | c2, -1.0 / sq2 * rr(), 0.0))
        elif abs(K) == 1:
            c1 = (l1 == l2) & (s1 == s2 + 2 * K)
            c2 = (l1 == l2 + K) & (s1 == s2)
            out = np.where(c1, -K * sq3 * zz(), np.where(c2, -K * s1 * sq3 / 2.0 * rr(), 0.0))
        else:
            c1 = (l1 == l2 + K // 2) & (s1 == s2 + K)
            out = np.where(c1, sq3 * rr(), 0.0)
    elif label == "PS0":
        c1 = (l1 == l2 - 1) & (s1 == s2 + 2)
        c2 = (l1 == l2 + 1) & (s1 == s2 - 2)
        a = dot(wf1, dr2)
        b = l2 * dot(wf1, wf2 * y)
        out = np.where(same, -s1 * dot(wf1, dz2), np.where(c1, -a - b, np.where(c2, -a + b, 0.0)))
    else:
        raise ExtFieldError(f'Unknown operator "{label}" in extfield.')
    return out


def init_external_field(hfb, beta_type: str, label: str, k: int, use_2bc: tuple = (0,) * 6,
                        lecs: LECs = None) -> ExternalField:
    """The operator's F_sp; ``use_2bc`` (the digits of two_body_current_mode) and
    ``lecs`` select the two-body-current weights of P, PS0, the spin-dipole
    operators and the GT contact pass (pnfam_extfield.f90:158-198)."""
    label = label.strip().upper()
    if beta_type not in ("-", "+"):
        raise ExtFieldError(f"Unknown operator \"beta_type={beta_type}\" in extfield.")
    if label in EVEN_OPS:
        even = True
    elif label in ODD_OPS:
        even = False
    else:
        raise ExtFieldError(f'Unknown operator "{label}" in extfield.')
    rank = RANK[label]
    if abs(k) > rank:
        raise ExtFieldError(f'K out of range for operator "{label}" in extfield. Expected |K| <= {rank}')
    cols = init_fam_mapping(hfb, k, even)
    use_2bc = tuple(use_2bc)
    if any(use_2bc) and lecs is None:
        raise ExtFieldError("two-body-current weights need the LECs")
    if label == "GT":
        weight = gt_density_factor(hfb, use_2bc, lecs) if use_2bc[1] != 0 and use_2bc[3] != 0 else None
    else:
        weight = operator_weight(hfb, label, use_2bc, lecs)
    mat = BlockMatrix.empty(cols, hfb.db)
    for i1, i2 in enumerate(cols):
        if i2 < 0:
            continue
        r = np.arange(hfb.isstart[i1], hfb.isstart[i1] + hfb.db[i1])
        c = np.arange(hfb.isstart[i2], hfb.isstart[i2] + hfb.db[i2])
        if len(r) and len(c):
            mat.blocks[i1] = _element_block(label, k, hfb, r, c, weight)
    return ExternalField(label, k, beta_type == "-", even, rank, mat)


def number_crossterms(op: ExternalField) -> int:
    if op.parity_even:
        return 0
    if op.label in ("R", "P", "RS1", "RI", "RS1I"):
        return 3
    if op.label in ("RS0", "PS0", "RS0I"):
        return 2
    return 0


def setup_crossterms(hfb, op: ExternalField, use_2bc: tuple = (0,) * 6, lecs: LECs = None) -> list:
    """Cross-term operators; all but R carry the two-body-current weights
    (pnfam_extfield.f90:882-949)."""
    n = number_crossterms(op)
    beta = "-" if op.beta_minus else "+"
    if n == 0:
        return []
    labels = ("RS0", "PS0") if n == 2 else ("R", "RS1", "P")
    out = []
    for lab in labels:
        u = (0,) * 6 if lab == "R" else use_2bc
        g = init_external_field(hfb, beta, lab, op.k, u, lecs)
        g.label = f"{op.label}x{lab}"
        out.append(g)
    return out
