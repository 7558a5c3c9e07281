"""Two-body-current (2BC) corrections to the charge-changing external field.

The reference folds the axial two-body current into the one-body operators
(pnfam_solver.f90:556-654 ``setup_extfield``, pnfam_extfield.f90):

* the mode ``two_body_current_mode`` is six decimal digits (``set_use_2bc``,
  pnfam_extfield.f90:683-722): [1+2 body | 2 body only], [GT form: full FAM,
  SNM+LDA, ASNM+LDA, DME exchange, DME exchange + FAM direct], [Gamma, Delta],
  [GT current on; >= 2 also corrects the rank-L spin-dipole operators, 3 with
  asymmetric matter], [P current: 2BC or DME], [PS0 current: 2BC or DME];
* GT: F = -sigma tau (the one-body part, when 1+2 body) + sigma tau f(r), with
  f(r) the contact term 2 caux cd rho(r) plus the nuclear-matter (LDA) or DME
  exchange function; the full-FAM forms add the finite-range (Yukawa) field
  contracted once with the ground-state densities, which the reference caches
  in ``<fam_output_filename>.tbc`` with the LECs stripped (pnfam_storage.f90:
  488-727) and recomputes from two-body matrix elements when the file is
  absent (pnfam_extfield_2bc.f90:26, O(N^10) in the oscillator shells); here
  that contraction runs on the GPU (``finite_range.gamma_pieces``);
* P, PS0 and the spin-dipole operators RS0/RS1/RS2 (and their I-function
  variants) multiply the one-body integrand by 1 + c(r) (or c(r) alone for
  2 body only), c(r) from nuclear matter at a fixed pair momentum or from the
  DME (pnfam_extfield.f90:1152-1719).

Every function here but the finite-range contraction is a mesh function of the
ground-state densities rho, tau and Laplacian rho (``HFBSolution``) and runs
once per set-up, on the host.
"""
from __future__ import annotations

import os
import struct
from dataclasses import dataclass

import numpy as np

# pnfam_constants.f90:36-67
PI = 3.141592653589793238462643
HBARC = 197.3269718     # MeV fm
MN = 939.0              # MeV
FPI = 92.4              # MeV
MPI = 138.04            # MeV
GA = 1.27

# pair momentum of the nuclear-matter P and PS0 corrections: the reference
# evaluates sqrt(1.2)*1.30465/2.0 in default (single) precision
# (pnfam_extfield.f90:1332,1363)
P_PAIR = float(np.float32(np.float32(np.sqrt(np.float32(1.2))) * np.float32(1.30465)) / np.float32(2.0))


class TwoBodyCurrentError(RuntimeError):
    pass


def parse_mode(mode: int) -> tuple:
    """The six digits of two_body_current_mode, most significant first
    (``set_use_2bc``, pnfam_extfield.f90:683-722); (0,)*6 for mode 0."""
    mode = int(mode)
    if mode == 0:
        return (0, 0, 0, 0, 0, 0)
    d = tuple(mode // 10 ** p - 10 * (mode // 10 ** (p + 1)) for p in (5, 4, 3, 2, 1, 0))
    i1, i2, i3 = d[0], d[1], d[2]
    if not (1 <= i1 <= 2) or not (1 <= i2 <= 5) or not (1 <= i3 <= 3) or (i1 != 1 and i3 != 1):
        raise TwoBodyCurrentError("Invalid value supplied for two_body_current_mode.")
    if i3 != 1:
        raise TwoBodyCurrentError("This two_body_current_mode is not yet operational.")
    if d[4] > 2 or d[5] > 2:
        raise TwoBodyCurrentError("Invalid value supplied for two_body_current_mode.")
    return d


@dataclass
class LECs:
    """Low-energy constants and derived factors (``init_extfield_2bc_type``,
    pnfam_type_extfield_2bc.f90:47-84); c3, c4 in 1/GeV as given.

    The last four fields are constants that the reference hard-codes in its
    correction functions and that differ between its revisions; the defaults
    are the current source's.  Earlier revisions (the ones that recorded some
    of the reference's two-body-current test runs) used the pair momentum
    sqrt(1.2)*1.361/2 fm^-1 or fixed values of 108-300 MeV, the opposite sign
    of the P correction, the constant-density DME vector current (only the
    U_1^0 and U_2^2 terms) and the earlier DME axial charge (U_1^-1, U_1^1)."""
    c3: float
    c4: float
    cd: float
    d1: float
    d2: float
    caux: float
    use_p: bool
    pair_momentum: float = P_PAIR          # fm^-1, nuclear-matter P and PS0 corrections
    p_sign: float = 1.0                    # sign of the nuclear-matter P correction
    dme_vector_form: str = "full"          # "full" | "constant_density"
    dme_axial_form: str = "current"        # "current" | "earlier"

    @staticmethod
    def from_namelist(lecs, use_p=False, **revision) -> "LECs":
        c3, c4, c = (float(x) for x in lecs)
        cd = c * (-0.25)
        return LECs(c3, c4, cd, cd * 0.5, cd * 0.25, HBARC ** 3 / (2.0 * MN * FPI * FPI), bool(use_p), **revision)


# ----------------------------------------------------------------------------
# nuclear matter + LDA (pnfam_extfield.f90:976-1130)
# ----------------------------------------------------------------------------
def kf_snm(rho):
    return (1.5 * PI * PI * rho) ** (1.0 / 3.0)


def kf_asnm(rho):
    return (3.0 * PI * PI * rho) ** (1.0 / 3.0)


def nmlda_i0(kf):
    """I(kf) at zero momentum transfer (Klos 2013 Eq. 14)."""
    m = MPI / HBARC
    with np.errstate(divide="ignore", invalid="ignore"):
        return 1.0 - 3.0 * m * m / (kf * kf) + 3.0 * m * m * m / (kf * kf * kf) * np.arctan(kf / m)


def nmlda_da1(rhon, rhop, snm: bool, lec: LECs):
    """Density-dependent coefficient of sigma tau from the effective 2BC at
    zero momentum transfer (``tbc_nmlda_da1``, :1067-1130)."""
    caux0 = HBARC ** 3 / (MN * FPI * FPI)
    caux3 = -1.0 / 3.0 * lec.c3
    if lec.use_p:
        caux3 = caux3 + 1.0 / 12.0
    caux4 = 1.0 / 3.0 * (lec.c4 + 0.25)
    parts = [(rhop + rhon, kf_snm(rhop + rhon))] if snm else [(rhon, kf_asnm(rhon)), (rhop, kf_asnm(rhop))]
    da1 = np.zeros_like(rhon)
    for rho, kf in parts:
        i0 = nmlda_i0(kf)
        da1 = da1 + caux0 * rho * (caux4 * (3.0 * i0 - i0) + caux3 * i0)
    return da1


def rsl_correction(hfb, snm: bool, lec: LECs):
    """2BC correction of the rank-L spin-dipole operators (``forbidden_2bc_rsL``,
    :1152-1193)."""
    ca = 2 * lec.caux
    ch = 1.0 / 3.0 * (2 * lec.c4 - lec.c3 + 0.5)
    if snm:
        rho = hfb.rho_n + hfb.rho_p
        return ca * rho * (lec.cd + ch * nmlda_i0(kf_snm(rho)))
    rn, rp = hfb.rho_n, hfb.rho_p
    return ca * (rn + rp) * lec.cd + ca * ch * rn * nmlda_i0(kf_asnm(rn)) + ca * ch * rp * nmlda_i0(kf_asnm(rp))


# ----------------------------------------------------------------------------
# DME functions U_l^k(kf) (:1195-1546)
# ----------------------------------------------------------------------------
def _m():
    return MPI / HBARC


def dme_u00(kf):
    m = _m()
    with np.errstate(divide="ignore", invalid="ignore"):
        u = 1.5 / (kf * kf) * (1 - m / kf * np.arctan(2 * kf / m) + m * m / (4.0 * kf * kf) * np.log(1 + 4 * kf * kf / (m * m)))
    return np.where(kf < np.float32(0.001), 1.0 / (m * m), u)


def dme_u02(kf):
    m = _m()
    with np.errstate(divide="ignore", invalid="ignore"):
        u = 0.75 / (kf * kf) * (np.log(1.0 + 4.0 * kf * kf / (m * m)) - 4.0 * kf * kf / (4.0 * kf * kf + m * m))
    return np.where(kf < np.float32(0.00005), 0.0, u)


def dme_u02_kf2(kf):
    m = _m()
    with np.errstate(divide="ignore", invalid="ignore"):
        u = 0.75 / (kf * kf * kf * kf) * (np.log(1.0 + 4.0 * kf * kf / (m * m)) - 4.0 * kf * kf / (4.0 * kf * kf + m * m))
    return np.where(kf < np.float32(0.001), 6.0 / m ** 4, u)


def dme_u10(kf):
    m = _m()
    with np.errstate(divide="ignore", invalid="ignore"):
        u = 1.5 / (kf * kf) * (1.0 - m * m / (4.0 * kf * kf) * np.log(1.0 + 4.0 * kf * kf / (m * m)))
    return np.where(kf < np.float32(0.001), 3.0 / (m * m), u)


def dme_u11(kf):
    m = _m()
    with np.errstate(divide="ignore", invalid="ignore"):
        return 1.5 / (kf * kf) * (np.arctan(2.0 * kf / m) - 2.0 * kf * m / (4.0 * kf * kf + m * m))


def dme_u11_kf2(kf):
    m = _m()
    with np.errstate(divide="ignore", invalid="ignore"):
        u = 1.5 / (kf * kf * kf * kf) * (np.arctan(2.0 * kf / m) - 2.0 * kf * m / (4.0 * kf * kf + m * m))
        return np.where(kf < np.float32(0.001), 8.0 / (m * m * m * kf), u)


def dme_u1_1(kf):
    m = _m()
    with np.errstate(divide="ignore", invalid="ignore"):
        u = m / 2.0 * (1.0 + (2.0 * kf / m - 1.5 * m / kf) * np.arctan(2.0 * kf / m)
                       + m * m / (2.0 * kf * kf) * np.log(1.0 + 4.0 * kf * kf / (m * m)))
    return np.where(kf < np.float32(0.0001), 0.0, u)


def dme_u12(kf):
    m = _m()
    a = 4.0 * kf * kf
    with np.errstate(divide="ignore", invalid="ignore"):
        u = 3.0 / (a + m * m) * ((a - m * m) / (a + m * m) + (1.0 + m * m / a) * np.log(1.0 + a / (m * m)))
    return np.where(kf < np.float32(0.0001), 0.0, u)


def dme_u12_kf2(kf):
    m = _m()
    a = 4.0 * kf * kf
    with np.errstate(divide="ignore", invalid="ignore"):
        u = 3.0 / (kf * kf * (a + m * m)) * ((a - m * m) / (a + m * m) + (1.0 + m * m / a) * np.log(1.0 + a / (m * m)))
    return np.where(kf < np.float32(0.001), 30.0 / m ** 4 + (-224.0 / m ** 6) * kf ** 2, u)


def dme_u22(kf):
    m = _m()
    with np.errstate(divide="ignore", invalid="ignore"):
        return -1.0 * kf / (3.0 * PI * PI) * (1.0 + 8.0 * kf * kf / (4.0 * kf * kf + m * m)
                                             - m * m / (4.0 * kf * kf) * np.log(1.0 + 4.0 * kf * kf / (m * m)))


def dme_u24(kf):
    m = _m()
    return kf * kf * (80.0 * kf ** 4 + 40.0 * kf * kf * m * m - 3.0 * m ** 4) / (4.0 * kf * kf + m * m) ** 3 \
        + 0.75 * np.log(1.0 + 4.0 * kf * kf / (m * m))


def dme_u24_kf4(kf):
    m = _m()
    with np.errstate(divide="ignore", invalid="ignore"):
        u = 1.0 / (6.0 * kf * kf * kf * kf) * dme_u24(kf)
    return np.where(kf < np.float32(0.001), 35.0 / (3.0 * m ** 4) + (-112.0 / m ** 6) * kf ** 2, u)


def dme_exchange(hfb, lec: LECs):
    """DME exchange function of the GT current (``dme_exc``, :1271-1303)."""
    m = _m()
    ca = 2 * lec.caux
    ch = 1.0 / 3.0 * (2 * lec.c4 - lec.c3 + 0.5)
    cc = -lec.d1 + 2 * lec.d2
    rho = hfb.rho_n + hfb.rho_p
    d2r0 = hfb.d2rho_n + hfb.d2rho_p
    tau0 = hfb.tau_n + hfb.tau_p
    kf = kf_snm(rho)
    u00, u02, u02_kf2 = dme_u00(kf), dme_u02(kf), dme_u02_kf2(kf)
    rf1 = ca * (ch * (1 - m * m * u00 - m * m * u02 * 0.1) + cc) * rho
    rf2 = ca * ch * m * m / 6 * u02_kf2 * (0.25 * d2r0 - tau0)
    return rf1 - rf2


def _log_ratio(kf, P):
    m = _m()
    return np.log((m * m + (P + kf) ** 2) / (m * m + (P - kf) ** 2))


def p_correction(hfb, lec: LECs):
    """Nuclear-matter 2BC correction of the P operator at the pair momentum
    (``forbidden_2bc_P``, :1323-1352)."""
    m = _m()
    P = lec.pair_momentum
    kf = kf_snm(hfb.rho_n + hfb.rho_p)
    iout = 1.0 / P ** 3 * (P * m * m * kf - 0.25 * m * m * (m * m + P * P + kf * kf) * _log_ratio(kf, P))
    return lec.p_sign * (GA * GA * HBARC * MN / (4 * PI * PI * FPI * FPI) * iout)


def ps0_correction(hfb, lec: LECs):
    """Nuclear-matter 2BC correction of the axial charge PS0 (``forbidden_2bc_PS0``,
    :1354-1377)."""
    m = _m()
    P = lec.pair_momentum
    kf = kf_snm(hfb.rho_n + hfb.rho_p)
    iout = 1.0 / P ** 3 * (-P * kf * (kf * kf + m * m + P * P)
                           + 0.25 * (((m * m + P * P) ** 2 + kf * kf * (kf * kf - 2 * P * P + 2 * m * m)) * _log_ratio(kf, P)))
    return -HBARC * MN / (8 * PI * PI * FPI * FPI) * iout


def dme_axial(hfb, lec: LECs):
    """DME correction of the axial charge (``dme_axial_2``, :1572-1618; the
    earlier form is kept in the reference as comments, :1549-1570)."""
    rho = hfb.rho_n + hfb.rho_p
    d2r0 = hfb.d2rho_n + hfb.d2rho_p
    tau0 = hfb.tau_n + hfb.tau_p
    kf = kf_snm(rho)
    if lec.dme_axial_form == "earlier":
        return HBARC * MN / (6.0 * FPI * FPI) * (dme_u1_1(kf) * (2.0 / (3.0 * PI * PI)) + 0.6 * dme_u11(kf) * rho
                                                 + dme_u11_kf2(kf) * (0.25 * d2r0 - tau0))
    u10, u12, u12_kf2 = dme_u10(kf), dme_u12(kf), dme_u12_kf2(kf)
    return HBARC * MN / (6.0 * FPI * FPI) * ((u10 + 0.1 * u12) * rho + u12_kf2 / 6.0 * (0.25 * d2r0 - tau0))


def dme_vector(hfb, lec: LECs):
    """DME correction of the vector current P (``dme_vector``, :1621-1678; the
    constant-density form keeps its U_1^0 and U_2^2 terms, :1668)."""
    rho = hfb.rho_n + hfb.rho_p
    d2r0 = hfb.d2rho_n + hfb.d2rho_p
    tau0 = hfb.tau_n + hfb.tau_p
    kf = kf_snm(rho)
    if lec.dme_vector_form == "constant_density":
        return GA * GA * MN * HBARC / (4.0 * FPI * FPI) * (dme_u10(kf) * rho + dme_u22(kf))
    u10, u12, u22, u24 = dme_u10(kf), dme_u12(kf), dme_u22(kf), dme_u24(kf)
    u12_kf2, u24_kf4 = dme_u12_kf2(kf), dme_u24_kf4(kf)
    return GA * GA * MN * HBARC / (4.0 * FPI * FPI) * ((u10 + 0.1 * u12) * rho + u22 - u24 * kf / (15.0 * PI * PI)
                                                       + (u12_kf2 / 6.0 - u24_kf4) * (0.25 * d2r0 - tau0))


def i1111(hfb):
    """I(1,1,1,1; r) of a uniformly charged sphere of radius 1.2 A^(1/3) fm
    (``calculate_I1111_r``, :1683-1719)."""
    A = int(hfb.Z) + int(hfb.N)
    R = 1.2 * float(A) ** (1.0 / 3.0)
    radius = ((1.0 / hfb.y) ** 2 + hfb.z ** 2) ** 0.5
    with np.errstate(divide="ignore"):
        out = 1.5 * (R / radius - 0.2 * R ** 3 / radius ** 3)
    return np.where(radius <= R, 1.5 * (1.0 - 0.2 * radius ** 2 / R ** 2), out)


# ----------------------------------------------------------------------------
# weights of the one-body integrands
# ----------------------------------------------------------------------------
def gt_density_factor(hfb, use2bc: tuple, lec: LECs):
    """rho_fac of the GT contact pass (pnfam_extfield.f90:158-181)."""
    rho_fac = (lec.caux * 2.0 * lec.cd) * (hfb.rho_n + hfb.rho_p)
    form = use2bc[1]
    if form == 2:
        rho_fac = rho_fac + nmlda_da1(hfb.rho_n, hfb.rho_p, True, lec)
    elif form == 3:
        rho_fac = rho_fac + nmlda_da1(hfb.rho_n, hfb.rho_p, False, lec)
    elif form in (4, 5):
        rho_fac = rho_fac + dme_exchange(hfb, lec)
    return rho_fac


def operator_weight(hfb, label: str, use2bc: tuple, lec: LECs):
    """Mesh weight that multiplies the one-body integrand of ``label`` under the
    given 2BC digits (None: the plain one-body operator)."""
    i1, _, _, i4, i5, i6 = use2bc
    w = None
    if label in ("RI", "RS0I", "RS1I"):
        w = i1111(hfb)
    if label in ("RS0", "RS1", "RS2", "RS0I", "RS1I") and i4 >= 2:
        c = 1.0 - rsl_correction(hfb, i4 != 3, lec)
        w = c if w is None else w * c
    if label == "P" and i1 != 0 and i5 != 0:
        c = p_correction(hfb, lec) if i5 == 1 else dme_vector(hfb, lec)
        w = 1.0 + c if i1 == 1 else c
    if label == "PS0" and i1 != 0 and i6 != 0:
        c = ps0_correction(hfb, lec) if i6 == 1 else dme_axial(hfb, lec)
        w = 1.0 + c if i1 == 1 else c
    return w


# ----------------------------------------------------------------------------
# .tbc file: the finite-range GT field with the LECs stripped
# ----------------------------------------------------------------------------
TBC_VERSION = 1


def _records(blob: bytes):
    off, n = 0, len(blob)
    while off < n:
        if off + 4 > n:
            raise TwoBodyCurrentError("truncated record marker")
        (ln,) = struct.unpack_from("<i", blob, off)
        end = off + 4 + ln
        if ln < 0 or end + 4 > n or struct.unpack_from("<i", blob, end)[0] != ln:
            raise TwoBodyCurrentError("corrupted record")
        yield blob[off + 4:end]
        off = end + 4


@dataclass
class TBCField:
    """Contents of a ``.tbc`` file (pnfam_storage.f90:488-560)."""
    use_hblas: int
    mode: int
    usep: int
    lecs: np.ndarray
    nb: int
    dqp: int
    nxy: int
    nxy12: int
    label: str
    k: int
    rank: int
    beta_minus: int
    parity_even: int
    use_2bc: np.ndarray
    gam: dict          # c3d, c3e, c4d, c4e[, cpd, cpe] without LECs
    delta: dict = None
    nxterms: int = 0


def read_tbc(path: str) -> TBCField:
    with open(path, "rb") as fh:
        recs = list(_records(fh.read()))
    if not recs:
        raise TwoBodyCurrentError("empty .tbc file")
    version = struct.unpack_from("<i", recs[0])[0] if len(recs[0]) >= 4 else -1
    if version != TBC_VERSION:
        raise TwoBodyCurrentError(f".tbc version {version} is not {TBC_VERSION}")
    i = 1
    while i < len(recs) and recs[i][:8] != b"extf_2bc":
        i += 1
    if i >= len(recs):
        raise TwoBodyCurrentError("no extf_2bc record in the .tbc file")
    i += 1
    ints = lambda r: np.frombuffer(r, dtype="<i4")
    f8 = lambda r: np.frombuffer(r, dtype="<f8")
    try:
        use_hblas = int(ints(recs[i])[0]); mode = int(ints(recs[i + 1])[0]); usep = int(ints(recs[i + 2])[0])
        lecs = f8(recs[i + 3]).copy()
        nb, dqp, nxy, nxy12 = (int(x) for x in ints(recs[i + 4])[:4])
        label = recs[i + 5].decode(errors="replace").strip()
        k = int(ints(recs[i + 6])[0]); rank = int(ints(recs[i + 7])[0])
        bm = int(ints(recs[i + 8])[0]); pe = int(ints(recs[i + 9])[0])
        u2 = ints(recs[i + 10]).copy()
        i += 11
        names = ["c3d", "c3e", "c4d", "c4e"] + (["cpd", "cpe"] if usep else [])
        gam = {}
        for nm in names:
            gam[nm] = f8(recs[i]).copy(); i += 1
        delta = None
        if nxy12 > 0:
            delta = {}
            for nm in names:
                delta[nm] = f8(recs[i]).copy(); i += 1
        nxt = int(ints(recs[i])[0])
    except (IndexError, struct.error, ValueError) as e:
        raise TwoBodyCurrentError(f"corrupted .tbc file: {e}")
    for nm, v in gam.items():
        if len(v) != nxy:
            raise TwoBodyCurrentError(f".tbc field {nm} has {len(v)} elements, expected {nxy}")
    return TBCField(use_hblas, mode, usep, lecs, nb, dqp, nxy, nxy12, label, k, rank, bm, pe, u2, gam, delta, nxt)


def write_tbc(path: str, t: TBCField) -> None:
    """Write ``t`` in the layout ``read_tbc`` reads (pnfam_storage.f90:488-560)."""
    def rec(b):
        return struct.pack("<i", len(b)) + b + struct.pack("<i", len(b))
    i4 = lambda *v: np.asarray(v, dtype="<i4").tobytes()
    out = [rec(i4(TBC_VERSION)), rec(b"extf_2bc"), rec(i4(t.use_hblas)), rec(i4(t.mode)), rec(i4(t.usep)),
           rec(np.asarray(t.lecs, dtype="<f8").tobytes()), rec(i4(t.nb, t.dqp, t.nxy, t.nxy12)),
           rec(t.label.ljust(80).encode()), rec(i4(t.k)), rec(i4(t.rank)), rec(i4(t.beta_minus)),
           rec(i4(t.parity_even)), rec(np.asarray(t.use_2bc, dtype="<i4").tobytes())]
    names = ["c3d", "c3e", "c4d", "c4e"] + (["cpd", "cpe"] if t.usep else [])
    for nm in names:
        out.append(rec(np.asarray(t.gam[nm], dtype="<f8").tobytes()))
    if t.nxy12 > 0:
        for nm in names:
            out.append(rec(np.asarray(t.delta[nm], dtype="<f8").tobytes()))
    out.append(rec(i4(t.nxterms)))
    with open(path, "wb") as fh:
        fh.write(b"".join(out))


def _tbc_compatible(t: TBCField, hfb, F, usep_requested: bool) -> bool:
    """read_tbc's compatibility checks (pnfam_storage.f90:601-628)."""
    return not (t.use_hblas != 1 or (t.usep == 0 and usep_requested) or t.nb != hfb.nb or t.dqp != hfb.dqp
                or t.nxy != F.mat.nelem or t.nxy12 != -1 or t.label != F.label or t.k != F.k
                or t.rank != F.rank or t.beta_minus != int(F.beta_minus) or t.parity_even != int(F.parity_even))


def compute_tbc(hfb, F, lec: LECs, usep: bool, mode: int = 0, nxterms: int = 0, compute=None) -> TBCField:
    """The finite-range field of the operator ``F`` computed from the two-body matrix
    elements (``effective_2bc_extfield``, on the GPU: ``finite_range.gamma_pieces``), as
    the ``.tbc`` record write_tbc stores (pnfam_storage.f90:488-560): LECs stripped,
    Gamma only.  ``compute`` replaces the GPU contraction (tests of the host logic)."""
    if compute is None:
        from .finite_range import gamma_pieces as compute
    try:
        pieces = compute(hfb, F, usep)
    except (OSError, RuntimeError) as e:
        raise TwoBodyCurrentError(f"computing the finite-range two-body-current field (.tbc) needs the CUDA "
                                  f"library and a GPU: {e}")
    names = ["c3d", "c3e", "c4d", "c4e"] + (["cpd", "cpe"] if usep else [])
    lecs = np.array([lec.c3, lec.c4, lec.cd / -0.25])
    return TBCField(1, int(mode), int(bool(usep)), lecs, int(hfb.nb), int(hfb.dqp), int(F.mat.nelem), -1,
                    str(F.label), int(F.k), int(F.rank), int(bool(F.beta_minus)), int(bool(F.parity_even)),
                    np.asarray(parse_mode(mode) if mode else (0,) * 6, dtype=np.int32),
                    {nm: np.asarray(pieces[nm], dtype=np.float64) for nm in names}, None, int(nxterms))


def finite_range_field(path: str, hfb, F, lec: LECs, usep_requested: bool, direct_only: bool, mode: int = 0,
                       nxterms: int = 0, log=None, compute=None) -> np.ndarray:
    """The finite-range GT field with the namelist LECs applied: sum of the direct
    and exchange c3, c4 (and pion-pole) parts, c3 -> c3, c4 -> c4 + 1/4
    (calc_totgamdel, pnfam_type_gamdel_2bc.f90:85-116).  The pieces come from the
    ``.tbc`` file at ``path`` (``read_tbc``, pnfam_storage.f90:562-727); a missing,
    incompatible or corrupted file is recomputed from the two-body matrix elements
    and stored there, as setup_extfield does (pnfam_solver.f90:617-633)."""
    say = log or (lambda msg: None)
    t = None
    if os.path.exists(path):
        say(f"  * Reading from extfield file: {path}")
        try:
            t = read_tbc(path)
        except TwoBodyCurrentError as e:
            say(f"  * The file '{path}' is corrupted! ({e})")
        if t is not None and not _tbc_compatible(t, hfb, F, usep_requested):
            say(f"  * The file '{path}' is incompatible with the current calculation!")
            t = None
    if t is None:
        say("  * Calculating 2BC matrix elements...")
        try:
            t = compute_tbc(hfb, F, lec, usep_requested, mode, nxterms, compute)
        except TwoBodyCurrentError as e:
            raise TwoBodyCurrentError(f"no usable finite-range field file '{path}': {e}")
        try:
            write_tbc(path, t)
        except OSError as e:
            # the file only caches the field for later runs; this run goes on without it
            say(f"  * Could not store the field in '{path}': {e}")
    nxy = F.mat.nelem
    c3, c4 = lec.c3, lec.c4 + 0.25
    g = t.gam
    zero = np.zeros(nxy)
    # calc_totgamdel (pnfam_type_gamdel_2bc.f90:85-116), summed in its order
    tot = zero + g["c3d"] * c3 + g["c4d"] * c4 + g.get("cpd", zero)
    if not direct_only:
        tot = tot + g["c3e"] * c3 + g["c4e"] * c4 + g.get("cpe", zero)
    return tot
