"""CPU oracle of the finite-range two-body-current field (test infrastructure).

This module is the checker for the GPU contraction of the two-body (Yukawa)
axial current with the ground-state density matrices; only tests and the
smoke/benchmark checkers import it.  It restates, loop for loop, the optimised
branch of the reference's ``effective_2bc_extfield``
(pnfam_extfield_2bc.f90:128-465) and the matrix-element routines it calls:

* the Gaussian fit of the Yukawa function and the 1D two-body Gaussian matrix
  elements, with up to two derivatives on the oscillator functions
  (pnfam_spatial_mtxels.f90:52-55, 78-209, 703-927);
* HFBTHO's hypergeometric form of the 1D element and the coefficient tables
  T_z and Cp2c (hfbtho_gogny.f90:651-686, 884-915, 991-1045, 1246-1380;
  HFBTHO built with GOGNY_HYPER = 1);
* the spherical-derivative elements ddGz, ddGr and radx
  (pnfam_spatial_mtxels.f90:223-450, 609-688);
* the current's spatial pieces and their spin-isospin contraction
  (pnfam_type_extfield_2bc.f90:47-84, 182-398, 750-825, 869-1463);
* the (k, r, l, s) groups of the basis that HFBTHO's ``base`` builds for
  finite-range forces (hfbtho_solver.f90:3246-3301).

The result is the six pieces c3d, c3e, c4d, c4e, cpd, cpe of the Gamma field
in the flat block layout of the operator, with the LECs stripped the way the
``.tbc`` file stores them (pnfam_storage.f90:488-560): the c3 pieces are
computed with c3 = 1, the c4 pieces with c4 + 1/4 = 1.  Elements are placed at
HFBTHO's state order inside each block (the position ``ita_tr - isstart`` the
reference uses) and then reordered into the spin-sorted basis, the layout of
the ``.tbc`` file.  The Gaussian sum
is vectorised (numpy over the six Gaussians); everything else is plain loops
with memoised matrix elements, so an N_sh = 6 operator takes seconds.
"""
from __future__ import annotations

import math
from functools import lru_cache

import numpy as np

from pynfam_gb300.extfield_2bc import FPI, HBARC, MN, MPI, PI

# Gaussian fit of exp(-x)/x = sum_i b_i exp(-a_i x^2) (pnfam_spatial_mtxels.f90:52-55)
Y0_A = (34.0, 6.60, 1.44, 0.38, 0.15, 0.13)
Y0_B = (6.79, 2.41, 0.786, 0.241, -0.062, 0.078)
NG = len(Y0_A)
SQ2 = math.sqrt(2.0)

# the 14 spatial pieces of the current (type extfield_2bc)
RKP, RKZ, RKM, RPZ, RPM, RZM, R0P, R0Z, R0M, RP0, RZ0, RM0, RPZ2, RZM2 = range(14)
NCOMP = 14


# ----------------------------------------------------------------------------
# HFBTHO helpers (hfbtho_gogny.f90)
# ----------------------------------------------------------------------------
_FACT = [1.0]


def factrl(n: int) -> float:
    while len(_FACT) <= n:
        _FACT.append(len(_FACT) * _FACT[-1])
    return _FACT[n]


def binomialco(m: int, n: int) -> float:
    if n < 0 or n > m:
        return 0.0
    if n == 0 or n == m:
        return 1.0
    if n == 1 or n == m - 1:
        return float(m)
    if n <= m // 2:
        return (factrl(m) / factrl(m - n)) / factrl(n)
    return (factrl(m) / factrl(n)) / factrl(m - n)


def upperfactrl(x: float, i: int) -> float:
    u = 1.0
    for j in range(i):
        u *= x + j
    return u


def hypergeom2f1(a: int, b: int, c: float, x: float) -> float:
    """2F1(a, b; c; x) for non-positive integers a, b (hfbtho_gogny.f90:1286-1311)."""
    d, e = abs(max(a, b)), abs(min(a, b))
    return sum(binomialco(d, i) * binomialco(e, i) * x ** i * factrl(i) / upperfactrl(c, i) for i in range(d + 1))


@lru_cache(maxsize=None)
def t_z(n1: int, n2: int, n: int) -> float:
    """T_{n1 n2}^n (calculateTz, hfbtho_gogny.f90:651-686)."""
    if n1 > n2:
        n1, n2 = n2, n1
    if n < abs(n2 - n1) or n > n1 + n2 or (n - n1 - n2) % 2:
        return 0.0
    m1, m2, m3 = (-n1 + n2 + n) // 2, (n1 - n2 + n) // 2, (n1 + n2 - n) // 2
    return (math.sqrt(factrl(n2)) / factrl(m1)) * (math.sqrt(factrl(n)) / factrl(m2)) * (math.sqrt(factrl(n1)) / factrl(m3))


@lru_cache(maxsize=None)
def cp2c(n: int, k: int, ny: int) -> float:
    """Polar -> Cartesian coefficient C_{nx ny}^{n k} (calculateCpolar2cartesian,
    hfbtho_gogny.f90:884-915)."""
    ak = abs(k)
    if ny > 2 * n + ak or ny < 0:
        return 0.0
    nx = 2 * n + ak - ny
    a = ((-1) ** n * (2.0 ** (-n - ak * 0.5)) * math.sqrt(factrl(n + ak))
         * (math.sqrt(factrl(n)) / (math.sqrt(factrl(nx)) * math.sqrt(factrl(ny)))))
    h = (ak - k) // 2
    xs = 0.0
    for q in range(min(ny, n + h) + 1):
        xs += binomialco(nx, n - q + h) * binomialco(ny, q) * (-1) ** (ny - q)
    return a * xs


def matrix_element_z(ni: int, nj: int, nk: int, nl: int, mu: float, b: float) -> float:
    """<ni nj|exp(-(z1-z2)^2/mu^2)|nk nl> in the hypergeometric form
    (MatrixElement_z with GOGNY_HYPER = 1, hfbtho_gogny.f90:991-1045)."""
    s1 = (nj + nl - abs(nj - nl)) // 2 + 1
    s2 = (ni + nk - abs(ni - nk)) // 2 + 1
    if s1 == s2:
        s1, s2 = min(ni, nk), min(nj, nl)
    if s1 <= s2:
        ii, ij, ik, il = ni, nj, nk, nl
    else:
        ii, ij, ik, il = nj, ni, nl, nk
    z = 1.0 + mu ** 2 / (2.0 * b ** 2)
    v = 0.0
    for nz in range(abs(ij - il), ij + il + 1, 2):
        if (ii + ik + nz) % 2:
            break
        xi = (ii + ik + nz + 1) * 0.5
        fbar = (math.gamma(xi - ii) * math.gamma(xi - ik) * math.gamma(xi - nz)
                / (z ** xi * math.sqrt(factrl(ii) * factrl(ik) * factrl(nz)))
                * hypergeom2f1(-ii, -ik, nz + 1 - xi, 1 - z))
        v += t_z(ij, il, nz) * fbar
    return mu / (math.sqrt(2.0 * PI ** 3) * b) * v


# ----------------------------------------------------------------------------
# Gaussian matrix elements with derivatives (pnfam_spatial_mtxels.f90)
# ----------------------------------------------------------------------------
class SpatialElements:
    """The 1D Gaussian elements of both directions and the spherical-derivative
    elements built from them, each an array over the six Gaussians."""

    def __init__(self, bz: float, bp: float):
        m = MPI / HBARC
        # prep_gaussian: widths and prefactors of Y0(x) = exp(-mpi x)/(4 pi x)
        self.mu = [(1.0 / math.sqrt(a)) / m for a in Y0_A]
        self.pf = [b * m * 0.25 / PI for b in Y0_B]
        self.b = {True: bz, False: bp}
        self.pd1 = {True: 1.0 / (bz * SQ2), False: 1.0 / (bp * SQ2)}
        self.pd2 = {True: 1.0 / (bz * bz * 2.0), False: 1.0 / (bp * bp * 2.0)}
        self.me1d = lru_cache(maxsize=None)(self._me1d)
        self.me_1d = lru_cache(maxsize=None)(self._me_1d)
        self.radx = lru_cache(maxsize=None)(self._radx)
        self._tables = {}
        self.radw = lru_cache(maxsize=None)(self._radw)

    # ME1Dz (with the Gaussian prefactors) and ME1Dr (without) (calculateME1D)
    def _me1d(self, z: bool, ni: int, nj: int, nk: int, nl: int) -> np.ndarray:
        if min(ni, nj, nk, nl) < 0 or (ni + nj + nk + nl) % 2:
            return np.zeros(NG)
        b = self.b[z]
        v = [matrix_element_z(ni, nj, nk, nl, self.mu[g], b) for g in range(NG)]
        if z:
            v = [v[g] * self.pf[g] for g in range(NG)]
        return np.array(v)

    def ho_derivative(self, n: int, d: int, z: bool):
        """d^d/dx^d of a 1D oscillator function as (n', coefficient) pairs (ho_derivative)."""
        p1, p2 = self.pd1[z], self.pd2[z]
        if d == 0:
            return [(n, 1.0)]
        if d == 1:
            out = [(n + 1, -math.sqrt(float(n + 1)) * p1)]
            if n - 1 >= 0:
                out.append((n - 1, math.sqrt(float(n)) * p1))
            return out
        out = [(n + 2, math.sqrt(float((n + 1) * (n + 2))) * p2), (n, -(2.0 * n + 1.0) * p2)]
        if n - 2 >= 0:
            out.append((n - 2, math.sqrt(float(n * (n - 1))) * p2))
        return out

    def me_1d_dho(self, ni, nj, nk, nl, di, dj, dk, dl, z):
        """MatrixElement_1d_dho: derivatives on the four oscillator functions."""
        v = np.zeros(NG)
        for nnl, cl in self.ho_derivative(nl, dl, z):
            for nnk, ck in self.ho_derivative(nk, dk, z):
                for nnj, cj in self.ho_derivative(nj, dj, z):
                    for nni, ci in self.ho_derivative(ni, di, z):
                        if (nni + nnj + nnk + nnl) % 2:
                            continue
                        v = v + self.me1d(z, nni, nnj, nnk, nnl) * ci * cj * ck * cl
        return v

    def _me_1d(self, ni, nj, nk, nl, z, d, p) -> np.ndarray:
        """MatrixElement_1d: d derivatives on the Gaussian, or 2i p of particle p."""
        zero = np.zeros(NG)
        if p == 0:
            if (ni + nj + nk + nl + d) % 2:
                return zero
        else:
            if (ni + nj + nk + nl + d + 1) % 2:
                return zero
            if p == 1 and ni == nk:
                return zero
            if p == 2 and nj == nl:
                return zero
        f = self.me_1d_dho
        if d == 0 and p == 0:
            return self.me1d(z, ni, nj, nk, nl)
        if d == 1 and p == 0:
            return f(ni, nj, nk, nl, 1, 0, 0, 0, z) * (-1.0) + f(ni, nj, nk, nl, 0, 0, 1, 0, z) * (-1.0)
        if d == 2 and p == 0:
            return f(ni, nj, nk, nl, 2, 0, 0, 0, z) + f(ni, nj, nk, nl, 0, 0, 2, 0, z) + f(ni, nj, nk, nl, 1, 0, 1, 0, z) * 2.0
        if d == 1 and p == 1:
            return f(ni, nj, nk, nl, 0, 0, 2, 0, z) * (-1.0) + f(ni, nj, nk, nl, 2, 0, 0, 0, z)
        if d == 1 and p == 2:
            return f(ni, nj, nk, nl, 0, 0, 0, 2, z) + f(ni, nj, nk, nl, 0, 2, 0, 0, z) * (-1.0)
        if d == 0 and p == 1:
            return f(ni, nj, nk, nl, 0, 0, 1, 0, z) + f(ni, nj, nk, nl, 1, 0, 0, 0, z) * (-1.0)
        if d == 0 and p == 2:
            return f(ni, nj, nk, nl, 0, 0, 0, 1, z) + f(ni, nj, nk, nl, 0, 1, 0, 0, z) * (-1.0)
        raise ValueError((d, p))

    def ddgz(self, ni, nj, nk, nl, di, dj, dip) -> np.ndarray:
        """MatrixElement_ddGz: z part of d_i d_j G (d_i -> 2i P_dip when dip > 0)."""
        p = 1 if dip else 0
        if di == 0 and dj == 0:
            return self.me_1d(ni, nj, nk, nl, True, 2 - p, dip)
        if abs(di + dj) in (0, 2):
            return self.me_1d(ni, nj, nk, nl, True, 0, 0)
        if di == 0:
            return self.me_1d(ni, nj, nk, nl, True, 1 - p, dip)
        return self.me_1d(ni, nj, nk, nl, True, 1, 0)

    def _table(self, dx, px, n):
        """Dense [NG, n+1, n+1, n+1, n+1] copy of me_1d(., False, dx, px) (the
        ME1Dr / ME1Dr_xx tables of calculateME1D)."""
        t = self._tables.get((dx, px))
        if t is None or t.shape[1] <= n:
            t = np.zeros((NG, n + 1, n + 1, n + 1, n + 1))
            for a in range(n + 1):
                for b in range(n + 1):
                    for c in range(n + 1):
                        for d in range(n + 1):
                            t[:, a, b, c, d] = self.me_1d(a, b, c, d, False, dx, px)
            self._tables[(dx, px)] = t
        return t

    def _radw(self, ni, li, nj, lj, nk, lk, nl, ll) -> np.ndarray:
        """Weights sign * Ci Cj Ck Cl over (nyi, nyj, nyk, nyl), 0 for odd total ny."""
        A = (2 * ni + abs(li), 2 * nj + abs(lj), 2 * nk + abs(lk), 2 * nl + abs(ll))
        c = [np.array([cp2c(q, l, ny) for ny in range(a + 1)]) for (q, l), a in
             zip(((ni, li), (nj, lj), (nk, lk), (nl, ll)), A)]
        y = np.ix_(*[np.arange(a + 1) for a in A])
        ny_sum = y[0] + y[1] + y[2] + y[3]
        sgn = np.where(ny_sum % 2 == 0, (-1.0) ** ((y[0] + y[1] + ny_sum // 2) % 2), 0.0)
        return sgn * c[0][:, None, None, None] * c[1][None, :, None, None] * c[2][None, None, :, None] \
            * c[3][None, None, None, :]

    def _radx(self, ni, li, nj, lj, nk, lk, nl, ll, dx, px) -> np.ndarray:
        """MatrixElement_radx: (r, phi) part with dx/px derivatives in x only.
        The quadruple sum over the Cartesian decompositions n = nx + ny of the
        four polar states, with the terms of odd total ny skipped, evaluated as
        one contraction over dense 1D tables."""
        A = (2 * ni + abs(li), 2 * nj + abs(lj), 2 * nk + abs(lk), 2 * nl + abs(ll))
        n = max(A)
        X = self._table(dx, px, n)
        Y = self._table(0, 0, n)
        w = self.radw(ni, li, nj, lj, nk, lk, nl, ll)
        # nx = A - ny runs backwards while ny runs forwards
        xs = X[:, A[0]::-1, A[1]::-1, A[2]::-1, A[3]::-1]
        ys = Y[:, :A[0] + 1, :A[1] + 1, :A[2] + 1, :A[3] + 1]
        return np.einsum("gijkl,gijkl,ijkl->g", xs, ys, w)

    def rad_cmplx_imag(self, ni, li, nj, lj, nk, lk, nl, ll, dx, dy, px, py) -> np.ndarray:
        """Imaginary part of MatrixElement_rad_cmplx (x and y derivatives)."""
        v = np.zeros(NG)
        for nyi in range(2 * ni + abs(li) + 1):
            nxi = 2 * ni + abs(li) - nyi
            ci = cp2c(ni, li, nyi)
            for nyj in range(2 * nj + abs(lj) + 1):
                nxj = 2 * nj + abs(lj) - nyj
                cj = cp2c(nj, lj, nyj)
                for nyk in range(2 * nk + abs(lk) + 1):
                    nxk = 2 * nk + abs(lk) - nyk
                    ck = cp2c(nk, lk, nyk)
                    for nyl in range(2 * nl + abs(ll) + 1):
                        nxl = 2 * nl + abs(ll) - nyl
                        cl = cp2c(nl, ll, nyl)
                        e = (nyi + nyj - nyk - nyl) % 4      # i^e
                        im = (0.0, 1.0, 0.0, -1.0)[e]
                        if im == 0.0:
                            continue
                        v = v + (im * ci * cj * ck * cl) * self.me_1d(nxi, nxj, nxk, nxl, False, dx, px) \
                            * self.me_1d(nyi, nyj, nyk, nyl, False, dy, py)
        return v

    def ddgr(self, ni, li, nj, lj, nk, lk, nl, ll, di, dj, dip) -> np.ndarray:
        """MatrixElement_ddGr: (r, phi) part of d_i d_j G."""
        if -li - lj + lk + ll + di + dj != 0:
            return np.zeros(NG)
        p = 1 if dip else 0
        q = (ni, li, nj, lj, nk, lk, nl, ll)
        if di == 0 and dj == 0:
            return self.radx(*q, 0, 0)
        if abs(di + dj) == 2:
            return self.radx(*q, 2 - p, dip) * 2.0
        if abs(di + dj) == 1:
            if dj == 0:
                return self.radx(*q, 1 - p, dip) * (-(di + dj) * SQ2)
            return self.radx(*q, 1, 0) * (-(di + dj) * SQ2)
        v = self.radx(*q, 2 - p, dip) * (-1.0)
        if dip:
            v = v + self.rad_cmplx_imag(*q, 1, 0, 0, dip)
        return v


# ----------------------------------------------------------------------------
# spatial pieces of the current (pnfam_type_extfield_2bc.f90)
# ----------------------------------------------------------------------------
class Current:
    """calc_Jz_opt / calc_Jr_opt for one K, LEC-stripped (c3 = 1, c4 + 1/4 = 1)."""

    def __init__(self, se: SpatialElements, K: int, use_p: bool):
        if K not in (-1, 0, 1):
            raise ValueError("invalid K for the two-body current")
        self.se, self.K, self.use_p = se, K, use_p
        caux = HBARC ** 3 / (2.0 * MN * FPI * FPI)
        c3, c4p14 = 1.0, 1.0
        cy0p = caux * (4.0 * c4p14)
        self.c_c3_c4r2 = caux * c3 * (4.0 * SQ2)
        self.c_c3_8 = caux * c3 * 8.0
        self.cy0p_c2r2 = cy0p * (2.0 * SQ2)
        self.cy0p_2 = cy0p * 2.0
        self.cy0p_4 = cy0p * 4.0
        self.caux_cr2 = caux * SQ2
        self.caux_2 = caux * 2.0
        self.jz = lru_cache(maxsize=None)(self._jz)
        self.jr = lru_cache(maxsize=None)(self._jr)

    def _jz(self, ni, nj, nk, nl) -> np.ndarray:
        se, K = self.se, self.K
        J = np.zeros((NCOMP, NG))
        z = lambda di, dj, dip: se.ddgz(ni, nj, nk, nl, di, dj, dip)
        if self.use_p:
            J[R0P] = +self.caux_cr2 * z(K, -1, 1)
            J[R0Z] = +self.caux_2 * z(K, 0, 1)
            J[R0M] = -self.caux_cr2 * z(K, +1, 1)
            J[RP0] = +self.caux_cr2 * z(K, -1, 2)
            J[RZ0] = +self.caux_2 * z(K, 0, 2)
            J[RM0] = -self.caux_cr2 * z(K, +1, 2)
        dpm, d00 = z(+1, -1, 0), z(0, 0, 0)
        if K == 1:
            dp0 = z(+1, 0, 0)
            dpp = dpm
            J[RKP] = -self.c_c3_c4r2 * dpm
            J[RKZ] = -self.c_c3_8 * dp0
            J[RKM] = +self.c_c3_c4r2 * dpp
            J[RPZ] = +self.cy0p_c2r2 * d00
            J[RPM] = -self.cy0p_2 * dp0
            J[RZM] = -self.cy0p_c2r2 * dpp
            J[RPZ2] = -self.cy0p_c2r2 * dpm
        elif K == 0:
            d0m = z(0, -1, 0)
            dp0 = d0m
            J[RKP] = -self.c_c3_c4r2 * d0m
            J[RKZ] = -self.c_c3_8 * d00
            J[RKM] = +self.c_c3_c4r2 * dp0
            J[RPZ] = +self.cy0p_c2r2 * d0m
            J[RPM] = -self.cy0p_4 * dpm
            J[RZM] = -self.cy0p_c2r2 * dp0
        else:
            d0m = z(0, -1, 0)
            dmm = dpm
            J[RKP] = -self.c_c3_c4r2 * dmm
            J[RKZ] = -self.c_c3_8 * d0m
            J[RKM] = +self.c_c3_c4r2 * dpm
            J[RPZ] = +self.cy0p_c2r2 * dmm
            J[RPM] = -self.cy0p_2 * d0m
            J[RZM] = -self.cy0p_c2r2 * d00
            J[RZM2] = +self.cy0p_c2r2 * dpm
        return J

    def _jr(self, ni, li, nj, lj, nk, lk, nl, ll) -> np.ndarray:
        se, K = self.se, self.K
        J = np.zeros((NCOMP, NG))
        r = lambda di, dj, dip: se.ddgr(ni, li, nj, lj, nk, lk, nl, ll, di, dj, dip)
        if self.use_p:
            J[R0P], J[R0Z], J[R0M] = r(K, -1, 1), r(K, 0, 1), r(K, +1, 1)
            J[RP0], J[RZ0], J[RM0] = r(K, -1, 2), r(K, 0, 2), r(K, +1, 2)
        dpm, d00 = r(+1, -1, 0), r(0, 0, 0)
        if K == 1:
            dp0, dpp = r(+1, 0, 0), r(+1, +1, 0)
            J[RKP], J[RKZ], J[RKM] = dpm, dp0, dpp
            J[RPZ], J[RPM], J[RZM] = d00, dp0, dpp
            J[RPZ2] = dpm
        elif K == 0:
            d0m, dp0 = r(0, -1, 0), r(+1, 0, 0)
            J[RKP], J[RKZ], J[RKM] = d0m, d00, dp0
            J[RPZ], J[RPM], J[RZM] = d0m, dpm, dp0
        else:
            d0m, dmm = r(0, -1, 0), r(-1, -1, 0)
            J[RKP], J[RKZ], J[RKM] = dmm, d0m, dpm
            J[RPZ], J[RPM], J[RZM] = dmm, d0m, d00
            J[RZM2] = dpm
        return J


# ----------------------------------------------------------------------------
# spin-isospin contraction (gam_Jrs*_dir/exc, calc_gam_sep)
# ----------------------------------------------------------------------------
H = 0.5


def _jrsa_dir(J, sa, sc, sd, sb):
    if sd + sb == 0:
        return 0.0
    if sa == sc:
        return (sa * H) * J[RKZ]
    return J[RKP] if sa == 1 else J[RKM]


def _jrsx_dir(J, sa, sc, sd, sb):
    du, ud, uu = (sd == -1 and sb == 1), (sd == 1 and sb == -1), sd + sb > 0
    if sa == sc:
        if du:
            return (sa * H) * (-J[RPZ])
        if ud:
            return (sa * H) * J[RZM]
        return 0.0
    if sa == 1:
        if du:
            return 0.0
        if ud:
            return J[RPM]
        return H * J[RPZ] if uu else -H * J[RPZ]
    if du:
        return -J[RPM]
    if ud:
        return 0.0
    return -H * J[RZM] if uu else H * J[RZM]


def _jrsxp_dir(J, sa, sc, sd, sb):
    du, ud, uu = (sd == -1 and sb == 1), (sd == 1 and sb == -1), sd + sb > 0
    if sa == sc:
        if du:
            return J[R0P]
        if ud:
            return J[R0M]
        return (sa * H) * J[RZ0] + H * J[R0Z] if uu else (sa * H) * J[RZ0] - H * J[R0Z]
    if du or ud:
        return 0.0
    return J[RP0] if sa == 1 else J[RM0]


def _jrsa_exc(J, sa, sc, sd, sb):
    du, ud, uu = (sd == -1 and sb == 1), (sd == 1 and sb == -1), sd + sb > 0
    if sa == 1 and sc == 1:
        return J[RKP] if du else 0.0 if ud else H * J[RKZ] if uu else 0.0
    if sa == -1 and sc == -1:
        return 0.0 if du else J[RKM] if ud else 0.0 if uu else -H * J[RKZ]
    if sa == 1:
        return 0.0 if du else H * J[RKZ] if ud else 0.0 if uu else J[RKP]
    return -H * J[RKZ] if du else 0.0 if ud else J[RKM] if uu else 0.0


def _jrsb_exc(J, sa, sc, sd, sb):
    du, ud, uu = (sd == -1 and sb == 1), (sd == 1 and sb == -1), sd + sb > 0
    if sa == 1 and sc == 1:
        return 0.0 if du else J[RKM] if ud else H * J[RKZ] if uu else 0.0
    if sa == -1 and sc == -1:
        return J[RKP] if du else 0.0 if ud else 0.0 if uu else -H * J[RKZ]
    if sa == 1:
        return 0.0 if du else -H * J[RKZ] if ud else J[RKP] if uu else 0.0
    return H * J[RKZ] if du else 0.0 if ud else 0.0 if uu else J[RKM]


def _jrsx_exc(J, sa, sc, sd, sb):
    du, ud, uu = (sd == -1 and sb == 1), (sd == 1 and sb == -1), sd + sb > 0
    if sa == sc:
        if du:
            return H * J[RPZ]
        if ud:
            return H * J[RZM]
        if sa == 1:
            return 0.0 if uu else J[RPM]
        return -J[RPM] if uu else 0.0
    if du or ud:
        return 0.0
    return -H * J[RPZ] if sa == 1 else -H * J[RZM]


def _jrsxp_exc(J, sa, sc, sd, sb):
    du, ud, uu = (sd == -1 and sb == 1), (sd == 1 and sb == -1), sd + sb > 0
    if sa == 1 and sc == 1:
        return J[RP0] if du else J[R0M] if ud else H * J[RZ0] + H * J[R0Z] if uu else 0.0
    if sa == -1 and sc == -1:
        return J[R0P] if du else J[RM0] if ud else 0.0 if uu else -H * J[RZ0] - H * J[R0Z]
    if sa == 1:
        return 0.0 if du else H * J[RZ0] - H * J[R0Z] if ud else J[R0P] if uu else J[RP0]
    return -H * J[RZ0] + H * J[R0Z] if du else 0.0 if ud else J[RM0] if uu else J[R0M]


def _fold2(J):
    """Add the second d_i d_j Y0 terms into rpz and rzm (calc_gam_sep)."""
    J = J.copy()
    J[RPZ] = J[RPZ] + J[RPZ2]
    J[RZM] = J[RZM] + J[RZM2]
    return J


def gam_sep(jdn, jdp, jen, jep, sa, sc, sd, sb, bminus):
    """calc_gam_sep: the six pieces (c3d, c3e, c4d, c4e, cpd, cpe), each [NG]."""
    jdn, jdp, jen, jep = _fold2(jdn), _fold2(jdp), _fold2(jen), _fold2(jep)
    a_dn, x_dn, xp_dn = _jrsa_dir(jdn, sa, sc, sd, sb), _jrsx_dir(jdn, sa, sc, sd, sb), _jrsxp_dir(jdn, sa, sc, sd, sb)
    a_dp, x_dp, xp_dp = _jrsa_dir(jdp, sa, sc, sd, sb), _jrsx_dir(jdp, sa, sc, sd, sb), _jrsxp_dir(jdp, sa, sc, sd, sb)
    a_en, b_en = _jrsa_exc(jen, sa, sc, sd, sb), _jrsb_exc(jen, sa, sc, sd, sb)
    x_en, xp_en = _jrsx_exc(jen, sa, sc, sd, sb), _jrsxp_exc(jen, sa, sc, sd, sb)
    a_ep, b_ep = _jrsa_exc(jep, sa, sc, sd, sb), _jrsb_exc(jep, sa, sc, sd, sb)
    x_ep, xp_ep = _jrsx_exc(jep, sa, sc, sd, sb), _jrsxp_exc(jep, sa, sc, sd, sb)
    if bminus:
        r = (a_dn + a_dp, -a_en - b_ep, +H * (x_dn - x_dp), -H * (x_en + x_ep),
             +H * (xp_dn - xp_dp), -H * (xp_en + xp_ep))
    else:
        r = (a_dn + a_dp, -b_en - a_ep, -H * (x_dn - x_dp), -H * (x_en + x_ep),
             -H * (xp_dn - xp_dp), -H * (xp_en + xp_ep))
    return np.array([np.broadcast_to(x, (NG,)) for x in r])


@lru_cache(maxsize=None)
def gam_sep_map(sa, sc, sd, sb, bminus) -> np.ndarray:
    """gam_sep as the [6, 4 * NCOMP] matrix that it is (every piece is linear in
    the products dn, dp, en, ep), found by applying it to unit vectors."""
    m = np.zeros((6, 4 * NCOMP))
    for col in range(4 * NCOMP):
        u = np.zeros((4 * NCOMP, NG))
        u[col] = 1.0
        m[:, col] = gam_sep(u[:NCOMP], u[NCOMP:2 * NCOMP], u[2 * NCOMP:3 * NCOMP], u[3 * NCOMP:], sa, sc, sd, sb,
                            bminus)[:, 0]
    return m


# ----------------------------------------------------------------------------
# basis bookkeeping and the contraction (pnfam_extfield_2bc.f90:128-465)
# ----------------------------------------------------------------------------
def krls_groups(nz, nr, nl, ns):
    """HFBTHO's (k, r, l, s) groups with their z lists (base, hfbtho_solver.f90:
    3262-3301): k ascending, then r, then (l, s) = (k-1, +1), (k, -1); z in
    even then odd z + l order, ascending.  Built from the basis states present."""
    present = {(int(a), int(b), int(c), int(d)) for a, b, c, d in zip(nz, nr, nl, ns)}
    kmax = max(int(l) + (int(s) + 1) // 2 for l, s in zip(nl, ns))
    rmax, zmax = int(max(nr)), int(max(nz))
    groups = []
    for k in range(1, kmax + 1):
        for r in range(rmax + 1):
            for l, s in ((k - 1, 1), (k, -1)):
                zs = [z for ip in (0, 1) for z in range(zmax + 1) if (z + l) % 2 == ip and (z, r, l, s) in present]
                if zs:
                    groups.append((k, r, l, s, zs))
    return groups


def two_body_gamma(nz, nr, nl, ns, block_sizes, bz, bp, rk_n, rk_p, cols, offsets, nxy, K, beta_minus,
                   use_p=False):
    """The LEC-stripped Gamma pieces of the finite-range field, {name: [nxy]}.

    nz, nr, nl, ns: the ntx basis states in HFBTHO order; block_sizes: HFBTHO's
    nbx block sizes; rk_n, rk_p: per HFBTHO block the density matrix ``rk``
    (twice rho) in HFBTHO state order; cols/offsets: block column (0-based,
    -1 empty) and flat start of every block row of the doubled operator."""
    nz, nr, nl, ns = (np.asarray(a, dtype=np.int64) for a in (nz, nr, nl, ns))
    ntx, nbx = len(nz), len(block_sizes)
    db = np.concatenate([block_sizes, block_sizes]).astype(np.int64)
    isstart = np.concatenate([[0], np.cumsum(db)[:-1]])
    ib_itx = np.repeat(np.arange(2 * nbx), db)
    index = {(int(nz[t]), int(nr[t]), int(nl[t]), int(ns[t])): t for t in range(ntx)}
    groups = krls_groups(nz, nr, nl, ns)
    nzx, nrx = int(nz.max()), int(nr.max())
    nrlx = int(max(2 * nr + nl))
    nox = max(g[0] for g in groups) - 1
    se = SpatialElements(bz, bp)
    cur = Current(se, K, use_p)
    out = np.zeros((6, nxy))
    shape = (nrx + 1, nrx + 1, 2, 2, nox + 1, NCOMP, NG)
    for za in range(nzx + 1):
        for zc in range(nzx + 1):
            Znd, Zpd, Zne, Zpe = (np.zeros(shape) for _ in range(4))
            for (kb, rb, lb, sb, zlb) in groups:
                nlb = (kb - lb + 1) % 2
                for (kd, rd, ld, sd, zld) in groups:
                    if kd != kb:
                        continue
                    nld = (kd - ld + 1) % 2
                    for zb in zlb:
                        jb = index[(zb, rb, lb, sb)]
                        ibb = ib_itx[jb]
                        inb = jb - isstart[ibb]
                        for zd in zld:
                            jd = index[(zd, rd, ld, sd)]
                            if ib_itx[jd] != ibb:
                                continue
                            ind = jd - isstart[ibb]
                            rho_n = rk_n[ibb][ind, inb] * 0.5
                            rho_p = rk_p[ibb][ind, inb] * 0.5
                            jdir = cur.jz(za, zb, zc, zd)
                            jexc = cur.jz(za, zb, zd, zc)
                            key = (rd, rb, nld, nlb, kb - 1)
                            Znd[key] += jdir * rho_n
                            Zpd[key] += jdir * rho_p
                            Zne[key] += jexc * rho_n
                            Zpe[key] += jexc * rho_p
            for ita_tr in range(2 * ntx):
                ita, a_tr = (ita_tr - ntx, -1) if ita_tr >= ntx else (ita_tr, 1)
                if nz[ita] != za:
                    continue
                ra, la, sa = int(nr[ita]), int(nl[ita]) * a_tr, int(ns[ita]) * a_tr
                iba = ib_itx[ita_tr]
                ina = ita_tr - isstart[iba]
                sign_a = -1 if (ita_tr >= ntx and ns[ita] < 0) else 1
                if cols[iba] < 0:
                    continue
                for itc_tr in range(2 * ntx):
                    itc, c_tr = (itc_tr - ntx, -1) if itc_tr >= ntx else (itc_tr, 1)
                    if nz[itc] != zc:
                        continue
                    rc, lc, sc = int(nr[itc]), int(nl[itc]) * c_tr, int(ns[itc]) * c_tr
                    ibc = ib_itx[itc_tr]
                    if cols[iba] != ibc:
                        continue
                    inc = itc_tr - isstart[ibc]
                    sign_c = -1 if (itc_tr >= ntx and ns[itc] < 0) else 1
                    gam = np.zeros((6, NG))
                    for ob in range(nox + 1):
                        for nlb in (0, 1):
                            lb, sb = ob + nlb, 1 - 2 * nlb
                            for nld in (0, 1):
                                ld, sd = ob + nld, 1 - 2 * nld
                                sign_db = -1 if sd + sb == 0 else 1
                                for rb in range(nrx + 1):
                                    if 2 * rb + lb > nrlx:
                                        continue
                                    for rd in range(nrx + 1):
                                        if 2 * rd + ld > nrlx:
                                            continue
                                        key = (rd, rb, nld, nlb, ob)
                                        if la + lb - lc - ld in (K + 1, K, K - 1):
                                            jd_ = cur.jr(ra, la, rb, lb, rc, lc, rd, ld)
                                            je_ = cur.jr(ra, la, rb, lb, rd, ld, rc, lc)
                                            gam += gam_sep_map(sa, sc, sd, sb, beta_minus) @ np.concatenate(
                                                [Znd[key] * jd_, Zpd[key] * jd_, Zne[key] * je_, Zpe[key] * je_])
                                        if la - lb - lc + ld in (K + 1, K, K - 1):
                                            jd_ = cur.jr(ra, la, rb, -lb, rc, lc, rd, -ld)
                                            je_ = cur.jr(ra, la, rb, -lb, rd, -ld, rc, lc)
                                            gam += sign_db * (gam_sep_map(sa, sc, -sd, -sb, beta_minus) @ np.concatenate(
                                                [Znd[key] * jd_, Zpd[key] * jd_, Zne[key] * je_, Zpe[key] * je_]))
                    nac = ina + inc * db[iba]
                    out[:, offsets[iba] + nac] = gam.sum(axis=1) * (sign_a * sign_c)
    # reorder rows and columns of every block into the spin-sorted basis, spin-up
    # states first (reorder_blockmatrix_basis 'a', pnfam_extfield_2bc.f90:901-913)
    nsd = np.concatenate([ns, -ns])
    order = []
    for ib in range(2 * nbx):
        s = nsd[isstart[ib]:isstart[ib] + db[ib]]
        order.append(np.concatenate([np.nonzero(s > 0)[0], np.nonzero(s < 0)[0]]))
    res = np.zeros_like(out)
    for ib in range(2 * nbx):
        ic = cols[ib]
        if ic < 0:
            continue
        dr, dc = db[ib], db[ic]
        blk = out[:, offsets[ib]:offsets[ib] + dr * dc].reshape(6, dc, dr)    # [piece, col, row]
        res[:, offsets[ib]:offsets[ib] + dr * dc] = blk[:, order[ic]][:, :, order[ib]].reshape(6, -1)
    return {nm: res[i] for i, nm in enumerate(("c3d", "c3e", "c4d", "c4e", "cpd", "cpe"))}
