"""Quasiparticle occupations of the statistical FAM (finite temperature, EFA blocking).

The reference switches on the statistical FAM when the HFBTHO solution is at
finite temperature or has a blocked quasiparticle (``setup_hfb_solution``,
pnfam_setup.f90:324-381): the FAM then carries the diagonal quadrants P and Q
besides X and Y, weighted by the occupations f_p, f_n of the doubled
quasiparticle basis.

* Temperature T: f = (1 - tanh(E / 2T)) / 2 for every quasiparticle, 0 above
  the pairing window (hfbtho_solution.f90:376-389, 426, 446).
* EFA blocking: f = 1/2 on the blocked quasiparticle and on its time-reversed
  partner (index +- dqp/2, ``qp_t_reverse``, hfbtho_solution.f90:514-529), 0
  elsewhere (pnfam_setup.f90:365-380).
"""
from __future__ import annotations

import numpy as np


def thermal_occupations(hfb, temperature: float):
    """(f_p, f_n) at temperature T (MeV) from the quasiparticle energies of ``hfb``
    (quasiparticles above the pairing window carry E = 0 and get f = 0)."""
    T = float(temperature)
    if not T > 0.0:
        raise ValueError("temperature must be positive")

    def occ(E):
        E = np.asarray(E, dtype=np.float64)
        f = 0.5 * (1.0 - np.tanh(0.5 * E / T))
        return np.where(E == 0.0, 0.0, f)
    return occ(hfb.Ep), occ(hfb.En)


def qp_t_reverse(hfb, iqp: int) -> int:
    """Time-reversed partner of quasiparticle ``iqp`` (0-based) of the doubled basis."""
    half = hfb.dqp // 2
    return iqp + half if iqp < half else iqp - half


def blocking_occupations(hfb, iqp_n: int = None, iqp_p: int = None):
    """(f_p, f_n) of an odd nucleus in the equal-filling approximation: 1/2 on the
    blocked neutron / proton quasiparticle (0-based index in the doubled basis, or
    None) and on its time-reversed partner."""
    fp = np.zeros(hfb.dqp); fn = np.zeros(hfb.dqp)
    for f, q in ((fn, iqp_n), (fp, iqp_p)):
        if q is None:
            continue
        if not 0 <= int(q) < hfb.dqp:
            raise ValueError("blocked quasiparticle index out of range")
        f[int(q)] = 0.5
        f[qp_t_reverse(hfb, int(q))] = 0.5
    return fp, fn
