"""The finite-range two-body-current field (the contraction of the Yukawa
current with the ground-state density matrices, pnfam_extfield_2bc.f90:26-915).

CPU: the oracle restatement reproduces the reference's own ``.tbc`` output for
the 40S Gamow-Teller K = 0 and K = 1 fields (written by the reference for these
runs, LECs stripped).
"""
import os

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden")
PIECES = ("c3d", "c3e", "c4d", "c4e")


def _case(K):
    from pynfam_gb300.extfield import init_external_field
    from pynfam_gb300.hfb_solution import load_hfb_solution
    hfb = load_hfb_solution(os.path.join(GOLD, "S40_2bc_fam.hel"))
    F = init_external_field(hfb, "-", "GT", K)
    return hfb, F


def _compare(got, want):
    # every piece within 1e-12 of the field's scale; the direct c4 piece vanishes
    # for this operator (both sides are rounding noise of ~1e-19)
    scale = max(np.abs(want[nm]).max() for nm in PIECES)
    for nm in PIECES:
        d = np.abs(np.asarray(got[nm]) - want[nm]).max()
        assert d <= 1e-12 * scale, (nm, d, scale)


@pytest.mark.parametrize("K", [0, 1])
def test_oracle_reproduces_reference_tbc(K):
    from oracle.tbc_oracle import two_body_gamma
    from pynfam_gb300.extfield_2bc import read_tbc
    hfb, F = _case(K)
    h = hfb.hel
    t = read_tbc(os.path.join(GOLD, "S40_2bc_fam", f"GT-K{K}.tbc"))
    assert t.usep == 0 and t.k == K and t.nxy == F.mat.nelem
    got = two_body_gamma(h.nz, h.nr, h.nl, h.ns, h.ID, h.bz, h.bp, hfb.density_matrices("n"),
                         hfb.density_matrices("p"), F.mat.cols, F.mat.offsets(), F.mat.nelem, K, True)
    _compare(got, t.gam)
