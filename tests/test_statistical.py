"""Statistical FAM (finite temperature / EFA blocking: quadrants P and Q beside X
and Y, pnfam_solver.f90:248-254,425-458) in the CPU oracle.

No recorded finite-temperature or blocked run exists among the reference's test
outputs, so the statistical form is held to limits it must reach: with all
occupations zero it is the T = 0 iteration (P = Q = 0, T factors 1), and at
T -> 0 its strength tends to the T = 0 strength.  The GPU statistical form is
compared with this oracle in tests/test_gpu_parity.py.
"""
import numpy as np
import pytest

from golden_cases import case_for
from oracle.fam_oracle import FAMOracle
from pynfam_gb300.statistics import blocking_occupations, qp_t_reverse, thermal_occupations


def _solve(c, occ, max_iter=None):
    s = c.nml["solver"]
    orc = FAMOracle(c.hfb, c.couplings, c.F, c.G, quench=c.quench, occupations=occ)
    return orc.solve(c.omega, max_iter=max_iter or s["max_iter"], eps=s["convergence_epsilon"],
                     broyden_m=s["broyden_history_size"])


@pytest.mark.parametrize("case,op,idx", [("S40", "GT-K0", 0), ("S40", "RS1-K1", 3)])
def test_zero_occupations_reproduce_ground_state_form(case, op, idx):
    c, _ = case_for(case, op, idx)
    z = np.zeros(c.hfb.dqp)
    r0 = _solve(c, None)
    r1 = _solve(c, (z, z))
    assert r1.iter_conv == r0.iter_conv
    np.testing.assert_allclose(r1.re_str, r0.re_str, rtol=1e-12, atol=1e-15)
    np.testing.assert_allclose(r1.im_str, r0.im_str, rtol=1e-12, atol=1e-15)
    for a, b in zip(r0.history, r1.history):
        assert a[1] == b[1] and abs(a[2] - b[2]) <= 1e-12 * max(1.0, abs(a[2]))


def test_low_temperature_limit():
    c, _ = case_for("S40", "GT-K0", 5)
    r0 = _solve(c, None)
    rt = _solve(c, thermal_occupations(c.hfb, 0.1))
    assert rt.iter_conv >= 0
    S0, St = complex(r0.re_str[0], r0.im_str[0]), complex(rt.re_str[0], rt.im_str[0])
    assert abs(St - S0) <= 1e-5 * abs(S0)
    # at 2 MeV the thermal quadrants change the strength visibly
    r2 = _solve(c, thermal_occupations(c.hfb, 2.0))
    assert r2.iter_conv >= 0
    assert abs(complex(r2.re_str[0], r2.im_str[0]) - S0) > 1e-3 * abs(S0)


def test_occupations():
    c, _ = case_for("S40", "GT-K0", 0)
    h = c.hfb
    fp, fn = thermal_occupations(h, 1.0)
    assert fp.shape == (h.dqp,) and np.all((fp >= 0) & (fp < 0.5))
    assert np.all(fp[h.Ep == 0] == 0) and np.all(fn[h.En == 0] == 0)
    # time-reversed partners carry the same occupation
    half = h.dqp // 2
    np.testing.assert_array_equal(fn[:half], fn[half:])
    bp, bn = blocking_occupations(h, iqp_n=3)
    assert bn[3] == 0.5 and bn[qp_t_reverse(h, 3)] == 0.5 and bn.sum() == 1.0 and not bp.any()
    with pytest.raises(ValueError):
        blocking_occupations(h, iqp_p=h.dqp)


def test_finite_temperature_ground_state_solves():
    """A finite-temperature ground state (the 40S fields rebuilt at T = 1 MeV) carries
    its occupations into the statistical FAM, which converges; pnfam_main passes the
    same occupations to the GPU solver."""
    import copy
    import os
    from golden_cases import GOLDEN, golden, namelist_for
    from pynfam_gb300.hel import read_hel
    from pynfam_gb300.hfb_solution import load_hfb_solution
    from pynfam_gb300.pnfam_setup import setup_case
    h = copy.copy(read_hel(os.path.join(GOLDEN, "S40.hel")))
    h.set_temperature, h.temperature = True, 1.0
    hot = load_hfb_solution(h)
    pt = golden("S40")["operators"]["GT-K0"][5]
    c = setup_case(namelist_for("S40", pt), None, hfb=hot)
    assert c.hfb.occupations is not None
    r = _solve(c, c.hfb.occupations)
    assert r.iter_conv > 0 and np.isfinite(r.re_str[0])
