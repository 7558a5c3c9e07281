"""The HFBTHO .hel reader and the HFB reconstruction (input side).

Checkpoints are the reference's own recorded HFBTHO output for the 40S ground
state (tests/S40_GT_All/000000/hfb_soln/thoout.dat of the reference): the
first quasiparticle energies of the first neutron block (:211-220) and of the
second block (:227-230), and the Fermi energies (:601).
"""
import os

import numpy as np
import pytest

from golden_cases import GOLDEN, hfb
from pynfam_gb300.hel import HelFormatError, read_hel
from pynfam_gb300.hfb_solution import build_mesh_basis, diagonalise, hfb_matrices, local_density

HEL = os.path.join(GOLDEN, "S40.hel")


def test_hel_records():
    h = read_hel(HEL)
    assert (h.Z, h.N, h.n00, h.nb, h.nt, h.ngh, h.ngl) == (16, 24, 6, 13, 84, 20, 20)
    assert h.skyrme == "SKOP" and h.pwi == 60.0
    assert int(h.ID.sum()) == 84 and len(h.nr) == 84
    assert h.fields["n"]["v"].shape == (400,)


def test_quasiparticle_energies_match_hfbtho():
    h = read_hel(HEL)
    mb = build_mesh_basis(h)
    hd = hfb_matrices(h, mb)
    qn = diagonalise(h, hd, "n", float(h.N))
    qp = diagonalise(h, hd, "p", float(h.Z))
    want1 = [6.233577, 7.625658, 11.096926, 11.356932, 14.134658, 15.979785, 16.217338, 19.199761, 33.257664, 35.784569]
    want2 = [1.523648, 3.183052, 4.904171, 7.480768]
    np.testing.assert_allclose(qn.E[0][:10], want1, atol=1.5e-6)
    np.testing.assert_allclose(qn.E[1][:4], want2, atol=1.5e-6)
    assert abs(qn.ala - (-4.926368)) < 1e-6 and abs(qp.ala - (-14.620134)) < 1e-6
    # density of the rebuilt solution vs the density stored with the fields
    rn = local_density(h, mb, qn, float(h.N))
    assert np.max(np.abs(rn - h.ro[0])) < 1e-7
    # normalised to the particle number
    assert abs(np.sum(rn / mb.wdcori) - 24.0) < 1e-9


def test_kinetic_density_and_laplacian():
    """tau and Laplacian rho of the rebuilt solution (the DME inputs): the kinetic
    energies hbar^2/2m int tau against HFBTHO's printed values (thoout.dat :618 of
    the same run), and int Laplacian rho = 0."""
    s = hfb("S40")
    mb = build_mesh_basis(s.hel)
    hb = s.hel.hbzero
    assert abs(hb * np.sum(s.tau_n / mb.wdcori) - 447.846356) < 1.5e-6
    assert abs(hb * np.sum(s.tau_p / mb.wdcori) - 265.730132) < 1.5e-6
    for d2 in (s.d2rho_n, s.d2rho_p):
        assert abs(np.sum(d2 / mb.wdcori)) < 1e-12


def test_doubled_solution_is_unitary():
    s = hfb("S40")
    nb, half = s.nb, s.nb // 2
    for i in range(nb):
        U, V = s.Up[i], s.Vp[(i + half) % nb]
        # columns of block i's quasiparticles: U block i and V of the partner row
        act = np.any(U != 0, axis=0)
        g = U.T @ U + V.T @ V
        np.testing.assert_allclose(g[np.ix_(act, act)], np.eye(int(act.sum())), atol=1e-12)
    assert s.dqp == 168 and s.nb == 26
    # spin-up states first in every block
    for i in range(nb):
        ns = s.ns[s.isstart[i]:s.isstart[i] + s.db[i]]
        assert np.all(ns[:s.num_spin_up[i]] > 0) and np.all(ns[s.num_spin_up[i]:] < 0)


def test_corrupt_file_rejected(tmp_path):
    blob = open(HEL, "rb").read()
    bad = tmp_path / "bad.hel"
    bad.write_bytes(blob[:5000])
    with pytest.raises(HelFormatError):
        read_hel(str(bad))
    bad.write_bytes(b"\x04\x00\x00\x00\x07\x00\x00\x00\x04\x00\x00\x00")
    with pytest.raises(HelFormatError):
        read_hel(str(bad))


def test_unsupported_ground_states_are_refused():
    """A blocked (odd-nucleus) solution needs HFBTHO's blocking equations, which this
    reader does not restate: loading one stops with a message instead of a wrong state."""
    import copy
    from pynfam_gb300.hfb_solution import load_hfb_solution
    h = copy.copy(read_hel(HEL))
    h.N = h.N + 1
    with pytest.raises(ValueError, match="not supported"):
        load_hfb_solution(h)


def test_finite_temperature_reconstruction():
    """The 40S fields rebuilt at finite temperature (thermal hfbdiag/ALambda/DENSIT):
    the particle numbers hold, T -> 0 gives the zero-temperature state, and the
    statistical FAM's occupations follow f = (1 - tanh(E/2T))/2, 0 above the window."""
    import copy
    from pynfam_gb300.hfb_solution import load_hfb_solution
    cold = hfb("S40")
    mb = build_mesh_basis(cold.hel)
    assert cold.occupations is None
    for T, close in ((1e-3, True), (1.5, False)):
        h = copy.copy(read_hel(HEL))
        h.set_temperature, h.temperature = True, T
        s = load_hfb_solution(h)
        fp, fn = s.occupations
        assert s.temperature == T and fp.shape == (s.dqp,)
        np.testing.assert_allclose(fn, np.where(s.En == 0, 0.0, 0.5 * (1 - np.tanh(0.5 * s.En / T))), rtol=0, atol=0)
        assert abs(np.sum(s.rho_n / mb.wdcori) - 24.0) < 1e-9 and abs(np.sum(s.rho_p / mb.wdcori) - 16.0) < 1e-9
        d = max(np.max(np.abs(s.rho_n - cold.rho_n)), np.max(np.abs(s.tau_p - cold.tau_p)),
                np.max(np.abs(s.En - cold.En)))
        if close:
            assert d < 1e-10, d
        else:
            assert d > 1e-4 and np.max(fn) > 0.05
