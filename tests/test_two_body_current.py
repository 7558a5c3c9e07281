"""Two-body-current (2BC) external fields against the reference's recorded runs.

Each case rebuilds the ground state from the recorded .hel file, composes the
2BC operator (GT with the cached finite-range field of a .tbc file; GT with the
DME exchange function; P and PS0 with the nuclear-matter corrections; P and
PS0 with the DME forms) and runs the CPU oracle for recorded points: the final
strength and cross terms against the recorded 19-digit values, and the whole
iteration table (10 printed decimals).  Cases recorded by an earlier revision
of the reference carry that revision's constants in their fixture.
"""
import os

import numpy as np
import pytest

from golden_cases import GOLDEN, case_for, golden, hfb
from oracle.fam_oracle import FAMOracle
from pynfam_gb300 import extfield_2bc as t2

REL = 1e-6

POINTS = [("S40_2bc_fam", "GT-K0", 0), ("S40_2bc_fam", "GT-K1", 1), ("S40_2bc_dme", "GT-K0", 0),
          ("S40_2bc_dme", "GT-K1", 2), ("S40_2bc_ps0", "PS0-K0", 0), ("S40_2bc_ps0", "RS0-K0", 1),
          ("Gd162_2bc_p", "P-K0", 0), ("Gd162_2bc_p", "P-K1", 1), ("Gd162_2bc_p", "R-K1", 0),
          ("S40_2bc_p_dme", "P-K0", 1), ("S40_2bc_ps0_dme", "PS0-K0", 0), ("S40_2bc_ps0_dme", "RS0-K0", 1)]


@pytest.mark.parametrize("case,op,idx", POINTS)
def test_two_body_current_matches_recorded(case, op, idx):
    c, pt = case_for(case, op, idx)
    assert int(c.nml["ext_field"]["two_body_current_mode"]) != 0
    s = c.nml["solver"]
    orc = FAMOracle(c.hfb, c.couplings, c.F, c.G, quench=c.quench)
    r = orc.solve(c.omega, max_iter=s["max_iter"], eps=s["convergence_epsilon"], broyden_m=s["broyden_history_size"])
    assert r.iter_conv == pt["converged"]
    for k, lab in enumerate(["Strength"] + orc.xlabels):
        want = pt["result"][lab]
        for got, w in ((r.re_str[k], want[0]), (r.im_str[k], want[1])):
            assert abs(got - w) <= REL * abs(w) + 1e-13, (lab, got, w)
    for (it, flag, si, re, im), h in zip(pt["history"], r.history):
        assert it == h[0] and flag == h[1]
        assert abs(si - h[2]) < 1.5e-10 * max(1.0, abs(si)) + 6e-11
        assert abs(re - h[3]) < 1.5e-10 * max(1.0, abs(re)) + 6e-11
        assert abs(im - h[4]) < 1.5e-10 * max(1.0, abs(im)) + 6e-11


def test_gt_finite_range_field_composition():
    """F = -F_1body + contact (cd = 0 here) + c3 (c3d + c3e) + (c4 + 1/4)(c4d + c4e)."""
    c, _ = case_for("S40_2bc_fam", "GT-K0", 0)
    from pynfam_gb300.extfield import init_external_field
    one = init_external_field(c.hfb, "-", "GT", 0).mat.flatten()
    t = t2.read_tbc(os.path.join(GOLDEN, "S40_2bc_fam", "GT-K0.tbc"))
    c3, c4 = -3.1962, 3.1962 + 0.25
    want = -one + (t.gam["c3d"] + t.gam["c3e"]) * c3 + (t.gam["c4d"] + t.gam["c4e"]) * c4
    np.testing.assert_allclose(c.F.mat.flatten(), want, rtol=0, atol=1e-15 * np.max(np.abs(want)))


def test_tbc_round_trip_and_compatibility(tmp_path):
    src = t2.read_tbc(os.path.join(GOLDEN, "S40_2bc_fam", "GT-K1.tbc"))
    assert (src.label, src.k, src.nb, src.dqp, src.nxy12, src.mode) == ("GT", 1, 26, 168, -1, 111100)
    p = tmp_path / "GT-K1.tbc"
    t2.write_tbc(str(p), src)
    back = t2.read_tbc(str(p))
    for k in src.gam:
        assert np.array_equal(src.gam[k], back.gam[k])
    assert p.read_bytes() == open(os.path.join(GOLDEN, "S40_2bc_fam", "GT-K1.tbc"), "rb").read()
    # a field for another operator, and a missing or corrupted file, are recomputed
    # (here by a stand-in for the GPU contraction that returns the reference's own
    # GT-K0 pieces) and stored, as setup_extfield does
    c, _ = case_for("S40_2bc_fam", "GT-K0", 0)
    lec = t2.LECs.from_namelist([-3.1962, 3.1962, 0.0])
    k0_path = os.path.join(GOLDEN, "S40_2bc_fam", "GT-K0.tbc")
    k0 = t2.read_tbc(k0_path)
    calls = []

    def stand_in(h, F, usep):
        calls.append((F.label, F.k, usep))
        return dict(k0.gam, cpd=np.zeros(k0.nxy), cpe=np.zeros(k0.nxy))
    from_file = t2.finite_range_field(k0_path, c.hfb, c.F, lec, False, False)
    absent = tmp_path / "absent.tbc"
    bad = tmp_path / "bad.tbc"
    bad.write_bytes(b"\x00" * 12)
    for path in (p, absent, bad):
        calls.clear()
        got = t2.finite_range_field(str(path), c.hfb, c.F, lec, False, False, 111100, 0, compute=stand_in)
        assert calls == [("GT", 0, False)]
        assert path.read_bytes() == open(k0_path, "rb").read()
        assert np.array_equal(got, from_file)
    # a compatible file is read, not recomputed
    calls.clear()
    t2.finite_range_field(str(absent), c.hfb, c.F, lec, False, False, 111100, 0, compute=stand_in)
    assert calls == []
    # a field without the pion-pole pieces is recomputed when they are requested
    t2.finite_range_field(str(absent), c.hfb, c.F, lec, True, False, 111100, 0, compute=stand_in)
    assert calls == [("GT", 0, True)]


def test_unwritable_tbc_location_keeps_the_computed_field(tmp_path):
    """A field computed where its .tbc cannot be stored is still used."""
    c, _ = case_for("S40_2bc_fam", "GT-K0", 0)
    lec = t2.LECs.from_namelist([-3.1962, 3.1962, 0.0])
    k0_path = os.path.join(GOLDEN, "S40_2bc_fam", "GT-K0.tbc")
    k0 = t2.read_tbc(k0_path)
    msgs = []
    got = t2.finite_range_field(str(tmp_path / "no_such_dir" / "GT-K0.tbc"), c.hfb, c.F, lec, False, False, 111100, 0,
                                log=msgs.append, compute=lambda h, F, usep: dict(k0.gam))
    assert np.array_equal(got, t2.finite_range_field(k0_path, c.hfb, c.F, lec, False, False))
    assert any("Could not store" in m for m in msgs)


def test_missing_tbc_is_computed_by_setup(tmp_path, monkeypatch):
    """setup_case computes a missing .tbc (stand-in contraction: the reference's
    pieces) and composes the same operator as from the reference's file."""
    from golden_cases import namelist_for
    from pynfam_gb300 import finite_range
    from pynfam_gb300.pnfam_setup import setup_case
    g = golden("S40_2bc_fam")
    nml = namelist_for("S40_2bc_fam", g["operators"]["GT-K0"][0])
    k0_path = os.path.join(GOLDEN, "S40_2bc_fam", "GT-K0.tbc")
    k0 = t2.read_tbc(k0_path)
    monkeypatch.setattr(finite_range, "gamma_pieces", lambda h, F, usep: dict(k0.gam))
    c = setup_case(nml, None, hfb=hfb("S40_2bc_fam"), tbc_dir=str(tmp_path))
    ref, _ = case_for("S40_2bc_fam", "GT-K0", 0)
    assert np.array_equal(c.F.mat.flatten(), ref.F.mat.flatten())
    assert (tmp_path / "GT-K0.tbc").read_bytes() == open(k0_path, "rb").read()


@pytest.mark.parametrize("mode,ok", [(0, True), (111100, True), (141100, True), (111001, True), (211100, True),
                                     (114, False), (311100, False), (161100, False), (112100, False),
                                     (211100 + 1000, False), (111003, False)])
def test_mode_digits(mode, ok):
    if ok:
        d = t2.parse_mode(mode)
        assert len(d) == 6 and (mode == 0 or d[0] in (1, 2))
    else:
        with pytest.raises(t2.TwoBodyCurrentError):
            t2.parse_mode(mode)


def test_i_function_and_density_factors():
    h = hfb("S40_2bc_dme")
    # I(1,1,1,1; r) is 3/2 at the centre, continuous at R and falls as 1/r outside
    I = t2.i1111(h)
    assert np.all(I > 0) and np.all(I <= 1.5)
    # DME exchange function vanishes with the density and is finite everywhere
    lec = t2.LECs.from_namelist([-3.1962, 3.1962, 0.0])
    f = t2.dme_exchange(h, lec)
    assert np.all(np.isfinite(f))
    # the U functions' small-kf branches join their closed forms (which lose
    # digits to cancellation there)
    kf = np.array([0.0011, 0.002])
    m = t2.MPI / t2.HBARC
    assert abs(t2.dme_u00(kf)[0] - 1.0 / m ** 2) < 1e-4 / m ** 2
    assert abs(t2.dme_u10(kf)[0] - 3.0 / m ** 2) < 1e-4 * 3.0 / m ** 2
