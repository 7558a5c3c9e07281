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


# ---------------------------------------------------------------------------------
# the GPU contraction's per-item arithmetic, run serially on the host by a test
# harness built from the same header (tests/tbc_host_check.cpp)
# ---------------------------------------------------------------------------------
@pytest.fixture(scope="module")
def host_harness(tmp_path_factory):
    import ctypes
    import shutil
    import subprocess
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    so = str(tmp_path_factory.mktemp("tbc") / "tbc_host.so")
    subprocess.run([cxx, "-O2", "-std=c++17", "-shared", "-fPIC", "-pthread", "-o", so,
                    os.path.join(ROOT, "tests", "tbc_host_check.cpp")], check=True)
    return ctypes.CDLL(so)


def _harness(lib, hfb, F, use_p):
    import ctypes
    from pynfam_gb300 import finite_range
    s, keep = finite_range.input_struct(hfb, F, use_p)
    out = np.zeros(6 * s.nxy)
    rc = lib.tbc_host_field(ctypes.byref(s), out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), None)
    assert rc == 0
    out = out.reshape(6, -1)
    return {nm: out[i] for i, nm in enumerate(("c3d", "c3e", "c4d", "c4e", "cpd", "cpe"))}


@pytest.mark.parametrize("K", [0, 1])
def test_kernel_arithmetic_reproduces_reference_tbc(K, host_harness):
    from pynfam_gb300.extfield_2bc import read_tbc
    hfb, F = _case(K)
    t = read_tbc(os.path.join(GOLD, "S40_2bc_fam", f"GT-K{K}.tbc"))
    got = _harness(host_harness, hfb, F, False)
    _compare(got, t.gam)
    assert not np.any(got["cpd"]) and not np.any(got["cpe"])


def test_kernel_arithmetic_matches_oracle_with_pion_pole(host_harness):
    """The pion-pole pieces (two_body_current_usep) and beta+ have no recorded
    reference run: the kernels' arithmetic against the oracle."""
    from oracle.tbc_oracle import two_body_gamma
    from pynfam_gb300.extfield import init_external_field
    from pynfam_gb300.hfb_solution import load_hfb_solution
    hfb = load_hfb_solution(os.path.join(GOLD, "S40_2bc_fam.hel"))
    F = init_external_field(hfb, "+", "GT", 0)
    h = hfb.hel
    want = two_body_gamma(h.nz, h.nr, h.nl, h.ns, h.ID, h.bz, h.bp, hfb.density_matrices("n"),
                          hfb.density_matrices("p"), F.mat.cols, F.mat.offsets(), F.mat.nelem, 0, False, use_p=True)
    got = _harness(host_harness, hfb, F, True)
    scale = max(np.abs(w).max() for w in want.values())
    assert np.abs(want["cpe"]).max() > 1e-3 * scale
    for nm, w in want.items():
        assert np.abs(got[nm] - w).max() <= 1e-12 * scale, nm


def test_kernel_arithmetic_matches_oracle_on_deformed_ground_state(host_harness):
    """The recorded 162Gd ground state (prolate; no recorded two-body-current run):
    the kernels' arithmetic against the oracle, GT K = 1."""
    from oracle.tbc_oracle import two_body_gamma
    from pynfam_gb300.extfield import init_external_field
    from pynfam_gb300.hfb_solution import load_hfb_solution
    hfb = load_hfb_solution(os.path.join(GOLD, "Gd162.hel"))
    F = init_external_field(hfb, "-", "GT", 1)
    h = hfb.hel
    want = two_body_gamma(h.nz, h.nr, h.nl, h.ns, h.ID, h.bz, h.bp, hfb.density_matrices("n"),
                          hfb.density_matrices("p"), F.mat.cols, F.mat.offsets(), F.mat.nelem, 1, True)
    got = _harness(host_harness, hfb, F, False)
    scale = max(np.abs(w).max() for w in want.values())
    for nm in PIECES:
        assert np.abs(got[nm] - want[nm]).max() <= 1e-12 * scale, nm


# ---------------------------------------------------------------------------------
# the GPU
# ---------------------------------------------------------------------------------
@pytest.mark.gpu
@pytest.mark.parametrize("K", [0, 1])
def test_gpu_field_reproduces_reference_tbc(K):
    from pynfam_gb300.extfield_2bc import read_tbc
    from pynfam_gb300.finite_range import gamma_pieces
    hfb, F = _case(K)
    t = read_tbc(os.path.join(GOLD, "S40_2bc_fam", f"GT-K{K}.tbc"))
    st = {}
    got = gamma_pieces(hfb, F, False, stats=st)
    _compare(got, t.gam)
    assert st["groups"] > 0 and st["terms"] > 0 and st["stage2_ms"] > 0


@pytest.mark.gpu
def test_gpu_field_matches_oracle_with_pion_pole():
    from oracle.tbc_oracle import two_body_gamma
    from pynfam_gb300.extfield import init_external_field
    from pynfam_gb300.finite_range import gamma_pieces
    from pynfam_gb300.hfb_solution import load_hfb_solution
    hfb = load_hfb_solution(os.path.join(GOLD, "S40_2bc_fam.hel"))
    F = init_external_field(hfb, "+", "GT", 0)
    h = hfb.hel
    want = two_body_gamma(h.nz, h.nr, h.nl, h.ns, h.ID, h.bz, h.bp, hfb.density_matrices("n"),
                          hfb.density_matrices("p"), F.mat.cols, F.mat.offsets(), F.mat.nelem, 0, False, use_p=True)
    got = gamma_pieces(hfb, F, True)
    scale = max(np.abs(w).max() for w in want.values())
    for nm, w in want.items():
        assert np.abs(got[nm] - w).max() <= 1e-12 * scale, nm


@pytest.mark.gpu
def test_gpu_computed_tbc_reproduces_recorded_strengths(tmp_path):
    """A run without the .tbc file: the set-up computes the finite-range field on
    the GPU, stores it, and the FAM solve on the GPU reproduces the reference's
    recorded 2BC strengths (GT K = 0 and K = 1 of 40S)."""
    from golden_cases import golden, hfb, namelist_for
    from pynfam_gb300.extfield_2bc import read_tbc
    from pynfam_gb300.pnfam_setup import setup_case
    from pynfam_gb300.solver import GPUSolver
    g = golden("S40_2bc_fam")
    for op in ("GT-K0", "GT-K1"):
        pts = g["operators"][op]
        c = setup_case(namelist_for("S40_2bc_fam", pts[0]), None, hfb=hfb("S40_2bc_fam"), tbc_dir=str(tmp_path))
        written = read_tbc(str(tmp_path / f"{op}.tbc"))
        ref = read_tbc(os.path.join(GOLD, "S40_2bc_fam", f"{op}.tbc"))
        _compare(written.gam, ref.gam)
        s = c.nml["solver"]
        gpu = GPUSolver(c.hfb, c.couplings)
        try:
            gpu.set_operator(c.F, c.G)
            omegas = [complex(p["namelist"]["real_eqrpa"], p["namelist"]["imag_eqrpa"]) for p in pts]
            r = gpu.solve(omegas, max_iter=s["max_iter"], eps=s["convergence_epsilon"],
                          broyden_m=s["broyden_history_size"], quench=c.quench)
        finally:
            gpu.close()
        for i, p in enumerate(pts):
            want = complex(*p["result"]["Strength"])
            assert abs(r.re_S[i, 0] - want.real) <= 1e-6 * abs(want.real), (op, i)
            assert abs(r.im_S[i, 0] - want.imag) <= 1e-6 * abs(want.imag), (op, i)


@pytest.mark.gpu
def test_gpu_field_matches_kernel_arithmetic_at_nsh10(host_harness):
    """A larger basis (162Gd fields in the full N_sh = 10 basis, 12,444 GT K = 1
    elements), where the oracle would take too long: the GPU against the same
    per-item arithmetic run serially on the host (summation order differs)."""
    from pynfam_gb300.extfield import init_external_field
    from pynfam_gb300.finite_range import gamma_pieces
    from pynfam_gb300.synthetic import ground_state
    hfb = ground_state(os.path.join(GOLD, "Gd162.hel"), 10)
    F = init_external_field(hfb, "-", "GT", 1)
    want = _harness(host_harness, hfb, F, True)
    got = gamma_pieces(hfb, F, True)
    scale = max(np.abs(w).max() for w in want.values())
    for nm, w in want.items():
        assert np.abs(got[nm] - w).max() <= 1e-12 * scale, nm
