"""Parity at the benchmark configurations that have no recorded FAM outputs.

Config 1: 40S in the N_sh = 8 basis (the reference's own ground state; its
recorded GT runs are empty), GT- K = 0 on 40 points of the half circle
(centre 10 MeV, radius 25 MeV), Broyden history 7 and mixing 0.4, epsilon 1e-7.
The FP64 GPU form is held to the CPU oracle (same iteration count, complex
strengths to 1e-8 of |S|: rounding differences grow over the ~40 Broyden steps; next to
a pole the count may differ by an iteration or two, the strengths then by < 1e-6),
and the mixed form to the FP64 fixed point (1e-6).

Config 2: a synthetic Bogoliubov ground state (seed 1) in the N_sh = 12 basis
with Omega-only blocks (up to 91), GT- K = 0 and K = 1 at Im omega = 0.5 MeV,
Re omega uniform in [-10, 30] MeV: the first iterations against the oracle, and
the mixed form against the FP64 fixed point.
"""
import os

import numpy as np
import pytest

from golden_cases import GOLDEN
from oracle.fam_oracle import FAMOracle

pytestmark = pytest.mark.gpu

REL = 1e-6
INTERACTION = {"interaction_name": "SKOP", "require_self_consistency": True, "require_gauge_invariance": True,
               "force_j2_terms": False, "vpair_t0": -346.352, "override_cs0": 128.279, "override_csr": 0.0,
               "override_cds": 0.0}


def _case(hfb, k, M, self_consistent=True, quench=1.0):
    from pynfam_gb300.namelist import defaults
    from pynfam_gb300.pnfam_setup import setup_case
    nml = defaults()
    nml["interaction"].update(INTERACTION)
    nml["interaction"]["require_self_consistency"] = self_consistent
    nml["ext_field"].update(operator_name="GT", operator_k=k, beta_type="-", compute_crossterms=False)
    nml["solver"].update(max_iter=300, convergence_epsilon=1e-7, broyden_history_size=M,
                         quench_residual_int=quench)
    return setup_case(nml, None, hfb=hfb)


def _mixed_vs_fixed_point(c, omegas, M, alpha):
    from pynfam_gb300.solver import GPUSolver
    gpu = GPUSolver(c.hfb, c.couplings)
    gpu.set_operator(c.F, c.G)
    kw = dict(broyden_m=M, quench=c.quench, alpha_mix=alpha)
    exact = gpu.solve(omegas, max_iter=1000, eps=1e-12, **kw)
    mixed = gpu.solve(omegas, max_iter=1000, eps=1e-9, precision=1, settle=8, **kw)
    gpu.close()
    worst, n = 0.0, 0
    for i in range(len(omegas)):
        if exact.iters[i] < 0:
            continue
        assert mixed.iters[i] >= 0, (i, mixed.si[i])
        w = complex(exact.re_S[i, 0], exact.im_S[i, 0])
        g = complex(mixed.re_S[i, 0], mixed.im_S[i, 0])
        for a, b in ((g.real, w.real), (g.imag, w.imag)):
            assert abs(a - b) <= REL * abs(b) + 1e-12 * abs(w), (i, a, b)
        worst = max(worst, abs(g - w) / abs(w))
        n += 1
    return worst, n


@pytest.fixture(scope="module")
def config1():
    from pynfam_gb300.contour import circle
    from pynfam_gb300.hfb_solution import load_hfb_solution
    hfb = load_hfb_solution(os.path.join(GOLDEN, "S40_nsh8.hel"))
    assert int(hfb.n00) == 8 and int(max(hfb.db)) == 25 and int(hfb.dqp) == 330
    return _case(hfb, 0, 7), circle(-15.0, 35.0, 80)


def test_config1_fp64_matches_oracle(config1):
    from pynfam_gb300.solver import GPUSolver
    c, omegas = config1
    assert len(omegas) == 40
    idx = [0, 5, 20, 39]
    gpu = GPUSolver(c.hfb, c.couplings)
    gpu.set_operator(c.F, c.G)
    r = gpu.solve(omegas[idx], max_iter=300, eps=1e-7, broyden_m=7, quench=c.quench, alpha_mix=0.4)
    gpu.close()
    orc = FAMOracle(c.hfb, c.couplings, c.F, c.G, quench=c.quench, alpha_mix=0.4)
    nconv = 0
    for k, i in enumerate(idx):
        ref = orc.solve(complex(omegas[i]), max_iter=300, eps=1e-7, broyden_m=7)
        if ref.iter_conv < 0:
            assert int(r.iters[k]) < 0, (i, r.iters[k])
            continue   # not converged in 300 iterations in either (the point next to the real axis)
        # near a pole the convergence test can fire an iteration earlier or later as the
        # rounding of the two implementations differs; the strengths then still agree to 1e-6
        assert abs(int(r.iters[k]) - ref.iter_conv) <= 2, (i, r.iters[k], ref.iter_conv)
        nconv += 1
        g = complex(r.re_S[k, 0], r.im_S[k, 0])
        w = complex(ref.re_str[0], ref.im_str[0])
        tol = 1e-8 if int(r.iters[k]) == ref.iter_conv else 1e-6
        assert abs(g - w) <= tol * abs(w), (i, g, w)
    assert nconv >= 2


def test_config1_mixed_matches_fp64_fixed_point(config1):
    c, omegas = config1
    worst, n = _mixed_vs_fixed_point(c, omegas, 7, 0.4)
    print(f"config 1: {n} points, mixed form worst relative error vs FP64 fixed point {worst:.2e}")
    assert n >= 30


@pytest.fixture(scope="module")
def config2():
    from pynfam_gb300.synthetic import bogoliubov_nucleus
    hfb = bogoliubov_nucleus(os.path.join(GOLDEN, "Gd162.hel"), 12, seed=1, parity=False)
    assert int(max(hfb.db)) == 91 and int(hfb.dqp) == 910
    rng = np.random.default_rng(1)
    omegas = rng.uniform(-10.0, 30.0, 12) + 0.5j
    return hfb, omegas


@pytest.mark.parametrize("k,tc_density,pair", [(0, False, False), (1, False, False), (1, True, False),
                                                (0, True, True), (1, True, True)])
def test_config2_synthetic_field_split_precision_vs_fp64(config2, k, tc_density, pair, monkeypatch):
    """The split-precision (3xTF32 tensor-core) field evaluation against FP64 on the
    synthetic state, whose blocks (up to 91) take the multi-tile tensor-core paths
    (with tensor-core densities: two column ranges per block), and through the
    pair-tensor GEMMs (pair: their M tiles span several blocks of a spin class)."""
    from pynfam_gb300.blockmatrix import BlockMatrix
    from pynfam_gb300.solver import GPUSolver
    monkeypatch.setenv("PNFAM_GB300_TC_DENSITY", "1" if tc_density else "0")
    monkeypatch.setenv("PNFAM_GB300_PAIR_GEMM", "1" if pair else "0")
    monkeypatch.setenv("PNFAM_GB300_PAIR_MIN", "1")
    hfb, _ = config2
    c = _case(hfb, k, 50, self_consistent=False)
    gpu = GPUSolver(c.hfb, c.couplings)
    gpu.set_operator(c.F, c.G)
    nb = hfb.nb
    half = nb // 2
    tr = np.array([(i + half) % nb for i in range(nb)])
    fc = np.asarray(c.F.mat.cols)
    xc = np.array([tr[fc[i]] if fc[i] >= 0 else -1 for i in range(nb)])
    yc = np.array([fc[tr[i]] for i in range(nb)])
    xtc = np.full(nb, -1); ytc = np.full(nb, -1)
    for i in range(nb):
        if xc[i] >= 0: xtc[xc[i]] = i
        if yc[i] >= 0: ytc[yc[i]] = i
    rng = np.random.default_rng(2 + k)
    ins = []
    for cols in (fc, xtc, fc, ytc):
        n = BlockMatrix.empty(cols, hfb.db).nelem
        ins.append(rng.standard_normal(n) + 1j * rng.standard_normal(n))
    want = gpu.calc_hamiltonian(*ins)
    got = gpu.calc_hamiltonian(*ins, mixed=True)
    gpu.close()
    worst = max(float(np.max(np.abs(g - w)) / np.max(np.abs(w))) for g, w in zip(got, want))
    print(f"config 2 GT K={k} (tensor-core densities {tc_density}, pair GEMMs {pair}): split-precision field worst "
          f"relative error {worst:.2e}")
    assert worst <= 1e-5


@pytest.mark.parametrize("k", [0, 1])
def test_config2_synthetic_mixed_matches_fp64_fixed_point(config2, k):
    """The mixed form reaches the FP64 fixed point (1e-6) on the synthetic state.

    With its full residual interaction the random Bogoliubov state gives a FAM
    iteration that does not converge at Im omega = 0.5 MeV (si stalls near 1e-2 in
    the FP64 form and the oracle alike), so there would be nothing to compare.  The
    residual interaction is quenched to 0.3 (the reference's quench_residual_int,
    pnfam_solver.f90:170): the iteration then converges (about 25 steps in the oracle
    at omega = 8.0 + 0.5i) and every point is compared."""
    hfb, omegas = config2
    c = _case(hfb, k, 50, self_consistent=False, quench=0.3)
    worst, n = _mixed_vs_fixed_point(c, omegas, 50, None)
    print(f"config 2 GT K={k} (residual interaction x 0.3): {n} of {len(omegas)} points converge; "
          f"mixed form worst relative error vs FP64 fixed point {worst:.2e}")
    assert n == len(omegas)


def test_config2_synthetic_history_matches_oracle(config2):
    from pynfam_gb300.solver import GPUSolver
    hfb, omegas = config2
    c = _case(hfb, 1, 50, self_consistent=False)
    gpu = GPUSolver(c.hfb, c.couplings)
    gpu.set_operator(c.F, c.G)
    r = gpu.solve([omegas[0]], max_iter=4, eps=1e-7, broyden_m=50, quench=c.quench, history=True)
    gpu.close()
    orc = FAMOracle(c.hfb, c.couplings, c.F, c.G, quench=c.quench)
    ref = orc.solve(complex(omegas[0]), max_iter=4, eps=1e-7, broyden_m=50)
    for h in ref.history:
        g = r.hist[0, h[0]]
        for a, b in ((g[0], h[2]), (g[1], h[3]), (g[2], h[4])):
            assert abs(a - b) <= 1e-10 * max(abs(b), 1e-6), (h, g)


@pytest.fixture(scope="module")
def config4():
    """The large-basis stress configuration: the synthetic Bogoliubov state of seed 3
    in the full N_sh = 20 basis with Omega-only blocks (1771 Omega>0 states, 3542 with
    partners, the largest block 231)."""
    import json
    from pynfam_gb300.synthetic import bogoliubov_nucleus
    with open(os.path.join(GOLDEN, "nsh20_oracle.json")) as fh:
        pin = json.load(fh)
    hfb = bogoliubov_nucleus(os.path.join(GOLDEN, "Gd162.hel"), pin["nsh"], seed=pin["seed"], parity=False)
    assert int(max(hfb.db)) == 231 == pin["max_block"] and int(hfb.dqp) == 3542 == pin["dqp"]
    return hfb, pin


@pytest.mark.parametrize("k", [0, 1])
def test_config4_history_matches_oracle(config4, k):
    """The FP64 form's first four iterations at N_sh = 20 against the oracle
    (tests/golden/nsh20_oracle.json, made by tests/golden/make_nsh20_oracle.py)."""
    from pynfam_gb300.solver import GPUSolver
    hfb, pin = config4
    c = _case(hfb, k, 50, self_consistent=False)
    assert int(c.F.mat.nelem) == pin["nxy"][f"GT-K{k}"]
    gpu = GPUSolver(c.hfb, c.couplings)
    gpu.set_operator(c.F, c.G)
    r = gpu.solve([complex(*pin["omega"])], max_iter=4, eps=1e-30, broyden_m=50, quench=c.quench, history=True)
    gpu.close()
    for it, si, re, im in pin["operators"][f"GT-K{k}"]:
        g = r.hist[0, it]
        for a, b in ((g[0], si), (g[1], re), (g[2], im)):
            assert abs(a - b) <= 1e-9 * max(abs(b), 1e-6), (k, it, g, (si, re, im))


@pytest.mark.parametrize("k", [0, 1])
def test_config4_split_precision_field_vs_fp64(config4, k):
    """The split-precision field evaluation at N_sh = 20 (blocks up to 231: several row
    and column tiles per block in every tensor-core kernel) against FP64."""
    from pynfam_gb300.blockmatrix import BlockMatrix
    from pynfam_gb300.solver import GPUSolver
    hfb, _ = config4
    c = _case(hfb, k, 50, self_consistent=False)
    gpu = GPUSolver(c.hfb, c.couplings)
    gpu.set_operator(c.F, c.G)
    nb = hfb.nb
    half = nb // 2
    tr = np.array([(i + half) % nb for i in range(nb)])
    fc = np.asarray(c.F.mat.cols)
    xc = np.array([tr[fc[i]] if fc[i] >= 0 else -1 for i in range(nb)])
    yc = np.array([fc[tr[i]] for i in range(nb)])
    xtc = np.full(nb, -1); ytc = np.full(nb, -1)
    for i in range(nb):
        if xc[i] >= 0: xtc[xc[i]] = i
        if yc[i] >= 0: ytc[yc[i]] = i
    rng = np.random.default_rng(20 + k)
    ins = []
    for cols in (fc, xtc, fc, ytc):
        n = BlockMatrix.empty(cols, hfb.db).nelem
        ins.append(rng.standard_normal(n) + 1j * rng.standard_normal(n))
    want = gpu.calc_hamiltonian(*ins)
    got = gpu.calc_hamiltonian(*ins, mixed=True)
    gpu.close()
    worst = max(float(np.max(np.abs(g - w)) / np.max(np.abs(w))) for g, w in zip(got, want))
    print(f"config 4 GT K={k}: split-precision field worst relative error {worst:.2e}")
    assert worst <= 1e-5
