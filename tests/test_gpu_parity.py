"""GPU parity: the CUDA FAM solver (through the C ABI) against the reference's
recorded FP64 pnfam_main output and against the CPU oracle.

Tolerance: 1e-6 relative per Re/Im strength value (plus 1e-12 of the largest
|S| on the operator's contour, for values that are zero up to rounding).
"""
import numpy as np
import pytest

from golden_cases import case_for, count_window, golden, hfb, oracle_counts
from oracle.fam_oracle import FAMOracle, _Basis, calc_hamiltonian
from pynfam_gb300.blockmatrix import BlockMatrix

pytestmark = pytest.mark.gpu

REL = 1e-6

# two-body-current operators (GT with the cached finite-range field, GT with the DME
# exchange function, P/PS0 with the nuclear-matter and DME corrections)
TWO_BODY_OPS = [(case, op) for case in ("S40_2bc_fam", "S40_2bc_dme", "S40_2bc_ps0", "Gd162_2bc_p",
                                         "S40_2bc_p_dme", "S40_2bc_ps0_dme")
                for op in sorted(golden(case)["operators"])]
ALL_OPS = [("S40", op) for op in sorted(golden("S40")["operators"])] + \
          [("Gd162", "GT-K0"), ("Gd162", "GT-K1"), ("Kr116", "P-K0")] + TWO_BODY_OPS


@pytest.fixture(scope="module")
def solvers():
    from pynfam_gb300.solver import GPUSolver
    cache = {}

    def get(case, c):
        if case not in cache:
            cache[case] = GPUSolver(c.hfb, c.couplings)
        return cache[case]
    yield get
    for s in cache.values():
        s.close()


def _solve(gpu, c, omegas, **kw):
    s = c.nml["solver"]
    gpu.set_operator(c.F, c.G)
    return gpu.solve(omegas, max_iter=s["max_iter"], eps=s["convergence_epsilon"],
                     broyden_m=s["broyden_history_size"], quench=c.quench, **kw)


@pytest.mark.parametrize("case,op", ALL_OPS)
def test_contour_batch_matches_recorded(case, op, solvers):
    pts = golden(case)["operators"][op]
    c, _ = case_for(case, op, 0)
    gpu = solvers(case, c)
    omegas = [complex(p["namelist"]["real_eqrpa"], p["namelist"]["imag_eqrpa"]) for p in pts]
    r = _solve(gpu, c, omegas)
    labels = ["Strength"] + [g.label for g in c.G]
    scale = max(abs(complex(*p["result"]["Strength"])) for p in pts)
    worst = 0.0
    moved = 0
    counts = oracle_counts()
    for i, p in enumerate(pts):
        assert r.iters[i] >= 0, (i, r.si[i])
        want, slack = count_window(p, {"near": counts["near"], "point": counts["counts"][case][op][i]})
        assert abs(int(r.iters[i]) - want) <= slack, (i, r.iters[i], want, p["converged"], slack)
        moved += int(r.iters[i]) != p["converged"]
        for k, lab in enumerate(labels):
            want = p["result"][lab]
            for got, w in ((r.re_S[i, k], want[0]), (r.im_S[i, k], want[1])):
                err = abs(got - w)
                assert err <= REL * abs(w) + 1e-12 * scale, (i, lab, got, w)
                if abs(w) > 1e-9 * scale:
                    worst = max(worst, err / abs(w))
    print(f"{case} {op}: {len(pts)} points, worst relative error vs recorded {worst:.2e}, "
          f"{moved} converged at a different iteration")


TIGHT = 1e-12      # FP64 convergence used as the exact fixed point
MIXED_EPS = 1e-10  # convergence asked of the mixed form
SETTLE = 8         # ... with every strength value settled to 1e-8 of itself (small cross
                   # terms of a contour sit three orders below its largest strength)


@pytest.mark.parametrize("case,op", ALL_OPS)
def test_mixed_precision_contour_matches_fp64(case, op, solvers):
    """Iterative refinement (FP32 field evaluation, FP64 residual checks) against the FP64
    solution of the same equations.

    The recorded outputs stop at si < 1e-7 (absolute), which leaves them up to ~6e-5
    relative from the fixed point they iterate to (S40 P-K0), so a solver that follows a
    different trajectory can only be held to 1e-6 against the fixed point itself: here the
    FP64 form converged to 1e-12.  The mixed form is run to 1e-10 and must agree to 1e-6.
    """
    pts = golden(case)["operators"][op]
    c, _ = case_for(case, op, 0)
    gpu = solvers(case, c)
    omegas = [complex(p["namelist"]["real_eqrpa"], p["namelist"]["imag_eqrpa"]) for p in pts]
    s = c.nml["solver"]
    gpu.set_operator(c.F, c.G)
    kw = dict(broyden_m=s["broyden_history_size"], quench=c.quench)
    exact = gpu.solve(omegas, max_iter=1500, eps=TIGHT, **kw)
    assert np.all(exact.iters >= 0), exact.si
    r = gpu.solve(omegas, max_iter=1500, eps=MIXED_EPS, precision=1, settle=SETTLE, **kw)
    prof, _ = gpu.last_profile()
    assert np.all(r.iters >= 0), r.si
    scale = np.max(np.abs(exact.re_S[:, 0] + 1j * exact.im_S[:, 0]))
    worst = worst_rec = 0.0
    for i, p in enumerate(pts):
        for k in range(r.re_S.shape[1]):
            for got, w in ((r.re_S[i, k], exact.re_S[i, k]), (r.im_S[i, k], exact.im_S[i, k])):
                err = abs(got - w)
                assert err <= REL * abs(w) + 1e-12 * scale, (i, k, got, w)
                if abs(w) > 1e-9 * scale:
                    worst = max(worst, err / abs(w))
        w = complex(exact.re_S[i, 0], exact.im_S[i, 0])
        rec = complex(*p["result"]["Strength"])
        worst_rec = max(worst_rec, abs(rec - w) / max(abs(w), 1e-300))
    print(f"{case} {op} mixed: worst rel err vs FP64 fixed point {worst:.2e} (recorded output: "
          f"{worst_rec:.2e}); evaluations fp32 {prof['point_iterations_fp32']:.0f}, "
          f"fp64 {prof['point_iterations_fp64']:.0f}")


def test_history_matches_oracle(solvers):
    c, pt = case_for("S40", "P-K1", 9)
    gpu = solvers("S40", c)
    r = _solve(gpu, c, [c.omega], history=True)
    s = c.nml["solver"]
    orc = FAMOracle(c.hfb, c.couplings, c.F, c.G, quench=c.quench)
    ref = orc.solve(c.omega, max_iter=s["max_iter"], eps=s["convergence_epsilon"],
                    broyden_m=s["broyden_history_size"])
    assert r.iters[0] == ref.iter_conv
    for h in ref.history:
        it = h[0]
        g = r.hist[0, it]
        assert abs(g[0] - h[2]) <= 1e-9 * max(abs(h[2]), 1e-3)
        assert abs(g[1] - h[3]) <= 1e-9 * abs(ref.re_str[0])
        assert abs(g[2] - h[4]) <= 1e-9 * abs(ref.im_str[0]) + 1e-15
    for k in range(len(ref.re_str)):
        assert abs(r.re_S[0, k] - ref.re_str[k]) <= 1e-10 * abs(ref.re_str[k])
        assert abs(r.im_S[0, k] - ref.im_str[k]) <= 1e-10 * abs(ref.im_str[k]) + 1e-15


def test_alone_equals_in_batch(solvers):
    pts = golden("Gd162")["operators"]["GT-K1"]
    c, _ = case_for("Gd162", "GT-K1", 0)
    gpu = solvers("Gd162", c)
    omegas = [complex(p["namelist"]["real_eqrpa"], p["namelist"]["imag_eqrpa"]) for p in pts[:12]]
    batch = _solve(gpu, c, omegas)
    for i in (0, 5, 11):
        alone = _solve(gpu, c, [omegas[i]])
        assert alone.iters[0] == batch.iters[i]
        np.testing.assert_allclose(alone.re_S[0], batch.re_S[i], rtol=1e-13, atol=0)
        np.testing.assert_allclose(alone.im_S[0], batch.im_S[i], rtol=1e-13, atol=1e-20)


def _structures(F, nb):
    half = nb // 2
    tr = np.array([(i + half) % nb for i in range(nb)])
    fc = np.asarray(F.mat.cols)
    xc = np.array([tr[fc[i]] if fc[i] >= 0 else -1 for i in range(nb)])
    yc = np.array([fc[tr[i]] for i in range(nb)])
    xtc = np.full(nb, -1); ytc = np.full(nb, -1)
    for i in range(nb):
        if xc[i] >= 0: xtc[xc[i]] = i
        if yc[i] >= 0: ytc[yc[i]] = i
    return fc, xc, yc, xtc, ytc


def test_calc_hamiltonian_plugin_matches_oracle(solvers):
    c, _ = case_for("S40", "RS1-K1", 0)
    gpu = solvers("S40", c)
    gpu.set_operator(c.F, c.G)
    h = c.hfb
    fc, xc, yc, xtc, ytc = _structures(c.F, h.nb)
    rng = np.random.default_rng(7)

    def rand(cols):
        m = BlockMatrix.empty(cols, h.db)
        re = m.copy(); im = m.copy()
        for i, b in enumerate(m.blocks):
            if b is not None:
                re.blocks[i] = rng.standard_normal(b.shape)
                im.blocks[i] = rng.standard_normal(b.shape)
        return re, im
    ins = [rand(fc), rand(xtc), rand(fc), rand(ytc)]
    got = gpu.calc_hamiltonian(*[r.flatten() + 1j * i.flatten() for r, i in ins])
    ref = calc_hamiltonian(_Basis(h), c.couplings, ins[0], ins[1], ins[2], ins[3],
                           {"h_pn": fc, "dp": xc, "h_np": fc, "dm": yc})
    for g, key, cols in zip(got, ("h_pn", "dp", "h_np", "dm"), (fc, xc, fc, yc)):
        want = np.concatenate([b.reshape(-1, order="F") for b in ref[key] if b is not None])
        assert np.max(np.abs(g - want)) <= 1e-11 * np.max(np.abs(want)), key


def test_no_residual_interaction_is_one_step(solvers):
    """quench_residual_int = 0: X = G F after one pass (converged at the next check)."""
    c, _ = case_for("S40", "GT-K0", 3)
    gpu = solvers("S40", c)
    c.nml["solver"]["quench_residual_int"] = 0.0
    r = _solve(gpu, c, [c.omega])
    orc = FAMOracle(c.hfb, c.couplings, c.F, c.G, quench=0.0)
    ref = orc.solve(c.omega, max_iter=10, eps=1e-7, broyden_m=50)
    assert ref.iter_conv == 2 and r.iters[0] == 2
    assert abs(r.re_S[0, 0] - ref.re_str[0]) <= 1e-12 * abs(ref.re_str[0])
    assert abs(r.im_S[0, 0] - ref.im_str[0]) <= 1e-12 * abs(ref.im_str[0])


def test_interrupted_iteration(solvers):
    c, _ = case_for("S40", "GT-K0", 3)
    gpu = solvers("S40", c)
    gpu.set_operator(c.F, c.G)
    r = gpu.solve([c.omega], max_iter=3, eps=1e-7, broyden_m=50, quench=1.0)
    assert r.iters[0] == -1 and r.si[0] > 1e-7


def test_error_codes(solvers):
    from pynfam_gb300 import _lib
    from pynfam_gb300.solver import GPUSolver
    c, _ = case_for("S40", "GT-K0", 0)
    fresh = GPUSolver(c.hfb, c.couplings)
    with pytest.raises(_lib.PnfamGPUError) as e:
        fresh.solve([c.omega])
    assert e.value.code == 5
    fresh.set_operator(c.F, c.G)
    with pytest.raises(_lib.PnfamGPUError) as e:
        fresh.solve([c.omega], broyden_m=65)
    assert e.value.code == 1
    fresh.close()


@pytest.fixture(scope="module")
def large_case():
    """The recorded 162Gd fields in a larger basis: blocks up to 49 (N_sh = 12),
    so every multi-tile path of the kernels is exercised."""
    from golden_cases import namelist_for
    from pynfam_gb300.pnfam_setup import setup_case
    from pynfam_gb300.synthetic import ground_state
    import os
    from golden_cases import GOLDEN
    g = ground_state(os.path.join(GOLDEN, "Gd162.hel"), 12)
    pt = golden("Gd162")["operators"]["GT-K1"][10]
    c = setup_case(namelist_for("Gd162", pt), None, hfb=g)
    return c


def test_large_basis_history_matches_oracle(large_case):
    from pynfam_gb300.solver import GPUSolver
    c = large_case
    assert int(c.hfb.db.max()) > 32
    gpu = GPUSolver(c.hfb, c.couplings)
    gpu.set_operator(c.F, c.G)
    r = gpu.solve([c.omega], max_iter=6, eps=1e-7, broyden_m=50, quench=c.quench, history=True)
    gpu.close()
    orc = FAMOracle(c.hfb, c.couplings, c.F, c.G, quench=c.quench)
    ref = orc.solve(c.omega, max_iter=6, eps=1e-7, broyden_m=50)
    assert r.iters[0] == ref.iter_conv == -1
    for h in ref.history:
        g = r.hist[0, h[0]]
        assert abs(g[0] - h[2]) <= 1e-10 * max(abs(h[2]), 1e-6), (h, g)
        assert abs(g[1] - h[3]) <= 1e-10 * max(abs(h[3]), 1e-6), (h, g)
        assert abs(g[2] - h[4]) <= 1e-10 * max(abs(h[4]), 1e-6), (h, g)


def test_large_basis_calc_hamiltonian(large_case):
    from pynfam_gb300.solver import GPUSolver
    c = large_case
    h = c.hfb
    gpu = GPUSolver(h, c.couplings)
    gpu.set_operator(c.F, c.G)
    fc, xc, yc, xtc, ytc = _structures(c.F, h.nb)
    rng = np.random.default_rng(11)

    def rand(cols):
        m = BlockMatrix.empty(cols, h.db)
        re = m.copy(); im = m.copy()
        for i, b in enumerate(m.blocks):
            if b is not None:
                re.blocks[i] = rng.standard_normal(b.shape)
                im.blocks[i] = rng.standard_normal(b.shape)
        return re, im
    ins = [rand(fc), rand(xtc), rand(fc), rand(ytc)]
    got = gpu.calc_hamiltonian(*[r.flatten() + 1j * i.flatten() for r, i in ins])
    gpu.close()
    ref = calc_hamiltonian(_Basis(h), c.couplings, ins[0], ins[1], ins[2], ins[3],
                           {"h_pn": fc, "dp": xc, "h_np": fc, "dm": yc})
    for g, key in zip(got, ("h_pn", "dp", "h_np", "dm")):
        want = np.concatenate([b.reshape(-1, order="F") for b in ref[key] if b is not None])
        assert np.max(np.abs(g - want)) <= 1e-11 * np.max(np.abs(want)), key


def _mixed_vs_fp64(c, seed):
    """pnfam_gpu_calc_hamiltonian_mixed (FP32 densities and fields, tensor-core
    projection with 3xTF32 products) against the FP64 entry point on random
    densities; returns the worst error relative to each field's largest element."""
    from pynfam_gb300.solver import GPUSolver
    h = c.hfb
    gpu = GPUSolver(h, c.couplings)
    gpu.set_operator(c.F, c.G)
    fc, xc, yc, xtc, ytc = _structures(c.F, h.nb)
    rng = np.random.default_rng(seed)
    ins = []
    for cols in (fc, xtc, fc, ytc):
        n = BlockMatrix.empty(cols, h.db).nelem
        ins.append(rng.standard_normal(n) + 1j * rng.standard_normal(n))
    want = gpu.calc_hamiltonian(*ins)
    got = gpu.calc_hamiltonian(*ins, mixed=True)
    gpu.close()
    worst = 0.0
    for g, w in zip(got, want):
        assert np.all(np.isfinite(g))
        worst = max(worst, float(np.max(np.abs(g - w)) / np.max(np.abs(w))))
    return worst


@pytest.mark.parametrize("case,op", [("S40", "RS1-K1"), ("S40", "GT-K0"), ("Kr116", "P-K0")])
def test_mixed_field_matches_fp64(case, op, monkeypatch):
    """The mixed field evaluation with the SIMT FP32 density kernel
    (PNFAM_GB300_TC_DENSITY=0 when the context is created) against the FP64 field."""
    monkeypatch.setenv("PNFAM_GB300_TC_DENSITY", "0")
    c, _ = case_for(case, op, 0)
    worst = _mixed_vs_fp64(c, 3)
    print(f"{case} {op}: mixed field worst relative error {worst:.2e}")
    assert worst <= 1e-5


@pytest.mark.parametrize("case,op", [("S40", "RS1-K1"), ("S40", "GT-K0"), ("Kr116", "P-K0"), ("Gd162", "GT-K1")])
def test_pair_gemm_field_matches_fp64(case, op, monkeypatch):
    """The mixed field evaluation through the pair-tensor GEMMs (densities and field
    projection as 3xTF32 GEMMs against the operator's pair tensor; taken for a one-point
    evaluation with PNFAM_GB300_PAIR_MIN=1 when the context is created) against the
    FP64 field."""
    monkeypatch.setenv("PNFAM_GB300_PAIR_GEMM", "1")
    monkeypatch.setenv("PNFAM_GB300_PAIR_MIN", "1")
    c, _ = case_for(case, op, 0)
    worst = _mixed_vs_fp64(c, 6)
    print(f"{case} {op}: pair-tensor GEMM field worst relative error {worst:.2e}")
    assert worst <= 1e-5


def test_large_basis_pair_gemm_field_matches_fp64(large_case, monkeypatch):
    monkeypatch.setenv("PNFAM_GB300_PAIR_GEMM", "1")
    monkeypatch.setenv("PNFAM_GB300_PAIR_MIN", "1")
    worst = _mixed_vs_fp64(large_case, 7)
    print(f"N_sh=12 162Gd GT-K1: pair-tensor GEMM field worst relative error {worst:.2e}")
    assert worst <= 1e-5


@pytest.mark.parametrize("kspan", [96, 192, 768])
def test_pair_gemm_density_task_spans_match_fp64(large_case, kspan, monkeypatch):
    """Every density task span the autotuner may choose (K chunks per CTA task, hence the
    number of partial sums the fold adds) gives the FP64 field within the FP32 tolerance
    (PNFAM_GB300_PAIR_KSPAN fixes the span when the context is created)."""
    monkeypatch.setenv("PNFAM_GB300_PAIR_GEMM", "1")
    monkeypatch.setenv("PNFAM_GB300_PAIR_MIN", "1")
    monkeypatch.setenv("PNFAM_GB300_PAIR_KSPAN", str(kspan))
    worst = _mixed_vs_fp64(large_case, 8)
    print(f"N_sh=12 162Gd GT-K1, density span {kspan}: pair-tensor GEMM field worst relative error {worst:.2e}")
    assert worst <= 1e-5


def test_pair_gemm_and_kernel_paths_agree_in_a_batch(monkeypatch):
    """A contour solved in the mixed form with the pair-tensor GEMMs (the default for
    evaluations of 4 or more points) and with the projection and density kernels
    (PNFAM_GB300_PAIR_GEMM=0): the same fixed point within 1e-6."""
    from pynfam_gb300.solver import GPUSolver
    pts = golden("S40")["operators"]["RS1-K1"]
    c, _ = case_for("S40", "RS1-K1", 0)
    omegas = [complex(p["namelist"]["real_eqrpa"], p["namelist"]["imag_eqrpa"]) for p in pts]
    kw = dict(broyden_m=c.nml["solver"]["broyden_history_size"], quench=c.quench, max_iter=1500,
              eps=MIXED_EPS, precision=1, settle=SETTLE)
    res = {}
    for mode in ("1", "0"):
        monkeypatch.setenv("PNFAM_GB300_PAIR_GEMM", mode)
        gpu = GPUSolver(c.hfb, c.couplings)
        gpu.set_operator(c.F, c.G)
        res[mode] = gpu.solve(omegas, **kw)
        gpu.close()
    a, b = res["1"], res["0"]
    assert np.all(a.iters >= 0) and np.all(b.iters >= 0)
    scale = np.max(np.abs(b.re_S[:, 0] + 1j * b.im_S[:, 0]))
    for x, y in ((a.re_S, b.re_S), (a.im_S, b.im_S)):
        assert np.all(np.abs(x - y) <= REL * np.abs(y) + 1e-12 * scale)


def test_large_basis_mixed_field_matches_fp64(large_case):
    worst = _mixed_vs_fp64(large_case, 4)
    print(f"N_sh=12 162Gd GT-K1: mixed field worst relative error {worst:.2e}")
    assert worst <= 1e-5


def test_tensor_core_density_matches_fp64(monkeypatch, large_case):
    """The tensor-core density kernel (the default; PNFAM_GB300_TC_DENSITY=0 when the
    context is created selects the SIMT kernel) in the mixed field evaluation, against
    the FP64 field."""
    monkeypatch.setenv("PNFAM_GB300_TC_DENSITY", "1")
    cases = [(f"{case} {op}", case_for(case, op, 0)[0]) for case, op in (("S40", "RS1-K1"), ("Kr116", "P-K0"))]
    for name, c in cases + [("N_sh=12 162Gd GT-K1", large_case)]:
        worst = _mixed_vs_fp64(c, 5)
        print(f"{name}: mixed field (tensor-core densities) worst relative error {worst:.2e}")
        assert worst <= 1e-5


@pytest.mark.parametrize("case,op", [("S40", "P-K0"), ("Gd162", "GT-K1")])
def test_tensor_core_density_mixed_solve(monkeypatch, case, op):
    """The mixed form with tensor-core densities reaches the FP64 fixed point (1e-6)."""
    from pynfam_gb300.solver import GPUSolver
    monkeypatch.setenv("PNFAM_GB300_TC_DENSITY", "1")
    pts = golden(case)["operators"][op]
    c, _ = case_for(case, op, 0)
    omegas = [complex(p["namelist"]["real_eqrpa"], p["namelist"]["imag_eqrpa"]) for p in pts]
    kw = dict(broyden_m=c.nml["solver"]["broyden_history_size"], quench=c.quench)
    gpu = GPUSolver(c.hfb, c.couplings)
    gpu.set_operator(c.F, c.G)
    exact = gpu.solve(omegas, max_iter=1500, eps=TIGHT, **kw)
    r = gpu.solve(omegas, max_iter=1500, eps=MIXED_EPS, precision=1, settle=SETTLE, **kw)
    gpu.close()
    assert np.all(exact.iters >= 0) and np.all(r.iters >= 0), r.si
    w = exact.re_S[:, 0] + 1j * exact.im_S[:, 0]
    g = r.re_S[:, 0] + 1j * r.im_S[:, 0]
    worst = float(np.max(np.abs(g - w) / np.abs(w)))
    print(f"{case} {op} mixed form, tensor-core densities: worst rel err vs FP64 fixed point {worst:.2e}")
    assert worst <= REL


# ---------------------------------------------------------------------------
# statistical FAM (finite temperature, EFA blocking): quadrants P and Q
# ---------------------------------------------------------------------------
def _stat_cases():
    from pynfam_gb300.statistics import blocking_occupations, thermal_occupations
    out = []
    for case, op, idx, kind in (("S40", "GT-K0", 5, 1.0), ("S40", "RS1-K1", 3, 2.0), ("Kr116", "P-K0", 4, "block")):
        c, _ = case_for(case, op, idx)
        if kind == "block":
            # one neutron quasiparticle inside the pairing window blocked (EFA)
            k = int(np.flatnonzero(c.hfb.En > 0)[3])
            occ = blocking_occupations(c.hfb, iqp_n=k)
        else:
            occ = thermal_occupations(c.hfb, kind)
        out.append((f"{case} {op} {kind}", c, occ))
    return out


def test_statistical_fam_matches_oracle():
    """GPU statistical FAM against the oracle: the whole iteration history (1e-9)
    and the final strength and cross terms (1e-10)."""
    from pynfam_gb300.solver import GPUSolver
    for name, c, occ in _stat_cases():
        gpu = GPUSolver(c.hfb, c.couplings, occupations=occ)
        gpu.set_operator(c.F, c.G)
        s = c.nml["solver"]
        r = gpu.solve([c.omega], max_iter=s["max_iter"], eps=s["convergence_epsilon"],
                      broyden_m=s["broyden_history_size"], quench=c.quench, history=True)
        gpu.close()
        orc = FAMOracle(c.hfb, c.couplings, c.F, c.G, quench=c.quench, occupations=occ)
        ref = orc.solve(c.omega, max_iter=s["max_iter"], eps=s["convergence_epsilon"],
                        broyden_m=s["broyden_history_size"])
        assert ref.iter_conv > 0 and r.iters[0] == ref.iter_conv, (name, r.iters[0], ref.iter_conv)
        for h in ref.history:
            g = r.hist[0, h[0]]
            assert abs(g[0] - h[2]) <= 1e-9 * max(abs(h[2]), 1e-3), (name, h, g)
            assert abs(g[1] - h[3]) <= 1e-9 * abs(ref.re_str[0]), (name, h, g)
            assert abs(g[2] - h[4]) <= 1e-9 * abs(ref.im_str[0]) + 1e-15, (name, h, g)
        for k in range(len(ref.re_str)):
            assert abs(r.re_S[0, k] - ref.re_str[k]) <= 1e-10 * abs(ref.re_str[k]) + 1e-15, (name, k)
            assert abs(r.im_S[0, k] - ref.im_str[k]) <= 1e-10 * abs(ref.im_str[k]) + 1e-15, (name, k)
        print(f"{name}: statistical FAM, {ref.iter_conv} iterations, S = {r.re_S[0, 0]:.12e} "
              f"{r.im_S[0, 0]:+.12e}i")


def test_statistical_fam_zero_occupations_is_ground_state_form(solvers):
    """All occupations zero: P = Q = 0 and the T factors are 1, so a contour solved in the
    statistical form equals the zero-temperature form (rounding level)."""
    from pynfam_gb300 import _lib
    from pynfam_gb300.solver import GPUSolver
    pts = golden("S40")["operators"]["GT-K1"][:6]
    c, _ = case_for("S40", "GT-K1", 0)
    omegas = [complex(p["namelist"]["real_eqrpa"], p["namelist"]["imag_eqrpa"]) for p in pts]
    r0 = _solve(solvers("S40", c), c, omegas)
    z = np.zeros(c.hfb.dqp)
    gpu = GPUSolver(c.hfb, c.couplings, occupations=(z, z))
    gpu.set_operator(c.F, c.G)
    r1 = _solve(gpu, c, omegas)
    assert np.array_equal(r0.iters, r1.iters)
    np.testing.assert_allclose(r1.re_S, r0.re_S, rtol=1e-11, atol=1e-15)
    np.testing.assert_allclose(r1.im_S, r0.im_S, rtol=1e-11, atol=1e-15)
    # clearing the occupations needs the operator again
    gpu.set_occupations(None, None)
    with pytest.raises(_lib.PnfamGPUError) as e:
        gpu.solve(omegas[:1])
    assert e.value.code == 5
    gpu.close()


@pytest.mark.parametrize("idx", [0, 1, 2])
def test_statistical_mixed_form_matches_fp64_fixed_point(idx):
    """The statistical FAM in the mixed form (P and Q quadrants in the FP32 increment
    evaluations, the 8-part state in pair-arithmetic Broyden, FP64 anchors): every
    converged point of a contour within 1e-6 of the FP64 statistical fixed point
    (converged to 1e-12), per Re/Im value of the strength and each cross term."""
    from pynfam_gb300.solver import GPUSolver
    name, c, occ = _stat_cases()[idx]
    case, op = name.split()[:2]
    pts = golden(case)["operators"][op][:12]
    omegas = [complex(p["namelist"]["real_eqrpa"], p["namelist"]["imag_eqrpa"]) for p in pts]
    s = c.nml["solver"]
    gpu = GPUSolver(c.hfb, c.couplings, occupations=occ)
    gpu.set_operator(c.F, c.G)
    kw = dict(max_iter=300, broyden_m=s["broyden_history_size"], quench=c.quench)
    ref = gpu.solve(omegas, eps=TIGHT, **kw)
    mix = gpu.solve(omegas, eps=MIXED_EPS, precision=1, settle=SETTLE, **kw)
    gpu.close()
    worst, n = 0.0, 0
    for i in range(len(omegas)):
        assert ref.iters[i] > 0, (name, i)
        if mix.iters[i] < 0:
            continue
        n += 1
        for k in range(ref.re_S.shape[1]):
            for got, want in ((mix.re_S[i, k], ref.re_S[i, k]), (mix.im_S[i, k], ref.im_S[i, k])):
                err = abs(got - want)
                assert err <= REL * abs(want) + 1e-12 * np.max(np.abs(ref.re_S[:, 0])), (name, i, k, got, want)
                if abs(want) > 1e-9:
                    worst = max(worst, err / abs(want))
    assert n >= len(omegas) - 1, (name, n)
    print(f"{name}: statistical mixed form, {n} of {len(omegas)} points converged, worst rel err vs FP64 "
          f"fixed point {worst:.2e}")
