"""The block-GEMM task tables of the GPU solver, executed on the host.

pnfam_gpu_set_operator turns the quadrant products of the reference
(triprod_bbm, pnfam_solver.f90:144-166: dR_sp = W1 dR_qp W2^T and
dH_qp = W1^T dH_sp W2 with the stored signs and transposes of :300-363) into
lists of block GEMMs that the CUDA kernels run.  ``pnfam_gpu_task_tables``
returns those lists without a device; this test executes them with numpy, plane
by plane exactly as k_gemm does (C = sum alpha[plane] op(A) op(B)), and compares
the result with the oracle's ``triprod_bbm`` on random quadrants -- for the
zero-temperature quadrants X, Y and for the statistical FAM's P and Q.
"""
import numpy as np
import pytest

from golden_cases import case_for
from oracle.fam_oracle import BBM, FAMOracle, triprod_bbm
from pynfam_gb300.blockmatrix import BlockMatrix

B_UP, B_VP, B_UN, B_VN, B_STATE, B_T, B_RSP, B_HSP, B_HQP = range(9)


def _run(records, bufs, plane):
    """Execute one task list on the host (one plane)."""
    for r in records:
        M, N, K, nterm, cbuf, coff, ldc = (int(x) for x in r[:7])
        acc = np.zeros((M, N))
        for i in range(nterm):
            q = r[7 + 10 * i: 17 + 10 * i]
            abuf, aoff, lda, tA, bbuf, boff, ldb, tB = (int(x) for x in q[:8])
            alpha = q[8 + plane]
            A = bufs[abuf][plane] if isinstance(bufs[abuf], list) else bufs[abuf]
            Bm = bufs[bbuf][plane] if isinstance(bufs[bbuf], list) else bufs[bbuf]
            # k_gemm reads op(A)[m, k] = A[m + k lda] (or A[k + m lda] transposed), op(B) alike
            if tA:
                a = A[aoff:aoff + lda * M].reshape(lda, M, order="F")[:K, :].T
            else:
                a = A[aoff:aoff + lda * K].reshape(lda, K, order="F")[:M, :]
            if tB:
                b = Bm[boff:boff + ldb * K].reshape(ldb, K, order="F")[:N, :].T
            else:
                b = Bm[boff:boff + ldb * N].reshape(ldb, N, order="F")[:K, :]
            acc += alpha * (a @ b)
        C = bufs[cbuf][plane]
        for col in range(N):
            C[coff + col * ldc: coff + col * ldc + M] = acc[:, col]


def _flat_u(blocks):
    return np.concatenate([np.asarray(b, dtype=np.float64).reshape(-1, order="F") for b in blocks])


@pytest.mark.parametrize("case,op,idx,statistical,bminus", [
    ("S40", "GT-K0", 0, False, True), ("S40", "GT-K1", 0, True, True), ("S40", "RS1-K1", 0, True, True),
    ("Kr116", "P-K0", 0, True, True), ("S40", "GT-K1", 0, True, False), ("S40", "RS2-K2", 0, False, False),
    ("synthetic12", "GT-K1", 0, True, True)])
def test_task_tables_match_oracle_products(case, op, idx, statistical, bminus):
    import copy
    from pynfam_gb300 import _lib, build
    build.build()
    if case == "synthetic12":
        # Omega-only blocks up to 91 (N_sh = 12): the multi-tile block shapes
        import os
        from golden_cases import GOLDEN, golden, namelist_for
        from pynfam_gb300.pnfam_setup import setup_case
        from pynfam_gb300.synthetic import bogoliubov_nucleus
        hs = bogoliubov_nucleus(os.path.join(GOLDEN, "Gd162.hel"), 12, seed=1, parity=False)
        nml = namelist_for("Gd162", golden("Gd162")["operators"][op][0])
        nml["interaction"]["require_self_consistency"] = False
        c = setup_case(nml, None, hfb=hs)
    else:
        c, _ = case_for(case, op, idx)
    h = c.hfb
    c.F = copy.copy(c.F)
    c.F.beta_minus = bminus
    rng = np.random.default_rng(7)
    occ = (np.zeros(h.dqp), np.zeros(h.dqp)) if statistical else None
    orc = FAMOracle(h, c.couplings, c.F, c.G, occupations=occ)
    quads = orc.quads
    cols = {q: orc.Fqp.q[q].cols for q in quads}
    db = h.db
    tabs = [_lib.task_tables(db, h.num_spin_up, c.F.mat.cols, bminus, statistical, st) for st in range(4)]
    nxy, scratch = tabs[0][1], tabs[0][2]
    assert nxy == c.F.mat.nelem and scratch == (16 if statistical else 8) * nxy
    nq = len(quads)
    # random QP quadrants in the stored layout [X, Y, P, Q], Re and Im planes
    R = {q: [None if k < 0 else rng.standard_normal((db[i], db[k])) + 1j * rng.standard_normal((db[i], db[k]))
             for i, k in enumerate(cols[q])] for q in quads}
    order = (12, 21, 11, 22)[:nq]
    state = [np.concatenate([_flat_u([b.real if pl == 0 else b.imag for b in R[q] if b is not None]) for q in order])
             for pl in (0, 1)]
    ground = {B_UP: _flat_u(h.Up), B_VP: _flat_u(h.Vp), B_UN: _flat_u(h.Un), B_VN: _flat_u(h.Vn)}
    bufs = dict(ground)
    bufs[B_STATE] = state
    bufs[B_T] = [np.zeros(scratch), np.zeros(scratch)]
    bufs[B_RSP] = [np.zeros(4 * nxy), np.zeros(4 * nxy)]
    bufs[B_HSP] = [np.zeros(4 * nxy), np.zeros(4 * nxy)]
    bufs[B_HQP] = [np.zeros(nq * nxy), np.zeros(nq * nxy)]
    for pl in (0, 1):
        _run(tabs[0][0], bufs, pl)
        _run(tabs[1][0], bufs, pl)
    # the oracle's dR_sp (stored quadrants rho_pn, kappa+, kappa-, rho_np)
    mkq = lambda q, part: BlockMatrix(cols[q], [None if b is None else getattr(b, part).copy() for b in R[q]])
    sp = {}
    for part, im in (("real", False), ("imag", True)):
        dRq = BBM(q={q: (mkq(q, part) if q in R else None) for q in (11, 12, 21, 22)},
                  s={11: 1.0, 12: 1.0, 21: -1.0, 22: -1.0}, imag=im)
        abc = BBM(q={11: True, 12: True, 21: True, 22: True},
                  s={11: 1.0, 12: -1.0, 21: 1.0 if not im else -1.0, 22: -1.0},
                  t={11: "n", 12: "t", 21: "t", 22: "t"}, imag=im)
        sp[part] = triprod_bbm("n", orc.W1, "n", dRq, "t", orc.W2, abc, h.nb, db)
    for pl, part in ((0, "real"), (1, "imag")):
        want = np.concatenate([sp[part].q[q].flatten() for q in (11, 12, 21, 22)])
        got = bufs[B_RSP][pl]
        np.testing.assert_allclose(got, want, rtol=0, atol=1e-12 * np.max(np.abs(want)))
    # K2: random SP fields in the solver's layout -> QP quadrants, against the oracle
    hcols = {11: c.F.mat.cols, 12: cols[12], 21: cols[21], 22: c.F.mat.cols}
    Hs = {q: [None if k < 0 else rng.standard_normal((db[i], db[k])) for i, k in enumerate(hcols[q])]
          for q in (11, 12, 21, 22)}
    Hi = {q: [None if k < 0 else rng.standard_normal((db[i], db[k])) for i, k in enumerate(hcols[q])]
          for q in (11, 12, 21, 22)}
    bufs[B_HSP] = [np.concatenate([_flat_u([b for b in H[q] if b is not None]) for q in (11, 12, 21, 22)])
                   for H in (Hs, Hi)]
    bufs[B_T] = [np.zeros(scratch), np.zeros(scratch)]
    for pl in (0, 1):
        _run(tabs[2][0], bufs, pl)
        _run(tabs[3][0], bufs, pl)
    d = True if statistical else None
    for pl, (H, im) in enumerate(((Hs, False), (Hi, True))):
        Hb = BBM(q={q: BlockMatrix(np.asarray(hcols[q]), list(H[q])) for q in (11, 12, 21, 22)},
                 s={11: 1.0, 12: 1.0, 21: 1.0 if im else -1.0, 22: -1.0}, t={11: "n", 12: "n", 21: "n", 22: "t"},
                 imag=im)
        qp = BBM(q={11: d, 12: True, 21: True, 22: d}, s={11: 1.0, 12: 1.0, 21: -1.0, 22: -1.0}, imag=im)
        Hq = triprod_bbm("t", orc.W1, "n", Hb, "n", orc.W2, qp, h.nb, db)
        want = np.concatenate([Hq.q[q].flatten() for q in order])
        np.testing.assert_allclose(bufs[B_HQP][pl], want, rtol=0, atol=1e-12 * np.max(np.abs(want)))
