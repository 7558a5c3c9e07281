"""The allocation-free field evaluation (pnfam_gpu_calc_hamiltonian_noalloc).

It serves callers that cannot allocate device memory through CUDA themselves:
they hand in device pointers for all inputs and outputs, and the library keeps
its intermediates in one fixed device array.  This test gives it device
buffers (allocated here by the test), calls it through the C ABI twice in a
row with different operators and inputs, and checks each result against the
context-based pnfam_gpu_calc_hamiltonian on the same inputs, at the 1e-11
relative tolerance the other field tests use.  The file is named so that
pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

from golden_cases import case_for
from pynfam_gb300.blockmatrix import BlockMatrix

pytestmark = pytest.mark.gpu

TOL = 1e-11


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
    return fc, xtc, ytc


def _random_inputs(c, seed):
    h = c.hfb
    fc, xtc, ytc = _structures(c.F, h.nb)
    rng = np.random.default_rng(seed)
    out = []
    for cols in (fc, xtc, fc, ytc):
        m = BlockMatrix.empty(cols, h.db)
        n = m.nelem
        out.append(rng.standard_normal(n) + 1j * rng.standard_normal(n))
    return out


def _bind(lib):
    from pynfam_gb300 import _lib
    dp = C.POINTER(C.c_double)
    f = lib.pnfam_gpu_calc_hamiltonian_noalloc
    f.argtypes = [C.POINTER(_lib.Basis), C.c_void_p, C.c_void_p, C.POINTER(_lib.Coupl), C.POINTER(C.c_int),
                  C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), C.c_void_p]
    f.restype = C.c_int
    return f


def test_noalloc_matches_context_entry_point():
    torch = pytest.importorskip("torch")
    from pynfam_gb300 import _lib
    from pynfam_gb300.solver import GPUSolver
    lib = _lib.load()
    f = _bind(lib)
    dev = torch.device("cuda")
    for call, (op, idx, seed) in enumerate((("GT-K0", 0, 3), ("P-K1", 2, 4))):
        c, _ = case_for("S40", op, idx)
        h = c.hfb
        ins = _random_inputs(c, seed)
        # the existing entry point (context with its own device buffers)
        ref_solver = GPUSolver(h, c.couplings)
        ref_solver.set_operator(c.F, c.G)
        want = ref_solver.calc_hamiltonian(*ins)
        ref_solver.close()
        # device buffers owned by the caller
        to_dev = lambda a: torch.tensor(np.ascontiguousarray(a, dtype=np.float64), device=dev)
        phi = to_dev(np.stack([h.wf, h.wfdr, h.wfdp, h.wfdz, h.wfd2_all]))
        wd = to_dev(h.wdcori)
        cpl = [to_dev(a) for a in (c.couplings.crho, c.couplings.cs, c.couplings.cpair, c.couplings.cspair)]
        d_in = []
        for a in ins:
            d_in += [to_dev(a.real), to_dev(a.imag)]
        d_out = [torch.full_like(d_in[k], np.nan) for k in range(8)]
        db = np.ascontiguousarray(h.db, dtype=np.int32)
        nup = np.ascontiguousarray(h.num_spin_up, dtype=np.int32)
        ns = np.ascontiguousarray(h.ns, dtype=np.int32)
        basis = _lib.Basis(h.nb, _lib.iptr(db), _lib.iptr(nup), _lib.iptr(ns), int(h.nghl))
        dcp = _lib.Coupl(*[C.cast(C.c_void_p(t.data_ptr()), C.POINTER(C.c_double)) for t in cpl],
                         (C.c_double * 12)(*c.couplings.scalars()))
        fcols = np.ascontiguousarray(c.F.mat.cols, dtype=np.int32)
        pin = (C.c_void_p * 8)(*[t.data_ptr() for t in d_in])
        pout = (C.c_void_p * 8)(*[t.data_ptr() for t in d_out])
        torch.cuda.synchronize()
        rc = f(C.byref(basis), phi.data_ptr(), wd.data_ptr(), C.byref(dcp), _lib.iptr(fcols), pin, pout, None)
        assert rc == 0, lib.pnfam_gpu_last_error()
        got = [d_out[2 * k].cpu().numpy() + 1j * d_out[2 * k + 1].cpu().numpy() for k in range(4)]
        for g, w, name in zip(got, want, ("h_pn", "Delta+", "h_np", "Delta-")):
            assert np.all(np.isfinite(g)), (call, name)
            assert np.max(np.abs(g - w)) <= TOL * np.max(np.abs(w)), (call, name)


def test_noalloc_matches_oracle():
    """The same entry point against the CPU oracle's calc_hamiltonian (the reference's
    density / meanfield / pairingfield, pnfam_hamiltonian_blas.f90:51-1262)."""
    torch = pytest.importorskip("torch")
    from oracle.fam_oracle import _Basis, calc_hamiltonian
    from pynfam_gb300 import _lib
    lib = _lib.load()
    f = _bind(lib)
    dev = torch.device("cuda")
    c, _ = case_for("S40", "RS1-K1", 0)
    h = c.hfb
    ins = _random_inputs(c, 9)
    to_dev = lambda a: torch.tensor(np.ascontiguousarray(a, dtype=np.float64), device=dev)
    phi = to_dev(np.stack([h.wf, h.wfdr, h.wfdp, h.wfdz, h.wfd2_all]))
    wd = to_dev(h.wdcori)
    cpl = [to_dev(a) for a in (c.couplings.crho, c.couplings.cs, c.couplings.cpair, c.couplings.cspair)]
    d_in = []
    for a in ins:
        d_in += [to_dev(a.real), to_dev(a.imag)]
    d_out = [torch.full_like(d_in[k], np.nan) for k in range(8)]
    db = np.ascontiguousarray(h.db, dtype=np.int32)
    nup = np.ascontiguousarray(h.num_spin_up, dtype=np.int32)
    ns = np.ascontiguousarray(h.ns, dtype=np.int32)
    basis = _lib.Basis(h.nb, _lib.iptr(db), _lib.iptr(nup), _lib.iptr(ns), int(h.nghl))
    dcp = _lib.Coupl(*[C.cast(C.c_void_p(t.data_ptr()), C.POINTER(C.c_double)) for t in cpl],
                     (C.c_double * 12)(*c.couplings.scalars()))
    fcols = np.ascontiguousarray(c.F.mat.cols, dtype=np.int32)
    pin = (C.c_void_p * 8)(*[t.data_ptr() for t in d_in])
    pout = (C.c_void_p * 8)(*[t.data_ptr() for t in d_out])
    torch.cuda.synchronize()
    rc = f(C.byref(basis), phi.data_ptr(), wd.data_ptr(), C.byref(dcp), _lib.iptr(fcols), pin, pout, None)
    assert rc == 0, lib.pnfam_gpu_last_error()
    got = [d_out[2 * k].cpu().numpy() + 1j * d_out[2 * k + 1].cpu().numpy() for k in range(4)]
    # the oracle on the same densities, in block-matrix form
    nb = h.nb
    half = nb // 2
    tr = np.array([(i + half) % nb for i in range(nb)])
    fc = np.asarray(c.F.mat.cols)
    xc = np.array([tr[fc[i]] if fc[i] >= 0 else -1 for i in range(nb)])
    yc = np.array([fc[tr[i]] for i in range(nb)])
    _, xtc, ytc = _structures(c.F, nb)

    def blocks(flat, cols):
        m = BlockMatrix.empty(cols, h.db)
        re, im = m.copy(), m.copy()
        pos = 0
        for i, b in enumerate(m.blocks):
            if b is None:
                continue
            n = b.size
            re.blocks[i] = flat[pos:pos + n].real.reshape(b.shape, order="F")
            im.blocks[i] = flat[pos:pos + n].imag.reshape(b.shape, order="F")
            pos += n
        return re, im
    args = [blocks(a, cols) for a, cols in zip(ins, (fc, xtc, fc, ytc))]
    ref = calc_hamiltonian(_Basis(h), c.couplings, *args, {"h_pn": fc, "dp": xc, "h_np": fc, "dm": yc})
    for g, key in zip(got, ("h_pn", "dp", "h_np", "dm")):
        want = np.concatenate([b.reshape(-1, order="F") for b in ref[key] if b is not None])
        assert np.max(np.abs(g - want)) <= TOL * np.max(np.abs(want)), key


def test_noalloc_rejects_oversized_basis():
    from pynfam_gb300 import _lib
    lib = _lib.load()
    f = _bind(lib)
    nb = 66
    db = np.full(nb, 1, dtype=np.int32); nup = np.ones(nb, dtype=np.int32); ns = np.ones(nb, dtype=np.int32)
    basis = _lib.Basis(nb, _lib.iptr(db), _lib.iptr(nup), _lib.iptr(ns), 400)
    dummy = np.zeros(1)
    dcp = _lib.Coupl(*[_lib.dptr(dummy)] * 4, (C.c_double * 12)())
    fcols = np.zeros(nb, dtype=np.int32)
    ptrs = (C.c_void_p * 8)(*[dummy.ctypes.data] * 8)
    rc = f(C.byref(basis), dummy.ctypes.data, dummy.ctypes.data, C.byref(dcp), _lib.iptr(fcols), ptrs, ptrs, None)
    assert rc == 1 and b"nb <= 64" in lib.pnfam_gpu_last_error()
