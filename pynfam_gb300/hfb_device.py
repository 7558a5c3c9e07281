"""The HFB reconstruction's arithmetic on the GPU.

``load_hfb_solution(path, device=True)`` rebuilds the ground state with the four
kernels of ``csrc/hfb.cuh`` in place of the host numpy steps: the basis functions on
the mesh (gaupol), the HFB matrices of every block (gamdel), the per-block
eigensolves inside the particle-number loop (hfbdiag's DSYEVR; batched cyclic Jacobi,
one launch for all blocks of an isospin per step) and the local densities (DENSIT).
The particle-number loop (ALambda) and the TR doubling / spin sort / pairing window
are the host code of ``hfb_solution``.  There is no CPU path here: without the CUDA
library or a GPU the calls raise.
"""
from __future__ import annotations

import ctypes as C
import time

import numpy as np

from . import _lib

# wall seconds spent in each step's library call (read by the benchmark)
TIMES = {"basis": 0.0, "matrices": 0.0, "eigen": 0.0, "eigen_calls": 0, "densities": 0.0}


def _timed(key, fn, *args):
    t0 = time.perf_counter()
    rc = fn(*args)
    TIMES[key] += time.perf_counter() - t0
    return rc

FIELDS = ("v", "vhb", "vr", "vz", "vd", "vs", "vSFIZ", "vSZFI", "vSFIR", "vSRFI", "dv")


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def basis_functions(h):
    """(qhla, fi1r, fi1z, fi2d), each [nt, nghl], of the basis of ``h`` on its mesh."""
    lib = _lib.load()
    nt, nghl = len(h.nr), h.ngh * h.ngl
    out = np.empty(4 * nt * nghl)
    xh, wh, xl, wl = _f64(h.xh), _f64(h.wh), _f64(h.xl), _f64(h.wl)
    nr, nz, nl = _i32(h.nr), _i32(h.nz), _i32(h.nl)
    _lib.check(_timed("basis", lib.pnfam_gpu_hfb_basis, h.ngh, h.ngl, _lib.dptr(xh), _lib.dptr(wh), _lib.dptr(xl), _lib.dptr(wl),
                                       float(h.bz), float(h.bp), nt, _lib.iptr(nr), _lib.iptr(nz), _lib.iptr(nl),
                                       _lib.dptr(out)))
    q = out.reshape(4, nt, nghl)
    return q[0].copy(), q[1].copy(), q[2].copy(), q[3].copy()


def _basis_stack(mb):
    return _f64(np.stack([mb.qhla, mb.fi1r, mb.fi1z, mb.fi2d]))


def hfb_matrices(h, mb):
    """{'n': [(h, Delta) per block], 'p': [...]}, as ``hfb_solution.hfb_matrices``."""
    lib = _lib.load()
    bs = _i32(h.ID)
    nghl = h.ngh * h.ngl
    fields = _f64(np.stack([np.stack([h.fields[t][k] for k in FIELDS]) for t in ("n", "p")]))
    tot = int(4 * np.sum(np.asarray(h.ID, dtype=np.int64) ** 2))
    out = np.empty(tot)
    basis = _basis_stack(mb)
    _lib.check(_timed("matrices", lib.pnfam_gpu_hfb_matrices, len(bs), _lib.iptr(bs), nghl, _lib.iptr(_i32(h.ns)), _lib.dptr(basis),
                                          _lib.dptr(_f64(mb.y)), _lib.dptr(_f64(mb.xlam)), _lib.dptr(_f64(mb.xlap)),
                                          _lib.dptr(fields), _lib.dptr(out)))
    res = {"n": [], "p": []}
    o = 0
    for nd in h.ID:
        nd = int(nd)
        for t in ("n", "p"):
            hm = out[o:o + nd * nd].reshape(nd, nd).copy(); o += nd * nd
            dm = out[o:o + nd * nd].reshape(nd, nd).copy(); o += nd * nd
            res[t].append((hm, dm))
    return res


def eigh_batch(mats, start=None, sweeps=None):
    """[(w ascending, eigenvectors as columns)] of real symmetric matrices, one GPU
    launch (cyclic Jacobi).  ``start``: orthogonal starting matrices (eigenvectors of
    nearby matrices); ``sweeps``: a list that receives the Jacobi sweeps used."""
    lib = _lib.load()
    dims = _i32([m.shape[0] for m in mats])
    a = _f64(np.concatenate([np.asarray(m, dtype=np.float64).reshape(-1) for m in mats]))
    v0 = _f64(np.concatenate([np.asarray(m, dtype=np.float64).reshape(-1) for m in start])) if start else None
    w = np.empty(int(dims.sum()))
    v = np.empty(a.size)
    sw = np.zeros(len(mats), dtype=np.int32)
    TIMES["eigen_calls"] += 1
    _lib.check(_timed("eigen", lib.pnfam_gpu_sym_eigen, len(mats), _lib.iptr(dims), _lib.dptr(a), _lib.dptr(v0) if start else None,
                                       _lib.dptr(w), _lib.dptr(v), _lib.iptr(sw)))
    if sweeps is not None:
        sweeps.extend(int(x) for x in sw)
    out, ow, ov = [], 0, 0
    for n in dims:
        n = int(n)
        out.append((w[ow:ow + n].copy(), v[ov:ov + n * n].reshape(n, n).copy()))
        ow += n
        ov += n * n
    return out


def eigh_chain():
    """An eigensolver for the steps of one particle-number loop: every call after the
    first starts from the eigenvectors of the previous call (the matrices change only
    by the shift of the Fermi energy), which cuts the Jacobi sweeps."""
    prev = {}

    def eigh(mats):
        key = tuple(m.shape[0] for m in mats)
        res = eigh_batch(mats, prev.get(key))
        prev[key] = [v for _, v in res]
        return res
    return eigh


def local_densities(h, mb, qp, tz):
    """(rho, tau, Laplacian rho) of one isospin, as ``hfb_solution.local_densities``."""
    lib = _lib.load()
    bs = _i32(h.ID)
    nghl = h.ngh * h.ngl
    thermal = qp.fwin is not None
    Ws, Us, fs = [], [], []
    for ib, nd in enumerate(h.ID):
        act = qp.active[ib]
        Ws.append(np.where(act[None, :], qp.V[ib], 0.0).reshape(-1))
        if thermal:
            Us.append(np.where(act[None, :], qp.U[ib], 0.0).reshape(-1))
            f = np.zeros(int(nd))
            f[act] = qp.fwin[ib]
            fs.append(f)
    W = _f64(np.concatenate(Ws))
    U = _f64(np.concatenate(Us)) if thermal else None
    f = _f64(np.concatenate(fs)) if thermal else None
    out = np.empty(3 * nghl)
    _lib.check(_timed("densities", lib.pnfam_gpu_hfb_densities, len(bs), _lib.iptr(bs), nghl, _lib.iptr(_i32(h.ns)),
                                           _lib.dptr(_basis_stack(mb)), _lib.dptr(_f64(mb.y)),
                                           _lib.dptr(_f64(mb.xlam)), _lib.dptr(_f64(mb.xlap)), _lib.dptr(W),
                                           _lib.dptr(U) if thermal else None, _lib.dptr(f) if thermal else None,
                                           _lib.dptr(out)))
    tro, ttau, tdro = out.reshape(3, nghl)
    s = 2.0 * tro.sum()
    wgt = mb.wdcori * (2.0 * tz / s)
    return tro * wgt, ttau * wgt, tdro * (2.0 * wgt)
