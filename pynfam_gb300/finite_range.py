"""The finite-range two-body-current field on the GPU.

``effective_2bc_extfield`` (pnfam_extfield_2bc.f90:26-915) contracts the Yukawa
part of the axial two-body current with the ground-state density matrices once
per operator; the reference caches the result, with the LECs stripped, in
``<fam_output_filename>.tbc`` (pnfam_storage.f90:488-560) because it takes hours
on the CPU at N_sh = 16.  ``gamma_pieces`` computes the same six pieces with
``pnfam_gpu_2bc_field`` (csrc/tbc.cuh): the host prepares the 1D Gaussian tables
and the basis bookkeeping, two kernels do the contraction.  There is no CPU path:
without the CUDA library or a GPU the call raises.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib

PIECES = ("c3d", "c3e", "c4d", "c4e", "cpd", "cpe")


def input_struct(hfb, F, use_p: bool):
    """The ``pnfam_2bc_input_t`` of a ground state and an operator (HFBTHO's state
    order and block sizes from the ``.hel``, the density matrices rk, the operator's
    block structure on the doubled basis).  Returns (struct, arrays kept alive)."""
    h = hfb.hel
    i32 = lambda a: np.ascontiguousarray(a, dtype=np.int32)
    keep = {
        "bs": i32(h.ID), "nz": i32(h.nz), "nr": i32(h.nr), "nl": i32(h.nl), "ns": i32(h.ns),
        "rkn": np.ascontiguousarray(np.concatenate([r.reshape(-1, order="F") for r in hfb.density_matrices("n")])),
        "rkp": np.ascontiguousarray(np.concatenate([r.reshape(-1, order="F") for r in hfb.density_matrices("p")])),
        "cols": i32(F.mat.cols),
        "offs": np.ascontiguousarray(F.mat.offsets(), dtype=np.int64),
    }
    s = _lib.TwoBodyInput()
    s.ntx, s.nbx = len(h.nz), len(h.ID)
    s.block_size, s.nz, s.nr, s.nl, s.ns = (_lib.iptr(keep[k]) for k in ("bs", "nz", "nr", "nl", "ns"))
    s.bz, s.bp = float(h.bz), float(h.bp)
    s.rk_n, s.rk_p = _lib.dptr(keep["rkn"]), _lib.dptr(keep["rkp"])
    s.K, s.beta_minus, s.use_p = int(F.k), int(bool(F.beta_minus)), int(bool(use_p))
    s.op_cols = _lib.iptr(keep["cols"])
    s.op_offsets = keep["offs"].ctypes.data_as(C.POINTER(C.c_longlong))
    s.nxy = F.mat.nelem
    return s, keep


def gamma_pieces(hfb, F, use_p: bool = False, stats: dict = None) -> dict:
    """{c3d, c3e, c4d, c4e, cpd, cpe: [nxy]} of the operator ``F`` (GT, K = F.k) on the
    GPU, LEC-stripped as in the ``.tbc`` file.  ``stats`` (optional) receives the
    host set-up and the two kernels' times in ms and the problem sizes."""
    lib = _lib.load()
    s, keep = input_struct(hfb, F, use_p)
    out = np.zeros(6 * s.nxy)
    st = np.zeros(6)
    _lib.check(lib.pnfam_gpu_2bc_field(C.byref(s), _lib.dptr(out), _lib.dptr(st)))
    if stats is not None:
        stats.update(host_ms=st[0], stage1_ms=st[1], stage2_ms=st[2], terms=int(st[3]), groups=int(st[4]),
                     pairs=int(st[5]))
    out = out.reshape(6, -1)
    return {nm: out[i].copy() for i, nm in enumerate(PIECES)}
