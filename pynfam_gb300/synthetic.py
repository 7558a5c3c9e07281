"""Larger-basis ground states built from a recorded HFBTHO solution.

No HFBTHO run at N_sh = 16 is available, so large workloads are built from a
recorded ground state by re-diagonalising its mean and pairing fields (stored
on the quadrature mesh in the .hel file) in a larger axial harmonic-oscillator
basis on the same mesh.  The quasiparticle solution then has the block
structure of a full N_sh basis and is close to self-consistent (the fields
come from a converged calculation), so the FAM iteration behaves like a
production run.

The basis follows HFBTHO's state ordering (hfbtho_solver.f90:3246-3445
``base``, reflection-symmetric case): blocks by Omega = k - 1/2 and parity,
inside a block the loops nr, nz, Lambda, spin.  With equal oscillator lengths
and no state-number cut the energy cut-off reduces to nz + 2 nr + Lambda <= N_sh.
"""
from __future__ import annotations

import copy

import numpy as np

from .hel import HelData


def hfbtho_basis(n00: int, parity: bool = True):
    """(ID, nr, nz, nl, ns) of the full N_sh = n00 basis, Omega > 0 half."""
    ID, nr, nz, nl, ns = [], [], [], [], []
    for k in range(1, n00 + 2):
        la, le = k - 1, min(n00, k)
        groups = (1, 2) if parity else (None,)
        start_all = len(nr)
        for ip in groups:
            start = len(nr)
            for ir in range(0, n00 // 2 + 1):
                for iz in range(0, n00 + 1):
                    for il in range(la, le + 1):
                        for is_ in (1, -1):
                            if iz + 2 * ir + il > n00:
                                continue
                            if il + (is_ + 1) // 2 != k:
                                continue
                            if ip is not None and (iz + il) % 2 != ip - 1:
                                continue
                            nr.append(ir); nz.append(iz); nl.append(il); ns.append(is_)
            if ip is not None and len(nr) > start:
                ID.append(len(nr) - start)
        if not parity and len(nr) > start_all:
            ID.append(len(nr) - start_all)
    a = lambda x: np.asarray(x, dtype=np.int64)
    return a(ID), a(nr), a(nz), a(nl), a(ns)


def extend_basis(h: HelData, n00: int) -> HelData:
    """Copy of ``h`` with the basis replaced by the full N_sh = n00 basis."""
    if abs(h.bz - h.bp) > 1e-12:
        raise ValueError("basis extension needs a spherical oscillator basis (bz == bp)")
    g = copy.copy(h)
    g.ID, g.nr, g.nz, g.nl, g.ns = hfbtho_basis(n00, parity=True)
    g.n00 = n00
    g.nb = len(g.ID)
    g.nt = int(g.ID.sum())
    return g


def ground_state(hel_path: str, n00: int):
    """HFBSolution of the recorded fields in the N_sh = n00 basis."""
    from .hel import read_hel
    from .hfb_solution import load_hfb_solution
    h = read_hel(hel_path)
    if n00 != h.n00:
        h = extend_basis(h, n00)
    return load_hfb_solution(h)


def bogoliubov_nucleus(hel_path: str, n00: int, seed: int, parity: bool = False):
    """A synthetic Bogoliubov ground state in the full N_sh = n00 basis: per block
    and isospin, U = A diag(u), V = B diag(v) with A, B the Q factors of Gaussian
    matrices, v_k^2 = 1/(1 + exp((e_k - lambda)/0.8 MeV)), e_k uniform in
    [-40, 40] MeV, lambda = -8 MeV and E_k = sqrt((e_k - lambda)^2 + 1.2^2) MeV.
    Neutrons use `seed`, protons `seed + 10**6`; blocks are drawn in block order.
    The mesh, the oscillator lengths and Z, N come from the recorded ``.hel``
    (the couplings follow from the synthetic densities).  ``parity=False`` gives
    Omega-only blocks."""
    from .hel import read_hel
    from .hfb_solution import QPSolution, assemble, build_mesh_basis
    h = read_hel(hel_path)
    if abs(h.bz - h.bp) > 1e-12:
        raise ValueError("the synthetic basis needs a spherical oscillator basis (bz == bp)")
    g = copy.copy(h)
    g.ID, g.nr, g.nz, g.nl, g.ns = hfbtho_basis(n00, parity=parity)
    g.n00 = n00
    g.nb = len(g.ID)
    g.nt = int(g.ID.sum())
    mb = build_mesh_basis(g)
    lam = -8.0

    def draw(rng):
        E, U, V, act = [], [], [], []
        for d in g.ID:
            d = int(d)
            A = np.linalg.qr(rng.standard_normal((d, d)))[0]
            Bm = np.linalg.qr(rng.standard_normal((d, d)))[0]
            e = rng.uniform(-40.0, 40.0, d)
            v2 = 1.0 / (1.0 + np.exp((e - lam) / 0.8))
            U.append(A * np.sqrt(1.0 - v2)[None, :])
            V.append(Bm * np.sqrt(v2)[None, :])
            E.append(np.sqrt((e - lam) ** 2 + 1.2 ** 2))
            act.append(np.ones(d, dtype=bool))
        return QPSolution(E, U, V, act, lam)

    qpn = draw(np.random.default_rng(seed))
    qpp = draw(np.random.default_rng(seed + 10 ** 6))
    return assemble(g, mb, qpn, qpp)
