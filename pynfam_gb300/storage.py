"""Restart storage of a FAM point: ``<fam_output_filename>.bin``.

Follows pnfam_storage.f90: with ``use_fam_storage`` = 1 or -1 in ``&general`` a
run starts from the Broyden vector stored by an earlier run of the same point
(``fam_io(1)``, :62-116, ``read_data`` :218-405); with -1 it also stores its own
final vector (``fam_io(2)``, :117-136, ``write_data`` :407-486).  The file is a
Fortran unformatted sequential file (4-byte little-endian record lengths before
and after each record, as gfortran writes it): a version record, then keyword
records ('hfb_soln', 'stat_hfb', 'interact', 'extfield', 'fam_soln') each
followed by its data records.

A stored vector is taken only if the block structure (nb, db), the operator
(name and K) and the number of FAM matrix elements (nxy) match the run; a
mismatch or a damaged file is reported in the log and the run starts from
scratch, as in the reference.  The strengths the file holds are shown at
iteration 0 either way (the reference reads them before it judges the file).
"""
from __future__ import annotations

import os
import struct
from dataclasses import dataclass

import numpy as np

VERSION_DATA = 1
HUGE = np.finfo(np.float64).max


class _Corrupted(Exception):
    def __init__(self, key):
        super().__init__(key)
        self.key = key


@dataclass
class Restart:
    """What a read gave: ``vector`` (the Broyden vector in the reference's part order,
    or None when the run starts from scratch), the stored ``si`` (1.0 from scratch)
    and the stored strength and cross terms ``s0`` (complex, None if none were read)."""
    vector: np.ndarray = None
    si: float = 1.0
    s0: np.ndarray = None


def storage_path(nml: dict, cwd: str = ".") -> str:
    """``<fam_output_filename>.bin`` in ``cwd``, or "" when the run has no output name
    (the reference then switches storage off, pnfam_setup.f90:146-153)."""
    name = str(nml["general"]["fam_output_filename"]).strip()
    return os.path.join(cwd, name + ".bin") if name else ""


def _fortran_name(s: str, n: int = 80) -> bytes:
    return str(s).encode("ascii", "replace")[:n].ljust(n)


class _Writer:
    def __init__(self):
        self.parts = []

    def rec(self, payload: bytes):
        n = struct.pack("<i", len(payload))
        self.parts += [n, payload, n]

    def ints(self, *v):
        self.rec(np.asarray(v, dtype="<i4").tobytes())

    def reals(self, *v):
        self.rec(np.asarray(v, dtype="<f8").tobytes())

    def array(self, a, dtype):
        self.rec(np.ascontiguousarray(a, dtype=dtype).tobytes())


def _records(data: bytes):
    i = 0
    while i < len(data):
        if i + 4 > len(data):
            raise _Corrupted(None)
        n = struct.unpack_from("<i", data, i)[0]
        if n < 0 or i + 8 + n > len(data) or struct.unpack_from("<i", data, i + 4 + n)[0] != n:
            raise _Corrupted(None)
        yield data[i + 4:i + 4 + n]
        i += 8 + n


def _resolved_pairing(inter: dict):
    """vpair_t0, vpair_t1 as init_interaction leaves them (pnfam_interaction.f90:151-200)."""
    out = []
    for t, old in (("vpair_t0", "vpair0"), ("vpair_t1", "vpair1")):
        v = inter.get(t)
        if v is None:
            w = inter.get(old)
            v = 0.0 if w is None else 2.0 * float(w)
        out.append(float(v))
    return out


def write_storage(path: str, case, nxy: int, si: float, re_S, im_S, vector) -> None:
    """write_data (pnfam_storage.f90:407-486) for the run of ``case``: its final
    Broyden ``vector`` (reference part order), ``si`` and strengths."""
    hfb, nml, cp = case.hfb, case.nml, case.couplings
    inter, ef, g, s = nml["interaction"], nml["ext_field"], nml["general"], nml["solver"]
    w = _Writer()
    w.ints(VERSION_DATA)
    w.rec(b"hfb_soln")
    w.ints(int(hfb.N), int(hfb.Z))
    w.ints(int(hfb.nb))
    w.array(hfb.db, "<i4")
    w.rec(b"stat_hfb")
    ft = float(getattr(hfb, "temperature", 0.0) or 0.0)
    w.ints(1 if hfb.occupations is not None else 0)
    w.ints(0)                      # no blocked quasiparticle (blocked solutions are refused)
    w.reals(ft)
    w.ints(0, 0)
    w.rec(b"interact")
    w.rec(_fortran_name(str(inter.get("interaction_name", "NONE")).strip()))
    for flag in ("require_gauge_invariance", "require_self_consistency", "force_j2_terms"):
        w.ints(1 if inter.get(flag) else 0)
    w.reals(*_resolved_pairing(inter))
    ov = lambda k: HUGE if inter.get(k) is None else float(inter[k])
    w.reals(ov("override_cs0"), ov("override_csr"), ov("override_cds"), ov("override_ct"))
    w.reals(ov("override_cf"), ov("override_cgs"), ov("override_cj"), ov("override_csdj"))
    nghl = len(hfb.rho_n)
    mesh = lambda a: np.zeros(nghl) if a is None else np.asarray(a, dtype=np.float64)
    w.ints(nghl)
    w.array(mesh(cp.crho), "<f8")
    w.reals(cp.cdrho, cp.ctau, cp.ctj0, cp.ctj1, cp.ctj2, cp.crdj)
    w.array(mesh(cp.cs), "<f8")
    w.reals(cp.cds, cp.ct, cp.cj, cp.cgs, cp.cf, cp.csdj)
    w.array(mesh(cp.cpair), "<f8")
    w.array(mesh(cp.cspair), "<f8")
    w.rec(b"extfield")
    w.rec(_fortran_name(ef["operator_name"]))
    w.ints(int(ef["operator_k"]))
    w.rec(b"fam_soln")
    w.reals(float(g["real_eqrpa"]), float(g["imag_eqrpa"]))
    w.reals(float(s["quench_residual_int"]))
    w.reals(float(si))
    w.ints(int(nxy))
    w.array(vector, "<f8")
    w.reals(float(re_S[0]), float(im_S[0]))
    nx = len(re_S) - 1
    w.ints(nx)
    for k in range(nx):
        w.reals(float(re_S[1 + k]), float(im_S[1 + k]))
    with open(path, "wb") as fh:
        fh.write(b"".join(w.parts))


def read_storage(path: str, case, nxy: int, state_size: int, log=None) -> Restart:
    """fam_io(1) + read_data for the run of ``case`` with ``nxy`` FAM matrix elements
    and a Broyden vector of ``state_size`` doubles.  A missing, unreadable or
    other-version file starts the run from scratch without a message."""
    try:
        with open(path, "rb") as fh:
            data = fh.read()
    except OSError:
        return Restart()
    recs = _records(data)
    try:
        version = struct.unpack("<i", next(recs)[:4])[0]
    except (StopIteration, _Corrupted, struct.error):
        return Restart()
    if version != VERSION_DATA:
        return Restart()
    say = (lambda s: log.write(s)) if log is not None else (lambda s: None)
    say(f"  * Reading from storage file: {os.path.basename(path)}")
    say("")
    hfb, ef = case.hfb, case.nml["ext_field"]
    nops = 1 + len(case.G)
    ok = True
    si, vector, s0 = 1.0, None, np.zeros(nops, dtype=complex)
    key, stat_r, seen = None, False, False

    def nxt(dtype=None, n=None):
        try:
            r = next(recs)
        except StopIteration:
            raise _Corrupted(key)
        if dtype is None:
            return r
        isz = np.dtype(dtype).itemsize
        a = np.frombuffer(r[:len(r) // isz * isz], dtype=dtype)
        if n is not None and a.size < n:
            raise _Corrupted(key)
        return a

    try:
        for r in recs:
            if len(r) < 8:
                key = r.decode("ascii", "replace").strip()
                raise _Corrupted(key)
            key = r[:8].decode("ascii", "replace").strip()
            if key == "hfb_soln":
                nxt("<i4", 2)
                nb_r = int(nxt("<i4", 1)[0])
                db_r = nxt("<i4", nb_r)[:nb_r]
                if nb_r != int(hfb.nb) or not np.array_equal(db_r, np.asarray(hfb.db)):
                    ok = False
            elif key == "stat_hfb":
                ft_r = int(nxt("<i4", 1)[0])
                blo_r = int(nxt("<i4", 1)[0])
                nxt("<f8", 1)
                nxt("<i4", 2)
                stat_r = ft_r == 1 or blo_r == 1
            elif key == "interact":
                nxt()
                for _ in range(3):
                    nxt("<i4", 1)
                nxt("<f8", 2); nxt("<f8", 4); nxt("<f8", 4)
                ng = int(nxt("<i4", 1)[0])
                nxt("<f8", ng); nxt("<f8", 6); nxt("<f8", ng); nxt("<f8", 6); nxt("<f8", ng); nxt("<f8", ng)
            elif key == "extfield":
                name_r = nxt()[:80].decode("ascii", "replace").strip().upper()
                k_r = int(nxt("<i4", 1)[0])
                if name_r != str(ef["operator_name"]).strip().upper() or k_r != int(ef["operator_k"]):
                    ok = False
            elif key == "fam_soln":
                seen = True
                nxt("<f8", 2)
                nxt("<f8", 1)
                si = float(nxt("<f8", 1)[0])
                nxy_r = int(nxt("<i4", 1)[0])
                if nxy_r == nxy:
                    v = nxt("<f8")
                    ibroy_r = 8 if stat_r else 4
                    if v.size < ibroy_r * nxy_r:
                        raise _Corrupted(key)
                    v = v[:ibroy_r * nxy_r]
                    x = np.zeros(state_size)
                    m = min(state_size, v.size)   # a 4-part vector into an 8-part run fills X and Y
                    x[:m] = v[:m]
                    vector = x
                else:
                    ok = False
                    nxt()
                a = nxt("<f8", 2)
                s0[0] = complex(a[0], a[1])
                nx_r = int(nxt("<i4", 1)[0])
                for k in range(max(nx_r, 0)):
                    a = nxt("<f8", 2) if nx_r == nops - 1 else nxt()
                    if nx_r == nops - 1:
                        s0[1 + k] = complex(a[0], a[1])
    except _Corrupted as c:
        say(f"  * The file '{os.path.basename(path)}' is corrupted!")
        say(f"  * Problem occurs for key: {c.key or key or ''}")
        say("  * Starting calculation from scratch...")
        say("")
        return Restart(None, 1.0, s0)
    if not seen:
        return Restart(None, 1.0, s0)
    if not ok or vector is None:
        say(f"  * The file '{os.path.basename(path)}' is incompatible with the current calculation!")
        say("  * Starting calculation from scratch...")
        say("")
        return Restart(None, 1.0, s0)
    return Restart(vector, si, s0)
