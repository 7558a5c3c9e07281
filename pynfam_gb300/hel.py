"""Reader for HFBTHO's ``.hel`` binary solution file (format version 5).

The file is a Fortran unformatted sequential stream: every record is framed
by a 4-byte little-endian length before and after its payload.  Records are
grouped under 8-character keywords ('Metadata', 'SkyFunct', 'HO-Basis',
'QuantNum', 'Various.', 'Constrai', 'Densits.', 'FieldsN.', 'FieldsP.',
'Blocking', 'Blk-rest', 'Temperat', ...), written in the order of HFBTHO's
``write_data`` (hfbtho_io.f90:745-897) and read back by ``read_data``
(hfbtho_io.f90:487-738).  Only the keyword groups that the pnFAM reader needs
are decoded; the rest are skipped by keyword.
"""
from __future__ import annotations

import struct
from dataclasses import dataclass, field

import numpy as np

VERSION_DATA = 5


class HelFormatError(RuntimeError):
    """The file is not a readable HFBTHO version-5 solution."""


def _records(blob: bytes):
    off = 0
    n = len(blob)
    while off < n:
        if off + 4 > n:
            raise HelFormatError("truncated record marker")
        (ln,) = struct.unpack_from("<i", blob, off)
        end = off + 4 + ln
        if ln < 0 or end + 4 > n:
            raise HelFormatError("truncated record")
        (ln2,) = struct.unpack_from("<i", blob, end)
        if ln2 != ln:
            raise HelFormatError("record markers disagree")
        yield blob[off + 4:end]
        off = end + 4


@dataclass
class HelData:
    """Decoded contents of a ``.hel`` file (names follow HFBTHO's variables)."""
    version: int = 0
    Z: int = 0
    N: int = 0
    # SkyFunct
    skyrme: str = ""
    use_j2terms: bool = False
    pwi: float = 0.0
    nm: np.ndarray = field(default_factory=lambda: np.zeros(9))  # E,K,SMASS,RHO,ASS,LASS,VMASS,P,KA
    Crho: np.ndarray = field(default_factory=lambda: np.zeros(2))
    Cdrho: np.ndarray = field(default_factory=lambda: np.zeros(2))
    Ctau: np.ndarray = field(default_factory=lambda: np.zeros(2))
    CrDr: np.ndarray = field(default_factory=lambda: np.zeros(2))
    CrdJ: np.ndarray = field(default_factory=lambda: np.zeros(2))
    CJ: np.ndarray = field(default_factory=lambda: np.zeros(2))
    CpV0: np.ndarray = field(default_factory=lambda: np.zeros(2))
    CpV1: np.ndarray = field(default_factory=lambda: np.zeros(2))
    sigma: float = 0.0
    hbzero: float = 0.0
    # HO-Basis
    b0: float = 0.0
    bz: float = 0.0
    bp: float = 0.0
    n00: int = 0
    nb: int = 0
    nt: int = 0
    ngh: int = 0
    ngl: int = 0
    xh: np.ndarray = None
    xl: np.ndarray = None
    wh: np.ndarray = None
    wl: np.ndarray = None
    # QuantNum
    ID: np.ndarray = None
    nr: np.ndarray = None
    nz: np.ndarray = None
    nl: np.ndarray = None
    ns: np.ndarray = None
    # Various.
    si: float = 0.0
    ala: np.ndarray = None
    del_: np.ndarray = None
    # Densits. / Fields
    ro: np.ndarray = None
    aka: np.ndarray = None
    fields: dict = field(default_factory=dict)   # 'n'/'p' -> dict of mesh arrays
    set_temperature: bool = False
    temperature: float = 0.0     # Temperat: HFBTHO's temper (MeV)
    has_blocking_request: bool = False


_FIELD_NAMES = ("v", "vhb", "vr", "vz", "vd", "vs", "vSFIZ", "vSZFI", "vSFIR", "vSRFI", "dv")


def read_hel(path: str) -> HelData:
    """Parse ``path``; raises :class:`HelFormatError` on a corrupt file."""
    with open(path, "rb") as fh:
        blob = fh.read()
    recs = list(_records(blob))
    if not recs:
        raise HelFormatError("empty file")
    h = HelData()
    (h.version,) = struct.unpack_from("<i", recs[0], 0)
    if h.version != VERSION_DATA:
        raise HelFormatError(f"unsupported .hel version {h.version}")
    i = 1
    f8 = lambda r: np.frombuffer(r, dtype="<f8")
    i4 = lambda r: np.frombuffer(r, dtype="<i4")
    while i < len(recs):
        key = recs[i]
        if len(key) != 8:
            raise HelFormatError(f"expected a keyword record at {i}")
        key = key.decode("ascii", "replace").strip()
        i += 1
        if key == "Metadata":
            h.Z, h.N = (int(v) for v in i4(recs[i])); i += 1
            i += 1  # collective_inertia, fission_fragments, pairing_regularization, localization
            flags = i4(recs[i]); i += 1  # switch_to_THO, projection_is_on, set_temperature, neck
            h.set_temperature = bool(flags[2])
        elif key == "SkyFunct":
            r = recs[i]; i += 1
            lg = struct.unpack_from("<5i", r, 0)
            h.use_j2terms = bool(lg[2])
            h.skyrme = r[20:50].decode("ascii", "replace").strip()
            (h.pwi,) = struct.unpack_from("<d", r, 54)
            h.nm = f8(recs[i]).copy(); i += 1
            c = f8(recs[i]); i += 1
            h.Crho, h.Cdrho, h.Ctau, h.CrDr, h.CrdJ, h.CJ = (c[2 * k:2 * k + 2].copy() for k in range(6))
            h.CpV0 = c[12:14].copy(); h.CpV1 = c[14:16].copy(); h.sigma = float(c[16])
            h.hbzero = float(f8(recs[i])[0]); i += 1
        elif key == "HO-Basis":
            h.b0, h.bz, h.bp = (float(v) for v in f8(recs[i])); i += 1
            h.n00, h.nb, h.nt, h.ngh, h.ngl, _nleg = (int(v) for v in i4(recs[i])); i += 1
            m = f8(recs[i]); i += 1
            ngh, ngl = h.ngh, h.ngl
            h.xh = m[:ngh].copy(); h.xl = m[ngh:ngh + ngl].copy()
            h.wh = m[ngh + ngl:2 * ngh + ngl].copy(); h.wl = m[2 * ngh + ngl:].copy()
        elif key == "QuantNum":
            h.ID = i4(recs[i]).astype(np.int64); i += 1
            nt = int(h.ID.sum())
            q = np.empty((nt, 4), dtype=np.int64)
            for k in range(nt):
                q[k] = i4(recs[i]); i += 1
            h.nr, h.nz, h.nl, h.ns = q[:, 0].copy(), q[:, 1].copy(), q[:, 2].copy(), q[:, 3].copy()
        elif key == "Various.":
            v1 = f8(recs[i]); i += 1
            h.si = float(v1[0])
            v2 = f8(recs[i]); i += 1
            h.pwi = float(v2[0]); h.del_ = v2[1:3].copy(); h.ala = v2[6:8].copy()
            i += 1
        elif key == "Constrai":
            i += 5  # numberCons/lambdaMax, multLambda, multRequested, qmoment, multLag
            i += 1  # qfield (neck records are absent for the supported inputs)
        elif key == "Densits.":
            nghl = h.ngh * h.ngl
            h.ro = f8(recs[i]).reshape(2, nghl).copy(); i += 1
            h.aka = f8(recs[i]).reshape(2, nghl).copy(); i += 1
        elif key in ("FieldsN.", "FieldsP."):
            t = "n" if key == "FieldsN." else "p"
            h.fields[t] = {}
            for name in _FIELD_NAMES:
                h.fields[t][name] = f8(recs[i]).copy(); i += 1
        elif key == "Blocking":
            i += 2
        elif key == "Blk-rest":
            i += 1
        elif key == "Temperat":
            h.temperature = float(f8(recs[i])[0])
            i += 4
        elif key == "Regular.":
            i += 3
        elif key == "THObasis":
            i += 2
        elif key == "HFBmatrX":
            i += 2
        else:
            raise HelFormatError(f"unknown keyword '{key}'")
    for req in ("n", "p"):
        if req not in h.fields:
            raise HelFormatError("fields record missing")
    if h.ID is None or h.xh is None:
        raise HelFormatError("basis records missing")
    return h
