"""The pnFAM namelist: groups, defaults and a Fortran-namelist reader.

Groups and defaults follow pnfam_setup.f90 (:96-108 declarations, :196-228
``init_pnfam_namelist``, :232-268 ``read_pnfam_namelist``).  The reader
accepts what gfortran's namelist input accepts for these groups as written by
f90nml (pynfam's writer): quoted strings, logicals (.true./T/...), integers,
reals with d/e exponents, comma-separated arrays, and empty values (", ,")
that keep the default.
"""
from __future__ import annotations

import re

import numpy as np

GROUPS = ("general", "ext_field", "interaction", "solver")


class NamelistError(RuntimeError):
    pass


def defaults() -> dict:
    """init_pnfam_namelist (pnfam_setup.f90:196-228)."""
    return {
        "general": {"fam_output_filename": "", "print_stdout": True, "use_fam_storage": 0,
                    "real_eqrpa": 0.0, "imag_eqrpa": 0.5},
        "ext_field": {"beta_type": "-", "operator_k": 0, "operator_name": "F",
                      "compute_crossterms": False, "two_body_current_mode": 0,
                      "two_body_current_usep": False,
                      # default-real literals in the reference (pnfam_setup.f90:189-191)
                      "two_body_current_lecs": [float(np.float32(-3.4)), float(np.float32(5.4)), 0.0]},
        "solver": {"broyden_history_size": 50, "convergence_epsilon": 1.0e-7, "max_iter": 200,
                   "energy_shift_prot": 0.0, "energy_shift_neut": 0.0,
                   "quench_residual_int": 1.0},
        # entries left unset (None) mean "not given" for the optional overrides
        "interaction": {"interaction_name": "NONE", "force_j2_terms": False,
                        "require_gauge_invariance": False, "require_self_consistency": True,
                        "vpair0": None, "vpair_t0": None, "vpair1": None, "vpair_t1": None,
                        "override_cs0": None, "override_csr": None, "override_cds": None,
                        "override_ct": None, "override_cf": None, "override_cgs": None,
                        "override_cj": None, "override_csdj": None},
    }


_TOKEN = re.compile(r"""\s*(?:'((?:[^']|'')*)'|"((?:[^"]|"")*)"|([^,\s/]+)|(,))""")


def _convert(tok: str):
    t = tok.strip()
    low = t.lower()
    if low in (".true.", "t", ".t.", "true"):
        return True
    if low in (".false.", "f", ".f.", "false"):
        return False
    try:
        return int(t)
    except ValueError:
        pass
    try:
        return float(low.replace("d", "e"))
    except ValueError:
        raise NamelistError(f"cannot parse value '{tok}'")


def _parse_values(text: str):
    """Comma/blank separated values; an empty slot between commas is None."""
    vals = []
    pending = True   # a value slot is open
    pos = 0
    while pos < len(text):
        m = _TOKEN.match(text, pos)
        if not m or m.end() == pos:
            break
        pos = m.end()
        if m.group(4):
            if pending:
                vals.append(None)
            pending = True
            continue
        if m.group(1) is not None:
            v = m.group(1).replace("''", "'")
        elif m.group(2) is not None:
            v = m.group(2).replace('""', '"')
        else:
            v = _convert(m.group(3))
        vals.append(v)
        pending = False
    return vals


def parse_namelist_text(text: str) -> dict:
    """All groups in ``text`` -> {group: {key: value}}; arrays become lists and
    a scalar given as an empty value is recorded as None."""
    # strip comments (outside quotes)
    lines = []
    for line in text.splitlines():
        out, q = [], None
        for ch in line:
            if q:
                out.append(ch)
                if ch == q:
                    q = None
            elif ch in "'\"":
                q = ch; out.append(ch)
            elif ch == "!":
                break
            else:
                out.append(ch)
        lines.append("".join(out))
    blocks = []
    cur = None
    for line in lines:
        s = line.strip()
        if cur is None:
            m = re.match(r"[&$](\w+)(.*)$", s)
            if m and m.group(1).lower() != "end":
                cur = [m.group(1).lower(), [m.group(2)]]
                s = m.group(2).strip()
                if s.endswith("/") and not s.endswith("'/") and s.count("'") % 2 == 0:
                    cur[1][-1] = s[:-1]
                    blocks.append(cur); cur = None
            continue
        if s == "/" or s.lower() in ("&end", "$end"):
            blocks.append(cur); cur = None
            continue
        if s.endswith("/") and s.count("'") % 2 == 0 and s.count('"') % 2 == 0:
            cur[1].append(s[:-1]); blocks.append(cur); cur = None
            continue
        cur[1].append(line)
    if cur is not None:
        raise NamelistError(f"namelist group &{cur[0]} is not terminated")
    groups = {}
    for name, body_lines in blocks:
        body = "\n".join(body_lines)
        entries = {}
        parts = re.split(r"(?:^|[\s,])(\w+(?:\(\s*\d+\s*\))?)\s*=", body)
        for k in range(1, len(parts) - 1, 2):
            key = parts[k].strip().lower()
            vals = _parse_values(parts[k + 1].strip().rstrip("/"))
            # drop the trailing None created by a separator after the last value
            while len(vals) > 1 and vals[-1] is None:
                vals.pop()
            entries[key] = vals[0] if len(vals) == 1 else (vals if vals else None)
        groups[name] = entries
    return groups


def parse_namelist_file(path: str) -> dict:
    with open(path) as fh:
        return parse_namelist_text(fh.read())


def read_pnfam_namelist(path: str) -> dict:
    """Defaults overlaid with the groups found in ``path``."""
    try:
        given = parse_namelist_file(path)
    except OSError as e:
        raise NamelistError(f"problem reading pnfam namelist: {e}")
    nml = defaults()
    for g in GROUPS:
        for k, v in given.get(g, {}).items():
            if k not in nml[g]:
                raise NamelistError(f"problem reading pnfam namelist: unknown entry {g}%{k}")
            if v is None:
                continue   # empty value keeps the default
            if isinstance(v, list) and not isinstance(nml[g][k], list):
                v = next((x for x in v if x is not None), None)
                if v is None:
                    continue
            nml[g][k] = v
    e = nml["ext_field"]
    e["operator_name"] = str(e["operator_name"]).strip().upper()
    e["beta_type"] = str(e["beta_type"]).strip()
    if e["beta_type"] not in ("-", "+"):
        raise NamelistError(f"unknown beta_type={e['beta_type']}")
    return nml
