"""Restart storage (use_fam_storage, pnfam_storage.f90): the <name>.bin file, the
oracle's restart from a stored Broyden vector, the GPU solve from a start vector
(pnfam_gpu_solve_state) against the oracle, and the pnfam_main drop-in that
reads and writes the file."""
import os
import shutil
import struct
import subprocess
import sys

import numpy as np
import pytest

from golden_cases import GOLDEN, case_for, golden
from oracle.fam_oracle import FAMOracle
from pynfam_gb300 import storage
from test_pnfam_main import EXE, parse_dat, write_in


class _Lines:
    def __init__(self):
        self.lines = []

    def write(self, s="", comment=True):
        self.lines.append(s)


def _oracle(c, **kw):
    s = c.nml["solver"]
    orc = FAMOracle(c.hfb, c.couplings, c.F, c.G, quench=c.quench, occupations=kw.pop("occupations", None))
    args = dict(max_iter=s["max_iter"], eps=s["convergence_epsilon"], broyden_m=s["broyden_history_size"])
    args.update(kw)
    return orc.solve(c.omega, **args)


def _strengths(r):
    return np.asarray(r.re_str) + 1j * np.asarray(r.im_str)


def test_storage_round_trip(tmp_path):
    """write_data then read_data give back the vector, si and every strength value;
    the file is Fortran unformatted sequential with the reference's records."""
    c, _ = case_for("S40", "RS1-K1", 3)
    nxy = c.F.mat.nelem
    rng = np.random.default_rng(7)
    v = rng.standard_normal(4 * nxy)
    re_S, im_S = rng.standard_normal(1 + len(c.G)), rng.standard_normal(1 + len(c.G))
    p = str(tmp_path / "RS1-K1.bin")
    storage.write_storage(p, c, nxy, 3.25e-5, re_S, im_S, v)
    data = open(p, "rb").read()
    n = struct.unpack_from("<i", data, 0)[0]
    assert n == 4 and struct.unpack_from("<i", data, 4)[0] == storage.VERSION_DATA
    assert data[12:16] == struct.pack("<i", 8) and data[16:24] == b"hfb_soln"
    for key in (b"stat_hfb", b"interact", b"extfield", b"fam_soln"):
        assert key in data
    log = _Lines()
    r = storage.read_storage(p, c, nxy, 4 * nxy, log)
    assert np.array_equal(r.vector, v) and r.si == 3.25e-5
    assert np.array_equal(r.s0, re_S + 1j * im_S)
    assert log.lines[0] == "  * Reading from storage file: RS1-K1.bin"


def test_storage_rejects_other_operator_and_damaged_files(tmp_path):
    c0, _ = case_for("S40", "GT-K0", 0)
    c1, _ = case_for("S40", "GT-K1", 0)
    nxy = c0.F.mat.nelem
    p = str(tmp_path / "GT.bin")
    storage.write_storage(p, c0, nxy, 0.5, [1.0], [2.0], np.ones(4 * nxy))
    log = _Lines()
    r = storage.read_storage(p, c1, c1.F.mat.nelem, 4 * c1.F.mat.nelem, log)
    assert r.vector is None and r.si == 1.0
    assert any("is incompatible with the current calculation" in l for l in log.lines)
    # the strength read before the file was judged is still shown at iteration 0
    assert r.s0[0] == 1.0 + 2.0j
    with open(p, "rb") as fh:
        data = fh.read()
    with open(p, "wb") as fh:
        fh.write(data[:len(data) - 40])
    log = _Lines()
    r = storage.read_storage(p, c0, nxy, 4 * nxy, log)
    assert r.vector is None and any("is corrupted" in l for l in log.lines)
    assert storage.read_storage(str(tmp_path / "missing.bin"), c0, nxy, 4 * nxy, log).vector is None


def test_oracle_restart_from_its_fixed_point():
    """Restarting from the converged Broyden vector: one more iteration reproduces the
    strength (the vector is the fixed point, in the reference's part order)."""
    c, pt = case_for("S40", "P-K1", 9)
    full = _oracle(c, eps=1e-12, max_iter=300)
    again = _oracle(c, x0=full.vector, si0=1.0, max_iter=1)
    np.testing.assert_allclose(_strengths(again), _strengths(full), rtol=1e-9)


def test_oracle_interrupted_run_resumes():
    """An interrupted run (max_iter 6) stored and resumed reaches the fixed point of
    the uninterrupted run (both to si < 1e-12; 1e-9 per value); the resumed run starts
    a fresh Broyden history, as in the reference, so the two trajectories differ."""
    c, pt = case_for("S40", "GT-K0", 5)
    part = _oracle(c, max_iter=6)
    assert part.iter_conv < 0
    rest = _oracle(c, x0=part.vector, si0=part.history[-1][2], s0=_strengths(part), eps=1e-12, max_iter=300)
    full = _oracle(c, eps=1e-12, max_iter=300)
    assert rest.iter_conv > 0 and rest.history[0][2] == part.history[-1][2]
    assert rest.history[0][3] == part.re_str[0]
    np.testing.assert_allclose(_strengths(rest), _strengths(full), rtol=1e-9)


def _run_dir(tmp_path, op, idx, use, max_iter=None, case="S40"):
    g = golden(case)
    pt = dict(g["operators"][op][idx])
    pt["namelist"] = dict(pt["namelist"])
    if max_iter is not None:
        pt["namelist"]["max_iter"] = max_iter
    write_in(tmp_path / f"{op}.in", pt, g["interaction"], op)
    txt = open(tmp_path / f"{op}.in").read().replace("use_fam_storage = 0", f"use_fam_storage = {use}")
    open(tmp_path / f"{op}.in", "w").write(txt)
    if not (tmp_path / "hfbtho_output.hel").exists():
        shutil.copyfile(os.path.join(GOLDEN, f"{case}.hel"), tmp_path / "hfbtho_output.hel")
    return pt


def _run(tmp_path, op):
    env = dict(os.environ, PNFAM_GB300_CACHE="off")
    return subprocess.run([sys.executable, EXE, f"{op}.in"], cwd=tmp_path, capture_output=True, text=True, env=env)


def test_cli_stored_converged_point_stops_at_iteration_zero(tmp_path):
    """A stored state whose si is below the convergence limit ends the run at iteration
    0 with the stored strengths (no device work), and use_fam_storage = -1 writes the
    same file back."""
    op = "GT-K0"
    pt = _run_dir(tmp_path, op, 2, -1)
    c, _ = case_for("S40", op, 2)
    ref = _oracle(c)
    assert ref.iter_conv > 0
    p = tmp_path / f"{op}.bin"
    storage.write_storage(str(p), c, c.F.mat.nelem, ref.si, ref.re_str, ref.im_str, ref.vector)
    before = open(p, "rb").read()
    r = _run(tmp_path, op)
    assert r.returncode == 0 and r.stderr.strip() == "", r.stderr
    out = open(tmp_path / f"{op}.dat").read()
    assert "Reading from storage file: GT-K0.bin" in out
    assert "converged after      0 steps" in out
    _, conv, _, rows = parse_dat(tmp_path / f"{op}.dat")
    assert conv == "Yes"
    assert rows["Strength"] == (float(f"{ref.re_str[0]:.19E}"), float(f"{ref.im_str[0]:.19E}"))
    assert open(p, "rb").read() == before


@pytest.mark.gpu
def test_gpu_solve_from_start_vector_matches_oracle():
    """pnfam_gpu_solve_state from the vector of an interrupted run: the whole history
    against the oracle's restart (1e-9), the final strengths (1e-10) and the final
    vector (1e-9 of its largest element)."""
    from pynfam_gb300.solver import GPUSolver
    c, _ = case_for("S40", "RS1-K1", 3)
    s = c.nml["solver"]
    part = _oracle(c, max_iter=5)
    ref = _oracle(c, x0=part.vector, si0=1.0)
    gpu = GPUSolver(c.hfb, c.couplings)
    gpu.set_operator(c.F, c.G)
    assert gpu.state_size == part.vector.size
    r = gpu.solve([c.omega], max_iter=s["max_iter"], eps=s["convergence_epsilon"],
                  broyden_m=s["broyden_history_size"], quench=c.quench, history=True,
                  x0=part.vector[None, :], return_state=True)
    gpu.close()
    assert r.iters[0] == ref.iter_conv > 0
    for h in ref.history[1:]:
        g = r.hist[0, h[0]]
        assert abs(g[0] - h[2]) <= 1e-9 * max(abs(h[2]), 1e-3), (h, g)
        assert abs(g[1] - h[3]) <= 1e-9 * abs(ref.re_str[0]), (h, g)
    for k in range(len(ref.re_str)):
        assert abs(r.re_S[0, k] - ref.re_str[k]) <= 1e-10 * abs(ref.re_str[k]) + 1e-15
        assert abs(r.im_S[0, k] - ref.im_str[k]) <= 1e-10 * abs(ref.im_str[k]) + 1e-15
    assert np.max(np.abs(r.state[0] - ref.vector)) <= 1e-9 * np.max(np.abs(ref.vector))


@pytest.mark.gpu
def test_gpu_statistical_start_vector_uses_reference_part_order():
    """The statistical FAM's 8-part vector (Re X, Re Y, Im X, Im Y, Re P, Re Q, Im P,
    Im Q in the reference) through pnfam_gpu_solve_state against the oracle."""
    from pynfam_gb300.solver import GPUSolver
    from pynfam_gb300.statistics import thermal_occupations
    c, _ = case_for("S40", "GT-K0", 5)
    occ = thermal_occupations(c.hfb, 1.0)
    s = c.nml["solver"]
    part = _oracle(c, max_iter=5, occupations=occ)
    ref = _oracle(c, x0=part.vector, si0=1.0, occupations=occ)
    gpu = GPUSolver(c.hfb, c.couplings, occupations=occ)
    gpu.set_operator(c.F, c.G)
    assert gpu.state_size == part.vector.size == 8 * c.F.mat.nelem
    r = gpu.solve([c.omega], max_iter=s["max_iter"], eps=s["convergence_epsilon"],
                  broyden_m=s["broyden_history_size"], quench=c.quench, history=True,
                  x0=part.vector[None, :], return_state=True)
    gpu.close()
    assert r.iters[0] == ref.iter_conv > 0
    for k in range(len(ref.re_str)):
        assert abs(r.re_S[0, k] - ref.re_str[k]) <= 1e-10 * abs(ref.re_str[k]) + 1e-15
    assert np.max(np.abs(r.state[0] - ref.vector)) <= 1e-9 * np.max(np.abs(ref.vector))


@pytest.mark.gpu
def test_cli_interrupted_run_resumes_from_its_file(tmp_path):
    """pnfam_main with use_fam_storage = -1: a run cut at max_iter 6 stores its vector;
    the rerun reads it, continues (here to si < 1e-12) and matches the oracle's fixed
    point of the point (1e-8), and stores the converged vector."""
    op = "P-K1"
    pt = _run_dir(tmp_path, op, 4, -1, max_iter=6)
    c, _ = case_for("S40", op, 4)
    full = _oracle(c, eps=1e-12, max_iter=300)
    r = _run(tmp_path, op)
    assert r.returncode == 0 and r.stderr.strip() == "", r.stderr
    _, conv, _, _ = parse_dat(tmp_path / f"{op}.dat")
    assert conv == "No" and (tmp_path / f"{op}.bin").exists()
    _run_dir(tmp_path, op, 4, -1, max_iter=300)
    txt = open(tmp_path / f"{op}.in").read()
    txt = txt.replace(f"convergence_epsilon = {pt['namelist']['convergence_epsilon']!r}", "convergence_epsilon = 1e-12")
    open(tmp_path / f"{op}.in", "w").write(txt)
    r = _run(tmp_path, op)
    assert r.returncode == 0 and r.stderr.strip() == "", r.stderr
    out = open(tmp_path / f"{op}.dat").read()
    assert "Reading from storage file" in out and "incompatible" not in out
    _, conv, _, rows = parse_dat(tmp_path / f"{op}.dat")
    assert conv == "Yes"
    labels = ["Strength"] + [g.label for g in c.G]
    for k, lab in enumerate(labels):
        assert abs(rows[lab][0] - full.re_str[k]) <= 1e-8 * abs(full.re_str[k]) + 1e-15, (lab, rows[lab])
        assert abs(rows[lab][1] - full.im_str[k]) <= 1e-8 * abs(full.im_str[k]) + 1e-15, (lab, rows[lab])
    # a third run starts from the converged vector and stops at iteration 0
    r = _run(tmp_path, op)
    assert r.returncode == 0
    assert "converged after      0 steps" in open(tmp_path / f"{op}.dat").read()
