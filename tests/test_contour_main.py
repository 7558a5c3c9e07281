"""The contour_main drop-in (contour_prog.f90, contour_setup.f90): contour
namelist, operator groups, per-point .dat files and per-operator summaries.
Host logic on the CPU with a fake device solver; one real solve on the GPU."""
import os
import shutil

import numpy as np
import pytest

from golden_cases import GOLDEN, golden
from pynfam_gb300 import contour_main
from pynfam_gb300.solver import SolveResult
from test_pnfam_main import parse_dat, write_in


class FakeSolver:
    def __init__(self, log):
        self.log = log
        self.nops = 1

    def set_operator(self, F, G=()):
        self.nops = 1 + len(G)
        self.log.append((F.label, F.k))

    def solve(self, omegas, history=True, max_iter=300, **kw):
        w = np.asarray(omegas, dtype=complex)
        P = len(w)
        hist = np.full((P, max_iter + 1, 3), np.nan)
        hist[:, 0] = (1.0, 0.0, 0.0)
        hist[:, 1] = (1e-9, 2.0, 3.0)
        re = np.repeat(w.real[:, None], self.nops, axis=1)
        im = np.repeat(w.imag[:, None], self.nops, axis=1)
        return SolveResult(re, im, np.ones(P, dtype=np.int32), np.full(P, 1e-9), hist, 0.0)

    def close(self):
        pass


def _ctr(path, groups, n=3):
    act = ", ".join("1" if g else "0" for g in groups)
    path.write_text(f"""&ctr_general
    fam_mode = 'STR'
    fam_input_filename = 'GT-K0.in'
/
&ctr_extfield
    operator_groups = '0+', '1+', '0-', '1-', '2-'
    operator_active = {act}
/
&str_parameters
    energy_start = 1.0
    energy_step = 0.5
    nr_points = {n}
    half_width = 0.25
/
""")


def _setup(tmp_path, name="GT-K0"):
    g = golden("S40")
    write_in(tmp_path / "GT-K0.in", g["operators"]["GT-K0"][0], g["interaction"], name)
    shutil.copyfile(os.path.join(GOLDEN, "S40.hel"), tmp_path / "hfbtho_output.hel")


def test_operator_groups_and_signs():
    ctr = contour_main.ctr_defaults()
    assert contour_main.operator_list(ctr, "GT", -1) == [("GT", -1)]
    ctr["operator_active"] = [0, 1, 0, 1, 0]
    assert contour_main.operator_list(ctr, "GT", -1) == [("GT", 0), ("GT", -1), ("R", 0), ("R", -1), ("P", 0),
                                                          ("P", -1), ("RS1", 0), ("RS1", -1)]
    ctr["nr_points"], ctr["energy_start"], ctr["energy_step"], ctr["half_width"] = 3, 1.0, 0.5, 0.25
    assert contour_main.energies(ctr) == [1.0 + 0.25j, 1.5 + 0.25j, 2.0 + 0.25j]


def test_contour_run_writes_points_and_summaries(tmp_path, monkeypatch):
    monkeypatch.setenv("PNFAM_GB300_CACHE", "off")
    _setup(tmp_path)
    _ctr(tmp_path / "pnfam_CONTOUR.dat", [0, 1, 1, 0, 0])
    log = []
    assert contour_main.run("pnfam_CONTOUR.dat", str(tmp_path), solver_factory=lambda case: FakeSolver(log)) == 0
    assert log == [("GT", 0), ("GT", 1), ("RS0", 0), ("PS0", 0)]
    for op, k, nx in (("GT", 0, 0), ("GT", 1, 0), ("RS0", 0, 2), ("PS0", 0, 2)):
        for i, w in enumerate((1.0, 1.5, 2.0)):
            version, conv, t, rows = parse_dat(tmp_path / f"{op}-K{k}_{i:06d}.dat")
            assert conv == "Yes" and rows["Energy"] == pytest.approx((w, 0.25))
            assert rows["Strength"] == pytest.approx((w, 0.25))
        lines = (tmp_path / f"{op}-K{k}.out").read_text().splitlines()
        assert lines[4] == f"# Operator: {op} with K = {k}" and lines[5] == "# Gamma (half-width): 0.2500"
        data = [l.split() for l in lines if not l.startswith("#")]
        assert len(data) == 3 and all(len(r) == 2 + 2 * (1 + nx) for r in data)
        assert [float(r[1]) for r in data] == [1.0, 1.5, 2.0] and all(r[0] == "1" for r in data)


def test_contour_without_groups_uses_the_namelist_operator(tmp_path, monkeypatch):
    monkeypatch.setenv("PNFAM_GB300_CACHE", "off")
    _setup(tmp_path, name="")
    _ctr(tmp_path / "pnfam_CONTOUR.dat", [0, 0, 0, 0, 0], n=2)
    log = []
    assert contour_main.run("pnfam_CONTOUR.dat", str(tmp_path), solver_factory=lambda case: FakeSolver(log)) == 0
    assert log == [("GT", 0)]
    # no fam_output_filename: the points print, only the summary is a file
    assert not list(tmp_path.glob("GT-K0_*.dat")) and (tmp_path / "GT-K0.out").exists()


@pytest.mark.gpu
def test_contour_on_the_gpu(tmp_path, monkeypatch):
    """Two recorded GT K=0 energies as a contour: the recorded strengths (1e-6)."""
    monkeypatch.setenv("PNFAM_GB300_CACHE", "off")
    _setup(tmp_path)
    pts = golden("S40")["operators"]["GT-K0"]
    w0 = complex(pts[0]["namelist"]["real_eqrpa"], pts[0]["namelist"]["imag_eqrpa"])
    (tmp_path / "pnfam_CONTOUR.dat").write_text(f"""&ctr_general
    fam_input_filename = 'GT-K0.in'
/
&str_parameters
    energy_start = {w0.real!r}
    energy_step = 0.0
    nr_points = 2
    half_width = {w0.imag!r}
/
""")
    assert contour_main.run("pnfam_CONTOUR.dat", str(tmp_path)) == 0
    want = pts[0]["result"]["Strength"]
    for i in range(2):
        _, conv, _, rows = parse_dat(tmp_path / f"GT-K0_{i:06d}.dat")
        got = rows["Strength"]
        assert abs(got[0] - want[0]) <= 1e-6 * abs(want[0]) and abs(got[1] - want[1]) <= 1e-6 * abs(want[1])
