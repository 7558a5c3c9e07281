"""The pnfam_main drop-in: namelist + hfbtho_output.hel in, <name>.dat out,
parsed the way pynfam's pnfamParser reads it (pynfam/outputs/pnfam_parser.py)."""
import os
import re
import shutil
import subprocess
import sys

import pytest

from golden_cases import GOLDEN, golden

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EXE = os.path.join(ROOT, "pynfam_gb300", "bin", "pnfam_main.x")


def write_in(path, pt, interaction, name):
    n = pt["namelist"]
    mode = n.get("two_body_current_mode", 0)
    lecs = ", ".join(repr(float(x)) for x in n.get("two_body_current_lecs", [-3.1962, 3.1962, 0]))
    txt = f"""&general
    fam_output_filename = '{name}'
    print_stdout = .false.
    use_fam_storage = 0
    real_eqrpa = {n['real_eqrpa']!r}
    imag_eqrpa = {n['imag_eqrpa']!r}
/

&ext_field
    beta_type = '{n['beta_type']}'
    operator_name = '{n['operator_name']}'
    operator_k = {n['operator_k']}
    compute_crossterms = {'.true.' if n['compute_crossterms'] else '.false.'}
    two_body_current_mode = {mode}
    two_body_current_usep = .false.
    two_body_current_lecs = {lecs}
/

{interaction}
&solver
    max_iter = {n['max_iter']}
    convergence_epsilon = {n['convergence_epsilon']!r}
    broyden_history_size = {n['broyden_history_size']}
    energy_shift_prot = 0.0
    energy_shift_neut = 0.0
    quench_residual_int = {n['quench_residual_int']!r}
/
"""
    open(path, "w").write(txt)


def parse_dat(path):
    """What pnfamParser extracts: version, convergence, time and the table."""
    lines = open(path).read().splitlines()
    version = [l for l in lines if "Version:" in l][0].split()[-1]
    conv = "Yes" if any("iteration converged" in l for l in lines) else \
        ("No" if any("iteration interrupted" in l for l in lines) else None)
    time_line = [l for l in lines if "Total CPU time" in l][0]
    t = float(time_line.split()[-2])
    table = [l.split() for l in lines if l.strip() and not l.startswith("#")]
    assert table[0] == ["Real", "Imag"]
    rows = {r[0]: (float(r[1]), float(r[2])) for r in table[1:]}
    return version, conv, t, rows


def test_cli_reports_missing_ground_state(tmp_path):
    g = golden("S40")
    write_in(tmp_path / "GT-K0.in", g["operators"]["GT-K0"][0], g["interaction"], "GT-K0")
    env = dict(os.environ, PNFAM_GB300_CACHE="off")
    p = subprocess.run([sys.executable, EXE, "GT-K0.in"], cwd=tmp_path, capture_output=True, text=True, env=env)
    assert p.returncode == 1
    assert "hfbtho_output.hel" in p.stderr
    out = open(tmp_path / "GT-K0.dat").read()
    assert "ERROR" in out and "Strength" not in out


def _gpu_present():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def test_cli_two_body_current_without_tbc_and_gpu(tmp_path):
    """Mode 111100 reads the finite-range field from <fam_output_filename>.tbc and
    computes it on the GPU when the file is missing; with neither, the run fails with
    a message naming the file and writes no result table."""
    if _gpu_present():
        pytest.skip("a GPU is present: the field is computed (see the GPU test below)")
    g = golden("S40_2bc_fam")
    write_in(tmp_path / "GT-K0.in", g["operators"]["GT-K0"][0], g["interaction"], "GT-K0")
    shutil.copyfile(os.path.join(GOLDEN, "S40_2bc_fam.hel"), tmp_path / "hfbtho_output.hel")
    env = dict(os.environ, PNFAM_GB300_CACHE="off")
    p = subprocess.run([sys.executable, EXE, "GT-K0.in"], cwd=tmp_path, capture_output=True, text=True, env=env)
    assert p.returncode == 1 and "GT-K0.tbc" in p.stderr
    out = open(tmp_path / "GT-K0.dat").read()
    assert "GT-K0.tbc" in out and "Strength" not in out
    assert not (tmp_path / "GT-K0.tbc").exists()


@pytest.mark.gpu
def test_cli_two_body_current_computes_its_tbc_file(tmp_path):
    """Mode 111100 without a .tbc file: the finite-range field is computed on the GPU
    and stored, and the run reproduces the recorded 2BC strength."""
    g = golden("S40_2bc_fam")
    pt = g["operators"]["GT-K0"][0]
    write_in(tmp_path / "GT-K0.in", pt, g["interaction"], "GT-K0")
    shutil.copyfile(os.path.join(GOLDEN, "S40_2bc_fam.hel"), tmp_path / "hfbtho_output.hel")
    env = dict(os.environ, PNFAM_GB300_CACHE="off")
    p = subprocess.run([sys.executable, EXE, "GT-K0.in"], cwd=tmp_path, capture_output=True, text=True, env=env)
    assert p.returncode == 0, p.stderr
    assert (tmp_path / "GT-K0.tbc").exists()
    version, conv, t, rows = parse_dat(tmp_path / "GT-K0.dat")
    re_, im_ = pt["result"]["Strength"]
    got = rows["Strength"]
    assert abs(got[0] - re_) <= 1e-6 * abs(re_) and abs(got[1] - im_) <= 1e-6 * abs(im_)


def test_cli_rejects_two_arguments(tmp_path):
    p = subprocess.run([sys.executable, EXE, "a", "b"], cwd=tmp_path, capture_output=True, text=True)
    assert p.returncode == 1 and "More than one" in p.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("op,idx", [("GT-K0", 0), ("P-K1", 4)])
def test_cli_point_matches_recorded(tmp_path, op, idx):
    g = golden("S40")
    pt = g["operators"][op][idx]
    write_in(tmp_path / f"{op}.in", pt, g["interaction"], op)
    shutil.copyfile(os.path.join(GOLDEN, "S40.hel"), tmp_path / "hfbtho_output.hel")
    env = dict(os.environ, PNFAM_GB300_CACHE=str(tmp_path / "cache"))
    p = subprocess.run([sys.executable, EXE, f"{op}.in"], cwd=tmp_path, capture_output=True, text=True, env=env)
    assert p.returncode == 0 and p.stderr.strip() == "", p.stderr
    version, conv, t, rows = parse_dat(tmp_path / f"{op}.dat")
    assert conv == "Yes" and t >= 0.0 and version
    for lab, (re_, im_) in pt["result"].items():
        got = rows[lab]
        assert abs(got[0] - re_) <= 1e-6 * abs(re_) + 1e-15, (lab, got, re_)
        assert abs(got[1] - im_) <= 1e-6 * abs(im_) + 1e-15, (lab, got, im_)


@pytest.mark.gpu
def test_cli_two_body_current_point_matches_recorded(tmp_path):
    """GT with the two-body current (one-body part with the Park sign plus the
    cached finite-range field of GT-K0.tbc in the working directory)."""
    g = golden("S40_2bc_fam")
    pt = g["operators"]["GT-K0"][0]
    write_in(tmp_path / "GT-K0.in", pt, g["interaction"], "GT-K0")
    shutil.copyfile(os.path.join(GOLDEN, "S40_2bc_fam.hel"), tmp_path / "hfbtho_output.hel")
    shutil.copyfile(os.path.join(GOLDEN, "S40_2bc_fam", "GT-K0.tbc"), tmp_path / "GT-K0.tbc")
    env = dict(os.environ, PNFAM_GB300_CACHE="off")
    p = subprocess.run([sys.executable, EXE, "GT-K0.in"], cwd=tmp_path, capture_output=True, text=True, env=env)
    assert p.returncode == 0 and p.stderr.strip() == "", p.stderr
    version, conv, t, rows = parse_dat(tmp_path / "GT-K0.dat")
    assert conv == "Yes"
    for lab, (re_, im_) in pt["result"].items():
        got = rows[lab]
        assert abs(got[0] - re_) <= 1e-6 * abs(re_) + 1e-15, (lab, got, re_)
        assert abs(got[1] - im_) <= 1e-6 * abs(im_) + 1e-15, (lab, got, im_)
