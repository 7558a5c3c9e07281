"""The point server: pnfam_main runs handed to a resident process and batched.

Runs on the CPU with a fake device solver: each client is a pnfam_main run in its
own run directory (namelist + .hel, as pynfam prepares them); the server prepares
the points with the real host code, batches the concurrent points of one key into
one solve, and every run directory gets the .dat a standalone run writes.
"""
import json
import os
import shutil
import threading

import numpy as np
import pytest

from golden_cases import GOLDEN, golden
from pynfam_gb300 import pnfam_main
from pynfam_gb300.pointserver import PointServer, submit
from pynfam_gb300.solver import SolveResult
from test_pnfam_main import parse_dat, write_in


class FakeSolver:
    """Strength = (Re w, Im w) of each point; the iteration table converges at 2."""

    def __init__(self, pt, log):
        self.nops = 1 + len(pt.case.G)
        self.log = log

    def solve(self, omegas, history=True, max_iter=300, **kw):
        w = np.asarray(omegas, dtype=complex)
        P = len(w)
        self.log.append(P)
        re = np.repeat(w.real[:, None], self.nops, axis=1)
        im = np.repeat(w.imag[:, None], self.nops, axis=1)
        hist = np.full((P, max_iter + 1, 3), np.nan)
        hist[:, 0] = (1.0, 0.0, 0.0)
        hist[:, 1] = (1e-3, 0.5, 0.5)
        hist[:, 2] = (1e-9, 1.0, 1.0)
        return SolveResult(re, im, np.full(P, 2, dtype=np.int32), np.full(P, 1e-9), hist, 0.0)

    def close(self):
        pass


def _run_dir(tmp_path, name, pt, interaction, op):
    d = tmp_path / name
    d.mkdir()
    write_in(d / f"{op}.in", pt, interaction, op)
    shutil.copyfile(os.path.join(GOLDEN, "S40.hel"), d / "hfbtho_output.hel")
    return d


def test_concurrent_runs_share_one_batch(tmp_path, monkeypatch):
    monkeypatch.setenv("PNFAM_GB300_CACHE", "off")
    g = golden("S40")
    pts = g["operators"]["GT-K0"][:3]
    log = []
    sock = str(tmp_path / "pnfam.sock")
    srv = PointServer(sock, solver_factory=lambda pt: FakeSolver(pt, log), window=1.0).start()
    try:
        dirs = [_run_dir(tmp_path, f"run{i}", p, g["interaction"], "GT-K0") for i, p in enumerate(pts)]
        rcs = [None] * len(dirs)

        def client(i):
            rcs[i] = submit(sock, str(dirs[i]), "GT-K0.in")
        th = [threading.Thread(target=client, args=(i,)) for i in range(len(dirs))]
        for t in th:
            t.start()
        for t in th:
            t.join(timeout=60)
        assert rcs == [0, 0, 0]
        assert log == [3]   # one batch of the three points
        for d, p in zip(dirs, pts):
            version, conv, t, rows = parse_dat(d / "GT-K0.dat")
            assert conv == "Yes" and version
            w = complex(p["namelist"]["real_eqrpa"], p["namelist"]["imag_eqrpa"])
            assert rows["Strength"] == pytest.approx((w.real, w.imag), rel=1e-15)
            assert "Two-body current mode" in open(d / "GT-K0.dat").read()
        # another operator is another key: its own batch and context
        d = _run_dir(tmp_path, "other", g["operators"]["GT-K1"][0], g["interaction"], "GT-K1")
        assert submit(sock, str(d), "GT-K1.in") == 0
        assert log == [3, 1] and len(srv.solvers) == 2
    finally:
        srv.stop()
    assert not os.path.exists(sock)


def test_server_reports_errors_like_a_run(tmp_path, monkeypatch, capsys):
    monkeypatch.setenv("PNFAM_GB300_CACHE", "off")
    g = golden("S40")
    sock = str(tmp_path / "pnfam.sock")
    srv = PointServer(sock, solver_factory=lambda pt: FakeSolver(pt, []), window=0.0).start()
    try:
        d = tmp_path / "nohel"
        d.mkdir()
        write_in(d / "GT-K0.in", g["operators"]["GT-K0"][0], g["interaction"], "GT-K0")
        assert submit(sock, str(d), "GT-K0.in") == 1
        err = capsys.readouterr().err
        assert "hfbtho_output.hel" in err
        assert "Strength" not in open(d / "GT-K0.dat").read()
    finally:
        srv.stop()


class StuckSolver(FakeSolver):
    """A device solve that does not come back until the test releases it."""

    def __init__(self, pt, release):
        super().__init__(pt, [])
        self.release = release

    def solve(self, omegas, **kw):
        self.release.wait(30)
        return super().solve(omegas, **kw)


def test_a_point_that_gets_no_result_fails_instead_of_waiting(tmp_path, monkeypatch, capsys):
    """The server gives up on a point after point_timeout, the client after its own
    timeout; both report a failed run (exit status 1, message on stderr)."""
    monkeypatch.setenv("PNFAM_GB300_CACHE", "off")
    g = golden("S40")
    pt = g["operators"]["GT-K0"][0]
    release = threading.Event()
    sock = str(tmp_path / "pnfam.sock")
    srv = PointServer(sock, solver_factory=lambda p: StuckSolver(p, release), window=0.0,
                      point_timeout=0.5).start()
    try:
        d = _run_dir(tmp_path, "server_gives_up", pt, g["interaction"], "GT-K0")
        assert submit(sock, str(d), "GT-K0.in", timeout=20) == 1
        assert "no result within" in capsys.readouterr().err
        srv.point_timeout = 60.0
        d = _run_dir(tmp_path, "client_gives_up", pt, g["interaction"], "GT-K0")
        assert submit(sock, str(d), "GT-K0.in", timeout=0.5) == 1
        assert "no reply within" in capsys.readouterr().err
    finally:
        release.set()
        srv.stop()


def test_points_queued_at_stop_are_failed(tmp_path, monkeypatch):
    monkeypatch.setenv("PNFAM_GB300_CACHE", "off")
    g = golden("S40")
    sock = str(tmp_path / "pnfam.sock")
    srv = PointServer(sock, solver_factory=lambda p: FakeSolver(p, []), window=0.0)
    pt = pnfam_main.prepare("GT-K0.in", str(_run_dir(tmp_path, "late", g["operators"]["GT-K0"][0],
                                                          g["interaction"], "GT-K0")), sink=[])
    done, box = threading.Event(), {}
    srv.pending.put(("key", pt, done, box))
    srv.stop()          # never started: the queued point is answered with an error
    assert done.is_set() and isinstance(box["error"], RuntimeError)


def test_client_without_server_runs_the_point_itself(tmp_path):
    assert submit(str(tmp_path / "absent.sock"), str(tmp_path), "x.in") is None


@pytest.mark.gpu
def test_point_server_on_the_gpu(tmp_path, monkeypatch):
    """Three concurrent runs of recorded points through the server's device batch:
    the recorded strengths (1e-6), one batch, one context."""
    monkeypatch.setenv("PNFAM_GB300_CACHE", "off")
    g = golden("S40")
    pts = g["operators"]["GT-K0"][:3]
    sock = str(tmp_path / "pnfam.sock")
    srv = PointServer(sock, window=2.0).start()
    try:
        dirs = [_run_dir(tmp_path, f"run{i}", p, g["interaction"], "GT-K0") for i, p in enumerate(pts)]
        rcs = [None] * len(dirs)

        def client(i):
            rcs[i] = submit(sock, str(dirs[i]), "GT-K0.in")
        th = [threading.Thread(target=client, args=(i,)) for i in range(len(dirs))]
        for t in th:
            t.start()
        for t in th:
            t.join(timeout=120)
        assert rcs == [0, 0, 0] and srv.batches == [3] and len(srv.solvers) == 1
        for d, p in zip(dirs, pts):
            _, conv, _, rows = parse_dat(d / "GT-K0.dat")
            assert conv == "Yes"
            for lab, (re_, im_) in p["result"].items():
                got = rows[lab]
                assert abs(got[0] - re_) <= 1e-6 * abs(re_) + 1e-15, (lab, got, re_)
                assert abs(got[1] - im_) <= 1e-6 * abs(im_) + 1e-15, (lab, got, im_)
    finally:
        srv.stop()
