"""A resident point server for the pnfam_main drop-in.

pynfam runs ``pnfam_main.x`` once per omega point, each in its own short-lived
process (pynfam/fortran/pnfam_run.py:140-167), so every point would pay a CUDA
context, the ground-state upload and the operator set-up, and would run alone on
the GPU.  A point server keeps those resident: ``python -m pynfam_gb300.pointserver
<socket>`` listens on a Unix socket; a ``pnfam_main.x`` run with
``PNFAM_GB300_SERVER=<socket>`` sends it its run directory and namelist and waits.
The server prepares the point in that directory (namelist, ``.hel``, operator,
header of the ``.dat``), and points that share a ground state, operator and solver
settings and arrive within ``window`` seconds of each other are solved as one
batch (pnfam_gpu_solve) on a device context kept for that key.  Each point's
``.dat`` is then written exactly as a standalone run writes it, and the client
exits with the run's status and prints its output.

All device work runs on the server's batch thread; connections are handled on
their own threads.  The protocol is one JSON line each way:
``{"cwd": ..., "namelist": ...}`` -> ``{"rc": 0|1, "stdout": ..., "stderr": ...}``.
"""
from __future__ import annotations

import hashlib
import json
import os
import queue
import socket
import sys
import threading
import time

import numpy as np

from . import pnfam_main


# how long a client waits for its point (seconds; $PNFAM_GB300_SERVER_TIMEOUT overrides):
# a server that stops answering fails the point instead of holding pynfam's worker
DEFAULT_TIMEOUT = 3600.0


class _Answered(Exception):
    """A point answered without the device (its stored state had converged)."""


def submit(path: str, cwd: str, nml_path: str, timeout: float = None):
    """Client side: run the point through the server at ``path``.  Returns the run's
    exit status (1 if no reply came within ``timeout`` seconds), or None if no server
    answers there (the caller runs the point)."""
    if timeout is None:
        timeout = float(os.environ.get("PNFAM_GB300_SERVER_TIMEOUT", DEFAULT_TIMEOUT))
    try:
        s = socket.socket(socket.AF_UNIX, socket.SOCK_STREAM)
        s.connect(path)
    except OSError:
        return None
    buf = b""
    with s:
        s.settimeout(timeout)
        try:
            s.sendall((json.dumps({"cwd": os.path.abspath(cwd), "namelist": nml_path}) + "\n").encode())
            while not buf.endswith(b"\n"):
                chunk = s.recv(65536)
                if not chunk:
                    break
                buf += chunk
        except socket.timeout:
            sys.stderr.write(f"pnfam point server: no reply within {timeout:g} s\n")
            return 1
        except OSError as e:
            sys.stderr.write(f"pnfam point server: {e}\n")
            return 1
    try:
        rep = json.loads(buf.decode())
    except ValueError:
        sys.stderr.write("pnfam point server: no reply\n")
        return 1
    if rep.get("stdout"):
        sys.stdout.write(rep["stdout"])
    if rep.get("stderr"):
        sys.stderr.write(rep["stderr"])
    return int(rep.get("rc", 1))


def point_key(pt) -> str:
    """Points with the same key share a device context and a batch: the ground state,
    the operator (namelist &ext_field, two-body-current inputs included), the
    interaction and the solver settings."""
    nml = pt.nml
    h = hashlib.sha256()
    h.update(repr(sorted(nml["ext_field"].items())).encode())
    h.update(repr(sorted(nml["interaction"].items())).encode())
    h.update(repr(sorted(nml["solver"].items())).encode())
    hfb = pt.case.hfb
    for a in (hfb.Ep, hfb.En, hfb.wdcori, pt.case.F.mat.flatten()):
        h.update(a.tobytes())
    if hfb.occupations is not None:
        for a in hfb.occupations:
            h.update(a.tobytes())
    return h.hexdigest()


def gpu_solver(pt):
    """Default device context of a key: the ground state, couplings, occupations and
    operator of its first point."""
    from .solver import GPUSolver
    gpu = GPUSolver(pt.case.hfb, pt.case.couplings, occupations=pt.case.hfb.occupations)
    gpu.set_operator(pt.case.F, pt.case.G)
    return gpu


class PointServer:
    """``solver_factory(point) -> solver`` with ``solve(omegas, history=True, **kw)``
    and ``close()``; ``max_contexts`` device contexts are kept (least recently used
    first out)."""

    def __init__(self, path: str, solver_factory=gpu_solver, window: float = 0.05, max_batch: int = 256,
                 max_contexts: int = 8, point_timeout: float = DEFAULT_TIMEOUT):
        self.path = path
        self.point_timeout = float(point_timeout)
        self.factory = solver_factory
        self.window = float(window)
        self.max_batch = int(max_batch)
        self.max_contexts = int(max_contexts)
        self.pending = queue.Queue()
        self.solvers = {}          # key -> solver, in use order
        self.batches = []          # sizes of the batches solved (for tests and logs)
        self._stop = threading.Event()
        self._sock = None
        self._threads = []

    # -- connections ----------------------------------------------------------
    def _handle(self, conn):
        with conn:
            buf = b""
            while not buf.endswith(b"\n"):
                chunk = conn.recv(65536)
                if not chunk:
                    return
                buf += chunk
            sink = []
            rc, err = 1, ""
            pt = None
            try:
                req = json.loads(buf.decode())
                pt = pnfam_main.prepare(req["namelist"], req["cwd"], sink=sink)
                if pt.done_at_start:
                    pnfam_main.finish(pt, pnfam_main.stored_result(pt), 0, 0.0)
                    rc = 0
                    raise _Answered()
                done = threading.Event()
                box = {}
                if self._stop.is_set():
                    raise RuntimeError("the point server is shutting down")
                self.pending.put((point_key(pt), pt, done, box))
                if not done.wait(self.point_timeout):
                    raise RuntimeError(f"no result within {self.point_timeout:g} s")
                if "error" in box:
                    raise box["error"]
                pnfam_main.finish(pt, box["res"], box["index"], box["seconds"])
                rc = 0
            except _Answered:
                pass
            except Exception as e:
                err = pnfam_main.fail(e, pt.log if pt else None)
            rep = {"rc": rc, "stdout": "".join(l + "\n" for l in sink), "stderr": err}
            try:
                conn.sendall((json.dumps(rep) + "\n").encode())
            except OSError:
                pass

    def _accept(self):
        while not self._stop.is_set():
            try:
                conn, _ = self._sock.accept()
            except socket.timeout:
                continue
            except OSError:
                break
            t = threading.Thread(target=self._handle, args=(conn,), daemon=True)
            t.start()

    # -- batches on the device ------------------------------------------------
    def _solver(self, key, pt):
        if key in self.solvers:
            s = self.solvers.pop(key)
        else:
            while len(self.solvers) >= self.max_contexts:
                old = next(iter(self.solvers))
                self.solvers.pop(old).close()
            s = self.factory(pt)
        self.solvers[key] = s
        return s

    def _batch_loop(self):
        held = []
        while not self._stop.is_set() or held:
            try:
                item = self.pending.get(timeout=0.05)
                held.append((time.monotonic(), item))
            except queue.Empty:
                pass
            while True:   # drain without waiting
                try:
                    held.append((time.monotonic(), self.pending.get_nowait()))
                except queue.Empty:
                    break
            if not held:
                continue
            t0, (key, _, _, _) = held[0]
            same = [h for h in held if h[1][0] == key]
            if time.monotonic() - t0 < self.window and len(same) < self.max_batch and not self._stop.is_set():
                continue
            batch = same[:self.max_batch]
            held = [h for h in held if h not in batch]
            items = [h[1] for h in batch]
            pt0 = items[0][1]
            try:
                gpu = self._solver(key, pt0)
                t = time.perf_counter()
                kw = dict(pt0.solve_kwargs)
                if any(it[1].x0 is not None for it in items):
                    # points with a stored start vector; the others start from X = 0,
                    # whose field is exactly zero, so their iterations are unchanged
                    n = len(items[[it[1].x0 is not None for it in items].index(True)][1].x0)
                    kw["x0"] = np.stack([it[1].x0 if it[1].x0 is not None else np.zeros(n) for it in items])
                if any(it[1].store for it in items):
                    kw["return_state"] = True
                res = gpu.solve([it[1].case.omega for it in items], history=True, **kw)
                dt = time.perf_counter() - t
                self.batches.append(len(items))
                for i, (_, _, done, box) in enumerate(items):
                    box.update(res=res, index=i, seconds=dt)
                    done.set()
            except Exception as e:
                for _, _, done, box in items:
                    box["error"] = e
                    done.set()
        self._fail_pending()

    def _fail_pending(self):
        """Points queued after the batch loop has stopped get an error, not a wait."""
        while True:
            try:
                _, _, done, box = self.pending.get_nowait()
            except queue.Empty:
                return
            box["error"] = RuntimeError("the point server stopped before solving this point")
            done.set()

    # -- lifecycle ------------------------------------------------------------
    def start(self):
        if os.path.exists(self.path):
            os.unlink(self.path)
        self._sock = socket.socket(socket.AF_UNIX, socket.SOCK_STREAM)
        self._sock.bind(self.path)
        self._sock.listen(256)
        self._sock.settimeout(0.2)
        for fn in (self._accept, self._batch_loop):
            t = threading.Thread(target=fn, daemon=True)
            t.start()
            self._threads.append(t)
        return self

    def stop(self):
        self._stop.set()
        for t in self._threads:
            t.join(timeout=5.0)
        if self._sock is not None:
            self._sock.close()
        if os.path.exists(self.path):
            os.unlink(self.path)
        self._fail_pending()
        for s in self.solvers.values():
            s.close()
        self.solvers.clear()


def main(argv=None) -> int:
    argv = sys.argv[1:] if argv is None else argv
    if not argv:
        sys.stderr.write("usage: python -m pynfam_gb300.pointserver <socket> [window_seconds]\n")
        return 2
    srv = PointServer(argv[0], window=float(argv[1]) if len(argv) > 1 else 0.05).start()
    try:
        while True:
            time.sleep(3600)
    except KeyboardInterrupt:
        pass
    finally:
        srv.stop()
    return 0


if __name__ == "__main__":
    sys.exit(main())
