"""Benchmark: converged FAM omega-points per second at N_sh = 16 within 1e-6
relative error, with p50/p99 point latency.

Workload (one "step" = one serving run of 600 solves to completion):
  ground state  the recorded 162Gd SkO' solution (tests/golden/Gd162.hel)
                re-diagonalised in the full N_sh = 16 axial HO basis
                (969 Omega>0 states, 33 parity blocks, 1938 states with
                time-reversed partners, largest block 81), 20 x 20 Gauss mesh
  operators     beta-: Gamow-Teller K = 0 and K = 1, and the first-forbidden
                operators RS1 K = 0, RS1 K = 1 (each with its cross terms R, RS1, P)
                and RS2 K = 2: one resident context each
  requests      one request per operator per step, each the 120 points of
                pynfam's CIRCLE contour (centre 10 MeV, radius 25 MeV,
                Gauss-Legendre angles, 240 points, first 120 used), all arriving
                at the start of the step; each engine has 64 slots (--slots), so
                the points enter as earlier points retire
  solver        the reference's defaults: max_iter 200, Broyden history 50; SkO'
                residual interaction
  form          the mixed form (FP32 increment evaluations with 3xTF32 tensor-core
                GEMMs, FP64 anchors -- the last ones the defect correction that
                certifies convergence -- FP64 Broyden solve and residual) converged
                to 1e-8 with every strength value settled to 1e-8 (one FP64 anchor
                per point, at si < 1e-5), served by
                continuous-batching engines, one per operator, overlapping on the GPU
A point counts when it converged and its strength and every cross term are
within 1e-6 (relative) of the FP64 fixed point of the same equations (the FP64
form converged to 1e-12, computed once and kept in
tests/golden/bench_fixed_point_nsh16.json).  The plain FP64 form (the drop-in:
the reference's arithmetic and trajectory, epsilon 1e-7) is measured on the
same stream and reported beside it.  The pair-tensor GEMMs are tuned once per
operator when the contexts are set up (outside the timed steps; the choices are
in the line's "autotune" object).

The same line also carries, unless --no-config4 / --no-stream:
  config4         the large-basis stress configuration: a synthetic Bogoliubov
                  state (seed 3) in the full N_sh = 20 basis (blocks up to 231),
                  GT- K = 0, 1 at 256 CIRCLE points each, a fixed number of FAM
                  iterations per point (the random state does not converge):
                  point-iterations/s of both forms and per-stage rates
  serving_stream  a stream of requests for several nuclei and bases (the three
                  recorded ground states in N_sh from {8, 12, 16, 20}), Poisson
                  arrivals at several rates, engines admitted within 150 GB:
                  converged points/s and p50/p99 latency per rate
  finite_range_2bc  (unless --no-2bc) the set-up contraction of the finite-range
                  two-body current for GT- K = 0, 1 of the same ground state
                  (what the reference caches in .tbc files), wall and kernel
                  times, and the 40S N_sh = 6 field against the reference's file
  hfb_reconstruction  (unless --no-hfb) the ground state rebuilt from the .hel
                  fields at N_sh = 16 and 20, on the host and with its arithmetic
                  on the GPU, wall times and the largest differences

Arms:
  default           this repository's GB300 solver through its C ABI
  --impl reference  the reference algorithm on the host CPU cores (the FP64
                    numpy restatement, the only CPU implementation runnable
                    on these machines), timed on a bounded sample: single FAM
                    iterations of points of every operator plus one whole
                    converged point, scaled by the workload's iteration count
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NSH = 16
HEL = os.path.join(ROOT, "tests", "golden", "Gd162.hel")
FIXED_POINT = os.path.join(ROOT, "tests", "golden", "bench_fixed_point_nsh16.json")
INTERACTION = {"interaction_name": "SKOP", "require_self_consistency": True, "require_gauge_invariance": True,
               "force_j2_terms": False, "vpair_t0": -346.352, "override_cs0": 128.279, "override_csr": 0.0,
               "override_cds": 0.0}
# the reference's solver defaults (pnfam_setup.f90:191-195)
SOLVER = {"max_iter": 200, "convergence_epsilon": 1e-7, "broyden_history_size": 50}
# Gamow-Teller K = 0, 1 and first-forbidden K = 0, 1, 2
OPERATORS = (("GT", 0), ("GT", 1), ("RS1", 0), ("RS1", 1), ("RS2", 2))
POINTS = 120
SLOTS = 64
MIXED_EPS = 1e-8
# the mixed form also waits until every strength value has settled to 1e-8 of itself
SETTLE = 8
# ... and takes its FP64 anchor when si < 1e-5 (one per converged point, 1.07 on average)
SWITCH_EXP = 5
TIGHT = 1e-12
# the mixed form's "near its anchor" bound: 10^4 epsilon (the FP32 error of an increment
# evaluation there is ~1e-6 of 1e-5, far below epsilon)
NEAR_EXP = 4
# DRAM traffic (dram__bytes_read.sum + dram__bytes_write.sum) over the algorithmic bytes of
# one pair-tensor GEMM launch, from one ncu capture (N_sh = 12, 16 points)
TRAFFIC_RATIO = {"density_fp32": 1.662e9 / 1.578e9, "field_projection_fp32": 1.773e9 / 1.739e9}
TRAFFIC_SOURCE = "profiles/k_pg_gemm_nsh12.md"
REL = 1e-6
# mixed form: FP64 anchors beside FP32 increments run asynchronously (--async-anchors)
ASYNC_ANCHORS = False
METRIC = "converged FAM omega-points/s at N_sh=16 within 1e-6 rel err; p50/p99 point latency"
WORKLOAD = (f"162Gd SkO' N_sh={NSH} full basis (1938 states, 66 blocks, max 81), 20x20 mesh; beta- GT K=0,1 and "
            f"first-forbidden RS1 K=0,1 (cross terms R, RS1, P) and RS2 K=2; {POINTS} CIRCLE-contour points per "
            f"operator = {POINTS * len(OPERATORS)} solves per step, served")


def opname(op):
    return f"{op[0]}-K{op[1]}"


def workload(P=POINTS, operators=OPERATORS, nsh=NSH):
    """Cases (one per operator, sharing the ground state) and the omega points."""
    from pynfam_gb300.contour import circle
    from pynfam_gb300.namelist import defaults
    from pynfam_gb300.pnfam_setup import setup_case
    from pynfam_gb300.synthetic import ground_state
    hfb = ground_state(HEL, nsh)
    cases = []
    for name, k in operators:
        nml = defaults()
        nml["interaction"].update(INTERACTION)
        nml["ext_field"].update(operator_name=name, operator_k=k, beta_type="-", compute_crossterms=True)
        nml["solver"].update(SOLVER)
        cases.append(setup_case(nml, None, hfb=hfb))
    omegas = circle(-15.0, 35.0, 2 * P)
    return cases, omegas


def flops_per_iteration(case):
    """Algorithmic FLOPs of one FAM iteration of one point (reference operation
    counts): block GEMMs 128*S3, density 40*nghl*S2 (+ reduction), field
    projection 48*nghl*S2."""
    h = case.hfb
    fc = case.F.mat.cols
    S2 = sum(int(h.db[i]) * int(h.db[fc[i]]) for i in range(h.nb) if fc[i] >= 0)
    S3 = sum(int(h.db[i]) ** 2 * int(h.db[fc[i]]) for i in range(h.nb) if fc[i] >= 0)
    n = h.nghl
    return {"block_gemm": 128.0 * S3, "density": 40.0 * n * S2 + 240.0 * n * h.dqp,
            "field_projection": 48.0 * n * S2, "S2": S2, "S3": S3}


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, gpu_index):
        import tempfile
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), f"pnfam_gb300_clocks_{os.getpid()}.csv")
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={gpu_index}",
                 "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                 "clocks_event_reasons.sw_power_cap", "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0])); mx.append(float(f[1]))
            except ValueError:
                continue
            for name, v in zip(names, f[3:7]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def _plain(o):
    """numpy scalars in the JSON line"""
    return o.item() if hasattr(o, "item") else str(o)


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return {}


def dist_init(args):
    from pynfam_gb300 import replicas
    return replicas.env()


def solver_kw(case, precision, eps, **extra):
    s = case.nml["solver"]
    kw = dict(max_iter=s["max_iter"], eps=eps, broyden_m=s["broyden_history_size"], quench=case.quench,
              precision=precision)
    kw.update(extra)
    return kw


def signature(P=POINTS, operators=OPERATORS):
    return {"nsh": NSH, "points": P, "operators": [list(o) for o in operators], "solver": SOLVER,
            "interaction": INTERACTION, "crossterms": True}


def load_fixed_point(P=POINTS, operators=OPERATORS):
    """The committed fixed point of this workload, or None if the file is for another one."""
    try:
        with open(FIXED_POINT) as fh:
            d = json.load(fh)
    except (OSError, ValueError):
        return None
    if d.get("signature") != signature(P, operators):
        return None
    return {tuple(x["operator"]): x for x in d["results"]}


def fixed_point(cases, omegas, P=POINTS, out_dir="."):
    """Per operator: the FP64 fixed point (epsilon 1e-12) of every omega, and the FP64
    form's own run (epsilon 1e-7, the reference's trajectory) with its iteration
    counts: from the committed file when it matches this workload, else computed here
    (untimed) and written to out_dir (--out-dir) for committing."""
    fp = load_fixed_point(P)
    if fp is not None:
        return fp, "file"
    from pynfam_gb300.solver import GPUSolver
    rec = []
    for op, c in zip(OPERATORS, cases):
        g = GPUSolver(c.hfb, c.couplings)
        g.set_operator(c.F, c.G)
        kw = solver_kw(c, 0, TIGHT)
        kw["max_iter"] = 600
        ex = g.solve(omegas, **kw)
        ref = g.solve(omegas, **solver_kw(c, 0, SOLVER["convergence_epsilon"]))
        g.close()
        S = ex.re_S + 1j * ex.im_S
        rec.append({"operator": list(op), "labels": ["Strength"] + [x.label for x in c.G],
                    "S": [[[float(z.real), float(z.imag)] for z in row] if it >= 0 else None
                          for row, it in zip(S, ex.iters)],
                    "iters": ex.iters.tolist(), "iters_ref": ref.iters.tolist(),
                    "S_ref": [[float(z.real), float(z.imag)] for z in ref.re_S[:, 0] + 1j * ref.im_S[:, 0]]})
        print(f"fixed point {opname(op)}: {int(np.sum(ex.iters >= 0))} of {len(omegas)} at {TIGHT}, "
              f"{int(np.sum(ref.iters >= 0))} at {SOLVER['convergence_epsilon']}", file=sys.stderr, flush=True)
    path = os.path.join(out_dir, os.path.basename(FIXED_POINT))
    os.makedirs(out_dir, exist_ok=True)
    with open(path, "w") as fh:
        json.dump({"signature": signature(P), "omegas": [[float(w.real), float(w.imag)] for w in omegas],
                   "how": f"FP64 form, epsilon {TIGHT}, max_iter 600 (S, iters); FP64 form with the "
                          f"reference's settings (iters_ref, S_ref); bench.py", "results": rec},
                  fh, separators=(",", ":"))
    return {tuple(x["operator"]): x for x in rec}, "computed"


class Stream:
    """One serving run of the workload's requests on resident contexts."""

    def __init__(self, cases, omegas, precision, eps, nreq, slots, live=False):
        from pynfam_gb300.solver import GPUSolver
        self.cases, self.omegas, self.precision, self.eps, self.nreq = cases, omegas, precision, eps, nreq
        self.slots = slots
        self.live = live
        self.solvers = {}
        for op, c in zip(OPERATORS, cases):
            g = GPUSolver(c.hfb, c.couplings)
            g.set_operator(c.F, c.G)
            self.solvers[op] = g

    def run(self, timed=False):
        from pynfam_gb300.serve import Request, Server
        kws = {op: solver_kw(c, self.precision, self.eps, live=self.live and not timed,
                             settle=SETTLE if self.precision == 1 else 0,
                             near_exp=NEAR_EXP if self.precision == 1 else 0,
                             switch_exp=SWITCH_EXP if self.precision == 1 else 0,
                             async_anchors=ASYNC_ANCHORS and self.precision == 1)
               for op, c in zip(OPERATORS, self.cases)}

        def factory(key, slots):
            return self.solvers[key].engine(slots, timed=timed, **kws[key])
        reqs = [Request(i * self.nreq + r, op, self.omegas, 0.0) for i, op in enumerate(OPERATORS)
                for r in range(self.nreq)]
        server = Server(factory, lambda key, n: 1, slots=self.slots, budget_bytes=len(OPERATORS))
        out, st = server.run(reqs)
        profs = {op: g.last_profile() for op, g in self.solvers.items()}
        return out, st, profs

    def close(self):
        for g in self.solvers.values():
            g.close()


def score(out, fp, nreq):
    """Per operator and overall: points converged, converged with the strength and
    every cross term within REL of the fixed point, worst relative error."""
    per = {op: {"converged": 0, "within_1e-6": 0, "worst_rel_err": 0.0} for op in OPERATORS}
    for o in out:
        op = OPERATORS[o.rid // nreq]
        if o.iters < 0:
            continue
        d = per[op]
        d["converged"] += 1
        w = fp[op]["S"][o.index]
        if w is None:
            continue
        w = np.array([complex(*x) for x in w])
        scale = max(abs(complex(*x[0])) for x in fp[op]["S"] if x is not None)
        good = True
        for g, v in zip(o.S, w):
            for a, b in ((g.real, v.real), (g.imag, v.imag)):
                err = abs(a - b)
                good &= err <= REL * abs(b) + 1e-12 * scale
                if abs(b) > 1e-9 * scale:
                    d["worst_rel_err"] = max(d["worst_rel_err"], err / abs(b))
        d["within_1e-6"] += int(good)
    tot = {k: sum(d[k] for d in per.values()) for k in ("converged", "within_1e-6")}
    tot["worst_rel_err"] = max(d["worst_rel_err"] for d in per.values())
    return tot, {opname(op): d for op, d in per.items()}


def pair_bytes(case, stage, npts):
    """Algorithmic bytes of one pair-tensor GEMM launch of npts points: the pair tensor
    (TF32 hi + lo: 16 density pairs or 18 projection pairs per element and mesh point,
    plus the pairing parts), the points' operands and results."""
    S2 = flops_per_iteration(case)["S2"]
    n = case.hfb.nghl
    if stage == "density_fp32":
        return (16 + 2) * n * S2 * 8 + npts * 8 * S2 * 8 + npts * 4 * 18 * n * 4
    return (18 + 2) * n * S2 * 8 + npts * (4 * 18 + 4) * n * 8 + npts * 8 * S2 * 4


def cpu_iteration_sample(cases, omegas, n_per_op=1):
    """The FP64 restatement on the host cores: single FAM iterations of a mid-contour
    point of every operator; returns the mean seconds per iteration."""
    from oracle.fam_oracle import FAMOracle
    ts = []
    for c in cases:
        orc = FAMOracle(c.hfb, c.couplings, c.F, c.G, quench=c.quench)
        for _ in range(n_per_op):
            t0 = time.perf_counter()
            orc.solve(complex(omegas[len(omegas) // 2]), max_iter=1, eps=1e-7,
                      broyden_m=SOLVER["broyden_history_size"])
            ts.append(time.perf_counter() - t0)
    return float(np.mean(ts))


def cpu_full_point(cases, omegas, fp):
    """One whole converged point on the host cores (GT K = 0, mid-contour, the
    reference's settings): seconds and iterations, with the iteration count the FP64
    GPU form took for the same point."""
    from oracle.fam_oracle import FAMOracle
    c = cases[0]
    i = len(omegas) // 2
    orc = FAMOracle(c.hfb, c.couplings, c.F, c.G, quench=c.quench)
    t0 = time.perf_counter()
    r = orc.solve(complex(omegas[i]), max_iter=SOLVER["max_iter"], eps=SOLVER["convergence_epsilon"],
                  broyden_m=SOLVER["broyden_history_size"])
    dt = time.perf_counter() - t0
    return {"seconds": dt, "iterations": int(r.iter_conv),
            "gpu_fp64_form_iterations": int(fp[OPERATORS[0]]["iters_ref"][i]) if fp else None,
            "point": f"{opname(OPERATORS[0])} omega = {complex(omegas[i]):.4f}"}


def workload_iterations(fp):
    """FAM iterations of the whole workload in the reference's form (a point that does
    not converge runs to max_iter) and the number of converged points, from the FP64
    form's own run of every point."""
    total, conv = 0, 0
    for op in OPERATORS:
        for it in fp[op]["iters_ref"]:
            total += it if it >= 0 else SOLVER["max_iter"]
            conv += it >= 0
    return total, conv


def run_reference(args):
    world, rank, local = dist_init(args)
    if rank != 0:
        return
    cases, omegas = workload()
    fp = load_fixed_point()
    if fp is None:
        print(json.dumps({"impl": "reference", "unavailable": "the workload's iteration counts "
                          "(tests/golden/bench_fixed_point_nsh16.json) do not match this workload"}), flush=True)
        return
    cores = os.cpu_count()
    per_iter = []
    for s in range(args.warmup + args.steps):
        c = cases[s % len(cases)]
        dt = cpu_iteration_sample([c], omegas)
        if s >= args.warmup:
            per_iter.append(dt)
    t_iter = statistics.mean(per_iter)
    full = cpu_full_point(cases, omegas, fp)
    total, conv = workload_iterations(fp)
    value = conv / (t_iter * total)
    sample = (f"{args.steps} timed single FAM iterations of mid-contour points, rotating over the {len(cases)} "
              f"operators ({t_iter:.3f} s each), scaled by the workload's {total} FAM iterations for {conv} "
              f"converged points (the FP64 form's run of every point, max_iter for the ones that do not "
              f"converge); one whole converged point took {full['seconds']:.1f} s, {full['iterations']} "
              f"iterations ({full['point']}; the FP64 GPU form: {full['gpu_fp64_form_iterations']})")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "points/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_iter * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic inputs from a recorded ground state",
            "config": {"workload": WORKLOAD, "points_per_step": POINTS * len(OPERATORS), "nghl": cases[0].hfb.nghl,
                       "nxy": [int(c.F.mat.nelem) for c in cases]},
            "full_point": full,
            "cpu_baseline": {"value": value, "unit": "points/s", "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "points/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line, default=_plain), flush=True)


def run_gpu(args):
    import torch
    from pynfam_gb300 import replicas
    world, rank, local = dist_init(args)
    torch.cuda.set_device(local)
    replicas.init("nccl")
    cases, omegas = workload(args.points)
    P = len(omegas)
    R = args.requests
    npts = P * len(OPERATORS) * R
    fp, fp_src = fixed_point(cases, omegas, args.points, args.out_dir)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MB > L2

    def barrier():
        replicas.barrier("cuda")

    # ---- the mixed serving form: warm-up, then K timed serving runs ----
    slots = args.slots
    mixed = Stream(cases, omegas, 1, MIXED_EPS, R, slots, live=True)
    for _ in range(args.warmup):
        mixed.run()
    clocks = Clocks(local)
    barrier()
    walls, lat, launches = [], [], 0
    counts = None
    live = {"density_fp32": [0, 0.0], "field_projection_fp32": [0, 0.0]}
    pit32 = pit64 = 0.0
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        ev0.record()
        out, st, profs = mixed.run()
        torch.cuda.synchronize()   # every engine's stream has finished
        ev1.record()
        ev1.synchronize()
        walls.append(ev0.elapsed_time(ev1) / 1e3)
        lat += st.latencies
        for prof, n in profs.values():
            launches += n
            live["density_fp32"][0] += prof["live_density_launches"]
            live["density_fp32"][1] += prof["live_density_ms"]
            live["field_projection_fp32"][0] += prof["live_projection_launches"]
            live["field_projection_fp32"][1] += prof["live_projection_ms"]
            pit32 += prof["point_iterations_fp32"]
            pit64 += prof["point_iterations_fp64"]
        counts = score(out, fp, R)
        unconverged = sum(1 for o in out if o.iters < 0)
    barrier()
    ck = clocks.stop()
    step_s = replicas.max_over_ranks(statistics.mean(walls), "cuda")
    (tot, per_op) = counts
    value = replicas.job_rate(tot["within_1e-6"], step_s, world)
    # ---- per-stage device time of one more run (events between stages, serialised) ----
    out_t, st_t, profs_t = mixed.run(timed=True)
    mixed.close()
    # ---- the plain FP64 form (the drop-in) on the same stream ----
    fp64 = Stream(cases, omegas, 0, SOLVER["convergence_epsilon"], R, slots)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out64, st64, profs64 = fp64.run()
    torch.cuda.synchronize()
    wall64 = time.perf_counter() - t0
    fp64.close()
    tot64, per64 = score(out64, fp, R)
    iters64 = [o.iters for o in out64 if o.iters >= 0]
    # ---- end to end through the public API from host buffers ----
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    s2 = Stream(cases, omegas, 1, MIXED_EPS, R, slots)
    out2, st2, _ = s2.run()
    s2.close()
    e2e_wall = time.perf_counter() - t0
    e2e_ok = score(out2, fp, R)[0]["within_1e-6"]
    hf = cases[0].hfb
    h2d_ctx = 8 * (5 * hf.dqp * hf.nghl + 4 * sum(int(b.size) for b in hf.Up) + 2 * hf.dqp + 5 * hf.nghl) \
        + 4 * (2 * hf.nb + hf.dqp)
    h2d = len(OPERATORS) * h2d_ctx + sum(8 * c.F.mat.nelem * (1 + len(c.G)) for c in cases) + 16 * npts
    d2h = sum(npts // len(OPERATORS) * (16 * (1 + len(c.G)) + 4 + 8 + 8) for c in cases)
    e2e_value = world * e2e_ok / e2e_wall
    # ---- roofline of the dominant FP32 kernel (the pair-tensor GEMMs: HBM-bound) ----
    fl = flops_per_iteration(cases[0])
    stages = {}
    for prof, _ in profs_t.values():
        for k, v in prof.items():
            if k != "total" and not k.startswith("live_") and not k.startswith("tuned_") and k != "autotune_ms":
                stages[k] = stages.get(k, 0.0) + v
    autotune = {opname(op): {"pair_tensor_from_points": int(p["tuned_pair_min_points"]),
                             "density_k_chunks_per_task": int(p["tuned_density_kspan"]),
                             "ms": p["autotune_ms"]}
                for op, (p, _) in profs_t.items()}
    stage_fl = {"field_projection_fp32": fl["field_projection"], "density_fp32": fl["density"]}
    dom = max(live, key=lambda k: live[k][1])
    nl, ms = live[dom]
    pts_per_launch = pit32 / max(nl, 1)
    launch_ms = ms / max(nl, 1)
    alg = pair_bytes(cases[0], dom, pts_per_launch)
    achieved = alg / (launch_ms / 1e3) / 1e9
    # the same launches alone on the GPU: the serialised stage run
    pit32_t = max(stages.get("point_iterations_fp32", 0.0), 1.0)
    alone_ms = stages.get(dom, 0.0) / pit32_t * pts_per_launch
    achieved_alone = alg / max(alone_ms / 1e3, 1e-12) / 1e9
    peaks = measured_peaks()
    peak = peaks.get("hbm_gbs")
    src = "measured STREAM-style copy bandwidth (MEASURED_PEAKS.json hbm_gbs)"
    if peak is None:
        peak = 6800.0
        src = "fallback HBM copy bandwidth 6.8 TB/s"
    bf16 = peaks.get("bf16_tflops_sustained", 1700.0)
    line = {"metric": METRIC, "value": value, "unit": "points/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": step_s * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "fp32 (3xTF32 tensor cores) increments + fp64 anchors and Broyden",
            "data": "synthetic inputs from a recorded ground state",
            "config": {"workload": WORKLOAD, "points_per_step": npts, "nghl": int(hf.nghl),
                       "nxy": {opname(op): int(c.F.mat.nelem) for op, c in zip(OPERATORS, cases)},
                       "solver": SOLVER,
                       "form": f"mixed, epsilon {MIXED_EPS}, strength values settled to 1e-{SETTLE}"
                       + (", asynchronous anchors" if ASYNC_ANCHORS else ""),
                       "engines": len(OPERATORS), "slots_per_engine": slots,
                       "l2": "256 MB buffer written between timed steps",
                       "timing": "CUDA events around each serving run, the device synchronized on both sides "
                                 "(the engines run on their own streams)",
                       "parallelism": f"replicas{world}"},
            "latency_ms": {"p50": float(np.percentile(lat, 50)) * 1e3, "p99": float(np.percentile(lat, 99)) * 1e3,
                           "note": "per point, from request arrival (start of the step) to its result"},
            "accuracy": dict(tot, reference=f"FP64 fixed point (epsilon {TIGHT}), {fp_src}", per_operator=per_op),
            "fp64_form": {"value": world * tot64["within_1e-6"] / wall64, "unit": "points/s", "wall_s": wall64,
                          "converged_per_s": world * tot64["converged"] / wall64,
                          "converged": tot64["converged"], "within_1e-6": tot64["within_1e-6"],
                          "worst_rel_err": tot64["worst_rel_err"],
                          "mean_iterations": float(np.mean(iters64)) if iters64 else None,
                          "per_operator": per64,
                          "note": "the drop-in: FP64 throughout, epsilon 1e-7, same serving stream"},
            "e2e": {"value": e2e_value, "unit": "points/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h),
                    "note": "context creation (ground state and operator upload) + serving run + results"},
            "work": {"fp32_evaluations_per_step": pit32 / args.steps, "fp64_evaluations_per_step": pit64 / args.steps,
                     "evaluations_per_converged_point": (pit32 + pit64) / args.steps / max(tot["converged"], 1),
                     "share_on_unconverged_points": unconverged * SOLVER["max_iter"] / max((pit32 + pit64) / args.steps, 1),
                     "fp64_form_iterations_per_converged_point": float(np.mean(iters64)) if iters64 else None,
                     "note": "evaluations of the timed steps; a point that does not converge runs to max_iter in "
                             "both forms (the reference's rule)"},
            "gpu_launches": launches,
            "stages_ms": {k: round(v, 3) for k, v in stages.items()},
            "stages_note": "one extra serialised run with events between stages (not the timed steps)",
            "autotune": autotune,
            "roofline": {"bound": "hbm", "kernel": f"k_pg_gemm ({dom})", "achieved": achieved, "peak": peak,
                         "unit": "GB/s", "frac": achieved / peak,
                         "traffic": alg * TRAFFIC_RATIO[dom],
                         "traffic_unit": f"DRAM bytes read + written per launch ({pts_per_launch:.1f} points): "
                                         f"algorithmic bytes x the DRAM/algorithmic ratio of one ncu capture "
                                         f"({TRAFFIC_SOURCE}); the pair tensor grows with S2, so the ratio carries",
                         "algorithmic_bytes": alg, "launches": nl, "mean_launch_ms": launch_ms,
                         "points_per_launch": pts_per_launch,
                         "achieved_alone": achieved_alone, "frac_alone": achieved_alone / peak,
                         "mean_launch_ms_alone": alone_ms,
                         "reference_tflops": stage_fl[dom] * pts_per_launch / (launch_ms / 1e3) / 1e12,
                         "reference_tflops_alone": stage_fl[dom] * pts_per_launch / max(alone_ms / 1e3, 1e-12) / 1e12,
                         "tf32_peak_tflops": bf16 / 2,
                         "peak_source": src,
                         "note": "achieved = algorithmic bytes per launch (pair tensor + the points' operands "
                                 "and results) / mean launch time, CUDA events around every launch of the kernel "
                                 "on its own stream in the timed steps, where the five engines' kernels share "
                                 "the GPU; *_alone: the same launches from the serialised stage run; "
                                 "reference_tflops: the reference's operation count of the stage at that rate"},
            "clocks": ck}
    if rank == 0 and world == 1:
        t_iter = cpu_iteration_sample(cases, omegas)
        total, conv = workload_iterations(fp)
        cv = conv / (t_iter * total)
        line["cpu_baseline"] = {"value": cv, "unit": "points/s", "cores": os.cpu_count(), "kind": "port",
                                "sample": f"one FAM iteration of a mid-contour point of each operator "
                                          f"({t_iter:.3f} s each), scaled by the workload's {total} FAM "
                                          f"iterations for {conv} converged points (FP64 form, reference "
                                          f"settings)"}
    if rank == 0 and world == 1 and not args.no_config4:
        line["config4"] = run_config4(args, emit=False)
    if rank == 0 and world == 1 and not args.no_2bc:
        line["finite_range_2bc"] = run_tbc(args, emit=False)
    if rank == 0 and world == 1 and not args.no_hfb:
        line["hfb_reconstruction"] = run_hfb(args, emit=False)
    if rank == 0 and world == 1 and not args.no_stream:
        sl = run_serve_stream(args, emit=False)
        line["serving_stream"] = {
            "config": f"{args.nuclei} nuclei drawn from the recorded 40S, 116Kr, 162Gd ground states re-diagonalised "
                      f"in N_sh from {{{args.nsh}}}; GT- K=0,1 requests of 40-200 CIRCLE points x {args.stream_scale}; "
                      f"Poisson arrivals; {args.budget_gb:g} GB budget; {args.stream_slots} slots per engine",
            "nuclei": sl[0]["nuclei"] if sl else [], "form": sl[0]["form"] if sl else None,
            "rates": [{k: x[k] for k in ("rate_req_per_s", "requests", "points", "converged", "wall_s",
                                         "converged_per_s", "latency_ms", "peak_engines", "peak_gb")} for x in sl]}
    if rank == 0:
        print(json.dumps(line, default=_plain), flush=True)
    replicas.finish()


def run_tbc(args, emit=True):
    """Finite-range two-body-current field: the contraction of the Yukawa part of the
    axial two-body current with the ground-state density matrices, which the
    reference computes once per operator on the CPU and caches in a .tbc file
    (pnfam_extfield_2bc.f90; 1.5-2.5 h per K component at 16 shells with OpenMP,
    per its README_2bc.md).  On the GPU (host table set-up + two kernels): GT- K = 0
    and K = 1 of the benchmark ground state in the N_sh = --tbc-nsh basis, and the
    40S N_sh = 6 GT- K = 0 field of the reference's own runs, checked against the
    reference's .tbc file, beside the CPU oracle's time for that field (unless
    --no-cpu).  Wall times include the host set-up; the kernels' times are CUDA
    events."""
    from pynfam_gb300.extfield import init_external_field
    from pynfam_gb300.extfield_2bc import read_tbc
    from pynfam_gb300.finite_range import gamma_pieces
    from pynfam_gb300.hfb_solution import load_hfb_solution
    from pynfam_gb300.synthetic import ground_state
    gold = os.path.join(ROOT, "tests", "golden")
    s40 = load_hfb_solution(os.path.join(gold, "S40_2bc_fam.hel"))
    F6 = init_external_field(s40, "-", "GT", 0)
    gamma_pieces(s40, F6)                       # CUDA context and module load
    st6 = {}
    t0 = time.perf_counter()
    g6 = gamma_pieces(s40, F6, stats=st6)
    wall6 = time.perf_counter() - t0
    ref = read_tbc(os.path.join(gold, "S40_2bc_fam", "GT-K0.tbc"))
    scale = max(np.abs(v).max() for v in ref.gam.values())
    err6 = max(float(np.abs(g6[k] - ref.gam[k]).max()) for k in ref.gam) / scale
    small = {"workload": "40S (recorded SkO' ground state, N_sh = 6) GT- K=0, 1,640 elements",
             "wall_ms": 1e3 * wall6, "stage1_ms": st6["stage1_ms"], "stage2_ms": st6["stage2_ms"],
             "max_err_vs_reference_tbc": err6}
    if not args.no_cpu:
        from oracle.tbc_oracle import two_body_gamma
        h = s40.hel
        t0 = time.perf_counter()
        two_body_gamma(h.nz, h.nr, h.nl, h.ns, h.ID, h.bz, h.bp, s40.density_matrices("n"),
                       s40.density_matrices("p"), F6.mat.cols, F6.mat.offsets(), F6.mat.nelem, 0, True)
        small["cpu_oracle_s"] = time.perf_counter() - t0
        small["cpu_oracle"] = "numpy restatement of the reference's loops, memoised elements, 1 host core"
    hfb = ground_state(HEL, args.tbc_nsh)
    per_k = []
    for K in (0, 1):
        F = init_external_field(hfb, "-", "GT", K)
        st = {}
        t0 = time.perf_counter()
        gamma_pieces(hfb, F, stats=st)
        wall = time.perf_counter() - t0
        per_k.append({"K": K, "elements": int(F.mat.nelem), "wall_s": wall, "host_ms": st["host_ms"],
                      "stage1_ms": st["stage1_ms"], "stage2_ms": st["stage2_ms"], "radial_groups": st["groups"],
                      "radial_terms": st["terms"], "zpairs": st["pairs"]})
    total_el = sum(x["elements"] for x in per_k)
    total_s = sum(x["wall_s"] for x in per_k)
    obj = {"workload": f"finite-range 2BC field, GT- K=0 and K=1, 162Gd SkO' fields in the full N_sh = "
                       f"{args.tbc_nsh} basis", "per_K": per_k, "elements_per_s": total_el / total_s,
           "s40_nsh6": small,
           "reference_published": "1.5-2.5 h per K component at 16 shells, OpenMP CPU (README_2bc.md)",
           "bound": "FP64 pipe (the Cartesian sums of the radial elements; k_tbc_field)"}
    if emit:
        print(json.dumps({"metric": "finite-range 2BC field elements per second", "value": obj["elements_per_s"],
                          "unit": "elements/s", "n_gpus": 1, "higher_is_better": True, "dtype": "f64",
                          "data": "recorded ground state re-diagonalised", "config": {"workload": obj["workload"]},
                          "finite_range_2bc": obj}, default=_plain), flush=True)
    return obj


def run_hfb(args, emit=True):
    """HFB reconstruction of the benchmark ground state (162Gd SkO' fields in the full
    N_sh = 16 and 20 bases): the host (numpy + LAPACK) form against the form with the
    basis functions, HFB matrices, eigensolves (batched Jacobi) and densities on the
    GPU, wall time of each (after one warm-up of each), and the largest differences
    of the quasiparticle energies (MeV) and of the local density (relative)."""
    from pynfam_gb300.hel import read_hel
    from pynfam_gb300.hfb_solution import load_hfb_solution
    from pynfam_gb300.synthetic import extend_basis
    rows = []
    load_hfb_solution(read_hel(HEL), device=True)
    for nsh in (16, 20):
        h = extend_basis(read_hel(HEL), nsh)
        from pynfam_gb300 import hfb_device
        t = {}
        sol = {}
        for dev in (False, True):
            for k in hfb_device.TIMES:
                hfb_device.TIMES[k] = 0
            t0 = time.perf_counter()
            sol[dev] = load_hfb_solution(h, device=dev)
            t[dev] = time.perf_counter() - t0
        steps = dict(hfb_device.TIMES)
        a, b = sol[False], sol[True]
        rows.append({"nsh": nsh, "states": int(len(h.nr)), "blocks": int(len(h.ID)), "host_s": t[False],
                     "device_s": t[True], "device_calls_s": steps,
                     "max_dE_MeV": float(max(np.abs(a.En - b.En).max(), np.abs(a.Ep - b.Ep).max())),
                     "max_drho_rel": float(max(np.abs(a.rho_n - b.rho_n).max() / np.abs(a.rho_n).max(),
                                               np.abs(a.rho_p - b.rho_p).max() / np.abs(a.rho_p).max()))})
    obj = {"workload": "HFB reconstruction of the 162Gd SkO' ground state in the full N_sh = 16 and 20 bases",
           "rows": rows}
    if emit:
        print(json.dumps({"metric": "HFB reconstruction wall time", "value": rows[0]["device_s"], "unit": "s",
                          "n_gpus": 1, "higher_is_better": False, "dtype": "f64", "data": "recorded fields",
                          "config": {"workload": obj["workload"]}, "hfb_reconstruction": obj}, default=_plain),
              flush=True)
    return obj


def run_serve_stream(args, emit=True):
    """Serving stream (the serving configuration of many nuclei and bases, scaled by --stream-scale):
    nuclei drawn (seeded) from the three recorded ground states (40S, 116Kr, 162Gd)
    re-diagonalised in a basis of N_sh drawn from --nsh, each requesting GT- K = 0
    and K = 1 strengths on a CIRCLE contour of 40-200 points (times the scale);
    Poisson arrivals at each rate of --rates; engines admitted within a device-memory
    budget (--budget-gb, 150 GB); mixed form to 1e-8, values settled to 1e-8.  (The synthetic Bogoliubov
    states of the batching configuration give a FAM iteration that does not converge,
    so they cannot stand in for converged throughput.)  One JSON line per rate."""
    import torch
    from pynfam_gb300.contour import circle
    from pynfam_gb300.namelist import defaults, parse_namelist_text
    from pynfam_gb300.pnfam_setup import setup_case
    from pynfam_gb300.serve import Request, Server, poisson_arrivals, slot_bytes
    from pynfam_gb300.solver import GPUSolver
    from pynfam_gb300.synthetic import ground_state
    rng = np.random.default_rng(args.stream_seed)
    nshs = [int(x) for x in args.nsh.split(",")]
    names = ("S40", "Kr116", "Gd162")
    nuclei = sorted({(str(rng.choice(names)), int(rng.choice(nshs))) for _ in range(args.nuclei)})
    cases, states = {}, {}
    t0 = time.perf_counter()
    for name, nsh in nuclei:
        hfb = ground_state(os.path.join(ROOT, "tests", "golden", f"{name}.hel"), nsh)
        with open(os.path.join(ROOT, "tests", "golden", f"{name}.json")) as fh:
            inter = parse_namelist_text(json.load(fh)["interaction"])["interaction"]
        for k in (0, 1):
            nml = defaults()
            nml["interaction"].update({kk: v for kk, v in inter.items() if v is not None})
            nml["interaction"]["require_self_consistency"] = False
            nml["ext_field"].update(operator_name="GT", operator_k=k, beta_type="-", compute_crossterms=False)
            nml["solver"].update(SOLVER)
            cases[(name, nsh, k)] = setup_case(nml, None, hfb=hfb)
    setup_s = time.perf_counter() - t0
    slots = args.stream_slots
    M = SOLVER["broyden_history_size"]

    def engine_bytes(key, n):
        c = cases[key]
        h = c.hfb
        ground = 12 * (5 * h.dqp * h.nghl + 4 * int(sum(int(b.size) for b in h.Up)))
        return n * slot_bytes(c.F.mat.nelem, M, True) + ground

    def factory(key, n):
        c = cases[key]
        g = GPUSolver(c.hfb, c.couplings)
        g.set_operator(c.F, c.G)
        return g.engine(n, owns_solver=True, **solver_kw(c, 1, MIXED_EPS, settle=SETTLE, near_exp=NEAR_EXP,
                                                                  switch_exp=SWITCH_EXP))

    keys = list(cases)
    npts = {key: max(4, int(round(rng.integers(40, 201) * args.stream_scale))) for key in keys}
    lines = []
    # with several ranks (one GPU each) whole nuclei go to ranks by estimated work
    from pynfam_gb300 import replicas
    world, rank, local = replicas.env()
    if world > 1:
        torch.cuda.set_device(local)
        replicas.init("nccl")
    for rate in [float(x) for x in args.rates.split(",")]:
        arr = poisson_arrivals(len(keys), rate, seed=args.stream_seed)
        order = rng.permutation(len(keys))
        reqs = [Request(i, keys[j], circle(-15.0, 35.0, 2 * npts[keys[j]]), float(arr[i]))
                for i, j in enumerate(order)]
        if world > 1:
            reqs = replicas.partition(reqs, world, cost=lambda r: len(r.omegas) * cases[r.key].F.mat.nelem)[rank]
        torch.cuda.synchronize()
        replicas.barrier("cuda")
        server = Server(factory, engine_bytes, slots=slots, budget_bytes=int(args.budget_gb * 1e9))
        out, st = server.run(reqs)
        torch.cuda.synchronize()
        if world > 1:
            import torch.distributed as dist
            t = torch.tensor([float(st.points), float(st.converged)], dtype=torch.float64, device="cuda")
            dist.all_reduce(t)
            st.points, st.converged = int(t[0].item()), int(t[1].item())
            st.wall = replicas.max_over_ranks(st.wall, "cuda")
        if rank != 0:
            continue
        line = {"serve_stream": True, "rate_req_per_s": rate, "requests": len(reqs),
                "nuclei": [f"{n} N_sh={s_}" for n, s_ in nuclei], "points": st.points, "converged": st.converged,
                "wall_s": st.wall, "points_per_s": st.points / st.wall, "converged_per_s": st.converged / st.wall,
                "latency_ms": {"p50": st.percentile(50) * 1e3, "p99": st.percentile(99) * 1e3},
                "peak_engines": st.peak_engines, "peak_gb": st.peak_bytes / 1e9, "slots_per_engine": slots,
                "setup_s": setup_s, "form": f"mixed, epsilon {MIXED_EPS}, settled to 1e-{SETTLE}",
                "data": "recorded ground states re-diagonalised in larger bases", "ranks": world,
                "latency_note": "p50/p99 over rank 0's points" if world > 1 else "all points"}
        lines.append(line)
        if emit:
            print(json.dumps(line, default=_plain), flush=True)
    return lines


def config4_cases(nsh=20, seed=3):
    """The large-basis stress configuration: the synthetic Bogoliubov state (seed 3) in
    the full N_sh = 20 basis with Omega-only blocks (3542 states, blocks up to 231), GT-
    K = 0 and K = 1 (no cross terms), the benchmark's interaction without the
    self-consistency check (the random state is not self-consistent)."""
    from pynfam_gb300.namelist import defaults
    from pynfam_gb300.pnfam_setup import setup_case
    from pynfam_gb300.synthetic import bogoliubov_nucleus
    hfb = bogoliubov_nucleus(HEL, nsh, seed=seed, parity=False)
    cases = []
    for k in (0, 1):
        nml = defaults()
        nml["interaction"].update(INTERACTION)
        nml["interaction"]["require_self_consistency"] = False
        nml["ext_field"].update(operator_name="GT", operator_k=k, beta_type="-", compute_crossterms=False)
        nml["solver"].update(SOLVER)
        cases.append(setup_case(nml, None, hfb=hfb))
    return hfb, cases


def run_config4(args, emit=True):
    """Large-basis stress: GT- K = 0 and K = 1 at 256 CIRCLE points each on the N_sh = 20
    synthetic state, every point iterated a fixed number of FAM iterations (the random
    state's iteration does not converge, so the measure is FAM point-iterations per
    second), through one continuous-batching engine per operator, in the mixed form and
    in the FP64 form.  A separate timed run gives the per-stage device time, from which
    the stage rates (reference FLOP counts per TF32 or FP64 peak; HBM bytes of the
    pair-tensor stream per measured HBM peak) follow."""
    import torch
    from pynfam_gb300.contour import circle
    from pynfam_gb300.serve import Request, Server
    from pynfam_gb300.solver import GPUSolver
    torch.cuda.set_device(0)
    # the pair tensors of N_sh = 20 (about 62 GB per operator) stay off: the per-block
    # tensor-core kernels evaluate these points
    t0 = time.perf_counter()
    hfb, cases = config4_cases()
    omegas = circle(-15.0, 35.0, 2 * args.c4_points)
    iters = args.c4_iters
    gpus = []
    for c in cases:
        g = GPUSolver(c.hfb, c.couplings)
        g.set_operator(c.F, c.G)
        gpus.append(g)
    setup_s = time.perf_counter() - t0

    def serve(precision, timed=False, npts=None):
        def factory(key, slots):
            c = cases[key]
            return gpus[key].engine(slots, timed=timed, max_iter=iters, eps=1e-300,
                                    broyden_m=c.nml["solver"]["broyden_history_size"], quench=c.quench,
                                    precision=precision, near_exp=NEAR_EXP if precision else 0)
        reqs = [Request(k, k, omegas[:npts], 0.0) for k in range(len(cases))]
        server = Server(factory, lambda key, n: 1, slots=args.c4_slots, budget_bytes=len(cases))
        torch.cuda.synchronize()
        ta = time.perf_counter()
        out, _ = server.run(reqs)
        torch.cuda.synchronize()
        return time.perf_counter() - ta, out

    res = {}
    # the FP64 form (about 40 point-iterations/s here) on the first c4_fp64_points points
    for precision, name, npts in ((1, "mixed", None), (0, "fp64", args.c4_fp64_points)):
        if precision == 1:
            serve(precision)                   # warm-up (FP32 scratch, autotuning)
        wall, out = serve(precision, npts=npts)
        npi = sum(iters if o.iters < 0 else o.iters for o in out)
        res[name] = {"point_iterations_per_s": npi / wall, "wall_s": wall, "point_iterations": npi,
                     "points": len(out)}
    # stage times of the mixed form (serialised, events between stages)
    serve(1, timed=True)
    stages = {}
    pit32 = pit64 = 0.0
    for g in gpus:
        prof = g.last_profile()[0]
        for k, v in prof.items():
            if isinstance(v, (int, float)):
                stages[k] = stages.get(k, 0.0) + v
        pit32 += prof["point_iterations_fp32"]
        pit64 += prof["point_iterations_fp64"]
    peaks = measured_peaks()
    tf32 = peaks["bf16_tflops"] / 2.0
    per_stage = {}
    for stage, key in (("block_gemm", ("k1_blockgemm_fp32", "k2_blockgemm_fp32")),
                       ("density", ("density_fp32",)), ("field_projection", ("field_projection_fp32",))):
        ms = sum(stages.get(k, 0.0) for k in key)
        flops = sum(flops_per_iteration(c)[stage] for c in cases) / len(cases) * pit32
        d = {"ms": ms, "tflops": flops / (ms * 1e-3) / 1e12 if ms > 0 else None}
        d["tensor_frac_of_tf32_peak"] = d["tflops"] / tf32 if d["tflops"] else None
        if stage != "block_gemm":
            key2 = "density_fp32" if stage == "density" else "field_projection_fp32"
            byts = sum(pair_bytes(c, key2, 0) for c in cases) / len(cases)
            d["pair_tensor_gb"] = byts / 1e9
        per_stage[stage] = d
    per_stage["broyden"] = {"ms": stages.get("broyden", 0.0)}
    line = {"config": "large-basis stress (N_sh=20 synthetic Bogoliubov seed 3, Omega-only blocks up to 231, "
                      f"3542 states; GT- K=0,1 at {len(omegas)} CIRCLE points each, {iters} FAM iterations per "
                      f"point, {args.c4_slots} slots per engine)",
            "nxy": {f"GT-K{k}": int(c.F.mat.nelem) for k, c in enumerate(cases)},
            "max_block": int(max(hfb.db)), "setup_s": setup_s,
            "unit": "FAM point-iterations/s", "mixed": res["mixed"], "fp64_form": res["fp64"],
            "mixed_over_fp64": res["mixed"]["point_iterations_per_s"] / res["fp64"]["point_iterations_per_s"],
            "stages_mixed": per_stage, "stage_point_iterations": {"fp32": pit32, "fp64": pit64},
            "note": "stage rates from one serialised run with events between stages; tensor fraction = reference "
                    "FLOPs per second over the TF32 dense peak (half the measured bf16 peak), 3xTF32 issues three "
                    "MMAs per product"}
    for g in gpus:
        g.close()
    if emit:
        print(json.dumps(line), flush=True)
    return line


def run_solve_only(args):
    from pynfam_gb300.solver import GPUSolver
    ops = tuple(OPERATORS[i] for i in (int(x) for x in args.operators.split(",")))
    cases, omegas = workload(args.points, ops, args.nsh_solve)
    case = cases[0]
    s = case.nml["solver"]
    kw = dict(max_iter=args.max_iter or s["max_iter"], eps=args.eps or s["convergence_epsilon"],
              broyden_m=s["broyden_history_size"] if args.broyden_m is None else args.broyden_m,
              quench=case.quench, precision=args.precision, switch_exp=args.switch_exp,
              settle=SETTLE if args.precision == 1 else 0, near_exp=NEAR_EXP if args.precision == 1 else 0)
    gpu = GPUSolver(case.hfb, case.couplings)
    gpu.set_operator(case.F, case.G)
    for _ in range(args.warmup):
        gpu.solve(omegas, **kw)
    ms, its = [], None
    for _ in range(args.steps):
        r = gpu.solve(omegas, timed=args.timed, **kw)
        prof = gpu.last_profile()[0]
        ms.append(prof["total"])
        its = r.iters.tolist()
    gpu.close()
    print(json.dumps({"solve_only": True, "precision": args.precision, "points": len(omegas), "ms": ms,
                      "stages_ms": {k: v for k, v in prof.items() if args.timed},
                      "iters": its, "pit64": prof["point_iterations_fp64"], "pit32": prof["point_iterations_fp32"],
                      "S": [[float(a), float(b)] for a, b in zip(r.re_S[:, 0], r.im_S[:, 0])],
                      "omegas": [[float(w.real), float(w.imag)] for w in omegas]}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--points", type=int, default=POINTS, help="omega points per request")
    ap.add_argument("--requests", type=int, default=1, help="requests per operator per step")
    ap.add_argument("--slots", type=int, default=SLOTS, help="slots per engine")
    ap.add_argument("--impl", default="gb300", choices=("gb300", "reference"))
    ap.add_argument("--precision", type=int, default=0, choices=(0, 1),
                    help="solve-only: 0 FP64 throughout; 1 mixed form")
    ap.add_argument("--eps", type=float, default=None, help="solve-only: convergence epsilon override")
    ap.add_argument("--max-iter", type=int, default=None, help="solve-only: max_iter override")
    ap.add_argument("--broyden-m", type=int, default=None, help="solve-only: Broyden history override")
    ap.add_argument("--timed", action="store_true", help="solve-only: per-stage event timing")
    ap.add_argument("--switch-exp", type=int, default=0,
                    help="solve-only: mixed form takes its first FP64 anchor below si = 10**-switch_exp")
    ap.add_argument("--serve-stream", action="store_true",
                    help="serving stream of several nuclei and bases with Poisson arrivals (one JSON line per rate)")
    ap.add_argument("--nuclei", type=int, default=6, help="serve-stream: nuclei drawn (with repeats)")
    ap.add_argument("--nsh", default="8,12,16,20", help="serve-stream: N_sh values to draw from")
    ap.add_argument("--rates", default="5,50,200", help="serve-stream: request arrival rates (1/s)")
    ap.add_argument("--stream-scale", type=float, default=0.25, help="serve-stream: points per request x scale")
    ap.add_argument("--stream-slots", type=int, default=32, help="serve-stream: slots per engine")
    ap.add_argument("--stream-seed", type=int, default=0)
    ap.add_argument("--budget-gb", type=float, default=150.0)
    ap.add_argument("--out-dir", default=".", help="where a newly computed FP64 fixed point is written")
    ap.add_argument("--nsh-solve", type=int, default=NSH, help="solve-only: N_sh of the basis")
    ap.add_argument("--operators", default="0",
                    help="solve-only: indices into the workload's operator list (first: the one solved)")
    ap.add_argument("--config4", action="store_true",
                    help="the large-basis stress configuration (N_sh = 20) alone, one JSON line")
    ap.add_argument("--c4-points", type=int, default=256, help="config 4: CIRCLE points per operator")
    ap.add_argument("--c4-iters", type=int, default=6, help="config 4: FAM iterations per point")
    ap.add_argument("--c4-slots", type=int, default=16, help="config 4: slots per engine")
    ap.add_argument("--c4-fp64-points", type=int, default=32, help="config 4: points per operator, FP64 form")
    ap.add_argument("--no-config4", action="store_true", help="leave the config 4 object out of the line")
    ap.add_argument("--no-stream", action="store_true", help="leave the serving-stream object out of the line")
    ap.add_argument("--no-2bc", action="store_true", help="leave the finite-range 2BC field object out of the line")
    ap.add_argument("--tbc-only", action="store_true", help="only the finite-range 2BC field timing (own line)")
    ap.add_argument("--hfb-only", action="store_true", help="only the HFB reconstruction timing, host and GPU")
    ap.add_argument("--no-hfb", action="store_true", help="leave the HFB reconstruction object out of the line")
    ap.add_argument("--tbc-nsh", type=int, default=NSH, help="finite-range 2BC field: N_sh of the basis")
    ap.add_argument("--no-cpu", action="store_true", help="finite-range 2BC field: skip the CPU oracle timing")
    ap.add_argument("--async-anchors", action="store_true",
                    help="mixed form: FP64 anchors beside FP32 increments run asynchronously")
    ap.add_argument("--solve-only", action="store_true",
                    help="one operator, batch solves only (no serving, e2e or CPU legs); used for kernel profiling")
    args = ap.parse_args()
    global ASYNC_ANCHORS
    ASYNC_ANCHORS = args.async_anchors
    if args.hfb_only:
        run_hfb(args)
    elif args.tbc_only:
        run_tbc(args)
    elif args.config4:
        run_config4(args)
    elif args.solve_only:
        run_solve_only(args)
    elif args.serve_stream:
        run_serve_stream(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
