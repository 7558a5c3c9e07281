"""Benchmark: converged FAM omega-points per second at N_sh = 16.

Workload (one "step" = one batch solve to convergence):
  ground state  the recorded 162Gd SkO' solution (tests/golden/Gd162.hel)
                re-diagonalised in the full N_sh = 16 axial HO basis
                (969 Omega>0 states, 33 parity blocks, 1938 states with
                time-reversed partners, largest block 81), 20 x 20 Gauss mesh
  operator      Gamow-Teller beta-, K = 0 (nxy = 94482 FAM matrix elements)
  omega points  a batch of P points of pynfam's CIRCLE contour (centre 10 MeV,
                radius 25 MeV, Gauss-Legendre angles, 2P points, first P used)
  solver        max_iter 300, epsilon 1e-7, Broyden history 50, SkO' residual
                interaction with pynfam's default overrides, FP64 throughout
The same points always converge in the same number of iterations, so each
step does identical work.

Arms:
  default           this repository's GB300 solver through its C ABI
  --impl reference  the reference algorithm on the host CPU cores (the FP64
                    numpy restatement, the only CPU implementation runnable
                    on these machines), timed on a bounded sample
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
INTERACTION = {"interaction_name": "SKOP", "require_self_consistency": True, "require_gauge_invariance": True,
               "force_j2_terms": False, "vpair_t0": -346.352, "override_cs0": 128.279, "override_csr": 0.0,
               "override_cds": 0.0}
SOLVER = {"max_iter": 300, "convergence_epsilon": 1e-7, "broyden_history_size": 50}
METRIC = "converged FAM omega-points/s at N_sh=16 within 1e-6 rel err; p50/p99 point latency"
# mean FAM iterations per converged point of this workload's contour (measured by
# the GPU solver, which follows the same iteration trajectory as the FP64
# restatement); used to turn the CPU arm's per-iteration time into points/s
ITERS_PER_POINT = 26.0


def workload(P):
    from pynfam_gb300.contour import circle
    from pynfam_gb300.namelist import defaults
    from pynfam_gb300.pnfam_setup import setup_case
    from pynfam_gb300.synthetic import ground_state
    hfb = ground_state(HEL, NSH)
    nml = defaults()
    nml["interaction"].update(INTERACTION)
    nml["ext_field"].update(operator_name="GT", operator_k=0, beta_type="-", compute_crossterms=False)
    nml["solver"].update(SOLVER)
    case = setup_case(nml, None, hfb=hfb)
    omegas = circle(-15.0, 35.0, 2 * P)
    return case, omegas


def flops_per_iteration(case):
    """Algorithmic FLOPs of one FAM iteration of one point (reference operation
    counts): block GEMMs 128*S3, density 40*nghl*S2 (+ reduction), field
    projection 48*nghl*S2, all FP64."""
    h = case.hfb
    fc = case.F.mat.cols
    half = h.nb // 2
    tr = lambda i: (i + half) % h.nb
    S2 = sum(int(h.db[i]) * int(h.db[fc[i]]) for i in range(h.nb) if fc[i] >= 0)
    S3 = sum(int(h.db[i]) ** 2 * int(h.db[fc[i]]) for i in range(h.nb) if fc[i] >= 0)
    n = h.nghl
    return {"block_gemm": 128.0 * S3, "density": 40.0 * n * S2 + 240.0 * n * h.dqp,
            "field_projection": 48.0 * n * S2, "S2": S2, "S3": S3}


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, gpu_index):
        self.proc = None
        self.path = os.path.join(ROOT, "gpurun_out", f"clocks_{os.getpid()}.csv")
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
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


def fp64_peak_tflops():
    """cuBLAS DGEMM throughput on this GPU (the FP64 roofline; the driver's
    measured-peaks file has HBM and BF16 figures only)."""
    import torch
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    for _ in range(2):
        torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 1e9
    for _ in range(5):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(); torch.matmul(a, b); e.record(); e.synchronize()
        best = min(best, s.elapsed_time(e) / 1e3)
    return 2.0 * n ** 3 / best / 1e12


def cpu_sample(case, omegas, iters):
    """The FP64 restatement on the host cores: `iters` FAM iterations of one
    point of the workload; returns seconds per iteration."""
    from oracle.fam_oracle import FAMOracle
    orc = FAMOracle(case.hfb, case.couplings, case.F, case.G, quench=case.quench)
    t0 = time.perf_counter()
    orc.solve(complex(omegas[len(omegas) // 2]), max_iter=iters, eps=1e-7, broyden_m=SOLVER["broyden_history_size"])
    return (time.perf_counter() - t0) / iters


def dist_init(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def run_reference(args):
    world, rank, local = dist_init(args)
    if rank != 0:
        return
    case, omegas = workload(args.points)
    cores = os.cpu_count()
    per_iter = []
    for s in range(args.warmup + args.steps):
        dt = cpu_sample(case, omegas, 1)
        if s >= args.warmup:
            per_iter.append(dt)
    t_iter = statistics.mean(per_iter)
    value = 1.0 / (t_iter * ITERS_PER_POINT)
    sample = (f"{args.steps} timed samples of one FAM iteration of one omega point of the workload "
              f"({t_iter:.3f} s each), scaled by {ITERS_PER_POINT} iterations per converged point")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "points/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_iter * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic inputs from a recorded ground state",
            "config": {"workload": f"162Gd SkO' N_sh={NSH} full basis, GT- K=0, CIRCLE contour",
                       "points_per_step": 1, "nghl": case.hfb.nghl, "nxy": case.F.mat.nelem},
            "cpu_baseline": {"value": value, "unit": "points/s", "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "points/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_gpu(args):
    import torch
    world, rank, local = dist_init(args)
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from pynfam_gb300 import _lib
    from pynfam_gb300.solver import GPUSolver
    case, omegas = workload(args.points)
    P = len(omegas)
    s = case.nml["solver"]
    kw = dict(max_iter=s["max_iter"], eps=s["convergence_epsilon"], broyden_m=s["broyden_history_size"],
              quench=case.quench)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MB > L2

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    gpu = GPUSolver(case.hfb, case.couplings)
    gpu.set_operator(case.F, case.G)
    for _ in range(args.warmup):
        r = gpu.solve(omegas, **kw)
    # ---- timed region: device-resident ground state, K batch solves ----
    clocks = Clocks(local)
    barrier()
    dev_ms, wall, launches, iters = [], [], 0, []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = gpu.solve(omegas, **kw)
        wall.append(time.perf_counter() - t0)
        prof, nl = gpu.last_profile()
        dev_ms.append(prof["total"])
        launches += nl
        iters.append(r.iters.copy())
    barrier()
    ck = clocks.stop()
    step_ms = statistics.mean(dev_ms)
    if world > 1:
        t = torch.tensor([step_ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        step_ms = float(t.item())
    nconv = int(np.sum(iters[-1] >= 0))
    value = world * nconv / (step_ms / 1e3)
    mean_iters = float(np.mean(iters[-1][iters[-1] >= 0])) if nconv else float("nan")
    # ---- end to end: host buffers through the C ABI (init + set_operator + solve) ----
    e2e_wall = []
    h2d = 0
    for k in range(2):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        g2 = GPUSolver(case.hfb, case.couplings)
        g2.set_operator(case.F, case.G)
        r2 = g2.solve(omegas, **kw)
        g2.close()
        e2e_wall.append(time.perf_counter() - t0)
    hf = case.hfb
    h2d = 8 * (5 * hf.dqp * hf.nghl + 4 * sum(int(b.size) for b in hf.Up) + 2 * hf.dqp + 5 * hf.nghl
               + case.F.mat.nelem + 2 * P) + 4 * (2 * hf.nb + hf.dqp)
    d2h = 8 * (P * (2 + 1 + 1) + sum(int(i) + 1 for i in r2.iters) * 2)
    e2e_value = world * int(np.sum(r2.iters >= 0)) / min(e2e_wall)
    # ---- per-stage profile of one extra solve (events between stages) ----
    rp = gpu.solve(omegas, timed=True, **kw)
    stages, _ = gpu.last_profile()
    fl = flops_per_iteration(case)
    it_sum = float(np.sum(np.where(rp.iters >= 0, rp.iters, s["max_iter"])))
    stage_flops = {"field_projection": fl["field_projection"] * it_sum, "density": fl["density"] * it_sum,
                   "k1_blockgemm": fl["block_gemm"] / 2 * it_sum, "k2_blockgemm": fl["block_gemm"] / 2 * it_sum}
    dom = max(("field_projection", "density", "k1_blockgemm", "k2_blockgemm"), key=lambda k: stages[k])
    achieved = stage_flops[dom] / (stages[dom] / 1e3) / 1e12
    peak = fp64_peak_tflops()
    total_flops = sum(fl[k] for k in ("block_gemm", "density", "field_projection")) * it_sum
    line = {"metric": METRIC, "value": value, "unit": "points/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic inputs from a recorded ground state",
            "config": {"workload": f"162Gd SkO' N_sh={NSH} full basis (1938 states, 66 blocks, max 81), "
                                   f"GT- K=0, {P} CIRCLE-contour points per step",
                       "points_per_step": P, "nghl": hf.nghl, "nxy": case.F.mat.nelem,
                       "mean_iterations_per_point": mean_iters, "converged_points_per_step": nconv,
                       "l2": "256 MB buffer written between timed steps",
                       "parallelism": f"replicas{world}"},
            "latency_ms": {"p50": float(np.percentile(dev_ms, 50)), "p99": float(np.percentile(dev_ms, 99)),
                           "note": "batch solve: every point of a step completes with the step"},
            "e2e": {"value": e2e_value, "unit": "points/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h)},
            "gpu_launches": launches,
            "stages_ms": {k: round(v, 3) for k, v in stages.items()},
            "achieved_fp64_tflops_whole_solve": total_flops / (stages["total"] / 1e3) / 1e12,
            "roofline": {"bound": "fp64", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak, "traffic": None,
                         "peak_source": "cuBLAS DGEMM 4096^3 measured in this run (no FP64 figure in the measured peaks)"},
            "clocks": ck}
    if rank == 0 and world == 1:
        t_iter = cpu_sample(case, omegas, 2)
        cv = 1.0 / (t_iter * mean_iters)
        line["cpu_baseline"] = {"value": cv, "unit": "points/s", "cores": os.cpu_count(), "kind": "port",
                                "sample": f"2 FAM iterations of one point ({t_iter:.3f} s each) of the same "
                                          f"workload, scaled by the measured {mean_iters:.2f} iterations/point"}
    gpu.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def run_solve_only(args):
    from pynfam_gb300.solver import GPUSolver
    case, omegas = workload(args.points)
    s = case.nml["solver"]
    kw = dict(max_iter=args.max_iter or s["max_iter"], eps=args.eps or s["convergence_epsilon"],
              broyden_m=s["broyden_history_size"] if args.broyden_m is None else args.broyden_m,
              quench=case.quench, precision=args.precision)
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
    ap.add_argument("--points", type=int, default=32)
    ap.add_argument("--impl", default="gb300", choices=("gb300", "reference"))
    ap.add_argument("--precision", type=int, default=0, choices=(0, 1),
                    help="0: FP64 throughout; 1: FP32 field evaluation with FP64 finish")
    ap.add_argument("--eps", type=float, default=None, help="solve-only: convergence epsilon override")
    ap.add_argument("--max-iter", type=int, default=None, help="solve-only: max_iter override")
    ap.add_argument("--broyden-m", type=int, default=None, help="solve-only: Broyden history override")
    ap.add_argument("--timed", action="store_true", help="solve-only: per-stage event timing")
    ap.add_argument("--solve-only", action="store_true",
                    help="warm-up and timed solves only (no e2e/CPU/DGEMM legs); used for kernel profiling")
    args = ap.parse_args()
    if args.solve_only:
        run_solve_only(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
