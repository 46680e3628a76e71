"""Benchmark: arc-length equilibrium points per second on the shallow cylindrical roof.

Workload (default): Crisfield arc-length (gsALMCrisfield options Length, TolF=1e-8, TolU=1e-6,
Scaling=0, BifurcationMethod=-1) on a degree-2, 128x128-element roof (50,700 dofs, 49,920 free),
point load at the centre, optional seeded modal imperfection.  A step is one accepted arc-length
point (retries after halving the length count as time, not points).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--predictor plain|learned]

Our arm prints one JSON line with value (device-resident points/s, CUDA events on the library
stream), e2e (the same steps through the C-ABI with host vectors copied in and out every step),
roofline (dominant kernel, measured live), cpu_baseline (the FP64 CPU oracle on a bounded sample)
and clocks.  The reference arm (--impl reference) times the FP64 CPU restatement of the
reference path (C++ OpenMP assembly + SuperLU LDL^T stand-in + restated Crisfield) on the same
workload, bounded to a few points.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from gsstructuralanalysis_gb300 import problems as P  # noqa: E402

WORKLOAD = dict(m=128, p=2, load=1.0)
ALM_OPTS = dict(Length=0.02, TolF=1e-8, TolU=1e-6, Scaling=0.0, MaxIter=25, BifurcationMethod=-1)
METRIC = "arc-length path points/s at 50k dofs, learned vs plain predictor, ||R||/||F||<=1e-8"
MAX_RETRIES = 6


def workload_problem(m=None, p=None):
    return P.cylindrical_panel(m=m or WORKLOAD["m"], p=p or WORKLOAD["p"], load=WORKLOAD["load"])


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1"))


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def reduce_max(x, world):
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def host_cores():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    def __init__(self):
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits", "-lms", "200",
                                          "-f", self.path], stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": []}
        if not self.proc:
            return out
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) < 9:
                    continue
                try:
                    sm.append(float(f[1])); mx.append(float(f[2]))
                except ValueError:
                    continue
                for n, v in zip(names, f[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(n)
            os.unlink(self.path)
        except Exception:
            pass
        if sm:
            out = {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                   "samples": len(sm)}
        return out


def step_with_retry(alm, G):
    """One accepted point; on non-convergence halve the length and retry (benchmark_Roof.cpp:420-431)."""
    for _ in range(MAX_RETRIES):
        st = alm.step()
        if st == G.SUCCESS:
            return True
        alm.reduceLength(0.5)
    return False


# ---------------------------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------------------------
def run_ours(args):
    import gsstructuralanalysis_gb300 as G
    from gsstructuralanalysis_gb300 import build as B
    rank, world = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    B.build()
    G.load_library()
    prob = workload_problem()
    if args.imperfection:
        prob = imperfect(prob, G, seed=args.seed + rank)
    gp = G.Problem(prob)
    stats = gp.stats()
    alm = G.ALMCrisfield(gp, ALM_OPTS)
    alm.initialize()
    for _ in range(args.warmup):
        step_with_retry(alm, G)
    gp.sync()
    barrier(world)
    l0 = G.launch_count()
    clk = ClockSampler()
    clk.start()
    gp.record(0)
    t_wall = time.perf_counter()
    pts = 0
    for _ in range(args.steps):
        pts += 1 if step_with_retry(alm, G) else 0
    gp.record(1)
    ms = gp.elapsed_ms(0, 1)
    t_wall = time.perf_counter() - t_wall
    clocks = clk.stop()
    launches = G.launch_count() - l0
    ms = reduce_max(ms, world)
    barrier(world)
    value = world * pts / (ms / 1e3)
    U_end, L_end = alm.solutionU(), alm.solutionL()

    if args.lean:
        # timed leg only (used for ncu launch lists)
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": "points/s", "steps": args.steps,
                              "ms_per_step": ms / max(pts, 1), "gpu_launches": int(launches), "lean": True}))
        return
    # e2e: the same steps again through the C-ABI with host vectors in and out every step
    alm2 = G.ALMCrisfield(gp, ALM_OPTS)
    alm2.initialize()
    U = np.zeros(gp.ndof)
    L = 0.0
    pin_bytes = 8 * gp.ndof
    for _ in range(args.warmup):
        alm2.setSolution(U, L)
        step_with_retry(alm2, G)
        U, L = alm2.solutionU(), alm2.solutionL()
    gp.sync()
    barrier(world)
    t0 = time.perf_counter()
    pts2 = 0
    for _ in range(args.steps):
        alm2.setSolution(U, L)                 # H2D: the step's input state
        pts2 += 1 if step_with_retry(alm2, G) else 0
        U, L = alm2.solutionU(), alm2.solutionL()   # D2H: the step's result
    gp.sync()
    e2e_s = reduce_max(time.perf_counter() - t0, world)
    e2e = {"value": world * pts2 / e2e_s, "unit": "points/s", "h2d_bytes_per_step": pin_bytes,
           "d2h_bytes_per_step": pin_bytes + 8}

    # per-phase profile (separate replay with per-launch CUDA events; not part of `value`)
    prof = profile_phases(G, gp, args)
    roof = roofline(prof, stats, args)

    # residual check of the final point with the oracle's own FP64 assembly is done in tests;
    # here report the library's own convergence measure of the last point
    info = alm.info()
    cpu = None
    if rank == 0 and not args.skip_cpu:
        cpu = cpu_baseline(prob)
    line = {
        "metric": METRIC, "value": value, "unit": "points/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / max(pts, 1), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "config": {"workload": "Crisfield arc-length, shallow cylindrical roof R=2.5 L=2.5 span=0.2 t=0.01, "
                               "degree 2, 128x128 elements (50,700 dofs)",
                   "ndof_free": int(gp.ndof), "nnz": int(gp.nnz), "predictor": args.predictor,
                   "imperfection": bool(args.imperfection), "arc_length": ALM_OPTS["Length"], "TolF": 1e-8,
                   "TolU": 1e-6, "solver": "SimplicialLDLT -> nested-dissection multifrontal LDL^T (FP32 fronts)",
                   "l2": "inputs larger than L2 (multifrontal fronts %.0f MB)" % (stats["front_bytes"] / 1e6),
                   "final_load_factor": L_end, "parallelism": f"replicas x{world}"},
        "e2e": e2e, "gpu_launches": int(launches), "roofline": roof, "cpu_baseline": cpu, "clocks": clocks,
        "phases_ms_per_step": prof["per_step"], "wall_s_timed": t_wall,
        "last_point": {"iterations": info["iterations"], "residueF": info["residueF"]},
    }
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def profile_phases(G, gp, args, nsteps=None):
    nsteps = nsteps or min(args.steps, 20)
    alm = G.ALMCrisfield(gp, ALM_OPTS)
    alm.initialize()
    for _ in range(args.warmup):
        step_with_retry(alm, G)
    gp.sync()
    G.profile_reset()
    G.profile_enable(True)
    for _ in range(nsteps):
        step_with_retry(alm, G)
    gp.sync()
    G.profile_enable(False)
    ph = G.profile_read()
    per_step = {k: v[0] / nsteps for k, v in ph.items()}
    return {"raw": ph, "per_step": per_step, "nsteps": nsteps}


def roofline(prof, stats, args):
    """Dominant phase/kernel vs the measured peaks.  The multifrontal trailing update is a dense
    FP32 GEMM on CUDA cores; its algorithmic work per launch is the factorisation flops divided by
    the update launches (the update does ~all of them)."""
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    raw = prof["raw"]
    upd_ms, upd_n = raw["mf_update"]
    fac_ms, fac_n = raw["factorization"]
    asm_ms, asm_n = raw["assembly"]
    res_ms, res_n = raw["residual"]
    sol_ms, sol_n = raw["solve"]
    hbm = peaks.get("hbm_gbs", 6800.0)
    out = {}
    # factorisation as a whole: flops per factorisation / time per factorisation
    if fac_n:
        t_fac = fac_ms / fac_n / 1e3
        fl = stats["factor_flops"]
        out["factorization"] = {"achieved": fl / t_fac / 1e12, "unit": "TFLOP/s (FP32 CUDA cores)",
                                "ms_per_launch": fac_ms / fac_n, "flops": fl}
    if sol_n:
        # each solve reads the factor (fronts' L parts) once forward and once backward
        bytes_solve = 2 * stats["front_bytes"] / 2
        t = sol_ms / sol_n / 1e3
        out["solve"] = {"achieved": bytes_solve / t / 1e9, "unit": "GB/s", "ms_per_call": sol_ms / sol_n}
    if asm_n:
        t = asm_ms / asm_n / 1e3
        out["assembly"] = {"achieved": stats["tangent_flops"] / t / 1e12, "unit": "TFLOP/s (FP32)",
                           "ms_per_call": asm_ms / asm_n}
    if res_n:
        out["residual_ms"] = res_ms / res_n
    # dominant kernel by time share
    shares = {k: raw[k][0] for k in ("mf_update", "mf_diag", "mf_panel", "solve", "assembly", "residual")}
    dom = max(shares, key=shares.get)
    # the multifrontal trailing update streams W and L tiles and read-modify-writes the front:
    # algorithmic bytes per launch ~ fronts touched; report it against HBM.
    t_upd = upd_ms / max(upd_n, 1) / 1e3
    bytes_upd = 3 * stats["front_bytes"] / max(upd_n / max(fac_n, 1), 1)
    achieved = bytes_upd / t_upd / 1e9 if upd_n else 0.0
    line = {"bound": "hbm", "kernel": "mf_update_kernel", "achieved": achieved, "peak": hbm, "unit": "GB/s",
            "frac": achieved / hbm, "traffic": None, "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)",
            "dominant_phase": dom, "phase_ms": {k: v for k, v in shares.items()}, "detail": out}
    return line


def imperfect(prob, G, seed=0, nmodes=5):
    """Imperfection = sum of the first 5 buckling modes (unit max |w|, sign fixed so that the
    largest |w| entry is positive), amplitudes ~ N(0, (0.01 t)^2) from numpy default_rng(seed)."""
    gp = G.Problem(prob)
    st, vals, vecs = G.buckling(gp, nmodes, shift=-0.5, scaling=1000.0)
    modes = []
    for v in vecs:
        full = np.zeros(prob.ndof_full)
        full[prob.free_index()] = v
        w = full[2 * prob.ncp:]
        if w[np.argmax(np.abs(w))] < 0:
            full = -full
        modes.append(full)
    gp.close()
    amps = np.random.default_rng(seed).normal(0.0, 0.01 * prob.t, size=nmodes)
    return P.add_imperfection(prob, modes, amps)


# ---------------------------------------------------------------------------------------------
# CPU baseline / reference arm: FP64 restatement on the host cores
# ---------------------------------------------------------------------------------------------
def cpu_points(prob, npoints, warm=0):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build_oracle()
    A = O.OracleAssembler(prob, nthreads=host_cores())
    alm = O.ALMCrisfield(A.jacobian, A.al_residual, A.force(), dict(ALM_OPTS))
    for _ in range(warm):
        _cpu_step(alm)
    t0 = time.perf_counter()
    ok = 0
    for _ in range(npoints):
        ok += 1 if _cpu_step(alm) else 0
    dt = time.perf_counter() - t0
    return ok, dt


def _cpu_step(alm):
    for _ in range(MAX_RETRIES):
        if alm.step() == 0:
            return True
        alm.reduce_length(0.5)
    return False


def cpu_baseline(prob):
    n, dt = cpu_points(prob, 1)
    return {"value": n / dt, "unit": "points/s", "cores": host_cores(), "kind": "port",
            "sample": "first arc-length point of the same workload (1 point: FP64 C++ OpenMP assembly on all "
                      "host cores, scipy SuperLU LDL^T stand-in, restated Crisfield logic)"}


def run_reference(args):
    rank, world = dist_env()
    if rank != 0:
        return
    prob = workload_problem()
    npts = max(1, min(args.steps, 3))
    warm = min(args.warmup, 0)
    n, dt = cpu_points(prob, npts, warm)
    value = n / dt
    line = {"metric": METRIC, "value": value, "unit": "points/s", "n_gpus": world, "steps": npts,
            "warmup": warm, "ms_per_step": 1e3 * dt / max(n, 1), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": "Crisfield arc-length, shallow cylindrical roof, degree 2, 128x128 elements "
                                   "(50,700 dofs)", "predictor": "plain"},
            "cpu_baseline": {"value": value, "unit": "points/s", "cores": host_cores(), "kind": "port",
                             "sample": f"first {npts} arc-length points of the workload (bounded sample)"},
            "e2e": {"value": value, "unit": "points/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=197)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--predictor", default="plain", choices=["plain", "learned"])
    ap.add_argument("--imperfection", type=int, default=0)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--lean", action="store_true", help="timed leg only (no e2e / profile / CPU legs)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
