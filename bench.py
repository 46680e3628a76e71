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
ALM_OPTS = dict(Length=0.005, TolF=1e-8, TolU=1e-6, Scaling=0.0, MaxIter=25, BifurcationMethod=-1)
TEST_SEED = 1000          # first held-out imperfection seed (training seeds are 0..n_train-1)
TRAIN_POINTS = 200        # arc-length steps per path, training and test
COARSE_M = 16             # imperfection modes: buckling modes of the 16x16 roof, transferred exactly
METRIC = "arc-length path points/s at 50k dofs, learned vs plain predictor, ||R||/||F||<=1e-8"
MAX_RETRIES = 6
QGEO = 25                 # FP64 values per Gauss point in the device geometry table


def workload_problem(m=None, p=None):
    return P.cylindrical_panel(m=m or WORKLOAD["m"], p=p or WORKLOAD["p"], load=WORKLOAD["load"])


def profiler_range(on):
    """Mark the timed region for a profiler started with --profile-from-start off (CUDA driver
    API cuProfilerStart/Stop on the current context); a no-op when libcuda is absent."""
    try:
        import ctypes
        cu = ctypes.CDLL("libcuda.so.1")
        (cu.cuProfilerStart if on else cu.cuProfilerStop)()
    except OSError:
        pass


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


def alm_options(mode, frozen):
    """Crisfield options of an arm: the reference's for the plain predictor; the guess arms add
    FrozenIterations (the first corrector iterations after a placed guess reuse the held
    factorisation)."""
    return dict(ALM_OPTS, FrozenIterations=int(frozen)) if (mode != "plain" and frozen) else dict(ALM_OPTS)


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
def train_predictor(G, learned, base, modes, args):
    """Training set of the learned predictor: ``args.train_paths`` seeded imperfect roofs (seeds
    0..n-1), each a Crisfield path of TRAIN_POINTS points generated by the library's GPU
    arc-length solver, several paths at a time on separate host threads.  The first
    ``args.pod_paths`` paths (placed extrapolation guesses) give the POD basis and a bootstrap
    network; the other paths are generated with that network's guesses (every point still meets
    the same arc-length constraint and TolF/TolU test, so they are the same equilibrium points)
    and kept as modal projections only.  The final network trains on all paths; the last path is
    held out for early stopping."""
    n_train = max(2, args.train_paths)
    n_pod = max(2, min(args.pod_paths, n_train))

    def fit(paths, Phi):
        samples = sum(max(len(L) - 4, 0) for _, L in paths)
        batch = 128 if samples < 20000 else 256
        epochs = int(np.clip(np.ceil(args.train_updates / max(samples / batch, 1.0)), 10, 400))
        tp = learned.train(G, paths, nm=32, hidden=256, epochs=epochs, batch=batch, lr=1e-3,
                           chunk=max(1, epochs // 40), Phi=Phi)
        return tp, epochs, batch

    t0 = time.perf_counter()
    pod = learned.generate_paths(G, base, modes, range(n_pod), ALM_OPTS, TRAIN_POINTS, workers=args.train_workers)
    Phi = learned.pod_modes(pod, 32)
    paths = [(U @ Phi.T, L) for U, L in pod]
    del pod
    t1 = time.perf_counter()
    boot = None
    if n_train > n_pod:
        boot, _, _ = fit(paths, Phi)
        paths += learned.generate_paths(G, base, modes, range(n_pod, n_train), ALM_OPTS, TRAIN_POINTS,
                                        workers=args.train_workers, Phi=Phi, tp=boot)
    t2 = time.perf_counter()
    tp, epochs, batch = fit(paths, Phi)
    points = int(sum(len(L) - 1 for _, L in paths))
    info = {"paths": n_train, "points_per_path": TRAIN_POINTS, "pod_paths": n_pod,
            "points_generated": points, "samples": tp.nsamples, "epochs": epochs, "batch": batch,
            "path_generation_s": (t1 - t0) + (t2 - t1) - (boot.seconds["train"] if boot else 0.0),
            "path_generation_points_per_s": points / max((t2 - t0) - (boot.seconds["train"] if boot else 0.0), 1e-9),
            "generation": (f"{n_pod} paths with placed cubic-extrapolation guesses, then {n_train - n_pod} with the "
                           f"guesses of a bootstrap network trained on them (held-out error "
                           f"{boot.val_rel_error:.3f} of the extrapolation's)") if boot else
                          f"{n_pod} paths with placed cubic-extrapolation guesses",
            "generation_workers": args.train_workers, "training_s": tp.seconds["train"], "alpha": tp.alpha,
            "best_epoch": tp.best_epoch, "val_rel_error_vs_extrapolation": tp.val_rel_error,
            "seeds": f"0..{n_train - 1} (held out for early stopping: {n_train - 1})"}
    return tp, info


def run_ours(args):
    import gsstructuralanalysis_gb300 as G
    from gsstructuralanalysis_gb300 import build as B, learned
    rank, world = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    B.build()
    G.load_library()
    base = workload_problem()
    t_setup = time.perf_counter()
    modes, bvals, _ = learned.buckling_modes(G, base, nmodes=5, shift=-0.5, coarse=workload_problem(m=COARSE_M))
    tp, train_info = None, None
    if args.predictor == "learned":
        tp, train_info = train_predictor(G, learned, base, modes, args)
    # the test shells: held-out seeds, one device problem each, primed (graphs captured) before timing
    n_prob = max(1, min(args.steps, args.test_problems))
    seeds = [TEST_SEED + (rank * n_prob + i) % 64 for i in range(n_prob)]
    gps = [G.Problem(learned.imperfect_problem(base, modes, sd)) for sd in seeds]
    for g in gps:
        alm = G.ALMCrisfield(g, ALM_OPTS)
        alm.initialize(stability=False)
        alm.step()
        del alm
    t_setup = time.perf_counter() - t_setup
    gp0 = gps[0]
    stats = gp0.stats()

    def make_arm(gp, mode, frozen):
        """A fresh Crisfield path on ``gp`` and its step function.  The guess modes place the
        predicted point and, with frozen > 0, start the corrector on the factorisation the solver
        already holds (FrozenIterations); the plain mode is the reference's tangent predictor."""
        alm = G.ALMCrisfield(gp, alm_options(mode, frozen))
        alm.initialize(stability=False)
        pred = None if mode == "plain" else learned.make_predictor(G, gp, tp, use_net=(mode == "learned"))
        gmi = frozen + 4 if (frozen and pred is not None) else 6

        def one():
            if pred is None:
                return step_with_retry(alm, G)
            st, _ = pred.step(alm, guess_max_iter=gmi)
            return st == G.SUCCESS or step_with_retry(alm, G)
        return alm, pred, one

    def run_path(gp, mode, frozen):
        """One whole TRAIN_POINTS-point path; device time between events on the problem's stream
        (every step synchronises with the host, so the span covers the path's GPU timeline)."""
        alm, pred, one = make_arm(gp, mode, frozen)
        j0 = alm.info()["n_jac"]
        gp.record(2)
        pts = sum(1 for _ in range(TRAIN_POINTS) if one())
        gp.record(3)
        ms = gp.elapsed_ms(2, 3)
        return dict(pts=pts, ms=ms, jac=alm.info()["n_jac"] - j0, L=alm.solutionL())

    def run_arm(mode, frozen, npaths, warm=0):
        for i in range(warm):
            run_path(gps[i % n_prob], mode, frozen)
        for g in gps:
            g.sync()
        barrier(world)
        l0 = G.launch_count()
        profiler_range(True)
        gp0.record(0)
        t_wall = time.perf_counter()
        per = [run_path(gps[i % n_prob], mode, frozen) for i in range(npaths)]
        gp0.record(1)
        profiler_range(False)
        ms = gp0.elapsed_ms(0, 1)
        return dict(per=per, pts=sum(r["pts"] for r in per), ms=ms, wall=time.perf_counter() - t_wall,
                    launches=G.launch_count() - l0,
                    jac_per_point=sum(r["jac"] for r in per) / max(sum(r["pts"] for r in per), 1))

    mode = args.predictor
    clk = ClockSampler()
    clk.start()
    main = run_arm(mode, args.frozen_it, args.steps, args.warmup)
    clocks = clk.stop()
    ms = reduce_max(main["ms"], world)
    barrier(world)
    value = world * main["pts"] / (ms / 1e3)
    launches = main["launches"]
    pts = main["pts"]
    if args.lean:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": "points/s", "steps": args.steps,
                              "ms_per_step": ms / max(args.steps, 1), "gpu_launches": int(launches), "lean": True}))
        return
    # comparison arms on the same test paths (the first n_cmp of the timed ones)
    compare, top = {}, {}
    if mode == "learned":
        n_cmp = max(1, min(args.compare_paths, args.steps))
        same = main["per"][:n_cmp]
        learned_same = sum(r["pts"] for r in same) / (sum(r["ms"] for r in same) / 1e3)
        arms = [("plain", "plain", 0), ("extrapolation", "extrapolation", args.frozen_it)]
        if args.frozen_it:
            arms.append(("learned_full_newton", "learned", 0))
        for name, m, fz in arms:
            r = run_arm(m, fz, n_cmp)
            compare[name] = {"points_per_s": world * r["pts"] / (reduce_max(r["ms"], world) / 1e3),
                             "jacobians_per_point": r["jac_per_point"], "frozen_iterations": fz,
                             "final_load_factors": [x["L"] for x in r["per"]]}
        compare["learned"] = {"points_per_s": learned_same, "jacobians_per_point":
                              sum(r["jac"] for r in same) / max(sum(r["pts"] for r in same), 1),
                              "frozen_iterations": args.frozen_it, "final_load_factors": [x["L"] for x in same]}
        compare["paths"] = n_cmp
        top = {"plain_points_per_s": compare["plain"]["points_per_s"],
               "learned_over_plain": learned_same / compare["plain"]["points_per_s"],
               "network_over_extrapolation": learned_same / compare["extrapolation"]["points_per_s"]}

    # e2e: the same paths again through the C-ABI with host vectors in and out every step
    pin_bytes = 8 * gp0.ndof
    record = []
    gp0.sync()
    barrier(world)
    t0 = time.perf_counter()
    pts2 = 0
    for i in range(args.steps):
        g = gps[i % n_prob]
        alm2, pred2, one2 = make_arm(g, mode, args.frozen_it)
        U, L = np.zeros(g.ndof), 0.0
        for _ in range(TRAIN_POINTS):
            alm2.setSolution(U, L)                 # H2D: the step's input state
            pts2 += 1 if one2() else 0
            U, L = alm2.solutionU(), alm2.solutionL()   # D2H: the step's result
            if i == 0:
                record.append((U, L))
        del alm2, pred2
    for g in gps:
        g.sync()
    e2e_s = reduce_max(time.perf_counter() - t0, world)
    e2e = {"value": world * pts2 / e2e_s, "unit": "points/s", "h2d_bytes_per_step": pin_bytes * TRAIN_POINTS,
           "d2h_bytes_per_step": (pin_bytes + 8) * TRAIN_POINTS}

    prof = profile_phases(G, gps[0], args, lambda: make_arm(gps[0], mode, args.frozen_it)[::2])
    roof = roofline(prof, stats, args)
    cpu, parity = None, None
    if rank == 0 and not args.skip_cpu:
        cpu, parity = cpu_baseline_and_parity(record, gps[0].prob, args.parity_points)
    line = {
        "metric": METRIC, "value": value, "unit": "points/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / max(args.steps, 1), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        **top,
        "config": {"workload": "Crisfield arc-length, shallow cylindrical roof R=2.5 L=2.5 span=0.2 t=0.01, "
                               "degree 2, 128x128 elements (50,700 dofs), imperfection of 5 buckling modes; "
                               f"one step = one {TRAIN_POINTS}-point path of a held-out imperfect roof "
                               f"(test seeds {seeds[0]}..{seeds[-1]}, cycled)",
                   "ndof_free": int(gp0.ndof), "nnz": int(gp0.nnz), "predictor": mode,
                   "points_per_step": TRAIN_POINTS, "points_timed": int(pts),
                   "arc_length": ALM_OPTS["Length"], "TolF": 1e-8, "TolU": 1e-6,
                   "solver": "SimplicialLDLT -> nested-dissection multifrontal LDL^T (FP32 fronts)",
                   "l2": "inputs larger than L2 (multifrontal fronts %.0f MB per roof)" % (stats["front_bytes"] / 1e6),
                   "corrector": ("Crisfield; after a placed guess the first %d iteration(s) reuse the held "
                                 "factorisation (FrozenIterations), then a fresh Jacobian per iteration"
                                 % args.frozen_it) if (mode != "plain" and args.frozen_it) else "Crisfield, full Newton",
                   "final_load_factors": [r["L"] for r in main["per"][:n_prob]],
                   "jacobians_per_point": main["jac_per_point"],
                   "setup_s": t_setup, "training": train_info, "compare": compare,
                   "parallelism": f"replicas x{world}"},
        "e2e": e2e, "gpu_launches": int(launches), "roofline": roof, "cpu_baseline": cpu, "parity": parity,
        "clocks": clocks, "phases_ms_per_point": prof["per_step"], "wall_s_timed": main["wall"],
    }
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def profile_phases(G, gp, args, make_arm, nsteps=40, warm=8):
    """Per-phase device times of the measured arm (serialised launches with CUDA events), per
    point, over ``nsteps`` points after ``warm`` points of a fresh path."""
    alm, one = make_arm()
    for _ in range(warm):
        one()
    gp.sync()
    G.profile_reset()
    G.profile_enable(True)
    for _ in range(nsteps):
        one()
    gp.sync()
    G.profile_enable(False)
    ph = G.profile_read()
    per_step = {k: v[0] / nsteps for k, v in ph.items()}
    return {"raw": ph, "per_step": per_step, "nsteps": nsteps}


def roofline(prof, stats, args):
    """Per-kernel achieved bandwidth / flop rate from CUDA-event launch durations measured live
    (profiling replay) and the algorithmic bytes / flops of each kernel kind; the dominant kind
    (largest time share) is the headline.  Peaks: MEASURED_PEAKS.json (HBM copy bandwidth)."""
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm = peaks.get("hbm_gbs", 6800.0)
    src = "MEASURED_PEAKS.json hbm_gbs (of measured)" if "hbm_gbs" in peaks else "fallback 6.8 TB/s (of fallback)"
    raw = prof["raw"]
    fac_n = max(raw["factorization"][1], 1)
    n_qp, nel = stats["gauss_points"], stats["elements"]
    d = 27  # element dofs (degree 2)
    kinds = {
        # kind: (ms total, launches, algorithmic bytes per launch, flops per launch)
        "mf_update_kernel": (raw["mf_update"][0], raw["mf_update"][1],
                             stats["bytes_update"] / max(stats["launches_update"], 1),
                             2 * stats["flops_update"] / max(stats["launches_update"], 1)),
        "mf_diag_kernel": (raw["mf_diag"][0], raw["mf_diag"][1],
                           stats["bytes_diag"] / max(stats["launches_diag"], 1),
                           2 * stats["flops_diag"] / max(stats["launches_diag"], 1)),
        "mf_panel_kernel": (raw["mf_panel"][0], raw["mf_panel"][1],
                            stats["bytes_panel"] / max(stats["launches_panel"], 1),
                            2 * stats["flops_panel"] / max(stats["launches_panel"], 1)),
        "mf_fwd+bwd (solve)": (raw["solve"][0], raw["solve"][1], stats["solve_bytes"], 0.0),
        "kl_tangent+csr_gather": (raw["assembly"][0], raw["assembly"][1],
                                  n_qp * QGEO * 8 + 2 * nel * d * d * 4 + stats["nnz"] * 8, stats["tangent_flops"]),
        "kl_fint+gather (FP64)": (raw["residual"][0], raw["residual"][1], n_qp * QGEO * 8 + 2 * nel * d * 8, 0.0),
    }
    detail = {}
    for k, (ms, n, byts, fl) in kinds.items():
        if not n:
            continue
        t = ms / n / 1e3
        detail[k] = {"ms_per_point": ms / prof["nsteps"], "avg_launch_us": 1e6 * t,
                     "gbs": byts / t / 1e9, "tflops": fl / t / 1e12, "bytes_per_launch": byts}
    dom = max(detail, key=lambda k: detail[k]["ms_per_point"])
    ach = detail[dom]["gbs"]
    notes = {
        "kl_fint+gather (FP64)": "the residual is bound by FP64 issue (FP64 strains and stresses per Gauss point; "
                                 "ncu: FP64 pipe about 62% of peak), not by HBM; its HBM fraction is reported",
        "mf_fwd+bwd (solve)": "the dataflow triangular solve is bound by its dependency chain across the "
                              "elimination-tree levels (ncu: DRAM about 9% of peak)",
    }
    return {"bound": "hbm", "kernel": dom, "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
            "traffic": None, "peak_source": src,
            "note": notes.get(dom, "multifrontal kernels are bound by the latency of the pivot-tile chain, not by "
                                   "HBM or FLOP rate") + "; per-kernel bandwidth and FLOP rates in detail",
            "factorization_ms": raw["factorization"][0] / fac_n,
            "factorization_tflops_fp32": stats["factor_flops"] / (raw["factorization"][0] / fac_n / 1e3) / 1e12,
            "detail": detail}


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


def cpu_workload_problem():
    """The measured workload with its imperfection computed by the CPU oracle: first 5 buckling
    modes of the 16x16 roof (SuperLU + ARPACK), sign fixed, transferred exactly into the 128x128
    spline space, amplitudes from the same seed."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from gsstructuralanalysis_gb300 import learned
    base = workload_problem()
    coarse = workload_problem(m=COARSE_M)
    A = O.OracleAssembler(coarse, nthreads=host_cores())
    vals, vecs, _ = O.buckling_dense(A.linear(), A.force(), A.jacobian, nev=5, shift=-0.5, scaling=1000.0)
    modes = [P.transfer_field(coarse, m, base) for m in learned.sign_fixed_modes(coarse, vecs.T)]
    a = np.random.default_rng(TEST_SEED).normal(0.0, 0.01 * base.t, size=5)
    return P.add_imperfection(base, modes, a)


def _cpu_step(alm):
    for _ in range(MAX_RETRIES):
        if alm.step() == 0:
            return True
        alm.reduce_length(0.5)
    return False


def cpu_baseline_and_parity(record, gpu_prob, k):
    """CPU baseline and parity of the headline path, after the timed region.

    * residueF at every GPU point of the first recorded path, with the FP64 oracle's residual
      on the identical shell: ||Fint(U) - lambda F|| / ||lambda F|| (gsALMBase.hpp:156-168
      measures the converged point against (lambda + dlambda) F, which is lambda F here);
    * the oracle's own first ``k`` points (plain tangent predictor, restated gsALMCrisfield,
      SuperLU as the SimplicialLDLT stand-in), timed: the CPU baseline;
    * the relative difference of the GPU's first ``k`` points from the oracle's."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build_oracle()
    A = O.OracleAssembler(gpu_prob, nthreads=host_cores())
    F = A.force()
    resF = [float(np.linalg.norm(A.al_residual(U, L)) / np.linalg.norm(L * F)) for U, L in record]
    alm = O.ALMCrisfield(A.jacobian, A.al_residual, F, dict(ALM_OPTS))
    pts = []
    t0 = time.perf_counter()
    for _ in range(k):
        if not _cpu_step(alm):
            break
        pts.append((alm.U.copy(), float(alm.L)))
    dt = time.perf_counter() - t0
    dU = [float(np.linalg.norm(record[i][0] - u) / np.linalg.norm(u)) for i, (u, _) in enumerate(pts)]
    dL = [float(abs(record[i][1] - l) / abs(l)) for i, (_, l) in enumerate(pts)]
    cpu = {"value": len(pts) / dt, "unit": "points/s", "cores": host_cores(), "kind": "port",
           "sample": f"first {len(pts)} arc-length points of the first test path (FP64 C++ OpenMP assembly on "
                     "all host cores, scipy SuperLU LDL^T stand-in, restated gsALMCrisfield, plain predictor)"}
    parity = {"oracle_residueF_max": max(resF), "oracle_residueF_points": len(resF),
              "oracle_residueF_bound": 1e-8, "dU_rel_max": max(dU) if dU else None,
              "dL_rel_max": max(dL) if dL else None, "points_compared": len(pts), "point_bound": 1e-6,
              "ok": bool(max(resF) <= 1e-8 and (not dU or (max(dU) <= 1e-6 and max(dL) <= 1e-6)))}
    return cpu, parity


def run_reference(args):
    rank, world = dist_env()
    if rank != 0:
        return
    prob = cpu_workload_problem()
    npts = max(1, min(args.steps, 3))
    warm = 0
    n, dt = cpu_points(prob, npts, warm)
    value = n / dt
    line = {"metric": METRIC, "value": value, "unit": "points/s", "n_gpus": world, "steps": npts,
            "warmup": warm, "ms_per_step": 1e3 * dt / max(n, 1), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": "Crisfield arc-length, shallow cylindrical roof R=2.5 L=2.5 span=0.2 t=0.01, "
                                   "degree 2, 128x128 elements (50,700 dofs), imperfection of 5 buckling modes "
                                   f"(seed {TEST_SEED})", "predictor": "plain (tangent), the reference's own"},
            "cpu_baseline": {"value": value, "unit": "points/s", "cores": host_cores(), "kind": "port",
                             "sample": f"first {npts} arc-length points of the workload (bounded sample): FP64 C++ "
                                       "OpenMP assembly on all host cores, scipy SuperLU as the SimplicialLDLT "
                                       "stand-in, restated gsALMCrisfield logic"},
            "e2e": {"value": value, "unit": "points/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


# ---------------------------------------------------------------------------------------------
# batched uneven Newton solves (256 panels)
# ---------------------------------------------------------------------------------------------
BATCH_N = 256
BATCH_SEED = 5000
BATCH_OPTS = {"tol": 1e-8, "maxIt": 25, "Refinement": 1}
BATCH_METRIC = "batched Newton solves/s, 256 uneven roof panels (16..96 elements, degree 2/3), |R|/|R0|<=1e-8"


def batch_spec(i, seed=BATCH_SEED):
    """Instance i: elements per direction ~ U{16..96}, degree ~ U{2,3}, thickness log-uniform in
    [0.005, 0.05], imperfection amplitudes ~ N(0, (0.01 t)^2) on 5 buckling modes."""
    rng = np.random.default_rng(seed + i)
    m = int(rng.integers(16, 97))
    p = int(rng.choice([2, 3]))
    t = float(np.exp(rng.uniform(np.log(0.005), np.log(0.05))))
    amps = rng.normal(0.0, 0.01 * t, size=5)
    return m, p, t, amps


def batch_instance(G, i, seed=BATCH_SEED):
    """Imperfect roof with its point load at 50% of the peak load.  Peak load: the lowest linear
    buckling load under the downward central point load of the perfect roof, from a 16x16-element
    patch of the same degree and thickness (the imperfection modes come from the same analysis,
    interpolated into the instance's spline space at its Greville points, exact when nested)."""
    from gsstructuralanalysis_gb300 import learned
    m, p, t, amps = batch_spec(i, seed)
    base = P.cylindrical_panel(m=m, p=p, t=t)
    coarse = P.cylindrical_panel(m=16, p=p, t=t)
    scale = 2560.0 * (t / 0.01) ** 2.5          # keeps the wanted eigenvalues near the shift -0.5
    modes, vals, _ = learned.buckling_modes(G, base, nmodes=5, shift=-0.5, scaling=scale, coarse=coarse)
    neg = [abs(v) for v in vals if v < 0]
    peak = scale * (min(neg) if neg else abs(vals[0]))
    prob = P.add_imperfection(base, modes, amps)
    prob.point_loads = np.array([[0.5, 0.5, 0.0, 0.0, -0.5 * peak]])
    prob.name = f"batch-{i}-p{p}-m{m}"
    return prob, {"m": m, "p": p, "t": t, "peak_load": peak}


def run_batched(args):
    import gsstructuralanalysis_gb300 as G
    from gsstructuralanalysis_gb300 import build as B
    rank, world = dist_env()
    B.build()
    G.load_library()
    n = args.batch
    t0 = time.perf_counter()
    made = [batch_instance(G, rank * n + i) for i in range(n)]
    probs = [pm[0] for pm in made]
    t_inst = time.perf_counter() - t0
    t0 = time.perf_counter()
    bp = G.BatchedProblem(probs)
    info = bp.info()
    t_batch = time.perf_counter() - t0
    t0 = time.perf_counter()
    tune = bp.autotune()
    t_tune = time.perf_counter() - t0
    bn = G.BatchedNewton(bp, BATCH_OPTS)
    for _ in range(args.warmup):
        bn.reset()
        bn.solve()
    bp.sync()
    barrier(world)
    l0 = G.launch_count()
    clk = ClockSampler()
    clk.start()
    profiler_range(True)
    bp.record(0)
    statuses = []
    for _ in range(args.steps):
        bn.reset()
        statuses.append(bn.solve())
    bp.record(1)
    profiler_range(False)
    clocks = clk.stop()
    ms = reduce_max(bp.elapsed_ms(0, 1), world)
    launches = G.launch_count() - l0
    st, its = bn.results()
    value = world * n * args.steps / (ms / 1e3)
    # end to end: the same solves through the public API with every solution read back to host
    U = None
    t0 = time.perf_counter()
    for _ in range(args.steps):
        bn.reset()
        bn.solve()
        U = [bn.solution(i) for i in range(n)]
    e2e_s = reduce_max(time.perf_counter() - t0, world)
    d2h = 8 * sum(len(u) for u in U)
    # size-independent parity: the oracle's FP64 residual at the GPU solutions of a few instances
    check = []
    if rank == 0 and not args.skip_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        order = np.argsort([pm[1]["m"] for pm in made])
        for i in list(order[:2]) + list(order[-1:]):
            A = O.OracleAssembler(probs[i], nthreads=host_cores())
            R = A.residual(U[i])
            check.append({"instance": int(i), "m": made[i][1]["m"], "p": made[i][1]["p"],
                          "rel_residual_oracle": float(np.linalg.norm(R) / np.linalg.norm(A.force()))})
    cpu = None
    if rank == 0 and not args.skip_cpu:
        cpu = batch_cpu_baseline(probs, made)
    hist = {int(k): int(v) for k, v in zip(*np.unique(its, return_counts=True))}
    line = {
        "metric": BATCH_METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "config": {"workload": f"{n} independent imperfect roofs per GPU, one Newton solve each from zero to 50% "
                               "of the linear buckling load (seeded per instance)",
                   "instances": n, "ndof_free_total": int(info["ndof"]), "nnz_total": int(info["nnz"]),
                   "front_pool_GB": info["front_bytes"] / 1e9, "options": BATCH_OPTS,
                   "degree_counts": {str(p): sum(1 for pm in made if pm[1]["p"] == p) for p in (2, 3)},
                   "newton_iterations_histogram": hist, "all_converged": bool((st == 0).all()),
                   "setup_s": {"instances_and_imperfection_modes": t_inst, "batch_symbolic": t_batch,
                               "autotune": t_tune},
                   "autotuned_blocks_per_sm": tune_summary(tune),
                   "l2": "inputs larger than L2 (front pool %.1f GB)" % (info["front_bytes"] / 1e9),
                   "parallelism": f"instances sharded, x{world}"},
        "e2e": {"value": world * n * args.steps / e2e_s, "unit": "solves/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": d2h},
        "gpu_launches": int(launches), "clocks": clocks, "cpu_baseline": cpu, "oracle_residual_check": check,
    }
    if rank == 0:
        print(json.dumps(line))


def run_batched_reference(args):
    """The oracle's CPU Newton on a bounded sample of the batch (its two smallest instances)."""
    import gsstructuralanalysis_gb300 as G
    from gsstructuralanalysis_gb300 import build as B
    rank, world = dist_env()
    if rank != 0:
        return
    B.build()
    G.load_library()
    made = [batch_instance(G, i) for i in range(args.batch)]
    probs = [pm[0] for pm in made]
    cpu = batch_cpu_baseline(probs, made)
    line = {"metric": BATCH_METRIC, "value": cpu["value"], "unit": "solves/s", "n_gpus": world, "steps": 2,
            "warmup": 0, "ms_per_step": 1e3 / cpu["value"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": f"{args.batch} imperfect roofs; bounded sample: {cpu['sample']}"},
            "cpu_baseline": cpu,
            "e2e": {"value": cpu["value"], "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def tune_summary(log):
    best = {}
    for kind, deg, bps, ms in log:
        key = ("tangent" if kind == 0 else "internal_force") + f"_p{int(deg)}"
        if key not in best or ms < best[key][1]:
            best[key] = (int(bps), float(ms))
    return {k: {"blocks_per_sm": v[0], "ms": v[1]} for k, v in best.items()}


def batch_cpu_baseline(probs, made):
    """The oracle's gsStaticNewton restatement (FP64 C++ OpenMP assembly, SuperLU) on the two
    smallest instances: a bounded sample, reported per solve."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    order = np.argsort([pm[1]["m"] for pm in made])[:2]
    t0 = time.perf_counter()
    for i in order:
        A = O.OracleAssembler(probs[i], nthreads=host_cores())
        ref = O.StaticNewton(A.linear(), A.force(), A.jacobian, A.residual, dict(BATCH_OPTS))
        ref.solve()
    dt = time.perf_counter() - t0
    return {"value": len(order) / dt, "unit": "solves/s", "cores": host_cores(), "kind": "port",
            "sample": "the two smallest instances (%s elements per direction): FP64 C++ OpenMP assembly, scipy "
                      "SuperLU, restated gsStaticNewton; the batch's average instance is larger"
                      % ", ".join(str(made[i][1]["m"]) for i in order)}


# ---------------------------------------------------------------------------------------------
# static Newton load ramp (degree 3, 64x64 elements)
# ---------------------------------------------------------------------------------------------
RAMP_M, RAMP_P, RAMP_LOAD, RAMP_STEPS = 64, 3, 30000.0, 10
RAMP_OPTS = {"Solver": "SimplicialLDLT", "tol": 1e-8, "maxIt": 50}
RAMP_METRIC = "static Newton load steps/s, degree-3 64x64 roof (13,467 dofs), 10-step ramp through snap-through"


def centre_deflection(prob, U):
    full = np.zeros(prob.ndof_full)
    full[prob.free_index()] = U
    b1 = P.bspline_basis_matrix(prob.knots1, prob.p, [0.5])[0]
    b2 = P.bspline_basis_matrix(prob.knots2, prob.p, [0.5])[0]
    return float(b2 @ full[2 * prob.ncp:].reshape(prob.n2, prob.n1) @ b1)


def run_ramp(args):
    import gsstructuralanalysis_gb300 as G
    from gsstructuralanalysis_gb300 import build as B
    rank, world = dist_env()
    B.build()
    G.load_library()
    prob = P.cylindrical_panel(m=RAMP_M, p=RAMP_P, load=RAMP_LOAD)
    gp = G.Problem(prob)

    def ramp():
        st = G.StaticNewton(gp, RAMP_OPTS)
        its = []
        for k in range(1, RAMP_STEPS + 1):
            st.setLoad(k / RAMP_STEPS)
            if st.solve() != G.SUCCESS:
                raise RuntimeError(f"load step {k} did not converge")
            its.append(st.iterations())
        return st, its

    for _ in range(args.warmup):
        ramp()
    gp.sync()
    barrier(world)
    l0 = G.launch_count()
    clk = ClockSampler()
    clk.start()
    profiler_range(True)
    gp.record(0)
    for _ in range(args.steps):
        st, its = ramp()
    gp.record(1)
    profiler_range(False)
    clocks = clk.stop()
    ms = reduce_max(gp.elapsed_ms(0, 1), world)
    launches = G.launch_count() - l0
    U = st.solution()
    value = world * RAMP_STEPS * args.steps / (ms / 1e3)
    # end to end through the public API: the ramp with the solution read back after every step
    t0 = time.perf_counter()
    for _ in range(args.steps):
        stn = G.StaticNewton(gp, RAMP_OPTS)
        for k in range(1, RAMP_STEPS + 1):
            stn.setLoad(k / RAMP_STEPS)
            stn.solve()
            stn.solution()
    e2e_s = reduce_max(time.perf_counter() - t0, world)
    cpu, parity = None, None
    if rank == 0 and not args.skip_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        A = O.OracleAssembler(prob, nthreads=host_cores())
        F = A.force()
        R = F - A.fint(U)
        parity = {"rel_residual_oracle_final_step": float(np.linalg.norm(R) / np.linalg.norm(F))}
        t0 = time.perf_counter()
        ref = O.StaticNewton(A.linear(), F / RAMP_STEPS, A.jacobian, lambda x: F / RAMP_STEPS - A.fint(x),
                             dict(tol=1e-8, maxIt=50))
        ref.solve()
        dt = time.perf_counter() - t0
        cpu = {"value": 1.0 / dt, "unit": "load steps/s", "cores": host_cores(), "kind": "port",
               "sample": "the first load step (from zero to 10% of the peak load, past the limit point): FP64 C++ "
                         "OpenMP assembly, scipy SuperLU, restated gsStaticNewton"}
    line = {
        "metric": RAMP_METRIC, "value": value, "unit": "load steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "config": {"workload": f"shallow roof degree {RAMP_P}, {RAMP_M}x{RAMP_M} elements, central point load ramped "
                               f"to {RAMP_LOAD:g} N in {RAMP_STEPS} steps; one step = the whole ramp",
                   "ndof_free": gp.ndof, "options": RAMP_OPTS, "newton_iterations_per_load_step": its,
                   "centre_deflection_over_t": -centre_deflection(prob, U) / prob.t,
                   "l2": "fronts %.0f MB + CSR; working set near L2 size" % (gp.stats()["front_bytes"] / 1e6)},
        "e2e": {"value": world * RAMP_STEPS * args.steps / e2e_s, "unit": "load steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 8 * gp.ndof * RAMP_STEPS},
        "gpu_launches": int(launches), "clocks": clocks, "cpu_baseline": cpu, "parity": parity,
    }
    if rank == 0:
        print(json.dumps(line))


# ---------------------------------------------------------------------------------------------
# linear buckling + modal (degree 3, 256x256 elements)
# ---------------------------------------------------------------------------------------------
EIG_M, EIG_P, EIG_NEV = 256, 3, 20
EIG_SCALING = 5.0e4     # reference load of the buckling analysis: the lowest buckling factors near -1.2
EIG_METRIC = "buckling + modal eigenpairs/s, degree-3 256x256 roof (201,243 dofs), 20 + 20 pairs"


def run_eigen(args):
    import gsstructuralanalysis_gb300 as G
    from gsstructuralanalysis_gb300 import build as B
    import scipy.sparse as sp
    rank, world = dist_env()
    B.build()
    G.load_library()
    prob = P.axial_panel(m=args.eig_m, p=EIG_P)
    gp = G.Problem(prob)
    bopt = {"tolerance": 1e-10, "ncvFac": 3}

    def both():
        st1, bv, bvec = G.buckling(gp, EIG_NEV, shift=args.eig_shift, scaling=EIG_SCALING, options=bopt)
        st2, mv, mvec = G.modal(gp, EIG_NEV, shift=0.0, options=bopt)
        return st1, bv, bvec, st2, mv, mvec

    for _ in range(args.warmup):
        both()
    gp.sync()
    l0 = G.launch_count()
    clk = ClockSampler()
    clk.start()
    profiler_range(True)
    gp.record(0)
    for _ in range(args.steps):
        res = both()
    gp.record(1)
    profiler_range(False)
    clocks = clk.stop()
    ms = gp.elapsed_ms(0, 1)
    launches = G.launch_count() - l0
    st1, bv, bvec, st2, mv, mvec = res
    value = 2 * EIG_NEV * args.steps / (ms / 1e3)
    # parity with the FP64 oracle's matrices (assembled on the host, rank 0): the pre-stress state
    # solves the oracle's K_L u = s F, and the Rayleigh quotients of the GPU eigenvectors with the
    # oracle's K_L, B = K(u_L) - K_L and M -- within the squared residual of an oracle eigenvalue --
    # agree with the GPU eigenvalues
    sn = G.StaticNewton(gp, {"Solver": "SimplicialLDLT", "FrontPrecision": 64, "Refinement": 4, "RefineTol": 1e-15})
    sn.setLoad(EIG_SCALING)
    sn.solveLinear()
    uL = sn.solution()
    parity = None
    if rank == 0 and not args.skip_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        O.build_oracle()
        oa = O.OracleAssembler(prob, nthreads=host_cores())
        KL, M, F = oa.linear(), oa.mass(), oa.force()
        Bm = oa.jacobian(uL) - KL
        rb = [float(np.linalg.norm(KL @ v - lam * (Bm @ v)) / np.linalg.norm(KL @ v)) for lam, v in zip(bv, bvec)]
        rm = [float(np.linalg.norm(KL @ v - lam * (M @ v)) / np.linalg.norm(KL @ v)) for lam, v in zip(mv, mvec)]
        qb = [float(abs((v @ (KL @ v)) / (v @ (Bm @ v)) - lam) / abs(lam)) for lam, v in zip(bv, bvec)]
        qm = [float(abs((v @ (KL @ v)) / (v @ (M @ v)) - lam) / abs(lam)) for lam, v in zip(mv, mvec)]
        parity = {"prestress_rel_residual_oracle": float(np.linalg.norm(KL @ uL - EIG_SCALING * F) /
                                                          np.linalg.norm(EIG_SCALING * F)),
                  "max_rayleigh_rel_diff_buckling": max(qb), "max_rayleigh_rel_diff_modal": max(qm),
                  "max_rel_residual_buckling": max(rb), "max_rel_residual_modal": max(rm), "bound": 1e-6,
                  "ok": bool(max(qb) <= 1e-6 and max(qm) <= 1e-6)}
    cpu = None
    if rank == 0 and not args.skip_cpu:
        cpu = eigen_cpu_baseline()
    line = {
        "metric": EIG_METRIC, "value": value, "unit": "eigenpairs/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "config": {"workload": f"roof degree {EIG_P}, {args.eig_m}x{args.eig_m} elements under uniform axial compression: "
                               f"{EIG_NEV} buckling pairs (shift {args.eig_shift}) + {EIG_NEV} modal pairs (shift 0); "
                               "one step = both analyses",
                   "ndof_free": gp.ndof, "nnz": gp.nnz, "status": [int(st1), int(st2)],
                   "buckling_values": bv.tolist(), "modal_values": mv.tolist(),
                   "l2": "inputs larger than L2 (fronts %.1f GB)" % (gp.stats()["front_bytes"] / 1e9)},
        "e2e": {"value": value, "unit": "eigenpairs/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 8 * gp.ndof * 2 * EIG_NEV},
        "gpu_launches": int(launches), "clocks": clocks, "cpu_baseline": cpu, "parity": parity,
    }
    if rank == 0:
        print(json.dumps(line))


def eigen_cpu_baseline():
    """scipy ARPACK shift-invert (SuperLU) modal analysis with the oracle's FP64 matrices on the
    same roof at 64x64 elements (13k dofs): a bounded sample, per eigenpair."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    prob = P.axial_panel(m=64, p=EIG_P)
    A = O.OracleAssembler(prob, nthreads=host_cores())
    t0 = time.perf_counter()
    K, M = A.linear(), A.mass()
    O.modal(K, M, nev=EIG_NEV, shift=0.0)
    dt = time.perf_counter() - t0
    return {"value": EIG_NEV / dt, "unit": "eigenpairs/s", "cores": host_cores(), "kind": "port",
            "sample": "20 modal pairs of the same roof at 64x64 elements (13k dofs, not the 201k-dof case): FP64 "
                      "C++ OpenMP assembly, scipy SuperLU + ARPACK"}


# ---------------------------------------------------------------------------------------------
# preconditioned CG against the multifrontal LDL^T on the shell tangents
# ---------------------------------------------------------------------------------------------
PCG_METRIC = "linear solves/s on shell tangents: preconditioned CG (Jacobi, nodal block-Jacobi) vs multifrontal LDL^T"


def run_pcg(args):
    """The preconditioned-CG alternatives for the Newton and Lanczos inner systems, measured on the
    tangents of the ramp roof (degree 3, 64x64, K at zero and at the 10%-load solution) and of the
    headline roof (degree 2, 128x128, K at zero): CG to a relative residual of 1e-8 with the
    Jacobi (CGDiagonal) and nodal 3x3 block-Jacobi (GPUPCG) preconditioners, against the
    multifrontal LDL^T (factorisation + solve, FP64 fronts).  One step = every case once."""
    import gsstructuralanalysis_gb300 as G
    from gsstructuralanalysis_gb300 import build as B
    B.build()
    G.load_library()
    cases = []
    for m, p, load, state in ((64, 3, RAMP_LOAD, "zero"), (64, 3, RAMP_LOAD, "load10"), (128, 2, 1.0, "zero")):
        prob = P.cylindrical_panel(m=m, p=p, load=load)
        gp = G.Problem(prob)
        x = np.zeros(gp.ndof)
        if state == "load10":
            sn = G.StaticNewton(gp, {"Solver": "SimplicialLDLT", "tol": 1e-8, "maxIt": 50})
            sn.setLoad(0.1)
            sn.solve()
            x = sn.solution()
        cases.append((f"degree {p}, {m}x{m}, K({state})", gp, x))
    rows = []
    t_all = time.perf_counter()
    for _ in range(max(1, args.steps)):
        rows = []
        for name, gp, x in cases:
            F = gp.force()
            row = {"case": name, "ndof": int(gp.ndof)}
            for sname, opts in (("SimplicialLDLT", {"FrontPrecision": 64}),
                                ("CGDiagonal", {"CGTolerance": 1e-8, "CGMaxIterations": args.cg_max_it}),
                                ("GPUPCG", {"CGTolerance": 1e-8, "CGMaxIterations": args.cg_max_it})):
                S = G.SparseSolver(gp, sname, opts)
                gp.sync()
                t0 = time.perf_counter()
                S.compute_jacobian(x)
                u = S.solve(F)
                gp.sync()
                dt = time.perf_counter() - t0
                K = gp.jacobian(x, 1)
                rel = float(np.linalg.norm(K @ u - F) / np.linalg.norm(F))
                row[sname] = {"s": dt, "iterations": int(S.iterations()), "rel_residual": rel}
            rows.append(row)
    total = time.perf_counter() - t_all
    nsolves = 3 * len(cases) * max(1, args.steps)
    line = {"metric": PCG_METRIC, "value": nsolves / total, "unit": "solves/s", "n_gpus": 1, "steps": args.steps,
            "warmup": 0, "ms_per_step": 1e3 * total / max(1, args.steps), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
            "config": {"workload": "F = K x solves on shell tangents, per solver and case", "cases": rows,
                       "cg_tolerance": 1e-8, "cg_max_iterations": args.cg_max_it}}
    print(json.dumps(line))


# ---------------------------------------------------------------------------------------------
# the hot path's kernels one by one (50k-dof roof)
# ---------------------------------------------------------------------------------------------
KERNELS_METRIC = "Newton iterations/s from device phase times at 50k dofs (tangent + LDL^T, 2-RHS solve, FP64 residual)"


def run_kernels(args):
    """The three device phases of an arc-length iteration on the headline roof (degree 2,
    128x128, 49,920 free dofs) at a deformed state, each timed alone with CUDA events over
    ``steps`` repetitions on the problem's stream: the FP32 tangent with its LDL^T factorisation,
    the two-right-hand-side triangular solve (one persistent launch) and the FP64 residual.
    One step = one of each.  Inputs stay in HBM; the front pool (front_bytes in the config line)
    is larger than L2.  The line is the committed command behind the per-kernel ncu captures."""
    import gsstructuralanalysis_gb300 as G
    from gsstructuralanalysis_gb300 import build as B
    B.build()
    G.load_library()
    gp = G.Problem(workload_problem())
    stats = gp.stats()
    rng = np.random.default_rng(0)
    x = 1e-4 * rng.standard_normal(gp.ndof)
    S = G.SparseSolver(gp, "SimplicialLDLT", {"Refinement": 0})
    b = rng.standard_normal((2, gp.ndof))
    for _ in range(args.warmup):
        S.compute_jacobian(x)
        S.solve(b)
        gp.al_residual(x, 0.5)
    gp.sync()
    G.profile_reset()
    G.profile_enable(True)
    l0 = G.launch_count()
    for _ in range(args.steps):
        S.compute_jacobian(x)
        S.solve(b)
        gp.al_residual(x, 0.5)
    gp.sync()
    G.profile_enable(False)
    ph = G.profile_read()
    launches = G.launch_count() - l0
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm = peaks.get("hbm_gbs", 6800.0)
    ms_fac = ph["factorization"][0] / max(ph["factorization"][1], 1)
    ms_tan = ph["assembly"][0] / max(ph["assembly"][1], 1)
    ms_sol = ph["solve"][0] / max(ph["solve"][1], 1)
    ms_res = ph["residual"][0] / max(ph["residual"][1], 1)
    n_qp, nel, d = stats["gauss_points"], stats["elements"], 27
    res_bytes = n_qp * QGEO * 8 + 2 * nel * d * 8
    detail = {
        "tangent_assembly": {"ms": ms_tan, "tflops_fp32": stats["tangent_flops"] / (ms_tan / 1e3) / 1e12},
        "ldlt_factorisation": {"ms": ms_fac, "tflops_fp32": stats["factor_flops"] / (ms_fac / 1e3) / 1e12},
        "solve_2rhs": {"ms": ms_sol, "algorithmic_bytes": stats["solve_bytes"],
                       "gbs": stats["solve_bytes"] / (ms_sol / 1e3) / 1e9,
                       "frac_of_hbm": stats["solve_bytes"] / (ms_sol / 1e3) / 1e9 / hbm},
        "residual_fp64": {"ms": ms_res, "algorithmic_bytes": res_bytes, "gbs": res_bytes / (ms_res / 1e3) / 1e9},
    }
    total_ms = ms_tan + ms_fac + ms_sol + ms_res
    line = {"metric": KERNELS_METRIC, "value": 1e3 / total_ms, "unit": "iterations/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
            "config": {"workload": "one tangent + factorisation, one 2-RHS solve and one residual of the degree-2 "
                                   "128x128 roof (49,920 free dofs) at a small deformation",
                       "l2": "inputs larger than L2 (fronts %.0f MB)" % (stats["front_bytes"] / 1e6),
                       "hbm_peak_gbs": hbm},
            "kernels": detail, "gpu_launches": int(launches)}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=6,
                    help="timed steps; arc-length: one step = one whole 200-point path of a held-out roof")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--predictor", default="learned", choices=["plain", "extrapolation", "learned"])
    ap.add_argument("--train-paths", type=int, default=512, help="training paths (seeds 0..n-1), 200 points each")
    ap.add_argument("--pod-paths", type=int, default=32, help="training paths whose full vectors give the POD basis")
    ap.add_argument("--train-workers", type=int, default=16, help="paths generated concurrently (host threads)")
    ap.add_argument("--train-updates", type=int, default=40000, help="Adam updates of the training (sets the epochs)")
    ap.add_argument("--test-problems", type=int, default=8, help="distinct held-out roofs the timed paths cycle over")
    ap.add_argument("--compare-paths", type=int, default=2, help="test paths the plain / extrapolation arms run")
    ap.add_argument("--parity-points", type=int, default=3, help="oracle points compared with the GPU path")
    ap.add_argument("--frozen-it", type=int, default=1,
                    help="corrector iterations on the held factorisation after a placed guess (0: full Newton)")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--lean", action="store_true", help="timed leg only (no e2e / profile / CPU legs)")
    ap.add_argument("--workload", default="arc-length", choices=["arc-length", "batched", "ramp", "eigen", "pcg", "kernels"],
                    help="arc-length: the headline path-following workload; batched: 256 uneven Newton solves; "
                         "ramp: degree-3 static Newton load ramp; eigen: buckling + modal at 201k dofs")
    ap.add_argument("--batch", type=int, default=BATCH_N, help="instances per GPU of the batched workload")
    ap.add_argument("--eig-m", type=int, default=EIG_M, help="elements per direction of the eigen workload")
    ap.add_argument("--eig-shift", type=float, default=-1.0, help="buckling shift of the eigen workload")
    ap.add_argument("--cg-max-it", type=int, default=20000, help="CG iteration limit of the pcg workload")
    args = ap.parse_args()
    if args.workload == "pcg":
        return run_pcg(args)
    if args.workload == "kernels":
        return run_kernels(args)
    if args.workload == "ramp":
        return run_ramp(args)
    if args.workload == "eigen":
        return run_eigen(args)
    if args.workload == "batched":
        if args.impl == "reference":
            run_batched_reference(args)
        else:
            run_batched(args)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
