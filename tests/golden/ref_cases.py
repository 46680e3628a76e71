"""Cases whose answers come from the reference's own solver code (golden fixtures).

Each case names a problem builder of gsstructuralanalysis_gb300.problems with its arguments, the
solver and its gsOptionList entries, and the steps to run.  make_ref_fixtures.py runs every case
through oracle/_ref/libref_solvers.so (the reference's gsStaticNewton / gsALM* / gsModalSolver
compiled unchanged) with the FP64 oracle operators and writes ref_solvers.npz;
tests/test_gpu_ref_fixtures.py runs the same cases on the GPU and compares.
"""
from __future__ import annotations

import numpy as np

from gsstructuralanalysis_gb300 import problems as P

ALM_BASE = dict(TolF=1e-8, TolU=1e-6, Scaling=0.0, MaxIter=30, BifurcationMethod=-1)

CASES = {
    # arc-length paths: every converged point (U, lambda) and the corrector iterations
    "crisfield": dict(kind="alm", method="Crisfield", problem=("cylindrical_panel", dict(m=6, p=2, load=1.0)),
                      options=dict(ALM_BASE, Length=0.004), steps=10),
    "riks": dict(kind="alm", method="Riks", problem=("cylindrical_panel", dict(m=6, p=2, load=1e5)),
                 options=dict(ALM_BASE, Length=0.003), steps=5),
    "loadcontrol": dict(kind="alm", method="LoadControl", problem=("cylindrical_panel", dict(m=6, p=2, load=1.0)),
                        options=dict(ALM_BASE, Length=100.0), steps=6),
    "consistent_crisfield": dict(kind="alm", method="ConsistentCrisfield",
                                 problem=("cylindrical_panel", dict(m=6, p=2, load=1.0)),
                                 options=dict(ALM_BASE, Length=0.004), steps=8),
    "crisfield_quasi": dict(kind="alm", method="Crisfield", problem=("cylindrical_panel", dict(m=6, p=2, load=1.0)),
                            options=dict(ALM_BASE, Length=0.004, Quasi=True, QuasiIterations=2), steps=6),
    "crisfield_adaptive": dict(kind="alm", method="Crisfield", problem=("cylindrical_panel", dict(m=6, p=2, load=1.0)),
                               options=dict(ALM_BASE, Length=0.004, AdaptiveLength=True, AdaptiveIterations=3),
                               steps=6),
    # BifurcationMethod 0 (Determinant): stability flag per step through the limit point
    "crisfield_determinant": dict(kind="alm", method="Crisfield", problem=("cylindrical_panel", dict(m=6, p=2, load=1.0)),
                                  options=dict(ALM_BASE, Length=0.006, BifurcationMethod=0), steps=14),
    # setInitialGuess in the reference's own mode (guesses stored with the case)
    "crisfield_guess": dict(kind="alm_guess", method="Crisfield", problem=("cylindrical_panel", dict(m=6, p=2, load=1.0)),
                            options=dict(ALM_BASE, Length=0.004), steps=5),
    "riks_guess": dict(kind="alm_guess", method="Riks", problem=("cylindrical_panel", dict(m=6, p=2, load=1e5)),
                       options=dict(ALM_BASE, Length=0.003), steps=5),
    # gsStaticNewton from zero, and a load ramp continued from the previous solution
    "newton": dict(kind="newton", problem=("cylindrical_panel", dict(m=6, p=3, load=800.0)),
                   options=dict(tol=1e-8, maxIt=30, Solver="SimplicialLDLT"), loads=[1.0]),
    "newton_ramp": dict(kind="newton", problem=("cylindrical_panel", dict(m=8, p=3, load=30000.0)),
                        options=dict(tol=1e-8, maxIt=50, Solver="SimplicialLDLT"), loads=[0.2, 0.4, 0.6, 0.8, 1.0]),
    # gsModalSolver::compute (all pairs) and ::computePower
    "modal_dense": dict(kind="eigen", problem=("flat_plate", dict(m=4, p=2, bc="simply")), options=dict(tolerance=1e-12)),
}


def build(case: dict):
    name, kw = case["problem"]
    return getattr(P, name)(**kw)


def guesses(U_prev, L_prev, U, L, k, n):
    """The host guess of step k (k >= 2): the linear extrapolation of the last two points plus a
    seeded perturbation of 1e-3 of the last increment."""
    rng = np.random.default_rng(1000 + k)
    dU = U - U_prev
    return 2 * U - U_prev + 1e-3 * np.linalg.norm(dU) * rng.standard_normal(n) / np.sqrt(n), 2 * L - L_prev
