"""Failure paths of the GPU solvers, driven from the host only (no device fault is provoked).

The reference maps ``throw 1/2/3`` inside its solvers to gsStatus NotConverged, AssemblyError
and SolverError and never lets an exception cross the public API (gsStaticNewton.hpp:75-98,
gsALMBase.hpp:328-351).  Each test builds the failing input on the host -- too few iterations,
a stiffness that is exactly zero, a NaN in a host input copy, a deliberately wrong learned
guess -- checks the status the library returns, and then checks that the same context still
solves a good problem (the kernels returned normally).
"""
import time

import numpy as np
import pytest

from gsstructuralanalysis_gb300 import problems as P

pytestmark = pytest.mark.gpu

NOT_CONVERGED, ASSEMBLY_ERROR, SOLVER_ERROR = 1, 2, 3


def _context_still_solves(G):
    prob = P.flat_plate(m=4, p=2)
    gp = G.Problem(prob)
    st = G.StaticNewton(gp, {"Solver": "SimplicialLDLT", "Refinement": 4})
    assert st.solveLinear() == G.SUCCESS
    assert np.isfinite(st.solution()).all()


def test_static_newton_max_iterations_is_not_converged(lib, oracle_mod):
    """maxIt = 1 on a nonlinear load: gsStaticNewton throws 1 -> NotConverged (both)."""
    import gsstructuralanalysis_gb300 as G
    prob = P.cylindrical_panel(m=6, p=3, load=800.0)
    gp, oa = G.Problem(prob), oracle_mod.OracleAssembler(prob)
    for solver in ("SimplicialLDLT", "CGDiagonal"):
        st = G.StaticNewton(gp, {"Solver": solver, "tol": 1e-8, "maxIt": 1})
        assert st.solve() == NOT_CONVERGED
    ref = oracle_mod.StaticNewton(oa.linear(), oa.force(), oa.jacobian, oa.residual, dict(tol=1e-8, maxIt=1))
    assert ref.solve() == NOT_CONVERGED
    _context_still_solves(G)


def test_arc_length_max_iterations_is_not_converged(lib, oracle_mod):
    """MaxIter = 2 leaves one corrector iteration: the step throws 1 -> NotConverged, and the
    solver state stays at the last converged point (both)."""
    import gsstructuralanalysis_gb300 as G
    prob = P.cylindrical_panel(m=8, p=2, load=1.0)
    gp, oa = G.Problem(prob), oracle_mod.OracleAssembler(prob)
    opts = dict(Length=0.004, TolF=1e-12, TolU=1e-12, Scaling=0.0, MaxIter=2, BifurcationMethod=-1)
    alm = G.ALMCrisfield(gp, opts)
    alm.initialize()
    ref = oracle_mod.ALMCrisfield(oa.jacobian, oa.al_residual, oa.force(), opts)
    assert alm.step() == NOT_CONVERGED
    assert ref.step() == NOT_CONVERGED
    assert np.all(alm.solutionU() == 0.0) and alm.solutionL() == 0.0
    _context_still_solves(G)


def test_zero_stiffness_is_solver_error(lib, oracle_mod):
    """E = 0 makes K exactly zero: the first pivot of the LDL^T is zero, the diagonal-tile
    kernel sets the factorisation's status word, and the solve reports SolverError (the
    reference: factorisation failure -> throw 3).  The oracle's LDL^T stand-in fails too."""
    import gsstructuralanalysis_gb300 as G
    prob = P.flat_plate(m=4, p=2, E=0.0)
    gp, oa = G.Problem(prob), oracle_mod.OracleAssembler(prob)
    for prec in (32, 64):
        st = G.StaticNewton(gp, {"Solver": "SimplicialLDLT", "FrontPrecision": prec})
        assert st.solveLinear() == SOLVER_ERROR
        assert st.solve() == SOLVER_ERROR
    ref = oracle_mod.StaticNewton(oa.linear(), oa.force(), oa.jacobian, oa.residual, dict(tol=1e-8, maxIt=5))
    assert ref.solve() == SOLVER_ERROR
    _context_still_solves(G)


def test_nan_in_host_input_is_not_success(lib):
    """A NaN in a host vector copied in (the start displacement of gsStaticNewton, the state of
    an arc-length path) never yields Success: the convergence test of a NaN residual fails and
    a non-finite pivot sets the factorisation's status word."""
    import gsstructuralanalysis_gb300 as G
    prob = P.cylindrical_panel(m=6, p=2, load=500.0)
    gp = G.Problem(prob)
    U = np.zeros(gp.ndof)
    U[gp.ndof // 3] = np.nan
    st = G.StaticNewton(gp, {"Solver": "SimplicialLDLT", "tol": 1e-8, "maxIt": 5})
    st.setDisplacement(U)
    assert st.solve() != G.SUCCESS
    alm = G.ALMCrisfield(gp, dict(Length=0.004, TolF=1e-8, TolU=1e-6, Scaling=0.0, MaxIter=5,
                                  BifurcationMethod=-1))
    alm.initialize(stability=False)
    alm.setSolution(U, 0.5)
    assert alm.step() != G.SUCCESS
    R = gp.al_residual(U, 0.5)
    assert not np.isfinite(R).all()
    _context_still_solves(G)


def test_poisoned_learned_guess_falls_back_to_tangent_predictor(lib):
    """A learned predictor whose output statistics are deliberately wrong by orders of magnitude
    (a host-side perturbation of its de-standardisation) places starts the corrector cannot
    bring back within the guess budget.  The library then redoes the step from the last point
    with the plain tangent predictor, so the path is the plain path, point for point."""
    import gsstructuralanalysis_gb300 as G
    prob = P.cylindrical_panel(m=8, p=2, load=1.0)
    opts = dict(Length=0.004, TolF=1e-8, TolU=1e-6, Scaling=0.0, MaxIter=25, BifurcationMethod=-1)
    nm = 4
    rng = np.random.default_rng(11)
    gp_plain, gp_pois = G.Problem(prob), G.Problem(prob)
    Phi, _ = np.linalg.qr(rng.standard_normal((gp_pois.ndof, nm)))
    net = G.MLP(4 * (nm + 1), 16, 16, nm + 1, seed=5)
    in_mu, in_sd = np.zeros(4 * (nm + 1)), np.ones(4 * (nm + 1))
    out_mu = np.full(nm + 1, 1e3)             # the poison: a correction of ~1e3 in every coefficient
    out_sd = np.full(nm + 1, 1e3)
    pred = G.Predictor(gp_pois, net, Phi.T.copy(), in_mu, in_sd, out_mu, out_sd)
    plain = G.ALMCrisfield(gp_plain, opts)
    pois = G.ALMCrisfield(gp_pois, opts)
    plain.initialize(stability=False)
    pois.initialize(stability=False)
    used = 0
    for k in range(10):
        assert plain.step() == G.SUCCESS
        st, u = pred.step(pois, guess_max_iter=4)
        assert st == G.SUCCESS, k
        used += u
        U, L = pois.solutionU(), pois.solutionL()
        Up, Lp = plain.solutionU(), plain.solutionL()
        assert np.linalg.norm(U - Up) <= 1e-6 * np.linalg.norm(Up), k
        assert abs(L - Lp) <= 1e-6 * abs(Lp), k
    assert used == 0          # every placed start failed and the tangent predictor took over


def test_solve_wait_budget_gives_non_finite_solution(lib, monkeypatch):
    """Every wait of the dataflow triangular solve is bounded.  KLSA_SOLVE_STALL_NODE=k (read when
    a problem's factorisation is set up) makes the k-th leaf's completion count unreachable: the
    waits of its parent run out after about 0.1 s, the launch still ends, the solution comes
    back non-finite (the library's error signal for an expired wait), and the context then
    solves a good problem."""
    import gsstructuralanalysis_gb300 as G
    monkeypatch.setenv("KLSA_SOLVE_STALL_NODE", "0")
    prob = P.cylindrical_panel(m=16, p=2)
    gp = G.Problem(prob)
    s = G.SparseSolver(gp, "SimplicialLDLT")
    assert s.compute_jacobian(np.zeros(gp.ndof)) == 0
    t0 = time.perf_counter()
    y = s.solve(np.ones((2, gp.ndof)))
    assert time.perf_counter() - t0 < 10.0
    assert not np.isfinite(y).all()
    monkeypatch.delenv("KLSA_SOLVE_STALL_NODE")
    gp2 = G.Problem(prob)
    s2 = G.SparseSolver(gp2, "SimplicialLDLT", {"Refinement": 8, "RefineTol": 1e-12})
    assert s2.compute_jacobian(np.zeros(gp2.ndof)) == 0
    assert np.isfinite(s2.solve(np.ones((2, gp2.ndof)))).all()
    _context_still_solves(G)
