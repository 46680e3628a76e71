"""APALM on the device (klsa_apalm_*, the native gsAPALM over the device Crisfield solver) against
the FP64 restatement (oracle/apalm.py over the oracle's Crisfield): the same points, curve times
and levels for serialSolve + parallelSolve and for solve."""
import numpy as np
import pytest

from gsstructuralanalysis_gb300 import problems as P

pytestmark = pytest.mark.gpu

ALM_OPTS = dict(Length=0.02, TolF=1e-8, TolU=1e-6, Scaling=0.0, MaxIter=30, BifurcationMethod=-1)
AP_OPTS = dict(SubIntervals=2, MaxLevel=2, Tolerance=1e-3, MaxIt=40)


@pytest.mark.parametrize("mode", ["serial+parallel", "solve"])
def test_apalm_matches_oracle(lib, oracle_mod, mode):
    import gsstructuralanalysis_gb300 as G
    import apalm as AP
    prob = P.cylindrical_panel(m=6, p=2, load=1.0)
    gp, oa = G.Problem(prob), oracle_mod.OracleAssembler(prob)
    alm = G.ALMCrisfield(gp, ALM_OPTS)
    alm.initialize(stability=False)
    ap = G.APALM(alm, AP_OPTS)
    ap.initialize()
    ref = AP.APALM(oracle_mod.ALMCrisfield(oa.jacobian, oa.al_residual, oa.force(), ALM_OPTS), AP_OPTS)
    ref.initialize()
    if mode == "solve":
        ap.solve(5)
        ref.solve(5)
    else:
        ap.serialSolve(5)
        ref.serial_solve(5)
        ap.parallelSolve()
        ref.parallel_solve()
    assert ap.nBranches() == len(ref.times) == 1
    t, lv = ap.getFlatTimes(0), ap.getFlatLevels(0)
    sols = ap.getFlatSolutions(0)
    assert len(t) == len(ref.times[0]) >= 20
    assert list(lv) == list(ref.levels[0])
    np.testing.assert_allclose(t, ref.times[0], rtol=1e-6, atol=1e-9)
    for (U, L), (Ur, Lr) in zip(sols, ref.solutions[0]):
        assert abs(L - Lr) <= 1e-6 * max(abs(Lr), 1.0)
        assert np.linalg.norm(U - Ur) <= 1e-6 * max(np.linalg.norm(Ur), 1e-30)


def test_alm_distance_and_previous(lib, oracle_mod):
    """setPrevious and distance of the device Crisfield object agree with the restatement."""
    import gsstructuralanalysis_gb300 as G
    prob = P.cylindrical_panel(m=6, p=2, load=1.0)
    gp, oa = G.Problem(prob), oracle_mod.OracleAssembler(prob)
    alm = G.ALMCrisfield(gp, dict(ALM_OPTS, Scaling=0.5))
    alm.initialize(stability=False)
    ref = oracle_mod.ALMCrisfield(oa.jacobian, oa.al_residual, oa.force(), dict(ALM_OPTS, Scaling=0.5))
    rng = np.random.default_rng(4)
    DU = rng.normal(size=gp.ndof) * 1e-3
    assert abs(alm.distance(DU, 3.0) - ref.distance(DU, 3.0)) <= 1e-12 * ref.distance(DU, 3.0)
    assert alm.step() == 0 and ref.step() == 0
    U1, L1 = alm.solutionU(), alm.solutionL()
    alm.setPrevious(np.zeros(gp.ndof), 0.0)
    ref.set_previous(np.zeros(gp.ndof), 0.0)
    assert alm.step() == 0 and ref.step() == 0
    assert abs(alm.solutionL() - ref.L) <= 1e-6 * abs(ref.L)
    assert alm.solutionL() != L1


def test_apalm_workers_match_oracle(lib, oracle_mod):
    """parallelSolve with three solvers running concurrently on the GPU (each on its own problem
    and stream, driven by its own host thread) in the reference's MPI schedule
    (gsAPALM.hpp:276-378): the same points, curve times and levels as the restatement's schedule
    with three workers.  Two refinement levels, so jobs are handed out before earlier ones are
    submitted, as the MPI main process does."""
    import gsstructuralanalysis_gb300 as G
    import apalm as AP
    prob = P.cylindrical_panel(m=6, p=2, load=1.0)
    oa = oracle_mod.OracleAssembler(prob)
    gps = [G.Problem(prob) for _ in range(3)]
    alms = [G.ALMCrisfield(g, ALM_OPTS) for g in gps]
    for a in alms:
        a.initialize(stability=False)
    ap = G.APALM(alms[0], AP_OPTS)
    ap.addWorker(alms[1])
    ap.addWorker(alms[2])
    ap.initialize()
    mk = lambda: oracle_mod.ALMCrisfield(oa.jacobian, oa.al_residual, oa.force(), ALM_OPTS)
    ref = AP.APALM(mk(), AP_OPTS)
    ref.add_worker(mk())
    ref.add_worker(mk())
    ref.initialize()
    ap.serialSolve(5)
    ref.serial_solve(5)
    ap.parallelSolve()
    ref.parallel_solve()
    t, lv = ap.getFlatTimes(0), ap.getFlatLevels(0)
    sols = ap.getFlatSolutions(0)
    assert len(t) == len(ref.times[0]) >= 20
    assert list(lv) == list(ref.levels[0])
    assert max(lv) == 2
    np.testing.assert_allclose(t, ref.times[0], rtol=1e-6, atol=1e-9)
    for (U, L), (Ur, Lr) in zip(sols, ref.solutions[0]):
        assert abs(L - Lr) <= 1e-6 * max(abs(Lr), 1.0)
        assert np.linalg.norm(U - Ur) <= 1e-6 * max(np.linalg.norm(Ur), 1e-30)
