"""The APALM restatement (oracle/apalm.py) on CPU: the coarse serial path is the plain
arc-length path, every correction lands between the coarse points it refines, the curve times
grow along the path, and with one branch the interleaved solve() schedule gives the same points
as serialSolve() followed by parallelSolve() (initiation jobs are queued at the front)."""
import numpy as np

import apalm as AP
from gsstructuralanalysis_gb300 import problems as P


def _alm(oracle_mod, oa):
    return oracle_mod.ALMCrisfield(oa.jacobian, oa.al_residual, oa.force(),
                                   dict(Length=0.02, TolF=1e-8, TolU=1e-6, Scaling=0.0, MaxIter=30, BifurcationMethod=-1))


def test_apalm_restatement(oracle_mod):
    from gsstructuralanalysis_gb300 import problems as P
    prob = P.cylindrical_panel(m=6, p=2, load=1.0)
    oa = oracle_mod.OracleAssembler(prob)
    opts = dict(SubIntervals=2, MaxLevel=2, Tolerance=1e-3, MaxIt=40)

    # plain arc-length path with the same length
    plain = _alm(oracle_mod, oa)
    Ls = [0.0]
    for _ in range(4):
        assert plain.step() == 0
        Ls.append(plain.L)

    a = AP.APALM(_alm(oracle_mod, oa), opts)
    a.initialize()
    a.serial_solve(5)
    np.testing.assert_allclose([s[1] for s in a.solutions[0]], Ls, rtol=1e-12)
    np.testing.assert_allclose(a.times[0], [0.0, 0.02, 0.04, 0.06, 0.08], rtol=1e-9)
    coarse = list(a.solutions[0])
    a.parallel_solve()
    t, lv = np.array(a.times[0]), np.array(a.levels[0])
    assert np.all(np.diff(t) >= 0) and t[-1] >= 0.08
    assert lv.max() == 2 and lv.min() == 0
    # the level-0 points are the coarse path, in order
    L0 = [s[1] for s, l in zip(a.solutions[0], lv) if l == 0]
    np.testing.assert_allclose(L0, [s[1] for s in coarse], rtol=1e-12)

    b = AP.APALM(_alm(oracle_mod, oa), opts)
    b.initialize()
    b.solve(5)
    np.testing.assert_allclose(b.times[0], a.times[0], rtol=1e-10, atol=1e-14)
    np.testing.assert_allclose([s[1] for s in b.solutions[0]], [s[1] for s in a.solutions[0]], rtol=1e-9)
    assert list(b.levels[0]) == list(a.levels[0])


def test_apalm_over_riks(oracle_mod):
    """APALM over Riks measures its intervals in Riks's norm (gsALMRiks.h:81-84): the corrected
    sub-steps cover every interval (the check in gsAPALMData::submit) and the times grow."""
    from gsstructuralanalysis_gb300 import problems as P
    prob = P.cylindrical_panel(m=5, p=2, load=1e5)
    oa = oracle_mod.OracleAssembler(prob)
    alm = oracle_mod.ALMRiks(oa.jacobian, oa.al_residual, oa.force(),
                             dict(Length=0.003, TolF=1e-8, TolU=1e-6, MaxIter=30, BifurcationMethod=-1))
    a = AP.APALM(alm, dict(SubIntervals=2, MaxLevel=1, Tolerance=1e-4, MaxIt=20))
    a.initialize()
    a.solve(4)
    t, lv = np.array(a.times[0]), np.array(a.levels[0])
    assert len(t) >= 7 and np.all(np.diff(t) > 0) and lv.max() == 1


def test_worker_schedule_one_level_equals_serial(oracle_mod):
    """The MPI schedule of parallelSolve (gsAPALM.hpp:276-378) in the restatement, with three
    workers: with one refinement level every job corrects a coarse interval that no other job's
    submission changes, and the workers' corrections are identical (Scaling fixed), so the flat
    path is the one-process schedule's point for point."""
    import apalm as AP
    prob = P.cylindrical_panel(m=4, p=2, load=1.0)
    oa = oracle_mod.OracleAssembler(prob)
    opts = dict(Length=0.02, TolF=1e-8, TolU=1e-6, Scaling=0.0, MaxIter=30, BifurcationMethod=-1)
    ap_opts = dict(SubIntervals=2, MaxLevel=1, Tolerance=1e-3, MaxIt=40)
    mk = lambda: oracle_mod.ALMCrisfield(oa.jacobian, oa.al_residual, oa.force(), opts)
    serial = AP.APALM(mk(), ap_opts)
    serial.initialize()
    serial.serial_solve(4)
    serial.parallel_solve()
    par = AP.APALM(mk(), ap_opts)
    par.add_worker(mk())
    par.add_worker(mk())
    par.initialize()
    par.serial_solve(4)
    par.parallel_solve()
    # with one refinement level the corrections of the coarse intervals are independent jobs
    assert list(par.levels[0]) == list(serial.levels[0])
    np.testing.assert_allclose(par.times[0], serial.times[0], rtol=1e-12, atol=1e-14)
    for (U, L), (Us, Ls) in zip(par.solutions[0], serial.solutions[0]):
        assert abs(L - Ls) <= 1e-12 * max(abs(Ls), 1.0)
