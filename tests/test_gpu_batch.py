"""Batched Newton solves of patches of uneven size, degree and thickness (one launch sequence and
one CUDA graph per Newton iteration for all instances) against the oracle's gsStaticNewton
restatement per instance and against the single-patch GPU Newton."""
import numpy as np
import pytest

from gsstructuralanalysis_gb300 import problems as P

pytestmark = pytest.mark.gpu

# (elements per direction, degree, thickness, point load): loads below each panel's limit load
SPECS = [(4, 2, 0.01, 1500.0), (5, 3, 0.02, 9000.0), (6, 2, 0.005, 90.0), (7, 3, 0.01, 1500.0),
         (8, 2, 0.05, 2e5), (9, 3, 0.005, 60.0)]
OPTS = {"tol": 1e-8, "maxIt": 30}


def _instances():
    return [P.cylindrical_panel(m=m, p=p, t=t, load=load) for m, p, t, load in SPECS]


def test_batched_newton_vs_oracle(lib, oracle_mod):
    import gsstructuralanalysis_gb300 as G
    probs = _instances()
    bp = G.BatchedProblem(probs)
    info = bp.info()
    assert info["instances"] == len(probs)
    bn = G.BatchedNewton(bp, OPTS)
    assert bn.solve() == 0
    st, its = bn.results()
    assert (st == 0).all()
    for i, prob in enumerate(probs):
        oa = oracle_mod.OracleAssembler(prob)
        ref = oracle_mod.StaticNewton(oa.linear(), oa.force(), oa.jacobian, oa.residual, dict(OPTS))
        assert ref.solve() == 0
        U = bn.solution(i)
        assert np.linalg.norm(U - ref.U) / np.linalg.norm(ref.U) < 1e-6, i
        # the converged point satisfies the reference's force criterion, residual by the oracle
        R = oa.residual(U)
        assert np.linalg.norm(R) <= 1e-8 * np.linalg.norm(oa.force()) * 10, i


def test_batched_newton_equals_single_patch_path(lib):
    """Per instance the batched kernels do the single-patch arithmetic (same element kernel body,
    same fronts, same extend-add order), so the result matches the single-patch Newton with the
    same FP32 LDL^T solver to rounding."""
    import gsstructuralanalysis_gb300 as G
    probs = _instances()
    bp = G.BatchedProblem(probs)
    bn = G.BatchedNewton(bp, dict(OPTS, Refinement=0))
    assert bn.solve() == 0
    _, its = bn.results()
    for i, prob in enumerate(probs):
        gp = G.Problem(prob)
        sn = G.StaticNewton(gp, dict(OPTS, Solver="SimplicialLDLT"))
        assert sn.solve() == 0
        U, Us = bn.solution(i), sn.solution()
        assert np.linalg.norm(U - Us) / np.linalg.norm(Us) < 1e-9, i
        assert its[i] == sn.iterations(), i
    # a second solve after reset repeats the first
    U0 = [bn.solution(i) for i in range(len(probs))]
    bn.reset()
    assert bn.solve() == 0
    for i in range(len(probs)):
        assert np.array_equal(bn.solution(i), U0[i])


def test_batched_autotune_log(lib):
    import gsstructuralanalysis_gb300 as G
    bp = G.BatchedProblem(_instances()[:3])
    log = bp.autotune()
    assert len(log) > 0
    assert set(np.unique(log[:, 0])) <= {0.0, 1.0}
    assert (log[:, 3] > 0).all()
