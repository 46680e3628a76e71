"""GPU solvers against the answers of the reference's own solver code.

tests/golden/ref_solvers.npz holds what the reference's gsALMCrisfield / gsALMRiks /
gsALMLoadControl / gsALMConsistentCrisfield / gsStaticNewton / gsModalSolver, compiled unchanged
from its source tree (oracle/_ref, written by tests/golden/make_ref_fixtures.py), computed on the
cases of tests/golden/ref_cases.py with FP64 operators.  The GPU runs the same cases through the
C-ABI with FP64 fronts (FrontPrecision 64: the exact Newton of the reference, so the iteration
counts must agree too) and must reproduce every converged point to 1e-8, every iteration count
and every stability flag.
"""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import ref_cases as C  # noqa: E402

from gsstructuralanalysis_gb300 import problems as P  # noqa: E402

pytestmark = pytest.mark.gpu
FIX = np.load(os.path.join(HERE, "golden", "ref_solvers.npz"))
EXACT = {"FrontPrecision": 64}


def _rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300)


ALM_CASES = [k for k, c in C.CASES.items() if c["kind"] in ("alm", "alm_guess")]


@pytest.mark.parametrize("name", ALM_CASES)
def test_arc_length_case_matches_reference(lib, name):
    import gsstructuralanalysis_gb300 as G
    case = C.CASES[name]
    gp = G.Problem(C.build(case))
    cls = {"Crisfield": G.ALMCrisfield, "Riks": G.ALMRiks, "LoadControl": G.ALMLoadControl,
           "ConsistentCrisfield": G.ALMConsistentCrisfield}[case["method"]]
    alm = cls(gp, dict(case["options"], **EXACT))
    stab = case["options"].get("BifurcationMethod", -1) >= 0
    alm.initialize(stability=stab)
    U_ref, L_ref = FIX[f"{name}/U"], FIX[f"{name}/L"]
    its_ref = FIX[f"{name}/iterations"]
    for k in range(case["steps"]):
        if case["kind"] == "alm_guess" and k >= 2:
            alm.setInitialGuess(FIX[f"{name}/guess_U"][k - 2], float(FIX[f"{name}/guess_L"][k - 2]))
        assert alm.step() == 0, k
        assert _rel(alm.solutionU(), U_ref[k]) < 1e-8, k
        assert abs(alm.solutionL() - L_ref[k]) <= 1e-8 * abs(L_ref[k]), k
        assert alm.info()["iterations"] == its_ref[k], k
        if stab:
            assert alm.stability() == int(FIX[f"{name}/stability"][k]), k
            assert alm.stabilityChange() == bool(FIX[f"{name}/stability_change"][k]), k
    if name == "crisfield_determinant":
        assert FIX[f"{name}/stability_change"].sum() >= 1


@pytest.mark.parametrize("name", [k for k, c in C.CASES.items() if c["kind"] == "newton"])
def test_static_newton_case_matches_reference(lib, name):
    import gsstructuralanalysis_gb300 as G
    case = C.CASES[name]
    gp = G.Problem(C.build(case))
    st = G.StaticNewton(gp, dict(case["options"], **EXACT))
    for k, L in enumerate(case["loads"]):
        st.setLoad(L)
        assert st.solve() == int(FIX[f"{name}/status"][k]) == 0, k
        assert _rel(st.solution(), FIX[f"{name}/U"][k]) < 1e-8, k
        assert st.iterations() == int(FIX[f"{name}/iterations"][k]), k


def test_dense_compute_matches_reference(lib, oracle_mod):
    """gsEigenProblemBase::compute of gsModalSolver: every eigenvalue as the reference's own
    compute() gives it (Eigen's GeneralizedSelfAdjointEigenSolver behind the test shim's dense
    solver), with and without the shift option; the vectors are B-normalised eigenvectors of
    the oracle's pencil (sign and the basis inside a repeated eigenvalue are free)."""
    import gsstructuralanalysis_gb300 as G
    case = C.CASES["modal_dense"]
    prob = C.build(case)
    gp, oa = G.Problem(prob), oracle_mod.OracleAssembler(prob)
    ref = FIX["modal_dense/values"]
    for shift in (0.0, 0.5 * ref[0]):
        st, vals, vecs = G.eigen_dense(gp, "modal", options=dict(case["options"], shift=shift))
        assert st == 0
        np.testing.assert_allclose(vals, ref, rtol=1e-10, atol=1e-12 * np.abs(ref).max())
    K, M = oa.linear(), oa.mass()
    for lam, v in zip(vals, vecs):
        assert np.linalg.norm(K @ v - lam * (M @ v)) <= 1e-8 * np.linalg.norm(K @ v)
        assert abs(v @ (M @ v) - 1.0) <= 1e-10


def test_power_method_matches_reference(lib):
    """gsEigenProblemBase::computePower: the same iterates as the reference's (all-ones start,
    Euclidean normalisation), so the same value and vector."""
    import gsstructuralanalysis_gb300 as G
    case = C.CASES["modal_dense"]
    gp = G.Problem(C.build(case))
    st, val, vec = G.eigen_power(gp, "modal", options=case["options"])
    assert st == int(FIX["modal_dense/power_status"][0])
    assert abs(val - float(FIX["modal_dense/power_value"][0])) <= 1e-10 * abs(val)
    assert np.linalg.norm(vec - FIX["modal_dense/power_vector"]) <= 1e-8


def test_power_method_buckling_pencil(lib):
    """computePower of gsBucklingSolver's pencil on the simply supported square plate: the
    critical load factor (the smallest |lambda|, well separated from the next one), which the
    shift-invert Lanczos (Buckling mode) finds too.  The reference load is a tension, so lambda
    (and the dominant eigenvalue of A^-1 B) is positive; under a compressive reference load it is
    negative, the power iterates flip sign every step and, as in the reference, the method stops
    NotConverged after 100 steps."""
    import gsstructuralanalysis_gb300 as G
    prob = P.flat_plate(m=8, p=3, E=1.0, nu=0.3, t=0.01, pressure=0.0, bc="simply")
    n, ncp = prob.n1, prob.ncp
    ii, jj = np.arange(ncp) % n, np.arange(ncp) // n
    bnd = (ii == 0) | (ii == n - 1) | (jj == 0) | (jj == n - 1)
    fixed = np.zeros((3, ncp), dtype=bool)
    fixed[2, bnd] = True
    fixed[0, ii == 0] = True
    fixed[1, 0] = True
    prob.fixed = fixed.ravel()
    prob.edge_loads = np.array([[1, 1.0, 0.0, 0.0]])
    gp = G.Problem(prob)
    s = 1e-8
    st, val, _ = G.eigen_power(gp, "buckling", scaling=s, options={"tolerance": 1e-12})
    assert st == 0
    st, vals, _ = G.buckling(gp, 3, shift=1.05 * val, scaling=s, vectors=False)
    assert st == 0
    lam = vals[np.argmin(np.abs(vals))]
    assert abs(val - lam) <= 1e-8 * abs(lam)
    D = 0.01 ** 3 / (12 * (1 - 0.3 ** 2))
    assert abs(val * s / (4 * np.pi ** 2 * D) - 1) < 1e-4         # q_cr = 4 pi^2 D / b^2
