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
