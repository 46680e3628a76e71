"""GPU mirrors of gsStaticNewton and the arc-length family vs the FP64 oracle restatement."""
import numpy as np
import pytest
import scipy.sparse.linalg as spla

from gsstructuralanalysis_gb300 import problems as P

pytestmark = pytest.mark.gpu


def test_linear_plate_config1(lib, oracle_mod):
    """Config 1: clamped plate, one K u = F solve, FP64-refined LDL^T vs the oracle's FP64 solve."""
    import gsstructuralanalysis_gb300 as G
    prob = P.flat_plate(m=8, p=2)
    gp, oa = G.Problem(prob), oracle_mod.OracleAssembler(prob)
    st = G.StaticNewton(gp, {"Solver": "SimplicialLDLT", "Refinement": 10, "RefineTol": 1e-14})
    assert st.solveLinear() == 0
    u = st.solution()
    ur = spla.spsolve(oa.linear().tocsc(), oa.force())
    assert np.linalg.norm(u - ur) / np.linalg.norm(ur) < 1e-10
    assert gp.ndof == 164


@pytest.mark.parametrize("solver", ["SimplicialLDLT", "CGDiagonal"])
def test_static_newton_panel(lib, oracle_mod, solver):
    import gsstructuralanalysis_gb300 as G
    prob = P.cylindrical_panel(m=6, p=3, load=800.0)
    gp, oa = G.Problem(prob), oracle_mod.OracleAssembler(prob)
    opts = {"Solver": solver, "tol": 1e-8, "maxIt": 30}
    st = G.StaticNewton(gp, opts)
    assert st.solve() == 0
    ref = oracle_mod.StaticNewton(oa.linear(), oa.force(), oa.jacobian, oa.residual, dict(tol=1e-8, maxIt=30))
    assert ref.solve() == 0
    u, ur = st.solution(), ref.U
    assert np.linalg.norm(u - ur) / np.linalg.norm(ur) < 1e-6


@pytest.mark.parametrize("method", ["Crisfield", "Riks", "LoadControl"])
def test_arc_length_path(lib, oracle_mod, method):
    import gsstructuralanalysis_gb300 as G
    # Riks (phi = 1/numDof) is nearly load control: scale the load so that its steps move the
    # load factor, and stop before the limit point it cannot pass
    prob = P.cylindrical_panel(m=8, p=2, load=1e5 if method == "Riks" else 1.0)
    gp, oa = G.Problem(prob), oracle_mod.OracleAssembler(prob)
    length = {"Crisfield": 0.004, "Riks": 0.003, "LoadControl": 100.0}[method]
    nsteps = {"Crisfield": 12, "Riks": 5, "LoadControl": 8}[method]
    opts = dict(Length=length, TolF=1e-8, TolU=1e-6, Scaling=0.0, MaxIter=30)
    cls = {"Crisfield": G.ALMCrisfield, "Riks": G.ALMRiks, "LoadControl": G.ALMLoadControl}[method]
    rcls = {"Crisfield": oracle_mod.ALMCrisfield, "Riks": oracle_mod.ALMRiks,
            "LoadControl": oracle_mod.ALMLoadControl}[method]
    alm = cls(gp, opts)
    alm.initialize()
    ref = rcls(oa.jacobian, oa.al_residual, oa.force(), opts)
    for k in range(nsteps):
        assert alm.step() == 0
        assert ref.step() == 0
        U, L = alm.solutionU(), alm.solutionL()
        assert np.linalg.norm(U - ref.U) / np.linalg.norm(ref.U) < 1e-6, k
        assert abs(L - ref.L) / abs(ref.L) < 1e-6, k
        # the GPU point is as much in equilibrium as the oracle's own point
        R, Rr = oa.al_residual(U, L), oa.al_residual(ref.U, ref.L)
        assert np.linalg.norm(R) <= 10 * np.linalg.norm(Rr) + 1e-12 * np.linalg.norm(oa.force())
