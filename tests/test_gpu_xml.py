"""A problem file in the reference's XML layout through the GPU path: the roof of
tests/golden/xml/roof_point_load.xml, refined as the reference's XML solvers refine it, solved
with its own option lists (id 91 for gsStaticNewton, id 93 for the arc-length method) and
compared with the oracle's restatement on the same problem."""
import os

import numpy as np
import pytest

from gsstructuralanalysis_gb300 import xmlio as X

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "xml")


def test_xml_roof_static_newton_and_arc_length(lib, oracle_mod):
    import gsstructuralanalysis_gb300 as G
    r = X.read(os.path.join(GOLD, "roof_point_load.xml"), elevate=1, refine=3)
    prob = r.problem
    prob.point_loads[:, 2:] *= 800.0            # a load with a visibly nonlinear response
    gp, oa = G.Problem(prob), oracle_mod.OracleAssembler(prob)
    nr = r.options[91]
    st = G.StaticNewton(gp, nr)
    assert st.solve() == 0
    ref = oracle_mod.StaticNewton(oa.linear(), oa.force(), oa.jacobian, oa.residual,
                                  {k: v for k, v in nr.items() if k != "Solver"})
    assert ref.solve() == 0
    u, ur = st.solution(), ref.U
    assert np.linalg.norm(u - ur) <= 1e-6 * np.linalg.norm(ur)

    alm_opts = dict(r.options[93])
    alm = G.ALMCrisfield(gp, alm_opts)
    alm.initialize(stability=False)
    ref_alm = oracle_mod.ALMCrisfield(oa.jacobian, oa.al_residual, oa.force(),
                                      {k: v for k, v in alm_opts.items() if k != "Solver"})
    ref_alm.initialize(stability=False)
    for k in range(4):
        assert alm.step() == 0, k
        assert ref_alm.step() == 0, k
    U, L = alm.solutionU(), alm.solutionL()
    assert abs(L - ref_alm.L) <= 1e-6 * abs(ref_alm.L)
    assert np.linalg.norm(U - ref_alm.U) <= 1e-6 * np.linalg.norm(ref_alm.U)


@pytest.mark.parametrize("fronts", [64, 32])
def test_benchmark_roof_from_reference_geometry(lib, fronts):
    """benchmark_Roof's problem built from the reference's own geometry file (the golden fixture
    holds the geometry as this repository's reader returns it, and the answers of the
    reference's compiled gsALMCrisfield): the GPU Crisfield path with Determinant stability.
    FP64 fronts reproduce the reference's iterations; FP32 fronts the same points."""
    import os
    import sys
    import gsstructuralanalysis_gb300 as G
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, os.path.join(here, "golden"))
    import ref_roof_xml as R
    fix = np.load(os.path.join(here, "golden", "roof_xml.npz"))
    prob = R.problem(int(fix["p"]), fix["knots1"], fix["knots2"], fix["ctrl"])
    gp = G.Problem(prob)
    opts = dict(R.ALM, FrontPrecision=fronts)
    alm = G.ALMCrisfield(gp, opts)
    alm.initialize()
    tol = 1e-8 if fronts == 64 else 1e-6
    for k in range(R.STEPS):
        assert alm.step() == 0, k
        U, L = alm.solutionU(), alm.solutionL()
        assert np.linalg.norm(U - fix["U"][k]) <= tol * np.linalg.norm(fix["U"][k]), k
        assert abs(L - fix["L"][k]) <= tol * abs(fix["L"][k]), k
        assert alm.stability() == int(fix["stability"][k]), k
        if fronts == 64:
            assert alm.info()["iterations"] == int(fix["iterations"][k]), k
