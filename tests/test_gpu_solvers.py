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


@pytest.mark.parametrize("solver", ["SimplicialLDLT", "CGDiagonal", "GPUPCG"])
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


@pytest.mark.parametrize("method", ["Crisfield", "Riks", "LoadControl", "ConsistentCrisfield"])
def test_arc_length_path(lib, oracle_mod, method):
    import gsstructuralanalysis_gb300 as G
    # Riks (phi = 1/numDof) is nearly load control: scale the load so that its steps move the
    # load factor, and stop before the limit point it cannot pass
    prob = P.cylindrical_panel(m=8, p=2, load=1e5 if method == "Riks" else 1.0)
    gp, oa = G.Problem(prob), oracle_mod.OracleAssembler(prob)
    length = {"Crisfield": 0.004, "Riks": 0.003, "LoadControl": 100.0, "ConsistentCrisfield": 0.004}[method]
    nsteps = {"Crisfield": 12, "Riks": 5, "LoadControl": 8, "ConsistentCrisfield": 12}[method]
    opts = dict(Length=length, TolF=1e-8, TolU=1e-6, Scaling=0.0, MaxIter=30)
    cls = {"Crisfield": G.ALMCrisfield, "Riks": G.ALMRiks, "LoadControl": G.ALMLoadControl,
           "ConsistentCrisfield": G.ALMConsistentCrisfield}[method]
    rcls = {"Crisfield": oracle_mod.ALMCrisfield, "Riks": oracle_mod.ALMRiks,
            "LoadControl": oracle_mod.ALMLoadControl, "ConsistentCrisfield": oracle_mod.ALMConsistentCrisfield}[method]
    alm = cls(gp, opts)
    alm.initialize()
    ref = rcls(oa.jacobian, oa.al_residual, oa.force(), opts)
    for k in range(nsteps):
        assert alm.step() == 0
        assert ref.step() == 0
        U, L = alm.solutionU(), alm.solutionL()
        assert np.linalg.norm(U - ref.U) / np.linalg.norm(ref.U) < 1e-6, k
        assert abs(L - ref.L) / abs(ref.L) < 1e-6, k
        # the GPU point meets the reference's force criterion when its residual is evaluated by
        # the oracle: ||R|| <= TolF ||(L) F|| (gsALMBase.hpp:156-168, 392-407)
        R = oa.al_residual(U, L)
        assert np.linalg.norm(R) <= 1e-8 * abs(L) * np.linalg.norm(oa.force()) * (1 + 1e-6)


@pytest.mark.parametrize("method", [0, 1])
def test_alm_stability_indicator(lib, oracle_mod, method):
    """BifurcationMethod 0 (Determinant: sign pattern of the LDL^T D = inertia of the Jacobian) and
    1 (Eigenvalue: shift-invert Lanczos, shift -100, LargestAlge) along a Crisfield path through
    the limit point of the roof, step by step against the oracle (gsALMBase.hpp:381-390, 547-627).
    The Determinant run passes a stability change on entering and on leaving the unstable
    branch; the Eigenvalue selection (eigenvalues just above the shift) does not see the negative
    eigenvalue there, as in the reference."""
    import gsstructuralanalysis_gb300 as G
    prob = P.cylindrical_panel(m=8, p=2, load=1.0)
    gp, oa = G.Problem(prob), oracle_mod.OracleAssembler(prob)
    opts = dict(Length=0.004, TolF=1e-8, TolU=1e-6, Scaling=0.0, MaxIter=30, BifurcationMethod=method)
    alm = G.ALMCrisfield(gp, opts)
    assert alm.initialize() == 0
    ref = oracle_mod.ALMCrisfield(oa.jacobian, oa.al_residual, oa.force(), opts)
    ref.initialize()
    assert alm.stability() == ref.stability
    changes = 0
    for k in range(16):
        assert alm.step() == 0
        assert ref.step() == 0
        assert abs(alm.solutionL() - ref.L) / abs(ref.L) < 1e-6, k
        assert alm.stability() == ref.stability, k
        assert alm.stabilityChange() == ref.stability_change(), k
        assert alm.negatives() == ref.negatives, k
        if method == 1:
            assert abs(alm.indicator() - ref.indicator) <= 1e-6 * abs(ref.indicator), k
        changes += alm.stabilityChange()
    assert changes == (2 if method == 0 else 0)


def test_static_newton_load_ramp_through_snap(lib, oracle_mod):
    """Config-2 style load ramp (degree 3, central point load to ~5 thicknesses of deflection in 10
    load steps, the first step jumping past the limit point) at a size the oracle finishes in
    seconds: each converged step against the oracle's gsStaticNewton restatement, which starts
    every later step from the previous solution (no head start after the first call)."""
    import gsstructuralanalysis_gb300 as G
    Pmax = 30000.0
    prob = P.cylindrical_panel(m=12, p=3, load=Pmax)
    gp, oa = G.Problem(prob), oracle_mod.OracleAssembler(prob)
    F = oa.force()
    st = G.StaticNewton(gp, {"Solver": "SimplicialLDLT", "tol": 1e-8, "maxIt": 50})
    ref = None
    for k in range(1, 11):
        L = k / 10.0
        st.setLoad(L)
        assert st.solve() == 0, k
        if ref is None:
            ref = oracle_mod.StaticNewton(oa.linear(), L * F, oa.jacobian, lambda U, L=L: L * F - oa.fint(U),
                                          dict(tol=1e-8, maxIt=50))
        else:
            ref.F = L * F
            ref.res = (lambda U, L=L: L * F - oa.fint(U))
        assert ref.solve() == 0, k
        U = st.solution()
        assert np.linalg.norm(U - ref.U) / np.linalg.norm(ref.U) < 1e-6, k
        assert np.linalg.norm(L * F - oa.fint(U)) <= 1e-7 * np.linalg.norm(L * F), k


def test_fp64_fronts(lib, oracle_mod):
    """FrontPrecision 64: the multifrontal LDL^T in FP64 (no refinement) solves the linear plate to
    FP64 accuracy, and the Newton corrector with it is the exact Newton of the oracle (same
    iteration count, same converged point)."""
    import gsstructuralanalysis_gb300 as G
    prob = P.flat_plate(m=8, p=2)
    gp, oa = G.Problem(prob), oracle_mod.OracleAssembler(prob)
    st = G.StaticNewton(gp, {"Solver": "SimplicialLDLT", "FrontPrecision": 64})
    assert st.solveLinear() == 0
    ur = spla.spsolve(oa.linear().tocsc(), oa.force())
    assert np.linalg.norm(st.solution() - ur) / np.linalg.norm(ur) < 1e-12
    prob = P.cylindrical_panel(m=6, p=3, load=800.0)
    gp, oa = G.Problem(prob), oracle_mod.OracleAssembler(prob)
    st = G.StaticNewton(gp, {"Solver": "SimplicialLDLT", "FrontPrecision": 64, "tol": 1e-10, "maxIt": 30})
    assert st.solve() == 0
    ref = oracle_mod.StaticNewton(oa.linear(), oa.force(), oa.jacobian, oa.residual, dict(tol=1e-10, maxIt=30))
    assert ref.solve() == 0
    assert np.linalg.norm(st.solution() - ref.U) / np.linalg.norm(ref.U) < 1e-9
    assert st.iterations() == ref.num_iterations


@pytest.mark.parametrize("method", ["Crisfield", "Riks", "LoadControl", "ConsistentCrisfield"])
def test_quasi_newton_adaptive_length(lib, oracle_mod, method):
    """Quasi-Newton corrector (Jacobian refreshed every QuasiIterations) with adaptive arc length
    (gsALMBase.hpp:106-117, 376-387; the factor an integer quotient) against the oracle step by
    step; the oracle's lengths are the compiled reference's (tests/test_ref_oracle.py)."""
    import gsstructuralanalysis_gb300 as G
    prob = P.cylindrical_panel(m=8, p=2, load=1e5 if method == "Riks" else 1.0)
    gp, oa = G.Problem(prob), oracle_mod.OracleAssembler(prob)
    length = {"Crisfield": 0.004, "Riks": 0.003, "LoadControl": 100.0, "ConsistentCrisfield": 0.004}[method]
    opts = dict(Length=length, TolF=1e-8, TolU=1e-6, Scaling=0.0, MaxIter=60, Quasi=1, QuasiIterations=2,
                AdaptiveLength=1, AdaptiveIterations=4, BifurcationMethod=-1)
    cls = {"Crisfield": G.ALMCrisfield, "Riks": G.ALMRiks, "LoadControl": G.ALMLoadControl,
           "ConsistentCrisfield": G.ALMConsistentCrisfield}[method]
    rcls = {"Crisfield": oracle_mod.ALMCrisfield, "Riks": oracle_mod.ALMRiks,
            "LoadControl": oracle_mod.ALMLoadControl, "ConsistentCrisfield": oracle_mod.ALMConsistentCrisfield}[method]
    alm = cls(gp, opts)
    alm.initialize()
    ref = rcls(oa.jacobian, oa.al_residual, oa.force(), opts)
    for k in range(5):
        assert alm.step() == 0
        assert ref.step() == 0
        assert abs(alm.getLength() - ref.arcLength) <= 1e-12 * ref.arcLength, k
        U, L = alm.solutionU(), alm.solutionL()
        assert np.linalg.norm(U - ref.U) / np.linalg.norm(ref.U) < 1e-6, k
        assert abs(L - ref.L) / abs(ref.L) < 1e-6, k


@pytest.mark.parametrize("tolB", [0.0, 0.1])
def test_singular_point_and_branch_switch(lib, oracle_mod, tolB):
    """At the limit point of the roof (stability change of the Determinant indicator): the
    singular-point test (a limit point, not a bifurcation), the extended-system Newton for the
    critical point (with and without the bisection stage) and switchBranch, against the oracle
    (gsALMBase.hpp:421-512, 628-852).  The critical load factor is converged to FP64 accuracy."""
    import gsstructuralanalysis_gb300 as G
    prob = P.cylindrical_panel(m=8, p=2, load=1.0)
    gp, oa = G.Problem(prob), oracle_mod.OracleAssembler(prob)
    opts = dict(Length=0.004, TolF=1e-8, TolU=1e-6, Scaling=0.0, MaxIter=8, BifurcationMethod=0,
                SingularPointComputeTolB=tolB)
    alm = G.ALMCrisfield(gp, opts)
    alm.initialize()
    ref = oracle_mod.ALMCrisfield(oa.jacobian, oa.al_residual, oa.force(), opts)
    ref.initialize()
    found = False
    for k in range(12):
        Uold, Lold = alm.solutionU(), alm.solutionL()
        Uref, Lref = ref.U.copy(), ref.L
        assert alm.step() == 0 and ref.step() == 0
        assert alm.stabilityChange() == ref.stability_change(), k
        if ref.stability_change():
            found = True
            assert alm.isBifurcation(False) == ref.is_bifurcation(False)
            assert alm.computeSingularPoint(Uold, Lold, False, False, False) == 0
            assert ref.compute_singular_point(Uref, Lref, False, False, False) == 0
            U, L = alm.solutionU(), alm.solutionL()
            assert abs(L - ref.L) <= 1e-8 * abs(ref.L)
            assert np.linalg.norm(U - ref.U) <= 1e-6 * np.linalg.norm(ref.U)
            if tolB == 0.0:
                # without the bisection stage both use the null vector of the same Jacobian (with it,
                # the number of bisection steps depends on min D, which differs with the ordering)
                alm.switchBranch()
                ref.switch_branch()
                assert np.linalg.norm(alm.solutionU() - ref.U) <= 1e-6 * np.linalg.norm(ref.U)
            break
    assert found


def test_bifurcation_and_branch_switch(lib, oracle_mod):
    """A genuine bifurcation (the flat plate under in-plane compression, no imperfection): the
    singular-point test finds the null vector orthogonal to the load, the extended system
    converges to the critical point, switchBranch steps onto the buckled branch and two steps
    follow it, against the oracle (gsALMBase.hpp:421-512, 628-852); the oracle's points are the
    compiled reference's (tests/test_ref_oracle.py)."""
    import gsstructuralanalysis_gb300 as G
    prob = P.flat_plate(m=6, p=2, E=1.0, nu=0.3, t=0.01, pressure=0.0, bc="simply")
    n, ncp = prob.n1, prob.ncp
    ii, jj = np.arange(ncp) % n, np.arange(ncp) // n
    bnd = (ii == 0) | (ii == n - 1) | (jj == 0) | (jj == n - 1)
    fixed = np.zeros((3, ncp), dtype=bool)
    fixed[2, bnd] = True
    fixed[0, ii == 0] = True
    fixed[1, 0] = True
    prob.fixed = fixed.ravel()
    prob.edge_loads = np.array([[1, -1e-6, 0.0, 0.0]])
    gp, oa = G.Problem(prob), oracle_mod.OracleAssembler(prob)
    opts = dict(Length=2e-4, TolF=1e-9, TolU=1e-9, Scaling=0.0, MaxIter=20, BifurcationMethod=0,
                SingularPointComputeTolB=0.0)
    alm = G.ALMCrisfield(gp, dict(opts, FrontPrecision=64))
    alm.initialize()
    ref = oracle_mod.ALMCrisfield(oa.jacobian, oa.al_residual, oa.force(), opts)
    ref.initialize()
    for k in range(15):
        Uold, Lold = alm.solutionU(), alm.solutionL()
        Uref, Lref = ref.U.copy(), ref.L
        assert alm.step() == 0 and ref.step() == 0, k
        assert alm.stabilityChange() == ref.stability_change(), k
        if ref.stability_change():
            break
    else:
        pytest.fail("no stability change")
    assert alm.isBifurcation(False) and ref.is_bifurcation(False)
    assert alm.computeSingularPoint(Uold, Lold, False, False, False) == 0
    assert ref.compute_singular_point(Uref, Lref, False, False, False) == 0
    assert abs(alm.solutionL() - ref.L) <= 1e-8 * abs(ref.L)
    assert np.linalg.norm(alm.solutionU() - ref.U) <= 1e-6 * np.linalg.norm(ref.U)
    alm.switchBranch()
    ref.switch_branch()
    for k in range(2):
        assert alm.step() == 0 and ref.step() == 0, k
        assert abs(alm.solutionL() - ref.L) <= 1e-6 * abs(ref.L), k
        assert np.linalg.norm(alm.solutionU() - ref.U) <= 1e-5 * np.linalg.norm(ref.U), k


def test_crisfield_complex_roots(lib, oracle_mod):
    """Quasi-Newton Crisfield with a long step on the coarse roof, where the constraint
    quadratic has no real root inside step 2: the corrector takes Lam's modified quadratic and
    the complex-root fallback (gsALMCrisfield.hpp:236-330) and still converges.  FP64 fronts;
    every step's status, iteration count and point (up to the panel's mirror symmetry) against
    the oracle, whose points are the compiled reference's (tests/test_ref_oracle.py).  Before
    the fix the complex-root branch multiplied by the FP32 CSR values, which FP64 fronts never
    assemble, and the step ended in OtherError."""
    import gsstructuralanalysis_gb300 as G
    prob = P.cylindrical_panel(m=4, p=2, load=1.0)
    gp, oa = G.Problem(prob), oracle_mod.OracleAssembler(prob)
    opts = dict(Length=0.01, TolF=1e-8, TolU=1e-6, Scaling=0.0, MaxIter=40, BifurcationMethod=-1, Quasi=True,
                QuasiIterations=8)
    alm = G.ALMCrisfield(gp, dict(opts, FrontPrecision=64))
    alm.initialize(stability=False)
    ref = oracle_mod.ALMCrisfield(oa.jacobian, oa.al_residual, oa.force(), opts)
    ref.initialize()
    # From step 2 on the path leaves the panel's symmetry about x = L / 2 (xi1 -> 1 - xi1,
    # u_x -> -u_x; a mirrored equilibrium point stays one), and rounding picks the side: the
    # device may follow the mirror image of the oracle's branch, with the same load factor.
    free = prob.free_index()
    pos = np.full(3 * prob.ncp, -1)
    pos[free] = np.arange(len(free))
    comp, cp = free // prob.ncp, free % prob.ncp
    mirror = pos[comp * prob.ncp + (cp // prob.n1) * prob.n1 + (prob.n1 - 1 - cp % prob.n1)]
    sign = np.where(comp == 0, -1.0, 1.0)
    for k in range(5):
        assert alm.step() == 0 and ref.step() == 0, k
        assert int(alm.info()["iterations"]) == ref.num_iterations, k
        assert abs(alm.solutionL() - ref.L) <= 1e-8 * abs(ref.L), k
        U = alm.solutionU()
        err = min(np.linalg.norm(U - ref.U), np.linalg.norm(U - sign * ref.U[mirror]))
        assert err <= 1e-7 * np.linalg.norm(ref.U), k


@pytest.mark.parametrize("variant", ["Relaxation", "AutoScaling"])
def test_crisfield_relaxation_and_scaling(lib, oracle_mod, variant):
    """Relaxation 0.7 (gsALMCrisfield.hpp:84-90) on ten converging steps, and the default Scaling
    -1 (phi from the first predictor) up to the step that ends NotConverged: FP64 fronts, every
    status, iteration count and point against the oracle (which matches the compiled
    reference, tests/test_ref_oracle.py)."""
    import gsstructuralanalysis_gb300 as G
    prob = P.cylindrical_panel(m=6, p=2, load=1.0)
    gp, oa = G.Problem(prob), oracle_mod.OracleAssembler(prob)
    extra = {"Relaxation": dict(Relaxation=0.7, Scaling=0.0), "AutoScaling": dict(Scaling=-1.0)}[variant]
    opts = dict(Length=0.01, TolF=1e-8, TolU=1e-6, MaxIter=40, BifurcationMethod=-1, **extra)
    alm = G.ALMCrisfield(gp, dict(opts, FrontPrecision=64))
    alm.initialize(stability=False)
    ref = oracle_mod.ALMCrisfield(oa.jacobian, oa.al_residual, oa.force(), opts)
    ref.initialize()
    statuses = []
    for k in range(10):
        st = ref.step()
        assert alm.step() == st, k
        assert int(alm.info()["iterations"]) == ref.num_iterations, k
        assert abs(alm.solutionL() - ref.L) <= 1e-8 * abs(ref.L), k
        assert np.linalg.norm(alm.solutionU() - ref.U) <= 1e-7 * np.linalg.norm(ref.U), k
        statuses.append(st)
        if st != 0:
            break
    assert statuses == ([0] * 10 if variant == "Relaxation" else [0] * 6 + [1])


@pytest.mark.parametrize("method", ["Crisfield", "Riks"])
def test_reference_predictor_guess(lib, oracle_mod, method):
    """setInitialGuess in the reference's own mode, step by step against the oracle.  Crisfield
    uses the guess only as the old increment that orients the tangent predictor
    (gsALMCrisfield.hpp:167-191); Riks rescales the guessed chord by Length / previous Length
    (gsALMRiks.hpp:137-170).  The guess is selected only when it differs from the current point
    in U and in lambda (gsALMBase.hpp:365-368).  Both sides get the identical host guess: the
    linear extrapolation of the oracle's last two points, perturbed."""
    import gsstructuralanalysis_gb300 as G
    prob = P.cylindrical_panel(m=8, p=2, load=1e5 if method == "Riks" else 1.0)
    gp, oa = G.Problem(prob), oracle_mod.OracleAssembler(prob)
    length = {"Crisfield": 0.004, "Riks": 0.003}[method]
    opts = dict(Length=length, TolF=1e-8, TolU=1e-6, Scaling=0.0, MaxIter=30)
    cls = {"Crisfield": G.ALMCrisfield, "Riks": G.ALMRiks}[method]
    rcls = {"Crisfield": oracle_mod.ALMCrisfield, "Riks": oracle_mod.ALMRiks}[method]
    alm = cls(gp, opts)
    alm.initialize()
    ref = rcls(oa.jacobian, oa.al_residual, oa.force(), opts)
    rng = np.random.default_rng(3)
    prev = (np.zeros(gp.ndof), 0.0)
    guessed = 0
    for k in range(5):
        if k >= 2:
            Ug = 2 * ref.U - prev[0] + 1e-3 * np.linalg.norm(ref.U - prev[0]) * rng.standard_normal(gp.ndof) / np.sqrt(gp.ndof)
            Lg = 2 * ref.L - prev[1]
            alm.setInitialGuess(Ug, Lg)
            ref.set_initial_guess(Ug, Lg)
            guessed += 1
        prev = (ref.U.copy(), ref.L)
        assert alm.step() == 0, k
        assert ref.step() == 0, k
        U, L = alm.solutionU(), alm.solutionL()
        assert np.linalg.norm(U - ref.U) / np.linalg.norm(ref.U) < 1e-6, k
        assert abs(L - ref.L) / abs(ref.L) < 1e-6, k
    assert guessed == 3
