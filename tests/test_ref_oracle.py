"""The restatements (oracle/oracle.py, oracle/apalm.py, oracle/dynamics.py) pinned against the
reference's OWN solver code.

oracle/_ref/libref_solvers.so is gsStaticNewton, gsALMCrisfield, gsALMRiks, gsALMLoadControl,
gsALMConsistentCrisfield, gsAPALM (without MPI), gsModalSolver, gsBucklingSolver and the six
time integrators of gsDynamicSolvers, compiled unchanged from the reference tree against the
test-only linear-algebra stand-in (oracle/refshim/; its GMRES, used by gsDynamicImplicitEuler,
solves the block operator exactly).  Both sides get the same FP64 KL-shell operators
(oracle.OracleAssembler), so every difference would be a difference of solver logic.  The
reference tree exists only where the library can be built; elsewhere these tests skip (the
golden fixtures written from it, tests/golden/ref_solvers.npz, carry the pin to the GPU tests).
"""
import numpy as np
import pytest

from gsstructuralanalysis_gb300 import problems as P

RS = pytest.importorskip("refsolvers")
pytestmark = pytest.mark.skipif(not RS.available(), reason="reference tree not present: reference solvers not built")

ALM_BASE = dict(TolF=1e-8, TolU=1e-6, Scaling=0.0, MaxIter=30, BifurcationMethod=-1)


def _rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("solver", ["SimplicialLDLT", "CGDiagonal"])
def test_static_newton_matches_reference(oracle_mod, solver):
    """gsStaticNewton::solve from zero (after initialize(), as the reference's drivers call it):
    same iterations, same point."""
    prob = P.cylindrical_panel(m=6, p=3, load=800.0)
    A = oracle_mod.OracleAssembler(prob)
    ops = RS.Operators.from_assembler(A)
    ref = RS.StaticNewton(ops, dict(tol=1e-8, maxIt=30, Solver=solver))
    assert ref.solve() == 0
    ora = oracle_mod.StaticNewton(A.linear(), A.force(), A.jacobian, A.residual, dict(tol=1e-8, maxIt=30))
    assert ora.solve() == 0
    assert _rel(ora.U, ref.solution()) < 1e-12
    assert ora.num_iterations == ref.iterations()


def test_static_newton_statuses_match_reference(oracle_mod):
    """throw 1 (maxIt) -> NotConverged; a zero pivot (E = 0) -> SolverError (gsStaticNewton.hpp:75-98)."""
    prob = P.cylindrical_panel(m=6, p=3, load=800.0)
    A = oracle_mod.OracleAssembler(prob)
    ref = RS.StaticNewton(RS.Operators.from_assembler(A), dict(tol=1e-8, maxIt=1))
    ora = oracle_mod.StaticNewton(A.linear(), A.force(), A.jacobian, A.residual, dict(tol=1e-8, maxIt=1))
    assert ref.solve() == ora.solve() == 1
    # the factorising solver (gsStaticNewton's default, CGDiagonal, has no pivot to fail)
    prob = P.flat_plate(m=4, p=2, E=0.0)
    A = oracle_mod.OracleAssembler(prob)
    ref = RS.StaticNewton(RS.Operators.from_assembler(A), dict(tol=1e-8, maxIt=5, Solver="SimplicialLDLT"))
    ora = oracle_mod.StaticNewton(A.linear(), A.force(), A.jacobian, A.residual, dict(tol=1e-8, maxIt=5))
    assert ref.solve() == ora.solve() == 3


def test_static_newton_nan_start_is_not_converged(oracle_mod):
    """A NaN in the start displacement stays in the iteration (no head start replaces it) and the
    reference's convergence test never passes: NotConverged, with either solver (Eigen's LDL^T
    flags only an exact zero pivot).  The oracle's SuperLU and the GPU's pivot check reject the
    non-finite matrix instead (SolverError): a different failure status, never Success."""
    prob = P.cylindrical_panel(m=6, p=2, load=500.0)
    A = oracle_mod.OracleAssembler(prob)
    U = np.zeros(len(A.force()))
    U[len(U) // 3] = np.nan
    for solver in ("CGDiagonal", "SimplicialLDLT"):
        ref = RS.StaticNewton(RS.Operators.from_assembler(A), dict(tol=1e-8, maxIt=5, Solver=solver))
        ref.set_displacement(U)
        assert ref.solve() == 1
    ora = oracle_mod.StaticNewton(A.linear(), A.force(), A.jacobian, A.residual, dict(tol=1e-8, maxIt=5))
    ora.set_displacement(U)
    assert ora.solve() in (1, 3)


def test_static_newton_load_ramp_matches_reference(oracle_mod):
    """Load steps continued from the previous solution (setLoad through the Residual_t closure,
    as the reference's ramp drivers rebuild it), through the limit point of the roof."""
    Pmax = 30000.0
    prob = P.cylindrical_panel(m=8, p=3, load=Pmax)
    A = oracle_mod.OracleAssembler(prob)
    F = A.force()
    load = {"L": 0.0}
    ops = RS.Operators(len(F), F, A.jacobian, lambda x, lam: A.fint(x) - lam * F,
                       lambda x: load["L"] * F - A.fint(x))
    ref = RS.StaticNewton(ops, dict(tol=1e-8, maxIt=50))
    ora = None
    for k in range(1, 6):
        L = k / 5.0
        load["L"] = L
        if ora is None:
            ora = oracle_mod.StaticNewton(A.linear(), L * F, A.jacobian, lambda U, L=L: L * F - A.fint(U),
                                          dict(tol=1e-8, maxIt=50))
        else:
            ora.F = L * F
            ora.res = (lambda U, L=L: L * F - A.fint(U))
        assert ref.solve() == 0, k
        assert ora.solve() == 0, k
        assert _rel(ora.U, ref.solution()) < 1e-10, k
        assert ora.num_iterations == ref.iterations(), k


@pytest.mark.parametrize("method", ["Crisfield", "Riks", "LoadControl", "ConsistentCrisfield"])
def test_arc_length_path_matches_reference(oracle_mod, method):
    """Five steps of each arc-length method: same points, same iteration counts."""
    prob = P.cylindrical_panel(m=6, p=2, load=1e5 if method == "Riks" else 1.0)
    A = oracle_mod.OracleAssembler(prob)
    length = {"Crisfield": 0.004, "Riks": 0.003, "LoadControl": 100.0, "ConsistentCrisfield": 0.004}[method]
    opts = dict(ALM_BASE, Length=length)
    cls = {"Crisfield": oracle_mod.ALMCrisfield, "Riks": oracle_mod.ALMRiks,
           "LoadControl": oracle_mod.ALMLoadControl, "ConsistentCrisfield": oracle_mod.ALMConsistentCrisfield}[method]
    ref = RS.ALM(RS.Operators.from_assembler(A), method, opts)
    ref.initialize()
    ora = cls(A.jacobian, A.al_residual, A.force(), opts)
    ora.initialize()
    for k in range(5):
        assert ref.step() == 0, k
        assert ora.step() == 0, k
        U, L = ref.solution()
        assert _rel(ora.U, U) < 1e-10, k
        assert abs(ora.L - L) <= 1e-10 * abs(L), k
        assert ora.num_iterations == ref.info()["iterations"], k


@pytest.mark.parametrize("variant", ["Quasi", "AdaptiveLength", "AngleMethod"])
def test_crisfield_variants_match_reference(oracle_mod, variant):
    """Quasi-Newton (QuasiIterations), AdaptiveLength and the angle-method root choice."""
    prob = P.cylindrical_panel(m=6, p=2, load=1.0)
    A = oracle_mod.OracleAssembler(prob)
    extra = {"Quasi": dict(Quasi=True, QuasiIterations=2), "AdaptiveLength": dict(AdaptiveLength=True,
             AdaptiveIterations=3), "AngleMethod": dict(AngleMethod=1)}[variant]
    opts = dict(ALM_BASE, Length=0.004, **extra)
    ref = RS.ALM(RS.Operators.from_assembler(A), "Crisfield", opts)
    ref.initialize()
    ora = oracle_mod.ALMCrisfield(A.jacobian, A.al_residual, A.force(), opts)
    ora.initialize()
    for k in range(5):
        assert ref.step() == ora.step() == 0, k
        U, L = ref.solution()
        assert _rel(ora.U, U) < 1e-9, k
        assert abs(ora.L - L) <= 1e-9 * abs(L), k
        assert abs(ora.arcLength - ref.info()["length"]) <= 1e-12 * abs(ora.arcLength), k


@pytest.mark.parametrize("method", ["Crisfield", "Riks", "ConsistentCrisfield", "LoadControl"])
def test_predictor_guess_matches_reference(oracle_mod, method):
    """setInitialGuess -> predictorGuess (gsALMCrisfield.hpp:167-191, gsALMRiks.hpp:137-170,
    gsALMConsistentCrisfield.hpp:150-175, gsALMLoadControl.hpp)."""
    prob = P.cylindrical_panel(m=6, p=2, load=1e5 if method == "Riks" else 1.0)
    A = oracle_mod.OracleAssembler(prob)
    opts = dict(ALM_BASE, Length={"Crisfield": 0.004, "Riks": 0.003, "ConsistentCrisfield": 0.004,
                                  "LoadControl": 100.0}[method])
    cls = {"Crisfield": oracle_mod.ALMCrisfield, "Riks": oracle_mod.ALMRiks,
           "ConsistentCrisfield": oracle_mod.ALMConsistentCrisfield, "LoadControl": oracle_mod.ALMLoadControl}[method]
    ref = RS.ALM(RS.Operators.from_assembler(A), method, opts)
    ref.initialize()
    ora = cls(A.jacobian, A.al_residual, A.force(), opts)
    ora.initialize()
    rng = np.random.default_rng(3)
    prev = (np.zeros(len(A.force())), 0.0)
    for k in range(5):
        if k >= 2:
            Ug = 2 * ora.U - prev[0] + 1e-3 * np.linalg.norm(ora.U - prev[0]) * rng.standard_normal(len(ora.U)) / np.sqrt(len(ora.U))
            Lg = 2 * ora.L - prev[1]
            ref.set_initial_guess(Ug, Lg)
            ora.set_initial_guess(Ug, Lg)
        prev = (ora.U.copy(), ora.L)
        assert ref.step() == ora.step() == 0, k
        U, L = ref.solution()
        assert _rel(ora.U, U) < 1e-10, k
        assert abs(ora.L - L) <= 1e-10 * abs(L), k


def test_stability_determinant_matches_reference(oracle_mod):
    """BifurcationMethod 0 (Determinant: the LDL^T D, gsALMBase.hpp:547-570) along a Crisfield path
    through the limit point: the same stability flag and stability change at every step."""
    prob = P.cylindrical_panel(m=6, p=2, load=1.0)
    A = oracle_mod.OracleAssembler(prob)
    opts = dict(ALM_BASE, Length=0.006, BifurcationMethod=0)
    ref = RS.ALM(RS.Operators.from_assembler(A), "Crisfield", opts)
    ref.initialize()
    ora = oracle_mod.ALMCrisfield(A.jacobian, A.al_residual, A.force(), opts)
    ora.initialize()
    changes = 0
    for k in range(14):
        assert ref.step() == ora.step() == 0, k
        info = ref.info()
        assert int(info["stability"]) == ora.stability, k
        assert bool(info["stability_change"]) == ora.stability_change(), k
        changes += int(info["stability_change"])
    assert changes >= 1


@pytest.mark.parametrize("variant", ["Relaxation", "AutoScaling"])
def test_crisfield_relaxation_and_scaling_match_reference(oracle_mod, variant):
    """Relaxation 0.7 (the corrector's load-factor update is damped when it changes sign and
    shrinks, gsALMCrisfield.hpp:84-90) on ten converging steps, and the default Scaling -1 (phi
    from the first predictor, gsALMCrisfield.hpp:111-164) up to the step where both stop
    NotConverged: every status, iteration count and point is the reference's."""
    A = oracle_mod.OracleAssembler(P.cylindrical_panel(m=6, p=2, load=1.0))
    extra = {"Relaxation": dict(Relaxation=0.7, Scaling=0.0), "AutoScaling": dict(Scaling=-1.0)}[variant]
    opts = dict(ALM_BASE, Length=0.01, MaxIter=40, **extra)
    ref = RS.ALM(RS.Operators.from_assembler(A), "Crisfield", opts)
    ref.initialize()
    ora = oracle_mod.ALMCrisfield(A.jacobian, A.al_residual, A.force(), opts)
    ora.initialize()
    statuses = []
    for k in range(10):
        st = ref.step()
        assert ora.step() == st, k
        assert int(ref.info()["iterations"]) == ora.num_iterations, k
        U, L = ref.solution()
        assert abs(ora.L - L) <= 1e-12 * abs(L) and _rel(ora.U, U) < 1e-12, k
        statuses.append(st)
        if st != 0:
            break
    assert statuses == ([0] * 10 if variant == "Relaxation" else [0] * 6 + [1])


def test_dense_eigen_compute_and_power_match_reference(oracle_mod):
    """gsEigenProblemBase::compute (dense generalized solver, all pairs, with and without a shift)
    and ::computePower (power iteration on A^-1 B: the pair of smallest |lambda|) of
    gsModalSolver, against scipy's dense generalized eigensolver."""
    import scipy.linalg as sla
    prob = P.flat_plate(m=4, p=2, bc="simply")
    A = oracle_mod.OracleAssembler(prob)
    K, M = A.linear().toarray(), A.mass().toarray()
    w = sla.eigh(K, M, eigvals_only=True)
    for shift in (0.0, 0.5 * w[0]):
        st, vals, vecs = RS.eigen_dense("modal", K, M, dict(shift=shift))
        assert st == 0
        assert np.abs(vals - w).max() <= 1e-9 * np.abs(w).max()
        for j in range(len(w)):
            v = vecs[:, j]
            assert np.linalg.norm(K @ v - vals[j] * (M @ v)) <= 1e-8 * np.linalg.norm(K @ v)
    st, val, vec = RS.eigen_dense("modal", K, M, dict(tolerance=1e-12), power=True)
    assert st == 0
    assert abs(val[0] - w[0]) <= 1e-8 * w[0]


DYN_METHODS = ["Newmark", "Bathe", "Wilson", "ExplicitEuler", "ImplicitEuler", "RK4"]


def _dyn_pair(callbacks, n, method, nonlinear, opts):
    import dynamics as D
    ora = D.Dynamic(method, nonlinear, callbacks["mass"], callbacks["damping"], callbacks["jacobian"],
                    callbacks["residual"], callbacks["force"], opts)
    ref = RS.Dynamic(method, nonlinear, n, callbacks["mass"], callbacks["damping"], callbacks["jacobian"],
                     callbacks["residual"], callbacks["force"], opts)
    return ora, ref


def _close(a, b, tol):
    return np.abs(np.asarray(a) - b).max() <= tol * max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("nonlinear", [False, True])
@pytest.mark.parametrize("method", DYN_METHODS)
def test_integrator_matches_reference_on_spring_mass(method, nonlinear):
    """Three damped masses on springs under a force growing in time, F(t) = (1 + 40 t) F0, from
    the consistent start acceleration: every integrator of the restatement (oracle/dynamics.py)
    and of the reference reach the same U, V and A after each of 6 steps, and the same status."""
    import scipy.sparse as sp
    M = sp.diags([1.0, 2.0, 1.5]).tocsr()
    K = sp.csr_matrix(np.array([[300.0, -100.0, 0.0], [-100.0, 250.0, -150.0], [0.0, -150.0, 200.0]]))
    C = 0.3 * M + 1e-3 * K
    F0 = np.array([1.0, -2.0, 3.0])
    cb = dict(mass=lambda: M, damping=lambda U, t: C, jacobian=lambda U, t: K, force=lambda t: (1 + 40 * t) * F0,
              residual=lambda U, t: (1 + 40 * t) * F0 - K @ U)
    ora, ref = _dyn_pair(cb, 3, method, nonlinear, {"TolF": 1e-12, "TolU": 1e-12})
    A0 = np.linalg.solve(M.toarray(), F0)
    ora.set_state(np.zeros(3), np.zeros(3), A0)
    ref.set_state(np.zeros(3), np.zeros(3), A0)
    for k in range(6):
        assert ora.step(2e-3) == ref.step(2e-3) == 0, k
        U, V, A, t, _ = ref.state()
        assert abs(t - 2e-3 * (k + 1)) < 1e-15
        assert _close(ora.U, U, 1e-12) and _close(ora.V, V, 1e-12) and _close(ora.A, A, 1e-10), k


@pytest.mark.parametrize("nonlinear", [False, True])
@pytest.mark.parametrize("method", DYN_METHODS)
def test_integrator_matches_reference_on_shell(oracle_mod, method, nonlinear):
    """The cylindrical panel with Rayleigh damping under a load ramped from 0.2 to 1 (the KL-shell
    operators of the FP64 oracle, the same on both sides): 4 steps of each integrator, the
    restatement against the reference.  Explicit integrators take a step below their stability
    limit and mass-proportional damping only."""
    import dynamics as D
    A = oracle_mod.OracleAssembler(P.cylindrical_panel(m=4, p=2, load=400.0))
    explicit = method in ("ExplicitEuler", "RK4")
    cb = D.shell_callbacks(A, nonlinear, 0.5, 0.0 if explicit else 1e-4, D.load_table([0.0, 2e-3], [0.2, 1.0]))
    n = len(A.force())
    ora, ref = _dyn_pair(cb, n, method, nonlinear, {"TolF": 1e-10, "TolU": 1e-10})
    z = np.zeros(n)
    ora.set_state(z, z, z)
    ref.set_state(z, z, z)
    dt = 2e-7 if explicit else 5e-4
    for k in range(4):
        assert ora.step(dt) == ref.step(dt) == 0, k
        U, V, A_, _, _ = ref.state()
        assert _close(ora.U, U, 1e-11) and _close(ora.V, V, 1e-11), k
        if not explicit:            # the explicit integrators carry A unchanged
            assert _close(ora.A, A_, 1e-9), k
    assert np.abs(U).max() > 0      # the ramped load has moved the shell


try:
    import pytest_timeout  # noqa: F401
    # gsAPALM::_initiation retries a failed step with `while (diverged)` and no bound, so a
    # mistake in the harness would hang the run: end it instead
    _bounded = pytest.mark.timeout(300, method="thread")
except ImportError:
    def _bounded(f):
        return f


def _apalm_pair(oracle_mod, oa, method, alm_opts, ap_opts, data_opts):
    """The reference's APALM and the restatement's over the same arc-length method, each ALM
    initialised before the APALM is built, as the reference's APALM drivers do
    (examples/snapping_example_shell_APALM.cpp:488-537)."""
    import apalm as AP
    ref_alm = RS.ALM(RS.Operators.from_assembler(oa), method, alm_opts)
    ref_alm.initialize()
    ref = RS.APALM(ref_alm, ap_opts, data_opts)
    cls = {"Crisfield": oracle_mod.ALMCrisfield, "Riks": oracle_mod.ALMRiks}[method]
    ora_alm = cls(oa.jacobian, oa.al_residual, oa.force(), alm_opts)
    ora_alm.initialize()
    ora = AP.APALM(ora_alm, dict(ap_opts, **data_opts))
    return ref, ora


def _same_flat_path(ref, ora):
    assert ref.branches() == len(ora.times) == 1
    Us, Ls, ts, lvs = ref.flat(0)
    assert len(ts) == len(ora.times[0]) > 8
    assert lvs == list(ora.levels[0])
    np.testing.assert_allclose(ora.times[0], ts, rtol=1e-12, atol=1e-15)
    for U, L, (Uo, Lo) in zip(Us, Ls, ora.solutions[0]):
        assert abs(Lo - L) <= 1e-12 * max(abs(L), 1.0)
        assert _rel(Uo, U) < 1e-12 or np.abs(U).max() == np.abs(Uo).max() == 0


@_bounded
@pytest.mark.parametrize("schedule", ["serial_then_parallel", "solve"])
def test_apalm_matches_reference(oracle_mod, schedule):
    """gsAPALM (the build without MPI) over gsALMCrisfield: the coarse serial path, then the
    interval corrections of two refinement levels with two sub-intervals each -- either
    serialSolve + parallelSolve, or the interleaved solve() -- give the restatement's flat path:
    the same points in the same order, the same levels, the same curve times."""
    oa = oracle_mod.OracleAssembler(P.cylindrical_panel(m=6, p=2, load=1.0))
    alm_opts = dict(ALM_BASE, Length=0.02)
    ref, ora = _apalm_pair(oracle_mod, oa, "Crisfield", alm_opts, dict(SubIntervals=2, MaxIt=40),
                           dict(MaxLevel=2, Tolerance=1e-3))
    ref.initialize()
    ora.initialize()
    if schedule == "solve":
        ref.solve(5)
        ora.solve(5)
    else:
        ref.serial_solve(5)
        ora.serial_solve(5)
        ref.parallel_solve()
        ora.parallel_solve()
    _same_flat_path(ref, ora)


@_bounded
def test_apalm_over_riks_matches_reference(oracle_mod):
    """gsAPALM over gsALMRiks, whose interval distances are measured in Riks's norm: three
    sub-intervals, one refinement level."""
    oa = oracle_mod.OracleAssembler(P.cylindrical_panel(m=5, p=2, load=1e5))
    alm_opts = dict(TolF=1e-8, TolU=1e-6, MaxIter=30, BifurcationMethod=-1, Length=0.003)
    ref, ora = _apalm_pair(oracle_mod, oa, "Riks", alm_opts, dict(SubIntervals=3, MaxIt=20),
                           dict(MaxLevel=1, Tolerance=1e-4))
    ref.initialize()
    ora.initialize()
    ref.solve(4)
    ora.solve(4)
    _same_flat_path(ref, ora)


@pytest.mark.parametrize("tolB", [0.0, 1e-2])
def test_singular_point_matches_reference(oracle_mod, tolB):
    """At the roof's limit point (the step where the Determinant indicator changes sign):
    isBifurcation (_testSingularPoint: inverse iteration, |V.F| against the tolerance),
    computeSingularPoint without and with the bisection stage (SingularPointComputeTolB), and
    switchBranch, of the compiled gsALMBase against the restatement (gsALMBase.hpp:421-512,
    628-852).  The reference's unqualified abs() is the floating-point one here (the stand-in
    sees the <stdlib.h> / <math.h> overloads)."""
    A = oracle_mod.OracleAssembler(P.cylindrical_panel(m=8, p=2, load=1.0))
    opts = dict(Length=0.004, TolF=1e-8, TolU=1e-6, Scaling=0.0, MaxIter=8, BifurcationMethod=0,
                SingularPointComputeTolB=tolB)
    ref = RS.ALM(RS.Operators.from_assembler(A), "Crisfield", opts)
    ref.initialize()
    ora = oracle_mod.ALMCrisfield(A.jacobian, A.al_residual, A.force(), opts)
    ora.initialize()
    for k in range(12):
        Ur, Lr = ref.solution()
        Uo, Lo = ora.U.copy(), ora.L
        assert ref.step() == ora.step() == 0, k
        assert bool(ref.info()["stability_change"]) == ora.stability_change(), k
        if ora.stability_change():
            break
    else:
        pytest.fail("no stability change")
    assert ref.is_bifurcation(False) == ora.is_bifurcation(False) is False      # a limit point
    assert ref.compute_singular_point(Ur, Lr, False, False, False) == ora.compute_singular_point(Uo, Lo, False, False, False) == 0
    U, L = ref.solution()
    assert abs(ora.L - L) <= 1e-12 * abs(L) and _rel(ora.U, U) < 1e-10
    ref.switch_branch()
    ora.switch_branch()
    U, L = ref.solution()
    assert abs(ora.L - L) <= 1e-12 * abs(L) and _rel(ora.U, U) < 1e-10


def test_eigenvalue_stability_indicator_against_reference_builds(oracle_mod):
    """BifurcationMethod 1 (Eigenvalue) along a Crisfield path through the limit point.  The
    reference has two builds (gsALMBase.hpp:_computeStability): with Spectra, a shift-invert
    solve at the shift -100 that keeps the eigenvalues with the largest 1/(lambda + 100), so its
    indicator is the smallest eigenvalue ABOVE the shift; without Spectra (as compiled here), a
    dense SelfAdjointEigenSolver, the smallest eigenvalue.  The restatement (and the GPU) follow
    the Spectra build.  So: wherever the dense indicator is above the shift the two agree, flags
    included; where an eigenvalue lies below the shift the Spectra-build indicator stays above
    it (the path is then called stable there)."""
    A = oracle_mod.OracleAssembler(P.cylindrical_panel(m=5, p=2, load=1.0))
    opts = dict(ALM_BASE, Length=0.006, BifurcationMethod=1)
    ref = RS.ALM(RS.Operators.from_assembler(A), "Crisfield", opts)
    ref.initialize()
    ora = oracle_mod.ALMCrisfield(A.jacobian, A.al_residual, A.force(), opts)
    ora.initialize()
    agree = below = 0
    for k in range(10):
        assert ref.step() == ora.step() == 0, k
        U, L = ref.solution()
        assert _rel(ora.U, U) < 1e-10, k
        dense = ref.info()["indicator"]
        if dense > -100.0:
            assert abs(ora.indicator - dense) <= 1e-8 * abs(dense), k
            agree += 1
        else:
            assert ora.indicator > -100.0, k
            below += 1
    assert agree >= 5 and below >= 1


@pytest.mark.parametrize("edge_load", [1.0, -1.0])
def test_buckling_solver_power_matches_reference(oracle_mod, edge_load):
    """gsBucklingSolver built from K_L, the load and the Jacobian callback (its own set-up: u_L =
    K_L^-1 s F, B = K(u_L) - K_L), then computePower, on the simply supported square plate:
    the eigenvalue of smallest |lambda| is the restatement's (the dense pencil's) and gives
    q_cr = 4 pi^2 D / b^2.  Under tension the iterates converge (Success); under compression the
    dominant eigenvalue of A^-1 B is negative, the iterates flip sign every step and the
    reference stops NotConverged after its 100 steps -- with the same value."""
    E, nu, t = 1.0, 0.3, 0.01
    prob = P.flat_plate(m=8, p=3, E=E, nu=nu, t=t, pressure=0.0, bc="simply")
    n, ncp = prob.n1, prob.ncp
    ii, jj = np.arange(ncp) % n, np.arange(ncp) // n
    bnd = (ii == 0) | (ii == n - 1) | (jj == 0) | (jj == n - 1)
    fixed = np.zeros((3, ncp), dtype=bool)
    fixed[2, bnd] = True
    fixed[0, ii == 0] = True
    fixed[1, 0] = True
    prob.fixed = fixed.ravel()
    prob.edge_loads = np.array([[1, edge_load, 0.0, 0.0]])
    A = oracle_mod.OracleAssembler(prob)
    s = 1e-8
    st, val, vec = RS.buckling_power(RS.Operators.from_assembler(A), s, {"tolerance": 1e-12})
    assert st == (0 if edge_load > 0 else 1)
    lam, _, _ = oracle_mod.buckling_dense(A.linear(), A.force(), A.jacobian, nev=1, shift=0.0, scaling=s)
    assert abs(val - lam[0]) <= 1e-8 * abs(lam[0])
    D = E * t ** 3 / (12 * (1 - nu ** 2))
    assert abs(abs(val) * s / (4 * np.pi ** 2 * D) - 1) < 1e-4
    assert np.sign(val) == np.sign(edge_load)


def test_bifurcation_and_branch_switch_match_reference(oracle_mod):
    """A genuine bifurcation: the flat simply supported plate under in-plane compression (no
    imperfection).  Crisfield with the Determinant indicator runs up the membrane path; at the
    stability change the singular-point test finds the null vector orthogonal to the load
    (isBifurcation true), the extended system converges to the critical point (within 1.2 % of
    q_cr = 4 pi^2 D / b^2 on this 6 x 6 quadratic mesh), switchBranch steps onto the buckled
    branch, and three steps follow it -- every point the restatement's."""
    E, nu, t = 1.0, 0.3, 0.01
    prob = P.flat_plate(m=6, p=2, E=E, nu=nu, t=t, pressure=0.0, bc="simply")
    n, ncp = prob.n1, prob.ncp
    ii, jj = np.arange(ncp) % n, np.arange(ncp) // n
    bnd = (ii == 0) | (ii == n - 1) | (jj == 0) | (jj == n - 1)
    fixed = np.zeros((3, ncp), dtype=bool)
    fixed[2, bnd] = True
    fixed[0, ii == 0] = True
    fixed[1, 0] = True
    prob.fixed = fixed.ravel()
    prob.edge_loads = np.array([[1, -1e-6, 0.0, 0.0]])
    A = oracle_mod.OracleAssembler(prob)
    opts = dict(Length=2e-4, TolF=1e-9, TolU=1e-9, Scaling=0.0, MaxIter=20, BifurcationMethod=0,
                SingularPointComputeTolB=0.0)
    ref = RS.ALM(RS.Operators.from_assembler(A), "Crisfield", opts)
    ref.initialize()
    ora = oracle_mod.ALMCrisfield(A.jacobian, A.al_residual, A.force(), opts)
    ora.initialize()
    for k in range(15):
        Ur, Lr = ref.solution()
        Uo, Lo = ora.U.copy(), ora.L
        assert ref.step() == ora.step() == 0, k
        assert bool(ref.info()["stability_change"]) == ora.stability_change(), k
        if ora.stability_change():
            break
    else:
        pytest.fail("no stability change")
    assert ref.is_bifurcation(False) is True and ora.is_bifurcation(False) is True
    assert ref.compute_singular_point(Ur, Lr, False, False, False) == ora.compute_singular_point(Uo, Lo, False, False, False) == 0
    U, L = ref.solution()
    assert abs(ora.L - L) <= 1e-12 * abs(L) and _rel(ora.U, U) < 1e-10
    D = E * t ** 3 / (12 * (1 - nu ** 2))
    assert abs(L * 1e-6 / (4 * np.pi ** 2 * D) - 1) < 0.012
    ref.switch_branch()
    ora.switch_branch()
    for k in range(3):
        U, L = ref.solution()
        assert abs(ora.L - L) <= 1e-12 * abs(L) and _rel(ora.U, U) < 1e-10, k
        assert ref.step() == ora.step() == 0, k
    U, L = ref.solution()
    assert abs(ora.L - L) <= 1e-12 * abs(L) and _rel(ora.U, U) < 1e-10


def test_crisfield_complex_roots_match_reference(oracle_mod):
    """Quasi-Newton Crisfield (the tangent refreshed every 8 iterations) with a long step on the
    coarse roof: in step 2 the constraint quadratic has no real root, so the corrector takes Lam's
    modified quadratic for eta with the 0.05 |eta2 - eta1| shift and, where that fails too, the
    complex-root fallback (gsALMCrisfield.hpp:236-330); the step still converges, after 25
    iterations.  Every step -- its status, iteration count and point -- is the reference's, and
    the restatement is seen to take both paths."""
    A = oracle_mod.OracleAssembler(P.cylindrical_panel(m=4, p=2, load=1.0))
    opts = dict(Length=0.01, TolF=1e-8, TolU=1e-6, Scaling=0.0, MaxIter=40, BifurcationMethod=-1, Quasi=True,
                QuasiIterations=8)
    ref = RS.ALM(RS.Operators.from_assembler(A), "Crisfield", opts)
    ref.initialize()
    ora = oracle_mod.ALMCrisfield(A.jacobian, A.al_residual, A.force(), opts)
    ora.initialize()
    calls = {"modified": 0, "complex": 0}
    modified, complex_ = ora._lambdas_modified, ora._lambdas_complex

    def count(name, fn):
        def wrapped():
            calls[name] += 1
            return fn()
        return wrapped

    ora._lambdas_modified = count("modified", modified)
    ora._lambdas_complex = count("complex", complex_)
    converged_with = 0
    for k in range(6):
        before = dict(calls)
        st = ref.step()
        assert ora.step() == st, k
        assert int(ref.info()["iterations"]) == ora.num_iterations, k
        U, L = ref.solution()
        assert abs(ora.L - L) <= 1e-12 * abs(L) and _rel(ora.U, U) < 1e-12, k
        if st == 0 and calls["modified"] > before["modified"] and calls["complex"] > before["complex"]:
            converged_with += 1
        if st != 0:
            break
    assert converged_with >= 1


@pytest.mark.parametrize("method,variant", [(m, v) for m in ("Riks", "LoadControl", "ConsistentCrisfield")
                                            for v in ("Quasi", "AdaptiveLength")])
def test_method_variants_match_reference(oracle_mod, method, variant):
    """Quasi-Newton and AdaptiveLength for Riks, LoadControl and ConsistentCrisfield.  The
    adaptive factor is AdaptiveIterations / iterations as a quotient of two index_t, an integer
    division (gsALMBase.hpp:105-116): after a 5-iteration Riks step with 3 desired iterations it
    is 0, clamped to 0.5 (a real division would give 0.6)."""
    load, length = {"Riks": (1e5, 0.003), "LoadControl": (1.0, 100.0), "ConsistentCrisfield": (1.0, 0.004)}[method]
    A = oracle_mod.OracleAssembler(P.cylindrical_panel(m=6, p=2, load=load))
    extra = dict(Quasi=True, QuasiIterations=2) if variant == "Quasi" else dict(AdaptiveLength=True, AdaptiveIterations=3)
    opts = dict(ALM_BASE, Length=length, **extra)
    ref = RS.ALM(RS.Operators.from_assembler(A), method, opts)
    ref.initialize()
    cls = {"Riks": oracle_mod.ALMRiks, "LoadControl": oracle_mod.ALMLoadControl,
           "ConsistentCrisfield": oracle_mod.ALMConsistentCrisfield}[method]
    ora = cls(A.jacobian, A.al_residual, A.force(), opts)
    ora.initialize()
    for k in range(6):
        assert ref.step() == ora.step() == 0, k
        assert int(ref.info()["iterations"]) == ora.num_iterations, k
        U, L = ref.solution()
        assert abs(ora.L - L) <= 1e-12 * abs(L) and _rel(ora.U, U) < 1e-12, k
        assert abs(ora.arcLength - ref.info()["length"]) <= 1e-12 * abs(ora.arcLength), k
    if method == "Riks" and variant == "AdaptiveLength":
        assert ref.info()["length"] == 0.5 * length


@pytest.mark.parametrize("solver", ["SimplicialLDLT", "CGDiagonal"])
def test_static_newton_relaxation_matches_reference(oracle_mod, solver):
    """gsStaticNewton with Relaxation 0.7 (the update scaled, gsStaticNewton.hpp:160-185): the
    same iteration count (16, against 4 unrelaxed) and the same solution."""
    A = oracle_mod.OracleAssembler(P.cylindrical_panel(m=6, p=3, load=800.0))
    opts = dict(tol=1e-8, maxIt=60, Relaxation=0.7)
    ref = RS.StaticNewton(RS.Operators.from_assembler(A), dict(opts, Solver=solver))
    ora = oracle_mod.StaticNewton(A.linear(), A.force(), A.jacobian, A.residual, opts)
    assert ref.solve() == ora.solve() == 0
    assert ref.iterations() == ora.num_iterations == 16
    assert _rel(ora.U, ref.solution()) < 1e-12


@pytest.mark.parametrize("method", ["Newmark", "Bathe", "Wilson", "ImplicitEuler"])
def test_quasi_newton_integrators_match_reference(oracle_mod, method):
    """The nonlinear integrators with Quasi (the tangent refreshed every QuasiIterations = 2
    corrector iterations) on the damped shell under a ramped load: 4 steps, U to 1e-12."""
    import dynamics as D
    A = oracle_mod.OracleAssembler(P.cylindrical_panel(m=4, p=2, load=400.0))
    cb = D.shell_callbacks(A, True, 0.5, 1e-4, D.load_table([0.0, 2e-3], [0.2, 1.0]))
    n = len(A.force())
    ora, ref = _dyn_pair(cb, n, method, True, {"TolF": 1e-10, "TolU": 1e-10, "Quasi": 1, "QuasiIterations": 2})
    z = np.zeros(n)
    ora.set_state(z, z, z)
    ref.set_state(z, z, z)
    for k in range(4):
        assert ora.step(5e-4) == ref.step(5e-4) == 0, k
        U, V, _, _, _ = ref.state()
        assert _close(ora.U, U, 1e-12) and _close(ora.V, V, 1e-11), k


def _compressed_plate():
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
    return prob


@pytest.mark.parametrize("variant,extra,switch,jacobian", [
    ("Perturbation", dict(Perturbation=1e2), True, False),
    ("TestIt", dict(SingularPointTestIt=2), False, False),
    ("ComputeTolE", dict(SingularPointComputeTolE=1e-4), False, False),
    ("SwitchInside", {}, True, False),
    ("Jacobian", {}, True, True),
    ("Bisection", dict(SingularPointComputeTolB=1e-2), True, False),
    ("FailureSwitch", dict(SingularPointFailure=1, SingularPointComputeTolE=1e-14), True, False),
])
def test_singular_point_options_match_reference(oracle_mod, variant, extra, switch, jacobian):
    """The options of computeSingularPoint at the plate's bifurcation (gsALMBase.hpp:41-46,
    628-852): the perturbation tau of the extended system, the power iterations of the test, the
    extended-system tolerance, switching inside the call, a fresh Jacobian, the bisection stage,
    and SingularPointFailure 1 (switch even when the extended iterations do not converge); the
    critical point and the next step on the buckled branch are the reference's."""
    A = oracle_mod.OracleAssembler(_compressed_plate())
    opts = dict(Length=2e-4, TolF=1e-9, TolU=1e-9, Scaling=0.0, MaxIter=20, BifurcationMethod=0,
                SingularPointComputeTolB=0.0)
    opts.update(extra)
    ref = RS.ALM(RS.Operators.from_assembler(A), "Crisfield", opts)
    ref.initialize()
    ora = oracle_mod.ALMCrisfield(A.jacobian, A.al_residual, A.force(), opts)
    ora.initialize()
    for k in range(15):
        Ur, Lr = ref.solution()
        Uo, Lo = ora.U.copy(), ora.L
        assert ref.step() == ora.step() == 0, k
        if ora.stability_change():
            break
    else:
        pytest.fail("no stability change")
    st = ref.compute_singular_point(Ur, Lr, switch, jacobian, True)
    assert ora.compute_singular_point(Uo, Lo, switch, jacobian, True) == st
    U, L = ref.solution()
    assert abs(ora.L - L) <= 1e-12 * abs(L) and _rel(ora.U, U) < 1e-12
    assert ref.step() == ora.step() == 0
    U, L = ref.solution()
    assert abs(ora.L - L) <= 1e-12 * abs(L) and _rel(ora.U, U) < 1e-12


@_bounded
@pytest.mark.parametrize("schedule", ["serial", "solve"])
def test_apalm_branches_at_bifurcation_match_reference(oracle_mod, schedule):
    """gsAPALM with SingularPoint on the compressed plate: the initiation job that crosses the
    bifurcation computes the critical point, switches branch and queues the buckled branch as a
    new start (gsAPALM.hpp:934-1011, BifLengthMultiplier for its first step); serialSolve, or
    solve with the interval corrections, gives the same two branches as the restatement --
    points, levels and curve times."""
    import apalm as AP
    A = oracle_mod.OracleAssembler(_compressed_plate())
    alm_opts = dict(Length=2e-4, TolF=1e-9, TolU=1e-9, Scaling=0.0, MaxIter=20, BifurcationMethod=0,
                    SingularPointComputeTolB=0.0)
    ap_opts = dict(SubIntervals=2, MaxIt=40, SingularPoint=True, BranchLengthMultiplier=1.0, BifLengthMultiplier=0.1)
    data_opts = dict(MaxLevel=1, Tolerance=1e-3)
    ref_alm = RS.ALM(RS.Operators.from_assembler(A), "Crisfield", alm_opts)
    ref_alm.initialize()
    ref = RS.APALM(ref_alm, ap_opts, data_opts)
    ora_alm = oracle_mod.ALMCrisfield(A.jacobian, A.al_residual, A.force(), alm_opts)
    ora_alm.initialize()
    ora = AP.APALM(ora_alm, dict(ap_opts, **data_opts))
    ref.initialize()
    ora.initialize()
    if schedule == "serial":
        ref.serial_solve(14)
        ora.serial_solve(14)
    else:
        ref.solve(14)
        ora.solve(14)
    assert ref.branches() == len(ora.times) == 2
    for b in range(2):
        Us, Ls, ts, lvs = ref.flat(b)
        assert len(ts) == len(ora.times[b]) > 10 and lvs == list(ora.levels[b])
        np.testing.assert_allclose(ora.times[b], ts, rtol=1e-12, atol=1e-15)
        for U, L, (Uo, Lo) in zip(Us, Ls, ora.solutions[b]):
            assert abs(Lo - L) <= 1e-12 * max(abs(L), 1e-300)
            assert _rel(Uo, U) < 1e-12 or np.abs(U).max() == np.abs(Uo).max() == 0


@pytest.mark.parametrize("method", ["ConsistentCrisfield", "Riks"])
def test_determinant_flags_other_methods_match_reference(oracle_mod, method):
    """BifurcationMethod 0 along ConsistentCrisfield (through both limit points of the roof: two
    stability changes) and Riks (up to the step where both stop NotConverged): every status,
    stability flag and point is the reference's."""
    load, length, steps = {"ConsistentCrisfield": (1.0, 0.004, 20), "Riks": (1e5, 0.002, 40)}[method]
    A = oracle_mod.OracleAssembler(P.cylindrical_panel(m=6, p=2, load=load))
    opts = dict(ALM_BASE, Length=length, MaxIter=60, BifurcationMethod=0)
    ref = RS.ALM(RS.Operators.from_assembler(A), method, opts)
    ref.initialize()
    cls = {"ConsistentCrisfield": oracle_mod.ALMConsistentCrisfield, "Riks": oracle_mod.ALMRiks}[method]
    ora = cls(A.jacobian, A.al_residual, A.force(), opts)
    ora.initialize()
    changes = 0
    for k in range(steps):
        st = ref.step()
        assert ora.step() == st, k
        if st != 0:
            break
        info = ref.info()
        assert int(info["stability"]) == ora.stability and bool(info["stability_change"]) == ora.stability_change(), k
        changes += int(info["stability_change"])
        U, L = ref.solution()
        assert abs(ora.L - L) <= 1e-12 * abs(L) and _rel(ora.U, U) < 1e-12, k
    assert changes == (2 if method == "ConsistentCrisfield" else 0)
    assert (st == 0) == (method == "ConsistentCrisfield")


@pytest.mark.parametrize("solver", ["SimplicialLDLT", "CGDiagonal"])
def test_static_newton_solve_linear_matches_reference(oracle_mod, solver):
    """gsStaticNewton::solveLinear (gsStaticNewton.hpp:57-99, 195-213): K_L u = F with the named
    solver, on the clamped plate and on the roof; then a zero pivot (E = 0) is SolverError for
    the factorising solver."""
    for prob in (P.flat_plate(m=4, p=2), P.cylindrical_panel(m=6, p=3, load=800.0)):
        A = oracle_mod.OracleAssembler(prob)
        ref = RS.StaticNewton(RS.Operators.from_assembler(A), dict(Solver=solver))
        ora = oracle_mod.StaticNewton(A.linear(), A.force(), A.jacobian, A.residual, {})
        assert ref.solve_linear() == 0
        U = ora.solve_linear()                                  # the restatement returns u (_solveLinear)
        tol = 1e-12 if solver == "SimplicialLDLT" else 1e-8      # CG to machine-epsilon residual
        assert _rel(U, ref.solution()) < tol
    A = oracle_mod.OracleAssembler(P.flat_plate(m=4, p=2, E=0.0))
    ref = RS.StaticNewton(RS.Operators.from_assembler(A), dict(Solver="SimplicialLDLT"))
    assert ref.solve_linear() == 3


def test_failure_recovery_with_reduce_length_matches_reference(oracle_mod):
    """The reference drivers' recovery: after a NotConverged step, reduceLength(0.5) and step
    again from the last converged point (gsALMBase.hpp:118-123, 328-351).  Fourteen steps with the
    default automatic Scaling, three of them failing: every status, iteration count, arc length
    and point is the reference's."""
    A = oracle_mod.OracleAssembler(P.cylindrical_panel(m=6, p=2, load=1.0))
    opts = dict(ALM_BASE, Scaling=-1.0, MaxIter=40, Length=0.01)
    ref = RS.ALM(RS.Operators.from_assembler(A), "Crisfield", opts)
    ref.initialize()
    ora = oracle_mod.ALMCrisfield(A.jacobian, A.al_residual, A.force(), opts)
    ora.initialize()
    failures = 0
    for k in range(14):
        st = ref.step()
        assert ora.step() == st, k
        assert int(ref.info()["iterations"]) == ora.num_iterations, k
        U, L = ref.solution()
        assert abs(ora.L - L) <= 1e-12 * abs(L) and _rel(ora.U, U) < 1e-12, k
        if st != 0:
            failures += 1
            ref.reduce_length(0.5)
            ora.reduce_length(0.5)
        assert ora.arcLength == ref.info()["length"], k
    assert failures == 3


@pytest.mark.parametrize("nonlinear", [False, True])
@pytest.mark.parametrize("method,params", [("Newmark", dict(alpha=0.3025, delta=0.6)), ("Bathe", dict(gamma=0.6)),
                                           ("Wilson", dict(gamma=1.37)),
                                           ("Bathe", dict(alpha=0.3025, delta=0.6, gamma=0.5))])
def test_integrator_parameters_match_reference(oracle_mod, method, params, nonlinear):
    """The integrators' own options away from their defaults (gsDynamicNewmark / Bathe / Wilson
    defaultOptions): Newmark with numerical damping (alpha 0.3025, delta 0.6), Bathe's sub-step
    gamma and its Newmark stage parameters, Wilson's theta (gamma); 4 steps on the damped shell,
    U and V to 1e-12 of their maxima."""
    import dynamics as D
    A = oracle_mod.OracleAssembler(P.cylindrical_panel(m=4, p=2, load=400.0))
    cb = D.shell_callbacks(A, nonlinear, 0.5, 1e-4, D.load_table([0.0, 2e-3], [0.2, 1.0]))
    n = len(A.force())
    ora, ref = _dyn_pair(cb, n, method, nonlinear, dict({"TolF": 1e-10, "TolU": 1e-10}, **params))
    z = np.zeros(n)
    ora.set_state(z, z, z)
    ref.set_state(z, z, z)
    for k in range(4):
        assert ora.step(5e-4) == ref.step(5e-4) == 0, k
        U, V, _, _, _ = ref.state()
        assert _close(ora.U, U, 1e-12) and _close(ora.V, V, 1e-12), k
