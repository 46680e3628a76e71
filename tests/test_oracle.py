"""CPU tests of the FP64 oracle: B-splines, finite-difference consistency of K and Fint,
closed-form plate answers, and the restated solver logic on analytic problems."""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from gsstructuralanalysis_gb300 import problems as P


def test_bspline_partition_of_unity(oracle_mod):
    for p in (2, 3):
        U = P.open_uniform_knots(p, 7)
        for u in np.linspace(0, 1, 23):
            _, b = oracle_mod.basis(p, U, u)
            assert abs(b[0].sum() - 1) < 1e-13
            assert abs(b[1].sum()) < 1e-10 and abs(b[2].sum()) < 1e-8


def test_bspline_derivatives_fd(oracle_mod):
    p, U, h = 3, P.open_uniform_knots(3, 5), 1e-6
    for u in (0.11, 0.37, 0.52, 0.93):
        s0, b0 = oracle_mod.basis(p, U, u)
        sp_, bp = oracle_mod.basis(p, U, u + h)
        sm, bm = oracle_mod.basis(p, U, u - h)
        assert s0 == sp_ == sm
        np.testing.assert_allclose((bp[0] - bm[0]) / (2 * h), b0[1], atol=1e-6)
        np.testing.assert_allclose((bp[1] - bm[1]) / (2 * h), b0[2], atol=1e-4)


@pytest.mark.parametrize("make", [lambda: P.cylindrical_panel(m=3, p=2), lambda: P.cylindrical_panel(m=2, p=3),
                                  lambda: P.flat_plate(m=3, p=2)])
def test_tangent_is_derivative_of_internal_force(oracle_mod, make):
    prob = make()
    A = oracle_mod.OracleAssembler(prob)
    x = 2e-3 * np.random.default_rng(0).standard_normal(A.nfree)
    K = A.jacobian(x).toarray()
    assert np.abs(K - K.T).max() <= 1e-12 * np.abs(K).max()
    h = 1e-7
    cols = np.random.default_rng(1).choice(A.nfree, size=min(24, A.nfree), replace=False)
    for k in cols:
        e = np.zeros(A.nfree); e[k] = h
        fd = (A.fint(x + e) - A.fint(x - e)) / (2 * h)
        assert np.abs(fd - K[:, k]).max() <= 1e-6 * np.abs(K).max()


def test_rigid_body_motion_is_stress_free(oracle_mod):
    prob = P.cylindrical_panel(m=3, p=2)
    prob.fixed[:] = False
    A = oracle_mod.OracleAssembler(prob)
    ncp = prob.ncp
    u = np.zeros(3 * ncp)
    u[:ncp] = 0.3; u[ncp:2 * ncp] = -0.1; u[2 * ncp:] = 0.05   # translation
    _, f = A.full_tangent_and_fint(u, False)
    assert np.abs(f).max() < 1e-6
    # finite rotation about z
    th = 0.4
    X = prob.ctrl
    R = np.array([[np.cos(th), -np.sin(th), 0], [np.sin(th), np.cos(th), 0], [0, 0, 1]])
    d = X @ R.T - X
    u = np.concatenate([d[:, 0], d[:, 1], d[:, 2]])
    _, f = A.full_tangent_and_fint(u, False)
    assert np.abs(f).max() < 1e-5


def test_clamped_plate_series_answer(oracle_mod):
    """Clamped square plate under uniform load: w_max = 0.00126532 q a^4 / D (Timoshenko)."""
    prob = P.flat_plate(m=16, p=2)
    A = oracle_mod.OracleAssembler(prob)
    u = A.to_full(spla.spsolve(A.linear().tocsc(), A.force()))
    D = prob.E * prob.t ** 3 / (12 * (1 - prob.nu ** 2))
    s1, b1 = oracle_mod.basis(2, prob.knots1, 0.5)
    s2, b2 = oracle_mod.basis(2, prob.knots2, 0.5)
    w = sum(b1[0][a] * b2[0][b] * u[2 * prob.ncp + (s2 - 2 + b) * prob.n1 + (s1 - 2 + a)]
            for a in range(3) for b in range(3))
    assert abs(w / (0.00126532 / D) - 1) < 0.02


def test_simply_supported_plate_frequencies(oracle_mod):
    """omega_mn = (m^2+n^2) pi^2 sqrt(D/(rho t)) -- the known answer printed by
    examples/gsThinShell_Modal.cpp:333 (t=0.01, E=1, nu=0.3, rho=1, unit square)."""
    prob = P.flat_plate(m=16, p=3, E=1.0, t=0.01, rho=1.0, bc="simply", pressure=0.0)
    A = oracle_mod.OracleAssembler(prob)
    vals, _ = oracle_mod.modal(A.linear(), A.mass(), nev=4, shift=0.0)
    D = prob.E * prob.t ** 3 / (12 * (1 - prob.nu ** 2))
    c = np.pi ** 2 * np.sqrt(D / (prob.rho * prob.t))
    omega = np.sort(np.sqrt(vals))
    expected = np.array([2, 5, 5, 8]) * c
    np.testing.assert_allclose(omega, expected, rtol=2e-3)


# ---- restated solver logic on analytic problems ---------------------------------------------
def _truss():
    """Two-dof shallow two-bar truss with a snap-through (Fint cubic in u1, spring on u2)."""
    k1, k2 = 1.0, 0.5

    def fint(x):
        u1, u2 = x
        return np.array([k1 * (u1 - 1.5 * u1 ** 2 + 0.5 * u1 ** 3) + 0.1 * (u1 - u2), k2 * u2 + 0.1 * (u2 - u1)])

    def jac(x):
        u1, u2 = x
        return sp.csr_matrix(np.array([[k1 * (1 - 3 * u1 + 1.5 * u1 ** 2) + 0.1, -0.1], [-0.1, k2 + 0.1]]))

    return fint, jac, np.array([1.0, 0.0])


@pytest.mark.parametrize("cls", ["ALMCrisfield", "ALMRiks", "ALMConsistentCrisfield"])
def test_arc_length_traces_snap_through(oracle_mod, cls):
    fint, jac, F = _truss()
    res = lambda x, lam: fint(x) - lam * F
    opts = dict(Length=0.05, TolF=1e-10, TolU=1e-10, MaxIter=30)
    if cls == "ALMConsistentCrisfield":
        # with the automatic phi = |u_t|/|F| the secant predictor turns back at the limit point
        opts["Scaling"] = 0.0
    alm = getattr(oracle_mod, cls)(jac, res, F, opts)
    lams, us = [], []
    for _ in range(80):
        assert alm.step() == 0
        lams.append(alm.L); us.append(alm.U[0])
        assert np.linalg.norm(res(alm.U, alm.L)) < 1e-8
    # passes the limit point (load decreases after a maximum) and keeps going
    assert max(lams) > lams[-1] or us[-1] > 1.5
    assert us[-1] > 1.0


def test_crisfield_constraint_is_met(oracle_mod):
    fint, jac, F = _truss()
    res = lambda x, lam: fint(x) - lam * F
    alm = oracle_mod.ALMCrisfield(jac, res, F, dict(Length=0.05, TolF=1e-12, TolU=1e-12, MaxIter=30, Scaling=0.0))
    for _ in range(10):
        U0 = alm.U.copy()
        assert alm.step() == 0
        assert abs(np.linalg.norm(alm.U - U0) - 0.05) < 1e-9


def test_consistent_crisfield_constraint_is_met(oracle_mod):
    """At convergence the linearised constraint of gsALMConsistentCrisfield is the spherical one."""
    fint, jac, F = _truss()
    res = lambda x, lam: fint(x) - lam * F
    alm = oracle_mod.ALMConsistentCrisfield(jac, res, F, dict(Length=0.05, TolF=1e-12, TolU=1e-12, MaxIter=30,
                                                              Scaling=0.0))
    for _ in range(10):
        U0 = alm.U.copy()
        assert alm.step() == 0
        assert abs(np.linalg.norm(alm.U - U0) - 0.05) < 1e-9


def test_static_newton_converges_quadratically(oracle_mod):
    fint, jac, F = _truss()
    F = 0.05 * F
    newton = oracle_mod.StaticNewton(jac(np.zeros(2)), F, jac, lambda x: F - fint(x), dict(tol=1e-12))
    assert newton.solve() == 0
    assert np.linalg.norm(F - fint(newton.U)) < 1e-12
    rs = [h[0] for h in newton.history]
    assert len(rs) <= 6


def test_newton_not_converged_status(oracle_mod):
    fint, jac, F = _truss()
    newton = oracle_mod.StaticNewton(jac(np.zeros(2)), 0.05 * F, jac, lambda x: 0.05 * F - fint(x),
                                     dict(tol=1e-14, maxIt=1))
    assert newton.solve() == oracle_mod.NOT_CONVERGED


def test_assembly_error_status(oracle_mod):
    fint, jac, F = _truss()
    newton = oracle_mod.StaticNewton(jac(np.zeros(2)), F, jac, lambda x: None, dict(tol=1e-10))
    assert newton.solve() == oracle_mod.ASSEMBLY_ERROR


def test_svk_membrane_uniaxial_stretch(oracle_mod):
    """Nonlinear pin of the membrane part, the edge loads and gsStaticNewton: a flat SVK sheet
    (nu = 0) pulled by a dead line load q on its right edge stretches uniformly to lambda with
    t E lambda (lambda^2 - 1) / 2 = q (first Piola stress of the Green-Lagrange strain).  The
    displacement field (lambda - 1) x lies in the spline space, so the discrete solution is exact."""
    lam, E, t = 1.2, 1e3, 0.01
    q = t * E * lam * (lam ** 2 - 1) / 2
    prob = P.flat_plate(m=4, p=2, E=E, t=t, nu=0.0, pressure=0.0)
    n, ncp = prob.n1, prob.ncp
    ii = np.arange(ncp) % n
    fixed = np.zeros((3, ncp), dtype=bool)
    fixed[0, ii == 0] = True          # x on the left edge
    fixed[1, 0] = True                # y at one corner
    fixed[2, :] = True                # flat: no out-of-plane motion
    prob.fixed = fixed.ravel()
    prob.edge_loads = np.array([[1, q, 0.0, 0.0]])
    A = oracle_mod.OracleAssembler(prob)
    N = oracle_mod.StaticNewton(A.linear(), A.force(), A.jacobian, A.residual, dict(tol=1e-12, maxIt=50))
    assert N.solve() == 0
    u = A.to_full(N.U).reshape(3, ncp)
    np.testing.assert_allclose(u[0], (lam - 1) * prob.ctrl[:, 0], atol=1e-10)
    assert np.abs(u[1]).max() < 1e-10


def test_plate_buckling_under_uniaxial_compression(oracle_mod):
    """Pin of the geometric stiffness (second variation of the membrane strain): a simply
    supported square plate under a uniform compressive edge load q buckles at
    q_cr = 4 pi^2 D / b^2 (one half-wave each way).  The gsBucklingSolver pencil
    K_L v = lambda B v, B = K(u_L) - K_L with u_L = K_L^-1 (s F), is the linear geometric
    stiffness of the load s F for a small reference load s; the critical load is -lambda s."""
    E, nu, t = 1.0, 0.3, 0.01
    prob = P.flat_plate(m=8, p=3, E=E, nu=nu, t=t, pressure=0.0, bc="simply")
    n, ncp = prob.n1, prob.ncp
    ii, jj = np.arange(ncp) % n, np.arange(ncp) // n
    bnd = (ii == 0) | (ii == n - 1) | (jj == 0) | (jj == n - 1)
    fixed = np.zeros((3, ncp), dtype=bool)
    fixed[2, bnd] = True              # w = 0 on the boundary (simple support)
    fixed[0, ii == 0] = True          # x held on the loaded opposite edge
    fixed[1, 0] = True                # y at one corner: free Poisson expansion
    prob.fixed = fixed.ravel()
    prob.edge_loads = np.array([[1, -1.0, 0.0, 0.0]])
    A = oracle_mod.OracleAssembler(prob)
    D = E * t ** 3 / (12 * (1 - nu ** 2))
    expected = 4 * np.pi ** 2 * D
    s = 1e-8                          # pre-buckling strain s q / (E t) = 1e-6
    lam, _, _ = oracle_mod.buckling_dense(A.linear(), A.force(), A.jacobian, nev=1, shift=-expected / s, scaling=s)
    assert abs(-lam[0] * s / expected - 1) < 1e-4      # 1.8e-5 at 8x8 cubic elements
