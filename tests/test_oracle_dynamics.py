"""The time-integrator restatement (oracle/dynamics.py) pinned without the reference: the
reference ships no test of gsDynamicSolvers, so the pins are closed-form answers of a
spring-mass system, the integrators' orders of accuracy, the reduction of each nonlinear variant
to its linear one on a linear problem, and a short nonlinear shell run."""
import numpy as np
import pytest
import scipy.linalg as sla
import scipy.sparse as sp

import dynamics as D


def _spring_mass(damp=0.0):
    # 3 masses on springs: M u'' + C u' + K u = F, from rest
    M = sp.diags([1.0, 2.0, 1.5]).tocsr()
    K = sp.csr_matrix(np.array([[300.0, -100.0, 0.0], [-100.0, 250.0, -150.0], [0.0, -150.0, 150.0]]) + np.diag([0, 0, 50.0]))
    C = damp * M
    F = np.array([1.0, -2.0, 3.0])
    return M, C, K, F


def _exact(M, C, K, F, t):
    """u(t) of M u'' + C u' + K u = F with u(0) = u'(0) = 0 (first-order form, matrix exponential)."""
    n = M.shape[0]
    Md, Cd, Kd = M.toarray(), C.toarray(), K.toarray()
    Mi = np.linalg.inv(Md)
    A = np.block([[np.zeros((n, n)), np.eye(n)], [-Mi @ Kd, -Mi @ Cd]])
    b = np.concatenate([np.zeros(n), Mi @ F])
    # x' = A x + b, x(0) = 0  ->  x(t) = A^-1 (e^{At} - I) b
    x = np.linalg.solve(A, (sla.expm(A * t) - np.eye(2 * n)) @ b)
    return x[:n], x[n:]


def _linear_solver(method, M, C, K, F, nonlinear=False, opts=None):
    cb = dict(mass=lambda: M, damping=lambda U, t: C, jacobian=lambda U, t: K,
              force=lambda t: F, residual=lambda U, t: F - K @ U)
    o = {"TolF": 1e-12, "TolU": 1e-12}
    o.update(opts or {})
    s = D.Dynamic(method, nonlinear, cb["mass"], cb["damping"], cb["jacobian"], cb["residual"], cb["force"], o)
    n = M.shape[0]
    # consistent initial acceleration M a0 = F - K u0 - C v0
    s.set_state(np.zeros(n), np.zeros(n), np.linalg.solve(M.toarray(), F))
    return s


def _run(s, dt, nsteps):
    for _ in range(nsteps):
        assert s.step(dt) == D.SUCCESS
    return s.U


@pytest.mark.parametrize("method,order", [("Newmark", 2), ("Bathe", 2), ("RK4", 4), ("ImplicitEuler", 1)])
def test_order_of_accuracy_against_closed_form(method, order):
    M, C, K, F = _spring_mass(damp=0.3)
    T = 0.5
    errs = []
    for nsteps in (100, 200):
        s = _linear_solver(method, M, C, K, F)
        U = _run(s, T / nsteps, nsteps)
        errs.append(np.linalg.norm(U - _exact(M, C, K, F, T)[0]))
    rate = np.log2(errs[0] / errs[1])
    assert abs(rate - order) < 0.3, (errs, rate)
    assert errs[1] < {1: 0.06, 2: 3e-4, 4: 5e-8}[order] * np.linalg.norm(_exact(M, C, K, F, T)[0])


def test_newmark_trapezoidal_conserves_energy_undamped():
    """Average acceleration (alpha 1/4, delta 1/2) conserves the energy of a free undamped
    linear system exactly."""
    M, C, K, F = _spring_mass()
    F0 = np.zeros(3)
    cb = dict(mass=lambda: M, damping=lambda U, t: C, jacobian=lambda U, t: K, force=lambda t: F0)
    s = D.Dynamic("Newmark", False, cb["mass"], cb["damping"], cb["jacobian"], None, cb["force"])
    U0 = np.array([0.01, -0.02, 0.015])
    s.set_state(U0, np.zeros(3), np.linalg.solve(M.toarray(), -K @ U0))

    def energy():
        return 0.5 * s.V @ (M @ s.V) + 0.5 * s.U @ (K @ s.U)
    e0 = energy()
    for _ in range(300):
        assert s.step(0.01) == D.SUCCESS
    assert abs(energy() - e0) <= 1e-12 * e0


@pytest.mark.parametrize("method", ["Newmark", "Bathe", "ImplicitEuler", "RK4"])
def test_nonlinear_variant_reduces_to_linear(method):
    M, C, K, F = _spring_mass(damp=0.1)
    a = _linear_solver(method, M, C, K, F, nonlinear=False)
    b = _linear_solver(method, M, C, K, F, nonlinear=True)
    for _ in range(20):
        assert a.step(0.01) == D.SUCCESS
        assert b.step(0.01) == D.SUCCESS
    for x, y in ((a.U, b.U), (a.V, b.V), (a.A, b.A)):
        np.testing.assert_allclose(y, x, rtol=1e-9, atol=1e-12 * np.abs(x).max())


def test_wilson_and_explicit_euler_formulas():
    """One step of the formulas as the reference writes them (gsDynamicWilson.hpp:52-56,
    gsDynamicExplicitEuler.hpp:81-82 and :117)."""
    M, C, K, F = _spring_mass(damp=0.2)
    dt = 0.01
    U0, V0 = np.array([0.001, 0.0, -0.002]), np.array([0.1, -0.05, 0.0])
    A0 = np.linalg.solve(M.toarray(), F - K @ U0 - C @ V0)
    # Wilson linear: a Newmark step with gamma*dt, A = (1 - 1/g) A0 + At/g, V = V0 + delta dt A, U = U0 + alpha dt^2 A
    g = 1.4
    nm = _linear_solver("Newmark", M, C, K, F)
    nm.set_state(U0, V0, A0)
    nm.step(g * dt)
    w = _linear_solver("Wilson", M, C, K, F)
    w.set_state(U0, V0, A0)
    w.step(dt)
    A = (1 - 1 / g) * A0 + nm.A / g
    np.testing.assert_allclose(w.A, A, rtol=1e-13)
    np.testing.assert_allclose(w.V, V0 + 0.5 * dt * A, rtol=1e-13)
    np.testing.assert_allclose(w.U, U0 + 0.25 * dt * dt * A, rtol=1e-13)
    # explicit Euler: linear uses F - K U - C V, the nonlinear variant -R - C V
    for nl, acc in ((False, F - K @ U0 - C @ V0), (True, -(F - K @ U0) - C @ V0)):
        e = _linear_solver("ExplicitEuler", M, C, K, F, nonlinear=nl)
        e.set_state(U0, V0, A0)
        e.step(dt)
        np.testing.assert_allclose(e.U, U0 + dt * V0, rtol=1e-14)
        np.testing.assert_allclose(e.V, V0 + dt * np.linalg.solve(M.toarray(), acc), rtol=1e-12)


def test_load_table_interpolates():
    f = D.load_table([0.0, 1.0, 3.0], [0.0, 2.0, 2.0])
    assert f(-1.0) == 0.0 and f(0.5) == 1.0 and f(2.0) == 2.0 and f(10.0) == 2.0
    assert D.load_table([], [])(5.0) == 1.0


def test_nonlinear_newmark_shell_plate(oracle_mod):
    """A clamped plate under a suddenly applied pressure that deflects it by about its
    thickness: the nonlinear Newmark steps converge, and the response differs from the linear
    one (membrane stiffening)."""
    from gsstructuralanalysis_gb300 import problems as P
    prob = P.flat_plate(m=4, p=2, E=1e7, t=0.01, rho=1.0, pressure=200.0)
    oa = oracle_mod.OracleAssembler(prob)
    res = {}
    for nl in (False, True):
        cb = D.shell_callbacks(oa, nl)
        s = D.Dynamic("Newmark", nl, cb["mass"], cb["damping"], cb["jacobian"], cb["residual"], cb["force"],
                      {"TolF": 1e-8, "TolU": 1e-8})
        n = oa.nfree
        s.set_state(np.zeros(n), np.zeros(n), np.zeros(n))
        for _ in range(4):
            assert s.step(2e-3) == D.SUCCESS
        res[nl] = s.U.copy()
        if nl:
            assert s.num_iterations >= 2
    w_lin, w_nl = np.abs(res[False]).max(), np.abs(res[True]).max()
    assert w_lin > 0.5 * prob.t
    assert w_nl < 0.99 * w_lin


def test_nonlinear_integrators_converge_to_one_trajectory(oracle_mod):
    """Nonlinear Newmark, Bathe and implicit Euler on a suddenly loaded plate that deflects by
    about its thickness: each approaches a fine-step Newmark reference as dt halves, at its
    order (second for Newmark and Bathe, first for implicit Euler; measured 2.05, 2.04, 1.08)."""
    from gsstructuralanalysis_gb300 import problems as P
    prob = P.flat_plate(m=4, p=2, E=1e7, t=0.01, rho=1.0, pressure=200.0)
    oa = oracle_mod.OracleAssembler(prob)
    cb = D.shell_callbacks(oa, True)
    n = oa.nfree
    T = 8e-3
    # consistent initial acceleration M a0 = F - Fint(0) = F: the orders hold from the first step
    import scipy.sparse.linalg as spla
    A0 = spla.spsolve(cb["mass"]().tocsc(), cb["force"](0.0))

    def run(method, nsteps):
        s = D.Dynamic(method, True, cb["mass"], cb["damping"], cb["jacobian"], cb["residual"], cb["force"],
                      {"TolF": 1e-10, "TolU": 1e-10})
        s.set_state(np.zeros(n), np.zeros(n), A0)
        for _ in range(nsteps):
            assert s.step(T / nsteps) == D.SUCCESS
        return s.U

    ref = run("Newmark", 1024)
    assert np.abs(ref).max() > 0.5 * prob.t
    # implicit Euler's damping of the plate's higher modes keeps it pre-asymptotic until ~T/128
    for method, order, steps in (("Newmark", 2, (32, 64)), ("Bathe", 2, (32, 64)), ("ImplicitEuler", 1, (128, 256))):
        e = [np.linalg.norm(run(method, k) - ref) for k in steps]
        rate = np.log2(e[0] / e[1])
        assert rate > order - 0.4, (method, e, rate)
