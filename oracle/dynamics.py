"""FP64 CPU restatement of the reference's time integrators (TEST INFRASTRUCTURE ONLY).

Only tests/ import this module, as the checker of the device-resident integrators.

Callbacks follow gsStructuralAnalysisTools/gsStructuralAnalysisTypes.h and the time-dependent
wrappers of gsDynamicSolvers/gsDynamicBase.h:60-170:
  mass()            -> M (sparse)
  damping(U, t)     -> C (sparse)
  jacobian(U, t)    -> K (sparse); the constant stiffness for the linear integrators
  residual(U, t)    -> R = Fext(t) - Fint(U)            (nonlinear integrators)
  force(t)          -> Fext(t)                          (linear integrators)

Restated integrators (``nonlinear`` selects the reference's ``_NL`` template flag):
  Newmark        gsDynamicSolvers/gsDynamicNewmark.hpp:30-145
  Bathe          gsDynamicSolvers/gsDynamicBathe.hpp:30-163 (stage 1 = Newmark with gamma*dt)
  Wilson         gsDynamicSolvers/gsDynamicWilson.hpp:30-82  (Newmark with gamma*dt)
  ExplicitEuler  gsDynamicSolvers/gsDynamicExplicitEuler.hpp:53-131
  ImplicitEuler  gsDynamicSolvers/gsDynamicImplicitEuler.hpp:24-163
  RK4            gsDynamicSolvers/gsDynamicRK4.hpp:18-150
Options and defaults: gsDynamicBase.hpp:19-33 and the defaultOptions() of each integrator.

ImplicitEuler: the reference solves the 2x2 block system [[I, -dt I], [dt K, M + dt C]] with
unpreconditioned GMRES; here the same system is solved exactly by eliminating the displacement
block, (M + dt C + dt^2 K) V = ..., which is the solution GMRES converges to.
The mass inverse of the explicit integrators (gsDynamicBase.h:291-304, a dense LU inverse) is
applied as a sparse LU solve with M.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse.linalg as spla

SUCCESS, NOT_CONVERGED = 0, 1

DEFAULTS = {"MaxIter": 100, "TolF": 1e-3, "TolU": 1e-6, "DT": 1e-2, "Quasi": 0, "QuasiIterations": 1}
METHOD_DEFAULTS = {
    "Newmark": {"alpha": 0.25, "delta": 0.5},
    "Bathe": {"alpha": 0.25, "delta": 0.5, "gamma": 0.5},
    "Wilson": {"alpha": 0.25, "delta": 0.5, "gamma": 1.4},
    "ExplicitEuler": {},
    "ImplicitEuler": {},
    "RK4": {},
}


def _solve(A, b):
    return spla.splu(A.tocsc()).solve(np.asarray(b, dtype=np.float64))


def _bad(x):
    n = np.linalg.norm(x)
    return bool(np.isinf(n) or np.isnan(n))


class Dynamic:
    """gsDynamicBase (gsDynamicBase.h:185-230: step(), time, U/V/A state) with one of the
    restated integrators."""

    def __init__(self, method, nonlinear, mass, damping, jacobian, residual=None, force=None, options=None):
        if method not in METHOD_DEFAULTS:
            raise ValueError(method)
        self.method, self.nl = method, bool(nonlinear)
        self.mass, self.damping, self.jacobian = mass, damping, jacobian
        self.residual, self.force = residual, force
        self.opts = dict(DEFAULTS)
        self.opts.update(METHOD_DEFAULTS[method])
        if options:
            self.opts.update(options)
        self.time = 0.0
        self.U = self.V = self.A = None
        self.num_iterations = 0
        self._minv = None

    def set_state(self, U, V, A):
        self.U, self.V, self.A = (np.array(v, dtype=np.float64) for v in (U, V, A))

    def step(self, dt=None):
        dt = self.opts["DT"] if dt is None else dt
        U, V, A = self.U.copy(), self.V.copy(), self.A.copy()
        st, U, V, A = getattr(self, "_" + self.method)(self.time, dt, U, V, A)
        self.U, self.V, self.A = U, V, A
        self.time += dt
        return st

    # -- helpers ------------------------------------------------------------------------------
    def _minv_apply(self, M, b):
        if self._minv is None:            # constant mass: factorised once (gsDynamicBase.h:291-304)
            self._minv = spla.splu(M.tocsc())
        return self._minv.solve(np.asarray(b, dtype=np.float64))

    def _quasi_refresh(self, it):
        o = self.opts
        return (not o["Quasi"]) or it == 0 or it % int(o["QuasiIterations"]) == 0

    # -- Newmark (gsDynamicNewmark.hpp:30-145) ------------------------------------------------------
    def _Newmark(self, t, dt, U, V, A):
        al, de = self.opts["alpha"], self.opts["delta"]
        Uold, Vold, Aold = U.copy(), V.copy(), A.copy()
        if not self.nl:
            M, F = self.mass(), self.force(t + dt)
            U = Uold + dt * Vold + Aold * (0.5 - al) * dt * dt
            V = Vold + Aold * (1 - de) * dt
            C, K = self.damping(U, t + dt), self.jacobian(U, t + dt)
            lhs = M + de * dt * C + dt * dt * al * K
            rhs = F - K @ U - C @ V
            A = _solve(lhs, rhs)
            V = V + A * de * dt
            U = U + A * al * dt * dt
            self.num_iterations = 1
            return (NOT_CONVERGED if _bad(U) else SUCCESS), U, V, A
        A = np.zeros_like(A)
        U = Uold + dt * Vold + Aold * (0.5 - al) * dt * dt + al * dt * dt * A
        V = Vold + Aold * (1 - de) * dt + de * dt * A
        M = self.mass()
        C = self.damping(U, t + dt)
        R = self.residual(U, t + dt)
        rhs = R - C @ V - M @ A
        tolU, tolF = self.opts["TolU"], self.opts["TolF"]
        r0 = np.linalg.norm(rhs)
        r0 = r0 if r0 != 0 else 1.0
        K = None
        for it in range(int(self.opts["MaxIter"])):
            if self._quasi_refresh(it):
                C, K = self.damping(U, t + dt), self.jacobian(U, t + dt)
            lhs = M + de * dt * C + dt * dt * al * K
            dA = _solve(lhs, rhs)
            A = A + dA
            V = V + dA * de * dt
            U = U + dA * al * dt * dt
            An, dAn = np.linalg.norm(A), np.linalg.norm(dA)
            upd = dAn / An if An != 0 else dAn
            R = self.residual(U, t + dt)
            rhs = R - C @ V - M @ A
            res = np.linalg.norm(rhs) / r0
            self.num_iterations = it + 1
            if upd < tolU and res < tolF:
                return SUCCESS, U, V, A
        return NOT_CONVERGED, U, V, A

    # -- Bathe (gsDynamicBathe.hpp:30-163) -------------------------------------------------------
    def _Bathe(self, t, dt, U, V, A):
        g = self.opts["gamma"]
        Uold, Vold = U.copy(), V.copy()
        _, Us, Vs, As = self._Newmark(t, g * dt, U.copy(), V.copy(), A.copy())
        c1 = (1 - g) / (g * dt)
        c2 = -1.0 / ((1 - g) * g * dt)
        c3 = (2 - g) / ((1 - g) * dt)
        M = self.mass()
        if not self.nl:
            F = self.force(t + dt)
            C, K = self.damping(Uold, t + dt), self.jacobian(Uold, t + dt)
            lhs = K + c3 * c3 * M + c3 * C
            rhs = F - M @ (c1 * Vold + c2 * Vs + c1 * c3 * Uold + c3 * c2 * Us) - C @ (c2 * Us + c1 * Uold)
            U = _solve(lhs, rhs)
            V = c1 * Uold + c2 * Us + c3 * U
            A = c1 * Vold + c2 * Vs + c3 * V
            self.num_iterations = 1
            return (NOT_CONVERGED if _bad(U) else SUCCESS), U, V, A
        C = self.damping(Uold, t + dt)
        R = self.residual(Uold, t + dt)          # evaluated before U is reset to the stage-1 state
        U, V, A = Us.copy(), Vs.copy(), As.copy()

        def rhs_of(R, C, U):
            return R - M @ (c1 * Vold + c2 * Vs + c1 * c3 * Uold + c3 * c2 * Us + c3 * c3 * U) \
                - C @ (c1 * Uold + c2 * Us + c3 * U)
        rhs = rhs_of(R, C, U)
        tolU, tolF = self.opts["TolU"], self.opts["TolF"]
        r0 = np.linalg.norm(rhs)
        r0 = r0 if r0 != 0 else 1.0
        K = None
        for it in range(int(self.opts["MaxIter"])):
            if self._quasi_refresh(it):
                C, K = self.damping(U, t + dt), self.jacobian(U, t + dt)
            lhs = K + c3 * c3 * M + c3 * C
            dU = _solve(lhs, rhs)
            U = U + dU
            R = self.residual(U, t + dt)
            rhs = rhs_of(R, C, U)
            res = np.linalg.norm(rhs) / r0
            upd = np.linalg.norm(dU) / np.linalg.norm(U)
            self.num_iterations = it + 1
            if upd < tolU and res < tolF:
                V = c1 * Uold + c2 * Us + c3 * U
                A = c1 * Vold + c2 * Vs + c3 * V
                return SUCCESS, U, V, A
        V = c1 * Uold + c2 * Us + c3 * U
        A = c1 * Vold + c2 * Vs + c3 * V
        return NOT_CONVERGED, U, V, A

    # -- Wilson (gsDynamicWilson.hpp:30-82) ------------------------------------------------------
    def _Wilson(self, t, dt, U, V, A):
        al, de, g = self.opts["alpha"], self.opts["delta"], self.opts["gamma"]
        Uold, Vold, Aold = U.copy(), V.copy(), A.copy()
        _, _, _, At = self._Newmark(t, g * dt, U.copy(), V.copy(), A.copy())
        A = (1 - 1 / g) * Aold + 1 / g * At
        if not self.nl:
            V = Vold + A * de * dt
            U = Uold + A * al * dt * dt
        else:
            U = Uold + dt * Vold + Aold * (0.5 - al) * dt * dt + al * dt * dt * A
            V = Vold + Aold * (1 - de) * dt + de * dt * A
        return SUCCESS, U, V, A

    # -- explicit Euler (gsDynamicExplicitEuler.hpp:53-131) ---------------------------------------
    def _ExplicitEuler(self, t, dt, U, V, A):
        Uold, Vold = U.copy(), V.copy()
        M = self.mass()
        C = self.damping(Uold, t)
        if not self.nl:
            F, K = self.force(t), self.jacobian(Uold, t)
            Vn = Vold + dt * self._minv_apply(M, F - K @ Uold - C @ Vold)
        else:
            R = self.residual(Uold, t)
            Vn = Vold + dt * self._minv_apply(M, -R - C @ Vold)   # the reference's sign (hpp:117)
        Un = Uold + dt * Vold
        self.num_iterations = 1
        bad = _bad(np.concatenate([Un, Vn]))
        return (NOT_CONVERGED if bad else SUCCESS), Un, Vn, A

    # -- implicit Euler (gsDynamicImplicitEuler.hpp:24-163) ---------------------------------------
    def _ImplicitEuler(self, t, dt, U, V, A):
        Uold, Vold = U.copy(), V.copy()
        M = self.mass()
        if not self.nl:
            F = self.force(t + dt)
            C, K = self.damping(Uold, t + dt), self.jacobian(Uold, t)
            Vn = _solve(M + dt * C + dt * dt * K, dt * F + M @ Vold - dt * (K @ Uold))
            self.num_iterations = 1
            return SUCCESS, Uold + dt * Vn, Vn, A
        C = self.damping(U, t + dt)
        R = self.residual(U, t + dt)
        r_top, r_bot = -dt * V, dt * (C @ V) - dt * R
        r0 = np.sqrt(np.dot(r_top, r_top) + np.dot(r_bot, r_bot))
        r0 = r0 if r0 != 0 else 1.0
        tolU, tolF = self.opts["TolU"], self.opts["TolF"]
        K = None
        for it in range(int(self.opts["MaxIter"])):
            if self._quasi_refresh(it):
                C, K = self.damping(U, t + dt), self.jacobian(U, t + dt)
            r_top = U - Uold - dt * V
            r_bot = M @ (V - Vold) + dt * (C @ V) - dt * R
            # [[I, -dt I], [dt K, M + dt C]] d = -r, eliminated for the velocity block
            dV = _solve(M + dt * C + dt * dt * K, -r_bot + dt * (K @ r_top))
            dU = dt * dV - r_top
            U, V = U + dU, V + dV
            sn = np.sqrt(np.dot(U, U) + np.dot(V, V))
            dn = np.sqrt(np.dot(dU, dU) + np.dot(dV, dV))
            upd = dn / sn if sn != 0 else dn
            R = self.residual(U, t)                       # the reference evaluates it at t (hpp:142)
            res = np.sqrt(np.dot(r_top, r_top) + np.dot(r_bot, r_bot)) / r0
            self.num_iterations = it + 1
            if upd < tolU and res < tolF:
                return SUCCESS, U, V, A
        return NOT_CONVERGED, U, V, A

    # -- RK4 (gsDynamicRK4.hpp:18-150) ----------------------------------------------------------
    def _RK4(self, t, dt, U, V, A):
        Uold, Vold = U.copy(), V.copy()
        M = self.mass()
        C = self.damping(Uold, t)
        if not self.nl:
            K = self.jacobian(Uold, t)

            def acc(Ux, Vx, tx):
                return self._minv_apply(M, self.force(tx) - K @ Ux - C @ Vx)
        else:
            def acc(Ux, Vx, tx):
                return self._minv_apply(M, self.residual(Ux, tx) - C @ Vx)
        k1u, k1v = Vold, acc(Uold, Vold, t)
        Ut, Vt = Uold + dt / 2 * k1u, Vold + dt / 2 * k1v
        k2u, k2v = Vt, acc(Ut, Vt, t + dt / 2)
        Ut, Vt = Uold + dt / 2 * k2u, Vold + dt / 2 * k2v
        k3u, k3v = Vt, acc(Ut, Vt, t + dt / 2)
        Ut, Vt = Uold + dt * k3u, Vold + dt * k3v
        k4u, k4v = Vt, acc(Ut, Vt, t + dt)
        Un = Uold + 1.0 / 6 * dt * (k1u + 2 * k2u + 2 * k3u + k4u)
        Vn = Vold + 1.0 / 6 * dt * (k1v + 2 * k2v + 2 * k3v + k4v)
        self.num_iterations = 1
        bad = _bad(np.concatenate([Un, Vn]))
        return (NOT_CONVERGED if bad else SUCCESS), Un, Vn, A


def load_table(ts, fs):
    """Piecewise-linear load factor f(t) through (ts, fs), constant beyond the ends; no points = 1."""
    ts, fs = np.asarray(ts, dtype=np.float64), np.asarray(fs, dtype=np.float64)
    if len(ts) == 0:
        return lambda t: 1.0
    return lambda t: float(np.interp(t, ts, fs))


def shell_callbacks(assembler, nonlinear, damping_mass=0.0, damping_stiffness=0.0, load=None):
    """Callbacks of a KL-shell problem from the FP64 oracle assembler: mass M, Rayleigh damping
    C = cM M + cK K_L, the tangent K(U) (nonlinear) or K_L (linear), R = f(t) F - Fint(U) and
    Fext(t) = f(t) F."""
    f = load if load is not None else (lambda t: 1.0)
    M = assembler.mass()
    KL = assembler.linear()
    F = assembler.force()
    C = damping_mass * M + damping_stiffness * KL
    cb = {
        "mass": lambda: M,
        "damping": lambda U, t: C,
        "force": lambda t: f(t) * F,
        "residual": lambda U, t: f(t) * F - assembler.fint(U),
    }
    cb["jacobian"] = (lambda U, t: assembler.jacobian(U)) if nonlinear else (lambda U, t: KL)
    return cb
