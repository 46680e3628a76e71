"""FP64 CPU oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of bench.py
import this module, and only as the checker or the timed CPU comparator.  The
shipped library never imports it.

Parts
  * ``OracleAssembler``: ctypes front-end of kl_oracle.cpp (FP64 KL-shell
    K(u), Fint(u), M, F), Dirichlet elimination in free-dof order.
  * Solver logic restated from the reference, line for line in behaviour:
      - ``StaticNewton``   gsStaticSolvers/gsStaticNewton.hpp:142-193 (_solveNonlinear),
                           :274-316 (_start), :101-112 (_solveLinear); options gsStaticBase.h:66-75
      - ``ALMCrisfield``   gsALMSolvers/gsALMCrisfield.hpp:66-206 (iteration, predictor,
                           predictorGuess, iterationFinish), :213-427 (computeLambdas*, MU, DOT)
      - ``ALMRiks``        gsALMSolvers/gsALMRiks.hpp:40-170
      - ``ALMLoadControl`` gsALMSolvers/gsALMLoadControl.hpp:49-108
      - step driver        gsALMSolvers/gsALMBase.hpp:354-416 (_step), :151-183 (residual norms)
  * Eigen problems with scipy ARPACK in place of Spectra (Spectra is not in the
    reference tree): buckling mode = scipy ``mode='buckling'`` (Spectra
    GEigsMode::Buckling), modal = shift-invert normal mode (GEigsMode::ShiftInvert),
    following gsEigenProblemBase.hpp:152-215 and gsBucklingSolver.h:127-149.
  * The sparse factorisation behind ``Solver=SimplicialLDLT`` (Eigen, not in the
    reference tree) is stood in for by scipy SuperLU in FP64.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "_build", "libkl_oracle.so")
_lib = None

_dp = ctypes.POINTER(ctypes.c_double)


def build_oracle(force: bool = False) -> str:
    if force or not os.path.exists(_LIB) or os.path.getmtime(_LIB) < os.path.getmtime(os.path.join(_HERE, "kl_oracle.cpp")):
        subprocess.check_call(["make", "-s", "-C", _HERE])
    return _LIB


def lib():
    global _lib
    if _lib is None:
        build_oracle()
        L = ctypes.CDLL(_LIB)
        L.klo_full_nnz.restype = ctypes.c_int64
        L.klo_full_nnz.argtypes = [ctypes.c_int] * 3
        L.klo_full_pattern.argtypes = [ctypes.c_int] * 3 + [ctypes.c_void_p, ctypes.c_void_p]
        L.klo_assemble.argtypes = ([ctypes.c_int] * 3 + [ctypes.c_void_p] * 3 + [ctypes.c_double] * 3 +
                                   [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                    ctypes.c_void_p])
        L.klo_mass.argtypes = ([ctypes.c_int] * 3 + [ctypes.c_void_p] * 3 + [ctypes.c_double] * 2 +
                               [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p])
        L.klo_force.argtypes = ([ctypes.c_int] * 3 + [ctypes.c_void_p] * 3 + [ctypes.c_int, ctypes.c_void_p,
                                ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                ctypes.c_void_p])
        L.klo_basis.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_double, ctypes.c_void_p]
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def basis(p: int, knots: np.ndarray, u: float) -> tuple[int, np.ndarray]:
    knots = np.ascontiguousarray(knots, dtype=np.float64)
    out = np.zeros(3 * (p + 1))
    span = lib().klo_basis(p, len(knots) - p - 1, _ptr(knots), u, _ptr(out))
    return span, out.reshape(3, p + 1)


def constraint_matrix(fixed, ties):
    """u = T q for fixed dofs (zero) and tied dofs (``ties`` rows [dof, equal to dof]): each dof
    maps to the independent dof at the end of its chain of ties, or to nothing when the chain
    reaches a fixed dof; the independent dofs are numbered in full-layout order."""
    n = len(fixed)
    master = np.arange(n)
    ties = np.asarray(ties, dtype=np.int64).reshape(-1, 2)
    master[ties[:, 0]] = ties[:, 1]
    master[np.asarray(fixed, dtype=bool)] = -1
    while True:
        m = master >= 0
        nxt = master.copy()
        nxt[m] = master[master[m]]
        if np.array_equal(nxt, master):
            break
        master = nxt
    keep = np.unique(master[master >= 0])
    col = np.full(n, -1)
    col[keep] = np.arange(len(keep))
    rows = np.flatnonzero(master >= 0)
    return sp.csr_matrix((np.ones(len(rows)), (rows, col[master[rows]])), shape=(n, len(keep)))


class OracleAssembler:
    """FP64 assembly of one patch problem; matrices/vectors in free-dof order."""

    def __init__(self, prob, nthreads: int = 0):
        self.prob = prob
        self.nthreads = nthreads
        P = prob
        self._U1 = np.ascontiguousarray(P.knots1, dtype=np.float64)
        self._U2 = np.ascontiguousarray(P.knots2, dtype=np.float64)
        self._X = np.ascontiguousarray(P.ctrl, dtype=np.float64)
        w = getattr(P, "weights", None)
        self._W = None if w is None else np.ascontiguousarray(w, dtype=np.float64)   # NURBS weights
        L = lib()
        nnz = L.klo_full_nnz(P.p, P.n1, P.n2)
        self.rowptr = np.zeros(3 * P.ncp + 1, dtype=np.int64)
        self.cols = np.zeros(nnz, dtype=np.int32)
        L.klo_full_pattern(P.p, P.n1, P.n2, _ptr(self.rowptr), _ptr(self.cols))
        self.free = P.free_index()
        self.nfree = len(self.free)
        # tied dofs (clamped symmetry sides): u = T q over the independent dofs instead of the
        # selection of the free ones
        ties = getattr(P, "ties", None)
        self.T = None if ties is None or not len(ties) else constraint_matrix(P.fixed, ties)
        if self.T is not None:
            self.nfree = self.T.shape[1]
        self._F = None

    def _wptr(self):
        return _ptr(self._W) if self._W is not None else None

    # -- full-space pieces ---------------------------------------------------------------
    def full_tangent_and_fint(self, ufull: np.ndarray, want_K: bool = True):
        P = self.prob
        u = np.ascontiguousarray(ufull, dtype=np.float64)
        vals = np.zeros(len(self.cols)) if want_K else None
        fint = np.zeros(3 * P.ncp)
        rc = lib().klo_assemble(P.p, P.n1, P.n2, _ptr(self._U1), _ptr(self._U2), _ptr(self._X), P.E, P.nu, P.t,
                                P.nq, _ptr(u), _ptr(vals) if want_K else None, _ptr(fint), self.nthreads,
                                self._wptr())
        if rc != 0:
            raise RuntimeError("oracle assembly failed")
        K = None
        if want_K:
            K = sp.csr_matrix((vals, self.cols, self.rowptr), shape=(3 * P.ncp, 3 * P.ncp))
        return K, fint

    def full_force(self) -> np.ndarray:
        P = self.prob
        F = np.zeros(3 * P.ncp)
        qs = np.ascontiguousarray(P.surface_load, dtype=np.float64)
        pl = np.ascontiguousarray(P.point_loads, dtype=np.float64).reshape(-1, 5)
        ed = np.ascontiguousarray(P.edge_loads, dtype=np.float64).reshape(-1, 4)
        lib().klo_force(P.p, P.n1, P.n2, _ptr(self._U1), _ptr(self._U2), _ptr(self._X), P.nq, _ptr(qs),
                        len(pl), _ptr(pl), len(ed), _ptr(ed), _ptr(F), self._wptr())
        return F

    def full_mass(self):
        P = self.prob
        vals = np.zeros(len(self.cols))
        lib().klo_mass(P.p, P.n1, P.n2, _ptr(self._U1), _ptr(self._U2), _ptr(self._X), P.rho, P.t, P.nq, _ptr(vals),
                       self._wptr())
        return sp.csr_matrix((vals, self.cols, self.rowptr), shape=(3 * P.ncp, 3 * P.ncp))

    # -- free-dof (eliminated) versions, the objects the reference's callbacks return -----
    def to_full(self, x: np.ndarray) -> np.ndarray:
        if self.T is not None:
            return self.T @ x
        u = np.zeros(3 * self.prob.ncp)
        u[self.free] = x
        return u

    def restrict(self, A):
        if self.T is not None:
            return (self.T.T @ A @ self.T).tocsr()
        return A[self.free][:, self.free].tocsr()

    def restrict_vector(self, v: np.ndarray) -> np.ndarray:
        return self.T.T @ v if self.T is not None else v[self.free]

    def force(self) -> np.ndarray:
        if self._F is None:
            self._F = self.restrict_vector(self.full_force())
        return self._F.copy()

    def jacobian(self, x: np.ndarray):
        K, _ = self.full_tangent_and_fint(self.to_full(x), True)
        return self.restrict(K)

    def fint(self, x: np.ndarray) -> np.ndarray:
        _, f = self.full_tangent_and_fint(self.to_full(x), False)
        return self.restrict_vector(f)

    def residual(self, x: np.ndarray) -> np.ndarray:
        """Residual_t convention: R = Fext - Fint (tutorials/nonlinear_shell_static.cpp:128-135)."""
        return self.force() - self.fint(x)

    def al_residual(self, x: np.ndarray, lam: float) -> np.ndarray:
        """ALResidual_t convention: R = Fint - lam*F (tutorials/nonlinear_shell_arcLength.cpp:135-142)."""
        return self.fint(x) - lam * self.force()

    def linear(self):
        return self.jacobian(np.zeros(self.nfree))

    def mass(self):
        return self.restrict(self.full_mass())


# ---------------------------------------------------------------------------------------------
# Sparse "SimplicialLDLT" stand-in
# ---------------------------------------------------------------------------------------------
class SuperLUSolver:
    def __init__(self):
        self._lu = None

    def compute(self, A):
        try:
            self._lu = spla.splu(sp.csc_matrix(A), permc_spec="MMD_AT_PLUS_A", diag_pivot_thresh=0.0,
                                 options=dict(SymmetricMode=True))
        except RuntimeError as exc:  # singular
            raise SolverError(str(exc)) from exc

    def solve(self, b):
        return self._lu.solve(np.asarray(b, dtype=np.float64))


class SolverError(Exception):
    pass


class NotConverged(Exception):
    pass


class AssemblyError(Exception):
    pass


# gsStatus (gsStructuralAnalysisTools/gsStructuralAnalysisTypes.h:22-30)
SUCCESS, NOT_CONVERGED, ASSEMBLY_ERROR, SOLVER_ERROR, NOT_STARTED, OTHER_ERROR = range(6)


def _status_of(fn):
    try:
        fn()
        return SUCCESS
    except NotConverged:
        return NOT_CONVERGED
    except AssemblyError:
        return ASSEMBLY_ERROR
    except SolverError:
        return SOLVER_ERROR


class StaticNewton:
    """gsStaticNewton restated (gsStaticNewton.hpp:101-193, 274-316)."""

    def __init__(self, K_lin, F, jacobian=None, residual=None, options=None):
        self.K_lin, self.F = K_lin, np.asarray(F, dtype=np.float64)
        self.jac, self.res = jacobian, residual
        self.opts = dict(tol=1e-6, tolF=-1.0, tolU=-1.0, maxIt=25, verbose=0, Relaxation=1.0)
        if options:
            self.opts.update(options)
        n = len(self.F)
        # the state after the constructor: gsStaticNewton::_init calls its reset(), which sets
        # the dofs from the force vector and sizes DeltaU to them (gsStaticNewton.hpp:243-250,
        # gsStaticBase.h:136-144), so the linear head start of gsStaticNewton.hpp:148-153 (taken
        # only while DeltaU has no rows) never runs
        self.U = np.zeros(n)
        self.DeltaU = np.zeros(n)
        self.deltaU = np.zeros(n)
        self.headstart = False
        self.num_iterations = 0
        self.history = []
        self.solver = SuperLUSolver()

    def _get(self):
        o = self.opts
        self.tolF = o["tolF"] if o["tolF"] != -1 else o["tol"]
        self.tolU = o["tolU"] if o["tolU"] != -1 else o["tol"]
        self.maxIt = int(o["maxIt"])
        self.relax = float(o["Relaxation"])

    def _residual(self, U):
        r = self.res(U)
        if r is None:
            raise AssemblyError()
        return r

    def solve_linear(self):
        self._get()
        self.solver.compute(self.K_lin)
        self.U = self.solver.solve(self.F)
        return self.U

    def _solve_nonlinear(self):
        self._get()
        if len(self.DeltaU) == 0:
            self.deltaU = self.DeltaU = self.solve_linear().copy()
            self.U = np.zeros_like(self.DeltaU)
            self.headstart = True
        # _start (hpp:274-316)
        if not self.headstart:
            self.DeltaU = np.zeros_like(self.U)
            self.R = self._residual(self.U)
            r = np.linalg.norm(self.R)
            self.residual = r if r != 0 else 1.0
            self.residualIni = self.residualOld = self.residual
        else:
            self.R = self._residual(self.U + self.DeltaU)
            r = np.linalg.norm(self.R)
            self.residual = r if r != 0 else 1.0
            self.residualOld = self.residual
            r0 = np.linalg.norm(self._residual(self.U))
            self.residualIni = r0 if r0 != 0 else 1.0
            self.headstart = False
        self.deltaU = np.zeros_like(self.U)
        for it in range(self.maxIt):
            self.num_iterations = it
            K = self.jac(self.U + self.DeltaU)
            if K is None:
                raise AssemblyError()
            self.solver.compute(K)
            self.deltaU = self.solver.solve(self.R)
            self.DeltaU = self.DeltaU + self.relax * self.deltaU
            self.R = self._residual(self.U + self.DeltaU)
            self.residual = np.linalg.norm(self.R)
            self.history.append((self.residual / self.residualIni,
                                 self.relax * np.linalg.norm(self.deltaU) / np.linalg.norm(self.DeltaU)))
            self.residualOld = self.residual
            if (self.relax * np.linalg.norm(self.deltaU) / np.linalg.norm(self.DeltaU) < self.tolU and
                    self.residual / self.residualIni < self.tolF):
                self.U = self.U + self.DeltaU
                break
            elif it + 1 == self.maxIt:
                self.U = self.U + self.DeltaU
                raise NotConverged()
        return self.U

    def solve(self):
        if self.jac is None or self.res is None:
            return _status_of(self.solve_linear)
        return _status_of(self._solve_nonlinear)

    def set_displacement(self, U):
        self.U = np.asarray(U, dtype=np.float64).copy()

    def set_update(self, DU):
        self.headstart = True
        self.DeltaU = np.asarray(DU, dtype=np.float64).copy()


class _ALMBase:
    """Step driver and residual norms of gsALMBase (gsALMBase.hpp:22-103, 136-223, 354-416)."""

    def __init__(self, jacobian, al_residual, F, options=None):
        self.jacobian, self.res = jacobian, al_residual
        self.F = np.asarray(F, dtype=np.float64)
        self.opts = dict(MaxIter=100, Tol=1e-6, TolF=1e-3, TolU=1e-6, Length=1e-2, AdaptiveLength=False,
                         AdaptiveIterations=10, Quasi=False, QuasiIterations=-1, BifurcationMethod=1,
                         Relaxation=1.0, Scaling=-1.0, AngleMethod=0, Perturbation=1e3, SingularPointFailure=1,
                         SingularPointTestTol=1e-6, SingularPointTestIt=5, SingularPointComputeTolE=1e-10,
                         SingularPointComputeTolB=0.0)
        if options:
            self.opts.update(options)
        self.solver = SuperLUSolver()
        self.apply_options()
        n = len(self.F)
        self.numDof = n
        self.U = np.zeros(n); self.L = 0.0
        self.DeltaU = np.zeros(n); self.DeltaL = 0.0
        self.deltaU = np.zeros(n); self.deltaL = 0.0
        self.deltaUt = np.zeros(n); self.deltaUbar = np.zeros(n)
        self.DeltaUold = np.zeros(n); self.DeltaLold = 0.0
        self.Uprev = np.zeros(n); self.Lprev = 0.0
        self.Uguess = None; self.Lguess = 0.0
        self.num_iterations = 0
        self.converged = False
        self.counts = dict(jac=0, res=0, solve=0)
        self.stabilityVec = np.zeros(0)
        self.indicator = 0.0
        self.negatives = 0
        self.stability = -1
        self.stabilityPrev = -1

    def initialize(self, stability=True):
        """gsALMBase::initialize / init (gsALMBase.h:110-115, gsALMBase.hpp:95-103)."""
        if stability:
            self.compute_stability(jacobian=True)

    def compute_stability(self, jacobian=True, shift=-1e2):
        """gsALMBase::_computeStability (gsALMBase.hpp:547-615).  Determinant (0): the reference
        takes D of the LDL^T; its count of negative entries is the inertia of K (Sylvester's law),
        which the oracle reads from the dense eigenvalues (min D itself depends on the elimination
        order and is not restated).  Eigenvalue (1): shift-invert Lanczos with
        nev = min(floor(n/5), 10), ncv = 5 nev, selection LargestAlge of 1/(lambda - shift),
        values ascending; without enough dofs for that, all eigenvalues (the dense branch)."""
        if jacobian:
            K = self.jacobian(self.U)
            self.counts["jac"] += 1
            self.solver.compute(K)
            self.jacMat = K
        bm = int(self.opts["BifurcationMethod"])
        K = self.jacMat
        if bm == 0:
            self.stabilityVec = np.linalg.eigvalsh(K.toarray())
        elif bm == 1:
            number = min(int(np.floor(K.shape[0] / 5.0)), 10)
            if number < 1 or 5 * number >= K.shape[0]:
                self.stabilityVec = np.linalg.eigvalsh(K.toarray())[:max(number, 1)]
            else:
                import scipy.sparse.linalg as _spla
                w = _spla.eigsh(K.tocsc(), k=number, sigma=shift, which="LA", ncv=5 * number, tol=1e-12,
                                v0=np.ones(K.shape[0]), return_eigenvectors=False)
                self.stabilityVec = np.sort(w)
        else:
            self.stabilityVec = np.zeros(K.shape[0])
        self.negatives = int(np.sum(self.stabilityVec < 0))
        self.indicator = float(np.min(self.stabilityVec))
        self.stability = 1 if self.indicator < 0 else -1

    def stability_change(self):
        return self.stability * self.stabilityPrev < 0

    # ---- singular points (gsALMBase.hpp:421-512, 628-728, 839-852) ---------------------------
    def is_bifurcation(self, jacobian=False):
        """_testSingularPoint: a few inverse iterations from the normalised ones vector; the point is
        a bifurcation when the approximate null vector is orthogonal to the load."""
        if jacobian:
            K = self.jacobian(self.U)
            self.counts["jac"] += 1
            self.solver.compute(K)
            self.jacMat = K
        n = self.numDof
        V = np.ones(n) / np.sqrt(n)
        self.solver.compute(self.jacMat)
        for _ in range(int(self.opts["SingularPointTestIt"])):
            V = self.solver.solve(V)
            V = V / np.linalg.norm(V)
        self.V = V
        return abs(float(V @ self.F)) < float(self.opts["SingularPointTestTol"])

    def compute_singular_point(self, U, L, switch_branch=False, jacobian=False, test_point=True):
        return _status_of(lambda: self._compute_singular_point(U, L, switch_branch, jacobian, test_point))

    def _compute_singular_point(self, U, L, switch_branch, jacobian, test_point):
        test = self.is_bifurcation(jacobian) if test_point else True
        self.U = np.asarray(U, dtype=np.float64).copy()
        self.L = float(L)
        if test:
            if float(self.opts["SingularPointComputeTolB"]) != 0:
                self._bisection_solve(self.U, self.L, float(self.opts["SingularPointComputeTolB"]))
            converged = self._extended_system_solve(self.U, self.L, float(self.opts["SingularPointComputeTolE"]))
            if switch_branch and (converged or int(self.opts["SingularPointFailure"]) == 1):
                self.switch_branch()
            self.stability = self.stabilityPrev

    def _extended_system_solve(self, U, L, tol):
        self.U, self.L = U.copy(), L
        K = self.jacobian(self.U)
        self.solver.compute(K)
        self.jacMat = K
        n = self.numDof
        self.DeltaV = np.zeros(n); self.DeltaU = np.zeros(n); self.DeltaL = 0.0
        self.deltaV = np.zeros(n); self.deltaU = np.zeros(n); self.deltaL = 0.0
        for it in range(self.maxIt):
            self.num_iterations = it
            self._extended_system_iteration()
            self.DeltaU = self.DeltaU + self.deltaU
            self.DeltaL += self.deltaL
            self.DeltaV = self.DeltaV + self.deltaV
            K = self.jacobian(self.U + self.DeltaU)
            self.solver.compute(K)
            self.jacMat = K
            self.residueKTPhi = float(np.linalg.norm(K @ (self.V + self.DeltaV)))
            self.resVec = self.res(self.U + self.DeltaU, self.L + self.DeltaL)
            self.compute_residual_norms()
            if self.residueKTPhi < tol:
                self.U = self.U + self.DeltaU
                self.L += self.DeltaL
                return True
            if it == self.maxIt - 1:
                if int(self.opts["SingularPointFailure"]) == 1:
                    self.U = self.U + self.DeltaU
                    self.L += self.DeltaL
                else:
                    self.DeltaV = np.zeros(n); self.DeltaU = np.zeros(n); self.DeltaL = 0.0
                    self.deltaV = np.zeros(n); self.deltaU = np.zeros(n); self.deltaL = 0.0
                return False
        return True

    def _extended_system_iteration(self):
        x = self.U + self.DeltaU
        R = self.res(x, self.L + self.DeltaL)
        K = self.jacobian(x)
        self.solver.compute(K)
        ut = self.solver.solve(self.F)
        ubar = self.solver.solve(-R)
        eps = 1e-8
        W = self.V + self.DeltaV
        Keps = self.jacobian(x + eps * W)
        h1 = (Keps @ ut) / eps - self.F / eps
        h2 = K @ W + (Keps @ ubar + R) / eps
        Vt = self.solver.solve(-h1)
        Vbar = self.solver.solve(-h2)
        nW = float(np.linalg.norm(W))
        Wn = W / nW
        self.deltaL = -(float(Wn @ Vbar) + nW - 1.0) / float(Wn @ Vt)
        self.deltaU = self.deltaL * ut + ubar
        self.deltaV = self.deltaL * Vt + Vbar

    def _bisection_solve(self, U, L, tol):
        """_bisectionSolve (gsALMBase.hpp:758-837): arc-length steps from the last point with the same
        number of negative pivots, halving the length when the count changes, until the indicator
        drops below tol of its start value; then the null vector by inverse iteration."""
        self.U, self.L = U.copy(), L
        U_old, L_old = self.U.copy(), self.L
        dL = self.arcLength
        adaptive = self.adaptive
        self.adaptive = False
        converged = False
        self.compute_stability(jacobian=True)
        reference = self.indicator
        self.compute_stability(jacobian=False)
        fa = self.negatives
        for _ in range(1, self.maxIt):
            self.U, self.L = U_old.copy(), L_old
            status = self.step()
            self.compute_stability(jacobian=True)
            fb = self.negatives
            if fa == fb and status == 0:
                U_old, L_old = self.U.copy(), self.L
                fa = fb
            else:
                self.arcLength = self.arcLength / 2.0
            self.compute_stability(jacobian=False)
            if abs(self.indicator / reference) < tol:
                converged = True
                break
        self.arcLength = dL
        self.adaptive = adaptive
        n = self.numDof
        self.V = np.ones(n) / np.sqrt(n)
        Vold = np.zeros(n)
        for _ in range(5):
            self.solver.compute(self.jacMat)
            self.V = self.solver.solve(self.V)
            self.V = self.V / np.linalg.norm(self.V)
            if np.linalg.norm(self.V - Vold) < float(self.opts["Tol"]):
                converged = True
                break
            Vold = self.V.copy()
        return converged

    def switch_branch(self):
        """switchBranch (gsALMBase.hpp:839-852): perturb U along the null vector by |V| / tau."""
        self.V = self.V / np.linalg.norm(self.V)
        xi = float(np.linalg.norm(self.V)) / float(self.opts["Perturbation"])
        self.DeltaU = xi * self.V
        self.U = self.U + self.DeltaU
        self.DeltaLold = 0.0
        self.DeltaUold = np.zeros(self.numDof)

    def apply_options(self):
        o = self.opts
        self.maxIt = int(o["MaxIter"]); self.tolF = float(o["TolF"]); self.tolU = float(o["TolU"])
        self.arcLength = self.arcLength_prev = self.arcLength_ori = float(o["Length"])
        self.adaptive = bool(o["AdaptiveLength"]); self.desiredIt = int(o["AdaptiveIterations"])
        self.relax = float(o["Relaxation"])

    def set_length(self, length):
        self.opts["Length"] = length
        self.arcLength = self.arcLength_prev = self.arcLength_ori = float(length)

    def set_solution(self, U, L):
        self.U = np.asarray(U, dtype=np.float64).copy(); self.L = float(L)

    def set_initial_guess(self, Ug, Lg):
        self.Uguess = np.asarray(Ug, dtype=np.float64).copy(); self.Lguess = float(Lg)

    def set_previous(self, Uprev, Lprev):
        """gsALMBase::setPrevious (gsALMBase.h:185-191)."""
        self.Uprev = np.asarray(Uprev, dtype=np.float64).copy(); self.Lprev = float(Lprev)
        self.DeltaUold = self.U - self.Uprev
        self.DeltaLold = self.L - self.Lprev

    def distance(self, DU, DL):
        raise NotImplementedError("gsALMBase::distance has no implementation (gsALMBase.h:211-214)")

    def reduce_length(self, fac):
        self.arcLength *= fac
        return self.arcLength

    def compute_length(self):
        """gsALMBase::computeLength (gsALMBase.hpp:105-116): the factor is the quotient of two
        index_t, an integer division, clamped to [0.5, 2]."""
        fac = float(self.desiredIt // self.num_iterations)
        fac = min(max(fac, 0.5), 2.0)
        self.arcLength_prev = self.arcLength
        self.arcLength = self.arcLength * fac

    # gsALMBase.hpp:214-223: the Jacobian call factorises
    def compute_jacobian(self):
        K = self.jacobian(self.U + self.DeltaU)
        if K is None:
            raise AssemblyError()
        self.counts["jac"] += 1
        self.solver.compute(K)
        self.jacMat = K
        return K

    def solve_system(self, b):
        self.counts["solve"] += 1
        return self.solver.solve(b)

    def compute_residual(self):
        r = self.res(self.U + self.DeltaU, self.L + self.DeltaL)
        if r is None:
            raise AssemblyError()
        self.counts["res"] += 1
        self.resVec = r

    def compute_residual_norms(self):
        if self.num_iterations == 0:
            self.basisResidualF = np.linalg.norm((self.L + self.DeltaL) * self.F)
            self.basisResidualU = np.linalg.norm(self.DeltaU)
            self.residueF = np.linalg.norm(self.resVec) / np.linalg.norm((self.L + self.DeltaL) * self.F)
            self.residueU = np.linalg.norm(self.deltaU) / np.linalg.norm(self.DeltaU)
        else:
            self.residueF = np.linalg.norm(self.resVec) / self.basisResidualF
            self.residueU = np.linalg.norm(self.deltaU) / self.basisResidualU

    def compute_ubar(self):
        self.deltaUbar = self.solve_system(-self.resVec)

    def quasi_newton_predictor(self):
        """quasiNewtonPredictor (gsALMCrisfield.hpp:56-63, gsALMRiks.hpp:38-45): the Jacobian at the
        predicted point, kept for the iterations; LoadControl needs no u_t (gsALMLoadControl.hpp:23-29)."""
        self.compute_jacobian()
        if not isinstance(self, ALMLoadControl):
            self.compute_ut()
        self.compute_ubar()

    def compute_ut(self):
        self.deltaUt = self.solve_system(self.F)

    def _step(self):
        self.converged = False
        self.num_iterations = 0
        self.initiate_step()
        if (self.Uguess is not None and len(self.Uguess) and np.linalg.norm(self.Uguess - self.U) != 0
                and (self.Lguess - self.L) != 0):
            self.predictor_guess()
        else:
            self.predictor()
        self.compute_residual()
        self.compute_residual_norms()
        quasi = bool(self.opts["Quasi"])
        interval = int(self.opts["QuasiIterations"])
        if quasi:
            self.quasi_newton_predictor()
        self.stabilityPrev = self.stability
        for it in range(1, self.maxIt):
            self.num_iterations = it
            if (not quasi) or (interval > 0 and it % interval == 0):
                self.quasi_newton_iteration()
            self.iteration()
            if int(self.opts["BifurcationMethod"]) in (0, 1):
                self.compute_stability(jacobian=False)
            else:
                self.indicator, self.negatives, self.stability = 0.0, 0, -1
            self.compute_residual()
            self.compute_residual_norms()
            if self.residueF < self.tolF and self.residueU < self.tolU:
                self.iteration_finish()
                if self.adaptive:
                    self.compute_length()
                else:
                    self.arcLength_prev = self.arcLength
                return
            elif it == self.maxIt - 1:
                raise NotConverged()

    def step(self):
        return _status_of(self._step)


class ALMCrisfield(_ALMBase):
    """gsALMCrisfield restated (gsALMCrisfield.hpp:22-427); AngleMethod 0 (Step) and 1 (Iteration)."""

    def distance(self, DU, DL):
        """gsALMCrisfield.h:79-83."""
        return float(np.sqrt(float(DU @ DU) + self.phi ** 2 * float(self.F @ self.F) * DL ** 2))

    def apply_options(self):
        super().apply_options()
        self.phi = float(self.opts["Scaling"])
        self.phi_user = self.phi != -1
        self.angle = int(self.opts["AngleMethod"])

    def initiate_step(self):
        n = self.numDof
        self.DeltaU = np.zeros(n); self.deltaUbar = np.zeros(n); self.deltaUt = np.zeros(n)
        self.DeltaL = self.deltaL = 0.0
        self.eta = 1.0

    def quasi_newton_iteration(self):
        self.compute_jacobian()
        self.compute_ut()

    def _A0(self):
        return self.phi ** 2 * float(self.F @ self.F)

    def compute_lambda_mu(self):
        A0 = self._A0()
        s = float(self.DeltaUold @ self.deltaUt) + A0 * self.DeltaLold
        direction = 1 if s > 0 else (-1 if s < 0 else 0)
        denum = np.sqrt(float(self.deltaUt @ self.deltaUt) + A0)
        mu = self.arcLength if denum == 0 else self.arcLength / denum
        self.deltaL = direction * mu
        self.deltaU = self.deltaL * self.deltaUt

    def predictor(self):
        self.compute_jacobian()
        self.deltaUt = self.solve_system(self.F)
        if float(self.DeltaUold @ self.DeltaUold) == 0 and self.DeltaLold * self.DeltaLold == 0:
            self.deltaL = self.arcLength / np.sqrt(2 * float(self.deltaUt @ self.deltaUt))
            self.deltaU = self.deltaUbar + self.deltaL * self.deltaUt
            if not self.phi_user:
                self.phi = np.sqrt(float(self.deltaUt @ self.deltaUt) / float(self.F @ self.F))
        else:
            if not self.phi_user:
                self.phi = np.sqrt(float(self.U @ self.U) / (self.L ** 2 * float(self.F @ self.F)))
            self.compute_lambda_mu()
        self.DeltaU = self.DeltaU + self.deltaU
        self.DeltaL = self.DeltaL + self.deltaL
        if self.angle in (1, 2):
            self.DeltaUold = self.DeltaU.copy(); self.DeltaLold = self.DeltaL

    def predictor_guess(self):
        self.compute_jacobian()
        self.deltaUt = self.solve_system(self.F)
        if not self.phi_user:
            self.phi = np.sqrt(float(self.deltaUt @ self.deltaUt) / float(self.F @ self.F))
        self.DeltaUold = -(self.Uguess - self.U)
        self.DeltaLold = -(self.Lguess - self.L)
        self.compute_lambda_mu()
        self.DeltaU = self.deltaU.copy()
        self.DeltaL = self.deltaL
        self.Uguess = None

    def _lambdas_simple(self):
        A0 = self._A0()
        ut, ub, DU = self.deltaUt, self.deltaUbar, self.DeltaU
        self.a0 = float(ut @ ut) + A0
        self.b0 = 2 * (float(ut @ DU) + self.DeltaL * A0)
        self.b1 = 2 * float(ub @ ut)
        self.c0 = float(DU @ DU) + self.DeltaL ** 2 * A0 - self.arcLength ** 2
        self.c1 = 2 * float(DU @ ub)
        self.c2 = float(ub @ ub)
        self.al1 = self.a0
        self.al2 = self.b0 + self.eta * self.b1
        self.al3 = self.c0 + self.eta * self.c1 + self.eta ** 2 * self.c2
        self.disc = self.al2 ** 2 - 4 * self.al1 * self.al3

    def _lambda_dot(self):
        d0 = self.deltaLs[0] * (float(self.DeltaUold @ self.deltaUt) + self.phi ** 2 * self.DeltaLold)
        d1 = self.deltaLs[1] * (float(self.DeltaUold @ self.deltaUt) + self.phi ** 2 * self.DeltaLold)
        k = 1 if d0 < d1 else 0
        self.deltaL = self.deltaLs[k]
        self.deltaU = self.eta * self.deltaUbar + self.deltaUt * self.deltaLs[k]

    def _lambdas_modified(self):
        self.al1 = self.b1 * self.b1 - 4.0 * self.a0 * self.c2
        self.al2 = 2.0 * self.b0 * self.b1 - 4.0 * self.a0 * self.c1
        self.al3 = self.b0 * self.b0 - 4.0 * self.a0 * self.c0
        self.disc = self.al2 ** 2 - 4.0 * self.al1 * self.al3
        if self.disc >= 0:
            e0 = (-self.al2 + np.sqrt(self.disc)) / (2.0 * self.al1)
            e1 = (-self.al2 - np.sqrt(self.disc)) / (2.0 * self.al1)
            eta1, eta2 = min(e0, e1), max(e0, e1)
            xi = 0.05 * abs(eta2 - eta1)
            if eta2 < 1.0:
                self.eta = eta2 - xi
            elif eta2 > 1.0 and -self.al2 / self.al1 < 1.0:
                self.eta = eta2 + xi
            elif eta1 < 1.0 and -self.al2 / self.al1 > 1.0:
                self.eta = eta1 - xi
            elif eta1 > 1.0:
                self.eta = eta1 + xi

    def _lambdas_eta(self):
        self.al1 = self.a0
        self.al2 = self.b0 + self.eta * self.b1
        self.al3 = self.c0 + self.eta * self.c1 + self.eta ** 2 * self.c2
        self.deltaLs = [-self.al2 / (2 * self.al1)] * 2

    def _lambdas_complex(self):
        A0 = self._A0()
        DUcr = self.DeltaU + self.deltaUbar
        Fint = self.jacMat @ (self.U + self.DeltaU)
        Lcr = float(Fint @ self.F) / float(self.F @ self.F)
        DLcr = Lcr - self.L
        arc_cr = np.sqrt(float(DUcr @ DUcr) + A0 * DLcr ** 2)
        mu = self.arcLength / arc_cr
        self.deltaL = mu * DLcr - self.DeltaL
        self.deltaU = mu * DUcr - self.DeltaU

    def compute_lambdas(self):
        self.deltaLs = [0.0, 0.0]
        self._lambdas_simple()
        if self.disc >= 0:
            self.eta = 1.0
            self.deltaLs = [(-self.al2 + np.sqrt(self.disc)) / (2 * self.al1),
                            (-self.al2 - np.sqrt(self.disc)) / (2 * self.al1)]
            self._lambda_dot()
        else:
            self._lambdas_modified()
            if self.disc >= 0 and self.eta > 0.05:
                self._lambdas_eta()
                self._lambda_dot()
            else:
                self.eta = 1.0
                self._lambdas_complex()

    def iteration(self):
        self.compute_ubar()
        self.eta = 1.0
        lamold = self.deltaL
        self.compute_lambdas()
        if (lamold * self.deltaL < 0 and abs(self.deltaL) <= abs(lamold)) and self.relax != 1.0:
            self.deltaU = self.relax * (self.deltaL * self.deltaUt + self.eta * self.deltaUbar)
            self.deltaL = self.relax * self.deltaL
        self.DeltaU = self.DeltaU + self.deltaU
        self.DeltaL = self.DeltaL + self.deltaL
        if self.angle == 1:
            self.DeltaUold = self.DeltaU.copy(); self.DeltaLold = self.DeltaL

    def iteration_finish(self):
        self.converged = True
        self.Uprev, self.Lprev = self.U.copy(), self.L
        self.U = self.U + self.DeltaU
        self.L = self.L + self.DeltaL
        if self.angle == 0:
            self.DeltaUold = self.DeltaU.copy(); self.DeltaLold = self.DeltaL


class ALMRiks(_ALMBase):
    """gsALMRiks restated (gsALMRiks.hpp:40-170)."""

    def distance(self, DU, DL):
        """gsALMRiks.h:81-84."""
        return float(np.sqrt(self.phi * float(DU @ DU) + (1.0 - self.phi) * DL ** 2))

    def initiate_step(self):
        self.DeltaU = np.zeros(self.numDof); self.deltaU = np.zeros(self.numDof)
        self.DeltaL = self.deltaL = 0.0

    def quasi_newton_iteration(self):
        self.compute_jacobian()
        self.compute_ut()

    def predictor(self):
        self.compute_jacobian()
        self.phi = 0.99999999999 if self.numDof == 1 else 1.0 / self.numDof
        tol = 1e-10
        if np.linalg.norm(self.U - self.Uprev) < tol and (self.L - self.Lprev) ** 2 < tol:
            DL = 1.0
            self.deltaUt = self.solve_system(self.F)
            den = np.sqrt(float(self.deltaUt @ self.deltaUt) + self.DeltaL * DL)
            self.deltaU = self.deltaUt / den
            self.deltaL = DL / den
        else:
            self.deltaL = 1.0 / self.arcLength_prev * (self.L - self.Lprev)
            self.deltaU = 1.0 / self.arcLength_prev * (self.U - self.Uprev)
        self.deltaL *= self.arcLength
        self.deltaU = self.deltaU * self.arcLength
        self.DeltaU = self.DeltaU + self.deltaU
        self.DeltaL += self.deltaL

    def predictor_guess(self):
        self.compute_jacobian()
        self.deltaUt = self.solve_system(self.F)
        tol = 1e-10
        if np.linalg.norm(self.Uguess - self.U) < tol and (self.Lguess - self.L) ** 2 < tol:
            DL = 1.0
            self.deltaUt = self.solve_system(self.F)
            den = np.sqrt(float(self.deltaUt @ self.deltaUt) + self.DeltaL * DL)
            self.deltaU = self.deltaUt / den
            self.deltaL = DL / den
        else:
            self.deltaL = 1.0 / self.arcLength_prev * (self.Lguess - self.L)
            self.deltaU = 1.0 / self.arcLength_prev * (self.Uguess - self.U)
        self.deltaL *= self.arcLength
        self.deltaU = self.deltaU * self.arcLength
        self.DeltaU = self.deltaU.copy()
        self.DeltaL = self.deltaL
        self.Uguess = None

    def iteration(self):
        self.compute_ubar()
        r = (self.phi * float(self.DeltaU @ self.DeltaU) + (1 - self.phi) * self.DeltaL ** 2
             - self.arcLength ** 2)
        self.deltaL = -(r + 2 * self.phi * float(self.DeltaU @ self.deltaUbar)) / (
            2 * (1 - self.phi) * self.DeltaL + 2 * self.phi * float(self.DeltaU @ self.deltaUt))
        self.deltaU = self.deltaUbar + self.deltaL * self.deltaUt
        self.DeltaU = self.DeltaU + self.deltaU
        self.DeltaL += self.deltaL

    def iteration_finish(self):
        self.converged = True
        self.Uprev, self.Lprev = self.U.copy(), self.L
        self.U = self.U + self.DeltaU
        self.L += self.DeltaL


class ALMLoadControl(_ALMBase):
    """gsALMLoadControl restated (gsALMLoadControl.hpp:33-108)."""

    def initiate_step(self):
        self.DeltaU = np.zeros(self.numDof); self.deltaU = np.zeros(self.numDof)
        self.DeltaL = self.deltaL = 0.0

    def quasi_newton_iteration(self):
        self.compute_jacobian()

    def predictor(self):
        self.compute_jacobian()
        self.DeltaL = self.deltaL = self.arcLength
        self.deltaUt = self.solve_system(self.F)
        self.DeltaU = self.deltaL * self.deltaUt

    def predictor_guess(self):
        self.compute_jacobian()
        self.DeltaL = self.deltaL = self.Lguess - self.L
        self.deltaUt = self.solve_system(self.F)
        self.DeltaU = self.deltaL * self.deltaUt

    def iteration(self):
        self.compute_ubar()
        self.deltaU = self.deltaUbar
        self.DeltaU = self.DeltaU + self.deltaU

    def iteration_finish(self):
        self.converged = True
        self.Uprev, self.Lprev = self.U.copy(), self.L
        self.U = self.U + self.DeltaU
        self.L += self.DeltaL


class ALMConsistentCrisfield(_ALMBase):
    """gsALMConsistentCrisfield restated (gsALMConsistentCrisfield.hpp:22-209): secant predictor,
    linearised constraint corrector (Carrera 1994, eqs. 20-21)."""

    def apply_options(self):
        super().apply_options()
        self.phi = float(self.opts["Scaling"])
        self.phi_user = self.phi != -1

    def initiate_step(self):
        self.DeltaU = np.zeros(self.numDof); self.deltaU = np.zeros(self.numDof)
        self.DeltaL = self.deltaL = 0.0

    def quasi_newton_iteration(self):
        self.compute_jacobian()
        self.compute_ut()

    def _predict(self, dU_sec, dL_sec):
        tol = 1e-10
        if np.linalg.norm(dU_sec) < tol and dL_sec * dL_sec < tol:
            DL = 1.0
            self.deltaUt = self.solve_system(self.F)
            den = np.sqrt(float(self.deltaUt @ self.deltaUt) + self.DeltaL * DL)
            self.deltaU = self.deltaUt / den
            self.deltaL = DL / den
        else:
            self.deltaL = dL_sec / self.arcLength_prev
            self.deltaU = dU_sec / self.arcLength_prev
        if not self.phi_user:
            self.phi = np.sqrt(float(self.deltaUt @ self.deltaUt) / float(self.F @ self.F))
        self.deltaL *= self.arcLength
        self.deltaU = self.deltaU * self.arcLength
        self.DeltaU = self.DeltaU + self.deltaU
        self.DeltaL += self.deltaL

    def predictor(self):
        self.compute_jacobian()
        self._predict(self.U - self.Uprev, self.L - self.Lprev)

    def predictor_guess(self):
        self.compute_jacobian()
        self._predict(self.Uguess - self.U, self.Lguess - self.L)

    def iteration(self):
        self.compute_ubar()
        FF = float(self.F @ self.F)
        cres = float(self.DeltaU @ self.DeltaU) + self.phi ** 2 * self.DeltaL ** 2 * FF - self.arcLength ** 2
        num = cres + 2.0 * float(self.DeltaU @ self.deltaUbar)
        denum = 2.0 * float(self.DeltaU @ self.deltaUt) + self.phi ** 2 * 2.0 * self.DeltaL * FF
        self.deltaL = -num / denum
        self.deltaU = self.deltaL * self.deltaUt + self.deltaUbar
        self.DeltaU = self.DeltaU + self.deltaU
        self.DeltaL += self.deltaL

    def iteration_finish(self):
        self.converged = True
        self.Uprev, self.Lprev = self.U.copy(), self.L
        self.U = self.U + self.DeltaU
        self.L += self.DeltaL
        self.DeltaUold, self.DeltaLold = self.DeltaU.copy(), self.DeltaL


# ---------------------------------------------------------------------------------------------
# Eigen problems (Spectra stand-in: scipy ARPACK)
# ---------------------------------------------------------------------------------------------
def buckling(K_lin, F, jacobian, nev=10, shift=0.0, scaling=1.0, tol=1e-10):
    """gsBucklingSolver (gsBucklingSolver.h:127-149): u_L = K_L^-1 (s F), B = K_NL(u_L) - K_L,
    eigenpairs of K_L x = lambda B x in Spectra's Buckling mode (shift-invert about ``shift``)."""
    lu = SuperLUSolver()
    lu.compute(K_lin)
    uL = lu.solve(scaling * F)
    B = (jacobian(uL) - K_lin).tocsc()
    v0 = np.ones(K_lin.shape[0])
    vals, vecs = spla.eigsh(sp.csc_matrix(K_lin), k=nev, M=B, sigma=shift, mode="buckling", which="LM", tol=tol,
                            v0=v0)
    order = np.argsort(np.abs(vals))
    return vals[order], vecs[:, order], uL


def buckling_dense(K_lin, F, jacobian, nev=10, shift=0.0, scaling=1.0):
    """Dense variant of ``buckling`` for small pencils: B v = mu K_L v with K_L symmetric positive
    definite (scipy.linalg.eigh), lambda = 1/mu; the nev eigenvalues nearest ``shift`` (the set
    Spectra's Buckling mode targets), ordered by |lambda|.  Unlike ARPACK from a start vector it
    cannot miss an eigenvalue of the requested set."""
    import scipy.linalg as sla
    lu = SuperLUSolver()
    lu.compute(K_lin)
    uL = lu.solve(scaling * F)
    B = (jacobian(uL) - K_lin).toarray()
    mu, V = sla.eigh(B, K_lin.toarray())
    keep = np.abs(mu) > 1e-300
    lam, V = 1.0 / mu[keep], V[:, keep]
    sel = np.argsort(np.abs(lam - shift))[:nev]
    order = sel[np.argsort(np.abs(lam[sel]))]
    return lam[order], V[:, order], uL


def modal(K, M, nev=10, shift=0.0, tol=1e-10):
    """gsModalSolver pencil (K, M) in shift-invert mode (gsModalSolver.h:46-51)."""
    v0 = np.ones(K.shape[0])
    vals, vecs = spla.eigsh(sp.csc_matrix(K), k=nev, M=sp.csc_matrix(M), sigma=shift, which="LM", tol=tol, v0=v0)
    order = np.argsort(np.abs(vals - shift))
    return vals[order], vecs[:, order]
