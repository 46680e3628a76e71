"""Bindings of oracle/_ref/libref_solvers.so -- the reference's own solver classes compiled from
its unchanged headers (gsStaticNewton, gsALMCrisfield, gsALMRiks, gsALMLoadControl,
gsALMConsistentCrisfield, gsModalSolver, gsBucklingSolver, and the time integrators
gsDynamicNewmark, gsDynamicBathe, gsDynamicWilson, gsDynamicExplicitEuler,
gsDynamicImplicitEuler, gsDynamicRK4)
against the test-only stand-in in oracle/refshim/.  TEST INFRASTRUCTURE ONLY: the tests use it to pin the Python restatement
(oracle.py) and to write golden fixtures; the product never imports it.

The library exists only where the reference tree is present (``make -C oracle ref``);
``available()`` says whether it could be built.  The operators come from the FP64 KL-shell
oracle assembler: Jacobian_t (dense CSR pattern), ALResidual_t (Fint - lambda F) and Residual_t
(F - Fint), as gsStructuralAnalysisTypes.h:58-93 define them.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_ref", "libref_solvers.so")
APALM_DATA_DRIVER = os.path.join(HERE, "_ref", "ref_apalm_data")   # gsAPALMData on a scripted job run
REF_TREE = os.environ.get("KLSA_REFERENCE_TREE", "/root/reference")

_JAC = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double))
_ALRES = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.POINTER(ctypes.c_double), ctypes.c_double,
                          ctypes.POINTER(ctypes.c_double))
_RES = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double))
_TMAT = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.POINTER(ctypes.c_double), ctypes.c_double,
                         ctypes.POINTER(ctypes.c_double))
_TVEC = _TMAT
_vp = ctypes.c_void_p
_lib = None

STATUS = {0: "Success", 1: "NotConverged", 2: "AssemblyError", 3: "SolverError", 4: "NotStarted", 5: "OtherError"}


def build() -> bool:
    """Build the library from the reference tree (only where it exists)."""
    if not os.path.isdir(os.path.join(REF_TREE, "src", "gsALMSolvers")):
        return os.path.exists(LIB)
    r = subprocess.run(["make", "-C", HERE, "ref", f"REF_SRC={REF_TREE}"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("building the reference solver oracle failed:\n" + r.stdout + r.stderr)
    return True


def available() -> bool:
    try:
        return build() and os.path.exists(LIB)
    except RuntimeError:
        return False


def lib():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(LIB)
        L.refh_last_error.restype = ctypes.c_char_p
        L.refh_problem_create.restype = _vp
        L.refh_problem_create.argtypes = [ctypes.c_int, ctypes.c_int64, _vp, _vp, _JAC, _ALRES, _RES, _vp]
        L.refh_problem_destroy.argtypes = [_vp]
        L.refh_alm_create.restype = _vp
        L.refh_alm_create.argtypes = [_vp, ctypes.c_char_p, ctypes.c_char_p]
        L.refh_alm_destroy.argtypes = [_vp]
        for f in ("refh_alm_initialize",):
            getattr(L, f).argtypes = [_vp, ctypes.c_int]
        L.refh_alm_step.argtypes = [_vp]
        L.refh_alm_solution.argtypes = [_vp, _vp, _vp]
        L.refh_alm_set_initial_guess.argtypes = [_vp, _vp, ctypes.c_double]
        L.refh_alm_set_solution.argtypes = [_vp, _vp, ctypes.c_double]
        L.refh_alm_set_length.argtypes = [_vp, ctypes.c_double]
        L.refh_alm_reduce_length.argtypes = [_vp, ctypes.c_double]
        L.refh_alm_info.argtypes = [_vp, _vp]
        L.refh_alm_is_bifurcation.argtypes = [_vp, ctypes.c_int]
        L.refh_alm_compute_singular_point.argtypes = [_vp, _vp, ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.refh_alm_switch_branch.argtypes = [_vp]
        L.refh_newton_create.restype = _vp
        L.refh_newton_create.argtypes = [_vp, ctypes.c_char_p]
        L.refh_newton_destroy.argtypes = [_vp]
        L.refh_newton_solve.argtypes = [_vp]
        L.refh_newton_solve_linear.argtypes = [_vp]
        L.refh_newton_set_displacement.argtypes = [_vp, _vp]
        L.refh_newton_solution.argtypes = [_vp, _vp]
        L.refh_newton_iterations.argtypes = [_vp]
        L.refh_eigen_dense.argtypes = [ctypes.c_int, ctypes.c_int, _vp, _vp, ctypes.c_char_p, ctypes.c_int, _vp, _vp]
        L.refh_apalm_create.restype = _vp
        L.refh_apalm_create.argtypes = [_vp, ctypes.c_char_p, ctypes.c_char_p]
        L.refh_apalm_destroy.argtypes = [_vp]
        L.refh_apalm_initialize.argtypes = [_vp]
        L.refh_apalm_serial_solve.argtypes = [_vp, ctypes.c_int]
        L.refh_apalm_parallel_solve.argtypes = [_vp]
        L.refh_apalm_solve.argtypes = [_vp, ctypes.c_int]
        L.refh_apalm_branches.argtypes = [_vp]
        L.refh_apalm_points.argtypes = [_vp, ctypes.c_int]
        L.refh_apalm_point.argtypes = [_vp, ctypes.c_int, ctypes.c_int, _vp, _vp, _vp, _vp]
        L.refh_buckling_power.argtypes = [_vp, ctypes.c_double, ctypes.c_char_p, _vp, _vp]
        L.refh_dyn_create.restype = _vp
        L.refh_dyn_create.argtypes = [ctypes.c_int, ctypes.c_int64, _vp, _vp, ctypes.c_char_p, ctypes.c_int, _TMAT,
                                      _TMAT, _TMAT, _TVEC, ctypes.c_char_p]
        L.refh_dyn_destroy.argtypes = [_vp]
        L.refh_dyn_set_state.argtypes = [_vp, _vp, _vp, _vp]
        L.refh_dyn_step.argtypes = [_vp, ctypes.c_double]
        L.refh_dyn_state.argtypes = [_vp, _vp, _vp, _vp, _vp]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(_vp)


def _err():
    return lib().refh_last_error().decode()


def option_spec(opts: dict) -> bytes:
    """gsOptionList entries as the harness's "key=type:value;..." string (bool -> switch, int ->
    int, float -> real, str -> string)."""
    parts = []
    for k, v in opts.items():
        if isinstance(v, bool):
            parts.append(f"{k}=b:{int(v)}")
        elif isinstance(v, (int, np.integer)):
            parts.append(f"{k}=i:{int(v)}")
        elif isinstance(v, (float, np.floating)):
            parts.append(f"{k}=r:{float(v)!r}")
        else:
            parts.append(f"{k}=s:{v}")
    return ";".join(parts).encode()


class Operators:
    """The reference's callbacks over a dense CSR pattern, from Python functions
    jacobian(x) -> sparse/dense matrix, al_residual(x, lam) -> Fint - lam F and
    residual(x) -> F - Fint."""

    def __init__(self, n, F, jacobian, al_residual, residual):
        self.n = n
        self.F = np.ascontiguousarray(F, dtype=np.float64)
        self._jac, self._alres, self._res = jacobian, al_residual, residual
        self.rowptr = np.arange(0, n * n + 1, n, dtype=np.int64)
        self.cols = np.tile(np.arange(n, dtype=np.int32), n)
        self.failures = 0

        def jac(x, vals):
            try:
                K = self._jac(np.ctypeslib.as_array(x, shape=(n,)).copy())
                K = K.toarray() if hasattr(K, "toarray") else np.asarray(K)
                np.ctypeslib.as_array(vals, shape=(n * n,))[:] = K.ravel()
                return 0
            except Exception:
                self.failures += 1
                return 1

        def alres(x, lam, R):
            try:
                np.ctypeslib.as_array(R, shape=(n,))[:] = self._alres(np.ctypeslib.as_array(x, shape=(n,)).copy(), lam)
                return 0
            except Exception:
                self.failures += 1
                return 1

        def res(x, R):
            try:
                np.ctypeslib.as_array(R, shape=(n,))[:] = self._res(np.ctypeslib.as_array(x, shape=(n,)).copy())
                return 0
            except Exception:
                self.failures += 1
                return 1

        self._cb = (_JAC(jac), _ALRES(alres), _RES(res))
        h = lib().refh_problem_create(n, n * n, _p(self.rowptr), _p(self.cols), *self._cb, _p(self.F))
        if not h:
            raise RuntimeError(_err())
        self.h = h

    @classmethod
    def from_assembler(cls, A, F=None):
        """Operators of an oracle.OracleAssembler (F: the reference load, default the problem's)."""
        F = A.force() if F is None else np.asarray(F, dtype=np.float64)
        return cls(len(F), F, A.jacobian, lambda x, lam: A.fint(x) - lam * F, lambda x: F - A.fint(x))

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.refh_problem_destroy(self.h)
            self.h = None


class ALM:
    """gsALMCrisfield / gsALMRiks / gsALMLoadControl / gsALMConsistentCrisfield of the reference."""

    def __init__(self, ops: Operators, method: str, options: dict):
        self.ops = ops
        h = lib().refh_alm_create(ops.h, method.encode(), option_spec(options))
        if not h:
            raise RuntimeError(_err())
        self.h = h

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.refh_alm_destroy(self.h)
            self.h = None

    def initialize(self, stability=True):
        if lib().refh_alm_initialize(self.h, int(stability)) < 0:
            raise RuntimeError(_err())

    def step(self) -> int:
        st = lib().refh_alm_step(self.h)
        if st < 0:
            raise RuntimeError(_err())
        return st

    def solution(self):
        U = np.zeros(self.ops.n)
        L = np.zeros(1)
        lib().refh_alm_solution(self.h, _p(U), _p(L))
        return U, float(L[0])

    def set_initial_guess(self, U, L):
        U = np.ascontiguousarray(U, dtype=np.float64)
        lib().refh_alm_set_initial_guess(self.h, _p(U), float(L))

    def set_solution(self, U, L):
        U = np.ascontiguousarray(U, dtype=np.float64)
        lib().refh_alm_set_solution(self.h, _p(U), float(L))

    def set_length(self, length):
        lib().refh_alm_set_length(self.h, float(length))

    def reduce_length(self, fac=0.5):
        lib().refh_alm_reduce_length(self.h, float(fac))

    def is_bifurcation(self, jacobian=False) -> bool:
        r = lib().refh_alm_is_bifurcation(self.h, int(jacobian))
        if r < 0:
            raise RuntimeError(_err())
        return bool(r)

    def compute_singular_point(self, U, L, switch_branch=False, jacobian=False, test_point=True) -> int:
        U = np.ascontiguousarray(U, dtype=np.float64)
        st = lib().refh_alm_compute_singular_point(self.h, _p(U), float(L), int(switch_branch), int(jacobian),
                                                   int(test_point))
        if st < 0:
            raise RuntimeError(_err())
        return st

    def switch_branch(self):
        if lib().refh_alm_switch_branch(self.h) < 0:
            raise RuntimeError(_err())

    def info(self):
        out = np.zeros(5)
        lib().refh_alm_info(self.h, _p(out))
        return dict(zip(["iterations", "indicator", "stability", "stability_change", "length"], out.tolist()))


class StaticNewton:
    """gsStaticNewton(K_L, F, Jacobian_t, Residual_t) of the reference, initialised as its
    drivers do (options set, then initialize())."""

    def __init__(self, ops: Operators, options: dict):
        self.ops = ops
        h = lib().refh_newton_create(ops.h, option_spec(options))
        if not h:
            raise RuntimeError(_err())
        self.h = h

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.refh_newton_destroy(self.h)
            self.h = None

    def solve(self) -> int:
        return lib().refh_newton_solve(self.h)

    def solve_linear(self) -> int:
        return lib().refh_newton_solve_linear(self.h)

    def set_displacement(self, U):
        U = np.ascontiguousarray(U, dtype=np.float64)
        lib().refh_newton_set_displacement(self.h, _p(U))

    def solution(self):
        U = np.zeros(self.ops.n)
        lib().refh_newton_solution(self.h, _p(U))
        return U

    def iterations(self) -> int:
        return lib().refh_newton_iterations(self.h)


def eigen_dense(kind: str, A, B, options: dict | None = None, power: bool = False):
    """gsEigenProblemBase::compute (all pairs, dense generalized solver) or ::computePower (one
    pair) of gsModalSolver(A, B) (kind "modal") or gsBucklingSolver(A, Bnl) (kind "buckling": the
    pencil (A, Bnl - A)).  Returns (status, values, vectors)."""
    A = np.asfortranarray(A.toarray() if hasattr(A, "toarray") else A, dtype=np.float64)
    B = np.asfortranarray(B.toarray() if hasattr(B, "toarray") else B, dtype=np.float64)
    n = A.shape[0]
    vals = np.zeros(1 if power else n)
    vecs = np.zeros((n, 1) if power else (n, n), order="F")
    st = lib().refh_eigen_dense(0 if kind == "modal" else 1, n, _p(A), _p(B), option_spec(options or {}), int(power),
                                _p(vals), vecs.ctypes.data_as(_vp))
    if st < 0:
        raise RuntimeError(_err())
    return st, vals, vecs


def buckling_power(ops: Operators, scaling: float, options: dict | None = None):
    """gsBucklingSolver(K_L, F, Jacobian_t, scaling).computePower(): (status, value, vector)."""
    val, vec = np.zeros(1), np.zeros(ops.n)
    st = lib().refh_buckling_power(ops.h, float(scaling), option_spec(options or {}), _p(val), _p(vec))
    if st < 0:
        raise RuntimeError(_err())
    return st, float(val[0]), vec


class APALM:
    """gsAPALM of the reference over an ``ALM`` (built without MPI: serialSolve, the one-process
    parallelSolve, and solve).  ``options`` are gsAPALM's (SubIntervals, MaxIt, ...),
    ``data_options`` gsAPALMData's (MaxLevel, Tolerance)."""

    def __init__(self, alm: ALM, options: dict, data_options: dict):
        self.alm = alm
        h = lib().refh_apalm_create(alm.h, option_spec(options), option_spec(data_options))
        if not h:
            raise RuntimeError(_err())
        self.h = h

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.refh_apalm_destroy(self.h)
            self.h = None

    def _call(self, rc):
        if rc < 0:
            raise RuntimeError(_err())
        return rc

    def initialize(self):
        self._call(lib().refh_apalm_initialize(self.h))

    def serial_solve(self, nsteps):
        self._call(lib().refh_apalm_serial_solve(self.h, int(nsteps)))

    def parallel_solve(self):
        self._call(lib().refh_apalm_parallel_solve(self.h))

    def solve(self, nsteps):
        self._call(lib().refh_apalm_solve(self.h, int(nsteps)))

    def branches(self) -> int:
        return self._call(lib().refh_apalm_branches(self.h))

    def flat(self, branch=0):
        """(U per point, L per point, times, levels) of getFlatSolutions / Times / Levels."""
        n = self._call(lib().refh_apalm_points(self.h, int(branch)))
        Us, Ls, ts, lvs = [], [], [], []
        for k in range(n):
            U, L, t, lv = np.zeros(self.alm.ops.n), np.zeros(1), np.zeros(1), np.zeros(1, dtype=np.int32)
            self._call(lib().refh_apalm_point(self.h, int(branch), k, _p(U), _p(L), _p(t), _p(lv)))
            Us.append(U)
            Ls.append(float(L[0]))
            ts.append(float(t[0]))
            lvs.append(int(lv[0]))
        return Us, Ls, ts, lvs


class Dynamic:
    """gsDynamicNewmark / gsDynamicBathe / gsDynamicWilson / gsDynamicExplicitEuler /
    gsDynamicImplicitEuler / gsDynamicRK4 of the reference (template flag _NL = ``nonlinear``), built with the linear constructor
    (Mass_t, Damping_t, Stiffness_t, TForce_t) or the nonlinear one (Mass_t, Damping_t,
    Jacobian_t, TResidual_t) of gsDynamicBase.h:58-130.  The callbacks have the signatures of
    oracle/dynamics.py: mass(), damping(U, t), jacobian(U, t), residual(U, t) = Fext(t) - Fint(U),
    force(t); the reference calls mass, damping and the stiffness without a time (they get 0)."""

    def __init__(self, method, nonlinear, n, mass, damping, jacobian, residual=None, force=None, options=None):
        self.n = n
        self.rowptr = np.arange(0, n * n + 1, n, dtype=np.int64)
        self.cols = np.tile(np.arange(n, dtype=np.int32), n)
        self.failures = 0

        def dense(K):
            return K.toarray() if hasattr(K, "toarray") else np.asarray(K)

        def wrap_mat(fn):
            def f(x, t, vals):
                try:
                    U = None if not x else np.ctypeslib.as_array(x, shape=(n,)).copy()
                    np.ctypeslib.as_array(vals, shape=(n * n,))[:] = dense(fn(U, t)).ravel()
                    return 0
                except Exception:
                    self.failures += 1
                    return 1
            return _TMAT(f)

        def vec(x, t, out):
            try:
                if x:
                    r = residual(np.ctypeslib.as_array(x, shape=(n,)).copy(), t)
                else:
                    r = force(t)
                np.ctypeslib.as_array(out, shape=(n,))[:] = r
                return 0
            except Exception:
                self.failures += 1
                return 1

        self._cb = (wrap_mat(lambda U, t: mass()), wrap_mat(damping),
                    wrap_mat(lambda U, t: jacobian(np.zeros(n) if U is None else U, t)), _TVEC(vec))
        h = lib().refh_dyn_create(n, n * n, _p(self.rowptr), _p(self.cols), method.encode(), int(bool(nonlinear)),
                                  *self._cb, option_spec(options or {}))
        if not h:
            raise RuntimeError(_err())
        self.h = h

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.refh_dyn_destroy(self.h)
            self.h = None

    def set_state(self, U, V, A):
        U, V, A = (np.ascontiguousarray(v, dtype=np.float64) for v in (U, V, A))
        if lib().refh_dyn_set_state(self.h, _p(U), _p(V), _p(A)) < 0:
            raise RuntimeError(_err())

    def step(self, dt) -> int:
        st = lib().refh_dyn_step(self.h, float(dt))
        if st < 0:
            raise RuntimeError(_err())
        return st

    def state(self):
        """(U, V, A, time, iterations of the last step)."""
        U, V, A, info = np.zeros(self.n), np.zeros(self.n), np.zeros(self.n), np.zeros(2)
        if lib().refh_dyn_state(self.h, _p(U), _p(V), _p(A), _p(info)) < 0:
            raise RuntimeError(_err())
        return U, V, A, float(info[0]), int(info[1])
