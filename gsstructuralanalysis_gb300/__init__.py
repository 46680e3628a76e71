"""GB300 (sm_103a) Kirchhoff-Love shell hot path of gsStructuralAnalysis -- Python front-end.

ctypes bindings of the C-ABI in include/klshell_gb300.h.  The classes mirror the reference's
solver classes and callbacks (gsStaticNewton, gsALMCrisfield/Riks/LoadControl,
gsBucklingSolver, gsModalSolver, the Jacobian_t / Residual_t / ALResidual_t callbacks) with
the same option keys.  Everything runs in the CUDA library: there is no CPU code path, and
loading fails loudly if the library was not built.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import problems  # noqa: F401

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libklshell_gb300.so")
_lib = None

SUCCESS, NOT_CONVERGED, ASSEMBLY_ERROR, SOLVER_ERROR, NOT_STARTED, OTHER_ERROR = range(6)

_c_int, _c_i64, _c_dbl, _c_vp, _c_char_p = ctypes.c_int, ctypes.c_int64, ctypes.c_double, ctypes.c_void_p, ctypes.c_char_p


class PatchDesc(ctypes.Structure):
    _fields_ = [("p", ctypes.c_int32), ("n1", ctypes.c_int32), ("n2", ctypes.c_int32), ("nq", ctypes.c_int32),
                ("knots1", _c_vp), ("knots2", _c_vp), ("ctrl", _c_vp),
                ("E", _c_dbl), ("nu", _c_dbl), ("thickness", _c_dbl), ("density", _c_dbl),
                ("fixed", _c_vp), ("surface_load", _c_vp),
                ("n_point_loads", ctypes.c_int32), ("point_loads", _c_vp),
                ("n_edge_loads", ctypes.c_int32), ("edge_loads", _c_vp)]


# exported symbol -> (restype, argtypes)
SIGNATURES = {
    "klsa_last_error": (_c_char_p, []),
    "klsa_launch_count": (ctypes.c_uint64, []),
    "klsa_problem_create": (_c_int, [ctypes.POINTER(PatchDesc), ctypes.POINTER(_c_vp)]),
    "klsa_problem_destroy": (_c_int, [_c_vp]),
    "klsa_problem_ndof": (_c_i64, [_c_vp]),
    "klsa_problem_nnz": (_c_i64, [_c_vp]),
    "klsa_force": (_c_int, [_c_vp, _c_vp]),
    "klsa_residual": (_c_int, [_c_vp, _c_vp, _c_vp]),
    "klsa_al_residual": (_c_int, [_c_vp, _c_vp, _c_dbl, _c_vp]),
    "klsa_al_residual_noalloc": (_c_int, [_c_vp, _c_vp, _c_dbl, _c_vp]),
    "klsa_jacobian_csr": (_c_int, [_c_vp, _c_vp, _c_int, _c_vp, _c_vp, _c_vp]),
    "klsa_djacobian_csr": (_c_int, [_c_vp, _c_vp, _c_vp, _c_int, _c_vp, _c_vp, _c_vp]),
    "klsa_eigen_dense": (_c_int, [_c_vp, _c_vp, _c_int, _c_dbl, _c_vp, _c_vp]),
    "klsa_eigen_power": (_c_int, [_c_vp, _c_vp, _c_int, _c_dbl, _c_vp, _c_vp]),
    "klsa_mass_csr": (_c_int, [_c_vp, _c_vp, _c_vp, _c_vp]),
    "klsa_options_create": (_c_vp, []),
    "klsa_options_destroy": (None, [_c_vp]),
    "klsa_options_set_real": (_c_int, [_c_vp, _c_char_p, _c_dbl]),
    "klsa_options_set_int": (_c_int, [_c_vp, _c_char_p, _c_i64]),
    "klsa_options_set_string": (_c_int, [_c_vp, _c_char_p, _c_char_p]),
    "klsa_solver_create": (_c_int, [_c_vp, _c_char_p, _c_vp, ctypes.POINTER(_c_vp)]),
    "klsa_solver_destroy": (_c_int, [_c_vp]),
    "klsa_solver_compute_jacobian": (_c_int, [_c_vp, _c_vp]),
    "klsa_solver_compute_linear": (_c_int, [_c_vp]),
    "klsa_solver_solve": (_c_int, [_c_vp, _c_vp, _c_vp, _c_int]),
    "klsa_solver_iterations": (_c_int, [_c_vp]),
    "klsa_solver_stability": (_c_int, [_c_vp, _c_vp, _c_vp]),
    "klsa_static_create": (_c_int, [_c_vp, _c_vp, ctypes.POINTER(_c_vp)]),
    "klsa_static_destroy": (_c_int, [_c_vp]),
    "klsa_static_solve": (_c_int, [_c_vp]),
    "klsa_static_solve_linear": (_c_int, [_c_vp]),
    "klsa_static_set_load_factor": (_c_int, [_c_vp, _c_dbl]),
    "klsa_static_set_displacement": (_c_int, [_c_vp, _c_vp]),
    "klsa_static_solution": (_c_int, [_c_vp, _c_vp]),
    "klsa_static_iterations": (_c_int, [_c_vp]),
    "klsa_alm_create": (_c_int, [_c_vp, _c_char_p, _c_vp, ctypes.POINTER(_c_vp)]),
    "klsa_alm_destroy": (_c_int, [_c_vp]),
    "klsa_alm_initialize": (_c_int, [_c_vp, _c_int]),
    "klsa_alm_compute_stability": (_c_int, [_c_vp, _c_int, _c_dbl]),
    "klsa_alm_stability": (_c_int, [_c_vp, _c_vp, _c_vp, _c_vp, _c_vp]),
    "klsa_alm_is_bifurcation": (_c_int, [_c_vp, _c_int]),
    "klsa_alm_compute_singular_point": (_c_int, [_c_vp, _c_vp, _c_dbl, _c_int, _c_int, _c_int]),
    "klsa_alm_switch_branch": (_c_int, [_c_vp]),
    "klsa_alm_solution_v": (_c_int, [_c_vp, _c_vp]),
    "klsa_alm_step": (_c_int, [_c_vp]),
    "klsa_alm_set_length": (_c_int, [_c_vp, _c_dbl]),
    "klsa_alm_reduce_length": (_c_int, [_c_vp, _c_dbl]),
    "klsa_alm_get_length": (_c_dbl, [_c_vp]),
    "klsa_alm_set_solution": (_c_int, [_c_vp, _c_vp, _c_dbl]),
    "klsa_alm_set_solution_step": (_c_int, [_c_vp, _c_vp, _c_dbl]),
    "klsa_alm_set_previous": (_c_int, [_c_vp, _c_vp, _c_dbl]),
    "klsa_alm_distance": (_c_int, [_c_vp, _c_vp, _c_dbl, _c_vp]),
    "klsa_apalm_create": (_c_int, [_c_vp, _c_vp, ctypes.POINTER(_c_vp)]),
    "klsa_apalm_destroy": (_c_int, [_c_vp]),
    "klsa_apalm_initialize": (_c_int, [_c_vp]),
    "klsa_apalm_add_start": (_c_int, [_c_vp, _c_vp, _c_dbl, _c_dbl]),
    "klsa_apalm_serial_solve": (_c_int, [_c_vp, _c_int]),
    "klsa_apalm_add_worker": (_c_int, [_c_vp, _c_vp]),
    "klsa_apalm_parallel_solve": (_c_int, [_c_vp]),
    "klsa_apalm_solve": (_c_int, [_c_vp, _c_int]),
    "klsa_apalm_branches": (_c_int, [_c_vp]),
    "klsa_apalm_solutions": (_c_int, [_c_vp, _c_int]),
    "klsa_apalm_solution": (_c_int, [_c_vp, _c_int, _c_int, _c_vp, _c_vp, _c_vp, _c_vp]),
    "klsa_alm_set_initial_guess": (_c_int, [_c_vp, _c_vp, _c_dbl]),
    "klsa_alm_solution": (_c_int, [_c_vp, _c_vp, _c_vp]),
    "klsa_alm_info": (_c_int, [_c_vp, _c_vp]),
    "klsa_alm_history": (_c_int, [_c_vp, _c_vp, _c_vp, _c_vp, _c_vp]),
    "klsa_mlp_create": (_c_int, [_c_int, _c_int, _c_int, _c_int, ctypes.c_uint64, ctypes.POINTER(_c_vp)]),
    "klsa_mlp_destroy": (_c_int, [_c_vp]),
    "klsa_mlp_num_params": (_c_i64, [_c_vp]),
    "klsa_mlp_get_params": (_c_int, [_c_vp, _c_vp]),
    "klsa_mlp_set_params": (_c_int, [_c_vp, _c_vp]),
    "klsa_mlp_forward": (_c_int, [_c_vp, _c_vp, _c_int, _c_vp]),
    "klsa_mlp_loss_grad": (_c_int, [_c_vp, _c_vp, _c_vp, _c_int, _c_vp, _c_vp]),
    "klsa_mlp_train": (_c_int, [_c_vp, _c_vp, _c_vp, _c_int, _c_int, _c_int, ctypes.c_float, ctypes.c_uint64, _c_vp]),
    "klsa_predictor_create": (_c_int, [_c_vp, _c_vp, _c_vp, _c_int, _c_vp, _c_vp, _c_vp, _c_vp, ctypes.POINTER(_c_vp)]),
    "klsa_predictor_destroy": (_c_int, [_c_vp]),
    "klsa_predictor_reset": (_c_int, [_c_vp]),
    "klsa_predictor_push": (_c_int, [_c_vp, _c_vp, _c_dbl]),
    "klsa_predictor_guess": (_c_int, [_c_vp, _c_vp, _c_vp, _c_vp]),
    "klsa_alm_step_learned": (_c_int, [_c_vp, _c_vp, _c_int, _c_vp]),
    "klsa_buckling": (_c_int, [_c_vp, _c_vp, _c_int, _c_dbl, _c_dbl, _c_vp, _c_vp]),
    "klsa_modal": (_c_int, [_c_vp, _c_vp, _c_int, _c_dbl, _c_vp, _c_vp]),
    "klsa_dynamic_create": (_c_int, [_c_vp, _c_char_p, _c_int, _c_vp, ctypes.POINTER(_c_vp)]),
    "klsa_dynamic_destroy": (_c_int, [_c_vp]),
    "klsa_dynamic_set_load_table": (_c_int, [_c_vp, _c_vp, _c_vp, _c_int]),
    "klsa_dynamic_set_state": (_c_int, [_c_vp, _c_vp, _c_vp, _c_vp]),
    "klsa_dynamic_state": (_c_int, [_c_vp, _c_vp, _c_vp, _c_vp]),
    "klsa_dynamic_step": (_c_int, [_c_vp, _c_dbl]),
    "klsa_dynamic_set_time": (_c_int, [_c_vp, _c_dbl]),
    "klsa_dynamic_time": (_c_dbl, [_c_vp]),
    "klsa_dynamic_iterations": (_c_int, [_c_vp]),
    "klsa_batch_create": (_c_int, [_c_vp, _c_int, ctypes.POINTER(_c_vp)]),
    "klsa_batch_destroy": (_c_int, [_c_vp]),
    "klsa_batch_info": (_c_int, [_c_vp, _c_vp]),
    "klsa_batch_instance_ndof": (_c_i64, [_c_vp, _c_int]),
    "klsa_batch_autotune": (_c_int, [_c_vp, _c_vp, _c_int]),
    "klsa_batch_newton_create": (_c_int, [_c_vp, _c_vp, ctypes.POINTER(_c_vp)]),
    "klsa_batch_newton_destroy": (_c_int, [_c_vp]),
    "klsa_batch_newton_solve": (_c_int, [_c_vp]),
    "klsa_batch_newton_reset": (_c_int, [_c_vp]),
    "klsa_batch_newton_results": (_c_int, [_c_vp, _c_vp, _c_vp]),
    "klsa_batch_newton_solution": (_c_int, [_c_vp, _c_int, _c_vp]),
    "klsa_batch_sync": (_c_int, [_c_vp]),
    "klsa_batch_event_record": (_c_int, [_c_vp, _c_int]),
    "klsa_batch_event_elapsed": (_c_int, [_c_vp, _c_int, _c_int, _c_vp]),
    "klsa_profile_enable": (_c_int, [_c_int]),
    "klsa_profile_read": (_c_int, [_c_vp, _c_vp]),
    "klsa_profile_reset": (_c_int, []),
    "klsa_event_record": (_c_int, [_c_vp, _c_int]),
    "klsa_event_elapsed": (_c_int, [_c_vp, _c_int, _c_int, _c_vp]),
    "klsa_problem_sync": (_c_int, [_c_vp]),
    "klsa_problem_stats": (_c_int, [_c_vp, _c_vp]),
    "klsa_nd_stats": (_c_int, [_c_int, _c_int, _c_int, _c_vp, _c_int, _c_vp]),
    "klsa_nd_export": (_c_int, [_c_int, _c_int, _c_int, _c_vp, _c_int, _c_vp, _c_vp, _c_vp, _c_i64, _c_i64]),
}


class KLSAError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"status {code}: {msg}")
        self.code = code


def load_library(path: str | None = None):
    """Load the CUDA library (raises if it was not built -- there is no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(f"CUDA library not built: {p} (run gsstructuralanalysis_gb300/build.py)")
    L = ctypes.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def _ptr(a):
    return None if a is None else a.ctypes.data_as(_c_vp)


def _check(code):
    if code < 0:
        raise KLSAError(code, _lib.klsa_last_error().decode())
    return code


def launch_count() -> int:
    return int(load_library().klsa_launch_count())


PHASES = ["assembly", "factorization", "solve", "residual", "mf_update", "mf_diag", "mf_panel", "other"]


def profile_enable(on: bool = True):
    load_library().klsa_profile_enable(1 if on else 0)


def profile_reset():
    load_library().klsa_profile_reset()


def profile_read():
    ms = np.zeros(8)
    cnt = np.zeros(8, dtype=np.uint64)
    _check(load_library().klsa_profile_read(_ptr(ms), _ptr(cnt)))
    return {k: (float(m), int(c)) for k, m, c in zip(PHASES, ms, cnt)}


class Options:
    """gsOptionList-like key/value store handed to the solvers."""

    def __init__(self, values: dict | None = None):
        L = load_library()
        self.h = L.klsa_options_create()
        for k, v in (values or {}).items():
            self[k] = v

    def __setitem__(self, key, value):
        L = load_library()
        k = key.encode()
        if isinstance(value, str):
            L.klsa_options_set_string(self.h, k, value.encode())
        elif isinstance(value, (bool, int, np.integer)):
            L.klsa_options_set_int(self.h, k, int(value))
        else:
            L.klsa_options_set_real(self.h, k, float(value))

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.klsa_options_destroy(self.h)
            self.h = None


def _reject_rational(prob):
    """The device kernels evaluate a polynomial B-spline basis; a NURBS patch (weights other than
    1) is assembled only by the FP64 oracle for now."""
    w = getattr(prob, "weights", None)
    if w is not None and not np.allclose(np.asarray(w, dtype=np.float64), 1.0):
        raise NotImplementedError("rational (NURBS) patch: the device kernels evaluate a polynomial B-spline basis")


def _reject_ties(prob):
    """The device problem eliminates fixed dofs only; dofs tied to others (clamped symmetry
    sides) are solved by the FP64 oracle for now."""
    t = getattr(prob, "ties", None)
    if t is not None and len(t):
        raise NotImplementedError("tied dofs (clamped symmetry sides): the device problem eliminates fixed dofs only")


def _patch_desc(prob, keep):
    """PatchDesc of a problems.PatchProblem; the arrays it points to are stored in ``keep``."""
    _reject_rational(prob)
    _reject_ties(prob)
    k = dict(
        k1=np.ascontiguousarray(prob.knots1, dtype=np.float64),
        k2=np.ascontiguousarray(prob.knots2, dtype=np.float64),
        X=np.ascontiguousarray(prob.ctrl, dtype=np.float64),
        fx=np.ascontiguousarray(prob.fixed, dtype=np.uint8),
        qs=np.ascontiguousarray(prob.surface_load, dtype=np.float64),
        pl=np.ascontiguousarray(prob.point_loads, dtype=np.float64).reshape(-1, 5),
        ed=np.ascontiguousarray(prob.edge_loads, dtype=np.float64).reshape(-1, 4),
    )
    keep.append(k)
    return PatchDesc(prob.p, prob.n1, prob.n2, prob.nq, _ptr(k["k1"]), _ptr(k["k2"]), _ptr(k["X"]),
                     prob.E, prob.nu, prob.t, prob.rho, _ptr(k["fx"]), _ptr(k["qs"]),
                     len(k["pl"]), _ptr(k["pl"]), len(k["ed"]), _ptr(k["ed"]))


class Problem:
    """Device-resident patch problem: the Jacobian_t / Residual_t / ALResidual_t / Mass_t /
    Force_t callbacks of the reference (gsStructuralAnalysisTypes.h:58-93)."""

    def __init__(self, prob):
        L = load_library()
        self.prob = prob
        self._keep = []
        d = _patch_desc(prob, self._keep)
        h = _c_vp()
        _check(L.klsa_problem_create(ctypes.byref(d), ctypes.byref(h)))
        self.h = h
        self.ndof = int(L.klsa_problem_ndof(h))
        self.nnz = int(L.klsa_problem_nnz(h))

    def close(self):
        if getattr(self, "h", None):
            _lib.klsa_problem_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def stats(self):
        out = np.zeros(18)
        _check(_lib.klsa_problem_stats(self.h, _ptr(out)))
        keys = ["ndof", "nnz", "elements", "gauss_points", "front_bytes", "factor_flops", "tangent_flops", "nodes",
                "bytes_diag", "bytes_panel", "bytes_update", "flops_diag", "flops_panel", "flops_update",
                "launches_diag", "launches_panel", "launches_update", "solve_bytes"]
        return dict(zip(keys, out.tolist()))

    def record(self, slot):
        _check(_lib.klsa_event_record(self.h, int(slot)))

    def elapsed_ms(self, a, b):
        ms = np.zeros(1, dtype=np.float32)
        _check(_lib.klsa_event_elapsed(self.h, int(a), int(b), _ptr(ms)))
        return float(ms[0])

    def sync(self):
        _check(_lib.klsa_problem_sync(self.h))

    def force(self):
        F = np.zeros(self.ndof)
        _check(_lib.klsa_force(self.h, _ptr(F)))
        return F

    def residual(self, x):
        """Residual_t: R = Fext - Fint(x)."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        R = np.zeros(self.ndof)
        _check(_lib.klsa_residual(self.h, _ptr(x), _ptr(R)))
        return R

    def al_residual(self, x, lam):
        """ALResidual_t: R = Fint(x) - lam F."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        R = np.zeros(self.ndof)
        _check(_lib.klsa_al_residual(self.h, _ptr(x), float(lam), _ptr(R)))
        return R

    def _csr(self, fn, *args):
        import scipy.sparse as sp
        rp = np.zeros(self.ndof + 1, dtype=np.int64)
        cols = np.zeros(self.nnz, dtype=np.int32)
        vals = np.zeros(self.nnz)
        _check(fn(self.h, *args, _ptr(rp), _ptr(cols), _ptr(vals)))
        return sp.csr_matrix((vals, cols, rp), shape=(self.ndof, self.ndof))

    def jacobian(self, x, precision: int = 1):
        """Jacobian_t: K(x); precision 0 = FP32 element integration, 1 = FP64."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        return self._csr(_lib.klsa_jacobian_csr, _ptr(x), int(precision))

    def djacobian(self, x, dx, precision: int = 1):
        """dJacobian_t: the Jacobian called with the solution update (gsALMBase.hpp:214-223)."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        dx = np.ascontiguousarray(dx, dtype=np.float64)
        return self._csr(_lib.klsa_djacobian_csr, _ptr(x), _ptr(dx), int(precision))

    def mass(self):
        return self._csr(_lib.klsa_mass_csr)


class SparseSolver:
    """Named solver plug-in (gsSparseSolver<T>::get(name)): 'SimplicialLDLT' (multifrontal
    LDL^T) or 'CGDiagonal' (Jacobi PCG)."""

    def __init__(self, problem: Problem, name: str = "SimplicialLDLT", options: dict | None = None):
        self.problem = problem
        self.opts = Options(options)
        h = _c_vp()
        _check(_lib.klsa_solver_create(problem.h, name.encode(), self.opts.h, ctypes.byref(h)))
        self.h = h

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.klsa_solver_destroy(self.h)
            self.h = None

    def compute_jacobian(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        return _check(_lib.klsa_solver_compute_jacobian(self.h, _ptr(x)))

    def compute_linear(self):
        return _check(_lib.klsa_solver_compute_linear(self.h))

    def solve(self, b):
        b = np.ascontiguousarray(b, dtype=np.float64)
        nrhs = 1 if b.ndim == 1 else b.shape[0]
        x = np.zeros_like(b)
        _check(_lib.klsa_solver_solve(self.h, _ptr(b), _ptr(x), nrhs))
        return x

    def iterations(self):
        """CG iterations (PCG solvers) or refinement sweeps (LDL^T) of the last solve."""
        return _check(_lib.klsa_solver_iterations(self.h))

    def stability(self):
        mn = np.zeros(1)
        ng = np.zeros(1, dtype=np.int64)
        _check(_lib.klsa_solver_stability(self.h, _ptr(mn), _ptr(ng)))
        return float(mn[0]), int(ng[0])


class StaticNewton:
    """gsStaticNewton (gsStaticSolvers/gsStaticNewton.hpp) on the device."""

    def __init__(self, problem: Problem, options: dict | None = None):
        self.problem = problem
        self.opts = Options(options)
        h = _c_vp()
        _check(_lib.klsa_static_create(problem.h, self.opts.h, ctypes.byref(h)))
        self.h = h

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.klsa_static_destroy(self.h)
            self.h = None

    def solve(self):
        return _check(_lib.klsa_static_solve(self.h))

    def solveLinear(self):
        return _check(_lib.klsa_static_solve_linear(self.h))

    def setLoad(self, lam):
        _check(_lib.klsa_static_set_load_factor(self.h, float(lam)))

    def setDisplacement(self, U):
        U = np.ascontiguousarray(U, dtype=np.float64)
        _check(_lib.klsa_static_set_displacement(self.h, _ptr(U)))

    def solution(self):
        U = np.zeros(self.problem.ndof)
        _check(_lib.klsa_static_solution(self.h, _ptr(U)))
        return U

    def iterations(self):
        return int(_lib.klsa_static_iterations(self.h))


class _ALM:
    method = ""

    def __init__(self, problem: Problem, options: dict | None = None):
        self.problem = problem
        self.opts = Options(options)
        h = _c_vp()
        _check(_lib.klsa_alm_create(problem.h, self.method.encode(), self.opts.h, ctypes.byref(h)))
        self.h = h

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.klsa_alm_destroy(self.h)
            self.h = None

    def initialize(self, stability=True):
        """initialize(bool stability = true) (gsALMBase.h:110-115) -> gsStatus of the stability test."""
        return _check(_lib.klsa_alm_initialize(self.h, 1 if stability else 0))

    def computeStability(self, jacobian=True, shift=-1e2):
        return _check(_lib.klsa_alm_compute_stability(self.h, 1 if jacobian else 0, float(shift)))

    def indicator(self):
        v = ctypes.c_double()
        _check(_lib.klsa_alm_stability(self.h, ctypes.byref(v), None, None, None))
        return v.value

    def stability(self):
        """+1 unstable, -1 stable (gsALMBase.hpp:616-619)."""
        v = ctypes.c_int()
        _check(_lib.klsa_alm_stability(self.h, None, ctypes.byref(v), None, None))
        return v.value

    def stabilityChange(self):
        v = ctypes.c_int()
        _check(_lib.klsa_alm_stability(self.h, None, None, ctypes.byref(v), None))
        return bool(v.value)

    def negatives(self):
        v = ctypes.c_int64()
        _check(_lib.klsa_alm_stability(self.h, None, None, None, ctypes.byref(v)))
        return v.value

    def isBifurcation(self, jacobian=False):
        return bool(_check(_lib.klsa_alm_is_bifurcation(self.h, 1 if jacobian else 0)))

    def computeSingularPoint(self, U, L, switchBranch=False, jacobian=False, testPoint=True):
        U = np.ascontiguousarray(U, dtype=np.float64)
        return _check(_lib.klsa_alm_compute_singular_point(self.h, _ptr(U), float(L), int(bool(switchBranch)),
                                                           int(bool(jacobian)), int(bool(testPoint))))

    def switchBranch(self):
        _check(_lib.klsa_alm_switch_branch(self.h))

    def solutionV(self):
        V = np.zeros(self.problem.ndof)
        _check(_lib.klsa_alm_solution_v(self.h, _ptr(V)))
        return V

    def step(self):
        return _check(_lib.klsa_alm_step(self.h))

    def setLength(self, length):
        _check(_lib.klsa_alm_set_length(self.h, float(length)))

    def reduceLength(self, fac=0.5):
        _check(_lib.klsa_alm_reduce_length(self.h, float(fac)))

    def getLength(self):
        return float(_lib.klsa_alm_get_length(self.h))

    def setSolution(self, U, L):
        U = np.ascontiguousarray(U, dtype=np.float64)
        _check(_lib.klsa_alm_set_solution(self.h, _ptr(U), float(L)))

    def setSolutionStep(self, DU, DL):
        DU = np.ascontiguousarray(DU, dtype=np.float64)
        _check(_lib.klsa_alm_set_solution_step(self.h, _ptr(DU), float(DL)))

    def setPrevious(self, Uprev, Lprev):
        Uprev = np.ascontiguousarray(Uprev, dtype=np.float64)
        _check(_lib.klsa_alm_set_previous(self.h, _ptr(Uprev), float(Lprev)))

    def distance(self, DU, DL):
        DU = np.ascontiguousarray(DU, dtype=np.float64)
        out = ctypes.c_double()
        _check(_lib.klsa_alm_distance(self.h, _ptr(DU), float(DL), ctypes.byref(out)))
        return out.value

    def setInitialGuess(self, U, L):
        U = np.ascontiguousarray(U, dtype=np.float64)
        _check(_lib.klsa_alm_set_initial_guess(self.h, _ptr(U), float(L)))

    def solutionU(self):
        U = np.zeros(self.problem.ndof)
        _check(_lib.klsa_alm_solution(self.h, _ptr(U), None))
        return U

    def solutionL(self):
        L = np.zeros(1)
        _check(_lib.klsa_alm_solution(self.h, None, _ptr(L)))
        return float(L[0])

    def info(self):
        out = np.zeros(10)
        _check(_lib.klsa_alm_info(self.h, _ptr(out)))
        keys = ["iterations", "residueF", "residueU", "phi", "converged", "Lprev", "DLold", "n_jac", "n_res",
                "n_solve"]
        return dict(zip(keys, out.tolist()))

    def history(self):
        n = self.problem.ndof
        Up, DUo = np.zeros(n), np.zeros(n)
        Lp, DLo = np.zeros(1), np.zeros(1)
        _check(_lib.klsa_alm_history(self.h, _ptr(Up), _ptr(Lp), _ptr(DUo), _ptr(DLo)))
        return Up, float(Lp[0]), DUo, float(DLo[0])


class ALMCrisfield(_ALM):
    """gsALMCrisfield (gsALMSolvers/gsALMCrisfield.hpp)."""
    method = "Crisfield"


class ALMRiks(_ALM):
    """gsALMRiks (gsALMSolvers/gsALMRiks.hpp)."""
    method = "Riks"


class ALMLoadControl(_ALM):
    """gsALMLoadControl (gsALMSolvers/gsALMLoadControl.hpp)."""
    method = "LoadControl"


class ALMConsistentCrisfield(_ALM):
    """gsALMConsistentCrisfield (gsALMSolvers/gsALMConsistentCrisfield.hpp)."""
    method = "ConsistentCrisfield"


def buckling(problem: Problem, nev: int, shift: float, scaling: float = 1.0, options: dict | None = None,
             vectors: bool = True):
    """gsBucklingSolver + Buckling-mode shift-invert Lanczos: K_L v = lambda (K(u_L) - K_L) v."""
    o = Options(options)
    vals = np.zeros(nev)
    vecs = np.zeros((nev, problem.ndof)) if vectors else None
    st = _check(_lib.klsa_buckling(problem.h, o.h, int(nev), float(shift), float(scaling), _ptr(vals), _ptr(vecs)))
    return st, vals, vecs


def modal(problem: Problem, nev: int, shift: float = 0.0, options: dict | None = None, vectors: bool = True):
    """gsModalSolver + ShiftInvert-mode Lanczos: K v = lambda M v."""
    o = Options(options)
    vals = np.zeros(nev)
    vecs = np.zeros((nev, problem.ndof)) if vectors else None
    st = _check(_lib.klsa_modal(problem.h, o.h, int(nev), float(shift), _ptr(vals), _ptr(vecs)))
    return st, vals, vecs


def eigen_dense(problem: Problem, kind: str = "modal", scaling: float = 1.0, options: dict | None = None,
                vectors: bool = True):
    """gsEigenProblemBase::compute: all eigenpairs of the modal or buckling pencil (dense sizes)."""
    o = Options(options)
    n = problem.ndof
    vals = np.zeros(n)
    vecs = np.zeros((n, n)) if vectors else None
    st = _check(_lib.klsa_eigen_dense(problem.h, o.h, 0 if kind == "modal" else 1, float(scaling), _ptr(vals),
                                      _ptr(vecs)))
    return st, vals, vecs


def eigen_power(problem: Problem, kind: str = "modal", scaling: float = 1.0, options: dict | None = None):
    """gsEigenProblemBase::computePower: the pair of smallest |lambda| by power iteration."""
    o = Options(options)
    val = np.zeros(1)
    vec = np.zeros(problem.ndof)
    st = _check(_lib.klsa_eigen_power(problem.h, o.h, 0 if kind == "modal" else 1, float(scaling), _ptr(val),
                                      _ptr(vec)))
    return st, float(val[0]), vec


class APALM:
    """gsAPALM over an arc-length object (ALMCrisfield or ALMRiks): serialSolve / parallelSolve /
    solve and the flat solutions, times and levels per branch (public free-dof order)."""

    def __init__(self, alm: "_ALM", options: dict | None = None):
        self.alm = alm
        self.opts = Options(options)
        h = _c_vp()
        _check(_lib.klsa_apalm_create(alm.h, self.opts.h, ctypes.byref(h)))
        self.h = h

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.klsa_apalm_destroy(self.h)
            self.h = None

    def initialize(self):
        _check(_lib.klsa_apalm_initialize(self.h))

    def addStart(self, U, L, dL):
        U = np.ascontiguousarray(U, dtype=np.float64)
        _check(_lib.klsa_apalm_add_start(self.h, _ptr(U), float(L), float(dL)))

    def serialSolve(self, nsteps=10):
        _check(_lib.klsa_apalm_serial_solve(self.h, int(nsteps)))

    def addWorker(self, alm: "_ALM"):
        """Another solver (same method and options, its own Problem of the same description) for
        parallelSolve: the reference's MPI workers as concurrent solvers on one GPU."""
        self._workers = getattr(self, "_workers", []) + [alm]
        _check(_lib.klsa_apalm_add_worker(self.h, alm.h))

    def parallelSolve(self):
        _check(_lib.klsa_apalm_parallel_solve(self.h))

    def solve(self, nsteps=10):
        _check(_lib.klsa_apalm_solve(self.h, int(nsteps)))

    def nBranches(self):
        return _check(_lib.klsa_apalm_branches(self.h))

    def _branch(self, branch, want_u=True):
        n = _check(_lib.klsa_apalm_solutions(self.h, int(branch)))
        U = np.zeros((n, self.alm.problem.ndof)) if want_u else None
        L, t = np.zeros(n), np.zeros(n)
        lv = np.zeros(n, dtype=np.int32)
        for k in range(n):
            Lk, tk, lk = ctypes.c_double(), ctypes.c_double(), ctypes.c_int()
            _check(_lib.klsa_apalm_solution(self.h, int(branch), k, _ptr(U[k]) if want_u else None,
                                            ctypes.byref(Lk), ctypes.byref(tk), ctypes.byref(lk)))
            L[k], t[k], lv[k] = Lk.value, tk.value, lk.value
        return U, L, t, lv

    def getFlatSolutions(self, branch=0):
        U, L, _, _ = self._branch(branch)
        return list(zip(U, L))

    def getFlatTimes(self, branch=0):
        return self._branch(branch, want_u=False)[2]

    def getFlatLevels(self, branch=0):
        return self._branch(branch, want_u=False)[3]


class Dynamic:
    """gsDynamicSolvers time integrators on the device: ``method`` is "Newmark", "Bathe", "Wilson",
    "ExplicitEuler", "ImplicitEuler" or "RK4"; ``nonlinear`` is the reference's _NL flag.  Vectors
    are in the public free-dof order."""

    def __init__(self, problem: Problem, method: str, nonlinear: bool = True, options: dict | None = None):
        self.problem = problem
        self.opts = Options(options)
        h = _c_vp()
        _check(_lib.klsa_dynamic_create(problem.h, method.encode(), 1 if nonlinear else 0, self.opts.h,
                                        ctypes.byref(h)))
        self.h = h

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.klsa_dynamic_destroy(self.h)
            self.h = None

    def setLoadTable(self, t, f):
        t = np.ascontiguousarray(t, dtype=np.float64)
        f = np.ascontiguousarray(f, dtype=np.float64)
        _check(_lib.klsa_dynamic_set_load_table(self.h, _ptr(t), _ptr(f), len(t)))

    def _set(self, U=None, V=None, A=None):
        c = [None if x is None else np.ascontiguousarray(x, dtype=np.float64) for x in (U, V, A)]
        _check(_lib.klsa_dynamic_set_state(self.h, *(_ptr(x) for x in c)))

    def setU(self, U):
        self._set(U=U)

    def setV(self, V):
        self._set(V=V)

    def setA(self, A):
        self._set(A=A)

    def _get(self, which):
        out = [None, None, None]
        out[which] = np.zeros(self.problem.ndof)
        _check(_lib.klsa_dynamic_state(self.h, *(_ptr(x) for x in out)))
        return out[which]

    def solutionU(self):
        return self._get(0)

    def solutionV(self):
        return self._get(1)

    def solutionA(self):
        return self._get(2)

    def step(self, dt: float | None = None):
        return _check(_lib.klsa_dynamic_step(self.h, float(dt) if dt is not None else 0.0))

    def setTime(self, t):
        _check(_lib.klsa_dynamic_set_time(self.h, float(t)))

    def time(self):
        return float(_lib.klsa_dynamic_time(self.h))

    def iterations(self):
        return int(_lib.klsa_dynamic_iterations(self.h))


class MLP:
    """Device MLP (in -> h1 -> h2 -> out, GELU) with hand-written FP32 forward/backward/Adam."""

    def __init__(self, n_in, n_h1, n_h2, n_out, seed=0):
        L = load_library()
        h = _c_vp()
        _check(L.klsa_mlp_create(n_in, n_h1, n_h2, n_out, seed, ctypes.byref(h)))
        self.h = h
        self.shape = (n_in, n_h1, n_h2, n_out)
        self.nparams = int(L.klsa_mlp_num_params(h))

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.klsa_mlp_destroy(self.h)
            self.h = None

    def params(self):
        p = np.zeros(self.nparams, dtype=np.float32)
        _check(_lib.klsa_mlp_get_params(self.h, _ptr(p)))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        _check(_lib.klsa_mlp_set_params(self.h, _ptr(p)))

    def forward(self, X):
        X = np.ascontiguousarray(X, dtype=np.float32)
        Y = np.zeros((X.shape[0], self.shape[3]), dtype=np.float32)
        _check(_lib.klsa_mlp_forward(self.h, _ptr(X), X.shape[0], _ptr(Y)))
        return Y

    def loss_grad(self, X, T):
        X = np.ascontiguousarray(X, dtype=np.float32)
        T = np.ascontiguousarray(T, dtype=np.float32)
        loss = np.zeros(1, dtype=np.float32)
        g = np.zeros(self.nparams, dtype=np.float32)
        _check(_lib.klsa_mlp_loss_grad(self.h, _ptr(X), _ptr(T), X.shape[0], _ptr(loss), _ptr(g)))
        return float(loss[0]), g

    def train(self, X, T, epochs=200, batch=256, lr=1e-3, seed=0):
        X = np.ascontiguousarray(X, dtype=np.float32)
        T = np.ascontiguousarray(T, dtype=np.float32)
        loss = np.zeros(1, dtype=np.float32)
        _check(_lib.klsa_mlp_train(self.h, _ptr(X), _ptr(T), X.shape[0], int(epochs), int(batch), float(lr), int(seed),
                                   _ptr(loss)))
        return float(loss[0])


class Predictor:
    """Learned arc-length predictor bound to one problem (modes: nmodes x ndof, public order)."""

    def __init__(self, problem: Problem, net: MLP | None, modes, in_mean=None, in_std=None, out_mean=None,
                 out_std=None):
        self.problem = problem
        self.net = net
        modes = np.ascontiguousarray(modes, dtype=np.float64).reshape(-1, problem.ndof)
        self._keep = [modes] + [None if a is None else np.ascontiguousarray(a, dtype=np.float64)
                                for a in (in_mean, in_std, out_mean, out_std)]
        h = _c_vp()
        _check(_lib.klsa_predictor_create(problem.h, net.h if net is not None else None, _ptr(modes), modes.shape[0],
                                          *[_ptr(a) for a in self._keep[1:]], ctypes.byref(h)))
        self.h = h

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.klsa_predictor_destroy(self.h)
            self.h = None

    def reset(self):
        _check(_lib.klsa_predictor_reset(self.h))

    def push(self, U, L):
        """Record a converged point (public order)."""
        U = np.ascontiguousarray(U, dtype=np.float64)
        _check(_lib.klsa_predictor_push(self.h, _ptr(U), float(L)))

    def guess(self):
        """(U, L) of the predicted next point, or None while fewer than four points are recorded."""
        U = np.zeros(self.problem.ndof)
        L = np.zeros(1)
        ok = np.zeros(1, dtype=np.int32)
        _check(_lib.klsa_predictor_guess(self.h, _ptr(U), _ptr(L), _ptr(ok)))
        return (U, float(L[0])) if ok[0] else None

    def step(self, alm, guess_max_iter=6):
        used = np.zeros(1, dtype=np.int32)
        st = _check(_lib.klsa_alm_step_learned(alm.h, self.h, int(guess_max_iter), _ptr(used)))
        return st, bool(used[0])


class BatchedProblem:
    """Many independent patches sharing every launch (no reference counterpart: the reference
    runs one assembler and one gsStaticNewton per patch)."""

    def __init__(self, probs):
        L = load_library()
        self.probs = list(probs)
        self._keep = []
        arr = (PatchDesc * len(self.probs))(*[_patch_desc(p, self._keep) for p in self.probs])
        self._arr = arr
        h = _c_vp()
        _check(L.klsa_batch_create(ctypes.cast(arr, _c_vp), len(self.probs), ctypes.byref(h)))
        self.h = h
        self.ndofs = [int(L.klsa_batch_instance_ndof(h, i)) for i in range(len(self.probs))]

    def close(self):
        if getattr(self, "h", None):
            _lib.klsa_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def info(self):
        out = np.zeros(4)
        _check(_lib.klsa_batch_info(self.h, _ptr(out)))
        return dict(zip(["instances", "ndof", "nnz", "front_bytes"], out.tolist()))

    def autotune(self):
        log = np.zeros((256, 4))
        rows = _check(_lib.klsa_batch_autotune(self.h, _ptr(log), 256))
        return log[:rows]

    def sync(self):
        _check(_lib.klsa_batch_sync(self.h))

    def record(self, slot):
        _check(_lib.klsa_batch_event_record(self.h, int(slot)))

    def elapsed_ms(self, a, b):
        ms = ctypes.c_float()
        _check(_lib.klsa_batch_event_elapsed(self.h, int(a), int(b), ctypes.byref(ms)))
        return float(ms.value)


class BatchedNewton:
    """gsStaticNewton::solve() on every instance of a BatchedProblem (gsStaticNewton.hpp:101-193)."""

    def __init__(self, batch: BatchedProblem, options: dict | None = None):
        self.batch = batch
        self.opts = Options(options)
        h = _c_vp()
        _check(_lib.klsa_batch_newton_create(batch.h, self.opts.h, ctypes.byref(h)))
        self.h = h

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.klsa_batch_newton_destroy(self.h)
            self.h = None

    def solve(self):
        return _check(_lib.klsa_batch_newton_solve(self.h))

    def reset(self):
        _check(_lib.klsa_batch_newton_reset(self.h))

    def results(self):
        n = len(self.batch.probs)
        st = np.zeros(n, dtype=np.int32)
        it = np.zeros(n, dtype=np.int32)
        _check(_lib.klsa_batch_newton_results(self.h, _ptr(st), _ptr(it)))
        return st, it

    def solution(self, i):
        U = np.zeros(self.batch.ndofs[i])
        _check(_lib.klsa_batch_newton_solution(self.h, int(i), _ptr(U)))
        return U
