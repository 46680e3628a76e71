"""Single-patch Kirchhoff-Love shell problem descriptions.

A problem is pure data: a tensor-product B-spline surface (degree, open knot
vectors, control net), an SVK material, thickness, Dirichlet mask and loads.
The same description feeds the CUDA library and the CPU oracle, so both start
from identical inputs.

Layouts
  * control point A = j*n1 + i (i along parameter 1, j along parameter 2)
  * full dof vector: component-blocked [x_0..x_{ncp-1}, y_0.., z_0..], the layout
    of the reference assembler's full solution vector
    (benchmarks/benchmark_Wrinkling.cpp:684-686); free dofs keep that order
    with the Dirichlet dofs removed (gismo's dof mapper numbers component by
    component).

Workloads
  * ``flat_plate``: square plate, all edges clamped, uniform load (config 1;
    clamped = boundary row fixed plus the normal component of the second row,
    the elimination the reference applies for ``condition_type::clamped``).
  * ``cylindrical_panel``: shallow cylindrical roof, straight edges pinned, curved
    edges free, central point load (benchmarks/benchmark_Roof.cpp:200-236).
  * ``axial_panel``: the same surface under a uniform compressive line load on a
    curved edge (buckling / modal workload).
The curved direction is the exact degree-2 Bezier net of the shallow roof
(end rows at rise 0, middle row at twice the rise R(1-cos(span/2))), raised to
degree p and refined to m elements by evaluating its blossoms at the knots, so
the geometry is identical for every p and m.
"""
from __future__ import annotations

from dataclasses import dataclass, field
import itertools
import numpy as np


def open_uniform_knots(p: int, m: int) -> np.ndarray:
    """Open uniform knot vector of degree p with m elements (n = m + p functions)."""
    inner = [k / m for k in range(1, m)]
    return np.array([0.0] * (p + 1) + inner + [1.0] * (p + 1), dtype=np.float64)


def _blossom_monomials(knots: np.ndarray, p: int) -> tuple[np.ndarray, np.ndarray]:
    """Control coefficients of f(t)=t and f(t)=t^2 in the B-spline basis (Marsden's identity)."""
    n = len(knots) - p - 1
    lin = np.zeros(n)
    quad = np.zeros(n)
    for i in range(n):
        args = knots[i + 1:i + p + 1]
        lin[i] = args.mean()
        if p >= 2:
            s = sum(a * b for a, b in itertools.combinations(args, 2))
            quad[i] = 2.0 * s / (p * (p - 1))
        else:
            quad[i] = np.nan
    return lin, quad


@dataclass
class PatchProblem:
    p: int
    n1: int
    n2: int
    knots1: np.ndarray
    knots2: np.ndarray
    ctrl: np.ndarray                     # (n1*n2, 3) reference control points
    E: float
    nu: float
    t: float
    rho: float = 1.0
    fixed: np.ndarray | None = None      # bool (3*ncp,), full layout
    surface_load: np.ndarray = field(default_factory=lambda: np.zeros(3))
    point_loads: np.ndarray = field(default_factory=lambda: np.zeros((0, 5)))
    edge_loads: np.ndarray = field(default_factory=lambda: np.zeros((0, 4)))
    nq: int = 0                          # Gauss points per direction (0: p+1)
    name: str = ""
    weights: np.ndarray | None = None    # NURBS weights (ncp,); None: B-spline
    ties: np.ndarray | None = None       # (k, 2) full-layout dofs [dof, equal to dof]; None: none

    @property
    def ncp(self) -> int:
        return self.n1 * self.n2

    @property
    def ndof_full(self) -> int:
        return 3 * self.ncp

    @property
    def m1(self) -> int:
        return self.n1 - self.p

    @property
    def m2(self) -> int:
        return self.n2 - self.p

    def free_index(self) -> np.ndarray:
        """Full-layout indices of the free dofs, in free-dof (reference) order."""
        return np.flatnonzero(~self.fixed)

    @property
    def nfree(self) -> int:
        return int((~self.fixed).sum())

    def with_ctrl(self, ctrl: np.ndarray) -> "PatchProblem":
        q = PatchProblem(**{k: getattr(self, k) for k in self.__dataclass_fields__})
        q.ctrl = np.ascontiguousarray(ctrl, dtype=np.float64)
        return q


def _grid_masks(n1: int, n2: int):
    ii, jj = np.meshgrid(np.arange(n1), np.arange(n2), indexing="xy")
    return ii.ravel(), jj.ravel()


def flat_plate(m: int = 8, p: int = 2, L: float = 1.0, t: float = 0.01, E: float = 1e7,
               nu: float = 0.3, rho: float = 1.0, bc: str = "clamped", pressure: float = 1.0) -> PatchProblem:
    """Square plate [0,L]^2 in the xy-plane, uniform load ``pressure`` in +z (dead load).

    bc = "clamped": every boundary control point fixed in x,y,z and the second row fixed
    in z; bc = "simply": boundary control points fixed in x,y,z.
    """
    U = open_uniform_knots(p, m)
    n = m + p
    g, _ = _blossom_monomials(U, p)
    ii, jj = _grid_masks(n, n)
    ctrl = np.stack([L * g[ii], L * g[jj], np.zeros(n * n)], axis=1)
    fixed = np.zeros((3, n * n), dtype=bool)
    bnd = (ii == 0) | (ii == n - 1) | (jj == 0) | (jj == n - 1)
    fixed[:, bnd] = True
    if bc == "clamped":
        second = (ii == 1) | (ii == n - 2) | (jj == 1) | (jj == n - 2)
        fixed[2, second] = True
    elif bc != "simply":
        raise ValueError(bc)
    return PatchProblem(p=p, n1=n, n2=n, knots1=U, knots2=U.copy(), ctrl=ctrl, E=E, nu=nu, t=t, rho=rho,
                        fixed=fixed.ravel(), surface_load=np.array([0.0, 0.0, pressure]),
                        name=f"plate-p{p}-m{m}")


def _panel_ctrl(p: int, m1: int, m2: int, R: float, span: float, L: float) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    U1 = open_uniform_knots(p, m1)
    U2 = open_uniform_knots(p, m2)
    g1, _ = _blossom_monomials(U1, p)
    g2, q2 = _blossom_monomials(U2, p)
    phi = 0.5 * span
    h = R * (1.0 - np.cos(phi))
    n1, n2 = m1 + p, m2 + p
    ii, jj = _grid_masks(n1, n2)
    x = L * g1[ii]
    y = R * np.sin(phi) * (2.0 * g2[jj] - 1.0)
    z = 4.0 * h * (g2[jj] - q2[jj])
    return U1, U2, np.stack([x, y, z], axis=1)


def cylindrical_panel(m: int = 64, p: int = 3, R: float = 2.5, span: float = 0.2, L: float = 2.5,
                      t: float = 0.01, E: float = 3.10275e9, nu: float = 0.3, rho: float = 1.0,
                      load: float = 1.0) -> PatchProblem:
    """Shallow cylindrical roof: parameter 1 along the straight generator (length L), parameter 2
    along the arc.  Straight edges (xi2 = 0, 1) pinned in x,y,z, curved edges free, point load
    ``load`` in -z at the parametric centre (0.5, 0.5) (benchmarks/benchmark_Roof.cpp:200-236)."""
    U1, U2, ctrl = _panel_ctrl(p, m, m, R, span, L)
    n1 = n2 = m + p
    ii, jj = _grid_masks(n1, n2)
    fixed = np.zeros((3, n1 * n2), dtype=bool)
    fixed[:, (jj == 0) | (jj == n2 - 1)] = True
    return PatchProblem(p=p, n1=n1, n2=n2, knots1=U1, knots2=U2, ctrl=ctrl, E=E, nu=nu, t=t, rho=rho,
                        fixed=fixed.ravel(), point_loads=np.array([[0.5, 0.5, 0.0, 0.0, -load]]),
                        name=f"panel-p{p}-m{m}")


def axial_panel(m: int = 256, p: int = 3, R: float = 2.5, span: float = 0.2, L: float = 2.5,
                t: float = 0.01, E: float = 3.10275e9, nu: float = 0.3, rho: float = 7850.0,
                line_load: float = 1.0) -> PatchProblem:
    """The roof surface under uniform axial compression: curved edge xi1 = 0 pinned, curved edge
    xi1 = 1 loaded by ``line_load`` per unit length in -x and held in y,z, straight edges
    simply supported (z fixed)."""
    U1, U2, ctrl = _panel_ctrl(p, m, m, R, span, L)
    n1 = n2 = m + p
    ii, jj = _grid_masks(n1, n2)
    fixed = np.zeros((3, n1 * n2), dtype=bool)
    fixed[:, ii == 0] = True
    fixed[1, ii == n1 - 1] = True
    fixed[2, ii == n1 - 1] = True
    fixed[2, (jj == 0) | (jj == n2 - 1)] = True
    return PatchProblem(p=p, n1=n1, n2=n2, knots1=U1, knots2=U2, ctrl=ctrl, E=E, nu=nu, t=t, rho=rho,
                        fixed=fixed.ravel(), edge_loads=np.array([[1.0, -line_load, 0.0, 0.0]]),
                        name=f"axial-p{p}-m{m}")


def add_imperfection(prob: PatchProblem, modes_full: np.ndarray, amplitudes: np.ndarray) -> PatchProblem:
    """Perturb the control net by sum_i a_i * phi_i, each mode (full layout, component-blocked)
    scaled to unit max |w| (z component)."""
    ncp = prob.ncp
    d = np.zeros((ncp, 3))
    for a, phi in zip(amplitudes, modes_full):
        ph = phi.reshape(3, ncp).T
        s = np.max(np.abs(ph[:, 2]))
        if s > 0:
            d += a * ph / s
    return prob.with_ctrl(prob.ctrl + d)


def bspline_basis_matrix(knots: np.ndarray, p: int, pts: np.ndarray) -> np.ndarray:
    """B[k, i] = N_{i,p}(pts[k]) on an open knot vector (Cox-de Boor, right end included)."""
    knots = np.asarray(knots, dtype=np.float64)
    n = len(knots) - p - 1
    pts = np.asarray(pts, dtype=np.float64)
    B = np.zeros((len(pts), n))
    for k, u in enumerate(pts):
        N = np.zeros(len(knots) - 1)
        if u >= knots[-1]:
            N[n - 1] = 1.0
        else:
            j = np.searchsorted(knots, u, side="right") - 1
            N[j] = 1.0
        for d in range(1, p + 1):
            M = np.zeros(len(knots) - 1 - d)
            for i in range(len(M)):
                a = knots[i + d] - knots[i]
                b = knots[i + d + 1] - knots[i + 1]
                v = 0.0
                if a > 0:
                    v += (u - knots[i]) / a * N[i]
                if b > 0:
                    v += (knots[i + d + 1] - u) / b * N[i + 1]
                M[i] = v
            N = M
        B[k] = N[:n]
    return B


def greville(knots: np.ndarray, p: int) -> np.ndarray:
    n = len(knots) - p - 1
    return np.array([np.mean(knots[i + 1:i + p + 1]) for i in range(n)])


def transfer_field(coarse: PatchProblem, field_full: np.ndarray, fine: PatchProblem) -> np.ndarray:
    """Exact transfer of a spline field (full component-blocked layout) from ``coarse`` to the
    nested spline space of ``fine`` (same degree, fine knots a superset of the coarse ones):
    interpolation at the fine Greville points of the coarse field."""
    T = []
    for Uc, Uf in ((coarse.knots1, fine.knots1), (coarse.knots2, fine.knots2)):
        g = greville(Uf, fine.p)
        Af = bspline_basis_matrix(Uf, fine.p, g)
        Ac = bspline_basis_matrix(Uc, coarse.p, g)
        T.append(np.linalg.solve(Af, Ac))
    out = np.zeros(3 * fine.ncp)
    for c in range(3):
        C = field_full[c * coarse.ncp:(c + 1) * coarse.ncp].reshape(coarse.n2, coarse.n1)
        out[c * fine.ncp:(c + 1) * fine.ncp] = (T[1] @ C @ T[0].T).ravel()
    return out
