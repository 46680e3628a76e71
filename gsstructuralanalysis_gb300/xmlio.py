"""Problem input in the reference's XML layout (gsFileData), for the single-patch SVK shell.

The reader follows what ``solvers/static_shell_XML.cpp:92-199`` takes from a file:

  id 0        the geometry: a ``MultiPatch`` whose ``patches`` name one ``Geometry``, or a
              ``Geometry`` directly (``TensorBSpline2`` or ``TensorNurbs2``)
  id 10       the material: ``MaterialMatrix type="Linear3"`` (Thickness, Density,
              Parameters E and nu), or the older ``Function`` ids 10-13 tagged ``Material``
              (thickness, E, nu, density)
  id 20       ``boundaryConditions``: ``Dirichlet`` (homogeneous), ``Clamped`` (zero slope
              across the side: the second row of control points is fixed where the boundary
              row is fixed, and tied to the boundary row where it is free, as on a symmetry
              plane), ``Neumann`` (constant edge load), corner values ``cv`` (zero)
  id 21 / 22  surface force (constant 3-vector) / pressure (must be zero: the device path has
              dead loads only)
  id 30-32    point loads: parametric points (2 x N), forces (3 x N), patch indices
  id 50-52    reference points, patches and values (returned as metadata)
  id 90-95    option lists (returned as dicts with the reference's keys)

Degree elevation and uniform refinement follow ``gsGeometry::degreeElevate`` (every knot's
multiplicity grows by one, smoothness kept) and ``uniformRefine`` (one knot in the middle of every
nonzero span), applied as in static_shell_XML.cpp:95-104 (elevate, then refine).  Control points
of the elevated / refined patch come from interpolation at the Greville points of the new space,
which reproduces the (nested) geometry exactly; a rational (NURBS) patch is transferred in
homogeneous coordinates (w X, w), which is exact as well.

Side numbers are gismo's boxSide (1 west xi1=0, 2 east xi1=1, 3 south xi2=0, 4 north xi2=1) and
corner numbers its boxCorner (1 (0,0), 2 (1,0), 3 (0,1), 4 (1,1)).  Anything the device path
cannot represent (several patches, unequal degrees, repeated interior knots, non-SVK materials,
inhomogeneous conditions, pressure, non-constant functions) raises ``NotImplementedError`` with
the reason.  NURBS weights are read into ``PatchProblem.weights`` and the ties of clamped
symmetry sides into ``PatchProblem.ties``; the FP64 oracle takes both, the device problem
neither yet (it raises).

As the reference's XML shell example (examples/gsThinShell_Static_XML.cpp:108-109), ``read``
takes the geometry and the problem (material, conditions, loads, options) from one file or from
two.
"""
from __future__ import annotations

import ast
import math
import xml.etree.ElementTree as ET
from dataclasses import dataclass, field

import numpy as np

from . import problems as P

SIDE_TO_EDGE = {1: 0, 2: 1, 3: 2, 4: 3}      # gismo boxSide -> klsa edge index


# -------------------------------------------------------------------------------------------
# constant expressions of FunctionExpr (exprtk syntax: ^ is the power)
# -------------------------------------------------------------------------------------------
_FUNCS = {"sin": math.sin, "cos": math.cos, "tan": math.tan, "sqrt": math.sqrt, "exp": math.exp,
          "log": math.log, "abs": abs, "asin": math.asin, "acos": math.acos, "atan": math.atan}
_CONSTS = {"pi": math.pi}
_BINOPS = {ast.Add: lambda a, b: a + b, ast.Sub: lambda a, b: a - b, ast.Mult: lambda a, b: a * b,
           ast.Div: lambda a, b: a / b, ast.Pow: lambda a, b: a ** b}


def eval_constant(expr: str) -> float:
    """Value of a constant FunctionExpr component; variables (x, y, z, t) are not supported."""
    src = expr.strip().replace("^", "**")
    tree = ast.parse(src, mode="eval")

    def ev(n):
        if isinstance(n, ast.Expression):
            return ev(n.body)
        if isinstance(n, ast.Constant) and isinstance(n.value, (int, float)):
            return float(n.value)
        if isinstance(n, ast.UnaryOp) and isinstance(n.op, (ast.USub, ast.UAdd)):
            v = ev(n.operand)
            return -v if isinstance(n.op, ast.USub) else v
        if isinstance(n, ast.BinOp) and type(n.op) in _BINOPS:
            return _BINOPS[type(n.op)](ev(n.left), ev(n.right))
        if isinstance(n, ast.Name) and n.id in _CONSTS:
            return _CONSTS[n.id]
        if isinstance(n, ast.Call) and isinstance(n.func, ast.Name) and n.func.id in _FUNCS and not n.keywords:
            return float(_FUNCS[n.func.id](*[ev(a) for a in n.args]))
        if isinstance(n, ast.Name):
            raise NotImplementedError(f"non-constant function '{expr.strip()}' (variable {n.id})")
        raise NotImplementedError(f"unsupported expression '{expr.strip()}'")
    return ev(tree)


def _function_values(el) -> np.ndarray:
    """Values of a FunctionExpr element: vector (<c> children) or scalar text."""
    cs = el.findall("c")
    if cs:
        return np.array([eval_constant(c.text or "0") for c in cs])
    return np.array([eval_constant(el.text or "0")])


def _numbers(text) -> np.ndarray:
    return np.array([float(v) for v in (text or "").split()], dtype=np.float64)


def _matrix(el) -> np.ndarray:
    r, c = int(el.get("rows")), int(el.get("cols"))
    v = _numbers(el.text)
    if v.size != r * c:
        raise ValueError(f"Matrix id={el.get('id')}: {v.size} values for {r}x{c}")
    # gsFileData matrices are written row by row
    return v.reshape(r, c) if r * c else np.zeros((r, c))


# -------------------------------------------------------------------------------------------
# B-spline refinement (exact, by interpolation in the nested space)
# -------------------------------------------------------------------------------------------
def elevate_knots(U: np.ndarray) -> np.ndarray:
    """Knot vector of gsBSplineBasis::degreeElevate(1): every distinct knot once more."""
    vals, mult = np.unique(U, return_counts=True)
    return np.repeat(vals, mult + 1)


def refine_knots(U: np.ndarray) -> np.ndarray:
    """Knot vector of uniformRefine(1): the midpoint of every nonzero span inserted once."""
    vals = np.unique(U)
    mids = 0.5 * (vals[:-1] + vals[1:])
    return np.sort(np.concatenate([U, mids]))


def transfer(U1, U2, p1, p2, ctrl, V1, V2, q1, q2) -> np.ndarray:
    """Control net (n1*n2, 3) of the surface (U1, U2, p1, p2, ctrl) in the nested space
    (V1, V2, q1, q2): interpolation at the Greville points of the new space."""
    T = []
    for U, p, V, q in ((U1, p1, V1, q1), (U2, p2, V2, q2)):
        g = P.greville(V, q)
        Af = P.bspline_basis_matrix(V, q, g)
        Ac = P.bspline_basis_matrix(U, p, g)
        T.append(np.linalg.solve(Af, Ac))
    n1c, n2c = len(U1) - p1 - 1, len(U2) - p2 - 1
    n1f, n2f = len(V1) - q1 - 1, len(V2) - q2 - 1
    out = np.zeros((n1f * n2f, ctrl.shape[1]))
    for c in range(ctrl.shape[1]):
        C = ctrl[:, c].reshape(n2c, n1c)
        out[:, c] = (T[1] @ C @ T[0].T).ravel()
    return out


def _elevate_refine(U1, U2, p1, p2, ctrl, weights, elevate, refine):
    """Degree elevation (``elevate`` times) and uniform refinement (``refine`` times); a rational
    patch goes through its homogeneous net (w X, w)."""
    net = ctrl if weights is None else np.hstack([ctrl * weights[:, None], weights[:, None]])
    for _ in range(elevate):
        V1, V2 = elevate_knots(U1), elevate_knots(U2)
        net = transfer(U1, U2, p1, p2, net, V1, V2, p1 + 1, p2 + 1)
        U1, U2, p1, p2 = V1, V2, p1 + 1, p2 + 1
    for _ in range(refine):
        V1, V2 = refine_knots(U1), refine_knots(U2)
        net = transfer(U1, U2, p1, p2, net, V1, V2, p1, p2)
        U1, U2 = V1, V2
    if weights is None:
        return U1, U2, p1, p2, net, None
    w = net[:, 3].copy()
    return U1, U2, p1, p2, net[:, :3] / w[:, None], w


# -------------------------------------------------------------------------------------------
@dataclass
class XMLProblem:
    problem: P.PatchProblem
    options: dict = field(default_factory=dict)         # option-list id -> {key: value}
    reference_points: np.ndarray = field(default_factory=lambda: np.zeros((0, 0)))
    reference_patches: np.ndarray = field(default_factory=lambda: np.zeros((0,), dtype=int))
    reference_values: np.ndarray = field(default_factory=lambda: np.zeros((0, 0)))


def _by_id(root):
    out = {}
    for el in root:
        i = el.get("id")
        if i is not None:
            out.setdefault(int(i), []).append(el)
    return out


def _geometry(root, ids):
    g = None
    if 0 in ids:
        for el in ids[0]:
            if el.tag == "MultiPatch":
                pl = el.find("patches")
                if pl is None:
                    raise ValueError("MultiPatch without patches")
                if pl.get("type", "id_range") == "id_range":
                    a, b = (int(v) for v in pl.text.split())
                    pids = list(range(a, b + 1))
                else:
                    pids = [int(v) for v in pl.text.split()]
                if len(pids) != 1:
                    raise NotImplementedError(f"{len(pids)} patches: the device path takes one patch")
                cand = [e for e in ids.get(pids[0], []) if e.tag == "Geometry"]
                if not cand:
                    raise ValueError(f"geometry id {pids[0]} missing")
                g = cand[0]
            elif el.tag == "Geometry":
                g = el
    if g is None:
        others = sorted(int(e.get("id")) for e in root.iter("Geometry") if e.get("id") is not None)
        if len(others) > 1:
            # a file of several patches without a MultiPatch naming them (gsReadFile reads them all)
            raise NotImplementedError(f"{len(others)} patches (geometry ids {others}): the device path takes one patch")
        if len(others) == 1:
            g = next(e for e in root.iter("Geometry") if e.get("id") is not None)
        else:
            raise ValueError("no geometry in the file")
    typ = g.get("type")
    basis = g.find("Basis")
    weights = None
    if typ == "TensorNurbs2":
        w = _numbers(basis.find("weights").text)
        if not np.allclose(w, 1.0):
            weights = np.asarray(w, dtype=np.float64)
        basis = basis.find("Basis")
    elif typ != "TensorBSpline2":
        raise NotImplementedError(f"geometry type {typ}")
    kv, deg = {}, {}
    for b in basis.findall("Basis"):
        k = b.find("KnotVector")
        idx = int(b.get("index"))
        kv[idx] = _numbers(k.text)
        deg[idx] = int(k.get("degree"))
    coefs = g.find("coefs")
    if int(coefs.get("geoDim", "3")) != 3:
        raise NotImplementedError("planar geometry: the shell needs geoDim 3")
    ctrl = _numbers(coefs.text).reshape(-1, 3)
    if weights is not None and len(weights) != len(ctrl):
        raise ValueError(f"{len(weights)} weights for {len(ctrl)} control points")
    return kv[0], kv[1], deg[0], deg[1], ctrl, weights


def _material(ids):
    for el in ids.get(10, []):
        if el.tag == "MaterialMatrix":
            typ = el.get("type", "")
            if typ not in ("Linear3", "Linear"):
                raise NotImplementedError(f"material {typ}: the device path is Saint Venant-Kirchhoff (Linear3)")
            t = eval_constant(el.find("Thickness/Function").text)
            dn = el.find("Density/Function")
            rho = eval_constant(dn.text) if dn is not None else 1.0
            pars = {int(f.get("index")): eval_constant(f.text) for f in el.findall("Parameters/Function")}
            return pars[0], pars[1], t, rho
    # older layout: Function ids 10 (thickness), 11 (E), 12 (nu), 13 (density) tagged Material
    vals = {}
    for k in (10, 11, 12, 13):
        for el in ids.get(k, []):
            if el.tag == "Function":
                vals[k] = float(_function_values(el)[0])
    if 10 in vals and 11 in vals and 12 in vals:
        return vals[11], vals[12], vals[10], vals.get(13, 1.0)
    raise ValueError("no material (id 10)")


def _named_sides(root):
    """boundary name -> side numbers, from the MultiPatch's named boundary lists."""
    out = {}
    for mp in root.iter("MultiPatch"):
        for b in mp.findall("boundary"):
            nm = b.get("name")
            if nm:
                v = [int(x) for x in (b.text or "").split()]
                out[nm] = v[1::2]
    return out


def _bc_sides(bc, named):
    nm = bc.get("name")
    if nm is not None:
        if nm not in named:
            raise ValueError(f"unknown boundary name {nm}")
        return named[nm]
    v = [int(x) for x in (bc.text or "").split()]
    return v[1::2]


def _side_rows(side, n1, n2, depth):
    """Control-point indices (A = j*n1 + i) of row ``depth`` (0 = boundary) along a side."""
    if side == 1:
        return [j * n1 + depth for j in range(n2)]
    if side == 2:
        return [j * n1 + (n1 - 1 - depth) for j in range(n2)]
    if side == 3:
        return [depth * n1 + i for i in range(n1)]
    if side == 4:
        return [(n2 - 1 - depth) * n1 + i for i in range(n1)]
    raise ValueError(f"side {side}")


def _corner(corner, n1, n2):
    return {1: 0, 2: n1 - 1, 3: (n2 - 1) * n1, 4: n2 * n1 - 1}[corner]


def _parse(path: str):
    """Root element of a gsFileData file.  gismo's reader accepts an XML declaration after a
    leading comment (filedata/surface/scordelis_lo_roof_shallow.xml starts with one); a strict
    XML parser does not, so the declaration is dropped wherever it stands."""
    import re
    with open(path, "r", encoding="utf-8") as f:
        text = f.read()
    return ET.fromstring(re.sub(r"<\?xml[^>]*\?>", "", text))


def read_geometry(path: str, elevate: int = 0, refine: int = 0, with_weights: bool = False):
    """The geometry of a file that holds only a surface (gsReadFile<>(file, mp) on a file with a
    ``Geometry`` or single-patch ``MultiPatch`` id 0, as benchmarks/benchmark_Roof.cpp:146-157
    reads filedata/surface/scordelis_lo_roof_shallow.xml), degree-elevated ``elevate`` times and
    uniformly refined ``refine`` times.  Returns (p, knots1, knots2, ctrl (n1*n2, 3)), and the
    NURBS weights (None for a B-spline) as a fifth item with ``with_weights``."""
    root = _parse(path)
    U1, U2, p1, p2, ctrl, w = _geometry(root, _by_id(root))
    U1, U2, p1, p2, ctrl, w = _elevate_refine(U1, U2, p1, p2, ctrl, w, elevate, refine)
    if p1 != p2:
        raise NotImplementedError(f"degrees {p1} and {p2}: the device path takes equal degrees")
    return (p1, U1, U2, ctrl, w) if with_weights else (p1, U1, U2, ctrl)


def read(path: str, elevate: int = 0, refine: int = 0, nq: int = 0, pde: str | None = None) -> XMLProblem:
    """Read a problem file; ``elevate`` / ``refine`` as the -e / -r arguments of the reference's
    XML solvers (static_shell_XML.cpp:95-104).  With ``pde`` the geometry comes from ``path``
    and everything else from ``pde``."""
    groot = _parse(path)
    U1, U2, p1, p2, ctrl, weights = _geometry(groot, _by_id(groot))
    root = groot if pde is None else _parse(pde)
    ids = _by_id(root)
    U1, U2, p1, p2, ctrl, weights = _elevate_refine(U1, U2, p1, p2, ctrl, weights, elevate, refine)
    if p1 != p2:
        raise NotImplementedError(f"degrees {p1} and {p2}: the device path takes equal degrees")
    p = p1
    for U in (U1, U2):
        vals, mult = np.unique(U, return_counts=True)
        if mult[0] != p + 1 or mult[-1] != p + 1:
            raise NotImplementedError("knot vector is not open")
        if np.any(mult[1:-1] > 1):
            raise NotImplementedError("repeated interior knots (C^0 lines): the shell needs C^1")
    n1, n2 = len(U1) - p - 1, len(U2) - p - 1
    E, nu, t, rho = _material(ids)

    fixed = np.zeros((3, n1 * n2), dtype=bool)
    edge_loads = []
    named = _named_sides(root)
    bcs = ids.get(20, [])
    clamped = []
    for bcel in bcs:
        funcs = {int(f.get("index")): _function_values(f) for f in bcel.findall("Function")}

        def comps(el):
            c = int(el.get("component", "-1"))
            return [0, 1, 2] if c == -1 else [c]

        for bc in bcel.findall("bc"):
            typ = bc.get("type")
            sides = _bc_sides(bc, named)
            if not sides:
                continue
            fv = funcs.get(int(bc.get("function", "0")), np.zeros(1))
            if typ == "Dirichlet":
                if np.any(fv != 0.0):
                    raise NotImplementedError("inhomogeneous Dirichlet condition")
                for s in sides:
                    for c in comps(bc):
                        fixed[c, _side_rows(s, n1, n2, 0)] = True
            elif typ == "Clamped":
                clamped += [(s, c) for s in sides for c in comps(bc)]
            elif typ == "Neumann":
                q = fv if fv.size == 3 else np.array([0.0, 0.0, fv[0]])
                for s in sides:
                    edge_loads.append([SIDE_TO_EDGE[s], *q])
            else:
                raise NotImplementedError(f"boundary condition type {typ}")
        for cv in bcel.findall("cv"):
            if eval_constant(cv.text or "0") != 0.0:
                raise NotImplementedError("nonzero corner value")
            A = _corner(int(cv.get("corner")), n1, n2)
            for c in comps(cv):
                fixed[c, A] = True
    ties = []
    for s, c in clamped:
        # gsThinShellAssembler couples the second row to the boundary row (zero normal slope);
        # with the boundary row fixed that fixes the second row
        rows0, rows1 = _side_rows(s, n1, n2, 0), _side_rows(s, n1, n2, 1)
        if fixed[c, rows0].all():
            fixed[c, rows1] = True
        else:
            ties += [(c * n1 * n2 + b, c * n1 * n2 + a) for a, b in zip(rows0, rows1)]

    surface = np.zeros(3)
    for el in ids.get(21, []):
        v = _function_values(el)
        surface = v if v.size == 3 else np.array([0.0, 0.0, v[0]])
    for el in ids.get(22, []):
        if np.any(_function_values(el) != 0.0):
            raise NotImplementedError("pressure load: the device path has dead loads only")
    pts = next((_matrix(e) for e in ids.get(30, []) if e.tag == "Matrix"), np.zeros((2, 0)))
    frc = next((_matrix(e) for e in ids.get(31, []) if e.tag == "Matrix"), np.zeros((3, 0)))
    point_loads = np.zeros((0, 5))
    if pts.shape[1]:
        if frc.shape[1] != pts.shape[1]:
            raise ValueError("point load points and forces differ in number")
        point_loads = np.concatenate([pts.T, frc.T], axis=1)

    prob = P.PatchProblem(p=p, n1=n1, n2=n2, knots1=U1, knots2=U2, ctrl=np.ascontiguousarray(ctrl), E=E, nu=nu,
                          t=t, rho=rho, fixed=fixed.ravel(), surface_load=surface, point_loads=point_loads,
                          edge_loads=np.array(edge_loads, dtype=np.float64).reshape(-1, 4), nq=nq,
                          name=f"xml:{path.rsplit('/', 1)[-1]}", weights=weights,
                          ties=np.array(ties, dtype=np.int64).reshape(-1, 2) if ties else None)
    out = XMLProblem(prob)
    for k in range(90, 96):
        for el in ids.get(k, []):
            if el.tag == "OptionList":
                out.options[k] = read_options(el)
    rp = next((_matrix(e) for e in ids.get(50, []) if e.tag == "Matrix"), None)
    if rp is not None:
        out.reference_points = rp
    rpa = next((_matrix(e) for e in ids.get(51, []) if e.tag == "Matrix"), None)
    if rpa is not None:
        out.reference_patches = rpa.astype(int).ravel()
    rv = next((_matrix(e) for e in ids.get(52, []) if e.tag == "Matrix"), None)
    if rv is not None:
        out.reference_values = rv
    return out


def read_options(el) -> dict:
    """gsOptionList entries (int, real, string, bool/switch) keyed by label."""
    out = {}
    for e in el:
        lab, val = e.get("label"), e.get("value")
        if lab is None or val is None:
            continue
        if e.tag == "int":
            out[lab] = int(val)
        elif e.tag == "real":
            out[lab] = float(val)
        elif e.tag in ("bool", "switch"):
            out[lab] = val.strip().lower() in ("1", "true")
        else:
            out[lab] = val
    return out
