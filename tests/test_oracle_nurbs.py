"""Rational (NURBS) patches in the FP64 oracle and the XML reader, on CPU.

The oracle's rational basis (oracle/kl_oracle.cpp `rationalize`: R_A = w_A N_A / W and the
quotient rule for first and second derivatives) is pinned by
* unit and constant weights reproducing the B-spline assembly (R = N when W is constant);
* the tangent being the derivative of the internal force, and a rigid translation giving no
  internal force (partition of unity through the quotient rule);
* the Scordelis-Lo roof on an exact NURBS cylinder (R 25, L 50, 40 degree half-angle, E 4.32e8,
  nu 0, t 0.25, self-weight 90 per unit area, rigid diaphragms at the ends), whose free-edge
  midpoint deflection converges to the published Kirchhoff-Love value 0.3006;
* the pinched hemisphere and the pinched cylinder of the reference's own problem files
  (filedata/pde/kirchhoff_shell_hemisphere.xml and kirchhoff_shell_pinchedCylinder.xml, test
  cases 3 and 4 of examples/gsThinShell_Static_XML.cpp) on exact NURBS geometry with the files'
  symmetry conditions, whose load-point displacements converge to the published 0.0924 and
  1.8248e-5.
The device problem does not take rational patches yet and says so.
"""
import math
import os

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from gsstructuralanalysis_gb300 import problems as P, xmlio


def _panel(weights_fn):
    prob = P.cylindrical_panel(m=4, p=2, load=1.0)
    prob.surface_load = np.array([0.3, -0.2, -1.0])
    w = weights_fn(prob)
    prob.weights = None if w is None else np.asarray(w, dtype=np.float64)
    return prob


def test_unit_and_constant_weights_reproduce_bspline(oracle_mod):
    ref = oracle_mod.OracleAssembler(_panel(lambda p: None))
    rng = np.random.default_rng(2)
    u = 1e-3 * rng.standard_normal(3 * ref.prob.ncp)
    K0, f0 = ref.full_tangent_and_fint(u)
    M0, F0 = ref.full_mass(), ref.full_force()
    for c in (1.0, 2.5):
        oa = oracle_mod.OracleAssembler(_panel(lambda p: np.full(p.ncp, c)))
        K, f = oa.full_tangent_and_fint(u)
        assert abs(K - K0).max() <= 1e-12 * abs(K0).max()
        assert np.abs(f - f0).max() <= 1e-12 * np.abs(f0).max()
        assert abs(oa.full_mass() - M0).max() <= 1e-12 * abs(M0).max()
        assert np.abs(oa.full_force() - F0).max() <= 1e-12 * np.abs(F0).max()


def _rational_panel():
    rng = np.random.default_rng(7)
    return _panel(lambda p: 0.7 + 0.6 * rng.random(p.ncp))


def test_rational_tangent_is_the_derivative_of_the_internal_force(oracle_mod):
    oa = oracle_mod.OracleAssembler(_rational_panel())
    rng = np.random.default_rng(3)
    n = 3 * oa.prob.ncp
    u = 1e-2 * rng.standard_normal(n)
    K, _ = oa.full_tangent_and_fint(u)
    for _ in range(3):
        v = rng.standard_normal(n)
        h = 1e-6
        _, fp = oa.full_tangent_and_fint(u + h * v, want_K=False)
        _, fm = oa.full_tangent_and_fint(u - h * v, want_K=False)
        fd = (fp - fm) / (2 * h)
        assert np.linalg.norm(fd - K @ v) <= 1e-6 * np.linalg.norm(K @ v)


def test_rational_rigid_translation_has_no_internal_force(oracle_mod):
    oa = oracle_mod.OracleAssembler(_rational_panel())
    ncp = oa.prob.ncp
    u = np.concatenate([np.full(ncp, 0.3), np.full(ncp, -0.7), np.full(ncp, 1.1)])
    _, f = oa.full_tangent_and_fint(u, want_K=False)
    _, f_def = oa.full_tangent_and_fint(1e-3 * np.random.default_rng(1).standard_normal(3 * ncp), want_K=False)
    assert np.abs(f).max() <= 1e-10 * np.abs(f_def).max()


def _scordelis_lo_xml(path, R=25.0, L=50.0, theta_deg=40.0):
    """The roof as a gsFileData TensorNurbs2: degree 2 in both directions, the length (index 0)
    a straight line written at degree 2, the arc (index 1) a rational quadratic with the middle
    weight cos(theta) and the middle control point where the end tangents meet."""
    th = math.radians(theta_deg)
    half, rise = R * math.sin(th), R * (1.0 / math.cos(th) - math.cos(th))
    arc = [(0.0, 0.0, 1.0), (-half, rise, math.cos(th)), (-2.0 * half, 0.0, 1.0)]
    coefs, w = [], []
    for y, z, wa in arc:
        for x in (0.0, L / 2, L):
            coefs.append(f"{x} {y} {z}")
            w.append(wa)
    with open(path, "w") as f:
        f.write(f"""<?xml version="1.0" encoding="UTF-8"?>
<xml>
 <Geometry type="TensorNurbs2" id="0">
  <Basis type="TensorNurbsBasis2">
   <Basis type="TensorBSplineBasis2">
    <Basis type="BSplineBasis" index="0"><KnotVector degree="2">0 0 0 1 1 1</KnotVector></Basis>
    <Basis type="BSplineBasis" index="1"><KnotVector degree="2">0 0 0 1 1 1</KnotVector></Basis>
   </Basis>
   <weights>{' '.join(repr(v) for v in w)}</weights>
  </Basis>
  <coefs geoDim="3">{' '.join(coefs)}</coefs>
 </Geometry>
</xml>""")


def _scordelis_lo_problem(path, elevate, refine):
    p, U1, U2, ctrl, w = xmlio.read_geometry(path, elevate, refine, with_weights=True)
    n1, n2 = len(U1) - p - 1, len(U2) - p - 1
    ii = np.arange(n1 * n2) % n1
    fixed = np.zeros((3, n1 * n2), dtype=bool)
    ends = (ii == 0) | (ii == n1 - 1)
    fixed[1, ends] = True                     # rigid diaphragms: no displacement in their plane
    fixed[2, ends] = True
    fixed[0, ii == (n1 - 1) // 2] = True      # the symmetry section x = L / 2 (n1 is odd)
    return P.PatchProblem(p=p, n1=n1, n2=n2, knots1=U1, knots2=U2, ctrl=ctrl, E=4.32e8, nu=0.0, t=0.25, rho=1.0,
                          fixed=fixed.ravel(), surface_load=np.array([0.0, 0.0, -90.0]), weights=w)


def test_xml_reader_keeps_nurbs_weights_through_elevation_and_refinement(tmp_path):
    path = os.path.join(tmp_path, "roof.xml")
    _scordelis_lo_xml(path)
    p, U1, U2, ctrl, w = xmlio.read_geometry(path, 1, 2, with_weights=True)
    assert p == 3 and w is not None and len(w) == len(ctrl)
    # every point of the refined net's surface lies on the cylinder of radius 25
    n1, n2 = len(U1) - p - 1, len(U2) - p - 1
    xi = np.linspace(0.0, 1.0, 7)
    N1, N2 = P.bspline_basis_matrix(U1, p, xi), P.bspline_basis_matrix(U2, p, xi)
    Wn = (N2 @ w.reshape(n2, n1) @ N1.T)
    Y = (N2 @ (w * ctrl[:, 1]).reshape(n2, n1) @ N1.T) / Wn
    Z = (N2 @ (w * ctrl[:, 2]).reshape(n2, n1) @ N1.T) / Wn
    yc, zc = -25.0 * math.sin(math.radians(40.0)), 25.0 * math.cos(math.radians(40.0))
    r = np.hypot(Y - yc, Z + zc)
    assert np.abs(r - 25.0).max() < 1e-10


def test_scordelis_lo_roof_matches_the_published_kirchhoff_love_value(tmp_path, oracle_mod):
    path = os.path.join(tmp_path, "roof.xml")
    _scordelis_lo_xml(path)
    vals = []
    for refine in (3, 4):
        prob = _scordelis_lo_problem(path, 1, refine)
        oa = oracle_mod.OracleAssembler(prob)
        u = oa.to_full(spla.spsolve(oa.linear().tocsc(), oa.force()))
        n1, n2 = prob.n1, prob.n2
        N1 = P.bspline_basis_matrix(prob.knots1, prob.p, np.array([0.5]))[0]
        vals.append(u[2 * n1 * n2:].reshape(n2, n1)[0] @ N1)   # free edge xi2 = 0, weights 1 along it
    assert abs(vals[-1] + 0.3006) <= 0.003 * 0.3006
    assert abs(vals[-1] - vals[-2]) <= 0.005 * abs(vals[-1])


def _quarter_hemisphere_xml(path, R=10.0):
    """The closed quarter hemisphere as a TensorNurbs2 surface of revolution: direction 0 the
    azimuth (0 to 90 degrees), direction 1 the latitude (equator to the pole, where the net
    collapses to one point); both quarter circles rational quadratics with the middle weight
    cos(45 degrees), the weights of the net their products."""
    c = math.cos(math.pi / 4)
    quarter = [(1.0, 0.0, 1.0), (1.0, 1.0, c), (0.0, 1.0, 1.0)]
    coefs, w = [], []
    for r, z, wj in quarter:                 # latitude profile (radius, height)
        for ax, ay, wi in quarter:           # azimuth
            coefs.append(f"{R * r * ax!r} {R * r * ay!r} {R * z!r}")
            w.append(wi * wj)
    with open(path, "w") as f:
        f.write(f"""<?xml version="1.0" encoding="UTF-8"?>
<xml>
 <Geometry type="TensorNurbs2" id="0">
  <Basis type="TensorNurbsBasis2">
   <Basis type="TensorBSplineBasis2">
    <Basis type="BSplineBasis" index="0"><KnotVector degree="2">0 0 0 1 1 1</KnotVector></Basis>
    <Basis type="BSplineBasis" index="1"><KnotVector degree="2">0 0 0 1 1 1</KnotVector></Basis>
   </Basis>
   <weights>{' '.join(repr(v) for v in w)}</weights>
  </Basis>
  <coefs geoDim="3">{' '.join(coefs)}</coefs>
 </Geometry>
</xml>""")


def _side_row(side, k, n1, n2):
    """(i, j) of the control points in row k (0 the boundary row) from gismo side 1-4."""
    if side == 1:
        return [(k, j) for j in range(n2)]
    if side == 2:
        return [(n1 - 1 - k, j) for j in range(n2)]
    if side == 3:
        return [(i, k) for i in range(n1)]
    return [(i, n2 - 1 - k) for i in range(n1)]


def _hand_problem(path, elevate, refine, material, point_loads, dirichlet, clamped):
    """The problem of a reference problem file built by hand: ``dirichlet`` and ``clamped`` map a
    component to its sides.  "Clamped" ties the second row of control points to the boundary
    row (zero slope across the side); where the boundary row is fixed the tie fixes it too."""
    p, U1, U2, ctrl, w = xmlio.read_geometry(path, elevate, refine, with_weights=True)
    n1, n2 = len(U1) - p - 1, len(U2) - p - 1
    ncp = n1 * n2
    fixed = np.zeros((3, n2, n1), dtype=bool)
    ties = []
    for c, sides in dirichlet.items():
        for side in sides:
            for i, j in _side_row(side, 0, n1, n2):
                fixed[c, j, i] = True
    for c, sides in clamped.items():
        for side in sides:
            for (i0, j0), (i1, j1) in zip(_side_row(side, 0, n1, n2), _side_row(side, 1, n1, n2)):
                ties.append((c * ncp + j1 * n1 + i1, c * ncp + j0 * n1 + i0))
    E, nu, t = material
    return P.PatchProblem(p=p, n1=n1, n2=n2, knots1=U1, knots2=U2, ctrl=ctrl, E=E, nu=nu, t=t, rho=1.0,
                          fixed=fixed.ravel(), surface_load=np.zeros(3),
                          point_loads=np.asarray(point_loads, dtype=np.float64), weights=w,
                          ties=np.array(ties, dtype=np.int64))


def _linear_solution(oracle_mod, prob):
    """K_L q = F over the independent dofs (the oracle's u = T q for fixed and tied dofs); the
    displacement per control point (ncp x 3)."""
    oa = oracle_mod.OracleAssembler(prob)
    u = oa.to_full(spla.spsolve(oa.linear().tocsc(), oa.force()))
    return u.reshape(3, prob.ncp).T


HEMISPHERE = dict(material=(6.825e7, 0.3, 0.04), point_loads=[[0.0, 0.0, 1.0, 0.0, 0.0], [1.0, 0.0, 0.0, -1.0, 0.0]],
                  dirichlet={0: [2, 4], 1: [1, 4], 2: [4]}, clamped={0: [1], 1: [2], 2: [1, 2]})
CYLINDER = dict(material=(3e6, 0.3, 3.0), point_loads=[[1.0, 1.0, 0.0, 0.0, -0.25]],
                dirichlet={0: [2], 1: [1, 4], 2: [1, 3]}, clamped={0: [3, 4], 1: [2, 3], 2: [2, 4]})


def _pinched_hemisphere(oracle_mod, path, elevate, refine):
    """filedata/pde/kirchhoff_shell_hemisphere.xml: t 0.04, E 6.825e7, nu 0.3; unit point loads
    +x at (0, 0) and -y at (1, 0); Dirichlet x on sides 2 and 4, y on 1 and 4, z on 4 (the
    pole); clamped x on side 1, y on side 2, z on sides 1 and 2.  Returns the outward
    displacement at the +x load and the inward one at the -y load."""
    prob = _hand_problem(path, elevate, refine, **HEMISPHERE)
    u = _linear_solution(oracle_mod, prob)
    return u[0, 0], -u[prob.n1 - 1, 1]


def test_pinched_hemisphere_matches_the_published_kirchhoff_love_value(tmp_path, oracle_mod):
    path = os.path.join(tmp_path, "quarter_hemisphere.xml")
    _quarter_hemisphere_xml(path)
    vals = []
    for refine in (4, 5):                    # degree 4, 16 x 16 and 32 x 32 elements
        a, b = _pinched_hemisphere(oracle_mod, path, 2, refine)
        assert abs(a - b) <= 1e-8 * a        # the two loads see the same displacement
        vals.append(a)
    assert abs(vals[-1] - 0.0924) <= 0.002 * 0.0924
    assert abs(vals[-1] - vals[-2]) <= 0.001 * vals[-1]


def _cylinder_eighth_xml(path, R=300.0, L=600.0):
    """One eighth of the pinched cylinder as a TensorNurbs2: direction 0 along the axis x from
    the diaphragm (x = 0) to the mid-section (x = L / 2), direction 1 the quarter circle from
    (y, z) = (R, 0) to (0, R) (rational quadratic, middle weight cos(45 degrees)).  This is the
    orientation the conditions of filedata/pde/kirchhoff_shell_pinchedCylinder.xml describe:
    side 1 the rigid diaphragm, side 2 the mid-section, sides 3 and 4 the planes z = 0 and
    y = 0, the load at corner (1, 1)."""
    c = math.cos(math.pi / 4)
    coefs, w = [], []
    for y, z, wj in [(R, 0.0, 1.0), (R, R, c), (0.0, R, 1.0)]:
        for x in (0.0, L / 4, L / 2):
            coefs.append(f"{x!r} {y!r} {z!r}")
            w.append(wj)
    with open(path, "w") as f:
        f.write(f"""<?xml version="1.0" encoding="UTF-8"?>
<xml>
 <Geometry type="TensorNurbs2" id="0">
  <Basis type="TensorNurbsBasis2">
   <Basis type="TensorBSplineBasis2">
    <Basis type="BSplineBasis" index="0"><KnotVector degree="2">0 0 0 1 1 1</KnotVector></Basis>
    <Basis type="BSplineBasis" index="1"><KnotVector degree="2">0 0 0 1 1 1</KnotVector></Basis>
   </Basis>
   <weights>{' '.join(repr(v) for v in w)}</weights>
  </Basis>
  <coefs geoDim="3">{' '.join(coefs)}</coefs>
 </Geometry>
</xml>""")


def test_pinched_cylinder_matches_the_published_value(tmp_path, oracle_mod):
    """filedata/pde/kirchhoff_shell_pinchedCylinder.xml (test case 4 of
    examples/gsThinShell_Static_XML.cpp): R 300, L 600, t 3, E 3e6, nu 0.3, rigid diaphragms,
    a quarter of the unit pinching load at the one-eighth model's corner; Dirichlet x on side 2,
    y on sides 1 and 4, z on sides 1 and 3; clamped x on sides 3 and 4, y on 2 and 3, z on 2
    and 4.  The displacement under the load converges to the published 1.8248e-5."""
    path = os.path.join(tmp_path, "pinched_cylinder.xml")
    _cylinder_eighth_xml(path)
    vals = []
    for refine in (4, 5):                    # degree 4, 16 x 16 and 32 x 32 elements
        u = _linear_solution(oracle_mod, _hand_problem(path, 2, refine, **CYLINDER))
        vals.append(-u[-1, 2])
    assert abs(vals[-1] - 1.8248e-5) <= 0.003 * 1.8248e-5
    assert abs(vals[-1] - vals[-2]) <= 0.005 * vals[-1]


REFERENCE_TREE = os.environ.get("KLSA_REFERENCE_TREE", "/root/reference")


@pytest.mark.parametrize("case", ["hemisphere", "pinchedCylinder"])
def test_reference_problem_files_through_the_reader(tmp_path, oracle_mod, case):
    """The reference's own problem files read by xmlio.read(geometry, pde=file), as its XML shell
    example reads them (a geometry file and a problem file): the material, the point loads, the
    fixed dofs and the ties of the clamped symmetry sides are the hand-built problem's, and the
    oracle solves it to the same displacement."""
    from oracle import constraint_matrix
    pde = os.path.join(REFERENCE_TREE, "filedata", "pde", f"kirchhoff_shell_{case}.xml")
    if not os.path.exists(pde):
        pytest.skip("reference tree not present")
    geo = os.path.join(tmp_path, "geometry.xml")
    (_quarter_hemisphere_xml if case == "hemisphere" else _cylinder_eighth_xml)(geo)
    spec = HEMISPHERE if case == "hemisphere" else CYLINDER
    r = xmlio.read(geo, elevate=2, refine=4, pde=pde)
    hand = _hand_problem(geo, 2, 4, **spec)
    got = r.problem
    assert (got.E, got.nu, got.t) == spec["material"]
    np.testing.assert_array_equal(got.point_loads, np.asarray(spec["point_loads"]))
    assert got.ties is not None and len(got.ties)
    Tg, Th = constraint_matrix(got.fixed, got.ties), constraint_matrix(hand.fixed, hand.ties)
    assert Tg.shape == Th.shape and (Tg != Th).nnz == 0
    ug, uh = _linear_solution(oracle_mod, got), _linear_solution(oracle_mod, hand)
    assert np.abs(ug - uh).max() <= 1e-12 * np.abs(uh).max()


def test_device_problem_refuses_tied_dofs(lib, tmp_path):
    import gsstructuralanalysis_gb300 as G
    geo = os.path.join(tmp_path, "cylinder.xml")
    _cylinder_eighth_xml(geo)
    prob = _hand_problem(geo, 0, 1, **CYLINDER)
    prob.weights = None                      # keep only the ties to refuse
    with pytest.raises(NotImplementedError, match="tied dofs"):
        G.Problem(prob)
    with pytest.raises(NotImplementedError, match="tied dofs"):
        G.BatchedProblem([prob])


def test_device_problem_refuses_rational_patches(lib):
    import gsstructuralanalysis_gb300 as G
    with pytest.raises(NotImplementedError, match="rational"):
        G.Problem(_rational_panel())
