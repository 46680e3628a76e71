"""GPU vs FP64-oracle parity of the KL-shell callbacks and the named sparse solvers."""
import numpy as np
import pytest
import scipy.sparse.linalg as spla

from gsstructuralanalysis_gb300 import problems as P

pytestmark = pytest.mark.gpu

CASES = [
    ("plate", lambda: P.flat_plate(m=8, p=2)),
    ("panel-p2", lambda: P.cylindrical_panel(m=6, p=2)),
    ("panel-p3", lambda: P.cylindrical_panel(m=5, p=3)),
    ("axial-p3", lambda: P.axial_panel(m=6, p=3)),
]


def _pair(lib, oracle_mod, make):
    import gsstructuralanalysis_gb300 as G
    prob = make()
    return prob, G.Problem(prob), oracle_mod.OracleAssembler(prob)


@pytest.mark.parametrize("name,make", CASES)
def test_force_matches(lib, oracle_mod, name, make):
    prob, gp, oa = _pair(lib, oracle_mod, make)
    assert gp.ndof == oa.nfree
    F, Fr = gp.force(), oa.force()
    assert np.linalg.norm(F - Fr) <= 1e-12 * np.linalg.norm(Fr)


@pytest.mark.parametrize("name,make", CASES)
def test_residual_fp64_matches(lib, oracle_mod, name, make):
    prob, gp, oa = _pair(lib, oracle_mod, make)
    rng = np.random.default_rng(1)
    for scale in (0.0, 1e-3, 2e-2):
        x = scale * rng.standard_normal(gp.ndof)
        r, rr = gp.residual(x), oa.residual(x)
        assert np.linalg.norm(r - rr) <= 1e-10 * max(np.linalg.norm(rr), 1e-300) + 1e-12
        a, ar = gp.al_residual(x, 0.7), oa.al_residual(x, 0.7)
        assert np.linalg.norm(a - ar) <= 1e-10 * np.linalg.norm(ar)


@pytest.mark.parametrize("name,make", CASES)
@pytest.mark.parametrize("precision,tol", [(1, 1e-11), (0, 2e-5)])
def test_jacobian_matches(lib, oracle_mod, name, make, precision, tol):
    prob, gp, oa = _pair(lib, oracle_mod, make)
    rng = np.random.default_rng(2)
    x = 1e-2 * rng.standard_normal(gp.ndof)
    K = gp.jacobian(x, precision)
    Kr = oa.jacobian(x)
    assert K.nnz == Kr.nnz
    D = (K - Kr).toarray()
    # entry-wise error relative to the largest entry of the row
    rowmax = np.abs(Kr.toarray()).max(axis=1, keepdims=True)
    assert np.max(np.abs(D) / rowmax) < tol


@pytest.mark.parametrize("name,make", CASES[:2])
def test_mass_matches(lib, oracle_mod, name, make):
    prob, gp, oa = _pair(lib, oracle_mod, make)
    M, Mr = gp.mass(), oa.mass()
    assert abs(M - Mr).max() <= 1e-12 * abs(Mr).max()


@pytest.mark.parametrize("name,make", CASES)
def test_multifrontal_solve(lib, oracle_mod, name, make):
    import gsstructuralanalysis_gb300 as G
    prob, gp, oa = _pair(lib, oracle_mod, make)
    rng = np.random.default_rng(3)
    x = 1e-2 * rng.standard_normal(gp.ndof)
    Kr = oa.jacobian(x)
    b = rng.standard_normal((2, gp.ndof))
    ref = np.stack([spla.spsolve(Kr.tocsc(), bi) for bi in b])
    # FP32 factorisation alone (the Newton / arc-length tangent solve)
    s = G.SparseSolver(gp, "SimplicialLDLT")
    assert s.compute_jacobian(x) == 0
    y = s.solve(b)
    assert np.linalg.norm(y - ref) / np.linalg.norm(ref) < 1e-3
    # FP32 factorisation + FP64 refinement
    s2 = G.SparseSolver(gp, "SimplicialLDLT", {"Refinement": 10, "RefineTol": 1e-13})
    assert s2.compute_jacobian(x) == 0
    y2 = s2.solve(b)
    assert np.linalg.norm(y2 - ref) / np.linalg.norm(ref) < 1e-9


@pytest.mark.parametrize("m,p", [(32, 2), (20, 3)])
def test_solve_schedules_agree(lib, oracle_mod, m, p, monkeypatch):
    """The three schedules of the multifrontal triangular solve on one factorisation -- the
    dataflow launch (default), the level-barrier launch (KLSA_SOLVE_KERNEL=barrier) and five
    launches per level (KLSA_SOLVE_KERNEL=levels) -- with FP32 and FP64 fronts, two right-hand
    sides, against SuperLU on the oracle's tangent.  The schedules add the same tile products in
    different orders.  With FP32 fronts every result carries the FP32 factor's own error (1e-3 to
    4e-2 relative on these thin shells): each schedule must stay within three times the error of
    the five-launch solve.  With FP64 fronts a tile read before its inputs were complete would
    show at O(1), against 1e-10 required."""
    import gsstructuralanalysis_gb300 as G
    prob = P.cylindrical_panel(m=m, p=p)
    gp, oa = G.Problem(prob), oracle_mod.OracleAssembler(prob)
    rng = np.random.default_rng(11)
    x = 1e-3 * rng.standard_normal(gp.ndof)
    Kr = oa.jacobian(x).tocsc()
    b = rng.standard_normal((2, gp.ndof))
    ref = np.stack([spla.spsolve(Kr, bi) for bi in b])

    def rel(a, r):
        return np.linalg.norm(a - r) / np.linalg.norm(r)

    for prec in (32, 64):
        s = G.SparseSolver(gp, "SimplicialLDLT", {"FrontPrecision": prec, "Refinement": 0})
        assert s.compute_jacobian(x) == 0
        ys = {}
        for kern in ("dataflow", "barrier", "levels"):
            if kern == "dataflow":
                monkeypatch.delenv("KLSA_SOLVE_KERNEL", raising=False)
            else:
                monkeypatch.setenv("KLSA_SOLVE_KERNEL", kern)
            ys[kern] = s.solve(b)
        monkeypatch.delenv("KLSA_SOLVE_KERNEL", raising=False)
        tol = 1e-10 if prec == 64 else 3.0 * rel(ys["levels"], ref)
        assert prec == 64 or tol < 0.2
        for kern, y in ys.items():
            assert rel(y, ref) <= tol, (prec, kern, rel(y, ref), tol)


def test_tensor_core_trailing_update(lib, oracle_mod, monkeypatch):
    """The trailing update of the factorisation on the tensor cores (tcgen05 kind::tf32 with a
    three-term TF32 split; KLSA_UPDATE_KERNEL=tc, read when a problem's factorisation is set up)
    against the CUDA-core tiles and SuperLU.  The TF32 split drops the lo*lo term and the tensor
    core reads the lo parts as TF32, so the FP32 factor is somewhat less accurate than with FMA
    tiles (measured 1.6e-2 against 4.9e-3 relative on this shell); FP64 refinement brings both to
    1e-9."""
    import gsstructuralanalysis_gb300 as G
    prob = P.cylindrical_panel(m=32, p=2)
    oa = oracle_mod.OracleAssembler(prob)
    rng = np.random.default_rng(5)
    ys = {}
    for mode in ("tc", "fma"):
        if mode == "tc":
            monkeypatch.setenv("KLSA_UPDATE_KERNEL", "tc")
        else:
            monkeypatch.delenv("KLSA_UPDATE_KERNEL", raising=False)
        gp = G.Problem(prob)
        if mode == "tc":
            x = 1e-3 * rng.standard_normal(gp.ndof)
            b = rng.standard_normal((2, gp.ndof))
            Kr = oa.jacobian(x).tocsc()
            ref = np.stack([spla.spsolve(Kr, bi) for bi in b])
        s1 = G.SparseSolver(gp, "SimplicialLDLT", {"Refinement": 0})
        assert s1.compute_jacobian(x) == 0
        s2 = G.SparseSolver(gp, "SimplicialLDLT", {"Refinement": 10, "RefineTol": 1e-13})
        assert s2.compute_jacobian(x) == 0
        ys[mode] = (s1.solve(b), s2.solve(b))
    monkeypatch.delenv("KLSA_UPDATE_KERNEL", raising=False)

    def rel(a, r):
        return np.linalg.norm(a - r) / np.linalg.norm(r)

    e_tc, e_fma = rel(ys["tc"][0], ref), rel(ys["fma"][0], ref)
    assert e_fma < 0.2 and e_tc <= 5.0 * e_fma + 1e-6, (e_tc, e_fma)
    assert rel(ys["tc"][1], ref) < 1e-9 and rel(ys["fma"][1], ref) < 1e-9


def test_djacobian_matches(lib, oracle_mod):
    """dJacobian_t (gsStructuralAnalysisTypes.h:91-92), called with a solution update as
    gsALMBase::_computeJacobian does (gsALMBase.hpp:214-223): the oracle's tangent at x, for
    any update (the reference wraps a Jacobian_t the same way, gsALMBase.h:57-60)."""
    prob, gp, oa = _pair(lib, oracle_mod, CASES[1][1])
    rng = np.random.default_rng(5)
    x = 1e-2 * rng.standard_normal(gp.ndof)
    Kr = oa.jacobian(x)
    rowmax = np.abs(Kr.toarray()).max(axis=1, keepdims=True)
    for dx in (np.zeros(gp.ndof), 1e-3 * rng.standard_normal(gp.ndof)):
        K = gp.djacobian(x, dx)
        assert K.nnz == Kr.nnz
        assert np.max(np.abs((K - Kr).toarray()) / rowmax) < 1e-10


@pytest.mark.parametrize("m,p", [(128, 2), (48, 3)])
def test_residual_double_float_matches_fp64_kernel(lib, m, p, monkeypatch):
    """The internal force sums in double-float arithmetic on the FP32 pipes (the default) against
    the plain FP64 kernel (KLSA_RESIDUAL_FP64=1, read when a problem is created), at the
    headline's 50k dofs and at degree 3: displacements of the size met on the path, near zero
    (where the membrane strains are smallest), and vanishingly small (an iteration converging to
    the undeformed state: the kernel keeps those elements on FP64 sums, since FP32 pairs
    underflow)."""
    import gsstructuralanalysis_gb300 as G
    prob = P.cylindrical_panel(m=m, p=p, load=1.0)
    gp_df = G.Problem(prob)
    monkeypatch.setenv("KLSA_RESIDUAL_FP64", "1")
    gp_64 = G.Problem(prob)
    monkeypatch.delenv("KLSA_RESIDUAL_FP64")
    rng = np.random.default_rng(9)
    for scale in (1e-2, 1e-7, 1e-30, 1e-150):
        x = scale * rng.standard_normal(gp_df.ndof)
        r_df, r_64 = gp_df.al_residual(x, 0.7), gp_64.al_residual(x, 0.7)
        assert np.linalg.norm(r_df - r_64) <= 1e-12 * np.linalg.norm(r_64), scale
        f_df, f_64 = gp_df.al_residual(x, 0.0), gp_64.al_residual(x, 0.0)   # Fint alone
        assert np.linalg.norm(f_df - f_64) <= 1e-12 * np.linalg.norm(f_64), scale
