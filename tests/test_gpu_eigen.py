"""Shift-invert Lanczos (buckling and modal pencils) vs scipy ARPACK on the oracle's FP64
matrices, and the simply-supported plate frequencies (examples/gsThinShell_Modal.cpp:333)."""
import numpy as np
import pytest

from gsstructuralanalysis_gb300 import problems as P

pytestmark = pytest.mark.gpu


def test_modal_plate_known_answer(lib, oracle_mod):
    import gsstructuralanalysis_gb300 as G
    prob = P.flat_plate(m=16, p=3, E=1.0, t=0.01, rho=1.0, bc="simply", pressure=0.0)
    gp, oa = G.Problem(prob), oracle_mod.OracleAssembler(prob)
    st, vals, vecs = G.modal(gp, nev=6, shift=0.0)
    assert st == 0
    # dense generalized eigensolve of the oracle's FP64 matrices: it cannot miss a copy of the
    # plate's double eigenvalues (an ARPACK run from a random start vector sometimes does)
    import scipy.linalg as sla
    ref = sla.eigh(oa.linear().toarray(), oa.mass().toarray(), eigvals_only=True, subset_by_index=[0, 5])
    np.testing.assert_allclose(np.sort(vals), np.sort(ref), rtol=1e-6)
    D = prob.E * prob.t ** 3 / (12 * (1 - prob.nu ** 2))
    c = np.pi ** 2 * np.sqrt(D / (prob.rho * prob.t))
    np.testing.assert_allclose(np.sort(np.sqrt(vals))[:4], np.array([2, 5, 5, 8]) * c, rtol=2e-3)
    # eigenvectors: K v = lambda M v
    K, M = oa.linear(), oa.mass()
    for lam, v in zip(vals, vecs):
        r = K @ v - lam * (M @ v)
        assert np.linalg.norm(r) <= 1e-6 * np.linalg.norm(K @ v)


def test_buckling_panel_matches_arpack(lib, oracle_mod):
    import gsstructuralanalysis_gb300 as G
    prob = P.axial_panel(m=10, p=3, line_load=1000.0)
    gp, oa = G.Problem(prob), oracle_mod.OracleAssembler(prob)
    shift = -1.0
    st, vals, vecs = G.buckling(gp, nev=5, shift=shift, scaling=1.0)
    assert st == 0
    ref, rvecs, _ = oracle_mod.buckling(oa.linear(), oa.force(), oa.jacobian, nev=5, shift=shift)
    np.testing.assert_allclose(np.sort(vals), np.sort(ref), rtol=1e-6)


def test_imperfection_modes_agree_with_oracle(lib, oracle_mod):
    """The benchmark's imperfection (buckling modes of the coarse roof, sign fixed, transferred to
    the fine spline space) is the same whether computed on the GPU or by the CPU oracle."""
    import gsstructuralanalysis_gb300 as G
    from gsstructuralanalysis_gb300 import learned
    coarse, fine = P.cylindrical_panel(m=16, p=2), P.cylindrical_panel(m=32, p=2)
    gm, gvals, st = learned.buckling_modes(G, fine, nmodes=5, shift=-0.5, scaling=1000.0, coarse=coarse)
    assert st == 0
    oa = oracle_mod.OracleAssembler(coarse)
    vals, vecs, _ = oracle_mod.buckling_dense(oa.linear(), oa.force(), oa.jacobian, nev=5, shift=-0.5, scaling=1000.0)
    om = [P.transfer_field(coarse, m, fine) for m in learned.sign_fixed_modes(coarse, vecs.T)]
    np.testing.assert_allclose(np.sort(gvals), np.sort(vals), rtol=1e-6)
    for a, b in zip(gm, om):
        assert np.abs(a - b).max() <= 1e-5 * np.abs(b).max()
