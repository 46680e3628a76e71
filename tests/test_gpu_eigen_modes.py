"""The five operator modes of gsEigenProblemBase::computeSparse (gsEigenProblemBase.hpp:54-215:
Cholesky, RegularInverse, ShiftInvert, Buckling, Cayley) and its selectionRule / sortRule options
(gsEigenProblemBase.h:55-84), on a small roof's modal pencil (distinct eigenvalues) whose whole
spectrum the dense FP64 eigensolver gives from the oracle's matrices: each mode must return
exactly the eigenvalues its rule selects, in the order its sort rule asks for.  The regular modes
(Lanczos on B^-1 A) converge slowly at the low end of a stiff shell's spectrum, so they run with
a Krylov space as large as the pencil; the shift modes run with the usual ncv = 4 nev."""
import numpy as np
import pytest

from gsstructuralanalysis_gb300 import problems as P

pytestmark = pytest.mark.gpu

LARGEST_MAGN, LARGEST_ALGE, SMALLEST_MAGN, SMALLEST_ALGE, BOTH_ENDS = 0, 3, 4, 7, 8


@pytest.fixture(scope="module")
def pencil(lib, oracle_mod):
    import gsstructuralanalysis_gb300 as G
    import scipy.linalg as sla
    prob = P.cylindrical_panel(m=4, p=2)
    oa = oracle_mod.OracleAssembler(prob)
    w = sla.eigh(oa.linear().toarray(), oa.mass().toarray(), eigvals_only=True)
    return G, G.Problem(prob), w


def _run(G, gp, mode, sel, srt, nev, shift, ncv_fac=4):
    opts = {"solver": mode, "selectionRule": sel, "sortRule": srt, "tolerance": 1e-11, "maxRestarts": 2000,
            "ncvFac": ncv_fac}
    st, vals, _ = G.modal(gp, nev, shift=shift, options=opts, vectors=False)
    assert st == 0, (mode, sel, st)
    return vals


def _expect(w, key, nev, largest):
    idx = np.argsort(key(w))
    idx = idx[::-1] if largest else idx
    return w[idx[:nev]]


@pytest.mark.parametrize("mode", [0, 1])
def test_regular_modes(pencil, mode):
    G, gp, w = pencil
    full = -(-len(w) // 4)            # ncv = ncvFac * nev reaches the pencil's size
    # SmallestMagn of nu = lambda (shift 0): the lowest frequencies; LargestAlge: the highest
    lo = _run(G, gp, mode, SMALLEST_MAGN, SMALLEST_ALGE, 4, 0.0, full)
    np.testing.assert_allclose(lo, np.sort(w)[:4], rtol=1e-8)
    hi = _run(G, gp, mode, LARGEST_ALGE, LARGEST_ALGE, 3, 0.0, full)
    np.testing.assert_allclose(hi, np.sort(w)[::-1][:3], rtol=1e-8)
    both = _run(G, gp, mode, BOTH_ENDS, SMALLEST_ALGE, 4, 0.0, full)
    np.testing.assert_allclose(both, np.sort(np.concatenate([np.sort(w)[:2], np.sort(w)[-2:]])), rtol=1e-8)


@pytest.mark.parametrize("mode", [2, 4])
def test_shift_modes_select_around_the_shift(pencil, mode):
    G, gp, w = pencil
    sigma = 0.5 * (np.sort(w)[6] + np.sort(w)[7])
    near = _run(G, gp, mode, LARGEST_MAGN, SMALLEST_MAGN, 4, sigma)
    exp = _expect(w, lambda x: np.abs(x - sigma), 4, largest=False)
    np.testing.assert_allclose(np.sort(near), np.sort(exp), rtol=1e-8)
    assert np.all(np.diff(np.abs(near)) >= 0)          # sortRule SmallestMagn
    if mode == 2:
        # LargestAlge of nu = 1/(lambda - sigma): the eigenvalues just above sigma
        above = _run(G, gp, mode, LARGEST_ALGE, LARGEST_ALGE, 3, sigma)
        np.testing.assert_allclose(np.sort(above), np.sort(w[w > sigma])[:3], rtol=1e-8)
        assert np.all(np.diff(above) <= 0)             # sortRule LargestAlge
        # SmallestAlge of nu: the eigenvalues just below sigma
        below = _run(G, gp, mode, SMALLEST_ALGE, LARGEST_MAGN, 3, sigma)
        np.testing.assert_allclose(np.sort(below), np.sort(w[w < sigma])[-3:], rtol=1e-8)
        assert np.all(np.diff(np.abs(below)) <= 0)     # sortRule LargestMagn


def test_unknown_rules_are_rejected(pencil):
    G, gp, _ = pencil
    for opts in ({"solver": 2, "selectionRule": 2}, {"solver": 2, "sortRule": 6}, {"solver": 7}):
        with pytest.raises(G.KLSAError):
            G.modal(gp, 2, shift=1.0, options=opts)
