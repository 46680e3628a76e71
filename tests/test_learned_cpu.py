"""CPU checks of the learned-predictor pieces: the NumPy reference MLP backward (finite
differences), the POD basis and the cubic-extrapolation targets."""
import numpy as np

from gsstructuralanalysis_gb300 import learned


def test_reference_mlp_backward_matches_finite_differences():
    import mlp_ref
    rng = np.random.default_rng(0)
    shape = (6, 5, 4, 3)
    n = 5 * 6 + 5 + 4 * 5 + 4 + 3 * 4 + 3
    p = 0.5 * rng.standard_normal(n)
    X, T = rng.standard_normal((7, 6)), rng.standard_normal((7, 3))
    loss, g = mlp_ref.loss_grad(p, shape, X, T)
    h = 1e-6
    for i in rng.choice(n, 20, replace=False):
        e = np.zeros(n); e[i] = h
        fd = (mlp_ref.loss_grad(p + e, shape, X, T)[0] - mlp_ref.loss_grad(p - e, shape, X, T)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i]))


def test_pod_basis_is_orthonormal_and_captures_a_low_rank_path():
    rng = np.random.default_rng(1)
    n, r = 200, 3
    B = rng.standard_normal((r, n))
    paths = []
    for s in range(3):
        t = np.linspace(0, 1, 30)[:, None]
        coef = np.hstack([t, t ** 2, np.sin(3 * t + s)])
        U = coef @ B
        paths.append((U, t.ravel()))
    Phi = learned.pod_modes(paths, 5)
    assert np.allclose(Phi @ Phi.T, np.eye(5), atol=1e-10)
    D = np.diff(paths[0][0], axis=0)
    resid = D - (D @ Phi[:3].T) @ Phi[:3]
    assert np.linalg.norm(resid) <= 1e-8 * np.linalg.norm(D)


def test_cubic_path_has_zero_extrapolation_targets():
    rng = np.random.default_rng(2)
    n = 50
    A, B, C = rng.standard_normal((3, n))
    s = np.arange(12.0)[:, None]
    U = A * s + B * s ** 2 + C * s ** 3
    L = (0.3 * s + 0.01 * s ** 3).ravel()
    Phi = np.linalg.qr(rng.standard_normal((n, 8)))[0].T
    X, T = learned.features_targets([(U, L)], Phi)
    assert X.shape == (12 - 4, 4 * 9) and T.shape == (8, 9)
    assert np.abs(T).max() <= 1e-8 * np.abs(U).max()
