"""GPU tests of the learned predictor: MLP gradients vs the FP64 NumPy reference, training, and
arc-length paths with the learned guess (same points as the plain path, fewer tangents)."""
import numpy as np
import pytest

from gsstructuralanalysis_gb300 import learned, problems as P

pytestmark = pytest.mark.gpu


def test_mlp_gradient_matches_reference(lib):
    import gsstructuralanalysis_gb300 as G
    import mlp_ref
    shape = (12, 16, 8, 5)
    net = G.MLP(*shape, seed=3)
    rng = np.random.default_rng(4)
    p = (0.3 * rng.standard_normal(net.nparams)).astype(np.float32)
    net.set_params(p)
    X = rng.standard_normal((17, 12)).astype(np.float32)
    T = rng.standard_normal((17, 5)).astype(np.float32)
    Y = net.forward(X)
    Yr, _ = mlp_ref.forward(p.astype(np.float64), shape, X.astype(np.float64))
    assert np.abs(Y - Yr).max() <= 1e-5 * max(1.0, np.abs(Yr).max())
    loss, g = net.loss_grad(X, T)
    lr_, gr = mlp_ref.loss_grad(p.astype(np.float64), shape, X, T)
    assert abs(loss - lr_) <= 1e-5 * lr_
    assert np.linalg.norm(g - gr) <= 1e-4 * np.linalg.norm(gr)


def test_predictor_guess_matches_numpy_restatement(lib):
    """Predictor.guess against a NumPy restatement of the learned guess: projections q = Phi U of
    the last four recorded points (newest first), the 4 (nm + 1) standardised features, the
    network (mlp_ref, FP64), the destandardised correction added to the cubic extrapolation
    4 P_k - 6 P_{k-1} + 4 P_{k-2} - P_{k-3}.  Two predictors on two problems share one network
    and run from two host threads at once, as the path-generation threads do."""
    import threading
    import gsstructuralanalysis_gb300 as G
    import mlp_ref
    prob = P.cylindrical_panel(m=8, p=2, load=1.0)
    gps = [G.Problem(prob), G.Problem(prob)]
    n, nm = gps[0].ndof, 6
    rng = np.random.default_rng(3)
    Phi = np.linalg.qr(rng.standard_normal((n, nm)))[0].T.copy()
    shape = (4 * (nm + 1), 16, 16, nm + 1)
    net = G.MLP(*shape, seed=5)
    p = (0.3 * rng.standard_normal(net.nparams)).astype(np.float32)
    net.set_params(p)
    in_mu, in_sd = 0.1 * rng.standard_normal(shape[0]), 0.5 + rng.random(shape[0])
    out_mu, out_sd = 0.1 * rng.standard_normal(shape[3]), 0.5 + rng.random(shape[3])
    preds = [G.Predictor(g, net, Phi, in_mu, in_sd, out_mu, out_sd) for g in gps]
    npts = 40
    paths = [[(1e-2 * (k + 1) * rng.standard_normal(n), 0.1 * (k + 1) + 0.01 * j) for k in range(npts)]
             for j in range(2)]
    got = [[None] * npts for _ in range(2)]

    def run(j):
        for k in range(npts):
            preds[j].push(*paths[j][k])
            got[j][k] = preds[j].guess()

    threads = [threading.Thread(target=run, args=(j,)) for j in range(2)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()

    def reference(pts):
        (U0, L0), (U1, L1), (U2, L2), (U3, L3) = pts[::-1][:4]
        q = [Phi @ U for U in (U0, U1, U2, U3)]
        L = [L0, L1, L2, L3]
        f = np.concatenate([np.append(q[0], L[0])] + [np.append(q[b] - q[0], L[b] - L[0]) for b in (1, 2, 3)])
        X = ((f - in_mu) / in_sd).astype(np.float32).astype(np.float64)
        Y, _ = mlp_ref.forward(p.astype(np.float64), shape, X[None, :])
        corr = Y[0] * out_sd + out_mu
        Ug = 4 * U0 - 6 * U1 + 4 * U2 - U3 + Phi.T @ corr[:nm]
        return Ug, 4 * L0 - 6 * L1 + 4 * L2 - L3 + corr[nm], Phi.T @ corr[:nm]

    for j in range(2):
        for k in range(npts):
            g = got[j][k]
            if k < 3:
                assert g is None
                continue
            Ug, Lg, dU = reference(paths[j][:k + 1])
            assert np.linalg.norm(g[0] - Ug) <= 1e-5 * np.linalg.norm(dU) + 1e-12 * np.linalg.norm(Ug), (k, j)
            assert abs(g[1] - Lg) <= 1e-5 * max(1.0, abs(Lg)), (k, j)
    # without a network: the plain cubic extrapolation
    ext = G.Predictor(gps[0], None, Phi)
    for U, L in paths[0][:4]:
        ext.push(U, L)
    (U0, L0), (U1, L1), (U2, L2), (U3, L3) = paths[0][:4][::-1]
    Ug, Lg = ext.guess()
    assert np.linalg.norm(Ug - (4 * U0 - 6 * U1 + 4 * U2 - U3)) <= 1e-14 * np.linalg.norm(Ug)
    assert abs(Lg - (4 * L0 - 6 * L1 + 4 * L2 - L3)) <= 1e-15 * abs(Lg)


def test_mlp_training_fits_a_smooth_map(lib):
    import gsstructuralanalysis_gb300 as G
    rng = np.random.default_rng(5)
    X = rng.standard_normal((512, 8)).astype(np.float32)
    W = rng.standard_normal((8, 3))
    T = (np.tanh(X @ W) + 0.1 * X[:, :3]).astype(np.float32)
    net = G.MLP(8, 64, 64, 3, seed=1)
    l0, _ = net.loss_grad(X, T)
    loss = net.train(X, T, epochs=300, batch=64, lr=3e-3, seed=2)
    assert loss < 0.05 * l0


def _paths(G, seeds, modes, opts, nsteps):
    base = P.cylindrical_panel(m=12, p=2, load=1.0)
    return [learned.generate_path(G, learned.imperfect_problem(base, modes, s), opts, nsteps) for s in seeds]


def test_learned_predictor_same_path_fewer_tangents(lib):
    import gsstructuralanalysis_gb300 as G
    opts = dict(Length=0.0025, TolF=1e-8, TolU=1e-6, Scaling=0.0, MaxIter=25, BifurcationMethod=-1)
    base = P.cylindrical_panel(m=12, p=2, load=1.0)
    modes, _, st = learned.buckling_modes(G, base, nmodes=3, shift=-0.5)
    assert st == 0
    paths = _paths(G, [0, 1, 2], modes, opts, 40)
    tp = learned.train(G, paths, nm=16, hidden=64, epochs=300, batch=64, lr=2e-3)
    test_prob = learned.imperfect_problem(base, modes, 1000)
    results = {}
    for mode in ("plain", "extrapolation", "learned"):
        gp = G.Problem(test_prob)
        alm = G.ALMCrisfield(gp, opts)
        alm.initialize()
        pred = None if mode == "plain" else learned.make_predictor(G, gp, tp, use_net=(mode == "learned"))
        pts, used = [], 0
        for _ in range(30):
            if pred is None:
                assert alm.step() == 0
            else:
                st, u = pred.step(alm, guess_max_iter=6)
                assert st == 0
                used += u
            pts.append((alm.solutionU(), alm.solutionL()))
        results[mode] = (pts, alm.info()["n_jac"], used)
    Up, Lp = results["plain"][0][-1]
    for mode in ("extrapolation", "learned"):
        U, L = results[mode][0][-1]
        assert np.linalg.norm(U - Up) <= 1e-5 * np.linalg.norm(Up)
        assert abs(L - Lp) <= 1e-5 * abs(Lp)
        assert results[mode][2] >= 20                     # the guess is used on most steps
        assert results[mode][1] < results["plain"][1]     # fewer tangent assemblies/factorisations
    print({k: (v[1], v[2]) for k, v in results.items()})


def test_frozen_tangent_corrector_same_points(lib, oracle_mod):
    """FrozenIterations: after a placed guess the corrector first iterates on the factorisation
    the solver already holds.  The points are the points of the full-Newton run (same path, same
    arc length), and each meets the reference's force criterion when its residual is evaluated by
    the oracle.  The frozen iterations happen: they save Jacobians, or (with this small network's
    rougher guesses) add residual evaluations ahead of the same fresh Jacobians."""
    import gsstructuralanalysis_gb300 as G
    opts = dict(Length=0.0025, TolF=1e-8, TolU=1e-6, Scaling=0.0, MaxIter=25, BifurcationMethod=-1)
    base = P.cylindrical_panel(m=12, p=2, load=1.0)
    modes, _, st = learned.buckling_modes(G, base, nmodes=3, shift=-0.5)
    assert st == 0
    paths = _paths(G, [0, 1, 2], modes, opts, 40)
    tp = learned.train(G, paths, nm=16, hidden=64, epochs=300, batch=64, lr=2e-3)
    test_prob = learned.imperfect_problem(base, modes, 1000)
    oa = oracle_mod.OracleAssembler(test_prob)
    F = oa.force()
    runs = {}
    for frozen in (0, 1, 2):
        gp = G.Problem(test_prob)
        alm = G.ALMCrisfield(gp, dict(opts, FrozenIterations=frozen) if frozen else opts)
        alm.initialize()
        pred = learned.make_predictor(G, gp, tp, use_net=True)
        pts = []
        for _ in range(30):
            st, _ = pred.step(alm, guess_max_iter=frozen + 4 if frozen else 6)
            if st != 0:
                assert alm.step() == 0
            U, L = alm.solutionU(), alm.solutionL()
            pts.append((U, L))
            R = oa.al_residual(U, L)
            assert np.linalg.norm(R) <= 1e-8 * abs(L) * np.linalg.norm(F) * (1 + 1e-6)
        info = alm.info()
        runs[frozen] = (pts, info["n_jac"], info["n_res"])
    for frozen in (1, 2):
        for (U, L), (Ur, Lr) in zip(runs[frozen][0], runs[0][0]):
            assert abs(L - Lr) <= 1e-6 * abs(Lr)
            assert np.linalg.norm(U - Ur) <= 1e-5 * np.linalg.norm(Ur)
        assert runs[frozen][1] < runs[0][1] or runs[frozen][2] > runs[0][2]
    print({k: v[1:] for k, v in runs.items()})


def test_network_gains_over_extrapolation(lib):
    """What the trained network adds to the method without it.  The held-out path runs twice with
    the same placement corrector (FrozenIterations = 1: the first iteration after a placed guess
    reuses the held factorisation, as in the measured configuration): with the cubic
    extrapolation alone, and with the network's correction of it.  The network's guesses are
    closer -- its held-out error is well below the extrapolation's on a path it was not trained
    on -- so more steps finish on the held factorisation: fewer Jacobians for the same points.
    (With the full-Newton corrector both need two iterations per point, because the second one
    is what passes TolU; the gain shows in the Jacobians, not in the iteration count.)"""
    import gsstructuralanalysis_gb300 as G
    opts = dict(Length=0.0025, TolF=1e-8, TolU=1e-6, Scaling=0.0, MaxIter=25, BifurcationMethod=-1)
    base = P.cylindrical_panel(m=12, p=2, load=1.0)
    modes, _, st = learned.buckling_modes(G, base, nmodes=5, shift=-0.5)
    assert st == 0
    paths = learned.generate_paths(G, base, modes, range(24), opts, 80, workers=8)
    tp = learned.train(G, paths, nm=16, hidden=64, epochs=300, batch=64, lr=2e-3)
    assert tp.val_rel_error < 0.5, tp.val_rel_error
    test_prob = learned.imperfect_problem(base, modes, 1000)
    runs = {}
    for use_net in (False, True):
        gp = G.Problem(test_prob)
        alm = G.ALMCrisfield(gp, dict(opts, FrozenIterations=1))
        alm.initialize(stability=False)
        pred = learned.make_predictor(G, gp, tp, use_net=use_net)
        pts = []
        for _ in range(60):
            st, _ = pred.step(alm, guess_max_iter=5)
            assert st == 0
            pts.append((alm.solutionU(), alm.solutionL()))
        runs[use_net] = (pts, alm.info()["n_jac"])
    for (U, L), (Ue, Le) in zip(runs[True][0], runs[False][0]):
        assert abs(L - Le) <= 1e-6 * abs(Le)
        assert np.linalg.norm(U - Ue) <= 1e-5 * np.linalg.norm(Ue)
    print({"extrapolation_jacobians": runs[False][1], "network_jacobians": runs[True][1],
           "val_rel_error": tp.val_rel_error})
    assert runs[True][1] < runs[False][1]
