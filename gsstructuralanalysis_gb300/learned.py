"""Learned arc-length predictor: data generation, reduced modal basis, training.

Pipeline (all arc-length paths are computed by the library's own GPU arc-length solver):
  1. imperfection modes: the first buckling modes of the perfect shell (GPU Lanczos);
  2. training paths: Crisfield arc-length runs on shells with seeded random imperfections
     (sum of the modes, each scaled to unit max |w|, amplitudes ~ N(0, (a t)^2));
  3. reduced modal basis Phi: proper orthogonal decomposition of the path increments (method of
     snapshots), orthonormal, nm modes;
  4. dataset: features of the last four points (q = Phi^T U and lambda, newest absolute, older
     relative) -> target = correction of the cubic extrapolation inside the modal subspace;
  5. the MLP (4(nm+1) -> 256 -> 256 -> nm+1, GELU) is trained on the GPU by the library's
     forward/backward/Adam kernels.
At run time the predictor proposes U_ext + Phi dq, L_ext + dL as the corrector's start and the
plain tangent predictor takes over whenever that start does not converge.
"""
from __future__ import annotations

import time
from dataclasses import dataclass

import numpy as np

from . import problems as P

EXTRAP = np.array([4.0, -6.0, 4.0, -1.0])   # cubic extrapolation weights of P_k, P_{k-1}, P_{k-2}, P_{k-3}


def sign_weights(ncp):
    """Fixed positive weights of the control points for the sign convention of the modes.  The
    largest |w| of a mode that is antisymmetric about a mid-line is met at two mirror points with
    opposite signs, so "largest |w| positive" is decided by rounding; the sign of the weighted sum
    sum_A c_A w_A with these non-symmetric weights is not."""
    return np.random.default_rng(20240607).uniform(0.5, 1.5, size=ncp)


def sign_fixed_modes(prob, vecs):
    """Free-dof eigenvectors -> full-layout modes, sign fixed so that sum_A c_A w_A > 0 (c: fixed
    weights of ``sign_weights``)."""
    c = sign_weights(prob.ncp)
    modes = []
    for v in vecs:
        full = np.zeros(prob.ndof_full)
        full[prob.free_index()] = v
        w = full[2 * prob.ncp:]
        if float(c @ w) < 0:
            full = -full
        modes.append(full)
    return modes


def buckling_modes(G, prob, nmodes=5, shift=-0.5, scaling=1000.0, coarse=None):
    """First buckling modes of ``prob`` (GPU Lanczos, Buckling mode).  With ``coarse`` (a nested
    coarser patch of the same surface) the modes are computed there and transferred exactly into
    the spline space of ``prob``."""
    src = coarse if coarse is not None else prob
    gp = G.Problem(src)
    st, vals, vecs = G.buckling(gp, nmodes, shift=shift, scaling=scaling)
    gp.close()
    modes = sign_fixed_modes(src, vecs)
    if coarse is not None:
        modes = [P.transfer_field(coarse, m, prob) for m in modes]
    return modes, vals, st


def imperfect_problem(prob, modes, seed, amp=0.01):
    a = np.random.default_rng(seed).normal(0.0, amp * prob.t, size=len(modes))
    return P.add_imperfection(prob, modes, a)


def step_with_retry(alm, G, retries=6):
    for _ in range(retries):
        if alm.step() == G.SUCCESS:
            return True
        alm.reduceLength(0.5)
    return False


def generate_path(G, prob, alm_opts, nsteps):
    """Converged points (U, lambda) of one Crisfield path, including the undeformed start."""
    gp = G.Problem(prob)
    alm = G.ALMCrisfield(gp, alm_opts)
    alm.initialize()
    Us = [np.zeros(gp.ndof)]
    Ls = [0.0]
    for _ in range(nsteps):
        if not step_with_retry(alm, G):
            break
        Us.append(alm.solutionU())
        Ls.append(alm.solutionL())
    del alm                      # the solver's device state goes before the problem's
    gp.close()
    return np.array(Us), np.array(Ls)


def generate_paths(G, base, modes, seeds, alm_opts, nsteps, workers=8, frozen=1, Phi=None, on_done=None, tp=None):
    """Converged Crisfield paths of the imperfect shells ``seeds``, generated concurrently: each
    host thread drives its own problem (own stream, own fronts) through ``nsteps`` points.

    The corrector starts from the cubic extrapolation of the last four points (the placement
    mode with ``frozen`` iterations on the held factorisation, plain tangent steps for the first
    points and whenever a placed start fails).  Every point meets the same arc-length constraint
    and the same TolF/TolU test as the plain predictor, so the paths are the same equilibrium
    points.  With ``tp`` (a trained predictor) the placed start is the network-corrected
    extrapolation instead.  With ``Phi`` each point is stored as its modal projection
    q = Phi U (nm numbers); without, as the full vector.  Returns [(U or q, lambda)] in the order
    of ``seeds``."""
    import threading
    from concurrent.futures import ThreadPoolExecutor

    opts = dict(alm_opts, FrozenIterations=int(frozen)) if frozen else dict(alm_opts)
    gmi = frozen + 4 if frozen else 6
    lock = threading.Lock()

    def one(seed):
        gp = G.Problem(imperfect_problem(base, modes, seed))
        alm = G.ALMCrisfield(gp, opts)
        alm.initialize(stability=False)
        pred = G.Predictor(gp, None, np.zeros((0, gp.ndof))) if tp is None else make_predictor(G, gp, tp)
        U0 = np.zeros(gp.ndof)
        Us = [U0 if Phi is None else Phi @ U0]
        Ls = [0.0]
        for _ in range(nsteps):
            st, _ = pred.step(alm, guess_max_iter=gmi)
            if st != G.SUCCESS and not step_with_retry(alm, G):
                break
            U = alm.solutionU()
            Us.append(U if Phi is None else Phi @ U)
            Ls.append(alm.solutionL())
        del pred, alm
        gp.close()
        out = (np.array(Us), np.array(Ls))
        if on_done is not None:
            with lock:
                on_done(seed, out)
        return out

    with ThreadPoolExecutor(max_workers=max(1, int(workers))) as ex:
        return list(ex.map(one, seeds))


def pod_modes(paths, nm):
    """Orthonormal POD basis of the path increments (method of snapshots)."""
    S = np.concatenate([np.diff(U, axis=0) for U, _ in paths], axis=0)   # (N, n)
    C = S @ S.T
    w, V = np.linalg.eigh(C)
    order = np.argsort(w)[::-1][:nm]
    Phi = (V[:, order].T @ S) / np.sqrt(np.maximum(w[order], 1e-300))[:, None]
    Q, _ = np.linalg.qr(Phi.T)
    return Q.T.copy()


def features_targets(paths, Phi):
    """Features and targets of every point that has four predecessors and a successor.  A path
    is (U, lambda) with full vectors, or (q, lambda) with modal projections (q.shape[1] = nm)."""
    nm = Phi.shape[0]
    X, T = [], []
    for U, L in paths:
        q = U if U.shape[1] == nm else U @ Phi.T          # (N, nm)
        for k in range(3, len(U) - 1):
            f = []
            for b in range(4):
                if b == 0:
                    f.extend(q[k]); f.append(L[k])
                else:
                    f.extend(q[k - b] - q[k]); f.append(L[k - b] - L[k])
            qe = sum(EXTRAP[b] * q[k - b] for b in range(4))
            le = sum(EXTRAP[b] * L[k - b] for b in range(4))
            X.append(f)
            T.append(np.concatenate([q[k + 1] - qe, [L[k + 1] - le]]))
    return np.array(X), np.array(T)


@dataclass
class TrainedPredictor:
    Phi: np.ndarray
    net: object
    in_mean: np.ndarray
    in_std: np.ndarray
    out_mean: np.ndarray
    out_std: np.ndarray
    train_loss: float
    nsamples: int
    seconds: dict


def train(G, paths, nm=32, hidden=256, epochs=400, batch=128, lr=2e-3, seed=0, chunk=25, val_paths=1, Phi=None):
    """Train on all but the last ``val_paths`` paths, early-stop on the held-out paths, and scale
    the network's correction by the validation-optimal trust factor alpha in [0, 1]
    (alpha = 0 reduces the predictor to the cubic extrapolation).  ``Phi`` (nm x ndof) is the
    modal basis when the paths are already projected; without it the POD of the paths is used."""
    t0 = time.perf_counter()
    if Phi is None:
        Phi = pod_modes(paths, nm)
    tr, va = (paths[:-val_paths], paths[-val_paths:]) if len(paths) > val_paths else (paths, paths)
    X, T = features_targets(tr, Phi)
    Xv, Tv = features_targets(va, Phi)
    if len(X) == 0 or len(Xv) == 0:
        raise ValueError("training paths too short: every path needs at least 5 points")
    mu, sd = X.mean(0), X.std(0) + 1e-30
    omu, osd = T.mean(0), T.std(0) + 1e-30
    sd[sd < 1e-12 * np.abs(mu).max()] = 1.0
    Xn, Tn = (X - mu) / sd, (T - omu) / osd
    Xvn, Tvn = (Xv - mu) / sd, (Tv - omu) / osd
    t1 = time.perf_counter()
    net = G.MLP(X.shape[1], hidden, hidden, T.shape[1], seed=seed)

    def val_error(a=1.0):
        Y = net.forward(Xvn).astype(np.float64)
        corr = Y * osd + omu
        return np.sum((Tv - a * corr) ** 2), corr

    best = (val_error()[0], net.params(), 0)
    history = []
    for ep in range(chunk, epochs + 1, chunk):
        loss = net.train(Xn, Tn, epochs=chunk, batch=min(batch, len(X)), lr=lr, seed=seed + ep)
        ve = val_error()[0]
        history.append((ep, loss, ve))
        if ve < best[0]:
            best = (ve, net.params(), ep)
    net.set_params(best[1])
    ve, corr = val_error()
    base = np.sum(Tv ** 2)          # error of the plain cubic extrapolation on the held-out paths
    alpha = float(np.clip(np.sum(Tv * corr) / max(np.sum(corr * corr), 1e-300), 0.0, 1.0))
    t2 = time.perf_counter()
    tp = TrainedPredictor(Phi, net, mu, sd, omu * alpha, osd * alpha, history[-1][1] if history else 0.0, len(X),
                          {"prep": t1 - t0, "train": t2 - t1})
    tp.alpha = alpha
    tp.best_epoch = best[2]
    tp.val_rel_error = float(np.sqrt(np.sum((Tv - alpha * corr) ** 2) / max(base, 1e-300)))
    tp.history = history
    return tp


def make_predictor(G, gp, tp: TrainedPredictor | None, Phi=None, use_net=True):
    if tp is None:
        return G.Predictor(gp, None, np.zeros((0, gp.ndof)))
    return G.Predictor(gp, tp.net if use_net else None, tp.Phi if Phi is None else Phi, tp.in_mean, tp.in_std,
                       tp.out_mean, tp.out_std)
