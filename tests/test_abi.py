"""CPU checks of the C-ABI library: it loads, exports every declared entry point, and its
host-only symbolic analysis (nested dissection) is exact (numpy emulation of the factorisation)."""
import ctypes
import os
import re

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from gsstructuralanalysis_gb300 import problems as P

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "klshell_gb300.h")).read()
    return sorted(set(re.findall(r"\b(klsa_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol(lib):
    import gsstructuralanalysis_gb300 as G
    syms = declared_symbols()
    assert len(syms) > 30
    for s in syms:
        assert hasattr(lib, s), s
        assert s in G.SIGNATURES, f"python binding missing for {s}"


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _nd_export(lib, prob, leaf=8):
    fx = prob.fixed.astype(np.uint8)
    full2int = np.zeros(3 * prob.ncp, dtype=np.int32)
    cap = 4 * prob.ncp + 16
    info = np.zeros(6 * cap, dtype=np.int32)
    halo = np.zeros(64 * prob.ncp * 3 + 1024, dtype=np.int32)
    nn = lib.klsa_nd_export(prob.n1, prob.n2, prob.p, _ptr(fx), leaf, _ptr(full2int), _ptr(info), _ptr(halo),
                            cap, len(halo))
    assert nn > 0
    return full2int, info[:6 * nn].reshape(nn, 6), halo


@pytest.mark.parametrize("make", [lambda: P.cylindrical_panel(m=13, p=2), lambda: P.cylindrical_panel(m=11, p=3),
                                  lambda: P.flat_plate(m=12, p=2), lambda: P.axial_panel(m=9, p=3)])
def test_nested_dissection_fronts_are_exact(lib, oracle_mod, make):
    prob = make()
    A = oracle_mod.OracleAssembler(prob)
    K = A.linear()
    F = A.force() + 1.0
    full2int, info, halo = _nd_export(lib, prob, leaf=4)
    pub2int = full2int[prob.free_index()]
    n = len(pub2int)
    assert sorted(pub2int) == list(range(n))
    Pm = sp.csr_matrix((np.ones(n), (pub2int, np.arange(n))), shape=(n, n))
    Ki = (Pm @ K @ Pm.T).tocsr()
    Fi = Pm @ F
    nn = len(info)
    children = {i: [] for i in range(nn)}
    for i in range(nn):
        if info[i, 3] >= 0:
            children[info[i, 3]].append(i)
    order = np.argsort(info[:, 4], kind="stable")
    upd, fac = {}, {}
    for nd in order:
        o, k, h, par, hgt, off = info[nd]
        ids = np.concatenate([np.arange(o, o + k), halo[off:off + h]])
        f = k + h
        sub = Ki[ids][:, ids].toarray()
        Fr = np.zeros((f, f))
        Fr[:, :k] = sub[:, :k]
        Fr[:k, :] = sub[:k, :]
        pos = {v: i for i, v in enumerate(ids)}
        for c in children[nd]:
            cids, S = upd[c]
            mp = np.array([pos[v] for v in cids])   # every child halo id is in the parent front
            Fr[np.ix_(mp, mp)] += S
        A11, A21 = Fr[:k, :k], Fr[k:, :k]
        L11 = np.linalg.cholesky(A11) if k else np.zeros((0, 0))
        L21 = np.linalg.solve(L11, A21.T).T if k else np.zeros((h, 0))
        upd[nd] = (ids[k:], Fr[k:, k:] - L21 @ L21.T)
        fac[nd] = (ids, L11, L21)
    y = Fi.copy()
    for nd in order:
        ids, L11, L21 = fac[nd]
        k = len(L11)
        yo = np.linalg.solve(L11, y[ids[:k]]) if k else np.zeros(0)
        y[ids[:k]] = yo
        y[ids[k:]] -= L21 @ yo
    x = y
    for nd in order[::-1]:
        ids, L11, L21 = fac[nd]
        k = len(L11)
        if k:
            x[ids[:k]] = np.linalg.solve(L11.T, x[ids[:k]] - L21.T @ x[ids[k:]])
    xr = spla.spsolve(Ki.tocsc(), Fi)
    assert np.linalg.norm(x - xr) / np.linalg.norm(xr) < 1e-10
