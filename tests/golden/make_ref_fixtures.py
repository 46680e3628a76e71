"""Writes tests/golden/ref_solvers.npz: the answers of the reference's own solver code.

Runs every case of ref_cases.py through oracle/_ref/libref_solvers.so -- the reference's
gsStaticNewton, gsALM* and gsModalSolver compiled unchanged from its source tree against the
test-only stand-in in oracle/refshim/ -- with the FP64 KL-shell oracle as the operators.  Needs the
reference tree (it builds the library from it); run from the repository root:

    python tests/golden/make_ref_fixtures.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle"), os.path.dirname(os.path.abspath(__file__))]

import oracle as O  # noqa: E402
import refsolvers as RS  # noqa: E402
import ref_cases as C  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "ref_solvers.npz")


def run_alm(case, A):
    ops = RS.Operators.from_assembler(A)
    alm = RS.ALM(ops, case["method"], case["options"])
    alm.initialize(stability=case["options"].get("BifurcationMethod", -1) >= 0)
    n = ops.n
    out = {"U": [], "L": [], "iterations": [], "status": [], "stability": [], "stability_change": [],
           "guess_U": [], "guess_L": []}
    U_prev, L_prev = np.zeros(n), 0.0
    U, L = np.zeros(n), 0.0
    for k in range(case["steps"]):
        if case["kind"] == "alm_guess" and k >= 2:
            Ug, Lg = C.guesses(U_prev, L_prev, U, L, k, n)
            alm.set_initial_guess(Ug, Lg)
            out["guess_U"].append(Ug)
            out["guess_L"].append(Lg)
        st = alm.step()
        U_prev, L_prev = U, L
        U, L = alm.solution()
        info = alm.info()
        if case["options"].get("BifurcationMethod", -1) < 0:
            # without a stability method gsALMBase never sets m_indicator or m_stability
            # (gsALMBase.hpp:97-103, 381, 613-614): the flags would be uninitialised memory
            info["stability"] = info["stability_change"] = 0.0
        for key, v in (("U", U), ("L", L), ("iterations", info["iterations"]), ("status", st),
                       ("stability", info["stability"]), ("stability_change", info["stability_change"])):
            out[key].append(v)
        if st != 0:
            raise RuntimeError(f"reference step {k} failed with status {st}")
    return out


def run_newton(case, A):
    F = A.force()
    load = {"L": 0.0}
    ops = RS.Operators(len(F), F, A.jacobian, lambda x, lam: A.fint(x) - lam * F, lambda x: load["L"] * F - A.fint(x))
    N = RS.StaticNewton(ops, case["options"])
    out = {"U": [], "iterations": [], "status": []}
    for L in case["loads"]:
        load["L"] = L
        st = N.solve()
        out["U"].append(N.solution())
        out["iterations"].append(N.iterations())
        out["status"].append(st)
    return out


def run_eigen(case, A):
    K, M = A.linear().toarray(), A.mass().toarray()
    st, vals, vecs = RS.eigen_dense("modal", K, M, case["options"])
    stp, valp, vecp = RS.eigen_dense("modal", K, M, case["options"], power=True)
    return {"values": vals, "vectors": vecs, "status": [st], "power_value": valp, "power_vector": vecp[:, 0],
            "power_status": [stp]}


def main():
    if not RS.available():
        raise SystemExit("the reference tree is needed to build oracle/_ref/libref_solvers.so")
    O.build_oracle()
    arrays = {}
    for name, case in C.CASES.items():
        A = O.OracleAssembler(C.build(case))
        res = {"alm": run_alm, "alm_guess": run_alm, "newton": run_newton, "eigen": run_eigen}[case["kind"]](case, A)
        for k, v in res.items():
            if isinstance(v, list) and len(v) == 0:
                continue
            arrays[f"{name}/{k}"] = np.asarray(v)
        print(name, {k: np.asarray(v).shape for k, v in res.items()})
    np.savez_compressed(OUT, **arrays)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
