"""Writes tests/golden/roof_xml.npz: the benchmark_Roof problem read from the reference's own
geometry file (ref_roof_xml.py) and the answers of the reference's own gsALMCrisfield (compiled
unchanged, oracle/_ref) on it with the FP64 oracle operators.  Needs the reference tree; run from
the repository root:  python tests/golden/make_roof_xml_fixture.py"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle"), os.path.dirname(os.path.abspath(__file__))]

import oracle as O  # noqa: E402
import refsolvers as RS  # noqa: E402
import ref_roof_xml as R  # noqa: E402
from gsstructuralanalysis_gb300 import xmlio  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "roof_xml.npz")


def main():
    if not RS.available():
        raise SystemExit("the reference tree is needed (geometry file and compiled solvers)")
    O.build_oracle()
    p, U1, U2, ctrl = xmlio.read_geometry(os.path.join(RS.REF_TREE, R.GEOMETRY), R.ELEVATE, R.REFINE)
    prob = R.problem(p, U1, U2, ctrl)
    A = O.OracleAssembler(prob)
    ops = RS.Operators.from_assembler(A)
    alm = RS.ALM(ops, "Crisfield", R.ALM)
    alm.initialize(stability=True)
    Us, Ls, its, stab = [], [], [], []
    for k in range(R.STEPS):
        st = alm.step()
        if st != 0:
            raise RuntimeError(f"reference step {k}: status {st}")
        U, L = alm.solution()
        info = alm.info()
        Us.append(U); Ls.append(L); its.append(info["iterations"]); stab.append(info["stability"])
    Ulin = np.linalg.solve(A.linear().toarray(), A.force())
    np.savez_compressed(OUT, p=p, knots1=U1, knots2=U2, ctrl=ctrl, U=np.array(Us), L=np.array(Ls),
                        iterations=np.array(its), stability=np.array(stab), U_linear=Ulin)
    print("wrote", OUT, os.path.getsize(OUT), "bytes; load factors", np.round(Ls, 6))


if __name__ == "__main__":
    main()
