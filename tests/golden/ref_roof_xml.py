"""The shallow-roof benchmark built from the reference's own geometry file.

benchmarks/benchmark_Roof.cpp (test case 1, no symmetry) reads
filedata/surface/scordelis_lo_roof_shallow.xml, elevates and refines it, pins the north and south
edges (v = 0 and v = 1, every component, :196-204), loads the centre (0.5, 0.5) with -10 in z
(:221-232), and uses E = 3102.75, nu = 0.3, t = 6.35, density 1 (:127-139).  `problem` builds that
problem from the geometry this repository's XML reader returns."""
from __future__ import annotations

import numpy as np

from gsstructuralanalysis_gb300 import problems as P

GEOMETRY = "filedata/surface/scordelis_lo_roof_shallow.xml"
ELEVATE, REFINE = 1, 3
ALM = dict(Length=0.5, TolF=1e-8, TolU=1e-6, Scaling=0.0, MaxIter=30, BifurcationMethod=0, AngleMethod=0)
STEPS = 6


def problem(p, U1, U2, ctrl):
    n1, n2 = len(U1) - p - 1, len(U2) - p - 1
    jj = np.arange(n1 * n2) // n1
    fixed = np.zeros((3, n1 * n2), dtype=bool)
    fixed[:, (jj == 0) | (jj == n2 - 1)] = True
    return P.PatchProblem(p=p, n1=n1, n2=n2, knots1=np.asarray(U1, float), knots2=np.asarray(U2, float),
                          ctrl=np.ascontiguousarray(ctrl, dtype=np.float64), E=3102.75, nu=0.3, t=6.35, rho=1.0,
                          fixed=fixed.ravel(), point_loads=np.array([[0.5, 0.5, 0.0, 0.0, -10.0]]),
                          name="benchmark-roof-xml")
