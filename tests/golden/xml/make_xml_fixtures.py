"""Writes the XML problem fixtures of tests/test_xml_input.py: the clamped plate and the
point-loaded roof of gsstructuralanalysis_gb300.problems as coarse single-element patches in
the reference's gsFileData layout (geometry, material id 10, boundary conditions id 20, loads
ids 21/22/30-32, reference points ids 50-52, option lists ids 91/93).

Run from the repository root: python tests/golden/xml/make_xml_fixtures.py
"""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.dirname(HERE))))

from gsstructuralanalysis_gb300 import problems as P  # noqa: E402


def geometry(gid, p, ctrl):
    kv = " ".join(["0"] * (p + 1) + ["1"] * (p + 1))
    rows = "\n".join("    %.17g %.17g %.17g" % tuple(c) for c in ctrl)
    return f"""<Geometry type="TensorBSpline2" id="{gid}">
  <Basis type="TensorBSplineBasis2">
    <Basis type="BSplineBasis" index="0"><KnotVector degree="{p}">{kv}</KnotVector></Basis>
    <Basis type="BSplineBasis" index="1"><KnotVector degree="{p}">{kv}</KnotVector></Basis>
  </Basis>
  <coefs geoDim="3">
{rows}
  </coefs>
</Geometry>"""


STATIC_OPTIONS = """<OptionList id="91">
  <real label="tol" desc="Relative tolerance" value="1e-10"/>
  <int label="maxIt" desc="Maximum number of iterations" value="30"/>
  <real label="Relaxation" desc="Relaxation" value="1"/>
  <string label="Solver" desc="Sparse solver" value="SimplicialLDLT"/>
</OptionList>"""


def plate():
    ctrl = [(0, 0, 0), (1, 0, 0), (0, 1, 0), (1, 1, 0)]
    return f"""<?xml version="1.0" encoding="UTF-8"?>
<xml>
<MultiPatch parDim="2" id="0">
  <patches type="id_range">700 700</patches>
</MultiPatch>
{geometry(700, 1, ctrl)}
<MaterialMatrix type="Linear3" id="10">
  <Thickness><Function type="FunctionExpr" dim="3" index="0">1e-2</Function></Thickness>
  <Density><Function type="FunctionExpr" dim="3" index="0">1</Function></Density>
  <Parameters>
    <Function type="FunctionExpr" dim="3" index="0">1e7</Function>
    <Function type="FunctionExpr" dim="3" index="1">0.3</Function>
  </Parameters>
</MaterialMatrix>
<boundaryConditions id="20" multipatch="0">
  <Function type="FunctionExpr" dim="3" index="0">0</Function>
  <bc type="Dirichlet" function="0" unknown="0" component="-1">
    0 1
    0 2
    0 3
    0 4
  </bc>
  <bc type="Clamped" function="0" unknown="0" component="2">
    0 1
    0 2
    0 3
    0 4
  </bc>
  <bc type="Collapsed" function="0" unknown="0" component="2">
  </bc>
</boundaryConditions>
<Function type="FunctionExpr" id="21" tag="Loads" dim="3">
  <c> 0 </c>
  <c> 0 </c>
  <c> 2^0 </c>
</Function>
<Function type="FunctionExpr" id="22" tag="Loads" dim="3">0</Function>
<Matrix rows="2" cols="0" id="30" tag="Loads"></Matrix>
<Matrix rows="3" cols="0" id="31" tag="Loads"></Matrix>
{STATIC_OPTIONS}
</xml>
"""


def roof():
    U1, U2, ctrl = P._panel_ctrl(2, 1, 1, 2.5, 0.2, 2.5)
    return f"""<?xml version="1.0" encoding="UTF-8"?>
<xml>
<MultiPatch parDim="2" id="0">
  <patches type="id_range">5 5</patches>
  <boundary name="free">
    5 1
    5 2
  </boundary>
  <boundary name="straight">
    5 3
    5 4
  </boundary>
</MultiPatch>
{geometry(5, 2, ctrl)}
<MaterialMatrix type="Linear3" id="10">
  <Thickness><Function type="FunctionExpr" dim="3" index="0">0.01</Function></Thickness>
  <Density><Function type="FunctionExpr" dim="3" index="0">1.0</Function></Density>
  <Parameters>
    <Function type="FunctionExpr" dim="3" index="0">3.10275e9</Function>
    <Function type="FunctionExpr" dim="3" index="1">0.3</Function>
  </Parameters>
</MaterialMatrix>
<boundaryConditions id="20" multipatch="0">
  <Function type="FunctionExpr" dim="3" index="0">0</Function>
  <bc type="Dirichlet" function="0" unknown="0" component="-1" name="straight">
  </bc>
</boundaryConditions>
<Function type="FunctionExpr" id="21" tag="Loads" dim="3">
  <c>0</c>
  <c>0</c>
  <c>0</c>
</Function>
<Matrix rows="2" cols="1" id="30" tag="Loads">
  0.5
  0.5
</Matrix>
<Matrix rows="3" cols="1" id="31" tag="Loads">
  0
  0
  -1
</Matrix>
<Matrix rows="1" cols="1" id="32" tag="Loads">
  0
</Matrix>
<Matrix rows="2" cols="1" id="50">
  0.5
  0.5
</Matrix>
<Matrix rows="1" cols="1" id="51">
  0
</Matrix>
<Matrix rows="0" cols="0" id="52">
</Matrix>
{STATIC_OPTIONS}
<OptionList id="93">
  <string label="Solver" desc="Sparse linear solver" value="SimplicialLDLT"/>
  <int label="MaxIter" desc="Maximum iterations" value="100"/>
  <real label="Length" desc="Arclength" value="5e-3"/>
  <real label="Scaling" desc="Scaling factor" value="0"/>
  <real label="TolF" desc="Tolerance" value="1e-8"/>
  <real label="TolU" desc="Tolerance" value="1e-6"/>
  <bool label="AdaptiveLength" desc="Adaptive length" value="0"/>
  <int label="BifurcationMethod" desc="Bifurcation method" value="-1"/>
</OptionList>
</xml>
"""


if __name__ == "__main__":
    for name, text in (("plate_clamped.xml", plate()), ("roof_point_load.xml", roof())):
        with open(os.path.join(HERE, name), "w") as f:
            f.write(text)
