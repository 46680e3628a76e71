"""Device-resident time integrators (klsa_dynamic_*) against the FP64 restatement of
gsDynamicSolvers (oracle/dynamics.py) on the oracle's matrices: the same states U, V, A after a
few steps, for every integrator, linear and nonlinear, with a load ramp and Rayleigh damping."""
import numpy as np
import pytest

from gsstructuralanalysis_gb300 import problems as P

pytestmark = pytest.mark.gpu

METHODS = ["Newmark", "Bathe", "Wilson", "ExplicitEuler", "ImplicitEuler", "RK4"]
EXPLICIT = {"ExplicitEuler", "RK4"}


def _pair(G, D, oa, gp, method, nl, opts, dt, table):
    cb = D.shell_callbacks(oa, nl, opts.get("DampingMass", 0.0), opts.get("DampingStiffness", 0.0),
                           load=D.load_table(*table))
    o = {k: v for k, v in opts.items() if k not in ("DampingMass", "DampingStiffness")}
    ref = D.Dynamic(method, nl, cb["mass"], cb["damping"], cb["jacobian"], cb["residual"], cb["force"], o)
    gpu = G.Dynamic(gp, method, nonlinear=nl, options=dict(opts, DT=dt))
    gpu.setLoadTable(*table)
    return ref, gpu


def _close(a, b, rtol):
    scale = max(np.abs(b).max(), 1e-300)
    return np.abs(a - b).max() <= rtol * scale


@pytest.mark.parametrize("nl", [False, True])
@pytest.mark.parametrize("method", METHODS)
def test_integrator_matches_oracle(lib, oracle_mod, method, nl):
    import gsstructuralanalysis_gb300 as G
    import dynamics as D
    prob = P.flat_plate(m=5, p=2, E=1e7, t=0.01, rho=1.0, pressure=200.0)
    oa, gp = oracle_mod.OracleAssembler(prob), G.Problem(prob)
    dt = 1e-5 if method in EXPLICIT else 2e-3
    table = ([0.0, 2 * dt], [0.0, 1.0])              # load ramp over the first two steps
    opts = {"TolF": 1e-9, "TolU": 1e-9, "DampingMass": 5.0, "DampingStiffness": 1e-5}
    ref, gpu = _pair(G, D, oa, gp, method, nl, opts, dt, table)
    n = oa.nfree
    ref.set_state(np.zeros(n), np.zeros(n), np.zeros(n))
    for k in range(4):
        st_r = ref.step(dt)
        st_g = gpu.step()
        assert st_g == st_r == 0, (k, st_g, st_r)
        if nl and method in ("Newmark", "ImplicitEuler"):
            assert gpu.iterations() == ref.num_iterations
    assert abs(gpu.time() - 4 * dt) <= 1e-15
    U, V, A = gpu.solutionU(), gpu.solutionV(), gpu.solutionA()
    assert np.abs(ref.U).max() > 0.0
    assert _close(U, ref.U, 1e-8), np.abs(U - ref.U).max() / np.abs(ref.U).max()
    assert _close(V, ref.V, 1e-8), np.abs(V - ref.V).max() / np.abs(ref.V).max()
    if method not in EXPLICIT and method != "ImplicitEuler":
        assert _close(A, ref.A, 1e-8), np.abs(A - ref.A).max() / np.abs(ref.A).max()


def test_newmark_nonlinear_roof_large_deflection(lib, oracle_mod):
    """A point-loaded roof stepped through a large-deflection response with the nonlinear
    Newmark integrator; the Newton iteration counts agree with the oracle's step by step."""
    import gsstructuralanalysis_gb300 as G
    import dynamics as D
    prob = P.cylindrical_panel(m=6, p=2, load=20000.0, rho=7850.0)
    oa, gp = oracle_mod.OracleAssembler(prob), G.Problem(prob)
    dt = 2e-3
    opts = {"TolF": 1e-8, "TolU": 1e-8}
    ref, gpu = _pair(G, D, oa, gp, "Newmark", True, opts, dt, ([], []))
    n = oa.nfree
    ref.set_state(np.zeros(n), np.zeros(n), np.zeros(n))
    its_r, its_g = [], []
    for _ in range(6):
        assert ref.step(dt) == 0
        assert gpu.step(dt) == 0
        its_r.append(ref.num_iterations)
        its_g.append(gpu.iterations())
    assert its_g == its_r
    assert max(its_r) >= 4
    U = gpu.solutionU()
    assert _close(U, ref.U, 1e-8)
    assert np.abs(U).max() > 3 * prob.t        # about 4.8 t after 6 steps


def test_state_round_trip_and_factor_reuse(lib, oracle_mod):
    """setU/setV/setA round-trip exactly.  The linear Newmark with a constant time step reuses its
    factorisation, and refactorises when another integrator of the same problem has factorised
    a different matrix in between: its next step equals that of a fresh integrator restarted
    from the same state."""
    import gsstructuralanalysis_gb300 as G
    prob = P.flat_plate(m=4, p=2, pressure=50.0)
    gp = G.Problem(prob)
    n = gp.ndof
    rng = np.random.default_rng(3)
    U0, V0, A0 = (rng.normal(size=n) * 1e-4 for _ in range(3))
    a = G.Dynamic(gp, "Newmark", nonlinear=False, options={"DT": 1e-3})
    a.setU(U0); a.setV(V0); a.setA(A0)
    assert np.array_equal(a.solutionU(), U0) and np.array_equal(a.solutionA(), A0)
    for _ in range(3):
        assert a.step() == 0
    S = a.solutionU(), a.solutionV(), a.solutionA()
    c = G.Dynamic(gp, "Newmark", nonlinear=False, options={"DT": 5e-4})
    c.setU(U0)
    assert c.step() == 0                       # factorises M + (5e-4)^2/4 K_L in the shared fronts
    b = G.Dynamic(gp, "Newmark", nonlinear=False, options={"DT": 1e-3})
    b.setU(S[0]); b.setV(S[1]); b.setA(S[2])
    assert a.step() == 0 and b.step() == 0
    np.testing.assert_allclose(a.solutionU(), b.solutionU(), rtol=0, atol=1e-13 * np.abs(b.solutionU()).max())
