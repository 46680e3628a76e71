"""The allocation-free ALResidual entry point (klsa_al_residual_noalloc).

It exists for callers that must not allocate device memory where they need a residual -- a host
framework that owns the whole device memory pool, or a service whose device footprint is fixed
at start-up -- and keeps its element-force scratch in a fixed file-scope device array instead of
growing a buffer.  The test compares it, through the C-ABI, with the allocating
klsa_al_residual on two calls in a row (the second call reuses the shared scratch left by the
first), and checks that a problem larger than the scratch is rejected.  As the entry point
requires, every write to the input vector is complete (torch.cuda.synchronize) before the call.
This file is collected last so that a stop-at-first-failure run has already run every other test.
"""
import numpy as np
import pytest

from gsstructuralanalysis_gb300 import problems as P

pytestmark = pytest.mark.gpu


def _device_copy(torch, a):
    return torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


def test_al_residual_noalloc_matches_allocating_entry_point(lib):
    torch = pytest.importorskip("torch")
    import gsstructuralanalysis_gb300 as G
    prob = P.cylindrical_panel(m=10, p=3, load=50.0)
    gp = G.Problem(prob)
    rng = np.random.default_rng(7)
    for call, lam in enumerate((0.4, 1.3)):
        x = (1e-3 if call == 0 else 5e-3) * rng.standard_normal(gp.ndof)
        ref = gp.al_residual(x, lam)                      # allocating entry point, host vectors
        dx = _device_copy(torch, x)
        dR = torch.full_like(dx, float("nan"))
        torch.cuda.synchronize()
        st = lib.klsa_al_residual_noalloc(gp.h, dx.data_ptr(), lam, dR.data_ptr())
        assert st == 0, lib.klsa_last_error()
        R = dR.cpu().numpy()
        # same tolerance as the FP64 residual parity tests
        assert np.linalg.norm(R - ref) <= 1e-10 * np.linalg.norm(ref)


def test_al_residual_noalloc_rejects_problems_beyond_the_scratch(lib):
    torch = pytest.importorskip("torch")
    import gsstructuralanalysis_gb300 as G
    prob = P.cylindrical_panel(m=150, p=3)             # 22,500 elements x 48 > 2^20 entries
    gp = G.Problem(prob)
    dx = torch.zeros(gp.ndof, dtype=torch.float64, device="cuda")
    dR = torch.zeros_like(dx)
    torch.cuda.synchronize()
    st = lib.klsa_al_residual_noalloc(gp.h, dx.data_ptr(), 1.0, dR.data_ptr())
    assert st == -1
    assert b"at most" in lib.klsa_last_error()
