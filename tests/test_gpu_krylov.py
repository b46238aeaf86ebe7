"""FP64 FGMRES around complex64 multigrid cycles (options.krylov > 0) on the
GPU: convergence with and without restarts, batches of RHS against FP64
solves, and the per-RHS status.  On these 16^3 models with a large air
layer the complex64 preconditioner stops both mixed variants near 1e-9
(FGMRES at 1.5-2e-9, refinement at 7e-10); FP64 cycles go further, so the
tests solve to 1e-8."""
import numpy as np
import pytest

from _cases import below_sea_mask, golden_level, rel_err
from test_gpu_solver import _G, _solver

gpu = pytest.mark.gpu


@gpu
@pytest.mark.parametrize("krylov", [4, 8])
def test_fgmres_reaches_1e8_with_and_without_restarts(golden, krylov):
    g = golden("tiny_aniso")
    G = _G()
    s = _solver(g, precision=G.PREC_MIXED, ncycle=80, tol=1e-8, krylov=krylov)
    x, h, st = s.solve(g["b_f0"][None])
    assert st[0]["status"] == "ok", st
    assert st[0]["rel"] <= 1e-8
    s64 = _solver(g, precision=G.PREC_FP64, ncycle=120, tol=1e-12)
    x64, h64, _ = s64.solve(g["b_f0"][None])
    n = tuple(int(v) for v in g["n"])
    assert rel_err(x[0], x64[0], below_sea_mask(n, g["x3"])) < 1e-5
    assert rel_err(h[0], h64[0]) < 1e-5


@gpu
def test_fgmres_batch_matches_fp64(golden):
    """Forward and adjoint RHS at two frequencies: each RHS keeps its own
    restart state, and the batch result is the FP64 solution."""
    g = golden("tiny_layered")
    G = _G()
    n, xx, raw, om = golden_level(g)
    bs = np.stack([g["b_f0"], g["badj_f0"], g["b_f0"], g["badj_f0"]])
    oms = np.array([om, om, 0.5 * om, 0.5 * om], np.float32)
    mk = lambda **o: G.Solver(n, *[v.astype(np.float32) for v in xx], raw[None], oms,
                              op=np.zeros(4, np.int32), options=G.Options(**o))
    xb, hb, stb = mk(precision=G.PREC_MIXED, ncycle=80, tol=1e-8, krylov=6).solve(bs)
    x64, h64, st64 = mk(precision=G.PREC_FP64, ncycle=150, tol=1e-12).solve(bs)
    sea = below_sea_mask(n, g["x3"])
    for r in range(4):
        assert stb[r]["status"] == "ok", stb[r]
        assert stb[r]["rel"] <= 1e-8
        assert rel_err(xb[r], x64[r], sea) < 1e-5
        assert rel_err(hb[r], h64[r]) < 1e-5


@gpu
def test_fgmres_nonfinite_rhs_reports_status(golden):
    g = golden("tiny_layered")
    G = _G()
    b = np.stack([g["b_f0"], g["b_f0"]])
    b[1, 100] = np.nan
    n, xx, raw, om = golden_level(g)
    s = G.Solver(n, *[v.astype(np.float32) for v in xx], raw[None], np.full(2, om, np.float32),
                 op=np.zeros(2, np.int32),
                 options=G.Options(precision=G.PREC_MIXED, ncycle=40, tol=1e-8, krylov=8))
    x, h, st = s.solve(b)
    assert st[0]["status"] == "ok"
    assert st[1]["status"] == "nonfinite"
