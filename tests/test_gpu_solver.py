"""Full multigrid solves on the GPU against the reference's outputs (golden
fixtures) and the CPU oracle, through the C ABI.

Parity bars (from the task's own statement of done):
  * receiver E/H within 1e-4 relative to the channel's largest amplitude and
    within 0.05 degrees in phase wherever the amplitude is above 1e-3 of
    that maximum (channels near zero by symmetry carry no phase);
  * FP64 cycles reproduce the oracle's multicolour iterates to roundoff.
"""
import numpy as np
import pytest

import oracle as O
from _cases import below_sea_mask, golden_level, rel_err

gpu = pytest.mark.gpu


def _G():
    from libemmi_mgfd_gb300 import gpu as G
    return G


def _grid(g):
    n = tuple(int(v) for v in g["n"])
    return O.Grid(n, g["x1"], g["x2"], g["x3"], g["x1s"], g["x2s"], g["x3s"], g["d1"], g["d2"],
                  g["d3"], g["sigma33"], float(g["rho_water"][0]))


def _solver(g, nrhs=1, **opt):
    G = _G()
    n, x, raw, om = golden_level(g)
    return G.Solver(n, x[0].astype(np.float32), x[1].astype(np.float32), x[2].astype(np.float32),
                    raw[None], np.full(nrhs, om, np.float32), op=np.zeros(nrhs, np.int32),
                    options=G.Options(**opt))


def receiver_parity(d, dref, chans, floor=1e-3):
    """Worst amplitude error (relative to the channel's scale) and phase error
    (degrees) over receivers.  A channel's scale is its largest amplitude but
    at least `floor` times the largest amplitude of any channel of the same
    kind (E or H): channels that vanish by symmetry (Ey, Hx on the inline of
    a 1D model) hold only roundoff, which has no meaningful relative error.
    Phase is compared where the amplitude exceeds `floor` times the scale."""
    nch = len(chans)
    d = np.asarray(d).reshape(nch, -1)
    dref = np.asarray(dref).reshape(nch, -1)
    kind_max = {}
    for c, nm in enumerate(chans):
        kind_max[nm[0]] = max(kind_max.get(nm[0], 0.0), float(np.abs(dref[c]).max()))
    worst_amp, worst_ph = 0.0, 0.0
    for c, nm in enumerate(chans):
        scale = max(float(np.abs(dref[c]).max()), floor * kind_max[nm[0]])
        if scale == 0:
            continue
        worst_amp = max(worst_amp, float(np.abs(d[c] - dref[c]).max()) / scale)
        sel = np.abs(dref[c]) > floor * scale
        if sel.any():
            ph = np.degrees(np.abs(np.angle(d[c][sel] / dref[c][sel])))
            worst_ph = max(worst_ph, float(ph.max()))
    return worst_amp, worst_ph


@gpu
def test_fp64_iterates_match_oracle_multicolour(golden):
    g = golden("tiny_layered_it3")
    G = _G()
    s = _solver(g, precision=G.PREC_FP64, ncycle=3, tol=0.0)
    x, h, st = s.solve(g["b_f0"][None])
    n, xx, raw, om = golden_level(g)
    xr, hr, nc, hist = O.gmg_solve(n, *[v.astype(np.float32) for v in xx], *raw, om, g["b_f0"],
                                   ncycle=3, tol=0.0, ordering=O.ORDER_COLOR)
    sea = below_sea_mask(n, g["x3"])
    assert rel_err(x[0], xr, sea) < 1e-11
    assert rel_err(h[0], hr) < 1e-11
    assert st[0]["cycles"] == 3


@gpu
@pytest.mark.parametrize("cycleopt,ncyc", [(1, 3), (3, 2)])
def test_fp64_v_w_cycles_match_oracle(golden, cycleopt, ncyc):
    g = golden("tiny_layered_it3")
    G = _G()
    s = _solver(g, precision=G.PREC_FP64, ncycle=ncyc, tol=0.0, cycleopt=cycleopt)
    x, h, st = s.solve(g["b_f0"][None])
    n, xx, raw, om = golden_level(g)
    xr, hr, nc, hist = O.gmg_solve(n, *[v.astype(np.float32) for v in xx], *raw, om, g["b_f0"],
                                   ncycle=ncyc, tol=0.0, ordering=O.ORDER_COLOR,
                                   cycleopt=cycleopt)
    assert rel_err(h[0], hr) < 1e-11


@gpu
@pytest.mark.parametrize("prec,krylov", [(0, 0), (1, 0)])
@pytest.mark.parametrize("name", ["tiny_layered", "tiny_aniso"])
def test_converged_receivers_match_reference(golden, name, prec, krylov):
    g = golden(name)
    # the fixture was solved by the reference to 1e-10; FP64 solves to the
    # same.  On these 16^3 models with a large air layer the complex64
    # preconditioner stops the mixed solver near 7e-10, so it solves to
    # 1e-9, far inside the 1e-4 receiver bar.
    tol = 1e-10 if prec == 0 else 1e-9
    s = _solver(g, precision=prec, ncycle=120, tol=tol, krylov=krylov)
    x, h, st = s.solve(g["b_f0"][None])
    assert st[0]["status"] == "ok", st
    assert st[0]["rel"] <= tol
    ch = str(g["chrec"]).split(",")
    rec = g["srcrec"][5:].reshape(-1, 5)
    d = O.extract_emf_data(_grid(g), rec, ch, x[0], h[0])
    amp, ph = receiver_parity(d, g["dcal"], ch)
    assert amp < 1e-4, amp
    assert ph < 0.05, ph
    # the converged fields themselves, below the sea surface and H
    n = tuple(int(v) for v in g["n"])
    assert rel_err(h[0], g["h_f0"]) < 1e-5
    assert rel_err(x[0], g["x_f0"], below_sea_mask(n, g["x3"])) < 1e-5


@gpu
def test_cycle_count_close_to_reference(golden):
    g = golden("tiny_layered")
    G = _G()
    s = _solver(g, precision=G.PREC_FP64, ncycle=80, tol=1e-10)
    x, h, st = s.solve(g["b_f0"][None])
    ref_cycles = len(g["rnorm_fwd"]) - 1
    assert abs(st[0]["cycles"] - ref_cycles) <= max(3, ref_cycles // 5)


@gpu
def test_batch_of_rhs_equals_individual_solves(golden):
    """Forward and adjoint RHS of one operator at two frequencies in one batch."""
    g = golden("tiny_layered")
    G = _G()
    n, xx, raw, om = golden_level(g)
    bs = np.stack([g["b_f0"], g["badj_f0"], g["b_f0"], g["badj_f0"]])
    oms = np.array([om, om, 0.5 * om, 0.5 * om], np.float32)
    # the default air floor depends on the batch's lowest frequency: pin it
    opt = dict(precision=G.PREC_MIXED, ncycle=80, tol=1e-8, sigma_floor=2e-4)
    s = G.Solver(n, *[v.astype(np.float32) for v in xx], raw[None], oms, op=np.zeros(4, np.int32),
                 options=G.Options(**opt))
    xb, hb, stb = s.solve(bs)
    for r in range(4):
        s1 = G.Solver(n, *[v.astype(np.float32) for v in xx], raw[None], oms[r:r + 1],
                      options=G.Options(**opt))
        x1, h1, st1 = s1.solve(bs[r:r + 1])
        assert stb[r]["status"] == "ok"
        # same arithmetic per RHS: the batch must not couple RHS (norms are
        # atomic sums, so refinement points may shift by a cycle)
        assert rel_err(xb[r], x1[0], below_sea_mask(n, g["x3"])) < 1e-6
        assert abs(stb[r]["cycles"] - st1[0]["cycles"]) <= 1


@gpu
def test_config1_64_receivers_match_reference(golden):
    """The reference's CPU-runnable configuration (101x101x51 model, 64^3
    mesh, 1 Hz, 101 receivers, Ex/Ey/Hx/Hy) in mixed precision to 1e-8."""
    g = golden("c1_layered_64")
    G = _G()
    n, xx, raw, om = golden_level(g)
    src = g["srcrec"][:5]
    b = O.inject_source(_grid(g), src, str(g["chsrc"]).split(","), om)
    s = G.Solver(n, *[v.astype(np.float32) for v in xx], raw[None], np.array([om], np.float32),
                 options=G.Options(precision=G.PREC_MIXED, ncycle=60, tol=1e-8))
    x, h, st = s.solve(b[None])
    assert st[0]["status"] == "ok", st
    ch = str(g["chrec"]).split(",")
    rec = g["srcrec"][5:].reshape(-1, 5)
    d = O.extract_emf_data(_grid(g), rec, ch, x[0], h[0])
    amp, ph = receiver_parity(d, g["dcal"], ch)
    assert amp < 1e-4, amp
    assert ph < 0.05, ph
    # both against an FP64 solve to 1e-12 (the error of each is stated)
    s64 = G.Solver(n, *[v.astype(np.float32) for v in xx], raw[None], np.array([om], np.float32),
                   options=G.Options(precision=G.PREC_FP64, ncycle=100, tol=1e-12))
    x64, h64, st64 = s64.solve(b[None])
    d64 = O.extract_emf_data(_grid(g), rec, ch, x64[0], h64[0])
    ours, _ = receiver_parity(d, d64, ch)
    ref, _ = receiver_parity(g["dcal"], d64, ch)
    print(f"receiver error vs FP64 1e-12 solve: ours {ours:.2e}, reference {ref:.2e}")
    assert ours < 1e-4 and ref < 1e-4


@gpu
def test_nonfinite_rhs_reports_status(golden):
    g = golden("tiny_layered")
    b = g["b_f0"].copy()
    b[100] = np.nan
    s = _solver(g, ncycle=10, tol=1e-8)
    x, h, st = s.solve(b[None])
    assert st[0]["status"] == "nonfinite"


@gpu
def test_stored_line_factors_give_the_same_iterates(golden):
    """Mixed cycles with the line factors kept from set-up (the default) and
    factored in every sweep: the same operations in the same order (the
    compiler may fuse multiply-adds differently in the two kernels, so
    roundoff, amplified in the air layer's curl-free E, is all that differs)."""
    g = golden("tiny_layered")
    G = _G()
    n, xx, raw, om = golden_level(g)
    bs = np.stack([g["b_f0"], g["badj_f0"], g["b_f0"]])
    oms = np.array([om, om, 0.5 * om], np.float32)
    out = {}
    for lf in (1, 0):
        s = G.Solver(n, *[v.astype(np.float32) for v in xx], raw[None], oms,
                     op=np.zeros(3, np.int32),
                     options=G.Options(precision=G.PREC_MIXED, ncycle=6, tol=0.0,
                                       sigma_floor=2e-4, line_factors=lf, line_sweep=0))
        x, h, st = s.solve(bs)
        out[lf] = (x, h, [q["cycles"] for q in st], s.device_bytes)
        s.close()
    assert out[1][3] > out[0][3]          # the factors are held
    assert out[1][2] == out[0][2] == [6, 6, 6]
    sea = below_sea_mask(n, g["x3"])
    for r in range(3):
        assert rel_err(out[1][0][r], out[0][0][r], sea) < 1e-6
        assert rel_err(out[1][1][r], out[0][1][r]) < 1e-6


@gpu
def test_fp16_line_factors_converge_like_fp32(golden):
    """Stored factors with L in fp16 (the default) against fp32 factors: the
    substitution reads 28 instead of 48 bytes per row; the smoother's line
    solves change by the fp16 rounding of L, the FP64 refinement keeps the
    answer.  Cycle counts within 10 % and the same converged fields."""
    g = golden("tiny_layered")
    G = _G()
    n, xx, raw, om = golden_level(g)
    bs = np.stack([g["b_f0"], g["badj_f0"], g["b_f0"]])
    oms = np.array([om, om, 0.5 * om], np.float32)
    out = {}
    for lf in (2, 1):
        s = G.Solver(n, *[v.astype(np.float32) for v in xx], raw[None], oms,
                     op=np.zeros(3, np.int32),
                     options=G.Options(precision=G.PREC_MIXED, ncycle=120, tol=1e-8,
                                       sigma_floor=2e-4, line_factors=lf, line_sweep=0))
        x, h, st = s.solve(bs)
        out[lf] = (x, h, st)
        s.close()
    for lf in (2, 1):
        print("line_factors", lf, [(q["status"], q["cycles"], q["rel"]) for q in out[lf][2]])
    sea = below_sea_mask(n, g["x3"])
    for r in range(3):
        assert out[2][2][r]["status"] == "ok" and out[1][2][r]["status"] == "ok"
        c2, c1 = out[2][2][r]["cycles"], out[1][2][r]["cycles"]
        assert abs(c2 - c1) <= max(2, c1 // 10), (c2, c1)
        assert rel_err(out[2][0][r], out[1][0][r], sea) < 1e-6
        assert rel_err(out[2][1][r], out[1][1][r]) < 1e-6


@gpu
def test_fp16_factor_overflow_falls_back_to_fp32():
    """Cells 10^6 times thinner along x than along y and z make the x-line
    factors' L values exceed the fp16 range: set-up detects it and keeps fp32
    factors (a normal grid keeps fp16); the solve runs on them."""
    G = _G()
    n = (8, 8, 8)
    rng = np.random.default_rng(3)
    raw = np.concatenate([10.0 ** rng.uniform(-2, 0, (3, 8, 8, 8)),
                          np.ones((1, 8, 8, 8))]).astype(np.float32)
    b = np.zeros((1, 3 * 9 ** 3), np.complex128)
    b[0, 3 * 9 ** 3 // 2] = 1.0
    fmts = {}
    for name, dx in (("normal", 100.0), ("thin", 1e-4)):
        x = [np.arange(9, dtype=np.float32) * dx, np.arange(9, dtype=np.float32) * 100.0,
             np.arange(9, dtype=np.float32) * 100.0]
        s = G.Solver(n, *x, raw[None], np.array([6.28], np.float32),
                     options=G.Options(precision=G.PREC_MIXED, ncycle=3, tol=0.0, line_sweep=0))
        fmts[name] = s.line_factor_format
        xs, hs, st = s.solve(b)
        assert np.all(np.isfinite(xs)), name
        s.close()
    assert fmts == {"normal": 1, "thin": 0}, fmts


@gpu
def test_pooled_memory_is_reused_and_trimmed(golden):
    """Solver memory comes from the device's stream-ordered pool: a second
    solver of the same size reuses what the first gave back, and
    emmi_trim_memory returns the pool's unused memory to the device."""
    import torch
    G = _G()
    g = golden("tiny_layered")
    for _ in range(2):
        s = _solver(g, ncycle=2, tol=0.0)
        s.solve(g["b_f0"][None])
        s.close()
    assert G.lib().emmi_trim_memory() == 0
    torch.cuda.synchronize()


@gpu
def test_sweep_shapes_never_change_the_result(golden):
    """Every level-0 sweep shape the autotuner chooses from (forced one at a
    time) gives the defaults' iterates bit for bit; the autotuner times the
    shapes on a new grid and a second solver of the same shape takes them
    from the process cache."""
    g = golden("tiny_layered")
    G = _G()
    n, xx, raw, om = golden_level(g)
    bs = np.stack([g["b_f0"], g["badj_f0"], g["b_f0"]])
    oms = np.array([om, om, 0.5 * om], np.float32)

    def run(autotune):
        s = G.Solver(n, *[v.astype(np.float32) for v in xx], raw[None], oms,
                     op=np.zeros(3, np.int32),
                     options=G.Options(precision=G.PREC_MIXED, ncycle=6, tol=0.0,
                                       sigma_floor=2e-4, autotune=autotune, line_sweep=0))
        x, h, st = s.solve(bs)
        shapes = s.sweep_shapes()
        s.close()
        return x, h, shapes

    x0, h0, (sh0, _) = run(0)
    assert all(sh == (64, 6, 256) for sh in sh0), sh0
    seen = set()
    for k in range(1, 11):
        x, h, (sh, tuned) = run(-k)
        assert not tuned
        seen.add(sh[0])
        assert np.array_equal(x, x0) and np.array_equal(h, h0), (k, sh)
    assert len(seen) == 10
    _, _, (sh1, tuned1) = run(1)
    x2, h2, (sh2, tuned2) = run(1)
    assert sh1 == sh2 and not tuned2
    assert np.array_equal(x2, x0)


_TUNE_CHILD = r"""
import json, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
from libemmi_mgfd_gb300 import gpu as G
n = (12, 12, 12)
rng = np.random.default_rng(5)
raw = np.concatenate([10.0 ** rng.uniform(-2, 0, (3,) + n[::-1]),
                      np.ones((1,) + n[::-1])]).astype(np.float32)
x = [np.arange(v + 1, dtype=np.float32) * 100.0 for v in n]
s = G.Solver(n, *x, raw[None], np.full(2, 6.28, np.float32), op=np.zeros(2, np.int32),
             options=G.Options(precision=G.PREC_MIXED, ncycle=2, tol=0.0, line_sweep=0))
print(json.dumps(s.sweep_shapes()))
s.close()
"""


@gpu
def test_tuned_shapes_persist_as_json(tmp_path):
    """With EMMI_TUNE_FILE the autotuner's choices outlive the process: a
    first process times the shapes and writes them as JSON, a second one
    reads them back and times nothing."""
    import json
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    path = tmp_path / "tune.json"
    env = dict(os.environ, EMMI_TUNE_FILE=str(path))
    out = []
    for _ in range(2):
        r = subprocess.run([sys.executable, "-c", _TUNE_CHILD, root], env=env,
                           capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stderr[-2000:]
        out.append(json.loads(r.stdout.strip().splitlines()[-1]))
    (sh1, tuned1), (sh2, tuned2) = out
    assert tuned1 and not tuned2 and sh1 == sh2
    doc = json.loads(path.read_text())
    entries = doc["sweep_shapes"]
    assert len(entries) >= 1
    for e in entries:
        assert e["grid"] == [12, 12, 12] and e["nrhs"] == 2 and e["rhs_threads"] in (128, 256)


@gpu
def test_config2_batch_mixed_matches_fp64_solve():
    """The batched configuration at full size -- 25 shots x 2 frequencies
    (0.25, 0.75 Hz) = 50 right-hand sides on 25 operators in one solver,
    96^3 mesh, VTI sediment, random bathymetry, a resistive box, 200
    receivers: every mixed-precision solve converges to 1e-8 and its
    receiver data agree with an FP64 solve of the same batch to 1e-10
    within 1e-4 of each channel's largest value (channels above 1e-3 of
    the batch's largest)."""
    from libemmi_mgfd_gb300 import host
    from libemmi_mgfd_gb300 import workloads as W
    G = _G()
    s = W.config2(96)
    m = host.Model.from_survey(s)
    src = s.sources.astype(np.float32).copy()
    src[:, 3:] = np.deg2rad(src[:, 3:])
    rec = s.receivers.astype(np.float32).copy()
    rec[:, 3:] = np.deg2rad(rec[:, 3:])
    grids = [m.regrid(float(p[0]), float(p[1]), float(p[2])) for p in s.sources]
    X = [np.stack([g[k] for g in grids]) for k in ("x1", "x2", "x3")]
    cells = np.stack([np.stack([g["sigma11"], g["sigma22"], g["sigma33"], g["invmur"]])
                      for g in grids])
    nf = len(s.freqs)
    om = np.array([2 * np.pi * s.freqs[r % nf] for r in range(len(src) * nf)], np.float32)
    op = np.repeat(np.arange(len(src), dtype=np.int32), nf)
    srcr = np.repeat(src, nf, axis=0)
    out = {}
    for prec, tol in ((G.PREC_MIXED, 1e-8), (G.PREC_FP64, 1e-10)):
        sv = G.Solver(s.n, *X, cells, om, op=op,
                      options=G.Options(precision=prec, tol=tol, ncycle=100),
                      rho_water=np.float32(m.rho_water()))
        d, st, _ = sv.modelling(srcr, rec, s.chsrc, s.chrec)
        sv.close()
        assert all(q["status"] == "ok" for q in st), [q["status"] for q in st]
        out[prec] = (d, np.mean([q["cycles"] for q in st]))
    d, d64 = out[G.PREC_MIXED][0], out[G.PREC_FP64][0]
    print("cycles mixed / fp64:", out[G.PREC_MIXED][1], out[G.PREC_FP64][1])
    top = np.abs(d64).max()
    worst = 0.0
    for r in range(d.shape[0]):
        for c in range(d.shape[1]):
            mx = np.abs(d64[r, c]).max()
            if mx < 1e-3 * top:
                continue
            worst = max(worst, float(np.abs(d[r, c] - d64[r, c]).max() / mx))
    print(f"largest receiver error vs FP64: {worst:.2e}")
    assert worst < 1e-4, worst


@gpu
@pytest.mark.parametrize("prec, lf", [(1, 2), (1, 1), (0, 2)])
def test_one_launch_line_sweep_gives_the_three_launch_iterates(golden, prec, lf):
    """The one-launch line sweep (default) against the three-launch sweep
    with the same multiplier arithmetic -- stored fp16 L (lf 2) or fp32
    (lf 1) for complex64 cycles, records for FP64 -- after six cycles of
    three RHS: the same operations in the same order, so only the
    compiler's multiply-add fusion differs (roundoff, amplified in the air
    layer's curl-free E: compared below the sea surface and in H)."""
    g = golden("tiny_layered")
    G = _G()
    n, xx, raw, om = golden_level(g)
    bs = np.stack([g["b_f0"], g["badj_f0"], g["b_f0"]])
    oms = np.array([om, om, 0.5 * om], np.float32)
    out = {}
    for sweep in (1, 0):
        s = G.Solver(n, *[v.astype(np.float32) for v in xx], raw[None], oms,
                     op=np.zeros(3, np.int32),
                     options=G.Options(precision=prec, ncycle=6, tol=0.0, sigma_floor=2e-4,
                                       line_factors=lf, line_sweep=sweep))
        x, h, st = s.solve(bs)
        fmt = s.line_format
        out[sweep] = (x, h, [q["cycles"] for q in st], s.last_launches)
        s.close()
        if sweep == 1:
            assert fmt == (1 if (prec == 1 and lf == 2) else 0), fmt
    assert out[1][2] == out[0][2] == [6, 6, 6]
    assert out[1][3] < out[0][3]  # one launch per colour instead of three
    sea = below_sea_mask(n, g["x3"])
    tol = 1e-6 if prec == 1 else 1e-10
    for r in range(3):
        assert rel_err(out[1][0][r], out[0][0][r], sea) < tol
        assert rel_err(out[1][1][r], out[0][1][r]) < tol


@gpu
def test_one_launch_sweep_fp16_overflow_switches_to_fp32():
    """Cells 10^6 times thinner along x than along y and z: the x-line
    multipliers leave the fp16 range during the first cycle; the solver
    notices at the next norm check, keeps fp32 multipliers from then on and
    restarts its inner cycles, so the solve stays finite and reduces its
    residual (a normal grid keeps fp16)."""
    G = _G()
    n = (8, 8, 8)
    rng = np.random.default_rng(3)
    raw = np.concatenate([10.0 ** rng.uniform(-2, 0, (3, 8, 8, 8)),
                          np.ones((1, 8, 8, 8))]).astype(np.float32)
    b = np.zeros((1, 3 * 9 ** 3), np.complex128)
    b[0, 3 * 9 ** 3 // 2] = 1.0
    fmts = {}
    for name, dx in (("normal", 100.0), ("thin", 1e-4)):
        x = [np.arange(9, dtype=np.float32) * dx, np.arange(9, dtype=np.float32) * 100.0,
             np.arange(9, dtype=np.float32) * 100.0]
        s = G.Solver(n, *x, raw[None], np.array([6.28], np.float32),
                     options=G.Options(precision=G.PREC_MIXED, ncycle=12, tol=1e-6,
                                       line_sweep=1))
        xs, hs, st = s.solve(b)
        fmts[name] = s.line_format
        assert np.all(np.isfinite(xs)), name
        assert st[0]["status"] != "nonfinite" and st[0]["rel"] < 0.5, (name, st)
        s.close()
    assert fmts == {"normal": 1, "thin": 0}, fmts


@gpu
def test_fp64_stored_line_factors_give_the_same_iterates(golden):
    """Complex128 cycles with the lines' LDL^T factors kept from set-up in
    FP64 (line_factors = 1) against refactoring every line in every sweep
    (line_factors = 0): the same operations in the same order, so the
    iterates agree to roundoff after six cycles of three RHS."""
    g = golden("tiny_layered")
    G = _G()
    n, xx, raw, om = golden_level(g)
    bs = np.stack([g["b_f0"], g["badj_f0"], g["b_f0"]])
    oms = np.array([om, om, 0.5 * om], np.float32)
    out = {}
    for lf in (1, 0):
        s = G.Solver(n, *[v.astype(np.float32) for v in xx], raw[None], oms,
                     op=np.zeros(3, np.int32),
                     options=G.Options(precision=G.PREC_FP64, ncycle=6, tol=0.0,
                                       line_factors=lf))
        x, h, st = s.solve(bs)
        out[lf] = (x, h, [q["cycles"] for q in st], s.line_factor_format)
        s.close()
    assert out[1][3] == 0 and out[0][3] == -1
    assert out[1][2] == out[0][2] == [6, 6, 6]
    sea = below_sea_mask(n, g["x3"])
    for r in range(3):
        assert rel_err(out[1][0][r], out[0][0][r], sea) < 1e-10
        assert rel_err(out[1][1][r], out[0][1][r]) < 1e-10


@gpu
def test_geometric_cell_weights_match_the_stored_ones(golden):
    """With every invmur exactly 1 (the front end's value) the complex64
    operator forms its coefficients from the spacings; one invmur of
    1 + 2^-23 makes it read the stored volume-weighted cells instead.  The
    two operators differ by float rounding (and that one cell), so six
    mixed cycles of three RHS agree to 1e-5 below the sea surface and in
    H; the FP64 refinement keeps the true operator in both."""
    g = golden("tiny_layered")
    G = _G()
    n, xx, raw, om = golden_level(g)
    bs = np.stack([g["b_f0"], g["badj_f0"], g["b_f0"]])
    oms = np.array([om, om, 0.5 * om], np.float32)
    out = {}
    for name in ("ones", "stored"):
        r = raw.copy()
        if name == "stored":
            r[3].reshape(-1)[0] = np.float32(1.0) + np.float32(2.0 ** -23)
        s = G.Solver(n, *[v.astype(np.float32) for v in xx], r[None], oms,
                     op=np.zeros(3, np.int32),
                     options=G.Options(precision=G.PREC_MIXED, ncycle=6, tol=0.0,
                                       sigma_floor=2e-4))
        x, h, st = s.solve(bs)
        out[name] = (x, h, s.geometric_weights)
        s.close()
    assert out["ones"][2] and not out["stored"][2]
    sea = below_sea_mask(n, g["x3"])
    for r in range(3):
        assert rel_err(out["ones"][0][r], out["stored"][0][r], sea) < 1e-5
        assert rel_err(out["ones"][1][r], out["stored"][1][r]) < 1e-5


@gpu
@pytest.mark.parametrize("case", ["tiny_layered", "tiny_aniso", "c1_layered_64"])
def test_staged_residual_gives_the_plain_iterates(golden, case):
    """The complex64 residual with its halos staged in shared memory by
    tensor copies (tiles of rows x 32 planes, the default) against the plain
    residual: the same edge equations, so six mixed cycles give the same
    iterates to rounding (the norms add in another order; the refinement
    points are the same).  The cases cover one and several plane chunks,
    a non-cubic grid and partial row tiles."""
    g = golden(case)
    G = _G()
    n, xx, raw, om = golden_level(g)
    b = g["b_f0"] if "b_f0" in g else None
    if b is None:
        src = g["srcrec"][:5]
        b = O.inject_source(_grid(g), src, str(g["chsrc"]).split(","), om)
    out = {}
    for staged in (1, 0):
        s = G.Solver(n, *[v.astype(np.float32) for v in xx], raw[None],
                     np.array([om], np.float32),
                     options=G.Options(precision=G.PREC_MIXED, ncycle=6, tol=0.0,
                                       sigma_floor=2e-4, staged=staged))
        x, h, st = s.solve(b[None])
        out[staged] = (x, h, st[0]["cycles"])
        s.close()
    assert out[1][2] == out[0][2] == 6
    sea = below_sea_mask(n, g["x3"])
    assert rel_err(out[1][0][0], out[0][0][0], sea) < 1e-6
    assert rel_err(out[1][1][0], out[0][1][0]) < 1e-6


@gpu
@pytest.mark.parametrize("precision", [1, 0])
def test_skipped_post_smoothing_converges_to_the_same_field(golden, precision):
    """emmi_options.skip_post = 3 (no post-smoothing on levels 0 and 1): a
    weaker cycle with fewer launches, run to the same tolerance as the
    reference's cycle; the fields agree to the tolerance's order below the
    sea, every level's launches of the left-out smoothing are gone from the
    cycle, and skip_post = 0 is the reference's cycle (the other tests)."""
    g = golden("c1_layered_64")
    G = _G()
    n, xx, raw, om = golden_level(g)
    b = g["b_f0"] if "b_f0" in g else None
    if b is None:
        src = g["srcrec"][:5]
        b = O.inject_source(_grid(g), src, str(g["chsrc"]).split(","), om)
    out = {}
    for mask in (0, 3):
        s = G.Solver(n, *[v.astype(np.float32) for v in xx], raw[None],
                     np.array([om], np.float32),
                     options=G.Options(precision=precision, ncycle=60, tol=1e-8,
                                       skip_post=mask))
        x, h, st = s.solve(b[None])
        out[mask] = (x, h, st[0], s.last_launches)
        s.close()
    for mask in (0, 3):
        assert out[mask][2]["status"] == "ok" and out[mask][2]["rel"] <= 1e-8, out[mask][2]
    sea = below_sea_mask(n, g["x3"])
    assert rel_err(out[3][0][0], out[0][0][0], sea) < 1e-5
    # fewer launches per cycle without the two levels' post-smoothing
    per = {m: out[m][3] / out[m][2]["cycles"] for m in (0, 3)}
    assert per[3] < per[0], per


@gpu
def test_staged_residual_wait_that_runs_out_reports_and_recovers(golden):
    """The staged residual's bounded waits: with the test hook no tensor copy
    of plane 3 or beyond is issued and a wait gives up after 2e6 clocks
    (about a millisecond), so the first level-0 residual's wait for plane 3
    runs out; the CTA waits for the copies it did issue and returns, the
    solve reports the failure at its norm check, and with the hook cleared
    the same solver on the same GPU solves to tolerance."""
    g = golden("tiny_layered")
    G = _G()
    n, xx, raw, om = golden_level(g)
    b = g["b_f0"][None]
    s = G.Solver(n, *[v.astype(np.float32) for v in xx], raw[None], np.array([om], np.float32),
                 options=G.Options(precision=G.PREC_MIXED, ncycle=60, tol=1e-8, use_graphs=0))
    assert s.staged
    s.stencil_wait_hook(2_000_000, 3)
    with pytest.raises(RuntimeError, match="staged residual"):
        s.solve(b)
    s.stencil_wait_hook(0, -1)
    x, h, st = s.solve(b)
    assert st[0]["status"] == "ok" and st[0]["rel"] <= 1e-8, st
    s.close()
