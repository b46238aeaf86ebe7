"""Parity at the sizes the benchmark configurations are measured on, through
the C ABI, against the reference's own runs (tests/golden/*_ref.npz, made by
tests/golden/make_golden.py from the reference compiled from its sources)
and against FP64 solves of the same batches.

  * the 128^3 log-normal configuration: all 25 shots, complex64 cycles with
    the learned correction and FP64 refinement to 1e-8, against an FP64
    solve of the batch to 1e-12 (every shot) and against the reference's
    receiver data of shots 1 and 13 (solved by the reference to 1e-10); and
    the benchmark's cycle (no post-smoothing on levels 0 and 1) against the
    same reference data;
  * the VTI / bathymetry configuration (25 shots x 2 frequencies) on the
    48x48x64 mesh the reference can build for it: shots 1 and 13 at both
    frequencies against the reference's receiver data;
  * the gradient configuration (reservoir data, half-space start model, 3
    frequencies) at 64^3: the reference's mode=2 gradient summed over shots
    1 and 13, against emmi_main mode=2 on the same files.

Bars: receivers within 1e-4 of the channel's scale and 0.05 degrees in
phase (test_gpu_solver.receiver_parity); gradients within 1e-3 relative.
"""
import concurrent.futures as cf
import os
import subprocess

import numpy as np
import pytest

from libemmi_mgfd_gb300 import host
from libemmi_mgfd_gb300 import workloads as W
from test_gpu_solver import receiver_parity

gpu = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
MAIN = os.path.join(ROOT, "libemmi_mgfd_gb300", "emmi_main")


def _batch(s, shots=None):
    """Mesh axes and cells of every listed shot through the host front end,
    every frequency per shot (RHS order shot-major), angles in radians."""
    m = host.Model.from_survey(s)
    shots = list(range(1, s.nshots + 1)) if shots is None else list(shots)
    src = s.sources.astype(np.float32).copy()
    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        grids = list(ex.map(lambda k: m.regrid(*[float(v) for v in src[k - 1, :3]]), shots))
    X = [np.stack([g[k] for g in grids]) for k in ("x1", "x2", "x3")]
    cells = np.stack([np.stack([g["sigma11"], g["sigma22"], g["sigma33"], g["invmur"]])
                      for g in grids])
    nf = len(s.freqs)
    om = np.array([np.float32(2 * np.pi * s.freqs[r % nf]) for r in range(len(shots) * nf)],
                  np.float32)
    op = np.repeat(np.arange(len(shots), dtype=np.int32), nf)
    srcr = src[[k - 1 for k in shots]].copy()
    srcr[:, 3:] = np.deg2rad(srcr[:, 3:])
    srcr = np.repeat(srcr, nf, axis=0)
    rec = s.receivers.astype(np.float32).copy()
    rec[:, 3:] = np.deg2rad(rec[:, 3:])
    return dict(X=X, cells=cells, omega=om, op=op, src=srcr, rec=rec,
                rho_water=np.float32(m.rho_water()), nf=nf)


def _model(s, b, precision, tol, ncycle=200, learned=None, skip_post=0):
    from libemmi_mgfd_gb300 import gpu as G
    sv = G.Solver(s.n, *b["X"], b["cells"], b["omega"], op=b["op"],
                  options=G.Options(precision=precision, tol=tol, ncycle=ncycle,
                                    skip_post=skip_post),
                  rho_water=b["rho_water"])
    if learned is not None:
        sv.set_learned(learned)
    d, st, _ = sv.modelling(b["src"], b["rec"], s.chsrc, s.chrec)
    sv.close()
    return np.asarray(d), st


@gpu
def test_config3_batch_receivers_against_fp64_and_reference(golden):
    """128^3 log-normal configuration, 25 shots at 1 Hz: the benchmark's
    learned + mixed solve against an FP64 solve to 1e-12 for every shot, and
    both against the reference's receiver data of shots 1 and 13."""
    from libemmi_mgfd_gb300 import gpu as G
    from libemmi_mgfd_gb300 import learned as LS
    g = golden("c3_lognormal_128_ref")
    s = W.config3(128)
    b = _batch(s)
    ch = list(s.chrec)
    tr = LS.train(n=48, models=6, per_rhs=6, steps=300, lr=3e-3, seed=100)
    d, st = _model(s, b, G.PREC_MIXED, 1e-8, ncycle=100, learned=tr["weights"])
    assert all(q["status"] == "ok" and q["rel"] <= 1e-8 for q in st), st
    d64, st64 = _model(s, b, G.PREC_FP64, 1e-12)
    assert all(q["status"] == "ok" and q["rel"] <= 1e-12 for q in st64), st64
    worst = [receiver_parity(d[r], d64[r], ch) for r in range(d.shape[0])]
    amp = max(w[0] for w in worst)
    ph = max(w[1] for w in worst)
    print(f"learned+mixed vs FP64 1e-12 over 25 shots: amplitude {amp:.2e}, phase {ph:.2e} deg")
    assert amp < 1e-4 and ph < 0.05, (amp, ph)
    for k in g["shots"]:
        ref = g[f"s{k}_dcal"]
        a1, p1 = receiver_parity(d[k - 1], ref, ch)
        a2, p2 = receiver_parity(d64[k - 1], ref, ch)
        print(f"shot {k} vs reference (tol 1e-10, {int(g[f's{k}_cycles'][0])} F-cycles): "
              f"learned+mixed {a1:.2e} / {p1:.2e} deg, FP64 {a2:.2e} / {p2:.2e} deg")
        assert a1 < 1e-4 and p1 < 0.05, (k, a1, p1)
        assert a2 < 1e-4 and p2 < 0.05, (k, a2, p2)


@gpu
def test_config3_bench_cycle_receivers_match_reference(golden):
    """The benchmark's own configuration: the 25 shots at 1 Hz, complex64
    cycles without the post-smoothing of levels 0 and 1 (skip_post = 3) and
    the learned correction trained on residuals of that cycle, FP64
    refinement to 1e-8, against the reference's receiver data of shots 1
    and 13 (solved by the reference to 1e-10)."""
    from libemmi_mgfd_gb300 import gpu as G
    from libemmi_mgfd_gb300 import learned as LS
    g = golden("c3_lognormal_128_ref")
    s = W.config3(128)
    b = _batch(s)
    ch = list(s.chrec)
    tr = LS.train(n=48, models=6, per_rhs=6, steps=300, lr=3e-3, seed=100, skip_post=3)
    d, st = _model(s, b, G.PREC_MIXED, 1e-8, ncycle=100, learned=tr["weights"], skip_post=3)
    assert all(q["status"] == "ok" and q["rel"] <= 1e-8 for q in st), st
    for k in g["shots"]:
        a1, p1 = receiver_parity(d[k - 1], g[f"s{k}_dcal"], ch)
        print(f"shot {k} vs reference: bench cycle + learned {a1:.2e} / {p1:.2e} deg")
        assert a1 < 1e-4 and p1 < 0.05, (k, a1, p1)


@gpu
def test_config2_mesh_receivers_match_reference(golden):
    """VTI sediment, random bathymetry, resistive box: shots 1 and 13 at 0.25
    and 0.75 Hz on the 48x48x64 mesh, complex64 cycles to 1e-8 and FP64 to
    1e-10, against the reference's receiver data (200 receivers)."""
    from libemmi_mgfd_gb300 import gpu as G
    g = golden("c2_vti_48x48x64_ref")
    s = W.config2(96)
    s.n = tuple(int(v) for v in g["n"])
    shots = [int(k) for k in g["shots"]]
    b = _batch(s, shots)
    ch = list(s.chrec)
    nf, nrec = b["nf"], len(s.receivers)
    for prec, tol in ((G.PREC_MIXED, 1e-8), (G.PREC_FP64, 1e-10)):
        d, st = _model(s, b, prec, tol)
        assert all(q["status"] == "ok" for q in st), st
        for i, k in enumerate(shots):
            ref = g[f"s{k}_dcal"].reshape(len(ch), nf, nrec)
            for f in range(nf):
                a, p = receiver_parity(d[i * nf + f], ref[:, f], ch)
                print(f"precision {prec} shot {k} f{f}: amplitude {a:.2e}, phase {p:.2e} deg")
                assert a < 1e-4 and p < 0.05, (prec, k, f, a, p)


@gpu
@pytest.mark.parametrize("prec,tol", [(0, "1e-10"), (1, "1e-9")])
def test_config4_gradient_matches_reference(golden, tmp_path, prec, tol):
    """The gradient configuration at 64^3: observed data of the 100 ohm-m
    reservoir model (the reference's mode=0 output, no noise), gradient of
    the 1 ohm-m half-space start model for Rh and Rv (npar=2), 0.25 / 0.5 /
    1 Hz, shots 1 and 13 summed -- emmi_main mode=2 against the reference's
    gradient files, within 1e-3 in the L2 norm and of the largest value."""
    g = golden("c4_reservoir_64_grad_ref")
    start = W.config4(64, true_model=False)
    start.write(str(tmp_path))
    shots = [int(k) for k in g["shots"]]
    for k in shots:
        (tmp_path / f"emf_{k:04d}.txt").write_text(str(g[f"s{k}_obs_text"]))
    args = [a for a in start.params(str(tmp_path))
            if not a.startswith(("mode=", "verb=", "shots="))]
    args += ["mode=2", "verb=1", "addnoise=0", "npar=2", "idxpar=1,2", "preco=1",
             "shots=" + ",".join(str(k) for k in shots), f"tol={tol}", "ncycle=200",
             f"gmg_precision={prec}"]
    r = subprocess.run([MAIN] + args, cwd=tmp_path, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    for nm in ("Rv", "Rh"):
        ours = np.fromfile(tmp_path / ("gradient_dat_" + nm), np.float32)
        ref = np.asarray(g["grad_" + nm], np.float32)
        assert ours.shape == ref.shape
        l2 = np.linalg.norm(ours - ref) / np.linalg.norm(ref)
        mx = np.abs(ours - ref).max() / np.abs(ref).max()
        print(f"{nm}: L2 {l2:.2e}, max {mx:.2e}")
        assert l2 < 1e-3 and mx < 1e-3, (nm, l2, mx)
