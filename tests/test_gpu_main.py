"""The reference's command line (key=value parameters, float32 model files,
acquisition text files) run by emmi_main on the GPU path: the emf_XXXX.txt
of mode=0 matches the reference's receiver data, the gradient files of
mode=2 match the reference's gradient."""
import os
import subprocess

import numpy as np
import pytest

from libemmi_mgfd_gb300 import workloads as W

gpu = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
MAIN = os.path.join(ROOT, "libemmi_mgfd_gb300", "emmi_main")


def read_emf(path):
    rows = open(path).read().splitlines()
    assert rows[0].startswith("iTx \tiRx")
    out = {}
    for r in rows[1:]:
        t = r.split("\t")
        isrc, irec, ch, f, re, im = (t[0].strip(), t[1].strip(), t[2].strip(), t[3].strip(),
                                     t[4].strip(), t[5].strip())
        out.setdefault(ch, []).append((int(irec), float(f), float(re) + 1j * float(im)))
    return {k: np.array([v[2] for v in sorted(vs)]) for k, vs in out.items()}


@gpu
@pytest.mark.parametrize("batch", [0, 1])
@pytest.mark.parametrize("prec", [0, 1])
def test_emmi_main_matches_reference_output(golden, tmp_path, prec, batch):
    """mode=0: every shot and frequency in one device solver (batch=1) or
    shot by shot through the drop-in entry points (batch=0)."""
    from test_gpu_solver import receiver_parity
    g = golden("tiny_layered")
    s = W.tiny_layered()
    s.write(str(tmp_path))
    args = [MAIN] + s.params(str(tmp_path)) + ["tol=1e-10", "ncycle=120",
                                               f"gmg_precision={prec}", "verb=1",
                                               f"batch={batch}"]
    r = subprocess.run(args, cwd=tmp_path, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    d = read_emf(os.path.join(tmp_path, "emf_0001.txt"))
    ch = list(s.chrec)
    got = np.stack([d[c] for c in ch])
    amp, ph = receiver_parity(got, g["dcal"], ch)
    # the text format keeps 7 significant digits (%e)
    assert amp < 1e-4 and ph < 0.05, (amp, ph)


@gpu
@pytest.mark.parametrize("batch", [0, 1])
@pytest.mark.parametrize("prec,tol", [(0, "1e-10"), (1, "1e-9")])
def test_emmi_main_gradient_matches_reference(golden, tmp_path, prec, tol, batch):
    """mode=2 (one data gradient, src/fg_fwi.c) on the 16^3 layered case:
    observed data from the reference's mode=0 run on the true model, the
    gradient of the start model, against the reference's gradient files
    (within 1e-3 of the largest value, and in the L2 norm); batch=1 is the
    device evaluation of every shot at once, batch=0 the drop-in entry
    points shot by shot."""
    import dataclasses
    g = golden("tiny_grad")
    true = W.tiny_layered()
    rho = np.asarray(g["rho_start"], np.float32)
    start = dataclasses.replace(true, rho11=rho, rho22=rho.copy(), rho33=rho.copy())
    start.write(str(tmp_path))
    (tmp_path / "emf_0001.txt").write_text(str(g["obs_text"]))
    args = [a for a in start.params(str(tmp_path)) if not a.startswith(("mode=", "verb="))]
    args += ["mode=2", "verb=1", "addnoise=0", "npar=2", "idxpar=1,2", "preco=1",
             f"tol={tol}", "ncycle=120", f"gmg_precision={prec}", f"batch={batch}"]
    r = subprocess.run([MAIN] + args, cwd=tmp_path, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    for nm in ("grad_Rv", "grad_Rh"):
        ours = np.fromfile(tmp_path / ("gradient_dat_" + nm[5:]), np.float32)
        ref = np.asarray(g[nm], np.float32)
        assert ours.shape == ref.shape
        l2 = np.linalg.norm(ours - ref) / np.linalg.norm(ref)
        mx = np.abs(ours - ref).max() / np.abs(ref).max()
        print(f"{nm}: L2 {l2:.2e}, max {mx:.2e}")
        assert l2 < 1e-3 and mx < 1e-3, (nm, l2, mx)
    fcost = [float(l.split("=")[1].split(",")[0]) for l in r.stdout.splitlines()
             if l.startswith("fcost_dat=")]
    assert abs(fcost[0] - float(g["fcost"][0])) <= 1e-4 * float(g["fcost"][0])


def _iterate_rows(text):
    rows = []
    for line in str(text).splitlines():
        t = line.split()
        if len(t) == 7 and t[0].isdigit():
            rows.append([int(t[0]), float(t[1]), float(t[2]), float(t[3]), float(t[4]), int(t[5]),
                         int(t[6])])
    return rows


def _trace(stdout):
    """The inversion's path from its stdout: the start model's evaluation,
    then per iteration the objective of every evaluation (the printed total)
    and the Wolfe condition each failed evaluation broke (1 or 2; 0 =
    accepted or out of searches)."""
    cur = []
    its = [cur]
    for line in str(stdout).splitlines():
        l = line.strip()
        if l.startswith("# iter="):
            cur = []
            its.append(cur)
        elif l.startswith("fcost="):
            cur.append([float(l.split("=")[1]), 0])
        elif l.startswith("Wolfe condition") and cur:
            cur[-1][1] = int(l.split()[2])
    return its


@gpu
@pytest.mark.parametrize("batch", [0, 1])
@pytest.mark.parametrize("prec,tol", [(0, "1e-10"), (1, "1e-9")])
def test_emmi_main_inversion_matches_reference(golden, tmp_path, prec, tol, batch):
    """mode=1 (the l-BFGS inversion, src/do_fwi.c) for two iterations on the
    layered case (21 x 21 x 11 cells) from the start model, against the
    reference's own run.

    Pinned: the objective, gradient norm and counters of every iteration
    (iterate.txt to its three printed digits, counts exactly), the misfit of
    every iteration (rmse_misfit.txt), the whole first iteration -- scaled
    and preconditioned first gradient, the line search's evaluations and
    decisions, the resistivities it ends with (Rv/Rh_iteration_00).

    Not pinned: the second l-BFGS direction.  It divides the gradient
    difference of the two iterates by the pseudo-Hessian, which is 1e-5 of
    its peak in cells the survey hardly sees, and amplifies the solver's
    last digits there: the reference's own second iterate moves by 0.06 in
    log-resistivity (step 0.6) when its solver tolerance goes from 1e-10 to
    1e-8 (tests/golden/make_golden.py sensitivity).  The second iteration
    is held to what the inversion is for: its line search ends with a
    decrease and its objective is no worse than the reference's.  The
    optimizer of every later iteration is pinned bitwise, on the CPU, to the
    reference's own (tests/test_fwi_host.py)."""
    import dataclasses
    g = golden("tiny_fwi")
    true = W.tiny_layered()
    rho = np.asarray(g["rho_start"], np.float32)
    start = dataclasses.replace(true, rho11=rho, rho22=rho.copy(), rho33=rho.copy())
    start.write(str(tmp_path))
    (tmp_path / "emf_0001.txt").write_text(str(g["obs_text"]))
    args = [a for a in start.params(str(tmp_path)) if not a.startswith(("mode=", "verb="))]
    args += ["mode=1", "verb=1", "addnoise=0", "npar=2", "idxpar=1,2", "preco=1", "niter=2",
             f"tol={tol}", "ncycle=120", f"gmg_precision={prec}", f"batch={batch}"]
    r = subprocess.run([MAIN] + args, cwd=tmp_path, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr
    ours = _iterate_rows(open(tmp_path / "iterate.txt").read())
    ref = _iterate_rows(g["iterate"])
    print("ours", ours)
    print("ref ", ref)
    assert len(ours) == len(ref) == 2
    for a, b in zip(ours, ref):
        assert a[0] == b[0] and a[5] == b[5] and a[6] == b[6], (a, b)
        for k in (1, 2, 3, 4):
            assert abs(a[k] - b[k]) <= 6e-3 * abs(b[k]), (k, a, b)
    m_ours = np.loadtxt(tmp_path / "rmse_misfit.txt")
    m_ref = np.array([[float(v) for v in l.split()] for l in str(g["rmse_misfit"]).splitlines()])
    assert np.allclose(m_ours, m_ref, rtol=1e-4), (m_ours, m_ref)
    # the first iteration, evaluation by evaluation
    t_ours, t_ref = _trace(r.stdout), _trace(g["trace"])
    print("trace ours", t_ours)
    print("trace ref ", t_ref)
    assert len(t_ours) == len(t_ref) == 3
    for k in (0, 1):  # the start model, the first iteration
        assert [w for _, w in t_ours[k]] == [w for _, w in t_ref[k]]
        for (fa, _), (fb, _) in zip(t_ours[k], t_ref[k]):
            assert abs(fa - fb) <= 2e-5 * abs(fb), (fa, fb)
    for nm in ("Rv", "Rh"):
        o = np.fromfile(tmp_path / f"{nm}_iteration_00", np.float32)
        e = np.asarray(g[f"{nm}_00"], np.float32).ravel()
        d = np.abs(np.log(o) - np.log(e)).max()
        step = np.abs(np.log(e) - np.log(rho.ravel())).max()
        print(f"{nm} iteration 0: max |dlog| {d:.2e} (model step {step:.2e})")
        assert d <= 1e-3 * max(step, 1e-6) + 1e-6, (nm, d, step)
    # the second iteration: an accepted step, no worse than the reference's
    last_ours, last_ref = t_ours[2][-1], t_ref[2][-1]
    assert last_ours[1] == 0 and last_ref[1] == 0, (t_ours[2], t_ref[2])
    assert last_ours[0] <= last_ref[0] * (1 + 1e-4), (last_ours, last_ref)
    assert last_ours[0] < t_ours[1][-1][0], "no decrease in the second iteration"
    for nm in ("Rv", "Rh"):
        o = np.fromfile(tmp_path / f"{nm}_iteration_01", np.float32)
        assert np.isfinite(o).all() and (o > 0).all()


def _ragged_three_shots():
    """The layered case with three sources, two frequencies and a different
    receiver set per shot (all 21, the first 15, every other one)."""
    import dataclasses
    s = W.tiny_layered()
    src = np.array([[-1000.0, 0.0, 950.0, 0.0, 0.0], [0.0, 500.0, 950.0, 30.0, 0.0],
                    [1500.0, -500.0, 950.0, -20.0, 0.0]], np.float32)
    nrec = len(s.receivers)
    pairs = [(1, r) for r in range(1, nrec + 1)] + [(2, r) for r in range(1, 16)] + \
            [(3, r) for r in range(1, nrec + 1, 2)]
    return dataclasses.replace(s, sources=src, pairs=np.array(pairs), freqs=[0.5, 1.0])



@gpu
@pytest.mark.parametrize("preco", [1, 0])
def test_batched_evaluation_matches_shot_by_shot(tmp_path, preco):
    """mode=2 over three shots with ragged receiver sets and two frequencies:
    the device evaluation of every shot and frequency at once (batch=1)
    against the drop-in entry points shot by shot (batch=0), both FP64 to
    1e-10: gradients, pseudo-Hessian, misfits, synthetic data and rmse
    files."""
    import dataclasses
    true = _ragged_three_shots()
    tdir = tmp_path / "true"
    true.write(str(tdir))
    args = [a for a in true.params(str(tdir)) if not a.startswith("shots=")]
    r = subprocess.run([MAIN] + args + ["shots=1,2,3", "tol=1e-10", "ncycle=120",
                                        "gmg_precision=0"],
                       cwd=tdir, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    rho = true.rho11.copy()
    rho[rho == 100.0] = 1.0  # the start model: no resistive layer
    start = dataclasses.replace(true, rho11=rho, rho22=rho.copy(), rho33=rho.copy())
    out = {}
    for batch in (0, 1):
        d = tmp_path / f"b{batch}"
        start.write(str(d))
        for k in (1, 2, 3):
            (d / f"emf_{k:04d}.txt").write_text((tdir / f"emf_{k:04d}.txt").read_text())
        a = [x for x in start.params(str(d)) if not x.startswith(("mode=", "verb=", "shots="))]
        a += ["mode=2", "verb=1", "shots=1,2,3", "addnoise=0", "npar=2", "idxpar=1,2",
              f"preco={preco}", "tol=1e-10", "ncycle=120", "gmg_precision=0", f"batch={batch}"]
        r = subprocess.run([MAIN] + a, cwd=d, capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stdout[-3000:] + r.stderr
        o = {nm: np.fromfile(d / nm, np.float32)
             for nm in ("gradient_dat_Rv", "gradient_dat_Rh")}
        if preco == 1:
            o["gradient_phess"] = np.fromfile(d / "gradient_phess", np.float32)
        o["fcost"] = [float(l.split("fcost=")[1].split(",")[0]) for l in r.stdout.splitlines()
                      if l.startswith("isrc=")]
        for k in (1, 2, 3):
            o[f"syn{k}"] = read_emf(d / f"syn_{k:04d}.txt")
            o[f"rmse{k}"] = np.loadtxt(d / f"rmse_{k:04d}.txt", skiprows=1, usecols=(4,))
        out[batch] = o
    a, b = out[0], out[1]
    assert len(a["fcost"]) == len(b["fcost"]) == 3
    np.testing.assert_allclose(b["fcost"], a["fcost"], rtol=1e-5)
    for nm in [k for k in a if k.startswith("gradient")]:
        err = np.abs(b[nm] - a[nm]).max() / np.abs(a[nm]).max()
        print(nm, f"max {err:.2e}")
        assert err < 1e-5, (nm, err)
    for k in (1, 2, 3):
        for ch in a[f"syn{k}"]:
            x, y = a[f"syn{k}"][ch], b[f"syn{k}"][ch]
            assert x.shape == y.shape and np.abs(y - x).max() <= 1e-5 * np.abs(x).max(), (k, ch)
        np.testing.assert_allclose(b[f"rmse{k}"], a[f"rmse{k}"], rtol=1e-5, atol=1e-6)
    assert [len(a[f"rmse{k}"]) for k in (1, 2, 3)] == [2 * 4 * 21, 2 * 4 * 15, 2 * 4 * 11]


@gpu
@pytest.mark.parametrize("tag", ["p2", "p3", "bound"])
def test_emmi_main_inversion_variants_first_iteration(golden, tmp_path, tag):
    """mode=1, one iteration, with the depth preconditioner (preco=2), the
    triangle smoothing (preco=3, r1=r2=r3=2) and the box bounds (bound=1,
    minpar=0.5,0.5 maxpar=3,3): the start model's and every line-search
    evaluation's objective and Wolfe decision, iterate.txt and the
    resistivities after the iteration against the reference's own runs
    (FP64, the batched evaluation)."""
    import dataclasses
    g = {k[len(tag) + 1:]: v for k, v in golden("tiny_fwi_variants").items()
         if k.startswith(tag + "_")}
    true = W.tiny_layered()
    rho = np.asarray(g["rho_start"], np.float32)
    start = dataclasses.replace(true, rho11=rho, rho22=rho.copy(), rho33=rho.copy())
    start.write(str(tmp_path))
    (tmp_path / "emf_0001.txt").write_text(str(g["obs_text"]))
    args = [a for a in start.params(str(tmp_path)) if not a.startswith(("mode=", "verb="))]
    args += [a for a in str(g["params"]).split() if not a.startswith(("tol=", "ncycle="))]
    args += ["mode=1", "verb=1", "tol=1e-10", "ncycle=120", "gmg_precision=0"]
    r = subprocess.run([MAIN] + args, cwd=tmp_path, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr
    ours = _iterate_rows(open(tmp_path / "iterate.txt").read())
    ref = _iterate_rows(g["iterate"])
    assert len(ours) == len(ref) == 1
    assert ours[0][0] == ref[0][0] and ours[0][5:] == ref[0][5:], (ours, ref)
    t_ours, t_ref = _trace(r.stdout), _trace(g["trace"])
    print("trace ours", t_ours)
    print("trace ref ", t_ref)
    assert len(t_ours) == len(t_ref) == 2
    for k in (0, 1):
        assert [w for _, w in t_ours[k]] == [w for _, w in t_ref[k]]
        for (fa, _), (fb, _) in zip(t_ours[k], t_ref[k]):
            assert abs(fa - fb) <= 2e-5 * abs(fb), (fa, fb)
    for nm in ("Rv", "Rh"):
        o = np.fromfile(tmp_path / f"{nm}_iteration_00", np.float32)
        e = np.asarray(g[f"{nm}_00"], np.float32).ravel()
        d = np.abs(np.log(o) - np.log(e)).max()
        step = np.abs(np.log(e) - np.log(rho.ravel())).max()
        print(f"{tag} {nm}: max |dlog| {d:.2e} (model step {step:.2e})")
        assert d <= 1e-3 * max(step, 1e-6) + 1e-6, (nm, d, step)
    if tag == "bound":
        # below the sea floor plus one cell the model stays inside [0.5, 3]
        o = np.fromfile(tmp_path / "Rv_iteration_00", np.float32).reshape(rho.shape)
        zc = start.oz + (np.arange(start.nz) + 0.5) * start.dz
        below = zc > 1000.0 + start.dz
        assert o[below].min() >= 0.5 * (1 - 1e-6) and o[below].max() <= 3 * (1 + 1e-6)


@gpu
def test_batched_modelling_matches_shot_by_shot(tmp_path):
    """mode=0 over three shots with ragged receiver sets and two
    frequencies: all shots in one device solver against the drop-in entry
    points shot by shot (FP64 to 1e-10); the emf files agree to 1e-6 of
    each channel's largest value."""
    s = _ragged_three_shots()
    out = {}
    for batch in (0, 1):
        d = tmp_path / f"b{batch}"
        s.write(str(d))
        a = [x for x in s.params(str(d)) if not x.startswith("shots=")]
        r = subprocess.run([MAIN] + a + ["shots=1,2,3", "tol=1e-10", "ncycle=120",
                                         "gmg_precision=0", f"batch={batch}"],
                           cwd=d, capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stdout[-2000:] + r.stderr
        out[batch] = [read_emf(d / f"emf_{k:04d}.txt") for k in (1, 2, 3)]
    for k in range(3):
        for ch, x in out[0][k].items():
            y = out[1][k][ch]
            assert x.shape == y.shape == ((21, 15, 11)[k] * 2,)
            assert np.abs(y - x).max() <= 1e-6 * np.abs(x).max(), (k, ch)
