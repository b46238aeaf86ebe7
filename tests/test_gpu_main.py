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
@pytest.mark.parametrize("prec", [0, 1])
def test_emmi_main_matches_reference_output(golden, tmp_path, prec):
    from test_gpu_solver import receiver_parity
    g = golden("tiny_layered")
    s = W.tiny_layered()
    s.write(str(tmp_path))
    args = [MAIN] + s.params(str(tmp_path)) + ["tol=1e-10", "ncycle=120",
                                               f"gmg_precision={prec}", "verb=1"]
    r = subprocess.run(args, cwd=tmp_path, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    d = read_emf(os.path.join(tmp_path, "emf_0001.txt"))
    ch = list(s.chrec)
    got = np.stack([d[c] for c in ch])
    amp, ph = receiver_parity(got, g["dcal"], ch)
    # the text format keeps 7 significant digits (%e)
    assert amp < 1e-4 and ph < 0.05, (amp, ph)


@gpu
@pytest.mark.parametrize("prec,tol", [(0, "1e-10"), (1, "1e-9")])
def test_emmi_main_gradient_matches_reference(golden, tmp_path, prec, tol):
    """mode=2 (one data gradient, src/fg_fwi.c) on the 16^3 layered case:
    observed data from the reference's mode=0 run on the true model, the
    gradient of the start model, against the reference's gradient files
    (within 1e-3 of the largest value, and in the L2 norm)."""
    import dataclasses
    g = golden("tiny_grad")
    true = W.tiny_layered()
    rho = np.asarray(g["rho_start"], np.float32)
    start = dataclasses.replace(true, rho11=rho, rho22=rho.copy(), rho33=rho.copy())
    start.write(str(tmp_path))
    (tmp_path / "emf_0001.txt").write_text(str(g["obs_text"]))
    args = [a for a in start.params(str(tmp_path)) if not a.startswith(("mode=", "verb="))]
    args += ["mode=2", "verb=1", "addnoise=0", "npar=2", "idxpar=1,2", "preco=1",
             f"tol={tol}", "ncycle=120", f"gmg_precision={prec}"]
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
    fcost = [float(l.split("=")[1]) for l in r.stdout.splitlines() if l.startswith("fcost_dat=")]
    assert abs(fcost[0] - float(g["fcost"][0])) <= 1e-4 * float(g["fcost"][0])
