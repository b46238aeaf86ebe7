"""The reference's modelling command line (key=value parameters, float32
model files, acquisition text files) run by emmi_main on the GPU path: the
emf_XXXX.txt it writes matches the reference's receiver data."""
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
