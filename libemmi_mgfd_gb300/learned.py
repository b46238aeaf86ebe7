"""Learned correction of the mixed-precision cycle: training problems, the
GPU training driver and weight initialisation.

The network (csrc/emmi_learned.cu) corrects the level-0 complex64 iterate
after every cycle: u += N(D^-1 (f - A u)).  It is trained on the GPU, by the
library's own forward and backward kernels, on residuals that plain cycles
leave behind for random conductivity models.  The models are built the way
survey models are: a water layer over log-normal sediment with resistive
bodies, regridded by the host front end (stretched padding and the air layer
included), one x-directed dipole per model at a random position above the
seafloor.
"""
from __future__ import annotations

import time
from typing import Dict

import numpy as np

from . import gpu as G
from . import host
from . import workloads as W

LAYERS, TAPS, CH = 2, 27, 8
N_WEIGHTS = LAYERS * TAPS * CH * CH


def init_weights(seed: int = 0, scale: float = 0.05) -> np.ndarray:
    """[2, 27, 8, 8] (layer, tap, cin, cout) flattened.  Layer 1 random on
    the 6 input channels that carry data, layer 2 zero: the untrained
    correction is exactly zero."""
    rng = np.random.default_rng(seed)
    w = np.zeros((LAYERS, TAPS, CH, CH), np.float32)
    w[0, :, :6, :] = (scale * rng.standard_normal((TAPS, 6, CH))).astype(np.float32)
    return w.reshape(-1)


def random_survey(n: int, seed: int) -> W.Survey:
    """A 4 x 4 x 1.5 km model (water to 800-1200 m, log-normal sediment, one
    resistive body) with one dipole at a random position, on an n^3 mesh,
    1 Hz."""
    rng = np.random.default_rng(seed)
    # the front end keeps the input z nodes down to 5 cells below the
    # source: coarser input cells in z for small meshes
    dz = 50.0 if n >= 48 else 100.0
    nx, ny, nz = 40, 40, int(1500.0 / dz)
    dx = dy = 100.0
    ox, oy, oz = -2000.0, -2000.0, 0.0
    zc = oz + (np.arange(nz) + 0.5) * dz
    xc = ox + (np.arange(nx) + 0.5) * dx
    yc = oy + (np.arange(ny) + 0.5) * dy
    logr = rng.uniform(0.15, 0.45) * W._smooth_field(rng, (nz, ny, nx),
                                                     (300.0 / dz, 6.0, 6.0))
    rho = (10.0 ** logr).astype(np.float32)
    water = rng.uniform(800.0, 1200.0)
    rho[zc < water] = W.RHO_WATER
    cx, cy = rng.uniform(-1200, 1200, 2)
    cz = rng.uniform(water + 300.0, 1400.0 + 0.5 * water)
    hx, hy, hz = rng.uniform(300, 900), rng.uniform(300, 900), rng.uniform(50, 150)
    body = ((np.abs(xc - cx)[None, None, :] <= hx) & (np.abs(yc - cy)[None, :, None] <= hy)
            & (np.abs(zc - cz)[:, None, None] <= hz))
    rho[body] = rng.uniform(20.0, 100.0)
    sx, sy = (float(np.float32(v)) for v in rng.uniform(-1000.0, 1000.0, 2))
    sz = float(np.float32(water - rng.uniform(30.0, 100.0)))
    src = np.array([[sx, sy, sz, 0.0, 0.0]], np.float32)
    rec = np.array([[0.0, 0.0, float(np.float32(water)), 0.0, 0.0]], np.float32)
    return W.Survey(f"train_{seed}", nx, ny, nz, dx, dy, dz, ox, oy, oz, rho, rho.copy(),
                    rho.copy(), src, rec, np.array([[1, 1]]), [1.0], (n, n, n))


def training_problem(n: int, models: int, seed: int) -> Dict:
    """Grids, conductivities, frequencies and sources of `models` random
    surveys through the host front end (one operator and one RHS each)."""
    xs, cells, src = [[], [], []], [], []
    rho_w = []
    for m in range(models):
        s = random_survey(n, seed + m)
        mod = host.Model.from_survey(s)
        p = s.sources[0]
        g = mod.regrid(float(p[0]), float(p[1]), float(p[2]))
        for e, k in enumerate(("x1", "x2", "x3")):
            xs[e].append(g[k])
        cells.append(np.stack([g["sigma11"], g["sigma22"], g["sigma33"], g["invmur"]]))
        src.append([p[0], p[1], p[2], 0.0, 0.0])
        rho_w.append(mod.rho_water())
    return dict(n=(n, n, n), x1=np.stack(xs[0]), x2=np.stack(xs[1]), x3=np.stack(xs[2]),
                cells=np.stack(cells), omega=np.full(models, 2 * np.pi, np.float32),
                src=np.asarray(src, np.float32), rho_water=np.asarray(rho_w, np.float32))


def make_solver(p: Dict, **opt) -> G.Solver:
    nrhs = p["x1"].shape[0]
    return G.Solver(p["n"], p["x1"], p["x2"], p["x3"], p["cells"], p["omega"],
                    op=np.arange(nrhs, dtype=np.int32), options=G.Options(**opt),
                    rho_water=p["rho_water"])


def train(n: int = 48, models: int = 6, per_rhs: int = 6, steps: int = 300, lr: float = 3e-3,
          seed: int = 100, weights=None, skip_post: int = 0) -> Dict:
    """Collect residual samples of plain complex64 cycles on `models` random
    surveys and train the network on them with full-batch Adam on the GPU.
    Returns the weights, the loss history (mean |r - A c|^2/|r|^2, 1.0 for
    the zero correction) and the seconds spent.  skip_post: the cycles
    whose residuals are collected leave out the post-smoothing of the levels
    whose bit is set (emmi_options.skip_post; bit 0 puts the correction in
    the place of the level-0 post-smoothing)."""
    t0 = time.perf_counter()
    p = training_problem(n, models, seed)
    s = make_solver(p, precision=G.PREC_MIXED, tol=1e-8, ncycle=per_rhs + 4,
                    skip_post=skip_post)
    b = s.inject_sources(p["src"])
    st = s.learned_collect(b.data_ptr(), per_rhs, device=True)
    t1 = time.perf_counter()
    w0 = init_weights(seed) if weights is None else np.asarray(weights, np.float32)
    w, loss = s.learned_train(w0, steps, lr)
    t2 = time.perf_counter()
    out = dict(weights=w, loss=loss, samples=s.learned_samples, collect_seconds=t1 - t0,
               train_seconds=t2 - t1, collect_cycles=[x["cycles"] for x in st])
    s.close()
    return out
