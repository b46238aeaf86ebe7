"""Seeded synthetic CSEM workloads in the reference's input formats.

The reference reads float32 resistivity cubes (``frho11/22/33``, [nz][ny][nx]
with x fastest, src/emf_init_free.c:73-105), three ASCII acquisition files
with one header line each (``fsrc``/``frec``: ``x y z heading pitch idx``,
``fsrcrec``: ``isrc irec``; src/acq_init_free.c:88-210) and key=value
parameters.  This module builds those inputs for the benchmark
configurations (seeded numpy generators stand in for the reference's example
models; there is no public dataset) and for the small cases the parity
tests use.  Coordinates are chosen exactly representable in float32 so the
reference's domain checks (src/acq_init_free.c:63-66) pass.
"""
from __future__ import annotations

import dataclasses
import os
from typing import Dict, List, Optional, Sequence

import numpy as np

RHO_WATER = 0.3125


@dataclasses.dataclass
class Survey:
    """One modelling job: model cube, acquisition and solver parameters."""

    name: str
    nx: int
    ny: int
    nz: int
    dx: float
    dy: float
    dz: float
    ox: float
    oy: float
    oz: float
    rho11: np.ndarray  # [nz, ny, nx] float32
    rho22: np.ndarray
    rho33: np.ndarray
    sources: np.ndarray  # [nsrc, 5]: x y z heading(deg) pitch(deg)
    receivers: np.ndarray  # [nrec, 5]
    pairs: np.ndarray  # [npair, 2] 1-based (isrc, irec)
    freqs: Sequence[float]
    n: Sequence[int]  # n1, n2, n3
    chsrc: Sequence[str] = ("Ex",)
    chrec: Sequence[str] = ("Ex", "Ey", "Hx", "Hy")
    extra: Dict[str, str] = dataclasses.field(default_factory=dict)
    bathy: Optional[np.ndarray] = None  # [ny, nx] float32 seafloor depth

    def params(self, workdir: str, shot: int = 1) -> List[str]:
        """key=value arguments for the reference's main / our drop-in main."""
        p = {
            "mode": "0",
            "freqs": ",".join(f"{f:g}" for f in self.freqs),
            "chsrc": ",".join(self.chsrc),
            "chrec": ",".join(self.chrec),
            "nx": str(self.nx), "ny": str(self.ny), "nz": str(self.nz),
            "dx": f"{self.dx:g}", "dy": f"{self.dy:g}", "dz": f"{self.dz:g}",
            "ox": f"{self.ox:g}", "oy": f"{self.oy:g}", "oz": f"{self.oz:g}",
            "n1": str(self.n[0]), "n2": str(self.n[1]), "n3": str(self.n[2]),
            "frho11": os.path.join(workdir, "frho11"),
            "frho22": os.path.join(workdir, "frho22"),
            "frho33": os.path.join(workdir, "frho33"),
            "fsrc": os.path.join(workdir, "sources.txt"),
            "frec": os.path.join(workdir, "receivers.txt"),
            "fsrcrec": os.path.join(workdir, "src_rec_table.txt"),
            "shots": str(shot),
            "verb": "0",
        }
        if self.bathy is not None:
            p["fbathy"] = os.path.join(workdir, "fbathy")
        p.update(self.extra)
        return [f"{k}={v}" for k, v in p.items()]

    def write(self, workdir: str) -> None:
        os.makedirs(workdir, exist_ok=True)
        for nm, arr in (("frho11", self.rho11), ("frho22", self.rho22),
                        ("frho33", self.rho33)):
            np.ascontiguousarray(arr, dtype=np.float32).tofile(os.path.join(workdir, nm))
        if self.bathy is not None:
            np.ascontiguousarray(self.bathy, dtype=np.float32).tofile(
                os.path.join(workdir, "fbathy"))
        _write_points(os.path.join(workdir, "sources.txt"), self.sources)
        _write_points(os.path.join(workdir, "receivers.txt"), self.receivers)
        with open(os.path.join(workdir, "src_rec_table.txt"), "w") as fp:
            fp.write("isrc irec\n")
            for s, r in self.pairs:
                fp.write(f"{int(s)} {int(r)}\n")

    @property
    def nshots(self) -> int:
        return int(self.sources.shape[0])


def _write_points(path: str, pts: np.ndarray) -> None:
    with open(path, "w") as fp:
        fp.write("x y z heading pitch idx\n")
        for i, (x, y, z, hd, pit) in enumerate(pts):
            fp.write(f"{x:.6f} {y:.6f} {z:.6f} {hd:.6f} {pit:.6f} {i + 1}\n")


def _layered(nz: int, ny: int, nx: int, oz: float, dz: float,
             layers: Sequence[tuple]) -> np.ndarray:
    """layers: (top_depth, rho) by cell-centre depth, ascending tops."""
    zc = oz + (np.arange(nz) + 0.5) * dz
    rho = np.empty(nz, np.float32)
    for k, z in enumerate(zc):
        val = layers[0][1]
        for top, r in layers:
            if z >= top:
                val = r
        rho[k] = val
    return np.broadcast_to(rho[:, None, None], (nz, ny, nx)).astype(np.float32).copy()


def all_pairs(nsrc: int, nrec: int) -> np.ndarray:
    s, r = np.meshgrid(np.arange(1, nsrc + 1), np.arange(1, nrec + 1), indexing="ij")
    return np.stack([s.ravel(), r.ravel()], axis=1)


# ---------------------------------------------------------------------------
# benchmark configurations
# ---------------------------------------------------------------------------
def config1(n: int = 64) -> Survey:
    """Plain GMG forward modelling, 1 shot, 1 Hz, Ex dipole 50 m above the
    seafloor; 101x101x51 model (100/100/40 m), layers water 0.3125 to
    1000 m, sediment 1, resistor 100 ohm-m 1480-1600 m, 1 below; 101 inline
    seafloor receivers at 100 m spacing; internal mesh n^3."""
    nx, ny, nz = 101, 101, 51
    rho = _layered(nz, ny, nx, 0.0, 40.0,
                   [(0.0, RHO_WATER), (1000.0, 1.0), (1480.0, 100.0), (1600.0, 1.0)])
    src = np.array([[0.0, 0.0, 950.0, 0.0, 0.0]], np.float32)
    rx = np.arange(-5000.0, 5000.0 + 1, 100.0)
    rec = np.stack([rx, np.zeros_like(rx), np.full_like(rx, 1000.0),
                    np.zeros_like(rx), np.zeros_like(rx)], axis=1)
    return Survey("c1_layered", nx, ny, nz, 100.0, 100.0, 40.0, -5050.0, -5050.0, 0.0,
                  rho, rho.copy(), rho.copy(), src, rec, all_pairs(1, len(rx)),
                  [1.0], (n, n, n))


def _smooth_field(rng: np.random.Generator, shape, sigma_cells) -> np.ndarray:
    """White noise Gaussian-filtered in Fourier space, unit variance."""
    w = rng.standard_normal(shape)
    f = np.fft.fftn(w)
    grids = np.meshgrid(*[np.fft.fftfreq(s) for s in shape], indexing="ij")
    k2 = sum((g * s) ** 2 for g, s in zip(grids, sigma_cells))
    sm = np.real(np.fft.ifftn(f * np.exp(-2.0 * np.pi ** 2 * k2)))
    sm -= sm.mean()
    sd = sm.std()
    return sm / (sd if sd > 0 else 1.0)


def config2(n: int = 96, seed: int = 2) -> Survey:
    """Batched plain GMG: 25 shots x 2 frequencies (0.25, 0.75 Hz), VTI
    sediment (rho33 = 2 rho11), Gaussian-filtered random bathymetry
    1000 +- 100 m, a 3x3x0.12 km 50 ohm-m box, sources on a 5x5 grid at 1 km,
    200 receivers on a 2 km grid, n^3 mesh."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = 200, 100, 100
    dx = dy = 200.0
    dz = 40.0
    ox, oy, oz = -20000.0, -10000.0, 0.0
    bath = 1000.0 + 100.0 * _smooth_field(rng, (ny, nx), (10.0, 10.0))
    bath = np.clip(bath, 850.0, 1150.0).astype(np.float32)
    zc = oz + (np.arange(nz) + 0.5) * dz
    xc = ox + (np.arange(nx) + 0.5) * dx
    yc = oy + (np.arange(ny) + 0.5) * dy
    below = zc[:, None, None] > bath[None, :, :]
    rho11 = np.where(below, 1.0, RHO_WATER).astype(np.float32)
    box = ((np.abs(xc)[None, None, :] <= 1500.0) & (np.abs(yc)[None, :, None] <= 1500.0)
           & ((zc >= 1800.0) & (zc <= 1920.0))[:, None, None])
    rho11 = np.where(box, 50.0, rho11).astype(np.float32)
    rho33 = np.where(below & ~box, 2.0 * rho11, rho11).astype(np.float32)
    sx, sy = np.meshgrid(np.arange(-2000.0, 2001.0, 1000.0), np.arange(-2000.0, 2001.0, 1000.0))
    sx, sy = sx.ravel(), sy.ravel()
    sz = np.array([_bath_at(bath, ox, oy, dx, dy, x, y) - 50.0 for x, y in zip(sx, sy)])
    src = np.stack([sx, sy, sz, np.zeros_like(sx), np.zeros_like(sx)], 1).astype(np.float32)
    rxg, ryg = np.meshgrid(np.arange(-19000.0, 19001.0, 2000.0), np.arange(-9000.0, 9001.0, 2000.0))
    rxg, ryg = rxg.ravel(), ryg.ravel()
    rz = np.array([_bath_at(bath, ox, oy, dx, dy, x, y) for x, y in zip(rxg, ryg)])
    rec = np.stack([rxg, ryg, rz, np.zeros_like(rxg), np.zeros_like(rxg)], 1).astype(np.float32)
    return Survey("c2_vti_bathy", nx, ny, nz, dx, dy, dz, ox, oy, oz, rho11, rho11.copy(),
                  rho33, src, rec, all_pairs(len(sx), len(rxg)), [0.25, 0.75], (n, n, n),
                  bathy=bath)


def _bath_at(bath, ox, oy, dx, dy, x, y) -> float:
    i = int(np.clip((x - ox) / dx, 0, bath.shape[1] - 1))
    j = int(np.clip((y - oy) / dy, 0, bath.shape[0] - 1))
    return float(np.float32(bath[j, i]))


def config3(n: int = 128, seed: int = 3) -> Survey:
    """Mixed-precision GMG at n^3: 1000 m water column over log-normal
    sediment (log10 rho ~ N(0, 0.3), 500 m correlation length), two
    resistive bodies of 20-100 ohm-m, 25 shots on a 5x5 grid at 1 km, 1 Hz."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = 100, 100, 60
    dx = dy = 100.0
    dz = 50.0
    ox, oy, oz = -5000.0, -5000.0, 0.0
    zc = oz + (np.arange(nz) + 0.5) * dz
    xc = ox + (np.arange(nx) + 0.5) * dx
    yc = oy + (np.arange(ny) + 0.5) * dy
    logr = 0.3 * _smooth_field(rng, (nz, ny, nx), (500.0 / dz, 500.0 / dy, 500.0 / dx))
    rho = (10.0 ** logr).astype(np.float32)
    rho[zc < 1000.0] = RHO_WATER
    for _ in range(2):
        cx, cy = rng.uniform(-3000, 3000, 2)
        cz = rng.uniform(1500, 2400)
        hx, hy, hz = rng.uniform(600, 1500), rng.uniform(600, 1500), rng.uniform(60, 200)
        val = rng.uniform(20.0, 100.0)
        m = ((np.abs(xc - cx)[None, None, :] <= hx) & (np.abs(yc - cy)[None, :, None] <= hy)
             & (np.abs(zc - cz)[:, None, None] <= hz))
        rho[m] = val
    rho = rho.astype(np.float32)
    sx, sy = np.meshgrid(np.arange(-2000.0, 2001.0, 1000.0), np.arange(-2000.0, 2001.0, 1000.0))
    sx, sy = sx.ravel(), sy.ravel()
    src = np.stack([sx, sy, np.full_like(sx, 950.0), np.zeros_like(sx), np.zeros_like(sx)],
                   1).astype(np.float32)
    rxg, ryg = np.meshgrid(np.arange(-4500.0, 4501.0, 1000.0), np.arange(-4500.0, 4501.0, 1000.0))
    rxg, ryg = rxg.ravel(), ryg.ravel()
    rec = np.stack([rxg, ryg, np.full_like(rxg, 1000.0), np.zeros_like(rxg),
                    np.zeros_like(rxg)], 1).astype(np.float32)
    return Survey("c3_lognormal", nx, ny, nz, dx, dy, dz, ox, oy, oz, rho, rho.copy(),
                  rho.copy(), src, rec, all_pairs(len(sx), len(rxg)), [1.0], (n, n, n))


def config5(n=(256, 256, 128), seed: int = 5) -> Survey:
    """Learned-smoother configuration: the log-normal model family of
    config3 (1000 m of water, log10 rho ~ N(0, 0.3) with 500 m correlation,
    two resistive bodies of 20-100 ohm-m) under 50 shots on a 10 x 5 grid at
    1 km, 1 Hz, 100 seafloor receivers, on a 256 x 256 x 128 mesh (about 25 M
    edge unknowns per right-hand side)."""
    s = config3(128, seed=seed)
    sx, sy = np.meshgrid(np.arange(-4500.0, 4501.0, 1000.0), np.arange(-2000.0, 2001.0, 1000.0))
    sx, sy = sx.ravel(), sy.ravel()
    src = np.stack([sx, sy, np.full_like(sx, 950.0), np.zeros_like(sx), np.zeros_like(sx)],
                   1).astype(np.float32)
    return Survey("c5_lognormal", s.nx, s.ny, s.nz, s.dx, s.dy, s.dz, s.ox, s.oy, s.oz, s.rho11,
                  s.rho22, s.rho33, src, s.receivers, all_pairs(len(sx), len(s.receivers)),
                  [1.0], tuple(n))


def config4(n: int = 128, seed: int = 4, true_model: bool = True) -> Survey:
    """Gradient mode: 25 shots x 3 frequencies (0.25, 0.5, 1 Hz), n^3 mesh.
    True model: a 100 ohm-m 4x4x0.1 km reservoir in 1 ohm-m sediment under
    1000 m water; start model: the 1 ohm-m half-space (true_model=False)."""
    nx, ny, nz = 100, 100, 60
    dx = dy = 100.0
    dz = 50.0
    ox, oy, oz = -5000.0, -5000.0, 0.0
    rho = _layered(nz, ny, nx, oz, dz, [(0.0, RHO_WATER), (1000.0, 1.0)])
    if true_model:
        zc = oz + (np.arange(nz) + 0.5) * dz
        xc = ox + (np.arange(nx) + 0.5) * dx
        yc = oy + (np.arange(ny) + 0.5) * dy
        m = ((np.abs(xc)[None, None, :] <= 2000.0) & (np.abs(yc)[None, :, None] <= 2000.0)
             & ((zc >= 1800.0) & (zc < 1900.0))[:, None, None])
        rho[m] = 100.0
    sx, sy = np.meshgrid(np.arange(-2000.0, 2001.0, 1000.0), np.arange(-2000.0, 2001.0, 1000.0))
    sx, sy = sx.ravel(), sy.ravel()
    src = np.stack([sx, sy, np.full_like(sx, 950.0), np.zeros_like(sx), np.zeros_like(sx)],
                   1).astype(np.float32)
    rxg, ryg = np.meshgrid(np.arange(-4500.0, 4501.0, 500.0), np.arange(-4500.0, 4501.0, 500.0))
    rxg, ryg = rxg.ravel(), ryg.ravel()
    rec = np.stack([rxg, ryg, np.full_like(rxg, 1000.0), np.zeros_like(rxg),
                    np.zeros_like(rxg)], 1).astype(np.float32)
    bath = np.full((ny, nx), 1000.0, np.float32)
    return Survey("c4_reservoir" if true_model else "c4_start", nx, ny, nz, dx, dy, dz,
                  ox, oy, oz, rho, rho.copy(), rho.copy(), src, rec,
                  all_pairs(len(sx), len(rxg)), [0.25, 0.5, 1.0], (n, n, n), bathy=bath)


# ---------------------------------------------------------------------------
# small cases for parity tests
# ---------------------------------------------------------------------------
def tiny_layered(n=(16, 16, 16), nb: int = 4, freq: float = 1.0) -> Survey:
    """A coarse version of the layered model: 21x21x11 cells of 500/500/200 m,
    water to 1000 m, 1 ohm-m sediment with a 100 ohm-m layer at 1400-1600 m."""
    nx, ny, nz = 21, 21, 11
    rho = _layered(nz, ny, nx, 0.0, 200.0,
                   [(0.0, RHO_WATER), (1000.0, 1.0), (1400.0, 100.0), (1600.0, 1.0)])
    src = np.array([[0.0, 0.0, 950.0, 0.0, 0.0]], np.float32)
    rx = np.arange(-5000.0, 5001.0, 500.0)
    rec = np.stack([rx, np.zeros_like(rx), np.full_like(rx, 1000.0),
                    np.zeros_like(rx), np.zeros_like(rx)], 1)
    return Survey("tiny_layered", nx, ny, nz, 500.0, 500.0, 200.0, -5250.0, -5250.0, 0.0,
                  rho, rho.copy(), rho.copy(), src, rec, all_pairs(1, len(rx)), [freq], n,
                  extra={"nb": str(nb), "d3min": "40"},
                  bathy=np.full((ny, nx), 1000.0, np.float32))


def tiny_aniso(n=(16, 16, 16), nb: int = 4, seed: int = 11) -> Survey:
    """Anisotropic random model with a rotated, tilted source and receivers:
    exercises the rotations, every channel and the VTI averaging."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = 20, 16, 12
    dx, dy, dz = 500.0, 500.0, 200.0
    ox, oy, oz = -5000.0, -4000.0, 0.0
    zc = oz + (np.arange(nz) + 0.5) * dz
    rho11 = (10.0 ** rng.uniform(-0.3, 0.7, (nz, ny, nx))).astype(np.float32)
    rho11[zc < 1000.0] = RHO_WATER
    rho22 = (rho11 * 10.0 ** rng.uniform(-0.1, 0.1, rho11.shape)).astype(np.float32)
    rho22[zc < 1000.0] = RHO_WATER
    rho33 = (2.0 * rho11).astype(np.float32)
    rho33[zc < 1000.0] = RHO_WATER
    src = np.array([[250.0, -300.0, 940.0, 30.0, 10.0]], np.float32)
    pts = []
    for x in np.arange(-4000.0, 4001.0, 1000.0):
        for y in (-1000.0, 500.0):
            pts.append([x, y, 1000.0, 15.0 + x / 400.0, -5.0])
    rec = np.array(pts, np.float32)
    return Survey("tiny_aniso", nx, ny, nz, dx, dy, dz, ox, oy, oz, rho11, rho22, rho33,
                  src, rec, all_pairs(1, len(rec)), [0.5], n,
                  chsrc=("Ex", "Ey", "Ez"), chrec=("Ex", "Ey", "Ez", "Hx", "Hy", "Hz"),
                  extra={"nb": str(nb), "d3min": "40"},
                  bathy=np.full((ny, nx), 1000.0, np.float32))
