"""Helpers shared by the parity tests: level data from golden fixtures and
seeded random levels."""
from __future__ import annotations

import numpy as np


def stagger(x):
    x = np.asarray(x, np.float64)
    n = len(x) - 1
    ds = np.empty(n + 1)
    xs = np.empty(n + 1)
    ds[:n] = x[1:] - x[:-1]
    xs[:n] = 0.5 * (x[:-1] + x[1:])
    xs[n] = x[n] + 0.5 * ds[n - 1]
    ds[n] = xs[n] - x[n]
    d = np.empty(n + 1)
    d[1:] = xs[1:] - xs[:-1]
    d[0] = xs[0] - x[0]
    return xs, d, ds


def weighted_cells(n, x, raw):
    """raw float32 [4, n3, n2, n1] -> volume weighted float64 (gmg.c:1791-1802)."""
    n1, n2, n3 = n
    ds = [stagger(v)[2] for v in x]
    vol = (ds[0][None, None, :n1] * ds[1][None, :n2, None]) * ds[2][:n3, None, None]
    raw = np.asarray(raw).reshape(4, n3, n2, n1)
    return (raw.astype(np.float64) * vol[None]).reshape(4, -1)


def dual_volumes(n, x):
    n1, n2, n3 = n
    st = [stagger(v) for v in x]
    d = [s[1] for s in st]
    ds = [s[2] for s in st]
    dv = np.empty((3, n3 + 1, n2 + 1, n1 + 1))
    dv[0] = (ds[0][None, None, :] * d[1][None, :, None]) * d[2][:, None, None]
    dv[1] = (d[0][None, None, :] * ds[1][None, :, None]) * d[2][:, None, None]
    dv[2] = (d[0][None, None, :] * d[1][None, :, None]) * ds[2][:, None, None]
    return dv.ravel()


def golden_level(g):
    """(n, x[3] float64, raw cells [4,ncell] float32, omega) of a fixture."""
    n = tuple(int(v) for v in g["n"])
    x = [g["x1"].astype(np.float64), g["x2"].astype(np.float64), g["x3"].astype(np.float64)]
    raw = np.stack([g["sigma11"], g["sigma22"], g["sigma33"], g["invmur"]]).astype(np.float32)
    return n, x, raw, float(g["omegas"][0])


def random_level(n, seed, air=False, stretch=3.0):
    """A seeded level with stretched spacings and random conductivity."""
    rng = np.random.default_rng(seed)
    x = []
    for e in range(3):
        h = 50.0 * stretch ** rng.uniform(0, 1, n[e])
        x.append(np.concatenate([[0.0], np.cumsum(h)]) - 1000.0)
    n1, n2, n3 = n
    sig = 10.0 ** rng.uniform(-2.5, 0.5, (3, n3, n2, n1))
    if air:
        sig[:, : max(1, n3 // 4)] = 1e-8
    raw = np.concatenate([sig, np.ones((1, n3, n2, n1))]).astype(np.float32)
    cells = weighted_cells(n, x, raw)
    S = (n1 + 1) * (n2 + 1) * (n3 + 1)
    u = rng.standard_normal(3 * S) + 1j * rng.standard_normal(3 * S)
    f = rng.standard_normal(3 * S) + 1j * rng.standard_normal(3 * S)
    omega = float(np.float32(2 * np.pi * 0.5))
    return n, x, raw, cells, omega, u, f


def unknown_mask(n):
    """Boolean [3, S] mask of the edge unknowns (interior tangential E)."""
    n1, n2, n3 = n
    k, j, i = np.meshgrid(np.arange(n3 + 1), np.arange(n2 + 1), np.arange(n1 + 1), indexing="ij")
    P = [i, j, k]
    m = []
    for c in range(3):
        p, q = (c + 1) % 3, (c + 2) % 3
        m.append((P[c] < n[c]) & (P[p] >= 1) & (P[p] < n[p]) & (P[q] >= 1) & (P[q] < n[q]))
    return np.stack(m).reshape(3, -1)


def below_sea_mask(n, x3):
    """[3, S] mask of slots at or below z = 0 (outside the air layer)."""
    n1, n2, n3 = n
    z = np.asarray(x3)
    m = np.broadcast_to((z >= 0)[:, None, None], (n3 + 1, n2 + 1, n1 + 1))
    return np.stack([m, m, m]).reshape(3, -1)


def rel_err(a, b, mask=None):
    a = np.asarray(a).reshape(-1)
    b = np.asarray(b).reshape(-1)
    if mask is not None:
        mask = np.asarray(mask).reshape(-1)
        a, b = a[mask], b[mask]
    den = np.abs(b).max()
    return float(np.abs(a - b).max() / (den if den > 0 else 1.0))
