"""Single-operator parity of the CUDA kernels against the CPU oracle, through
the C ABI (emmi_level_residual / emmi_level_smooth).

The smoothers are compared against the oracle's multicolour ordering (the
order the GPU computes); the oracle's lexicographic order is the
reference's and is pinned separately in test_oracle_golden.py.
FP64 tolerances are roundoff-level; complex64 tolerances are relative to the
largest entry and allow for single-precision block solves.
"""
import numpy as np
import pytest

import oracle as O
from _cases import random_level, rel_err, unknown_mask

gpu = pytest.mark.gpu


def _gpu():
    from libemmi_mgfd_gb300 import gpu as G
    return G


SHAPES = [(8, 6, 10), (12, 12, 12), (16, 8, 4)]


@gpu
@pytest.mark.parametrize("n", SHAPES)
@pytest.mark.parametrize("air", [False, True])
def test_residual_fp64(n, air):
    G = _gpu()
    n, x, raw, cells, om, u, f = random_level(n, seed=1, air=air)
    L = O.Level(n, x, cells[:3], cells[3], om)
    r_ref = L.residual(u, f)
    r, nrm = G.level_residual(n, x, cells, om, u, f, prec=G.PREC_FP64)
    assert rel_err(r, r_ref) < 1e-13
    assert abs(nrm - np.linalg.norm(r_ref)) <= 1e-12 * np.linalg.norm(r_ref)


@gpu
@pytest.mark.parametrize("n", SHAPES)
def test_residual_c64(n):
    G = _gpu()
    n, x, raw, cells, om, u, f = random_level(n, seed=2)
    L = O.Level(n, x, cells[:3], cells[3], om)
    r_ref = L.residual(u, f)
    r, _ = G.level_residual(n, x, cells, om, u, f, prec=G.PREC_MIXED)
    # complex64 residual: relative to the operator scale |A||u|
    scale = np.abs(L.apply(u)).max() + np.abs(f).max()
    assert np.abs(r - r_ref).max() / scale < 2e-6


@gpu
@pytest.mark.parametrize("n", SHAPES)
@pytest.mark.parametrize("direction", [0, 1, 2])
@pytest.mark.parametrize("it", [0, 1])
def test_line_sweep_fp64(n, direction, it):
    G = _gpu()
    n, x, raw, cells, om, u, f = random_level(n, seed=3 + direction)
    u = u * unknown_mask(n).ravel()  # boundary slots hold zero
    L = O.Level(n, x, cells[:3], cells[3], om)
    ref = L.line_sweep(u, f, direction, ordering=O.ORDER_COLOR, iter=it)
    got = G.level_smooth(n, x, cells, om, u, f, direction, prec=G.PREC_FP64, iter=it)
    assert rel_err(got, ref) < 1e-10


@gpu
@pytest.mark.parametrize("n", SHAPES)
@pytest.mark.parametrize("it", [0, 1])
def test_point_sweep_fp64(n, it):
    G = _gpu()
    n, x, raw, cells, om, u, f = random_level(n, seed=7)
    u = u * unknown_mask(n).ravel()
    L = O.Level(n, x, cells[:3], cells[3], om)
    ref = L.point_sweep(u, f, ordering=O.ORDER_COLOR, iter=it)
    got = G.level_smooth(n, x, cells, om, u, f, 3, prec=G.PREC_FP64, iter=it)
    assert rel_err(got, ref) < 1e-10


@gpu
@pytest.mark.parametrize("direction", [0, 1, 2, 3])
def test_sweeps_c64(direction):
    G = _gpu()
    n, x, raw, cells, om, u, f = random_level((12, 10, 8), seed=11)
    u = u * unknown_mask(n).ravel()
    L = O.Level(n, x, cells[:3], cells[3], om)
    if direction < 3:
        ref = L.line_sweep(u, f, direction, ordering=O.ORDER_COLOR)
    else:
        ref = L.point_sweep(u, f, ordering=O.ORDER_COLOR)
    got = G.level_smooth(n, x, cells, om, u, f, direction, prec=G.PREC_MIXED)
    # complex64 block solves on cells stretched 3x with conductivity over
    # three decades: the 6x6 patch systems are the worse conditioned
    assert rel_err(got, ref) < (1e-4 if direction < 3 else 5e-4)


@gpu
def test_sweep_reduces_residual():
    """A smoothing sweep on an unknown-restricted field lowers the residual."""
    G = _gpu()
    n, x, raw, cells, om, u, f = random_level((16, 16, 16), seed=5)
    u = np.zeros_like(u)
    f = f * unknown_mask(n).ravel()
    r0 = np.linalg.norm(G.level_residual(n, x, cells, om, u, f, prec=G.PREC_FP64)[0])
    for d in (0, 1, 2):
        u = G.level_smooth(n, x, cells, om, u, f, d, prec=G.PREC_FP64)
    r1 = np.linalg.norm(G.level_residual(n, x, cells, om, u, f, prec=G.PREC_FP64)[0])
    assert r1 < 0.5 * r0


XFER = [((8, 6, 10), (1, 2, 2)), ((12, 12, 12), (2, 1, 2)), ((16, 8, 4), (2, 2, 1)),
        ((8, 8, 8), (2, 2, 2))]


@gpu
@pytest.mark.parametrize("n,sc", XFER)
@pytest.mark.parametrize("prec", [0, 1])
def test_restriction_and_prolongation(n, sc, prec):
    """One restriction and one prolongation (emmi_level_transfer: the
    solver's kernels with the level's weight table) against the oracle's
    (src/gmg.c:1463-1573) on stretched coordinates, for the semi-coarsening
    masks of the three hierarchies and full coarsening.  The coarse
    coordinates are the fine ones sub-sampled, as the hierarchy builds them."""
    G = _gpu()
    n, x, raw, cells, om, u, f = random_level(n, seed=7)
    nc = tuple(a // b for a, b in zip(n, sc))
    xc = [np.asarray(x[e])[::sc[e]].copy() for e in range(3)]
    rng = np.random.default_rng(8)
    sc_n = 3 * (nc[0] + 1) * (nc[1] + 1) * (nc[2] + 1)
    uc = rng.standard_normal(sc_n) + 1j * rng.standard_normal(sc_n)
    fc_ref = O.restrict(n, x, nc, xc, sc, f)
    fc = G.level_transfer(n, x, sc, f, np.zeros(sc_n, np.complex128), 0, prec)
    pf_ref = O.prolong(n, x, nc, xc, sc, uc, u)
    pf = G.level_transfer(n, x, sc, uc, u, 1, prec)
    tol = 1e-14 if prec == G.PREC_FP64 else 2e-6
    assert rel_err(fc, fc_ref) < tol
    assert rel_err(pf, pf_ref) < tol
