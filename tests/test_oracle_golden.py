"""The CPU oracle against the reference's own outputs (tests/golden/, made by
the reference compiled from its sources).  This pins the oracle before it
checks the CUDA path.

Below the sea surface and in H the oracle reproduces the reference to
roundoff; in the air layer (sigma = 1e-8 S/m) the curl-free part of E is
determined only weakly by the residual and carries roundoff amplified by the
operator's near-null space, so E there is compared at a looser bound.
"""
import numpy as np
import pytest

import oracle as O
from _cases import below_sea_mask, golden_level, rel_err


def _solve_like_fixture(g, **kw):
    n, x, raw, om = golden_level(g)
    return O.gmg_solve(n, *[v.astype(np.float32) for v in x], *raw, om, g["b_f0"], **kw)


@pytest.mark.parametrize("name,kw", [
    ("tiny_layered_it3", dict(ncycle=3, tol=0.0)),
    ("tiny_vcycle_it3", dict(ncycle=3, tol=0.0, cycleopt=1)),
    ("tiny_wcycle_it2", dict(ncycle=2, tol=0.0, cycleopt=3)),
    ("tiny_point_it3", dict(ncycle=3, tol=0.0, isemicoarsen=0)),
])
def test_iterates_match_reference(oracle_lib, golden, name, kw):
    g = golden(name)
    x, h, nc, hist = _solve_like_fixture(g, **kw)
    n = tuple(g["n"])
    sea = below_sea_mask(n, g["x3"])
    assert rel_err(x, g["x_f0"], sea) < 1e-12
    assert rel_err(h, g["h_f0"]) < 1e-12
    assert rel_err(x, g["x_f0"]) < 1e-8  # air layer included


@pytest.mark.parametrize("name,ncycle", [("tiny_layered", 60), ("tiny_aniso", 80)])
def test_converged_solution_and_cycle_count(oracle_lib, golden, name, ncycle):
    g = golden(name)
    x, h, nc, hist = _solve_like_fixture(g, ncycle=ncycle, tol=1e-10)
    ref = g["rnorm_fwd"]  # printed by the reference, 7 significant digits
    assert nc == len(ref) - 1  # lines icycle=0..k, the solve stops at k
    np.testing.assert_allclose(hist[: len(ref)], ref, rtol=2e-6)
    sea = below_sea_mask(tuple(g["n"]), g["x3"])
    assert rel_err(x, g["x_f0"], sea) < 1e-11
    assert rel_err(h, g["h_f0"]) < 1e-11


def _grid(g):
    n = tuple(int(v) for v in g["n"])
    return O.Grid(n, g["x1"], g["x2"], g["x3"], g["x1s"], g["x2s"], g["x3s"], g["d1"], g["d2"],
                  g["d3"], g["sigma33"], float(g["rho_water"][0]))


@pytest.mark.parametrize("name", ["tiny_layered", "tiny_aniso"])
def test_injection_bitwise(oracle_lib, golden, name):
    g = golden(name)
    src = g["srcrec"][:5]
    b = O.inject_source(_grid(g), src, str(g["chsrc"]).split(","), float(g["omegas"][0]))
    assert np.array_equal(b, g["b_f0"])


@pytest.mark.parametrize("name", ["tiny_layered", "tiny_aniso"])
def test_receiver_extraction_bitwise(oracle_lib, golden, name):
    g = golden(name)
    rec = g["srcrec"][5:].reshape(-1, 5)
    ch = str(g["chrec"]).split(",")
    d = O.extract_emf_data(_grid(g), rec, ch, g["x_f0"], g["h_f0"])
    assert np.array_equal(d.ravel(), g["dcal"])


@pytest.mark.parametrize("name", ["tiny_layered", "tiny_aniso"])
def test_volume_extraction_bitwise(oracle_lib, golden, name):
    g = golden(name)
    nx, ny, nz = (int(v) for v in g["nxyz"])
    E = O.extract_electric_field(_grid(g), (nx, ny, nz), g["o"], g["dxyz"], g["rho33"], g["x_f0"])
    H = O.extract_magnetic_field(_grid(g), (nx, ny, nz), g["o"], g["dxyz"], g["h_f0"])
    for a, nm in zip(E + H, ("E1", "E2", "E3", "H1", "H2", "H3")):
        assert np.array_equal(a.ravel(), g[nm]), nm


def test_adjoint_injection_and_gradient(oracle_lib, golden):
    g = golden("tiny_layered")
    rec = g["srcrec"][5:].reshape(-1, 5)
    ch = str(g["chrec"]).split(",")
    dres = g["dres"].reshape(len(ch), -1)
    m, b = O.inject_adj_source(_grid(g), rec, ch, dres, float(g["omegas"][0]))
    assert np.array_equal(b, g["badj_f0"])
    assert np.array_equal(m, g["madj_f0"])
    nx, ny, nz = (int(v) for v in g["nxyz"])
    bathy = np.full((ny, nx), float(g["bathy"]), np.float32)
    grad, phess = O.build_gradient(
        (nx, ny, nz), g["o"], g["dxyz"], [1, 2], 1,
        [g["E1"], g["E2"], g["E3"]], [g["E1a"], g["E2a"], g["E3a"]],
        g["rho11"], g["rho33"], bathy, g["srcrec"][:5], rec)
    assert np.array_equal(grad.ravel(), g["grad"])
    assert np.array_equal(phess.ravel(), g["phess"])


def test_adjoint_solve_matches(oracle_lib, golden):
    g = golden("tiny_layered")
    n, x, raw, om = golden_level(g)
    xa, h, nc, hist = O.gmg_solve(n, *[v.astype(np.float32) for v in x], *raw, om, g["badj_f0"],
                                  ncycle=60, tol=1e-10)
    sea = below_sea_mask(n, g["x3"])
    assert rel_err(xa, g["xa_f0"], sea) < 1e-11


def test_find_index_matches_search_rule(oracle_lib):
    x = np.array([0.0, 1.0, 2.5, 4.0, 9.0], np.float32)
    for v, k in [(0.0, 0), (0.5, 0), (1.0, 1), (2.49, 1), (2.5, 2), (8.9, 3), (9.0, 3), (12.0, 3),
                 (-1.0, 0)]:
        assert O.find_index(x, v) == k
