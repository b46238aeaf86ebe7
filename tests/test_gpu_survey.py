"""Device injection, extraction and gradient against the reference's own
outputs (golden fixtures), through the C ABI.

The survey unit is compiled without FMA contraction and follows the
reference's operand order, so results match to the last bits; double cos/sin
of rotated channels may differ from the host libm by an ulp, hence
tolerances of a few ulps rather than exact equality where rotations enter.
"""
import ctypes as C

import numpy as np
import pytest

from _cases import golden_level

gpu = pytest.mark.gpu


def _solver(g, nrhs=1):
    from libemmi_mgfd_gb300 import gpu as G
    n, x, raw, om = golden_level(g)
    return G.Solver(n, *[v.astype(np.float32) for v in x], raw[None],
                    np.full(nrhs, om, np.float32), op=np.zeros(nrhs, np.int32),
                    rho_water=float(g["rho_water"][0]))


def _dev(a):
    import torch
    t = torch.from_numpy(np.ascontiguousarray(a)).cuda()
    return t


def _chans(names):
    from libemmi_mgfd_gb300.gpu import CHANNELS
    return np.array([CHANNELS[c] for c in names], np.int32)


def _close(a, b, tol):
    a, b = np.asarray(a).ravel(), np.asarray(b).ravel()
    return np.abs(a - b).max() <= tol * max(np.abs(b).max(), 1e-300)


@gpu
@pytest.mark.parametrize("name", ["tiny_layered", "tiny_aniso"])
def test_inject_source_matches_reference(golden, name):
    import torch
    from libemmi_mgfd_gb300 import gpu as G
    g = golden(name)
    s = _solver(g)
    src = _dev(g["srcrec"][:5].astype(np.float32))
    b = torch.zeros(g["b_f0"].size * 2, dtype=torch.float64, device="cuda")
    ch = _chans(str(g["chsrc"]).split(","))
    rc = G.lib().emmi_inject_sources_dev(s._h, C.c_void_p(src.data_ptr()), len(ch),
                                         ch.ctypes.data_as(C.c_void_p), C.c_void_p(b.data_ptr()))
    assert rc == 0
    torch.cuda.synchronize()
    got = b.cpu().numpy().view(np.complex128)
    if name == "tiny_layered":  # azimuth = dip = 0: no rotation error at all
        assert np.array_equal(got, g["b_f0"])
    else:
        assert _close(got, g["b_f0"], 1e-14)


@gpu
@pytest.mark.parametrize("name", ["tiny_layered", "tiny_aniso"])
def test_extract_receivers_matches_reference(golden, name):
    import torch
    from libemmi_mgfd_gb300 import gpu as G
    g = golden(name)
    s = _solver(g)
    ch = _chans(str(g["chrec"]).split(","))
    rec = g["srcrec"][5:].reshape(-1, 5).astype(np.float32)
    drec = _dev(rec)
    x = _dev(g["x_f0"].view(np.float64))
    h = _dev(g["h_f0"].view(np.float64))
    out = torch.zeros(len(ch) * rec.shape[0] * 2, dtype=torch.float32, device="cuda")
    rc = G.lib().emmi_extract_receivers_dev(s._h, C.c_void_p(drec.data_ptr()), rec.shape[0],
                                            len(ch), ch.ctypes.data_as(C.c_void_p),
                                            C.c_void_p(x.data_ptr()), C.c_void_p(h.data_ptr()),
                                            C.c_void_p(out.data_ptr()))
    assert rc == 0
    torch.cuda.synchronize()
    got = out.cpu().numpy().view(np.complex64)
    if name == "tiny_layered":
        assert np.array_equal(got, g["dcal"])
    else:
        assert _close(got, g["dcal"], 1e-6)


@gpu
@pytest.mark.parametrize("name", ["tiny_layered", "tiny_aniso"])
def test_volume_extraction_matches_reference(golden, name):
    g = golden(name)
    s = _solver(g)
    nxyz = tuple(int(v) for v in g["nxyz"])
    E = s.extract_volume(0, 0, nxyz, g["o"], g["dxyz"], g["x_f0"], rho33=g["rho33"])
    H = s.extract_volume(0, 1, nxyz, g["o"], g["dxyz"], g["h_f0"])
    for a, nm in zip(E + H, ("E1", "E2", "E3", "H1", "H2", "H3")):
        assert np.array_equal(a.ravel(), g[nm]), nm


@gpu
def test_inject_adjoint_matches_reference(golden):
    import torch
    from libemmi_mgfd_gb300 import gpu as G
    g = golden("tiny_layered")
    s = _solver(g)
    ch = _chans(str(g["chrec"]).split(","))
    rec = g["srcrec"][5:].reshape(-1, 5).astype(np.float32)
    drec = _dev(rec)
    dres = _dev(g["dres"].view(np.float32))
    b = torch.zeros(g["b_f0"].size * 2, dtype=torch.float64, device="cuda")
    m = torch.zeros_like(b)
    rc = G.lib().emmi_inject_adjoint_dev(s._h, C.c_void_p(drec.data_ptr()), rec.shape[0], len(ch),
                                         ch.ctypes.data_as(C.c_void_p),
                                         C.c_void_p(dres.data_ptr()), C.c_void_p(b.data_ptr()),
                                         C.c_void_p(m.data_ptr()))
    assert rc == 0
    torch.cuda.synchronize()
    assert np.array_equal(m.cpu().numpy().view(np.complex128), g["madj_f0"])
    assert _close(b.cpu().numpy().view(np.complex128), g["badj_f0"], 1e-15)


@gpu
def test_gradient_matches_reference(golden):
    from libemmi_mgfd_gb300 import gpu as G
    g = golden("tiny_layered")
    nx, ny, nz = (int(v) for v in g["nxyz"])
    shp = (1, 1, nz, ny, nx)
    Ef = [g[k].reshape(shp) for k in ("E1", "E2", "E3")]
    Ea = [g[k].reshape(shp) for k in ("E1a", "E2a", "E3a")]
    rec = g["srcrec"][5:].reshape(-1, 5)[None, :, :3]
    bathy = np.full((ny, nx), float(g["bathy"]), np.float32)
    grad, phess = G.build_gradient((nx, ny, nz), g["o"], g["dxyz"], [1, 2], 1, Ef, Ea,
                                   g["rho11"], g["rho33"], bathy, g["srcrec"][None, :3], rec)
    assert np.array_equal(grad.ravel(), g["grad"])
    assert _close(phess, g["phess"], 1e-6)


@gpu
def test_gradient_shot_sum_is_linear(golden):
    """Two identical shots give twice the one-shot gradient (the device
    reduction over shots replaces the reference's MPI_Allreduce)."""
    from libemmi_mgfd_gb300 import gpu as G
    g = golden("tiny_layered")
    nx, ny, nz = (int(v) for v in g["nxyz"])
    shp = (1, 1, nz, ny, nx)
    Ef = [np.concatenate([g[k].reshape(shp)] * 2) for k in ("E1", "E2", "E3")]
    Ea = [np.concatenate([g[k].reshape(shp)] * 2) for k in ("E1a", "E2a", "E3a")]
    rec = np.concatenate([g["srcrec"][5:].reshape(-1, 5)[None, :, :3]] * 2)
    src = np.concatenate([g["srcrec"][None, :3]] * 2)
    bathy = np.full((ny, nx), float(g["bathy"]), np.float32)
    grad2, _ = G.build_gradient((nx, ny, nz), g["o"], g["dxyz"], [1, 2], 0, Ef, Ea, g["rho11"],
                                g["rho33"], bathy, src, rec)
    assert np.array_equal(grad2.ravel(), 2 * g["grad"])


@gpu
def test_modelling_batch_end_to_end(golden):
    """Host model in, receiver data out through one C-ABI call, against the
    reference's receiver data."""
    g = golden("tiny_layered")
    from libemmi_mgfd_gb300 import gpu as G
    n, x, raw, om = golden_level(g)
    s = G.Solver(n, *[v.astype(np.float32) for v in x], raw[None], np.array([om], np.float32),
                 options=G.Options(precision=G.PREC_MIXED, ncycle=120, tol=1e-10),
                 rho_water=float(g["rho_water"][0]))
    rec = g["srcrec"][5:].reshape(-1, 5)
    ch = str(g["chrec"]).split(",")
    d, st, (h2d, d2h) = s.modelling(g["srcrec"][:5][None], rec, chsrc=str(g["chsrc"]).split(","),
                                    chrec=ch)
    assert st[0]["status"] == "ok"
    from test_gpu_solver import receiver_parity
    amp, ph = receiver_parity(d[0], g["dcal"], ch)
    assert amp < 1e-4 and ph < 0.05, (amp, ph)
    assert h2d == 5 * 4 + rec.size * 4 and d2h == d.nbytes
