"""The front end on the device (emmi_homogenize_batch): the per-shot cells
of a batch, homogenized on the GPU, are the host front end's (eh_regrid)
bit for bit; the host front end is itself pinned to the reference's
regrid stage (tests/test_host_frontend.py).  The padded model and the
axes come from the host library's split of eh_regrid."""
import numpy as np
import pytest

gpu = pytest.mark.gpu


def _model(n=64):
    from libemmi_mgfd_gb300 import host, workloads as W
    s = W.config3(n)
    return s, host.Model.from_survey(s)


def test_split_axes_equal_regrid():
    s, m = _model()
    padded = m.padded()
    for p in s.sources[:3]:
        ref = m.regrid(float(p[0]), float(p[1]), float(p[2]))
        ax = m.axes(*padded[:3], float(p[0]), float(p[1]), float(p[2]))
        for nm, v in ax.items():
            assert np.array_equal(v, ref[nm]), nm


@gpu
def test_device_homogenization_matches_host_bitwise():
    import torch
    from libemmi_mgfd_gb300 import gpu as G
    s, m = _model()
    padded = m.padded()
    src = s.sources[[0, 7, 24]]
    axes = [m.axes(*padded[:3], float(p[0]), float(p[1]), float(p[2])) for p in src]
    n = (m.n1, m.n2, m.n3)
    nc = m.n1 * m.n2 * m.n3
    cells = torch.full((len(src), 4, nc), -1.0, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    G.homogenize_batch(padded, axes, n, cells.data_ptr())
    got = cells.cpu().numpy()
    for k, p in enumerate(src):
        ref = m.regrid(float(p[0]), float(p[1]), float(p[2]))
        for a, nm in enumerate(("sigma11", "sigma22", "sigma33", "invmur")):
            assert np.array_equal(got[k, a], ref[nm]), (k, nm, np.abs(got[k, a] - ref[nm]).max())


@gpu
def test_solver_from_device_cells_equals_host_cells():
    """emmi_solver_create_dc on the device cells gives the host-array
    solver's solution."""
    import torch
    from libemmi_mgfd_gb300 import gpu as G
    s, m = _model()
    padded = m.padded()
    src = s.sources[:2]
    axes = [m.axes(*padded[:3], float(p[0]), float(p[1]), float(p[2])) for p in src]
    n = (m.n1, m.n2, m.n3)
    nc = m.n1 * m.n2 * m.n3
    cells = torch.zeros((len(src), 4, nc), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    G.homogenize_batch(padded, axes, n, cells.data_ptr())
    X = [np.stack([a[k] for a in axes]) for k in ("x1", "x2", "x3")]
    om = np.full(len(src), 2 * np.pi * 1.0, np.float32)
    opt = G.Options(precision=G.PREC_MIXED, ncycle=4, tol=0.0)
    rng = np.random.default_rng(4)
    b = rng.standard_normal((len(src), 3 * (m.n1 + 1) ** 3)) + 0j
    sd = G.Solver(n, *X, cells.data_ptr(), om, options=opt)
    xd, hd, _ = sd.solve(b)
    sd.close()
    sh = G.Solver(n, *X, cells.cpu().numpy(), om, options=opt)
    xh, hh, _ = sh.solve(b)
    sh.close()
    assert np.array_equal(xd, xh)
