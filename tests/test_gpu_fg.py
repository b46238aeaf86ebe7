"""The batched objective evaluation through its Python wrapper (gpu.Fg over
emmi_fg_create / emmi_fg_eval) against the reference's own mode=2 run on
the layered case: gradient (both parameters), misfit and rmse."""
import dataclasses

import numpy as np
import pytest

from libemmi_mgfd_gb300 import host
from libemmi_mgfd_gb300 import workloads as W

gpu = pytest.mark.gpu


@gpu
@pytest.mark.parametrize("prec,tol", [(0, 1e-10), (1, 1e-9)])
def test_fg_gradient_matches_reference(golden, prec, tol):
    from libemmi_mgfd_gb300 import gpu as G
    from test_misfit import parse_data
    g = golden("tiny_grad")
    true = W.tiny_layered()
    rho = np.asarray(g["rho_start"], np.float32)
    start = dataclasses.replace(true, rho11=rho, rho22=rho.copy(), rho33=rho.copy())
    ms = host.Model.from_survey(start)
    ch = list(start.chrec)
    nrec = len(start.receivers)
    dobs = parse_data(str(g["obs_text"]), ch, 1, nrec)
    az = np.float32(np.pi * start.receivers[:, 3] / 180.0)
    delta = host.uncertainty(ch, dobs, az, np.float32(0.0))
    f = G.Fg(ms, start, dobs[None], delta[None], start.bathy,
             options=G.Options(precision=prec, tol=tol, ncycle=120))
    fcost, grad, phess, dcal, rmse, cyc = f.eval(ms)
    f.close()
    for k, nm in enumerate(("grad_Rv", "grad_Rh")):
        ref = np.asarray(g[nm], np.float32)
        ours = grad[k].ravel()
        l2 = np.linalg.norm(ours - ref) / np.linalg.norm(ref)
        mx = np.abs(ours - ref).max() / np.abs(ref).max()
        print(f"{nm}: L2 {l2:.2e}, max {mx:.2e}")
        assert l2 < 1e-3 and mx < 1e-3, (nm, l2, mx)
    assert abs(fcost[0] - float(g["fcost"][0])) <= 1e-4 * float(g["fcost"][0])
    ref = np.asarray(g["rmse"]).reshape(rmse[0].shape)
    assert np.array_equal(rmse[0] == 0, ref == 0)
    live = ref > 0
    # data that nearly cancel (rmse near 0) carry the synthetic data's own
    # 1e-6 difference: an absolute floor at 1e-5 of the largest rmse
    np.testing.assert_allclose(rmse[0][live], ref[live], rtol=1e-4, atol=1e-5 * ref.max())
    assert (phess > 0).any() and (cyc > 0).all()


@gpu
def test_gradient_matches_finite_differences():
    """The adjoint gradient of the data misfit w.r.t. ln(rho) (both
    parameters) against central finite differences of the misfit (step 0.1
    in ln rho) on 10 random cells below the sea floor, outside the source
    and receiver mutes, with at least 5 % of the largest gradient (32^3
    mesh, FP64 solves to 1e-12; observed data from the resistive-layer model
    with 1 % seeded Gaussian noise; the gradient at the start model without
    the layer).  The misfit of the differences is recomputed in float64
    from the returned receiver data.

    The reference's gradient (which this one reproduces to 1e-5) takes the
    forward and adjoint fields at each 500 m input cell's centre, not their
    average through the homogenization, so it is the derivative of the
    discrete misfit only to within tens of percent where the fields decay
    steeply: the check is the sign on every cell, each ratio within a
    factor 2, and the direction over the cells (cosine >= 0.95)."""
    from libemmi_mgfd_gb300 import gpu as G
    true = W.tiny_layered(n=(32, 32, 32))
    rho = true.rho11.copy()
    rho[rho == 100.0] = 1.0
    start = dataclasses.replace(true, rho11=rho, rho22=rho.copy(), rho33=rho.copy())
    mt, ms = host.Model.from_survey(true), host.Model.from_survey(start)
    nch, nrec = len(true.chrec), len(true.receivers)
    shape = (1, nch, 1, nrec)
    opts = G.Options(precision=G.PREC_FP64, tol=1e-12, ncycle=200)
    f = G.Fg(mt, true, np.zeros(shape, np.complex64), np.ones(shape, np.float32), true.bathy,
             options=opts)
    d_true = f.eval(mt)[3]
    f.close()
    rng = np.random.default_rng(7)
    noise = (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) / np.sqrt(2)
    dobs = (d_true * (1 + 0.01 * noise)).astype(np.complex64)
    az = np.float32(np.pi * true.receivers[:, 3] / 180.0)
    delta = host.uncertainty(list(true.chrec), dobs[0], az, np.float32(0.0))[None]
    f = G.Fg(ms, start, dobs, delta, start.bathy, options=opts)
    fc, grad, _, dcal, rmse, _ = f.eval(ms)
    live = rmse > 0

    def misfit(model):
        d = f.eval(model)[3]
        r = (dobs.astype(np.complex128) - d) / delta
        return 0.5 * float(np.sum(np.abs(r[live]) ** 2))

    assert abs(misfit(ms) - float(fc[0])) <= 1e-5 * float(fc[0])
    nz, ny, nx = rho.shape
    zc = start.oz + (np.arange(nz) + 0.5) * start.dz
    xc = start.ox + (np.arange(nx) + 0.5) * start.dx
    yc = start.oy + (np.arange(ny) + 0.5) * start.dy
    adj, fds = [], []
    for kp, names in ((0, ("rho11", "rho22")), (1, ("rho33",))):
        gmax = np.abs(grad[kp]).max()
        cand = [(k, j, i) for k in range(nz) for j in range(ny) for i in range(nx)
                if zc[k] > 1400 and abs(xc[i]) <= 2500 and 600 <= abs(yc[j]) <= 2500
                and abs(grad[kp, k, j, i]) >= 0.05 * gmax]
        for q in rng.choice(len(cand), 5, replace=False):
            k, j, i = cand[q]
            fd = []
            for sgn in (1, -1):
                m = dataclasses.replace(ms, **{nm: getattr(ms, nm).copy() for nm in names})
                for nm in names:
                    getattr(m, nm)[k, j, i] *= np.float32(np.exp(sgn * 0.1))
                fd.append(misfit(m))
            g_fd = (fd[0] - fd[1]) / 0.2
            print(f"par {kp + 1} cell {(k, j, i)}: adjoint {grad[kp, k, j, i]:+.4e} "
                  f"fd {g_fd:+.4e} ratio {grad[kp, k, j, i] / g_fd:.3f}")
            adj.append(float(grad[kp, k, j, i]))
            fds.append(g_fd)
    f.close()
    adj, fds = np.array(adj), np.array(fds)
    ratio = adj / fds
    cos = float(adj @ fds / (np.linalg.norm(adj) * np.linalg.norm(fds)))
    print("cosine", cos)
    assert (ratio > 0.5).all() and (ratio < 2.0).all(), ratio
    assert cos >= 0.95, cos


@gpu
def test_fg_forward_matches_reference(golden):
    """Forward modelling through the batched object without observed data
    (gpu.Fg(...).forward, emmi_fg_forward) against the reference's receiver
    data on the layered case; an evaluation on it is refused."""
    from libemmi_mgfd_gb300 import gpu as G
    from test_gpu_solver import receiver_parity
    g = golden("tiny_layered")
    s = W.tiny_layered()
    m = host.Model.from_survey(s)
    f = G.Fg(m, s, options=G.Options(precision=G.PREC_FP64, tol=1e-10, ncycle=120))
    dcal, cyc = f.forward(m)
    with pytest.raises(G.EmmiError, match="without observed data"):
        f.eval(m)
    f.close()
    assert (cyc > 0).all()
    ch = list(s.chrec)
    amp, ph = receiver_parity(dcal[0, :, 0, :], g["dcal"], ch)
    assert amp < 1e-4 and ph < 0.05, (amp, ph)
