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
