"""The data misfit of the gradient mode (src/fg_fwi.c:208-226) and the data
uncertainties (src/cal_uncertainty_noise.c) restated in the host library,
against the reference's own mode=2 output on the 16^3 layered case: its
rmse file (7 digits) and its printed misfit (6 digits).  The synthetic data
come from the reference's syn file (7 digits), so agreement is to 1e-5."""
import numpy as np

from libemmi_mgfd_gb300 import host
from libemmi_mgfd_gb300 import workloads as W


def parse_data(text, chrec, nfreq, nrec):
    d = np.zeros((len(chrec), nfreq, nrec), np.complex64)
    for line in text.splitlines()[1:]:
        t = line.split()
        if len(t) < 6:
            continue
        d[chrec.index(t[2]), 0, int(t[1]) - 1] = float(t[4]) + 1j * float(t[5])
    return d


def test_misfit_and_uncertainty_match_the_reference(golden):
    g = golden("tiny_grad")
    s = W.tiny_layered()
    ch = list(s.chrec)
    nrec = len(s.receivers)
    dobs = parse_data(str(g["obs_text"]), ch, 1, nrec)
    dcal = np.asarray(g["syn"]).reshape(len(ch), 1, nrec)
    rec = s.receivers.astype(np.float32)
    az = np.float32(np.pi * rec[:, 3] / 180.0)
    delta = host.uncertainty(ch, dobs, az, np.float32(0.0))
    rho_w = np.float32(W.RHO_WATER)
    om = np.array([2 * np.pi * 1.0], np.float32)
    fcost, dres, rmse = host.misfit(dobs, dcal, delta, om, rho_w, s.sources[0, :2], rec[:, 0],
                                    rec[:, 1])
    ref = np.asarray(g["rmse"]).reshape(rmse.shape)
    # receivers within 5.5 skin depths of water are left out in both
    assert np.array_equal(rmse == 0, ref == 0)
    live = ref > 0
    assert live.sum() > 0
    np.testing.assert_allclose(rmse[live], ref[live], rtol=1e-5)
    assert abs(fcost - float(g["fcost"][0])) <= 1e-5 * float(g["fcost"][0])
    # the adjoint source is conj(res / delta): |dres| * delta = rmse
    np.testing.assert_allclose(np.abs(dres[live]) * delta[live], rmse[live], rtol=1e-5)
