"""The device data misfit of the batched inversion evaluation against the
host library's eh_misfit (the reference's fg_fwi.c:208-226 arithmetic,
pinned to the reference's own rmse file and misfit in test_misfit.py):
bit for bit, over shots with ragged receiver counts, several channels and
frequencies, and receivers on both sides of the 5.5-skin-depth cut."""
import numpy as np
import pytest

from libemmi_mgfd_gb300 import host
from libemmi_mgfd_gb300 import workloads as W

gpu = pytest.mark.gpu


def ragged_survey(seed):
    rng = np.random.default_rng(seed)
    nshot, nch, nfreq, nrec = 5, 3, 2, 40
    nrec_shot = np.array([40, 17, 0, 33, 1], np.int32)
    src = np.zeros((nshot, 5), np.float32)
    src[:, 0] = rng.uniform(-3000, 3000, nshot)
    src[:, 1] = rng.uniform(-3000, 3000, nshot)
    src[:, 2] = 950.0
    rec = np.zeros((nshot, nrec, 5), np.float32)
    rec[..., 0] = rng.uniform(-6000, 6000, (nshot, nrec))
    rec[..., 1] = rng.uniform(-2000, 2000, (nshot, nrec))
    rec[..., 2] = 1000.0
    rec[..., 3] = rng.uniform(-np.pi, np.pi, (nshot, nrec))
    shape = (nshot, nch, nfreq, nrec)
    amp = 10.0 ** rng.uniform(-14, -9, shape)
    dcal = (amp * np.exp(1j * rng.uniform(-np.pi, np.pi, shape))).astype(np.complex64)
    dobs = (dcal * (1 + 0.05 * (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)))
            ).astype(np.complex64)
    delta = (0.03 * np.abs(dobs) + 1e-15).astype(np.float32)
    omegas = (2 * np.pi * np.array([0.25, 1.0])).astype(np.float32)
    return src, rec, nrec_shot, dobs, dcal, delta, omegas


@gpu
@pytest.mark.parametrize("seed", [0, 1, 2])
def test_device_misfit_is_the_host_misfit_bitwise(seed):
    from libemmi_mgfd_gb300 import gpu as G
    src, rec, nrs, dobs, dcal, delta, om = ragged_survey(seed)
    rho_w = np.float32(W.RHO_WATER)
    fc, dres, rmse = G.misfit_batch(dobs, dcal, delta, om, rho_w, src, rec, nrs)
    live_total = 0
    for sh in range(len(nrs)):
        nr = int(nrs[sh])
        if nr == 0:
            assert fc[sh] == 0 and not dres[sh].any() and not rmse[sh].any()
            continue
        f0, r0, m0 = host.misfit(dobs[sh, :, :, :nr], dcal[sh, :, :, :nr], delta[sh, :, :, :nr],
                                 om, rho_w, src[sh, :2], rec[sh, :nr, 0], rec[sh, :nr, 1])
        assert np.float32(f0) == fc[sh], (sh, f0, fc[sh])
        assert np.array_equal(dres[sh, :, :, :nr], r0), sh
        assert np.array_equal(rmse[sh, :, :, :nr], m0), sh
        # padded receivers carry nothing
        assert not dres[sh, :, :, nr:].any() and not rmse[sh, :, :, nr:].any()
        live_total += int((m0 > 0).sum())
        assert (m0 == 0).any() or sh != 0  # the near-offset cut is exercised
    assert live_total > 50
