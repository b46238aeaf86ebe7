"""The CPU oracle of the learned correction: its analytic gradient against
central finite differences (float64, no bf16 rounding), the adjoint identity
of its convolution, and bf16 rounding to nearest even."""
import numpy as np
import pytest

import oracle as O
from learned_oracle import Net, TAPS, CH, bf16, conv, conv_transpose, far_mask, taps
from _cases import random_level


def _level(n=(6, 5, 4), seed=3):
    n, x, raw, cells, om, u, f = random_level(n, seed, air=True)
    c = cells.reshape(4, -1)
    return O.Level(n, x, c[:3], c[3], om)


def test_conv_transpose_is_the_adjoint():
    rng = np.random.default_rng(0)
    x = rng.standard_normal((4, 5, 6, CH))
    g = rng.standard_normal((4, 5, 6, CH))
    w = rng.standard_normal((TAPS, CH, CH))
    assert np.isclose(np.sum(conv(x, w) * g), np.sum(x * conv_transpose(g, w)), rtol=1e-12)


@pytest.mark.parametrize("shape", [(5, 6, 7), (3, 4, 17), (6, 3, 3)])
def test_flattened_convolution_equals_zero_padded_off_the_last_planes(shape):
    """The tensor-core kernels convolve on the flattened slot index
    s = i + X j + X Y k, two right-hand sides back to back between zero
    guards: a tap that leaves the grid lands on the last plane of a lower
    direction, on the other RHS's last plane or in a guard.  With inputs zero
    on the last plane of each direction (no unknown edge there; the hidden
    layer is masked to zero there) this equals the zero-padded convolution
    everywhere off those planes, the only slots whose outputs are used."""
    rng = np.random.default_rng(2)
    Z, Y, X = shape
    m = far_mask(shape)[..., None]
    xs = [rng.standard_normal((Z, Y, X, CH)) * m for _ in range(2)]
    w = rng.standard_normal((TAPS, CH, CH))
    S, G = Z * Y * X, X * Y + X + 1
    flat = np.concatenate([np.zeros((G, CH))] + [x.reshape(-1, CH) for x in xs]
                          + [np.zeros((G, CH))])
    keep = m[..., 0].astype(bool)
    for b in range(2):
        out = np.zeros((S, CH))
        for t, (di, dj, dk) in enumerate(taps()):
            o = G + b * S + di + X * dj + X * Y * dk
            out += flat[o:o + S] @ w[t]
        ref = conv(xs[b], w)
        assert np.allclose(out.reshape(Z, Y, X, CH)[keep], ref[keep], rtol=1e-12, atol=1e-12)


def test_bf16_rounds_to_nearest_even():
    v = np.array([1.0, 1.00390625, 1.005859375, 1.0078125 + 2 ** -9, -3.0e-3], np.float32)
    r = bf16(v)
    assert r[0] == 1.0
    assert r[1] == 1.0                      # halfway: to even (1.0)
    assert r[2] == 1.0078125                # above halfway: up
    assert abs(r[4] - (-3.0e-3)) / 3.0e-3 < 2 ** -8


def test_oracle_gradient_matches_finite_differences():
    lev = _level()
    net = Net(lev, bf16_round=False)
    rng = np.random.default_rng(1)
    S3 = 3 * net.S
    samples = [rng.standard_normal(S3) + 1j * rng.standard_normal(S3) for _ in range(2)]
    W = 0.05 * rng.standard_normal((2, TAPS, CH, CH))
    W[0, :, 6:, :] = 0.0
    W[1, :, :, 6:] = 0.0
    W = W.reshape(-1)
    loss, g = net.loss_grad(W, samples)
    assert np.isclose(loss, net.loss(W, samples))
    live = np.flatnonzero(np.abs(g) > 1e-3 * np.abs(g).max())
    idx = rng.choice(live, 12, replace=False)
    h = 1e-5
    for i in idx:
        wp, wm = W.copy(), W.copy()
        wp[i] += h
        wm[i] -= h
        fd = (net.loss(wp, samples) - net.loss(wm, samples)) / (2 * h) * len(samples)
        assert abs(fd - g[i]) <= 1e-5 * max(1.0, abs(g[i])), (i, fd, g[i])
