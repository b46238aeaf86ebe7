"""CPU oracle of the learned correction and of its training gradient.

TEST INFRASTRUCTURE ONLY: the tests use this module to check the GPU kernels
of csrc/emmi_learned.cu; the library never imports it.

The learned correction has no counterpart in the reference.  Its operator A
is the reference's curl-curl operator (src/gmg.c:1316-1410), taken here from
the C restatement (oracle.Level.apply); everything else is restated from the
network's definition:

  z      = D^-1 r on unknown edges (D the diagonal of A), 8 channels per slot
           (Ex, Ey, Ez real/imaginary, 2 zero channels), bf16-rounded
  h      = conv(z, W1) rounded to bf16      (3x3x3, zero padding), set to
           zero on the last slot plane of each direction (i = n1, j = n2,
           k = n3: no component has an unknown edge there)
  c      = conv(h, W2), channels 0..5 -> complex components, unknown edges
  loss_b = |r_b - A c_b|^2 / |r_b|^2

Weights are [2][27][8][8] (layer, tap, cin, cout), tap = (dk+1)*9 +
(dj+1)*3 + (di+1).  With bf16=True the forward pass rounds z, h and the
weights to bfloat16 (round to nearest even) like the tensor-core kernels,
and the gradient is taken at the rounded weights; with bf16=False the whole
computation is float64 (for finite-difference checks).
"""
from __future__ import annotations

import numpy as np

TAPS, CH = 27, 8


def bf16(a):
    """Round float32 values to bfloat16 (nearest even), returned as float64."""
    x = np.ascontiguousarray(a, np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def taps():
    return [(t % 3 - 1, (t // 3) % 3 - 1, t // 9 - 1) for t in range(TAPS)]


def unknown_masks(n):
    """[3][Z][Y][X] booleans: interior tangential edges per component."""
    n1, n2, n3 = n
    k, j, i = np.meshgrid(np.arange(n3 + 1), np.arange(n2 + 1), np.arange(n1 + 1), indexing="ij")
    P = [i, j, k]
    out = []
    for c in range(3):
        p, q = (c + 1) % 3, (c + 2) % 3
        out.append((P[c] < n[c]) & (P[p] >= 1) & (P[p] < n[p]) & (P[q] >= 1) & (P[q] < n[q]))
    return np.stack(out)


def far_mask(shape):
    """[Z, Y, X] 1.0 off the last plane of each direction, 0.0 on it."""
    m = np.ones(shape)
    m[-1, :, :] = 0.0
    m[:, -1, :] = 0.0
    m[:, :, -1] = 0.0
    return m


def diagonal(level):
    """Diagonal of A on every slot ([3S] complex), by probing the oracle's
    operator with unit vectors spaced 3 slots apart (stencils reach 1)."""
    n1, n2, n3 = level.n
    X, Y, Z = n1 + 1, n2 + 1, n3 + 1
    S = X * Y * Z
    k, j, i = np.meshgrid(np.arange(Z), np.arange(Y), np.arange(X), indexing="ij")
    d = np.zeros(3 * S, np.complex128)
    for c in range(3):
        for a in range(3):
            for b in range(3):
                for e in range(3):
                    sel = ((i % 3 == a) & (j % 3 == b) & (k % 3 == e)).ravel()
                    u = np.zeros(3 * S, np.complex128)
                    u[c * S:(c + 1) * S][sel] = 1.0
                    Au = level.apply(u)
                    d[c * S:(c + 1) * S][sel] = Au[c * S:(c + 1) * S][sel]
    return d


def conv(x, w):
    """x [Z, Y, X, 8], w [27, 8, 8] -> [Z, Y, X, 8], zero padding."""
    Z, Y, X, _ = x.shape
    p = np.pad(x, ((1, 1), (1, 1), (1, 1), (0, 0)))
    out = np.zeros((Z, Y, X, CH))
    for t, (di, dj, dk) in enumerate(taps()):
        out += p[1 + dk:1 + dk + Z, 1 + dj:1 + dj + Y, 1 + di:1 + di + X, :] @ w[t]
    return out


def conv_transpose(g, w):
    """Adjoint of conv in its input: g [Z, Y, X, 8] -> [Z, Y, X, 8]."""
    Z, Y, X, _ = g.shape
    p = np.pad(g, ((1, 1), (1, 1), (1, 1), (0, 0)))
    out = np.zeros((Z, Y, X, CH))
    for t, (di, dj, dk) in enumerate(taps()):
        out += p[1 - dk:1 - dk + Z, 1 - dj:1 - dj + Y, 1 - di:1 - di + X, :] @ w[t].T
    return out


def weight_grad(g, x):
    """dW[t][cin][cout] = sum_s g[s][cout] x[s + off(t)][cin]."""
    Z, Y, X, _ = x.shape
    p = np.pad(x, ((1, 1), (1, 1), (1, 1), (0, 0)))
    dw = np.zeros((TAPS, CH, CH))
    G = g.reshape(-1, CH)
    for t, (di, dj, dk) in enumerate(taps()):
        sh = p[1 + dk:1 + dk + Z, 1 + dj:1 + dj + Y, 1 + di:1 + di + X, :].reshape(-1, CH)
        dw[t] = sh.T @ G
    return dw


class Net:
    """Loss and gradient of the learned correction over residual samples of
    one operator (an oracle.Level)."""

    def __init__(self, level, bf16_round: bool = True):
        self.level = level
        self.n = level.n
        n1, n2, n3 = level.n
        self.shape = (n3 + 1, n2 + 1, n1 + 1)
        self.S = int(np.prod(self.shape))
        self.mask = unknown_masks(level.n)
        self.diag = diagonal(level).reshape(3, *self.shape)
        self.far = far_mask(self.shape)[..., None]
        self.rb = bf16_round

    def _round(self, a):
        return bf16(a) if self.rb else np.asarray(a, np.float64)

    def channels(self, r):
        r = np.asarray(r).reshape(3, *self.shape)
        z = np.where(self.mask, r / np.where(self.mask, self.diag, 1.0), 0.0)
        x = np.zeros((*self.shape, CH))
        for c in range(3):
            x[..., 2 * c] = z[c].real
            x[..., 2 * c + 1] = z[c].imag
        return self._round(x)

    def forward(self, W, r):
        w = self._round(np.asarray(W, np.float64).reshape(2, TAPS, CH, CH))
        x = self.channels(r)
        h = self._round(conv(x, w[0])) * self.far
        o = conv(h, w[1])
        c = np.zeros((3, *self.shape), np.complex128)
        for k in range(3):
            c[k] = np.where(self.mask[k], o[..., 2 * k] + 1j * o[..., 2 * k + 1], 0.0)
        return c.reshape(-1), (w, x, h)

    def loss_grad(self, W, samples):
        """(mean normalised loss, d(sum of normalised losses)/dW [2*27*8*8])."""
        total, grad = 0.0, np.zeros((2, TAPS, CH, CH))
        for r in samples:
            r = np.asarray(r, np.complex128).reshape(-1)
            rn2 = float(np.vdot(r, r).real)
            c, (w, x, h) = self.forward(W, r)
            e = r - self.level.apply(c)
            total += float(np.vdot(e, e).real) / rn2
            m = self.mask.reshape(-1)
            q = self.level.apply(np.where(np.concatenate([m]), np.conj(e), 0.0))
            # dL/dRe c = -2 Re q, dL/dIm c = 2 Im q (A symmetric), unknown edges only
            q = q.reshape(3, *self.shape)
            gc = np.zeros((*self.shape, CH))
            for k in range(3):
                gc[..., 2 * k] = np.where(self.mask[k], -2.0 * q[k].real / rn2, 0.0)
                gc[..., 2 * k + 1] = np.where(self.mask[k], 2.0 * q[k].imag / rn2, 0.0)
            grad[1] += weight_grad(gc, h)
            gh = conv_transpose(gc, w[1]) * self.far
            grad[0] += weight_grad(gh, x)
        return total / len(samples), grad.reshape(-1)

    def loss(self, W, samples):
        tot = 0.0
        for r in samples:
            r = np.asarray(r, np.complex128).reshape(-1)
            c, _ = self.forward(W, r)
            e = r - self.level.apply(c)
            tot += float(np.vdot(e, e).real) / float(np.vdot(r, r).real)
        return tot / len(samples)
