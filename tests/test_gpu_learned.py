"""The learned correction on the GPU: its loss and gradient against the CPU
oracle, training by the library's own kernels, and what the trained network
gains over plain cycles on a model it was not trained on."""
import numpy as np
import pytest

import oracle as O
from learned_oracle import Net, TAPS, CH
from _cases import golden_level, weighted_cells

gpu = pytest.mark.gpu


def _tiny(golden):
    from libemmi_mgfd_gb300 import gpu as G
    g = golden("tiny_layered")
    n, x, raw, om = golden_level(g)
    # sigma_floor far below the air conductivity: the complex64 operator is
    # the true one, which the oracle restates in FP64
    s = G.Solver(n, *[v.astype(np.float32) for v in x], raw[None], np.array([om], np.float32),
                 options=G.Options(precision=G.PREC_MIXED, sigma_floor=1e-30))
    xs = [v.astype(np.float32).astype(np.float64) for v in x]
    c = weighted_cells(n, xs, raw)
    lev = O.Level(n, xs, c[:3], c[3], float(np.float32(om)))
    return s, lev


@gpu
def test_gpu_loss_and_gradient_match_oracle(golden):
    s, lev = _tiny(golden)
    net = Net(lev, bf16_round=True)
    rng = np.random.default_rng(5)
    S3 = 3 * net.S
    samples = [(rng.standard_normal(S3) + 1j * rng.standard_normal(S3)).astype(np.complex64)
               for _ in range(2)]
    s.learned_add_samples(np.stack(samples), [0, 0])
    W = 0.05 * rng.standard_normal((2, TAPS, CH, CH))
    W[0, :, 6:, :] = 0.0
    W = W.astype(np.float32).reshape(-1)
    loss_gpu, g_gpu = s.learned_grad(W)
    loss_cpu, g_cpu = net.loss_grad(W.astype(np.float64), samples)
    assert abs(loss_gpu - loss_cpu) <= 1e-3 * loss_cpu, (loss_gpu, loss_cpu)
    err = np.linalg.norm(g_gpu - g_cpu) / np.linalg.norm(g_cpu)
    assert err < 1e-2, err


@gpu
def test_gpu_correction_matches_oracle(golden):
    """One deployment application (residual, two tensor-core convolutions,
    u += c on unknown edges) on two RHS of one batch against the oracle's
    network: the second RHS's convolution windows start in the first RHS's
    last plane, the first RHS's in the buffer's zero guard."""
    import torch
    from libemmi_mgfd_gb300 import gpu as G
    from learned_oracle import unknown_masks
    g = golden("tiny_layered")
    n, x, raw, om = golden_level(g)
    oms = np.array([om, 0.5 * om], np.float32)
    s = G.Solver(n, *[v.astype(np.float32) for v in x], raw[None], oms, op=np.zeros(2, np.int32),
                 options=G.Options(precision=G.PREC_MIXED, sigma_floor=1e-30))
    xs = [v.astype(np.float32).astype(np.float64) for v in x]
    c = weighted_cells(n, xs, raw)
    rng = np.random.default_rng(7)
    W = (0.05 * rng.standard_normal((2, TAPS, CH, CH))).astype(np.float32).reshape(-1)
    s.set_learned(W)
    unk = unknown_masks(n).reshape(-1)
    S3 = unk.size
    u = np.zeros((2, S3), np.complex64)
    f = np.zeros((2, S3), np.complex64)
    for r in range(2):
        u[r][unk] = rng.standard_normal(unk.sum()) + 1j * rng.standard_normal(unk.sum())
        f[r][unk] = rng.standard_normal(unk.sum()) + 1j * rng.standard_normal(unk.sum())
    du = torch.tensor(u, device="cuda")
    df = torch.tensor(f, device="cuda")
    s.learned_apply(df, du)
    got = du.cpu().numpy().astype(np.complex128) - u.astype(np.complex128)
    for r in range(2):
        lev = O.Level(n, xs, c[:3], c[3], float(oms[r]))
        net = Net(lev, bf16_round=True)
        res = f[r].astype(np.complex128) - lev.apply(u[r].astype(np.complex128))
        want, _ = net.forward(W.astype(np.float64), res)
        err = np.linalg.norm(got[r] - want) / np.linalg.norm(want)
        assert err < 2e-3, (r, err)
        assert np.all(got[r][~unk] == 0)


@gpu
def test_training_on_gpu_reduces_the_loss():
    from libemmi_mgfd_gb300 import learned as LS
    out = LS.train(n=32, models=3, per_rhs=4, steps=120, lr=3e-3, seed=200)
    loss = out["loss"]
    assert out["samples"] == 12
    assert abs(loss[0] - 1.0) < 1e-3          # zero correction at the start
    assert loss[-1] < 0.9 * loss[0], loss[::20]


@gpu
def test_trained_network_gain_on_held_out_models():
    """What the trained network gains over plain cycles: cycles to 1e-8 on
    four random 64^3 models that are not in the training set, one solver,
    with and without the correction."""
    import torch
    from libemmi_mgfd_gb300 import gpu as G
    from libemmi_mgfd_gb300 import learned as LS
    out = LS.train(n=48, models=6, per_rhs=6, steps=300, lr=3e-3, seed=100)
    assert out["loss"][-1] < 0.5            # residual energy after a cycle halved
    p = LS.training_problem(64, 4, 900)
    s = LS.make_solver(p, precision=G.PREC_MIXED, tol=1e-8, ncycle=60)
    b = s.inject_sources(p["src"])
    x = torch.zeros_like(b)
    plain = s.solve(b.data_ptr(), device=True, x_out=x.data_ptr())
    s.set_learned(out["weights"])
    learned = s.solve(b.data_ptr(), device=True, x_out=x.data_ptr())
    c0 = [q["cycles"] for q in plain]
    c1 = [q["cycles"] for q in learned]
    print(f"cycles to 1e-8, plain {c0} ({sum(c0)}), learned {c1} ({sum(c1)})")
    # both reach 1e-8 in the FP64 residual, the learned one in no more cycles
    assert all(q["status"] == "ok" and q["rel"] <= 1e-8 for q in plain + learned)
    assert sum(c1) <= sum(c0)
    assert not any(q["fallback"] for q in learned)


@gpu
def test_convolution_wait_that_runs_out_reports_and_recovers(golden):
    """The tensor-core convolution's bounded waits: with the test hook the
    producer issues no copy and no MMA, so the epilogue waits on an
    accumulator nothing will fill; with a limit of 2e6 clocks (about a
    millisecond) the wait runs out, the kernel frees its tensor memory and
    returns, emmi_learned_apply reports the failure, and on the same GPU
    the next application and a full solve succeed."""
    import ctypes as C
    import torch
    from libemmi_mgfd_gb300 import gpu as G
    g = golden("tiny_layered")
    n, x, raw, om = golden_level(g)
    s = G.Solver(n, *[v.astype(np.float32) for v in x], raw[None], np.array([om], np.float32),
                 options=G.Options(precision=G.PREC_MIXED, ncycle=60, tol=1e-8))
    rng = np.random.default_rng(9)
    W = 0.05 * rng.standard_normal((2, TAPS, CH, CH))
    W[0, :, 6:, :] = 0.0
    s.set_learned(W.astype(np.float32).reshape(-1))
    shape = (1, 3 * s.nslots)
    f = torch.complex(torch.randn(shape, device="cuda"), torch.randn(shape, device="cuda"))
    u = torch.zeros_like(f)
    L = G.lib()
    L.emmi_learned_wait_hook.argtypes = [C.c_void_p, C.c_longlong, C.c_int]
    L.emmi_learned_wait_hook.restype = C.c_int
    assert L.emmi_learned_wait_hook(s._h, 2000000, 1) == 0
    with pytest.raises(RuntimeError, match="gave up waiting"):
        s.learned_apply(f, u)
    assert torch.count_nonzero(u).item() == 0  # nothing written
    assert L.emmi_learned_wait_hook(s._h, 0, 0) == 0
    s.learned_apply(f, u)
    assert torch.isfinite(torch.view_as_real(u)).all() and torch.count_nonzero(u).item() > 0
    xs, hs, st = s.solve(g["b_f0"][None])
    assert st[0]["status"] == "ok", st
    s.close()
