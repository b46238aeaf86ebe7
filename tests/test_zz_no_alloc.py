"""The allocation-free line sweep (emmi_level_line_sweep_noalloc) against the
ordinary single-level sweep (emmi_level_smooth): the same kernels, the same
level, so the results agree to the tolerance the level tests use, on two
calls in a row that share the library's static scratch.

This file is named to be collected last: it must pass both alone in a fresh
process and after every other test has used the library on the same GPU."""
import ctypes as C

import numpy as np
import pytest

from _cases import random_level, rel_err, unknown_mask
from libemmi_mgfd_gb300 import gpu as G

gpu = pytest.mark.gpu


def _fn():
    L = G.lib()
    fn = L.emmi_level_line_sweep_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.POINTER(C.c_int), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                   C.c_double, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    return L, fn


def _device_level(cells, u, f, prec):
    """The caller's own device buffers (allocated by torch, not by the call)."""
    import torch
    real = torch.float64 if prec == G.PREC_FP64 else torch.float32
    cplx = torch.complex128 if prec == G.PREC_FP64 else torch.complex64
    dc = torch.tensor(np.ascontiguousarray(cells), dtype=real, device="cuda")
    du = torch.tensor(np.ascontiguousarray(u), dtype=cplx, device="cuda")
    df = torch.tensor(np.ascontiguousarray(f), dtype=cplx, device="cuda")
    return dc, du, df


def _call(fn, n, x, dc, omega, du, df, direction, prec, it, stream=None):
    xs = [np.ascontiguousarray(v, np.float64) for v in x]
    n3 = (C.c_int * 3)(*n)
    return fn(n3, *[v.ctypes.data for v in xs], dc.data_ptr(), C.c_double(omega), prec,
              int(direction), int(it), du.data_ptr(), df.data_ptr(), stream)


def _noalloc_sweep(n, x, cells, omega, u, f, direction, prec, it):
    """One line sweep through the C ABI on device buffers the caller owns;
    the device's free memory must not change across the call."""
    import torch
    L, fn = _fn()
    dc, du, df = _device_level(cells, u, f, prec)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    rc = _call(fn, n, x, dc, omega, du, df, direction, prec, it)
    assert rc == 0, L.emmi_last_error().decode()
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    return du.cpu().numpy().astype(np.complex128), free1 - free0


@gpu
@pytest.mark.parametrize("prec, tol", [(G.PREC_FP64, 1e-12), (G.PREC_MIXED, 1e-4)])
def test_noalloc_sweep_matches_level_smooth(prec, tol):
    # two calls in a row: a larger level, then a smaller one along another
    # direction, so the second call runs over the first call's leftovers
    for n, seed, direction, it in [((24, 16, 20), 5, 0, 0), ((12, 18, 10), 6, 2, 1)]:
        n, x, raw, cells, omega, u, f = random_level(n, seed, air=True)
        want = G.level_smooth(n, x, cells, omega, u, f, direction, prec=prec, iter=it)
        got, dfree = _noalloc_sweep(n, x, cells, omega, u, f, direction, prec, it)
        m = unknown_mask(n).reshape(-1)
        err = rel_err(got[m], want[m])
        assert err < tol, (n, direction, err)
    # the first call on the device reserved the static array (lazy module
    # loading); the second call took no device memory at all
    assert dfree == 0, dfree


@gpu
@pytest.mark.parametrize("prec, tol", [(G.PREC_FP64, 1e-12), (G.PREC_MIXED, 1e-4)])
def test_noalloc_sweeps_ordered_on_a_caller_stream(prec, tol):
    """Two sweeps (x, then z) queued on the caller's own non-default stream
    with no synchronization between them, against the same two sweeps of
    emmi_level_smooth one after the other."""
    import torch
    n, x, raw, cells, omega, u, f = random_level((20, 14, 16), 11, air=True)
    want = G.level_smooth(n, x, cells, omega, u, f, 0, prec=prec, iter=0)
    want = G.level_smooth(n, x, cells, omega, want, f, 2, prec=prec, iter=1)
    L, fn = _fn()
    dc, du, df = _device_level(cells, u, f, prec)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        for direction, it in [(0, 0), (2, 1)]:
            rc = _call(fn, n, x, dc, omega, du, df, direction, prec, it, stream=s.cuda_stream)
            assert rc == 0, L.emmi_last_error().decode()
    s.synchronize()
    got = du.cpu().numpy().astype(np.complex128)
    m = unknown_mask(n).reshape(-1)
    err = rel_err(got[m], want[m])
    assert err < tol, err


@gpu
def test_noalloc_rejects_levels_beyond_the_scratch():
    import torch
    L, fn = _fn()
    n = (256, 256, 256)  # an x sweep here needs ~1.2 GB of records
    x = [np.arange(v + 1, dtype=np.float64) for v in n]
    n3 = (C.c_int * 3)(*n)
    dummy = torch.zeros(16, dtype=torch.float64, device="cuda")  # never touched
    rc = fn(n3, *[v.ctypes.data for v in x], dummy.data_ptr(), C.c_double(1.0), G.PREC_FP64, 0,
            0, dummy.data_ptr(), dummy.data_ptr(), None)
    assert rc == -1
    assert "the maximum is" in L.emmi_last_error().decode()
