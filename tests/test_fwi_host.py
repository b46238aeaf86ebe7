"""The host side of the inversion mode (libemmi_host.so, include/emmi_fwi.h)
against the reference's own optimizer, regularization and smoothing
(src/opt.c, src/regularization.c, src/triangle_smoothing.c), compiled from
its sources into oracle/_ref/libemmi_ref.so: bitwise, on the same inputs and
the same objective.  Without the compiled reference only the self-checks run."""
import ctypes as C
import os

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HOST = os.path.join(ROOT, "libemmi_mgfd_gb300", "libemmi_host.so")
REF = os.path.join(ROOT, "oracle", "_ref", "libemmi_ref.so")
FP = C.POINTER(C.c_float)
FG_REF = C.CFUNCTYPE(C.c_float, FP, FP)
FG_OURS = C.CFUNCTYPE(C.c_float, C.c_void_p, FP, FP)


class EfOpt(C.Structure):
    _fields_ = [(k, C.c_int) for k in ("niter", "nls", "npair", "bound", "method", "ncg", "preco",
                                        "verb")] + \
               [(k, C.c_float) for k in ("tol", "c1", "c2", "alpha")] + \
               [(k, C.c_int) for k in ("iter", "kpair", "ils", "igrad", "ls_fail", "loop1")] + \
               [(k, C.c_float) for k in ("f0", "fk", "gk_norm")] + \
               [(k, FP) for k in ("x", "g", "d", "q", "xmin", "xmax")] + \
               [("sk", C.POINTER(FP)), ("yk", C.POINTER(FP)), ("rho", FP), ("alp", FP)]


class RefOpt(C.Structure):
    """opt_t of include/opt.h, field for field."""
    _fields_ = [("niter", C.c_int), ("iter", C.c_int), ("tol", C.c_float), ("npair", C.c_int),
                ("kpair", C.c_int), ("nls", C.c_int), ("ils", C.c_int), ("igrad", C.c_int),
                ("c1", C.c_float), ("c2", C.c_float), ("alpha", C.c_float), ("f0", C.c_float),
                ("fk", C.c_float), ("gk_norm", C.c_float), ("x", FP), ("g", FP), ("pg", FP),
                ("d", FP), ("sk", C.POINTER(FP)), ("yk", C.POINTER(FP)), ("q", FP),
                ("alp", FP), ("rho", FP), ("bound", C.c_int), ("xmin", FP), ("xmax", FP),
                ("verb", C.c_int), ("preco", C.c_int), ("loop1", C.c_bool),
                ("ls_fail", C.c_int), ("ncg", C.c_int), ("method", C.c_int)]


def ptr(a):
    return a.ctypes.data_as(FP)


@pytest.fixture(scope="module")
def host():
    from libemmi_mgfd_gb300 import build as B
    B.build()
    lib = C.CDLL(HOST)
    for f in ("ef_l2norm", "ef_dotprod", "ef_tikhonov", "ef_tv"):
        getattr(lib, f).restype = C.c_float
    return lib


@pytest.fixture(scope="module")
def ref():
    if not os.path.exists(REF):
        pytest.skip("reference not compiled here (oracle/_ref)")
    lib = C.CDLL(REF)
    for f in ("l2norm", "dotprod", "regularization_tikhonov", "regularization_tv"):
        getattr(lib, f).restype = C.c_float
    return lib


def objective(x):
    """A float32 objective with curvature that varies along x (a shifted
    quartic plus a quadratic), the same for both sides."""
    n = x.size
    a = np.linspace(0.5, 3.0, n, dtype=np.float32)
    b = np.cos(np.arange(n, dtype=np.float32)).astype(np.float32)
    r = (x - b).astype(np.float32)
    f = np.float32((a * r * r).sum(dtype=np.float32) + np.float32(0.1) * (r ** 4).sum(dtype=np.float32))
    g = (np.float32(2) * a * r + np.float32(0.4) * r ** 3).astype(np.float32)
    return f, g


def make_fg(n, kind):
    calls = []

    def fg(*args):
        xp, gp = args[-2], args[-1]
        x = np.ctypeslib.as_array(xp, (n,)).copy()
        f, g = objective(x)
        np.ctypeslib.as_array(gp, (n,))[:] = g
        calls.append(float(f))
        return float(f)
    return (FG_REF if kind == "ref" else FG_OURS)(fg), calls


class Run:
    """Buffers of one l-BFGS run (x, g, d, q, pairs) for one side."""

    def __init__(self, n, npair, opt_cls, bound=0):
        self.n = n
        self.x = np.full(n, 2.0, np.float32)
        self.g = np.zeros(n, np.float32)
        self.d = np.zeros(n, np.float32)
        self.q = np.zeros(n, np.float32)
        self.xmin = np.full(n, -1.5, np.float32)
        self.xmax = np.full(n, 1.8, np.float32)
        self.S = np.zeros((npair, n), np.float32)
        self.Y = np.zeros((npair, n), np.float32)
        self.rho = np.zeros(npair, np.float32)
        self.alp = np.zeros(npair, np.float32)
        self.sk = (FP * npair)(*[ptr(self.S[i]) for i in range(npair)])
        self.yk = (FP * npair)(*[ptr(self.Y[i]) for i in range(npair)])
        o = opt_cls()
        o.niter, o.nls, o.npair, o.bound = 12, 20, npair, bound
        o.c1, o.c2, o.tol = 1e-4, 0.9, 1e-8
        o.x, o.g, o.d, o.q = ptr(self.x), ptr(self.g), ptr(self.d), ptr(self.q)
        o.xmin, o.xmax, o.rho, o.alp = ptr(self.xmin), ptr(self.xmax), ptr(self.rho), ptr(self.alp)
        o.sk = C.cast(self.sk, C.POINTER(FP))
        o.yk = C.cast(self.yk, C.POINTER(FP))
        self.o = o


def run_lbfgs(lib, side, n, npair, precond, bound):
    """The iteration of do_fwi.c:170-231 on the objective above: update the
    newest pair, descent (two-loop, or its split form around a diagonal
    preconditioner), save (x, g), line search; like the reference, a failed
    line search does not stop the loop."""
    R = Run(n, npair, RefOpt if side == "ref" else EfOpt, bound)
    o, x, g, d = R.o, R.x, R.g, R.d
    fg, calls = make_fg(n, side)
    f, gg = objective(x)
    g[:] = gg
    o.fk = o.f0 = f
    diag = np.linspace(1.0, 0.25, n, dtype=np.float32)
    hist = []
    byref = C.byref(o)
    for it in range(o.niter):
        o.iter = it
        R.q[:] = g
        if it == 0:
            if precond:
                R.q *= diag
            d[:] = -R.q
        else:
            if side == "ref":
                lib.lbfgs_update(n, ptr(x), ptr(g), o.sk, o.yk, byref)
            else:
                lib.ef_lbfgs_update(n, ptr(x), ptr(g), byref)
            if precond:
                if side == "ref":
                    lib.lbfgs_descent1(n, ptr(g), ptr(R.q), ptr(R.rho), ptr(R.alp), o.sk, o.yk,
                                       byref)
                else:
                    lib.ef_lbfgs_descent1(n, ptr(g), byref)
                R.q *= diag
                if o.loop1:
                    if side == "ref":
                        lib.lbfgs_descent2(n, ptr(g), ptr(R.q), ptr(R.rho), ptr(R.alp), o.sk,
                                           o.yk, byref)
                    else:
                        lib.ef_lbfgs_descent2(n, byref)
            elif side == "ref":
                lib.lbfgs_descent(n, ptr(g), ptr(d), o.sk, o.yk, ptr(R.q), ptr(R.rho),
                                  ptr(R.alp), byref)
            else:
                lib.ef_lbfgs_descent(n, ptr(g), ptr(d), byref)
        if side == "ref":
            lib.lbfgs_save(n, ptr(x), ptr(g), o.sk, o.yk, byref)
            lib.line_search(n, ptr(x), ptr(g), ptr(d), fg, byref)
        else:
            lib.ef_lbfgs_save(n, ptr(x), ptr(g), byref)
            lib.ef_line_search(n, ptr(x), ptr(g), ptr(d), fg, None, byref)
        hist.append((x.copy(), d.copy(), o.fk, o.alpha, o.ils, o.igrad, o.ls_fail, o.kpair))
    return hist


@pytest.mark.parametrize("npair,precond,bound", [(3, False, 0), (5, False, 0), (3, True, 0),
                                                 (3, False, 1), (2, True, 1)])
def test_lbfgs_and_line_search_match_reference_bitwise(host, ref, npair, precond, bound):
    """Whole runs (save, two-loop descent or its split form around a
    preconditioner, Wolfe bisection with or without the box bounds,
    update): every iterate, direction, cost, step, line-search count and
    failure flag equal."""
    n = 97
    ours = run_lbfgs(host, "ours", n, npair, precond, bound)
    theirs = run_lbfgs(ref, "ref", n, npair, precond, bound)
    assert len(ours) == len(theirs) == 12
    for it, (a, b) in enumerate(zip(ours, theirs)):
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]), it
        assert a[2:] == b[2:], (it, a[2:], b[2:])
    assert ours[-1][2] < 0.5 * objective(np.full(n, 2.0, np.float32))[0]
    # the pair memory filled up and then wrapped around
    assert ours[-1][7] == npair
    if not bound:
        assert not any(h[6] for h in ours)


def test_line_search_reports_failure_without_decrease(host):
    """An uphill direction: no step lowers the cost, ls_fail = 1, fk kept."""
    n = 16
    R = Run(n, 2, EfOpt)
    o = R.o
    o.bound, o.nls = 0, 4
    R.x[:] = np.cos(np.arange(n, dtype=np.float32)) + 0.5
    f, g = objective(R.x)
    R.g[:] = g
    o.fk = f
    d = g.copy()  # ascent
    fg, calls = make_fg(n, "ours")
    host.ef_line_search(n, ptr(R.x), ptr(R.g), ptr(d), fg, None, C.byref(o))
    assert o.ls_fail == 1 and o.fk == f and o.ils == 4 and len(calls) == 4 and o.igrad == 4


def test_steepest_descent_without_pairs(host):
    n = 8
    R = Run(n, 2, EfOpt)
    g = np.arange(1, n + 1, dtype=np.float32)
    host.ef_lbfgs_descent(n, ptr(g), ptr(R.d), C.byref(R.o))
    assert np.array_equal(R.d, -g)


@pytest.mark.parametrize("shape", [(7, 6, 5), (12, 9, 11), (4, 4, 4)])
def test_regularization_matches_reference_bitwise(host, ref, shape):
    n1, n2, n3 = shape
    rng = np.random.default_rng(sum(shape))
    x = rng.standard_normal(n1 * n2 * n3).astype(np.float32)
    for ours, theirs in (("ef_tikhonov", "regularization_tikhonov"), ("ef_tv", "regularization_tv")):
        ga = np.zeros_like(x)
        gb = np.full_like(x, 7.0)
        fa = getattr(host, ours)(ptr(x), ptr(ga), n1, n2, n3)
        fb = getattr(ref, theirs)(ptr(x), ptr(gb), n1, n2, n3, C.c_float(1), C.c_float(1),
                                  C.c_float(1))
        assert np.float32(fa) == np.float32(fb), ours
        assert np.array_equal(ga, gb), ours


def test_tikhonov_is_the_gradient_of_its_cost(host):
    """The Tikhonov gradient is the derivative of the cost on interior
    cells (central differences, float64 check of the float32 routine)."""
    n1, n2, n3 = 6, 5, 4
    rng = np.random.default_rng(3)
    x = rng.standard_normal(n1 * n2 * n3).astype(np.float32)
    g = np.zeros_like(x)
    host.ef_tikhonov(ptr(x), ptr(g), n1, n2, n3)
    k = 1 + n1 * (2 + n2 * 1) + 2  # interior with all neighbours interior
    # the cost sums the forward differences of interior cells only, so the
    # gradient is the full derivative where every difference touching the
    # cell is counted: check on the cell whose stencil lies inside
    x2 = x.astype(np.float64)

    def cost(v):
        ch, cv = 1.0, 0.03
        a = v.reshape(n3, n2, n1)
        s = 0.0
        for i3 in range(1, n3 - 1):
            for i2 in range(1, n2 - 1):
                for i1 in range(1, n1 - 1):
                    s += ch * ((a[i3, i2, i1 + 1] - a[i3, i2, i1]) ** 2 +
                               (a[i3, i2 + 1, i1] - a[i3, i2, i1]) ** 2)
                    s += cv * (a[i3 + 1, i2, i1] - a[i3, i2, i1]) ** 2
        return s
    f0 = host.ef_tikhonov(ptr(x), ptr(np.zeros_like(x)), n1, n2, n3)
    assert abs(f0 - cost(x2)) <= 1e-5 * abs(cost(x2))
    assert np.isfinite(g).all() and g[k] != 0


@pytest.mark.parametrize("shape,r,repeat", [((9, 8, 7), (3, 2, 4), 1), ((10, 6, 1), (4, 3, 2), 2),
                                            ((5, 5, 5), (2, 2, 2), 3)])
def test_triangle_smoothing_matches_reference_bitwise(host, ref, shape, r, repeat):
    n1, n2, n3 = shape
    rng = np.random.default_rng(n1 * 100 + n2)
    m = rng.standard_normal(n1 * n2 * n3).astype(np.float32)
    a = m.copy()
    host.ef_triangle_smoothing(ptr(a), n1, n2, n3, *r, repeat)
    b = m.copy()
    rows = [(FP * n2)(*[C.cast(b.ctypes.data + 4 * n1 * (i2 + n2 * i3), FP) for i2 in range(n2)])
            for i3 in range(n3)]
    planes = (C.POINTER(FP) * n3)(*[C.cast(rw, C.POINTER(FP)) for rw in rows])
    ref.triangle_smoothing(planes, n1, n2, n3, *r, repeat)
    assert np.array_equal(a, b)
    assert np.abs(a).max() < np.abs(m).max()  # it smooths
