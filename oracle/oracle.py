"""ctypes front of the CPU oracle (oracle/liboracle.so) -- TEST INFRASTRUCTURE.

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module, and only as the checker.  Field arrays are
numpy complex128 of length 3*(n1+1)*(n2+1)*(n3+1) in the reference layout
(component-major, i fastest); cell arrays are [n3, n2, n1].
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from typing import Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

ORDER_LEX = 0
ORDER_COLOR = 1
CHANNELS = {"Ex": 0, "Ey": 1, "Ez": 2, "Hx": 3, "Hy": 4, "Hz": 5}

_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle with make (gcc only)."""
    if force or not os.path.exists(LIB_PATH) or (
            os.path.getmtime(LIB_PATH) < os.path.getmtime(os.path.join(HERE, "emmi_oracle.c"))):
        subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)
    return LIB_PATH


class _Params(C.Structure):
    _fields_ = [("cycleopt", C.c_int), ("ncycle", C.c_int), ("v1", C.c_int), ("v2", C.c_int),
                ("tol", C.c_double), ("isemicoarsen", C.c_int), ("ordering", C.c_int),
                ("verb", C.c_int)]


class _Level(C.Structure):
    _fields_ = [("n", C.c_int * 3), ("x", C.c_void_p * 3), ("sig", C.c_void_p * 3),
                ("imu", C.c_void_p), ("omega", C.c_double)]


class _Grid(C.Structure):
    _fields_ = [("n1", C.c_int), ("n2", C.c_int), ("n3", C.c_int)] + [
        (nm, C.c_void_p) for nm in ("x1", "x2", "x3", "x1s", "x2s", "x3s", "d1", "d2", "d3",
                                    "sigma33")] + [("rho_water", C.c_float)]


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(LIB_PATH)
        _lib.eo_gmg_solve.restype = C.c_int
        _lib.eo_gmg_solve_timed.restype = C.c_int
        _lib.eo_find_index.restype = C.c_int
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def _c128(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.complex128)


def gmg_solve(n, x1, x2, x3, sigma11, sigma22, sigma33, invmur, omega, b,
              cycleopt=2, ncycle=30, v1=1, v2=1, tol=1e-6, isemicoarsen=1,
              ordering=ORDER_LEX, verb=0, timing=False):
    """Reference-algorithm solve (gmg_apply).  Returns (E, H, ncycles, rnorms),
    and with timing=True also (set-up seconds, seconds of the cycles)."""
    prm = _Params(cycleopt, ncycle, v1, v2, tol, isemicoarsen, ordering, verb)
    bb = _c128(b).copy()
    x = np.zeros_like(bb)
    hist = np.full(ncycle + 1, np.nan)
    sec = np.zeros(2)
    keep = [_f32(x1), _f32(x2), _f32(x3), _f32(sigma11), _f32(sigma22), _f32(sigma33),
            _f32(invmur)]
    nc = lib().eo_gmg_solve_timed(int(n[0]), int(n[1]), int(n[2]), *[_p(k) for k in keep],
                                  C.c_double(float(np.float32(omega))), C.byref(prm), _p(bb),
                                  _p(x), _p(hist), _p(sec))
    if timing:
        return x, bb, nc, hist[: nc + 1], (float(sec[0]), float(sec[1]))
    return x, bb, nc, hist[: nc + 1]


class Level:
    """A single multigrid level: double node coordinates and volume-weighted
    cell arrays, for the single-operator parity checks."""

    def __init__(self, n, x, sig, imu, omega):
        self.n = tuple(int(v) for v in n)
        self.x = [_f64(v) for v in x]
        self.sig = [_f64(v) for v in sig]
        self.imu = _f64(imu)
        self.omega = float(omega)
        self._d = _Level((C.c_int * 3)(*self.n), (C.c_void_p * 3)(*[v.ctypes.data for v in self.x]),
                         (C.c_void_p * 3)(*[v.ctypes.data for v in self.sig]),
                         self.imu.ctypes.data, self.omega)

    @property
    def nslots(self):
        n1, n2, n3 = self.n
        return (n1 + 1) * (n2 + 1) * (n3 + 1)

    def residual(self, u, f):
        u, f = _c128(u), _c128(f)
        r = np.zeros_like(u)
        lib().eo_residual(C.byref(self._d), _p(u), _p(f), _p(r))
        return r

    def apply(self, u):
        u = _c128(u)
        out = np.zeros_like(u)
        lib().eo_apply(C.byref(self._d), _p(u), _p(out))
        return out

    def line_sweep(self, u, f, direction, ordering=ORDER_COLOR, iter=0):
        u = _c128(u).copy()
        f = _c128(f)
        lib().eo_line_sweep(C.byref(self._d), int(direction), int(ordering), int(iter), _p(u), _p(f))
        return u

    def point_sweep(self, u, f, ordering=ORDER_COLOR, iter=0):
        u = _c128(u).copy()
        f = _c128(f)
        lib().eo_point_sweep(C.byref(self._d), int(ordering), int(iter), _p(u), _p(f))
        return u

    def curl_h(self, u):
        u = _c128(u)
        h = np.zeros_like(u)
        lib().eo_curl_h(C.byref(self._d), _p(u), _p(h))
        return h


def _n3(n):
    return (C.c_int * 3)(*[int(v) for v in n])


def restrict(nf, xf, nc, xc, sc, rf):
    xf = [_f64(v) for v in xf]
    xc = [_f64(v) for v in xc]
    rf = _c128(rf)
    out = np.zeros(3 * (nc[0] + 1) * (nc[1] + 1) * (nc[2] + 1), np.complex128)
    lib().eo_restrict(_n3(nf), (C.c_void_p * 3)(*[v.ctypes.data for v in xf]), _n3(nc),
                      (C.c_void_p * 3)(*[v.ctypes.data for v in xc]), _n3(sc), _p(rf), _p(out))
    return out


def prolong(nf, xf, nc, xc, sc, uc, uf):
    xf = [_f64(v) for v in xf]
    xc = [_f64(v) for v in xc]
    uc = _c128(uc)
    out = _c128(uf).copy()
    lib().eo_prolong(_n3(nf), (C.c_void_p * 3)(*[v.ctypes.data for v in xf]), _n3(nc),
                     (C.c_void_p * 3)(*[v.ctypes.data for v in xc]), _n3(sc), _p(uc), _p(out))
    return out


def coarsen_cells(nf, sc, cf):
    cf = _f64(cf)
    out = np.zeros((nf[2] // sc[2]) * (nf[1] // sc[1]) * (nf[0] // sc[0]), np.float64)
    lib().eo_coarsen_cells(_n3(nf), _n3(sc), _p(cf), _p(out))
    return out


def stagger(x):
    """x -> (xs, d, ds) as the reference's generate_xs_dx (gmg.c:1672)."""
    x = np.asarray(x, np.float64)
    n = len(x) - 1
    ds = np.empty(n + 1)
    xs = np.empty(n + 1)
    ds[:n] = x[1:] - x[:-1]
    xs[:n] = 0.5 * (x[:-1] + x[1:])
    xs[n] = x[n] + 0.5 * ds[n - 1]
    ds[n] = xs[n] - x[n]
    d = np.empty(n + 1)
    d[1:] = xs[1:] - xs[:-1]
    d[0] = xs[0] - x[0]
    return xs, d, ds


class Grid:
    """emf_t grid after regrid_init (float arrays) for injection/extraction."""

    def __init__(self, n, x1, x2, x3, x1s, x2s, x3s, d1, d2, d3, sigma33, rho_water):
        self.n = tuple(int(v) for v in n)
        self.arrs = [_f32(v) for v in (x1, x2, x3, x1s, x2s, x3s, d1, d2, d3, sigma33)]
        self._g = _Grid(*self.n, *[a.ctypes.data for a in self.arrs], C.c_float(rho_water))

    @property
    def nfield(self):
        n1, n2, n3 = self.n
        return 3 * (n1 + 1) * (n2 + 1) * (n3 + 1)


def find_index(x, val):
    x = _f32(x)
    return lib().eo_find_index(len(x), _p(x), C.c_float(val))


def _pts(p):
    p = _f32(p)
    return [_f32(p[:, i]) for i in range(5)]


def inject_source(g: Grid, src, chsrc: Sequence[str], omega):
    cols = _pts(np.atleast_2d(src))
    ch = np.array([CHANNELS[c] for c in chsrc], np.int32)
    b = np.zeros(g.nfield, np.complex128)
    lib().eo_inject_source(C.byref(g._g), len(cols[0]), *[_p(c) for c in cols], len(ch), _p(ch),
                           C.c_float(omega), _p(b))
    return b


def inject_adj_source(g: Grid, rec, chrec, dres, omega):
    cols = _pts(rec)
    ch = np.array([CHANNELS[c] for c in chrec], np.int32)
    dres = np.ascontiguousarray(dres, np.complex64)
    x = np.zeros(g.nfield, np.complex128)
    b = np.zeros(g.nfield, np.complex128)
    lib().eo_inject_adj_source(C.byref(g._g), len(cols[0]), *[_p(c) for c in cols], len(ch),
                               _p(ch), _p(dres), C.c_float(omega), _p(x), _p(b))
    return x, b


def extract_emf_data(g: Grid, rec, chrec, x, h):
    cols = _pts(rec)
    ch = np.array([CHANNELS[c] for c in chrec], np.int32)
    out = np.zeros((len(ch), len(cols[0])), np.complex64)
    x, h = _c128(x), _c128(h)
    lib().eo_extract_emf_data(C.byref(g._g), len(cols[0]), *[_p(c) for c in cols], len(ch),
                              _p(ch), _p(x), _p(h), _p(out))
    return out


def extract_electric_field(g: Grid, nxyz, o, d, rho33, x):
    nx, ny, nz = nxyz
    out = [np.zeros((nz, ny, nx), np.complex64) for _ in range(3)]
    rho33 = _f32(rho33)
    x = _c128(x)
    lib().eo_extract_electric_field(C.byref(g._g), nx, ny, nz, *[C.c_float(v) for v in o],
                                    *[C.c_float(v) for v in d], _p(rho33), _p(x),
                                    *[_p(a) for a in out])
    return out


def extract_magnetic_field(g: Grid, nxyz, o, d, h):
    nx, ny, nz = nxyz
    out = [np.zeros((nz, ny, nx), np.complex64) for _ in range(3)]
    h = _c128(h)
    lib().eo_extract_magnetic_field(C.byref(g._g), nx, ny, nz, *[C.c_float(v) for v in o],
                                    *[C.c_float(v) for v in d], _p(h), *[_p(a) for a in out])
    return out


def build_gradient(nxyz, o, d, idxpar, preco, Ef, Ea, rho11, rho33, bathy, src, rec,
                   dsmute=800.0, drmute=200.0):
    nx, ny, nz = nxyz
    Ef = [np.ascontiguousarray(a, np.complex64) for a in Ef]
    Ea = [np.ascontiguousarray(a, np.complex64) for a in Ea]
    nfreq = Ef[0].size // (nx * ny * nz)
    npar = len(idxpar)
    idx = np.array(idxpar, np.int32)
    grad = np.zeros((npar, nz, ny, nx), np.float32)
    phess = np.zeros((npar, nz, ny, nx), np.float32)
    s, r = _pts(np.atleast_2d(src)), _pts(rec)
    keep = [_f32(rho11), _f32(rho33), _f32(bathy)]
    lib().eo_build_gradient(nx, ny, nz, *[C.c_float(v) for v in o], *[C.c_float(v) for v in d],
                            nfreq, npar, _p(idx), int(preco), *[_p(a) for a in Ef],
                            *[_p(a) for a in Ea], *[_p(k) for k in keep], len(s[0]), _p(s[0]),
                            _p(s[1]), _p(s[2]), C.c_float(dsmute), len(r[0]), _p(r[0]),
                            _p(r[1]), _p(r[2]), C.c_float(drmute), _p(grad), _p(phess))
    return grad, phess
