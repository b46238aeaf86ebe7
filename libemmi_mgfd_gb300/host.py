"""ctypes front of libemmi_host.so: the C host front end (regridding and
homogenization) that prepares each shot's mesh and conductivities, and the
data misfit of the gradient mode."""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
HOST_LIB = os.path.join(HERE, "libemmi_host.so")
_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(HOST_LIB):
            raise RuntimeError(f"{HOST_LIB} missing: run libemmi_mgfd_gb300.build.build()")
        _lib = C.CDLL(HOST_LIB)
        _lib.eh_create_nugrid.restype = C.c_float
        _lib.eh_rho_water.restype = C.c_float
        _lib.eh_misfit.restype = C.c_float
        _lib.eh_misfit.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_float, C.c_float,
                                   C.c_float, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                   C.c_void_p, C.c_void_p, C.c_void_p]
        _lib.eh_uncertainty.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_void_p,
                                        C.c_float, C.c_void_p, C.c_float, C.c_float, C.c_float,
                                        C.c_float, C.c_void_p]
    return _lib


CHANNELS = {"Ex": 0, "Ey": 1, "Ez": 2, "Hx": 3, "Hy": 4, "Hz": 5}


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def uncertainty(chrec, dobs, rec_azimuth, src_azimuth, amp_perc=0.03, delta_phi=0.0,
                noisefloorE=1e-15, noisefloorH=1e-13):
    """Standard deviation of every datum (cal_uncertainty_noise.c:17-97,
    without the noise): dobs complex64 [nchrec, nfreq, nrec]."""
    dobs = np.ascontiguousarray(dobs, np.complex64)
    nch, nf, nr = dobs.shape
    ch = np.array([CHANNELS[c] for c in chrec], np.int32)
    az = np.ascontiguousarray(rec_azimuth, np.float32)
    delta = np.zeros(dobs.shape, np.float32)
    lib().eh_uncertainty(nch, _ptr(ch), nf, nr, _ptr(az), C.c_float(src_azimuth), _ptr(dobs),
                         C.c_float(amp_perc), C.c_float(delta_phi), C.c_float(noisefloorE),
                         C.c_float(noisefloorH), _ptr(delta))
    return delta


def misfit(dobs, dcal, delta, omegas, rho_water, src_xy, rec_x, rec_y):
    """fg_fwi.c:208-226: (fcost, dres, rmse) for one shot; arrays
    [nchrec, nfreq, nrec]."""
    dobs = np.ascontiguousarray(dobs, np.complex64)
    dcal = np.ascontiguousarray(dcal, np.complex64)
    delta = np.ascontiguousarray(delta, np.float32)
    nch, nf, nr = dobs.shape
    om = np.ascontiguousarray(omegas, np.float32)
    rx = np.ascontiguousarray(rec_x, np.float32)
    ry = np.ascontiguousarray(rec_y, np.float32)
    dres = np.zeros_like(dobs)
    rmse = np.zeros(dobs.shape, np.float32)
    f = lib().eh_misfit(nch, nf, nr, _ptr(om), C.c_float(rho_water), C.c_float(src_xy[0]),
                        C.c_float(src_xy[1]), _ptr(rx), _ptr(ry), _ptr(dobs), _ptr(dcal),
                        _ptr(delta), _ptr(dres), _ptr(rmse))
    return float(f), dres, rmse


class _Model(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("dx", C.c_float),
                ("dy", C.c_float), ("dz", C.c_float), ("ox", C.c_float), ("oy", C.c_float),
                ("oz", C.c_float), ("rho11", C.c_void_p), ("rho22", C.c_void_p),
                ("rho33", C.c_void_p), ("nb", C.c_int), ("lextend", C.c_float),
                ("rho_air", C.c_float), ("d1min", C.c_float), ("d2min", C.c_float),
                ("d3min", C.c_float), ("n1", C.c_int), ("n2", C.c_int), ("n3", C.c_int)]


GRID_FIELDS = ("x1", "x2", "x3", "x1s", "x2s", "x3s", "d1", "d2", "d3", "d1s", "d2s", "d3s",
               "sigma11", "sigma22", "sigma33", "invmur")


class _Grid(C.Structure):
    _fields_ = [(nm, C.c_void_p) for nm in GRID_FIELDS]


@dataclass
class Model:
    """The regrid inputs of one survey (defaults of src/emf_init_free.c)."""
    nx: int
    ny: int
    nz: int
    dx: float
    dy: float
    dz: float
    ox: float
    oy: float
    oz: float
    rho11: np.ndarray
    rho22: np.ndarray
    rho33: np.ndarray
    n1: int = 128
    n2: int = 128
    n3: int = 128
    nb: int = 10
    lextend: float = 5e4
    rho_air: float = 1e8
    d1min: float = 100.0
    d2min: float = 100.0
    d3min: float = 20.0

    @classmethod
    def from_survey(cls, s) -> "Model":
        ex = dict(s.extra)
        return cls(s.nx, s.ny, s.nz, s.dx, s.dy, s.dz, s.ox, s.oy, s.oz, s.rho11, s.rho22,
                   s.rho33, int(s.n[0]), int(s.n[1]), int(s.n[2]), int(ex.get("nb", 10)),
                   float(ex.get("lextend", 5e4)), float(ex.get("rho_air", 1e8)),
                   float(ex.get("d1min", 100)), float(ex.get("d2min", 100)),
                   float(ex.get("d3min", 20)))

    def _c(self):
        self._keep = [np.ascontiguousarray(a, np.float32) for a in (self.rho11, self.rho22,
                                                                     self.rho33)]
        return _Model(self.nx, self.ny, self.nz, self.dx, self.dy, self.dz, self.ox, self.oy,
                      self.oz, *[a.ctypes.data for a in self._keep], self.nb, self.lextend,
                      self.rho_air, self.d1min, self.d2min, self.d3min, self.n1, self.n2, self.n3)

    def rho_water(self) -> float:
        return float(lib().eh_rho_water(C.byref(self._c())))

    def padded(self):
        """(xx, yy, zz, pad): the padded node axes and the padded model
        [3, nzp, nyp, nxp] (sigma11, sigma22, rho33), once per model
        (regrid_init_free.c:47-141)."""
        m = self._c()
        d = [C.c_int(), C.c_int(), C.c_int()]
        if lib().eh_pad_dims(C.byref(m), *[C.byref(v) for v in d]) != 0:
            raise RuntimeError("eh_pad_dims failed")
        nxp, nyp, nzp = (v.value for v in d)
        xx = np.zeros(nxp + 1, np.float32)
        yy = np.zeros(nyp + 1, np.float32)
        zz = np.zeros(nzp + 1, np.float32)
        pad = np.zeros((3, nzp, nyp, nxp), np.float32)
        if lib().eh_pad_model(C.byref(m), _ptr(xx), _ptr(yy), _ptr(zz), _ptr(pad)) != 0:
            raise RuntimeError("eh_pad_model failed")
        return xx, yy, zz, pad

    def axes(self, xx, yy, zz, sx: float, sy: float, sz: float) -> dict:
        """The mesh axes of a shot at (sx, sy, sz) and their staggered copies
        (regrid_init_free.c:156-214), on the padded axes of padded()."""
        out = {}
        for nm in GRID_FIELDS[:12]:
            n = {"1": self.n1, "2": self.n2, "3": self.n3}[nm[1]]
            out[nm] = np.zeros(n + 1, np.float32)
        g = _Grid(*([out[nm].ctypes.data for nm in GRID_FIELDS[:12]] + [None] * 4))
        rc = lib().eh_regrid_axes(C.byref(self._c()), _ptr(xx), _ptr(yy), _ptr(zz), C.c_float(sx),
                                  C.c_float(sy), C.c_float(sz), C.byref(g))
        if rc != 0:
            raise RuntimeError(f"eh_regrid_axes failed ({rc})")
        return out

    def regrid(self, sx: float, sy: float, sz: float) -> dict:
        """Mesh and homogenized conductivities for a source at (sx, sy, sz)."""
        out = {}
        for nm in GRID_FIELDS[:12]:
            n = {"1": self.n1, "2": self.n2, "3": self.n3}[nm[1]]
            out[nm] = np.zeros(n + 1, np.float32)
        nc = self.n1 * self.n2 * self.n3
        for nm in GRID_FIELDS[12:]:
            out[nm] = np.zeros(nc, np.float32)
        g = _Grid(*[out[nm].ctypes.data for nm in GRID_FIELDS])
        rc = lib().eh_regrid(C.byref(self._c()), C.c_float(sx), C.c_float(sy), C.c_float(sz),
                             C.byref(g))
        if rc != 0:
            raise RuntimeError(f"eh_regrid failed ({rc})")
        return out
