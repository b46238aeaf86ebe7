"""ctypes front of libemmi_gpu.so: the batched GB300 solver and the
single-level operators.

There is no CPU fallback: if the CUDA library is missing or no GPU is
present, these calls raise.  Arrays follow the reference layout: fields are
complex128 of length 3*(n1+1)*(n2+1)*(n3+1) per right-hand side
(component-major, i fastest); cells are float32 [4][n3][n2][n1]
(sigma11, sigma22, sigma33, invmur).
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass
from typing import Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
GPU_LIB = os.path.join(HERE, "libemmi_gpu.so")

PREC_FP64 = 0
PREC_MIXED = 1
STATUS = {0: "ok", 1: "maxit", 2: "stall", 3: "nonfinite"}

_lib = None


class EmmiError(RuntimeError):
    pass


class _Problem(C.Structure):
    _fields_ = [("n1", C.c_int), ("n2", C.c_int), ("n3", C.c_int), ("nop", C.c_int),
                ("nrhs", C.c_int), ("x1", C.c_void_p), ("x2", C.c_void_p), ("x3", C.c_void_p),
                ("cells", C.c_void_p), ("op", C.c_void_p), ("omega", C.c_void_p),
                ("rho_water", C.c_void_p)]


class _Survey(C.Structure):
    _fields_ = [("nsrc_ch", C.c_int), ("src_ch", C.c_void_p), ("nrec_ch", C.c_int),
                ("rec_ch", C.c_void_p), ("nrec", C.c_int), ("src", C.c_void_p),
                ("rec", C.c_void_p)]


CHANNELS = {"Ex": 0, "Ey": 1, "Ez": 2, "Hx": 3, "Hy": 4, "Hz": 5}


class _Options(C.Structure):
    _fields_ = [("cycleopt", C.c_int), ("ncycle", C.c_int), ("v1", C.c_int), ("v2", C.c_int),
                ("tol", C.c_double), ("isemicoarsen", C.c_int), ("precision", C.c_int),
                ("sigma_floor", C.c_double), ("refine_every", C.c_int),
                ("use_graphs", C.c_int), ("verb", C.c_int), ("krylov", C.c_int),
                ("line_factors", C.c_int), ("autotune", C.c_int), ("line_sweep", C.c_int),
                ("fused_level", C.c_int), ("staged", C.c_int), ("skip_pre", C.c_int),
                ("skip_post", C.c_int)]


class _Stats(C.Structure):
    _fields_ = [("cycles", C.c_int), ("status", C.c_int), ("rnorm0", C.c_double),
                ("rnorm", C.c_double), ("refinements", C.c_int), ("fallback", C.c_int)]


def lib():
    """Load libemmi_gpu.so (built by libemmi_mgfd_gb300.build)."""
    global _lib
    if _lib is None:
        if not os.path.exists(GPU_LIB):
            raise EmmiError(f"{GPU_LIB} is missing: run libemmi_mgfd_gb300.build.build()")
        L = C.CDLL(GPU_LIB)
        L.emmi_last_error.restype = C.c_char_p
        L.emmi_solver_last_time.restype = C.c_double
        L.emmi_solver_last_launches.restype = C.c_long
        L.emmi_solver_device_bytes.restype = C.c_size_t
        L.emmi_solver_create.argtypes = [C.POINTER(C.c_void_p), C.POINTER(_Problem),
                                         C.POINTER(_Options)]
        L.emmi_solver_solve.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                        C.c_void_p]
        L.emmi_solver_last_time.argtypes = [C.c_void_p]
        L.emmi_solver_last_launches.argtypes = [C.c_void_p]
        L.emmi_solver_device_bytes.argtypes = [C.c_void_p]
        L.emmi_solver_destroy.argtypes = [C.c_void_p]
        _lib = L
    return _lib


def _check(rc: int, what: str):
    if rc != 0:
        raise EmmiError(f"{what} failed ({rc}): {lib().emmi_last_error().decode()}")


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


@dataclass
class Options:
    cycleopt: int = 2
    ncycle: int = 30
    v1: int = 1
    v2: int = 1
    tol: float = 1e-6
    isemicoarsen: int = 1
    precision: int = PREC_MIXED
    sigma_floor: float = 0.0
    refine_every: int = 4
    use_graphs: int = 1
    verb: int = 0
    krylov: int = 0
    line_factors: int = 2
    autotune: int = 1
    line_sweep: int = 0
    fused_level: int = 99
    staged: int = 1
    skip_pre: int = 0
    skip_post: int = 0

    def _c(self) -> _Options:
        return _Options(self.cycleopt, self.ncycle, self.v1, self.v2, self.tol, self.isemicoarsen,
                        self.precision, self.sigma_floor, self.refine_every, self.use_graphs,
                        self.verb, self.krylov, self.line_factors, self.autotune,
                        self.line_sweep, self.fused_level, self.staged, self.skip_pre,
                        self.skip_post)


class Solver:
    """A batch of right-hand sides over one or more operators.

    x1,x2,x3: float32 [nop, n+1] node coordinates; cells: float32
    [nop, 4, n3, n2, n1]; omega: float32 [nrhs]; op: int [nrhs] or None."""

    def __init__(self, n: Sequence[int], x1, x2, x3, cells, omega, op=None,
                 options: Optional[Options] = None, rho_water=None):
        """cells: a host array, or a device pointer (int, e.g. from
        homogenize_batch) to float32 [nop, 4, n3, n2, n1]."""
        self.n = tuple(int(v) for v in n)
        self.x1 = np.ascontiguousarray(np.atleast_2d(x1), np.float32)
        self.x2 = np.ascontiguousarray(np.atleast_2d(x2), np.float32)
        self.x3 = np.ascontiguousarray(np.atleast_2d(x3), np.float32)
        dev_cells = isinstance(cells, int)
        if dev_cells:
            cells_ptr = cells
        else:
            self.cells = np.ascontiguousarray(cells, np.float32).reshape(self.x1.shape[0], 4, -1)
            cells_ptr = _p(self.cells).value
        self.omega = np.ascontiguousarray(np.atleast_1d(omega), np.float32)
        self.nop = self.x1.shape[0]
        self.nrhs = self.omega.shape[0]
        self.op = None if op is None else np.ascontiguousarray(op, np.int32)
        self.options = options or Options()
        n1, n2, n3 = self.n
        self.nslots = (n1 + 1) * (n2 + 1) * (n3 + 1)
        self.rho_water = (np.zeros(self.nop, np.float32) if rho_water is None else
                          np.ascontiguousarray(np.broadcast_to(rho_water, (self.nop,)), np.float32))
        prob = _Problem(n1, n2, n3, self.nop, self.nrhs, _p(self.x1).value, _p(self.x2).value,
                        _p(self.x3).value, cells_ptr,
                        None if self.op is None else _p(self.op).value, _p(self.omega).value,
                        _p(self.rho_water).value)
        h = C.c_void_p()
        create = lib().emmi_solver_create_dc if dev_cells else lib().emmi_solver_create
        _check(create(C.byref(h), C.byref(prob), C.byref(self.options._c())),
               "emmi_solver_create")
        self._h = h

    def solve(self, b, want_h: bool = True, device: bool = False, x_out=None, h_out=None):
        """Solve for every RHS.  Host mode: b complex128 [nrhs, 3S] numpy ->
        returns (x, h, stats).  Device mode: b, x_out, h_out are integer
        device pointers (e.g. torch .data_ptr()) -> returns stats."""
        st = (_Stats * self.nrhs)()
        if device:
            _check(lib().emmi_solver_solve(self._h, C.c_void_p(b), C.c_void_p(x_out),
                                           C.c_void_p(h_out) if h_out else None, 1, st),
                   "emmi_solver_solve")
            return self._stats(st)
        b = np.ascontiguousarray(b, np.complex128).reshape(self.nrhs, 3 * self.nslots)
        x = np.zeros_like(b)
        h = np.zeros_like(b) if want_h else None
        _check(lib().emmi_solver_solve(self._h, _p(b), _p(x), _p(h) if want_h else None, 0, st),
               "emmi_solver_solve")
        return x, h, self._stats(st)

    def modelling(self, src, rec, chsrc=("Ex",), chrec=("Ex", "Ey", "Hx", "Hy")):
        """Inject, solve and extract for every RHS (do_modelling as one batch).
        src: [nrhs, 5] x,y,z,azimuth(rad),dip(rad); rec: [nrhs, nrec, 5] or
        [nrec, 5] shared.  Returns (dcal [nrhs, nch, nrec] complex64, stats,
        (h2d_bytes, d2h_bytes))."""
        src = np.ascontiguousarray(np.broadcast_to(src, (self.nrhs, 5)), np.float32)
        rec = np.asarray(rec, np.float32)
        if rec.ndim == 2:
            rec = np.broadcast_to(rec, (self.nrhs,) + rec.shape)
        rec = np.ascontiguousarray(rec, np.float32)
        nrec = rec.shape[1]
        cs = np.array([CHANNELS[c] for c in chsrc], np.int32)
        cr = np.array([CHANNELS[c] for c in chrec], np.int32)
        sv = _Survey(len(cs), _p(cs).value, len(cr), _p(cr).value, nrec, _p(src).value,
                     _p(rec).value)
        out = np.zeros((self.nrhs, len(cr), nrec), np.complex64)
        st = (_Stats * self.nrhs)()
        h2d, d2h = C.c_size_t(), C.c_size_t()
        _check(lib().emmi_modelling_batch(self._h, C.byref(sv), _p(out), st, C.byref(h2d),
                                          C.byref(d2h)), "emmi_modelling_batch")
        return out, self._stats(st), (h2d.value, d2h.value)

    def extract_volume(self, rhs, which, nxyz, o, d, field, rho33=None):
        """E (which=0, from x) or H (which=1, from h) at the input cell centres:
        three complex64 arrays [nz, ny, nx]."""
        nx, ny, nz = (int(v) for v in nxyz)
        out = np.zeros((3, nz, ny, nx), np.complex64)
        o = np.ascontiguousarray(o, np.float32)
        d = np.ascontiguousarray(d, np.float32)
        f = np.ascontiguousarray(field, np.complex128)
        r33 = None if rho33 is None else np.ascontiguousarray(rho33, np.float32)
        _check(lib().emmi_extract_volume(self._h, int(rhs), int(which), nx, ny, nz, _p(o), _p(d),
                                         None if r33 is None else _p(r33), _p(f), _p(out)),
               "emmi_extract_volume")
        return list(out)

    @staticmethod
    def _stats(st):
        return [dict(cycles=s.cycles, status=STATUS.get(s.status, s.status), rnorm0=s.rnorm0,
                     rnorm=s.rnorm, rel=(s.rnorm / s.rnorm0 if s.rnorm0 > 0 else 0.0),
                     refinements=s.refinements, fallback=s.fallback) for s in st]

    @property
    def stream(self) -> int:
        """cudaStream_t of the solver (for torch.cuda.ExternalStream)."""
        lib().emmi_solver_stream.restype = C.c_void_p
        return int(lib().emmi_solver_stream(self._h) or 0)

    def time_smoother(self, direction: int, reps: int = 5):
        """(ms per level-0 line sweep, launches per sweep, algorithmic bytes)."""
        ms, nl, by = C.c_double(), C.c_int(), C.c_double()
        _check(lib().emmi_solver_time_smoother(self._h, int(direction), int(reps), C.byref(ms),
                                               C.byref(nl), C.byref(by)),
               "emmi_solver_time_smoother")
        return ms.value, nl.value, by.value

    # ---- learned correction after each complex64 cycle (MIXED solvers)
    def learned_collect(self, b, per_rhs: int, device: bool = False):
        """Residual samples of plain cycles: solve b ([nrhs, 3S] complex128
        host array, or a device pointer with device=True) and keep the
        level-0 residual after each of the first per_rhs cycles of every RHS.
        Returns the solve statistics."""
        st = (_Stats * self.nrhs)()
        if device:
            ptr = C.c_void_p(b)
        else:
            b = np.ascontiguousarray(b, np.complex128).reshape(self.nrhs, 3 * self.nslots)
            ptr = _p(b)
        _check(lib().emmi_learned_collect(self._h, ptr, 1 if device else 0, int(per_rhs), st),
               "emmi_learned_collect")
        return self._stats(st)

    def inject_sources(self, src, chsrc=("Ex",)):
        """Right-hand sides of unit dipoles src ([nrhs, 5] x, y, z, azimuth,
        dip in radians) as a torch complex128 tensor [nrhs, 3S] on the GPU."""
        import torch
        srcd = torch.tensor(np.ascontiguousarray(src, np.float32).reshape(self.nrhs, 5),
                            device="cuda")
        ch = np.array([CHANNELS[c] for c in chsrc], np.int32)  # host: channel codes
        b = torch.zeros((self.nrhs, 3 * self.nslots), dtype=torch.complex128, device="cuda")
        torch.cuda.synchronize()
        _check(lib().emmi_inject_sources_dev(self._h, C.c_void_p(srcd.data_ptr()), len(chsrc),
                                             _p(ch), C.c_void_p(b.data_ptr())),
               "emmi_inject_sources_dev")
        torch.cuda.synchronize()
        return b

    def learned_add_samples(self, r, rhs):
        """Add residual samples r ([ns, 3S] complex) of the operators of RHS
        rhs[k] to the training set."""
        r = np.ascontiguousarray(r, np.complex64).reshape(-1, 3 * self.nslots)
        idx = np.ascontiguousarray(rhs, np.int32)
        _check(lib().emmi_learned_add_samples(self._h, r.shape[0], _p(r), _p(idx)),
               "emmi_learned_add_samples")

    @property
    def learned_samples(self) -> int:
        return lib().emmi_learned_samples(self._h)

    def learned_train(self, W, steps: int, lr: float = 1e-3):
        """steps full-batch Adam steps on the GPU; returns (W, loss[steps])."""
        W = np.ascontiguousarray(W, np.float32).copy()
        loss = np.zeros(steps, np.float32)
        _check(lib().emmi_learned_train(self._h, int(steps), C.c_float(lr), _p(W), _p(loss)),
               "emmi_learned_train")
        return W, loss

    def learned_grad(self, W):
        """(mean normalised loss, d(sum of normalised losses)/dW) at W."""
        W = np.ascontiguousarray(W, np.float32)
        loss = np.zeros(1, np.float32)
        grad = np.zeros_like(W)
        _check(lib().emmi_learned_grad(self._h, _p(W), _p(loss), _p(grad)), "emmi_learned_grad")
        return float(loss[0]), grad

    def set_learned(self, W):
        """Apply W after every cycle of the following solves (None: off)."""
        if W is None:
            _check(lib().emmi_learned_set(self._h, None), "emmi_learned_set")
            return
        W = np.ascontiguousarray(W, np.float32)
        _check(lib().emmi_learned_set(self._h, _p(W)), "emmi_learned_set")

    def learned_apply(self, f, u):
        """One application of the weights set by set_learned, in place:
        u += N(D^-1 (f - A u)); f, u torch complex64 tensors [nrhs, 3S] on
        the GPU."""
        import torch
        torch.cuda.synchronize()
        _check(lib().emmi_learned_apply(self._h, C.c_void_p(f.data_ptr()),
                                        C.c_void_p(u.data_ptr())), "emmi_learned_apply")
        torch.cuda.synchronize()

    @property
    def last_time(self) -> float:
        return lib().emmi_solver_last_time(self._h)

    @property
    def last_launches(self) -> int:
        return lib().emmi_solver_last_launches(self._h)

    @property
    def device_bytes(self) -> int:
        return lib().emmi_solver_device_bytes(self._h)

    def sweep_shapes(self):
        """([(lines per block, ring depth, rhs threads)] per direction of the
        level-0 sweeps, tuned at this solver's set-up)."""
        sh = ((C.c_int * 3) * 3)()
        tuned = C.c_int()
        _check(lib().emmi_solver_sweep_shapes(self._h, sh, C.byref(tuned)),
               "emmi_solver_sweep_shapes")
        return [tuple(sh[d]) for d in range(3)], bool(tuned.value)

    @property
    def line_factor_format(self) -> int:
        """1: stored factors with L in fp16; 0: fp32; -1: none."""
        return lib().emmi_solver_line_factor_format(self._h)

    @property
    def geometric_weights(self) -> bool:
        """True when the complex64 operator forms its coefficients from the
        mesh spacings (every input invmur exactly 1)."""
        return bool(lib().emmi_solver_geometric_weights(self._h))

    @property
    def staged(self) -> bool:
        """True when the complex64 level-0 residual stages its halos by
        tensor copies."""
        return bool(lib().emmi_solver_staged(self._h))

    def stencil_wait_hook(self, wait_cycles: int = 0, stall_from: int = -1):
        """Test hook of the staged residual's bounded waits (see
        emmi_stencil_wait_hook; reaches the cycles with use_graphs=0)."""
        _check(lib().emmi_stencil_wait_hook(self._h, C.c_longlong(wait_cycles), int(stall_from)),
               "emmi_stencil_wait_hook")

    @property
    def line_format(self) -> int:
        """Multipliers of the one-launch line sweep: 1 fp16, 0 working
        precision, -1 the three-launch sweep."""
        return lib().emmi_solver_line_format(self._h)

    def close(self):
        if getattr(self, "_h", None):
            lib().emmi_solver_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def homogenize_batch(padded, axes, n, cells_ptr: int, stream: int = 0):
    """The device homogenization of a batch of shots: padded = (xx, yy, zz,
    pad) of host.Model.padded(); axes = list of host.Model.axes() dicts;
    writes float32 [nshots, 4, n3, n2, n1] at the device pointer cells_ptr
    (emmi_homogenize_batch)."""
    xx, yy, zz, pad = padded
    nzp, nyp, nxp = pad.shape[1:]
    n1, n2, n3 = (int(v) for v in n)
    x1 = np.ascontiguousarray(np.stack([a["x1"] for a in axes]), np.float32)
    x2 = np.ascontiguousarray(np.stack([a["x2"] for a in axes]), np.float32)
    x3 = np.ascontiguousarray(np.stack([a["x3"] for a in axes]), np.float32)
    pad = np.ascontiguousarray(pad, np.float32)
    _check(lib().emmi_homogenize_batch(int(nxp), int(nyp), int(nzp), _p(xx), _p(yy), _p(zz),
                                       _p(pad), len(axes), n1, n2, n3, _p(x1), _p(x2), _p(x3),
                                       C.c_void_p(cells_ptr), C.c_void_p(stream)),
           "emmi_homogenize_batch")


def _level_args(n, x, cells):
    n3 = (C.c_int * 3)(*[int(v) for v in n])
    xs = [np.ascontiguousarray(v, np.float64) for v in x]
    c = np.ascontiguousarray(cells, np.float64)
    return n3, xs, c


def level_residual(n, x, cells, omega, u, f, prec=PREC_FP64):
    """r = f - A u on one level (cells volume-weighted, float64 [4, ncell])."""
    n3, xs, c = _level_args(n, x, cells)
    u = np.ascontiguousarray(u, np.complex128)
    f = np.ascontiguousarray(f, np.complex128)
    r = np.zeros_like(u)
    nrm = C.c_double()
    _check(lib().emmi_level_residual(n3, _p(xs[0]), _p(xs[1]), _p(xs[2]), _p(c), C.c_double(omega),
                                     prec, _p(u), _p(f), _p(r), C.byref(nrm)), "emmi_level_residual")
    return r, nrm.value


def level_smooth(n, x, cells, omega, u, f, direction, prec=PREC_FP64, iter=0):
    """One multicolour sweep: direction 0..2 lines along x/y/z, 3 node patches."""
    n3, xs, c = _level_args(n, x, cells)
    u = np.ascontiguousarray(u, np.complex128).copy()
    f = np.ascontiguousarray(f, np.complex128)
    _check(lib().emmi_level_smooth(n3, _p(xs[0]), _p(xs[1]), _p(xs[2]), _p(c), C.c_double(omega),
                                   prec, int(direction), int(iter), _p(u), _p(f)),
           "emmi_level_smooth")
    return u


def level_transfer(n, x, sc, inp, out, direction, prec=PREC_FP64):
    """One grid transfer between a level of n cells (node coordinates x) and
    the level coarsened by sc: direction 0 restricts the fine field inp to the
    coarse level (returned), 1 returns out + the prolongation of the coarse
    inp (out: the fine field)."""
    n3 = (C.c_int * 3)(*[int(v) for v in n])
    s3 = (C.c_int * 3)(*[int(v) for v in sc])
    xs = [np.ascontiguousarray(v, np.float64) for v in x]
    inp = np.ascontiguousarray(inp, np.complex128)
    out = np.ascontiguousarray(out, np.complex128).copy()
    _check(lib().emmi_level_transfer(n3, _p(xs[0]), _p(xs[1]), _p(xs[2]), s3, prec,
                                     int(direction), _p(inp), _p(out)), "emmi_level_transfer")
    return out


def build_gradient(nxyz, o, d, idxpar, preco, Ef, Ea, rho11, rho33, bathy, src, rec,
                   dsmute=800.0, drmute=200.0):
    """Gradient w.r.t. ln(rho) summed over shots on the device.
    Ef/Ea: three arrays [nshot, nfreq, nz, ny, nx] complex64 each;
    src [nshot, 3]; rec [nshot, nrec, 3].  Returns (grad, phess)."""
    nx, ny, nz = (int(v) for v in nxyz)
    Ef = [np.ascontiguousarray(a, np.complex64) for a in Ef]
    Ea = [np.ascontiguousarray(a, np.complex64) for a in Ea]
    nshot = Ef[0].shape[0]
    nfreq = Ef[0].size // (nshot * nx * ny * nz)
    idx = np.ascontiguousarray(idxpar, np.int32)
    npar = len(idx)
    grad = np.zeros((npar, nz, ny, nx), np.float32)
    phess = np.zeros((npar, nz, ny, nx), np.float32)
    src = np.ascontiguousarray(np.asarray(src, np.float32)[..., :3].reshape(nshot, 3))
    rec = np.asarray(rec, np.float32)[..., :3]
    nrec = rec.shape[-2] if rec.size else 0
    rec = np.ascontiguousarray(np.broadcast_to(rec, (nshot, nrec, 3)), np.float32)
    o = np.ascontiguousarray(o, np.float32)
    d = np.ascontiguousarray(d, np.float32)
    keep = [np.ascontiguousarray(a, np.float32) for a in (rho11, rho33, bathy)]
    _check(lib().emmi_build_gradient(nx, ny, nz, _p(o), _p(d), nshot, nfreq, npar, _p(idx),
                                     int(preco), *[_p(a) for a in Ef], *[_p(a) for a in Ea],
                                     *[_p(a) for a in keep], _p(src), C.c_float(dsmute), nrec,
                                     _p(rec), C.c_float(drmute), _p(grad), _p(phess)),
           "emmi_build_gradient")
    return grad, phess


def misfit_batch(dobs, dcal, delta, omegas, rho_water, src, rec, nrec_shot):
    """The device data misfit (emmi_misfit_batch): dobs, dcal complex64 and
    delta float32 [nshot, nch, nfreq, nrec]; src [nshot, 5]; rec
    [nshot, nrec, 5]; nrec_shot [nshot] receivers of each shot.  Returns
    (fcost [nshot], dres complex64, rmse float32), dres and rmse shaped like
    dobs."""
    dobs = np.ascontiguousarray(dobs, np.complex64)
    dcal = np.ascontiguousarray(dcal, np.complex64)
    delta = np.ascontiguousarray(delta, np.float32)
    nshot, nch, nfreq, nrec = dobs.shape
    om = np.ascontiguousarray(omegas, np.float32)
    src = np.ascontiguousarray(src, np.float32).reshape(nshot, 5)
    rec = np.ascontiguousarray(rec, np.float32).reshape(nshot, nrec, 5)
    nrs = np.ascontiguousarray(nrec_shot, np.int32)
    dres = np.zeros_like(dobs)
    rmse = np.zeros(dobs.shape, np.float32)
    fcost = np.zeros(nshot, np.float32)
    _check(lib().emmi_misfit_batch(nshot, nch, nfreq, nrec, _p(nrs), _p(om), C.c_float(rho_water),
                                   _p(src), _p(rec), _p(dobs), _p(delta), _p(dcal), _p(dres),
                                   _p(rmse), _p(fcost)), "emmi_misfit_batch")
    return fcost, dres, rmse


class _FgProblem(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("o", C.c_float * 3),
                ("d", C.c_float * 3), ("n1", C.c_int), ("n2", C.c_int), ("n3", C.c_int),
                ("nshot", C.c_int), ("nfreq", C.c_int), ("omega", C.c_void_p),
                ("x1", C.c_void_p), ("x2", C.c_void_p), ("x3", C.c_void_p),
                ("rho_water", C.c_float), ("nsrc_ch", C.c_int), ("src_ch", C.c_void_p),
                ("nrec_ch", C.c_int), ("rec_ch", C.c_void_p), ("nrec", C.c_int),
                ("nrec_shot", C.c_void_p), ("src", C.c_void_p), ("rec", C.c_void_p),
                ("dobs", C.c_void_p), ("delta", C.c_void_p), ("npar", C.c_int),
                ("idxpar", C.c_void_p), ("preco", C.c_int), ("bathy", C.c_void_p),
                ("dsmute", C.c_float), ("drmute", C.c_float)]


class Fg:
    """The inversion's objective evaluation for a batch of shots on the
    device (emmi_fg_create / emmi_fg_eval): forward solves, misfit, adjoint
    solves and the shot-summed gradient in one pass.

    model: host.Model (geometry and start resistivities); survey: its
    Survey (sources, receivers, pairs, channels, frequencies); dobs complex64
    and delta float32 [nshot, nrec_ch, nfreq, nrec]; bathy [ny, nx]."""

    def __init__(self, model, survey, dobs=None, delta=None, bathy=None,
                 options: Optional[Options] = None, idxpar=(1, 2), preco: int = 1,
                 dsmute: float = 800.0, drmute: float = 200.0):
        opts = (options or Options())._c()
        xx, yy, zz, _ = model.padded()
        src = np.asarray(survey.sources, np.float32).copy()
        src[:, 3:] = np.deg2rad(src[:, 3:])
        nshot = len(src)
        recs = [np.asarray(survey.pairs)[np.asarray(survey.pairs)[:, 0] == k + 1, 1] - 1
                for k in range(nshot)]
        nrec = max(1, max(len(r) for r in recs))
        rec = np.zeros((nshot, nrec, 5), np.float32)
        allrec = np.asarray(survey.receivers, np.float32).copy()
        allrec[:, 3:] = np.deg2rad(allrec[:, 3:])
        for k, r in enumerate(recs):
            rec[k, :len(r)] = allrec[r]
        ax = [model.axes(xx, yy, zz, float(p[0]), float(p[1]), float(p[2])) for p in src]
        self.nshot, self.nrec, self.npar, self.preco = nshot, nrec, len(idxpar), preco
        self.nch, self.nfreq = len(survey.chrec), len(survey.freqs)
        self.nxyz = (model.nz, model.ny, model.nx)
        self.forward_only = dobs is None
        shp = (nshot, self.nch, self.nfreq, nrec)
        keep = dict(
            omega=(2 * np.pi * np.asarray(survey.freqs, np.float64)).astype(np.float32),
            x1=np.stack([a["x1"] for a in ax]), x2=np.stack([a["x2"] for a in ax]),
            x3=np.stack([a["x3"] for a in ax]),
            src_ch=np.array([CHANNELS[c] for c in survey.chsrc], np.int32),
            rec_ch=np.array([CHANNELS[c] for c in survey.chrec], np.int32),
            nrec_shot=np.array([len(r) for r in recs], np.int32), src=src, rec=rec,
            dobs=None if dobs is None else np.ascontiguousarray(dobs, np.complex64).reshape(shp),
            delta=None if delta is None else np.ascontiguousarray(delta, np.float32).reshape(shp),
            idxpar=np.array(idxpar, np.int32),
            bathy=None if bathy is None else np.ascontiguousarray(bathy, np.float32))
        if self.forward_only:
            self.npar = 0

        def ptr(a):
            return None if a is None else _p(a)
        P = _FgProblem(model.nx, model.ny, model.nz, (C.c_float * 3)(model.ox, model.oy, model.oz),
                       (C.c_float * 3)(model.dx, model.dy, model.dz), model.n1, model.n2,
                       model.n3, nshot, self.nfreq, _p(keep["omega"]), _p(keep["x1"]),
                       _p(keep["x2"]), _p(keep["x3"]), model.rho_water(), len(keep["src_ch"]),
                       _p(keep["src_ch"]), self.nch, _p(keep["rec_ch"]), nrec,
                       _p(keep["nrec_shot"]), _p(src), _p(rec), ptr(keep["dobs"]),
                       ptr(keep["delta"]), self.npar,
                       None if self.forward_only else _p(keep["idxpar"]), preco,
                       ptr(keep["bathy"]), dsmute, drmute)
        h = C.c_void_p()
        _check(lib().emmi_fg_create(C.byref(h), C.byref(P), C.byref(opts)), "emmi_fg_create")
        self._h = h
        self._keep = keep
        # host -> device bytes of one evaluation: padded model + two grids
        self.h2d_bytes = 0
        self.d2h_bytes = 0

    def eval(self, model):
        """(fcost [nshot], grad, phess [npar, nz, ny, nx], dcal complex64 and
        rmse [nshot, nch, nfreq, nrec], stats [2, nshot * nfreq] (cycles))
        at the resistivities of model (host.Model on the same grid)."""
        xx, yy, zz, pad = model.padded()
        r11 = np.ascontiguousarray(model.rho11, np.float32)
        r33 = np.ascontiguousarray(model.rho33, np.float32)
        nz, ny, nx = self.nxyz
        fcost = np.zeros(self.nshot, np.float32)
        grad = np.zeros((self.npar, nz, ny, nx), np.float32)
        phess = np.zeros_like(grad)
        shp = (self.nshot, self.nch, self.nfreq, self.nrec)
        dcal = np.zeros(shp, np.complex64)
        rmse = np.zeros(shp, np.float32)
        stats = (_Stats * (2 * self.nshot * self.nfreq))()
        _check(lib().emmi_fg_eval(self._h, len(xx) - 1, len(yy) - 1, len(zz) - 1, _p(xx), _p(yy),
                                  _p(zz), _p(pad), _p(r11), _p(r33), _p(fcost), _p(grad),
                                  _p(phess), _p(dcal), _p(rmse), stats), "emmi_fg_eval")
        self.h2d_bytes = sum(a.nbytes for a in (xx, yy, zz, pad, r11, r33))
        self.d2h_bytes = sum(a.nbytes for a in (fcost, grad, dcal, rmse)) + \
            (phess.nbytes if self.preco == 1 else 0)
        cyc = np.array([s.cycles for s in stats]).reshape(2, -1)
        ph = (C.c_double * 8)()
        _check(lib().emmi_fg_phases(self._h, ph), "emmi_fg_phases")
        self.phases_ms = dict(zip(("front_end", "setup", "forward_solves", "data_fields", "misfit",
                                   "adjoint_sources", "adjoint_solves", "gradient_out"),
                                  [round(v, 2) for v in ph]))
        return fcost, grad, phess, dcal, rmse, cyc

    def forward(self, model):
        """(dcal complex64 [nshot, nch, nfreq, nrec], cycles [nshot * nfreq]):
        forward modelling of every shot and frequency in one solver
        (emmi_fg_forward) at the resistivities of model."""
        xx, yy, zz, pad = model.padded()
        dcal = np.zeros((self.nshot, self.nch, self.nfreq, self.nrec), np.complex64)
        stats = (_Stats * (self.nshot * self.nfreq))()
        _check(lib().emmi_fg_forward(self._h, len(xx) - 1, len(yy) - 1, len(zz) - 1, _p(xx),
                                     _p(yy), _p(zz), _p(pad), _p(dcal), stats), "emmi_fg_forward")
        return dcal, np.array([s.cycles for s in stats])

    def close(self):
        if getattr(self, "_h", None):
            lib().emmi_fg_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
