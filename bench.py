#!/usr/bin/env python3
"""Benchmark of the GB300 hot path: solves/s to 1e-8 relative residual at
128^3, mixed-precision GMG against plain FP64 GMG.

Workload (one step): the mixed-precision 128^3 configuration -- 25 shots on
a 5x5 grid at 1 km over a log-normal sediment under 1000 m of water with two
resistive bodies, 1 Hz, 100 seafloor receivers, Ex source, Ex/Ey/Hx/Hy
channels -- as one batch: inject the 25 sources, solve all 25 systems to
|b - A x| <= 1e-8 |b| (FP64 residual), extract the receiver data.

  value  solves/s with the operators and right-hand sides resident in HBM
  e2e    the same through the C ABI from the model on the host, as the
         reference's modelling runs a shot (regrid, solve, extract): the
         padded model and every shot's mesh axes on the host, H2D of the
         padded model, the 25 shots' homogenization on the device, solver
         setup, inject, solve, extract, D2H of the receiver data
  plain_fp64   the same batch with complex128 cycles (the reference's
         arithmetic), for the mixed-vs-plain ratio
  roofline     the level-0 line-relaxation sweep (dominant kernel), timed
         live with CUDA events on the solver's stream
  cpu_baseline the CPU restatement of the reference's algorithm on the host
         cores, one F-cycle per thread as a bounded sample, scaled by the
         cycles a solve takes
  fwi_eval     one objective evaluation of the inversion (the reference's
         fg_fwi) on the gradient configuration -- 25 shots x 3 frequencies
         (0.25, 0.5, 1 Hz) at 128^3, the gradient of the half-space start
         model against the reservoir model's data -- through the C ABI
         (emmi_fg_eval) from host arrays: 75 forward and 75 adjoint solves,
         misfit, adjoint sources and the shot-summed gradient

  python bench.py [--steps K] [--warmup W] [--impl reference]
Under torchrun each rank solves its own copy of the batch (weak scaling).
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "solves/s to 1e-8 rel. residual at 128³ on 1 GB300: learned+mixed vs plain GMG"
UNIT = "solves/s"
# The cycle of the measured configurations: the reference's F(1,1) (V(1,1)
# for config5) without the post-smoothing of levels 0 and 1
# (emmi_options.skip_post = 3), the fastest mask measured on these batches;
# the learned correction after each cycle takes the level-0 post-smoothing's
# place.  The reference's own cycle is timed beside it (reference_cycle).
SKIP_POST = 3
CYCLE = "F(1,1) without the post-smoothing of levels 0 and 1 (skip_post=3)"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--n", type=int, default=128)
    p.add_argument("--tol", type=float, default=1e-8)
    p.add_argument("--no-fp64", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-config5", action="store_true",
                   help="skip the 256x256x128 learned-vs-plain configuration (config5)")
    p.add_argument("--no-parity", action="store_true",
                   help="skip the receiver parity report (FP64 solve of the batch to 1e-12)")
    p.add_argument("--no-fwi", action="store_true",
                   help="skip the inversion objective evaluation (fwi_eval)")
    p.add_argument("--only-fwi", action="store_true",
                   help="run only the inversion objective evaluation and print it")
    p.add_argument("--nrhs", type=int, default=0, help="use only the first k shots")
    p.add_argument("--no-learned", action="store_true",
                   help="plain complex64 cycles (no learned correction)")
    p.add_argument("--krylov", type=int, default=0, help="FGMRES restart length (0: refinement)")
    p.add_argument("--no-staged", action="store_true",
                   help="the plain complex64 residual instead of the tensor-copy staged one")
    p.add_argument("--profile", action="store_true",
                   help="one shot: a short solve, then one level-0 line sweep inside the NVTX "
                        "range emmi_profile (for ncu --nvtx-include emmi_profile/)")
    p.add_argument("--profile-dir", type=int, default=0, choices=(0, 1, 2),
                   help="with --profile: the line direction of the sweep (0 x, 1 y, 2 z)")
    p.add_argument("--profile-residual", action="store_true",
                   help="with --profile: one complex64 residual r = f - A u of a seeded 128^3 "
                        "level (unit spacing, random conductivity), one RHS")
    p.add_argument("--profile-learned", action="store_true",
                   help="with --profile: one application of the learned correction (seeded "
                        "weights, seeded level-0 iterates) instead of the line sweep")
    return p.parse_args()


def dist():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as D
        D.init_process_group("gloo")
        pg = D
    return rank, world, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def max_over_ranks(pg, v):
    if pg is None:
        return v
    import torch
    t = torch.tensor([float(v)])
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------- workload
def build_workload(n: int):
    """25 shots of the 128^3 configuration through the C host front end."""
    from libemmi_mgfd_gb300 import host
    from libemmi_mgfd_gb300 import workloads as W
    s = W.config3(n)
    m = host.Model.from_survey(s)
    src = s.sources.astype(np.float32)
    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        grids = list(ex.map(lambda p: m.regrid(float(p[0]), float(p[1]), float(p[2])), src))
    X1 = np.stack([g["x1"] for g in grids])
    X2 = np.stack([g["x2"] for g in grids])
    X3 = np.stack([g["x3"] for g in grids])
    cells = np.stack([np.stack([g["sigma11"], g["sigma22"], g["sigma33"], g["invmur"]])
                      for g in grids])
    om = np.float32(2.0 * np.pi * s.freqs[0])
    srcr = src.copy()
    srcr[:, 3:] = np.deg2rad(srcr[:, 3:])
    rec = s.receivers.astype(np.float32).copy()
    rec[:, 3:] = np.deg2rad(rec[:, 3:])
    return dict(survey=s, X1=X1, X2=X2, X3=X3, cells=cells, omega=np.full(len(src), om, np.float32),
                rho_water=np.float32(m.rho_water()), src=srcr, rec=rec, grids=grids, model=m,
                src_xyz=src[:, :3].copy())


def fwi_eval_bench(n: int, tol: float):
    """Seconds per inversion objective evaluation (fg_fwi) of the gradient
    configuration, host arrays in and out through emmi_fg_eval.  The
    observed data are the reservoir model's own synthetic data (one
    evaluation with zero data), uncertainties 3% of the amplitude plus a
    floor; the timed evaluation is the second one at the start model."""
    from libemmi_mgfd_gb300 import gpu as G
    from libemmi_mgfd_gb300 import host
    from libemmi_mgfd_gb300 import workloads as W
    true = W.config4(n, true_model=True)
    start = W.config4(n, true_model=False)
    mt, ms = host.Model.from_survey(true), host.Model.from_survey(start)
    nshot, nch, nf = len(true.sources), len(true.chrec), len(true.freqs)
    nrec = int(np.bincount(np.asarray(true.pairs)[:, 0]).max())
    opts = G.Options(precision=G.PREC_MIXED, tol=tol, ncycle=100, skip_post=SKIP_POST)
    shape = (nshot, nch, nf, nrec)
    f = G.Fg(mt, true, np.zeros(shape, np.complex64), np.ones(shape, np.float32), true.bathy,
             options=opts)
    dobs = f.eval(mt)[3]
    f.close()
    delta = (0.03 * np.abs(dobs) + 1e-15).astype(np.float32)
    f = G.Fg(ms, start, dobs, delta, start.bathy, options=opts)
    f.eval(ms)
    t0 = time.perf_counter()
    fcost, grad, phess, dcal, rmse, cyc = f.eval(ms)
    dt = time.perf_counter() - t0
    out = {"seconds_per_evaluation": round(dt, 3), "shots": nshot, "freqs": nf,
           "solves": 2 * nshot * nf, "solves_per_s": round(2 * nshot * nf / dt, 2),
           "cycles_mean_forward": float(cyc[0].mean()), "cycles_mean_adjoint": float(cyc[1].mean()),
           "fcost": float(fcost.astype(np.float64).sum()),
           "grad_finite": bool(np.isfinite(grad).all() and np.abs(grad).max() > 0),
           "h2d_bytes": int(f.h2d_bytes), "d2h_bytes": int(f.d2h_bytes),
           "phases_ms": f.phases_ms,
           "workload": f"c4_reservoir_{n}^3_25shots_3freqs, gradient at the half-space start "
                       "model, mixed precision to tol", "tol": tol}
    f.close()
    return out


def config5_bench(a):
    """The learned-smoother configuration: 50 shots of the log-normal model
    family on a 256 x 256 x 128 mesh (about 25 M edge unknowns each), V(1,1)
    cycles to 1e-8, with and without the learned correction.  The network is
    trained on the GPU by the library's kernels on residuals of plain cycles
    on random survey models (water over log-normal sediment with a resistive
    body, through the host front end) at 96^3; the cells of the 50 shots are
    homogenized on the device.  Each variant: one untimed batch, one timed
    (CUDA events on the solver's stream)."""
    import torch
    from libemmi_mgfd_gb300 import gpu as G
    from libemmi_mgfd_gb300 import host
    from libemmi_mgfd_gb300 import learned as LS
    from libemmi_mgfd_gb300 import workloads as W
    s = W.config5()
    m = host.Model.from_survey(s)
    src = s.sources.astype(np.float32).copy()
    padded = m.padded()
    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        axes = list(ex.map(lambda p: m.axes(*padded[:3], float(p[0]), float(p[1]), float(p[2])),
                           src))
    nsh = len(src)
    dcells = torch.empty((nsh, 4, int(np.prod(s.n))), dtype=torch.float32, device="cuda")
    G.homogenize_batch(padded, axes, s.n, dcells.data_ptr())
    X = [np.stack([ax[k] for ax in axes]) for k in ("x1", "x2", "x3")]
    om = np.full(nsh, np.float32(2 * np.pi * s.freqs[0]), np.float32)
    srcr = src.copy()
    srcr[:, 3:] = np.deg2rad(srcr[:, 3:])
    rec = s.receivers.astype(np.float32).copy()
    rec[:, 3:] = np.deg2rad(rec[:, 3:])
    tr = LS.train(n=96, models=16, per_rhs=4, steps=300, lr=3e-3, seed=500, skip_post=SKIP_POST)
    out = {"workload": "c5_lognormal_256x256x128_50shots_1Hz",
           "cycle": "V(1,1) without the post-smoothing of levels 0 and 1 (skip_post=3)",
           "tol": a.tol, "rhs": nsh,
           "training": {"models": 16, "mesh": "96^3", "samples": int(tr["samples"]),
                        "collect_seconds": round(tr["collect_seconds"], 2),
                        "train_seconds": round(tr["train_seconds"], 2),
                        "loss_end": round(float(tr["loss"][-1]), 4)}}
    for name, wts in (("plain", None), ("learned", tr["weights"])):
        sv = G.Solver(s.n, *X, dcells.data_ptr(), om, op=np.arange(nsh, dtype=np.int32),
                      options=G.Options(precision=G.PREC_MIXED, tol=a.tol, ncycle=100,
                                        cycleopt=1, skip_post=SKIP_POST),
                      rho_water=np.float32(m.rho_water()))
        if wts is not None:
            sv.set_learned(wts)
        sv.modelling(srcr, rec, s.chsrc, s.chrec)
        ext = torch.cuda.ExternalStream(sv.stream)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        _, st, _ = sv.modelling(srcr, rec, s.chsrc, s.chrec)
        e1.record(ext)
        e1.synchronize()
        t = e0.elapsed_time(e1) / 1e3
        out[name] = {"seconds": round(t, 3), "solves_per_s": round(nsh / t, 3),
                     "cycles_mean": float(np.mean([q["cycles"] for q in st])),
                     "cycles_max": int(max(q["cycles"] for q in st)),
                     "all_converged": all(q["status"] == "ok" for q in st),
                     "max_rel_residual": float(max(q["rel"] for q in st)),
                     "fallback_rate": float(np.mean([q["fallback"] for q in st]))}
        sv.close()
    del dcells
    torch.cuda.empty_cache()
    return out


def parity_report(w, d, a):
    """Receiver errors of d (the benchmark's solve: [nrhs, nch, nrec]) against
    an FP64 solve of the same batch to 1e-12 and against the reference's
    receiver data where a fixture holds them."""
    from libemmi_mgfd_gb300 import gpu as G
    from libemmi_mgfd_gb300.parity import receiver_errors
    s = w["survey"]
    ch = list(s.chrec)
    sp = make_solver(w, G.PREC_FP64, 1e-12, ncycle=200, skip_post=0)
    d64, st64, _ = sp.modelling(w["src"], w["rec"], s.chsrc, s.chrec)
    sp.close()
    per = [receiver_errors(d[r], d64[r], ch) for r in range(d.shape[0])]
    out = {"bar": "amplitude <= 1e-4 of the channel scale, phase <= 0.05 deg",
           "vs_fp64": {"tol": 1e-12,
                       "all_converged": all(q["status"] == "ok" for q in st64),
                       "cycles_mean": float(np.mean([q["cycles"] for q in st64])),
                       "amplitude_max": max(p[0] for p in per),
                       "phase_deg_max": max(p[1] for p in per),
                       "per_shot": [[float(f"{p[0]:.3e}"), float(f"{p[1]:.3e}")] for p in per]}}
    path = os.path.join(ROOT, "tests", "golden", "c3_lognormal_128_ref.npz")
    if a.n == 128 and d.shape[0] == 25 and os.path.exists(path):
        g = np.load(path)
        ref = {"reference_tol": 1e-10, "shots": [], "amplitude": [], "phase_deg": [],
               "fp64_amplitude": [], "fp64_phase_deg": []}
        for k in g["shots"]:
            k = int(k)
            am, ph = receiver_errors(d[k - 1], g[f"s{k}_dcal"], ch)
            a64, p64 = receiver_errors(d64[k - 1], g[f"s{k}_dcal"], ch)
            ref["shots"].append(k)
            ref["amplitude"].append(float(f"{am:.3e}"))
            ref["phase_deg"].append(float(f"{ph:.3e}"))
            ref["fp64_amplitude"].append(float(f"{a64:.3e}"))
            ref["fp64_phase_deg"].append(float(f"{p64:.3e}"))
        out["vs_reference"] = ref
    return out


def make_solver(w, precision, tol, krylov=0, ncycle=100, line_factors=2, skip_post=SKIP_POST,
                staged=1):
    from libemmi_mgfd_gb300 import gpu as G
    n = w["survey"].n
    nrhs = w["X1"].shape[0]
    return G.Solver(n, w["X1"], w["X2"], w["X3"], w["cells"], w["omega"],
                    op=np.arange(nrhs, dtype=np.int32),
                    options=G.Options(precision=precision, tol=tol, ncycle=ncycle, krylov=krylov,
                                      line_factors=line_factors, skip_post=skip_post,
                                      staged=staged),
                    rho_water=w["rho_water"])


# ---------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.idx = gpu_index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([v.strip() for v in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for nm, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(self.rows)}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def ncu_traffic():
    """DRAM bytes of one level-0 x sweep (12 launches, 25 RHS) from the
    committed ncu summary (captured at 4 RHS, scaled by 25/4)."""
    path = os.path.join(ROOT, "profiles", "line_sweep_x_c3_128.txt")
    try:
        for line in open(path):
            if line.startswith("dram_bytes_per_sweep_scaled="):
                return float(line.split("=")[1])
    except Exception:
        pass
    return None


# ---------------------------------------------------------------- CPU leg
def reference_cycles(n: int, tol: float):
    """F-cycles the reference itself needs to reach tol on this workload:
    the residual histories it printed solving shots 1 and 13 of the 128^3
    configuration (tests/golden/c3_lognormal_128_ref.npz, made by running
    the reference compiled from its sources); None for other sizes."""
    path = os.path.join(ROOT, "tests", "golden", "c3_lognormal_128_ref.npz")
    if n != 128 or not os.path.exists(path):
        return None
    g = np.load(path)
    counts = []
    for k in g["shots"]:
        h = g[f"s{k}_rnorm_f0"]
        below = np.nonzero(h / h[0] < tol)[0]
        if len(below) == 0:
            return None
        counts.append(int(below[0]))
    return float(np.mean(counts)), [int(k) for k in g["shots"]], counts


def cpu_sample(w, nthreads, cycles_per_solve, cycles_note):
    """Oracle (the reference's algorithm, lexicographic sweeps) on host
    threads, one shot per thread, each one F-cycle of its own solve with the
    set-up before it timed apart.  A solve is the set-up plus
    `cycles_per_solve` cycles; the batch of `nthreads` concurrent solves
    takes as long as its slowest thread.  Returns (solves/s, seconds,
    sample text)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build()
    s = w["survey"]
    n = s.n
    nshots = w["X1"].shape[0]
    # right-hand sides by the oracle's restatement of inject_source
    grids = w["grids"]
    bs = []
    for i in range(nthreads):
        g = grids[i % nshots]
        G = O.Grid(n, g["x1"], g["x2"], g["x3"], g["x1s"], g["x2s"], g["x3s"], g["d1"], g["d2"],
                   g["d3"], g["sigma33"], float(w["rho_water"]))
        bs.append(O.inject_source(G, w["src"][i % nshots], s.chsrc, float(w["omega"][0])))

    def one(i):
        g = grids[i % nshots]
        r = O.gmg_solve(n, g["x1"], g["x2"], g["x3"], g["sigma11"], g["sigma22"], g["sigma33"],
                        g["invmur"], float(w["omega"][0]), bs[i], ncycle=1, tol=0.0,
                        ordering=O.ORDER_LEX, timing=True)
        return r[4]

    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(max_workers=nthreads) as ex:
        tm = list(ex.map(one, range(nthreads)))
    dt = time.perf_counter() - t0
    per_solve = max(su + cycles_per_solve * cy for su, cy in tm)
    value = nthreads / per_solve
    su = max(t[0] for t in tm)
    cy = max(t[1] for t in tm)
    sample = (f"{nthreads} concurrent shots of the {n[0]}^3 system, one F-cycle each: set-up "
              f"{su:.2f} s and {cy:.2f} s per F-cycle (slowest thread); a solve = set-up + "
              f"{cycles_per_solve:.1f} F-cycles ({cycles_note})")
    return value, dt, sample


# ---------------------------------------------------------------- main
def main():
    a = parse()
    rank, world, local, pg = dist()
    if a.impl == "reference":
        return reference_arm(a, rank, world, pg)
    import torch
    from libemmi_mgfd_gb300 import build as B
    from libemmi_mgfd_gb300 import gpu as G
    B.build()
    torch.cuda.set_device(local)
    if a.only_fwi:
        if rank == 0:
            print(json.dumps({"fwi_eval": fwi_eval_bench(a.n, a.tol)}), flush=True)
        return
    w = build_workload(a.n)
    s = w["survey"]
    if a.nrhs > 0 or a.profile:
        k = a.nrhs if a.nrhs > 0 else 1
        for key in ("X1", "X2", "X3", "cells", "omega", "src"):
            w[key] = np.ascontiguousarray(w[key][:k])
        w["grids"] = w["grids"][:k]
    nrhs = w["X1"].shape[0]
    if a.profile:
        sp = make_solver(w, G.PREC_MIXED, a.tol)
        sp.modelling(w["src"], w["rec"], s.chsrc, s.chrec)
        if a.profile_residual:
            rng = np.random.default_rng(12)
            n3 = (a.n, a.n, a.n)
            xs = [np.arange(v + 1, dtype=np.float64) for v in n3]
            cells = np.concatenate([10.0 ** rng.uniform(-2, 0, (3, a.n ** 3)),
                                    np.ones((1, a.n ** 3))])
            S3 = 3 * (a.n + 1) ** 3
            u = rng.standard_normal(S3) + 1j * rng.standard_normal(S3)
            f = rng.standard_normal(S3) + 1j * rng.standard_normal(S3)
            G.level_residual(n3, xs, cells, 6.28, u, f, prec=G.PREC_MIXED)  # warm-up
            torch.cuda.nvtx.range_push("emmi_profile")
            G.level_residual(n3, xs, cells, 6.28, u, f, prec=G.PREC_MIXED)
            torch.cuda.nvtx.range_pop()
        elif a.profile_learned:
            rng = np.random.default_rng(11)
            sp.set_learned((0.05 * rng.standard_normal(2 * 27 * 64)).astype(np.float32))
            shape = (nrhs, 3 * sp.nslots)
            f = torch.complex(torch.randn(shape, device="cuda"), torch.randn(shape, device="cuda"))
            u = torch.zeros_like(f)
            sp.learned_apply(f, u)  # warm-up outside the range
            torch.cuda.nvtx.range_push("emmi_profile")
            sp.learned_apply(f, u)
            torch.cuda.nvtx.range_pop()
        else:
            torch.cuda.nvtx.range_push("emmi_profile")
            sp.time_smoother(a.profile_dir, reps=1)
            torch.cuda.nvtx.range_pop()
        sp.close()
        print(json.dumps({"profile": "done", "n": a.n, "nrhs": nrhs}))
        return

    # learned correction: trained here on the GPU (untimed) on random models
    learned, W = None, None
    if not a.no_learned:
        from libemmi_mgfd_gb300 import learned as LS
        tr = LS.train(n=48, models=6, per_rhs=6, steps=300, lr=3e-3, seed=100,
                      skip_post=SKIP_POST)
        W = tr["weights"]
        learned = {"trained_on": "6 random 48^3 survey models (host front end), residuals after "
                                 "each of the first 6 plain complex64 cycles (same cycle)",
                   "samples": int(tr["samples"]), "collect_seconds": round(tr["collect_seconds"], 2),
                   "train_seconds": round(tr["train_seconds"], 2), "adam_steps": 300,
                   "loss_start": round(float(tr["loss"][0]), 4),
                   "loss_end": round(float(tr["loss"][-1]), 4)}

    solver = make_solver(w, G.PREC_MIXED, a.tol, krylov=a.krylov, staged=0 if a.no_staged else 1)
    shapes, _ = solver.sweep_shapes()
    if W is not None:
        solver.set_learned(W)
    ext = torch.cuda.ExternalStream(solver.stream)
    launches = []
    stats = None

    def step():
        d, st, _ = solver.modelling(w["src"], w["rec"], s.chsrc, s.chrec)
        launches.append(solver.last_launches + 2)  # + injection + extraction
        return d, st

    for _ in range(a.warmup):
        step()
    barrier(pg)
    torch.cuda.synchronize()
    times = []
    launches.clear()
    with ClockSampler(local) as clk:
        for _ in range(a.steps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(ext)
            d, stats = step()
            e1.record(ext)
            e1.synchronize()
            times.append(e0.elapsed_time(e1) / 1e3)
    torch.cuda.synchronize()
    barrier(pg)
    total = max_over_ranks(pg, sum(times))
    value = nrhs * a.steps * world / total
    timed_launches = int(sum(launches))
    cycles = [x["cycles"] for x in stats]
    rels = [x["rel"] for x in stats]
    refs = [x["refinements"] for x in stats]
    ok = all(x["status"] == "ok" for x in stats)
    without = None
    if W is not None:
        learned["fallback_rate"] = float(np.mean([x["fallback"] for x in stats]))
        # the same solver without the correction, for comparison (one step)
        solver.set_learned(None)
        step()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        _, st0 = step()
        e1.record(ext)
        e1.synchronize()
        t0 = e0.elapsed_time(e1) / 1e3
        without = {"value": round(nrhs * world / max_over_ranks(pg, t0), 3), "unit": UNIT,
                   "cycles_mean": float(np.mean([x["cycles"] for x in st0])),
                   "all_converged": all(x["status"] == "ok" for x in st0)}
    # the reference's own cycle (every level post-smooths), no learned
    # correction: one untimed and one timed batch
    refcyc = None
    if not a.no_fp64:
        sr = make_solver(w, G.PREC_MIXED, a.tol, krylov=a.krylov, skip_post=0)
        extr = torch.cuda.ExternalStream(sr.stream)
        sr.modelling(w["src"], w["rec"], s.chsrc, s.chrec)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(extr)
        _, str_, _ = sr.modelling(w["src"], w["rec"], s.chsrc, s.chrec)
        e1.record(extr)
        e1.synchronize()
        tr_ = max_over_ranks(pg, e0.elapsed_time(e1) / 1e3)
        refcyc = {"value": round(nrhs * world / tr_, 3), "unit": UNIT, "cycle": "F(1,1)",
                  "learned": False,
                  "cycles_mean": float(np.mean([x["cycles"] for x in str_])),
                  "all_converged": all(x["status"] == "ok" for x in str_)}
        sr.close()

    # roofline of the dominant kernel (level-0 line relaxation)
    ms, nl, by = solver.time_smoother(0, reps=5)
    ms_dir = [round(ms, 4)] + [round(solver.time_smoother(d, reps=3)[0], 4) for d in (1, 2)]
    peak, peak_kind = peaks()
    achieved = by / (ms * 1e-3) / 1e9
    traffic = ncu_traffic()
    roof = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "traffic": traffic,
            # the DRAM bytes the sweep really moves (ncu, scaled to 25 RHS) per
            # second: what the kernels achieve against the memory system
            "traffic_GBps": round(traffic / (ms * 1e-3) / 1e9, 1) if traffic else None,
            "traffic_frac": round(traffic / (ms * 1e-3) / 1e9 / peak, 4) if traffic else None,
            "kernel": "level-0 line sweep along x, 4 colours x (k_line_rhs, k_line_subst, "
                      "k_line_apply_rb)<float> with stored line factors, 25 RHS",
            "ms_per_sweep": round(ms, 4), "ms_per_sweep_xyz": ms_dir, "launches_per_sweep": nl,
            "algorithmic_bytes_per_launch": by / nl, "peak_kind": peak_kind}
    solver.close()

    # parity of the timed step's receiver data: against an FP64 solve of the
    # same batch to 1e-12 (every shot) and against the reference's own data
    # for the shots it was run on (tests/golden/c3_lognormal_128_ref.npz)
    parity = None
    if not a.no_parity:
        parity = parity_report(w, d, a)

    # e2e: from host arrays through the C ABI, solver setup included
    e2e_times, h2d, d2h = [], 0, 0
    m = w["model"]
    nsh = w["X1"].shape[0]
    nc = int(np.prod(s.n))
    dcells = torch.empty((nsh, 4, nc), dtype=torch.float32, device="cuda")
    for it in range(0 if a.no_e2e else 2):
        torch.cuda.synchronize()
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record()
        # the front end: padded model and mesh axes on the host (1D work),
        # the homogenization of every shot on the device
        padded = m.padded()
        axes = [m.axes(*padded[:3], float(p[0]), float(p[1]), float(p[2])) for p in w["src_xyz"]]
        G.homogenize_batch(padded, axes, s.n, dcells.data_ptr())
        X = [np.stack([ax[k] for ax in axes]) for k in ("x1", "x2", "x3")]
        sv = G.Solver(s.n, *X, dcells.data_ptr(), w["omega"], op=np.arange(nsh, dtype=np.int32),
                      options=G.Options(precision=G.PREC_MIXED, tol=a.tol, ncycle=100,
                                        krylov=a.krylov, skip_post=SKIP_POST),
                      rho_water=w["rho_water"])
        if W is not None:
            sv.set_learned(W)  # the weights trained above, as a caller would reuse them
        _, _, (hb, db) = sv.modelling(w["src"], w["rec"], s.chsrc, s.chrec)
        sv.close()
        t1.record()
        t1.synchronize()
        if it > 0:
            e2e_times.append(t0.elapsed_time(t1) / 1e3)
        h2d = (padded[3].nbytes + sum(v.nbytes for v in padded[:3]) + sum(x.nbytes for x in X)
               + w["omega"].nbytes + hb)
        d2h = db
    e2e = None
    if e2e_times:
        e2e_t = max_over_ranks(pg, statistics.mean(e2e_times))
        e2e = {"value": round(nrhs * world / e2e_t, 3), "unit": UNIT,
               "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
               "seconds_per_step": round(e2e_t, 4)}

    # plain FP64 GMG on the same batch
    # plain FP64 GMG (the reference's arithmetic) with its best line sweep
    # (FP64 line factors stored at set-up), and with every line refactored in
    # every sweep
    plain, plain_rec = None, None
    if not a.no_fp64:
        def fp64_arm(line_factors):
            sp = make_solver(w, G.PREC_FP64, a.tol, line_factors=line_factors)
            ext64 = torch.cuda.ExternalStream(sp.stream)
            sp.modelling(w["src"], w["rec"], s.chsrc, s.chrec)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(ext64)
            _, st64, _ = sp.modelling(w["src"], w["rec"], s.chsrc, s.chrec)
            e1.record(ext64)
            e1.synchronize()
            t64 = max_over_ranks(pg, e0.elapsed_time(e1) / 1e3)
            ms64, _, by64 = sp.time_smoother(0, reps=2)
            out = {"value": round(nrhs * world / t64, 3), "unit": UNIT,
                   "cycles_mean": float(np.mean([x["cycles"] for x in st64])),
                   "all_converged": all(x["status"] == "ok" for x in st64),
                   "smoother_GBps": round(by64 / (ms64 * 1e-3) / 1e9, 1),
                   "line_factors": "stored FP64" if sp.line_factor_format == 0
                                   else "refactored every sweep", "cycle": CYCLE}
            sp.close()
            return out
        plain = fp64_arm(1)
        plain_rec = fp64_arm(0)

    cpu = None
    if rank == 0 and world == 1 and not a.no_cpu:
        cps, note = ref_cycle_count(a, plain, cycles)
        nthr = os.cpu_count() or 1
        v, dt, sample = cpu_sample(w, nthr, cps, note)
        cpu = {"value": round(v, 5), "unit": UNIT, "cores": nthr, "kind": "port",
               "sample": sample}

    fwi = None
    if rank == 0 and world == 1 and not a.no_fwi:  # a one-GPU figure, like cpu_baseline
        fwi = fwi_eval_bench(a.n, a.tol)

    c5 = None
    if rank == 0 and world == 1 and not a.no_config5:
        c5 = config5_bench(a)

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world,
            "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": round(1e3 * total / a.steps, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c64 cycles + f64 refinement",
            "data": "synthetic (seeded log-normal model, no public dataset)",
            "config": {"workload": f"c3_lognormal_{a.n}^3_25shots_1Hz", "n": a.n,
                       "rhs_per_step": nrhs, "tol": a.tol, "precision": "mixed",
                       "smoother": "zebra line relaxation (4 colours), rotating semi-coarsening"
                                   + ("" if a.no_learned else
                                      " + learned 3x3x3 conv correction after each cycle"
                                      " (in the level-0 post-smoothing's place)"),
                       "outer": f"FGMRES({a.krylov})" if a.krylov else "FP64 refinement",
                       "cycle": CYCLE, "parallelism": f"replicas x{world}",
                       "l2": "inputs larger than L2 (25 x 128^3 systems, ~12 GB)",
                       "sweep_shapes": {"xyz": [list(v) for v in shapes],
                                        "fields": "substitution lines/block, ring rows, "
                                                  "rhs threads/block (set-up autotuner)"}},
            "cycles_mean": float(np.mean(cycles)), "refinements_mean": float(np.mean(refs)),
            "max_rel_residual": float(max(rels)), "all_converged": ok,
            "learned": learned, "mixed_without_learned": without,
            "reference_cycle": refcyc,
            "plain_fp64": plain,
            "speedup_vs_plain_fp64": round(value / plain["value"], 3) if plain else None,
            "plain_fp64_refactoring": plain_rec,
            "speedup_vs_plain_fp64_refactoring":
                round(value / plain_rec["value"], 3) if plain_rec else None,
            "roofline": roof, "parity": parity, "cpu_baseline": cpu, "e2e": e2e,
            "fwi_eval": fwi, "config5": c5,
            "gpu_launches": timed_launches, "clocks": clk.summary(),
        }
        print(json.dumps(line), flush=True)


def ref_cycle_count(a, plain, cycles):
    """(F-cycles per solve of the reference's algorithm, where the number
    comes from): the reference's own count on this configuration, else the
    FP64 GPU count of the same algorithm (multicolour sweeps)."""
    rc = reference_cycles(a.n, a.tol)
    if rc is not None:
        mean, shots, counts = rc
        return mean, (f"the reference's own F-cycle count to {a.tol:g} on shots "
                      f"{', '.join(map(str, shots))} of this configuration: "
                      f"{', '.join(map(str, counts))}")
    if plain:
        return plain["cycles_mean"], "the FP64 GPU count of the same algorithm"
    if cycles:
        return float(np.mean(cycles)), "the GPU's cycle count"
    return 16.0, "the reference's count at 128^3 on the layered model"


def reference_arm(a, rank, world, pg):
    """The reference's own CPU algorithm (oracle restatement: the reference
    cannot be built on the GPU machine) on all host threads."""
    if rank != 0:
        return
    from libemmi_mgfd_gb300 import build as B
    B.build()
    w = build_workload(a.n)
    nthr = os.cpu_count() or 1
    cps, note = ref_cycle_count(a, None, None)
    for _ in range(max(0, a.warmup)):
        cpu_sample(w, nthr, cps, note)
    vals, secs = [], 0.0
    for _ in range(max(1, a.steps)):
        v, dt, sample = cpu_sample(w, nthr, cps, note)
        vals.append(v)
        secs += dt
    value = statistics.mean(vals)
    line = {
        "metric": METRIC, "value": round(value, 5), "unit": UNIT, "n_gpus": world,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": round(1e3 * secs / max(1, a.steps), 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
        "data": "synthetic (seeded log-normal model, no public dataset)",
        "config": {"workload": f"c3_lognormal_{a.n}^3_25shots_1Hz", "n": a.n, "tol": a.tol,
                   "precision": "fp64", "ordering": "lexicographic (the reference's)"},
        "impl": "reference",
        "cpu_baseline": {"value": round(value, 5), "unit": UNIT, "cores": nthr, "kind": "port",
                         "sample": sample},
        "e2e": {"value": round(value, 5), "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
