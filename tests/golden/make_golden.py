"""Generate the golden fixtures in tests/golden/ from the reference itself.

Runs oracle/_ref/ref_dump (the reference compiled from its own C sources by
``make -C oracle ref``) on small seeded cases and stores what it wrote --
grids, homogenized conductivities, injected right-hand sides, converged E/H
slot fields, receiver data, volume extractions, adjoint sources and the
mode=2 gradient -- as compressed .npz files.  The reference does not exist on
GPU machines; these fixtures carry its outputs there.

    python tests/golden/make_golden.py            (needs oracle/_ref built)
    python tests/golden/make_golden.py tiny_grad  (the mode=2 gradient case only)
    python tests/golden/make_golden.py tiny_fwi   (the mode=1 inversion case only)
    python tests/golden/make_golden.py c3 c2 c4   (benchmark configurations, minutes each)
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from libemmi_mgfd_gb300 import workloads as W  # noqa: E402

REF_DUMP = os.path.join(ROOT, "oracle", "_ref", "ref_dump")
REF_MAIN = os.path.join(ROOT, "oracle", "_ref", "emmi_ref")


def run_ref(s: W.Survey, extra, adjoint: int):
    d = tempfile.mkdtemp(prefix="golden_")
    s.write(d)
    args = [REF_DUMP] + s.params(d) + [f"dumpdir={d}", f"adjoint={adjoint}", "verb=1"] + list(extra)
    r = subprocess.run(args, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(r.stdout + r.stderr)
    return d, r.stdout


def load(d, nm, dt):
    return np.fromfile(os.path.join(d, nm), dt)


def case(s: W.Survey, extra, adjoint=0, keep_fields=True, nfreq=1, tag=None):
    d, out = run_ref(s, extra, adjoint)
    f32, c128, c64 = np.float32, np.complex128, np.complex64
    rec = {
        "name": np.array(tag or s.name),
        "params": np.array(" ".join(extra)),
        "n": np.array(s.n, np.int32),
        "nxyz": np.array([s.nx, s.ny, s.nz], np.int32),
        "o": np.array([s.ox, s.oy, s.oz], f32),
        "dxyz": np.array([s.dx, s.dy, s.dz], f32),
        "rho11": s.rho11, "rho22": s.rho22, "rho33": s.rho33,
        "sources": s.sources.astype(f32), "receivers": s.receivers.astype(f32),
        "chsrc": np.array(",".join(s.chsrc)), "chrec": np.array(",".join(s.chrec)),
        "freqs": np.array(s.freqs, f32),
        "extra_keys": np.array(" ".join(f"{k}={v}" for k, v in s.extra.items())),
        "omegas": load(d, "omegas", f32), "rho_water": load(d, "rho_water", f32),
        "srcrec": load(d, "srcrec", f32), "dcal": load(d, "dcal", c64),
    }
    # residual history of each solve, as the reference prints it (gmg.c:1627)
    solves, cur = [], None
    for line in out.splitlines():
        if "gmg_init" in line:
            cur = []
            solves.append(cur)
        elif line.startswith("icycle=") and cur is not None:
            cur.append(float(line.split("rnorm=")[1]))
    rec["rnorm_fwd"] = np.array(solves[0] if solves else [], np.float64)
    if adjoint and len(solves) > nfreq:
        rec["rnorm_adj"] = np.array(solves[nfreq], np.float64)
    for nm in ("x1", "x2", "x3", "x1s", "x2s", "x3s", "d1", "d2", "d3", "d1s", "d2s", "d3s",
               "sigma11", "sigma22", "sigma33", "invmur"):
        rec[nm] = load(d, nm, f32)
    if keep_fields:
        for f in range(nfreq):
            for nm in (f"b_f{f}", f"x_f{f}", f"h_f{f}"):
                rec[nm] = load(d, nm, c128)
        for nm in ("E1", "E2", "E3", "H1", "H2", "H3"):
            rec[nm] = load(d, nm, c64)
    if adjoint:
        rec["dres"] = load(d, "dres", c64)
        for f in range(nfreq):
            for nm in (f"badj_f{f}", f"madj_f{f}", f"xa_f{f}"):
                rec[nm] = load(d, nm, c128)
        for nm in ("E1a", "E2a", "E3a"):
            rec[nm] = load(d, nm, c64)
        rec["grad"] = load(d, "grad", f32)
        rec["phess"] = load(d, "phess", f32)
        rec["bathy"] = np.array(1000.0, f32)
    return rec


def start_model(s: W.Survey) -> W.Survey:
    """The starting model of the gradient case: the resistive layer of the
    layered model removed (1 ohm-m below the water)."""
    rho = np.where(s.rho11 > 10.0, 1.0, s.rho11).astype(np.float32)
    return W.Survey(s.name + "_start", s.nx, s.ny, s.nz, s.dx, s.dy, s.dz, s.ox, s.oy, s.oz,
                    rho, rho.copy(), rho.copy(), s.sources, s.receivers, s.pairs, s.freqs, s.n,
                    s.chsrc, s.chrec, dict(s.extra), s.bathy)


def mode2_case(tol="1e-10"):
    """The reference's main in mode=2 (one data gradient, src/fg_fwi.c):
    observed data from a mode=0 run on the layered model, gradient of the
    start model, without noise."""
    true = W.tiny_layered()
    start = start_model(true)
    d = tempfile.mkdtemp(prefix="golden_m2_")
    true.write(os.path.join(d, "true"))
    start.write(d)
    common = [f"tol={tol}", "ncycle=80"]
    r0 = subprocess.run([REF_MAIN] + true.params(os.path.join(d, "true")) + common, cwd=d,
                        capture_output=True, text=True)
    if r0.returncode != 0:
        raise RuntimeError(r0.stdout + r0.stderr)
    obs_text = open(os.path.join(d, "emf_0001.txt")).read()
    args = [a for a in start.params(d) if not a.startswith("mode=") and not a.startswith("verb=")]
    args += ["mode=2", "verb=1", "addnoise=0", "npar=2", "idxpar=1,2", "preco=1"] + common
    r2 = subprocess.run([REF_MAIN] + args, cwd=d, capture_output=True, text=True)
    if r2.returncode != 0:
        raise RuntimeError(r2.stdout + r2.stderr)
    n = start.nx * start.ny * start.nz
    fcost = [float(l.split("fcost=")[1].split(",")[0]) for l in r2.stdout.splitlines()
             if l.startswith("isrc=")]
    rm = np.loadtxt(os.path.join(d, "rmse_0001.txt"), skiprows=1, usecols=(4,))
    syn = np.loadtxt(os.path.join(d, "syn_0001.txt"), skiprows=1, usecols=(4, 5))
    return {
        "name": np.array("tiny_grad"),
        "params": np.array(" ".join(args[-6:])),
        "rho_true": true.rho11, "rho_start": start.rho11,
        "obs_text": np.array(obs_text),
        "grad_Rv": np.fromfile(os.path.join(d, "gradient_dat_Rv"), np.float32, n),
        "grad_Rh": np.fromfile(os.path.join(d, "gradient_dat_Rh"), np.float32, n),
        "rmse": rm.astype(np.float32),
        "syn": (syn[:, 0] + 1j * syn[:, 1]).astype(np.complex64),
        "fcost": np.array(fcost, np.float64),
        "stdout": np.array(r2.stdout[-4000:]),
    }


def trace_lines(stdout):
    """The lines of the inversion's stdout that record its path: the
    iteration header, each evaluation's objective, the first-gradient
    scaling and each failed Wolfe condition (src/do_fwi.c, src/opt.c,
    src/fg_fwi.c)."""
    keep = ("# iter=", "fcost=", "|x|_1=", "Wolfe condition")
    return [l.strip() for l in stdout.splitlines() if l.strip().startswith(keep)]


def mode1_case(tol="1e-10", niter=2, preco=1, extra=()):
    """The reference's main in mode=1 (the l-BFGS inversion, src/do_fwi.c)
    for niter iterations from the start model of mode2_case, without noise:
    iterate.txt, rmse_misfit.txt and the resistivities after every
    iteration."""
    true = W.tiny_layered()
    start = start_model(true)
    d = tempfile.mkdtemp(prefix="golden_m1_")
    true.write(os.path.join(d, "true"))
    start.write(d)
    common = [f"tol={tol}", "ncycle=80"]
    r0 = subprocess.run([REF_MAIN] + true.params(os.path.join(d, "true")) + common, cwd=d,
                        capture_output=True, text=True)
    if r0.returncode != 0:
        raise RuntimeError(r0.stdout + r0.stderr)
    obs_text = open(os.path.join(d, "emf_0001.txt")).read()
    args = [a for a in start.params(d) if not a.startswith("mode=") and not a.startswith("verb=")]
    args += ["mode=1", "verb=1", "addnoise=0", "npar=2", "idxpar=1,2", f"preco={preco}",
             f"niter={niter}"] + list(extra) + common
    r1 = subprocess.run([REF_MAIN] + args, cwd=d, capture_output=True, text=True)
    if r1.returncode != 0:
        raise RuntimeError(r1.stdout + r1.stderr)
    n = start.nx * start.ny * start.nz
    rec = {
        "name": np.array("tiny_fwi"),
        "params": np.array(" ".join(args[-7 - len(extra):])),
        "rho_start": start.rho11,
        "obs_text": np.array(obs_text),
        "iterate": np.array(open(os.path.join(d, "iterate.txt")).read()),
        "rmse_misfit": np.array(open(os.path.join(d, "rmse_misfit.txt")).read()),
        "stdout": np.array(r1.stdout[-6000:]),
        # every objective evaluation and line-search decision, in order
        "trace": np.array("\n".join(trace_lines(r1.stdout))),
    }
    for it in range(niter):
        for nm in ("Rv", "Rh"):
            rec[f"{nm}_{it:02d}"] = np.fromfile(os.path.join(d, f"{nm}_iteration_{it:02d}"),
                                                np.float32, n)
    return rec


def sensitivity(niter=2):
    """How far the reference's own inversion moves when only the solver's
    stopping tolerance changes (1e-10 against 1e-8): per preconditioner and
    iteration, the largest log-resistivity difference between the two runs
    beside the largest step from the start model."""
    for preco in (1, 0, 2):
        a = mode1_case(tol="1e-10", niter=niter, preco=preco)
        b = mode1_case(tol="1e-8", niter=niter, preco=preco)
        rho = np.asarray(a["rho_start"]).ravel()
        for it in range(niter):
            for nm in ("Rv", "Rh"):
                x, y = a[f"{nm}_{it:02d}"], b[f"{nm}_{it:02d}"]
                print(f"preco={preco} {nm} iteration {it}: max |dlog rho| "
                      f"{np.abs(np.log(x) - np.log(y)).max():.3g}, step "
                      f"{np.abs(np.log(x) - np.log(rho)).max():.3g}")


def _receivers_one(s: W.Survey, shot: int, extra):
    """ref_dump on one shot; the receiver data, residual history and mesh axes."""
    d = tempfile.mkdtemp(prefix=f"golden_rx{shot}_")
    s.write(d)
    args = ([REF_DUMP] + s.params(d, shot=shot) + [f"dumpdir={d}", "adjoint=0", "verb=1"]
            + list(extra))
    r = subprocess.run(args, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(r.stdout + r.stderr)
    f32, c64 = np.float32, np.complex64
    hist = []
    for line in r.stdout.splitlines():
        if "gmg_init" in line:
            hist.append([])
        elif line.startswith("icycle=") and hist:
            hist[-1].append(float(line.split("rnorm=")[1]))
    out = {"dcal": load(d, "dcal", c64), "omegas": load(d, "omegas", f32),
           "rho_water": load(d, "rho_water", f32), "srcrec": load(d, "srcrec", f32),
           "x1": load(d, "x1", f32), "x2": load(d, "x2", f32), "x3": load(d, "x3", f32),
           "cycles": np.array([len(h) - 1 for h in hist], np.int32),
           "rnorm_last": np.array([h[-1] / h[0] if h else np.nan for h in hist], np.float64)}
    # the printed residual history of each frequency's solve (gmg.c:1627)
    for f, h in enumerate(hist):
        out[f"rnorm_f{f}"] = np.array(h, np.float64)
    subprocess.run(["rm", "-rf", d])
    return out


def receivers_case(s: W.Survey, shots, extra, tag):
    """The reference's receiver data (dcal [nch][nfreq][nrec], complex
    float) for a few shots of a benchmark configuration at the size it is
    measured on, one reference process per shot (the reference runs one shot
    per MPI rank, src/acq_init_free.c:119-140).  Receivers only: the fields
    at these sizes are hundreds of MB."""
    import concurrent.futures as cf
    with cf.ThreadPoolExecutor(max_workers=len(shots)) as ex:
        outs = list(ex.map(lambda k: _receivers_one(s, k, extra), shots))
    rec = {"name": np.array(tag), "params": np.array(" ".join(extra)),
           "n": np.array(s.n, np.int32), "shots": np.array(shots, np.int32),
           "chsrc": np.array(",".join(s.chsrc)), "chrec": np.array(",".join(s.chrec))}
    for k, o in zip(shots, outs):
        for nm, v in o.items():
            rec[f"s{k}_{nm}"] = v
    return rec


def gradient_case(true: W.Survey, start: W.Survey, shots, extra, tag):
    """The reference's mode=2 gradient summed over a few shots: per shot a
    mode=0 run on the true model writes the observed emf_XXXX.txt, then a
    mode=2 run on the start model (addnoise=0) writes gradient_dat_Rv/Rh;
    the per-shot gradients are added in float32 as MPI_Allreduce does
    (src/fg_fwi.c:265-268; two addends, so the order cannot matter)."""
    import concurrent.futures as cf

    def one(k):
        d = tempfile.mkdtemp(prefix=f"golden_g{k}_")
        true.write(os.path.join(d, "true"))
        start.write(d)
        r0 = subprocess.run([REF_MAIN] + true.params(os.path.join(d, "true"), shot=k)
                            + list(extra), cwd=d, capture_output=True, text=True)
        if r0.returncode != 0:
            raise RuntimeError(r0.stdout + r0.stderr)
        obs = open(os.path.join(d, f"emf_{k:04d}.txt")).read()
        args = [a for a in start.params(d, shot=k)
                if not a.startswith("mode=") and not a.startswith("verb=")]
        args += ["mode=2", "verb=1", "addnoise=0", "npar=2", "idxpar=1,2", "preco=1"] + list(extra)
        r2 = subprocess.run([REF_MAIN] + args, cwd=d, capture_output=True, text=True)
        if r2.returncode != 0:
            raise RuntimeError(r2.stdout + r2.stderr)
        n = start.nx * start.ny * start.nz
        g = {nm: np.fromfile(os.path.join(d, "gradient_dat_" + nm), np.float32, n)
             for nm in ("Rv", "Rh")}
        fc = [float(l.split("=")[1].split(",")[0]) for l in r2.stdout.splitlines()
              if l.startswith("fcost_dat=")]
        subprocess.run(["rm", "-rf", d])
        return obs, g, fc

    with cf.ThreadPoolExecutor(max_workers=len(shots)) as ex:
        outs = list(ex.map(one, shots))
    rec = {"name": np.array(tag), "params": np.array(" ".join(extra)),
           "n": np.array(start.n, np.int32), "shots": np.array(shots, np.int32)}
    for nm in ("Rv", "Rh"):
        acc = np.zeros_like(outs[0][1][nm])
        for o in outs:
            acc = (acc + o[1][nm]).astype(np.float32)
        rec[f"grad_{nm}"] = acc
    for k, o in zip(shots, outs):
        rec[f"s{k}_obs_text"] = np.array(o[0])
        rec[f"s{k}_fcost_dat"] = np.array(o[2], np.float64)
    return rec


def config_cases(which):
    """Fixtures at the benchmark configurations' sizes (minutes of CPU):
    c3: two shots of the 128^3 log-normal configuration to 1e-10;
    c2: two shots x two frequencies of the VTI/bathymetry configuration on a
        48x48x64 mesh (the reference cannot mesh it with n3 = 40: the source
        sits 39 input cells down, which leaves one cell for the bottom
        stretch, and create_nugrid's fixed-point loop never ends there);
    c4: the mode=2 gradient of the half-space start model against the
        reservoir model's data, two shots x three frequencies at 64^3."""
    if which == "c3":
        s = W.config3(128)
        rec = receivers_case(s, [1, 13], ["tol=1e-10", "ncycle=200"], "c3_lognormal_128_ref")
    elif which == "c2":
        s = W.config2(96)
        s.n = (48, 48, 64)
        rec = receivers_case(s, [1, 13], ["tol=1e-10", "ncycle=200"], "c2_vti_48x48x64_ref")
    else:
        true = W.config4(64, true_model=True)
        start = W.config4(64, true_model=False)
        rec = gradient_case(true, start, [1, 13], ["tol=1e-10", "ncycle=200"],
                            "c4_reservoir_64_grad_ref")
    path = os.path.join(HERE, str(rec["name"]) + ".npz")
    np.savez_compressed(path, **rec)
    print(rec["name"], os.path.getsize(path) // 1024, "KB")


def main():
    if not os.path.exists(REF_DUMP):
        sys.exit("oracle/_ref/ref_dump missing: run `make -C oracle ref` first")
    only = set(sys.argv[1:])
    if only and only <= {"c2", "c3", "c4"}:
        for w in sorted(only):
            config_cases(w)
        return
    if only == {"sensitivity"}:
        sensitivity()
        return
    if only == {"tiny_fwi_variants"}:
        # the first inversion iteration with the depth preconditioner, the
        # triangle smoothing and the box bounds (one iteration: the second
        # is not reproducible, see mode1_case's test)
        out = {}
        for tag, preco, extra in (("p2", 2, ()), ("p3", 3, ("r1=2", "r2=2", "r3=2")),
                                  ("bound", 1, ("bound=1", "minpar=0.5,0.5",
                                                "maxpar=3,3"))):
            rec = mode1_case(niter=1, preco=preco, extra=extra)
            for k, v in rec.items():
                out[f"{tag}_{k}"] = v
        np.savez_compressed(os.path.join(HERE, "tiny_fwi_variants.npz"), **out)
        print("tiny_fwi_variants",
              os.path.getsize(os.path.join(HERE, "tiny_fwi_variants.npz")) // 1024, "KB")
        return
    if only == {"tiny_fwi"}:
        rec = mode1_case()
        np.savez_compressed(os.path.join(HERE, "tiny_fwi.npz"), **rec)
        print("tiny_fwi", os.path.getsize(os.path.join(HERE, "tiny_fwi.npz")) // 1024, "KB")
        return
    if only == {"tiny_grad"}:
        rec = mode2_case()
        np.savez_compressed(os.path.join(HERE, "tiny_grad.npz"), **rec)
        print("tiny_grad", os.path.getsize(os.path.join(HERE, "tiny_grad.npz")) // 1024, "KB")
        return
    out = {}
    # 1. tiny layered, F-cycles: converged fields + mode=2 adjoint/gradient
    out["tiny_layered"] = case(W.tiny_layered(), ["tol=1e-10", "ncycle=60"], adjoint=1)
    # 2. the same after exactly 3 cycles (iterate-level pin of the oracle)
    out["tiny_layered_it3"] = case(W.tiny_layered(), ["tol=0", "ncycle=3"], tag="tiny_layered_it3")
    # 3. anisotropic, rotated/tilted source, all channels, non-cubic mesh
    out["tiny_aniso"] = case(W.tiny_aniso(n=(16, 8, 16)), ["tol=1e-10", "ncycle=80"])
    # 4. V-cycle / W-cycle / no semi-coarsening iterates
    out["tiny_vcycle_it3"] = case(W.tiny_layered(), ["tol=0", "ncycle=3", "cycleopt=1"],
                                  tag="tiny_vcycle_it3")
    out["tiny_wcycle_it2"] = case(W.tiny_layered(), ["tol=0", "ncycle=2", "cycleopt=3"],
                                  tag="tiny_wcycle_it2")
    out["tiny_point_it3"] = case(W.tiny_layered(), ["tol=0", "ncycle=3", "isemicoarsen=0"],
                                 tag="tiny_point_it3")
    # 5. the reference's own CPU-runnable configuration (64^3), receivers only
    out["c1_layered_64"] = case(W.config1(64), ["tol=1e-8", "ncycle=60"], keep_fields=False,
                                tag="c1_layered_64")
    for k, rec in out.items():
        if k == "c1_layered_64":
            # keep the fixture small: conductivities are layered, compress well
            pass
        np.savez_compressed(os.path.join(HERE, f"{k}.npz"), **rec)
        print(k, os.path.getsize(os.path.join(HERE, f"{k}.npz")) // 1024, "KB")


if __name__ == "__main__":
    main()
