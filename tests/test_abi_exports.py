"""Every function the C headers in include/ declare is exported by the
library that implements it (no compute call: this runs without a GPU)."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")
PKG = os.path.join(ROOT, "libemmi_mgfd_gb300")
LIBS = {"emmi_gpu.h": "libemmi_gpu.so", "emmi_dropin.h": "libemmi_gpu.so",
        "emmi_host.h": "libemmi_host.so", "emmi_fwi.h": "libemmi_host.so"}

DECL = re.compile(r"^[A-Za-z_][\w \t\*]*?\b([A-Za-z_]\w*)\s*\(", re.M)


def declared(header):
    text = open(os.path.join(INCLUDE, header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"^\s*#.*$", "", text, flags=re.M)
    names = []
    for m in DECL.finditer(text):
        line = text[m.start():text.find(";", m.start()) + 1]
        if "typedef" in line or "(*" in line or not line.rstrip().endswith(";"):
            continue
        names.append(m.group(1))
    return sorted(set(names))


@pytest.fixture(scope="module")
def built():
    from libemmi_mgfd_gb300 import build as B
    B.build()


def test_headers_cover_the_libraries():
    assert set(LIBS) == {f for f in os.listdir(INCLUDE) if f.endswith(".h")}


@pytest.mark.parametrize("header", sorted(LIBS))
def test_every_declared_function_is_exported(built, header):
    names = declared(header)
    assert names, header
    lib = C.CDLL(os.path.join(PKG, LIBS[header]))
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, (header, missing)


def test_reference_entry_points_are_declared():
    names = set(declared("emmi_dropin.h"))
    for n in ("gmg_init", "gmg_apply", "gmg_free", "inject_source", "inject_adj_source",
              "extract_emf_data", "extract_electric_field", "extract_magnetic_field",
              "build_gradient"):
        assert n in names, n


def test_create_refuses_grids_beyond_32_bit_offsets(built):
    """The stencil kernels use 32-bit slot offsets: emmi_solver_create turns
    down a grid with 2^31 or more edge slots before it touches the device."""
    import numpy as np
    from libemmi_mgfd_gb300 import gpu as G
    n = (1300, 1300, 1300)
    x = [np.arange(v + 1, dtype=np.float32) for v in n]
    with pytest.raises(G.EmmiError, match="2\\^31"):
        G.Solver(n, *x, np.zeros((1, 4, 1), np.float32), np.ones(1, np.float32))


@pytest.mark.parametrize("args,msg", [(["mode=3"], "mode must be"),
                                      (["mode=1", "method=1"], "Gauss-Newton")])
def test_main_refuses_bad_parameters_before_any_work(built, tmp_path, args, msg):
    """emmi_main checks mode= and the inversion method before it reads a
    file or touches the device, so this runs without a GPU."""
    import subprocess
    r = subprocess.run([os.path.join(PKG, "emmi_main")] + args + ["freqs=1"], cwd=tmp_path,
                       capture_output=True, text=True, timeout=60)
    assert r.returncode != 0 and msg in (r.stdout + r.stderr), r.stdout + r.stderr


def test_main_refuses_a_truncated_model_file(built, tmp_path):
    """A model file shorter than nx*ny*nz floats stops emmi_main with an
    error naming the file, before any device work (no GPU needed)."""
    import subprocess
    from libemmi_mgfd_gb300 import workloads as W
    s = W.tiny_layered()
    s.write(str(tmp_path))
    f = tmp_path / "frho11"
    f.write_bytes(f.read_bytes()[:-4])
    r = subprocess.run([os.path.join(PKG, "emmi_main")] + s.params(str(tmp_path)), cwd=tmp_path,
                       capture_output=True, text=True, timeout=60)
    assert r.returncode != 0 and "frho11" in (r.stdout + r.stderr), r.stdout + r.stderr
