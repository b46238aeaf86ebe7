"""The drop-in boundary against the reference's own build: the reference's
object files -- every one but the hot path's gmg.o, inject_extract.o and
build_gradient.o -- link against libemmi_gpu.so into the reference's main
with no undefined symbol.  The objects are the
ones `make -C oracle ref` compiles from the reference's sources with the
single-rank MPI stub; where the reference is absent the test is skipped.
Linking needs no GPU; running the linked program needs one and the
reference's model files, which the GPU tests cover through emmi_main."""
import glob
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
OBJ = os.path.join(ROOT, "oracle", "_ref", "obj")
HOT = {"gmg.o", "inject_extract.o", "build_gradient.o"}


def test_reference_objects_link_against_the_gpu_library(tmp_path):
    from libemmi_mgfd_gb300 import build
    build.build()
    objs = sorted(glob.glob(os.path.join(OBJ, "*.o")))
    names = {os.path.basename(o) for o in objs}
    if "main.o" not in names or not HOT <= names:
        pytest.skip("reference objects not built here (make -C oracle ref needs its sources)")
    keep = [o for o in objs if os.path.basename(o) not in HOT | {"ref_globals.o"}]
    lib = os.path.join(ROOT, "libemmi_mgfd_gb300")
    exe = tmp_path / "main_gpu"
    r = subprocess.run(["gcc", "-o", str(exe)] + keep +
                       ["-L" + lib, "-lemmi_gpu", "-Wl,-rpath," + lib, "-Wl,--no-undefined",
                        "-lm"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    # the hot-path entry points resolve to the library, not to the reference
    undef = subprocess.run(["nm", "-u", str(exe)], capture_output=True, text=True).stdout
    for sym in ("gmg_init", "gmg_apply", "gmg_free", "inject_source", "inject_adj_source",
                "extract_emf_data", "extract_electric_field", "extract_magnetic_field",
                "build_gradient"):
        assert sym in undef.split(), sym
