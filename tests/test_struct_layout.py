"""The Python ctypes mirrors of the C ABI's structs have the C layout: a
small C program built against include/emmi_gpu.h and include/emmi_fwi.h
prints every field's offset and each struct's size, compared with ctypes
(no GPU)."""
import ctypes as C
import os
import subprocess

import pytest

from libemmi_mgfd_gb300 import gpu as G
from test_fwi_host import EfOpt

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
STRUCTS = {"emmi_options": G._Options, "emmi_problem": G._Problem,
           "emmi_survey": G._Survey, "emmi_fg_problem": G._FgProblem,
           "emmi_rhs_stats": G._Stats, "ef_opt": EfOpt}


@pytest.fixture(scope="module")
def c_layout(tmp_path_factory):
    d = tmp_path_factory.mktemp("layout")
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "emmi_gpu.h"',
             '#include "emmi_fwi.h"', "int main(void) {"]
    for cname, py in STRUCTS.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'  printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["  return 0;", "}"]
    src = d / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = d / "layout"
    subprocess.run(["gcc", "-std=gnu99", "-I" + os.path.join(ROOT, "include"), str(src), "-o",
                    str(exe)], check=True, capture_output=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    return {tuple(l.split()[:2]): int(l.split()[2]) for l in out.splitlines()}


@pytest.mark.parametrize("cname", sorted(STRUCTS))
def test_ctypes_mirror_matches_the_c_struct(c_layout, cname):
    py = STRUCTS[cname]
    assert C.sizeof(py) == c_layout[(cname, "size")], cname
    for fname, _ in py._fields_:
        assert getattr(py, fname).offset == c_layout[(cname, fname)], (cname, fname)


def _dropin_layout():
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "make_ref_layout", os.path.join(ROOT, "tests", "golden", "make_ref_layout.py"))
    mk = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mk)
    members = mk.dropin_members(os.path.join(ROOT, "include", "emmi_dropin.h"))
    src = mk.layout_program(members, "emmi_", ["emmi_dropin.h"])
    return mk, mk.run_layout(src, os.path.join(ROOT, "include"))


def test_dropin_structs_have_the_reference_layout():
    """include/emmi_dropin.h against the reference's emf_t / acq_t / fwi_t
    (include/emf.h:4-48, acq.h:4-19, fwi.h:4-28): every member's offset and
    each struct's size, from the table tests/golden/make_ref_layout.py
    compiled out of the reference's own headers; where those headers are
    present (REF_ROOT, default: a checkout named `reference` beside this
    repository) the table is also rebuilt from them live."""
    import json
    mk, ours = _dropin_layout()
    with open(os.path.join(ROOT, "tests", "golden", "ref_struct_layout.json")) as f:
        ref = json.load(f)["layout"]
    assert ours == ref
    ref_root = os.environ.get("REF_ROOT", os.path.join(os.path.dirname(ROOT), "reference"))
    if os.path.exists(os.path.join(ref_root, "include", "emf.h")):
        assert mk.reference_layout(ref_root) == ours
