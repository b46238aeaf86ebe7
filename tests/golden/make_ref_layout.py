"""The reference's struct layouts (emf_t, acq_t, fwi_t) as a JSON table.

Compiles a small C program against the reference's own headers
(include/emf.h, include/acq.h, include/fwi.h under REF_ROOT) that prints
sizeof of each struct and offsetof of every member, the members being those
include/emmi_dropin.h restates (emmi_emf_t, emmi_acq_t, emmi_fwi_t), and
writes tests/golden/ref_struct_layout.json.  The reference's headers do not
exist on GPU machines; the table carries their layout there
(tests/test_struct_layout.py compares the drop-in header with it).

    REF_ROOT=<reference checkout> python tests/golden/make_ref_layout.py
"""
from __future__ import annotations

import json
import os
import re
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
PAIRS = {"emf_t": "emmi_emf_t", "acq_t": "emmi_acq_t", "fwi_t": "emmi_fwi_t"}


def dropin_members(header: str) -> dict:
    """Member names of the drop-in structs, in declaration order."""
    text = open(header).read()
    out = {}
    for ref, ours in PAIRS.items():
        m = re.search(r"typedef struct \{([^{}]*)\}\s*" + ours + ";", text)
        body = re.sub(r"/\*.*?\*/", "", m.group(1), flags=re.S)
        names = []
        for decl in body.split(";"):
            decl = decl.strip()
            if not decl:
                continue
            first, *rest = decl.split(",")
            names.append(first.split()[-1].lstrip("*"))
            names += [r.strip().lstrip("*") for r in rest]
        out[ref] = names
    return out


def layout_program(members: dict, prefix: str, includes) -> str:
    lines = ["#include <stddef.h>", "#include <stdio.h>"] + [f'#include "{h}"' for h in includes]
    lines.append("int main(void) {")
    for ref, names in members.items():
        cname = prefix + ref if prefix else ref
        lines.append(f'  printf("{ref} size %zu\\n", sizeof({cname}));')
        for nm in names:
            lines.append(f'  printf("{ref} {nm} %zu\\n", offsetof({cname}, {nm}));')
    lines += ["  return 0;", "}"]
    return "\n".join(lines) + "\n"


def run_layout(src: str, incdir: str) -> dict:
    d = tempfile.mkdtemp(prefix="layout_")
    c = os.path.join(d, "layout.c")
    exe = os.path.join(d, "layout")
    with open(c, "w") as f:
        f.write(src)
    subprocess.run(["gcc", "-std=gnu99", "-I" + incdir, c, "-o", exe], check=True,
                   capture_output=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    table = {}
    for line in out.splitlines():
        ref, nm, v = line.split()
        table.setdefault(ref, {})[nm] = int(v)
    return table


def reference_layout(ref_root: str) -> dict:
    members = dropin_members(os.path.join(ROOT, "include", "emmi_dropin.h"))
    # the reference's headers use its complex type from cstd.h
    src = layout_program(members, "", ["cstd.h", "emf.h", "acq.h", "fwi.h"])
    return run_layout(src, os.path.join(ref_root, "include"))


def main():
    ref_root = os.environ.get("REF_ROOT", os.path.join(os.path.dirname(ROOT), "reference"))
    if not os.path.exists(os.path.join(ref_root, "include", "emf.h")):
        sys.exit(f"reference headers not found under {ref_root}")
    table = reference_layout(ref_root)
    path = os.path.join(HERE, "ref_struct_layout.json")
    with open(path, "w") as f:
        json.dump({"source": "include/emf.h, include/acq.h, include/fwi.h of the reference "
                             "(gcc, this machine's ABI)", "layout": table}, f, indent=1,
                  sort_keys=True)
    print(path, {k: v["size"] for k, v in table.items()})


if __name__ == "__main__":
    main()
