"""The drop-in headers against the reference's own.

* Every struct of the C ABI (sizeof and the offset of every member) and every
  enumerator of include/cp_al_types.h and include/fa_cp_types.h equals the
  reference's LP/CP_AL/include/cp_al_types.h and QP/FA_CP/include/
  fa_cp_types.h, as recorded in tests/golden/ref_layouts.json by
  tests/golden/make_ref_layouts.py (compiled against the reference headers).
* Where the reference checkout is present (PDAL_REFERENCE_DIR), the record is
  regenerated and must be current, and the C examples of the reference's own
  documentation (LP/CP_AL/docs/C_API.md, QP/FA_CP/docs/C_API.md), compiled
  against the reference's headers, link against this repository's
  libraries: code written for the reference builds unchanged on them.
No GPU is needed (nothing is run on a device).
"""
from __future__ import annotations

import json
import os
import re
import subprocess
from pathlib import Path

import pytest

import ref_layouts as RL

ROOT = Path(__file__).resolve().parent.parent
GOLDEN = ROOT / "tests" / "golden" / "ref_layouts.json"
REF = Path(os.environ.get("PDAL_REFERENCE_DIR", "/root/reference"))
HAVE_REF = (REF / "LP" / "CP_AL" / "include" / "cp_al_types.h").exists()


@pytest.mark.parametrize("kind", ["lp", "qp"])
def test_headers_have_the_reference_layout(kind, tmp_path):
    ours = RL.run_probe(kind, [ROOT / "include"], tmp_path)
    ref = json.loads(GOLDEN.read_text())[kind]
    diff = {k: (ours.get(k), v) for k, v in ref.items() if ours.get(k) != v}
    assert not diff, diff


@pytest.mark.skipif(not HAVE_REF, reason="reference checkout not present")
def test_recorded_layout_is_current():
    import sys

    sys.path.insert(0, str(ROOT / "tests" / "golden"))
    import make_ref_layouts as M

    assert M.reference_layouts(REF) == json.loads(GOLDEN.read_text())


def _doc_example(md: Path, title: str) -> str:
    text = md.read_text()
    at = text.index(title)
    m = re.search(r"```c\n(.*?)```", text[at:], flags=re.S)
    return m.group(1)


@pytest.mark.skipif(not HAVE_REF, reason="reference checkout not present")
@pytest.mark.parametrize("kind", ["lp", "qp"])
def test_documented_examples_link_against_this_library(kind, tmp_path, lp_lib, qp_lib):
    from pdal_gb300 import _native as N

    proj, lib, title = (("LP/CP_AL", "libcp_al_gb300.so", "Example: Solving a Small LP") if kind == "lp"
                        else ("QP/FA_CP", "libfa_cp_gb300.so", "Example: Solving a Small QP"))
    src = tmp_path / f"example_{kind}.c"
    src.write_text(_doc_example(REF / proj / "docs" / "C_API.md", title))
    exe = tmp_path / f"example_{kind}"
    cmd = ["gcc", "-std=gnu99", "-I", str(ROOT / "oracle" / "ref_shim"), "-I", str(REF / proj / "include"),
           str(src), "-o", str(exe), "-L", str(N.LIBDIR), f"-l:{lib}", f"-Wl,-rpath,{N.LIBDIR}", "-lm"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
