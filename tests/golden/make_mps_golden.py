"""Writes the MPS reader fixtures: each case's text (tests/golden/mps/<case>.mps)
and what the reference's own reader makes of it (<case>.json), so that the
reader parity test runs where the reference sources are absent.

The reference readers are LP/CP_AL/src/mps_parser.c and
QP/FA_CP/src/mps_parser.c, compiled unmodified by oracle/build.py (build_ref)
into oracle/_ref/.  Arrays are stored as float.hex() strings (exact, with
inf and nan).  Run from the repository root:

    python tests/golden/make_mps_golden.py
"""
from __future__ import annotations

import ctypes as C
import json
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

from mps_cases import FIXED_CASES, messy_mps  # noqa: E402
from oracle import build as ob  # noqa: E402
from pdal_gb300 import _native as N  # noqa: E402
from pdal_gb300.mps import lp_arrays, qp_arrays  # noqa: E402

OUT = HERE / "mps"
LP_SEEDS = range(0, 12)
QP_SEEDS = range(100, 106)


def cases():
    for name, text in FIXED_CASES.items():
        yield name, text, name.startswith("qps")
    for s in LP_SEEDS:
        yield f"messy_lp_{s}", messy_mps(s, False), False
    for s in QP_SEEDS:
        yield f"messy_qp_{s}", messy_mps(s, True), True


def encode(a: dict) -> dict:
    out = {}
    for k, v in a.items():
        if v is None:
            out[k] = None
        elif isinstance(v, tuple):
            out[k] = [encode({"x": x})["x"] for x in v]
        elif hasattr(v, "dtype"):
            out[k] = [float(x).hex() for x in v] if v.dtype.kind == "f" else [int(x) for x in v]
        elif isinstance(v, float):
            out[k] = v.hex()
        else:
            out[k] = v
    return out


def reference_parse(lib, path: Path, quadratic: bool):
    ptr = lib.read_mps_file(str(path).encode())
    if not ptr:
        return None
    a = qp_arrays(ptr.contents) if quadratic else lp_arrays(ptr.contents)
    (lib.qp_problem_free if quadratic else lib.lp_problem_free)(ptr)
    return a


def load_reference():
    built = {p.name: p for p in ob.build_ref()}
    if not built:
        raise SystemExit("the reference sources are needed to generate these fixtures")
    libs = {}
    for name, quad, st in (("libref_mps_lp.so", False, N.LpProblem), ("libref_mps_qp.so", True, N.QpProblem)):
        lib = C.CDLL(str(built[name]))
        lib.read_mps_file.restype = C.POINTER(st)
        lib.read_mps_file.argtypes = [C.c_char_p]
        free = lib.qp_problem_free if quad else lib.lp_problem_free
        free.argtypes = [C.POINTER(st)]
        free.restype = None
        libs[quad] = lib
    return libs


def main():
    libs = load_reference()
    OUT.mkdir(exist_ok=True)
    for name, text, quad in cases():
        src = OUT / (name + (".qps" if quad else ".mps"))
        src.write_bytes(text.encode())
        a = reference_parse(libs[quad], src, quad)
        (OUT / (name + ".json")).write_text(json.dumps(None if a is None else encode(a), indent=0) + "\n")
        print(name, "NULL" if a is None else f"{a['num_constraints']} x {a['num_variables']}")


if __name__ == "__main__":
    main()
