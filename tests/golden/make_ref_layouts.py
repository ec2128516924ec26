"""Records the struct layouts and enumerator values of the reference's public
headers (LP/CP_AL/include/cp_al_types.h, QP/FA_CP/include/fa_cp_types.h) in
tests/golden/ref_layouts.json, by compiling the probe of tests/ref_layouts.py
against them (with oracle/ref_shim for the absent presolve library's empty
PSLP_stats.h).  Reads the reference from PDAL_REFERENCE_DIR (default: the
reference's usual location).

    python tests/golden/make_ref_layouts.py
"""
from __future__ import annotations

import json
import os
import sys
import tempfile
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT / "tests"))

import ref_layouts as RL  # noqa: E402


def reference_dir() -> Path:
    return Path(os.environ.get("PDAL_REFERENCE_DIR", "/root/reference"))


def reference_layouts(ref: Path) -> dict:
    shim = ROOT / "oracle" / "ref_shim"
    with tempfile.TemporaryDirectory() as td:
        return {"lp": RL.run_probe("lp", [shim, ref / "LP" / "CP_AL" / "include"], Path(td)),
                "qp": RL.run_probe("qp", [shim, ref / "QP" / "FA_CP" / "include"], Path(td))}


def main() -> None:
    out = ROOT / "tests" / "golden" / "ref_layouts.json"
    out.write_text(json.dumps(reference_layouts(reference_dir()), indent=1, sort_keys=True) + "\n")
    print(out)


if __name__ == "__main__":
    main()
