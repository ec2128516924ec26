"""MPS / QPS reader parity and the drop-in commands (no GPU).

The reader (read_mps_file of libcp_al_gb300.so and libfa_cp_gb300.so) must
give bit-identical problems to the reference's own readers
(LP/CP_AL/src/mps_parser.c, QP/FA_CP/src/mps_parser.c): against fixtures the
reference reader produced (tests/golden/mps, see make_mps_golden.py), and,
where the reference sources are present, against the reference readers
themselves (built by oracle/build.py into oracle/_ref/) on more seeded
texts.  Reading is host code: nothing here touches a GPU.
"""
import ctypes as C
import gzip
import json
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

from pdal_gb300 import _native as N
from pdal_gb300 import mps

sys.path.insert(0, str(Path(__file__).resolve().parent))
from mps_cases import messy_mps  # noqa: E402

ROOT = Path(__file__).resolve().parent.parent
GOLDEN = ROOT / "tests" / "golden" / "mps"


def ours(lib, path: Path, quadratic: bool):
    ptr = lib.read_mps_file(str(path).encode())
    if not ptr:
        return None
    try:
        return mps.qp_arrays(ptr.contents) if quadratic else mps.lp_arrays(ptr.contents)
    finally:
        (lib.qp_problem_free if quadratic else lib.lp_problem_free)(ptr)


def bits(v):
    a = np.asarray(v)
    return a.view(np.int64) if a.dtype == np.float64 else a


def decode(x):
    if isinstance(x, list):
        if x and isinstance(x[0], str):
            return np.array([float.fromhex(s) for s in x])
        return np.array(x, dtype=np.int64) if x and isinstance(x[0], int) else np.array(x)
    return float.fromhex(x) if isinstance(x, str) else x


def assert_same(got: dict, want: dict, where: str):
    for k, w in want.items():
        g = got[k]
        if isinstance(w, tuple) or (isinstance(w, list) and w and isinstance(w[0], (list, np.ndarray))):
            assert len(g) == len(w), (where, k)
            for gi, wi in zip(g, w):
                assert np.array_equal(bits(np.asarray(gi, dtype=np.asarray(wi).dtype)), bits(wi)), (where, k)
        elif isinstance(w, np.ndarray):
            g = np.asarray(g, dtype=w.dtype) if g is not None else np.zeros(0, w.dtype)
            assert np.array_equal(bits(g), bits(w)), (where, k, g, w)
        elif isinstance(w, float):
            assert np.float64(g).view(np.int64) == np.float64(w).view(np.int64), (where, k, g, w)
        else:
            assert g == w, (where, k, g, w)


def golden_cases():
    return sorted(p.stem for p in GOLDEN.glob("*.json"))


@pytest.mark.parametrize("case", golden_cases())
def test_reader_matches_reference_fixtures(case, lp_lib, qp_lib):
    quad = (GOLDEN / f"{case}.qps").exists()
    src = GOLDEN / (case + (".qps" if quad else ".mps"))
    raw = json.loads((GOLDEN / f"{case}.json").read_text())
    got = ours(qp_lib if quad else lp_lib, src, quad)
    if raw is None:
        assert got is None
        return
    want = {}
    for k, v in raw.items():
        if k in ("A", "Q") and v is not None:
            want[k] = tuple(decode(x) for x in v)
        else:
            want[k] = decode(v)
    for k in ("row_ptr", "col_ind", "num_variables", "num_constraints", "nnz", "num_rank_lowrank_obj",
              "lowrank_nnz"):
        if k in want and isinstance(want[k], np.ndarray):
            want[k] = want[k].astype(np.int32)
    if "A" in want:
        want["A"] = (want["A"][0].astype(np.int32), want["A"][1].astype(np.int32), want["A"][2])
        want["Q"] = (want["Q"][0].astype(np.int32), want["Q"][1].astype(np.int32), want["Q"][2])
    assert_same(got, want, case)


def reference_libs():
    sys.path.insert(0, str(ROOT))
    from oracle import build as ob

    try:
        built = {p.name: p for p in ob.build_ref()}
    except RuntimeError as e:  # the reference is present but did not compile here
        pytest.skip(str(e))
    if not built:
        pytest.skip("reference sources absent: the fixtures carry the parity check")
    libs = {}
    for name, quad, st in (("libref_mps_lp.so", False, N.LpProblem), ("libref_mps_qp.so", True, N.QpProblem)):
        lib = C.CDLL(str(built[name]))
        lib.read_mps_file.restype = C.POINTER(st)
        lib.read_mps_file.argtypes = [C.c_char_p]
        free = lib.qp_problem_free if quad else lib.lp_problem_free
        free.argtypes, free.restype = [C.POINTER(st)], None
        libs[quad] = lib
    return libs


@pytest.mark.parametrize("quad", [False, True])
def test_reader_matches_reference_reader(quad, lp_lib, qp_lib, tmp_path):
    ref = reference_libs()[quad]
    for seed in range(1000, 1060):
        src = tmp_path / f"case{seed}.{'qps' if quad else 'mps'}"
        src.write_bytes(messy_mps(seed, quad).encode())
        want = ours(ref, src, quad)
        got = ours(qp_lib if quad else lp_lib, src, quad)
        if want is None:
            assert got is None, seed
        else:
            assert_same(got, want, f"seed {seed}")


def test_gzip_input_reads_like_plain(lp_lib, tmp_path):
    text = messy_mps(7).encode()
    (tmp_path / "a.mps").write_bytes(text)
    with gzip.open(tmp_path / "a.mps.gz", "wb") as f:
        f.write(text)
    a = ours(lp_lib, tmp_path / "a.mps", False)
    b = ours(lp_lib, tmp_path / "a.mps.gz", False)
    assert_same(b, a, "gz")


def test_reader_errors(lp_lib, qp_lib, tmp_path):
    assert not lp_lib.read_mps_file(str(tmp_path / "missing.mps").encode())
    assert "Could not open" in N.last_error(lp_lib)
    assert not qp_lib.read_mps_file(str(tmp_path / "missing.qps").encode())
    assert "Could not open" in N.last_error(qp_lib)
    bad = tmp_path / "bad.mps"
    bad.write_text("ROWS\n N OBJ\n E R\nCOLUMNS\n R 1\nENDATA\n")  # data before any column name
    assert not lp_lib.read_mps_file(str(bad).encode())
    assert "Column data found before any column name" in N.last_error(lp_lib)
    long = tmp_path / "long.mps"
    long.write_text("ROWS\n N OBJ\n* " + "x" * 5000 + "\nENDATA\n")
    assert not lp_lib.read_mps_file(str(long).encode())
    assert "longer than 4095" in N.last_error(lp_lib)


def test_maximize_negates_objective(qp_lib, tmp_path):
    # OBJSENSE is honoured only when its body line has two or more tokens (a
    # lone "MAX" is taken for a section header, as in the reference reader)
    text = "ROWS\n N OBJ\n E C\nCOLUMNS\n X OBJ 2 C 1\nRHS\n RHS OBJ 3 C 1\nQUADOBJ\n X X 4\nENDATA\n"
    lone = tmp_path / "lone.qps"
    lone.write_text("OBJSENSE\n MAX\n" + text)
    two = tmp_path / "two.qps"
    two.write_text("OBJSENSE\n MAX yes\n" + text)
    a, b = ours(qp_lib, lone, True), ours(qp_lib, two, True)
    assert a["c"][0] == 2.0 and a["objective_constant"] == -3.0 and a["Q"][2][0] == 4.0
    assert b["c"][0] == -2.0 and b["objective_constant"] == 3.0 and b["Q"][2][0] == -4.0


def test_writer_round_trip(lp_lib, qp_lib, tmp_path):
    from pdal_gb300 import instances
    from pdal_gb300.qp import QPData

    d = instances.batch_lps(count=1, seed=5, m_range=(40, 41))[0]
    d.c0 = 1.25
    d.con_lb = np.asarray(d.con_lb, dtype=np.float64).copy()
    d.con_ub = np.asarray(d.con_ub, dtype=np.float64).copy()
    d.con_lb[0], d.con_ub[0] = -np.inf, 3.0
    d.con_lb[1], d.con_ub[1] = 2.0, np.inf
    d.con_lb[2], d.con_ub[2] = -np.inf, np.inf
    d.var_lb = np.asarray(d.var_lb, dtype=np.float64).copy()
    d.var_ub = np.asarray(d.var_ub, dtype=np.float64).copy()
    d.var_lb[0], d.var_ub[0] = -np.inf, np.inf
    d.var_lb[1], d.var_ub[1] = -np.inf, 5.0
    d.var_lb[2], d.var_ub[2] = 1.5, 1.5
    d.var_lb[3] = -2.0
    path = mps.write_lp(d, tmp_path / "rt.mps")
    r = mps.read_lp(path)
    rp, ci, v, shape = d.csr()
    rp2, ci2, v2, shape2 = r.csr()
    assert shape2 == shape
    assert np.array_equal(rp2, rp) and np.array_equal(ci2, ci) and np.array_equal(v2, v)
    for k in ("c", "con_lb", "con_ub", "var_lb", "var_ub"):
        assert np.array_equal(np.asarray(getattr(r, k)), np.asarray(getattr(d, k))), k
    assert r.c0 == d.c0

    import scipy.sparse as sp

    rng = np.random.default_rng(3)
    B = sp.random(6, 8, density=0.4, random_state=4, format="csr")
    Q = (B.T @ B + sp.diags(rng.uniform(0.1, 1, 8))).tocsr()
    q = QPData(rng.standard_normal(8), sp.random(5, 8, density=0.5, random_state=5, format="csr"),
               np.full(5, -1.0), np.full(5, 1.0), np.full(8, -2.0), np.full(8, 2.0), Q=Q, c0=-0.5)
    qr = mps.read_qp(mps.write_qp(q, tmp_path / "rt.qps.gz"))
    Qr = sp.csr_matrix((qr.Q[2], qr.Q[1], qr.Q[0]), shape=(8, 8))
    assert abs(Qr - Q).max() == 0.0
    assert np.array_equal(qr.c, q.c) and qr.c0 == q.c0


# ---------------------------------------------------------------- the commands

def _exe(name):
    p = N.LIBDIR / name
    if not p.exists():
        from pdal_gb300 import build

        build.build_product()
    return p


@pytest.mark.parametrize("name", ["cp_al", "fa_cp"])
def test_cli_usage_and_argument_errors(name, tmp_path):
    exe = str(_exe(name))
    h = subprocess.run([exe, "-h"], capture_output=True, text=True)
    assert h.returncode == 0 and "Usage:" in h.stderr and "<output_dir>" in h.stderr
    r = subprocess.run([exe, "only_one_arg"], capture_output=True, text=True)
    assert r.returncode == 1 and "You must specify an input file and an output directory" in r.stderr
    r = subprocess.run([exe, "--opt_norm", "l3", "a", "b"], capture_output=True, text=True)
    assert r.returncode == 1 and "opt_norm must be" in r.stderr
    r = subprocess.run([exe, "--no_such_option", "a", "b"], capture_output=True, text=True)
    assert r.returncode == 1
    r = subprocess.run([exe, str(tmp_path / "missing.mps"), str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 1 and "Failed to read or parse the file." in r.stderr


def test_cli_sigma_rule_names(tmp_path):
    r = subprocess.run([str(_exe("fa_cp")), "--sigma_update", "bogus", "a", "b"], capture_output=True, text=True)
    assert r.returncode == 1 and "sigma_update must be" in r.stderr


def test_cli_policy_audit_without_a_solve(tmp_path):
    """The `cp_al` command's policy layer in the reference's order
    (LP/CP_AL/src/cli.c:1031-1064): with CP_AL_UNIFIED_POLICY the features
    are computed, the decision list picks the structural-tail route of a
    transportation LP (all rows equalities, dense costs, unit coefficients),
    the feature policy picks its Curtis-Reid effort, and
    CP_AL_FEATURE_AUDIT_ONLY stops before any solve (so no GPU is needed)."""
    from pdal_gb300 import instances, mps

    src = mps.write_lp(instances.transport_lp(5, 6, seed=4001), tmp_path / "t.mps")
    env = {"PATH": "/usr/bin:/bin", "CP_AL_UNIFIED_POLICY": "1", "CP_AL_FEATURE_AUDIT_ONLY": "1"}
    r = subprocess.run([str(_exe("cp_al")), str(src), str(tmp_path)], capture_output=True, text=True, env=env)
    assert r.returncode == 0, r.stderr
    assert "[unified-policy] version=2 route=high_equality_tail_or_base" in r.stderr
    assert "[feature-matrix-stats] computed=1 feature_policy=1 structural_tail=1" in r.stderr
    assert "variant=safe0" in r.stderr and "cr_selected=5" in r.stderr
    assert "[feature-auto-policy-time] seconds=" in r.stderr
    assert not (tmp_path / "t_summary.txt").exists()


@pytest.mark.parametrize("quad", [False, True])
def test_reader_matches_reference_on_mutated_texts(quad, lp_lib, qp_lib, tmp_path):
    """Seeded mutations of valid texts (lines dropped or repeated, tokens
    dropped, stray tokens such as 1e309, nan, -inf, hex floats, names,
    'MARKER' appended): the two readers agree on every one, refusal included."""
    import random

    ref = reference_libs()[quad]
    rng = random.Random(7 + quad)
    extras = ["1e309", "nan", "-inf", "X1", "R0", "'MARKER'", "0x1p3", "+", "COST"]
    for it in range(150):
        lines = messy_mps(7000 + it, quad).split("\n")
        for _ in range(rng.randint(1, 6)):
            op, i = rng.randint(0, 3), rng.randrange(len(lines))
            if op == 0 and len(lines) > 1:
                del lines[i]
            elif op == 1:
                lines.insert(i, lines[rng.randrange(len(lines))])
            elif op == 2:
                toks = lines[i].split()
                if toks:
                    del toks[rng.randrange(len(toks))]
                lines[i] = " ".join(toks)
            else:
                lines[i] = lines[i] + " " + rng.choice(extras)
        src = tmp_path / f"m{it}.{'qps' if quad else 'mps'}"
        src.write_text("\n".join(lines))
        want = ours(ref, src, quad)
        got = ours(qp_lib if quad else lp_lib, src, quad)
        if want is None:
            assert got is None, it
        else:
            assert_same(got, want, f"mutation {it}")
