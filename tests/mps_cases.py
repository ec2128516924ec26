"""Seeded MPS / QPS texts for the reader parity tests: every section and
bound type, the layout variations the reader has to handle (comments, blank
lines, tabs, CRLF, continuation lines, MARKER lines, more than six tokens)
and the reference reader's corner cases (no N row, a second N row, unknown
rows and columns, duplicate names and entries, OBJSENSE forms, data after
ENDATA)."""
from __future__ import annotations

import numpy as np

NUMBER_FORMS = ["{:d}", "{:.1f}", "{:.6g}", "{:.3e}", "{:.17g}", "{:+.2E}"]


def _num(rng, allow_zero=True) -> str:
    k = rng.integers(0, 10)
    if k == 0 and allow_zero:
        return "0"
    if k == 1:
        return str(int(rng.integers(-9, 10)))
    v = float(rng.standard_normal() * 10.0 ** int(rng.integers(-3, 4)))
    f = NUMBER_FORMS[int(rng.integers(1, len(NUMBER_FORMS)))]
    return f.format(v)


def _sep(rng) -> str:
    return rng.choice([" ", "  ", "\t", "   ", " \t "])


def _line(rng, tokens) -> str:
    lead = rng.choice(["", " ", "    ", "\t"])
    return lead + _sep(rng).join(tokens)


def messy_mps(seed: int, quadratic: bool = False) -> str:
    rng = np.random.default_rng(seed)
    m = int(rng.integers(0, 9))
    n = int(rng.integers(1, 11))
    rows = [(str(rng.choice(list("ELG"))), f"R{i}") for i in range(m)]
    obj_pos = int(rng.integers(0, m + 1))
    variant = rng.random()
    if variant < 0.8:
        rows.insert(obj_pos, ("N", "COST"))
    if rng.random() < 0.2:
        rows.append(("N", "COST2"))
    if rng.random() < 0.15 and m:
        rows.append(("e", "LOWER"))
    if rng.random() < 0.15 and m:
        rows.append((str(rng.choice(list("ELG"))), rows[-1][1]))  # repeated name
    names = [r[1] for r in rows]
    cols = [f"X{j}" for j in range(n)]

    L = []
    if rng.random() < 0.5:
        L.append("* generated case %d" % seed)
    L.append(f"NAME          CASE{seed}")
    if rng.random() < 0.25:
        L += ["OBJSENSE", "    MAX"]
    elif rng.random() < 0.25:
        L += ["OBJSENSE", "    MAXIMIZE  x"]
    L.append("ROWS")
    for t, nm in rows:
        L.append(_line(rng, [t, nm]))
        if rng.random() < 0.1:
            L.append("")
    L.append("COLUMNS")
    in_int = False
    for j, c in enumerate(cols):
        if rng.random() < 0.15:
            L.append(_line(rng, ["MARKER", "'MARKER'", "'INTEND'" if in_int else "'INTORG'"]))
            in_int = not in_int
        k = int(rng.integers(0, min(len(names), 5) + 2))
        targets = list(rng.choice(names + ["NOSUCHROW"], size=k)) if names else []
        pairs = [(t, _num(rng)) for t in targets]
        if not pairs:
            pairs = [(names[0] if names else "COST", _num(rng))]
        first = True
        while pairs:
            take = 2 if len(pairs) >= 2 and rng.random() < 0.5 else 1
            chunk, pairs = pairs[:take], pairs[take:]
            flat = [x for p in chunk for x in p]
            if first or rng.random() < 0.7:
                L.append(_line(rng, [c] + flat))
            else:
                L.append(_line(rng, flat))  # continuation of the current column
            first = False
        if rng.random() < 0.05:
            L.append(_line(rng, [c] + [x for p in [(names[0] if names else "COST", "1")] * 3 for x in p]))
    L.append("RHS")
    for nm in names + ["NOSUCHROW"]:
        if rng.random() < 0.6:
            if rng.random() < 0.3:
                other = str(rng.choice(names)) if names else nm
                L.append(_line(rng, ["RHS", nm, _num(rng), other, _num(rng)]))
            else:
                L.append(_line(rng, ["RHS", nm, _num(rng)]))
    if rng.random() < 0.1 and names:
        L.append(_line(rng, [names[0], _num(rng)]))  # no set name: ignored by the reader
    if rng.random() < 0.6:
        L.append("RANGES")
        for nm in names:
            if rng.random() < 0.4:
                L.append(_line(rng, ["RNG", nm, _num(rng)]))
    L.append("BOUNDS")
    for c in cols + ["NOSUCHCOL"]:
        for _ in range(int(rng.integers(0, 3))):
            t = str(rng.choice(["LO", "UP", "FX", "FR", "MI", "PL", "BV", "LI", "UI", "SC"]))
            if t in ("FR", "MI", "PL", "BV") and rng.random() < 0.7:
                L.append(_line(rng, [t, "BND", c]))
            else:
                L.append(_line(rng, [t, "BND", c, _num(rng)]))
    if quadratic:
        sec = "QUADOBJ" if rng.random() < 0.6 else "QMATRIX"
        L.append(sec)
        for _ in range(int(rng.integers(0, 2 * n + 2))):
            a, b = rng.integers(0, n, 2)
            if sec == "QUADOBJ" and a > b:
                a, b = b, a
            ca = cols[a] if rng.random() > 0.05 else "NOSUCHCOL"
            L.append(_line(rng, [ca, cols[b], _num(rng)]))
    L.append("ENDATA")
    if rng.random() < 0.2:
        L += ["COLUMNS", " X0 R0 99"]  # after ENDATA: never read
    eol = "\r\n" if rng.random() < 0.15 else "\n"
    text = eol.join(L) + (eol if rng.random() < 0.9 else "")
    return text


FIXED_CASES = {
    "basic": """NAME          BASIC
ROWS
 N  COST
 L  LIM1
 G  LIM2
 E  MYEQN
COLUMNS
    X1        COST         1.0   LIM1         1.0
    X1        LIM2         1.0
    X2        COST         2.0   LIM1         1.0
    X2        MYEQN       -1.0
    X3        COST        -1.0   MYEQN        1.0
RHS
    RHS       COST        -3.5
    RHS       LIM1         4.0   LIM2         1.0
    RHS       MYEQN        7.0
RANGES
    RNG       LIM1         2.5   MYEQN       -3
BOUNDS
 UP BND       X1           4.0
 MI BND       X2
 UP BND       X2           1.0
 FX BND       X3           2.5
ENDATA
""",
    "no_objective_row": """NAME NOOBJ
ROWS
 E R1
 L R2
COLUMNS
 X R1 1 R2 2
 Y R1 3 R2 4
RHS
 RHS R1 5 R2 6
ENDATA
""",
    "qps_quadobj": """NAME QP
ROWS
 N OBJ
 G C1
COLUMNS
 X OBJ 1 C1 1
 Y OBJ -2 C1 1
 Z C1 -1
RHS
 RHS C1 1 OBJ 4
BOUNDS
 FR BND Z
 UP BND Y 3
QUADOBJ
 X X 2
 X Y 0.5
 Y Y 1
 Y Z 0
 Z Z 4e-1
ENDATA
""",
    "qps_qmatrix": """NAME QPM
ROWS
 N OBJ
 E C1
COLUMNS
 X OBJ 1 C1 1
 Y C1 1
RHS
 RHS C1 2
QMATRIX
 X X 2
 X Y 1
 Y X 1
 Y Y 3
ENDATA
""",
    "empty": "",
    "rows_only": "NAME R\nROWS\n N OBJ\n E A\n",
}
