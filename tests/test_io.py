"""CPU: MPS / warmup CSV readers and the File<ii> writer of the C library."""
from __future__ import annotations

import math
import os
from pathlib import Path

import numpy as np
import pytest

from conftest import GOLDEN



def test_read_golden_mps(native, pkg, golden):
    m = pkg.read_mps(GOLDEN / "small.mps")
    assert m.n_rxns == int(golden["n_rxns"]) and m.n_mets == int(golden["n_mets"])
    assert np.array_equal(m.lb, golden["lb"]) and np.array_equal(m.ub, golden["ub"])
    got = {(int(r), int(c)): v for r, c, v in zip(m.row, m.col, m.val)}
    want = {(int(r), int(c)): v for r, c, v in zip(golden["row"], golden["col"], golden["val"])}
    assert got == want


def _independent_mps_parse(path):
    """Column-position-free restatement used to cross-check the C reader."""
    rows, cols, obj = {}, {}, None
    trip, lb, ub = [], {}, {}
    sec = None
    for line in Path(path).read_text().splitlines():
        if not line.strip() or line.startswith("*"):
            continue
        if not line[0].isspace():
            sec = line.split()[0]
            continue
        t = line.split()
        if sec == "ROWS":
            if t[0] == "N" and obj is None:
                obj = t[1]
            else:
                rows[t[1]] = len(rows)
        elif sec == "COLUMNS":
            if t[0] not in cols:
                cols[t[0]] = len(cols)
                lb[t[0]], ub[t[0]] = 0.0, math.inf
            for k in range(1, len(t) - 1, 2):
                if t[k] != obj:
                    trip.append((rows[t[k]], cols[t[0]], float(t[k + 1])))
        elif sec == "BOUNDS":
            typ, name, v = t[0], t[2], float(t[3]) if len(t) > 3 else None
            if typ == "UP":
                ub[name] = v
                if v < 0 and lb[name] == 0:
                    lb[name] = -math.inf
            elif typ == "LO":
                lb[name] = v
            elif typ == "FX":
                lb[name] = ub[name] = v
    order = sorted(cols, key=cols.get)
    return len(rows), len(cols), trip, np.array([lb[c] for c in order]), np.array([ub[c] for c in order])


def test_read_reference_putida_model(native, pkg, putida_files):
    """The reference's own fixture model (VFWarmup/lib/P_Putida.mps): 911 rows, 1060 columns."""
    mps, _ = putida_files
    m = pkg.read_mps(mps)
    nm, nr, trip, lb, ub = _independent_mps_parse(mps)
    assert (m.n_mets, m.n_rxns) == (nm, nr) == (911, 1060)
    assert np.array_equal(m.lb, lb) and np.array_equal(m.ub, ub)
    got = sorted(zip(m.row.tolist(), m.col.tolist(), m.val.tolist()))
    assert got == sorted(trip)
    assert (m.val != np.round(m.val)).sum() > 0  # non-integer coefficients


def test_read_reference_form_warmup_csv(native, pkg, putida_files):
    """2n %f-rounded warmup points of P_Putida: every value has at most six decimals, and the
    rounding leaves S w non-zero, as the reference's input does."""
    mps, csv = putida_files
    m = pkg.read_mps(mps)
    w = pkg.read_warmup_csv(csv, m.n_rxns)
    assert w.shape == (1060, 2120)
    assert np.abs(np.round(w * 1e6) - w * 1e6).max() < 1e-3 * np.abs(w).max()
    assert (w >= m.lb[:, None]).all() and (w <= m.ub[:, None]).all()
    r = np.abs(m.dense() @ w).max()
    assert 1e-9 < r < 1e-4


def _write(tmp_path, name, text):
    p = tmp_path / name
    p.write_text(text)
    return p


MPS_BOUNDS = """NAME          T
ROWS
 N  COST
 E  R1
 E  R2
COLUMNS
    A         R1        1            R2        -2
    B         R1        -1
    C         R2        1            COST      3
    D         R1        0.5
    E         R2        -0.25
    F         R1        1
RHS
    RHS       R1        7
BOUNDS
 UP BND       A         5
 LO BND       B         -3
 UP BND       B         4
 FR BND       C
 MI BND       D
 UP BND       D         -1
 FX BND       E         2.5
 UP BND       F         -2
ENDATA
"""


def test_mps_bound_types(native, pkg, tmp_path):
    m = pkg.read_mps(_write(tmp_path, "b.mps", MPS_BOUNDS))
    assert (m.n_mets, m.n_rxns, int(m.row.size)) == (2, 6, 7)
    inf = math.inf
    assert m.lb.tolist() == [0.0, -3.0, -inf, -inf, 2.5, -inf]
    assert m.ub.tolist() == [5.0, 4.0, inf, -1.0, 2.5, -2.0]


@pytest.mark.parametrize("text", [
    "ROWS\n E  R1\nCOLUMNS\n    A  R9  1\nENDATA\n",             # unknown row
    "ROWS\n E  R1\nCOLUMNS\n    A  R1  x\nENDATA\n",             # bad number
    "ROWS\n E  R1\nCOLUMNS\n    A  R1  1\n",                     # no ENDATA
    "ROWS\n Q  R1\nENDATA\n",                                   # bad row type
    "ROWS\n E  R1\nCOLUMNS\n    A  R1  1\nBOUNDS\n UP B Z 1\nENDATA\n",  # bound on unknown column
    "BOGUS\nENDATA\n",
])
def test_mps_malformed(native, pkg, tmp_path, text):
    with pytest.raises(pkg.AchrError) as e:
        pkg.read_mps(_write(tmp_path, "bad.mps", text))
    assert e.value.status == 5


def test_mps_missing_file(native, pkg, tmp_path):
    with pytest.raises(pkg.AchrError) as e:
        pkg.read_mps(tmp_path / "nope.mps")
    assert e.value.status == 4


def test_read_golden_warmup_csv(native, pkg, golden):
    w = pkg.read_warmup_csv(GOLDEN / "small_warmup.csv", int(golden["n_rxns"]))
    assert np.array_equal(w, golden["warmup"])


def test_csv_strtok_semantics(native, pkg, tmp_path):
    # runs of commas collapse (strtok), a trailing comma adds nothing, CRLF is fine
    p = _write(tmp_path, "w.csv", "1.5,,2,3,\r\n-1,0.25,4e2\n\n")
    w = pkg.read_warmup_csv(p, 2)
    assert w.tolist() == [[1.5, 2.0, 3.0], [-1.0, 0.25, 400.0]]


@pytest.mark.parametrize("text,n", [
    ("1,2,3\n4,5\n", 2),          # ragged
    ("1,2\n3,4\n5,6\n", 2),       # too many lines
    ("1,2\n", 2),                 # too few lines (truncated)
    ("1,nan\n3,4\n", 2),          # NaN
    ("1,abc\n3,4\n", 2),          # not a number
    ("", 1),                      # empty
])
def test_csv_malformed(native, pkg, tmp_path, text, n):
    with pytest.raises(pkg.AchrError) as e:
        pkg.read_warmup_csv(_write(tmp_path, "bad.csv", text), n)
    assert e.value.status == 5


def test_format_f_matches_printf(native, pkg):
    rng = np.random.default_rng(1)
    vals = list(rng.standard_normal(3000) * 10.0 ** rng.integers(-9, 12, 3000))
    vals += [0.0, -0.0, 0.5e-6, 1.5e-6, 2.5e-6, -0.5e-6, 1e-7, -1e-7, 0.0000005, 0.0000015, 1e300, -1e300,
             math.inf, -math.inf, 5e-324, 123456.0000005, 999.9999995, 9007199254740991.0, 9007199254740993.0,
             4503599627370495.5, 0.1, 0.125, 1000.0, -1000.0]
    vals += [k / 2**20 for k in range(-3000, 3000, 7)]
    for v in vals:
        assert pkg.format_f(v) == "%f" % v, v


def test_write_points_csv_bytes(native, pkg, tmp_path):
    rng = np.random.default_rng(2)
    pts = rng.standard_normal((7, 13)) * 300
    pts[0, 0] = -0.0
    pts[1, 2] = 2.5e-7
    for threads in (1, 3):
        p = tmp_path / f"File{threads}"
        pkg.write_points_csv(p, pts, threads=threads)
        want = "".join(",".join("%f" % v for v in row) + "\n" for row in pts)
        assert p.read_text() == want
