"""CSV and model-file I/O (crates/geostat-cli/src/io_utils.rs) on the host.

The reference's own io_utils tests (io_utils.rs:336-460) restated against the
native reader and writer, then parity with the oracle's restatement (Python's
csv module plus the reference's field rules; Rust's f64 Display) on seeded
files with quoting, CRLF, blank lines, a byte-order mark, missing values and
every number form; writer output is compared byte for byte.
"""
import math
import os

import numpy as np
import pytest

import pyoracle as O
import geostat_rs as G
from geostat_rs import io as gio
from geostat_rs.model import Structure, VariogramModel


def _w(path, text):
    with open(path, "w", newline="") as f:
        f.write(text)
    return path


def test_read_happy_path_and_extras(tmp_path):
    # io_utils.rs:336-344, 376-384, 399-412
    p = _w(tmp_path / "points.csv", "x,y,z\n0,0,1.0\n1,0,2.0\n0,1,1.5\n")
    t = gio._read_columns(p, ["x", "y", "z"], "rows")
    np.testing.assert_array_equal(t, [[0, 0, 1.0], [1, 0, 2.0], [0, 1, 1.5]])
    p = _w(tmp_path / "targets.csv", "x,y,sdist\n0,0,0.1\n1,1,0.2\n")
    c, e = gio.read_targets(p, "x", "y", ["sdist"])
    np.testing.assert_array_equal(c, [[0, 0], [1, 1]])
    np.testing.assert_array_equal(e, [[0.1], [0.2]])
    p = _w(tmp_path / "targets3.csv", "x,y,z\n0,0,5\n1,2,3\n")
    np.testing.assert_array_equal(gio.read_targets3(p, "x", "y", "z"), [[0, 0, 5], [1, 2, 3]])


def test_missing_column_lists_available(tmp_path):
    # io_utils.rs:346-355
    p = _w(tmp_path / "bad.csv", "east,north,val\n0,0,1.0\n")
    with pytest.raises(G.InvalidParameter) as e:
        gio._read_columns(p, ["x", "y", "val"], "rows")
    assert "column 'x' not found" in str(e.value) and "east" in str(e.value)


def test_skips_missing_or_non_numeric_rows(tmp_path, capsys):
    # io_utils.rs:357-372, 374-381
    p = _w(tmp_path / "m.csv", "x,y,z\n0,0,1.0\n1,0,\n2,0,NaN\n3,0,na\n4,0,not_a_number\n5,0,2.0\n")
    t = gio._read_columns(p, ["x", "y", "z"], "rows")
    np.testing.assert_array_equal(t[:, 2], [1.0, 2.0])
    assert "skipped 4 rows" in capsys.readouterr().err
    p = _w(tmp_path / "all.csv", "x,y,z\n0,0,\n1,0,na\n")
    with pytest.raises(G.InvalidParameter, match="no valid data rows"):
        gio._read_columns(p, ["x", "y", "z"], "rows")


def test_grid_csv_and_model_json(tmp_path):
    # io_utils.rs:445-459, 414-437
    p = tmp_path / "grid.csv"
    gio.write_grid_csv(p, [0.0, 0.0], [1.0, 1.0], [2, 2], [1.0, 2.0, 3.0, 4.0],
                       [0.1, 0.2, 0.3, 0.4])
    lines = open(p).read().splitlines()
    assert lines[0] == "x,y,prediction,variance" and len(lines) == 5
    assert lines[1:] == ["0.25,0.25,1,0.1", "0.75,0.25,2,0.2", "0.25,0.75,3,0.3",
                         "0.75,0.75,4,0.4"]
    m = VariogramModel(0.1, [Structure("spherical", 0.9, 10.0)])
    gio.write_model(tmp_path / "model.json", m)
    back = gio.read_model(tmp_path / "model.json")
    assert back.nugget == m.nugget and len(back.structures) == 1
    with pytest.raises(OSError, match="cannot open model file"):
        gio.read_model(tmp_path / "does-not-exist.json")
    with pytest.raises(G.IoError, match="cannot open input file"):
        gio._read_columns(tmp_path / "nope.csv", ["x"], "rows")


_TOKENS = ["1", "-2.5", "+3", ".5", "5.", "1e5", "1E-3", "-0", "inf", "-Infinity", "+inf",
           " 7.25 ", "", "na", "NA", "nan", "NaN", "1e", "e5", "0x10", "1_0", "abc", "1.2.3",
           "nan(1)", "--1", "1e400", "-1e-400", "123456789012345678901234567890", "0.1"]


def _random_csv(path, rng, nrows, crlf=False, bom=False):
    cols = ["x", "y", "val", "note", "cov"]
    nl = "\r\n" if crlf else "\n"
    out = ["﻿" if bom else "", ",".join(cols), nl]
    for r in range(nrows):
        fields = []
        for c in cols:
            if c == "note":
                tok = rng.choice(["plain", '"quoted, with comma"', '"a ""b"" c"', ""])
            else:
                if rng.random() < 0.8:
                    tok = repr(float(rng.normal() * 10.0 ** rng.integers(-5, 6)))
                else:
                    tok = str(rng.choice(_TOKENS))
                if rng.random() < 0.1 and "," not in tok and '"' not in tok:
                    tok = '"' + tok + '"'
            fields.append(tok)
        out.append(",".join(fields) + nl)
        if rng.random() < 0.05:
            out.append(nl)  # blank line
    with open(path, "w", newline="", encoding="utf-8") as f:
        f.write("".join(out))


@pytest.mark.parametrize("seed,crlf,bom", [(1, False, False), (2, True, False), (3, False, True)])
def test_reader_matches_oracle(tmp_path, seed, crlf, bom):
    rng = np.random.default_rng(seed)
    p = tmp_path / "r.csv"
    _random_csv(p, rng, 3000, crlf, bom)
    cols = ["x", "y", "val", "cov"]
    ref, skipped = O.csv_read(p, cols)
    for threads in (1, 7):
        got = gio._read_columns(p, cols, "rows", nthreads=threads)
        assert got.shape == ref.shape
        assert np.array_equal(got.view(np.uint64), ref.view(np.uint64))
    assert skipped > 0


def test_unequal_record_is_an_error(tmp_path):
    p = _w(tmp_path / "u.csv", "x,y,z\n0,0,1\n1,2\n")
    with pytest.raises(G.IoError, match="row 3"):
        gio._read_columns(p, ["x", "y", "z"], "rows")


def test_writer_matches_rust_display(tmp_path):
    specials = [0.0, -0.0, 1.0, -1.5, 0.1, 0.1 + 0.2, 1e-7, 1e21, 1e22, 123456789012345678.0,
                5e-324, 2.2250738585072014e-308, 1.7976931348623157e308, math.nan, math.inf,
                -math.inf, 1 / 3, 2.5e-5, 100.0, 1234.5]
    rng = np.random.default_rng(9)
    vals = np.concatenate([specials, rng.normal(size=2000) * 10.0 ** rng.integers(-30, 30, 2000)])
    a, b = vals, vals[::-1].copy()
    p = tmp_path / "w.csv"
    gio.write_csv(p, "a,b", [a, b], nthreads=3)
    text = open(p, newline="").read()
    want = "a,b\n" + "".join(f"{O.rust_display(x)},{O.rust_display(y)}\n" for x, y in zip(a, b))
    assert text == want


def test_large_round_trip_is_bit_exact(tmp_path):
    rng = np.random.default_rng(11)
    n = 300_000
    cols = [rng.uniform(0, 1e4, n), rng.uniform(0, 1e4, n), rng.normal(size=n),
            rng.lognormal(size=n) * 1e-9]
    p = tmp_path / "big.csv"
    gio.write_csv(p, "x,y,prediction,variance", cols)
    back = gio._read_columns(p, ["x", "y", "prediction", "variance"], "rows")
    assert np.array_equal(back.view(np.uint64), np.stack(cols, 1).view(np.uint64))
