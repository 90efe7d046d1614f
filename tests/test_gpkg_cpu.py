"""GeoPackage point layers (crates/geostat-cli/src/gpkg.rs) on the host: the
reference's decoder and round-trip tests (gpkg.rs:872-918, 1095-1118)."""
import struct

import numpy as np
import pytest

pytest.importorskip("sqlite3")
from geostat_rs import gpkg  # noqa: E402
from geostat_rs.errors import IoError  # noqa: E402


def _gpb_point(x, y):
    return b"GP\x00\x01" + struct.pack("<i", 4326) + b"\x01" + struct.pack("<I", 1) + \
        struct.pack("<dd", x, y)


def test_decoder_known_answers():
    assert gpkg.decode_point(_gpb_point(123.5, -45.25)) == (123.5, -45.25)
    b = b"GP\x00\x03" + struct.pack("<i", 4326) + struct.pack("<4d", 10, 20, 30, 40) + \
        b"\x01" + struct.pack("<I", 1) + struct.pack("<dd", 15.0, 25.0)
    assert gpkg.decode_point(b) == (15.0, 25.0)
    with pytest.raises(IoError):
        gpkg.decode_point(b"not a blob at all")
    e = b"GP\x00\x01" + struct.pack("<i", 4326) + b"\x01" + struct.pack("<I", 1 | 0x20000000) + \
        struct.pack("<i", 4326) + struct.pack("<dd", 123.5, -45.25)
    assert gpkg.decode_point(e) == (123.5, -45.25)
    big = b"GP\x00\x00" + struct.pack(">i", 4326) + b"\x00" + struct.pack(">I", 1001) + \
        struct.pack(">ddd", 1.0, 2.0, 3.0)
    assert gpkg.decode_point(big) == (1.0, 2.0)
    assert gpkg.quote_ident("zinc") == '"zinc"' and gpkg.quote_ident('a"b') == '"a""b"'


def test_write_then_read_round_trips(tmp_path):
    p = tmp_path / "rt.gpkg"
    coords = np.array([[10.0, 20.0], [30.5, 40.25], [-5.0, 0.0]])
    vals = np.array([1.5, 2.5, 3.5])
    gpkg.write_points(p, "kriging", 28992, coords, [("pred", vals)])
    layers = gpkg.list_feature_layers(p)
    assert len(layers) == 1 and layers[0].name == "kriging"
    assert layers[0].geometry_type == "POINT" and layers[0].srs_id == 28992
    assert layers[0].n_features == 3
    c, v = gpkg.read_points_arrays(p, None, "pred")
    assert np.array_equal(c, coords) and np.array_equal(v, vals)


def test_large_layer_and_errors(tmp_path):
    rng = np.random.default_rng(3)
    c = rng.uniform(0, 1e5, (20000, 2))
    pred, var = rng.normal(size=20000), rng.uniform(size=20000)
    var[5] = np.nan
    p = tmp_path / "big.gpkg"
    gpkg.write_points(p, "est", 4326, c, [("prediction", pred), ("variance", var)])
    cc, vv = gpkg.read_points_arrays(p, "est", "prediction")
    assert np.array_equal(cc, c) and np.array_equal(vv, pred)
    # a NaN is stored as NULL by SQLite: that row is skipped on reading
    cv, vv = gpkg.read_points_arrays(p, "est", "variance")
    assert len(vv) == 19999
    with pytest.raises(IoError, match="not found"):
        gpkg.read_points_arrays(p, "nope", "prediction")
    with pytest.raises(IoError):
        gpkg.read_points_arrays(p, "est", "missing_column")
    with pytest.raises(IoError):
        gpkg.read_points_arrays(tmp_path / "absent.gpkg", None, "x")


# ------------------------------------------------------------- rasters -----
def test_encode_raster_reconstructs_values():
    # gpkg.rs:920-953
    nx, ny = 2, 3
    values = [1.0, 2.0, 3.0, 4.0, float("nan"), 6.0]
    png, scale, offset, vmin, vmax, _, _ = gpkg.encode_raster(nx, ny, values)
    assert vmin == 1.0 and vmax == 6.0
    px = gpkg.decode_png_u16(png, nx, ny)
    for r in range(ny):
        iy = ny - 1 - r
        for c in range(nx):
            v = values[iy * nx + c]
            if np.isfinite(v):
                assert abs(px[r, c] * scale + offset - v) <= scale
            else:
                assert px[r, c] == 0


def test_write_raster_builds_gridded_coverage(tmp_path):
    # gpkg.rs:955-994
    import sqlite3
    p = tmp_path / "r.gpkg"
    gpkg.write_raster(p, "kriging", 4326, 4, 3, [0.0, 0.0, 4.0, 3.0], np.arange(12.0))
    con = sqlite3.connect(p)
    assert con.execute("SELECT data_type FROM gpkg_contents WHERE table_name='kriging'"
                       ).fetchone()[0] == "2d-gridded-coverage"
    assert con.execute('SELECT COUNT(*) FROM "kriging"').fetchone()[0] == 1
    assert con.execute("SELECT datatype FROM gpkg_2d_gridded_coverage_ancillary"
                       ).fetchone()[0] == "integer"
    con.close()


def test_raster_write_then_read_round_trips(tmp_path):
    # gpkg.rs:996-1052
    p = tmp_path / "dem.gpkg"
    nx, ny = 5, 4
    values = 2.0 + 0.5 * np.arange(nx * ny)
    values[7] = np.nan
    bbox = [100.0, 200.0, 150.0, 240.0]
    gpkg.write_raster(p, "dem", 32719, nx, ny, bbox, values)
    assert gpkg.list_raster_layers(p) == ["dem"]
    assert gpkg.list_feature_layers(p) == []
    g = gpkg.read_raster(p)
    assert (g.nx, g.ny, g.srs_id) == (nx, ny, 32719) and list(g.bbox) == bbox
    fin = values[np.isfinite(values)]
    step = (fin.max() - fin.min()) / 65534.0
    for i, v in enumerate(values):
        if np.isfinite(v):
            assert abs(g.values[i] - v) <= step + 1e-9
        else:
            assert np.isnan(g.values[i])
    px, py = (bbox[2] - bbox[0]) / nx, (bbox[3] - bbox[1]) / ny
    assert abs(g.sample(bbox[0] + 0.5 * px, bbox[1] + 0.5 * py) - g.values[0]) <= step + 1e-9
    assert g.sample(bbox[0] - 1.0, bbox[1]) is None
    assert g.sample(bbox[0] + 2.5 * px, bbox[1] + 1.5 * py) is None


def test_read_raster_rejects_corrupt_tile_matrix_dimensions(tmp_path):
    # gpkg.rs:1054-1093
    import sqlite3
    p = tmp_path / "c.gpkg"
    gpkg.write_raster(p, "dem", 32719, 3, 3, [0.0, 0.0, 30.0, 30.0], np.arange(9.0))
    for col, bad, good in (("matrix_width", -1, 1), ("tile_width", 2 ** 63 - 1, 3)):
        con = sqlite3.connect(p)
        con.execute(f"UPDATE gpkg_tile_matrix SET {col} = ? WHERE table_name = 'dem'", (bad,))
        con.commit()
        con.close()
        with pytest.raises(IoError):
            gpkg.read_raster(p)
        con = sqlite3.connect(p)
        con.execute(f"UPDATE gpkg_tile_matrix SET {col} = ? WHERE table_name = 'dem'", (good,))
        con.commit()
        con.close()
    assert gpkg.read_raster(p).nx == 3


def _filtered_png(px, filters):
    """A 16-bit grayscale PNG whose rows use the given filter types (PNG
    specification, section 9), to check the decoder's unfiltering."""
    import zlib
    h, w = px.shape
    rows = np.asarray(px, dtype=">u2").view(np.uint8).reshape(h, 2 * w).astype(np.int64)
    out, prev = [], np.zeros(2 * w, dtype=np.int64)
    for r in range(h):
        cur, ft = rows[r], filters[r % len(filters)]
        enc = np.zeros(2 * w, dtype=np.int64)
        for x in range(2 * w):
            a = cur[x - 2] if x >= 2 else 0
            b, c = prev[x], (prev[x - 2] if x >= 2 else 0)
            if ft == 0:
                pred = 0
            elif ft == 1:
                pred = a
            elif ft == 2:
                pred = b
            elif ft == 3:
                pred = (a + b) >> 1
            else:
                p = a + b - c
                pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
                pred = a if pa <= pb and pa <= pc else (b if pb <= pc else c)
            enc[x] = (cur[x] - pred) & 0xFF
        out.append(bytes([ft]) + enc.astype(np.uint8).tobytes())
        prev = cur
    ihdr = struct.pack(">IIBBBBB", w, h, 16, 0, 0, 0, 0)
    return (gpkg._PNG_SIG + gpkg._png_chunk(b"IHDR", ihdr) +
            gpkg._png_chunk(b"IDAT", zlib.compress(b"".join(out))) + gpkg._png_chunk(b"IEND", b""))


def test_png_decoder_undoes_every_filter_type():
    rng = np.random.default_rng(4)
    px = rng.integers(0, 65536, size=(9, 7), dtype=np.uint16)
    for filters in ([0], [1], [2], [3], [4], [0, 1, 2, 3, 4]):
        got = gpkg.decode_png_u16(_filtered_png(px, filters), 7, 9)
        assert np.array_equal(got, px), filters
    with pytest.raises(IoError):
        gpkg.decode_png_u16(_filtered_png(px, [0]), 9, 7)  # wrong declared size
