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
