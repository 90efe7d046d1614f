"""GeoPackage point layers (crates/geostat-cli/src/gpkg.rs:1-310, 786-860).

A GeoPackage is an SQLite database with the OGC schema; this module reads and
writes 2-D point feature layers through Python's sqlite3 (the same SQLite
engine the reference bundles through rusqlite).  Geometry blobs are
StandardGeoPackageBinary: a ``GP`` header (optional envelope) and WKB, of
which X and Y are taken (ISO Z/M and EWKB SRID forms accepted).  Blobs are
packed and unpacked in bulk with numpy.  Raster (tiled PNG) coverages are not
handled here.
"""
from __future__ import annotations

import os
import sqlite3
import struct
from dataclasses import dataclass
from typing import List, Optional, Sequence, Tuple

import numpy as np

from .errors import IoError

_PT = np.dtype([("magic", "S2"), ("version", "u1"), ("flags", "u1"), ("srs", "<i4"),
                ("order", "u1"), ("type", "<u4"), ("x", "<f8"), ("y", "<f8")])  # 29 bytes


@dataclass
class LayerInfo:
    """gpkg.rs:20-32."""
    name: str
    geometry_column: str
    geometry_type: str
    srs_id: int
    n_features: int


def quote_ident(ident: str) -> str:
    """gpkg.rs:155-158: a double-quoted SQL identifier."""
    return '"' + ident.replace('"', '""') + '"'


def _open(path) -> sqlite3.Connection:
    if not os.path.exists(path):
        raise IoError(f"opening GeoPackage {path}: no such file")
    try:
        return sqlite3.connect(f"file:{os.fspath(path)}?mode=ro", uri=True)
    except sqlite3.Error as e:
        raise IoError(f"opening GeoPackage {path}: {e}") from e


def list_feature_layers(path) -> List[LayerInfo]:
    """gpkg.rs:40-89: feature layers from gpkg_contents and
    gpkg_geometry_columns, by table name."""
    con = _open(path)
    try:
        has = con.execute("SELECT 1 FROM sqlite_master WHERE type='table' AND "
                          "name='gpkg_geometry_columns'").fetchone()
        if not has:
            return []
        try:
            rows = con.execute(
                "SELECT c.table_name, g.column_name, g.geometry_type_name, c.srs_id "
                "FROM gpkg_contents c JOIN gpkg_geometry_columns g ON c.table_name = "
                "g.table_name WHERE c.data_type = 'features' ORDER BY c.table_name").fetchall()
        except sqlite3.Error as e:
            raise IoError(f"querying gpkg_contents (is this a GeoPackage?): {e}") from e
        out = []
        for name, gcol, gtype, srs in rows:
            try:
                nf = con.execute(f"SELECT COUNT(*) FROM {quote_ident(name)}").fetchone()[0]
            except sqlite3.Error:
                nf = -1
            out.append(LayerInfo(name, gcol, gtype, int(srs), int(nf)))
        return out
    finally:
        con.close()


def decode_point(blob: bytes) -> Tuple[float, float]:
    """gpkg.rs:809-860: (x, y) of a GeoPackageBinary point."""
    b = bytes(blob)
    if len(b) < 8 or b[:2] != b"GP":
        raise IoError("not a GeoPackage geometry blob")
    flags = b[3]
    if (flags >> 4) & 1:
        raise IoError("empty geometry")
    code = (flags >> 1) & 7
    env = {0: 0, 1: 32, 2: 48, 3: 48, 4: 64}.get(code)
    if env is None:
        raise IoError(f"invalid GPB envelope code {code}")
    wkb = b[8 + env:]
    if len(wkb) < 21:
        raise IoError("WKB too short for a point")
    le = wkb[0] == 1
    raw = struct.unpack("<I" if le else ">I", wkb[1:5])[0]
    base = (raw & 0x1FFFFFFF) % 1000
    if base != 1:
        raise IoError(f"geometry is not a POINT (WKB base type {base})")
    start = 9 if raw & 0x20000000 else 5
    if len(wkb) < start + 16:
        raise IoError("WKB too short for a point")
    return struct.unpack("<dd" if le else ">dd", wkb[start:start + 16])


def _decode_many(blobs: Sequence[bytes]) -> np.ndarray:
    # the writer's own form (29-byte little-endian blobs) in bulk, any other
    # blob through decode_point
    out = np.empty((len(blobs), 2))
    fast = [i for i, b in enumerate(blobs) if len(b) == 29 and b[:4] == b"GP\x00\x01"
            and b[8] == 1 and b[9:13] == b"\x01\x00\x00\x00"]
    if fast:
        arr = np.frombuffer(b"".join(blobs[i] for i in fast), dtype=_PT)
        out[fast, 0], out[fast, 1] = arr["x"], arr["y"]
    rest = np.setdiff1d(np.arange(len(blobs)), fast, assume_unique=True)
    for i in rest:
        out[i] = decode_point(blobs[i])
    return out


def read_points_arrays(path, layer: Optional[str], value_col: str):
    """gpkg.rs:91-153: (coords n x 2, values) of a point layer; rows with a
    NULL geometry or value are skipped."""
    layers = list_feature_layers(path)
    if not layers:
        raise IoError(f"no vector feature layers found in {path}")
    if layer is not None:
        info = next((l for l in layers if l.name == layer), None)
        if info is None:
            raise IoError(f"layer '{layer}' not found in {path}")
    else:
        if len(layers) > 1:
            raise IoError(f"{path} has multiple layers; choose one with --layer (available: "
                          f"{', '.join(l.name for l in layers)})")
        info = layers[0]
    if "POINT" not in info.geometry_type.upper():
        raise IoError(f"layer '{info.name}' is {info.geometry_type} -- only point layers are "
                      "supported")
    con = _open(path)
    try:
        try:
            rows = con.execute(f"SELECT {quote_ident(info.geometry_column)}, "
                               f"{quote_ident(value_col)} FROM {quote_ident(info.name)}").fetchall()
        except sqlite3.Error as e:
            raise IoError(f"reading column '{value_col}' from layer '{info.name}': {e}") from e
    finally:
        con.close()
    rows = [(g, v) for g, v in rows if g is not None and v is not None]
    for _, v in rows:
        # rusqlite's f64 accepts INTEGER and REAL values only (an unknown
        # quoted column name reads back as its own TEXT in SQLite)
        if isinstance(v, (str, bytes)) or not isinstance(v, (int, float)):
            raise IoError(f"reading column '{value_col}' from layer '{info.name}': invalid "
                          f"column type {type(v).__name__}")
    if not rows:
        raise IoError(f"layer '{info.name}' yielded no usable point/value rows")
    coords = _decode_many([bytes(g) for g, _ in rows])
    return coords, np.array([float(v) for _, v in rows])


def read_points(path, layer: Optional[str], value_col: str):
    """gpkg.rs:91-153 as a :class:`PointSet`."""
    from .api import PointSet
    c, v = read_points_arrays(path, layer, value_col)
    return PointSet(c, v)


def encode_points(coords, srs_id: int) -> List[bytes]:
    """gpkg.rs:161-175 encode_point for every row of ``coords``."""
    c = np.asarray(coords, dtype=np.float64).reshape(-1, 2)
    arr = np.zeros(len(c), dtype=_PT)
    arr["magic"], arr["version"], arr["flags"], arr["srs"] = b"GP", 0, 1, srs_id
    arr["order"], arr["type"], arr["x"], arr["y"] = 1, 1, c[:, 0], c[:, 1]
    raw = arr.tobytes()
    return [raw[i * 29:(i + 1) * 29] for i in range(len(c))]


def write_points(path, layer: str, srs_id: int, coords, columns: Sequence[Tuple[str, object]]):
    """gpkg.rs:183-310: a new GeoPackage (replacing the file) with one point
    feature layer and a REAL attribute column per (name, values)."""
    c = np.asarray(coords, dtype=np.float64).reshape(-1, 2)
    cols = [(name, np.asarray(v, dtype=np.float64)) for name, v in columns]
    for name, v in cols:
        if len(v) != len(c):
            raise IoError(f"column '{name}' has {len(v)} values but there are {len(c)} points")
    if os.path.exists(path):
        os.remove(path)
    con = sqlite3.connect(os.fspath(path))
    try:
        con.execute(f"PRAGMA application_id = {0x47504B47}")
        con.execute("PRAGMA user_version = 10300")
        con.executescript(
            "CREATE TABLE gpkg_spatial_ref_sys (srs_name TEXT NOT NULL, srs_id INTEGER PRIMARY "
            "KEY, organization TEXT NOT NULL, organization_coordsys_id INTEGER NOT NULL, "
            "definition TEXT NOT NULL, description TEXT);"
            "CREATE TABLE gpkg_contents (table_name TEXT NOT NULL PRIMARY KEY, data_type TEXT "
            "NOT NULL, identifier TEXT UNIQUE, description TEXT DEFAULT '', last_change TEXT NOT "
            "NULL DEFAULT (strftime('%Y-%m-%dT%H:%M:%fZ','now')), min_x DOUBLE, min_y DOUBLE, "
            "max_x DOUBLE, max_y DOUBLE, srs_id INTEGER);"
            "CREATE TABLE gpkg_geometry_columns (table_name TEXT NOT NULL, column_name TEXT NOT "
            "NULL, geometry_type_name TEXT NOT NULL, srs_id INTEGER NOT NULL, z TINYINT NOT "
            "NULL, m TINYINT NOT NULL, CONSTRAINT pk_geom_cols PRIMARY KEY (table_name, "
            "column_name));")
        wgs84 = ('GEOGCS["WGS 84",DATUM["WGS_1984",SPHEROID["WGS 84",6378137,298.257223563]],'
                 'PRIMEM["Greenwich",0],UNIT["degree",0.0174532925199433]]')
        con.executemany("INSERT INTO gpkg_spatial_ref_sys VALUES (?, ?, ?, ?, ?, NULL)",
                        [("Undefined cartesian SRS", -1, "NONE", -1, "undefined"),
                         ("Undefined geographic SRS", 0, "NONE", 0, "undefined"),
                         ("WGS 84 geodetic", 4326, "EPSG", 4326, wgs84)])
        if srs_id not in (-1, 0, 4326):
            con.execute("INSERT INTO gpkg_spatial_ref_sys VALUES (?, ?, 'EPSG', ?, 'undefined', "
                        "NULL)", (f"SRS {srs_id}", srs_id, srs_id))
        attr = "".join(f", {quote_ident(n)} REAL" for n, _ in cols)
        con.execute(f"CREATE TABLE {quote_ident(layer)} (fid INTEGER PRIMARY KEY AUTOINCREMENT, "
                    f"geom BLOB{attr})")
        bounds = ((float(c[:, 0].min()), float(c[:, 1].min()), float(c[:, 0].max()),
                   float(c[:, 1].max())) if len(c) else
                  (float("inf"), float("inf"), float("-inf"), float("-inf")))
        con.execute("INSERT INTO gpkg_contents (table_name, data_type, identifier, min_x, min_y, "
                    "max_x, max_y, srs_id) VALUES (?, 'features', ?, ?, ?, ?, ?, ?)",
                    (layer, layer, *bounds, srs_id))
        con.execute("INSERT INTO gpkg_geometry_columns VALUES (?, 'geom', 'POINT', ?, 0, 0)",
                    (layer, srs_id))
        names = "".join(f", {quote_ident(n)}" for n, _ in cols)
        marks = "".join(", ?" for _ in cols)
        blobs = encode_points(c, srs_id)
        vals = [v.tolist() for _, v in cols]
        con.executemany(f"INSERT INTO {quote_ident(layer)} (geom{names}) VALUES (?{marks})",
                        ((blobs[i], *[v[i] for v in vals]) for i in range(len(c))))
        con.commit()
    finally:
        con.close()
