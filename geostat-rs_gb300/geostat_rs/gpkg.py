"""GeoPackage point layers and rasters (crates/geostat-cli/src/gpkg.rs).

A GeoPackage is an SQLite database with the OGC schema; this module reads and
writes 2-D point feature layers and single-band 2D Gridded Coverage rasters
through Python's sqlite3 (the same SQLite engine the reference bundles
through rusqlite).  Geometry blobs are StandardGeoPackageBinary: a ``GP``
header (optional envelope) and WKB, of which X and Y are taken (ISO Z/M and
EWKB SRID forms accepted); they are packed and unpacked in bulk with numpy.
"""
from __future__ import annotations

import math
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


# --------------------------------------------------------------- rasters ---
# gpkg.rs:314-785: a kriged grid as a single-band OGC 2D Gridded Coverage --
# one 16-bit grayscale PNG tile with the linear map value = pixel * scale +
# offset, pixel 0 = no data -- and its reader.  PNG (ISO/IEC 15948) is
# written with filter type 0 and zlib; the reader undoes all five filter
# types of non-interlaced 16-bit grayscale images.

_PNG_SIG = b"\x89PNG\r\n\x1a\n"


def _png_chunk(kind: bytes, data: bytes) -> bytes:
    import zlib
    return struct.pack(">I", len(data)) + kind + data + struct.pack(
        ">I", zlib.crc32(kind + data) & 0xFFFFFFFF)


def encode_png_u16(pixels) -> bytes:
    """A 16-bit grayscale PNG of the (height, width) array ``pixels``."""
    import zlib
    px = np.asarray(pixels, dtype=">u2")
    h, w = px.shape
    raw = np.zeros((h, 1 + 2 * w), dtype=np.uint8)  # filter byte 0 per row
    raw[:, 1:] = px.view(np.uint8).reshape(h, 2 * w)
    ihdr = struct.pack(">IIBBBBB", w, h, 16, 0, 0, 0, 0)
    return (_PNG_SIG + _png_chunk(b"IHDR", ihdr) +
            _png_chunk(b"IDAT", zlib.compress(raw.tobytes(), 6)) + _png_chunk(b"IEND", b""))


def decode_png_u16(blob: bytes, tw: int, th: int) -> np.ndarray:
    """gpkg.rs:757-784: a 16-bit grayscale tile of tw x th pixels (row-major)."""
    import zlib
    b = bytes(blob)
    if b[:8] != _PNG_SIG:
        raise IoError("PNG header: not a PNG")
    pos, ihdr, idat = 8, None, []
    while pos + 8 <= len(b):
        n, kind = struct.unpack(">I4s", b[pos:pos + 8])
        data = b[pos + 8:pos + 8 + n]
        if len(data) != n:
            raise IoError("PNG data: truncated chunk")
        if kind == b"IHDR":
            ihdr = struct.unpack(">IIBBBBB", data)
        elif kind == b"IDAT":
            idat.append(data)
        elif kind == b"IEND":
            break
        pos += 12 + n
    if ihdr is None:
        raise IoError("PNG header: no IHDR")
    w, h, depth, color, _, _, interlace = ihdr
    if depth != 16 or color != 0:
        raise IoError(f"tile is {depth}-bit colour type {color}; expected 16-bit grayscale")
    if interlace != 0:
        raise IoError("PNG data: interlaced tiles are not supported")
    if w != tw or h != th:
        raise IoError(f"tile is {w}x{h} but the tile matrix declares {tw}x{th}")
    try:
        raw = zlib.decompress(b"".join(idat))
    except zlib.error as e:
        raise IoError(f"PNG data: {e}") from e
    stride, bpp = 2 * w, 2
    if len(raw) < h * (1 + stride):
        raise IoError("PNG data: short image data")
    out = np.zeros((h, stride), dtype=np.int64)
    prev = np.zeros(stride, dtype=np.int64)
    for r in range(h):
        ft = raw[r * (1 + stride)]
        line = np.frombuffer(raw, dtype=np.uint8, count=stride, offset=r * (1 + stride) + 1)
        line = line.astype(np.int64)
        if ft == 0:
            cur = line
        elif ft == 2:
            cur = (line + prev) & 0xFF
        elif ft in (1, 3, 4):
            cur = np.zeros(stride, dtype=np.int64)
            for x in range(stride):
                a = cur[x - bpp] if x >= bpp else 0
                up = prev[x]
                if ft == 1:
                    pred = a
                elif ft == 3:
                    pred = (a + up) >> 1
                else:
                    c = prev[x - bpp] if x >= bpp else 0
                    p = a + up - c
                    pa, pb, pc = abs(p - a), abs(p - up), abs(p - c)
                    pred = a if pa <= pb and pa <= pc else (up if pb <= pc else c)
                cur[x] = (line[x] + pred) & 0xFF
        else:
            raise IoError(f"PNG data: unknown filter type {ft}")
        out[r] = cur
        prev = cur
    by = out.astype(np.uint8)
    return (by[:, 0::2].astype(np.uint16) << 8 | by[:, 1::2].astype(np.uint16)).reshape(h, w)


def encode_raster(nx: int, ny: int, values):
    """gpkg.rs:324-375: (png, scale, offset, min, max, mean, std_dev).  Finite
    values map linearly onto pixels 1..65535 (min -> 1, max -> 65535,
    rounded half away from zero), non-finite ones to 0; image rows run north
    to south."""
    v = np.asarray(values, dtype=np.float64).reshape(ny, nx)
    fin = v[np.isfinite(v)]
    if fin.size == 0:
        raise IoError("raster has no finite values")
    vmin, vmax = float(fin.min()), float(fin.max())
    mean = float(np.cumsum(fin)[-1] / fin.size)
    std = math.sqrt(float(np.cumsum((fin - mean) ** 2)[-1] / fin.size))
    span = max(vmax - vmin, 2.2250738585072014e-308)
    scale = span / 65534.0
    offset = vmin - scale
    with np.errstate(invalid="ignore"):
        px = np.clip(np.floor(1.0 + (v - vmin) / span * 65534.0 + 0.5), 1.0, 65535.0)
    px = np.where(np.isfinite(v), px, 0.0).astype(np.uint16)
    return encode_png_u16(px[::-1]), scale, offset, vmin, vmax, mean, std


def write_raster(path, layer: str, srs_id: int, nx: int, ny: int, bbox, values) -> None:
    """gpkg.rs:384-518: a new GeoPackage holding the grid (values in grid
    order, iy * nx + ix, y increasing; bbox = [min_x, min_y, max_x, max_y])
    as one 2D Gridded Coverage tile."""
    vals = np.asarray(values, dtype=np.float64).reshape(-1)
    if len(vals) != nx * ny:
        raise IoError(f"{len(vals)} values for an {nx}x{ny} grid")
    png, scale, offset, vmin, vmax, mean, std = encode_raster(nx, ny, vals)
    min_x, min_y, max_x, max_y = (float(b) for b in bbox)
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
            "CREATE TABLE gpkg_tile_matrix_set (table_name TEXT NOT NULL PRIMARY KEY, srs_id "
            "INTEGER NOT NULL, min_x DOUBLE NOT NULL, min_y DOUBLE NOT NULL, max_x DOUBLE NOT "
            "NULL, max_y DOUBLE NOT NULL);"
            "CREATE TABLE gpkg_tile_matrix (table_name TEXT NOT NULL, zoom_level INTEGER NOT "
            "NULL, matrix_width INTEGER NOT NULL, matrix_height INTEGER NOT NULL, tile_width "
            "INTEGER NOT NULL, tile_height INTEGER NOT NULL, pixel_x_size DOUBLE NOT NULL, "
            "pixel_y_size DOUBLE NOT NULL, CONSTRAINT pk_ttm PRIMARY KEY (table_name, "
            "zoom_level));"
            "CREATE TABLE gpkg_extensions (table_name TEXT, column_name TEXT, extension_name "
            "TEXT NOT NULL, definition TEXT NOT NULL, scope TEXT NOT NULL, CONSTRAINT ge_tce "
            "UNIQUE (table_name, column_name, extension_name));"
            "CREATE TABLE gpkg_2d_gridded_coverage_ancillary (id INTEGER PRIMARY KEY "
            "AUTOINCREMENT, tile_matrix_set_name TEXT NOT NULL UNIQUE, datatype TEXT NOT NULL "
            "DEFAULT 'integer', scale REAL NOT NULL DEFAULT 1.0, offset REAL NOT NULL DEFAULT "
            "0.0, precision REAL DEFAULT 1.0, data_null REAL, grid_cell_encoding TEXT DEFAULT "
            "'grid-value-is-center', uom TEXT, field_name TEXT DEFAULT 'Height', "
            "quantity_definition TEXT DEFAULT 'Height');"
            "CREATE TABLE gpkg_2d_gridded_tile_ancillary (id INTEGER PRIMARY KEY AUTOINCREMENT, "
            "tpudt_name TEXT NOT NULL, tpudt_id INTEGER NOT NULL, scale REAL NOT NULL DEFAULT "
            "1.0, offset REAL NOT NULL DEFAULT 0.0, min REAL, max REAL, mean REAL, std_dev REAL, "
            "UNIQUE (tpudt_name, tpudt_id));")
        con.executemany("INSERT INTO gpkg_spatial_ref_sys VALUES (?, ?, ?, ?, 'undefined', NULL)",
                        [("Undefined cartesian SRS", -1, "NONE", -1),
                         ("Undefined geographic SRS", 0, "NONE", 0),
                         ("WGS 84 geodetic", 4326, "EPSG", 4326)])
        if srs_id not in (-1, 0, 4326):
            con.execute("INSERT INTO gpkg_spatial_ref_sys VALUES (?, ?, 'EPSG', ?, 'undefined', "
                        "NULL)", (f"SRS {srs_id}", srs_id, srs_id))
        q = quote_ident(layer)
        con.execute(f"CREATE TABLE {q} (id INTEGER PRIMARY KEY AUTOINCREMENT, zoom_level INTEGER "
                    "NOT NULL, tile_column INTEGER NOT NULL, tile_row INTEGER NOT NULL, tile_data "
                    "BLOB NOT NULL, UNIQUE (zoom_level, tile_column, tile_row))")
        con.execute("INSERT INTO gpkg_contents (table_name, data_type, identifier, min_x, min_y, "
                    "max_x, max_y, srs_id) VALUES (?, '2d-gridded-coverage', ?, ?, ?, ?, ?, ?)",
                    (layer, layer, min_x, min_y, max_x, max_y, srs_id))
        con.execute("INSERT INTO gpkg_tile_matrix_set VALUES (?, ?, ?, ?, ?, ?)",
                    (layer, srs_id, min_x, min_y, max_x, max_y))
        con.execute("INSERT INTO gpkg_tile_matrix VALUES (?, 0, 1, 1, ?, ?, ?, ?)",
                    (layer, nx, ny, (max_x - min_x) / nx, (max_y - min_y) / ny))
        d = "http://docs.opengeospatial.org/is/17-066r1/17-066r1.html"
        con.executemany("INSERT INTO gpkg_extensions VALUES (?, ?, 'gpkg_2d_gridded_coverage', "
                        "?, 'read-write')",
                        [("gpkg_2d_gridded_coverage_ancillary", None, d),
                         ("gpkg_2d_gridded_tile_ancillary", None, d), (layer, "tile_data", d)])
        con.execute("INSERT INTO gpkg_2d_gridded_coverage_ancillary (tile_matrix_set_name, "
                    "datatype, scale, offset, precision, data_null, field_name, "
                    "quantity_definition) VALUES (?, 'integer', ?, ?, ?, 0.0, 'prediction', "
                    "'prediction')", (layer, scale, offset, scale))
        cur = con.execute(f"INSERT INTO {q} (zoom_level, tile_column, tile_row, tile_data) "
                          "VALUES (0, 0, 0, ?)", (png,))
        con.execute("INSERT INTO gpkg_2d_gridded_tile_ancillary (tpudt_name, tpudt_id, scale, "
                    "offset, min, max, mean, std_dev) VALUES (?, ?, 1.0, 0.0, ?, ?, ?, ?)",
                    (layer, cur.lastrowid, vmin, vmax, mean, std))
        con.commit()
    finally:
        con.close()


@dataclass
class RasterGrid:
    """gpkg.rs:523-583: a coverage read back, values in grid order (NaN =
    no data)."""
    name: str
    srs_id: int
    nx: int
    ny: int
    bbox: Tuple[float, float, float, float]
    values: np.ndarray

    def sample(self, x: float, y: float) -> Optional[float]:
        """Nearest cell's value at (x, y); None outside the extent or on no
        data."""
        if self.nx == 0 or self.ny == 0:
            return None
        min_x, min_y, max_x, max_y = self.bbox
        if x < min_x or x > max_x or y < min_y or y > max_y:
            return None
        ix = min(int((x - min_x) / ((max_x - min_x) / self.nx)), self.nx - 1)
        iy = min(int((y - min_y) / ((max_y - min_y) / self.ny)), self.ny - 1)
        v = float(self.values[iy * self.nx + ix])
        return v if math.isfinite(v) else None


def list_raster_layers(path) -> List[str]:
    """gpkg.rs:586-599."""
    con = _open(path)
    try:
        try:
            rows = con.execute("SELECT table_name FROM gpkg_contents WHERE data_type = "
                               "'2d-gridded-coverage' ORDER BY table_name").fetchall()
        except sqlite3.Error as e:
            raise IoError(f"querying gpkg_contents (is this a GeoPackage?): {e}") from e
        return [r[0] for r in rows]
    finally:
        con.close()


_MAX_TILE_DIM = 1 << 16
_MAX_RASTER_CELLS = 1 << 28


def read_raster(path, layer: Optional[str] = None) -> RasterGrid:
    """gpkg.rs:609-755: an integer (PNG-tile) coverage at its finest zoom
    level, tiles mosaicked, rows flipped into grid order; tile-matrix
    dimensions outside [1, 65536] or more than 2^28 cells are rejected."""
    names = list_raster_layers(path)
    if not names:
        raise IoError(f"no 2d-gridded-coverage layers found in {path}")
    if layer is not None:
        if layer not in names:
            raise IoError(f"raster layer '{layer}' not found in {path}")
        name = layer
    else:
        if len(names) > 1:
            raise IoError(f"{path} has multiple raster layers; choose one with --layer "
                          f"(available: {', '.join(names)})")
        name = names[0]
    con = _open(path)
    try:
        row = con.execute("SELECT datatype, scale, offset, data_null FROM "
                          "gpkg_2d_gridded_coverage_ancillary WHERE tile_matrix_set_name = ?",
                          (name,)).fetchone()
        if row is None:
            raise IoError(f"reading coverage ancillary for '{name}'")
        datatype, scale, offset, data_null = row
        if datatype != "integer":
            raise IoError(f"coverage '{name}' has datatype '{datatype}'; only 'integer' (PNG) "
                          "is supported")
        null_px = 0.0 if data_null is None else float(data_null)
        srs, min_x, min_y, max_x, max_y = con.execute(
            "SELECT srs_id, min_x, min_y, max_x, max_y FROM gpkg_tile_matrix_set WHERE "
            "table_name = ?", (name,)).fetchone()
        zoom, mw, mh, tw, th = con.execute(
            "SELECT zoom_level, matrix_width, matrix_height, tile_width, tile_height FROM "
            "gpkg_tile_matrix WHERE table_name = ? ORDER BY zoom_level DESC LIMIT 1",
            (name,)).fetchone()
        for label, val in (("matrix_width", mw), ("matrix_height", mh), ("tile_width", tw),
                           ("tile_height", th)):
            if not 1 <= val <= _MAX_TILE_DIM:
                raise IoError(f"coverage '{name}': {label} = {val} is out of the expected range "
                              f"[1, {_MAX_TILE_DIM}]")
        nx, ny = mw * tw, mh * th
        if nx * ny > _MAX_RASTER_CELLS:
            raise IoError(f"coverage '{name}': raster is {nx}x{ny} ({nx * ny} cells), exceeding "
                          f"the {_MAX_RASTER_CELLS}-cell sanity limit")
        img = np.full((ny, nx), np.nan)
        for tcol, trow, blob in con.execute(
                f"SELECT tile_column, tile_row, tile_data FROM {quote_ident(name)} WHERE "
                "zoom_level = ?", (zoom,)):
            px = decode_png_u16(blob, tw, th).astype(np.float64)
            vals = np.where(px == null_px, np.nan, px * scale + offset)
            r0, c0 = trow * th, tcol * tw
            if r0 >= ny or c0 >= nx or r0 < 0 or c0 < 0:
                continue
            r1, c1 = min(r0 + th, ny), min(c0 + tw, nx)
            img[r0:r1, c0:c1] = vals[:r1 - r0, :c1 - c0]
    finally:
        con.close()
    return RasterGrid(name, int(srs), int(nx), int(ny), (min_x, min_y, max_x, max_y),
                      img[::-1].reshape(-1).copy())
