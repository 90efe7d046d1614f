"""CSV and model-file input/output (crates/geostat-cli/src/io_utils.rs).

The CSV reader and writer are native (``gs_csv_read`` / ``gs_csv_write`` in
the C ABI, multi-threaded on the host): data points and targets come in with
the reference's column selection and missing-value rules, and estimates go
out in its column layouts with numbers formatted as Rust's ``{}`` prints an
f64, so files round-trip with the geostat CLI's.
"""
from __future__ import annotations

import ctypes as C
import os
import sys
from typing import Optional, Sequence, Tuple

import numpy as np

from . import _abi
from .api import PointSet, _f64, _p
from .errors import InvalidParameter
from .model import VariogramModel


def _read_columns(path, names: Sequence[str], what: str, nthreads: int = 0):
    lib = _abi.load()
    arr = (C.c_char_p * len(names))(*[n.encode() for n in names])
    tab = C.c_void_p()
    _abi.check(lib.gs_csv_read(os.fsencode(str(path)), arr, len(names), int(nthreads),
                               C.byref(tab)))
    try:
        rows, skipped = C.c_int64(), C.c_int64()
        _abi.check(lib.gs_csv_table_info(tab, C.byref(rows), C.byref(skipped)))
        out = np.empty((rows.value, len(names)))
        _abi.check(lib.gs_csv_table_copy(tab, _p(out)))
    finally:
        lib.gs_csv_table_destroy(tab)
    if skipped.value > 0:
        sys.stderr.write(f"warning: skipped {skipped.value} {what} with missing or non-numeric "
                         "entries\n")
    if rows.value == 0:
        raise InvalidParameter(f"no valid {'target' if 'target' in what else 'data'} rows in "
                               f"{path}")
    return out


def read_points_with_extras(path, x_col: str, y_col: str, value_col: str,
                            extra_cols: Sequence[str] = ()) -> Tuple[PointSet, np.ndarray]:
    """io_utils.rs:37-75: points (x, y, value) and the extra numeric columns
    (n x len(extra_cols)) of every row whose requested fields all parse."""
    t = _read_columns(path, [x_col, y_col, value_col, *extra_cols], "rows")
    return PointSet(t[:, :2], t[:, 2]), t[:, 3:]


def read_points(path, x_col: str, y_col: str, value_col: str) -> PointSet:
    """io_utils.rs:77-80."""
    return read_points_with_extras(path, x_col, y_col, value_col)[0]


def read_points3(path, x_col: str, y_col: str, z_col: str, value_col: str) -> PointSet:
    """io_utils.rs:82-104: 3-D points (x, y, z, value)."""
    t = _read_columns(path, [x_col, y_col, z_col, value_col], "rows")
    return PointSet(t[:, :3], t[:, 3])


def read_targets(path, x_col: str, y_col: str,
                 extra_cols: Sequence[str] = ()) -> Tuple[np.ndarray, np.ndarray]:
    """io_utils.rs:159-194: target coordinates (n x 2) and covariate rows."""
    t = _read_columns(path, [x_col, y_col, *extra_cols], "target rows")
    return np.ascontiguousarray(t[:, :2]), np.ascontiguousarray(t[:, 2:])


def read_targets3(path, x_col: str, y_col: str, z_col: str) -> np.ndarray:
    """io_utils.rs:106-114: 3-D targets (n x 3)."""
    return np.ascontiguousarray(_read_columns(path, [x_col, y_col, z_col], "target rows"))


def write_csv(path, header: str, columns: Sequence[np.ndarray], nthreads: int = 0) -> None:
    """``header`` then one row per index of the equally long ``columns``."""
    cols = [_f64(c).reshape(-1) for c in columns]
    n = len(cols[0]) if cols else 0
    if any(len(c) != n for c in cols):
        raise InvalidParameter("columns differ in length")
    ptrs = (C.POINTER(C.c_double) * len(cols))(*[_p(c) for c in cols])
    _abi.check(_abi.load().gs_csv_write(os.fsencode(str(path)), header.encode(), len(cols), ptrs,
                                        n, int(nthreads)))


def write_estimates_csv(path, coords, value, variance) -> None:
    """io_utils.rs:226-238 (``x,y,prediction,variance``)."""
    c = _f64(coords)
    write_csv(path, "x,y,prediction,variance", [c[:, 0], c[:, 1], value, variance])


def write_estimates3_csv(path, coords, value, variance) -> None:
    """io_utils.rs:116-128 (``x,y,z,prediction,variance``)."""
    c = _f64(coords)
    write_csv(path, "x,y,z,prediction,variance", [c[:, 0], c[:, 1], c[:, 2], value, variance])


def grid_centers(bbox_min, bbox_max, ncell) -> np.ndarray:
    """Grid2D::centers (grid.rs:80-96): min + (i + 0.5) * step, x fastest."""
    lo, hi = _f64(bbox_min), _f64(bbox_max)
    nx, ny = int(ncell[0]), int(ncell[1])
    dx, dy = (hi[0] - lo[0]) / nx, (hi[1] - lo[1]) / ny
    x = lo[0] + (np.arange(nx) + 0.5) * dx
    y = lo[1] + (np.arange(ny) + 0.5) * dy
    return np.stack([np.tile(x, ny), np.repeat(y, nx)], 1)


def write_grid_csv(path, bbox_min, bbox_max, ncell, value, variance) -> None:
    """io_utils.rs:216-224 (``x,y,prediction,variance`` at the cell centres)."""
    c = grid_centers(bbox_min, bbox_max, ncell)
    write_csv(path, "x,y,prediction,variance", [c[:, 0], c[:, 1], value, variance])


def write_cv_csv(path, data: PointSet, cv) -> None:
    """io_utils.rs:254-272 (``x,y,observed,predicted,variance,residual``)."""
    c = data.coords
    pred, obs = _f64(cv.predicted), _f64(cv.observed)
    write_csv(path, "x,y,observed,predicted,variance,residual",
              [c[:, 0], c[:, 1], obs, pred, cv.variance, pred - obs])


def read_model(path) -> VariogramModel:
    """io_utils.rs:274-282: a serde-JSON model, re-validated."""
    try:
        with open(path) as f:
            text = f.read()
    except OSError as e:
        raise OSError(f"cannot open model file {path}: {e}") from e
    return VariogramModel.from_json(text)


def write_model(path, model: VariogramModel) -> None:
    """io_utils.rs:284-290."""
    with open(path, "w") as f:
        f.write(model.to_json())
