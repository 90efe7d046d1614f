"""Host-side mirror of geostat-rs's kriging / Vecchia interface over the C ABI.

Two layers:

* ``PointSet`` / ``KrigingConfig`` / ``Kriging`` follow the core Rust API
  (crates/geostat-core/src/data.rs, kriging.rs): ``Kriging.new``,
  ``with_external_drift``, ``with_measurement_error``, ``predict_many``,
  ``predict_many_with_drift``, ``predict_grid``.
* ``krige``, ``krige_grid``, ``krige_3d``, ``vecchia_loglik``,
  ``vecchia_mle``, ``vecchia_krige`` follow the reference's Python binding
  (crates/geostat-python/src/lib.rs) argument for argument, returning the same
  ``(predictions, variances)`` numpy pairs and raising ``ValueError``
  subclasses for ``GeostatError``s.

Every computation runs in libgeostat_gb300.so on the GPU; nothing here
computes estimates.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass
from typing import Optional, Sequence, Tuple

import numpy as np

from . import _abi
from .errors import DimensionMismatch, InvalidParameter
from .model import KIND_CODES, Anisotropy, Structure, VariogramModel

PRECISIONS = {"mixed": _abi.PREC_MIXED, "fp64": _abi.PREC_FP64}


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64))


def _p(a, ct=C.c_double):
    return None if a is None else a.ctypes.data_as(C.POINTER(ct))


def seq_mean(values) -> float:
    """Left-to-right mean, as PointSet::mean (data.rs:344-346) sums."""
    v = _f64(values)
    return float(np.add.accumulate(v)[-1] / len(v))


def model_struct(model: VariogramModel) -> _abi.Model:
    m = _abi.Model()
    m.nugget = float(model.nugget)
    m.n_structures = len(model.structures)
    for i, s in enumerate(model.structures):
        m.s[i].kind = KIND_CODES[s.kind]
        m.s[i].param = float(s.param)
        m.s[i].sill = float(s.sill)
        m.s[i].range = float(s.range)
        if s.anis is not None:
            m.s[i].has_anis = 1
            m.s[i].azimuth_deg = s.anis.azimuth_deg
            m.s[i].ratio = s.anis.ratio
            m.s[i].ratio_z = s.anis.ratio_z
            m.s[i].dip_deg = s.anis.dip_deg
            m.s[i].rake_deg = s.anis.rake_deg
        else:
            m.s[i].ratio = m.s[i].ratio_z = 1.0
    return m


class PointSet:
    """Device-resident ``PointSet<D>`` (data.rs:8-83)."""

    def __init__(self, coords, values):
        coords = _f64(coords)
        if coords.ndim != 2 or coords.shape[1] not in (2, 3):
            raise DimensionMismatch("coords must be an (n, 2) or (n, 3) array")
        values = _f64(values)
        if len(values) != len(coords):
            raise DimensionMismatch(f"{len(coords)} coordinates vs {len(values)} values")
        self.dim = coords.shape[1]
        self.n = len(coords)
        self.coords = coords
        self.values = values
        lib = _abi.load()
        x = _f64(coords[:, 0])
        y = _f64(coords[:, 1])
        z = _f64(coords[:, 2]) if self.dim == 3 else None
        h = C.c_void_p()
        _abi.check(lib.gs_pointset_create(self.dim, self.n, _p(x), _p(y), _p(z), _p(values),
                                          C.byref(h)))
        self._h = h

    @classmethod
    def from_xyz(cls, x, y, values):
        x, y = _f64(x), _f64(y)
        if not (len(x) == len(y) == len(values)):
            raise DimensionMismatch(f"x: {len(x)}, y: {len(y)}, z: {len(values)}")
        return cls(np.stack([x, y], axis=1), values)

    @classmethod
    def from_xyzv(cls, x, y, z, values):
        x, y, z = _f64(x), _f64(y), _f64(z)
        if not (len(x) == len(y) == len(z) == len(values)):
            raise DimensionMismatch(
                f"x: {len(x)}, y: {len(y)}, z: {len(z)}, values: {len(values)}")
        return cls(np.stack([x, y, z], axis=1), values)

    def mean(self) -> float:
        return seq_mean(self.values)

    def duplicate_pair(self):
        i, j = C.c_int64(), C.c_int64()
        if _abi.load().gs_pointset_duplicate_pair(self._h, C.byref(i), C.byref(j)):
            return (i.value, j.value)
        return None

    def close(self):
        if getattr(self, "_h", None):
            _abi.load().gs_pointset_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass
class KrigingConfig:
    """``KrigingConfig`` (kriging.rs:73-115).  ``method`` is one of
    "simple", "ordinary", "universal", "external_drift"."""
    method: str = "ordinary"
    mean: Optional[float] = None      # simple kriging's known mean
    degree: int = 1                   # universal kriging drift degree
    n_vars: int = 0                   # external-drift covariates
    max_neighbors: Optional[int] = None
    search_radius: Optional[float] = None
    min_neighbors: Optional[int] = None
    max_per_octant: Optional[int] = None
    anisotropic_search: Optional[Anisotropy] = None

    def to_struct(self) -> _abi.Kcfg:
        if self.method not in _abi.METHODS:
            raise InvalidParameter(f"unknown kriging method '{self.method}'")
        c = _abi.Kcfg()
        c.method = _abi.METHODS[self.method]
        c.sk_mean = float(self.mean) if self.mean is not None else 0.0
        c.uk_degree = int(self.degree)
        c.ked_nvars = int(self.n_vars)
        c.max_neighbors = -1 if self.max_neighbors is None else int(self.max_neighbors)
        c.min_neighbors = -1 if self.min_neighbors is None else int(self.min_neighbors)
        c.max_per_octant = -1 if self.max_per_octant is None else int(self.max_per_octant)
        c.has_search_radius = 0 if self.search_radius is None else 1
        c.search_radius = float(self.search_radius) if self.search_radius is not None else 0.0
        a = self.anisotropic_search
        if a is not None:
            c.has_anisotropic_search = 1
            c.search_azimuth_deg = a.azimuth_deg
            c.search_ratio = a.ratio
            c.search_ratio_z = a.ratio_z
            c.search_dip_deg = a.dip_deg
            c.search_rake_deg = a.rake_deg
        return c


@dataclass
class KrigingResult:
    value: np.ndarray
    variance: np.ndarray
    lagrange: np.ndarray
    status: np.ndarray


class Kriging:
    """``Kriging<'_, D>`` over a device-resident ``PointSet`` (kriging.rs:138-408)."""

    def __init__(self, data: PointSet, model: VariogramModel, config: KrigingConfig, _ctor=0,
                 _aux=None):
        self.data = data
        self.model = model
        self.config = config
        lib = _abi.load()
        m = model_struct(model)
        cfg = config.to_struct()
        h = C.c_void_p()
        if _ctor == 0:
            rc = lib.gs_kriging_new(data._h, C.byref(m), C.byref(cfg), C.byref(h))
        elif _ctor == 1:
            rc = lib.gs_kriging_with_external_drift(data._h, C.byref(m), C.byref(cfg), _p(_aux),
                                                    C.byref(h))
        else:
            rc = lib.gs_kriging_with_measurement_error(data._h, C.byref(m), C.byref(cfg),
                                                       _p(_aux), C.byref(h))
        _abi.check(rc)
        self._h = h

    @classmethod
    def new(cls, data, model, config=None):
        return cls(data, model, config or KrigingConfig())

    @classmethod
    def with_external_drift(cls, data, model, config, drift_data):
        """``drift_data[i]`` holds the covariates of data point ``i``."""
        if config.method != "external_drift":
            raise InvalidParameter("with_external_drift requires KrigingMethod::ExternalDrift")
        d = _f64(drift_data).reshape(data.n, -1) if len(drift_data) == data.n else None
        if d is None:
            raise DimensionMismatch(f"{len(drift_data)} drift rows vs {data.n} data points")
        if config.n_vars and d.shape[1] != config.n_vars:
            raise DimensionMismatch(
                f"drift rows have {d.shape[1]} values, expected {config.n_vars}")
        return cls(data, model, config, 1, np.ascontiguousarray(d))

    @classmethod
    def with_measurement_error(cls, data, model, config, errors):
        e = _f64(errors)
        if len(e) != data.n:
            raise DimensionMismatch(f"{len(e)} error variances vs {data.n} data points")
        return cls(data, model, config, 2, e)

    def _targets(self, targets):
        t = _f64(targets)
        if t.ndim != 2 or t.shape[1] != self.data.dim:
            raise DimensionMismatch(f"targets must be (nt, {self.data.dim})")
        cols = [_f64(t[:, d]) for d in range(self.data.dim)]
        if self.data.dim == 2:
            cols.append(None)
        return len(t), cols

    def predict_many(self, targets, precision: str = "mixed", full: bool = False,
                     _tdrift=None):
        """Estimates at ``targets`` (nt x D).  Returns ``(value, variance)``,
        or a :class:`KrigingResult` with ``full=True``."""
        nt, (x, y, z) = self._targets(targets)
        v, var = np.empty(nt), np.empty(nt)
        lag = np.empty(nt)
        st = np.empty(nt, dtype=np.uint8)
        rc = _abi.load().gs_kriging_predict_many(self._h, nt, _p(x), _p(y), _p(z), _p(_tdrift),
                                                 _p(v), _p(var), _p(lag), _p(st, C.c_uint8),
                                                 PRECISIONS[precision], None)
        _abi.check(rc)
        if full:
            return KrigingResult(v, var, lag, st)
        return v, var

    def predict_many_with_drift(self, targets, drifts, precision: str = "mixed",
                                full: bool = False):
        """External-drift estimates; ``drifts[i]`` holds target ``i``'s covariates."""
        if len(targets) != len(drifts):
            raise DimensionMismatch(f"{len(targets)} targets vs {len(drifts)} drift rows")
        d = _f64(drifts).reshape(len(targets), -1)
        return self.predict_many(targets, precision, full, _tdrift=np.ascontiguousarray(d))

    def predict_grid(self, bbox_min, bbox_max, ncell, precision: str = "mixed", full=False):
        """``predict_grid`` over Grid2D/Grid3D cell centres (x fastest)."""
        nc = np.ascontiguousarray(ncell, dtype=np.int64)
        total = int(np.prod(nc))
        v, var = np.empty(total), np.empty(total)
        st = np.empty(total, dtype=np.uint8)
        rc = _abi.load().gs_kriging_predict_grid(self._h, _p(_f64(bbox_min)), _p(_f64(bbox_max)),
                                                 _p(nc, C.c_int64), _p(v), _p(var),
                                                 _p(st, C.c_uint8), PRECISIONS[precision], None)
        _abi.check(rc)
        if full:
            return KrigingResult(v, var, np.full(total, np.nan), st)
        return v, var

    def predict_block_many(self, centers, offsets, full: bool = False):
        """``Kriging::predict_block`` (kriging.rs:674-779) for many blocks
        sharing one discretisation (``offsets``: noff x D).  Returns
        ``(value, variance)``, or a :class:`KrigingResult` with ``full=True``;
        a failing block is NaN with its status."""
        nb, (x, y, z) = self._targets(centers)
        off = _f64(offsets).reshape(-1, self.data.dim)
        v, var, lag = np.empty(nb), np.empty(nb), np.empty(nb)
        st = np.empty(nb, dtype=np.uint8)
        _abi.check(_abi.load().gs_kriging_predict_block(self._h, nb, _p(x), _p(y), _p(z), _p(off),
                                                        len(off), _p(v), _p(var), _p(lag),
                                                        _p(st, C.c_uint8), None))
        if full:
            return KrigingResult(v, var, lag, st)
        return v, var

    def predict_block(self, center, offsets):
        """One block: ``(value, variance, lagrange)``; raises as the
        reference does (NoNeighbors, SingularSystem, ...)."""
        r = self.predict_block_many(_f64(center).reshape(1, -1), offsets, full=True)
        code = int(r.status[0]) & 0x3f
        if code:
            from .errors import raise_for
            raise_for(code, "block kriging failed")
        lag = None if self.config.method == "simple" else float(r.lagrange[0])
        return float(r.value[0]), float(r.variance[0]), lag

    def predict_block_grid(self, bbox_min, bbox_max, ncell, block_size, discr=(4, 4),
                           full: bool = False):
        """``Kriging::predict_block_grid`` (kriging.rs:787-805): a block of
        ``block_size`` at every 2-D cell centre (x fastest)."""
        nc = np.ascontiguousarray(ncell, dtype=np.int64)
        total = int(np.prod(nc))
        v, var = np.empty(total), np.empty(total)
        st = np.empty(total, dtype=np.uint8)
        _abi.check(_abi.load().gs_kriging_predict_block_grid(
            self._h, _p(_f64(bbox_min)), _p(_f64(bbox_max)), _p(nc, C.c_int64),
            _p(_f64(block_size)), _p(np.ascontiguousarray(discr, dtype=np.int64), C.c_int64),
            _p(v), _p(var), _p(st, C.c_uint8), None))
        if full:
            return KrigingResult(v, var, np.full(total, np.nan), st)
        return v, var

    def neighbors(self, targets, kcap: int):
        """Conditioning indices per target (``Kriging::neighbors``), -1 padded."""
        nt, (x, y, z) = self._targets(targets)
        idx = np.empty(nt * kcap, dtype=np.int32)
        cnt = np.empty(nt, dtype=np.int32)
        _abi.check(_abi.load().gs_kriging_neighbors(self._h, nt, _p(x), _p(y), _p(z), kcap,
                                                    _p(idx, C.c_int32), _p(cnt, C.c_int32),
                                                    None))
        return idx.reshape(nt, kcap), cnt

    def predict_device(self, nt, x_ptr, y_ptr, z_ptr, v_ptr, var_ptr, st_ptr,
                       precision="mixed", stream=None, tdrift_ptr=None, lag_ptr=None,
                       asynchronous=False):
        """Device-pointer variant (inputs/outputs already in HBM).  With
        ``asynchronous`` the call only enqueues its work on ``stream`` (it can
        be captured into a CUDA graph)."""
        fn = (_abi.load().gs_kriging_predict_many_async if asynchronous
              else _abi.load().gs_kriging_predict_many_device)
        rc = fn(self._h, nt, x_ptr, y_ptr, z_ptr, tdrift_ptr, v_ptr, var_ptr, lag_ptr, st_ptr,
                PRECISIONS[precision], stream)
        _abi.check(rc)

    def set_tiles(self, run: int = 0, bins: int = 0, systems_per_block: int = 1):
        """Pin the mixed solver's launch shape (run 0 returns to autotuning)."""
        _abi.check(_abi.load().gs_kriging_set_tiles(self._h, int(run), int(bins),
                                                    int(systems_per_block)))

    def tiles(self, nt: int):
        """(run, bins, systems_per_block, source) a call with ``nt`` targets
        would use; source is "default", "tuned" or "pinned"."""
        r, b, sp, t = C.c_int32(), C.c_int32(), C.c_int32(), C.c_int32()
        _abi.check(_abi.load().gs_kriging_tiles(self._h, int(nt), C.byref(r), C.byref(b),
                                                C.byref(sp), C.byref(t)))
        return r.value, b.value, sp.value, ("default", "tuned", "pinned")[t.value]

    def close(self):
        if getattr(self, "_h", None):
            _abi.load().gs_kriging_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def last_timings():
    """Per-phase device milliseconds of the last predict call on this thread:
    (search, mixed solve, FP64 re-solve, whole call)."""
    out = np.zeros(4)
    _abi.load().gs_last_timings(_p(out))
    return tuple(out.tolist())


def last_vecchia_tiers():
    """Systems of the last mixed Vecchia likelihood call on this thread that
    were (accepted at the double-float refinement floor, refined with FP64
    residuals, re-solved by the FP64 kernel)."""
    out = np.zeros(2, dtype=np.int64)
    lib = _abi.load()
    lib.gs_last_vecchia_tiers(out.ctypes.data_as(_abi._pi64))
    return int(out[0]), int(out[1]), int(lib.gs_last_fallbacks())


# -------------------------------------------------- reference Python API --
# ------------------------------------------------------- cross-validation --
@dataclass
class CvResult:
    """Cross-validation result (validation.rs:10-117): observed values in data
    order, held-out predictions and kriging variances."""
    observed: np.ndarray
    predicted: np.ndarray
    variance: np.ndarray

    def _res(self):
        return self.predicted - self.observed

    def mean_error(self) -> float:
        return float(np.sum(self._res()) / len(self.observed))

    def mae(self) -> float:
        return float(np.sum(np.abs(self._res())) / len(self.observed))

    def mse(self) -> float:
        r = self._res()
        return float(np.sum(r * r) / len(self.observed))

    def rmse(self) -> float:
        return float(np.sqrt(self.mse()))

    def _obs_mean(self) -> float:
        return float(np.sum(self.observed) / len(self.observed))

    def rme(self) -> float:
        m = self._obs_mean()
        return float("nan") if abs(m) < np.finfo(float).eps else -self.mean_error() / m * 100.0

    def rmae(self) -> float:
        m = self._obs_mean()
        return float("nan") if abs(m) < np.finfo(float).eps else self.mae() / m * 100.0

    def rrmse(self) -> float:
        m = self._obs_mean()
        return float("nan") if abs(m) < np.finfo(float).eps else self.rmse() / m * 100.0

    def vecv(self) -> float:
        m = self._obs_mean()
        r = self._res()
        sst = float(np.sum((self.observed - m) ** 2))
        return float("nan") if sst <= 0.0 else (1.0 - float(np.sum(r * r)) / sst) * 100.0

    def e1(self) -> float:
        m = self._obs_mean()
        sad = float(np.sum(np.abs(self.observed - m)))
        return float("nan") if sad <= 0.0 else (1.0 - float(np.sum(np.abs(self._res()))) / sad) * 100.0

    def msdr(self) -> float:
        ok = self.variance > 1e-12
        if not ok.any():
            return float("nan")
        e = (self.predicted - self.observed)[ok]
        return float(np.sum(e * e / self.variance[ok]) / int(ok.sum()))


def _cross_validate(k: "Kriging", data: "PointSet", nfolds: int, seed: int,
                    precision: str) -> CvResult:
    n = data.n
    pred, var = np.empty(n), np.empty(n)
    st = np.empty(n, dtype=np.uint8)
    _abi.check(_abi.load().gs_kriging_cross_validate(k._h, int(nfolds), int(seed) & (2**64 - 1),
                                                     _p(pred), _p(var), _p(st, C.c_uint8),
                                                     PRECISIONS[precision]))
    return CvResult(np.array(data.values, dtype=float), pred, var)


def leave_one_out(data: "PointSet", model: VariogramModel, config: KrigingConfig = None,
                  precision: str = "mixed") -> CvResult:
    """``validation::leave_one_out`` (validation.rs:136-159): every point
    predicted from all the others."""
    if data.n < 3:
        from .errors import InsufficientData
        raise InsufficientData("leave-one-out cross-validation requires at least 3 points")
    return _cross_validate(Kriging.new(data, model, config), data, 0, 0, precision)


def leave_one_out_with_drift(data: "PointSet", drift_data, model: VariogramModel,
                             config: KrigingConfig, precision: str = "mixed") -> CvResult:
    """``validation::leave_one_out_with_drift`` (validation.rs:161-192)."""
    if data.n < 3:
        from .errors import InsufficientData
        raise InsufficientData("leave-one-out cross-validation requires at least 3 points")
    if len(drift_data) != data.n:
        raise DimensionMismatch(f"{len(drift_data)} drift rows vs {data.n} data points")
    k = Kriging.with_external_drift(data, model, config, drift_data)
    return _cross_validate(k, data, 0, 0, precision)


def k_fold(data: "PointSet", model: VariogramModel, config: KrigingConfig, k: int, seed: int,
           precision: str = "mixed") -> CvResult:
    """``validation::k_fold`` (validation.rs:236-253): seeded fold assignment,
    each fold predicted from the others."""
    if data.n < 3:
        from .errors import InsufficientData
        raise InsufficientData("cross-validation requires at least 3 points")
    if not 2 <= k <= data.n:
        raise InvalidParameter(f"k-fold requires 2 <= k <= n (k={k}, n={data.n})")
    return _cross_validate(Kriging.new(data, model, config), data, k, seed, precision)


def block_cv(data: "PointSet", model: VariogramModel, config: KrigingConfig, blocks_per_dim,
             precision: str = "mixed") -> CvResult:
    """``validation::block_cv`` (validation.rs:348-374): the data's bounding
    box cut into a regular grid of blocks, each block predicted from the
    points outside it."""
    bpd = np.ascontiguousarray(blocks_per_dim, dtype=np.int64)
    if len(bpd) != data.dim:
        raise DimensionMismatch(f"{len(bpd)} block counts for {data.dim} dimensions")
    k = Kriging.new(data, model, config)
    n = data.n
    pred, var = np.empty(n), np.empty(n)
    st = np.empty(n, dtype=np.uint8)
    _abi.check(_abi.load().gs_kriging_block_cv(k._h, _p(bpd, C.c_int64), _p(pred), _p(var),
                                               _p(st, C.c_uint8), PRECISIONS[precision]))
    return CvResult(np.array(data.values, dtype=float), pred, var)


def loo_cv(x, y, values, model, method="ordinary", mean=None, degree=1, max_neighbors=None,
           radius=None, folds=None, seed=0, min_neighbors=None, octant=None, blocks=None,
           precision: str = "mixed") -> dict:
    """lib.rs:695-745 ``loo_cv``: leave-one-out, ``folds``-fold or spatial
    ``blocks`` = (nx, ny) cross-validation, as a dict of the accuracy
    measures plus observed / predicted / variance."""
    data = PointSet.from_xyz(x, y, values)
    cfg = _build_method(method, mean, degree, values)
    cfg.max_neighbors = max_neighbors
    cfg.search_radius = radius
    cfg.min_neighbors = min_neighbors
    cfg.max_per_octant = octant
    if blocks is not None and folds is not None:
        raise InvalidParameter("blocks and folds are mutually exclusive")
    if blocks is not None:
        cv = block_cv(data, model, cfg, [blocks[0], blocks[1]], precision)
    elif folds is not None:
        cv = k_fold(data, model, cfg, int(folds), int(seed), precision)
    else:
        cv = leave_one_out(data, model, cfg, precision)
    return {"me": cv.mean_error(), "mae": cv.mae(), "mse": cv.mse(), "rmse": cv.rmse(),
            "msdr": cv.msdr(), "rme": cv.rme(), "rmae": cv.rmae(), "rrmse": cv.rrmse(),
            "vecv": cv.vecv(), "e1": cv.e1(), "observed": cv.observed,
            "predicted": cv.predicted, "variance": cv.variance}


@dataclass
class TuneResult:
    """``tuning::TuneResult``: the best candidate, its VEcv and the trace."""
    best: object
    best_vecv: float
    trace: list


def tune_kriging_neighbors(data: "PointSet", model: VariogramModel, method: str,
                           candidates: Sequence[int], radius: Optional[float] = None,
                           precision: str = "mixed") -> TuneResult:
    """``tuning::tune_kriging_neighbors`` (tuning.rs:97-125): leave-one-out
    VEcv per neighbourhood size (NaN where the cross-validation fails); the
    largest finite VEcv wins."""
    if len(candidates) == 0:
        raise InvalidParameter("no neighborhood sizes to try")
    trace = []
    for nb in candidates:
        cfg = KrigingConfig(method, max_neighbors=int(nb), search_radius=radius)
        try:
            v = leave_one_out(data, model, cfg, precision).vecv()
        except Exception:
            v = float("nan")
        trace.append((int(nb), v))
    finite = [t for t in trace if np.isfinite(t[1])]
    if not finite:
        raise InvalidParameter("no candidate produced a finite VEcv")
    best = finite[0]
    for t in finite[1:]:
        if t[1] >= best[1]:  # max_by keeps the last of equal maxima
            best = t
    return TuneResult(best[0], best[1], trace)


def _build_method(method: str, mean, degree, data_values) -> KrigingConfig:
    # crates/geostat-python/src/lib.rs:104-121 build_method
    if method == "ordinary":
        return KrigingConfig("ordinary")
    if method == "simple":
        return KrigingConfig("simple", mean=mean if mean is not None else seq_mean(data_values))
    if method == "universal":
        return KrigingConfig("universal", degree=degree)
    raise InvalidParameter(
        f"unknown method '{method}' (expected ordinary, simple or universal)")


def _anisotropic_search(search_azimuth, ratio, ratio_z, dip, rake):
    if search_azimuth is None:
        return None
    return Anisotropy(search_azimuth, ratio, ratio_z, dip, rake)


def krige(x, y, values, model, target_x, target_y, method="ordinary", mean=None, degree=1,
          max_neighbors=None, radius=None, min_neighbors=None, octant=None,
          measurement_error=None, search_azimuth=None, search_ratio=1.0, search_ratio_z=1.0,
          search_dip=0.0, search_rake=0.0, precision="mixed"):
    """lib.rs:500-571 ``krige``: returns ``(predictions, variances)``."""
    if len(target_x) != len(target_y):
        raise InvalidParameter("target_x and target_y differ in length")
    data = PointSet.from_xyz(x, y, values)
    cfg = _build_method(method, mean, degree, values)
    cfg.max_neighbors = max_neighbors
    cfg.search_radius = radius
    cfg.min_neighbors = min_neighbors
    cfg.max_per_octant = octant
    cfg.anisotropic_search = _anisotropic_search(search_azimuth, search_ratio, search_ratio_z,
                                                 search_dip, search_rake)
    if measurement_error is not None:
        k = Kriging.with_measurement_error(data, model, cfg, measurement_error)
    else:
        k = Kriging.new(data, model, cfg)
    t = np.stack([_f64(target_x), _f64(target_y)], axis=1)
    return k.predict_many(t, precision)


def krige_grid(x, y, values, model, bbox, nx, ny, method="ordinary", mean=None, degree=1,
               max_neighbors=None, radius=None, block=None, block_discr=(4, 4),
               min_neighbors=None, octant=None, search_azimuth=None, search_ratio=1.0,
               search_ratio_z=1.0, search_dip=0.0, search_rake=0.0, precision="mixed"):
    """lib.rs:632-696 ``krige_grid``: point kriging, or block kriging of
    ``block`` = (width, height) blocks discretised ``block_discr``."""
    if nx == 0 or ny == 0:
        raise InvalidParameter("grid must have at least one cell per axis")
    if not (bbox[2] > bbox[0]) or not (bbox[3] > bbox[1]):
        raise InvalidParameter(f"degenerate bbox: {bbox}")
    data = PointSet.from_xyz(x, y, values)
    cfg = _build_method(method, mean, degree, values)
    cfg.max_neighbors = max_neighbors
    cfg.search_radius = radius
    cfg.min_neighbors = min_neighbors
    cfg.max_per_octant = octant
    cfg.anisotropic_search = _anisotropic_search(search_azimuth, search_ratio, search_ratio_z,
                                                 search_dip, search_rake)
    k = Kriging.new(data, model, cfg)
    if block is not None:
        return k.predict_block_grid([bbox[0], bbox[1]], [bbox[2], bbox[3]], [nx, ny],
                                    [block[0], block[1]], [block_discr[0], block_discr[1]])
    return k.predict_grid([bbox[0], bbox[1]], [bbox[2], bbox[3]], [nx, ny], precision)


def block_offsets(size, n):
    """``block_offsets`` (kriging.rs:815-838): an n[0] x n[1] grid of cell
    centres covering a block of ``size``, centred on the origin."""
    nn = np.ascontiguousarray(n, dtype=np.int64)
    if nn[0] <= 0 or nn[1] <= 0:
        raise InvalidParameter("block discretization needs at least 1 point per axis")
    out = np.empty((int(nn[0] * nn[1]), 2))
    _abi.check(_abi.load().gs_block_offsets(_p(_f64(size)), _p(nn, C.c_int64), _p(out)))
    return out


def krige_3d(x, y, z, values, model, target_x, target_y, target_z, method="ordinary",
             mean=None, degree=1, max_neighbors=None, radius=None, precision="mixed"):
    """lib.rs:1650-1717 ``krige_3d``."""
    if not (len(target_x) == len(target_y) == len(target_z)):
        raise InvalidParameter("target_x, target_y and target_z differ in length")
    data = PointSet.from_xyzv(x, y, z, values)
    cfg = _build_method(method, mean, degree, values)
    cfg.max_neighbors = max_neighbors
    cfg.search_radius = radius
    k = Kriging.new(data, model, cfg)
    t = np.stack([_f64(target_x), _f64(target_y), _f64(target_z)], axis=1)
    return k.predict_many(t, precision)


class VecchiaPlan:
    """``VecchiaPlan`` (vecchia.rs:223-282) with its neighbour sets on the device."""

    def __init__(self, data: PointSet, m: int, order=None):
        self.data = data
        self.m = int(m)
        o = None if order is None else np.ascontiguousarray(order, dtype=np.int64)
        if o is not None and len(o) != data.n:
            raise DimensionMismatch(f"order has {len(o)} entries for {data.n} points")
        h = C.c_void_p()
        _abi.check(_abi.load().gs_vecchia_plan_create(data._h, self.m, _p(o, C.c_int64),
                                                      C.byref(h)))
        self._h = h
        self.m_eff = min(self.m, data.n - 1)

    def arrays(self):
        n, m = self.data.n, self.m_eff
        order = np.empty(n, dtype=np.int64)
        nb = np.empty(n * m, dtype=np.int64)
        cnt = np.empty(n, dtype=np.int32)
        _abi.check(_abi.load().gs_vecchia_plan_get(self._h, _p(order, C.c_int64),
                                                   _p(nb, C.c_int64), _p(cnt, C.c_int32)))
        return order, nb.reshape(n, m), cnt

    def loglik_grad(self, models, precision="mixed"):
        """loglik_grad_with_plan for single-structure isotropic models:
        returns (loglik[ncand], grad[ncand, 3], status[ncand])."""
        arr = (_abi.Model * len(models))(*[model_struct(m) for m in models])
        n = len(models)
        ll, g = np.empty(n), np.empty((n, 3))
        st = np.empty(n, dtype=np.int32)
        _abi.check(_abi.load().gs_vecchia_loglik_grad_batch(self._h, n, arr, _p(ll), _p(g),
                                                            _p(st, C.c_int32),
                                                            PRECISIONS[precision], None))
        return ll, g, st

    def loglik(self, models: Sequence[VariogramModel], precision="mixed"):
        """Log-likelihood of each candidate model in one batched launch.
        Returns ``(loglik, status)``."""
        arr = (_abi.Model * len(models))(*[model_struct(m) for m in models])
        ll = np.empty(len(models))
        st = np.empty(len(models), dtype=np.int32)
        _abi.check(_abi.load().gs_vecchia_loglik_batch(self._h, len(models), arr, _p(ll),
                                                       _p(st, C.c_int32),
                                                       PRECISIONS[precision], None))
        return ll, st

    def loglik_range(self, lo: int, hi: int, models: Sequence[VariogramModel],
                     precision="mixed"):
        """Sum of the log-likelihood terms of the ordered positions
        ``[lo, hi)`` of each candidate model (one shard of the points).
        Returns ``(partial_loglik, status)``."""
        arr = (_abi.Model * len(models))(*[model_struct(m) for m in models])
        ll = np.empty(len(models))
        st = np.empty(len(models), dtype=np.int32)
        _abi.check(_abi.load().gs_vecchia_loglik_batch_range(self._h, int(lo), int(hi),
                                                             len(models), arr, _p(ll),
                                                             _p(st, C.c_int32),
                                                             PRECISIONS[precision], None))
        return ll, st

    def loglik_grouped(self, models: Sequence[VariogramModel], group_size: int):
        """``loglik_with_plan_grouped`` (vecchia.rs:604-668, Guinness
        grouping) of each candidate model; ``group_size <= 1`` is
        :meth:`loglik`.  Returns ``(loglik, status)``."""
        arr = (_abi.Model * len(models))(*[model_struct(m) for m in models])
        ll = np.empty(len(models))
        st = np.empty(len(models), dtype=np.int32)
        _abi.check(_abi.load().gs_vecchia_loglik_grouped_batch(self._h, len(models), arr,
                                                               int(group_size), _p(ll),
                                                               _p(st, C.c_int32), None))
        return ll, st

    def reml_loglik(self, models: Sequence[VariogramModel], drift_degree: int = 1, drift=None,
                    group_size: int = 1):
        """Vecchia REML log-likelihood (vecchia.rs:1278-1457) of each
        candidate: the mean a GLS trend over a polynomial basis of
        ``drift_degree`` or, with ``drift`` (n x ncov covariates), the
        intercept plus standardised covariates.  Returns ``(loglik, status)``."""
        arr = (_abi.Model * len(models))(*[model_struct(m) for m in models])
        ll = np.empty(len(models))
        st = np.empty(len(models), dtype=np.int32)
        d = None if drift is None else _f64(drift).reshape(self.data.n, -1)
        _abi.check(_abi.load().gs_vecchia_reml_loglik_batch(
            self._h, len(models), arr, int(drift_degree), _p(d),
            0 if d is None else d.shape[1], int(group_size), _p(ll), _p(st, C.c_int32), None))
        return ll, st

    def close(self):
        if getattr(self, "_h", None):
            _abi.load().gs_vecchia_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def maxmin_order(coords):
    """``maxmin_order`` (vecchia.rs:144-215), on the host."""
    c = _f64(coords)
    dim = c.shape[1]
    out = np.empty(len(c), dtype=np.int64)
    cols = [_f64(c[:, d]) for d in range(dim)] + ([None] if dim == 2 else [])
    _abi.check(_abi.load().gs_maxmin_order(dim, len(c), _p(cols[0]), _p(cols[1]), _p(cols[2]),
                                           _p(out, C.c_int64)))
    return out


def vecchia_loglik(x, y, values, model, m=20):
    """lib.rs:478-490 ``vecchia_loglik``."""
    data = PointSet.from_xyz(x, y, values)
    ll = C.c_double()
    _abi.check(_abi.load().gs_vecchia_loglik(data._h, C.byref(model_struct(model)), int(m), None,
                                             C.byref(ll)))
    return ll.value


def vecchia_loglik_grouped(data: PointSet, model: VariogramModel, m: int, order=None,
                           group_size: int = 1) -> float:
    """``vecchia_loglik_grouped`` (vecchia.rs:891-901)."""
    plan = VecchiaPlan(data, m, order)
    ll, st = plan.loglik_grouped([model], group_size)
    if st[0] != 0:
        from .errors import raise_for
        raise_for(int(st[0]), "singular conditioning system")
    return float(ll[0])


def _fit_kind(kind):
    from .model import parse_kind
    kname, _ = parse_kind(kind) if kind not in KIND_CODES else (kind, 0.0)
    return kname


def vecchia_mle_fit(data: PointSet, kind="exponential", m=20, order=None):
    """``vecchia_mle`` (vecchia.rs:921-1081): the reference's BFGS fit with the
    analytical gradient; returns ``(model, loglik, x, n_evals)``."""
    kname = _fit_kind(kind)
    o = None if order is None else np.ascontiguousarray(order, dtype=np.int64)
    out = _abi.Model()
    ll = C.c_double()
    x = np.zeros(3)
    ne = C.c_int64()
    _abi.check(_abi.load().gs_vecchia_mle(data._h, KIND_CODES[kname], int(m), _p(o, C.c_int64),
                                          C.byref(out), C.byref(ll), _p(x), C.byref(ne)))
    model = VariogramModel(out.nugget, [Structure(kname, out.s[0].sill, out.s[0].range)])
    return model, ll.value, x, ne.value


def vecchia_mle_nm_fit(data: PointSet, kind="exponential", m=20, starts=None, nstarts=3, step=0.3,
                       max_iter=2000, order=None):
    """Batched multi-start Nelder-Mead fit; returns ``(model, loglik, x, n_evals)``."""
    kname = _fit_kind(kind)
    st = None if starts is None else _f64(starts).reshape(-1, 3)
    ns = len(st) if st is not None else int(nstarts)
    o = None if order is None else np.ascontiguousarray(order, dtype=np.int64)
    out = _abi.Model()
    ll = C.c_double()
    x = np.zeros(3)
    ne = C.c_int64()
    _abi.check(_abi.load().gs_vecchia_mle_nm(data._h, KIND_CODES[kname], int(m), _p(o, C.c_int64),
                                             ns, _p(st), float(step), int(max_iter), C.byref(out),
                                             C.byref(ll), _p(x), C.byref(ne)))
    model = VariogramModel(out.nugget, [Structure(kname, out.s[0].sill, out.s[0].range)])
    return model, ll.value, x, ne.value


def _fit_result(kname, out, ll, x, ne):
    model = VariogramModel(out.nugget, [Structure(kname, out.s[0].sill, out.s[0].range)])
    return model, ll.value, x, ne.value


def vecchia_mle_grouped_fit(data: PointSet, kind="exponential", m=20, order=None,
                            group_size: int = 1):
    """``vecchia_mle_grouped`` (vecchia.rs:939-950); returns
    ``(model, loglik, x, n_evals)``."""
    kname = _fit_kind(kind)
    o = None if order is None else np.ascontiguousarray(order, dtype=np.int64)
    out, ll, x, ne = _abi.Model(), C.c_double(), np.zeros(3), C.c_int64()
    _abi.check(_abi.load().gs_vecchia_mle_grouped(data._h, KIND_CODES[kname], int(m),
                                                  _p(o, C.c_int64), int(group_size), C.byref(out),
                                                  C.byref(ll), _p(x), C.byref(ne)))
    return _fit_result(kname, out, ll, x, ne)


def vecchia_reml_fit(data: PointSet, kind="exponential", m=20, drift_degree: int = 1, order=None,
                     group_size: int = 1):
    """``vecchia_reml`` / ``vecchia_reml_grouped`` (vecchia.rs:1460-1493);
    returns ``(model, loglik, x, n_evals)``."""
    kname = _fit_kind(kind)
    o = None if order is None else np.ascontiguousarray(order, dtype=np.int64)
    out, ll, x, ne = _abi.Model(), C.c_double(), np.zeros(3), C.c_int64()
    _abi.check(_abi.load().gs_vecchia_reml(data._h, KIND_CODES[kname], int(m), int(drift_degree),
                                           _p(o, C.c_int64), int(group_size), C.byref(out),
                                           C.byref(ll), _p(x), C.byref(ne)))
    return _fit_result(kname, out, ll, x, ne)


def vecchia_reml_drift_fit(data: PointSet, drift, kind="exponential", m=20, order=None,
                           group_size: int = 1):
    """``vecchia_reml_drift`` / ``vecchia_reml_drift_grouped``
    (vecchia.rs:1500-1568), ``drift`` one row of covariates per point;
    returns ``(model, loglik, x, n_evals)``."""
    kname = _fit_kind(kind)
    rows = [list(r) for r in drift] if not isinstance(drift, np.ndarray) else None
    if rows is not None:
        ncov = len(rows[0]) if rows else 0
        if any(len(r) != ncov for r in rows):
            raise DimensionMismatch("all drift rows must have the same number of covariates")
        d = np.array(rows, dtype=np.float64).reshape(len(rows), ncov)
    else:
        d = drift.reshape(len(drift), -1) if drift.ndim == 1 else drift
    d = _f64(d)
    o = None if order is None else np.ascontiguousarray(order, dtype=np.int64)
    out, ll, x, ne = _abi.Model(), C.c_double(), np.zeros(3), C.c_int64()
    _abi.check(_abi.load().gs_vecchia_reml_drift(data._h, KIND_CODES[kname], int(m), _p(d),
                                                 d.shape[0], d.shape[1] if d.ndim == 2 else 0,
                                                 _p(o, C.c_int64), int(group_size), C.byref(out),
                                                 C.byref(ll), _p(x), C.byref(ne)))
    return _fit_result(kname, out, ll, x, ne)


def _se_from_hessian(hess):
    """vecchia.rs:1918-1935 se_from_hessian: sqrt of the diagonal of the
    inverse (lu_factor's partial pivoting and singular test), NaN for a
    singular matrix or a non-positive diagonal entry."""
    n = len(hess)
    a = [list(map(float, row)) for row in hess]
    scale = max(max(abs(v) for v in row) for row in a)
    scale = max(scale, 2.2250738585072014e-308)
    piv = list(range(n))
    for k in range(n):
        p = max(range(k, n), key=lambda i: (abs(a[i][k]), -i))
        if abs(a[p][k]) < 1e-12 * scale:
            return [float("nan")] * n
        piv[k] = p
        a[k], a[p] = a[p], a[k]
        for i in range(k + 1, n):
            f = a[i][k] / a[k][k]
            a[i][k] = f
            if f != 0.0:
                for j in range(k + 1, n):
                    a[i][j] -= f * a[k][j]
    out = []
    for col in range(n):
        b = [1.0 if q == col else 0.0 for q in range(n)]
        for k in range(n):
            b[k], b[piv[k]] = b[piv[k]], b[k]
        for i in range(n):
            b[i] -= sum(a[i][j] * b[j] for j in range(i))
        for i in range(n - 1, -1, -1):
            b[i] = (b[i] - sum(a[i][j] * b[j] for j in range(i + 1, n))) / a[i][i]
        out.append(math.sqrt(b[col]) if b[col] > 0.0 else float("nan"))
    return out


def vecchia_param_se_fit(data: PointSet, model: VariogramModel, m: int = 20, order=None):
    """``vecchia_param_se`` (vecchia.rs:1666-1918): asymptotic standard errors
    of (nugget, partial sill, range) from the semi-analytical Hessian -- the
    analytical gradient (one batched launch for all the +-h points)
    differenced centrally with h = max(1e-3 |theta|, 1e-5) and symmetrised.
    A nugget within one step of zero gives NaN for it and the SEs of the
    restricted (sill, range) problem."""
    from .model import GPU_KINDS
    if len(model.structures) != 1:
        raise InvalidParameter("standard errors are defined for a single-structure model")
    st0 = model.structures[0]
    kname = _fit_kind(st0.kind)
    if kname == "power":
        raise InvalidParameter("Vecchia needs a valid covariance function and cannot use the "
                               "unbounded Power model")
    if kname not in GPU_KINDS:
        raise InvalidParameter("the CUDA path has closed-form gradients for spherical, "
                               "exponential, gaussian, matern15 and matern25")
    plan = VecchiaPlan(data, m, order)
    theta = [model.nugget, st0.sill, st0.range]
    h = [max(abs(t) * 1e-3, 1e-5) for t in theta]
    free = [1, 2] if theta[0] - h[0] < 0.0 else [0, 1, 2]
    pts = []
    for i in free:
        for sgn in (1.0, -1.0):
            t = list(theta)
            t[i] += sgn * h[i]
            pts.append(t)
    ok = all(t[1] > 0.0 and t[2] > 0.0 and t[0] >= 0.0 for t in pts)
    hess = None
    if ok:
        mods = [VariogramModel(t[0], [Structure(kname, t[1], t[2])]) for t in pts]
        _, g, st = plan.loglik_grad(mods)
        if (st == 0).all() and np.isfinite(g).all():
            k = len(free)
            hess = [[0.0] * k for _ in range(k)]
            for a, i in enumerate(free):
                gp, gm = -g[2 * a], -g[2 * a + 1]  # gradients of the negative log-likelihood
                for b, j in enumerate(free):
                    hess[a][b] = (gp[j] - gm[j]) / (2.0 * h[i])
            for a in range(k):
                for b in range(a + 1, k):
                    avg = 0.5 * (hess[a][b] + hess[b][a])
                    hess[a][b] = hess[b][a] = avg
    if hess is None:
        # the fully numerical Hessian of the negative log-likelihood
        def nll_batch(ts):
            mods = [VariogramModel(t[0], [Structure(kname, t[1], t[2])]) for t in ts]
            ll, st = plan.loglik(mods)
            return [(-l if (s == 0 and np.isfinite(l) and t[1] > 0 and t[2] > 0 and t[0] >= 0)
                     else float("inf")) for l, s, t in zip(ll, st, ts)]
        k = len(free)
        ts = [list(theta)]
        for a, i in enumerate(free):
            for sgn in (1.0, -1.0):
                t = list(theta)
                t[i] += sgn * h[i]
                ts.append(t)
        for a in range(k):
            for b in range(a + 1, k):
                i, j = free[a], free[b]
                for si, sj in ((1, 1), (1, -1), (-1, 1), (-1, -1)):
                    t = list(theta)
                    t[i] += si * h[i]
                    t[j] += sj * h[j]
                    ts.append(t)
        f = nll_batch(ts)
        hess = [[0.0] * k for _ in range(k)]
        q = 1 + 2 * k
        for a, i in enumerate(free):
            hess[a][a] = (f[1 + 2 * a] - 2.0 * f[0] + f[2 + 2 * a]) / (h[i] * h[i])
        for a in range(k):
            for b in range(a + 1, k):
                i, j = free[a], free[b]
                v = (f[q] - f[q + 1] - f[q + 2] + f[q + 3]) / (4.0 * h[i] * h[j])
                q += 4
                hess[a][b] = hess[b][a] = v
    se = _se_from_hessian(hess)
    return (float("nan"), se[0], se[1]) if len(free) == 2 else tuple(se)


def vecchia_param_se(x, y, values, model, m=20):
    """lib.rs:419-437 ``vecchia_param_se``."""
    data = PointSet.from_xyz(x, y, values)
    return vecchia_param_se_fit(data, model, m)


def vecchia_reml(x, y, values, kind="exponential", m=20, drift_degree=1):
    """lib.rs:370-392 ``vecchia_reml``."""
    data = PointSet.from_xyz(x, y, values)
    return vecchia_reml_fit(data, kind, m, drift_degree)[0]


def vecchia_reml_drift(x, y, values, covariates, kind="exponential", m=20):
    """lib.rs:394-417 ``vecchia_reml_drift``."""
    data = PointSet.from_xyz(x, y, values)
    return vecchia_reml_drift_fit(data, covariates, kind, m)[0]


def vecchia_mle(x, y, values, kind="exponential", m=20):
    """lib.rs:351-367 ``vecchia_mle``."""
    data = PointSet.from_xyz(x, y, values)
    return vecchia_mle_fit(data, kind, m)[0]


def vecchia_krige(x, y, values, model, target_x, target_y, m=30):
    """lib.rs:445-476 ``vecchia_krige``: returns ``(predictions, variances)``."""
    if len(target_x) != len(target_y):
        raise InvalidParameter("target_x and target_y differ in length")
    data = PointSet.from_xyz(x, y, values)
    tx, ty = _f64(target_x), _f64(target_y)
    nt = len(tx)
    v, var = np.empty(nt), np.empty(nt)
    _abi.check(_abi.load().gs_vecchia_predict(data._h, C.byref(model_struct(model)), nt, _p(tx),
                                              _p(ty), None, int(m), _p(v), _p(var)))
    return v, var


class Server:
    """Continuous-batching request loop over resident data sets (the C ABI's
    gs_server_*): ``add_kriging`` / ``add_vecchia`` register built
    predictors and plans, ``submit_predict`` / ``submit_loglik`` queue
    requests from any thread and return a request object, ``wait`` blocks
    for one, ``stats`` gives (p50 ms, p99 ms, completed, launches)."""

    class _Req:
        def __init__(self, rid, keep, out):
            self.id, self._keep, self.out = rid, keep, out

    def __init__(self, mem_budget_bytes=64 << 30, executors=2):
        h = C.c_void_p()
        _abi.check(_abi.load().gs_server_create(int(mem_budget_bytes), int(executors),
                                                C.byref(h)))
        self._h = h
        self._keep = []

    def add_kriging(self, k: "Kriging") -> int:
        d = C.c_int32()
        _abi.check(_abi.load().gs_server_add_kriging(self._h, k._h, C.byref(d)))
        self._keep.append(k)
        return d.value

    def add_vecchia(self, plan: "VecchiaPlan") -> int:
        d = C.c_int32()
        _abi.check(_abi.load().gs_server_add_vecchia(self._h, plan._h, C.byref(d)))
        self._keep.append(plan)
        return d.value

    def submit_predict(self, dataset: int, targets):
        t = np.asarray(targets, dtype=np.float64)
        cols = [np.ascontiguousarray(t[:, d]) for d in range(t.shape[1])]
        nt = len(t)
        v, var = np.empty(nt), np.empty(nt)
        st = np.empty(nt, dtype=np.uint8)
        rid = C.c_int64()
        _abi.check(_abi.load().gs_server_submit_predict(
            self._h, int(dataset), nt, _p(cols[0]), _p(cols[1]),
            _p(cols[2]) if len(cols) == 3 else None, _p(v), _p(var), _p(st, C.c_uint8),
            C.byref(rid)))
        return Server._Req(rid.value, cols, (v, var, st))

    def submit_loglik(self, dataset: int, model: VariogramModel):
        ms = model_struct(model)
        ll = np.empty(1)
        st = np.empty(1, dtype=np.int32)
        rid = C.c_int64()
        _abi.check(_abi.load().gs_server_submit_loglik(self._h, int(dataset), C.byref(ms), _p(ll),
                                                       _p(st, C.c_int32), C.byref(rid)))
        return Server._Req(rid.value, ms, (ll, st))

    def set_precision(self, precision: str):
        """Precision of the launches formed from now on ("mixed" or "fp64")."""
        _abi.check(_abi.load().gs_server_set_precision(self._h, PRECISIONS[precision]))

    def cancel(self, req):
        """Cancels a request that has not started (raises InvalidParameter
        once it runs or has finished); its ``wait`` then raises Cancelled."""
        _abi.check(_abi.load().gs_server_cancel(self._h, req.id))

    def wait(self, req) -> float:
        lat = C.c_double()
        _abi.check(_abi.load().gs_server_wait(self._h, req.id, C.byref(lat)))
        return lat.value

    def stats(self):
        p50, p99 = C.c_double(), C.c_double()
        done, launches = C.c_int64(), C.c_int64()
        _abi.check(_abi.load().gs_server_stats(self._h, C.byref(p50), C.byref(p99),
                                               C.byref(done), C.byref(launches)))
        return p50.value, p99.value, done.value, launches.value

    def close(self):
        if getattr(self, "_h", None):
            _abi.load().gs_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def vecchia_predict(coords, values, model, targets, m=30, pointset=None):
    """``vecchia_predict`` (vecchia.rs:748-866) in 2-D or 3-D: joint Vecchia
    prediction at ``targets``; returns ``(values, variances)``.  An existing
    ``pointset`` of the same data may be passed instead of coords/values."""
    data = pointset if pointset is not None else PointSet(coords, values)
    targets = np.ascontiguousarray(np.asarray(targets, dtype=np.float64))
    if targets.ndim != 2 or targets.shape[1] != data.dim:
        raise DimensionMismatch("targets must be an (nt, dim) array matching the data")
    nt = len(targets)
    cols = [np.ascontiguousarray(targets[:, d]) for d in range(data.dim)]
    v, var = np.empty(nt), np.empty(nt)
    _abi.check(_abi.load().gs_vecchia_predict(data._h, C.byref(model_struct(model)), nt,
                                              _p(cols[0]), _p(cols[1]),
                                              _p(cols[2]) if data.dim == 3 else None, int(m),
                                              _p(v), _p(var)))
    return v, var


def nelder_mead_multistart(fn, starts, step, max_iter):
    """The library's Nelder-Mead state machine driven by a Python objective."""
    starts = _f64(starts)
    ns, n = starts.shape
    cb = _abi.OBJECTIVE(lambda xp, nn, ctx: float(fn(np.ctypeslib.as_array(xp, shape=(nn,)).copy())))
    x = np.zeros(n)
    f = C.c_double()
    _abi.check(_abi.load().gs_nelder_mead_multistart(cb, None, n, ns, _p(starts), float(step),
                                                     int(max_iter), _p(x), C.byref(f)))
    return x, f.value


def rng_uniform(seed: int, count: int) -> np.ndarray:
    out = np.empty(count)
    _abi.load().gs_rng_uniform(seed, count, _p(out))
    return out


def rng_normal(seed: int, count: int) -> np.ndarray:
    out = np.empty(count)
    _abi.load().gs_rng_normal(seed, count, _p(out))
    return out


