"""ctypes wrapper of the FP64 CPU oracle (oracle/geostat_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
and by the CPU-baseline / reference arm of ``bench.py`` -- never by the
product package.  The oracle restates the reference's CPU algorithms
(geostat-rs crates/geostat-core) and is the parity checker for the CUDA path.

Models are duck-typed: any object with ``nugget`` and ``structures`` (each
with ``kind``, ``sill``, ``range``, optional ``param`` and optional ``anis``
carrying ``azimuth_deg``, ``ratio``, ``ratio_z``, ``dip_deg``, ``rake_deg``)
works, so the product's ``geostat_rs.VariogramModel`` can be passed directly.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libgeostat_oracle.so")

KINDS = {
    "spherical": 0, "exponential": 1, "gaussian": 2, "matern15": 3, "matern25": 4,
    "circular": 5, "stable": 6, "hole": 7, "wave": 8, "power": 9,
}

OK, INSUFFICIENT_DATA, DIMENSION_MISMATCH, SINGULAR_SYSTEM = 0, 1, 2, 3
INVALID_PARAMETER, NO_NEIGHBORS, DUPLICATE_POINTS = 4, 5, 6


class OracleError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"oracle error {code}: {msg}")
        self.code = code


class _Structure(C.Structure):
    _fields_ = [("kind", C.c_int32), ("has_anis", C.c_int32), ("param", C.c_double),
                ("sill", C.c_double), ("range", C.c_double), ("azimuth_deg", C.c_double),
                ("ratio", C.c_double), ("ratio_z", C.c_double), ("dip_deg", C.c_double),
                ("rake_deg", C.c_double)]


class _Model(C.Structure):
    _fields_ = [("nugget", C.c_double), ("n_structures", C.c_int32), ("pad_", C.c_int32),
                ("s", _Structure * 4)]


class _Kcfg(C.Structure):
    _fields_ = [("method", C.c_int64), ("sk_mean", C.c_double), ("uk_degree", C.c_int64),
                ("ked_nvars", C.c_int64), ("max_neighbors", C.c_int64),
                ("min_neighbors", C.c_int64), ("max_per_octant", C.c_int64),
                ("has_search_radius", C.c_int64), ("search_radius", C.c_double),
                ("has_anisotropic_search", C.c_int64), ("search_azimuth_deg", C.c_double),
                ("search_ratio", C.c_double), ("search_ratio_z", C.c_double),
                ("search_dip_deg", C.c_double), ("search_rake_deg", C.c_double)]


def build(quiet: bool = True) -> str:
    """Compiles the oracle with its Makefile (no-op when up to date)."""
    out = subprocess.run(["make", "-C", _HERE], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    return _LIB_PATH


_lib = None
_OBJ = C.CFUNCTYPE(C.c_double, C.POINTER(C.c_double), C.c_int64, C.c_void_p)
_GRAD = C.CFUNCTYPE(None, C.POINTER(C.c_double), C.c_int64, C.POINTER(C.c_double), C.c_void_p)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        _lib = C.CDLL(_LIB_PATH)
        _declare(_lib)
    return _lib


def _declare(L):
    """Argument types for every entry point (int64_t parameters must not be
    passed as 32-bit C ints)."""
    d, i32, i64, u64, vp = C.c_double, C.c_int32, C.c_int64, C.c_uint64, C.c_void_p
    pd, pi8, pi32, pi64 = (C.POINTER(C.c_double), C.POINTER(C.c_int8), C.POINTER(C.c_int32),
                           C.POINTER(C.c_int64))
    pm, pk = C.POINTER(_Model), C.POINTER(_Kcfg)
    sig = {
        "or_last_error": (C.c_char_p, []),
        "or_model_validate": (C.c_int, [pm]),
        "or_gamma_dh": (d, [pm, C.c_int, pd]),
        "or_lu_solve": (C.c_int, [i64, pd, pd, pd]),
        "or_cholesky_solve": (C.c_int, [i64, pd, pd, pd]),
        "or_kdtree_knn": (i64, [C.c_int, i64, pd, pd, i64, C.c_int, d, pi64]),
        "or_knn_brute": (i64, [C.c_int, i64, pd, pd, i64, C.c_int, d, pi64]),
        "or_bucketgrid_queries": (C.c_int, [C.c_int, i64, pd, pd, pd, i64, i64, pi64, pd, i64,
                                            C.c_int, d, pi64, pi64, pi64]),
        "or_duplicate_pair": (C.c_int, [C.c_int, i64, pd, pi64, pi64]),
        "or_grid_centers": (C.c_int, [C.c_int, pd, pd, pi64, pd]),
        "or_krige": (C.c_int, [C.c_int, i64, pd, pd, pd, pd, C.c_int, pm, pk, i64, pd, pd, pd,
                               pd, pd, pi8, pi32, i64, pi32, pi64, C.c_int]),
        "or_maxmin_order": (C.c_int, [C.c_int, i64, pd, pi64]),
        "or_maxmin_order_brute": (C.c_int, [C.c_int, i64, pd, pi64]),
        "or_vecchia_plan": (C.c_int, [C.c_int, i64, pd, i64, pi64, pi64, pi64, pi32]),
        "or_vecchia_loglik_grouped": (C.c_int, [C.c_int, i64, pd, pd, pm, i64, pi64, pi64, pi32,
                                                i64, pd]),
        "or_vecchia_loglik_plan": (C.c_int, [C.c_int, i64, pd, pd, pm, i64, pi64, pi64, pi32,
                                             pd, pd]),
        "or_vecchia_loglik": (C.c_int, [C.c_int, i64, pd, pd, pm, i64, pi64, pd]),
        "or_exact_loglik": (C.c_int, [C.c_int, i64, pd, pd, pm, pd]),
        "or_vecchia_predict": (C.c_int, [C.c_int, i64, pd, pd, pm, i64, pd, i64, pd, pd]),
        "or_vecchia_mle_objective": (C.c_int, [C.c_int, i64, pd, pd, i32, d, i64, pi64, pi64,
                                               pi32, d, i64, pd, pd]),
        "or_vecchia_mle_setup": (C.c_int, [C.c_int, i64, pd, pd, pd, pd]),
        "or_vecchia_mle_nm": (C.c_int, [C.c_int, i64, pd, pd, i32, d, i64, pi64, i64, pd, d, i64,
                                        pd, pd, pi64]),
        "or_krige_block": (C.c_int, [C.c_int, i64, pd, pd, pd, C.c_int, pm, pk, i64, pd, pd, i64,
                                     pd, pd, pd, pi8]),
        "or_spatial_block_assignment": (C.c_int, [C.c_int, i64, pd, pi64, pi64]),
        "or_guinness_blocks": (C.c_int, [i64, i64, pi64, pi64, pi32, i64, pi64, pi64]),
        "or_poly_basis_terms": (i64, [C.c_int, i32]),
        "or_poly_basis": (C.c_int, [C.c_int, i64, pd, i32, pd]),
        "or_drift_basis": (C.c_int, [i64, i64, pd, pd]),
        "or_vecchia_reml_loglik": (C.c_int, [C.c_int, i64, pd, pd, pm, i64, pi64, pi64, pi32, pd,
                                             i64, i64, pd]),
        "or_vecchia_fit_nm": (C.c_int, [C.c_int, i64, pd, pd, i32, i64, pi64, pd, i64, i64, i64,
                                        pd, d, i64, pd, pd, pi64]),
        "or_rng_draw": (None, [C.c_uint64, i64, i64, pd]),
        "or_nelder_mead_multistart": (C.c_int, [_OBJ, vp, i64, i64, pd, d, i64, pd, pd]),
        "or_g_and_dg": (C.c_int, [i32, d, pd, pd]),
        "or_vecchia_loglik_grad": (C.c_int, [C.c_int, i64, pd, pd, i32, d, d, d, i64, pi64, pi64,
                                             pi32, pd, pd]),
        "or_vecchia_mle_bfgs": (C.c_int, [C.c_int, i64, pd, pd, i32, i64, pi64, i64, pd, pd,
                                          pi64]),
        "or_bfgs_multistart": (C.c_int, [_OBJ, _GRAD, vp, i64, i64, pd, i64, pd, pd]),
        "or_rng_u64": (None, [u64, i64, C.POINTER(C.c_uint64)]),
        "or_rng_uniform": (None, [u64, i64, pd]),
        "or_rng_normal": (None, [u64, i64, pd]),
        "or_test_field_2d": (None, [i64, u64, pd, pd]),
        "or_test_field_3d": (None, [i64, u64, pd, pd]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args


def _p(a, ct=C.c_double):
    return a.ctypes.data_as(C.POINTER(ct)) if a is not None else None


def _check(rc):
    if rc != 0:
        raise OracleError(rc, lib().or_last_error().decode())


def model_struct(model) -> _Model:
    m = _Model()
    m.nugget = float(model.nugget)
    structs = list(model.structures)
    if len(structs) > 4:
        raise ValueError("at most 4 structures")
    m.n_structures = len(structs)
    for i, s in enumerate(structs):
        kind = s.kind
        m.s[i].kind = KINDS[kind] if isinstance(kind, str) else int(kind)
        m.s[i].param = float(getattr(s, "param", 0.0) or 0.0)
        m.s[i].sill = float(s.sill)
        m.s[i].range = float(s.range)
        a = getattr(s, "anis", None)
        if a is not None:
            m.s[i].has_anis = 1
            m.s[i].azimuth_deg = a.azimuth_deg
            m.s[i].ratio = a.ratio
            m.s[i].ratio_z = getattr(a, "ratio_z", 1.0)
            m.s[i].dip_deg = getattr(a, "dip_deg", 0.0)
            m.s[i].rake_deg = getattr(a, "rake_deg", 0.0)
        else:
            m.s[i].ratio = m.s[i].ratio_z = 1.0
    return m


METHODS = {"simple": 0, "ordinary": 1, "universal": 2, "external_drift": 3}


def kcfg_struct(method="ordinary", mean=None, degree=1, n_vars=0, max_neighbors=None,
                min_neighbors=None, max_per_octant=None, radius=None, anisotropic_search=None):
    c = _Kcfg()
    c.method = METHODS[method]
    c.sk_mean = float(mean) if mean is not None else 0.0
    c.uk_degree = int(degree)
    c.ked_nvars = int(n_vars)
    c.max_neighbors = -1 if max_neighbors is None else int(max_neighbors)
    c.min_neighbors = -1 if min_neighbors is None else int(min_neighbors)
    c.max_per_octant = -1 if max_per_octant is None else int(max_per_octant)
    c.has_search_radius = 0 if radius is None else 1
    c.search_radius = float(radius) if radius is not None else 0.0
    if anisotropic_search is not None:
        a = anisotropic_search
        c.has_anisotropic_search = 1
        c.search_azimuth_deg = a.azimuth_deg
        c.search_ratio = a.ratio
        c.search_ratio_z = getattr(a, "ratio_z", 1.0)
        c.search_dip_deg = getattr(a, "dip_deg", 0.0)
        c.search_rake_deg = getattr(a, "rake_deg", 0.0)
    return c


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def gamma_dh(model, dh):
    dh = _f64(dh)
    m = model_struct(model)
    return lib().or_gamma_dh(C.byref(m), len(dh), _p(dh))


def model_validate(model):
    m = model_struct(model)
    _check(lib().or_model_validate(C.byref(m)))


def lu_solve(a, b):
    a, b = _f64(a), _f64(b)
    x = np.zeros_like(b)
    _check(lib().or_lu_solve(len(b), _p(a), _p(b), _p(x)))
    return x


def cholesky_solve(a, b):
    a, b = _f64(a), _f64(b)
    x = np.zeros_like(b)
    _check(lib().or_cholesky_solve(len(b), _p(a), _p(b), _p(x)))
    return x


def kdtree_knn(coords, target, k, radius=None):
    coords, target = _f64(coords), _f64(target)
    out = np.zeros(max(min(k, len(coords)), 1), dtype=np.int64)
    cnt = lib().or_kdtree_knn(coords.shape[1], len(coords), _p(coords), _p(target), int(k),
                              0 if radius is None else 1, C.c_double(radius or 0.0),
                              _p(out, C.c_int64))
    return out[:cnt].tolist()


def knn_brute(coords, target, k, radius=None):
    coords, target = _f64(coords), _f64(target)
    out = np.zeros(max(min(k, len(coords)), 1), dtype=np.int64)
    cnt = lib().or_knn_brute(coords.shape[1], len(coords), _p(coords), _p(target), int(k),
                             0 if radius is None else 1, C.c_double(radius or 0.0),
                             _p(out, C.c_int64))
    return out[:cnt].tolist()


def bucketgrid_queries(coords, bbox_min, bbox_max, expected, q_after, q_target, k, radius=None):
    coords = _f64(coords)
    dim = coords.shape[1]
    q_after = np.ascontiguousarray(q_after, dtype=np.int64)
    q_target = _f64(q_target).reshape(-1, dim)
    nq = len(q_after)
    out = np.full(nq * k, -1, dtype=np.int64)
    cnt = np.zeros(nq, dtype=np.int64)
    dims = np.zeros(3, dtype=np.int64)
    _check(lib().or_bucketgrid_queries(dim, len(coords), _p(coords), _p(_f64(bbox_min)),
                                       _p(_f64(bbox_max)), int(expected), nq,
                                       _p(q_after, C.c_int64), _p(q_target), int(k),
                                       0 if radius is None else 1, C.c_double(radius or 0.0),
                                       _p(out, C.c_int64), _p(cnt, C.c_int64),
                                       _p(dims, C.c_int64)))
    res = [out[i * k:i * k + cnt[i]].tolist() for i in range(nq)]
    return res, dims[:dim].tolist()


def duplicate_pair(coords):
    coords = _f64(coords)
    i, j = C.c_int64(), C.c_int64()
    found = lib().or_duplicate_pair(coords.shape[1], len(coords), _p(coords), C.byref(i),
                                    C.byref(j))
    return (i.value, j.value) if found else None


def grid_centers(bmin, bmax, ncell):
    dim = len(ncell)
    nc = np.ascontiguousarray(ncell, dtype=np.int64)
    out = np.zeros(int(np.prod(nc)) * dim)
    _check(lib().or_grid_centers(dim, _p(_f64(bmin)), _p(_f64(bmax)), _p(nc, C.c_int64),
                                 _p(out)))
    return out.reshape(-1, dim)


def krige(coords, values, model, targets, *, method="ordinary", mean=None, degree=1,
          max_neighbors=None, min_neighbors=None, max_per_octant=None, radius=None,
          anisotropic_search=None, drift=None, target_drift=None, measurement_error=None,
          nthreads=None, kcap=0):
    """Kriging::build + predict_many(_with_drift).  Returns a dict with
    value, variance, lagrange, status, and (kcap > 0) neighbour indices."""
    coords, values, targets = _f64(coords), _f64(values), _f64(targets)
    dim = coords.shape[1]
    nt = len(targets)
    n_vars = 0 if drift is None else np.asarray(drift).reshape(len(coords), -1).shape[1]
    if method == "external_drift":
        ctor = 1
    elif measurement_error is not None:
        ctor = 2
    else:
        ctor = 0
    cfg = kcfg_struct(method, mean, degree, n_vars, max_neighbors, min_neighbors,
                      max_per_octant, radius, anisotropic_search)
    m = model_struct(model)
    value, var, lag = np.zeros(nt), np.zeros(nt), np.zeros(nt)
    status = np.zeros(nt, dtype=np.int8)
    nbo = np.zeros(max(nt * kcap, 1), dtype=np.int32) if kcap else None
    nbc = np.zeros(max(nt, 1), dtype=np.int32)
    ties = C.c_int64(0)
    dr = _f64(drift).reshape(-1) if drift is not None else None
    tdr = _f64(target_drift).reshape(-1) if target_drift is not None else None
    me = _f64(measurement_error) if measurement_error is not None else None
    if nthreads is None:
        nthreads = os.cpu_count() or 1
    _check(lib().or_krige(dim, len(coords), _p(coords), _p(values), _p(dr), _p(me), ctor,
                          C.byref(m), C.byref(cfg), nt, _p(targets), _p(tdr), _p(value),
                          _p(var), _p(lag), _p(status, C.c_int8),
                          _p(nbo, C.c_int32) if nbo is not None else None, int(kcap),
                          _p(nbc, C.c_int32), C.byref(ties), int(nthreads)))
    out = dict(value=value, variance=var, lagrange=lag, status=status, nb_count=nbc[:nt],
               boundary_ties=ties.value)
    if kcap:
        out["neighbors"] = nbo[:nt * kcap].reshape(nt, kcap)
    return out


def krige_block(coords, values, model, centers, offsets, *, method="ordinary", mean=None,
                max_neighbors=None, min_neighbors=None, max_per_octant=None, radius=None,
                anisotropic_search=None, measurement_error=None):
    """Kriging::predict_block (kriging.rs:674-779) at each centre."""
    coords, values, centers = _f64(coords), _f64(values), _f64(centers)
    dim = coords.shape[1]
    offsets = _f64(offsets).reshape(-1, dim)
    nc = len(centers)
    cfg = kcfg_struct(method, mean, 1, 0, max_neighbors, min_neighbors, max_per_octant, radius,
                      anisotropic_search)
    m = model_struct(model)
    value, var, lag = np.zeros(nc), np.zeros(nc), np.zeros(nc)
    status = np.zeros(nc, dtype=np.int8)
    me = _f64(measurement_error) if measurement_error is not None else None
    _check(lib().or_krige_block(dim, len(coords), _p(coords), _p(values), _p(me),
                                2 if me is not None else 0, C.byref(m), C.byref(cfg), nc,
                                _p(centers), _p(offsets), len(offsets), _p(value), _p(var),
                                _p(lag), _p(status, C.c_int8)))
    return dict(value=value, variance=var, lagrange=lag, status=status)


def spatial_block_assignment(coords, blocks_per_dim):
    """validation.rs:298-328: the block (fold) index of every point."""
    coords = _f64(coords)
    bpd = np.ascontiguousarray(blocks_per_dim, dtype=np.int64)
    out = np.zeros(len(coords), dtype=np.int64)
    _check(lib().or_spatial_block_assignment(coords.shape[1], len(coords), _p(coords),
                                             _p(bpd, C.c_int64), _p(out, C.c_int64)))
    return out


def maxmin_order(coords):
    coords = _f64(coords)
    out = np.zeros(len(coords), dtype=np.int64)
    _check(lib().or_maxmin_order(coords.shape[1], len(coords), _p(coords), _p(out, C.c_int64)))
    return out


def maxmin_order_brute(coords):
    coords = _f64(coords)
    out = np.zeros(len(coords), dtype=np.int64)
    _check(lib().or_maxmin_order_brute(coords.shape[1], len(coords), _p(coords),
                                       _p(out, C.c_int64)))
    return out


def vecchia_plan(coords, m, order=None):
    coords = _f64(coords)
    n = len(coords)
    o_in = None if order is None else np.ascontiguousarray(order, dtype=np.int64)
    o_out = np.zeros(n, dtype=np.int64)
    nb = np.zeros(n * m, dtype=np.int64)
    cnt = np.zeros(n, dtype=np.int32)
    _check(lib().or_vecchia_plan(coords.shape[1], n, _p(coords), int(m),
                                 _p(o_in, C.c_int64) if o_in is not None else None,
                                 _p(o_out, C.c_int64), _p(nb, C.c_int64), _p(cnt, C.c_int32)))
    return o_out, nb.reshape(n, m), cnt


def vecchia_loglik_plan(coords, values, model, order, nb, cnt, terms=False):
    coords, values = _f64(coords), _f64(values)
    n, m = nb.shape
    ll = C.c_double()
    t = np.zeros(n) if terms else None
    mm = model_struct(model)
    _check(lib().or_vecchia_loglik_plan(coords.shape[1], n, _p(coords), _p(values), C.byref(mm),
                                        m, _p(np.ascontiguousarray(order, np.int64), C.c_int64),
                                        _p(np.ascontiguousarray(nb, np.int64), C.c_int64),
                                        _p(np.ascontiguousarray(cnt, np.int32), C.c_int32),
                                        C.byref(ll), _p(t)))
    return (ll.value, t) if terms else ll.value


def vecchia_loglik_grouped(coords, values, model, order, nb, cnt, group_size):
    """vecchia.rs:604-668 (Guinness grouping over an existing plan)."""
    coords, values = _f64(coords), _f64(values)
    n, m = nb.shape
    ll = C.c_double()
    mm = model_struct(model)
    _check(lib().or_vecchia_loglik_grouped(coords.shape[1], n, _p(coords), _p(values),
                                           C.byref(mm), m,
                                           _p(np.ascontiguousarray(order, np.int64), C.c_int64),
                                           _p(np.ascontiguousarray(nb, np.int64), C.c_int64),
                                           _p(np.ascontiguousarray(cnt, np.int32), C.c_int32),
                                           int(group_size), C.byref(ll)))
    return ll.value


def vecchia_loglik(coords, values, model, m, order=None):
    coords, values = _f64(coords), _f64(values)
    ll = C.c_double()
    mm = model_struct(model)
    o = None if order is None else np.ascontiguousarray(order, dtype=np.int64)
    _check(lib().or_vecchia_loglik(coords.shape[1], len(coords), _p(coords), _p(values),
                                   C.byref(mm), int(m),
                                   _p(o, C.c_int64) if o is not None else None, C.byref(ll)))
    return ll.value


def exact_loglik(coords, values, model):
    coords, values = _f64(coords), _f64(values)
    ll = C.c_double()
    mm = model_struct(model)
    _check(lib().or_exact_loglik(coords.shape[1], len(coords), _p(coords), _p(values),
                                 C.byref(mm), C.byref(ll)))
    return ll.value


def vecchia_predict(coords, values, model, targets, m):
    coords, values, targets = _f64(coords), _f64(values), _f64(targets)
    nt = len(targets)
    v, var = np.zeros(max(nt, 1)), np.zeros(max(nt, 1))
    mm = model_struct(model)
    _check(lib().or_vecchia_predict(coords.shape[1], len(coords), _p(coords), _p(values),
                                    C.byref(mm), nt, _p(targets), int(m), _p(v), _p(var)))
    return v[:nt], var[:nt]


def vecchia_mle_setup(coords, values):
    coords, values = _f64(coords), _f64(values)
    s9 = np.zeros(9)
    rmax = C.c_double()
    _check(lib().or_vecchia_mle_setup(coords.shape[1], len(coords), _p(coords), _p(values),
                                      _p(s9), C.byref(rmax)))
    return s9.reshape(3, 3), rmax.value


def vecchia_mle_objective(coords, values, kind, m, order, nb, cnt, range_max, xs, param=0.0):
    coords, values = _f64(coords), _f64(values)
    xs = _f64(xs).reshape(-1, 3)
    fx = np.zeros(len(xs))
    _check(lib().or_vecchia_mle_objective(
        coords.shape[1], len(coords), _p(coords), _p(values),
        KINDS[kind] if isinstance(kind, str) else int(kind), C.c_double(param), int(m),
        _p(np.ascontiguousarray(order, np.int64), C.c_int64),
        _p(np.ascontiguousarray(nb, np.int64), C.c_int64),
        _p(np.ascontiguousarray(cnt, np.int32), C.c_int32), C.c_double(range_max), len(xs),
        _p(xs), _p(fx)))
    return fx


def vecchia_mle_nm(coords, values, kind, m, starts, step=0.3, max_iter=2000, order=None,
                   param=0.0):
    coords, values = _f64(coords), _f64(values)
    starts = _f64(starts).reshape(-1, 3)
    x = np.zeros(3)
    f = C.c_double()
    ne = C.c_int64()
    o = None if order is None else np.ascontiguousarray(order, dtype=np.int64)
    _check(lib().or_vecchia_mle_nm(
        coords.shape[1], len(coords), _p(coords), _p(values),
        KINDS[kind] if isinstance(kind, str) else int(kind), C.c_double(param), int(m),
        _p(o, C.c_int64) if o is not None else None, len(starts), _p(starts), C.c_double(step),
        int(max_iter), _p(x), C.byref(f), C.byref(ne)))
    return x, f.value, ne.value


def guinness_blocks(order, nb, cnt, group_size):
    """vecchia.rs:577-602: the blocks [(k0, k1), ...] of a plan."""
    n, m = nb.shape
    k1 = np.zeros(n, dtype=np.int64)
    nbk = C.c_int64()
    _check(lib().or_guinness_blocks(n, m, _p(np.ascontiguousarray(order, np.int64), C.c_int64),
                                    _p(np.ascontiguousarray(nb, np.int64), C.c_int64),
                                    _p(np.ascontiguousarray(cnt, np.int32), C.c_int32),
                                    int(group_size), _p(k1, C.c_int64), C.byref(nbk)))
    ends = k1[:nbk.value].tolist()
    return list(zip([0] + ends[:-1], ends))


def poly_basis(coords, degree):
    """vecchia.rs:1181-1233: monomials of the centred, scaled coordinates."""
    coords = _f64(coords)
    p = lib().or_poly_basis_terms(coords.shape[1], int(degree))
    out = np.zeros((len(coords), p))
    _check(lib().or_poly_basis(coords.shape[1], len(coords), _p(coords), int(degree), _p(out)))
    return out


def drift_basis(drift):
    """vecchia.rs:1246-1272: intercept plus standardised covariates."""
    drift = _f64(drift)
    drift = drift.reshape(len(drift), -1)
    out = np.zeros((len(drift), drift.shape[1] + 1))
    _check(lib().or_drift_basis(len(drift), drift.shape[1], _p(drift), _p(out)))
    return out


def vecchia_reml_loglik(coords, values, model, order, nb, cnt, basis, group_size=1):
    """vecchia.rs:1278-1457 on an existing plan (group_size <= 1: ungrouped)."""
    coords, values, basis = _f64(coords), _f64(values), _f64(basis)
    n, m = nb.shape
    ll = C.c_double()
    mm = model_struct(model)
    _check(lib().or_vecchia_reml_loglik(coords.shape[1], n, _p(coords), _p(values), C.byref(mm), m,
                                        _p(np.ascontiguousarray(order, np.int64), C.c_int64),
                                        _p(np.ascontiguousarray(nb, np.int64), C.c_int64),
                                        _p(np.ascontiguousarray(cnt, np.int32), C.c_int32),
                                        _p(basis), basis.shape[1], int(group_size), C.byref(ll)))
    return ll.value


def vecchia_fit_nm(coords, values, kind, m, starts, basis=None, group_size=1, step=0.3,
                   max_iter=2000, order=None):
    """Nelder-Mead multistart: grouped ML (basis None) or REML with `basis`."""
    coords, values = _f64(coords), _f64(values)
    starts = _f64(starts).reshape(-1, 3)
    b = None if basis is None else _f64(basis)
    x = np.zeros(3)
    f = C.c_double()
    ne = C.c_int64()
    o = None if order is None else np.ascontiguousarray(order, dtype=np.int64)
    _check(lib().or_vecchia_fit_nm(
        coords.shape[1], len(coords), _p(coords), _p(values),
        KINDS[kind] if isinstance(kind, str) else int(kind), int(m),
        _p(o, C.c_int64) if o is not None else None, _p(b) if b is not None else None,
        0 if b is None else b.shape[1], int(group_size), len(starts), _p(starts),
        C.c_double(step), int(max_iter), _p(x), C.byref(f), C.byref(ne)))
    return x, f.value, ne.value


def rng_draw(seed, n_uniform, n_normal):
    """One xoshiro256++ stream: n_uniform uniforms, then n_normal normals."""
    out = np.zeros(n_uniform + n_normal)
    lib().or_rng_draw(int(seed), int(n_uniform), int(n_normal), _p(out))
    return out[:n_uniform], out[n_uniform:]


def g_and_dg(kind, d):
    g, dg = C.c_double(), C.c_double()
    rc = lib().or_g_and_dg(KINDS[kind] if isinstance(kind, str) else int(kind), C.c_double(d),
                           C.byref(g), C.byref(dg))
    return (g.value, dg.value) if rc == 0 else None


def vecchia_loglik_grad(coords, values, kind, nugget, psill, rng, order, nb, cnt):
    """loglik_grad_inner (vecchia.rs:428-530): (loglik, [d/dnugget, d/dpsill, d/drange])."""
    coords, values = _f64(coords), _f64(values)
    nb = np.ascontiguousarray(nb, dtype=np.int64)
    ll = C.c_double()
    g = np.zeros(3)
    _check(lib().or_vecchia_loglik_grad(
        coords.shape[1], len(coords), _p(coords), _p(values),
        KINDS[kind] if isinstance(kind, str) else int(kind), C.c_double(nugget), C.c_double(psill),
        C.c_double(rng), nb.shape[1] if nb.ndim == 2 else 1,
        _p(np.ascontiguousarray(order, np.int64), C.c_int64), _p(nb, C.c_int64),
        _p(np.ascontiguousarray(cnt, np.int32), C.c_int32), C.byref(ll), _p(g)))
    return ll.value, g


def vecchia_mle_bfgs(coords, values, kind, m, max_iter=200, order=None):
    """The BFGS path of mle_fit_with_plan (vecchia.rs:1018-1078)."""
    coords, values = _f64(coords), _f64(values)
    x = np.zeros(3)
    f = C.c_double()
    ne = C.c_int64()
    o = None if order is None else np.ascontiguousarray(order, dtype=np.int64)
    _check(lib().or_vecchia_mle_bfgs(
        coords.shape[1], len(coords), _p(coords), _p(values),
        KINDS[kind] if isinstance(kind, str) else int(kind), int(m),
        _p(o, C.c_int64) if o is not None else None, int(max_iter), _p(x), C.byref(f),
        C.byref(ne)))
    return x, f.value, ne.value


def bfgs_multistart(fn, grad, starts, max_iter):
    starts = _f64(starts)
    nstarts, n = starts.shape

    def gcb(xp, nn, gp, ctx):
        g = np.asarray(grad(np.ctypeslib.as_array(xp, shape=(nn,)).copy()), dtype=np.float64)
        for i in range(nn):
            gp[i] = float(g[i])

    cf = _OBJ(lambda xp, nn, ctx: float(fn(np.ctypeslib.as_array(xp, shape=(nn,)).copy())))
    cg = _GRAD(gcb)
    x = np.zeros(n)
    f = C.c_double()
    _check(lib().or_bfgs_multistart(cf, cg, None, n, nstarts, _p(starts), int(max_iter), _p(x),
                                    C.byref(f)))
    return x, f.value


def nelder_mead_multistart(fn, starts, step, max_iter):
    starts = _f64(starts)
    nstarts, n = starts.shape
    cb = _OBJ(lambda xp, nn, ctx: float(fn(np.ctypeslib.as_array(xp, shape=(nn,)).copy())))
    x = np.zeros(n)
    f = C.c_double()
    _check(lib().or_nelder_mead_multistart(cb, None, n, nstarts, _p(starts), C.c_double(step),
                                           int(max_iter), _p(x), C.byref(f)))
    return x, f.value


def rng_u64(seed, count):
    out = np.zeros(count, dtype=np.uint64)
    lib().or_rng_u64(C.c_uint64(seed), count, _p(out, C.c_uint64))
    return out


def rng_uniform(seed, count):
    out = np.zeros(count)
    lib().or_rng_uniform(C.c_uint64(seed), count, _p(out))
    return out


def rng_normal(seed, count):
    out = np.zeros(count)
    lib().or_rng_normal(C.c_uint64(seed), count, _p(out))
    return out


def test_field_2d(n, seed):
    c, v = np.zeros(n * 2), np.zeros(n)
    lib().or_test_field_2d(n, C.c_uint64(seed), _p(c), _p(v))
    return c.reshape(n, 2), v


def test_field_3d(n, seed):
    c, v = np.zeros(n * 3), np.zeros(n)
    lib().or_test_field_3d(n, C.c_uint64(seed), _p(c), _p(v))
    return c.reshape(n, 3), v


# ------------------------------------------------------------ CSV I/O ------
# crates/geostat-cli/src/io_utils.rs, restated with Python's csv module (the
# csv crate's RFC 4180 quoting) and the reference's field rules.  Pure Python:
# the checker for the native reader and writer.
def parse_field(s):
    """io_utils.rs:12-18 parse_field: None for empty / na / nan (any case) or
    text Rust's f64::from_str rejects."""
    import re
    s = s.strip()
    if not s or s.lower() in ("na", "nan"):
        return None
    body = s[1:] if s[:1] in "+-" else s
    if body.lower() in ("inf", "infinity"):
        return float(s[0] + "inf") if s[:1] == "-" else float("inf")
    if not re.fullmatch(r"(\d+\.?\d*|\.\d+)([eE][+-]?\d+)?", body):
        return None
    return float(s)


def csv_read(path, cols):
    """io_utils.rs:37-75: (rows x len(cols) array, skipped count); raises
    KeyError for a missing column."""
    import csv
    with open(path, newline="", encoding="utf-8-sig") as f:
        recs = [r for r in csv.reader(f) if r]
    header = recs[0]
    idx = []
    for c in cols:
        if c not in header:
            raise KeyError(f"column '{c}' not found; available columns: {', '.join(header)}")
        idx.append(header.index(c))
    rows, skipped = [], 0
    for r in recs[1:]:
        if len(r) != len(header):
            raise ValueError("unequal record length")
        vals = [parse_field(r[i]) for i in idx]
        if any(v is None for v in vals):
            skipped += 1
            continue
        rows.append(vals)
    return np.array(rows, dtype=float).reshape(-1, len(cols)), skipped


def rust_display(x):
    """Rust's `{}` for f64: shortest round-trip digits, never an exponent."""
    from decimal import Decimal
    x = float(x)
    if x != x:
        return "NaN"
    if x in (float("inf"), float("-inf")):
        return "inf" if x > 0 else "-inf"
    s = format(Decimal(repr(x)), "f")
    if "." in s:
        s = s.rstrip("0").rstrip(".")
    return s


# ------------------------------------------------- Vecchia parameter SEs ---
def vecchia_param_se(coords, values, kind, nugget, psill, rng, m, order=None):
    """vecchia.rs:1666-1935 vecchia_param_se for a closed-form kind: the
    central difference of the analytical gradient (loglik_grad_with_plan),
    symmetrised; a nugget within one step of zero gives NaN for it and the
    restricted (sill, range) SEs; sqrt of the inverse's diagonal through
    lu_factor / Lu::solve, NaN when singular or non-positive."""
    coords, values = _f64(coords), _f64(values)
    o, nb, cnt = vecchia_plan(coords, m, order)
    theta = [float(nugget), float(psill), float(rng)]
    h = [max(abs(t) * 1e-3, 1e-5) for t in theta]
    free = [1, 2] if theta[0] - h[0] < 0.0 else [0, 1, 2]

    def grad_nll(t):
        _, g = vecchia_loglik_grad(coords, values, kind, t[0], t[1], t[2], o, nb, cnt)
        return [-g[0], -g[1], -g[2]]

    k = len(free)
    hess = np.zeros((k, k))
    for a, i in enumerate(free):
        tp, tm = list(theta), list(theta)
        tp[i] += h[i]
        tm[i] -= h[i]
        gp, gm = grad_nll(tp), grad_nll(tm)
        for b, j in enumerate(free):
            hess[a, b] = (gp[j] - gm[j]) / (2.0 * h[i])
    for a in range(k):
        for b in range(a + 1, k):
            avg = 0.5 * (hess[a, b] + hess[b, a])
            hess[a, b] = hess[b, a] = avg
    se = []
    for col in range(k):
        e = np.zeros(k)
        e[col] = 1.0
        try:
            x = lu_solve(hess, e)
        except OracleError:
            return [float("nan")] * 3
        se.append(float(np.sqrt(x[col])) if x[col] > 0.0 else float("nan"))
    return [float("nan"), se[0], se[1]] if k == 2 else se
