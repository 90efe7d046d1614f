"""ctypes binding of libgeostat_gb300.so (include/geostat_gb300.h).

The library is loaded from this package's ``_lib`` directory (built in-tree
by ``geostat-rs_gb300/build.py``).  There is no fallback: if the library is
missing every call raises, so a silent CPU path can never stand in for the
CUDA one.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libgeostat_gb300.so")

# Return codes (GS_ERR_*) and per-target status bits (GS_ST_*).
OK = 0
ST_OK, ST_INSUFFICIENT_DATA, ST_SINGULAR, ST_NO_NEIGHBORS, ST_CAPACITY = 0, 1, 3, 5, 7
ST_FP64_RESOLVED = 0x40
PREC_MIXED, PREC_FP64 = 0, 1
METHODS = {"simple": 0, "ordinary": 1, "universal": 2, "external_drift": 3}


class Structure(C.Structure):
    _fields_ = [("kind", C.c_int32), ("has_anis", C.c_int32), ("param", C.c_double),
                ("sill", C.c_double), ("range", C.c_double), ("azimuth_deg", C.c_double),
                ("ratio", C.c_double), ("ratio_z", C.c_double), ("dip_deg", C.c_double),
                ("rake_deg", C.c_double)]


class Model(C.Structure):
    _fields_ = [("nugget", C.c_double), ("n_structures", C.c_int32), ("pad_", C.c_int32),
                ("s", Structure * 4)]


class Kcfg(C.Structure):
    _fields_ = [("method", C.c_int64), ("sk_mean", C.c_double), ("uk_degree", C.c_int64),
                ("ked_nvars", C.c_int64), ("max_neighbors", C.c_int64),
                ("min_neighbors", C.c_int64), ("max_per_octant", C.c_int64),
                ("has_search_radius", C.c_int64), ("search_radius", C.c_double),
                ("has_anisotropic_search", C.c_int64), ("search_azimuth_deg", C.c_double),
                ("search_ratio", C.c_double), ("search_ratio_z", C.c_double),
                ("search_dip_deg", C.c_double), ("search_rake_deg", C.c_double)]


OBJECTIVE = C.CFUNCTYPE(C.c_double, C.POINTER(C.c_double), C.c_int64, C.c_void_p)

_d, _i32, _i64, _u64, _vp, _int = C.c_double, C.c_int32, C.c_int64, C.c_uint64, C.c_void_p, C.c_int
_pd = C.POINTER(C.c_double)
_pi32 = C.POINTER(C.c_int32)
_pi64 = C.POINTER(C.c_int64)
_pu8 = C.POINTER(C.c_uint8)
_pm = C.POINTER(Model)
_pk = C.POINTER(Kcfg)
_pps = C.c_void_p

# name -> (restype, argtypes); the single source of truth for the exports
SIGNATURES = {
    "gs_last_error": (C.c_char_p, []),
    "gs_abi_version": (_int, []),
    "gs_pointset_create": (_int, [_int, _i64, _pd, _pd, _pd, _pd, C.POINTER(_vp)]),
    "gs_pointset_destroy": (None, [_vp]),
    "gs_pointset_duplicate_pair": (_int, [_vp, _pi64, _pi64]),
    "gs_kriging_new": (_int, [_vp, _pm, _pk, C.POINTER(_vp)]),
    "gs_kriging_with_external_drift": (_int, [_vp, _pm, _pk, _pd, C.POINTER(_vp)]),
    "gs_kriging_with_measurement_error": (_int, [_vp, _pm, _pk, _pd, C.POINTER(_vp)]),
    "gs_kriging_destroy": (None, [_vp]),
    "gs_kriging_predict_many": (_int, [_vp, _i64, _pd, _pd, _pd, _pd, _pd, _pd, _pd, _pu8, _int,
                                       _vp]),
    "gs_kriging_predict_many_device": (_int, [_vp, _i64, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                                              _int, _vp]),
    "gs_kriging_predict_many_async": (_int, [_vp, _i64, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                                             _int, _vp]),
    "gs_kriging_cross_validate": (_int, [_vp, _i64, C.c_uint64, _pd, _pd, _pu8, _int]),
    "gs_kriging_set_tiles": (_int, [_vp, _int, _int, _int]),
    "gs_kriging_tiles": (_int, [_vp, _i64, _pi32, _pi32, _pi32, _pi32]),
    "gs_kriging_predict_fp64_noalloc": (_int, [_vp, _i64, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                                               _vp, _vp]),
    "gs_last_fallbacks": (_i64, []),
    "gs_last_fit_rounds": (_i64, []),
    "gs_last_vecchia_tiers": (None, [_pi64]),
    "gs_debug_device_allocations": (_i64, []),
    "gs_debug_refuse_allocations": (_int, [_i64]),
    "gs_last_lu_resolves": (_i64, []),
    "gs_server_create": (_int, [_i64, _i32, C.POINTER(_vp)]),
    "gs_server_add_kriging": (_int, [_vp, _vp, _pi32]),
    "gs_server_add_vecchia": (_int, [_vp, _vp, _pi32]),
    "gs_server_submit_predict": (_int, [_vp, _i32, _i64, _pd, _pd, _pd, _pd, _pd, _pu8, _pi64]),
    "gs_server_submit_loglik": (_int, [_vp, _i32, _pm, _pd, _pi32, _pi64]),
    "gs_server_cancel": (_int, [_vp, _i64]),
    "gs_server_wait": (_int, [_vp, _i64, _pd]),
    "gs_server_set_precision": (_int, [_vp, _int]),
    "gs_server_stats": (_int, [_vp, _pd, _pd, _pi64, _pi64]),
    "gs_server_destroy": (None, [_vp]),
    "gs_kriging_predict_grid": (_int, [_vp, _pd, _pd, _pi64, _pd, _pd, _pu8, _int, _vp]),
    "gs_kriging_neighbors": (_int, [_vp, _i64, _pd, _pd, _pd, _i64, _pi32, _pi32, _vp]),
    "gs_maxmin_order": (_int, [_int, _i64, _pd, _pd, _pd, _pi64]),
    "gs_vecchia_plan_create": (_int, [_vp, _i64, _pi64, C.POINTER(_vp)]),
    "gs_vecchia_plan_get": (_int, [_vp, _pi64, _pi64, _pi32]),
    "gs_vecchia_plan_destroy": (None, [_vp]),
    "gs_vecchia_loglik_batch": (_int, [_vp, _i64, _pm, _pd, _pi32, _int, _vp]),
    "gs_vecchia_loglik_batch_range": (_int, [_vp, _i64, _i64, _i64, _pm, _pd, _pi32, _int, _vp]),
    "gs_vecchia_loglik_grouped_batch": (_int, [_vp, _i64, _pm, _i64, _pd, _pi32, _vp]),
    "gs_vecchia_loglik": (_int, [_vp, _pm, _i64, _pi64, _pd]),
    "gs_vecchia_mle": (_int, [_vp, _i32, _i64, _pi64, _pm, _pd, _pd, _pi64]),
    "gs_vecchia_mle_nm": (_int, [_vp, _i32, _i64, _pi64, _i64, _pd, _d, _i64, _pm, _pd, _pd, _pi64]),
    "gs_vecchia_loglik_grad_batch": (_int, [_vp, _i64, _pm, _pd, _pd, _pi32, _int, _vp]),
    "gs_csv_read": (_int, [C.c_char_p, C.POINTER(C.c_char_p), _int, _int, C.POINTER(_vp)]),
    "gs_csv_table_info": (_int, [_vp, _pi64, _pi64]),
    "gs_csv_table_copy": (_int, [_vp, _pd]),
    "gs_csv_table_destroy": (None, [_vp]),
    "gs_csv_write": (_int, [C.c_char_p, C.c_char_p, _int, C.POINTER(_pd), _i64, _int]),
    "gs_kriging_block_cv": (_int, [_vp, _pi64, _pd, _pd, _pu8, _int]),
    "gs_block_offsets": (_int, [_pd, _pi64, _pd]),
    "gs_kriging_predict_block": (_int, [_vp, _i64, _pd, _pd, _pd, _pd, _i64, _pd, _pd, _pd, _pu8,
                                        _vp]),
    "gs_kriging_predict_block_grid": (_int, [_vp, _pd, _pd, _pi64, _pd, _pi64, _pd, _pd, _pu8,
                                             _vp]),
    "gs_vecchia_reml_loglik_batch": (_int, [_vp, _i64, _pm, _i32, _pd, _i64, _i64, _pd, _pi32,
                                            _vp]),
    "gs_vecchia_mle_grouped": (_int, [_vp, _i32, _i64, _pi64, _i64, _pm, _pd, _pd, _pi64]),
    "gs_vecchia_reml": (_int, [_vp, _i32, _i64, _i32, _pi64, _i64, _pm, _pd, _pd, _pi64]),
    "gs_vecchia_reml_drift": (_int, [_vp, _i32, _i64, _pd, _i64, _i64, _pi64, _i64, _pm, _pd, _pd,
                                     _pi64]),
    "gs_vecchia_predict": (_int, [_vp, _pm, _i64, _pd, _pd, _pd, _i64, _pd, _pd]),
    "gs_nelder_mead_multistart": (_int, [OBJECTIVE, _vp, _i64, _i64, _pd, _d, _i64, _pd, _pd]),
    "gs_rng_uniform": (None, [_u64, _i64, _pd]),
    "gs_rng_normal": (None, [_u64, _i64, _pd]),
    "gs_last_timings": (_int, [_pd]),
    "gs_launch_count": (_i64, []),
}

_lib = None


def load():
    """Loads the library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"libgeostat_gb300.so not found at {LIB_PATH}: build it with "
                "`python -c 'import __graft_entry__ as g; g.build()'`")
        lib = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def check(rc: int):
    if rc != 0:
        from .errors import raise_for
        raise_for(rc, load().gs_last_error().decode())
