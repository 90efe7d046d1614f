"""gs_workload -- seeded synthetic workloads and measurement probes.

Used by the benchmark and the tests, not by the library's users: it is not
part of the drop-in library (libgeostat_gb300.so and the geostat_rs package).
Its kernels live in libgeostat_workload.so, built beside the library by
geostat-rs_gb300/build.py and linked against it.

* ``rff_field``: a random-Fourier-feature Gaussian field of a variogram model
  at given points (device), seeded with the reference's xoshiro256++ stream.
* ``clustered_points``: the clustered 2-D layout (Gaussian blobs plus a
  uniform background).
* ``probe_fma_tflops``: sustained CUDA-core FMA throughput, the roofline
  denominator of the per-system kernels.
* ``probe_expneg``: the FP64 re-solve kernels' exp(-x), for accuracy checks.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from geostat_rs import _abi
from geostat_rs.api import model_struct, rng_normal, rng_uniform
from geostat_rs.model import VariogramModel

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libgeostat_workload.so")

_pd = C.POINTER(C.c_double)
SIGNATURES = {
    "gs_synth_rff_field": (C.c_int, [C.c_int, C.c_int64, _pd, _pd, _pd, C.POINTER(_abi.Model),
                                     C.c_int64, C.c_uint64, _pd]),
    "gs_probe_fma_tflops": (C.c_int, [C.c_int, _pd]),
    "gs_probe_expneg": (C.c_int, [C.c_int64, _pd, _pd]),
}

_lib = None


def load():
    """Loads libgeostat_workload.so (after the library it links against)."""
    global _lib
    if _lib is None:
        _abi.load()
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"libgeostat_workload.so not found at {LIB_PATH}: build it with "
                               "`python -c 'import __graft_entry__ as g; g.build()'`")
        lib = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _p(a):
    return None if a is None else a.ctypes.data_as(_pd)


def rff_field(coords, model: VariogramModel, n_features: int, seed: int) -> np.ndarray:
    """Seeded random-Fourier-feature Gaussian field at ``coords`` (device)."""
    c = _f64(coords)
    dim = c.shape[1]
    cols = [_f64(c[:, d]) for d in range(dim)] + ([None] if dim == 2 else [])
    out = np.empty(len(c))
    _abi.check(load().gs_synth_rff_field(dim, len(c), _p(cols[0]), _p(cols[1]), _p(cols[2]),
                                         C.byref(model_struct(model)), int(n_features),
                                         int(seed), _p(out)))
    return out


def clustered_points(n: int, extent: float, n_blobs: int, sigma: float, frac_blobs: float,
                     seed: int) -> np.ndarray:
    """Seeded clustered 2-D layout: ``round(frac_blobs * n)`` points in
    ``n_blobs`` isotropic Gaussian blobs (standard deviation ``sigma``, centres
    uniform in [0, extent]^2, point i in blob i mod n_blobs) followed by the
    rest uniform in [0, extent]^2."""
    nb = int(round(frac_blobs * n))
    cen = rng_uniform(seed, 2 * n_blobs).reshape(n_blobs, 2) * extent
    g = rng_normal(seed + 1, 2 * nb).reshape(nb, 2) * sigma
    pb = cen[np.arange(nb) % n_blobs] + g
    pu = rng_uniform(seed + 2, 2 * (n - nb)).reshape(n - nb, 2) * extent
    return np.vstack([pb, pu])


def probe_fma_tflops(precision: int) -> float:
    """FMA throughput in TFLOP/s: 0 FP32, 1 FP64, 2 packed FP32x2."""
    out = C.c_double()
    _abi.check(load().gs_probe_fma_tflops(int(precision), C.byref(out)))
    return out.value


def probe_expneg(x) -> np.ndarray:
    """exp(-x) as the FP64 re-solve kernels evaluate it (x >= 0)."""
    x = _f64(x)
    out = np.empty_like(x)
    _abi.check(load().gs_probe_expneg(len(x), _p(x), _p(out)))
    return out
