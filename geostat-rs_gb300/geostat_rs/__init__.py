"""geostat_rs -- GB300-native moving-neighbourhood kriging and Vecchia likelihood.

A drop-in for geostat-rs's hot path: the same model format, kriging
configuration and entry points (``krige``, ``krige_grid``, ``krige_3d``,
``vecchia_loglik``, ``vecchia_mle``, ``vecchia_krige`` and the
``PointSet``/``Kriging`` core API), computed by hand-written sm_103a kernels in
libgeostat_gb300.so through its C ABI.
"""
from .errors import (Cancelled, CudaError, DimensionMismatch, DuplicatePoints, GeostatError,
                     InsufficientData, InvalidParameter, IoError, NoNeighbors, OutOfDeviceMemory,
                     SingularSystem)
from .model import Anisotropy, Structure, VariogramModel, parse_kind
from .api import (CvResult, Kriging, KrigingConfig, KrigingResult, PointSet, Server, TuneResult,
                  VecchiaPlan, block_cv, block_offsets, k_fold, krige,
                  krige_3d, krige_grid, loo_cv,
                  last_timings, last_vecchia_tiers, leave_one_out, leave_one_out_with_drift, maxmin_order,
                  tune_kriging_neighbors,
                  nelder_mead_multistart, rng_normal, rng_uniform, seq_mean,
                  vecchia_krige, vecchia_loglik, vecchia_loglik_grouped, vecchia_mle, vecchia_mle_fit,
                  vecchia_mle_grouped_fit, vecchia_mle_nm_fit, vecchia_param_se,
                  vecchia_param_se_fit, vecchia_predict, vecchia_reml,
                  vecchia_reml_drift, vecchia_reml_drift_fit, vecchia_reml_fit)
from . import io  # geostat_rs.gpkg (sqlite3) is imported on use
from ._abi import LIB_PATH, load as load_library

__all__ = [n for n in dir() if not n.startswith("_")]
