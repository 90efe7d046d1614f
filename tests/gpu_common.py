"""Helpers shared by the GPU parity tests: seeded inputs and the tolerance.

Tolerance (floating point): the CUDA path must agree with the FP64 oracle to
|a - b| <= 1e-9 * max(|b|, floor), where floor is a problem-scale magnitude
(the total sill for variances and log-likelihood terms, the mean absolute
value for estimates) so that quantities that are exactly zero in the oracle
(the kriging variance at a datum) are compared absolutely at 1e-9 * scale.
Integer results (neighbour indices, orders, statuses) must match exactly.
"""
import numpy as np

import pyoracle as O
import geostat_rs as G
from geostat_rs.model import Anisotropy, Structure, VariogramModel

REL_TOL = 1e-9


def max_rel(a, b, floor):
    a, b = np.asarray(a, float), np.asarray(b, float)
    both_nan = np.isnan(a) & np.isnan(b)
    if np.any(np.isnan(a) != np.isnan(b)):
        return np.inf
    d = np.abs(a - b)[~both_nan]
    den = np.maximum(np.abs(b), floor)[~both_nan]
    return float(np.max(d / den)) if d.size else 0.0


def assert_close(a, b, floor, tol=REL_TOL, what=""):
    r = max_rel(a, b, floor)
    assert r <= tol, f"{what}: max rel err {r:.3e} > {tol:.0e}"
    return r


def uniform_points(n, dim, seed, extent):
    u = O.rng_uniform(seed, n * dim).reshape(n, dim)
    return u * np.asarray(extent, float)


def smooth_values(coords, seed=1, nug=0.1):
    """A deterministic smooth field plus seeded noise (test data only)."""
    c = np.asarray(coords, float)
    s = c / (np.max(c, axis=0) + 1.0)
    v = 10.0 + np.sin(6.0 * s[:, 0]) + np.cos(4.0 * s[:, 1])
    if c.shape[1] == 3:
        v = v + 0.5 * np.sin(5.0 * s[:, 2])
    return v + nug * O.rng_normal(seed, len(c))


def clustered_points(n, seed, extent=10000.0, nblobs=50, sigma=15.0, frac=0.7):
    """70% of points in Gaussian blobs, 30% uniform (the clustered layout)."""
    u = O.rng_uniform(seed, 4 * n + 2 * nblobs)
    z = O.rng_normal(seed + 1, 2 * n)
    centres = u[:2 * nblobs].reshape(nblobs, 2) * extent
    nb = int(frac * n)
    which = (u[2 * nblobs:2 * nblobs + nb] * nblobs).astype(int)
    blob = centres[which] + sigma * z[:2 * nb].reshape(nb, 2)
    rest = u[2 * nblobs + nb:2 * nblobs + nb + 2 * (n - nb)].reshape(n - nb, 2) * extent
    pts = np.concatenate([blob, rest])
    return np.clip(pts, 0.0, extent)


def sph200_model():
    """Nugget 0.1 + spherical (sill 1, range 200 m): the 2-D 2,000-point workload's model."""
    return VariogramModel(0.1, [Structure("spherical", 1.0, 200.0)])


def rotated_3d_model():
    """The 3-D workload's model: nugget 0.05 + rotated spherical + exponential."""
    return VariogramModel(0.05, [Structure.with_rotation("spherical", 0.6, 300.0, 30.0, 10.0, 0.0,
                                                         0.5, 40.0 / 300.0),
                                 Structure("exponential", 0.35, 800.0)])


def clustered_matern_model():
    """The clustered workload's model: Matern 3/2, range 500 m, ratio 0.5 at 45 degrees."""
    return VariogramModel(0.0, [Structure.with_anisotropy("matern15", 1.0, 500.0, 45.0, 0.5)])
