"""The clustered uneven workload at reduced size, and the launch-shape tuner.

Data density matches the full workload (1,000,000 points over 10 km x 10 km,
70 % in 500 Gaussian blobs of sigma 15 m): 100,000 points over 3.16 km x
3.16 km with 50 blobs.  Matern 3/2 (range 500 m, ratio 0.5 at 45 degrees, no
nugget) makes most systems too ill-conditioned for the FP32 factorisation, so
this is the FP64 re-solve's workload.  Ordinary, universal (linear drift) and
external-drift kriging with octant search (4 x 16, at most 64, at least 4)
must match the oracle within 1e-9 with bit-exact neighbour sets and statuses.
"""
import numpy as np
import pytest

import pyoracle as O
import geostat_rs as G
import gs_workload as W
from gpu_common import assert_close, clustered_matern_model, clustered_points

pytestmark = pytest.mark.gpu

EXTENT = 3162.3
SEARCH = dict(max_per_octant=16, max_neighbors=64, min_neighbors=4)


def _data():
    c = clustered_points(100_000, 41, extent=EXTENT, nblobs=50)
    m = clustered_matern_model()
    v = W.rff_field(c, m, 1024, 42)
    cov = O.rng_uniform(43, len(c))
    g = (np.arange(36) + 0.5) * (EXTENT / 36)
    yy, xx = np.meshgrid(g, g, indexing="ij")
    grid = np.stack([xx.ravel(), yy.ravel()], 1)
    # targets in the blobs' cores, where the systems are densest
    u = O.rng_uniform(44, 2 * 50 + 400)
    centres = u[:100].reshape(50, 2) * EXTENT
    near = centres[np.arange(200) % 50] + (u[100:].reshape(200, 2) - 0.5) * 20.0
    # beyond the corners and edges: one or two octants only
    out = np.array([[-60.0, -60.0], [EXTENT + 60, -60.0], [-60.0, EXTENT + 60],
                    [EXTENT + 60, EXTENT + 60], [EXTENT / 2, -40.0], [-40.0, EXTENT / 3]])
    t = np.concatenate([grid, near, out])
    tcov = O.rng_uniform(45, len(t))
    return c, v, m, cov, t, tcov


@pytest.fixture(scope="module")
def data():
    return _data()


def _predictor(kind, c, v, m, cov):
    ps = G.PointSet(c, v)
    if kind == "ordinary":
        return G.Kriging.new(ps, m, G.KrigingConfig(**SEARCH))
    if kind == "universal":
        return G.Kriging.new(ps, m, G.KrigingConfig("universal", degree=1, **SEARCH))
    return G.Kriging.with_external_drift(ps, m, G.KrigingConfig("external_drift", n_vars=1,
                                                                **SEARCH), cov.reshape(-1, 1))


def _predict(k, kind, t, tcov, prec):
    if kind == "external_drift":
        return k.predict_many_with_drift(t, tcov.reshape(-1, 1), prec, full=True)
    return k.predict_many(t, prec, full=True)


@pytest.mark.parametrize("kind", ["ordinary", "universal", "external_drift"])
def test_clustered_kinds_match_oracle(data, kind):
    c, v, m, cov, t, tcov = data
    k = _predictor(kind, c, v, m, cov)
    ref = O.krige(c, v, m, t, method=kind, degree=1,
                  drift=cov.reshape(-1, 1) if kind == "external_drift" else None,
                  target_drift=tcov.reshape(-1, 1) if kind == "external_drift" else None,
                  kcap=64, **SEARCH)
    nb, cnt = k.neighbors(t, 64)
    assert (cnt == ref["nb_count"]).all()
    assert (nb == ref["neighbors"]).all()
    assert cnt.min() < 32 < cnt.max()  # both solver widths
    vs = float(np.mean(np.abs(v)))
    for prec in ("mixed", "fp64"):
        out = _predict(k, kind, t, tcov, prec)
        assert ((out.status & 0x3f) == ref["status"].astype(np.uint8)).all()
        assert_close(out.value, ref["value"], vs, 1e-9, f"{kind} {prec} value")
        assert_close(out.variance, ref["variance"], 1e-3, 1e-9, f"{kind} {prec} variance")


def test_tuner_and_pinned_shapes(data):
    c, v, m, cov, _, _ = data
    k = _predictor("ordinary", c, v, m, cov)
    nt = 70_000  # above the tuning threshold
    t = np.random.default_rng(5).uniform(0, EXTENT, size=(nt, 2))
    assert k.tiles(nt)[3] == "default"
    base = k.predict_many(t, "mixed", full=True)
    run, bins, spc, src = k.tiles(nt)
    assert src == "tuned" and run in (16, 32, 64, 128) and bins in (0, 1) and spc in (1, 2)
    again = k.predict_many(t, "mixed", full=True)
    # the tuned shape is kept: identical results
    np.testing.assert_array_equal(again.value, base.value)
    np.testing.assert_array_equal(again.variance, base.variance)
    vs = float(np.mean(np.abs(v)))
    for run, bins, spc in ((8, 0, 1), (128, 1, 2), (1, 1, 1), (32, 0, 2)):
        k.set_tiles(run, bins, spc)
        assert k.tiles(nt) == (run, bins, spc, "pinned")
        out = k.predict_many(t, "mixed", full=True)
        assert ((out.status & 0x3f) == (base.status & 0x3f)).all()
        assert_close(out.value, base.value, vs, 1e-9, f"run {run} bins {bins} spc {spc}")
        assert_close(out.variance, base.variance, 1e-3, 1e-9, f"run {run} bins {bins} spc {spc}")
    k.set_tiles(0)
    assert k.tiles(nt)[3] == "tuned"
    with pytest.raises(G.InvalidParameter):
        k.set_tiles(48)
    with pytest.raises(G.InvalidParameter):
        k.set_tiles(32, 0, 3)
    # an oracle check on a slice of the tuned call
    ref = O.krige(c, v, m, t[:600], **SEARCH)
    assert_close(base.value[:600], ref["value"], vs, 1e-9, "tuned value")


@pytest.mark.parametrize("kind", ["ordinary", "universal", "external_drift"])
def test_clustered_mixed_matches_fp64_build_at_scale(data, kind):
    """300,000 targets, half in the blobs' cores: the mixed path (FP32 attempt,
    routing, FP64 LDL^T and LU re-solves) against the plain FP64 build, whose
    agreement with the oracle the test above pins."""
    c, v, m, cov, _, _ = data
    k = _predictor(kind, c, v, m, cov)
    u = O.rng_uniform(46, 2 * 50 + 4 * 150_000)
    centres = u[:100].reshape(50, 2) * EXTENT
    near = centres[np.arange(150_000) % 50] + (u[100:300_100].reshape(-1, 2) - 0.5) * 60.0
    far = u[300_100:600_100].reshape(-1, 2) * EXTENT
    t = np.concatenate([near, far])
    tcov = O.rng_uniform(47, len(t))
    mixed = _predict(k, kind, t, tcov, "mixed")
    plain = _predict(k, kind, t, tcov, "fp64")
    assert ((mixed.status & 0x3f) == (plain.status & 0x3f)).all()
    vs = float(np.mean(np.abs(v)))
    assert_close(mixed.value, plain.value, vs, 1e-9, f"{kind} value")
    assert_close(mixed.variance, plain.variance, 1e-3, 1e-9, f"{kind} variance")


# ------------------------------------------------- the full-size workload --
FULL_EXTENT = 10000.0
FULL_GRID = 2048


@pytest.fixture(scope="module")
def full_data():
    """1,000,000 points over 10 km x 10 km, 70 % in 500 blobs of sigma 15 m;
    Matern 3/2 field; one U[0,1] covariate; the 2048 x 2048 grid."""
    c = W.clustered_points(1_000_000, FULL_EXTENT, 500, 15.0, 0.7, 61)
    m = clustered_matern_model()
    v = W.rff_field(c, m, 1024, 62)
    cov = O.rng_uniform(63, len(c))
    centres = O.rng_uniform(61, 2 * 500).reshape(500, 2) * FULL_EXTENT
    return c, v, m, cov, centres


@pytest.mark.parametrize("kind,row0", [("ordinary", 300), ("universal", 1000),
                                        ("external_drift", 1700)])
def test_clustered_full_size_matches_oracle_on_a_sample(full_data, kind, row0):
    """One band of 32 grid rows (65,536 targets) per kind through the whole
    pass (search, FP32 attempt, routing, FP64 re-solves), checked against the
    oracle on 150 random targets of the band and the 50 targets closest to a
    blob centre, at both precisions."""
    c, v, m, cov, centres = full_data
    k = _predictor(kind, c, v, m, cov)
    g = (np.arange(FULL_GRID) + 0.5) * (FULL_EXTENT / FULL_GRID)
    yy, xx = np.meshgrid(g[row0:row0 + 32], g, indexing="ij")
    t = np.stack([xx.ravel(), yy.ravel()], 1)
    tcov = O.rng_uniform(64 + row0, len(t))
    pick = np.random.default_rng(row0).choice(len(t), 150, replace=False)
    from scipy.spatial import cKDTree
    dmin = cKDTree(centres).query(t)[0]
    core = np.argsort(dmin, kind="stable")[:50]
    idx = np.unique(np.concatenate([pick, core]))
    ref = O.krige(c, v, m, t[idx], method=kind, degree=1,
                  drift=cov.reshape(-1, 1) if kind == "external_drift" else None,
                  target_drift=tcov[idx].reshape(-1, 1) if kind == "external_drift" else None,
                  **SEARCH)
    vs = float(np.mean(np.abs(v)))
    for prec in ("mixed", "fp64"):
        out = _predict(k, kind, t, tcov, prec)
        if prec == "mixed":
            assert ((out.status & 0x40) != 0).mean() > 0.5  # mostly the FP64 re-solve tiers
        assert ((out.status[idx] & 0x3f) == ref["status"].astype(np.uint8)).all()
        assert_close(out.value[idx], ref["value"], vs, 1e-9, f"{kind} {prec} value")
        assert_close(out.variance[idx], ref["variance"], 1e-3, 1e-9, f"{kind} {prec} variance")
