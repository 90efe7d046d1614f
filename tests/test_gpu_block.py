"""Block kriging (kriging.rs:674-838) and spatial block cross-validation
(validation.rs:298-374) on the GPU against the oracle.

Block estimates and variances agree with the oracle's predict_block within the
1e-9 parity bar for simple and ordinary kriging over kNN, octant, radius and
global neighbourhoods, with measurement error and in 3-D; predict_block_grid
equals predict_block at the cell centres; block CV equals the oracle's
per-block rebuilds.
"""
import numpy as np
import pytest

import pyoracle as O
import geostat_rs as G
from geostat_rs.model import Structure, VariogramModel
from gpu_common import assert_close, sph200_model, smooth_values, uniform_points

pytestmark = pytest.mark.gpu


def _cfg_kw(cfg):
    return dict(method=cfg.method, mean=cfg.mean, max_neighbors=cfg.max_neighbors,
                max_per_octant=cfg.max_per_octant, radius=cfg.search_radius,
                min_neighbors=cfg.min_neighbors)


@pytest.mark.parametrize("case", ["ok_knn", "sk_knn", "ok_octant", "ok_radius", "ok_global",
                                  "ok_meas_err", "ok_3d"])
def test_block_kriging_matches_oracle(case):
    dim = 3 if case == "ok_3d" else 2
    n = 80 if case == "ok_global" else 3000
    c = uniform_points(n, dim, 301, [1000.0] * dim)
    v = smooth_values(c)
    m = sph200_model()
    cfg = {"ok_knn": G.KrigingConfig(max_neighbors=24),
           "sk_knn": G.KrigingConfig("simple", mean=float(np.mean(v)), max_neighbors=24),
           "ok_octant": G.KrigingConfig(max_per_octant=4),
           "ok_radius": G.KrigingConfig(max_neighbors=32, search_radius=120.0, min_neighbors=3),
           "ok_global": G.KrigingConfig(),
           "ok_meas_err": G.KrigingConfig(max_neighbors=16),
           "ok_3d": G.KrigingConfig(max_neighbors=20)}[case]
    ps = G.PointSet(c, v)
    err = None
    if case == "ok_meas_err":
        err = 0.05 * O.rng_uniform(302, n)
        k = G.Kriging.with_measurement_error(ps, m, cfg, err)
    else:
        k = G.Kriging.new(ps, m, cfg)
    centers = uniform_points(500, dim, 303, [1000.0] * dim)
    centers[:3] = c[:3]  # blocks centred on data points
    if dim == 2:
        off = G.block_offsets([40.0, 25.0], [4, 3])
    else:
        g = (np.arange(3) + 0.5) / 3 - 0.5
        off = np.stack(np.meshgrid(g * 30, g * 30, g * 10, indexing="ij"), -1).reshape(-1, 3)
    r = k.predict_block_many(centers, off, full=True)
    ref = O.krige_block(c, v, m, centers, off, measurement_error=err, **_cfg_kw(cfg))
    assert ((r.status & 0x3f) == ref["status"].astype(np.uint8)).all()
    vs = float(np.mean(np.abs(v)))
    assert_close(r.value, ref["value"], vs, 1e-9, "block value")
    assert_close(r.variance, ref["variance"], 1e-3 * m.total_sill(), 1e-9, "block variance")
    if cfg.method == "ordinary":
        assert_close(r.lagrange, ref["lagrange"], 1e-3 * m.total_sill(), 1e-9, "lagrange")


def test_block_grid_and_single_block_and_errors():
    c = uniform_points(2000, 2, 304, [1000.0, 1000.0])
    v = smooth_values(c)
    m = sph200_model()
    k = G.Kriging.new(G.PointSet(c, v), m, G.KrigingConfig(max_neighbors=16))
    vals, var = k.predict_block_grid([0.0, 0.0], [1000.0, 1000.0], [20, 15], [50.0, 66.0], [3, 5])
    gx = (np.arange(20) + 0.5) * 50.0
    gy = (np.arange(15) + 0.5) * (1000.0 / 15)
    cen = np.stack(np.meshgrid(gx, gy, indexing="xy"), -1).reshape(-1, 2)
    ref = O.krige_block(c, v, m, cen, G.block_offsets([50.0, 66.0], [3, 5]), max_neighbors=16)
    assert_close(vals, ref["value"], float(np.mean(np.abs(v))), 1e-9, "grid value")
    assert_close(var, ref["variance"], 1e-3 * m.total_sill(), 1e-9, "grid variance")
    # the Python binding's krige_grid with block = (w, h)
    v2, _ = G.krige_grid(c[:, 0], c[:, 1], v, m, (0.0, 0.0, 1000.0, 1000.0), 20, 15,
                         max_neighbors=16, block=(50.0, 66.0), block_discr=(3, 5))
    np.testing.assert_array_equal(v2, vals)
    one = k.predict_block(cen[7], G.block_offsets([50.0, 66.0], [3, 5]))
    assert abs(one[0] - vals[7]) <= 1e-12 * abs(vals[7])
    # kriging.rs:1560-1566: drift methods and bad discretisations are rejected
    uk = G.Kriging.new(G.PointSet(c, v), m, G.KrigingConfig("universal", degree=1,
                                                             max_neighbors=16))
    with pytest.raises(G.InvalidParameter):
        uk.predict_block(cen[0], G.block_offsets([1.0, 1.0], [2, 2]))
    vu, varu = uk.predict_block_grid([0.0, 0.0], [1000.0, 1000.0], [4, 4], [50.0, 50.0], [2, 2])
    assert np.isnan(vu).all() and np.isnan(varu).all()
    with pytest.raises(G.InvalidParameter):
        G.block_offsets([0.0, 1.0], [4, 4])
    with pytest.raises(G.InvalidParameter):
        G.block_offsets([1.0, 1.0], [0, 4])
    with pytest.raises(G.InvalidParameter):
        k.predict_block(cen[0], np.zeros((0, 2)))
    # no neighbours within the radius: NoNeighbors, as Kriging::predict_block
    kr = G.Kriging.new(G.PointSet(c, v), m, G.KrigingConfig(max_neighbors=8, search_radius=5.0,
                                                            min_neighbors=2))
    with pytest.raises(G.NoNeighbors):
        kr.predict_block([5000.0, 5000.0], G.block_offsets([1.0, 1.0], [2, 2]))


def test_block_averages_point_predictions_on_device():
    # kriging.rs:1525-1550 with a global neighbourhood
    c = np.array([[0.0, 0.0], [1.0, 0.0], [0.0, 1.0], [1.0, 1.0], [0.4, 0.6]])
    v = np.array([1.0, 2.0, 1.5, 2.5, 1.7])
    m = VariogramModel(0.05, [Structure("spherical", 0.95, 2.0)])
    k = G.Kriging.new(G.PointSet(c, v), m, G.KrigingConfig())
    off = G.block_offsets([0.4, 0.4], [4, 4])
    val, var, _ = k.predict_block([0.6, 0.4], off)
    pts, pvar = k.predict_many(np.array([0.6, 0.4]) + off, "fp64")
    assert abs(val - pts.mean()) < 1e-10
    assert var < k.predict_many(np.array([[0.6, 0.4]]), "fp64")[1][0]


@pytest.mark.parametrize("bpd,cfgname", [((4, 4), "knn"), ((3, 2), "global"), ((5, 5), "octant")])
def test_block_cv_matches_oracle(bpd, cfgname):
    n = 120 if cfgname == "global" else 600
    u, _ = O.rng_draw(7, 2 * n, 0)
    c = u.reshape(n, 2) * 100.0
    v = np.sin(c[:, 0] / 20.0) + np.cos(c[:, 1] / 20.0)
    m = VariogramModel(0.01, [Structure("spherical", 1.0, 50.0)])
    cfg = {"knn": G.KrigingConfig(max_neighbors=16), "global": G.KrigingConfig(),
           "octant": G.KrigingConfig(max_per_octant=3)}[cfgname]
    fold_of = O.spatial_block_assignment(c, bpd)
    pred, var = np.empty(n), np.empty(n)
    for f in np.unique(fold_of):
        tr, te = fold_of != f, fold_of == f
        r = O.krige(c[tr], v[tr], m, c[te], max_neighbors=cfg.max_neighbors,
                    max_per_octant=cfg.max_per_octant)
        pred[te], var[te] = r["value"], r["variance"]
    for prec in ("mixed", "fp64"):
        cv = G.block_cv(G.PointSet(c, v), m, cfg, bpd, precision=prec)
        assert_close(cv.predicted, pred, 1.0, 1e-9, "block cv predicted")
        assert_close(cv.variance, var, 1e-3, 1e-9, "block cv variance")
    assert cv.vecv() > 0.0


def test_block_cv_rejects_bad_config():
    # validation.rs:1100-1110
    u, _ = O.rng_draw(2, 40, 0)
    c = u.reshape(20, 2) * 100.0
    v = np.sin(c[:, 0] / 20.0) + np.cos(c[:, 1] / 20.0)
    m = VariogramModel(0.01, [Structure("spherical", 1.0, 50.0)])
    ps = G.PointSet(c, v)
    with pytest.raises(G.InvalidParameter):
        G.block_cv(ps, m, G.KrigingConfig(), [0, 2])
    with pytest.raises(G.InvalidParameter):
        G.block_cv(ps, m, G.KrigingConfig(), [1, 1])
    G.block_cv(ps, m, G.KrigingConfig(), [3, 3])


def test_csv_end_to_end(tmp_path):
    """io_utils.rs read_points / read_targets / write_estimates_csv around a
    kriging run: the file written is the oracle's estimates, formatted as
    Rust prints them."""
    from geostat_rs import io as gio
    c = uniform_points(1500, 2, 305, [1000.0, 1000.0])
    v = smooth_values(c)
    t = uniform_points(400, 2, 306, [1000.0, 1000.0])
    gio.write_csv(tmp_path / "pts.csv", "east,north,grade", [c[:, 0], c[:, 1], v])
    with open(tmp_path / "tg.csv", "w") as f:
        f.write("x,y\n" + "".join(f"{float(a)!r},{float(b)!r}\n" for a, b in t))
    ps = gio.read_points(tmp_path / "pts.csv", "east", "north", "grade")
    assert np.array_equal(ps.coords, c) and np.array_equal(ps.values, v)
    tg, _ = gio.read_targets(tmp_path / "tg.csv", "x", "y")
    m = sph200_model()
    k = G.Kriging.new(ps, m, G.KrigingConfig(max_neighbors=16))
    val, var = k.predict_many(tg)
    gio.write_estimates_csv(tmp_path / "out.csv", tg, val, var)
    ref = O.krige(c, v, m, t, max_neighbors=16)
    back = gio._read_columns(tmp_path / "out.csv", ["x", "y", "prediction", "variance"], "rows")
    assert np.array_equal(back[:, 0], t[:, 0]) and np.array_equal(back[:, 1], t[:, 1])
    assert_close(back[:, 2], ref["value"], float(np.mean(np.abs(v))), 1e-9, "csv value")
    assert_close(back[:, 3], ref["variance"], 1e-3 * m.total_sill(), 1e-9, "csv variance")
