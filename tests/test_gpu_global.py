"""Global neighbourhoods (kriging.rs:396-406): the (n + p) system factored
once on the device at build, each target solved with the factors.

Parity with the oracle's global path (the same algorithm: one lu_factor, then
Lu::solve per target) within the usual tolerance; statuses exact, including a
singular global system and too few points for min_neighbors.
"""
import numpy as np
import pytest

import pyoracle as O
import geostat_rs as G
from geostat_rs.model import Structure, VariogramModel
from gpu_common import assert_close, sph200_model, smooth_values, uniform_points

pytestmark = pytest.mark.gpu


def _check(k, c, v, m, t, okw, tdrift=None, errors=None, drift=None):
    ref = O.krige(c, v, m, t, drift=drift, target_drift=tdrift, measurement_error=errors, **okw)
    for prec in ("mixed", "fp64"):
        out = (k.predict_many_with_drift(t, tdrift, prec, full=True) if tdrift is not None
               else k.predict_many(t, prec, full=True))
        assert ((out.status & 0x3f) == ref["status"].astype(np.uint8)).all()
        assert_close(out.value, ref["value"], float(np.mean(np.abs(v))), 1e-9, "value")
        assert_close(out.variance, ref["variance"], 1e-3 * m.total_sill(), 1e-9, "variance")
        ok = ref["status"] == 0
        if okw.get("method", "ordinary") != "simple":
            assert_close(out.lagrange[ok], ref["lagrange"][ok], 1.0, 1e-9, "lagrange")


@pytest.mark.parametrize("method", ["ordinary", "simple", "universal"])
def test_global_2d_methods(method):
    c = uniform_points(300, 2, 81, [1000.0, 1000.0])
    v = smooth_values(c)
    m = sph200_model()
    cfg = G.KrigingConfig(method, mean=float(np.mean(v)) if method == "simple" else None)
    k = G.Kriging.new(G.PointSet(c, v), m, cfg)
    t = uniform_points(500, 2, 82, [1100.0, 1100.0]) - 50.0
    _check(k, c, v, m, t, dict(method=method, mean=cfg.mean))


def test_global_large_3d_and_drift_and_errors():
    c = uniform_points(1500, 2, 83, [1000.0, 1000.0])
    v = smooth_values(c)
    m = VariogramModel(0.05, [Structure.with_anisotropy("spherical", 0.7, 300.0, 30.0, 0.5),
                              Structure("exponential", 0.3, 500.0)])
    k = G.Kriging.new(G.PointSet(c, v), m)
    t = uniform_points(2000, 2, 84, [1000.0, 1000.0])
    _check(k, c, v, m, t, {})
    c3 = uniform_points(400, 3, 85, [500.0, 500.0, 100.0])
    v3 = smooth_values(c3)
    m3 = VariogramModel(0.05, [Structure.with_rotation("spherical", 0.9, 250.0, 30.0, 10.0, 0.0,
                                                       0.5, 0.3)])
    k3 = G.Kriging.new(G.PointSet(c3, v3), m3)
    _check(k3, c3, v3, m3, uniform_points(300, 3, 86, [500.0, 500.0, 100.0]), {})
    cov = O.rng_uniform(87, 300)
    ck = uniform_points(300, 2, 88, [1000.0, 1000.0])
    vk = smooth_values(ck) + cov
    kk = G.Kriging.with_external_drift(G.PointSet(ck, vk), sph200_model(),
                                       G.KrigingConfig("external_drift", n_vars=1),
                                       cov.reshape(-1, 1))
    tk = uniform_points(200, 2, 89, [1000.0, 1000.0])
    tc = O.rng_uniform(90, 200).reshape(-1, 1)
    _check(kk, ck, vk, sph200_model(), tk, dict(method="external_drift"), tdrift=tc,
           drift=cov.reshape(-1, 1))
    err = 0.05 * O.rng_uniform(91, 300)
    ke = G.Kriging.with_measurement_error(G.PointSet(ck, vk), sph200_model(), G.KrigingConfig(), err)
    _check(ke, ck, vk, sph200_model(), tk, {}, errors=err)


def test_global_singular_and_min_neighbors_validation():
    # universal kriging with every point on one line: the drift block is singular
    x = np.linspace(0.0, 1000.0, 120)
    c = np.stack([x, 2.0 * x + 5.0], 1)
    v = np.sin(x / 100.0)
    m = sph200_model()
    k = G.Kriging.new(G.PointSet(c, v), m, G.KrigingConfig("universal", degree=1))
    t = uniform_points(50, 2, 92, [1000.0, 1000.0])
    ref = O.krige(c, v, m, t, method="universal", degree=1)
    out = k.predict_many(t, full=True)
    assert (out.status & 0x3f == ref["status"].astype(np.uint8)).all()
    assert (ref["status"] == 3).all() and np.isnan(out.value).all()
    # Kriging::build rejects min_neighbors above the number of points
    c2 = uniform_points(100, 2, 93, [1000.0, 1000.0])
    with pytest.raises(G.InsufficientData):
        G.Kriging.new(G.PointSet(c2, smooth_values(c2)), m, G.KrigingConfig(min_neighbors=200))


def test_global_equals_moving_at_k_equals_n():
    # kriging.rs:1570: the factored global system and the moving one at k = n
    c = uniform_points(120, 2, 94, [1000.0, 1000.0])
    v = smooth_values(c)
    m = sph200_model()
    t = uniform_points(300, 2, 95, [1000.0, 1000.0])
    g = G.Kriging.new(G.PointSet(c, v), m).predict_many(t, "fp64", full=True)
    mv = G.Kriging.new(G.PointSet(c, v), m,
                       G.KrigingConfig(max_neighbors=120)).predict_many(t, "fp64", full=True)
    assert np.max(np.abs(g.value - mv.value)) < 1e-10
    assert np.max(np.abs(g.variance - mv.variance)) < 1e-10


def test_global_matrix_form_over_several_target_chunks():
    """The mixed path's matrix-product form takes the targets in chunks (the
    split right-hand sides within 1 GiB: 67 108 targets at 2 001 unknowns);
    70 000 targets span two chunks.  Against the FP64 build (per-target
    solves with the same factors) on every target, and the oracle on a
    sample, statuses exact."""
    c = uniform_points(2000, 2, 96, [1000.0, 1000.0])
    v = smooth_values(c)
    m = sph200_model()
    k = G.Kriging.new(G.PointSet(c, v), m)
    t = uniform_points(70000, 2, 97, [1000.0, 1000.0])
    mixed = k.predict_many(t, "mixed", full=True)
    f64 = k.predict_many(t, "fp64", full=True)
    assert (mixed.status == f64.status).all() and (f64.status == 0).all()
    vs = float(np.mean(np.abs(v)))
    assert_close(mixed.value, f64.value, vs, 1e-9, "value")
    assert_close(mixed.variance, f64.variance, 1e-3 * m.total_sill(), 1e-9, "variance")
    assert_close(mixed.lagrange, f64.lagrange, 1.0, 1e-9, "lagrange")
    sample = np.r_[0:300, 67000:67300, 69700:70000]
    ref = O.krige(c, v, m, t[sample])
    assert_close(mixed.value[sample], ref["value"], vs, 1e-9, "value vs oracle")
    assert_close(mixed.variance[sample], ref["variance"], 1e-3 * m.total_sill(), 1e-9,
                 "variance vs oracle")


def test_global_matrix_form_falls_back_without_room():
    """When the matrix-product form's temporary buffers do not fit (the
    library's next stream-ordered device allocation refused, a host-side fake
    of an exhausted device), the mixed-precision call takes the per-target
    solves with the factors -- the FP64 build's kernel, so the results are
    identical -- and later calls keep doing so.  Device-resident targets, so
    the first allocation of the call is the matrix form's."""
    import torch
    from geostat_rs import _abi
    lib = _abi.load()
    c = uniform_points(300, 2, 98, [1000.0, 1000.0])
    v = smooth_values(c)
    m = sph200_model()
    k = G.Kriging.new(G.PointSet(c, v), m)
    t = uniform_points(400, 2, 99, [1000.0, 1000.0])
    dev = torch.device("cuda")
    tx = torch.from_numpy(np.ascontiguousarray(t[:, 0])).to(dev)
    ty = torch.from_numpy(np.ascontiguousarray(t[:, 1])).to(dev)

    def run(prec):
        val = torch.empty(len(t), dtype=torch.float64, device=dev)
        var = torch.empty_like(val)
        st = torch.empty(len(t), dtype=torch.uint8, device=dev)
        k.predict_device(len(t), tx.data_ptr(), ty.data_ptr(), 0, val.data_ptr(), var.data_ptr(),
                         st.data_ptr(), prec, torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        return val.cpu().numpy(), var.cpu().numpy(), st.cpu().numpy()

    _abi.check(lib.gs_debug_refuse_allocations(1))
    try:
        mixed = run("mixed")
    finally:
        _abi.check(lib.gs_debug_refuse_allocations(0))
    again = run("mixed")
    f64 = run("fp64")
    for out in (mixed, again):
        assert (out[2] == f64[2]).all() and (f64[2] == 0).all()
        assert np.array_equal(out[0], f64[0]) and np.array_equal(out[1], f64[1])


def test_global_small_calls_take_per_target_solves_until_a_large_one():
    """A mixed-precision call of fewer than N / 4 targets does not prepare the
    matrix-product form (its 2 N^3 FMAs would be more than four times the
    call's per-target solves): it takes the per-target solves with the
    factors, the FP64 build's kernel, so its results equal the FP64 call's.
    A call of at least N / 4 targets prepares the form; later small calls
    use it (within the mixed tolerance of the FP64 build)."""
    c = uniform_points(300, 2, 100, [1000.0, 1000.0])
    v = smooth_values(c)
    m = sph200_model()
    k = G.Kriging.new(G.PointSet(c, v), m)
    small = uniform_points(50, 2, 101, [1000.0, 1000.0])
    large = uniform_points(400, 2, 102, [1000.0, 1000.0])
    first = k.predict_many(small, "mixed", full=True)
    f64 = k.predict_many(small, "fp64", full=True)
    assert (first.status == f64.status).all() and (f64.status == 0).all()
    assert np.array_equal(first.value, f64.value)
    assert np.array_equal(first.variance, f64.variance)
    assert np.array_equal(first.lagrange, f64.lagrange)
    big = k.predict_many(large, "mixed", full=True)
    big64 = k.predict_many(large, "fp64", full=True)
    vs = float(np.mean(np.abs(v)))
    assert (big.status == big64.status).all()
    assert_close(big.value, big64.value, vs, 1e-9, "value")
    assert_close(big.variance, big64.variance, 1e-3 * m.total_sill(), 1e-9, "variance")
    again = k.predict_many(small, "mixed", full=True)
    assert (again.status == f64.status).all()
    assert_close(again.value, f64.value, vs, 1e-9, "value")
    assert_close(again.variance, f64.variance, 1e-3 * m.total_sill(), 1e-9, "variance")
    assert_close(again.lagrange, f64.lagrange, 1.0, 1e-9, "lagrange")
