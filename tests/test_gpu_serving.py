"""Serving loop: every result is the same alone and in the mix.

Prediction and log-likelihood requests of very different sizes are submitted
concurrently from several host threads to a server holding three resident data
sets; each result is compared with the same request run alone through the
direct entry points: estimates and variances within the parity tolerance
(the solves do not depend on the batch beyond the order of roundings),
statuses exactly, log-likelihoods bit for bit (computed per candidate in a
fixed order).
"""
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

import pyoracle as O
import geostat_rs as G
import gs_workload as W
from geostat_rs.model import Structure, VariogramModel
from gpu_common import assert_close, uniform_points

pytestmark = pytest.mark.gpu


def test_mixed_requests_match_their_results_alone():
    m2 = VariogramModel(0.05, [Structure.with_anisotropy("spherical", 0.7, 150.0, 30.0, 0.5),
                               Structure("exponential", 0.25, 400.0)])
    c2 = uniform_points(20000, 2, 501, [1000.0, 1000.0])
    v2 = 10.0 + W.rff_field(c2, m2, 512, 5)
    k2 = G.Kriging.new(G.PointSet(c2, v2), m2, G.KrigingConfig(max_neighbors=32))
    m3 = VariogramModel(0.05, [Structure.with_rotation("spherical", 0.9, 300.0, 30.0, 10.0, 0.0,
                                                       0.5, 0.2)])
    c3 = uniform_points(10000, 3, 502, [1000.0, 1000.0, 200.0])
    v3 = W.rff_field(c3, m3, 512, 6)
    k3 = G.Kriging.new(G.PointSet(c3, v3), m3, G.KrigingConfig(max_neighbors=24))
    # a second 2-D set with another neighbour count and frame count: its
    # launches use other shared-memory sizes of the same kernels
    mi = VariogramModel(0.1, [Structure("exponential", 1.0, 150.0)])
    ci = uniform_points(15000, 2, 505, [1000.0, 1000.0])
    vi = 5.0 + W.rff_field(ci, mi, 512, 8)
    ki = G.Kriging.new(G.PointSet(ci, vi), mi, G.KrigingConfig(max_neighbors=48))
    cv, vv = O.test_field_2d(5000, 503)
    plan = G.VecchiaPlan(G.PointSet(cv, vv), 20)

    srv = G.Server(mem_budget_bytes=1 << 30, executors=3)
    d2, d3, dv = srv.add_kriging(k2), srv.add_kriging(k3), srv.add_vecchia(plan)
    di = srv.add_kriging(ki)

    rng = np.random.default_rng(7)
    jobs = []
    for q in range(36):
        if q % 4 == 3:
            mdl = VariogramModel(0.05 + 0.01 * q, [Structure("exponential", 0.9, 20.0 + q)])
            jobs.append(("ll", dv, mdl))
        else:
            nt = int(np.exp(rng.uniform(0.0, np.log(30000))))
            if q % 6 == 0:
                jobs.append(("p", di, rng.uniform(0, 1000, size=(nt, 2))))
            elif q % 2 == 0:
                jobs.append(("p", d2, rng.uniform(0, 1000, size=(nt, 2))))
            else:
                jobs.append(("p", d3, rng.uniform(0, 1, size=(nt, 3)) * [1000.0, 1000.0, 200.0]))

    def submit(job):
        kind, ds, arg = job
        return srv.submit_predict(ds, arg) if kind == "p" else srv.submit_loglik(ds, arg)

    with ThreadPoolExecutor(4) as ex:
        reqs = list(ex.map(submit, jobs))
    for r in reqs:
        assert srv.wait(r) >= 0.0
    p50, p99, done, launches = srv.stats()
    assert done == len(jobs) and 0 < p50 <= p99 and 1 <= launches <= len(jobs)

    for (kind, ds, arg), r in zip(jobs, reqs):
        if kind == "ll":
            alone, st = plan.loglik([arg])
            assert r.out[1][0] == st[0] == 0
            assert r.out[0][0] == alone[0]
        else:
            k, vals, sill = {d2: (k2, v2, 1.0), d3: (k3, v3, 0.95), di: (ki, vi, 1.1)}[ds]
            alone = k.predict_many(arg, "mixed", full=True)
            v, var, st = r.out
            assert (st == alone.status).all()
            assert_close(v, alone.value, float(np.mean(np.abs(vals))), 1e-9, "value")
            assert_close(var, alone.variance, sill, 1e-9, "variance")
    srv.close()


def test_server_rejects_bad_requests():
    c = uniform_points(500, 2, 504, [1.0, 1.0])
    k = G.Kriging.new(G.PointSet(c, c[:, 0].copy()), VariogramModel(0.0, [Structure("exponential", 1.0, 0.3)]),
                      G.KrigingConfig(max_neighbors=8))
    srv = G.Server(mem_budget_bytes=1 << 28, executors=1)
    d = srv.add_kriging(k)
    with pytest.raises(G.InvalidParameter):
        srv.submit_predict(d + 5, np.zeros((3, 2)))
    with pytest.raises(G.InvalidParameter):
        srv.submit_loglik(d, VariogramModel(0.0, [Structure("exponential", 1.0, 0.3)]))
    r = srv.submit_predict(d, np.full((4, 2), 0.5))
    srv.wait(r)
    assert np.isfinite(r.out[0]).all()
    srv.close()


def _small_server_set():
    c = uniform_points(20000, 2, 511, [1000.0, 1000.0])
    m = VariogramModel(0.1, [Structure("exponential", 1.0, 150.0)])
    k = G.Kriging.new(G.PointSet(c, 5.0 + W.rff_field(c, m, 256, 512)), m,
                      G.KrigingConfig(max_neighbors=32))
    return k


def test_server_refuses_requests_beyond_its_budget():
    """A request whose device bytes exceed the budget is refused at submission
    with a clean error; the server keeps serving."""
    k = _small_server_set()
    srv = G.Server(mem_budget_bytes=64 << 20, executors=2)
    d = srv.add_kriging(k)
    rng = np.random.default_rng(3)
    with pytest.raises(G.OutOfDeviceMemory, match="more than the server's budget"):
        srv.submit_predict(d, rng.uniform(0, 1000, size=(1_000_000, 2)))
    r = srv.submit_predict(d, rng.uniform(0, 1000, size=(1000, 2)))
    srv.wait(r)
    assert np.isfinite(r.out[0]).all()
    srv.close()


def test_server_survives_a_refused_device_allocation():
    """The library's next device allocation is refused (a host-side fake of an
    exhausted device): the request it belonged to fails with
    OutOfDeviceMemory, and later requests are served normally."""
    from geostat_rs import _abi
    k = _small_server_set()
    srv = G.Server(mem_budget_bytes=1 << 30, executors=1)
    d = srv.add_kriging(k)
    t = np.random.default_rng(4).uniform(0, 1000, size=(5000, 2))
    lib = _abi.load()
    _abi.check(lib.gs_debug_refuse_allocations(1))
    try:
        r = srv.submit_predict(d, t)
        with pytest.raises(G.OutOfDeviceMemory, match="refused on request"):
            srv.wait(r)
    finally:
        _abi.check(lib.gs_debug_refuse_allocations(0))
    r2 = srv.submit_predict(d, t)
    srv.wait(r2)
    alone = k.predict_many(t, "mixed", full=True)
    assert (r2.out[2] == alone.status).all()
    assert_close(r2.out[0], alone.value, 5.0, 1e-9, "value after a refused allocation")
    assert srv.stats()[2] == 2
    srv.close()


def test_server_cancels_pending_requests_only():
    """With one executor busy on a large request, a request behind it can be
    cancelled (its wait raises Cancelled); a finished one cannot."""
    k = _small_server_set()
    srv = G.Server(mem_budget_bytes=8 << 30, executors=1)
    d = srv.add_kriging(k)
    rng = np.random.default_rng(5)
    big = srv.submit_predict(d, rng.uniform(0, 1000, size=(1_000_000, 2)))
    small = srv.submit_predict(d, rng.uniform(0, 1000, size=(100, 2)))
    srv.cancel(small)
    with pytest.raises(G.Cancelled):
        srv.wait(small)
    srv.wait(big)
    assert np.isfinite(big.out[0]).all()
    done = srv.submit_predict(d, rng.uniform(0, 1000, size=(10, 2)))
    srv.wait(done)
    with pytest.raises(G.InvalidParameter):
        srv.cancel(done)  # finished and already waited for: unknown
    srv.close()


def test_small_requests_do_not_wait_behind_large_ones():
    """Two executors: the large lane takes a 1,000,000-target request, the
    small lane serves the small requests submitted after it, which finish
    first."""
    k = _small_server_set()
    srv = G.Server(mem_budget_bytes=8 << 30, executors=2)
    d = srv.add_kriging(k)
    rng = np.random.default_rng(6)
    big = srv.submit_predict(d, rng.uniform(0, 1000, size=(1_000_000, 2)))
    smalls = [srv.submit_predict(d, rng.uniform(0, 1000, size=(200, 2))) for _ in range(5)]
    lat_small = [srv.wait(r) for r in smalls]
    lat_big = srv.wait(big)
    assert max(lat_small) < lat_big
    srv.close()
