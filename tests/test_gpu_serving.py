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
from geostat_rs.model import Structure, VariogramModel
from gpu_common import assert_close, uniform_points

pytestmark = pytest.mark.gpu


def test_mixed_requests_match_their_results_alone():
    m2 = VariogramModel(0.05, [Structure.with_anisotropy("spherical", 0.7, 150.0, 30.0, 0.5),
                               Structure("exponential", 0.25, 400.0)])
    c2 = uniform_points(20000, 2, 501, [1000.0, 1000.0])
    v2 = 10.0 + G.rff_field(c2, m2, 512, 5)
    k2 = G.Kriging.new(G.PointSet(c2, v2), m2, G.KrigingConfig(max_neighbors=32))
    m3 = VariogramModel(0.05, [Structure.with_rotation("spherical", 0.9, 300.0, 30.0, 10.0, 0.0,
                                                       0.5, 0.2)])
    c3 = uniform_points(10000, 3, 502, [1000.0, 1000.0, 200.0])
    v3 = G.rff_field(c3, m3, 512, 6)
    k3 = G.Kriging.new(G.PointSet(c3, v3), m3, G.KrigingConfig(max_neighbors=24))
    # a second 2-D set with another neighbour count and frame count: its
    # launches use other shared-memory sizes of the same kernels
    mi = VariogramModel(0.1, [Structure("exponential", 1.0, 150.0)])
    ci = uniform_points(15000, 2, 505, [1000.0, 1000.0])
    vi = 5.0 + G.rff_field(ci, mi, 512, 8)
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
