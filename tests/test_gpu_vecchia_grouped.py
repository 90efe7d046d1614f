"""Grouped (Guinness) Vecchia log-likelihood on the GPU against the oracle.

The blocks are built from the GPU plan (which equals the oracle's plan, see
test_gpu_vecchia.py), so both sides factor the same joint sets; log-likelihood
sums within 1e-9 relative; group size 1 is the ungrouped batch exactly; the
reference's grouped known answers hold on the device too.
"""
import numpy as np
import pytest

import pyoracle as O
import geostat_rs as G
import gs_workload as W
from geostat_rs.model import Structure, VariogramModel
from gpu_common import uniform_points

pytestmark = pytest.mark.gpu


def _models():
    return [VariogramModel(0.05, [Structure("exponential", 1.0, 0.1)]),
            VariogramModel(0.02, [Structure("matern25", 1.0, 0.05)]),
            VariogramModel(0.1, [Structure("spherical", 0.7, 0.3), Structure("gaussian", 0.3, 0.2)])]


@pytest.mark.parametrize("dim,m,g", [(2, 15, 2), (2, 30, 4), (2, 10, 8), (3, 20, 4)])
def test_grouped_loglik_matches_oracle(dim, m, g):
    c = uniform_points(3000, dim, 101 + dim, [1.0] * dim)
    v = 0.5 + W.rff_field(c, _models()[1], 512, 102)
    plan = G.VecchiaPlan(G.PointSet(c, v), m)
    order, nb, cnt = plan.arrays()
    ll, st = plan.loglik_grouped(_models(), g)
    assert (st == 0).all()
    for i, mdl in enumerate(_models()):
        ref = O.vecchia_loglik_grouped(c, v, mdl, order, nb, cnt, g)
        assert abs(ll[i] - ref) <= 1e-9 * abs(ref), (i, ll[i], ref)
    one, _ = plan.loglik_grouped(_models(), 1)
    batch, _ = plan.loglik(_models())
    np.testing.assert_array_equal(one, batch)


def test_grouped_known_answers_on_device():
    # vecchia.rs:2066-2085: full conditioning, any group size == exact
    c, v = O.test_field_2d(20, 4)
    m = VariogramModel(0.05, [Structure("exponential", 1.0, 40.0)])
    exact = O.exact_loglik(c, v, m)
    for g in (2, 3, 5, 8):
        got = G.vecchia_loglik_grouped(G.PointSet(c, v), m, len(c) - 1, None, g)
        assert abs(got - exact) < 1e-8
