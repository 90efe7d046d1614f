"""The CUDA path against the committed golden fixtures (oracle outputs frozen
by tests/golden/make_golden.py): neighbour lists and plans exactly, values,
variances and log-likelihoods within the 1e-9 parity bar."""
import os
import sys

import numpy as np
import pytest

import geostat_rs as G
from gpu_common import assert_close

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden as MG  # noqa: E402

pytestmark = pytest.mark.gpu
FIX = np.load(os.path.join(HERE, "golden", "path_cases.npz"))


def test_kriging_2d_and_3d_against_fixtures():
    c, v, t = FIX["k2_coords"], FIX["k2_values"], FIX["k2_targets"]
    vs = float(np.mean(np.abs(v)))
    ps = G.PointSet(c, v)
    k = G.Kriging.new(ps, MG.SPH, G.KrigingConfig(max_neighbors=16))
    nb, _ = k.neighbors(t, 16)
    assert (nb == FIX["k2_knn_neighbors"]).all()
    val, var = k.predict_many(t)
    assert_close(val, FIX["k2_knn_value"], vs, 1e-9, "knn value")
    assert_close(var, FIX["k2_knn_variance"], 1e-3, 1e-9, "knn variance")
    k = G.Kriging.new(ps, MG.SPH, G.KrigingConfig(max_neighbors=12, max_per_octant=3,
                                                   anisotropic_search=G.Anisotropy(30.0, 0.5)))
    nb, cnt = k.neighbors(t, 12)
    assert (cnt == FIX["k2_oct_count"]).all() and (nb == FIX["k2_oct_neighbors"]).all()
    val, var = k.predict_many(t)
    assert_close(val, FIX["k2_oct_value"], vs, 1e-9, "octant value")
    assert_close(var, FIX["k2_oct_variance"], 1e-3, 1e-9, "octant variance")
    k = G.Kriging.new(ps, MG.SPH, G.KrigingConfig("universal", degree=1, max_neighbors=20))
    val, var = k.predict_many(t)
    assert_close(val, FIX["k2_uk_value"], vs, 1e-9, "uk value")
    assert_close(var, FIX["k2_uk_variance"], 1e-3, 1e-9, "uk variance")
    cov, tcov = FIX["k2_cov"], FIX["k2_tcov"]
    k = G.Kriging.with_external_drift(G.PointSet(c, v + 3.0 * cov[:, 0]), MG.SPH,
                                      G.KrigingConfig("external_drift", n_vars=1,
                                                      max_neighbors=20), cov)
    val, var = k.predict_many_with_drift(t, tcov)
    assert_close(val, FIX["k2_ked_value"], vs, 1e-9, "ked value")
    assert_close(var, FIX["k2_ked_variance"], 1e-3, 1e-9, "ked variance")
    k = G.Kriging.new(ps, MG.SPH, G.KrigingConfig(max_neighbors=16))
    val, var = k.predict_block_many(t[:40], G.block_offsets([30.0, 30.0], [3, 3]))
    assert_close(val, FIX["k2_block_value"], vs, 1e-9, "block value")
    assert_close(var, FIX["k2_block_variance"], 1e-3, 1e-9, "block variance")
    c3, v3, t3 = FIX["k3_coords"], FIX["k3_values"], FIX["k3_targets"]
    k = G.Kriging.new(G.PointSet(c3, v3), MG.ROT, G.KrigingConfig(max_neighbors=24))
    nb, _ = k.neighbors(t3, 24)
    assert (nb == FIX["k3_neighbors"]).all()
    val, var = k.predict_many(t3)
    assert_close(val, FIX["k3_value"], float(np.mean(np.abs(v3))), 1e-9, "3-D value")
    assert_close(var, FIX["k3_variance"], 1e-3, 1e-9, "3-D variance")


def test_vecchia_against_fixtures():
    cv, vv = FIX["v_coords"], FIX["v_values"]
    plan = G.VecchiaPlan(G.PointSet(cv, vv), 10)
    o, nb, cnt = plan.arrays()
    assert o.tolist() == FIX["v_order"].tolist() and (cnt == FIX["v_cnt"]).all()
    assert (nb == FIX["v_nb"][:, :nb.shape[1]]).all()
    for got, key in ((plan.loglik(MG.VEC)[0], "v_loglik"),
                     (plan.loglik_grouped(MG.VEC, 4)[0], "v_grouped4"),
                     (plan.reml_loglik(MG.VEC, drift_degree=1)[0], "v_reml")):
        ref = FIX[key]
        assert np.all(np.abs(got - ref) <= 1e-9 * np.abs(ref)), (key, got, ref)
