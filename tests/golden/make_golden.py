"""Writes tests/golden/path_cases.npz: oracle outputs for seeded cases of the
path (kriging in 2-D and 3-D with kNN / octant / anisotropic search, universal
and external-drift kriging, block kriging, the Vecchia plan and likelihoods
including grouped and REML).  The oracle is pinned by the reference's own
known-answer tests (tests/test_oracle_kats.py); these fixtures freeze its
outputs so that the CUDA path and later oracle changes are checked against
fixed numbers.  Run from the repository root:

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "geostat-rs_gb300"))

import pyoracle as O  # noqa: E402
from geostat_rs.model import Anisotropy, Structure, VariogramModel  # noqa: E402

SPH = VariogramModel(0.1, [Structure("spherical", 1.0, 200.0)])
ROT = VariogramModel(0.05, [Structure.with_rotation("spherical", 0.6, 300.0, 30.0, 10.0, 0.0,
                                                    0.5, 40.0 / 300.0),
                            Structure("exponential", 0.35, 800.0)])
VEC = [VariogramModel(0.05, [Structure("exponential", 1.0, 0.1)]),
       VariogramModel(0.02, [Structure("matern25", 1.0, 0.05)])]


def field(c, seed):
    u = O.rng_uniform(seed, 8)
    s = c / (np.max(c, axis=0) + 1.0)
    return 10.0 + np.sin(6.0 * s[:, 0] + u[0]) + np.cos(4.0 * s[:, 1] + u[1])


def cases():
    out = {}
    # 2-D ordinary kriging, kNN 16 and octant 4 x 3, 600 points, 150 targets
    c = O.rng_uniform(701, 1200).reshape(600, 2) * 1000.0
    v = field(c, 702)
    t = O.rng_uniform(703, 300).reshape(150, 2) * 1000.0
    out["k2_coords"], out["k2_values"], out["k2_targets"] = c, v, t
    r = O.krige(c, v, SPH, t, max_neighbors=16, kcap=16)
    out["k2_knn_value"], out["k2_knn_variance"] = r["value"], r["variance"]
    out["k2_knn_neighbors"] = r["neighbors"]
    r = O.krige(c, v, SPH, t, max_neighbors=12, max_per_octant=3,
                anisotropic_search=Anisotropy(30.0, 0.5), kcap=12)
    out["k2_oct_value"], out["k2_oct_variance"] = r["value"], r["variance"]
    out["k2_oct_neighbors"], out["k2_oct_count"] = r["neighbors"], r["nb_count"]
    r = O.krige(c, v, SPH, t, method="universal", degree=1, max_neighbors=20)
    out["k2_uk_value"], out["k2_uk_variance"] = r["value"], r["variance"]
    cov = O.rng_uniform(704, 600).reshape(-1, 1)
    tcov = O.rng_uniform(705, 150).reshape(-1, 1)
    out["k2_cov"], out["k2_tcov"] = cov, tcov
    r = O.krige(c, v + 3.0 * cov[:, 0], SPH, t, method="external_drift", drift=cov,
                target_drift=tcov, max_neighbors=20)
    out["k2_ked_value"], out["k2_ked_variance"] = r["value"], r["variance"]
    off = np.array([[((ix + 0.5) / 3 - 0.5) * 30.0, ((iy + 0.5) / 3 - 0.5) * 30.0]
                    for iy in range(3) for ix in range(3)])
    r = O.krige_block(c, v, SPH, t[:40], off, max_neighbors=16)
    out["k2_block_value"], out["k2_block_variance"] = r["value"], r["variance"]
    # 3-D rotated model, 24 nearest
    c3 = O.rng_uniform(711, 1500).reshape(500, 3) * np.array([2000.0, 2000.0, 200.0])
    v3 = field(c3, 712)
    t3 = O.rng_uniform(713, 240).reshape(80, 3) * np.array([2000.0, 2000.0, 200.0])
    out["k3_coords"], out["k3_values"], out["k3_targets"] = c3, v3, t3
    r = O.krige(c3, v3, ROT, t3, max_neighbors=24, kcap=24)
    out["k3_value"], out["k3_variance"], out["k3_neighbors"] = (r["value"], r["variance"],
                                                                r["neighbors"])
    # Vecchia: plan, likelihoods, grouped, REML
    cv = O.rng_uniform(721, 1600).reshape(800, 2)
    vv = 0.5 + np.sin(7.0 * cv[:, 0]) * np.cos(5.0 * cv[:, 1])
    out["v_coords"], out["v_values"] = cv, vv
    o, nb, cnt = O.vecchia_plan(cv, 10)
    out["v_order"], out["v_nb"], out["v_cnt"] = o, nb, cnt
    out["v_loglik"] = np.array([O.vecchia_loglik_plan(cv, vv, m, o, nb, cnt) for m in VEC])
    out["v_grouped4"] = np.array([O.vecchia_loglik_grouped(cv, vv, m, o, nb, cnt, 4) for m in VEC])
    f = O.poly_basis(cv, 1)
    out["v_reml"] = np.array([O.vecchia_reml_loglik(cv, vv, m, o, nb, cnt, f, 1) for m in VEC])
    return out


if __name__ == "__main__":
    O.build()
    path = os.path.join(HERE, "path_cases.npz")
    np.savez_compressed(path, **cases())
    print(path, os.path.getsize(path), "bytes")
