"""The sharded paths with the library as each rank's per-shard work.

Two gloo ranks (processes) share the one GPU; neither rank's kernels wait on
the other's.  Each rank holds a replica of the predictor and of the Vecchia
plan, predicts its contiguous shard of the targets and sums the likelihood
terms of its ordered positions (gs_vecchia_loglik_batch_range); shards and
partial sums travel as arrays and are combined in rank order.

Against the unsharded library call in the same process:
* FP64 kriging: identical (one system per thread, no dependence on the
  batch); mixed kriging: statuses identical, values within 1e-12 (a target's
  neighbour slots, and so the order of its roundings, depend on the targets
  solved before it in its run);
* log-likelihood sums: within 1e-12 relative (the rank partials re-associate
  the fixed-order sum); identical from run to run.
"""
import os
import socket
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out_dir):
    for sub in ("", "tests", "geostat-rs_gb300", "oracle"):
        sys.path.insert(0, os.path.join(ROOT, sub))
    import torch.distributed as dist
    import geostat_rs as G
    import gs_workload as W
    from geostat_rs.distributed import predict_sharded, shard_range, sum_sharded
    from geostat_rs.model import Structure, VariogramModel
    from gpu_common import uniform_points
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    try:
        c = uniform_points(20000, 2, 501, [1000.0, 1000.0])
        m = VariogramModel(0.05, [Structure("spherical", 0.8, 150.0),
                                  Structure("exponential", 0.2, 400.0)])
        v = 3.0 + W.rff_field(c, m, 512, 502)
        ps = G.PointSet(c, v)
        k = G.Kriging.new(ps, m, G.KrigingConfig(max_neighbors=32))
        t = uniform_points(30001, 2, 503, [1000.0, 1000.0])
        res = {}
        for prec in ("mixed", "fp64"):
            def predict(tt, prec=prec):
                r = k.predict_many(tt, prec, full=True)
                return r.value, r.variance, r.status
            val, var, st = predict_sharded(predict, t)
            res[prec] = (val, var, st)
        plan = G.VecchiaPlan(ps, 20)
        models = [m, VariogramModel(0.02, [Structure("matern25", 1.0, 120.0)])]

        def partial(lo, hi):
            ll, st = plan.loglik_range(lo, hi, models)
            assert (st == 0).all()
            return ll

        ll = sum_sharded(partial, ps.n)
        lo, hi = shard_range(ps.n, rank, world)
        if rank == 0:
            ref = {prec: k.predict_many(t, prec, full=True) for prec in ("mixed", "fp64")}
            ref_ll, ref_st = plan.loglik(models)
            empty, _ = plan.loglik_range(7, 7, models)
            np.savez(os.path.join(out_dir, "out.npz"), ll=ll, ref_ll=ref_ll, ref_st=ref_st,
                     empty=empty, lo=lo, hi=hi,
                     **{f"{p}_{q}": res[p][i] for p in res for i, q in enumerate(("v", "var", "st"))},
                     **{f"ref_{p}_v": ref[p].value for p in ref},
                     **{f"ref_{p}_var": ref[p].variance for p in ref},
                     **{f"ref_{p}_st": ref[p].status for p in ref})
    finally:
        dist.destroy_process_group()


def _run(tmp_path):
    import torch.multiprocessing as mp
    tmp_path.mkdir(parents=True, exist_ok=True)
    mp.spawn(_worker, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True)
    return np.load(os.path.join(tmp_path, "out.npz"))


def test_sharded_library_on_two_gloo_ranks(tmp_path):
    a = _run(tmp_path / "a")
    assert a["hi"] - a["lo"] == 10000
    assert np.array_equal(a["fp64_v"], a["ref_fp64_v"], equal_nan=True)
    assert np.array_equal(a["fp64_var"], a["ref_fp64_var"], equal_nan=True)
    assert np.array_equal(a["fp64_st"], a["ref_fp64_st"])
    assert np.array_equal(a["mixed_st"], a["ref_mixed_st"])
    ok = a["ref_mixed_st"] == 0
    assert ok.mean() > 0.99
    assert np.max(np.abs(a["mixed_v"] - a["ref_mixed_v"])[ok]) <= 1e-12 * np.mean(np.abs(a["ref_mixed_v"]))
    assert np.max(np.abs(a["mixed_var"] - a["ref_mixed_var"])[ok]) <= 1e-12
    assert (a["ref_st"] == 0).all()
    assert np.allclose(a["ll"], a["ref_ll"], rtol=1e-12, atol=0)
    assert np.array_equal(a["empty"], np.zeros(2))
    b = _run(tmp_path / "b")
    assert np.array_equal(a["ll"], b["ll"])  # fixed reduction order


def test_point_range_rejects_bad_ranges():
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import geostat_rs as G
    from geostat_rs.model import Structure, VariogramModel
    from gpu_common import uniform_points
    c = uniform_points(500, 2, 7, [1.0, 1.0])
    plan = G.VecchiaPlan(G.PointSet(c, c[:, 0] + 1.0), 10)
    m = [VariogramModel(0.1, [Structure("exponential", 1.0, 0.3)])]
    for lo, hi in ((-1, 10), (10, 5), (0, 501)):
        with pytest.raises(G.InvalidParameter):
            plan.loglik_range(lo, hi, m)
    whole, _ = plan.loglik(m)
    parts = [plan.loglik_range(lo, hi, m)[0][0] for lo, hi in ((0, 1), (1, 250), (250, 500))]
    assert abs(sum(parts) - whole[0]) <= 1e-12 * abs(whole[0])
