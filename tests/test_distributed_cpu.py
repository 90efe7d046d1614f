"""Multi-process host logic of the sharded paths, as two gloo ranks on CPU.

Kriging targets shard into contiguous ranges gathered in rank order; Vecchia
log-likelihood partial sums are added in rank order.  The per-shard work here
is the oracle (the GPU predictors are the same callables on a GPU machine), so
the sharded results must equal the unsharded ones exactly for kriging and to
rounding for the re-associated likelihood sums -- and be identical run to run.
"""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out_dir):
    for sub in ("", "geostat-rs_gb300", "oracle"):
        sys.path.insert(0, os.path.join(ROOT, sub))
    import torch.distributed as dist
    import pyoracle as O
    from geostat_rs.distributed import predict_sharded, sum_sharded
    from geostat_rs.model import Structure, VariogramModel
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    try:
        c, v = O.test_field_2d(400, 5)
        m = VariogramModel(0.1, [Structure("spherical", 1.0, 30.0)])
        t = np.stack(np.meshgrid(np.linspace(0, 100, 23), np.linspace(0, 100, 19)), -1).reshape(-1, 2)

        def predict(tt):
            r = O.krige(c, v, m, tt, max_neighbors=12, nthreads=1)
            return r["value"], r["variance"]

        val, var = predict_sharded(predict, t)
        order = O.maxmin_order(c)
        _, nb, cnt = O.vecchia_plan(c, 10, order)
        models = [m, VariogramModel(0.05, [Structure("exponential", 1.0, 20.0)])]
        terms = [O.vecchia_loglik_plan(c, v, mm, order, nb, cnt, terms=True)[1] for mm in models]
        ll = sum_sharded(lambda lo, hi: np.array([tm[lo:hi].sum() for tm in terms]), len(c))
        if rank == 0:
            np.savez(os.path.join(out_dir, "out.npz"), val=val, var=var, ll=ll,
                     ref_val=predict(t)[0], ref_var=predict(t)[1],
                     ref_ll=np.array([O.vecchia_loglik_plan(c, v, mm, order, nb, cnt)
                                      for mm in models]))
    finally:
        dist.destroy_process_group()


def _run(tmp_path):
    import torch.multiprocessing as mp
    tmp_path.mkdir(parents=True, exist_ok=True)
    mp.spawn(_worker, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True)
    return np.load(os.path.join(tmp_path, "out.npz"))


def test_sharded_paths_on_two_gloo_ranks(tmp_path):
    a = _run(tmp_path / "a")
    assert np.array_equal(a["val"], a["ref_val"], equal_nan=True)
    assert np.array_equal(a["var"], a["ref_var"], equal_nan=True)
    assert np.allclose(a["ll"], a["ref_ll"], rtol=1e-12, atol=0)
    b = _run(tmp_path / "b")
    assert np.array_equal(a["ll"], b["ll"])  # fixed reduction order


def test_shard_ranges_cover_in_order():
    from geostat_rs.distributed import shard_range
    for n in (0, 1, 7, 8, 1000):
        for world in (1, 2, 3, 8):
            spans = [shard_range(n, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(spans[i][1] == spans[i + 1][0] for i in range(world - 1))
            sizes = [hi - lo for lo, hi in spans]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard_range(5, 2, 2)
