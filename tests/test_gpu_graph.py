"""Asynchronous prediction pass captured into a CUDA graph.

gs_kriging_predict_many_async enqueues search, mixed solve and FP64 re-solve
without waiting for the device (the re-solve list length is read on the
device), so the pass can be captured once and replayed on new targets written
into the same device buffers.  Every replay must equal the synchronous entry
point on those targets bit for bit: the same kernels run on the same inputs in
the same order (including the split of uneven neighbourhoods into the 32- and
64-thread solvers).
"""
import numpy as np
import pytest

import geostat_rs as G
import gs_workload as W
from geostat_rs.model import Structure, VariogramModel
from gpu_common import uniform_points

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

CASES = {
    # k nearest: one solver width, no binning
    "knn48": (2, G.KrigingConfig(max_neighbors=48)),
    # octant search (4 x 12): counts below and above 32 use both solvers
    "octant12": (2, G.KrigingConfig(max_per_octant=12)),
    # radius-limited: uneven counts, both solvers, some short of neighbours
    "radius": (2, G.KrigingConfig(max_neighbors=64, search_radius=28.0, min_neighbors=3)),
    "octant3d": (3, G.KrigingConfig(max_per_octant=6, max_neighbors=40)),
}


def _cols(t):
    return [torch.from_numpy(np.ascontiguousarray(t[:, d])).cuda() for d in range(t.shape[1])]


@pytest.mark.parametrize("case", sorted(CASES))
def test_captured_pass_replays_on_new_targets(case):
    dim, cfg = CASES[case]
    m = VariogramModel(0.05, [Structure.with_anisotropy("spherical", 0.7, 150.0, 30.0, 0.5),
                              Structure("exponential", 0.25, 400.0)])
    ext = [1000.0, 1000.0, 200.0][:dim]
    c = uniform_points(20000, dim, 611 + dim, ext)
    v = 10.0 + W.rff_field(c, m, 512, 9)
    k = G.Kriging.new(G.PointSet(c, v), m, cfg)
    nt = 6000
    rng = np.random.default_rng(17)
    # targets reach 10 % beyond the data: outside the hull octants run empty
    sets = [(rng.uniform(0, 1, size=(nt, dim)) * 1.2 - 0.1) * ext for _ in range(3)]
    X = [torch.empty(nt, dtype=torch.float64, device="cuda") for _ in range(dim)]
    V = torch.empty(nt, dtype=torch.float64, device="cuda")
    VAR = torch.empty(nt, dtype=torch.float64, device="cuda")
    ST = torch.empty(nt, dtype=torch.uint8, device="cuda")
    s = torch.cuda.Stream()

    def load(t):
        for d, col in enumerate(_cols(t)):
            X[d].copy_(col)
        torch.cuda.synchronize()

    def enqueue(asynchronous):
        z = X[2].data_ptr() if dim == 3 else None
        k.predict_device(nt, X[0].data_ptr(), X[1].data_ptr(), z, V.data_ptr(), VAR.data_ptr(),
                         ST.data_ptr(), "mixed", stream=s.cuda_stream, asynchronous=asynchronous)

    # an ordinary call first (constant tables, kernel attributes)
    load(sets[0])
    enqueue(False)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        enqueue(True)
    torch.cuda.synchronize()
    for t in (sets[1], sets[2], sets[1]):
        load(t)
        V.fill_(-1.0)
        g.replay()
        torch.cuda.synchronize()
        ref = k.predict_many(t, "mixed", full=True)
        st = ST.cpu().numpy()
        assert (st == ref.status).all()
        np.testing.assert_array_equal(V.cpu().numpy(), ref.value)
        np.testing.assert_array_equal(VAR.cpu().numpy(), ref.variance)
    if case != "knn48":
        # the uneven cases really do use both solver widths
        _, cnt = k.neighbors(sets[1], 64)
        assert (cnt <= 32).any() and (cnt > 32).any()


def test_async_pass_without_capture_matches():
    m = VariogramModel(0.1, [Structure("exponential", 1.0, 150.0)])
    c = uniform_points(15000, 2, 621, [1000.0, 1000.0])
    v = 5.0 + W.rff_field(c, m, 512, 3)
    k = G.Kriging.new(G.PointSet(c, v), m, G.KrigingConfig(max_per_octant=10))
    t = np.random.default_rng(3).uniform(0, 1000, size=(3000, 2))
    x, y = _cols(t)
    out = [torch.empty(3000, dtype=torch.float64, device="cuda") for _ in range(2)]
    st = torch.empty(3000, dtype=torch.uint8, device="cuda")
    s = torch.cuda.Stream()
    torch.cuda.synchronize()  # the copies above ran on the default stream
    k.predict_device(3000, x.data_ptr(), y.data_ptr(), None, out[0].data_ptr(), out[1].data_ptr(),
                     st.data_ptr(), "mixed", stream=s.cuda_stream, asynchronous=True)
    s.synchronize()
    ref = k.predict_many(t, "mixed", full=True)
    np.testing.assert_array_equal(out[0].cpu().numpy(), ref.value)
    np.testing.assert_array_equal(out[1].cpu().numpy(), ref.variance)
    assert (st.cpu().numpy() == ref.status).all()
