"""Allocation-free FP64 prediction (gs_kriging_predict_fp64_noalloc).

Compared, through the C ABI, with the generic device entry point at FP64 on
the same predictor and targets: two calls in a row must agree with it within
the parity tolerance (both run the same one-system-per-thread FP64 solve, so
the results are expected to be identical), report the same statuses, and the
second call must leave the device's free memory unchanged.  Collected last so
that it also runs after every other GPU test in the same process.
"""

import numpy as np
import pytest

import geostat_rs as G
from geostat_rs import _abi
from geostat_rs.model import Structure, VariogramModel
from gpu_common import assert_close, uniform_points

pytestmark = pytest.mark.gpu

TOL = 1e-12  # same kernel on both paths: agreement far inside the 1e-9 parity bar

def _dev(a, torch):
    return torch.from_numpy(np.ascontiguousarray(a)).to("cuda")

def _outputs(nt, torch):
    return (torch.full((nt,), -7.0, dtype=torch.float64, device="cuda"),
            torch.full((nt,), -7.0, dtype=torch.float64, device="cuda"),
            torch.full((nt,), -7.0, dtype=torch.float64, device="cuda"),
            torch.full((nt,), 255, dtype=torch.uint8, device="cuda"))

def _run(fn, kr, cols, outs, stream, generic):
    x, y, z = cols
    v, var, lag, st = outs
    zp = z.data_ptr() if z is not None else None
    args = [kr._h, x.numel(), x.data_ptr(), y.data_ptr(), zp, None,
            v.data_ptr(), var.data_ptr(), lag.data_ptr(), st.data_ptr()]
    if generic:
        args.append(1)  # GS_PREC_FP64
    args.append(stream)
    _abi.check(fn(*args))

@pytest.mark.parametrize("dim,cfg", [
    (3, dict(max_neighbors=40)),
    (2, dict(max_neighbors=24, method="universal", degree=1)),
    (2, dict(max_per_octant=4, search_radius=0.2)),
])
def test_noalloc_matches_generic_fp64_on_two_calls(dim, cfg):
    torch = pytest.importorskip("torch")
    lib = _abi.load()
    n = 20000 if dim == 3 else 8000
    coords = uniform_points(n, dim, 31 + dim, [1.0] * dim)
    model = VariogramModel(0.05, [Structure.with_anisotropy("spherical", 0.7, 0.3, 30.0, 0.5),
                                  Structure("exponential", 0.3, 0.4)]) if dim == 2 else \
        VariogramModel(0.05, [Structure.with_rotation("spherical", 0.7, 0.3, 30.0, 10.0, 0.0,
                                                      0.6, 0.4),
                              Structure("exponential", 0.3, 0.4)])
    values = 1.0 + G.rff_field(coords, model, 512, 9)
    kr = G.Kriging.new(G.PointSet(coords, values), model, G.KrigingConfig(**cfg))
    nt = 5000
    targets = uniform_points(nt, dim, 77 + dim, [1.0] * dim)
    cols = [_dev(targets[:, d], torch) for d in range(dim)] + ([None] if dim == 2 else [])
    stream = torch.cuda.current_stream().cuda_stream

    ref = _outputs(nt, torch)
    _run(lib.gs_kriging_predict_many_device, kr, cols, ref, stream, True)
    torch.cuda.synchronize()
    rv, rvar, rlag, rst = [t.cpu().numpy() for t in ref]
    assert (rst == 0).mean() > 0.9

    for call in range(2):
        out = _outputs(nt, torch)
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        _run(lib.gs_kriging_predict_fp64_noalloc, kr, cols, out, stream, False)
        torch.cuda.synchronize()
        free1 = torch.cuda.mem_get_info()[0]
        if call == 1:  # the first call on a device may set up; later calls allocate nothing
            assert free1 == free0, f"free device memory changed by {free0 - free1} bytes"
        v, var, lag, st = [t.cpu().numpy() for t in out]
        assert (st == rst).all(), f"call {call}: statuses differ"
        scale = float(np.mean(np.abs(values)))
        assert_close(v, rv, scale, TOL, f"call {call} value")
        assert_close(var, rvar, 1.0, TOL, f"call {call} variance")
        assert_close(lag, rlag, 1.0, TOL, f"call {call} lagrange")

def test_noalloc_rejects_batches_beyond_its_limit():
    torch = pytest.importorskip("torch")
    lib = _abi.load()
    coords = uniform_points(500, 2, 5, [1.0, 1.0])
    model = VariogramModel(0.0, [Structure("exponential", 1.0, 0.3)])
    kr = G.Kriging.new(G.PointSet(coords, coords[:, 0].copy()), model,
                       G.KrigingConfig(max_neighbors=16))
    too_many = 16384 + 1  # GS_NOALLOC_MAX_TARGETS + 1: rejected before any device access
    rc = lib.gs_kriging_predict_fp64_noalloc(kr._h, too_many, None, None, None, None, None, None,
                                             None, None, None)
    assert rc == G.InvalidParameter.code
    assert b"at most 16384 targets" in lib.gs_last_error()
    torch.cuda.synchronize()
