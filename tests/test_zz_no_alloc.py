"""Allocation-free FP64 prediction (gs_kriging_predict_fp64_noalloc).

Some callers cannot let a library allocate device memory while they
predict: a service that reserved its device memory once at start-up, a host
application that runs its own allocator over the whole device, a loop that
cannot take an allocation's implicit synchronisation.  The entry point keeps
its scratch in a static device array instead.

Checked through the C ABI on two calls in a row on the same predictor:

* the library's own device-allocation counter does not move during either
  call (it counts cudaMalloc and stream-ordered allocations alike, so an
  allocation served from the stream-ordered pool's reserve is seen too), and
  the device's free memory is unchanged by the second call;
* outputs agree with the generic device entry point at FP64 (statuses exact;
  values, variances and Lagrange multipliers within 1e-12: both run the
  same one-system-per-thread FP64 solve on moving neighbourhoods) and with
  the FP64 oracle within the 1e-9 parity tolerance;
* global neighbourhoods (no neighbour limit, 120 points): the allocation-free
  call solves each target's full system with the reference's LU, the
  generic call solves with the LU factored once at build; both are the
  reference's algorithm, so statuses match exactly and values agree within
  1e-9, including a predictor whose global system is singular.

Collected last so that it also runs after every other GPU test in the same
process.
"""

import numpy as np
import pytest

import pyoracle as O
import geostat_rs as G
import gs_workload as W
from geostat_rs import _abi
from geostat_rs.model import Structure, VariogramModel
from gpu_common import assert_close, smooth_values, sph200_model, uniform_points

pytestmark = pytest.mark.gpu

TOL_SAME = 1e-12  # same kernel on both paths: agreement far inside the 1e-9 parity bar
TOL = 1e-9


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


def _two_noalloc_calls(lib, kr, cols, nt, torch):
    """Two allocation-free calls; returns their outputs as numpy arrays."""
    stream = torch.cuda.current_stream().cuda_stream
    results = []
    for call in range(2):
        out = _outputs(nt, torch)
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        allocs0 = lib.gs_debug_device_allocations()
        _run(lib.gs_kriging_predict_fp64_noalloc, kr, cols, out, stream, False)
        torch.cuda.synchronize()
        allocs1 = lib.gs_debug_device_allocations()
        free1 = torch.cuda.mem_get_info()[0]
        assert allocs1 == allocs0, f"call {call}: the library allocated {allocs1 - allocs0} times"
        if call == 1:  # the first call on a device may set up; later calls allocate nothing
            assert free1 == free0, f"free device memory changed by {free0 - free1} bytes"
        results.append([t.cpu().numpy() for t in out])
    return results


def _generic_fp64(lib, kr, cols, nt, torch):
    ref = _outputs(nt, torch)
    _run(lib.gs_kriging_predict_many_device, kr, cols, ref, torch.cuda.current_stream().cuda_stream,
         True)
    torch.cuda.synchronize()
    return [t.cpu().numpy() for t in ref]


@pytest.mark.parametrize("dim,cfg", [
    (3, dict(max_neighbors=40)),
    (2, dict(max_neighbors=24, method="universal", degree=1)),
    (2, dict(max_per_octant=4, search_radius=0.2)),
])
def test_noalloc_matches_generic_fp64_and_oracle_on_two_calls(dim, cfg):
    torch = pytest.importorskip("torch")
    lib = _abi.load()
    n = 20000 if dim == 3 else 8000
    coords = uniform_points(n, dim, 31 + dim, [1.0] * dim)
    model = VariogramModel(0.05, [Structure.with_anisotropy("spherical", 0.7, 0.3, 30.0, 0.5),
                                  Structure("exponential", 0.3, 0.4)]) if dim == 2 else \
        VariogramModel(0.05, [Structure.with_rotation("spherical", 0.7, 0.3, 30.0, 10.0, 0.0,
                                                      0.6, 0.4),
                              Structure("exponential", 0.3, 0.4)])
    values = 1.0 + W.rff_field(coords, model, 512, 9)
    kr = G.Kriging.new(G.PointSet(coords, values), model, G.KrigingConfig(**cfg))
    nt = 5000
    targets = uniform_points(nt, dim, 77 + dim, [1.0] * dim)
    cols = [_dev(targets[:, d], torch) for d in range(dim)] + ([None] if dim == 2 else [])

    rv, rvar, rlag, rst = _generic_fp64(lib, kr, cols, nt, torch)
    assert (rst == 0).mean() > 0.9
    okw = dict(cfg)
    okw.pop("degree", None)
    if "search_radius" in okw:
        okw["radius"] = okw.pop("search_radius")
    ref = O.krige(coords, values, model, targets[:1000], degree=cfg.get("degree", 1), **okw)
    scale = float(np.mean(np.abs(values)))
    for call, (v, var, lag, st) in enumerate(_two_noalloc_calls(lib, kr, cols, nt, torch)):
        assert (st == rst).all(), f"call {call}: statuses differ"
        assert_close(v, rv, scale, TOL_SAME, f"call {call} value")
        assert_close(var, rvar, 1.0, TOL_SAME, f"call {call} variance")
        assert_close(lag, rlag, 1.0, TOL_SAME, f"call {call} lagrange")
        assert (st[:1000] == ref["status"].astype(np.uint8)).all(), f"call {call}: oracle statuses"
        assert_close(v[:1000], ref["value"], scale, TOL, f"call {call} value vs oracle")
        assert_close(var[:1000], ref["variance"], 1e-3, TOL, f"call {call} variance vs oracle")


@pytest.mark.parametrize("case", ["ordinary", "universal_singular"])
def test_noalloc_global_neighbourhood(case):
    """No neighbour limit and 120 points: every data point is a neighbour."""
    torch = pytest.importorskip("torch")
    lib = _abi.load()
    m = sph200_model()
    if case == "ordinary":
        c = uniform_points(120, 2, 94, [1000.0, 1000.0])
        v = smooth_values(c)
        kw = {}
    else:
        # every point on one line: the linear drift block is singular
        x = np.linspace(0.0, 1000.0, 120)
        c = np.stack([x, 2.0 * x + 5.0], 1)
        v = np.sin(x / 100.0)
        kw = dict(method="universal", degree=1)
    kr = G.Kriging.new(G.PointSet(c, v), m, G.KrigingConfig(kw.get("method", "ordinary"),
                                                            degree=kw.get("degree", 1)))
    nt = 300
    t = uniform_points(nt, 2, 95, [1000.0, 1000.0])
    cols = [_dev(t[:, 0], torch), _dev(t[:, 1], torch), None]
    rv, rvar, rlag, rst = _generic_fp64(lib, kr, cols, nt, torch)
    ref = O.krige(c, v, m, t, **kw)
    if case == "universal_singular":
        assert (ref["status"] == 3).all()
    else:
        assert (ref["status"] == 0).all()
    scale = float(np.mean(np.abs(v)))
    for call, (val, var, lag, st) in enumerate(_two_noalloc_calls(lib, kr, cols, nt, torch)):
        assert (st == rst).all(), f"call {call}: statuses differ from the generic call"
        assert (st == ref["status"].astype(np.uint8)).all(), f"call {call}: oracle statuses"
        assert_close(val, rv, scale, TOL, f"call {call} value")
        assert_close(var, rvar, 1e-3, TOL, f"call {call} variance")
        assert_close(val, ref["value"], scale, TOL, f"call {call} value vs oracle")
        assert_close(var, ref["variance"], 1e-3, TOL, f"call {call} variance vs oracle")
        ok = ref["status"] == 0
        assert_close(lag[ok], rlag[ok], 1.0, TOL, f"call {call} lagrange")


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
