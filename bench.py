#!/usr/bin/env python
"""Benchmark: kriged targets/s (and Vecchia points/s) on one GB300.

Workload (one step = one pass of the hot path over one batch):
  3-D ordinary kriging, n = 200,000 data points uniform in a 2000 x 2000 x 200 m
  box; values from a 4,096-feature random-Fourier-feature field of the nested
  model nugget 0.05 + Sph(0.6; ranges 300/150/40 m, azimuth 30, dip 10) +
  Exp(0.35, 800 m); targets = the 256 x 256 x 64 grid (4,194,304 cells); the
  64 nearest Euclidean neighbours per target; FP32 factorisation with
  double-float refinement and FP64 outputs.

`value` is measured with inputs resident in HBM (the device entry point), L2
flushed between steps; `e2e` goes through the host-buffer C-ABI call with the
host<->device copies inside the timed region.  The plain FP64 GPU build and a
Vecchia log-likelihood batch (2,000,000 points, m = 30, 16 candidates) are
timed beside it, and the CPU oracle is timed on a bounded sample of the same
workload on the host's cores.

--impl reference times the reference algorithm on the CPU (the oracle, all
host threads) on the same workload and prints the same JSON line.
"""
import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "geostat-rs_gb300"))

import numpy as np  # noqa: E402

import gs_workload as W  # noqa: E402  (synthetic workloads and probes; no device work at import)

METRIC = "kriged targets/s & Vecchia points/s, mixed-prec vs FP64 GPU @1e-9; p99 latency"
WORKLOAD = ("3-D ordinary kriging: n=200,000 points in 2000x2000x200 m, RFF field (4,096 "
            "features) of nugget 0.05 + Sph(0.6; 300/150/40 m; az 30, dip 10) + Exp(0.35, 800 m); "
            "targets 256x256x64 grid (4,194,304); n_max=64 Euclidean nearest")
N_DATA = 200_000
GRID = (256, 256, 64)
BOX = (2000.0, 2000.0, 200.0)
K_NEIGH = 64
SEED = 20260


def algorithmic_flops_per_target(n, p=1):
    """N^3/3 + 2N^2 + 4N for a system of N = n + p unknowns."""
    N = n + p
    return N ** 3 / 3.0 + 2.0 * N ** 2 + 4.0 * N


def make_model():
    from geostat_rs.model import Structure, VariogramModel
    return VariogramModel(0.05, [Structure.with_rotation("spherical", 0.6, 300.0, 30.0, 10.0, 0.0,
                                                         0.5, 40.0 / 300.0),
                                 Structure("exponential", 0.35, 800.0)])


def workload_config(n_targets, world):
    """The headline workload's config dict, identical in both arms."""
    return {"workload": WORKLOAD, "n_data": N_DATA, "n_targets": n_targets,
            "max_neighbors": K_NEIGH, "dim": 3,
            "l2": "flushed between steps (256 MiB write); neighbour lists 1 GiB > L2",
            "parallelism": f"replicas x{world} (targets independent)"}


def make_coords():
    import geostat_rs as G
    u = G.rng_uniform(SEED, 3 * N_DATA).reshape(N_DATA, 3)
    return u * np.asarray(BOX)


def grid_targets():
    nx, ny, nz = GRID
    ix = (np.arange(nx) + 0.5) * (BOX[0] / nx)
    iy = (np.arange(ny) + 0.5) * (BOX[1] / ny)
    iz = (np.arange(nz) + 0.5) * (BOX[2] / nz)
    z, y, x = np.meshgrid(iz, iy, ix, indexing="ij")
    return np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1)


class ClockSampler:
    """nvidia-smi samples during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for nm, val in zip(names, parts[4:8]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def read_profile_traffic():
    """DRAM bytes per target of the kriging kernel from the committed ncu summary
    (dram__bytes_read.sum + dram__bytes_write.sum of one captured launch divided by
    the targets it solved)."""
    path = os.path.join(ROOT, "profiles", "krige_rows_kernel_3d_ok64.md")
    try:
        text = open(path).read()
    except OSError:
        return None
    m = re.search(r"dram_bytes_per_target:\s*([0-9.eE+]+)", text)
    return float(m.group(1)) if m else None


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        return {}


# ------------------------------------------------------------------ ours --
def run_ours(args, rank, world):
    import torch
    import geostat_rs as G
    from geostat_rs import _abi

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    dev = torch.device("cuda")
    log = (lambda *a: print(*a, file=sys.stderr, flush=True)) if rank == 0 else (lambda *a: None)
    t0 = time.time()
    coords = make_coords()
    model = make_model()
    values = W.rff_field(coords, model, 4096, SEED + 1)
    ps = G.PointSet(coords, values)
    kr = G.Kriging.new(ps, model, G.KrigingConfig(max_neighbors=K_NEIGH))
    tg = grid_targets()
    nt = len(tg)
    log(f"[bench] data + grid build {time.time() - t0:.1f}s, nt={nt}")

    cols = [torch.from_numpy(np.ascontiguousarray(tg[:, d])).to(dev) for d in range(3)]
    out_v = torch.empty(nt, dtype=torch.float64, device=dev)
    out_var = torch.empty(nt, dtype=torch.float64, device=dev)
    out_st = torch.empty(nt, dtype=torch.uint8, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream

    def step(prec):
        kr.predict_device(nt, cols[0].data_ptr(), cols[1].data_ptr(), cols[2].data_ptr(),
                          out_v.data_ptr(), out_var.data_ptr(), out_st.data_ptr(), prec, sptr)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    def timed(prec, steps, warmup, collect=None):
        for _ in range(warmup):
            step(prec)
        torch.cuda.synchronize()
        barrier()
        times, phases, launches = [], [], 0
        for _ in range(steps):
            flush.zero_()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            l0 = _abi.load().gs_launch_count()
            e0.record(stream)
            step(prec)
            e1.record(stream)
            torch.cuda.synchronize()
            launches += _abi.load().gs_launch_count() - l0
            times.append(e0.elapsed_time(e1))
            phases.append(G.last_timings())
        barrier()
        mx = max(times)
        tot = sum(times)
        if world > 1:
            t = torch.tensor([tot], device=dev, dtype=torch.float64)
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            tot = float(t.item())
        return tot / steps, times, phases, launches

    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    ms_mixed, times, phases, launches = timed("mixed", args.steps, args.warmup)
    clk = clocks.stop()
    value = world * nt / (ms_mixed * 1e-3)
    mixed_ms = statistics.mean(p[1] for p in phases)
    search_ms = statistics.mean(p[0] for p in phases)
    resolve_ms = statistics.mean(p[2] for p in phases)
    st = out_st.cpu().numpy()
    n_fallback = int(((st & 0x40) != 0).sum())
    n_fail = int(((st & 0x3f) != 0).sum())
    log(f"[bench] mixed: {ms_mixed:.1f} ms/step (search {search_ms:.1f}, solve {mixed_ms:.1f}, "
        f"fp64 re-solve {resolve_ms:.1f}), fallback {n_fallback}, failed {n_fail}")
    mixed_value = out_v.cpu().numpy()
    mixed_var = out_var.cpu().numpy()

    # plain FP64 GPU build on the same workload
    ms_fp64, _, ph64, _ = timed("fp64", max(1, min(2, args.steps)), 1)
    fp64_value = world * nt / (ms_fp64 * 1e-3)
    fp64_v = out_v.cpu().numpy()
    log(f"[bench] fp64 plain build: {ms_fp64:.1f} ms/step")

    # end to end through the host-buffer call (pinned host memory)
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    hx, hy, hz = pin(tg[:, 0]), pin(tg[:, 1]), pin(tg[:, 2])
    hv = torch.empty(nt, dtype=torch.float64).pin_memory().numpy()
    hvar = torch.empty(nt, dtype=torch.float64).pin_memory().numpy()
    hlag = torch.empty(nt, dtype=torch.float64).pin_memory().numpy()
    hst = torch.empty(nt, dtype=torch.uint8).pin_memory().numpy()
    import ctypes as C
    P = lambda a, ct=C.c_double: a.ctypes.data_as(C.POINTER(ct))
    lib = _abi.load()

    def e2e_step():
        _abi.check(lib.gs_kriging_predict_many(kr._h, nt, P(hx), P(hy), P(hz), None, P(hv), P(hvar),
                                               P(hlag), P(hst, C.c_uint8), 0, None))

    for _ in range(max(1, args.warmup // 2)):
        e2e_step()
    barrier()
    e2e_times = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        e2e_step()
        e2e_times.append(time.perf_counter() - t1)
    barrier()
    e2e_ms = statistics.mean(e2e_times) * 1e3
    if world > 1:
        t = torch.tensor([e2e_ms], device=dev, dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_ms = float(t.item())
    e2e_value = world * nt / (e2e_ms * 1e-3)
    h2d = 3 * 8 * nt
    d2h = (8 + 8 + 8 + 1) * nt
    assert np.array_equal(hv, mixed_value, equal_nan=True)
    log(f"[bench] e2e: {e2e_ms:.1f} ms/step")

    result = None
    if rank == 0:
        # roofline: algorithmic FP32 flops of the dominant (mixed) kernel
        fpt = algorithmic_flops_per_target(K_NEIGH, 1)
        flops_per_launch_set = fpt * nt
        achieved = flops_per_launch_set / (mixed_ms * 1e-3) / 1e12
        peak_fp32 = C.c_double()
        peak_fp64 = C.c_double()
        peak_x2 = C.c_double()
        wl = W.load()
        _abi.check(wl.gs_probe_fma_tflops(0, C.byref(peak_fp32)))
        _abi.check(wl.gs_probe_fma_tflops(1, C.byref(peak_fp64)))
        _abi.check(wl.gs_probe_fma_tflops(2, C.byref(peak_x2)))
        bpt = read_profile_traffic()
        # one launch of the kriging kernel per step (the neighbour lists fit one chunk)
        traffic = bpt * nt if bpt is not None else None
        # accuracy and CPU baseline on a bounded sample
        acc, cpu = cpu_sample_and_accuracy(args, coords, values, model, tg, mixed_value, mixed_var,
                                           fp64_v, kr, log)
        cvr = cv_bench(args, coords, values, model, log) if args.cv_sample > 0 else None
        glb = global_bench(args, log) if not args.no_global else None
        blk = block_bench(args, log) if not args.no_block else None
        vec = vecchia_bench(args, log) if not args.no_vecchia else None
        clu = clustered_bench(args, log) if not args.no_clustered else None
        serve = serving_bench(args, log) if args.serve_requests > 0 else None
        peaks = measured_peaks()
        result = {
            "metric": METRIC,
            "value": value,
            "unit": "kriged targets/s",
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": ms_mixed,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f32 factor + df64 refinement + f64 outputs",
            "data": "synthetic: seeded xoshiro256++ coordinates, random-Fourier-feature field",
            "config": workload_config(nt, world),
            "phases_ms": {"search": search_ms, "mixed_solve": mixed_ms, "fp64_resolve": resolve_ms,
                          "fp64_resolved_targets": n_fallback, "failed_targets": n_fail},
            "fp64_gpu_build": {"value": fp64_value, "unit": "kriged targets/s",
                               "ms_per_step": ms_fp64,
                               "mixed_over_fp64": value / fp64_value},
            "accuracy": acc,
            "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak_fp32.value,
                         "unit": "TFLOP/s", "frac": achieved / peak_fp32.value,
                         "traffic": traffic,
                         "kernel": "krige_rows_kernel",
                         "peak_source": "measured FP32 FMA probe (gs_probe_fma_tflops); "
                                        "MEASURED_PEAKS.json has no CUDA-core number",
                         "fp32x2_peak_tflops": peak_x2.value,
                         "fp64_peak_tflops": peak_fp64.value,
                         "traffic_bytes_per_target": bpt,
                         "algorithmic_flops_per_target": fpt,
                         "hbm_peak_gbs": peaks.get("hbm_gbs")},
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": "kriged targets/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms},
            "gpu_launches": launches,
            "clocks": clk,
        }
        if vec is not None:
            result["vecchia"] = vec
        if clu is not None:
            result["clustered"] = clu
        if cvr is not None:
            result["cross_validation"] = cvr
        if glb is not None:
            result["global_neighbourhood"] = glb
        if blk is not None:
            result["block_kriging"] = blk
        if serve is not None:
            result["serving"] = serve
            result["p99_latency_ms"] = serve["p99_ms"]
    return result


def cpu_sample_and_accuracy(args, coords, values, model, tg, mixed_value, mixed_var, fp64_v, kr,
                            log):
    """Oracle on a bounded sample: CPU throughput and max rel error of both GPU paths."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as O
    O.build()
    cores = os.cpu_count() or 1
    rng = np.random.RandomState(7)
    probe = rng.choice(len(tg), 2000, replace=False)
    t0 = time.perf_counter()
    O.krige(coords, values, model, tg[probe], max_neighbors=K_NEIGH, nthreads=cores)
    per = (time.perf_counter() - t0) / len(probe)
    ns = int(min(len(tg), max(2000, args.cpu_seconds / max(per, 1e-9))))
    idx = np.sort(rng.choice(len(tg), ns, replace=False))
    t0 = time.perf_counter()
    ref = O.krige(coords, values, model, tg[idx], max_neighbors=K_NEIGH, nthreads=cores,
                  kcap=K_NEIGH)
    dt = time.perf_counter() - t0
    log(f"[bench] oracle: {ns} targets in {dt:.1f}s on {cores} threads")
    vs = float(np.mean(np.abs(values)))
    sill = model.total_sill()

    def rel(a, b, floor):
        return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), floor)))

    nbr_idx, _ = kr.neighbors(tg[idx[:5000]], K_NEIGH)
    mism = int((nbr_idx != ref["neighbors"][:5000]).any(axis=1).sum())
    acc = {"sample_targets": ns,
           "mixed_max_rel_value": rel(mixed_value[idx], ref["value"], vs),
           "mixed_max_rel_variance": rel(mixed_var[idx], ref["variance"], 1e-3 * sill),
           "fp64_max_rel_value": rel(fp64_v[idx], ref["value"], vs),
           "tolerance": "|a-b| <= 1e-9 max(|b|, floor); floor = mean|z| (values), 1e-3 sill (variances)",
           "neighbour_set_mismatches": mism, "neighbour_sample": min(5000, ns),
           "oracle_boundary_ties": ref["boundary_ties"]}
    cpu = {"value": ns / dt, "unit": "kriged targets/s", "cores": cores, "kind": "port",
           "sample": f"{ns} random targets of the 4,194,304-cell grid (same data, model, n_max=64)"}
    return acc, cpu


def cv_bench(args, coords, values, model, log):
    """Leave-one-out cross-validation of the 3-D workload's 200,000 points (64
    nearest, each point predicted from all the others), on the GPU; the oracle
    follows the reference (a predictor rebuilt without the held-out point, so
    a kd-tree build per point) on a bounded sample of points."""
    import geostat_rs as G
    ps = G.PointSet(coords, values)
    cfg = G.KrigingConfig(max_neighbors=K_NEIGH)
    cv = G.leave_one_out(ps, model, cfg)  # warm-up (and launch-shape tuning)
    ts = []
    for _ in range(3):
        t1 = time.perf_counter()
        cv = G.leave_one_out(ps, model, cfg)
        ts.append(time.perf_counter() - t1)
    dt = statistics.median(ts)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as O
    O.build()
    rng = np.random.RandomState(13)
    sample = rng.choice(len(coords), args.cv_sample, replace=False)
    t1 = time.perf_counter()
    ref_p, ref_v = [], []
    for i in sample:
        keep = np.ones(len(coords), bool)
        keep[i] = False
        r = O.krige(coords[keep], values[keep], model, coords[i:i + 1], max_neighbors=K_NEIGH,
                    nthreads=1)
        ref_p.append(r["value"][0])
        ref_v.append(r["variance"][0])
    dcpu = time.perf_counter() - t1
    vs = float(np.mean(np.abs(values)))
    rel = lambda a, b, f: float(np.max(np.abs(a - b) / np.maximum(np.abs(b), f)))
    log(f"[bench] leave-one-out: {len(coords)} points in {dt * 1e3:.1f} ms; oracle "
        f"{len(sample)} points in {dcpu:.1f}s")
    return {"points": len(coords), "max_neighbors": K_NEIGH, "seconds": dt,
            "points_per_s": len(coords) / dt, "vecv": cv.vecv(), "rmse": cv.rmse(),
            "oracle_sample": len(sample),
            "cpu_points_per_s": len(sample) / dcpu, "cpu_cores": 1,
            "cpu_kind": "port (a predictor rebuilt per held-out point, as validation.rs:148)",
            "max_rel_value": rel(cv.predicted[sample], np.array(ref_p), vs),
            "max_rel_variance": rel(cv.variance[sample], np.array(ref_v), 1e-3)}


def global_setup():
    """The global-neighbourhood workload: 2,000 points uniform in 1000 x 1000 m,
    10 + field of nugget 0.1 + Sph(1, 200 m), targets the 100 x 100 grid."""
    import geostat_rs as G
    from geostat_rs.model import Structure, VariogramModel
    n = 2000
    c = G.rng_uniform(SEED + 31, 2 * n).reshape(n, 2) * 1000.0
    m = VariogramModel(0.1, [Structure("spherical", 1.0, 200.0)])
    v = 10.0 + W.rff_field(c, m, 2048, SEED + 32)
    g = (np.arange(100) + 0.5) * 10.0
    yy, xx = np.meshgrid(g, g, indexing="ij")
    t = np.stack([xx.ravel(), yy.ravel()], 1)
    return n, c, v, m, t


def global_bench(args, log):
    """Global-neighbourhood ordinary kriging (kriging.rs:396-406): the 2-D
    workload's 2,000 points (uniform in 1000 x 1000 m, 10 + field, nugget 0.1 +
    Sph(1, 200 m)) with no neighbour limit -- one 2,001-unknown system factored
    at build -- predicted at the 100 x 100 grid: the mixed path (the system's
    matrix-product form: FP64 dot products for estimates, a double-float GEMM
    for variances) and the FP64 build (per-target solves with the LU
    factors); the oracle (the same global LU path) on all host cores."""
    import geostat_rs as G
    n, c, v, m, t = global_setup()
    t0 = time.perf_counter()
    k = G.Kriging.new(G.PointSet(c, v), m)
    build = time.perf_counter() - t0
    k.predict_many(t)
    ts = []
    for _ in range(3):
        t1 = time.perf_counter()
        out = k.predict_many(t, full=True)
        ts.append(time.perf_counter() - t1)
    dt = statistics.median(ts)
    out64 = k.predict_many(t, "fp64", full=True)
    ts64 = []
    for _ in range(3):
        t1 = time.perf_counter()
        out64 = k.predict_many(t, "fp64", full=True)
        ts64.append(time.perf_counter() - t1)
    dt64 = statistics.median(ts64)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as O
    O.build()
    cores = os.cpu_count() or 1
    t1 = time.perf_counter()
    ref = O.krige(c, v, m, t, nthreads=cores)
    dcpu = time.perf_counter() - t1
    vs = float(np.mean(np.abs(v)))
    rel = lambda a, b, f: float(np.max(np.abs(a - b) / np.maximum(np.abs(b), f)))
    log(f"[bench] global neighbourhood: build {build * 1e3:.0f} ms, {len(t)} targets in "
        f"{dt * 1e3:.1f} ms (fp64 build {dt64 * 1e3:.1f} ms); oracle {dcpu:.2f} s on {cores} threads")
    return {"data": n, "unknowns": n + 1, "targets": len(t), "build_seconds": build,
            "predict_seconds": dt, "targets_per_s": len(t) / dt,
            "includes": "host buffers in and out, copies included",
            "fp64_gpu_build": {"predict_seconds": dt64, "targets_per_s": len(t) / dt64,
                               "mixed_over_fp64": dt64 / dt,
                               "max_rel_value": rel(out64.value, ref["value"], vs),
                               "max_rel_variance": rel(out64.variance, ref["variance"], 1e-3)},
            "cpu_targets_per_s": len(t) / dcpu, "cpu_cores": cores, "cpu_seconds_incl_factor": dcpu,
            "max_rel_value": rel(out.value, ref["value"], vs),
            "max_rel_variance": rel(out.variance, ref["variance"], 1e-3),
            "max_rel_lagrange": rel(out.lagrange, ref["lagrange"], 1.0)}


def block_bench(args, log):
    """Block kriging (kriging.rs:674-838): 2-D ordinary kriging of 100,000
    points (uniform in 10 x 10 km, 10 + field, nugget 0.1 + Sph(1, 1500 m)),
    32 nearest neighbours, 20 x 20 m blocks discretised 4 x 4 at every cell of
    a 512 x 512 grid (predict_block_grid); the oracle's predict_block on a
    sample of 2,000 blocks on all host cores."""
    import geostat_rs as G
    from geostat_rs.model import Structure, VariogramModel
    n = 100_000
    c = G.rng_uniform(SEED + 41, 2 * n).reshape(n, 2) * 10000.0
    m = VariogramModel(0.1, [Structure("spherical", 1.0, 1500.0)])
    v = 10.0 + W.rff_field(c, m, 2048, SEED + 42)
    k = G.Kriging.new(G.PointSet(c, v), m, G.KrigingConfig(max_neighbors=32))
    lo, hi, nc, bs, disc = [0.0, 0.0], [10000.0, 10000.0], [512, 512], [20.0, 20.0], [4, 4]
    k.predict_block_grid(lo, hi, nc, bs, disc)
    ts = []
    for _ in range(3):
        t1 = time.perf_counter()
        val, var = k.predict_block_grid(lo, hi, nc, bs, disc)
        ts.append(time.perf_counter() - t1)
    dt = statistics.median(ts)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as O
    from geostat_rs.io import grid_centers
    cen = grid_centers(lo, hi, nc)
    pick = np.sort(np.random.default_rng(SEED).choice(len(cen), 2000, replace=False))
    off = G.block_offsets(bs, disc)
    t1 = time.perf_counter()
    ref = O.krige_block(c, v, m, cen[pick], off, max_neighbors=32)
    dcpu = time.perf_counter() - t1
    vs = float(np.mean(np.abs(v)))
    rel = lambda a, b, f: float(np.max(np.abs(a - b) / np.maximum(np.abs(b), f)))
    nb = int(np.prod(nc))
    log(f"[bench] block kriging: {nb} blocks (4 x 4 points) in {dt * 1e3:.1f} ms; oracle "
        f"{len(pick)} blocks in {dcpu:.2f} s")
    return {"blocks": nb, "discretisation": "4x4", "data": n, "max_neighbors": 32,
            "seconds": dt, "blocks_per_s": nb / dt, "includes": "grid centres, search, FP64 "
            "block systems, copies", "cpu_blocks_per_s": len(pick) / dcpu, "cpu_cores": 1,
            "cpu_kind": "port (predict_block per block)",
            "max_rel_value": rel(val[pick], ref["value"], vs),
            "max_rel_variance": rel(var[pick], ref["variance"], 1e-3)}


def vecchia_bench(args, log):
    """Vecchia log-likelihood: n = 2,000,000 points in [0,1]^2, m = 30, 16 candidates."""
    import geostat_rs as G
    from geostat_rs.model import Structure, VariogramModel
    n = args.vecchia_n
    t0 = time.time()
    c = G.rng_uniform(SEED + 5, 2 * n).reshape(n, 2)
    base = VariogramModel(0.02, [Structure("matern25", 1.0, 0.05)])
    v = 0.5 + W.rff_field(c, base, 8192, SEED + 6)
    ps = G.PointSet(c, v)
    t1 = time.time()
    plan = G.VecchiaPlan(ps, 30)
    t_plan = time.time() - t1
    log(f"[bench] vecchia data {t1 - t0:.1f}s, plan (host maxmin + device kNN) {t_plan:.1f}s")
    cands = [VariogramModel(0.02 * (1 + 0.05 * i), [Structure("matern25", 1.0 - 0.01 * i,
                                                              0.05 * (1 + 0.03 * i))])
             for i in range(16)]
    plan.loglik(cands)
    ts = []
    for _ in range(3):
        t1 = time.perf_counter()
        ll, st = plan.loglik(cands)
        ts.append(time.perf_counter() - t1)
    dt = statistics.median(ts)
    from geostat_rs import _abi
    phase = G.last_timings()
    floor_acc, fp64res, resolved = G.last_vecchia_tiers()
    t1 = time.perf_counter()
    ll64, _ = plan.loglik(cands, precision="fp64")
    dt64 = time.perf_counter() - t1
    t1 = time.perf_counter()
    ll1, _ = plan.loglik(cands[:1])
    dt1 = time.perf_counter() - t1
    # gradient batch: one BFGS round of the three reference starts
    gc = [VariogramModel(0.02 * f, [Structure("matern25", 1.0, 0.05 * f)]) for f in (0.5, 1.0, 2.0)]
    plan.loglik_grad(gc)
    t1 = time.perf_counter()
    _, _, gst = plan.loglik_grad(gc)
    dtg = time.perf_counter() - t1
    out = {"points_per_s": n * len(cands) / dt, "unit": "Vecchia points/s",
           "n": n, "m": 30, "candidates_per_batch": len(cands), "batch_ms": dt * 1e3,
           "fp64_gpu_points_per_s": n * len(cands) / dt64,
           "mixed_over_fp64": dt64 / dt,
           "single_candidate_points_per_s": n / dt1,
           "mixed_vs_fp64_max_rel_diff": float(np.max(np.abs(ll - ll64) / np.abs(ll64))),
           "gradient_points_per_s": n * len(gc) / dtg, "gradient_status_ok": bool((gst == 0).all()),
           "mixed_kernel_ms": phase[1], "fp64_resolve_ms": phase[2],
           "fp64_resolved_systems": resolved,
           "fp64_resolved_fraction": resolved / (n * len(cands)),
           "floor_accepted_systems": floor_acc,
           "fp64_residual_refined_systems": fp64res,
           "plan_seconds": t_plan, "status_ok": bool((st == 0).all())}
    # the oracle at full size: candidate 0's log-likelihood on the same plan
    # (sequential, as the reference sums), and the plan's predecessor sets at
    # sampled positions against a brute-force search among the earlier points
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as O
    po, pnb, pcnt = plan.arrays()
    if args.vecchia_oracle:
        t1 = time.perf_counter()
        ref0 = O.vecchia_loglik_plan(c, v, cands[0], po, pnb, pcnt)
        dto = time.perf_counter() - t1
        out["oracle_full_size"] = {
            "points": n, "candidate": 0, "oracle_loglik": float(ref0),
            "mixed_rel_err": float(abs(ll[0] - ref0) / abs(ref0)),
            "fp64_build_rel_err": float(abs(ll64[0] - ref0) / abs(ref0)),
            "oracle_seconds": dto, "cpu_points_per_s": n / dto, "cpu_cores": 1}
        log(f"[bench] vecchia oracle at {n} points: {dto:.1f}s, mixed rel err "
            f"{out['oracle_full_size']['mixed_rel_err']:.2e}")
    prng = np.random.default_rng(SEED + 8)
    pos = np.sort(prng.choice(np.arange(1, n), 200, replace=False))
    oc = c[po]
    bad = 0
    for k in pos:
        d = oc[:k] - oc[k]
        d2 = d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]
        keep = np.lexsort((np.arange(k), d2))[:min(30, k)]
        bad += int(not np.array_equal(po[keep], pnb[k, :pcnt[k]]))
    out["plan_spot_check"] = {"positions": len(pos), "mismatches": bad,
                              "rule": "30 nearest earlier points by (squared distance, position)"}
    # a Nelder-Mead fit with 16 starts, every round's simplex points of all
    # starts in one batched launch (bounded iterations)
    if args.mle_iters > 0:
        from geostat_rs import _abi as _ab
        t1 = time.perf_counter()
        fm, fll, fx, fne = G.vecchia_mle_nm_fit(ps, "matern25", 30, nstarts=16,
                                                max_iter=args.mle_iters, order=po)
        dtf = time.perf_counter() - t1
        out["mle_fit"] = {"starts": 16, "max_iter": args.mle_iters,
                          "rounds": int(_ab.load().gs_last_fit_rounds()), "evaluations": int(fne),
                          "seconds": dtf, "point_evaluations_per_s": fne * n / dtf,
                          "loglik": float(fll),
                          "model": {"nugget": fm.nugget, "psill": fm.structures[0].sill,
                                    "range": fm.structures[0].range},
                          "includes": "device plan from the given order, batched objective "
                                      "launches, host simplex updates"}
        log(f"[bench] vecchia 16-start NM fit: {fne} evaluations in {dtf:.1f}s")
    # Guinness-grouped likelihood (group size 8) and REML (linear trend), four
    # candidates each, on the same plan; oracle check on a 20,000-point plan
    g4 = cands[:4]
    plan.loglik_grouped(g4, 8)
    t1 = time.perf_counter()
    llg, stg = plan.loglik_grouped(g4, 8)
    dtg8 = time.perf_counter() - t1
    plan.reml_loglik(g4, drift_degree=1)
    t1 = time.perf_counter()
    llr, str_ = plan.reml_loglik(g4, drift_degree=1)
    dtr = time.perf_counter() - t1
    t1 = time.perf_counter()
    llr8, _ = plan.reml_loglik(g4, drift_degree=1, group_size=8)
    dtr8 = time.perf_counter() - t1
    small = G.VecchiaPlan(G.PointSet(c[:20000], v[:20000]), 30)
    so, snb, scnt = small.arrays()
    sg, _ = small.loglik_grouped(g4[:1], 8)
    sr, _ = small.reml_loglik(g4[:1], drift_degree=1)
    t1 = time.perf_counter()
    og = O.vecchia_loglik_grouped(c[:20000], v[:20000], g4[0], so, snb, scnt, 8)
    dto = time.perf_counter() - t1
    orr = O.vecchia_reml_loglik(c[:20000], v[:20000], g4[0], so, snb, scnt,
                                O.poly_basis(c[:20000], 1), 1)
    out["grouped"] = {"group_size": 8, "candidates": len(g4),
                      "points_per_s": n * len(g4) / dtg8, "batch_ms": dtg8 * 1e3,
                      "status_ok": bool((stg == 0).all()),
                      "over_ungrouped_ll": float(np.max(llg - ll[:4])),
                      "cpu_points_per_s": 20000 / dto, "cpu_cores": 1,
                      "oracle_check_rel": float(abs(sg[0] - og) / abs(og))}
    out["reml"] = {"drift_degree": 1, "candidates": len(g4),
                   "points_per_s": n * len(g4) / dtr, "batch_ms": dtr * 1e3,
                   "grouped8_points_per_s": n * len(g4) / dtr8,
                   "status_ok": bool((str_ == 0).all()),
                   "oracle_check_rel": float(abs(sr[0] - orr) / abs(orr))}
    log(f"[bench] vecchia grouped(8) {dtg8 * 1e3:.0f} ms, REML {dtr * 1e3:.0f} ms, "
        f"REML grouped(8) {dtr8 * 1e3:.0f} ms for {len(g4)} candidates")
    # joint prediction at args.vpred_n targets conditioning on the same data (m = 30)
    if args.vpred_n > 0:
        nt = args.vpred_n
        t = G.rng_uniform(SEED + 7, 2 * nt).reshape(nt, 2)
        t1 = time.perf_counter()
        pv, pvar = G.vecchia_predict(None, None, base, t, 30, pointset=ps)
        dtp = time.perf_counter() - t1
        out["predict"] = {"targets": nt, "targets_per_s": nt / dtp, "seconds": dtp,
                          "includes": "host max-min order of the targets, device search, "
                                      "level-scheduled solves and row merges, copies",
                          "finite": bool(np.isfinite(pv).all() and np.isfinite(pvar).all())}
        # accuracy against the oracle on a small instance of the same kind
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import pyoracle as O
        cs, ts_ = c[:20000], t[:4000]
        vs = v[:20000]
        gv, gvar = G.vecchia_predict(cs, vs, base, ts_, 30)
        rv, rvar = O.vecchia_predict(cs, vs, base, ts_, 30)
        out["predict"]["oracle_check"] = {
            "data": 20000, "targets": 4000,
            "max_rel_value": float(np.max(np.abs(gv - rv) / np.maximum(np.abs(rv), np.mean(np.abs(vs))))),
            "max_rel_variance": float(np.max(np.abs(gvar - rvar) / np.maximum(np.abs(rvar), 1e-3)))}
    return out


CL_N = 1_000_000
CL_EXTENT = 10000.0
CL_GRID = 2048
CL_SEARCH = dict(max_per_octant=16, max_neighbors=64, min_neighbors=4)
CL_KINDS = ("ordinary", "universal", "external_drift")


def clustered_setup(n=CL_N, grid=CL_GRID, extent=CL_EXTENT, nblobs=500):
    """Clustered uneven workload: n 2-D points (70 % in Gaussian blobs of
    sigma 15 m, 30 % uniform) over [0, extent]^2; Matern 3/2 field (sill 1,
    range 500 m, ratio 0.5 at azimuth 45, no nugget); one U[0,1] covariate;
    the grid x grid cell centres split into three bands of rows: ordinary,
    universal (linear drift) and external-drift kriging, all with octant
    search (4 x 16, at most 64, at least 4)."""
    import geostat_rs as G
    from geostat_rs.model import Structure, VariogramModel
    c = W.clustered_points(n, extent, nblobs, 15.0, 0.7, SEED + 21)
    m = VariogramModel(0.0, [Structure.with_anisotropy("matern15", 1.0, 500.0, 45.0, 0.5)])
    v = W.rff_field(c, m, 4096, SEED + 22)
    cov = G.rng_uniform(SEED + 23, n)
    g = (np.arange(grid) + 0.5) * (extent / grid)
    yy, xx = np.meshgrid(g, g, indexing="ij")
    tg = np.stack([xx.ravel(), yy.ravel()], 1)
    tcov = G.rng_uniform(SEED + 24, len(tg))
    cuts = [0, (grid // 3) * grid, (2 * grid // 3) * grid, grid * grid]
    ps = G.PointSet(c, v)
    preds = [G.Kriging.new(ps, m, G.KrigingConfig(**CL_SEARCH)),
             G.Kriging.new(ps, m, G.KrigingConfig("universal", degree=1, **CL_SEARCH)),
             G.Kriging.with_external_drift(ps, m, G.KrigingConfig("external_drift", n_vars=1,
                                                                  **CL_SEARCH),
                                           cov.reshape(-1, 1))]
    return c, v, m, cov, tg, tcov, cuts, preds


def clustered_bench(args, log):
    """The clustered uneven workload as one CUDA-graph replay per step."""
    import torch
    import geostat_rs as G
    from geostat_rs import _abi
    lib = _abi.load()
    t0 = time.time()
    c, v, m, cov, tg, tcov, cuts, preds = clustered_setup()
    nt = len(tg)
    log(f"[bench] clustered set-up {time.time() - t0:.1f}s")
    dev = torch.device("cuda")
    cols = [torch.from_numpy(np.ascontiguousarray(tg[:, d])).to(dev) for d in range(2)]
    tdr = torch.from_numpy(np.ascontiguousarray(tcov)).to(dev)
    out_v = torch.empty(nt, dtype=torch.float64, device=dev)
    out_var = torch.empty(nt, dtype=torch.float64, device=dev)
    out_st = torch.empty(nt, dtype=torch.uint8, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    s = torch.cuda.Stream()
    sp = s.cuda_stream

    def enqueue(prec, asynchronous):
        for b, k in enumerate(preds):
            lo, hi = cuts[b], cuts[b + 1]
            k.predict_device(hi - lo, cols[0][lo:].data_ptr(), cols[1][lo:].data_ptr(), None,
                             out_v[lo:].data_ptr(), out_var[lo:].data_ptr(),
                             out_st[lo:].data_ptr(), prec, stream=sp,
                             tdrift_ptr=tdr[lo:].data_ptr() if b == 2 else None,
                             asynchronous=asynchronous)

    # ordinary calls first: autotuning (per kind and size class), tables;
    # phases and re-solve counts per kind from the second call
    kinds = {}
    for rep in range(2):
        for b, k in enumerate(preds):
            lo, hi = cuts[b], cuts[b + 1]
            k.predict_device(hi - lo, cols[0][lo:].data_ptr(), cols[1][lo:].data_ptr(), None,
                             out_v[lo:].data_ptr(), out_var[lo:].data_ptr(),
                             out_st[lo:].data_ptr(), "mixed", stream=sp,
                             tdrift_ptr=tdr[lo:].data_ptr() if b == 2 else None)
            if rep == 1:
                ph = G.last_timings()
                run, bins, spc, src = k.tiles(hi - lo)
                kinds[CL_KINDS[b]] = {
                    "targets": hi - lo, "search_ms": ph[0], "mixed_ms": ph[1],
                    "fp64_resolve_ms": ph[2], "total_ms": ph[3],
                    "fp64_resolved": int(lib.gs_last_fallbacks()),
                    "lu_resolved": int(lib.gs_last_lu_resolves()),
                    "tiles": {"run": run, "bins": bins, "systems_per_block": spc,
                              "source": src}}
    torch.cuda.synchronize()
    l0 = lib.gs_launch_count()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        enqueue("mixed", True)
    nodes = lib.gs_launch_count() - l0
    torch.cuda.synchronize()
    for _ in range(args.warmup):
        g.replay()
    torch.cuda.synchronize()
    cur = torch.cuda.current_stream()
    times = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(cur)
        g.replay()
        e1.record(cur)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    ms = statistics.mean(times)
    mixed_v = out_v.cpu().numpy()
    mixed_var = out_var.cpu().numpy()
    st = out_st.cpu().numpy()
    # the plain FP64 build on the same job
    t64 = []
    for _ in range(2):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        enqueue("fp64", False)
        e1.record(s)
        torch.cuda.synchronize()
        t64.append(e0.elapsed_time(e1))
    ms64 = min(t64)
    fp64_v = out_v.cpu().numpy()
    log(f"[bench] clustered: {ms:.1f} ms/step (graph replay), fp64 build {ms64:.1f} ms")
    # oracle on a sample of each band
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as O
    O.build()
    cores = os.cpu_count() or 1
    rng = np.random.RandomState(11)
    vs = float(np.mean(np.abs(v)))
    acc, cpu_t, cpu_n = {}, 0.0, 0
    for b, kind in enumerate(CL_KINDS):
        lo, hi = cuts[b], cuts[b + 1]
        idx = np.sort(rng.choice(np.arange(lo, hi), args.cl_sample, replace=False))
        t1 = time.perf_counter()
        ref = O.krige(c, v, m, tg[idx], method=kind, degree=1,
                      drift=cov.reshape(-1, 1) if b == 2 else None,
                      target_drift=tcov[idx].reshape(-1, 1) if b == 2 else None,
                      nthreads=cores, **CL_SEARCH)
        cpu_t += time.perf_counter() - t1
        cpu_n += len(idx)
        rel = lambda a, r, f: float(np.max(np.abs(a - r) / np.maximum(np.abs(r), f)))
        acc[kind] = {"mixed_max_rel_value": rel(mixed_v[idx], ref["value"], vs),
                     "mixed_max_rel_variance": rel(mixed_var[idx], ref["variance"], 1e-3),
                     "fp64_max_rel_value": rel(fp64_v[idx], ref["value"], vs),
                     "status_match": bool(((st[idx] & 0x3f) == ref["status"]).all())}
    log(f"[bench] clustered oracle: {cpu_n} targets in {cpu_t:.1f}s on {cores} threads")
    return {"workload": "clustered uneven kriging: n=1,000,000 2-D points (70% in 500 Gaussian "
                        "blobs, sigma 15 m; 30% uniform) over [0,10000]^2 m; Matern 3/2 (sill 1, "
                        "range 500 m, ratio 0.5, azimuth 45, no nugget); 2048x2048 grid targets "
                        "(4,194,304) in three bands: ordinary, universal (linear drift), external "
                        "drift (one U[0,1] covariate); octant search 4 x 16, max 64, min 4",
            "value": nt / (ms * 1e-3), "unit": "kriged targets/s", "ms_per_step": ms,
            "steps": args.steps, "warmup": args.warmup,
            "step": "one CUDA-graph replay of the three passes (search, binned mixed solve, "
                    "device-side routing, FP64 LDL^T and LU re-solves)",
            "graph_kernel_nodes": nodes,
            "fp64_gpu_build": {"value": nt / (ms64 * 1e-3), "ms_per_step": ms64,
                               "mixed_over_fp64": ms64 / ms},
            "kinds": kinds, "accuracy": acc,
            "fp64_resolved_fraction": sum(k["fp64_resolved"] for k in kinds.values()) / nt,
            "cpu_baseline": {"value": cpu_n / cpu_t, "unit": "kriged targets/s", "cores": cores,
                             "kind": "port",
                             "sample": f"{args.cl_sample} random targets per band"},
            "l2": "flushed between steps (256 MiB write)"}


def serving_bench(args, log):
    """Serving loop on eight resident data sets -- 10k, 50k, 200k, 500k, 1M,
    1M, 2M and 4M points; 2-D (uniform in 1000 x 1000 m, nugget 0.1 +
    Sph(1, 200 m)): 10k, 200k, 1M, 2M; 3-D (the 3-D workload's box and model):
    50k, 500k, 1M, 4M -- each with ordinary-kriging predictors at n_max 16,
    32, 48 and 64, and Vecchia plans (m = 30) on the 2-D sets of 10k, 200k and
    1M points.  Poisson arrivals at 200 requests/s: 85 % predictions
    (log-uniform target counts in [1, 1e6], random data set and n_max), 15 %
    Vecchia log-likelihoods at a new parameter vector.  The first requests of
    the same stream are then served again at the same arrival times by the
    mixed path and by the plain FP64 build, and compared."""
    import geostat_rs as G
    from geostat_rs.model import Structure, VariogramModel
    rng = np.random.default_rng(SEED + 11)
    t0 = time.time()
    m2 = VariogramModel(0.1, [Structure("spherical", 1.0, 200.0)])
    m3 = make_model()
    specs = [(2, 10_000), (3, 50_000), (2, 200_000), (3, 500_000), (2, 1_000_000),
             (3, 1_000_000), (2, 2_000_000), (3, 4_000_000)]
    nmaxes = (16, 32, 48, 64)
    srv = G.Server(mem_budget_bytes=48 << 30, executors=3)
    kds, boxes, vds, keep = [], [], [], []
    for q, (dim, n) in enumerate(specs):
        box = np.array([1000.0, 1000.0]) if dim == 2 else np.asarray(BOX)
        mdl = m2 if dim == 2 else m3
        cc = G.rng_uniform(SEED + 100 + q, dim * n).reshape(n, dim) * box
        vv = W.rff_field(cc, mdl, 1024, SEED + 200 + q)
        ps = G.PointSet(cc, vv)
        row = []
        warm = G.rng_uniform(SEED + 300 + q, dim * 131072).reshape(-1, dim) * box
        for km in nmaxes:
            k = G.Kriging.new(ps, mdl, G.KrigingConfig(max_neighbors=km))
            k.predict_many(warm)  # registration: autotunes the predictor's launch shape
            keep.append(k)
            row.append(srv.add_kriging(k))
        kds.append(row)
        boxes.append(box)
        if dim == 2 and n <= 1_000_000:
            plan = G.VecchiaPlan(ps, 30)
            plan.loglik([VariogramModel(0.05, [Structure("matern25", 1.0, 60.0)])])
            keep.append(plan)
            vds.append(srv.add_vecchia(plan))
    log(f"[bench] serving set-up {time.time() - t0:.1f}s (8 data sets, 32 predictors, "
        f"{len(vds)} Vecchia plans)")
    nreq, rate = args.serve_requests, 200.0
    arrivals = np.cumsum(rng.exponential(1.0 / rate, nreq))
    jobs = []
    for q in range(nreq):
        if rng.uniform() < 0.15:
            f = rng.uniform(0.5, 2.0)
            mdl = VariogramModel(0.05 * f, [Structure("matern25", 1.0, 60.0 * f)])
            jobs.append(("ll", vds[int(rng.integers(0, len(vds)))], mdl))
        else:
            d = int(rng.integers(0, len(specs)))
            km = int(rng.integers(0, len(nmaxes)))
            nt = int(np.exp(rng.uniform(0.0, np.log(1e6))))
            t = rng.uniform(0, 1, size=(nt, specs[d][0])) * boxes[d]
            jobs.append(("p", kds[d][km], t))
    # warm-up: one request of each kind
    srv.wait(srv.submit_predict(kds[0][0], np.full((10, 2), 500.0)))
    srv.wait(srv.submit_loglik(vds[0], m2))
    _, _, done0, launches0 = srv.stats()

    def serve(subset, paced):
        reqs, targets = [], 0
        start = time.perf_counter()
        for q in subset:
            kind, ds, arg = jobs[q]
            if paced:
                delay = start + arrivals[q] - time.perf_counter()
                if delay > 0:
                    time.sleep(delay)
            reqs.append(srv.submit_predict(ds, arg) if kind == "p" else srv.submit_loglik(ds, arg))
            if kind == "p":
                targets += len(arg)
        lat = np.asarray([srv.wait(r) for r in reqs])
        return reqs, lat, time.perf_counter() - start, targets

    reqs, lat, wall, targets = serve(range(nreq), True)
    _, _, done, launches = srv.stats()
    # the first requests of the stream again, paced at the same arrival
    # times, through the mixed path and through the plain FP64 build
    nsub = min(nreq, args.serve_fp64_requests)
    reqsm, latm, wallm, targetsm = serve(range(nsub), True)
    srv.set_precision("fp64")
    reqs64, lat64, wall64, targets64 = serve(range(nsub), True)
    srv.set_precision("mixed")
    worst_v = worst_var = worst_ll = 0.0
    status_ok = True
    for q in range(nsub):
        (kind, ds, arg), a_, b_ = jobs[q], reqs[q].out, reqs64[q].out
        if kind == "p":
            vs = max(float(np.mean(np.abs(b_[0][np.isfinite(b_[0])]))) if len(b_[0]) else 1.0, 1e-300)
            ok = np.isfinite(b_[0])
            worst_v = max(worst_v, float(np.max(np.abs(a_[0][ok] - b_[0][ok]) /
                                                np.maximum(np.abs(b_[0][ok]), vs), initial=0.0)))
            worst_var = max(worst_var, float(np.max(np.abs(a_[1][ok] - b_[1][ok]) /
                                                    np.maximum(np.abs(b_[1][ok]), 1e-3),
                                                    initial=0.0)))
            status_ok = status_ok and bool(((a_[2] & 0x3f) == (b_[2] & 0x3f)).all())
        else:
            worst_ll = max(worst_ll, abs(a_[0][0] - b_[0][0]) / abs(b_[0][0]))
    srv.close()
    log(f"[bench] serving: p50 {np.percentile(lat, 50):.1f} ms, p99 {np.percentile(lat, 99):.1f} ms, "
        f"{targets / wall / 1e6:.1f} M targets/s; fp64 build on {nsub} requests "
        f"{targets64 / wall64 / 1e6:.2f} M targets/s")
    return {"requests": nreq, "arrival_rate_per_s": rate, "executors": 3,
            "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "mean_ms": float(lat.mean()), "wall_s": wall, "targets": targets,
            "targets_per_s": targets / wall, "requests_per_s": nreq / wall,
            "launches": launches - launches0,
            "same_stream_subset": {"requests": nsub, "paced": True, "targets": targetsm,
                                   "mixed_targets_per_s": targetsm / wallm,
                                   "mixed_p50_ms": float(np.percentile(latm, 50)),
                                   "mixed_p99_ms": float(np.percentile(latm, 99)),
                                   "fp64_targets_per_s": targets64 / wall64,
                                   "fp64_p50_ms": float(np.percentile(lat64, 50)),
                                   "fp64_p99_ms": float(np.percentile(lat64, 99)),
                                   "mixed_over_fp64_wall": wall64 / wallm},
            "fp64_gpu_build": {"requests": nsub, "paced": True, "targets": targets64,
                               "targets_per_s": targets64 / wall64,
                               "p50_ms": float(np.percentile(lat64, 50)),
                               "p99_ms": float(np.percentile(lat64, 99)),
                               "max_rel_value": worst_v, "max_rel_variance": worst_var,
                               "max_rel_loglik": worst_ll, "status_match": status_ok,
                               "tolerance": "1e-9 (floors: mean |estimate|, 1e-3 sill)"},
            "datasets": "2-D 10k/200k/1M/2M (1000 x 1000 m, 0.1 + Sph(1, 200 m)); 3-D "
                        "50k/500k/1M/4M (2000 x 2000 x 200 m, the 3-D workload's model); "
                        "ordinary kriging at n_max 16/32/48/64 each; Vecchia plans m = 30 on "
                        "the 2-D 10k/200k/1M sets",
            "mix": "85% predictions (target count log-uniform in [1, 1e6]), 15% log-likelihoods"}


# ------------------------------------------------------------- reference --
def run_reference(args, rank, world):
    if rank != 0:
        return None
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as O
    O.build()
    from geostat_rs.model import Structure, VariogramModel  # pure-Python model description
    cores = os.cpu_count() or 1
    u = O.rng_uniform(SEED, 3 * N_DATA).reshape(N_DATA, 3) * np.asarray(BOX)
    model = VariogramModel(0.05, [Structure.with_rotation("spherical", 0.6, 300.0, 30.0, 10.0, 0.0,
                                                          0.5, 40.0 / 300.0),
                                  Structure("exponential", 0.35, 800.0)])
    # the same random-Fourier-feature field values as the GPU arm's workload,
    # generated before any timing (input preparation, not the timed path)
    vals = W.rff_field(u, model, 4096, SEED + 1)
    tg = grid_targets()
    rng = np.random.RandomState(11)
    probe = rng.choice(len(tg), 1000, replace=False)
    t0 = time.perf_counter()
    O.krige(u, vals, model, tg[probe], max_neighbors=K_NEIGH, nthreads=cores)
    per = (time.perf_counter() - t0) / len(probe)
    ns = int(min(len(tg), max(1000, args.ref_step_seconds / max(per, 1e-9))))
    for _ in range(args.warmup):
        idx = rng.choice(len(tg), min(ns, 2000), replace=False)
        O.krige(u, vals, model, tg[idx], max_neighbors=K_NEIGH, nthreads=cores)
    times = []
    for _ in range(args.steps):
        idx = np.sort(rng.choice(len(tg), ns, replace=False))
        t0 = time.perf_counter()
        O.krige(u, vals, model, tg[idx], max_neighbors=K_NEIGH, nthreads=cores)
        times.append(time.perf_counter() - t0)
    mean = statistics.mean(times)
    value = ns / mean
    return {"impl": "reference", "metric": METRIC, "value": value, "unit": "kriged targets/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": mean * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(len(tg), world),
            "cpu_baseline": {"value": value, "unit": "kriged targets/s", "cores": cores,
                             "kind": "port",
                             "sample": f"{ns} random grid targets per step (same data size, model, "
                                       "n_max=64); the reference's Rust crate cannot be built "
                                       "without cargo, so its FP64 C++ restatement runs"},
            "e2e": {"value": value, "unit": "kriged targets/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}


def profile_case(args):
    """Small fixed case for ncu: the benchmark's data, a prefix of its targets."""
    import torch
    import geostat_rs as G
    if args.profile_case:
        coords = make_coords()
        model = make_model()
        values = W.rff_field(coords, model, 4096, SEED + 1)
        kr = G.Kriging.new(G.PointSet(coords, values), model, G.KrigingConfig(max_neighbors=K_NEIGH))
        tg = grid_targets()[:args.profile_case]
        for _ in range(2):
            v, var = kr.predict_many(tg)
        torch.cuda.synchronize()
        print(f"profile case: {len(tg)} targets, mean estimate {np.nanmean(v):.6f}")
    if args.profile_clustered:
        # the clustered workload's data with a band of grid rows as targets
        c, v, m, cov, tg, tcov, cuts, preds = clustered_setup()
        t = tg[CL_GRID * 1000:CL_GRID * 1000 + args.profile_clustered]
        for _ in range(2):
            r = preds[0].predict_many(t, "mixed", full=True)
        torch.cuda.synchronize()
        print(f"profile clustered: {len(t)} targets, mean estimate {np.nanmean(r.value):.6f}")
    if args.profile_global:
        # the global-neighbourhood workload; the first call prepares the
        # system's matrix-product form, the second is the steady state
        n, c, v, m, t = global_setup()
        t = t[:args.profile_global]
        k = G.Kriging.new(G.PointSet(c, v), m)
        for _ in range(2):
            out = k.predict_many(t, full=True)
        torch.cuda.synchronize()
        print(f"profile global: {len(t)} targets, mean estimate {np.nanmean(out.value):.6f}")
    if args.profile_vecchia:
        from geostat_rs.model import Structure, VariogramModel
        n = args.profile_vecchia
        c = G.rng_uniform(SEED + 5, 2 * n).reshape(n, 2)
        base = VariogramModel(0.02, [Structure("matern25", 1.0, 0.05)])
        v = 0.5 + W.rff_field(c, base, 1024, SEED + 6)
        plan = G.VecchiaPlan(G.PointSet(c, v), 30)
        cands = [VariogramModel(0.02 * (1 + 0.05 * i), [Structure("matern25", 1.0, 0.05)])
                 for i in range(16)]
        for _ in range(2):
            ll, st = plan.loglik(cands)
        print(f"profile vecchia: {n} points, loglik[0] {ll[0]:.6f}")
    if args.profile_reml:
        from geostat_rs.model import Structure, VariogramModel
        n = args.profile_reml
        c = G.rng_uniform(SEED + 5, 2 * n).reshape(n, 2)
        base = VariogramModel(0.02, [Structure("matern25", 1.0, 0.05)])
        v = 0.5 + W.rff_field(c, base, 1024, SEED + 6)
        # m = 40: beyond the mixed warp kernel, every point on the FP64 block kernel
        plan = G.VecchiaPlan(G.PointSet(c, v), 40)
        cands = [VariogramModel(0.02 * (1 + 0.05 * i), [Structure("matern25", 1.0, 0.05)])
                 for i in range(4)]
        for _ in range(2):
            ll, st = plan.reml_loglik(cands, drift_degree=1)
        print(f"profile reml: {n} points, loglik[0] {ll[0]:.6f}")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--ref-step-seconds", type=float, default=8.0)
    ap.add_argument("--vecchia-n", type=int, default=2_000_000)
    ap.add_argument("--no-vecchia", action="store_true")
    ap.add_argument("--no-clustered", action="store_true",
                    help="skip the clustered uneven workload")
    ap.add_argument("--no-block", action="store_true", help="skip the block-kriging leg")
    ap.add_argument("--no-global", action="store_true",
                    help="skip the global-neighbourhood leg")
    ap.add_argument("--cv-sample", type=int, default=40,
                    help="oracle points of the leave-one-out leg (0: skip the leg)")
    ap.add_argument("--cl-sample", type=int, default=200,
                    help="oracle targets per band of the clustered workload")
    ap.add_argument("--vecchia-oracle", type=int, default=1,
                    help="time the oracle's full-size Vecchia log-likelihood (0: skip)")
    ap.add_argument("--mle-iters", type=int, default=12,
                    help="Nelder-Mead iterations per start of the 16-start fit (0: skip)")
    ap.add_argument("--vpred-n", type=int, default=500_000,
                    help="targets of the Vecchia joint-prediction timing (0: skip)")
    ap.add_argument("--serve-fp64-requests", type=int, default=150,
                    help="leading requests of the serving stream re-served, paced, by the mixed "
                         "path and by the FP64 build")
    ap.add_argument("--serve-requests", type=int, default=1000,
                    help="requests of the serving-loop run (0: skip)")
    ap.add_argument("--profile-case", type=int, default=0,
                    help="run one mixed-precision pass over the first N grid targets and exit "
                         "(the small case for ncu captures)")
    ap.add_argument("--profile-clustered", type=int, default=0,
                    help="run two ordinary-kriging passes of the clustered workload over N "
                         "grid targets and exit")
    ap.add_argument("--profile-global", type=int, default=0,
                    help="run two mixed-precision passes of the global-neighbourhood workload "
                         "over its first N grid targets (at most 10,000) and exit")
    ap.add_argument("--profile-vecchia", type=int, default=0,
                    help="run one 16-candidate Vecchia batch on N points and exit")
    ap.add_argument("--profile-reml", type=int, default=0,
                    help="run a 4-candidate Vecchia REML batch (linear trend, m = 40) on N "
                         "points and exit")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1 and args.impl == "ours":
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        torch.distributed.init_process_group("nccl")
    if (args.profile_case or args.profile_vecchia or args.profile_clustered or args.profile_reml
            or args.profile_global):
        profile_case(args)
        return
    if args.impl == "reference":
        res = run_reference(args, rank, world)
    else:
        res = run_ours(args, rank, world)
    if rank == 0 and res is not None:
        print(json.dumps(res), flush=True)
    if world > 1 and args.impl == "ours":
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
