"""Builds libgeostat_gb300.so in-tree for sm_103a (GB300).

Each CUDA translation unit is compiled in parallel with nvcc, then linked
into geostat_rs/_lib/libgeostat_gb300.so (the drop-in library).  The
benchmark's and tests' synthetic workloads and probes are a second library,
gs_workload/_lib/libgeostat_workload.so, linked against the first.  Host code is compiled with
-ffp-contract=off: the host max-min ordering and Nelder-Mead driver must take
the same branches as the reference's (never-contracted) Rust arithmetic.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "geostat_rs", "_lib")
OBJ_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libgeostat_gb300.so")
SOURCES = ["gs_host.cu", "gs_search.cu", "gs_krige.cu", "gs_api.cu", "gs_noalloc.cu", "gs_serve.cu", "gs_vecchia.cu",
           "gs_io.cpp"]
WL_CSRC = os.path.join(HERE, "gs_workload", "csrc")
WL_SOURCES = ["gs_synth.cu", "gs_probe.cu"]
WL_OUT_DIR = os.path.join(HERE, "gs_workload", "_lib")
WL_LIB = os.path.join(WL_OUT_DIR, "libgeostat_workload.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
         "--expt-relaxed-constexpr", "-Xptxas", "-O3"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _needs(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(WL_OUT_DIR, exist_ok=True)
    os.makedirs(OBJ_DIR, exist_ok=True)
    nvcc = _nvcc()
    include = os.path.join(os.path.dirname(HERE), "include")
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(include, "geostat_gb300.h"))
    wl_headers = headers + [os.path.join(WL_CSRC, f) for f in os.listdir(WL_CSRC)
                            if f.endswith((".h", ".cuh"))]
    jobs = []
    units = [(os.path.join(CSRC, s), headers, []) for s in SOURCES]
    units += [(os.path.join(WL_CSRC, s), wl_headers, ["-I", CSRC, "-I", include, "-I", WL_CSRC])
              for s in WL_SOURCES]
    for s, deps, inc in units:
        o = os.path.join(OBJ_DIR, os.path.splitext(os.path.basename(s))[0] + ".o")
        if _needs(o, [s] + deps) or ptxas_info:
            cmd = [nvcc, *ARCH, *FLAGS, *inc, "-c", s, "-o", o]
            if ptxas_info:
                cmd += ["-Xptxas", "-v"]
            jobs.append((os.path.basename(s), cmd))
    objs = [os.path.join(OBJ_DIR, os.path.splitext(s)[0] + ".o") for s in SOURCES]
    wl_objs = [os.path.join(OBJ_DIR, os.path.splitext(s)[0] + ".o") for s in WL_SOURCES]

    def run(job):
        name, cmd = job
        r = subprocess.run(cmd, capture_output=True, text=True)
        return name, r

    failed = []
    with cf.ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        for name, r in ex.map(run, jobs):
            if verbose or ptxas_info:
                sys.stdout.write(r.stdout + r.stderr)
            if r.returncode != 0:
                failed.append((name, r.stdout + r.stderr))
    if failed:
        raise RuntimeError("nvcc failed:\n" + "\n".join(f"[{n}]\n{o}" for n, o in failed))
    if _needs(LIB, objs):
        cmd = [nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    if _needs(WL_LIB, wl_objs + [LIB]):
        rpath = os.path.relpath(OUT_DIR, WL_OUT_DIR)
        cmd = [nvcc, *ARCH, "-shared", "-o", WL_LIB, *wl_objs, "-L", OUT_DIR, "-lgeostat_gb300",
               "-lcudart", "-Xlinker", f"-rpath,$ORIGIN/{rpath}"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed (workload library):\n" + r.stdout + r.stderr)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, ptxas_info="-v" in sys.argv))
