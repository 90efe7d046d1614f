"""CPU tests of the product's host side: the C-ABI library loads and exports
every symbol its header declares, and the host algorithms that must match the
reference exactly (max-min ordering, Nelder-Mead, xoshiro256++) do so against
the oracle.  No compute call here needs a GPU."""
import os
import re

import numpy as np
import pytest

import pyoracle as O
import geostat_rs as G
from geostat_rs import _abi
from geostat_rs.model import Anisotropy, Structure, VariogramModel

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "geostat_gb300.h")


def _build_lib():
    import importlib.util
    spec = importlib.util.spec_from_file_location("gs_build", os.path.join(ROOT, "geostat-rs_gb300",
                                                                           "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build()


@pytest.fixture(scope="module", autouse=True)
def built():
    _build_lib()
    O.build()


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"\b(gs_[a-z0-9_]+)\s*\(", text)) - {"gs_objective_fn"})


def test_library_exports_every_declared_symbol():
    lib = _abi.load()
    names = declared_symbols()
    assert len(names) >= 25
    for n in names:
        assert hasattr(lib, n), n
    # and the ctypes signature table covers exactly the declared entry points
    assert sorted(_abi.SIGNATURES) == names


def test_library_has_no_unresolved_internal_symbols():
    """Every library-internal function the translation units call is defined
    in the library itself (a declaration that drifted from its definition
    would only fail when the library is loaded with immediate binding)."""
    import shutil
    import subprocess
    nm = shutil.which("nm")
    if nm is None:
        pytest.skip("nm not available")
    out = subprocess.run([nm, "-D", "--undefined-only", _abi.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    bad = [l for l in out.splitlines() if " gs_" in l or "_ZN2gs" in l or "_ZN12_GLOBAL" in l]
    assert not bad, bad


def test_abi_version_and_struct_layout(tmp_path):
    """The ctypes structs match the C header's layout (compiled with gcc)."""
    import ctypes as C
    import subprocess
    assert _abi.load().gs_abi_version() == 2
    src = tmp_path / "layout.c"
    src.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "geostat_gb300.h"\n'
        'int main(void){printf("%zu %zu %zu %zu %zu %zu\\n", sizeof(gs_model), sizeof(gs_structure),'
        ' sizeof(gs_kcfg), offsetof(gs_model, s), offsetof(gs_kcfg, search_radius),'
        ' offsetof(gs_structure, rake_deg)); return 0;}\n')
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                   check=True)
    got = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True,
                                          check=True).stdout.split()]
    assert got == [C.sizeof(_abi.Model), C.sizeof(_abi.Structure), C.sizeof(_abi.Kcfg),
                   _abi.Model.s.offset, _abi.Kcfg.search_radius.offset,
                   _abi.Structure.rake_deg.offset]
    assert C.sizeof(_abi.Model) == C.sizeof(O._Model)
    assert C.sizeof(_abi.Kcfg) == C.sizeof(O._Kcfg)


def test_product_rng_matches_reference_stream():
    for seed in (0, 1, 42, 2**63 + 5):
        assert G.rng_uniform(seed, 1000).tobytes() == O.rng_uniform(seed, 1000).tobytes()
        assert G.rng_normal(seed, 1000).tobytes() == O.rng_normal(seed, 1000).tobytes()


@pytest.mark.parametrize("seed,n,dim", [(3, 400, 2), (11, 400, 2), (29, 2000, 2), (5, 1500, 3)])
def test_host_maxmin_matches_oracle(seed, n, dim):
    if dim == 2:
        c, _ = O.test_field_2d(n, seed)
    else:
        c, _ = O.test_field_3d(n, seed)
    assert G.maxmin_order(c).tolist() == O.maxmin_order(c).tolist()


def test_host_maxmin_degenerate_inputs():
    line = np.array([[i * 10.0, 5.0] for i in range(60)])
    assert G.maxmin_order(line).tolist() == O.maxmin_order(line).tolist()
    one = np.array([[1.0, 2.0]])
    assert G.maxmin_order(one).tolist() == [0]


def _maxmin_layout_cases():
    """Inputs for both spatial layouts of the host ordering: spread-out sets
    (the uniform grid, including exact distance ties on lattices and
    coordinates far from the origin, where the grid's ball bounds must
    absorb rounding) and crowded ones (the k-d tree)."""
    rng = np.random.default_rng(17)
    g2 = np.stack(np.meshgrid(np.arange(30.0), np.arange(30.0)), -1).reshape(-1, 2)
    g3 = np.stack(np.meshgrid(np.arange(9.0), np.arange(9.0), np.arange(9.0)), -1).reshape(-1, 3)
    blobs = rng.random((40, 2))[rng.integers(0, 40, 4000)] + 0.003 * rng.standard_normal((4000, 2))
    crowd = rng.random((3000, 2))
    crowd[1:2970] = 0.5 + 1e-6 * rng.random((2969, 2))
    dup = rng.random((300, 3))
    return {
        "lattice 2-D": g2,
        "lattice 3-D": g3,
        "lattice, flat z": np.c_[g2, np.zeros(len(g2))],
        "far from the origin 2-D": 1e6 + 1e3 * rng.random((5000, 2)),
        "far from the origin 3-D": np.c_[5e5 + 1e4 * rng.random((3000, 2)), 100 * rng.random(3000)],
        "rounded coordinates": np.round(rng.random((5000, 2)) * 50) / 50,
        "blobs": blobs,
        "one crowded cell": crowd,
        "duplicates": np.r_[dup, dup[:120]],
        "identical points": np.ones((40, 2)),
        "tiny extent": 1e-300 * rng.random((500, 2)),
    }


@pytest.mark.parametrize("name", list(_maxmin_layout_cases()))
def test_host_maxmin_layouts_match_oracle(name):
    c = np.ascontiguousarray(_maxmin_layout_cases()[name], dtype=np.float64)
    assert G.maxmin_order(c).tolist() == O.maxmin_order(c).tolist()


def test_host_maxmin_matches_exact_traversal():
    # the O(n^2) farthest-point traversal of the reference's test helper
    # (vecchia.rs:2244-2275) on both layouts
    rng = np.random.default_rng(23)
    for c in (rng.random((700, 2)), rng.random((600, 3)),
              np.r_[rng.random((10, 2)), 0.5 + 1e-7 * rng.random((590, 2))]):
        assert G.maxmin_order(c).tolist() == O.maxmin_order_brute(c).tolist()


def test_host_maxmin_non_finite_input_gives_a_permutation():
    # point sets reject non-finite coordinates; the ordering itself still
    # returns a permutation for them (no ordering is defined by the reference)
    rng = np.random.default_rng(29)
    c = rng.random((500, 2))
    c[7, 0] = np.nan
    c[100, 1] = np.inf
    assert sorted(G.maxmin_order(c).tolist()) == list(range(500))


def test_nelder_mead_state_machine_matches_reference_sequence():
    rosen = lambda x: (1 - x[0]) ** 2 + 100 * (x[1] - x[0] ** 2) ** 2
    for starts in ([[-1.2, 1.0]], [[-1.2, 1.0], [0.5, 0.5], [2.0, -1.0]]):
        xa, fa = G.nelder_mead_multistart(rosen, starts, 0.1, 5000)
        xb, fb = O.nelder_mead_multistart(rosen, starts, 0.1, 5000)
        assert xa.tobytes() == xb.tobytes() and fa == fb
    wells = lambda x: -2 * np.exp(-0.5 * (x[0] + 3) ** 2) - 3 * np.exp(-0.5 * (x[0] - 3) ** 2)
    xa, fa = G.nelder_mead_multistart(wells, [[-3.0], [3.0], [0.0]], 0.1, 500)
    xb, fb = O.nelder_mead_multistart(wells, [[-3.0], [3.0], [0.0]], 0.1, 500)
    assert xa.tobytes() == xb.tobytes() and fa == fb
    # iteration cap honoured identically
    xa, fa = G.nelder_mead_multistart(rosen, [[-1.2, 1.0]], 0.1, 7)
    xb, fb = O.nelder_mead_multistart(rosen, [[-1.2, 1.0]], 0.1, 7)
    assert xa.tobytes() == xb.tobytes() and fa == fb


def test_model_json_roundtrip_and_validation():
    m = VariogramModel(0.05, [Structure.with_rotation("spherical", 0.6, 300.0, 30.0, 10.0, 0.0,
                                                      0.5, 40 / 300),
                              Structure("exponential", 0.35, 800.0)])
    m2 = VariogramModel.from_json(m.to_json())
    assert m2 == m
    ref_json = ('{"nugget":0.1,"structures":[{"kind":"spherical","sill":0.9,"range":100.0,'
                '"anis":{"azimuth_deg":45.0,"ratio":0.5}}]}')
    m3 = VariogramModel.from_json(ref_json)
    assert m3.structures[0].anis == Anisotropy(45.0, 0.5)
    with pytest.raises(G.InvalidParameter):
        VariogramModel(-0.1, [])
    with pytest.raises(G.InvalidParameter):
        VariogramModel(0.0, [Structure("spherical", 1.0, 0.0)])
    with pytest.raises(G.InvalidParameter):
        VariogramModel(0.0, [])
    with pytest.raises(G.InvalidParameter):
        VariogramModel(0.0, [Structure.with_anisotropy("spherical", 1.0, 1.0, 0.0, 0.0)])


def test_invalid_inputs_rejected_before_any_device_work():
    # PointSet::new validation happens on the host, like the reference's
    with pytest.raises(G.InsufficientData):
        G.PointSet(np.zeros((0, 2)), np.zeros(0))
    with pytest.raises(G.InvalidParameter):
        G.PointSet(np.array([[np.nan, 0.0]]), np.array([1.0]))
    with pytest.raises(G.InvalidParameter):
        G.PointSet(np.array([[0.0, 0.0]]), np.array([np.inf]))
    with pytest.raises(G.DimensionMismatch):
        G.PointSet(np.zeros((2, 2)), np.zeros(3))


def test_se_from_hessian_matches_the_oracle_lu():
    """vecchia.rs:1918-1935: sqrt of the inverse's diagonal through
    lu_factor / Lu::solve; NaN when singular or non-positive."""
    from geostat_rs.api import _se_from_hessian
    rng = np.random.default_rng(12)
    for _ in range(20):
        a = rng.normal(size=(3, 3))
        h = a @ a.T + 0.1 * np.eye(3)
        got = _se_from_hessian(h.tolist())
        inv = np.stack([O.lu_solve(h, np.eye(3)[i]) for i in range(3)], 1)
        want = [np.sqrt(inv[i, i]) if inv[i, i] > 0 else np.nan for i in range(3)]
        np.testing.assert_allclose(got, want, rtol=1e-12)
    assert all(np.isnan(_se_from_hessian([[1.0, 2.0], [2.0, 4.0]])))
    se = _se_from_hessian([[-1.0, 0.0], [0.0, 2.0]])
    assert np.isnan(se[0]) and abs(se[1] - np.sqrt(0.5)) < 1e-15
