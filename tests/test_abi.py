"""CPU checks of the C ABI: the header declares exactly the exported entry
points and the built library loads (no compute calls without a GPU)."""
import ctypes
import os
import re
import subprocess

import pytest

from gempy_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "gempy_gb300.h")


def header_functions():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(gk_[a-z0-9_]+)\s*\(", txt)))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(_lib.LIB_PATH):
        from gempy_gb300 import build
        build.build()
    return _lib.load()


def test_header_matches_binding_table():
    declared = header_functions()
    bound = sorted(name for name, _, _ in _lib.SIGNATURES)
    assert declared == bound


def test_library_exports_every_declared_symbol(lib):
    for name in header_functions():
        assert hasattr(lib, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (gk_[a-z0-9_]+)", out))
    assert set(header_functions()) <= exported
    # and nothing is exported under the library's prefix that the header does not declare
    assert exported <= set(header_functions())


def test_version_and_size_queries_without_gpu(lib):
    assert b"sm_103a" in lib.gk_version()
    s = _lib.GkSystem()
    s.n_ori, s.n_sp, s.n_iface, s.uni_degree = 2, 20, 18, 1
    assert lib.gk_system_size(ctypes.byref(s)) == 6 + 18 + 3
    s.uni_degree = 2
    assert lib.gk_system_size(ctypes.byref(s)) == 6 + 18 + 9
    assert lib.gk_eval_model_bytes(ctypes.byref(s)) > 0
    assert lib.gk_octree_workspace_bytes(1000) >= 8
    s.n_fault = 2          # two offsetting faults: one drift unknown each
    assert lib.gk_system_size(ctypes.byref(s)) == 6 + 18 + 9 + 2


def test_struct_layouts_match_header():
    assert ctypes.sizeof(_lib.GkInfo) == 24
    assert ctypes.sizeof(_lib.GkSystem) == 6 * 4 + 4 * 8 + 8 * 8
    assert ctypes.sizeof(_lib.GkPoints) == 16 + 8 + 48 + 8 + 8 + 8
    assert ctypes.sizeof(_lib.GkSegment) == 8 + 8 + 8 * 32 + 8 * 33
    assert ctypes.sizeof(_lib.GkMlp) == 4 + 4 + 8
    assert ctypes.sizeof(_lib.GkAdam) == 5 * 4


def test_struct_layouts_match_compiled_header(tmp_path):
    """sizeof / offsetof of every ABI struct as a C compiler sees the header."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    src = tmp_path / "layout.c"
    src.write_text("""
#include <stdio.h>
#include <stddef.h>
#include "gempy_gb300.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\\n", sizeof(gk_info), sizeof(gk_system), sizeof(gk_points),
         sizeof(gk_segment), sizeof(gk_mlp), sizeof(gk_adam), offsetof(gk_mlp, params), offsetof(gk_system, range),
         offsetof(gk_system, fault_sp), offsetof(gk_points, fault_values), offsetof(gk_points, fault_ld));
  printf("%zu %zu %zu %zu\\n", sizeof(gk_series_eval), offsetof(gk_series_eval, min_iso), sizeof(gk_cta_job),
         offsetof(gk_cta_job, info));
  printf("%zu %zu %zu\\n", sizeof(gk_octree_level_layout), offsetof(gk_octree_level_layout, points),
         offsetof(gk_octree_level_layout, total));
  return 0;
}
""")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", inc, str(src), "-o", str(exe)], check=True)
    got = [int(v) for v in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()]
    want = [ctypes.sizeof(_lib.GkInfo), ctypes.sizeof(_lib.GkSystem), ctypes.sizeof(_lib.GkPoints),
            ctypes.sizeof(_lib.GkSegment), ctypes.sizeof(_lib.GkMlp), ctypes.sizeof(_lib.GkAdam),
            _lib.GkMlp.params.offset, _lib.GkSystem.range.offset, _lib.GkSystem.fault_sp.offset,
            _lib.GkPoints.fault_values.offset, _lib.GkPoints.fault_ld.offset,
            ctypes.sizeof(_lib.GkSeriesEval), _lib.GkSeriesEval.min_iso.offset, ctypes.sizeof(_lib.GkCtaJob),
            _lib.GkCtaJob.info.offset, ctypes.sizeof(_lib.GkOctreeLevelLayout),
            _lib.GkOctreeLevelLayout.points.offset, _lib.GkOctreeLevelLayout.total.offset]
    assert got == want


def test_octree_level_plan_on_the_host(lib):
    """gk_octree_level_plan is host arithmetic: every piece 256-aligned, in
    order, sized for its rows; the children and count only when refining."""
    L = _lib.GkOctreeLevelLayout()
    ns, n = 3, 1000
    assert lib.gk_octree_level_plan(ns, n, 1, 1, ctypes.byref(L)) == _lib.GK_OK
    np_ = 9 * n
    assert (L.n, L.n_points, L.n_series, L.corners, L.refine) == (n, np_, ns, 1, 1)
    order = ["points", "fields", "values", "ids", "block", "lith_ids", "masks", "children", "count", "work", "total"]
    offs = [getattr(L, k) for k in order]
    assert offs == sorted(offs) and all(o % 256 == 0 for o in offs) and L.points == 0
    need = {"points": 24 * np_, "fields": 8 * ns * np_, "values": 8 * ns * np_, "ids": 4 * ns * np_,
            "block": 8 * np_, "lith_ids": 4 * np_, "masks": ns * np_, "children": 8 * n * 24, "count": 8,
            "work": lib.gk_octree_workspace_bytes(n)}
    for a, b in zip(order[:-1], order[1:]):
        assert getattr(L, b) - getattr(L, a) >= need[a], a
    # the last level: no children; without corners the points are the centres
    assert lib.gk_octree_level_plan(ns, n, 0, 0, ctypes.byref(L)) == _lib.GK_OK
    assert L.n_points == n and L.children == L.count == L.work == L.total
    # marking needs the corners; bad sizes and modes are rejected
    assert lib.gk_octree_level_plan(ns, n, 0, 1, ctypes.byref(L)) == _lib.GK_ERR_ARG
    assert lib.gk_octree_level_plan(0, n, 1, 1, ctypes.byref(L)) == _lib.GK_ERR_ARG
    assert lib.gk_octree_level_plan(ns, -1, 1, 1, ctypes.byref(L)) == _lib.GK_ERR_ARG
    assert lib.gk_octree_level_plan(ns, n, 1, 4, ctypes.byref(L)) == _lib.GK_ERR_ARG
    assert lib.gk_octree_level_plan(ns, n, 0, 3, ctypes.byref(L)) == _lib.GK_ERR_ARG
    # the error test (refine 3) keeps n_series x n errors and the thresholds after the scan workspace
    assert lib.gk_octree_level_plan(ns, n, 1, 3, ctypes.byref(L)) == _lib.GK_OK
    assert L.total - L.work >= lib.gk_octree_workspace_bytes(n) + 8 * ns * n + 8 * ns
    items = (_lib.GkSeriesEval * ns)()
    sp3 = (ctypes.c_double * 3)(1.0, 1.0, 1.0)
    buf = ctypes.c_void_p(256)
    for t in (0.0, -1.0, float("nan"), float("inf")):   # the error test needs a finite threshold > 0
        assert lib.gk_octree_level(ns, items, buf, sp3, 0, 0, None, t, ctypes.byref(L), buf, L.total, None,
                                   None) == _lib.GK_ERR_ARG
    # a layout that the plan did not make, or a short buffer, is refused before any launch
    assert lib.gk_octree_level_plan(ns, n, 1, 1, ctypes.byref(L)) == _lib.GK_OK
    assert lib.gk_octree_level(ns, items, buf, sp3, 0, 0, None, 0.0, ctypes.byref(L), buf, L.total - 1, None,
                               None) == _lib.GK_ERR_SIZE
    L.masks += 256
    assert lib.gk_octree_level(ns, items, buf, sp3, 0, 0, None, 0.0, ctypes.byref(L), buf, L.total, None,
                               None) == _lib.GK_ERR_ARG


def test_invalid_arguments_rejected_before_any_launch(lib):
    # argument checks run on the host and return GK_ERR_ARG without touching the GPU
    assert lib.gk_build(None, 0, None, 0, None, None) == _lib.GK_ERR_ARG
    s = _lib.GkSystem()
    s.n_ori, s.n_sp, s.n_iface, s.uni_degree, s.range = 1, 2, 1, 5, 1.0
    assert lib.gk_build(ctypes.byref(s), 0, None, 0, None, None) == _lib.GK_ERR_ARG
    assert lib.gk_lu_factor(0, -1, None, 0, None, None, 0, None, None) == _lib.GK_ERR_ARG
    assert lib.gk_solve_mixed(0, None, 0, None, None, 1e-10, 10, None, 0, None, None) == _lib.GK_ERR_ARG
    # two-level: landmark count / block size rules, x0 aliasing x, precision enum
    buf = ctypes.c_void_p(64)  # never dereferenced: the checks come first
    for r, bs, prec, x0 in [(100, 64, 0, None), (64, 100, 0, None), (64, 8192, 0, None), (64, 64, 7, None),
                            (64, 64, 0, buf)]:
        assert lib.gk_solve_twolevel(1000, buf, 1000, buf, buf, x0, buf, r, bs, prec, 1e-8, 10, None, 0, None,
                                     None) == _lib.GK_ERR_ARG
    assert lib.gk_solve_twolevel_workspace_bytes(1000, 7) == 0
    assert lib.gk_solve_twolevel_workspace_bytes(1000, _lib.GK_FF) > lib.gk_solve_twolevel_workspace_bytes(
        1000, _lib.GK_F64)
    # network entry points
    net = _lib.GkMlp()
    net.in_dim, net.out_dim, net.params = 21, 3, None
    assert lib.gk_mlp_fwd_tc(ctypes.byref(net), 1, buf, buf, None, None) == _lib.GK_ERR_ARG
    net.params = 64
    assert lib.gk_mlp_fwd_tc(ctypes.byref(net), 0, buf, buf, None, None) == _lib.GK_ERR_SIZE
    assert lib.gk_mlp_adam(10, None, None, None, None, None, None, 1, None) == _lib.GK_ERR_ARG
    assert lib.gk_gemv(10, None, 10, None, None, None) == _lib.GK_ERR_ARG
    # fault drift: too many faults, or fault values missing
    s = _lib.GkSystem()
    s.n_ori, s.n_sp, s.n_iface, s.uni_degree, s.range = 1, 2, 1, 1, 1.0
    s.dip_positions = s.dip_gradients = s.nugget_grad = s.sp_coords = s.nugget_sp = 64
    s.ref_index = s.rest_index = 64
    s.n_fault = _lib.GK_MAX_FAULTS + 1
    assert lib.gk_build(ctypes.byref(s), 0, buf, 64, buf, None) == _lib.GK_ERR_SIZE
    s.n_fault = 1
    assert lib.gk_build(ctypes.byref(s), 0, buf, 64, buf, None) == _lib.GK_ERR_ARG   # fault_sp NULL
    # combination: ids are required; an ONLAP last series has nothing to onlap
    rel = (ctypes.c_int32 * 2)(3, 2)
    iso = (ctypes.c_double * 2)(0.0, 0.0)
    assert lib.gk_combine_series(2, 10, buf, buf, None, rel, iso, iso, None, None, None, None) == _lib.GK_ERR_ARG
    assert lib.gk_combine_series(2, 10, buf, buf, buf, rel, iso, iso, None, None, None, None) == _lib.GK_ERR_ARG
    # octree marking needs at least one id set
    sp3 = (ctypes.c_double * 3)(1.0, 1.0, 1.0)
    cnt = ctypes.c_int64(0)
    assert lib.gk_octree_refine(8, buf, buf, 0, 0, sp3, buf, ctypes.byref(cnt), buf, 1024, None) == _lib.GK_ERR_ARG


def test_tuning_tables_are_well_formed():
    import glob
    import json
    for p in glob.glob(os.path.join(ROOT, "gempy_gb300", "tuning", "*.json")):
        t = json.load(open(p))
        assert "gpu" in t and "choices" in t
        for name, ch in t["choices"].items():
            assert name in _lib.TUNABLES
            assert 0 <= int(ch["variant"]) < 4
            assert ch["points_per_thread"] in (2, 4) and ch["stage_kb"] in (16, 32)
