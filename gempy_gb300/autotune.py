"""Autotuner for the evaluation kernels' tile shapes.

Every kernel family in ``gk_tunable`` (float-float field on grids and on
point lists, FP32 field, batched field) has ``gk_tune_variants()`` tile shapes (grid points per thread x bytes
per shared-memory record stage).  ``tune()`` times every variant with CUDA
events on a representative workload on the current GPU, keeps the fastest,
and writes ``gempy_gb300/tuning/<gpu>.json``; ``apply_saved()`` loads that
table for the current GPU and installs it with ``gk_tune_set`` (called on first
use of the kernels).
"""
import ctypes
import json
import os
import re
import time

import numpy as np
import torch

from . import _lib

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuning")
_applied = False


def _gpu_key():
    name = torch.cuda.get_device_name(torch.cuda.current_device())
    return re.sub(r"[^A-Za-z0-9]+", "_", name).strip("_")


def table_path():
    return os.path.join(HERE, f"{_gpu_key()}.json")


def variants():
    lib = _lib.load()
    out = []
    for v in range(lib.gk_tune_variants()):
        ppt, kb = ctypes.c_int32(), ctypes.c_int32()
        _lib.check("gk_tune_describe", lib.gk_tune_describe(v, ctypes.byref(ppt), ctypes.byref(kb)))
        out.append({"variant": v, "points_per_thread": ppt.value, "stage_kb": kb.value})
    return out


def apply_saved():
    """Install the saved table of this GPU, if any.  Returns the table or None."""
    global _applied
    _applied = True
    p = table_path()
    if not os.path.exists(p):
        return None
    with open(p) as f:
        table = json.load(f)
    lib = _lib.load()
    for name, choice in table.get("choices", {}).items():
        if name in _lib.TUNABLES:
            lib.gk_tune_set(_lib.TUNABLES[name], int(choice["variant"]))
    return table


def ensure_applied():
    if not _applied and torch.cuda.is_available():
        apply_saved()


def _time(fn, reps=3):
    s = torch.cuda.current_stream()
    fn()
    torch.cuda.synchronize()
    ts = []
    for _ in range(reps):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(s)
        fn()
        b.record(s)
        torch.cuda.synchronize()
        ts.append(a.elapsed_time(b))
    return float(np.median(ts))


def _eval_workload(prec, grid=96):
    from . import kernels as K
    from . import synthetic
    m = synthetic.precision(resolution=(grid,) * 3)
    ii, dd, ko = m.interpolation_input, m.data_descriptor, m.options.kernel_options
    ds = K.DeviceSeries(ii.orientations.dip_positions, ii.orientations.dip_gradients,
                        ii.orientations.nugget_effect_grad, ii.surface_points.sp_coords,
                        ii.surface_points.nugget_effect_scalar, dd.tensors_structure.number_of_points_per_surface,
                        range=ko.range, c_o=ko.c_o, uni_degree=ko.uni_degree)
    w, _ = K.solve_mixed(ds, tol=1e-11)
    model = K.prepare(ds, w)
    pts = K.Points.regular(ii.grid.dense_grid)
    out = {"field": torch.empty(pts.n, dtype=torch.float64, device="cuda")}
    return lambda: K.evaluate(ds, model, pts, prec, out=out)


def _list_workload(n_points=300000, seed=0):
    """The float-float field of the octree workload's first series at a
    random point list (octree levels and custom grids are point lists)."""
    from . import kernels as K
    from . import synthetic
    m = synthetic.folded_series(octree_levels=7)
    ii, dd, ko = m.interpolation_input, m.data_descriptor, m.options.kernel_options
    ss = dd.stack_structure
    n_p, n_o = int(ss.number_of_points_per_stack[0]), int(ss.number_of_orientations_per_stack[0])
    n_s = int(ss.number_of_surfaces_per_stack[0])
    ds = K.DeviceSeries(ii.orientations.dip_positions[:n_o], ii.orientations.dip_gradients[:n_o],
                        ii.orientations.nugget_effect_grad[:n_o], ii.surface_points.sp_coords[:n_p],
                        ii.surface_points.nugget_effect_scalar[:n_p],
                        dd.tensors_structure.number_of_points_per_surface[:n_s],
                        range=ko.range, c_o=ko.c_o, uni_degree=ko.uni_degree)
    w, _ = K.solve_mixed(ds, tol=1e-11)
    model = K.prepare(ds, w)
    og = ii.grid.octree_grid
    ext = np.asarray(og.orthogonal_extent, dtype=np.float64)
    rng = np.random.default_rng(seed)
    xyz = ext[0::2] + rng.random((n_points, 3)) * (ext[1::2] - ext[0::2])
    pts = K.Points(xyz=torch.as_tensor(xyz, device="cuda"))
    out = {"field": torch.empty(n_points, dtype=torch.float64, device="cuda")}
    return lambda: K.evaluate(ds, model, pts, K.GK_FF, out=out)


def _batch_workload(n=48, grid=32):
    from . import synthetic
    from .batch import BatchRunner
    br = BatchRunner([synthetic.realisation(i, resolution=(grid,) * 3) for i in range(n)])
    return br.run


def tune(families=("eval_ff", "eval_f32", "batch_eval", "eval_ff_list"), persist=True, reps=3):
    """Time every variant of each family; install and (optionally) save the fastest."""
    from . import kernels as K
    lib = _lib.load()
    vs = variants()
    table = {"gpu": torch.cuda.get_device_name(torch.cuda.current_device()),
             "when": time.strftime("%Y-%m-%dT%H:%M:%SZ", time.gmtime()), "choices": {}}
    for fam in families:
        tid = _lib.TUNABLES[fam]
        if fam == "eval_ff":
            fn = _eval_workload(K.GK_FF)
        elif fam == "eval_f32":
            fn = _eval_workload(K.GK_F32)
        elif fam == "eval_ff_list":
            fn = _list_workload()
        else:
            fn = _batch_workload()
        times = {}
        for v in vs:
            lib.gk_tune_set(tid, v["variant"])
            times[v["variant"]] = _time(fn, reps)
        best = min(times, key=times.get)
        lib.gk_tune_set(tid, best)
        table["choices"][fam] = dict(vs[best], ms=times[best],
                                     all_ms={str(k): round(t, 4) for k, t in times.items()})
    if persist:
        os.makedirs(HERE, exist_ok=True)
        with open(table_path(), "w") as f:
            json.dump(table, f, indent=1)
    return table


if __name__ == "__main__":
    print(json.dumps(tune(), indent=1))
