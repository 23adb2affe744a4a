"""``compute_model``: drop-in for the engine call at ``gempy/API/compute_API.py:68-73``.

Signature and inputs are the ones the reference passes
(``compute_model(interpolation_input, options, data_descriptor,
geophysics_input)``, also called directly at
``test/test_api/test_model_construction_granular.py:130-134``); the returned
``Solutions`` carries the fields gempy reads back (``geo_model.py:100-127``,
``_engine_factory.py:45-48``, ``compute_API.py:114``).

Flow per call, all arithmetic on the GPU through ``libgempy_gb300.so``:
  1. split the inputs into series (``data_descriptor.stack_structure``);
  2. per series, in stack order: the blocks of the FAULT series that offset it
     (``stack_structure.faults_relations``) at its surface points become its
     fault-drift functions; build K, solve for the weights -- FP64 LU
     ("float64", the plain form) or FP32 LU + FP64 refinement ("float32", the
     mixed form) -- and pack the weights for evaluation;
  3. isovalues: the field at each surface's reference point, in FP64;
  4. evaluate every series on each point set (octree levels, dense grid,
     custom grid) in stack order, each fault's block feeding the series it
     offsets, segment with the sigmoid, combine the series with masks; octree
     levels refine voxels whose corners differ in lithology or fault id.
There is no CPU path: without the CUDA library this raises.
"""
import os
import time
from dataclasses import dataclass
from typing import List, Optional

import numpy as np
import torch

from . import kernels as K
from ._lib import GK_F32, GK_F64, GK_FF
from .data import (CombinedOutput, ExportedFields, InterpOutput, OctreeLevel, RawArraysSolution, RootOutput,
                   Solutions, StackRelationType)


@dataclass
class EngineConfig:
    """Mirror of the reference's ``GemPyEngineConfig`` (``gempy_engine_config.py:9-14``):
    ``dtype`` "float64" selects the plain FP64 form; "float32" the mixed form:
    FP32 LU preconditioning an FP64 FGMRES solve, and the field evaluated in
    float-float on the FP32 pipe (cubic kernel; other kernels evaluate in
    FP64) with FP64 isovalues.  ``eval_precision`` overrides the evaluation
    arithmetic ("f64", "ff" or "f32"; "f32" is only accurate to ~1e-7 times
    the cancellation factor sum|w_j k_j| / |Z| of the kriging sum).

    In the mixed form, series with at least ``learned_min_n`` unknowns are
    solved by FGMRES to ``learned_tol`` with the two-level preconditioner the
    trained network picks (``learned.py``; FP64 LU fallback) when a trained
    model is available (``learned_model``, default: the packaged one);
    ``learned_min_n`` = 0 disables this."""
    dtype: str = "float64"
    use_gpu: bool = True
    keep_on_device: bool = False
    solver_tol: float = 1e-12
    solver_max_iter: int = 60
    eval_precision: Optional[str] = None
    timings: bool = False
    learned_min_n: int = 16384
    learned_tol: float = 1e-8
    learned_model: Optional[str] = None


class _Series:
    def __init__(self, dev_series, iso, order, unit_values, relation, weights, solve_info, faults):
        self.dev = dev_series
        self.iso = iso                  # per surface, stack order (FP64)
        self.order = order              # surfaces sorted by isovalue, highest first
        self.unit_values = unit_values  # n_surf + 1 values
        self.relation = relation
        self.weights = weights
        self.solve_info = solve_info
        self.faults = faults            # indices of the FAULT series that offset this one
        self.model = None
        self.seg = K.make_segment(iso[order], unit_values, 0.0)

    def set_slope(self, slope):
        self.seg.slope = float(slope)


def _load_cost_model(path, device):
    from . import learned
    path = path or learned.DEFAULT_MODEL
    if not os.path.exists(path):
        return None
    return learned.CostModel.load(path, device=device)


def _warm_start(interpolation_input, i, n, device):
    """The series' previous weights (``InterpolationInput.weights``, as gempy
    passes them back, ``_engine_factory.py:45-48``) when their size fits."""
    ws = getattr(interpolation_input, "weights", None) or []
    if i < len(ws) and ws[i] is not None and np.size(ws[i]) == n:
        return torch.as_tensor(np.asarray(ws[i], dtype=np.float64).ravel()).to(device)
    return None


def _solve_learned(dev_s, cost_model, tol, x0=None):
    """Network-chosen two-level FGMRES (FP64 LU fallback); (w, gk_info tensor)."""
    from . import learned
    r = learned.solve_learned(dev_s, cost_model, tol=tol, x0=x0)
    rec = np.zeros(1, dtype=K.INFO_DTYPE)
    rec["status"] = 0 if r.fallback or r.status == 0 else r.status
    rec["iterations"] = r.iterations
    rec["where"] = int(r.fallback)  # 1: FGMRES missed the tolerance and the FP64 LU produced w
    rec["residual"] = r.residual
    info = torch.as_tensor(np.frombuffer(rec.tobytes(), dtype=np.uint8).copy()).to(dev_s.device)
    return r.x, info


def _split(interpolation_input, options, data_descriptor, device):
    ss = data_descriptor.stack_structure
    pps = np.asarray(data_descriptor.tensors_structure.number_of_points_per_surface, dtype=np.int64)
    sp = interpolation_input.surface_points
    ori = interpolation_input.orientations
    ko = options.kernel_options
    p_off = o_off = s_off = 0
    out = []
    for i in range(ss.n_stacks):
        n_p = int(ss.number_of_points_per_stack[i])
        n_o = int(ss.number_of_orientations_per_stack[i])
        n_s = int(ss.number_of_surfaces_per_stack[i])
        dev = K.DeviceSeries(
            ori.dip_positions[o_off:o_off + n_o], ori.dip_gradients[o_off:o_off + n_o],
            ori.nugget_effect_grad[o_off:o_off + n_o],
            sp.sp_coords[p_off:p_off + n_p], sp.nugget_effect_scalar[p_off:p_off + n_p],
            pps[s_off:s_off + n_s], range=ko.range, c_o=ko.c_o, uni_degree=ko.uni_degree,
            kernel=ko.kernel_function, i_res=ko.i_res, gi_res=ko.gi_res, device=device)
        faults = ss.fault_sources(i) if hasattr(ss, "fault_sources") else []
        out.append((dev, s_off, n_s, ss.masking_descriptor[i], faults))
        p_off += n_p
        o_off += n_o
        s_off += n_s
    return out


@dataclass
class _Evaluation:
    fields: torch.Tensor          # (n_series, n)
    values: torch.Tensor          # (n_series, n) soft segmented values
    ids: torch.Tensor             # (n_series, n) block ids
    grads: list                   # per series (n, 3) or None
    block: torch.Tensor           # combined soft values
    lith_ids: torch.Tensor        # combined lithology ids
    masks: torch.Tensor           # (n_series, n) squeezed masks
    fault_rows: List[int]         # series that are FAULT stacks

    def refinement_ids(self):
        """Id sets whose change across a voxel's corners refines it: the
        lithology, then each fault series' block."""
        return torch.stack([self.lith_ids] + [self.ids[i] for i in self.fault_rows])

    def slice(self, a, b):
        return _Evaluation(self.fields[:, a:b], self.values[:, a:b], self.ids[:, a:b],
                           [None if g is None else g[a:b] for g in self.grads], self.block[a:b],
                           self.lith_ids[a:b], self.masks[:, a:b], self.fault_rows)


class _Evaluator:
    def __init__(self, series, prec, slope):
        self.series = series
        self.prec = prec
        self.slope = slope
        for s in series:
            s.set_slope(slope)

    def series_values(self, pts: K.Points, upto, prec=GK_F64):
        """Soft values of series 0..upto-1 at pts (their fault chains included)."""
        vals = []
        for s in self.series[:upto]:
            fv = torch.stack([vals[j] for j in s.faults]) if s.faults else None
            _, _, v, _ = K.evaluate(s.dev, s.model, pts, prec, seg=s.seg, want_field=False, fault_values=fv)
            vals.append(v)
        return vals

    def run(self, pts: K.Points, gradient=False) -> _Evaluation:
        fields, values, ids, grads = [], [], [], []
        for s in self.series:
            fv = torch.stack([values[j] for j in s.faults]) if s.faults else None
            f, _, v, i = K.evaluate(s.dev, s.model, pts, self.prec, seg=s.seg, want_ids=True, fault_values=fv)
            g = None
            if gradient:   # gradients in FP64 (the float-float kernel computes the field only)
                _, g, _, _ = K.evaluate(s.dev, s.model, pts, GK_F64 if self.prec == GK_FF else self.prec,
                                        gradient=True, want_field=False, fault_values=fv)
            fields.append(f)
            values.append(v)
            ids.append(i)
            grads.append(g)
        F, V, I = torch.stack(fields), torch.stack(values), torch.stack(ids)
        rel = [int(s.relation) for s in self.series]
        mn = [float(np.min(s.iso)) if len(s.iso) else 0.0 for s in self.series]
        mx = [float(np.max(s.iso)) if len(s.iso) else 0.0 for s in self.series]
        cv, ci, masks = K.combine(F, V, I, rel, mn, mx)
        frows = [k for k, s in enumerate(self.series) if int(s.relation) == int(StackRelationType.FAULT)]
        return _Evaluation(F, V, I, grads, cv, ci, masks, frows)


def _np(t, keep):
    if t is None:
        return None
    return t if keep else t.cpu().numpy()


def _outputs(ev: _Evaluation, series, keep):
    outs = []
    for i, s in enumerate(series):
        g = ev.grads[i]
        ef = ExportedFields(scalar_field=_np(ev.fields[i], keep),
                            gx_field=_np(g[:, 0], keep) if g is not None else None,
                            gy_field=_np(g[:, 1], keep) if g is not None else None,
                            gz_field=_np(g[:, 2], keep) if g is not None else None,
                            scalar_field_at_surface_points=s.iso)
        outs.append(InterpOutput(ef, _np(ev.values[i], keep), weights=_np(s.weights, keep),
                                 mask=_np(ev.masks[i], keep)))
    return outs


def _combined(ev: _Evaluation, keep):
    return CombinedOutput(ExportedFields(scalar_field=_np(ev.fields[-1], keep)), _np(ev.block, keep),
                          _np(ev.lith_ids, keep), _np(ev.masks, keep))


def _solve_series(interpolation_input, options, data_descriptor, device, cfg, mixed):
    ko = options.kernel_options
    uv = np.asarray(interpolation_input.unit_values, dtype=np.float64)
    series = []
    cost_model = None
    conds = []
    ev = _Evaluator(series, GK_F64, options.sigmoid_slope)
    for si, (dev_s, s_off, n_s, rel, faults) in enumerate(_split(interpolation_input, options, data_descriptor,
                                                                  device)):
        if faults:
            # the fault blocks at this series' surface points are its fault-drift functions
            vals = ev.series_values(K.Points(xyz=dev_s.sp_coords), si)
            dev_s.set_fault_blocks(torch.stack([vals[j] for j in faults]))
        if getattr(ko, "compute_condition_number", False):
            Kc, _ = K.build(dev_s, GK_F64)
            conds.append(K.condition_number(Kc))
            del Kc
        if mixed and cfg.learned_min_n > 0 and dev_s.N >= cfg.learned_min_n:
            if cost_model is None:
                cost_model = _load_cost_model(cfg.learned_model, device)
        if mixed and cost_model is not None and dev_s.N >= cfg.learned_min_n:
            w, info = _solve_learned(dev_s, cost_model, cfg.learned_tol,
                                     _warm_start(interpolation_input, si, dev_s.N, device))
        elif mixed:
            w, info = K.solve_mixed(dev_s, tol=cfg.solver_tol, max_iter=cfg.solver_max_iter)
        else:
            w, info = K.solve_plain(dev_s)
        model = K.prepare(dev_s, w)
        # ---- 3: isovalues at the reference points, FP64
        if n_s:
            starts = torch.as_tensor(np.concatenate([[0], np.cumsum(dev_s.points_per_surface)[:-1]])).to(device)
            fv = dev_s.fault_sp[:, starts] if dev_s.n_faults else None
            iso_t, _, _, _ = K.evaluate(dev_s, model, K.Points(xyz=dev_s.ref_points), GK_F64, fault_values=fv)
            iso = iso_t.cpu().numpy()
        else:
            iso = np.zeros(0)
        order = np.argsort(-iso, kind="stable")
        s = _Series(dev_s, iso, order, uv[s_off:s_off + n_s + 1], rel, w, info, faults)
        s.model = model
        s.set_slope(options.sigmoid_slope)
        series.append(s)
    if conds:
        # the engine reports one number on the options; with several series, the largest
        ko.condition_number = float(max(conds))
    return series


def compute_model(interpolation_input, options, data_descriptor, geophysics_input=None,
                  config: Optional[EngineConfig] = None) -> Solutions:
    cfg = config or EngineConfig()
    if not torch.cuda.is_available():
        raise RuntimeError("gempy_gb300.compute_model needs a CUDA device (there is no CPU fallback)")
    device = torch.device("cuda")
    mixed = str(cfg.dtype) in ("float32", "mixed")
    ko = options.kernel_options
    cubic = K.kernel_id(ko.kernel_function) == 0
    if cfg.eval_precision is not None:
        prec = {"f64": GK_F64, "ff": GK_FF, "f32": GK_F32}[cfg.eval_precision]
    else:
        prec = GK_FF if (mixed and cubic) else GK_F64
    t0 = time.perf_counter()
    timings = {}

    # ---- 1-3: per-series solve and isovalues
    series = _solve_series(interpolation_input, options, data_descriptor, device, cfg, mixed)
    if cfg.timings:
        torch.cuda.synchronize()
        timings["solve_s"] = time.perf_counter() - t0

    ev = _Evaluator(series, prec, options.sigmoid_slope)
    keep = cfg.keep_on_device
    grid = interpolation_input.grid
    eo = options.evaluation_options
    want_grad = bool(eo.compute_scalar_gradient)

    # ---- 4a: octree levels.  Centres and (where needed) corners are one
    # point set: [centres; 8 corners per centre], evaluated once per series.
    t1 = time.perf_counter()
    octrees = []
    n_levels = int(eo.number_octree_levels)
    min_level = int(eo.octree_min_level)
    levels_surface = int(getattr(eo, "number_octree_levels_surface", getattr(eo, "_number_octree_levels_surface", 0)))
    if grid.octree_grid is not None and n_levels >= 1:
        og = grid.octree_grid
        centres = torch.as_tensor(og.values).to(device)
        d = np.array(og.dxdydz, dtype=np.float64)
        for level in range(n_levels):
            n = centres.shape[0]
            last = level == n_levels - 1
            surface = level < levels_surface
            refine_all = level + 1 < min_level
            need_corners = surface or (not last and not refine_all)
            if need_corners:
                pts_xyz = torch.empty((9 * n, 3), dtype=torch.float64, device=device)
                pts_xyz[:n] = centres
                pts_xyz[n:] = K.octree_corners(centres, d)
            else:
                pts_xyz = centres
            e = ev.run(K.Points(xyz=pts_xyz), gradient=want_grad)
            ec = e.slice(0, n)
            outs = _outputs(e if surface else ec, series, keep)
            corners_out = _combined(e.slice(n, 9 * n), keep) if surface else None
            octrees.append(OctreeLevel(_np(centres, keep), d.copy(), outs, _combined(ec, keep), corners_out,
                                       _np(pts_xyz[n:], keep) if surface else None))
            if last:
                break
            corner_ids = None if refine_all else e.slice(n, 9 * n).refinement_ids()
            centres = K.octree_refine(centres, corner_ids, d, refine_all=refine_all)
            d = d / 2.0
            if centres.shape[0] == 0:
                break
    if cfg.timings:
        torch.cuda.synchronize()
        timings["octree_s"] = time.perf_counter() - t1

    # ---- 4b: dense and custom grids
    raw = RawArraysSolution()
    t2 = time.perf_counter()
    if grid.dense_grid is not None:
        e = ev.run(K.Points.regular(grid.dense_grid), gradient=want_grad)
        raw.lith_block = _np(e.block, keep)
        raw.scalar_field_matrix = _np(e.fields, keep)
        raw.mask_matrix_squeezed = _np(e.masks, keep)
        raw.block_matrix = _np(e.values, keep)
    if grid.custom_grid is not None:
        pts = torch.as_tensor(grid.custom_grid.values).to(device)
        e = ev.run(K.Points(xyz=pts))
        raw.custom = _np(e.block, keep)
    if cfg.timings:
        torch.cuda.synchronize()
        timings["grids_s"] = time.perf_counter() - t2
        timings["total_s"] = time.perf_counter() - t0

    root = RootOutput([InterpOutput(ExportedFields(scalar_field=None, scalar_field_at_surface_points=s.iso),
                                    None, weights=_np(s.weights, keep)) for s in series])
    sfsp = [float(v) for s in series for v in s.iso]
    sol = Solutions(octrees_output=octrees, root_output=root, raw_arrays=raw,
                    scalar_field_at_surface_points=sfsp, _ordered_elements=[s.order for s in series],
                    block_solution_type=options.block_solutions_type, timings=timings,
                    solver_info=[K.read_info(s.solve_info) for s in series])
    return sol
