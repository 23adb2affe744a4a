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
import dataclasses
import os
import time
import warnings
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
    ``learned_min_n`` = 0 disables this.

    ``compute_grads`` (FP64 form only) returns the octree levels' scalar
    fields as torch tensors that back-propagate, through the adjoint kernels
    (``adjoint.py``), into ``Solutions.taped_interpolation_input``: the
    interpolation input with its surface points, nuggets and orientations as
    leaf tensors (transformed frame), as the reference's PyTorch tape does."""
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
    compute_grads: bool = False


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
    """Per-series DeviceSeries.  All series' inputs go to the device in two
    copies -- one FP64 buffer (points, nuggets, orientations, reference
    points), one int32 buffer (reference/rest indices) -- and each series
    holds views into them."""
    ss = data_descriptor.stack_structure
    pps = np.asarray(data_descriptor.tensors_structure.number_of_points_per_surface, dtype=np.int64)
    sp = interpolation_input.surface_points
    ori = interpolation_input.orientations
    ko = options.kernel_options
    spc = np.asarray(sp.sp_coords, dtype=np.float64).reshape(-1, 3)
    nsp = np.asarray(sp.nugget_effect_scalar, dtype=np.float64).ravel()
    dpos = np.asarray(ori.dip_positions, dtype=np.float64).reshape(-1, 3)
    dgr = np.asarray(ori.dip_gradients, dtype=np.float64).reshape(-1, 3)
    ngr = np.asarray(ori.nugget_effect_grad, dtype=np.float64).ravel()
    starts = np.concatenate([[0], np.cumsum(pps)[:-1]]).astype(np.int64) if len(pps) else np.zeros(0, np.int64)
    refp = spc[starts]
    parts = [spc.ravel(), nsp, dpos.ravel(), dgr.ravel(), ngr, refp.ravel()]
    offs = np.concatenate([[0], np.cumsum([len(a) for a in parts])])
    f64 = torch.as_tensor(np.concatenate(parts)).to(device)
    g_sp, g_nsp, g_dpos, g_dgr, g_ngr, g_ref = (f64[offs[i]:offs[i + 1]] for i in range(6))
    g_sp, g_dpos, g_dgr, g_ref = g_sp.view(-1, 3), g_dpos.view(-1, 3), g_dgr.view(-1, 3), g_ref.view(-1, 3)
    idx_parts, s_off = [], 0
    for i in range(ss.n_stacks):
        n_s = int(ss.number_of_surfaces_per_stack[i])
        ref, rest = K.ref_rest_indices(pps[s_off:s_off + n_s])
        idx_parts += [ref, rest]
        s_off += n_s
    ilen = np.concatenate([[0], np.cumsum([len(a) for a in idx_parts])])
    i32 = torch.as_tensor(np.concatenate(idx_parts).astype(np.int32) if idx_parts else np.zeros(0, np.int32)).to(device)
    p_off = o_off = s_off = 0
    out = []
    for i in range(ss.n_stacks):
        n_p = int(ss.number_of_points_per_stack[i])
        n_o = int(ss.number_of_orientations_per_stack[i])
        n_s = int(ss.number_of_surfaces_per_stack[i])
        dev = K.DeviceSeries(
            g_dpos[o_off:o_off + n_o], g_dgr[o_off:o_off + n_o], g_ngr[o_off:o_off + n_o],
            g_sp[p_off:p_off + n_p], g_nsp[p_off:p_off + n_p], pps[s_off:s_off + n_s],
            range=ko.range, c_o=ko.c_o, uni_degree=ko.uni_degree, kernel=ko.kernel_function, i_res=ko.i_res,
            gi_res=ko.gi_res, device=device,
            ref_index=i32[ilen[2 * i]:ilen[2 * i + 1]], rest_index=i32[ilen[2 * i + 1]:ilen[2 * i + 2]],
            ref_points=g_ref[s_off:s_off + n_s])
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

    def _set(self):
        if getattr(self, "_series_set", None) is None:
            self._series_set = K.SeriesSet([
                (s.dev, s.model, s.seg, int(s.relation), s.faults,
                 float(np.min(s.iso)) if len(s.iso) else 0.0, float(np.max(s.iso)) if len(s.iso) else 0.0)
                for s in self.series])
            self._frows = [k for k, s in enumerate(self.series) if int(s.relation) == int(StackRelationType.FAULT)]
        return self._series_set

    def run(self, pts: K.Points, gradient=False) -> _Evaluation:
        """Every series at ``pts`` and their combination: one library call
        (gk_eval_series_set); gradients, when asked for, in FP64 per series."""
        F, V, I, cv, ci, masks = self._set().evaluate(pts, self.prec)
        grads = self.gradients(pts, V) if gradient else [None] * len(self.series)
        return _Evaluation(F, V, I, grads, cv, ci, masks, self._frows)

    def gradients(self, pts: K.Points, V):
        """Per-series field gradients at pts (FP64: the float-float kernel
        computes the field only); V holds the series' soft values there."""
        grads = []
        for s in self.series:
            fv = V[s.faults] if s.faults else None
            _, g, _, _ = K.evaluate(s.dev, s.model, pts, GK_F64 if self.prec == GK_FF else self.prec,
                                    gradient=True, want_field=False, fault_values=fv)
            grads.append(g)
        return grads


def _outputs(ev: _Evaluation, series):
    outs = []
    for i, s in enumerate(series):
        g = ev.grads[i]
        ef = ExportedFields(scalar_field=ev.fields[i],
                            gx_field=g[:, 0] if g is not None else None,
                            gy_field=g[:, 1] if g is not None else None,
                            gz_field=g[:, 2] if g is not None else None,
                            scalar_field_at_surface_points=s.iso)
        outs.append(InterpOutput(ef, ev.values[i], weights=s.weights, mask=ev.masks[i]))
    return outs


def _combined(ev: _Evaluation):
    return CombinedOutput(ExportedFields(scalar_field=ev.fields[-1]), ev.block, ev.lith_ids, ev.masks)


_NP_DTYPE = {torch.float64: np.float64, torch.float32: np.float32, torch.int32: np.int32,
             torch.uint8: np.uint8, torch.int64: np.int64, torch.bool: np.bool_}


def _tensor_slots(obj):
    """(container, key, tensor) for every CUDA tensor reachable in obj."""
    slots = []

    def visit(o):
        if isinstance(o, list):
            for i, v in enumerate(o):
                if isinstance(v, torch.Tensor):
                    slots.append((o, i, v))
                else:
                    visit(v)
            return
        d = getattr(o, "__dict__", None)
        if d is None:
            return
        for k, v in list(d.items()):
            if isinstance(v, torch.Tensor):
                slots.append((o, k, v))
            elif isinstance(v, list) or hasattr(v, "__dict__"):
                visit(v)

    visit(obj)
    return slots


class _HostStager:
    """Moves result tensors to host numpy arrays with few, overlapped copies,
    made on a side stream (into page-locked memory from PyTorch's caching
    host allocator) while the compute stream goes on.

    * ``push(t)`` copies the bytes of a contiguous device tensor;
      ``host(t)`` is then its numpy copy.
    * ``stage(obj)`` copies every device tensor reachable from ``obj``: the
      tensors are views of a few allocations, each copied whole once, and each
      tensor becomes a numpy view of its copy (same offset, shape and strides).

    ``finish`` waits for the copies, then ``host`` answers and staged objects
    hold numpy arrays."""

    def __init__(self):
        self.stream = torch.cuda.Stream()
        self.jobs = []
        self.hosts = {}        # device storage address -> page-locked copy of the whole storage
        self.pushed = {}       # id(tensor) -> (tensor, page-locked copy of its bytes)
        self.pending = []

    def _copy(self, dev_bytes, nbytes):
        pinned = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
        self.pending.append((dev_bytes, pinned))
        return pinned

    def _launch(self):
        if not self.pending:
            return
        self.stream.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(self.stream):
            for dev, pinned in self.pending:
                pinned.copy_(dev, non_blocking=True)
        for dev, _ in self.pending:
            dev.record_stream(self.stream)
        self.pending = []

    def push(self, *tensors):
        for t in tensors:
            if t is None or id(t) in self.pushed:
                continue
            if not t.is_contiguous():
                raise ValueError("push() copies contiguous tensors")
            self.pushed[id(t)] = (t, self._copy(t.view(-1).view(torch.uint8), t.numel() * t.element_size()))
        self._launch()

    def host(self, t):
        if t is None:
            return None
        _, pinned = self.pushed[id(t)]
        return pinned.numpy().view(_NP_DTYPE[t.dtype]).reshape(tuple(t.shape))

    def stage(self, obj):
        slots = _tensor_slots(obj)
        if not slots:
            return
        meta = []
        for _, _, t in slots:
            st = t.untyped_storage()
            ptr = st.data_ptr()
            if ptr not in self.hosts:
                dev = torch.empty(0, dtype=torch.uint8, device=t.device).set_(st)
                self.hosts[ptr] = self._copy(dev, st.nbytes())
            meta.append((ptr, t.storage_offset() * t.element_size(), t.dtype, tuple(t.shape),
                         tuple(x * t.element_size() for x in t.stride())))
        self._launch()
        self.jobs.append((slots, meta))

    def finish(self):
        self.stream.synchronize()
        hosts = {ptr: pinned.numpy() for ptr, pinned in self.hosts.items()}
        for slots, meta in self.jobs:
            for (obj, k, _), (ptr, off, dt, shape, strides) in zip(slots, meta):
                arr = np.ndarray(shape, dtype=_NP_DTYPE[dt], buffer=hosts[ptr], offset=off, strides=strides)
                if isinstance(obj, list):
                    obj[k] = arr
                else:
                    setattr(obj, k, arr)
        self.jobs.clear()
        self.hosts.clear()


@dataclass
class _LevelRecord:
    """One octree level left on the device by gk_octree_level (its results:
    ``level.buffer[:level.result_bytes]``) and its per-series gradients."""
    level: K.OctreeLevel
    result: torch.Tensor
    spacing: np.ndarray
    surface: bool
    grads: list


def _level_output(rec: _LevelRecord, ev: "_Evaluator", series, buffer, grads):
    """The OctreeLevel of a record from its result bytes (the device buffer,
    or its host copy: the same layout either way)."""
    n = rec.level.n
    pts, F, V, I, B, L, M = rec.level.views(buffer)
    e = _Evaluation(F, V, I, grads, B, L, M, ev._frows)
    ec = e.slice(0, n)
    outs = _outputs(e if rec.surface else ec, series)
    corners_out = _combined(e.slice(n, 9 * n)) if rec.surface else None
    return OctreeLevel(pts[:n], rec.spacing.copy(), outs, _combined(ec), corners_out,
                       pts[n:] if rec.surface else None)


CTA_MAX_N = 4096   # mixed-form series up to this size are solved by one thread block


def _solve_one(dev_s, cfg, mixed, cost_model, interpolation_input, si, device):
    if mixed and cost_model is not None and dev_s.N >= cfg.learned_min_n:
        return _solve_learned(dev_s, cost_model, cfg.learned_tol,
                              _warm_start(interpolation_input, si, dev_s.N, device)) + (False,)
    if mixed and dev_s.N <= CTA_MAX_N:
        return K.solve_mixed_cta(dev_s, tol=cfg.solver_tol, max_iter=cfg.solver_max_iter) + (True,)
    if mixed:
        return K.solve_mixed(dev_s, tol=cfg.solver_tol, max_iter=cfg.solver_max_iter) + (False,)
    return K.solve_plain(dev_s) + (False,)


def _solve_series(interpolation_input, options, data_descriptor, device, cfg, mixed):
    """Per series: fault blocks, solve, packed model and FP64 isovalues.  The
    isovalues and solver statuses of all series are read back together with
    one synchronisation, except where a later series' fault drift needs a
    fault series' isovalues first."""
    ko = options.kernel_options
    uv = np.asarray(interpolation_input.unit_values, dtype=np.float64)
    series, pending = [], []
    cost_model = None
    conds = []
    ev = _Evaluator(series, GK_F64, options.sigmoid_slope)

    def finalize():
        if not pending:
            return
        # one copy: every pending series' status word (24 bytes) and isovalues
        packed = torch.cat([p["info"].view(torch.uint8) for p in pending] +
                           [p["iso"].contiguous().view(torch.uint8) for p in pending]).cpu().numpy()
        nb = 24 * len(pending)
        infos = list(np.frombuffer(packed[:nb].tobytes(), dtype=K.INFO_DTYPE))
        isos = packed[nb:].view(np.float64)
        o = 0
        for p, inf in zip(pending, infos):
            n_s = p["n_s"]
            iso = isos[o:o + n_s]
            o += n_s
            if p["cta"] and int(inf["status"]) != 0:
                # the one-block solve met a zero pivot or stalled: the full solver
                # (partial-pivoting fallback) takes over
                w, info = K.solve_mixed(p["dev"], tol=cfg.solver_tol, max_iter=cfg.solver_max_iter)
                p["w"], p["info"] = w, info
                p["model"] = K.prepare(p["dev"], w)
                iso = _isovalues(p["dev"], p["model"]).cpu().numpy()
                inf = K.read_info(info)
            order = np.argsort(-iso, kind="stable")
            sr = _Series(p["dev"], iso, order, p["uv"], p["rel"], p["w"], p["info"], p["faults"])
            sr.info_host = inf
            sr.model = p["model"]
            sr.set_slope(options.sigmoid_slope)
            series.append(sr)
        pending.clear()

    group = []   # small series of the mixed form, solved together in one launch

    def add_pending(dev_s, w, info, cta, s_off, n_s, rel, faults):
        model = K.prepare(dev_s, w)
        iso_t = _isovalues(dev_s, model) if n_s else torch.zeros(0, dtype=torch.float64, device=device)
        pending.append({"dev": dev_s, "w": w, "info": info, "model": model, "iso": iso_t, "n_s": n_s,
                        "uv": uv[s_off:s_off + n_s + 1], "rel": rel, "faults": faults, "cta": cta})

    def flush_group():
        if not group:
            return
        res = K.solve_mixed_cta_many([(g["K"], g["b"]) for g in group], tol=cfg.solver_tol,
                                     max_iter=cfg.solver_max_iter)
        for g, (w, info) in zip(group, res):
            add_pending(g["dev"], w, info, True, *g["meta"])
        group.clear()

    for si, (dev_s, s_off, n_s, rel, faults) in enumerate(_split(interpolation_input, options, data_descriptor,
                                                                  device)):
        if faults:
            flush_group()
            finalize()   # the fault series' isovalues are needed on the host
            # the fault blocks at this series' surface points are its fault-drift functions
            vals = ev.series_values(K.Points(xyz=dev_s.sp_coords), si)
            dev_s.set_fault_blocks(torch.stack([vals[j] for j in faults]))
        if getattr(ko, "compute_condition_number", False):
            Kc, _ = K.build(dev_s, GK_F64)
            conds.append(K.condition_number(Kc))
            del Kc
        if mixed and cfg.learned_min_n > 0 and dev_s.N >= cfg.learned_min_n and cost_model is None:
            cost_model = _load_cost_model(cfg.learned_model, device)
        learned = mixed and cost_model is not None and dev_s.N >= cfg.learned_min_n
        if mixed and not learned and dev_s.N <= CTA_MAX_N:
            Kd, b = K.build(dev_s, GK_F64)
            group.append({"dev": dev_s, "K": Kd, "b": b, "meta": (s_off, n_s, rel, faults)})
            continue
        flush_group()
        w, info, cta = _solve_one(dev_s, cfg, mixed, cost_model, interpolation_input, si, device)
        add_pending(dev_s, w, info, cta, s_off, n_s, rel, faults)
    flush_group()
    finalize()
    if conds:
        # the engine reports one number on the options; with several series, the largest
        ko.condition_number = float(max(conds))
    return series


def _isovalues(dev_s, model):
    """FP64 field at each surface's reference point (device tensor)."""
    fv = None
    if dev_s.n_faults:
        starts = torch.as_tensor(np.concatenate([[0], np.cumsum(dev_s.points_per_surface)[:-1]])).to(dev_s.device)
        fv = dev_s.fault_sp[:, starts]
    iso_t, _, _, _ = K.evaluate(dev_s, model, K.Points(xyz=dev_s.ref_points), GK_F64, fault_values=fv)
    return iso_t


def octree_refine_mode(level, n_levels, min_level, levels_surface, error_threshold):
    """``refine`` of gk_octree_level for octree level ``level``: 0 on the last
    level; 2 (every voxel) while the next level is below ``octree_min_level``;
    3 (corner ids and the interpolation-error statistic) while the next level
    is also below ``number_octree_levels_surface - 1`` and
    ``octree_error_threshold`` > 0; else 1 (corner ids)."""
    if level == n_levels - 1:
        return 0
    if level + 1 < min_level:
        return 2
    if error_threshold > 0 and level + 1 < levels_surface - 1:
        return 3
    return 1


def compute_model(interpolation_input, options, data_descriptor, geophysics_input=None,
                  config: Optional[EngineConfig] = None) -> Solutions:
    if not torch.cuda.is_available():
        raise RuntimeError("gempy_gb300.compute_model needs a CUDA device (there is no CPU fallback)")
    with K.on_current_stream():
        return _compute_model(interpolation_input, options, data_descriptor, geophysics_input, config)


def _attach_grads(sol, records, series, interpolation_input, options, data_descriptor, device):
    """Makes every octree level's scalar fields differentiable: one
    ``adjoint.series_field`` per series over all levels' points, split back
    into the levels, on leaf tensors of the inputs."""
    import copy

    from . import adjoint
    ii = interpolation_input
    leaf = lambda a: torch.as_tensor(np.asarray(a, dtype=np.float64)).to(device).requires_grad_(True)
    sp = leaf(np.asarray(ii.surface_points.sp_coords).reshape(-1, 3))
    nsp = leaf(ii.surface_points.nugget_effect_scalar)
    dpos = leaf(np.asarray(ii.orientations.dip_positions).reshape(-1, 3))
    dgr = leaf(np.asarray(ii.orientations.dip_gradients).reshape(-1, 3))
    ngr = leaf(ii.orientations.nugget_effect_grad)
    taped = copy.copy(ii)
    taped.surface_points = copy.copy(ii.surface_points)
    taped.orientations = copy.copy(ii.orientations)
    taped.surface_points.sp_coords, taped.surface_points.nugget_effect_scalar = sp, nsp
    taped.orientations.dip_positions, taped.orientations.dip_gradients = dpos, dgr
    taped.orientations.nugget_effect_grad = ngr
    sol.taped_interpolation_input = taped
    if not records:
        return
    ko = options.kernel_options
    ss = data_descriptor.stack_structure
    views = [r.level.views(r.result) for r in records]
    xyz = torch.cat([v[0] for v in views])
    sizes = [int(v[0].shape[0]) for v in views]
    p_off = o_off = 0
    for si, s in enumerate(series):
        n_p = int(ss.number_of_points_per_stack[si])
        n_o = int(ss.number_of_orientations_per_stack[si])
        fv = torch.cat([v[2][s.faults] for v in views], dim=1).detach() if s.faults else None
        spec = adjoint.SeriesSpec(s.dev.points_per_surface, ko.range, ko.c_o, ko.uni_degree, ko.kernel_function,
                                  ko.i_res, ko.gi_res, s.dev.fault_sp, fv)
        z = adjoint.series_field(sp[p_off:p_off + n_p], nsp[p_off:p_off + n_p], dpos[o_off:o_off + n_o],
                                 dgr[o_off:o_off + n_o], ngr[o_off:o_off + n_o], xyz, spec)
        for lv, r, zl in zip(sol.octrees_output, records, torch.split(z, sizes)):
            n = r.level.n
            lv.outputs[si].exported_fields.scalar_field = zl if r.surface else zl[:n]
            if si == len(series) - 1:
                lv.last_output_center.exported_fields.scalar_field = zl[:n]
                if lv.last_output_corners is not None:
                    lv.last_output_corners.exported_fields.scalar_field = zl[n:]
        p_off += n_p
        o_off += n_o


def _compute_model(interpolation_input, options, data_descriptor, geophysics_input, config) -> Solutions:
    cfg = config or EngineConfig()
    if cfg.compute_grads:
        if str(cfg.dtype) != "float64":
            raise ValueError("compute_grads needs the FP64 form (dtype='float64'): the adjoint reuses its LU factors")
        cfg = dataclasses.replace(cfg, keep_on_device=True)
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
    grid = interpolation_input.grid
    eo = options.evaluation_options
    want_grad = bool(eo.compute_scalar_gradient)

    # ---- 4a: octree levels.  One library call per level (gk_octree_level):
    # the level's points ([centres; 8 corners per centre] where corners are
    # needed), every series there, their combination and the children of the
    # refined voxels, in one device buffer.  The loop reads only the size of
    # the next level; each level's results go to the host while the next
    # level computes, and the output objects are built once, after the loop.
    t1 = time.perf_counter()
    stager = None if cfg.keep_on_device else _HostStager()
    records = []
    n_levels = int(eo.number_octree_levels)
    min_level = int(eo.octree_min_level)
    levels_surface = int(getattr(eo, "number_octree_levels_surface", getattr(eo, "_number_octree_levels_surface", 0)))
    error_threshold = float(getattr(eo, "octree_error_threshold", 1.0))
    if float(getattr(eo, "octree_curvature_threshold", -1.0)) >= 0 and grid.octree_grid is not None:
        warnings.warn("octree_curvature_threshold is not supported: the octree refines by corner ids and "
                      "the interpolation-error statistic only", RuntimeWarning, stacklevel=3)
    if grid.octree_grid is not None and n_levels >= 1:
        og = grid.octree_grid
        centres = torch.as_tensor(og.values).to(device)
        d = np.array(og.dxdydz, dtype=np.float64)
        ss = ev._set()
        for level in range(n_levels):
            last = level == n_levels - 1
            surface = level < levels_surface
            refine = octree_refine_mode(level, n_levels, min_level, levels_surface, error_threshold)
            lvl = K.OctreeLevel(ss, centres, d, prec, corners=surface or refine in (1, 3), refine=refine,
                                fault_series=ev._frows, error_threshold=error_threshold)
            grads = [None] * len(series)
            if want_grad:
                pts, _, V, _, _, _, _ = lvl.views(lvl.buffer)
                grads = ev.gradients(K.Points(xyz=pts), V)
            result = lvl.buffer[:lvl.result_bytes]
            records.append(_LevelRecord(lvl, result, d.copy(), surface, grads))
            if stager is not None:
                stager.push(result, *grads)   # copied while the next level computes
            if last:
                break
            centres = lvl.children()
            d = d / 2.0
            if cfg.timings:
                torch.cuda.synchronize()
                timings.setdefault("levels_s", []).append(time.perf_counter() - t1)
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
        raw.lith_block = e.block
        raw.scalar_field_matrix = e.fields
        raw.mask_matrix_squeezed = e.masks
        raw.block_matrix = e.values
    if grid.custom_grid is not None:
        pts = torch.as_tensor(grid.custom_grid.values).to(device)
        e = ev.run(K.Points(xyz=pts))
        raw.custom = e.block
    grav = None
    cg = getattr(grid, "geophysics_grid", None)
    if cg is not None and geophysics_input is not None and getattr(geophysics_input, "tz", None) is not None:
        # forward gravity: segment the centred grid's points, then density x tz per device
        from . import gravity as G
        e = ev.run(K.Points(xyz=torch.as_tensor(cg.values).to(device)))
        grav = G.device_gravity(e.lith_ids, cg, geophysics_input, device)
    if cfg.timings:
        torch.cuda.synchronize()
        timings["grids_s"] = time.perf_counter() - t2

    octrees = [] if stager is not None else [_level_output(r, ev, series, r.result, r.grads) for r in records]
    root = RootOutput([InterpOutput(ExportedFields(scalar_field=None, scalar_field_at_surface_points=s.iso),
                                    None, weights=s.weights) for s in series])
    sfsp = [float(v) for s in series for v in s.iso]
    sol = Solutions(octrees_output=octrees, root_output=root, raw_arrays=raw,
                    scalar_field_at_surface_points=sfsp, _ordered_elements=[s.order for s in series],
                    block_solution_type=options.block_solutions_type, timings=timings,
                    solver_info=[s.info_host for s in series],
                    gravity=None if grav is None else grav.cpu().numpy())
    if cfg.timings:
        torch.cuda.synchronize()
        t3 = time.perf_counter()
    if stager is not None:
        stager.stage(sol.root_output)     # the octree levels are already on their way
        stager.stage(sol.raw_arrays)
        stager.finish()
        sol.octrees_output = [_level_output(r, ev, series, stager.host(r.result), [stager.host(g) for g in r.grads])
                              for r in records]
    if cfg.compute_grads:
        _attach_grads(sol, records, series, interpolation_input, options, data_descriptor, device)
    if cfg.timings:
        timings["transfer_s"] = time.perf_counter() - t3
        timings["total_s"] = time.perf_counter() - t0
    return sol
