"""Multi-series compute_model restatement (CPU, FP64).

Mirrors the control flow the reference's single engine call site delegates
(``gempy/API/compute_API.py:68-73``): per series build K and solve for the
weights (``_engine_factory.py:45-48`` reads them back per stack), evaluate at the
grid, take the isovalues at the surface points (``geo_model.py:107-108``),
segment each series, combine the series with their masks
(``raw_arrays.mask_matrix_squeezed``), and refine an octree level by level.

Faults.  ``fault_relations[j, i]`` true means the FAULT series j offsets the
younger series i (``gempy/core/data/structural_frame.py:244-273``).  Series
are solved in stack order, so every fault series is solved before the series
it offsets; the fault's block (its soft segmented values) at the younger
series' surface points enters that series' kriging system as a drift column,
and at every evaluation point the fault block is evaluated first.

Octree.  A voxel is refined when its 8 corners differ in lithology id (the
combined block) or in the id of any fault series' block, and every voxel is
refined while the next level is below ``octree_min_level`` (default 2).
While the next level is below ``number_octree_levels_surface - 1`` voxels are
also refined by the interpolation-error statistic of ``octree.error_marks``
(``octree_error_threshold`` standard deviations, default 1).  Levels below ``number_octree_levels_surface`` (default 4) also evaluate their
voxel corners for the mesh extraction that follows, and the reference exports
those corner values after the centres' (``exported_fields.scalar_field`` of
``octrees_output[l].outputs[s]``); ``compute_octree`` returns them per level.
"""
from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import kriging, octree, segmentation


@dataclass
class Result:
    weights: list
    isovalues: list
    fields: list            # per series (n,)
    gradients: list         # per series (n,3) or None
    series_values: list     # per series soft values
    masks: np.ndarray       # (n_series, n)
    values: np.ndarray      # combined soft values
    ids: np.ndarray         # combined lithology ids
    series_ids: list = None     # per series block ids
    fault_ids: list = None      # block ids of the FAULT series


def series_unit_values(series_list, unit_values):
    out, off = [], 0
    for s in series_list:
        out.append(np.asarray(unit_values[off:off + s.n_k + 1], dtype=np.float64))
        off += s.n_k
    return out


def _fault_sources(fault_relations, i):
    if fault_relations is None:
        return []
    fr = np.asarray(fault_relations, dtype=bool)
    return [j for j in range(i) if fr[j, i]]


class Model:
    """Solved multi-series model: weights, isovalues and unit values."""

    def __init__(self, series_list, relations, unit_values, slope, fault_relations=None):
        self.series = series_list
        self.relations = list(relations)
        self.slope = float(slope)
        self.fault_relations = fault_relations
        self.uvs = series_unit_values(series_list, unit_values)
        self.ws, self.isos = [], []
        for i, s in enumerate(series_list):
            src = _fault_sources(fault_relations, i)
            if src:
                s.fault_sp = np.column_stack([self.block(j, s.sp_coords) for j in src])
                s.ref_rest = None
            K, b = kriging.build_system(s)
            w = kriging.solve(K, b)
            self.ws.append(w)
            self.isos.append(kriging.isovalues(s, w))

    def field(self, i, x, gradient=False, cache=None):
        src = _fault_sources(self.fault_relations, i)
        fx = np.column_stack([self.block(j, x, cache) for j in src]) if src else None
        return kriging.evaluate(self.series[i], self.ws[i], x, gradient=gradient, fault_x=fx)

    def block(self, j, x, cache=None):
        """Soft segmented values of series j at x (the fault-drift function)."""
        if cache is not None and j in cache:
            return cache[j]
        z = self.field(j, x, cache=cache)
        v = segmentation.segment(z, self.isos[j], self.uvs[j], self.slope)[0]
        if cache is not None:
            cache[j] = v
        return v

    def evaluate(self, points, gradient=False):
        n_s = len(self.series)
        fields, grads, svals, sids = [], [], [], []
        cache = {}
        for i, (s, iso, uv) in enumerate(zip(self.series, self.isos, self.uvs)):
            src = _fault_sources(self.fault_relations, i)
            fx = np.column_stack([cache[j] for j in src]) if src else None
            if gradient:
                z, g = kriging.evaluate(s, self.ws[i], points, gradient=True, fault_x=fx)
            else:
                z, g = kriging.evaluate(s, self.ws[i], points, fault_x=fx), None
            v = segmentation.segment(z, iso, uv, self.slope)[0]
            cache[i] = v
            fields.append(z)
            grads.append(g)
            svals.append(v)
            sids.append(segmentation.hard_ids(z, iso, uv))
        masks = segmentation.series_masks(fields, self.isos, self.relations)
        values = np.sum(masks * np.stack(svals), axis=0)
        ids = np.sum(masks * np.stack(sids), axis=0)
        fids = [sids[i] for i in range(n_s) if self.relations[i] == segmentation.FAULT]
        return Result(self.ws, self.isos, fields, grads, svals, masks, values, ids, sids, fids)


def solve_all(series_list, fault_relations=None, relations=None, unit_values=None, slope=5e6):
    if fault_relations is None:
        ws, isos = [], []
        for s in series_list:
            K, b = kriging.build_system(s)
            w = kriging.solve(K, b)
            ws.append(w)
            isos.append(kriging.isovalues(s, w))
        return ws, isos
    m = Model(series_list, relations, unit_values, slope, fault_relations)
    return m.ws, m.isos


def compute(series_list, relations, unit_values, slope, points, gradient=False, fault_relations=None):
    m = Model(series_list, relations, unit_values, slope, fault_relations)
    return m.evaluate(points, gradient)


def refinement_marks(result):
    """Voxels (8 consecutive corners each) whose lithology or fault ids differ."""
    sel = octree.mark(result.ids)
    for f in result.fault_ids or []:
        sel |= octree.mark(f)
    return sel


@dataclass
class Level:
    centres: np.ndarray
    spacing: np.ndarray
    result: Result
    corners: Optional[np.ndarray] = None
    corner_result: Optional[Result] = None

    def exported_field(self, s):
        """``exported_fields.scalar_field`` of series s: the centres' values,
        followed by the corners' when the level evaluated them for meshing."""
        z = self.result.fields[s]
        if self.corner_result is None:
            return z
        return np.concatenate([z, self.corner_result.fields[s]])


def compute_octree(series_list, relations, unit_values, slope, extent, base_resolution,
                   n_levels, min_level=2, fault_relations=None, levels_surface=None, model=None,
                   error_threshold=1.0):
    """List of (centres, Result) per level (``levels_surface`` None); with
    ``levels_surface`` set, a list of ``Level`` records whose levels below it
    keep their corner evaluation.  Voxels are refined by the corner rule, and
    while the next level is below ``levels_surface - 1`` (4 when None) also
    by the interpolation-error statistic with ``error_threshold`` standard
    deviations (off when <= 0)."""
    m = model or Model(series_list, relations, unit_values, slope, fault_relations)
    centres, d = octree.base_centres(extent, base_resolution)
    out = []
    for level in range(n_levels):
        res = m.evaluate(centres)
        last = level == n_levels - 1
        surface = levels_surface is not None and level < levels_surface
        need_corners = (not last and level + 1 >= min_level) or surface
        corners = rc = None
        if need_corners:
            corners = octree.corners(centres, d)
            rc = m.evaluate(corners)
        out.append(Level(centres, d, res, corners if surface else None, rc if surface else None)
                   if levels_surface is not None else (centres, res))
        if last:
            break
        if level + 1 < min_level:
            sel = np.ones(len(centres), dtype=bool)
        else:
            sel = refinement_marks(rc)
            ls = 4 if levels_surface is None else levels_surface
            if error_threshold > 0 and level + 1 < ls - 1:
                sel |= octree.error_marks(res.fields, rc.fields, error_threshold)
        centres = octree.children(centres[sel], d)
        d = d / 2.0
    return out
