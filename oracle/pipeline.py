"""Multi-series compute_model restatement (CPU, FP64).

Mirrors the control flow the reference's single engine call site delegates
(``gempy/API/compute_API.py:68-73``): per series build K and solve for the
weights (``_engine_factory.py:45-48`` reads them back per stack), evaluate at the
grid, take the isovalues at the surface points (``geo_model.py:107-108``),
segment each series, combine the series with their masks
(``raw_arrays.mask_matrix_squeezed``), and refine an octree level by level.
"""
from dataclasses import dataclass

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
    ids: np.ndarray         # combined ids


def series_unit_values(series_list, unit_values):
    out, off = [], 0
    for s in series_list:
        out.append(np.asarray(unit_values[off:off + s.n_k + 1], dtype=np.float64))
        off += s.n_k
    return out


def solve_all(series_list):
    ws, isos = [], []
    for s in series_list:
        K, b = kriging.build_system(s)
        w = kriging.solve(K, b)
        ws.append(w)
        isos.append(kriging.isovalues(s, w))
    return ws, isos


def evaluate_all(series_list, relations, unit_values, slope, points, ws, isos, gradient=False):
    uvs = series_unit_values(series_list, unit_values)
    fields, grads, svals = [], [], []
    for s, w, iso, uv in zip(series_list, ws, isos, uvs):
        if gradient:
            z, g = kriging.evaluate(s, w, points, gradient=True)
        else:
            z, g = kriging.evaluate(s, w, points), None
        fields.append(z)
        grads.append(g)
        svals.append(segmentation.segment(z, iso, uv, slope)[0])
    masks = segmentation.series_masks(fields, isos, relations)
    values = np.sum(masks * np.stack(svals), axis=0)
    return Result(ws, isos, fields, grads, svals, masks, values, np.rint(values))


def compute(series_list, relations, unit_values, slope, points, gradient=False):
    ws, isos = solve_all(series_list)
    return evaluate_all(series_list, relations, unit_values, slope, points, ws, isos, gradient)


def compute_octree(series_list, relations, unit_values, slope, extent, base_resolution,
                   n_levels, min_level=2):
    """List of (centres, Result) per level."""
    ws, isos = solve_all(series_list)
    centres, d = octree.base_centres(extent, base_resolution)
    levels = []
    for level in range(n_levels):
        res = evaluate_all(series_list, relations, unit_values, slope, centres, ws, isos)
        levels.append((centres, res))
        if level == n_levels - 1:
            break
        if level + 1 < min_level:
            sel = np.ones(len(centres), dtype=bool)
        else:
            rc = evaluate_all(series_list, relations, unit_values, slope,
                              octree.corners(centres, d), ws, isos)
            sel = octree.mark(rc.ids)
        centres = octree.children(centres[sel], d)
        d = d / 2.0
    return levels
