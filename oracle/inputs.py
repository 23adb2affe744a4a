"""Oracle ``Series`` lists from engine-style inputs or from golden fixtures.

Test infrastructure, like the rest of ``oracle/``.  The split of the
concatenated inputs into series follows the engine's input descriptor
(``InputDataDescriptor.stack_structure``: points, orientations and surfaces
per stack, ``gempy/core/data/structural_frame.py:306-317``).
"""
import numpy as np

from . import kriging, segmentation

RELATIONS = {"ERODE": segmentation.ERODE, "ONLAP": segmentation.ONLAP, "FAULT": segmentation.FAULT,
             "BASEMENT": segmentation.BASEMENT}


def series_from_engine_inputs(interpolation_input, options, data_descriptor):
    """Oracle Series of engine inputs (``InterpolationInput``, options, descriptor)."""
    ii, dd, ko = interpolation_input, data_descriptor, options.kernel_options
    ss = dd.stack_structure
    pps = dd.tensors_structure.number_of_points_per_surface
    out = []
    p = o = s = 0
    for i in range(ss.n_stacks):
        n_p, n_o, n_s = (int(ss.number_of_points_per_stack[i]), int(ss.number_of_orientations_per_stack[i]),
                         int(ss.number_of_surfaces_per_stack[i]))
        out.append(kriging.Series(ii.orientations.dip_positions[o:o + n_o], ii.orientations.dip_gradients[o:o + n_o],
                                  ii.orientations.nugget_effect_grad[o:o + n_o], ii.surface_points.sp_coords[p:p + n_p],
                                  ii.surface_points.nugget_effect_scalar[p:p + n_p], pps[s:s + n_s],
                                  range=ko.range, c_o=ko.c_o, uni_degree=ko.uni_degree,
                                  kernel=getattr(ko.kernel_function, "value", ko.kernel_function),
                                  i_res=ko.i_res, gi_res=ko.gi_res))
        p += n_p
        o += n_o
        s += n_s
    return out


def series_from_golden(g):
    """(series, relations, fault_relations) of a golden fixture.  Single-series
    fixtures (no ``series`` key) are one BASEMENT series without faults."""
    ko = g["kernel_options"]
    sp = np.asarray(g["sp_coords"], dtype=np.float64)
    nsp = np.asarray(g["nugget_sp"], dtype=np.float64)
    dp = np.asarray(g["dip_positions"], dtype=np.float64).reshape(-1, 3)
    dg = np.asarray(g["dip_gradients"], dtype=np.float64).reshape(-1, 3)
    ng = np.asarray(g["nugget_grad"], dtype=np.float64)
    pps = list(g["points_per_surface"])
    groups = g.get("series") or [{"elements": g["elements"], "relation": "BASEMENT"}]
    # orientations follow the element order of the fixture
    ori_counts = g.get("orientations_per_element")
    if ori_counts is None:
        ori_counts = _orientations_per_element(g)
    out, rels = [], []
    e = p = o = 0
    for grp in groups:
        ne = len(grp["elements"])
        n_p = int(sum(pps[e:e + ne]))
        n_o = int(sum(ori_counts[e:e + ne]))
        out.append(kriging.Series(dp[o:o + n_o], dg[o:o + n_o], ng[o:o + n_o], sp[p:p + n_p], nsp[p:p + n_p],
                                  np.asarray(pps[e:e + ne]), range=ko["range"], c_o=ko["c_o"],
                                  uni_degree=ko["uni_degree"], kernel=ko["kernel_function"], i_res=ko["i_res"],
                                  gi_res=ko["gi_res"]))
        rels.append(RELATIONS[grp["relation"]])
        e += ne
        p += n_p
        o += n_o
    rels[-1] = segmentation.BASEMENT
    fr = g.get("fault_relations")
    return out, rels, (None if fr is None else np.asarray(fr, dtype=bool))


def _orientations_per_element(g):
    """Orientations per element, recovered from the fixture's element order
    (the fixture lists them element by element; fixtures written before this
    field existed have a single series)."""
    counts = g.get("orientation_counts")
    if counts is not None:
        return counts
    if "series" not in g:
        return [len(g["dip_positions"])] + [0] * (len(g["elements"]) - 1)
    raise KeyError("multi-series fixture without orientation_counts")


def golden_extent(g):
    """Model extent in the transformed frame."""
    pos = np.array(g["transform"]["position"], dtype=np.float64)
    sc = g["transform"]["scale"]
    return (np.array(g["extent"], float).reshape(3, 2) + pos[:, None]).ravel() * sc
