"""Shared fixtures: golden-vector models and oracle adapters for the tests."""
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_golden(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


def oracle_series_from_golden(g):
    from oracle import kriging
    ko = g["kernel_options"]
    return kriging.Series(np.array(g["dip_positions"]), np.array(g["dip_gradients"]), np.array(g["nugget_grad"]),
                          np.array(g["sp_coords"]), np.array(g["nugget_sp"]), np.array(g["points_per_surface"]),
                          range=ko["range"], c_o=ko["c_o"], uni_degree=ko["uni_degree"],
                          kernel=ko["kernel_function"], i_res=ko["i_res"], gi_res=ko["gi_res"])


def golden_extent(g):
    pos = np.array(g["transform"]["position"])
    sc = g["transform"]["scale"]
    return (np.array(g["extent"], float).reshape(3, 2) + pos[:, None]).ravel() * sc


def oracle_series_list(model):
    """Oracle Series objects of a gempy_gb300 synthetic model (same split as the engine)."""
    from oracle import kriging
    ii, dd, ko = model.interpolation_input, model.data_descriptor, model.options.kernel_options
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
