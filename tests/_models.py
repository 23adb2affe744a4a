"""Shared fixtures: golden-vector models and oracle adapters for the tests."""
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_golden(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


def oracle_series_from_golden(g):
    """The single series of a one-series fixture."""
    from oracle import inputs
    series, _, _ = inputs.series_from_golden(g)
    assert len(series) == 1
    return series[0]


def golden_extent(g):
    from oracle import inputs
    return inputs.golden_extent(g)


def oracle_series_list(model):
    """Oracle Series objects of a gempy_gb300 synthetic model (same split as the engine)."""
    from oracle import inputs
    return inputs.series_from_engine_inputs(model.interpolation_input, model.options, model.data_descriptor)


def engine_inputs_from_golden(g, levels=None, custom=None):
    """(interpolation_input, options, data_descriptor, extent) of a golden
    fixture, as the reference's adapter would hand them to the engine
    (``gempy/modules/data_manipulation/_engine_factory.py:14-105``)."""
    import gempy_gb300 as gg
    from oracle import inputs
    ko = g["kernel_options"]
    oc = g.get("octree", {})
    levels = oc.get("levels", 1) if levels is None else levels
    opts = gg.InterpolationOptions.from_args(range=ko["range"], c_o=ko["c_o"], uni_degree=ko["uni_degree"],
                                             i_res=ko["i_res"], gi_res=ko["gi_res"],
                                             kernel_function=ko["kernel_function"], number_octree_levels=levels)
    if "levels_surface" in oc:
        opts.evaluation_options.number_octree_levels_surface = oc["levels_surface"]
    ext = inputs.golden_extent(g)
    grid = gg.EngineGrid(octree_grid=gg.RegularGrid(ext, oc.get("base_resolution", [2, 2, 2])),
                         custom_grid=gg.GenericGrid(np.asarray(custom)) if custom is not None else None)
    ii = gg.InterpolationInput(gg.SurfacePoints(g["sp_coords"], g["nugget_sp"]),
                               gg.Orientations(g["dip_positions"], g["dip_gradients"], g["nugget_grad"]),
                               grid, unit_values=np.array(g["unit_values"], float))
    groups = g.get("series") or [{"elements": g["elements"], "relation": "BASEMENT"}]
    pps = list(g["points_per_surface"])
    ocount = g["orientation_counts"]
    sps, ops, rels = [], [], []
    e = 0
    for grp in groups:
        ne = len(grp["elements"])
        sps.append(ne)
        ops.append(int(sum(ocount[e:e + ne])))
        rels.append(gg.StackRelationType[grp["relation"]])
        e += ne
    dd = gg.InputDataDescriptor.from_arrays(pps, sps, ops, rels, g.get("fault_relations"))
    return ii, opts, dd, ext
