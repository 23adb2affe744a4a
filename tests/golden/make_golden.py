"""Generate the golden fixtures under tests/golden/ from the reference's own
bundled inputs and known answers.  Run in a container that has the reference
checkout (it reads it as data; nothing here runs reference code):

    python tests/golden/make_golden.py /path/to/gempy-reference

Fixtures written:

* ``anticline_corners.json`` -- the anticline example model
  (``gempy/API/examples_generator.py:165-195``: extent [0,1000]^3, series
  ``Strat_Series`` = (rock2, rock1), inputs
  ``examples/data/input_data/jan_models/model2_{surface_points,orientations}.csv``)
  transformed with the input transform pinned by the reference's approved JSON
  (``test/test_modules/test_grids/test_custom_grid.test_custom_grid.verify/
  fold.approved.txt:108-126``: position [-500,-500,-510], scale 5e-4), the
  kernel options of the same file (:127-160), the 8 cube corners of
  ``test_custom_grid.py:10-21`` and their expected ids ``[3,3,3,3,1,1,1,1]``
  (``test_custom_grid.py:44-47, 62-65``), plus the 51 scalar-field values
  of the finest octree level (refinement 5, base resolution 2^3) from
  ``test/test_model_types/test_example_models_I.test_generate_fold_model.
  Anticline Scalar Field.approved.txt`` sampled as in
  ``test_example_models_I.py:19-23`` (every ``len // 50``-th value).
* ``horizontal_inputs.json`` -- the horizontal-strata example
  (``examples_generator.py:132-162``, ``model1_*.csv``) with the transform of
  ``...Horizontal Stratigraphic Model serialization.approved.txt:107-126``, used
  for the exact-linear-field known answer.
* ``fault_model.json`` -- the one-fault example (``examples_generator.py:
  198-241``: extent [0,1000]^3, refinement 6, ``Fault_Series`` = fault (FAULT,
  offsetting ``Strat_Series`` = (rock2, rock1)), ``model5_*.csv``) with the 51
  approved values of ``test_example_models_I.test_generate_fault_model.Fault
  Scalar Field.approved.txt`` (``test_example_models_I.py:56-68``).
* ``combination_model.json`` -- the fold/unconformity/fault example
  (``examples_generator.py:244-293``: extent [0,2500]x[0,1000]^2, refinement
  4, octree base resolution from the extent ratios (``gempy/core/data/
  grid.py:128-151``), ``number_octree_levels_surface`` 4, series
  fault (FAULT) / rock3 (ERODE) / (rock2, rock1), ``model7_*.csv``) with the 51
  approved values of ``...test_generate_combination_model.Combination Scalar
  Field.approved.txt`` (``test_example_models_I.py:71-88``).

The input transform of the fault and combination models is not serialized in
the reference; it follows the rule that reproduces both serialized ones (the
anticline's and the horizontal model's): position = -(centre of the bounding
box of all surface points and orientations), scale = 1 / (2 x the largest
bounding-box side).

Usage: ``python tests/golden/make_golden.py <path-to-reference-checkout>``.
"""
import csv
import json
import os
import sys

import numpy as np


def read_csv(path):
    with open(path) as f:
        return list(csv.DictReader(f))


def pole(az, dip, pol):
    # gempy/API/io_API.py:96-103
    az, dip = np.deg2rad(float(az)), np.deg2rad(float(dip))
    return [np.sin(dip) * np.sin(az) * float(pol), np.sin(dip) * np.cos(az) * float(pol),
            np.cos(dip) * float(pol)]


def input_transform(ref_root, stem):
    """(position, scale) from the bounding box of every input point."""
    d = os.path.join(ref_root, "examples/data/input_data/jan_models")
    pts = [[float(r["X"]), float(r["Y"]), float(r["Z"])]
           for f in ("surface_points", "orientations") for r in read_csv(os.path.join(d, f"{stem}_{f}.csv"))]
    pts = np.asarray(pts)
    hi, lo = pts.max(0), pts.min(0)
    return (-(hi + lo) / 2.0).tolist(), float(1.0 / (2.0 * np.max(hi - lo)))


def approved_values(ref_root, name):
    path = os.path.join(ref_root, "test/test_model_types", f"test_example_models_I.{name}.approved.txt")
    with open(path) as f:
        return [float(v) for v in f.read().replace("[", " ").replace("]", " ").split()]


def multi_series(ref_root, stem, groups, relations, fault_relations, extent, refinement, base_resolution,
                 levels_surface, approved):
    order = [e for g in groups for e in g]
    position, scale = input_transform(ref_root, stem)
    m = model(ref_root, stem, order, position, scale)
    m["extent"] = list(extent)
    m["series"] = [{"elements": list(g), "relation": r} for g, r in zip(groups, relations)]
    m["fault_relations"] = fault_relations
    m["octree"] = {"levels": refinement, "base_resolution": base_resolution, "levels_surface": levels_surface,
                   "approved_scalar_field_last_level": approved_values(ref_root, approved),
                   "approved_rtol": 1e-5, "approved_atol": 1e-5}
    return m


def model(ref_root, stem, order, position, scale):
    d = os.path.join(ref_root, "examples/data/input_data/jan_models")
    sp = read_csv(os.path.join(d, f"{stem}_surface_points.csv"))
    ori = read_csv(os.path.join(d, f"{stem}_orientations.csv"))
    pos = np.asarray(position, float)
    sc = float(scale)
    tr = lambda p: ((np.asarray(p, float) + pos) * sc).tolist()
    sp_xyz, counts, ori_xyz, grads, ocounts = [], [], [], [], []
    for name in order:  # structural elements in stack order (map_stack_to_surfaces)
        pts = [[float(r["X"]), float(r["Y"]), float(r["Z"])] for r in sp if r["formation"] == name]
        sp_xyz += pts
        counts.append(len(pts))
        ocounts.append(0)
        for r in ori:
            if r["formation"] == name:
                ori_xyz.append([float(r["X"]), float(r["Y"]), float(r["Z"])])
                grads.append(pole(r["azimuth"], r["dip"], r["polarity"]))
                ocounts[-1] += 1
    return {
        "elements": list(order),
        "sp_coords": tr(sp_xyz),
        "points_per_surface": counts,
        "orientation_counts": ocounts,
        "nugget_sp": [2e-5] * len(sp_xyz),        # surface_points.py:11
        "dip_positions": tr(ori_xyz),
        "dip_gradients": grads,                   # uniform scale, no rotation
        "nugget_grad": [0.01] * len(ori_xyz),     # orientations.py:11
        "transform": {"position": list(position), "scale": sc},
        "kernel_options": {"range": 1.7, "c_o": 10.0, "uni_degree": 1, "i_res": 4.0,
                           "gi_res": 2.0, "kernel_function": "cubic"},
        "sigmoid_slope": 5_000_000,
        "unit_values": list(range(1, len(order) + 2)),
        "extent": [0, 1000, 0, 1000, 0, 1000],
    }


def main(ref_root):
    out = os.path.dirname(os.path.abspath(__file__))
    anti = model(ref_root, "model2", ("rock2", "rock1"), [-500.0, -500.0, -510.0], 0.0005)
    corners = [[0, 0, 0], [1000, 0, 0], [0, 1000, 0], [1000, 1000, 0],
               [0, 0, 1000], [1000, 0, 1000], [0, 1000, 1000], [1000, 1000, 1000]]
    anti["custom_points_world"] = corners
    anti["custom_points"] = ((np.asarray(corners, float) + np.asarray(anti["transform"]["position"]))
                             * anti["transform"]["scale"]).tolist()
    anti["expected_ids"] = [3, 3, 3, 3, 1, 1, 1, 1]
    approved = os.path.join(ref_root, "test/test_model_types/test_example_models_I."
                            "test_generate_fold_model.Anticline Scalar Field.approved.txt")
    with open(approved) as f:
        txt = f.read().replace("[", " ").replace("]", " ")
    anti["octree"] = {"levels": 5, "base_resolution": [2, 2, 2],
                      "approved_scalar_field_last_level": [float(v) for v in txt.split()],
                      "approved_rtol": 1e-5, "approved_atol": 1e-5}
    with open(os.path.join(out, "anticline_corners.json"), "w") as f:
        json.dump(anti, f, indent=1)
    hor = model(ref_root, "model1", ("rock2", "rock1"), [-500.0, -500.0, -500.0], 0.000625)
    with open(os.path.join(out, "horizontal_inputs.json"), "w") as f:
        json.dump(hor, f, indent=1)
    fault = multi_series(ref_root, "model5", [("fault",), ("rock2", "rock1")], ["FAULT", "BASEMENT"],
                         [[0, 1], [0, 0]], [0, 1000, 0, 1000, 0, 1000], 6, [2, 2, 2], 4,
                         "test_generate_fault_model.Fault Scalar Field")
    with open(os.path.join(out, "fault_model.json"), "w") as f:
        json.dump(fault, f, indent=1)
    comb = multi_series(ref_root, "model7", [("fault",), ("rock3",), ("rock2", "rock1")],
                        ["FAULT", "ERODE", "BASEMENT"], [[0, 1, 1], [0, 0, 0], [0, 0, 0]],
                        [0, 2500, 0, 1000, 0, 1000], 4, [4, 2, 2], 4,
                        "test_generate_combination_model.Combination Scalar Field")
    with open(os.path.join(out, "combination_model.json"), "w") as f:
        json.dump(comb, f, indent=1)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <path-to-reference-checkout>")
    main(sys.argv[1])
