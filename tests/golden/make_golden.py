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


def model(ref_root, stem, order, position, scale):
    d = os.path.join(ref_root, "examples/data/input_data/jan_models")
    sp = read_csv(os.path.join(d, f"{stem}_surface_points.csv"))
    ori = read_csv(os.path.join(d, f"{stem}_orientations.csv"))
    pos = np.asarray(position, float)
    sc = float(scale)
    tr = lambda p: ((np.asarray(p, float) + pos) * sc).tolist()
    sp_xyz, counts, ori_xyz, grads = [], [], [], []
    for name in order:  # structural elements in stack order (map_stack_to_surfaces)
        pts = [[float(r["X"]), float(r["Y"]), float(r["Z"])] for r in sp if r["formation"] == name]
        sp_xyz += pts
        counts.append(len(pts))
        for r in ori:
            if r["formation"] == name:
                ori_xyz.append([float(r["X"]), float(r["Y"]), float(r["Z"])])
                grads.append(pole(r["azimuth"], r["dip"], r["polarity"]))
    return {
        "elements": list(order),
        "sp_coords": tr(sp_xyz),
        "points_per_surface": counts,
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


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
