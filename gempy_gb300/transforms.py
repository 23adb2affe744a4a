"""Input transform: centre the data and scale it into a unit-size box.

Mirrors the transform gempy builds with ``Transform.from_input_points``
(``gempy/core/data/geo_model.py:244-247``), whose values are pinned by the
reference's approved model JSONs: the anticline inputs give position
[-500, -500, -510], scale 5e-4 (``test/test_modules/test_grids/
test_custom_grid.test_custom_grid.verify/fold.approved.txt:108-126``) and the
horizontal inputs [-500, -500, -500], 6.25e-4 -- i.e. position = -(midpoint of
the bounding box of surface points and orientations) and scale =
1 / (2 * largest side of that box).  Transformed = (x + position) * scale.
"""
from dataclasses import dataclass

import numpy as np


@dataclass
class Transform:
    position: np.ndarray
    scale: np.ndarray

    @classmethod
    def from_input_points(cls, sp_xyz, ori_xyz):
        pts = np.concatenate([np.reshape(sp_xyz, (-1, 3)), np.reshape(ori_xyz, (-1, 3))])
        lo, hi = pts.min(0), pts.max(0)
        centre = (lo + hi) / 2.0
        side = float(np.max(hi - lo))
        s = 1.0 / (2.0 * side) if side > 0 else 1.0
        return cls(position=-centre, scale=np.full(3, s))

    def apply(self, xyz):
        return (np.asarray(xyz, dtype=np.float64) + self.position) * self.scale

    def apply_inverse(self, xyz):
        return np.asarray(xyz, dtype=np.float64) / self.scale - self.position

    def transform_gradient(self, g):
        # uniform scale, no rotation: directions are unchanged
        return np.asarray(g, dtype=np.float64)

    def extent(self, extent_world):
        e = np.asarray(extent_world, dtype=np.float64).reshape(3, 2)
        return ((e + self.position[:, None]) * self.scale[:, None]).ravel()
