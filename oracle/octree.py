"""Corner-based octree refinement over a regular base grid.

The reference defines the octree grid as a base resolution refined
``number_octree_levels`` times (``gempy/core/data/grid.py:128-151``,
``gempy/core/data/grid_modules/regular_grid.py:36-43``: the finest level has
``base * 2**(levels-1)`` cells per axis) with cell-centre coordinates
(``regular_grid.py:192-201``) in ``ij`` meshgrid order (``regular_grid.py:58-71``).
The engine's refinement rule is not in the reference; this restatement refines a
voxel when the lithology ids at its 8 corners are not all equal, refines every
voxel while the next level is below ``octree_min_level`` (default 2, approved
options JSON), and lists the 8 children of each refined voxel in corner order
(x slowest, z fastest) at centre +- spacing/4.
"""
import numpy as np

CORNER_SIGNS = np.array([[ix, iy, iz] for ix in (-1, 1) for iy in (-1, 1) for iz in (-1, 1)],
                        dtype=np.float64)


def base_centres(extent, resolution):
    extent = np.asarray(extent, dtype=np.float64)
    res = np.asarray(resolution, dtype=np.int64)
    d = (extent[1::2] - extent[0::2]) / res
    axes = [np.linspace(extent[2 * i] + d[i] / 2, extent[2 * i + 1] - d[i] / 2, res[i]) for i in range(3)]
    g = np.meshgrid(*axes, indexing="ij")
    return np.stack([a.ravel() for a in g], axis=1), d


def corners(centres, spacing):
    """(n*8, 3) corner coordinates, 8 consecutive per voxel."""
    half = np.asarray(spacing) / 2.0
    return (centres[:, None, :] + CORNER_SIGNS[None] * half).reshape(-1, 3)


def mark(corner_ids):
    c = np.asarray(corner_ids).reshape(-1, 8)
    return np.any(c != c[:, :1], axis=1)


def children(centres, spacing):
    q = np.asarray(spacing) / 4.0
    return (centres[:, None, :] + CORNER_SIGNS[None] * q).reshape(-1, 3)
