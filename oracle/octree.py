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

The engine also refines voxels by an error statistic (``octree_error_threshold``,
default 1.0; the developer log contrasts voxels "marked by stats" with those
"marked by corners", docs/developers_notes/dev_log/log_2024-06.md:26-39).  Its
definition is not in the reference either.  ``error_marks`` restates it as: per
series, the error of trilinear interpolation at the voxel centre, |Z(centre) -
mean of the 8 corner values|, in units of the corners' standard deviation; a
voxel is marked when that error exceeds the level's mean error by
``octree_error_threshold`` standard deviations of the level's errors.  It is
applied while the next level is below ``number_octree_levels_surface - 1``.
This form was fitted to the combination model's approval file (its 51 sampled
last-level values fix the finest level's 4328 voxels, 96 more than the corner
rule gives, all children of four level-1 voxels that this statistic picks); on
the anticline and the one-fault model it adds no voxel, so their point lists
are unchanged.  Errors at or below ``ERROR_FLOOR`` are the rounding of a field
that is linear over the voxel and never mark it.
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


ERROR_FLOOR = 1e-6


def interpolation_error(centre_field, corner_field):
    """|Z(centre) - mean of its 8 corners| / std of the 8 corners (0 where the
    corners are all equal), per voxel."""
    zc = np.asarray(corner_field, dtype=np.float64).reshape(-1, 8)
    z0 = np.asarray(centre_field, dtype=np.float64)
    sd = zc.std(axis=1)
    return np.where(sd > 0, np.abs(z0 - zc.mean(axis=1)) / np.where(sd > 0, sd, 1.0), 0.0)


def error_marks(centre_fields, corner_fields, n_std):
    """Voxels whose interpolation error, in any series, exceeds that series'
    level mean by ``n_std`` standard deviations (and ERROR_FLOOR)."""
    sel = np.zeros(len(np.asarray(centre_fields[0])), dtype=bool)
    for z0, zc in zip(centre_fields, corner_fields):
        e = interpolation_error(z0, zc)
        sel |= (e > e.mean() + n_std * e.std()) & (e > ERROR_FLOOR)
    return sel


def children(centres, spacing):
    q = np.asarray(spacing) / 4.0
    return (centres[:, None, :] + CORNER_SIGNS[None] * q).reshape(-1, 3)
