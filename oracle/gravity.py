"""Forward gravity on centred grids, restated on the CPU -- TEST INFRASTRUCTURE.

The reference computes gravity in its engine: ``gp.set_centered_grid(grid,
centers, resolution, radius)`` (``gempy/API/grid_API.py:99-108``) places a
kernel of voxels around every device, ``gp.calculate_gravity_gradient``
gives the vertical attraction ``tz`` of each voxel per unit density, the
engine's adapter moves the centres and radius into the transformed frame
(``gempy/modules/data_manipulation/_engine_factory.py:82-87``) where the
voxels are segmented, and ``Solutions.gravity`` is the density-weighted sum
per device (``test/test_modules/test_geophysics/test_gravity.py:67-89``).
The kernel construction and the tz formula live in the absent engine; this
module restates the published design (GemPy's centred grid, carried over from
its version 2, as the test's own comment on the radius says):

* the kernel, per axis: x and y symmetric about the device at
  ``radius * [-g[::-1], 0, g]`` with ``g = geomspace(0.01, 1, resolution // 2)``;
  z only below it at ``-1.2 * radius * (0.05 + [0, geomspace(0.01, 1,
  resolution)])`` (the vertical axis reaches 1.2 radii);
  each voxel reaches half-way to its neighbours, and the outermost voxels
  as far out as they reach in (so the voxels tile a box); voxels in ``ij``
  order (x slowest);
* tz: the closed-form vertical attraction of a rectangular prism (Nagy 1966;
  Plouff 1976), z up, so mass below the device gives a negative value, with
  G = 6.674e-3 (lengths in m, densities in g/cm^3, tz in mGal);
* gravity[d] = sum_v densities[id(d, v) - 1] * tz[v], id the lithology id of
  voxel v of device d.

``tests/test_oracle.py`` checks the prism formula against numerical
quadrature, the tiling against the attraction of the whole box, and the
reference's value for its two-layer model: every kernel voxel lies in the
basement (density 3.2), and 3.2 x sum(tz) = -1624.17138, the reference's
-1624.1714 to its 4 decimals (``test_gravity.py:89``).
"""
import numpy as np

G_MGAL = 6.674e-3
Z_STRETCH = 1.2     # the vertical axis of the kernel reaches 1.2 radii below the device


def axis_nodes(resolution, radius, vertical):
    """Voxel centres along one axis and their lower/upper half-widths."""
    if vertical:
        g = np.geomspace(0.01, 1.0, int(resolution))
        c = -Z_STRETCH * radius * (0.05 + np.concatenate(([0.0], g)))
        c = c[::-1]                      # increasing z
    else:
        g = np.geomspace(0.01, 1.0, int(resolution) // 2)
        c = radius * np.concatenate((-g[::-1], [0.0], g))
    gaps = np.diff(c)
    lo = np.concatenate(([gaps[0]], gaps)) / 2.0
    hi = np.concatenate((gaps, [gaps[-1]])) / 2.0
    return c, lo, hi


def kernel(resolution, radius):
    """(centres (n, 3), lower half-widths (n, 3), upper half-widths (n, 3)) of
    the voxels around a device at the origin, ``ij`` order."""
    radius = np.broadcast_to(np.asarray(radius, dtype=np.float64), (3,))
    ax = [axis_nodes(resolution[a], radius[a], a == 2) for a in range(3)]
    mesh = lambda k: np.stack([m.ravel() for m in np.meshgrid(ax[0][k], ax[1][k], ax[2][k], indexing="ij")], 1)
    return mesh(0), mesh(1), mesh(2)


def prism_tz(x0, x1, y0, y1, z0, z1):
    """Vertical attraction (z up, per unit density, mGal for lengths in m and
    g/cm^3) at the origin of the prism [x0, x1] x [y0, y1] x [z0, z1]."""
    s = 0.0
    for i, x in enumerate((x0, x1)):
        for j, y in enumerate((y0, y1)):
            for k, z in enumerate((z0, z1)):
                r = np.sqrt(x * x + y * y + z * z)
                sign = -1.0 if (i + j + k) % 2 else 1.0
                s = s + sign * (x * np.log(y + r) + y * np.log(x + r) - z * np.arctan(x * y / (z * r)))
    return G_MGAL * s


def tz(resolution, radius):
    c, lo, hi = kernel(resolution, radius)
    a, b = c - lo, c + hi
    return prism_tz(a[:, 0], b[:, 0], a[:, 1], b[:, 1], a[:, 2], b[:, 2])


def points(centers, resolution, radius):
    """Evaluation points of every device's kernel, device-major."""
    c, _, _ = kernel(resolution, radius)
    centers = np.asarray(centers, dtype=np.float64).reshape(-1, 3)
    return (centers[:, None, :] + c[None]).reshape(-1, 3)


def gravity(ids, densities, tz_values):
    """Density-weighted sum per device of ``ids`` (n_devices * n_voxels)."""
    tz_values = np.asarray(tz_values, dtype=np.float64)
    ids = np.asarray(ids).reshape(-1, len(tz_values)).astype(np.int64)
    rho = np.asarray(densities, dtype=np.float64)[ids - 1]
    return (rho * tz_values[None]).sum(1)
