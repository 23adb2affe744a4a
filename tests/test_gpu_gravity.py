"""Forward gravity on the GPU (``gk_gravity_tz``, ``gk_gravity`` and
``compute_model(..., geophysics_input)``) against the oracle's restatement
(``oracle/gravity.py``), on the reference's two-layer gravity model
(``test/test_modules/test_geophysics/test_gravity.py:10-89``).

Tolerances: tz is a sum of eight FP64 log/atan terms per voxel whose
cancellation grows with the voxel's distance; CUDA's and the host's log and
atan differ by an ulp or two, so tz agrees to 1e-11 of the largest |tz|.
Gravity sums density x tz over the voxels in a fixed order on each side:
1e-11 relative.  Lithology ids of the kernel points are compared exactly.

The reference's value for this model, -1624.1714 (test_gravity.py:89,
``assert_almost_equal(..., decimal=4)``), is reproduced through
compute_model on the GPU."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import gravity as ograv  # noqa: E402
from oracle import kriging, pipeline, segmentation  # noqa: E402

pytestmark = pytest.mark.gpu

# the reference's two-layer model (test_gravity.py:10-60) and its transform
# (test_gravity.test_gravity.verify/2-layers.approved.txt, "input_transform")
POSITION = np.array([-6.0, -0.0, -2.51])
SCALE = np.array([0.08333333333333333, 0.16778523489932887, 0.08333333333333333])
SP = np.array([[3, 0, 3.05], [9, 0, 3.05], [3, 0, 1.02], [9, 0, 1.02]], dtype=np.float64)
ORI = np.array([[6, 0, 4]], dtype=np.float64)
DENSITIES = np.array([2.6, 2.4, 3.2])


def _tr(p):
    return (np.asarray(p, dtype=np.float64) + POSITION) * SCALE


def _model(centers, resolution, radius):
    import gempy_gb300 as gg
    cg_model = gg.data.CenteredGrid(centers, resolution, radius)               # model units: tz
    cg = gg.data.CenteredGrid(_tr(centers), resolution, np.asarray(radius) * SCALE)   # engine frame
    opts = gg.InterpolationOptions.from_args(range=1.7, c_o=10.0, uni_degree=1, number_octree_levels=1)
    ii = gg.InterpolationInput(gg.SurfacePoints(_tr(SP)), gg.Orientations(_tr(ORI), [[0.0, 0.0, 1.0]]),
                               gg.EngineGrid(geophysics_grid=cg), unit_values=np.array([1.0, 2.0, 3.0]))
    dd = gg.InputDataDescriptor.from_arrays([2, 2], [2], [1], [gg.StackRelationType.BASEMENT])
    return ii, opts, dd, cg_model, cg


def _oracle_ids(cg):
    s = kriging.Series(_tr(ORI), np.array([[0.0, 0.0, 1.0]]), np.full(1, 0.01), _tr(SP), np.full(4, 2e-5),
                       np.array([2, 2]), range=1.7, c_o=10.0, uni_degree=1)
    r = pipeline.compute([s], [segmentation.BASEMENT], [1.0, 2.0, 3.0], 5e6, cg.values)
    return r.ids


def test_tz_kernel_matches_oracle():
    from gempy_gb300 import gravity
    from gempy_gb300.data import CenteredGrid
    for res, rad in (([10, 10, 100], 16000.0), ([24, 6, 30], [150.0, 10.0, 300.0])):
        cg = CenteredGrid(np.zeros((1, 3)), res, rad)
        t = gravity.calculate_gravity_gradient(cg)
        to = ograv.tz(res, rad)
        assert np.abs(t - to).max() <= 1e-11 * np.abs(to).max()


@pytest.mark.parametrize("centers,resolution,radius", [
    ([[6.0, 0.0, 4.0]], [10, 10, 100], [16000.0] * 3),                     # the reference's test grid
    ([[2.0, 0.0, 4.0], [6.0, 0.0, 4.0], [10.0, 0.0, 3.5]], [8, 4, 40], [3.0, 1.0, 3.5]),  # kernels across the layers
])
def test_compute_model_gravity_matches_oracle(centers, resolution, radius):
    import gempy_gb300 as gg
    from gempy_gb300 import gravity
    ii, opts, dd, cg_model, cg = _model(np.array(centers), resolution, radius)
    tz = gravity.calculate_gravity_gradient(cg_model)
    sol = gg.compute_model(ii, opts, dd, gg.data.GeophysicsInput(tz=tz, densities=DENSITIES))
    ids = _oracle_ids(cg)
    g_ref = ograv.gravity(ids, DENSITIES, ograv.tz(resolution, radius))
    assert sol.gravity.shape == (len(centers),)
    np.testing.assert_allclose(sol.gravity, g_ref, rtol=1e-11, atol=0)
    if len(centers) > 1:
        # the smaller kernels straddle the layers: more than one lithology is summed
        assert len(np.unique(ids)) > 1
    else:
        # the reference's kernel lies far below both surfaces: basement only
        assert (ids == 3).all()
        assert abs(sol.gravity[0] - 3.2 * ograv.tz(resolution, radius).sum()) <= 1e-11 * abs(sol.gravity[0])
        # the reference's own check (test_gravity.py:89)
        np.testing.assert_almost_equal(sol.gravity, np.array([-1624.1714]), decimal=4)


def test_gravity_reduction_is_deterministic():
    from gempy_gb300 import kernels as K
    rng = np.random.default_rng(0)
    n_dev, n_vox = 5, 12221
    ids = torch.as_tensor(rng.integers(1, 4, n_dev * n_vox).astype(np.int32)).cuda()
    tz = torch.as_tensor(rng.normal(size=n_vox)).cuda()
    rho = torch.as_tensor(DENSITIES).cuda()
    a = K.gravity(ids, n_dev, rho, tz).cpu().numpy()
    b = K.gravity(ids, n_dev, rho, tz).cpu().numpy()
    np.testing.assert_array_equal(a, b)
    ref = ograv.gravity(ids.cpu().numpy(), DENSITIES, tz.cpu().numpy())
    np.testing.assert_allclose(a, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())
