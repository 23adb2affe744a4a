"""CPU tests of the FP64 oracle: pinned golden vectors and known answers."""
import numpy as np
import pytest

from oracle import covariance, kriging, octree, pipeline, segmentation
from tests._models import golden_extent, load_golden, oracle_series_from_golden


def test_anticline_corner_ids_pinned():
    """test/test_modules/test_grids/test_custom_grid.py:44-47: ids at the cube corners."""
    g = load_golden("anticline_corners.json")
    s = oracle_series_from_golden(g)
    r = pipeline.compute([s], [segmentation.BASEMENT], g["unit_values"], g["sigmoid_slope"],
                         np.array(g["custom_points"]))
    np.testing.assert_array_equal(r.ids, np.array(g["expected_ids"], float))


def _anticline_sampled():
    g = load_golden("anticline_corners.json")
    s = oracle_series_from_golden(g)
    oc = g["octree"]
    levels = pipeline.compute_octree([s], [segmentation.BASEMENT], g["unit_values"], g["sigmoid_slope"],
                                     golden_extent(g), oc["base_resolution"], oc["levels"])
    z = levels[-1][1].fields[0]
    assert len(z) == 7808
    return z[:: len(z) // 50], np.array(oc["approved_scalar_field_last_level"])


def test_anticline_scalar_field_approval_file():
    """Finest octree level of the anticline vs the reference's approval file
    (test_example_models_I.py:19-23, 41-53), judged with the reference's own
    comparator np.allclose(rtol=1e-5, atol=1e-5) (test/verify_helper.py:70-103)."""
    sampled, approved = _anticline_sampled()
    assert sampled.shape == approved.shape
    assert np.allclose(sampled, approved, rtol=1e-5, atol=1e-5)
    assert np.abs(sampled - approved).max() < 4e-6


def test_anticline_approval_pins_distance_regulariser(monkeypatch):
    """The approval file selects the distance regulariser: without it (a bare
    sqrt at the r = 0 diagonal) 37 of the 51 values fail the reference's
    comparator; a hundred times larger one fails too."""
    for eps2 in (0.0, 1e-8):
        monkeypatch.setattr(kriging, "DIST_EPS2", eps2)
        sampled, approved = _anticline_sampled()
        assert not np.allclose(sampled, approved, rtol=1e-5, atol=1e-5), eps2


def test_kernel_symmetric_and_rhs():
    g = load_golden("anticline_corners.json")
    s = oracle_series_from_golden(g)
    K, b = kriging.build_system(s)
    assert K.shape == (s.size, s.size)
    np.testing.assert_allclose(K, K.T, atol=1e-14)
    ng = 3 * s.n_o
    assert np.all(np.diag(K)[:ng] > 0)
    assert np.all(np.diag(K)[ng:ng + s.n_i] > 0)
    np.testing.assert_array_equal(b[:ng], s.dip_gradients.T.reshape(-1))
    assert not b[ng:].any()


def test_exact_interpolation_and_drift_orthogonality():
    g = load_golden("anticline_corners.json")
    s = oracle_series_from_golden(g)
    s.nugget_sp = np.full(s.n_p, 1e-12)
    s.nugget_grad = np.full(s.n_o, 1e-12)
    K, b = kriging.build_system(s)
    w = kriging.solve(K, b)
    z = kriging.evaluate(s, w, s.sp_coords)
    start = 0
    for n in s.points_per_surface:
        seg = z[start:start + n]
        assert np.ptp(seg) < 1e-8 * max(1.0, np.abs(seg).max())
        start += n
    # drift rows: U^T w = 0
    ng, ni = 3 * s.n_o, s.n_i
    np.testing.assert_allclose(K[ng + ni:, :ng + ni] @ w[:ng + ni], 0.0, atol=1e-10)
    # field gradient at the orientations follows the data (nugget -> 0); not
    # exactly, because the 1e-5 regulariser of h_u h_v / r^2 makes the
    # gradient block differ slightly from the kernel's exact second derivative
    _, G = kriging.evaluate(s, w, s.dip_positions, gradient=True)
    np.testing.assert_allclose(G / s.gi_res, s.dip_gradients, atol=2e-3)


def test_horizontal_inputs_give_linear_field():
    """Perfectly horizontal surfaces + vertical orientations: the co-kriging
    solution is the linear drift alone, so Z = gi_res * z exactly."""
    g = load_golden("horizontal_inputs.json")
    s = oracle_series_from_golden(g)
    K, b = kriging.build_system(s)
    w = kriging.solve(K, b)
    rng = np.random.default_rng(0)
    x = rng.uniform(-0.3, 0.3, (50, 3))
    np.testing.assert_allclose(kriging.evaluate(s, w, x), s.gi_res * x[:, 2], atol=1e-12)


@pytest.mark.parametrize("kernel", [covariance.CUBIC, covariance.EXPONENTIAL])
def test_covariance_derivatives_match_finite_differences(kernel):
    C, d1r, d2, d3r = covariance.functions(kernel)
    a = 1.3
    r = np.linspace(0.05, 1.25, 40)
    h = 1e-6
    dC = (C(r + h, a) - C(r - h, a)) / (2 * h)
    np.testing.assert_allclose(d1r(r, a) * r, dC, rtol=1e-6, atol=1e-8)
    d2n = (C(r + h, a) - 2 * C(r, a) + C(r - h, a)) / h**2
    np.testing.assert_allclose(d2(r, a), d2n, rtol=1e-3, atol=1e-3)
    g = lambda rr: d1r(rr, a)
    d3n = (g(r + h) - g(r - h)) / (2 * h) / r
    np.testing.assert_allclose(d3r(r, a), d3n, rtol=1e-5, atol=1e-6)


def test_gradient_of_field_matches_finite_differences():
    g = load_golden("anticline_corners.json")
    s = oracle_series_from_golden(g)
    w = kriging.solve(*kriging.build_system(s))
    rng = np.random.default_rng(3)
    x = rng.uniform(-0.25, 0.25, (20, 3))
    _, G = kriging.evaluate(s, w, x, gradient=True)
    h = 1e-6
    for u in range(3):
        e = np.zeros(3); e[u] = h
        fd = (kriging.evaluate(s, w, x + e) - kriging.evaluate(s, w, x - e)) / (2 * h)
        np.testing.assert_allclose(G[:, u], fd, rtol=1e-5, atol=1e-7)


def test_segmentation_step_and_order():
    iso = np.array([0.1, 0.3, -0.2])           # unsorted on purpose
    uv = np.array([1.0, 2.0, 3.0, 4.0])
    Z = np.array([0.5, 0.2, 0.0, -0.5, 0.3 + 1e-3, 0.1 - 1e-3])
    v, ids = segmentation.segment(Z, iso, uv, 5e6)
    np.testing.assert_array_equal(ids, [1, 2, 3, 4, 1, 3])
    np.testing.assert_array_equal(segmentation.hard_ids(Z, iso, uv), ids)


def test_series_masks_squeezed():
    f0 = np.array([1.0, -1.0, -1.0])
    f1 = np.array([0.0, 1.0, -1.0])
    f2 = np.array([0.0, 0.0, 0.0])
    m = segmentation.series_masks([f0, f1, f2], [np.array([0.5, 0.0]), np.array([0.2]), np.array([0.0])],
                                  [segmentation.ERODE, segmentation.ERODE, segmentation.BASEMENT])
    np.testing.assert_array_equal(m, [[1, 0, 0], [0, 1, 0], [0, 0, 1]])
    assert m.sum(0).tolist() == [1, 1, 1]


def test_octree_children_order_and_marking():
    c, d = octree.base_centres([0, 1, 0, 1, 0, 1], [2, 2, 2])
    assert c.shape == (8, 3)
    np.testing.assert_allclose(c[1], [0.25, 0.25, 0.75])   # z fastest
    ch = octree.children(c[:1], d)
    np.testing.assert_allclose(ch[0], [0.125, 0.125, 0.125])
    np.testing.assert_allclose(ch[7], [0.375, 0.375, 0.375])
    ids = np.array([[1] * 8, [1, 1, 1, 1, 1, 1, 1, 2]]).ravel()
    np.testing.assert_array_equal(octree.mark(ids), [False, True])


def _octree_levels(name):
    from oracle import inputs
    g = load_golden(name)
    series, rels, fr = inputs.series_from_golden(g)
    oc = g["octree"]
    levels = pipeline.compute_octree(series, rels, g["unit_values"], g["sigmoid_slope"], inputs.golden_extent(g),
                                     oc["base_resolution"], oc["levels"], fault_relations=fr,
                                     levels_surface=oc.get("levels_surface", 4))
    return g, series, levels


def test_fault_model_approval_file():
    """The one-fault model (examples_generator.py:198-241) against its approval
    file (test_example_models_I.py:56-68), with the reference's comparator.
    Nothing was chosen with this file: it checks the kriging conventions, the
    fault drift and the lithology + fault-block octree refinement (24624
    centres at the sixth level) independently of the anticline."""
    g, series, levels = _octree_levels("fault_model.json")
    last = levels[-1]
    assert len(last.centres) == 24624
    z = last.exported_field(0)
    sampled = z[:: len(z) // 50]
    approved = np.array(g["octree"]["approved_scalar_field_last_level"])
    assert sampled.shape == approved.shape
    assert np.allclose(sampled, approved, rtol=1e-5, atol=1e-5)
    assert np.abs(sampled - approved).max() < 4e-6


def test_fault_drift_offsets_horizontal_layers_exactly():
    """Known answer: horizontal layers (gradient (0,0,1)) displaced by a fault
    are reproduced exactly by the linear drift plus the fault-block drift, with
    zero covariance weights: Z = gi_res (z + nu F) and every surface point of a
    surface, on either side of the fault, at the same isovalue."""
    from oracle import inputs
    g = load_golden("fault_model.json")
    series, rels, fr = inputs.series_from_golden(g)
    m = pipeline.Model(series, rels, g["unit_values"], g["sigmoid_slope"], fr)
    strat = series[1]
    w = m.ws[1]
    ncov = 3 * strat.n_o + strat.n_i
    assert np.abs(w[:ncov]).max() < 1e-12
    np.testing.assert_allclose(w[ncov:ncov + 3], [0.0, 0.0, 1.0], atol=1e-12)
    z = m.field(1, strat.sp_coords)
    start = 0
    for n, iso in zip(strat.points_per_surface, m.isos[1]):
        np.testing.assert_allclose(z[start:start + n], iso, atol=1e-12)
        start += n
    # the fault block does separate the two sides of the fault
    F = strat.fault_sp[:, 0]
    x = strat.sp_coords[:, 0]
    assert set(np.unique(np.rint(F[x < 0]))) != set(np.unique(np.rint(F[x > 0])))


def test_combination_model_approval_file():
    """The combination model (examples_generator.py:244-293; four levels with
    number_octree_levels_surface 4) against its approval file
    (test_example_models_I.py:71-88) with the reference's comparator: the last
    level exports the centres' values followed by the 8 corners of every
    centre, and its 4328 voxels include the 96 that the interpolation-error
    statistic adds (children of four level-1 voxels whose corners agree)."""
    g, series, levels = _octree_levels("combination_model.json")
    assert [len(l.centres) for l in levels] == [16, 128, 776, 4328]
    last = levels[-1]
    z = last.exported_field(0)
    assert len(z) == 9 * len(last.centres)
    sampled = z[:: len(z) // 50]
    approved = np.array(g["octree"]["approved_scalar_field_last_level"])
    assert sampled.shape == approved.shape
    assert np.allclose(sampled, approved, rtol=1e-5, atol=1e-5)


def test_error_statistic_adds_nothing_where_corners_suffice():
    """Without the interpolation-error statistic the combination model's
    sampled values no longer match (the corner rule alone gives 4232 voxels),
    and on the one-fault model the statistic adds no voxel."""
    from oracle import inputs
    g = load_golden("combination_model.json")
    series, rels, fr = inputs.series_from_golden(g)
    oc = g["octree"]
    lv = pipeline.compute_octree(series, rels, g["unit_values"], g["sigmoid_slope"], inputs.golden_extent(g),
                                 oc["base_resolution"], oc["levels"], fault_relations=fr, levels_surface=4,
                                 error_threshold=0.0)
    assert len(lv[-1].centres) == 4232
    z = lv[-1].exported_field(0)
    approved = np.array(oc["approved_scalar_field_last_level"])
    assert not np.allclose(z[:: len(z) // 50], approved, rtol=1e-5, atol=1e-5)
    g = load_golden("fault_model.json")
    series, rels, fr = inputs.series_from_golden(g)
    oc = g["octree"]
    counts = [len(l.centres) for l in pipeline.compute_octree(
        series, rels, g["unit_values"], g["sigmoid_slope"], inputs.golden_extent(g), oc["base_resolution"],
        oc["levels"], fault_relations=fr, levels_surface=4, error_threshold=0.0)]
    assert counts == [8, 64, 320, 1440, 6032, 24624]


def test_interpolation_error_is_zero_for_a_linear_field():
    """A field linear over the voxel has zero interpolation error up to
    rounding, which the floor keeps from marking anything."""
    from oracle import octree
    rng = np.random.default_rng(3)
    c = rng.uniform(-1, 1, (500, 3))
    d = np.array([0.1, 0.07, 0.05])
    a = np.array([0.3, -1.2, 0.8])
    z0 = c @ a + 0.25
    zc = octree.corners(c, d) @ a + 0.25
    e = octree.interpolation_error(z0, zc)
    assert e.max() < 1e-12
    assert not octree.error_marks([z0], [zc], 1.0).any()
    zq = zc + 0.5 * (octree.corners(c, d)[:, 0] - np.repeat(c[:, 0], 8)) ** 2
    assert octree.error_marks([z0], [zq], 1.0).any() or octree.interpolation_error(z0, zq).std() == 0


def test_marching_cubes_vertex_counts_of_combination_model():
    """G4: the reference's marching-cubes vertex counts of the combination
    model on a 40 x 20 x 20 dense grid (test/test_modules/
    test_marching_cubes.py:13-47): 600 (fault), 860 (eroding series), 1256
    and 1680 (basement series), from the oracle's field, masks and isovalues
    with the mesh rule of oracle/mesh.py (cube processed when the mask is set
    at its far corner, one vertex per crossed edge of a processed cube)."""
    from oracle import inputs, mesh
    g = load_golden("combination_model.json")
    series, rels, fr = inputs.series_from_golden(g)
    ext = inputs.golden_extent(g)
    res = np.array([40, 20, 20])
    d = (ext[1::2] - ext[0::2]) / res
    axes = [ext[2 * a] + (np.arange(res[a]) + 0.5) * d[a] for a in range(3)]
    X = np.stack(np.meshgrid(*axes, indexing="ij"), -1).reshape(-1, 3)
    r = pipeline.Model(series, rels, g["unit_values"], g["sigmoid_slope"], fr).evaluate(X)
    counts = []
    for s in range(len(series)):
        mask = None if rels[s] == segmentation.FAULT else r.masks[s]
        for level in r.isovalues[s]:
            v, t = mesh.marching_cubes(r.fields[s], res, level, d, ext[0::2], mask)
            counts.append(len(v))
            assert t.min() >= 0 and t.max() < len(v)
    assert counts == [600, 860, 1256, 1680]


def test_marching_cubes_cycles_close_for_every_cube_configuration():
    """Every one of the 256 corner-sign configurations (random magnitudes, so
    both pairings of four-crossing faces occur) links its crossing edges into
    closed cycles, and a closed level surface is a consistently oriented
    sphere (Euler characteristic 2)."""
    from oracle import mesh
    rng = np.random.default_rng(0)
    for cfg in range(256):
        for _ in range(8):
            g = np.array([(1 if (cfg >> q) & 1 else -1) * rng.uniform(0.1, 1) for q in range(8)])
            n_cross = sum((g[q0] > 0) != (g[q1] > 0) for _, q0, q1 in mesh.EDGES)
            assert sum(len(c) for c in mesh.cube_cycles(g)) == n_cross
    n = 20
    ax = np.arange(n, dtype=np.float64)
    X, Y, Z = np.meshgrid(ax, ax, ax, indexing="ij")
    F = np.sqrt((X - 9.3) ** 2 + (Y - 9.9) ** 2 + (Z - 9.6) ** 2) + 0.8 * np.sin(0.9 * X) * np.cos(0.7 * Y)
    v, t = mesh.marching_cubes(F, (n, n, n), 6.0)
    e = np.concatenate([t[:, [0, 1]], t[:, [1, 2]], t[:, [2, 0]]]).astype(np.int64)
    key, rkey = e[:, 0] * len(v) + e[:, 1], e[:, 1] * len(v) + e[:, 0]
    u, c = np.unique(key, return_counts=True)
    assert (c == 1).all() and np.isin(rkey, u).all()
    assert len(v) - len(u) // 2 + len(t) == 2


def test_prism_attraction_matches_quadrature_and_kernel_tiles_its_box():
    """The closed-form prism attraction (Nagy 1966; Plouff 1976) against
    Gauss-Legendre quadrature of G z / r^3, and the centred-grid kernel of the
    reference's gravity test (resolution [10, 10, 100], radius 16000,
    test/test_modules/test_geophysics/test_gravity.py:67-72) tiling its box:
    the voxels' tz add up to the whole box's."""
    from oracle import gravity
    x, w = np.polynomial.legendre.leggauss(40)
    for box in [(-1, 2, -0.5, 1.5, -3, -1), (0.5, 1.5, 0.2, 0.9, -2, -0.7), (-2, -1, 1, 3, 0.5, 2.5)]:
        x0, x1, y0, y1, z0, z1 = box
        X, Y, Z = [(b - a) / 2 * x + (b + a) / 2 for a, b in ((x0, x1), (y0, y1), (z0, z1))]
        W = np.einsum("i,j,k->ijk", w, w, w) * (x1 - x0) * (y1 - y0) * (z1 - z0) / 8
        XX, YY, ZZ = np.meshgrid(X, Y, Z, indexing="ij")
        q = gravity.G_MGAL * (W * ZZ / np.sqrt(XX ** 2 + YY ** 2 + ZZ ** 2) ** 3).sum()
        assert abs(gravity.prism_tz(*box) - q) <= 1e-12 * abs(q)
    c, lo, hi = gravity.kernel([10, 10, 100], 16000.0)
    assert len(c) == 11 * 11 * 101
    a, b = c - lo, c + hi
    box = gravity.prism_tz(a[:, 0].min(), b[:, 0].max(), a[:, 1].min(), b[:, 1].max(), a[:, 2].min(), b[:, 2].max())
    t = gravity.tz([10, 10, 100], 16000.0)
    assert abs(t.sum() - box) <= 1e-9 * abs(box)
    assert (t < 0).all()        # every voxel lies below the device


def test_two_layer_gravity_value():
    """The reference's gravity pin (test/test_modules/test_geophysics/
    test_gravity.py:67-89): its kernel ([10, 10, 100], radius 16000, device at
    the model's top) lies wholly in the basement (density 3.2, id 3 of the two
    horizontal surfaces at z = 3.05 and 1.02), so the value is 3.2 x sum(tz);
    the reference checks it to 4 decimals.  The vertical stretch of the kernel
    decides it: without it the sum would be 10 % smaller."""
    from oracle import gravity
    c, lo, hi = gravity.kernel([10, 10, 100], 16000.0)
    assert (c[:, 2] + hi[:, 2] + 4.0 < 1.02).all()      # every voxel below the lower surface
    g = 3.2 * gravity.tz([10, 10, 100], 16000.0).sum()
    np.testing.assert_almost_equal(np.array([g]), np.array([-1624.1714]), decimal=4)


def test_centered_grid_matches_oracle_kernel():
    """The package's CenteredGrid (host set-up of the gravity grid) builds the
    oracle's kernel: same voxel centres and half-widths, device-major points."""
    from gempy_gb300.data import CenteredGrid
    from oracle import gravity
    cg = CenteredGrid(np.array([[6.0, 0.0, 4.0], [1.0, 2.0, 3.0]]), [10, 10, 100], [16000.0, 8000.0, 16000.0])
    c, lo, hi = gravity.kernel([10, 10, 100], [16000.0, 8000.0, 16000.0])
    np.testing.assert_array_equal(cg.kernel_grid_centers, c)
    np.testing.assert_array_equal(cg.left_voxel_edges, lo)
    np.testing.assert_array_equal(cg.right_voxel_edges, hi)
    np.testing.assert_array_equal(cg.values, gravity.points(cg.centers, [10, 10, 100], [16000.0, 8000.0, 16000.0]))


def test_engine_refine_modes_follow_the_oracle(monkeypatch):
    """The engine's choice of refinement per octree level (gk_octree_level's
    ``refine``: 0 last, 2 all, 3 corners + error statistic, 1 corners) is the
    oracle's: the levels where the oracle applies its error statistic are
    exactly those where the engine asks for mode 3."""
    from gempy_gb300.engine import octree_refine_mode
    from oracle import inputs, octree
    g = load_golden("anticline_corners.json")
    series, rels, fr = inputs.series_from_golden(g)
    ext = inputs.golden_extent(g)
    for n_levels, min_level, ls, t in [(4, 2, 4, 1.0), (4, 2, 4, 0.0), (4, 1, 4, 1.0), (4, 2, 5, 1.0),
                                       (3, 2, 2, 1.0), (4, 3, 6, 2.0)]:
        called = []
        real = octree.error_marks

        def spy(centre_fields, corner_fields, n_std):
            called.append(len(np.asarray(centre_fields[0])))
            return real(centre_fields, corner_fields, n_std)
        monkeypatch.setattr(octree, "error_marks", spy)
        lv = pipeline.compute_octree(series, rels, g["unit_values"], g["sigmoid_slope"], ext, [2, 2, 2], n_levels,
                                     min_level=min_level, fault_relations=fr, levels_surface=ls, error_threshold=t)
        monkeypatch.setattr(octree, "error_marks", real)
        sizes = [len(l.centres) for l in lv]
        modes = [octree_refine_mode(L, n_levels, min_level, ls, t) for L in range(len(lv))]
        assert modes[-1] == 0
        assert [sizes[L] for L, m in enumerate(modes) if m == 3] == called
        assert all(m == 2 for L, m in enumerate(modes) if L + 1 < min_level and L < n_levels - 1)


def test_field_pool_matches_serial_evaluation():
    """The CPU baseline's worker pool (oracle/parallel.py) returns the serial
    evaluation's field bit for bit, in point order."""
    from oracle.parallel import FieldPool
    g = load_golden("anticline_corners.json")
    s = oracle_series_from_golden(g)
    w = kriging.solve(*kriging.build_system(s))
    x = np.random.default_rng(5).uniform(-0.3, 0.3, (5000, 3))
    with FieldPool(s, 2) as pool:
        z = pool.evaluate(x, w)
    np.testing.assert_array_equal(z, kriging.evaluate(s, w, x))
