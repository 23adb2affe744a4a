"""GPU parity tests: every kernel against the FP64 oracle through the C ABI.

Tolerances (written here, used by the check of each test):
  * FP64 build: |K_gpu - K_oracle| <= 1e-13 max|K|
  * FP64 LU/solve: ||b - K x||_inf <= 50 n eps ||K||_inf ||x||_inf (normwise
    backward error of a stable LU), x vs LAPACK <= 1e-8 relative
  * FP64 field/gradient: max|dZ| / max|Z| <= 1e-9
  * FP32 (mixed) field: max|dZ| / max|Z| <= 1e-6; weights from the mixed solve
    <= 1e-6 relative to the FP64 solve
  * ids: identical outside the band |Z - z_k| <= band around each isovalue
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import kriging, octree, pipeline, segmentation  # noqa: E402
from tests._models import (engine_inputs_from_golden, golden_extent, load_golden,  # noqa: E402
                           oracle_series_from_golden, oracle_series_list)

pytestmark = pytest.mark.gpu


def _dev_series(s, device="cuda"):
    from gempy_gb300 import kernels as K
    return K.DeviceSeries(s.dip_positions, s.dip_gradients, s.nugget_grad, s.sp_coords, s.nugget_sp,
                          s.points_per_surface, range=s.range, c_o=s.c_o, uni_degree=s.uni_degree,
                          kernel=s.kernel, i_res=s.i_res, gi_res=s.gi_res, device=device)


def _random_series(seed, n_surf=3, per=12, n_o=7, degree=1, kernel="cubic", a=0.9):
    rng = np.random.default_rng(seed)
    pts = []
    for k in range(n_surf):
        xy = rng.uniform(-0.4, 0.4, (per, 2))
        z = -0.3 + 0.3 * k + 0.05 * np.sin(4 * xy[:, 0])
        pts.append(np.column_stack([xy, z]))
    sp = np.concatenate(pts)
    xo = rng.uniform(-0.4, 0.4, (n_o, 3))
    g = rng.normal(0, 0.1, (n_o, 3)) + [0, 0, 1]
    g /= np.linalg.norm(g, axis=1, keepdims=True)
    return kriging.Series(xo, g, np.full(n_o, 0.01), sp, np.full(len(sp), 2e-5), np.full(n_surf, per),
                          range=a, c_o=a * a / 14 / 3, uni_degree=degree, kernel=kernel)


def _anticline():
    return oracle_series_from_golden(load_golden("anticline_corners.json"))


SERIES_CASES = {
    "anticline": _anticline,
    "random_deg1_cubic": lambda: _random_series(1),
    "random_deg2_cubic": lambda: _random_series(2, degree=2),
    "random_deg0_exp": lambda: _random_series(3, degree=0, kernel="exponential", a=0.5),
    "random_deg2_exp": lambda: _random_series(4, degree=2, kernel="exponential", a=0.7),
    "one_point_pair": lambda: _random_series(5, n_surf=1, per=2, n_o=1),
}


@pytest.mark.parametrize("case", list(SERIES_CASES))
def test_build_f64_matches_oracle(case):
    from gempy_gb300 import kernels as K
    s = SERIES_CASES[case]()
    Kr, br = kriging.build_system(s)
    ds = _dev_series(s)
    Kg, bg = K.build(ds, K.GK_F64)
    N = Kr.shape[0]
    Kg = Kg[:, :N].cpu().numpy()
    assert np.abs(Kg - Kr).max() <= 1e-13 * np.abs(Kr).max()
    np.testing.assert_array_equal(bg.cpu().numpy(), br)


@pytest.mark.parametrize("case", list(SERIES_CASES))
def test_build_tables_match_direct_build(case):
    """The table-driven FP64 build (gk_build_tables, the default) and the
    direct build (gk_build) give the same matrix to rounding: the interface
    entries come from the same covariances, formed once."""
    from gempy_gb300 import kernels as K
    s = SERIES_CASES[case]()
    ds = _dev_series(s)
    Kt, bt = K.build(ds, K.GK_F64, tables=True)
    Kd, bd = K.build(ds, K.GK_F64, tables=False)
    N = ds.N
    a, b = Kt[:, :N].cpu().numpy(), Kd[:, :N].cpu().numpy()
    assert np.abs(a - b).max() <= 1e-14 * np.abs(b).max()
    np.testing.assert_array_equal(bt.cpu().numpy(), bd.cpu().numpy())


def test_build_f32_matches_oracle():
    from gempy_gb300 import kernels as K
    s = _anticline()
    Kr, _ = kriging.build_system(s)
    Kg, _ = K.build(_dev_series(s), K.GK_F32)
    N = Kr.shape[0]
    assert np.abs(Kg[:, :N].double().cpu().numpy() - Kr).max() <= 2e-6 * np.abs(Kr).max()


@pytest.mark.parametrize("panel", ["cluster", "cooperative"])
@pytest.mark.parametrize("n", [1, 2, 5, 31, 32, 33, 63, 64, 65, 127, 200, 513, 1100])
@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_lu_factor_solve_random(n, prec, panel, monkeypatch):
    from gempy_gb300 import kernels as K
    if panel == "cooperative":
        monkeypatch.setenv("GK_PANEL_COOPERATIVE", "1")
    rng = np.random.default_rng(n)
    A = rng.normal(size=(n, n)) + n ** 0.5 * np.eye(n) * rng.choice([-1, 1], n)
    b = rng.normal(size=n)
    dt = torch.float64 if prec == "f64" else torch.float32
    ld = K.leading_dim(n, K.GK_F64 if prec == "f64" else K.GK_F32)
    At = torch.zeros((n, ld), dtype=dt, device="cuda")
    At[:, :n] = torch.as_tensor(A, dtype=dt)
    f = K.lu_factor(At)
    x = K.lu_solve(f, torch.as_tensor(b, dtype=dt, device="cuda")).double().cpu().numpy()
    info = K.read_info(f.info)
    assert info["status"] == 0
    res = np.abs(b - A @ x).max() / (np.abs(A).max() * np.abs(x).max() * n)
    assert res < (1e-15 if prec == "f64" else 1e-6)
    # pivots agree with LAPACK's partial pivoting on distinct-magnitude columns
    if prec == "f64":
        import scipy.linalg
        _, piv = scipy.linalg.lu_factor(A)
        np.testing.assert_array_equal(f.ipiv.cpu().numpy(), piv)


@pytest.mark.parametrize("case", ["anticline", "random_deg2_cubic", "random_deg2_exp"])
def test_plain_solve_matches_lapack(case):
    from gempy_gb300 import kernels as K
    s = SERIES_CASES[case]()
    Kr, br = kriging.build_system(s)
    w_ref = kriging.solve(Kr, br)
    w, info = K.solve_plain(_dev_series(s))
    w = w.cpu().numpy()
    assert K.read_info(info)["status"] == 0
    # normwise backward error of a stable LU: ||b - K x|| <= c n eps ||K|| ||x||
    n = len(br)
    bound = 50 * n * np.finfo(float).eps * np.abs(Kr).sum(1).max() * np.abs(w).max()
    assert np.abs(br - Kr @ w).max() <= bound
    assert np.abs(w - w_ref).max() <= 1e-8 * np.abs(w_ref).max()


@pytest.mark.parametrize("case", ["anticline", "random_deg1_cubic", "random_deg2_exp"])
def test_mixed_solve_reaches_fp64_residual(case):
    from gempy_gb300 import kernels as K
    s = SERIES_CASES[case]()
    Kr, br = kriging.build_system(s)
    w_ref = kriging.solve(Kr, br)
    w, info = K.solve_mixed(_dev_series(s), tol=1e-12)
    inf = K.read_info(info)
    w = w.cpu().numpy()
    assert inf["residual"] <= 1e-11, inf
    assert np.linalg.norm(br - Kr @ w) <= 1e-11 * np.linalg.norm(br)
    assert np.abs(w - w_ref).max() <= 1e-6 * np.abs(w_ref).max()


@pytest.mark.parametrize("per,n_o", [(4, 2), (30, 12), (52, 22), (52, 23), (150, 60)])
def test_cta_mixed_solve_matches_lapack(per, n_o):
    """The one-block mixed solve on both preconditioner forms: systems up to
    224 unknowns invert their equilibrated FP32 matrix in shared memory,
    larger ones factor it in global memory.  Here N = 3 (per + n_o): 18, 126,
    222 (shared), 225, 630 (global).  Single and many-system entries agree
    with LAPACK to the FGMRES tolerance."""
    from gempy_gb300 import kernels as K
    s = _random_series(per + n_o, n_surf=3, per=per, n_o=n_o)
    Kr, br = kriging.build_system(s)
    N = len(br)
    w_ref = kriging.solve(Kr, br)
    ds = _dev_series(s)
    x, info = K.solve_mixed_cta(ds, tol=1e-12)
    inf = K.read_info(info)
    assert inf["status"] == 0 and inf["residual"] <= 1e-12, (N, inf)
    x = x.cpu().numpy()
    assert np.linalg.norm(br - Kr @ x) <= 1e-11 * np.linalg.norm(br)
    assert np.abs(x - w_ref).max() <= 1e-6 * np.abs(w_ref).max()
    # one launch over systems of different sizes: the largest decides the form
    small = _random_series(7, n_surf=2, per=5, n_o=3)
    Ks, bs = K.build(_dev_series(small), K.GK_F64)
    Kb, bb = K.build(ds, K.GK_F64)
    (xs, i_s), (xb, i_b) = K.solve_mixed_cta_many([(Ks, bs), (Kb, bb)], tol=1e-12)
    assert K.read_info(i_s)["status"] == 0 and K.read_info(i_b)["status"] == 0
    np.testing.assert_allclose(xb.cpu().numpy(), x, rtol=0, atol=1e-9 * np.abs(x).max())
    Kr2, br2 = kriging.build_system(small)
    assert np.linalg.norm(br2 - Kr2 @ xs.cpu().numpy()) <= 1e-11 * np.linalg.norm(br2)


def _eval_gpu(s, w, x, prec, gradient=False, seg=None):
    from gempy_gb300 import kernels as K
    ds = _dev_series(s)
    wt = torch.as_tensor(w, device="cuda")
    model = K.prepare(ds, wt)
    pts = K.Points(xyz=torch.as_tensor(x, device="cuda"))
    f, g, v, ids = K.evaluate(ds, model, pts, prec, seg=seg, gradient=gradient, want_ids=seg is not None)
    out = [f.cpu().numpy()]
    if gradient:
        out.append(g.cpu().numpy())
    if seg is not None:
        out += [v.cpu().numpy(), ids.cpu().numpy()]
    return out


@pytest.mark.parametrize("case", list(SERIES_CASES))
def test_eval_f64_field_and_gradient_match_oracle(case):
    from gempy_gb300 import kernels as K
    s = SERIES_CASES[case]()
    w = kriging.solve(*kriging.build_system(s))
    rng = np.random.default_rng(7)
    x = rng.uniform(-0.45, 0.45, (3000, 3))
    k = min(5, s.n_p)
    x[:k] = s.sp_coords[:k]          # exactly on data points (r = 0)
    x[k:k + min(2, s.n_o)] = s.dip_positions[:2]
    Zr, Gr = kriging.evaluate(s, w, x, gradient=True)
    Z, G = _eval_gpu(s, w, x, K.GK_F64, gradient=True)
    assert np.abs(Z - Zr).max() <= 1e-9 * np.abs(Zr).max()
    assert np.abs(G - Gr).max() <= 1e-9 * np.abs(Gr).max()


@pytest.mark.parametrize("case", ["anticline", "random_deg1_cubic", "random_deg2_cubic", "one_point_pair"])
def test_eval_ff_field_within_1e9(case):
    """Float-float evaluation (the mixed form's field kernel) vs FP64 oracle."""
    from gempy_gb300 import kernels as K
    s = SERIES_CASES[case]()
    w = kriging.solve(*kriging.build_system(s))
    rng = np.random.default_rng(8)
    x = rng.uniform(-0.45, 0.45, (20000, 3))
    x[: min(5, s.n_p)] = s.sp_coords[:5]
    x[-1] = [40.0, -30.0, 55.0]        # far outside the data: exact two-sum path, beyond range
    Zr = kriging.evaluate(s, w, x)
    (Z,) = _eval_gpu(s, w, x, K.GK_FF)
    assert np.abs(Z - Zr).max() <= 1e-9 * np.abs(Zr).max()


def test_eval_ff_precision_workload_subsample():
    """The 4000-point / 1500-orientation series, whose kriging sum cancels by a
    factor ~3e4: float-float stays within 1e-9, plain FP32 does not reach 1e-6."""
    from gempy_gb300 import kernels as K
    from gempy_gb300 import synthetic
    m = synthetic.precision(resolution=(8, 8, 8))
    (s,) = oracle_series_list(m)
    w = kriging.solve(*kriging.build_system(s))
    rng = np.random.default_rng(9)
    x = rng.uniform(-0.5, 0.5, (4096, 3))
    Zr = kriging.evaluate(s, w, x)
    (Zff,) = _eval_gpu(s, w, x, K.GK_FF)
    (Z32,) = _eval_gpu(s, w, x, K.GK_F32)
    e_ff = np.abs(Zff - Zr).max() / np.abs(Zr).max()
    e_32 = np.abs(Z32 - Zr).max() / np.abs(Zr).max()
    assert e_ff <= 1e-9
    assert e_32 > 1e-6   # documents why the mixed form evaluates in float-float


@pytest.mark.parametrize("n", [1, 5, 257, 3000, 20000])
def test_eval_record_split_small_point_sets(n):
    """Point sets too small to fill the GPU share each chunk of points among
    the CTAs of a cluster (records split, partials added in rank order): every
    precision still matches the oracle, and two runs agree bit for bit.  The
    series has 5500 records, enough for every split size."""
    from gempy_gb300 import kernels as K
    from gempy_gb300 import synthetic
    m = synthetic.precision(resolution=(8, 8, 8))
    (s,) = oracle_series_list(m)
    w = kriging.solve(*kriging.build_system(s))
    rng = np.random.default_rng(n)
    x = rng.uniform(-0.5, 0.5, (n, 3))
    x[0] = s.sp_coords[0]
    Zr, Gr = kriging.evaluate(s, w, x, gradient=True)
    scale_z, scale_g = np.abs(Zr).max(), np.abs(Gr).max()
    Z, G = _eval_gpu(s, w, x, K.GK_F64, gradient=True)
    assert np.abs(Z - Zr).max() <= 1e-9 * scale_z
    assert np.abs(G - Gr).max() <= 1e-9 * scale_g
    (Z64,) = _eval_gpu(s, w, x, K.GK_F64)
    assert np.abs(Z64 - Zr).max() <= 1e-9 * scale_z
    (Zff,) = _eval_gpu(s, w, x, K.GK_FF)
    assert np.abs(Zff - Zr).max() <= 1e-9 * scale_z
    (Zff2,) = _eval_gpu(s, w, x, K.GK_FF)
    np.testing.assert_array_equal(Zff, Zff2)
    alpha = kriging.point_coefficients(s, w)
    cancel = (s.c_o * s.gi_res * (np.abs(alpha).sum() + np.abs(w[:3 * s.n_o]).sum() * 14 / s.range) / scale_z)
    Z32, G32 = _eval_gpu(s, w, x, K.GK_F32, gradient=True)
    assert np.abs(Z32 - Zr).max() <= 1e-6 * cancel * scale_z
    (Z32n,) = _eval_gpu(s, w, x, K.GK_F32)
    assert np.abs(Z32n - Zr).max() <= 1e-6 * cancel * scale_z


@pytest.mark.parametrize("case", ["anticline", "random_deg2_cubic", "random_deg0_exp"])
def test_eval_f32_field_and_gradient_bounded(case):
    """Plain FP32 evaluation: accurate to ~1e-7 times the cancellation factor."""
    from gempy_gb300 import kernels as K
    s = SERIES_CASES[case]()
    w = kriging.solve(*kriging.build_system(s))
    rng = np.random.default_rng(8)
    x = rng.uniform(-0.45, 0.45, (20000, 3))
    Zr, Gr = kriging.evaluate(s, w, x, gradient=True)
    Z, G = _eval_gpu(s, w, x, K.GK_F32, gradient=True)
    alpha = kriging.point_coefficients(s, w)
    cancel = (s.c_o * s.gi_res * (np.abs(alpha).sum() + np.abs(w[:3 * s.n_o]).sum() * 14 / s.range)
              / np.abs(Zr).max())
    assert np.abs(Z - Zr).max() <= 1e-6 * cancel * np.abs(Zr).max()
    assert np.abs(G - Gr).max() <= 1e-5 * cancel * np.abs(Gr).max()


@pytest.mark.parametrize("prec", ["f64", "ff", "f32"])
def test_regular_grid_segmentation_ids(prec):
    """50^3 dense grid of the plain configuration: field vs oracle and ids
    identical outside the isovalue band."""
    from gempy_gb300 import kernels as K
    from gempy_gb300 import synthetic
    m = synthetic.plain_horizontal()
    (s,) = oracle_series_list(m)
    w = kriging.solve(*kriging.build_system(s))
    iso = kriging.isovalues(s, w)
    grid = m.interpolation_input.grid.dense_grid
    x = grid.values
    Zr = kriging.evaluate(s, w, x)
    uv = m.interpolation_input.unit_values
    vr, idr = segmentation.segment(Zr, iso, uv, m.options.sigmoid_slope)
    ds = _dev_series(s)
    model = K.prepare(ds, torch.as_tensor(w, device="cuda"))
    order = segmentation.order_surfaces(iso)
    seg = K.make_segment(iso[order], uv, m.options.sigmoid_slope)
    p = {"f64": K.GK_F64, "ff": K.GK_FF, "f32": K.GK_F32}[prec]
    f, _, v, ids = K.evaluate(ds, model, K.Points.regular(grid), p, seg=seg, want_ids=True)
    Z = f.cpu().numpy()
    tol = {"f64": 1e-9, "ff": 1e-9, "f32": 1e-4}[prec]
    err = np.abs(Z - Zr).max() / np.abs(Zr).max()
    assert err <= tol
    band = max(10.0 / m.options.sigmoid_slope, 4 * err * np.abs(Zr).max())
    outside = np.all(np.abs(Zr[:, None] - iso[None, :]) > band, axis=1)
    assert outside.mean() > 0.99
    np.testing.assert_array_equal(ids.cpu().numpy()[outside], idr[outside].astype(np.int32))
    if prec == "f64":
        np.testing.assert_allclose(v.cpu().numpy(), vr, atol=1e-9)


def test_octree_refinement_matches_oracle():
    from gempy_gb300 import kernels as K
    c, d = octree.base_centres([-0.5, 0.5, -0.5, 0.5, -0.5, 0.5], [2, 3, 2])
    ct = torch.as_tensor(c, device="cuda")
    corners = K.octree_corners(ct, d).cpu().numpy()
    np.testing.assert_array_equal(corners, octree.corners(c, d))
    rng = np.random.default_rng(0)
    ids = rng.integers(1, 3, (len(c), 8)).astype(np.int32)
    ids[::3] = 1                                   # some voxels unmarked
    ch = K.octree_refine(ct, torch.as_tensor(ids.ravel(), device="cuda"), d).cpu().numpy()
    np.testing.assert_array_equal(ch, octree.children(c[octree.mark(ids.ravel())], d))
    ch_all = K.octree_refine(ct, None, d, refine_all=True).cpu().numpy()
    np.testing.assert_array_equal(ch_all, octree.children(c, d))


def _compute_anticline(levels, dtype="float64"):
    import __graft_entry__ as ge
    import gempy_gb300 as gg
    g, ii, opts, dd, ext = ge._anticline_model(levels=levels)
    return g, ext, gg.compute_model(ii, opts, dd, config=gg.EngineConfig(dtype=dtype))


def test_compute_model_anticline_pins():
    """Reference known answers through compute_model: cube-corner ids
    (test_custom_grid.py:44-47) and the approved finest-level scalar field
    (test_example_models_I.py:41-53), plus octree parity with the oracle."""
    g, ext, sol = _compute_anticline(5)
    np.testing.assert_array_equal(sol.raw_arrays.custom, np.array(g["expected_ids"], float))
    z = sol.octrees_output[-1].outputs[0].scalar_field
    approved = np.array(g["octree"]["approved_scalar_field_last_level"])
    assert len(z) == 7808
    # the reference's comparator (test/verify_helper.py:70-103)
    assert np.allclose(z[:: len(z) // 50], approved, rtol=1e-5, atol=1e-5)
    s = oracle_series_from_golden(g)
    lv = pipeline.compute_octree([s], [segmentation.BASEMENT], g["unit_values"], g["sigmoid_slope"], ext,
                                 [2, 2, 2], 5, levels_surface=4)
    _assert_levels_match(sol, lv, 1)


def _assert_levels_match(sol, lv, n_series, tol=1e-9):
    """Octree levels of compute_model against the oracle's: identical centres,
    exported fields (centres, then corners on surface levels) within ``tol``
    of max|Z|, identical lithology ids and squeezed masks."""
    assert len(sol.octrees_output) == len(lv)
    for L, ol in zip(lv, sol.octrees_output):
        np.testing.assert_array_equal(ol.grid_centers, L.centres)
        for i in range(n_series):
            zr = L.exported_field(i)
            z = ol.outputs[i].scalar_field
            assert z.shape == zr.shape
            assert np.abs(z - zr).max() <= tol * np.abs(zr).max()
        np.testing.assert_array_equal(ol.last_output_center.ids_block, L.result.ids.astype(np.int32))
        np.testing.assert_array_equal(ol.last_output_center.mask_matrix.astype(bool), L.result.masks)


def test_compute_model_mixed_anticline():
    g, ext, sol = _compute_anticline(4, dtype="float32")
    np.testing.assert_array_equal(sol.raw_arrays.custom, np.array(g["expected_ids"], float))
    _, _, ref = _compute_anticline(4, dtype="float64")
    for a, b in zip(sol.octrees_output, ref.octrees_output):
        np.testing.assert_array_equal(a.grid_centers, b.grid_centers)
        zb = b.outputs[0].scalar_field
        assert np.abs(a.outputs[0].scalar_field - zb).max() <= 1e-6 * np.abs(zb).max()
    assert sol.solver_info[0]["residual"] <= 1e-11


def test_compute_model_three_series_octree_matches_oracle():
    """Three folded series (ERODE, ERODE, BASEMENT), quadratic drift, octree."""
    import gempy_gb300 as gg
    from gempy_gb300 import synthetic
    m = synthetic.folded_series(octree_levels=4)
    sol = gg.compute_model(m.interpolation_input, m.options, m.data_descriptor)
    ss = oracle_series_list(m)
    og = m.interpolation_input.grid.octree_grid
    rel = [int(r) for r in m.data_descriptor.stack_structure.masking_descriptor]
    lv = pipeline.compute_octree(ss, rel, m.interpolation_input.unit_values, m.options.sigmoid_slope,
                                 og.orthogonal_extent, og.regular_grid_shape, 4, levels_surface=4)
    _assert_levels_match(sol, lv, len(ss))
    _, isos = pipeline.solve_all(ss)
    iso_ref = np.concatenate(isos)
    np.testing.assert_allclose(sol.scalar_field_at_surface_points, iso_ref, rtol=1e-9, atol=0)


def _golden_octree(name, dtype="float64", error_threshold=1.0):
    import gempy_gb300 as gg
    from oracle import inputs
    g = load_golden(name)
    ii, opts, dd, ext = engine_inputs_from_golden(g)
    opts.evaluation_options.octree_error_threshold = error_threshold
    sol = gg.compute_model(ii, opts, dd, config=gg.EngineConfig(dtype=dtype))
    series, rels, fr = inputs.series_from_golden(g)
    oc = g["octree"]
    lv = pipeline.compute_octree(series, rels, g["unit_values"], g["sigmoid_slope"], ext, oc["base_resolution"],
                                 oc["levels"], fault_relations=fr, levels_surface=oc.get("levels_surface", 4),
                                 error_threshold=error_threshold)
    return g, sol, lv, series


def test_compute_model_fault_model_pins():
    """The one-fault model through compute_model: the reference's approval
    file (test_example_models_I.py:56-68) under its own comparator, and every
    octree level against the oracle (centres, fields of both series, lithology
    ids, masks) -- the fault's block drives the strata's fault drift and the
    refinement."""
    g, sol, lv, series = _golden_octree("fault_model.json")
    z = sol.octrees_output[-1].outputs[0].scalar_field
    assert len(z) == 24624
    approved = np.array(g["octree"]["approved_scalar_field_last_level"])
    assert np.allclose(z[:: len(z) // 50], approved, rtol=1e-5, atol=1e-5)
    _assert_levels_match(sol, lv, len(series))
    from oracle import inputs
    series, rels, fr = inputs.series_from_golden(g)
    m = pipeline.Model(series, rels, g["unit_values"], g["sigmoid_slope"], fr)
    np.testing.assert_allclose(sol.scalar_field_at_surface_points, np.concatenate(m.isos), rtol=1e-9, atol=1e-12)


@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_compute_model_keep_on_device_matches_host_outputs(dtype):
    """The device-resident result (torch tensors) and the host result (numpy
    views of the staged copies) hold the same arrays, level by level."""
    import gempy_gb300 as gg
    g = load_golden("fault_model.json")
    ii, opts, dd, ext = engine_inputs_from_golden(g)
    host = gg.compute_model(ii, opts, dd, config=gg.EngineConfig(dtype=dtype))
    dev = gg.compute_model(ii, opts, dd, config=gg.EngineConfig(dtype=dtype, keep_on_device=True))
    assert len(host.octrees_output) == len(dev.octrees_output) == g["octree"]["levels"]

    def same(a, b):
        if a is None or b is None:
            assert a is None and b is None
            return
        assert isinstance(a, np.ndarray) and isinstance(b, torch.Tensor)
        np.testing.assert_array_equal(a, b.cpu().numpy())

    for lh, ld in zip(host.octrees_output, dev.octrees_output):
        same(lh.grid_centers, ld.grid_centers)
        same(lh.grid_corners, ld.grid_corners)
        for oh, od in zip(lh.outputs, ld.outputs):
            same(oh.exported_fields.scalar_field, od.exported_fields.scalar_field)
            same(oh.values_block, od.values_block)
            same(oh.mask, od.mask)
        for ch, cd in [(lh.last_output_center, ld.last_output_center),
                       (lh.last_output_corners, ld.last_output_corners)]:
            if ch is None:
                assert cd is None
                continue
            same(ch.block, cd.block)
            same(ch.ids_block, cd.ids_block)
            same(ch.mask_matrix, cd.mask_matrix)


def test_compute_model_combination_model_pins():
    """Fault + eroding unconformity + folded strata (three series, the fault
    offsetting both): the reference's approval file (test_example_models_I.py:
    71-88) under its own comparator -- which needs the interpolation-error
    refinement (4328 voxels at the last level, 4232 by the corners alone) --
    and every octree level of compute_model against the oracle, including the
    corner values the surface levels export."""
    g, sol, lv, series = _golden_octree("combination_model.json")
    assert [len(o.grid_centers) for o in sol.octrees_output] == [16, 128, 776, 4328]
    z = sol.octrees_output[-1].outputs[0].scalar_field
    assert len(z) == 9 * len(sol.octrees_output[-1].grid_centers)
    approved = np.array(g["octree"]["approved_scalar_field_last_level"])
    assert np.allclose(z[:: len(z) // 50], approved, rtol=1e-5, atol=1e-5)
    _assert_levels_match(sol, lv, len(series))


def test_compute_model_error_refinement_off_matches_oracle():
    """octree_error_threshold <= 0 switches the interpolation-error test off:
    the corner rule alone, on the GPU and in the oracle."""
    g, sol, lv, series = _golden_octree("combination_model.json", error_threshold=0.0)
    assert len(sol.octrees_output[-1].grid_centers) == 4232
    _assert_levels_match(sol, lv, len(series))


def test_compute_model_fault_model_mixed_matches_plain():
    """The mixed form on the fault model: the same octree and ids as the FP64
    form, fields within 1e-7 of it."""
    _, mixed, _, _ = _golden_octree("fault_model.json", dtype="float32")
    _, plain, _, _ = _golden_octree("fault_model.json", dtype="float64")
    for a, b in zip(mixed.octrees_output, plain.octrees_output):
        np.testing.assert_array_equal(a.grid_centers, b.grid_centers)
        np.testing.assert_array_equal(a.last_output_center.ids_block, b.last_output_center.ids_block)
        for i in range(2):
            zb = b.outputs[i].scalar_field
            assert np.abs(a.outputs[i].scalar_field - zb).max() <= 1e-7 * np.abs(zb).max()


def test_compute_model_onlap_series_matches_oracle():
    """An ONLAP series over an eroding one over the basement series: masks,
    ids and fields against the oracle (segmentation.series_masks)."""
    import gempy_gb300 as gg
    from gempy_gb300 import synthetic
    m = synthetic.folded_series(octree_levels=3)
    ss = m.data_descriptor.stack_structure
    rel = list(ss.masking_descriptor)
    rel[0] = gg.StackRelationType.ONLAP
    ss.masking_descriptor = rel
    sol = gg.compute_model(m.interpolation_input, m.options, m.data_descriptor)
    series = oracle_series_list(m)
    og = m.interpolation_input.grid.octree_grid
    lv = pipeline.compute_octree(series, [int(r) for r in rel], m.interpolation_input.unit_values,
                                 m.options.sigmoid_slope, og.orthogonal_extent, og.regular_grid_shape, 3,
                                 levels_surface=4)
    _assert_levels_match(sol, lv, len(series))
    masks = sol.octrees_output[-1].last_output_center.mask_matrix.astype(bool)
    assert masks[0].any() and masks[1].any() and masks[2].any()


def test_nan_input_reports_status_without_fault():
    from gempy_gb300 import kernels as K
    s = _random_series(11)
    s.dip_positions = s.dip_positions.copy()
    s.dip_positions[0, 0] = np.nan
    w, info = K.solve_plain(_dev_series(s))
    torch.cuda.synchronize()
    assert K.read_info(info)["status"] in (4, 6)   # SINGULAR or NONFINITE reported, GPU still usable
    x = torch.ones(4, device="cuda")
    assert float(x.sum()) == 4.0


def test_bad_arguments_raise():
    from gempy_gb300 import _lib
    from gempy_gb300 import kernels as K
    s = _random_series(12)
    ds = _dev_series(s)
    ds.sys.uni_degree = 7
    with pytest.raises(_lib.GkError):
        K.build(ds)


def _mixed_solve_raw(A, b):
    from gempy_gb300 import _lib
    from gempy_gb300 import kernels as K
    import ctypes
    lib = _lib.load()
    n = A.shape[0]
    ld = K.leading_dim(n, K.GK_F64)
    Kt = torch.zeros((n, ld), dtype=torch.float64, device="cuda")
    Kt[:, :n] = torch.as_tensor(A)
    bt = torch.as_tensor(b, device="cuda")
    x = torch.empty(n, dtype=torch.float64, device="cuda")
    wb = lib.gk_solve_mixed_workspace_bytes(n)
    work = torch.empty(wb, dtype=torch.uint8, device="cuda")
    info = K.new_info("cuda")
    _lib.check("gk_solve_mixed", lib.gk_solve_mixed(n, K._ptr(Kt), ld, K._ptr(bt), K._ptr(x), 1e-12, 60,
                                                    K._ptr(work), wb, K._ptr(info), K._stream()))
    return x.cpu().numpy(), K.read_info(info)


def test_mixed_solve_falls_back_to_pivoting_on_zero_pivot():
    rng = np.random.default_rng(21)
    n = 300
    A = rng.normal(size=(n, n)) + 30 * np.eye(n)
    A[0, 0] = 0.0                       # the unpivoted factorization breaks down at once
    b = rng.normal(size=n)
    x, info = _mixed_solve_raw(A, b)
    assert info["pivoted"] == 1
    assert info["status"] == 0
    assert np.linalg.norm(b - A @ x) <= 1e-11 * np.linalg.norm(b)


def test_mixed_solve_without_pivoting_on_kriging_matrix():
    s = _anticline()
    Kr, br = kriging.build_system(s)
    x, info = _mixed_solve_raw(Kr, br)
    assert info["pivoted"] == 0
    assert np.linalg.norm(br - Kr @ x) <= 1e-11 * np.linalg.norm(br)


@pytest.mark.parametrize("n_land,block,prec,policy", [(256, 64, 1, "random"), (512, 128, 1, "stratified"),
                                                      (1024, 256, 1, "random"), (256, 64, 0, "stratified"),
                                                      (1024, 256, 0, "random"), (256, 64, 2, "stratified"),
                                                      (512, 128, 2, "random")])
def test_twolevel_fgmres_checked_against_fp64_lu(n_land, block, prec, policy):
    """Block-Jacobi + low-rank preconditioned FGMRES reaches 1e-8; the FP64 LU
    (plain form) is the reference for the solution."""
    from gempy_gb300 import kernels as K
    from gempy_gb300 import synthetic
    m = synthetic.learned(n_points=1500, n_orient=400, n_surf=5)
    (s,) = oracle_series_list(m)
    ds = _dev_series(s)
    Kt, bt = K.build(ds, K.GK_F64)
    x, info, r = K.solve_twolevel(ds, n_landmarks=n_land, block=block, tol=1e-8, K=Kt, b=bt, prec=prec,
                                  policy=policy)
    inf = K.read_info(info)
    assert inf["status"] == 0, inf
    assert inf["residual"] <= 1e-8
    w_lu, _ = K.solve_plain(ds)
    x, w_lu = x.cpu().numpy(), w_lu.cpu().numpy()
    Kr, br = kriging.build_system(s)
    assert np.linalg.norm(br - Kr @ x) <= 1.01e-8 * np.linalg.norm(br)
    # the check: fields from both weight vectors agree
    pts = np.random.default_rng(0).uniform(-0.45, 0.45, (2000, 3))
    z_tl, z_lu = kriging.evaluate(s, x, pts), kriging.evaluate(s, w_lu, pts)
    assert np.abs(z_tl - z_lu).max() <= 1e-4 * np.abs(z_lu).max()


def test_condition_number_matches_oracle():
    """compute_condition_number: kappa_2(K) estimated on the GPU (power and
    inverse iteration with the FP64 LU) against numpy's SVD-based cond."""
    import gempy_gb300 as gg
    from gempy_gb300 import kernels as K
    s = _anticline()
    Kr, _ = kriging.build_system(s)
    ref = np.linalg.cond(Kr)
    Kt, _ = K.build(_dev_series(s), K.GK_F64)
    est = K.condition_number(Kt, iters=300)
    assert abs(est - ref) <= 0.02 * ref, (est, ref)
    # through compute_model: the options carry the number afterwards
    from __graft_entry__ import _anticline_model
    g, ii, opts, dd, ext = _anticline_model(levels=2, custom=False)
    opts.kernel_options.compute_condition_number = True
    gg.compute_model(ii, opts, dd)
    assert abs(opts.kernel_options.condition_number - ref) <= 0.02 * ref
