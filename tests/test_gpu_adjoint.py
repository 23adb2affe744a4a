"""Adjoint derivatives on the GPU against central differences of the oracle.

J = sum_x g(x) Z(x) is differentiated through build -> solve -> evaluate by
``gempy_gb300.adjoint.series_field`` (forward: FP64 kernels; backward: the
adjoint kernels and one more solve with the same LU factors).  The oracle's
central differences (FP64, transformed frame, eps below) are the check:
  * positions and dip gradients: eps = 1e-5, agreement <= 1e-6 x max|grad|
    (the solve's ~1e-12 noise in J over 2 eps stays near 1e-7);
  * nuggets: eps = 1e-7 (surface points, ~2e-5) and 1e-6 (orientations,
    ~1e-2), agreement <= 1e-4 x max|grad| (the differences' own rounding
    through the ill-conditioned solve is ~1e-5 of it).
The reference-style check (test/test_modules/test_ad/test_ad_I.py:158-258:
real-space eps = 1e-3 on the fold model, rel or abs error < 1e-2) runs
through compute_model(compute_grads=True) on the same model (model2).
"""
import dataclasses

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import kriging  # noqa: E402
from tests._models import engine_inputs_from_golden, load_golden, oracle_series_from_golden  # noqa: E402

pytestmark = pytest.mark.gpu


def _random_series(seed, n_surf=3, per=10, n_o=6, degree=1, kernel="cubic", a=0.9):
    rng = np.random.default_rng(seed)
    pts = []
    for k in range(n_surf):
        xy = rng.uniform(-0.4, 0.4, (per, 2))
        pts.append(np.column_stack([xy, -0.3 + 0.3 * k + 0.05 * np.sin(4 * xy[:, 0])]))
    sp = np.concatenate(pts)
    xo = rng.uniform(-0.4, 0.4, (n_o, 3))
    g = rng.normal(0, 0.1, (n_o, 3)) + [0, 0, 1]
    g /= np.linalg.norm(g, axis=1, keepdims=True)
    return kriging.Series(xo, g, rng.uniform(0.005, 0.02, n_o), sp, rng.uniform(1e-5, 4e-5, len(sp)),
                          np.full(n_surf, per), range=a, c_o=a * a / 14 / 3, uni_degree=degree, kernel=kernel)


CASES = {
    "anticline": lambda: oracle_series_from_golden(load_golden("anticline_corners.json")),
    "random_deg2_cubic": lambda: _random_series(11, degree=2),
    "random_deg1_exp": lambda: _random_series(12, kernel="exponential", a=0.6),
}


def _J(s, x, g):
    w = kriging.solve(*kriging.build_system(s))
    return float(g @ kriging.evaluate(s, w, x))


def _fd(s, x, g, name, idx, eps):
    arr = getattr(s, name)
    out = []
    for i in idx:
        vals = []
        for sgn in (1, -1):
            a = arr.copy()
            a.flat[i] += sgn * eps
            vals.append(_J(dataclasses.replace(s, **{name: a}), x, g))
        out.append((vals[0] - vals[1]) / (2 * eps))
    return np.array(out)


def _gpu_grads(s, x, g):
    from gempy_gb300 import adjoint
    t = lambda a: torch.as_tensor(np.asarray(a, dtype=np.float64), device="cuda").requires_grad_(True)
    sp, nsp, dpos, dgr, ngr = t(s.sp_coords), t(s.nugget_sp), t(s.dip_positions), t(s.dip_gradients), \
        t(s.nugget_grad)
    xyz = t(x)
    spec = adjoint.SeriesSpec(s.points_per_surface, s.range, s.c_o, s.uni_degree, s.kernel, s.i_res, s.gi_res)
    z = adjoint.series_field(sp, nsp, dpos, dgr, ngr, xyz, spec)
    (z * torch.as_tensor(g, device="cuda")).sum().backward()
    return {k: v.grad.cpu().numpy() for k, v in dict(sp_coords=sp, nugget_sp=nsp, dip_positions=dpos,
                                                    dip_gradients=dgr, nugget_grad=ngr, xyz=xyz).items()}, \
        z.detach().cpu().numpy()


@pytest.mark.parametrize("case", list(CASES))
def test_adjoint_matches_oracle_central_differences(case):
    s = CASES[case]()
    rng = np.random.default_rng(3)
    x = rng.uniform(-0.45, 0.45, (7, 3))
    x[0] = s.sp_coords[1]                       # on a data point (r = 0 with the regulariser)
    g = rng.normal(size=len(x))
    grads, z = _gpu_grads(s, x, g)
    w = kriging.solve(*kriging.build_system(s))
    np.testing.assert_allclose(z, kriging.evaluate(s, w, x), rtol=0, atol=1e-9 * np.abs(z).max())
    checks = [("sp_coords", 1e-5, 1e-6), ("dip_positions", 1e-5, 1e-6), ("dip_gradients", 1e-5, 1e-6),
              ("nugget_sp", 1e-7, 1e-4), ("nugget_grad", 1e-6, 1e-4)]
    for name, eps, tol in checks:
        arr = getattr(s, name)
        idx = rng.choice(arr.size, size=min(arr.size, 12), replace=False)
        fd = _fd(s, x, g, name, idx, eps)
        ad = grads[name].ravel()[idx]
        scale = max(np.abs(grads[name]).max(), 1e-12)
        assert np.abs(ad - fd).max() <= tol * scale, (name, ad, fd)
    # the evaluation points: dJ/dx = g(x) grad Z(x)
    _, G = kriging.evaluate(s, w, x, gradient=True)
    np.testing.assert_allclose(grads["xyz"], g[:, None] * G, rtol=0, atol=1e-9 * np.abs(g[:, None] * G).max())


def test_compute_model_grads_match_real_space_differences():
    """The reference's own check on the fold model (model2), through
    compute_model: d Z(level-0 voxel 0) / d z(surface point 0) in real space,
    adjoint x input-transform scale vs (Z(z + 1e-3) - Z(z - 1e-3)) / 2e-3."""
    import gempy_gb300 as gg
    g = load_golden("anticline_corners.json")
    scale = float(g["transform"]["scale"])
    ii, opts, dd, _ = engine_inputs_from_golden(g, levels=3)
    sol = gg.compute_model(ii, opts, dd, config=gg.EngineConfig(dtype="float64", compute_grads=True))
    sf = sol.octrees_output[0].last_output_center.exported_fields.scalar_field
    sp = sol.taped_interpolation_input.surface_points.sp_coords
    assert sp.requires_grad and sf.requires_grad
    sf[0].backward()
    ad_real = float(sp.grad[0, 2]) * scale
    vals = []
    for sgn in (1, -1):
        ii2, _, _, _ = engine_inputs_from_golden(g, levels=3)
        ii2.surface_points.sp_coords[0, 2] += sgn * 1e-3 * scale
        s2 = gg.compute_model(ii2, opts, dd, config=gg.EngineConfig(dtype="float64"))
        vals.append(float(s2.octrees_output[0].last_output_center.exported_fields.scalar_field[0]))
    num = (vals[0] - vals[1]) / 2e-3
    abs_err = abs(ad_real - num)
    assert abs_err / (abs(ad_real) + 1e-10) < 1e-2 or abs_err < 1e-2, (ad_real, num)
    # the same derivative from the oracle, tighter (transformed frame)
    s = oracle_series_from_golden(g)
    x = sol.octrees_output[0].grid_centers[:1].detach().cpu().numpy()
    fd = _fd(s, x, np.ones(1), "sp_coords", [2], 1e-5)[0]
    assert abs(float(sp.grad[0, 2]) - fd) <= 1e-6 * max(abs(fd), 1e-9)
    # the forward values are those of the plain run
    plain = gg.compute_model(ii, opts, dd, config=gg.EngineConfig(dtype="float64"))
    np.testing.assert_allclose(sf.detach().cpu().numpy(),
                               plain.octrees_output[0].last_output_center.exported_fields.scalar_field,
                               rtol=0, atol=1e-12)


def test_compute_grads_rejects_the_mixed_form():
    import gempy_gb300 as gg
    g = load_golden("anticline_corners.json")
    ii, opts, dd, _ = engine_inputs_from_golden(g, levels=2)
    with pytest.raises(ValueError):
        gg.compute_model(ii, opts, dd, config=gg.EngineConfig(dtype="float32", compute_grads=True))
