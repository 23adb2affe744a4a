"""Batched realisations (gk_batch_*) against the single-system path and the
FP64 oracle, eager and replayed from a CUDA graph.

Tolerances: weights <= 1e-6 relative to the FP64 solve; field <= 1e-9
relative (float-float evaluation); ids identical outside the isovalue band;
graph replay bitwise equal to the eager run.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import kriging, segmentation  # noqa: E402
from tests._models import oracle_series_list  # noqa: E402

pytestmark = pytest.mark.gpu


def _models(n=6, res=(12, 10, 14)):
    from gempy_gb300 import synthetic
    return [synthetic.realisation(i, resolution=res, base_seed=7) for i in range(n)]


def test_batch_matches_oracle_per_realisation():
    from gempy_gb300.batch import BatchRunner
    models = _models()
    br = BatchRunner(models)
    br.run()
    torch.cuda.synchronize()
    infos = br.infos_host()
    field = br.field.cpu().numpy()
    ids = br.ids.cpu().numpy()
    for i, m in enumerate(models):
        (s,) = oracle_series_list(m)
        K, b = kriging.build_system(s)
        w_ref = kriging.solve(K, b)
        assert infos[i]["status"] == 0, infos[i]
        assert infos[i]["residual"] <= 1e-10
        w, iso = br.results(i)
        assert np.abs(w - w_ref).max() <= 1e-6 * np.abs(w_ref).max()
        iso_ref = kriging.isovalues(s, w_ref)
        np.testing.assert_allclose(iso, iso_ref, rtol=1e-7, atol=1e-12)
        x = m.interpolation_input.grid.dense_grid.values
        Zr = kriging.evaluate(s, w_ref, x)
        Z = field[br.item_slice(i)]
        assert np.abs(Z - Zr).max() <= 1e-6 * np.abs(Zr).max()
        _, idr = segmentation.segment(Zr, iso_ref, m.interpolation_input.unit_values, m.options.sigmoid_slope)
        band = max(10.0 / m.options.sigmoid_slope, 4e-6 * np.abs(Zr).max())
        outside = np.all(np.abs(Zr[:, None] - iso_ref[None, :]) > band, axis=1)
        np.testing.assert_array_equal(ids[br.item_slice(i)][outside], idr[outside].astype(np.int32))


def test_batch_field_matches_single_system_path():
    """Same weights in: the batched float-float field equals the single-system
    float-float kernel's to 1e-9 relative."""
    from gempy_gb300 import kernels as K
    from gempy_gb300.batch import BatchRunner
    models = _models(3)
    br = BatchRunner(models)
    br.run()
    torch.cuda.synchronize()
    for i, m in enumerate(models):
        (s,) = oracle_series_list(m)
        w, _ = br.results(i)
        ds = K.DeviceSeries(s.dip_positions, s.dip_gradients, s.nugget_grad, s.sp_coords, s.nugget_sp,
                            s.points_per_surface, range=s.range, c_o=s.c_o, uni_degree=s.uni_degree)
        model = K.prepare(ds, torch.as_tensor(w, device="cuda"))
        f, _, _, _ = K.evaluate(ds, model, K.Points.regular(m.interpolation_input.grid.dense_grid), K.GK_FF)
        Z1 = f.cpu().numpy()
        Zb = br.field[br.item_slice(i)].cpu().numpy()
        assert np.abs(Zb - Z1).max() <= 1e-9 * np.abs(Z1).max()


def test_batch_graph_replay_is_bitwise_equal_to_eager():
    from gempy_gb300.batch import BatchRunner
    br = BatchRunner(_models(5))
    br.run()
    torch.cuda.synchronize()
    f0, i0 = br.field.clone(), br.ids.clone()
    br.capture()
    for _ in range(2):
        br.field.zero_()
        br.ids.zero_()
        br.replay()
        torch.cuda.synchronize()
        assert torch.equal(br.field, f0)
        assert torch.equal(br.ids, i0)


def test_every_tile_variant_gives_the_same_field():
    """All autotuner variants of the float-float, FP32 and batched field
    kernels agree: tile boundaries change where the per-tile float-float sum
    is added into FP64, so variants agree to the float-float accuracy."""
    from gempy_gb300 import _lib, autotune
    from gempy_gb300 import kernels as K
    from gempy_gb300.batch import BatchRunner
    from gempy_gb300 import synthetic
    lib = _lib.load()
    m = synthetic.precision(resolution=(20, 18, 22))
    (s,) = oracle_series_list(m)
    w = kriging.solve(*kriging.build_system(s))
    ds = K.DeviceSeries(s.dip_positions, s.dip_gradients, s.nugget_grad, s.sp_coords, s.nugget_sp,
                        s.points_per_surface, range=s.range, c_o=s.c_o, uni_degree=s.uni_degree)
    model = K.prepare(ds, torch.as_tensor(w, device="cuda"))
    pts = K.Points.regular(m.interpolation_input.grid.dense_grid)
    br = BatchRunner(_models(4))
    # plain FP32 sums are accurate to ~1e-7 x the cancellation factor of the kriging sum
    f64, _, _, _ = K.evaluate(ds, model, pts, K.GK_F64)
    zmax = float(f64.abs().max())
    alpha = kriging.point_coefficients(s, w)
    cancel = s.c_o * s.gi_res * (np.abs(alpha).sum() + np.abs(w[:3 * s.n_o]).sum() * 14 / s.range) / zmax
    saved = {t: lib.gk_tune_get(t) for t in _lib.TUNABLES.values()}
    try:
        for prec, fam in ((K.GK_FF, _lib.GK_TUNE_EVAL_FF), (K.GK_F32, _lib.GK_TUNE_EVAL_F32)):
            ref = None
            for v in autotune.variants():
                lib.gk_tune_set(fam, v["variant"])
                f, _, _, _ = K.evaluate(ds, model, pts, prec)
                f = f.cpu().numpy()
                if ref is None:
                    ref = f
                tol = 1e-9 if prec == K.GK_FF else 2e-6 * cancel   # float-float accuracy / FP32 bound
                assert np.abs(f - ref).max() <= tol * np.abs(ref).max(), (prec, v)
        ref = None
        for v in autotune.variants():
            lib.gk_tune_set(_lib.GK_TUNE_BATCH_EVAL, v["variant"])
            br.run()
            torch.cuda.synchronize()
            f = br.field.cpu().numpy()
            if ref is None:
                ref = f
            assert np.abs(f - ref).max() <= 1e-9 * np.abs(ref).max(), v
    finally:
        for t, v in saved.items():
            lib.gk_tune_set(t, max(v, 0))


def test_autotuner_picks_and_installs_a_variant():
    from gempy_gb300 import _lib, autotune
    lib = _lib.load()
    saved = lib.gk_tune_get(_lib.GK_TUNE_EVAL_FF)
    try:
        table = autotune.tune(families=("eval_ff",), persist=False, reps=1)
        ch = table["choices"]["eval_ff"]
        assert lib.gk_tune_get(_lib.GK_TUNE_EVAL_FF) == ch["variant"]
        assert len(ch["all_ms"]) == lib.gk_tune_variants()
        assert ch["ms"] == min(ch["all_ms"].values()) or abs(ch["ms"] - min(ch["all_ms"].values())) < 1e-3
    finally:
        lib.gk_tune_set(_lib.GK_TUNE_EVAL_FF, max(saved, 0))
