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
