"""Failure paths the kernels claim to handle, made to happen without a GPU fault.

* Waits that run out: ``gk_set_wait_limit(0)`` makes every capped spin wait
  give up before its first poll -- the block flags of the triangular solve,
  the first wait on each staged record tile of the evaluation kernels (single
  system and batched).  The call must report GK_ERR_TIMEOUT in its status word
  and return; a CTA that gave up drains its copies in flight first.
* Iteration caps: FGMRES with ``max_iter`` 1 reports GK_ERR_NOT_CONVERGED.
* The learned solve's fallback: when FGMRES misses the tolerance the FP64 LU
  produces the weights.

Every test then checks that the GPU still computes the right answer.  Nothing
here traps, faults or hangs a GPU.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import kriging  # noqa: E402

pytestmark = pytest.mark.gpu

GK_ERR_NOT_CONVERGED, GK_ERR_TIMEOUT = 5, 7


def _series(seed=3, n_surf=3, per=60, n_o=40):
    """A folded three-surface series: N = 3 n_o + n_surf (per - 1) + 3 = 300."""
    rng = np.random.default_rng(seed)
    pts = []
    for k in range(n_surf):
        xy = rng.uniform(-0.4, 0.4, (per, 2))
        pts.append(np.column_stack([xy, -0.3 + 0.3 * k + 0.05 * np.sin(4 * xy[:, 0])]))
    sp = np.concatenate(pts)
    xo = rng.uniform(-0.4, 0.4, (n_o, 3))
    g = rng.normal(0, 0.1, (n_o, 3)) + [0, 0, 1]
    g /= np.linalg.norm(g, axis=1, keepdims=True)
    return kriging.Series(xo, g, np.full(n_o, 0.01), sp, np.full(len(sp), 2e-5), np.full(n_surf, per),
                          range=0.9, c_o=0.9 ** 2 / 14 / 3)


def _device(s):
    from gempy_gb300 import kernels as K
    return K.DeviceSeries(s.dip_positions, s.dip_gradients, s.nugget_grad, s.sp_coords, s.nugget_sp,
                          s.points_per_surface, range=s.range, c_o=s.c_o, uni_degree=s.uni_degree,
                          kernel=s.kernel, i_res=s.i_res, gi_res=s.gi_res)


@pytest.fixture
def wait_limit():
    """Sets the wait cap for the test body; always restores the defaults."""
    from gempy_gb300 import kernels as K
    yield K.set_wait_limit
    torch.cuda.synchronize()
    K.set_wait_limit(None)


def test_triangular_solve_wait_runs_out_and_reports_timeout(wait_limit):
    from gempy_gb300 import kernels as K
    s = _series()
    ds = _device(s)
    assert ds.N == 300                               # three 128-row blocks: later blocks wait on flags
    Kd, b = K.build(ds, K.GK_F64)
    f = K.lu_factor(Kd, K.GK_F64)
    assert K.read_info(f.info)["status"] == 0
    wait_limit(0)
    K.lu_solve(f, b)
    torch.cuda.synchronize()
    inf = K.read_info(f.info)
    assert inf["status"] == GK_ERR_TIMEOUT and inf["where"] >= 0, inf
    # defaults back: the same factors solve correctly
    wait_limit(None)
    f.info.zero_()
    x = K.lu_solve(f, b).cpu().numpy()
    assert K.read_info(f.info)["status"] == 0
    Kr, br = kriging.build_system(s)
    np.testing.assert_allclose(x, kriging.solve(Kr, br), rtol=0, atol=1e-8 * np.abs(x).max())


@pytest.mark.parametrize("prec", ["f64", "ff", "f32"])
def test_evaluation_copy_wait_runs_out_and_reports_timeout(wait_limit, prec):
    from gempy_gb300 import kernels as K
    s = _series()
    ds = _device(s)
    w, _ = K.solve_plain(ds)
    model = K.prepare(ds, w)
    x = np.random.default_rng(0).uniform(-0.5, 0.5, (50_000, 3))
    pts = K.Points(xyz=torch.as_tensor(x, device="cuda"))
    p = {"f64": K.GK_F64, "ff": K.GK_FF, "f32": K.GK_F32}[prec]
    info = K.new_info(ds.device)
    wait_limit(0)
    K.evaluate(ds, model, pts, p, info=info)
    torch.cuda.synchronize()
    assert K.read_info(info)["status"] == GK_ERR_TIMEOUT
    wait_limit(None)
    info.zero_()
    z, _, _, _ = K.evaluate(ds, model, pts, p, info=info)
    assert K.read_info(info)["status"] == 0
    zr = kriging.evaluate(s, w.cpu().numpy(), x)
    tol = {"f64": 1e-9, "ff": 1e-9, "f32": 1e-3}[prec]
    assert np.abs(z.cpu().numpy() - zr).max() <= tol * np.abs(zr).max()


def test_batch_evaluation_wait_runs_out_and_reports_in_realisation_status(wait_limit):
    from gempy_gb300 import synthetic
    from gempy_gb300.batch import BatchRunner
    models = [synthetic.realisation(i, resolution=(16, 12, 10), base_seed=5) for i in range(3)]
    br = BatchRunner(models)
    br.run()
    torch.cuda.synchronize()
    ref = br.field.clone()
    assert all(int(i["status"]) == 0 for i in br.infos_host())
    wait_limit(0)
    br.run()
    torch.cuda.synchronize()
    st = [int(i["status"]) for i in br.infos_host()]
    assert GK_ERR_TIMEOUT in st and set(st) <= {0, GK_ERR_TIMEOUT}, st
    wait_limit(None)
    br.run()
    torch.cuda.synchronize()
    assert all(int(i["status"]) == 0 for i in br.infos_host())
    assert torch.equal(br.field, ref)


def test_fgmres_iteration_cap_reports_not_converged():
    from gempy_gb300 import kernels as K
    ds = _device(_series())
    x, info = K.solve_mixed(ds, tol=1e-15, max_iter=1)
    inf = K.read_info(info)
    assert inf["status"] == GK_ERR_NOT_CONVERGED and inf["iterations"] <= 1, inf
    x, info, _ = K.solve_twolevel(ds, n_landmarks=64, block=64, tol=1e-15, max_iter=1)
    inf = K.read_info(info)
    assert inf["status"] == GK_ERR_NOT_CONVERGED, inf
    # with a reachable tolerance the same solver converges
    x, info = K.solve_mixed(ds, tol=1e-11, max_iter=60)
    assert K.read_info(info)["status"] == 0


def test_learned_solve_falls_back_to_the_lu():
    """FGMRES cannot meet a 1e-30 tolerance: the FP64 LU produces the weights."""
    import os

    from gempy_gb300 import kernels as K
    from gempy_gb300 import learned
    if not os.path.exists(learned.DEFAULT_MODEL):
        pytest.skip("no trained model in the package")
    model = learned.CostModel.load(learned.DEFAULT_MODEL, device="cuda")
    ds = _device(_series())
    cfg = learned.PrecondConfig(64, 64, "random", K.GK_F64)
    r = learned.solve_learned(ds, model, tol=1e-30, max_iter=5, config=cfg)
    assert r.fallback and r.status == GK_ERR_NOT_CONVERGED
    w_lu, _ = K.solve_plain(ds)
    torch.testing.assert_close(r.x, w_lu, rtol=0, atol=1e-12 * float(w_lu.abs().max()))


def test_compute_model_reports_the_learned_fallback():
    """Through compute_model: the series' solver status says the LU made w
    (``where`` 1), and the model matches the plain form's."""
    import os

    import __graft_entry__ as ge
    import gempy_gb300 as gg
    from gempy_gb300 import learned
    if not os.path.exists(learned.DEFAULT_MODEL):
        pytest.skip("no trained model in the package")
    g, ii, opts, dd, ext = ge._anticline_model(levels=3)
    sol = gg.compute_model(ii, opts, dd, config=gg.EngineConfig(dtype="float32", learned_min_n=1,
                                                                 learned_tol=1e-30))
    info = sol.solver_info[0]
    assert int(info["where"]) == 1 and int(info["status"]) == 0, info
    ref = gg.compute_model(ii, opts, dd, config=gg.EngineConfig(dtype="float64"))
    np.testing.assert_allclose(sol.root_output.outputs[0].weights, ref.root_output.outputs[0].weights,
                               rtol=0, atol=1e-12)
    np.testing.assert_array_equal(sol.raw_arrays.custom, np.array(g["expected_ids"], float))


def test_tensor_core_update_wait_runs_out_and_reports_timeout(wait_limit):
    """The FP32 LU's tensor-core trailing update gives up on its MMA-completion
    wait (cap 0): GK_ERR_TIMEOUT in the status word, the kernel still waits
    (default cap) for its MMAs in flight and frees its tensor memory, and the
    next factorization with the default caps is correct."""
    from gempy_gb300 import _lib
    from gempy_gb300 import kernels as K
    n = 1000
    rng = np.random.default_rng(11)
    A = rng.normal(size=(n, n)) + 4.0 * n ** 0.5 * np.eye(n)
    ld = K.leading_dim(n, K.GK_F32)
    At = torch.zeros((n, ld), dtype=torch.float32, device="cuda")
    At[:, :n] = torch.as_tensor(A, dtype=torch.float32)
    with K.lu_update_engine(_lib.GK_LU_UPDATE_TC):
        wait_limit(0)
        f = K.lu_factor(At)
        torch.cuda.synchronize()
        inf = K.read_info(f.info)
        assert inf["status"] == GK_ERR_TIMEOUT and inf["where"] >= 0, inf
        wait_limit(None)
        f = K.lu_factor(At)
        b = rng.normal(size=n)
        x = K.lu_solve(f, torch.as_tensor(b, dtype=torch.float32, device="cuda")).double().cpu().numpy()
    assert K.read_info(f.info)["status"] == 0
    assert np.abs(b - A @ x).max() / (np.abs(A).max() * np.abs(x).max() * n) < 1e-6
