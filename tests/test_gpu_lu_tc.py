"""The FP32 trailing update on the tensor cores (tcgen05.mma kind::tf32,
three TF32 products per update: ``gk_lu_tc.cu``) against the FP32 SIMT
update (``sgemm_update_kernel``), through the C ABI.

Tolerances: both engines compute every update to about FP32 accuracy, in a
different order, so factors of a matrix whose pivots are its diagonal agree to
a few hundred FP32 ulps of the largest factor entry (2e-5 relative), and
solutions meet the same backward-error bound as the FP32 LU tests elsewhere
(1e-6 of ||A|| ||x|| n)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import kriging  # noqa: E402
from tests.test_gpu_parity import SERIES_CASES, _dev_series  # noqa: E402

pytestmark = pytest.mark.gpu


def _engines():
    from gempy_gb300 import _lib
    return [_lib.GK_LU_UPDATE_TC, _lib.GK_LU_UPDATE_SIMT]


def _factor(A, engine):
    from gempy_gb300 import kernels as K
    n = A.shape[0]
    ld = K.leading_dim(n, K.GK_F32)
    At = torch.zeros((n, ld), dtype=torch.float32, device="cuda")
    At[:, :n] = torch.as_tensor(A, dtype=torch.float32)
    with K.lu_update_engine(engine):
        f = K.lu_factor(At)
    torch.cuda.synchronize()
    return f


def test_engine_switch_round_trips():
    from gempy_gb300 import _lib
    lib = _lib.load()
    assert lib.gk_lu_update_engine() == _lib.GK_LU_UPDATE_TC      # the default
    assert lib.gk_lu_update_select(7) == _lib.GK_ERR_ARG
    assert lib.gk_lu_update_select(_lib.GK_LU_UPDATE_SIMT) == 0
    assert lib.gk_lu_update_engine() == _lib.GK_LU_UPDATE_SIMT
    assert lib.gk_lu_update_select(_lib.GK_LU_UPDATE_TC) == 0


@pytest.mark.parametrize("n", [100, 257, 1037, 2500])
def test_tensor_core_factors_match_simt_factors(n):
    """Diagonally dominant matrix (the pivots are the diagonal under both
    engines): the packed L\\U factors agree entry by entry."""
    from gempy_gb300 import kernels as K
    rng = np.random.default_rng(n)
    A = rng.normal(size=(n, n)) + 4.0 * n ** 0.5 * np.eye(n)
    ftc = _factor(A, _engines()[0])
    fsi = _factor(A, _engines()[1])
    for f in (ftc, fsi):
        assert K.read_info(f.info)["status"] == 0
        np.testing.assert_array_equal(f.ipiv.cpu().numpy(), np.arange(n, dtype=np.int32))
    a = ftc.LU[:, :n].double().cpu().numpy()
    b = fsi.LU[:, :n].double().cpu().numpy()
    assert np.abs(a - b).max() <= 2e-5 * np.abs(b).max()


@pytest.mark.parametrize("n", [64, 100, 1037, 4099])
def test_tensor_core_lu_solve_backward_error(n):
    from gempy_gb300 import kernels as K
    rng = np.random.default_rng(n + 1)
    A = rng.normal(size=(n, n)) + n ** 0.5 * np.eye(n) * rng.choice([-1, 1], n)
    bvec = rng.normal(size=n)
    f = _factor(A, _engines()[0])
    x = K.lu_solve(f, torch.as_tensor(bvec, dtype=torch.float32, device="cuda")).double().cpu().numpy()
    assert K.read_info(f.info)["status"] == 0
    res = np.abs(bvec - A @ x).max() / (np.abs(A).max() * np.abs(x).max() * n)
    assert res < 1e-6


@pytest.mark.parametrize("case", ["anticline", "random_deg1_cubic", "random_deg2_exp"])
def test_mixed_solve_on_tensor_core_preconditioner(case):
    """The mixed solve (FP32 LU preconditioner + FP64 FGMRES) reaches the
    same FP64 residual with either engine, within two more iterations."""
    from gempy_gb300 import kernels as K
    s = SERIES_CASES[case]()
    Kr, br = kriging.build_system(s)
    out = {}
    for e in _engines():
        with K.lu_update_engine(e):
            w, info = K.solve_mixed(_dev_series(s), tol=1e-12)
        inf = K.read_info(info)
        w = w.cpu().numpy()
        assert inf["status"] == 0 and inf["residual"] <= 1e-11, inf
        assert np.linalg.norm(br - Kr @ w) <= 1e-11 * np.linalg.norm(br)
        out[e] = inf["iterations"]
    assert out[_engines()[0]] <= out[_engines()[1]] + 2


def test_mixed_solve_with_lookahead_matches_lapack():
    """A system above the look-ahead threshold (N = 3495: the next panel's
    diagonal block is factored on a second stream while the rest of the
    update runs): the mixed solve reaches the FP64 residual on both engines
    and its weights match LAPACK's solution."""
    from gempy_gb300 import kernels as K
    from gempy_gb300 import synthetic
    from tests._models import oracle_series_list
    m = synthetic.precision(n_points=2000, n_orient=500, resolution=(8, 8, 8))
    (s,) = oracle_series_list(m)
    Kr, br = kriging.build_system(s)
    assert Kr.shape[0] > 2048
    w_ref = kriging.solve(Kr, br)
    for e in _engines():
        with K.lu_update_engine(e):
            w, info = K.solve_mixed(_dev_series(s), tol=1e-12)
        inf = K.read_info(info)
        w = w.cpu().numpy()
        assert inf["status"] == 0 and inf["residual"] <= 1e-11, inf
        assert np.linalg.norm(br - Kr @ w) <= 1e-11 * np.linalg.norm(br)
        assert np.abs(w - w_ref).max() <= 1e-6 * np.abs(w_ref).max()
