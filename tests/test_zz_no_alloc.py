"""The allocation-free mixed solve (gk_solve_mixed_noalloc) against the
allocating one (gk_solve_mixed), through the C ABI.

gk_solve_mixed_noalloc serves callers that cannot call cudaMalloc (a host
framework that owns the device memory budget, or a runtime that binds the C
ABI without any way to pass device workspace): its scratch is a device array
inside the library, limited to systems of n <= GK_NOALLOC_MAX_N.  This file is
collected last so that, if it fails, a run stopped at the first failure has
run every other test already; it also passes on its own in a fresh process.

Tolerance: the tests of the mixed solve elsewhere accept a relative residual
of 1e-11; both entry points run the same arithmetic on the same inputs, so
their solutions must agree to 1e-12 relative and both meet the 1e-11 residual.
"""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import kriging  # noqa: E402
from tests._models import load_golden, oracle_series_from_golden  # noqa: E402

pytestmark = pytest.mark.gpu


def _random_system(seed, n_surf=4, per=60, n_o=40):
    rng = np.random.default_rng(seed)
    pts = []
    for k in range(n_surf):
        xy = rng.uniform(-0.4, 0.4, (per, 2))
        pts.append(np.column_stack([xy, -0.3 + 0.2 * k + 0.05 * np.sin(4 * xy[:, 0])]))
    g = rng.normal(0, 0.1, (n_o, 3)) + [0, 0, 1]
    g /= np.linalg.norm(g, axis=1, keepdims=True)
    s = kriging.Series(rng.uniform(-0.4, 0.4, (n_o, 3)), g, np.full(n_o, 0.01), np.concatenate(pts),
                       np.full(n_surf * per, 2e-5), np.full(n_surf, per), range=0.9, c_o=0.9 ** 2 / 42)
    return kriging.build_system(s)


def _systems():
    return [kriging.build_system(oracle_series_from_golden(load_golden("anticline_corners.json"))),
            _random_system(3)]


def _device_system(K, b):
    from gempy_gb300 import kernels as KK
    n = K.shape[0]
    ld = KK.leading_dim(n, KK.GK_F64)
    Kt = torch.zeros((n, ld), dtype=torch.float64, device="cuda")
    Kt[:, :n] = torch.as_tensor(K)
    return Kt, ld, torch.as_tensor(b, device="cuda")


def _solve_allocating(K, b):
    from gempy_gb300 import _lib
    from gempy_gb300 import kernels as KK
    lib = _lib.load()
    n = K.shape[0]
    Kt, ld, bt = _device_system(K, b)
    x = torch.empty(n, dtype=torch.float64, device="cuda")
    wb = lib.gk_solve_mixed_workspace_bytes(n)
    work = torch.empty(wb, dtype=torch.uint8, device="cuda")
    info = KK.new_info("cuda")
    _lib.check("gk_solve_mixed", lib.gk_solve_mixed(n, KK._ptr(Kt), ld, KK._ptr(bt), KK._ptr(x), 1e-12, 60,
                                                    KK._ptr(work), wb, KK._ptr(info), KK._stream()))
    return x.cpu().numpy(), KK.read_info(info)


def _solve_noalloc(K, b):
    from gempy_gb300 import _lib
    from gempy_gb300 import kernels as KK
    lib = _lib.load()
    n = K.shape[0]
    Kt, ld, bt = _device_system(K, b)
    x = torch.empty(n, dtype=torch.float64, device="cuda")
    info = KK.new_info("cuda")
    st = lib.gk_solve_mixed_noalloc(n, KK._ptr(Kt), ld, KK._ptr(bt), KK._ptr(x), 1e-12, 60, KK._ptr(info),
                                    KK._stream())
    _lib.check("gk_solve_mixed_noalloc", st)
    torch.cuda.synchronize()
    return x.cpu().numpy(), KK.read_info(info)


def test_noalloc_solve_matches_allocating_solve_on_two_calls_in_a_row():
    for K, b in _systems():
        assert K.shape[0] <= 1024
        x_ref, info_ref = _solve_allocating(K, b)
        assert info_ref["residual"] <= 1e-11
        for _ in range(2):      # the shared scratch keeps the previous call's contents
            x, info = _solve_noalloc(K, b)
            assert info["status"] == 0, info
            assert info["residual"] <= 1e-11
            assert np.linalg.norm(b - K @ x) <= 1e-11 * np.linalg.norm(b)
            assert np.abs(x - x_ref).max() <= 1e-12 * np.abs(x_ref).max()


def test_noalloc_solve_at_its_largest_accepted_size():
    """n = GK_NOALLOC_MAX_N (1024 unknowns: 99 orientations, 4 surfaces of 182
    points, linear drift): the scratch it needs fits the library's array on
    this device, and the result matches the allocating solve."""
    from gempy_gb300 import _lib
    lib = _lib.load()
    K, b = _random_system(5, n_surf=4, per=182, n_o=99)
    n = K.shape[0]
    assert n == _lib.GK_NOALLOC_MAX_N
    assert lib.gk_solve_mixed_workspace_bytes(n) <= 8 << 20
    x_ref, info_ref = _solve_allocating(K, b)
    assert info_ref["residual"] <= 1e-11
    for _ in range(2):
        x, info = _solve_noalloc(K, b)
        assert info["status"] == 0, info
        assert info["residual"] <= 1e-11
        assert np.abs(x - x_ref).max() <= 1e-12 * np.abs(x_ref).max()


def test_noalloc_solve_rejects_systems_above_its_limit():
    from gempy_gb300 import _lib
    lib = _lib.load()
    n = _lib.GK_NOALLOC_MAX_N + 1
    # rejected on the host before any device pointer is touched
    st = lib.gk_solve_mixed_noalloc(n, ctypes.c_void_p(1), n, ctypes.c_void_p(1), ctypes.c_void_p(1), 1e-12, 10,
                                    None, None)
    assert st == _lib.GK_ERR_SIZE
