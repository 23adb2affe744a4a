"""Learned preconditioner selection: the network kernels against the CPU
oracle (forward, gradients, loss, AdamW step, geometry descriptor), the FP64
two-level solve against the FP64 LU, training, and the gain of the trained
network over the fixed configuration it replaces."""
import os

import numpy as np
import pytest
import torch

from oracle import mlp as omlp


# ---------------------------------------------------------------- CPU ------
def test_oracle_gradient_matches_finite_differences():
    # the oracle's analytic gradient vs central differences (float64, no BF16)
    rng = np.random.default_rng(0)
    F, O, B = 5, 2, 7
    n = omlp.param_count(F, O)
    p = rng.normal(0, 0.2, n)
    x = rng.normal(0, 1, (B, F))
    t = rng.normal(0, 1, (B, O))
    w = rng.uniform(0.5, 2.0, B)

    def loss(q):
        y, _ = omlp.forward(q, x, F, O)
        return omlp.mse(y, t, w)[0]

    y, acts = omlp.forward(p, x, F, O)
    _, dy = omlp.mse(y, t, w)
    g = omlp.backward(p, acts, dy, F, O)
    idx = rng.choice(n, 60, replace=False)
    h = 1e-6
    for i in idx:
        e = np.zeros(n)
        e[i] = h
        fd = (loss(p + e) - loss(p - e)) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, g[i])


def test_bf16_rounding_matches_torch():
    rng = np.random.default_rng(1)
    x = np.concatenate([rng.normal(0, 1, 5000), rng.normal(0, 1e-3, 1000), [0.0, -0.0, 1.0, -2.5]]).astype(np.float32)
    # exact ties: mantissa low half 0x8000
    ties = (np.arange(64, dtype=np.uint32) << 16 | 0x3F808000).view(np.float32)
    x = np.concatenate([x, ties])
    ours = omlp.bf16_bits(x)
    ref = torch.as_tensor(x).to(torch.bfloat16).view(torch.int16).numpy().view(np.uint16)
    assert np.array_equal(ours, ref)


def test_param_count_matches_library():
    from gempy_gb300 import _lib
    lib = _lib.load()
    for F, O in [(20, 1), (5, 2), (64, 16), (1, 1)]:
        assert lib.gk_mlp_param_count(F, O) == omlp.param_count(F, O)
    assert lib.gk_mlp_param_count(0, 1) == -1
    assert lib.gk_mlp_param_count(65, 1) == -1
    assert lib.gk_mlp_workspace_bytes(20, 1, 0) == 0


def test_config_features_and_candidates():
    from gempy_gb300 import learned
    assert learned.IN_DIM == 21
    c = learned.CANDIDATES
    assert len(c) == len(set(c)) == 72
    f = np.stack([x.features() for x in c])
    assert np.unique(f, axis=0).shape[0] == len(c)
    assert all(x.landmarks <= 3000 for x in learned.candidates_for(6000))
    assert learned.DEFAULT_CONFIG in c


def test_training_system_is_deterministic():
    from gempy_gb300 import synthetic
    a, b = synthetic.training_system(3), synthetic.training_system(3)
    assert np.array_equal(a.sp_world, b.sp_world) and a.meta == b.meta
    assert 1000 <= a.meta["n_points"] <= 16000


def test_packaged_model_is_consistent():
    """The shipped network: BF16 weights of the right shape, the master copy
    they round from, and finite predictions through the oracle."""
    from gempy_gb300 import learned
    if not os.path.exists(learned.DEFAULT_MODEL):
        pytest.skip("no trained model in the package")
    z = np.load(learned.DEFAULT_MODEL)
    F, O = int(z["mlp_in_dim"]), int(z["mlp_out_dim"])
    assert (F, O) == (learned.IN_DIM, learned.OUT_DIM)
    bits = z["mlp_params"].view(np.uint16)
    assert bits.size == omlp.param_count(F, O)
    assert np.array_equal(bits, omlp.bf16_bits(z["mlp_master"]))
    p = omlp.bf16_value(bits).astype(np.float64)
    X = np.random.default_rng(0).normal(0, 1, (48, F))
    y, _ = omlp.forward(p, X, F, O)
    assert np.isfinite(y).all()
    assert z["x_mean"].shape == (F,) and z["y_mean"].shape == (O,)


# ---------------------------------------------------------------- GPU ------
def _net(F, O, seed):
    from gempy_gb300 import learned
    net = learned.Mlp(F, O, seed=seed)
    rng = np.random.default_rng(seed + 100)
    flat = rng.normal(0, 0.15, net.master.numel()).astype(np.float32)
    net.master.copy_(torch.as_tensor(flat))
    net._sync_params()
    bits = net.params.cpu().numpy().view(np.uint16)
    return net, omlp.bf16_value(bits).astype(np.float64)


@pytest.mark.gpu
@pytest.mark.parametrize("F,O,B", [(20, 1, 300), (7, 3, 1), (64, 16, 1100)])
def test_mlp_forward_matches_oracle(F, O, B):
    net, p = _net(F, O, 1)
    x = np.random.default_rng(2).normal(0, 1, (B, F)).astype(np.float32)
    y = net.forward(torch.as_tensor(x).cuda()).cpu().numpy()
    yo, _ = omlp.forward(p, x.astype(np.float64), F, O)
    # FP32 accumulation of <= 257-term sums
    assert np.abs(y - yo).max() <= 1e-4 * max(1.0, np.abs(yo).max())


@pytest.mark.gpu
@pytest.mark.parametrize("F,O,B", [(20, 1, 300), (5, 2, 1700), (64, 16, 40)])
def test_mlp_gradient_matches_oracle(F, O, B):
    net, p = _net(F, O, 3)
    rng = np.random.default_rng(4)
    x = rng.normal(0, 1, (B, F)).astype(np.float32)
    dy = rng.normal(0, 1, (B, O)).astype(np.float32)
    g = net.gradient(torch.as_tensor(x).cuda(), torch.as_tensor(dy).cuda()).cpu().numpy()
    _, acts = omlp.forward(p, x.astype(np.float64), F, O)
    go = omlp.backward(p, acts, dy.astype(np.float64), F, O)
    scale = np.abs(go).max()
    assert np.abs(g - go).max() <= 2e-4 * scale
    # per layer, relative to that layer's own scale
    o = 0
    for n, k in omlp.layer_shapes(F, O):
        sl = slice(o, o + n * (k + 1))
        assert np.abs(g[sl] - go[sl]).max() <= 2e-4 * max(np.abs(go[sl]).max(), 1e-3 * scale)
        o += n * (k + 1)
    # bitwise reproducible
    g2 = net.gradient(torch.as_tensor(x).cuda(), torch.as_tensor(dy).cuda()).cpu().numpy()
    assert np.array_equal(g, g2)


@pytest.mark.gpu
def test_mse_and_adam_match_oracle():
    import ctypes
    from gempy_gb300 import _lib, kernels
    lib = _lib.load()
    rng = np.random.default_rng(5)
    B, O = 777, 3
    y = rng.normal(0, 1, (B, O)).astype(np.float32)
    t = rng.normal(0, 1, (B, O)).astype(np.float32)
    w = rng.uniform(0.1, 3, B).astype(np.float32)
    yd, td, wd = (torch.as_tensor(a).cuda() for a in (y, t, w))
    dy = torch.empty_like(yd)
    loss = torch.empty(1, dtype=torch.float32, device="cuda")
    assert lib.gk_mlp_mse(B, O, kernels._ptr(yd), kernels._ptr(td), kernels._ptr(wd), kernels._ptr(dy),
                          kernels._ptr(loss), kernels._stream()) == 0
    lo, dyo = omlp.mse(y, t, w)
    assert abs(float(loss) - lo) <= 1e-5 * lo
    assert np.abs(dy.cpu().numpy() - dyo).max() <= 1e-5 * np.abs(dyo).max()

    n = 5000
    master = rng.normal(0, 0.3, n).astype(np.float32)
    grad = rng.normal(0, 1e-2, n).astype(np.float32)
    m = rng.normal(0, 1e-3, n).astype(np.float32)
    v = rng.uniform(0, 1e-4, n).astype(np.float32)
    md, gd, mm, vv = (torch.as_tensor(a.copy()).cuda() for a in (master, grad, m, v))
    params = torch.empty(n, dtype=torch.int16, device="cuda")
    hp = _lib.GkAdam(1e-3, 0.9, 0.999, 1e-8, 1e-2)
    assert lib.gk_mlp_adam(n, kernels._ptr(md), kernels._ptr(params), kernels._ptr(gd), kernels._ptr(mm),
                           kernels._ptr(vv), ctypes.byref(hp), 7, kernels._stream()) == 0
    mo, m_o, v_o = omlp.adam(master.astype(np.float64), grad.astype(np.float64), m.astype(np.float64),
                             v.astype(np.float64), 1e-3, 0.9, 0.999, 1e-8, 1e-2, 7)
    got = md.cpu().numpy()
    assert np.abs(got - mo).max() <= 1e-6 * np.abs(mo).max()
    assert np.abs(mm.cpu().numpy() - m_o).max() <= 1e-6 * np.abs(m_o).max()
    assert np.array_equal(params.cpu().numpy().view(np.uint16), omlp.bf16_bits(got))


@pytest.mark.gpu
def test_mlp_arguments_are_checked():
    import ctypes
    from gempy_gb300 import _lib, kernels
    lib = _lib.load()
    net = _lib.GkMlp()
    net.in_dim, net.out_dim, net.params = 0, 1, 0
    x = torch.zeros(4, dtype=torch.float32, device="cuda")
    assert lib.gk_mlp_fwd(ctypes.byref(net), 1, kernels._ptr(x), kernels._ptr(x), kernels._ptr(x), 16,
                          kernels._stream()) == _lib.GK_ERR_ARG
    net.in_dim = 1
    net.params = x.data_ptr()
    assert lib.gk_mlp_fwd(ctypes.byref(net), 1, kernels._ptr(x), kernels._ptr(x), kernels._ptr(x), 16,
                          kernels._stream()) == _lib.GK_ERR_SIZE


@pytest.mark.gpu
def test_system_features_match_oracle():
    from gempy_gb300 import learned, synthetic
    for idx in (0, 5):
        m = synthetic.training_system(idx)
        s = learned.series_of(m)
        f = learned.system_features(s).cpu().numpy()
        ii, ko = m.interpolation_input, m.options.kernel_options
        fo = omlp.system_features(ii.orientations.dip_positions, ii.orientations.dip_gradients,
                                  ii.orientations.nugget_effect_grad, ii.surface_points.sp_coords,
                                  ii.surface_points.nugget_effect_scalar, s.sys.n_iface, ko.uni_degree, ko.range)
        assert np.abs(f - fo).max() <= 1e-5 * max(1.0, np.abs(fo).max()), (f, fo)


@pytest.mark.gpu
def test_training_reduces_loss():
    # end to end fwd/bwd/AdamW on a smooth regression target
    from gempy_gb300 import learned
    rng = np.random.default_rng(6)
    X = rng.normal(0, 1, (4096, learned.IN_DIM)).astype(np.float32)
    y = (np.sin(X[:, 0]) + 0.5 * X[:, 1] * X[:, 2] - 0.3 * X[:, 3] ** 2).astype(np.float64)
    ds = dict(sys_feats=X[:, :16], cfg_feats=X[:, 16:], t_run=np.exp(y), ok=(X[:, 5] > 0).astype(float),
              t_lu=np.exp(0.5 * X[:, 6]))
    model, hist = learned.train(ds, epochs=60, batch=256, lr=2e-3, weight_decay=1e-4, seed=0)
    assert hist[-1] < 0.1 * hist[0], hist[::10]
    # checkpoint round trip, then training resumes from the saved state
    st = model.mlp.state()
    net2 = learned.Mlp.from_state(st)
    x = torch.as_tensor(model._norm(X[:64])).cuda()
    assert torch.equal(model.mlp.forward(x), net2.forward(x))
    assert net2.step == model.mlp.step


@pytest.mark.gpu
def test_twolevel_fp64_and_ff_storage_match_lu():
    from gempy_gb300 import kernels, learned, synthetic
    m = synthetic.training_system(1, base_seed=3, n_min=3000, n_max=3500)
    s = learned.series_of(m)
    K, b = kernels.build(s, kernels.GK_F64)
    x_lu, _ = learned.solve_plain_K(K, b)
    pts = learned.check_points(s)
    f_lu = learned.field_at(s, x_lu, pts)
    for policy, prec in (("random", kernels.GK_F64), ("stratified", kernels.GK_F64), ("stratified", kernels.GK_FF)):
        x, inf = learned.solve_with(s, learned.PrecondConfig(512, 256, policy, prec), K, b, tol=1e-10,
                                    max_iter=1500)
        assert int(inf["status"]) == 0, inf
        assert learned.field_error(s, x, f_lu, pts) < 1e-6


@pytest.mark.gpu
def test_learned_choice_beats_fixed_configuration():
    """The gain of the trained network: on held-out systems (not in its
    training set) the learned solve -- the network's pick, with its fallbacks
    -- reproduces the FP64 LU's scalar field within 1e-6 and takes less total
    time than the fixed default configuration (charged the LU time when it
    fails, as its fallback)."""
    import time
    from gempy_gb300 import kernels, learned, synthetic
    if not os.path.exists(learned.DEFAULT_MODEL):
        pytest.skip("no trained model in the package")
    model = learned.CostModel.load()

    def clock(fn):
        torch.cuda.synchronize()
        t = time.perf_counter()
        out = fn()
        torch.cuda.synchronize()
        return out, time.perf_counter() - t

    t_learned = t_default = 0.0
    for idx in range(5):
        m = synthetic.training_system(idx, base_seed=99, n_min=6000, n_max=12000)
        s = learned.series_of(m)
        K, b = kernels.build(s, kernels.GK_F64)
        (x_lu, _), t_lu = clock(lambda: learned.solve_plain_K(K, b))
        pts = learned.check_points(s)
        f_lu = learned.field_at(s, x_lu, pts)
        res, t = clock(lambda: learned.solve_learned(s, model, K, b))
        assert learned.field_error(s, res.x, f_lu, pts) <= 1e-6, (idx, res.config, res.fallback)
        t_learned += t
        (_, inf), t = clock(lambda: learned.solve_with(s, learned.DEFAULT_CONFIG, K, b))
        t_default += t if int(inf["status"]) == 0 else t + t_lu
    assert t_learned < 0.8 * t_default, (t_learned, t_default)


@pytest.mark.gpu
def test_compute_model_routes_large_series_through_learned_solve():
    """compute_model (mixed form) with the learned solve enabled for the
    series gives the plain FP64 form's field within 1e-6 and the same ids
    outside the isovalue band."""
    import gempy_gb300 as gg
    from gempy_gb300 import learned, synthetic
    if not os.path.exists(learned.DEFAULT_MODEL):
        pytest.skip("no trained model in the package")
    m = synthetic.learned(n_points=2500, n_orient=700, n_surf=5)
    args = (m.interpolation_input, m.options, m.data_descriptor)
    plain = gg.compute_model(*args, config=gg.EngineConfig(dtype="float64"))
    lrn = gg.compute_model(*args, config=gg.EngineConfig(dtype="float32", learned_min_n=1000))
    zp = np.asarray(plain.raw_arrays.scalar_field_matrix)[0]
    zl = np.asarray(lrn.raw_arrays.scalar_field_matrix)[0]
    assert np.abs(zl - zp).max() <= 1e-6 * np.abs(zp).max()
    info = lrn.solver_info[0]
    assert int(info["status"]) == 0 and int(info["iterations"]) > 0 and int(info["where"]) == 0, info
    ids_p, ids_l = np.asarray(plain.raw_arrays.lith_block), np.asarray(lrn.raw_arrays.lith_block)
    iso = np.asarray(plain.scalar_field_at_surface_points)
    band = 1e-5 * np.abs(zp).max()
    outside = (np.abs(zp[:, None] - iso[None, :]) > band).all(1)
    assert np.array_equal(ids_p[outside], ids_l[outside])


@pytest.mark.gpu
@pytest.mark.parametrize("F,O,B", [(21, 3, 48), (21, 3, 300), (7, 1, 1), (64, 16, 257)])
def test_mlp_tensor_core_forward_matches_oracle(F, O, B):
    """tcgen05 inference pass vs the oracle with BF16-rounded layer inputs
    (FP32 accumulation on the tensor cores vs float64 sums)."""
    net, p = _net(F, O, 7)
    x = np.random.default_rng(8).normal(0, 1, (B, F)).astype(np.float32)
    y = net.forward_tc(torch.as_tensor(x).cuda()).cpu().numpy()
    yo = omlp.forward_bf16_activations(p, x, F, O)
    assert np.abs(y - yo).max() <= 2e-3 * max(1.0, np.abs(yo).max()), np.abs(y - yo).max()


@pytest.mark.gpu
def test_tensor_core_inference_agrees_with_training_path():
    """The trained network's cost predictions on the tensor cores (BF16 layer
    inputs) and on the FP32 path it was trained with pick equally good
    configurations."""
    from gempy_gb300 import learned, synthetic
    if not os.path.exists(learned.DEFAULT_MODEL):
        pytest.skip("no trained model in the package")
    model = learned.CostModel.load()
    for idx in range(4):
        s = learned.series_of(synthetic.training_system(idx, base_seed=77))
        cands = learned.candidates_for(s.N)
        f = learned.system_features(s).cpu().numpy()
        c_tc = model.expected_cost(f, cands, tensor_cores=True)
        c_32 = model.expected_cost(f, cands, tensor_cores=False)
        assert np.abs(np.log(c_tc) - np.log(c_32)).max() < 0.15
        assert c_32[int(np.argmin(c_tc))] <= 1.1 * c_32.min()


@pytest.mark.gpu
def test_twolevel_warm_start_from_previous_weights():
    """FGMRES started from the previous weights (InterpolationInput.weights)
    needs no iteration when they already solve the system and fewer than a
    cold start when they are perturbed."""
    from gempy_gb300 import kernels, learned, synthetic
    s = learned.series_of(synthetic.training_system(2, base_seed=5, n_min=3000, n_max=3500))
    K, b = kernels.build(s, kernels.GK_F64)
    cfg = learned.PrecondConfig(512, 256, "stratified", kernels.GK_FF)
    x, inf = learned.solve_with(s, cfg, K, b)
    assert int(inf["status"]) == 0
    x2, inf2 = learned.solve_with(s, cfg, K, b, x0=x)
    assert int(inf2["status"]) == 0 and int(inf2["iterations"]) == 0
    assert torch.equal(x2, x)
    xp = x * (1 + 1e-6 * torch.randn_like(x))
    x3, inf3 = learned.solve_with(s, cfg, K, b, x0=xp)
    assert int(inf3["status"]) == 0 and int(inf3["iterations"]) < int(inf["iterations"])


@pytest.mark.parametrize("policy", ["random", "stratified"])
def test_twolevel_permutation_layout(policy):
    """Host-side permutation of the two-level solve: a permutation of all
    unknowns, r a multiple of 64, every drift unknown among the landmarks,
    the rest in Morton order, stratified landmarks spread over the Z-curve."""
    from gempy_gb300 import kernels, learned, synthetic
    m = synthetic.training_system(4, base_seed=11, n_min=1500, n_max=1600)
    s = learned.series_of(m, device="cpu")
    perm, r = kernels.twolevel_permutation(s, 300, seed=3, policy=policy)
    N = s.N
    assert sorted(perm.tolist()) == list(range(N))
    assert r % 64 == 0 and 300 <= r < N
    pos, nd = kernels.unknown_positions(s)
    assert set(range(N - nd, N)) <= set(perm[:r].tolist())
    rest = perm[r:]
    codes = kernels.morton_codes(pos[rest])
    assert np.all(np.diff(codes) >= 0)
    if policy == "stratified":
        # one landmark per equal stretch of the Z-curve over the covariance unknowns
        order = np.argsort(kernels.morton_codes(pos[:N - nd]), kind="stable")
        rank = np.empty(N - nd, dtype=np.int64)
        rank[order] = np.arange(N - nd)
        lm = np.sort(rank[perm[:r][perm[:r] < N - nd]])
        step = (N - nd) / (r - nd)
        assert np.all(np.diff(lm) <= 2 * step + 1)


def test_cost_model_checkpoint_round_trip(tmp_path):
    """Weights, optimizer state, step and normalisation survive save/load
    (host-side; no network evaluation)."""
    from gempy_gb300 import learned
    net = learned.Mlp(seed=4, device="cpu")
    net.m.fill_(0.25)
    net.v.fill_(0.5)
    net.step = 17
    model = learned.CostModel(net, np.arange(learned.IN_DIM), np.ones(learned.IN_DIM) * 2, [1.0, 2.0, 3.0],
                              [0.5, 0.5, 0.5], {"note": "test"})
    path = tmp_path / "m.npz"
    model.save(str(path))
    back = learned.CostModel.load(str(path), device="cpu")
    assert back.mlp.step == 17 and back.meta == {"note": "test"}
    assert torch.equal(back.mlp.params, net.params) and torch.equal(back.mlp.master, net.master)
    assert torch.equal(back.mlp.m, net.m) and torch.equal(back.mlp.v, net.v)
    assert np.array_equal(back.y_mean, [1.0, 2.0, 3.0]) and np.array_equal(back.x_std, model.x_std)
