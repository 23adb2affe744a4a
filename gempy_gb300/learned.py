"""Learned choice of the two-level preconditioner for FGMRES.

The reference solves every kriging system with the dense FP64 direct solve.
Here large systems can instead be solved by FGMRES with a two-level
"block-Jacobi plus low-rank" preconditioner (``gk_solve_twolevel``), whose
speed -- and whether it converges at all -- depends on the landmark count r,
the block size, the landmark policy and the storage precision.  A small
network (3 layers, width 256, BF16 weights, FP32 accumulation; CUDA forward,
backward and AdamW kernels in ``gk_mlp.cu``) maps the system's geometry
descriptor (``gk_system_features``) plus one candidate configuration to the
predicted log time of the FGMRES run, the probability that it fails, and the
log time of the LU fallback; the candidate with the least expected cost
t_run + p_fail t_lu is used.  The
dense FP64 LU is the fallback (a candidate that does not reach the tolerance
falls back to it) and the arbiter (training labels record each candidate's
error against the LU solution; a run whose FGMRES residual meets the
tolerance but whose scalar field misses the LU solution's by more than
``LU_AGREEMENT_TOL`` is labelled as failed).

Everything here calls the C ABI; PyTorch only provides device memory.
"""
import ctypes
import json
import os
import time
from dataclasses import asdict, dataclass

import numpy as np
import torch

from . import _lib, kernels
from ._lib import GK_F32, GK_F64, GK_FF, GK_SYSTEM_FEATURES, GkAdam, GkMlp, check

CONFIG_FEATURES = 5
IN_DIM = GK_SYSTEM_FEATURES + CONFIG_FEATURES
# outputs: log(seconds of the FGMRES run), failure indicator, log(seconds of the FP64 LU fallback)
OUT_DIM = 3
MAX_ITER = 1000
LU_AGREEMENT_TOL = 1e-6   # relative scalar-field error of an accepted solution vs the FP64 LU's
DEFAULT_MODEL = os.path.join(os.path.dirname(os.path.abspath(__file__)), "models", "precond_cost.npz")


@dataclass(frozen=True)
class PrecondConfig:
    landmarks: int        # requested landmark count (rounded up to a multiple of 64 with the drift)
    block: int            # block-Jacobi block size
    policy: str           # kernels.LANDMARK_POLICIES
    prec: int             # GK_F32, GK_FF (FP64 storage, float-float updates) or GK_F64

    def features(self):
        return np.array([np.log2(self.landmarks) / 13.0, np.log2(self.block) / 10.0,
                         float(kernels.LANDMARK_POLICIES.index(self.policy)), float(self.prec != GK_F32),
                         float(self.prec == GK_FF)], dtype=np.float32)


CANDIDATES = tuple(PrecondConfig(r, bs, pol, pr)
                   for r in (512, 1024, 2048, 4096, 8192, 16384)
                   for bs in (256, 512)
                   for pol in kernels.LANDMARK_POLICIES
                   for pr in (GK_F32, GK_FF, GK_F64))

# The method without the network: one fixed configuration for every system.
DEFAULT_CONFIG = PrecondConfig(1024, 512, "random", GK_F64)


def candidates_for(N):
    """Candidates whose landmark set leaves at least half the unknowns to the blocks."""
    return [c for c in CANDIDATES if c.landmarks <= N // 2]


def _stream():
    return kernels._stream()


def _ptr(t):
    return kernels._ptr(t)


def system_features(series):
    """GK_SYSTEM_FEATURES floats (device tensor) describing the system's geometry."""
    lib = _lib.load()
    out = torch.empty(GK_SYSTEM_FEATURES, dtype=torch.float32, device=series.device)
    check("gk_system_features", lib.gk_system_features(ctypes.byref(series.sys), _ptr(out), _stream()))
    return out


# ---------------------------------------------------------------------------
# the network
# ---------------------------------------------------------------------------
class Mlp:
    """in_dim -> 256 -> 256 -> out_dim perceptron on the GPU: BF16 weights for
    the kernels, FP32 master weights and AdamW moments for training."""

    def __init__(self, in_dim=IN_DIM, out_dim=OUT_DIM, seed=0, device="cuda"):
        self.in_dim, self.out_dim = int(in_dim), int(out_dim)
        self.device = torch.device(device)
        n = self.param_count(self.in_dim, self.out_dim)
        rng = np.random.default_rng(seed)
        flat = np.zeros(n, dtype=np.float32)
        o = 0
        for nout, nin in ((256, self.in_dim), (256, 256), (self.out_dim, 256)):
            lim = np.sqrt(6.0 / nin)  # He-uniform for ReLU layers
            blk = np.zeros((nout, nin + 1), dtype=np.float32)
            blk[:, :nin] = rng.uniform(-lim, lim, (nout, nin))
            flat[o:o + blk.size] = blk.ravel()
            o += blk.size
        self.master = torch.as_tensor(flat).to(self.device)
        self.m = torch.zeros_like(self.master)
        self.v = torch.zeros_like(self.master)
        self.step = 0
        self.params = torch.empty(n, dtype=torch.int16, device=self.device)
        self._sync_params()
        self._work = None
        self._work_batch = 0

    @staticmethod
    def param_count(in_dim, out_dim):
        n = int(_lib.load().gk_mlp_param_count(int(in_dim), int(out_dim)))
        if n <= 0:
            raise ValueError("bad network dimensions")
        return n

    def _sync_params(self):
        # BF16 image of the master weights (round to nearest even)
        self.params.copy_(self.master.to(torch.bfloat16).view(torch.int16))

    def _net(self):
        net = GkMlp()
        net.in_dim, net.out_dim, net.params = self.in_dim, self.out_dim, self.params.data_ptr()
        return net

    def _workspace(self, batch):
        if self._work is None or self._work_batch < batch:
            nb = _lib.load().gk_mlp_workspace_bytes(self.in_dim, self.out_dim, int(batch))
            if nb == 0:
                raise ValueError("batch out of range")
            self._work = torch.empty(nb, dtype=torch.uint8, device=self.device)
            self._work_batch = batch
        return self._work

    def forward(self, x):
        x = x.to(device=self.device, dtype=torch.float32).contiguous()
        B = x.shape[0]
        y = torch.empty((B, self.out_dim), dtype=torch.float32, device=self.device)
        w = self._workspace(B)
        check("gk_mlp_fwd", _lib.load().gk_mlp_fwd(ctypes.byref(self._net()), B, _ptr(x), _ptr(y), _ptr(w),
                                                    w.numel(), _stream()))
        return y

    def forward_tc(self, x):
        """Inference on the tensor cores (BF16 activations between layers)."""
        x = x.to(device=self.device, dtype=torch.float32).contiguous()
        B = x.shape[0]
        y = torch.empty((B, self.out_dim), dtype=torch.float32, device=self.device)
        err = torch.zeros(1, dtype=torch.int32, device=self.device)
        check("gk_mlp_fwd_tc", _lib.load().gk_mlp_fwd_tc(ctypes.byref(self._net()), B, _ptr(x), _ptr(y), _ptr(err),
                                                          _stream()))
        if int(err.item()) != 0:
            raise _lib.GkError("gk_mlp_fwd_tc", int(err.item()))
        return y

    def gradient(self, x, dy):
        """Forward on x, then the gradient of sum(dy * y) (FP32, parameter layout)."""
        lib = _lib.load()
        x = x.to(device=self.device, dtype=torch.float32).contiguous()
        self.forward(x)
        grad = torch.empty_like(self.master)
        w = self._workspace(x.shape[0])
        check("gk_mlp_bwd", lib.gk_mlp_bwd(ctypes.byref(self._net()), x.shape[0], _ptr(x),
                                           _ptr(dy.contiguous()), _ptr(grad), _ptr(w), w.numel(), _stream()))
        return grad

    def train_step(self, x, t, weight=None, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8, weight_decay=1e-4):
        """One AdamW step on the weighted MSE; returns the loss (device scalar)."""
        lib = _lib.load()
        B = x.shape[0]
        y = self.forward(x)
        dy = torch.empty_like(y)
        loss = torch.empty(1, dtype=torch.float32, device=self.device)
        check("gk_mlp_mse", lib.gk_mlp_mse(B, self.out_dim, _ptr(y), _ptr(t.contiguous()),
                                           _ptr(None if weight is None else weight.contiguous()), _ptr(dy),
                                           _ptr(loss), _stream()))
        grad = torch.empty_like(self.master)
        w = self._workspace(B)
        check("gk_mlp_bwd", lib.gk_mlp_bwd(ctypes.byref(self._net()), B, _ptr(x), _ptr(dy), _ptr(grad), _ptr(w),
                                           w.numel(), _stream()))
        self.step += 1
        hp = GkAdam(lr, beta1, beta2, eps, weight_decay)
        check("gk_mlp_adam", lib.gk_mlp_adam(self.master.numel(), _ptr(self.master), _ptr(self.params), _ptr(grad),
                                             _ptr(self.m), _ptr(self.v), ctypes.byref(hp), self.step, _stream()))
        return loss

    # checkpoint: weights, optimizer state and step (training can resume)
    def state(self):
        return dict(in_dim=self.in_dim, out_dim=self.out_dim, step=self.step,
                    params=self.params.cpu().numpy().view(np.uint16), master=self.master.cpu().numpy(),
                    m=self.m.cpu().numpy(), v=self.v.cpu().numpy())

    @classmethod
    def from_state(cls, st, device="cuda"):
        net = cls(int(st["in_dim"]), int(st["out_dim"]), device=device)
        net.master.copy_(torch.as_tensor(np.asarray(st["master"], np.float32)))
        net.m.copy_(torch.as_tensor(np.asarray(st["m"], np.float32)))
        net.v.copy_(torch.as_tensor(np.asarray(st["v"], np.float32)))
        net.params.copy_(torch.as_tensor(np.asarray(st["params"], np.uint16).view(np.int16)))
        net.step = int(st["step"])
        return net


# ---------------------------------------------------------------------------
# cost model: network + feature / label normalisation
# ---------------------------------------------------------------------------
class CostModel:
    def __init__(self, mlp, x_mean, x_std, y_mean, y_std, meta=None):
        self.mlp = mlp
        self.x_mean = np.asarray(x_mean, np.float32)
        self.x_std = np.asarray(x_std, np.float32)
        self.y_mean = np.asarray(y_mean, np.float64).reshape(-1)
        self.y_std = np.asarray(y_std, np.float64).reshape(-1)
        self.meta = meta or {}

    def _norm(self, X):
        return (np.asarray(X, np.float32) - self.x_mean) / self.x_std

    def predict(self, sys_feats, configs, tensor_cores=True):
        """Per candidate: (run seconds, failure probability, LU seconds).
        Inference runs on the tensor cores (tcgen05, BF16 layer inputs) unless
        ``tensor_cores`` is False (the FP32-activation path used in training)."""
        sf = np.asarray(sys_feats, np.float32).reshape(1, -1)
        X = np.concatenate([np.repeat(sf, len(configs), 0), np.stack([c.features() for c in configs])], 1)
        xt = torch.as_tensor(self._norm(X)).to(self.mlp.device)
        y = (self.mlp.forward_tc(xt) if tensor_cores else self.mlp.forward(xt)).cpu().numpy().astype(np.float64)
        y = y * self.y_std + self.y_mean
        return np.exp(y[:, 0]), np.clip(y[:, 1], 0.0, 1.0), np.exp(y[:, 2])

    def expected_cost(self, sys_feats, configs, tensor_cores=True):
        t_run, p_fail, t_lu = self.predict(sys_feats, configs, tensor_cores)
        return t_run + p_fail * t_lu

    def choose(self, series, N=None):
        N = series.N if N is None else N
        cands = candidates_for(N)
        if not cands:
            return None
        feats = system_features(series).cpu().numpy()
        return cands[int(np.argmin(self.expected_cost(feats, cands)))]

    def save(self, path):
        os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
        st = self.mlp.state()
        np.savez(path, **{f"mlp_{k}": v for k, v in st.items()}, x_mean=self.x_mean, x_std=self.x_std,
                 y_mean=self.y_mean, y_std=self.y_std, meta=json.dumps(self.meta))

    @classmethod
    def load(cls, path=DEFAULT_MODEL, device="cuda"):
        z = np.load(path, allow_pickle=False)
        st = {k[4:]: z[k] for k in z.files if k.startswith("mlp_")}
        return cls(Mlp.from_state(st, device), z["x_mean"], z["x_std"], z["y_mean"], z["y_std"],
                   json.loads(str(z["meta"])))


def targets(dataset):
    """Network targets: log run seconds, failure indicator, log LU seconds."""
    return np.stack([np.log(dataset["t_run"]), 1.0 - dataset["ok"], np.log(dataset["t_lu"])], 1)


def train(dataset, epochs=300, batch=256, lr=2e-3, weight_decay=1e-3, seed=0, model=None, device="cuda",
          log_every=0, lu_weight_alpha=0.0):
    """Fit (or, given ``model``, continue fitting) the cost model on a dataset
    from ``generate`` with AdamW under a cosine learning-rate schedule.  With
    ``lu_weight_alpha`` > 0 each sample's loss is weighted by (its system's LU
    time)^alpha, so the large systems -- where a wrong pick costs seconds --
    count for more.  Returns (model, per-epoch mean losses)."""
    X = np.concatenate([dataset["sys_feats"], dataset["cfg_feats"]], 1).astype(np.float32)
    Y = targets(dataset)
    wts = None
    if lu_weight_alpha > 0:
        w = np.asarray(dataset["t_lu"], np.float64) ** lu_weight_alpha
        wts = torch.as_tensor((w / w.mean()).astype(np.float32)).to(device)
    if model is None:
        x_mean, x_std = X.mean(0), X.std(0) + 1e-3
        model = CostModel(Mlp(IN_DIM, OUT_DIM, seed=seed, device=device), x_mean, x_std, Y.mean(0),
                          Y.std(0) + 1e-6)
    Xn = torch.as_tensor(model._norm(X)).to(device)
    Yn = torch.as_tensor(((Y - model.y_mean) / model.y_std).astype(np.float32)).to(device)
    rng = np.random.default_rng(seed)
    n = len(X)
    hist = []
    for ep in range(epochs):
        lr_ep = lr * 0.5 * (1.0 + np.cos(np.pi * ep / max(epochs, 1)))
        order = torch.as_tensor(rng.permutation(n)).to(device)
        losses = []
        for i in range(0, n, batch):
            idx = order[i:i + batch]
            losses.append(model.mlp.train_step(Xn[idx], Yn[idx], None if wts is None else wts[idx], lr=lr_ep,
                                               weight_decay=weight_decay))
        hist.append(float(torch.stack(losses).mean()))
        if log_every and ep % log_every == 0:
            print(f"epoch {ep} loss {hist[-1]:.4f}", flush=True)
    return model, hist


# ---------------------------------------------------------------------------
# solving
# ---------------------------------------------------------------------------
@dataclass
class LearnedResult:
    x: torch.Tensor
    config: PrecondConfig
    status: int
    iterations: int
    residual: float
    fallback: bool          # the FP64 LU produced x
    seconds_choose: float


def solve_with(series, cfg, K, b, tol=1e-8, max_iter=MAX_ITER, seed=0, x0=None):
    x, info, _ = kernels.solve_twolevel(series, n_landmarks=cfg.landmarks, block=cfg.block, tol=tol,
                                        max_iter=max_iter, K=K, b=b, seed=seed, policy=cfg.policy, prec=cfg.prec,
                                        x0=x0)
    return x, kernels.read_info(info)


def solve_plain_K(K, b):
    """FP64 LU solve of an already built system (K is not modified)."""
    f = kernels.lu_factor(K, GK_F64, overwrite=False)
    return kernels.lu_solve(f, b), kernels.read_info(f.info)


# FP32 configurations either converge quickly or stall at a large residual;
# at inference they get this iteration cap so a wrong pick costs little.
MAX_ITER_F32 = 400


def solve_learned(series, model, K=None, b=None, tol=1e-8, max_iter=MAX_ITER, config=None, x0=None):
    """Solve with the configuration the network ranks first (or ``config``).
    If FGMRES misses the tolerance with an FP32 configuration, the best-ranked
    FP64-storage configuration is tried next; the FP64 LU is the last resort.
    ``x0``: initial guess of FGMRES (e.g. the series' previous weights)."""
    if K is None:
        K, b = kernels.build(series, GK_F64)
    N = K.shape[0]
    t0 = time.perf_counter()
    if config is not None:
        ranked = [config]
    else:
        cands = candidates_for(N)
        if cands:
            feats = system_features(series).cpu().numpy()
            ranked = [cands[i] for i in np.argsort(model.expected_cost(feats, cands), kind="stable")]
        else:
            ranked = []
    t_choose = time.perf_counter() - t0
    tries = ranked[:1]
    if ranked and ranked[0].prec == GK_F32:
        tries += [c for c in ranked if c.prec != GK_F32][:1]
    cfg, inf, total_its = None, None, 0
    for cfg in tries:
        cap = min(max_iter, MAX_ITER_F32) if cfg.prec == GK_F32 else max_iter
        x, inf = solve_with(series, cfg, K, b, tol, cap, x0=x0)
        total_its += int(inf["iterations"])
        if int(inf["status"]) == 0:
            return LearnedResult(x, cfg, 0, total_its, float(inf["residual"]), False, t_choose)
    x, _ = solve_plain_K(K, b)
    return LearnedResult(x, cfg, int(inf["status"]) if inf is not None else 0, total_its,
                         float(inf["residual"]) if inf is not None else 0.0, True, t_choose)


def series_of(model, device="cuda"):
    """DeviceSeries of a single-series synthetic model."""
    ii, dd, ko = model.interpolation_input, model.data_descriptor, model.options.kernel_options
    return kernels.DeviceSeries(ii.orientations.dip_positions, ii.orientations.dip_gradients,
                                ii.orientations.nugget_effect_grad, ii.surface_points.sp_coords,
                                ii.surface_points.nugget_effect_scalar,
                                dd.tensors_structure.number_of_points_per_surface, range=ko.range, c_o=ko.c_o,
                                uni_degree=ko.uni_degree, kernel=ko.kernel_function, i_res=ko.i_res,
                                gi_res=ko.gi_res, device=device)


# ---------------------------------------------------------------------------
# training data
# ---------------------------------------------------------------------------
def _timed(fn):
    torch.cuda.synchronize()
    t = time.perf_counter()
    out = fn()
    torch.cuda.synchronize()
    return out, time.perf_counter() - t


def check_points(series, n=4096, seed=0):
    """Points where the LU solution's field is compared: uniform in the data's bounding box."""
    P = torch.cat([series.dip_positions, series.sp_coords]).cpu().numpy()
    lo, hi = P.min(0), P.max(0)
    xyz = np.random.default_rng(seed).uniform(lo, hi, (n, 3))
    return kernels.Points(xyz=torch.as_tensor(xyz).to(series.device))


def field_at(series, w, pts):
    f, _, _, _ = kernels.evaluate(series, kernels.prepare(series, w), pts, GK_F64)
    return f


def field_error(series, w, f_ref, pts):
    """max |field(w) - f_ref| / max |f_ref| at the check points."""
    f = field_at(series, w, pts)
    return float((f - f_ref).abs().max() / f_ref.abs().max())


def label_system(series, configs, tol=1e-8, max_iter=MAX_ITER, K=None, b=None):
    """Run every config on one system; the FP64 LU solution is the arbiter:
    a run counts as solved when FGMRES met the tolerance and its scalar field
    matches the LU solution's within LU_AGREEMENT_TOL (relative, at check_points).
    Returns (rows, lu_seconds)."""
    if K is None:
        K, b = kernels.build(series, GK_F64)
    (x_lu, inf_lu), t_lu = _timed(lambda: solve_plain_K(K, b))
    if int(inf_lu["status"]) != 0:
        raise RuntimeError("FP64 LU failed on a training system")
    pts = check_points(series)
    f_lu = field_at(series, x_lu, pts)
    rows = []
    for cfg in configs:
        (x, inf), t = _timed(lambda: solve_with(series, cfg, K, b, tol, max_iter))
        err = field_error(series, x, f_lu, pts) if int(inf["status"]) == 0 else float("inf")
        ok = int(inf["status"]) == 0 and err <= LU_AGREEMENT_TOL
        rows.append(dict(config=asdict(cfg), seconds=t, status=int(inf["status"]), iterations=int(inf["iterations"]),
                         residual=float(inf["residual"]), field_error_vs_lu=err, ok=ok,
                         cost_s=t if ok else t + t_lu))
    return rows, t_lu


def generate(n_systems, base_seed=0, configs_per_system=12, tol=1e-8, max_iter=MAX_ITER, n_min=1000, n_max=16000,
             seed=0, log=None):
    """Training data: ``n_systems`` systems of ``synthetic.training_system``,
    each labelled on a random subset of the candidates (all of them if
    configs_per_system <= 0)."""
    from . import synthetic
    rng = np.random.default_rng(seed)
    sys_feats, cfg_feats, cost, t_run, okl, t_lus, records = [], [], [], [], [], [], []
    for i in range(n_systems):
        m = synthetic.training_system(i, base_seed, n_min, n_max)
        s = series_of(m)
        N = s.N
        cands = candidates_for(N)
        if configs_per_system > 0 and len(cands) > configs_per_system:
            cands = [cands[j] for j in rng.choice(len(cands), configs_per_system, replace=False)]
        try:
            feats = system_features(s).cpu().numpy()
            rows, t_lu = label_system(s, cands, tol, max_iter)
        except (RuntimeError, _lib.GkError) as e:  # the FP64 LU itself failed: skip the system, keep going
            if log:
                log(f"system {i}: N={N} skipped ({e})")
            continue
        for r in rows:
            cfg = PrecondConfig(**r["config"])
            sys_feats.append(feats)
            cfg_feats.append(cfg.features())
            cost.append(r["cost_s"])
            t_run.append(r["seconds"])
            okl.append(float(r["ok"]))
            t_lus.append(t_lu)
        records.append(dict(index=i, N=N, lu_seconds=t_lu, meta={k: float(v) for k, v in m.meta.items()},
                            runs=rows))
        if log:
            best = min(rows, key=lambda r: r["cost_s"])
            log(f"system {i}: N={N} lu={t_lu:.3f}s best={best['config']} {best['cost_s']:.3f}s "
                f"ok={sum(r['ok'] for r in rows)}/{len(rows)}")
        del s, m
        torch.cuda.empty_cache()
    return dict(sys_feats=np.asarray(sys_feats, np.float32), cfg_feats=np.asarray(cfg_feats, np.float32),
                cost_s=np.asarray(cost, np.float64), t_run=np.asarray(t_run, np.float64),
                ok=np.asarray(okl, np.float64), t_lu=np.asarray(t_lus, np.float64)), records
