"""CPU oracle of the preconditioner-selection network (test infrastructure).

The reference has no learned component; this module restates, in float64
numpy, the computation the CUDA kernels of ``gk_mlp.cu`` perform, so their
forward pass, gradients, loss, optimizer step and geometry descriptor can be
checked.  The oracle's own gradient is checked against central finite
differences in the tests, following the reference's FD-vs-AD template
(``test/test_modules/test_ad/test_ad_I.py:158-258``).

Network: in_dim -> 256 -> 256 -> out_dim, ReLU between layers.  Parameters
are one flat array; per layer a row-major (n_out, n_in + 1) block whose last
column is the bias.  Weights live in BF16 (round-to-nearest-even of the FP32
master copy).
"""
import numpy as np

HIDDEN = 256


def layer_shapes(in_dim, out_dim):
    return [(HIDDEN, in_dim), (HIDDEN, HIDDEN), (out_dim, HIDDEN)]


def param_count(in_dim, out_dim):
    return sum(n * (k + 1) for n, k in layer_shapes(in_dim, out_dim))


def bf16_bits(x):
    """Round float32 values to bfloat16 (nearest, ties to even); uint16 bits."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    rounding = ((u >> 16) & 1) + 0x7FFF
    return ((u + rounding) >> 16).astype(np.uint16)


def bf16_value(bits):
    return (np.asarray(bits, dtype=np.uint16).astype(np.uint32) << 16).view(np.float32)


def unpack(flat, in_dim, out_dim):
    """[(W, b)] per layer (float64 views of the flat parameter array)."""
    flat = np.asarray(flat, dtype=np.float64)
    out, o = [], 0
    for n, k in layer_shapes(in_dim, out_dim):
        blk = flat[o:o + n * (k + 1)].reshape(n, k + 1)
        out.append((blk[:, :k], blk[:, k]))
        o += n * (k + 1)
    return out


def forward(flat, x, in_dim, out_dim):
    """(y, cache) for x (batch, in_dim)."""
    layers = unpack(flat, in_dim, out_dim)
    h = np.asarray(x, dtype=np.float64)
    acts = [h]
    for li, (W, b) in enumerate(layers):
        z = h @ W.T + b
        h = np.maximum(z, 0.0) if li < 2 else z
        acts.append(h)
    return h, acts


def forward_bf16_activations(flat, x, in_dim, out_dim):
    """Forward pass with the layer inputs rounded to BF16 (nearest even), as
    the tensor-core inference kernel feeds them to the MMA; sums in float64."""
    layers = unpack(flat, in_dim, out_dim)
    h = np.asarray(x, dtype=np.float64)
    for li, (W, b) in enumerate(layers):
        h = bf16_value(bf16_bits(h.astype(np.float32))).astype(np.float64)
        z = h @ W.T + b
        h = np.maximum(z, 0.0) if li < 2 else z
    return h


def backward(flat, acts, dy, in_dim, out_dim):
    """Gradient of sum(dy * y) with respect to the flat parameters."""
    layers = unpack(flat, in_dim, out_dim)
    grads = []
    d = np.asarray(dy, dtype=np.float64)
    for li in (2, 1, 0):
        W, _ = layers[li]
        h_in = acts[li]
        gW = d.T @ h_in
        gb = d.sum(0)
        grads.append(np.concatenate([gW, gb[:, None]], 1).ravel())
        if li > 0:
            d = (d @ W) * (acts[li] > 0)
    return np.concatenate(grads[::-1])


def mse(y, t, w=None):
    """Weighted MSE sum_i w_i |y_i - t_i|^2 / sum_i w_i and its gradient."""
    y = np.asarray(y, dtype=np.float64)
    t = np.asarray(t, dtype=np.float64)
    w = np.ones(len(y)) if w is None else np.asarray(w, dtype=np.float64)
    W = w.sum()
    d = y - t
    loss = float((w[:, None] * d * d).sum() / W)
    return loss, 2.0 * w[:, None] * d / W


def adam(master, grad, m, v, lr, beta1, beta2, eps, weight_decay, step):
    """AdamW step (bias-corrected moments, decoupled decay); float64 arrays."""
    m = beta1 * m + (1 - beta1) * grad
    v = beta2 * v + (1 - beta2) * grad * grad
    mh = m / (1 - beta1 ** step)
    vh = v / (1 - beta2 ** step)
    master = master - lr * (mh / (np.sqrt(vh) + eps) + weight_decay * master)
    return master, m, v


def system_features(dip_positions, dip_gradients, nugget_grad, sp_coords, nugget_sp, n_iface, uni_degree, rng):
    """Geometry descriptor of one system (16 values), same definition as the
    ``gk_system_features`` kernel."""
    n_ori, n_sp = len(dip_positions), len(sp_coords)
    nd = {0: 0, 1: 3, 2: 9}[uni_degree]
    N = 3 * n_ori + n_iface + nd
    P = np.concatenate([np.asarray(dip_positions, float).reshape(-1, 3), np.asarray(sp_coords, float).reshape(-1, 3)])
    ext = P.max(0) - P.min(0)
    sd = np.sqrt(np.maximum((P * P).mean(0) - P.mean(0) ** 2, 0.0))
    g = np.asarray(dip_gradients, float).reshape(-1, 3)
    gn = g / np.linalg.norm(g, axis=1, keepdims=True)
    f = np.zeros(16)
    f[0] = np.log(N) / 10
    f[1] = 3 * n_ori / N
    f[2] = n_iface / N
    f[3:6] = ext / rng
    f[6:9] = sd / rng
    f[9] = np.linalg.norm(gn.sum(0)) / n_ori
    f[10] = np.abs(gn[:, 2]).mean()
    f[11] = np.log10(np.maximum(nugget_sp, 1e-30)).mean() / 10
    f[12] = np.log10(np.maximum(nugget_grad, 1e-30)).mean() / 10
    f[13] = uni_degree / 2
    vol = np.prod(np.maximum(ext, 1e-3 * rng))
    f[14] = np.log(np.cbrt(vol / len(P)) / rng) / 5
    f[15] = np.log(1.0 + (n_sp - n_iface)) / 5
    return f
