"""FP64 restatement of the co-kriging system: build, solve, evaluate.

Follows the published method (GemPy 1.0, GMD 12:1-32, section "Interpolation
of the potential field"), with the input conventions of the reference's engine
adapter ``gempy/modules/data_manipulation/_engine_factory.py:27-56``
(``sp_coords``, ``nugget_effect_scalar``, ``dip_positions``, ``dip_gradients``,
``nugget_effect_grad``) and the kernel options serialized at
``...Horizontal Stratigraphic Model serialization.approved.txt:127-139``
(``range``, ``c_o``, ``uni_degree``, ``i_res``, ``gi_res``, ``kernel_function``).

Unknown ordering of one series (n_o orientations, n_k surfaces, n_p points):

* gradient unknowns, component-major: index ``u * n_o + o`` (u = x, y, z);
* interface unknowns: surfaces in input order; within a surface its first
  point is the reference point and every other point ("rest") gives one row;
  n_i = n_p - n_k;
* drift unknowns: uni_degree 1 -> (x, y, z); uni_degree 2 -> additionally
  (x^2, y^2, z^2, xy, xz, yz); uni_degree 0 -> none;
* fault-drift unknowns: one per older FAULT series that offsets this one
  (``fault_relations[j, i]``, ``gempy/core/data/structural_frame.py:244-273``).
  Its drift function F_f is that fault series' block -- its sigmoid-segmented
  values -- so the column holds gi_res (F_f(rest_i) - F_f(ref_i)) on the
  interface rows and 0 on the gradient rows (a block is piecewise constant).

Matrix entries (c_o = sill, C = unit covariance, h = x_a - x_b, r = |h|):

* GG[(u,o),(v,q)] = c_o [h_u h_v / (r^2 + 1e-5) (C'/r - C'') - delta_uv C'/r
                           + delta nugget_grad[o]]
* GI[(u,o), i]    = gi_res c_o [C'/r(x_o,rest_i)(x_o-rest_i)_u
                                - C'/r(x_o,ref_i)(x_o-ref_i)_u]
* II[i,j]         = c_o [i_res (C(rest_i,rest_j) - C(rest_i,ref_j)
                                - C(ref_i,rest_j) + C(ref_i,ref_j)) + delta nugget[rest_i]]
* UG[(u,o), d]    = d f_d / d x_u at x_o;  UI[i, d] = gi_res (f_d(rest_i) - f_d(ref_i))
* FI[i, f]        = gi_res (F_f(rest_i) - F_f(ref_i));  FG = 0
* rhs: b[(u,o)] = G[o, u]; zero elsewhere.

With the defaults i_res = gi_res^2 (4 and 2) the interface rows are a symmetric
diagonal rescaling of the textbook system.

Field at x:  Z(x) = gi_res * ( sum_(u,o) w c_o C'/r(x_o,x) (x_o - x)_u
                   + sum_i gi_res w_i c_o [C(x,rest_i) - C(x,ref_i)] + sum_d mu_d f_d(x)
                   + sum_f nu_f F_f(x) )

Distances.  Every distance is r = sqrt(|h|^2 + DIST_EPS2), DIST_EPS2 = 1e-10
(transformed frame).  The reference runs its kernel under PyTorch autodiff
with respect to the point and orientation positions and asserts finite
gradients (``test/test_modules/test_ad/test_ad_I.py:48-54``); a bare sqrt at
the r = 0 diagonal entries would make them NaN, so the engine's distances
carry a regulariser.  It matters through the linear term of C'/r at r = 0:
the gradient-gradient diagonal moves by c_o 105/4 sqrt(DIST_EPS2) / a^3.

How these conventions were pinned.  The engine that holds them is absent.
The 1e-5 regulariser of the gradient-gradient term, the nuggets inside the
``c_o`` factor (orientation 0.01 -> 0.1, interface 2e-5 -> 2e-4), the
placement of ``i_res``/``gi_res`` and the drift scaling are each pinned
sharply by the reference's approval file ``test/test_model_types/
test_example_models_I.test_generate_fold_model.Anticline Scalar Field.
approved.txt`` (51 values of the finest octree level of the anticline): a
factor 2 on either nugget, a drift scale other than gi_res, or a regulariser
other than 1e-5 each moves the field by 1e-4 to 1e-1.  DIST_EPS2 is the one
continuous constant the same file selects (its optimum is 9e-11; 1e-10 is
used).  With these values all 51 values pass the reference's comparator
``np.allclose(rtol=1e-5, atol=1e-5)`` (``test/verify_helper.py:70-103``),
max |error| 3.2e-6.  The fault and combination models' approval files
(``test_example_models_I.py:56-88``) check the same conventions on inputs
that were not used to choose them.
"""
from dataclasses import dataclass, field

import numpy as np
import scipy.linalg

from .covariance import functions, kernel_id

GRAD_EPS = 1e-5     # regulariser of h_u h_v / r^2 in the gradient-gradient block
DIST_EPS2 = 1e-10   # every distance is sqrt(|h|^2 + DIST_EPS2)


@dataclass
class Series:
    """One series' transformed inputs (numpy FP64) and kernel options."""
    dip_positions: np.ndarray            # (n_o, 3)
    dip_gradients: np.ndarray            # (n_o, 3)
    nugget_grad: np.ndarray              # (n_o,)
    sp_coords: np.ndarray                # (n_p, 3), grouped by surface
    nugget_sp: np.ndarray                # (n_p,)
    points_per_surface: np.ndarray       # (n_k,)
    range: float = 1.7
    c_o: float = 10.0
    uni_degree: int = 1
    kernel: str = "cubic"
    i_res: float = 4.0
    gi_res: float = 2.0
    fault_sp: np.ndarray = None          # (n_p, n_f) fault-block values at the points
    ref_rest: tuple = field(default=None, repr=False)

    @property
    def n_o(self):
        return int(self.dip_positions.shape[0])

    @property
    def n_p(self):
        return int(self.sp_coords.shape[0])

    @property
    def n_k(self):
        return int(len(self.points_per_surface))

    @property
    def n_d(self):
        return {0: 0, 1: 3, 2: 9}[int(self.uni_degree)]

    @property
    def n_i(self):
        return self.n_p - self.n_k

    @property
    def n_f(self):
        return 0 if self.fault_sp is None else int(np.shape(self.fault_sp)[1])

    @property
    def size(self):
        return 3 * self.n_o + self.n_i + self.n_d + self.n_f

    def ref_rest_index(self):
        """(ref_idx, rest_idx) arrays of length n_i; ref = first point of its surface."""
        if self.ref_rest is None:
            ref, rest = [], []
            start = 0
            for n in np.asarray(self.points_per_surface, dtype=np.int64):
                n = int(n)
                for j in range(start + 1, start + n):
                    ref.append(start)
                    rest.append(j)
                start += n
            self.ref_rest = (np.asarray(ref, dtype=np.int64), np.asarray(rest, dtype=np.int64))
        return self.ref_rest


def drift_values(x, degree):
    """f_d(x) for all drift functions, shape (n, n_d)."""
    x = np.atleast_2d(x)
    if degree == 0:
        return np.zeros((x.shape[0], 0))
    cols = [x[:, 0], x[:, 1], x[:, 2]]
    if degree == 2:
        cols += [x[:, 0] ** 2, x[:, 1] ** 2, x[:, 2] ** 2,
                 x[:, 0] * x[:, 1], x[:, 0] * x[:, 2], x[:, 1] * x[:, 2]]
    return np.stack(cols, axis=1)


def drift_gradients(x, degree):
    """d f_d / d x_u, shape (n, 3, n_d)."""
    x = np.atleast_2d(x)
    n = x.shape[0]
    nd = {0: 0, 1: 3, 2: 9}[degree]
    g = np.zeros((n, 3, nd))
    if nd == 0:
        return g
    for u in range(3):
        g[:, u, u] = 1.0
    if degree == 2:
        for u in range(3):
            g[:, u, 3 + u] = 2.0 * x[:, u]
        g[:, 0, 6] = x[:, 1]; g[:, 1, 6] = x[:, 0]   # xy
        g[:, 0, 7] = x[:, 2]; g[:, 2, 7] = x[:, 0]   # xz
        g[:, 1, 8] = x[:, 2]; g[:, 2, 8] = x[:, 1]   # yz
    return g


def _dist(a, b):
    d = a[:, None, :] - b[None, :, :]
    return d, np.sqrt((d * d).sum(-1) + DIST_EPS2)


def build_system(s: Series):
    """Dense K (N x N) and rhs b (N,) in FP64."""
    C, dC_r, d2C, _ = functions(kernel_id(s.kernel))
    a, c_o = float(s.range), float(s.c_o)
    n_o, n_i, n_d, n_f = s.n_o, s.n_i, s.n_d, s.n_f
    ng = 3 * n_o
    N = ng + n_i + n_d + n_f
    K = np.zeros((N, N))
    ref_idx, rest_idx = s.ref_rest_index()
    ref = s.sp_coords[ref_idx]
    rest = s.sp_coords[rest_idx]
    xo = s.dip_positions

    # GG block
    h, r = _dist(xo, xo)                               # (n_o, n_o, 3)
    k1 = dC_r(r, a)
    k2 = d2C(r, a)
    f = (k1 - k2) / (r * r + GRAD_EPS)
    for u in range(3):
        for v in range(3):
            blk = h[..., u] * h[..., v] * f
            if u == v:
                blk = blk - k1
            K[u * n_o:(u + 1) * n_o, v * n_o:(v + 1) * n_o] = c_o * blk
    K[np.arange(ng), np.arange(ng)] += c_o * np.tile(s.nugget_grad, 3)

    # GI block
    if n_i:
        hr, rr = _dist(xo, rest)
        hf, rf = _dist(xo, ref)
        gi = (dC_r(rr, a)[..., None] * hr - dC_r(rf, a)[..., None] * hf) * (s.gi_res * c_o)
        Kgi = gi.transpose(2, 0, 1).reshape(ng, n_i)
        K[:ng, ng:ng + n_i] = Kgi
        K[ng:ng + n_i, :ng] = Kgi.T
        # II block
        cc = lambda p, q: C(_dist(p, q)[1], a)
        Kii = (cc(rest, rest) - cc(rest, ref) - cc(ref, rest) + cc(ref, ref)) * (s.i_res * c_o)
        Kii[np.arange(n_i), np.arange(n_i)] += c_o * s.nugget_sp[rest_idx]
        K[ng:ng + n_i, ng:ng + n_i] = Kii

    # drift
    if n_d:
        UG = drift_gradients(xo, s.uni_degree)          # (n_o, 3, n_d)
        UG = UG.transpose(1, 0, 2).reshape(ng, n_d)
        K[:ng, ng + n_i:ng + n_i + n_d] = UG
        K[ng + n_i:ng + n_i + n_d, :ng] = UG.T
        if n_i:
            UI = (drift_values(rest, s.uni_degree) - drift_values(ref, s.uni_degree)) * s.gi_res
            K[ng:ng + n_i, ng + n_i:ng + n_i + n_d] = UI
            K[ng + n_i:ng + n_i + n_d, ng:ng + n_i] = UI.T

    # fault drift
    if n_f and n_i:
        F = np.asarray(s.fault_sp, dtype=np.float64)
        FI = (F[rest_idx] - F[ref_idx]) * s.gi_res
        K[ng:ng + n_i, ng + n_i + n_d:] = FI
        K[ng + n_i + n_d:, ng:ng + n_i] = FI.T

    b = np.zeros(N)
    b[:ng] = s.dip_gradients.T.reshape(-1)
    return K, b


def solve(K, b):
    """Dense LU with partial pivoting (LAPACK getrf/getrs), the reference's
    direct solver choice ``kernel_solver: 1`` (approved options JSON :136)."""
    lu, piv = scipy.linalg.lu_factor(K, check_finite=True)
    return scipy.linalg.lu_solve((lu, piv), b)


def point_coefficients(s: Series, w):
    """Per-unique-surface-point weights alpha_p with
    sum_i w_i [C(x,rest_i) - C(x,ref_i)] * gi_res = sum_p alpha_p C(x, p)."""
    ref_idx, rest_idx = s.ref_rest_index()
    ng = 3 * s.n_o
    wi = w[ng:ng + s.n_i] * s.gi_res
    alpha = np.zeros(s.n_p)
    np.add.at(alpha, rest_idx, wi)
    np.add.at(alpha, ref_idx, -wi)
    return alpha


def evaluate(s: Series, w, x, gradient=False, chunk=200_000, fault_x=None):
    """Scalar field (and gradient) at points x (n, 3); chunked like the
    reference's ``evaluation_chunk_size``.  ``fault_x`` (n, n_f) holds the
    offsetting faults' block values at x (required when the series has fault
    drift); the block is piecewise constant, so it adds nothing to the gradient."""
    C, dC_r, _, d3C_r = functions(kernel_id(s.kernel))
    a, c_o = float(s.range), float(s.c_o)
    x = np.atleast_2d(np.asarray(x, dtype=np.float64))
    n = x.shape[0]
    ng = 3 * s.n_o
    wg = w[:ng].reshape(3, s.n_o).T                   # (n_o, 3)
    mu = w[ng + s.n_i:ng + s.n_i + s.n_d]
    nu = w[ng + s.n_i + s.n_d:]
    if s.n_f:
        if fault_x is None:
            raise ValueError("the series has fault drift: fault block values at x are required")
        fault_x = np.asarray(fault_x, dtype=np.float64).reshape(n, s.n_f)
    alpha = point_coefficients(s, w)
    Z = np.empty(n)
    G = np.empty((n, 3)) if gradient else None
    chunk = max(256, min(chunk, 20_000_000 // max(1, s.n_o + s.n_p)))   # bound temporaries
    for c0 in range(0, n, chunk):
        xc = x[c0:c0 + chunk]
        h, r = _dist(s.dip_positions, xc)              # h = x_o - x, (n_o, m, 3)
        k1 = dC_r(r, a)
        wh = np.einsum("omu,ou->om", h, wg)
        z = c_o * (k1 * wh).sum(0)
        hp, rp = _dist(xc, s.sp_coords)                # x - p, (m, n_p, 3)
        z += c_o * (C(rp, a) * alpha[None, :]).sum(1)
        if len(mu):
            z += drift_values(xc, s.uni_degree) @ mu
        if s.n_f:
            z += fault_x[c0:c0 + chunk] @ nu
        Z[c0:c0 + chunk] = s.gi_res * z
        if gradient:
            k3 = d3C_r(r, a)
            g = -c_o * (np.einsum("om,omu->mu", k3 * wh, h) + np.einsum("om,ou->mu", k1, wg))
            g += c_o * np.einsum("mp,mpu->mu", dC_r(rp, a) * alpha[None, :], hp)
            if len(mu):
                g += np.einsum("mud,d->mu", drift_gradients(xc, s.uni_degree), mu)
            G[c0:c0 + chunk] = s.gi_res * g
    return (Z, G) if gradient else Z


def reference_starts(s: Series):
    return np.concatenate([[0], np.cumsum(s.points_per_surface)[:-1]]).astype(np.int64)


def isovalues(s: Series, w):
    """Scalar field at each surface's reference (first) point
    (``scalar_field_at_surface_points``, ``gempy/core/data/geo_model.py:107-108``)."""
    starts = reference_starts(s)
    fx = None if s.fault_sp is None else np.asarray(s.fault_sp)[starts]
    return evaluate(s, w, s.sp_coords[starts], fault_x=fx)
