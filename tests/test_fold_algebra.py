"""The polynomial split behind the float-float field kernel's per-tile folds
(``cta_fold_sums`` / ``tile_fold`` / ``ff_tile_col<NP, false, true>`` in
``gempy_gb300/csrc/gk_ff.cuh``), checked on the CPU against the oracle's
cubic covariance (``oracle/covariance.py``).

On a tile whose every point-record pair lies within the range the kernel
writes, with s = r / a,
  C(s)        = 1 - 7 s^2 + s^3 m(s),    m(s)   = 8.75 + s^2 (-3.5 + 0.75 s^2)
  a^2 C'(r)/r = -14 + s m_o(s),          m_o(s) = 26.25 + s^2 (-17.5 + 5.25 s^2)
and starts each point's accumulator at the tile's sum of the first two terms,
which are polynomials in the point x: about the centre o of the CTA's points,
  sum_i W_i (1 - 7 (|x - p_i|^2 + e)) = F0 - 7 (F0 (|x - o|^2 + e)
                                        - 2 (x - o) . F1 + F4),
  -14 sum_j w_j . (x_j - x)          = -14 (G0 - (x - o) . G1),
with F0 = sum W, F1 = sum W (p - o), F4 = sum W |p - o|^2, G0 = sum w . (x_j -
o), G1 = sum w.  The pairs then add W s^3 m(s) and s m_o(s) (w . (x_j - x)).
"""
import numpy as np

from oracle import covariance


def _m(s2):
    return 8.75 + s2 * (-3.5 + 0.75 * s2)


def _m_o(s2):
    return 26.25 + s2 * (-17.5 + 5.25 * s2)


def test_cubic_split_matches_the_oracle_covariances():
    a = 1.7
    r = np.linspace(0.0, a * 0.999, 4001)
    s = r / a
    np.testing.assert_allclose(1 - 7 * s**2 + s**3 * _m(s**2), covariance.cubic(r, a), rtol=0, atol=1e-14)
    np.testing.assert_allclose((-14 + s * _m_o(s**2)) / a**2, covariance.cubic_d1_r(r, a), rtol=0, atol=1e-12)


def test_tile_sums_reproduce_the_folded_terms():
    rng = np.random.default_rng(7)
    e = 1e-10
    p = rng.uniform(-0.4, 0.4, (1024, 3))          # surface-point records (scaled)
    W = rng.normal(scale=3e4, size=1024)           # large weights of both signs
    xo = rng.uniform(-0.4, 0.4, (512, 3))          # orientation records
    w = rng.normal(scale=1e2, size=(512, 3))
    x = rng.uniform(-0.05, 0.05, (64, 3)) + 0.1    # the CTA's points, around their centre
    o = 0.5 * (x.min(0) + x.max(0))
    F0, F1, F4 = W.sum(), (W[:, None] * (p - o)).sum(0), (W * ((p - o) ** 2).sum(1)).sum()
    G0, G1 = (w * (xo - o)).sum(), w.sum(0)
    for xi in x:
        d = xi - o
        direct = (W * (1 - 7 * (((xi - p) ** 2).sum(1) + e))).sum()
        folded = F0 - 7 * (F0 * (d @ d + e) - 2 * d @ F1 + F4)
        assert abs(folded - direct) <= 1e-12 * np.abs(W).sum()
        direct_o = -14 * (w * (xo - xi)).sum()
        folded_o = -14 * (G0 - d @ G1)
        assert abs(folded_o - direct_o) <= 1e-12 * np.abs(w).sum()
        # the whole in-range contribution: folded start + per-pair remainders
        r = np.sqrt(((xi - p) ** 2).sum(1) + e)
        s2 = r**2
        total = folded + (W * s2 * np.sqrt(s2) * _m(s2)).sum()
        ref = (W * covariance.cubic(r, 1.0)).sum()
        assert abs(total - ref) <= 1e-11 * np.abs(W).sum()
