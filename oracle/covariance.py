"""Isotropic covariance functions and the radial derivatives the co-kriging needs.

Restates the published GemPy covariances (GMD 2019, eqs. for the cubic model;
option ``kernel_function`` with values ``"cubic"`` / ``"exponential"`` as
serialized at ``test/test_modules/test_serialize_model.test_generate_horizontal_
stratigraphic_model.verify/Horizontal Stratigraphic Model serialization.approved.txt:127-139``).

For a radial covariance C(r) (unit sill; the caller multiplies by ``c_o``) each
function returns, for distance r and range a:

* ``C(r)``
* ``dC_r(r)  = C'(r) / r``                 (finite at r = 0)
* ``d2C(r)   = C''(r)``
* ``d3C_r(r) = d/dr (C'(r)/r) / r``        (only used for field gradients;
  multiplied by a factor that vanishes like r^2, so a finite value at r = 0 is
  all that is needed)

Cubic (compact support, zero beyond r >= a):
    C(r) = 1 - 7 s^2 + 35/4 s^3 - 7/2 s^5 + 3/4 s^7,  s = r/a.
"Exponential": the reference names a twice-differentiable kernel
"exponential"; its exact form lives in the absent engine.  The oracle uses the
squared-exponential C(r) = exp(-r^2 / (2 a^2)), the smooth kernel that satisfies
the twice-differentiability the gradient block needs.  (Unpinned convention.)
"""
import numpy as np

CUBIC = 0
EXPONENTIAL = 1


def kernel_id(name):
    name = str(name).lower()
    if name.startswith("cubic"):
        return CUBIC
    if name.startswith("exp"):
        return EXPONENTIAL
    raise ValueError(f"unsupported kernel_function {name!r}")


def cubic(r, a):
    s = r / a
    v = 1.0 - 7.0 * s**2 + 35.0 / 4.0 * s**3 - 7.0 / 2.0 * s**5 + 3.0 / 4.0 * s**7
    return np.where(r < a, v, 0.0)


def cubic_d1_r(r, a):
    v = (-14.0 / a**2 + 105.0 / 4.0 * r / a**3 - 35.0 / 2.0 * r**3 / a**5
         + 21.0 / 4.0 * r**5 / a**7)
    return np.where(r < a, v, 0.0)


def cubic_d2(r, a):
    v = (-14.0 / a**2 + 105.0 / 2.0 * r / a**3 - 70.0 * r**3 / a**5
         + 63.0 / 2.0 * r**5 / a**7)
    return np.where(r < a, v, 0.0)


def cubic_d3_r(r, a):
    # d/dr(C'/r) = 105/(4a^3) - 105 r^2/(2a^5) + 105 r^4/(4a^7); divided by r.
    with np.errstate(divide="ignore", invalid="ignore"):
        v = (105.0 / 4.0 / a**3 - 105.0 / 2.0 * r**2 / a**5
             + 105.0 / 4.0 * r**4 / a**7) / r
    return np.where((r < a) & (r > 0), v, 0.0)


def sqexp(r, a):
    return np.exp(-(r * r) / (2.0 * a * a))


def sqexp_d1_r(r, a):
    return -sqexp(r, a) / a**2


def sqexp_d2(r, a):
    return (r * r / a**4 - 1.0 / a**2) * sqexp(r, a)


def sqexp_d3_r(r, a):
    return sqexp(r, a) / a**4


def functions(kernel):
    """(C, C'/r, C'', (C'/r)'/r) for a kernel id."""
    if kernel == CUBIC:
        return cubic, cubic_d1_r, cubic_d2, cubic_d3_r
    if kernel == EXPONENTIAL:
        return sqexp, sqexp_d1_r, sqexp_d2, sqexp_d3_r
    raise ValueError(kernel)
