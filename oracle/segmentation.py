"""Sigmoid segmentation of a series' scalar field and the series masks.

Restates the published segmentation (GMD 2019, "Block model"): each surface k
with isovalue z_k is a soft step of slope ``sigmoid_slope`` (5e6 by default,
``approved.txt:159``).  Surfaces are ordered by isovalue, highest first (the
element reordering of ``gempy/core/data/geo_model.py:123-127``); unit values
u_1.. u_m of that order plus u_(m+1) for the unit below the last surface give

    v(Z) = u_1 + sum_k (u_(k+1) - u_k) * sigma(slope * (z_(k) - Z)),
    sigma(t) = 1 / (1 + exp(-t)),

and ids = rint(v).  Element ids are ``1..n`` in stack order with the basement
last (``gempy/core/data/structural_frame.py:368-370``); the top surface maps to
id 1 (pinned by ``test/test_modules/test_grids/test_custom_grid.py:44-47``).

Block ids.  ids are the hard classification the soft values approach: a
point takes the unit of the highest surface it lies below,
    id(Z) = u_1 + sum_k (u_(k+1) - u_k) [Z < z_(k) - TIE_TOL],
which equals rint(v) except within TIE_TOL of an isovalue.  A point that lies
exactly on a surface -- an octree corner that coincides with a surface's
reference point, where Z == z_k up to rounding -- belongs to the unit above
it.  The reference's own result is set by its rounding at such ties; the
combination model (``test_example_models_I.py:71-88``, corner (0, 0, 250) m,
rock1's reference point) shows the unit above.

Series masks (``structural_frame.py:326-330``: the last group is forced to
BASEMENT): an ERODE series owns the points above its lowest isovalue; an ONLAP
series owns the points above the highest isovalue of the next (older) series;
BASEMENT owns everything; a FAULT series owns no lithology (its block offsets
the younger series through their fault drift); a younger series' points are
removed from all older ones.
"""
import numpy as np

ERODE, ONLAP, FAULT, BASEMENT = 1, 2, 3, 4
TIE_TOL = 1e-9     # field distance below which a point counts as on a surface


def sigmoid(t):
    t = np.asarray(t, dtype=np.float64)
    out = np.empty_like(t)
    pos = t >= 0
    out[pos] = 1.0 / (1.0 + np.exp(-t[pos]))
    e = np.exp(t[~pos])
    out[~pos] = e / (1.0 + e)
    return out


def order_surfaces(iso):
    """Surface order by isovalue, highest first (stable)."""
    return np.argsort(-np.asarray(iso), kind="stable")


def segment(Z, iso, unit_values, slope):
    """Soft values and ids for one series.

    unit_values: m+1 values -- the series' elements in stack order followed by
    the value of the unit below its last surface."""
    iso = np.asarray(iso, dtype=np.float64)
    u = np.asarray(unit_values, dtype=np.float64)
    order = order_surfaces(iso)
    zs = iso[order]
    v = np.full(np.shape(Z), u[0], dtype=np.float64)
    for k in range(len(zs)):
        v += (u[k + 1] - u[k]) * sigmoid(slope * (zs[k] - Z))
    return v, np.rint(v)


def hard_ids(Z, iso, unit_values, tol=None):
    """Block ids: the slope -> infinity limit of the soft values, a point on
    a surface (within ``tol``, default TIE_TOL) taking the unit above it."""
    tol = TIE_TOL if tol is None else tol
    iso = np.asarray(iso, dtype=np.float64)
    u = np.asarray(unit_values, dtype=np.float64)
    zs = iso[order_surfaces(iso)]
    v = np.full(np.shape(Z), u[0])
    for k in range(len(zs)):
        v += (u[k + 1] - u[k]) * (np.asarray(Z) < zs[k] - tol)
    return v


def series_masks(fields, isos, relations):
    """Squeezed masks (n_series, n): each point belongs to exactly one series."""
    n_s = len(fields)
    raw = []
    for s in range(n_s):
        rel = relations[s]
        if rel == BASEMENT or s == n_s - 1:
            raw.append(np.ones(np.shape(fields[s]), dtype=bool))
        elif rel == ERODE:
            raw.append(fields[s] >= np.min(isos[s]))
        elif rel == ONLAP:
            raw.append(fields[s + 1] >= np.max(isos[s + 1]))
        elif rel == FAULT:
            raw.append(np.zeros(np.shape(fields[s]), dtype=bool))
        else:
            raise ValueError(f"unknown relation {rel}")
    taken = np.zeros(np.shape(fields[0]), dtype=bool)
    out = []
    for s in range(n_s):
        m = raw[s] & ~taken
        out.append(m)
        taken |= m
    return np.stack(out)
