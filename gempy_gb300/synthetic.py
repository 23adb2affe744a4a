"""Seeded synthetic models with the shapes of the benchmark configurations.

The reference measures on no public suite; its test workloads are the example
models of ``gempy/API/examples_generator.py`` (horizontal strata
:132-162, anticline :165-195).  These generators produce models of the same
kind at the sizes of the five configurations this package is measured on:

* ``plain_horizontal``  two horizontal surfaces in a 1000^3 m cube (z = 400,
  600 m), 10 points each with N(0, 5 m) z jitter, 2 orientations (0,0,1),
  cubic kernel, range sqrt(3)*1000 m, c_o = range^2/14/3, nugget 1e-6,
  linear drift, 50^3 regular grid;
* ``folded_series``     3 series x 2 sinusoidally folded surfaces
  (z = z0 + A sin(2 pi x / lambda), A ~ U(50,150) m, lambda ~ U(300,800) m),
  200 points, 60 orientations (fold normals + N(0, 0.05)), quadratic drift,
  7 octree levels (128^3 effective);
* ``precision``         one series, 8 folded surfaces, 4000 points, 1500
  orientations (N = 8495 + 3), 256^3 regular grid;
* ``batch``             realisations with 50-2000 points (log-uniform) and
  10-600 orientations, positions + N(0, 10 m), normals + N(0, 0.05), 64^3 grid;
* ``learned``           20000 points / 6000 orientations on random multi-fold
  geometry (N ~ 38k).

Seeds follow the reference's test seed ``np.random.seed(1234)``
(``test/conftest.py:8``) through ``numpy.random.default_rng(1234 + index)``.
Range and c_o are given in metres as the reference's legacy defaults and
converted to the transformed frame (a_t = a * scale, c_o = a_t^2 / 14 / 3).
"""
from dataclasses import dataclass, field
from typing import List

import numpy as np

from .data import (EngineGrid, GenericGrid, InputDataDescriptor, InterpolationInput, InterpolationOptions,
                   Orientations, RegularGrid, StackRelationType, SurfacePoints)
from .transforms import Transform

EXTENT = np.array([0.0, 1000.0, 0.0, 1000.0, 0.0, 1000.0])


@dataclass
class SyntheticModel:
    name: str
    interpolation_input: InterpolationInput
    options: InterpolationOptions
    data_descriptor: InputDataDescriptor
    transform: Transform
    extent: np.ndarray
    sp_world: np.ndarray
    ori_world: np.ndarray
    meta: dict = field(default_factory=dict)

    @property
    def n_points(self):
        return len(self.sp_world)

    @property
    def n_orientations(self):
        return len(self.ori_world)


def _fold_surface(rng, n, z0, amp, lam, phase, jitter, extent=EXTENT):
    x = rng.uniform(extent[0], extent[1], n)
    y = rng.uniform(extent[2], extent[3], n)
    z = z0 + amp * np.sin(2 * np.pi * x / lam + phase) + rng.normal(0.0, jitter, n) if jitter else \
        z0 + amp * np.sin(2 * np.pi * x / lam + phase)
    return np.stack([x, y, z], 1)


def _fold_normals(x, amp, lam, phase, rng, noise):
    dz = amp * 2 * np.pi / lam * np.cos(2 * np.pi * x / lam + phase)
    g = np.stack([-dz, np.zeros_like(dz), np.ones_like(dz)], 1)
    g /= np.linalg.norm(g, axis=1, keepdims=True)
    if noise:
        g = g + rng.normal(0.0, noise, g.shape)
        g /= np.linalg.norm(g, axis=1, keepdims=True)
    return g


def _assemble(name, surfaces, orientations, grads, surfaces_per_series, relations, uni_degree,
              nug_sp=None, nug_ori=None, octree_levels=1, dense_res=None, custom=None, meta=None,
              range_m=np.sqrt(3) * 1000.0):
    sp_world = np.concatenate(surfaces)
    pps = np.array([len(s) for s in surfaces], dtype=np.int64)
    ori_world = np.concatenate(orientations)
    g = np.concatenate(grads)
    tr = Transform.from_input_points(sp_world, ori_world)
    a_t = range_m * tr.scale[0]
    c_o = a_t ** 2 / 14.0 / 3.0
    opts = InterpolationOptions.from_args(range=a_t, c_o=c_o, uni_degree=uni_degree,
                                          number_octree_levels=octree_levels)
    ext_t = tr.extent(EXTENT)
    octree = RegularGrid(ext_t, np.array([2, 2, 2])) if octree_levels >= 1 and dense_res is None else None
    dense = RegularGrid(ext_t, np.asarray(dense_res)) if dense_res is not None else None
    cust = GenericGrid(tr.apply(custom)) if custom is not None else None
    grid = EngineGrid(octree_grid=octree, dense_grid=dense, custom_grid=cust)
    n_sp = len(sp_world)
    n_o = len(ori_world)
    sp = SurfacePoints(tr.apply(sp_world), None if nug_sp is None else np.full(n_sp, nug_sp))
    ori = Orientations(tr.apply(ori_world), tr.transform_gradient(g), None if nug_ori is None else np.full(n_o, nug_ori))
    n_elem = len(surfaces)
    ii = InterpolationInput(sp, ori, grid, unit_values=np.arange(1, n_elem + 2, dtype=np.float64))
    # per-series orientation counts
    opst = np.array([len(o) for o in meta.pop("_ori_per_series")], dtype=np.int64)
    dd = InputDataDescriptor.from_arrays(pps, surfaces_per_series, opst, relations)
    return SyntheticModel(name, ii, opts, dd, tr, EXTENT.copy(), sp_world, ori_world, meta or {})


def plain_horizontal(seed=0, n_per_surface=10, resolution=(50, 50, 50)):
    rng = np.random.default_rng(1234 + seed)
    surfaces, oris, grads = [], [], []
    for z0 in (600.0, 400.0):  # stack order: top surface first
        xy = rng.uniform(0, 1000, (n_per_surface, 2))
        z = z0 + rng.normal(0, 5.0, n_per_surface)
        surfaces.append(np.column_stack([xy, z]))
    for z0 in (600.0, 400.0):
        oris.append(np.array([[rng.uniform(200, 800), rng.uniform(200, 800), z0]]))
        grads.append(np.array([[0.0, 0.0, 1.0]]))
    meta = {"_ori_per_series": [np.concatenate(oris)]}
    return _assemble("plain_horizontal", surfaces, oris, grads, [2], [StackRelationType.BASEMENT], 1,
                     nug_sp=1e-6, nug_ori=1e-6, dense_res=resolution, meta=meta)


def folded_series(seed=0, n_points=200, n_orient=60, octree_levels=7):
    rng = np.random.default_rng(1234 + seed)
    z0s = [(850.0, 750.0), (600.0, 500.0), (350.0, 250.0)]
    surfaces, oris, grads, per_series = [], [], [], []
    n_surf = 6
    counts = np.full(n_surf, n_points // n_surf)
    counts[: n_points - counts.sum()] += 1
    k = 0
    for s, pair in enumerate(z0s):
        amp, lam, ph = rng.uniform(50, 150), rng.uniform(300, 800), rng.uniform(0, 2 * np.pi)
        so = []
        for z0 in pair:
            surfaces.append(_fold_surface(rng, int(counts[k]), z0, amp, lam, ph, 0.0))
            k += 1
        n_o = n_orient // 3
        base = _fold_surface(rng, n_o, pair[0] - 50.0, amp, lam, ph, 0.0)
        oris.append(base)
        grads.append(_fold_normals(base[:, 0], amp, lam, ph, rng, 0.05))
        so.append(base)
        per_series.append(np.concatenate(so))
    meta = {"_ori_per_series": per_series}
    return _assemble("folded_series", surfaces, oris, grads, [2, 2, 2],
                     [StackRelationType.ERODE, StackRelationType.ERODE, StackRelationType.BASEMENT], 2,
                     octree_levels=octree_levels, meta=meta)


def precision(seed=0, n_points=4000, n_orient=1500, n_surf=8, resolution=(256, 256, 256)):
    rng = np.random.default_rng(1234 + seed)
    amp, lam, ph = rng.uniform(50, 150), rng.uniform(300, 800), rng.uniform(0, 2 * np.pi)
    z0s = np.linspace(850.0, 150.0, n_surf)
    counts = np.full(n_surf, n_points // n_surf)
    counts[: n_points - counts.sum()] += 1
    surfaces = [_fold_surface(rng, int(c), z0, amp, lam, ph, 0.0) for c, z0 in zip(counts, z0s)]
    which = rng.integers(0, n_surf, n_orient)
    base = np.concatenate([_fold_surface(rng, 1, z0s[w], amp, lam, ph, 0.0) for w in which])
    g = _fold_normals(base[:, 0], amp, lam, ph, rng, 0.05)
    meta = {"_ori_per_series": [base], "fold": (amp, lam, ph)}
    return _assemble("precision", surfaces, [base], [g], [n_surf], [StackRelationType.BASEMENT], 1,
                     dense_res=resolution, meta=meta)


def realisation(index, n_surf=4, resolution=(64, 64, 64), base_seed=0):
    """One realisation of the batched configuration."""
    rng = np.random.default_rng(1234 + base_seed * 100003 + index)
    n_p = int(np.exp(rng.uniform(np.log(50), np.log(2000))))
    n_o = int(np.exp(rng.uniform(np.log(10), np.log(600))))
    n_p = max(n_p, 2 * n_surf)
    amp, lam, ph = rng.uniform(50, 150), rng.uniform(300, 800), rng.uniform(0, 2 * np.pi)
    z0s = np.linspace(800.0, 200.0, n_surf)
    counts = np.full(n_surf, n_p // n_surf)
    counts[: n_p - counts.sum()] += 1
    surfaces = []
    for c, z0 in zip(counts, z0s):
        p = _fold_surface(rng, int(c), z0, amp, lam, ph, 0.0)
        surfaces.append(p + rng.normal(0.0, 10.0, p.shape))
    which = rng.integers(0, n_surf, n_o)
    base = np.concatenate([_fold_surface(rng, 1, z0s[w], amp, lam, ph, 0.0) for w in which])
    g = _fold_normals(base[:, 0], amp, lam, ph, rng, 0.05)
    base = base + rng.normal(0.0, 10.0, base.shape)
    meta = {"_ori_per_series": [base]}
    return _assemble(f"batch_{index}", surfaces, [base], [g], [n_surf], [StackRelationType.BASEMENT], 1,
                     dense_res=resolution, meta=meta)


def learned(seed=0, n_points=20000, n_orient=6000, n_surf=10, range_m=np.sqrt(3) * 1000.0, nug_sp=None,
            nug_ori=None):
    """Large multi-fold system (N ~ 38k) of the learned-preconditioner config."""
    rng = np.random.default_rng(1234 + seed)
    k = rng.uniform(1, 3, (3, 2)) * 2 * np.pi / 1000.0
    a = rng.uniform(20, 80, 3)
    ph = rng.uniform(0, 2 * np.pi, (3, 2))

    def zf(x, y, z0):
        return z0 + sum(a[i] * np.sin(k[i, 0] * x + ph[i, 0]) * np.cos(k[i, 1] * y + ph[i, 1]) for i in range(3))

    def grad(x, y):
        dzx = sum(a[i] * k[i, 0] * np.cos(k[i, 0] * x + ph[i, 0]) * np.cos(k[i, 1] * y + ph[i, 1]) for i in range(3))
        dzy = sum(-a[i] * k[i, 1] * np.sin(k[i, 0] * x + ph[i, 0]) * np.sin(k[i, 1] * y + ph[i, 1]) for i in range(3))
        g = np.stack([-dzx, -dzy, np.ones_like(dzx)], 1)
        return g / np.linalg.norm(g, axis=1, keepdims=True)

    z0s = np.linspace(900.0, 100.0, n_surf)
    counts = np.full(n_surf, n_points // n_surf)
    counts[: n_points - counts.sum()] += 1
    surfaces = []
    for c, z0 in zip(counts, z0s):
        x, y = rng.uniform(0, 1000, int(c)), rng.uniform(0, 1000, int(c))
        surfaces.append(np.stack([x, y, zf(x, y, z0)], 1))
    x, y = rng.uniform(0, 1000, n_orient), rng.uniform(0, 1000, n_orient)
    z = zf(x, y, z0s[rng.integers(0, n_surf, n_orient)])
    base = np.stack([x, y, z], 1)
    g = grad(x, y) + rng.normal(0, 0.05, (n_orient, 3))
    g /= np.linalg.norm(g, axis=1, keepdims=True)
    meta = {"_ori_per_series": [base]}
    return _assemble("learned", surfaces, [base], [g], [n_surf], [StackRelationType.BASEMENT], 1,
                     nug_sp=nug_sp, nug_ori=nug_ori, dense_res=(8, 8, 8), meta=meta, range_m=range_m)


def training_system(index, base_seed=0, n_min=1000, n_max=16000):
    """One system of the preconditioner-selection training distribution:
    random multi-fold geometry as ``learned`` with 1k-16k surface points
    (log-uniform), 10-40 % as many orientations, 3-12 surfaces, range
    0.5-1.5 x the default and surface-point nuggets 1e-7..1e-4 (log-uniform)."""
    rng = np.random.default_rng(7_000_003 + base_seed * 100_003 + index)
    n_p = int(np.exp(rng.uniform(np.log(n_min), np.log(n_max))))
    n_o = max(8, int(n_p * rng.uniform(0.1, 0.4)))
    n_s = int(rng.integers(3, 13))
    rm = np.sqrt(3) * 1000.0 * rng.uniform(0.5, 1.5)
    nug = float(np.exp(rng.uniform(np.log(1e-7), np.log(1e-4))))
    m = learned(seed=100_000 + base_seed * 100_003 + index, n_points=n_p, n_orient=n_o, n_surf=n_s, range_m=rm,
                nug_sp=nug)
    m.meta.update(dict(n_points=n_p, n_orient=n_o, n_surf=n_s, range_m=rm, nug_sp=nug))
    return m
