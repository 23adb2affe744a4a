"""Marching-cubes mesh extraction on the GPU (``gk_mc_count`` / ``gk_mc_emit``)
against the oracle's restatement (``oracle/mesh.py``), and the reference's
vertex counts of the combination model
(``test/test_modules/test_marching_cubes.py:13-47``).  Vertices, triangles
and their order are integer/index work plus one interpolation per vertex done
with the same rounded operations, so the comparison is bit-exact."""
import collections

import numpy as np
import pytest

from oracle import mesh as omesh

from tests._models import engine_inputs_from_golden, load_golden

pytestmark = pytest.mark.gpu


def _gpu_mesh(F, dims, level, spacing=(1.0, 1.0, 1.0), origin=(0.0, 0.0, 0.0), mask=None):
    import torch

    from gempy_gb300 import kernels as K
    f = torch.as_tensor(np.ascontiguousarray(F, dtype=np.float64).reshape(-1)).cuda()
    m = None if mask is None else torch.as_tensor(np.asarray(mask, dtype=np.uint8).reshape(-1)).cuda()
    v, t = K.marching_cubes(f, dims, level, spacing, origin, m)
    return v.cpu().numpy(), t.cpu().numpy()


def _wobbly_sphere(n, r):
    ax = np.arange(n, dtype=np.float64)
    X, Y, Z = np.meshgrid(ax, ax, ax, indexing="ij")
    c = (n - 1) / 2 + 0.31
    return np.sqrt((X - c) ** 2 + (Y - c + 0.17) ** 2 + (Z - c - 0.23) ** 2) + 0.8 * np.sin(0.9 * X) * np.cos(0.7 * Y)


def _closed_and_oriented(faces):
    """Every directed mesh edge once, with its reverse present: a closed,
    consistently oriented surface."""
    E = collections.Counter()
    for t in faces:
        for i in range(3):
            E[(int(t[i]), int(t[(i + 1) % 3]))] += 1
    return all(c == 1 and E.get((b, a), 0) == 1 for (a, b), c in E.items()), len(E) // 2


@pytest.mark.parametrize("seed,dims,masked", [(0, (9, 7, 8), False), (1, (17, 13, 11), True),
                                              (2, (1, 5, 5), False), (3, (24, 3, 30), True)])
def test_random_volume_matches_oracle_bitwise(seed, dims, masked):
    rng = np.random.default_rng(seed)
    F = rng.normal(0.0, 1.0, dims)
    mask = rng.random(dims) < 0.7 if masked else None
    sp, org = (0.5, 0.25, 2.0), (-1.0, 3.0, 0.125)
    v, t = _gpu_mesh(F, dims, 0.1, sp, org, mask)
    vo, to = omesh.marching_cubes(F, dims, 0.1, sp, org, mask)
    np.testing.assert_array_equal(v, vo)
    np.testing.assert_array_equal(t, to)


def test_closed_surface_is_manifold_and_matches_oracle():
    n = 24
    F = _wobbly_sphere(n, 7.5)
    v, t = _gpu_mesh(F, (n, n, n), 7.5)
    vo, to = omesh.marching_cubes(F, (n, n, n), 7.5)
    np.testing.assert_array_equal(v, vo)
    np.testing.assert_array_equal(t, to)
    ok, n_edges = _closed_and_oriented(t)
    assert ok
    assert len(v) - n_edges + len(t) == 2          # Euler characteristic of a sphere


def test_empty_and_degenerate_volumes():
    F = np.zeros((6, 5, 4))
    v, t = _gpu_mesh(F, F.shape, 1.0)                 # the level is never crossed
    assert v.shape == (0, 3) and t.shape == (0, 3)
    F = np.random.default_rng(4).normal(size=(8, 8, 8))
    v, t = _gpu_mesh(F, F.shape, 0.0, mask=np.zeros(F.shape, bool))   # nothing processed
    assert v.shape == (0, 3) and t.shape == (0, 3)


def test_full_size_surface_is_closed():
    """A 256^3 closed surface (the precision workload's grid size): the mesh
    is closed and consistently oriented, Euler characteristic 2, and the
    vertices lie on grid edges at the level of the linear interpolant."""
    n = 256
    ax = np.arange(n, dtype=np.float64)
    X, Y, Z = np.meshgrid(ax, ax, ax, indexing="ij")
    F = np.sqrt((X - 127.3) ** 2 + (Y - 128.1) ** 2 + (Z - 126.7) ** 2)
    v, t = _gpu_mesh(F, (n, n, n), 100.0)
    # edge key of every triangle edge, counted with orientation
    a = t.astype(np.int64)
    e = np.concatenate([a[:, [0, 1]], a[:, [1, 2]], a[:, [2, 0]]])
    key = e[:, 0] * len(v) + e[:, 1]
    rkey = e[:, 1] * len(v) + e[:, 0]
    u, c = np.unique(key, return_counts=True)
    assert (c == 1).all()
    assert np.isin(rkey, u).all()
    assert len(v) - len(u) // 2 + len(t) == 2
    r = np.sqrt(((v - [127.3, 128.1, 126.7]) ** 2).sum(1))
    assert np.abs(r - 100.0).max() < 0.01     # linear interpolation of a distance field


def test_combination_model_vertex_counts_match_reference():
    """The combination model (fault, eroding series, basement series) on the
    40 x 20 x 20 dense grid of the reference's test: the vertex counts of its
    four elements are the reference's 600, 860, 1256 and 1680, and each mesh
    equals the oracle's restatement on the same field bit for bit."""
    import gempy_gb300 as gg
    from gempy_gb300 import mesh
    g = load_golden("combination_model.json")
    ii, opts, dd, ext = engine_inputs_from_golden(g)
    rg = gg.RegularGrid(ext, [40, 20, 20])
    ii.grid = gg.EngineGrid(dense_grid=rg)
    opts = gg.InterpolationOptions.init_dense_grid_options()
    sol = gg.compute_model(ii, opts, dd)
    meshes = mesh.set_meshes_with_marching_cubes(sol, rg, dd)
    counts = [len(m.vertices) for ms in meshes for m in ms]
    assert counts == [600, 860, 1256, 1680]
    raw = sol.raw_arrays
    res, ext, spacing = mesh.grid_shape_and_extent(rg)
    for s, ms in enumerate(meshes):
        fault = dd.stack_structure.masking_descriptor[s] == gg.StackRelationType.FAULT
        isos = sol.root_output.outputs[s].exported_fields.scalar_field_at_surface_points
        for level, m in zip(isos, ms):
            vo, to = omesh.marching_cubes(raw.scalar_field_matrix[s], res, level, spacing, ext[0::2],
                                          None if fault else raw.mask_matrix_squeezed[s])
            np.testing.assert_array_equal(m.vertices, vo)
            np.testing.assert_array_equal(m.edges, to)
