"""Surface meshes of the structural elements, extracted on the GPU.

Mirrors the reference's mesh module ``gempy/modules/mesh_extranction/
marching_cubes.py``: ``set_meshes_with_marching_cubes`` (``:12-56``) walks the
series of a dense-grid solution and extracts, for every element of a series,
the level surface of the series' dense-grid field at the element's isovalue,
masked by the series' squeezed mask (every point for a FAULT series);
``extract_mesh_for_element`` (``:59-101``) makes one mesh and shifts its
vertices by the extent minimum.  The reference calls scikit-image's
marching cubes there; here every mesh comes from ``gk_mc_count`` and
``gk_mc_emit`` (``include/gempy_gb300.h``), whose vertex rule reproduces the
reference's vertex counts (``test/test_modules/test_marching_cubes.py:44-47``).
"""
from dataclasses import dataclass
from typing import List, Optional

import numpy as np
import torch

from . import kernels as K
from .data import StackRelationType


@dataclass
class ElementMesh:
    """``vertices`` (n_v x 3) and ``edges`` (n_t x 3 vertex ids), the two
    arrays the reference stores on its StructuralElement (``marching_cubes.py:
    100-101``)."""
    vertices: np.ndarray
    edges: np.ndarray


def _device_tensor(a, dtype):
    if isinstance(a, torch.Tensor):
        return a.to(device="cuda", dtype=dtype)
    return torch.as_tensor(np.ascontiguousarray(a)).to(device="cuda", dtype=dtype)


def grid_shape_and_extent(regular_grid):
    """(resolution, extent) of this package's RegularGrid or of a grid with
    the reference's ``resolution`` / ``extent`` attributes."""
    res = getattr(regular_grid, "regular_grid_shape", None)
    if res is None:
        res = regular_grid.resolution
    ext = getattr(regular_grid, "orthogonal_extent", None)
    if ext is None:
        ext = regular_grid.extent
    res = [int(v) for v in res]
    ext = np.asarray(ext, dtype=np.float64)
    return res, ext, (ext[1::2] - ext[0::2]) / np.asarray(res, dtype=np.float64)


def extract_mesh_for_element(scalar_field, level: float, regular_grid, mask: Optional[np.ndarray] = None,
                             to_host: bool = True):
    """One element's mesh: the ``level`` surface of ``scalar_field`` (the dense
    grid's points in ``ij`` order), vertices at grid index x spacing plus the
    extent minimum (``marching_cubes.py:86-98``)."""
    res, ext, spacing = grid_shape_and_extent(regular_grid)
    f = _device_tensor(scalar_field, torch.float64).reshape(-1)
    m = None if mask is None else _device_tensor(mask, torch.uint8).reshape(-1)
    verts, faces = K.marching_cubes(f, res, level, spacing, ext[0::2], m)
    if to_host:
        return ElementMesh(verts.cpu().numpy(), faces.cpu().numpy())
    return ElementMesh(verts, faces)


def set_meshes_with_marching_cubes(solutions, regular_grid, data_descriptor) -> List[List[ElementMesh]]:
    """Meshes of every element, per series (``marching_cubes.py:12-56``).

    ``solutions`` must hold dense-grid results (``raw_arrays.
    scalar_field_matrix`` and ``mask_matrix_squeezed``), as ``compute_model``
    returns for a grid with a ``dense_grid``; the isovalues are the series'
    ``scalar_field_at_surface_points``."""
    raw = solutions.raw_arrays
    if raw is None or raw.scalar_field_matrix is None:
        raise ValueError("Model solutions must contain dense grid data for mesh extraction.")
    ss = data_descriptor.stack_structure
    out = []
    for s in range(ss.n_stacks):
        if s >= len(raw.scalar_field_matrix):
            continue
        field = raw.scalar_field_matrix[s]
        fault = ss.masking_descriptor[s] == StackRelationType.FAULT
        mask = None if fault else raw.mask_matrix_squeezed[s]
        isos = solutions.root_output.outputs[s].exported_fields.scalar_field_at_surface_points
        out.append([extract_mesh_for_element(field, float(level), regular_grid, mask) for level in isos])
    return out
