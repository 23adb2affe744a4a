"""Forward gravity: the engine's geophysics step on the GPU.

``calculate_gravity_gradient(centered_grid)`` mirrors the reference's
``gp.calculate_gravity_gradient`` (imported at ``gempy/API/__init__.py:65``,
used at ``test/test_modules/test_geophysics/test_gravity.py:67-80``): the
vertical attraction tz of every kernel voxel per unit density, computed by
``gk_gravity_tz``.  ``compute_model`` turns ``geophysics_input`` into
``Solutions.gravity``: it evaluates and segments every series at the centred
grid's points and reduces density x tz per device with ``gk_gravity``.
"""
import numpy as np
import torch

from . import kernels as K


def calculate_gravity_gradient(centered_grid, device="cuda"):
    """tz (n_voxels,) of a ``CenteredGrid`` in its own units (lengths in m:
    mGal per g/cm^3), as a host array."""
    c = torch.as_tensor(centered_grid.kernel_grid_centers, dtype=torch.float64).to(device)
    lo = torch.as_tensor(centered_grid.left_voxel_edges, dtype=torch.float64).to(device)
    hi = torch.as_tensor(centered_grid.right_voxel_edges, dtype=torch.float64).to(device)
    return K.gravity_tz(c, lo, hi).cpu().numpy()


def _host(a):
    if isinstance(a, torch.Tensor):
        return a.detach().to(dtype=torch.float64)
    return torch.as_tensor(np.asarray(a, dtype=np.float64))


def device_gravity(lith_ids, centered_grid, geophysics_input, device):
    """gravity per device from the lithology ids of the centred grid's points
    (device tensor, device-major) and the input's tz and densities."""
    tz = _host(geophysics_input.tz).to(device).reshape(-1)
    if tz.numel() != centered_grid.n_voxels:
        raise ValueError(f"tz has {tz.numel()} values for a kernel of {centered_grid.n_voxels} voxels")
    rho = _host(geophysics_input.densities).to(device).reshape(-1)
    return K.gravity(lith_ids, centered_grid.n_devices, rho, tz)
