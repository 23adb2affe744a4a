"""Reverse-mode derivatives of the interpolation: the engine's autodiff path.

The reference differentiates ``compute_model`` with a PyTorch tape
(``compute_grads``), checks it against central differences at
test/test_modules/test_ad/test_ad_I.py:158-258 and drives its nugget
optimiser with it (gempy/modules/optimize_nuggets/_optimizer.py:9-62).  Here
the forward pass is the FP64 build, LU and evaluation kernels, and the
backward pass is the adjoint: one more solve with the same LU factors (the
kriging matrix is symmetric) and three kernels -- ``gk_adjoint_rhs``,
``gk_build_adjoint`` (dK/d(positions) from the build's own entry formulas on
dual numbers) and ``gk_eval_adjoint`` (the evaluation records at fixed
weights).  ``series_field`` is a ``torch.autograd.Function``: a field built
from it back-propagates into the surface-point coordinates and nuggets, the
orientation positions, gradients and nuggets, and the evaluation points.
The fault-drift functions of a faulted series (the blocks of the faults that
offset it) are treated as constants.
"""
from dataclasses import dataclass
from typing import Optional

import numpy as np
import torch

from . import kernels as K
from ._lib import GK_F64


@dataclass
class SeriesSpec:
    """What ``series_field`` does not differentiate: the surface counts, the
    kernel options and the fault blocks (at the surface points, and at the
    evaluation points)."""
    points_per_surface: np.ndarray
    range: float
    c_o: float
    uni_degree: int = 1
    kernel: str = "cubic"
    i_res: float = 4.0
    gi_res: float = 2.0
    fault_sp: Optional[torch.Tensor] = None       # (n_fault, n_sp)
    fault_values: Optional[torch.Tensor] = None   # (n_fault, n_points)


class _SeriesField(torch.autograd.Function):
    @staticmethod
    def forward(ctx, sp_coords, nugget_sp, dip_positions, dip_gradients, nugget_grad, xyz, spec):
        ds = K.DeviceSeries(dip_positions.detach(), dip_gradients.detach(), nugget_grad.detach(),
                            sp_coords.detach(), nugget_sp.detach(), spec.points_per_surface, range=spec.range,
                            c_o=spec.c_o, uni_degree=spec.uni_degree, kernel=spec.kernel, i_res=spec.i_res,
                            gi_res=spec.gi_res, device=sp_coords.device)
        if spec.fault_sp is not None:
            ds.set_fault_blocks(spec.fault_sp)
        Kd, b = K.build(ds, GK_F64)
        f = K.lu_factor(Kd, GK_F64, overwrite=True)
        w = K.lu_solve(f, b)
        model = K.prepare(ds, w)
        pts = K.Points(xyz=xyz.detach().to(torch.float64))
        need_x = ctx.needs_input_grad[5]
        z, g, _, _ = K.evaluate(ds, model, pts, GK_F64, gradient=need_x, fault_values=spec.fault_values)
        ctx.state = (ds, f, w, model, pts, g, spec)
        return z

    @staticmethod
    def backward(ctx, gz):
        ds, f, w, model, pts, g, spec = ctx.state
        gz = gz.to(torch.float64).contiguous()
        r = K.adjoint_rhs(ds, pts, gz, spec.fault_values)
        lam = K.lu_solve(f, r)
        d_sp, d_dip, d_nsp, d_ngr = K.build_adjoint(ds, lam, w)
        K.eval_adjoint(ds, model, pts, gz, d_sp, d_dip, spec.fault_values)
        n_o = ds.sys.n_ori
        d_dgr = lam[:3 * n_o].view(3, n_o).t()
        d_x = gz[:, None] * g if g is not None else None
        return d_sp, d_nsp, d_dip, d_dgr, d_ngr, d_x, None


def series_field(sp_coords, nugget_sp, dip_positions, dip_gradients, nugget_grad, xyz, spec: SeriesSpec):
    """Scalar field of one series at ``xyz`` (n, 3), FP64, differentiable with
    respect to every tensor argument (transformed frame)."""
    return _SeriesField.apply(sp_coords, nugget_sp, dip_positions, dip_gradients, nugget_grad, xyz, spec)
