"""Batched realisations: many single-series models, each with its own 3-D
grid, built, solved, evaluated and segmented by the persistent kernels of
``gk_batch_run`` -- no host synchronisation inside, so the whole sequence is
captured once in a CUDA graph and replayed.

This is the GPU form of running the reference's ``compute_model``
(``gempy/API/compute_API.py:68-73``) once per stochastic realisation.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from ._lib import GK_MAX_SURFACES, GkBatch, GkBatchItem, check
from .kernels import _ptr, _stream, kernel_id, ref_rest_indices

INFO_DTYPE = np.dtype([("status", "<i4"), ("where", "<i4"), ("iterations", "<i4"), ("pivoted", "<i4"),
                       ("residual", "<f8")])


class BatchRunner:
    """Lays out a batch of models on the GPU.

    ``models``: objects with ``interpolation_input`` (one series, a dense
    regular grid), ``options`` and ``data_descriptor`` (e.g. the models of
    ``gempy_gb300.synthetic.realisation``).
    """

    def __init__(self, models, device="cuda", tol=1e-11, max_iter=60):
        self.device = torch.device(device)
        self.tol, self.max_iter = float(tol), int(max_iter)
        lib = _lib.load()
        n = len(models)
        items = (GkBatchItem * n)()
        dips, grads, nug_g, sps, nug_s, refs, rests = [], [], [], [], [], [], []
        o_off = s_off = i_off = 0
        self.points = []
        for i, m in enumerate(models):
            ii, opts, dd = m.interpolation_input, m.options, m.data_descriptor
            if dd.stack_structure.n_stacks != 1:
                raise ValueError("batched realisations are single-series models")
            ko = opts.kernel_options
            pps = np.asarray(dd.tensors_structure.number_of_points_per_surface, dtype=np.int64)
            if len(pps) > GK_MAX_SURFACES:
                raise ValueError(f"at most {GK_MAX_SURFACES} surfaces per realisation")
            ref, rest = ref_rest_indices(pps)
            sp, ori = ii.surface_points, ii.orientations
            g = ii.grid.dense_grid
            it = items[i]
            it.n_ori, it.n_sp, it.n_iface = len(ori.dip_positions), len(sp.sp_coords), len(ref)
            it.uni_degree, it.kernel, it.n_surf = int(ko.uni_degree), kernel_id(ko.kernel_function), len(pps)
            it.range, it.c_o, it.i_res, it.gi_res = float(ko.range), float(ko.c_o), float(ko.i_res), float(ko.gi_res)
            it.ori_offset, it.sp_offset, it.iface_offset = o_off, s_off, i_off
            for k, c in enumerate(pps):
                it.points_per_surface[k] = int(c)
            for k in range(3):
                it.dims[k] = int(g.regular_grid_shape[k])
                it.origin[k] = float(g.origin[k])
                it.spacing[k] = float(g.dxdydz[k])
            it.slope = float(opts.sigmoid_slope)
            uv = np.asarray(ii.unit_values, dtype=np.float64)
            for k in range(len(pps) + 1):
                it.unit_values[k] = float(uv[k])
            dips.append(ori.dip_positions); grads.append(ori.dip_gradients); nug_g.append(ori.nugget_effect_grad)
            sps.append(sp.sp_coords); nug_s.append(sp.nugget_effect_scalar); refs.append(ref); rests.append(rest)
            o_off += it.n_ori
            s_off += it.n_sp
            i_off += it.n_iface
            self.points.append(g.n_points)
        f64 = lambda xs, shape: torch.as_tensor(np.concatenate(xs).reshape(shape).astype(np.float64)).to(self.device)
        self.dip = f64(dips, (-1, 3))
        self.grad = f64(grads, (-1, 3))
        self.nug_g = f64(nug_g, (-1,))
        self.sp = f64(sps, (-1, 3))
        self.nug_s = f64(nug_s, (-1,))
        self.ref = torch.as_tensor(np.concatenate(refs).astype(np.int32)).to(self.device)
        self.rest = torch.as_tensor(np.concatenate(rests).astype(np.int32)).to(self.device)
        self.items = items
        self.batch = GkBatch()
        b = self.batch
        b.n_items = n
        b.items = ctypes.cast(items, ctypes.POINTER(GkBatchItem))
        b.dip_positions, b.dip_gradients, b.nugget_grad = self.dip.data_ptr(), self.grad.data_ptr(), self.nug_g.data_ptr()
        b.sp_coords, b.nugget_sp = self.sp.data_ptr(), self.nug_s.data_ptr()
        b.ref_index, b.rest_index = self.ref.data_ptr(), self.rest.data_ptr()
        self.work_bytes = lib.gk_batch_workspace_bytes(ctypes.byref(b))
        if self.work_bytes == 0:
            raise ValueError("invalid batch")
        self.work = torch.empty(self.work_bytes, dtype=torch.uint8, device=self.device)
        self.n_points = int(lib.gk_batch_points(ctypes.byref(b)))
        self.field = torch.empty(self.n_points, dtype=torch.float64, device=self.device)
        self.values = torch.empty(self.n_points, dtype=torch.float64, device=self.device)
        self.ids = torch.empty(self.n_points, dtype=torch.int32, device=self.device)
        self.infos = torch.zeros(n * 24, dtype=torch.uint8, device=self.device)
        self.offsets = np.concatenate([[0], np.cumsum(self.points)]).astype(np.int64)
        check("gk_batch_plan", lib.gk_batch_plan(ctypes.byref(b), _ptr(self.work), self.work_bytes, _stream()))
        self.graph = None
        self.n = n

    def run(self):
        lib = _lib.load()
        check("gk_batch_run", lib.gk_batch_run(ctypes.byref(self.batch), _ptr(self.work), self.work_bytes, self.tol,
                                               self.max_iter, _ptr(self.field), _ptr(self.values), _ptr(self.ids),
                                               _ptr(self.infos), _stream()))

    def capture(self):
        """Capture ``run`` in a CUDA graph (after one eager run for set-up)."""
        self.run()
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s):
                self.run()
        torch.cuda.current_stream().wait_stream(s)
        self.graph = g
        return g

    def replay(self):
        if self.graph is None:
            self.capture()
        self.graph.replay()

    def infos_host(self):
        return np.frombuffer(self.infos.cpu().numpy().tobytes(), dtype=INFO_DTYPE)

    def item_slice(self, i):
        return slice(int(self.offsets[i]), int(self.offsets[i + 1]))

    def results(self, i):
        """(weights, isovalues in stack order) of realisation i, as host arrays."""
        lib = _lib.load()
        it = self.items[i]
        N = 3 * it.n_ori + it.n_iface + {0: 0, 1: 3, 2: 9}[it.uni_degree]
        w = torch.empty(N, dtype=torch.float64, device=self.device)
        iso = torch.empty(max(it.n_surf, 1), dtype=torch.float64, device=self.device)
        check("gk_batch_results", lib.gk_batch_results(ctypes.byref(self.batch), _ptr(self.work), self.work_bytes, i,
                                                       _ptr(w), _ptr(iso), _stream()))
        return w.cpu().numpy(), iso.cpu().numpy()[: it.n_surf]
