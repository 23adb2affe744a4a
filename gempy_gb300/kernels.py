"""Thin Python wrappers over the C ABI (``include/gempy_gb300.h``).

Device memory, streams and host<->device copies come from PyTorch (plumbing
only); every computation is a call into ``libgempy_gb300.so``.  Tensors passed
in must be CUDA tensors; nothing here runs on the CPU.
"""
import contextlib
import ctypes
import threading
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from ._lib import GK_F32, GK_F64, GK_FF, GkPoints, GkSegment, GkSystem, check

INFO_DTYPE = np.dtype([("status", "<i4"), ("where", "<i4"), ("iterations", "<i4"), ("pivoted", "<i4"),
                       ("residual", "<f8")])


_tuned = False


_local = threading.local()


def _stream():
    global _tuned
    if not _tuned:
        from . import autotune
        autotune.ensure_applied()
        _tuned = True
    h = getattr(_local, "stream", None)
    if h is not None:
        return h
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


@contextlib.contextmanager
def on_current_stream():
    """Within the block every library call of this thread goes to the stream
    that is current on entry (looked up once instead of per call)."""
    prev = getattr(_local, "stream", None)
    _local.stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    try:
        yield
    finally:
        _local.stream = prev


def _ptr(t):
    return ctypes.c_void_p(0 if t is None else t.data_ptr())


def new_info(device):
    return torch.zeros(24, dtype=torch.uint8, device=device)


def read_info(info):
    return np.frombuffer(info.cpu().numpy().tobytes(), dtype=INFO_DTYPE)[0]


def kernel_id(name):
    name = getattr(name, "value", name)
    name = str(name).lower()
    if name.startswith("cubic"):
        return _lib.GK_KERNEL_CUBIC
    if name.startswith("exp"):
        return _lib.GK_KERNEL_EXPONENTIAL
    raise ValueError(f"unsupported kernel_function {name!r}")


def ref_rest_indices(points_per_surface):
    """Interface rows: per surface, its first point is the reference point and
    each other point gives one row (rest)."""
    ref, rest = [], []
    start = 0
    for n in np.asarray(points_per_surface, dtype=np.int64):
        n = int(n)
        ref.extend([start] * max(n - 1, 0))
        rest.extend(range(start + 1, start + n))
        start += n
    return np.asarray(ref, dtype=np.int32), np.asarray(rest, dtype=np.int32)


class DeviceSeries:
    """One series' inputs resident on the GPU, with its ``gk_system``."""

    def __init__(self, dip_positions, dip_gradients, nugget_grad, sp_coords, nugget_sp, points_per_surface,
                 range, c_o, uni_degree=1, kernel="cubic", i_res=4.0, gi_res=2.0, device="cuda",
                 ref_index=None, rest_index=None, ref_points=None):
        """Inputs are numpy arrays (uploaded here) or CUDA tensors already on
        ``device`` (used as they are); ``ref_index``/``rest_index``/``ref_points``
        may be given precomputed (device tensors) to avoid further uploads."""
        dev = torch.device(device)

        def f64(a, shape=None):
            if isinstance(a, torch.Tensor):
                t = a.to(device=dev, dtype=torch.float64)
            else:
                t = torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64)).to(dev)
            t = t.reshape(shape) if shape is not None else t
            return t.contiguous()

        self.points_per_surface = np.asarray(points_per_surface, dtype=np.int64)
        self.dip_positions = f64(dip_positions, (-1, 3))
        self.dip_gradients = f64(dip_gradients, (-1, 3))
        self.nugget_grad = f64(nugget_grad)
        self.sp_coords = f64(sp_coords, (-1, 3))
        self.nugget_sp = f64(nugget_sp)
        if ref_index is None or rest_index is None:
            ref, rest = ref_rest_indices(self.points_per_surface)
            ref_index, rest_index = torch.as_tensor(ref).to(dev), torch.as_tensor(rest).to(dev)
        self.ref_index = ref_index
        self.rest_index = rest_index
        n_iface = int(ref_index.shape[0])
        if ref_points is None:
            starts = np.concatenate([[0], np.cumsum(self.points_per_surface)[:-1]]).astype(np.int64)
            ref_points = self.sp_coords[torch.as_tensor(starts).to(dev)].contiguous() \
                if len(starts) else self.sp_coords[:0]
        self.ref_points = ref_points
        self.device = dev
        self.sys = GkSystem()
        s = self.sys
        s.n_ori = int(self.dip_positions.shape[0])
        s.n_sp = int(self.sp_coords.shape[0])
        s.n_iface = n_iface
        s.uni_degree = int(uni_degree)
        s.kernel = kernel_id(kernel)
        s.range, s.c_o, s.i_res, s.gi_res = float(range), float(c_o), float(i_res), float(gi_res)
        s.dip_positions = self.dip_positions.data_ptr()
        s.dip_gradients = self.dip_gradients.data_ptr()
        s.nugget_grad = self.nugget_grad.data_ptr()
        s.sp_coords = self.sp_coords.data_ptr()
        s.nugget_sp = self.nugget_sp.data_ptr()
        s.ref_index = self.ref_index.data_ptr()
        s.rest_index = self.rest_index.data_ptr()
        self.fault_sp = None
        s.n_fault = 0
        s.fault_sp = 0

    def set_fault_blocks(self, fault_sp):
        """Fault-drift functions of this series: the blocks of the faults that
        offset it at its surface points, an (n_fault, n_sp) FP64 CUDA tensor
        (row f: fault f's soft segmented values)."""
        if fault_sp is None or len(fault_sp) == 0:
            self.fault_sp = None
            self.sys.n_fault = 0
            self.sys.fault_sp = 0
            return
        f = fault_sp.to(device=self.device, dtype=torch.float64).contiguous()
        if f.dim() != 2 or f.shape[1] != self.sys.n_sp:
            raise ValueError("fault blocks must be (n_fault, n_sp)")
        if f.shape[0] > _lib.GK_MAX_FAULTS:
            raise ValueError(f"at most {_lib.GK_MAX_FAULTS} faults offset one series")
        self.fault_sp = f
        self.sys.n_fault = int(f.shape[0])
        self.sys.fault_sp = f.data_ptr()

    @property
    def n_faults(self):
        return int(self.sys.n_fault)

    @property
    def n_surfaces(self):
        return len(self.points_per_surface)

    @property
    def N(self):
        return int(_lib.load().gk_system_size(ctypes.byref(self.sys)))


def leading_dim(n, prec):
    align = 32 if prec == GK_F64 else 64
    return (n + align - 1) // align * align


# largest covariance-table workspace of the FP64 build (gk_build_tables)
BUILD_TABLES_MAX_BYTES = 16 << 30


def build(series: DeviceSeries, prec=GK_F64, tables=True):
    """K (N x ld) and rhs.  FP64 builds use the covariance tables
    (gk_build_tables) when their workspace is at most BUILD_TABLES_MAX_BYTES;
    ``tables=False`` forces the direct build (gk_build)."""
    lib = _lib.load()
    N = series.N
    ld = leading_dim(N, prec)
    dt = torch.float64 if prec == GK_F64 else torch.float32
    K = torch.empty((N, ld), dtype=dt, device=series.device)
    b = torch.empty(N, dtype=dt, device=series.device)
    wb = lib.gk_build_tables_bytes(ctypes.byref(series.sys)) if (tables and prec == GK_F64) else 0
    if 0 < wb <= BUILD_TABLES_MAX_BYTES:
        work = torch.empty(wb, dtype=torch.uint8, device=series.device)
        check("gk_build_tables", lib.gk_build_tables(ctypes.byref(series.sys), _ptr(K), ld, _ptr(b), _ptr(work), wb,
                                                     _stream()))
    else:
        check("gk_build", lib.gk_build(ctypes.byref(series.sys), prec, _ptr(K), ld, _ptr(b), _stream()))
    return K, b


@dataclass
class LUFactors:
    LU: torch.Tensor
    ipiv: torch.Tensor
    work: torch.Tensor
    prec: int
    n: int
    info: torch.Tensor


def lu_factor(A, prec=None, overwrite=False):
    """In-place blocked LU with partial pivoting of a row-major (n, ld) tensor."""
    lib = _lib.load()
    if prec is None:
        prec = GK_F64 if A.dtype == torch.float64 else GK_F32
    n = A.shape[0]
    LU = A if overwrite else A.clone()
    ipiv = torch.empty(n, dtype=torch.int32, device=A.device)
    wb = lib.gk_lu_workspace_bytes(prec, n)
    work = torch.empty(wb, dtype=torch.uint8, device=A.device)
    info = new_info(A.device)
    check("gk_lu_factor", lib.gk_lu_factor(prec, n, _ptr(LU), LU.stride(0), _ptr(ipiv), _ptr(work), wb,
                                           _ptr(info), _stream()))
    return LUFactors(LU, ipiv, work, prec, n, info)


def lu_solve(f: LUFactors, b):
    lib = _lib.load()
    x = b.clone()
    check("gk_lu_solve", lib.gk_lu_solve(f.prec, f.n, _ptr(f.LU), f.LU.stride(0), _ptr(f.ipiv), _ptr(x),
                                         _ptr(f.work), f.work.numel(), _ptr(f.info), _stream()))
    return x


def solve_plain(series: DeviceSeries):
    """FP64 build + FP64 blocked LU + FP64 triangular solves."""
    K, b = build(series, GK_F64)
    f = lu_factor(K, GK_F64, overwrite=True)
    w = lu_solve(f, b)
    return w, f.info


def solve_mixed(series: DeviceSeries, tol=1e-12, max_iter=30, K=None, b=None):
    """FP64 build, FP32 LU of the equilibrated matrix, FP64 refinement."""
    lib = _lib.load()
    if K is None:
        K, b = build(series, GK_F64)
    n = K.shape[0]
    wb = lib.gk_solve_mixed_workspace_bytes(n)
    work = torch.empty(wb, dtype=torch.uint8, device=K.device)
    x = torch.empty(n, dtype=torch.float64, device=K.device)
    info = new_info(K.device)
    check("gk_solve_mixed", lib.gk_solve_mixed(n, _ptr(K), K.stride(0), _ptr(b), _ptr(x), float(tol),
                                               int(max_iter), _ptr(work), wb, _ptr(info), _stream()))
    return x, info


def solve_mixed_cta(series: DeviceSeries, tol=1e-12, max_iter=60, K=None, b=None):
    """The mixed solve of a small system (N <= GK_CTA_MAX_N) in one thread
    block: one launch, no host synchronisation; (x, info)."""
    lib = _lib.load()
    if K is None:
        K, b = build(series, GK_F64)
    n = K.shape[0]
    wb = lib.gk_solve_mixed_cta_workspace_bytes(n, K.stride(0))
    if wb == 0:
        raise ValueError(f"system of {n} unknowns is above GK_CTA_MAX_N")
    work = torch.empty(wb, dtype=torch.uint8, device=K.device)
    x = torch.empty(n, dtype=torch.float64, device=K.device)
    info = new_info(K.device)
    check("gk_solve_mixed_cta", lib.gk_solve_mixed_cta(n, _ptr(K), K.stride(0), _ptr(b), _ptr(x), float(tol),
                                                       int(max_iter), _ptr(work), wb, _ptr(info), _stream()))
    return x, info


def solve_mixed_cta_many(systems, tol=1e-12, max_iter=60):
    """Small independent systems ``[(K, b), ...]`` solved in one launch (one
    thread block each, ``gk_solve_mixed_cta_many``); [(x, info), ...]."""
    lib = _lib.load()
    out, jobs, keep = [], [], []
    for K, b in systems:
        n = K.shape[0]
        wb = lib.gk_solve_mixed_cta_workspace_bytes(n, K.stride(0))
        if wb == 0:
            raise ValueError(f"system of {n} unknowns is above GK_CTA_MAX_N")
        work = torch.empty(wb, dtype=torch.uint8, device=K.device)
        x = torch.empty(n, dtype=torch.float64, device=K.device)
        info = new_info(K.device)
        jobs.append(_lib.GkCtaJob(n, K.data_ptr(), K.stride(0), b.data_ptr(), x.data_ptr(), work.data_ptr(), wb,
                                  info.data_ptr()))
        keep.append(work)
        out.append((x, info))
    for c0 in range(0, len(jobs), _lib.GK_CTA_MAX_JOBS):
        chunk = jobs[c0:c0 + _lib.GK_CTA_MAX_JOBS]
        arr = (_lib.GkCtaJob * len(chunk))(*chunk)
        check("gk_solve_mixed_cta_many", lib.gk_solve_mixed_cta_many(len(chunk), arr, float(tol), int(max_iter),
                                                                     _stream()))
    return out


def gemv(K, x):
    """y = K x (FP64, on the GPU)."""
    lib = _lib.load()
    n = K.shape[0]
    x = x.contiguous()
    y = torch.empty(n, dtype=torch.float64, device=K.device)
    check("gk_gemv", lib.gk_gemv(n, _ptr(K), K.stride(0), _ptr(x), _ptr(y), _stream()))
    return y


def condition_number(K, factors=None, iters=60, seed=0):
    """2-norm condition number of the symmetric FP64 matrix K: the largest
    |eigenvalue| by power iteration on K, the smallest by inverse iteration
    with the FP64 LU (``factors``, computed from a copy when not given)."""
    n = K.shape[0]
    g = torch.Generator(device="cpu").manual_seed(seed)
    v = torch.randn(n, generator=g, dtype=torch.float64).to(K.device)
    v /= torch.linalg.vector_norm(v)
    big = 0.0
    for _ in range(iters):
        w = gemv(K, v)
        big = float(torch.linalg.vector_norm(w))
        v = w / big
    f = factors if factors is not None else lu_factor(K, GK_F64, overwrite=False)
    v = torch.randn(n, generator=g, dtype=torch.float64).to(K.device)
    v /= torch.linalg.vector_norm(v)
    inv_small = 0.0
    for _ in range(iters):
        w = lu_solve(f, v)
        inv_small = float(torch.linalg.vector_norm(w))
        v = w / inv_small
    return big * inv_small


def unknown_positions(series: DeviceSeries):
    """Position of every unknown: orientation position for gradient rows, rest
    point for interface rows (drift rows: the centroid)."""
    xo = series.dip_positions.cpu().numpy()
    sp = series.sp_coords.cpu().numpy()
    rest = series.rest_index.cpu().numpy()
    nd = series.N - 3 * len(xo) - len(rest)
    pos = np.concatenate([np.tile(xo, (3, 1)), sp[rest], np.repeat(sp.mean(0, keepdims=True), nd, 0)])
    return pos, nd


def morton_codes(p):
    p = np.asarray(p, dtype=np.float64)
    q = ((p - p.min(0)) / (np.ptp(p, 0) + 1e-300) * 1023).astype(np.int64)
    code = np.zeros(len(p), dtype=np.int64)
    for bit in range(10):
        for d in range(3):
            code |= ((q[:, d] >> bit) & 1) << (3 * bit + d)
    return code


LANDMARK_POLICIES = ("random", "stratified")


def twolevel_permutation(series: DeviceSeries, n_landmarks, seed=0, policy="random"):
    """(perm, r): r = landmark count rounded up to a multiple of 64 (covariance
    unknowns plus every drift unknown) placed first, the other unknowns after
    them in Morton (Z-curve) order of their positions.  ``policy`` picks the
    covariance landmarks: "random" samples them uniformly, "stratified" takes
    every k-th unknown along the Morton curve (an even spatial spread) from a
    seeded offset."""
    if policy not in LANDMARK_POLICIES:
        raise ValueError(f"unknown landmark policy {policy!r}")
    pos, nd = unknown_positions(series)
    N = len(pos)
    nc = N - nd
    r = int(min(max(64, -(-(int(n_landmarks) + nd) // 64) * 64), (N - 1) // 64 * 64))
    rng = np.random.default_rng(seed)
    nl = r - nd
    if policy == "random":
        land = np.sort(rng.choice(nc, nl, replace=False))
    else:
        order = np.argsort(morton_codes(pos[:nc]), kind="stable")
        step = nc / nl
        idx = np.minimum((rng.uniform(0, step) + step * np.arange(nl)).astype(np.int64), nc - 1)
        land = np.sort(order[idx])
    mask = np.ones(N, dtype=bool)
    mask[land] = False
    mask[nc:] = False
    rest = np.nonzero(mask)[0]
    rest = rest[np.argsort(morton_codes(pos[rest]), kind="stable")]
    perm = np.concatenate([land, np.arange(nc, N), rest]).astype(np.int32)
    return perm, r


def solve_twolevel(series: DeviceSeries, n_landmarks=1024, block=512, tol=1e-8, max_iter=2000, K=None, b=None,
                   seed=0, policy="random", prec=None, x0=None):
    """FGMRES with the two-level (block-Jacobi + low-rank) preconditioner;
    ``prec`` is the preconditioner's arithmetic: GK_F32, GK_FF (FP64 storage,
    float-float updates) or GK_F64 (the default); ``x0`` an initial guess."""
    lib = _lib.load()
    prec = GK_F64 if prec is None else int(prec)
    if K is None:
        K, b = build(series, GK_F64)
    n = K.shape[0]
    perm, r = twolevel_permutation(series, n_landmarks, seed, policy)
    pt = torch.as_tensor(perm).to(K.device)
    wb = lib.gk_solve_twolevel_workspace_bytes(n, prec)
    work = torch.empty(wb, dtype=torch.uint8, device=K.device)
    x = torch.empty(n, dtype=torch.float64, device=K.device)
    info = new_info(K.device)
    if x0 is not None:
        x0 = x0.to(device=K.device, dtype=torch.float64).contiguous()
        if x0.shape != (n,):
            raise ValueError("initial guess has the wrong size")
    check("gk_solve_twolevel", lib.gk_solve_twolevel(n, _ptr(K), K.stride(0), _ptr(b), _ptr(x), _ptr(x0), _ptr(pt), r,
                                                     int(block), prec, float(tol), int(max_iter), _ptr(work), wb,
                                                     _ptr(info), _stream()))
    return x, info, r


def prepare(series: DeviceSeries, w):
    lib = _lib.load()
    nb = lib.gk_eval_model_bytes(ctypes.byref(series.sys))
    model = torch.empty(nb, dtype=torch.uint8, device=series.device)
    check("gk_eval_prepare", lib.gk_eval_prepare(ctypes.byref(series.sys), _ptr(w), _ptr(model), _stream()))
    return model


class Points:
    """Evaluation point set: a regular grid generated in the kernel, or a list."""

    def __init__(self, xyz=None, origin=None, spacing=None, dims=None):
        self.gk = GkPoints()
        if xyz is not None:
            self.xyz = xyz.contiguous()
            self.gk.kind = 1
            self.gk.n = int(self.xyz.shape[0])
            self.gk.xyz = self.xyz.data_ptr()
        else:
            self.xyz = None
            self.gk.kind = 0
            for i in range(3):
                self.gk.dims[i] = int(dims[i])
                self.gk.origin[i] = float(origin[i])
                self.gk.spacing[i] = float(spacing[i])
            self.gk.n = int(np.prod([int(d) for d in dims]))

    @property
    def n(self):
        return int(self.gk.n)

    @classmethod
    def regular(cls, grid):
        return cls(origin=grid.origin, spacing=grid.dxdydz, dims=grid.regular_grid_shape)


def make_segment(isovalues_sorted, unit_values, slope):
    seg = GkSegment()
    m = len(isovalues_sorted)
    if m > _lib.GK_MAX_SURFACES:
        raise ValueError(f"at most {_lib.GK_MAX_SURFACES} surfaces per series")
    seg.n_surf = m
    seg.slope = float(slope)
    for i, v in enumerate(isovalues_sorted):
        seg.isovalues[i] = float(v)
    for i, v in enumerate(unit_values):
        seg.unit_values[i] = float(v)
    return seg


def evaluate(series: DeviceSeries, model, pts: Points, prec=GK_F64, seg=None, gradient=False, want_field=True,
             want_values=True, want_ids=False, out=None, fault_values=None, info=None):
    """Field (gradient, soft values, block ids) of one series at ``pts``;
    ``fault_values`` (n_fault, n) holds the blocks of the faults that offset
    the series at these points (required when it has fault drift); ``info``
    an optional gk_info tensor (``new_info``) for device-side failures."""
    lib = _lib.load()
    n = pts.n
    if series.n_faults:
        if fault_values is None or tuple(fault_values.shape) != (series.n_faults, n):
            raise ValueError("this series has fault drift: pass its faults' blocks at the points, (n_fault, n)")
        fault_values = fault_values.contiguous()
        pts.gk.fault_values = fault_values.data_ptr()
        pts.gk.fault_ld = n
    else:
        pts.gk.fault_values = 0
        pts.gk.fault_ld = 0
    dev = series.device
    o = out or {}
    field = o.get("field") if want_field else None
    if want_field and field is None:
        field = torch.empty(n, dtype=torch.float64, device=dev)
    grad = torch.empty((n, 3), dtype=torch.float64, device=dev) if gradient else None
    values = None
    ids = None
    if seg is not None and want_values:
        values = o.get("values")
        if values is None:
            values = torch.empty(n, dtype=torch.float64, device=dev)
    if seg is not None and want_ids:
        ids = o.get("ids")
        if ids is None:
            ids = torch.empty(n, dtype=torch.int32, device=dev)
    check("gk_eval", lib.gk_eval(ctypes.byref(series.sys), _ptr(model), ctypes.byref(pts.gk), prec,
                                 ctypes.byref(seg) if seg is not None else None, _ptr(field), _ptr(grad),
                                 _ptr(values), _ptr(ids), _ptr(info), _stream()))
    return field, grad, values, ids


class SeriesSet:
    """The series of one model prepared for ``gk_eval_series_set``: one
    ``gk_series_eval`` per series (system, packed model, segmentation,
    relation, fault sources, extreme isovalues), built once and reused for
    every point set."""

    def __init__(self, items):
        """items: (DeviceSeries, model, GkSegment, relation, fault_sources, min_iso, max_iso) per series."""
        n = len(items)
        if not 1 <= n <= _lib.GK_MAX_SURFACES:
            raise ValueError("1 .. GK_MAX_SURFACES series")
        self.items = items
        self.arr = (_lib.GkSeriesEval * n)()
        for i, (ds, model, seg, rel, faults, mn, mx) in enumerate(items):
            e = self.arr[i]
            e.sys = ctypes.pointer(ds.sys)
            e.model = model.data_ptr()
            e.seg = seg
            e.relation = int(rel)
            e.n_faults = len(faults)
            for f, j in enumerate(faults):
                e.faults[f] = int(j)
            e.min_iso, e.max_iso = float(mn), float(mx)
        self.n = n
        self.device = items[0][0].device

    def set_slope(self, slope):
        for i in range(self.n):
            self.arr[i].seg.slope = float(slope)

    def evaluate(self, pts: Points, prec, combine=True, info=None):
        """fields, values, ids (n_series x n), block, lith ids, masks."""
        lib = _lib.load()
        n, dev, ns = pts.n, self.device, self.n
        # one allocation, carved into the outputs (8-byte aligned pieces)
        sizes = [8 * ns * n, 8 * ns * n, 4 * ns * n] + ([8 * n, 4 * n, ns * n] if combine else [])
        offs = [0]
        for b in sizes:
            offs.append(offs[-1] + (b + 255) // 256 * 256)
        buf = torch.empty(offs[-1], dtype=torch.uint8, device=dev)
        piece = lambda i, dt, shape: buf[offs[i]:offs[i] + sizes[i]].view(dt).view(shape)
        F = piece(0, torch.float64, (ns, n))
        V = piece(1, torch.float64, (ns, n))
        I = piece(2, torch.int32, (ns, n))
        B = L = M = None
        if combine:
            B = piece(3, torch.float64, (n,))
            L = piece(4, torch.int32, (n,))
            M = piece(5, torch.uint8, (ns, n))
        check("gk_eval_series_set", lib.gk_eval_series_set(self.n, self.arr, ctypes.byref(pts.gk), prec, _ptr(F),
                                                           _ptr(V), _ptr(I), _ptr(B), _ptr(L), _ptr(M),
                                                           _ptr(info), _stream()))
        return F, V, I, B, L, M


_NP_OF = {torch.float64: np.float64, torch.int32: np.int32, torch.uint8: np.uint8, torch.int64: np.int64}
_ITEMSIZE = {torch.float64: 8, torch.int32: 4, torch.uint8: 1, torch.int64: 8}


def combine(fields, values, ids, relations, min_iso, max_iso, want_masks=True):
    """Lithology block of several series (rows of ``fields``, ``values`` and
    block ``ids``) with the squeezed series masks."""
    lib = _lib.load()
    n_series, n = fields.shape
    dev = fields.device
    out_v = torch.empty(n, dtype=torch.float64, device=dev)
    out_i = torch.empty(n, dtype=torch.int32, device=dev)
    masks = torch.empty((n_series, n), dtype=torch.uint8, device=dev) if want_masks else None
    rel = (ctypes.c_int32 * n_series)(*[int(r) for r in relations])
    mn = (ctypes.c_double * n_series)(*[float(v) for v in min_iso])
    mx = (ctypes.c_double * n_series)(*[float(v) for v in max_iso])
    ids = ids.contiguous()
    check("gk_combine_series", lib.gk_combine_series(n_series, n, _ptr(fields), _ptr(values), _ptr(ids), rel, mn,
                                                     mx, _ptr(out_v), _ptr(out_i), _ptr(masks), _stream()))
    return out_v, out_i, masks


def octree_corners(centres, spacing, out=None):
    """The 8 corners of every voxel (8n x 3), into ``out`` when given."""
    lib = _lib.load()
    n = centres.shape[0]
    if out is None:
        out = torch.empty((8 * n, 3), dtype=torch.float64, device=centres.device)
    sp = (ctypes.c_double * 3)(*[float(v) for v in spacing])
    check("gk_octree_corners", lib.gk_octree_corners(n, _ptr(centres), sp, _ptr(out), _stream()))
    return out


def octree_refine(centres, corner_ids, spacing, refine_all=False):
    """Children of the voxels whose corners differ in any id set:
    ``corner_ids`` is (8n,) or (n_sets, 8n) -- the lithology ids, then each
    fault series' block ids."""
    lib = _lib.load()
    n = centres.shape[0]
    n_sets = 0
    if corner_ids is not None:
        corner_ids = corner_ids.reshape(-1, 8 * n).contiguous() if n else corner_ids
        n_sets = int(corner_ids.shape[0]) if n else 1
    dev = centres.device
    wb = lib.gk_octree_workspace_bytes(n)
    # one allocation: children (8n x 3 FP64), the count (written by the scan), workspace
    cb = 8 * n * 3 * 8
    buf = torch.empty(cb + 256 + max(wb, 8), dtype=torch.uint8, device=dev)
    children = buf[:cb].view(torch.float64).view(8 * n, 3)
    count = buf[cb:cb + 8].view(torch.int64)
    work = buf[cb + 256:]
    sp = (ctypes.c_double * 3)(*[float(v) for v in spacing])
    check("gk_octree_refine", lib.gk_octree_refine(n, _ptr(centres), _ptr(corner_ids), n_sets,
                                                   int(bool(refine_all)), sp, _ptr(children), _ptr(count),
                                                   _ptr(work), wb, _stream()))
    m = int(count.item())
    return children[:m]


def _adjoint_points(series: DeviceSeries, pts: Points, fault_values=None):
    gp = GkPoints()
    ctypes.pointer(gp)[0] = pts.gk
    keep = None
    if series.n_faults:
        if fault_values is None:
            raise ValueError("a series with fault drift needs its faults' blocks at the points")
        keep = fault_values.to(dtype=torch.float64).contiguous()
        gp.fault_values = keep.data_ptr()
        gp.fault_ld = int(keep.shape[1])
    return gp, keep


def adjoint_rhs(series: DeviceSeries, pts: Points, g, fault_values=None):
    """r = sum_x g(x) dZ(x)/dw (N)."""
    lib = _lib.load()
    gp, keep = _adjoint_points(series, pts, fault_values)
    g = g.to(dtype=torch.float64).contiguous()
    r = torch.empty(series.N, dtype=torch.float64, device=series.device)
    check("gk_adjoint_rhs", lib.gk_adjoint_rhs(ctypes.byref(series.sys), ctypes.byref(gp), _ptr(g), _ptr(r),
                                               _stream()))
    return r


def build_adjoint(series: DeviceSeries, lam, w):
    """-lambda^T (dK/dtheta) w: (d surface points (n_sp, 3), d orientation
    positions (n_ori, 3), d surface-point nuggets (n_sp), d orientation
    nuggets (n_ori))."""
    lib = _lib.load()
    dev, s = series.device, series.sys
    d_sp = torch.empty((s.n_sp, 3), dtype=torch.float64, device=dev)
    d_dip = torch.empty((s.n_ori, 3), dtype=torch.float64, device=dev)
    d_nsp = torch.empty(s.n_sp, dtype=torch.float64, device=dev)
    d_ngr = torch.empty(s.n_ori, dtype=torch.float64, device=dev)
    check("gk_build_adjoint", lib.gk_build_adjoint(ctypes.byref(s), _ptr(lam.contiguous()), _ptr(w.contiguous()),
                                                   _ptr(d_sp), _ptr(d_dip), _ptr(d_nsp), _ptr(d_ngr), _stream()))
    return d_sp, d_dip, d_nsp, d_ngr


def eval_adjoint(series: DeviceSeries, model, pts: Points, g, d_sp, d_dip, fault_values=None):
    """Adds sum_x g(x) dZ(x)/d(record positions) at fixed weights into d_sp, d_dip."""
    lib = _lib.load()
    gp, keep = _adjoint_points(series, pts, fault_values)
    g = g.to(dtype=torch.float64).contiguous()
    check("gk_eval_adjoint", lib.gk_eval_adjoint(ctypes.byref(series.sys), _ptr(model), ctypes.byref(gp), _ptr(g),
                                                 _ptr(d_sp), _ptr(d_dip), _stream()))


class OctreeLevel:
    """One octree level computed by ``gk_octree_level``: every series at the
    level's points ([centres; corners] or the centres), their combination and
    -- unless it is the last level -- the children of the refined voxels, all
    in one device buffer.  ``result_bytes`` covers the level's results (points
    to masks); the children follow.  ``refine`` 3 adds the interpolation-
    error test with ``error_threshold`` standard deviations."""

    def __init__(self, series_set: "SeriesSet", centres, spacing, prec, corners, refine, fault_series=(),
                 info=None, error_threshold=0.0):
        lib = _lib.load()
        n = int(centres.shape[0])
        L = _lib.GkOctreeLevelLayout()
        check("gk_octree_level_plan", lib.gk_octree_level_plan(series_set.n, n, int(bool(corners)),
                                                                   int(refine), ctypes.byref(L)))
        self.layout, self.n, self.n_points, self.ns = L, n, int(L.n_points), series_set.n
        self.buffer = torch.empty(int(L.total), dtype=torch.uint8, device=centres.device)
        fs = (ctypes.c_int32 * max(1, len(fault_series)))(*[int(f) for f in fault_series])
        sp = (ctypes.c_double * 3)(*[float(v) for v in spacing])
        check("gk_octree_level", lib.gk_octree_level(series_set.n, series_set.arr, _ptr(centres.contiguous()), sp,
                                                     prec, len(fault_series), fs, float(error_threshold),
                                                     ctypes.byref(L),
                                                     self.buffer.data_ptr(), int(L.total), _ptr(info), _stream()))
        self.result_bytes = int(L.children)

    def views(self, buffer):
        """points, fields, values, ids, block, lith ids, masks as views of
        ``buffer``: this level's device buffer, or a host copy (numpy bytes)
        of its first ``result_bytes``."""
        L, np_, ns = self.layout, self.n_points, self.ns
        torch_buf = isinstance(buffer, torch.Tensor)

        def piece(off, dt, shape):
            nbytes = int(np.prod(shape)) * _ITEMSIZE[dt]
            b = buffer[int(off):int(off) + nbytes]
            return b.view(dt).view(shape) if torch_buf else b.view(_NP_OF[dt]).reshape(shape)
        return (piece(L.points, torch.float64, (np_, 3)), piece(L.fields, torch.float64, (ns, np_)),
                piece(L.values, torch.float64, (ns, np_)), piece(L.ids, torch.int32, (ns, np_)),
                piece(L.block, torch.float64, (np_,)), piece(L.lith_ids, torch.int32, (np_,)),
                piece(L.masks, torch.uint8, (ns, np_)))

    def children(self):
        """The next level's centres (reads the count: one synchronisation)."""
        L = self.layout
        if not L.refine or self.n == 0:
            return self.buffer[:0].view(torch.float64).view(0, 3)
        m = int(self.buffer[int(L.count):int(L.count) + 8].view(torch.int64).item())
        return self.buffer[int(L.children):int(L.children) + 24 * m].view(torch.float64).view(m, 3)


def set_wait_limit(spins):
    """Iteration cap of the kernels' spin waits (``gk_set_wait_limit``): 0
    makes them give up at once, None or a negative value restores the
    defaults.  For tests of the failure paths."""
    check("gk_set_wait_limit", _lib.load().gk_set_wait_limit(-1 if spins is None else int(spins)))


def marching_cubes(field, dims, level, spacing, origin, mask=None):
    """Vertices (n_v x 3, FP64) and triangles (n_t x 3, int32) of the level
    surface of a dense-grid field on the device (``gk_mc_count`` then
    ``gk_mc_emit``; one host read of the two counts in between)."""
    lib = _lib.load()
    field = field.to(dtype=torch.float64).contiguous()
    dev = field.device
    m = None if mask is None else mask.to(device=dev, dtype=torch.uint8).contiguous()
    d3 = (ctypes.c_int32 * 3)(*[int(v) for v in dims])
    n = int(dims[0]) * int(dims[1]) * int(dims[2])
    if field.numel() != n or (m is not None and m.numel() != n):
        raise ValueError(f"field/mask of {field.numel()} points for dims {tuple(dims)}")
    vol = _lib.GkMcVolume()
    vol.field = field.data_ptr()
    vol.mask = 0 if m is None else m.data_ptr()
    vol.dims = d3
    vol.level = float(level)
    vol.spacing = (ctypes.c_double * 3)(*[float(v) for v in spacing])
    vol.origin = (ctypes.c_double * 3)(*[float(v) for v in origin])
    wb = lib.gk_mc_workspace_bytes(d3)
    work = torch.empty(max(wb, 8), dtype=torch.uint8, device=dev)
    counts = torch.empty(2, dtype=torch.int64, device=dev)
    st = _stream()
    check("gk_mc_count", lib.gk_mc_count(ctypes.byref(vol), _ptr(work), wb, _ptr(counts), st))
    nv, nt = (int(v) for v in counts.tolist())
    verts = torch.empty((nv, 3), dtype=torch.float64, device=dev)
    faces = torch.empty((nt, 3), dtype=torch.int32, device=dev)
    check("gk_mc_emit", lib.gk_mc_emit(ctypes.byref(vol), _ptr(work), wb, _ptr(verts), nv, _ptr(faces), nt, st))
    return verts, faces


@contextlib.contextmanager
def lu_update_engine(engine):
    """Within the block the FP32 trailing updates run on ``engine``
    (``_lib.GK_LU_UPDATE_TC`` or ``_lib.GK_LU_UPDATE_SIMT``)."""
    lib = _lib.load()
    prev = lib.gk_lu_update_engine()
    check("gk_lu_update_select", lib.gk_lu_update_select(int(engine)))
    try:
        yield
    finally:
        lib.gk_lu_update_select(prev)


def gravity_tz(centres, lower, upper):
    """tz of every voxel of a centred-grid kernel (gk_gravity_tz); (n, 3)
    CUDA FP64 tensors in, (n,) out."""
    lib = _lib.load()
    n = int(centres.shape[0])
    c, lo, hi = (t.to(dtype=torch.float64).contiguous() for t in (centres, lower, upper))
    out = torch.empty(n, dtype=torch.float64, device=c.device)
    check("gk_gravity_tz", lib.gk_gravity_tz(n, _ptr(c), _ptr(lo), _ptr(hi), _ptr(out), _stream()))
    return out


def gravity(ids, n_devices, densities, tz):
    """Density-weighted tz sum per device over lithology ids (gk_gravity)."""
    lib = _lib.load()
    n_vox = int(tz.shape[0])
    ids = ids.to(dtype=torch.int32).contiguous()
    rho = densities.to(device=ids.device, dtype=torch.float64).contiguous()
    tz = tz.to(device=ids.device, dtype=torch.float64).contiguous()
    if ids.numel() != n_devices * n_vox:
        raise ValueError(f"{ids.numel()} ids for {n_devices} devices x {n_vox} voxels")
    out = torch.empty(n_devices, dtype=torch.float64, device=ids.device)
    check("gk_gravity", lib.gk_gravity(int(n_devices), n_vox, _ptr(ids), int(rho.numel()), _ptr(rho), _ptr(tz),
                                       _ptr(out), _stream()))
    return out
