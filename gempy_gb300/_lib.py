"""ctypes binding of ``libgempy_gb300.so`` (declared in ``include/gempy_gb300.h``).

The library is built in-tree by ``gempy_gb300/build.py`` (or
``__graft_entry__.build()``).  Loading fails loudly when it is missing or when
no CUDA device is usable: this package has no CPU path.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgempy_gb300.so")

GK_OK, GK_ERR_ARG, GK_ERR_SIZE, GK_ERR_CUDA = 0, 1, 2, 3
GK_ERR_SINGULAR, GK_ERR_NOT_CONVERGED, GK_ERR_NONFINITE, GK_ERR_TIMEOUT = 4, 5, 6, 7
STATUS_NAMES = {0: "OK", 1: "ERR_ARG", 2: "ERR_SIZE", 3: "ERR_CUDA", 4: "ERR_SINGULAR",
                5: "ERR_NOT_CONVERGED", 6: "ERR_NONFINITE", 7: "ERR_TIMEOUT"}
GK_F64, GK_F32, GK_FF = 0, 1, 2
GK_KERNEL_CUBIC, GK_KERNEL_EXPONENTIAL = 0, 1
GK_MAX_SURFACES = 32
GK_MAX_FAULTS = 16
GK_TIE_TOL = 1e-9
GK_NOALLOC_MAX_N = 1024
GK_LU_UPDATE_SIMT, GK_LU_UPDATE_TC = 0, 1
GK_CTA_MAX_N = 4096
GK_TUNE_EVAL_FF, GK_TUNE_EVAL_F32, GK_TUNE_BATCH_EVAL, GK_TUNE_EVAL_FF_LIST = 0, 1, 2, 3
TUNABLES = {"eval_ff": GK_TUNE_EVAL_FF, "eval_f32": GK_TUNE_EVAL_F32, "batch_eval": GK_TUNE_BATCH_EVAL,
            "eval_ff_list": GK_TUNE_EVAL_FF_LIST}

c_int32_p = ctypes.POINTER(ctypes.c_int32)
c_double_p = ctypes.POINTER(ctypes.c_double)


class GkInfo(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int32), ("where", ctypes.c_int32), ("iterations", ctypes.c_int32),
                ("pivoted", ctypes.c_int32), ("residual", ctypes.c_double)]


class GkSystem(ctypes.Structure):
    _fields_ = [("n_ori", ctypes.c_int32), ("n_sp", ctypes.c_int32), ("n_iface", ctypes.c_int32),
                ("uni_degree", ctypes.c_int32), ("kernel", ctypes.c_int32), ("n_fault", ctypes.c_int32),
                ("range", ctypes.c_double), ("c_o", ctypes.c_double), ("i_res", ctypes.c_double),
                ("gi_res", ctypes.c_double),
                ("dip_positions", ctypes.c_void_p), ("dip_gradients", ctypes.c_void_p),
                ("nugget_grad", ctypes.c_void_p), ("sp_coords", ctypes.c_void_p),
                ("nugget_sp", ctypes.c_void_p), ("ref_index", ctypes.c_void_p),
                ("rest_index", ctypes.c_void_p), ("fault_sp", ctypes.c_void_p)]


class GkPoints(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("dims", ctypes.c_int32 * 3), ("n", ctypes.c_int64),
                ("origin", ctypes.c_double * 3), ("spacing", ctypes.c_double * 3),
                ("xyz", ctypes.c_void_p), ("fault_values", ctypes.c_void_p), ("fault_ld", ctypes.c_int64)]


class GkSegment(ctypes.Structure):
    _fields_ = [("n_surf", ctypes.c_int32), ("reserved", ctypes.c_int32), ("slope", ctypes.c_double),
                ("isovalues", ctypes.c_double * GK_MAX_SURFACES),
                ("unit_values", ctypes.c_double * (GK_MAX_SURFACES + 1))]


class GkBatchItem(ctypes.Structure):
    _fields_ = [("n_ori", ctypes.c_int32), ("n_sp", ctypes.c_int32), ("n_iface", ctypes.c_int32),
                ("uni_degree", ctypes.c_int32), ("kernel", ctypes.c_int32), ("n_surf", ctypes.c_int32),
                ("range", ctypes.c_double), ("c_o", ctypes.c_double), ("i_res", ctypes.c_double),
                ("gi_res", ctypes.c_double), ("ori_offset", ctypes.c_int64), ("sp_offset", ctypes.c_int64),
                ("iface_offset", ctypes.c_int64), ("points_per_surface", ctypes.c_int32 * GK_MAX_SURFACES),
                ("dims", ctypes.c_int32 * 3), ("reserved", ctypes.c_int32), ("origin", ctypes.c_double * 3),
                ("spacing", ctypes.c_double * 3), ("slope", ctypes.c_double),
                ("unit_values", ctypes.c_double * (GK_MAX_SURFACES + 1))]


class GkBatch(ctypes.Structure):
    _fields_ = [("n_items", ctypes.c_int32), ("reserved", ctypes.c_int32),
                ("items", ctypes.POINTER(GkBatchItem)), ("dip_positions", ctypes.c_void_p),
                ("dip_gradients", ctypes.c_void_p), ("nugget_grad", ctypes.c_void_p),
                ("sp_coords", ctypes.c_void_p), ("nugget_sp", ctypes.c_void_p),
                ("ref_index", ctypes.c_void_p), ("rest_index", ctypes.c_void_p)]


GK_CTA_MAX_JOBS = 16


class GkSeriesEval(ctypes.Structure):
    _fields_ = [("sys", ctypes.POINTER(GkSystem)), ("model", ctypes.c_void_p), ("seg", GkSegment),
                ("relation", ctypes.c_int32), ("n_faults", ctypes.c_int32),
                ("faults", ctypes.c_int32 * GK_MAX_FAULTS), ("min_iso", ctypes.c_double),
                ("max_iso", ctypes.c_double)]


class GkOctreeLevelLayout(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64), ("n_points", ctypes.c_int64), ("n_series", ctypes.c_int32),
                ("corners", ctypes.c_int32), ("refine", ctypes.c_int32), ("reserved", ctypes.c_int32)] + \
               [(k, ctypes.c_uint64) for k in ("points", "fields", "values", "ids", "block", "lith_ids", "masks",
                                               "children", "count", "work", "total")]


class GkCtaJob(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64), ("K", ctypes.c_void_p), ("ldk", ctypes.c_int64), ("b", ctypes.c_void_p),
                ("x", ctypes.c_void_p), ("work", ctypes.c_void_p), ("work_bytes", ctypes.c_size_t),
                ("info", ctypes.c_void_p)]


GK_MLP_HIDDEN = 256
GK_MLP_MAX_IN = 64
GK_MLP_MAX_OUT = 16
GK_MLP_MAX_BATCH = 1 << 22
GK_SYSTEM_FEATURES = 16


class GkMlp(ctypes.Structure):
    _fields_ = [("in_dim", ctypes.c_int32), ("out_dim", ctypes.c_int32), ("params", ctypes.c_void_p)]


class GkAdam(ctypes.Structure):
    _fields_ = [("lr", ctypes.c_float), ("beta1", ctypes.c_float), ("beta2", ctypes.c_float),
                ("eps", ctypes.c_float), ("weight_decay", ctypes.c_float)]


# (name, restype, argtypes) of every exported symbol; tests check the header
# declares exactly these.
class GkMcVolume(ctypes.Structure):
    _fields_ = [("field", ctypes.c_void_p), ("mask", ctypes.c_void_p), ("dims", ctypes.c_int32 * 3),
                ("reserved", ctypes.c_int32), ("level", ctypes.c_double), ("spacing", ctypes.c_double * 3),
                ("origin", ctypes.c_double * 3)]


SIGNATURES = [
    ("gk_system_size", ctypes.c_int64, [ctypes.POINTER(GkSystem)]),
    ("gk_build", ctypes.c_int, [ctypes.POINTER(GkSystem), ctypes.c_int, ctypes.c_void_p, ctypes.c_int64,
                                ctypes.c_void_p, ctypes.c_void_p]),
    ("gk_lu_workspace_bytes", ctypes.c_size_t, [ctypes.c_int, ctypes.c_int64]),
    ("gk_lu_factor", ctypes.c_int, [ctypes.c_int, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64,
                                    ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p,
                                    ctypes.c_void_p]),
    ("gk_lu_solve", ctypes.c_int, [ctypes.c_int, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64,
                                   ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                   ctypes.c_void_p, ctypes.c_void_p]),
    ("gk_build_tables_bytes", ctypes.c_size_t, [ctypes.POINTER(GkSystem)]),
    ("gk_build_tables", ctypes.c_int, [ctypes.POINTER(GkSystem), ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                       ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    ("gk_lu_update_select", ctypes.c_int, [ctypes.c_int32]),
    ("gk_lu_update_engine", ctypes.c_int32, []),
    ("gk_gemv", ctypes.c_int, [ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p,
                               ctypes.c_void_p]),
    ("gk_solve_mixed_workspace_bytes", ctypes.c_size_t, [ctypes.c_int64]),
    ("gk_solve_mixed", ctypes.c_int, [ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                      ctypes.c_void_p, ctypes.c_double, ctypes.c_int32, ctypes.c_void_p,
                                      ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p]),
    ("gk_solve_mixed_noalloc", ctypes.c_int, [ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                              ctypes.c_void_p, ctypes.c_double, ctypes.c_int32, ctypes.c_void_p,
                                              ctypes.c_void_p]),
    ("gk_solve_mixed_cta_workspace_bytes", ctypes.c_size_t, [ctypes.c_int64, ctypes.c_int64]),
    ("gk_solve_mixed_cta", ctypes.c_int, [ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                          ctypes.c_void_p, ctypes.c_double, ctypes.c_int32, ctypes.c_void_p,
                                          ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p]),
    ("gk_solve_mixed_cta_many", ctypes.c_int, [ctypes.c_int32, ctypes.POINTER(GkCtaJob), ctypes.c_double,
                                               ctypes.c_int32, ctypes.c_void_p]),
    ("gk_solve_twolevel_workspace_bytes", ctypes.c_size_t, [ctypes.c_int64, ctypes.c_int]),
    ("gk_solve_twolevel", ctypes.c_int, [ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                                         ctypes.c_int32,
                                         ctypes.c_int, ctypes.c_double, ctypes.c_int32, ctypes.c_void_p,
                                         ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p]),
    ("gk_eval_model_bytes", ctypes.c_size_t, [ctypes.POINTER(GkSystem)]),
    ("gk_eval_prepare", ctypes.c_int, [ctypes.POINTER(GkSystem), ctypes.c_void_p, ctypes.c_void_p,
                                       ctypes.c_void_p]),
    ("gk_eval", ctypes.c_int, [ctypes.POINTER(GkSystem), ctypes.c_void_p, ctypes.POINTER(GkPoints),
                               ctypes.c_int, ctypes.POINTER(GkSegment), ctypes.c_void_p, ctypes.c_void_p,
                               ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    ("gk_eval_series_set", ctypes.c_int, [ctypes.c_int32, ctypes.POINTER(GkSeriesEval), ctypes.POINTER(GkPoints),
                                          ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                          ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                          ctypes.c_void_p]),
    ("gk_combine_series", ctypes.c_int, [ctypes.c_int32, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p,
                                         ctypes.c_void_p, c_int32_p, c_double_p, c_double_p, ctypes.c_void_p,
                                         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    ("gk_octree_corners", ctypes.c_int, [ctypes.c_int64, ctypes.c_void_p, c_double_p, ctypes.c_void_p,
                                         ctypes.c_void_p]),
    ("gk_octree_workspace_bytes", ctypes.c_size_t, [ctypes.c_int64]),
    ("gk_octree_refine", ctypes.c_int, [ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
                                        ctypes.c_int32, c_double_p, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    ("gk_octree_level_plan", ctypes.c_int, [ctypes.c_int32, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32,
                                              ctypes.POINTER(GkOctreeLevelLayout)]),
    ("gk_octree_level", ctypes.c_int, [ctypes.c_int32, ctypes.POINTER(GkSeriesEval), ctypes.c_void_p, c_double_p,
                                       ctypes.c_int, ctypes.c_int32, c_int32_p, ctypes.c_double,
                                       ctypes.POINTER(GkOctreeLevelLayout),
                                       ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p]),
    ("gk_adjoint_rhs", ctypes.c_int, [ctypes.POINTER(GkSystem), ctypes.POINTER(GkPoints), ctypes.c_void_p,
                                      ctypes.c_void_p, ctypes.c_void_p]),
    ("gk_build_adjoint", ctypes.c_int, [ctypes.POINTER(GkSystem), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    ("gk_eval_adjoint", ctypes.c_int, [ctypes.POINTER(GkSystem), ctypes.c_void_p, ctypes.POINTER(GkPoints),
                                       ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    ("gk_mc_workspace_bytes", ctypes.c_size_t, [c_int32_p]),
    ("gk_mc_count", ctypes.c_int, [ctypes.POINTER(GkMcVolume), ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p,
                                   ctypes.c_void_p]),
    ("gk_mc_emit", ctypes.c_int, [ctypes.POINTER(GkMcVolume), ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p,
                                  ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p]),
    ("gk_gravity_tz", ctypes.c_int, [ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                     ctypes.c_void_p, ctypes.c_void_p]),
    ("gk_gravity", ctypes.c_int, [ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p,
                                  ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    ("gk_batch_workspace_bytes", ctypes.c_size_t, [ctypes.POINTER(GkBatch)]),
    ("gk_batch_points", ctypes.c_int64, [ctypes.POINTER(GkBatch)]),
    ("gk_batch_plan", ctypes.c_int, [ctypes.POINTER(GkBatch), ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    ("gk_batch_run", ctypes.c_int, [ctypes.POINTER(GkBatch), ctypes.c_void_p, ctypes.c_size_t, ctypes.c_double,
                                    ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                    ctypes.c_void_p, ctypes.c_void_p]),
    ("gk_batch_results", ctypes.c_int, [ctypes.POINTER(GkBatch), ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int32,
                                        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    ("gk_tune_variants", ctypes.c_int32, []),
    ("gk_tune_describe", ctypes.c_int, [ctypes.c_int32, c_int32_p, c_int32_p]),
    ("gk_tune_set", ctypes.c_int, [ctypes.c_int32, ctypes.c_int32]),
    ("gk_tune_get", ctypes.c_int32, [ctypes.c_int32]),
    ("gk_mlp_param_count", ctypes.c_int64, [ctypes.c_int32, ctypes.c_int32]),
    ("gk_mlp_workspace_bytes", ctypes.c_size_t, [ctypes.c_int32, ctypes.c_int32, ctypes.c_int64]),
    ("gk_mlp_fwd", ctypes.c_int, [ctypes.POINTER(GkMlp), ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p,
                                  ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    ("gk_mlp_bwd", ctypes.c_int, [ctypes.POINTER(GkMlp), ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p,
                                  ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    ("gk_mlp_fwd_tc", ctypes.c_int, [ctypes.POINTER(GkMlp), ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p,
                                     ctypes.c_void_p, ctypes.c_void_p]),
    ("gk_mlp_mse", ctypes.c_int, [ctypes.c_int64, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                                  ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    ("gk_mlp_adam", ctypes.c_int, [ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                   ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(GkAdam), ctypes.c_int32,
                                   ctypes.c_void_p]),
    ("gk_system_features", ctypes.c_int, [ctypes.POINTER(GkSystem), ctypes.c_void_p, ctypes.c_void_p]),
    ("gk_set_wait_limit", ctypes.c_int, [ctypes.c_int64]),
    ("gk_version", ctypes.c_char_p, []),
    ("gk_launch_count", ctypes.c_uint64, []),
]

_lib = None


class GkError(RuntimeError):
    def __init__(self, func, status, where=None):
        self.status = status
        msg = f"{func} failed: {STATUS_NAMES.get(status, status)}"
        if where is not None:
            msg += f" (at {where})"
        super().__init__(msg)


def load():
    """Load the library once; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
            "(gempy_gb300 has no CPU fallback)")
    lib = ctypes.CDLL(LIB_PATH)
    for name, res, args in SIGNATURES:
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def check(func, status):
    if status != GK_OK:
        raise GkError(func, status)
