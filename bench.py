"""Benchmark of the co-kriging hot path on one workload.

Workload (one "step"): the precision configuration -- one series, 4000
surface points on 8 folded surfaces, 1500 orientations (N = 8498), cubic
kernel, linear drift, a 256^3 regular grid (16.8M points): kriging-matrix
build, solve, isovalues, evaluation with fused segmentation, series
combination.  ``value`` is grid points/s of the mixed form (FP64 build, FP32
LU + FP64 FGMRES, FP32 evaluation with FP64 isovalues) with inputs resident in
HBM; the plain FP64 form is timed on the same inputs in the same run.  The
mixed form evaluates the field in float-float on the FP32 pipe: the kriging
sum of this workload cancels by a factor ~3e4, so plain FP32 terms would miss
the 1e-6 field-error bar by three orders of magnitude.
``e2e`` runs the same step through ``gempy_gb300.compute_model`` from host
(numpy) inputs with the host<->device copies inside the timed region.

``--impl reference`` times the CPU restatement of the reference's algorithm
(the FP64 oracle; the reference's own engine is not available) on a bounded
sample of the same workload, with all host threads.

Multi-GPU: the path runs as independent replicas (one per rank), no
collective on the data path; ``value`` sums all ranks' points over the slowest
rank's time.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "grid points/s + kriging solves/s: mixed/learned vs FP64 GPU at 1e-6 field error"
# thread instructions per point-record pair of the float-float field kernel,
# from ncu's executed-instruction count (profiles/eval_ff_precision_64.md)
FF_OPS_PER_PAIR = 76
WORKLOAD = ("precision: 1 series, 4000 surface points on 8 folded surfaces, 1500 orientations "
            "(N=8495), cubic, linear drift, 256^3 regular grid")

# algorithmic work per unit (fixed constants: F_C = 20 per surface-point kernel,
# F_G = 30 per orientation kernel, 2N for the drift/weights, x2 with gradients)
F_C, F_G, F_K = 20, 30, 40


def eval_flops_per_point(n_p, n_k, n_o, N, gradient=False):
    f = (n_p + n_k) * F_C + n_o * F_G + 2 * N
    return 2 * f if gradient else f


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        d["_source"] = "measured"
        return d
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "sm_max_mhz": 2070.0, "_source": "fallback"}


class ClockSampler:
    """nvidia-smi sampling during the timed region (read only)."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        # raw samples go to $GK_CLOCKS_DIR when set (kept for inspection), else a temp file
        out_dir = os.environ.get("GK_CLOCKS_DIR")
        self.path = os.path.join(out_dir, f"clocks_rank{index}.csv") if out_dir and os.path.isdir(out_dir) \
            else os.path.join(tempfile.gettempdir(), f"gk_clocks_{os.getpid()}_{index}.csv")

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    rows.append((float(parts[1]), float(parts[2]), float(parts[3]), parts[5:9]))
                except ValueError:
                    continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = np.array([r[0] for r in rows])
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i, v in enumerate(r[3]) if v.lower() == "active"})
        load = sm[sm > 0.5 * sm.max()] if len(sm) else sm
        return {"sm_mhz": float(np.median(load)), "sm_max_mhz": float(rows[0][1]), "reasons": reasons,
                "samples": len(rows), "power_w_max": float(max(r[2] for r in rows))}


def slowest_rank_ms(ms, world):
    """Replicas: the job takes as long as its slowest rank (max all-reduce of
    the rank's own time; the only collective of the multi-GPU path)."""
    if world <= 1:
        return ms
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([ms], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(points_per_rank, ms, world):
    """Whole-job grid points/s: every rank evaluates its own grid (weak
    scaling), the time is the slowest rank's."""
    return world * points_per_rank / (ms * 1e-3)


def launch_count():
    """Kernels launched so far by libgempy_gb300.so (its own counter)."""
    from gempy_gb300 import _lib
    return int(_lib.load().gk_launch_count())


def reference_arm(args):
    """CPU restatement timed on the host cores (bounded sample per step)."""
    import torch  # noqa: F401  (rank handling below uses env only)
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from gempy_gb300 import synthetic
    from oracle import kriging, segmentation
    from oracle.inputs import series_from_engine_inputs
    from oracle.parallel import FieldPool, host_cores
    m = synthetic.precision()
    (s,) = series_from_engine_inputs(m.interpolation_input, m.options, m.data_descriptor)
    grid = m.interpolation_input.grid.dense_grid
    n_total = grid.n_points
    rng = np.random.default_rng(0)
    cores = host_cores()
    sample = int(os.environ.get("GK_REF_SAMPLE", str(4096 * cores)))
    idx = np.sort(rng.choice(n_total, sample, replace=False))
    xs = grid.values[idx]
    pool = FieldPool(s, cores)     # one single-threaded evaluation worker per core, started before timing

    def step():
        t0 = time.perf_counter()
        K, b = kriging.build_system(s)
        w = kriging.solve(K, b)
        iso = kriging.isovalues(s, w)
        t1 = time.perf_counter()
        z = pool.evaluate(xs, w)
        segmentation.segment(z, iso, m.interpolation_input.unit_values, m.options.sigmoid_slope)
        t2 = time.perf_counter()
        return t1 - t0, (t2 - t1) / sample

    # every sample step is a full FP64 build + LU on the host cores (seconds each):
    # at most 1 warm-up and 3 timed steps run, and the line reports what ran
    n_warm = max(0, min(args.warmup, 1))
    n_steps = max(1, min(args.steps, 3))
    t_start = time.perf_counter()
    for _ in range(n_warm):
        step()
    ts, te = [], []
    for _ in range(n_steps):
        a, b = step()
        ts.append(a)
        te.append(b)
    wall = time.perf_counter() - t_start
    pool.close()
    t_solve, t_pt = float(np.mean(ts)), float(np.mean(te))
    t_step = t_solve + t_pt * n_total
    v = n_total / t_step
    sample_ms = 1e3 * (t_solve + t_pt * sample)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "grid points/s", "n_gpus": args.gpus,
            "steps": n_steps, "warmup": n_warm, "ms_per_step": sample_ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "grid_points": n_total},
            "requested": {"steps": args.steps, "warmup": args.warmup},
            "extrapolated": True,
            "value_basis": "value = grid_points / (build+LU seconds + per-point seconds x grid_points); "
                           "ms_per_step is the measured sample step",
            "sample_points": sample, "measured_steps": n_steps, "measured_seconds": wall,
            "extrapolated_ms_per_workload_step": 1e3 * t_step,
            "solves_per_s": 1.0 / t_solve,
            "cpu_baseline": {"value": v, "unit": "grid points/s", "cores": cores, "kind": "port",
                             "extrapolated": True, "sample_points": sample,
                             "sample": f"FP64 numpy/scipy oracle: full build+LU (N={s.size}, BLAS on all {cores} "
                                       f"cores) per step + {sample}-point subsample of the 256^3 grid "
                                       f"evaluated by {cores} worker processes, extrapolated to {n_total} points"},
            "e2e": {"value": v, "unit": "grid points/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--plain-steps", type=int, default=2)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--grid", type=int, default=256)
    ap.add_argument("--no-extra", action="store_true", help="skip the batch and octree sections")
    ap.add_argument("--batch-realisations", type=int, default=512)
    ap.add_argument("--only-learned", action="store_true",
                    help="run only the config-5 section (learned two-level solve vs FP64 LU) and print it")
    ap.add_argument("--learned-points", type=int, default=20000,
                    help="surface points of the config-5 system (orientations: 30 %%)")
    ap.add_argument("--learned-config", default=None,
                    help="landmarks,block,policy,f32|ff|f64: use this two-level configuration instead of the network's")
    args = ap.parse_args()
    if args.impl == "reference":
        return reference_arm(args)
    if args.only_learned:
        print(json.dumps({"learned": learned_section(args.learned_points, args.learned_config)}, default=float),
              flush=True)
        return

    import torch
    import torch.distributed as dist

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")

    import gempy_gb300 as gg
    from gempy_gb300 import kernels as K
    from gempy_gb300 import synthetic

    m = synthetic.precision(resolution=(args.grid,) * 3)
    ii, opts, dd = m.interpolation_input, m.options, m.data_descriptor
    grid = ii.grid.dense_grid
    n_pts = grid.n_points
    ko = opts.kernel_options
    sp, ori = ii.surface_points, ii.orientations
    pps = dd.tensors_structure.number_of_points_per_surface
    ds = K.DeviceSeries(ori.dip_positions, ori.dip_gradients, ori.nugget_effect_grad, sp.sp_coords,
                        sp.nugget_effect_scalar, pps, range=ko.range, c_o=ko.c_o, uni_degree=ko.uni_degree,
                        kernel=ko.kernel_function, i_res=ko.i_res, gi_res=ko.gi_res)
    N = ds.N
    uv = ii.unit_values
    pts = K.Points.regular(grid)
    ref_pts = K.Points(xyz=ds.ref_points)
    stream = torch.cuda.current_stream()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    out_buf = {"field": torch.empty(n_pts, dtype=torch.float64, device="cuda"),
               "values": torch.empty(n_pts, dtype=torch.float64, device="cuda")}
    ev_times = []

    def step(mixed, record=None):
        K64, b = K.build(ds, K.GK_F64)
        if mixed:
            w, info = K.solve_mixed(ds, tol=1e-11, K=K64, b=b)
        else:
            f = K.lu_factor(K64, K.GK_F64, overwrite=True)
            w = K.lu_solve(f, b)
            info = f.info
        del K64
        model = K.prepare(ds, w)
        iso_t, _, _, _ = K.evaluate(ds, model, ref_pts, K.GK_F64)
        iso = iso_t.cpu().numpy()
        order = np.argsort(-iso, kind="stable")
        seg = K.make_segment(iso[order], uv, opts.sigmoid_slope)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fld, _, vals, bid = K.evaluate(ds, model, pts, K.GK_FF if mixed else K.GK_F64, seg=seg, out=out_buf,
                                       want_ids=True)
        e1.record(stream)
        cv, ci, _ = K.combine(fld[None], vals[None], bid[None], [4], [iso.min()], [iso.max()], want_masks=False)
        if record is not None:
            record.append((e0, e1))
        return w, info, iso, fld, ci

    def timed(mixed, steps, warmup):
        for _ in range(warmup):
            step(mixed)
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()
        evs, per = [], []
        for _ in range(steps):
            flush.fill_(1.0)                                  # L2 flush between steps (256 MB)
            s0 = torch.cuda.Event(enable_timing=True)
            s1 = torch.cuda.Event(enable_timing=True)
            s0.record(stream)
            step(mixed, evs)
            s1.record(stream)
            torch.cuda.synchronize()
            per.append(s0.elapsed_time(s1))
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
        ms = slowest_rank_ms(float(np.sum(per)), world)
        ev_ms = float(np.mean([a.elapsed_time(b) for a, b in evs]))
        return ms / steps, ev_ms

    # ---- mixed form, timed
    for _ in range(args.warmup):
        step(True)
    torch.cuda.synchronize()
    l0 = launch_count()
    with ClockSampler(local) as clk:
        ms_mixed, ev_mixed = timed(True, args.steps, 0)
    launches = launch_count() - l0
    clocks = clk.summary()
    # ---- plain FP64 form, same inputs
    ms_plain, ev_plain = timed(False, args.plain_steps, 1)

    # ---- accuracy of the mixed form vs the plain FP64 form on the full grid
    w_m, info_m, iso_m, fld_m, ids_m = step(True)
    fld_m = fld_m.clone()
    ids_m = ids_m.clone()
    w_p, _, iso_p, fld_p, ids_p = step(False)
    zp = fld_p
    err_field = float((fld_m - zp).abs().max() / zp.abs().max())
    err_w = float((w_m - w_p).abs().max() / w_p.abs().max())
    band = max(10.0 / opts.sigmoid_slope, 4 * err_field * float(zp.abs().max()))
    iso_t = torch.as_tensor(iso_p, device="cuda")
    outside = ((zp[:, None] - iso_t[None, :]).abs() > band).all(dim=1)
    mism = int(((ids_m != ids_p) & outside).sum())
    info_mixed = K.read_info(info_m)
    # gradient error: mixed-form weights vs plain FP64 weights, FP64 gradient kernel on a 64^3 sub-grid
    sub = gg.RegularGrid(grid.orthogonal_extent, np.array([64, 64, 64]))
    gpts = K.Points.regular(sub)
    _, g_m, _, _ = K.evaluate(ds, K.prepare(ds, w_m), gpts, K.GK_F64, gradient=True, want_field=False)
    _, g_p, _, _ = K.evaluate(ds, K.prepare(ds, w_p), gpts, K.GK_F64, gradient=True, want_field=False)
    err_grad = float((g_m - g_p).abs().max() / g_p.abs().max())
    # per-kernel evidence on this workload (CUDA events on the launching stream)
    def _ev(fn, reps=3):
        fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(reps):
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(b))
        return float(np.median(ts))
    t_build = _ev(lambda: K.build(ds, K.GK_F64))
    K64_, _ = K.build(ds, K.GK_F64)
    K32_ = torch.empty((N, K.leading_dim(N, K.GK_F32)), dtype=torch.float32, device="cuda")
    K32_[:, :N] = K64_[:, :N].float()
    t_lu32 = _ev(lambda: K.lu_factor(K32_, K.GK_F32))
    t_lu64 = _ev(lambda: K.lu_factor(K64_, K.GK_F64), reps=1)
    # the FP32 trailing updates on either engine: the partially pivoted FP32
    # LU and the mixed solve (whose preconditioner is the unpivoted FP32 LU)
    from gempy_gb300 import _lib as L
    b64_ = K.build(ds, K.GK_F64)[1]
    eng = {}
    for name, e in (("tensor_cores_3xtf32", L.GK_LU_UPDATE_TC), ("fp32_simt", L.GK_LU_UPDATE_SIMT)):
        with K.lu_update_engine(e):
            its = []
            t_m = _ev(lambda: its.append(K.solve_mixed(ds, tol=1e-11, K=K64_, b=b64_)[1]))
            eng[name] = {"lu_f32_partial_pivoting_ms": _ev(lambda: K.lu_factor(K32_, K.GK_F32)),
                         "mixed_solve_ms": t_m, "fgmres_iterations": int(K.read_info(its[-1])["iterations"])}
    del K64_, K32_, b64_
    mesh = mesh_section(fld_m, iso_m, grid) if rank == 0 else None
    pk0 = peaks()
    kern = {
        "build_f64": {"ms": t_build, "bytes": N * N * 8, "achieved_GBps": N * N * 8 / (t_build * 1e-3) / 1e9,
                      "hbm_peak_GBps": pk0.get("hbm_gbs"), "flops_per_entry": F_K,
                      "note": "table-driven (gk_build_tables): covariances of point pairs, orientation-point pairs "
                              "and orientation pairs formed once (FP64, DFMA-bound), entries assembled from "
                              "them; the tables and the gathers, not the K write, set the time"},
        "lu_f32_partial_pivoting": {"ms": t_lu32, "TFLOPs": 2 / 3 * N ** 3 / (t_lu32 * 1e-3) / 1e12},
        "lu_f64_partial_pivoting": {"ms": t_lu64, "TFLOPs": 2 / 3 * N ** 3 / (t_lu64 * 1e-3) / 1e12,
                                    "note": "GB300 FP64 is ~1.2 TFLOP/s; the trailing GEMM runs at that rate"},
        "eval_ff": {"ms": ev_mixed, "points": n_pts},
        "segmentation": {"fused": True, "bytes_per_point": 8 + 8,
                         "note": "written in the evaluation epilogue; no separate pass over the field"},
        "lu_f32_update_engines": eng,
        "tensor_pipe": {"used": True,
                        "where": "FP32 LU trailing updates (tcgen05.mma kind::tf32, 3 split-operand products, "
                                 "TMEM accumulators) of the mixed solve's preconditioner and of gk_lu_factor(F32)",
                        "not_used_for": "the field evaluation: float-float on the FP32 pipe, because TF32/BF16 "
                                        "products cannot meet the 1e-6 field-error target on this workload"},
    }

    # ---- end to end through compute_model with host inputs (H2D + D2H inside)
    cfg = gg.EngineConfig(dtype="float32")
    e2e_ii = ii
    opts_e2e = opts
    for _ in range(1):
        gg.compute_model(e2e_ii, opts_e2e, dd, config=cfg)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e2e_steps = max(1, min(args.steps, 3))
    for _ in range(e2e_steps):
        sol = gg.compute_model(e2e_ii, opts_e2e, dd, config=cfg)
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    h2d = sum(a.nbytes for a in (sp.sp_coords, sp.nugget_effect_scalar, ori.dip_positions, ori.dip_gradients,
                                 ori.nugget_effect_grad)) + 8 * len(pps)
    d2h = sum(np.asarray(a).nbytes for a in (sol.raw_arrays.lith_block, sol.raw_arrays.scalar_field_matrix,
                                             sol.raw_arrays.mask_matrix_squeezed, sol.raw_arrays.block_matrix))

    # ---- roofline of the dominant kernel (the FP32 evaluation)
    pk = peaks()
    n_k = len(pps)
    fl_pt = eval_flops_per_point(sp.sp_coords.shape[0], n_k, ori.dip_positions.shape[0], N)
    achieved_tf = fl_pt * n_pts / (ev_mixed * 1e-3) / 1e12
    sm_mhz = pk.get("sm_max_mhz", 2070.0)
    fp32_peak = 152 * 128 * 2 * sm_mhz * 1e6 / 1e12

    ms_step = ms_mixed
    line = {
        "metric": METRIC,
        "value": replica_throughput(n_pts, ms_step, world),
        "unit": "grid points/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_step,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 (LU); float-float on the FP32 pipe (field); f64 (build, residual, update, isovalues)",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "grid_points": n_pts, "N": N,
                   "l2": "flushed between steps (256 MB write); K (FP64, 578 MB) is larger than L2",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "solves_per_s": 1e3 / (ms_step - ev_mixed) if ms_step > ev_mixed else None,
        "plain_fp64": {"ms_per_step": ms_plain, "grid_points_per_s": n_pts / (ms_plain * 1e-3),
                       "eval_ms": ev_plain, "solve_build_ms": ms_plain - ev_plain,
                       "solves_per_s": 1e3 / (ms_plain - ev_plain)},
        "speedup_vs_plain_fp64": {"grid_points_per_s": ms_plain / ms_step,
                                  "eval_kernel": ev_plain / ev_mixed,
                                  "solve_build": (ms_plain - ev_plain) / (ms_step - ev_mixed)},
        "kernels": kern,
        "errors_vs_fp64": {"field_rel_max": err_field, "weights_rel_max": err_w, "gradient_rel_max": err_grad,
                           "ids_mismatch_outside_band": mism, "band": band,
                           "solver_residual": float(info_mixed["residual"]),
                           "solver_iterations": int(info_mixed["iterations"])},
        "clocks": clocks,
        "e2e": {"value": n_pts / e2e_s, "unit": "grid points/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "ms_per_step": 1e3 * e2e_s},
        "gpu_launches": launches,
        "gpu_launches_per_step": launches / args.steps,
        "roofline": {"kernel": "gk::eval_ff_kernel (float-float field + fused segmentation, autotuned shape)",
                     "bound": "fp32", "achieved": achieved_tf, "peak": fp32_peak, "unit": "TFLOP/s",
                     "frac": achieved_tf / fp32_peak,
                     # DRAM bytes of one full-size launch from an ncu capture (dram__bytes_read.sum 14.4 MB +
                     # dram__bytes_write.sum 222.3 MB at 256^3 = 16.8M points; scaled by the points here):
                     # the field and soft values written once, the records read once
                     "traffic": int(round(236625152 / 16777216 * n_pts)),
                     "peak_source": f"nominal FP32 SIMT: 152 SMs x 128 lanes x 2 x {sm_mhz:.0f} MHz "
                                    f"(max SM clock from MEASURED_PEAKS.json, {pk['_source']})",
                     "work": f"{fl_pt} algorithmic flops/point x {n_pts} points per launch",
                     "eval_ms": ev_mixed,
                     # float-float executes ~80 thread instructions per point-record pair (ncu count of the
                     # shipped kernel at 64^3, profiles/eval_ff_precision_64.md)
                     # where the algorithmic count has 20: the pipe view
                     "fp32_pipe_ops_per_pair": FF_OPS_PER_PAIR, "algorithmic_flops_per_pair": 20,
                     "fp32_pipe_achieved": achieved_tf * FF_OPS_PER_PAIR / 20,
                     "fp32_pipe_frac": achieved_tf * FF_OPS_PER_PAIR / 20 / fp32_peak},
    }
    if mesh is not None:
        line["mesh"] = mesh
    if not args.no_extra and rank == 0:
        line["plain"] = plain_section()
        line["batch"] = batch_section(n_real=args.batch_realisations)
        line["octree"] = octree_section()
        line["learned"] = learned_section(args.learned_points, args.learned_config)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:   # host cores are shared by all ranks at N > 1
        line["cpu_baseline"] = cpu_baseline(m)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def mesh_section(field, isovalues, grid):
    """Marching cubes of every surface of the precision workload on its 256^3
    dense-grid field (gk_mc_count + gk_mc_emit per surface, one host read of
    the counts in between), timed with CUDA events.  Algorithmic bytes: the
    field read once per surface plus the vertices and triangles written."""
    import torch
    from gempy_gb300 import kernels as K
    res = [int(v) for v in grid.regular_grid_shape]
    ext = np.asarray(grid.orthogonal_extent, dtype=np.float64)
    sp = (ext[1::2] - ext[0::2]) / np.asarray(res, dtype=np.float64)
    f = field.reshape(-1).contiguous()
    out = []

    def run():
        out.clear()
        for lev in isovalues:
            out.append(K.marching_cubes(f, res, float(lev), sp, ext[0::2]))
    run()
    torch.cuda.synchronize()
    ts = []
    for _ in range(3):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        run()
        b.record()
        torch.cuda.synchronize()
        ts.append(a.elapsed_time(b))
    ms = float(np.median(ts))
    nv = sum(int(v.shape[0]) for v, _ in out)
    nt = sum(int(t.shape[0]) for _, t in out)
    n = int(np.prod(res))
    alg = len(isovalues) * n * 8 + nv * 24 + nt * 12
    pk = peaks()
    return {"workload": f"{len(isovalues)} level surfaces of the {res[0]}^3 precision-workload field",
            "ms": ms, "ms_per_surface": ms / len(isovalues), "vertices": nv, "triangles": nt,
            "launches_per_surface": 4,
            "algorithmic_bytes": alg, "achieved_GBps": alg / (ms * 1e-3) / 1e9,
            "hbm_peak_GBps": pk.get("hbm_gbs"),
            "frac_of_hbm": alg / (ms * 1e-3) / 1e9 / pk["hbm_gbs"] if pk.get("hbm_gbs") else None,
            "note": "per surface: a count pass and a vertex pass over the field, a triangle pass over the "
                    "cubes, a scan of block counts; the host reads the two counts to size the outputs"}


def batch_section(n_real=512, res=64, plain=True):
    """Config 4: ``n_real`` uneven realisations, each on its own res^3 grid, in
    one captured CUDA graph (mixed form), against the plain FP64 form run per
    realisation with the single-system kernels."""
    import torch
    from gempy_gb300 import kernels as K
    from gempy_gb300 import synthetic
    from gempy_gb300.batch import BatchRunner
    models = [synthetic.realisation(i, resolution=(res,) * 3) for i in range(n_real)]
    br = BatchRunner(models)
    br.capture()
    stream = torch.cuda.current_stream()
    for _ in range(2):
        br.replay()
    torch.cuda.synchronize()
    evs = []
    for _ in range(3):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        br.replay()
        b.record(stream)
        torch.cuda.synchronize()
        evs.append(a.elapsed_time(b))
    ms = float(np.median(evs))
    infos = br.infos_host()
    out = {"realisations": n_real, "grid": f"{res}^3 each", "points": br.n_points,
           "N_max": int(max(3 * m.n_orientations + m.n_points - 4 + 3 for m in models)),
           "ms": ms, "grid_points_per_s": br.n_points / (ms * 1e-3), "solves_per_s": n_real / (ms * 1e-3),
           "launches_per_replay": 4, "captured_in_cuda_graph": True,
           "solver": {"converged": int((infos["status"] == 0).sum()),
                      "max_residual": float(infos["residual"].max()),
                      "max_iterations": int(infos["iterations"].max())}}
    if plain:
        field_b = br.field.clone()
        ids_b = br.ids.clone()
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        t0.record(stream)
        err, mism = 0.0, 0
        fields = []
        for i, m in enumerate(models):
            ii, dd, ko = m.interpolation_input, m.data_descriptor, m.options.kernel_options
            ds = K.DeviceSeries(ii.orientations.dip_positions, ii.orientations.dip_gradients,
                                ii.orientations.nugget_effect_grad, ii.surface_points.sp_coords,
                                ii.surface_points.nugget_effect_scalar,
                                dd.tensors_structure.number_of_points_per_surface, range=ko.range, c_o=ko.c_o,
                                uni_degree=ko.uni_degree)
            w, _ = K.solve_plain(ds)
            model = K.prepare(ds, w)
            iso_t, _, _, _ = K.evaluate(ds, model, K.Points(xyz=ds.ref_points), K.GK_F64)
            iso = iso_t.cpu().numpy()
            order = np.argsort(-iso, kind="stable")
            seg = K.make_segment(iso[order], ii.unit_values, m.options.sigmoid_slope)
            f, _, _, ids = K.evaluate(ds, model, K.Points.regular(ii.grid.dense_grid), K.GK_F64, seg=seg,
                                      want_ids=True)
            fields.append((f, ids, iso))
        t1.record(stream)
        torch.cuda.synchronize()
        ms_p = t0.elapsed_time(t1)
        for i, (f, ids, iso) in enumerate(fields):
            sl = br.item_slice(i)
            fb = field_b[sl]
            err = max(err, float((fb - f).abs().max() / f.abs().max()))
            band = max(10.0 / models[i].options.sigmoid_slope, 4e-6 * float(f.abs().max()))
            it = torch.as_tensor(iso, device=f.device)
            outside = ((f[:, None] - it[None, :]).abs() > band).all(dim=1)
            mism += int(((ids_b[sl] != ids) & outside).sum())
        out["plain_fp64"] = {"ms": ms_p, "grid_points_per_s": br.n_points / (ms_p * 1e-3),
                             "solves_per_s": n_real / (ms_p * 1e-3),
                             "note": "single-system FP64 kernels, one realisation after another"}
        out["speedup_vs_plain_fp64"] = ms_p / ms
        out["errors_vs_fp64"] = {"field_rel_max": err, "ids_mismatch_outside_band": mism}
    return out


def plain_section():
    """Config 1: the plain horizontal model (2 surfaces x 10 points, 2
    orientations, linear drift, 50^3 dense grid) through compute_model from
    host inputs: plain FP64 and mixed on the GPU, and the FP64 oracle on the
    host cores, all on the full grid."""
    import torch
    import gempy_gb300 as gg
    from gempy_gb300 import synthetic
    from oracle import kriging, segmentation
    from oracle.inputs import series_from_engine_inputs
    from oracle.parallel import FieldPool, host_cores
    m = synthetic.plain_horizontal()
    args_ = (m.interpolation_input, m.options, m.data_descriptor)
    n_pts = m.interpolation_input.grid.dense_grid.n_points
    out = {"workload": "2 horizontal surfaces x 10 points, 2 orientations, cubic, linear drift, 50^3 dense grid",
           "grid_points": n_pts}
    sols = {}
    for name, dt in (("plain_fp64", "float64"), ("mixed", "float32")):
        cfg = gg.EngineConfig(dtype=dt)
        for _ in range(3):
            gg.compute_model(*args_, config=cfg)
        torch.cuda.synchronize()
        reps = 10
        t0 = time.perf_counter()
        for _ in range(reps):
            sols[name] = gg.compute_model(*args_, config=cfg)
        torch.cuda.synchronize()
        dt_s = (time.perf_counter() - t0) / reps
        out[name] = {"ms": 1e3 * dt_s, "points_per_s": n_pts / dt_s, "solves_per_s": 1.0 / dt_s}
    (s,) = series_from_engine_inputs(*args_)
    cores = host_cores()
    with FieldPool(s, cores) as pool:      # spawned workers, started before the timed region
        t0 = time.perf_counter()
        w = kriging.solve(*kriging.build_system(s))
        iso = kriging.isovalues(s, w)
        z = pool.evaluate(m.interpolation_input.grid.dense_grid.values, w)
        segmentation.segment(z, iso, m.interpolation_input.unit_values, m.options.sigmoid_slope)
        t_cpu = time.perf_counter() - t0
    out["cpu_oracle"] = {"ms": 1e3 * t_cpu, "points_per_s": n_pts / t_cpu, "cores": cores, "extrapolated": False,
                         "note": f"the grid evaluated by {cores} worker processes"}
    zp = np.asarray(sols["plain_fp64"].raw_arrays.scalar_field_matrix)[0]
    zm = np.asarray(sols["mixed"].raw_arrays.scalar_field_matrix)[0]
    out["errors"] = {"plain_vs_oracle_rel": float(np.abs(zp - z).max() / np.abs(z).max()),
                     "mixed_vs_plain_rel": float(np.abs(zm - zp).max() / np.abs(zp).max()),
                     "ids_identical": bool(np.array_equal(np.rint(sols["plain_fp64"].raw_arrays.lith_block),
                                                          np.rint(sols["mixed"].raw_arrays.lith_block)))}
    out["speedup_vs_plain_fp64"] = out["plain_fp64"]["ms"] / out["mixed"]["ms"]
    out["speedup_plain_gpu_vs_cpu_oracle"] = t_cpu * 1e3 / out["plain_fp64"]["ms"]
    return out


def octree_section():
    """Config 2: three folded series, quadratic drift, 7 octree levels, through
    compute_model (host inputs), plain FP64 and mixed: 3 warm-up calls, then
    the median of 10 calls each timed alone."""
    import torch
    import gempy_gb300 as gg
    from gempy_gb300 import synthetic
    m = synthetic.folded_series(octree_levels=7)
    out = {"workload": "3 series x 2 folded surfaces, 200 points, 60 orientations, quadratic drift, "
                       "7 octree levels (128^3 effective)"}
    for name, dt in (("plain_fp64", "float64"), ("mixed", "float32")):
        cfg = gg.EngineConfig(dtype=dt)
        for _ in range(3):
            gg.compute_model(m.interpolation_input, m.options, m.data_descriptor, config=cfg)
        torch.cuda.synchronize()
        times = []
        for _ in range(10):   # each call timed alone (host inputs, results on the host)
            t0 = time.perf_counter()
            sol = gg.compute_model(m.interpolation_input, m.options, m.data_descriptor, config=cfg)
            torch.cuda.synchronize()
            times.append(time.perf_counter() - t0)
        dt_s = float(np.median(times))
        npts = sum(len(l.grid_centers) for l in sol.octrees_output)
        out[name] = {"ms": 1e3 * dt_s, "mean_ms": 1e3 * float(np.mean(times)), "calls": len(times),
                     "octree_points": npts, "points_per_s": npts / dt_s,
                     "levels": [len(l.grid_centers) for l in sol.octrees_output]}
        out.setdefault("_ids", {})[name] = sol.octrees_output[-1].last_output_center.ids_block
    a, b = out.pop("_ids").values()
    out["ids_identical_last_level"] = bool(np.array_equal(a, b))
    out["speedup_vs_plain_fp64"] = out["plain_fp64"]["ms"] / out["mixed"]["ms"]
    return out


def learned_section(n_points=20000, force_config=None):
    """Config 5: one 20000-point / 6000-orientation multi-fold system
    (N = 37993; ``n_points`` scales it down for profiling).  Plain FP64 form (build + blocked LU + solves) against the
    learned form (network picks the two-level configuration, FGMRES to 1e-8,
    FP64 LU fallback), with the fixed default configuration as the ablation;
    the LU solution is the reference for the scalar field.  Also times the network kernels."""
    import torch
    from gempy_gb300 import kernels as K
    from gempy_gb300 import learned, synthetic
    forced = None
    if force_config:
        r_, bs_, pol_, pr_ = force_config.split(",")
        forced = learned.PrecondConfig(int(r_), int(bs_), pol_, {"f32": K.GK_F32, "ff": K.GK_FF, "f64": K.GK_F64}[pr_])
    elif not os.path.exists(learned.DEFAULT_MODEL):
        return {"unavailable": "no trained model in the package"}
    model = None if forced else learned.CostModel.load()
    m = synthetic.learned(n_points=n_points, n_orient=int(0.3 * n_points))
    s = learned.series_of(m)

    def clock(fn):
        torch.cuda.synchronize()
        t = time.perf_counter()
        r = fn()
        torch.cuda.synchronize()
        return r, time.perf_counter() - t

    (Kt, bt), t_build = clock(lambda: K.build(s, K.GK_F64))
    N = int(Kt.shape[0])
    (x_lu, _), t_lu = clock(lambda: learned.solve_plain_K(Kt, bt))
    pts = learned.check_points(s)
    f_lu = learned.field_at(s, x_lu, pts)
    res, t_learned = clock(lambda: learned.solve_learned(s, model, Kt, bt, tol=1e-8, config=forced))
    err = learned.field_error(s, res.x, f_lu, pts)
    (xd, infd), t_def = clock(lambda: learned.solve_with(s, learned.DEFAULT_CONFIG, Kt, bt, 1e-8))
    def_ok = int(infd["status"]) == 0
    t_def_total = t_def if def_ok else t_def + t_lu
    # network kernels: inference over a large batch and one training step
    # the dominant per-iteration kernel: the FP64 product K v of FGMRES (gk_gemv), CUDA events
    xv = torch.randn(N, dtype=torch.float64, device="cuda")
    for _ in range(3):
        K.gemv(Kt, xv)
    g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    g0.record()
    for _ in range(10):
        K.gemv(Kt, xv)
    g1.record()
    torch.cuda.synchronize()
    gemv_ms = g0.elapsed_time(g1) / 10
    pk = peaks()
    gemv_gbs = N * N * 8 / (gemv_ms * 1e-3) / 1e9
    gemv_tf = 2.0 * N * N / (gemv_ms * 1e-3) / 1e12
    roof = {"kernel": "gk::gemv_kernel (FP64 K v of FGMRES, 4 rows per warp)", "bound": "fp64",
            "achieved": gemv_tf, "peak": 1.25, "unit": "TFLOP/s", "frac": gemv_tf / 1.25,
            "peak_source": "nominal GB300 FP64 rate (no measured FP64 peak is available)",
            "hbm_gbs": gemv_gbs, "hbm_frac_of_measured": gemv_gbs / pk["hbm_gbs"],
            "work": f"{N}^2 x 8 bytes and 2 x {N}^2 flops per launch", "ms": gemv_ms}
    if model is None:
        model = learned.CostModel(learned.Mlp(), np.zeros(learned.IN_DIM), np.ones(learned.IN_DIM),
                                  np.zeros(learned.OUT_DIM), np.ones(learned.OUT_DIM), {"untrained": True})
    B = 65536
    x = torch.randn(B, learned.IN_DIM, device="cuda")
    for _ in range(3):
        model.mlp.forward(x)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    reps = 10
    for _ in range(reps):
        model.mlp.forward(x)
    ev1.record()
    torch.cuda.synchronize()
    fwd_ms = ev0.elapsed_time(ev1) / reps
    for _ in range(3):
        model.mlp.forward_tc(x)
    ev0.record()
    for _ in range(reps):
        model.mlp.forward_tc(x)
    ev1.record()
    torch.cuda.synchronize()
    tc_ms = ev0.elapsed_time(ev1) / reps
    flops = 2.0 * B * (256 * (learned.IN_DIM + 1) + 256 * 257 + learned.OUT_DIM * 257)
    return {
        "workload": f"{n_points} surface points, {int(0.3 * n_points)} orientations, 10 folded surfaces, "
                    "linear drift",
        "N": N,
        "build_s": t_build,
        "plain_fp64_lu_s": t_lu,
        "learned": {"s": t_learned, "config": None if res.config is None else vars(res.config),
                    "iterations": res.iterations, "residual": res.residual, "fallback_to_lu": res.fallback,
                    "choose_ms": 1e3 * res.seconds_choose, "field_rel_err_vs_lu": err},
        "default_config": {"s": t_def_total, "config": vars(learned.DEFAULT_CONFIG), "converged": def_ok,
                           "iterations": int(infd["iterations"])},
        "solves_per_s": {"plain_fp64": 1.0 / t_lu, "learned": 1.0 / t_learned,
                         "default_config": 1.0 / t_def_total},
        "speedup_vs_plain_fp64": t_lu / t_learned,
        "roofline": roof,
        "gain_vs_default_config": t_def_total / t_learned,
        "network": {"samples_per_forward": B, "forward_ms": fwd_ms, "forward_tflops": flops / (fwd_ms * 1e-3) / 1e12,
                    "forward_tc_ms": tc_ms, "forward_tc_tflops": flops / (tc_ms * 1e-3) / 1e12,
                    "training": model.meta},
    }


def cpu_baseline(m, sample_per_core=4096):
    from oracle import kriging, segmentation
    from oracle.inputs import series_from_engine_inputs
    from oracle.parallel import FieldPool, host_cores
    (s,) = series_from_engine_inputs(m.interpolation_input, m.options, m.data_descriptor)
    grid = m.interpolation_input.grid.dense_grid
    n_total = grid.n_points
    cores = host_cores()
    sample = sample_per_core * cores
    rng = np.random.default_rng(0)
    idx = np.sort(rng.choice(n_total, sample, replace=False))
    xs = grid.values[idx]
    with FieldPool(s, cores) as pool:      # spawned workers: safe after the GPU work in this process
        t0 = time.perf_counter()
        K, b = kriging.build_system(s)
        w = kriging.solve(K, b)
        iso = kriging.isovalues(s, w)
        t1 = time.perf_counter()
        z = pool.evaluate(xs, w)
        segmentation.segment(z, iso, m.interpolation_input.unit_values, m.options.sigmoid_slope)
        t2 = time.perf_counter()
    t_step = (t1 - t0) + (t2 - t1) / sample * n_total
    return {"value": n_total / t_step, "unit": "grid points/s", "cores": cores, "kind": "port",
            "extrapolated": True, "sample_points": sample,
            "sample": f"FP64 numpy/scipy oracle: full build+LU (N={s.size}, BLAS on all {cores} cores) + "
                      f"{sample}-point subsample of the grid evaluated by {cores} worker processes, "
                      f"extrapolated to {n_total} points",
            "solve_s": t1 - t0, "eval_s_per_point": (t2 - t1) / sample}


if __name__ == "__main__":
    main()
