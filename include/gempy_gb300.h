/*
 * gempy_gb300 -- C ABI of the GB300 co-kriging hot path.
 *
 * The reference has exactly one production entry into the arithmetic of this
 * path: ``gempy_engine.compute_model(interpolation_input, options,
 * data_descriptor, geophysics_input)`` called at
 * ``gempy/API/compute_API.py:68-73`` (also ``gempy/modules/optimize_nuggets/
 * _ops.py:18-23`` and ``compute_API.py:140-145``).  That engine is a Python
 * package with no native code; its four steps -- kriging-matrix build, dense
 * solve, field/gradient evaluation on regular and octree grids, sigmoid
 * segmentation -- are what the functions below replace.  The Python package
 * ``gempy_gb300`` binds them with ctypes and mirrors the engine's
 * ``compute_model`` signature on top.
 *
 * Conventions
 *  - Every pointer argument is a DEVICE pointer unless its comment says HOST.
 *  - Matrices are row-major with a leading dimension (``ld*``) in elements.
 *  - The caller allocates every buffer (query sizes with the *_bytes calls);
 *    the library allocates no device memory and keeps no device state.
 *  - Work is enqueued on ``stream`` (a cudaStream_t; NULL = legacy stream).
 *    Functions return after enqueueing; device-side failures (singular pivot,
 *    iteration caps, non-finite values) are reported through a caller-provided
 *    device ``gk_info`` word, which the caller reads after synchronising.
 *  - No exception crosses this ABI, and there is no CPU fallback: without a
 *    usable CUDA device every call returns GK_ERR_CUDA.
 */
#ifndef GEMPY_GB300_H
#define GEMPY_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* gk_stream; /* == cudaStream_t */

typedef enum gk_status {
    GK_OK = 0,
    GK_ERR_ARG = 1,           /* NULL pointer, negative size, bad enum        */
    GK_ERR_SIZE = 2,          /* size above a documented limit / workspace too small */
    GK_ERR_CUDA = 3,          /* a CUDA runtime call failed (launch, no device) */
    GK_ERR_SINGULAR = 4,      /* zero pivot met during LU (device info)       */
    GK_ERR_NOT_CONVERGED = 5, /* iteration cap hit (device info)              */
    GK_ERR_NONFINITE = 6,     /* NaN/Inf met (device info)                    */
    GK_ERR_TIMEOUT = 7        /* an inter-CTA wait gave up (device info)      */
} gk_status;

/* Arithmetic of a kernel.  GK_FF is float-float ("double-single"): values
 * carried as pairs of FP32 words (~48-bit significand) on the FP32 pipe,
 * available for the field evaluation of the cubic kernel. */
typedef enum gk_prec { GK_F64 = 0, GK_F32 = 1, GK_FF = 2 } gk_prec;

/* ``kernel_function`` of the reference's KernelOptions (serialized options
 * JSON, ``...serialization.approved.txt:135``). */
typedef enum gk_kernel { GK_KERNEL_CUBIC = 0, GK_KERNEL_EXPONENTIAL = 1 } gk_kernel;

/* Device status word written by the kernels.  ``status`` is a gk_status;
 * ``where`` locates the failure (pivot column, iteration, ...); the solver
 * fields report refinement progress; ``pivoted`` is set by gk_solve_mixed
 * when its FP32 factorization had to fall back to partial pivoting. */
typedef struct gk_info {
    int32_t status;
    int32_t where;
    int32_t iterations;
    int32_t pivoted;
    double residual;          /* final ||b - K x||_inf / ||b||_inf (solvers) */
} gk_info;

/* One series' kriging inputs, FP64 device arrays in the engine's transformed
 * frame.  Field meaning follows ``InterpolationInput`` as built at
 * ``gempy/modules/data_manipulation/_engine_factory.py:27-56``:
 * ``SurfacePoints(sp_coords, nugget_effect_scalar)`` and
 * ``Orientations(dip_positions, dip_gradients, nugget_effect_grad)``; the
 * options are ``KernelOptions{range, c_o, uni_degree, i_res, gi_res,
 * kernel_function}``.  ``ref_index``/``rest_index`` give, per interface row,
 * the surface's reference point and the other ("rest") point.
 *
 * Fault drift: ``n_fault`` older FAULT series offset this one (the engine's
 * ``faults_relations``, set by ``gempy/core/data/structural_frame.py:
 * 244-273``).  Each adds one drift unknown whose function is that fault's
 * block -- its segmented soft values -- given at this series' surface points
 * in ``fault_sp`` (n_fault x n_sp, row per fault); the unknown comes after the
 * polynomial drift, with gi_res (F(rest) - F(ref)) on the interface rows and
 * 0 on the gradient rows. */
#define GK_MAX_FAULTS 16
typedef struct gk_system {
    int32_t n_ori;        /* orientations                                    */
    int32_t n_sp;         /* surface points of the series                    */
    int32_t n_iface;      /* interface rows = n_sp - n_surfaces              */
    int32_t uni_degree;   /* 0, 1 or 2 (drift functions: 0, 3, 9)            */
    int32_t kernel;       /* gk_kernel                                       */
    int32_t n_fault;      /* 0 .. GK_MAX_FAULTS fault-drift unknowns         */
    double range, c_o, i_res, gi_res;
    const double* dip_positions; /* n_ori x 3 */
    const double* dip_gradients; /* n_ori x 3 */
    const double* nugget_grad;   /* n_ori     */
    const double* sp_coords;     /* n_sp x 3  */
    const double* nugget_sp;     /* n_sp      */
    const int32_t* ref_index;    /* n_iface   */
    const int32_t* rest_index;   /* n_iface   */
    const double* fault_sp;      /* n_fault x n_sp (may be NULL if n_fault 0) */
} gk_system;

/* Evaluation points.  kind 0: regular grid of cell centres generated in the
 * kernel, ``ij`` order (x slowest, z fastest) as the reference's
 * ``RegularGrid`` (``gempy/core/data/grid_modules/regular_grid.py:58-71,
 * 192-201``); kind 1: an explicit n x 3 FP64 list (octree centres/corners,
 * custom grid, surface points).  ``fault_values`` holds, for a series with
 * fault drift, the blocks of its n_fault offsetting faults at these points
 * (row f at fault_values + f * fault_ld, fault_ld >= n; the soft values
 * gk_eval wrote for that fault series); NULL when the series has none. */
typedef struct gk_points {
    int32_t kind;
    int32_t dims[3];
    int64_t n;
    double origin[3];     /* first cell centre (kind 0)                      */
    double spacing[3];    /* cell size (kind 0)                              */
    const double* xyz;    /* n x 3 (kind 1)                                  */
    const double* fault_values; /* n_fault x fault_ld, or NULL               */
    int64_t fault_ld;
} gk_points;

/* Segmentation of one series (``sigmoid_slope``, element ids, isovalues).
 * ``n_surf`` <= GK_MAX_SURFACES; isovalues are the series' surfaces sorted by
 * isovalue, highest first; ``unit_values`` has n_surf + 1 entries. All HOST
 * values (copied into the launch).  Soft values are
 * u_0 + sum_k (u_(k+1) - u_k) sigmoid(slope (z_k - Z)); block ids are their
 * slope -> infinity limit, u_0 + sum_k (u_(k+1) - u_k) [Z < z_k - GK_TIE_TOL]:
 * rint(soft value) except that a point lying on a surface (an octree corner
 * on a surface's reference point) takes the unit above it. */
#define GK_TIE_TOL 1e-9
#define GK_MAX_SURFACES 32
typedef struct gk_segment {
    int32_t n_surf;
    int32_t reserved;
    double slope;
    double isovalues[GK_MAX_SURFACES];
    double unit_values[GK_MAX_SURFACES + 1];
} gk_segment;

/* ---------------- kriging-matrix build (engine covariance build) -------- */

/* N = 3 n_ori + n_iface + n_drift + n_fault. */
int64_t gk_system_size(const gk_system* sys /* HOST struct */);

/* Fills K (N x N, row-major, ld ``ldk`` >= N) and rhs (N) in ``prec``
 * (double* for GK_F64, float* for GK_F32).  Replaces the engine's covariance
 * build reached from ``compute_API.py:68-73``. */
gk_status gk_build(const gk_system* sys, gk_prec prec, void* K, int64_t ldk,
                   void* rhs, gk_stream stream);

/* The FP64 build from covariance tables: C over every pair of surface
 * points, C'/r (x_o - x_p) over every orientation-point pair and the
 * gradient-gradient terms over every orientation pair are formed once in
 * ``work`` (gk_build_tables_bytes), then the covariance entries are
 * assembled from them with the operations of gk_build -- the same matrix (to
 * rounding) with a fraction of the covariance evaluations.  The workspace is
 * n_sp^2 + 3 n_ori n_sp + 6 n_ori^2 doubles (16-byte aligned).  Same
 * reference call site as gk_build. */
size_t gk_build_tables_bytes(const gk_system* sys /* HOST struct */);
gk_status gk_build_tables(const gk_system* sys, double* K, int64_t ldk,
                          double* rhs, void* work, size_t work_bytes,
                          gk_stream stream);

/* ---------------- dense solve (engine ``kernel_solver``, approved JSON :136) */

/* Workspace for gk_lu_factor (device bytes). */
size_t gk_lu_workspace_bytes(gk_prec prec, int64_t n);

/* Blocked right-looking LU with partial pivoting, in place: A = P L U with
 * ipiv[i] (0-based) the row swapped with row i (LAPACK getrf semantics). */
gk_status gk_lu_factor(gk_prec prec, int64_t n, void* A, int64_t lda,
                       int32_t* ipiv, void* work, size_t work_bytes,
                       gk_info* info, gk_stream stream);

/* Engine of the FP32 trailing updates (Schur-complement products) of every
 * FP32 factorization -- gk_lu_factor(GK_F32), the FP32 preconditioner of
 * gk_solve_mixed and the FP32 two-level setup of gk_solve_twolevel: the
 * tensor cores (GK_LU_UPDATE_TC, the default: tcgen05.mma kind::tf32 with
 * split operands, three TF32 products per update, ~FP32 accuracy) or the
 * FP32 SIMT pipe (GK_LU_UPDATE_SIMT).  Process-wide; the FP64 updates always
 * run on the FP64 pipe.  No reference counterpart: the engine's solve is a
 * library call. */
#define GK_LU_UPDATE_SIMT 0
#define GK_LU_UPDATE_TC 1
gk_status gk_lu_update_select(int32_t engine);
int32_t gk_lu_update_engine(void);

/* Solves A x = b with the factors of gk_lu_factor; b is overwritten by x.
 * ``work`` must be the workspace the factorization used: it holds the row
 * permutation gk_lu_factor derived from ipiv. */
gk_status gk_lu_solve(gk_prec prec, int64_t n, const void* LU, int64_t lda,
                      const int32_t* ipiv, void* b, void* work,
                      size_t work_bytes, gk_info* info, gk_stream stream);

/* y = K x for the FP64 matrix (row-major, ld ``ldk``); x and y must not
 * overlap.  Used with gk_lu_solve for the condition-number estimate the
 * engine reports when ``KernelOptions.compute_condition_number`` is set. */
gk_status gk_gemv(int64_t n, const double* K, int64_t ldk, const double* x,
                  double* y, gk_stream stream);

/* Mixed-precision solve of the FP64 system K x = b (no reference
 * counterpart beyond the FP64 solve it replaces): an FP32 copy of the
 * symmetrically equilibrated K is LU-factored on the GPU -- without pivoting
 * (the equilibrated covariance block is SPD with unit diagonal; the drift
 * block comes last), or with partial pivoting if a pivot is zero or
 * non-finite -- and preconditions an
 * FP64 restarted FGMRES(50) whose residuals r = b - K x use the FP64 K, until
 * ||r||_2 <= tol ||b||_2, stagnation, or ``max_iter`` Krylov steps.  ``work``
 * holds the FP32 factors and the Krylov vectors
 * (gk_solve_mixed_workspace_bytes); ``info`` receives the status, the
 * iteration count and the final relative residual. */
size_t gk_solve_mixed_workspace_bytes(int64_t n);
gk_status gk_solve_mixed(int64_t n, const double* K, int64_t ldk,
                         const double* b, double* x, double tol,
                         int32_t max_iter, void* work, size_t work_bytes,
                         gk_info* info, gk_stream stream);

/* Single-CTA form of gk_solve_mixed for small systems (n <= GK_CTA_MAX_N),
 * e.g. the series of an octree model (no reference counterpart beyond the
 * FP64 solve it replaces): one thread block equilibrates K, factors an FP32
 * copy without pivoting and runs FGMRES(30) in FP64 on the FP64 K with the
 * Givens rotations and convergence tests on the device, so the call queues one
 * launch and never synchronises the host.  A zero or non-finite pivot is
 * reported as GK_ERR_SINGULAR (the caller then uses gk_solve_mixed, which
 * refactors with partial pivoting).  FGMRES stops at
 * ||b - K x||_2 <= tol ||b||_2, at ``max_iter`` steps or when a restart cycle
 * gains less than 2 %; ``info`` (written by the kernel, may be NULL) reports
 * status, iterations and the residual.  ``work``:
 * gk_solve_mixed_cta_workspace_bytes(n, ldk) bytes (K's FP32 copy with the
 * same leading dimension, Krylov vectors). */
#define GK_CTA_MAX_N 4096
size_t gk_solve_mixed_cta_workspace_bytes(int64_t n, int64_t ldk);
gk_status gk_solve_mixed_cta(int64_t n, const double* K, int64_t ldk,
                             const double* b, double* x, double tol,
                             int32_t max_iter, void* work, size_t work_bytes,
                             gk_info* info, gk_stream stream);

/* Up to GK_CTA_MAX_JOBS independent systems (the series of one model) solved
 * as gk_solve_mixed_cta in one launch, one thread block each.  ``jobs`` is a
 * HOST array; each job's arguments mean what gk_solve_mixed_cta's do. */
#define GK_CTA_MAX_JOBS 16
typedef struct gk_cta_job {
    int64_t n;
    const double* K;
    int64_t ldk;
    const double* b;
    double* x;
    void* work;
    size_t work_bytes;
    gk_info* info;
} gk_cta_job;
gk_status gk_solve_mixed_cta_many(int32_t n_jobs, const gk_cta_job* jobs,
                                  double tol, int32_t max_iter,
                                  gk_stream stream);

/* FGMRES on the FP64 system K x = b preconditioned by a two-level
 * "block-Jacobi plus low-rank" operator, for systems too large for an LU
 * preconditioner (no reference counterpart beyond the FP64 solve it
 * replaces).  ``perm`` (device, n entries) lists the unknowns in the new order:
 * first ``r`` landmark unknowns (r a multiple of 64; the drift unknowns must be
 * among them), then the others in spatially contiguous blocks of ``bs`` (a
 * multiple of 64, at most 4096).  Setup, in ``prec`` (GK_F32, GK_FF or GK_F64)
 * on the equilibrated, permuted matrix: LU without pivoting of the landmark block,
 * the landmark rows/columns (the rank-r coupling), and LU of the bs x bs
 * diagonal blocks of the Schur complement (with FP64 storage, then their
 * explicit inverses, kept in unused off-diagonal space, when at least two
 * blocks are full).  GK_F32 halves the setup's memory traffic but only
 * preconditions systems with kappa(K) eps32 well below 1; GK_F64 covers the
 * densely sampled, nugget-dominated systems beyond that; GK_FF keeps FP64
 * storage but runs the O(N r^2) restricted updates in float-float on the FP32
 * pipe (~1e-12 relative per update), several times faster than FP64 on this
 * part.  The Krylov iteration is FGMRES(200) in FP64 on the FP64 K, to
 * ||b - K x||_2 <= tol ||b||_2 or ``max_iter`` steps (it also stops when a
 * whole restart cycle gains less than 2 %); ``info`` reports status,
 * iterations and the final residual.  ``x0`` (device, may be NULL; must not
 * be ``x``) is the initial guess -- the engine passes the series' previous
 * weights (``InterpolationInput.weights``) -- otherwise FGMRES starts from 0. */
size_t gk_solve_twolevel_workspace_bytes(int64_t n, gk_prec prec);
gk_status gk_solve_twolevel(int64_t n, const double* K, int64_t ldk,
                            const double* b, double* x, const double* x0,
                            const int32_t* perm,
                            int64_t r, int32_t bs, gk_prec prec, double tol,
                            int32_t max_iter, void* work, size_t work_bytes,
                            gk_info* info, gk_stream stream);

/* Allocation-free form of gk_solve_mixed, with no counterpart in the
 * reference.  It is for callers that cannot call cudaMalloc -- for example
 * code running inside a framework that owns the whole device-memory budget
 * through its own pool or caching allocator and forbids side allocations, or a
 * host runtime that binds this C ABI but has no way to hand it device
 * workspace.  The solver's scratch is a file-scope device array of the
 * library (8 MiB, held on every GPU that loads the library until the process
 * exits), so only systems with n <= GK_NOALLOC_MAX_N are accepted; larger n
 * returns GK_ERR_SIZE before any work is queued.  The caller still passes K,
 * b and x.  Like gk_solve_mixed it synchronizes its stream between Krylov
 * steps and reads results on the host, so it cannot be captured in a CUDA
 * graph.  The first call made on a device looks up the array's device
 * address (cudaGetSymbolAddress), which is kept for the life of the process:
 * after a cudaDeviceReset the library must be reloaded before this entry
 * point is called again.  All calls share the one array: calls that overlap on the GPU
 * race, so serialize them (one stream, or explicit ordering).  Nothing here
 * calls cudaMalloc, cudaFree or an allocating library routine.  Arguments,
 * results and ``info`` are as for gk_solve_mixed (``info`` may be NULL). */
#define GK_NOALLOC_MAX_N 1024
gk_status gk_solve_mixed_noalloc(int64_t n, const double* K, int64_t ldk,
                                 const double* b, double* x, double tol,
                                 int32_t max_iter, gk_info* info,
                                 gk_stream stream);

/* ---------------- evaluation + segmentation (engine evaluation) ---------- */

/* Packs the solved model (weights ``w`` of length N) into the layout the
 * evaluation kernels read: ``model`` must hold gk_eval_model_bytes bytes. */
size_t gk_eval_model_bytes(const gk_system* sys);
gk_status gk_eval_prepare(const gk_system* sys, const double* w, void* model,
                          gk_stream stream);

/* Scalar field (times gi_res, the engine's reported scale), optional
 * gradient (n x 3), optional soft segmentation values and ids.  ``info``
 * (may be NULL) receives GK_ERR_TIMEOUT if a wait for a staged record tile
 * gives up (the outputs are then incomplete).  ``prec``
 * selects FP64, FP32 or float-float arithmetic (GK_FF: field only, cubic
 * kernel); outputs are always FP64 for field/values and int32 for ids.  Any
 * output pointer may be NULL.  ``seg`` may be NULL (no segmentation). */
gk_status gk_eval(const gk_system* sys, const void* model,
                  const gk_points* pts, gk_prec prec,
                  const gk_segment* seg, double* field, double* grad,
                  double* values, int32_t* ids, gk_info* info,
                  gk_stream stream);

/* Every series of a model at one point set, in stack order, then their
 * combination (the engine's evaluation of all stacks at a grid, reached from
 * ``compute_API.py:68-73``): series i is evaluated as by gk_eval with its
 * segmentation, the soft values of the FAULT series listed in ``faults``
 * serving as its fault blocks (each must be an older series), into row i of
 * ``fields``, ``values`` and ``ids`` (n_series x n); then gk_combine_series
 * writes ``block``, ``lith_ids`` and ``masks`` (any may be NULL: no
 * combination).  ``series`` is a HOST array. */
typedef struct gk_series_eval {
    const gk_system* sys;       /* HOST                                      */
    const void* model;          /* packed model (gk_eval_prepare)           */
    gk_segment seg;
    int32_t relation;           /* 1 ERODE, 2 ONLAP, 3 FAULT, 4 BASEMENT     */
    int32_t n_faults;           /* == sys->n_fault                           */
    int32_t faults[GK_MAX_FAULTS];  /* indices of the offsetting series     */
    double min_iso, max_iso;    /* the series' extreme isovalues             */
} gk_series_eval;
gk_status gk_eval_series_set(int32_t n_series, const gk_series_eval* series,
                             const gk_points* pts, gk_prec prec,
                             double* fields, double* values, int32_t* ids,
                             double* block, int32_t* lith_ids,
                             uint8_t* masks, gk_info* info, gk_stream stream);

/* Combination of series with the squeezed masks (ERODE / ONLAP / FAULT /
 * BASEMENT, ``gempy/core/data/structural_frame.py:326-330``; a FAULT series
 * owns no lithology): ``fields``, ``values`` and ``ids`` (block ids) are
 * n_series x n (row per series), ``relations`` and ``min_iso``/``max_iso`` are
 * HOST arrays of n_series.  Writes the final soft values, the lithology ids
 * and the squeezed masks (uint8, n_series x n, may be NULL). */
gk_status gk_combine_series(int32_t n_series, int64_t n, const double* fields,
                            const double* values, const int32_t* ids,
                            const int32_t* relations,
                            const double* min_iso, const double* max_iso,
                            double* out_values, int32_t* out_ids,
                            uint8_t* masks, gk_stream stream);

/* ---------------- octree refinement (engine octree) --------------------- */

/* Voxel corners: 8 per centre, corner order x slowest, z fastest. */
gk_status gk_octree_corners(int64_t n, const double* centres,
                            const double spacing[3] /* HOST */,
                            double* corners, gk_stream stream);

/* Marks voxels whose 8 corners differ in any of ``n_id_sets`` id arrays
 * (``corner_ids``: n_id_sets x 8n, row per set -- the lithology ids followed
 * by each fault series' block ids), or all voxels when ``refine_all``, and
 * writes the children of marked voxels (8 each, same corner order, at centre
 * +- spacing/4) in parent order.  ``count`` (device int64) receives the number
 * of children; ``work`` needs gk_octree_workspace_bytes(n). */
size_t gk_octree_workspace_bytes(int64_t n);
gk_status gk_octree_refine(int64_t n, const double* centres,
                           const int32_t* corner_ids, int32_t n_id_sets,
                           int32_t refine_all,
                           const double spacing[3] /* HOST */,
                           double* children, int64_t* count, void* work,
                           size_t work_bytes, gk_stream stream);

/* One level of the octree loop of compute_model (gempy/API/compute_API.py:
 * 68-73 over the octree grid of gempy/core/data/grid.py:128-151) in one call:
 * the level's points -- its voxel centres, followed by 8 corners per voxel
 * when ``corners`` -- every series at those points and their combination
 * (gk_eval_series_set), and, when ``refine`` (1: voxels whose corners differ
 * in lithology or in the block of a fault series ``fault_series[0..
 * n_fault_sets-1]``; 2: every voxel; 3: as 1, plus the voxels whose
 * interpolation error is an outlier -- in some series, |Z(centre) - mean of
 * the 8 corners| / std of the 8 corners above the level's mean of that error
 * by ``error_threshold`` (> 0) of its standard deviations, and above 1e-6:
 * the engine's ``octree_error_threshold`` test), the children of the refined
 * voxels and 8 x their count.  Every output lands in one device buffer of ``total``
 * bytes laid out by gk_octree_level_plan (byte offsets, 256-aligned):
 *   points   n_points x 3 FP64      fields, values  n_series x n_points FP64
 *   ids      n_series x n_points i32   block  n_points FP64
 *   lith_ids n_points i32           masks  n_series x n_points u8
 *   children 8n x 3 FP64            count  int64 (refine only), then scratch
 *   (refine 3 also keeps the errors, n_series x n FP64, there).
 * Everything before ``children`` is the level's result; ``children[0..count)``
 * are the next level's centres.  ``centres`` may lie in the previous level's
 * buffer. */
typedef struct gk_octree_level_layout {
    int64_t n;          /* voxels of the level                        */
    int64_t n_points;   /* n, or 9n with corners                      */
    int32_t n_series;
    int32_t corners;    /* 1: points are [centres; corners]           */
    int32_t refine;     /* 0: last level, 1: marked voxels, 2: all,
                           3: marked by corners or by the error test  */
    int32_t reserved;
    uint64_t points, fields, values, ids, block, lith_ids, masks;
    uint64_t children, count, work, total;
} gk_octree_level_layout;
gk_status gk_octree_level_plan(int32_t n_series, int64_t n, int32_t corners,
                                 int32_t refine, gk_octree_level_layout* out);
gk_status gk_octree_level(int32_t n_series, const gk_series_eval* series,
                          const double* centres,
                          const double spacing[3] /* HOST */, gk_prec prec,
                          int32_t n_fault_sets,
                          const int32_t* fault_series /* HOST */,
                          double error_threshold,
                          const gk_octree_level_layout* layout /* HOST */,
                          void* buf, size_t buf_bytes, gk_info* info,
                          gk_stream stream);

/* ---------------- adjoint derivatives (engine autodiff) ------------------ */

/* Reverse-mode derivatives of J = sum_x g(x) Z(x) for one series, the
 * gradients the reference takes through compute_model with a PyTorch tape
 * (``compute_grads``, checked against central differences at
 * test/test_modules/test_ad/test_ad_I.py:158-258; used by the nugget
 * optimiser, gempy/modules/optimize_nuggets/_optimizer.py:9-62).  With
 * Z(x) = sum_i w_i e_i(x) and K w = b:
 *   gk_adjoint_rhs    r = sum_x g(x) e(x)                         (N)
 *   solve K lambda = r (K is symmetric: the forward LU factors serve)
 *   gk_build_adjoint  -lambda^T (dK/dtheta) w for theta = surface-point
 *                     coordinates (n_sp x 3), orientation positions
 *                     (n_ori x 3) and, when not NULL, the nuggets of the
 *                     surface points (n_sp) and orientations (n_ori); the
 *                     outputs are overwritten
 *   gk_eval_adjoint   adds sum_x g(x) dZ(x)/dtheta at fixed weights (the
 *                     surface points' and orientations' positions) into the
 *                     same position outputs; ``model`` from gk_eval_prepare
 *   dJ/d(dip gradient of orientation o, component u) = lambda[u n_ori + o].
 * The fault-drift functions (other series' blocks) are held constant; ``g``
 * has pts->n entries. */
gk_status gk_adjoint_rhs(const gk_system* sys, const gk_points* pts,
                         const double* g, double* r, gk_stream stream);
gk_status gk_build_adjoint(const gk_system* sys, const double* lambda,
                           const double* w, double* d_sp, double* d_dip,
                           double* d_nugget_sp, double* d_nugget_grad,
                           gk_stream stream);
gk_status gk_eval_adjoint(const gk_system* sys, const void* model,
                          const gk_points* pts, const double* g, double* d_sp,
                          double* d_dip, gk_stream stream);

/* ---------------- mesh extraction (marching cubes) ----------------------- */

/* One level surface of a dense-grid field, the mesh the reference makes per
 * structural element with skimage.measure.marching_cubes(volume, level,
 * spacing, mask, method="lewiner") and the extent minimum added
 * (gempy/modules/mesh_extranction/marching_cubes.py:12-56, 86-98).  A cube
 * is processed when ``mask`` is set at its far corner (lower corner + 1 on
 * every axis); a grid edge that the level crosses and that a processed cube
 * holds carries one vertex (ids in edge order 3 * point + axis, position
 * (i + t) * spacing + origin); the vertex counts of the reference's
 * combination model test follow this rule (test/test_modules/
 * test_marching_cubes.py:44-47).  Triangles come cube by cube: each cube's
 * F <= level boundary cycles on its faces (four-crossing faces split by the
 * bilinear saddle value), fanned from their first edge, oriented with
 * F <= level on the left of each cube-face segment seen from outside. */
typedef struct gk_mc_volume {
    const double* field;   /* dims[0] x dims[1] x dims[2], ij order (z fastest) */
    const uint8_t* mask;   /* same layout, nonzero = inside; NULL = all points  */
    int32_t dims[3];
    int32_t reserved;
    double level;
    double spacing[3];
    double origin[3];      /* position of grid point (0,0,0)                  */
} gk_mc_volume;
/* Workspace of gk_mc_count / gk_mc_emit (0 for invalid dims).  3 * points
 * must stay below 2^31 (vertex ids are int32). */
size_t gk_mc_workspace_bytes(const int32_t dims[3]);
/* Counts the vertices and triangles: counts[0], counts[1] (device int64),
 * and keeps per-block offsets in ``work`` for gk_mc_emit. */
gk_status gk_mc_count(const gk_mc_volume* vol, void* work, size_t work_bytes,
                      int64_t* counts, gk_stream stream);
/* Writes vertices (n_v x 3 FP64) and triangles (n_t x 3 int32) after a
 * gk_mc_count of the same volume on the same workspace; writes beyond
 * max_vertices / max_faces are dropped. */
gk_status gk_mc_emit(const gk_mc_volume* vol, void* work, size_t work_bytes,
                     double* vertices, int64_t max_vertices, int32_t* faces,
                     int64_t max_faces, gk_stream stream);

/* ---------------- forward gravity (engine geophysics) -------------------- */

/* Vertical attraction per unit density of each voxel of a centred-grid
 * kernel at its device, the reference's gp.calculate_gravity_gradient
 * (imported at gempy/API/__init__.py:65, used at test/test_modules/
 * test_geophysics/test_gravity.py:67-80): the closed-form prism attraction
 * (Nagy 1966; Plouff 1976), z up (mass below gives tz < 0), G = 6.674e-3
 * (lengths in m, densities in g/cm^3, tz in mGal).  ``centres``, ``lower``
 * and ``upper`` are n_voxels x 3: voxel centres relative to the device and
 * the half-widths below and above them per axis. */
gk_status gk_gravity_tz(int64_t n_voxels, const double* centres,
                        const double* lower, const double* upper, double* tz,
                        gk_stream stream);
/* Solutions.gravity: gravity[d] = sum_v densities[ids[d n_voxels + v] - 1]
 * tz[v] for every device d (ids are lithology ids 1..n_units of the
 * segmented kernel points, device-major; ids outside that range add 0),
 * reduced in a fixed order.  ``densities`` has n_units entries (device). */
gk_status gk_gravity(int64_t n_devices, int64_t n_voxels, const int32_t* ids,
                     int32_t n_units, const double* densities, const double* tz,
                     double* gravity, gk_stream stream);

/* ---------------- batched realisations (many compute_model calls) ------- */

/* One realisation of a batch: a single-series model, its 3-D regular grid
 * and its segmentation.  Offsets locate its rows in the batch's concatenated
 * device arrays; ref/rest indices are local to the realisation. */
typedef struct gk_batch_item {
    int32_t n_ori, n_sp, n_iface, uni_degree, kernel, n_surf;
    double range, c_o, i_res, gi_res;
    int64_t ori_offset;   /* first orientation in the batch arrays          */
    int64_t sp_offset;    /* first surface point                            */
    int64_t iface_offset; /* first interface row of ref_index / rest_index  */
    int32_t points_per_surface[GK_MAX_SURFACES];
    int32_t dims[3];
    int32_t reserved;
    double origin[3], spacing[3];
    double slope;
    double unit_values[GK_MAX_SURFACES + 1];
} gk_batch_item;

typedef struct gk_batch {
    int32_t n_items;
    int32_t reserved;
    const gk_batch_item* items;                     /* HOST array            */
    const double* dip_positions;                    /* device, n x 3          */
    const double* dip_gradients;
    const double* nugget_grad;
    const double* sp_coords;
    const double* nugget_sp;
    const int32_t* ref_index;
    const int32_t* rest_index;
} gk_batch;

/* Workspace of a batch (all realisations' matrices, Krylov vectors and
 * records) and the total number of grid points (output length). */
size_t gk_batch_workspace_bytes(const gk_batch* batch);
int64_t gk_batch_points(const gk_batch* batch);

/* Lays the batch out in ``work`` (descriptors, work lists, largest-first
 * solve order).  Synchronous; call once per batch, outside stream capture. */
gk_status gk_batch_plan(const gk_batch* batch, void* work, size_t work_bytes,
                        gk_stream stream);

/* Builds, solves (FP32 LU without pivoting preconditioning FP64 FGMRES, one
 * CTA per realisation, tolerance ``tol`` on ||b - K x||_2 / ||b||_2),
 * evaluates every realisation's grid in float-float and segments it, with
 * four persistent launches and no host synchronisation, so the sequence can
 * be captured in a CUDA graph and replayed on new inputs of the same layout.
 * Outputs are concatenated in item order; ``infos`` has one entry per item
 * (may be NULL).  Cubic kernel only. */
gk_status gk_batch_run(const gk_batch* batch, void* work, size_t work_bytes,
                       double tol, int32_t max_iter, double* field,
                       double* values, int32_t* ids, gk_info* infos,
                       gk_stream stream);

/* Copies one realisation's weights (N) and isovalues (stack order) out of the
 * workspace into device buffers (either may be NULL). */
gk_status gk_batch_results(const gk_batch* batch, const void* work,
                           size_t work_bytes, int32_t item, double* weights,
                           double* isovalues, gk_stream stream);

/* ---------------- tile-shape autotuning -------------------------------- */

/* Kernel families whose tile shape (grid points per thread, bytes per
 * shared-memory record stage) is chosen at run time.  The table is process
 * state on the host; gempy_gb300/autotune.py times every variant on the GPU
 * and persists the fastest per GPU model.  Defaults: variant 0. */
typedef enum gk_tunable {
    GK_TUNE_EVAL_FF = 0,     /* gk_eval, GK_FF                  */
    GK_TUNE_EVAL_F32 = 1,    /* gk_eval, GK_F32 without gradient */
    GK_TUNE_BATCH_EVAL = 2,  /* gk_batch_run evaluation          */
    GK_TUNE_EVAL_FF_LIST = 3, /* gk_eval, GK_FF on point lists (octree levels, custom points) */
    GK_TUNE_COUNT = 4
} gk_tunable;

int32_t gk_tune_variants(void);
gk_status gk_tune_describe(int32_t variant, int32_t* points_per_thread,
                           int32_t* stage_kb);
gk_status gk_tune_set(int32_t tunable, int32_t variant);
int32_t gk_tune_get(int32_t tunable);

/* ---------------- learned preconditioner selection --------------------- */

/* The network that picks the two-level preconditioner of gk_solve_twolevel
 * (landmark count r, block size bs, landmark policy) for a system from its
 * geometry.  No reference counterpart: the reference solves every system
 * with the dense FP64 direct solve (``kernel_solver: 1``), which stays the
 * fallback and the judge of every learned-path solution.
 *
 * A 3-layer perceptron in_dim -> 256 -> 256 -> out_dim with ReLU between
 * layers, BF16 weights and FP32 accumulation.  ``params`` holds the weights
 * as BF16 bit patterns: per layer a row-major n_out x (n_in + 1) matrix whose
 * last column is the bias, layers in order (gk_mlp_param_count values). */
#define GK_MLP_HIDDEN 256
#define GK_MLP_MAX_IN 64
#define GK_MLP_MAX_OUT 16
#define GK_MLP_MAX_BATCH (1 << 22)
#define GK_SYSTEM_FEATURES 16

typedef struct gk_mlp {
    int32_t in_dim;          /* 1 .. GK_MLP_MAX_IN   */
    int32_t out_dim;         /* 1 .. GK_MLP_MAX_OUT  */
    const uint16_t* params;  /* device, BF16 bits    */
} gk_mlp;

typedef struct gk_adam {
    float lr, beta1, beta2, eps, weight_decay;
} gk_adam;

/* Number of parameters (-1 for bad dimensions). */
int64_t gk_mlp_param_count(int32_t in_dim, int32_t out_dim);
/* Workspace of gk_mlp_fwd / gk_mlp_bwd for ``batch`` samples (0 if invalid). */
size_t gk_mlp_workspace_bytes(int32_t in_dim, int32_t out_dim, int64_t batch);
/* y (batch x out_dim, FP32) = net(x) for x (batch x in_dim, FP32, row-major).
 * Saves the hidden activations in ``work`` for gk_mlp_bwd. */
gk_status gk_mlp_fwd(const gk_mlp* net, int64_t batch, const float* x,
                     float* y, void* work, size_t work_bytes,
                     gk_stream stream);
/* grad (gk_mlp_param_count FP32, overwritten, parameter layout) = the
 * gradient of sum(dy * y) with respect to the parameters, for the x and the
 * activations of the preceding gk_mlp_fwd on the same ``work``.  The sample
 * sum runs in fixed chunks added in a fixed order: bitwise reproducible. */
gk_status gk_mlp_bwd(const gk_mlp* net, int64_t batch, const float* x,
                     const float* dy, float* grad, void* work,
                     size_t work_bytes, gk_stream stream);
/* Inference pass of the same network on the tensor cores (tcgen05.mma,
 * BF16 x BF16 -> FP32 in tensor memory, 128 samples per CTA): y = net(x) with
 * the activations between layers rounded to BF16.  ``err`` (device, may be
 * NULL) receives GK_ERR_TIMEOUT if an MMA completion wait gives up. */
gk_status gk_mlp_fwd_tc(const gk_mlp* net, int64_t batch, const float* x,
                        float* y, int32_t* err, gk_stream stream);
/* Weighted mean-squared error loss = sum_i w_i |y_i - t_i|^2 / sum_i w_i
 * (w may be NULL: all ones) into loss[0], and its gradient dy (may be NULL). */
gk_status gk_mlp_mse(int64_t batch, int32_t out_dim, const float* y,
                     const float* target, const float* weight, float* dy,
                     float* loss, gk_stream stream);
/* One AdamW step (bias-corrected moments; decoupled weight decay) on the
 * FP32 master parameters, then params = master rounded to BF16 (nearest
 * even).  ``step`` counts from 1. */
gk_status gk_mlp_adam(int64_t n, float* master, uint16_t* params,
                      const float* grad, float* m, float* v,
                      const gk_adam* hp, int32_t step, gk_stream stream);
/* Geometry descriptor of a system: GK_SYSTEM_FEATURES floats (device) --
 * sizes, position extents and spread relative to the range, orientation
 * alignment, nugget levels, drift degree, point spacing, surface count. */
gk_status gk_system_features(const gk_system* s, float* features,
                             gk_stream stream);

/* ---------------- failure-path testing ---------------------------------- */

/* Iteration cap of the kernels' spin waits, for tests of the failure paths
 * (no reference counterpart: the reference has no device code).  The capped
 * waits are the inter-CTA ones -- the grid barrier of the cooperative LU
 * panel, the block flags of the triangular solves -- and each first wait on a
 * bulk copy of the evaluation kernels (single-system and batched).  A wait
 * that reaches its cap records GK_ERR_TIMEOUT in the call's gk_info (for
 * gk_batch_run, in the realisation's) and its kernel returns early; a CTA
 * that gave up first waits, with the default cap, for its copies still in
 * flight.  ``spins`` 0 makes every capped wait give up before its first poll;
 * a negative value restores the defaults (2e7 polls inter-CTA, 4e6 per copy).
 * The network's tensor-core pass keeps its own fixed cap.  Applies to the
 * current device; call it while no kernel of this library is running. */
gk_status gk_set_wait_limit(int64_t spins);

/* Library version string (HOST). */
const char* gk_version(void);

/* Number of kernels this library has launched in the process (telemetry). */
uint64_t gk_launch_count(void);

#ifdef __cplusplus
}
#endif

#endif /* GEMPY_GB300_H */
