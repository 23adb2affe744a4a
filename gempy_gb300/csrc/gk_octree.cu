// Octree refinement: voxel corners, marking and ordered compaction of the
// children of marked voxels.  Replaces the engine's octree step over the
// reference's octree grid (gempy/core/data/grid.py:128-151,
// grid_modules/regular_grid.py:36-43).  A voxel is refined when its 8 corners
// differ in any id set -- the lithology ids, then each fault series' block
// ids; children are listed 8 per refined voxel (x slowest, z fastest) in
// parent order, which matches the point order of the reference's approved
// anticline and fault-model scalar fields
// (test/test_model_types/test_example_models_I.py:19-23, 41-68).
//
// The engine's second refinement test, by an error statistic
// (``octree_error_threshold``; "marked by stats" in
// docs/developers_notes/dev_log/log_2024-06.md:26-39), is restated as: per
// series, the error of trilinear interpolation at the voxel centre,
// |Z(centre) - mean of the 8 corners|, in units of the corners' standard
// deviation; a voxel is marked when that error exceeds the level's mean error
// by ``error_threshold`` standard deviations of the level's errors (and
// kErrorFloor, below which it is the rounding of a field linear over the
// voxel).  With it the combination model's approved last level
// (test_example_models_I.py:71-88) is reproduced.
#include <cstring>

#include "gk_common.cuh"

namespace gk {

__device__ __forceinline__ void corner_sign(int c, double& sx, double& sy, double& sz) {
    sx = (c & 4) ? 1.0 : -1.0;
    sy = (c & 2) ? 1.0 : -1.0;
    sz = (c & 1) ? 1.0 : -1.0;
}

__global__ void corners_kernel(int64_t n, const double* __restrict__ c, double hx, double hy, double hz,
                               double* __restrict__ out) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 8 * n) return;
    int64_t v = i >> 3;
    int k = (int)(i & 7);
    double sx, sy, sz;
    corner_sign(k, sx, sy, sz);
    out[3 * i] = c[3 * v] + sx * hx;
    out[3 * i + 1] = c[3 * v + 1] + sy * hy;
    out[3 * i + 2] = c[3 * v + 2] + sz * hz;
}

constexpr int kScanBlock = 256;
constexpr int kMaxIdSets = 1 + GK_MAX_SURFACES;

constexpr double kErrorFloor = 1e-6;
constexpr int kStatThreads = 1024;

// The id arrays a voxel's refinement looks at: set s holds the 8 corner ids
// of voxel v at p[s][8 v .. 8 v + 7].  With n_err > 0, voxel v is also marked
// when err[s n_vox + v] > thr[s] for some series s < n_err.
struct IdSets {
    const int32_t* p[kMaxIdSets];
    int n;
    int n_err;
    int64_t n_vox;
    const double* err;
    const double* thr;
};

// voxel v is marked when its 8 corners differ in any id set, or when its
// interpolation error is an outlier in any series
__device__ __forceinline__ int voxel_marked(const IdSets& ids, int64_t v) {
    int m = 0;
    for (int s = 0; s < ids.n && !m; ++s) {
        const int32_t* c = ids.p[s] + 8 * v;
        const int32_t a = c[0];
        for (int k = 1; k < 8; ++k) m |= (c[k] != a);
    }
    for (int s = 0; s < ids.n_err && !m; ++s) m = ids.err[s * ids.n_vox + v] > ids.thr[s];
    return m;
}

// err[s n + v] = |Z_s(centre v) - mean_k Z_s(corner k of v)| / std_k Z_s(corner
// k of v), 0 where the 8 corners are equal.  fields: n_series x np, the
// centres' values first, then 8 corners per centre.
__global__ void interp_error_kernel(int64_t n, int64_t np, int n_series, const double* __restrict__ fields,
                                    double* __restrict__ err) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n * n_series) return;
    const int s = (int)(i / n);
    const int64_t v = i - (int64_t)s * n;
    const double* f = fields + (int64_t)s * np;
    const double* c = f + n + 8 * v;
    double z[8], mean = 0.0;
    for (int k = 0; k < 8; ++k) {
        z[k] = c[k];
        mean += z[k];
    }
    mean *= 0.125;
    double var = 0.0;
    for (int k = 0; k < 8; ++k) var += (z[k] - mean) * (z[k] - mean);
    const double sd = sqrt(var * 0.125);
    err[i] = sd > 0.0 ? fabs(f[v] - mean) / sd : 0.0;
}

// fixed-order sum over the CTA (kStatThreads threads)
__device__ double cta_sum(double x, double* red) {
    red[threadIdx.x] = x;
    __syncthreads();
    for (int off = kStatThreads / 2; off > 0; off >>= 1) {
        if ((int)threadIdx.x < off) red[threadIdx.x] += red[threadIdx.x + off];
        __syncthreads();
    }
    const double r = red[0];
    __syncthreads();
    return r;
}

// One CTA per series: thr[s] = max(mean + t std, kErrorFloor) of err[s n ..
// s n + n - 1] (two passes, population std; the order of the sums is fixed,
// so the threshold is the same on every run).
__global__ void error_threshold_kernel(int64_t n, const double* __restrict__ err, double t,
                                       double* __restrict__ thr) {
    __shared__ double red[kStatThreads];
    const double* e = err + (int64_t)blockIdx.x * n;
    double a = 0.0;
    for (int64_t v = threadIdx.x; v < n; v += kStatThreads) a += e[v];
    const double mean = cta_sum(a, red) / (double)n;
    a = 0.0;
    for (int64_t v = threadIdx.x; v < n; v += kStatThreads) a += (e[v] - mean) * (e[v] - mean);
    const double sd = sqrt(cta_sum(a, red) / (double)n);
    if (threadIdx.x == 0) thr[blockIdx.x] = fmax(mean + t * sd, kErrorFloor);
}

// per-block count of marked voxels
__global__ void mark_count_kernel(int64_t n, const IdSets ids, int refine_all, int64_t* __restrict__ block_counts) {
    int64_t v = (int64_t)blockIdx.x * kScanBlock + threadIdx.x;
    int m = 0;
    if (v < n) m = refine_all ? 1 : voxel_marked(ids, v);
    int w = __syncthreads_count(m);
    if (threadIdx.x == 0) block_counts[blockIdx.x] = w;
}

// exclusive scan of block counts in one CTA (sequential over chunks of 1024)
__global__ void scan_blocks_kernel(int64_t nb, int64_t* __restrict__ counts, int64_t* __restrict__ total) {
    __shared__ int64_t buf[1024];
    __shared__ int64_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int64_t base = 0; base < nb; base += 1024) {
        int64_t i = base + threadIdx.x;
        int64_t v = i < nb ? counts[i] : 0;
        buf[threadIdx.x] = v;
        __syncthreads();
        for (int off = 1; off < 1024; off <<= 1) {
            int64_t t = threadIdx.x >= off ? buf[threadIdx.x - off] : 0;
            __syncthreads();
            buf[threadIdx.x] += t;
            __syncthreads();
        }
        if (i < nb) counts[i] = carry + buf[threadIdx.x] - v;  // exclusive
        __syncthreads();
        if (threadIdx.x == 1023) carry += buf[1023];
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry * 8;
}

__global__ void scatter_children_kernel(int64_t n, const double* __restrict__ c, const IdSets ids, int refine_all,
                                        const int64_t* __restrict__ block_off, double qx, double qy, double qz,
                                        double* __restrict__ out) {
    __shared__ int pref[kScanBlock];
    int64_t v = (int64_t)blockIdx.x * kScanBlock + threadIdx.x;
    int m = 0;
    if (v < n) m = refine_all ? 1 : voxel_marked(ids, v);
    pref[threadIdx.x] = m;
    __syncthreads();
    for (int off = 1; off < kScanBlock; off <<= 1) {
        int t = threadIdx.x >= off ? pref[threadIdx.x - off] : 0;
        __syncthreads();
        pref[threadIdx.x] += t;
        __syncthreads();
    }
    if (!m) return;
    int64_t slot = block_off[blockIdx.x] + pref[threadIdx.x] - 1;
    for (int k = 0; k < 8; ++k) {
        double sx, sy, sz;
        corner_sign(k, sx, sy, sz);
        int64_t o = 8 * slot + k;
        out[3 * o] = c[3 * v] + sx * qx;
        out[3 * o + 1] = c[3 * v + 1] + sy * qy;
        out[3 * o + 2] = c[3 * v + 2] + sz * qz;
    }
}

// Marks, counts and scatters the children of the n voxels at `centres`
// (spacing h): children into `children` (8 per marked voxel), 8 x the marked
// count into *count.
static gk_status refine_voxels(int64_t n, const double* centres, const IdSets& ids, int refine_all, const double* h,
                               double* children, int64_t* count, void* work, cudaStream_t st) {
    const int64_t nb = (n + kScanBlock - 1) / kScanBlock;
    if (nb > 0x7fffffff) return GK_ERR_SIZE;
    int64_t* bc = (int64_t*)work;
    mark_count_kernel<<<(unsigned)nb, kScanBlock, 0, st>>>(n, ids, refine_all, bc);
    GK_LAUNCH_CHECK();
    scan_blocks_kernel<<<1, 1024, 0, st>>>(nb, bc, count);
    GK_LAUNCH_CHECK();
    scatter_children_kernel<<<(unsigned)nb, kScanBlock, 0, st>>>(n, centres, ids, refine_all, bc, h[0] / 4,
                                                                   h[1] / 4, h[2] / 4, children);
    GK_LAUNCH_CHECK();
    return GK_OK;
}

}  // namespace gk

using namespace gk;

extern "C" gk_status gk_octree_corners(int64_t n, const double* centres, const double spacing[3], double* corners,
                                       gk_stream stream) {
    if (n < 0 || spacing == nullptr) return GK_ERR_ARG;
    if (n == 0) return GK_OK;
    if (centres == nullptr || corners == nullptr) return GK_ERR_ARG;
    corners_kernel<<<(unsigned)((8 * n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
        n, centres, spacing[0] / 2, spacing[1] / 2, spacing[2] / 2, corners);
    GK_LAUNCH_CHECK();
    return GK_OK;
}

extern "C" size_t gk_octree_workspace_bytes(int64_t n) {
    int64_t nb = (n + kScanBlock - 1) / kScanBlock;
    return (size_t)(nb + 1) * sizeof(int64_t);
}

extern "C" gk_status gk_octree_refine(int64_t n, const double* centres, const int32_t* corner_ids,
                                      int32_t n_id_sets, int32_t refine_all, const double spacing[3],
                                      double* children, int64_t* count, void* work, size_t work_bytes,
                                      gk_stream stream) {
    if (n < 0 || spacing == nullptr || count == nullptr) return GK_ERR_ARG;
    if (!refine_all && (n_id_sets < 1 || n_id_sets > 1 + GK_MAX_SURFACES)) return GK_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    if (n == 0) {
        GK_CUDA_TRY(cudaMemsetAsync(count, 0, sizeof(int64_t), st));
        return GK_OK;
    }
    if (centres == nullptr || children == nullptr || (corner_ids == nullptr && !refine_all)) return GK_ERR_ARG;
    if (work == nullptr || work_bytes < gk_octree_workspace_bytes(n)) return GK_ERR_SIZE;
    IdSets ids;
    memset(&ids, 0, sizeof(ids));
    ids.n = refine_all ? 0 : n_id_sets;
    for (int s = 0; s < ids.n; ++s) ids.p[s] = corner_ids + (int64_t)s * 8 * n;
    return refine_voxels(n, centres, ids, refine_all, spacing, children, count, work, st);
}

static size_t al256(size_t x) { return (x + 255) & ~(size_t)255; }

extern "C" gk_status gk_octree_level_plan(int32_t n_series, int64_t n, int32_t corners, int32_t refine,
                                            gk_octree_level_layout* L) {
    if (L == nullptr || n_series < 1 || n_series > GK_MAX_SURFACES || n < 0) return GK_ERR_ARG;
    if (refine < 0 || refine > 3 || ((refine == 1 || refine == 3) && !corners)) return GK_ERR_ARG;
    memset(L, 0, sizeof(*L));
    const int64_t np = corners ? 9 * n : n;
    L->n = n;
    L->n_points = np;
    L->n_series = n_series;
    L->corners = corners ? 1 : 0;
    L->refine = refine;
    size_t o = 0;
    L->points = o;   o += al256((size_t)np * 3 * sizeof(double));
    L->fields = o;   o += al256((size_t)n_series * np * sizeof(double));
    L->values = o;   o += al256((size_t)n_series * np * sizeof(double));
    L->ids = o;      o += al256((size_t)n_series * np * sizeof(int32_t));
    L->block = o;    o += al256((size_t)np * sizeof(double));
    L->lith_ids = o; o += al256((size_t)np * sizeof(int32_t));
    L->masks = o;    o += al256((size_t)n_series * np);
    L->children = o;
    if (refine) {
        o += al256((size_t)8 * n * 3 * sizeof(double));
        L->count = o;  o += 256;
        L->work = o;   o += al256(gk_octree_workspace_bytes(n));
        if (refine == 3) o += al256((size_t)n_series * n * sizeof(double)) + al256((size_t)n_series * sizeof(double));
    } else {
        L->count = L->work = o;
    }
    L->total = o;
    return GK_OK;
}

extern "C" gk_status gk_octree_level(int32_t n_series, const gk_series_eval* series, const double* centres,
                                     const double spacing[3], gk_prec prec, int32_t n_fault_sets,
                                     const int32_t* fault_series, double error_threshold,
                                     const gk_octree_level_layout* L, void* buf, size_t buf_bytes, gk_info* info,
                                     gk_stream stream) {
    if (L == nullptr || series == nullptr || spacing == nullptr || n_series != L->n_series) return GK_ERR_ARG;
    if (L->refine == 3 && !(error_threshold > 0.0 && error_threshold < 1e300)) return GK_ERR_ARG;
    if (n_fault_sets < 0 || n_fault_sets > GK_MAX_SURFACES || (n_fault_sets > 0 && fault_series == nullptr))
        return GK_ERR_ARG;
    gk_octree_level_layout chk;
    gk_status st = gk_octree_level_plan(n_series, L->n, L->corners, L->refine, &chk);
    if (st != GK_OK) return st;
    if (memcmp(&chk, L, sizeof(chk)) != 0) return GK_ERR_ARG;
    if (buf == nullptr || buf_bytes < L->total) return GK_ERR_SIZE;
    const int64_t n = L->n, np = L->n_points;
    cudaStream_t cs = (cudaStream_t)stream;
    char* b = (char*)buf;
    if (n == 0) {
        if (L->refine) GK_CUDA_TRY(cudaMemsetAsync(b + L->count, 0, sizeof(int64_t), cs));
        return GK_OK;
    }
    if (centres == nullptr) return GK_ERR_ARG;
    double* pts = (double*)(b + L->points);
    GK_CUDA_TRY(cudaMemcpyAsync(pts, centres, (size_t)n * 3 * sizeof(double), cudaMemcpyDeviceToDevice, cs));
    if (L->corners) {
        st = gk_octree_corners(n, centres, spacing, pts + 3 * n, stream);
        if (st != GK_OK) return st;
    }
    gk_points gp;
    memset(&gp, 0, sizeof(gp));
    gp.kind = 1;
    gp.n = np;
    gp.xyz = pts;
    double* fields = (double*)(b + L->fields);
    int32_t* ids = (int32_t*)(b + L->ids);
    int32_t* lith = (int32_t*)(b + L->lith_ids);
    st = gk_eval_series_set(n_series, series, &gp, prec, fields, (double*)(b + L->values), ids,
                            (double*)(b + L->block), lith, (uint8_t*)(b + L->masks), info, stream);
    if (st != GK_OK) return st;
    if (!L->refine) return GK_OK;
    IdSets sets;
    memset(&sets, 0, sizeof(sets));
    if (L->refine == 1 || L->refine == 3) {
        sets.p[sets.n++] = lith + n;   // the corners' lithology, then each fault series' block ids
        for (int f = 0; f < n_fault_sets; ++f) {
            const int s = fault_series[f];
            if (s < 0 || s >= n_series) return GK_ERR_ARG;
            sets.p[sets.n++] = ids + (int64_t)s * np + n;
        }
    }
    if (L->refine == 3) {
        double* err = (double*)(b + L->work + al256(gk_octree_workspace_bytes(n)));
        double* thr = (double*)((char*)err + al256((size_t)n_series * n * sizeof(double)));
        const int64_t ne = n * n_series;
        interp_error_kernel<<<(unsigned)((ne + 255) / 256), 256, 0, cs>>>(n, np, n_series, fields, err);
        GK_LAUNCH_CHECK();
        error_threshold_kernel<<<n_series, kStatThreads, 0, cs>>>(n, err, error_threshold, thr);
        GK_LAUNCH_CHECK();
        sets.n_err = n_series;
        sets.n_vox = n;
        sets.err = err;
        sets.thr = thr;
    }
    return refine_voxels(n, pts, sets, L->refine == 2, spacing, (double*)(b + L->children), (int64_t*)(b + L->count),
                         b + L->work, cs);
}

extern "C" const char* gk_version(void) { return "gempy_gb300 0.1.0 (sm_103a)"; }

extern "C" uint64_t gk_launch_count(void) { return gk_launch_counter().load(std::memory_order_relaxed); }
