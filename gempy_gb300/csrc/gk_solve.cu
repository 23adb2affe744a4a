// Mixed-precision solve of the FP64 kriging system.
//
//   1. equilibrate: D = diag(1/sqrt(max_j |K_ij|)), K32 = fp32(D K D);
//   2. FP32 blocked LU of K32 (gk_lu.cu);
//   3. FGMRES in FP64 (restart m, right preconditioner M^-1 = D LU32^-1 D,
//      classical Gram-Schmidt applied twice) on the FP64 K held in HBM.
// FP64 is used only for the residual/Krylov vectors, the products with the
// FP64 K and the solution update; the O(N^3) factorization runs in FP32.
// Plain iterative refinement (x += M^-1 (b - K x)) diverges on kriging systems
// with kappa(K) eps32 > 1, which the FP64-GMRES outer iteration tolerates
// (it converges while kappa eps32 eps64-scale products stay small).
// Convergence is tested on the host between Arnoldi steps (one small
// device-to-host copy per step).
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "gk_common.cuh"

gk_status gk_internal_lu_factor_f32(int64_t n, float* A, int64_t lda, int32_t* ipiv, void* work, size_t wb,
                                    gk_info* info, cudaStream_t st);
gk_status gk_internal_lu_solve_f32(int64_t n, const float* LU, int64_t lda, const int32_t* ipiv, float* b, void* work,
                                   size_t wb, gk_info* info, cudaStream_t st);
size_t gk_internal_lu_ws_f32(int64_t n);
size_t gk_internal_lu_ws_f64(int64_t n);
gk_status gk_internal_twolevel_setup_f64(int64_t n, const double* K, int64_t ldk, const int32_t* perm,
                                         const double* d, int64_t r, int bs, double* A, int64_t lda, int32_t* ipiv,
                                         void* work, size_t wbytes, gk_info* info, cudaStream_t st,
                                         float* ffpanel);
size_t gk_internal_ff_panel_floats(int64_t n);
gk_status gk_internal_twolevel_apply_f64(int64_t n, const double* A, int64_t lda, const int32_t* perm,
                                         const double* d, int64_t r, int bs, const double* v, double* z, double* t,
                                         void* work, size_t wbytes, gk_info* info, cudaStream_t st);
gk_status gk_internal_lu_factor_nopiv_f32(int64_t n, float* A, int64_t lda, int32_t* ipiv, void* work, size_t wb,
                                          gk_info* info, cudaStream_t st);
gk_status gk_internal_twolevel_setup(int64_t n, const double* K, int64_t ldk, const int32_t* perm, const double* d,
                                     int64_t r, int bs, float* A, int64_t lda, int32_t* ipiv, void* work,
                                     size_t wbytes, gk_info* info, cudaStream_t st);
gk_status gk_internal_twolevel_apply(int64_t n, const float* A, int64_t lda, const int32_t* perm, const double* d,
                                     int64_t r, int bs, const double* v, double* z, float* t, void* work,
                                     size_t wbytes, gk_info* info, cudaStream_t st);

namespace gk {

static size_t al(size_t x) { return (x + 255) & ~(size_t)255; }
static int64_t ld32_of(int64_t n) { return (n + 63) / 64 * 64; }

constexpr int kRestart = 50;           // LU-preconditioned FGMRES
constexpr int kRestartTwoLevel = 200;  // two-level: many more outlying eigenvalues to resolve
constexpr int kDotBlocks = 128;

struct MixedWork {
    float* K32;     // preconditioner matrix (FP32 layout) ...
    double* K64;    // ... or the same region as FP64 (two-level, FP64 storage)
    int32_t* ipiv;
    void* luw;
    size_t luw_bytes;
    double* d;      // equilibration
    double* r;      // residual / work vector
    float* t32;     // preconditioner vector (FP32) ...
    double* t64;    // ... or FP64, same region
    double* V;      // (m+1) x n Krylov basis (vector-major)
    double* Z;      // m x n preconditioned directions
    double* w;      // n
    double* part;   // kDotBlocks x (m+1) partial dots
    double* h;      // m+1 reduced dots
    double* y;      // m coefficients
    gk_info* iinfo; // status word used when the caller passes none
};

// es: bytes per element of the preconditioner's matrix and vector (4 or 8);
// m: restart length (Krylov basis size).
static size_t mixed_bytes(int64_t n, int es = 4, int m = kRestart) {
    int64_t ld = ld32_of(n);
    const size_t luws = es == 8 ? gk_internal_lu_ws_f64(n) : gk_internal_lu_ws_f32(n);
    return al((size_t)n * ld * es) + al(n * sizeof(int32_t)) + al(luws) + 2 * al(n * sizeof(double)) +
           al((size_t)n * es) + al((size_t)(m + 1) * n * sizeof(double)) + al((size_t)m * n * sizeof(double)) +
           al(n * sizeof(double)) + al((size_t)kDotBlocks * (m + 1) * sizeof(double)) +
           2 * al((m + 1) * sizeof(double)) + al(sizeof(gk_info));
}

static MixedWork carve(void* base, int64_t n, int es = 4, int m = kRestart) {
    MixedWork w;
    char* p = (char*)base;
    int64_t ld = ld32_of(n);
    w.K32 = (float*)p; w.K64 = (double*)p; p += al((size_t)n * ld * es);
    w.ipiv = (int32_t*)p; p += al(n * sizeof(int32_t));
    w.luw = p; w.luw_bytes = al(es == 8 ? gk_internal_lu_ws_f64(n) : gk_internal_lu_ws_f32(n)); p += w.luw_bytes;
    w.d = (double*)p; p += al(n * sizeof(double));
    w.r = (double*)p; p += al(n * sizeof(double));
    w.t32 = (float*)p; w.t64 = (double*)p; p += al((size_t)n * es);
    w.V = (double*)p; p += al((size_t)(m + 1) * n * sizeof(double));
    w.Z = (double*)p; p += al((size_t)m * n * sizeof(double));
    w.w = (double*)p; p += al(n * sizeof(double));
    w.part = (double*)p; p += al((size_t)kDotBlocks * (m + 1) * sizeof(double));
    w.h = (double*)p; p += al((m + 1) * sizeof(double));
    w.y = (double*)p; p += al((m + 1) * sizeof(double));
    w.iinfo = (gk_info*)p;
    return w;
}

// d_i = 1 / sqrt(max_j |K_ij|); one warp per row.
__global__ void equil_kernel(const double* __restrict__ K, int64_t ldk, int64_t n, double* __restrict__ d) {
    int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (row >= n) return;
    double m = 0.0;
    const double* k = K + row * ldk;
    for (int64_t j = lane; j < n; j += 32) m = fmax(m, fabs(k[j]));
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
    if (lane == 0) d[row] = m > 0.0 ? 1.0 / sqrt(m) : 1.0;
}

__global__ void convert_kernel(const double* __restrict__ K, int64_t ldk, int64_t n, const double* __restrict__ d,
                               float* __restrict__ K32, int64_t ld32) {
    int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t i = blockIdx.y;
    for (; i < n; i += gridDim.y) {
        if (j < n) K32[i * ld32 + j] = (float)(d[i] * K[i * ldk + j] * d[j]);
    }
}

// y = b - K x (b may be NULL: y = K x).  One warp per kGemvRows consecutive
// rows: each x element is loaded once and used for all of them (every warp
// streams x from L2, so sharing it cuts that traffic by kGemvRows), 16-byte
// loads of K when its rows are 16-byte aligned, one accumulator per row.
constexpr int kGemvRows = 4;
static unsigned gemv_blocks(int64_t n) { return (unsigned)(((n + kGemvRows - 1) / kGemvRows * 32 + 255) / 256); }

__global__ void __launch_bounds__(256) gemv_kernel(const double* __restrict__ K, int64_t ldk, int64_t n,
                                                   const double* __restrict__ b, const double* __restrict__ x,
                                                   double* __restrict__ y) {
    const int64_t r0 = (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * kGemvRows;
    const int lane = threadIdx.x & 31;
    if (r0 >= n) return;
    const int nr = (int)min((int64_t)kGemvRows, n - r0);
    double acc[kGemvRows];
#pragma unroll
    for (int r = 0; r < kGemvRows; ++r) acc[r] = 0.0;
    int64_t j0 = 0;
    if ((ldk & 1) == 0 && ((uintptr_t)K & 15) == 0) {
        const int64_t np = n >> 1;
        for (int64_t p = lane; p < np; p += 32) {
            const double x0 = x[2 * p], x1 = x[2 * p + 1];
#pragma unroll
            for (int r = 0; r < kGemvRows; ++r) {
                if (r < nr) {
                    const double2 kv = reinterpret_cast<const double2*>(K + (r0 + r) * ldk)[p];
                    acc[r] = fma(kv.x, x0, acc[r]);
                    acc[r] = fma(kv.y, x1, acc[r]);
                }
            }
        }
        j0 = np << 1;
    }
    for (int64_t j = j0 + lane; j < n; j += 32) {
        const double xv = x[j];
#pragma unroll
        for (int r = 0; r < kGemvRows; ++r)
            if (r < nr) acc[r] = fma(K[(r0 + r) * ldk + j], xv, acc[r]);
    }
#pragma unroll
    for (int r = 0; r < kGemvRows; ++r)
        for (int o = 16; o > 0; o >>= 1) acc[r] += __shfl_down_sync(0xffffffffu, acc[r], o);
    if (lane == 0) {
#pragma unroll
        for (int r = 0; r < kGemvRows; ++r)
            if (r < nr) y[r0 + r] = b ? b[r0 + r] - acc[r] : acc[r];
    }
}

// partial dots part[blk][c] = sum_{i in blk} V[c][i] * w[i], c < ncol; one
// warp per column, each block over its own contiguous index range.
__global__ void dots_partial_kernel(const double* __restrict__ V, int64_t n, int ncol, const double* __restrict__ w,
                                    double* __restrict__ part) {
    const int64_t per = (n + gridDim.x - 1) / gridDim.x;
    const int64_t i0 = (int64_t)blockIdx.x * per, i1 = min(n, i0 + per);
    const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int c = threadIdx.x >> 5; c < ncol; c += nw) {
        const double* v = V + (int64_t)c * n;
        double s = 0.0;
        for (int64_t i = i0 + lane; i < i1; i += 32) s = fma(v[i], w[i], s);
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (lane == 0) part[(int64_t)blockIdx.x * ncol + c] = s;
    }
}

// h[c] = sum_blk part[blk][c] (fixed order: deterministic); acc: h += result
__global__ void dots_final_kernel(const double* __restrict__ part, int nblk, int ncol, double* __restrict__ h,
                                  int accumulate) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncol) return;
    double t = 0.0;
    for (int b = 0; b < nblk; ++b) t += part[(int64_t)b * ncol + c];
    h[c] = accumulate ? h[c] + t : t;
}

// w -= sum_c V[c] * coef[c]
__global__ void sub_basis_kernel(const double* __restrict__ V, int64_t n, int ncol, const double* __restrict__ coef,
                                 double* __restrict__ w) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double s = w[i];
    for (int c = 0; c < ncol; ++c) s -= V[(int64_t)c * n + i] * coef[c];
    w[i] = s;
}

// x += sum_c Z[c] * y[c]
__global__ void add_basis_kernel(const double* __restrict__ Z, int64_t n, int ncol, const double* __restrict__ y,
                                 double* __restrict__ x) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double s = x[i];
    for (int c = 0; c < ncol; ++c) s += Z[(int64_t)c * n + i] * y[c];
    x[i] = s;
}

__global__ void scale_kernel(const double* __restrict__ src, double a, int64_t n, double* __restrict__ dst) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = a * src[i];
}

__global__ void scale_to_f32_kernel(const double* __restrict__ r, const double* __restrict__ d, int64_t n,
                                    float* __restrict__ t) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) t[i] = (float)(d[i] * r[i]);
}

__global__ void from_f32_kernel(const float* __restrict__ t, const double* __restrict__ d, int64_t n,
                                double* __restrict__ z) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) z[i] = d[i] * (double)t[i];
}

}  // namespace gk

using namespace gk;

extern "C" size_t gk_solve_mixed_workspace_bytes(int64_t n) { return n > 0 ? mixed_bytes(n) : 0; }

namespace {

struct Solver {
    int64_t n;
    const double* K;
    int64_t ldk;
    MixedWork w;
    int64_t ld32;
    gk_info* info;
    cudaStream_t st;
    unsigned vb, rb;
    // preconditioner: 0 = FP32 LU of the equilibrated K, 1 = two-level
    // (FP32 storage), 2 = two-level (FP64 storage)
    int mode = 0;
    const int32_t* perm = nullptr;
    int64_t r = 0;
    int bs = 0;
    int m = kRestart;  // restart length; the workspace holds m + 1 basis vectors

    // dot products h[0..ncol) = V[0..ncol)^T v  (accumulate: h += ...)
    gk_status dots(const double* V, int ncol, const double* v, double* h, int accumulate) {
        dots_partial_kernel<<<kDotBlocks, 256, 0, st>>>(V, n, ncol, v, w.part);
        GK_LAUNCH_CHECK();
        dots_final_kernel<<<(unsigned)((ncol + 63) / 64), 64, 0, st>>>(w.part, kDotBlocks, ncol, h, accumulate);
        GK_LAUNCH_CHECK();
        return GK_OK;
    }
    gk_status norm2(const double* v, double& out) {
        gk_status s = dots(v, 1, v, w.h + m, 0);
        if (s != GK_OK) return s;
        GK_CUDA_TRY(cudaMemcpyAsync(&out, w.h + m, sizeof(double), cudaMemcpyDeviceToHost, st));
        GK_CUDA_TRY(cudaStreamSynchronize(st));
        out = sqrt(out);
        return GK_OK;
    }
    // z = D LU32^-1 D v, or the two-level preconditioner
    gk_status precond(const double* v, double* z) {
        if (mode == 1)
            return gk_internal_twolevel_apply(n, w.K32, ld32, perm, w.d, r, bs, v, z, w.t32, w.luw, w.luw_bytes,
                                              info, st);
        if (mode == 2)
            return gk_internal_twolevel_apply_f64(n, w.K64, ld32, perm, w.d, r, bs, v, z, w.t64, w.luw,
                                                  w.luw_bytes, info, st);
        scale_to_f32_kernel<<<vb, 256, 0, st>>>(v, w.d, n, w.t32);
        GK_LAUNCH_CHECK();
        gk_status s = gk_internal_lu_solve_f32(n, w.K32, ld32, w.ipiv, w.t32, w.luw, w.luw_bytes, info, st);
        if (s != GK_OK) return s;
        from_f32_kernel<<<vb, 256, 0, st>>>(w.t32, w.d, n, z);
        GK_LAUNCH_CHECK();
        return GK_OK;
    }
};

}  // namespace

// Restarted FGMRES(S.m) in FP64 with right preconditioning S.precond;
// convergence tested on the host between Arnoldi steps.
static gk_status fgmres(Solver& S, const double* b, double* x, const double* x0, double tol, int max_iter,
                        int& status, int& its,
                        double& rel) {
    MixedWork& w = S.w;
    const int64_t n = S.n;
    const double* K = S.K;
    const int64_t ldk = S.ldk;
    cudaStream_t st = S.st;
    gk_status s;
    double bnorm = 0.0;
    if ((s = S.norm2(b, bnorm)) != GK_OK) return s;
    if (x0 != nullptr)  // warm start (e.g. the previous weights of the same series)
        GK_CUDA_TRY(cudaMemcpyAsync(x, x0, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
    else
        GK_CUDA_TRY(cudaMemsetAsync(x, 0, n * sizeof(double), st));
    status = GK_ERR_NOT_CONVERGED;
    its = 0;
    rel = 1.0;
    double prev_true = INFINITY;
    if (!(bnorm > 0.0)) {
        status = bnorm == 0.0 ? GK_OK : GK_ERR_NONFINITE;
        rel = 0.0;
    }
    const int m = S.m;
    std::vector<double> H((m + 1) * m), cs(m), sn(m), g(m + 1), hcol(m + 2), y(m);
    while (status == GK_ERR_NOT_CONVERGED && its < max_iter) {
        // true residual r = b - K x
        gemv_kernel<<<gemv_blocks(n), 256, 0, st>>>(K, ldk, n, b, x, w.r);
        GK_LAUNCH_CHECK();
        double beta;
        if ((s = S.norm2(w.r, beta)) != GK_OK) return s;
        rel = beta / bnorm;
        if (!std::isfinite(rel)) { status = GK_ERR_NONFINITE; break; }
        if (rel <= tol) { status = GK_OK; break; }
        // a whole restart cycle gained less than 2%: stagnated (FP64 floor or a weak preconditioner)
        if (rel > 0.98 * prev_true) break;
        prev_true = rel;
        scale_kernel<<<S.vb, 256, 0, st>>>(w.r, 1.0 / beta, n, w.V);
        GK_LAUNCH_CHECK();
        std::fill(g.begin(), g.end(), 0.0);
        g[0] = beta;
        int j = 0;
        for (; j < m && its < max_iter; ++j, ++its) {
            double* vj = w.V + (int64_t)j * n;
            double* zj = w.Z + (int64_t)j * n;
            if ((s = S.precond(vj, zj)) != GK_OK) return s;
            gemv_kernel<<<gemv_blocks(n), 256, 0, st>>>(K, ldk, n, nullptr, zj, w.w);
            GK_LAUNCH_CHECK();
            // CGS2
            for (int pass = 0; pass < 2; ++pass) {
                if ((s = S.dots(w.V, j + 1, w.w, pass == 0 ? w.h : w.y, 0)) != GK_OK) return s;
                sub_basis_kernel<<<S.vb, 256, 0, st>>>(w.V, n, j + 1, pass == 0 ? w.h : w.y, w.w);
                GK_LAUNCH_CHECK();
            }
            double hn;
            if ((s = S.norm2(w.w, hn)) != GK_OK) return s;
            GK_CUDA_TRY(cudaMemcpyAsync(hcol.data(), w.h, (j + 1) * sizeof(double), cudaMemcpyDeviceToHost, st));
            GK_CUDA_TRY(cudaMemcpyAsync(y.data(), w.y, (j + 1) * sizeof(double), cudaMemcpyDeviceToHost, st));
            GK_CUDA_TRY(cudaStreamSynchronize(st));
            for (int i = 0; i <= j; ++i) hcol[i] += y[i];
            hcol[j + 1] = hn;
            if (hn > 0.0) {
                scale_kernel<<<S.vb, 256, 0, st>>>(w.w, 1.0 / hn, n, w.V + (int64_t)(j + 1) * n);
                GK_LAUNCH_CHECK();
            }
            // Givens rotations
            for (int i = 0; i < j; ++i) {
                double t = cs[i] * hcol[i] + sn[i] * hcol[i + 1];
                hcol[i + 1] = -sn[i] * hcol[i] + cs[i] * hcol[i + 1];
                hcol[i] = t;
            }
            double den = std::hypot(hcol[j], hcol[j + 1]);
            cs[j] = den > 0 ? hcol[j] / den : 1.0;
            sn[j] = den > 0 ? hcol[j + 1] / den : 0.0;
            hcol[j] = den;
            hcol[j + 1] = 0.0;
            g[j + 1] = -sn[j] * g[j];
            g[j] = cs[j] * g[j];
            for (int i = 0; i <= j; ++i) H[i * m + j] = hcol[i];
            if (std::fabs(g[j + 1]) <= tol * bnorm || hn == 0.0) { ++j; ++its; break; }
        }
        // y = H^-1 g (upper triangular j x j), x += Z y
        for (int i = j - 1; i >= 0; --i) {
            double t = g[i];
            for (int k = i + 1; k < j; ++k) t -= H[i * m + k] * y[k];
            y[i] = H[i * m + i] != 0.0 ? t / H[i * m + i] : 0.0;
        }
        if (j > 0) {
            GK_CUDA_TRY(cudaMemcpyAsync(w.y, y.data(), j * sizeof(double), cudaMemcpyHostToDevice, st));
            add_basis_kernel<<<S.vb, 256, 0, st>>>(w.Z, n, j, w.y, x);
            GK_LAUNCH_CHECK();
        }
    }
    if (status == GK_ERR_NOT_CONVERGED) {
        // final true residual
        gemv_kernel<<<gemv_blocks(n), 256, 0, st>>>(K, ldk, n, b, x, w.r);
        GK_LAUNCH_CHECK();
        double beta;
        if ((s = S.norm2(w.r, beta)) != GK_OK) return s;
        rel = beta / bnorm;
        if (rel <= tol) status = GK_OK;
    }
    return GK_OK;
}

extern "C" gk_status gk_gemv(int64_t n, const double* K, int64_t ldk, const double* x, double* y,
                             gk_stream stream) {
    if (n <= 0 || K == nullptr || x == nullptr || y == nullptr || ldk < n || x == y) return GK_ERR_ARG;
    gemv_kernel<<<gemv_blocks(n), 256, 0, (cudaStream_t)stream>>>(K, ldk, n, nullptr, x, y);
    GK_LAUNCH_CHECK();
    return GK_OK;
}

extern "C" gk_status gk_solve_mixed(int64_t n, const double* K, int64_t ldk, const double* b, double* x, double tol,
                                    int32_t max_iter, void* work, size_t work_bytes, gk_info* info,
                                    gk_stream stream) {
    cudaStream_t st = (cudaStream_t)stream;
    if (n <= 0 || K == nullptr || b == nullptr || x == nullptr || ldk < n || max_iter < 1) return GK_ERR_ARG;
    if (work == nullptr || work_bytes < mixed_bytes(n)) return GK_ERR_SIZE;
    Solver S;
    S.n = n; S.K = K; S.ldk = ldk; S.w = carve(work, n); S.ld32 = ld32_of(n); S.st = st;
    if (info == nullptr) info = S.w.iinfo;
    S.info = info;
    S.vb = (unsigned)((n + 255) / 256);
    S.rb = (unsigned)((n * 32 + 255) / 256);
    MixedWork& w = S.w;
    GK_CUDA_TRY(cudaMemsetAsync(info, 0, sizeof(gk_info), st));
    equil_kernel<<<S.rb, 256, 0, st>>>(K, ldk, n, w.d);
    GK_LAUNCH_CHECK();
    dim3 cg((unsigned)((n + 255) / 256), (unsigned)(n < 4096 ? n : 4096));
    convert_kernel<<<cg, 256, 0, st>>>(K, ldk, n, w.d, w.K32, S.ld32);
    GK_LAUNCH_CHECK();
    // FP32 LU of the equilibrated matrix: first without pivoting (no inter-CTA
    // pivot exchange); on a zero / non-finite pivot, again with partial pivoting.
    gk_status s = gk_internal_lu_factor_nopiv_f32(n, w.K32, S.ld32, w.ipiv, w.luw, w.luw_bytes, info, st);
    if (s != GK_OK) return s;
    int pivoted = 0;
    {
        int32_t fst = 0;
        GK_CUDA_TRY(cudaMemcpyAsync(&fst, &info->status, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
        GK_CUDA_TRY(cudaStreamSynchronize(st));
        if (fst != 0) {
            convert_kernel<<<cg, 256, 0, st>>>(K, ldk, n, w.d, w.K32, S.ld32);
            GK_LAUNCH_CHECK();
            s = gk_internal_lu_factor_f32(n, w.K32, S.ld32, w.ipiv, w.luw, w.luw_bytes, info, st);
            if (s != GK_OK) return s;
            pivoted = 1;
        }
    }

    int status = GK_ERR_NOT_CONVERGED, its = 0;
    double rel = 1.0;
    if ((s = fgmres(S, b, x, nullptr, tol, max_iter, status, its, rel)) != GK_OK) return s;
    {
        gk_info hi;
        GK_CUDA_TRY(cudaMemcpyAsync(&hi, info, sizeof(gk_info), cudaMemcpyDeviceToHost, st));
        GK_CUDA_TRY(cudaStreamSynchronize(st));
        if (hi.status == 0 && status != GK_OK) hi.status = status;
        hi.iterations = its;
        hi.pivoted = pivoted;
        hi.residual = rel;
        GK_CUDA_TRY(cudaMemcpyAsync(info, &hi, sizeof(gk_info), cudaMemcpyHostToDevice, st));
        GK_CUDA_TRY(cudaStreamSynchronize(st));
    }
    return GK_OK;
}

// ---------------------------------------------------------------------------
// FGMRES with the two-level (block-Jacobi + low-rank) preconditioner
// ---------------------------------------------------------------------------
// GK_FF: FP64 storage, restricted updates in float-float on the FP32 pipe
// (panel split buffers appended to the workspace).
static size_t twolevel_bytes(int64_t n, gk_prec prec) {
    size_t b = mixed_bytes(n, prec == GK_F32 ? 4 : 8, kRestartTwoLevel);
    if (prec == GK_FF) b += al(gk_internal_ff_panel_floats(n) * sizeof(float));
    return b;
}

extern "C" size_t gk_solve_twolevel_workspace_bytes(int64_t n, gk_prec prec) {
    if (n <= 0 || (prec != GK_F32 && prec != GK_F64 && prec != GK_FF)) return 0;
    return twolevel_bytes(n, prec);
}

extern "C" gk_status gk_solve_twolevel(int64_t n, const double* K, int64_t ldk, const double* b, double* x,
                                       const double* x0, const int32_t* perm, int64_t r, int32_t bs, gk_prec prec, double tol,
                                       int32_t max_iter, void* work, size_t work_bytes, gk_info* info,
                                       gk_stream stream) {
    cudaStream_t st = (cudaStream_t)stream;
    if (n <= 0 || K == nullptr || b == nullptr || x == nullptr || perm == nullptr || ldk < n || max_iter < 1)
        return GK_ERR_ARG;
    if (x0 == x) return GK_ERR_ARG;
    if (r <= 0 || r >= n || (r % 64) != 0 || bs <= 0 || (bs % 64) != 0 || bs > 4096) return GK_ERR_ARG;
    if (prec != GK_F32 && prec != GK_F64 && prec != GK_FF) return GK_ERR_ARG;
    const int es = prec == GK_F32 ? 4 : 8;
    if (work == nullptr || work_bytes < twolevel_bytes(n, prec)) return GK_ERR_SIZE;
    float* ffpanel = prec == GK_FF ? (float*)((char*)work + mixed_bytes(n, es, kRestartTwoLevel)) : nullptr;
    Solver S;
    S.n = n; S.K = K; S.ldk = ldk; S.w = carve(work, n, es, kRestartTwoLevel); S.ld32 = ld32_of(n); S.st = st;
    S.m = kRestartTwoLevel;
    if (info == nullptr) info = S.w.iinfo;
    S.info = info;
    S.vb = (unsigned)((n + 255) / 256);
    S.rb = (unsigned)((n * 32 + 255) / 256);
    S.mode = prec == GK_F32 ? 1 : 2;
    S.perm = perm;
    S.r = r;
    S.bs = bs;
    MixedWork& w = S.w;
    GK_CUDA_TRY(cudaMemsetAsync(info, 0, sizeof(gk_info), st));
    equil_kernel<<<S.rb, 256, 0, st>>>(K, ldk, n, w.d);
    GK_LAUNCH_CHECK();
    gk_status s = prec != GK_F32
                      ? gk_internal_twolevel_setup_f64(n, K, ldk, perm, w.d, r, bs, w.K64, S.ld32, w.ipiv, w.luw,
                                                       w.luw_bytes, info, st, ffpanel)
                      : gk_internal_twolevel_setup(n, K, ldk, perm, w.d, r, bs, w.K32, S.ld32, w.ipiv, w.luw,
                                                   w.luw_bytes, info, st);
    if (s != GK_OK) return s;
    int32_t fst = 0;
    GK_CUDA_TRY(cudaMemcpyAsync(&fst, &info->status, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    GK_CUDA_TRY(cudaStreamSynchronize(st));
    int status = GK_ERR_NOT_CONVERGED, its = 0;
    double rel = 1.0;
    if (fst == 0) {
        if ((s = fgmres(S, b, x, x0, tol, max_iter, status, its, rel)) != GK_OK) return s;
    } else {
        status = fst;
    }
    gk_info hi;
    GK_CUDA_TRY(cudaMemcpyAsync(&hi, info, sizeof(gk_info), cudaMemcpyDeviceToHost, st));
    GK_CUDA_TRY(cudaStreamSynchronize(st));
    if (hi.status == 0 && status != GK_OK) hi.status = status;
    hi.iterations = its;
    hi.pivoted = 0;
    hi.residual = rel;
    GK_CUDA_TRY(cudaMemcpyAsync(info, &hi, sizeof(gk_info), cudaMemcpyHostToDevice, st));
    GK_CUDA_TRY(cudaStreamSynchronize(st));
    return GK_OK;
}

// ---------------------------------------------------------------------------
// Allocation-free variant of gk_solve_mixed.
//
// Its scratch is this file-scope device array.  Every GPU that loads the
// library holds it (8 MiB) until the process exits, and every call shares it:
// each call rewrites or clears everything it reads before reading it, and two
// calls that overlap on the GPU (different streams, or without ordering
// between them) race on it.  Host code cannot use the array's name as a device
// address; the address is looked up once per device with
// cudaGetSymbolAddress, by the first call made with that device current.
// ---------------------------------------------------------------------------
namespace {
constexpr size_t kNoAllocBytes = (size_t)8 << 20;
constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mutex;
void* g_noalloc_ptr[kMaxDevices] = {};
}  // namespace

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

extern "C" gk_status gk_solve_mixed_noalloc(int64_t n, const double* K, int64_t ldk, const double* b, double* x,
                                            double tol, int32_t max_iter, gk_info* info, gk_stream stream) {
    if (n <= 0 || K == nullptr || b == nullptr || x == nullptr || ldk < n || max_iter < 1) return GK_ERR_ARG;
    if (n > GK_NOALLOC_MAX_N) return GK_ERR_SIZE;
    if (mixed_bytes(n) > kNoAllocBytes) return GK_ERR_SIZE;
    int dev = -1;
    GK_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return GK_ERR_CUDA;
    void* ptr = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_noalloc_mutex);
        if (g_noalloc_ptr[dev] == nullptr) {
            void* p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess || p == nullptr) {
                (void)cudaGetLastError();
                return GK_ERR_CUDA;
            }
            g_noalloc_ptr[dev] = p;
        }
        ptr = g_noalloc_ptr[dev];
    }
    return gk_solve_mixed(n, K, ldk, b, x, tol, max_iter, ptr, kNoAllocBytes, info, stream);
}
