// Batched co-kriging: many realisations of uneven size built, solved and
// evaluated by a fixed sequence of persistent kernels, with every decision
// (work claiming, convergence, segmentation thresholds) taken on the device,
// so the whole sequence can be captured once in a CUDA graph and replayed.
//
//   batch_build_kernel    32 x 32 tiles of every realisation's FP64 K, claimed
//                         from one global counter (tiles of all systems in one
//                         list), plus the right-hand sides.
//   batch_solve_kernel    one CTA per realisation, largest first: symmetric
//                         equilibration, FP32 LU without pivoting, FGMRES(30)
//                         in FP64 preconditioned by the FP32 factors, Givens
//                         rotations and convergence tests on the device.
//   batch_prepare_kernel  one CTA per realisation: interface weights per point,
//                         float-float records, drift weights, FP64 isovalues at
//                         the reference points (warp-shuffle reductions), sort.
//   batch_eval_kernel     float-float field + fused segmentation over
//                         (realisation, 1024-point chunk) items; record tiles
//                         staged by cp.async.bulk with mbarrier completion.
//
// Replaces, for many models at once, the engine work behind
// gempy/API/compute_API.py:68-73 (one compute_model per realisation).
#include <cstring>
#include <vector>
#include <algorithm>

#include "gk_ff.cuh"
#include "gk_kriging.cuh"
#include "gk_cta.cuh"
#include "gk_tune.h"

namespace gk {

constexpr int kBatchRestart = 30;

struct BatchDesc {
    // inputs (pointers into the caller's concatenated arrays)
    const double* dip;
    const double* grad;
    const double* nug_g;
    const double* sp;
    const double* nug_sp;
    const int32_t* ref;
    const int32_t* rest;
    int n_ori, n_sp, n_iface, degree, kernel, N, ld;
    double range, c_o, i_res, gi_res;
    // workspace
    double* K64;
    float* K32;
    double* b;
    double* x;
    double* dsc;
    double* r;
    double* w;
    double* V;     // (restart + 1) x N
    double* Z;     // restart x N
    float* t32;
    double* alpha;
    float* rec;    // float-float records: n_ori x 16 floats, then n_sp x 8 floats
    double* meta;  // [0] quantum, [1] max|u| bits, [2] 1/range, [3..18] drift weights
    double* iso;   // isovalues sorted, highest first
    // segmentation and grid
    int n_surf;
    int surf_start[GK_MAX_SURFACES];
    double slope;
    double unit_values[GK_MAX_SURFACES + 1];
    double origin[3], spacing[3];
    int dims[3];
    int64_t n_points, out_off;
    int64_t tile_begin, chunk_begin;
    int tile_side;
};

__device__ __forceinline__ int find_system(const int64_t* prefix, int n, int64_t item) {
    int lo = 0, hi = n;  // prefix[lo] <= item < prefix[hi]
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (prefix[mid] <= item) lo = mid; else hi = mid;
    }
    return lo;
}

// ---------------------------------------------------------------------------
// build
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) batch_build_kernel(const BatchDesc* __restrict__ D, int n_sys,
                                                          const int64_t* __restrict__ tile_prefix, int* counter) {
    __shared__ Item rows[32], cols[32];
    __shared__ int64_t s_item;
    __shared__ int s_sys;
    const int tid = threadIdx.y * 32 + threadIdx.x;
    const int64_t total = tile_prefix[n_sys];
    while (true) {
        if (tid == 0) {
            s_item = atomicAdd(counter, 1);
            s_sys = s_item < total ? find_system(tile_prefix, n_sys, s_item) : -1;
        }
        __syncthreads();
        const int64_t item = s_item;
        const int sys = s_sys;
        if (item >= total) return;
        const BatchDesc& d = D[sys];
        BuildParams P;
        P.n_ori = d.n_ori; P.n_iface = d.n_iface; P.degree = d.degree; P.n_drift = drift_count(d.degree);
        P.kernel = d.kernel; P.N = d.N; P.range = d.range; P.c_o = d.c_o; P.i_res = d.i_res; P.gi_res = d.gi_res;
        P.dip_positions = d.dip; P.dip_gradients = d.grad; P.nugget_grad = d.nug_g; P.sp_coords = d.sp;
        P.nugget_sp = d.nug_sp; P.ref_index = d.ref; P.rest_index = d.rest;
        P.n_fault = 0; P.fault_sp = nullptr; P.n_sp = d.n_sp;
        const int64_t t = item - tile_prefix[sys];
        const int64_t r0 = (t / d.tile_side) * 32, c0 = (t % d.tile_side) * 32;
        if (tid < 32) {
            if (r0 + tid < P.N) decode(P, r0 + tid, rows[tid]);
        } else if (tid < 64) {
            if (c0 + tid - 32 < P.N) decode(P, c0 + tid - 32, cols[tid - 32]);
        }
        __syncthreads();
        const Cov<double> cv = Cov<double>::make(P.kernel, P.range);
        const int64_t j = c0 + threadIdx.x;
        for (int k = 0; k < 4; ++k) {
            const int rl = threadIdx.y + 8 * k;
            const int64_t i = r0 + rl;
            if (i < P.N && j < P.N) d.K64[i * d.ld + j] = entry<double>(P, cv, rows[rl], cols[threadIdx.x], i == j);
            if (c0 == 0 && threadIdx.x == 0 && i < P.N) {
                const Item& it = rows[rl];
                d.b[i] = it.type == 0 ? P.dip_gradients[3 * it.idx + it.comp] : 0.0;
            }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// solve: one CTA per system
// ---------------------------------------------------------------------------
constexpr int kSolveThreads = 512;

template <typename T>
__device__ __forceinline__ T block_sum(T v, T* red) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    __syncthreads();
    if (lane == 0) red[wid] = v;
    __syncthreads();
    T t = (T)0;
    if (threadIdx.x < (blockDim.x >> 5)) t = red[threadIdx.x];
    if (wid == 0)
        for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
    if (threadIdx.x == 0) red[0] = t;
    __syncthreads();
    T out = red[0];
    __syncthreads();
    return out;
}

// y = K64 x (rows by warps) ; b == nullptr -> y = K x, else y = b - K x
__device__ void cta_gemv64(const double* K, int ld, int N, const double* x, const double* b, double* y) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int row = wid; row < N; row += nw) {
        const double* k = K + (int64_t)row * ld;
        double s = 0.0;
        for (int j = lane; j < N; j += 32) s = fma(k[j], x[j], s);
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (lane == 0) y[row] = b ? b[row] - s : s;
    }
    __syncthreads();
}

// One system of the in-CTA mixed solve: K64 (FP64, read only), its FP32
// equilibrated copy K32, the right-hand side b, the solution x and scratch.
struct CtaSystem {
    const double* K64;
    int ld, N;
    float* K32;
    const double* b;
    double* x;
    double* dsc;
    double* r;
    double* w;
    double* V;     // (restart + 1) x N
    double* Z;     // restart x N
    float* t32;
};

struct CtaSolveShared {
    float Ds[kLNB][kLNB + 1];
    double red[32];
    float xs[kLNB];
    int s_bad;
    double H[(kBatchRestart + 1) * kBatchRestart];
    double cs[kBatchRestart], sn[kBatchRestart], g[kBatchRestart + 1], yv[kBatchRestart];
    double hcol[kBatchRestart + 2];
};

// Systems up to kSmemLuMaxN keep their equilibrated FP32 matrix in shared
// memory (N x (N + 1) floats, then 3N floats of scratch); up to kRegInvMaxN it
// is inverted there by register-resident Gauss-Jordan and every
// preconditioner application is one FP32 matrix-vector product, above that it
// is LU-factored in place and applied by triangular sweeps.
constexpr int kSmemLuMaxN = 224;
constexpr int kRegInvMaxN = 160;
__host__ __device__ constexpr size_t cta_smem_lu_bytes(int n) {
    return ((size_t)n * (n + 1) + 3 * (size_t)n) * sizeof(float);
}

// 2^-floor(e/2) for the binary exponent e of |v| (v >= 0, finite or not):
// a power-of-two row scale near 1/sqrt(max|row|), from the bits alone -- the
// FP64 pipe is ~1/64 of the FP32 one, and its sqrt and division sequences
// dominated the equilibration.  Zero rows keep scale 1.
__device__ __forceinline__ double pow2_rsqrt_scale(unsigned long long bits) {
    const int e = (int)((bits >> 52) & 0x7ff);
    if (e == 0) return 1.0;                       // zero or subnormal
    const int ub = e - 1023;                      // |v| in [2^ub, 2^(ub+1))
    const int h = ub >= 0 ? ub / 2 : -((-ub + 1) / 2);   // floor(ub / 2)
    return __longlong_as_double((long long)(1023 - h) << 52);
}

// The whole mixed solve of one system by the calling CTA: symmetric
// equilibration by powers of two, an FP32 preconditioner without pivoting,
// FGMRES(30) in FP64 with Givens rotations and convergence tests on the
// device.  When ``sm`` is given the FP32 matrix lives in shared memory
// (leading dimension ``sld``, then 3N floats of scratch) and is inverted
// (N <= kRegInvMaxN) or LU-factored there; otherwise it is LU-factored in the
// global workspace.  Returns the status, iteration count and final relative
// residual.
__device__ void cta_mixed_solve(const CtaSystem& d, double tol, int max_iter, CtaSolveShared& sh, int& status_out,
                                int& its_out, double& rel_out, float* sm = nullptr, int sld = 0) {
    auto& Ds = sh.Ds;
    double* red = sh.red;
    float* xs = sh.xs;
    int& s_bad = sh.s_bad;
    double* H = sh.H;
    double* cs = sh.cs;
    double* sn = sh.sn;
    double* g = sh.g;
    double* yv = sh.yv;
    double* hcol = sh.hcol;
    const int tid = threadIdx.x, nt = blockDim.x;
    const int N = d.N, ld = d.ld;
    // equilibration (row and column scales, powers of two) and FP32 copy
    {
        const int lane = tid & 31, wid = tid >> 5;
        for (int row = wid; row < N; row += nt >> 5) {
            const unsigned long long* k = reinterpret_cast<const unsigned long long*>(d.K64 + (int64_t)row * ld);
            unsigned long long m = 0;   // max |K_ij| compared as bit patterns (sign cleared)
            for (int j = lane; j < N; j += 32) m = max(m, k[j] & 0x7fffffffffffffffULL);
            for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_down_sync(0xffffffffu, m, o));
            if (lane == 0) d.dsc[row] = pow2_rsqrt_scale(m);
        }
        __syncthreads();
        for (int row = wid; row < N; row += nt >> 5) {
            const float di = (float)d.dsc[row];
            const double* k = d.K64 + (int64_t)row * ld;
            float* k32 = sm ? sm + (int64_t)row * sld : d.K32 + (int64_t)row * ld;
            // scaling by powers of two is exact: one rounding, in the conversion
            for (int j = lane; j < N; j += 32) k32[j] = (float)k[j] * (di * (float)d.dsc[j]);
        }
        __syncthreads();
    }
    int status = GK_OK, its = 0;
    double rel = 1.0;
    float* const K32 = sm ? sm : d.K32;
    const int ld32 = sm ? sld : ld;
    float* const t32 = sm ? sm + (int64_t)N * sld : d.t32;
    const bool inverse = sm != nullptr && N <= kRegInvMaxN;
    bool factored;
    if (inverse)
        factored = N <= 128 ? cta_gauss_jordan_regs<8, 4>(K32, ld32, N, t32 + N, t32 + 2 * N)
                            : cta_gauss_jordan_regs<10, 5>(K32, ld32, N, t32 + N, t32 + 2 * N);
    else
        factored = cta_lu_nopiv(K32, ld32, N, Ds, &s_bad);
    if (!factored) {
        status = GK_ERR_SINGULAR;
    } else {
        // FGMRES(restart) in FP64
        for (int i = tid; i < N; i += nt) d.x[i] = 0.0;
        __syncthreads();
        double bn = 0.0;
        {
            double s = 0.0;
            for (int i = tid; i < N; i += nt) s += d.b[i] * d.b[i];
            bn = sqrt(block_sum(s, red));
        }
        double prev = INFINITY;
        status = GK_ERR_NOT_CONVERGED;
        if (!(bn > 0.0)) { status = GK_OK; rel = 0.0; }
        bool x_zero = true;   // the first residual is b itself
        while (status == GK_ERR_NOT_CONVERGED && its < max_iter) {
            if (x_zero) {
                for (int i = tid; i < N; i += nt) d.r[i] = d.b[i];
                __syncthreads();
                x_zero = false;
            } else {
                cta_gemv64(d.K64, ld, N, d.x, d.b, d.r);
            }
            double s = 0.0;
            for (int i = tid; i < N; i += nt) s += d.r[i] * d.r[i];
            const double beta = sqrt(block_sum(s, red));
            rel = beta / bn;
            if (!(rel == rel)) { status = GK_ERR_NONFINITE; break; }
            if (rel <= tol) { status = GK_OK; break; }
            if (rel > 0.98 * prev) break;
            prev = rel;
            const double ibeta = 1.0 / beta;
            for (int i = tid; i < N; i += nt) d.V[i] = d.r[i] * ibeta;
            if (tid == 0) { for (int q = 0; q <= kBatchRestart; ++q) g[q] = 0.0; g[0] = beta; }
            __syncthreads();
            int j = 0;
            bool done = false;
            for (; j < kBatchRestart && its < max_iter; ++j, ++its) {
                const double* vj = d.V + (int64_t)j * N;
                double* zj = d.Z + (int64_t)j * N;
                for (int i = tid; i < N; i += nt) t32[i] = (float)vj[i] * (float)d.dsc[i];
                __syncthreads();
                if (inverse) {
                    // z = D Kinv D v: warp per row of the inverse
                    const int lane = tid & 31, wid = tid >> 5;
                    for (int row = wid; row < N; row += nt >> 5) {
                        const float* ar = K32 + (int64_t)row * ld32;
                        float acc = 0.f;
                        for (int c = lane; c < N; c += 32) acc = fmaf(ar[c], t32[c], acc);
                        for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
                        if (lane == 0) zj[row] = d.dsc[row] * (double)acc;
                    }
                } else {
                    cta_lu_solve(K32, ld32, N, t32, xs);
                    for (int i = tid; i < N; i += nt) zj[i] = d.dsc[i] * (double)t32[i];
                }
                __syncthreads();
                cta_gemv64(d.K64, ld, N, zj, nullptr, d.w);
                // CGS2: warp w computes the dot products c = w, w + 16, ...
                for (int pass = 0; pass < 2; ++pass) {
                    {
                        const int lane = tid & 31, wid = tid >> 5;
                        for (int c = wid; c <= j; c += nt >> 5) {
                            const double* vc = d.V + (int64_t)c * N;
                            double sd = 0.0;
                            for (int i = lane; i < N; i += 32) sd = fma(vc[i], d.w[i], sd);
                            for (int o = 16; o > 0; o >>= 1) sd += __shfl_down_sync(0xffffffffu, sd, o);
                            if (lane == 0) {
                                yv[c] = sd;
                                hcol[c] = (pass == 0 ? 0.0 : hcol[c]) + sd;
                            }
                        }
                    }
                    __syncthreads();
                    for (int i = tid; i < N; i += nt) {
                        double v = d.w[i];
                        for (int c = 0; c <= j; ++c) v -= d.V[(int64_t)c * N + i] * yv[c];
                        d.w[i] = v;
                    }
                    __syncthreads();
                }
                double sn2 = 0.0;
                for (int i = tid; i < N; i += nt) sn2 += d.w[i] * d.w[i];
                const double hn = sqrt(block_sum(sn2, red));
                if (hn > 0.0) {
                    const double ihn = 1.0 / hn;
                    for (int i = tid; i < N; i += nt) d.V[(int64_t)(j + 1) * N + i] = d.w[i] * ihn;
                }
                if (tid == 0) {
                    hcol[j + 1] = hn;
                    for (int i = 0; i < j; ++i) {
                        double t = cs[i] * hcol[i] + sn[i] * hcol[i + 1];
                        hcol[i + 1] = -sn[i] * hcol[i] + cs[i] * hcol[i + 1];
                        hcol[i] = t;
                    }
                    const double den = hypot(hcol[j], hcol[j + 1]);
                    const double iden = den > 0 ? 1.0 / den : 0.0;
                    cs[j] = den > 0 ? hcol[j] * iden : 1.0;
                    sn[j] = hcol[j + 1] * iden;
                    hcol[j] = den;
                    g[j + 1] = -sn[j] * g[j];
                    g[j] = cs[j] * g[j];
                    for (int i = 0; i <= j; ++i) H[i * kBatchRestart + j] = hcol[i];
                    red[31] = (fabs(g[j + 1]) <= tol * bn || hn == 0.0) ? 1.0 : 0.0;
                }
                __syncthreads();
                if (red[31] != 0.0) { ++j; ++its; done = true; break; }
            }
            (void)done;
            if (tid == 0) {
                for (int i = j - 1; i >= 0; --i) {
                    double t = g[i];
                    for (int q = i + 1; q < j; ++q) t -= H[i * kBatchRestart + q] * yv[q];
                    yv[i] = H[i * kBatchRestart + i] != 0.0 ? t / H[i * kBatchRestart + i] : 0.0;
                }
            }
            __syncthreads();
            for (int i = tid; i < N; i += nt) {
                double v = d.x[i];
                for (int c = 0; c < j; ++c) v += d.Z[(int64_t)c * N + i] * yv[c];
                d.x[i] = v;
            }
            __syncthreads();
        }
        if (status == GK_ERR_NOT_CONVERGED) {
            cta_gemv64(d.K64, ld, N, d.x, d.b, d.r);
            double s = 0.0;
            for (int i = tid; i < N; i += nt) s += d.r[i] * d.r[i];
            rel = sqrt(block_sum(s, red)) / bn;
            if (rel <= tol) status = GK_OK;
        }
    }
    status_out = status;
    its_out = its;
    rel_out = rel;
}

__global__ void __launch_bounds__(kSolveThreads) batch_solve_kernel(const BatchDesc* __restrict__ D, int n_sys,
                                                                    const int32_t* __restrict__ order,
                                                                    int* counter, double tol, int max_iter,
                                                                    gk_info* infos) {
    __shared__ CtaSolveShared sh;
    __shared__ int s_sys;
    const int tid = threadIdx.x;
    while (true) {
        if (tid == 0) {
            int k = atomicAdd(counter, 1);
            s_sys = k < n_sys ? order[k] : -1;
        }
        __syncthreads();
        const int sys = s_sys;
        if (sys < 0) return;
        const BatchDesc& bd = D[sys];
        const CtaSystem d{bd.K64, bd.ld, bd.N, bd.K32, bd.b, bd.x, bd.dsc, bd.r, bd.w, bd.V, bd.Z, bd.t32};
        int status, its;
        double rel;
        cta_mixed_solve(d, tol, max_iter, sh, status, its, rel);
        if (tid == 0 && infos != nullptr) {
            infos[sys].status = status;
            infos[sys].where = 0;
            infos[sys].iterations = its;
            infos[sys].pivoted = 0;
            infos[sys].residual = rel;
        }
        __syncthreads();
    }
}

// Independent systems, one CTA each (systems passed by value).
constexpr int kCtaJobs = GK_CTA_MAX_JOBS;
struct CtaJobs {
    CtaSystem sys[kCtaJobs];
    gk_info* info[kCtaJobs];
};

// sld > 0: every system fits kSmemLuMaxN and the dynamic shared memory holds
// its FP32 matrix and factors (leading dimension sld) and N floats.
__global__ void __launch_bounds__(kSolveThreads) mixed_cta_kernel(const __grid_constant__ CtaJobs jobs, double tol,
                                                                  int max_iter, int sld) {
    __shared__ CtaSolveShared sh;
    extern __shared__ float cta_dyn[];
    int status, its;
    double rel;
    cta_mixed_solve(jobs.sys[blockIdx.x], tol, max_iter, sh, status, its, rel, sld > 0 ? cta_dyn : nullptr, sld);
    gk_info* info = jobs.info[blockIdx.x];
    if (threadIdx.x == 0 && info != nullptr) {
        info->status = status;
        info->where = 0;
        info->iterations = its;
        info->pivoted = 0;
        info->residual = rel;
    }
}

// ---------------------------------------------------------------------------
// prepare: per-point interface weights, float-float records, isovalues
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) batch_prepare_kernel(const BatchDesc* __restrict__ D, int n_sys) {
    __shared__ unsigned int s_max;
    __shared__ double s_iso[GK_MAX_SURFACES];
    const int sys = blockIdx.x;
    if (sys >= n_sys) return;
    const BatchDesc& d = D[sys];
    const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, wid = tid >> 5;
    const double gi = d.gi_res, inv_a = 1.0 / d.range;
    const double* wv = d.x;
    const int ng = 3 * d.n_ori;
    // alpha: rest points get gi w_t, each reference point minus the sum over its run
    for (int i = tid; i < d.n_sp; i += nt) d.alpha[i] = 0.0;
    __syncthreads();
    for (int t = tid; t < d.n_iface; t += nt) d.alpha[d.rest[t]] = gi * wv[ng + t];
    __syncthreads();
    for (int t = tid; t < d.n_iface; t += nt) {
        if (t > 0 && d.ref[t - 1] == d.ref[t]) continue;
        double s = 0.0;
        for (int u = t; u < d.n_iface && d.ref[u] == d.ref[t]; ++u) s += wv[ng + u];
        atomicAdd(d.alpha + d.ref[t], -gi * s);
    }
    if (tid == 0) s_max = 0u;
    __syncthreads();
    // quantum of the float-float split
    for (int i = tid; i < 3 * d.n_ori; i += nt) atomicMax(&s_max, __float_as_uint((float)fabs(d.dip[i] * inv_a)));
    for (int i = tid; i < 3 * d.n_sp; i += nt) atomicMax(&s_max, __float_as_uint((float)fabs(d.sp[i] * inv_a)));
    __syncthreads();
    float mx = __uint_as_float(s_max);
    if (!(mx > 1e-30f)) mx = 1.f;
    const double q = ldexp(1.0, (int)ceil(log2((double)mx)) + 4 - 23);
    if (tid == 0) {
        d.meta[0] = q;
        d.meta[2] = inv_a;
        for (int k = 0; k < 16; ++k) d.meta[3 + k] = k < drift_count(d.degree) ? gi * wv[ng + d.n_iface + k] : 0.0;
    }
    const double so = d.c_o * gi * inv_a, ss = d.c_o * gi;
    for (int i = tid; i < d.n_ori; i += nt) {
        float* r = d.rec + 16 * (int64_t)i;
        for (int k = 0; k < 3; ++k) ff_split(d.dip[3 * i + k] * inv_a, q, r[2 * k], r[2 * k + 1]);
        for (int k = 0; k < 3; ++k) {
            ff v = ff_from_double(so * wv[k * d.n_ori + i]);
            r[6 + 2 * k] = v.h;
            r[7 + 2 * k] = v.l;
        }
        for (int k = 12; k < 16; ++k) r[k] = 0.f;
    }
    __syncthreads();
    for (int i = tid; i < d.n_sp; i += nt) {
        float* r = d.rec + 16 * (int64_t)d.n_ori + 8 * (int64_t)i;
        for (int k = 0; k < 3; ++k) ff_split(d.sp[3 * i + k] * inv_a, q, r[2 * k], r[2 * k + 1]);
        ff v = ff_from_double(ss * d.alpha[i]);
        r[6] = v.h;
        r[7] = v.l;
    }
    // FP64 isovalues at each surface's reference point: one warp per surface
    const Cov<double> cv = Cov<double>::make(d.kernel, d.range);
    for (int k = wid; k < d.n_surf; k += nt >> 5) {
        // reference point of surface k: its first point
        const int start = d.surf_start[k];
        const double x0 = d.sp[3 * start], y0 = d.sp[3 * start + 1], z0 = d.sp[3 * start + 2];
        double z = 0.0;
        for (int o = lane; o < d.n_ori; o += 32) {
            const double hx = d.dip[3 * o] - x0, hy = d.dip[3 * o + 1] - y0, hz = d.dip[3 * o + 2] - z0;
            const double rr = sqrt(hx * hx + hy * hy + hz * hz + kDistEps2);
            z += d.c_o * cv.d1_r(rr) *
                 (wv[o] * hx + wv[d.n_ori + o] * hy + wv[2 * d.n_ori + o] * hz);
        }
        for (int p = lane; p < d.n_sp; p += 32) {
            const double hx = x0 - d.sp[3 * p], hy = y0 - d.sp[3 * p + 1], hz = z0 - d.sp[3 * p + 2];
            z += d.c_o * d.alpha[p] * cv.C(sqrt(hx * hx + hy * hy + hz * hz + kDistEps2));
        }
        for (int o = 16; o > 0; o >>= 1) z += __shfl_down_sync(0xffffffffu, z, o);
        if (lane == 0) {
            const int nd = drift_count(d.degree);
            const double* mu = wv + ng + d.n_iface;
            if (nd >= 3) z += mu[0] * x0 + mu[1] * y0 + mu[2] * z0;
            if (nd >= 9)
                z += mu[3] * x0 * x0 + mu[4] * y0 * y0 + mu[5] * z0 * z0 + mu[6] * x0 * y0 + mu[7] * x0 * z0 +
                     mu[8] * y0 * z0;
            s_iso[k] = gi * z;
        }
    }
    __syncthreads();
    if (tid == 0) {
        // sort isovalues, highest first (n_surf <= 32: insertion sort)
        double v[GK_MAX_SURFACES];
        for (int k = 0; k < d.n_surf; ++k) v[k] = s_iso[k];
        for (int a = 1; a < d.n_surf; ++a) {
            double t = v[a];
            int c = a - 1;
            while (c >= 0 && v[c] < t) { v[c + 1] = v[c]; --c; }
            v[c + 1] = t;
        }
        for (int k = 0; k < d.n_surf; ++k) d.iso[k] = v[k];
        for (int k = 0; k < d.n_surf; ++k) d.iso[GK_MAX_SURFACES + k] = s_iso[k];  // stack order, for callers
    }
}

// ---------------------------------------------------------------------------
// evaluation: float-float field + segmentation over (system, chunk) items
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

constexpr int kChunkPoints = 1024;  // points per (system, chunk) item, whatever the variant

struct Cursor {
    int64_t k;   // index into this CTA's item list
    int t;       // tile within the item
};

template <int kPPT, int kStage>
__global__ void __launch_bounds__(256) batch_eval_kernel(const BatchDesc* __restrict__ D, int n_sys,
                                                         const int64_t* __restrict__ chunk_prefix, double* field,
                                                         double* values, int32_t* ids, gk_info* infos) {
    static_assert(kChunkPoints % (256 * kPPT) == 0, "chunk is a whole number of passes");
    constexpr int kPasses = kChunkPoints / (256 * kPPT);
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t mbar[2];
    __shared__ int s_fail;
    __shared__ float s_box[6 * 8];
    const int tid = threadIdx.x;
    unsigned char* stage[2] = {smem, smem + kStage};
    const int rec_ori = kStage / 64, rec_sp = kStage / 32;
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&mbar[0])), "r"(1) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&mbar[1])), "r"(1) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        s_fail = 0;
    }
    __syncthreads();
    const int64_t total = chunk_prefix[n_sys];
    const int64_t my_items = total > blockIdx.x ? (total - 1 - blockIdx.x) / gridDim.x + 1 : 0;
    auto tiles_of = [&](int s) {
        const BatchDesc& d = D[s];
        return (d.n_ori + rec_ori - 1) / rec_ori + (d.n_sp + rec_sp - 1) / rec_sp;
    };
    // producer cursor (thread 0 only)
    Cursor pc{0, 0};
    int64_t issued = 0;
    auto issue_next = [&]() {
        if (tid != 0) return;
        while (pc.k < my_items) {
            const int64_t item = blockIdx.x + pc.k * gridDim.x;
            const int s = find_system(chunk_prefix, n_sys, item);
            const int nt = tiles_of(s);
            // every pass over the item's points consumes all of its tiles once
            if (pc.t >= nt * kPasses) { pc.k++; pc.t = 0; continue; }
            const int tt = pc.t % nt;
            const BatchDesc& d = D[s];
            const int to = (d.n_ori + rec_ori - 1) / rec_ori;
            const void* src;
            uint32_t bytes;
            if (tt < to) {
                int r0 = tt * rec_ori, nr = min(rec_ori, d.n_ori - r0);
                src = d.rec + 16 * (int64_t)r0;
                bytes = (uint32_t)(nr * 64);
            } else {
                int r0 = (tt - to) * rec_sp, nr = min(rec_sp, d.n_sp - r0);
                src = d.rec + 16 * (int64_t)d.n_ori + 8 * (int64_t)r0;
                bytes = (uint32_t)(nr * 32);
            }
            const int sg = (int)(issued & 1);
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(&mbar[sg])),
                         "r"(bytes)
                         : "memory");
            asm volatile(
                "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                    smem_u32(stage[sg])),
                "l"(src), "r"(bytes), "r"(smem_u32(&mbar[sg]))
                : "memory");
            issued++;
            pc.t++;
            return;
        }
    };
    issue_next();
    issue_next();
    int64_t consumed = 0;
    for (int64_t k = 0; k < my_items; ++k) {
        const int64_t item = blockIdx.x + k * gridDim.x;
        const int s = find_system(chunk_prefix, n_sys, item);
        const BatchDesc& d = D[s];
        const int64_t c = item - chunk_prefix[s];
        const double q = d.meta[0], inv_a = d.meta[2];
        const float eps2 = fmaxf((float)(kDistEps2 * inv_a * inv_a), 1.17549435e-38f);  // a positive normal float
        const int nt = tiles_of(s);
        const int to = (d.n_ori + rec_ori - 1) / rec_ori;
        const int nyz = d.dims[1] * d.dims[2];
        // columns holding a multiple of kPPT points: each thread's points are
        // consecutive in one column and share x and y (ff_tile_col)
        const bool col = d.dims[2] % kPPT == 0;
        for (int pass = 0; pass < kPasses; ++pass) {
        PointFF X[kPPT];
        int64_t pid[kPPT];
        double Z[kPPT];
#pragma unroll
        for (int p = 0; p < kPPT; ++p) {
            pid[p] = c * kChunkPoints + pass * (256 * kPPT) + (col ? kPPT * tid + p : tid + p * 256);
            const int64_t qd = pid[p] < d.n_points ? pid[p] : d.n_points - 1;
            const int64_t ix = qd / nyz, rem = qd - ix * nyz;
            const int64_t iy = rem / d.dims[2], iz = rem - iy * d.dims[2];
            double xd[3] = {d.origin[0] + ix * d.spacing[0], d.origin[1] + iy * d.spacing[1],
                            d.origin[2] + iz * d.spacing[2]};
            ff_point(xd, inv_a, q, X[p]);
            Z[p] = 0.0;
        }
        bool all_exact = true, act[kPPT], any_act = false, all_act = true;
#pragma unroll
        for (int p = 0; p < kPPT; ++p) {
            act[p] = pid[p] < d.n_points;
            all_exact = all_exact && (X[p].exact || !act[p]);
            any_act = any_act || act[p];
            all_act = all_act && act[p];
        }
        // this pass's bounding box (high words), for the per-tile range test
        // of the column path (col is uniform over the CTA)
        float pbox[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
        if (col) {
#pragma unroll
            for (int p = 0; p < kPPT; ++p)
                if (act[p])
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        pbox[c] = fminf(pbox[c], X[p].h[c]);
                        pbox[3 + c] = fmaxf(pbox[3 + c], X[p].h[c]);
                    }
            cta_bbox(pbox, s_box);
        }
        for (int t = 0; t < nt; ++t) {
            const int sg = (int)(consumed & 1);
            const uint32_t parity = (uint32_t)((consumed >> 1) & 1);
            bool ok = false;
            const long long cap = wait_cap(kCopySpin);
            for (long long i = 0; i < cap && !ok; ++i) {
                uint32_t r;
                asm volatile(
                    "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, "
                    "p;\n}\n"
                    : "=r"(r)
                    : "r"(smem_u32(&mbar[sg])), "r"(parity)
                    : "memory");
                ok = r != 0;
            }
            if (!ok) {
                report(infos ? infos + s : nullptr, GK_ERR_TIMEOUT, -2);  // this realisation's status
                s_fail = 1;
            }
            __syncthreads();
            if (s_fail) {
                // wait (bounded) for the copies still in flight, then leave
                if (tid == 0) {
                    for (int64_t u = consumed; u < issued; ++u) {
                        for (long long i = 0; i < kCopySpin; ++i) {
                            uint32_t r;
                            asm volatile(
                                "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n "
                                "selp.u32 %0, 1, 0, p;\n}\n"
                                : "=r"(r)
                                : "r"(smem_u32(&mbar[u & 1])), "r"((uint32_t)((u >> 1) & 1))
                                : "memory");
                            if (r) break;
                        }
                    }
                }
                __syncthreads();
                return;
            }
            ffacc acc[kPPT];
#pragma unroll
            for (int p = 0; p < kPPT; ++p) acc[p] = {0.f, 0.f};
            const float* rec = reinterpret_cast<const float*>(stage[sg]);
            const bool ori = t < to;
            const int nr = ori ? min(rec_ori, d.n_ori - t * rec_ori) : min(rec_sp, d.n_sp - (t - to) * rec_sp);
            bool in_range = false;
            if (col) {
                // every point-record pair of the tile within the range?
                float rbox[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
                for (int r = tid; r < nr; r += blockDim.x) {
                    const float* R = rec + (ori ? 16 : 8) * r;
                    const float rx = R[0], ry = R[2], rz = R[4];
                    rbox[0] = fminf(rbox[0], rx);
                    rbox[1] = fminf(rbox[1], ry);
                    rbox[2] = fminf(rbox[2], rz);
                    rbox[3] = fmaxf(rbox[3], rx);
                    rbox[4] = fmaxf(rbox[4], ry);
                    rbox[5] = fmaxf(rbox[5], rz);
                }
                cta_bbox(rbox, s_box);
                float far2 = 0.f;
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const float m = fmaxf(pbox[3 + c] - rbox[c], rbox[3 + c] - pbox[c]) + (float)q;
                    far2 += m * m;
                }
                in_range = far2 * 1.001f + eps2 < 0.999f;
            }
            ff wsum = {0.f, 0.f};
            if (in_range && !ori) wsum = cta_weight_sum(rec, nr, s_box);   // uniform over the CTA
            if (!any_act) {
            } else if (col && all_exact && all_act) {
                if (in_range) {
                    if (!ori) {
#pragma unroll
                        for (int p = 0; p < kPPT; ++p) acc[p] = {wsum.h, wsum.l};
                    }
                    ff_tile_col<kPPT, false>(rec, ori, nr, X, eps2, acc);
                } else {
                    ff_tile_col<kPPT, true>(rec, ori, nr, X, eps2, acc);
                }
            } else if (all_exact && all_act) {
                ff_tile<kPPT, true, true>(rec, ori, nr, X, act, eps2, acc);
            } else if (all_exact) {
                ff_tile<kPPT, true>(rec, ori, nr, X, act, eps2, acc);
            } else {
                ff_tile<kPPT, false>(rec, ori, nr, X, act, eps2, acc);
            }
#pragma unroll
            for (int p = 0; p < kPPT; ++p) Z[p] += ff_acc_to_double(acc[p]);
            __syncthreads();
            consumed++;
            issue_next();
        }
        const double* mu = d.meta + 3;
        const int nd = drift_count(d.degree);
#pragma unroll
        for (int p = 0; p < kPPT; ++p) {
            if (pid[p] >= d.n_points) continue;
            const int64_t ix = pid[p] / nyz, rem = pid[p] - ix * nyz;
            const int64_t iy = rem / d.dims[2], iz = rem - iy * d.dims[2];
            const double X0 = d.origin[0] + ix * d.spacing[0], Y0 = d.origin[1] + iy * d.spacing[1],
                         Z0 = d.origin[2] + iz * d.spacing[2];
            double z = Z[p];
            if (nd >= 3) z += mu[0] * X0 + mu[1] * Y0 + mu[2] * Z0;
            if (nd >= 9)
                z += mu[3] * X0 * X0 + mu[4] * Y0 * Y0 + mu[5] * Z0 * Z0 + mu[6] * X0 * Y0 + mu[7] * X0 * Z0 +
                     mu[8] * Y0 * Z0;
            const int64_t o = d.out_off + pid[p];
            if (field) field[o] = z;
            double v = d.unit_values[0], vid = d.unit_values[0];
            for (int k2 = 0; k2 < d.n_surf; ++k2) {
                const double targ = d.slope * (d.iso[k2] - z);
                const float tf = (float)targ;
                const float sg = tf >= 0.f ? 1.f / (1.f + expf(-tf)) : expf(tf) / (1.f + expf(tf));
                v += (d.unit_values[k2 + 1] - d.unit_values[k2]) * (double)sg;
                // block id: a point on a surface takes the unit above it
                if (z < d.iso[k2] - GK_TIE_TOL) vid += d.unit_values[k2 + 1] - d.unit_values[k2];
            }
            if (values) values[o] = v;
            if (ids) ids[o] = (int32_t)rint(vid);
        }
        }  // pass
    }
}

cudaError_t wait_cap_set_batch(long long v) { return set_wait_cap_here(v); }

}  // namespace gk

// ---------------------------------------------------------------------------
// host API
// ---------------------------------------------------------------------------
using namespace gk;

namespace {

size_t al256(size_t x) { return (x + 255) & ~(size_t)255; }

struct Layout {
    size_t counters, tile_prefix, chunk_prefix, order, descs, data_begin, total;
    std::vector<size_t> sys_off;  // start of each system's region
};

int64_t item_N(const gk_batch_item& it) { return 3 * (int64_t)it.n_ori + it.n_iface + drift_count(it.uni_degree); }
int64_t item_ld(const gk_batch_item& it) { return (item_N(it) + 31) / 32 * 32; }
int64_t item_points(const gk_batch_item& it) { return (int64_t)it.dims[0] * it.dims[1] * it.dims[2]; }

size_t sys_bytes(const gk_batch_item& it) {
    const size_t N = (size_t)item_N(it), ld = (size_t)item_ld(it);
    size_t b = 0;
    b += al256(N * ld * sizeof(double));                    // K64
    b += al256(N * ld * sizeof(float));                     // K32
    b += 5 * al256(N * sizeof(double));                     // b, x, dsc, r, w
    b += al256((kBatchRestart + 1) * N * sizeof(double));   // V
    b += al256(kBatchRestart * N * sizeof(double));         // Z
    b += al256(N * sizeof(float));                          // t32
    b += al256((size_t)it.n_sp * sizeof(double));           // alpha
    b += al256(((size_t)16 * it.n_ori + 8 * (size_t)it.n_sp) * sizeof(float));  // records
    b += al256(32 * sizeof(double));                        // meta
    b += al256(2 * GK_MAX_SURFACES * sizeof(double));       // isovalues
    return b;
}

gk_status check_batch(const gk_batch* b) {
    if (b == nullptr || b->n_items <= 0 || b->items == nullptr) return GK_ERR_ARG;
    for (int i = 0; i < b->n_items; ++i) {
        const gk_batch_item& it = b->items[i];
        if (it.n_ori < 0 || it.n_sp < 0 || it.n_iface < 0 || it.n_iface > it.n_sp) return GK_ERR_ARG;
        if (it.uni_degree < 0 || it.uni_degree > 2 || it.kernel != GK_KERNEL_CUBIC) return GK_ERR_ARG;
        if (!(it.range > 0.0) || it.n_surf < 0 || it.n_surf > GK_MAX_SURFACES) return GK_ERR_ARG;
        if (it.dims[0] <= 0 || it.dims[1] <= 0 || it.dims[2] <= 0) return GK_ERR_ARG;
        int64_t sum = 0;
        for (int k = 0; k < it.n_surf; ++k) sum += it.points_per_surface[k];
        if (sum != it.n_sp || it.n_iface != it.n_sp - it.n_surf) return GK_ERR_ARG;
        if (item_N(it) <= 0 || item_N(it) > 16384) return GK_ERR_SIZE;
    }
    if (!b->dip_positions || !b->dip_gradients || !b->nugget_grad || !b->sp_coords || !b->nugget_sp ||
        !b->ref_index || !b->rest_index)
        return GK_ERR_ARG;
    return GK_OK;
}

Layout layout(const gk_batch* b) {
    Layout L;
    const size_t n = (size_t)b->n_items;
    size_t o = 0;
    L.counters = o; o += 256;
    L.tile_prefix = o; o += al256((n + 1) * sizeof(int64_t));
    L.chunk_prefix = o; o += al256((n + 1) * sizeof(int64_t));
    L.order = o; o += al256(n * sizeof(int32_t));
    L.descs = o; o += al256(n * sizeof(BatchDesc));
    L.data_begin = o;
    L.sys_off.resize(n);
    for (size_t i = 0; i < n; ++i) {
        L.sys_off[i] = o;
        o += sys_bytes(b->items[i]);
    }
    L.total = o;
    return L;
}

}  // namespace

extern "C" size_t gk_batch_workspace_bytes(const gk_batch* b) {
    if (check_batch(b) != GK_OK) return 0;
    return layout(b).total;
}

extern "C" int64_t gk_batch_points(const gk_batch* b) {
    if (check_batch(b) != GK_OK) return -1;
    int64_t t = 0;
    for (int i = 0; i < b->n_items; ++i) t += item_points(b->items[i]);
    return t;
}

extern "C" gk_status gk_batch_plan(const gk_batch* b, void* work, size_t work_bytes, gk_stream stream) {
    gk_status st = check_batch(b);
    if (st != GK_OK) return st;
    Layout L = layout(b);
    if (work == nullptr || work_bytes < L.total) return GK_ERR_SIZE;
    char* base = (char*)work;
    const int n = b->n_items;
    std::vector<BatchDesc> descs(n);
    std::vector<int64_t> tiles(n + 1, 0), chunks(n + 1, 0);
    std::vector<int32_t> order(n);
    int64_t out_off = 0;
    for (int i = 0; i < n; ++i) {
        const gk_batch_item& it = b->items[i];
        BatchDesc& d = descs[i];
        memset(&d, 0, sizeof(d));
        d.dip = b->dip_positions + 3 * it.ori_offset;
        d.grad = b->dip_gradients + 3 * it.ori_offset;
        d.nug_g = b->nugget_grad + it.ori_offset;
        d.sp = b->sp_coords + 3 * it.sp_offset;
        d.nug_sp = b->nugget_sp + it.sp_offset;
        d.ref = b->ref_index + it.iface_offset;
        d.rest = b->rest_index + it.iface_offset;
        d.n_ori = it.n_ori; d.n_sp = it.n_sp; d.n_iface = it.n_iface; d.degree = it.uni_degree;
        d.kernel = it.kernel; d.N = (int)item_N(it); d.ld = (int)item_ld(it);
        d.range = it.range; d.c_o = it.c_o; d.i_res = it.i_res; d.gi_res = it.gi_res;
        const size_t N = (size_t)d.N, ld = (size_t)d.ld;
        char* p = base + L.sys_off[i];
        d.K64 = (double*)p; p += al256(N * ld * sizeof(double));
        d.K32 = (float*)p; p += al256(N * ld * sizeof(float));
        d.b = (double*)p; p += al256(N * sizeof(double));
        d.x = (double*)p; p += al256(N * sizeof(double));
        d.dsc = (double*)p; p += al256(N * sizeof(double));
        d.r = (double*)p; p += al256(N * sizeof(double));
        d.w = (double*)p; p += al256(N * sizeof(double));
        d.V = (double*)p; p += al256((kBatchRestart + 1) * N * sizeof(double));
        d.Z = (double*)p; p += al256(kBatchRestart * N * sizeof(double));
        d.t32 = (float*)p; p += al256(N * sizeof(float));
        d.alpha = (double*)p; p += al256((size_t)it.n_sp * sizeof(double));
        d.rec = (float*)p; p += al256(((size_t)16 * it.n_ori + 8 * (size_t)it.n_sp) * sizeof(float));
        d.meta = (double*)p; p += al256(32 * sizeof(double));
        d.iso = (double*)p;
        d.n_surf = it.n_surf;
        int start = 0;
        for (int k = 0; k < it.n_surf; ++k) {
            d.surf_start[k] = start;
            start += it.points_per_surface[k];
        }
        d.slope = it.slope;
        for (int k = 0; k <= GK_MAX_SURFACES; ++k) d.unit_values[k] = it.unit_values[k];
        for (int k = 0; k < 3; ++k) {
            d.origin[k] = it.origin[k];
            d.spacing[k] = it.spacing[k];
            d.dims[k] = it.dims[k];
        }
        d.n_points = item_points(it);
        d.out_off = out_off;
        out_off += d.n_points;
        d.tile_side = (d.N + 31) / 32;
        tiles[i + 1] = tiles[i] + (int64_t)d.tile_side * d.tile_side;
        chunks[i + 1] = chunks[i] + (d.n_points + kChunkPoints - 1) / kChunkPoints;
        d.tile_begin = tiles[i];
        d.chunk_begin = chunks[i];
        order[i] = i;
    }
    // largest systems first (longest-processing-time order for the solve)
    std::stable_sort(order.begin(), order.end(), [&](int a, int c) { return descs[a].N > descs[c].N; });
    cudaStream_t s = (cudaStream_t)stream;
    GK_CUDA_TRY(cudaMemcpyAsync(base + L.tile_prefix, tiles.data(), (n + 1) * sizeof(int64_t),
                                cudaMemcpyHostToDevice, s));
    GK_CUDA_TRY(cudaMemcpyAsync(base + L.chunk_prefix, chunks.data(), (n + 1) * sizeof(int64_t),
                                cudaMemcpyHostToDevice, s));
    GK_CUDA_TRY(cudaMemcpyAsync(base + L.order, order.data(), n * sizeof(int32_t), cudaMemcpyHostToDevice, s));
    GK_CUDA_TRY(cudaMemcpyAsync(base + L.descs, descs.data(), n * sizeof(BatchDesc), cudaMemcpyHostToDevice, s));
    GK_CUDA_TRY(cudaStreamSynchronize(s));  // host vectors go out of scope
    return GK_OK;
}

template <int PPT, int STAGE>
static gk_status launch_batch_eval(const BatchDesc* D, int n, const int64_t* chunk_prefix, double* field,
                                   double* values, int32_t* ids, gk_info* infos, int sms, cudaStream_t s) {
    auto k = batch_eval_kernel<PPT, STAGE>;
    const size_t smem = 2 * (size_t)STAGE;
    int occ = 1;
    {
        const gk_status st = cached_occupancy((const void*)k, 256, smem, occ);
        if (st != GK_OK) return st;
    }
    k<<<sms * occ, 256, smem, s>>>(D, n, chunk_prefix, field, values, ids, infos);
    GK_LAUNCH_CHECK();
    return GK_OK;
}

extern "C" gk_status gk_batch_run(const gk_batch* b, void* work, size_t work_bytes, double tol, int32_t max_iter,
                                  double* field, double* values, int32_t* ids, gk_info* infos, gk_stream stream) {
    if (b == nullptr || b->n_items <= 0 || work == nullptr || max_iter < 1) return GK_ERR_ARG;
    // the plan fixed the layout; only its header offsets are needed here
    const size_t n = (size_t)b->n_items;
    size_t o = 256;
    const size_t tile_prefix = o; o += al256((n + 1) * sizeof(int64_t));
    const size_t chunk_prefix = o; o += al256((n + 1) * sizeof(int64_t));
    const size_t order = o; o += al256(n * sizeof(int32_t));
    const size_t descs = o;
    if (work_bytes < descs + al256(n * sizeof(BatchDesc))) return GK_ERR_SIZE;
    char* base = (char*)work;
    cudaStream_t s = (cudaStream_t)stream;
    int* counters = (int*)base;
    const BatchDesc* D = (const BatchDesc*)(base + descs);
    const int sms = device_sm_count();
    GK_CUDA_TRY(cudaMemsetAsync(counters, 0, 256, s));
    batch_build_kernel<<<sms * 4, dim3(32, 8), 0, s>>>(D, (int)n, (const int64_t*)(base + tile_prefix), counters);
    GK_LAUNCH_CHECK();
    const int solve_grid = (int)std::min<size_t>(n, (size_t)sms * 2);
    batch_solve_kernel<<<solve_grid, kSolveThreads, 0, s>>>(D, (int)n, (const int32_t*)(base + order), counters + 1,
                                                            tol, max_iter, infos);
    GK_LAUNCH_CHECK();
    batch_prepare_kernel<<<(unsigned)n, 256, 0, s>>>(D, (int)n);
    GK_LAUNCH_CHECK();
    const TuneVariant v = tune_variant(GK_TUNE_BATCH_EVAL);
    if (v.ppt == 4 && v.stage_kb == 32)
        return launch_batch_eval<4, 32 * 1024>(D, (int)n, (const int64_t*)(base + chunk_prefix), field, values, ids,
                                               infos, sms, s);
    if (v.ppt == 2 && v.stage_kb == 32)
        return launch_batch_eval<2, 32 * 1024>(D, (int)n, (const int64_t*)(base + chunk_prefix), field, values, ids,
                                               infos, sms, s);
    if (v.ppt == 4)
        return launch_batch_eval<4, 16 * 1024>(D, (int)n, (const int64_t*)(base + chunk_prefix), field, values, ids,
                                               infos, sms, s);
    return launch_batch_eval<2, 16 * 1024>(D, (int)n, (const int64_t*)(base + chunk_prefix), field, values, ids,
                                           infos, sms, s);
}

extern "C" gk_status gk_batch_results(const gk_batch* b, const void* work, size_t work_bytes, int32_t item,
                                      double* weights, double* isovalues, gk_stream stream) {
    gk_status st = check_batch(b);
    if (st != GK_OK) return st;
    if (item < 0 || item >= b->n_items) return GK_ERR_ARG;
    Layout L = layout(b);
    if (work == nullptr || work_bytes < L.total) return GK_ERR_SIZE;
    BatchDesc d;
    cudaStream_t s = (cudaStream_t)stream;
    GK_CUDA_TRY(cudaMemcpyAsync(&d, (const char*)work + L.descs + item * sizeof(BatchDesc), sizeof(BatchDesc),
                                cudaMemcpyDeviceToHost, s));
    GK_CUDA_TRY(cudaStreamSynchronize(s));
    if (weights) GK_CUDA_TRY(cudaMemcpyAsync(weights, d.x, d.N * sizeof(double), cudaMemcpyDeviceToDevice, s));
    if (isovalues)
        GK_CUDA_TRY(cudaMemcpyAsync(isovalues, d.iso + GK_MAX_SURFACES, d.n_surf * sizeof(double),
                                    cudaMemcpyDeviceToDevice, s));
    return GK_OK;
}

// ---------------------------------------------------------------------------
// single-system mixed solve in one CTA
// ---------------------------------------------------------------------------
static size_t cta_ws_layout(int64_t n, int64_t ld, size_t* off) {
    size_t o = 0;
    off[0] = o; o += al256((size_t)n * ld * sizeof(float));                     // K32
    off[1] = o; o += al256((size_t)n * sizeof(double));                          // dsc
    off[2] = o; o += al256((size_t)n * sizeof(double));                          // r
    off[3] = o; o += al256((size_t)n * sizeof(double));                          // w
    off[4] = o; o += al256((size_t)(kBatchRestart + 1) * n * sizeof(double));    // V
    off[5] = o; o += al256((size_t)kBatchRestart * n * sizeof(double));          // Z
    off[6] = o; o += al256((size_t)n * sizeof(float));                           // t32
    return o;
}

extern "C" size_t gk_solve_mixed_cta_workspace_bytes(int64_t n, int64_t ldk) {
    if (n < 1 || n > GK_CTA_MAX_N || ldk < n) return 0;
    size_t off[7];
    return cta_ws_layout(n, ldk, off);
}

static gk_status cta_job(const gk_cta_job& j, CtaSystem& d) {
    if (j.n < 1 || j.K == nullptr || j.b == nullptr || j.x == nullptr || j.ldk < j.n) return GK_ERR_ARG;
    if (j.n > GK_CTA_MAX_N) return GK_ERR_SIZE;
    size_t off[7];
    const size_t need = cta_ws_layout(j.n, j.ldk, off);
    if (j.work == nullptr || j.work_bytes < need) return GK_ERR_SIZE;
    char* w = (char*)j.work;
    d = CtaSystem{j.K, (int)j.ldk, (int)j.n, (float*)(w + off[0]), j.b, j.x, (double*)(w + off[1]),
                  (double*)(w + off[2]), (double*)(w + off[3]), (double*)(w + off[4]), (double*)(w + off[5]),
                  (float*)(w + off[6])};
    return GK_OK;
}

extern "C" gk_status gk_solve_mixed_cta_many(int32_t n_jobs, const gk_cta_job* jobs, double tol, int32_t max_iter,
                                             gk_stream stream) {
    if (n_jobs < 1 || jobs == nullptr || max_iter < 1 || !(tol > 0.0)) return GK_ERR_ARG;
    if (n_jobs > kCtaJobs) return GK_ERR_SIZE;
    CtaJobs J;
    memset(&J, 0, sizeof(J));
    for (int i = 0; i < n_jobs; ++i) {
        gk_status st = cta_job(jobs[i], J.sys[i]);
        if (st != GK_OK) return st;
        J.info[i] = jobs[i].info;
    }
    int n_max = 0;
    for (int i = 0; i < n_jobs; ++i) n_max = std::max(n_max, J.sys[i].N);
    int sld = 0;
    size_t smem = 0;
    if (n_max <= kSmemLuMaxN) {
        sld = n_max + 1;
        smem = cta_smem_lu_bytes(n_max);
        int occ = 0;
        if (cached_occupancy((const void*)mixed_cta_kernel, kSolveThreads, smem, occ) != GK_OK) {
            (void)cudaGetLastError();
            sld = 0;
            smem = 0;
        }
    }
    mixed_cta_kernel<<<n_jobs, kSolveThreads, smem, (cudaStream_t)stream>>>(J, tol, max_iter, sld);
    GK_LAUNCH_CHECK();
    return GK_OK;
}

extern "C" gk_status gk_solve_mixed_cta(int64_t n, const double* K, int64_t ldk, const double* b, double* x,
                                        double tol, int32_t max_iter, void* work, size_t work_bytes, gk_info* info,
                                        gk_stream stream) {
    gk_cta_job j{n, K, ldk, b, x, work, work_bytes, info};
    return gk_solve_mixed_cta_many(1, &j, tol, max_iter, stream);
}
