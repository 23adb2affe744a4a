// Kriging-matrix build: K = [[C_GG, C_GI, U_G, 0], [C_IG, C_II, U_I, F_I],
// [U_G^T, U_I^T, 0, 0], [0, F_I^T, 0, 0]] and the right-hand side, for one
// series, in FP64 or FP32 (F_I: the fault-block drift of the faults that offset
// the series).
//
// Row/column ordering (shared with the Python host code and the oracle):
//   gradient unknowns component-major (u * n_ori + o), interface rows in the
//   order of ref_index/rest_index, then the drift functions
//   (x, y, z [, x^2, y^2, z^2, xy, xz, yz]), then the fault drifts.
// Entry formulas restate the published co-kriging (GemPy 1.0, GMD 2019); the
// placement of i_res / gi_res, the nuggets inside the c_o factor and the 1e-5
// regulariser follow the conventions fitted to the reference's anticline
// approval file (test/test_model_types/test_example_models_I.py:41-53).
//
// Layout in HBM: K row-major with leading dimension ldk.  Each CTA computes a
// 32 x 32 tile; the 64 row/column descriptors of the tile are staged in shared
// memory once, then each thread evaluates 4 entries.  Writes are coalesced
// along rows (one warp = one tile row of 32 consecutive columns).
#include "gk_kriging.cuh"

namespace gk {

template <typename T>
__global__ void __launch_bounds__(256) build_kernel(BuildParams P, T* K, int64_t ldk, T* rhs) {
    __shared__ Item rows[32], cols[32];
    const int64_t r0 = (int64_t)blockIdx.y * 32, c0 = (int64_t)blockIdx.x * 32;
    const int tid = threadIdx.y * 32 + threadIdx.x;
    if (tid < 32) {
        if (r0 + tid < P.N) decode(P, r0 + tid, rows[tid]);
    } else if (tid < 64) {
        if (c0 + tid - 32 < P.N) decode(P, c0 + tid - 32, cols[tid - 32]);
    }
    __syncthreads();
    const Cov<T> cv = Cov<T>::make(P.kernel, P.range);
    const int64_t j = c0 + threadIdx.x;
    for (int k = 0; k < 4; ++k) {
        const int rl = threadIdx.y + 8 * k;
        const int64_t i = r0 + rl;
        if (i < P.N && j < P.N) K[i * ldk + j] = entry<T>(P, cv, rows[rl], cols[threadIdx.x], i == j);
    }
    if (rhs != nullptr && blockIdx.x == 0) {
        for (int k = 0; k < 4; ++k) {
            const int rl = threadIdx.y + 8 * k;
            const int64_t i = r0 + rl;
            if (threadIdx.x == 0 && i < P.N) {
                const Item& it = rows[rl];
                rhs[i] = it.type == 0 ? (T)P.dip_gradients[3 * it.idx + it.comp] : (T)0;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Table-driven FP64 build.  The interface entries repeat covariances: the
// interface-interface entry is a four-term difference over the rest and
// reference points of two rows, and the gradient-interface entry a difference
// over the rest and reference points of one row, while the reference points
// are shared by every row of a surface; the nine gradient-gradient entries
// of an orientation pair share one distance and two covariances.  Three
// tables hold each distinct value once -- C over every pair of surface points
// (n_sp x n_sp), C'/r (x_o - x_p)_u over every orientation-point pair
// (n_ori x n_sp x 3), and h, C'/r - C'', r^2 + 1e-5 and C'/r over every
// orientation pair (n_ori x n_ori x 6) -- and the entries are formed from them
// with the operations of entry_at, so K is the same matrix to rounding.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(256) point_cov_kernel(BuildParams P, T* __restrict__ Pc) {
    const int64_t a = (int64_t)blockIdx.y * 32 + threadIdx.y, b0 = (int64_t)blockIdx.x * 32;
    const Cov<T> cv = Cov<T>::make(P.kernel, P.range);
    const int64_t b = b0 + threadIdx.x;
    for (int k = 0; k < 4; ++k) {
        const int64_t aa = a + 8 * k;
        if (aa >= P.n_sp || b >= P.n_sp) continue;
        T x[3], y[3], h[3];
        for (int c = 0; c < 3; ++c) {
            x[c] = (T)P.sp_coords[3 * aa + c];
            y[c] = (T)P.sp_coords[3 * b + c];
        }
        Pc[aa * P.n_sp + b] = cv.C(dist(x, y, h));
    }
}

template <typename T>
__global__ void __launch_bounds__(256) ori_point_kernel(BuildParams P, T* __restrict__ Q) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)P.n_ori * P.n_sp) return;
    const int64_t o = t / P.n_sp, p = t - o * P.n_sp;
    const Cov<T> cv = Cov<T>::make(P.kernel, P.range);
    T x[3], y[3], h[3];
    for (int c = 0; c < 3; ++c) {
        x[c] = (T)P.dip_positions[3 * o + c];
        y[c] = (T)P.sp_coords[3 * p + c];
    }
    const T k1 = cv.d1_r(dist(x, y, h));
    for (int u = 0; u < 3; ++u) Q[3 * t + u] = k1 * h[u];
}

// per orientation pair (o, q): h = x_o - x_q, C'/r - C'', r^2 + 1e-5 and C'/r
template <typename T>
__global__ void __launch_bounds__(256) ori_pair_kernel(BuildParams P, T* __restrict__ G) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)P.n_ori * P.n_ori) return;
    const int64_t o = t / P.n_ori, q = t - o * P.n_ori;
    const Cov<T> cv = Cov<T>::make(P.kernel, P.range);
    T x[3], y[3], h[3];
    for (int c = 0; c < 3; ++c) {
        x[c] = (T)P.dip_positions[3 * o + c];
        y[c] = (T)P.dip_positions[3 * q + c];
    }
    const T r = dist(x, y, h);
    const T k1 = cv.d1_r(r), k2 = cv.d2(r);
    T* g = G + 6 * t;
    g[0] = h[0];
    g[1] = h[1];
    g[2] = h[2];
    g[3] = k1 - k2;
    g[4] = r * r + (T)kGradEps;
    g[5] = k1;
}

template <typename T>
__global__ void __launch_bounds__(256) build_table_kernel(BuildParams P, const T* __restrict__ Pc,
                                                          const T* __restrict__ Q, const T* __restrict__ G, T* K,
                                                          int64_t ldk, T* rhs) {
    __shared__ Item rows[32], cols[32];
    const int64_t r0 = (int64_t)blockIdx.y * 32, c0 = (int64_t)blockIdx.x * 32;
    const int tid = threadIdx.y * 32 + threadIdx.x;
    if (tid < 32) {
        if (r0 + tid < P.N) decode(P, r0 + tid, rows[tid]);
    } else if (tid < 64) {
        if (c0 + tid - 32 < P.N) decode(P, c0 + tid - 32, cols[tid - 32]);
    }
    __syncthreads();
    const Cov<T> cv = Cov<T>::make(P.kernel, P.range);
    const int64_t j = c0 + threadIdx.x;
    const T c_o = (T)P.c_o;
    for (int k = 0; k < 4; ++k) {
        const int rl = threadIdx.y + 8 * k;
        const int64_t i = r0 + rl;
        if (i >= P.N || j >= P.N) continue;
        const Item& A = rows[rl];
        const Item& B = cols[threadIdx.x];
        T v;
        if (A.type == 0 && B.type == 0) {
            const T* g = G + 6 * ((int64_t)A.idx * P.n_ori + B.idx);
            v = g[A.comp] * g[B.comp] * g[3] / g[4];
            if (A.comp == B.comp) v -= g[5];
            v *= c_o;
            if (i == j) v += (T)A.nug;
        } else if (A.type == 1 && B.type == 1) {
            const int64_t n = P.n_sp;
            v = Pc[A.rest * n + B.rest] - Pc[A.rest * n + B.ref] - Pc[A.ref * n + B.rest] + Pc[A.ref * n + B.ref];
            v *= (T)P.i_res * c_o;
            if (i == j) v += (T)A.nug;
        } else if (A.type == 0 && B.type == 1) {
            const T* q = Q + 3 * ((int64_t)A.idx * P.n_sp);
            v = (T)P.gi_res * c_o * (q[3 * B.rest + A.comp] - q[3 * B.ref + A.comp]);
        } else if (A.type == 1 && B.type == 0) {
            const T* q = Q + 3 * ((int64_t)B.idx * P.n_sp);
            v = (T)P.gi_res * c_o * (q[3 * A.rest + B.comp] - q[3 * A.ref + B.comp]);
        } else {
            v = entry<T>(P, cv, A, B, i == j);
        }
        K[i * ldk + j] = v;
    }
    if (rhs != nullptr && blockIdx.x == 0) {
        for (int k = 0; k < 4; ++k) {
            const int rl = threadIdx.y + 8 * k;
            const int64_t i = r0 + rl;
            if (threadIdx.x == 0 && i < P.N) {
                const Item& it = rows[rl];
                rhs[i] = it.type == 0 ? (T)P.dip_gradients[3 * it.idx + it.comp] : (T)0;
            }
        }
    }
}

static size_t table_bytes(const gk_system* s, size_t& q_off, size_t& g_off) {
    const size_t pc = (size_t)s->n_sp * s->n_sp * sizeof(double);
    q_off = (pc + 255) & ~(size_t)255;
    g_off = (q_off + (size_t)s->n_ori * s->n_sp * 3 * sizeof(double) + 255) & ~(size_t)255;
    return g_off + (size_t)s->n_ori * s->n_ori * 6 * sizeof(double);
}

}  // namespace gk

using namespace gk;

extern "C" int64_t gk_system_size(const gk_system* s) {
    if (s == nullptr) return -1;
    return 3 * (int64_t)s->n_ori + s->n_iface + drift_count(s->uni_degree) + s->n_fault;
}

static gk_status check_system(const gk_system* s) {
    if (s == nullptr) return GK_ERR_ARG;
    if (s->n_ori < 0 || s->n_sp < 0 || s->n_iface < 0 || s->n_iface > s->n_sp) return GK_ERR_ARG;
    if (s->uni_degree < 0 || s->uni_degree > 2) return GK_ERR_ARG;
    if (s->kernel != GK_KERNEL_CUBIC && s->kernel != GK_KERNEL_EXPONENTIAL) return GK_ERR_ARG;
    if (!(s->range > 0.0)) return GK_ERR_ARG;
    if (s->n_ori > 0 && (!s->dip_positions || !s->dip_gradients || !s->nugget_grad)) return GK_ERR_ARG;
    if (s->n_iface > 0 && (!s->sp_coords || !s->nugget_sp || !s->ref_index || !s->rest_index)) return GK_ERR_ARG;
    if (s->n_fault < 0) return GK_ERR_ARG;
    if (s->n_fault > GK_MAX_FAULTS) return GK_ERR_SIZE;
    if (s->n_fault > 0 && s->n_iface > 0 && !s->fault_sp) return GK_ERR_ARG;
    if (gk_system_size(s) <= 0) return GK_ERR_SIZE;
    return GK_OK;
}

gk_status gk_check_system(const gk_system* s) { return check_system(s); }

extern "C" gk_status gk_build(const gk_system* s, gk_prec prec, void* K, int64_t ldk, void* rhs, gk_stream stream) {
    gk_status st = check_system(s);
    if (st != GK_OK) return st;
    const int64_t N = gk_system_size(s);
    if (K == nullptr || ldk < N) return GK_ERR_ARG;
    if (N > (int64_t)1 << 20) return GK_ERR_SIZE;
    const BuildParams P = build_params(s);
    dim3 block(32, 8), grid((unsigned)((N + 31) / 32), (unsigned)((N + 31) / 32));
    cudaStream_t st_ = (cudaStream_t)stream;
    if (prec == GK_F64)
        build_kernel<double><<<grid, block, 0, st_>>>(P, (double*)K, ldk, (double*)rhs);
    else if (prec == GK_F32)
        build_kernel<float><<<grid, block, 0, st_>>>(P, (float*)K, ldk, (float*)rhs);
    else
        return GK_ERR_ARG;
    GK_LAUNCH_CHECK();
    return GK_OK;
}

extern "C" size_t gk_build_tables_bytes(const gk_system* s) {
    if (check_system(s) != GK_OK) return 0;
    size_t q_off = 0, g_off = 0;
    return table_bytes(s, q_off, g_off);
}

extern "C" gk_status gk_build_tables(const gk_system* s, double* K, int64_t ldk, double* rhs, void* work,
                                     size_t work_bytes, gk_stream stream) {
    gk_status st = check_system(s);
    if (st != GK_OK) return st;
    const int64_t N = gk_system_size(s);
    if (K == nullptr || ldk < N) return GK_ERR_ARG;
    if (N > (int64_t)1 << 20) return GK_ERR_SIZE;
    size_t q_off = 0, g_off = 0;
    const size_t need = table_bytes(s, q_off, g_off);
    if (work == nullptr || work_bytes < need || ((uintptr_t)work % 16) != 0) return GK_ERR_SIZE;
    const BuildParams P = build_params(s);
    cudaStream_t st_ = (cudaStream_t)stream;
    double* Pc = (double*)work;
    double* Q = (double*)((char*)work + q_off);
    double* G = (double*)((char*)work + g_off);
    const int64_t ng = (int64_t)s->n_ori * s->n_ori;
    if (ng > 0) {
        ori_pair_kernel<double><<<(unsigned)((ng + 255) / 256), 256, 0, st_>>>(P, G);
        GK_LAUNCH_CHECK();
    }
    if (s->n_sp > 0) {
        dim3 b2(32, 8), g2((unsigned)((s->n_sp + 31) / 32), (unsigned)((s->n_sp + 31) / 32));
        point_cov_kernel<double><<<g2, b2, 0, st_>>>(P, Pc);
        GK_LAUNCH_CHECK();
        const int64_t nq = (int64_t)s->n_ori * s->n_sp;
        if (nq > 0) {
            ori_point_kernel<double><<<(unsigned)((nq + 255) / 256), 256, 0, st_>>>(P, Q);
            GK_LAUNCH_CHECK();
        }
    }
    dim3 block(32, 8), grid((unsigned)((N + 31) / 32), (unsigned)((N + 31) / 32));
    build_table_kernel<double><<<grid, block, 0, st_>>>(P, Pc, Q, G, K, ldk, rhs);
    GK_LAUNCH_CHECK();
    return GK_OK;
}
