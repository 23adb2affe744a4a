// Adjoint (reverse-mode) derivatives of the interpolation, for
//   J = sum_x g(x) Z(x),   Z(x) = sum_i w_i e_i(x),   K w = b,
// the gradients the reference's PyTorch tape provides through compute_model
// (checked against central differences at
// test/test_modules/test_ad/test_ad_I.py:158-258, used by the nugget optimiser
// gempy/modules/optimize_nuggets/_optimizer.py:9-62):
//   r = sum_x g(x) e(x)                                  gk_adjoint_rhs
//   K lambda = r        (K is symmetric: the forward solve's factors serve)
//   dJ/dtheta = sum_x g(x) dZ(x)/dtheta |_w              gk_eval_adjoint
//             - lambda^T (dK/dtheta) w                   gk_build_adjoint
//             + lambda^T (db/dtheta)   (b's gradient rows are the dip gradients)
// theta: surface-point and orientation positions, both nugget kinds.  The
// fault-drift functions (other series' blocks) are held constant.
//
// dK/d(positions) comes from the build's own entry formulas (entry_at)
// evaluated on dual numbers seeded on the row item's positions.  With K
// symmetric, sum_ij lambda_i w_j dK_ij = sum_ij (lambda_i w_j + lambda_j w_i)
// d_A K_ij, d_A the derivative with respect to the row item's positions only
// (K_ij as a function of the two items is symmetric), so one warp per row
// covers the whole sum with 6 dual directions (the item's p and q).
#include <cstring>

#include "gk_kriging.cuh"

namespace gk {

// Value and M directional derivatives.
template <int M>
struct Dual {
    double v, d[M];
    __host__ __device__ Dual() {}
    __host__ __device__ Dual(double x) : v(x) {
        for (int k = 0; k < M; ++k) d[k] = 0.0;
    }
};
template <int M> __device__ __forceinline__ Dual<M> operator+(Dual<M> a, const Dual<M>& b) {
    a.v += b.v;
    for (int k = 0; k < M; ++k) a.d[k] += b.d[k];
    return a;
}
template <int M> __device__ __forceinline__ Dual<M> operator-(Dual<M> a, const Dual<M>& b) {
    a.v -= b.v;
    for (int k = 0; k < M; ++k) a.d[k] -= b.d[k];
    return a;
}
template <int M> __device__ __forceinline__ Dual<M> operator-(Dual<M> a) {
    a.v = -a.v;
    for (int k = 0; k < M; ++k) a.d[k] = -a.d[k];
    return a;
}
template <int M> __device__ __forceinline__ Dual<M> operator*(const Dual<M>& a, const Dual<M>& b) {
    Dual<M> c;
    c.v = a.v * b.v;
    for (int k = 0; k < M; ++k) c.d[k] = a.v * b.d[k] + a.d[k] * b.v;
    return c;
}
template <int M> __device__ __forceinline__ Dual<M> operator/(const Dual<M>& a, const Dual<M>& b) {
    Dual<M> c;
    const double ib = 1.0 / b.v;
    c.v = a.v * ib;
    for (int k = 0; k < M; ++k) c.d[k] = (a.d[k] - c.v * b.d[k]) * ib;
    return c;
}
template <int M> __device__ __forceinline__ Dual<M>& operator+=(Dual<M>& a, const Dual<M>& b) { return a = a + b; }
template <int M> __device__ __forceinline__ Dual<M>& operator-=(Dual<M>& a, const Dual<M>& b) { return a = a - b; }
template <int M> __device__ __forceinline__ Dual<M>& operator*=(Dual<M>& a, const Dual<M>& b) { return a = a * b; }
template <int M> __device__ __forceinline__ bool operator<(const Dual<M>& a, const Dual<M>& b) { return a.v < b.v; }
template <int M> __device__ __forceinline__ bool operator>(const Dual<M>& a, const Dual<M>& b) { return a.v > b.v; }
template <int M> __device__ __forceinline__ bool operator<=(const Dual<M>& a, const Dual<M>& b) { return a.v <= b.v; }
template <int M> __device__ __forceinline__ bool operator>=(const Dual<M>& a, const Dual<M>& b) { return a.v >= b.v; }

using D6 = Dual<6>;

template <>
__device__ __forceinline__ D6 gsqrt<D6>(D6 x) {
    D6 y;
    y.v = sqrt(x.v);
    const double h = 0.5 / y.v;   // x.v >= the distance regulariser > 0
    for (int k = 0; k < 6; ++k) y.d[k] = x.d[k] * h;
    return y;
}
template <>
__device__ __forceinline__ D6 Cov<D6>::gexp(D6 x) {
    D6 y;
    y.v = exp(x.v);
    for (int k = 0; k < 6; ++k) y.d[k] = x.d[k] * y.v;
    return y;
}

// -lambda^T (dK/dtheta) w: warp per row item A; lanes over the columns.
__global__ void __launch_bounds__(256) build_adjoint_kernel(const BuildParams P, const double* __restrict__ lam,
                                                            const double* __restrict__ w, double* d_sp,
                                                            double* d_dip, double* d_nug_sp, double* d_nug_grad) {
    const int lane = threadIdx.x & 31;
    const int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (i >= P.N) return;
    Item A;
    decode(P, i, A);
    if (A.type >= 2) return;   // drift and fault-drift items have no position
    const Cov<D6> cv = Cov<D6>::make(P.kernel, P.range);
    D6 ap[3], aq[3];
    for (int k = 0; k < 3; ++k) {
        ap[k] = D6(A.p[k]);
        aq[k] = D6(A.q[k]);
        ap[k].d[k] = 1.0;
        aq[k].d[3 + k] = 1.0;
    }
    double acc[6] = {0, 0, 0, 0, 0, 0};
    const double li = lam[i], wi = w[i];
    for (int64_t j = lane; j < P.N; j += 32) {
        Item B;
        decode(P, j, B);
        const double c = li * w[j] + lam[j] * wi;
        if (c == 0.0) continue;
        D6 bp[3], bq[3];
        for (int k = 0; k < 3; ++k) {
            bp[k] = D6(B.p[k]);
            bq[k] = D6(B.q[k]);
        }
        const D6 e = entry_at<D6>(P, cv, A, B, i == j, ap, aq, bp, bq);
        for (int k = 0; k < 6; ++k) acc[k] += c * e.d[k];
    }
    for (int k = 0; k < 6; ++k)
        for (int o = 16; o > 0; o >>= 1) acc[k] += __shfl_down_sync(0xffffffffu, acc[k], o);
    if (lane != 0) return;
    if (A.type == 0) {
        for (int k = 0; k < 3; ++k) atomicAdd(d_dip + 3 * A.idx + k, -acc[k]);
        if (d_nug_grad) atomicAdd(d_nug_grad + A.idx, -P.c_o * li * wi);
    } else {
        for (int k = 0; k < 3; ++k) {
            atomicAdd(d_sp + 3 * A.rest + k, -acc[k]);
            atomicAdd(d_sp + 3 * A.ref + k, -acc[3 + k]);
        }
        if (d_nug_sp) atomicAdd(d_nug_sp + A.rest, -P.c_o * li * wi);
    }
}

struct AdjPoints {
    int kind;
    int dims[3];
    int64_t n;
    double origin[3], spacing[3];
    const double* xyz;
    const double* fault_values;
    int64_t fault_ld;
};

__device__ __forceinline__ void adj_point(const AdjPoints& Q, int64_t q, double* x) {
    if (Q.kind == 0) {
        const int64_t nyz = (int64_t)Q.dims[1] * Q.dims[2];
        const int64_t ix = q / nyz, rem = q - ix * nyz;
        const int64_t iy = rem / Q.dims[2], iz = rem - iy * Q.dims[2];
        x[0] = Q.origin[0] + (double)ix * Q.spacing[0];
        x[1] = Q.origin[1] + (double)iy * Q.spacing[1];
        x[2] = Q.origin[2] + (double)iz * Q.spacing[2];
    } else {
        x[0] = Q.xyz[3 * q];
        x[1] = Q.xyz[3 * q + 1];
        x[2] = Q.xyz[3 * q + 2];
    }
}

constexpr int kAdjTile = 256;

// r_i = sum_x g(x) e_i(x): thread per unknown, points staged in shared memory.
__global__ void __launch_bounds__(kAdjTile) adjoint_rhs_kernel(const BuildParams P, const AdjPoints Q,
                                                               const double* __restrict__ g, double* r) {
    __shared__ double sx[kAdjTile][3], sg[kAdjTile];
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    Item A;
    if (i < P.N) decode(P, i, A);
    const Cov<double> cv = Cov<double>::make(P.kernel, P.range);
    const double sc = P.c_o * P.gi_res;
    double acc = 0.0;
    for (int64_t q0 = 0; q0 < Q.n; q0 += kAdjTile) {
        const int64_t q = q0 + threadIdx.x;
        if (q < Q.n) {
            double x[3];
            adj_point(Q, q, x);
            sx[threadIdx.x][0] = x[0];
            sx[threadIdx.x][1] = x[1];
            sx[threadIdx.x][2] = x[2];
            sg[threadIdx.x] = g[q];
        }
        __syncthreads();
        const int nq = (int)min((int64_t)kAdjTile, Q.n - q0);
        if (i < P.N) {
            for (int t = 0; t < nq; ++t) {
                const double gx = sg[t];
                if (gx == 0.0) continue;
                const double* x = sx[t];
                double h[3], e;
                if (A.type == 0) {
                    const double rr = dist<double>(A.p, x, h);   // h = x_o - x
                    e = sc * cv.d1_r(rr) * h[A.comp];
                } else if (A.type == 1) {
                    // the evaluation's point weights carry gi_res once more (alpha = gi_res sum w)
                    double h2[3];
                    e = sc * P.gi_res * (cv.C(dist<double>(x, A.p, h)) - cv.C(dist<double>(x, A.q, h2)));
                } else if (A.type == 2) {
                    e = P.gi_res * drift_f<double>(A.comp, x);
                } else {
                    e = P.gi_res * Q.fault_values[(int64_t)A.comp * Q.fault_ld + q0 + t];
                }
                acc += gx * e;
            }
        }
        __syncthreads();
    }
    if (i < P.N) r[i] = acc;
}

// sum_x g(x) dZ(x)/d(record position) at fixed weights, from the packed
// records (orientation: x_o and c_o gi_res w_o; surface point: x_p and
// c_o gi_res alpha_p); thread per record, added into d_dip / d_sp.
__global__ void __launch_bounds__(kAdjTile) eval_adjoint_kernel(int n_ori, int n_sp, int kernel, double range,
                                                                const double* __restrict__ ori64,
                                                                const double* __restrict__ sp64, const AdjPoints Q,
                                                                const double* __restrict__ g, double* d_dip,
                                                                double* d_sp) {
    __shared__ double sx[kAdjTile][3], sg[kAdjTile];
    const int64_t rix = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool is_ori = rix < n_ori, live = rix < (int64_t)n_ori + n_sp;
    const Cov<double> cv = Cov<double>::make(kernel, range);
    double rp[3] = {0, 0, 0}, rw[3] = {0, 0, 0}, al = 0.0;
    if (live) {
        if (is_ori) {
            const double* R = ori64 + 8 * rix;
            for (int k = 0; k < 3; ++k) { rp[k] = R[k]; rw[k] = R[3 + k]; }
        } else {
            const double* R = sp64 + 4 * (rix - n_ori);
            for (int k = 0; k < 3; ++k) rp[k] = R[k];
            al = R[3];
        }
    }
    double acc[3] = {0, 0, 0};
    for (int64_t q0 = 0; q0 < Q.n; q0 += kAdjTile) {
        const int64_t q = q0 + threadIdx.x;
        if (q < Q.n) {
            double x[3];
            adj_point(Q, q, x);
            sx[threadIdx.x][0] = x[0];
            sx[threadIdx.x][1] = x[1];
            sx[threadIdx.x][2] = x[2];
            sg[threadIdx.x] = g[q];
        }
        __syncthreads();
        const int nq = (int)min((int64_t)kAdjTile, Q.n - q0);
        if (live) {
            for (int t = 0; t < nq; ++t) {
                const double gx = sg[t];
                if (gx == 0.0) continue;
                double h[3];
                const double r = dist<double>(rp, sx[t], h);   // h = record - x
                if (is_ori) {
                    // d/dx_o [C'/r(r) (w . h)] = (C'/r)'/r (w . h) h + C'/r w
                    const double k1 = cv.d1_r(r), k3 = cv.d3_r(r);
                    const double wh = rw[0] * h[0] + rw[1] * h[1] + rw[2] * h[2];
                    for (int k = 0; k < 3; ++k) acc[k] += gx * (k3 * wh * h[k] + k1 * rw[k]);
                } else {
                    // d/dx_p [alpha C(r)] = alpha C'/r (x_p - x)
                    const double k1 = al * cv.d1_r(r);
                    for (int k = 0; k < 3; ++k) acc[k] += gx * k1 * h[k];
                }
            }
        }
        __syncthreads();
    }
    if (!live) return;
    double* out = is_ori ? d_dip + 3 * rix : d_sp + 3 * (rix - n_ori);
    for (int k = 0; k < 3; ++k) out[k] += acc[k];
}

}  // namespace gk

using namespace gk;

gk_status gk_check_system(const gk_system* s);
void gk_eval_model_records(const gk_system* s, const void* model, const double** ori64, const double** sp64);

static gk_status adj_points(const gk_system* s, const gk_points* p, AdjPoints& Q) {
    if (p == nullptr || p->n < 0) return GK_ERR_ARG;
    memset(&Q, 0, sizeof(Q));
    Q.kind = p->kind;
    Q.n = p->n;
    for (int k = 0; k < 3; ++k) {
        Q.dims[k] = p->dims[k];
        Q.origin[k] = p->origin[k];
        Q.spacing[k] = p->spacing[k];
    }
    Q.xyz = p->xyz;
    Q.fault_values = p->fault_values;
    Q.fault_ld = p->fault_ld;
    if (p->kind == 0) {
        if ((int64_t)p->dims[0] * p->dims[1] * p->dims[2] != p->n) return GK_ERR_ARG;
    } else if (p->kind != 1 || (p->n > 0 && p->xyz == nullptr)) {
        return GK_ERR_ARG;
    }
    if (s->n_fault > 0 && p->n > 0 && (p->fault_values == nullptr || p->fault_ld < p->n)) return GK_ERR_ARG;
    return GK_OK;
}

extern "C" gk_status gk_adjoint_rhs(const gk_system* s, const gk_points* pts, const double* g, double* r,
                                    gk_stream stream) {
    gk_status st = gk_check_system(s);
    if (st != GK_OK) return st;
    AdjPoints Q;
    if ((st = adj_points(s, pts, Q)) != GK_OK) return st;
    if (r == nullptr || (Q.n > 0 && g == nullptr)) return GK_ERR_ARG;
    const BuildParams P = build_params(s);
    adjoint_rhs_kernel<<<(unsigned)((P.N + kAdjTile - 1) / kAdjTile), kAdjTile, 0, (cudaStream_t)stream>>>(P, Q, g,
                                                                                                         r);
    GK_LAUNCH_CHECK();
    return GK_OK;
}

extern "C" gk_status gk_build_adjoint(const gk_system* s, const double* lam, const double* w, double* d_sp,
                                      double* d_dip, double* d_nug_sp, double* d_nug_grad, gk_stream stream) {
    gk_status st = gk_check_system(s);
    if (st != GK_OK) return st;
    if (lam == nullptr || w == nullptr || (s->n_sp > 0 && d_sp == nullptr) || (s->n_ori > 0 && d_dip == nullptr))
        return GK_ERR_ARG;
    cudaStream_t cs = (cudaStream_t)stream;
    if (s->n_sp > 0) GK_CUDA_TRY(cudaMemsetAsync(d_sp, 0, (size_t)s->n_sp * 3 * sizeof(double), cs));
    if (s->n_ori > 0) GK_CUDA_TRY(cudaMemsetAsync(d_dip, 0, (size_t)s->n_ori * 3 * sizeof(double), cs));
    if (d_nug_sp && s->n_sp > 0) GK_CUDA_TRY(cudaMemsetAsync(d_nug_sp, 0, (size_t)s->n_sp * sizeof(double), cs));
    if (d_nug_grad && s->n_ori > 0)
        GK_CUDA_TRY(cudaMemsetAsync(d_nug_grad, 0, (size_t)s->n_ori * sizeof(double), cs));
    const BuildParams P = build_params(s);
    const int64_t threads = P.N * 32;
    build_adjoint_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, cs>>>(P, lam, w, d_sp, d_dip, d_nug_sp,
                                                                            d_nug_grad);
    GK_LAUNCH_CHECK();
    return GK_OK;
}

extern "C" gk_status gk_eval_adjoint(const gk_system* s, const void* model, const gk_points* pts, const double* g,
                                     double* d_sp, double* d_dip, gk_stream stream) {
    gk_status st = gk_check_system(s);
    if (st != GK_OK) return st;
    AdjPoints Q;
    if ((st = adj_points(s, pts, Q)) != GK_OK) return st;
    if (model == nullptr || (Q.n > 0 && g == nullptr) || (s->n_sp > 0 && d_sp == nullptr) ||
        (s->n_ori > 0 && d_dip == nullptr))
        return GK_ERR_ARG;
    const double *ori64, *sp64;
    gk_eval_model_records(s, model, &ori64, &sp64);
    const int64_t n_rec = (int64_t)s->n_ori + s->n_sp;
    if (n_rec == 0 || Q.n == 0) return GK_OK;
    eval_adjoint_kernel<<<(unsigned)((n_rec + kAdjTile - 1) / kAdjTile), kAdjTile, 0, (cudaStream_t)stream>>>(
        s->n_ori, s->n_sp, s->kernel, s->range, ori64, sp64, Q, g, d_dip, d_sp);
    GK_LAUNCH_CHECK();
    return GK_OK;
}
