// Kriging-matrix entries of one series, shared by the single-system build
// (gk_build.cu) and the batched build (gk_batch.cu).
//
// Row/column ordering (shared with the Python host code and the oracle):
//   gradient unknowns component-major (u * n_ori + o), interface rows in the
//   order of ref_index/rest_index, then the drift functions
//   (x, y, z [, x^2, y^2, z^2, xy, xz, yz]), then one fault-drift unknown per
//   offsetting fault, whose function is that fault's block F_f (given at the
//   surface points): gi_res (F_f(rest) - F_f(ref)) on the interface rows, 0 on
//   the gradient rows (a block is piecewise constant) and in the drift block.
// Entry formulas restate the published co-kriging (GemPy 1.0, GMD 2019); the
// placement of i_res / gi_res, the nuggets inside the c_o factor and the 1e-5
// regulariser follow the conventions fitted to the reference's anticline
// approval file (test/test_model_types/test_example_models_I.py:41-53).
#pragma once

#include "gk_common.cuh"

namespace gk {

struct Item {          // one row/column of K, decoded
    int type;          // 0 = gradient, 1 = interface, 2 = drift, 3 = fault drift
    int comp;          // gradient component u, drift index d, or fault f
    int idx;           // orientation o, interface row t
    int rest, ref;     // surface-point indices (interface rows)
    double p[3];       // orientation position, or rest point
    double q[3];       // reference point (interface rows)
    double nug;        // diagonal nugget (already times c_o)
};

struct BuildParams {
    int n_ori, n_iface, n_drift, degree, kernel, n_fault;
    int64_t N;
    double range, c_o, i_res, gi_res;
    const double* dip_positions;
    const double* dip_gradients;
    const double* nugget_grad;
    const double* sp_coords;
    const double* nugget_sp;
    const int32_t* ref_index;
    const int32_t* rest_index;
    const double* fault_sp;   // n_fault x n_sp
    int n_sp;
};

// Build parameters of one series' system (N = 3 n_ori + n_iface + n_drift + n_fault).
inline BuildParams build_params(const gk_system* s) {
    BuildParams P;
    P.n_ori = s->n_ori; P.n_iface = s->n_iface; P.degree = s->uni_degree;
    P.n_drift = drift_count(s->uni_degree); P.kernel = s->kernel;
    P.N = 3 * (int64_t)s->n_ori + s->n_iface + P.n_drift + s->n_fault;
    P.range = s->range; P.c_o = s->c_o; P.i_res = s->i_res; P.gi_res = s->gi_res;
    P.dip_positions = s->dip_positions; P.dip_gradients = s->dip_gradients; P.nugget_grad = s->nugget_grad;
    P.sp_coords = s->sp_coords; P.nugget_sp = s->nugget_sp; P.ref_index = s->ref_index; P.rest_index = s->rest_index;
    P.n_fault = s->n_fault; P.fault_sp = s->fault_sp; P.n_sp = s->n_sp;
    return P;
}

__device__ inline void decode(const BuildParams& P, int64_t i, Item& it) {
    const int ng = 3 * P.n_ori;
    it.nug = 0.0;
    it.rest = it.ref = 0;
    if (i < ng) {
        it.type = 0;
        it.comp = (int)(i / P.n_ori);
        it.idx = (int)(i % P.n_ori);
        for (int k = 0; k < 3; ++k) it.p[k] = P.dip_positions[3 * it.idx + k];
        for (int k = 0; k < 3; ++k) it.q[k] = 0.0;
        it.nug = P.c_o * P.nugget_grad[it.idx];
    } else if (i < ng + P.n_iface) {
        it.type = 1;
        it.idx = (int)(i - ng);
        it.comp = 0;
        int rest = P.rest_index[it.idx], ref = P.ref_index[it.idx];
        it.rest = rest;
        it.ref = ref;
        for (int k = 0; k < 3; ++k) it.p[k] = P.sp_coords[3 * rest + k];
        for (int k = 0; k < 3; ++k) it.q[k] = P.sp_coords[3 * ref + k];
        it.nug = P.c_o * P.nugget_sp[rest];
    } else if (i < ng + P.n_iface + P.n_drift) {
        it.type = 2;
        it.comp = (int)(i - ng - P.n_iface);
        it.idx = it.comp;
        for (int k = 0; k < 3; ++k) { it.p[k] = 0.0; it.q[k] = 0.0; }
    } else {
        it.type = 3;
        it.comp = (int)(i - ng - P.n_iface - P.n_drift);
        it.idx = it.comp;
        for (int k = 0; k < 3; ++k) { it.p[k] = 0.0; it.q[k] = 0.0; }
    }
}

// f_d(x) and d f_d / d x_u
template <typename T>
__device__ inline T drift_f(int d, const T* x) {
    switch (d) {
        case 0: return x[0];
        case 1: return x[1];
        case 2: return x[2];
        case 3: return x[0] * x[0];
        case 4: return x[1] * x[1];
        case 5: return x[2] * x[2];
        case 6: return x[0] * x[1];
        case 7: return x[0] * x[2];
        default: return x[1] * x[2];
    }
}
template <typename T>
__device__ inline T drift_df(int d, int u, const T* x) {
    switch (d) {
        case 0: case 1: case 2: return (T)(d == u ? 1 : 0);
        case 3: case 4: case 5: return d - 3 == u ? (T)2 * x[u] : (T)0;
        case 6: return u == 0 ? x[1] : (u == 1 ? x[0] : (T)0);
        case 7: return u == 0 ? x[2] : (u == 2 ? x[0] : (T)0);
        default: return u == 1 ? x[2] : (u == 2 ? x[1] : (T)0);
    }
}

template <typename T>
__device__ inline T dist(const T* a, const T* b, T* h) {
    h[0] = a[0] - b[0];
    h[1] = a[1] - b[1];
    h[2] = a[2] - b[2];
    return gsqrt<T>(h[0] * h[0] + h[1] * h[1] + h[2] * h[2] + (T)kDistEps2);
}

// K(A, B) with the items' positions given in T (the adjoint evaluates it on
// dual numbers seeded on A's positions).
template <typename T>
__device__ T entry_at(const BuildParams& P, const Cov<T>& cv, const Item& A, const Item& B, bool diag,
                      const T* ap, const T* aq, const T* bp, const T* bq) {
    const T c_o = (T)P.c_o;
    T h[3], g[3];
    if (A.type == 0 && B.type == 0) {
        T r = dist(ap, bp, h);
        T k1 = cv.d1_r(r), k2 = cv.d2(r);
        T v = h[A.comp] * h[B.comp] * (k1 - k2) / (r * r + (T)kGradEps);
        if (A.comp == B.comp) v -= k1;
        v *= c_o;
        if (diag) v += (T)A.nug;
        return v;
    }
    if (A.type == 0 && B.type == 1) {
        T rr = dist(ap, bp, h);
        T rf = dist(ap, bq, g);
        return (T)P.gi_res * c_o * (cv.d1_r(rr) * h[A.comp] - cv.d1_r(rf) * g[A.comp]);
    }
    if (A.type == 1 && B.type == 0) {
        T rr = dist(bp, ap, h);
        T rf = dist(bp, aq, g);
        return (T)P.gi_res * c_o * (cv.d1_r(rr) * h[B.comp] - cv.d1_r(rf) * g[B.comp]);
    }
    if (A.type == 1 && B.type == 1) {
        T v = cv.C(dist(ap, bp, h)) - cv.C(dist(ap, bq, h)) - cv.C(dist(aq, bp, h)) + cv.C(dist(aq, bq, h));
        v *= (T)P.i_res * c_o;
        if (diag) v += (T)A.nug;
        return v;
    }
    if (A.type == 0 && B.type == 2) return drift_df<T>(B.comp, A.comp, ap);
    if (A.type == 2 && B.type == 0) return drift_df<T>(A.comp, B.comp, bp);
    if (A.type == 1 && B.type == 2) return (T)P.gi_res * (drift_f<T>(B.comp, ap) - drift_f<T>(B.comp, aq));
    if (A.type == 2 && B.type == 1) return (T)P.gi_res * (drift_f<T>(A.comp, bp) - drift_f<T>(A.comp, bq));
    if (A.type == 1 && B.type == 3) {
        const double* F = P.fault_sp + (int64_t)B.comp * P.n_sp;
        return (T)(P.gi_res * (F[A.rest] - F[A.ref]));
    }
    if (A.type == 3 && B.type == 1) {
        const double* F = P.fault_sp + (int64_t)A.comp * P.n_sp;
        return (T)(P.gi_res * (F[B.rest] - F[B.ref]));
    }
    return (T)0;
}

template <typename T>
__device__ T entry(const BuildParams& P, const Cov<T>& cv, const Item& A, const Item& B, bool diag) {
    T ap[3] = {(T)A.p[0], (T)A.p[1], (T)A.p[2]};
    T aq[3] = {(T)A.q[0], (T)A.q[1], (T)A.q[2]};
    T bp[3] = {(T)B.p[0], (T)B.p[1], (T)B.p[2]};
    T bq[3] = {(T)B.q[0], (T)B.q[1], (T)B.q[2]};
    return entry_at<T>(P, cv, A, B, diag, ap, aq, bp, bq);
}

}  // namespace gk
