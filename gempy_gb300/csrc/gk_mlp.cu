// The learned part of the solver: a 3-layer perceptron (in_dim -> 256 -> 256
// -> out_dim, ReLU between layers) with BF16 weights and FP32 accumulation,
// trained on the GPU by the forward, backward and AdamW kernels below.  It
// maps a kriging system's geometry descriptor plus one candidate
// preconditioner configuration to the predicted cost of solving the system
// with that configuration; the host picks the cheapest candidate.  The
// reference has no counterpart (its solver is the dense FP64 LU).
//
// Parameter layout (BF16 bit patterns, one contiguous array): for each layer
// l with k_l inputs and n_l outputs a row-major n_l x (k_l + 1) matrix whose
// last column is the bias, layers in order.  Every product below treats the
// layer input as augmented with a trailing column of ones, so the bias is
// just one more weight column in the forward product and one more column of
// the weight gradient.
//
// All three products (forward X W^T, backward dZ W and weight gradient
// dZ^T X) run through one 64 x 64-tile shared-memory kernel (FP32 FMA on
// operands converted from BF16 on load).  The network is small (75k weights);
// a training batch is a few thousand samples, so it is latency- not
// throughput-bound and the tensor pipe would buy nothing.  The weight gradient
// is split over fixed sample chunks and the chunks are summed in a fixed
// order, so gradients are bitwise reproducible.
#include <cuda_bf16.h>

#include "gk_common.cuh"

namespace gk {
namespace mlp {

constexpr int kHidden = GK_MLP_HIDDEN;
constexpr int kTile = 64, kBK = 16, kThreads = 256;
constexpr int kMaxChunks = 32;

__host__ __device__ inline int64_t layer_in(int l, int in_dim) { return l == 0 ? in_dim : kHidden; }
__host__ __device__ inline int64_t layer_out(int l, int out_dim) { return l == 2 ? out_dim : kHidden; }
__host__ __device__ inline int64_t layer_params(int l, int in_dim, int out_dim) {
    return layer_out(l, out_dim) * (layer_in(l, in_dim) + 1);
}
__host__ __device__ inline int64_t layer_offset(int l, int in_dim, int out_dim) {
    int64_t o = 0;
    for (int i = 0; i < l; ++i) o += layer_params(i, in_dim, out_dim);
    return o;
}

inline int chunks_for(int64_t batch) {
    int64_t c = (batch + 511) / 512;
    return (int)(c < 1 ? 1 : (c > kMaxChunks ? kMaxChunks : c));
}

// Workspace: H1, H2 (saved activations), D1, D2 (gradient scratch), each
// batch x 256 FP32, then the chunked weight-gradient partials.
struct Work {
    float *h1, *h2, *d1, *d2, *part;
};

inline size_t work_bytes(int in_dim, int out_dim, int64_t batch) {
    int64_t big = layer_params(1, in_dim, out_dim);
    int64_t l0 = layer_params(0, in_dim, out_dim);
    if (l0 > big) big = l0;
    return sizeof(float) * (size_t)(4 * batch * kHidden + (int64_t)kMaxChunks * big);
}

inline Work carve(void* w, int64_t batch) {
    Work k;
    float* p = (float*)w;
    k.h1 = p; p += batch * kHidden;
    k.h2 = p; p += batch * kHidden;
    k.d1 = p; p += batch * kHidden;
    k.d2 = p; p += batch * kHidden;
    k.part = p;
    return k;
}

__device__ __forceinline__ float bf(const __nv_bfloat16* p, int64_t i) { return __bfloat162float(p[i]); }

// ---- operand accessors: at(row, k) of an (rows x depth) A or (depth x cols) B.
// kDepthContig says whether consecutive threads should walk the depth index
// (true) or the row/column index (false) for coalesced loads.

struct XAugA {  // A(m, k) = X[m][k] for k < K, 1 at k == K  (X row-major, ld)
    const float* p; int64_t ld, K;
    static constexpr bool kDepthContig = true;
    __device__ float at(int64_t m, int64_t k) const { return k < K ? p[m * ld + k] : 1.f; }
};
struct RowA {  // A(m, k) = P[m][k]
    const float* p; int64_t ld;
    static constexpr bool kDepthContig = true;
    __device__ float at(int64_t m, int64_t k) const { return p[m * ld + k]; }
};
struct TransA {  // A(n, m) = P[m][n]   (weight gradient: dZ^T)
    const float* p; int64_t ld;
    static constexpr bool kDepthContig = false;
    __device__ float at(int64_t n, int64_t m) const { return p[m * ld + n]; }
};
struct WeightKB {  // B(k, n) = W[n][k]   (forward: X W^T)
    const __nv_bfloat16* p; int64_t ld;
    static constexpr bool kDepthContig = true;
    __device__ float at(int64_t k, int64_t n) const { return bf(p, n * ld + k); }
};
struct WeightNB {  // B(n, j) = W[n][j]   (backward: dZ W)
    const __nv_bfloat16* p; int64_t ld;
    static constexpr bool kDepthContig = false;
    __device__ float at(int64_t n, int64_t j) const { return bf(p, n * ld + j); }
};
struct XAugB {  // B(m, j) = X[m][j] for j < K, 1 at j == K   (weight gradient)
    const float* p; int64_t ld, K;
    static constexpr bool kDepthContig = false;
    __device__ float at(int64_t m, int64_t j) const { return j < K ? p[m * ld + j] : 1.f; }
};

// ---- epilogues
struct EpiAct {  // out[i][j] = relu?(acc)
    float* out; int64_t ld; bool relu;
    __device__ void operator()(int64_t i, int64_t j, int, float acc) const {
        out[i * ld + j] = relu ? fmaxf(acc, 0.f) : acc;
    }
};
struct EpiMask {  // out[i][j] = acc where the layer's post-ReLU activation h > 0
    float* out; const float* h; int64_t ld;
    __device__ void operator()(int64_t i, int64_t j, int, float acc) const {
        out[i * ld + j] = h[i * ld + j] > 0.f ? acc : 0.f;
    }
};
struct EpiPart {  // part[z][i][j] = acc
    float* part; int64_t rows, cols;
    __device__ void operator()(int64_t i, int64_t j, int z, float acc) const {
        part[((int64_t)z * rows + i) * cols + j] = acc;
    }
};

// C[i][j] = sum_{k in chunk z} A(i, k) B(k, j), i < rows, j < cols; depth
// chunk z covers [z * chunk, min(depth, (z + 1) * chunk)).
template <class TA, class TB, class Epi>
__global__ void __launch_bounds__(kThreads) gemm_kernel(int64_t rows, int64_t cols, int64_t depth, int64_t chunk,
                                                        TA A, TB B, Epi epi) {
    __shared__ __align__(16) float As[kBK][kTile + 4];
    __shared__ __align__(16) float Bs[kBK][kTile + 4];
    const int t = threadIdx.x, tx = t % 16, ty = t / 16;
    const int64_t i0 = (int64_t)blockIdx.y * kTile, j0 = (int64_t)blockIdx.x * kTile;
    const int z = blockIdx.z;
    const int64_t k_lo = (int64_t)z * chunk;
    const int64_t k_hi = min(depth, k_lo + chunk);
    float acc[4][4] = {};
    for (int64_t k0 = k_lo; k0 < k_hi; k0 += kBK) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int e = t + kThreads * q;
            int ii, kk;
            if (TA::kDepthContig) { ii = e / kBK; kk = e % kBK; } else { kk = e / kTile; ii = e % kTile; }
            const int64_t gi = i0 + ii, gk = k0 + kk;
            As[kk][ii] = (gi < rows && gk < k_hi) ? A.at(gi, gk) : 0.f;
            int jj;
            if (TB::kDepthContig) { jj = e / kBK; kk = e % kBK; } else { kk = e / kTile; jj = e % kTile; }
            const int64_t gj = j0 + jj, gk2 = k0 + kk;
            Bs[kk][jj] = (gj < cols && gk2 < k_hi) ? B.at(gk2, gj) : 0.f;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < kBK; ++kk) {
            const float4 a = *reinterpret_cast<const float4*>(&As[kk][ty * 4]);
            const float4 b = *reinterpret_cast<const float4*>(&Bs[kk][tx * 4]);
            const float av[4] = {a.x, a.y, a.z, a.w}, bv[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
            for (int r = 0; r < 4; ++r)
#pragma unroll
                for (int c = 0; c < 4; ++c) acc[r][c] = fmaf(av[r], bv[c], acc[r][c]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const int64_t i = i0 + ty * 4 + r, j = j0 + tx * 4 + c;
            if (i < rows && j < cols) epi(i, j, z, acc[r][c]);
        }
}

template <class TA, class TB, class Epi>
gk_status gemm(int64_t rows, int64_t cols, int64_t depth, int chunks, TA A, TB B, Epi epi, cudaStream_t s) {
    const int64_t chunk = (depth + chunks - 1) / chunks;
    dim3 grid((unsigned)((cols + kTile - 1) / kTile), (unsigned)((rows + kTile - 1) / kTile), (unsigned)chunks);
    gemm_kernel<TA, TB, Epi><<<grid, kThreads, 0, s>>>(rows, cols, depth, chunk, A, B, epi);
    GK_LAUNCH_CHECK();
    return GK_OK;
}

// grad[p] = sum_z part[z][p], z ascending.
__global__ void reduce_chunks_kernel(const float* part, int chunks, int64_t n, float* grad) {
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
        float s = 0.f;
        for (int z = 0; z < chunks; ++z) s += part[(int64_t)z * n + p];
        grad[p] = s;
    }
}

// Weighted mean-squared error over the batch and its gradient:
//   loss = sum_i w_i sum_o (y_io - t_io)^2 / sum_i w_i,  dy = dloss/dy.
// One CTA, fixed-order tree reductions: deterministic.
__global__ void __launch_bounds__(1024) mse_kernel(int64_t batch, int out_dim, const float* y, const float* t,
                                                   const float* w, float* dy, float* loss) {
    __shared__ float red[1024];
    float ws = 0.f;
    for (int64_t i = threadIdx.x; i < batch; i += blockDim.x) ws += w ? w[i] : 1.f;
    red[threadIdx.x] = ws;
    __syncthreads();
    for (int s = 512; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    const float W = red[0];
    __syncthreads();
    const float inv = W > 0.f ? 1.f / W : 0.f;
    float ls = 0.f;
    const int64_t n = batch * out_dim;
    for (int64_t e = threadIdx.x; e < n; e += blockDim.x) {
        const int64_t i = e / out_dim;
        const float wi = w ? w[i] : 1.f;
        const float d = y[e] - t[e];
        ls += wi * d * d;
        if (dy) dy[e] = 2.f * wi * d * inv;
    }
    red[threadIdx.x] = ls;
    __syncthreads();
    for (int s = 512; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0 && loss) *loss = red[0] * inv;
}

// AdamW on the FP32 master copy; the BF16 copy the kernels read is the
// round-to-nearest-even image of the updated master.
__global__ void adam_kernel(int64_t n, float* master, __nv_bfloat16* params, const float* grad, float* m, float* v,
                            gk_adam hp, float c1, float c2) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float g = grad[i];
        const float mi = hp.beta1 * m[i] + (1.f - hp.beta1) * g;
        const float vi = hp.beta2 * v[i] + (1.f - hp.beta2) * g * g;
        m[i] = mi;
        v[i] = vi;
        const float mh = mi / c1, vh = vi / c2;
        float th = master[i];
        th -= hp.lr * (mh / (sqrtf(vh) + hp.eps) + hp.weight_decay * th);
        master[i] = th;
        params[i] = __float2bfloat16_rn(th);
    }
}

gk_status check_net(const gk_mlp* net) {
    if (net == nullptr || net->params == nullptr) return GK_ERR_ARG;
    if (net->in_dim < 1 || net->in_dim > GK_MLP_MAX_IN) return GK_ERR_ARG;
    if (net->out_dim < 1 || net->out_dim > GK_MLP_MAX_OUT) return GK_ERR_ARG;
    return GK_OK;
}

}  // namespace mlp
}  // namespace gk

using namespace gk;
using namespace gk::mlp;

extern "C" int64_t gk_mlp_param_count(int32_t in_dim, int32_t out_dim) {
    if (in_dim < 1 || in_dim > GK_MLP_MAX_IN || out_dim < 1 || out_dim > GK_MLP_MAX_OUT) return -1;
    return layer_offset(3, in_dim, out_dim);
}

extern "C" size_t gk_mlp_workspace_bytes(int32_t in_dim, int32_t out_dim, int64_t batch) {
    if (in_dim < 1 || in_dim > GK_MLP_MAX_IN || out_dim < 1 || out_dim > GK_MLP_MAX_OUT || batch < 1 ||
        batch > GK_MLP_MAX_BATCH)
        return 0;
    return work_bytes(in_dim, out_dim, batch);
}

extern "C" gk_status gk_mlp_fwd(const gk_mlp* net, int64_t batch, const float* x, float* y, void* work,
                                size_t work_bytes_, gk_stream stream) {
    gk_status st = check_net(net);
    if (st != GK_OK) return st;
    if (batch < 1 || x == nullptr || y == nullptr || work == nullptr) return GK_ERR_ARG;
    if (batch > GK_MLP_MAX_BATCH) return GK_ERR_SIZE;
    if (work_bytes_ < work_bytes(net->in_dim, net->out_dim, batch)) return GK_ERR_SIZE;
    cudaStream_t s = (cudaStream_t)stream;
    const int F = net->in_dim, O = net->out_dim;
    const __nv_bfloat16* P = reinterpret_cast<const __nv_bfloat16*>(net->params);
    Work w = carve(work, batch);
    const __nv_bfloat16* W0 = P + layer_offset(0, F, O);
    const __nv_bfloat16* W1 = P + layer_offset(1, F, O);
    const __nv_bfloat16* W2 = P + layer_offset(2, F, O);
    if ((st = gemm(batch, kHidden, F + 1, 1, XAugA{x, F, F}, WeightKB{W0, F + 1}, EpiAct{w.h1, kHidden, true}, s)) != GK_OK)
        return st;
    if ((st = gemm(batch, kHidden, kHidden + 1, 1, XAugA{w.h1, kHidden, kHidden}, WeightKB{W1, kHidden + 1},
                   EpiAct{w.h2, kHidden, true}, s)) != GK_OK)
        return st;
    return gemm(batch, O, kHidden + 1, 1, XAugA{w.h2, kHidden, kHidden}, WeightKB{W2, kHidden + 1},
                EpiAct{y, O, false}, s);
}

extern "C" gk_status gk_mlp_bwd(const gk_mlp* net, int64_t batch, const float* x, const float* dy, float* grad,
                                void* work, size_t work_bytes_, gk_stream stream) {
    gk_status st = check_net(net);
    if (st != GK_OK) return st;
    if (batch < 1 || x == nullptr || dy == nullptr || grad == nullptr || work == nullptr) return GK_ERR_ARG;
    if (batch > GK_MLP_MAX_BATCH) return GK_ERR_SIZE;
    if (work_bytes_ < work_bytes(net->in_dim, net->out_dim, batch)) return GK_ERR_SIZE;
    cudaStream_t s = (cudaStream_t)stream;
    const int F = net->in_dim, O = net->out_dim;
    const __nv_bfloat16* P = reinterpret_cast<const __nv_bfloat16*>(net->params);
    Work w = carve(work, batch);
    const int ch = chunks_for(batch);
    const int64_t n0 = layer_params(0, F, O), n1 = layer_params(1, F, O), n2 = layer_params(2, F, O);
    const int64_t o0 = layer_offset(0, F, O), o1 = layer_offset(1, F, O), o2 = layer_offset(2, F, O);
    const unsigned rgrid = 2 * kSMs;
    // layer 3: dW2 = dy^T [H2 | 1]; dH2 = dy W2 masked by H2 > 0
    if ((st = gemm(O, kHidden + 1, batch, ch, TransA{dy, O}, XAugB{w.h2, kHidden, kHidden},
                   EpiPart{w.part, O, kHidden + 1}, s)) != GK_OK)
        return st;
    reduce_chunks_kernel<<<rgrid, 256, 0, s>>>(w.part, ch, n2, grad + o2);
    GK_LAUNCH_CHECK();
    if ((st = gemm(batch, kHidden, O, 1, RowA{dy, O}, WeightNB{P + o2, kHidden + 1}, EpiMask{w.d2, w.h2, kHidden},
                   s)) != GK_OK)
        return st;
    // layer 2
    if ((st = gemm(kHidden, kHidden + 1, batch, ch, TransA{w.d2, kHidden}, XAugB{w.h1, kHidden, kHidden},
                   EpiPart{w.part, kHidden, kHidden + 1}, s)) != GK_OK)
        return st;
    reduce_chunks_kernel<<<rgrid, 256, 0, s>>>(w.part, ch, n1, grad + o1);
    GK_LAUNCH_CHECK();
    if ((st = gemm(batch, kHidden, kHidden, 1, RowA{w.d2, kHidden}, WeightNB{P + o1, kHidden + 1},
                   EpiMask{w.d1, w.h1, kHidden}, s)) != GK_OK)
        return st;
    // layer 1
    if ((st = gemm(kHidden, F + 1, batch, ch, TransA{w.d1, kHidden}, XAugB{x, F, F}, EpiPart{w.part, kHidden, F + 1},
                   s)) != GK_OK)
        return st;
    reduce_chunks_kernel<<<rgrid, 256, 0, s>>>(w.part, ch, n0, grad + o0);
    GK_LAUNCH_CHECK();
    return GK_OK;
}

extern "C" gk_status gk_mlp_mse(int64_t batch, int32_t out_dim, const float* y, const float* target,
                                const float* weight, float* dy, float* loss, gk_stream stream) {
    if (batch < 1 || out_dim < 1 || out_dim > GK_MLP_MAX_OUT || y == nullptr || target == nullptr) return GK_ERR_ARG;
    mse_kernel<<<1, 1024, 0, (cudaStream_t)stream>>>(batch, out_dim, y, target, weight, dy, loss);
    GK_LAUNCH_CHECK();
    return GK_OK;
}

extern "C" gk_status gk_mlp_adam(int64_t n, float* master, uint16_t* params, const float* grad, float* m, float* v,
                                 const gk_adam* hp, int32_t step, gk_stream stream) {
    if (n < 1 || !master || !params || !grad || !m || !v || !hp || step < 1) return GK_ERR_ARG;
    if (!(hp->lr >= 0.f) || !(hp->beta1 >= 0.f && hp->beta1 < 1.f) || !(hp->beta2 >= 0.f && hp->beta2 < 1.f) ||
        !(hp->eps > 0.f))
        return GK_ERR_ARG;
    const float c1 = (float)(1.0 - pow((double)hp->beta1, step));
    const float c2 = (float)(1.0 - pow((double)hp->beta2, step));
    adam_kernel<<<2 * kSMs, 256, 0, (cudaStream_t)stream>>>(n, master, reinterpret_cast<__nv_bfloat16*>(params), grad,
                                                              m, v, *hp, c1, c2);
    GK_LAUNCH_CHECK();
    return GK_OK;
}

// ----------------------------------------------------------------------------
// Geometry descriptor of one kriging system (GK_SYSTEM_FEATURES floats), the
// system-dependent half of the network input.  One CTA, FP64 accumulation,
// fixed-order reductions (deterministic).  Features:
//   0 log(N)/10              1 3 n_ori / N          2 n_iface / N
//   3-5 extent / range (x,y,z) of all point and orientation positions
//   6-8 standard deviation / range (x,y,z)
//   9 |mean unit gradient|   10 mean |unit gradient z|
//   11 mean log10 nugget_sp / 10        12 mean log10 nugget_grad / 10
//   13 drift degree / 2
//   14 log(mean spacing / range) / 5, spacing = (box volume / points)^(1/3)
//   15 log(1 + surfaces) / 5
// ----------------------------------------------------------------------------
namespace gk {
namespace mlp {

enum Op { kSum, kMin, kMax };

__device__ double block_reduce(double v, Op op, double* sh) {
    for (int o = 16; o > 0; o >>= 1) {
        const double u = __shfl_down_sync(0xffffffffu, v, o);
        v = op == kSum ? v + u : (op == kMin ? fmin(v, u) : fmax(v, u));
    }
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) sh[w] = v;
    __syncthreads();
    if (w == 0) {
        const int nw = blockDim.x >> 5;
        v = lane < nw ? sh[lane] : (op == kSum ? 0.0 : (op == kMin ? 1e300 : -1e300));
        for (int o = 16; o > 0; o >>= 1) {
            const double u = __shfl_down_sync(0xffffffffu, v, o);
            v = op == kSum ? v + u : (op == kMin ? fmin(v, u) : fmax(v, u));
        }
        if (lane == 0) sh[32] = v;
    }
    __syncthreads();
    return sh[32];
}

__global__ void __launch_bounds__(1024) features_kernel(gk_system s, int64_t N, float* out) {
    __shared__ double sh[33];
    const int64_t np = (int64_t)s.n_ori + s.n_sp;
    double mn[3], mx[3], sm[3], sq[3], g[3] = {0, 0, 0}, gz = 0, lsp = 0, lgr = 0;
    for (int k = 0; k < 3; ++k) { mn[k] = 1e300; mx[k] = -1e300; sm[k] = 0; sq[k] = 0; }
    for (int64_t i = threadIdx.x; i < np; i += blockDim.x) {
        const double* p = i < s.n_ori ? s.dip_positions + 3 * i : s.sp_coords + 3 * (i - s.n_ori);
        for (int k = 0; k < 3; ++k) {
            mn[k] = fmin(mn[k], p[k]);
            mx[k] = fmax(mx[k], p[k]);
            sm[k] += p[k];
            sq[k] += p[k] * p[k];
        }
        if (i < s.n_ori) {
            const double* q = s.dip_gradients + 3 * i;
            const double nq = sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]);
            const double inv = nq > 0 ? 1.0 / nq : 0.0;
            for (int k = 0; k < 3; ++k) g[k] += q[k] * inv;
            gz += fabs(q[2]) * inv;
            lgr += log10(fmax(s.nugget_grad[i], 1e-30));
        } else {
            lsp += log10(fmax(s.nugget_sp[i - s.n_ori], 1e-30));
        }
    }
    double ext[3], sd[3], gm[3];
    const double inp = np > 0 ? 1.0 / (double)np : 0.0;
    for (int k = 0; k < 3; ++k) {
        const double a = block_reduce(mn[k], kMin, sh), b = block_reduce(mx[k], kMax, sh);
        const double m1 = block_reduce(sm[k], kSum, sh) * inp, m2 = block_reduce(sq[k], kSum, sh) * inp;
        ext[k] = np > 0 ? b - a : 0.0;
        sd[k] = sqrt(fmax(m2 - m1 * m1, 0.0));
        gm[k] = block_reduce(g[k], kSum, sh);
    }
    const double gzs = block_reduce(gz, kSum, sh), ls = block_reduce(lsp, kSum, sh), lg = block_reduce(lgr, kSum, sh);
    if (threadIdx.x == 0) {
        const double R = s.range, no = s.n_ori > 0 ? (double)s.n_ori : 1.0, ns = s.n_sp > 0 ? (double)s.n_sp : 1.0;
        double vol = 1.0;
        for (int k = 0; k < 3; ++k) vol *= fmax(ext[k], 1e-3 * R);
        float f[GK_SYSTEM_FEATURES];
        f[0] = (float)(log((double)N) / 10.0);
        f[1] = (float)(3.0 * s.n_ori / (double)N);
        f[2] = (float)((double)s.n_iface / (double)N);
        for (int k = 0; k < 3; ++k) {
            f[3 + k] = (float)(ext[k] / R);
            f[6 + k] = (float)(sd[k] / R);
        }
        f[9] = (float)(sqrt(gm[0] * gm[0] + gm[1] * gm[1] + gm[2] * gm[2]) / no);
        f[10] = (float)(gzs / no);
        f[11] = (float)(ls / ns / 10.0);
        f[12] = (float)(lg / no / 10.0);
        f[13] = (float)(s.uni_degree / 2.0);
        f[14] = (float)(log(cbrt(vol / (double)(np > 0 ? np : 1)) / R) / 5.0);
        f[15] = (float)(log(1.0 + (double)(s.n_sp - s.n_iface)) / 5.0);
        for (int k = 0; k < GK_SYSTEM_FEATURES; ++k) out[k] = f[k];
    }
}

}  // namespace mlp
}  // namespace gk

gk_status gk_check_system(const gk_system* s);

extern "C" gk_status gk_system_features(const gk_system* s, float* features, gk_stream stream) {
    gk_status st = gk_check_system(s);
    if (st != GK_OK) return st;
    if (features == nullptr) return GK_ERR_ARG;
    const int64_t N = gk_system_size(s);
    gk::mlp::features_kernel<<<1, 1024, 0, (cudaStream_t)stream>>>(*s, N, features);
    GK_LAUNCH_CHECK();
    return GK_OK;
}
