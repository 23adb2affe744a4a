// Scalar-field / gradient evaluation with fused sigmoid segmentation, and the
// series combination.  Replaces the engine's grid evaluation and
// segmentation reached from gempy/API/compute_API.py:68-73 (outputs read back
// as exported_fields.scalar_field, values_block / ids_block).
//
// Contraction.  With the solved weights folded into packed "records"
//   orientation o : (x_o, c_o gi_res w_o)          -> Z += C'/r(|x-x_o|) (w_o . (x_o - x))
//   surface point p: (x_p, c_o gi_res alpha_p)     -> Z += alpha_p C(|x - x_p|)
// every grid point needs one radial kernel per record; records are streamed
// through shared memory in tiles by the TMA engine (1-D cp.async.bulk with an
// mbarrier, two stages), so a CTA's 256 threads x PPT points reuse each tile.
// Grid coordinates of regular grids are generated in the kernel.  In FP32 mode
// the per-tile partial sums are FP32 and are added into FP64 accumulators once
// per tile; the drift, the segmentation thresholds and the outputs are FP64.
#include <cooperative_groups.h>

#include <algorithm>
#include <cstring>

#include "gk_common.cuh"
#include "gk_ff.cuh"
#include "gk_tune.h"

namespace gk {

static size_t al256(size_t x) { return (x + 255) & ~(size_t)255; }

// Drift weights of the packed model (times gi_res): slots 0..8 the polynomial
// drift, slots kFaultSlot.. the fault drifts.
constexpr int kFaultSlot = 9;
constexpr int kMuSlots = 32;
static_assert(kFaultSlot + GK_MAX_FAULTS <= kMuSlots, "drift slots");

struct ModelLayout {
    size_t ori64, sp64, mu64, ori32, sp32, alpha, ffori, ffsp, ffmeta, total;
};

static ModelLayout model_layout(int n_ori, int n_sp) {
    ModelLayout L;
    size_t o = 0;
    L.ori64 = o; o += al256((size_t)n_ori * 8 * sizeof(double));
    L.sp64 = o;  o += al256((size_t)n_sp * 4 * sizeof(double));
    L.mu64 = o;  o += al256(kMuSlots * sizeof(double));
    L.ori32 = o; o += al256((size_t)n_ori * 8 * sizeof(float));
    L.sp32 = o;  o += al256((size_t)n_sp * 4 * sizeof(float));
    L.alpha = o; o += al256((size_t)n_sp * sizeof(double));
    L.ffori = o; o += al256((size_t)n_ori * 16 * sizeof(float));
    L.ffsp = o;  o += al256((size_t)n_sp * 8 * sizeof(float));
    L.ffmeta = o; o += al256(8 * sizeof(double));
    L.total = o;
    return L;
}

// alpha[rest_t] += gi w_t   (rest points are unique per interface row)
__global__ void alpha_rest_kernel(const int32_t* __restrict__ rest, int n_iface, const double* __restrict__ wi,
                                  double gi, double* alpha) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n_iface) atomicAdd(alpha + rest[t], gi * wi[t]);
}

// alpha[ref] -= gi sum_{t in run} w_t, one thread per run of equal ref_index
__global__ void alpha_ref_kernel(const int32_t* __restrict__ ref, int n_iface, const double* __restrict__ wi, double gi,
                                 double* alpha) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_iface) return;
    if (t > 0 && ref[t - 1] == ref[t]) return;
    double s = 0.0;
    int u = t;
    for (; u < n_iface && ref[u] == ref[t]; ++u) s += wi[u];
    atomicAdd(alpha + ref[t], -gi * s);
}

__global__ void pack_kernel(int n_ori, int n_sp, int n_iface, int n_drift, int n_fault, double scale, double gi,
                            const double* __restrict__ dip, const double* __restrict__ sp,
                            const double* __restrict__ w, const double* __restrict__ alpha, double* ori64,
                            double* sp64, double* mu64, float* ori32, float* sp32) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n_ori) {
        double rec[8] = {dip[3 * i], dip[3 * i + 1], dip[3 * i + 2], scale * w[i], scale * w[n_ori + i],
                         scale * w[2 * n_ori + i], 0.0, 0.0};
        for (int k = 0; k < 8; ++k) { ori64[8 * i + k] = rec[k]; ori32[8 * i + k] = (float)rec[k]; }
    }
    if (i < n_sp) {
        double rec[4] = {sp[3 * i], sp[3 * i + 1], sp[3 * i + 2], scale * alpha[i]};
        for (int k = 0; k < 4; ++k) { sp64[4 * i + k] = rec[k]; sp32[4 * i + k] = (float)rec[k]; }
    }
    if (i < kMuSlots) {
        const int64_t d0 = 3 * (int64_t)n_ori + n_iface;
        double m = 0.0;
        if (i < n_drift) m = gi * w[d0 + i];
        else if (i >= kFaultSlot && i < kFaultSlot + n_fault) m = gi * w[d0 + n_drift + (i - kFaultSlot)];
        mu64[i] = m;
    }
}

// Float-float records.  Coordinates are scaled by 1/range (so s = |x-p|/a
// directly) and split into hi + lo with hi a multiple of the quantum q: every
// hi with |hi| <= 2^23 q differs from another such hi by an exactly
// representable float, so x_hi - p_hi is exact.  q = 2^(ceil(log2 max|u|) + 4
// - 23) leaves room for evaluation points 16x farther out than any datum;
// points beyond that take an exact two-sum path.  meta[0] = q,
// meta[1] = max|u| bits (as float), meta[2] = 1/range.
__global__ void ff_maxabs_kernel(const double* __restrict__ a, int n3, double inv_a, unsigned int* maxbits) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    float v = i < n3 ? (float)fabs(a[i] * inv_a) : 0.f;
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_down_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0) atomicMax(maxbits, __float_as_uint(v));
}

__global__ void pack_ff_kernel(int n_ori, int n_sp, double inv_a, double w_scale_ori, double w_scale_sp,
                               const double* __restrict__ dip, const double* __restrict__ sp,
                               const double* __restrict__ w, const double* __restrict__ alpha,
                               const unsigned int* maxbits, float* ffori, float* ffsp, double* meta) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    const double q = ff_quantum(maxbits);
    if (i == 0) { meta[0] = q; meta[2] = inv_a; }
    if (i < n_ori) {
        float* r = ffori + 16 * i;
        for (int k = 0; k < 3; ++k) ff_split(dip[3 * i + k] * inv_a, q, r[2 * k], r[2 * k + 1]);
        for (int k = 0; k < 3; ++k) {
            ff v = ff_from_double(w_scale_ori * w[k * n_ori + i]);
            r[6 + 2 * k] = v.h;
            r[7 + 2 * k] = v.l;
        }
        for (int k = 12; k < 16; ++k) r[k] = 0.f;
    }
    if (i < n_sp) {
        float* r = ffsp + 8 * i;
        for (int k = 0; k < 3; ++k) ff_split(sp[3 * i + k] * inv_a, q, r[2 * k], r[2 * k + 1]);
        ff v = ff_from_double(w_scale_sp * alpha[i]);
        r[6] = v.h;
        r[7] = v.l;
    }
}

// ---------------------------------------------------------------------------
// TMA (bulk copy) + mbarrier helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}
__device__ __forceinline__ bool mbar_try(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait for a stage's bulk copy: the first wait on a stage uses the
// module's cap (wait_cap), the drain before an early exit the default.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, long long cap) {
    for (long long i = 0; i < cap; ++i)
        if (mbar_try(bar, parity)) return true;
    return false;
}

struct EvalParams {
    int kind;
    int dims[3];
    int64_t n;
    double origin[3], spacing[3];
    const double* xyz;
    int n_ori, n_sp, n_drift, degree, kernel, n_fault;
    double range;
    const double* fault_rows[GK_MAX_FAULTS];  // block of each offsetting fault at the points
    const void* ori;   // packed records in T
    const void* sp;
    const double* mu;
    int tiles_ori, tiles_sp, rec_ori, rec_sp;  // records per tile
    int stage_bytes;
    int split;         // CTAs of one cluster sharing a chunk of points (1: no cluster)
    int has_seg;
    gk_segment seg;
    double* field;
    double* grad;
    double* values;
    int32_t* ids;
    gk_info* info;     // device status word (timeouts), may be NULL
    int col;           // float-float path: each thread takes PPT consecutive points of one grid column
};

template <typename T> __device__ __forceinline__ T fast_r(T r2);
template <> __device__ __forceinline__ float fast_r<float>(float r2) { return r2 > 0.f ? r2 * rsqrtf(r2) : 0.f; }
template <> __device__ __forceinline__ double fast_r<double>(double r2) { return sqrt(r2); }

template <typename T> __device__ __forceinline__ T sigm(double t);
template <> __device__ __forceinline__ double sigm<double>(double t) {
    if (t >= 0.0) return 1.0 / (1.0 + exp(-t));
    double e = exp(t);
    return e / (1.0 + e);
}
template <> __device__ __forceinline__ float sigm<float>(double t) {
    float tf = (float)t;
    if (tf >= 0.f) return 1.f / (1.f + expf(-tf));
    float e = expf(tf);
    return e / (1.f + e);
}

// Fault-drift contribution at point i: sum_f nu_f F_f(x_i).
__device__ __forceinline__ double fault_term(const EvalParams& P, int64_t i) {
    double z = 0.0;
    for (int f = 0; f < P.n_fault; ++f) z += P.mu[kFaultSlot + f] * P.fault_rows[f][i];
    return z;
}

// Block id: u_0 + sum_k (u_(k+1) - u_k) [z < z_k - GK_TIE_TOL] (a point on a
// surface takes the unit above it).
__device__ __forceinline__ int32_t block_id(const gk_segment& S, double z) {
    double v = S.unit_values[0];
    for (int k = 0; k < S.n_surf; ++k)
        if (z < S.isovalues[k] - GK_TIE_TOL) v += S.unit_values[k + 1] - S.unit_values[k];
    return (int32_t)rint(v);
}

__device__ __forceinline__ void point_coords(const EvalParams& P, int64_t q, double* xd) {
    if (P.kind == 0) {
        const int64_t nyz = (int64_t)P.dims[1] * P.dims[2];
        const int64_t ix = q / nyz, rem = q - ix * nyz;
        const int64_t iy = rem / P.dims[2], iz = rem - iy * P.dims[2];
        xd[0] = P.origin[0] + (double)ix * P.spacing[0];
        xd[1] = P.origin[1] + (double)iy * P.spacing[1];
        xd[2] = P.origin[2] + (double)iz * P.spacing[2];
    } else {
        xd[0] = P.xyz[3 * q];
        xd[1] = P.xyz[3 * q + 1];
        xd[2] = P.xyz[3 * q + 2];
    }
}

// Outputs of point i from the covariance sums z (and gradient sums g, or
// NULL): drift, fault drift, field, gradient, sigmoid segmentation and ids.
// Ts is the type the sigmoid is computed in.
template <typename Ts>
__device__ __forceinline__ void finish_point(const EvalParams& P, int64_t i, const double* xd, double z,
                                             const double* g) {
    const double* mu = P.mu;
    const double X = xd[0], Y = xd[1], Zc = xd[2];
    if (P.n_drift >= 3) z += mu[0] * X + mu[1] * Y + mu[2] * Zc;
    if (P.n_drift >= 9)
        z += mu[3] * X * X + mu[4] * Y * Y + mu[5] * Zc * Zc + mu[6] * X * Y + mu[7] * X * Zc + mu[8] * Y * Zc;
    if (P.n_fault) z += fault_term(P, i);
    if (P.field) P.field[i] = z;
    if (g != nullptr && P.grad) {
        double gx = g[0], gy = g[1], gz = g[2];
        if (P.n_drift >= 3) { gx += mu[0]; gy += mu[1]; gz += mu[2]; }
        if (P.n_drift >= 9) {
            gx += 2.0 * mu[3] * X + mu[6] * Y + mu[7] * Zc;
            gy += 2.0 * mu[4] * Y + mu[6] * X + mu[8] * Zc;
            gz += 2.0 * mu[5] * Zc + mu[7] * X + mu[8] * Y;
        }
        P.grad[3 * i] = gx;
        P.grad[3 * i + 1] = gy;
        P.grad[3 * i + 2] = gz;
    }
    if (P.has_seg) {
        double v = P.seg.unit_values[0];
        for (int k = 0; k < P.seg.n_surf; ++k)
            v += (P.seg.unit_values[k + 1] - P.seg.unit_values[k]) *
                 (double)sigm<Ts>(P.seg.slope * (P.seg.isovalues[k] - z));
        if (P.values) P.values[i] = v;
        if (P.ids) P.ids[i] = block_id(P.seg, z);
    }
}

// Record split.  When the chunks of points would fill less than half of the
// GPU, `split` CTAs of one thread-block cluster share each chunk: rank r
// streams record tiles r, r + split, r + 2 split, ... and leaves its partial
// sums in shared memory (`red`, NV values per point slot).  Past a cluster
// barrier every CTA adds the partials of all ranks in rank order through
// distributed shared memory -- the result does not depend on scheduling -- and
// finishes its share of the chunk's points; a second barrier keeps the
// partials alive until every rank has read them.  A CTA whose copy wait gave
// up sets the abort word of every CTA of its cluster before the first barrier,
// so the whole cluster passes the same barriers and stops together.
namespace cg = cooperative_groups;

template <typename Ts, int NV>
__device__ __forceinline__ bool split_finish(const EvalParams& P, int64_t chunk, int64_t chunk_pts, int rank,
                                             double* red, int* s_abort, bool failed) {
    cg::cluster_group cl = cg::this_cluster();
    if (failed && threadIdx.x == 0)
        for (int r = 0; r < P.split; ++r) *cl.map_shared_rank(s_abort, r) = 1;
    cl.sync();
    const bool aborted = *(volatile int*)s_abort != 0;
    if (!aborted) {
        for (int64_t f = (int64_t)rank * blockDim.x + threadIdx.x; f < chunk_pts; f += (int64_t)P.split * blockDim.x) {
            const int64_t i = chunk * chunk_pts + f;
            if (i >= P.n) continue;
            double v[NV];
#pragma unroll
            for (int c = 0; c < NV; ++c) v[c] = 0.0;
            for (int r = 0; r < P.split; ++r) {
                const double* rr = cl.map_shared_rank(red, r);
#pragma unroll
                for (int c = 0; c < NV; ++c) v[c] += rr[c * chunk_pts + f];
            }
            double xd[3];
            point_coords(P, i, xd);
            finish_point<Ts>(P, i, xd, v[0], NV == 4 ? v + 1 : nullptr);
        }
    }
    cl.sync();
    return aborted;
}

template <typename T, int PPT, bool GRAD, bool SPLIT>
__global__ void __launch_bounds__(256) eval_kernel(const EvalParams P) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t mbar[2];
    __shared__ int s_fail, s_abort;
    const int tid = threadIdx.x;
    const int split = SPLIT ? P.split : 1;
    unsigned char* stage[2] = {smem, smem + P.stage_bytes};
    if (tid == 0) {
        mbar_init(&mbar[0], 1);
        mbar_init(&mbar[1], 1);
        mbar_fence_init();
        s_fail = 0;
        s_abort = 0;
    }
    __syncthreads();
    if (SPLIT) cg::this_cluster().sync();  // abort words initialised before any peer can set one

    const Cov<T> cv = Cov<T>::make(P.kernel, P.range);
    const int64_t chunk_pts = (int64_t)blockDim.x * PPT;
    const int64_t n_chunks = (P.n + chunk_pts - 1) / chunk_pts;
    const int n_tiles = P.tiles_ori + P.tiles_sp;
    const int rank = SPLIT ? (int)cg::this_cluster().block_rank() : 0;
    const int64_t group = blockIdx.x / split, n_groups = gridDim.x / split;
    const int my_tiles = n_tiles > rank ? (n_tiles - 1 - rank) / split + 1 : 0;
    const int64_t my_chunks = n_chunks > group ? (n_chunks - 1 - group) / n_groups + 1 : 0;
    const int64_t n_items = my_chunks * my_tiles;

    auto tile_src = [&](int t, uint32_t& bytes) -> const void* {
        if (t < P.tiles_ori) {
            int r0 = t * P.rec_ori;
            int nr = min(P.rec_ori, P.n_ori - r0);
            bytes = (uint32_t)(nr * 8 * sizeof(T));
            return (const T*)P.ori + (size_t)r0 * 8;
        }
        int ts = t - P.tiles_ori;
        int r0 = ts * P.rec_sp;
        int nr = min(P.rec_sp, P.n_sp - r0);
        bytes = (uint32_t)(nr * 4 * sizeof(T));
        return (const T*)P.sp + (size_t)r0 * 4;
    };
    auto issue = [&](int64_t item) {
        if (tid != 0) return;
        int s = (int)(item & 1);
        int t = rank + (int)(item % my_tiles) * split;
        uint32_t bytes;
        const void* src = tile_src(t, bytes);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_expect_tx(&mbar[s], bytes);
        bulk_g2s(stage[s], src, bytes, &mbar[s]);
    };
    if (n_items > 0) issue(0);
    if (n_items > 1) issue(1);

    int64_t item = 0;
    for (int64_t lc = 0; lc < my_chunks; ++lc) {
        const int64_t chunk = group + lc * n_groups;
        T x[PPT][3];
        double xd[PPT][3];
        int64_t pid[PPT];
        bool act[PPT];   // slots past the end of the point list compute nothing
#pragma unroll
        for (int p = 0; p < PPT; ++p) {
            pid[p] = chunk * chunk_pts + tid + (int64_t)p * blockDim.x;
            act[p] = pid[p] < P.n;
            point_coords(P, act[p] ? pid[p] : P.n - 1, xd[p]);
            for (int k = 0; k < 3; ++k) x[p][k] = (T)xd[p][k];
        }
        double Z[PPT], G[PPT][3];
#pragma unroll
        for (int p = 0; p < PPT; ++p) {
            Z[p] = 0.0;
            G[p][0] = G[p][1] = G[p][2] = 0.0;
        }

        for (int k = 0; k < my_tiles; ++k, ++item) {
            const int t = rank + k * split;
            const int s = (int)(item & 1);
            const uint32_t parity = (uint32_t)((item >> 1) & 1);
            if (!mbar_wait(&mbar[s], parity, wait_cap(kCopySpin))) {
                report(P.info, GK_ERR_TIMEOUT, (int)blockIdx.x);
                s_fail = 1;
            }
            __syncthreads();
            if (s_fail) {
                if (!SPLIT) goto drain;
                break;  // the cluster learns of it at the next barrier
            }
            {
                T zt[PPT], gt[PPT][3];
#pragma unroll
                for (int p = 0; p < PPT; ++p) { zt[p] = (T)0; gt[p][0] = gt[p][1] = gt[p][2] = (T)0; }
                if (t < P.tiles_ori) {
                    const T* rec = reinterpret_cast<const T*>(stage[s]);
                    const int nr = min(P.rec_ori, P.n_ori - t * P.rec_ori);
                    for (int q = 0; q < nr; ++q) {
                        const T ox = rec[8 * q], oy = rec[8 * q + 1], oz = rec[8 * q + 2];
                        const T wx = rec[8 * q + 3], wy = rec[8 * q + 4], wz = rec[8 * q + 5];
#pragma unroll
                        for (int p = 0; p < PPT; ++p) {
                            if (!act[p]) continue;
                            const T hx = ox - x[p][0], hy = oy - x[p][1], hz = oz - x[p][2];
                            const T r = fast_r<T>(hx * hx + hy * hy + hz * hz + (T)kDistEps2);
                            const T k1 = cv.d1_r(r);
                            const T wh = wx * hx + wy * hy + wz * hz;
                            zt[p] += k1 * wh;
                            if (GRAD) {
                                const T k3 = cv.d3_r(r) * wh;
                                gt[p][0] -= k3 * hx + k1 * wx;
                                gt[p][1] -= k3 * hy + k1 * wy;
                                gt[p][2] -= k3 * hz + k1 * wz;
                            }
                        }
                    }
                } else {
                    const T* rec = reinterpret_cast<const T*>(stage[s]);
                    const int ts = t - P.tiles_ori;
                    const int nr = min(P.rec_sp, P.n_sp - ts * P.rec_sp);
                    for (int q = 0; q < nr; ++q) {
                        const T px = rec[4 * q], py = rec[4 * q + 1], pz = rec[4 * q + 2], al = rec[4 * q + 3];
#pragma unroll
                        for (int p = 0; p < PPT; ++p) {
                            if (!act[p]) continue;
                            const T hx = x[p][0] - px, hy = x[p][1] - py, hz = x[p][2] - pz;
                            const T r = fast_r<T>(hx * hx + hy * hy + hz * hz + (T)kDistEps2);
                            zt[p] += al * cv.C(r);
                            if (GRAD) {
                                const T k1 = al * cv.d1_r(r);
                                gt[p][0] += k1 * hx;
                                gt[p][1] += k1 * hy;
                                gt[p][2] += k1 * hz;
                            }
                        }
                    }
                }
#pragma unroll
                for (int p = 0; p < PPT; ++p) {
                    Z[p] += (double)zt[p];
                    if (GRAD) { G[p][0] += (double)gt[p][0]; G[p][1] += (double)gt[p][1]; G[p][2] += (double)gt[p][2]; }
                }
            }
            __syncthreads();  // stage s fully consumed
            if (item + 2 < n_items) issue(item + 2);
        }
        if (SPLIT) {
            constexpr int NV = GRAD ? 4 : 1;
            double* red = reinterpret_cast<double*>(smem + 2 * (size_t)P.stage_bytes);
#pragma unroll
            for (int p = 0; p < PPT; ++p) {
                const int64_t f = tid + (int64_t)p * blockDim.x;
                red[f] = Z[p];
                if (GRAD) for (int c = 0; c < 3; ++c) red[(c + 1) * chunk_pts + f] = G[p][c];
            }
            if (split_finish<T, NV>(P, chunk, chunk_pts, rank, red, &s_abort, s_fail != 0)) goto drain;
        } else {
#pragma unroll
            for (int p = 0; p < PPT; ++p)
                if (act[p]) finish_point<T>(P, pid[p], xd[p], Z[p], GRAD ? G[p] : nullptr);
        }
    }
    return;
drain:
    // a copy wait gave up (here or in the cluster): wait, bounded, for the
    // copies still in flight, then leave
    if (tid == 0)
        for (int64_t it = item; it < n_items && it < item + 2; ++it)
            mbar_wait(&mbar[it & 1], (uint32_t)((it >> 1) & 1), kCopySpin);
    __syncthreads();
}

// ---------------------------------------------------------------------------
// float-float evaluation (cubic kernel, field only)
// ---------------------------------------------------------------------------
template <int PPT, bool SPLIT>
__global__ void __launch_bounds__(256) eval_ff_kernel(const EvalParams P, const double* __restrict__ meta) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t mbar[2];
    __shared__ int s_fail, s_abort;
    __shared__ float s_box[6 * 8];
    __shared__ float s_fold[10 * 8];
    const int tid = threadIdx.x;
    const int split = SPLIT ? P.split : 1;
    unsigned char* stage[2] = {smem, smem + P.stage_bytes};
    if (tid == 0) {
        mbar_init(&mbar[0], 1);
        mbar_init(&mbar[1], 1);
        mbar_fence_init();
        s_fail = 0;
        s_abort = 0;
    }
    __syncthreads();
    if (SPLIT) cg::this_cluster().sync();  // abort words initialised before any peer can set one
    const double q = meta[0], inv_a = meta[2];
    const float eps2 = fmaxf((float)(kDistEps2 * inv_a * inv_a), 1.17549435e-38f);  // a positive normal float
    const int64_t chunk_pts = (int64_t)blockDim.x * PPT;
    const int64_t n_chunks = (P.n + chunk_pts - 1) / chunk_pts;
    const int n_tiles = P.tiles_ori + P.tiles_sp;
    const int rank = SPLIT ? (int)cg::this_cluster().block_rank() : 0;
    const int64_t group = blockIdx.x / split, n_groups = gridDim.x / split;
    const int my_tiles = n_tiles > rank ? (n_tiles - 1 - rank) / split + 1 : 0;
    const int64_t my_chunks = n_chunks > group ? (n_chunks - 1 - group) / n_groups + 1 : 0;
    const int64_t n_items = my_chunks * my_tiles;

    auto issue = [&](int64_t item) {
        if (tid != 0) return;
        int s = (int)(item & 1);
        int t = rank + (int)(item % my_tiles) * split;
        const void* src;
        uint32_t bytes;
        if (t < P.tiles_ori) {
            int r0 = t * P.rec_ori;
            int nr = min(P.rec_ori, P.n_ori - r0);
            bytes = (uint32_t)(nr * 16 * sizeof(float));
            src = (const float*)P.ori + (size_t)r0 * 16;
        } else {
            int r0 = (t - P.tiles_ori) * P.rec_sp;
            int nr = min(P.rec_sp, P.n_sp - r0);
            bytes = (uint32_t)(nr * 8 * sizeof(float));
            src = (const float*)P.sp + (size_t)r0 * 8;
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_expect_tx(&mbar[s], bytes);
        bulk_g2s(stage[s], src, bytes, &mbar[s]);
    };
    if (n_items > 0) issue(0);
    if (n_items > 1) issue(1);
    // point of slot p within a chunk: strided by the block, or (col) PPT
    // consecutive points of one grid column, which share x and y
    const bool col = P.col != 0;
    auto slot = [&](int p) -> int64_t { return col ? (int64_t)PPT * tid + p : tid + (int64_t)p * blockDim.x; };

    int64_t item = 0;
    for (int64_t lc = 0; lc < my_chunks; ++lc) {
        const int64_t chunk = group + lc * n_groups;
        PointFF X[PPT];
        bool all_exact = true, act[PPT], any_act = false, all_act = true;
#pragma unroll
        for (int p = 0; p < PPT; ++p) {
            const int64_t pidp = chunk * chunk_pts + slot(p);
            act[p] = pidp < P.n;
            double xd[3];
            point_coords(P, act[p] ? pidp : P.n - 1, xd);
            ff_point(xd, inv_a, q, X[p]);
            all_exact = all_exact && (X[p].exact || !act[p]);
            any_act = any_act || act[p];
            all_act = all_act && act[p];
        }
        double Z[PPT];
#pragma unroll
        for (int p = 0; p < PPT; ++p) Z[p] = 0.0;
        // the chunk's bounding box (high words), for the per-tile range test
        // of the column path (col is uniform over the CTA)
        float pbox[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
        if (PPT >= 4 && col) {   // (the 2-point variant keeps its registers for the point lists)
#pragma unroll
            for (int p = 0; p < PPT; ++p)
                if (act[p])
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        pbox[c] = fminf(pbox[c], X[p].h[c]);
                        pbox[3 + c] = fmaxf(pbox[3 + c], X[p].h[c]);
                    }
            cta_bbox(pbox, s_box);
        }

        for (int k = 0; k < my_tiles; ++k, ++item) {
            const int t = rank + k * split;
            const int s = (int)(item & 1);
            const uint32_t parity = (uint32_t)((item >> 1) & 1);
            if (!mbar_wait(&mbar[s], parity, wait_cap(kCopySpin))) {
                report(P.info, GK_ERR_TIMEOUT, (int)blockIdx.x);
                s_fail = 1;
            }
            __syncthreads();
            if (s_fail) {
                if (!SPLIT) goto drain;
                break;  // the cluster learns of it at the next barrier
            }
            {
                ffacc acc[PPT];
#pragma unroll
                for (int p = 0; p < PPT; ++p) acc[p] = {0.f, 0.f};
                const float* rec = reinterpret_cast<const float*>(stage[s]);
                const bool ori = t < P.tiles_ori;
                const int nr = ori ? min(P.rec_ori, P.n_ori - t * P.rec_ori)
                                   : min(P.rec_sp, P.n_sp - (t - P.tiles_ori) * P.rec_sp);
                // every point-record pair of the tile within the range (r < 1
                // in scaled units)?  Box distance of the high words plus the
                // split quantum for the low words, with a margin for rounding.
                bool in_range = false;
                if (PPT >= 4 && col) {
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
                // the in-range column path folds the constant and r^2 terms of
                // the covariances into per-tile sums, which start the points'
                // accumulators (all threads take part in the reduction: in_range
                // and ori are uniform over the CTA)
                ff fold[5];
                const float o[3] = {0.5f * (pbox[0] + pbox[3]), 0.5f * (pbox[1] + pbox[4]),
                                    0.5f * (pbox[2] + pbox[5])};
                if (in_range) cta_fold_sums(rec, nr, ori, o, fold, s_fold);
                bool done = !any_act;
                if (!done && col && all_exact && all_act) {
                    if (in_range) {
#pragma unroll
                        for (int p = 0; p < PPT; ++p) {
                            const ff f0 = tile_fold(fold, ori, X[p], o, eps2);
                            acc[p] = {f0.h, f0.l};
                        }
                        ff_tile_col<PPT, false, true>(rec, ori, nr, X, eps2, acc);
                    } else {
                        ff_tile_col<PPT, true>(rec, ori, nr, X, eps2, acc);
                    }
                    done = true;
                }
                if (done) {
                } else if (all_exact && all_act) {
                    ff_tile<PPT, true, true>(rec, ori, nr, X, act, eps2, acc);
                } else if (all_exact) {
                    ff_tile<PPT, true>(rec, ori, nr, X, act, eps2, acc);
                } else {
                    ff_tile<PPT, false>(rec, ori, nr, X, act, eps2, acc);
                }
#pragma unroll
                for (int p = 0; p < PPT; ++p) Z[p] += ff_acc_to_double(acc[p]);
            }
            __syncthreads();
            if (item + 2 < n_items) issue(item + 2);
        }
        if (SPLIT) {
            double* red = reinterpret_cast<double*>(smem + 2 * (size_t)P.stage_bytes);
#pragma unroll
            for (int p = 0; p < PPT; ++p) red[slot(p)] = Z[p];
            if (split_finish<float, 1>(P, chunk, chunk_pts, rank, red, &s_abort, s_fail != 0)) goto drain;
        } else {
#pragma unroll
            for (int p = 0; p < PPT; ++p) {
                if (!act[p]) continue;
                const int64_t pidp = chunk * chunk_pts + slot(p);
                double xd[3];
                point_coords(P, pidp, xd);
                finish_point<float>(P, pidp, xd, Z[p], nullptr);
            }
        }
    }
    return;
drain:
    if (tid == 0)
        for (int64_t it = item; it < n_items && it < item + 2; ++it)
            mbar_wait(&mbar[it & 1], (uint32_t)((it >> 1) & 1), kCopySpin);
    __syncthreads();
}

// ---------------------------------------------------------------------------
// series combination
// ---------------------------------------------------------------------------
struct CombineParams {
    int n_series;
    int64_t n;
    const double* fields;
    const double* values;
    const int32_t* ids;
    int relations[GK_MAX_SURFACES];
    double min_iso[GK_MAX_SURFACES];
    double max_iso[GK_MAX_SURFACES];
    double* out_values;
    int32_t* out_ids;
    uint8_t* masks;
};

__global__ void combine_kernel(const CombineParams P) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    bool taken = false;
    double v = 0.0;
    int32_t id = 0;
    for (int s = 0; s < P.n_series; ++s) {
        bool raw;
        const int rel = P.relations[s];
        if (rel == 4 || s == P.n_series - 1) raw = true;                              // BASEMENT / last
        else if (rel == 1) raw = P.fields[(int64_t)s * P.n + i] >= P.min_iso[s];      // ERODE
        else if (rel == 2) raw = P.fields[(int64_t)(s + 1) * P.n + i] >= P.max_iso[s + 1];  // ONLAP
        else raw = false;                                                             // FAULT: no lithology
        bool m = raw && !taken;
        taken = taken || m;
        if (m) {
            v += P.values[(int64_t)s * P.n + i];
            id += P.ids[(int64_t)s * P.n + i];
        }
        if (P.masks) P.masks[(int64_t)s * P.n + i] = m ? 1 : 0;
    }
    if (P.out_values) P.out_values[i] = v;
    if (P.out_ids) P.out_ids[i] = id;
}

cudaError_t wait_cap_set_eval(long long v) { return set_wait_cap_here(v); }

}  // namespace gk

using namespace gk;

gk_status gk_check_system(const gk_system* s);

// The FP64 records of a packed model (for the adjoint): orientations
// (x, c_o gi_res w, 0, 0) x n_ori, surface points (x, c_o gi_res alpha) x n_sp.
void gk_eval_model_records(const gk_system* s, const void* model, const double** ori64, const double** sp64) {
    const ModelLayout L = model_layout(s->n_ori, s->n_sp);
    *ori64 = (const double*)((const char*)model + L.ori64);
    *sp64 = (const double*)((const char*)model + L.sp64);
}

extern "C" size_t gk_eval_model_bytes(const gk_system* s) {
    if (s == nullptr) return 0;
    return model_layout(s->n_ori, s->n_sp).total;
}

extern "C" gk_status gk_eval_prepare(const gk_system* s, const double* w, void* model, gk_stream stream) {
    gk_status st = gk_check_system(s);
    if (st != GK_OK) return st;
    if (w == nullptr || model == nullptr) return GK_ERR_ARG;
    cudaStream_t cs = (cudaStream_t)stream;
    ModelLayout L = model_layout(s->n_ori, s->n_sp);
    char* m = (char*)model;
    double* alpha = (double*)(m + L.alpha);
    const int n_drift = drift_count(s->uni_degree);
    const int ng = 3 * s->n_ori;
    GK_CUDA_TRY(cudaMemsetAsync(alpha, 0, (size_t)s->n_sp * sizeof(double), cs));
    if (s->n_iface > 0) {
        unsigned b = (unsigned)((s->n_iface + 255) / 256);
        alpha_rest_kernel<<<b, 256, 0, cs>>>(s->rest_index, s->n_iface, w + ng, s->gi_res, alpha);
        GK_LAUNCH_CHECK();
        alpha_ref_kernel<<<b, 256, 0, cs>>>(s->ref_index, s->n_iface, w + ng, s->gi_res, alpha);
        GK_LAUNCH_CHECK();
    }
    int nmax = s->n_ori > s->n_sp ? s->n_ori : s->n_sp;
    if (nmax < 16) nmax = 16;
    if (nmax < kMuSlots) nmax = kMuSlots;
    pack_kernel<<<(unsigned)((nmax + 255) / 256), 256, 0, cs>>>(
        s->n_ori, s->n_sp, s->n_iface, n_drift, s->n_fault, s->c_o * s->gi_res, s->gi_res, s->dip_positions, s->sp_coords, w,
        alpha, (double*)(m + L.ori64), (double*)(m + L.sp64), (double*)(m + L.mu64), (float*)(m + L.ori32),
        (float*)(m + L.sp32));
    GK_LAUNCH_CHECK();
    // float-float records (coordinates / range, weights with every constant folded in)
    double* meta = (double*)(m + L.ffmeta);
    unsigned int* maxbits = (unsigned int*)(meta + 1);
    GK_CUDA_TRY(cudaMemsetAsync(meta, 0, 8 * sizeof(double), cs));
    const double inv_a = 1.0 / s->range;
    if (s->n_ori > 0) {
        ff_maxabs_kernel<<<(unsigned)((3 * s->n_ori + 255) / 256), 256, 0, cs>>>(s->dip_positions, 3 * s->n_ori,
                                                                                inv_a, maxbits);
        GK_LAUNCH_CHECK();
    }
    if (s->n_sp > 0) {
        ff_maxabs_kernel<<<(unsigned)((3 * s->n_sp + 255) / 256), 256, 0, cs>>>(s->sp_coords, 3 * s->n_sp, inv_a,
                                                                               maxbits);
        GK_LAUNCH_CHECK();
    }
    pack_ff_kernel<<<(unsigned)((nmax + 255) / 256), 256, 0, cs>>>(
        s->n_ori, s->n_sp, inv_a, s->c_o * s->gi_res * inv_a, s->c_o * s->gi_res, s->dip_positions, s->sp_coords, w,
        alpha, maxbits, (float*)(m + L.ffori), (float*)(m + L.ffsp), meta);
    GK_LAUNCH_CHECK();
    return GK_OK;
}

// Record tiles of `rec_bytes_ori` / `rec_bytes_sp` bytes per record, at most
// `stage_bytes` bytes per tile; split > 1 cuts the records into about `split`
// tiles of each kind so every rank of a cluster streams about one of each.
static void plan_tiles(EvalParams& P, int stage_bytes, int rec_bytes_ori, int rec_bytes_sp, int split) {
    int ro = stage_bytes / rec_bytes_ori, rs = stage_bytes / rec_bytes_sp;
    if (split > 1) {
        ro = std::min(ro, std::max(1, (P.n_ori + split - 1) / split));
        rs = std::min(rs, std::max(1, (P.n_sp + split - 1) / split));
        stage_bytes = (std::max(ro * rec_bytes_ori, rs * rec_bytes_sp) + 127) & ~127;
    }
    P.stage_bytes = stage_bytes;
    P.rec_ori = ro;
    P.rec_sp = rs;
    P.tiles_ori = (P.n_ori + ro - 1) / ro;
    P.tiles_sp = (P.n_sp + rs - 1) / rs;
    P.split = split;
}

constexpr int kMaxSplit = 16;          // cluster sizes above 8 are opted into per kernel
constexpr int kMinSplitRecords = 8;    // records per rank below which a split does not pay

// Launches `kernel` over the chunks of P or, when the chunks alone would fill
// less than half of the GPU, `split_kernel` with the records split over a
// cluster of up to kMaxSplit CTAs per chunk.
template <typename Kernel, typename... Args>
static gk_status launch_chunks(Kernel kernel, Kernel split_kernel, EvalParams& P, int ppt, int stage_kb,
                               int rec_bytes_ori, int rec_bytes_sp, int nv, cudaStream_t st, Args... args) {
    const int64_t chunk_pts = 256LL * ppt;
    const int64_t n_chunks = (P.n + chunk_pts - 1) / chunk_pts;
    const int sms = device_sm_count();
    const int n_rec = P.n_ori + P.n_sp;
    int occ = 1;
    plan_tiles(P, stage_kb * 1024, rec_bytes_ori, rec_bytes_sp, 1);
    size_t smem = 2 * (size_t)P.stage_bytes;
    gk_status rc = cached_occupancy((const void*)kernel, 256, smem, occ);
    if (rc != GK_OK) return rc;
    int split = 1;
    while (split < kMaxSplit && n_chunks * (2 * split) <= (int64_t)occ * sms &&
           n_rec >= 2 * split * kMinSplitRecords)
        split *= 2;
    for (; split > 1; split /= 2) {
        plan_tiles(P, stage_kb * 1024, rec_bytes_ori, rec_bytes_sp, split);
        smem = 2 * (size_t)P.stage_bytes + (size_t)chunk_pts * nv * sizeof(double);
        int occ_s = 1;
        if (cached_occupancy((const void*)split_kernel, 256, smem, occ_s) != GK_OK) return GK_ERR_CUDA;
        if (cached_cluster_fits((const void*)split_kernel, 256, smem, split)) break;
    }
    if (split == 1) {
        plan_tiles(P, stage_kb * 1024, rec_bytes_ori, rec_bytes_sp, 1);
        smem = 2 * (size_t)P.stage_bytes;
        int64_t grid = std::min<int64_t>((int64_t)occ * sms, n_chunks);
        if (grid < 1) grid = 1;
        kernel<<<(unsigned)grid, 256, smem, st>>>(P, args...);
        GK_LAUNCH_CHECK();
        return GK_OK;
    }
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)split;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3((unsigned)(n_chunks * split));
    cfg.blockDim = dim3(256);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (cudaLaunchKernelEx(&cfg, split_kernel, P, args...) != cudaSuccess) {
        (void)cudaGetLastError();
        return GK_ERR_CUDA;
    }
    GK_LAUNCH_CHECK();
    return GK_OK;
}

template <typename T, int PPT, bool GRAD>
static gk_status launch_eval(EvalParams& P, cudaStream_t st, int stage_kb = 32) {
    return launch_chunks(eval_kernel<T, PPT, GRAD, false>, eval_kernel<T, PPT, GRAD, true>, P, PPT, stage_kb,
                         (int)(8 * sizeof(T)), (int)(4 * sizeof(T)), GRAD ? 4 : 1, st);
}

template <int PPT>
static gk_status launch_eval_ff(EvalParams& P, const double* meta, cudaStream_t st, int stage_kb) {
    // a regular grid whose columns hold a multiple of PPT points: each
    // thread's PPT points share their column (x, y)
    P.col = (P.kind == 0 && P.dims[2] % PPT == 0) ? 1 : 0;
    return launch_chunks(eval_ff_kernel<PPT, false>, eval_ff_kernel<PPT, true>, P, PPT, stage_kb,
                         (int)(16 * sizeof(float)), (int)(8 * sizeof(float)), 1, st, meta);
}

// gk_eval with the offsetting faults' blocks given as row pointers.
static gk_status eval_impl(const gk_system* s, const void* model, const gk_points* pts,
                           const double* const* fault_rows, gk_prec prec, const gk_segment* seg, double* field,
                           double* grad, double* values, int32_t* ids, gk_info* info, gk_stream stream) {
    gk_status st = gk_check_system(s);
    if (st != GK_OK) return st;
    if (model == nullptr || pts == nullptr) return GK_ERR_ARG;
    if (pts->n < 0) return GK_ERR_ARG;
    if (pts->n == 0) return GK_OK;
    if (pts->kind == 0) {
        if (pts->dims[0] <= 0 || pts->dims[1] <= 0 || pts->dims[2] <= 0) return GK_ERR_ARG;
        if ((int64_t)pts->dims[0] * pts->dims[1] * pts->dims[2] != pts->n) return GK_ERR_ARG;
    } else if (pts->kind != 1 || pts->xyz == nullptr) {
        return GK_ERR_ARG;
    }
    if (seg != nullptr && (seg->n_surf < 0 || seg->n_surf > GK_MAX_SURFACES)) return GK_ERR_SIZE;
    if ((values || ids) && seg == nullptr) return GK_ERR_ARG;
    if (s->n_ori + s->n_sp == 0) return GK_ERR_ARG;
    if (s->n_fault > 0 && fault_rows == nullptr) return GK_ERR_ARG;
    for (int f = 0; f < s->n_fault; ++f)
        if (fault_rows[f] == nullptr) return GK_ERR_ARG;
    ModelLayout L = model_layout(s->n_ori, s->n_sp);
    const char* m = (const char*)model;
    EvalParams P;
    memset(&P, 0, sizeof(P));
    P.kind = pts->kind;
    for (int k = 0; k < 3; ++k) {
        P.dims[k] = pts->dims[k];
        P.origin[k] = pts->origin[k];
        P.spacing[k] = pts->spacing[k];
    }
    P.n = pts->n;
    P.xyz = pts->xyz;
    P.n_ori = s->n_ori;
    P.n_sp = s->n_sp;
    P.n_drift = drift_count(s->uni_degree);
    P.degree = s->uni_degree;
    P.kernel = s->kernel;
    P.range = s->range;
    P.n_fault = s->n_fault;
    for (int f = 0; f < s->n_fault; ++f) P.fault_rows[f] = fault_rows[f];
    P.mu = (const double*)(m + L.mu64);
    P.has_seg = seg != nullptr;
    if (seg) P.seg = *seg;
    P.field = field;
    P.grad = grad;
    P.values = values;
    P.ids = ids;
    P.info = info;
    cudaStream_t cs = (cudaStream_t)stream;
    if (prec == GK_F64) {
        P.ori = m + L.ori64;
        P.sp = m + L.sp64;
        return grad ? launch_eval<double, 1, true>(P, cs) : launch_eval<double, 1, false>(P, cs);
    }
    if (prec == GK_F32) {
        P.ori = m + L.ori32;
        P.sp = m + L.sp32;
        if (grad) return launch_eval<float, 2, true>(P, cs);
        const TuneVariant v = tune_variant(GK_TUNE_EVAL_F32);
        return v.ppt == 2 ? launch_eval<float, 2, false>(P, cs, v.stage_kb)
                          : launch_eval<float, 4, false>(P, cs, v.stage_kb);
    }
    if (prec == GK_FF) {
        if (grad != nullptr || s->kernel != GK_KERNEL_CUBIC) return GK_ERR_ARG;
        P.ori = m + L.ffori;
        P.sp = m + L.ffsp;
        const TuneVariant v = tune_variant(P.kind == 0 ? GK_TUNE_EVAL_FF : GK_TUNE_EVAL_FF_LIST);
        return v.ppt == 2 ? launch_eval_ff<2>(P, (const double*)(m + L.ffmeta), cs, v.stage_kb)
                          : launch_eval_ff<4>(P, (const double*)(m + L.ffmeta), cs, v.stage_kb);
    }
    return GK_ERR_ARG;
}

extern "C" gk_status gk_eval(const gk_system* s, const void* model, const gk_points* pts, gk_prec prec,
                             const gk_segment* seg, double* field, double* grad, double* values, int32_t* ids,
                             gk_info* info, gk_stream stream) {
    if (s == nullptr || pts == nullptr) return GK_ERR_ARG;
    const double* rows[GK_MAX_FAULTS] = {nullptr};
    if (s->n_fault > 0) {
        if (s->n_fault > GK_MAX_FAULTS) return GK_ERR_SIZE;
        if (pts->fault_values == nullptr || pts->fault_ld < pts->n) return GK_ERR_ARG;
        for (int f = 0; f < s->n_fault; ++f) rows[f] = pts->fault_values + (int64_t)f * pts->fault_ld;
    }
    return eval_impl(s, model, pts, rows, prec, seg, field, grad, values, ids, info, stream);
}

extern "C" gk_status gk_eval_series_set(int32_t n_series, const gk_series_eval* series, const gk_points* pts,
                                        gk_prec prec, double* fields, double* values, int32_t* ids, double* block,
                                        int32_t* lith_ids, uint8_t* masks, gk_info* info, gk_stream stream) {
    if (n_series < 1 || n_series > GK_MAX_SURFACES || series == nullptr || pts == nullptr) return GK_ERR_ARG;
    if (fields == nullptr || values == nullptr || ids == nullptr) return GK_ERR_ARG;
    const int64_t n = pts->n;
    if (n < 0) return GK_ERR_ARG;
    if (n == 0) return GK_OK;
    int32_t rel[GK_MAX_SURFACES];
    double mn[GK_MAX_SURFACES], mx[GK_MAX_SURFACES];
    for (int i = 0; i < n_series; ++i) {
        const gk_series_eval& e = series[i];
        if (e.sys == nullptr) return GK_ERR_ARG;
        if (e.n_faults != e.sys->n_fault) return GK_ERR_ARG;
        const double* rows[GK_MAX_FAULTS] = {nullptr};
        for (int f = 0; f < e.n_faults; ++f) {
            const int j = e.faults[f];
            if (j < 0 || j >= i) return GK_ERR_ARG;  // a fault offsets younger series only
            rows[f] = values + (int64_t)j * n;
        }
        gk_status st = eval_impl(e.sys, e.model, pts, rows, prec, &e.seg, fields + (int64_t)i * n, nullptr,
                                 values + (int64_t)i * n, ids + (int64_t)i * n, info, stream);
        if (st != GK_OK) return st;
        rel[i] = e.relation;
        mn[i] = e.min_iso;
        mx[i] = e.max_iso;
    }
    if (block == nullptr && lith_ids == nullptr && masks == nullptr) return GK_OK;
    return gk_combine_series(n_series, n, fields, values, ids, rel, mn, mx, block, lith_ids, masks, stream);
}

extern "C" gk_status gk_combine_series(int32_t n_series, int64_t n, const double* fields, const double* values,
                                       const int32_t* ids, const int32_t* relations, const double* min_iso,
                                       const double* max_iso, double* out_values, int32_t* out_ids, uint8_t* masks,
                                       gk_stream stream) {
    if (n_series < 1 || n_series > GK_MAX_SURFACES || n < 0) return GK_ERR_ARG;
    if (fields == nullptr || values == nullptr || ids == nullptr || relations == nullptr || min_iso == nullptr ||
        max_iso == nullptr)
        return GK_ERR_ARG;
    if (n == 0) return GK_OK;
    CombineParams P;
    memset(&P, 0, sizeof(P));
    P.n_series = n_series;
    P.n = n;
    P.fields = fields;
    P.values = values;
    P.ids = ids;
    for (int s = 0; s < n_series; ++s) {
        if (relations[s] < 1 || relations[s] > 4) return GK_ERR_ARG;
        if (relations[s] == 2 && s == n_series - 1) return GK_ERR_ARG;  // ONLAP needs an older series
        P.relations[s] = relations[s];
        P.min_iso[s] = min_iso[s];
        P.max_iso[s] = max_iso[s];
    }
    P.out_values = out_values;
    P.out_ids = out_ids;
    P.masks = masks;
    combine_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(P);
    GK_LAUNCH_CHECK();
    return GK_OK;
}
