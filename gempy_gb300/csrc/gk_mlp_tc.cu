// Tensor-core inference pass of the preconditioner-choice network: the same
// in_dim -> 256 -> 256 -> out_dim perceptron as gk_mlp.cu, with every layer
// one tcgen05.mma chain (kind::f16, BF16 x BF16 -> FP32 accumulators in
// tensor memory).  The activations between layers are rounded to BF16 (the
// tensor-core operand type); the training path (gk_mlp_fwd / gk_mlp_bwd)
// keeps them in FP32.
//
// One CTA of 4 warps handles 128 samples (the MMA's M; sample m is TMEM lane
// m).  Per layer the CTA stages its operands in shared memory in the
// canonical no-swizzle K-major layout -- "core matrices" of 8 rows x 16 bytes,
// the 8-row groups of a row block SBO bytes apart and the K-adjacent core
// matrices LBO = 128 bytes apart -- one thread issues the K/16 MMAs and a
// tcgen05.commit to an mbarrier, and after the (bounded) wait every warp reads
// its 32 TMEM lanes back with tcgen05.ld, applies ReLU and writes the next
// layer's A operand (or the FP32 output).  The bias rides along as an extra
// input column of ones, as in the parameter layout.
#include <cuda_bf16.h>

#include "gk_common.cuh"

namespace gk {
namespace mlp_tc {

constexpr int kM = 128;         // samples per CTA = TMEM lanes used
constexpr int kN = GK_MLP_HIDDEN;
constexpr int kKmax = 272;      // 256 activations + bias column, padded to a multiple of 16
constexpr int kThreads = 128;   // warp w owns TMEM lanes [32 w, 32 w + 32)
constexpr uint32_t kABytes = kM * kKmax * 2;
constexpr uint32_t kBBytes = kN * kKmax * 2;
constexpr uint32_t kSmemBytes = kABytes + kBBytes;
constexpr uint32_t kTmemCols = 512;  // the whole tensor memory of the SM (one CTA per SM)
constexpr long long kSpin = 4LL * 1000 * 1000;

__host__ __device__ inline int pad16(int k) { return (k + 15) / 16 * 16; }

__device__ __forceinline__ uint32_t saddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Byte offset of element (row, k) of a K-major operand with kp (padded) columns.
__device__ __forceinline__ uint32_t core_off(int row, int k, int kp) {
    return (uint32_t)(((row >> 3) * (kp >> 3) + (k >> 3)) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

// Shared-memory matrix descriptor: start address, leading (K) and stride
// (M/N) byte offsets, all >> 4; bit 46 set (descriptor version of sm_100
// family); base offset 0, relative LBO mode, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor, kind::f16: D F32 (bits 4-5 = 1), A and B BF16
// (bits 7-9, 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 at bits
// 17-22, M >> 4 at bits 24-28.
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(saddr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t* r) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void put_bf16(unsigned char* base, uint32_t off, float v) {
    *reinterpret_cast<__nv_bfloat16*>(base + off) = __float2bfloat16_rn(v);
}

__global__ void __launch_bounds__(kThreads, 1) fwd_kernel(const __nv_bfloat16* __restrict__ P, int F, int O,
                                                          int64_t B, const float* __restrict__ x,
                                                          float* __restrict__ y, int* __restrict__ err) {
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_slot;
    unsigned char* As = smem;
    unsigned char* Bs = smem + kABytes;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int64_t m0 = (int64_t)blockIdx.x * kM;

    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(saddr(&mbar)), "r"(1) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(saddr(&tmem_slot)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    // layer-0 A operand: the samples, a ones column at F, zeros up to the padded
    // width; one 16-byte core-matrix row (8 consecutive k) per store
    const int k1p = pad16(F + 1);
    for (int e = tid; e < kM * (k1p / 8); e += kThreads) {
        const int row = e / (k1p / 8), k0 = (e % (k1p / 8)) * 8;
        __align__(16) __nv_bfloat16 v[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int k = k0 + j;
            float f = 0.f;
            if (m0 + row < B) f = k < F ? x[(m0 + row) * F + k] : (k == F ? 1.f : 0.f);
            v[j] = __float2bfloat16_rn(f);
        }
        *reinterpret_cast<uint4*>(As + core_off(row, k0, k1p)) = *reinterpret_cast<const uint4*>(v);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_slot;

    int64_t off = 0;
    int kin = F;
    uint32_t phase = 0;
    for (int L = 0; L < 3; ++L) {
        const int nout = L == 2 ? O : kN;
        const int np = L == 2 ? 16 : kN;  // MMA N: a multiple of 16, at least 16
        const int kp = pad16(kin + 1);
        const __nv_bfloat16* W = P + off;
        for (int e = tid; e < np * (kp / 8); e += kThreads) {
            const int n = e / (kp / 8), k0 = (e % (kp / 8)) * 8;
            __align__(16) __nv_bfloat16 v[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int k = k0 + j;
                v[j] = (n < nout && k <= kin) ? W[(int64_t)n * (kin + 1) + k] : __float2bfloat16_rn(0.f);
            }
            *reinterpret_cast<uint4*>(Bs + core_off(n, k0, kp)) = *reinterpret_cast<const uint4*>(v);
        }
        off += (int64_t)nout * (kin + 1);
        // generic-proxy writes of the operands -> visible to the tensor core
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        if (tid == 0) {
            const uint32_t a0 = saddr(As), b0 = saddr(Bs);
            const uint32_t sbo = (uint32_t)(kp / 8) * 128u;
            const uint32_t idesc = idesc_bf16(kM, np);
            for (int kk = 0; kk < kp / 16; ++kk) {
                const uint64_t ad = smem_desc(a0 + (uint32_t)kk * 256u, 128u, sbo);
                const uint64_t bd = smem_desc(b0 + (uint32_t)kk * 256u, 128u, sbo);
                const uint32_t accumulate = kk > 0 ? 1u : 0u;
                asm volatile(
                    "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
                    " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(idesc), "r"(accumulate)
                    : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             saddr(&mbar))
                         : "memory");
        }
        bool done = false;
        for (long long i = 0; i < kSpin && !done; ++i) done = mbar_try_wait(&mbar, phase);
        phase ^= 1u;
        if (__syncthreads_or(done ? 0 : 1)) {
            // the MMAs did not signal in time: report, wait once more (bounded)
            // for anything still in flight, release the tensor memory and leave
            if (tid == 0 && err) atomicExch(err, GK_ERR_TIMEOUT);
            for (long long i = 0; i < kSpin && !mbar_try_wait(&mbar, phase ^ 1u); ++i) {
            }
            break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const int row = warp * 32 + lane;
        const uint32_t lanes = tmem + ((uint32_t)(warp * 32) << 16);
        if (L < 2) {
            for (int c0 = 0; c0 < kN; c0 += 16) {
                uint32_t r[16];
                tmem_ld16(lanes + (uint32_t)c0, r);
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    __align__(16) __nv_bfloat16 v[8];
#pragma unroll
                    for (int j = 0; j < 8; ++j) v[j] = __float2bfloat16_rn(fmaxf(__uint_as_float(r[8 * h + j]), 0.f));
                    *reinterpret_cast<uint4*>(As + core_off(row, c0 + 8 * h, kKmax)) =
                        *reinterpret_cast<const uint4*>(v);
                }
            }
            for (int k = kN; k < kKmax; ++k) put_bf16(As, core_off(row, k, kKmax), k == kN ? 1.f : 0.f);
        } else {
            uint32_t r[16];
            tmem_ld16(lanes, r);
            if (m0 + row < B)
                for (int j = 0; j < O; ++j) y[(m0 + row) * O + j] = __uint_as_float(r[j]);
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
        kin = kN;
    }
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
}

}  // namespace mlp_tc
}  // namespace gk

using namespace gk;

extern "C" gk_status gk_mlp_fwd_tc(const gk_mlp* net, int64_t batch, const float* x, float* y, int32_t* err,
                                   gk_stream stream) {
    if (net == nullptr || net->params == nullptr || x == nullptr || y == nullptr) return GK_ERR_ARG;
    if (net->in_dim < 1 || net->in_dim > GK_MLP_MAX_IN || net->out_dim < 1 || net->out_dim > GK_MLP_MAX_OUT)
        return GK_ERR_ARG;
    if (batch < 1 || batch > GK_MLP_MAX_BATCH) return GK_ERR_SIZE;
    auto k = mlp_tc::fwd_kernel;
    GK_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)mlp_tc::kSmemBytes));
    const unsigned grid = (unsigned)((batch + mlp_tc::kM - 1) / mlp_tc::kM);
    k<<<grid, mlp_tc::kThreads, mlp_tc::kSmemBytes, (cudaStream_t)stream>>>(
        reinterpret_cast<const __nv_bfloat16*>(net->params), net->in_dim, net->out_dim, batch, x, y, err);
    GK_LAUNCH_CHECK();
    return GK_OK;
}
