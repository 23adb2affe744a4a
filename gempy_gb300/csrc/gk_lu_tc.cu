// FP32 trailing update of the blocked LU on the tensor cores:
//   C[i][j] -= sum_p A[i][k+p] * A[k+p][j],  i in [r_lo, r_hi), j in [c_lo, c_hi),
// p < kb <= 64, the same operation as sgemm_update_kernel (gk_lu.cu) and the
// update of the reference's dense solve (kernel_solver 1, the engine's direct
// solve reached from gempy/API/compute_API.py:68-73).
//
// Precision: three TF32 products ("3xTF32").  Each FP32 operand is split into
// hi = its value with the low 13 mantissa bits cleared (exactly a TF32 number)
// and lo = value - hi (exact in FP32); the tensor core forms
// A_hi B_hi + A_hi B_lo + A_lo B_hi with FP32 accumulation, which drops only
// the A_lo B_lo term (~2^-22 relative) and the TF32 truncation of lo
// (~2^-21 of lo, ~2^-32 of the operand): about FP32 accuracy per update,
// which is what the preconditioner of the mixed solve needs (its FGMRES
// absorbs rounding of that size, as it does the SIMT kernel's).
//
// One CTA of 8 warps per 128 x 128 tile of C.  The CTA stages the tile's
// 128 x kb slice of the panel (A operand, K-major as stored) and the kb x 128
// slice of the row block (B operand, transposed to K-major while staging),
// both split into hi/lo, in shared memory in the canonical no-swizzle K-major
// layout: core matrices of 8 rows x 16 bytes (4 TF32), K-adjacent core
// matrices 128 bytes apart (LBO), 8-row groups 2048 bytes apart (SBO, 16 core
// matrices along K = 64); every thread issues all of its staging loads before
// its first store.  One thread issues 3 x kb/8 tcgen05.mma (cta_group::1,
// kind::tf32, M = N = 128, K = 8) into a 128-column FP32 accumulator in
// tensor memory and commits them to an mbarrier; meanwhile every thread loads
// its 64 entries of C (one row, half the columns).  After the bounded wait
// each warp reads its row's accumulators with tcgen05.ld (warps w and w + 4
// share TMEM lanes 32 (w % 4) ..) and writes C back.
#include <atomic>

#include "gk_common.cuh"

namespace gk {
namespace lu_tc {

constexpr int kBM = 128;
constexpr int kBN = 128;
constexpr int kKP = 64;                        // largest panel width (LuCfg<float>::NB)
constexpr int kThreads = 256;
constexpr int kAIters = kBM * kKP / 4 / kThreads;     // float4 loads of A per thread
constexpr int kBIters = (kBN / 4) * (kKP / 4) / kThreads;  // 4 x 4 blocks of B per thread
constexpr uint32_t kOpBytes = kBM * kKP * 4;   // one operand buffer: 32 KB
constexpr uint32_t kSmemBytes = 4 * kOpBytes;  // A hi, A lo, B hi, B lo
constexpr uint32_t kTmemCols = 128;
constexpr uint32_t kSbo = (kKP / 4) * 128;

__device__ __forceinline__ uint32_t saddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// byte offset of element (row, k) in a K-major operand of kKP columns
__device__ __forceinline__ uint32_t core_off(int row, int k) {
    return (uint32_t)(((row >> 3) * (kKP / 4) + (k >> 2)) * 128 + (row & 7) * 16 + (k & 3) * 4);
}

// shared-memory matrix descriptor: start, LBO, SBO (all >> 4), bit 46 set
// (sm_100 family descriptor), no swizzle
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// instruction descriptor, kind::tf32: D F32 (bits 4-5 = 1), A and B TF32
// (bits 7-9 and 10-12 = 2), both K-major, N >> 3 at bits 17-22, M >> 4 at
// bits 24-28
__host__ __device__ constexpr uint32_t idesc_tf32(int m, int n) {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
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

__device__ __forceinline__ float tf32_hi(float v) { return __uint_as_float(__float_as_uint(v) & 0xFFFFE000u); }

__device__ __forceinline__ void store_split(unsigned char* hi, unsigned char* lo, uint32_t off, float4 v) {
    const float4 h = make_float4(tf32_hi(v.x), tf32_hi(v.y), tf32_hi(v.z), tf32_hi(v.w));
    const float4 l = make_float4(v.x - h.x, v.y - h.y, v.z - h.z, v.w - h.w);
    *reinterpret_cast<float4*>(hi + off) = h;
    *reinterpret_cast<float4*>(lo + off) = l;
}

__global__ void __launch_bounds__(kThreads, 1) update_kernel(float* __restrict__ A, int64_t lda, int64_t k, int kb,
                                                             int64_t r_lo, int64_t r_hi, int64_t c_lo, int64_t c_hi,
                                                             int diag_bs, gk_info* info) {
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_slot;
    if (diag_bs > 0) {
        const int64_t b0 = r_lo + (int64_t)blockIdx.z * diag_bs;
        r_lo = c_lo = b0;
        r_hi = c_hi = min(r_hi, b0 + diag_bs);
    }
    const int64_t i0 = r_lo + (int64_t)blockIdx.y * kBM, j0 = c_lo + (int64_t)blockIdx.x * kBN;
    if (i0 >= r_hi || j0 >= c_hi) return;
    unsigned char* Ah = smem;
    unsigned char* Al = smem + kOpBytes;
    unsigned char* Bh = smem + 2 * kOpBytes;
    unsigned char* Bl = smem + 3 * kOpBytes;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int kp8 = (kb + 7) & ~7;    // K staged (zero-filled past kb), a multiple of the MMA's K

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
    // Every global load of the staging is issued before the first store (8
    // float4 of A and 8 of B per thread in flight), then split and stored.
    // A operand: rows i0.., k columns; a quarter-warp takes 8 rows of one
    // 4-column group (conflict-free 16-byte stores), a warp 8 rows x 64 bytes.
    const int nq = kp8 / 4;                 // 4-column groups staged
    float4 va[kAIters];
#pragma unroll
    for (int it = 0; it < kAIters; ++it) {
        const int e = tid + it * kThreads;
        const int l = e & 31, g = e >> 5;
        const int row = (l & 7) + 8 * (g % (kBM / 8));
        const int kq = 4 * ((l >> 3) + 4 * (g / (kBM / 8)));
        const int64_t gi = i0 + row;
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (gi < r_hi && kq < kb) {
            const float* src = A + gi * lda + k + kq;
            if (kq + 3 < kb) {
                v = *reinterpret_cast<const float4*>(src);
            } else {
                v.x = src[0];
                if (kq + 1 < kb) v.y = src[1];
                if (kq + 2 < kb) v.z = src[2];
            }
        }
        va[it] = v;
    }
    // B operand: element (n, p) = A[k + p][j0 + n], staged K-major: each
    // thread loads 4 x 4 blocks (4 rows p, 4 consecutive n) and stores their
    // transposes as 16-byte rows
    float4 vb[kBIters][4];
#pragma unroll
    for (int it = 0; it < kBIters; ++it) {
        const int e = tid + it * kThreads;
        const int n4 = 4 * (e % (kBN / 4)), p4 = 4 * (e / (kBN / 4));
        const int64_t gj = j0 + n4;
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int p = p4 + r;
            float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
            if (p < kb) {
                const float* src = A + (k + p) * lda + gj;
                if (gj + 3 < c_hi) {
                    v = *reinterpret_cast<const float4*>(src);
                } else {
                    if (gj < c_hi) v.x = src[0];
                    if (gj + 1 < c_hi) v.y = src[1];
                    if (gj + 2 < c_hi) v.z = src[2];
                }
            }
            vb[it][r] = v;
        }
    }
#pragma unroll
    for (int it = 0; it < kAIters; ++it) {
        const int e = tid + it * kThreads;
        const int l = e & 31, g = e >> 5;
        const int row = (l & 7) + 8 * (g % (kBM / 8));
        const int kq = 4 * ((l >> 3) + 4 * (g / (kBM / 8)));
        if (kq < kp8) store_split(Ah, Al, core_off(row, kq), va[it]);
    }
#pragma unroll
    for (int it = 0; it < kBIters; ++it) {
        const int e = tid + it * kThreads;
        const int n4 = 4 * (e % (kBN / 4)), p4 = 4 * (e / (kBN / 4));
        if (p4 >= kp8) continue;
        store_split(Bh, Bl, core_off(n4 + 0, p4), make_float4(vb[it][0].x, vb[it][1].x, vb[it][2].x, vb[it][3].x));
        store_split(Bh, Bl, core_off(n4 + 1, p4), make_float4(vb[it][0].y, vb[it][1].y, vb[it][2].y, vb[it][3].y));
        store_split(Bh, Bl, core_off(n4 + 2, p4), make_float4(vb[it][0].z, vb[it][1].z, vb[it][2].z, vb[it][3].z));
        store_split(Bh, Bl, core_off(n4 + 3, p4), make_float4(vb[it][0].w, vb[it][1].w, vb[it][2].w, vb[it][3].w));
    }
    (void)nq;
    // generic-proxy stores -> visible to the tensor core; the TMEM address
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_slot;
    if (tid == 0) {
        const uint32_t idesc = idesc_tf32(kBM, kBN);
        const uint32_t ops[3][2] = {{saddr(Ah), saddr(Bh)}, {saddr(Ah), saddr(Bl)}, {saddr(Al), saddr(Bh)}};
        uint32_t accumulate = 0;
        for (int pr = 0; pr < 3; ++pr)
            for (int kk = 0; kk < kp8 / 8; ++kk) {
                const uint64_t ad = smem_desc(ops[pr][0] + (uint32_t)kk * 256u, 128u, kSbo);
                const uint64_t bd = smem_desc(ops[pr][1] + (uint32_t)kk * 256u, 128u, kSbo);
                asm volatile(
                    "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
                    " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(idesc), "r"(accumulate)
                    : "memory");
                accumulate = 1;
            }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                         saddr(&mbar))
                     : "memory");
    }
    // While the MMAs run, each thread loads its part of C: warp w holds TMEM
    // lanes 32 (w % 4) .. + 31 (its rows), warps 0-3 columns 0-63, warps 4-7
    // columns 64-127.
    const int row = (warp & 3) * 32 + lane;
    const int half = warp >> 2;
    const int64_t gi = i0 + row;
    const int64_t jc = j0 + half * (kBN / 2);
    float4 cv[kBN / 8];
#pragma unroll
    for (int q = 0; q < kBN / 8; ++q) {
        const int64_t gj = jc + 4 * q;
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (gi < r_hi) {
            const float* c = A + gi * lda + gj;
            if (gj + 3 < c_hi) {
                v = *reinterpret_cast<const float4*>(c);
            } else {
                if (gj < c_hi) v.x = c[0];
                if (gj + 1 < c_hi) v.y = c[1];
                if (gj + 2 < c_hi) v.z = c[2];
            }
        }
        cv[q] = v;
    }
    const long long cap = wait_cap(kCopySpin);
    bool done = false;
    for (long long i = 0; i < cap && !done; ++i) done = mbar_try_wait(&mbar, 0);
    if (__syncthreads_or(done ? 0 : 1)) {
        // the MMAs did not signal in time: report, wait once more (default
        // cap) for anything still in flight, release the tensor memory
        if (tid == 0 && info) atomicExch(&info->status, (int)GK_ERR_TIMEOUT);
        for (long long i = 0; i < kCopySpin && !mbar_try_wait(&mbar, 0); ++i) {
        }
    } else {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t lanes = tmem + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)(half * (kBN / 2));
#pragma unroll
        for (int c0 = 0; c0 < kBN / 2; c0 += 16) {
            uint32_t r[16];
            tmem_ld16(lanes + (uint32_t)c0, r);     // warp-collective: every lane loads
#pragma unroll
            for (int q4 = 0; q4 < 4; ++q4) {
                float4& v = cv[c0 / 4 + q4];
                v.x -= __uint_as_float(r[4 * q4 + 0]);
                v.y -= __uint_as_float(r[4 * q4 + 1]);
                v.z -= __uint_as_float(r[4 * q4 + 2]);
                v.w -= __uint_as_float(r[4 * q4 + 3]);
            }
        }
        if (gi < r_hi) {
#pragma unroll
            for (int q = 0; q < kBN / 8; ++q) {
                const int64_t gj = jc + 4 * q;
                float* c = A + gi * lda + gj;
                if (gj + 3 < c_hi) {
                    *reinterpret_cast<float4*>(c) = cv[q];
                } else {
                    if (gj < c_hi) c[0] = cv[q].x;
                    if (gj + 1 < c_hi) c[1] = cv[q].y;
                    if (gj + 2 < c_hi) c[2] = cv[q].z;
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
}

std::atomic<int> g_engine{GK_LU_UPDATE_TC};

}  // namespace lu_tc

cudaError_t wait_cap_set_lu_tc(long long v) { return set_wait_cap_here(v); }

// Whether the FP32 trailing updates go to the tensor cores.
bool lu_update_on_tensor_cores() { return lu_tc::g_engine.load(std::memory_order_relaxed) == GK_LU_UPDATE_TC; }

// The FP32 trailing update on the tensor cores (grid: column tiles, row
// tiles, nz diagonal blocks).  A, lda and k + kb are multiples of 4 floats
// (16-byte rows), like the SIMT kernel's fast path.
gk_status lu_tc_update(float* A, int64_t lda, int64_t k, int kb, int64_t r_lo, int64_t r_hi, int64_t c_lo,
                       int64_t c_hi, int diag_bs, unsigned nz, gk_info* info, cudaStream_t st) {
    if (kb < 1 || kb > lu_tc::kKP) return GK_ERR_ARG;
    const int64_t rows = diag_bs > 0 ? diag_bs : r_hi - r_lo;
    const int64_t cols = diag_bs > 0 ? diag_bs : c_hi - c_lo;
    if (rows <= 0 || cols <= 0) return GK_OK;
    int occ = 0;
    gk_status s = cached_occupancy((const void*)lu_tc::update_kernel, lu_tc::kThreads, lu_tc::kSmemBytes, occ);
    if (s != GK_OK) return s;
    dim3 grid((unsigned)((cols + lu_tc::kBN - 1) / lu_tc::kBN), (unsigned)((rows + lu_tc::kBM - 1) / lu_tc::kBM),
              nz < 1 ? 1u : nz);
    lu_tc::update_kernel<<<grid, lu_tc::kThreads, lu_tc::kSmemBytes, st>>>(A, lda, k, kb, r_lo, r_hi, c_lo, c_hi,
                                                                          diag_bs, info);
    GK_LAUNCH_CHECK();
    return GK_OK;
}

}  // namespace gk

extern "C" gk_status gk_lu_update_select(int32_t engine) {
    if (engine != GK_LU_UPDATE_SIMT && engine != GK_LU_UPDATE_TC) return GK_ERR_ARG;
    gk::lu_tc::g_engine.store(engine, std::memory_order_relaxed);
    return GK_OK;
}

extern "C" int32_t gk_lu_update_engine(void) { return gk::lu_tc::g_engine.load(std::memory_order_relaxed); }
