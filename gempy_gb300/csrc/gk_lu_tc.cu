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
// Tiles of 128 x 128 of C, walked by one persistent 8-warp CTA per SM.  Per
// tile the CTA stages the 128 x kb slice of the panel (A operand, K-major as
// stored) and the kb x 128 slice of the row block (B operand, transposed to
// K-major while staging), both split into hi/lo, in shared memory in the
// canonical no-swizzle K-major layout: core matrices of 8 rows x 16 bytes (4
// TF32), K-adjacent core matrices 128 bytes apart (LBO), 8-row groups 2048
// bytes apart (SBO, 16 core matrices along K = 64).  One thread issues
// 3 x kb/8 tcgen05.mma (cta_group::1, kind::tf32, M = N = 128, K = 8) into
// one of two 128-column FP32 accumulators in tensor memory and commits them
// to an mbarrier.  While they run, the CTA writes back the previous tile
// (tcgen05.ld of its accumulator, warps w and w + 4 sharing TMEM lanes
// 32 (w % 4) ..) and loads this tile's C and the next tile's operands into
// registers, so loads, MMAs and write-backs of neighbouring tiles overlap.
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
constexpr uint32_t kTmemCols = 2 * kBN;       // two accumulators: MMA of one tile, write-back of the previous
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

// One tile of C: rows [i0, i0 + 128) x columns [j0, j0 + 128), clipped to
// r_hi / c_hi.  Tiles are numbered column tile fastest, then row tile, then
// diagonal block (diag_bs > 0: block z covers [r_lo + z diag_bs, ...) in
// both ranges).
struct Tile {
    int64_t i0, j0, r_hi, c_hi;
};

__device__ __forceinline__ Tile tile_of(int64_t t, int tx, int ty, int64_t r_lo, int64_t r_hi, int64_t c_lo,
                                        int64_t c_hi, int diag_bs) {
    const int64_t per = (int64_t)tx * ty;
    const int64_t z = t / per, rem = t - z * per;
    const int64_t by = rem / tx, bx = rem - by * tx;
    if (diag_bs > 0) {
        const int64_t b0 = r_lo + z * diag_bs;
        r_lo = c_lo = b0;
        r_hi = c_hi = min(r_hi, b0 + diag_bs);
    }
    return {r_lo + by * kBM, c_lo + bx * kBN, r_hi, c_hi};
}

// Persistent: one CTA per SM walks the tiles t = blockIdx.x + i gridDim.x.
// Iteration i: wait for the MMAs of tile i-1 (its operands in shared memory
// are then free and its accumulator readable), store tile i's operands
// (loaded into registers during iteration i-1), issue its MMAs into tensor
// memory buffer i & 1, write back tile i-1 (accumulator from buffer
// (i-1) & 1, C prefetched during iteration i-1), then load tile i's C and
// tile i+1's operands into registers.  The loads of one tile overlap the
// MMAs of the next and the write-back of the previous.
__global__ void __launch_bounds__(kThreads, 1) update_kernel(float* __restrict__ A, int64_t lda, int64_t k, int kb,
                                                             int64_t r_lo, int64_t r_hi, int64_t c_lo, int64_t c_hi,
                                                             int diag_bs, int tx, int ty, int64_t n_tiles,
                                                             gk_info* info) {
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_slot;
    if ((int64_t)blockIdx.x >= n_tiles) return;
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
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_slot;

    float4 va[kAIters];
    float4 vb[kBIters][4];
    float4 cv[kBN / 8];
    // A operand: a quarter-warp takes 8 rows of one 4-column group
    // (conflict-free 16-byte stores), a warp 8 rows x 64 bytes
    auto a_slot = [&](int it, int& row, int& kq) {
        const int e = tid + it * kThreads;
        const int l = e & 31, g = e >> 5;
        row = (l & 7) + 8 * (g % (kBM / 8));
        kq = 4 * ((l >> 3) + 4 * (g / (kBM / 8)));
    };
    // B operand: element (n, p) = A[k + p][j0 + n]; each thread loads 4 x 4
    // blocks (4 rows p, 4 consecutive n) and stores their transposes
    auto b_slot = [&](int it, int& n4, int& p4) {
        const int e = tid + it * kThreads;
        n4 = 4 * (e % (kBN / 4));
        p4 = 4 * (e / (kBN / 4));
    };
    auto load4 = [&](const float* src, int64_t avail) {
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (avail >= 4) {
            v = *reinterpret_cast<const float4*>(src);
        } else {
            if (avail > 0) v.x = src[0];
            if (avail > 1) v.y = src[1];
            if (avail > 2) v.z = src[2];
        }
        return v;
    };
    auto load_ab = [&](const Tile& T) {
#pragma unroll
        for (int it = 0; it < kAIters; ++it) {
            int row, kq;
            a_slot(it, row, kq);
            const int64_t gi = T.i0 + row;
            va[it] = (gi < T.r_hi && kq < kb) ? load4(A + gi * lda + k + kq, kb - kq) : make_float4(0.f, 0.f, 0.f, 0.f);
        }
#pragma unroll
        for (int it = 0; it < kBIters; ++it) {
            int n4, p4;
            b_slot(it, n4, p4);
            const int64_t gj = T.j0 + n4;
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                const int p = p4 + r;
                vb[it][r] = (p < kb && gj < T.c_hi) ? load4(A + (k + p) * lda + gj, T.c_hi - gj)
                                                    : make_float4(0.f, 0.f, 0.f, 0.f);
            }
        }
    };
    auto store_ab = [&]() {
#pragma unroll
        for (int it = 0; it < kAIters; ++it) {
            int row, kq;
            a_slot(it, row, kq);
            if (kq < kp8) store_split(Ah, Al, core_off(row, kq), va[it]);
        }
#pragma unroll
        for (int it = 0; it < kBIters; ++it) {
            int n4, p4;
            b_slot(it, n4, p4);
            if (p4 >= kp8) continue;
            store_split(Bh, Bl, core_off(n4 + 0, p4), make_float4(vb[it][0].x, vb[it][1].x, vb[it][2].x, vb[it][3].x));
            store_split(Bh, Bl, core_off(n4 + 1, p4), make_float4(vb[it][0].y, vb[it][1].y, vb[it][2].y, vb[it][3].y));
            store_split(Bh, Bl, core_off(n4 + 2, p4), make_float4(vb[it][0].z, vb[it][1].z, vb[it][2].z, vb[it][3].z));
            store_split(Bh, Bl, core_off(n4 + 3, p4), make_float4(vb[it][0].w, vb[it][1].w, vb[it][2].w, vb[it][3].w));
        }
    };
    // each thread owns one row of the tile (TMEM lane 32 (w % 4) + lane) and
    // half of its columns (warps 0-3 the first 64, warps 4-7 the last 64)
    const int row = (warp & 3) * 32 + lane;
    const int half = warp >> 2;
    auto load_c = [&](const Tile& T) {
        const int64_t gi = T.i0 + row;
        const int64_t jc = T.j0 + half * (kBN / 2);
#pragma unroll
        for (int q = 0; q < kBN / 8; ++q) {
            const int64_t gj = jc + 4 * q;
            cv[q] = (gi < T.r_hi && gj < T.c_hi) ? load4(A + gi * lda + gj, T.c_hi - gj)
                                                 : make_float4(0.f, 0.f, 0.f, 0.f);
        }
    };
    auto write_back = [&](const Tile& T, uint32_t buf) {
        const uint32_t lanes = tmem + ((uint32_t)((warp & 3) * 32) << 16) + buf * kBN + (uint32_t)(half * (kBN / 2));
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
        const int64_t gi = T.i0 + row;
        if (gi >= T.r_hi) return;
        const int64_t jc = T.j0 + half * (kBN / 2);
#pragma unroll
        for (int q = 0; q < kBN / 8; ++q) {
            const int64_t gj = jc + 4 * q;
            float* c = A + gi * lda + gj;
            if (gj + 3 < T.c_hi) {
                *reinterpret_cast<float4*>(c) = cv[q];
            } else {
                if (gj < T.c_hi) c[0] = cv[q].x;
                if (gj + 1 < T.c_hi) c[1] = cv[q].y;
                if (gj + 2 < T.c_hi) c[2] = cv[q].z;
            }
        }
    };
    // true when the MMAs committed as the it-th arrival have completed
    auto wait_mma = [&](uint32_t it) {
        const long long cap = wait_cap(kCopySpin);
        bool done = false;
        for (long long i = 0; i < cap && !done; ++i) done = mbar_try_wait(&mbar, it & 1u);
        return __syncthreads_or(done ? 0 : 1) == 0;
    };

    Tile cur = tile_of(blockIdx.x, tx, ty, r_lo, r_hi, c_lo, c_hi, diag_bs), prev = cur;
    load_ab(cur);
    uint32_t it = 0;
    bool ok = true;
    for (int64_t t = blockIdx.x; t < n_tiles; t += gridDim.x, ++it) {
        if (it > 0) {
            if (!wait_mma(it - 1)) {
                ok = false;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        }
        store_ab();
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        if (tid == 0) {
            const uint32_t idesc = idesc_tf32(kBM, kBN);
            const uint32_t dst = tmem + (it & 1u) * kBN;
            const uint32_t ops[3][2] = {{saddr(Ah), saddr(Bh)}, {saddr(Ah), saddr(Bl)}, {saddr(Al), saddr(Bh)}};
            uint32_t accumulate = 0;
            for (int pr = 0; pr < 3; ++pr)
                for (int kk = 0; kk < kp8 / 8; ++kk) {
                    const uint64_t ad = smem_desc(ops[pr][0] + (uint32_t)kk * 256u, 128u, kSbo);
                    const uint64_t bd = smem_desc(ops[pr][1] + (uint32_t)kk * 256u, 128u, kSbo);
                    asm volatile(
                        "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
                        " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(dst),
                        "l"(ad), "l"(bd), "r"(idesc), "r"(accumulate)
                        : "memory");
                    accumulate = 1;
                }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             saddr(&mbar))
                         : "memory");
        }
        if (it > 0) write_back(prev, (it - 1) & 1u);
        load_c(cur);
        prev = cur;
        const int64_t nt = t + gridDim.x;
        if (nt < n_tiles) {
            cur = tile_of(nt, tx, ty, r_lo, r_hi, c_lo, c_hi, diag_bs);
            load_ab(cur);
        }
    }
    if (ok) {
        if (wait_mma(it - 1)) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            write_back(prev, (it - 1) & 1u);
        } else {
            ok = false;
        }
    }
    if (!ok) {
        // the MMAs did not signal in time: report, wait once more (default
        // cap) for the commit still outstanding, then release tensor memory
        if (tid == 0) report(info, GK_ERR_TIMEOUT, (int)blockIdx.x);
        for (long long i = 0; i < kCopySpin && !mbar_try_wait(&mbar, (it - 1) & 1u); ++i) {
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

// The FP32 trailing update on the tensor cores: one persistent CTA per SM
// (at most max_ctas when > 0) over the column tiles, row tiles and nz
// diagonal blocks.  A, lda and k + kb are multiples of 4 floats (16-byte
// rows), like the SIMT kernel's fast path.
gk_status lu_tc_update(float* A, int64_t lda, int64_t k, int kb, int64_t r_lo, int64_t r_hi, int64_t c_lo,
                       int64_t c_hi, int diag_bs, unsigned nz, gk_info* info, cudaStream_t st, int max_ctas) {
    if (kb < 1 || kb > lu_tc::kKP) return GK_ERR_ARG;
    const int64_t rows = diag_bs > 0 ? diag_bs : r_hi - r_lo;
    const int64_t cols = diag_bs > 0 ? diag_bs : c_hi - c_lo;
    if (rows <= 0 || cols <= 0) return GK_OK;
    int occ = 0;
    gk_status s = cached_occupancy((const void*)lu_tc::update_kernel, lu_tc::kThreads, lu_tc::kSmemBytes, occ);
    if (s != GK_OK) return s;
    const int tx = (int)((cols + lu_tc::kBN - 1) / lu_tc::kBN), ty = (int)((rows + lu_tc::kBM - 1) / lu_tc::kBM);
    const int64_t n_tiles = (int64_t)tx * ty * (nz < 1 ? 1 : nz);
    int64_t ctas = min(n_tiles, (int64_t)device_sm_count() * occ);
    if (max_ctas > 0) ctas = min(ctas, (int64_t)max_ctas);
    lu_tc::update_kernel<<<(unsigned)ctas, lu_tc::kThreads, lu_tc::kSmemBytes, st>>>(
        A, lda, k, kb, r_lo, r_hi, c_lo, c_hi, diag_bs, tx, ty, n_tiles, info);
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
