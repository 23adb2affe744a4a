// Blocked right-looking LU with partial pivoting (FP64 and FP32), in place on
// a row-major matrix, and the triangular solves that use its factors.
//
// Replaces the engine's dense direct solve (``kernel_solver: 1`` in the
// reference's serialized options, ...serialization.approved.txt:136; the
// engine calls numpy/torch LAPACK getrf/getrs).
//
// Per panel of nb columns starting at k:
//   1. panel_kernel   cooperative launch; CTA c owns a contiguous chunk of
//                     the panel rows in shared memory.  One bounded grid
//                     barrier per column: each CTA publishes its local
//                     pivot candidate (value, row, whole panel row) and the
//                     owner of the diagonal row publishes that row, so after
//                     the barrier every CTA knows the pivot, swaps rows
//                     locally and applies the rank-1 update.
//   2. laswp_kernel   applies the nb row interchanges to the other columns.
//   3. trsm_kernel    U12 = L11^-1 A12 (L11 unit lower, staged in smem).
//   4. gemm_kernel    A22 -= L21 U12 (register-tiled SIMT, smem tiles).
// Solves use a permutation gather and two blocked triangular solves whose
// CTAs claim block rows in order and wait (bounded) on earlier blocks' flags.
#include <cooperative_groups.h>

#include "gk_common.cuh"

namespace gk {

template <typename T> struct LuCfg;
template <> struct LuCfg<double> { static constexpr int NB = 32; };
template <> struct LuCfg<float>  { static constexpr int NB = 64; };

template <typename T>
__device__ __forceinline__ T gabs(T x) { return x < (T)0 ? -x : x; }

// ----------------------------------------------------------------------------
// Panel factorization
// ----------------------------------------------------------------------------
template <typename T, int NB>
struct PanelWork {
    T* cand_val;        // [2][P]
    int* cand_row;      // [2][P]
    T* cand_rows;       // [2][P][NB]
    T* cur_row;         // [2][NB]
    unsigned int* bar;  // [2]
    int* abort;         // [1]
};

template <typename T, int NB>
__global__ void __launch_bounds__(256) panel_kernel(T* __restrict__ A, int64_t lda, int64_t n, int64_t k, int kb,
                                                    int chunk, PanelWork<T, NB> W, int32_t* __restrict__ ipiv,
                                                    gk_info* info) {
    extern __shared__ unsigned char smem_raw[];
    T* S = reinterpret_cast<T*>(smem_raw);  // chunk x NB
    __shared__ T red_v[8];
    __shared__ int red_r[8];
    __shared__ T piv_row[NB];
    __shared__ int s_p;
    __shared__ int s_win;

    const int P = gridDim.x;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int64_t m = n - k;                       // panel rows
    const int64_t rb = (int64_t)blockIdx.x * chunk;  // local row range [rb, re) of the panel
    const int64_t re = min(m, rb + chunk);
    const int nr = (int)max((int64_t)0, re - rb);
    GridBarrier gb{W.bar, W.abort, info};

    // load owned rows
    for (int idx = tid; idx < nr * NB; idx += blockDim.x) {
        int r = idx / NB, c = idx % NB;
        S[idx] = c < kb ? A[(k + rb + r) * lda + k + c] : (T)0;
    }
    __syncthreads();

    for (int j = 0; j < kb; ++j) {
        const int buf = j & 1;
        const int64_t dj = j;  // diagonal row, panel-local
        // publish the current diagonal row (its owner)
        if (dj >= rb && dj < re) {
            for (int c = tid; c < NB; c += blockDim.x) W.cur_row[buf * NB + c] = S[(dj - rb) * NB + c];
        }
        // local argmax of |S[:, j]| over rows >= dj
        T best = (T)-1;
        int brow = -1;
        for (int r = tid; r < nr; r += blockDim.x) {
            int64_t gr = rb + r;
            if (gr < dj) continue;
            T v = gabs(S[r * NB + j]);
            if (v > best || (v == best && brow >= 0 && gr < brow)) { best = v; brow = (int)gr; }
        }
        for (int o = 16; o > 0; o >>= 1) {
            T ov = __shfl_down_sync(0xffffffffu, best, o);
            int orow = __shfl_down_sync(0xffffffffu, brow, o);
            if (ov > best || (ov == best && orow >= 0 && (brow < 0 || orow < brow))) { best = ov; brow = orow; }
        }
        if (lane == 0) { red_v[wid] = best; red_r[wid] = brow; }
        __syncthreads();
        if (tid == 0) {
            for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
                if (red_v[w] > best || (red_v[w] == best && red_r[w] >= 0 && (brow < 0 || red_r[w] < brow))) {
                    best = red_v[w]; brow = red_r[w];
                }
            }
            W.cand_val[buf * P + blockIdx.x] = best;
            W.cand_row[buf * P + blockIdx.x] = brow;
            red_r[0] = brow;
        }
        __syncthreads();
        brow = red_r[0];
        if (brow >= 0) {
            for (int c = tid; c < NB; c += blockDim.x)
                W.cand_rows[((int64_t)buf * P + blockIdx.x) * NB + c] = S[(brow - rb) * NB + c];
        }
        __threadfence();
        if (!gb.sync(P)) return;

        // global pivot
        if (tid < 32) {
            T bv = (T)-1;
            int br = -1, bw = -1;
            for (int c = tid; c < P; c += 32) {
                T v = __ldcg(&W.cand_val[buf * P + c]);
                int r = __ldcg(&W.cand_row[buf * P + c]);
                if (r >= 0 && (v > bv || (v == bv && (br < 0 || r < br)))) { bv = v; br = r; bw = c; }
            }
            for (int o = 16; o > 0; o >>= 1) {
                T ov = __shfl_down_sync(0xffffffffu, bv, o);
                int orr = __shfl_down_sync(0xffffffffu, br, o);
                int ow = __shfl_down_sync(0xffffffffu, bw, o);
                if (orr >= 0 && (ov > bv || (ov == bv && (br < 0 || orr < br)))) { bv = ov; br = orr; bw = ow; }
            }
            if (tid == 0) { s_p = br; s_win = bw; }
        }
        __syncthreads();
        const int p = s_p, win = s_win;
        if (p < 0) {  // only NaN candidates
            if (tid == 0) report(info, GK_ERR_NONFINITE, (int)(k + j));
            if (blockIdx.x == 0 && tid == 0) ipiv[k + j] = (int32_t)(k + j);
            continue;
        }
        for (int c = tid; c < NB; c += blockDim.x) piv_row[c] = __ldcg(&W.cand_rows[((int64_t)buf * P + win) * NB + c]);
        __syncthreads();
        if (blockIdx.x == 0 && tid == 0) ipiv[k + j] = (int32_t)(k + p);
        // swap rows dj <-> p (panel-local)
        if (p != dj) {
            if (p >= rb && p < re)
                for (int c = tid; c < NB; c += blockDim.x) S[(p - rb) * NB + c] = __ldcg(&W.cur_row[buf * NB + c]);
            if (dj >= rb && dj < re)
                for (int c = tid; c < NB; c += blockDim.x) S[(dj - rb) * NB + c] = piv_row[c];
        }
        __syncthreads();
        const T pv = piv_row[j];
        if (pv == (T)0) {
            if (blockIdx.x == 0 && tid == 0) report(info, GK_ERR_SINGULAR, (int)(k + j));
            continue;
        }
        const T inv = (T)1 / pv;
        // rank-1 update of rows below the diagonal: one warp per row
        for (int r = wid; r < nr; r += (int)(blockDim.x >> 5)) {
            int64_t gr = rb + r;
            if (gr <= dj) continue;
            T l = S[r * NB + j] * inv;
            for (int c = j + 1 + lane; c < kb; c += 32) S[r * NB + c] -= l * piv_row[c];
            __syncwarp();
            if (lane == 0) S[r * NB + j] = l;
        }
        __syncthreads();
    }
    // write back
    for (int idx = tid; idx < nr * NB; idx += blockDim.x) {
        int r = idx / NB, c = idx % NB;
        if (c < kb) A[(k + rb + r) * lda + k + c] = S[idx];
    }
}

// ----------------------------------------------------------------------------
// Row interchanges on the columns outside the panel
// ----------------------------------------------------------------------------
template <typename T>
__global__ void laswp_kernel(T* __restrict__ A, int64_t lda, int64_t n, int64_t k, int kb, const int32_t* __restrict__ ipiv) {
    int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    // columns [0, k) and [k + kb, n)
    int64_t left = k, right = n - (k + kb);
    if (c >= left + right) return;
    int64_t col = c < left ? c : c - left + k + kb;
    for (int j = 0; j < kb; ++j) {
        int64_t p = ipiv[k + j];
        int64_t d = k + j;
        if (p != d) {
            T t = A[d * lda + col];
            A[d * lda + col] = A[p * lda + col];
            A[p * lda + col] = t;
        }
    }
}

// ----------------------------------------------------------------------------
// U12 = L11^-1 A12
// ----------------------------------------------------------------------------
template <typename T, int NB>
__global__ void __launch_bounds__(128) trsm_kernel(T* __restrict__ A, int64_t lda, int64_t n, int64_t k, int kb) {
    __shared__ T L[NB][NB + 1];
    for (int idx = threadIdx.x; idx < NB * NB; idx += blockDim.x) {
        int i = idx / NB, j = idx % NB;
        L[i][j] = (i < kb && j < kb) ? A[(k + i) * lda + k + j] : (T)0;
    }
    __syncthreads();
    int64_t col = k + kb + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (col >= n) return;
    T x[NB];
#pragma unroll
    for (int i = 0; i < NB; ++i) x[i] = i < kb ? A[(k + i) * lda + col] : (T)0;
#pragma unroll
    for (int i = 1; i < NB; ++i) {
        T s = x[i];
#pragma unroll
        for (int j = 0; j < i; ++j) s -= L[i][j] * x[j];
        x[i] = s;
    }
#pragma unroll
    for (int i = 0; i < NB; ++i)
        if (i < kb) A[(k + i) * lda + col] = x[i];
}

// ----------------------------------------------------------------------------
// A22 -= L21 U12: C[i][j] -= sum_p A[i][k+p] * A[k+p][j], i, j >= k + kb
// Tile BM x BN per CTA, 16 x 16 threads, TM x TN outputs per thread strided by
// 16 so shared-memory reads of a warp hit consecutive words.
// ----------------------------------------------------------------------------
template <typename T, int BM, int BN, int BK>
__global__ void __launch_bounds__(256) gemm_update_kernel(T* __restrict__ A, int64_t lda, int64_t n, int64_t k, int kb) {
    constexpr int TM = BM / 16, TN = BN / 16;
    __shared__ T As[BK][BM + 1];
    __shared__ T Bs[BK][BN];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int64_t off = k + kb;
    const int64_t i0 = off + (int64_t)blockIdx.y * BM, j0 = off + (int64_t)blockIdx.x * BN;
    T acc[TM][TN];
#pragma unroll
    for (int a = 0; a < TM; ++a)
#pragma unroll
        for (int b = 0; b < TN; ++b) acc[a][b] = (T)0;

    for (int p0 = 0; p0 < kb; p0 += BK) {
        // L tile: rows i0..i0+BM, cols k+p0..k+p0+BK  -> As[p][m]
        for (int idx = threadIdx.x; idx < BM * BK; idx += 256) {
            int m = idx / BK, p = idx % BK;
            int64_t gi = i0 + m;
            As[p][m] = (gi < n && p0 + p < kb) ? A[gi * lda + k + p0 + p] : (T)0;
        }
        // U tile: rows k+p0.., cols j0..j0+BN -> Bs[p][c]
        for (int idx = threadIdx.x; idx < BK * BN; idx += 256) {
            int p = idx / BN, c = idx % BN;
            int64_t gj = j0 + c;
            Bs[p][c] = (gj < n && p0 + p < kb) ? A[(k + p0 + p) * lda + gj] : (T)0;
        }
        __syncthreads();
#pragma unroll
        for (int p = 0; p < BK; ++p) {
            T av[TM], bv[TN];
#pragma unroll
            for (int a = 0; a < TM; ++a) av[a] = As[p][ty + 16 * a];
#pragma unroll
            for (int b = 0; b < TN; ++b) bv[b] = Bs[p][tx + 16 * b];
#pragma unroll
            for (int a = 0; a < TM; ++a)
#pragma unroll
                for (int b = 0; b < TN; ++b) acc[a][b] += av[a] * bv[b];
        }
        __syncthreads();
    }
#pragma unroll
    for (int a = 0; a < TM; ++a) {
        int64_t gi = i0 + ty + 16 * a;
        if (gi >= n) continue;
#pragma unroll
        for (int b = 0; b < TN; ++b) {
            int64_t gj = j0 + tx + 16 * b;
            if (gj < n) A[gi * lda + gj] -= acc[a][b];
        }
    }
}

// ----------------------------------------------------------------------------
// Solves
// ----------------------------------------------------------------------------
// perm[i] = original row placed at position i after all interchanges.  The
// interchanges are sequential by nature; one thread applies them to a
// shared-memory copy (n <= kPermSmem) or to global memory otherwise.
constexpr int kPermSmem = 48 * 1024;
__global__ void perm_from_ipiv_kernel(const int32_t* __restrict__ ipiv, int64_t n, int32_t* __restrict__ perm) {
    extern __shared__ int32_t sp[];
    const bool use_smem = n <= kPermSmem;
    int32_t* q = use_smem ? sp : perm;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) q[i] = (int32_t)i;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int64_t i = 0; i < n; ++i) {
            int64_t p = ipiv[i];
            if (p != i && p >= 0 && p < n) {
                int32_t t = q[i];
                q[i] = q[p];
                q[p] = t;
            }
        }
    }
    __syncthreads();
    if (use_smem)
        for (int64_t i = threadIdx.x; i < n; i += blockDim.x) perm[i] = sp[i];
}

template <typename Tin, typename Tout>
__global__ void gather_kernel(const Tin* __restrict__ src, const int32_t* __restrict__ perm, int64_t n, Tout* __restrict__ dst) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = (Tout)src[perm[i]];
}

// Blocked triangular solve, in place on x.  lower: unit-diagonal L, forward;
// upper: U with diagonal, backward.  CTAs claim block rows in solve order
// through ``counter``; block b waits for every earlier block's flag.
template <typename T, int BS>
__global__ void __launch_bounds__(256) trsv_kernel(const T* __restrict__ A, int64_t lda, int64_t n, T* x,
                                                   int lower, int* counter, int* flags, gk_info* info) {
    __shared__ int s_blk;
    __shared__ T part[8][BS];
    __shared__ T xs[BS];
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int nblk = (int)((n + BS - 1) / BS);
    if (tid == 0) s_blk = atomicAdd(counter, 1);
    __syncthreads();
    const int ord = s_blk;
    if (ord >= nblk) return;
    const int blk = lower ? ord : nblk - 1 - ord;
    const int64_t r0 = (int64_t)blk * BS;
    const int rows = (int)min((int64_t)BS, n - r0);
    // accumulate contributions of solved blocks: warp w handles rows w, w+8, ...
    T acc[BS / 8];
#pragma unroll
    for (int q = 0; q < BS / 8; ++q) acc[q] = (T)0;
    for (int o = 0; o < ord; ++o) {
        const int dep = lower ? o : nblk - 1 - o;
        if (tid == 0) {
            long long spins = 0;
            while (true) {
                int f;
                asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(f) : "l"(flags + dep) : "memory");
                if (f) break;
                if (++spins > kSpinLimit) { report(info, GK_ERR_TIMEOUT, dep); f = -1; break; }
            }
        }
        __syncthreads();
        const int64_t c0 = (int64_t)dep * BS;
        const int cols = (int)min((int64_t)BS, n - c0);
        if (tid < cols) xs[tid] = ((volatile T*)x)[c0 + tid];
        __syncthreads();
#pragma unroll
        for (int q = 0; q < BS / 8; ++q) {
            int r = wid + 8 * q;
            if (r < rows) {
                const T* row = A + (r0 + r) * lda + c0;
                T s = (T)0;
                for (int c = lane; c < cols; c += 32) s += row[c] * xs[c];
                acc[q] += s;
            }
        }
        __syncthreads();
    }
    // reduce per row
#pragma unroll
    for (int q = 0; q < BS / 8; ++q) {
        T s = acc[q];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (lane == 0) part[0][wid + 8 * q] = s;
    }
    __syncthreads();
    // diagonal block solve by warp 0
    if (wid == 0) {
        // load rhs minus contributions
        for (int r = lane; r < rows; r += 32) xs[r] = x[r0 + r] - part[0][r];
        __syncwarp();
        if (lower) {
            for (int r = 0; r < rows; ++r) {
                T s = (T)0;
                for (int c = lane; c < r; c += 32) s += A[(r0 + r) * lda + r0 + c] * xs[c];
                for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
                if (lane == 0) xs[r] -= s;
                __syncwarp();
            }
        } else {
            for (int r = rows - 1; r >= 0; --r) {
                T s = (T)0;
                for (int c = r + 1 + lane; c < rows; c += 32) s += A[(r0 + r) * lda + r0 + c] * xs[c];
                for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
                if (lane == 0) {
                    T d = A[(r0 + r) * lda + r0 + r];
                    if (d == (T)0) { report(info, GK_ERR_SINGULAR, (int)(r0 + r)); xs[r] = (T)0; }
                    else xs[r] = (xs[r] - s) / d;
                }
                __syncwarp();
            }
        }
        for (int r = lane; r < rows; r += 32) x[r0 + r] = xs[r];
        __threadfence();
        __syncwarp();
        if (lane == 0) {
            asm volatile("st.release.gpu.global.b32 [%0], %1;" :: "l"(flags + blk), "r"(1) : "memory");
        }
    }
}

// ----------------------------------------------------------------------------
// host drivers
// ----------------------------------------------------------------------------
static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

template <typename T, int NB>
struct PanelPlan {
    int P, chunk;
    size_t smem;
};

template <typename T, int NB>
static gk_status plan_panel(int64_t m, int sms, PanelPlan<T, NB>& pl) {
    // enough CTAs that each holds <= max_rows panel rows; at least 32 rows each
    const size_t max_smem = 200 * 1024;
    const int max_rows = (int)(max_smem / (NB * sizeof(T)));
    int P = (int)((m + 63) / 64);
    if (P < 1) P = 1;
    if (P > sms) P = sms;
    int chunk = (int)((m + P - 1) / P);
    if (chunk > max_rows) {
        P = (int)((m + max_rows - 1) / max_rows);
        chunk = (int)((m + P - 1) / P);
        if (P > sms) return GK_ERR_SIZE;
    }
    pl.P = P;
    pl.chunk = chunk;
    pl.smem = (size_t)chunk * NB * sizeof(T);
    return GK_OK;
}

template <typename T, int NB>
static size_t panel_ws_bytes(int sms) {
    size_t b = 0;
    b += align256(2 * sms * sizeof(T));
    b += align256(2 * sms * sizeof(int));
    b += align256((size_t)2 * sms * NB * sizeof(T));
    b += align256(2 * NB * sizeof(T));
    b += align256(4 * sizeof(unsigned int));
    return b;
}

template <typename T, int NB>
static PanelWork<T, NB> panel_ws_carve(void* base, int sms) {
    PanelWork<T, NB> w;
    char* p = (char*)base;
    w.cand_val = (T*)p; p += align256(2 * sms * sizeof(T));
    w.cand_row = (int*)p; p += align256(2 * sms * sizeof(int));
    w.cand_rows = (T*)p; p += align256((size_t)2 * sms * NB * sizeof(T));
    w.cur_row = (T*)p; p += align256(2 * NB * sizeof(T));
    w.bar = (unsigned int*)p;
    w.abort = (int*)(w.bar + 2);
    return w;
}

template <typename T>
static size_t lu_ws_bytes(int64_t n) {
    constexpr int NB = LuCfg<T>::NB;
    int sms = device_sm_count();
    return panel_ws_bytes<T, NB>(sms) + align256((size_t)(n + 1) * sizeof(int32_t)) * 2 +
           align256((size_t)((n + 63) / 64 + 2) * sizeof(int)) + align256((size_t)n * sizeof(T));
}

template <typename T>
static gk_status lu_factor(int64_t n, T* A, int64_t lda, int32_t* ipiv, void* work, size_t wbytes, gk_info* info,
                           cudaStream_t st) {
    constexpr int NB = LuCfg<T>::NB;
    if (n <= 0 || A == nullptr || ipiv == nullptr || lda < n) return GK_ERR_ARG;
    if (n > (1LL << 31) - 1) return GK_ERR_SIZE;
    int sms = device_sm_count();
    if (work == nullptr || wbytes < lu_ws_bytes<T>(n)) return GK_ERR_SIZE;
    PanelWork<T, NB> W = panel_ws_carve<T, NB>(work, sms);
    GK_CUDA_TRY(cudaMemsetAsync(W.bar, 0, 4 * sizeof(unsigned int), st));
    if (info) GK_CUDA_TRY(cudaMemsetAsync(info, 0, sizeof(gk_info), st));
    auto pk = panel_kernel<T, NB>;
    GK_CUDA_TRY(cudaFuncSetAttribute(pk, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    for (int64_t k = 0; k < n; k += NB) {
        int kb = (int)min((int64_t)NB, n - k);
        PanelPlan<T, NB> pl;
        gk_status s = plan_panel<T, NB>(n - k, sms, pl);
        if (s != GK_OK) return s;
        int occ = 0;
        GK_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, pk, 256, pl.smem));
        if (occ < 1 || pl.P > occ * sms) return GK_ERR_SIZE;
        int64_t kk = k;
        int chunk = pl.chunk;
        void* args[] = {&A, &lda, &n, &kk, &kb, &chunk, &W, &ipiv, &info};
        GK_CUDA_TRY(cudaLaunchCooperativeKernel((void*)pk, dim3(pl.P), dim3(256), args, pl.smem, st));
        gk_launch_counter().fetch_add(1, std::memory_order_relaxed);
        int64_t others = n - kb;
        if (others > 0) {
            laswp_kernel<T><<<(unsigned)((others + 255) / 256), 256, 0, st>>>(A, lda, n, k, kb, ipiv);
            GK_LAUNCH_CHECK();
        }
        int64_t rest = n - k - kb;
        if (rest > 0) {
            trsm_kernel<T, NB><<<(unsigned)((rest + 127) / 128), 128, 0, st>>>(A, lda, n, k, kb);
            GK_LAUNCH_CHECK();
            constexpr int BM = sizeof(T) == 8 ? 64 : 128;
            constexpr int BN = BM;
            dim3 grid((unsigned)((rest + BN - 1) / BN), (unsigned)((rest + BM - 1) / BM));
            gemm_update_kernel<T, BM, BN, 16><<<grid, 256, 0, st>>>(A, lda, n, k, kb);
            GK_LAUNCH_CHECK();
        }
    }
    // row permutation for the solves, kept in the workspace
    int32_t* perm = (int32_t*)((char*)work + panel_ws_bytes<T, NB>(sms));
    size_t psmem = n <= kPermSmem ? (size_t)n * sizeof(int32_t) : 0;
    GK_CUDA_TRY(cudaFuncSetAttribute(perm_from_ipiv_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kPermSmem * 4));
    perm_from_ipiv_kernel<<<1, 256, psmem, st>>>(ipiv, n, perm);
    GK_LAUNCH_CHECK();
    return GK_OK;
}

// Solve with the factors.  ``work`` is the workspace of the factorization:
// after the panel area it holds perm (n+1, written by lu_factor), then the
// block flags + claim counter, then a temporary vector.  ``b`` is overwritten.
template <typename T>
static gk_status lu_solve(int64_t n, const T* LU, int64_t lda, const int32_t* ipiv, T* b, void* work, size_t wbytes,
                          gk_info* info, cudaStream_t st) {
    constexpr int NB = LuCfg<T>::NB;
    constexpr int BS = 64;
    if (n <= 0 || LU == nullptr || ipiv == nullptr || b == nullptr) return GK_ERR_ARG;
    if (work == nullptr || wbytes < lu_ws_bytes<T>(n)) return GK_ERR_SIZE;
    int sms = device_sm_count();
    char* p = (char*)work + panel_ws_bytes<T, NB>(sms);
    int32_t* perm = (int32_t*)p; p += align256((size_t)(n + 1) * sizeof(int32_t)) * 2;
    int nblk = (int)((n + BS - 1) / BS);
    int* flags = (int*)p; p += align256((size_t)((n + 63) / 64 + 2) * sizeof(int));
    T* tmp = (T*)p;
    gather_kernel<T, T><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(b, perm, n, tmp);
    GK_LAUNCH_CHECK();
    int* counter = flags + nblk;
    for (int pass = 0; pass < 2; ++pass) {
        GK_CUDA_TRY(cudaMemsetAsync(flags, 0, (nblk + 1) * sizeof(int), st));
        // one CTA per block row; CTAs claim rows in solve order, so a CTA only
        // ever waits on rows claimed by CTAs that are already running
        trsv_kernel<T, BS><<<nblk, 256, 0, st>>>(LU, lda, n, tmp, pass == 0 ? 1 : 0, counter, flags, info);
        GK_LAUNCH_CHECK();
    }
    GK_CUDA_TRY(cudaMemcpyAsync(b, tmp, n * sizeof(T), cudaMemcpyDeviceToDevice, st));
    return GK_OK;
}

}  // namespace gk

using namespace gk;

extern "C" size_t gk_lu_workspace_bytes(gk_prec prec, int64_t n) {
    if (n <= 0) return 0;
    return prec == GK_F64 ? lu_ws_bytes<double>(n) : lu_ws_bytes<float>(n);
}

extern "C" gk_status gk_lu_factor(gk_prec prec, int64_t n, void* A, int64_t lda, int32_t* ipiv, void* work,
                                  size_t work_bytes, gk_info* info, gk_stream stream) {
    cudaStream_t st = (cudaStream_t)stream;
    if (prec == GK_F64) return lu_factor<double>(n, (double*)A, lda, ipiv, work, work_bytes, info, st);
    if (prec == GK_F32) return lu_factor<float>(n, (float*)A, lda, ipiv, work, work_bytes, info, st);
    return GK_ERR_ARG;
}

extern "C" gk_status gk_lu_solve(gk_prec prec, int64_t n, const void* LU, int64_t lda, const int32_t* ipiv, void* b,
                                 void* work, size_t work_bytes, gk_info* info, gk_stream stream) {
    cudaStream_t st = (cudaStream_t)stream;
    if (prec == GK_F64) return lu_solve<double>(n, (const double*)LU, lda, ipiv, (double*)b, work, work_bytes, info, st);
    if (prec == GK_F32) return lu_solve<float>(n, (const float*)LU, lda, ipiv, (float*)b, work, work_bytes, info, st);
    return GK_ERR_ARG;
}

// Internal entry points used by the mixed solver (same translation unit set).
gk_status gk_internal_lu_factor_f32(int64_t n, float* A, int64_t lda, int32_t* ipiv, void* work, size_t wb,
                                    gk_info* info, cudaStream_t st) {
    return lu_factor<float>(n, A, lda, ipiv, work, wb, info, st);
}
gk_status gk_internal_lu_solve_f32(int64_t n, const float* LU, int64_t lda, const int32_t* ipiv, float* b, void* work,
                                   size_t wb, gk_info* info, cudaStream_t st) {
    return lu_solve<float>(n, LU, lda, ipiv, b, work, wb, info, st);
}
size_t gk_internal_lu_ws_f32(int64_t n) { return lu_ws_bytes<float>(n); }
