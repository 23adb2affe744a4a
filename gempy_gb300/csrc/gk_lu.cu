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
#include <cstdlib>

#include "gk_common.cuh"
#include "gk_cta.cuh"

namespace gk {

template <typename T> struct LuCfg;
template <> struct LuCfg<double> { static constexpr int NB = 32; };
template <> struct LuCfg<float>  { static constexpr int NB = 64; };

template <typename T>
__device__ __forceinline__ T gabs(T x) { return x < (T)0 ? -x : x; }

// Rank-1 update of the panel rows below the diagonal, parallel over
// (row, column): first the multipliers l_r = S[r][j] / pivot are written in
// place, then every thread updates elements S[r][c], c > j.
template <typename T, int NB>
__device__ __forceinline__ void rank1_update(T* S, int nr, int64_t rb, int64_t dj, int j, int kb, T inv,
                                             const T* piv_row) {
    constexpr int SP = NB + 1;  // padded row stride: column accesses hit distinct banks
    const int r_first = (int)max((int64_t)0, dj + 1 - rb);
    for (int r = r_first + (int)threadIdx.x; r < nr; r += blockDim.x) S[r * SP + j] *= inv;
    __syncthreads();
    const int w = kb - j - 1;
    if (w > 0) {
        // w threads per row, rows_par rows at a time: one division per thread
        const int rows_par = (int)blockDim.x / w;
        const int t = (int)threadIdx.x;
        if (t < rows_par * w) {
            const int c = j + 1 + t % w;
            const T pc = piv_row[c];
            for (int r = r_first + t / w; r < nr; r += rows_par) S[r * SP + c] -= S[r * SP + j] * pc;
        }
    }
    __syncthreads();
}

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
    T* S = reinterpret_cast<T*>(smem_raw);  // chunk x (NB + 1)
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
        S[r * (NB + 1) + c] = c < kb ? A[(k + rb + r) * lda + k + c] : (T)0;
    }
    __syncthreads();

    for (int j = 0; j < kb; ++j) {
        const int buf = j & 1;
        const int64_t dj = j;  // diagonal row, panel-local
        // publish the current diagonal row (its owner)
        if (dj >= rb && dj < re) {
            for (int c = tid; c < NB; c += blockDim.x) W.cur_row[buf * NB + c] = S[(dj - rb) * (NB + 1) + c];
        }
        // local argmax of |S[:, j]| over rows >= dj
        T best = (T)-1;
        int brow = -1;
        for (int r = tid; r < nr; r += blockDim.x) {
            int64_t gr = rb + r;
            if (gr < dj) continue;
            T v = gabs(S[r * (NB + 1) + j]);
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
                W.cand_rows[((int64_t)buf * P + blockIdx.x) * NB + c] = S[(brow - rb) * (NB + 1) + c];
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
                for (int c = tid; c < NB; c += blockDim.x) S[(p - rb) * (NB + 1) + c] = __ldcg(&W.cur_row[buf * NB + c]);
            if (dj >= rb && dj < re)
                for (int c = tid; c < NB; c += blockDim.x) S[(dj - rb) * (NB + 1) + c] = piv_row[c];
        }
        __syncthreads();
        const T pv = piv_row[j];
        if (pv == (T)0) {
            if (blockIdx.x == 0 && tid == 0) report(info, GK_ERR_SINGULAR, (int)(k + j));
            continue;
        }
        const T inv = (T)1 / pv;
        rank1_update<T, NB>(S, nr, rb, dj, j, kb, inv, piv_row);
    }
    // write back
    for (int idx = tid; idx < nr * NB; idx += blockDim.x) {
        int r = idx / NB, c = idx % NB;
        if (c < kb) A[(k + rb + r) * lda + k + c] = S[r * (NB + 1) + c];
    }
}

// ----------------------------------------------------------------------------
// Panel factorization inside one thread-block cluster (<= 16 CTAs).  Each CTA
// holds a contiguous chunk of the panel rows in shared memory.  Per column,
// every CTA posts its pivot candidate (value, row, and a copy of the whole
// panel row) and the owner of the diagonal row posts that row in its own
// shared-memory mailbox; after one hardware cluster barrier all CTAs read the
// mailboxes through distributed shared memory, agree on the pivot (largest
// magnitude, lowest row on ties), swap locally and apply the rank-1 update.
// Mailboxes alternate by column parity, so a mailbox is only rewritten after
// the next barrier, when every reader is done with it.
// ----------------------------------------------------------------------------
namespace cg = cooperative_groups;

template <typename T, int NB>
__global__ void __launch_bounds__(256) panel_cluster_kernel(T* __restrict__ A, int64_t lda, int64_t n, int64_t k,
                                                            int kb, int chunk, int32_t* __restrict__ ipiv,
                                                            gk_info* info) {
    extern __shared__ unsigned char smem_raw[];
    T* S = reinterpret_cast<T*>(smem_raw);  // chunk x (NB + 1)
    __shared__ T mb_val[2];
    __shared__ int mb_row[2];
    __shared__ T mb_rowdata[2][NB];
    __shared__ T mb_cur[2][NB];
    __shared__ T red_v[8];
    __shared__ int red_r[8];
    __shared__ T piv_row[NB];
    __shared__ T cur_row[NB];
    __shared__ int s_p, s_win;

    cg::cluster_group cl = cg::this_cluster();
    const int C = (int)cl.num_blocks();
    const int me = (int)cl.block_rank();
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int64_t m = n - k;
    const int64_t rb = (int64_t)me * chunk;
    const int64_t re = min(m, rb + chunk);
    const int nr = (int)max((int64_t)0, re - rb);

    for (int idx = tid; idx < nr * NB; idx += blockDim.x) {
        int r = idx / NB, c = idx % NB;
        S[r * (NB + 1) + c] = c < kb ? A[(k + rb + r) * lda + k + c] : (T)0;
    }
    __syncthreads();

    for (int j = 0; j < kb; ++j) {
        const int buf = j & 1;
        const int64_t dj = j;
        if (dj >= rb && dj < re)
            for (int c = tid; c < NB; c += blockDim.x) mb_cur[buf][c] = S[(dj - rb) * (NB + 1) + c];
        T best = (T)-1;
        int brow = -1;
        for (int r = tid; r < nr; r += blockDim.x) {
            int64_t gr = rb + r;
            if (gr < dj) continue;
            T v = gabs(S[r * (NB + 1) + j]);
            if (v > best) { best = v; brow = (int)gr; }
        }
        for (int o = 16; o > 0; o >>= 1) {
            T ov = __shfl_down_sync(0xffffffffu, best, o);
            int orow = __shfl_down_sync(0xffffffffu, brow, o);
            if (orow >= 0 && (ov > best || (ov == best && (brow < 0 || orow < brow)))) { best = ov; brow = orow; }
        }
        if (lane == 0) { red_v[wid] = best; red_r[wid] = brow; }
        __syncthreads();
        if (tid == 0) {
            for (int w = 1; w < (int)(blockDim.x >> 5); ++w)
                if (red_r[w] >= 0 && (red_v[w] > best || (red_v[w] == best && (brow < 0 || red_r[w] < brow)))) {
                    best = red_v[w]; brow = red_r[w];
                }
            mb_val[buf] = best;
            mb_row[buf] = brow;
            red_r[0] = brow;
        }
        __syncthreads();
        brow = red_r[0];
        if (brow >= 0)
            for (int c = tid; c < NB; c += blockDim.x) mb_rowdata[buf][c] = S[(brow - rb) * (NB + 1) + c];
        cl.sync();

        if (tid < 32) {
            T bv = (T)-1;
            int br = -1, bw = -1;
            for (int c = tid; c < C; c += 32) {
                T v = *cl.map_shared_rank(&mb_val[buf], c);
                int r = *cl.map_shared_rank(&mb_row[buf], c);
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
        if (p < 0) {
            if (tid == 0) report(info, GK_ERR_NONFINITE, (int)(k + j));
            if (me == 0 && tid == 0) ipiv[k + j] = (int32_t)(k + j);
            continue;
        }
        const T* wrow = cl.map_shared_rank(&mb_rowdata[buf][0], win);
        const int owner_dj = (int)(dj / chunk);
        const T* crow = cl.map_shared_rank(&mb_cur[buf][0], owner_dj);
        for (int c = tid; c < NB; c += blockDim.x) {
            piv_row[c] = wrow[c];
            cur_row[c] = crow[c];
        }
        __syncthreads();
        if (me == 0 && tid == 0) ipiv[k + j] = (int32_t)(k + p);
        if (p != dj) {
            if (p >= rb && p < re)
                for (int c = tid; c < NB; c += blockDim.x) S[(p - rb) * (NB + 1) + c] = cur_row[c];
            if (dj >= rb && dj < re)
                for (int c = tid; c < NB; c += blockDim.x) S[(dj - rb) * (NB + 1) + c] = piv_row[c];
        }
        __syncthreads();
        const T pv = piv_row[j];
        if (pv == (T)0) {
            if (me == 0 && tid == 0) report(info, GK_ERR_SINGULAR, (int)(k + j));
            continue;
        }
        const T inv = (T)1 / pv;
        rank1_update<T, NB>(S, nr, rb, dj, j, kb, inv, piv_row);
    }
    // keep every CTA's mailboxes alive until all remote reads are done
    cl.sync();
    for (int idx = tid; idx < nr * NB; idx += blockDim.x) {
        int r = idx / NB, c = idx % NB;
        if (c < kb) A[(k + rb + r) * lda + k + c] = S[r * (NB + 1) + c];
    }
}

// ----------------------------------------------------------------------------
// LU without pivoting (preconditioner factorization of the mixed solve).
// After symmetric equilibration the covariance block of the kriging matrix is
// SPD with unit diagonal, so the natural order (covariance unknowns first,
// drift last) has non-zero pivots; the drift rows end with negative pivots
// of the Schur complement.  No pivot search means no inter-CTA exchange:
// per panel one CTA factors the diagonal block, L21 = A21 U11^-1 and
// U12 = L11^-1 A12 are row/column parallel, then the trailing GEMM.
// A zero or non-finite pivot is reported as GK_ERR_SINGULAR so the caller can
// fall back to partial pivoting.
// ----------------------------------------------------------------------------
template <typename T, int NB>
__global__ void __launch_bounds__(256) diag_lu_kernel(T* __restrict__ A, int64_t lda, int64_t k, int kb,
                                                      int32_t* __restrict__ ipiv, gk_info* info,
                                                      T* __restrict__ uinv = nullptr) {
    __shared__ T S[NB][NB + 1];
    const int tid = threadIdx.x;
    for (int idx = tid; idx < NB * NB; idx += blockDim.x) {
        int r = idx / NB, c = idx % NB;
        S[r][c] = (r < kb && c < kb) ? A[(k + r) * lda + k + c] : (T)0;
    }
    if (tid < kb) ipiv[k + tid] = (int32_t)(k + tid);
    __syncthreads();
    // Right-looking sweep with one barrier per step: the multipliers are used
    // unscaled (S[i][j] * inv on the fly) and column j, which no later step
    // reads, is scaled in one pass after the sweep.
    int steps = kb;
    for (int j = 0; j < kb; ++j) {
        const T pv = S[j][j];
        const bool bad = !(pv == pv) || pv == (T)0 || !(gabs(pv) < (T)INFINITY);
        if (bad) {
            if (tid == 0) report(info, GK_ERR_SINGULAR, (int)(k + j));
            steps = j;
            break;  // uniform: every thread sees the same pivot
        }
        const T inv = (T)1 / pv;
        const int w = kb - j - 1;
        for (int idx = tid; idx < w * w; idx += blockDim.x) {
            const int i = j + 1 + idx / w, c = j + 1 + idx % w;
            S[i][c] -= (S[i][j] * inv) * S[j][c];
        }
        __syncthreads();
    }
    for (int idx = tid; idx < NB * NB; idx += blockDim.x) {
        const int i = idx / NB, j = idx % NB;
        if (j < steps && i > j && i < kb) S[i][j] *= (T)1 / S[j][j];  // the same rounding as inv above
    }
    __syncthreads();
    for (int idx = tid; idx < NB * NB; idx += blockDim.x) {
        int r = idx / NB, c = idx % NB;
        if (r < kb && c < kb) A[(k + r) * lda + k + c] = S[r][c];
    }
    // U11^-1 (row-major NB x NB, zero below the diagonal) for the
    // right-looking triangular solve L21 = A21 U11^-1: thread c back-
    // substitutes column c with the column held in registers (rows below c
    // come out zero); only for full panels that factored without a bad pivot
    if (uinv == nullptr || kb != NB || steps != kb) return;
    if (tid < NB) {
        const int c = tid;
        T x[NB];
#pragma unroll
        for (int i = NB - 1; i >= 0; --i) {
            T s = (i == c) ? (T)1 : (T)0;
#pragma unroll
            for (int j = i + 1; j < NB; ++j) s -= S[i][j] * x[j];
            x[i] = s / S[i][i];
        }
#pragma unroll
        for (int i = 0; i < NB; ++i) uinv[i * NB + c] = x[i];
    }
}

// L21 = A21 U11^-1 with the explicit inverse from diag_lu_kernel: 64 rows per
// CTA, four threads per row, 16 output columns each (upper-triangular
// inverse: column c sums over rows j <= c).  A full panel (kb = NB) only.
template <typename T, int NB>
__global__ void __launch_bounds__(256) trsm_right_inv_kernel(T* __restrict__ A, int64_t lda, int64_t n, int64_t k,
                                                             const T* __restrict__ uinv) {
    __shared__ T U[NB][NB + 1];
    __shared__ T X[64][NB + 1];
    const int tid = threadIdx.x;
    for (int idx = tid; idx < NB * NB; idx += 256) U[idx / NB][idx % NB] = uinv[idx];
    const int64_t row0 = k + NB + (int64_t)blockIdx.x * 64;
    for (int idx = tid; idx < 64 * NB; idx += 256) {
        const int r = idx / NB, c = idx % NB;
        const int64_t gr = row0 + r;
        X[r][c] = gr < n ? A[gr * lda + k + c] : (T)0;
    }
    __syncthreads();
    const int r = tid >> 2, c0 = (tid & 3) * (NB / 4);
    const int64_t gr = row0 + r;
    if (gr >= n) return;
    T out[NB / 4];
#pragma unroll
    for (int q = 0; q < NB / 4; ++q) out[q] = (T)0;
    for (int j = 0; j < c0 + NB / 4; ++j) {
        const T xj = X[r][j];
#pragma unroll
        for (int q = 0; q < NB / 4; ++q)
            if (j <= c0 + q) out[q] += xj * U[j][c0 + q];
    }
#pragma unroll
    for (int q = 0; q < NB / 4; ++q) A[gr * lda + k + c0 + q] = out[q];
}

// L21 = A21 U11^-1: rows r >= k + kb, 64 rows per CTA staged in shared memory.
// Four threads share a row: for each column j they split the dot product over
// the earlier columns, combine it with two shuffles and the row's first lane
// finishes x_j, so the sequential chain per row is a quarter as long as with
// one thread per row.
constexpr int kTrsmRows = 64, kTrsmLanes = 4;

template <typename T, int NB>
__global__ void __launch_bounds__(kTrsmRows * kTrsmLanes) trsm_right_kernel(T* __restrict__ A, int64_t lda,
                                                                            int64_t n, int64_t k, int kb) {
    __shared__ T U[NB][NB + 1];
    __shared__ T X[kTrsmRows][NB + 1];  // X[row][c]
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int idx = tid; idx < NB * NB; idx += nt) {
        const int r = idx / NB, c = idx % NB;
        U[r][c] = (r < kb && c < kb) ? A[(k + r) * lda + k + c] : (T)0;
    }
    const int64_t row0 = k + kb + (int64_t)blockIdx.x * kTrsmRows;
    for (int idx = tid; idx < kTrsmRows * NB; idx += nt) {
        const int r = idx / NB, c = idx % NB;
        const int64_t gr = row0 + r;
        X[r][c] = (gr < n && c < kb) ? A[gr * lda + k + c] : (T)0;
    }
    __syncthreads();
    const int r = tid / kTrsmLanes, part = tid % kTrsmLanes;
    for (int j = 0; j < kb; ++j) {
        T s = (T)0;
        for (int i = part; i < j; i += kTrsmLanes) s += X[r][i] * U[i][j];
        s += __shfl_xor_sync(0xffffffffu, s, 1);
        s += __shfl_xor_sync(0xffffffffu, s, 2);
        if (part == 0) X[r][j] = (X[r][j] - s) / U[j][j];
        __syncwarp();
    }
    __syncthreads();
    for (int idx = tid; idx < kTrsmRows * NB; idx += nt) {
        const int rr = idx / NB, c = idx % NB;
        const int64_t gr = row0 + rr;
        if (gr < n && c < kb) A[gr * lda + k + c] = X[rr][c];
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

// Restricted form of gemm_update_kernel for the two-level setup (any T):
// C[i][j] -= sum_p A[i][k+p] A[k+p][j] for i in [r_lo, r_hi), j in [c_lo, c_hi);
// with diag_bs > 0 the grid's z index selects the diagonal block
// [r_lo + z diag_bs, ...) of both ranges.
template <typename T, int BM, int BN, int BK>
__global__ void __launch_bounds__(256) gemm_range_kernel(T* __restrict__ A, int64_t lda, int64_t k, int kb,
                                                         int64_t r_lo, int64_t r_hi, int64_t c_lo, int64_t c_hi,
                                                         int diag_bs) {
    constexpr int TM = BM / 16, TN = BN / 16;
    __shared__ T As[BK][BM + 1];
    __shared__ T Bs[BK][BN];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    if (diag_bs > 0) {
        const int64_t b0 = r_lo + (int64_t)blockIdx.z * diag_bs;
        r_lo = c_lo = b0;
        r_hi = c_hi = min(r_hi, b0 + diag_bs);
    }
    const int64_t i0 = r_lo + (int64_t)blockIdx.y * BM, j0 = c_lo + (int64_t)blockIdx.x * BN;
    if (i0 >= r_hi || j0 >= c_hi) return;
    T acc[TM][TN];
#pragma unroll
    for (int a = 0; a < TM; ++a)
#pragma unroll
        for (int b = 0; b < TN; ++b) acc[a][b] = (T)0;
    for (int p0 = 0; p0 < kb; p0 += BK) {
        for (int idx = threadIdx.x; idx < BM * BK; idx += 256) {
            int m = idx / BK, p = idx % BK;
            int64_t gi = i0 + m;
            As[p][m] = (gi < r_hi && p0 + p < kb) ? A[gi * lda + k + p0 + p] : (T)0;
        }
        for (int idx = threadIdx.x; idx < BK * BN; idx += 256) {
            int p = idx / BN, c = idx % BN;
            int64_t gj = j0 + c;
            Bs[p][c] = (gj < c_hi && p0 + p < kb) ? A[(k + p0 + p) * lda + gj] : (T)0;
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
        if (gi >= r_hi) continue;
#pragma unroll
        for (int b = 0; b < TN; ++b) {
            int64_t gj = j0 + tx + 16 * b;
            if (gj < c_hi) A[gi * lda + gj] -= acc[a][b];
        }
    }
}

// ----------------------------------------------------------------------------
// Float-float restricted update for the two-level setup (GK_FF): the same
// C -= L_panel U_panel as gemm_range_kernel<double> on FP64 storage, with the
// products on the FP32 pipe.  GB300 issues ~2 FP64 FMAs per clock per SM, so
// FP64 updates run at ~1.2 TFLOP/s; here each panel entry is split once into
// a float pair (hi + lo, ~48 bits) by split_panel_kernel and every
// multiply-add is ~12 FP32 operations: the exact product error from an FMA,
// the cross terms, and a TwoSum into a (hi, lo) accumulator whose low word
// collects the errors (accuracy ~1e-12 of sum |a b| per update; the FP32 form
// gives ~1e-6).  Only the epilogue (C -= hi + lo) touches the FP64 pipe.
// Panels come in pairs of two 32-column LU steps, so each trailing-update
// launch covers 64 columns and the FP64 epilogue is paid half as often:
// L rows x pair columns as Lh/Ll[i * kFfPair + c], U pair rows x columns as
// Uh/Ul[c * n + j] (c = column of the pair).
// ----------------------------------------------------------------------------
constexpr int kFfPanel = 32;  // == LuCfg<double>::NB: one LU step
constexpr int kFfPair = 2 * kFfPanel;

// Split the panel at k (kb columns; L rows [o, n), U columns [o, n)) into
// pair columns [coff, coff + kb).
__global__ void split_panel_kernel(const double* __restrict__ A, int64_t lda, int64_t n, int64_t k, int kb,
                                   int64_t o, int coff, float* __restrict__ Lh, float* __restrict__ Ll,
                                   float* __restrict__ Uh, float* __restrict__ Ul) {
    const int64_t m = (n - o) * kFfPanel;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < 2 * m; e += (int64_t)gridDim.x * blockDim.x) {
        const bool upper = e >= m;
        const int64_t f = upper ? e - m : e;
        double v = 0.0;
        int64_t dst;
        if (!upper) {
            const int64_t i = o + f / kFfPanel;
            const int p = (int)(f % kFfPanel);
            if (p < kb) v = A[i * lda + k + p];
            dst = i * kFfPair + coff + p;
        } else {
            const int p = (int)(f / (n - o));
            const int64_t j = o + f % (n - o);
            if (p < kb) v = A[(k + p) * lda + j];
            dst = (int64_t)(coff + p) * n + j;
        }
        const float h = (float)v;
        const float l = (float)(v - (double)h);
        if (!upper) { Lh[dst] = h; Ll[dst] = l; } else { Uh[dst] = h; Ul[dst] = l; }
    }
}

__global__ void __launch_bounds__(256) ffgemm_range_kernel(double* __restrict__ A, int64_t lda, int64_t n, int kb,
                                                           const float* __restrict__ Lh, const float* __restrict__ Ll,
                                                           const float* __restrict__ Uh, const float* __restrict__ Ul,
                                                           int64_t r_lo, int64_t r_hi, int64_t c_lo, int64_t c_hi,
                                                           int diag_bs) {
    // the whole 32-column panel slice is staged at once: one barrier pair per tile
    constexpr int BM = 64, BN = 64, BK = kFfPanel, TM = 4, TN = 4;
    __shared__ float Ash[BK][BM + 1], Asl[BK][BM + 1];
    __shared__ float Bsh[BK][BN], Bsl[BK][BN];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    if (diag_bs > 0) {
        const int64_t b0 = r_lo + (int64_t)blockIdx.z * diag_bs;
        r_lo = c_lo = b0;
        r_hi = c_hi = min(r_hi, b0 + diag_bs);
    }
    const int64_t i0 = r_lo + (int64_t)blockIdx.y * BM, j0 = c_lo + (int64_t)blockIdx.x * BN;
    if (i0 >= r_hi || j0 >= c_hi) return;
    float ah[TM][TN], al[TM][TN];
#pragma unroll
    for (int a = 0; a < TM; ++a)
#pragma unroll
        for (int b = 0; b < TN; ++b) { ah[a][b] = 0.f; al[a][b] = 0.f; }
    for (int p0 = 0; p0 < kb; p0 += BK) {
        for (int idx = threadIdx.x; idx < BM * BK; idx += 256) {
            const int m = idx / BK, p = idx % BK;
            const int64_t gi = i0 + m;
            const bool ok = gi < r_hi && p0 + p < kb;
            Ash[p][m] = ok ? Lh[gi * kFfPair + p0 + p] : 0.f;
            Asl[p][m] = ok ? Ll[gi * kFfPair + p0 + p] : 0.f;
        }
        for (int idx = threadIdx.x; idx < BK * BN; idx += 256) {
            const int p = idx / BN, c = idx % BN;
            const int64_t gj = j0 + c;
            const bool ok = gj < c_hi && p0 + p < kb;
            Bsh[p][c] = ok ? Uh[(int64_t)(p0 + p) * n + gj] : 0.f;
            Bsl[p][c] = ok ? Ul[(int64_t)(p0 + p) * n + gj] : 0.f;
        }
        __syncthreads();
#pragma unroll 4
        for (int p = 0; p < BK; ++p) {
            float xh[TM], xl[TM], yh[TN], yl[TN];
#pragma unroll
            for (int a = 0; a < TM; ++a) { xh[a] = Ash[p][ty + 16 * a]; xl[a] = Asl[p][ty + 16 * a]; }
#pragma unroll
            for (int b = 0; b < TN; ++b) { yh[b] = Bsh[p][tx + 16 * b]; yl[b] = Bsl[p][tx + 16 * b]; }
#pragma unroll
            for (int a = 0; a < TM; ++a)
#pragma unroll
                for (int b = 0; b < TN; ++b) {
                    const float ph = __fmul_rn(xh[a], yh[b]);
                    float pl = __fmaf_rn(xh[a], yh[b], -ph);
                    pl = __fmaf_rn(xh[a], yl[b], pl);
                    pl = __fmaf_rn(xl[a], yh[b], pl);
                    const float s = __fadd_rn(ah[a][b], ph);
                    const float v = __fsub_rn(s, ah[a][b]);
                    const float e = __fadd_rn(__fsub_rn(ah[a][b], __fsub_rn(s, v)), __fsub_rn(ph, v));
                    ah[a][b] = s;
                    al[a][b] = __fadd_rn(al[a][b], __fadd_rn(e, pl));
                }
        }
        __syncthreads();
    }
#pragma unroll
    for (int a = 0; a < TM; ++a) {
        const int64_t gi = i0 + ty + 16 * a;
        if (gi >= r_hi) continue;
#pragma unroll
        for (int b = 0; b < TN; ++b) {
            const int64_t gj = j0 + tx + 16 * b;
            if (gj < c_hi) A[gi * lda + gj] -= (double)ah[a][b] + (double)al[a][b];
        }
    }
}

// FP32 trailing update for aligned panels (offsets and lda multiples of 4):
// 128 x 128 tile per CTA, 16 x 16 threads each owning an 8 x 8 block split in
// four 4 x 4 quadrants, float4 shared-memory reads (A stored k-major), the
// next k-slice prefetched into registers while the current one is consumed.
// C[i][j] -= sum_p A[i][k+p] A[k+p][j] for i in [r_lo, r_hi), j in [c_lo, c_hi);
// with diag_bs > 0 the grid's z index selects the diagonal block
// [r_lo + z diag_bs, ...) of both ranges (block-diagonal update).
__global__ void __launch_bounds__(256, 2) sgemm_update_kernel(float* __restrict__ A, int64_t lda, int64_t k, int kb,
                                                              int64_t r_lo, int64_t r_hi, int64_t c_lo,
                                                              int64_t c_hi, int diag_bs) {
    constexpr int BM = 128, BN = 128, BK = 16;
    __shared__ __align__(16) float As[2][BK][BM];
    __shared__ __align__(16) float Bs[2][BK][BN];
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    if (diag_bs > 0) {
        const int64_t b0 = r_lo + (int64_t)blockIdx.z * diag_bs;
        r_lo = c_lo = b0;
        r_hi = c_hi = min(r_hi, b0 + diag_bs);
    }
    const int64_t n = r_hi;      // row bound
    const int64_t ncol = c_hi;   // column bound
    const int64_t i0 = r_lo + (int64_t)blockIdx.y * BM, j0 = c_lo + (int64_t)blockIdx.x * BN;
    if (i0 >= r_hi || j0 >= c_hi) return;
    float acc[8][8];
#pragma unroll
    for (int a = 0; a < 8; ++a)
#pragma unroll
        for (int b = 0; b < 8; ++b) acc[a][b] = 0.f;
    // loader mapping
    const int la_row = tid >> 1, la_k = (tid & 1) * 8;          // A: 128 rows x 16 k
    const int lb_row = tid >> 5, lb_col = (tid & 31) * 4;        // B: rows lb_row, lb_row + 8
    float4 ra[2], rb[2];
    auto gload = [&](int p0) {
        const int64_t gi = i0 + la_row;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int kk = p0 + la_k + 4 * h;
            if (gi < n && kk + 3 < kb) {
                ra[h] = *reinterpret_cast<const float4*>(A + gi * lda + k + kk);
            } else {
                float t[4];
                for (int e = 0; e < 4; ++e) t[e] = (gi < n && kk + e < kb) ? A[gi * lda + k + kk + e] : 0.f;
                ra[h] = make_float4(t[0], t[1], t[2], t[3]);
            }
        }
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int kk = p0 + lb_row + 8 * h;
            const int64_t gj = j0 + lb_col;
            if (kk < kb && gj + 3 < ncol) {
                rb[h] = *reinterpret_cast<const float4*>(A + (k + kk) * lda + gj);
            } else {
                float t[4];
                for (int e = 0; e < 4; ++e) t[e] = (kk < kb && gj + e < ncol) ? A[(k + kk) * lda + gj + e] : 0.f;
                rb[h] = make_float4(t[0], t[1], t[2], t[3]);
            }
        }
    };
    auto sstore = [&](int buf) {
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            As[buf][la_k + 4 * h + 0][la_row] = ra[h].x;
            As[buf][la_k + 4 * h + 1][la_row] = ra[h].y;
            As[buf][la_k + 4 * h + 2][la_row] = ra[h].z;
            As[buf][la_k + 4 * h + 3][la_row] = ra[h].w;
            *reinterpret_cast<float4*>(&Bs[buf][lb_row + 8 * h][lb_col]) = rb[h];
        }
    };
    const int nk = (kb + BK - 1) / BK;
    gload(0);
    sstore(0);
    __syncthreads();
    for (int it = 0; it < nk; ++it) {
        const int buf = it & 1;
        if (it + 1 < nk) gload((it + 1) * BK);
#pragma unroll
        for (int p = 0; p < BK; ++p) {
            const float4 a0 = *reinterpret_cast<const float4*>(&As[buf][p][ty * 4]);
            const float4 a1 = *reinterpret_cast<const float4*>(&As[buf][p][64 + ty * 4]);
            const float4 b0 = *reinterpret_cast<const float4*>(&Bs[buf][p][tx * 4]);
            const float4 b1 = *reinterpret_cast<const float4*>(&Bs[buf][p][64 + tx * 4]);
            const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
            const float bv[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
            for (int a = 0; a < 8; ++a)
#pragma unroll
                for (int b = 0; b < 8; ++b) acc[a][b] = __fmaf_rn(av[a], bv[b], acc[a][b]);
        }
        if (it + 1 < nk) {
            sstore(buf ^ 1);
        }
        __syncthreads();
    }
#pragma unroll
    for (int a = 0; a < 8; ++a) {
        const int64_t gi = i0 + (a < 4 ? ty * 4 + a : 64 + ty * 4 + a - 4);
        if (gi >= n) continue;
#pragma unroll
        for (int hb = 0; hb < 2; ++hb) {
            const int64_t gj = j0 + hb * 64 + tx * 4;
            float* c = A + gi * lda + gj;
            if (gj + 3 < ncol) {
                float4 v = *reinterpret_cast<float4*>(c);
                v.x -= acc[a][4 * hb + 0];
                v.y -= acc[a][4 * hb + 1];
                v.z -= acc[a][4 * hb + 2];
                v.w -= acc[a][4 * hb + 3];
                *reinterpret_cast<float4*>(c) = v;
            } else {
                for (int e = 0; e < 4; ++e)
                    if (gj + e < ncol) c[e] -= acc[a][4 * hb + e];
            }
        }
    }
}

// The tensor-core form of the FP32 trailing update (gk_lu_tc.cu) and the
// switch between it and sgemm_update_kernel (gk_lu_update_select).
gk_status lu_tc_update(float* A, int64_t lda, int64_t k, int kb, int64_t r_lo, int64_t r_hi, int64_t c_lo,
                       int64_t c_hi, int diag_bs, unsigned nz, gk_info* info, cudaStream_t st, int max_ctas);
bool lu_update_on_tensor_cores();
cudaError_t wait_cap_set_lu_tc(long long v);

// C -= L U over rows [r_lo, r_hi) x columns [c_lo, c_hi) (or nz diagonal
// blocks of diag_bs), on the engine gk_lu_update_select chose.
static gk_status sgemm_update(float* A, int64_t lda, int64_t k, int kb, int64_t r_lo, int64_t r_hi, int64_t c_lo,
                              int64_t c_hi, int diag_bs, unsigned nz, gk_info* info, cudaStream_t st,
                              int max_ctas = 0) {
    if (lu_update_on_tensor_cores())
        return lu_tc_update(A, lda, k, kb, r_lo, r_hi, c_lo, c_hi, diag_bs, nz, info, st, max_ctas);
    const int64_t rows = diag_bs > 0 ? diag_bs : r_hi - r_lo;
    const int64_t cols = diag_bs > 0 ? diag_bs : c_hi - c_lo;
    if (rows <= 0 || cols <= 0) return GK_OK;
    dim3 grid((unsigned)((cols + 127) / 128), (unsigned)((rows + 127) / 128), nz < 1 ? 1u : nz);
    sgemm_update_kernel<<<grid, 256, 0, st>>>(A, lda, k, kb, r_lo, r_hi, c_lo, c_hi, diag_bs);
    GK_LAUNCH_CHECK();
    return GK_OK;
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

// Inverses of the 128 x 128 diagonal blocks of L (unit lower) and U (upper),
// computed once per factorization: CTA b, thread c solves for column c of the
// inverse, all threads stepping through the rows together (L/U entries are
// warp-broadcast loads, the partial inverse lives in shared memory).
constexpr int kTB = 128;         // triangular-solve block
constexpr int kFlagStride = 32;  // one 128-byte line per block flag

template <typename T>
__global__ void __launch_bounds__(kTB) tri_inv_kernel(const T* __restrict__ A, int64_t lda, int64_t n,
                                                      T* __restrict__ invL, T* __restrict__ invU, gk_info* info) {
    extern __shared__ unsigned char smem_raw[];
    T* Y = reinterpret_cast<T*>(smem_raw);  // kTB x kTB, Y[r * kTB + c]
    const int b = blockIdx.x, c = threadIdx.x;
    const int64_t r0 = (int64_t)b * kTB;
    const int rows = (int)min((int64_t)kTB, n - r0);
    auto at = [&](int r, int k) -> T { return A[(r0 + r) * lda + r0 + k]; };
    // L^-1 (unit diagonal; padding rows act as identity)
    for (int r = 0; r < kTB; ++r) {
        T v = (r == c) ? (T)1 : (T)0;
        if (r > c && r < rows) {
            for (int k = c; k < r; ++k) v -= at(r, k) * Y[k * kTB + c];
        }
        Y[r * kTB + c] = v;
        __syncwarp();
        __syncthreads();
    }
    for (int r = 0; r < kTB; ++r) invL[((int64_t)b * kTB + r) * kTB + c] = Y[r * kTB + c];
    __syncthreads();
    // U^-1
    for (int r = kTB - 1; r >= 0; --r) {
        T v = (r == c) ? (T)1 : (T)0;
        if (r < rows) {
            if (r < c) {
                for (int k = r + 1; k <= c && k < rows; ++k) v -= at(r, k) * Y[k * kTB + c];
            }
            T d = at(r, r);
            if (d == (T)0) {
                if (c == 0) report(info, GK_ERR_SINGULAR, (int)(r0 + r));
                v = (T)0;
            } else {
                v = (r <= c) ? v / d : (T)0;
            }
        }
        Y[r * kTB + c] = v;
        __syncthreads();
    }
    for (int r = 0; r < kTB; ++r) invU[((int64_t)b * kTB + r) * kTB + c] = Y[r * kTB + c];
}

// Blocked triangular solve, in place on x.  lower: L (unit), forward; upper:
// U, backward.  CTAs claim 128-row blocks in solve order through ``counter``;
// each warp owns 16 rows and, per earlier block, polls that block's flag
// (bounded) and accumulates its 16 x 128 product without block-wide barriers.
// The block's unknowns are then x_b = inv(D_b) (x_b - acc), a warp-parallel
// matvec with the precomputed inverse of the diagonal block.
template <typename T>
__global__ void __launch_bounds__(256) trsv_kernel(const T* __restrict__ A, int64_t lda, int64_t n, T* x,
                                                   const T* __restrict__ dinv, int lower, int* counter, int* flags,
                                                   gk_info* info) {
    __shared__ int s_blk;
    __shared__ T rhs[kTB];
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int nblk = (int)((n + kTB - 1) / kTB);
    if (tid == 0) s_blk = atomicAdd(counter, 1);
    __syncthreads();
    const int ord = s_blk;
    if (ord >= nblk) return;
    const int blk = lower ? ord : nblk - 1 - ord;
    const int64_t r0 = (int64_t)blk * kTB;
    const int rows = (int)min((int64_t)kTB, n - r0);
    // this warp's 16 rows of inv(D_b), prefetched before any wait
    const T* Di = dinv + (int64_t)blk * kTB * kTB;
    T dv[16][4];
#pragma unroll
    for (int q = 0; q < 16; ++q)
#pragma unroll
        for (int e = 0; e < 4; ++e) dv[q][e] = Di[(int64_t)(wid * 16 + q) * kTB + lane + 32 * e];
    T acc[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) acc[q] = (T)0;
    for (int o = 0; o < ord; ++o) {
        const int dep = lower ? o : nblk - 1 - o;
        const int64_t c0 = (int64_t)dep * kTB;
        const int cols = (int)min((int64_t)kTB, n - c0);
        // the matrix block does not depend on the flag: load it first
        T av[16][4];
#pragma unroll
        for (int q = 0; q < 16; ++q) {
            const int r = wid * 16 + q;
            const T* row = A + (r0 + (r < rows ? r : 0)) * lda + c0;
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int c = lane + 32 * e;
                av[q][e] = (r < rows && c < cols) ? row[c] : (T)0;
            }
        }
        if (lane == 0) {
            const long long cap = wait_cap(kSpinLimit);
            for (long long spins = 0;; ++spins) {
                if (spins >= cap) { report(info, GK_ERR_TIMEOUT, dep); break; }
                int f;
                asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(f) : "l"(flags + kFlagStride * dep)
                             : "memory");
                if (f) break;
                if (spins > 64) __nanosleep(20);
            }
        }
        __syncwarp();
        T xv[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const int c = lane + 32 * e;
            xv[e] = c < cols ? ((volatile T*)x)[c0 + c] : (T)0;
        }
#pragma unroll
        for (int q = 0; q < 16; ++q)
#pragma unroll
            for (int e = 0; e < 4; ++e) acc[q] += av[q][e] * xv[e];
    }
#pragma unroll
    for (int q = 0; q < 16; ++q) {
        T sv = acc[q];
        for (int o = 16; o > 0; o >>= 1) sv += __shfl_down_sync(0xffffffffu, sv, o);
        const int r = wid * 16 + q;
        if (lane == 0) rhs[r] = r < rows ? x[r0 + r] - sv : (T)0;
    }
    __syncthreads();
    // x_b = inv(D_b) rhs
    T rv[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) rv[e] = rhs[lane + 32 * e];
#pragma unroll
    for (int q = 0; q < 16; ++q) {
        T sv = dv[q][0] * rv[0] + dv[q][1] * rv[1] + dv[q][2] * rv[2] + dv[q][3] * rv[3];
        for (int o = 16; o > 0; o >>= 1) sv += __shfl_down_sync(0xffffffffu, sv, o);
        const int r = wid * 16 + q;
        if (lane == 0 && r < rows) x[r0 + r] = sv;
    }
    __syncthreads();
    if (tid == 0) {
        __threadfence();
        asm volatile("st.release.gpu.global.b32 [%0], %1;" :: "l"(flags + kFlagStride * blk), "r"(1) : "memory");
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
    const int max_rows = (int)(max_smem / ((NB + 1) * sizeof(T)));
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
    pl.smem = (size_t)chunk * (NB + 1) * sizeof(T);
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

// Workspace: [panel exchange][perm (n+1)][flags + counter][tmp vector (n)]
//            [inverse diagonal blocks of L][... of U]
template <typename T>
static size_t lu_ws_bytes(int64_t n) {
    constexpr int NB = LuCfg<T>::NB;
    int sms = device_sm_count();
    const size_t nblk = (size_t)((n + kTB - 1) / kTB);
    return panel_ws_bytes<T, NB>(sms) + align256((size_t)(n + 1) * sizeof(int32_t)) * 2 +
           align256(((size_t)(n + kTB - 1) / kTB + 2) * kFlagStride * sizeof(int)) +
           align256((size_t)n * sizeof(T)) + 2 * align256(nblk * kTB * kTB * sizeof(T));
}

template <typename T>
static T* lu_ws_dinv(void* work, int64_t n, int upper) {
    constexpr int NB = LuCfg<T>::NB;
    int sms = device_sm_count();
    const size_t nblk = (size_t)((n + kTB - 1) / kTB);
    char* p = (char*)work + panel_ws_bytes<T, NB>(sms) + align256((size_t)(n + 1) * sizeof(int32_t)) * 2 +
              align256(((size_t)(n + kTB - 1) / kTB + 2) * kFlagStride * sizeof(int)) +
              align256((size_t)n * sizeof(T));
    if (upper) p += align256(nblk * kTB * kTB * sizeof(T));
    return (T*)p;
}

// Largest cluster size (<= 16) the device can schedule with ~200 KB of shared
// memory per CTA; 0 when clusters are unavailable.
template <typename T, int NB>
static int cluster_capacity() {
    static int cached = -1;
    if (cached >= 0) return cached;
    cached = 0;
    auto ck = panel_cluster_kernel<T, NB>;
    if (cudaFuncSetAttribute(ck, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024) != cudaSuccess ||
        cudaFuncSetAttribute(ck, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
        (void)cudaGetLastError();
        return cached;
    }
    for (int C = 16; C >= 2; C /= 2) {
        cudaLaunchConfig_t cfg = {};
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = C;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.gridDim = dim3(C);
        cfg.blockDim = dim3(256);
        cfg.dynamicSmemBytes = 200 * 1024;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        int nc = 0;
        if (cudaOccupancyMaxActiveClusters(&nc, ck, &cfg) == cudaSuccess && nc > 0) {
            cached = C;
            return cached;
        }
        (void)cudaGetLastError();
    }
    return cached;
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
    auto ck = panel_cluster_kernel<T, NB>;
    GK_CUDA_TRY(cudaFuncSetAttribute(ck, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    GK_CUDA_TRY(cudaFuncSetAttribute(ck, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    // GK_PANEL_COOPERATIVE=1 selects the grid-barrier panel for every size
    // (the path large panels take), so both implementations can be tested.
    const char* force_coop = getenv("GK_PANEL_COOPERATIVE");
    const int max_cluster = (force_coop && force_coop[0] == '1') ? 0 : cluster_capacity<T, NB>();
    for (int64_t k = 0; k < n; k += NB) {
        int kb = (int)min((int64_t)NB, n - k);
        if (max_cluster > 0) {
            const int64_t m = n - k;
            const int max_rows = (int)((200 * 1024) / ((NB + 1) * sizeof(T)));
            int C = (int)((m + 127) / 128);
            if (C < 1) C = 1;
            if (C > max_cluster) C = max_cluster;
            int chunk = (int)((m + C - 1) / C);
            if (chunk <= max_rows) {
                cudaLaunchConfig_t cfg = {};
                cudaLaunchAttribute attr[1];
                attr[0].id = cudaLaunchAttributeClusterDimension;
                attr[0].val.clusterDim.x = C;
                attr[0].val.clusterDim.y = 1;
                attr[0].val.clusterDim.z = 1;
                cfg.gridDim = dim3(C);
                cfg.blockDim = dim3(256);
                cfg.dynamicSmemBytes = (size_t)chunk * (NB + 1) * sizeof(T);
                cfg.stream = st;
                cfg.attrs = attr;
                cfg.numAttrs = 1;
                GK_CUDA_TRY(cudaLaunchKernelEx(&cfg, ck, A, lda, n, (int64_t)k, kb, chunk, ipiv, info));
                gk_launch_counter().fetch_add(1, std::memory_order_relaxed);
                goto after_panel;
            }
        }
        {
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
        }
    after_panel:
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
            if (sizeof(T) == 4 && ((k + kb) % 4) == 0 && (lda % 4) == 0 &&
                ((uintptr_t)A % 16) == 0) {
                gk_status s = sgemm_update((float*)A, lda, k, kb, k + kb, n, k + kb, n, 0, 1, info, st);
                if (s != GK_OK) return s;
            } else {
                gemm_update_kernel<T, BM, BN, 16><<<grid, 256, 0, st>>>(A, lda, n, k, kb);
                GK_LAUNCH_CHECK();
            }
        }
    }
    // row permutation for the solves, kept in the workspace
    int32_t* perm = (int32_t*)((char*)work + panel_ws_bytes<T, NB>(sms));
    size_t psmem = n <= kPermSmem ? (size_t)n * sizeof(int32_t) : 0;
    GK_CUDA_TRY(cudaFuncSetAttribute(perm_from_ipiv_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kPermSmem * 4));
    perm_from_ipiv_kernel<<<1, 256, psmem, st>>>(ipiv, n, perm);
    GK_LAUNCH_CHECK();
    // inverses of the diagonal blocks for the triangular solves
    const size_t ysmem = (size_t)kTB * kTB * sizeof(T);
    GK_CUDA_TRY(cudaFuncSetAttribute(tri_inv_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ysmem));
    tri_inv_kernel<T><<<(unsigned)((n + kTB - 1) / kTB), kTB, ysmem, st>>>(A, lda, n, lu_ws_dinv<T>(work, n, 0),
                                                                          lu_ws_dinv<T>(work, n, 1), info);
    GK_LAUNCH_CHECK();
    return GK_OK;
}

// The second stream of the unpivoted FP32 LU's look-ahead: per device, the
// highest priority, created on first use and kept for the process.
static gk_status lookahead_stream(cudaStream_t& out) {
    static std::mutex mu;
    static cudaStream_t tab[64] = {};
    int dev = 0;
    GK_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return GK_ERR_CUDA;
    std::lock_guard<std::mutex> g(mu);
    if (tab[dev] == nullptr) {
        int lo = 0, hi = 0;
        GK_CUDA_TRY(cudaDeviceGetStreamPriorityRange(&lo, &hi));
        GK_CUDA_TRY(cudaStreamCreateWithPriority(&tab[dev], cudaStreamNonBlocking, hi));
    }
    out = tab[dev];
    return GK_OK;
}

// Systems above this size factor with look-ahead (below it the panels are
// too short to hide anything).
constexpr int64_t kLookaheadMinN = 2048;

// Unpivoted blocked LU.  Per panel k: the diagonal block (one CTA; for FP32
// full panels it also writes U11^-1), L21 = A21 U11^-1 (a product with that
// inverse for FP32 full panels, else a row-parallel triangular solve),
// U12 = L11^-1 A12, then the trailing update.  For FP32
// systems above kLookaheadMinN the update is split: first the next panel's
// columns, then the rest; the next diagonal block is factored on a second,
// higher-priority stream while the rest of the update runs (which then
// leaves one SM free on the tensor-core engine), so the one-CTA factorization
// leaves the critical path.
template <typename T>
static gk_status lu_factor_nopiv(int64_t n, T* A, int64_t lda, int32_t* ipiv, void* work, size_t wbytes,
                                 gk_info* info, cudaStream_t st) {
    constexpr int NB = LuCfg<T>::NB;
    if (n <= 0 || A == nullptr || ipiv == nullptr || lda < n) return GK_ERR_ARG;
    if (work == nullptr || wbytes < lu_ws_bytes<T>(n)) return GK_ERR_SIZE;
    int sms = device_sm_count();
    if (info) GK_CUDA_TRY(cudaMemsetAsync(info, 0, sizeof(gk_info), st));
    const bool fast = sizeof(T) == 4 && (lda % 4) == 0 && ((uintptr_t)A % 16) == 0;
    const bool lookahead = fast && n > kLookaheadMinN;
    // U11^-1 of the current panel; the inverse blocks of the solves (written
    // after the factorization) are free until then
    T* uinv = lu_ws_dinv<T>(work, n, 0);
    cudaStream_t side = nullptr;
    cudaEvent_t ev_ready = nullptr, ev_diag = nullptr;
    if (lookahead) {
        gk_status s = lookahead_stream(side);
        if (s != GK_OK) return s;
        GK_CUDA_TRY(cudaEventCreateWithFlags(&ev_ready, cudaEventDisableTiming));
        if (cudaEventCreateWithFlags(&ev_diag, cudaEventDisableTiming) != cudaSuccess) {
            cudaEventDestroy(ev_ready);
            return GK_ERR_CUDA;
        }
    }
    gk_status status = GK_OK;
    bool diag_ready = false;   // the diagonal block of panel k was factored ahead
    for (int64_t k = 0; k < n && status == GK_OK; k += NB) {
        int kb = (int)min((int64_t)NB, n - k);
        if (!diag_ready) {
            diag_lu_kernel<T, NB><<<1, 256, 0, st>>>(A, lda, k, kb, ipiv, info, fast ? uinv : nullptr);
            gk_launch_counter().fetch_add(1, std::memory_order_relaxed);
            if (cudaPeekAtLastError() != cudaSuccess) { (void)cudaGetLastError(); status = GK_ERR_CUDA; break; }
        }
        diag_ready = false;
        int64_t rest = n - k - kb;
        if (rest <= 0) break;
        if (fast && kb == NB) {
            trsm_right_inv_kernel<T, NB><<<(unsigned)((rest + 63) / 64), 256, 0, st>>>(A, lda, n, k, uinv);
        } else {
            trsm_right_kernel<T, NB><<<(unsigned)((rest + kTrsmRows - 1) / kTrsmRows), kTrsmRows * kTrsmLanes, 0,
                                       st>>>(A, lda, n, k, kb);
        }
        trsm_kernel<T, NB><<<(unsigned)((rest + 127) / 128), 128, 0, st>>>(A, lda, n, k, kb);
        gk_launch_counter().fetch_add(2, std::memory_order_relaxed);
        if (cudaPeekAtLastError() != cudaSuccess) { (void)cudaGetLastError(); status = GK_ERR_CUDA; break; }
        constexpr int BM = sizeof(T) == 8 ? 64 : 128;
        constexpr int BN = BM;
        if (fast && ((k + kb) % 4) == 0) {
            const int64_t c0 = k + kb;
            const int nkb = (int)min((int64_t)NB, rest);
            if (lookahead && c0 + nkb < n) {
                // the next panel's columns, then its diagonal block on the side stream
                status = sgemm_update((float*)A, lda, k, kb, c0, n, c0, c0 + nkb, 0, 1, info, st, 0);
                if (status != GK_OK) break;
                if (cudaEventRecord(ev_ready, st) != cudaSuccess || cudaStreamWaitEvent(side, ev_ready, 0) != cudaSuccess) {
                    status = GK_ERR_CUDA;
                    break;
                }
                diag_lu_kernel<T, NB><<<1, 256, 0, side>>>(A, lda, c0, nkb, ipiv, info, uinv);
                gk_launch_counter().fetch_add(1, std::memory_order_relaxed);
                if (cudaPeekAtLastError() != cudaSuccess || cudaEventRecord(ev_diag, side) != cudaSuccess) {
                    (void)cudaGetLastError();
                    status = GK_ERR_CUDA;
                    break;
                }
                // the rest of the update, one SM left to the side stream
                status = sgemm_update((float*)A, lda, k, kb, c0, n, c0 + nkb, n, 0, 1, info, st, sms - 1);
                if (cudaStreamWaitEvent(st, ev_diag, 0) != cudaSuccess && status == GK_OK) status = GK_ERR_CUDA;
                if (status != GK_OK) break;
                diag_ready = true;
            } else {
                status = sgemm_update((float*)A, lda, k, kb, c0, n, c0, n, 0, 1, info, st, 0);
            }
        } else {
            dim3 grid((unsigned)((rest + BN - 1) / BN), (unsigned)((rest + BM - 1) / BM));
            gemm_update_kernel<T, BM, BN, 16><<<grid, 256, 0, st>>>(A, lda, n, k, kb);
            gk_launch_counter().fetch_add(1, std::memory_order_relaxed);
            if (cudaPeekAtLastError() != cudaSuccess) { (void)cudaGetLastError(); status = GK_ERR_CUDA; }
        }
    }
    if (ev_ready) cudaEventDestroy(ev_ready);
    if (ev_diag) cudaEventDestroy(ev_diag);
    if (status != GK_OK) return status;
    int32_t* perm = (int32_t*)((char*)work + panel_ws_bytes<T, NB>(sms));
    size_t psmem = n <= kPermSmem ? (size_t)n * sizeof(int32_t) : 0;
    GK_CUDA_TRY(cudaFuncSetAttribute(perm_from_ipiv_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kPermSmem * 4));
    perm_from_ipiv_kernel<<<1, 256, psmem, st>>>(ipiv, n, perm);
    GK_LAUNCH_CHECK();
    const size_t ysmem = (size_t)kTB * kTB * sizeof(T);
    GK_CUDA_TRY(cudaFuncSetAttribute(tri_inv_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ysmem));
    tri_inv_kernel<T><<<(unsigned)((n + kTB - 1) / kTB), kTB, ysmem, st>>>(A, lda, n, lu_ws_dinv<T>(work, n, 0),
                                                                          lu_ws_dinv<T>(work, n, 1), info);
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
    constexpr int BS = kTB;
    if (n <= 0 || LU == nullptr || ipiv == nullptr || b == nullptr) return GK_ERR_ARG;
    if (work == nullptr || wbytes < lu_ws_bytes<T>(n)) return GK_ERR_SIZE;
    int sms = device_sm_count();
    char* p = (char*)work + panel_ws_bytes<T, NB>(sms);
    int32_t* perm = (int32_t*)p; p += align256((size_t)(n + 1) * sizeof(int32_t)) * 2;
    int nblk = (int)((n + BS - 1) / BS);
    int* flags = (int*)p; p += align256(((size_t)nblk + 2) * kFlagStride * sizeof(int));
    T* tmp = (T*)p;
    gather_kernel<T, T><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(b, perm, n, tmp);
    GK_LAUNCH_CHECK();
    int* counter = flags + (size_t)nblk * kFlagStride;
    for (int pass = 0; pass < 2; ++pass) {
        GK_CUDA_TRY(cudaMemsetAsync(flags, 0, ((size_t)nblk + 1) * kFlagStride * sizeof(int), st));
        // one CTA per block row; CTAs claim rows in solve order, so a CTA only
        // ever waits on rows claimed by CTAs that are already running
        trsv_kernel<T><<<nblk, 256, 0, st>>>(LU, lda, n, tmp, lu_ws_dinv<T>(work, n, pass), pass == 0 ? 1 : 0,
                                             counter, flags, info);
        GK_LAUNCH_CHECK();
    }
    GK_CUDA_TRY(cudaMemcpyAsync(b, tmp, n * sizeof(T), cudaMemcpyDeviceToDevice, st));
    return GK_OK;
}

// ----------------------------------------------------------------------------
// Two-level preconditioner: block-Jacobi on a Schur complement plus a low-rank
// (landmark) correction.
//
// The matrix is symmetrically permuted so that r landmark unknowns come first
// and the remaining ones follow in spatially contiguous blocks of bs.  A
// partial LU without pivoting over the first r columns computes
//     [A_LL A_LR; A_RL A_RR] = [L_LL 0; L_RL I] [U_LL U_LR; 0 S],
// but of the trailing update S = A_RR - L_RL U_LR only the bs x bs diagonal
// blocks are formed and LU-factored (block-Jacobi on S).  Applying
//     M^-1 = [U_LL U_LR; 0 blockdiag(S)]^-1 [L_LL 0; L_RL I]^-1
// costs two triangular solves of order r, two rectangular products and the
// block solves.  L_RL U_LR is the low-rank (rank r) part of the operator.
// ----------------------------------------------------------------------------
// FP64 blocks use 256 threads so the per-thread 32-entry row buffers of
// cta_lu_nopiv stay in registers.
template <typename T>
constexpr int block_lu_threads() { return sizeof(T) == 8 ? 256 : 512; }

template <typename T>
__global__ void __launch_bounds__(block_lu_threads<T>()) block_lu_kernel(T* A, int64_t lda, int64_t r, int64_t n, int bs,
                                                       gk_info* info) {
    __shared__ T Ds[kLNB][kLNB + 1];
    __shared__ int s_bad;
    const int64_t b0 = r + (int64_t)blockIdx.x * bs;
    const int nb = (int)min((int64_t)bs, n - b0);
    if (nb <= 0) return;
    if (!cta_lu_nopiv(A + b0 * lda + b0, (int)lda, nb, Ds, &s_bad)) {
        if (threadIdx.x == 0) report(info, GK_ERR_SINGULAR, (int)b0);
    }
}

template <typename T>
__global__ void __launch_bounds__(256) block_solve_kernel(const T* A, int64_t lda, int64_t r, int64_t n, int bs,
                                                          T* t) {
    __shared__ T xs[kLNB];
    const int64_t b0 = r + (int64_t)blockIdx.x * bs;
    const int nb = (int)min((int64_t)bs, n - b0);
    if (nb <= 0) return;
    cta_lu_solve(A + b0 * lda + b0, (int)lda, nb, t + b0, xs);
}

// Explicit inverses of the Schur diagonal blocks, so that the block-Jacobi
// step of every application is a matrix-vector product instead of two
// latency-bound in-CTA triangular sweeps.  The inverse of block b (rows and
// columns [b0, b0 + nb)) is stored in rows [b0, b0 + nb) of an off-diagonal
// column range of the Schur part, which the preconditioner never reads: the
// next block's columns when that block is full, else the previous block's.
// Used with FP64 storage when at least two blocks are full (every block then
// has a home): the inverses cost ~40 ms of setup and save ~0.3 ms per FP64
// application; FP32 configurations converge in too few iterations to gain.
template <typename T>
__host__ __device__ inline bool block_inverse_mode(int64_t n, int64_t r, int bs) {
    return sizeof(T) == 8 && (n - r) / bs >= 2;
}

__host__ __device__ inline int64_t block_inverse_col(int64_t n, int64_t r, int bs, int64_t b) {
    const int64_t nfull = (n - r) / bs;
    const int64_t b0 = r + b * bs;
    return b + 1 < nfull ? b0 + bs : b0 - bs;
}

// X = U^-1 L^-1 of the LU (unit L) held in the diagonal block; one CTA per
// block, one thread per column of X (column-parallel substitutions; the
// factor entry of a step is the same for the whole warp).
template <typename T>
__global__ void __launch_bounds__(256) block_inv_kernel(T* A, int64_t lda, int64_t r, int64_t n, int bs) {
    const int64_t b = blockIdx.x;
    const int64_t b0 = r + b * bs;
    const int nb = (int)min((int64_t)bs, n - b0);
    if (nb <= 0) return;
    const T* F = A + b0 * lda + b0;
    T* X = A + b0 * lda + block_inverse_col(n, r, bs, b);
    for (int j = threadIdx.x; j < nb; j += blockDim.x) {
        // L^-1 e_j (lower triangular: rows >= j)
        for (int i = 0; i < j; ++i) X[(int64_t)i * lda + j] = (T)0;
        X[(int64_t)j * lda + j] = (T)1;
        for (int i = j + 1; i < nb; ++i) {
            const T* Li = F + (int64_t)i * lda;
            T s = (T)0;
            for (int k = j; k < i; ++k) s = cta_fma(Li[k], X[(int64_t)k * lda + j], s);
            X[(int64_t)i * lda + j] = -s;
        }
        // U^-1 (in place, rows descending)
        for (int i = nb - 1; i >= 0; --i) {
            const T* Ui = F + (int64_t)i * lda;
            T s = X[(int64_t)i * lda + j];
            for (int k = i + 1; k < nb; ++k) s = cta_fma(-Ui[k], X[(int64_t)k * lda + j], s);
            X[(int64_t)i * lda + j] = s / Ui[i];
        }
    }
}

// t_b <- inv(S_b) t_b for every block: t_b is staged in shared memory, then
// each warp computes kInvRows rows at once (one accumulator per row, so
// kInvRows independent loads are in flight per lane).
constexpr int kInvRows = 8;

template <typename T>
__global__ void __launch_bounds__(512) block_inv_apply_kernel(const T* __restrict__ A, int64_t lda, int64_t r,
                                                              int64_t n, int bs, T* t) {
    extern __shared__ unsigned char smem_raw[];
    T* ts = reinterpret_cast<T*>(smem_raw);
    const int64_t b = blockIdx.x;
    const int64_t b0 = r + b * bs;
    const int nb = (int)min((int64_t)bs, n - b0);
    if (nb <= 0) return;
    for (int j = threadIdx.x; j < nb; j += blockDim.x) ts[j] = t[b0 + j];
    __syncthreads();
    const T* X = A + b0 * lda + block_inverse_col(n, r, bs, b);
    const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int i0 = (threadIdx.x >> 5) * kInvRows; i0 < nb; i0 += nw * kInvRows) {
        T acc[kInvRows];
#pragma unroll
        for (int q = 0; q < kInvRows; ++q) acc[q] = (T)0;
        for (int j = lane; j < nb; j += 32) {
            const T tj = ts[j];
#pragma unroll
            for (int q = 0; q < kInvRows; ++q)
                if (i0 + q < nb) acc[q] = cta_fma(X[(int64_t)(i0 + q) * lda + j], tj, acc[q]);
        }
#pragma unroll
        for (int q = 0; q < kInvRows; ++q) {
            T v = acc[q];
            for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
            acc[q] = v;
        }
        if (lane == 0) {
#pragma unroll
            for (int q = 0; q < kInvRows; ++q)
                if (i0 + q < nb) t[b0 + i0 + q] = acc[q];
        }
    }
}

// y[i] -= sum_j A[i][j] x[j], i in [r_lo, r_hi), j in [c_lo, c_hi).  One warp
// per kRectRows consecutive rows, so each x element is loaded once for all of
// them; 16-byte loads of A when the row segments are 16-byte aligned.
constexpr int kRectRows = 4;

template <typename T> struct Vec16;
template <> struct Vec16<float> {
    static constexpr int W = 4;
    __device__ static void load(const float* p, float* o) {
        const float4 v = *reinterpret_cast<const float4*>(p);
        o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
    }
};
template <> struct Vec16<double> {
    static constexpr int W = 2;
    __device__ static void load(const double* p, double* o) {
        const double2 v = *reinterpret_cast<const double2*>(p);
        o[0] = v.x; o[1] = v.y;
    }
};

template <typename T>
__global__ void __launch_bounds__(256) rect_gemv_kernel(const T* __restrict__ A, int64_t lda, int64_t r_lo,
                                                        int64_t r_hi, int64_t c_lo, int64_t c_hi,
                                                        const T* __restrict__ x, T* __restrict__ y) {
    constexpr int W = Vec16<T>::W;
    const int64_t row0 = r_lo + (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * kRectRows;
    const int lane = threadIdx.x & 31;
    if (row0 >= r_hi) return;
    const int nr = (int)min((int64_t)kRectRows, r_hi - row0);
    T acc[kRectRows];
#pragma unroll
    for (int r = 0; r < kRectRows; ++r) acc[r] = (T)0;
    int64_t j0 = c_lo;
    if ((lda % W) == 0 && (c_lo % W) == 0 && ((uintptr_t)A % 16) == 0) {
        const int64_t nv = (c_hi - c_lo) / W;
        for (int64_t q = lane; q < nv; q += 32) {
            const int64_t j = c_lo + q * W;
            T xv[W];
#pragma unroll
            for (int e = 0; e < W; ++e) xv[e] = x[j + e];
#pragma unroll
            for (int r = 0; r < kRectRows; ++r) {
                if (r < nr) {
                    T av[W];
                    Vec16<T>::load(A + (row0 + r) * lda + j, av);
#pragma unroll
                    for (int e = 0; e < W; ++e) acc[r] = cta_fma(av[e], xv[e], acc[r]);
                }
            }
        }
        j0 = c_lo + nv * W;
    }
    for (int64_t j = j0 + lane; j < c_hi; j += 32) {
        const T xv = x[j];
#pragma unroll
        for (int r = 0; r < kRectRows; ++r)
            if (r < nr) acc[r] = cta_fma(A[(row0 + r) * lda + j], xv, acc[r]);
    }
#pragma unroll
    for (int r = 0; r < kRectRows; ++r)
        for (int o = 16; o > 0; o >>= 1) acc[r] += __shfl_down_sync(0xffffffffu, acc[r], o);
    if (lane == 0) {
#pragma unroll
        for (int r = 0; r < kRectRows; ++r)
            if (r < nr) y[row0 + r] -= acc[r];
    }
}

static unsigned rect_blocks(int64_t rows) { return (unsigned)(((rows + kRectRows - 1) / kRectRows * 32 + 255) / 256); }

template <typename T>
__global__ void permute_scale_kernel(const double* __restrict__ K, int64_t ldk, int64_t n,
                                     const int32_t* __restrict__ perm, const double* __restrict__ d,
                                     T* __restrict__ A, int64_t lda) {
    const int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (row >= n) return;
    const int64_t pi = perm[row];
    const double di = d[pi];
    const double* k = K + pi * ldk;
    T* a = A + row * lda;
    for (int64_t j = lane; j < n; j += 32) {
        const int64_t pj = perm[j];
        a[j] = (T)(di * k[pj] * d[pj]);
    }
}

template <typename T>
__global__ void gather_scale_kernel(const double* __restrict__ v, const int32_t* __restrict__ perm,
                                    const double* __restrict__ d, int64_t n, T* __restrict__ t) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const int64_t p = perm[i];
        t[i] = (T)(d[p] * v[p]);
    }
}

template <typename T>
__global__ void scatter_scale_kernel(const T* __restrict__ t, const int32_t* __restrict__ perm,
                                     const double* __restrict__ d, int64_t n, double* __restrict__ z) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const int64_t p = perm[i];
        z[p] = d[p] * (double)t[i];
    }
}

cudaError_t wait_cap_set_eval(long long v);
cudaError_t wait_cap_set_batch(long long v);

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
// Two-level setup: A (n x lda, FP32 or FP64) <- P D K D P^T, partial LU over the first
// r columns with restricted updates, LU of the Schur diagonal blocks, and the
// inverses of the 128 x 128 diagonal blocks of L_LL / U_LL for the solves.
template <typename T>
static gk_status twolevel_setup(int64_t n, const double* K, int64_t ldk, const int32_t* perm, const double* d,
                                     int64_t r, int bs, T* A, int64_t lda, int32_t* ipiv, void* work,
                                     size_t wbytes, gk_info* info, cudaStream_t st, float* ffpanel = nullptr) {
    constexpr int NB = LuCfg<T>::NB;
    if (n <= 0 || r <= 0 || r >= n || bs <= 0 || (r % 64) != 0 || (bs % 64) != 0 || (lda % 4) != 0 ||
        ((uintptr_t)A % 16) != 0)
        return GK_ERR_ARG;
    if (work == nullptr || wbytes < lu_ws_bytes<T>(n)) return GK_ERR_SIZE;
    permute_scale_kernel<T><<<(unsigned)((n * 32 + 255) / 256), 256, 0, st>>>(K, ldk, n, perm, d, A, lda);
    GK_LAUNCH_CHECK();
    const int64_t nblk = (n - r + bs - 1) / bs;
    if (sizeof(T) == 8 && ffpanel != nullptr) {
        // float-float updates, two LU steps per trailing update (r % 64 == 0)
        double* Ad = (double*)A;
        constexpr int BT = 64;
        float* Lh = ffpanel;
        float* Ll = Lh + n * kFfPair;
        float* Uh = Ll + n * kFfPair;
        float* Ul = Uh + n * kFfPair;
        auto step = [&](int64_t kk) -> gk_status {  // diagonal block, L below it, U right of it
            diag_lu_kernel<T, NB><<<1, 256, 0, st>>>(A, lda, kk, NB, ipiv, info);
            GK_LAUNCH_CHECK();
            const int64_t rest = n - kk - NB;
            trsm_right_kernel<T, NB><<<(unsigned)((rest + kTrsmRows - 1) / kTrsmRows), kTrsmRows * kTrsmLanes, 0,
                                       st>>>(A, lda, n, kk, NB);
            GK_LAUNCH_CHECK();
            trsm_kernel<T, NB><<<(unsigned)((rest + 127) / 128), 128, 0, st>>>(A, lda, n, kk, NB);
            GK_LAUNCH_CHECK();
            return GK_OK;
        };
        auto update = [&](int kb, int64_t r_lo, int64_t r_hi, int64_t c_lo, int64_t c_hi, int diag) -> gk_status {
            if (r_hi <= r_lo || c_hi <= c_lo) return GK_OK;
            const int64_t rows = diag ? diag : r_hi - r_lo, cols = diag ? diag : c_hi - c_lo;
            dim3 g((unsigned)((cols + BT - 1) / BT), (unsigned)((rows + BT - 1) / BT), diag ? (unsigned)nblk : 1u);
            ffgemm_range_kernel<<<g, 256, 0, st>>>(Ad, lda, n, kb, Lh, Ll, Uh, Ul, r_lo, r_hi, c_lo, c_hi, diag);
            GK_LAUNCH_CHECK();
            return GK_OK;
        };
        const unsigned sgrid = 4 * kSMs;
        gk_status e;
        for (int64_t k = 0; k < r; k += kFfPair) {
            const int64_t o1 = k + kFfPanel, o2 = k + kFfPair;
            if ((e = step(k)) != GK_OK) return e;
            split_panel_kernel<<<sgrid, 256, 0, st>>>(Ad, lda, n, k, kFfPanel, o1, 0, Lh, Ll, Uh, Ul);
            GK_LAUNCH_CHECK();
            // the second step's columns (all rows below) and rows (all columns right)
            if ((e = update(kFfPanel, o1, n, o1, o2, 0)) != GK_OK) return e;
            if ((e = update(kFfPanel, o1, o2, o2, n, 0)) != GK_OK) return e;
            if ((e = step(o1)) != GK_OK) return e;
            split_panel_kernel<<<sgrid, 256, 0, st>>>(Ad, lda, n, o1, kFfPanel, o2, kFfPanel, Lh, Ll, Uh, Ul);
            GK_LAUNCH_CHECK();
            // both steps at once: landmark rows x all columns, other rows x landmark
            // columns, diagonal blocks of the Schur complement
            if ((e = update(kFfPair, o2, r, o2, n, 0)) != GK_OK) return e;
            if ((e = update(kFfPair, r, n, o2, r, 0)) != GK_OK) return e;
            if ((e = update(kFfPair, r, n, r, n, bs)) != GK_OK) return e;
        }
    }
    for (int64_t k = 0; k < r && ffpanel == nullptr; k += NB) {
        const int kb = (int)min((int64_t)NB, r - k);
        diag_lu_kernel<T, NB><<<1, 256, 0, st>>>(A, lda, k, kb, ipiv, info);
        GK_LAUNCH_CHECK();
        const int64_t rest = n - k - kb;
        trsm_right_kernel<T, NB><<<(unsigned)((rest + kTrsmRows - 1) / kTrsmRows), kTrsmRows * kTrsmLanes, 0, st>>>(
                A, lda, n, k, kb);
        GK_LAUNCH_CHECK();
        trsm_kernel<T, NB><<<(unsigned)((rest + 127) / 128), 128, 0, st>>>(A, lda, n, k, kb);
        GK_LAUNCH_CHECK();
        const int64_t o = k + kb;
        if (sizeof(T) == 8) {
            double* Ad = (double*)A;
            constexpr int BT = 64;
            if (o < r) {
                dim3 ga((unsigned)((n - o + BT - 1) / BT), (unsigned)((r - o + BT - 1) / BT));
                gemm_range_kernel<double, BT, BT, 16><<<ga, 256, 0, st>>>(Ad, lda, k, kb, o, r, o, n, 0);
                GK_LAUNCH_CHECK();
                dim3 gb((unsigned)((r - o + BT - 1) / BT), (unsigned)((n - r + BT - 1) / BT));
                gemm_range_kernel<double, BT, BT, 16><<<gb, 256, 0, st>>>(Ad, lda, k, kb, r, n, o, r, 0);
                GK_LAUNCH_CHECK();
            }
            dim3 gc((unsigned)((bs + BT - 1) / BT), (unsigned)((bs + BT - 1) / BT), (unsigned)nblk);
            gemm_range_kernel<double, BT, BT, 16><<<gc, 256, 0, st>>>(Ad, lda, k, kb, r, n, r, n, bs);
            GK_LAUNCH_CHECK();
            continue;
        }
        float* Af = (float*)A;
        if (o < r) {
            // landmark rows, all columns to the right
            gk_status s = sgemm_update(Af, lda, k, kb, o, r, o, n, 0, 1, info, st);
            if (s != GK_OK) return s;
            // remaining rows, landmark columns
            s = sgemm_update(Af, lda, k, kb, r, n, o, r, 0, 1, info, st);
            if (s != GK_OK) return s;
        }
        // diagonal blocks of the Schur complement
        gk_status s = sgemm_update(Af, lda, k, kb, r, n, r, n, bs, (unsigned)nblk, info, st);
        if (s != GK_OK) return s;
    }
    block_lu_kernel<T><<<(unsigned)nblk, block_lu_threads<T>(), 0, st>>>(A, lda, r, n, bs, info);
    GK_LAUNCH_CHECK();
    if (block_inverse_mode<T>(n, r, bs)) {
        block_inv_kernel<T><<<(unsigned)nblk, 256, 0, st>>>(A, lda, r, n, bs);
        GK_LAUNCH_CHECK();
    }
    const size_t ysmem = (size_t)kTB * kTB * sizeof(T);
    GK_CUDA_TRY(cudaFuncSetAttribute(tri_inv_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ysmem));
    tri_inv_kernel<T><<<(unsigned)((r + kTB - 1) / kTB), kTB, ysmem, st>>>(A, lda, r, lu_ws_dinv<T>(work, r, 0),
                                                                          lu_ws_dinv<T>(work, r, 1), info);
    GK_LAUNCH_CHECK();
    return GK_OK;
}

// z = M^-1 v (FP64 in/out; T inside).  t: n values of scratch.
template <typename T>
static gk_status twolevel_apply(int64_t n, const T* A, int64_t lda, const int32_t* perm, const double* d,
                                     int64_t r, int bs, const double* v, double* z, T* t, void* work,
                                     size_t wbytes, gk_info* info, cudaStream_t st) {
    const unsigned vb = (unsigned)((n + 255) / 256);
    gather_scale_kernel<T><<<vb, 256, 0, st>>>(v, perm, d, n, t);
    GK_LAUNCH_CHECK();
    // forward: L_LL w_L = t_L, then t_R -= L_RL w_L
    int sms = device_sm_count();
    // flags and diagonal inverses both use the workspace layout of order r
    char* p = (char*)work + panel_ws_bytes<T, LuCfg<T>::NB>(sms);
    p += align256((size_t)(r + 1) * sizeof(int32_t)) * 2;
    const int nblk_r = (int)((r + kTB - 1) / kTB);
    int* flags = (int*)p;
    int* counter = flags + (size_t)nblk_r * kFlagStride;
    GK_CUDA_TRY(cudaMemsetAsync(flags, 0, ((size_t)nblk_r + 1) * kFlagStride * sizeof(int), st));
    trsv_kernel<T><<<nblk_r, 256, 0, st>>>(A, lda, r, t, lu_ws_dinv<T>(work, r, 0), 1, counter, flags, info);
    GK_LAUNCH_CHECK();
    rect_gemv_kernel<T><<<rect_blocks(n - r), 256, 0, st>>>(A, lda, r, n, 0, r, t, t);
    GK_LAUNCH_CHECK();
    // block-Jacobi on the Schur complement
    const int64_t nblk = (n - r + bs - 1) / bs;
    if (block_inverse_mode<T>(n, r, bs)) {
        block_inv_apply_kernel<T><<<(unsigned)nblk, 512, (size_t)bs * sizeof(T), st>>>(A, lda, r, n, bs, t);
    } else {
        block_solve_kernel<T><<<(unsigned)nblk, 256, 0, st>>>(A, lda, r, n, bs, t);
    }
    GK_LAUNCH_CHECK();
    // backward: t_L -= U_LR x_R, then U_LL x_L = t_L
    rect_gemv_kernel<T><<<rect_blocks(r), 256, 0, st>>>(A, lda, 0, r, r, n, t, t);
    GK_LAUNCH_CHECK();
    GK_CUDA_TRY(cudaMemsetAsync(flags, 0, ((size_t)nblk_r + 1) * kFlagStride * sizeof(int), st));
    trsv_kernel<T><<<nblk_r, 256, 0, st>>>(A, lda, r, t, lu_ws_dinv<T>(work, r, 1), 0, counter, flags, info);
    GK_LAUNCH_CHECK();
    scatter_scale_kernel<T><<<vb, 256, 0, st>>>(t, perm, d, n, z);
    GK_LAUNCH_CHECK();
    return GK_OK;
}

gk_status gk_internal_lu_factor_nopiv_f32(int64_t n, float* A, int64_t lda, int32_t* ipiv, void* work, size_t wb,
                                          gk_info* info, cudaStream_t st) {
    return lu_factor_nopiv<float>(n, A, lda, ipiv, work, wb, info, st);
}

gk_status gk_internal_twolevel_setup(int64_t n, const double* K, int64_t ldk, const int32_t* perm, const double* d,
                                     int64_t r, int bs, float* A, int64_t lda, int32_t* ipiv, void* work,
                                     size_t wbytes, gk_info* info, cudaStream_t st) {
    return twolevel_setup<float>(n, K, ldk, perm, d, r, bs, A, lda, ipiv, work, wbytes, info, st);
}
gk_status gk_internal_twolevel_setup_f64(int64_t n, const double* K, int64_t ldk, const int32_t* perm,
                                         const double* d, int64_t r, int bs, double* A, int64_t lda, int32_t* ipiv,
                                         void* work, size_t wbytes, gk_info* info, cudaStream_t st,
                                         float* ffpanel) {
    return twolevel_setup<double>(n, K, ldk, perm, d, r, bs, A, lda, ipiv, work, wbytes, info, st, ffpanel);
}
size_t gk_internal_ff_panel_floats(int64_t n) { return (size_t)4 * kFfPair * (size_t)n; }
gk_status gk_internal_twolevel_apply(int64_t n, const float* A, int64_t lda, const int32_t* perm, const double* d,
                                     int64_t r, int bs, const double* v, double* z, float* t, void* work,
                                     size_t wbytes, gk_info* info, cudaStream_t st) {
    return twolevel_apply<float>(n, A, lda, perm, d, r, bs, v, z, t, work, wbytes, info, st);
}
gk_status gk_internal_twolevel_apply_f64(int64_t n, const double* A, int64_t lda, const int32_t* perm,
                                         const double* d, int64_t r, int bs, const double* v, double* z, double* t,
                                         void* work, size_t wbytes, gk_info* info, cudaStream_t st) {
    return twolevel_apply<double>(n, A, lda, perm, d, r, bs, v, z, t, work, wbytes, info, st);
}
size_t gk_internal_lu_ws_f64(int64_t n) { return lu_ws_bytes<double>(n); }

extern "C" gk_status gk_set_wait_limit(int64_t spins) {
    const long long v = spins < 0 ? -1 : (long long)spins;
    if (set_wait_cap_here(v) != cudaSuccess) return GK_ERR_CUDA;
    if (wait_cap_set_lu_tc(v) != cudaSuccess) return GK_ERR_CUDA;
    if (wait_cap_set_eval(v) != cudaSuccess) return GK_ERR_CUDA;
    if (wait_cap_set_batch(v) != cudaSuccess) return GK_ERR_CUDA;
    return GK_OK;
}
