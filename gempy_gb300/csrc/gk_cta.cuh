// In-CTA dense kernels shared by the batched solver (gk_batch.cu) and the
// two-level preconditioner (gk_lu.cu): blocked LU without pivoting of an
// FP32 or FP64 matrix by one CTA, and the matching triangular solves (the
// matrix may sit in global or in shared memory: generic addressing); and a
// register-resident Gauss-Jordan inversion of a small FP32 matrix.
#pragma once

#include "gk_common.cuh"

namespace gk {

constexpr int kLNB = 32;

template <typename T> __device__ __forceinline__ T cta_fma(T a, T b, T c);
template <> __device__ __forceinline__ float cta_fma(float a, float b, float c) { return fmaf(a, b, c); }
template <> __device__ __forceinline__ double cta_fma(double a, double b, double c) { return fma(a, b, c); }
template <typename T> __device__ __forceinline__ T cta_abs(T x) { return x < (T)0 ? -x : x; }

// In-CTA blocked LU without pivoting of A (N x ld, FP32 or FP64); returns false on a
// zero / non-finite pivot.
template <typename T>
static __device__ bool cta_lu_nopiv(T* A, int ld, int N, T (*Ds)[kLNB + 1], int* s_bad) {
    const int tid = threadIdx.x, nt = blockDim.x;
    if (tid == 0) *s_bad = 0;
    __syncthreads();
    for (int k = 0; k < N; k += kLNB) {
        const int kb = min(kLNB, N - k);
        for (int idx = tid; idx < kLNB * kLNB; idx += nt) {
            int r = idx / kLNB, c = idx % kLNB;
            Ds[r][c] = (r < kb && c < kb) ? A[(int64_t)(k + r) * ld + k + c] : (T)0;
        }
        __syncthreads();
        for (int j = 0; j < kb; ++j) {
            const T pv = Ds[j][j];
            if (!(pv == pv) || pv == (T)0 || !(cta_abs(pv) < (T)INFINITY)) {
                if (tid == 0) *s_bad = 1;
            }
            __syncthreads();
            if (*s_bad) return false;
            const T inv = (T)1 / pv;
            for (int i = j + 1 + tid; i < kb; i += nt) Ds[i][j] *= inv;
            __syncthreads();
            const int w = kb - j - 1;
            for (int idx = tid; idx < w * w; idx += nt) {
                const int i = j + 1 + idx / w, c = j + 1 + idx % w;
                Ds[i][c] -= Ds[i][j] * Ds[j][c];
            }
            __syncthreads();
        }
        for (int idx = tid; idx < kb * kb; idx += nt) {
            int r = idx / kb, c = idx % kb;
            A[(int64_t)(k + r) * ld + k + c] = Ds[r][c];
        }
        const int m = N - k - kb;
        if (m > 0) {
            // U12 = L11^-1 A12 (thread per column) and L21 = A21 U11^-1 (thread per row)
            for (int c = tid; c < m; c += nt) {
                T xv[kLNB];
                const int64_t col = k + kb + c;
#pragma unroll
                for (int i = 0; i < kLNB; ++i) xv[i] = i < kb ? A[(int64_t)(k + i) * ld + col] : (T)0;
#pragma unroll
                for (int i = 1; i < kLNB; ++i) {
                    T s = xv[i];
#pragma unroll
                    for (int q = 0; q < i; ++q) s -= Ds[i][q] * xv[q];
                    xv[i] = s;
                }
#pragma unroll
                for (int i = 0; i < kLNB; ++i)
                    if (i < kb) A[(int64_t)(k + i) * ld + col] = xv[i];
            }
            for (int rr = tid; rr < m; rr += nt) {
                T xv[kLNB];
                T* row = A + (int64_t)(k + kb + rr) * ld + k;
#pragma unroll
                for (int j = 0; j < kLNB; ++j) xv[j] = j < kb ? row[j] : (T)0;
#pragma unroll
                for (int j = 0; j < kLNB; ++j) {
                    if (j < kb) {
                        T s = xv[j];
#pragma unroll
                        for (int q = 0; q < j; ++q) s -= xv[q] * Ds[q][j];
                        xv[j] = s / Ds[j][j];
                    }
                }
#pragma unroll
                for (int j = 0; j < kLNB; ++j)
                    if (j < kb) row[j] = xv[j];
            }
            __syncthreads();
            // A22 -= L21 U12, 4 x 4 micro-tiles
            const int mb = (m + 3) / 4;
            for (int t = tid; t < mb * mb; t += nt) {
                const int bi = t / mb, bj = t % mb;
                T acc[4][4] = {};
                for (int p = 0; p < kb; ++p) {
                    T lv[4], uv[4];
#pragma unroll
                    for (int a = 0; a < 4; ++a) {
                        const int rr = 4 * bi + a;
                        lv[a] = rr < m ? A[(int64_t)(k + kb + rr) * ld + k + p] : (T)0;
                    }
#pragma unroll
                    for (int c = 0; c < 4; ++c) {
                        const int cc = 4 * bj + c;
                        uv[c] = cc < m ? A[(int64_t)(k + p) * ld + k + kb + cc] : (T)0;
                    }
#pragma unroll
                    for (int a = 0; a < 4; ++a)
#pragma unroll
                        for (int c = 0; c < 4; ++c) acc[a][c] = cta_fma(lv[a], uv[c], acc[a][c]);
                }
#pragma unroll
                for (int a = 0; a < 4; ++a) {
                    const int rr = 4 * bi + a;
                    if (rr >= m) continue;
#pragma unroll
                    for (int c = 0; c < 4; ++c) {
                        const int cc = 4 * bj + c;
                        if (cc < m) A[(int64_t)(k + kb + rr) * ld + k + kb + cc] -= acc[a][c];
                    }
                }
            }
        }
        __syncthreads();
    }
    return true;
}

// In-CTA triangular solves with the factors, in place on t (length N):
// forward (unit L) then backward (U), block column sweeps of kLNB.
template <typename T>
static __device__ void cta_lu_solve(const T* A, int ld, int N, T* t, T* xs) {
    const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, wid = tid >> 5;
    for (int k = 0; k < N; k += kLNB) {
        const int kb = min(kLNB, N - k);
        if (wid == 0) {
            // the lane's row of the diagonal block, loaded before the serial sweep
            T arow[kLNB];
            const T* ar = A + (int64_t)(k + (lane < kb ? lane : 0)) * ld + k;
#pragma unroll
            for (int c = 0; c < kLNB; ++c) arow[c] = c < kb ? ar[c] : (T)0;
            T v = lane < kb ? t[k + lane] : (T)0;
#pragma unroll
            for (int c = 0; c < kLNB; ++c) {
                const T xc = __shfl_sync(0xffffffffu, v, c);
                if (lane > c && lane < kb) v -= arow[c] * xc;
            }
            if (lane < kb) { t[k + lane] = v; xs[lane] = v; }
        }
        __syncthreads();
        for (int r = k + kb + tid; r < N; r += nt) {
            const T* row = A + (int64_t)r * ld + k;
            T s = (T)0;
            for (int c = 0; c < kb; ++c) s += row[c] * xs[c];
            t[r] -= s;
        }
        __syncthreads();
    }
    const int nblk = (N + kLNB - 1) / kLNB;
    for (int bk = nblk - 1; bk >= 0; --bk) {
        const int k = bk * kLNB;
        const int kb = min(kLNB, N - k);
        if (wid == 0) {
            T arow[kLNB];
            const T* ar = A + (int64_t)(k + (lane < kb ? lane : 0)) * ld + k;
#pragma unroll
            for (int c = 0; c < kLNB; ++c) arow[c] = c < kb ? ar[c] : (T)0;
            T v = lane < kb ? t[k + lane] : (T)0;
#pragma unroll
            for (int c = kLNB - 1; c >= 0; --c) {
                if (c < kb) {  // warp-uniform
                    const T mine = __shfl_sync(0xffffffffu, v, c);
                    const T dcc = __shfl_sync(0xffffffffu, arow[c], c);
                    const T xc = mine / dcc;
                    if (lane == c) v = xc;
                    if (lane < c) v -= arow[c] * xc;
                }
            }
            if (lane < kb) { t[k + lane] = v; xs[lane] = v; }
        }
        __syncthreads();
        for (int r = tid; r < k; r += nt) {
            const T* row = A + (int64_t)r * ld + k;
            T s = (T)0;
            for (int c = 0; c < kb; ++c) s += row[c] * xs[c];
            t[r] -= s;
        }
        __syncthreads();
    }
}

// In-CTA Gauss-Jordan inversion without pivoting of the N x N FP32 matrix A
// (shared memory, leading dimension lda), in place, for N <= 16 RA and
// N <= 32 CB with 512 threads.  During the elimination the matrix lives in
// registers: warp ty owns rows ty + 16 r, lane tx columns tx + 32 c.  Step k
// publishes pivot row k and column k in shared memory (rowbuf, colbuf: N
// floats each) and updates every owned element with one FMA; the owners of
// row k (one warp) and of column k (one lane per warp) then overwrite theirs.
// The pivots are those of LU without pivoting.  Returns false on a zero or
// non-finite pivot (every thread sees the same pivot).
template <int RA, int CB>
static __device__ __noinline__ bool cta_gauss_jordan_regs(float* A, int lda, int N, float* rowbuf, float* colbuf) {
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    float a[RA][CB];
#pragma unroll
    for (int r = 0; r < RA; ++r)
#pragma unroll
        for (int c = 0; c < CB; ++c) {
            const int i = ty + 16 * r, j = tx + 32 * c;
            a[r][c] = (i < N && j < N) ? A[(int64_t)i * lda + j] : 0.f;
        }
    bool ok = true;
    for (int k = 0; k < N; ++k) {
#pragma unroll
        for (int r = 0; r < RA; ++r)
            if (ty + 16 * r == k)   // warp-uniform
#pragma unroll
                for (int c = 0; c < CB; ++c)
                    if (tx + 32 * c < N) rowbuf[tx + 32 * c] = a[r][c];
#pragma unroll
        for (int c = 0; c < CB; ++c)
            if (tx + 32 * c == k)
#pragma unroll
                for (int r = 0; r < RA; ++r)
                    if (ty + 16 * r < N) colbuf[ty + 16 * r] = a[r][c];
        __syncthreads();
        const float p = colbuf[k];
        if (!(fabsf(p) > 0.f) || !(fabsf(p) < INFINITY)) { ok = false; break; }
        const float ip = 1.f / p;
        float rv[CB], cv[RA];
#pragma unroll
        for (int c = 0; c < CB; ++c) rv[c] = tx + 32 * c < N ? rowbuf[tx + 32 * c] * ip : 0.f;
#pragma unroll
        for (int r = 0; r < RA; ++r) cv[r] = ty + 16 * r < N ? colbuf[ty + 16 * r] : 0.f;
#pragma unroll
        for (int r = 0; r < RA; ++r)
#pragma unroll
            for (int c = 0; c < CB; ++c) a[r][c] = fmaf(-cv[r], rv[c], a[r][c]);
#pragma unroll
        for (int r = 0; r < RA; ++r)
            if (ty + 16 * r == k)
#pragma unroll
                for (int c = 0; c < CB; ++c) a[r][c] = rv[c];
#pragma unroll
        for (int c = 0; c < CB; ++c)
            if (tx + 32 * c == k)
#pragma unroll
                for (int r = 0; r < RA; ++r) a[r][c] = ty + 16 * r == k ? ip : -cv[r] * ip;
        __syncthreads();   // rowbuf / colbuf are rewritten by the next step
    }
    if (!ok) return false;
#pragma unroll
    for (int r = 0; r < RA; ++r)
#pragma unroll
        for (int c = 0; c < CB; ++c) {
            const int i = ty + 16 * r, j = tx + 32 * c;
            if (i < N && j < N) A[(int64_t)i * lda + j] = a[r][c];
        }
    __syncthreads();
    return true;
}

}  // namespace gk
