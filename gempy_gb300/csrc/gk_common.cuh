// Shared device helpers of the co-kriging kernels: covariance functions,
// status reporting and a bounded grid barrier for cooperative launches.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <map>
#include <mutex>
#include <tuple>

#include "../../include/gempy_gb300.h"

#define GK_CUDA_TRY(expr)                                   \
    do {                                                    \
        cudaError_t _e = (expr);                            \
        if (_e != cudaSuccess) return GK_ERR_CUDA;          \
    } while (0)

// Process-wide count of kernels this library has launched (telemetry).
inline std::atomic<unsigned long long>& gk_launch_counter() {
    static std::atomic<unsigned long long> c{0};
    return c;
}

#define GK_LAUNCH_CHECK()                                   \
    do {                                                    \
        gk_launch_counter().fetch_add(1, std::memory_order_relaxed); \
        if (cudaPeekAtLastError() != cudaSuccess) {         \
            (void)cudaGetLastError();                       \
            return GK_ERR_CUDA;                             \
        }                                                   \
    } while (0)

namespace gk {

constexpr int kSMs = 152;  // GB300: 2 dies x 76 SMs (queried at run time too)

// Regulariser of h_u h_v / r^2 in the gradient-gradient block.
constexpr double kGradEps = 1e-5;

// Every distance is r = sqrt(|h|^2 + kDistEps2).  The reference engine
// differentiates its kernel with PyTorch autodiff with respect to the point
// and orientation positions and asserts finite gradients
// (test/test_modules/test_ad/test_ad_I.py:48-54), which a bare sqrt at r = 0
// (the diagonal) would make NaN, so its distances carry a regulariser.  The
// value 1e-10 (r = 1e-5 at coincident points, transformed frame) is the one
// the anticline approval file selects; it moves C'/r(0) by 105/4 * 1e-5 / a^3.
constexpr double kDistEps2 = 1e-10;

// Default iteration caps of the spin waits: ~seconds at worst, then the
// kernel records GK_ERR_TIMEOUT and returns instead of hanging the GPU.
constexpr long long kSpinLimit = 20LL * 1000 * 1000;  // inter-CTA waits (grid barrier, block flags)
constexpr long long kCopySpin = 4LL * 1000 * 1000;    // bulk-copy completion waits (mbarrier)

// Cap in force for the waits of this module (each translation unit has its
// own copy): negative selects the defaults above.  gk_set_wait_limit sets it
// so tests can make the waits run out (0: give up before the first poll).
// A CTA that gave up still waits for its bulk copies in flight with the
// default cap before it exits.
static __constant__ long long g_wait_cap = -1;
__device__ __forceinline__ long long wait_cap(long long dflt) { return g_wait_cap < 0 ? dflt : g_wait_cap; }
static inline cudaError_t set_wait_cap_here(long long v) {
    return cudaMemcpyToSymbol(g_wait_cap, &v, sizeof(v));
}

__host__ __device__ inline int drift_count(int degree) {
    return degree == 1 ? 3 : (degree == 2 ? 9 : 0);
}

// Radial covariance with unit sill and its radial derivatives:
//   C(r), C'(r)/r, C''(r), (C'/r)'(r)/r.
// Cubic: C = 1 - 7 s^2 + 35/4 s^3 - 7/2 s^5 + 3/4 s^7 for s = r/a < 1, else 0.
// Exponential: squared exponential exp(-r^2 / (2 a^2)).
template <typename T>
struct Cov {
    int kind;
    T a, ia, ia2, ia4;  // a, 1/a, 1/a^2, 1/a^4

    __host__ __device__ static Cov make(int kind, double a) {
        Cov c;
        c.kind = kind;
        c.a = (T)a;
        c.ia = (T)(1.0 / a);
        c.ia2 = (T)(1.0 / (a * a));
        c.ia4 = (T)(1.0 / (a * a * a * a));
        return c;
    }

    __device__ __forceinline__ T C(T r) const {
        if (kind == GK_KERNEL_CUBIC) {
            T s = r * ia;
            if (s >= (T)1) return (T)0;
            T s2 = s * s;
            return (T)1 + s2 * ((T)-7 + s * ((T)8.75 + s2 * ((T)-3.5 + (T)0.75 * s2)));
        }
        return gexp(-(T)0.5 * r * r * ia2);
    }
    __device__ __forceinline__ T d1_r(T r) const {
        if (kind == GK_KERNEL_CUBIC) {
            T s = r * ia;
            if (s >= (T)1) return (T)0;
            T s2 = s * s;
            return ia2 * ((T)-14 + s * ((T)26.25 + s2 * ((T)-17.5 + (T)5.25 * s2)));
        }
        return -ia2 * gexp(-(T)0.5 * r * r * ia2);
    }
    __device__ __forceinline__ T d2(T r) const {
        if (kind == GK_KERNEL_CUBIC) {
            T s = r * ia;
            if (s >= (T)1) return (T)0;
            T s2 = s * s;
            return ia2 * ((T)-14 + s * ((T)52.5 + s2 * ((T)-70 + (T)31.5 * s2)));
        }
        T e = gexp(-(T)0.5 * r * r * ia2);
        return (r * r * ia4 - ia2) * e;
    }
    // (C'/r)'/r; finite at r = 0 is enough (it multiplies terms O(r^2)).
    __device__ __forceinline__ T d3_r(T r) const {
        if (kind == GK_KERNEL_CUBIC) {
            T s = r * ia;
            if (s >= (T)1 || s <= (T)0) return (T)0;
            T s2 = s * s;
            return ia4 * ((T)26.25 / s + s * ((T)-52.5 + (T)26.25 * s2));
        }
        return ia4 * gexp(-(T)0.5 * r * r * ia2);
    }
    __device__ __forceinline__ static T gexp(T x);
};

template <>
__device__ __forceinline__ double Cov<double>::gexp(double x) { return exp(x); }
template <>
__device__ __forceinline__ float Cov<float>::gexp(float x) { return expf(x); }

template <typename T>
__device__ __forceinline__ T gsqrt(T x);
template <>
__device__ __forceinline__ double gsqrt<double>(double x) { return sqrt(x); }
template <>
__device__ __forceinline__ float gsqrt<float>(float x) { return sqrtf(x); }

// Records the first failure into a device info word.
__device__ inline void report(gk_info* info, int status, int where) {
    if (info == nullptr) return;
    if (atomicCAS(&info->status, 0, status) == 0) info->where = where;
}

// Sense-free grid barrier for cooperative launches.  ``bar[0]`` counts
// arrivals, ``bar[1]`` is the generation.  Every wait is bounded: on timeout
// the barrier sets ``*abort`` and reports GK_ERR_TIMEOUT; callers test
// ``*abort`` after each barrier and return.
struct GridBarrier {
    unsigned int* bar;      // 2 words, zero before the launch
    volatile int* abort;    // 1 word, zero before the launch
    gk_info* info;

    __device__ bool sync(unsigned int nblocks) {
        __syncthreads();
        __shared__ int s_ok;
        if (threadIdx.x == 0) {
            s_ok = 1;
            unsigned int gen = atomicAdd(&bar[1], 0u);
            __threadfence();
            unsigned int arrived = atomicAdd(&bar[0], 1u);
            if (arrived == nblocks - 1) {
                atomicExch(&bar[0], 0u);
                __threadfence();
                atomicAdd(&bar[1], 1u);
            } else {
                const long long cap = wait_cap(kSpinLimit);
                for (long long spins = 0;; ++spins) {
                    if (spins >= cap) {
                        *abort = 1;
                        report(info, GK_ERR_TIMEOUT, -1);
                        s_ok = 0;
                        break;
                    }
                    unsigned int g;
                    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(g) : "l"(bar + 1) : "memory");
                    if (g != gen) break;
                    if (*abort) { s_ok = 0; break; }
                }
            }
            __threadfence();
        }
        __syncthreads();
        return s_ok != 0;
    }
};

inline int device_sm_count() {
    static std::atomic<int> cache[64];
    int dev = 0, n = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return kSMs;
    if (dev >= 0 && dev < 64 && (n = cache[dev].load(std::memory_order_relaxed)) > 0) return n;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) return kSMs;
    if (dev >= 0 && dev < 64) cache[dev].store(n, std::memory_order_relaxed);
    return n;
}

// Resident CTAs per SM of ``kernel`` at ``threads`` threads and ``smem`` bytes
// of dynamic shared memory; computed once per (kernel, threads, smem, device)
// and cached, so launches of small point sets do not pay the runtime queries
// each time.  The kernel's dynamic shared-memory limit is only ever raised
// (to the largest size requested so far on the device), so every cached
// configuration stays launchable.
inline gk_status cached_occupancy(const void* kernel, int threads, size_t smem, int& occ) {
    static std::mutex mu;
    static std::map<std::tuple<const void*, int, size_t, int>, int> table;
    static std::map<std::pair<const void*, int>, size_t> limit;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return GK_ERR_CUDA;
    const auto key = std::make_tuple(kernel, threads, smem, dev);
    std::lock_guard<std::mutex> g(mu);
    auto it = table.find(key);
    if (it != table.end()) {
        occ = it->second;
        return GK_OK;
    }
    size_t& lim = limit[std::make_pair(kernel, dev)];
    if (smem > lim) {
        if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
            return GK_ERR_CUDA;
        lim = smem;
    }
    int o = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, kernel, threads, smem) != cudaSuccess) return GK_ERR_CUDA;
    occ = o < 1 ? 1 : o;
    table[key] = occ;
    return GK_OK;
}

// Whether clusters of `size` CTAs of `kernel` (threads, smem bytes of dynamic
// shared memory each) can be scheduled on the device; cached.  Sizes above 8
// are opted into on the kernel first.  Call after cached_occupancy with the
// same smem, which raises the kernel's shared-memory limit.
inline bool cached_cluster_fits(const void* kernel, int threads, size_t smem, int size) {
    static std::mutex mu;
    static std::map<std::tuple<const void*, int, size_t, int, int>, bool> table;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return false;
    const auto key = std::make_tuple(kernel, threads, smem, size, dev);
    std::lock_guard<std::mutex> g(mu);
    auto it = table.find(key);
    if (it != table.end()) return it->second;
    bool ok = true;
    if (size > 8 && cudaFuncSetAttribute(kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess)
        ok = false;
    if (ok) {
        cudaLaunchConfig_t cfg = {};
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = (unsigned)size;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.gridDim = dim3((unsigned)size);
        cfg.blockDim = dim3((unsigned)threads);
        cfg.dynamicSmemBytes = smem;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        int nc = 0;
        ok = cudaOccupancyMaxActiveClusters(&nc, kernel, &cfg) == cudaSuccess && nc > 0;
    }
    if (!ok) (void)cudaGetLastError();
    table[key] = ok;
    return ok;
}

}  // namespace gk
