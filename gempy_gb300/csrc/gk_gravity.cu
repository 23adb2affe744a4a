// Forward gravity on centred grids, after segmentation.  Replaces the engine's
// gravity step behind Solutions.gravity: the reference places a kernel of
// voxels around every device (gp.set_centered_grid, gempy/API/grid_API.py:
// 99-108), takes the vertical attraction tz of each voxel per unit density
// (gp.calculate_gravity_gradient), segments the voxels in the transformed
// frame (gempy/modules/data_manipulation/_engine_factory.py:82-87) and sums
// density x tz per device (test/test_modules/test_geophysics/test_gravity.py:
// 67-89).
//
// tz is the closed-form attraction of a rectangular prism (Nagy 1966; Plouff
// 1976), z up -- mass below the device gives a negative value -- with
// G = 6.674e-3 (lengths in m, densities in g/cm^3, tz in mGal), one thread per
// voxel in FP64.  The reduction runs one CTA per device over that device's
// voxels, each thread striding the voxels and the CTA combining the partial
// sums in a fixed tree: the same inputs give the same bits.
#include "gk_common.cuh"

namespace gk {
namespace grav {

constexpr double kG = 6.674e-3;
constexpr int kThreads = 256;

__global__ void tz_kernel(int64_t n, const double* __restrict__ c, const double* __restrict__ lo,
                          const double* __restrict__ hi, double* __restrict__ tz) {
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    double b[3][2];
    for (int a = 0; a < 3; ++a) {
        b[a][0] = c[3 * v + a] - lo[3 * v + a];
        b[a][1] = c[3 * v + a] + hi[3 * v + a];
    }
    double s = 0.0;
    for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j)
            for (int k = 0; k < 2; ++k) {
                const double x = b[0][i], y = b[1][j], z = b[2][k];
                const double r = sqrt(x * x + y * y + z * z);
                const double t = x * log(y + r) + y * log(x + r) - z * atan(x * y / (z * r));
                s += ((i + j + k) & 1) ? -t : t;
            }
    tz[v] = kG * s;
}

__global__ void __launch_bounds__(kThreads) sum_kernel(int64_t n_vox, const int32_t* __restrict__ ids, int n_units,
                                                       const double* __restrict__ rho, const double* __restrict__ tz,
                                                       double* __restrict__ out) {
    __shared__ double part[kThreads];
    const int64_t d = blockIdx.x;
    const int32_t* id = ids + d * n_vox;
    double s = 0.0;
    for (int64_t v = threadIdx.x; v < n_vox; v += kThreads) {
        const int u = id[v];
        if (u >= 1 && u <= n_units) s += rho[u - 1] * tz[v];
    }
    part[threadIdx.x] = s;
    __syncthreads();
    for (int w = kThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) part[threadIdx.x] += part[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[d] = part[0];
}

}  // namespace grav
}  // namespace gk

using namespace gk;

extern "C" gk_status gk_gravity_tz(int64_t n_voxels, const double* centres, const double* lower,
                                   const double* upper, double* tz, gk_stream stream) {
    if (n_voxels < 0) return GK_ERR_ARG;
    if (n_voxels == 0) return GK_OK;
    if (centres == nullptr || lower == nullptr || upper == nullptr || tz == nullptr) return GK_ERR_ARG;
    if (n_voxels > ((int64_t)1 << 31) * 128) return GK_ERR_SIZE;
    grav::tz_kernel<<<(unsigned)((n_voxels + 127) / 128), 128, 0, (cudaStream_t)stream>>>(n_voxels, centres, lower,
                                                                                            upper, tz);
    GK_LAUNCH_CHECK();
    return GK_OK;
}

extern "C" gk_status gk_gravity(int64_t n_devices, int64_t n_voxels, const int32_t* ids, int32_t n_units,
                                const double* densities, const double* tz, double* gravity, gk_stream stream) {
    if (n_devices < 0 || n_voxels < 0 || n_units < 1) return GK_ERR_ARG;
    if (n_devices == 0) return GK_OK;
    if (gravity == nullptr || (n_voxels > 0 && (ids == nullptr || densities == nullptr || tz == nullptr)))
        return GK_ERR_ARG;
    if (n_devices > 0x7fffffff) return GK_ERR_SIZE;
    grav::sum_kernel<<<(unsigned)n_devices, grav::kThreads, 0, (cudaStream_t)stream>>>(n_voxels, ids, n_units,
                                                                                      densities, tz, gravity);
    GK_LAUNCH_CHECK();
    return GK_OK;
}
