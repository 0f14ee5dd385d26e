// k_util.cu -- state conversion between the reference's per-cell order
// (40 doubles, TPORd::outputAllStates order, SingleCell/TPORd.cc:200-252) and
// the device structure of arrays.
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace lqt {

template <typename R>
__global__ void k_pack(const double *__restrict__ aos, SoA<R> s, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double *a = aos + i * 40;
        if (s.v) s.v[i] = (R)a[0];
        if (sizeof(R) == 8) {
            for (int j = 0; j < kNConc; ++j) s.conc[j * s.ld + i] = a[1 + j];
        } else {
            float *f = reinterpret_cast<float *>(s.conc);
            for (int j = 0; j < kNConc; ++j) {
                const float hi = (float)a[1 + j];
                f[j * s.ld + i] = hi;
                f[(8 + j) * s.ld + i] = (float)(a[1 + j] - (double)hi);
            }
        }
        for (int j = 0; j < kNGate; ++j) s.gate[j * s.ld + i] = (R)a[9 + j];
    }
}

template <typename R>
__global__ void k_unpack(SoA<R> s, double *__restrict__ aos, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double *a = aos + i * 40;
        a[0] = s.v ? (double)s.v[i] : 0.0;
        if (sizeof(R) == 8) {
            for (int j = 0; j < kNConc; ++j) a[1 + j] = s.conc[j * s.ld + i];
        } else {
            const float *f = reinterpret_cast<const float *>(s.conc);
            for (int j = 0; j < kNConc; ++j) a[1 + j] = (double)f[j * s.ld + i] + (double)f[(8 + j) * s.ld + i];
        }
        for (int j = 0; j < kNGate; ++j) a[9 + j] = (double)s.gate[j * s.ld + i];
    }
}

static unsigned grid_for(int64_t n, int bs)
{
    int64_t nb = (n + bs - 1) / bs;
    return (unsigned)(nb < 1 ? 1 : (nb > 152 * 32 ? 152 * 32 : nb));
}

template <typename R> cudaError_t launch_pack(const double *aos, const SoA<R> &s, int64_t n, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    k_pack<R><<<grid_for(n, 256), 256, 0, st>>>(aos, s, n);
    return cudaGetLastError();
}
template <typename R> cudaError_t launch_unpack(const SoA<R> &s, double *aos, int64_t n, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    k_unpack<R><<<grid_for(n, 256), 256, 0, st>>>(s, aos, n);
    return cudaGetLastError();
}
template cudaError_t launch_pack<double>(const double *, const SoA<double> &, int64_t, cudaStream_t);
template cudaError_t launch_pack<float>(const double *, const SoA<float> &, int64_t, cudaStream_t);
template cudaError_t launch_unpack<double>(const SoA<double> &, double *, int64_t, cudaStream_t);
template cudaError_t launch_unpack<float>(const SoA<float> &, double *, int64_t, cudaStream_t);

}  // namespace lqt

namespace lqt {

// V of tissue voxels <-> dense grid.
template <typename R, typename T>
__global__ void k_gather_v(const R *__restrict__ vg, const int32_t *__restrict__ gidx, T *__restrict__ out, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = (T)vg[gidx ? (int64_t)gidx[i] : i];
}
template <typename R>
__global__ void k_scatter_v(const R *__restrict__ v, const int32_t *__restrict__ gidx, R *__restrict__ vg, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        vg[gidx ? (int64_t)gidx[i] : i] = v[i];
}

template <typename R, typename T>
cudaError_t launch_gather_v(const R *vg, const int32_t *gidx, T *out, int64_t n, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    k_gather_v<R, T><<<grid_for(n, 256), 256, 0, st>>>(vg, gidx, out, n);
    return cudaGetLastError();
}
template <typename R> cudaError_t launch_scatter_v(const R *v, const int32_t *gidx, R *vg, int64_t n, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    k_scatter_v<R><<<grid_for(n, 256), 256, 0, st>>>(v, gidx, vg, n);
    return cudaGetLastError();
}
template cudaError_t launch_gather_v<float, float>(const float *, const int32_t *, float *, int64_t, cudaStream_t);
template cudaError_t launch_gather_v<float, double>(const float *, const int32_t *, double *, int64_t, cudaStream_t);
template cudaError_t launch_gather_v<double, float>(const double *, const int32_t *, float *, int64_t, cudaStream_t);
template cudaError_t launch_gather_v<double, double>(const double *, const int32_t *, double *, int64_t, cudaStream_t);
template cudaError_t launch_scatter_v<float>(const float *, const int32_t *, float *, int64_t, cudaStream_t);
template cudaError_t launch_scatter_v<double>(const double *, const int32_t *, double *, int64_t, cudaStream_t);

// V on the lattice of every `stride`-th voxel per axis, in the order the
// reference's VTK writer visits it (z outermost, x innermost); -100 where the
// grid voxel is not tissue (GPU3D.cu:145-158, new_11.cu:164-175).
template <typename R>
__global__ void k_sample_v(const R *__restrict__ vg, const uint8_t *__restrict__ tissue, int32_t nx, int32_t ny,
                           int32_t nz, int32_t stride, int64_t sx, int64_t sy, double *__restrict__ out)
{
    const int64_t cx = (nx + stride - 1) / stride, cy = (ny + stride - 1) / stride, cz = (nz + stride - 1) / stride;
    const int64_t n = cx * cy * cz;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t xi = i % cx, r = i / cx, yi = r % cy, zi = r / cy;
        const int64_t g = xi * stride * sx + yi * stride * sy + zi * stride;
        out[i] = tissue[g] ? (double)vg[g] : -100.0;
    }
}
template <typename R>
cudaError_t launch_sample_v(const R *vg, const uint8_t *tissue, int32_t nx, int32_t ny, int32_t nz, int32_t stride,
                            int64_t sx, int64_t sy, double *out, cudaStream_t st)
{
    const int64_t n = ((nx + stride - 1) / stride) * (int64_t)((ny + stride - 1) / stride) * ((nz + stride - 1) / stride);
    if (n <= 0) return cudaSuccess;
    k_sample_v<R><<<grid_for(n, 256), 256, 0, st>>>(vg, tissue, nx, ny, nz, stride, sx, sy, out);
    return cudaGetLastError();
}
// FP16 copies of the FP32 tensor rows (6 per voxel) and divergence rows (3
// per voxel, padded to 4) for the surrogate's substep.
// The substep's FP16 tensor rows.  Every tensor is D = D_t I + dd f f^T
// (xx yy zz xy xz yz in d6), so D - D_t I = sgn g g^T with g = sqrt|dd| f:
// g is read off the largest diagonal entry of sgn (D - D_t I) (at least a
// third of |dd| |f|^2) and the off-diagonal entries of its row.
__global__ void k_tensor_f16(const float *__restrict__ d6, const float *__restrict__ b3, int64_t n, float dtr,
                             float sgn, __half2 *__restrict__ t3h)
{
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        const float *d = d6 + 6 * k, *b = b3 + 3 * k;
        const float a[3] = {sgn * (d[0] - dtr), sgn * (d[1] - dtr), sgn * (d[2] - dtr)};
        const float off[3][3] = {{0.f, d[3], d[4]}, {d[3], 0.f, d[5]}, {d[4], d[5], 0.f}};
        const int i = a[0] >= a[1] ? (a[0] >= a[2] ? 0 : 2) : (a[1] >= a[2] ? 1 : 2);
        float g[3] = {0.f, 0.f, 0.f};
        if (a[i] > 0.f) {
            g[i] = sqrtf(a[i]);
            for (int j = 0; j < 3; ++j)
                if (j != i) g[j] = sgn * off[i][j] / g[i];
        }
        t3h[3 * k + 0] = __floats2half2_rn(g[0], g[1]);
        t3h[3 * k + 1] = __floats2half2_rn(g[2], b[0]);
        t3h[3 * k + 2] = __floats2half2_rn(b[1], b[2]);
    }
}

cudaError_t launch_tensor_f16(const float *d6, const float *b3, int64_t n, float dtr, float sgn, __half2 *t3h,
                              cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    k_tensor_f16<<<grid_for(n, 256), 256, 0, st>>>(d6, b3, n, dtr, sgn, t3h);
    return cudaGetLastError();
}

template cudaError_t launch_sample_v<float>(const float *, const uint8_t *, int32_t, int32_t, int32_t, int32_t, int64_t,
                                            int64_t, double *, cudaStream_t);
template cudaError_t launch_sample_v<double>(const double *, const uint8_t *, int32_t, int32_t, int32_t, int32_t,
                                             int64_t, int64_t, double *, cudaStream_t);

}  // namespace lqt
