// ecg_noalloc.cu -- pseudo-ECG of a caller-owned V grid without any device
// allocation.
//
// Who needs it: callers that own every byte of device memory themselves, such
// as a host framework that hands plugins fixed buffers from its own pool or a
// fixed memory budget, or a time-critical stepping loop that must not hit the
// implicit device synchronisation of cudaMalloc/cudaFree.  They pass the V
// grid, the tissue index, the electrodes and the output; the only scratch this
// path needs (one FP64 partial per block and electrode) lives in a fixed
// file-scope device array instead of a cudaMalloc'd buffer.
//
// The array is kNoAllocBlocks x kMaxEl doubles = 2048 x 8 x 8 B = 128 KiB of
// partials plus a 256-byte tail that holds the call's status word.  It is part
// of the library image, so every GPU that loads the library holds it until the
// process exits.  All calls share it and it keeps the last call's contents:
// each call clears the status word, overwrites exactly the partials it reads
// back, and calls whose kernels overlap on the GPU (different streams, other
// threads) race on it, so callers must serialise them.
//
// The caller's tissue index is checked on the device before any V access: a
// voxel outside the grid or on a grid face (whose stencil would leave the grid
// or wrap into the next row) is skipped and sets the status word, and the call
// then writes NaN to every electrode.  The call stays asynchronous, so this is
// how a bad index shows up: NaN in phi, never a read outside the V grid.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <mutex>
#include <string>

#include "../../include/lqt.h"
#include "api_common.h"

namespace {

constexpr int kNoAllocBlocks = 2048;   // grid-stride blocks, also the scratch rows
constexpr int kNoAllocThreads = 256;
constexpr int kMaxEl = 8;              // electrodes per call
constexpr int kMaxDevices = 64;

constexpr int kStatusSlot = kNoAllocBlocks * kMaxEl;   // first double of the 256-byte tail
static __device__ __align__(256) double g_ecg_scratch[kNoAllocBlocks * kMaxEl + 32];

struct Electrodes {
    float x[kMaxEl], y[kMaxEl], z[kMaxEl];
};

// Same sum as k_ecg_partial (3D form of PlotScript/plot1DECG_compare.py:89-105),
// over a grid-stride loop so the number of partials is bounded.  Grid index
// g = (x*ny + y)*nz + z; a 2D/3D tissue voxel must have 1 <= x <= nx-2,
// 1 <= y <= ny-2 and, in 3D, 1 <= z <= nz-2 (its stencil stays inside the
// grid); any other index is skipped and flagged in *status.
__global__ void __launch_bounds__(kNoAllocThreads)
    k_ecg_noalloc_partial(const float *__restrict__ V, const int32_t *__restrict__ gidx, int64_t n, int64_t nx,
                          int64_t ny, int64_t nz, int dim, double dx, Electrodes el, int nel,
                          double *__restrict__ partial, unsigned int *__restrict__ status)
{
    __shared__ double red[kNoAllocThreads / 32][kMaxEl];
    double acc[kMaxEl];
#pragma unroll
    for (int e = 0; e < kMaxEl; ++e) acc[e] = 0.0;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        float p[3] = {0.f, 0.f, 0.f}, h[3] = {0.f, 0.f, 0.f};
        if (dim == 1) {
            p[0] = (float)(k * dx);
            if (n > 1) h[0] = k == 0 ? V[1] - V[0] : (k == n - 1 ? V[k] - V[k - 1] : 0.5f * (V[k + 1] - V[k - 1]));
        } else {
            const int64_t g = gidx[k];
            const int64_t sx = ny * nz, sy = dim == 2 ? 1 : nz;
            const int64_t x = g / sx, rem = g - x * sx;
            const int64_t y = rem / sy, z = rem - y * sy;
            const bool inside = g >= 0 && x >= 1 && x <= nx - 2 && y >= 1 && y <= ny - 2 &&
                                (dim == 2 || (z >= 1 && z <= nz - 2));
            if (!inside) {
                atomicOr(status, 1u);
                continue;
            }
            p[0] = (float)(x * dx);
            p[1] = (float)(y * dx);
            p[2] = (float)((dim == 3 ? z : 0) * dx);
            h[0] = 0.5f * (V[g + sx] - V[g - sx]);
            h[1] = 0.5f * (V[g + sy] - V[g - sy]);
            if (dim == 3) h[2] = 0.5f * (V[g + 1] - V[g - 1]);
        }
#pragma unroll
        for (int e = 0; e < kMaxEl; ++e) {
            if (e < nel) {
                const float rx = p[0] - el.x[e], ry = p[1] - el.y[e], rz = p[2] - el.z[e];
                const float inv = rsqrtf(rx * rx + ry * ry + rz * rz);
                acc[e] += (double)((h[0] * rx + h[1] * ry + h[2] * rz) * (inv * inv * inv));
            }
        }
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int e = 0; e < kMaxEl; ++e) {
        double v = acc[e];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) red[wid][e] = v;
    }
    __syncthreads();
    if (threadIdx.x < nel) {
        double s = 0.0;
        for (int w = 0; w < kNoAllocThreads / 32; ++w) s += red[w][threadIdx.x];
        partial[blockIdx.x * kMaxEl + threadIdx.x] = s;    // every used row is rewritten by its block
    }
}

// Sum the partials of the blocks that ran, in block order (deterministic);
// NaN for every electrode when the partial kernel flagged a bad voxel.
__global__ void __launch_bounds__(kNoAllocThreads)
    k_ecg_noalloc_final(const double *__restrict__ partial, int nblocks, int nel, const unsigned int *status,
                        double *__restrict__ out)
{
    __shared__ double red[kNoAllocThreads];
    if (*status != 0u) {
        if ((int)threadIdx.x < nel) out[threadIdx.x] = __longlong_as_double(0x7ff8000000000000LL);
        return;
    }
    for (int e = 0; e < nel; ++e) {
        double s = 0.0;
        for (int b = threadIdx.x; b < nblocks; b += blockDim.x) s += partial[b * kMaxEl + e];
        red[threadIdx.x] = s;
        __syncthreads();
        for (int w = blockDim.x / 2; w > 0; w >>= 1) {
            if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
            __syncthreads();
        }
        if (threadIdx.x == 0) out[e] = red[0];
        __syncthreads();
    }
}

std::mutex g_setup_mu;
double *g_scratch_addr[kMaxDevices] = {nullptr};

// Device address of the scratch array for the current device (set up once per
// device; host code cannot use the symbol's host-side name as an address).
int scratch_for_current_device(double **out)
{
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return lqt::fail(LQT_ERR_CUDA, std::string("lqt_ecg_grid_noalloc: cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return lqt::fail(LQT_ERR_INVALID, "lqt_ecg_grid_noalloc: device index above 63");
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_ecg_scratch);
        if (e != cudaSuccess || !p)
            return lqt::fail(LQT_ERR_CUDA, std::string("lqt_ecg_grid_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        g_scratch_addr[dev] = static_cast<double *>(p);
    }
    *out = g_scratch_addr[dev];
    return LQT_OK;
}

// The cached address belongs to the device's context: drop it when a launch
// fails, so a context torn down and re-created (cudaDeviceReset) gets a fresh
// lookup on the next call.
void forget_scratch_for_current_device()
{
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return;
    std::lock_guard<std::mutex> lock(g_setup_mu);
    g_scratch_addr[dev] = nullptr;
}

}  // namespace

extern "C" int lqt_ecg_grid_noalloc(const float *v_grid_dev, int32_t nx, int32_t ny, int32_t nz, double dx,
                                    const int32_t *tissue_index_dev, int64_t ntissue, const double *electrodes_host,
                                    int32_t nel, double *phi_dev, void *stream)
{
    if (!v_grid_dev || !phi_dev || !electrodes_host)
        return lqt::fail(LQT_ERR_INVALID, "lqt_ecg_grid_noalloc: NULL V grid, output or electrodes");
    if (nel < 1 || nel > kMaxEl)
        return lqt::fail(LQT_ERR_INVALID, "lqt_ecg_grid_noalloc: nel must be 1..8 (the scratch holds 8 electrodes)");
    if (nx < 1 || ny < 1 || nz < 1 || ntissue < 1 || ntissue > (int64_t)INT32_MAX ||
        (int64_t)nx * ny * nz > (int64_t)INT32_MAX || !(dx > 0))
        return lqt::fail(LQT_ERR_INVALID, "lqt_ecg_grid_noalloc: grid and tissue sizes must be 1..2^31-1, dx > 0");
    const int dim = (ny == 1 && nz == 1) ? 1 : (nz == 1 ? 2 : 3);
    if (dim > 1 && !tissue_index_dev)
        return lqt::fail(LQT_ERR_INVALID, "lqt_ecg_grid_noalloc: 2D/3D grids need the tissue index");
    if (dim == 1 && ntissue != nx) return lqt::fail(LQT_ERR_INVALID, "lqt_ecg_grid_noalloc: 1D needs ntissue == nx");
    double *scratch = nullptr;
    int rc = scratch_for_current_device(&scratch);
    if (rc) return rc;
    Electrodes el{};
    for (int e = 0; e < nel; ++e) {
        el.x[e] = (float)electrodes_host[3 * e];
        el.y[e] = (float)electrodes_host[3 * e + 1];
        el.z[e] = (float)electrodes_host[3 * e + 2];
    }
    int64_t nb = (ntissue + kNoAllocThreads - 1) / kNoAllocThreads;
    if (nb > kNoAllocBlocks) nb = kNoAllocBlocks;
    cudaStream_t st = (cudaStream_t)stream;
    unsigned int *status = reinterpret_cast<unsigned int *>(scratch + kStatusSlot);
    // the status word keeps the last call's value: clear it first
    cudaError_t e = cudaMemsetAsync(status, 0, sizeof(unsigned int), st);
    if (e == cudaSuccess) {
        k_ecg_noalloc_partial<<<(unsigned)nb, kNoAllocThreads, 0, st>>>(v_grid_dev, tissue_index_dev, ntissue, nx,
                                                                         ny, nz, dim, dx, el, nel, scratch, status);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        k_ecg_noalloc_final<<<1, kNoAllocThreads, 0, st>>>(scratch, (int)nb, nel, status, phi_dev);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) {
        forget_scratch_for_current_device();   // looked up again on the next call (e.g. after a device reset)
        return lqt::fail(LQT_ERR_CUDA, std::string("lqt_ecg_grid_noalloc: ") + cudaGetErrorString(e));
    }
    return LQT_OK;
}
