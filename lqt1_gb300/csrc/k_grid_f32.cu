// k_grid_f32.cu -- grid kernels for the mixed form (R = float): launchers, the
// default occupancy variant and the pseudo-ECG.
#include "k_grid.cuh"

namespace lqt {

template <> cudaError_t launch_grid_step_minb<float>(const GridDev<float> &gd, const StepT<float> &kk, int cur,
                                                     int dim, int minb, cudaStream_t st);

template <> cudaError_t launch_grid_step<float>(const GridDev<float> &gd, const StepK &k, int cur, int dim, int minb,
                                                cudaStream_t st)
{
    if (gd.ntissue <= 0) return cudaSuccess;
    return launch_grid_step_minb<float>(gd, step_as<float>(k), cur, dim, minb, st);
}

template <> cudaError_t launch_ghost<float>(const GridDev<float> &gd, int nxt, cudaStream_t st)
{
    int64_t nb = (gd.nbnd + 255) / 256;
    if (nb < 1) nb = 1;
    if (nb > 152 * 16) nb = 152 * 16;
    k_ghost<float><<<(unsigned)nb, 256, 0, st>>>(gd, nxt);
    return cudaGetLastError();
}

template <>
cudaError_t launch_ecg<float>(const GridDev<float> &gd, int cur, const float4 *el, int nel, double *partial, double *out,
                              double *t_out, int64_t *counter, int64_t cap, int dim, cudaStream_t st)
{
    const int64_t nb = ecg_blocks(gd.ntissue);
    if (dim == 1) k_ecg_partial<float, 1><<<(unsigned)nb, 256, 0, st>>>(gd, gd.vg[cur], el, nel, partial);
    else if (dim == 2) k_ecg_partial<float, 2><<<(unsigned)nb, 256, 0, st>>>(gd, gd.vg[cur], el, nel, partial);
    else k_ecg_partial<float, 3><<<(unsigned)nb, 256, 0, st>>>(gd, gd.vg[cur], el, nel, partial);
    k_ecg_final<<<nel, 256, 0, st>>>(partial, nb, nel, out, t_out, counter, cap, gd.clk);
    return cudaGetLastError();
}

int64_t ecg_blocks(int64_t ntissue) { return ntissue <= 0 ? 1 : (ntissue + 255) / 256; }

// Sum the per-block partials of each electrode in block order (deterministic):
// one block per electrode; the last block to finish (a counter in the same
// launch) records the time and advances the sample counter.
__global__ void k_ecg_final(const double *__restrict__ partial, int64_t nblocks, int nel, double *__restrict__ out,
                            double *__restrict__ t_out, int64_t *__restrict__ counter, int64_t cap,
                            const Clock *__restrict__ clk)
{
    __shared__ double red[256];
    const int64_t slot = counter[0];
    if (slot >= cap) return;
    const int e = blockIdx.x;
    double s = 0.0;
    for (int64_t b = threadIdx.x; b < nblocks; b += blockDim.x) s += partial[b * nel + e];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[slot * nel + e] = red[0];
        __threadfence();
        // counter[1]: blocks of this sample done
        const unsigned long long done = atomicAdd(reinterpret_cast<unsigned long long *>(counter + 1), 1ull) + 1;
        if (done == (unsigned long long)nel) {
            t_out[slot] = clk->time;
            counter[1] = 0;
            __threadfence();
            counter[0] = slot + 1;
        }
    }
}

}  // namespace lqt
