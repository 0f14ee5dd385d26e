// k_grid_f64.cu -- grid kernels for the FP64 form: launchers, occupancy
// variants and the pseudo-ECG.
#include "k_grid.cuh"

namespace lqt {

template <> cudaError_t launch_grid_step_minb<double>(const GridDev<double> &gd, const StepT<double> &kk, int cur,
                                                      int dim, int minb, cudaStream_t st)
{
    if (gd.plist) return cudaErrorInvalidValue;   // the surrogate's voxel list exists in the mixed form only
    const unsigned nb = (unsigned)((gd.ntissue + 255) / 256);
    if (dim == 1) k_grid_step<double, 1, 1><<<nb, 256, 0, st>>>(gd, kk, cur);
    else if (dim == 2) {
        if (minb >= 2) k_grid_step<double, 2, 2><<<nb, 256, 0, st>>>(gd, kk, cur);
        else k_grid_step<double, 2, 1><<<nb, 256, 0, st>>>(gd, kk, cur);
    } else {
        if (minb >= 2) k_grid_step<double, 3, 2><<<nb, 256, 0, st>>>(gd, kk, cur);
        else k_grid_step<double, 3, 1><<<nb, 256, 0, st>>>(gd, kk, cur);
    }
    return cudaGetLastError();
}

template <> cudaError_t launch_grid_step<double>(const GridDev<double> &gd, const StepK &k, int cur, int dim, int minb,
                                                 cudaStream_t st)
{
    if (gd.ntissue <= 0) return cudaSuccess;
    return launch_grid_step_minb<double>(gd, step_as<double>(k), cur, dim, minb, st);
}

template <> cudaError_t launch_ghost<double>(const GridDev<double> &gd, int nxt, cudaStream_t st)
{
    int64_t nb = (gd.nbnd + 255) / 256;
    if (nb < 1) nb = 1;
    if (nb > 152 * 16) nb = 152 * 16;
    k_ghost<double><<<(unsigned)nb, 256, 0, st>>>(gd, nxt);
    return cudaGetLastError();
}

template <>
cudaError_t launch_ecg<double>(const GridDev<double> &gd, int cur, const float4 *el, int nel, double *partial,
                               double *out, double *t_out, int64_t *counter, int64_t cap, int dim, cudaStream_t st)
{
    const int64_t nb = ecg_blocks(gd.ntissue);
    if (dim == 1) k_ecg_partial<double, 1><<<(unsigned)nb, 256, 0, st>>>(gd, gd.vg[cur], el, nel, partial);
    else if (dim == 2) k_ecg_partial<double, 2><<<(unsigned)nb, 256, 0, st>>>(gd, gd.vg[cur], el, nel, partial);
    else k_ecg_partial<double, 3><<<(unsigned)nb, 256, 0, st>>>(gd, gd.vg[cur], el, nel, partial);
    k_ecg_final<<<nel, 256, 0, st>>>(partial, nb, nel, out, t_out, counter, cap, gd.clk);
    return cudaGetLastError();
}

}  // namespace lqt
