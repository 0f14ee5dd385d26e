// k_grid_f32_d1.cu -- 1D mixed-form step kernel and the variant dispatch.
#include "k_grid.cuh"

namespace lqt {

cudaError_t launch_f32_d2(const GridDev<float> &gd, const StepT<float> &kk, int cur, int minb, cudaStream_t st);
cudaError_t launch_f32_d3(const GridDev<float> &gd, const StepT<float> &kk, int cur, int minb, cudaStream_t st);

template <> cudaError_t launch_grid_step_minb<float>(const GridDev<float> &gd, const StepT<float> &kk, int cur,
                                                     int dim, int minb, cudaStream_t st)
{
    if (dim == 2) return launch_f32_d2(gd, kk, cur, minb, st);
    if (dim == 3) return launch_f32_d3(gd, kk, cur, minb, st);
    if (gd.plist) {
        k_grid_step_list<float, 1><<<grid_list_blocks(gd.ntissue), 256, 0, st>>>(gd, kk, cur);
        return cudaGetLastError();
    }
    const unsigned nb = (unsigned)((gd.ntissue + 255) / 256);
    k_grid_step<float, 1, 2><<<nb, 256, 0, st>>>(gd, kk, cur);
    return cudaGetLastError();
}

}  // namespace lqt
