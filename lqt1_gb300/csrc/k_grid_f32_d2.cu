// k_grid_f32_d2.cu -- occupancy variants of the 2D mixed-form step kernel
// (separate translation unit so the variants compile in parallel).
#include "k_grid.cuh"

namespace lqt {

cudaError_t launch_f32_d2(const GridDev<float> &gd, const StepT<float> &kk, int cur, int minb, cudaStream_t st)
{
    if (gd.plist) {
        k_grid_step_list<float, 2><<<grid_list_blocks(gd.ntissue), 256, 0, st>>>(gd, kk, cur);
        return cudaGetLastError();
    }
    const unsigned nb = (unsigned)((gd.ntissue + 255) / 256);
    if (minb >= 4) k_grid_step<float, 2, 4><<<nb, 256, 0, st>>>(gd, kk, cur);
    else if (minb == 3) k_grid_step<float, 2, 3><<<nb, 256, 0, st>>>(gd, kk, cur);
    else k_grid_step<float, 2, 2><<<nb, 256, 0, st>>>(gd, kk, cur);
    return cudaGetLastError();
}

}  // namespace lqt
