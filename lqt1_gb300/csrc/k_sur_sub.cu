// k_sur_sub.cu -- the V-only step of the voxels inside a surrogate macro step
// (k_sur_substep in k_grid.cuh), mixed form, 1D/2D/3D.
#include "k_grid.cuh"

namespace lqt {

cudaError_t launch_sur_substep(const GridDev<float> &gd, double dt, int cur, int dim, cudaStream_t st)
{
    if (gd.ntissue <= 0) return cudaSuccess;
    const unsigned nb = (unsigned)((gd.ntissue + 256 * kSubU - 1) / (256 * kSubU));
    if (dim == 1) k_sur_substep<1><<<nb, 256, 0, st>>>(gd, (float)dt, cur);
    else if (dim == 2) k_sur_substep<2><<<nb, 256, 0, st>>>(gd, (float)dt, cur);
    else k_sur_substep<3><<<nb, 256, 0, st>>>(gd, (float)dt, cur);
    return cudaGetLastError();
}

}  // namespace lqt
