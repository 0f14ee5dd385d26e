// k_sur_sub.cu -- the V-only step of the voxels inside a surrogate macro step
// (k_sur_substep in k_grid.cuh), mixed form, 1D/2D/3D.
#include "k_grid.cuh"

namespace lqt {

template <int MINB> static void launch_minb(const GridDev<float> &gd, double dt, int cur, int dim, unsigned nb,
                                            cudaStream_t st)
{
    if (dim == 1) k_sur_substep<1, MINB><<<nb, 256, 0, st>>>(gd, (float)dt, cur);
    else if (dim == 2) k_sur_substep<2, MINB><<<nb, 256, 0, st>>>(gd, (float)dt, cur);
    else k_sur_substep<3, MINB><<<nb, 256, 0, st>>>(gd, (float)dt, cur);
}

cudaError_t launch_sur_substep(const GridDev<float> &gd, double dt, int cur, int dim, int minb, cudaStream_t st)
{
    if (gd.ntissue <= 0) return cudaSuccess;
    const unsigned nb = (unsigned)((gd.ntissue + 256 * kSubU - 1) / (256 * kSubU));
    if (minb == 8) launch_minb<8>(gd, dt, cur, dim, nb, st);
    else if (minb == 6) launch_minb<6>(gd, dt, cur, dim, nb, st);
    else launch_minb<5>(gd, dt, cur, dim, nb, st);
    return cudaGetLastError();
}

}  // namespace lqt
