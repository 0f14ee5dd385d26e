// geometry.h -- host preprocessing of tissue grids (geometry.cc).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/lqt.h"

namespace lqt {

extern thread_local std::string g_err;

struct TissueMap {
    std::vector<int32_t> tissue_of;   // grid -> tissue index or -1
    std::vector<int64_t> cells;       // tissue -> grid index (x-major)
    std::vector<int64_t> bnd_dst;     // boundary voxels (grid index)
    std::vector<int64_t> bnd_src;     // their mirror source (grid index of a tissue voxel)
};

int64_t build_tissue_map(int32_t nx, int32_t ny, int32_t nz, const uint8_t *types, TissueMap &out);
// The same map built on the current device (k_geom.cu); returns an lqt status.
int build_tissue_map_gpu(int32_t nx, int32_t ny, int32_t nz, const uint8_t *types_host, cudaStream_t st,
                         TissueMap &out);
void build_tensor(int32_t nx, int32_t ny, int32_t nz, double dx, const TissueMap &tm, const float *fibre,
                  double d_f, double d_t, std::vector<float> &d6, std::vector<float> &b3);

}  // namespace lqt
