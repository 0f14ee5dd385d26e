// sur.h -- the learned surrogate's data layout (k_sur.cu, api_mlp.cu).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "tpord.cuh"

namespace lqt {

constexpr int kSurSteps = 5;     // plain steps per surrogate macro step (0.1 ms at dt = 0.02 ms)
constexpr int kSurFeat = 44;     // raw features: 38 states + GKs, PCa, GKs-ISO factors + endo/epi/M one-hot

// One paced cell of the training-data generator.
struct SurCell {
    int64_t nsteps, warm_steps, bcl_steps;
    int64_t stim_on, stim_off;   // step range within each cycle
    int32_t model, ctype;
    float stim;                  // pA/pF
    float gks_scale, pca_scale, iso_scale;
};

cudaError_t launch_sur_datagen(const SurCell *cells, int64_t ncells, const ModelK *models, const StepK &k, float *X,
                               float *D, unsigned long long *counter, int64_t cap, uint64_t seed, float dvdt_max,
                               float prob, cudaStream_t st);
cudaError_t launch_sur_prepare(const float *X, const float *D, const int64_t *idx, int64_t n, const float *norm,
                               __nv_bfloat16 *xb, float *t, cudaStream_t st);

}  // namespace lqt
