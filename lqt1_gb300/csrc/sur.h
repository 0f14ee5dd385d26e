// sur.h -- the learned surrogate's data layout (k_sur.cu, api_mlp.cu).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "grid_dev.h"
#include "mlp.h"
#include "tpord.cuh"

namespace lqt {

constexpr int kSurSteps = 5;     // plain steps per surrogate macro step (0.1 ms at dt = 0.02 ms)
// A macro-step length (plain steps per macro step) must divide the 50-step
// span of a captured step graph, so that every graph starts on a macro-step
// boundary: 1, 2, 5, 10, 25 or 50.  0 in the C ABI selects kSurSteps.
constexpr int kSurSpan = 50;
// Counters of a tissue run with a surrogate: offered, accepted, and the
// offered voxels failing each residual check (network bound, gate range,
// concentration sign, ionic V step).
constexpr int kSurNStats = 6;
inline bool sur_nsub_ok(int n) { return n >= 1 && n <= kSurSpan && kSurSpan % n == 0; }
inline int sur_nsub_or_default(int n) { return n == 0 ? kSurSteps : n; }
constexpr int kSurFeat = 44;     // raw features: 38 states + GKs, PCa, GKs-ISO factors + endo/epi/M one-hot

// One paced cell of the training-data generator.
struct SurCell {
    int64_t nsteps, warm_steps, bcl_steps;
    int64_t stim_on, stim_off;   // step range within each cycle
    int32_t model, ctype;
    float stim;                  // pA/pF
    float gks_scale, pca_scale, iso_scale;
};

// The tissue macro step (k_sur_grid.cu).
struct SurGrid {
    MlpDev w;
    const float *norm;              // in_mean[48], in_scale[48], out_scale[48], out_bound[48]
    float *rate;                    // per tissue voxel: ionic dV/dt of the macro step, NaN = plain step
    uint8_t *dflag;                 // per tissue voxel: 1 = its AP detector runs on the substeps
    int32_t *plist;                 // voxels that run the plain step during the macro step
    unsigned long long *plist_n;    // their count (zero before the launch)
    unsigned long long *stats;      // [0] voxels offered, [1] accepted, [2..5] offered voxels failing a check (kSurNStats)
    int *err;                       // set when an mbarrier wait ran out
    StepT<float> kmac;              // the coarse step (dt = nsub * plain dt)
    float par[3];                   // GKs, PCa and GKs-ISO factors of the model
    float dvdt_max;                 // offer only where |dV/dt| <= dvdt_max (mV/ms)
    float foot_dvdt, foot_v;        // and not where V < foot_v rises faster than foot_dvdt (0 = off)
    float kappa;                    // multiplier of out_bound in the residual check
    float vstep_max;                // bound on the macro step's ionic V change (mV)
    int nsub;                       // plain steps per macro step
    float inv_dt, inv_mac;          // 1 / dt and 1 / (nsub dt), rounded from FP64 on the host
    int use_net;                    // 0: coarse step without the network
};
cudaError_t launch_sur_grid(const GridDev<float> &gd, const SurGrid &sg, int cur, int dim, cudaStream_t st);
uint32_t sur_grid_smem_bytes();

cudaError_t launch_sur_datagen(const SurCell *cells, int64_t ncells, const ModelK *models, const StepK &k,
                               const StepK &kmac, float *X, float *D, int64_t *counts, const int64_t *offsets,
                               int64_t cap, uint64_t seed, float dvdt_max, float prob, float jitter, int nsub,
                               cudaStream_t st);
cudaError_t launch_sur_prepare(const float *X, const float *D, const int64_t *idx, int64_t n, const float *norm,
                               __nv_bfloat16 *xb, float *t, cudaStream_t st);

}  // namespace lqt
