// k_sur.cu -- the learned surrogate around the plain integrator:
//   * training pairs generated by the plain mixed-form TPORd step,
//   * feature normalisation into the network's BF16 inputs.
// A surrogate macro step advances a cell by kSurSteps plain steps (0.1 ms at
// dt = 0.02 ms) with no diffusion and no stimulus: the network predicts the
// change of the 38 evolving states.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"
#include "mlp.h"
#include "sur.h"

namespace lqt {

// The 38 evolving states in network order: V, 8 concentrations, 29 gates.
template <typename R> __device__ __forceinline__ void state38(const CellState<R> &c, float *x)
{
    x[0] = (float)c.v;
    const typename CellState<R>::C *cc[8] = {&c.nai, &c.nass, &c.ki, &c.kss, &c.cai, &c.cass, &c.cansr, &c.cajsr};
#pragma unroll
    for (int j = 0; j < 8; ++j) x[1 + j] = (float)cval(*cc[j]);
    const R g[29] = {c.sm, c.sh, c.sj, c.mL, c.hL, c.hLp, c.a, c.iF, c.iS, c.ap, c.iFp, c.iSp, c.d, c.ff, c.fs,
                     c.fcaf, c.fcas, c.jca, c.nca, c.ffp, c.fcafp, c.xrf, c.xrs, c.xs1, c.xs2, c.xk1, c.Jrelnp,
                     c.Jrelp, c.CaMKt};
#pragma unroll
    for (int j = 0; j < 29; ++j) x[9 + j] = (float)g[j];
}

__device__ __forceinline__ uint32_t hash3(uint64_t s, uint64_t a, uint64_t b)
{
    uint64_t x = s ^ (a * 0x9E3779B97F4A7C15ull) ^ (b * 0xC2B2AE3D27D4EB4Full);
    x ^= x >> 33;
    x *= 0xFF51AFD7ED558CCDull;
    x ^= x >> 33;
    x *= 0xC4CEB9FE1A85EC53ull;
    x ^= x >> 33;
    return (uint32_t)x;
}

// One thread per cell: pace with the plain mixed step, and at macro-step
// boundaries in the surrogate's regime (|dV/dt| <= dvdt_max, no stimulus in
// the coming macro step, past the warm-up) record, with probability `prob`,
// the inputs and the state change over the macro step.
__global__ void __launch_bounds__(128) k_sur_datagen(const SurCell *__restrict__ cells, int64_t ncells,
                                                     const ModelK *__restrict__ models, StepT<float> k,
                                                     float *__restrict__ X, float *__restrict__ D,
                                                     unsigned long long *__restrict__ counter, int64_t cap,
                                                     uint64_t seed, float dvdt_max, float prob)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= ncells) return;
    const SurCell sc = cells[i];
    const ModelT<float> m = model_as<float>(models[sc.model]);
    CellState<float> c;
    c.v = -87.5f;
    const float2 z = make_float2(0.f, 0.f);
    c.nai = make_float2(7.f, 0.f); c.nass = make_float2(7.f, 0.f);
    c.ki = make_float2(145.f, 0.f); c.kss = make_float2(145.f, 0.f);
    c.cai = make_float2(1.0e-4f, 0.f); c.cass = make_float2(1.0e-4f, 0.f);
    c.cansr = make_float2(1.2f, 0.f); c.cajsr = make_float2(1.2f, 0.f);
    (void)z;
    c.sm = 0.f; c.sh = 1.f; c.sj = 1.f; c.mL = 0.f; c.hL = 1.f; c.hLp = 1.f; c.a = 0.f; c.iF = 1.f; c.iS = 1.f;
    c.ap = 0.f; c.iFp = 1.f; c.iSp = 1.f; c.d = 0.f; c.ff = 1.f; c.fs = 1.f; c.fcaf = 1.f; c.fcas = 1.f;
    c.jca = 1.f; c.nca = 0.f; c.ffp = 1.f; c.fcafp = 1.f; c.xrf = 0.f; c.xrs = 0.f; c.xs1 = 0.f; c.xs2 = 0.f;
    c.xk1 = 1.f; c.Jrelnp = 0.f; c.Jrelp = 0.f; c.CaMKt = 0.f;
    const int ct = sc.ctype;
    const int cls = ct == 2 ? 1 : (ct == 4 ? 2 : 0);
    StepOut<float> o{};
    int64_t slot = -1;
    float x0[kMlpNState];
    float lo0[8];
    for (int64_t st = 0; st < sc.nsteps; ++st) {
        const int64_t ph = st % sc.bcl_steps;
        if (st % kSurSteps == 0) {
            if (slot >= 0) {
                // finish the pending sample: change over the macro step
                float x1[kMlpNState];
                state38(c, x1);
                float *d = D + slot * kMlpNState;
                const float2 *cc[8] = {&c.nai, &c.nass, &c.ki, &c.kss, &c.cai, &c.cass, &c.cansr, &c.cajsr};
                d[0] = x1[0] - x0[0];
#pragma unroll
                for (int j = 0; j < 8; ++j) d[1 + j] = (cc[j]->x - x0[1 + j]) + (cc[j]->y - lo0[j]);
#pragma unroll
                for (int j = 9; j < kMlpNState; ++j) d[j] = x1[j] - x0[j];
                slot = -1;
            }
            const bool stim_ahead = ph + kSurSteps > sc.stim_on && ph < sc.stim_off;
            if (st >= sc.warm_steps && !stim_ahead && fabsf(o.dvdt) <= dvdt_max && st + kSurSteps <= sc.nsteps &&
                (hash3(seed, (uint64_t)i, (uint64_t)st) & 0xFFFFFF) < (uint32_t)(prob * 16777216.f)) {
                const unsigned long long s = atomicAdd(counter, 1ull);
                if (s < (unsigned long long)cap) {
                    slot = (int64_t)s;
                    state38(c, x0);
                    const float2 *cc[8] = {&c.nai, &c.nass, &c.ki, &c.kss, &c.cai, &c.cass, &c.cansr, &c.cajsr};
#pragma unroll
                    for (int j = 0; j < 8; ++j) lo0[j] = cc[j]->y;
                    float *xr = X + slot * kSurFeat;
#pragma unroll
                    for (int j = 0; j < kMlpNState; ++j) xr[j] = x0[j];
                    xr[38] = sc.gks_scale;
                    xr[39] = sc.pca_scale;
                    xr[40] = sc.iso_scale;
                    xr[41] = cls == 0;
                    xr[42] = cls == 1;
                    xr[43] = cls == 2;
                }
            }
        }
        const float ist = (ph >= sc.stim_on && ph < sc.stim_off) ? sc.stim : 0.f;
        tpord_step<float>(c, ct, m, k, ist, 0.f, &o);
    }
}

// Raw features (kSurFeat floats per row) -> normalised BF16 network inputs
// (48 per row, zero padded); optional raw changes -> normalised FP32 targets.
__global__ void k_sur_prepare(const float *__restrict__ X, const float *__restrict__ D, const int64_t *__restrict__ idx,
                              int64_t n, const float *__restrict__ norm, __nv_bfloat16 *__restrict__ xb,
                              float *__restrict__ t)
{
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        const int64_t s = idx ? idx[r] : r;
        const float *xr = X + s * kSurFeat;
        for (int j = 0; j < kMlpIn; ++j) {
            const float v = j < kSurFeat ? (xr[j] - norm[j]) * norm[kMlpIn + j] : 0.f;
            xb[r * kMlpIn + j] = __float2bfloat16(v);
        }
        if (t) {
            const float *dr = D + s * kMlpNState;
            for (int j = 0; j < kMlpOut; ++j) t[r * kMlpOut + j] = j < kMlpNState ? dr[j] / norm[2 * kMlpIn + j] : 0.f;
        }
    }
}

cudaError_t launch_sur_datagen(const SurCell *cells, int64_t ncells, const ModelK *models, const StepK &k, float *X,
                               float *D, unsigned long long *counter, int64_t cap, uint64_t seed, float dvdt_max,
                               float prob, cudaStream_t st)
{
    if (ncells <= 0) return cudaSuccess;
    k_sur_datagen<<<(unsigned)((ncells + 127) / 128), 128, 0, st>>>(cells, ncells, models, step_as<float>(k), X, D,
                                                                    counter, cap, seed, dvdt_max, prob);
    return cudaGetLastError();
}

cudaError_t launch_sur_prepare(const float *X, const float *D, const int64_t *idx, int64_t n, const float *norm,
                               __nv_bfloat16 *xb, float *t, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    int64_t nb = (n + 255) / 256;
    if (nb > 4096) nb = 4096;
    k_sur_prepare<<<(unsigned)nb, 256, 0, st>>>(X, D, idx, n, norm, xb, t);
    return cudaGetLastError();
}

}  // namespace lqt
