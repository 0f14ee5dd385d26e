// k_sur.cu -- the learned surrogate around the plain integrator:
//   * training pairs generated by the plain mixed-form TPORd step,
//   * feature normalisation into the network's BF16 inputs.
// A surrogate macro step advances a cell by nsub plain steps (nsub = 5: 0.1 ms
// at dt = 0.02 ms) with no diffusion and no stimulus: one coarse TPORd step of
// the macro length plus the network's correction of the 38 evolving states.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"
#include "mlp.h"
#include "sur.h"
#include "sur_dev.cuh"

namespace lqt {

__device__ __forceinline__ void sur_init_cell(CellState<float> &c)
{
    c.v = -87.5f;
    c.nai = make_float2(7.f, 0.f); c.nass = make_float2(7.f, 0.f);
    c.ki = make_float2(145.f, 0.f); c.kss = make_float2(145.f, 0.f);
    c.cai = make_float2(1.0e-4f, 0.f); c.cass = make_float2(1.0e-4f, 0.f);
    c.cansr = make_float2(1.2f, 0.f); c.cajsr = make_float2(1.2f, 0.f);
    c.sm = 0.f; c.sh = 1.f; c.sj = 1.f; c.mL = 0.f; c.hL = 1.f; c.hLp = 1.f; c.a = 0.f; c.iF = 1.f; c.iS = 1.f;
    c.ap = 0.f; c.iFp = 1.f; c.iSp = 1.f; c.d = 0.f; c.ff = 1.f; c.fs = 1.f; c.fcaf = 1.f; c.fcas = 1.f;
    c.jca = 1.f; c.nca = 0.f; c.ffp = 1.f; c.fcafp = 1.f; c.xrf = 0.f; c.xrs = 0.f; c.xs1 = 0.f; c.xs2 = 0.f;
    c.xk1 = 1.f; c.Jrelnp = 0.f; c.Jrelp = 0.f; c.CaMKt = 0.f;
}

// One thread per cell: pace with the plain mixed step, and at macro-step
// boundaries in the surrogate's regime (|dV/dt| <= dvdt_max, no stimulus in
// the coming macro step, past the warm-up) record, with probability `prob`,
// the inputs and the correction: state after nsub plain steps minus the
// state after one coarse step of the macro length from the same start.
// Macro steps that are not recorded carry a constant current uniform in
// +-jitter (a stand-in for the electrotonic load of tissue).
// Two passes make the pair set and its order independent of thread timing:
// with counts != NULL the kernel only counts each cell's recorded macro steps;
// with offsets != NULL the j-th pair of cell i goes to row offsets[i] + j
// (rows at or past cap are dropped, so a truncated set keeps the first cells
// in cell order).  A cell's trajectory is the same in both passes: a macro
// step chosen for recording carries no jitter current whether or not its row
// is kept.
__global__ void __launch_bounds__(128) k_sur_datagen(const SurCell *__restrict__ cells, int64_t ncells,
                                                     const ModelK *__restrict__ models, StepT<float> k,
                                                     StepT<float> kmac, float *__restrict__ X,
                                                     float *__restrict__ D, int64_t *__restrict__ counts,
                                                     const int64_t *__restrict__ offsets, int64_t cap, uint64_t seed,
                                                     float dvdt_max, float prob, float jitter, int nsub)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= ncells) return;
    const SurCell sc = cells[i];
    const ModelT<float> m = model_as<float>(models[sc.model]);
    CellState<float> c;
    sur_init_cell(c);
    const int ct = sc.ctype;
    const int cls = sur_class(ct);
    StepOut<float> o{};
    int64_t slot = -1, nrec = 0;
    float xc[kMlpNState];   // coarse end state (hi parts) of the pending sample
    float loc[8];           // and its concentration lo parts
    float ipert = 0.f;
    for (int64_t st = 0; st < sc.nsteps; ++st) {
        const int64_t ph = st % sc.bcl_steps;
        if (st % nsub == 0) {
            if (slot >= 0) {
                // finish the pending sample: fine minus coarse
                float x1[kMlpNState];
                state38(c, x1);
                float2 *cp[8];
                conc_ptrs(c, cp);
                float *d = D + slot * kMlpNState;
                d[0] = x1[0] - xc[0];
#pragma unroll
                for (int j = 0; j < 8; ++j) d[1 + j] = (cp[j]->x - xc[1 + j]) + (cp[j]->y - loc[j]);
#pragma unroll
                for (int j = 9; j < kMlpNState; ++j) d[j] = x1[j] - xc[j];
                slot = -1;
            }
            const bool stim_ahead = ph + nsub > sc.stim_on && ph < sc.stim_off;
            ipert = 0.f;
            if (st >= sc.warm_steps && !stim_ahead && fabsf(o.dvdt) <= dvdt_max && st + nsub <= sc.nsteps &&
                (sur_hash(seed, (uint64_t)i, (uint64_t)st) & 0xFFFFFF) < (uint32_t)(prob * 16777216.f)) {
                const int64_t s = counts ? -1 : offsets[i] + nrec;
                ++nrec;
                if (s >= 0 && s < cap) {
                    slot = s;
                    float x0[kMlpNState];
                    state38(c, x0);
                    float *xr = X + slot * kSurFeat;
#pragma unroll
                    for (int j = 0; j < kMlpNState; ++j) xr[j] = x0[j];
                    xr[38] = sc.gks_scale;
                    xr[39] = sc.pca_scale;
                    xr[40] = sc.iso_scale;
                    xr[41] = cls == 0;
                    xr[42] = cls == 1;
                    xr[43] = cls == 2;
                    CellState<float> cc = c;
                    StepOut<float> oc;
                    tpord_step<float>(cc, ct, m, kmac, 0.f, 0.f, &oc);
                    state38(cc, xc);
                    float2 *cp[8];
                    conc_ptrs(cc, cp);
#pragma unroll
                    for (int j = 0; j < 8; ++j) loc[j] = cp[j]->y;
                }
            } else if (jitter > 0.f && !stim_ahead) {
                const uint32_t h = sur_hash(seed ^ 0x5bd1e995ull, (uint64_t)i, (uint64_t)st);
                ipert = jitter * ((float)(h >> 8) * (2.0f / 16777216.0f) - 1.0f);
            }
        }
        const float ist = (ph >= sc.stim_on && ph < sc.stim_off) ? sc.stim : (slot >= 0 ? 0.f : ipert);
        tpord_step<float>(c, ct, m, k, ist, 0.f, &o);
    }
    if (counts) counts[i] = nrec;
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

cudaError_t launch_sur_datagen(const SurCell *cells, int64_t ncells, const ModelK *models, const StepK &k,
                               const StepK &kmac, float *X, float *D, int64_t *counts, const int64_t *offsets,
                               int64_t cap, uint64_t seed, float dvdt_max, float prob, float jitter, int nsub,
                               cudaStream_t st)
{
    if (ncells <= 0) return cudaSuccess;
    k_sur_datagen<<<(unsigned)((ncells + 127) / 128), 128, 0, st>>>(cells, ncells, models, step_as<float>(k),
                                                                    step_as<float>(kmac), X, D, counts, offsets, cap,
                                                                    seed, dvdt_max, prob, jitter, nsub);
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
