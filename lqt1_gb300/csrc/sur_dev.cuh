// sur_dev.cuh -- device helpers of the learned surrogate shared by the
// training-data generator (k_sur.cu) and the tissue macro step (k_sur_grid.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "mlp.h"
#include "sur.h"
#include "tpord.cuh"

namespace lqt {

// Pointers to the 8 concentrations / 29 evolving gates in network order.
template <typename R> __device__ __forceinline__ void conc_ptrs(CellState<R> &c, typename CellState<R>::C *p[8])
{
    p[0] = &c.nai; p[1] = &c.nass; p[2] = &c.ki; p[3] = &c.kss;
    p[4] = &c.cai; p[5] = &c.cass; p[6] = &c.cansr; p[7] = &c.cajsr;
}
template <typename R> __device__ __forceinline__ void gate_ptrs(CellState<R> &c, R *g[29])
{
    g[0] = &c.sm; g[1] = &c.sh; g[2] = &c.sj; g[3] = &c.mL; g[4] = &c.hL; g[5] = &c.hLp; g[6] = &c.a;
    g[7] = &c.iF; g[8] = &c.iS; g[9] = &c.ap; g[10] = &c.iFp; g[11] = &c.iSp; g[12] = &c.d; g[13] = &c.ff;
    g[14] = &c.fs; g[15] = &c.fcaf; g[16] = &c.fcas; g[17] = &c.jca; g[18] = &c.nca; g[19] = &c.ffp;
    g[20] = &c.fcafp; g[21] = &c.xrf; g[22] = &c.xrs; g[23] = &c.xs1; g[24] = &c.xs2; g[25] = &c.xk1;
    g[26] = &c.Jrelnp; g[27] = &c.Jrelp; g[28] = &c.CaMKt;
}
// Gates 26..28 (Jrelnp, Jrelp, CaMKt) are not probabilities.
constexpr int kSurNProb = 26;

// The 38 evolving states in network order: V, 8 concentrations (hi part), 29 gates.
__device__ __forceinline__ void state38(CellState<float> &c, float *x)
{
    float2 *cp[8];
    float *gp[29];
    conc_ptrs(c, cp);
    gate_ptrs(c, gp);
    x[0] = c.v;
#pragma unroll
    for (int j = 0; j < 8; ++j) x[1 + j] = cp[j]->x;
#pragma unroll
    for (int j = 0; j < 29; ++j) x[9 + j] = *gp[j];
}

// One-hot class of a cell type: 0 endo (and other), 1 epi, 2 M.
__device__ __forceinline__ int sur_class(int ctype) { return ctype == 2 ? 1 : (ctype == 4 ? 2 : 0); }

__device__ __forceinline__ uint32_t sur_hash(uint64_t s, uint64_t a, uint64_t b)
{
    uint64_t x = s ^ (a * 0x9E3779B97F4A7C15ull) ^ (b * 0xC2B2AE3D27D4EB4Full);
    x ^= x >> 33;
    x *= 0xFF51AFD7ED558CCDull;
    x ^= x >> 33;
    x *= 0xC4CEB9FE1A85EC53ull;
    x ^= x >> 33;
    return (uint32_t)x;
}

}  // namespace lqt
