// mlp.h -- the learned surrogate's network (48 -> 128 -> 128 -> 48, SiLU).
//
// Inputs (48): the 38 evolving states of a cell (V, 8 concentrations, the 29
// gates/fluxes that change) and 6 parameters (GKs, PCa and GKs-ISO factors of
// the cell's model, endo/epi/M one-hot), normalised per feature, zero padded.
// Outputs (48): the normalised correction of the 38 states over one macro step
// (nsub plain steps minus one coarse step) without diffusion or stimulus, zero
// padded.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace lqt {

constexpr int kMlpIn = 48, kMlpHid = 128, kMlpOut = 48;
constexpr int kMlpNState = 38, kMlpNParam = 6;

// Device view of the network: weights stored [out][in] row-major (BF16), biases FP32.
struct MlpDev {
    const __nv_bfloat16 *w1t, *w2t, *w3t;   // [128][48], [128][128], [48][128]
    const float *b1, *b2, *b3;              // [128], [128], [48]
    const float *w2f, *w3f;                 // FP32 master copies of W2, W3
};

}  // namespace lqt
struct lqt_mlp;
namespace lqt {
// Device weights and normalisation (in_mean, in_scale, out_scale) of a network.
bool mlp_device_view(const lqt_mlp *m, MlpDev *w, const float **norm);

cudaError_t launch_mlp_infer_tc(const __nv_bfloat16 *X, float *Y, const MlpDev &w, int64_t n, int *err, int swap,
                                cudaStream_t st);

// C[M][N] (op) = op(A)[M][K] * op(B)[K][N]; A, B BF16 row-major with the
// given leading dimensions; TA/TB = operand stored transposed.
enum { kEpiStore = 0, kEpiDact = 1, kEpiAtomic = 2 };
struct GemmArgs {
    const __nv_bfloat16 *A, *B;
    int64_t lda, ldb;
    int ta, tb;
    int M, N, K;
    int epi;
    const float *bias;           // kEpiStore: + bias[n]
    float *C;                    // kEpiStore / kEpiAtomic: FP32 out [M][N]
    __nv_bfloat16 *Cb;           // kEpiStore: BF16 of act(C); kEpiDact: BF16 of acc * silu'(Z)
    int act;                     // kEpiStore: 1 = SiLU for Cb
    const float *Z;              // kEpiDact: pre-activation [M][N]
    int ksplit;                  // kEpiAtomic: split K over grid.z
    int *err;                    // set to 2 if a tensor-core completion wait ran out (or NULL)
    float *partial;              // kEpiAtomic with ksplit > 1: [slices][M][N] workspace; the slices
                                 // are then added into C in slice order (same bits every run);
                                 // NULL = float atomics into C (order-dependent last bits)
};
// Slices of a split-K GEMM and the workspace floats it needs (0 without a split).
int gemm_splitk_slices(int K, int ksplit);
cudaError_t launch_gemm_bf16(const GemmArgs &g, cudaStream_t st);
// W2^T [in][out] and W3^T [in][out] from W2 [out][in], W3 [out][in] (BF16).
cudaError_t launch_transpose_w(const __nv_bfloat16 *w2, const __nv_bfloat16 *w3, __nv_bfloat16 *w2t,
                               __nv_bfloat16 *w3t, cudaStream_t st);

}  // namespace lqt
