// k_mlp_tc.cu -- BF16 MLP inference on the 5th-generation tensor cores.
//
// Network of the learned surrogate: 48 -> 128 -> 128 -> 48, SiLU between
// layers, BF16 weights and activations, FP32 accumulation.  A persistent CTA of
// 128 threads (one warpgroup) holds the three weight matrices in shared memory
// and walks tiles of 128 rows: per layer one elected thread issues
// tcgen05.mma (M = 128, K = 16 per instruction) into a TMEM accumulator and
// commits to an mbarrier; the four warps read their 32 TMEM lanes back with
// tcgen05.ld, add the bias, apply SiLU and write the next layer's BF16
// operand into shared memory.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "mlp.h"
#include "tc.cuh"

namespace lqt {

namespace {

constexpr int kTile = 128;
constexpr uint32_t kTmemCols = 256;        // [0,128): hidden accumulator, [128,176): output
constexpr uint32_t kWaitLimit = 1u << 24;  // bounded mbarrier polls

// shared-memory plan (bytes), all 1024-aligned
constexpr uint32_t kOffW1 = 0;                                      // 128 x 48
constexpr uint32_t kOffW2 = kOffW1 + kMlpHid * kMlpIn * 2;          // 128 x 128
constexpr uint32_t kOffW3 = kOffW2 + kMlpHid * kMlpHid * 2;         // 48 x 128
constexpr uint32_t kOffX = kOffW3 + kMlpOut * kMlpHid * 2;          // 128 x 48
constexpr uint32_t kOffH = kOffX + kTile * kMlpIn * 2;              // 128 x 128
constexpr uint32_t kOffBar = kOffH + kTile * kMlpHid * 2;           // mbarrier + tmem slot
constexpr uint32_t kSmemBytes = kOffBar + 64;

// Copy a row-major [R][K] BF16 matrix from global into the K-major core layout.
__device__ void stage_kmajor(uint8_t *dst, const __nv_bfloat16 *src, int R, int K)
{
    const int chunks = R * (K / 8);
    for (int c = threadIdx.x; c < chunks; c += blockDim.x) {
        const int r = c / (K / 8), kg = c % (K / 8);
        const uint4 v = *reinterpret_cast<const uint4 *>(src + (int64_t)r * K + kg * 8);
        *reinterpret_cast<uint4 *>(dst + tc::kmaj_off(r, kg * 8, K)) = v;
    }
}

__device__ __forceinline__ float silu(float x) { return x / (1.0f + __expf(-x)); }

// GEMM D[128 x N] = A[128 x K] * B[N x K]^T from shared memory into TMEM.
__device__ __forceinline__ void gemm(uint32_t tmem_d, const uint8_t *A, const uint8_t *B, int K, int N, bool swap)
{
    const uint32_t lbo = 128, sbo = (uint32_t)(K / 8) * 128;
    const uint32_t l = swap ? sbo : lbo, s = swap ? lbo : sbo;
    const uint32_t id = tc::idesc_bf16_f32(128, N);
    const uint32_t a0 = tc::smem_u32(A), b0 = tc::smem_u32(B);
    for (int kk = 0; kk < K / 16; ++kk) {
        const uint32_t step = (uint32_t)kk * 256;     // two core matrices along K
        tc::mma_bf16(tmem_d, tc::smem_desc(a0 + step, l, s), tc::smem_desc(b0 + step, l, s), id, kk > 0);
    }
}

}  // namespace

// X: [n][48] BF16 (normalised inputs), Y: [n][48] FP32 outputs.
__global__ void __launch_bounds__(128, 1) k_mlp_infer_tc(const __nv_bfloat16 *__restrict__ X, float *__restrict__ Y,
                                                         MlpDev w, int64_t n, int *err, int swap)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + kOffBar);
    uint32_t *tslot = reinterpret_cast<uint32_t *>(smem + kOffBar + 16);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    stage_kmajor(smem + kOffW1, w.w1t, kMlpHid, kMlpIn);
    stage_kmajor(smem + kOffW2, w.w2t, kMlpHid, kMlpHid);
    stage_kmajor(smem + kOffW3, w.w3t, kMlpOut, kMlpHid);
    if (tid == 0) {
        tc::mbar_init(bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) tc::tmem_alloc(tslot, kTmemCols);
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = *tslot;
    const uint32_t t_hid = tmem, t_out = tmem + 128;
    const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
    uint32_t phase = 0;
    bool ok = true;
    const int64_t ntiles = (n + kTile - 1) / kTile;

    for (int64_t tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
        const int64_t row = tile * kTile + tid;
        // this thread's input row -> sX
        uint4 xin[kMlpIn / 8];
#pragma unroll
        for (int j = 0; j < kMlpIn / 8; ++j)
            xin[j] = row < n ? *reinterpret_cast<const uint4 *>(X + row * kMlpIn + j * 8) : make_uint4(0, 0, 0, 0);
#pragma unroll
        for (int j = 0; j < kMlpIn / 8; ++j)
            *reinterpret_cast<uint4 *>(smem + kOffX + tc::kmaj_off(tid, j * 8, kMlpIn)) = xin[j];
        tc::fence_proxy_async();
        __syncthreads();

        // three layers
        for (int layer = 0; layer < 3 && ok; ++layer) {
            if (tid == 0) {
                tc::fence_after();
                if (layer == 0) gemm(t_hid, smem + kOffX, smem + kOffW1, kMlpIn, kMlpHid, swap);
                else if (layer == 1) gemm(t_hid, smem + kOffH, smem + kOffW2, kMlpHid, kMlpHid, swap);
                else gemm(t_out, smem + kOffH, smem + kOffW3, kMlpHid, kMlpOut, swap);
                tc::mma_commit(bar);
            }
            if (!tc::mbar_wait(bar, phase, kWaitLimit)) {
                // give the MMA in flight one more bounded wait before TMEM is freed
                tc::mbar_wait(bar, phase, kWaitLimit);
                if (tid == 0) atomicExch(err, 1);
                ok = false;
                break;
            }
            phase ^= 1;
            tc::fence_after();
            if (layer < 2) {
                const float *bias = layer == 0 ? w.b1 : w.b2;
#pragma unroll
                for (int c = 0; c < kMlpHid; c += 16) {
                    float v[16];
                    tc::tmem_ld16(t_hid + lane_base + c, v);
                    uint32_t packed[8];
#pragma unroll
                    for (int i = 0; i < 8; ++i) {
                        const float a = silu(v[2 * i] + bias[c + 2 * i]);
                        const float b = silu(v[2 * i + 1] + bias[c + 2 * i + 1]);
                        __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
                        packed[i] = *reinterpret_cast<uint32_t *>(&h);
                    }
                    uint8_t *dst = smem + kOffH;
                    *reinterpret_cast<uint4 *>(dst + tc::kmaj_off(tid, c, kMlpHid)) =
                        make_uint4(packed[0], packed[1], packed[2], packed[3]);
                    *reinterpret_cast<uint4 *>(dst + tc::kmaj_off(tid, c + 8, kMlpHid)) =
                        make_uint4(packed[4], packed[5], packed[6], packed[7]);
                }
                tc::fence_before();
                tc::fence_proxy_async();
                __syncthreads();
            } else {
#pragma unroll
                for (int c = 0; c < kMlpOut; c += 16) {
                    float v[16];
                    tc::tmem_ld16(t_out + lane_base + c, v);
                    if (row < n) {
#pragma unroll
                        for (int i = 0; i < 16; ++i) Y[row * kMlpOut + c + i] = v[i] + w.b3[c + i];
                    }
                }
                tc::fence_before();
                __syncthreads();
            }
        }
        (void)lane;
    }
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, kTmemCols);
}

cudaError_t launch_mlp_infer_tc(const __nv_bfloat16 *X, float *Y, const MlpDev &w, int64_t n, int *err, int swap,
                                cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    static std::atomic<uint64_t> attr_done{0};
    cudaError_t e = tc::smem_attr_once(k_mlp_infer_tc, kSmemBytes, attr_done);
    if (e != cudaSuccess) return e;
    int dev = 0, nsm = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int64_t ntiles = (n + kTile - 1) / kTile;
    // at most 2 CTAs per SM (shared memory admits 2; 2 x 256 TMEM columns =
    // the SM's 512), so tcgen05.alloc never waits for another CTA
    const int64_t grid = ntiles < 2LL * nsm ? ntiles : 2LL * nsm;
    k_mlp_infer_tc<<<(unsigned)grid, 128, kSmemBytes, st>>>(X, Y, w, n, err, swap);
    return cudaGetLastError();
}

}  // namespace lqt
