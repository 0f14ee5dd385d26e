// k_mlp_train.cu -- training kernels of the learned surrogate: a BF16
// GEMM on the 5th-generation tensor cores (tcgen05.mma into a TMEM
// accumulator, FP32) with the epilogues the forward and backward passes need,
// the loss gradient and the Adam update.  Training runs once, off the
// simulation's hot path; the per-macro-step inference uses the tcgen05 kernel
// in k_sur_grid.cu / k_mlp_tc.cu.
#include <algorithm>

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "mlp.h"
#include "tc.cuh"

namespace lqt {

namespace {

constexpr int kTM = 128;                   // rows per CTA (TMEM lanes)
constexpr int kKC = 64;                    // K per staged chunk (4 MMAs of K = 16)
constexpr int kMaxN = 256;                 // N per CTA (one MMA)
constexpr uint32_t kWaitLimit = 1u << 24;  // bounded mbarrier polls
// dynamic shared memory per CTA: A chunk, B chunk, mbarrier and TMEM slot;
// padded to 60 KB so that at most 3 CTAs share an SM (3 x 128 TMEM columns
// of the SM's 512: tcgen05.alloc never has to wait)
constexpr uint32_t kOffA = 0;
constexpr uint32_t kOffB = kOffA + kTM * kKC * 2;
constexpr uint32_t kOffBar = kOffB + kMaxN * kKC * 2;
constexpr uint32_t kSmemBytes = 60 * 1024;
constexpr int kEpPitch = 33;               // epilogue slab row pitch (floats): no bank conflicts
static_assert(kOffBar + 16 <= kSmemBytes, "shared memory plan");
static_assert(kTM * kEpPitch * 4 <= kOffBar, "epilogue slab fits the staging buffers");

__device__ __forceinline__ float sigm(float z) { return 1.0f / (1.0f + __expf(-z)); }

// K per slice of a split-K GEMM: whole staging chunks.
__host__ __device__ inline int splitk_chunk(int K, int ksplit)
{
    return ((K + ksplit - 1) / ksplit + kKC - 1) / kKC * kKC;
}

// C[o] += the split-K slices of element o, added in slice order.
__global__ void k_splitk_reduce(const float *__restrict__ partial, int64_t mn, int slices, float *__restrict__ C)
{
    for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < mn; o += (int64_t)gridDim.x * blockDim.x) {
        // unrolled: the slices' loads are issued together, the additions
        // stay in slice order
        float acc = 0.f;
#pragma unroll 16
        for (int z = 0; z < slices; ++z) acc += partial[(int64_t)z * mn + o];
        C[o] += acc;
    }
}

// One 8-element K chunk of row r of op(X) (X[r][k] = ta ? src[k * ld + r] :
// src[r * ld + k]) for k = k0 .. k0 + 7, zero outside rows < R and k < kend.
__device__ __forceinline__ uint4 load_chunk8(const __nv_bfloat16 *src, int64_t ld, int t, int r, int R, int k0,
                                             int kend)
{
    if (r >= R) return make_uint4(0, 0, 0, 0);
    if (!t && k0 + 8 <= kend && (ld & 7) == 0 && (k0 & 7) == 0)
        return *reinterpret_cast<const uint4 *>(src + (int64_t)r * ld + k0);
    uint32_t p[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        uint16_t h[2];
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const int k = k0 + 2 * i + j;
            __nv_bfloat16 v = __float2bfloat16(0.0f);
            if (k < kend) v = t ? src[(int64_t)k * ld + r] : src[(int64_t)r * ld + k];
            h[j] = __bfloat16_as_ushort(v);
        }
        p[i] = (uint32_t)h[0] | ((uint32_t)h[1] << 16);
    }
    return make_uint4(p[0], p[1], p[2], p[3]);
}

// C[M][N] (epilogue) = op(A)[M][K] * op(B)[K][N].  One CTA of 128 threads per
// 128-row tile and (for the split weight gradients) K range: the tile's A rows
// and all N rows of op(B)^T are staged chunk by chunk in the K-major core
// layout; one elected thread issues the MMAs and commits to an mbarrier; the
// accumulator (row m in TMEM lane m) goes through the epilogue by its thread.
__global__ void __launch_bounds__(128) k_gemm_tc(GemmArgs g)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + kOffBar);
    uint32_t *tslot = reinterpret_cast<uint32_t *>(smem + kOffBar + 8);
    const int tid = threadIdx.x, warp = tid >> 5;
    const int m0 = blockIdx.y * kTM;
    const int npad = (g.N + 15) / 16 * 16;
    uint32_t ncols = 32;
    while ((int)ncols < npad) ncols <<= 1;
    int kbeg = 0, kend = g.K;
    if (g.epi == kEpiAtomic && g.ksplit > 1) {
        const int chunk = splitk_chunk(g.K, g.ksplit);
        kbeg = blockIdx.z * chunk;
        kend = min(g.K, kbeg + chunk);
    }
    // this CTA's slice of a split-K GEMM with a workspace: plain stores
    float *const slab = (g.epi == kEpiAtomic && g.partial) ? g.partial + (int64_t)blockIdx.z * g.M * g.N : nullptr;
    if (tid == 0) {
        tc::mbar_init(bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) tc::tmem_alloc(tslot, ncols);
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = *tslot;
    const uint32_t idesc = tc::idesc_bf16_f32(kTM, npad);
    uint32_t phase = 0;
    bool ok = true;
    int nchunk = 0;
    for (int k0 = kbeg; k0 < kend && ok; k0 += kKC, ++nchunk) {
        // stage: consecutive threads take consecutive rows (coalesced for the
        // transposed operands, whose rows are contiguous in memory)
        for (int c = tid; c < kTM * (kKC / 8); c += 128) {
            const int r = c % kTM, kg = c / kTM;
            *reinterpret_cast<uint4 *>(smem + kOffA + tc::kmaj_off(r, kg * 8, kKC)) =
                load_chunk8(g.A, g.lda, g.ta, m0 + r, g.M, k0 + kg * 8, kend);
        }
        for (int c = tid; c < npad * (kKC / 8); c += 128) {
            const int r = c % npad, kg = c / npad;
            // op(B)^T row n: B[n][k] when stored transposed (tb), else B[k][n]
            *reinterpret_cast<uint4 *>(smem + kOffB + tc::kmaj_off(r, kg * 8, kKC)) =
                load_chunk8(g.B, g.ldb, !g.tb, r, g.N, k0 + kg * 8, kend);
        }
        tc::fence_proxy_async();
        tc::fence_before();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after();
            const uint32_t lbo = 128, sbo = (kKC / 8) * 128;
            const uint32_t a0 = tc::smem_u32(smem + kOffA), b0 = tc::smem_u32(smem + kOffB);
            for (int kk = 0; kk < kKC / 16; ++kk)
                tc::mma_bf16(tmem, tc::smem_desc(a0 + kk * 256, lbo, sbo), tc::smem_desc(b0 + kk * 256, lbo, sbo),
                             idesc, (nchunk > 0 || kk > 0) ? 1u : 0u);
            tc::mma_commit(bar);
        }
        // the chunk's smem is reused only after its MMAs completed; the
        // decision is made for the whole CTA at once
        const bool w_ok = tc::mbar_wait(bar, phase, kWaitLimit);
        if (!__syncthreads_and(w_ok ? 1 : 0)) {
            if (!w_ok) tc::mbar_wait(bar, phase, kWaitLimit);   // let the MMAs in flight land before TMEM is freed
            if (tid == 0 && g.err) atomicExch(g.err, 2);
            ok = false;
        }
        phase ^= 1;
        tc::fence_after();
        __syncthreads();
    }
    if (ok && nchunk > 0) {
        // epilogue in 32-column slabs: each thread moves its row (TMEM lane)
        // into shared memory, then every warp writes whole row segments, so
        // the stores (or atomics) of a warp are 32 consecutive elements
        float *ep = reinterpret_cast<float *>(smem);          // the staging buffers are free now
        const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16);
        const int lane = tid & 31;
        for (int n0 = 0; n0 < g.N; n0 += 32) {
            float v[32];
            tc::tmem_ld32(taddr + n0, v);                     // whole warp
#pragma unroll
            for (int i = 0; i < 32; ++i) ep[tid * kEpPitch + i] = v[i];
            __syncthreads();
            // a warp takes rows warp, warp + 4, ...: the loop is unrolled and
            // the pointers restrict-qualified, so that its global loads (the
            // bias once, Z of every row) are issued together instead of one
            // latency per row behind the previous row's stores
            const int n = n0 + lane;
            const bool nin = n < g.N;
            const float *__restrict__ Zp = g.Z;
            float *__restrict__ Cp = g.C;
            __nv_bfloat16 *__restrict__ Cbp = g.Cb;
            constexpr int kRows = kTM / 4;
            if (g.epi == kEpiDact) {
                float zv[kRows];
#pragma unroll
                for (int i = 0; i < kRows; ++i) {
                    const int m = m0 + warp + 4 * i;
                    zv[i] = (nin && m < g.M) ? Zp[(int64_t)m * g.N + n] : 0.f;
                }
#pragma unroll
                for (int i = 0; i < kRows; ++i) {
                    const int r = warp + 4 * i, m = m0 + r;
                    if (!nin || m >= g.M) continue;
                    const float x = ep[r * kEpPitch + lane], z = zv[i], sz = sigm(z);
                    Cbp[(int64_t)m * g.N + n] = __float2bfloat16(x * (sz + z * sz * (1.0f - sz)));
                }
            } else if (g.epi == kEpiStore) {
                const float bn = (nin && g.bias) ? g.bias[n] : 0.f;
#pragma unroll 8
                for (int i = 0; i < kRows; ++i) {
                    const int r = warp + 4 * i, m = m0 + r;
                    if (!nin || m >= g.M) continue;
                    const int64_t o = (int64_t)m * g.N + n;
                    const float x = ep[r * kEpPitch + lane] + bn;
                    if (Cp) Cp[o] = x;
                    if (Cbp) Cbp[o] = __float2bfloat16(g.act ? x * sigm(x) : x);
                }
            } else {
#pragma unroll 8
                for (int i = 0; i < kRows; ++i) {
                    const int r = warp + 4 * i, m = m0 + r;
                    if (!nin || m >= g.M) continue;
                    const int64_t o = (int64_t)m * g.N + n;
                    const float x = ep[r * kEpPitch + lane];
                    if (slab) slab[o] = x;
                    else atomicAdd(&Cp[o], x);
                }
            }
            __syncthreads();
        }
    }
    tc::fence_before();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, ncols);
}

}  // namespace

cudaError_t launch_gemm_bf16(const GemmArgs &g, cudaStream_t st)
{
    if (g.M <= 0 || g.N <= 0 || g.K <= 0) return cudaSuccess;
    if (g.N > kMaxN) return cudaErrorInvalidValue;
    static std::atomic<uint64_t> attr_done{0};
    cudaError_t e = tc::smem_attr_once(k_gemm_tc, kSmemBytes, attr_done);
    if (e != cudaSuccess) return e;
    const int slices = gemm_splitk_slices(g.K, g.epi == kEpiAtomic ? g.ksplit : 1);
    dim3 grid(1, (g.M + kTM - 1) / kTM, slices > 0 ? slices : 1);
    k_gemm_tc<<<grid, 128, kSmemBytes, st>>>(g);
    e = cudaGetLastError();
    if (e == cudaSuccess && slices > 0 && g.partial) {
        const int64_t mn = (int64_t)g.M * g.N;
        k_splitk_reduce<<<(unsigned)std::min<int64_t>((mn + 255) / 256, 1024), 256, 0, st>>>(g.partial, mn, slices,
                                                                                            g.C);
        e = cudaGetLastError();
    }
    return e;
}

// Only slices that hold at least one chunk of K are launched, so every slice
// of the workspace is written before the reduction reads it.
int gemm_splitk_slices(int K, int ksplit)
{
    if (ksplit <= 1 || K <= 0) return 0;
    const int chunk = splitk_chunk(K, ksplit);
    return (K + chunk - 1) / chunk;
}

// dst[c][r] = src[r][c] for the hidden and output weights (BF16): the
// backward pass's data-gradient GEMMs read W as an N x K operand with K
// contiguous, which the staging then copies with 16-byte loads.
__global__ void k_transpose_w(const __nv_bfloat16 *__restrict__ w2, const __nv_bfloat16 *__restrict__ w3,
                              __nv_bfloat16 *__restrict__ w2t, __nv_bfloat16 *__restrict__ w3t)
{
    const int n2 = kMlpHid * kMlpHid, n3 = kMlpOut * kMlpHid;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n2 + n3; i += gridDim.x * blockDim.x) {
        if (i < n2) {
            const int r = i / kMlpHid, c = i - r * kMlpHid;
            w2t[c * kMlpHid + r] = w2[i];
        } else {
            const int j = i - n2, r = j / kMlpHid, c = j - r * kMlpHid;
            w3t[c * kMlpOut + r] = w3[j];
        }
    }
}

// ---- loss gradient and Adam -------------------------------------------------
// dY = 2 (Y - T) mask / (B * nvalid); loss += sum (Y - T)^2 mask (FP64 atomics per block).
__global__ void k_mse_grad(const float *__restrict__ Y, const float *__restrict__ T, int64_t B, int nvalid,
                           __nv_bfloat16 *__restrict__ dY, double *__restrict__ loss)
{
    __shared__ double red[256];
    double acc = 0.0;
    const float s = 2.0f / (float)(B * nvalid);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < B * kMlpOut;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int c = (int)(i % kMlpOut);
        float d = 0.0f;
        if (c < nvalid) {
            d = Y[i] - T[i];
            acc += (double)d * d;
        }
        dY[i] = __float2bfloat16(s * d);
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicAdd(loss, red[0]);
}

// Column sums of a BF16 [B][N] matrix into FP32 g[N] (bias gradients).
__global__ void k_colsum(const __nv_bfloat16 *__restrict__ X, int64_t B, int N, float *__restrict__ g)
{
    const int n = blockIdx.x;
    float acc = 0.f;
    for (int64_t r = threadIdx.x; r < B; r += blockDim.x) acc += __bfloat162float(X[r * N + n]);
    __shared__ float red[256];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) g[n] = red[0];
}

// Adam with bias correction; master weights FP32, a BF16 copy for the kernels.
__global__ void k_adam(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m, float *__restrict__ v,
                       __nv_bfloat16 *__restrict__ pb, int64_t n, float lr, float b1, float b2, float eps, float c1,
                       float c2)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float pn = p[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
        p[i] = pn;
        if (pb) pb[i] = __float2bfloat16(pn);
    }
}

cudaError_t launch_mse_grad(const float *Y, const float *T, int64_t B, int nvalid, __nv_bfloat16 *dY, double *loss,
                            cudaStream_t st)
{
    k_mse_grad<<<256, 256, 0, st>>>(Y, T, B, nvalid, dY, loss);
    return cudaGetLastError();
}
cudaError_t launch_colsum(const __nv_bfloat16 *X, int64_t B, int N, float *g, cudaStream_t st)
{
    k_colsum<<<N, 256, 0, st>>>(X, B, N, g);
    return cudaGetLastError();
}
cudaError_t launch_transpose_w(const __nv_bfloat16 *w2, const __nv_bfloat16 *w3, __nv_bfloat16 *w2t,
                               __nv_bfloat16 *w3t, cudaStream_t st)
{
    k_transpose_w<<<(kMlpHid * (kMlpHid + kMlpOut) + 255) / 256, 256, 0, st>>>(w2, w3, w2t, w3t);
    return cudaGetLastError();
}

cudaError_t launch_adam(float *p, const float *g, float *m, float *v, __nv_bfloat16 *pb, int64_t n, float lr,
                        float b1, float b2, float eps, float c1, float c2, cudaStream_t st)
{
    const int64_t nb = (n + 255) / 256;
    k_adam<<<(unsigned)(nb > 1024 ? 1024 : nb), 256, 0, st>>>(p, g, m, v, pb, n, lr, b1, b2, eps, c1, c2);
    return cudaGetLastError();
}

}  // namespace lqt
