// k_mlp_train.cu -- training kernels of the learned surrogate: a BF16
// tensor-core GEMM (mma.sync m16n8k16, FP32 accumulate) with the epilogues the
// forward and backward passes need, the loss gradient and the Adam update.
// Training runs once, off the simulation's hot path; the per-macro-step
// inference uses the tcgen05 kernel in k_mlp_tc.cu.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "mlp.h"

namespace lqt {

namespace {

constexpr int kBM = 64, kBN = 64, kBK = 16;

__device__ __forceinline__ float sigm(float z) { return 1.0f / (1.0f + __expf(-z)); }

__device__ __forceinline__ void mma16816(float *c, const uint32_t *a, const uint32_t *b)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ uint32_t pack2(__nv_bfloat16 lo, __nv_bfloat16 hi)
{
    __nv_bfloat162 v;
    v.x = lo;
    v.y = hi;
    return *reinterpret_cast<uint32_t *>(&v);
}

// 128 threads, CTA tile 64 x 64, warp tile 32 x 32 (2 x 4 mma tiles).
__global__ void __launch_bounds__(128) k_gemm_bf16(GemmArgs g)
{
    __shared__ __nv_bfloat16 sA[kBM][kBK + 8];
    __shared__ __nv_bfloat16 sB[kBK][kBN + 8];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.y * kBM, n0 = blockIdx.x * kBN;
    const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
    const int grp = lane >> 2, tig = lane & 3;
    float acc[2][4][4] = {};
    int kbeg = 0, kend = g.K;
    if (g.epi == kEpiAtomic && g.ksplit > 1) {
        const int chunk = ((g.K + g.ksplit - 1) / g.ksplit + kBK - 1) / kBK * kBK;
        kbeg = blockIdx.z * chunk;
        kend = min(g.K, kbeg + chunk);
    }
    const __nv_bfloat16 zero = __float2bfloat16(0.0f);
    for (int k0 = kbeg; k0 < kend; k0 += kBK) {
        for (int i = tid; i < kBM * kBK; i += 128) {
            const int r = i / kBK, c = i % kBK;
            const int m = m0 + r, k = k0 + c;
            __nv_bfloat16 v = zero;
            if (m < g.M && k < kend) v = g.ta ? g.A[(int64_t)k * g.lda + m] : g.A[(int64_t)m * g.lda + k];
            sA[r][c] = v;
        }
        for (int i = tid; i < kBK * kBN; i += 128) {
            const int r = i / kBN, c = i % kBN;
            const int k = k0 + r, n = n0 + c;
            __nv_bfloat16 v = zero;
            if (n < g.N && k < kend) v = g.tb ? g.B[(int64_t)n * g.ldb + k] : g.B[(int64_t)k * g.ldb + n];
            sB[r][c] = v;
        }
        __syncthreads();
#pragma unroll
        for (int mi = 0; mi < 2; ++mi) {
            uint32_t a[4];
            const int r = wm + mi * 16 + grp;
            a[0] = pack2(sA[r][tig * 2], sA[r][tig * 2 + 1]);
            a[1] = pack2(sA[r + 8][tig * 2], sA[r + 8][tig * 2 + 1]);
            a[2] = pack2(sA[r][tig * 2 + 8], sA[r][tig * 2 + 9]);
            a[3] = pack2(sA[r + 8][tig * 2 + 8], sA[r + 8][tig * 2 + 9]);
#pragma unroll
            for (int ni = 0; ni < 4; ++ni) {
                uint32_t b[2];
                const int c = wn + ni * 8 + grp;
                b[0] = pack2(sB[tig * 2][c], sB[tig * 2 + 1][c]);
                b[1] = pack2(sB[tig * 2 + 8][c], sB[tig * 2 + 9][c]);
                mma16816(acc[mi][ni], a, b);
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int mi = 0; mi < 2; ++mi)
#pragma unroll
        for (int ni = 0; ni < 4; ++ni)
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int m = m0 + wm + mi * 16 + grp + (e >= 2 ? 8 : 0);
                const int n = n0 + wn + ni * 8 + tig * 2 + (e & 1);
                if (m >= g.M || n >= g.N) continue;
                const int64_t o = (int64_t)m * g.N + n;
                float v = acc[mi][ni][e];
                if (g.epi == kEpiStore) {
                    if (g.bias) v += g.bias[n];
                    if (g.C) g.C[o] = v;
                    if (g.Cb) g.Cb[o] = __float2bfloat16(g.act ? v * sigm(v) : v);
                } else if (g.epi == kEpiDact) {
                    const float z = g.Z[o], s = sigm(z);
                    g.Cb[o] = __float2bfloat16(v * (s + z * s * (1.0f - s)));
                } else {
                    atomicAdd(&g.C[o], v);
                }
            }
}

}  // namespace

cudaError_t launch_gemm_bf16(const GemmArgs &g, cudaStream_t st)
{
    if (g.M <= 0 || g.N <= 0 || g.K <= 0) return cudaSuccess;
    dim3 grid((g.N + kBN - 1) / kBN, (g.M + kBM - 1) / kBM, g.epi == kEpiAtomic && g.ksplit > 1 ? g.ksplit : 1);
    k_gemm_bf16<<<grid, 128, 0, st>>>(g);
    return cudaGetLastError();
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
cudaError_t launch_adam(float *p, const float *g, float *m, float *v, __nv_bfloat16 *pb, int64_t n, float lr,
                        float b1, float b2, float eps, float c1, float c2, cudaStream_t st)
{
    const int64_t nb = (n + 255) / 256;
    k_adam<<<(unsigned)(nb > 1024 ? 1024 : nb), 256, 0, st>>>(p, g, m, v, pb, n, lr, b1, b2, eps, c1, c2);
    return cudaGetLastError();
}

}  // namespace lqt
