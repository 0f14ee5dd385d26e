// k_sur_grid.cu -- the learned surrogate's macro step on a tissue grid.
//
// At every macro-step boundary (every nsub plain steps) one persistent
// kernel walks the tissue voxels in tiles of 128.  A voxel is offered to the
// surrogate when |dV/dt| over the last plain step (both V buffers are still
// resident) is at most dvdt_max and no stimulus reaches it during the macro
// step (the fast upstroke always takes plain steps; a slow rise into the dome
// may take macro steps, with the detector run at every substep so that the
// running peak that sets the APD90 level is kept).  For the offered voxels of
// a tile
//   1. each thread writes its voxel's normalised BF16 features into shared
//      memory (row = thread, tcgen05 K-major core-matrix layout);
//   2. one elected thread runs the 48 -> 128 -> 128 -> 48 network with
//      tcgen05.mma into TMEM (three layers, each bias added by one more MMA
//      k-step against a constant ones tile; the threads read the hidden
//      accumulators back with tcgen05.ld, apply SiLU and write the next FP16
//      operand into shared memory);
//   3. each thread reloads its state, advances it by one coarse TPORd step of
//      the macro length (dt = nsub * dt, no diffusion) and adds the
//      network's output, the correction to the state after nsub plain
//      steps, read from TMEM.
// Residual check: every normalised correction within +-kappa times its bound
// (the largest correction of the training set: the network is not
// extrapolating), gates within [0, 1] up to a small tolerance (then clamped),
// concentrations positive, and the macro step's ionic V change at most
// vstep_max.  A voxel that passes stores its new state and its ionic
// dV/dt for the macro step in `rate`; during the next nsub steps
// k_sur_substep moves its V by that rate plus diffusion only.  Every other
// voxel gets rate = NaN and joins the list of voxels that k_grid_step
// advances with the plain step.
//
// Layout: one CTA of four warpgroups per SM.  The weights (BF16, 56 KB), the
// bias tiles and the normalisation are staged once per CTA; each warpgroup owns a
// 32 KB operand buffer (the 128 x 48 feature tile, then the 128 x 128 hidden
// tile in the same bytes) and 128 TMEM columns (hidden accumulator; the
// 48-column output reuses them once the hidden values are read), so the four
// warpgroups work on four tiles independently, synchronised by named
// barriers.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "k_grid.cuh"
#include "sur_dev.cuh"
#include "tc.cuh"

namespace lqt {

namespace {

constexpr int kTile = 128;
constexpr int kGroups = 4;                 // warpgroups (tiles in flight) per CTA
constexpr int kThreads = 128 * kGroups;
constexpr uint32_t kColsPerGroup = 128;
constexpr uint32_t kTmemCols = kColsPerGroup * kGroups;   // the SM's 512 columns
constexpr uint32_t kWaitLimit = 1u << 24;  // bounded mbarrier polls
constexpr float kDetMargin = 2.f;          // mV a surrogate voxel cannot cover in one macro step

// Operand types: the first layer's inputs and weights are BF16; the hidden
// layers' activations and weights are FP16 (finer rounding for the packed SiLU
// below); accumulation is FP32 throughout.  No MMA mixes the two types.
constexpr uint32_t kOffW1 = 0;                                      // 128 x 48 BF16
constexpr uint32_t kOffW2 = kOffW1 + kMlpHid * kMlpIn * 2;          // 128 x 128 FP16
constexpr uint32_t kOffW3 = kOffW2 + kMlpHid * kMlpHid * 2;         // 48 x 128 FP16
constexpr uint32_t kOffXH = kOffW3 + kMlpOut * kMlpHid * 2;         // per group: BF16 features, then FP16 hidden
constexpr uint32_t kXHBytes = kTile * kMlpHid * 2;
// bias k-step operands (K = 16 core-matrix tiles): A = ones in columns 0, 1;
// B = the bias split into hi + lo parts in columns 0, 1
constexpr uint32_t kBiasK = 16;
constexpr uint32_t kOffOnes = kOffXH + kGroups * kXHBytes;          // 128 x 16 BF16
constexpr uint32_t kOffOnesH = kOffOnes + kTile * kBiasK * 2;       // 128 x 16 FP16
constexpr uint32_t kOffB1 = kOffOnesH + kTile * kBiasK * 2;         // 128 x 16 (b1 / 2, BF16)
constexpr uint32_t kOffB2 = kOffB1 + kMlpHid * kBiasK * 2;          // 128 x 16 (b2 / 2, FP16)
constexpr uint32_t kOffB3 = kOffB2 + kMlpHid * kBiasK * 2;          // 48 x 16 (b3, FP16)
constexpr uint32_t kOffNorm = kOffB3 + kMlpOut * kBiasK * 2;        // 4 x 48 floats
constexpr uint32_t kOffBar = kOffNorm + 4 * kMlpIn * 4;             // per group mbarrier; tmem slot
constexpr uint32_t kSmemBytes = kOffBar + 8 * kGroups + 16;
static_assert(kOffXH % 1024 == 0 && kXHBytes % 1024 == 0, "operand tiles 1 KB aligned");
static_assert(kSmemBytes <= 227 * 1024, "shared memory");
static_assert(kOffNorm % 16 == 0, "normalisation pairs read as float4");

// Copy a row-major [R][K] BF16 matrix into the K-major core layout, times
// `scale` (a power of two: exact in BF16).
__device__ void stage_kmajor(uint8_t *dst, const __nv_bfloat16 *src, int R, int K, float scale)
{
    const int chunks = R * (K / 8);
    const __nv_bfloat162 sc = __floats2bfloat162_rn(scale, scale);
    for (int c = threadIdx.x; c < chunks; c += blockDim.x) {
        const int r = c / (K / 8), kg = c % (K / 8);
        uint4 v = *reinterpret_cast<const uint4 *>(src + (int64_t)r * K + kg * 8);
        __nv_bfloat162 *h = reinterpret_cast<__nv_bfloat162 *>(&v);
#pragma unroll
        for (int i = 0; i < 4; ++i) h[i] = __hmul2(h[i], sc);
        *reinterpret_cast<uint4 *>(dst + tc::kmaj_off(r, kg * 8, K)) = v;
    }
}

// A row-major [R][K] FP32 matrix into the K-major core layout as FP16, times `scale`.
__device__ void stage_kmajor_f16(uint8_t *dst, const float *src, int R, int K, float scale)
{
    const int chunks = R * (K / 8);
    for (int c = threadIdx.x; c < chunks; c += blockDim.x) {
        const int r = c / (K / 8), kg = c % (K / 8);
        const float *s = src + (int64_t)r * K + kg * 8;
        uint32_t p[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const __half2 h = __floats2half2_rn(scale * s[2 * i], scale * s[2 * i + 1]);
            p[i] = *reinterpret_cast<const uint32_t *>(&h);
        }
        *reinterpret_cast<uint4 *>(dst + tc::kmaj_off(r, kg * 8, K)) = make_uint4(p[0], p[1], p[2], p[3]);
    }
}

// Bias operand of the extra k-step: row n = (hi, lo, 0, ...) with
// hi + lo = scale * b[n] to about twice the type's precision.
template <bool F16> __device__ void stage_bias(uint8_t *dst, const float *b, int N, float scale)
{
    for (int c = threadIdx.x; c < N * 2; c += blockDim.x) {
        const int n = c >> 1, kg = c & 1;
        uint4 v = make_uint4(0, 0, 0, 0);
        if (kg == 0) {
            const float x = scale * b[n];
            if (F16) {
                const __half hi = __float2half_rn(x);
                const __half lo = __float2half_rn(x - __half2float(hi));
                v.x = (uint32_t)__half_as_ushort(hi) | ((uint32_t)__half_as_ushort(lo) << 16);
            } else {
                const __nv_bfloat16 hi = __float2bfloat16_rn(x);
                const __nv_bfloat16 lo = __float2bfloat16_rn(x - __bfloat162float(hi));
                v.x = (uint32_t)__bfloat16_as_ushort(hi) | ((uint32_t)__bfloat16_as_ushort(lo) << 16);
            }
        }
        *reinterpret_cast<uint4 *>(dst + tc::kmaj_off(n, kg * 8, kBiasK)) = v;
    }
}

// SiLU of two hidden pre-activations, packed to the FP16 operand of the next
// layer: the hidden layers run with halved weights and biases, so the
// accumulator is h = x / 2 and SiLU(x) = x * sigmoid(x) = h + h * tanh(h).  h
// is rounded once to FP16, then one MUFU tanh.approx.f16x2 and one
// fma.rn.f16x2 produce the pair (three instructions for two values).
__device__ __forceinline__ uint32_t silu2_f16(float h0, float h1)
{
    const __half2 h = __floats2half2_rn(h0, h1);
    const uint32_t hu = *reinterpret_cast<const uint32_t *>(&h);
    uint32_t tu;
    asm("tanh.approx.f16x2 %0, %1;" : "=r"(tu) : "r"(hu));
    const __half2 r = __hfma2(h, *reinterpret_cast<const __half2 *>(&tu), h);
    return *reinterpret_cast<const uint32_t *>(&r);
}

// D[128 x N] = A[128 x K] * B[N x K]^T + ones * bias^T: K / 16 MMAs over the
// operands, then one k-step of the constant ones tile against the bias tile;
// every operand of the call is BF16 (f16 = false) or every one FP16.
__device__ __forceinline__ void gemm(uint32_t tmem_d, const uint8_t *A, const uint8_t *B, int K, int N,
                                     const uint8_t *ones, const uint8_t *bias, bool f16)
{
    const uint32_t lbo = 128, sbo = (uint32_t)(K / 8) * 128;
    const uint32_t id = f16 ? tc::idesc_f16_f32(128, N) : tc::idesc_bf16_f32(128, N);
    const uint32_t a0 = tc::smem_u32(A), b0 = tc::smem_u32(B);
    for (int kk = 0; kk < K / 16; ++kk) {
        const uint32_t step = (uint32_t)kk * 256;     // two core matrices along K
        tc::mma_bf16(tmem_d, tc::smem_desc(a0 + step, lbo, sbo), tc::smem_desc(b0 + step, lbo, sbo), id, kk > 0);
    }
    const uint32_t sb = (kBiasK / 8) * 128;
    tc::mma_bf16(tmem_d, tc::smem_desc(tc::smem_u32(ones), lbo, sb), tc::smem_desc(tc::smem_u32(bias), lbo, sb), id,
                 1u);
}

// Named barrier of one warpgroup (ids 1..4; 0 is __syncthreads).
__device__ __forceinline__ void wg_sync(int id) { asm volatile("bar.sync %0, 128;" ::"r"(id) : "memory"); }
__device__ __forceinline__ int wg_or(int id, int v)
{
    int r;
    asm volatile(
        "{\n.reg .pred p, q;\nsetp.ne.s32 p, %1, 0;\nbar.red.or.pred q, %2, 128, p;\nselp.s32 %0, 1, 0, q;\n}\n"
        : "=r"(r)
        : "r"(v), "r"(id)
        : "memory");
    return r;
}
__device__ __forceinline__ int wg_and(int id, int v)
{
    int r;
    asm volatile(
        "{\n.reg .pred p, q;\nsetp.ne.s32 p, %1, 0;\nbar.red.and.pred q, %2, 128, p;\nselp.s32 %0, 1, 0, q;\n}\n"
        : "=r"(r)
        : "r"(v), "r"(id)
        : "memory");
    return r;
}

// 32 consecutive FP32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float *v)
{
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// Per-voxel onsets: could the S1 stimulus of a voxel with this onset start
// within the next nsub + 1 steps (this cycle's or the next's)?  FP64, out of
// line for the reason given at onset_s1_on.
__device__ __noinline__ bool onset_s1_ahead(const GridDev<float> &gd, double tb, int nsub, float onset)
{
    const double on = gd.s1_start + (double)onset;
    const double span = (nsub + 1) * gd.dt;
    return (tb + span >= on && tb <= on + gd.s1_dur) || (tb - gd.bcl + span >= on);
}

// Does any stimulus reach voxel k during steps [ck.step, ck.step + nsub)?
// Window schedule: the current window (first with off > step) is the only
// candidate.  Per-voxel onsets: a conservative test on the within-cycle time.
__device__ __forceinline__ bool stim_ahead(const GridDev<float> &gd, const Clock &ck, uint8_t ctl, int64_t k,
                                           int nsub)
{
    const int64_t s0 = ck.step, s1 = ck.step + nsub;
    if ((ctl & kCtlS2) && gd.s2_win.on < s1 && gd.s2_win.off > s0) return true;
    if (!(ctl & kCtlS1)) return false;
    if (gd.onset) return onset_s1_ahead(gd, ck.tb, nsub, gd.onset[k]);
    const int32_t nwin = gd.win ? gd.nwin : 0;
    const int32_t w = ck.widx < 0 ? 0 : ck.widx;
    return w < nwin && gd.win[w].on < s1 && gd.win[w].off > s0;
}

}  // namespace

__global__ void __launch_bounds__(kThreads, 1) k_sur_grid(GridDev<float> gd, SurGrid sg, int cur, int dim)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int grp = tid >> 7, t = tid & 127;          // warpgroup, row within its tile
    const int bar_id = 1 + grp;
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + kOffBar) + grp;
    uint32_t *tslot = reinterpret_cast<uint32_t *>(smem + kOffBar + 8 * kGroups);
    float *nrm = reinterpret_cast<float *>(smem + kOffNorm);
    uint8_t *xh = smem + kOffXH + grp * kXHBytes;
    const bool use_net = sg.use_net != 0;

    // normalisation, rearranged once per CTA: (scale, -mean * scale) per
    // input (one FMA per feature), the output scales, and kappa times the
    // residual bounds
    for (int j = tid; j < kMlpIn; j += blockDim.x) {
        const float mu = sg.norm[j], sc = sg.norm[kMlpIn + j];
        nrm[2 * j] = sc;
        nrm[2 * j + 1] = -mu * sc;
        nrm[2 * kMlpIn + j] = sg.norm[2 * kMlpIn + j];
        nrm[3 * kMlpIn + j] = sg.kappa * sg.norm[3 * kMlpIn + j];
    }
    if (use_net) {
        // hidden layers halved (see silu2_bf16); biases as an extra k-step
        stage_kmajor(smem + kOffW1, sg.w.w1t, kMlpHid, kMlpIn, 0.5f);
        stage_kmajor_f16(smem + kOffW2, sg.w.w2f, kMlpHid, kMlpHid, 0.5f);
        stage_kmajor_f16(smem + kOffW3, sg.w.w3f, kMlpOut, kMlpHid, 1.0f);
        stage_bias<false>(smem + kOffB1, sg.w.b1, kMlpHid, 0.5f);
        stage_bias<true>(smem + kOffB2, sg.w.b2, kMlpHid, 0.5f);
        stage_bias<true>(smem + kOffB3, sg.w.b3, kMlpOut, 1.0f);
        for (int c = tid; c < kTile * 2; c += blockDim.x) {
            const int r = c >> 1, kg = c & 1;
            const uint32_t one_b = 0x3F80u, one_h = 0x3C00u;     // 1.0 in BF16, FP16
            const uint4 vb = kg == 0 ? make_uint4(one_b | (one_b << 16), 0, 0, 0) : make_uint4(0, 0, 0, 0);
            const uint4 vh = kg == 0 ? make_uint4(one_h | (one_h << 16), 0, 0, 0) : make_uint4(0, 0, 0, 0);
            *reinterpret_cast<uint4 *>(smem + kOffOnes + tc::kmaj_off(r, kg * 8, kBiasK)) = vb;
            *reinterpret_cast<uint4 *>(smem + kOffOnesH + tc::kmaj_off(r, kg * 8, kBiasK)) = vh;
        }
        if (t == 0) {
            tc::mbar_init(bar, 1);
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        }
        if (warp == 0) tc::tmem_alloc(tslot, kTmemCols);
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = use_net ? *tslot : 0u;
    // warp w of the CTA may access TMEM lanes 32 * (w % 4) .. + 31
    const uint32_t t_acc = tmem + grp * kColsPerGroup + ((uint32_t)((warp & 3) * 32) << 16);
    const uint32_t t_acc_mma = tmem + grp * kColsPerGroup;
    uint32_t phase = 0;
    bool net_ok = true;

    const Clock ck = *gd.clk;
    const float *__restrict__ V = gd.vg[cur];
    const float *__restrict__ Vp = gd.vg[cur ^ 1];
    const float inv_dt = sg.inv_dt, inv_mac = sg.inv_mac;
    const int64_t nt = gd.ntissue;
    const int64_t ntiles = (nt + kTile - 1) / kTile;
    unsigned long long n_offer = 0, n_acc = 0;
    const int64_t tstride = (int64_t)gridDim.x * kGroups;
    // an S1 window opens during this macro step: every detector records its rest
    bool opens = false;
    {
        const int32_t nwin = gd.win ? gd.nwin : 0;
        const int32_t w = ck.widx < 0 ? 0 : ck.widx;
        for (int32_t i = w; i < nwin && i < w + 2; ++i)
            opens |= gd.win[i].on >= ck.step && gd.win[i].on < ck.step + sg.nsub;
    }

    // the warpgroups are independent (own tiles, barrier, TMEM columns and
    // operand buffer); the loop is uniform within a warpgroup
    for (int64_t tile = (int64_t)blockIdx.x * kGroups + grp; tile < ntiles; tile += tstride) {
        const int64_t k = tile * kTile + t;
        bool elig = false, need_det = false;
        float vc = 0.f;
        int ct = 0;
        // 1. the state, loaded once (its loads need only k, so they are in
        //    flight while the index, V and detector loads resolve): the
        //    features are built from it and the coarse step advances it in
        //    registers while the first layer's MMAs run
        CellState<float> c;
        if (k < nt) {
            load_cell(c, gd.s, k);
            const int64_t g = dim == 1 ? k : (int64_t)gd.gidx[k];
            vc = V[g];
            const float dv = (vc - Vp[g]) * inv_dt;
            const uint8_t ctl = gd.ctl[k];
            ct = ctl & kCtlType;
            if (gd.det) {
                const float4 d = gd.det[k];
                const uint32_t ph = __float_as_uint(d.w) & 7u;
                // does the detector need this voxel's substeps?  A cycle that
                // opens; an activation crossing within reach; a slow rise
                // towards the peak (a dome without a notch: the fast upstroke
                // is excluded by the dV/dt bound); in the fall, the running
                // peak, the 50% (EAD) and the 90% levels
                const float amp = d.y - d.x;
                need_det = opens || ph == kDetRise || (ph == kDetWait && vc > gd.act_thr - kDetMargin) ||
                           (ph == kDetFall && !(vc < d.y - kDetMargin && vc > d.y - 0.5f * amp + kDetMargin));
            }
            // (a NaN dV/dt fails the first test; the foot test keeps a rising
            // voxel below the foot voltage on the plain step)
            elig = net_ok && fabsf(dv) <= sg.dvdt_max && !(vc < sg.foot_v && dv > sg.foot_dvdt) &&
                   !stim_ahead(gd, ck, ctl, k, sg.nsub);
        }
        c.v = vc;
        if (use_net) {
            // features (the previous tile's MMAs have all completed)
            uint4 *row[kMlpIn / 8];
#pragma unroll
            for (int j = 0; j < kMlpIn / 8; ++j) row[j] = reinterpret_cast<uint4 *>(xh + tc::kmaj_off(t, j * 8, kMlpIn));
            if (elig) {
                float f[kMlpIn];
                state38(c, f);
                f[38] = sg.par[0];
                f[39] = sg.par[1];
                f[40] = sg.par[2];
                const int cls = sur_class(ct);
                f[41] = cls == 0;
                f[42] = cls == 1;
                f[43] = cls == 2;
#pragma unroll
                for (int j = 44; j < kMlpIn; ++j) f[j] = 0.f;
#pragma unroll
                for (int j = 0; j < kMlpIn / 8; ++j) {
                    uint32_t p[4];
#pragma unroll
                    for (int i = 0; i < 4; ++i) {
                        const int a = j * 8 + 2 * i;
                        const float4 q = *reinterpret_cast<const float4 *>(nrm + 2 * a);
                        __nv_bfloat162 h = __floats2bfloat162_rn(fmaf(f[a], q.x, q.y), fmaf(f[a + 1], q.z, q.w));
                        p[i] = *reinterpret_cast<uint32_t *>(&h);
                    }
                    *row[j] = make_uint4(p[0], p[1], p[2], p[3]);
                }
            } else {
#pragma unroll
                for (int j = 0; j < kMlpIn / 8; ++j) *row[j] = make_uint4(0, 0, 0, 0);
            }
            tc::fence_proxy_async();   // feature rows -> visible to tcgen05.mma
        }
        tc::fence_before();            // previous tile's tcgen05.ld before the barrier
        const int any = wg_or(bar_id, elig ? 1 : 0);
        const bool run_net = use_net && any && net_ok;
        if (run_net && t == 0) {
            tc::fence_after();
            gemm(t_acc_mma, xh, smem + kOffW1, kMlpIn, kMlpHid, smem + kOffOnes, smem + kOffB1, false);
            tc::mma_commit(bar);
        }
        // 2. coarse TPORd step of the macro length, overlapping layer 1
        if (elig) {
            StepOut<float> o;
            tpord_step<float>(c, ct, gd.model, sg.kmac, 0.f, 0.f, &o);
        }
        // 3. the rest of the network
        bool have_net = false;
        if (run_net) {
            for (int layer = 0; layer < 3; ++layer) {
                if (layer > 0 && t == 0) {
                    tc::fence_after();
                    if (layer == 1)
                        gemm(t_acc_mma, xh, smem + kOffW2, kMlpHid, kMlpHid, smem + kOffOnesH, smem + kOffB2, true);
                    else gemm(t_acc_mma, xh, smem + kOffW3, kMlpHid, kMlpOut, smem + kOffOnesH, smem + kOffB3, true);
                    tc::mma_commit(bar);
                }
                // every thread of the group takes the same branch: a wait that
                // ran out anywhere ends the network for this kernel
                const bool w_ok = tc::mbar_wait(bar, phase, kWaitLimit);
                if (!wg_and(bar_id, w_ok ? 1 : 0)) {
                    if (!w_ok) tc::mbar_wait(bar, phase, kWaitLimit);
                    if (t == 0) atomicExch(sg.err, 1);
                    net_ok = false;
                    break;
                }
                phase ^= 1;
                tc::fence_after();
                if (layer == 2) break;
                // hidden layer: TMEM -> SiLU -> FP16 operand (over the feature
                // tile, which the finished MMA no longer needs)
#pragma unroll 1
                for (int cc = 0; cc < kMlpHid; cc += 32) {
                    float v[32];
                    tmem_ld32(t_acc + cc, v);
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        uint32_t packed[4];
#pragma unroll
                        for (int i = 0; i < 4; ++i) packed[i] = silu2_f16(v[q * 8 + 2 * i], v[q * 8 + 2 * i + 1]);
                        *reinterpret_cast<uint4 *>(xh + tc::kmaj_off(t, cc + q * 8, kMlpHid)) =
                            make_uint4(packed[0], packed[1], packed[2], packed[3]);
                    }
                }
                tc::fence_before();
                tc::fence_proxy_async();
                wg_sync(bar_id);
            }
            have_net = net_ok;
        }
        // 4. the correction
        bool ok = elig && (net_ok || !use_net);
        uint32_t why = 0;   // failed checks: 1 network bound, 2 gate range, 4 concentration, 8 ionic V step
        if (have_net) {
            float2 *cp[8];
            float *gp[29];
            conc_ptrs(c, cp);
            gate_ptrs(c, gp);
            const float *osc = nrm + 2 * kMlpIn;
            const float *kbd = nrm + 3 * kMlpIn;     // kappa * bound
#pragma unroll
            for (int cc = 0; cc < 48; cc += 16) {
                float v[16];
                tc::tmem_ld16(t_acc + cc, v);    // whole warp, eligible or not
                if (elig) {
#pragma unroll
                    for (int i = 0; i < 16; ++i) {
                        const int j = cc + i;
                        if (j < kMlpNState) {
                            const float z = v[i];
                            if (!(fabsf(z) <= kbd[j])) why |= 1u;
                            const float d = z * osc[j];
                            if (j == 0) c.v += d;
                            else if (j < 9) cadd(*cp[j - 1], d);
                            else *gp[j - 9] += d;
                        }
                    }
                }
            }
        }
        if (elig) {
            float2 *cp[8];
            float *gp[29];
            conc_ptrs(c, cp);
            gate_ptrs(c, gp);
#pragma unroll
            for (int j = 0; j < kSurNProb; ++j) {
                const float x = *gp[j];
                if (!(x >= -1e-3f && x <= 1.001f)) why |= 2u;
                *gp[j] = fminf(fmaxf(x, 0.f), 1.f);
            }
#pragma unroll
            for (int j = kSurNProb; j < 29; ++j)
                if (!(*gp[j] == *gp[j])) why |= 2u;
#pragma unroll
            for (int j = 0; j < 8; ++j)
                if (!(cp[j]->x > 0.f)) why |= 4u;
            const float dvm = c.v - vc;
            if (!(fabsf(dvm) <= sg.vstep_max)) why |= 8u;    // NaN fails as well
            ok = ok && why == 0;
            if (ok) {
                store_cell(c, gd.s, k);
                sg.rate[k] = dvm * inv_mac;
                sg.dflag[k] = need_det ? 1 : 0;
            }
        }
        const bool plain = k < nt && !ok;
        if (plain) sg.rate[k] = __int_as_float(0x7fc00000);
        // append the plain voxels to the list (one atomic per warp)
        const unsigned mp = __ballot_sync(0xffffffffu, plain);
        if (mp) {
            unsigned long long base = 0;
            if (lane == 0) base = atomicAdd(sg.plist_n, (unsigned long long)__popc(mp));
            base = __shfl_sync(0xffffffffu, base, 0);
            if (plain) sg.plist[base + __popc(mp & ((1u << lane) - 1u))] = (int32_t)k;
        }
        // offered voxels that failed each check (one atomic per warp and reason)
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const unsigned mr = __ballot_sync(0xffffffffu, elig && ((why >> r) & 1u));
            if (lane == 0 && mr) atomicAdd(sg.stats + 2 + r, (unsigned long long)__popc(mr));
        }
        const unsigned mo = __ballot_sync(0xffffffffu, elig), ma = __ballot_sync(0xffffffffu, ok);
        if (lane == 0) {
            n_offer += __popc(mo);
            n_acc += __popc(ma);
        }
    }
    if (lane == 0 && (n_offer | n_acc)) {
        atomicAdd(sg.stats + 0, n_offer);
        atomicAdd(sg.stats + 1, n_acc);
    }
    tc::fence_before();
    __syncthreads();
    if (use_net && warp == 0) tc::tmem_dealloc(tmem, kTmemCols);
}

uint32_t sur_grid_smem_bytes() { return kSmemBytes; }

cudaError_t launch_sur_grid(const GridDev<float> &gd, const SurGrid &sg, int cur, int dim, cudaStream_t st)
{
    if (gd.ntissue <= 0) return cudaSuccess;
    static std::atomic<uint64_t> attr_done{0};
    cudaError_t e = tc::smem_attr_once(k_sur_grid, kSmemBytes, attr_done);
    if (e != cudaSuccess) return e;
    int dev = 0, nsm = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int64_t ntiles = (gd.ntissue + kTile - 1) / kTile;
    // one CTA per SM: its 512 TMEM columns are the SM's whole TMEM, and the
    // shared memory admits one CTA, so tcgen05.alloc never waits
    int64_t grid = (ntiles + kGroups - 1) / kGroups;
    if (grid > nsm) grid = nsm;
    k_sur_grid<<<(unsigned)grid, kThreads, kSmemBytes, st>>>(gd, sg, cur, dim);
    return cudaGetLastError();
}

}  // namespace lqt
