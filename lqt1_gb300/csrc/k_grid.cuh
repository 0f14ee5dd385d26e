// k_grid.cuh -- fused diffusion + stimulus + TPORd step on 1D/2D/3D grids.
//
// Replaces the reference's per-step kernel chain calc_du -> init_Istim ->
// set_Istim -> Itot -> new_u_v (GPU3D.cu:370-425,1222-1230; new_11.cu:352-455,
// 1241-1255) with one kernel per step plus a small ghost-fill kernel.
//
// Layout: V lives in a dense grid (x-major, z fastest, as GPU3D.cu:29-33),
// double-buffered; the other 39 states live in structure-of-arrays order over
// the tissue voxels (common.cuh).  One thread per tissue voxel: it reads its V
// stencil from the dense grid (neighbour rows are shared through L1/L2), its
// state with streaming loads, and writes V into the other grid.  Empty voxels
// next to tissue hold the V of their mirror source (GPU3D.cu:1487-1604),
// refreshed after every step by k_ghost, so the stencil needs no branches.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"
#include "grid_dev.h"

namespace lqt {

// du = sum_i D_ii V_ii + 2 sum_{i<j} D_ij V_ij + sum_j b_j V_j
// (new_11.cu:352-417 in 2D; 7-point D*lap(V) when isotropic, GPU3D.cu:370-385).
template <typename R, int DIM>
__device__ __forceinline__ R grid_du(const GridDev<R> &gd, const R *__restrict__ V, int64_t g, int64_t k, R vc)
{
    if constexpr (DIM == 1) {
        // OneD.cc:371-391: mirrored ends, dD/dx term
        const int64_t n = gd.ntissue;
        R fo, so;
        if (n == 1) return (R)0;
        if (g == 0) {
            const R vp = V[g + 1];
            fo = (vp - vc) * gd.inv_dx;
            so = (vp + vc - (R)2 * vc) * gd.inv_dx2;
        } else if (g == n - 1) {
            const R vm = V[g - 1];
            fo = (vc - vm) * gd.inv_dx;
            so = (vc + vm - (R)2 * vc) * gd.inv_dx2;
        } else {
            const R vp = V[g + 1], vm = V[g - 1];
            fo = (vp - vm) * gd.inv_2dx;
            so = (vp + vm - (R)2 * vc) * gd.inv_dx2;
        }
        return (R)gd.dcoeff[k] * fo + (R)gd.coeff[k] * so;
    } else {
        const int64_t sx = gd.sx, sy = gd.sy;
        const R vxp = V[g + sx], vxm = V[g - sx], vyp = V[g + sy], vym = V[g - sy];
        const R c2 = gd.inv_dx2;
        const R lxx = (vxp + vxm - (R)2 * vc) * c2;
        const R lyy = (vyp + vym - (R)2 * vc) * c2;
        R lzz = 0, vzp = 0, vzm = 0;
        if constexpr (DIM == 3) {
            vzp = V[g + 1];
            vzm = V[g - 1];
            lzz = (vzp + vzm - (R)2 * vc) * c2;
        }
        if (!gd.d6) return gd.diso * (lxx + lyy + lzz);
        const R *D = gd.d6 + 6 * k;
        const R *B = gd.b3 + 3 * k;
        const R c4 = gd.inv_4dx2, c1 = gd.inv_2dx;
        const R lxy = (V[g + sx + sy] + V[g - sx - sy] - V[g - sx + sy] - V[g + sx - sy]) * c4;
        R du = D[0] * lxx + D[1] * lyy + (R)2 * D[3] * lxy + B[0] * ((vxp - vxm) * c1) + B[1] * ((vyp - vym) * c1);
        if constexpr (DIM == 3) {
            const R lxz = (V[g + sx + 1] + V[g - sx - 1] - V[g - sx + 1] - V[g + sx - 1]) * c4;
            const R lyz = (V[g + sy + 1] + V[g - sy - 1] - V[g - sy + 1] - V[g + sy - 1]) * c4;
            du += D[2] * lzz + (R)2 * (D[4] * lxz + D[5] * lyz) + B[2] * ((vzp - vzm) * c1);
        }
        return du;
    }
}

// AP detector update of voxel k (record d) for one step from vc to vn.
template <typename R>
__device__ __forceinline__ void grid_detect_rec(const GridDev<R> &gd, const Clock &ck, int64_t k, float4 d, float vc,
                                                float vn, float dvdt)
{
    DetState ds;
    ds.vrest = d.x;
    ds.vpeak = d.y;
    uint32_t bits = __float_as_uint(d.w);
    ds.phase = bits & 7u;
    ds.ead = (bits >> 3) & 1u;
    ds.dvdt_max = 0.f;
    float t_act = d.z;
    bool dirty = false;
    if (ck.opened) {
        det_open_cycle(ds, vc);
        dirty = true;
    }
    if (ds.phase != kDetIdle && ds.phase != kDetDone) {
        DetEvent ev;
        const uint8_t ph0 = ds.phase;
        const float vp0 = ds.vpeak;
        const uint8_t e0 = ds.ead;
        if (det_step(ds, vc, vn, dvdt, ck.time_f, gd.act_thr, t_act, ev, true)) {
            if (ev.t_90 >= 0.f) gd.apd90[k] = ev.apd90;
        }
        dirty |= ds.phase != ph0 || ds.vpeak != vp0 || ds.ead != e0;
    }
    if (dirty) {
        const uint32_t nb = (bits >> 4) + (ck.opened ? 1u : 0u);
        gd.det[k] = make_float4(ds.vrest, ds.vpeak, t_act, __uint_as_float((nb << 4) | (ds.ead << 3) | ds.phase));
    }
}

template <typename R>
__device__ __forceinline__ void grid_detect(const GridDev<R> &gd, const Clock &ck, int64_t k, float vc, float vn,
                                            float dvdt)
{
    grid_detect_rec(gd, ck, k, gd.det[k], vc, vn, dvdt);
}

// Is the S1 stimulus of a voxel with this onset on at within-cycle time tb?
// Per-voxel onset within each cycle, compared in FP64 as GPU3D.cu:397-409
// does.  Out of line on purpose: inlined, the compiler evaluates these FP64
// operations under a predicate for every voxel of the kernels that never use
// onsets, and GB300's FP64 pipe is slow enough for five of them per warp to
// keep it half busy in the V-only substep.
static __device__ __noinline__ bool onset_s1_on(double tb, double s1_start, double s1_dur, float onset)
{
    const double on = s1_start + (double)onset;
    return tb >= on && tb < on + s1_dur;
}

// Stimulus current of voxel k at the clock's step.
template <typename R>
__device__ __forceinline__ R grid_stim(const GridDev<R> &gd, const Clock &ck, uint8_t ctl, int64_t k)
{
    R ist = 0;
    if (gd.onset) {
        if ((ctl & kCtlS1) && ck.s1_cycle_ok && onset_s1_on(ck.tb, gd.s1_start, gd.s1_dur, gd.onset[k]))
            ist = gd.s1_strength;
    } else if (ck.s1_on && (ctl & kCtlS1)) {
        ist = gd.s1_strength;
    }
    if (ck.s2_on && (ctl & kCtlS2)) ist = gd.s2_strength;
    return ist;
}

template <typename R> __device__ __forceinline__ void grid_count_bad(const GridDev<R> &gd, R vn)
{
    const bool bad = !(vn == vn) || vn < gd.vmin_ok || vn > gd.vmax_ok;
    const unsigned m = __ballot_sync(__activemask(), bad);
    if (m && (threadIdx.x & 31) == __ffs(m) - 1) atomicAdd(gd.nbad, (unsigned long long)__popc(m));
}

// One plain step of tissue voxel k: diffusion, stimulus, the TPORd update,
// the new V, the detector and the blow-up count.
template <typename R, int DIM>
__device__ __forceinline__ void grid_step_voxel(const GridDev<R> &gd, const StepT<R> &kst, int cur, int64_t k,
                                                const Clock &ck)
{
    const R *__restrict__ V = gd.vg[cur];
    R *__restrict__ Vn = gd.vg[cur ^ 1];
    const int64_t g = DIM == 1 ? k : (int64_t)gd.gidx[k];
    const R vc = V[g];
    const R du = grid_du<R, DIM>(gd, V, g, k, vc);
    const uint8_t ctl = gd.ctl[k];
    const R ist = grid_stim(gd, ck, ctl, k);

    CellState<R> c;
    load_cell(c, gd.s, k);
    c.v = vc;
    StepOut<R> o{};
    tpord_step<R>(c, ctl & kCtlType, gd.model, kst, ist, du, &o);
    store_cell(c, gd.s, k);
    Vn[g] = c.v;
    if (gd.det) grid_detect(gd, ck, k, (float)vc, (float)c.v, (float)o.dvdt);
    grid_count_bad(gd, c.v);
}

// The same step as a called function: the list kernel's loop keeps only its
// own index live across voxels instead of constants hoisted out of the step.
template <typename R, int DIM>
__device__ __noinline__ void grid_step_voxel_call(const GridDev<R> &gd, const StepT<R> &kst, int cur, int64_t k,
                                                  const Clock &ck)
{
    grid_step_voxel<R, DIM>(gd, kst, cur, k, ck);
}

// MINB = minimum resident CTAs per SM the register allocation must allow
// (occupancy variants picked at run time by the autotuner in api_sim.cu; they
// differ only in register allocation, not in arithmetic).  One thread per
// tissue voxel.
template <typename R, int DIM, int MINB>
__global__ void __launch_bounds__(256, MINB) k_grid_step(GridDev<R> gd, StepT<R> kst, int cur)
{
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= gd.ntissue) return;
    grid_step_voxel<R, DIM>(gd, kst, cur, k, *gd.clk);
}

// With the learned surrogate attached: the plain step of the voxels listed in
// plist (plist_n of them, written by the macro-step kernel), grid-stride over
// a launch of a few waves of CTAs, so that a short list costs its own voxels
// and not a pass over every tissue voxel.  The step is a called function at 2
// CTAs/SM (128 registers): inlined into the loop, constants hoisted out of
// the step stay live across voxels and spill.
template <typename R, int DIM>
__global__ void __launch_bounds__(256, 2) k_grid_step_list(GridDev<R> gd, StepT<R> kst, int cur)
{
    const int64_t n = *gd.plist_n;
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Clock ck = *gd.clk;
    for (; i < n; i += (int64_t)gridDim.x * blockDim.x) grid_step_voxel_call<R, DIM>(gd, kst, cur, gd.plist[i], ck);
}

// CTAs of a list-step launch: four waves at 2 CTAs/SM, never more than one
// thread per tissue voxel.
inline unsigned grid_list_blocks(int64_t ntissue)
{
    int dev = 0, nsm = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int64_t full = (ntissue + 255) / 256;
    const int64_t cap = (int64_t)nsm * 2 * 4;
    return (unsigned)(full < cap ? (full < 1 ? 1 : full) : cap);
}

// Inside a surrogate macro step: the voxels whose ionic change is fixed
// (srate not NaN) move V by it plus diffusion, in the update form of
// TPORd.cc:928-930; the others are left to k_grid_step over plist.  A thread
// takes kSubU voxels (k and k + blockDim.x ...), and every load that depends
// only on k (rate, grid index, control and detector flags, diffusion tensor)
// is issued before the first use, so the loads of both voxels overlap in two
// memory round trips (those, then the V stencils).  The detector record is
// read only where the macro-step kernel flagged that it can change.
constexpr int kSubU = 2;

// The surrogate substep's tensor row in FP16 (3 half2 per voxel: g_x g_y |
// g_z b_x | b_y b_z, see GridDev::t3h): streaming loads, widened to FP32.
__device__ __forceinline__ void sub_tensor_f16(const __half2 *t, float2 (&q)[3])
{
#pragma unroll
    for (int i = 0; i < 3; ++i) q[i] = __half22float2(__ldcs(t + i));
}

// The tensor (xx yy zz xy xz yz) and its divergence from a row:
// D = dtr I + dsg g g^T.
template <int DIM>
__device__ __forceinline__ void sub_tensor_unpack(const float2 (&q)[3], float dtr, float dsg, float *Dt, float *Bt)
{
    const float g0 = q[0].x, g1 = q[0].y, g2 = DIM == 3 ? q[1].x : 0.f;
    const float s0 = dsg * g0, s1 = dsg * g1, s2 = dsg * g2;
    Dt[0] = fmaf(s0, g0, dtr);
    Dt[1] = fmaf(s1, g1, dtr);
    Dt[2] = fmaf(s2, g2, dtr);
    Dt[3] = s0 * g1;
    Dt[4] = s0 * g2;
    Dt[5] = s1 * g2;
    Bt[0] = q[1].y;
    Bt[1] = q[2].x;
    Bt[2] = DIM == 3 ? q[2].y : 0.f;
}

// The anisotropic stencil of grid_du with the tensor already loaded, on any
// x-major array of V with strides sx, sy (z stride 1): the dense grid, or a
// tile's box of it staged in shared memory (the same values in the same
// order of operations, so the same bits).
template <int DIM>
__device__ __forceinline__ float sub_du_at(const GridDev<float> &gd, const float *__restrict__ V, int64_t g,
                                           int64_t sx, int64_t sy, float vc, const float *Dt, const float *Bt)
{
    const float vxp = V[g + sx], vxm = V[g - sx], vyp = V[g + sy], vym = V[g - sy];
    const float c2 = gd.inv_dx2, c4 = gd.inv_4dx2, c1 = gd.inv_2dx;
    const float lxx = (vxp + vxm - 2.f * vc) * c2;
    const float lyy = (vyp + vym - 2.f * vc) * c2;
    const float lxy = (V[g + sx + sy] + V[g - sx - sy] - V[g - sx + sy] - V[g + sx - sy]) * c4;
    float du = Dt[0] * lxx + Dt[1] * lyy + 2.f * Dt[3] * lxy + Bt[0] * ((vxp - vxm) * c1) + Bt[1] * ((vyp - vym) * c1);
    if constexpr (DIM == 3) {
        const float vzp = V[g + 1], vzm = V[g - 1];
        const float lzz = (vzp + vzm - 2.f * vc) * c2;
        const float lxz = (V[g + sx + 1] + V[g - sx - 1] - V[g - sx + 1] - V[g + sx - 1]) * c4;
        const float lyz = (V[g + sy + 1] + V[g - sy - 1] - V[g - sy + 1] - V[g + sy - 1]) * c4;
        du += Dt[2] * lzz + 2.f * (Dt[4] * lxz + Dt[5] * lyz) + Bt[2] * ((vzp - vzm) * c1);
    }
    return du;
}

template <int DIM>
__device__ __forceinline__ float sub_du(const GridDev<float> &gd, const float *__restrict__ V, int64_t g, int64_t k,
                                        float vc, const float *Dt, const float *Bt)
{
    if (DIM == 1 || !gd.d6) return grid_du<float, DIM>(gd, V, g, k, vc);
    return sub_du_at<DIM>(gd, V, g, gd.sx, gd.sy, vc, Dt, Bt);
}

// MINB: minimum resident CTAs per SM (occupancy variants, picked at run time
// by the autotuner; 5 / 6 / 8 CTAs of 256 threads = 48 / 40 / 32 registers).
template <int DIM, int MINB>
__global__ void __launch_bounds__(256, MINB) k_sur_substep(GridDev<float> gd, float dt, int cur)
{
    const int64_t k0 = blockIdx.x * (int64_t)(blockDim.x * kSubU) + threadIdx.x;
    const bool aniso = DIM > 1 && gd.d6 && gd.t3h;
    float r[kSubU], Dt[kSubU][6], Bt[kSubU][3];
    int64_t g[kSubU];
    uint8_t ctl[kSubU], fl[kSubU];
    bool on[kSubU];
#pragma unroll
    for (int u = 0; u < kSubU; ++u) {
        const int64_t k = k0 + u * (int64_t)blockDim.x;
        on[u] = k < gd.ntissue;
        r[u] = on[u] ? gd.srate[k] : __int_as_float(0x7fc00000);
        g[u] = on[u] ? (DIM == 1 ? k : (int64_t)gd.gidx[k]) : 0;
        ctl[u] = on[u] ? gd.ctl[k] : 0;
        fl[u] = on[u] && gd.det ? gd.sdflag[k] : 0;
#pragma unroll
        for (int i = 0; i < 6; ++i) Dt[u][i] = 0.f;
#pragma unroll
        for (int i = 0; i < 3; ++i) Bt[u][i] = 0.f;
        if (aniso && on[u]) {
            // the FP16 copies, streamed once per step: evict-first, the L2 is
            // for the V rows
            float2 q[3];
            sub_tensor_f16(gd.t3h + 3 * k, q);
            sub_tensor_unpack<DIM>(q, gd.sub_dtr, gd.sub_dsg, Dt[u], Bt[u]);
        }
    }
    bool any = false;
#pragma unroll
    for (int u = 0; u < kSubU; ++u) {
        on[u] = on[u] && r[u] == r[u];
        any |= on[u];
    }
    if (!any) return;
    const Clock ck = *gd.clk;
    const float *__restrict__ V = gd.vg[cur];
    float *__restrict__ Vn = gd.vg[cur ^ 1];
#pragma unroll
    for (int u = 0; u < kSubU; ++u) {
        if (!on[u]) continue;
        const int64_t k = k0 + u * (int64_t)blockDim.x;
        const float vc = V[g[u]];
        const float du = sub_du<DIM>(gd, V, g[u], k, vc, Dt[u], Bt[u]);
        const float ist = grid_stim(gd, ck, ctl[u], k);
        const float dvdt = r[u] - ist;
        const float vn = vc + (dvdt + du) * dt;
        Vn[g[u]] = vn;
        if (fl[u]) grid_detect(gd, ck, k, vc, vn, dvdt);
        const bool bad = !(vn == vn) || vn < gd.vmin_ok || vn > gd.vmax_ok;
        if (bad) atomicAdd(gd.nbad, 1ull);
    }
}

// Mirror-boundary refresh of the new grid, then the clock advance for the
// next step (block 0, thread 0).
template <typename R>
__global__ void __launch_bounds__(256) k_ghost(GridDev<R> gd, int nxt)
{
    R *V = gd.vg[nxt];
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < gd.nbnd; j += (int64_t)gridDim.x * blockDim.x)
        V[gd.bnd_dst[j]] = V[gd.bnd_src[j]];
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        Clock ck = *gd.clk;
        ck.step += 1;
        ck.time += gd.dt;
        ck.time_f = (float)ck.time;
        int32_t w = ck.widx < 0 ? 0 : ck.widx;
        const int32_t nwin = gd.win ? gd.nwin : 0;
        while (w < nwin && ck.step >= gd.win[w].off) ++w;
        ck.widx = w;
        ck.s1_on = w < nwin && ck.step >= gd.win[w].on;
        ck.opened = w < nwin && ck.step == gd.win[w].on;
        ck.s2_on = ck.step >= gd.s2_win.on && ck.step < gd.s2_win.off;
        if (gd.onset) {
            ck.tb = ck.time - floor(ck.time / gd.bcl) * gd.bcl;
            ck.s1_cycle_ok = gd.s1_beats <= 0 || floor(ck.time / gd.bcl) < gd.s1_beats;
        }
        *gd.clk = ck;
    }
}

// Compensated FP32 sum (hi, lo) += x: TwoSum of hi and x, error folded into lo.
__device__ __forceinline__ void kahan2_add(float &hi, float &lo, float x)
{
    const float s = __fadd_rn(hi, x);
    const float bb = __fsub_rn(s, hi);
    const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(x, bb));
    hi = s;
    lo = __fadd_rn(lo, e);
}

// Pseudo-ECG partial sums: 3D form of PlotScript/plot1DECG_compare.py:89-105,
// phi(r0) = sum_i sum_axis (V[i+e] - V[i-e])/2 (r_i - r0)_axis / |r_i - r0|^3.
// Warps sum their 32 FP32 terms as compensated FP32 pairs (a fixed shuffle
// tree; FP64 arithmetic runs at a small fraction of the FP32 rate on this
// GPU), the block's warp sums are added in FP64, and k_ecg_final adds the
// per-block partials in a fixed order, so the result does not depend on
// scheduling.
template <typename R, int DIM>
__global__ void __launch_bounds__(256) k_ecg_partial(GridDev<R> gd, const R *__restrict__ V,
                                                     const float4 *__restrict__ el, int nel,
                                                     double *__restrict__ partial)
{
    __shared__ float2 red[8][kMaxElectrodes];
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    float acc[kMaxElectrodes];
#pragma unroll
    for (int e = 0; e < kMaxElectrodes; ++e) acc[e] = 0.f;
    if (k < gd.ntissue) {
        const int64_t g = DIM == 1 ? k : (int64_t)gd.gidx[k];
        float p[3] = {0.f, 0.f, 0.f}, h[3] = {0.f, 0.f, 0.f};
        if constexpr (DIM == 1) {
            p[0] = (float)(k * gd.dx);
            const int64_t n = gd.ntissue;
            if (n > 1) h[0] = k == 0 ? (float)(V[1] - V[0]) : (k == n - 1 ? (float)(V[k] - V[k - 1]) : 0.5f * (float)(V[k + 1] - V[k - 1]));
        } else {
            // grids are below 2^31 voxels: 32-bit index arithmetic
            const int32_t g32 = (int32_t)g, sx32 = (int32_t)gd.sx, sy32 = (int32_t)gd.sy;
            const int32_t x = g32 / sx32, rem = g32 - x * sx32;
            const int32_t y = rem / sy32, z = rem - y * sy32;
            // coordinates from the host's table (no FP64 arithmetic per voxel:
            // GB300's FP64 pipe would set this kernel's pace); the grid's
            // origin offset is 0
            p[0] = gd.xpos[x];
            p[1] = gd.xpos[y];
            p[2] = DIM == 3 ? gd.xpos[z] : 0.f;
            h[0] = 0.5f * (float)(V[g + gd.sx] - V[g - gd.sx]);
            h[1] = 0.5f * (float)(V[g + gd.sy] - V[g - gd.sy]);
            if constexpr (DIM == 3) h[2] = 0.5f * (float)(V[g + 1] - V[g - 1]);
        }
#pragma unroll
        for (int e = 0; e < kMaxElectrodes; ++e) {
            if (e < nel) {
                const float rx = p[0] - el[e].x, ry = p[1] - el[e].y, rz = p[2] - el[e].z;
                const float r2 = rx * rx + ry * ry + rz * rz;
                const float inv = rsqrtf(r2);
                acc[e] = (h[0] * rx + h[1] * ry + h[2] * rz) * (inv * inv * inv);
            }
        }
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int e = 0; e < kMaxElectrodes; ++e) {
        if (e >= nel) break;
        float hi = acc[e], lo = 0.f;
        for (int o = 16; o > 0; o >>= 1) {
            const float oh = __shfl_down_sync(0xffffffffu, hi, o);
            const float ol = __shfl_down_sync(0xffffffffu, lo, o);
            kahan2_add(hi, lo, oh);
            lo = __fadd_rn(lo, ol);
        }
        if (lane == 0) red[wid][e] = make_float2(hi, lo);
    }
    __syncthreads();
    // the block's warps, still as compensated FP32 pairs: one FP64 sum per
    // electrode and block (a per-warp FP64 sum kept GB300's FP64 pipe busy
    // for most of this kernel's time)
    if (threadIdx.x < nel) {
        float hi = 0.f, lo = 0.f;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            const float2 v = red[w][threadIdx.x];
            kahan2_add(hi, lo, v.x);
            lo = __fadd_rn(lo, v.y);
        }
        partial[(int64_t)blockIdx.x * nel + threadIdx.x] = (double)hi + (double)lo;
    }
}

__global__ void k_ecg_final(const double *__restrict__ partial, int64_t nblocks, int nel, double *__restrict__ out,
                            double *__restrict__ t_out, int64_t *__restrict__ counter, int64_t cap,
                            const Clock *__restrict__ clk);

}  // namespace lqt
