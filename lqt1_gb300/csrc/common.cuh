// common.cuh -- device data layout shared by the kernels.
//
// State layout in HBM (structure of arrays, leading dimension ld, padded to a
// multiple of 128 cells so every array starts 512-byte aligned):
//   v      R     [ld]        membrane potential (cells and strands; grids keep
//                            V in a dense double-buffered grid instead)
//   conc   double[8][ld]     nai nass ki kss cai cass cansr cajsr (FP64 form);
//          float[16][ld]     the mixed form's Kahan pairs in the same bytes:
//                            hi parts [0..8), lo parts [8..16)
//   gate   R     [31][ld]    reference state indices 9..39 (sm .. CaMKt);
//                            slots 3, 4 (hsp, jp) are constant and not touched
// R = double for the FP64 form, float for the mixed form.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "lqt_internal.h"
#include "tpord.cuh"

namespace lqt {

// Streaming loads/stores for state read and written once per step: they keep
// the 129 MB L2 for data that is reused (the V grid, neighbour rows).
template <typename T> __device__ __forceinline__ T ld_stream(const T *p) { return __ldcs(p); }
template <typename T> __device__ __forceinline__ void st_stream(T *p, T v) { __stcs(p, v); }

__device__ __forceinline__ void load_conc(double *dst[8], const double *conc, int64_t ld, int64_t i)
{
#pragma unroll
    for (int j = 0; j < 8; ++j) *dst[j] = ld_stream(conc + j * ld + i);
}
__device__ __forceinline__ void load_conc(float2 *dst[8], const double *conc, int64_t ld, int64_t i)
{
    const float *f = reinterpret_cast<const float *>(conc);
#pragma unroll
    for (int j = 0; j < 8; ++j) *dst[j] = make_float2(ld_stream(f + j * ld + i), ld_stream(f + (8 + j) * ld + i));
}
__device__ __forceinline__ void store_conc(double *const src[8], double *conc, int64_t ld, int64_t i)
{
#pragma unroll
    for (int j = 0; j < 8; ++j) st_stream(conc + j * ld + i, *src[j]);
}
__device__ __forceinline__ void store_conc(float2 *const src[8], double *conc, int64_t ld, int64_t i)
{
    float *f = reinterpret_cast<float *>(conc);
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        st_stream(f + j * ld + i, src[j]->x);
        st_stream(f + (8 + j) * ld + i, src[j]->y);
    }
}

template <typename R>
__device__ __forceinline__ void load_cell(CellState<R> &c, const SoA<R> &s, int64_t i)
{
    const int64_t ld = s.ld;
    const R *G = s.gate + i;
    typename CellState<R>::C *cp[8] = {&c.nai, &c.nass, &c.ki, &c.kss, &c.cai, &c.cass, &c.cansr, &c.cajsr};
    load_conc(cp, s.conc, ld, i);
    c.sm = ld_stream(G + 0 * ld); c.sh = ld_stream(G + 1 * ld); c.sj = ld_stream(G + 2 * ld);
    c.mL = ld_stream(G + 5 * ld); c.hL = ld_stream(G + 6 * ld); c.hLp = ld_stream(G + 7 * ld);
    c.a = ld_stream(G + 8 * ld); c.iF = ld_stream(G + 9 * ld); c.iS = ld_stream(G + 10 * ld);
    c.ap = ld_stream(G + 11 * ld); c.iFp = ld_stream(G + 12 * ld); c.iSp = ld_stream(G + 13 * ld);
    c.d = ld_stream(G + 14 * ld); c.ff = ld_stream(G + 15 * ld); c.fs = ld_stream(G + 16 * ld);
    c.fcaf = ld_stream(G + 17 * ld); c.fcas = ld_stream(G + 18 * ld); c.jca = ld_stream(G + 19 * ld);
    c.nca = ld_stream(G + 20 * ld); c.ffp = ld_stream(G + 21 * ld); c.fcafp = ld_stream(G + 22 * ld);
    c.xrf = ld_stream(G + 23 * ld); c.xrs = ld_stream(G + 24 * ld); c.xs1 = ld_stream(G + 25 * ld);
    c.xs2 = ld_stream(G + 26 * ld); c.xk1 = ld_stream(G + 27 * ld); c.Jrelnp = ld_stream(G + 28 * ld);
    c.Jrelp = ld_stream(G + 29 * ld); c.CaMKt = ld_stream(G + 30 * ld);
}

template <typename R>
__device__ __forceinline__ void store_cell(const CellState<R> &c, const SoA<R> &s, int64_t i)
{
    const int64_t ld = s.ld;
    R *G = s.gate + i;
    CellState<R> &cc = const_cast<CellState<R> &>(c);
    typename CellState<R>::C *cp[8] = {&cc.nai, &cc.nass, &cc.ki, &cc.kss, &cc.cai, &cc.cass, &cc.cansr, &cc.cajsr};
    store_conc(cp, s.conc, ld, i);
    st_stream(G + 0 * ld, c.sm); st_stream(G + 1 * ld, c.sh); st_stream(G + 2 * ld, c.sj);
    st_stream(G + 5 * ld, c.mL); st_stream(G + 6 * ld, c.hL); st_stream(G + 7 * ld, c.hLp);
    st_stream(G + 8 * ld, c.a); st_stream(G + 9 * ld, c.iF); st_stream(G + 10 * ld, c.iS);
    st_stream(G + 11 * ld, c.ap); st_stream(G + 12 * ld, c.iFp); st_stream(G + 13 * ld, c.iSp);
    st_stream(G + 14 * ld, c.d); st_stream(G + 15 * ld, c.ff); st_stream(G + 16 * ld, c.fs);
    st_stream(G + 17 * ld, c.fcaf); st_stream(G + 18 * ld, c.fcas); st_stream(G + 19 * ld, c.jca);
    st_stream(G + 20 * ld, c.nca); st_stream(G + 21 * ld, c.ffp); st_stream(G + 22 * ld, c.fcafp);
    st_stream(G + 23 * ld, c.xrf); st_stream(G + 24 * ld, c.xrs); st_stream(G + 25 * ld, c.xs1);
    st_stream(G + 26 * ld, c.xs2); st_stream(G + 27 * ld, c.xk1); st_stream(G + 28 * ld, c.Jrelnp);
    st_stream(G + 29 * ld, c.Jrelp); st_stream(G + 30 * ld, c.CaMKt);
}

// ---- per-cell AP detector -------------------------------------------------
// One cycle per stimulus window.  When the cycle's S1 window opens the cell
// records its resting V (the V before that step, as SingleCell.cc:148-157
// records rest_potential) and waits.  An upward crossing of the activation
// threshold (OneD.cc:422-428) starts the upstroke; the first step whose V is
// not above the previous V ends it (SingleCell.cc:160-198: overshoot = last
// rising V).  APD90 is the first step at or below
// overshoot - 0.9 * (overshoot - rest) (SingleCell.cc:195,211).  An EAD is a
// rise of V by more than 1e-3 mV in one step after V fell below the 50% level
// and before the 90% crossing.  Times are the step's pre-increment time, as
// the reference drivers print them.
enum : uint8_t { kDetIdle = 0, kDetWait = 1, kDetRise = 2, kDetFall = 3, kDetDone = 4 };

struct DetState {
    float vrest, vpeak, dvdt_max;
    uint8_t phase, ead;
};

struct DetEvent {       // what a step produced (-1 = nothing)
    float t_act, t_90, apd90, dvdt_max;
    int ead;
};

__device__ __forceinline__ void det_open_cycle(DetState &d, float v_old)
{
    d.vrest = v_old;
    d.vpeak = v_old;
    d.dvdt_max = 0.f;
    d.phase = kDetWait;
    d.ead = 0;
}

// Returns true when an event (activation or APD90) happened this step.
// peak_max: tissue grids keep the overshoot at the maximum V since activation
// (a wave collision can stall an upstroke for one step, where the single-cell
// rule "first non-rising step" would flip between the stall and the true peak
// on a perturbation of a few microvolts); single cells and strands keep the
// SingleCell.cc rule (peak_max = false).
__device__ __forceinline__ bool det_step(DetState &d, float v_old, float v_new, float dvdt, float time,
                                         float act_thr, float &t_act, DetEvent &ev, bool peak_max = false)
{
    bool evt = false;
    ev.t_act = -1.f;
    ev.t_90 = -1.f;
    switch (d.phase) {
    case kDetWait:
        if (v_old < act_thr && v_new >= act_thr) {
            d.phase = kDetRise;
            d.vpeak = v_new;
            d.dvdt_max = fabsf(dvdt);
            t_act = time;
            ev.t_act = time;
            evt = true;
        }
        break;
    case kDetRise:
        if (v_new > v_old) {
            d.vpeak = v_new;
            d.dvdt_max = fmaxf(d.dvdt_max, fabsf(dvdt));
        } else {
            d.vpeak = v_old;
            d.phase = kDetFall;
        }
        break;
    case kDetFall: {
        if (peak_max && v_new > d.vpeak) {
            d.vpeak = v_new;
            break;
        }
        const float amp = d.vpeak - d.vrest;
        const float thr90 = d.vpeak - 0.9f * amp;
        const float thr50 = d.vpeak - 0.5f * amp;
        if (v_new <= thr90 && v_old >= thr90) {
            d.phase = kDetDone;
            ev.t_90 = time;
            ev.apd90 = time - t_act;
            ev.dvdt_max = d.dvdt_max;
            ev.ead = d.ead;
            evt = true;
        } else if (v_old < thr50 && v_new > v_old + 1e-3f) {
            d.ead = 1;
        }
        break;
    }
    default:
        break;
    }
    return evt;
}

}  // namespace lqt
