// tpord.cuh -- device implementation of one TPORd step (the reference's
// TPORd::update(), SingleCell/TPORd.cc:379-1021; GPU copies GPU3D.cu:425-1220,
// new_11.cu:459-1239) for the sm_103a kernels.
//
// One source serves two arithmetic forms through a precision policy:
//   R = double : the plain FP64 form.  Divisions, exp and log follow the
//                reference expression by expression; integer powers are
//                multiplications and constant-tau decays are precomputed on
//                the host (same glibc values the reference computes).
//   R = float  : the mixed form.  Gates, currents and fluxes in FP32 with the
//                hardware exp2/log2/rcp approximations; the eight
//                concentrations are Kahan-compensated FP32 pairs (hi + lo,
//                about 48 significant bits, the same 8 bytes as FP64) and every
//                difference of two concentrations (Jdiff*, Jtr) is formed from
//                both parts, because at rest kss - ki is ~1e-5 mM against an
//                FP32 ulp of 1.5e-5 mM at 145 mM.  No FP64 instruction is left
//                on this path: GB300 issues FP64 at about 1/64 of the FP32 rate.
//                GHK terms use x/expm1(x), finite at V = 0.
//
// States hsp and jp are carried in the state vector but never change (their
// ORd INa is commented out in SingleCell/TPORd.cc:436-460), so the step does
// not touch them.
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

namespace lqt {

// Scenario parameters (from lqt_model, include/lqt.h).  PCa and GKs per cell
// class (0 endo, 1 epi, 2 mid) are computed on the host in the reference's
// order (TPORd.cc:622-639 and 692-733: base value, ISO1, type factor; LQT1,
// SUPREP, ISO1), so the FP64 form sees the same doubles.
template <typename R> struct ModelT {
    R pca[3];
    R gks[3];
    R dss_shift, fss_shift;          // ISO1 gate shifts (TPORd.cc:582,588)
};
using ModelK = ModelT<double>;

template <typename R> __host__ __device__ inline ModelT<R> model_as(const ModelK &m)
{
    ModelT<R> o;
    for (int i = 0; i < 3; ++i) {
        o.pca[i] = (R)m.pca[i];
        o.gks[i] = (R)m.gks[i];
    }
    o.dss_shift = m.dss_shift;
    o.fss_shift = m.fss_shift;
    return o;
}

// Per-step constants computed on the host with glibc, shared by all cells.
template <typename R> struct StepT {
    R dt;
    R e_hl, e_hlp, e_jca;            // exp(-dt/200), exp(-dt/600), exp(-dt/75) (TPORd.cc:517-521,605-606)
};
using StepK = StepT<double>;

template <typename R> __host__ __device__ inline StepT<R> step_as(const StepK &k)
{
    return StepT<R>{(R)k.dt, (R)k.e_hl, (R)k.e_hlp, (R)k.e_jca};
}

// ---- concentration storage -------------------------------------------------
// FP64 form: double.  Mixed form: float2 {hi, lo} with hi + lo the value.
template <typename R> struct ConcOf { using T = double; };
template <> struct ConcOf<float> { using T = float2; };

__device__ __forceinline__ double cval(double c) { return c; }
__device__ __forceinline__ float cval(float2 c) { return c.x; }
__device__ __forceinline__ double cdiff(double a, double b) { return a - b; }
__device__ __forceinline__ float cdiff(float2 a, float2 b) { return __fadd_rn(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y)); }
__device__ __forceinline__ void cadd(double &c, double inc) { c += inc; }
// c += inc as a compensated sum (TwoSum of hi and inc, error folded into lo,
// renormalised); the _rn intrinsics keep the compiler from contracting it.
__device__ __forceinline__ void cadd(float2 &c, float inc)
{
    const float s = __fadd_rn(c.x, inc);
    const float bb = __fsub_rn(s, c.x);
    const float e = __fadd_rn(__fsub_rn(c.x, __fsub_rn(s, bb)), __fsub_rn(inc, bb));
    const float l = __fadd_rn(c.y, e);
    const float h = __fadd_rn(s, l);
    c.y = __fsub_rn(l, __fsub_rn(h, s));
    c.x = h;
}

// ---- math policy ----------------------------------------------------------
template <typename R> struct Mth;

template <> struct Mth<double> {
    static __device__ __forceinline__ double ex(double x) { return exp(x); }
    static __device__ __forceinline__ double lg(double x) { return log(x); }
    static __device__ __forceinline__ double pw(double x, double y) { return pow(x, y); }
    static __device__ __forceinline__ double dv(double a, double b) { return a / b; }
    // divide by a literal: kept a true division in FP64 (reference rounding)
    static __device__ __forceinline__ double dk(double a, double k) { return a / k; }
    // GHK factor vffrt*(A e^z - B)/(e^z - 1) written as in TPORd.cc:618-620
    static __device__ __forceinline__ double ghk(double vffrt, double ez, double A, double B) {
        return vffrt * (A * ez - B) / (ez - 1.0);
    }
};

template <> struct Mth<float> {
    static __device__ __forceinline__ float ex(float x) { return __expf(x); }
    static __device__ __forceinline__ float lg(float x) { return __logf(x); }
    static __device__ __forceinline__ float pw(float x, float y) { return __powf(x, y); }
    static __device__ __forceinline__ float dv(float a, float b) { return __fdividef(a, b); }
    static __device__ __forceinline__ float dk(float a, double k) { return a * (float)(1.0 / k); }
};

// x / (e^x - 1), finite and accurate near x = 0 (FP32 form only).
__device__ __forceinline__ float x_over_expm1(float x, float em1)
{
    return fabsf(x) < 1e-4f ? 1.0f - 0.5f * x : __fdividef(x, em1);
}

// ---- cell state in registers ---------------------------------------------
template <typename R> struct CellState {
    using C = typename ConcOf<R>::T;
    R v;
    C nai, nass, ki, kss, cai, cass, cansr, cajsr;
    R sm, sh, sj, mL, hL, hLp, a, iF, iS, ap, iFp, iSp, d, ff, fs;
    R fcaf, fcas, jca, nca, ffp, fcafp, xrf, xrs, xs1, xs2, xk1;
    R Jrelnp, Jrelp, CaMKt;
};

template <typename R> struct StepOut {
    R dvdt;        // -(Iion + Ist) (TPORd.cc:928)
    R ical, iks;   // ICaL and IKs of the step (TPORd::getICaL / getIKs, SingleCell.cc:134-135)
    R ina, ikr, ik1;   // INa, IKr, IK1 of the step (TPORd::getINa / getIKr / getIK1, TPORd.cc:365-370)
};

// One TPORd update.  ctype: 2 = EPI, 4 = MCELL, other = endocardial
// (SingleCell/Cell.cc:20; only EPI and MCELL change parameters).
template <typename R>
__device__ __forceinline__ void tpord_step(CellState<R> &c, int ctype, const ModelT<R> &m, const StepT<R> &k,
                                           R Ist, R dVgap_dt, StepOut<R> *out)
{
    using M = Mth<R>;
    const bool epi = (ctype == 2);
    const bool mid = (ctype == 4);
    const R dt = k.dt;
    const R v = c.v;

    // constants, TPORd.cc:382-421
    constexpr double nao = 140.0, cao = 1.8, ko = 5.4;
    constexpr double R_ = 8314.0, T_ = 310.0, F_ = 96485.0;
    constexpr double KmCaMK = 0.15, KmCaM = 0.0015, CaMKo = 0.05;
    constexpr double L_ = 0.01, rad = 0.0011;
    constexpr double vcell = 1000 * 3.14 * rad * rad * L_;
    constexpr double Ageo = 2 * 3.14 * rad * rad + 2 * 3.14 * rad * L_;
    constexpr double Acap = 2 * Ageo;
    constexpr double vmyo = 0.68 * vcell, vnsr = 0.0552 * vcell, vjsr = 0.0048 * vcell, vss = 0.02 * vcell;
    constexpr double RTF = R_ * T_ / F_;
    constexpr double FFRT = F_ * F_ / (R_ * T_);
    constexpr double FRT = F_ / (R_ * T_);

    const R nai = cval(c.nai), nass = cval(c.nass), ki = cval(c.ki), kss = cval(c.kss);
    const R cai = cval(c.cai), cass = cval(c.cass), cajsr = cval(c.cajsr), cansr = cval(c.cansr);

    // reversal potentials, TPORd.cc:425-427
    const R ENa = (R)RTF * M::lg(M::dv((R)nao, nai));
    const R EK = (R)RTF * M::lg(M::dv((R)ko, ki));
    const R EKs = (R)RTF * M::lg(M::dv((R)(ko + 0.01833 * nao), ki + (R)0.01833 * nai));

    // CaMK, TPORd.cc:430-433
    const R CaMKb = M::dv((R)CaMKo * ((R)1 - c.CaMKt), (R)1 + M::dv((R)KmCaM, cass));
    const R CaMKa = CaMKb + c.CaMKt;
    const R fP = M::dv((R)1, (R)1 + M::dv((R)KmCaMK, CaMKa));   // phosphorylated fraction (fINaLp, fItop, ...)
    const R vffrt = v * (R)FFRT;
    const R vfrt = v * (R)FRT;

    // TP06 fast INa, TPORd.cc:465-504
    {
        const R AM = M::dv((R)1, (R)1 + M::ex(M::dk((R)-60 - v, 5.)));
        const R BM = M::dv((R)0.1, (R)1 + M::ex(M::dk(v + (R)35, 5.))) +
                     M::dv((R)0.10, (R)1 + M::ex(M::dk(v - (R)50, 200.)));
        const R TAU_M = AM * BM;
        const R em = (R)1 + M::ex(M::dk((R)-56.86 - v, 9.03));
        const R M_INF = M::dv((R)1, em * em);
        R rate_h, rate_j;   // 1/tau
        if (v >= (R)-40) {
            rate_h = M::dv((R)0.77, (R)0.13 * ((R)1 + M::ex(M::dk(-(v + (R)10.66), 11.1))));
            rate_j = M::dv((R)0.6 * M::ex((R)0.057 * v), (R)1 + M::ex((R)-0.1 * (v + (R)32)));
        } else {
            rate_h = (R)0.057 * M::ex(M::dk(-(v + (R)80), 6.8)) +
                     ((R)2.7 * M::ex((R)0.079 * v) + (R)3.1e5 * M::ex((R)0.3485 * v));
            const R AJ = M::dv(((R)-2.5428e4 * M::ex((R)0.2444 * v) - (R)6.948e-6 * M::ex((R)-0.04391 * v)) *
                                   (v + (R)37.78),
                               (R)1 + M::ex((R)0.311 * (v + (R)79.23)));
            const R BJ = M::dv((R)0.02424 * M::ex((R)-0.01052 * v), (R)1 + M::ex((R)-0.1378 * (v + (R)40.14)));
            rate_j = AJ + BJ;
        }
        const R eh = (R)1 + M::ex(M::dk(v + (R)71.55, 7.43));
        const R H_INF = M::dv((R)1, eh * eh);
        c.sm = M_INF - (M_INF - c.sm) * M::ex(M::dv(-dt, TAU_M));
        // exp(-dt/TAU) with TAU = 1/rate (TPORd.cc:475,481,488,496)
        if constexpr (sizeof(R) == 8) {
            c.sh = H_INF - (H_INF - c.sh) * M::ex(-dt / ((R)1 / rate_h));
            c.sj = H_INF - (H_INF - c.sj) * M::ex(-dt / ((R)1 / rate_j));
        } else {
            c.sh = H_INF - (H_INF - c.sh) * M::ex(-dt * rate_h);
            c.sj = H_INF - (H_INF - c.sj) * M::ex(-dt * rate_j);
        }
    }
    const R INa = (R)14.838 * c.sm * c.sm * c.sm * c.sh * c.sj * (v - ENa);

    // INaL, TPORd.cc:509-528
    const R mLss = M::dv((R)1, (R)1 + M::ex(M::dk(-(v + (R)42.85), 5.264)));
    const R tm = M::dv((R)1, (R)6.765 * M::ex(M::dk(v + (R)11.64, 34.77)) +
                                 (R)8.552 * M::ex(M::dk(-(v + (R)77.42), 5.955)));
    c.mL = mLss - (mLss - c.mL) * M::ex(M::dv(-dt, tm));
    const R hLss = M::dv((R)1, (R)1 + M::ex(M::dk(v + (R)87.61, 7.488)));
    c.hL = hLss - (hLss - c.hL) * k.e_hl;
    const R hLssp = M::dv((R)1, (R)1 + M::ex(M::dk(v + (R)93.81, 7.488)));
    c.hLp = hLssp - (hLssp - c.hLp) * k.e_hlp;
    const R GNaL = epi ? (R)(0.0075 * 0.6) : (R)0.0075;
    const R INaL = GNaL * (v - ENa) * c.mL * (((R)1 - fP) * c.hL + fP * c.hLp);

    // Ito, TPORd.cc:530-571
    const R ass = M::dv((R)1, (R)1 + M::ex(M::dk(-(v - (R)14.34), 14.82)));
    const R ta = M::dv((R)1.0515, M::dv((R)1, (R)1.2089 * ((R)1 + M::ex(M::dk(-(v - (R)18.4099), 29.3814)))) +
                                      M::dv((R)3.5, (R)1 + M::ex(M::dk(v + (R)100, 29.3814))));
    const R e_ta = M::ex(M::dv(-dt, ta));
    c.a = ass - (ass - c.a) * e_ta;
    const R iss = M::dv((R)1, (R)1 + M::ex(M::dk(v + (R)43.94, 5.711)));
    const R delta_epi = epi ? (R)1 - M::dv((R)0.95, (R)1 + M::ex(M::dk(v + (R)70, 5.))) : (R)1;
    R tiF = (R)4.562 + M::dv((R)1, (R)0.3933 * M::ex(M::dk(-(v + (R)100), 100.)) +
                                      (R)0.08004 * M::ex(M::dk(v + (R)50, 16.59)));
    R tiS = (R)23.62 + M::dv((R)1, (R)0.001416 * M::ex(M::dk(-(v + (R)96.52), 59.05)) +
                                       (R)1.780e-8 * M::ex(M::dk(v + (R)114.1, 8.079)));
    tiF *= delta_epi;
    tiS *= delta_epi;
    const R AiF = M::dv((R)1, (R)1 + M::ex(M::dk(v - (R)213.6, 151.2)));
    const R AiS = (R)1 - AiF;
    c.iF = iss - (iss - c.iF) * M::ex(M::dv(-dt, tiF));
    c.iS = iss - (iss - c.iS) * M::ex(M::dv(-dt, tiS));
    const R ii = AiF * c.iF + AiS * c.iS;
    const R assp = M::dv((R)1, (R)1 + M::ex(M::dk(-(v - (R)24.34), 14.82)));
    c.ap = assp - (assp - c.ap) * e_ta;
    const R dti_develop = (R)1.354 + M::dv((R)1.0e-4, M::ex(M::dk(v - (R)167.4, 15.89)) +
                                                         M::ex(M::dk(-(v - (R)12.23), 0.2154)));
    const R dti_recover = (R)1 - M::dv((R)0.5, (R)1 + M::ex(M::dk(v + (R)70, 20.)));
    const R tiFp = dti_develop * dti_recover * tiF;
    const R tiSp = dti_develop * dti_recover * tiS;
    c.iFp = iss - (iss - c.iFp) * M::ex(M::dv(-dt, tiFp));
    c.iSp = iss - (iss - c.iSp) * M::ex(M::dv(-dt, tiSp));
    const R ip = AiF * c.iFp + AiS * c.iSp;
    const R Gto = (epi || mid) ? (R)(0.02 * 4.0) : (R)0.02;
    const R Ito = Gto * (v - EK) * (((R)1 - fP) * c.a * ii + fP * c.ap * ip);

    // ICaL, ICaNa, ICaK, TPORd.cc:573-652
    const R dss = M::dv((R)1, (R)1 + M::ex(M::dk(-(v + (R)3.940 + m.dss_shift), 4.230)));
    const R td = (R)0.6 + M::dv((R)1, M::ex((R)-0.05 * (v + (R)6)) + M::ex((R)0.09 * (v + (R)14)));
    c.d = dss - (dss - c.d) * M::ex(M::dv(-dt, td));
    const R fss = M::dv((R)1, (R)1 + M::ex(M::dk(v + (R)19.58 + m.fss_shift, 3.696)));
    const R tff = (R)7 + M::dv((R)1, (R)0.0045 * M::ex(M::dk(-(v + (R)20), 10.)) +
                                     (R)0.0045 * M::ex(M::dk(v + (R)20, 10.)));
    const R tfs = (R)1000 + M::dv((R)1, (R)0.000035 * M::ex(M::dk(-(v + (R)5), 4.)) +
                                        (R)0.000035 * M::ex(M::dk(v + (R)5, 6.)));
    constexpr double Aff = 0.6, Afs = 1.0 - Aff;
    c.ff = fss - (fss - c.ff) * M::ex(M::dv(-dt, tff));
    c.fs = fss - (fss - c.fs) * M::ex(M::dv(-dt, tfs));
    const R f = (R)Aff * c.ff + (R)Afs * c.fs;
    const R fcass = fss;
    const R tfcaf = (R)7 + M::dv((R)1, (R)0.04 * M::ex(M::dk(-(v - (R)4), 7.)) +
                                       (R)0.04 * M::ex(M::dk(v - (R)4, 7.)));
    const R tfcas = (R)100 + M::dv((R)1, (R)0.00012 * M::ex(M::dk(-v, 3.)) + (R)0.00012 * M::ex(M::dk(v, 7.)));
    const R Afcaf = (R)0.3 + M::dv((R)0.6, (R)1 + M::ex(M::dk(v - (R)10, 10.)));
    const R Afcas = (R)1 - Afcaf;
    c.fcaf = fcass - (fcass - c.fcaf) * M::ex(M::dv(-dt, tfcaf));
    c.fcas = fcass - (fcass - c.fcas) * M::ex(M::dv(-dt, tfcas));
    const R fca = Afcaf * c.fcaf + Afcas * c.fcas;
    c.jca = fcass - (fcass - c.jca) * k.e_jca;
    c.ffp = fss - (fss - c.ffp) * M::ex(M::dv(-dt, (R)2.5 * tff));
    const R fp = (R)Aff * c.ffp + (R)Afs * c.fs;
    c.fcafp = fcass - (fcass - c.fcafp) * M::ex(M::dv(-dt, (R)2.5 * tfcaf));
    const R fcap = Afcaf * c.fcafp + Afcas * c.fcas;
    {
        const R km2n = c.jca * (R)1;
        const R q = (R)1 + M::dv((R)0.002, cass);
        const R q2 = q * q;
        const R anca = M::dv((R)1, M::dv((R)1000, km2n) + q2 * q2);
        const R nss = M::dv(anca * (R)1000, km2n);
        c.nca = nss - (nss - c.nca) * M::ex(-km2n * dt);
    }
    R PhiCaL, PhiCaNa, PhiCaK, INab_phi, ICab_phi;
    if constexpr (sizeof(R) == 8) {
        const R e1 = exp(1.0 * vfrt), e2 = exp(2.0 * vfrt);
        PhiCaL = 4.0 * vffrt * (cass * e2 - 0.341 * cao) / (e2 - 1.0);
        PhiCaNa = 1.0 * vffrt * (0.75 * nass * e1 - 0.75 * nao) / (e1 - 1.0);
        PhiCaK = 1.0 * vffrt * (0.75 * kss * e1 - 0.75 * ko) / (e1 - 1.0);
        INab_phi = vffrt * (nai * e1 - nao) / (e1 - 1.0);
        ICab_phi = 4.0 * vffrt * (cai * e2 - 0.341 * cao) / (e2 - 1.0);
    } else {
        // vffrt/(e^z - 1) = (F/z_) * (z/(e^z - 1)) / z_-scaled: vffrt = F*vfrt
        const float em1 = expm1f(vfrt);
        const float e1 = em1 + 1.0f;
        const float e2m1 = em1 * (e1 + 1.0f);
        const float e2 = e2m1 + 1.0f;
        const float g1 = (float)(F_) * x_over_expm1(vfrt, em1);               // vffrt/(e1-1)
        const float g2 = (float)(F_ * 0.5) * x_over_expm1(2.0f * vfrt, e2m1); // vffrt/(e2-1)
        PhiCaL = 4.0f * g2 * (cass * e2 - (float)(0.341 * cao));
        PhiCaNa = g1 * (0.75f * nass * e1 - (float)(0.75 * nao));
        PhiCaK = g1 * (0.75f * kss * e1 - (float)(0.75 * ko));
        INab_phi = g1 * (nai * e1 - (float)nao);
        ICab_phi = 4.0f * g2 * (cai * e2 - (float)(0.341 * cao));
    }
    const int cls = epi ? 1 : (mid ? 2 : 0);
    const R PCa = m.pca[cls];
    const R PCap = (R)1.1 * PCa;
    const R gate_np = c.d * (f * ((R)1 - c.nca) + c.jca * fca * c.nca);
    const R gate_p = c.d * (fp * ((R)1 - c.nca) + c.jca * fcap * c.nca);
    const R ICaL = ((R)1 - fP) * PCa * PhiCaL * gate_np + fP * PCap * PhiCaL * gate_p;
    const R ICaNa = ((R)1 - fP) * ((R)0.00125 * PCa) * PhiCaNa * gate_np + fP * ((R)0.00125 * PCap) * PhiCaNa * gate_p;
    const R ICaK = ((R)1 - fP) * ((R)3.574e-4 * PCa) * PhiCaK * gate_np + fP * ((R)3.574e-4 * PCap) * PhiCaK * gate_p;

    // IKr, TPORd.cc:654-678 (sqrt(ko/5.4) = 1)
    const R xrss = M::dv((R)1, (R)1 + M::ex(M::dk(-(v + (R)8.337), 6.789)));
    const R txrf = (R)12.98 + M::dv((R)1, (R)0.3652 * M::ex(M::dk(v - (R)31.66, 3.869)) +
                                          (R)4.123e-5 * M::ex(M::dk(-(v - (R)47.78), 20.38)));
    const R txrs = (R)1.865 + M::dv((R)1, (R)0.06629 * M::ex(M::dk(v - (R)34.70, 7.355)) +
                                          (R)1.128e-5 * M::ex(M::dk(-(v - (R)29.74), 25.94)));
    const R Axrf = M::dv((R)1, (R)1 + M::ex(M::dk(v + (R)54.81, 38.21)));
    const R Axrs = (R)1 - Axrf;
    c.xrf = xrss - (xrss - c.xrf) * M::ex(M::dv(-dt, txrf));
    c.xrs = xrss - (xrss - c.xrs) * M::ex(M::dv(-dt, txrs));
    const R xr = Axrf * c.xrf + Axrs * c.xrs;
    const R rkr = M::dv((R)1, ((R)1 + M::ex(M::dk(v + (R)55, 75.))) * ((R)1 + M::ex(M::dk(v - (R)10, 30.))));
    const R GKr = epi ? (R)(0.046 * 1.3) : (mid ? (R)(0.046 * 0.8) : (R)0.046);
    const R IKr = GKr * xr * rkr * (v - EK);

    // IKs, TPORd.cc:680-735
    const R xs1ss = M::dv((R)1, (R)1 + M::ex(M::dk(-(v + (R)11.60), 8.932)));
    const R txs1 = (R)817.3 + M::dv((R)1, (R)2.326e-4 * M::ex(M::dk(v + (R)48.28, 17.80)) +
                                          (R)0.001292 * M::ex(M::dk(-(v + (R)210), 230.)));
    c.xs1 = xs1ss - (xs1ss - c.xs1) * M::ex(M::dv(-dt, txs1));
    const R rate_xs2 = (R)0.01 * M::ex(M::dk(v - (R)50, 20.)) + (R)0.0193 * M::ex(M::dk(-(v + (R)66.54), 31.));
    if constexpr (sizeof(R) == 8)
        c.xs2 = xs1ss - (xs1ss - c.xs2) * exp(-dt / (1.0 / rate_xs2));
    else
        c.xs2 = xs1ss - (xs1ss - c.xs2) * M::ex(-dt * rate_xs2);
    const R KsCa = (R)1 + M::dv((R)0.6, (R)1 + M::pw(M::dv((R)3.8e-5, cai), (R)1.4));
    const R IKs = m.gks[cls] * KsCa * c.xs1 * c.xs2 * (v - EKs);

    // IK1, TPORd.cc:738-751 (sqrt(ko) constant)
    const R xk1ss = M::dv((R)1, (R)1 + M::ex(M::dk(-(v + (R)(2.5538 * ko + 144.59)), 1.5692 * ko + 3.8115)));
    const R txk1 = M::dv((R)122.2, M::ex(M::dk(-(v + (R)127.2), 20.36)) + M::ex(M::dk(v + (R)236.8, 69.33)));
    c.xk1 = xk1ss - (xk1ss - c.xk1) * M::ex(M::dv(-dt, txk1));
    const R rk1 = M::dv((R)1, (R)1 + M::ex(M::dk(v + (R)(105.8 - 2.6 * ko), 9.493)));
    const R GK1 = epi ? (R)(0.1908 * 1.2) : (mid ? (R)(0.1908 * 1.3) : (R)0.1908);
    const R IK1 = GK1 * (R)2.32379000772445 /* sqrt(ko) */ * rk1 * c.xk1 * (v - EK);

    // INaCa_i and INaCa_ss, TPORd.cc:753-852
    constexpr double kna1 = 15.0, kna2 = 5.0, kna3 = 88.12, kasymm = 12.5;
    constexpr double wna = 6.0e4, wca = 6.0e4, wnaca = 5.0e3, kcaon = 1.5e6, kcaoff = 5.0e3;
    constexpr double h10 = kasymm + 1.0 + nao / kna1 * (1.0 + nao / kna2);
    constexpr double h11 = nao * nao / (h10 * kna1 * kna2);
    constexpr double h12 = 1.0 / h10;
    constexpr double k1 = h12 * cao * kcaon;
    constexpr double k2 = kcaoff, k5 = kcaoff;
    const R hca = M::ex((R)(0.1670 * FRT) * v);
    const R hna = M::ex((R)(0.5224 * FRT) * v);
    const R h7 = (R)1 + M::dk((R)nao, kna3) * ((R)1 + M::dv((R)1, hna));
    const R h8 = M::dv((R)nao, (R)kna3 * hna * h7);
    const R h9 = M::dv((R)1, h7);
    const R k3p = h9 * (R)wca;
    const R k3pp = h8 * (R)wnaca;
    const R k3 = k3p + k3pp;
    const R k8 = h8 * (R)h11 * (R)wna;
    const R Gncx = epi ? (R)(0.0008 * 1.1) : (mid ? (R)(0.0008 * 1.4) : (R)0.0008);
    R INaCa_i, INaCa_ss;
#pragma unroll
    for (int pass = 0; pass < 2; ++pass) {
        const R na = pass == 0 ? nai : nass;
        const R ca = pass == 0 ? cai : cass;
        const R h1 = (R)1 + M::dk(na, kna3) * ((R)1 + hna);
        const R h2 = M::dv(na * hna, (R)kna3 * h1);
        const R h3 = M::dv((R)1, h1);
        const R h4 = (R)1 + M::dk(na, kna1) * ((R)1 + M::dk(na, kna2));
        const R h5 = M::dv(na * na, h4 * (R)(kna1 * kna2));
        const R h6 = M::dv((R)1, h4);
        const R k4p = M::dv(h3 * (R)wca, hca);
        const R k4pp = h2 * (R)wnaca;
        const R k4 = k4p + k4pp;
        const R k6 = h6 * ca * (R)kcaon;
        const R k7 = h5 * h2 * (R)wna;
        const R x1 = (R)k2 * k4 * (k7 + k6) + (R)k5 * k7 * ((R)k2 + k3);
        const R x2 = (R)k1 * k7 * (k4 + (R)k5) + k4 * k6 * ((R)k1 + k8);
        const R x3 = (R)k1 * k3 * (k7 + k6) + k8 * k6 * ((R)k2 + k3);
        const R x4 = (R)k2 * k8 * (k4 + (R)k5) + k3 * (R)k5 * ((R)k1 + k8);
        const R xs = x1 + x2 + x3 + x4;
        const R E1 = M::dv(x1, xs), E2 = M::dv(x2, xs), E3 = M::dv(x3, xs), E4 = M::dv(x4, xs);
        const R r = M::dv((R)150.0e-6, ca);
        const R allo = M::dv((R)1, (R)1 + r * r);
        const R JncxNa = (R)3 * (E4 * k7 - E1 * k8) + E3 * k4pp - E2 * k3pp;
        const R JncxCa = E2 * (R)k2 - E1 * (R)k1;
        const R val = Gncx * allo * (JncxNa + (R)2 * JncxCa);
        if (pass == 0) INaCa_i = (R)0.8 * val;
        else INaCa_ss = (R)0.2 * val;
    }
    const R INaCa = INaCa_i + INaCa_ss;

    // INaK, TPORd.cc:854-906
    constexpr double k1p = 949.5, k1m = 182.4, k2p = 687.2, k2m = 39.4;
    constexpr double k3p_ = 1899.0, k3m = 79300.0, k4p_ = 639.0, k4m = 40.0;
    constexpr double Knai0 = 9.073, Knao0 = 27.78, delta = -0.1550;
    constexpr double Kki = 0.5, Kko = 0.3582, MgADP = 0.05, MgATP = 9.8, Kmgatp = 1.698e-7;
    constexpr double H = 1.0e-7, eP = 4.2, Khp = 1.698e-7, Knap = 224.0, Kxkur = 292.0;
    const R Knai = (R)Knai0 * M::ex((R)(delta * F_ / (3.0 * R_ * T_)) * v);
    const R Knao = (R)Knao0 * M::ex((R)((1.0 - delta) * F_ / (3.0 * R_ * T_)) * v);
    const R P = M::dv((R)eP, (R)(1.0 + H / Khp) + M::dk(nai, Knap) + M::dk(ki, Kxkur));
    const R rnai = M::dv(nai, Knai), rnao = M::dv((R)nao, Knao);
    const R rki = M::dk(ki, Kki);
    constexpr double rko = ko / Kko;
    const R pnai = (R)1 + rnai, pnao = (R)1 + rnao, pki = (R)1 + rki;
    const R den_i = pnai * pnai * pnai + pki * pki - (R)1;
    const R den_o = pnao * pnao * pnao + (R)((1.0 + rko) * (1.0 + rko)) - (R)1;
    const R a1 = M::dv((R)k1p * (rnai * rnai * rnai), den_i);
    constexpr double b1 = k1m * MgADP;
    constexpr double a2 = k2p;
    const R b2 = M::dv((R)k2m * (rnao * rnao * rnao), den_o);
    const R a3 = M::dv((R)(k3p_ * rko * rko), den_o);
    const R b3 = (R)(k3m * H / (1.0 + MgATP / Kmgatp)) * P;
    constexpr double a4 = (k4p_ * MgATP / Kmgatp) / (1.0 + MgATP / Kmgatp);
    const R b4 = M::dv((R)k4m * (rki * rki), den_i);
    const R y1 = (R)a4 * a1 * (R)a2 + b2 * b4 * b3 + (R)a2 * b4 * b3 + b3 * a1 * (R)a2;
    const R y2 = b2 * (R)b1 * b4 + a1 * (R)a2 * a3 + a3 * (R)b1 * b4 + (R)a2 * a3 * b4;
    const R y3 = (R)a2 * a3 * (R)a4 + b3 * b2 * (R)b1 + b2 * (R)b1 * (R)a4 + a3 * (R)a4 * (R)b1;
    const R y4 = b4 * b3 * b2 + a3 * (R)a4 * a1 + b2 * (R)a4 * a1 + b3 * b2 * a1;
    const R ys = y1 + y2 + y3 + y4;
    const R E1 = M::dv(y1, ys), E2 = M::dv(y2, ys), E3 = M::dv(y3, ys), E4 = M::dv(y4, ys);
    const R JnakNa = (R)3 * (E1 * a3 - E2 * b3);
    const R JnakK = (R)2 * (E4 * (R)b1 - E3 * a1);
    const R Pnak = epi ? (R)(30 * 0.9) : (mid ? (R)(30 * 0.7) : (R)30);
    const R INaK = Pnak * (JnakNa + JnakK);

    // background currents and pump, TPORd.cc:908-923
    const R xkb = M::dv((R)1, (R)1 + M::ex(M::dk(-(v - (R)14.48), 18.34)));
    const R GKb = epi ? (R)(0.003 * 0.6) : (R)0.003;
    const R IKb = GKb * xkb * (v - EK);
    const R INab = (R)3.75e-10 * INab_phi;
    const R ICab = (R)2.5e-8 * ICab_phi;
    const R IpCa = M::dv((R)0.0005 * cai, (R)0.0005 + cai);

    // membrane potential, TPORd.cc:927-935
    const R Iion = INa + INaL + Ito + ICaL + ICaNa + ICaK + IKr + IKs + IK1 + INaCa + INaK + INab + IKb + IpCa + ICab;
    const R dV_dt = (R)-1 * (Iion + Ist);
    c.v = v + (dV_dt + dVgap_dt) * dt;
    if (out) {
        out->dvdt = dV_dt;
        out->ical = ICaL;
        out->iks = IKs;
        out->ina = INa;
        out->ikr = IKr;
        out->ik1 = IK1;
    }

    // CaMK and fluxes, TPORd.cc:939-995
    c.CaMKt += dt * ((R)0.05 * CaMKb * (CaMKb + c.CaMKt) - (R)0.00068 * c.CaMKt);
    // concentration differences from the full-precision values (file comment)
    const R JdiffNa = cdiff(c.nass, c.nai) * (R)0.5;
    const R JdiffK = cdiff(c.kss, c.ki) * (R)0.5;
    const R Jdiff = M::dk(cdiff(c.cass, c.cai), 0.2);
    const R Jtr = M::dk(cdiff(c.cansr, c.cajsr), 100.);
    {
        const R r15 = M::dv((R)1.5, cajsr);
        const R r2 = r15 * r15, r4 = r2 * r2;
        const R den = (R)1 + r4 * r4;
        R Jrel_inf = M::dv((R)(0.5 * 4.75) * (-ICaL), den);
        R Jrel_infp = M::dv((R)(0.5 * 1.25 * 4.75) * (-ICaL), den);
        if (mid) {
            Jrel_inf *= (R)1.7;
            Jrel_infp *= (R)1.7;
        }
        const R tq = (R)1 + M::dv((R)0.0123, cajsr);
        R tau_rel = M::dv((R)4.75, tq);
        R tau_relp = M::dv((R)(1.25 * 4.75), tq);
        if (tau_rel < (R)0.005) tau_rel = (R)0.005;
        if (tau_relp < (R)0.005) tau_relp = (R)0.005;
        c.Jrelnp = Jrel_inf - (Jrel_inf - c.Jrelnp) * M::ex(M::dv(-dt, tau_rel));
        c.Jrelp = Jrel_infp - (Jrel_infp - c.Jrelp) * M::ex(M::dv(-dt, tau_relp));
    }
    const R Jrel = ((R)1 - fP) * c.Jrelnp + fP * c.Jrelp;
    R Jupnp = M::dv((R)0.004375 * cai, cai + (R)0.00092);
    R Jupp = M::dv((R)(2.75 * 0.004375) * cai, cai + (R)(0.00092 - 0.00017));
    if (epi) {
        Jupnp *= (R)1.3;
        Jupp *= (R)1.3;
    }
    const R Jleak = M::dk((R)0.0039375 * cansr, 15.);
    const R Jup = ((R)1 - fP) * Jupnp + fP * Jupp - Jleak;

    // concentrations, forward Euler, TPORd.cc:997-1020
    const R dnai = -(INa + INaL + (R)3 * INaCa_i + (R)3 * INaK + INab) * (R)(Acap / (F_ * vmyo)) + JdiffNa * (R)(vss / vmyo);
    const R dnass = -(ICaNa + (R)3 * INaCa_ss) * (R)(Acap / (F_ * vss)) - JdiffNa;
    const R dki = -(Ito + IKr + IKs + IK1 + IKb + Ist - (R)2 * INaK) * (R)(Acap / (F_ * vmyo)) + JdiffK * (R)(vss / vmyo);
    const R dkss = -ICaK * (R)(Acap / (F_ * vss)) - JdiffK;
    constexpr double cmdnmax = 0.05, kmcmdn = 0.00238, trpnmax = 0.07, kmtrpn = 0.0005;
    const R qc = (R)kmcmdn + cai, qt = (R)kmtrpn + cai;
    const R Bcai = M::dv((R)1, (R)1 + M::dv(epi ? (R)(1.3 * cmdnmax * kmcmdn) : (R)(cmdnmax * kmcmdn), qc * qc) +
                                   M::dv((R)(trpnmax * kmtrpn), qt * qt));
    const R dcai = Bcai * (-(IpCa + ICab - (R)2 * INaCa_i) * (R)(Acap / (2.0 * F_ * vmyo)) - Jup * (R)(vnsr / vmyo) +
                           Jdiff * (R)(vss / vmyo));
    constexpr double BSRmax = 0.047, KmBSR = 0.00087, BSLmax = 1.124, KmBSL = 0.0087;
    const R qsr = (R)KmBSR + cass, qsl = (R)KmBSL + cass;
    const R Bcass = M::dv((R)1, (R)1 + M::dv((R)(BSRmax * KmBSR), qsr * qsr) + M::dv((R)(BSLmax * KmBSL), qsl * qsl));
    const R dcass = Bcass * (-(ICaL - (R)2 * INaCa_ss) * (R)(Acap / (2.0 * F_ * vss)) + Jrel * (R)(vjsr / vss) - Jdiff);
    const R dcansr = Jup - Jtr * (R)(vjsr / vnsr);
    constexpr double csqnmax = 10.0, kmcsqn = 0.8;
    const R qj = (R)kmcsqn + cajsr;
    const R Bcajsr = M::dv((R)1, (R)1 + M::dv((R)(csqnmax * kmcsqn), qj * qj));
    const R dcajsr = Bcajsr * (Jtr - Jrel);
    cadd(c.nai, dt * dnai);
    cadd(c.nass, dt * dnass);
    cadd(c.ki, dt * dki);
    cadd(c.kss, dt * dkss);
    cadd(c.cai, dt * dcai);
    cadd(c.cass, dt * dcass);
    cadd(c.cansr, dt * dcansr);
    cadd(c.cajsr, dt * dcajsr);
}

}  // namespace lqt
