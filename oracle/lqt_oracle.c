/*
 * lqt_oracle.c -- TEST INFRASTRUCTURE ONLY (see lqt_oracle.h).
 *
 * FP64 CPU restatement of the reference's TPORd path.  Build with
 * -O3 -ffp-contract=off (oracle/Makefile) so that x86 and Arm agree and the
 * single-cell update matches the reference's own g++ -O3 build bit for bit.
 *
 * The model equations are the published ten Tusscher 2006 INa and O'Hara-Rudy
 * 2011 formulations as combined in SingleCell/TPORd.cc; each block cites the
 * lines it restates and keeps their association order, because bitwise parity
 * with the reference depends on it.
 */
#include "lqt_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------ */
/* SingleCell/TPORd.cc:142-198                                              */
void orc_initial_state(double v0, double *s)
{
    static const double rest[LQT_NSTATE] = {
        -87.5,                     /* v (replaced by v0)         */
        7.0, 7.0, 145.0, 145.0,    /* nai nass ki kss            */
        1.0e-4, 1.0e-4, 1.2, 1.2,  /* cai cass cansr cajsr       */
        0.0, 1.0, 1.0,             /* sm sh sj (TP06 INa)        */
        1.0, 1.0,                  /* hsp jp                     */
        0.0, 1.0, 1.0,             /* mL hL hLp                  */
        0.0, 1.0, 1.0,             /* a iF iS                    */
        0.0, 1.0, 1.0,             /* ap iFp iSp                 */
        0.0, 1.0, 1.0,             /* d ff fs                    */
        1.0, 1.0, 1.0, 0.0,        /* fcaf fcas jca nca          */
        1.0, 1.0,                  /* ffp fcafp                  */
        0.0, 0.0, 0.0, 0.0, 1.0,   /* xrf xrs xs1 xs2 xk1        */
        0.0, 0.0, 0.0              /* Jrelnp Jrelp CaMKt         */
    };
    memcpy(s, rest, sizeof(rest));
    s[LQT_S_V] = v0;
}

/* ------------------------------------------------------------------------ */
/* One TPORd::update(), SingleCell/TPORd.cc:379-1021.                        */
void orc_update(double *s, int ctype, const lqt_model *m, double dt,
                double Ist, double dVgap_dt, orc_aux *aux)
{
    const int is_epi = (ctype == LQT_EPI);
    const int is_mid = (ctype == LQT_MCELL);

    double v = s[LQT_S_V];
    double nai = s[LQT_S_NAI], nass = s[LQT_S_NASS];
    double ki = s[LQT_S_KI], kss = s[LQT_S_KSS];
    double cai = s[LQT_S_CAI], cass = s[LQT_S_CASS];
    double cansr = s[LQT_S_CANSR], cajsr = s[LQT_S_CAJSR];
    double sm = s[LQT_S_SM], sh = s[LQT_S_SH], sj = s[LQT_S_SJ];
    double hsp = s[LQT_S_HSP], jp = s[LQT_S_JP];
    double mL = s[LQT_S_ML], hL = s[LQT_S_HL], hLp = s[LQT_S_HLP];
    double a = s[LQT_S_A], iF = s[LQT_S_IF], iS = s[LQT_S_IS];
    double ap = s[LQT_S_AP], iFp = s[LQT_S_IFP], iSp = s[LQT_S_ISP];
    double d = s[LQT_S_D], ff = s[LQT_S_FF], fs = s[LQT_S_FS];
    double fcaf = s[LQT_S_FCAF], fcas = s[LQT_S_FCAS];
    double jca = s[LQT_S_JCA], nca = s[LQT_S_NCA];
    double ffp = s[LQT_S_FFP], fcafp = s[LQT_S_FCAFP];
    double xrf = s[LQT_S_XRF], xrs = s[LQT_S_XRS];
    double xs1 = s[LQT_S_XS1], xs2 = s[LQT_S_XS2], xk1 = s[LQT_S_XK1];
    double Jrelnp = s[LQT_S_JRELNP], Jrelp = s[LQT_S_JRELP];
    double CaMKt = s[LQT_S_CAMKT];
    (void)hsp; (void)jp;   /* carried, unused by the TP06 INa (TPORd.cc:436-460) */

    /* constants, TPORd.cc:382-421 */
    const double nao = 140.0, cao = 1.8, ko = 5.4;
    const double BSRmax = 0.047, KmBSR = 0.00087, BSLmax = 1.124, KmBSL = 0.0087;
    const double cmdnmax = 0.05, kmcmdn = 0.00238, trpnmax = 0.07, kmtrpn = 0.0005;
    const double csqnmax = 10.0, kmcsqn = 0.8;
    const double aCaMK = 0.05, bCaMK = 0.00068, CaMKo = 0.05, KmCaM = 0.0015, KmCaMK = 0.15;
    const double R = 8314.0, T = 310.0, F = 96485.0;
    const double L = 0.01, rad = 0.0011;
    const double vcell = 1000 * 3.14 * rad * rad * L;
    const double Ageo = 2 * 3.14 * rad * rad + 2 * 3.14 * rad * L;
    const double Acap = 2 * Ageo;
    const double vmyo = 0.68 * vcell;
    const double vnsr = 0.0552 * vcell;
    const double vjsr = 0.0048 * vcell;
    const double vss = 0.02 * vcell;

    /* reversal potentials, TPORd.cc:425-427 */
    double ENa = (R * T / F) * log(nao / nai);
    double EK = (R * T / F) * log(ko / ki);
    double EKs = (R * T / F) * log((ko + 0.01833 * nao) / (ki + 0.01833 * nai));

    /* CaMK, TPORd.cc:430-433 */
    double CaMKb = CaMKo * (1.0 - CaMKt) / (1.0 + KmCaM / cass);
    double CaMKa = CaMKb + CaMKt;
    double vffrt = v * F * F / (R * T);
    double vfrt = v * F / (R * T);

    /* TP06 fast INa, TPORd.cc:465-504 */
    double AM = 1. / (1. + exp((-60. - v) / 5.));
    double BM = 0.1 / (1. + exp((v + 35.) / 5.)) + 0.10 / (1. + exp((v - 50.) / 200.));
    double TAU_M = AM * BM;
    double M_INF = 1. / ((1. + exp((-56.86 - v) / 9.03)) * (1. + exp((-56.86 - v) / 9.03)));
    double TAU_H, TAU_J;
    if (v >= -40.) {
        double BH_1 = (0.77 / (0.13 * (1. + exp(-(v + 10.66) / 11.1))));
        TAU_H = 1.0 / (0. + BH_1);
    } else {
        double AH_2 = (0.057 * exp(-(v + 80.) / 6.8));
        double BH_2 = (2.7 * exp(0.079 * v) + (3.1e5) * exp(0.3485 * v));
        TAU_H = 1.0 / (AH_2 + BH_2);
    }
    double H_INF = 1. / ((1. + exp((v + 71.55) / 7.43)) * (1. + exp((v + 71.55) / 7.43)));
    if (v >= -40.) {
        double BJ_1 = (0.6 * exp((0.057) * v) / (1. + exp(-0.1 * (v + 32.))));
        TAU_J = 1.0 / (0. + BJ_1);
    } else {
        double AJ_2 = (((-2.5428e4) * exp(0.2444 * v) - (6.948e-6) * exp(-0.04391 * v)) * (v + 37.78) /
                       (1. + exp(0.311 * (v + 79.23))));
        double BJ_2 = (0.02424 * exp(-0.01052 * v) / (1. + exp(-0.1378 * (v + 40.14))));
        TAU_J = 1.0 / (AJ_2 + BJ_2);
    }
    double J_INF = H_INF;
    sm = M_INF - (M_INF - sm) * exp(-dt / TAU_M);
    sh = H_INF - (H_INF - sh) * exp(-dt / TAU_H);
    sj = J_INF - (J_INF - sj) * exp(-dt / TAU_J);
    double GNa = 14.838;
    double INa = GNa * sm * sm * sm * sh * sj * (v - ENa);

    /* INaL, TPORd.cc:509-528 */
    double mLss = 1.0 / (1.0 + exp((-(v + 42.85)) / 5.264));
    double tm = 1.0 / (6.765 * exp((v + 11.64) / 34.77) + 8.552 * exp(-(v + 77.42) / 5.955));
    double tmL = tm;
    mL = mLss - (mLss - mL) * exp(-dt / tmL);
    double hLss = 1.0 / (1.0 + exp((v + 87.61) / 7.488));
    double thL = 200.0;
    hL = hLss - (hLss - hL) * exp(-dt / thL);
    double hLssp = 1.0 / (1.0 + exp((v + 93.81) / 7.488));
    double thLp = 3.0 * thL;
    hLp = hLssp - (hLssp - hLp) * exp(-dt / thLp);
    double GNaL = 0.0075;
    if (is_epi) GNaL *= 0.6;
    double fINaLp = (1.0 / (1.0 + KmCaMK / CaMKa));
    double INaL = GNaL * (v - ENa) * mL * ((1.0 - fINaLp) * hL + fINaLp * hLp);

    /* Ito, TPORd.cc:530-571 */
    double ass = 1.0 / (1.0 + exp((-(v - 14.34)) / 14.82));
    double ta = 1.0515 / (1.0 / (1.2089 * (1.0 + exp(-(v - 18.4099) / 29.3814))) +
                          3.5 / (1.0 + exp((v + 100.0) / 29.3814)));
    a = ass - (ass - a) * exp(-dt / ta);
    double iss = 1.0 / (1.0 + exp((v + 43.94) / 5.711));
    double delta_epi = is_epi ? 1.0 - (0.95 / (1.0 + exp((v + 70.0) / 5.0))) : 1.0;
    double tiF = 4.562 + 1 / (0.3933 * exp((-(v + 100.0)) / 100.0) + 0.08004 * exp((v + 50.0) / 16.59));
    double tiS = 23.62 + 1 / (0.001416 * exp((-(v + 96.52)) / 59.05) + 1.780e-8 * exp((v + 114.1) / 8.079));
    tiF *= delta_epi;
    tiS *= delta_epi;
    double AiF = 1.0 / (1.0 + exp((v - 213.6) / 151.2));
    double AiS = 1.0 - AiF;
    iF = iss - (iss - iF) * exp(-dt / tiF);
    iS = iss - (iss - iS) * exp(-dt / tiS);
    double i_ = AiF * iF + AiS * iS;
    double assp = 1.0 / (1.0 + exp((-(v - 24.34)) / 14.82));
    ap = assp - (assp - ap) * exp(-dt / ta);
    double dti_develop = 1.354 + 1.0e-4 / (exp((v - 167.4) / 15.89) + exp(-(v - 12.23) / 0.2154));
    double dti_recover = 1.0 - 0.5 / (1.0 + exp((v + 70.0) / 20.0));
    double tiFp = dti_develop * dti_recover * tiF;
    double tiSp = dti_develop * dti_recover * tiS;
    iFp = iss - (iss - iFp) * exp(-dt / tiFp);
    iSp = iss - (iss - iSp) * exp(-dt / tiSp);
    double ip = AiF * iFp + AiS * iSp;
    double Gto = 0.02;
    if (is_epi) Gto *= 4.0;
    if (is_mid) Gto *= 4.0;
    double fItop = (1.0 / (1.0 + KmCaMK / CaMKa));
    double Ito = Gto * (v - EK) * ((1.0 - fItop) * a * i_ + fItop * ap * ip);

    /* ICaL, ICaNa, ICaK, TPORd.cc:573-652 (ISO1 gate shifts as parameters) */
    double dss = 1.0 / (1.0 + exp((-(v + 3.940 + m->dss_shift)) / 4.230));
    double td = 0.6 + 1.0 / (exp(-0.05 * (v + 6.0)) + exp(0.09 * (v + 14.0)));
    d = dss - (dss - d) * exp(-dt / td);
    double fss = 1.0 / (1.0 + exp((v + 19.58 + m->fss_shift) / 3.696));
    double tff = 7.0 + 1.0 / (0.0045 * exp(-(v + 20.0) / 10.0) + 0.0045 * exp((v + 20.0) / 10.0));
    double tfs = 1000.0 + 1.0 / (0.000035 * exp(-(v + 5.0) / 4.0) + 0.000035 * exp((v + 5.0) / 6.0));
    double Aff = 0.6;
    double Afs = 1.0 - Aff;
    ff = fss - (fss - ff) * exp(-dt / tff);
    fs = fss - (fss - fs) * exp(-dt / tfs);
    double f = Aff * ff + Afs * fs;
    double fcass = fss;
    double tfcaf = 7.0 + 1.0 / (0.04 * exp(-(v - 4.0) / 7.0) + 0.04 * exp((v - 4.0) / 7.0));
    double tfcas = 100.0 + 1.0 / (0.00012 * exp(-v / 3.0) + 0.00012 * exp(v / 7.0));
    double Afcaf = 0.3 + 0.6 / (1.0 + exp((v - 10.0) / 10.0));
    double Afcas = 1.0 - Afcaf;
    fcaf = fcass - (fcass - fcaf) * exp(-dt / tfcaf);
    fcas = fcass - (fcass - fcas) * exp(-dt / tfcas);
    double fca = Afcaf * fcaf + Afcas * fcas;
    double tjca = 75.0;
    jca = fcass - (fcass - jca) * exp(-dt / tjca);
    double tffp = 2.5 * tff;
    ffp = fss - (fss - ffp) * exp(-dt / tffp);
    double fp = Aff * ffp + Afs * fs;
    double tfcafp = 2.5 * tfcaf;
    fcafp = fcass - (fcass - fcafp) * exp(-dt / tfcafp);
    double fcap = Afcaf * fcafp + Afcas * fcas;
    double Kmn = 0.002;
    double k2n = 1000.0;
    double km2n = jca * 1.0;
    double anca = 1.0 / (k2n / km2n + pow(1.0 + Kmn / cass, 4.0));
    nca = anca * k2n / km2n - (anca * k2n / km2n - nca) * exp(-km2n * dt);
    double PhiCaL = 4.0 * vffrt * (cass * exp(2.0 * vfrt) - 0.341 * cao) / (exp(2.0 * vfrt) - 1.0);
    double PhiCaNa = 1.0 * vffrt * (0.75 * nass * exp(1.0 * vfrt) - 0.75 * nao) / (exp(1.0 * vfrt) - 1.0);
    double PhiCaK = 1.0 * vffrt * (0.75 * kss * exp(1.0 * vfrt) - 0.75 * ko) / (exp(1.0 * vfrt) - 1.0);
    double zca = 2.0;
    double PCa = 0.0001;
    PCa *= m->pca_scale;
    if (is_epi) PCa *= 1.2;
    if (is_mid) PCa *= 2.5;
    double PCap = 1.1 * PCa;
    double PCaNa = 0.00125 * PCa;
    double PCaK = 3.574e-4 * PCa;
    double PCaNap = 0.00125 * PCap;
    double PCaKp = 3.574e-4 * PCap;
    double fICaLp = (1.0 / (1.0 + KmCaMK / CaMKa));
    double ICaL = (1.0 - fICaLp) * PCa * PhiCaL * d * (f * (1.0 - nca) + jca * fca * nca) +
                  fICaLp * PCap * PhiCaL * d * (fp * (1.0 - nca) + jca * fcap * nca);
    double ICaNa = (1.0 - fICaLp) * PCaNa * PhiCaNa * d * (f * (1.0 - nca) + jca * fca * nca) +
                   fICaLp * PCaNap * PhiCaNa * d * (fp * (1.0 - nca) + jca * fcap * nca);
    double ICaK = (1.0 - fICaLp) * PCaK * PhiCaK * d * (f * (1.0 - nca) + jca * fca * nca) +
                  fICaLp * PCaKp * PhiCaK * d * (fp * (1.0 - nca) + jca * fcap * nca);

    /* IKr, TPORd.cc:654-678 */
    double xrss = 1.0 / (1.0 + exp((-(v + 8.337)) / 6.789));
    double txrf = 12.98 + 1.0 / (0.3652 * exp((v - 31.66) / 3.869) + 4.123e-5 * exp((-(v - 47.78)) / 20.38));
    double txrs = 1.865 + 1.0 / (0.06629 * exp((v - 34.70) / 7.355) + 1.128e-5 * exp((-(v - 29.74)) / 25.94));
    double Axrf = 1.0 / (1.0 + exp((v + 54.81) / 38.21));
    double Axrs = 1.0 - Axrf;
    xrf = xrss - (xrss - xrf) * exp(-dt / txrf);
    xrs = xrss - (xrss - xrs) * exp(-dt / txrs);
    double xr = Axrf * xrf + Axrs * xrs;
    double rkr = 1.0 / (1.0 + exp((v + 55.0) / 75.0)) * 1.0 / (1.0 + exp((v - 10.0) / 30.0));
    double GKr = 0.046;
    if (is_epi) GKr *= 1.3;
    if (is_mid) GKr *= 0.8;
    double IKr = GKr * sqrt(ko / 5.4) * xr * rkr * (v - EK);

    /* IKs with LQT1 / SUPREP / ISO1 factors, TPORd.cc:680-735 */
    double xs1ss = 1.0 / (1.0 + exp((-(v + 11.60)) / 8.932));
    double txs1 = 817.3 + 1.0 / (2.326e-4 * exp((v + 48.28) / 17.80) + 0.001292 * exp((-(v + 210.0)) / 230.0));
    xs1 = xs1ss - (xs1ss - xs1) * exp(-dt / txs1);
    double xs2ss = xs1ss;
    double txs2 = 1.0 / (0.01 * exp((v - 50.0) / 20.0) + 0.0193 * exp((-(v + 66.54)) / 31.0));
    xs2 = xs2ss - (xs2ss - xs2) * exp(-dt / txs2);
    double KsCa = 1.0 + 0.6 / (1.0 + pow(3.8e-5 / cai, 1.4));
    double GKs = 0.0034 * 1;
    if (is_epi) GKs *= 1.4;
    GKs = m->gks_scale * GKs;
    if (m->suprep_dose > 0.0) {
        double dose = m->suprep_dose;
        double GKs_sup = GKs;
        double GKs_rep = is_epi ? 1.4 * 0.0034 : 0.0034;
        double frac_wt = 1.0;
        if (dose >= 25)
            frac_wt = 3.129 * pow(dose, -0.560);
        else
            frac_wt = pow(0.974, dose);
        double frac_shIMM = 2.018 * (1.0 - exp(-2.0 * dose * 0.0059)) / (1.0 + exp(-2.0 * dose * 0.0059));
        GKs = frac_wt * GKs_sup + frac_shIMM * GKs_rep;
    }
    GKs *= m->gks_iso_scale;
    double IKs = GKs * KsCa * xs1 * xs2 * (v - EKs);

    /* IK1, TPORd.cc:738-751 */
    double xk1ss = 1.0 / (1.0 + exp(-(v + 2.5538 * ko + 144.59) / (1.5692 * ko + 3.8115)));
    double txk1 = 122.2 / (exp((-(v + 127.2)) / 20.36) + exp((v + 236.8) / 69.33));
    xk1 = xk1ss - (xk1ss - xk1) * exp(-dt / txk1);
    double rk1 = 1.0 / (1.0 + exp((v + 105.8 - 2.6 * ko) / 9.493));
    double GK1 = 0.1908;
    if (is_epi) GK1 *= 1.2;
    if (is_mid) GK1 *= 1.3;
    double IK1 = GK1 * sqrt(ko) * rk1 * xk1 * (v - EK);

    /* INaCa_i and INaCa_ss, TPORd.cc:753-852 */
    double kna1 = 15.0, kna2 = 5.0, kna3 = 88.12, kasymm = 12.5;
    double wna = 6.0e4, wca = 6.0e4, wnaca = 5.0e3;
    double kcaon = 1.5e6, kcaoff = 5.0e3, qna = 0.5224, qca = 0.1670;
    double hca = exp((qca * v * F) / (R * T));
    double hna = exp((qna * v * F) / (R * T));
    double Gncx = 0.0008;
    if (is_epi) Gncx *= 1.1;
    if (is_mid) Gncx *= 1.4;
    double zna = 1.0;
    double INaCa_i, INaCa_ss;
    for (int pass = 0; pass < 2; ++pass) {
        /* pass 0: myoplasm (nai, cai); pass 1: subspace (nass, cass) */
        double na = pass == 0 ? nai : nass;
        double ca = pass == 0 ? cai : cass;
        double h1 = 1 + na / kna3 * (1 + hna);
        double h2 = (na * hna) / (kna3 * h1);
        double h3 = 1.0 / h1;
        double h4 = 1.0 + na / kna1 * (1 + na / kna2);
        double h5 = na * na / (h4 * kna1 * kna2);
        double h6 = 1.0 / h4;
        double h7 = 1.0 + nao / kna3 * (1.0 + 1.0 / hna);
        double h8 = nao / (kna3 * hna * h7);
        double h9 = 1.0 / h7;
        double h10 = kasymm + 1.0 + nao / kna1 * (1.0 + nao / kna2);
        double h11 = nao * nao / (h10 * kna1 * kna2);
        double h12 = 1.0 / h10;
        double k1 = h12 * cao * kcaon;
        double k2 = kcaoff;
        double k3p = h9 * wca;
        double k3pp = h8 * wnaca;
        double k3 = k3p + k3pp;
        double k4p = h3 * wca / hca;
        double k4pp = h2 * wnaca;
        double k4 = k4p + k4pp;
        double k5 = kcaoff;
        double k6 = h6 * ca * kcaon;
        double k7 = h5 * h2 * wna;
        double k8 = h8 * h11 * wna;
        double x1 = k2 * k4 * (k7 + k6) + k5 * k7 * (k2 + k3);
        double x2 = k1 * k7 * (k4 + k5) + k4 * k6 * (k1 + k8);
        double x3 = k1 * k3 * (k7 + k6) + k8 * k6 * (k2 + k3);
        double x4 = k2 * k8 * (k4 + k5) + k3 * k5 * (k1 + k8);
        double E1 = x1 / (x1 + x2 + x3 + x4);
        double E2 = x2 / (x1 + x2 + x3 + x4);
        double E3 = x3 / (x1 + x2 + x3 + x4);
        double E4 = x4 / (x1 + x2 + x3 + x4);
        double KmCaAct = 150.0e-6;
        double allo = 1.0 / (1.0 + pow(KmCaAct / ca, 2.0));
        double JncxNa = 3.0 * (E4 * k7 - E1 * k8) + E3 * k4pp - E2 * k3pp;
        double JncxCa = E2 * k2 - E1 * k1;
        if (pass == 0)
            INaCa_i = 0.8 * Gncx * allo * (zna * JncxNa + zca * JncxCa);
        else
            INaCa_ss = 0.2 * Gncx * allo * (zna * JncxNa + zca * JncxCa);
    }
    double INaCa = INaCa_i + INaCa_ss;

    /* INaK, TPORd.cc:854-906 */
    double k1p = 949.5, k1m = 182.4, k2p = 687.2, k2m = 39.4;
    double k3p = 1899.0, k3m = 79300.0, k4p = 639.0, k4m = 40.0;
    double Knai0 = 9.073, Knao0 = 27.78, delta = -0.1550;
    double Knai = Knai0 * exp((delta * v * F) / (3.0 * R * T));
    double Knao = Knao0 * exp(((1.0 - delta) * v * F) / (3.0 * R * T));
    double Kki = 0.5, Kko = 0.3582, MgADP = 0.05, MgATP = 9.8, Kmgatp = 1.698e-7;
    double H = 1.0e-7, eP = 4.2, Khp = 1.698e-7, Knap = 224.0, Kxkur = 292.0;
    double P = eP / (1.0 + H / Khp + nai / Knap + ki / Kxkur);
    double a1 = (k1p * pow(nai / Knai, 3.0)) / (pow(1.0 + nai / Knai, 3.0) + pow(1.0 + ki / Kki, 2.0) - 1.0);
    double b1 = k1m * MgADP;
    double a2 = k2p;
    double b2 = (k2m * pow(nao / Knao, 3.0)) / (pow(1.0 + nao / Knao, 3.0) + pow(1.0 + ko / Kko, 2.0) - 1.0);
    double a3 = (k3p * pow(ko / Kko, 2.0)) / (pow(1.0 + nao / Knao, 3.0) + pow(1.0 + ko / Kko, 2.0) - 1.0);
    double b3 = (k3m * P * H) / (1.0 + MgATP / Kmgatp);
    double a4 = (k4p * MgATP / Kmgatp) / (1.0 + MgATP / Kmgatp);
    double b4 = (k4m * pow(ki / Kki, 2.0)) / (pow(1.0 + nai / Knai, 3.0) + pow(1.0 + ki / Kki, 2.0) - 1.0);
    double y1 = a4 * a1 * a2 + b2 * b4 * b3 + a2 * b4 * b3 + b3 * a1 * a2;
    double y2 = b2 * b1 * b4 + a1 * a2 * a3 + a3 * b1 * b4 + a2 * a3 * b4;
    double y3 = a2 * a3 * a4 + b3 * b2 * b1 + b2 * b1 * a4 + a3 * a4 * b1;
    double y4 = b4 * b3 * b2 + a3 * a4 * a1 + b2 * a4 * a1 + b3 * b2 * a1;
    double E1 = y1 / (y1 + y2 + y3 + y4);
    double E2 = y2 / (y1 + y2 + y3 + y4);
    double E3 = y3 / (y1 + y2 + y3 + y4);
    double E4 = y4 / (y1 + y2 + y3 + y4);
    double zk = 1.0;
    double JnakNa = 3.0 * (E1 * a3 - E2 * b3);
    double JnakK = 2.0 * (E4 * b1 - E3 * a1);
    double Pnak = 30;
    if (is_epi) Pnak *= 0.9;
    if (is_mid) Pnak *= 0.7;
    double INaK = Pnak * (zna * JnakNa + zk * JnakK);

    /* background currents and pump, TPORd.cc:908-923 */
    double xkb = 1.0 / (1.0 + exp(-(v - 14.48) / 18.34));
    double GKb = 0.003;
    if (is_epi) GKb *= 0.6;
    double IKb = GKb * xkb * (v - EK);
    double PNab = 3.75e-10;
    double INab = PNab * vffrt * (nai * exp(vfrt) - nao) / (exp(vfrt) - 1.0);
    double PCab = 2.5e-8;
    double ICab = PCab * 4.0 * vffrt * (cai * exp(2.0 * vfrt) - 0.341 * cao) / (exp(2.0 * vfrt) - 1.0);
    double GpCa = 0.0005;
    double IpCa = GpCa * cai / (0.0005 + cai);

    /* membrane potential, TPORd.cc:927-935 */
    double Iion = INa + INaL + Ito + ICaL + ICaNa + ICaK + IKr + IKs + IK1 + INaCa + INaK + INab + IKb + IpCa + ICab;
    double dV_dt = -1.0 * (Iion + Ist);
    v += (dV_dt + dVgap_dt) * dt;

    /* CaMK and fluxes, TPORd.cc:939-995 (CaMKa is unchanged by its recompute
       at :939-940 because cass and CaMKt still hold their old values) */
    double CaMKb2 = CaMKo * (1.0 - CaMKt) / (1.0 + KmCaM / cass);
    CaMKt += dt * (aCaMK * CaMKb2 * (CaMKb2 + CaMKt) - bCaMK * CaMKt);
    double JdiffNa = (nass - nai) / 2.0;
    double JdiffK = (kss - ki) / 2.0;
    double Jdiff = (cass - cai) / 0.2;
    double bt = 4.75;
    double a_rel = 0.5 * bt;
    double Jrel_inf = a_rel * (-ICaL) / (1.0 + pow(1.5 / cajsr, 8.0));
    if (is_mid) Jrel_inf *= 1.7;
    double tau_rel = bt / (1.0 + 0.0123 / cajsr);
    if (tau_rel < 0.005) tau_rel = 0.005;
    Jrelnp = Jrel_inf - (Jrel_inf - Jrelnp) * exp(-dt / tau_rel);
    double btp = 1.25 * bt;
    double a_relp = 0.5 * btp;
    double Jrel_infp = a_relp * (-ICaL) / (1.0 + pow(1.5 / cajsr, 8.0));
    if (is_mid) Jrel_infp *= 1.7;
    double tau_relp = btp / (1.0 + 0.0123 / cajsr);
    if (tau_relp < 0.005) tau_relp = 0.005;
    Jrelp = Jrel_infp - (Jrel_infp - Jrelp) * exp(-dt / tau_relp);
    double fJrelp = (1.0 / (1.0 + KmCaMK / CaMKa));
    double Jrel = (1.0 - fJrelp) * Jrelnp + fJrelp * Jrelp;
    double Jupnp = 0.004375 * cai / (cai + 0.00092);
    double Jupp = 2.75 * 0.004375 * cai / (cai + 0.00092 - 0.00017);
    if (is_epi) {
        Jupnp *= 1.3;
        Jupp *= 1.3;
    }
    double fJupp = (1.0 / (1.0 + KmCaMK / CaMKa));
    double Jleak = 0.0039375 * cansr / 15.0;
    double Jup = (1.0 - fJupp) * Jupnp + fJupp * Jupp - Jleak;
    double Jtr = (cansr - cajsr) / 100.0;

    /* concentrations, forward Euler, TPORd.cc:997-1020 */
    nai += dt * (-(INa + INaL + 3.0 * INaCa_i + 3.0 * INaK + INab) * Acap / (F * vmyo) + JdiffNa * vss / vmyo);
    nass += dt * (-(ICaNa + 3.0 * INaCa_ss) * Acap / (F * vss) - JdiffNa);
    ki += dt * (-(Ito + IKr + IKs + IK1 + IKb + Ist - 2.0 * INaK) * Acap / (F * vmyo) + JdiffK * vss / vmyo);
    kss += dt * (-(ICaK)*Acap / (F * vss) - JdiffK);
    double Bcai;
    if (is_epi)
        Bcai = 1.0 / (1.0 + 1.3 * cmdnmax * kmcmdn / pow(kmcmdn + cai, 2.0) + trpnmax * kmtrpn / pow(kmtrpn + cai, 2.0));
    else
        Bcai = 1.0 / (1.0 + cmdnmax * kmcmdn / pow(kmcmdn + cai, 2.0) + trpnmax * kmtrpn / pow(kmtrpn + cai, 2.0));
    cai += dt * (Bcai * (-(IpCa + ICab - 2.0 * INaCa_i) * Acap / (2.0 * F * vmyo) - Jup * vnsr / vmyo + Jdiff * vss / vmyo));
    double Bcass = 1.0 / (1.0 + BSRmax * KmBSR / pow(KmBSR + cass, 2.0) + BSLmax * KmBSL / pow(KmBSL + cass, 2.0));
    cass += dt * (Bcass * (-(ICaL - 2.0 * INaCa_ss) * Acap / (2.0 * F * vss) + Jrel * vjsr / vss - Jdiff));
    cansr += dt * (Jup - Jtr * vjsr / vnsr);
    double Bcajsr = 1.0 / (1.0 + csqnmax * kmcsqn / pow(kmcsqn + cajsr, 2.0));
    cajsr += dt * (Bcajsr * (Jtr - Jrel));

    s[LQT_S_V] = v;
    s[LQT_S_NAI] = nai; s[LQT_S_NASS] = nass; s[LQT_S_KI] = ki; s[LQT_S_KSS] = kss;
    s[LQT_S_CAI] = cai; s[LQT_S_CASS] = cass; s[LQT_S_CANSR] = cansr; s[LQT_S_CAJSR] = cajsr;
    s[LQT_S_SM] = sm; s[LQT_S_SH] = sh; s[LQT_S_SJ] = sj;
    s[LQT_S_ML] = mL; s[LQT_S_HL] = hL; s[LQT_S_HLP] = hLp;
    s[LQT_S_A] = a; s[LQT_S_IF] = iF; s[LQT_S_IS] = iS;
    s[LQT_S_AP] = ap; s[LQT_S_IFP] = iFp; s[LQT_S_ISP] = iSp;
    s[LQT_S_D] = d; s[LQT_S_FF] = ff; s[LQT_S_FS] = fs;
    s[LQT_S_FCAF] = fcaf; s[LQT_S_FCAS] = fcas; s[LQT_S_JCA] = jca; s[LQT_S_NCA] = nca;
    s[LQT_S_FFP] = ffp; s[LQT_S_FCAFP] = fcafp;
    s[LQT_S_XRF] = xrf; s[LQT_S_XRS] = xrs; s[LQT_S_XS1] = xs1; s[LQT_S_XS2] = xs2;
    s[LQT_S_XK1] = xk1; s[LQT_S_JRELNP] = Jrelnp; s[LQT_S_JRELP] = Jrelp;
    s[LQT_S_CAMKT] = CaMKt;

    if (aux) {
        aux->dvdt = dV_dt;
        aux->iion = Iion;
        aux->ina = INa; aux->inal = INaL; aux->ito = Ito; aux->ical = ICaL;
        aux->ikr = IKr; aux->iks = IKs; aux->ik1 = IK1; aux->inaca = INaCa;
        aux->inak = INaK;
    }
}

/* ------------------------------------------------------------------------ */
static void set_threads(int nthreads)
{
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
}

void orc_cells_update(int64_t n, double *s, const uint8_t *ctype,
                      const lqt_model *m, double dt, const double *ist,
                      const double *dvgap, int64_t nsteps, int nthreads)
{
    set_threads(nthreads);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        double is = ist ? ist[i] : 0.0;
        double dg = dvgap ? dvgap[i] : 0.0;
        for (int64_t k = 0; k < nsteps; ++k)
            orc_update(s + i * LQT_NSTATE, ctype[i], m, dt, is, dg, NULL);
    }
}

/* nsteps updates of n cells, then the getters of the last update:
 * cur[n][6] = getINa, getICaL, getIKr, getIKs, getIK1, getAbsDvdt
 * (SingleCell/TPORd.cc:358-376; getAbsDvdt is abs(dV_dt) on a double,
 * TPORd.cc:364). */
void orc_cells_currents(int64_t n, double *s, const uint8_t *ctype,
                        const lqt_model *m, double dt, const double *ist,
                        const double *dvgap, int64_t nsteps, double *cur)
{
    for (int64_t i = 0; i < n; ++i) {
        double is = ist ? ist[i] : 0.0;
        double dg = dvgap ? dvgap[i] : 0.0;
        orc_aux a = {0};
        for (int64_t k = 0; k < nsteps; ++k)
            orc_update(s + i * LQT_NSTATE, ctype[i], m, dt, is, dg, &a);
        double *c = cur + 6 * i;
        c[0] = a.ina;
        c[1] = a.ical;
        c[2] = a.ikr;
        c[3] = a.iks;
        c[4] = a.ik1;
        c[5] = fabs(a.dvdt);
    }
}

/* OneD.cc:337-338 */
int orc_in_window(double time, double bcl, double start, double dur)
{
    double tb = time - floor(time / bcl) * bcl;
    return tb >= start && tb < start + dur;
}

/* ------------------------------------------------------------------------ */
/* SingleCell.cc:95-232.  The reference declares its APD tracking variables
 * inside the loop body and relies on them keeping their values between
 * iterations; here they live outside the loop. */
int64_t orc_single_cell_run(int ctype, const lqt_model *m, double v0,
                            double dt, double bcl, double numS1,
                            double stimStart, double stimDuration,
                            double stimStrength, double *stats,
                            int64_t trace_every, double *trace,
                            int64_t trace_cap, double *final_state)
{
    double s[LQT_NSTATE];
    orc_initial_state(v0, s);
    double stopTime = numS1 * bcl;
    double apd20 = 0, apd25 = 0, apd50 = 0, apd75 = 0, apd80 = 0, apd90 = 0;
    double dvdt_max = 0, rest_potential = 0, amplitude = 0, overshoot = 0;
    double oldV = 0, repo20 = 0, repo25 = 0, repo50 = 0, repo75 = 0, repo80 = 0, repo90 = 0;
    int peakfound = 0;
    int64_t ntrace = 0;
    double time;
    int64_t step;
    orc_aux aux;
    for (time = 0.0, step = 0; time < stopTime; time += dt, step++) {
        double ist = orc_in_window(time, bcl, stimStart, stimDuration) ? stimStrength : 0.0;
        orc_update(s, ctype, m, dt, ist, 0.0, &aux);
        double V = s[LQT_S_V];
        double absdvdt = fabs(aux.dvdt);
        if (trace && trace_every > 0 && step % trace_every == 0 && ntrace < trace_cap)
            trace[ntrace++] = V;
        if (floor((time - stimStart) / bcl) == numS1 - 2 &&
            floor((time + dt - stimStart) / bcl) == numS1 - 1) {
            rest_potential = V;
            oldV = V;
            peakfound = 0;
            dvdt_max = -1;
        }
        if (floor((time - stimStart) / bcl) == numS1 - 1) {
            if (V > oldV) {
                oldV = V;
                if (absdvdt > dvdt_max) dvdt_max = absdvdt;
            } else if (V <= oldV && !peakfound) {
                peakfound = 1;
                overshoot = oldV;
                amplitude = overshoot - rest_potential;
                repo20 = overshoot - 0.20 * amplitude;
                repo25 = overshoot - 0.25 * amplitude;
                repo50 = overshoot - 0.50 * amplitude;
                repo75 = overshoot - 0.75 * amplitude;
                repo80 = overshoot - 0.80 * amplitude;
                repo90 = overshoot - 0.90 * amplitude;
                oldV = V;
            } else if (V <= oldV && peakfound) {
                double rel = time - floor(time / bcl) * bcl - stimStart - stimDuration;
                if (oldV >= repo20 && V <= repo20) apd20 = rel;
                else if (oldV >= repo25 && V <= repo25) apd25 = rel;
                else if (oldV >= repo50 && V <= repo50) apd50 = rel;
                else if (oldV >= repo75 && V <= repo75) apd75 = rel;
                else if (oldV >= repo80 && V <= repo80) apd80 = rel;
                else if (oldV >= repo90 && V <= repo90) apd90 = rel;
                oldV = V;
            }
        }
    }
    if (stats) {
        stats[0] = rest_potential; stats[1] = dvdt_max; stats[2] = overshoot;
        stats[3] = amplitude; stats[4] = apd20; stats[5] = apd25; stats[6] = apd50;
        stats[7] = apd75; stats[8] = apd80; stats[9] = apd90;
    }
    if (final_state) memcpy(final_state, s, sizeof(s));
    return ntrace;
}

/* ------------------------------------------------------------------------ */
/* OneD.cc:100-436 */
int64_t orc_strand_run(const orc_strand_cfg *cfg, const uint8_t *ctype,
                       const double *coeff, const lqt_model *m, double v0,
                       int64_t rec_every, double *rec, double *rec_t,
                       int64_t rec_cap, int32_t max_beats, double *act,
                       double *cv_out, double *final_state, int nthreads)
{
    const int n = cfg->n;
    const double dx = cfg->dx, dt = cfg->dt;
    double *s = (double *)malloc(sizeof(double) * LQT_NSTATE * n);
    double *oldV = (double *)malloc(sizeof(double) * n);
    double *dcoeff = (double *)malloc(sizeof(double) * n);
    int32_t *nact = (int32_t *)calloc(n, sizeof(int32_t));
    if (!s || !oldV || !dcoeff || !nact) {
        free(s); free(oldV); free(dcoeff); free(nact);
        return -1;
    }
    for (int i = 0; i < n; ++i) orc_initial_state(v0, s + i * LQT_NSTATE);
    /* OneD.cc:123-131 */
    for (int i = 0; i < n; ++i) {
        if (n == 1) dcoeff[i] = 0.0;
        else if (i == 0) dcoeff[i] = (coeff[i + 1] - coeff[i]) / dx;
        else if (i == n - 1) dcoeff[i] = (coeff[i] - coeff[i - 1]) / dx;
        else dcoeff[i] = (coeff[i + 1] - coeff[i - 1]) / (2.0 * dx);
    }
    if (act)
        for (int64_t k = 0; k < (int64_t)n * max_beats; ++k) act[k] = -1.0;
    double cvStart = 0, cvEnd = 0;
    int cvStartFlag = 0, cvEndFlag = 0;
    int64_t nrec = 0;
    set_threads(nthreads);

    double time;
    int64_t step;
    for (time = 0.0, step = 0; time <= cfg->stop_time; time += dt, step++) {
        for (int i = 0; i < n; ++i) oldV[i] = s[i * LQT_NSTATE + LQT_S_V];
        const int stim_on = orc_in_window(time, cfg->bcl, cfg->stim_start, cfg->stim_dur);
#pragma omp parallel for schedule(static) if (n >= 64)
        for (int i = 0; i < n; ++i) {
            double ist = (stim_on && i < cfg->n_stim) ? cfg->stim_strength : 0.0;
            double first_order = 0.0, second_order = 0.0;
            /* OneD.cc:371-388, mirrored (no-flux) ends */
            if (n == 1) {
                first_order = 0.0;
                second_order = 0.0;
            } else if (i == 0) {
                first_order = (oldV[i + 1] - oldV[i]) / (1.0 * dx);
                second_order = (oldV[i + 1] + oldV[i] - 2.0 * oldV[i]) / (dx * dx);
            } else if (i < n - 1) {
                first_order = (oldV[i + 1] - oldV[i - 1]) / (2.0 * dx);
                second_order = (oldV[i + 1] + oldV[i - 1] - 2.0 * oldV[i]) / (dx * dx);
            } else {
                first_order = (oldV[i] - oldV[i - 1]) / (1.0 * dx);
                second_order = (oldV[i] + oldV[i - 1] - 2.0 * oldV[i]) / (dx * dx);
            }
            double dVgap_dt = dcoeff[i] * first_order + coeff[i] * second_order;
            orc_update(s + i * LQT_NSTATE, ctype[i], m, dt, ist, dVgap_dt, NULL);
        }
        /* activation crossings (upward through act_thr) */
        if (act) {
            for (int i = 0; i < n; ++i) {
                double vn = s[i * LQT_NSTATE + LQT_S_V];
                if (oldV[i] < cfg->act_thr && vn >= cfg->act_thr && nact[i] < max_beats)
                    act[(int64_t)i * max_beats + nact[i]++] = time;
            }
        }
        /* OneD.cc:402-415 */
        if (rec && rec_every > 0 && step % rec_every == 0 && nrec < rec_cap) {
            for (int i = 0; i < n; ++i) rec[nrec * n + i] = s[i * LQT_NSTATE + LQT_S_V];
            if (rec_t) rec_t[nrec] = time;
            nrec++;
        }
        /* OneD.cc:419-436 */
        if (n > 90 && floor(time / cfg->bcl) == cfg->num_s1) {
            if (s[10 * LQT_NSTATE + LQT_S_V] >= cfg->act_thr && cvStartFlag == 0) {
                cvStart = time;
                cvStartFlag = 1;
            }
            if (s[90 * LQT_NSTATE + LQT_S_V] >= cfg->act_thr && cvEndFlag == 0) {
                cvEnd = time;
                cvEndFlag = 1;
            }
        }
    }
    if (cv_out) {
        if (cvStartFlag && cvEndFlag) {
            cv_out[0] = (dx * 80) / (cvEnd - cvStart);
            cv_out[1] = cvStart;
            cv_out[2] = cvEnd;
        } else {
            cv_out[0] = cv_out[1] = cv_out[2] = NAN;
        }
    }
    if (final_state) memcpy(final_state, s, sizeof(double) * LQT_NSTATE * n);
    free(s); free(oldV); free(dcoeff); free(nact);
    return nrec;
}

/* OneD_VW.cc:199-349 (see lqt_oracle.h). */
int64_t orc_vw_trial(const orc_strand_cfg *cfg, const uint8_t *ctype,
                     const double *coeff, const lqt_model *m, double v0,
                     double s2_time, double s2_dur, double s2_strength,
                     int32_t s2_cell0, int32_t s2_ncells, double *max_endo,
                     double *max_epi, double *rec, int64_t rec_cap)
{
    const int n = cfg->n;
    const double dx = cfg->dx, dt = cfg->dt;
    const double s2_base = (cfg->num_s1 - 1) * cfg->bcl;
    double *s = (double *)malloc(sizeof(double) * LQT_NSTATE * n);
    double *oldV = (double *)malloc(sizeof(double) * n);
    double *dcoeff = (double *)malloc(sizeof(double) * n);
    if (!s || !oldV || !dcoeff) {
        free(s); free(oldV); free(dcoeff);
        return -1;
    }
    for (int i = 0; i < n; ++i) orc_initial_state(v0, s + i * LQT_NSTATE);
    for (int i = 0; i < n; ++i) {
        if (n == 1) dcoeff[i] = 0.0;
        else if (i == 0) dcoeff[i] = (coeff[i + 1] - coeff[i]) / dx;
        else if (i == n - 1) dcoeff[i] = (coeff[i] - coeff[i - 1]) / dx;
        else dcoeff[i] = (coeff[i + 1] - coeff[i - 1]) / (2.0 * dx);
    }
    double mendo = -100.0, mepi = -100.0;
    int64_t nrec = 0;
    double time;
    int64_t step;
    for (time = 0.0, step = 0; time <= cfg->stop_time; time += dt, step++) {
        for (int i = 0; i < n; ++i) oldV[i] = s[i * LQT_NSTATE + LQT_S_V];
        const int s1 = orc_in_window(time, cfg->bcl, cfg->stim_start, cfg->stim_dur);
        const int s2 = !s1 && time - s2_base >= s2_time && time - s2_base < s2_time + s2_dur;
#pragma omp parallel for schedule(static) if (n >= 64)
        for (int i = 0; i < n; ++i) {
            double ist = 0.0;
            if (s1 && i < cfg->n_stim) ist = cfg->stim_strength;
            else if (s2 && i >= s2_cell0 && i < s2_cell0 + s2_ncells) ist = s2_strength;
            double fo, so;
            if (n == 1) {
                fo = so = 0.0;
            } else if (i == 0) {
                fo = (oldV[i + 1] - oldV[i]) / (1.0 * dx);
                so = (oldV[i + 1] + oldV[i] - 2.0 * oldV[i]) / (dx * dx);
            } else if (i < n - 1) {
                fo = (oldV[i + 1] - oldV[i - 1]) / (2.0 * dx);
                so = (oldV[i + 1] + oldV[i - 1] - 2.0 * oldV[i]) / (dx * dx);
            } else {
                fo = (oldV[i] - oldV[i - 1]) / (1.0 * dx);
                so = (oldV[i] + oldV[i - 1] - 2.0 * oldV[i]) / (dx * dx);
            }
            orc_update(s + i * LQT_NSTATE, ctype[i], m, dt, ist, dcoeff[i] * fo + coeff[i] * so, NULL);
        }
        if (rec && floor(time / cfg->bcl) == cfg->num_s1 - 1 && step % 50 == 0 && nrec < rec_cap) {
            for (int i = 0; i < n; ++i) rec[nrec * n + i] = s[i * LQT_NSTATE + LQT_S_V];
            nrec++;
        }
        if (time - s2_base >= s2_time) {
            if (s[(n - 1) * LQT_NSTATE + LQT_S_V] >= mepi) mepi = s[(n - 1) * LQT_NSTATE + LQT_S_V];
            if (s[LQT_S_V] >= mendo) mendo = s[LQT_S_V];
        }
    }
    if (max_endo) *max_endo = mendo;
    if (max_epi) *max_epi = mepi;
    free(s); free(oldV); free(dcoeff);
    return nrec;
}

/* The device AP detector restated in FP64 (see lqt_oracle.h). */
typedef struct {
    double vrest, vpeak, dvdt_max, t_act;
    int phase, ead;
} orc_det;

enum { DET_IDLE = 0, DET_WAIT = 1, DET_RISE = 2, DET_FALL = 3, DET_DONE = 4 };

int64_t orc_strand_detect(const orc_strand_cfg *cfg, int32_t s1_beats, const uint8_t *ctype, const double *coeff,
                          const lqt_model *m, double v0, int32_t max_beats, double *t_act, double *apd90,
                          uint8_t *ead, int32_t *nact, double *final_state)
{
    const int n = cfg->n;
    const double dx = cfg->dx, dt = cfg->dt;
    double *s = (double *)malloc(sizeof(double) * LQT_NSTATE * n);
    double *oldV = (double *)malloc(sizeof(double) * n);
    double *dcoeff = (double *)malloc(sizeof(double) * n);
    orc_det *det = (orc_det *)calloc(n, sizeof(orc_det));
    if (!s || !oldV || !dcoeff || !det) {
        free(s); free(oldV); free(dcoeff); free(det);
        return -1;
    }
    for (int i = 0; i < n; ++i) orc_initial_state(v0, s + i * LQT_NSTATE);
    for (int i = 0; i < n; ++i) {
        if (n == 1) dcoeff[i] = 0.0;
        else if (i == 0) dcoeff[i] = (coeff[i + 1] - coeff[i]) / dx;
        else if (i == n - 1) dcoeff[i] = (coeff[i] - coeff[i - 1]) / dx;
        else dcoeff[i] = (coeff[i + 1] - coeff[i - 1]) / (2.0 * dx);
        nact[i] = 0;
        ead[i] = 0;
    }
    for (int64_t k = 0; k < (int64_t)n * max_beats; ++k) t_act[k] = apd90[k] = -1.0;
    int prev_on = 0;
    double time;
    int64_t step;
    for (time = 0.0, step = 0; time <= cfg->stop_time; time += dt, step++) {
        const int on = orc_in_window(time, cfg->bcl, cfg->stim_start, cfg->stim_dur) &&
                       (s1_beats <= 0 || floor(time / cfg->bcl) < s1_beats);
        const int opened = on && !prev_on;
        prev_on = on;
        for (int i = 0; i < n; ++i) oldV[i] = s[i * LQT_NSTATE + LQT_S_V];
        for (int i = 0; i < n; ++i) {
            double ist = (on && i < cfg->n_stim) ? cfg->stim_strength : 0.0;
            double fo = 0.0, so = 0.0;
            if (n > 1) {
                if (i == 0) {
                    fo = (oldV[1] - oldV[0]) / (1.0 * dx);
                    so = (oldV[1] + oldV[0] - 2.0 * oldV[0]) / (dx * dx);
                } else if (i < n - 1) {
                    fo = (oldV[i + 1] - oldV[i - 1]) / (2.0 * dx);
                    so = (oldV[i + 1] + oldV[i - 1] - 2.0 * oldV[i]) / (dx * dx);
                } else {
                    fo = (oldV[i] - oldV[i - 1]) / (1.0 * dx);
                    so = (oldV[i] + oldV[i - 1] - 2.0 * oldV[i]) / (dx * dx);
                }
            }
            orc_aux aux;
            orc_update(s + i * LQT_NSTATE, ctype[i], m, dt, ist, dcoeff[i] * fo + coeff[i] * so, &aux);
            const double vo = oldV[i], vn = s[i * LQT_NSTATE + LQT_S_V];
            orc_det *d = &det[i];
            if (opened) {
                d->vrest = vo;
                d->vpeak = vo;
                d->dvdt_max = 0;
                d->phase = DET_WAIT;
                d->ead = 0;
            }
            if (d->phase == DET_WAIT) {
                if (vo < cfg->act_thr && vn >= cfg->act_thr) {
                    d->phase = DET_RISE;
                    d->vpeak = vn;
                    d->t_act = time;
                    if (nact[i] < max_beats) t_act[(int64_t)i * max_beats + nact[i]] = time;
                    nact[i]++;
                }
            } else if (d->phase == DET_RISE) {
                if (vn > vo) d->vpeak = vn;
                else {
                    d->vpeak = vo;
                    d->phase = DET_FALL;
                }
            } else if (d->phase == DET_FALL) {
                const double amp = d->vpeak - d->vrest;
                const double thr90 = d->vpeak - 0.9 * amp, thr50 = d->vpeak - 0.5 * amp;
                if (vn <= thr90 && vo >= thr90) {
                    d->phase = DET_DONE;
                    if (nact[i] - 1 < max_beats) apd90[(int64_t)i * max_beats + nact[i] - 1] = time - d->t_act;
                    if (d->ead) ead[i] = 1;
                } else if (vo < thr50 && vn > vo + 1e-3) {
                    d->ead = 1;
                }
            }
        }
    }
    if (final_state) memcpy(final_state, s, sizeof(double) * LQT_NSTATE * n);
    free(s); free(oldV); free(dcoeff); free(det);
    return step;
}

/* PlotScript/plot1DECG_compare.py:89-105 */
double orc_ecg_1d(int32_t n, const double *v, double dx, double x0)
{
    double fai = 0.0;
    for (int i = 0; i < n; ++i) {
        double r = i * dx - x0;
        if (i == 0)
            fai += -(v[i + 1] - v[i]) / (r * r);
        else if (i == n - 1)
            fai += -(v[i] - v[i - 1]) / (r * r);
        else
            fai += -(v[i + 1] - v[i - 1]) / (2 * r * r);
    }
    return fai;
}

/* ------------------------------------------------------------------------ */
/* Grids.  Index of voxel (x, y, z) is (x*ny + y)*nz + z (GPU3D.cu:29-33). */
static inline int64_t gidx(int32_t ny, int32_t nz, int64_t x, int64_t y, int64_t z)
{
    return (x * ny + y) * nz + z;
}

/* Mirror map: GPU3D.cu:1487-1604 (3D, 26 neighbours) and new_11.cu:1535-1640
 * (2D, 8 neighbours; used when nz == 1).  The outward normal is a weighted
 * occupancy sum (weights 1, 1/sqrt2, 1/sqrt3) accumulated in the reference's
 * term order (the order decides last-bit ties in the nearest-voxel search),
 * scaled by its largest component; the boundary voxel then mirrors the
 * tissue neighbour nearest to that direction (first strict minimum in z, y, x
 * loop order). */

/* Neighbour slot k (1..26) of GPU3D.cu:1492-1544 -> offset (dx, dy, dz). */
static void slot3(int k, int *ox, int *oy, int *oz)
{
    int j = k <= 13 ? k - 1 : k;          /* skip the centre (x,y,z) */
    *ox = j / 9 - 1;
    *oy = (j / 3) % 3 - 1;
    *oz = j % 3 - 1;
}
/* Slot k (1..8) of new_11.cu:1544-1565: | 1 2 3 | 4 s 5 | 6 7 8 | (x right, y down). */
static void slot2(int k, int *ox, int *oy)
{
    static const int tx[9] = {0, -1, 0, 1, -1, 1, -1, 0, 1};
    static const int ty[9] = {0, -1, -1, -1, 0, 0, 1, 1, 1};
    *ox = tx[k];
    *oy = ty[k];
}
/* Terms of il (x), ir (y), ic (z) as {slot, weight kind (1, 2 = 1/sqrt2,
 * 3 = 1/sqrt3), sign}, in source order: GPU3D.cu:1566-1570, new_11.cu:1583-1586. */
static const int8_t ic3[18][3] = {{3,3,1},{1,3,-1},{6,2,1},{9,3,1},{7,3,-1},{4,2,-1},{12,2,1},{10,2,-1},{14,1,1},
                                  {17,2,1},{15,2,-1},{13,1,-1},{20,3,1},{18,3,-1},{23,2,1},{26,3,1},{24,3,-1},{21,2,-1}};
static const int8_t ir3[18][3] = {{9,3,1},{2,2,-1},{3,3,-1},{1,3,-1},{8,2,1},{7,3,1},{17,2,1},{11,1,-1},{12,2,-1},
                                  {10,2,-1},{16,1,1},{15,2,1},{26,3,1},{19,2,-1},{20,3,-1},{18,3,-1},{25,2,1},{24,3,1}};
static const int8_t il3[18][3] = {{18,3,1},{19,2,1},{20,3,1},{21,2,1},{22,1,1},{23,2,1},{24,3,1},{25,2,1},{26,3,1},
                                  {1,3,-1},{2,2,-1},{3,3,-1},{4,2,-1},{5,1,-1},{6,2,-1},{7,3,-1},{8,2,-1},{9,3,-1}};
static const int8_t il2[6][3] = {{1,2,-1},{3,2,1},{4,1,-1},{5,1,1},{6,2,-1},{8,2,1}};
static const int8_t ir2[6][3] = {{1,2,-1},{2,1,-1},{3,2,-1},{6,2,1},{7,1,1},{8,2,1}};

static double occ_sum(const int8_t (*terms)[3], int nterms, const int *gg,
                      double root2, double root3)
{
    double acc = 0.0;
    for (int t = 0; t < nterms; ++t) {
        int g = gg[terms[t][0]];
        double term = terms[t][1] == 1 ? (double)g : (terms[t][1] == 2 ? g / root2 : g / root3);
        acc = terms[t][2] > 0 ? acc + term : acc - term;
    }
    return acc;
}

int64_t orc_build_map(int32_t nx, int32_t ny, int32_t nz, const uint8_t *grid,
                      int32_t *tissue_of)
{
    const int64_t total = (int64_t)nx * ny * nz;
    int64_t nt = 0;
    for (int64_t i = 0; i < total; ++i)
        tissue_of[i] = (grid[i] != LQT_EMPTY) ? (int32_t)(nt++) : INT32_MIN;
    const int is2d = (nz == 1);
    const double root2 = sqrt(2.0), root3 = sqrt(3.0);
#define TISSUE(xx, yy, zz) ((xx) >= 0 && (xx) < nx && (yy) >= 0 && (yy) < ny && (zz) >= 0 && (zz) < nz && \
                            grid[gidx(ny, nz, (xx), (yy), (zz))] != LQT_EMPTY)
    for (int32_t x = 0; x < nx; ++x)
        for (int32_t y = 0; y < ny; ++y)
            for (int32_t z = 0; z < nz; ++z) {
                int64_t id = gidx(ny, nz, x, y, z);
                if (grid[id] != LQT_EMPTY) continue;
                int gg[27] = {0};
                int isbound = 0;
                int nslots = is2d ? 8 : 26;
                for (int k = 1; k <= nslots; ++k) {
                    int ox, oy, oz = 0;
                    if (is2d) slot2(k, &ox, &oy);
                    else slot3(k, &ox, &oy, &oz);
                    gg[k] = TISSUE(x + ox, y + oy, z + oz) ? 1 : 0;
                    isbound += gg[k];
                }
                if (isbound == 0) continue;
                double il, ir, ic = 0.0;
                if (is2d) {
                    il = occ_sum(il2, 6, gg, root2, root3);
                    ir = occ_sum(ir2, 6, gg, root2, root3);
                } else {
                    ic = occ_sum(ic3, 18, gg, root2, root3);
                    ir = occ_sum(ir3, 18, gg, root2, root3);
                    il = occ_sum(il3, 18, gg, root2, root3);
                }
                double imax = fabs(is2d ? il : ic);
                if (is2d) {
                    if (fabs(ir) > imax) imax = fabs(ir);
                } else {
                    if (fabs(ir) > imax) imax = fabs(ir);
                    if (fabs(il) > imax) imax = fabs(il);
                }
                double n0 = il / imax, n1 = ir / imax, n2 = is2d ? 0.0 : ic / imax;
                if (imax - 0 < 0.0001) n0 = n1 = n2 = 0.0;
                double dislow = 1000;
                int bx = 0, by = 0, bz = 0;
                for (int zc = is2d ? 0 : -1; zc <= (is2d ? 0 : 1); ++zc)
                    for (int yc = -1; yc <= 1; ++yc)
                        for (int xc = -1; xc <= 1; ++xc) {
                            double dis = is2d
                                ? sqrt(1.0 * (xc - n0) * (xc - n0) + (yc - n1) * (yc - n1))
                                : sqrt(1.0 * (xc - n0) * (xc - n0) + (yc - n1) * (yc - n1) + (zc - n2) * (zc - n2));
                            if (TISSUE(x + xc, y + yc, z + zc) && dis < dislow) {
                                bx = xc; by = yc; bz = zc;
                                dislow = dis;
                            }
                        }
                tissue_of[id] = -(tissue_of[gidx(ny, nz, x + bx, y + by, z + bz)] + 1);
            }
#undef TISSUE
    return nt;
}

void orc_build_tensor(int32_t nx, int32_t ny, int32_t nz, double dx,
                      const int32_t *tissue_of, const int64_t *tissue_cell,
                      int64_t ntissue, const float *fibre, double d_f,
                      double d_t, double *d6, double *b3)
{
    const double dd = d_f - d_t;
    for (int64_t k = 0; k < ntissue; ++k) {
        int64_t g = tissue_cell[k];
        double f0 = 0, f1 = 0, f2 = 0;
        if (fibre) {
            f0 = fibre[3 * g];
            f1 = fibre[3 * g + 1];
            f2 = fibre[3 * g + 2];
        }
        double dt_ = fibre ? d_t : d_f;
        double ddd = fibre ? dd : 0.0;
        d6[6 * k + 0] = dt_ + ddd * f0 * f0;
        d6[6 * k + 1] = dt_ + ddd * f1 * f1;
        d6[6 * k + 2] = dt_ + ddd * f2 * f2;
        d6[6 * k + 3] = ddd * f0 * f1;
        d6[6 * k + 4] = ddd * f0 * f2;
        d6[6 * k + 5] = ddd * f1 * f2;
    }
    /* divergence of D: b_j = sum_i dD_ij/dx_i.  Component map for D_ij. */
    static const int comp[3][3] = {{0, 3, 4}, {3, 1, 5}, {4, 5, 2}};
    const int64_t stride[3] = {(int64_t)ny * nz, nz, 1};
    const int32_t dims[3] = {nx, ny, nz};
    for (int64_t k = 0; k < ntissue; ++k) {
        int64_t g = tissue_cell[k];
        int64_t c[3] = {g / ((int64_t)ny * nz), (g / nz) % ny, g % nz};
        double b[3] = {0, 0, 0};
        for (int i = 0; i < 3; ++i) {
            if (dims[i] == 1) continue;
            int32_t tp = (c[i] + 1 < dims[i]) ? tissue_of[g + stride[i]] : INT32_MIN;
            int32_t tm = (c[i] - 1 >= 0) ? tissue_of[g - stride[i]] : INT32_MIN;
            for (int j = 0; j < 3; ++j) {
                int cc = comp[i][j];
                double der;
                if (tp >= 0 && tm >= 0) der = (d6[6 * (int64_t)tp + cc] - d6[6 * (int64_t)tm + cc]) / (2 * dx);
                else if (tp >= 0) der = (d6[6 * (int64_t)tp + cc] - d6[6 * k + cc]) / dx;
                else if (tm >= 0) der = (d6[6 * k + cc] - d6[6 * (int64_t)tm + cc]) / dx;
                else der = 0;
                b[j] += der;
            }
        }
        b3[3 * k + 0] = b[0];
        b3[3 * k + 1] = b[1];
        b3[3 * k + 2] = b[2];
    }
}

/* V of grid voxel g: tissue -> its V; mirrored boundary -> V of the mapped
 * tissue voxel (GPU3D.cu:258-308). */
static inline double vget(const int32_t *tissue_of, const double *state, int64_t g)
{
    int32_t t = tissue_of[g];
    if (t >= 0) return state[(int64_t)t * LQT_NSTATE];
    if (t != INT32_MIN) return state[(int64_t)(-t - 1) * LQT_NSTATE];
    return -90.0;
}

/* Anisotropic diffusion: new_11.cu:352-417 generalised to 3D,
 * du = sum_i D_ii V_ii + 2 sum_{i<j} D_ij V_ij + sum_j b_j V_j. */
static double grid_du(int32_t nx, int32_t ny, int32_t nz, double dx,
                      const int32_t *tissue_of, int64_t g, int64_t k,
                      const double *d6, const double *b3, const double *state)
{
    (void)nx;
    const int64_t st[3] = {(int64_t)ny * nz, nz, 1};
    const int active[3] = {nx > 1, ny > 1, nz > 1};
    double vc = vget(tissue_of, state, g);
    double du = 0.0;
    double grad[3] = {0, 0, 0};
    for (int i = 0; i < 3; ++i) {
        if (!active[i]) continue;
        double vp = vget(tissue_of, state, g + st[i]);
        double vm = vget(tissue_of, state, g - st[i]);
        du += d6[6 * k + i] * ((vm + vp - 2 * vc) / (dx * dx));
        grad[i] = (vp - vm) / (2 * dx);
    }
    static const int pairs[3][3] = {{0, 1, 3}, {0, 2, 4}, {1, 2, 5}};
    for (int p = 0; p < 3; ++p) {
        int i = pairs[p][0], j = pairs[p][1], c = pairs[p][2];
        if (!active[i] || !active[j]) continue;
        double vpp = vget(tissue_of, state, g + st[i] + st[j]);
        double vmm = vget(tissue_of, state, g - st[i] - st[j]);
        double vmp = vget(tissue_of, state, g - st[i] + st[j]);
        double vpm = vget(tissue_of, state, g + st[i] - st[j]);
        du += 2 * (d6[6 * k + c] * ((vpp + vmm - vmp - vpm) / (4 * dx * dx)));
    }
    du += b3[3 * k + 0] * grad[0] + b3[3 * k + 1] * grad[1] + b3[3 * k + 2] * grad[2];
    return du;
}

void orc_grid_step(int32_t nx, int32_t ny, int32_t nz, double dx,
                   const int32_t *tissue_of, const int64_t *tissue_cell,
                   int64_t ntissue, const double *d6, const double *b3,
                   double *state, const uint8_t *ctype, const lqt_model *m,
                   double dt, const double *istim, double *du_out,
                   int nthreads)
{
    double *du = du_out ? du_out : (double *)malloc(sizeof(double) * ntissue);
    set_threads(nthreads);
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < ntissue; ++k)
        du[k] = grid_du(nx, ny, nz, dx, tissue_of, tissue_cell[k], k, d6, b3, state);
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < ntissue; ++k)
        orc_update(state + k * LQT_NSTATE, ctype[k], m, dt, istim ? istim[k] : 0.0, du[k], NULL);
    if (!du_out) free(du);
}

double orc_ecg_grid(int32_t nx, int32_t ny, int32_t nz, double dx,
                    const int32_t *tissue_of, const int64_t *tissue_cell,
                    int64_t ntissue, const double *state, const double *r0)
{
    const int64_t st[3] = {(int64_t)ny * nz, nz, 1};
    const int active[3] = {nx > 1, ny > 1, nz > 1};
    double phi = 0.0;
    for (int64_t k = 0; k < ntissue; ++k) {
        int64_t g = tissue_cell[k];
        int64_t c[3] = {g / st[0], (g / nz) % ny, g % nz};
        double r[3], r2 = 0;
        for (int i = 0; i < 3; ++i) {
            r[i] = c[i] * dx - r0[i];
            r2 += r[i] * r[i];
        }
        double inv = 1.0 / (r2 * sqrt(r2));
        double acc = 0;
        for (int i = 0; i < 3; ++i) {
            if (!active[i]) continue;
            double vp = vget(tissue_of, state, g + st[i]);
            double vm = vget(tissue_of, state, g - st[i]);
            acc += 0.5 * (vp - vm) * r[i];
        }
        phi += acc * inv;
    }
    return phi;
}
