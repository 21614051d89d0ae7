/*
 * balance.c - CPU FP64 restatement of the per-cell balance of the reference
 * (updateCell and the routines it contains, source/update_mod.f90) and of the
 * multi-level atom solver equilibrium (source/emission_mod.f90:2505-3106).
 *
 * TEST INFRASTRUCTURE ONLY: the checker of libmcx.so's balance kernels.
 *
 * Precision: every quantity is carried in FP64 (the reference keeps most in
 * default REAL); constants the reference declares as default REAL are taken at
 * their single-precision values.  The recursions of iterateT and ionBalance
 * are written as loops with the same exit conditions.
 *
 * Where the reference reads outside its arrays (He switched off: elementXref(2)
 * = 0 in ionBalance's convergence test and in compton's recoil heating) the
 * restatement takes the He terms as absent.
 */
#include "oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* exp, log, log10 and pow from the portable FP64 routines that the device's
 * FP64 balance uses too: both sides then round every step alike and every
 * cell takes the same iterateT / ionBalance branches */
#include "mcx_fmath.h"
#define exp(x) mcx_fm_exp(x)
#define log(x) mcx_fm_log(x)
#define log10(x) mcx_fm_log10(x)
#define pow(x, y) mcx_fm_pow((x), (y))

#define R(x) ((double)(x##f))     /* a default-REAL constant of the reference */
#define NEL 30
#define MAXST 32

/* constants_mod.f90:18, :20, :57; update_mod.f90:62-65 */
static const double kBoltz = R(1.380658e-16);
static const double kRyd2erg = R(2.1799e-11);
static const double kHcRyd = R(2.1799153e-11);
static const double kXMax = R(0.99999);

static inline int on(const orc_balance_in* in, int elem) { return in->elem_xref[elem - 1] > 0; }
static inline int xref(const orc_balance_in* in, int elem) { return in->elem_xref[elem - 1]; }
static inline double abun(const orc_balance_in* in, int elem) { return (double)in->elem_abun[elem - 1]; }

/* ------------------------------------------------------------ per-cell state */
typedef struct {
    double te, ne, hden;
    double ion[NEL + 1][MAXST];              /* ionDenUsed(elementXref(elem), ion) at [elem][ion] */
    double alpha[NEL + 1][MAXST];            /* alphaTot */
    double pi1[NEL + 1][MAXST][11];          /* photoIon(1, shell, elem, ion) */
    double pi2[NEL + 1][MAXST][11];          /* photoIon(2, ...) */
    double coll1[NEL + 1][MAXST], coll2[NEL + 1][MAXST];
    double comptonHeat, comptonCool, comptonRecoilHeat;
    int nIterateX;
} cell_t;

/* ----------------------------------------------------------- rate functions */

/* RRbadnell, source/update_mod.f90:2415-2433 */
static double rr_badnell(const orc_balance_in* in, double te, int elem, int nel) {
    const float* t = in->rr_badnell;
#define RB(k) ((double)t[((k) * NEL + (elem - 1)) * (NEL + 1) + nel])
    double A = RB(0), B = RB(1), T0 = RB(2), T1 = RB(3), Cc = RB(4), T2 = RB(5);
#undef RB
    double bbad = B + Cc * exp(-T2 / te);
    return A / (pow(te / T0, 0.5) * pow(1. + pow(te / T0, 0.5), 1. - bbad) * pow(1. + pow(te / T1, 0.5), 1. + bbad));
}

/* DRbadnell, source/update_mod.f90:2435-2450 */
static double dr_badnell(const orc_balance_in* in, double te, int elem, int nel) {
    double dr = 0.;
    for (int idr = 0; idr < 9; ++idr) {
        double E = in->dr_e[((elem - 1) * (NEL + 1) + nel) * 9 + idr];
        double Cc = in->dr_c[((elem - 1) * (NEL + 1) + nel) * 9 + idr];
        if (E / te < 87.) dr = dr + Cc * exp(-E / te);
    }
    return dr * pow(te, -1.5);
}

/* radRecFit, source/update_mod.f90:3094-3202 (Fe I-XV table of :3160-3166) */
static const double kFeFit[3][10] = {
    {R(4.33e-10), R(3.91e-10), R(3.49e-10), R(3.16e-10), R(2.96e-10), R(2.59e-10), R(2.24e-10), R(1.91e-10), R(1.68e-10), R(1.46e-10)},
    {R(0.531), R(0.523), R(0.521), R(0.534), R(0.557), R(0.567), R(0.579), R(0.601), R(0.602), R(0.597)},
    {R(5.77e-02), R(6.15e-02), R(6.22e-02), R(6.02e-02), R(5.79e-02), R(5.65e-02), R(5.49e-02), R(5.10e-02), R(5.07e-02), R(5.22e-02)}};

static double rad_rec_fit(const orc_balance_in* in, double te, int z, int n) {
    if ((n <= 3) || (n == 11) || ((z > 5) && (z < 9)) || (z == 10) || ((z == 26) && (n > 11))) {
        const float* r = &in->rnew[((z - 1) * NEL + (n - 1)) * 4];
        double tt = sqrt(te / (double)r[2]);
        return (double)r[0] / (tt * pow(tt + 1., 1. - (double)r[1]) * pow(1. + sqrt(te / (double)r[3]), 1. + (double)r[1]));
    }
    double tt = te * R(1.e-4);
    if ((z == 26) && (n <= 13))
        return kFeFit[0][n - 4] / pow(tt, kFeFit[1][n - 4] + kFeFit[2][n - 4] * log10(tt));
    const float* r = &in->rrec[((z - 1) * NEL + (n - 1)) * 2];
    return (double)r[0] / pow(tt, (double)r[1]);
}

/* dielectronic, source/update_mod.f90:3204-3305 */
static void dielectronic(const orc_balance_in* in, double te, double diRec[NEL + 1][MAXST]) {
    double t = te > 1000. ? te / 10000. : R(0.1);
    for (int r = 0; r < in->n_diel; ++r) {
        const float* d = &in->diel[r * 8];
        int elem = (int)d[0], n = (int)d[1], g = (int)d[7];
        double a = d[2], b = d[3], c = d[4], dd = d[5], f = d[6];
        int ion = elem + 1 - n;
        if (ion <= in->nstages) {
            double v = R(1e-12) * (a / t + b + c * t + dd * (t * t)) * pow(t, -1.5) * exp(-f / t);
            if (g == 0) diRec[elem][ion] = v;
            else if (g == 1) { if (te < 20000.) diRec[elem][ion] = v; }
            else if (g == 2) { if (te >= 20000.) diRec[elem][ion] = v; }
        }
    }
    if (te > 60000.) {
        double ap[NEL + 1][MAXST];
        memset(ap, 0, sizeof(ap));
        for (int r = 0; r < in->n_aldro; ++r) {
            const float* d = &in->aldro[r * 6];
            int elem = (int)d[0], n = (int)d[1];
            double a = d[2], b = d[3], t0 = d[4], t1 = d[5];
            double alpha = a * pow(te, -1.5) * exp(-t0 / te) * (1. + b * exp(-t1 / te));
            int ion = elem - n + 1;
            if (ion <= in->nstages) ap[elem][ion] = alpha;
        }
        memcpy(diRec, ap, sizeof(ap));
    }
}

/* calcAlpha, source/update_mod.f90:2298-2413 (nahar coefficients not offered) */
static void calc_alpha(const orc_balance_in* in, cell_t* c) {
    double diRec[NEL + 1][MAXST];
    memset(diRec, 0, sizeof(diRec));
    memset(c->alpha, 0, sizeof(c->alpha));
    dielectronic(in, c->te, diRec);
    const int ns = in->nstages;
    if (in->lg_badnell) {
        for (int elem = 1; elem <= NEL; ++elem) {
            if (!on(in, elem)) continue;
            for (int ion = 1; ion <= (ns - 1 < elem ? ns - 1 : elem); ++ion) {
                int nel = elem - ion;
                if (nel <= 11) {
                    c->alpha[elem][ion] = rr_badnell(in, c->te, elem, nel);
                    c->alpha[elem][ion] = c->alpha[elem][ion] + dr_badnell(in, c->te, elem, nel);
                } else {
                    c->alpha[elem][ion] = rad_rec_fit(in, c->te, elem, elem - ion + 1);
                    if (diRec[elem][ion] == 0. && ion < 7 && on(in, 8)) diRec[elem][ion] = diRec[8][ion];
                    c->alpha[elem][ion] = c->alpha[elem][ion] + (diRec[elem][ion] > 0. ? diRec[elem][ion] : 0.);
                }
            }
        }
    } else {
        for (int elem = 1; elem <= NEL; ++elem) {
            if (!on(in, elem)) continue;
            for (int ion = 1; ion <= (ns - 1 < elem ? ns - 1 : elem); ++ion)
                c->alpha[elem][ion] = rad_rec_fit(in, c->te, elem, elem - ion + 1);
        }
        for (int elem = 3; elem <= NEL; ++elem) {
            if (!on(in, elem)) continue;
            for (int ion = 1; ion <= (ns - 1 < elem ? ns - 1 : elem); ++ion) {
                if (diRec[elem][ion] == 0. && ion < 7) diRec[elem][ion] = diRec[8][ion];
                c->alpha[elem][ion] = c->alpha[elem][ion] + (diRec[elem][ion] > 0. ? diRec[elem][ion] : 0.);
            }
        }
    }
}

/* charge-exchange coefficients (a, b, c, d) of ionBalance and photoionisation,
 * source/update_mod.f90:1649-1701 and :3727-3779; the Ca rows overwrite Ar's. */
static void chex_table(double chex[NEL + 1][MAXST][4]) {
    memset(chex, 0, sizeof(double) * (NEL + 1) * MAXST * 4);
#define CX(e, i, a, b, c, d) do { chex[e][i][0] = R(a); chex[e][i][1] = R(b); chex[e][i][2] = R(c); chex[e][i][3] = R(d); } while (0)
    CX(2, 1, 7.47e-6, 2.06, 9.93, -3.89);
    CX(2, 2, 1.e-5, 0., 0., 0.);
    CX(3, 2, 1.26, 0.96, 3.02, -0.65);
    CX(3, 3, 1.e-5, 0., 0., 0.);
    CX(4, 2, 1.e-5, 0., 0., 0.);
    CX(4, 3, 1.e-5, 0., 0., 0.);
    CX(4, 4, 5.17, 0.82, -.69, -1.12);
    CX(5, 2, 2.e-2, 0., 0., 0.);
    CX(5, 3, 1.e-5, 0., 0., 0.);
    CX(5, 4, 5.27e-1, 0.76, -0.63, -1.17);
    CX(6, 1, 1.76e-9, 8.33, 4278.78, -6.41);
    CX(6, 2, 1.67e-4, 2.79, 304.72, -4.07);
    CX(6, 3, 3.25, 0.21, 0.19, -3.29);
    CX(6, 4, 332.46, -0.11, -0.995, -1.58e-3);
    CX(7, 1, 1.01e-3, -0.29, -0.92, -8.38);
    CX(7, 2, 3.05e-1, 0.60, 2.65, -0.93);
    CX(7, 3, 4.54, 0.57, -0.65, -0.89);
    CX(7, 4, 3.28, 0.52, -0.52, -0.19);
    CX(8, 1, 1.04, 3.15e-2, -0.61, -9.73);
    CX(8, 2, 1.04, 0.27, 2.02, -5.92);
    CX(8, 3, 3.98, 0.26, 0.56, -2.62);
    CX(8, 4, 2.52e-1, 0.63, 2.08, -4.16);
    CX(9, 2, 1.e-5, 0., 0., 0.);
    CX(9, 3, 9.86, 0.29, -0.21, -1.15);
    CX(9, 4, 7.15e-1, 1.21, -0.70, -0.85);
    CX(10, 2, 1.e-5, 0., 0., 0.);
    CX(10, 3, 14.73, 4.52e-2, -0.84, -0.31);
    CX(10, 4, 6.47, 0.54, 3.59, -5.22);
    CX(11, 2, 1.e-5, 0., 0., 0.);
    CX(11, 3, 1.33, 1.15, 1.20, -0.32);
    CX(11, 4, 1.01e-1, 1.34, 10.05, -6.41);
    CX(12, 2, 8.58e-5, 2.49e-3, 2.93e-2, -4.33);
    CX(12, 3, 6.49, 0.53, 2.82, -7.63);
    CX(12, 4, 6.36, 0.55, 3.86, -5.19);
    CX(13, 2, 1.e-5, 0., 0., 0.);
    CX(13, 3, 7.11e-5, 4.12, 1.72e4, -22.24);
    CX(13, 4, 7.52e-1, 0.77, 6.24, -5.67);
    CX(14, 2, 1.23, 0.24, 3.17, 4.18e-3);
    CX(14, 3, 4.900e-1, -8.74e-2, -0.36, -0.79);
    CX(14, 4, 7.58, 0.37, 1.06, -4.09);
    CX(16, 1, 3.82e-7, 11.10, 2.57e4, -8.22);
    CX(16, 2, 1.e-5, 0., 0., 0.);
    CX(16, 3, 2.29, 4.02e-2, 1.59, -6.06);
    CX(16, 4, 6.44, 0.13, 2.69, -5.69);
    CX(18, 2, 1.e-5, 0., 0., 0.);
    CX(18, 3, 3.17e-2, 2.12, 12.06, -0.40);   /* "Ca+2" written into Ar's row */
    CX(18, 4, 2.68, 0.69, -0.68, -4.47);      /* "Ca+3" written into Ar's row */
    CX(26, 2, 1.26, 7.72e-2, -0.41, -7.31);
    CX(26, 3, 3.42, 0.51, -2.06, -8.99);
#undef CX
    for (int e = 0; e <= NEL; ++e)
        for (int i = 0; i < MAXST; ++i) chex[e][i][0] = chex[e][i][0] * R(1.e-9);
}

static double deltaE_k(int elem, int ion) {
    if (elem == 7 && ion == 1) return R(10863.);
    if (elem == 8 && ion == 1) return R(2205.);
    return 0.;
}

/* chex(elem,ion,1) at Te (source/update_mod.f90:1711-1720, :3788-3797) */
static double chex_fit(const double c[4], double te) {
    double t4 = te / 10000.;
    double v;
    if (te < 6000. || te > 5.e4) v = 0.;
    else v = c[0] * pow(t4, c[1]) * (1. + c[2] * exp(c[3] * t4));
    if (v < 0.) v = 0.;
    return v;
}

/* getPhotoRates, source/update_mod.f90:3971-4040 */
static void get_photo_rates(const orc_balance_in* in, const double* J, int elem, int ion, int shell, int nu1P,
                            int nu2P, double yield1, double heatef, double* gamma, double* heat) {
    const float* nu = in->nu;
    const float* xs = in->xsec;
    const int nb = in->nbins;
    const int secIonP = in->ptr[9];
    *heat = 0.;
    *gamma = 0.;
    int iup = nu2P < nb ? nu2P : nb;
    double augerE = kHcRyd * (double)nu[nu1P - 1] * yield1;
    if (!on(in, elem)) return;
    int IPnuP = nu1P;
    int xSecP = in->element_p[(((elem - 1) * NEL + (ion - 1)) * 7 + (shell - 1)) * 3 + 2];
    double g = 0., h = 0.;
    int top = iup < secIonP - 1 ? iup : secIonP - 1;
    for (int i = nu1P + 1; i <= top; ++i) {
        if (J[i - 1] > 0.) {
            double ph = xs[i + xSecP - IPnuP - 1];
            if (ph < R(1.e-35)) ph = 0.;
            g = g + J[i - 1] * ph / (kHcRyd * (double)nu[i - 1]);
            h = h + J[i - 1] * ph;
        }
    }
    h = h - g * augerE;
    double ph = xs[xSecP - 1];
    g = g + J[IPnuP - 1] * ph / (kHcRyd * (double)nu[IPnuP - 1]);
    h = h + J[IPnuP - 1] * ph * (kHcRyd * (double)nu[IPnuP - 1] - augerE) / (kHcRyd * (double)nu[IPnuP - 1]);
    double gh = 0., hh = 0.;
    int ilow = IPnuP + 1 > secIonP ? IPnuP + 1 : secIonP;
    for (int i = ilow; i <= iup; ++i) {
        double p = xs[i + xSecP - IPnuP - 1];
        gh = gh + J[IPnuP - 1] * p / (kHcRyd * (double)nu[i - 1]);   /* radField(IPnuP), as the reference */
        hh = hh + J[IPnuP - 1] * p;
    }
    g = g + gh;
    hh = hh - gh * augerE;
    h = h + hh * heatef;
    *gamma = g;
    *heat = h;
}

/* photoionisation, source/update_mod.f90:3584-3832 */
static void photoionisation(const orc_balance_in* in, const double* J, cell_t* c) {
    const int ns = in->nstages, nb = in->nbins;
    const float* nu = in->nu;
    const float* xs = in->xsec;
    double xe = 0.;
    for (int elem = 1; elem <= NEL; ++elem)
        if (on(in, elem)) xe = xe + c->ion[elem][1] * abun(in, elem) * c->hden;
    xe = c->ne / xe;
    double heatef;
    if (xe > R(0.95)) heatef = 1.;
    else {
        if (xe < R(1.e-4)) xe = R(1.e-4);
        heatef = R(0.9971) * (1. - pow(1. - pow(xe, R(0.2663)), R(1.3163)));
    }
    for (int elem = 0; elem <= NEL; ++elem)
        for (int ion = 0; ion < MAXST; ++ion)
            for (int s = 0; s <= 10; ++s) { c->pi1[elem][ion][s] = R(1.e-20); c->pi2[elem][ion][s] = 0.; }
    for (int elem = 1; elem <= NEL; ++elem) {
        if (!on(in, elem)) continue;
        for (int ion = 1; ion <= (elem < ns - 1 ? elem : ns - 1); ++ion) {
            int nsh = in->n_shells[(elem - 1) * NEL + (ion - 1)];
            for (int shell = 1; shell <= nsh; ++shell) {
                int IPnuP, highNuP, P = 0;
                if (elem > 2) {
                    IPnuP = in->element_p[(((elem - 1) * NEL + (ion - 1)) * 7 + (shell - 1)) * 3 + 0];
                    highNuP = in->element_p[(((elem - 1) * NEL + (ion - 1)) * 7 + (shell - 1)) * 3 + 1];
                } else if (elem == 1) {
                    IPnuP = in->ptr[ORC_P_HLEVNUP1]; highNuP = nb; P = in->ptr[ORC_P_HLEVXSECP1];
                } else if (ion == 1) {
                    IPnuP = in->ptr[ORC_P_HEILEVNUP1]; highNuP = nb; P = in->ptr[ORC_P_HEISINGXSECP1];
                } else {
                    IPnuP = in->ptr[ORC_P_HEIILEVNUP1]; highNuP = nb; P = in->ptr[ORC_P_HEIIXSECP1];
                }
                if (elem < 3) {
                    double n1 = R(1.e-20), h1 = 0.;
                    for (int j = IPnuP; j <= highNuP; ++j) {
                        double ph = xs[j - IPnuP + 1 + P - 1 - 1];
                        if (ph < R(1.e-35)) ph = 0.;
                        if (J[j - 1] > 0.) {
                            n1 = n1 + J[j - 1] * ph / (kHcRyd * (double)nu[j - 1]);
                            h1 = h1 + ph * J[j - 1] * ((double)nu[j - 1] - (double)nu[IPnuP - 1]) / (double)nu[j - 1];
                        }
                    }
                    c->pi1[elem][ion][shell] = n1;
                    c->pi2[elem][ion][shell] = h1;
                } else {
                    double y1 = in->auger[(((elem - 1) * NEL + (ion - 1)) * 10 + (shell - 1)) * 10 + 0];
                    get_photo_rates(in, J, elem, ion, shell, IPnuP, highNuP, y1, heatef, &c->pi1[elem][ion][shell],
                                    &c->pi2[elem][ion][shell]);
                }
            }
        }
    }
    /* reverse charge exchange with the Te fit applied to every element */
    double chex[NEL + 1][MAXST][4];
    chex_table(chex);
    for (int elem = 1; elem <= NEL; ++elem) {
        if (!on(in, elem)) continue;
        for (int ion = 1; ion <= (elem < ns - 1 ? elem : ns - 1); ++ion) {
            double cx = chex_fit(chex[elem][ion], c->te);
            int nElec = elem - ion + 1;
            const int32_t* o = &in->outer[((elem - 1) * NEL + (nElec - 1)) * 3];
            double rev = 0.;
            if (deltaE_k(elem, ion) > 1.)
                rev = cx * (1. - c->ion[1][1]) * c->hden * 2. * exp(-deltaE_k(elem, ion) / c->te) /
                      ((double)(float)o[1] / (double)(float)o[2]);
            c->pi1[elem][ion][o[0]] = c->pi1[elem][ion][o[0]] + rev;
        }
    }
}

/* collisionalIonisation, source/update_mod.f90:3552-3582 (returns at the
 * first u > 80, leaving the remaining rates at zero) */
static void collisional_ionisation(const orc_balance_in* in, cell_t* c) {
    memset(c->coll1, 0, sizeof(c->coll1));
    memset(c->coll2, 0, sizeof(c->coll2));
    const int ns = in->nstages;
    double te = c->te * R(8.617385e-05);
    for (int elem = 1; elem <= NEL; ++elem) {
        if (!on(in, elem)) continue;
        for (int ion = 1; ion <= (ns - 1 < elem - 1 ? ns - 1 : elem - 1); ++ion) {
            int elec = elem - ion + 1;
            const float* cf = &in->cf[((elem - 1) * NEL + (elec - 1)) * 5];
            double u = (double)cf[0] / te;
            if (u > 80.) return;
            c->coll1[elem][ion] = (double)cf[2] * (1. + (double)cf[1] * sqrt(u)) / ((double)cf[3] + u) * pow(u, (double)cf[4]) * exp(-u);
            c->coll2[elem][ion] = (double)in->cion_therm[(elem - 1) * NEL + (ion - 1)] * c->coll1[elem][ion] * kBoltz;
        }
    }
}

/* compton, source/update_mod.f90:3834-3897 */
static void compton(const orc_balance_in* in, const double* J, cell_t* c) {
    const float* nu = in->nu;
    const int nb = in->nbins;
    const int cRecoilHP = in->ptr[10], cRecoilHeP = in->ptr[11];
    double s1 = 0., s2 = 0., rhH = 0., rhHe = 0., rIonH = 0.;
    for (int i = 1; i <= nb; ++i) {
        double rf = J[i - 1];
        s1 = s1 + rf;
        s2 = s2 + rf / (double)nu[i - 1];
        if (i > cRecoilHP) {
            double energy = R(2.66e-5) * (double)nu[i - 1] * (double)nu[i - 1] - 1.;
            rhH = rhH + (double)in->xsec_recoil[i - 1] * rf * energy;
            rIonH = rIonH + (double)in->xsec_recoil[i - 1] * rf;
        }
        if (i > cRecoilHeP) {
            double energy = R(2.66e-5) * (double)nu[i - 1] * (double)nu[i - 1] - R(1.8);
            rhHe = rhHe + (double)in->xsec_recoil[i - 1] * rf * energy;
        }
    }
    s1 = s1 * kRyd2erg;
    c->comptonCool = (R(6.65e-25) * R(6.75e-10) * c->te * s2) / c->hden;
    c->comptonHeat = (R(6.65e-25) * s1 / R(8.184e-7)) / c->hden;
    double he = on(in, 2) ? rhHe * (c->ion[2][1] * abun(in, 2)) * 2. : 0.;
    c->comptonRecoilHeat = (rhH * c->ion[1][1] * abun(in, 1) + he) * kRyd2erg;
}

/* ionBalance, source/update_mod.f90:1575-1992 (recursion as a loop); returns
 * lgConv.  x_tol is the limit on the relative X(H0), X(He0), X(He+) changes
 * that ends the X-iterations (the reference's 0.01). */
static int ion_balance(const orc_balance_in* in, cell_t* c, double x_tol) {
    const int ns = in->nstages;
    double chexRaw[NEL + 1][MAXST][4];
    chex_table(chexRaw);
    for (;;) {
        int lgConv = 1;
        double ionRatio[3][3] = {{0}}, ionProd[3][3], den[3] = {1., 1., 1.};
        for (int a = 0; a < 3; ++a) for (int b = 0; b < 3; ++b) ionProd[a][b] = 1.;
        double expFact = (double)R(157893.94) / c->te;
        if (expFact > 75.) expFact = 75.;
        double collIonH = R(2.75E-16) * c->te * sqrt(c->te) * ((double)R(157893.94) / c->te + 2.) * exp(-expFact);
        double HIOld = c->ion[1][1];
        double HeIOld = on(in, 2) ? c->ion[2][1] : 0.;
        double HeIIOld = on(in, 2) ? c->ion[2][2] : 0.;
        for (int elem = 1; elem <= 2; ++elem) {
            if (!on(in, elem)) continue;
            for (int ion = 1; ion <= (elem < ns - 1 ? elem : ns - 1); ++ion) {
                double cx = chex_fit(chexRaw[elem][ion], c->te);
                int nElec = elem - ion + 1;
                int outShell = in->outer[((elem - 1) * NEL + (nElec - 1)) * 3 + 0];
                double revRate = 0.;   /* deltaE_k(1..2, :) = 0 */
                if (elem > 1 || ion > 1) collIonH = 0.;
                ionRatio[elem][ion] = (c->pi1[elem][ion][outShell] + collIonH * c->ne + revRate) /
                                      (c->ne * c->alpha[elem][ion] + cx * c->hden * c->ion[1][1]);
            }
        }
        for (int elem = 1; elem <= 2; ++elem) {
            if (!on(in, elem)) continue;
            for (int ion = 1; ion <= (elem < ns - 1 ? elem : ns - 1); ++ion)
                for (int i = 1; i <= ion; ++i) ionProd[elem][ion] = ionProd[elem][ion] * ionRatio[elem][i];
        }
        for (int elem = 1; elem <= 2; ++elem) {
            if (!on(in, elem)) continue;
            for (int ion = 1; ion <= (elem < ns - 1 ? elem : ns - 1); ++ion) den[elem] = den[elem] + ionProd[elem][ion];
        }
        for (int elem = 1; elem <= 2; ++elem) {
            if (!on(in, elem)) continue;
            for (int ion = 1; ion <= (elem + 1 < ns ? elem + 1 : ns); ++ion) {
                double v = ion == 1 ? 1. / den[elem] : ionProd[elem][ion - 1] / den[elem];
                if (v > kXMax) v = kXMax;
                if (v < R(1.e-20)) v = R(1.e-20);
                c->ion[elem][ion] = v;
            }
        }
        /* heavy elements: bidiagonal ladder */
        for (int elem = 3; elem <= NEL; ++elem) {
            if (!on(in, elem)) continue;
            double out[MAXST + 1], inn[MAXST + 1], mat[MAXST + 1];
            memset(out, 0, sizeof(out));
            memset(inn, 0, sizeof(inn));
            const int topI = elem < ns - 1 ? elem : ns - 1;
            for (int ion = 1; ion <= topI; ++ion) {
                out[ion] = out[ion] + c->coll1[elem][ion] * c->ne;
                int nsh = in->n_shells[(elem - 1) * NEL + (ion - 1)];
                for (int shell = 1; shell <= nsh; ++shell) {
                    out[ion] = out[ion] + c->pi1[elem][ion][shell];
                    int nAug = in->nauger[((elem - 1) * NEL + (ion - 1)) * 10 + (shell - 1)];
                    for (int nelec = 2; nelec <= nAug; ++nelec) {
                        int lim = ns - 1 < elem ? ns - 1 : elem;
                        int maxim = ion + nelec - 1 < lim ? ion + nelec - 1 : lim;
                        double ratio = c->ion[elem][maxim] > 1e-30 ? c->ion[elem][ion] / c->ion[elem][maxim] : 1.;
                        out[maxim] = out[maxim] + c->pi1[elem][ion][shell] *
                                     (double)in->auger[(((elem - 1) * NEL + (ion - 1)) * 10 + (shell - 1)) * 10 + (nelec - 1)] * ratio;
                    }
                }
            }
            for (int ion = 1; ion <= topI; ++ion)
                inn[ion] = c->ne * c->alpha[elem][ion] + chexRaw[elem][ion][0] * c->hden * c->ion[1][1];
            mat[1] = 1.;
            double sumMat = 1.;
            const int top = ns < elem + 1 ? ns : elem + 1;
            for (int ion = 2; ion <= top; ++ion) {
                mat[ion] = mat[ion - 1] * out[ion - 1] / inn[ion - 1];
                sumMat = sumMat + mat[ion];
            }
            sumMat = 1. / sumMat;
            c->ion[elem][top] = mat[top] * sumMat;
            for (int ion = 1; ion <= topI; ++ion) {
                double v;
                if (c->nIterateX < 2 && mat[ion] * sumMat > 0.) {
                    double old = c->ion[elem][ion];
                    if (old <= 0.) old = R(1.e-5);
                    v = pow(10., 0.5 * (log10(old) + log10(mat[ion] * sumMat)));
                } else {
                    v = mat[ion] * sumMat;
                }
                if (v > kXMax) v = kXMax;
                if (v < R(1.e-20)) v = R(1.e-20);
                c->ion[elem][ion] = v;
            }
        }
        /* electron density */
        double ne = 0.;
        for (int elem = 1; elem <= NEL; ++elem) {
            if (!on(in, elem)) continue;
            for (int ion = 2; ion <= (elem + 1 < ns ? elem + 1 : ns); ++ion)
                if (c->ion[elem][ion] >= R(1.e-10)) ne = ne + (double)(ion - 1) * abun(in, elem) * c->ion[elem][ion];
        }
        ne = ne * c->hden;
        if (ne == 0.) ne = 1.;
        c->ne = ne;
        double dHI = (c->ion[1][1] - HIOld) / HIOld;
        double dHeI = on(in, 2) ? (c->ion[2][1] - HeIOld) / HeIOld : 0.;
        double dHeII = on(in, 2) ? (c->ion[2][2] - HeIIOld) / HeIIOld : 0.;
        int big = fabs(dHI) > x_tol || fabs(dHeI) > x_tol || fabs(dHeII) > x_tol;
        if (big && c->nIterateX < 15) {
            c->nIterateX = c->nIterateX + 1;
            continue;
        } else if (big && c->nIterateX == 15) {
            lgConv = 0;
        }
        return lgConv;
    }
}

/* ------------------------------------------------------------- equilibrium */

/* splint, source/interpolation_mod.f90:286-335 */
static double splint(const double* xa, const double* ya, const double* y2a, int n, double x) {
    if (x <= xa[0]) return ya[0];
    if (x >= xa[n - 1]) return ya[n - 1];
    int klo = 1, khi = n;
    for (int i = 0; i < 1000; ++i) {
        if (khi - klo <= 1) break;
        int k = (khi + klo) / 2;
        if (xa[k - 1] > x) khi = k; else klo = k;
    }
    double h = xa[khi - 1] - xa[klo - 1];
    double a = (xa[khi - 1] - x) / h;
    double b = (x - xa[klo - 1]) / h;
    return a * ya[klo - 1] + b * ya[khi - 1] + ((a * a * a - a) * y2a[klo - 1] + (b * b * b - b) * y2a[khi - 1]) * (h * h) / 6.;
}

/* spline with natural end conditions, source/interpolation_mod.f90:207-278 */
static void spline_natural(const double* x, const double* y, int n, double* y2) {
    double u[64];
    y2[0] = 0.;
    u[0] = 0.;
    for (int i = 1; i < n - 1; ++i) {
        double sig = (x[i] - x[i - 1]) / (x[i + 1] - x[i - 1]);
        double p = sig * y2[i - 1] + 2.;
        y2[i] = (sig - 1.) / p;
        double t = y[i + 1];
        t = t - y[i];
        t = t / (x[i + 1] - x[i]);
        t = t - (y[i] - y[i - 1]) / (x[i] - x[i - 1]);
        u[i] = (6. * t / (x[i + 1] - x[i - 1]) - sig * u[i - 1]) / p;
    }
    y2[n - 1] = (0. - 0. * u[n - 2]) / (0. * y2[n - 2] + 1.);
    for (int k = n - 2; k >= 0; --k) y2[k] = y2[k] * y2[k + 1] + u[k];
}

int orc_equilibrium(const orc_balance_in* in, int32_t atom, double Te, double Ne, double ionDenUp, int32_t rec,
                    double* nOut, double* em) {
    const int32_t* h = &in->atom_hdr[atom * ORC_AT_HDR];
    const double* D = in->atom_data;
    const int nLev = h[ORC_AT_NLEV], nT = h[ORC_AT_NTEMP];
    const double* logT = D + h[ORC_AT_OFF_LOGT];
    const double* qom = D + h[ORC_AT_OFF_QOM];
    const double* A = D + h[ORC_AT_OFF_A];
    const double* g = D + h[ORC_AT_OFF_G];
    const double* e = D + h[ORC_AT_OFF_E];
    const double atp = D[h[ORC_AT_OFF_ATP]];
    const int iup2p = h[ORC_AT_IUP2P];
#define AA(j, i) A[((j) - 1) * nLev + ((i) - 1)]
    double sqrTe = sqrt(Te), log10Te = log10(Te);
    double alphaTotal[32];
    memset(alphaTotal, 0, sizeof(alphaTotal));
    if (rec) {
        const double* rr = D + h[ORC_AT_OFF_REC];
        if (h[ORC_AT_RECTYPE] == 1) {
            for (int r = 0; r < h[ORC_AT_NREC]; ++r) {
                const double* v = rr + r * 11;
                int j = r + 2;
                double br = (double)(float)v[0], z = (double)(float)v[1];
                double ar[4], ad[5];
                for (int k = 0; k < 4; ++k) ar[k] = (double)(float)v[2 + k];
                for (int k = 0; k < 5; ++k) ad[k] = (double)(float)v[6 + k];
                alphaTotal[1] = 1.;
                if (z > 0.) {
                    double tz = Te * R(1.e-4) / (z * z);
                    double t4 = Te * R(1.e-4);
                    alphaTotal[j] = R(1.e-13) * br * z * ar[0] * pow(tz, ar[1]) / (1. + ar[2] * pow(tz, ar[3])) +
                                    R(1.0e-12) * br * (ad[0] / t4 + ad[1] + ad[2] * Te * R(1.e-4) + ad[3] * (t4 * t4)) *
                                        pow(t4, -1.5) * exp(-ad[4] * R(1.e4) / Te);
                }
            }
        } else if (h[ORC_AT_RECTYPE] == 2) {
            for (int r = 0; r < h[ORC_AT_NREC]; ++r) {
                const double* v = rr + r * 5;
                int jj = (int)v[0];
                double a = (double)(float)v[1], b = (double)(float)v[2], cc = (double)(float)v[3], d = (double)(float)v[4];
                double L = log10(Te);
                alphaTotal[1] = 1.;
                alphaTotal[jj] = pow(10., a + b * L + cc * (L * L) + d * (L * L * L));
            }
        }
    }
    /* qeff */
    double qeff[32][32];
    double x[32][32], y[32];
    memset(qeff, 0, sizeof(qeff));
    memset(x, 0, sizeof(x));
    memset(y, 0, sizeof(y));
    int p = 0;
    for (int i = 2; i <= nLev; ++i) {
        for (int j = i; j <= nLev; ++j, ++p) {
            const double* qq = qom + (size_t)p * nT;
            double qomInt;
            if (nT == 1) qomInt = qq[0];
            else if (nT == 2) qomInt = qq[0] + (qq[1] - qq[0]) / (logT[1] - logT[0]) * (log10Te - logT[0]);
            else {
                double y2[64];
                spline_natural(logT, qq, nT, y2);
                qomInt = splint(logT, qq, y2, nT, log10Te);
            }
            double cs = qomInt;
            const double constant = 1.4388463;
            if (e[i - 2] <= e[j - 1]) {
                double delTeK = (e[i - 2] - e[j - 1]) * constant;
                double expFac = exp(delTeK / Te);
                qeff[i - 1][j] = 8.63e-6 * cs * expFac / (g[i - 2] * sqrTe);
                qeff[j][i - 1] = 8.63e-6 * cs / (g[j - 1] * sqrTe);
            } else {
                double delTeK = (e[j - 1] - e[i - 2]) * constant;
                double expFac = exp(delTeK / Te);
                qeff[j][i - 1] = 8.63e-6 * cs * expFac / (g[i - 2] * sqrTe);
                qeff[i - 1][j] = 8.63e-6 * cs / (g[j - 1] * sqrTe);
            }
        }
    }
    /* rate matrix, row 1 = normalisation */
    for (int j = 1; j <= nLev; ++j) x[1][j] = 1.;
    y[1] = 1.;
    for (int i = 2; i <= nLev; ++i) {
        for (int j = 1; j <= nLev; ++j) {
            if (j != i) {
                x[i][j] = x[i][j] + Ne * qeff[j][i];
                x[i][i] = x[i][i] - Ne * qeff[i][j];
                if (j > i) x[i][j] = x[i][j] + AA(j, i);
                else x[i][i] = x[i][i] - AA(i, j);
            }
        }
        y[i] = -Ne * ionDenUp * alphaTotal[i];
    }
    /* luSlv = lured + reslv (no pivoting), source/emission_mod.f90:3010-3106 */
    int n = nLev;
    if (n > 1) {
        for (int i = 1; i <= n - 1; ++i)
            for (int k = i + 1; k <= n; ++k) {
                double factor = x[k][i] / x[i][i];
                for (int j = i + 1; j <= n; ++j) x[k][j] = x[k][j] - x[i][j] * factor;
            }
        for (int i = 1; i <= n - 1; ++i)
            for (int j = i + 1; j <= n; ++j) y[j] = y[j] - y[i] * x[j][i] / x[i][i];
        y[n] = y[n] / x[n][n];
        for (int i = 1; i <= n - 1; ++i) {
            int k = n - i;
            for (int j = k + 1; j <= n; ++j) y[k] = y[k] - y[j] * x[k][j];
            y[k] = y[k] / x[k][k];
        }
    } else {
        y[1] = y[1] / x[1][1];
    }
    double sumN = 0.;
    for (int i = 1; i <= nLev; ++i) sumN = sumN + y[i];
    for (int i = 1; i <= nLev; ++i) y[i] = y[i] / sumN;
    if (nOut) for (int i = 1; i <= nLev; ++i) nOut[i - 1] = y[i];
    if (em) {
        for (int i = 0; i < nLev * nLev; ++i) em[i] = 0.;
        for (int i = 1; i <= nLev - 1; ++i)
            for (int j = i + 1; j <= nLev; ++j) {
                double aji = AA(j, i);
                if (aji != 0.) {
                    double Eji = e[j - 1] - e[i - 1];
                    if (j == iup2p && i == 1 && atp > 0.) aji = aji - atp;
                    em[(i - 1) * nLev + (j - 1)] = aji * Eji * y[j];
                }
            }
    }
#undef AA
    return 0;
}

/* forLines of update_mod (source/update_mod.f90:1221-1262) summed the way
 * thermBalance adds it to coolColl (:1061-1088): coolColl += each line > 1e-35 */
static double for_lines_cool(const orc_balance_in* in, const cell_t* c, double coolColl) {
    const int ns = in->nstages;
    double em[32 * 32];
    for (int elem = 3; elem <= NEL; ++elem) {
        if (!on(in, elem)) continue;
        for (int ion = 1; ion <= (elem + 1 < ns ? elem + 1 : ns); ++ion) {
            int at = in->atom_index[(elem - 1) * (NEL + 1) + (ion - 1)];
            if (at < 0) continue;
            double up = 0.;
            if (ion < (elem + 1 < ns ? elem + 1 : ns) && c->ion[elem][ion] > 0.) up = c->ion[elem][ion + 1] / c->ion[elem][ion];
            orc_equilibrium(in, at, c->te, c->ne, up, 0, NULL, em);
            int nLev = in->atom_hdr[at * ORC_AT_HDR + ORC_AT_NLEV];
            for (int j = 1; j <= nLev; ++j)
                for (int k = 1; k <= nLev; ++k) {
                    double f = em[(j - 1) * nLev + (k - 1)] * abun(in, elem) * c->ion[elem][ion] * R(1.9865e-16);
                    if (f > R(1.e-35)) coolColl = coolColl + f;
                }
        }
    }
    return coolColl;
}

/* thermBalance, source/update_mod.f90:887-1215 */
static void therm_balance(const orc_balance_in* in, const cell_t* c, double* heatInt, double* coolInt) {
    const int ns = in->nstages;
    const double Te = c->te, Ne = c->ne;
    double coolFF = 0., coolRec = 0., L, Te4 = 0.;
    for (int i = 1; i <= NEL; ++i) {
        if (!(on(in, i) && ns > i)) continue;
        L = log10(Te / (double)(i * i));
        Te4 = Te / ((double)(i * i) * R(1.e4));
        double Np = c->ion[i][i + 1] * abun(in, i);
        double betaFF = (double)i * (R(1.0108464E-11) + R(9.7930778E-13) * L - R(6.6433144E-13) * L * L +
                                     R(2.4793747E-13) * L * L * L - R(2.3938215E-14) * L * L * L * L);
        double t = Np * Ne * betaFF * kBoltz * Te / sqrt(Te);
        if (!isnan(t)) coolFF = coolFF + t;
        double betaRec = (double)i * (R(9.4255985E-11) - R(4.04794384E-12) * L - R(1.0055237E-11) * L * L +
                                      R(1.99266862E-12) * L * L * L - R(1.06681387E-13) * L * L * L * L);
        t = Np * Ne * betaRec * kBoltz * Te / sqrt(Te);
        if (!isnan(t)) coolRec = coolRec + t;
    }
    L = log10(Te);
    Te4 = Te / R(1.e4);
    for (int i = 2; i <= NEL; ++i) {
        if (!(on(in, i) && ns > i)) continue;
        L = log10(4. * Te / (double)(i * i));
        Te4 = 4. * Te / ((double)(i * i) * R(1.e4));
        double Np = c->ion[i][i] * abun(in, i);
        double betaFF = ((double)i / 2.) * (R(1.070073e-11) - R(2.5730207e-13) * L + R(2.109134e-13) * L * L);
        double t = Np * Ne * betaFF * kBoltz * Te / sqrt(Te);
        if (!isnan(t)) coolFF = coolFF + t;
        double betaRec = ((double)i / 2.) * (R(1.06926e-10) - R(2.41756e-11) * L + R(1.14542e-12) * L * L -
                                             R(5.06535e-13) * L * L * L + R(9.16745e-14) * L * L * L * L);
        t = Np * Ne * betaRec * kBoltz * Te / sqrt(Te);
        if (!isnan(t)) coolRec = coolRec + t;
    }
    /* collisional excitation of H (Te4 as left by the loop above) */
    double coolColl;
    if (Te > 5000.)
        coolColl = (R(2.47e-8) * exp(-R(118338.) / Te) * pow(Te4, R(-0.228)) +
                    R(1.32e-8) * exp(-R(140252.) / Te) * pow(Te4, R(-0.460))) * kHcRyd * c->ion[1][1] * Ne;
    else
        coolColl = 0.;
    double coolCollH = 0.;
    for (int elem = 1; elem <= NEL; ++elem) {
        if (!on(in, elem)) continue;
        for (int ion = 1; ion <= (elem < ns - 1 ? elem : ns - 1); ++ion)
            coolCollH = coolCollH + abun(in, elem) * c->ion[elem][ion] * c->coll2[elem][ion] * Ne;
    }
    coolColl = for_lines_cool(in, c, coolColl);
    double heatSte = 0.;
    for (int elem = 1; elem <= NEL; ++elem) {
        if (!on(in, elem)) continue;
        for (int ion = 1; ion <= (elem < ns - 1 ? elem : ns - 1); ++ion) {
            int nsh = in->n_shells[(elem - 1) * NEL + (ion - 1)];
            for (int s = 1; s <= nsh; ++s) heatSte = heatSte + c->pi2[elem][ion][s] * c->ion[elem][ion] * abun(in, elem);
        }
    }
    double heat = heatSte;
    double cool = coolFF + coolRec + coolColl + coolCollH;
    if (in->lg_compton) {
        heat = heat + c->comptonHeat * Ne + c->comptonRecoilHeat;
        cool = cool + c->comptonCool * Ne;
    }
    *heatInt = heat;
    *coolInt = cool;
}

/* updateCell + iterateT for one cell, source/update_mod.f90:15-482 */
static void update_cell_tr(const orc_balance_in* in, orc_balance_state* st, int cell, cell_t* c, double* J,
                           orc_balance_stats* s, double* trace);

static void update_cell(const orc_balance_in* in, orc_balance_state* st, int cell, cell_t* c, double* J,
                        orc_balance_stats* s) {
    update_cell_tr(in, st, cell, c, J, s, NULL);
}

/* the same with a record of each T-iteration: Te, heating, cooling, Ne, X(H0) */
/* a cell's J and grid state into c; returns 0 for a cell no photon reached */
static int load_cell(const orc_balance_in* in, const orc_balance_state* st, int cell, cell_t* c, double* J) {
    const int C1 = in->n_cells + 1, nb = in->nbins, ns = in->nstages, E = in->n_elem_used;
    int hit = 0;
    for (int b = 0; b < nb; ++b) {
        J[b] = in->jste[(size_t)b * C1 + cell];
        if (J[b] > 0.) hit = 1;
    }
    if (!hit) return 0;
    memset(c->ion, 0, sizeof(c->ion));
    for (int elem = 1; elem <= NEL; ++elem) {
        if (!on(in, elem)) continue;
        for (int ion = 1; ion <= ns; ++ion)
            c->ion[elem][ion] = (double)st->ionden[((size_t)(ion - 1) * E + (xref(in, elem) - 1)) * C1 + cell];
    }
    c->te = st->te[cell];
    c->ne = st->ne[cell];
    c->hden = in->hden[cell];
    return 1;
}

/* Ne and the ion fractions of c into the grid state (FP32, as the grid holds them) */
static void store_cell(const orc_balance_in* in, orc_balance_state* st, int cell, const cell_t* c) {
    const int C1 = in->n_cells + 1, ns = in->nstages, E = in->n_elem_used;
    st->ne[cell] = (float)c->ne;
    for (int elem = 1; elem <= NEL; ++elem) {
        if (!on(in, elem)) continue;
        for (int ion = 1; ion <= ns; ++ion)
            st->ionden[((size_t)(ion - 1) * E + (xref(in, elem) - 1)) * C1 + cell] = (float)c->ion[elem][ion];
    }
}

static void update_cell_tr(const orc_balance_in* in, orc_balance_state* st, int cell, cell_t* c, double* J,
                           orc_balance_stats* s, double* trace) {
    st->black[cell] = 0;
    st->converged[cell] = 0;
    st->n_iter_t[cell] = 0;
    if (!load_cell(in, st, cell, c, J)) {
        st->black[cell] = 1;
        s->no_hit += 1.;
        return;
    }
    const double XOldHI = c->ion[1][1];
    const double thLimit = R(0.02);
    int nIterateT = 0, lgIBConv = 1;
    double resHigh = 0., resLow = 0., Thigh = 0., Tlow = 0.;
    for (;;) {
        nIterateT = nIterateT + 1;
        calc_alpha(in, c);
        photoionisation(in, J, c);
        collisional_ionisation(in, c);
        c->nIterateX = 1;
        if (in->lg_compton) compton(in, J, c);
        lgIBConv = ion_balance(in, c, R(0.01));
        double heat, cool;
        therm_balance(in, c, &heat, &cool);
        if (trace && nIterateT <= 20) {
            double* t = trace + (nIterateT - 1) * 5;
            t[0] = c->te; t[1] = heat; t[2] = cool; t[3] = c->ne; t[4] = c->ion[1][1];
        }
        double res = heat - cool;
        if (fabs(res) >= thLimit * (fabs(cool) + fabs(heat)) / 2.) {
            if (nIterateT < 20) {
                if (res < 0.) {
                    resLow = res;
                    Tlow = c->te;
                    if (Thigh != 0.) c->te = Tlow - (Thigh - Tlow) * resLow / (resHigh - resLow);
                    else c->te = c->te / R(1.2);
                } else {
                    resHigh = res;
                    Thigh = c->te;
                    if (Tlow != 0.) c->te = Tlow - (Thigh - Tlow) * resLow / (resHigh - resLow);
                    else c->te = c->te * R(1.2);
                }
                if (nIterateT >= 6 && fabs(Thigh - Tlow) <= (R(0.002) * (Thigh + Tlow))) {
                    if (res < 0.) { c->te = Thigh - 100.; Thigh = 0.; }
                    else { c->te = Tlow + 100.; Tlow = 0.; }
                }
                if (c->te <= 0.) c->te = 1.;
                continue;
            } else {
                if (Thigh == 0.) c->te = Tlow;
                else if (Tlow == 0.) c->te = Thigh;
                else c->te = (Thigh + Tlow) * 0.5;
                s->no_te_bal += 1.;
            }
        }
        break;
    }
    if (!lgIBConv) s->no_ion_bal += 1.;
    double deltaXHI = (c->ion[1][1] - XOldHI) / XOldHI;
    st->converged[cell] = fabs(deltaXHI) <= (double)in->xhi_limit ? 1 : 0;
    if (st->converged[cell]) s->converged += 1;
    st->n_iter_t[cell] = nIterateT;
    st->te[cell] = (float)c->te;
    store_cell(in, st, cell, c);
}

/* The balance of one cell with its Te held: calcAlpha, photoionisation,
 * collisional ionisation, Compton and ionBalance at that Te, repeated from
 * where ionBalance stopped until its X changes fall within x_tol (at most 64
 * times, as the tight device balance does), then thermBalance; returns
 * heating - cooling (0 for a cell no photon reached, which is marked black). */
static double fixed_te_cell(const orc_balance_in* in, orc_balance_state* st, int cell, cell_t* c, double* J,
                            double x_tol) {
    st->black[cell] = 0;
    st->n_iter_t[cell] = 0;
    st->converged[cell] = 0;
    if (!load_cell(in, st, cell, c, J)) {
        st->black[cell] = 1;
        return 0.;
    }
    int round = 0, lgIBConv = 0;
    while (!lgIBConv && round < 64) {
        round = round + 1;
        calc_alpha(in, c);
        photoionisation(in, J, c);
        collisional_ionisation(in, c);
        c->nIterateX = 1;
        if (in->lg_compton) compton(in, J, c);
        lgIBConv = ion_balance(in, c, x_tol);
    }
    double heat, cool;
    therm_balance(in, c, &heat, &cool);
    st->n_iter_t[cell] = round;
    st->converged[cell] = lgIBConv;
    store_cell(in, st, cell, c);
    return heat - cool;
}

typedef struct {
    const orc_balance_in* in;
    orc_balance_state* st;
    int c0, c1;
    orc_balance_stats stats;
    double x_tol;
    double* resid;              /* non-NULL: the balance with Te held */
} job_t;

static void* worker(void* arg) {
    job_t* j = (job_t*)arg;
    cell_t* c = (cell_t*)malloc(sizeof(cell_t));
    double* J = (double*)malloc(sizeof(double) * (size_t)j->in->nbins);
    memset(&j->stats, 0, sizeof(j->stats));
    for (int cell = j->c0; cell < j->c1; ++cell) {
        if (j->resid) j->resid[cell] = fixed_te_cell(j->in, j->st, cell, c, J, j->x_tol);
        else update_cell(j->in, j->st, cell, c, J, &j->stats);
    }
    free(J);
    free(c);
    return NULL;
}

static void run_jobs(const orc_balance_in* in, orc_balance_state* st, int32_t nthreads, double x_tol,
                     double* resid, orc_balance_stats* stats) {
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    job_t jobs[256];
    pthread_t th[256];
    const int C = in->n_cells;
    for (int t = 0; t < nthreads; ++t) {
        jobs[t].in = in;
        jobs[t].st = st;
        jobs[t].c0 = 1 + (int)((int64_t)C * t / nthreads);
        jobs[t].c1 = 1 + (int)((int64_t)C * (t + 1) / nthreads);
        jobs[t].x_tol = x_tol;
        jobs[t].resid = resid;
        pthread_create(&th[t], NULL, worker, &jobs[t]);
    }
    if (stats) memset(stats, 0, sizeof(*stats));
    for (int t = 0; t < nthreads; ++t) {
        pthread_join(th[t], NULL);
        if (!stats) continue;
        stats->no_hit += jobs[t].stats.no_hit;
        stats->no_ion_bal += jobs[t].stats.no_ion_bal;
        stats->no_te_bal += jobs[t].stats.no_te_bal;
        stats->converged += jobs[t].stats.converged;
    }
}

int orc_balance(const orc_balance_in* in, orc_balance_state* st, int32_t nthreads, orc_balance_stats* stats) {
    run_jobs(in, st, nthreads, 0., NULL, stats);
    return 0;
}

int orc_balance_fixed_te(const orc_balance_in* in, orc_balance_state* st, int32_t nthreads, double x_tol,
                         double* resid) {
    if (!resid) return 1;
    resid[0] = 0.;
    run_jobs(in, st, nthreads, x_tol, resid, NULL);
    return 0;
}

/* forLines of emission_mod (rec = .true., scale 1.9865e9) and the normFor sum
 * of emissionDriver (source/emission_mod.f90:1481-1524, :1780-1795) */
int orc_for_lines_emission(const orc_balance_in* in, const float* te, const float* ne, const float* ionden,
                           const uint8_t* compute, double* for_lines) {
    const int C1 = in->n_cells + 1, ns = in->nstages, E = in->n_elem_used;
    double em[32 * 32];
    for (int cell = 0; cell < C1; ++cell) {
        double normFor = 0.;
        if (compute && !compute[cell]) { for_lines[cell] = 0.; continue; }
        for (int elem = 3; elem <= NEL; ++elem) {
            if (!on(in, elem)) continue;
            const int top = elem + 1 < ns ? elem + 1 : ns;
            for (int ion = 1; ion <= top; ++ion) {
                int at = in->atom_index[(elem - 1) * (NEL + 1) + (ion - 1)];
                if (at < 0) continue;
                double x = ionden[((size_t)(ion - 1) * E + (xref(in, elem) - 1)) * C1 + cell];
                double up = 0.;
                if (ion < top && x > 0.) up = (double)ionden[((size_t)ion * E + (xref(in, elem) - 1)) * C1 + cell] / x;
                orc_equilibrium(in, at, (double)te[cell], (double)ne[cell], up, 1, NULL, em);
                int nLev = in->atom_hdr[at * ORC_AT_HDR + ORC_AT_NLEV];
                for (int j = 1; j <= nLev; ++j)
                    for (int k = 1; k <= nLev; ++k) {
                        double f = em[(j - 1) * nLev + (k - 1)] * abun(in, elem) * x * R(1.9865e9);
                        if (f > R(1.e-35)) normFor = normFor + f;
                    }
            }
        }
        for_lines[cell] = normFor;
    }
    return 0;
}

/* updateCell of one cell with a record of its T-iterations (trace[20][5]:
 * Te, heating, cooling, Ne, X(H0)); returns the number of T-iterations. */
int orc_balance_trace(const orc_balance_in* in, orc_balance_state* st, int32_t cell, double* trace) {
    cell_t* c = (cell_t*)malloc(sizeof(cell_t));
    double* J = (double*)malloc(sizeof(double) * (size_t)in->nbins);
    orc_balance_stats s;
    memset(&s, 0, sizeof(s));
    update_cell_tr(in, st, cell, c, J, &s, trace);
    free(J);
    free(c);
    return st->n_iter_t[cell];
}
