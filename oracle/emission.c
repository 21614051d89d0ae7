/*
 * emission.c - FP64 restatement of the per-cell emission phase of MOCASSIN:
 * the diffuse re-emission CDF recPDF(cell,:) and the line fraction
 * totalLines(cell).
 *
 * TEST INFRASTRUCTURE ONLY (checker of libmcx.so's emission kernel).  Follows
 *   emissionDriver    source/emission_mod.f90:36-252
 *   fb_ff             source/emission_mod.f90:336-618
 *   twoPhoton / hydro2phot / HeI2photSub   source/emission_mod.f90:620-760
 *   free_free / ffCoeff                    source/emission_mod.f90:762-800
 *   RecLinesEmission  source/emission_mod.f90:856-1151
 *   setDiffusePDF     source/emission_mod.f90:1528-1919 (gas, no dust)
 * The forbidden-line emissivities of forLines (equilibrium) enter as a
 * per-cell total `for_lines` supplied by the caller (0 when no heavy ion has
 * atomic data).  An element that is off contributes zero wherever the
 * reference indexes ionDenUsed with elementXref = 0.
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define PI_ 3.141592654
#define FOURPI (4. * PI_)
static const double hcRyd_k = 157893.94, hcRyd = 2.1799153e-11, cRyd = 3.2898423e15, hPlanck = 6.6262e-27;

static int locate_d(const float* xa, int n, double x) {
    if (x > (double)xa[n - 1]) return n;
    if (x < (double)xa[0]) return 0;
    int jlow = 0, jup = n + 1;
    for (int it = 0; it < 10000; ++it) {
        if (jup - jlow < 1) break;
        int jm = (jup + jlow) / 2;
        if ((double)xa[jm - 1] == x) return jm;
        if (x > (double)xa[jm - 1]) { if (jlow == jm) break; jlow = jm; } else jup = jm;
    }
    return jlow;
}

static double ion_den(const orc_emission_in* in, size_t c, int elem, int stage) {
    int xr = in->elem_xref[elem - 1];
    if (xr <= 0 || stage < 1 || stage > in->nstages) return 0.;
    size_t C1 = (size_t)in->n_cells + 1;
    return (double)in->ionden[c + C1 * ((size_t)(xr - 1) + (size_t)in->n_elem_used * (size_t)(stage - 1))];
}

/* hydro2phot (source/emission_mod.f90:637-733) */
static double hydro2phot(double nu, int Z, double Te, double Ne) {
    if (Z == 1) {
        double nu0 = 0.7496, y = nu / nu0;
        if (nu >= nu0) return 0.;
        double alphaEffH22S = 0.8368 * pow(Te * 1.e-4, -0.723);
        double Ay = 202.0 * (y * (1 - y) * (1 - pow(4 * y * (1 - y), 0.8)) +
                             0.88 * pow(y * (1 - y), 1.53) * pow(4 * y * (1 - y), 0.8));
        double gNu = hPlanck * y * Ay / 8.2249 * 1e27;
        double Q;
        if (Te <= 10000.) Q = 5.31e-4;
        else if (Te >= 20000.) Q = 4.71e-4;
        else {
            double factor = log10(4.71e-4 / 5.31e-4) / log10(2.);
            Q = pow(10., log10(5.31e-4) + factor * log10(Te / 10000.));
        }
        return alphaEffH22S * gNu / (1. + (Ne * Q) / 8.23);
    } else {
        double nu0 = 3.00, y = nu / nu0;
        if (nu >= nu0) return 0.;
        double a;
        if (Te <= 5000.) a = 6.161;
        else if (Te >= 30000.) a = 2.035;
        else if (Te > 5000. && Te <= 10000.) a = pow(10., log10(6.161) + log10(4.091 / 6.161) / log10(2.) * log10(Te / 5000.));
        else if (Te > 10000. && Te <= 15000.) a = pow(10., log10(4.091) + log10(3.189 / 4.091) / log10(1.5) * log10(Te / 10000.));
        else a = pow(10., log10(3.189) + log10(2.035 / 3.189) / log10(2.) * log10(Te / 15000.));
        double z6 = 64.;
        double Ay = z6 * 0.9994667 * 202.0 * (y * (1 - y) * (1 - pow(4 * y * (1 - y), 0.8)) +
                                               0.88 * pow(y * (1 - y), 1.53) * pow(4 * y * (1 - y), 0.8));
        double gNu = hPlanck * y * Ay / (8.226 * z6) * 1e27;
        return a * gNu;
    }
}

/* interpolate logGamma(T) of species k at log-log in T (fb_ff, source/emission_mod.f90:388-424) */
static void gamma_at_T(const orc_emission_in* in, int k, double Te, double* loc) {
    const int nt = in->n_tk, nl = in->nlim[k];
    const float* lg = in->log_gamma + (size_t)k * nt * 32;
    if (Te <= (double)in->tk[0]) { for (int i = 0; i < nl; ++i) loc[i] = lg[i]; return; }
    if (Te >= (double)in->tk[nt - 1]) { for (int i = 0; i < nl; ++i) loc[i] = lg[(size_t)(nt - 1) * 32 + i]; return; }
    int nT = locate_d(in->tk, nt, Te);
    double factor = log10(Te / (double)in->tk[nT - 1]);
    for (int i = 0; i < nl; ++i) {
        double aFit = ((double)lg[(size_t)nT * 32 + i] - (double)lg[(size_t)(nT - 1) * 32 + i]) /
                      log10((double)in->tk[nT] / (double)in->tk[nT - 1]);
        loc[i] = (double)lg[(size_t)(nT - 1) * 32 + i] + aFit * factor;
    }
}

int orc_emission(const orc_emission_in* in, float* rec_pdf, float* total_lines) {
    const int nb = in->nbins;
    const size_t C1 = (size_t)in->n_cells + 1;
    double *gHI = malloc(sizeof(double) * nb), *gHeI = malloc(sizeof(double) * nb), *gHeII = malloc(sizeof(double) * nb);
    double *gHv = malloc(sizeof(double) * nb), *ff1 = malloc(sizeof(double) * nb), *ff2 = malloc(sizeof(double) * nb);
    double *t2H = malloc(sizeof(double) * nb), *t2He = malloc(sizeof(double) * nb), *t2HeII = malloc(sizeof(double) * nb);
    double *sHI = malloc(sizeof(double) * nb), *sHeI = malloc(sizeof(double) * nb), *sHeII = malloc(sizeof(double) * nb);
    if (!gHI || !gHeI || !gHeII || !gHv || !ff1 || !ff2 || !t2H || !t2He || !t2HeII || !sHI || !sHeI || !sHeII) return 3;
    const int32_t* P = in->ptr;
    const int HIPnuP = P[1], HeIPnuP = P[3], HeIIPnuP = P[5];
    const int HlevXSecP1 = P[0], HeISingXSecP1 = P[2], HeIIXSecP1 = P[4];
    const float* nu = in->nu;
    const double aH = in->elem_abun[0], aHe = in->elem_abun[1];
    double hydroLines[31][16][9];      /* module array: persists across cells like the reference's */
    memset(hydroLines, 0, sizeof(hydroLines));
    for (size_t c = 1; c < C1; ++c) {
        if (!in->compute[c]) continue;
        double Te = in->te[c], NeCell = in->ne[c], Ne = NeCell;
        double sqrTe = sqrt(Te), log10Te = log10(Te), log10Ne = log10(Ne);
        if (Ne < 1.e-5) Ne = 1.e-5;
        for (int i = 0; i < nb; ++i) { gHI[i] = gHeI[i] = gHeII[i] = gHv[i] = ff1[i] = ff2[i] = t2H[i] = t2He[i] = t2HeII[i] = 0.; }
        /* gamma interpolation between series edges */
        double loc[3][32];
        for (int k = 0; k < 3; ++k) gamma_at_T(in, k, Te, loc[k]);
        double* gk[3] = {gHI, gHeI, gHeII};
        for (int k = 0; k < 3; ++k) {
            const int32_t* E = in->gamma_edge_p + k * 32;
            for (int i = 1; i <= in->nlim[k] / 2; ++i) {
                int iup = E[2 * i - 1], ilow = E[2 * i - 2];
                if (iup == ilow) return 4;
                double aFit = (loc[k][2 * i - 1] - loc[k][2 * i - 2]) / ((double)nu[iup - 1] - (double)nu[ilow - 1]);
                for (int j = ilow; j <= iup - 1; ++j)
                    gk[k][j - 1] = pow(10., loc[k][2 * i - 1] + aFit * ((double)nu[j - 1] - (double)nu[iup - 1]));
            }
        }
        /* free_free (ffCoeff, source/emission_mod.f90:782-800) */
        for (int i = 0; i < nb; ++i) {
            double ex = exp(-(double)nu[i] * hcRyd_k / Te);
            ff1[i] = FOURPI * 54.43 * 1. * (double)in->gaunt_ff[i] * ex / sqrTe;
            ff2[i] = FOURPI * 54.43 * 4. * (double)in->gaunt_ff_heii[i] * ex / sqrTe;
        }
        /* Milne relation above the edges */
        const double constant = 4.9874105e-6, statW[3] = {2., 0.5, 2.};
        const int HeIlast = in->gamma_edge_p[32 + in->nlim[1] - 1], HeIIlast = in->gamma_edge_p[64 + in->nlim[2] - 1];
        for (int i = HIPnuP; i <= nb; ++i) {
            double factor = ((double)nu[i - 1] * nu[i - 1] * nu[i - 1]) / (Te * sqrTe);
            double ex = exp((-(double)nu[i - 1] + (double)nu[HIPnuP - 1]) * hcRyd_k / Te);
            int xi = i - HIPnuP + 1 + HlevXSecP1 - 1;
            double xs = (xi >= 1 && xi <= in->n_xsec) ? in->xsec[xi - 1] : 0.;
            gHI[i - 1] = FOURPI * xs * statW[0] * hcRyd * constant * factor * ex * 1e20 * 1e20 + ff1[i - 1];
            if (i >= HeIlast) {
                ex = exp((-(double)nu[i - 1] + (double)nu[HeIPnuP - 1]) * hcRyd_k / Te);
                xi = i - HeIPnuP + 1 + HeISingXSecP1 - 1;
                xs = (xi >= 1 && xi <= in->n_xsec) ? in->xsec[xi - 1] : 0.;
                gHeI[i - 1] = FOURPI * xs * statW[1] * hcRyd * constant * factor * ex * 1e20 * 1e20 + ff1[i - 1];
                if (i >= HeIIlast) {
                    ex = exp((-(double)nu[i - 1] + (double)nu[HeIIPnuP - 1]) * hcRyd_k / Te);
                    xi = i - HeIIPnuP + 1 + HeIIXSecP1 - 1;
                    xs = (xi >= 1 && xi <= in->n_xsec) ? in->xsec[xi - 1] : 0.;
                    gHeII[i - 1] = FOURPI * xs * statW[2] * hcRyd * constant * factor * ex * 1e20 * 1e20 + ff2[i - 1];
                }
            }
        }
        /* heavy-ion free-bound (source/emission_mod.f90:550-614) */
        for (int i = 1; i <= nb; ++i) {
            double sum = 0.;
            for (int t = 0; t < in->n_fb_heavy; ++t) {
                const int32_t* T = in->fb_heavy + 7 * t;
                int elem = T[0], ion = T[1], IPnuP = T[2], highNuP = T[3], xSecP = T[4], g0 = T[5], g1 = T[6];
                if (i >= IPnuP && i < highNuP) {
                    int xi = i + xSecP - IPnuP + 1 - 1;
                    double xs = (xi >= 1 && xi <= in->n_xsec) ? in->xsec[xi - 1] : 0.;
                    double ex = exp((-(double)nu[i - 1] + (double)nu[IPnuP - 1]) * hcRyd_k / Te);
                    sum += ex * xs * ((double)g0 / (double)g1) * ion_den(in, c, elem, ion + 1) * (double)in->elem_abun[elem - 1];
                }
            }
            double factor = (double)nu[i - 1] * nu[i - 1] * nu[i - 1] / (Te * sqrTe);
            gHv[i - 1] = sum * FOURPI * constant * hcRyd * factor * 1e20 * 1e20;
        }
        /* two-photon continua */
        for (int i = 0; i < nb; ++i) { t2H[i] = hydro2phot(nu[i], 1, Te, Ne); t2HeII[i] = hydro2phot(nu[i], 2, Te, Ne); }
        {
            double alpha21S = 6.23 * pow(Te / 10000., -0.827);
            int j = 1;
            for (int i = 1; i <= nb; ++i) {
                double y = (double)nu[i - 1] / 1.514;
                if (y > (double)in->hei2phot[j - 1]) j = j + 1;
                if (j >= 41) break;
                double fit1 = ((double)in->hei2phot[41 + j] - (double)in->hei2phot[41 + j - 1]) /
                              ((double)in->hei2phot[j] - (double)in->hei2phot[j - 1]);
                double fit2 = (double)in->hei2phot[41 + j - 1] - (double)in->hei2phot[j - 1] * fit1;
                double Ay = fit1 * y + fit2;
                if (Ay < 9.2163086E-03) Ay = 0.;
                t2He[i - 1] = alpha21S * Ay * 0.66262 * y / 51.3;
            }
        }
        /* total continuum emission coefficients and the partial sums of setDiffusePDF */
        const double xH2 = ion_den(in, c, 1, 2), xHe2 = ion_den(in, c, 2, 2), xHe3 = ion_den(in, c, 2, 3);
        double normHI = 0., normHeI = 0., normHeII = 0.;
        for (int i = 0; i < nb; ++i) {
            double eHI = (gHI[i] + t2H[i]) * aH * xH2 * Ne + gHv[i] * Ne;
            double eHeI = (gHeI[i] + t2He[i]) * aHe * xHe2 * Ne;
            double eHeII = (gHeII[i] + t2HeII[i]) * aHe * xHe3 * Ne;
            if (eHI < 1.e-15) eHI = 0.;
            if (eHeI < 1.e-15) eHeI = 0.;
            if (eHeII < 1.e-15) eHeII = 0.;
            sHI[i] = cRyd * (double)in->widflx[i] * eHI / 1.e15; normHI += sHI[i];
            sHeI[i] = cRyd * (double)in->widflx[i] * eHeI / 1.e15; normHeI += sHeI[i];
            sHeII[i] = cRyd * (double)in->widflx[i] * eHeII / 1.e15; normHeII += sHeII[i];
        }
        double T4 = Te * 1.e-4;
        double corr = 27.2 * pow(T4, -0.678) * Ne * aHe * xHe2 * 1.45673 * hcRyd * 1e11;
        sHeI[in->j2ts_p - 1] += corr; normHeI += corr;
        {
            double lyA = pow(10., -0.792 * log10(Te) + 6.01) * Ne * xHe3 * aHe;
            for (int i = 0; i < 4; ++i) {
                double line = (i == 3) ? lyA : (double)in->heii_lyman[i] * lyA;
                int p = in->heii_lyman_p[i];
                if (p >= 1) sHeII[p - 1] += line;
                normHeII += line;
            }
        }
        /* RecLinesEmission: hydrogenic lines (source/emission_mod.f90:878-1085) */
        T4 = Te / 10000.;
        int elUp = (T4 > (double)in->hydro_temps[11]) ? 2 : 8;
        for (int izp = 1; izp <= 30; ++izp) {
            if (in->elem_xref[izp - 1] <= 0 || !(in->nstages > izp)) continue;
            int useRow;
            double T4u, Neu, log10Neu;
            if (izp <= elUp) { useRow = izp; T4u = T4; Neu = Ne; log10Neu = log10Ne; }
            else { useRow = 2; T4u = T4 * 4. / (izp * izp); Neu = Ne * 4. / (izp * izp); log10Neu = log10(Ne * 4. / (izp * izp)); }
            int itemp = 1;
            for (int i = 1; i <= 12; ++i) if (T4u > (double)in->hydro_temps[i - 1]) itemp = i;
            if (itemp < 12 && T4u > ((double)in->hydro_temps[itemp] + (double)in->hydro_temps[itemp - 1]) / 2.) itemp = itemp + 1;
            int f = in->hydro_file_map[(useRow - 1) * 12 + (itemp - 1)];
            const float* dens = in->hydro_dens + (size_t)f * 13;
            const float* L = in->hydro_lines + (size_t)f * 13 * 14 * 8;
#define HL(iden, iup, ilow) ((double)L[(((size_t)(iden) - 1) * 14 + ((iup) - 2)) * 8 + ((ilow) - 1)])
            int idenp = 1;
            for (int iden = 1; iden <= 13; ++iden) if (Neu > (double)dens[iden - 1] && dens[iden - 1] > 0.f) idenp = iden;
            int interp = (dens[12] > 0.f && idenp < 13) || (dens[12] == 0.f && idenp < 9);
            for (int iup = 2; iup <= 15; ++iup)
                for (int ilow = 1; ilow <= 8; ++ilow) {
                    double v;
                    if (interp) {
                        if (ilow > (iup - 1 < 8 ? iup - 1 : 8)) continue;   /* only these entries are assigned */
                        v = HL(idenp, iup, ilow) + (HL(idenp + 1, iup, ilow) - HL(idenp, iup, ilow)) *
                                                       (Neu - (double)dens[idenp - 1]) / ((double)dens[idenp] - (double)dens[idenp - 1]);
                    } else {
                        v = HL(idenp, iup, ilow);
                    }
                    hydroLines[izp][iup][ilow] = v;
                }
#undef HL
            double Hbeta;
            const float* HbA = in->hb_coeff + (size_t)((izp <= elUp ? izp : 2) - 1) * 4;
            const float* HbB = in->hb_coeff + 36 + (size_t)((izp <= elUp ? izp : 2) - 1) * 4;
            if (izp <= elUp) {
                if ((izp == 1 && T4 <= 3.) || (izp > 1 && T4 <= (double)in->hydro_temps[11])) {
                    double zfit = (log10Ne - HbA[1]) / HbA[2];
                    double Afit = HbA[0] * exp(-zfit * zfit / 2.) + HbA[3];
                    zfit = (log10Ne - HbB[1]) / HbB[2];
                    double Bfit = HbB[0] * exp(-zfit * zfit / 2.) + HbB[3];
                    Hbeta = pow(10., Afit + Bfit * log10Te);
                } else if (izp == 1 || izp == 2) {
                    double yy1, yy2, x1, x2;
                    if (izp == 1) {
                        const float* e3 = in->rb_edge + 0 * 78 + 2 * 26;   /* rbEdge(1,3,:) */
                        const float* e1 = in->rb_edge + 0 * 78 + 0 * 26;
                        if (idenp < 13) {
                            double w = (Ne - (double)dens[idenp - 1]) / ((double)dens[idenp] - (double)dens[idenp - 1]);
                            yy1 = e3[idenp - 1] + ((double)e3[idenp - 1] - e3[idenp]) * w;
                            yy2 = e3[13 + idenp - 1] + ((double)e3[13 + idenp - 1] - e3[13 + idenp]) * w;
                        } else { yy1 = e3[idenp - 1]; yy2 = e3[13 + idenp - 1]; }
                        x1 = e1[0]; x2 = e1[13];
                    } else {
                        const float* e3 = in->r2a_edge + 2 * 18, *e1 = in->r2a_edge;
                        if (idenp < 13) {
                            double w = (Ne - (double)dens[idenp - 1]) / ((double)dens[idenp] - (double)dens[idenp - 1]);
                            yy1 = e3[idenp - 1] + ((double)e3[idenp - 1] - e3[idenp]) * w;
                            /* r2aEdge(3, 9+idenp+1) lies past the table for idenp = 9: read as r2aEdge(3,18) */
                            yy2 = e3[9 + idenp - 1] + ((double)e3[9 + idenp - 1] - e3[9 + idenp < 18 ? 9 + idenp : 17]) * w;
                        } else { yy1 = e3[idenp - 1]; yy2 = e3[9 + idenp - 1]; }
                        x1 = e1[0]; x2 = e1[9];
                    }
                    double xx = log10(T4 * 1.e4);
                    Hbeta = pow(10., yy1 - (yy1 - yy2) * (xx - x1) / (x2 - x1));
                } else {
                    return 5;   /* the reference stops: "izp insanity" */
                }
            } else {
                double log10TeZ = log10(Te * 4. / (izp * izp));
                double zfit = (log10Neu - HbA[1]) / HbA[2];
                double Afit = HbA[0] * exp(-zfit * zfit / 2.) + HbA[3];
                zfit = (log10Neu - HbB[1]) / HbB[2];
                double Bfit = HbB[0] * exp(-zfit * zfit / 2.) + HbB[3];
                Hbeta = ((double)(izp * izp * izp) / 8.) * pow(10., Afit + Bfit * log10TeZ);
            }
            Hbeta = Hbeta * Ne * ion_den(in, c, izp, izp + 1) * (double)in->elem_abun[izp - 1];
            for (int iup = 2; iup <= 15; ++iup)
                for (int ilow = 1; ilow <= 8; ++ilow) hydroLines[izp][iup][ilow] *= Hbeta;
        }
        /* HeI recombination lines (source/emission_mod.f90:1100-1146) */
        double HeIRec[34];
        {
            double T4h = T4;
            if (T4h < 0.5) T4h = 0.5;
            if (T4h < 2.0) T4h = 2.0;
            int denint;
            if (NeCell <= 100.) denint = 0;
            else if (NeCell <= 1.e4) denint = 1;
            else if (NeCell <= 1.e6) denint = 2;
            else denint = 3;
            for (int i = 0; i < 34; ++i) {
                const float* C0 = in->hei_rec + (size_t)i * 12;   /* [iline][iden][4] */
#define CF(iden, k) ((double)C0[((iden) - 1) * 4 + ((k) - 1)])
                if (denint > 0 && denint < 3) {
                    double x1 = CF(denint, 1) * pow(T4h, CF(denint, 2)) * exp(CF(denint, 3) / T4h);
                    double x2 = CF(denint + 1, 1) * pow(T4h, CF(denint + 1, 2)) * exp(CF(denint + 1, 3) / T4h);
                    HeIRec[i] = x1 + ((x2 - x1) * (Ne - pow(100., denint)) / (pow(100., denint + 1) - pow(100., denint)));
                } else if (denint == 0) {
                    HeIRec[i] = CF(1, 1) * pow(T4h, CF(1, 2)) * exp(CF(1, 3) / T4h);
                } else {
                    HeIRec[i] = CF(3, 1) * pow(T4h, CF(3, 2)) * exp(CF(3, 3) / T4h);
                }
#undef CF
                HeIRec[i] = HeIRec[i] * Ne * aHe * xHe2;
            }
        }
        /* setDiffusePDF: line fraction and the cumulative CDF */
        double normRec = 0.;
        for (int izp = 1; izp <= 30; ++izp)
            for (int iup = 2; iup <= 15; ++iup)
                for (int ilow = 1; ilow <= (iup - 1 < 8 ? iup - 1 : 8); ++ilow) normRec += hydroLines[izp][iup][ilow];
        for (int i = 0; i < 34; ++i) normRec += HeIRec[i];
        double normFor = in->for_lines ? (double)in->for_lines[c] : 0.;
        double tl = normRec + normFor;
        double cum = 0.;
        for (int i = 0; i < nb; ++i) {
            cum = cum + (sHI[i] + sHeI[i] + sHeII[i]);
            rec_pdf[c + C1 * (size_t)i] = (float)cum;
        }
        double last = (double)rec_pdf[c + C1 * (size_t)(nb - 1)];
        for (int i = 0; i < nb; ++i) rec_pdf[c + C1 * (size_t)i] = (float)((double)rec_pdf[c + C1 * (size_t)i] / last);
        rec_pdf[c + C1 * (size_t)(nb - 1)] = 1.f;
        double normalize = normHI + normHeI + normHeII + tl;
        total_lines[c] = (float)(tl / normalize);
    }
    free(gHI); free(gHeI); free(gHeII); free(gHv); free(ff1); free(ff2);
    free(t2H); free(t2He); free(t2HeII); free(sHI); free(sHeI); free(sHeII);
    return 0;
}
