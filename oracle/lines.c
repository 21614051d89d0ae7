/*
 * lines.c - FP64 restatement of the analytical line luminosities and ionic
 * volume averages of outputGas.
 *
 * TEST INFRASTRUCTURE ONLY (checker of libmcx.so's mcx_line_luminosities).
 * Follows
 *   outputGas cell loop               source/output_mod.f90:280-680
 *   forLines (outputGas's copy)       source/output_mod.f90:1943-1984
 *   RecLinesEmission (outputGas's)    source/output_mod.f90:1987-2276
 * Each cell's line emissivities are formed line by line as the reference
 * does (fLineEm(i,j) * elemAbun * ionDen * 1.9865e9, then * Hden * dV) and
 * added in cell order.  The normalisation of :684-805 is left to the caller.
 * Where the reference reads r2aEdge(3, 9+idenp+1) past the table's 18
 * columns (idenp = 9 in the HeII edge branch) this reads r2aEdge(3,18).
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define R(x) ((double)(x##f))     /* a default-REAL constant of the reference */

static double ion_frac(const orc_emission_in* em, int elem, int stage, int cell) {
    const int xr = em->elem_xref[elem - 1];
    if (xr <= 0 || stage > em->nstages) return 0.;
    const size_t C1 = (size_t)em->n_cells + 1;
    return (double)em->ionden[((size_t)(stage - 1) * em->n_elem_used + (xr - 1)) * C1 + cell];
}

/* itemp of the hydroLinesTemps search (source/output_mod.f90:2017-2025) */
static int temp_bin(const float* temps, double t4) {
    int itemp = 1;
    for (int i = 1; i <= 12; ++i)
        if (t4 > (double)temps[i - 1]) itemp = i;
    if (itemp < 12) {
        if (t4 > ((double)temps[itemp] + (double)temps[itemp - 1]) / 2.) itemp = itemp + 1;
    }
    return itemp;
}

/* hydroLines(izp, :, :) of one cell into hl[14][8] (source/output_mod.f90:2027-2229) */
static void rec_lines_izp(const orc_emission_in* em, int izp, int elUp, int itemp, double Te, double Ne, int cell,
                          double hl[14][8]) {
    const double T4 = Te / 10000.;
    const double log10Te = log10(Te), log10Ne = log10(Ne);
    const float* HbA;
    const float* HbB;
    double dens[13];
    int idenp, f;
    double Hbeta;
    memset(hl, 0, sizeof(double) * 14 * 8);
    if (izp <= elUp) {
        f = em->hydro_file_map[(izp - 1) * 12 + (itemp - 1)];
        for (int i = 0; i < 13; ++i) dens[i] = em->hydro_dens[(size_t)f * 13 + i];
        const float* loc = em->hydro_lines + (size_t)f * 13 * 14 * 8;
        idenp = 1;
        for (int iden = 1; iden <= 13; ++iden)
            if (Ne >= dens[iden - 1] && dens[iden - 1] > 0.) idenp = iden;
        if ((dens[12] > 0. && idenp < 13) || (dens[12] == 0. && idenp < 9)) {
            for (int iup = 2; iup <= 15; ++iup)
                for (int ilow = 1; ilow <= (iup - 1 < 8 ? iup - 1 : 8); ++ilow) {
                    double a = loc[((idenp - 1) * 14 + (iup - 2)) * 8 + (ilow - 1)];
                    double b = loc[(idenp * 14 + (iup - 2)) * 8 + (ilow - 1)];
                    hl[iup - 2][ilow - 1] = a + (b - a) * (Ne - dens[idenp - 1]) / (dens[idenp] - dens[idenp - 1]);
                }
        } else {
            for (int iup = 2; iup <= 15; ++iup)
                for (int ilow = 1; ilow <= 8; ++ilow)
                    hl[iup - 2][ilow - 1] = loc[((idenp - 1) * 14 + (iup - 2)) * 8 + (ilow - 1)];
        }
        if ((izp == 1 && T4 <= 3.) || (izp > 1 && T4 <= (double)em->hydro_temps[11])) {
            HbA = em->hb_coeff + (izp - 1) * 4;
            HbB = em->hb_coeff + 36 + (izp - 1) * 4;
            double zfit = (log10Ne - HbA[1]) / HbA[2];
            double Afit = HbA[0] * exp(-zfit * zfit / 2.) + HbA[3];
            zfit = (log10Ne - HbB[1]) / HbB[2];
            double Bfit = HbB[0] * exp(-zfit * zfit / 2.) + HbB[3];
            Hbeta = pow(10., Afit + Bfit * log10Te);
        } else {
            double yy1, yy2, x1, x2;
            if (izp == 1) {
                const float* r3 = em->rb_edge + 2 * 26;        /* rbEdge(1,3,:) */
                if (idenp < 13) {
                    yy1 = r3[idenp - 1] + ((double)r3[idenp - 1] - r3[idenp]) * (Ne - dens[idenp - 1]) /
                                              (dens[idenp] - dens[idenp - 1]);
                    yy2 = r3[13 + idenp - 1] + ((double)r3[13 + idenp - 1] - r3[13 + idenp]) *
                                                   (Ne - dens[idenp - 1]) / (dens[idenp] - dens[idenp - 1]);
                } else {
                    yy1 = r3[idenp - 1];
                    yy2 = r3[13 + idenp - 1];
                }
                x1 = em->rb_edge[0];
                x2 = em->rb_edge[13];
            } else {
                const float* r3 = em->r2a_edge + 2 * 18;       /* r2aEdge(3,:) */
                if (idenp < 13) {
                    int hi = 9 + idenp < 18 ? 9 + idenp : 17;
                    yy1 = r3[idenp - 1] + ((double)r3[idenp - 1] - r3[idenp]) * (Ne - dens[idenp - 1]) /
                                              (dens[idenp] - dens[idenp - 1]);
                    yy2 = r3[9 + idenp - 1] + ((double)r3[9 + idenp - 1] - r3[hi]) * (Ne - dens[idenp - 1]) /
                                                  (dens[idenp] - dens[idenp - 1]);
                } else {
                    yy1 = r3[idenp - 1];
                    yy2 = r3[9 + idenp - 1];
                }
                x1 = em->r2a_edge[0];
                x2 = em->r2a_edge[9];
            }
            double xx = log10(T4 * 1.e4);
            Hbeta = yy1 - (yy1 - yy2) * (xx - x1) / (x2 - x1);
            Hbeta = pow(10., Hbeta);
        }
    } else {
        const double T4z = T4 * 4. / (double)(izp * izp);
        const double log10TeZ = log10(Te * 4. / (double)(izp * izp));
        const double Nez = Ne * 4. / (double)(izp * izp);
        const double log10Nez = log10(Ne * 4. / (double)(izp * izp));
        const int itz = temp_bin(em->hydro_temps, T4z);
        f = em->hydro_file_map[1 * 12 + (itz - 1)];
        for (int i = 0; i < 13; ++i) dens[i] = em->hydro_dens[(size_t)f * 13 + i];
        const float* loc = em->hydro_lines + (size_t)f * 13 * 14 * 8;
        idenp = 1;
        for (int iden = 1; iden <= 13; ++iden)
            if (Nez >= dens[iden - 1] && dens[iden - 1] > 0.) idenp = iden;
        if ((dens[12] > 0. && idenp < 13) || (dens[12] == 0. && idenp < 9)) {
            for (int iup = 2; iup <= 15; ++iup)
                for (int ilow = 1; ilow <= (iup - 1 < 8 ? iup - 1 : 8); ++ilow) {
                    double a = loc[((idenp - 1) * 14 + (iup - 2)) * 8 + (ilow - 1)];
                    double b = loc[(idenp * 14 + (iup - 2)) * 8 + (ilow - 1)];
                    hl[iup - 2][ilow - 1] = a + (b - a) * (Nez - dens[idenp - 1]) / (dens[idenp] - dens[idenp - 1]);
                }
        } else {
            for (int iup = 2; iup <= 15; ++iup)
                for (int ilow = 1; ilow <= 8; ++ilow)
                    hl[iup - 2][ilow - 1] = loc[((idenp - 1) * 14 + (iup - 2)) * 8 + (ilow - 1)];
        }
        HbA = em->hb_coeff + 1 * 4;
        HbB = em->hb_coeff + 36 + 1 * 4;
        double zfit = (log10Nez - HbA[1]) / HbA[2];
        double Afit = HbA[0] * exp(-zfit * zfit / 2.) + HbA[3];
        zfit = (log10Nez - HbB[1]) / HbB[2];
        double Bfit = HbB[0] * exp(-zfit * zfit / 2.) + HbB[3];
        Hbeta = ((double)(izp * izp * izp) / 8.) * pow(10., Afit + Bfit * log10TeZ);
    }
    Hbeta = Hbeta * Ne * ion_frac(em, izp, izp + 1, cell) * (double)em->elem_abun[izp - 1];
    for (int iup = 2; iup <= 15; ++iup)
        for (int ilow = 1; ilow <= 8; ++ilow) hl[iup - 2][ilow - 1] = hl[iup - 2][ilow - 1] * Hbeta;
}

int orc_line_sums(const orc_emission_in* em, const orc_balance_in* bal, const double* vol, const int32_t* black,
                  orc_lines_out* out) {
    const int C = em->n_cells, S = em->nstages;
    const size_t C1 = (size_t)C + 1;
    double* n = (double*)malloc(sizeof(double) * 32);
    double* fl = (double*)malloc(sizeof(double) * 32 * 32);
    out->hbeta = 0.;
    out->n_cells = 0;
    memset(out->hydro, 0, sizeof(double) * 30 * 14 * 8);
    memset(out->hei, 0, sizeof(double) * 34);
    memset(out->forb, 0, sizeof(double) * (size_t)bal->n_atoms * 30 * 30);
    memset(out->ion_num, 0, sizeof(double) * 30 * S);
    memset(out->ion_den, 0, sizeof(double) * 30 * S);
    for (int cell = 1; cell <= C; ++cell) {
        if (black[cell] >= 1) continue;
        out->n_cells++;
        const double Te = em->te[cell], Ne = em->ne[cell];
        const double Hden = bal->hden[cell], dV = vol[cell];
        const double T4 = Te / 10000.;
        const int itemp = temp_bin(em->hydro_temps, T4);
        const int elUp = T4 > (double)em->hydro_temps[11] ? 2 : 8;

        /* RecLinesEmission: hydrogenic lines, Hbeta (source/output_mod.f90:393-409) */
        double hl[14][8];
        for (int iz = 1; iz <= 30; ++iz) {
            if (em->elem_xref[iz - 1] <= 0 || !(S > iz)) continue;
            rec_lines_izp(em, iz, elUp, itemp, Te, Ne, cell, hl);
            if (iz == 1) {
                double hb = hl[4 - 2][2 - 1] * Hden * dV;
                if (hb > R(1.e-35)) out->hbeta += hb;
            }
            for (int iup = 2; iup <= 15; ++iup)
                for (int ilow = 1; ilow <= (iup - 1 < 8 ? iup - 1 : 8); ++ilow)
                    out->hydro[((iz - 1) * 14 + (iup - 2)) * 8 + (ilow - 1)] += hl[iup - 2][ilow - 1] * Hden * dV;
        }

        /* HeI recombination lines (source/output_mod.f90:2241-2273) */
        if (em->elem_xref[1] > 0) {
            int denint;
            if (Ne <= 100.) denint = 0;
            else if (Ne > 100. && Ne <= 1.e4) denint = 1;
            else if (Ne > 1.e4 && Ne <= 1.e6) denint = 2;
            else denint = 3;
            for (int i = 1; i <= 34; ++i) {
                const float* c0 = em->hei_rec + (size_t)(i - 1) * 12;   /* HeIrecLineCoeff(i,:,:) */
                double r;
                if (denint > 0 && denint < 3) {
                    const float* p = c0 + (denint - 1) * 4;
                    const float* q = c0 + denint * 4;
                    double x1 = p[0] * pow(T4, (double)p[1]) * exp((double)p[2] / T4);
                    double x2 = q[0] * pow(T4, (double)q[1]) * exp((double)q[2] / T4);
                    double lo = pow(100., (double)denint), hi = pow(100., (double)(denint + 1));
                    r = x1 + (x2 - x1) * (Ne - lo) / (hi - lo);
                } else if (denint == 0) {
                    r = c0[0] * pow(T4, (double)c0[1]) * exp((double)c0[2] / T4);
                } else {
                    const float* p = c0 + 2 * 4;
                    r = p[0] * pow(T4, (double)p[1]) * exp((double)p[2] / T4);
                }
                r = r * Ne * (double)em->elem_abun[1] * ion_frac(em, 2, 2, cell);
                out->hei[i - 1] += r * Hden * dV;
            }
        }

        /* forLines: forbidden lines (source/output_mod.f90:1943-1984, :410-432) */
        for (int elem = 3; elem <= 30; ++elem) {
            if (em->elem_xref[elem - 1] <= 0) continue;
            const int top = elem + 1 < S ? elem + 1 : S;
            for (int ion = 1; ion <= top; ++ion) {
                const int atom = bal->atom_index[(elem - 1) * 31 + (ion - 1)];
                if (atom < 0) continue;
                const int nLev = bal->atom_hdr[atom * ORC_AT_HDR + ORC_AT_NLEV];
                const double x = ion_frac(em, elem, ion, cell);
                double up = 0.;
                if (ion < top && x > 0.) up = ion_frac(em, elem, ion + 1, cell) / x;
                orc_equilibrium(bal, atom, Te, Ne, up, 1, n, fl);
                for (int i = 1; i <= nLev; ++i)
                    for (int j = 1; j <= nLev; ++j) {
                        double v = fl[(i - 1) * nLev + (j - 1)] * (double)em->elem_abun[elem - 1] * x;
                        v = v * R(1.9865e9);
                        out->forb[((size_t)atom * 30 + (i - 1)) * 30 + (j - 1)] += v * Hden * dV;
                    }
            }
        }

        /* ionic temperatures and fractions (source/output_mod.f90:644-674) */
        const double factor1 = Te * Ne * Hden * dV, factor2 = Ne * Hden * dV;
        for (int elem = 1; elem <= 30; ++elem) {
            if (em->elem_xref[elem - 1] <= 0) continue;
            const int top = elem + 1 < S ? elem + 1 : S;
            for (int ion = 1; ion <= top; ++ion) {
                const double x = ion_frac(em, elem, ion, cell);
                out->ion_num[(elem - 1) * S + (ion - 1)] += x * factor1;
                out->ion_den[(elem - 1) * S + (ion - 1)] += x * factor2;
            }
        }
    }
    (void)C1;
    free(n);
    free(fl);
    return 0;
}
