/*
 * opacity.c - FP64 restatement of the per-cell opacity of MOCASSIN.
 *
 * TEST INFRASTRUCTURE ONLY (checker of libmcx.so's opacity kernel).  Follows
 *   ionizationDriver  source/ionization_mod.f90:26-131
 *   BoltGaunt         source/ionization_mod.f90:136-178
 *   getGauntFF        source/ionization_mod.f90:196-334
 *   eDenSum           source/ionization_mod.f90:338-351
 *   addOpacity        source/ionization_mod.f90:353-477
 * including two behaviours of the reference that change the result:
 *   - ionizationDriver fills density(n,i) only for i <= min(n,nstages), so
 *     density(1,2) (H+) and density(2,3) (He++) stay zero in the free-free
 *     prefactor of addOpacity (source/ionization_mod.f90:71-84, :366-367);
 *   - an empty shell (elementP(:,:,:,1:2) = 2,1) still adds one term
 *     xSecArray(elementP(:,:,:,3)) * density at bin 2, because inOpacity's
 *     loop runs from nuLowP to max(nuLowP, min(nuHighP, nbins))
 *     (source/ionization_mod.f90:451-476).
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

static const double kDD[88] = {
    8.986940175e+00, -4.009515855e+00, 8.808871266e-01, 2.640245111e-02, -4.580645915e-02, -3.568055702e-03,
    2.827798067e-03, 3.365860195e-04, -8.006936989e-01, 9.466021705e-01, 9.043402532e-02, -9.608451450e-02,
    -1.885629865e-02, 1.050313890e-02, 2.800889961e-03, -1.078209202e-03, -3.781305103e-01, 1.102726332e-01,
    -1.543619180e-02, 8.310561114e-03, 2.179620525e-02, 4.259726289e-03, -4.181588794e-03, -1.770208330e-03,
    1.877213132e-02, -1.004885705e-01, -5.483366378e-02, -4.520154409e-03, 8.366530426e-03, 3.700273930e-03,
    6.889320423e-04, 9.460313195e-05, 7.300158392e-02, 3.576785497e-03, -4.545307025e-03, -1.017965604e-02,
    -9.530211924e-03, -3.450186162e-03, 1.040482914e-03, 1.407073544e-03, -1.744671550e-03, 2.864013856e-02,
    1.903394837e-02, 7.091074494e-03, -9.668371391e-04, -2.999107465e-03, -1.820642230e-03, -3.874082085e-04,
    -1.707268366e-02, -4.694254776e-03, 1.311691517e-03, 5.316703136e-03, 5.178193095e-03, 2.451228935e-03,
    -2.277321615e-05, -8.182359057e-04, 2.567331664e-04, -9.155339970e-03, -6.997479192e-03, -3.571518641e-03,
    -2.096101038e-04, 1.553822487e-03, 1.509584686e-03, 6.212627837e-04, 4.098322531e-03, 1.635218463e-03,
    -5.918883504e-04, -2.333091048e-03, -2.484138313e-03, -1.359996060e-03, -5.371426147e-05, 5.553549563e-04,
    3.837562402e-05, 2.938325230e-03, 2.393747064e-03, 1.328839809e-03, 9.135013312e-05, -7.137252303e-04,
    -7.656848158e-04, -3.504683798e-04, -8.491991820e-04, -3.615327726e-04, 3.148015257e-04, 8.909207650e-04,
    9.869737522e-04, 6.134671184e-04, 1.068883394e-04, -2.046080100e-04};

void orc_gaunt_ff(double z, double log10te, const float* nu, int32_t n, double* g) {
    /* d(j,i) = dd(j + 8(i-1)), j = 1..8, i = 1..11 */
#define D(j, i) kDD[((j) - 1) + 8 * ((i) - 1)]
    double xlrkt;
    if (log10te < 2.5) xlrkt = 5.1983649 - 2.5;
    else if (log10te > 8.) xlrkt = 5.1983649 - 8.;
    else xlrkt = 5.1983649 - log10te;
    double txg = 0.66666667 * (2.0 * z + xlrkt);
    double gamma2 = pow(10., txg * 1.5);
    double con = 0.72727273 * xlrkt + 0.90909091;
    double b[12], c[9];
    for (int j = 1; j <= 8; ++j) {
        int ir = 9;
        b[11] = D(j, 11);
        b[10] = txg * b[11] + D(j, 10);
        for (int i = 1; i <= 9; ++i) {
            b[ir] = txg * b[ir + 1] - b[ir + 2] + D(j, ir);
            ir = ir - 1;
        }
        c[j] = 0.25 * (b[1] - b[3]);
    }
    for (int i = 0; i < n; ++i) {
        double xlf = log10((double)nu[i]);
        double txu = 0.72727273 * xlf + con;
        double u = pow(10., (txu - .90909091) / .72727273);
        if (fabs(txu) <= 2.0) {
            int ir = 6;
            b[8] = c[8];
            b[7] = txu * b[8] + c[7];
            for (int j = 1; j <= 6; ++j) {
                b[ir] = txu * b[ir + 1] - b[ir + 2] + c[ir];
                ir = ir - 1;
            }
            g[i] = b[1] - b[3];
        } else if (log10(u) < -4.0 && gamma2 < 0.3) {
            g[i] = 0.551329 * log(2.24593 / u);
        } else if (log10(u) < -4.0 && gamma2 >= 0.3) {
            g[i] = 0.551329 * log(0.944931 / u / sqrt(gamma2));
        } else if (txu > 2.0) {
            if (log10(gamma2) < -3.) g[i] = sqrt(0.9549297 / u);
            else if (log10(gamma2) < 0.0) {
                double slope = (sqrt(12 * gamma2 / u) - sqrt(0.9549297 / u)) / 3.0;
                g[i] = sqrt(12 * gamma2 / u) + slope * log10(gamma2);
            } else {
                double v = sqrt(12. * gamma2 / u);
                g[i] = v < 1.05 ? v : 1.05;
            }
        } else {
            g[i] = 0.;   /* unreachable for txu < -2 (then log10(u) < -4) */
        }
    }
#undef D
}

void orc_gaunt_cache(int32_t nx, int32_t ny, int32_t nz, const int32_t* active, const float* te,
                     const uint8_t* compute, float* te_old, float* gaunt_te) {
    for (int i = 1; i <= nx; ++i)
        for (int j = 1; j <= ny; ++j)
            for (int k = 1; k <= nz; ++k) {
                int c = active[(size_t)(i - 1) + (size_t)nx * ((size_t)(j - 1) + (size_t)ny * (size_t)(k - 1))];
                if (c <= 0 || !compute[c]) continue;
                float t = te[c];
                if (fabsf(1.f - *te_old / t) > 0.10f) *te_old = t;
                gaunt_te[c] = *te_old;
            }
}

int orc_opacity(const orc_opacity_in* in, float* opacity) {
    const int nb = in->nbins, S = in->nstages, E = in->n_elem_used;
    const size_t C1 = (size_t)in->n_cells + 1;
    const double Te1Ryd = 1.578866e5;
    double* gff = (double*)malloc(sizeof(double) * (size_t)nb);
    double* boltz = (double*)malloc(sizeof(double) * (size_t)nb);
    double* op = (double*)malloc(sizeof(double) * (size_t)nb);
    if (!gff || !boltz || !op) { free(gff); free(boltz); free(op); return 3; }
    const int32_t* P = in->ptr;
    for (size_t c = 1; c < C1; ++c) {
        if (!in->compute[c]) continue;
        const double Te = in->te[c], Ne = in->ne[c], Hden = in->hden[c];
        /* density(n,i) = ionDen * abundance * Hden for i <= min(n, nstages) */
        double dens[31][32];
        memset(dens, 0, sizeof(dens));
        for (int n = 1; n <= 30; ++n) {
            int xr = in->elem_xref[n - 1];
            if (xr <= 0) continue;
            int top = n < S ? n : S;
            for (int i = 1; i <= top; ++i)
                dens[n][i] = (double)in->ionden[c + C1 * ((size_t)(xr - 1) + (size_t)E * (size_t)(i - 1))] *
                             (double)in->elem_abun[n - 1] * Hden;
        }
        /* BoltGaunt */
        int mx = nb + 1;
        for (int i = 1; i <= nb; ++i) {
            double ex = Te1Ryd / Te + (double)in->nu[i - 1];
            if (ex > 84.) { mx = i; break; }
            boltz[i - 1] = exp(-ex);
        }
        for (int i = mx; i <= nb; ++i) boltz[i - 1] = 0.;
        orc_gaunt_ff(0., log10((double)in->gaunt_te[c]), in->nu, nb, gff);
        /* eDenSum */
        double eden = 0.;
        for (int n = 3; n <= 30; ++n) {
            int top = n < S - 1 ? n : S - 1;
            for (int i = 1; i <= top; ++i) eden += (double)(i * i) * dens[n][i + 1];
        }
        /* addOpacity: free-free */
        double fac1 = (Ne / 1.e10) * ((dens[1][2] + dens[2][2] + 4. * dens[2][3] + eden) / 1.e10) / sqrt(Te);
        double fac2 = fac1 * Te1Ryd / Te;
        const int brems = P[ORC_P_BREMSXSECP];
        for (int i = 1; i <= nb; ++i) {
            double xs = in->xsec[i - 1 + brems - 1];
            if (boltz[i - 1] < 0.995) op[i - 1] = xs * (1. - boltz[i - 1]) * gff[i - 1] * fac1;
            else op[i - 1] = xs * (double)in->nu[i - 1] * gff[i - 1] * fac2;
        }
#define IN_OPACITY(xSecP, lo, hi, den)                                             \
        do {                                                                       \
            int k_ = (xSecP) - (lo);                                               \
            int iup_ = (hi) < nb ? (hi) : nb;                                      \
            if (iup_ < (lo)) iup_ = (lo);                                          \
            for (int i_ = (lo); i_ <= iup_; ++i_) {                                \
                int xi_ = i_ + k_;                                                 \
                double xs_ = (xi_ >= 1 && xi_ <= in->n_xsec) ? (double)in->xsec[xi_ - 1] : 0.; \
                op[i_ - 1] += xs_ * (den);                                         \
            }                                                                      \
        } while (0)
        IN_OPACITY(P[ORC_P_HLEVXSECP1], P[ORC_P_HLEVNUP1], nb, dens[1][1]);
        IN_OPACITY(P[ORC_P_HEISINGXSECP1], P[ORC_P_HEILEVNUP1], nb, dens[2][1]);
        IN_OPACITY(P[ORC_P_HEIIXSECP1], P[ORC_P_HEIILEVNUP1], nb, dens[2][2]);
        for (int n = 3; n <= 30; ++n) {
            if (in->elem_xref[n - 1] <= 0) continue;
            int top = n < S ? n : S;
            for (int ion = 1; ion <= top; ++ion) {
                int ns = in->n_shells[(n - 1) * 30 + (ion - 1)];
                for (int sh = 1; sh <= ns; ++sh) {
                    const int32_t* e = in->element_p + (((size_t)(n - 1) * 30 + (ion - 1)) * 7 + (sh - 1)) * 3;
                    IN_OPACITY(e[2], e[0], e[1], dens[n][ion]);
                }
            }
        }
#undef IN_OPACITY
        if (in->lg_compton)
            for (int i = 1; i <= nb; ++i) op[i - 1] += (double)in->kn_sigma_t[i - 1] * Ne;
        for (int i = 1; i <= nb; ++i) opacity[c + C1 * (size_t)(i - 1)] = (float)op[i - 1];
    }
    free(gff); free(boltz); free(op);
    return 0;
}
