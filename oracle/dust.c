/*
 * dust.c - CPU restatement of the grain phases of a dust-only grid, in the
 * reference's FP32 arithmetic:
 *   dust opacity    iterateMC's grain contribution (source/iteration_mod.f90:194-246)
 *   dust emission   setDustPDF (source/emission_mod.f90:1921-1986)
 *   grain balance   getDustT (source/update_mod.f90:3346-3453) with updateCell's
 *                   no-hit test and convergence flag (source/update_mod.f90:104-265)
 *
 * TEST INFRASTRUCTURE ONLY: the checker of libmcx.so's dust kernels.
 */
#include "oracle.h"

#include <math.h>
#include <string.h>

#define NTEMPS 3000

static float td_at(const float* td, int n, int ai, int nsz, int c, int C1) {
    return td[((size_t)n * (nsz + 1) + ai) * C1 + c];
}

/* getFlux of source/continuum_mod.f90:358-405 for a blackbody */
static float blackbody(float energy, float temperature) {
    const float hcRyd_k = 157893.94f, hPlanck = 6.6262e-27f;
    const float constant = 0.5250229f / hPlanck;
    if (hcRyd_k * energy / temperature > 86.f)
        return constant * energy * energy * energy * expf(-hcRyd_k * energy / temperature);
    float denominator = expf(hcRyd_k * energy / temperature) - 1.f;
    if (denominator <= 0.f) return 3.32154e-6f * energy * energy * temperature / hPlanck;
    return constant * energy * energy * energy / denominator;
}

int orc_dust_opacity(const orc_dust_in* in, const float* ndust, const float* tdust, float* opacity, float* sca_opac) {
    const int C1 = in->n_cells + 1, nb = in->nbins, nsz = in->n_sizes;
    for (int c = 1; c < C1; ++c)
        for (int f = 0; f < nb; ++f) {
            float sca = 0.f, ab = 0.f;
            for (int n = 0; n < in->n_species; ++n)
                for (int ai = 0; ai < nsz; ++ai)
                    if (td_at(tdust, n + 1, ai + 1, nsz, c, C1) < in->tsub[n]) {
                        size_t o = ((size_t)n * nsz + ai) * nb + f;
                        sca = sca + in->abun[n] * in->weight[ai] * ndust[c] * in->csca[o];
                        ab = ab + in->abun[n] * in->weight[ai] * ndust[c] * in->cabs[o];
                    }
            sca_opac[(size_t)f * C1 + c] = sca;
            opacity[(size_t)f * C1 + c] = opacity[(size_t)f * C1 + c] + (sca + ab);
        }
    return 0;
}

int orc_dust_pdf(const orc_dust_in* in, const float* tdust, float* pdf) {
    const int C1 = in->n_cells + 1, nb = in->nbins, nsz = in->n_sizes;
    for (int c = 1; c < C1; ++c) {
        for (int i = 0; i < nb; ++i) pdf[(size_t)i * C1 + c] = 0.f;
        for (int n = 0; n < in->n_species; ++n)
            for (int ai = 0; ai < nsz; ++ai) {
                float td = td_at(tdust, n + 1, ai + 1, nsz, c, C1);
                if (td > 0.f && td < in->tsub[n])
                    for (int i = 0; i < nb; ++i) {
                        float bb = blackbody(in->nu[i], td);
                        pdf[(size_t)i * C1 + c] = pdf[(size_t)i * C1 + c] +
                            in->cabs[((size_t)n * nsz + ai) * nb + i] * bb * in->widflx[i] * in->weight[ai] * in->abun[n];
                    }
            }
        for (int i = 1; i < nb; ++i) pdf[(size_t)i * C1 + c] = pdf[(size_t)(i - 1) * C1 + c] + pdf[(size_t)i * C1 + c];
        float tot = pdf[(size_t)(nb - 1) * C1 + c];
        for (int i = 0; i < nb; ++i) pdf[(size_t)i * C1 + c] = pdf[(size_t)i * C1 + c] / tot;
        pdf[(size_t)(nb - 1) * C1 + c] = 1.f;
    }
    return 0;
}

/* locate (source/interpolation_mod.f90:49-106) on an ascending table */
static int locate_asc(const float* xa, int n, float x) {
    if (x > xa[n - 1]) return n;
    if (x < xa[0]) return 0;
    int jlow = 0, jup = n + 1;
    for (int it = 0; it < 10000; ++it) {
        if (jup - jlow < 1) break;
        int jm = (jup + jlow) / 2;
        if (xa[jm - 1] == x) return jm;
        if (x > xa[jm - 1]) {
            if (jlow == jm) break;
            jlow = jm;
        } else {
            jup = jm;
        }
    }
    return jlow;
}

int orc_dust_t(const orc_dust_in* in, const double* jste, float* tdust, int32_t* converged, int32_t* black,
               orc_dust_stats* st) {
    const int C1 = in->n_cells + 1, nb = in->nbins, nsz = in->n_sizes;
    const float pi = 3.141592654f;
    memset(st, 0, sizeof(*st));
    for (int c = 1; c < C1; ++c) {
        int hit = 0;
        for (int i = 0; i < nb; ++i)
            if ((float)jste[(size_t)i * C1 + c] > 0.f) { hit = 1; break; }
        black[c] = hit ? 0 : 1;
        converged[c] = 0;
        if (!hit) { st->no_hit += 1; continue; }
        float xOld = tdust[c];
        for (int n = 0; n <= in->n_species; ++n)
            for (int ai = 0; ai <= nsz; ++ai) tdust[((size_t)n * (nsz + 1) + ai) * C1 + c] = 0.f;
        for (int n = 0; n < in->n_species; ++n) {
            for (int ai = 0; ai < nsz; ++ai) {
                const float* ca = in->cabs + ((size_t)n * nsz + ai) * nb;
                float integral = 0.f;
                for (int i = 0; i < nb; ++i) integral = integral + ca[i] * ((float)jste[(size_t)i * C1 + c] / pi);
                const float* em = in->em_int + ((size_t)n * nsz + ai) * NTEMPS;
                int iT = locate_asc(em, NTEMPS, integral);
                float t;
                if (iT <= 0) t = 1.f;
                else if (iT >= NTEMPS) t = (float)NTEMPS;
                else t = (float)iT + (integral - em[iT - 1]) * ((float)(iT + 1) - (float)iT) / (em[iT] - em[iT - 1]);
                tdust[((size_t)(n + 1) * (nsz + 1) + (ai + 1)) * C1 + c] = t;
                float* tn0 = &tdust[((size_t)(n + 1) * (nsz + 1)) * C1 + c];
                *tn0 = *tn0 + t * in->weight[ai];
            }
            tdust[c] = tdust[c] + tdust[((size_t)(n + 1) * (nsz + 1)) * C1 + c] * in->abun[n];
        }
        float delta = (tdust[c] - xOld) / xOld;
        converged[c] = fabsf(delta) <= in->xhi_limit ? 1 : 0;
        st->updated += 1;
        if (converged[c]) st->converged += 1;
    }
    return 0;
}
