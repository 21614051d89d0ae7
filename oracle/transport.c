/*
 * transport.c - FP64 restatement of the MOCASSIN Monte Carlo packet transport.
 *
 * TEST INFRASTRUCTURE ONLY (the checker of libmcx.so's transport kernels and
 * the CPU baseline of bench.py).  Follows, for a single mother grid without
 * plane-parallel illumination, fluorescence or sub-grids:
 *   energyPacketDriver   source/photon_mod.f90:28-416
 *   energyPacketRun      source/photon_mod.f90:418-741
 *   initPhotonPacket     source/photon_mod.f90:744-896
 *   getNu2               source/photon_mod.f90:928-972
 *   newPhotonPacket      source/photon_mod.f90:976-1756
 *   pathSegment          source/photon_mod.f90:1758-4085
 *   comptonScatter       source/photon_mod.f90:6805-6848
 *   randomUnitVector     source/vector_mod.f90:303-314
 *   locate               source/interpolation_mod.f90:49-106
 * The reference draws from the Fortran intrinsic random_number; here packet p
 * draws its k-th uniform u = (x + 0.5) 2^-32 from Philox4x32-10 word k%4 of
 * counter (p_lo, p_hi, k/4, 0), so that the GPU kernels can reproduce each
 * packet history exactly.  Wherever the reference uses `1 - random_number`
 * this uses `1 - u`.
 * Jste(0,:) (the dump row of inactive cells, never read by the reference) is
 * not accumulated.
 */
#include "oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* log, sin and cos from the portable FP64 routines that the device's FP64
 * transport uses too, so that every packet history is the same on both sides */
#include "mcx_fmath.h"
#define log(x) mcx_fm_log(x)
#define sin(x) mcx_fm_sin(x)
#define cos(x) mcx_fm_cos(x)

/* ------------------------------------------------------------ Philox */
static inline void mulhilo32(uint32_t a, uint32_t b, uint32_t* hi, uint32_t* lo) {
    uint64_t p = (uint64_t)a * (uint64_t)b;
    *hi = (uint32_t)(p >> 32);
    *lo = (uint32_t)p;
}

void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0, lo0, hi1, lo1;
        mulhilo32(0xD2511F53u, c0, &hi0, &lo0);
        mulhilo32(0xCD9E8D57u, c2, &hi1, &lo1);
        uint32_t n0 = hi1 ^ c1 ^ k0, n1 = lo1, n2 = hi0 ^ c3 ^ k1, n3 = lo0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
        if (r < 9) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

typedef struct {
    uint32_t key[2];
    uint32_t pid[2];
    uint32_t buf[4];
    uint64_t k;
} rng_t;

static void rng_init(rng_t* r, uint64_t seed, uint64_t pid) {
    r->key[0] = (uint32_t)seed; r->key[1] = (uint32_t)(seed >> 32);
    r->pid[0] = (uint32_t)pid;  r->pid[1] = (uint32_t)(pid >> 32);
    r->k = 0;
}

static double urand(rng_t* r) {
    if ((r->k & 3u) == 0) {
        uint32_t ctr[4] = {r->pid[0], r->pid[1], (uint32_t)(r->k >> 2), (uint32_t)(r->k >> 34)};
        orc_philox4x32_10(ctr, r->key, r->buf);
    }
    uint32_t x = r->buf[r->k & 3u];
    r->k++;
    return ((double)x + 0.5) * (1.0 / 4294967296.0);
}

/* ------------------------------------------------------------ helpers */
typedef struct {
    double x, y, z;
} vec3;

typedef struct {
    vec3 pos, dir;
    int xP, yP, zP;     /* 1-based */
    int nuP;            /* 1-based; 0 for line packets */
    double nu;
    int lgStellar, lgLine;
    int origin;         /* origin cell id */
} packet_t;

/* J entries are merged across threads in chunks of this many; a thread marks
 * the chunks it deposits into, so the merge visits only those */
#define JCHUNK 512

#define R_PI 3.141592654     /* pi of source/constants_mod.f90 */

typedef struct {
    const orc_transport_in* in;
    double* jste;
    double* jlo;        /* the exact rounding errors of the jste additions (TwoSum) */
    uint8_t* touched;   /* [nj / JCHUNK + 1] chunks of jste this thread deposited into */
    uint8_t* touched_e; /* [ne / JCHUNK + 1] chunks of escaped this thread added to */
    double* escaped;
    double* h_est;
    orc_transport_stats st;
    size_t C1;
} tctx_t;

enum { PT_STELLAR = 0, PT_DIFFUSE = 1, PT_DUSTEMI = 2 };

#define AX(a, i) ((double)(a)[(i) - 1])

static inline int active_at(const orc_transport_in* in, int i, int j, int k) {
    return in->active[(size_t)(i - 1) + (size_t)in->nx * ((size_t)(j - 1) + (size_t)in->ny * (size_t)(k - 1))];
}

/* locate (source/interpolation_mod.f90:49-106) over a float array */
static int locate_f(const float* xa, int n, double x) {
    if (x > (double)xa[n - 1]) return n;
    if (x < (double)xa[0]) return 0;
    int jlow = 0, jup = n + 1;
    const int asc = xa[n - 1] > xa[0];
    for (int it = 0; it < 10000; ++it) {
        if (jup - jlow < 1) break;
        int jm = (jup + jlow) / 2;
        if ((double)xa[jm - 1] == x) return jm;
        if (asc == (x > (double)xa[jm - 1])) {
            if (jlow == jm) break;
            jlow = jm;
        } else {
            jup = jm;
        }
    }
    return jlow;
}

/* getNu2 (source/photon_mod.f90:928-972): linear scan of a CDF whose entries
 * are `stride` apart; the scan length is bounded by nbins as in the reference. */
static int get_nu2(const float* cdf, size_t stride, int len, int nbins, rng_t* r) {
    double u = urand(r);
    int nuP = 1;
    int lim = len < nbins ? len : nbins;
    for (int i = 1; i <= lim; ++i) {
        if (u >= (double)cdf[(size_t)(i - 1) * stride]) nuP = i;
        else break;
    }
    if (nuP < nbins) nuP = nuP + 1;
    return nuP;
}

static vec3 random_unit_vector(rng_t* r) {
    double r1 = urand(r);
    double w = 2. * r1 - 1.;
    double t = sqrt(1. - w * w);
    double r2 = urand(r);
    double ang = 3.141592654 * (2. * r2 - 1.);
    vec3 v = {t * cos(ang), t * sin(ang), w};
    return v;
}

/* initPhotonPacket (source/photon_mod.f90:744-896) */
static void init_packet(tctx_t* c, packet_t* p, int nuP, vec3 pos, int lgLine, int lgStellar,
                        int xP, int yP, int zP, rng_t* r) {
    const orc_transport_in* in = c->in;
    p->pos = pos;
    p->nuP = nuP;
    p->lgStellar = lgStellar;
    if (lgLine) { p->nu = 0.; p->lgLine = 1; }
    else { p->nu = (double)in->nu[nuP - 1]; p->lgLine = 0; }
    if (lgStellar && in->plane) {
        /* the ionising plane (:795-856): y = 0, x and z uniform over the axes'
         * span, in the cell whose walls bracket them, moving along +y */
        const float* X = in->x_axis; const float* Z = in->z_axis;
        double rnd = 1. - urand(r);
        p->pos.x = AX(X, 1) + rnd * (AX(X, in->nx) - AX(X, 1));
        xP = locate_f(X, in->nx, p->pos.x);
        if (xP < in->nx && xP > 0 && p->pos.x >= (AX(X, xP) + AX(X, xP + 1)) / 2.) xP = xP + 1;
        p->pos.y = 0.;
        yP = 1;
        rnd = 1. - urand(r);
        p->pos.z = AX(Z, 1) + rnd * (AX(Z, in->nz) - AX(Z, 1));
        zP = locate_f(Z, in->nz, p->pos.z);
        if (zP < in->nz && zP > 0 && p->pos.z >= (AX(Z, zP) + AX(Z, zP + 1)) / 2.) zP = zP + 1;
        if (xP < 1) xP = 1;
        if (zP < 1) zP = 1;
        p->dir.x = 0.; p->dir.y = 1.; p->dir.z = 0.;
    } else {
        for (int irepeat = 0; irepeat < 1000000; ++irepeat) {
            p->dir = random_unit_vector(r);
            if (p->dir.x != 0. && p->dir.y != 0. && p->dir.z != 0.) break;
        }
        if (in->symmetric_xyz && lgStellar) {
            if (p->dir.x < 0.) p->dir.x = -p->dir.x;
            if (p->dir.y < 0.) p->dir.y = -p->dir.y;
            if (p->dir.z < 0.) p->dir.z = -p->dir.z;
        }
    }
    p->xP = xP; p->yP = yP; p->zP = zP;
    if (xP > 0 && yP > 0 && zP > 0) p->origin = active_at(in, xP, yP, zP);
    else p->origin = 0;
}

/* the escape tally (source/photon_mod.f90:2293-2378): plane 0 of
 * escapedPackets, and with viewing angles the plane of the view whose theta
 * and phi bins hold the escape direction; viewPointPtheta == viewPointPphi
 * == 0 (a direction in no view) passes the reference's test as view 0 */
static void escape_tally(tctx_t* c, const packet_t* p) {
    const orc_transport_in* in = c->in;
    const size_t idx = (size_t)p->origin + c->C1 * (size_t)p->nuP;
    if (in->n_angle > 0) {
        const size_t plane = c->C1 * (size_t)(in->nbins + 1);
        const double dTheta = R_PI / 20., dPhi = (2. * R_PI) / (double)in->tot_phi;
        int idirT = (int)(acos(p->dir.z) / dTheta) + 1;
        if (idirT > 20) idirT = 20;
        int idirP = p->dir.x < 1.e-35 ? 0 : (int)(atan(p->dir.y / p->dir.x) / dPhi);
        if (idirP < 0) idirP = in->tot_phi + idirP;
        idirP = idirP + 1;
        if (idirP > in->tot_phi) idirP = in->tot_phi;
        const int k = in->view_p_theta[idirT];
        if ((in->tot_phi > 1 && k == in->view_p_phi[idirP]) || (in->tot_phi == 1 && k > 0)) {
            c->escaped[plane * (size_t)k + idx] += in->delta_e;
            c->touched_e[(plane * (size_t)k + idx) / JCHUNK] = 1;
        }
    }
    c->escaped[idx] += in->delta_e;
    c->touched_e[idx / JCHUNK] = 1;
    c->st.escaped++;
}

static inline void deposit(tctx_t* c, int cell, int nuP, double dl, double dV, double costheta) {
    if (cell <= 0) return;
    size_t idx = (size_t)cell + c->C1 * (size_t)(nuP - 1);
    /* compensated accumulation: jste + jlo holds the sum of the deposits to
     * within the rounding of jlo, so the final jste + jlo is the correctly
     * rounded sum whatever the order of the deposits */
    const double v = dl * c->in->delta_e / dV, old = c->jste[idx], sum = old + v;
    c->jlo[idx] += mcx_fm_two_sum_err(old, v, sum);
    c->jste[idx] = sum;
    c->touched[idx / JCHUNK] = 1;
    if (c->h_est) c->h_est[idx] += (dl * c->in->delta_e) * costheta / dV;
}

double orc_cell_volume(const orc_transport_in* in, int32_t xP, int32_t yP, int32_t zP) {
    const float* X = in->x_axis; const float* Y = in->y_axis; const float* Z = in->z_axis;
    /* half-width first cells with symmetric axes, first and last with a plane
     * source (source/photon_mod.f90:2160-2215) */
    const int lo = in->symmetric_xyz || in->plane, hi = in->plane;
    double dx = 0., dy = 0., dz = 0.;
    if (xP > 1 && xP < in->nx) dx = fabs(AX(X, xP + 1) - AX(X, xP - 1)) / 2.;
    else if (xP == 1) dx = lo ? fabs(AX(X, 2) - AX(X, 1)) / 2. : fabs(AX(X, 2) - AX(X, 1));
    else if (xP == in->nx) dx = hi ? fabs(AX(X, xP) - AX(X, xP - 1)) / 2. : fabs(AX(X, xP) - AX(X, xP - 1));
    if (yP > 1 && yP < in->ny) dy = fabs(AX(Y, yP + 1) - AX(Y, yP - 1)) / 2.;
    else if (yP == 1) dy = lo ? fabs(AX(Y, 2) - AX(Y, 1)) / 2. : fabs(AX(Y, 2) - AX(Y, 1));
    else if (yP == in->ny) dy = hi ? fabs(AX(Y, yP) - AX(Y, yP - 1)) / 2. : fabs(AX(Y, yP) - AX(Y, yP - 1));
    if (zP > 1 && zP < in->nz) dz = fabs(AX(Z, zP + 1) - AX(Z, zP - 1)) / 2.;
    else if (zP == 1) dz = lo ? fabs(AX(Z, 2) - AX(Z, 1)) / 2. : fabs(AX(Z, 2) - AX(Z, 1));
    else if (zP == in->nz) dz = hi ? fabs(AX(Z, zP) - AX(Z, zP - 1)) / 2. : fabs(AX(Z, zP) - AX(Z, zP - 1));
    dx = dx / 1.e15; dy = dy / 1.e15; dz = dz / 1.e15;
    return dx * dy * dz;
}

/* comptonScatter (source/photon_mod.f90:6805-6848) */
static void compton_scatter(tctx_t* c, packet_t* p, rng_t* r) {
    const orc_transport_in* in = c->in;
    int nb = in->nbins;
    int newThetaP = get_nu2(in->kn_cdf + (p->nuP - 1), (size_t)nb, 180, nb, r);
    double newTheta = (double)newThetaP * 3.141592654 / 180.;
    double u = urand(r);
    double w = 2. * u - 1.;
    double t = sqrt(1 - w * w);
    p->dir.x = t * cos(newTheta);
    p->dir.y = t * sin(newTheta);
    p->dir.z = w;
    int th = newThetaP > 180 ? 180 : newThetaP;   /* PcompArray has 180 columns */
    double newNu = p->nu * (double)in->pcomp[(size_t)(th - 1) * nb + (p->nuP - 1)];
    int newNuP = locate_f(in->nu, nb, newNu);
    if (newNuP < 1) newNuP = 1;   /* guard: below nuArray(1) the reference indexes out of bounds */
    p->nu = newNu;
    p->nuP = newNuP;
}

/* pathSegment (source/photon_mod.f90:1758-4085).  Returns 0 when the packet
 * history ends, 1 when the packet was absorbed and must be re-emitted as
 * *retype at p->pos / p->xP..zP, -1 on an insane state. */
static int path_segment(tctx_t* c, packet_t* p, rng_t* r, int* retype) {
    const orc_transport_in* in = c->in;
    const int nx = in->nx, ny = in->ny, nz = in->nz;
    const float* X = in->x_axis; const float* Y = in->y_axis; const float* Z = in->z_axis;
    const size_t C1 = c->C1;
    if (p->xP <= 0 || p->xP > nx || p->yP <= 0 || p->yP > ny || p->zP <= 0 || p->zP > nz) return -1;
    vec3 rv = p->pos, vh = p->dir;
    int xP = p->xP, yP = p->yP, zP = p->zP;
    double dSx = 0., dSy = 0., dSz = 0.;
    double absTau = 0.;
    double passProb = -log(1. - urand(r));
    const int safeLimit = in->plane ? 5000 : 500000;   /* :1873-1878 */
    int packetType = PT_DIFFUSE;
    int i;
    for (i = 1; i <= safeLimit; ++i) {
        /* wall-snap heuristics (source/photon_mod.f90:1882-1919); the test
         * divides by the signed wall coordinate, as in the reference */
        if (xP < nx) { double m = (AX(X, xP) + AX(X, xP + 1)) / 2.; if (vh.x > 0. && fabs(rv.x - m) / m < 2.e-2) xP = xP + 1; }
        if (xP > 1)  { double m = (AX(X, xP) + AX(X, xP - 1)) / 2.; if (vh.x < 0. && fabs(rv.x - m) / m < 2.e-2) xP = xP - 1; }
        if (yP < ny) { double m = (AX(Y, yP) + AX(Y, yP + 1)) / 2.; if (vh.y > 0. && fabs(rv.y - m) / m < 2.e-2) yP = yP + 1; }
        if (yP > 1)  { double m = (AX(Y, yP) + AX(Y, yP - 1)) / 2.; if (vh.y < 0. && fabs(rv.y - m) / m < 2.e-2) yP = yP - 1; }
        if (zP < nz) { double m = (AX(Z, zP) + AX(Z, zP + 1)) / 2.; if (vh.z > 0. && fabs(rv.z - m) / m < 2.e-2) zP = zP + 1; }
        if (zP > 1)  { double m = (AX(Z, zP) + AX(Z, zP - 1)) / 2.; if (vh.z < 0. && fabs(rv.z - m) / m < 2.e-2) zP = zP - 1; }

        /* distances from the walls (source/photon_mod.f90:1933-2084) */
        for (int j = 1; j <= safeLimit; ++j) {
            if (xP > nx || xP < 1 || yP > ny || yP < 1 || zP > nz || zP < 1) return -1;
            if (active_at(in, xP, yP, zP) < 0) return -1;   /* sub-grids are not supported */
            if (in->symmetric_xyz) {
                if (rv.x <= AX(X, 1)) { if (vh.x < 0.) vh.x = -vh.x; rv.x = AX(X, 1); }
                if (rv.y <= AX(Y, 1)) { if (vh.y < 0.) vh.y = -vh.y; rv.y = AX(Y, 1); }
                if (rv.z <= AX(Z, 1)) { if (vh.z < 0.) vh.z = -vh.z; rv.z = AX(Z, 1); }
            }
            if (vh.x > 0.) {
                if (xP < nx) {
                    dSx = ((AX(X, xP + 1) + AX(X, xP)) / 2. - rv.x) / vh.x;
                    if (fabs(dSx) < 1.e-5) { rv.x = (AX(X, xP + 1) + AX(X, xP)) / 2.; xP = xP + 1; }
                } else {
                    dSx = (AX(X, nx) - rv.x) / vh.x;
                    if (fabs(dSx) < 1.e-5) { rv.x = AX(X, nx); if (!in->plane) return 0; }
                }
            } else if (vh.x < 0.) {
                if (xP > 1) {
                    dSx = ((AX(X, xP) + AX(X, xP - 1)) / 2. - rv.x) / vh.x;
                    if (fabs(dSx) < 1.e-5) { rv.x = (AX(X, xP) + AX(X, xP - 1)) / 2.; xP = xP - 1; }
                } else {
                    dSx = (AX(X, 1) - rv.x) / vh.x;
                    if (fabs(dSx) < 1.e-5) rv.x = AX(X, 1);
                }
            } else {
                dSx = AX(X, nx);
            }
            if (vh.y > 0.) {
                if (yP < ny) {
                    dSy = ((AX(Y, yP + 1) + AX(Y, yP)) / 2. - rv.y) / vh.y;
                    if (fabs(dSy) < 1.e-5) { rv.y = (AX(Y, yP + 1) + AX(Y, yP)) / 2.; yP = yP + 1; }
                } else {
                    dSy = (AX(Y, ny) - rv.y) / vh.y;
                    if (fabs(dSy) < 1.e-5) { rv.y = AX(Y, ny); if (!in->plane) return 0; }
                }
            } else if (vh.y < 0.) {
                if (yP > 1) {
                    dSy = ((AX(Y, yP) + AX(Y, yP - 1)) / 2. - rv.y) / vh.y;
                    if (fabs(dSy) < 1.e-5) { rv.y = (AX(Y, yP) + AX(Y, yP - 1)) / 2.; yP = yP - 1; }
                } else {
                    dSy = (AX(Y, 1) - rv.y) / vh.y;
                    if (fabs(dSy) < 1.e-5) rv.y = AX(Y, 1);
                }
            } else {
                dSy = AX(Y, ny);
            }
            if (vh.z > 0.) {
                if (zP < nz) {
                    dSz = ((AX(Z, zP + 1) + AX(Z, zP)) / 2. - rv.z) / vh.z;
                    if (fabs(dSz) < 1.e-5) { rv.z = (AX(Z, zP + 1) + AX(Z, zP)) / 2.; zP = zP + 1; }
                } else {
                    dSz = (AX(Z, nz) - rv.z) / vh.z;
                    if (fabs(dSz) < 1.e-5) { rv.z = AX(Z, nz); if (!in->plane) return 0; }
                }
            } else if (vh.z < 0.) {
                if (zP > 1) {
                    dSz = ((AX(Z, zP) + AX(Z, zP - 1)) / 2. - rv.z) / vh.z;
                    if (fabs(dSz) < 1.e-5) { rv.z = (AX(Z, zP) + AX(Z, zP - 1)) / 2.; zP = zP - 1; }
                } else {
                    dSz = (AX(Z, 1) - rv.z) / vh.z;
                    if (fabs(dSz) < 1.e-5) rv.z = AX(Z, 1);
                }
            } else {
                dSz = AX(Z, nz);
            }
            if (xP > nx || xP < 1 || yP > ny || yP < 1 || zP > nz || zP < 1) return -1;
            if (active_at(in, xP, yP, zP) >= 0) break;
        }

        /* nearest wall (source/photon_mod.f90:2087-2137) */
        if (fabs(dSx) < 1.e-5) dSx = AX(X, nx);
        if (fabs(dSy) < 1.e-5) dSy = AX(Y, ny);
        if (fabs(dSz) < 1.e-5) dSz = AX(Z, nz);
        dSx = fabs(dSx); dSy = fabs(dSy); dSz = fabs(dSz);
        double dS;
        if (dSx <= 0.) dS = fmin(dSy, dSz);
        else if (dSy <= 0.) dS = fmin(dSx, dSz);
        else if (dSz <= 0.) dS = fmin(dSx, dSy);
        else { dS = fmin(dSx, dSy); dS = fmin(dS, dSz); }
        if (dS <= 0.) return -1;

        const int cell = active_at(in, xP, yP, zP);
        const double kap = (double)in->opacity[(size_t)cell + C1 * (size_t)(p->nuP - 1)];
        double tauCell = dS * kap;
        double dV = orc_cell_volume(in, xP, yP, zP);
        double costheta = 1.;
        if (c->h_est) {
            if (!(rv.x == 0. && rv.y == 0. && rv.z == 0.)) {
                costheta = ((rv.x * vh.x) + (rv.y * vh.y) + (rv.z * vh.z)) /
                           (1.e10 * sqrt((rv.x / 1.e10) * (rv.x / 1.e10) + (rv.y / 1.e10) * (rv.y / 1.e10) +
                                         (rv.z / 1.e10) * (rv.z / 1.e10)));
            }
        }

        if ((absTau + tauCell > passProb) && cell > 0) {
            /* the packet interacts in this cell (source/photon_mod.f90:2244-2700) */
            double dlLoc = (passProb - absTau) / kap;
            rv.x = rv.x + dlLoc * vh.x; rv.y = rv.y + dlLoc * vh.y; rv.z = rv.z + dlLoc * vh.z;
            if (in->symmetric_xyz) {
                if (rv.x <= AX(X, 1)) { if (vh.x < 0.) vh.x = -vh.x; rv.x = AX(X, 1); }
                if (rv.y <= AX(Y, 1)) { if (vh.y < 0.) vh.y = -vh.y; rv.y = AX(Y, 1); }
                if (rv.z <= AX(Z, 1)) { if (vh.z < 0.) vh.z = -vh.z; rv.z = AX(Z, 1); }
            }
            deposit(c, cell, p->nuP, dlLoc, dV, costheta);
            c->st.interactions++;
            double rad = sqrt((rv.x / 1.e10) * (rv.x / 1.e10) + (rv.y / 1.e10) * (rv.y / 1.e10) +
                              (rv.z / 1.e10) * (rv.z / 1.e10)) * 1.e10;
            if (rad >= (double)in->r_out && in->r_out > 0.f) {
                escape_tally(c, p);
                return 0;
            }
            if (in->lg_dust) {
                double probSca = (double)in->sca_opac[(size_t)cell + C1 * (size_t)(p->nuP - 1)] / kap;
                double rnd = 1. - urand(r);
                if (rnd > probSca) {
                    c->st.absorptions++;
                    packetType = in->lg_gas ? PT_DIFFUSE : PT_DUSTEMI;
                    break;
                }
                c->st.scatterings++;
                p->xP = xP; p->yP = yP; p->zP = zP;
                init_packet(c, p, p->nuP, rv, 0, 0, xP, yP, zP, r);
                vh = p->dir;
                absTau = 0.;
                passProb = -log(1. - urand(r));
            } else {
                double probSca = in->lg_compton
                                     ? (double)in->kn_sigma_t[p->nuP - 1] * (double)in->ne[cell] / kap
                                     : 0.;
                double rnd = 1. - urand(r);
                if (rnd <= probSca) {
                    c->st.scatterings++;
                    p->xP = xP; p->yP = yP; p->zP = zP;
                    compton_scatter(c, p, r);
                    p->origin = cell;
                    vh = p->dir;
                    absTau = 0.;
                    passProb = -log(1. - urand(r));
                } else {
                    c->st.absorptions++;
                    packetType = PT_DIFFUSE;
                    break;
                }
            }
        } else {
            /* the packet crosses the cell (source/photon_mod.f90:2703-2881) */
            deposit(c, cell, p->nuP, dS, dV, costheta);
            c->st.crossings++;
            absTau = absTau + tauCell;
            rv.x = rv.x + dS * vh.x; rv.y = rv.y + dS * vh.y; rv.z = rv.z + dS * vh.z;
            if (dS == dSx && vh.x > 0.) xP = xP + 1;
            else if (dS == dSx && vh.x < 0.) xP = xP - 1;
            else if (dS == dSy && vh.y > 0.) yP = yP + 1;
            else if (dS == dSy && vh.y < 0.) yP = yP - 1;
            else if (dS == dSz && vh.z > 0.) zP = zP + 1;
            else if (dS == dSz && vh.z < 0.) zP = zP - 1;

            if (in->plane) {
                /* plane-parallel slab (source/photon_mod.f90:3249-3611): out
                 * through the y planes only, reflected at x and z (the lower z
                 * plane puts z at yAxis(1), as the reference does) */
                int ret = 0;
                if (rv.y < AX(Y, 1) || yP < 1) { yP = 1; ret = 1; }
                if (rv.y > AX(Y, ny) || yP > ny) { yP = ny; ret = 1; }
                if (rv.x <= AX(X, 1) || xP < 1) { xP = 1; rv.x = AX(X, 1); vh.x = -vh.x; }
                if (rv.x >= AX(X, nx) || xP > nx) { xP = nx; rv.x = AX(X, nx); vh.x = -vh.x; }
                if (rv.z <= AX(Z, 1) || zP < 1) { zP = 1; rv.z = AX(Y, 1); vh.z = -vh.z; }
                if (rv.z >= AX(Z, nz) || zP > nz) { zP = nz; rv.z = AX(Z, nz); vh.z = -vh.z; }
                if (ret) { escape_tally(c, p); return 0; }
            } else {
            if (!in->symmetric_xyz) {
                /* full-grid escape (source/photon_mod.f90:2884-3244) */
                int ret = 0;
                if (rv.y < AX(Y, 1) || yP < 1) { yP = 1; ret = 1; }
                if (rv.y > AX(Y, ny) || yP > ny) { yP = ny; ret = 1; }
                if (rv.x <= AX(X, 1) || xP < 1) { xP = 1; ret = 1; }
                if (rv.x >= AX(X, nx) || xP > nx) { xP = nx; ret = 1; }
                if (rv.z <= AX(Z, 1) || zP < 1) { zP = 1; ret = 1; }
                if (rv.z >= AX(Z, nz) || zP > nz) { zP = nz; ret = 1; }
                if (ret) { escape_tally(c, p); return 0; }
            }
            /* grid boundary and mirror planes (source/photon_mod.f90:3607-3890) */
            if ((!in->symmetric_xyz && (rv.x <= AX(X, 1) || rv.y <= AX(Y, 1) || rv.z <= AX(Z, 1))) ||
                rv.x >= AX(X, nx) || rv.y >= AX(Y, ny) || rv.z >= AX(Z, nz) ||
                xP > nx || yP > ny || zP > nz) {
                escape_tally(c, p);
                return 0;
            }
            if (in->symmetric_xyz) {
                if (rv.x <= AX(X, 1) || xP < 1) { if (vh.x < 0.) vh.x = -vh.x; xP = 1; rv.x = AX(X, 1); }
                if (rv.y <= AX(Y, 1) || yP < 1) { if (vh.y < 0.) vh.y = -vh.y; yP = 1; rv.y = AX(Y, 1); }
                if (rv.z <= AX(Z, 1) || zP < 1) { if (vh.z < 0.) vh.z = -vh.z; zP = 1; rv.z = AX(Z, 1); }
            }
            }
        }
        /* source/photon_mod.f90:3951-4036 */
        if (!in->plane && (xP > nx || yP > ny || zP > nz)) { escape_tally(c, p); return 0; }
    }
    if (i > safeLimit) { c->st.trapped++; return 0; }
    p->xP = xP; p->yP = yP; p->zP = zP;
    p->pos = rv;
    *retype = packetType;
    return 1;
}

/* energyPacketRun (source/photon_mod.f90:418-741) + newPhotonPacket
 * (source/photon_mod.f90:976-1756).  Returns 1 to re-run, 0 done, -1 error. */
static int packet_run(tctx_t* c, int type, packet_t* p, vec3 pos, int xP, int yP, int zP, rng_t* r, int* retype) {
    const orc_transport_in* in = c->in;
    if (type == PT_STELLAR) {
        int nuP = get_nu2(in->src_cdf, 1, in->nbins, in->nbins, r);
        c->st.emissions++;
        init_packet(c, p, nuP, pos, 0, 1, in->star_idx[0], in->star_idx[1], in->star_idx[2], r);
        if (p->nu >= 1.) c->st.q_phot += in->delta_e / (2.1799153e-11 * p->nu);
    } else if (type == PT_DIFFUSE) {
        int cell = active_at(in, xP, yP, zP);
        if (cell <= 0) return -1;
        double rnd = 1. - urand(r);
        if (rnd <= (double)in->total_lines[cell]) {
            init_packet(c, p, 0, pos, 1, 0, xP, yP, zP, r);
        } else {
            int nuP = get_nu2(in->rec_pdf + cell, c->C1, in->nbins, in->nbins, r);
            c->st.emissions++;
            init_packet(c, p, nuP, pos, 0, 0, xP, yP, zP, r);
        }
    } else {
        int cell = active_at(in, xP, yP, zP);
        if (cell <= 0) return -1;
        int nuP = get_nu2(in->dust_pdf + cell, c->C1, in->nbins, in->nbins, r);
        c->st.emissions++;
        init_packet(c, p, nuP, pos, 0, 0, xP, yP, zP, r);
    }
    if (!in->lg_dust && p->nu < (double)in->ion_edge1 && !p->lgLine) {
        escape_tally(c, p);
        return 0;
    }
    if (!p->lgLine) return path_segment(c, p, r, retype);
    c->st.line_escapes++;
    return 0;
}

typedef struct {
    tctx_t c;
    uint64_t seed, first, count;
    int err;
} job_t;

static void run_packets(job_t* jb) {
    tctx_t* c = &jb->c;
    const orc_transport_in* in = c->in;
    const int recursionLimit = 100000;
    vec3 star = {in->star_pos[0], in->star_pos[1], in->star_pos[2]};
    for (uint64_t k = 0; k < jb->count; ++k) {
        rng_t r;
        rng_init(&r, jb->seed, jb->first + k);
        packet_t p;
        memset(&p, 0, sizeof(p));
        int type = PT_STELLAR;
        vec3 pos = star;
        int xP = in->star_idx[0], yP = in->star_idx[1], zP = in->star_idx[2];
        int it;
        for (it = 1; it <= recursionLimit; ++it) {
            int retype = PT_DIFFUSE;
            int rc = packet_run(c, type, &p, pos, xP, yP, zP, &r, &retype);
            if (rc < 0) { jb->err = 1; c->st.error = 1; return; }
            if (rc == 0) break;
            type = retype; pos = p.pos; xP = p.xP; yP = p.yP; zP = p.zP;
        }
        if (it >= recursionLimit) c->st.trapped++;
    }
}

static void* thread_main(void* arg) {
    run_packets((job_t*)arg);
    return NULL;
}

/* Per-thread accumulators kept between calls, cleared chunk by chunk after
 * each merge: their pages are faulted in once instead of on every call (the
 * reference's MPI ranks likewise keep their full-grid arrays for the run).
 * A mutex serialises orc_transport calls, which share the pool. */
#define MAX_POOL 256
typedef struct {
    double *jste, *jlo, *esc, *h;
    uint8_t *tj, *te;
    size_t nj, ne;
} acc_t;
static acc_t g_pool[MAX_POOL];
static pthread_mutex_t g_pool_lock = PTHREAD_MUTEX_INITIALIZER;

static void pool_free(acc_t* a) {
    free(a->jste); free(a->jlo); free(a->esc); free(a->h); free(a->tj); free(a->te);
    memset(a, 0, sizeof(*a));
}

static int pool_ready(acc_t* a, size_t nj, size_t ne, int want_h) {
    if (a->nj != nj || a->ne != ne) {
        pool_free(a);
        a->jste = (double*)calloc(nj, sizeof(double));
        a->jlo = (double*)calloc(nj, sizeof(double));
        a->esc = (double*)calloc(ne, sizeof(double));
        a->tj = (uint8_t*)calloc(nj / JCHUNK + 1, 1);
        a->te = (uint8_t*)calloc(ne / JCHUNK + 1, 1);
        a->nj = nj; a->ne = ne;
        if (!a->jste || !a->jlo || !a->esc || !a->tj || !a->te) { pool_free(a); return 0; }
    }
    if (want_h && !a->h) {
        a->h = (double*)calloc(nj, sizeof(double));
        if (!a->h) return 0;
    }
    return 1;
}

/* zero the chunks of a marked in `mark` (and the marks) */
static void clear_chunks(double* v, uint8_t* mark, size_t n) {
    for (size_t ch = 0; ch < n / JCHUNK + 1; ++ch) {
        if (!mark[ch]) continue;
        const size_t k1 = (ch + 1) * JCHUNK < n ? (ch + 1) * JCHUNK : n;
        if (v) memset(v + ch * JCHUNK, 0, (k1 - ch * JCHUNK) * sizeof(double));
    }
}

int orc_transport(const orc_transport_in* in, uint64_t seed, uint64_t counter_base, int64_t n,
                  int32_t nthreads, orc_transport_out* out, orc_transport_stats* stats) {
    if (!in || !out || !out->jste || !out->escaped || n < 0) return 2;
    if (in->star_idx[0] < 1 || in->star_idx[1] < 1 || in->star_idx[2] < 1) return 2;
    const size_t C1 = (size_t)in->n_cells + 1;
    const size_t nj = C1 * (size_t)in->nbins, ne = C1 * (size_t)(in->nbins + 1) * (size_t)(in->n_angle + 1);
    if (nthreads < 1) nthreads = 1;
    if (nthreads > MAX_POOL) nthreads = MAX_POOL;
    if ((int64_t)nthreads > n) nthreads = n > 0 ? (int32_t)n : 1;
    const int want_h = in->rad_press && out->h_est;
    job_t* jobs = (job_t*)calloc((size_t)nthreads, sizeof(job_t));
    pthread_t* th = (pthread_t*)calloc((size_t)nthreads, sizeof(pthread_t));
    if (!jobs || !th) { free(jobs); free(th); return 3; }
    pthread_mutex_lock(&g_pool_lock);
    int rc = 0;
    uint64_t per = (uint64_t)n / (uint64_t)nthreads, rest = (uint64_t)n % (uint64_t)nthreads, first = counter_base;
    for (int t = 0; t < nthreads; ++t) {
        job_t* jb = &jobs[t];
        jb->c.in = in;
        jb->c.C1 = C1;
        jb->seed = seed;
        jb->first = first;
        jb->count = per + ((uint64_t)t < rest ? 1 : 0);
        first += jb->count;
        acc_t* a = &g_pool[t];
        if (!pool_ready(a, nj, ne, want_h && t > 0)) { rc = 3; continue; }
        jb->c.jlo = a->jlo; jb->c.touched = a->tj; jb->c.touched_e = a->te;
        if (t == 0) {
            jb->c.jste = out->jste; jb->c.escaped = out->escaped;
            jb->c.h_est = want_h ? out->h_est : NULL;
        } else {
            jb->c.jste = a->jste; jb->c.escaped = a->esc;
            jb->c.h_est = want_h ? a->h : NULL;
        }
    }
    if (rc == 0) {
        for (int t = 1; t < nthreads; ++t) pthread_create(&th[t], NULL, thread_main, &jobs[t]);
        run_packets(&jobs[0]);
        for (int t = 1; t < nthreads; ++t) pthread_join(th[t], NULL);
    }
    memset(stats, 0, sizeof(*stats));
    /* J: the compensated sum of every thread's (jste, jlo) pair, rounded once,
     * over the chunks some thread deposited into */
    if (rc == 0) {
        const size_t nch = nj / JCHUNK + 1;
        for (size_t ch = 0; ch < nch; ++ch) {
            int any = 0;
            for (int t = 0; t < nthreads && !any; ++t) any = jobs[t].c.touched[ch];
            if (!any) continue;
            const size_t k1 = (ch + 1) * JCHUNK < nj ? (ch + 1) * JCHUNK : nj;
            for (size_t k = ch * JCHUNK; k < k1; ++k) {
                double s = out->jste[k], e = jobs[0].c.jlo[k];
                for (int t = 1; t < nthreads; ++t) {
                    if (!jobs[t].c.touched[ch]) continue;
                    const double h = jobs[t].c.jste[k], s2 = s + h;
                    e += mcx_fm_two_sum_err(s, h, s2) + jobs[t].c.jlo[k];
                    s = s2;
                }
                out->jste[k] = s + e;
            }
        }
    }
    for (int t = 0; t < nthreads; ++t) {
        job_t* jb = &jobs[t];
        if (t > 0 && rc == 0) {
            for (size_t ch = 0; ch < ne / JCHUNK + 1; ++ch) {
                if (!jb->c.touched_e[ch]) continue;
                const size_t k1 = (ch + 1) * JCHUNK < ne ? (ch + 1) * JCHUNK : ne;
                for (size_t k = ch * JCHUNK; k < k1; ++k) out->escaped[k] += jb->c.escaped[k];
            }
            if (jb->c.h_est) for (size_t k = 0; k < nj; ++k) out->h_est[k] += jb->c.h_est[k];
        }
        if (jb->c.touched) {
            /* leave the pooled accumulators zero for the next call */
            clear_chunks(jb->c.jlo, jb->c.touched, nj);
            if (t > 0) {
                clear_chunks(jb->c.jste, jb->c.touched, nj);
                clear_chunks(jb->c.escaped, jb->c.touched_e, ne);
                if (jb->c.h_est) memset(jb->c.h_est, 0, nj * sizeof(double));
            }
            memset(jb->c.touched, 0, nj / JCHUNK + 1);
            memset(jb->c.touched_e, 0, ne / JCHUNK + 1);
        }
        stats->crossings += jb->c.st.crossings;
        stats->interactions += jb->c.st.interactions;
        stats->absorptions += jb->c.st.absorptions;
        stats->scatterings += jb->c.st.scatterings;
        stats->escaped += jb->c.st.escaped;
        stats->line_escapes += jb->c.st.line_escapes;
        stats->trapped += jb->c.st.trapped;
        stats->emissions += jb->c.st.emissions;
        stats->q_phot += jb->c.st.q_phot;
        if (jb->err) { stats->error = 1; rc = 1; }
    }
    pthread_mutex_unlock(&g_pool_lock);
    free(jobs); free(th);
    return rc;
}
