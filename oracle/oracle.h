/*
 * oracle.h - CPU FP64 restatement of the MOCASSIN iteration hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the GB300
 * kernels of libmcx.so and the timed CPU baseline of bench.py; nothing in the
 * product links, loads or calls it.  It restates the Fortran reference
 * (rwesson/mocassin_xray, "MOCASSIN 2007 Version 3") routine by routine; each
 * function cites the reference file:line it follows.
 *
 * Parity status: the reference has no tests, golden vectors or fixtures, and
 * it cannot be compiled here or on the GPU hosts (no Fortran compiler), so
 * this restatement is pinned only by analytic known-answer tests and by the
 * published Philox4x32-10 known-answer vectors: parity unpinned against the
 * reference's own outputs.
 *
 * Arrays use the reference's Fortran layouts:
 *   [nbins][nCells+1] for A(0:nCells,1:nbins), [nz][ny][nx] for active(nx,ny,nz).
 */
#ifndef MCX_ORACLE_H
#define MCX_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ RNG */
/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11).  Packet p draws its
 * k-th uniform from block k/4, word k%4 of philox(key=(seed_lo,seed_hi),
 * ctr=(p_lo, p_hi, k/4, 0)). */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* The portable FP64 routines of mcx_fmath.h over arrays: fn 0 exp(x), 1 log(x),
 * 2 log10(x), 3 pow(x, y), 4 sin(x), 5 cos(x). */
void orc_fm_eval(int32_t fn, const double* x, const double* y, int64_t n, double* out);

/* ------------------------------------------------------------ transport */
typedef struct orc_transport_in {
    int32_t nx, ny, nz, n_cells, nbins;
    int32_t symmetric_xyz, lg_dust, lg_gas, lg_compton, rad_press;
    const float* x_axis;        /* [nx] */
    const float* y_axis;        /* [ny] */
    const float* z_axis;        /* [nz] */
    const int32_t* active;      /* [nz][ny][nx] */
    const float* nu;            /* [nbins] nuArray */
    const float* src_cdf;       /* [nbins] inSpectrumProbDen(iStar,:) */
    const float* kn_sigma_t;    /* [nbins] */
    const float* kn_cdf;        /* [180][nbins] */
    const float* pcomp;         /* [180][nbins] */
    const float* opacity;       /* [nbins][C+1] */
    const float* sca_opac;      /* [nbins][C+1] or NULL (dust) */
    const float* rec_pdf;       /* [nbins][C+1] */
    const float* dust_pdf;      /* [nbins][C+1] or NULL (dust only) */
    const float* total_lines;   /* [C+1] */
    const float* ne;            /* [C+1] */
    float ion_edge1;            /* ionEdge(1) */
    float r_out;                /* R_out */
    float star_pos[3];
    int32_t star_idx[3];        /* 1-based */
    double delta_e;             /* Lstar/nPhotons */
    int32_t n_angle;            /* nAngleBins (0: escapes into plane 0 only)           */
    int32_t tot_phi;            /* totAngleBinsPhi                                     */
    int32_t view_p_theta[21];   /* viewPointPtheta(0:20)                               */
    int32_t view_p_phi[21];     /* viewPointPphi(0:tot_phi)                            */
    int32_t plane;              /* lgPlaneIonization                                   */
} orc_transport_in;

typedef struct orc_transport_out {
    double* jste;               /* [nbins][C+1], accumulated (not cleared) */
    double* escaped;            /* [n_angle+1][nbins+1][C+1], accumulated */
    double* h_est;              /* [nbins][C+1] or NULL */
} orc_transport_out;

typedef struct orc_transport_stats {
    int64_t crossings, interactions, absorptions, scatterings;
    int64_t escaped, line_escapes, trapped, emissions;
    double q_phot;
    int32_t error;              /* 0 ok; 1 insane state (the reference `stop`s) */
    int32_t pad;
} orc_transport_stats;

/* Transport packets [counter_base, counter_base + n) from the stellar source.
 * Returns 0 or a nonzero error code.  `nthreads` > 1 splits the packets over
 * OpenMP-free POSIX threads with private estimator copies summed at the end. */
int orc_transport(const orc_transport_in* in, uint64_t seed, uint64_t counter_base, int64_t n,
                  int32_t nthreads, orc_transport_out* out, orc_transport_stats* stats);

/* Volume [e45 cm^3] of cell (xP,yP,zP), 1-based (getVolume, source/grid_mod.f90:2887-2986). */
double orc_cell_volume(const orc_transport_in* in, int32_t xP, int32_t yP, int32_t zP);


/* -------------------------------------------------------------- opacity */
/* Packed set-up pointers (1-based like the reference), see mcx_setup_get(MCX_ARR_POINTERS). */
enum {
    ORC_P_HLEVXSECP1 = 0, ORC_P_HLEVNUP1, ORC_P_HEISINGXSECP1, ORC_P_HEILEVNUP1,
    ORC_P_HEIIXSECP1, ORC_P_HEIILEVNUP1, ORC_P_BREMSXSECP, ORC_P_LYMANP, ORC_P_COUNT_ = 32
};

typedef struct orc_opacity_in {
    int32_t n_cells, nbins, nstages, n_elem_used, lg_compton, n_xsec;
    const float* nu;            /* [nbins] */
    const float* xsec;          /* [n_xsec] xSecArray */
    const float* kn_sigma_t;    /* [nbins] */
    const int32_t* ptr;         /* [32] packed pointers (ORC_P_*) */
    const float* elem_abun;     /* [30] */
    const int32_t* elem_xref;   /* [30] 1-based, 0 = element off */
    const int32_t* n_shells;    /* [30][30]  nShells(elem,ion) at [elem-1][ion-1] */
    const int32_t* element_p;   /* [30][30][7][3] elementP(elem,ion,shell,k) */
    const float* hden;          /* [C+1] */
    const float* te;            /* [C+1] */
    const float* ne;            /* [C+1] */
    const float* ionden;        /* [nstages][n_elem_used][C+1] */
    const float* gaunt_te;      /* [C+1] Te at which gauntFF was tabulated for the cell */
    const uint8_t* compute;     /* [C+1] 1 = recompute the cell, 0 = keep (skip rule) */
} orc_opacity_in;

/* ionizationDriver/BoltGaunt/getGauntFF/eDenSum/addOpacity
 * (source/ionization_mod.f90:26-477) for every cell with compute[c] = 1;
 * writes opacity[nu][c] (Fortran layout); other cells are left untouched. */
int orc_opacity(const orc_opacity_in* in, float* opacity);

/* Hummer (1988) free-free Gaunt factor fit of getGauntFF
 * (source/ionization_mod.f90:196-334) at log10(Z) = z, log10(Te) and n frequencies. */
void orc_gaunt_ff(double z, double log10te, const float* nu, int32_t n, double* g);

/* The reference tabulates gauntFF only when Te moved by more than 10 % since
 * the last tabulation (BoltGaunt, source/ionization_mod.f90:136-178), a cache
 * shared by all cells in processing order (i, j, k nested, k fastest).  This
 * replays that cache: for each active cell in processing order with
 * compute[c] = 1 it updates *te_old (the saved TeOld2; start at -1) and writes
 * the tabulation temperature to gaunt_te[c]. */
void orc_gaunt_cache(int32_t nx, int32_t ny, int32_t nz, const int32_t* active, const float* te,
                     const uint8_t* compute, float* te_old, float* gaunt_te);

/* ------------------------------------------------------------- emission */
typedef struct orc_emission_in {
    int32_t n_cells, nbins, nstages, n_elem_used, n_xsec, n_fb_heavy;
    int32_t n_tk, nlim[3];
    int32_t j2ts_p;             /* locate(nuArray, 1.45673) */
    int32_t heii_lyman_p[4];
    const float* nu;            /* [nbins] */
    const float* widflx;        /* [nbins] */
    const float* xsec;          /* [n_xsec] */
    const int32_t* ptr;         /* [32] packed pointers (ORC_P_*) */
    const float* elem_abun;     /* [30] */
    const int32_t* elem_xref;   /* [30] */
    const float* tk;            /* [n_tk] */
    const int32_t* gamma_edge_p;/* [3][32] */
    const float* log_gamma;     /* [3][n_tk][32] */
    const int32_t* fb_heavy;    /* [n_fb_heavy][7] elem, ion, IPnuP, highNuP, xSecP, g0, g1 */
    const float* gaunt_ff;      /* [nbins] gauntFF as last tabulated by the opacity phase */
    const float* gaunt_ff_heii; /* [nbins] gauntFFHeII */
    const float* hei2phot;      /* [2][41] y, Ay */
    const float* heii_lyman;    /* [4] ratios */
    const int32_t* hydro_file_map; /* [9][12] */
    const float* hydro_dens;    /* [nFiles][13] */
    const float* hydro_lines;   /* [nFiles][13][14][8] */
    const float* hydro_temps;   /* [12] */
    const float* hb_coeff;      /* [2][9][4] */
    const float* rb_edge;       /* [2][3][26] */
    const float* r2a_edge;      /* [3][18] */
    const float* hei_rec;       /* [34][3][4] */
    const float* te;            /* [C+1] */
    const float* ne;            /* [C+1] */
    const float* ionden;        /* [nstages][n_elem_used][C+1] */
    const float* for_lines;     /* [C+1] forbidden-line total per cell, or NULL */
    const uint8_t* compute;     /* [C+1] */
} orc_emission_in;

/* emissionDriver for gas without dust: writes recPDF[nu][c] and totalLines[c]
 * for the cells with compute[c] = 1.  Returns 0, or 4 when the frequency mesh
 * is too coarse between two gamma edges (the reference stops there). */
int orc_emission(const orc_emission_in* in, float* rec_pdf, float* total_lines);

/* -------------------------------------------------------------- balance */
/* Packed multi-level atom header fields (mcx_setup_get(MCX_SARR_ATOM_HDR)). */
enum {
    ORC_AT_ELEM = 0, ORC_AT_ION, ORC_AT_NLEV, ORC_AT_NTEMP, ORC_AT_IUP2P, ORC_AT_RECTYPE, ORC_AT_NREC,
    ORC_AT_OFF_LOGT, ORC_AT_OFF_QOM, ORC_AT_OFF_Y2, ORC_AT_OFF_A, ORC_AT_OFF_G, ORC_AT_OFF_E,
    ORC_AT_OFF_REC, ORC_AT_OFF_ATP, ORC_AT_HDR = 16
};

typedef struct orc_balance_in {
    int32_t n_cells, nbins, nstages, n_elem_used, n_xsec;
    int32_t lg_badnell, lg_compton, n_diel, n_aldro, n_atoms;
    float xhi_limit;
    const float* nu;            /* [nbins] */
    const float* xsec;          /* [n_xsec] xSecArray */
    const int32_t* ptr;         /* [32] packed pointers */
    const float* xsec_recoil;   /* [nbins] */
    const float* elem_abun;     /* [30] */
    const int32_t* elem_xref;   /* [30] */
    const int32_t* n_shells;    /* [30][30] */
    const int32_t* element_p;   /* [30][30][7][3] */
    const float* cf;            /* [30][30][5] cion.dat CF(i,elem,nElec) */
    const float* cion_therm;    /* [30][30] */
    const int32_t* nauger;      /* [30][30][10] */
    const float* auger;         /* [30][30][10][10] */
    const float* rr_badnell;    /* [6][30][31] */
    const float* dr_c;          /* [30][31][9] */
    const float* dr_e;          /* [30][31][9] */
    const float* rrec;          /* [30][30][2] */
    const float* rnew;          /* [30][30][4] */
    const float* diel;          /* [n_diel][8] */
    const float* aldro;         /* [n_aldro][6] */
    const int32_t* outer;       /* [30][30][3] outShell, g0, g1 of (z, nElec) */
    const int32_t* atom_index;  /* [30][31] */
    const int32_t* atom_hdr;    /* [n_atoms][16] */
    const double* atom_data;
    const double* jste;         /* [nbins][C+1] */
    const float* hden;          /* [C+1] */
} orc_balance_in;

typedef struct orc_balance_state {
    float* te;                  /* [C+1] in/out */
    float* ne;                  /* [C+1] in/out */
    float* ionden;              /* [nstages][n_elem_used][C+1] in/out */
    int32_t* converged;         /* [C+1] out: lgConverged */
    int32_t* black;             /* [C+1] out: lgBlack (no photon hit) */
    int32_t* n_iter_t;          /* [C+1] out: T-iterations used (0 = not updated) */
} orc_balance_state;

typedef struct orc_balance_stats {
    double no_hit, no_ion_bal, no_te_bal;
    int64_t converged;
} orc_balance_stats;

/* updateCell (source/update_mod.f90:15-482) for every active cell: the
 * T-iteration (iterateT) around calcAlpha, photoionisation, collisional
 * ionisation, Compton, ionBalance and thermBalance (forLines/equilibrium).
 * Gas only (no grains).  Returns 0. */
int orc_balance(const orc_balance_in* in, orc_balance_state* st, int32_t nthreads, orc_balance_stats* stats);

/* The balance of every cell with its Te held (the evaluations of the
 * implicit-function adjoint of the converged balance): calcAlpha,
 * photoionisation, collisional ionisation, Compton and ionBalance at the
 * state's Te, repeated from where ionBalance stopped until its X(H0), X(He0),
 * X(He+) changes fall within x_tol (at most 64 times), then thermBalance.
 * Writes Ne and the ion fractions, n_iter_t = the repetitions, converged = 1
 * where ionBalance met x_tol, black = 1 where no photon reached the cell, and
 * resid[cell] = heating - cooling (resid[C+1]).  Returns 0. */
int orc_balance_fixed_te(const orc_balance_in* in, orc_balance_state* st, int32_t nthreads, double x_tol,
                         double* resid);

/* updateCell of one cell recording each T-iteration in trace[20][5] (Te,
 * heating, cooling, Ne, X(H0)); returns the number of T-iterations. */
int orc_balance_trace(const orc_balance_in* in, orc_balance_state* st, int32_t cell, double* trace);

/* equilibrium (source/emission_mod.f90:2505-3007) for atom slot `atom`:
 * level populations n[nLev] and line emissivities em[i][j] (lower i, upper j,
 * [nLev][nLev], zero where a(j,i) = 0).  rec selects the recombination term. */
int orc_equilibrium(const orc_balance_in* in, int32_t atom, double te, double ne, double ion_den_up,
                    int32_t rec, double* n, double* em);

/* The emission phase's forbidden-line total normFor of each cell with
 * compute[c] = 1 (all cells if compute is NULL; forLines with rec = .true.,
 * source/emission_mod.f90:1481-1524 and :1780-1795), in its units of 1e-25
 * erg/s per unit gas density. */
int orc_for_lines_emission(const orc_balance_in* in, const float* te, const float* ne, const float* ionden,
                           const uint8_t* compute, double* for_lines);

/* ---------------------------------------------------------------- lines */
typedef struct orc_lines_out {
    double hbeta;               /* sum of hydroLines(1,4,2)*Hden*dV over the terms > 1e-35 */
    double* hydro;              /* [30][14][8] hydroVol at [iz-1][iup-2][ilow-1]            */
    double* hei;                /* [34] HeIVol                                              */
    double* forb;               /* [n_atoms][30][30] forbVol of atom slot at [i-1][j-1],
                                   i the lower and j the upper level                        */
    double* ion_num;            /* [30][nstages] sum ionDen*Te*Ne*Hden*dV                   */
    double* ion_den;            /* [30][nstages] sum ionDen*Ne*Hden*dV                      */
    int64_t n_cells;            /* cells summed                                             */
} orc_lines_out;

/* outputGas's volume sums (source/output_mod.f90:280-680) over the cells with
 * black[c] < 1, from the grid state em->te, em->ne, em->ionden and bal->hden,
 * with the FP64 cell volumes vol[C+1].  Raw sums, not yet divided by Hbeta. */
int orc_line_sums(const orc_emission_in* em, const orc_balance_in* bal, const double* vol, const int32_t* black,
                  orc_lines_out* out);

/* ----------------------------------------------------------------- dust */
typedef struct orc_dust_in {
    int32_t n_cells, nbins, n_species, n_sizes;
    float xhi_limit;
    const float* nu;            /* [nbins] */
    const float* widflx;        /* [nbins] */
    const float* cabs;          /* [nSpecies][nSizes][nbins] cm^2 */
    const float* csca;
    const float* abun;          /* [nSpecies] grainAbun */
    const float* tsub;          /* [nSpecies] TdustSublime */
    const float* weight;        /* [nSizes] grainWeight */
    const float* em_int;        /* [nSpecies][nSizes][3000] dustEmIntegral */
} orc_dust_in;

typedef struct orc_dust_stats {
    int64_t no_hit, updated, converged;
} orc_dust_stats;

/* Tdust is [nSpecies+1][nSizes+1][C+1].  Grain scattering and absorption of
 * every cell below sublimation; opacity += their sum. */
int orc_dust_opacity(const orc_dust_in* in, const float* ndust, const float* tdust, float* opacity, float* sca_opac);
/* setDustPDF for every cell: pdf[nu][c] */
int orc_dust_pdf(const orc_dust_in* in, const float* tdust, float* pdf);
/* getDustT for every cell hit by a photon, with lgBlack and lgConverged */
int orc_dust_t(const orc_dust_in* in, const double* jste, float* tdust, int32_t* converged, int32_t* black,
               orc_dust_stats* stats);

#ifdef __cplusplus
}
#endif
#endif
