/*
 * mcx.h - C ABI of the GB300 transport + per-cell balance library (libmcx.so).
 *
 * This is the drop-in boundary for the MOCASSIN iteration hot path.  Every
 * entry point below replaces one loop (or one set-up routine) of the Fortran
 * reference; the reference routine it replaces is cited beside it as
 * path:line inside the MOCASSIN source tree (source/...).  A Fortran driver
 * binds these through ISO_C_BINDING; Python binds them through ctypes.
 *
 * Conventions
 *  - Plain C types only: pointers, sizes, int32/int64/float/double.
 *  - Arrays crossing the boundary use the reference's Fortran layout:
 *      per-cell x per-frequency arrays  A(0:nCells, 1:nbins)  -> [nbins][nCells+1]
 *        (cell index fastest, exactly the column-major memory of the Fortran array)
 *      ionDen(0:nCells, 1:nElementsUsed, 1:nstages)           -> [nstages][nElemUsed][nCells+1]
 *      active(1:nx,1:ny,1:nz)                                 -> [nz][ny][nx] (x fastest)
 *  - Every function returns an int status (MCX_OK == 0).  The library never
 *    exits the process (the reference calls `stop`); the message of the last
 *    failure is returned by mcx_last_error / mcx_setup_last_error.
 *  - A context (mcx_ctx) owns device memory, one CUDA stream and the
 *    device-resident copies of the tables and grid state.  One context per
 *    host thread / rank; there is no global mutable state.
 */
#ifndef MCX_H
#define MCX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
#define MCX_OK              0
#define MCX_ERR_INPUT       1   /* invalid argument / input deck           */
#define MCX_ERR_IO          2   /* data or input file missing / unreadable */
#define MCX_ERR_CUDA        3   /* CUDA runtime error                       */
#define MCX_ERR_NOMEM       4   /* allocation failure                       */
#define MCX_ERR_STATE       5   /* call out of order (e.g. no grid loaded)  */
#define MCX_ERR_STEP_LIMIT  6   /* a packet hit the reference's step limits */
#define MCX_ERR_TIMEOUT     7   /* a bounded device wait gave up            */
#define MCX_ERR_INTERNAL    8

/* ------------------------------------------------------------- array ids */
/* Ids used by mcx_setup_get / mcx_setup_set / mcx_get / mcx_put. */
enum mcx_array_id {
    MCX_ARR_NU = 1,          /* float [nbins]        nuArray [Ryd]                */
    MCX_ARR_WIDFLX,          /* float [nbins]        widFlx  [Ryd]                */
    MCX_ARR_XSEC,            /* float [nxsec]        xSecArray                    */
    MCX_ARR_SRC_CDF,         /* float [nbins]        inSpectrumProbDen(1,:)       */
    MCX_ARR_KN_SIGMA_T,      /* float [nbins]        KNsigmaT                     */
    MCX_ARR_KN_CDF,          /* float [180][nbins]   KNsigmaArray(nbins,180)      */
    MCX_ARR_PCOMP,           /* float [180][nbins]   PcompArray(nbins,180)        */
    MCX_ARR_XAXIS,           /* float [nx]                                        */
    MCX_ARR_YAXIS,           /* float [ny]                                        */
    MCX_ARR_ZAXIS,           /* float [nz]                                        */
    MCX_ARR_ACTIVE,          /* int32 [nz][ny][nx]   active(nx,ny,nz)             */
    MCX_ARR_HDEN,            /* float [nCells+1]                                  */
    MCX_ARR_TE,              /* float [nCells+1]                                  */
    MCX_ARR_NE,              /* float [nCells+1]                                  */
    MCX_ARR_TEOLD,           /* float [nCells+1]                                  */
    MCX_ARR_NEOLD,           /* float [nCells+1]                                  */
    MCX_ARR_IONDEN,          /* float [nstages][nElemUsed][nCells+1]              */
    MCX_ARR_OPACITY,         /* float [nbins][nCells+1]  opacity(0:C,1:B)         */
    MCX_ARR_RECPDF,          /* float [nbins][nCells+1]  recPDF(0:C,1:B)          */
    MCX_ARR_TOTAL_LINES,     /* float [nCells+1]         totalLines(0:C)          */
    MCX_ARR_JSTE,            /* double[nbins][nCells+1]  Jste(0:C,1:B)            */
    MCX_ARR_ESCAPED,         /* double[nAngleBins+1][nbins+1][nCells+1] escapedPackets(0:C,0:B,0:nAngleBins) */
    MCX_ARR_VOLUME,          /* float [nCells+1]      getVolume per active cell    */
    MCX_ARR_ELEM_ABUN,       /* float [30]            elemAbun(1,1:30)             */
    MCX_ARR_GAUNT_TE,        /* float [nCells+1]      Te at which the ff Gaunt factor
                                                      was last tabulated, per cell  */
    MCX_ARR_SCAOPAC,         /* float [nbins][nCells+1] dust scaOpac(0:C,1:B)      */
    MCX_ARR_DUSTPDF,         /* float [nbins][nCells+1] dustPDF(0:C,1:B)           */
    MCX_ARR_NDUST,           /* float [nCells+1]                                   */
    MCX_ARR_LG_CONVERGED,    /* int32 [nCells+1]                                   */
    MCX_ARR_H_EST,           /* double[nbins][nCells+1] H(0:C,1:B) (radPress only) */
    MCX_ARR_LG_BLACK,        /* int32 [nCells+1] lgBlack: no photon hit in the last balance */
    MCX_ARR_N_ITER_T,        /* int32 [nCells+1] T-iterations of the last balance (0 = not updated) */
    MCX_ARR_FOR_LINES,       /* float [nCells+1] forbidden-line total of the last emission phase */
    MCX_ARR_TDUST,           /* float [nSpecies+1][nSizes+1][nCells+1] Tdust(0:nSp,0:nSz,0:C) */
    MCX_ARR_BAL_RESID,       /* double[nCells+1] heating - cooling at the held Te of the last balance
                                run with fix_te = 1 (thermBalance's units, erg/cm^3/s per Hden^2 scale) */
    MCX_ARR_COUNT_
};

/* Set-up-only tables (mcx_setup_get only). */
#define MCX_SARR_POINTERS      1001  /* int32[32]: HlevXSecP(1), HlevNuP(1), HeISingXSecP(1), HeIlevNuP(1),
                                        HeIIXSecP(1), HeIIlevNuP(1), bremsXSecP, lymanP, KshellLimitP,
                                        secIonP, cRecoilHP, cRecoilHeP, xrayP, BjumpP, 0...          */
#define MCX_SARR_ELEMENT_P     1002  /* int32[30][30][7][3] elementP(elem,ion,shell,k) at [elem-1][ion-1][shell-1][k-1] */
#define MCX_SARR_N_SHELLS      1003  /* int32[30][30] nShells(elem,ion)                                */
#define MCX_SARR_ELEM_XREF     1004  /* int32[30] elementXref                                           */
#define MCX_SARR_ION_EDGE      1005  /* float[nEdges] ionEdge (sorted)                                  */
#define MCX_SARR_COMXSEC_H     1006  /* float[nbins] comXSecH                                           */
#define MCX_SARR_COMXSEC_C     1007  /* float[nbins] comXSecC                                           */
#define MCX_SARR_XSEC_RECOIL   1008  /* float[nbins] xSecRecoil                                         */
/* emission tables (read once from data/) */
#define MCX_SARR_EM_DIMS       1009  /* int32[16]: nTk, nlimHI, nlimHeI, nlimHeII, nFbHeavy, nHydroFiles,
                                        j2TsP, HeIILymanP(1:4), 0...                                   */
#define MCX_SARR_EM_TK         1010  /* float[nTk]                                                      */
#define MCX_SARR_EM_EDGE_P     1011  /* int32[3][32]                                                    */
#define MCX_SARR_EM_LOG_GAMMA  1012  /* float[3][nTk][32]                                               */
#define MCX_SARR_EM_FB_HEAVY   1013  /* int32[nFbHeavy][7]                                              */
#define MCX_SARR_EM_HYDRO_MAP  1014  /* int32[9][12]                                                    */
#define MCX_SARR_EM_HYDRO_DENS 1015  /* float[nHydroFiles][13]                                          */
#define MCX_SARR_EM_HYDRO_LINES 1016 /* float[nHydroFiles][13][14][8]                                   */
#define MCX_SARR_EM_HYDRO_TEMPS 1017 /* float[12]                                                       */
#define MCX_SARR_EM_HB_COEFF   1018  /* float[2][9][4]                                                  */
#define MCX_SARR_EM_RB_EDGE    1019  /* float[2][3][26]                                                 */
#define MCX_SARR_EM_R2A_EDGE   1020  /* float[3][18]                                                    */
#define MCX_SARR_EM_HEI_REC    1021  /* float[34][3][4]                                                 */
#define MCX_SARR_EM_HEI_2PHOT  1022  /* float[2][41]                                                    */
#define MCX_SARR_EM_HEII_LYMAN 1023  /* float[2][4] ratios, frequencies                                 */
/* balance tables (source/hydro_mod.f90:13-53, :334-418, :676-764; source/update_mod.f90:3094-3305) */
#define MCX_SARR_CION_CF       1024  /* float[30][30][5] CF(i,elem,nElec) at [elem-1][nElec-1][i-1]     */
#define MCX_SARR_CION_THERM    1025  /* float[30][30] cionTherm(elem,ion)                               */
#define MCX_SARR_NAUGER        1026  /* int32[30][30][10] nauger(elem,ion,shell)                        */
#define MCX_SARR_AUGER         1027  /* float[30][30][10][10] auger(elem,ion,shell,nelec)               */
#define MCX_SARR_RR_BADNELL    1028  /* float[6][30][31] RRbA,B,T0,T1,C,T2 at [k][z-1][n]              */
#define MCX_SARR_DR_BADNELL_C  1029  /* float[30][31][9] DRbC(idr,z,n) at [z-1][n][idr-1]              */
#define MCX_SARR_DR_BADNELL_E  1030  /* float[30][31][9] DRbE                                           */
#define MCX_SARR_RADREC_RREC   1031  /* float[30][30][2] rrec(i,z,n) at [z-1][n-1][i-1]                 */
#define MCX_SARR_RADREC_RNEW   1032  /* float[30][30][4] rnew(i,z,n)                                    */
#define MCX_SARR_DIELEC        1033  /* float[nRows][8] dielectronic.dat: elem,n,a,b,c,d,f,g            */
#define MCX_SARR_ALDRO         1034  /* float[nRows][6] aldrovandi.dat: elem,n,a,b,t0,t1                */
#define MCX_SARR_OUTER_SHELL   1035  /* int32[30][30][3] getOuterShell(z,nElec): outShell,g0,g1        */
#define MCX_SARR_ATOM_INDEX    1036  /* int32[30][31] multi-level atom slot of (elem,ion), -1 = no data */
#define MCX_SARR_ATOM_HDR      1037  /* int32[nAtoms][16] packed atom headers (fields:
                                        elem, ion, nLev, nTemp, iup2p, recType, nRec, offLogT, offQom,
                                        offY2, offA, offG, offE, offRec, offAtp, 0)                     */
#define MCX_SARR_DUST_DIMS     1039  /* int32[4] nSpecies, nSizes, nTemps, 0                           */
#define MCX_SARR_DUST_CABS     1040  /* float[nSpecies][nSizes][nbins] pi a^2 Qabs [cm^2]               */
#define MCX_SARR_DUST_CSCA     1041  /* float[nSpecies][nSizes][nbins] pi a^2 Qsca [cm^2]               */
#define MCX_SARR_DUST_CTABS    1042  /* float[nbins] abundance- and size-weighted absorption             */
#define MCX_SARR_DUST_CTSCA    1043  /* float[nbins] abundance- and size-weighted scattering             */
#define MCX_SARR_DUST_ABUN     1044  /* float[nSpecies] grainAbun                                       */
#define MCX_SARR_DUST_TSUB     1045  /* float[nSpecies] TdustSublime                                    */
#define MCX_SARR_DUST_RADIUS   1046  /* float[nSizes] grainRadius [um]                                  */
#define MCX_SARR_DUST_WEIGHT   1047  /* float[nSizes] normalised grainWeight                            */
#define MCX_SARR_DUST_EMINT    1048  /* float[nSpecies][nSizes][nTemps] dustEmIntegral                  */
#define MCX_SARR_STARS         1049  /* float[nStars][8] per source: Lstar [e36 erg/s], TStellar [K],
                                        starPosition x, y, z [cm], its cell's x, y, z indices
                                        (1-based, -1 outside the grid)                            */
#define MCX_SARR_SRC_CDFS      1050  /* float[nStars][nbins] inSpectrumProbDen(1:nStars,:)          */
#define MCX_SARR_ATOM_DATA     1038  /* double[n] packed atom data: log10 T[nTemp]; qom and its natural-
                                        spline second derivatives [pair (l<u) row-major][nTemp];
                                        a(j,i) at [j-1][i-1]; g; e [1/cm]; recombination fits; atp    */

/* -------------------------------------------------------------- set-up */
/* Host-side model built from an input deck.  Replaces readInput
 * (source/set_input_mod.f90:12-708), initCartesianGrid
 * (source/grid_mod.f90:21-608), initXSecArray (source/ph_mod.f90:204-517),
 * setContinuum/setProbDen (source/continuum_mod.f90:33-504), fillGrid /
 * setMotherGrid (source/grid_mod.f90:651-1832) and setStarPosition
 * (source/grid_mod.f90:3690-3790). */
typedef struct mcx_setup mcx_setup;

/* Frequency-mesh modes. */
#define MCX_MESH_REFERENCE  0   /* exactly the reference's choice (fill() mesh for nuMax > 25) */
#define MCX_MESH_LOG_EDGES  1   /* the reference's nuMax <= 25 construction (log mesh with the
                                   H series edges and ionisation thresholds inserted) forced at
                                   the deck's nbins for any nuMax                               */

typedef struct mcx_setup_opts {
    int32_t mesh_mode;          /* MCX_MESH_*                                        */
    int32_t reserved[7];
} mcx_setup_opts;

typedef struct mcx_setup_info {
    int32_t nx, ny, nz;
    int32_t n_cells;            /* active cells (ids 1..n_cells; 0 = inactive)        */
    int32_t nbins;
    int32_t n_xsec;             /* length of xSecArray                                */
    int32_t n_elem_used;        /* nElementsUsed                                      */
    int32_t nstages;
    int32_t symmetric_xyz, lg_gas, lg_dust, lg_compton;
    int32_t star_idx[3];        /* starIndeces(1,1:3), 1-based, -1 outside the grid    */
    int32_t lyman_p;            /* lymanP (1-based)                                   */
    int64_t n_photons;          /* nPhotons(1)                                        */
    int32_t max_iterate_mc;
    int32_t n_species, n_sizes;
    float   star_pos[3];        /* starPosition(1) [cm]                               */
    float   r_out, r_in;        /* R_out, R_in [cm]                                   */
    float   l_star;             /* Lstar(1) [e36 erg/s]                               */
    float   l_phot;             /* LPhot [e36 phot/s]                                 */
    float   ion_edge1;          /* ionEdge(1) [Ryd]                                   */
    float   te_start;
    float   min_convergence;    /* minConvergence [%]                                 */
    float   xhi_limit;          /* XHILimit                                           */
    int32_t n_angle_bins;       /* nAngleBins: viewing angles of the 'inclination' keyword
                                   (0..2); MCX_ARR_ESCAPED then holds 1 + n_angle_bins planes */
    float   view_theta[2];      /* viewPointTheta(1:2) [rad]                           */
    float   view_phi[2];        /* viewPointPhi(1:2) [rad]; < 0: no phi dependence     */
    int32_t plane_ionization;   /* 1: lgPlaneIonization (the source is the plane y = 0,
                                   l_star = transferred flux x the x-z extent)         */
    int32_t n_stars;            /* nStars: ionising sources (multiPhotoSources; else 1); star_*,
                                   l_star and MCX_ARR_SRC_CDF are source 1's, n_photons is
                                   nPhotons(1) = nPhotons / nStars                      */
    int32_t reserved[1];
} mcx_setup_info;

int  mcx_setup_from_input(const char* input_file, const char* data_dir,
                          const mcx_setup_opts* opts, mcx_setup** out);
void mcx_setup_free(mcx_setup* s);
int  mcx_setup_info_get(const mcx_setup* s, mcx_setup_info* info);
/* Copy an array out of / into the set-up (sizes in bytes must match exactly). */
int  mcx_setup_get(const mcx_setup* s, int32_t array_id, void* dst, size_t nbytes);
/* Number of elements of a set-up array (for MCX_SARR_ION_EDGE and the others). */
int  mcx_setup_len(const mcx_setup* s, int32_t array_id, int64_t* count);
int  mcx_setup_set(mcx_setup* s, int32_t array_id, const void* src, size_t nbytes);
/* Message of the last set-up failure of this thread. */
const char* mcx_setup_last_error(void);

/* ---------------------------------------------------------- device context */
typedef struct mcx_ctx mcx_ctx;

int  mcx_ctx_create(int32_t device, mcx_ctx** out);
void mcx_ctx_destroy(mcx_ctx* ctx);
int  mcx_last_error(const mcx_ctx* ctx, char* buf, size_t len);
int  mcx_sync(mcx_ctx* ctx);

/* Upload tables and the grid state of a set-up to the device (once per model). */
int  mcx_load(mcx_ctx* ctx, const mcx_setup* s);

/* Download / upload a device-resident array in the Fortran layout given above.
 * `host` must hold exactly `nbytes`; this is how a Fortran driver exchanges
 * state with the library between phases. */
int  mcx_get(mcx_ctx* ctx, int32_t array_id, void* host, size_t nbytes);
int  mcx_put(mcx_ctx* ctx, int32_t array_id, const void* host, size_t nbytes);

/* Raw device pointer of a context array (for zero-copy callers). */
int  mcx_device_ptr(mcx_ctx* ctx, int32_t array_id, void** dptr);

/* Device-side snapshots of everything an iteration hands to the next: the
 * gas state (Te, Ne, ionDen, TeOld, NeOld, lgConverged), the phase outputs
 * the skip rule keeps for unchanged cells (opacity, recPDF, totalLines,
 * forLines and the Gaunt-cache temperatures; the grain arrays of a dust
 * grid), in numbered slots held in device memory, stream-ordered with the
 * phases.  mcx_state_save / mcx_state_restore use slot 0.  No counterpart in
 * the reference, which keeps one grid state; used to rerun an iteration from
 * the state it started from (timing, tests, restarts in memory).  Each slot
 * holds about 3 nbins x (nCells+1) x 4 bytes. */
#define MCX_STATE_SLOTS 64
int  mcx_state_save(mcx_ctx* ctx);
int  mcx_state_restore(mcx_ctx* ctx);
int  mcx_state_save_slot(mcx_ctx* ctx, int32_t slot);
int  mcx_state_restore_slot(mcx_ctx* ctx, int32_t slot);

/* ------------------------------------------------------- phase: opacity */
/* Per-cell opacity kappa(nu): free-free + sum of bound-free x-sections times
 * ion densities + Klein-Nishina electron scattering.  Replaces the
 * ionizationDriver loop of iterateMC (source/iteration_mod.f90:112-192) and
 * ionizationDriver/BoltGaunt/getGauntFF/eDenSum/addOpacity
 * (source/ionization_mod.f90:26-477), including the skip rule for cells whose
 * Te and Ne changed by less than 0.5 % (source/iteration_mod.f90:131-149). */
#define MCX_PHASE_EXACT  0     /* the reference's arithmetic (FP64 multi-level atoms)      */
#define MCX_PHASE_MIXED  1     /* emission: forbidden lines from the cooling surfaces (or the
                                  mixed-precision solver), and the cumulative distribution summed
                                  over frequency chunks with offsets (differs from the sequential
                                  FP32 sum by rounding) */

typedef struct mcx_phase_opts {
    int32_t n_iterate_mc;       /* nIterateMC (1-based); the skip rule applies when > 1 */
    int32_t precision;          /* MCX_PHASE_*                                           */
    int32_t reserved[6];
} mcx_phase_opts;

typedef struct mcx_phase_stats {
    int64_t cells_computed;
    int64_t cells_skipped;
    float   kernel_ms;          /* CUDA-event time of the phase's kernels            */
    float   reserved_f[3];
    int64_t reserved[4];
} mcx_phase_stats;

int  mcx_opacity(mcx_ctx* ctx, const mcx_phase_opts* opts, mcx_phase_stats* stats);

/* ------------------------------------------------------- phase: emission */
/* Per-cell diffuse emission: the re-emission CDF recPDF(cell,:) (H, He and
 * heavy-ion free-bound + free-free continua, two-photon continua, the He I
 * 2^3S and He II Lyman lines) and the fraction of non-ionising line photons
 * totalLines(cell) (hydrogenic and He I recombination lines, plus forbidden
 * lines when heavy ions have atomic data).  Replaces the emissionDriver loop of
 * iterateMC (source/iteration_mod.f90:279-623) and emissionDriver / fb_ff /
 * twoPhoton / RecLinesEmission / setDiffusePDF (source/emission_mod.f90:36-252,
 * :336-1151, :1528-1919), with the same skip rule as the opacity phase.  The
 * free-free Gaunt factors are those last tabulated by mcx_opacity, as in the
 * reference, so mcx_opacity must have run at least once. */
int  mcx_emission(mcx_ctx* ctx, const mcx_phase_opts* opts, mcx_phase_stats* stats);

/* ------------------------------------------------------- phase: balance */
/* Per-cell thermal and ionisation balance from the normalised J (Jste after
 * mcx_normalize_j): the T-iteration of updateCell / iterateT
 * (source/update_mod.f90:15-482) with calcAlpha (:2298-2413, Badnell or the
 * radRecFit/dielectronic fits), photoionisation / getPhotoRates
 * (:3584-3832, :3971-4040), collisionalIonisation (:3552-3582), compton
 * (:3834-3897), ionBalance (:1575-1992) and thermBalance (:887-1215) with
 * forLines / equilibrium (:1221-1262; source/emission_mod.f90:2505-3106).
 * Replaces the updateCell loop of iterateMC (source/iteration_mod.f90:1136-1156):
 * TeOld/NeOld take Te/Ne first, then Te, Ne, ionDen, lgConverged and lgBlack
 * are updated on the device.  Gas only; grains are outside this phase. */
#define MCX_BAL_FP64  0         /* FP64 throughout (the plain path)                    */
#define MCX_BAL_MIXED 1         /* FP32 rates, collision strengths, exponentials,
                                   ionisation ladder (on the logarithms of its
                                   products) and level populations (state
                                   reduction), each ion's line cooling read from
                                   its cooling surface (see atom_solves); FP64 Te
                                   bracketing                                         */

typedef struct mcx_balance_opts {
    int32_t precision;          /* MCX_BAL_*                                            */
    int32_t max_rounds;         /* T-iteration cap; 0 = 20 (maxIterateT)                */
    int32_t atom_solves;        /* MCX_BAL_MIXED: 1 = solve every ion's levels in every cell and
                                   T-iteration instead of reading the cooling surfaces (ln of each
                                   ion's line cooling per ion tabulated over ln Te, ln Ne once per
                                   context, 4-point Lagrange in both; ~1e-6 relative)     */
    int32_t converge;           /* 1 = converge every cell tightly instead of iterateT's stopping
                                   rules: heating - cooling to 1e-9 of their mean and ionBalance's
                                   X(H0), X(He0), X(He+) changes to 1e-9 (MCX_BAL_MIXED: 1e-6 and
                                   1e-5), a residual with the ladder not yet converged evaluated
                                   again at the same Te, Illinois-weighted regula
                                   falsi without the 100 K step, unbracketed steps x(1 + 1e-4 2^n)
                                   (at most x1.2) at T-iteration n, up to 64 T-iterations
                                   (max_rounds up to 64).  The solution is then a smooth function
                                   of the inputs away from the balance's discontinuities (used for
                                   derivatives)                                           */
    int32_t fix_te;             /* 1 (with converge = 1) = hold every cell's Te: calcAlpha,
                                   photoionisation, Compton and ionBalance at that Te, repeated
                                   until ionBalance's X(H0), X(He0), X(He+) changes fall below
                                   1e-14 (MCX_BAL_MIXED: 1e-5), then thermBalance;
                                   heating - cooling there is left in MCX_ARR_BAL_RESID.  The
                                   evaluations of mcx_adjoint                             */
    int32_t reserved[3];
} mcx_balance_opts;

typedef struct mcx_balance_stats {
    int64_t cells_updated;      /* cells with at least one photon hit                  */
    int64_t no_hit;             /* grid%noHit                                          */
    int64_t no_ion_bal;         /* grid%noIonBal: ionBalance reached 15 X-iterations   */
    int64_t no_te_bal;          /* grid%noTeBal: iterateT reached 20 T-iterations      */
    int64_t converged;          /* cells with lgConverged = 1                          */
    int32_t max_iter_t;         /* most T-iterations any cell needed                    */
    float   kernel_ms;          /* CUDA-event time of the phase                         */
    int64_t reserved[4];
} mcx_balance_stats;

int  mcx_balance(mcx_ctx* ctx, const mcx_balance_opts* opts, mcx_balance_stats* stats);

/* ------------------------------------------------------ phase: transport */
/* Monte Carlo transport of n packets from source iStar, accumulating the
 * path-length estimator of the mean intensity J_nu (Jste) and the escape
 * tally.  Replaces energyPacketDriver / energyPacketRun / newPhotonPacket /
 * initPhotonPacket / getNu2 / pathSegment / comptonScatter
 * (source/photon_mod.f90:28-416, 418-741, 744-896, 928-972, 976-1756,
 * 1758-4085, 6805-6848) for a single mother grid without plane-parallel
 * illumination.  Packet k (0-based, global id counter_base + k) draws its
 * random numbers from its own Philox4x32-10 stream keyed by `seed`, so the
 * result does not depend on scheduling and ranks can shard packets by
 * counter range. */
#define MCX_PREC_FP32_GEOM  0   /* FP32 packet geometry / tau, FP64 J accumulation */
#define MCX_PREC_FP64       1   /* FP64 everywhere (the plain path)                */

typedef struct mcx_transport_opts {
    int32_t istar;              /* 1-based source index                                */
    int32_t precision;          /* MCX_PREC_*                                          */
    int64_t n_packets;          /* packets of this call                                */
    uint64_t seed;              /* Philox key                                          */
    uint64_t counter_base;      /* global id of the first packet of this call          */
    int64_t n_photons_norm;     /* nPhotons(iStar) used for deltaE = Lstar/nPhotons;
                                   0 means n_packets                                   */
    int32_t zero_estimators;    /* 1: clear Jste/escaped before transporting           */
    int32_t block_size;         /* 0 = library default                                 */
    int32_t grid_mult;          /* persistent blocks per SM; 0 = library default        */
    int32_t chunk;              /* packets handed out per queue grab; 0 = default       */
    int32_t emit_batch;         /* lanes of a warp that wait for an emission before the
                                   warp runs the emission code; 0 = library default (12) */
    int32_t handoff_emissions;  /* re-emissions after which a history is continued by the
                                   trapped-packet kernel; 0 = library default (256),
                                   -1 = never (every history stays in the main kernel) */
    int32_t reserved[2];
} mcx_transport_opts;

typedef struct mcx_transport_stats {
    int64_t crossings;          /* cell-wall crossings (estimator updates of a full segment) */
    int64_t interactions;       /* in-cell interactions (estimator update of a partial segment) */
    int64_t absorptions;        /* absorbed and re-emitted as diffuse / dustEmi packets      */
    int64_t scatterings;        /* Compton or dust scatterings                               */
    int64_t escaped;            /* packets that left the grid / R_out                         */
    int64_t line_escapes;       /* diffuse packets emitted as (untransported) line photons    */
    int64_t trapped;            /* histories that hit recursionLimit / safeLimit              */
    int64_t emissions;          /* frequency draws from a CDF (source + re-emission)          */
    double  q_phot;             /* Qphot (e36 photons/s above 1 Ryd emitted by the source)    */
    float   kernel_ms;          /* CUDA-event time of the transport kernels                   */
    float   reserved_f[3];
    int64_t handed_off;         /* histories continued by the trapped-packet kernel          */
    int64_t reserved[3];
} mcx_transport_stats;

int  mcx_transport(mcx_ctx* ctx, const mcx_transport_opts* opts, mcx_transport_stats* stats);

/* J normalisation after all sources: Jste *= 1e-9 and /8 in octant mode;
 * escaped /8 in octant mode (source/iteration_mod.f90:1002-1031). */
int  mcx_normalize_j(mcx_ctx* ctx);

/* ------------------------------------------------------ one MC iteration */
/* One pass of iterateMC's loop body (source/iteration_mod.f90:98-1260) for the
 * stellar source: mcx_opacity, mcx_emission, mcx_transport (Jste cleared
 * first), mcx_normalize_j and mcx_balance, in that order on the context's
 * stream.  The balance's 64 launches are captured as a CUDA graph on first
 * use and replayed.  The convergence test of :1270-1480 is left to the caller
 * (stats.balance.converged against nCells and minConvergence). */
typedef struct mcx_iterate_opts {
    int32_t n_iterate_mc;           /* nIterateMC (1-based): the skip rule applies when > 1 */
    int32_t transport_precision;    /* MCX_PREC_*                                          */
    int32_t balance_precision;      /* MCX_BAL_*                                           */
    int32_t emission_precision;     /* MCX_PHASE_*                                         */
    int64_t n_packets;              /* nPhotons: every source's packets (each of nStars
                                       sources sends n_packets / nStars)                   */
    uint64_t seed;                  /* Philox key                                          */
    uint64_t counter_base;          /* global id of the iteration's first packet           */
    int32_t transport_block_size;   /* the transport launch (mcx_transport_opts' fields of the */
    int32_t transport_grid_mult;    /* same names); 0 = library defaults                   */
    int32_t transport_emit_batch;
    int32_t reserved[5];
} mcx_iterate_opts;

typedef struct mcx_iterate_stats {
    mcx_phase_stats opacity;
    mcx_phase_stats emission;
    mcx_transport_stats transport;
    mcx_balance_stats balance;
    float   total_ms;               /* CUDA-event time of the whole iteration              */
    float   reserved_f[3];
    int64_t reserved[4];
} mcx_iterate_stats;

int  mcx_iterate(mcx_ctx* ctx, const mcx_iterate_opts* opts, mcx_iterate_stats* stats);

/* ------------------------------------------- frozen-field line sensitivities */
/* No counterpart in the reference.  With the radiation field of the context
 * (the normalised Jste of the last transport) held fixed, the balance of a
 * cell depends on that cell's density and on the abundances alone.  So one
 * balance with every Hden scaled by (1 + h) gives each cell's response to its
 * own density, and one balance per listed element its response to that
 * element's abundance.  For each requested forbidden line (element, ion and
 * the lower and upper level of fLineEm(i,j) in equilibrium) the call returns
 * its outputGas volume sum L (1e-25 erg/s x 1e45 cm^3, before the division by
 * Hbeta), dL/dHden of every cell and dL/d(elemAbun) of every listed element,
 * as forward differences from the unperturbed balance of the current state
 * (central differences: call twice with h and -h).  The balances are converged
 * tightly unless reference_stopping is set, so the differences approximate
 * the derivatives of the converged per-cell balance (the implicit-function
 * derivative of heating = cooling and the ionisation ladder at fixed J).
 * In that mode a perturbed balance continues from the converged unperturbed
 * one (whose first steps are small), so that it follows the same branch of
 * heating = cooling; a cell whose Te still moves by more than max(5|h|, 1e-4) has
 * crossed a discontinuity of the balance (the reference's charge-exchange fits
 * switch off below 6000 K and above 5e4 K) and has no derivative there; so has
 * a cell whose bracket closed on such a jump instead of a root, and a cell
 * that did not converge in 64 T-iterations has none either: they are left out
 * of the differences and counted in branch_cells_*.
 * The balance's response to J (the transport) is outside these derivatives.
 * The context is left as after the unperturbed balance.  Gas, one nebula. */
typedef struct mcx_line_ref {
    int32_t elem, ion, lower, upper;
} mcx_line_ref;

typedef struct mcx_sens_opts {
    int32_t n_lines;
    int32_t n_abun;
    const mcx_line_ref* lines;  /* [n_lines]                                           */
    const int32_t* abun_z;      /* [n_abun] atomic numbers whose abundance is varied    */
    double h;                   /* relative step (may be negative); 0 = 1e-3            */
    int32_t precision;          /* MCX_BAL_* of the balances                            */
    int32_t reference_stopping; /* 0: every balance converged tightly (mcx_balance_opts.converge),
                                   so that L is a smooth function of Hden and the abundances and
                                   the differences are derivatives of the converged balance;
                                   1: iterateT's own stopping rules (2 % residual), whose
                                   discrete stops make the differences noisy            */
    int32_t reserved[4];
} mcx_sens_opts;

typedef struct mcx_sens_out {
    double* L;                  /* [n_lines]                                            */
    double* dL_dhden;           /* [n_lines][nCells+1] or NULL                          */
    double* dL_dabun;           /* [n_lines][n_abun] or NULL                            */
    float   kernel_ms;          /* out: CUDA-event time of the balances and line sums   */
    float   reserved_f[3];
    int64_t branch_cells_hden;  /* out: cells left out of dL_dhden (tight mode)         */
    int64_t branch_cells_abun;  /* out: cell-balances left out of dL_dabun, summed over the elements */
    int64_t reserved[2];
} mcx_sens_out;

int  mcx_line_sensitivities(mcx_ctx* ctx, const mcx_sens_opts* opts, mcx_sens_out* out);

/* ----------------------------------- adjoint of the converged per-cell balance */
/* No counterpart in the reference.  The same derivatives as
 * mcx_line_sensitivities (frozen J), from the implicit-function theorem on the
 * converged balance instead of perturbed balances: at fixed J a cell's
 * converged Te is the root of R(Te; p) = heating - cooling of its ionisation
 * ladder converged at Te, so with L(Te; p) the cell's line luminosities
 *     dL/dp = dL/dp|Te - dL/dTe|p (dR/dp|Te) / (dR/dTe|p),
 * p = the cell's Hden or an element's abundance.  The call converges the
 * balance tightly from the current state (mcx_balance_opts.converge), then
 * evaluates R and L with every Te held (fix_te) at Te(1 +- h), Hden(1 +- h)
 * and each listed abundance (1 +- h), all cells at once, and an adjoint kernel
 * combines the central differences per cell.  No T-iteration is run for a
 * perturbed p, so a cell whose perturbed balance would take another branch of
 * the iteration still gets the derivative of its root.  A cell without a root
 * (its bracket closed on a jump of heating - cooling, or dR/dTe not finite and
 * non-zero) has its Te held: dTe/dp = 0, counted in pinned_cells.  A cell whose
 * balance did not converge in 64 T-iterations has no converged state: its
 * derivatives are 0, counted in no_solution_cells, and it is left out of the
 * evaluations (as are the held cells from those at Te(1 +- h)).  opts as for
 * mcx_line_sensitivities
 * (reference_stopping must be 0).  The context is left as after the converged
 * unperturbed balance.  Gas, one nebula. */
typedef struct mcx_adjoint_out {
    double* L;                  /* [n_lines] line sums of the converged balance         */
    double* dL_dhden;           /* [n_lines][nCells+1] or NULL                          */
    double* dL_dabun;           /* [n_lines][n_abun] or NULL                            */
    double* dte_dhden;          /* [nCells+1] or NULL: dTe/dHden of each cell's root    */
    float   kernel_ms;          /* out: CUDA-event time of the balances, lines and adjoint kernels */
    float   reserved_f[3];
    int64_t pinned_cells;       /* out: cells with their Te held (no root)              */
    int64_t no_solution_cells;  /* out: cells without a converged balance (derivatives 0) */
    int64_t reserved[2];
} mcx_adjoint_out;

int  mcx_adjoint(mcx_ctx* ctx, const mcx_sens_opts* opts, mcx_adjoint_out* out);

/* ------------------------------------------------------- batches of nebulae */
/* No counterpart in the reference, which runs one nebula per job.  A batch
 * holds n nebulae (gas only) that share the frequency mesh, the elements and
 * abundances, nstages and the data tables (set-ups read from one data
 * directory); each keeps its own grid, density, source and octant flag.  Their
 * cells are numbered batch-wide: nebula b owns cells cell_offset[b]+1 ..
 * cell_offset[b+1], and every per-cell array of the context (MCX_ARR_TE,
 * MCX_ARR_OPACITY, MCX_ARR_JSTE, ...) is the concatenation of the nebulae's
 * behind one dump cell 0.  mcx_opacity, mcx_emission, mcx_normalize_j,
 * mcx_balance, mcx_state_save / restore and mcx_get / put act on every nebula
 * at once, each nebula with its own Gaunt cache and octant factor; the
 * transport runs all nebulae's packets in one launch (mcx_transport_batched),
 * packet k of nebula b drawing from Philox stream (seed[b], counter_base[b] +
 * k) with deltaE = L*(b) / nPhotons(b), so that each nebula's histories are
 * those of a run of that nebula alone. */
int  mcx_load_batched(mcx_ctx* ctx, const mcx_setup* const* setups, int32_t n_nebulae);

/* Number of nebulae (0 for a context loaded by mcx_load) and, if cell_offset
 * is not NULL, the n+1 cell offsets. */
int  mcx_batch_info(mcx_ctx* ctx, int32_t* n_nebulae, int32_t* cell_offset);

typedef struct mcx_batch_packets {
    const int64_t*  n_packets;      /* [n] packets of each nebula (0 leaves it dark)            */
    const uint64_t* seed;           /* [n] Philox key of each nebula                            */
    const uint64_t* counter_base;   /* [n] global id of each nebula's first packet              */
    const int64_t*  n_photons_norm; /* [n] nPhotons of deltaE = Lstar / nPhotons, or NULL (n_packets) */
} mcx_batch_packets;

/* mcx_transport for every nebula of a batch; of opts only precision,
 * zero_estimators, block_size and grid_mult are read (istar must be 1). */
int  mcx_transport_batched(mcx_ctx* ctx, const mcx_transport_opts* opts, const mcx_batch_packets* packets,
                           mcx_transport_stats* stats);

/* mcx_iterate for a batch (opts.n_packets, seed and counter_base unused). */
int  mcx_iterate_batched(mcx_ctx* ctx, const mcx_iterate_opts* opts, const mcx_batch_packets* packets,
                         mcx_iterate_stats* stats);

/* ---------------------------------------------- analytical line luminosities */
/* The analytical part of outputGas (source/output_mod.f90:13-805) from the
 * current grid state: over the active cells with lgBlack < 1, the volume
 * emissivities sum(eps * Hden * dV) of Hbeta, of the hydrogenic recombination
 * lines of every element on with nstages > Z, of the 34 HeI recombination
 * lines and of every forbidden line of the ions with multi-level data
 * (equilibrium with the recombination term, 1e-25 erg/s units), and the
 * Ne * Hden * dV weighted ionic temperatures TeVol and fractions ionDenVol
 * (Harrington et al. 1982).  When HbetaVol > 0 the line sums are divided by
 * it ("relative" = 1); then HbetaVol is scaled to 1e36 erg/s (x 1e-16) and by
 * 8 in symmetricXYZ mode.  All sums are FP64 and reduced in a fixed order, so
 * repeated calls give the same bits.  Gas grids only.
 *
 * Output arrays are caller-owned, may be NULL, and use the reference's
 * column-major layouts of the iAb = 0 (total) slice:
 *   hydro_vol  double[8][14][30]        hydroVol(iz,iup,ilow)   at (iz-1) + 30*(iup-2) + 420*(ilow-1)
 *   hei_vol    double[34]               HeIVol(l)
 *   forb_vol   double[30][30][S][30]    forbVol(elem,ion,i,j)   at (elem-1) + 30*(ion-1) + 30*S*(i-1) + 900*S*(j-1)
 *              (S = nstages; i the lower and j the upper level, as fLineEm(i,j) of equilibrium)
 *   wav        double, forb_vol layout  wavelength 1e8/(E_j - E_i) [A] of each line with a(j,i) /= 0
 *   te_vol     double[S][30]            TeVol(elem,ion)         at (elem-1) + 30*(ion-1)
 *   ion_vol    double[S][30]            ionDenVol(elem,ion) */
typedef struct mcx_lines {
    double  hbeta_vol;          /* out: HbetaVol [1e36 erg/s]                              */
    int32_t relative;           /* out: 1 when the line sums were divided by HbetaVol      */
    int32_t n_cells;            /* out: cells summed (active, lgBlack < 1)                 */
    double* hydro_vol;
    double* hei_vol;
    double* forb_vol;
    double* wav;
    double* te_vol;
    double* ion_vol;
    float   kernel_ms;          /* out: CUDA-event time of the sums                        */
    float   reserved_f[3];
    int64_t reserved[4];
} mcx_lines;

int  mcx_line_luminosities(mcx_ctx* ctx, mcx_lines* out);

/* The same for nebula b of a batch (mcx_load_batched): its cells only, its
 * octant factor. */
int  mcx_line_luminosities_nebula(mcx_ctx* ctx, int32_t nebula, mcx_lines* out);

/* When each nebula's last packet of the latest mcx_transport_batched (or
 * mcx_iterate_batched) call finished, in ms after the launch began
 * (ms[nebula], n = the batch size; 0 for a nebula without packets).  The
 * batched kernel stamps the GPU's global timer as a lane finishes a packet.
 * No counterpart in the reference (one nebula per job). */
int  mcx_batch_transport_ms(mcx_ctx* ctx, double* ms, int32_t n);


/* ------------------------------------------- transport without allocation */
/* No counterpart in the reference.  Some callers cannot allocate device
 * memory themselves: a Fortran or C host that receives device buffers from a
 * framework's own pool, or code that runs where cudaMalloc is not allowed
 * while other work holds the device.  This entry point runs the same transport
 * kernel as mcx_transport but allocates nothing: the caller passes every input
 * and output as a device pointer, and the kernel's scratch (work-queue head and
 * counters, the per-cell volumes, the re-emission CDF rows and the Compton
 * tables transposed for sampling) lives in one file-scope __device__ array of
 * MCX_NOALLOC_SCRATCH_BYTES that every GPU loading libmcx.so holds until the
 * process exits.  Problems whose scratch would exceed it are rejected with
 * MCX_ERR_INPUT.
 *  - The first call on a device looks up that array's device address
 *    (cudaGetSymbolAddress) with the device current; make that first call
 *    before any stream capture.
 *  - Every call shares the one array: calls whose work overlaps on the GPU
 *    (different streams or threads at the same time) race on it.  The entry
 *    point clears the counters each call and rewrites the rest.
 *  - Gas only (no dust), single mother grid, source 1, arrays in the Fortran
 *    layouts given at the top of this header. */
#define MCX_NOALLOC_SCRATCH_BYTES (64u * 1024u * 1024u)

typedef struct mcx_noalloc_transport_args {
    int32_t nx, ny, nz, n_cells, nbins;
    int32_t symmetric_xyz, lg_compton, precision;  /* precision: MCX_PREC_* */
    int32_t star_idx[3];        /* 1-based                                   */
    int32_t zero_estimators;    /* 1: clear jste/escaped first               */
    float   star_pos[3];
    float   ion_edge1, r_out;
    int32_t pad0;
    double  delta_e;            /* Lstar / nPhotons                          */
    int64_t n_packets;
    uint64_t seed, counter_base;
    /* device pointers, caller-owned */
    const float*   x_axis;      /* [nx]                                     */
    const float*   y_axis;      /* [ny]                                     */
    const float*   z_axis;      /* [nz]                                     */
    const int32_t* active;      /* [nz][ny][nx]                             */
    const float*   nu;          /* [nbins]                                  */
    const float*   src_cdf;     /* [nbins]                                  */
    const float*   kn_sigma_t;  /* [nbins]                                  */
    const float*   kn_cdf;      /* [180][nbins] KNsigmaArray(nbins,180)     */
    const float*   pcomp;       /* [180][nbins] PcompArray(nbins,180)       */
    const float*   opacity;     /* [nbins][C+1]                             */
    const float*   rec_pdf;     /* [nbins][C+1]                             */
    const float*   total_lines; /* [C+1]                                    */
    const float*   ne;          /* [C+1]                                    */
    double*        jste;        /* [nbins][C+1]   accumulated               */
    double*        escaped;     /* [nbins+1][C+1] accumulated               */
    void*          stream;      /* cudaStream_t; NULL = legacy default stream */
} mcx_noalloc_transport_args;

int  mcx_transport_noalloc(const mcx_noalloc_transport_args* args, mcx_transport_stats* stats);
/* Message of the last mcx_transport_noalloc failure of this thread. */
const char* mcx_noalloc_last_error(void);

/* ------------------------------------------------------------- timing */
/* CUDA events on the context stream (for callers that time a group of calls). */
int  mcx_timer_start(mcx_ctx* ctx);
int  mcx_timer_stop(mcx_ctx* ctx, float* ms);

/* ------------------------------------------------------------- version */
const char* mcx_version(void);

#ifdef __cplusplus
}
#endif
#endif /* MCX_H */
