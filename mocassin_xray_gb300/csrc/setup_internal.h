// setup_internal.h - host-side model of one nebula: parsed input deck, frequency
// mesh, cross-section tables, source spectrum and the initial grid state.
// Built by setup.cpp; consumed by mcx_api.cu (upload to the device).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace mcx {

constexpr int kNElements = 30;      // nElements (source/constants_mod.f90:62)
constexpr int kNHlevel = 10;        // nHlevel
constexpr int kNHeIlevel = 9;       // nHeIlevel
constexpr int kNHeIIlevel = 9;      // nHeIIlevel
constexpr int kNAngles = 180;       // Compton theta bins (source/ph_mod.f90:1889)

// One ionising source of a multiPhotoSources file (setMultiPhotoSources,
// source/set_input_mod.f90:741-800): a row of Tstellar, Lstar, contShape,
// position (fractions of the axes' last values) and, for a spectrum file, its
// reader (spID 'rauch' or 'sb99') and the Starburst99 time step.
struct StarIn {
  float TStellar = 0.f, LStar = 0.f;
  std::string contShape, spID;
  float pos[3] = {0.f, 0.f, 0.f};
  float tStep = 0.f;
};

// Parsed input deck (keyword grammar of source/set_input_mod.f90:140-500,
// defaults of :33-117).
struct Params {
  bool lgBadnell = true, lgCompton = true, lgRadPress = false;
  bool lgHdenConstant = false, lgDfile = false, lgDlaw = false;
  bool lgDust = false, lgDustConstant = false, lgGas = true;
  bool lgSymmetricXYZ = false, lg1D = false, lgPlaneIonization = false;
  bool lgAutoPackets = false, lgTalk = false, lgOutput = false;
  bool lgMdMg = false, lgMdMh = false, lgDustScattering = true;
  int nx = 30, ny = 30, nz = 30;
  int maxIterateMC = 30, nbins = 600, nstages = 17;
  int64_t nPhotons = 0;
  int64_t maxPhotons = 0;
  float convIncPercent = 0.f, nPhotIncrease = 0.f, convWriteGrid = 0.f;
  float minConvergence = 95.f;
  float Hdensity = 0.f, fillingFactor = 1.f;
  float densityLaw[3] = {0.f, 0.f, 0.f};
  float LPhot = 0.f, LStar = 0.f, TStellar = 0.f;
  float nuMax = 15.f, nuMin = 1.001e-5f;
  float Rnx = -1.f, Rny = -1.f, Rnz = -1.f, R_in = -1.f, R_out = 0.f;
  float TeStart = 10000.f, XHILimit = 0.05f;
  float NdustValue = 0.f, MdMgValue = 0.f;
  float pwlIndex = 0.f, pwlMin = 0.f, pwlMax = 0.f;
  float starPos[3] = {0.f, 0.f, 0.f};
  // 'planeIonization meanField nu0 nu0Add' (source/set_input_mod.f90:257-262):
  // the ionising plane's photon flux above nu0 [Ryd], and the frequency below
  // which the plane emits nothing
  float meanFieldin = 0.f, nu0 = 0.f, nu0Add = 0.f;
  int nAngleBins = 0;             // 'inclination': viewing angles (at most 2)
  float viewTheta[2] = {0.f, 0.f}, viewPhi[2] = {0.f, 0.f};
  bool haveStarPos = false, haveLStar = false, haveTStellar = false;
  bool haveContShape = false, haveNPhotons = false, haveAbundance = false;
  std::string contShape;          // "blackbody" | "powerlaw" | a spectrum file (read by spID)
  std::string spID = "rauch";     // reader of a spectrum file: 'rauch' or 'sb99'
  float tStep = 0.f;              // the Starburst99 time step a 'sb99' file is read at
  std::string multiPhotoSources;  // the file of several ionising sources
  std::vector<StarIn> starsIn;    // its rows (empty: one source from the deck's keywords)
  std::string densityFile, abundanceFile, NdustFile;
  std::string dustFile[2];
  std::string baseDir;            // directory the deck's relative paths are resolved against
};

// Tables of the emission phase (source/emission_mod.f90:336-1919), read once.
struct EmissionTables {
  // continuum emission coefficients gamma(nu, T) at the series edges (initGammaCont,
  // source/ph_mod.f90:31-200): [3] = HI, HeI, HeII
  int nTk = 0;
  int nlim[3] = {0, 0, 0};
  std::vector<float> tk;                 // [nTk]
  std::vector<int32_t> edgeP;            // [3][32] 1-based bins
  std::vector<float> logGamma;           // [3][nTk][32]
  // heavy-element free-bound terms (fb_ff, source/emission_mod.f90:550-614):
  // {elem, ion, IPnuP, highNuP, xSecP, g0, g1}
  std::vector<int32_t> fbHeavy;
  // hydrogenic recombination lines (RecLinesEmission, source/emission_mod.f90:856-1151)
  int nHydroFiles = 0;
  std::vector<int32_t> hydroFileMap;     // [9][12] file index for (izp, itemp)
  std::vector<int32_t> hydroNDens;       // [nFiles]
  std::vector<float> hydroDens;          // [nFiles][13]
  std::vector<float> hydroLines;         // [nFiles][13][14][8]  (iup 2..15, ilow 1..8)
  float HbCoeff[2][9][4] = {};           // HbACoeff, HbBCoeff (data/gaussfitHb.dat)
  float rbEdge[2][3][26] = {};           // data/r1bEdge.dat, data/r2bEdge.dat
  float r2aEdge[3][18] = {};             // data/r2aEdge.dat
  float hydroLinesTemps[12] = {};
  float HeIrec[34][3][4] = {};           // HeIrecLineCoeff (coefficient 1 scaled by 1e25)
  float HeI2phot[2][41] = {};            // y, Ay (data/HeI2phot.dat)
  float HeIILyman[2][4] = {};            // ratio, nu (data/r2a0100old.dat)
  int32_t HeIILymanP[4] = {};            // locate(nuArray, nu)
  int32_t j2TsP = 0;                     // locate(nuArray, 1.45673)
};

// Packed multi-level atom of one ion (the data equilibrium reads from its ion
// file, source/emission_mod.f90:2589-2880), header fields per atom:
enum AtomHdr {
  kAtElem = 0, kAtIon, kAtNLev, kAtNTemp, kAtIup2p, kAtRecType, kAtNRec, kAtOffLogT,
  kAtOffQom, kAtOffY2, kAtOffA, kAtOffG, kAtOffE, kAtOffRec, kAtOffAtp, kAtHdrSize = 16
};
// recombination-coefficient fits at the end of an ion file
enum AtomRec { kRecNone = 0, kRecPowerLaw = 1, kRecChianti = 2 };
constexpr int kRecWidth[3] = {0, 11, 5};   // br,z,a_r(4),a_d(5) | jj,a,b,c,d
constexpr int kMaxLevels = 30;             // nForLevels (source/constants_mod.f90)

// Tables of the per-cell balance (updateCell and the routines it calls,
// source/update_mod.f90), read once at set-up.
struct BalanceTables {
  float CF[kNElements][kNElements][5] = {};        // cion.dat CF(i,elem,nElec) at [elem-1][nElec-1][i-1]
  float cionTherm[kNElements][kNElements] = {};    // [elem-1][ion-1]
  int32_t nauger[kNElements][kNElements][10] = {}; // auger.dat [elem-1][ion-1][shell-1]
  float auger[kNElements][kNElements][10][10] = {};// [elem-1][ion-1][shell-1][nelec-1]
  float RRb[6][kNElements][kNElements + 1] = {};   // rrBadnell A,B,T0,T1,C,T2 at [k][z-1][n]
  float DRbC[kNElements][kNElements + 1][9] = {};  // drBadnell at [z-1][n][idr-1]
  float DRbE[kNElements][kNElements + 1][9] = {};
  float rrec[kNElements][kNElements][2] = {};      // radrec.dat at [z-1][n-1][i-1]
  float rnew[kNElements][kNElements][4] = {};
  std::vector<float> diel;                         // dielectronic.dat rows: elem,n,a,b,c,d,f,g
  std::vector<float> aldro;                        // aldrovandi.dat rows: elem,n,a,b,t0,t1
  int32_t outer[kNElements][kNElements][3] = {};   // getOuterShell(z, nElec): outShell, g0, g1
  // multi-level atoms of the ions with data (lgDataAvailable)
  int32_t atomIndex[kNElements][kNElements + 1];   // [elem-1][ion-1] -> atom slot, -1 none
  std::vector<int32_t> atomHdr;                    // [nAtoms][kAtHdrSize]
  std::vector<double> atomData;
  int nAtoms = 0;
  int maxLev = 0;
};

// Grain species and sizes (makeDustXsec, source/ph_mod.f90:938-1720, the 'Q'
// file type) and the emission integrals of dustEmissionInt
// (source/dust_mod.f90:141-184).
constexpr int kNTemps = 3000;     // nTemps (source/constants_mod.f90:69)
struct DustTables {
  int nSpecies = 0, nSizes = 0;
  std::vector<std::string> grainLabel;
  std::vector<float> grainAbun, TdustSublime;        // [nSpecies]
  std::vector<float> grainRadius, grainWeight, da;   // [nSizes]
  std::vector<float> Cabs, Csca, gCos;               // [nSpecies][nSizes][nbins] cm^2
  std::vector<float> CTabs, CTsca;                   // [nbins] abundance- and size-weighted
  std::vector<float> emIntegral;                     // [nSpecies][nSizes][nTemps]
};

struct Setup {
  Params p;
  EmissionTables em;
  BalanceTables bal;
  DustTables dust;
  std::string dataDir;
  int meshMode = 0;

  // composition (source/composition_mod.f90:10-70)
  float elemAbun[kNElements] = {};
  bool elemOn[kNElements] = {};
  int elemXref[kNElements] = {};   // 1-based index among used elements, 0 if off
  int nElemUsed = 0;

  // Verner fits (source/ph_mod.f90:523-573): ph1(6,30,30,7), ph2(7,30,30)
  float ph1[7][kNElements][kNElements][6] = {};   // [shell][ne][nz][i]
  float ph2[kNElements][kNElements][7] = {};       // [ne][nz][i]

  // frequency mesh
  int nbins = 0;
  std::vector<float> nu, widFlx;
  std::vector<float> ionEdge;                        // sorted, nEdges entries

  // mesh pointers (1-based like the reference)
  int lymanP = 0, KshellLimitP = 0, secIonP = 0, cRecoilHP = 0, cRecoilHeP = 0;
  int xrayP = 0, BjumpP = 0;
  int HlevNuP[kNHlevel + 1] = {}, HeIlevNuP[kNHeIlevel + 1] = {}, HeIIlevNuP[kNHeIIlevel + 1] = {};
  float HlevEn[kNHlevel + 1] = {}, HeIlevEn[kNHeIlevel + 1] = {}, HeIIlevEn[kNHeIIlevel + 1] = {};
  int nShells[kNElements][kNElements] = {};          // [elem-1][ion-1]
  int elementP[kNElements][kNElements][7][3] = {};   // [elem-1][ion-1][shell-1][k]

  // cross sections (source/ph_mod.f90:204-517)
  std::vector<float> xSec;                           // xSecArray (0-based storage, 1-based pointers)
  int HlevXSecP[kNHlevel] = {}, HeISingXSecP[kNHeIlevel] = {}, HeIIXSecP[kNHeIIlevel] = {};
  int bremsXSecP = 0;

  // Compton tables (source/ph_mod.f90:1883-1924, :370-410)
  std::vector<float> KNsigmaT;                       // [nbins]
  std::vector<float> KNcdf, Pcomp;                   // [180][nbins] (frequency fastest)
  std::vector<float> comXSecH, comXSecC, xSecRecoil; // [nbins]

  // source spectrum (source/continuum_mod.f90:33-504)
  std::vector<double> inSpectrumErg, inSpectrumPhot;
  std::vector<float> srcCDF;                         // inSpectrumProbDen(1,:)
  double normConstantErg = 0., normConstantPhot = 0.;
  float LStar = 0.f, LPhot = 0.f, RStar = 0.f;

  // grid
  int nx = 0, ny = 0, nz = 0, nCells = 0;
  std::vector<float> xAxis, yAxis, zAxis;
  std::vector<int32_t> active;                       // [nz][ny][nx]
  std::vector<float> Hden, Te, Ne, TeOld, NeOld;     // [nCells+1]
  std::vector<float> ionDen;                         // [nstages][nElemUsed][nCells+1]
  std::vector<float> volume;                         // [nCells+1]
  std::vector<float> Ndust;                          // [nCells+1]
  std::vector<float> Tdust;                          // [nSpecies+1][nSizes+1][nCells+1]
  int starIdx[3] = {-1, -1, -1};
  float starPos[3] = {0.f, 0.f, 0.f};
  // every ionising source (source 1 first; its values are also the scalars above)
  struct Star {
    float LStar = 0.f, TStellar = 0.f;
    float pos[3] = {0.f, 0.f, 0.f};       // [cm]
    int idx[3] = {-1, -1, -1};            // its cell, 1-based; -1 outside the grid
    std::vector<float> cdf;               // inSpectrumProbDen(i,:)
  };
  std::vector<Star> stars;

  inline int activeAt(int i, int j, int k) const {   // 1-based Fortran indices
    return active[(size_t)(i - 1) + (size_t)nx * ((size_t)(j - 1) + (size_t)ny * (size_t)(k - 1))];
  }
};

// Outer shell and ground statistical weights of (z, nElec) (getOuterShell, source/hydro_mod.f90:89-180).
void getOuterShell(int z, int nElec, int& outShell, int& g0, int& g1);

// Reads the emission-phase tables (after the mesh and cross sections exist).
void buildEmissionTables(Setup& s);

// Reads the rate tables and the multi-level atoms of the balance phase.
void buildBalanceTables(Setup& s);

// Reads the grain species and sizes and tabulates their emission integrals.
void buildDustTables(Setup& s);

// getFlux of source/continuum_mod.f90:358-405 for a blackbody (FP32).
float blackbodyFlux(float energy, float temperature);

// Builds a Setup from an input deck; throws std::runtime_error with a message.
void buildSetup(Setup& s, const std::string& inputFile, const std::string& dataDir, int meshMode);

// Bisection locate of source/interpolation_mod.f90:49-106 (1-based result:
// 0 below range, n above range, the matched index on an exact hit).
int locate(const float* xa, int n, float x);

}  // namespace mcx
