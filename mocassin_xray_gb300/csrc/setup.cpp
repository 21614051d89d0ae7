// setup.cpp - builds the host-side model of one nebula from an input deck.
//
// Restates, in C++, the set-up routines that run once before the MOCASSIN
// iteration loop:
//   readInput                    source/set_input_mod.f90:12-708  (keyword grammar, defaults, checks)
//   setComposition               source/composition_mod.f90:10-70
//   phInit / phFitEl / phFitHIon source/ph_mod.f90:523-676
//   initCartesianGrid (nu mesh)  source/grid_mod.f90:21-608, fill() :610-648
//   setPointers / setShells      source/hydro_mod.f90:422-640, getOuterShell :89-180
//   initXSecArray                source/ph_mod.f90:204-517, powLawXSec :809-830, makeOpacity :833-880
//   setCompton                   source/ph_mod.f90:1883-1969
//   setContinuum / getFlux / setProbDen   source/continuum_mod.f90:33-504
//   fillGrid / setMotherGrid     source/grid_mod.f90:651-1832, getVolume :2887-2986
//   setStarPosition              source/grid_mod.f90:3690-3790
// Quantities the reference holds as default REAL are stored as float.
#include "setup_internal.h"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <stdexcept>

namespace mcx {

namespace {

// physical constants of source/constants_mod.f90 and source/continuum_mod.f90
constexpr float kRydToeV = 13.6056981f;
constexpr float kHIonPot = 0.99946f;
constexpr float kHPlanck = 6.6262e-27f;
constexpr float kSigmaSB = 5.66956e-5f;
constexpr float kPi = 3.141592654f;
constexpr float kFourPi = 4.f * kPi;
constexpr float kHcRyd_k = 157893.94f;
constexpr float kHcRyd = 2.1799153e-11f;
constexpr float kCRyd = 3.2898423e15f;
constexpr float kRadio4p9GHz = 1.489434e-6f;
constexpr float kKshellLimit = 7.35e4f;

[[noreturn]] void fail(const std::string& msg) { throw std::runtime_error(msg); }

std::string joinPath(const std::string& dir, const std::string& f) {
  if (f.empty() || f[0] == '/' || dir.empty()) return f;
  return dir + "/" + f;
}

// Fortran list-directed record: tokens separated by blanks or commas, strings
// optionally quoted with ' or ".  A '/' outside quotes ends the record.
std::vector<std::string> splitRecord(const std::string& line) {
  std::vector<std::string> out;
  size_t i = 0, n = line.size();
  while (i < n) {
    while (i < n && (std::isspace((unsigned char)line[i]) || line[i] == ',')) ++i;
    if (i >= n) break;
    if (line[i] == '/') break;
    if (line[i] == '\'' || line[i] == '"') {
      char q = line[i++];
      std::string tok;
      while (i < n && line[i] != q) tok += line[i++];
      ++i;
      out.push_back(tok);
    } else {
      std::string tok;
      while (i < n && !std::isspace((unsigned char)line[i]) && line[i] != ',') tok += line[i++];
      out.push_back(tok);
    }
  }
  return out;
}

float toF(const std::vector<std::string>& t, size_t k, const std::string& kw) {
  if (k >= t.size()) fail("input deck: keyword '" + kw + "' is missing a value");
  std::string v = t[k];
  for (auto& c : v) if (c == 'd' || c == 'D') c = 'e';   // Fortran double exponent
  char* end = nullptr;
  double d = std::strtod(v.c_str(), &end);
  if (end == v.c_str()) fail("input deck: keyword '" + kw + "' has a non-numeric value '" + t[k] + "'");
  return (float)d;
}

int64_t toI(const std::vector<std::string>& t, size_t k, const std::string& kw) {
  return (int64_t)std::llround((double)toF(t, k, kw));
}

std::string toS(const std::vector<std::string>& t, size_t k, const std::string& kw) {
  if (k >= t.size()) fail("input deck: keyword '" + kw + "' is missing a value");
  return t[k];
}

// setMultiPhotoSources (source/set_input_mod.f90:741-800): the number of
// sources, then one list-directed READ per source of Tstellar, Lstar,
// contShape, x, y, z (fractions of the axes' last values), spID and tStep.
// A READ starts a new record and takes its values across records.
void readMultiPhotoSources(Params& p) {
  const std::string path = joinPath(p.baseDir, p.multiPhotoSources);
  std::ifstream in(path);
  if (!in) fail("setMultiPhotoSources: can't open ionising sources file " + path);
  auto readValues = [&](size_t n) {
    std::vector<std::string> v;
    std::string line;
    while (v.size() < n && std::getline(in, line))
      for (auto& x : splitRecord(line))
        if (v.size() < n) v.push_back(x);
    if (v.size() < n) fail("setMultiPhotoSources: " + path + " ends before its last source");
    return v;
  };
  const int64_t n = toI(readValues(1), 0, "nStars");
  if (n < 1 || n > 4096) fail("setMultiPhotoSources: invalid number of sources in " + path);
  p.starsIn.clear();
  for (int64_t i = 0; i < n; ++i) {
    const auto v = readValues(8);
    StarIn st;
    st.TStellar = toF(v, 0, "Tstellar");
    st.LStar = toF(v, 1, "Lstar");
    st.contShape = v[2];
    for (int d = 0; d < 3; ++d) st.pos[d] = toF(v, 3 + d, "starPosition");
    st.spID = v[6];
    st.tStep = toF(v, 7, "tStep");
    p.starsIn.push_back(st);
  }
}

// The deck's single-source fields set to source `st` (each source's spectrum
// and position are built with them).
void useStar(Params& p, const StarIn& st) {
  p.contShape = st.contShape;
  p.spID = (st.contShape == "blackbody" || st.contShape == "powerlaw") ? st.contShape : st.spID;
  p.tStep = st.tStep;
  p.TStellar = st.TStellar;
  p.LStar = st.LStar;
  for (int d = 0; d < 3; ++d) p.starPos[d] = st.pos[d];
}

// readInput (source/set_input_mod.f90:140-500): one keyword per record.
void parseInput(Params& p, const std::string& path) {
  std::ifstream in(path);
  if (!in) fail("readInput: can't open input deck " + path);
  std::string line;
  while (std::getline(in, line)) {
    auto t = splitRecord(line);
    if (t.empty()) continue;
    const std::string& kw = t[0];
    if (kw == "radPress") p.lgRadPress = true;
    else if (kw == "noCompton") p.lgCompton = false;
    else if (kw == "noBadnell") p.lgBadnell = false;
    else if (kw == "nstages") p.nstages = (int)toI(t, 1, kw);
    else if (kw == "fillingFactor") p.fillingFactor = toF(t, 1, kw);
    else if (kw == "edges") { p.Rnx = toF(t, 1, kw); p.Rny = toF(t, 2, kw); p.Rnz = toF(t, 3, kw); }
    else if (kw == "output") p.lgOutput = true;
    else if (kw == "autoPackets") {
      p.lgAutoPackets = true;
      p.convIncPercent = toF(t, 1, kw); p.nPhotIncrease = toF(t, 2, kw); p.maxPhotons = toI(t, 3, kw);
    }
    else if (kw == "oneD") p.lg1D = true;
    else if (kw == "densityFile") { p.densityFile = toS(t, 1, kw); p.lgDfile = true; }
    else if (kw == "dustFile") { p.dustFile[0] = toS(t, 1, kw); p.dustFile[1] = toS(t, 2, kw); }
    else if (kw == "nbins") p.nbins = (int)toI(t, 1, kw);
    else if (kw == "talk") p.lgTalk = true;
    else if (kw == "symmetricXYZ") p.lgSymmetricXYZ = true;
    else if (kw == "contShape") {
      p.haveContShape = true;
      p.contShape = toS(t, 1, kw);
      if (p.contShape == "powerlaw") {
        p.pwlIndex = toF(t, 2, kw); p.pwlMin = toF(t, 3, kw); p.pwlMax = toF(t, 4, kw);
      }
      // any other shape names a spectrum file, read in the 'rauch' format
      // (source/set_input_mod.f90:320-324)
    }
    else if (kw == "nebComposition") {
      std::string v = toS(t, 1, kw);
      if (v == "noGas") p.lgGas = false; else { p.abundanceFile = v; p.haveAbundance = true; }
    }
    else if (kw == "Hdensity") { p.Hdensity = toF(t, 1, kw); p.lgHdenConstant = true; }
    else if (kw == "densityLaw") {
      for (int j = 0; j < 3; ++j) p.densityLaw[j] = toF(t, 1 + j, kw);
      p.lgDlaw = true;
    }
    else if (kw == "maxIterateMC") { p.maxIterateMC = (int)toI(t, 1, kw); p.minConvergence = toF(t, 2, kw); }
    else if (kw == "nPhotons") { p.nPhotons = toI(t, 1, kw); p.haveNPhotons = true; }
    else if (kw == "nx") p.nx = (int)toI(t, 1, kw);
    else if (kw == "ny") p.ny = (int)toI(t, 1, kw);
    else if (kw == "nz") p.nz = (int)toI(t, 1, kw);
    else if (kw == "starPosition") {
      for (int j = 0; j < 3; ++j) p.starPos[j] = toF(t, 1 + j, kw);
      p.haveStarPos = true;
    }
    else if (kw == "TeStart") p.TeStart = toF(t, 1, kw);
    else if (kw == "TStellar") { p.TStellar = toF(t, 1, kw); p.haveTStellar = true; }
    else if (kw == "convLimit") p.XHILimit = toF(t, 1, kw);
    else if (kw == "LStar") { p.LStar = toF(t, 1, kw); p.haveLStar = true; }
    else if (kw == "LPhot") p.LPhot = toF(t, 1, kw);
    else if (kw == "nuMax") p.nuMax = toF(t, 1, kw);
    else if (kw == "nuMin") p.nuMin = toF(t, 1, kw);
    else if (kw == "Rin") p.R_in = toF(t, 1, kw);
    else if (kw == "Rout") p.R_out = toF(t, 1, kw);
    else if (kw == "writeGrid") p.convWriteGrid = toF(t, 1, kw);
    else if (kw == "Ndust") {
      std::string mode = toS(t, 1, kw);
      if (mode == "constant") { p.NdustValue = toF(t, 2, kw); p.lgDustConstant = true; p.lgDust = true; }
      else if (mode == "file") { p.NdustFile = toS(t, 2, kw); p.lgDust = true; }
      else fail("readInput: Ndust needs 'constant' or 'file'");
    }
    else if (kw == "noScattering") p.lgDustScattering = false;
    else if (kw == "inclination") {
      // source/set_input_mod.f90:472-495: nAngleBins, then (theta, phi) [rad] per viewing angle
      p.nAngleBins = (int)toI(t, 1, kw);
      if (p.nAngleBins > 2)
        fail("readInput: only two inclination angles are allowed per simulation");
      if (p.nAngleBins < 0) fail("readInput: negative number of inclination angles");
      for (int j = 0; j < p.nAngleBins; ++j) {
        p.viewTheta[j] = toF(t, 2 + 2 * j, kw);
        p.viewPhi[j] = toF(t, 3 + 2 * j, kw);
      }
    }
    else if (kw == "H0Start" || kw == "NeStart" || kw == "debug" || kw == "traceHeating" ||
             kw == "noPhotoelectric" || kw == "separateSED") {
      // accepted; these do not change the transport + balance path built here
    }
    else if (kw == "planeIonization") {
      p.meanFieldin = toF(t, 1, kw); p.nu0 = toF(t, 2, kw); p.nu0Add = toF(t, 3, kw);
      p.lgPlaneIonization = true;
      p.LStar = 0.f;
    }
    else if (kw == "multiPhotoSources") p.multiPhotoSources = toS(t, 1, kw);
    else if (kw == "multiGrids" || kw == "multiChemistry" ||
             kw == "2D" || kw == "diffuseSource" ||
             kw == "quantumHeatGrain" || kw == "resLinesTransfer" || kw == "MdMg" || kw == "MdMh" ||
             kw == "fluorescence" || kw == "nahar") {
      fail("readInput: keyword '" + kw + "' selects a reference path outside this library's scope");
    }
    else fail("readInput: invalid keyword in model parameter input file: " + kw);
  }

  if (!p.multiPhotoSources.empty()) {
    // the sources come from the file (the deck's contShape, TStellar, Lstar and starPosition are not
    // used); the checks below see source 1
    readMultiPhotoSources(p);
    if (p.lgPlaneIonization) fail("readInput: planeIonization with multiPhotoSources");
    if (p.LPhot != 0.f) fail("readInput: LPhot with multiPhotoSources (each source's Lstar is in its file)");
    for (size_t i = 0; i < p.starsIn.size(); ++i) {
      const StarIn& st = p.starsIn[i];
      const std::string at = "setMultiPhotoSources: source " + std::to_string(i + 1);
      if (st.contShape == "powerlaw") fail(at + ": a powerlaw source needs pwlIndex, which the file does not carry");
      if (st.contShape == "blackbody" && st.TStellar <= 0.f) fail(at + ": TStellar must be given for a blackbody");
      if (st.contShape != "blackbody" && st.spID != "rauch" && st.spID != "sb99")
        fail(at + ": unsupported spectrum ID '" + st.spID + "'");
      if (st.LStar <= 0.f) fail(at + ": Lstar must be positive");
    }
    useStar(p, p.starsIn[0]);
    p.haveContShape = p.haveLStar = p.haveTStellar = true;
  }

  // consistency checks of source/set_input_mod.f90:560-704 (those on this path)
  if (!p.haveContShape) fail("readInput: no information about the continuum shape - contShape -");
  if (!p.haveNPhotons) fail("readInput: no information about the number of energy packets - nPhotons -");
  if (!p.lgPlaneIonization && !p.haveLStar && p.LPhot <= 0.f)
    fail("readInput: no information about the stellar luminosity - Lstar or Lphot -");
  if (p.lg1D) fail("readInput: oneD is outside this library's scope");
  if (p.lgGas && !p.haveAbundance) fail("readInput: no elemental abundance file has been specified");
  if (!p.lgDust && !p.lgGas) fail("readInput: the grid is completely empty. no gas or dust present.");
  if (p.fillingFactor > 1.f) fail("readInput: fillingFactor > 1");
  if (!p.lgDfile && (p.Rnx < 0.f || p.Rny < 0.f || p.Rnz < 0.f) && p.NdustFile.empty())
    fail("readInput: invalid or missing grid edges");
  if (p.contShape == "blackbody" && p.TStellar == 0.f) fail("readInput: TStellar must be given for a blackbody");
  if (p.R_in < 0.f) fail("readInput: invalid or missing inner radius Rin");
  if (p.LPhot == 0.f && p.LStar == 0.f && !p.lgPlaneIonization) fail("readInput: Lstar or LPhot must be given");
  if (p.lgPlaneIonization) {
    if (p.nx <= 2 || p.nz <= 2)
      fail("readInput: plane parallel simulation must have cuboid sides at least 3 cells deep (nx, nz >= 3)");
    if (!p.lgDfile)
      fail("readInput: plane ionizing field specified - must use user defined density distribution via densityFile");
    // the reference drops symmetricXYZ here, except where an earlier branch of its
    // else-if chain (the warning on edges given beside a density file) was taken
    if (p.lgSymmetricXYZ && !(p.Rnx >= 0.f || p.Rny >= 0.f || p.Rnz >= 0.f)) p.lgSymmetricXYZ = false;
    if (p.lgSymmetricXYZ) fail("readInput: planeIonization with symmetricXYZ");
  }
  if (p.LPhot != 0.f && p.LStar != 0.f) fail("readInput: Lstar and LPhot are mutually exclusive");
  if (p.maxIterateMC < 1) fail("readInput: invalid maxIterateMC");
  if (p.minConvergence < 0.f || p.minConvergence > 100.f) fail("readInput: invalid minConvergence");
  if (p.nPhotons < 0) fail("readInput: invalid nPhotons");
  if (p.lgDust && (p.dustFile[0].empty() || p.dustFile[1].empty())) fail("readInput: dust needs dustFile");
  if (p.nx < 1 || p.ny < 1 || p.nz < 1) fail("readInput: invalid nx, ny or nz");
  if (p.TStellar < 0.f || p.XHILimit < 0.f || p.LPhot < 0.f || p.LStar < 0.f || p.nuMax < 0.f ||
      p.nuMin < 0.f || p.R_out < 0.f)
    fail("readInput: negative physical parameter");
  if (p.R_in >= p.R_out && p.R_out > 0.f) fail("readInput: the inner radius must be smaller than the outer radius");
  if (p.fillingFactor < 1.f) fail("readInput: fillingFactor < 1 draws random numbers at set-up; outside this library's scope");
  if (p.lgDlaw) fail("readInput: densityLaw is outside this library's scope");
  if (p.nstages < 2 || p.nstages > 31) fail("readInput: nstages must be in [2,31]");
}

// sortUp (source/interpolation_mod.f90:7-35): ascending, duplicates dropped,
// the tail filled with 1e30.
void sortUp(float* arr, int n) {
  std::vector<float> tmp(n);
  float mn = 1.e30f;
  for (int i = 0; i < n; ++i) if (arr[i] < mn) mn = arr[i];
  tmp[0] = mn;
  for (int j = 1; j < n; ++j) {
    mn = 1.e30f;
    for (int i = 0; i < n; ++i) if (arr[i] < mn && arr[i] > tmp[j - 1]) mn = arr[i];
    tmp[j] = mn;
  }
  std::copy(tmp.begin(), tmp.end(), arr);
}

std::vector<std::vector<double>> readNumbers(const std::string& path) {
  std::ifstream in(path);
  if (!in) fail("can't open data file " + path);
  std::vector<std::vector<double>> rows;
  std::string line;
  while (std::getline(in, line)) {
    auto t = splitRecord(line);
    std::vector<double> r;
    for (auto& s : t) {
      std::string v = s;
      for (auto& c : v) if (c == 'd' || c == 'D') c = 'e';
      char* end = nullptr;
      double d = std::strtod(v.c_str(), &end);
      if (end == v.c_str()) break;
      r.push_back(d);
    }
    if (!r.empty()) rows.push_back(r);
  }
  return rows;
}

// ------------------------------------------------------------ composition
void setComposition(Setup& s) {
  auto rows = readNumbers(joinPath(s.p.baseDir, s.p.abundanceFile));
  if ((int)rows.size() < kNElements) fail("setComposition: abundance file needs 30 records: " + s.p.abundanceFile);
  s.nElemUsed = 0;
  int icount = 1;
  for (int e = 0; e < kNElements; ++e) {
    s.elemAbun[e] = (float)rows[e][0];
    if (s.elemAbun[e] > 1.e-12f) { s.elemOn[e] = true; s.elemXref[e] = icount++; ++s.nElemUsed; }
    else { s.elemOn[e] = false; s.elemXref[e] = 0; }
  }
}

// --------------------------------------------------------------- Verner
const int kNInn[30] = {0,0,1,1,1,1,1,1,1,1,3,3,3,3,3,3,3,3,5,5,5,5,5,5,5,5,5,5,5,5};
const int kNTot[30] = {1,1,2,2,3,3,3,3,3,3,4,4,5,5,5,5,5,5,6,6,6,6,6,6,6,6,6,6,7,7};
const int kLevel[7] = {0, 0, 1, 0, 1, 2, 0};

// ph1(i,nz,ne,shell) with 1-based arguments
inline float& PH1(Setup& s, int i, int nz, int ne, int shell) { return s.ph1[shell - 1][ne - 1][nz - 1][i - 1]; }
inline float PH1c(const Setup& s, int i, int nz, int ne, int shell) { return s.ph1[shell - 1][ne - 1][nz - 1][i - 1]; }
inline float& PH2(Setup& s, int i, int nz, int ne) { return s.ph2[ne - 1][nz - 1][i - 1]; }
inline float PH2c(const Setup& s, int i, int nz, int ne) { return s.ph2[ne - 1][nz - 1][i - 1]; }

void phInit(Setup& s) {
  auto r1 = readNumbers(joinPath(s.dataDir, "ph1.dat"));
  auto r2 = readNumbers(joinPath(s.dataDir, "ph2.dat"));
  size_t k1 = 0;
  for (int j = 1; j <= 30; ++j)
    for (int k = 1; k <= j; ++k) {
      int nt = kNTot[k - 1];
      if (j == k && k > 18) nt = 7;
      if (j == k + 1 && (j == 20 || j == 21 || j == 22 || j == 25 || j == 26)) nt = 7;
      for (int l = 1; l <= nt; ++l) {
        if (k1 >= r1.size() || r1[k1].size() < 6) fail("phInit: data/ph1.dat is truncated");
        for (int i = 1; i <= 6; ++i) PH1(s, i, j, k, l) = (float)r1[k1][i - 1];
        ++k1;
      }
    }
  size_t k2 = 0;
  for (int k = 1; k <= 30; ++k)
    for (int j = 1; j <= k; ++j)
      if (k != 15 && k != 17 && k != 19 && (k <= 20 || k == 26)) {
        if (k2 >= r2.size() || r2[k2].size() < 7) fail("phInit: data/ph2.dat is truncated");
        for (int i = 1; i <= 7; ++i) PH2(s, i, k, j) = (float)r2[k2][i - 1];
        ++k2;
      }
}

// phFitEl (source/ph_mod.f90:578-631): Verner et al. 1996 partial cross
// section of shell `shell` of ion (nz, ne) at photEn [eV], in Mb.
float phFitEl(const Setup& s, int nz, int ne, int shell, float photEn) {
  if (nz < 1 || nz > 30) return 0.f;
  if (ne < 1 || ne > nz) return 0.f;
  int nOut = kNTot[ne - 1];
  if (nz == ne && nz > 18) nOut = 7;
  if (nz == ne + 1 && (nz == 20 || nz == 21 || nz == 22 || nz == 25 || nz == 26)) nOut = 7;
  if (shell > nOut) return 0.f;
  if (photEn < PH1c(s, 1, nz, ne, shell)) return 0.f;
  int nInt = kNInn[ne - 1];
  float eInn;
  if (nz == 15 || nz == 17 || nz == 19 || (nz > 20 && nz != 26)) eInn = 0.f;
  else eInn = (ne < 3) ? 1.e30f : PH1c(s, 1, nz, ne, nInt);
  if (shell < nOut && shell > nInt && photEn < eInn) return 0.f;
  double xs;
  if (shell <= nInt || photEn >= eInn) {
    double p1 = -PH1c(s, 5, nz, ne, shell);
    double y = photEn / PH1c(s, 2, nz, ne, shell);
    double q = -0.5 * p1 - kLevel[shell - 1] - 5.5;
    double a = PH1c(s, 3, nz, ne, shell) * ((y - 1.0) * (y - 1.0) + (double)PH1c(s, 6, nz, ne, shell) * PH1c(s, 6, nz, ne, shell));
    double b = std::sqrt(y / PH1c(s, 4, nz, ne, shell)) + 1.;
    xs = a * std::pow(y, q) * std::pow(b, p1);
  } else {
    double p1 = -PH2c(s, 4, nz, ne);
    double q = -0.5 * p1 - 5.5;
    double x = photEn / PH2c(s, 1, nz, ne) - PH2c(s, 6, nz, ne);
    double z = std::sqrt(x * x + (double)PH2c(s, 7, nz, ne) * PH2c(s, 7, nz, ne));
    double a = PH2c(s, 2, nz, ne) * ((x - 1.) * (x - 1.) + (double)PH2c(s, 5, nz, ne) * PH2c(s, 5, nz, ne));
    double b = std::sqrt(z / PH2c(s, 3, nz, ne)) + 1.;
    xs = a * std::pow(z, q) * std::pow(b, p1);
  }
  return (float)xs;
}

// phFitHIon (source/ph_mod.f90:634-676): hydrogenic excited-level cross section [cm^2].
float phFitHIon(float x, int n, float z) {
  static const float a[10] = {-17.2004f,-16.8584f,-16.6670f,-16.5339f,-16.4319f,-16.3491f,-16.2795f,-16.2194f,-16.1666f,-16.1195f};
  static const float b[10] = {-2.6671f,-2.8068f,-2.8549f,-2.8812f,-2.8983f,-2.9103f,-2.9193f,-2.9264f,-2.9321f,-2.9369f};
  static const float c[10] = {-0.3228f,-0.1323f,-0.0931f,-0.0735f,-0.0612f,-0.0527f,-0.0465f,-0.0418f,-0.0380f,-0.0350f};
  static const float d[10] = {0.0608f,0.0224f,0.0224f,0.0204f,0.0181f,0.0163f,0.0147f,0.0135f,0.0125f,0.0117f};
  static const float e[10] = {-16.9991f,-16.7709f,-16.6188f,-16.5012f,-16.4069f,-16.3289f,-16.2624f,-16.2046f,-16.1536f,-16.1078f};
  static const float f[10] = {-3.1304f,-3.0041f,-2.9738f,-2.9671f,-2.9662f,-2.9669f,-2.9681f,-2.9694f,-2.9707f,-2.9719f};
  if (n > 10 || n < 1) fail("phFitHIon: quantum number n out of range [1,10]");
  double v = (x <= 1.f) ? a[n - 1] + x * (b[n - 1] + x * (c[n - 1] + x * d[n - 1])) : e[n - 1] + x * f[n - 1];
  return (float)(std::pow(10.0, v) / ((double)z * z));
}

// ------------------------------------------------------------ frequency mesh
// fill (source/grid_mod.f90:610-648), single precision as in the reference.
void fillSeg(float enlo, float enhi, float resolv, int& n0, std::vector<float>& nu, std::vector<float>& wid, int nbinsMax) {
  int ifill0 = n0 - 1;
  int nbin = (int)(logf(10.f) * log10f(enhi / enlo) / resolv + 1.f);
  float fildel = log10f(enhi / enlo) / (float)nbin;
  float filres;
  if (fildel < 0.01f) filres = logf(10.f) * fildel;
  else filres = (powf(10.f, 2.f * fildel) - 1.f) / 2.f / powf(10.f, fildel);
  if (n0 + nbin > nbinsMax) fail("fill: insufficient bins allowed for current frequency grid resolution");
  for (int i = 1; i <= nbin; ++i) {
    float v = enlo * powf(10.f, fildel * ((float)i - 0.5f));
    nu[i + ifill0 - 1] = v;
    wid[i + ifill0 - 1] = v * filres;
  }
  n0 += nbin;
}

void computeIonEdges(Setup& s) {
  std::vector<float> edges(450, 0.f);
  int nEdges = 1;
  for (int elem = 1; elem <= kNElements; ++elem) {
    for (int ion = 1; ion <= std::min(elem, s.p.nstages - 1); ++ion) {
      if (!s.elemOn[elem - 1]) break;
      if (elem > 2) {
        int nElec = elem - ion + 1, outShell, g0, g1;
        getOuterShell(elem, nElec, outShell, g0, g1);
        edges[nEdges - 1] = PH1c(s, 1, elem, nElec, outShell) / kRydToeV;
      } else if (elem == 1) {
        edges[nEdges - 1] = 0.999434f;
      } else if (elem == 2 && ion == 1) {
        edges[nEdges - 1] = 1.80804f;
      } else {
        edges[nEdges - 1] = 4.f;
      }
      if (edges[nEdges - 1] <= s.p.nuMax) ++nEdges;
    }
  }
  nEdges -= 1;
  if (nEdges > 0) sortUp(edges.data(), nEdges);
  s.ionEdge.assign(edges.begin(), edges.begin() + nEdges);
}

void buildMesh(Setup& s) {
  const Params& p = s.p;
  const bool fillMode = (p.nuMax > 25.f) && s.meshMode == 0;
  static const float seriesEdge[17] = {0.0069f, 0.0083f, 0.01f, 0.0123f, 0.0156f, 0.0204f, 0.0278f, 0.04f,
                                       0.0625f, 0.11117f, 0.11610f, 0.12248f, 0.13732f, 0.24763f, 0.24994f,
                                       0.26630f, 0.29189f};
  if (fillMode) {
    // source/grid_mod.f90:391-441 (non-fluorescence segments)
    int nb = 10000;
    std::vector<float> nu(nb, 0.f), wid(nb, 0.f);
    int n0 = 1;
    fillSeg(p.nuMin, 0.001f, 0.04f, n0, nu, wid, nb);
    fillSeg(0.001f, 0.109f, 0.03f, n0, nu, wid, nb);
    fillSeg(0.109f, 0.26f, 0.01f, n0, nu, wid, nb);
    fillSeg(0.26f, 0.90f, 0.009f, n0, nu, wid, nb);
    fillSeg(0.90f, 0.985f, 0.001f, n0, nu, wid, nb);
    fillSeg(0.985f, 1.01f, 0.001f, n0, nu, wid, nb);
    fillSeg(1.01f, 1.78f, 0.008f, n0, nu, wid, nb);
    fillSeg(1.78f, 1.82f, 0.002f, n0, nu, wid, nb);
    fillSeg(1.82f, 3.97f, 0.008f, n0, nu, wid, nb);
    fillSeg(3.97f, 4.05f, 0.002f, n0, nu, wid, nb);
    fillSeg(4.05f, 50.0f, 0.008f, n0, nu, wid, nb);
    fillSeg(50.f, 468.f, 0.01f, n0, nu, wid, nb);
    fillSeg(468.f, 472.f, 0.0005f, n0, nu, wid, nb);
    fillSeg(472.f, 600.f, 0.01f, n0, nu, wid, nb);
    fillSeg(600.f, 7e4f, 0.05f, n0, nu, wid, nb);
    fillSeg(7e4f, 7.3e6f, 0.10f, n0, nu, wid, nb);
    int nbins = n0 - 1;
    if (nu[nbins - 1] < p.nuMax) fail("initCartesianGrid: nuArray(nbins)<nuMaxArray");
    for (int i = 1; i <= n0; ++i) {
      if (nu[nbins - 1] > p.nuMax) --nbins; else break;
    }
    s.nbins = nbins;
    s.nu.assign(nu.begin(), nu.begin() + nbins);
    s.widFlx.assign(wid.begin(), wid.begin() + nbins);
  } else if (p.lgGas && !p.lgDust) {
    // source/grid_mod.f90:261-312 (log mesh with edges inserted)
    int nbins = p.nbins;
    std::vector<float> nu(nbins, 0.f);
    int nuCount;
    if (p.nuMin < kRadio4p9GHz) { nu[0] = kRadio4p9GHz; nuCount = 2; } else nuCount = 1;
    float nuMinArray = p.nuMin, nuMaxArray = p.nuMax;
    for (int i = 0; i < 17; ++i) {
      if (nuCount + 2 > nbins) fail("initCartesianGrid: nbins too small for the frequency edges");
      nu[nuCount - 1] = seriesEdge[i];
      nu[nuCount] = seriesEdge[i] - 0.0003f;
      nu[nuCount + 1] = seriesEdge[i] + 0.0003f;
      if (nu[nuCount - 1] < nuMinArray) nuMinArray = nu[nuCount - 1] - 0.0006f;
      if (nu[nuCount - 1] > nuMaxArray) nuMaxArray = nu[nuCount - 1];
      nuCount += 3;
    }
    for (size_t i = 0; i < s.ionEdge.size(); ++i) {
      if (s.ionEdge[i] < nuMaxArray) {
        if (nuCount + 2 > nbins) fail("initCartesianGrid: nbins too small for the frequency edges");
        nu[nuCount - 1] = s.ionEdge[i];
        nu[nuCount] = s.ionEdge[i] - 0.0003f;
        nu[nuCount + 1] = s.ionEdge[i] + 0.0003f;
        if (nu[nuCount - 1] < nuMinArray) nuMinArray = nu[nuCount - 1] - 0.0006f;
        nuCount += 3;
      }
    }
    int iCount = nbins - nuCount + 1;
    if (iCount < 2) fail("initCartesianGrid: nbins too small for the log mesh");
    float nuStepSize = (log10f(nuMaxArray) - log10f(nuMinArray)) / (float)(iCount - 1);
    nu[nuCount - 1] = nuMinArray;
    for (int i = nuCount + 1; i <= nbins; ++i) nu[i - 1] = powf(10.f, log10f(nu[i - 2]) + nuStepSize);
    sortUp(nu.data(), nbins);
    std::vector<float> wid(nbins);
    wid[0] = nu[1] - nu[0];
    for (int i = 2; i <= nbins - 1; ++i) wid[i - 1] = (nu[i] - nu[i - 2]) / 2.f;
    wid[nbins - 1] = nu[nbins - 1] - nu[nbins - 2];
    s.nbins = nbins; s.nu = nu; s.widFlx = wid;
  } else if (p.lgDust && !p.lgGas) {
    // source/grid_mod.f90:232-259: dustData/nuDustRyd.dat up to nuMax
    auto rows = readNumbers(joinPath(s.dataDir, "../dustData/nuDustRyd.dat"));
    std::vector<float> nu;
    for (auto& r : rows) {
      if ((int)nu.size() + 1 > p.nbins + 1) fail("initCartesianGrid: nbins is smaller than nuDustRyd.dat");
      float v = (float)r[0];
      nu.push_back(v);
      if (v > p.nuMax) break;
    }
    // the record that exceeded nuMax is read but not counted (nbins = i-1)
    if (!nu.empty() && nu.back() > p.nuMax) nu.pop_back();
    int nbins = (int)nu.size();
    std::vector<float> wid(nbins);
    wid[0] = nu[1] - nu[0];
    for (int i = 2; i <= nbins - 1; ++i) wid[i - 1] = (nu[i] - nu[i - 2]) / 2.f;
    wid[nbins - 1] = nu[nbins - 1] - nu[nbins - 2];
    s.nbins = nbins; s.nu = nu; s.widFlx = wid;
  } else {
    fail("initCartesianGrid: gas+dust frequency mesh is outside this library's scope");
  }
  if (s.widFlx[0] <= 0.f || s.widFlx[s.nbins - 1] <= 0.f) fail("initCartesianGrid: null or negative frequency bin");
}

// ----------------------------------------------------------- pointers
int limitShell(const Setup& s, int ion, int shell, int nElem) {
  switch (shell) {
    case 1: case 2: case 3: return s.KshellLimitP;
    case 4: case 5: case 6: return s.elementP[nElem - 1][ion - 1][0][0] - 1;
    case 7:
      if (s.elementP[nElem - 1][ion - 1][5][0] < 3) return s.elementP[nElem - 1][ion - 1][4][0] - 1;
      return s.elementP[nElem - 1][ion - 1][5][0] - 1;
    default: fail("limitShell: shell number out of range [1, 7]");
  }
}

void setShells(Setup& s, int nElem) {
  const float* nu = s.nu.data();
  for (int ion = 1; ion <= nElem; ++ion) {
    int nElec = nElem - ion + 1, outShell, g0, g1;
    getOuterShell(nElem, nElec, outShell, g0, g1);
    s.nShells[nElem - 1][ion - 1] = outShell;
    float thres = 0.f;
    for (int shell = 1; shell <= outShell; ++shell) {
      thres = PH1c(s, 1, nElem, nElec, shell) / kRydToeV;
      int* P = s.elementP[nElem - 1][ion - 1][shell - 1];
      if (thres <= 0.1f) { P[0] = 2; P[1] = 1; }
      else {
        P[0] = locate(nu, s.nbins, thres);
        P[1] = limitShell(s, ion, shell, nElem);
      }
    }
    s.elementP[nElem - 1][ion - 1][outShell - 1][0] = locate(nu, s.nbins, thres);
  }
}

void setPointers(Setup& s) {
  const float* nu = s.nu.data();
  int nb = s.nbins;
  s.KshellLimitP = locate(nu, nb, kKshellLimit);
  s.secIonP = locate(nu, nb, 7.353f);
  s.cRecoilHP = locate(nu, nb, 194.f);
  s.cRecoilHeP = locate(nu, nb, 260.f);
  s.xrayP = locate(nu, nb, 20.6f);
  s.BjumpP = locate(nu, nb, 0.25f);
  // makeHydro (source/hydro_mod.f90:62-86)
  for (int n = 1; n <= kNHlevel; ++n) s.HlevEn[n - 1] = kHIonPot / (float)(n * n);
  s.HlevEn[kNHlevel] = s.HlevEn[1];
  for (int n = 1; n <= kNHeIlevel; ++n) s.HeIlevEn[n - 1] = 1.f / (float)(n * n);
  s.HeIlevEn[0] = 1.80802f; s.HeIlevEn[1] = 0.2478f;
  s.HeIlevEn[kNHeIlevel] = s.HeIlevEn[1];
  for (int n = 1; n <= kNHeIIlevel; ++n) s.HeIIlevEn[n - 1] = 4.f / (float)(n * n);
  s.HeIIlevEn[kNHeIIlevel] = s.HeIIlevEn[1];
  for (int i = 1; i <= kNHlevel; ++i) s.HlevNuP[i - 1] = locate(nu, nb, s.HlevEn[i - 1]);
  s.HlevNuP[kNHlevel] = s.HlevNuP[1];
  for (int i = 1; i <= kNHeIlevel; ++i) s.HeIlevNuP[i - 1] = locate(nu, nb, s.HeIlevEn[i - 1]);
  s.HeIlevNuP[kNHeIlevel] = s.HeIlevNuP[1];
  for (int i = 1; i <= kNHeIIlevel; ++i) s.HeIIlevNuP[i - 1] = locate(nu, nb, s.HeIIlevEn[i - 1]);
  s.HeIIlevNuP[kNHeIIlevel] = s.HeIIlevNuP[1];
  s.nShells[0][0] = 1; s.nShells[1][0] = 1; s.nShells[1][1] = 1;
  static const int order[28] = {6, 8, 7, 10, 11, 12, 13, 14, 15, 16, 17, 26, 18, 19, 20, 21, 22, 23, 24, 25,
                                9, 3, 4, 5, 27, 28, 29, 30};
  for (int e : order) if (s.elemOn[e - 1]) setShells(s, e);
}

// --------------------------------------------------------------- x sections
void powLawXSec(Setup& s, std::vector<float>& tmp, int& xSecTop, int low, int high, float cross, float sExp, int& xSecP) {
  xSecP = xSecTop + 1;
  float thres = s.nu[low - 1];
  for (int i = low; i <= high; ++i) tmp[i - low + xSecP - 1] = cross * powf(s.nu[i - 1] / thres, -sExp);
  xSecTop += high - low + 1;
}

void setCompton(Setup& s) {
  int nb = s.nbins;
  s.KNsigmaT.assign(nb, 0.f);
  s.KNcdf.assign((size_t)kNAngles * nb, 0.f);
  s.Pcomp.assign((size_t)kNAngles * nb, 0.f);
  std::vector<float> kn((size_t)kNAngles);
  for (int i = 0; i < nb; ++i) {
    float E = s.nu[i];
    float tot = 0.f;
    for (int j = 1; j <= kNAngles; ++j) {
      float thetarad = (float)j * kPi / 180.f;
      float P = 1.f / (1.f + (E / 37557.66267f) * (1.f - cosf(thetarad)));          // Pcomp
      float st = sinf(thetarad);
      float knv = 3.970393838e-26f * (P - (P * P) * (st * st) + P * P * P);          // KNsigma
      s.Pcomp[(size_t)(j - 1) * nb + i] = P;
      kn[j - 1] = knv;
      tot += knv * 2.f * kPi * sinf((float)j * kPi / 180.f) * kPi / 180.f;
    }
    s.KNsigmaT[i] = tot;
    float c = kn[0] * 2.f * kPi * sinf(kPi / 180.f) * kPi / 180.f;
    s.KNcdf[i] = c;
    for (int j = 2; j <= kNAngles; ++j) {
      c = c + kn[j - 1] * 2.f * kPi * sinf((float)j * kPi / 180.f) * kPi / 180.f;
      s.KNcdf[(size_t)(j - 1) * nb + i] = c;
    }
    for (int j = 1; j <= kNAngles; ++j) s.KNcdf[(size_t)(j - 1) * nb + i] /= tot;
    s.KNcdf[(size_t)(kNAngles - 1) * nb + i] = 1.f;
  }
  // Compton heating / cooling x sections and recoil (source/ph_mod.f90:387-409)
  s.comXSecH.assign(nb, 0.f); s.comXSecC.assign(nb, 0.f); s.xSecRecoil.assign(nb, 0.f);
  const float thom = 6.65e-25f;
  for (int i = 1; i <= nb; ++i) {
    float v = s.nu[i - 1];
    float alpha = 1.f / (1.f + v * (1.1792e-4f + 7.084e-10f * v));
    float beta = (1.f - alpha * v * (1.1792e-4f + 2.f * 7.084e-10f * v) / 4.f);
    s.comXSecH[i - 1] = alpha * v * v * 3.858e-25f;
    s.comXSecC[i - 1] = alpha * beta * v * 3.858e-25f;
    if (i <= s.xrayP) s.xSecRecoil[i - 1] = thom;
    else {
      // The reference evaluates this in single precision, where the first
      // bracket (of order dx^3 against terms of order dx) cancels
      // catastrophically below dx ~ 0.05 (about 2000 Ryd): its values there
      // depend on the compiler's logf, swing up to 150 sigma_T and turn
      // negative.  The same formula (with the reference's (1+2dx)^3 in the
      // last term) is evaluated here in FP64 and stored in single precision.
      const double dx = (double)v / 3.7573e4;
      const double l = std::log(1. + 2. * dx);
      s.xSecRecoil[i - 1] = (float)((double)thom * 3. / 4. *
                                    ((1. + dx) / (dx * dx * dx) * (2. * dx * (1. + dx) / (1. + 2. * dx) - l) +
                                     1. / 2. / dx * l - (1. + 3. * dx) / ((1. + 2. * dx) * (1. + 2. * dx) * (1. + 2. * dx))));
    }
  }
}

void initXSecArray(Setup& s) {
  std::vector<float> tmp(1000000, 0.f);
  int xSecTop = 0;
  const int nb = s.nbins;
  const float* nu = s.nu.data();
  s.HlevXSecP[0] = xSecTop + 1;
  setPointers(s);
  if (s.p.lgCompton) setCompton(s);
  else { s.KNsigmaT.assign(nb, 0.f); s.KNcdf.assign((size_t)kNAngles * nb, 0.f); s.Pcomp.assign((size_t)kNAngles * nb, 0.f); }

  // H ground state
  for (int i = s.HlevNuP[0]; i <= nb; ++i) {
    float thres = std::max(nu[i - 1] * kRydToeV, PH1c(s, 1, 1, 1, 1));
    tmp[i - s.HlevNuP[0] + s.HlevXSecP[0] - 1] = phFitEl(s, 1, 1, 1, thres) * 1e-18f;
  }
  xSecTop += nb - s.HlevNuP[0] + 1;
  for (int n = 2; n <= kNHlevel; ++n) {
    s.HlevXSecP[n - 1] = xSecTop + 1;
    for (int i = s.HlevNuP[n - 1]; i <= s.HlevNuP[0]; ++i) {
      float x = log10f(nu[i - 1]) - log10f(nu[s.HlevNuP[n - 1] - 1]);
      tmp[i - s.HlevNuP[n - 1] + s.HlevXSecP[n - 1] - 1] = phFitHIon(x, n, 1.f);
    }
    xSecTop += s.HlevNuP[0] - s.HlevNuP[n - 1] + 1;
  }
  s.bremsXSecP = xSecTop + 1;
  for (int i = 1; i <= nb; ++i) tmp[i - 1 + s.bremsXSecP - 1] = 1.03680e-18f / (nu[i - 1] * nu[i - 1] * nu[i - 1]);
  xSecTop += nb;
  s.HeISingXSecP[0] = xSecTop + 1;
  for (int i = s.HeIlevNuP[0]; i <= nb; ++i)
    tmp[i - s.HeIlevNuP[0] + s.HeISingXSecP[0] - 1] = phFitEl(s, 2, 2, 1, nu[i - 1] * kRydToeV) * 1e-18f;
  xSecTop += nb - s.HeIlevNuP[0] + 1;
  powLawXSec(s, tmp, xSecTop, s.HeIlevNuP[1], s.HeIlevNuP[0], 0.4f * 8.7e-18f, 1.5f, s.HeISingXSecP[1]);
  for (int n = 3; n <= kNHeIlevel; ++n) {
    float xs = 7.906e-18f * (float)n / (1.f * 1.f);
    powLawXSec(s, tmp, xSecTop, s.HeIlevNuP[n - 1], s.HeIlevNuP[0], xs, 3.0f, s.HeISingXSecP[n - 1]);
  }
  s.HeIIXSecP[0] = xSecTop + 1;
  for (int i = s.HeIIlevNuP[0]; i <= nb; ++i) {
    float thres = std::max(nu[i - 1] * kRydToeV, PH1c(s, 1, 2, 1, 1));
    tmp[i - s.HeIIlevNuP[0] + s.HeIIXSecP[0] - 1] = phFitEl(s, 2, 1, 1, thres) * 1e-18f;
  }
  xSecTop += nb - s.HeIIlevNuP[0] + 1;
  for (int n = 2; n <= kNHeIIlevel; ++n) {
    s.HeIIXSecP[n - 1] = xSecTop + 1;
    for (int i = s.HeIIlevNuP[n - 1]; i <= s.HeIIlevNuP[0]; ++i) {
      float x = log10f(nu[i - 1]) - log10f(nu[s.HeIIlevNuP[n - 1] - 1]);
      tmp[i - s.HeIIlevNuP[n - 1] + s.HeIIXSecP[n - 1] - 1] = phFitHIon(x, n, 2.f);
    }
    xSecTop += s.HeIIlevNuP[0] - s.HeIIlevNuP[n - 1] + 1;
  }
  // heavy elements (makeOpacity, source/ph_mod.f90:833-880)
  for (int nElem = 3; nElem <= kNElements; ++nElem) {
    if (!s.elemOn[nElem - 1]) continue;
    for (int nIon = 1; nIon <= std::min(nElem, s.p.nstages); ++nIon) {
      int nElec = nElem - nIon + 1;
      for (int shell = 1; shell <= s.nShells[nElem - 1][nIon - 1]; ++shell) {
        int* P = s.elementP[nElem - 1][nIon - 1][shell - 1];
        P[2] = xSecTop + 1;
        int binsNeed = P[1] - P[0] + 1;
        if (xSecTop + binsNeed > 1000000) fail("makeOpacity: xSecMax exceeded");
        if (P[0] > P[1] && (P[0] != 2 || P[1] != 1))
          fail("makeOpacity: upper energy limit for this shell is smaller than threshold");
        for (int i = P[0]; i <= P[1]; ++i) {
          float energy = std::max(nu[i - 1] * kRydToeV, PH1c(s, 1, nElem, nElec, shell));
          tmp[i - P[0] + P[2] - 1] = phFitEl(s, nElem, nElec, shell, energy) * 1e-18f;
        }
        if (binsNeed >= 1) xSecTop += P[1] - P[0] + 1;
      }
    }
  }
  s.xSec.assign(tmp.begin(), tmp.begin() + xSecTop);
}

// ----------------------------------------------------------------- continuum
float getFlux(const Setup& s, float energy, float temperature) {
  if (s.p.contShape == "blackbody") {
    float constant = 0.5250229f / kHPlanck;
    if (kHcRyd_k * energy / temperature > 86.f)
      return constant * energy * energy * energy * expf(-kHcRyd_k * energy / temperature);
    float denominator = expf(kHcRyd_k * energy / temperature) - 1.f;
    if (denominator <= 0.f) return 3.32154e-6f * energy * energy * temperature / kHPlanck;
    return constant * energy * energy * energy / denominator;
  }
  // powerlaw
  return powf(energy, -s.p.pwlIndex) * expf(-energy / s.p.pwlMax) * expf(-s.p.pwlMin / energy);
}

// A tabulated spectrum in the 'rauch' format (setContinuum,
// source/continuum_mod.f90:214-262): rows of wavelength [A] (read as REAL)
// and H_lambda [erg/cm^2/s/A/sr] (FP64) in ascending wavelength; each row
// becomes H_nu (FP64) and nu [Ryd] (REAL), reversed into ascending frequency,
// and the mesh takes log-log interpolation between the rows that bracket it
// (zero where the row's flux is not above 1e-20); the caller multiplies by 4 pi.
void readSpectrumFile(Setup& s, std::vector<double>& erg) {
  const int nb = s.nbins;
  const auto rows = readNumbers(joinPath(s.p.baseDir, s.p.contShape));
  const float c = 2.9979250e10f;
  std::vector<double> hflux;
  std::vector<float> en;
  for (const auto& r : rows) {
    if (r.size() < 2) continue;
    const float lam = (float)r[0];
    hflux.push_back((r[1] * (double)(1.e-8f * (lam * lam))) / (double)c / 4.);
    en.push_back((c / (lam * 1.e-8f)) / kCRyd);
  }
  const int numLam = (int)en.size();
  if (numLam < 1) fail("setContinuum: no rows in spectrum file " + s.p.contShape);
  std::reverse(hflux.begin(), hflux.end());
  std::reverse(en.begin(), en.end());
  for (int i = 0; i < nb; ++i) {
    const float nu = s.nu[i];
    if (!(nu >= en[0] && nu <= en[numLam - 1])) continue;
    const int enP = locate(en.data(), numLam, nu);
    if (enP < numLam) {
      erg[i] = std::pow(10., std::log10(hflux[enP - 1]) + std::log10(hflux[enP] / hflux[enP - 1]) *
                                 (double)log10f(nu / en[enP - 1]) / (double)log10f(en[enP] / en[enP - 1]));
      if (!(hflux[enP - 1] > 1.e-20)) erg[i] = 0.;
    } else {
      erg[i] = hflux[enP - 1] > 1.e-20 ? hflux[enP - 1] : 0.;
    }
  }
}

// A Starburst99 spectrum (setContinuum, source/continuum_mod.f90:129-222): 7
// comment records, then records of time, wavelength [A], a skipped column and
// log L_lambda [erg/s/A]; the 1221 records that start at the first one of time
// tStep become L_nu [erg/s/Hz] (FP64) at nu [Ryd] (REAL) in ascending
// frequency.  Each is added to the mesh bin whose edges (the midpoints between
// mesh points; half widths at both ends) hold it, the bins are averaged, the
// photon spectrum is taken, and only then are the empty bins between filled
// ones interpolated linearly in the energy spectrum (so the photon spectrum
// stays 0 there, as in the reference).
void readSB99(Setup& s) {
  const int nb = s.nbins;
  constexpr int kSb99NuLim = 1221;
  const std::string path = joinPath(s.p.baseDir, s.p.contShape);
  std::ifstream in(path);
  if (!in) fail("setContinuum: can't open spectrum file " + path);
  std::string line;
  for (int j = 0; j < 7 && std::getline(in, line); ++j) {}
  std::vector<std::vector<std::string>> block;
  while (std::getline(in, line)) {
    auto t = splitRecord(line);
    if (t.empty()) continue;
    if (block.empty() && toF(t, 0, "sb99 time") != s.p.tStep) continue;
    block.push_back(t);
    if ((int)block.size() == kSb99NuLim) break;
  }
  if ((int)block.size() < kSb99NuLim)
    fail("setContinuum: " + path + " has no 1221 records at time step " + std::to_string(s.p.tStep));
  const float c = 2.9979250e10f;
  std::vector<double> hflux(kSb99NuLim);
  std::vector<float> en(kSb99NuLim);
  for (int k = 0; k < kSb99NuLim; ++k) {
    const float lam = toF(block[k], 1, "sb99 wavelength");
    std::string v = toS(block[k], 3, "sb99 log L");
    for (auto& ch : v) if (ch == 'd' || ch == 'D') ch = 'e';   // Fortran double exponent
    const double logL = std::strtod(v.c_str(), nullptr);
    // reversed into ascending frequency
    hflux[kSb99NuLim - 1 - k] = (std::pow(10., logL) * (double)(1.e-8f * (lam * lam))) / (double)c;
    en[kSb99NuLim - 1 - k] = (c / (lam * 1.e-8f)) / kCRyd;
  }
  std::vector<int> count(nb, 0);
  for (int j = 0; j < kSb99NuLim; ++j) {
    const float e = en[j];
    if (e >= s.nu[0] - s.widFlx[0] / 2.f && e < s.nu[0] + s.widFlx[0] / 2.f) {
      s.inSpectrumErg[0] += hflux[j];
      ++count[0];
    }
    for (int i = 1; i < nb - 1; ++i)
      if (e >= (s.nu[i - 1] + s.nu[i]) / 2.f && e < (s.nu[i + 1] + s.nu[i]) / 2.f) {
        s.inSpectrumErg[i] += hflux[j];
        ++count[i];
      }
    if (e >= s.nu[nb - 1] - s.widFlx[nb - 1] / 2.f && e < s.nu[nb - 1] + s.widFlx[nb - 1] / 2.f) {
      s.inSpectrumErg[nb - 1] += hflux[j];
      ++count[nb - 1];
    }
  }
  for (int i = 0; i < nb; ++i) {
    if (count[i] > 0) s.inSpectrumErg[i] = s.inSpectrumErg[i] / (double)(float)count[i];
    s.inSpectrumPhot[i] = s.inSpectrumErg[i] / (double)(s.nu[i] * kHcRyd);
  }
  for (int i = 1; i < nb - 1; ++i) {
    if (s.inSpectrumErg[i] <= 0. && s.inSpectrumErg[i - 1] > 0.) {
      for (int j = i + 1; j < nb; ++j)
        if (s.inSpectrumErg[j] > 0.) {
          s.inSpectrumErg[i] = s.inSpectrumErg[i - 1] - (double)(s.nu[i] - s.nu[i - 1]) *
                                                            (s.inSpectrumErg[i - 1] - s.inSpectrumErg[j]) /
                                                            (double)(s.nu[j] - s.nu[i - 1]);
          break;
        }
    }
  }
}

void setContinuum(Setup& s) {
  const int nb = s.nbins;
  s.lymanP = locate(s.nu.data(), nb, 1.f);
  s.inSpectrumErg.assign(nb, 0.);
  s.inSpectrumPhot.assign(nb, 0.);
  if (s.p.contShape == "blackbody" || s.p.contShape == "powerlaw") {
    for (int i = 0; i < nb; ++i) {
      s.inSpectrumErg[i] = getFlux(s, s.nu[i], s.p.TStellar);
      s.inSpectrumPhot[i] = s.inSpectrumErg[i] / ((double)s.nu[i] * (double)kHcRyd);
    }
  } else if (s.p.spID == "sb99") {
    readSB99(s);
  } else {
    readSpectrumFile(s, s.inSpectrumErg);
    for (int i = 0; i < nb; ++i) {
      s.inSpectrumPhot[i] = s.inSpectrumErg[i] / ((double)s.nu[i] * (double)kHcRyd);
      s.inSpectrumErg[i] = (double)kFourPi * s.inSpectrumErg[i];
      s.inSpectrumPhot[i] = (double)kFourPi * s.inSpectrumPhot[i];
    }
  }
  // setProbDen (source/continuum_mod.f90:415-504); inSpSum* are REAL there
  std::vector<float> sumErg(nb), sumPhot(nb);
  for (int i = 0; i < nb; ++i) { sumErg[i] = (float)s.inSpectrumErg[i]; sumPhot[i] = (float)s.inSpectrumPhot[i]; }
  float nce = 0.f, ncp = 0.f;
  for (int i = 0; i < nb; ++i) nce += sumErg[i] * s.widFlx[i];
  for (int i = s.lymanP; i <= nb; ++i) ncp += sumPhot[i - 1] * s.widFlx[i - 1];
  // a plane source emits nothing below nu0Add (source/continuum_mod.f90:472-483)
  int nu0AddP = 1;
  if (s.p.lgPlaneIonization && s.p.nu0Add > 0.f) nu0AddP = std::max(1, locate(s.nu.data(), nb, s.p.nu0Add));
  s.srcCDF.assign(nb, 0.f);
  s.srcCDF[nu0AddP - 1] = sumErg[nu0AddP - 1] * s.widFlx[nu0AddP - 1];
  for (int i = nu0AddP + 1; i <= nb; ++i) s.srcCDF[i - 1] = s.srcCDF[i - 2] + sumErg[i - 1] * s.widFlx[i - 1];
  float last = s.srcCDF[nb - 1];
  for (int i = 0; i < nb; ++i) s.srcCDF[i] /= last;
  float maxp = 0.f;
  for (int i = 0; i < nb; ++i) if (s.srcCDF[i] > maxp) maxp = s.srcCDF[i];
  for (int i = 0; i < nb; ++i) if (s.srcCDF[i] >= maxp) s.srcCDF[i] = 1.f;
  if (s.p.contShape == "blackbody") { nce = kPi * nce * kHPlanck; ncp = kPi * ncp * kHPlanck; }
  s.normConstantErg = nce; s.normConstantPhot = ncp;
  // Lstar <-> LPhot (source/continuum_mod.f90:308-335), for one source only
  s.LPhot = s.p.LPhot; s.LStar = s.p.LStar;
  if (s.p.starsIn.size() > 1) return;
  if (s.LPhot > 0.f) {
    if (s.p.contShape == "powerlaw") fail("setContinuum: powerlaw does not allow Lphot; use Lstar");
    s.RStar = sqrtf(s.LPhot / (kFourPi * ncp * kCRyd));
    s.LStar = kFourPi * s.RStar * s.RStar * kSigmaSB * powf(s.p.TStellar, 4.f);
  } else if (s.LStar > 0.f) {
    if (s.p.contShape != "powerlaw") {
      s.RStar = sqrtf(s.LStar / (kFourPi * kSigmaSB * powf(s.p.TStellar, 4.f)));
      s.LPhot = kFourPi * s.RStar * s.RStar * ncp * kCRyd;
    }
  }
}

// ---------------------------------------------------------------------- grid
float getVolume(const Setup& s, int xP, int yP, int zP) {
  const auto& X = s.xAxis; const auto& Y = s.yAxis; const auto& Z = s.zAxis;
  // half-width first cells for a symmetric grid, half-width first and last
  // cells for a plane-parallel one (source/grid_mod.f90:2925-2981)
  const bool lo = s.p.lgSymmetricXYZ || s.p.lgPlaneIonization, hi = s.p.lgPlaneIonization;
  float dx = 0.f, dy = 0.f, dz = 0.f;
  if (xP > 1 && xP < s.nx) dx = fabsf(X[xP] - X[xP - 2]) / 2.f;
  else if (xP == 1) dx = lo ? fabsf(X[1] - X[0]) / 2.f : fabsf(X[1] - X[0]);
  else if (xP == s.nx) dx = hi ? fabsf(X[xP - 1] - X[xP - 2]) / 2.f : fabsf(X[xP - 1] - X[xP - 2]);
  if (yP > 1 && yP < s.ny) dy = fabsf(Y[yP] - Y[yP - 2]) / 2.f;
  else if (yP == 1) dy = lo ? fabsf(Y[1] - Y[0]) / 2.f : fabsf(Y[1] - Y[0]);
  else if (yP == s.ny) dy = hi ? fabsf(Y[yP - 1] - Y[yP - 2]) / 2.f : fabsf(Y[yP - 1] - Y[yP - 2]);
  if (zP > 1 && zP < s.nz) dz = fabsf(Z[zP] - Z[zP - 2]) / 2.f;
  else if (zP == 1) dz = lo ? fabsf(Z[1] - Z[0]) / 2.f : fabsf(Z[1] - Z[0]);
  else if (zP == s.nz) dz = hi ? fabsf(Z[zP - 1] - Z[zP - 2]) / 2.f : fabsf(Z[zP - 1] - Z[zP - 2]);
  dx /= 1.e15f; dy /= 1.e15f; dz /= 1.e15f;
  return dx * dy * dz;
}

void fillGrid(Setup& s) {
  const Params& p = s.p;
  s.nx = p.nx; s.ny = p.ny; s.nz = p.nz;
  if (s.nx < 2 || s.ny < 2 || s.nz < 2) fail("fillGrid: each axis needs at least 2 points");
  s.xAxis.assign(s.nx, 0.f); s.yAxis.assign(s.ny, 0.f); s.zAxis.assign(s.nz, 0.f);
  if (!p.lgDfile && p.NdustFile.empty()) {
    if (p.lgSymmetricXYZ) {
      for (int i = 1; i <= s.nx; ++i) s.xAxis[i - 1] = (float)(i - 1) / (float)(s.nx - 1) * p.Rnx;
      for (int i = 1; i <= s.ny; ++i) s.yAxis[i - 1] = (float)(i - 1) / (float)(s.ny - 1) * p.Rny;
      for (int i = 1; i <= s.nz; ++i) s.zAxis[i - 1] = (float)(i - 1) / (float)(s.nz - 1) * p.Rnz;
    } else {
      if (s.nx % 2 == 0 || s.ny % 2 == 0 || s.nz % 2 == 0)
        fail("fillGrid: the automatic grid option requires odd nx, ny, nz if not symmetric");
      for (int i = 1; i <= s.nx; ++i) s.xAxis[i - 1] = (2.f * (float)(i - 1) / (float)(s.nx - 1) - 1.f) * p.Rnx;
      for (int i = 1; i <= s.ny; ++i) s.yAxis[i - 1] = (2.f * (float)(i - 1) / (float)(s.ny - 1) - 1.f) * p.Rny;
      for (int i = 1; i <= s.nz; ++i) s.zAxis[i - 1] = (2.f * (float)(i - 1) / (float)(s.nz - 1) - 1.f) * p.Rnz;
    }
  }
  const size_t nvox = (size_t)s.nx * s.ny * s.nz;
  std::vector<float> HdenTemp(nvox, 0.f), NdustTemp(nvox, 0.f);
  auto vidx = [&](int i, int j, int k) { return (size_t)(i - 1) + (size_t)s.nx * ((size_t)(j - 1) + (size_t)s.ny * (size_t)(k - 1)); };
  s.active.assign(nvox, 1);
  if (p.lgGas) {
    std::vector<std::vector<double>> rows;
    size_t r = 0;
    if (p.lgDfile) rows = readNumbers(joinPath(p.baseDir, p.densityFile));
    for (int i = 1; i <= s.nx; ++i)
      for (int j = 1; j <= s.ny; ++j)
        for (int k = 1; k <= s.nz; ++k) {
          if (p.lgHdenConstant) HdenTemp[vidx(i, j, k)] = p.Hdensity;
          else if (p.lgDfile) {
            if (r >= rows.size() || rows[r].size() < 4) fail("setMotherGrid: density file is truncated");
            s.xAxis[i - 1] = (float)rows[r][0]; s.yAxis[j - 1] = (float)rows[r][1]; s.zAxis[k - 1] = (float)rows[r][2];
            HdenTemp[vidx(i, j, k)] = (float)rows[r][3];
            ++r;
          } else fail("setMotherGrid: no density distribution was set");
        }
  }
  if (p.lgDust) {
    if (p.lgDustConstant) std::fill(NdustTemp.begin(), NdustTemp.end(), p.NdustValue);
    else {
      auto rows = readNumbers(joinPath(p.baseDir, p.NdustFile));
      size_t r = 0;
      for (int i = 1; i <= s.nx; ++i)
        for (int j = 1; j <= s.ny; ++j)
          for (int k = 1; k <= s.nz; ++k) {
            if (r >= rows.size() || rows[r].size() < 4) fail("setMotherGrid: Ndust file is truncated");
            s.xAxis[i - 1] = (float)rows[r][0]; s.yAxis[j - 1] = (float)rows[r][1]; s.zAxis[k - 1] = (float)rows[r][2];
            NdustTemp[vidx(i, j, k)] = (float)rows[r][3];
            ++r;
          }
    }
  }
  // active cells (source/grid_mod.f90:1222-1295): i outer, k fastest
  s.nCells = 0;
  for (int i = 1; i <= s.nx; ++i)
    for (int j = 1; j <= s.ny; ++j)
      for (int k = 1; k <= s.nz; ++k) {
        size_t v = vidx(i, j, k);
        float radius = 1.e10f * sqrtf((s.xAxis[i - 1] / 1.e10f) * (s.xAxis[i - 1] / 1.e10f) +
                                      (s.yAxis[j - 1] / 1.e10f) * (s.yAxis[j - 1] / 1.e10f) +
                                      (s.zAxis[k - 1] / 1.e10f) * (s.zAxis[k - 1] / 1.e10f));
        if (!p.lgPlaneIonization) {   // no radial cuts for a plane-parallel slab (source/grid_mod.f90:1258)
          if (radius < p.R_in) s.active[v] = 0;
          else if (radius > p.R_out && p.R_out > 0.f) s.active[v] = 0;
        }
        if (s.active[v] <= 0) { NdustTemp[v] = 0.f; HdenTemp[v] = 0.f; }
        bool on;
        if (p.lgDust && p.lgGas) on = HdenTemp[v] > 0.f || NdustTemp[v] > 0.f;
        else if (p.lgDust) on = NdustTemp[v] > 0.f;
        else on = HdenTemp[v] > 0.f;
        if (on) s.active[v] = ++s.nCells;
        else { s.active[v] = 0; HdenTemp[v] = 0.f; NdustTemp[v] = 0.f; }
      }
  if (s.nCells <= 0) fail("setMotherGrid: no active cells");
  const size_t C1 = (size_t)s.nCells + 1;
  s.Hden.assign(C1, 0.f); s.Te.assign(C1, 0.f); s.Ne.assign(C1, 0.f);
  s.TeOld.assign(C1, 0.f); s.NeOld.assign(C1, 0.f);
  s.volume.assign(C1, 0.f); s.Ndust.assign(C1, 0.f);
  const int E = std::max(s.nElemUsed, 1), S = p.nstages;
  s.ionDen.assign((size_t)S * E * C1, 0.f);
  auto ID = [&](int c, int e, int st) -> float& { return s.ionDen[(size_t)c + C1 * ((size_t)(e - 1) + (size_t)E * (size_t)(st - 1))]; };
  for (int i = 1; i <= s.nx; ++i)
    for (int j = 1; j <= s.ny; ++j)
      for (int k = 1; k <= s.nz; ++k) {
        int c = s.activeAt(i, j, k);
        if (c <= 0) continue;
        size_t v = vidx(i, j, k);
        if (p.lgGas) { s.Hden[c] = HdenTemp[v]; s.Te[c] = p.TeStart; }
        if (p.lgDust) s.Ndust[c] = NdustTemp[v];
        s.volume[c] = getVolume(s, i, j, k);
        if (!p.lgGas) continue;
        // initial ionisation state (source/grid_mod.f90:1600-1654)
        const float H0in = 1.e-5f;
        if (s.elemOn[0]) { ID(c, s.elemXref[0], 1) = H0in; ID(c, s.elemXref[0], 2) = 1.f - ID(c, s.elemXref[0], 1); }
        if (s.elemOn[1]) {
          ID(c, s.elemXref[1], 1) = ID(c, 1, 1);
          ID(c, s.elemXref[1], 2) = (1.f - ID(c, s.elemXref[1], 1)) / 2.f;
          ID(c, s.elemXref[1], 3) = ID(c, s.elemXref[1], 2);
        }
        s.Ne[c] = s.Hden[c];
        for (int elem = 3; elem <= kNElements; ++elem)
          for (int ion = 1; ion <= std::min(elem + 1, S); ++ion)
            if (s.elemOn[elem - 1]) {
              if (ion == 1) ID(c, s.elemXref[elem - 1], ion) = ID(c, 1, 1);
              else ID(c, s.elemXref[elem - 1], ion) = (1.f - ID(c, s.elemXref[0] > 0 ? s.elemXref[0] : 1, 1)) / (float)std::min(elem, S - 1);
            }
      }
}

// The ionising plane of a plane-parallel model (setMotherGrid,
// source/grid_mod.f90:1761-1822; fillGrid :852): the photon flux meanField
// above nu0 scales the spectrum, the part below nu0Add is cut, and the
// transferred energy flux times the x-z extent of the grid is the source's
// luminosity; R_out becomes the grid's largest extent.  REAL arithmetic, as
// in the reference.
void setPlaneSource(Setup& s) {
  Params& p = s.p;
  const int nb = s.nbins;
  const float* nu = s.nu.data();
  float meanField = p.meanFieldin;
  if (p.nu0 > 0.f) {
    int nu0P = locate(nu, nb, p.nu0);
    if (nu0P < nb && nu0P > 0 && p.nu0 > (nu[nu0P - 1] + nu[nu0P]) / 2.f) nu0P += 1;
    int nu0AddP;
    if (p.nu0Add != p.nu0) {
      nu0AddP = locate(nu, nb, p.nu0Add);
      if (nu0AddP < nb && nu0AddP > 0 && p.nu0Add > (nu[nu0AddP - 1] + nu[nu0AddP]) / 2.f) nu0AddP += 1;
    } else {
      nu0AddP = nu0P;
    }
    if (nu0P >= nb || nu0P < 1) fail("setMotherGrid: nu0 outside the frequency mesh");
    float norm = 0.f;
    for (int i = nu0P; i <= nb; ++i) norm = norm + (float)s.inSpectrumPhot[i - 1] * s.widFlx[i - 1];
    const float scale = meanField / norm;
    norm = 0.f;
    for (int i = 1; i <= nb; ++i) {
      if (i < nu0AddP) s.inSpectrumErg[i - 1] = 0.;
      norm = norm + (float)s.inSpectrumErg[i - 1] * s.widFlx[i - 1];
    }
    meanField = norm * scale;
  }
  s.LStar = (meanField / 1.e36f) * (s.xAxis[s.nx - 1] - s.xAxis[0]) * (s.zAxis[s.nz - 1] - s.zAxis[0]);
  s.LPhot = 0.f;
  p.R_out = 1.e10f * sqrtf((s.xAxis[s.nx - 1] / 1.e10f) * (s.xAxis[s.nx - 1] / 1.e10f) +
                           (s.yAxis[s.ny - 1] / 1.e10f) * (s.yAxis[s.ny - 1] / 1.e10f) +
                           (s.zAxis[s.nz - 1] / 1.e10f) * (s.zAxis[s.nz - 1] / 1.e10f));
}

void setStarPosition(Setup& s) {
  const Params& p = s.p;
  for (int d = 0; d < 3; ++d) s.starPos[d] = p.starPos[d];
  s.starPos[0] *= s.xAxis[s.nx - 1]; s.starPos[1] *= s.yAxis[s.ny - 1]; s.starPos[2] *= s.zAxis[s.nz - 1];
  const std::vector<float>* ax[3] = {&s.xAxis, &s.yAxis, &s.zAxis};
  int n[3] = {s.nx, s.ny, s.nz};
  int P[3];
  for (int d = 0; d < 3; ++d) {
    const float* A = ax[d]->data();
    P[d] = locate(A, n[d], s.starPos[d]);
    if (P[d] < n[d] && P[d] > 0 && s.starPos[d] > (A[P[d] - 1] + A[P[d]]) / 2.f) P[d] += 1;
  }
  bool outside = false;
  for (int d = 0; d < 3; ++d) {
    const float* A = ax[d]->data();
    if (s.starPos[d] > A[n[d] - 1] || s.starPos[d] < A[0]) outside = true;
  }
  if (outside) { s.starIdx[0] = s.starIdx[1] = s.starIdx[2] = -1; }
  else { for (int d = 0; d < 3; ++d) s.starIdx[d] = P[d]; }
}

}  // namespace

// getOuterShell (source/hydro_mod.f90:89-180)
void getOuterShell(int z, int nElec, int& outShell, int& g0, int& g1) {
  static const int ss[30] = {1,1,2,2,3,3,3,3,3,3,4,4,5,5,5,5,5,5,6,6,6,6,6,6,6,6,6,6,7,7};
  static const int gl[30] = {2,1,2,1,6,9,4,9,6,1,2,1,6,9,4,9,6,1,2,1,10,21,28,7,6,25,28,21,2,1};
  static const int glhigh[12] = {10,21,28,25,6,25,28,21,10,1,2,1};   // indices 19..30
  if (z > 30) fail("getOuterShell: atomic number out of range");
  if (nElec < 1 || nElec > z) fail("getOuterShell: number of electrons out of range");
  outShell = ss[nElec - 1];
  if (z == nElec && z > 18) outShell = 7;
  if (z == nElec + 1 && (z == 20 || z == 21 || z == 22 || z == 25 || z == 26)) outShell = 7;
  g0 = gl[nElec - 1];
  g1 = (nElec == 1) ? 1 : gl[nElec - 2];
  if (z > 20 && nElec >= 19 && (z - nElec) >= 1) {
    g0 = glhigh[nElec - 19];
    g1 = (nElec == 19) ? gl[nElec - 2] : glhigh[nElec - 20];
  }
  if (z == nElec) {
    if (z > 20 && nElec >= 21) g1 = glhigh[nElec - 20];
    switch (z) { case 21: g1 = 15; break; case 22: g1 = 28; break; case 25: g1 = 7; break; case 26: g1 = 30; break; default: break; }
  }
  if (z - nElec == 1) {
    switch (z) { case 21: g0 = 15; break; case 22: g0 = 28; break; case 25: g0 = 7; break; case 26: g0 = 30; break; default: break; }
  }
}


int locate(const float* xa, int n, float x) {
  if (x > xa[n - 1]) return n;
  if (x < xa[0]) return 0;
  int jlow = 0, jup = n + 1;
  const bool asc = xa[n - 1] > xa[0];
  for (int it = 0; it < 10000; ++it) {
    if (jup - jlow < 1) break;
    int jm = (jup + jlow) / 2;
    if (xa[jm - 1] == x) return jm;
    if (asc == (x > xa[jm - 1])) {
      if (jlow == jm) break;   // the bisection no longer moves: the reference loops to imax and returns jlow
      jlow = jm;
    } else {
      jup = jm;
    }
  }
  return jlow;
}

void buildSetup(Setup& s, const std::string& inputFile, const std::string& dataDir, int meshMode) {
  s.dataDir = dataDir;
  s.meshMode = meshMode;
  std::string base = inputFile;
  size_t slash = base.find_last_of('/');
  // relative file names in a deck are relative to the directory that holds input/ (the run directory)
  std::string deckDir = (slash == std::string::npos) ? "." : base.substr(0, slash);
  size_t s2 = deckDir.find_last_of('/');
  s.p.baseDir = (deckDir.size() >= 5 && deckDir.substr(deckDir.size() - 5) == "input")
                    ? (s2 == std::string::npos ? std::string(".") : deckDir.substr(0, s2))
                    : deckDir;
  parseInput(s.p, inputFile);
  if (s.p.lgGas) setComposition(s);
  phInit(s);
  if (s.p.lgGas) computeIonEdges(s);
  buildMesh(s);
  if (s.p.lgGas) initXSecArray(s);
  if (s.p.lgGas && s.p.lgDust) fail("makeDustXsec: gas and dust in one grid are outside this library's scope");
  if (s.p.lgDust) buildDustTables(s);
  if (!s.p.lgGas) {   // no Compton tables without gas (setCompton is part of initXSecArray)
    s.KNsigmaT.assign(s.nbins, 0.f);
    s.KNcdf.assign((size_t)kNAngles * s.nbins, 0.f);
    s.Pcomp.assign((size_t)kNAngles * s.nbins, 0.f);
  }
  if (s.p.lgGas) {
    buildEmissionTables(s);
    buildBalanceTables(s);
  }
  // every source's spectrum and position (multiPhotoSources), source 1 last so that the
  // single-source fields hold it
  const int nStars = s.p.starsIn.empty() ? 1 : (int)s.p.starsIn.size();
  s.stars.assign(nStars, Setup::Star{});
  for (int i = nStars - 1; i >= 0; --i) {
    if (!s.p.starsIn.empty()) useStar(s.p, s.p.starsIn[i]);
    setContinuum(s);
    s.stars[i].cdf = s.srcCDF;
  }
  fillGrid(s);
  if (s.p.lgPlaneIonization) setPlaneSource(s);
  for (int i = nStars - 1; i >= 0; --i) {
    if (!s.p.starsIn.empty()) useStar(s.p, s.p.starsIn[i]);
    setStarPosition(s);
    Setup::Star& st = s.stars[i];
    for (int d = 0; d < 3; ++d) { st.pos[d] = s.starPos[d]; st.idx[d] = s.starIdx[d]; }
    st.TStellar = s.p.TStellar;
    st.LStar = s.p.starsIn.empty() ? s.LStar : s.p.starsIn[i].LStar;
  }
  s.stars[0].cdf = s.srcCDF;   // (a plane source's luminosity and CDF cut are set above)
  if (s.p.lgDust) {   // dustDriver's initial grain temperatures (source/dust_mod.f90:66-73)
    const size_t planes = (size_t)(s.dust.nSpecies + 1) * (s.dust.nSizes + 1);
    s.Tdust.assign(planes * ((size_t)s.nCells + 1), 50.f);
  }
}

}  // namespace mcx
