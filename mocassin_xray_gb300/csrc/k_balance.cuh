// k_balance.cuh - per-cell balance phase on the device: the T-iteration of
// updateCell/iterateT (source/update_mod.f90:15-482) for every cell at once.
//
// The reference recurses per cell (iterateT calls itself up to maxIterateT =
// 20 times, ionBalance up to 15 times).  Here every cell advances one
// T-iteration per round, and a round is launches over the cells still
// iterating:
//   rates   (8 lanes per cell)        calcAlpha, photoionisation, collisional
//                                     ionisation, compton, ionBalance, and the
//                                     thermBalance terms that need no atom solve
//   atoms   (thread per cell and ion) forLines: every ion's line cooling, by
//                                     its equilibrium (FP64 balance, or on
//                                     request) or read from its cooling surface
//   secant  (thread per cell)         heating - cooling, the bracketing secant
//                                     step, convergence and the cell's results
// A J-only pass before the first round integrates the photoionisation rates
// and Compton sums, which the reference recomputes on every T-iteration from
// the same J.  Two precisions: FP64 throughout, or FP32 rates, ladder and
// level populations with FP64 Te bracketing (k_balance_impl.cuh).
//
// Cooling surfaces (mixed balance).  Without the recombination term an ion's
// level populations, and so the sum G(Te, Ne) = sum_j n_j sum_i a(j,i) E_ji of
// its forLines cooling per ion, depend on Te and Ne alone (not on the cell).
// ln G of every atom is tabulated once per context on a grid uniform in ln Te
// (1..1e6 K, 1280 nodes) and ln Ne (1e-6..1e9 cm^-3, 640 nodes) from the same
// FP32 state-reduction solve, and read back by 4-point Lagrange interpolation
// in both directions (relative error of G ~1e-6, the size of the solve's own
// FP32 error); cells outside the grid solve their atoms directly.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include <memory>
#include <string>

namespace mcx {

struct Setup;
struct LineSumArgs;

constexpr int kRefRounds = 20;   // maxIterateT (source/update_mod.f90:106-107)
constexpr int kMaxRounds = 64;   // T-iterations of the tightly converged balance

// alphaTotal of every (element, ion) pair of the mixed balance, tabulated in
// ln Te (1..1e7 K, kAlphaN nodes) and read by 4-point Lagrange; an interval
// where the reference's fits switch (a jump the interpolant cannot follow) is
// flagged at build time and evaluated directly
constexpr int kAlphaN = 4097;
constexpr double kAlphaLnT0 = 0., kAlphaLnT1 = 16.11809565095832;   // ln 1, ln 1e7

constexpr int kCoolNTe = 1280, kCoolNNe = 640;
constexpr double kCoolLnTe0 = 0.;                    // ln 1
constexpr double kCoolLnTe1 = 13.815510557964274;    // ln 1e6
constexpr double kCoolLnNe0 = -13.815510557964274;   // ln 1e-6
constexpr double kCoolLnNe1 = 20.723265836946411;    // ln 1e9

// One photoionised shell (elem, ion, shell) of an element that is on.
struct PhotoShell {
  int32_t elem, ion, shell;   // Z, stage, shell (1-based)
  int32_t ipNuP, highNuP;     // IPnuP, highNuP (1-based bins)
  int32_t xsecP;              // xSecArray pointer (1-based) of the shell (H/He: of the level)
  int32_t heavy;              // 1: getPhotoRates (elem > 2), 0: the H/He direct sum
  float yield1;               // auger(elem, ion, shell, 1)
};

struct BalanceCounters {
  unsigned long long noHit, noIonBal, noTeBal, converged, updated, maxIterT;
};

// A cell's place on the cooling surfaces (iT = -1: outside the grid).
struct CoolAt {
  int32_t iT, iN;
  float tT, tN;
};

// Device view (by value as a kernel parameter; pointers are device memory).
struct BalanceDev {
  int32_t nbins, nCells, nstages, nElemUsed, nShellsTot, nAtoms, nDiel, nAldro;
  int32_t lgBadnell, lgCompton;
  int32_t* list;               // [2][C+1] the cells of the current and the next T-iteration round
  unsigned int* listCount;     // [kMaxRounds+1] cells listed for each round
  int32_t cellReals;           // shared memory of one cell of the rates kernel, in values of the rate precision
  int32_t metaDoubles;         // its per-block element tables, in doubles
  int32_t ratesWarps[2];       // warps per block of the rates kernel (4 cells per warp), FP64 and mixed builds
  int32_t ratesGrid[2];        // its resident blocks on the GPU, the grid of the per-round launches
  int32_t smCount;
  int32_t augReals;            // mixed build: further shared memory per cell, in floats
  int32_t cellRealsMixed;      // mixed build: cellReals with one scratch row per ladder instead of three
  int32_t secIonP, cRecoilHP, cRecoilHeP;
  float xhiLimit;
  // T-iteration controls: the reference's (2 % residual, 1 % X(H0), X(He0),
  // X(He+) changes, 20 T-iterations, the 100 K step of a collapsed bracket),
  // or tight (converge = 1): residual 1e-9, X changes 1e-9 (mixed: 1e-6, 1e-5),
  // up to kMaxRounds T-iterations, a residual whose ladder has not converged
  // evaluated again at the same Te, Illinois-weighted regula falsi until the
  // bracket is 1e-12 wide, and unbracketed steps that start small (a converged
  // state stays on its branch of heating = cooling) and double up to x1.2
  int32_t converge, maxIterT;
  int32_t fixTe;               // 1: Te held (with converge = 1): the ladder converged at each cell's Te and
                               // heating - cooling left in resid; the evaluations of the balance's adjoint
  double resTol;
  double stepMin;              // tight mode: unbracketed steps 1 + stepMin 2^n at T-iteration n, at most 1.2
  float xTol;
  int32_t xref[31];            // elementXref by Z (index 1..30), 0 = off
  int32_t zOf[31];             // Z of used element e (1-based)
  float abun[31];              // elemAbun by Z
  int32_t pairShell0[31 * 32]; // [e-1][ion-1] first PhotoShell of (element e, ion), -1 none
  int32_t pairNShell[31 * 32];
  const float* nu;             // [nbins]
  const float* xsec;
  const float* xsecRecoil;     // [nbins]
  const PhotoShell* shells;    // [nShellsTot]
  const float* shellTail;      // [nShellsTot][2] sum of xs/(hc nu) and of xs above the secondary-ionisation threshold
  const float* CF;             // [30][30][5]
  const float* cionTherm;      // [30][30]
  const int32_t* nauger;       // [30][30][10]
  const float* auger;          // [30][30][10][10]
  const float* RRb;            // [6][30][31]
  const float* DRbC;           // [30][31][9]
  const float* DRbE;
  const float* rrec;           // [30][30][2]
  const float* rnew;           // [30][30][4]
  const float* diel;           // [nDiel][8]
  const float* aldro;          // [nAldro][6]
  const int16_t* dielRow;      // [31][32][3] by (Z, ion): last dielectronic row with flag 0|1, with 0|2; aldrovandi row
  const int32_t* outer;        // [30][30][3]
  const float4* chex;          // [31][32] charge-exchange a, b, c, d of (Z, ion), 0 where none
  const int32_t* atomHdr;      // [nAtoms][16]
  const double* atomData;
  const float* atomDataF;      // the same values in FP32 (mixed precision)
  const double* linePow;       // [nAtoms][kMaxLevels+1] sum over lines from level j of a(j,i) E_ji > 0
  const float* coolTab;        // [nAtoms][kCoolNNe][kCoolNTe] ln G, built before the first mixed balance
  const float* recTab;         // [nAtoms][kCoolNNe][kCoolNTe] B: the slope of forLines in ionDenUp with the
                               // recombination term (emission phase), built with coolTab
  CoolAt* coolAt;              // [C+1] the cell's stencil on the surfaces, set by the rates kernel
  const float* alphaTab;       // [nElemUsed * nstages][kAlphaN] ln alphaTotal (mixed balance), with coolTab
  const uint8_t* alphaJump;    // [nElemUsed * nstages][kAlphaN] 1: interval [i, i+1] evaluated directly
  // per-cell work, [k][C+1] (cell fastest)
  double* ion;                 // [nstages][nElemUsed]
  double* gam;                 // [nShellsTot] photoionisation rate (J integral; the rates kernel adds the reverse charge exchange to its copy)
  double* heatA;               // [nShellsTot] heating without the secondary-ionisation tail
  double* heatHi;              // [nShellsTot] tail heating, times heatef
  double* comp;                // [4] s1, s2, recoil H, recoil He
  double* te, *ne, *xOld;
  double* tHigh, *tLow, *resHigh, *resLow;
  double* heat;                // photoionisation heating
  double* coolA;               // coolFF + coolRec
  double* coolHex;             // H collisional excitation
  double* coolCollH;           // collisional ionisation cooling
  double* compHeat, *compRecoil, *compCool;   // Compton terms (times Ne where the reference multiplies)
  double* forSum;              // [nAtoms] forbidden-line cooling of each ion
  int32_t* nIterT;
  int8_t* state;               // 0 iterating, 1 done, 2 no photon hit
  int8_t* ibConv;
  int8_t* side;                // tight mode: bracket end replaced last (1 low, 2 high); 3 = the
                               // bracket closed on a discontinuity of heating - cooling
  double* resid;               // fixTe: heating - cooling at the held Te
  const uint8_t* evalMask;     // fixTe: 0 leaves the cell out of the evaluation (as if no photon reached
                               // it); null: every cell
  BalanceCounters* counters;
};

// Grid arrays the balance reads and writes (device memory).
struct BalanceGrid {
  const double* jste;          // [nbins][C+1], normalised
  const float* hden;           // [C+1]
  float* te, *ne, *ionDen;     // [C+1], [C+1], [nstages][nElemUsed][C+1]
  int32_t* converged, *black, *nIterT;   // [C+1]
};

class BalanceData {
 public:
  ~BalanceData();
  BalanceDev dev{};
  void* blocks[64] = {};
  int nBlocks = 0;
  // the whole balance (counters reset, J pass, 20 rounds, store) captured as
  // one CUDA graph per precision, replayed while the grid arrays stay put
  cudaGraphExec_t graph[2] = {nullptr, nullptr};
  BalanceGrid graphGrid[2] = {};
};

// Builds the device tables and the per-cell work arrays of a set-up.
std::string balanceDataCreate(const Setup& s, std::unique_ptr<BalanceData>& out);

constexpr int kBalFp64 = 0;    // FP64 throughout (the plain path)
constexpr int kBalMixed = 1;   // FP32 rates / splines / exponentials, FP64 solves and bracketing

// updateCell for every cell: up to maxRounds T-iterations (the reference's
// maxIterateT = 20).  Asynchronous on the stream; counters are left in
// BalanceDev::counters.
// atomSolves = 1: the mixed balance solves every ion's levels per cell and
// T-iteration instead of reading the cooling surfaces.
// fixTe = 1 (with converge = 1): every cell's Te is held; its ladder is
// converged at that Te and heating - cooling is left in BalanceDev::resid.
cudaError_t launchBalance(BalanceData& b, const BalanceGrid& g, int maxRounds, int precision, cudaStream_t s,
                          int atomSolves = 0, int converge = 0, int fixTe = 0);

// The forLines line total of every cell with compute[c] = 1 (the emission
// phase's normFor, rec = .true., units of 1e-25 erg/s per gas density) from
// the grid state.
cudaError_t launchForLinesEmission(BalanceData& b, const float* te, const float* ne, const float* ionDen,
                                   const uint8_t* compute, float* forLines, int precision, cudaStream_t s);

// outputGas forbidden-line level sums of every multi-level atom into the
// partial rows of `a` (FP64; the layout is described in k_lines.cuh).
cudaError_t launchForbLevelSums(BalanceData& b, const LineSumArgs& a, cudaStream_t s);

// Per-cell luminosities of requested forbidden lines (FP64, k_lines.cuh).
struct LineCellArgs;
cudaError_t launchLineCellLuminosities(BalanceData& b, const LineCellArgs& a, cudaStream_t s);

// Drops the captured balance graphs (after a change of the tables they bake in).
void invalidateBalanceGraphs(BalanceData& b);

}  // namespace mcx
