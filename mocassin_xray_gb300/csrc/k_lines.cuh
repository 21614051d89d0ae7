// k_lines.cuh - analytical line luminosities and ionic volume averages of
// outputGas (source/output_mod.f90:13-820) as per-warp partial sums.
//
// Every quantity outputGas integrates is a sum over the active cells with
// lgBlack < 1 of a per-cell value times Hden * dV.  Each warp takes 32
// consecutive cells of the range summed (group g = cells cellBase+32g+1 ..
// cellBase+32g+32: all cells, or one nebula of a batch), reduces every entry
// over its lanes with a fixed shuffle tree and writes one row of
// partial[group][entry]; a second kernel adds the rows in group order.  The
// sums are therefore the same from run to run.
//
// Entry layout (LineSumArgs):
//   0                              Hbeta: hydroLines(1,4,2)*Hden*dV where > 1e-35
//   hydroBase + 84 k + l           hydroVol of the k-th hydrogenic element, line l
//                                  (iup = 2..15, ilow = 1..min(8, iup-1), iup outer)
//   heiBase + l                    HeIVol, 34 lines (absent when He is off)
//   ionBase + 2 p, + 2 p + 1       TeVol numerator / denominator of the p-th
//                                  (element on, ion <= min(elem+1, nstages)) pair
//   forbBase[atom] + j - 1         sum of n_j * elemAbun * ionDen * 1.9865e9 * Hden * dV
//                                  for level j of the multi-level atom (the line
//                                  a(j,i) E_ji factors are applied on the host)
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace mcx {

struct EmissionDev;

constexpr int kHydroLinesPerElem = 84;

struct LineSumArgs {
  const float* te;          // [C+1]
  const float* ne;          // [C+1]
  const float* ionDen;      // [nstages][nElemUsed][C+1]
  const float* hden;        // [C+1]
  const double* vol;        // [C+1] getVolume in FP64
  const int32_t* black;     // [C+1] lgBlack
  double* partial;          // [nGroups][nEntries]
  const int32_t* forbBase;  // [nAtoms] device
  int32_t nCells, nGroups, nEntries;   // nCells: of the whole context (the arrays' C+1)
  int32_t cellBase, nRange;            // the cells summed: cellBase+1 .. cellBase+nRange
  int32_t nHydro, hydroBase, heiBase, ionBase, nIonElem;
  int32_t hydroIz[30];      // elements with hydrogenic lines, ascending
  int32_t ionElem[30];      // elements on, ascending
};

// Per-cell luminosity of requested forbidden lines (outputGas's forbVol terms
// before the sum over cells): out[k][cell] = fLineEm(lower, upper) * elemAbun
// * ionDen * 1.9865e9 * Hden * dV of line k, 0 where lgBlack >= 1.
struct LineCellArgs {
  const float* te;          // [C+1]
  const float* ne;          // [C+1]
  const float* ionDen;      // [nstages][nElemUsed][C+1]
  const float* hden;        // [C+1]
  const double* vol;        // [C+1]
  const int32_t* black;     // [C+1]
  const int32_t* req;       // [nReq][3] atom slot, lower level, upper level
  double* out;              // [nReq][C+1]
  int32_t nReq;
};

// The implicit-function adjoint of the converged balance at fixed J, one cell
// per thread (FP64).  From evaluations with every Te held, R = heating -
// cooling and L = the requested lines' luminosities, each at Te(1 +- h) and at
// a parameter stepped by +-h (each cell's Hden, or one abundance for all):
//   dR/dTe, dL/dTe, dR/dp, dL/dp   central differences (steps as stored),
//   dTe/dp = -(dR/dp) / (dR/dTe)   the root's response (0 where Te is held),
//   out[k][cell] = dL_k/dp + dL_k/dTe dTe/dp.
struct AdjointArgs {
  const double* rTp, *rTm;    // [C+1] R at Te(1+h), Te(1-h)
  const double* lTp, *lTm;    // [nL][C+1] L there
  const float* teP, *teM;     // [C+1] the held Te values
  const double* rPp, *rPm;    // [C+1] R at p(1+h), p(1-h)
  const double* lPp, *lPm;    // [nL][C+1]
  const float* pP, *pM;       // [C+1] the stepped per-cell parameter, or null: dpScalar
  double dpScalar;            // p(1+h) - p(1-h) of a parameter shared by all cells
  const uint8_t* hold;        // [C+1] 0 root, 1 Te held (no root), 2 no photon hit, 3 no converged balance
  double* dLdp;               // [nL][C+1] out
  double* dTdp;               // [C+1] out, or null
  unsigned long long* held;   // out: cells with hold = 0 whose dR/dTe or dR/dp is unusable (Te held), or null
  int32_t nCells, nL;
};

cudaError_t launchAdjointCombine(const AdjointArgs& a, cudaStream_t s);

// Shuffle-tree sum over the 32 lanes; lane 0 holds the result.
__device__ __forceinline__ double warpSumD(double v) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
  return v;
}

// Hbeta, hydrogenic and HeI recombination lines and the ionic Te/ionDen
// sums into partial rows (FP64).
cudaError_t launchGasLineSums(const EmissionDev& e, const LineSumArgs& a, cudaStream_t s);

// out[entry] = sum over groups of partial[group][entry], in group order.
cudaError_t launchLineSumReduce(const double* partial, int nGroups, int nEntries, double* out, cudaStream_t s);

}  // namespace mcx
