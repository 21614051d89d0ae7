// k_emission.cuh - per-cell emission phase: re-emission CDF and line fraction.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include <memory>
#include <string>

namespace mcx {

struct Setup;

// One heavy-ion free-bound term at one frequency bin.
struct FbTerm {
  float xsg;        // xSecArray(...) * g0/g1 of the ion at this bin
  float nuIP;       // nuArray(IPnuP) of the ion
  float abun;       // elemAbun of the element
  int32_t plane;    // ionDen plane (xref-1) + nElemUsed*(ion+1-1) of the recombining ion
};

// Device view of the emission tables (all pointers device memory).
constexpr int kEmChunksMax = 8;   // frequency chunks of the emission kernel

struct EmissionDev {
  int32_t nbins, nCells, nstages, nElemUsed, nTk, nlim[3], nHydroFiles;
  int32_t HIPnuP, HeIPnuP, HeIIPnuP, HeIlast, HeIIlast, j2TsP, HeIILymanP[4];
  int32_t xrefH, xrefHe;                 // elementXref of H and He (0 = off)
  float abunH, abunHe;
  float nuHIP, nuHeIP, nuHeIIP;
  const float* nu;            // [nbins]
  const float* cRydWid;       // [nbins] cRyd*widFlx/1e15
  const int16_t* pairIdx;     // [3][nbins] gamma-interpolation pair (1-based) covering the bin, 0 none
  const int32_t* edgeP;       // [3][32]
  const float* tk;            // [nTk]
  const float* logGamma;      // [3][nTk][32]
  const float* milne;         // [3][nbins] 4 pi xs statW hcRyd const nu^3 1e40 (0 where unused)
  float* ffK;                 // [2][nbins] 4 pi 54.43 Z^2 gauntFF(Z) (per phase); [nTables][2][nbins] in a batch
  const int16_t* ffIdx;       // [C+1] the Gaunt table of each cell in a batch (its nebula's), or null
  const int32_t* fbStart;     // [nbins+1]
  const FbTerm* fbTerm;
  const float* fbK;           // [nbins] 4 pi const hcRyd nu^3 1e40
  const float* twoPhH;        // [nbins] h y Ay(y) / A2q * 1e27 for HI (0 for nu >= nu0)
  const float* twoPhHeII;     // [nbins] the same for HeII
  const float* twoPhHeI;      // [nbins] Ay * 0.66262 * y / 51.3 for HeI
  const float* heiiLyman;     // [4] ratios
  const int32_t* hydroMap;    // [9][12]
  const float* hydroDens;     // [nFiles][13]
  const float* hydroLines;    // [nFiles][13][14][8]
  const float* hydroTemps;    // [12]
  const float* hbCoeff;       // [2][9][4]
  const float* rbEdge;        // [2][3][26]
  const float* r2aEdge;       // [3][18]
  const float* heiRec;        // [34][3][4]
  const int8_t* hydroOn;      // [31] izp computed (element on and nstages > izp)
  const int32_t* xrefAll;     // [30] elementXref
  const float* abunAll;       // [30] elemAbun
  float* part;                // [4][kEmChunksMax][C+1] per-chunk sums of the emission kernel's first pass
};

class EmissionData {
 public:
  ~EmissionData();
  EmissionDev dev{};
  void* blocks[32] = {};
  int nBlocks = 0;
};

// Builds and uploads the emission tables of a set-up; returns an error message or "".
std::string emissionDataCreate(const Setup& s, std::unique_ptr<EmissionData>& out);

// Tabulates 4 pi 54.43 Z^2 gauntFF(Z) at the Gaunt cache temperature (free_free).
cudaError_t launchEmissionGaunt(const EmissionDev& e, float gauntTe, cudaStream_t s);

// The same for the nebulae of a batch: table b of e.ffK at temps[b] (device array).
cudaError_t launchEmissionGauntBatched(const EmissionDev& e, const float* temps, int nTables, cudaStream_t s);

// emissionDriver for every cell with compute[c] = 1: writes recPDF[nu][c] and totalLines[c].
// chunked: the cumulative sums over frequency chunks with offsets (the mixed
// phase; the CDF then differs from the sequential FP32 sum by rounding); else
// one sequential sum per cell, operation for operation the reference's.
cudaError_t launchEmission(const EmissionDev& e, const float* te, const float* ne, const float* ionDen,
                           const uint8_t* compute, const float* forLines, float* recPDF, float* totalLines,
                           bool chunked, cudaStream_t s);

}  // namespace mcx
