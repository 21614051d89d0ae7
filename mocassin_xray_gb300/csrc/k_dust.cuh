// k_dust.cuh - the grain phases of a dust-only grid on the device:
//   dust opacity   iterateMC's dust contribution to the opacity
//                  (source/iteration_mod.f90:194-246)
//   dust emission  setDustPDF (source/emission_mod.f90:1921-1986)
//   grain balance  getDustT (source/update_mod.f90:3346-3453) with
//                  updateCell's no-hit test and convergence flag (:104-265)
// FP32 like the reference's REAL arithmetic, one thread per cell (per
// (cell, frequency) for the opacity).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include <memory>
#include <string>

namespace mcx {

struct Setup;

struct DustCounters {
  unsigned long long noHit, converged, updated;
};

struct DustDev {
  int32_t nbins, nCells, nSpecies, nSizes;
  float xhiLimit;
  const float* nu;        // [nbins]
  const float* widFlx;    // [nbins]
  const float* Cabs;      // [nSpecies][nSizes][nbins]
  const float* Csca;
  const float* abun;      // [nSpecies]
  const float* tsub;      // [nSpecies]
  const float* weight;    // [nSizes]
  const float* emInt;     // [nSpecies][nSizes][nTemps]
  DustCounters* counters;
};

class DustData {
 public:
  ~DustData();
  DustDev dev{};
  void* blocks[16] = {};
  int nBlocks = 0;
};

std::string dustDataCreate(const Setup& s, std::unique_ptr<DustData>& out);

// scaOpac and absOpac of every cell from the grains below sublimation, and
// opacity += scaOpac + absOpac (the reference never resets a dust-only
// grid's opacity between iterations).
cudaError_t launchDustOpacity(const DustDev& d, const float* ndust, const float* tdust, float* opacity, float* scaOpac,
                              cudaStream_t s);

// The grain re-emission CDF dustPDF[nu][c] of every cell.
cudaError_t launchDustPDF(const DustDev& d, const float* tdust, float* dustPDF, cudaStream_t s);

// Grain radiative equilibrium of every cell hit by a photon; lgConverged from
// the change of the mean grain temperature Tdust(0,0) against XHILimit.
cudaError_t launchDustT(const DustDev& d, const double* jste, float* tdust, int32_t* converged, int32_t* black,
                        cudaStream_t s);

}  // namespace mcx
