// k_opacity.cuh - device tables of the opacity kernel (see k_opacity.cu).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace mcx {

struct OpacityDev {
  int32_t nbins, nCells, nXsec, lgCompton, nSlots, bremsP0;
  const float* nu;            // [nbins]
  const float* log10nu;       // [nbins] log10(nuArray) as the reference's log10nuArray
  const float* xsec;          // [nXsec]
  const float* KNsigmaT;      // [nbins]
  const int32_t* csrStart;    // [nbins+1] bound-free terms of bin i in [csrStart[i-1], csrStart[i])
  const int2* csrTerm;        // {float bits of the cross section at the bin, ion slot}
  const int32_t* slotPlane;   // [nSlots] ionDen plane (xref-1) + nElemUsed*(ion-1)
  const float* slotAbun;      // [nSlots] elemAbun of the slot's element
  const float* slotFFWeight;  // [nSlots] weight of the slot in the free-free electron sum
};

cudaError_t launchOpacity(const OpacityDev& t, const float* hden, const float* te, const float* ne,
                          const float* ionDen, const float* gauntTe, const uint8_t* compute, float* opacity,
                          cudaStream_t stream);

}  // namespace mcx
