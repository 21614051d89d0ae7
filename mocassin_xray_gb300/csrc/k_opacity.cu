// k_opacity.cu - per-cell opacity kappa(nu) for every active cell at once.
//
// Restates ionizationDriver / BoltGaunt / getGauntFF / eDenSum / addOpacity
// (source/ionization_mod.f90:26-477) as one kernel: a thread owns one cell
// and walks one chunk of the frequency mesh (blockIdx.y), so that the store
// kappa[nu][cell] of a warp is one coalesced 128-byte row segment and the
// chunks give the SMs enough warps to hide the table reads.  The bound-free
// terms are grouped per frequency bin in a CSR list (built once on the host
// in the reference's summation order: H, HeI, HeII, then element / ion /
// shell), every lane of a warp reads the same cross section (a broadcast) and
// its own ion density from shared memory.  Arithmetic is FP32 as in the reference.
// Behaviours of the reference kept here: the free-free prefactor has no H+ or
// He++ term (density(1,2) and density(2,3) are never filled,
// source/ionization_mod.f90:71-84), and an empty shell adds one term at bin 2
// (inOpacity's loop bound, source/ionization_mod.f90:451-476).
#include <algorithm>

#include "k_opacity.cuh"
#include "k_gaunt.cuh"

namespace mcx {

__global__ void __launch_bounds__(128)
opacityKernel(OpacityDev t, const float* __restrict__ hden, const float* __restrict__ te,
              const float* __restrict__ ne, const float* __restrict__ ionDen, const float* __restrict__ gauntTe,
              const uint8_t* __restrict__ compute, float* __restrict__ opacity) {
  extern __shared__ float sDen[];   // [nSlots][blockDim.x]
  const int cell = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const bool valid = cell <= t.nCells && compute[cell];
  const size_t C1 = (size_t)t.nCells + 1;
  float Te = 1.f, Ne = 0.f, fac1 = 0.f, c[9], con = 0.f, gamma2 = 0.f;
  if (valid) {
    Te = te[cell]; Ne = ne[cell];
    const float H = hden[cell];
    float wsum = 0.f;
    for (int s = 0; s < t.nSlots; ++s) {
      float d = ionDen[(size_t)cell + C1 * (size_t)t.slotPlane[s]] * t.slotAbun[s] * H;
      sDen[s * blockDim.x + threadIdx.x] = d;
      wsum += t.slotFFWeight[s] * d;
    }
    // addOpacity free-free prefactor (source/ionization_mod.f90:366-368)
    fac1 = (Ne / 1.e10f) * (wsum / 1.e10f) / sqrtf(Te);
    gauntCoeffs(0.f, log10f(gauntTe[cell]), c, con, gamma2);
  }
  if (!valid) return;
  const float Te1Ryd = 1.578866e5f;
  const float fac2 = fac1 * Te1Ryd / Te;
  const float* den = sDen + threadIdx.x;
  const int stride = blockDim.x;
  const int chunk = (t.nbins + gridDim.y - 1) / gridDim.y;
  const int i0 = 1 + blockIdx.y * chunk, i1 = min(t.nbins, i0 + chunk - 1);
  for (int i = i0; i <= i1; ++i) {
    const float nui = t.nu[i - 1];
    const float ex = Te1Ryd / Te + nui;
    const float boltz = ex > 84.f ? 0.f : expf(-ex);
    const float g = gauntAt(c, con, gamma2, t.log10nu[i - 1]);
    const float xb = t.xsec[i - 1 + t.bremsP0];
    float op = boltz < 0.995f ? xb * (1.f - boltz) * g * fac1 : xb * nui * g * fac2;
    const int e0 = t.csrStart[i - 1], e1 = t.csrStart[i];
    for (int e = e0; e < e1; ++e) {
      const int2 term = __ldg(t.csrTerm + e);
      op += __int_as_float(term.x) * den[term.y * stride];
    }
    if (t.lgCompton) op += t.KNsigmaT[i - 1] * Ne;
    opacity[(size_t)cell + C1 * (size_t)(i - 1)] = op;
  }
}

cudaError_t launchOpacity(const OpacityDev& t, const float* hden, const float* te, const float* ne,
                          const float* ionDen, const float* gauntTe, const uint8_t* compute, float* opacity,
                          cudaStream_t stream) {
  int threads = 128;
  while (threads > 32 && (size_t)t.nSlots * threads * sizeof(float) > 200 * 1024) threads >>= 1;
  if ((size_t)t.nSlots * threads * sizeof(float) > 200 * 1024) return cudaErrorInvalidValue;
  const int blocks = (t.nCells + threads - 1) / threads;
  // enough blocks for ~8 per SM of the 152, in mesh chunks of at least 32 bins
  const int chunks = std::max(1, std::min((8 * 152 + blocks - 1) / blocks, t.nbins / 32));
  const size_t smem = (size_t)t.nSlots * threads * sizeof(float);
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(opacityKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  opacityKernel<<<dim3(blocks, chunks), threads, smem, stream>>>(t, hden, te, ne, ionDen, gauntTe, compute, opacity);
  return cudaGetLastError();
}

}  // namespace mcx
