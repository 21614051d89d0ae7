// k_opacity.cu - per-cell opacity kappa(nu) for every active cell at once.
//
// Restates ionizationDriver / BoltGaunt / getGauntFF / eDenSum / addOpacity
// (source/ionization_mod.f90:26-477) as one kernel: a thread owns one cell
// and walks the frequency mesh, so that the store kappa[nu][cell] of a warp is
// one coalesced 128-byte row segment.  The bound-free terms are grouped per
// frequency bin in a CSR list (built once on the host in the reference's
// summation order: H, HeI, HeII, then element / ion / shell), every lane of a
// warp reads the same cross section (a broadcast) and its own ion density
// from shared memory.  Arithmetic is FP32 as in the reference.
// Behaviours of the reference kept here: the free-free prefactor has no H+ or
// He++ term (density(1,2) and density(2,3) are never filled,
// source/ionization_mod.f90:71-84), and an empty shell adds one term at bin 2
// (inOpacity's loop bound, source/ionization_mod.f90:451-476).
#include "k_opacity.cuh"

namespace mcx {

namespace {

__constant__ double kGauntD[88] = {
    8.986940175e+00, -4.009515855e+00, 8.808871266e-01, 2.640245111e-02, -4.580645915e-02, -3.568055702e-03,
    2.827798067e-03, 3.365860195e-04, -8.006936989e-01, 9.466021705e-01, 9.043402532e-02, -9.608451450e-02,
    -1.885629865e-02, 1.050313890e-02, 2.800889961e-03, -1.078209202e-03, -3.781305103e-01, 1.102726332e-01,
    -1.543619180e-02, 8.310561114e-03, 2.179620525e-02, 4.259726289e-03, -4.181588794e-03, -1.770208330e-03,
    1.877213132e-02, -1.004885705e-01, -5.483366378e-02, -4.520154409e-03, 8.366530426e-03, 3.700273930e-03,
    6.889320423e-04, 9.460313195e-05, 7.300158392e-02, 3.576785497e-03, -4.545307025e-03, -1.017965604e-02,
    -9.530211924e-03, -3.450186162e-03, 1.040482914e-03, 1.407073544e-03, -1.744671550e-03, 2.864013856e-02,
    1.903394837e-02, 7.091074494e-03, -9.668371391e-04, -2.999107465e-03, -1.820642230e-03, -3.874082085e-04,
    -1.707268366e-02, -4.694254776e-03, 1.311691517e-03, 5.316703136e-03, 5.178193095e-03, 2.451228935e-03,
    -2.277321615e-05, -8.182359057e-04, 2.567331664e-04, -9.155339970e-03, -6.997479192e-03, -3.571518641e-03,
    -2.096101038e-04, 1.553822487e-03, 1.509584686e-03, 6.212627837e-04, 4.098322531e-03, 1.635218463e-03,
    -5.918883504e-04, -2.333091048e-03, -2.484138313e-03, -1.359996060e-03, -5.371426147e-05, 5.553549563e-04,
    3.837562402e-05, 2.938325230e-03, 2.393747064e-03, 1.328839809e-03, 9.135013312e-05, -7.137252303e-04,
    -7.656848158e-04, -3.504683798e-04, -8.491991820e-04, -3.615327726e-04, 3.148015257e-04, 8.909207650e-04,
    9.869737522e-04, 6.134671184e-04, 1.068883394e-04, -2.046080100e-04};

}  // namespace

// Hummer (1988) Chebyshev fit: per-temperature coefficients c(1..8) and
// gamma^2 (getGauntFF, source/ionization_mod.f90:262-276).
__device__ void gauntCoeffs(float z, float log10Te, float c[9], float& con, float& gamma2) {
  float xlrkt;
  if (log10Te < 2.5f) xlrkt = 5.1983649f - 2.5f;
  else if (log10Te > 8.f) xlrkt = 5.1983649f - 8.f;
  else xlrkt = 5.1983649f - log10Te;
  float txg = 0.66666667f * (2.0f * z + xlrkt);
  gamma2 = exp10f(txg * 1.5f);
  con = 0.72727273f * xlrkt + 0.90909091f;
  float b[12];
  for (int j = 1; j <= 8; ++j) {
    int ir = 9;
    b[11] = (float)kGauntD[(j - 1) + 8 * 10];
    b[10] = txg * b[11] + (float)kGauntD[(j - 1) + 8 * 9];
    for (int i = 1; i <= 9; ++i) {
      b[ir] = txg * b[ir + 1] - b[ir + 2] + (float)kGauntD[(j - 1) + 8 * (ir - 1)];
      ir = ir - 1;
    }
    c[j] = 0.25f * (b[1] - b[3]);
  }
}

// getGauntFF frequency part (source/ionization_mod.f90:278-331)
__device__ float gauntAt(const float c[9], float con, float gamma2, float log10nu) {
  float txu = 0.72727273f * log10nu + con;
  float u = exp10f((txu - .90909091f) / .72727273f);
  if (fabsf(txu) <= 2.0f) {
    float b[9];
    int ir = 6;
    b[8] = c[8];
    b[7] = txu * b[8] + c[7];
    for (int j = 1; j <= 6; ++j) { b[ir] = txu * b[ir + 1] - b[ir + 2] + c[ir]; ir = ir - 1; }
    return b[1] - b[3];
  }
  float lu = log10f(u);
  if (lu < -4.0f && gamma2 < 0.3f) return 0.551329f * logf(2.24593f / u);
  if (lu < -4.0f && gamma2 >= 0.3f) return 0.551329f * logf(0.944931f / u / sqrtf(gamma2));
  if (txu > 2.0f) {
    float lg = log10f(gamma2);
    if (lg < -3.f) return sqrtf(0.9549297f / u);
    if (lg < 0.0f) {
      float slope = (sqrtf(12.f * gamma2 / u) - sqrtf(0.9549297f / u)) / 3.0f;
      return sqrtf(12.f * gamma2 / u) + slope * lg;
    }
    return fminf(1.05f, sqrtf(12.f * gamma2 / u));
  }
  return 0.f;
}

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
  for (int i = 1; i <= t.nbins; ++i) {
    const float nui = t.nu[i - 1];
    const float ex = Te1Ryd / Te + nui;
    const float boltz = ex > 84.f ? 0.f : expf(-ex);
    const float g = gauntAt(c, con, gamma2, t.log10nu[i - 1]);
    const float xb = t.xsec[i - 1 + t.bremsP0];
    float op = boltz < 0.995f ? xb * (1.f - boltz) * g * fac1 : xb * nui * g * fac2;
    const int e0 = t.csrStart[i - 1], e1 = t.csrStart[i];
    for (int e = e0; e < e1; ++e) {
      const int2 term = t.csrTerm[e];
      const int xi = i + term.x;   // 1-based index into xSecArray
      const float xs = (xi >= 1 && xi <= t.nXsec) ? t.xsec[xi - 1] : 0.f;
      op += xs * den[term.y * stride];
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
  const size_t smem = (size_t)t.nSlots * threads * sizeof(float);
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(opacityKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  opacityKernel<<<blocks, threads, smem, stream>>>(t, hden, te, ne, ionDen, gauntTe, compute, opacity);
  return cudaGetLastError();
}

}  // namespace mcx
