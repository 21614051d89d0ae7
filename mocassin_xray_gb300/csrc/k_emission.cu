// k_emission.cu - the emission phase for every gas cell at once.
//
// Restates emissionDriver / fb_ff / twoPhoton / RecLinesEmission /
// setDiffusePDF (source/emission_mod.f90:36-252, :336-1151, :1528-1919) for gas
// without dust.  One thread owns one cell and walks the frequency mesh, so the
// store recPDF[nu][cell] of a warp is one coalesced row segment; the cumulative
// sum is taken in the reference's order and precision (REAL partial sums).
// Everything that depends only on the frequency mesh (Milne-relation
// prefactors, heavy-ion cross sections times g0/g1, two-photon spectral shapes,
// the gamma-edge pair covering each bin) is tabulated once on the host in FP64
// and stored in FP32, so the per-cell work is FP32 exponentials and FMAs.
#include "k_emission.cuh"

#include <algorithm>
#include "k_gaunt.cuh"
#include "setup_internal.h"

#include <cmath>
#include <vector>

namespace mcx {

namespace {

constexpr double kPi = 3.141592654;
constexpr double kHcRyd_k = 157893.94, kHcRyd = 2.1799153e-11, kCRyd = 3.2898423e15, kHPlanck = 6.6262e-27;

template <typename T>
cudaError_t up(EmissionData& d, const std::vector<T>& v, const T** out) {
  void* p = nullptr;
  size_t n = v.empty() ? sizeof(T) : v.size() * sizeof(T);
  cudaError_t e = cudaMalloc(&p, n);
  if (e != cudaSuccess) return e;
  d.blocks[d.nBlocks++] = p;
  if (!v.empty()) e = cudaMemcpy(p, v.data(), n, cudaMemcpyHostToDevice);
  *out = static_cast<const T*>(p);
  return e;
}

}  // namespace

EmissionData::~EmissionData() {
  for (int i = 0; i < nBlocks; ++i) cudaFree(blocks[i]);
}

std::string emissionDataCreate(const Setup& s, std::unique_ptr<EmissionData>& out) {
  auto d = std::make_unique<EmissionData>();
  EmissionDev& e = d->dev;
  const EmissionTables& em = s.em;
  const int nb = s.nbins;
  const int E = std::max(s.nElemUsed, 1);
  e.nbins = nb; e.nCells = s.nCells; e.nstages = s.p.nstages; e.nElemUsed = E; e.nTk = em.nTk;
  for (int k = 0; k < 3; ++k) e.nlim[k] = em.nlim[k];
  e.nHydroFiles = em.nHydroFiles;
  e.HIPnuP = s.HlevNuP[0]; e.HeIPnuP = s.HeIlevNuP[0]; e.HeIIPnuP = s.HeIIlevNuP[0];
  const int HeIlast = em.edgeP[32 + em.nlim[1] - 1], HeIIlast = em.edgeP[64 + em.nlim[2] - 1];
  e.HeIlast = std::max(e.HIPnuP, HeIlast);                 // Milne HeI from here
  e.HeIIlast = std::max(e.HeIlast, HeIIlast);              // Milne HeII from here
  e.j2TsP = em.j2TsP;
  for (int k = 0; k < 4; ++k) e.HeIILymanP[k] = em.HeIILymanP[k];
  e.xrefH = s.elemXref[0]; e.xrefHe = s.elemXref[1];
  e.abunH = s.elemAbun[0]; e.abunHe = s.elemAbun[1];
  e.nuHIP = s.nu[e.HIPnuP - 1]; e.nuHeIP = s.nu[e.HeIPnuP - 1]; e.nuHeIIP = s.nu[e.HeIIPnuP - 1];

  std::vector<float> cw(nb), milne((size_t)3 * nb, 0.f), fbK(nb), t2H(nb, 0.f), t2HeII(nb, 0.f), t2HeI(nb, 0.f);
  std::vector<int16_t> pair((size_t)3 * nb, 0);
  for (int k = 0; k < 3; ++k)
    for (int p = 1; p <= em.nlim[k] / 2; ++p) {
      int iup = em.edgeP[k * 32 + 2 * p - 1], ilow = em.edgeP[k * 32 + 2 * p - 2];
      if (iup == ilow) return "fb_ff: frequency grid too coarse - divide by zero";
      for (int j = ilow; j <= iup - 1; ++j) pair[(size_t)k * nb + (j - 1)] = (int16_t)p;
    }
  const double constant = 4.9874105e-6;
  auto xsAt = [&](int xi) -> double { return (xi >= 1 && xi <= (int)s.xSec.size()) ? (double)s.xSec[xi - 1] : 0.; };
  for (int i = 1; i <= nb; ++i) {
    const double v = s.nu[i - 1], v3 = v * v * v;
    cw[i - 1] = (float)(kCRyd * (double)s.widFlx[i - 1] / 1.e15);
    fbK[i - 1] = (float)(4. * kPi * constant * kHcRyd * v3 * 1e20 * 1e20);
    if (i >= e.HIPnuP)
      milne[i - 1] = (float)(4. * kPi * xsAt(i - e.HIPnuP + 1 + s.HlevXSecP[0] - 1) * 2. * kHcRyd * constant * v3 * 1e20 * 1e20);
    if (i >= e.HeIlast)
      milne[nb + i - 1] = (float)(4. * kPi * xsAt(i - e.HeIPnuP + 1 + s.HeISingXSecP[0] - 1) * 0.5 * kHcRyd * constant * v3 * 1e20 * 1e20);
    if (i >= e.HeIIlast)
      milne[2 * nb + i - 1] = (float)(4. * kPi * xsAt(i - e.HeIIPnuP + 1 + s.HeIIXSecP[0] - 1) * 2. * kHcRyd * constant * v3 * 1e20 * 1e20);
    // hydro2phot spectral shapes (source/emission_mod.f90:660-726)
    if (v < 0.7496) {
      double y = v / 0.7496;
      double Ay = 202.0 * (y * (1 - y) * (1 - pow(4 * y * (1 - y), 0.8)) + 0.88 * pow(y * (1 - y), 1.53) * pow(4 * y * (1 - y), 0.8));
      t2H[i - 1] = (float)(kHPlanck * y * Ay / 8.2249 * 1e27);
    }
    if (v < 3.0) {
      double y = v / 3.0;
      double Ay = 64. * 0.9994667 * 202.0 * (y * (1 - y) * (1 - pow(4 * y * (1 - y), 0.8)) + 0.88 * pow(y * (1 - y), 1.53) * pow(4 * y * (1 - y), 0.8));
      t2HeII[i - 1] = (float)(kHPlanck * y * Ay / (8.226 * 64.) * 1e27);
    }
  }
  {  // HeI2photSub's table walk (source/emission_mod.f90:762-778), cell independent
    int j = 1;
    for (int i = 1; i <= nb; ++i) {
      double y = (double)s.nu[i - 1] / 1.514;
      if (y > (double)em.HeI2phot[0][j - 1]) j = j + 1;
      if (j >= 41) break;
      double fit1 = ((double)em.HeI2phot[1][j] - (double)em.HeI2phot[1][j - 1]) / ((double)em.HeI2phot[0][j] - (double)em.HeI2phot[0][j - 1]);
      double fit2 = (double)em.HeI2phot[1][j - 1] - (double)em.HeI2phot[0][j - 1] * fit1;
      double Ay = fit1 * y + fit2;
      if (Ay < 9.2163086E-03) Ay = 0.;
      t2HeI[i - 1] = (float)(Ay * 0.66262 * y / 51.3);
    }
  }
  // heavy free-bound CSR in the reference's summation order (element, ion)
  std::vector<int32_t> fbStart(nb + 1, 0);
  std::vector<FbTerm> fbTerm;
  const size_t nt = em.fbHeavy.size() / 7;
  for (int i = 1; i <= nb; ++i) {
    fbStart[i - 1] = (int32_t)fbTerm.size();
    for (size_t t = 0; t < nt; ++t) {
      const int32_t* T = &em.fbHeavy[7 * t];
      int elem = T[0], ion = T[1], IPnuP = T[2], highNuP = T[3], xSecP = T[4], g0 = T[5], g1 = T[6];
      if (i >= IPnuP && i < highNuP) {
        FbTerm f;
        f.xsg = (float)(xsAt(i + xSecP - IPnuP + 1 - 1) * ((double)g0 / (double)g1));
        f.nuIP = s.nu[IPnuP - 1];
        f.abun = s.elemAbun[elem - 1];
        f.plane = (s.elemXref[elem - 1] - 1) + E * ion;   // stage ion+1
        fbTerm.push_back(f);
      }
    }
  }
  fbStart[nb] = (int32_t)fbTerm.size();
  std::vector<int32_t> xrefAll(s.elemXref, s.elemXref + kNElements);
  std::vector<float> abunAll(s.elemAbun, s.elemAbun + kNElements);
  std::vector<int8_t> hOn(31, 0);
  for (int izp = 1; izp <= 30; ++izp) hOn[izp] = (s.elemOn[izp - 1] && s.p.nstages > izp) ? 1 : 0;
  std::vector<float> ffK((size_t)2 * nb, 0.f);
  std::vector<float> hb(72), rb(156), r2a(54), heiRec(408), ly(4), temps(12);
  for (int a = 0; a < 2; ++a) for (int i = 0; i < 9; ++i) for (int j = 0; j < 4; ++j) hb[(a * 9 + i) * 4 + j] = em.HbCoeff[a][i][j];
  for (int a = 0; a < 2; ++a) for (int j = 0; j < 3; ++j) for (int i = 0; i < 26; ++i) rb[(a * 3 + j) * 26 + i] = em.rbEdge[a][j][i];
  for (int j = 0; j < 3; ++j) for (int i = 0; i < 18; ++i) r2a[j * 18 + i] = em.r2aEdge[j][i];
  for (int l = 0; l < 34; ++l) for (int d2 = 0; d2 < 3; ++d2) for (int k = 0; k < 4; ++k) heiRec[(l * 3 + d2) * 4 + k] = em.HeIrec[l][d2][k];
  for (int k = 0; k < 4; ++k) ly[k] = em.HeIILyman[0][k];
  for (int k = 0; k < 12; ++k) temps[k] = em.hydroLinesTemps[k];

  cudaError_t err = cudaSuccess;
#define UP(vec, field) if (err == cudaSuccess) err = up(*d, vec, &e.field)
  UP(s.nu, nu); UP(cw, cRydWid); UP(pair, pairIdx); UP(em.edgeP, edgeP); UP(em.tk, tk); UP(em.logGamma, logGamma);
  UP(milne, milne); UP(fbStart, fbStart); UP(fbTerm, fbTerm); UP(fbK, fbK); UP(t2H, twoPhH); UP(t2HeII, twoPhHeII);
  UP(t2HeI, twoPhHeI); UP(ly, heiiLyman); UP(em.hydroFileMap, hydroMap); UP(em.hydroDens, hydroDens);
  UP(em.hydroLines, hydroLines); UP(temps, hydroTemps); UP(hb, hbCoeff); UP(rb, rbEdge); UP(r2a, r2aEdge);
  UP(heiRec, heiRec); UP(hOn, hydroOn); UP(xrefAll, xrefAll); UP(abunAll, abunAll);
#undef UP
  if (err == cudaSuccess) {
    const float* fk = nullptr;
    err = up(*d, ffK, &fk);
    e.ffK = const_cast<float*>(fk);
  }
  if (err == cudaSuccess) {
    const float* pp = nullptr;
    err = up(*d, std::vector<float>((size_t)4 * kEmChunksMax * ((size_t)s.nCells + 1), 0.f), &pp);
    e.part = const_cast<float*>(pp);
  }
  if (err != cudaSuccess) return std::string("emission tables: ") + cudaGetErrorString(err);
  out = std::move(d);
  return "";
}

__global__ void emissionGauntKernel(EmissionDev e, float gauntTe) {
  float c0[9], con0, g20, c1[9], con1, g21;
  gauntCoeffs(0.f, log10f(gauntTe), c0, con0, g20);
  gauntCoeffs(0.30103f, log10f(gauntTe), c1, con1, g21);
  const float k = 4.f * 3.141592654f * 54.43f;
  for (int i = threadIdx.x + blockIdx.x * blockDim.x; i < e.nbins; i += blockDim.x * gridDim.x) {
    float l = log10f(e.nu[i]);
    e.ffK[i] = k * 1.f * gauntAt(c0, con0, g20, l);
    e.ffK[e.nbins + i] = k * 4.f * gauntAt(c1, con1, g21, l);
  }
}

cudaError_t launchEmissionGaunt(const EmissionDev& e, float gauntTe, cudaStream_t s) {
  emissionGauntKernel<<<(e.nbins + 255) / 256, 256, 0, s>>>(e, gauntTe);
  return cudaGetLastError();
}

// one table per nebula of a batch: table b (blockIdx.y) at temperature temps[b]
__global__ void emissionGauntBatchKernel(EmissionDev e, const float* __restrict__ temps) {
  const int b = blockIdx.y;
  float c0[9], con0, g20, c1[9], con1, g21;
  gauntCoeffs(0.f, log10f(temps[b]), c0, con0, g20);
  gauntCoeffs(0.30103f, log10f(temps[b]), c1, con1, g21);
  const float k = 4.f * 3.141592654f * 54.43f;
  float* ffK = e.ffK + (size_t)b * 2 * e.nbins;
  for (int i = threadIdx.x + blockIdx.x * blockDim.x; i < e.nbins; i += blockDim.x * gridDim.x) {
    float l = log10f(e.nu[i]);
    ffK[i] = k * 1.f * gauntAt(c0, con0, g20, l);
    ffK[e.nbins + i] = k * 4.f * gauntAt(c1, con1, g21, l);
  }
}

cudaError_t launchEmissionGauntBatched(const EmissionDev& e, const float* temps, int nTables, cudaStream_t s) {
  if (nTables <= 0) return cudaSuccess;
  emissionGauntBatchKernel<<<dim3((e.nbins + 255) / 256, nTables), 256, 0, s>>>(e, temps);
  return cudaGetLastError();
}

namespace {

__device__ __forceinline__ float ionFrac(const float* ionDen, size_t C1, size_t cell, int xref, int E, int stage,
                                         int nstages) {
  if (xref <= 0 || stage < 1 || stage > nstages) return 0.f;
  return ionDen[cell + C1 * (size_t)((xref - 1) + E * (stage - 1))];
}

// locate on an ascending float array (source/interpolation_mod.f90:49-106)
__device__ __forceinline__ int locateF(const float* xa, int n, float x) {
  if (x > xa[n - 1]) return n;
  if (x < xa[0]) return 0;
  int jlow = 0, jup = n + 1;
  for (int it = 0; it < 64; ++it) {
    if (jup - jlow < 1) break;
    int jm = (jup + jlow) >> 1;
    if (xa[jm - 1] == x) return jm;
    if (x > xa[jm - 1]) { if (jlow == jm) break; jlow = jm; } else jup = jm;
  }
  return jlow;
}

}  // namespace

// Two passes.  mode 1, grid (cells, chunks): the frequency mesh in nChunks
// contiguous chunks, each chunk's cumulative sums from 0 into recPDF and its
// totals (the chunk's sum and its HI, HeI, HeII parts) into part[4][nChunks][C+1];
// enough independent chunks per cell keep the SMs busy.  mode 2, one thread per
// cell: the chunk offsets added and the distribution normalised, then the
// recombination lines and totalLines.
__global__ void __launch_bounds__(128)
emissionKernel(EmissionDev e, const float* __restrict__ te, const float* __restrict__ ne,
               const float* __restrict__ ionDen, const uint8_t* __restrict__ compute,
               const float* __restrict__ forLines, float* __restrict__ recPDF, float* __restrict__ totalLines,
               float* __restrict__ part, int nChunks, int mode) {
  const int cell = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (cell > e.nCells || !compute[cell]) return;
  const size_t C1 = (size_t)e.nCells + 1;
  const int nb = e.nbins, E = e.nElemUsed, S = e.nstages;
  const float* ffK = e.ffK + (e.ffIdx ? (size_t)e.ffIdx[cell] * 2 * (size_t)nb : (size_t)0);
  const float Te = te[cell], NeCell = ne[cell];
  float Ne = NeCell;
  const float sqrTe = sqrtf(Te), log10Te = log10f(Te), log10Ne = log10f(Ne);
  if (Ne < 1.e-5f) Ne = 1.e-5f;
  const float invTe15 = 1.f / (Te * sqrTe);
  const float hk = 157893.94f / Te;

  // gamma(T) interpolation in log-log (fb_ff, source/emission_mod.f90:388-424)
  int nT = 0;
  float tfac = 0.f, tden = 1.f;
  int tmode;   // 0 below, 1 above, 2 interpolate
  if (Te <= e.tk[0]) tmode = 0;
  else if (Te >= e.tk[e.nTk - 1]) tmode = 1;
  else { tmode = 2; nT = locateF(e.tk, e.nTk, Te); tfac = log10f(Te / e.tk[nT - 1]); tden = log10f(e.tk[nT] / e.tk[nT - 1]); }
  auto logG = [&](int k, int idx1) -> float {   // 1-based edge index
    const float* lg = e.logGamma + (size_t)k * e.nTk * 32;
    if (tmode == 0) return lg[idx1 - 1];
    if (tmode == 1) return lg[(size_t)(e.nTk - 1) * 32 + idx1 - 1];
    float a = lg[(size_t)(nT - 1) * 32 + idx1 - 1], b = lg[(size_t)nT * 32 + idx1 - 1];
    return a + (b - a) / tden * tfac;
  };

  // two-photon temperature/density factors (hydro2phot, HeI2photSub)
  float Q;
  if (Te <= 10000.f) Q = 5.31e-4f;
  else if (Te >= 20000.f) Q = 4.71e-4f;
  else Q = exp10f(log10f(5.31e-4f) + (log10f(4.71e-4f / 5.31e-4f) / log10f(2.f)) * log10f(Te / 10000.f));
  const float fH2 = 0.8368f * powf(Te * 1.e-4f, -0.723f) / (1.f + (Ne * Q) / 8.23f);
  float aHeII;
  if (Te <= 5000.f) aHeII = 6.161f;
  else if (Te >= 30000.f) aHeII = 2.035f;
  else if (Te <= 10000.f) aHeII = exp10f(log10f(6.161f) + log10f(4.091f / 6.161f) / log10f(2.f) * log10f(Te / 5000.f));
  else if (Te <= 15000.f) aHeII = exp10f(log10f(4.091f) + log10f(3.189f / 4.091f) / log10f(1.5f) * log10f(Te / 10000.f));
  else aHeII = exp10f(log10f(3.189f) + log10f(2.035f / 3.189f) / log10f(2.f) * log10f(Te / 15000.f));
  const float aHeI = 6.23f * powf(Te / 10000.f, -0.827f);

  const float xH2 = ionFrac(ionDen, C1, cell, e.xrefH, E, 2, S);
  const float xHe2 = ionFrac(ionDen, C1, cell, e.xrefHe, E, 2, S);
  const float xHe3 = ionFrac(ionDen, C1, cell, e.xrefHe, E, 3, S);
  const float wH = e.abunH * xH2 * Ne, wHe2 = e.abunHe * xHe2 * Ne, wHe3 = e.abunHe * xHe3 * Ne;

  // lines added to the partial sums of setDiffusePDF (source/emission_mod.f90:1617-1668)
  const float T4 = Te * 1.e-4f;
  const float corrHeI = 27.2f * powf(T4, -0.678f) * Ne * e.abunHe * xHe2 * 1.45673f * 2.1799153e-11f * 1e11f;
  const float lyA = exp10f(-0.792f * log10Te + 6.01f) * Ne * xHe3 * e.abunHe;

  float normHI = 0.f, normHeI = 0.f, normHeII = 0.f, cum = 0.f;
  const int chunkLen = (nb + nChunks - 1) / nChunks;
  if (mode == 1) {
  const int q = blockIdx.y;
  const int i0 = 1 + q * chunkLen, i1 = min(nb, (q + 1) * chunkLen);
  int gP[3] = {0, 0, 0};
  float gL2[3] = {0.f, 0.f, 0.f}, gA[3] = {0.f, 0.f, 0.f}, gNu[3] = {0.f, 0.f, 0.f};
  for (int i = i0; i <= i1; ++i) {
    const float v = e.nu[i - 1];
    float gHI = 0.f, gHeI = 0.f, gHeII = 0.f;
    float g[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      int p = e.pairIdx[(size_t)k * nb + (i - 1)];
      if (p > 0) {
        if (p != gP[k]) {   // a new edge pair: its fit, kept for the following bins of the pair
          int iup = e.edgeP[k * 32 + 2 * p - 1], ilow = e.edgeP[k * 32 + 2 * p - 2];
          float l2 = logG(k, 2 * p), l1 = logG(k, 2 * p - 1);
          gP[k] = p;
          gL2[k] = l2;
          gA[k] = (l2 - l1) / (e.nu[iup - 1] - e.nu[ilow - 1]);
          gNu[k] = e.nu[iup - 1];
        }
        g[k] = exp10f(gL2[k] + gA[k] * (v - gNu[k]));
      }
    }
    gHI = g[0]; gHeI = g[1]; gHeII = g[2];
    const float exff = expf(-v * hk) / sqrTe;
    if (i >= e.HIPnuP) {
      gHI = e.milne[i - 1] * invTe15 * expf((e.nuHIP - v) * hk) + ffK[i - 1] * exff;
      if (i >= e.HeIlast) {
        gHeI = e.milne[nb + i - 1] * invTe15 * expf((e.nuHeIP - v) * hk) + ffK[i - 1] * exff;
        if (i >= e.HeIIlast) gHeII = e.milne[2 * nb + i - 1] * invTe15 * expf((e.nuHeIIP - v) * hk) + ffK[nb + i - 1] * exff;
      }
    }
    float hv = 0.f;
    for (int t = e.fbStart[i - 1]; t < e.fbStart[i]; ++t) {
      const FbTerm f = e.fbTerm[t];
      hv += expf((f.nuIP - v) * hk) * f.xsg * ionDen[(size_t)cell + C1 * (size_t)f.plane] * f.abun;
    }
    hv = hv * e.fbK[i - 1] * invTe15;
    float eHI = (gHI + e.twoPhH[i - 1] * fH2) * wH + hv * Ne;
    float eHeI = (gHeI + e.twoPhHeI[i - 1] * aHeI) * wHe2;
    float eHeII = (gHeII + e.twoPhHeII[i - 1] * aHeII) * wHe3;
    if (eHI < 1.e-15f) eHI = 0.f;
    if (eHeI < 1.e-15f) eHeI = 0.f;
    if (eHeII < 1.e-15f) eHeII = 0.f;
    const float cw = e.cRydWid[i - 1];
    float sHI = cw * eHI, sHeI = cw * eHeI, sHeII = cw * eHeII;
    normHI += sHI; normHeI += sHeI; normHeII += sHeII;
    if (i == e.j2TsP) sHeI += corrHeI;
#pragma unroll
    for (int k = 0; k < 4; ++k)
      if (i == e.HeIILymanP[k]) sHeII += (k == 3) ? lyA : e.heiiLyman[k] * lyA;
    cum = cum + (sHI + sHeI + sHeII);
    recPDF[(size_t)cell + C1 * (size_t)(i - 1)] = cum;
  }
  part[((size_t)0 * nChunks + q) * C1 + cell] = cum;
  part[((size_t)1 * nChunks + q) * C1 + cell] = normHI;
  part[((size_t)2 * nChunks + q) * C1 + cell] = normHeI;
  part[((size_t)3 * nChunks + q) * C1 + cell] = normHeII;
  return;
  }
  // mode 2: the chunks' offsets and the norms in chunk order
  float off[kEmChunksMax];
  for (int q = 0; q < nChunks; ++q) {
    off[q] = cum;
    cum = cum + part[((size_t)0 * nChunks + q) * C1 + cell];
    normHI += part[((size_t)1 * nChunks + q) * C1 + cell];
    normHeI += part[((size_t)2 * nChunks + q) * C1 + cell];
    normHeII += part[((size_t)3 * nChunks + q) * C1 + cell];
  }
  normHeI += corrHeI;
  normHeII += lyA * (1.f + e.heiiLyman[0] + e.heiiLyman[1] + e.heiiLyman[2]);

  // RecLinesEmission: hydrogenic recombination lines (source/emission_mod.f90:878-1085)
  float normRec = 0.f;
  const int elUp = (T4 > e.hydroTemps[11]) ? 2 : 8;
  for (int izp = 1; izp <= 30; ++izp) {
    if (!e.hydroOn[izp]) continue;
    const bool direct = izp <= elUp;
    const int row = direct ? izp : 2;
    const float scale = direct ? 1.f : 4.f / (float)(izp * izp);
    const float T4u = T4 * scale, Neu = Ne * scale;
    const float log10Neu = direct ? log10Ne : log10f(Ne * scale);
    int itemp = 1;
    for (int k = 1; k <= 12; ++k) if (T4u > e.hydroTemps[k - 1]) itemp = k;
    if (itemp < 12 && T4u > (e.hydroTemps[itemp] + e.hydroTemps[itemp - 1]) / 2.f) itemp = itemp + 1;
    const int f = e.hydroMap[(row - 1) * 12 + (itemp - 1)];
    const float* dens = e.hydroDens + (size_t)f * 13;
    const float* L = e.hydroLines + (size_t)f * 13 * 14 * 8;
    int idenp = 1;
    for (int k = 1; k <= 13; ++k) if (Neu > dens[k - 1] && dens[k - 1] > 0.f) idenp = k;
    const bool interp = (dens[12] > 0.f && idenp < 13) || (dens[12] == 0.f && idenp < 9);
    float sumL = 0.f;
    const float w = interp ? (Neu - dens[idenp - 1]) / (dens[idenp] - dens[idenp - 1]) : 0.f;
    for (int iup = 2; iup <= 15; ++iup)
      for (int ilow = 1; ilow <= (iup - 1 < 8 ? iup - 1 : 8); ++ilow) {
        float a = L[(((size_t)idenp - 1) * 14 + (iup - 2)) * 8 + (ilow - 1)];
        float vline = a;
        if (interp) vline = a + (L[(((size_t)idenp) * 14 + (iup - 2)) * 8 + (ilow - 1)] - a) * w;
        sumL += vline;
      }
    float Hbeta;
    const float* HbA = e.hbCoeff + (size_t)(row - 1) * 4;
    const float* HbB = e.hbCoeff + 36 + (size_t)(row - 1) * 4;
    if (direct) {
      if ((izp == 1 && T4 <= 3.f) || (izp > 1 && T4 <= e.hydroTemps[11])) {
        float zfit = (log10Ne - HbA[1]) / HbA[2];
        float Afit = HbA[0] * expf(-zfit * zfit / 2.f) + HbA[3];
        zfit = (log10Ne - HbB[1]) / HbB[2];
        float Bfit = HbB[0] * expf(-zfit * zfit / 2.f) + HbB[3];
        Hbeta = exp10f(Afit + Bfit * log10Te);
      } else {
        float yy1, yy2, x1, x2;
        const float wN = (idenp < 13) ? (Ne - dens[idenp - 1]) / (dens[idenp] - dens[idenp - 1]) : 0.f;
        if (izp == 1) {
          const float* e3 = e.rbEdge + 2 * 26;
          yy1 = e3[idenp - 1] + ((idenp < 13) ? (e3[idenp - 1] - e3[idenp]) * wN : 0.f);
          yy2 = e3[12 + idenp] + ((idenp < 13) ? (e3[12 + idenp] - e3[13 + idenp]) * wN : 0.f);
          x1 = e.rbEdge[0]; x2 = e.rbEdge[13];
        } else {
          const float* e3 = e.r2aEdge + 2 * 18;
          yy1 = e3[idenp - 1] + ((idenp < 13) ? (e3[idenp - 1] - e3[idenp]) * wN : 0.f);
          // r2aEdge(3, 9+idenp+1) lies past the table for idenp = 9: read as r2aEdge(3,18)
          yy2 = e3[8 + idenp] + ((idenp < 13) ? (e3[8 + idenp] - e3[9 + idenp < 18 ? 9 + idenp : 17]) * wN : 0.f);
          x1 = e.r2aEdge[0]; x2 = e.r2aEdge[9];
        }
        const float xx = log10f(T4 * 1.e4f);
        Hbeta = exp10f(yy1 - (yy1 - yy2) * (xx - x1) / (x2 - x1));
      }
    } else {
      const float log10TeZ = log10f(Te * scale);
      float zfit = (log10Neu - HbA[1]) / HbA[2];
      float Afit = HbA[0] * expf(-zfit * zfit / 2.f) + HbA[3];
      zfit = (log10Neu - HbB[1]) / HbB[2];
      float Bfit = HbB[0] * expf(-zfit * zfit / 2.f) + HbB[3];
      Hbeta = ((float)(izp * izp * izp) / 8.f) * exp10f(Afit + Bfit * log10TeZ);
    }
    const float xion = ionFrac(ionDen, C1, cell, e.xrefAll[izp - 1], E, izp + 1, S);
    Hbeta = Hbeta * Ne * xion * e.abunAll[izp - 1];
    normRec += sumL * Hbeta;
  }
  // HeI recombination lines (source/emission_mod.f90:1100-1146)
  {
    float T4h = T4;
    if (T4h < 0.5f) T4h = 0.5f;
    if (T4h < 2.0f) T4h = 2.0f;
    int denint;
    if (NeCell <= 100.f) denint = 0;
    else if (NeCell <= 1.e4f) denint = 1;
    else if (NeCell <= 1.e6f) denint = 2;
    else denint = 3;
    const float scaleHe = Ne * e.abunHe * xHe2;
    for (int l = 0; l < 34; ++l) {
      const float* C0 = e.heiRec + (size_t)l * 12;
      float r;
      if (denint > 0 && denint < 3) {
        const float* a = C0 + (denint - 1) * 4;
        const float* b = C0 + denint * 4;
        float x1 = a[0] * powf(T4h, a[1]) * expf(a[2] / T4h);
        float x2 = b[0] * powf(T4h, b[1]) * expf(b[2] / T4h);
        float p0 = exp10f(2.f * (float)denint), p1 = exp10f(2.f * (float)(denint + 1));
        r = x1 + ((x2 - x1) * (Ne - p0) / (p1 - p0));
      } else {
        const float* a = C0 + (denint == 0 ? 0 : 2) * 4;
        r = a[0] * powf(T4h, a[1]) * expf(a[2] / T4h);
      }
      normRec += r * scaleHe;
    }
  }
  const float tl = normRec + (forLines ? forLines[cell] : 0.f);

  // normalise the cumulative distribution (source/emission_mod.f90:1880-1884),
  // each chunk's entries shifted by the chunk's offset first
  const float last = off[(nb - 1) / chunkLen] + recPDF[(size_t)cell + C1 * (size_t)(nb - 1)];
  for (int i = 1; i < nb; ++i) {
    size_t idx = (size_t)cell + C1 * (size_t)(i - 1);
    recPDF[idx] = (off[(i - 1) / chunkLen] + recPDF[idx]) / last;
  }
  recPDF[(size_t)cell + C1 * (size_t)(nb - 1)] = 1.f;
  totalLines[cell] = tl / (normHI + normHeI + normHeII + tl);
}

cudaError_t launchEmission(const EmissionDev& e, const float* te, const float* ne, const float* ionDen,
                           const uint8_t* compute, const float* forLines, float* recPDF, float* totalLines,
                           bool chunked, cudaStream_t s) {
  const int threads = 128, blocks = (e.nCells + threads - 1) / threads;
  // enough chunks for ~8 blocks per SM of the 152, each at least 32 bins long
  const int nChunks =
      chunked ? std::max(1, std::min({kEmChunksMax, (8 * 152 + blocks - 1) / blocks, e.nbins / 32})) : 1;
  emissionKernel<<<dim3(blocks, nChunks), threads, 0, s>>>(e, te, ne, ionDen, compute, forLines, recPDF, totalLines,
                                                           e.part, nChunks, 1);
  emissionKernel<<<blocks, threads, 0, s>>>(e, te, ne, ionDen, compute, forLines, recPDF, totalLines, e.part, nChunks,
                                            2);
  return cudaGetLastError();
}

}  // namespace mcx
