// k_dust.cu - grain opacity, grain re-emission CDF and grain radiative
// equilibrium of a dust-only grid.  Compiled with --fmad=false: every FP32
// operation rounds separately, in the order the reference writes it.
#include "k_dust.cuh"
#include "setup_internal.h"

#include <vector>

namespace mcx {

namespace {

__device__ __forceinline__ float tdAt(const float* td, int n, int ai, int nSz, int c, int C1) {
  return td[((size_t)n * (nSz + 1) + ai) * C1 + c];
}

// getFlux of source/continuum_mod.f90:358-405 for a blackbody
__device__ float blackbody(float energy, float temperature) {
  const float hcRyd_k = 157893.94f, hPlanck = 6.6262e-27f;
  const float constant = 0.5250229f / hPlanck;
  if (hcRyd_k * energy / temperature > 86.f)
    return constant * energy * energy * energy * expf(-hcRyd_k * energy / temperature);
  const float denominator = expf(hcRyd_k * energy / temperature) - 1.f;
  if (denominator <= 0.f) return 3.32154e-6f * energy * energy * temperature / hPlanck;
  return constant * energy * energy * energy / denominator;
}

__global__ void dustOpacityKernel(DustDev d, const float* __restrict__ ndust, const float* __restrict__ tdust,
                                  float* opacity, float* scaOpac) {
  const int C1 = d.nCells + 1;
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (size_t)d.nbins * C1) return;
  const int c = (int)(idx % C1), freq = (int)(idx / C1);
  if (c == 0) return;
  const float nd = ndust[c];
  float sca = 0.f, absO = 0.f;
  for (int n = 0; n < d.nSpecies; ++n)
    for (int ai = 0; ai < d.nSizes; ++ai) {
      if (tdAt(tdust, n + 1, ai + 1, d.nSizes, c, C1) < d.tsub[n]) {
        const size_t o = ((size_t)n * d.nSizes + ai) * d.nbins + freq;
        sca = sca + d.abun[n] * d.weight[ai] * nd * d.Csca[o];
        absO = absO + d.abun[n] * d.weight[ai] * nd * d.Cabs[o];
      }
    }
  scaOpac[idx] = sca;
  opacity[idx] = opacity[idx] + (sca + absO);
}

__global__ void dustPDFKernel(DustDev d, const float* __restrict__ tdust, float* pdf) {
  const int C1 = d.nCells + 1;
  const int c = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (c > d.nCells) return;
  const int nb = d.nbins;
  for (int i = 0; i < nb; ++i) {
    float v = 0.f;
    for (int n = 0; n < d.nSpecies; ++n)
      for (int ai = 0; ai < d.nSizes; ++ai) {
        const float td = tdAt(tdust, n + 1, ai + 1, d.nSizes, c, C1);
        if (td > 0.f && td < d.tsub[n]) {
          const float bb = blackbody(d.nu[i], td);
          v = v + d.Cabs[((size_t)n * d.nSizes + ai) * nb + i] * bb * d.widFlx[i] * d.weight[ai] * d.abun[n];
        }
      }
    pdf[(size_t)i * C1 + c] = v;
  }
  for (int i = 1; i < nb; ++i) pdf[(size_t)i * C1 + c] = pdf[(size_t)(i - 1) * C1 + c] + pdf[(size_t)i * C1 + c];
  const float tot = pdf[(size_t)(nb - 1) * C1 + c];
  for (int i = 0; i < nb; ++i) pdf[(size_t)i * C1 + c] = pdf[(size_t)i * C1 + c] / tot;
  pdf[(size_t)(nb - 1) * C1 + c] = 1.f;
}

// locate (source/interpolation_mod.f90:49-106) on an ascending table
__device__ int locateAsc(const float* xa, int n, float x) {
  if (x > xa[n - 1]) return n;
  if (x < xa[0]) return 0;
  int jlow = 0, jup = n + 1;
  for (int it = 0; it < 10000; ++it) {
    if (jup - jlow < 1) break;
    const int jm = (jup + jlow) / 2;
    if (xa[jm - 1] == x) return jm;
    if (x > xa[jm - 1]) {
      if (jlow == jm) break;
      jlow = jm;
    } else {
      jup = jm;
    }
  }
  return jlow;
}

__global__ void dustTKernel(DustDev d, const double* __restrict__ jste, float* tdust, int32_t* converged,
                            int32_t* black) {
  const int C1 = d.nCells + 1;
  const int c = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (c > d.nCells) return;
  const int nb = d.nbins, nSz = d.nSizes;
  bool hit = false;
  for (int i = 0; i < nb; ++i)
    if ((float)jste[(size_t)i * C1 + c] > 0.f) { hit = true; break; }
  black[c] = hit ? 0 : 1;
  converged[c] = 0;
  if (!hit) {
    atomicAdd(&d.counters->noHit, 1ull);
    return;
  }
  const float pi = 3.141592654f;
  const float xOld = tdAt(tdust, 0, 0, nSz, c, C1);
  for (int n = 0; n <= d.nSpecies; ++n)
    for (int ai = 0; ai <= nSz; ++ai) tdust[((size_t)n * (nSz + 1) + ai) * C1 + c] = 0.f;
  for (int n = 0; n < d.nSpecies; ++n) {
    for (int ai = 0; ai < nSz; ++ai) {
      const float* ca = d.Cabs + ((size_t)n * nSz + ai) * nb;
      float integral = 0.f;
      for (int i = 0; i < nb; ++i) integral = integral + ca[i] * ((float)jste[(size_t)i * C1 + c] / pi);
      const float* em = d.emInt + ((size_t)n * nSz + ai) * kNTemps;
      const int iT = locateAsc(em, kNTemps, integral);
      float t;
      if (iT <= 0) t = 1.f;
      else if (iT >= kNTemps) t = (float)kNTemps;
      else t = (float)iT + (integral - em[iT - 1]) * ((float)(iT + 1) - (float)iT) / (em[iT] - em[iT - 1]);
      tdust[((size_t)(n + 1) * (nSz + 1) + (ai + 1)) * C1 + c] = t;
      float& tn0 = tdust[((size_t)(n + 1) * (nSz + 1)) * C1 + c];
      tn0 = tn0 + t * d.weight[ai];
    }
    float& t00 = tdust[c];
    t00 = t00 + tdust[((size_t)(n + 1) * (nSz + 1)) * C1 + c] * d.abun[n];
  }
  const float delta = (tdust[c] - xOld) / xOld;
  const int conv = fabsf(delta) <= d.xhiLimit ? 1 : 0;
  converged[c] = conv;
  atomicAdd(&d.counters->updated, 1ull);
  if (conv) atomicAdd(&d.counters->converged, 1ull);
}

}  // namespace

DustData::~DustData() {
  for (int i = 0; i < nBlocks; ++i)
    if (blocks[i]) cudaFree(blocks[i]);
}

std::string dustDataCreate(const Setup& s, std::unique_ptr<DustData>& out) {
  auto dd = std::make_unique<DustData>();
  DustDev& d = dd->dev;
  const DustTables& t = s.dust;
  d.nbins = s.nbins; d.nCells = s.nCells; d.nSpecies = t.nSpecies; d.nSizes = t.nSizes;
  d.xhiLimit = s.p.XHILimit;
  std::string err;
  auto up = [&](const void* src, size_t bytes) -> void* {
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, bytes ? bytes : 1);
    if (e != cudaSuccess) { err = std::string("dust tables: ") + cudaGetErrorString(e); return nullptr; }
    dd->blocks[dd->nBlocks++] = p;
    if (bytes && src) {
      e = cudaMemcpy(p, src, bytes, cudaMemcpyHostToDevice);
      if (e != cudaSuccess) err = std::string("dust tables: ") + cudaGetErrorString(e);
    }
    return p;
  };
  d.nu = (const float*)up(s.nu.data(), s.nu.size() * 4);
  d.widFlx = (const float*)up(s.widFlx.data(), s.widFlx.size() * 4);
  d.Cabs = (const float*)up(t.Cabs.data(), t.Cabs.size() * 4);
  d.Csca = (const float*)up(t.Csca.data(), t.Csca.size() * 4);
  d.abun = (const float*)up(t.grainAbun.data(), t.grainAbun.size() * 4);
  d.tsub = (const float*)up(t.TdustSublime.data(), t.TdustSublime.size() * 4);
  d.weight = (const float*)up(t.grainWeight.data(), t.grainWeight.size() * 4);
  d.emInt = (const float*)up(t.emIntegral.data(), t.emIntegral.size() * 4);
  d.counters = (DustCounters*)up(nullptr, sizeof(DustCounters));
  if (!err.empty()) return err;
  out = std::move(dd);
  return "";
}

cudaError_t launchDustOpacity(const DustDev& d, const float* ndust, const float* tdust, float* opacity, float* scaOpac,
                              cudaStream_t s) {
  const size_t n = (size_t)d.nbins * (d.nCells + 1);
  const int T = 256;
  dustOpacityKernel<<<(unsigned)((n + T - 1) / T), T, 0, s>>>(d, ndust, tdust, opacity, scaOpac);
  return cudaGetLastError();
}

cudaError_t launchDustPDF(const DustDev& d, const float* tdust, float* dustPDF, cudaStream_t s) {
  const int T = 128;
  dustPDFKernel<<<(d.nCells + T - 1) / T, T, 0, s>>>(d, tdust, dustPDF);
  return cudaGetLastError();
}

cudaError_t launchDustT(const DustDev& d, const double* jste, float* tdust, int32_t* converged, int32_t* black,
                        cudaStream_t s) {
  const int T = 128;
  cudaError_t e = cudaMemsetAsync(d.counters, 0, sizeof(DustCounters), s);
  if (e != cudaSuccess) return e;
  dustTKernel<<<(d.nCells + T - 1) / T, T, 0, s>>>(d, jste, tdust, converged, black);
  return cudaGetLastError();
}

}  // namespace mcx
