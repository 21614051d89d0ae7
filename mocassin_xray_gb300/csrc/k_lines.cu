// k_lines.cu - outputGas recombination-line and ionic volume sums (FP64).
//
// RecLinesEmission as outputGas has it (source/output_mod.f90:1987-2276),
// which differs from the emission phase's copy: the density bin test is
// Ne >= dens (not >), Ne is not floored at 1e-5 and the HeI fits take T4
// without the emission phase's bounds.  The volume sums follow
// source/output_mod.f90:393-432 and :644-674.
#include "k_emission.cuh"
#include "k_lines.cuh"

namespace mcx {
namespace {

// nearest of the 12 hydroLinesTemps (source/output_mod.f90:2017-2025)
__device__ __forceinline__ int tempBin(const float* temps, double t4) {
  int itemp = 1;
  for (int i = 1; i <= 12; ++i)
    if (t4 > (double)temps[i - 1]) itemp = i;
  if (itemp < 12 && t4 > ((double)temps[itemp] + (double)temps[itemp - 1]) / 2.) itemp = itemp + 1;
  return itemp;
}

__device__ __forceinline__ double ionAt(const EmissionDev& e, const LineSumArgs& a, int xr, int stage, int cell) {
  const size_t C1 = (size_t)a.nCells + 1;
  return (double)a.ionDen[((size_t)(stage - 1) * e.nElemUsed + (xr - 1)) * C1 + cell];
}

// Storey & Hummer Hbeta fit 10**(Afit + Bfit*log10T) with the coefficients of row `row`
__device__ __forceinline__ double hbFit(const EmissionDev& e, int row, double log10N, double log10T) {
  const float* A = e.hbCoeff + (row - 1) * 4;
  const float* B = e.hbCoeff + 36 + (row - 1) * 4;
  double z = (log10N - (double)A[1]) / (double)A[2];
  const double Afit = (double)A[0] * exp(-z * z / 2.) + (double)A[3];
  z = (log10N - (double)B[1]) / (double)B[2];
  const double Bfit = (double)B[0] * exp(-z * z / 2.) + (double)B[3];
  return pow(10., Afit + Bfit * log10T);
}

__global__ void __launch_bounds__(128) gasLineSumsKernel(EmissionDev e, LineSumArgs a) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int group = t >> 5;
  if (group >= a.nGroups) return;   // whole warps only
  const int lane = threadIdx.x & 31;
  const int cell = a.cellBase + t + 1;
  const bool valid = t + 1 <= a.nRange && a.black[cell] < 1;
  double* row = a.partial + (size_t)group * a.nEntries;
  // lanes without a cell evaluate a benign state and contribute 0
  double Te = 1.e4, Ne = 100., Hden = 0., dV = 0.;
  int c = 0;
  if (valid) { Te = a.te[cell]; Ne = a.ne[cell]; Hden = a.hden[cell]; dV = a.vol[cell]; c = cell; }

  // hydrogenic recombination lines (source/output_mod.f90:2011-2229)
  const double T4 = Te / 10000.;
  const double log10Te = log10(Te), log10Ne = log10(Ne);
  const int itemp = tempBin(e.hydroTemps, T4);
  const double t12 = (double)e.hydroTemps[11];
  const int elUp = T4 > t12 ? 2 : 8;
  double hb42 = 0.;
  for (int k = 0; k < a.nHydro; ++k) {
    const int izp = a.hydroIz[k];
    const bool direct = izp <= elUp;
    int it = itemp, fileRow = izp;
    double Nuse = Ne, log10Nuse = log10Ne, log10TeZ = log10Te;
    if (!direct) {
      const double z2 = (double)(izp * izp);
      const double T4z = T4 * 4. / z2;
      log10TeZ = log10(Te * 4. / z2);
      Nuse = Ne * 4. / z2;
      log10Nuse = log10(Ne * 4. / z2);
      it = tempBin(e.hydroTemps, T4z);
      fileRow = 2;
    }
    const int f = e.hydroMap[(fileRow - 1) * 12 + (it - 1)];
    const float* dens = e.hydroDens + (size_t)f * 13;
    const float* L = e.hydroLines + (size_t)f * 13 * 14 * 8;
    int idenp = 1;
    for (int i = 1; i <= 13; ++i)
      if (Nuse >= (double)dens[i - 1] && dens[i - 1] > 0.f) idenp = i;
    const bool interp = (dens[12] > 0.f && idenp < 13) || (dens[12] == 0.f && idenp < 9);
    const double d0 = dens[idenp - 1], d1 = idenp < 13 ? (double)dens[idenp] : 0.;

    double Hb = 0.;
    if (direct) {
      if ((izp == 1 && T4 <= 3.) || (izp > 1 && T4 <= t12)) {
        Hb = hbFit(e, izp, log10Ne, log10Te);
      } else if (izp <= 2) {
        // edge tables beyond the fits (source/output_mod.f90:2096-2136)
        const float* r3 = izp == 1 ? e.rbEdge + 2 * 26 : e.r2aEdge + 2 * 18;
        const int off2 = izp == 1 ? 13 : 9;
        double yy1, yy2;
        if (idenp < 13) {
          yy1 = (double)r3[idenp - 1] + ((double)r3[idenp - 1] - (double)r3[idenp]) * (Ne - d0) / (d1 - d0);
          // r2aEdge(3, 9+idenp+1) lies past the table for idenp = 9: read as r2aEdge(3,18)
          const int hiIdx = izp == 2 && off2 + idenp > 17 ? 17 : off2 + idenp;
          yy2 = (double)r3[off2 + idenp - 1] +
                ((double)r3[off2 + idenp - 1] - (double)r3[hiIdx]) * (Ne - d0) / (d1 - d0);
        } else {
          yy1 = r3[idenp - 1];
          yy2 = r3[off2 + idenp - 1];
        }
        const double x1 = izp == 1 ? (double)e.rbEdge[0] : (double)e.r2aEdge[0];
        const double x2 = izp == 1 ? (double)e.rbEdge[13] : (double)e.r2aEdge[9];
        const double xx = log10(T4 * 1.e4);
        Hb = pow(10., yy1 - (yy1 - yy2) * (xx - x1) / (x2 - x1));
      }
    } else {
      Hb = ((double)(izp * izp * izp) / 8.) * hbFit(e, 2, log10Nuse, log10TeZ);
    }
    const int xr = e.xrefAll[izp - 1];
    Hb = Hb * Ne * ionAt(e, a, xr, izp + 1, c) * (double)e.abunAll[izp - 1];

    const int base = a.hydroBase + k * kHydroLinesPerElem;
    int l = 0;
    for (int iup = 2; iup <= 15; ++iup) {
      const int nLow = iup - 1 < 8 ? iup - 1 : 8;
      for (int ilow = 1; ilow <= nLow; ++ilow, ++l) {
        const double lo = L[((size_t)(idenp - 1) * 14 + (iup - 2)) * 8 + (ilow - 1)];
        double v = lo;
        if (interp) {
          const double hi = L[((size_t)idenp * 14 + (iup - 2)) * 8 + (ilow - 1)];
          v = lo + (hi - lo) * (Nuse - d0) / (d1 - d0);
        }
        v = v * Hb;
        if (izp == 1 && iup == 4 && ilow == 2) hb42 = v;
        const double s = warpSumD(valid ? v * Hden * dV : 0.);
        if (lane == 0) row[base + l] = s;
      }
    }
  }
  {
    double hv = hb42 * Hden * dV;
    const double s = warpSumD(valid && hv > (double)1.e-35f ? hv : 0.);
    if (lane == 0) row[0] = s;
  }

  // HeI recombination lines (source/output_mod.f90:2241-2273)
  if (a.heiBase >= 0) {
    int denint;
    if (Ne <= 100.) denint = 0;
    else if (Ne <= 1.e4) denint = 1;
    else if (Ne <= 1.e6) denint = 2;
    else denint = 3;
    const double xHe = ionAt(e, a, e.xrefAll[1], 2, c);
    for (int l = 0; l < 34; ++l) {
      const float* C0 = e.heiRec + (size_t)l * 12;
      double r;
      if (denint > 0 && denint < 3) {
        const float* p = C0 + (denint - 1) * 4;
        const float* q = C0 + denint * 4;
        const double x1 = (double)p[0] * pow(T4, (double)p[1]) * exp((double)p[2] / T4);
        const double x2 = (double)q[0] * pow(T4, (double)q[1]) * exp((double)q[2] / T4);
        const double p0 = denint == 1 ? 100. : 1.e4, p1 = denint == 1 ? 1.e4 : 1.e6;
        r = x1 + (x2 - x1) * (Ne - p0) / (p1 - p0);
      } else {
        const float* p = C0 + (denint == 0 ? 0 : 2) * 4;
        r = (double)p[0] * pow(T4, (double)p[1]) * exp((double)p[2] / T4);
      }
      r = r * Ne * (double)e.abunAll[1] * xHe;
      const double s = warpSumD(valid ? r * Hden * dV : 0.);
      if (lane == 0) row[a.heiBase + l] = s;
    }
  }

  // mean ionic temperatures and fractions (source/output_mod.f90:644-674)
  const double factor1 = Te * Ne * Hden * dV, factor2 = Ne * Hden * dV;
  int p = 0;
  for (int q = 0; q < a.nIonElem; ++q) {
    const int elem = a.ionElem[q];
    const int top = elem + 1 < e.nstages ? elem + 1 : e.nstages;
    const int xr = e.xrefAll[elem - 1];
    for (int ion = 1; ion <= top; ++ion, ++p) {
      const double x = ionAt(e, a, xr, ion, c);
      const double s1 = warpSumD(valid ? x * factor1 : 0.);
      const double s2 = warpSumD(valid ? x * factor2 : 0.);
      if (lane == 0) { row[a.ionBase + 2 * p] = s1; row[a.ionBase + 2 * p + 1] = s2; }
    }
  }
}

__global__ void lineSumReduceKernel(const double* __restrict__ partial, int nGroups, int nEntries,
                                    double* __restrict__ out) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nEntries) return;
  double s = 0.;
  for (int g = 0; g < nGroups; ++g) s = s + partial[(size_t)g * nEntries + k];
  out[k] = s;
}

__global__ void __launch_bounds__(128) adjointCombineKernel(AdjointArgs a) {
  const int cell = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (cell > a.nCells) return;
  const size_t C1 = (size_t)a.nCells + 1;
  const uint8_t hold = a.hold[cell];
  const double dT = (double)a.teP[cell] - (double)a.teM[cell];
  const double dp = a.pP ? (double)a.pP[cell] - (double)a.pM[cell] : a.dpScalar;
  const bool some = hold < 2 && dT != 0. && dp != 0.;   // a cell with a derivative
  double dTdp = 0.;
  if (some) {
    const double dRdT = (a.rTp[cell] - a.rTm[cell]) / dT;
    const double dRdp = (a.rPp[cell] - a.rPm[cell]) / dp;
    const bool root = hold == 0 && isfinite(dRdT) && dRdT != 0. && isfinite(dRdp);
    if (root) dTdp = -dRdp / dRdT;
    else if (hold == 0 && a.held) atomicAdd(a.held, 1ull);   // a root whose dR/dTe is unusable
  }
  if (a.dTdp) a.dTdp[cell] = dTdp;
  for (int k = 0; k < a.nL; ++k) {
    const size_t i = (size_t)k * C1 + cell;
    double v = 0.;
    if (some) v = (a.lPp[i] - a.lPm[i]) / dp + (dTdp != 0. ? (a.lTp[i] - a.lTm[i]) / dT * dTdp : 0.);
    a.dLdp[i] = v;
  }
}

}  // namespace

cudaError_t launchAdjointCombine(const AdjointArgs& a, cudaStream_t s) {
  if (a.nCells <= 0) return cudaSuccess;
  adjointCombineKernel<<<(a.nCells + 127) / 128, 128, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launchGasLineSums(const EmissionDev& e, const LineSumArgs& a, cudaStream_t s) {
  if (a.nGroups <= 0) return cudaSuccess;
  const int T = 128, nb = (a.nGroups * 32 + T - 1) / T;
  gasLineSumsKernel<<<nb, T, 0, s>>>(e, a);
  return cudaGetLastError();
}

cudaError_t launchLineSumReduce(const double* partial, int nGroups, int nEntries, double* out, cudaStream_t s) {
  if (nEntries <= 0) return cudaSuccess;
  const int T = 128;
  lineSumReduceKernel<<<(nEntries + T - 1) / T, T, 0, s>>>(partial, nGroups, nEntries, out);
  return cudaGetLastError();
}

}  // namespace mcx
