// k_balance.cu - the balance phase: updateCell / iterateT for every cell
// (source/update_mod.f90:15-482 and the routines it calls), and the
// multi-level atom solve equilibrium (source/emission_mod.f90:2505-3106).
// Compiled with --fmad=false: every FP64 operation is rounded separately, in
// the order the reference writes it.
#include "k_balance.cuh"
#include "setup_internal.h"

#include <algorithm>
#include <cstring>
#include <vector>

namespace mcx {

namespace {

// a default-REAL constant of the reference, at its single-precision value
#define RF(x) ((double)(x##f))

__device__ __forceinline__ double kBoltz() { return RF(1.380658e-16); }    // constants_mod.f90:18
__device__ __forceinline__ double kRyd2erg() { return RF(2.1799e-11); }   // constants_mod.f90:20
__device__ __forceinline__ double kHcRyd() { return RF(2.1799153e-11); }  // update_mod.f90:64
__device__ __forceinline__ double kXMax() { return RF(0.99999); }         // constants_mod.f90:57

constexpr int kNE = 30;

struct CellIdx {
  int cell, C1;
};

// ionDen of (element Z, stage) in the work array
__device__ __forceinline__ double& ionAt(const BalanceDev& b, const CellIdx& c, int z, int st) {
  return b.ion[((size_t)(st - 1) * b.nElemUsed + (b.xref[z] - 1)) * c.C1 + c.cell];
}
__device__ __forceinline__ size_t pairOff(const BalanceDev& b, const CellIdx& c, int z, int ion) {
  return ((size_t)(b.xref[z] - 1) * b.nstages + (ion - 1)) * c.C1 + c.cell;
}

// ------------------------------------------------------------- rate functions

// RRbadnell, source/update_mod.f90:2415-2433
__device__ double rrBadnell(const BalanceDev& b, double te, int elem, int nel) {
  const float* t = b.RRb;
  auto RB = [&](int k) { return (double)t[((size_t)k * kNE + (elem - 1)) * (kNE + 1) + nel]; };
  double A = RB(0), B = RB(1), T0 = RB(2), T1 = RB(3), Cc = RB(4), T2 = RB(5);
  double bbad = B + Cc * exp(-T2 / te);
  return A / (pow(te / T0, 0.5) * pow(1. + pow(te / T0, 0.5), 1. - bbad) * pow(1. + pow(te / T1, 0.5), 1. + bbad));
}

// DRbadnell, source/update_mod.f90:2435-2450
__device__ double drBadnell(const BalanceDev& b, double te, int elem, int nel) {
  double dr = 0.;
  const float* E = b.DRbE + ((size_t)(elem - 1) * (kNE + 1) + nel) * 9;
  const float* Cc = b.DRbC + ((size_t)(elem - 1) * (kNE + 1) + nel) * 9;
  for (int idr = 0; idr < 9; ++idr)
    if ((double)E[idr] / te < 87.) dr = dr + (double)Cc[idr] * exp(-(double)E[idr] / te);
  return dr * pow(te, -1.5);
}

// radRecFit, source/update_mod.f90:3094-3202 (Fe I-XV fit table of :3160-3166)
__constant__ double kFeFit[3][10] = {
    {RF(4.33e-10), RF(3.91e-10), RF(3.49e-10), RF(3.16e-10), RF(2.96e-10), RF(2.59e-10), RF(2.24e-10), RF(1.91e-10),
     RF(1.68e-10), RF(1.46e-10)},
    {RF(0.531), RF(0.523), RF(0.521), RF(0.534), RF(0.557), RF(0.567), RF(0.579), RF(0.601), RF(0.602), RF(0.597)},
    {RF(5.77e-02), RF(6.15e-02), RF(6.22e-02), RF(6.02e-02), RF(5.79e-02), RF(5.65e-02), RF(5.49e-02), RF(5.10e-02),
     RF(5.07e-02), RF(5.22e-02)}};

__device__ double radRecFit(const BalanceDev& b, double te, int z, int n) {
  if ((n <= 3) || (n == 11) || ((z > 5) && (z < 9)) || (z == 10) || ((z == 26) && (n > 11))) {
    const float* r = b.rnew + ((size_t)(z - 1) * kNE + (n - 1)) * 4;
    double tt = sqrt(te / (double)r[2]);
    return (double)r[0] / (tt * pow(tt + 1., 1. - (double)r[1]) * pow(1. + sqrt(te / (double)r[3]), 1. + (double)r[1]));
  }
  double tt = te * RF(1.e-4);
  if ((z == 26) && (n <= 13)) return kFeFit[0][n - 4] / pow(tt, kFeFit[1][n - 4] + kFeFit[2][n - 4] * log10(tt));
  const float* r = b.rrec + ((size_t)(z - 1) * kNE + (n - 1)) * 2;
  return (double)r[0] / pow(tt, (double)r[1]);
}

// diRec(elem, ion) of dielectronic (source/update_mod.f90:3204-3305): the
// last row of dielectronic.dat for (elem, ion) whose temperature flag
// applies, or above 6e4 K the last row of aldrovandi.dat.
__device__ double diRecOf(const BalanceDev& b, double te, int elem, int ion) {
  if (ion > b.nstages) return 0.;
  if (te > 60000.) {
    double v = 0.;
    for (int r = 0; r < b.nAldro; ++r) {
      const float* d = b.aldro + (size_t)r * 6;
      if ((int)d[0] != elem || (int)d[0] - (int)d[1] + 1 != ion) continue;
      double a = d[2], bb = d[3], t0 = d[4], t1 = d[5];
      v = a * pow(te, -1.5) * exp(-t0 / te) * (1. + bb * exp(-t1 / te));
    }
    return v;
  }
  double t = te > 1000. ? te / 10000. : RF(0.1);
  double v = 0.;
  for (int r = 0; r < b.nDiel; ++r) {
    const float* d = b.diel + (size_t)r * 8;
    if ((int)d[0] != elem || (int)d[0] + 1 - (int)d[1] != ion) continue;
    int g = (int)d[7];
    bool use = g == 0 || (g == 1 && te < 20000.) || (g == 2 && te >= 20000.);
    if (!use) continue;
    double a = d[2], bb = d[3], cc = d[4], dd = d[5], f = d[6];
    v = RF(1e-12) * (a / t + bb + cc * t + dd * (t * t)) * pow(t, -1.5) * exp(-f / t);
  }
  return v;
}

// calcAlpha, source/update_mod.f90:2298-2413
__device__ void calcAlpha(const BalanceDev& b, const CellIdx& c, double te) {
  const int ns = b.nstages;
  for (int e = 1; e <= b.nElemUsed; ++e) {
    const int elem = b.zOf[e];
    const int top = min(ns - 1, elem);
    for (int ion = 1; ion <= top; ++ion) {
      double a;
      if (b.lgBadnell) {
        int nel = elem - ion;
        if (nel <= 11) {
          a = rrBadnell(b, te, elem, nel);
          a = a + drBadnell(b, te, elem, nel);
        } else {
          a = radRecFit(b, te, elem, elem - ion + 1);
          double di = diRecOf(b, te, elem, ion);
          if (di == 0. && ion < 7 && b.xref[8] > 0) di = diRecOf(b, te, 8, ion);
          a = a + (di > 0. ? di : 0.);
        }
      } else {
        a = radRecFit(b, te, elem, elem - ion + 1);
        if (elem >= 3) {
          double di = diRecOf(b, te, elem, ion);
          if (di == 0. && ion < 7) di = diRecOf(b, te, 8, ion);
          a = a + (di > 0. ? di : 0.);
        }
      }
      b.alpha[pairOff(b, c, elem, ion)] = a;
    }
  }
}

// charge-exchange coefficients (a, b, c, d) of ionBalance and photoionisation
// (source/update_mod.f90:1649-1701, :3727-3779), "Ca" rows written into Ar's
struct Chex {
  float z, ion, a, b, c, d;
};
__constant__ Chex kChex[] = {
    {2, 1, 7.47e-6f, 2.06f, 9.93f, -3.89f},       {2, 2, 1.e-5f, 0.f, 0.f, 0.f},
    {3, 2, 1.26f, 0.96f, 3.02f, -0.65f},          {3, 3, 1.e-5f, 0.f, 0.f, 0.f},
    {4, 2, 1.e-5f, 0.f, 0.f, 0.f},                {4, 3, 1.e-5f, 0.f, 0.f, 0.f},
    {4, 4, 5.17f, 0.82f, -.69f, -1.12f},          {5, 2, 2.e-2f, 0.f, 0.f, 0.f},
    {5, 3, 1.e-5f, 0.f, 0.f, 0.f},                {5, 4, 5.27e-1f, 0.76f, -0.63f, -1.17f},
    {6, 1, 1.76e-9f, 8.33f, 4278.78f, -6.41f},    {6, 2, 1.67e-4f, 2.79f, 304.72f, -4.07f},
    {6, 3, 3.25f, 0.21f, 0.19f, -3.29f},          {6, 4, 332.46f, -0.11f, -0.995f, -1.58e-3f},
    {7, 1, 1.01e-3f, -0.29f, -0.92f, -8.38f},     {7, 2, 3.05e-1f, 0.60f, 2.65f, -0.93f},
    {7, 3, 4.54f, 0.57f, -0.65f, -0.89f},         {7, 4, 3.28f, 0.52f, -0.52f, -0.19f},
    {8, 1, 1.04f, 3.15e-2f, -0.61f, -9.73f},      {8, 2, 1.04f, 0.27f, 2.02f, -5.92f},
    {8, 3, 3.98f, 0.26f, 0.56f, -2.62f},          {8, 4, 2.52e-1f, 0.63f, 2.08f, -4.16f},
    {9, 2, 1.e-5f, 0.f, 0.f, 0.f},                {9, 3, 9.86f, 0.29f, -0.21f, -1.15f},
    {9, 4, 7.15e-1f, 1.21f, -0.70f, -0.85f},      {10, 2, 1.e-5f, 0.f, 0.f, 0.f},
    {10, 3, 14.73f, 4.52e-2f, -0.84f, -0.31f},    {10, 4, 6.47f, 0.54f, 3.59f, -5.22f},
    {11, 2, 1.e-5f, 0.f, 0.f, 0.f},               {11, 3, 1.33f, 1.15f, 1.20f, -0.32f},
    {11, 4, 1.01e-1f, 1.34f, 10.05f, -6.41f},     {12, 2, 8.58e-5f, 2.49e-3f, 2.93e-2f, -4.33f},
    {12, 3, 6.49f, 0.53f, 2.82f, -7.63f},         {12, 4, 6.36f, 0.55f, 3.86f, -5.19f},
    {13, 2, 1.e-5f, 0.f, 0.f, 0.f},               {13, 3, 7.11e-5f, 4.12f, 1.72e4f, -22.24f},
    {13, 4, 7.52e-1f, 0.77f, 6.24f, -5.67f},      {14, 2, 1.23f, 0.24f, 3.17f, 4.18e-3f},
    {14, 3, 4.900e-1f, -8.74e-2f, -0.36f, -0.79f}, {14, 4, 7.58f, 0.37f, 1.06f, -4.09f},
    {16, 1, 3.82e-7f, 11.10f, 2.57e4f, -8.22f},   {16, 2, 1.e-5f, 0.f, 0.f, 0.f},
    {16, 3, 2.29f, 4.02e-2f, 1.59f, -6.06f},      {16, 4, 6.44f, 0.13f, 2.69f, -5.69f},
    {18, 2, 1.e-5f, 0.f, 0.f, 0.f},               {18, 3, 3.17e-2f, 2.12f, 12.06f, -0.40f},
    {18, 4, 2.68f, 0.69f, -0.68f, -4.47f},        {26, 2, 1.26f, 7.72e-2f, -0.41f, -7.31f},
    {26, 3, 3.42f, 0.51f, -2.06f, -8.99f}};
constexpr int kNChex = sizeof(kChex) / sizeof(Chex);

__device__ const Chex* chexOf(int z, int ion) {
  for (int i = 0; i < kNChex; ++i)
    if ((int)kChex[i].z == z && (int)kChex[i].ion == ion) return &kChex[i];
  return nullptr;
}
// chex(z, ion, 1) * 1e-9 without the temperature fit (ionBalance's heavy elements)
__device__ double chexRaw(int z, int ion) {
  const Chex* x = chexOf(z, ion);
  return x ? (double)x->a * RF(1.e-9) : 0.;
}
// chex(z, ion, 1) at Te (source/update_mod.f90:1711-1720, :3788-3797)
__device__ double chexFit(int z, int ion, double te) {
  const Chex* x = chexOf(z, ion);
  if (!x) return 0.;
  double a = (double)x->a * RF(1.e-9);
  double t4 = te / 10000.;
  double v = (te < 6000. || te > 5.e4) ? 0. : a * pow(t4, (double)x->b) * (1. + (double)x->c * exp((double)x->d * t4));
  return v < 0. ? 0. : v;
}

__device__ __forceinline__ const int32_t* outerOf(const BalanceDev& b, int z, int nElec) {
  return b.outer + ((size_t)(z - 1) * kNE + (nElec - 1)) * 3;
}

// ------------------------------------------------------ J-only integrals

// The parts of photoionisation / getPhotoRates / compton that depend on J
// alone (source/update_mod.f90:3641-3700, :3971-4040, :3834-3897); one
// thread per cell.
__global__ void __launch_bounds__(128) photoIntegralsKernel(BalanceDev b, const double* __restrict__ jste) {
  const int cell = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (cell > b.nCells) return;
  const int C1 = b.nCells + 1;
  const float* nu = b.nu;
  const float* xs = b.xsec;
  auto J = [&](int bin1) { return jste[(size_t)(bin1 - 1) * C1 + cell]; };
  bool hit = false;
  for (int i = 1; i <= b.nbins; ++i)
    if (J(i) > 0.) { hit = true; break; }
  b.state[cell] = hit ? 0 : 2;
  if (!hit) return;
  const double hcRyd = kHcRyd();
  for (int t = 0; t < b.nShellsTot; ++t) {
    const PhotoShell sh = b.shells[t];
    const size_t o = (size_t)t * C1 + cell;
    if (sh.ipNuP < 1 || sh.ipNuP > b.nbins) {   // threshold outside the mesh (set-up rejects it too)
      b.gam[o] = sh.heavy ? 0. : RF(1.e-20);
      b.heatA[o] = 0.;
      b.heatHi[o] = 0.;
      continue;
    }
    if (!sh.heavy) {
      double n1 = RF(1.e-20), h1 = 0.;
      for (int j = sh.ipNuP; j <= sh.highNuP; ++j) {
        double ph = xs[j - sh.ipNuP + sh.xsecP - 1];
        if (ph < RF(1.e-35)) ph = 0.;
        double jj = J(j);
        if (jj > 0.) {
          n1 = n1 + jj * ph / (hcRyd * (double)nu[j - 1]);
          h1 = h1 + ph * jj * ((double)nu[j - 1] - (double)nu[sh.ipNuP - 1]) / (double)nu[j - 1];
        }
      }
      b.gam[o] = n1;
      b.heatA[o] = h1;
      b.heatHi[o] = 0.;
      continue;
    }
    const int nu1P = sh.ipNuP, IPnuP = sh.ipNuP;
    const int iup = min(sh.highNuP, b.nbins);
    const double augerE = hcRyd * (double)nu[nu1P - 1] * (double)sh.yield1;
    double g = 0., h = 0.;
    const int top = min(iup, b.secIonP - 1);
    for (int i = nu1P + 1; i <= top; ++i) {
      double jj = J(i);
      if (jj > 0.) {
        double ph = xs[i + sh.xsecP - IPnuP - 1];
        if (ph < RF(1.e-35)) ph = 0.;
        g = g + jj * ph / (hcRyd * (double)nu[i - 1]);
        h = h + jj * ph;
      }
    }
    h = h - g * augerE;
    const double jIP = J(IPnuP);
    const double ph0 = xs[sh.xsecP - 1];
    g = g + jIP * ph0 / (hcRyd * (double)nu[IPnuP - 1]);
    h = h + jIP * ph0 * (hcRyd * (double)nu[IPnuP - 1] - augerE) / (hcRyd * (double)nu[IPnuP - 1]);
    double gh = 0., hh = 0.;
    const int ilow = max(IPnuP + 1, b.secIonP);
    for (int i = ilow; i <= iup; ++i) {
      double p = xs[i + sh.xsecP - IPnuP - 1];
      gh = gh + jIP * p / (hcRyd * (double)nu[i - 1]);   // radField(IPnuP), as the reference
      hh = hh + jIP * p;
    }
    g = g + gh;
    hh = hh - gh * augerE;
    b.gam[o] = g;
    b.heatA[o] = h;
    b.heatHi[o] = hh;
  }
  if (b.lgCompton) {
    double s1 = 0., s2 = 0., rhH = 0., rhHe = 0.;
    for (int i = 1; i <= b.nbins; ++i) {
      double rf = J(i);
      s1 = s1 + rf;
      s2 = s2 + rf / (double)nu[i - 1];
      if (i > b.cRecoilHP) {
        double energy = RF(2.66e-5) * (double)nu[i - 1] * (double)nu[i - 1] - 1.;
        rhH = rhH + (double)b.xsecRecoil[i - 1] * rf * energy;
      }
      if (i > b.cRecoilHeP) {
        double energy = RF(2.66e-5) * (double)nu[i - 1] * (double)nu[i - 1] - RF(1.8);
        rhHe = rhHe + (double)b.xsecRecoil[i - 1] * rf * energy;
      }
    }
    b.comp[0 * (size_t)C1 + cell] = s1 * kRyd2erg();
    b.comp[1 * (size_t)C1 + cell] = s2;
    b.comp[2 * (size_t)C1 + cell] = rhH;
    b.comp[3 * (size_t)C1 + cell] = rhHe;
  }
}

// Loads the grid state of the cells into the FP64 work arrays.
__global__ void loadStateKernel(BalanceDev b, const float* __restrict__ te, const float* __restrict__ ne,
                                const float* __restrict__ ionDen) {
  const int cell = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (cell > b.nCells) return;
  const int C1 = b.nCells + 1;
  b.te[cell] = te[cell];
  b.ne[cell] = ne[cell];
  const size_t nI = (size_t)b.nstages * b.nElemUsed;
  for (size_t k = 0; k < nI; ++k) b.ion[k * C1 + cell] = ionDen[k * C1 + cell];
  b.xOld[cell] = b.ion[(size_t)(b.xref[1] - 1) * C1 + cell];
  b.tHigh[cell] = 0.; b.tLow[cell] = 0.; b.resHigh[cell] = 0.; b.resLow[cell] = 0.;
  b.nIterT[cell] = 0;
  b.ibConv[cell] = 1;
}

// -------------------------------------------------------------- one round

// ionBalance, source/update_mod.f90:1575-1992 (recursion as a loop); returns lgConv.
__device__ bool ionBalance(const BalanceDev& b, const CellIdx& c, double te, double& ne, double hden) {
  const int ns = b.nstages;
  const int zH = 1, zHe = 2;
  const bool heOn = b.xref[zHe] > 0;
  const int C1 = c.C1;
  for (int nIterateX = 1;; ++nIterateX) {
    bool lgConv = true;
    double ionRatio[3][3] = {{0., 0., 0.}, {0., 0., 0.}, {0., 0., 0.}};
    double ionProd[3][3] = {{1., 1., 1.}, {1., 1., 1.}, {1., 1., 1.}};
    double den[3] = {1., 1., 1.};
    double expFact = (double)RF(157893.94) / te;
    if (expFact > 75.) expFact = 75.;
    double collIonH = RF(2.75E-16) * te * sqrt(te) * ((double)RF(157893.94) / te + 2.) * exp(-expFact);
    const double HIOld = ionAt(b, c, zH, 1);
    const double HeIOld = heOn ? ionAt(b, c, zHe, 1) : 0.;
    const double HeIIOld = heOn ? ionAt(b, c, zHe, 2) : 0.;
    const double xH0 = HIOld;
    for (int elem = 1; elem <= 2; ++elem) {
      if (!b.xref[elem]) continue;
      for (int ion = 1; ion <= min(elem, ns - 1); ++ion) {
        double cx = chexFit(elem, ion, te);
        int outShell = outerOf(b, elem, elem - ion + 1)[0];
        if (elem > 1 || ion > 1) collIonH = 0.;
        int p0 = b.pairShell0[(b.xref[elem] - 1) * 32 + (ion - 1)];
        double pi = b.pi1[(size_t)(p0 + outShell - 1) * C1 + c.cell];
        ionRatio[elem][ion] = (pi + collIonH * ne + 0.) /
                              (ne * b.alpha[pairOff(b, c, elem, ion)] + cx * hden * xH0);
      }
    }
    for (int elem = 1; elem <= 2; ++elem) {
      if (!b.xref[elem]) continue;
      for (int ion = 1; ion <= min(elem, ns - 1); ++ion)
        for (int i = 1; i <= ion; ++i) ionProd[elem][ion] = ionProd[elem][ion] * ionRatio[elem][i];
    }
    for (int elem = 1; elem <= 2; ++elem) {
      if (!b.xref[elem]) continue;
      for (int ion = 1; ion <= min(elem, ns - 1); ++ion) den[elem] = den[elem] + ionProd[elem][ion];
    }
    for (int elem = 1; elem <= 2; ++elem) {
      if (!b.xref[elem]) continue;
      for (int ion = 1; ion <= min(elem + 1, ns); ++ion) {
        double v = ion == 1 ? 1. / den[elem] : ionProd[elem][ion - 1] / den[elem];
        if (v > kXMax()) v = kXMax();
        if (v < RF(1.e-20)) v = RF(1.e-20);
        ionAt(b, c, elem, ion) = v;
      }
    }
    // heavy elements: the bidiagonal ladder
    for (int e = 1; e <= b.nElemUsed; ++e) {
      const int elem = b.zOf[e];
      if (elem < 3) continue;
      double out[33], inn[33], mat[33];
      for (int k = 0; k < 33; ++k) { out[k] = 0.; inn[k] = 0.; }
      const int topI = min(elem, ns - 1);
      const int lim = min(ns - 1, elem);
      for (int ion = 1; ion <= topI; ++ion) {
        out[ion] = out[ion] + b.coll1[pairOff(b, c, elem, ion)] * ne;
        const int p0 = b.pairShell0[(e - 1) * 32 + (ion - 1)];
        const int nsh = b.pairNShell[(e - 1) * 32 + (ion - 1)];
        for (int shell = 1; shell <= nsh; ++shell) {
          const double pi = b.pi1[(size_t)(p0 + shell - 1) * C1 + c.cell];
          out[ion] = out[ion] + pi;
          const int nAug = b.nauger[((size_t)(elem - 1) * kNE + (ion - 1)) * 10 + (shell - 1)];
          for (int nelec = 2; nelec <= nAug; ++nelec) {
            int maxim = min(ion + nelec - 1, lim);
            double xm = ionAt(b, c, elem, maxim);
            double ratio = xm > 1e-30 ? ionAt(b, c, elem, ion) / xm : 1.;
            out[maxim] = out[maxim] +
                         pi * (double)b.auger[(((size_t)(elem - 1) * kNE + (ion - 1)) * 10 + (shell - 1)) * 10 + (nelec - 1)] * ratio;
          }
        }
      }
      // X(H0) as just updated above (grid%ionDen in the reference)
      const double xH0now = ionAt(b, c, zH, 1);
      for (int ion = 1; ion <= topI; ++ion)
        inn[ion] = ne * b.alpha[pairOff(b, c, elem, ion)] + chexRaw(elem, ion) * hden * xH0now;
      mat[1] = 1.;
      double sumMat = 1.;
      const int top = min(ns, elem + 1);
      for (int ion = 2; ion <= top; ++ion) {
        mat[ion] = mat[ion - 1] * out[ion - 1] / inn[ion - 1];
        sumMat = sumMat + mat[ion];
      }
      sumMat = 1. / sumMat;
      ionAt(b, c, elem, top) = mat[top] * sumMat;
      for (int ion = 1; ion <= topI; ++ion) {
        double v;
        if (nIterateX < 2 && mat[ion] * sumMat > 0.) {
          double old = ionAt(b, c, elem, ion);
          if (old <= 0.) old = RF(1.e-5);
          v = pow(10., 0.5 * (log10(old) + log10(mat[ion] * sumMat)));
        } else {
          v = mat[ion] * sumMat;
        }
        if (v > kXMax()) v = kXMax();
        if (v < RF(1.e-20)) v = RF(1.e-20);
        ionAt(b, c, elem, ion) = v;
      }
    }
    // electron density
    double nE = 0.;
    for (int e = 1; e <= b.nElemUsed; ++e) {
      const int elem = b.zOf[e];
      for (int ion = 2; ion <= min(elem + 1, ns); ++ion) {
        double x = ionAt(b, c, elem, ion);
        if (x >= RF(1.e-10)) nE = nE + (double)(ion - 1) * (double)b.abun[elem] * x;
      }
    }
    nE = nE * hden;
    if (nE == 0.) nE = 1.;
    ne = nE;
    double dHI = (ionAt(b, c, zH, 1) - HIOld) / HIOld;
    double dHeI = heOn ? (ionAt(b, c, zHe, 1) - HeIOld) / HeIOld : 0.;
    double dHeII = heOn ? (ionAt(b, c, zHe, 2) - HeIIOld) / HeIIOld : 0.;
    bool big = fabs(dHI) > RF(0.01) || fabs(dHeI) > RF(0.01) || fabs(dHeII) > RF(0.01);
    if (big && nIterateX < 15) continue;
    if (big && nIterateX == 15) lgConv = false;
    return lgConv;
  }
}

// calcAlpha, photoionisation, collisionalIonisation, compton, ionBalance and
// the thermBalance terms without forLines (source/update_mod.f90:277-340,
// :887-1215); one thread per iterating cell.
__global__ void __launch_bounds__(128) ratesKernel(BalanceDev b, const float* __restrict__ hdenG) {
  const int cell = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (cell > b.nCells || b.state[cell] != 0) return;
  const CellIdx c{cell, b.nCells + 1};
  const int C1 = c.C1, ns = b.nstages;
  b.nIterT[cell] = b.nIterT[cell] + 1;
  const double te = b.te[cell];
  double ne = b.ne[cell];
  const double hden = hdenG[cell];
  calcAlpha(b, c, te);
  // photoionisation (source/update_mod.f90:3584-3832)
  double xe = 0.;
  for (int e = 1; e <= b.nElemUsed; ++e) {
    const int elem = b.zOf[e];
    xe = xe + ionAt(b, c, elem, 1) * (double)b.abun[elem] * hden;
  }
  xe = ne / xe;
  double heatef;
  if (xe > RF(0.95)) heatef = 1.;
  else {
    if (xe < RF(1.e-4)) xe = RF(1.e-4);
    heatef = RF(0.9971) * (1. - pow(1. - pow(xe, RF(0.2663)), RF(1.3163)));
  }
  for (int t = 0; t < b.nShellsTot; ++t) {
    const size_t o = (size_t)t * C1 + cell;
    b.pi1[o] = b.gam[o];
    b.pi2[o] = b.shells[t].heavy ? b.heatA[o] + b.heatHi[o] * heatef : b.heatA[o];
  }
  // reverse charge exchange: deltaE_k > 1 only for N0 and O0
  for (int k = 0; k < 2; ++k) {
    const int elem = k == 0 ? 7 : 8;
    const double dE = k == 0 ? RF(10863.) : RF(2205.);
    if (!b.xref[elem] || ns - 1 < 1) continue;
    const int32_t* o = outerOf(b, elem, elem);
    const int nsh = b.pairNShell[(b.xref[elem] - 1) * 32];
    if (o[0] > nsh) continue;
    double cx = chexFit(elem, 1, te);
    double rev = cx * (1. - ionAt(b, c, 1, 1)) * hden * 2. * exp(-dE / te) / ((double)o[1] / (double)o[2]);
    const size_t off = (size_t)(b.pairShell0[(b.xref[elem] - 1) * 32] + o[0] - 1) * C1 + cell;
    b.pi1[off] = b.pi1[off] + rev;
  }
  // collisionalIonisation (source/update_mod.f90:3552-3582)
  {
    for (int e = 1; e <= b.nElemUsed; ++e)
      for (int ion = 1; ion <= ns; ++ion) {
        size_t o = ((size_t)(e - 1) * ns + (ion - 1)) * C1 + cell;
        b.coll1[o] = 0.;
        b.coll2[o] = 0.;
      }
    const double tev = te * RF(8.617385e-05);
    bool stop = false;
    for (int e = 1; e <= b.nElemUsed && !stop; ++e) {
      const int elem = b.zOf[e];
      for (int ion = 1; ion <= min(ns - 1, elem - 1); ++ion) {
        const int elec = elem - ion + 1;
        const float* cf = b.CF + ((size_t)(elem - 1) * kNE + (elec - 1)) * 5;
        double u = (double)cf[0] / tev;
        if (u > 80.) { stop = true; break; }
        double c1 = (double)cf[2] * (1. + (double)cf[1] * sqrt(u)) / ((double)cf[3] + u) * pow(u, (double)cf[4]) * exp(-u);
        b.coll1[pairOff(b, c, elem, ion)] = c1;
        b.coll2[pairOff(b, c, elem, ion)] = (double)b.cionTherm[(elem - 1) * kNE + (ion - 1)] * c1 * kBoltz();
      }
    }
  }
  // compton (source/update_mod.f90:3834-3897), with the state before ionBalance
  if (b.lgCompton) {
    const double s1 = b.comp[0 * (size_t)C1 + cell], s2 = b.comp[1 * (size_t)C1 + cell];
    const double rhH = b.comp[2 * (size_t)C1 + cell], rhHe = b.comp[3 * (size_t)C1 + cell];
    double cool = (RF(6.65e-25) * RF(6.75e-10) * te * s2) / hden;
    double heat = (RF(6.65e-25) * s1 / RF(8.184e-7)) / hden;
    double he = b.xref[2] ? rhHe * (ionAt(b, c, 2, 1) * (double)b.abun[2]) * 2. : 0.;
    double recoil = (rhH * ionAt(b, c, 1, 1) * (double)b.abun[1] + he) * kRyd2erg();
    b.compCool[cell] = cool;
    b.compHeat[cell] = heat;
    b.compRecoil[cell] = recoil;
  }
  bool conv = ionBalance(b, c, te, ne, hden);
  b.ibConv[cell] = conv ? 1 : 0;
  b.ne[cell] = ne;
  // thermBalance without forLines
  double coolFF = 0., coolRec = 0., L, Te4;
  for (int e = 1; e <= b.nElemUsed; ++e) {
    const int i = b.zOf[e];
    if (!(ns > i)) continue;
    L = log10(te / (double)(i * i));
    Te4 = te / ((double)(i * i) * RF(1.e4));
    double Np = ionAt(b, c, i, i + 1) * (double)b.abun[i];
    double betaFF = (double)i * (RF(1.0108464E-11) + RF(9.7930778E-13) * L - RF(6.6433144E-13) * L * L +
                                 RF(2.4793747E-13) * L * L * L - RF(2.3938215E-14) * L * L * L * L);
    double t = Np * ne * betaFF * kBoltz() * te / sqrt(te);
    if (!isnan(t)) coolFF = coolFF + t;
    double betaRec = (double)i * (RF(9.4255985E-11) - RF(4.04794384E-12) * L - RF(1.0055237E-11) * L * L +
                                  RF(1.99266862E-12) * L * L * L - RF(1.06681387E-13) * L * L * L * L);
    t = Np * ne * betaRec * kBoltz() * te / sqrt(te);
    if (!isnan(t)) coolRec = coolRec + t;
  }
  Te4 = te / RF(1.e4);
  for (int e = 1; e <= b.nElemUsed; ++e) {
    const int i = b.zOf[e];
    if (i < 2 || !(ns > i)) continue;
    L = log10(4. * te / (double)(i * i));
    Te4 = 4. * te / ((double)(i * i) * RF(1.e4));
    double Np = ionAt(b, c, i, i) * (double)b.abun[i];
    double betaFF = ((double)i / 2.) * (RF(1.070073e-11) - RF(2.5730207e-13) * L + RF(2.109134e-13) * L * L);
    double t = Np * ne * betaFF * kBoltz() * te / sqrt(te);
    if (!isnan(t)) coolFF = coolFF + t;
    double betaRec = ((double)i / 2.) * (RF(1.06926e-10) - RF(2.41756e-11) * L + RF(1.14542e-12) * L * L -
                                         RF(5.06535e-13) * L * L * L + RF(9.16745e-14) * L * L * L * L);
    t = Np * ne * betaRec * kBoltz() * te / sqrt(te);
    if (!isnan(t)) coolRec = coolRec + t;
  }
  double coolColl;
  if (te > 5000.)
    coolColl = (RF(2.47e-8) * exp(-RF(118338.) / te) * pow(Te4, RF(-0.228)) +
                RF(1.32e-8) * exp(-RF(140252.) / te) * pow(Te4, RF(-0.460))) * kHcRyd() * ionAt(b, c, 1, 1) * ne;
  else
    coolColl = 0.;
  double coolCollH = 0.;
  for (int e = 1; e <= b.nElemUsed; ++e) {
    const int elem = b.zOf[e];
    for (int ion = 1; ion <= min(elem, ns - 1); ++ion)
      coolCollH = coolCollH + (double)b.abun[elem] * ionAt(b, c, elem, ion) * b.coll2[pairOff(b, c, elem, ion)] * ne;
  }
  double heatSte = 0.;
  for (int e = 1; e <= b.nElemUsed; ++e) {
    const int elem = b.zOf[e];
    for (int ion = 1; ion <= min(elem, ns - 1); ++ion) {
      const int p0 = b.pairShell0[(e - 1) * 32 + (ion - 1)];
      const int nsh = b.pairNShell[(e - 1) * 32 + (ion - 1)];
      for (int s = 0; s < nsh; ++s)
        heatSte = heatSte + b.pi2[(size_t)(p0 + s) * C1 + cell] * ionAt(b, c, elem, ion) * (double)b.abun[elem];
    }
  }
  b.coolA[cell] = coolFF + coolRec;
  b.coolHex[cell] = coolColl;
  b.coolCollH[cell] = coolCollH;
  b.heat[cell] = heatSte;
}

// ------------------------------------------------------------- equilibrium

// splint, source/interpolation_mod.f90:286-335
__device__ double splint(const double* xa, const double* ya, const double* y2a, int n, double x) {
  if (x <= xa[0]) return ya[0];
  if (x >= xa[n - 1]) return ya[n - 1];
  int klo = 1, khi = n;
  for (int i = 0; i < 1000; ++i) {
    if (khi - klo <= 1) break;
    int k = (khi + klo) / 2;
    if (xa[k - 1] > x) khi = k; else klo = k;
  }
  double h = xa[khi - 1] - xa[klo - 1];
  double a = (xa[khi - 1] - x) / h;
  double bb = (x - xa[klo - 1]) / h;
  return a * ya[klo - 1] + bb * ya[khi - 1] + ((a * a * a - a) * y2a[klo - 1] + (bb * bb * bb - bb) * y2a[khi - 1]) * (h * h) / 6.;
}

// equilibrium (source/emission_mod.f90:2505-3007) of one atom: returns the sum
// over its lines of a(j,i)*E_ji*n_j*m1*m2*m3 that exceed 1e-35, in the order
// lower level outer, upper level inner (forLines scales the emissivities by
// elemAbun, ionDen and the unit factor, in that order).
__device__ double equilibriumLines(const BalanceDev& b, int atom, double Te, double Ne, double ionDenUp, bool rec,
                                   double m1, double m2, double m3) {
  const int32_t* h = b.atomHdr + (size_t)atom * kAtHdrSize;
  const double* D = b.atomData;
  const int nLev = h[kAtNLev], nT = h[kAtNTemp];
  const double* logT = D + h[kAtOffLogT];
  const double* qom = D + h[kAtOffQom];
  const double* y2 = D + h[kAtOffY2];
  const double* A = D + h[kAtOffA];
  const double* g = D + h[kAtOffG];
  const double* e = D + h[kAtOffE];
  const double atp = D[h[kAtOffAtp]];
  const int iup2p = h[kAtIup2p];
  const double sqrTe = sqrt(Te), log10Te = log10(Te);
  double alphaTotal[kMaxLevels + 1];
  for (int i = 0; i <= nLev; ++i) alphaTotal[i] = 0.;
  if (rec) {
    const double* rr = D + h[kAtOffRec];
    if (h[kAtRecType] == kRecPowerLaw) {
      for (int r = 0; r < h[kAtNRec]; ++r) {
        const double* v = rr + r * 11;
        const int j = r + 2;
        double br = (double)(float)v[0], z = (double)(float)v[1];
        double ar0 = (float)v[2], ar1 = (float)v[3], ar2 = (float)v[4], ar3 = (float)v[5];
        double ad0 = (float)v[6], ad1 = (float)v[7], ad2 = (float)v[8], ad3 = (float)v[9], ad4 = (float)v[10];
        if (z > 0.) {
          double tz = Te * RF(1.e-4) / (z * z);
          double t4 = Te * RF(1.e-4);
          alphaTotal[j] = RF(1.e-13) * br * z * ar0 * pow(tz, ar1) / (1. + ar2 * pow(tz, ar3)) +
                          RF(1.0e-12) * br * (ad0 / t4 + ad1 + ad2 * Te * RF(1.e-4) + ad3 * (t4 * t4)) * pow(t4, -1.5) *
                              exp(-ad4 * RF(1.e4) / Te);
        }
      }
    } else if (h[kAtRecType] == kRecChianti) {
      for (int r = 0; r < h[kAtNRec]; ++r) {
        const double* v = rr + r * 5;
        int jj = (int)v[0];
        double a = (float)v[1], bb = (float)v[2], cc = (float)v[3], d = (float)v[4];
        double L = log10(Te);
        alphaTotal[jj] = pow(10., a + bb * L + cc * (L * L) + d * (L * L * L));
      }
    }
  }
  double qeff[kMaxLevels + 1][kMaxLevels + 1];
  double x[kMaxLevels + 1][kMaxLevels + 1], y[kMaxLevels + 1];
  for (int i = 1; i <= nLev; ++i) {
    y[i] = 0.;
    for (int j = 1; j <= nLev; ++j) { qeff[i][j] = 0.; x[i][j] = 0.; }
  }
  int p = 0;
  for (int i = 2; i <= nLev; ++i) {
    for (int j = i; j <= nLev; ++j, ++p) {
      const double* qq = qom + (size_t)p * nT;
      double cs;
      if (nT == 1) cs = qq[0];
      else if (nT == 2) cs = qq[0] + (qq[1] - qq[0]) / (logT[1] - logT[0]) * (log10Te - logT[0]);
      else cs = splint(logT, qq, y2 + (size_t)p * nT, nT, log10Te);
      const double constant = 1.4388463;
      if (e[i - 2] <= e[j - 1]) {
        double expFac = exp((e[i - 2] - e[j - 1]) * constant / Te);
        qeff[i - 1][j] = 8.63e-6 * cs * expFac / (g[i - 2] * sqrTe);
        qeff[j][i - 1] = 8.63e-6 * cs / (g[j - 1] * sqrTe);
      } else {
        double expFac = exp((e[j - 1] - e[i - 2]) * constant / Te);
        qeff[j][i - 1] = 8.63e-6 * cs * expFac / (g[i - 2] * sqrTe);
        qeff[i - 1][j] = 8.63e-6 * cs / (g[j - 1] * sqrTe);
      }
    }
  }
  for (int j = 1; j <= nLev; ++j) x[1][j] = 1.;
  y[1] = 1.;
  for (int i = 2; i <= nLev; ++i) {
    for (int j = 1; j <= nLev; ++j) {
      if (j != i) {
        x[i][j] = x[i][j] + Ne * qeff[j][i];
        x[i][i] = x[i][i] - Ne * qeff[i][j];
        if (j > i) x[i][j] = x[i][j] + A[(size_t)(j - 1) * nLev + (i - 1)];
        else x[i][i] = x[i][i] - A[(size_t)(i - 1) * nLev + (j - 1)];
      }
    }
    y[i] = -Ne * ionDenUp * alphaTotal[i];
  }
  const int n = nLev;
  if (n > 1) {
    for (int i = 1; i <= n - 1; ++i)
      for (int k = i + 1; k <= n; ++k) {
        double factor = x[k][i] / x[i][i];
        for (int j = i + 1; j <= n; ++j) x[k][j] = x[k][j] - x[i][j] * factor;
      }
    for (int i = 1; i <= n - 1; ++i)
      for (int j = i + 1; j <= n; ++j) y[j] = y[j] - y[i] * x[j][i] / x[i][i];
    y[n] = y[n] / x[n][n];
    for (int i = 1; i <= n - 1; ++i) {
      int k = n - i;
      for (int j = k + 1; j <= n; ++j) y[k] = y[k] - y[j] * x[k][j];
      y[k] = y[k] / x[k][k];
    }
  } else {
    y[1] = y[1] / x[1][1];
  }
  double sumN = 0.;
  for (int i = 1; i <= nLev; ++i) sumN = sumN + y[i];
  for (int i = 1; i <= nLev; ++i) y[i] = y[i] / sumN;
  double total = 0.;
  for (int i = 1; i <= nLev - 1; ++i)
    for (int j = i + 1; j <= nLev; ++j) {
      double aji = A[(size_t)(j - 1) * nLev + (i - 1)];
      if (aji != 0.) {
        double Eji = e[j - 1] - e[i - 1];
        if (j == iup2p && i == 1 && atp > 0.) aji = aji - atp;
        double f = aji * Eji * y[j] * m1 * m2 * m3;
        if (f > RF(1.e-35)) total = total + f;
      }
    }
  return total;
}

// forLines of update_mod (source/update_mod.f90:1221-1262): one thread per (cell, ion with data)
__global__ void __launch_bounds__(128) atomsKernel(BalanceDev b) {
  const int cell = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int atom = blockIdx.y;
  if (cell > b.nCells || b.state[cell] != 0) return;
  const CellIdx c{cell, b.nCells + 1};
  const int32_t* h = b.atomHdr + (size_t)atom * kAtHdrSize;
  const int elem = h[kAtElem], ion = h[kAtIon];
  const int top = min(elem + 1, b.nstages);
  const double x = ionAt(b, c, elem, ion);
  double up = 0.;
  if (ion < top && x > 0.) up = ionAt(b, c, elem, ion + 1) / x;
  // forbiddenLines = fLineEm * elemAbun * ionDen * 1.9865e-16, summed where > 1e-35
  b.forSum[(size_t)atom * c.C1 + cell] =
      equilibriumLines(b, atom, b.te[cell], b.ne[cell], up, false, (double)b.abun[elem], x, RF(1.9865e-16));
}

// The emission phase's forLines (rec = .true., 1e-25 erg units) and normFor
// sum (source/emission_mod.f90:1481-1524, :1780-1795) from the grid state.
__global__ void __launch_bounds__(128) forLinesEmissionKernel(BalanceDev b, const float* __restrict__ te,
                                                              const float* __restrict__ ne,
                                                              const float* __restrict__ ionDen,
                                                              const uint8_t* __restrict__ compute, float* forLines) {
  const int cell = blockIdx.x * blockDim.x + threadIdx.x;
  const int C1 = b.nCells + 1;
  if (cell >= C1 || !compute[cell]) return;
  double normFor = 0.;
  for (int atom = 0; atom < b.nAtoms; ++atom) {
    const int32_t* h = b.atomHdr + (size_t)atom * kAtHdrSize;
    const int elem = h[kAtElem], ion = h[kAtIon];
    const int top = min(elem + 1, b.nstages);
    const int e = b.xref[elem];
    const double x = ionDen[((size_t)(ion - 1) * b.nElemUsed + (e - 1)) * C1 + cell];
    double up = 0.;
    if (ion < top && x > 0.) up = (double)ionDen[((size_t)ion * b.nElemUsed + (e - 1)) * C1 + cell] / x;
    normFor = normFor + equilibriumLines(b, atom, te[cell], ne[cell], up, true, (double)b.abun[elem], x, RF(1.9865e9));
  }
  forLines[cell] = (float)normFor;
}

// heating - cooling, the secant step of iterateT (source/update_mod.f90:349-482)
__global__ void __launch_bounds__(128) secantKernel(BalanceDev b, int lastRound) {
  const int cell = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (cell > b.nCells || b.state[cell] != 0) return;
  const int C1 = b.nCells + 1;
  double coolColl = b.coolHex[cell];
  for (int a = 0; a < b.nAtoms; ++a) coolColl = coolColl + b.forSum[(size_t)a * C1 + cell];
  const double ne = b.ne[cell];
  double heat = b.heat[cell];
  double cool = b.coolA[cell] + coolColl + b.coolCollH[cell];
  if (b.lgCompton) {
    heat = heat + b.compHeat[cell] * ne + b.compRecoil[cell];
    cool = cool + b.compCool[cell] * ne;
  }
  const int nIterateT = b.nIterT[cell];
  const double res = heat - cool;
  double te = b.te[cell];
  double Thigh = b.tHigh[cell], Tlow = b.tLow[cell], resHigh = b.resHigh[cell], resLow = b.resLow[cell];
  bool done = true;
  if (fabs(res) >= RF(0.02) * (fabs(cool) + fabs(heat)) / 2.) {
    if (nIterateT < 20) {
      if (res < 0.) {
        resLow = res;
        Tlow = te;
        if (Thigh != 0.) te = Tlow - (Thigh - Tlow) * resLow / (resHigh - resLow);
        else te = te / RF(1.2);
      } else {
        resHigh = res;
        Thigh = te;
        if (Tlow != 0.) te = Tlow - (Thigh - Tlow) * resLow / (resHigh - resLow);
        else te = te * RF(1.2);
      }
      if (nIterateT >= 6 && fabs(Thigh - Tlow) <= (RF(0.002) * (Thigh + Tlow))) {
        if (res < 0.) { te = Thigh - 100.; Thigh = 0.; }
        else { te = Tlow + 100.; Tlow = 0.; }
      }
      if (te <= 0.) te = 1.;
      done = lastRound != 0;   // a caller-imposed round limit ends the cell here
    } else {
      if (Thigh == 0.) te = Tlow;
      else if (Tlow == 0.) te = Thigh;
      else te = (Thigh + Tlow) * 0.5;
      atomicAdd(&b.counters->noTeBal, 1ull);
    }
  }
  b.te[cell] = te;
  b.tHigh[cell] = Thigh; b.tLow[cell] = Tlow; b.resHigh[cell] = resHigh; b.resLow[cell] = resLow;
  if (done) {
    b.state[cell] = 1;
    if (!b.ibConv[cell]) atomicAdd(&b.counters->noIonBal, 1ull);
  }
}

// Writes the results of the cells back to the grid (FP32) and the flags.
__global__ void storeKernel(BalanceDev b, BalanceGrid g) {
  const int cell = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (cell > b.nCells) return;
  const int C1 = b.nCells + 1;
  const int8_t st = b.state[cell];
  g.black[cell] = st == 2 ? 1 : 0;
  g.nIterT[cell] = st == 2 ? 0 : b.nIterT[cell];
  if (st == 2) {
    g.converged[cell] = 0;
    atomicAdd(&b.counters->noHit, 1ull);
    return;
  }
  g.te[cell] = (float)b.te[cell];
  g.ne[cell] = (float)b.ne[cell];
  const size_t nI = (size_t)b.nstages * b.nElemUsed;
  for (size_t k = 0; k < nI; ++k) g.ionDen[k * C1 + cell] = (float)b.ion[k * C1 + cell];
  const double xH0 = b.ion[(size_t)(b.xref[1] - 1) * C1 + cell];
  const double d = (xH0 - b.xOld[cell]) / b.xOld[cell];
  const int conv = fabs(d) <= (double)b.xhiLimit ? 1 : 0;
  g.converged[cell] = conv;
  atomicAdd(&b.counters->updated, 1ull);
  if (conv) atomicAdd(&b.counters->converged, 1ull);
  atomicMax(&b.counters->maxIterT, (unsigned long long)b.nIterT[cell]);
}

template <typename T>
T* carve(std::vector<void*>& blocks, size_t n, std::string& err) {
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T));
  if (e != cudaSuccess) {
    err = std::string("balance tables: ") + cudaGetErrorString(e);
    return nullptr;
  }
  blocks.push_back(p);
  return (T*)p;
}

}  // namespace

BalanceData::~BalanceData() {
  for (int i = 0; i < nBlocks; ++i)
    if (blocks[i]) cudaFree(blocks[i]);
}

std::string balanceDataCreate(const Setup& s, std::unique_ptr<BalanceData>& out) {
  auto bd = std::make_unique<BalanceData>();
  BalanceDev& d = bd->dev;
  const BalanceTables& t = s.bal;
  const int C1 = s.nCells + 1, ns = s.p.nstages, E = std::max(s.nElemUsed, 1);
  d.nbins = s.nbins; d.nCells = s.nCells; d.nstages = ns; d.nElemUsed = s.nElemUsed;
  d.lgBadnell = s.p.lgBadnell; d.lgCompton = s.p.lgCompton;
  d.secIonP = s.secIonP; d.cRecoilHP = s.cRecoilHP; d.cRecoilHeP = s.cRecoilHeP;
  d.xhiLimit = s.p.XHILimit;
  d.nAtoms = t.nAtoms;
  d.nDiel = (int)(t.diel.size() / 8);
  d.nAldro = (int)(t.aldro.size() / 6);
  if (ns > 31) return "balance: nstages above 31";
  for (int z = 1; z <= 30; ++z) {
    d.xref[z] = s.elemXref[z - 1];
    d.abun[z] = s.elemAbun[z - 1];
    if (s.elemXref[z - 1] > 0) d.zOf[s.elemXref[z - 1]] = z;
  }
  if (d.xref[1] <= 0) return "balance: hydrogen must be on";
  // photoionised shells in the reference's loop order (elem, ion, shell)
  std::vector<PhotoShell> sh;
  for (int i = 0; i < 31 * 32; ++i) { d.pairShell0[i] = -1; d.pairNShell[i] = 0; }
  for (int z = 1; z <= 30; ++z) {
    if (s.elemXref[z - 1] <= 0) continue;
    for (int ion = 1; ion <= std::min(z, ns - 1); ++ion) {
      const int nsh = s.nShells[z - 1][ion - 1];
      d.pairShell0[(s.elemXref[z - 1] - 1) * 32 + (ion - 1)] = (int)sh.size();
      d.pairNShell[(s.elemXref[z - 1] - 1) * 32 + (ion - 1)] = nsh;
      for (int k = 1; k <= nsh; ++k) {
        PhotoShell p{};
        p.elem = z; p.ion = ion; p.shell = k;
        if (z > 2) {
          p.heavy = 1;
          p.ipNuP = s.elementP[z - 1][ion - 1][k - 1][0];
          p.highNuP = s.elementP[z - 1][ion - 1][k - 1][1];
          p.xsecP = s.elementP[z - 1][ion - 1][k - 1][2];
          p.yield1 = t.auger[z - 1][ion - 1][k - 1][0];
        } else {
          p.heavy = 0;
          p.highNuP = s.nbins;
          if (z == 1) { p.ipNuP = s.HlevNuP[0]; p.xsecP = s.HlevXSecP[0]; }
          else if (ion == 1) { p.ipNuP = s.HeIlevNuP[0]; p.xsecP = s.HeISingXSecP[0]; }
          else { p.ipNuP = s.HeIIlevNuP[0]; p.xsecP = s.HeIIXSecP[0]; }
        }
        sh.push_back(p);
      }
    }
  }
  // the outer shell of H and He must have a rate slot
  for (int z = 1; z <= 2; ++z) {
    if (s.elemXref[z - 1] <= 0) continue;
    for (int ion = 1; ion <= std::min(z, ns - 1); ++ion) {
      int os, g0, g1;
      getOuterShell(z, z - ion + 1, os, g0, g1);
      if (os > s.nShells[z - 1][ion - 1]) return "balance: outer shell of H/He has no photoionisation slot";
    }
  }
  d.nShellsTot = (int)sh.size();

  std::vector<void*> blocks;
  std::string err;
  auto up = [&](const void* src, size_t bytes) -> void* {
    void* p = carve<uint8_t>(blocks, bytes, err);
    if (p && bytes) {
      cudaError_t e = cudaMemcpy(p, src, bytes, cudaMemcpyHostToDevice);
      if (e != cudaSuccess) err = std::string("balance tables: ") + cudaGetErrorString(e);
    }
    return p;
  };
  d.nu = (const float*)up(s.nu.data(), s.nu.size() * sizeof(float));
  d.xsec = (const float*)up(s.xSec.data(), s.xSec.size() * sizeof(float));
  std::vector<float> rec = s.xSecRecoil;
  rec.resize(s.nbins, 0.f);
  d.xsecRecoil = (const float*)up(rec.data(), rec.size() * sizeof(float));
  d.shells = (const PhotoShell*)up(sh.data(), sh.size() * sizeof(PhotoShell));
  d.CF = (const float*)up(t.CF, sizeof(t.CF));
  d.cionTherm = (const float*)up(t.cionTherm, sizeof(t.cionTherm));
  d.nauger = (const int32_t*)up(t.nauger, sizeof(t.nauger));
  d.auger = (const float*)up(t.auger, sizeof(t.auger));
  d.RRb = (const float*)up(t.RRb, sizeof(t.RRb));
  d.DRbC = (const float*)up(t.DRbC, sizeof(t.DRbC));
  d.DRbE = (const float*)up(t.DRbE, sizeof(t.DRbE));
  d.rrec = (const float*)up(t.rrec, sizeof(t.rrec));
  d.rnew = (const float*)up(t.rnew, sizeof(t.rnew));
  d.diel = (const float*)up(t.diel.data(), t.diel.size() * sizeof(float));
  d.aldro = (const float*)up(t.aldro.data(), t.aldro.size() * sizeof(float));
  d.outer = (const int32_t*)up(t.outer, sizeof(t.outer));
  d.atomHdr = (const int32_t*)up(t.atomHdr.data(), t.atomHdr.size() * sizeof(int32_t));
  d.atomData = (const double*)up(t.atomData.data(), t.atomData.size() * sizeof(double));
  const size_t nPair = (size_t)E * ns;
  d.ion = carve<double>(blocks, nPair * C1, err);
  d.alpha = carve<double>(blocks, nPair * C1, err);
  d.coll1 = carve<double>(blocks, nPair * C1, err);
  d.coll2 = carve<double>(blocks, nPair * C1, err);
  const size_t nSh = std::max<size_t>(sh.size(), 1);
  d.gam = carve<double>(blocks, nSh * C1, err);
  d.heatA = carve<double>(blocks, nSh * C1, err);
  d.heatHi = carve<double>(blocks, nSh * C1, err);
  d.pi1 = carve<double>(blocks, nSh * C1, err);
  d.pi2 = carve<double>(blocks, nSh * C1, err);
  d.comp = carve<double>(blocks, 4 * (size_t)C1, err);
  double** scal[] = {&d.te, &d.ne, &d.xOld, &d.tHigh, &d.tLow, &d.resHigh, &d.resLow, &d.heat, &d.coolA,
                     &d.coolHex, &d.coolCollH, &d.compHeat, &d.compRecoil, &d.compCool};
  for (double** p : scal) *p = carve<double>(blocks, C1, err);
  d.forSum = carve<double>(blocks, (size_t)std::max(t.nAtoms, 1) * C1, err);
  d.nIterT = carve<int32_t>(blocks, C1, err);
  d.state = carve<int8_t>(blocks, C1, err);
  d.ibConv = carve<int8_t>(blocks, C1, err);
  d.counters = carve<BalanceCounters>(blocks, 1, err);
  if ((int)blocks.size() > (int)(sizeof(bd->blocks) / sizeof(bd->blocks[0]))) err = "balance: too many device blocks";
  for (size_t i = 0; i < blocks.size() && i < sizeof(bd->blocks) / sizeof(bd->blocks[0]); ++i) bd->blocks[i] = blocks[i];
  bd->nBlocks = (int)std::min(blocks.size(), sizeof(bd->blocks) / sizeof(bd->blocks[0]));
  if (!err.empty()) return err;
  // no photon hit until the J pass says otherwise
  cudaMemset(d.state, 2, C1);
  out = std::move(bd);
  return "";
}

cudaError_t launchBalance(BalanceData& bd, const BalanceGrid& g, int maxRounds, cudaStream_t s) {
  BalanceDev& b = bd.dev;
  const int C = b.nCells;
  if (C <= 0) return cudaSuccess;
  const int T = 128, nb = (C + T - 1) / T;
  cudaError_t e = cudaMemsetAsync(b.counters, 0, sizeof(BalanceCounters), s);
  if (e != cudaSuccess) return e;
  photoIntegralsKernel<<<nb, T, 0, s>>>(b, g.jste);
  loadStateKernel<<<nb, T, 0, s>>>(b, g.te, g.ne, g.ionDen);
  const int rounds = std::min(std::max(maxRounds, 1), 20);
  for (int r = 1; r <= rounds; ++r) {
    ratesKernel<<<nb, T, 0, s>>>(b, g.hden);
    if (b.nAtoms > 0) atomsKernel<<<dim3(nb, b.nAtoms), T, 0, s>>>(b);
    secantKernel<<<nb, T, 0, s>>>(b, r == rounds && rounds < 20 ? 1 : 0);
  }
  storeKernel<<<nb, T, 0, s>>>(b, g);
  return cudaGetLastError();
}

cudaError_t launchForLinesEmission(BalanceData& bd, const float* te, const float* ne, const float* ionDen,
                                   const uint8_t* compute, float* forLines, cudaStream_t s) {
  BalanceDev& b = bd.dev;
  const int C1 = b.nCells + 1, T = 128;
  forLinesEmissionKernel<<<(C1 + T - 1) / T, T, 0, s>>>(b, te, ne, ionDen, compute, forLines);
  return cudaGetLastError();
}

}  // namespace mcx
