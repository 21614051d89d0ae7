// k_balance_impl.cuh - device code of the balance phase, compiled twice:
//   k_balance_f64.cu    real = double, --fmad=false: the plain FP64 path that is
//                       checked against the oracle operation by operation; its
//                       exp, log, log10 and pow are the portable routines of
//                       mcx_fmath.h, which the oracle uses too
//   k_balance_mixed.cu  real = float: rates, splines and exponentials in FP32
//                       (the reference's own REAL); the X-iteration loop in
//                       FP32 too (the ionisation ladder on the base-2
//                       logarithms of its products, its normalisation, H/He
//                       ratios and Ne); level populations by FP32 state
//                       reduction (the FP64 LU only for a level without an
//                       exit below it); line cooling read from per-ion cooling
//                       surfaces; only the Te bracketing of the secant step
//                       stays FP64
// The including file defines MCX_BAL_REAL, MCX_BAL_NS and MCX_BAL_EXACT.
//
// Reference routines: updateCell / iterateT (source/update_mod.f90:15-482),
// calcAlpha (:2298-2413), RRbadnell / DRbadnell (:2415-2450), radRecFit
// (:3094-3202), dielectronic (:3204-3305), collisionalIonisation
// (:3552-3582), photoionisation (:3584-3832), compton (:3834-3897),
// getPhotoRates (:3971-4040), ionBalance (:1575-1992), thermBalance
// (:887-1215), forLines (:1221-1262), equilibrium / luSlv
// (source/emission_mod.f90:2505-3106), splint (source/interpolation_mod.f90:286-335).
#include "k_balance.cuh"
#include "k_lines.cuh"
#include "setup_internal.h"
#include "mcx_fmath.h"

#include <algorithm>

namespace mcx {
namespace MCX_BAL_NS {

typedef MCX_BAL_REAL real;

#if MCX_BAL_EXACT
// Unqualified exp / log / log10 / pow calls of this namespace resolve here
// (before the global CUDA overloads): the portable routines shared with the
// oracle, so that both round alike and take the same branches.
__host__ __device__ __forceinline__ double exp(double x) { return mcx_fm_exp(x); }
__host__ __device__ __forceinline__ double log(double x) { return mcx_fm_log(x); }
__host__ __device__ __forceinline__ double log10(double x) { return mcx_fm_log10(x); }
__host__ __device__ __forceinline__ double pow(double x, double y) { return mcx_fm_pow(x, y); }
#endif

// a default-REAL constant of the reference, at its single-precision value, in
// the rate precision (RF) or in FP64 (RD)
#define RF(x) ((real)(x##f))
#define RD(x) ((double)(x##f))

__device__ __forceinline__ real kBoltz() { return RF(1.380658e-16); }    // constants_mod.f90:18
__device__ __forceinline__ real kRyd2erg() { return RF(2.1799e-11); }   // constants_mod.f90:20
__device__ __forceinline__ real kHcRyd() { return RF(2.1799153e-11); }  // update_mod.f90:64
__device__ __forceinline__ double kXMax() { return RD(0.99999); }       // constants_mod.f90:57

constexpr int kNE = 30;
// mixed precision: ions with elemAbun * ionDen below this skip the atom solve
// (their forbidden lines carry below 1e-7 of any cell's cooling)
constexpr double kNegligibleIon = 1e-12;

struct CellIdx {
  int cell, C1;
};

// The rates kernel gives each cell a group of kGroup lanes (kCellsPerWarp
// cells per warp): the per-ion and per-shell loops stride over the group, the
// ladders of the heavy elements run one per lane, and the sums in the
// reference's order run on the group's first lane, four cells at a time.
constexpr int kGroup = 8, kCellsPerWarp = 32 / kGroup;

#if !MCX_BAL_EXACT
__device__ CoolAt coolStencil(double te, double ne);
__device__ __forceinline__ float2 surfaceAt(const float* tab, int atom, const CoolAt& a);
#endif
struct Lanes {
  int gl;           // lane within the cell's group
  unsigned mask;    // the group's lanes in the warp
};

__device__ __forceinline__ double& ionAt(const BalanceDev& b, const CellIdx& c, int z, int st) {
  return b.ion[((size_t)(st - 1) * b.nElemUsed + (b.xref[z] - 1)) * c.C1 + c.cell];
}

// ------------------------------------------------------------- rate functions

__device__ real rrBadnell(const BalanceDev& b, real te, int elem, int nel) {
  const float* t = b.RRb;
  auto RB = [&](int k) { return (real)t[((size_t)k * kNE + (elem - 1)) * (kNE + 1) + nel]; };
  real A = RB(0), B = RB(1), T0 = RB(2), T1 = RB(3), Cc = RB(4), T2 = RB(5);
  real bbad = B + Cc * exp(-T2 / te);
  const real h = (real)0.5, one = (real)1.;
  return A / (pow(te / T0, h) * pow(one + pow(te / T0, h), one - bbad) * pow(one + pow(te / T1, h), one + bbad));
}

__device__ real drBadnell(const BalanceDev& b, real te, int elem, int nel) {
  real dr = 0;
  const float* E = b.DRbE + ((size_t)(elem - 1) * (kNE + 1) + nel) * 9;
  const float* Cc = b.DRbC + ((size_t)(elem - 1) * (kNE + 1) + nel) * 9;
  for (int idr = 0; idr < 9; ++idr)
    if ((real)E[idr] / te < (real)87.) dr = dr + (real)Cc[idr] * exp(-(real)E[idr] / te);
  return dr * pow(te, (real)-1.5);
}

__constant__ float kFeFit[3][10] = {
    {4.33e-10f, 3.91e-10f, 3.49e-10f, 3.16e-10f, 2.96e-10f, 2.59e-10f, 2.24e-10f, 1.91e-10f, 1.68e-10f, 1.46e-10f},
    {0.531f, 0.523f, 0.521f, 0.534f, 0.557f, 0.567f, 0.579f, 0.601f, 0.602f, 0.597f},
    {5.77e-02f, 6.15e-02f, 6.22e-02f, 6.02e-02f, 5.79e-02f, 5.65e-02f, 5.49e-02f, 5.10e-02f, 5.07e-02f, 5.22e-02f}};

__device__ real radRecFit(const BalanceDev& b, real te, int z, int n) {
  const real one = (real)1.;
  if ((n <= 3) || (n == 11) || ((z > 5) && (z < 9)) || (z == 10) || ((z == 26) && (n > 11))) {
    const float* r = b.rnew + ((size_t)(z - 1) * kNE + (n - 1)) * 4;
    real tt = sqrt(te / (real)r[2]);
    return (real)r[0] / (tt * pow(tt + one, one - (real)r[1]) * pow(one + sqrt(te / (real)r[3]), one + (real)r[1]));
  }
  real tt = te * RF(1.e-4);
  if ((z == 26) && (n <= 13))
    return (real)kFeFit[0][n - 4] / pow(tt, (real)kFeFit[1][n - 4] + (real)kFeFit[2][n - 4] * log10(tt));
  const float* r = b.rrec + ((size_t)(z - 1) * kNE + (n - 1)) * 2;
  return (real)r[0] / pow(tt, (real)r[1]);
}

// diRec(elem, ion) of dielectronic: the last row of dielectronic.dat for
// (elem, ion) whose temperature flag applies, or above 6e4 K the last row of
// aldrovandi.dat (the whole diRec array is replaced there).  The row indices
// are found at set-up (dielRow: last row with flag 0 or 1, with flag 0 or 2,
// and the aldrovandi row; -1 none).
__device__ real diRecOf(const BalanceDev& b, real te, int elem, int ion) {
  if (ion > b.nstages || elem < 1 || elem > 30 || ion < 1 || ion > 31) return 0;
  const real one = (real)1.;
  const int16_t* idx = b.dielRow + ((size_t)elem * 32 + ion) * 3;
  if (te > (real)60000.) {
    const int r = idx[2];
    if (r < 0) return 0;
    const float* d = b.aldro + (size_t)r * 6;
    real a = d[2], bb = d[3], t0 = d[4], t1 = d[5];
    return a * pow(te, (real)-1.5) * exp(-t0 / te) * (one + bb * exp(-t1 / te));
  }
  real t = te > (real)1000. ? te / (real)10000. : RF(0.1);
  const int r = te < (real)20000. ? idx[0] : idx[1];
  if (r < 0) return 0;
  const float* d = b.diel + (size_t)r * 8;
  real a = d[2], bb = d[3], cc = d[4], dd = d[5], f = d[6];
  return RF(1e-12) * (a / t + bb + cc * t + dd * (t * t)) * pow(t, (real)-1.5) * exp(-f / t);
}

// calcAlpha of one (element, ion) pair (source/update_mod.f90:2298-2413)
__device__ real alphaOf(const BalanceDev& b, real te, int elem, int ion) {
  real a;
  if (b.lgBadnell) {
    int nel = elem - ion;
    if (nel <= 11) {
      a = rrBadnell(b, te, elem, nel);
      a = a + drBadnell(b, te, elem, nel);
    } else {
      a = radRecFit(b, te, elem, elem - ion + 1);
      real di = diRecOf(b, te, elem, ion);
      if (di == (real)0. && ion < 7 && b.xref[8] > 0) di = diRecOf(b, te, 8, ion);
      a = a + (di > (real)0. ? di : (real)0.);
    }
  } else {
    a = radRecFit(b, te, elem, elem - ion + 1);
    if (elem >= 3) {
      real di = diRecOf(b, te, elem, ion);
      if (di == (real)0. && ion < 7) di = diRecOf(b, te, 8, ion);
      a = a + (di > (real)0. ? di : (real)0.);
    }
  }
  return a;
}

#if !MCX_BAL_EXACT
__device__ __forceinline__ void lagrange4(float t, float* w);

// ln alphaTotal of pair k = (e - 1) * nstages + (ion - 1) at the nodes of its
// table, and the jump flags: an interval whose midpoint and quarter points the
// interpolant misses by more than 1e-5 holds a switch of the fits
__global__ void __launch_bounds__(128) alphaTableKernel(BalanceDev b, float* tab) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, k = blockIdx.y;
  if (i >= kAlphaN) return;
  const int e = k / b.nstages + 1, ion = k % b.nstages + 1;
  const int elem = b.zOf[e];
  const double h = (kAlphaLnT1 - kAlphaLnT0) / (kAlphaN - 1);
  const real a = ion <= min(b.nstages - 1, elem) ? alphaOf(b, (real)exp(kAlphaLnT0 + i * h), elem, ion) : (real)0.;
  tab[(size_t)k * kAlphaN + i] = a > 0.f ? logf(a) : -1.e30f;
}
__global__ void __launch_bounds__(128) alphaJumpKernel(BalanceDev b, const float* tab, uint8_t* jump) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, k = blockIdx.y;
  if (i >= kAlphaN) return;
  const int e = k / b.nstages + 1, ion = k % b.nstages + 1;
  const int elem = b.zOf[e];
  uint8_t bad = 1;
  if (i >= 1 && i + 2 < kAlphaN && ion <= min(b.nstages - 1, elem)) {
    const float* t = tab + (size_t)k * kAlphaN + (i - 1);
    bad = 0;
    if (t[0] < -1.e29f || t[1] < -1.e29f || t[2] < -1.e29f || t[3] < -1.e29f) bad = 1;
    const double h = (kAlphaLnT1 - kAlphaLnT0) / (kAlphaN - 1);
    for (int q = 1; q <= 3 && !bad; ++q) {
      const float f = 0.25f * q;
      float w[4];
      lagrange4(f, w);
      const float lnA = w[0] * t[0] + w[1] * t[1] + w[2] * t[2] + w[3] * t[3];
      const real ex = alphaOf(b, (real)exp(kAlphaLnT0 + (i + f) * h), elem, ion);
      if (!(ex > 0.f) || fabsf(expf(lnA - logf(ex)) - 1.f) > 1.e-5f) bad = 1;
    }
  }
  jump[(size_t)k * kAlphaN + i] = bad;
}

// alphaTotal of pair k at Te from the table (direct where the table cannot serve)
__device__ __forceinline__ real alphaLookup(const BalanceDev& b, int k, real teR, int elem, int ion) {
  const float s = (logf(teR) - (float)kAlphaLnT0) * (float)((kAlphaN - 1) / (kAlphaLnT1 - kAlphaLnT0));
  const int i = (int)s;
  if (s >= 1.f && i + 2 < kAlphaN && !b.alphaJump[(size_t)k * kAlphaN + i]) {
    const float* t = b.alphaTab + (size_t)k * kAlphaN + (i - 1);
    float w[4];
    lagrange4(s - (float)i, w);
    const float ref = __ldg(t + 1);
    return expf(ref) * expf(w[0] * (__ldg(t) - ref) + w[2] * (__ldg(t + 2) - ref) + w[3] * (__ldg(t + 3) - ref));
  }
  return alphaOf(b, teR, elem, ion);
}
#endif

// chex(z, ion, 1) * 1e-9 without the temperature fit (ionBalance's heavy elements)
__device__ __forceinline__ real chexRaw(const BalanceDev& b, int z, int ion) {
  return (real)b.chex[z * 32 + ion].x * RF(1.e-9);
}
// chex(z, ion, 1) at Te (source/update_mod.f90:1711-1720, :3788-3797)
__device__ real chexFit(const BalanceDev& b, int z, int ion, real te) {
  const float4 x = b.chex[z * 32 + ion];
  real a = (real)x.x * RF(1.e-9);
  real t4 = te / (real)10000.;
  real v = (te < (real)6000. || te > (real)5.e4) ? (real)0.
                                                 : a * pow(t4, (real)x.y) * ((real)1. + (real)x.z * exp((real)x.w * t4));
  return v < (real)0. ? (real)0. : v;
}

__device__ __forceinline__ const int32_t* outerOf(const BalanceDev& b, int z, int nElec) {
  return b.outer + ((size_t)(z - 1) * kNE + (nElec - 1)) * 3;
}

// ------------------------------------------------------ J-only integrals

// The parts of photoionisation / getPhotoRates / compton that depend on J
// alone.  hitComptonKernel (one thread per cell) marks the cells no packet
// reached and forms the Compton sums; shellIntegralsKernel (one thread per
// (cell, photoionised shell), the shell fastest in the block index) integrates J
// over each shell's cross section, so that a warp streams one shell's bins of
// 32 neighbouring cells' J rows.
__global__ void __launch_bounds__(128) hitComptonKernel(BalanceDev b, const double* __restrict__ jste) {
  const int cell = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (cell > b.nCells) return;
  const int C1 = b.nCells + 1;
  const float* nu = b.nu;
  auto J = [&](int bin1) { return (real)jste[(size_t)(bin1 - 1) * C1 + cell]; };
  // any J > 0, eight bins in flight at a time
  bool hit = false;
  for (int i0 = 1; i0 <= b.nbins && !hit; i0 += 8) {
    double v[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) v[k] = i0 + k <= b.nbins ? __ldg(jste + (size_t)(i0 + k - 1) * C1 + cell) : 0.;
#pragma unroll
    for (int k = 0; k < 8; ++k) hit = hit || v[k] > 0.;
  }
  if (b.evalMask && !b.evalMask[cell]) hit = false;
  b.state[cell] = hit ? 0 : 2;
  if (!hit) return;
  b.list[atomicAdd(&b.listCount[0], 1u)] = cell;   // the cells of the first T-iteration
  if (b.lgCompton) {
    real s1 = 0, s2 = 0, rhH = 0, rhHe = 0;
#pragma unroll 4
    for (int i = 1; i <= b.nbins; ++i) {
      real rf = J(i);
      s1 = s1 + rf;
      s2 = s2 + rf / (real)nu[i - 1];
      if (i > b.cRecoilHP) {
        real energy = RF(2.66e-5) * (real)nu[i - 1] * (real)nu[i - 1] - (real)1.;
        rhH = rhH + (real)b.xsecRecoil[i - 1] * rf * energy;
      }
      if (i > b.cRecoilHeP) {
        real energy = RF(2.66e-5) * (real)nu[i - 1] * (real)nu[i - 1] - RF(1.8);
        rhHe = rhHe + (real)b.xsecRecoil[i - 1] * rf * energy;
      }
    }
    b.comp[0 * (size_t)C1 + cell] = s1 * kRyd2erg();
    b.comp[1 * (size_t)C1 + cell] = s2;
    b.comp[2 * (size_t)C1 + cell] = rhH;
    b.comp[3 * (size_t)C1 + cell] = rhHe;
  }
}

__global__ void __launch_bounds__(128) shellIntegralsKernel(BalanceDev b, const double* __restrict__ jste) {
  // the shells of one block of cells launch next to each other, so their J rows are read from L2
  const int t = (int)(blockIdx.x % (unsigned)b.nShellsTot);
  const int cell = (int)(blockIdx.x / (unsigned)b.nShellsTot) * blockDim.x + threadIdx.x + 1;
  if (cell > b.nCells || b.state[cell] == 2) return;
  const int C1 = b.nCells + 1;
  const float* nu = b.nu;
  const float* xs = b.xsec;
  auto J = [&](int bin1) { return (real)jste[(size_t)(bin1 - 1) * C1 + cell]; };
  const real hcRyd = kHcRyd();
  const PhotoShell sh = b.shells[t];
  const size_t o = (size_t)t * C1 + cell;
  if (sh.ipNuP < 1 || sh.ipNuP > b.nbins) {   // threshold outside the mesh
    b.gam[o] = sh.heavy ? 0. : RD(1.e-20);
    b.heatA[o] = 0.;
    b.heatHi[o] = 0.;
    return;
  }
  if (!sh.heavy) {
    real n1 = RF(1.e-20), h1 = 0;
    const real nuIP = (real)nu[sh.ipNuP - 1];
    for (int j = sh.ipNuP; j <= sh.highNuP; ++j) {
      real ph = xs[j - sh.ipNuP + sh.xsecP - 1];
      if (ph < RF(1.e-35)) ph = 0;
      real jj = J(j);
      if (jj > (real)0.) {
        n1 = n1 + jj * ph / (hcRyd * (real)nu[j - 1]);
        h1 = h1 + ph * jj * ((real)nu[j - 1] - nuIP) / (real)nu[j - 1];
      }
    }
    b.gam[o] = n1;
    b.heatA[o] = h1;
    b.heatHi[o] = 0.;
    return;
  }
  const int nu1P = sh.ipNuP, IPnuP = sh.ipNuP;
  const int iup = min(sh.highNuP, b.nbins);
  const real augerE = hcRyd * (real)nu[nu1P - 1] * (real)sh.yield1;
  real g = 0, h = 0;
  const int top = min(iup, b.secIonP - 1);
  for (int i = nu1P + 1; i <= top; ++i) {
    real jj = J(i);
    if (jj > (real)0.) {
      real ph = xs[i + sh.xsecP - IPnuP - 1];
      if (ph < RF(1.e-35)) ph = 0;
      g = g + jj * ph / (hcRyd * (real)nu[i - 1]);
      h = h + jj * ph;
    }
  }
  h = h - g * augerE;
  const real jIP = J(IPnuP);
  const real ph0 = xs[sh.xsecP - 1];
  g = g + jIP * ph0 / (hcRyd * (real)nu[IPnuP - 1]);
  h = h + jIP * ph0 * (hcRyd * (real)nu[IPnuP - 1] - augerE) / (hcRyd * (real)nu[IPnuP - 1]);
  real gh = 0, hh = 0;
#if MCX_BAL_EXACT
  const int ilow = max(IPnuP + 1, b.secIonP);
  for (int i = ilow; i <= iup; ++i) {
    real p = xs[i + sh.xsecP - IPnuP - 1];
    gh = gh + jIP * p / (hcRyd * (real)nu[i - 1]);   // radField(IPnuP), as the reference
    hh = hh + jIP * p;
  }
#else
  // the same sums with radField(IPnuP) taken out of them (summed once at set-up)
  gh = jIP * (real)b.shellTail[2 * t];
  hh = jIP * (real)b.shellTail[2 * t + 1];
#endif
  g = g + gh;
  hh = hh - gh * augerE;
  b.gam[o] = g;
  b.heatA[o] = h;
  b.heatHi[o] = hh;
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
  b.side[cell] = 0;
}

// -------------------------------------------------------------- one round

// One cell per warp.  The cell's ionic fractions, recombination and
// collisional rates and photoionisation rates sit in the warp's slice of
// shared memory for the whole T-iteration, so the ionisation-balance
// X-iterations read nothing from global memory; the lanes share the per-ion
// and per-shell work (calcAlpha, collisionalIonisation, the photoionisation
// rates) and, inside each X-iteration, lane h runs the ionisation ladder of
// the h-th heavy element.  Every sum keeps the reference's order (one lane
// adds the terms in sequence), so the FP64 build matches the sequential code
// operation for operation.
// Per-element tables of the used elements, copied to shared memory once per
// block: the lanes of a warp index them by different elements at once, which
// the kernel-parameter (constant) bank would serialise.
struct ElemMeta {
  const int32_t* zOf;     // [32] Z of used element e
  const int32_t* xref;    // [32] e of Z (0 = off)
  const float* abun;      // [32] elemAbun by Z
  const int16_t* p0;      // [E][32] first photoionised shell of (e, ion)
  const int16_t* nsh;     // [E][32] its number of shells
};

// In the rate precision: FP64 in the plain build; FP32 in the mixed build,
// whose X-iterations then run without an FP64 instruction (GB300 issues FP64
// at 1/64 of the FP32 rate, and the loop is a long dependent chain).
struct WarpCell {
  real* X;       // [S][E] ionic fractions at (st-1)*E + (e-1), the global ionDen order
  real* AL;      // [E][S] alphaTotal at (e-1)*S + (ion-1)
  real* CC;      // [E][S] collisional ionisation rate coefficient (coll1)
  real* PI;      // [nShellsTot] photoIon(1): rate per shell, with the reverse charge exchange
  real* T;       // scratch for ordered sums
  real* LAD;     // [nHeavy][3][S+3] out, inn, mat of the ladders; later the thermBalance terms [4][E]
  real* AUG;     // mixed build: [nHeavy][13 (S+1)] per heavy element the sums over shells of the
                 // photoionisation rate per ion, charge exchange per ion, the Auger band
                 // A[ion][d] = sum of photoIon * auger feeding ion + d, and per ion the mask of
                 // the d with A[ion - d][d] != 0
};

__device__ __forceinline__ real& xAt(const BalanceDev& b, const ElemMeta& m, const WarpCell& w, int z, int st) {
  return w.X[(st - 1) * b.nElemUsed + (m.xref[z] - 1)];
}

// ionBalance (source/update_mod.f90:1575-1992; the recursion as a loop) for
// the warp's cell; returns lgConv (uniform across the warp).  In the mixed
// build the ladder runs on the logarithms of its products (FP32 cannot hold
// the products themselves).
__device__ bool ionBalanceWarp(const BalanceDev& b, const ElemMeta& m, const WarpCell& w, const Lanes& L, double te,
                               double& ne, double hden) {
  const int ns = b.nstages, E = b.nElemUsed;
  const int zH = 1, zHe = 2;
  const bool heOn = m.xref[zHe] > 0;
  const real teR = (real)te;
  // the Te-only terms are the same on every X-iteration (the reference
  // recomputes them on each recursive call)
  real expFact = RF(157893.94) / teR;
  if (expFact > (real)75.) expFact = (real)75.;
  const real collIonH0 = RF(2.75E-16) * teR * sqrt(teR) * (RF(157893.94) / teR + (real)2.) * exp(-expFact);
  const real hdenR = (real)hden;
  real neR = (real)ne;
  real cxHHe[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  real piHHe[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};   // the outer shell's photoionisation rate
  if (L.gl < 2)
    for (int elem = 1; elem <= 2; ++elem)
      for (int ion = 1; ion <= min(elem, ns - 1); ++ion) {
        cxHHe[elem][ion] = chexFit(b, elem, ion, teR);
        if (m.xref[elem]) {
          const int outShell = outerOf(b, elem, elem - ion + 1)[0];
          piHHe[elem][ion] = w.PI[m.p0[(m.xref[elem] - 1) * 32 + (ion - 1)] + outShell - 1];
        }
      }
  // this lane's heavy elements (the h-th element with Z >= 3, in element order,
  // for h = gl, gl + kGroup, ...; at most 32 heavy elements)
  int myE[32 / kGroup] = {}, myH[32 / kGroup] = {};
  int nMine = 0;
  for (int e = 1, h = 0; e <= E; ++e)
    if (m.zOf[e] >= 3) {
      if (h % kGroup == L.gl && nMine < 32 / kGroup) {
        myE[nMine] = e;
        myH[nMine++] = h;
      }
      ++h;
    }
#if !MCX_BAL_EXACT
  // the parts of the ladders' out and inn terms that stay put over the X-iterations: the
  // photoionisation rates summed per ion, the Auger terms summed per (ion, ion + d) (each is
  // multiplied by X(ion) / X(ion + d) in the X-iteration), the charge-exchange coefficients
  for (int q = 0; q < nMine; ++q) {
    const int e = myE[q], h = myH[q];
    const int elem = m.zOf[e];
    real* S = w.AUG + (size_t)h * 13 * (ns + 1);
    real* CH = S + (ns + 1);
    real* A = CH + (ns + 1);
    unsigned* feed = reinterpret_cast<unsigned*>(A + 10 * (ns + 1));   // [ion]: bit d set if A[ion - d][d] != 0
    const int topI = min(elem, ns - 1), lim = min(ns - 1, elem);
    for (int k = 0; k < 13 * (ns + 1); ++k) S[k] = 0;
    for (int ion = 1; ion <= topI; ++ion) {
      CH[ion] = chexRaw(b, elem, ion);
      const int p0 = m.p0[(e - 1) * 32 + (ion - 1)];
      const int nsh = m.nsh[(e - 1) * 32 + (ion - 1)];
      for (int shell = 1; shell <= nsh; ++shell) {
        const real pi = w.PI[p0 + shell - 1];
        S[ion] = S[ion] + pi;
        const int nAug = b.nauger[((size_t)(elem - 1) * kNE + (ion - 1)) * 10 + (shell - 1)];
        for (int nelec = 2; nelec <= nAug; ++nelec) {
          const int maxim = min(ion + nelec - 1, lim);
          A[ion * 10 + (maxim - ion)] +=
              pi * (real)b.auger[(((size_t)(elem - 1) * kNE + (ion - 1)) * 10 + (shell - 1)) * 10 + (nelec - 1)];
        }
      }
    }
    for (int t = 1; t <= topI; ++t) {
      unsigned mask = 0u;
      for (int d = 0; d <= 9 && d < t; ++d)
        if (A[(t - d) * 10 + d] != (real)0.) mask |= 1u << d;
      feed[t] = mask;
    }
  }
#endif
  for (int nIterateX = 1;; ++nIterateX) {
    bool lgConv = true;
    const real HIOld = xAt(b, m, w, zH, 1);
    const real HeIOld = heOn ? xAt(b, m, w, zHe, 1) : (real)0.;
    const real HeIIOld = heOn ? xAt(b, m, w, zHe, 2) : (real)0.;
    __syncwarp(L.mask);
    // H on the group's first lane, He on its second (independent of each other within an X-iteration)
    if (L.gl < 2 && m.xref[L.gl + 1]) {
      const int elem = L.gl + 1;
      real ionRatio[3] = {0, 0, 0};
      real ionProd[3] = {1, 1, 1};
      real den = 1;
      real collIonH = collIonH0;
      for (int ion = 1; ion <= min(elem, ns - 1); ++ion) {
        real cx = cxHHe[elem][ion];
        if (elem > 1 || ion > 1) collIonH = 0;
        real pi = piHHe[elem][ion];
        const real num = pi + collIonH * neR + (real)0.;
        const real dnm = neR * w.AL[(m.xref[elem] - 1) * ns + (ion - 1)] + cx * hdenR * HIOld;
        ionRatio[ion] = num / dnm;
      }
      for (int ion = 1; ion <= min(elem, ns - 1); ++ion)
        for (int i = 1; i <= ion; ++i) ionProd[ion] = ionProd[ion] * ionRatio[i];
      for (int ion = 1; ion <= min(elem, ns - 1); ++ion) den = den + ionProd[ion];
      for (int ion = 1; ion <= min(elem + 1, ns); ++ion) {
        real v = ion == 1 ? (real)1. / den : ionProd[ion - 1] / den;
        if (v > (real)kXMax()) v = (real)kXMax();
        if (v < (real)RD(1.e-20)) v = (real)RD(1.e-20);
        xAt(b, m, w, elem, ion) = v;
      }
    }
    __syncwarp(L.mask);
    // X(H0) as just updated above (grid%ionDen in the reference)
    const real xH0now = xAt(b, m, w, zH, 1);
    for (int q = 0; q < nMine; ++q) {
      const int e = myE[q], h = myH[q];
      const int elem = m.zOf[e];
      typedef real lad;
#if MCX_BAL_EXACT
      lad* out = w.LAD + (size_t)h * 3 * (ns + 3);
      lad* inn = out + (ns + 3);
      real* mat = inn + (ns + 3);
#else
      real* mat = w.LAD + (size_t)h * (ns + 3);   // the running logs only
#endif
      const int topI = min(elem, ns - 1);
#if MCX_BAL_EXACT
      for (int k = 0; k < ns + 3; ++k) { out[k] = 0; inn[k] = 0; }
      const int lim = min(ns - 1, elem);
      for (int ion = 1; ion <= topI; ++ion) {
        out[ion] = out[ion] + w.CC[(e - 1) * ns + (ion - 1)] * neR;
        const int p0 = m.p0[(e - 1) * 32 + (ion - 1)];
        const int nsh = m.nsh[(e - 1) * 32 + (ion - 1)];
        for (int shell = 1; shell <= nsh; ++shell) {
          const lad pi = w.PI[p0 + shell - 1];
          out[ion] = out[ion] + pi;
          const int nAug = b.nauger[((size_t)(elem - 1) * kNE + (ion - 1)) * 10 + (shell - 1)];
          for (int nelec = 2; nelec <= nAug; ++nelec) {
            int maxim = min(ion + nelec - 1, lim);
            real xm = xAt(b, m, w, elem, maxim);
            real ratio = xm > (real)1e-30 ? xAt(b, m, w, elem, ion) / xm : (real)1.;
            out[maxim] = out[maxim] +
                         pi * (lad)b.auger[(((size_t)(elem - 1) * kNE + (ion - 1)) * 10 + (shell - 1)) * 10 + (nelec - 1)] * ratio;
          }
        }
      }
      for (int ion = 1; ion <= topI; ++ion)
        inn[ion] = neR * w.AL[(e - 1) * ns + (ion - 1)] + chexRaw(b, elem, ion) * hdenR * xH0now;
#endif
      const int top = min(ns, elem + 1);
#if MCX_BAL_EXACT
      mat[1] = 1.;
      double sumMat = 1.;
      for (int ion = 2; ion <= top; ++ion) {
        mat[ion] = mat[ion - 1] * out[ion - 1] / inn[ion - 1];
        sumMat = sumMat + mat[ion];
      }
      sumMat = 1. / sumMat;
      xAt(b, m, w, elem, top) = mat[top] * sumMat;
      for (int ion = 1; ion <= topI; ++ion) {
        double v;
        if (nIterateX < 2 && mat[ion] * sumMat > 0.) {
          double old = xAt(b, m, w, elem, ion);
          if (old <= 0.) old = RD(1.e-5);
          v = pow(10., 0.5 * (log10(old) + log10(mat[ion] * sumMat)));
        } else {
          v = mat[ion] * sumMat;
        }
        if (v > kXMax()) v = kXMax();
        if (v < RD(1.e-20)) v = RD(1.e-20);
        xAt(b, m, w, elem, ion) = v;
      }
#else
      // the same ladder in FP32 on log2 of the products (the products span far
      // more than FP32's range; their logarithms do not), normalised against
      // the largest term; the first X-iteration's geometric mean is the mean
      // of the logarithms
      // one pass over the stages: out (collisional and photoionisation, the Auger electrons of
      // the lower stages ion - d into ion, times X(ion - d) / X(ion)) and inn of each stage, and
      // the running log of the ladder's product
      const real* S = w.AUG + (size_t)h * 13 * (ns + 1);
      const real* CH = S + (ns + 1);
      const real* A = CH + (ns + 1);
      const unsigned* feed = reinterpret_cast<const unsigned*>(A + 10 * (ns + 1));
      const real* XE = w.X + (e - 1);   // X of this element's stage ion at XE[(ion - 1) * E]
      float* lm = mat;
      lm[1] = 0.f;
      float lmax = 0.f, lcur = 0.f;
      for (int ion = 1; ion <= topI; ++ion) {
        const real xi = XE[(ion - 1) * E];
        real o = w.CC[(e - 1) * ns + (ion - 1)] * neR + S[ion];
        for (unsigned mk = feed[ion]; mk; mk &= mk - 1u) {   // the stages ion - d feeding ion (d = 0: clamped at lim)
          const int d = __ffs(mk) - 1;
          o = o + A[(ion - d) * 10 + d] * (xi > (real)1e-30 ? __fdividef(XE[(ion - d - 1) * E], xi) : (real)1.);
        }
        const real in_ = neR * w.AL[(e - 1) * ns + (ion - 1)] + CH[ion] * hdenR * xH0now;
        lcur = lcur + log2f(__fdividef(o, in_));
        lm[ion + 1] = lcur;
        lmax = fmaxf(lmax, lcur);
      }
      float sum = 0.f;
      for (int ion = 1; ion <= top; ++ion) sum += exp2f(lm[ion] - lmax);
      const float lsum = lmax + log2f(sum);
      xAt(b, m, w, elem, top) = exp2f(lm[top] - lsum);
      for (int ion = 1; ion <= topI; ++ion) {
        const float lx = lm[ion] - lsum;
        float v;
        if (nIterateX < 2 && lx > -1.e30f) {
          float old = xAt(b, m, w, elem, ion);
          if (old <= 0.f) old = 1.e-5f;
          v = exp2f(0.5f * (log2f(old) + lx));
        } else {
          v = exp2f(lx);
        }
        if (v > 0.99999f) v = 0.99999f;
        if (v < 1.e-20f) v = 1.e-20f;
        xAt(b, m, w, elem, ion) = v;
      }
#endif
    }
    __syncwarp(L.mask);
#if MCX_BAL_EXACT
    // Ne in the reference's order, by the group's first lane
    real nE = 0;
    if (L.gl == 0) {
      for (int e = 1; e <= E; ++e) {
        const int elem = m.zOf[e];
        for (int ion = 2; ion <= min(elem + 1, ns); ++ion) {
          real x = xAt(b, m, w, elem, ion);
          if (x >= (real)RD(1.e-10)) nE = nE + (real)(ion - 1) * (real)m.abun[elem] * x;
        }
      }
      nE = nE * hdenR;
      if (nE == (real)0.) nE = 1;
    }
    neR = __shfl_sync(L.mask, nE, 0, kGroup);
#else
    // Ne: the (element, stage) terms strided over the group's lanes, then a butterfly sum
    real nE = 0;
    for (int k = L.gl; k < E * ns; k += kGroup) {
      const int e = k / ns + 1, ion = k % ns + 1;
      const int elem = m.zOf[e];
      if (ion < 2 || ion > min(elem + 1, ns)) continue;
      const real x = w.X[(ion - 1) * E + (e - 1)];
      if (x >= (real)RD(1.e-10)) nE = nE + (real)(ion - 1) * (real)m.abun[elem] * x;
    }
#pragma unroll
    for (int o = kGroup / 2; o > 0; o >>= 1) nE += __shfl_xor_sync(L.mask, nE, o, kGroup);
    nE = nE * hdenR;
    if (nE == (real)0.) nE = 1;
    neR = nE;
#endif
    ne = (double)neR;
    real dHI = (xAt(b, m, w, zH, 1) - HIOld) / HIOld;
    real dHeI = heOn ? (xAt(b, m, w, zHe, 1) - HeIOld) / HeIOld : (real)0.;
    real dHeII = heOn ? (xAt(b, m, w, zHe, 2) - HeIIOld) / HeIIOld : (real)0.;
    const real lim = (real)b.xTol;
    bool big = fabs(dHI) > lim || fabs(dHeI) > lim || fabs(dHeII) > lim;
    if (big && nIterateX < 15) continue;
    if (big && nIterateX == 15) lgConv = false;
    return lgConv;
  }
}

// calcAlpha, photoionisation, collisionalIonisation, compton, ionBalance and
// the thermBalance terms without forLines, kGroup lanes per iterating cell
// (b.cellReals values of the rate precision in shared memory per cell).
// One listed cell of the rates kernel on its group of lanes.
__device__ __forceinline__ void ratesCell(const BalanceDev& b, const float* __restrict__ hdenG, int round, int li,
                                          const ElemMeta& m, const Lanes& L, double* wsm, int slot) {
  const int C1 = b.nCells + 1, ns = b.nstages, E = b.nElemUsed, NP = E * ns, nSh = b.nShellsTot;
  const int cell = b.list[(size_t)(round & 1) * C1 + li];
  WarpCell w;
#if MCX_BAL_EXACT
  w.X = reinterpret_cast<real*>(wsm + b.metaDoubles) + (size_t)slot * b.cellReals;
#else
  w.X = reinterpret_cast<real*>(wsm + b.metaDoubles) + (size_t)slot * (b.cellRealsMixed + b.augReals);
#endif
  w.AL = w.X + NP;
  w.CC = w.AL + NP;
  w.PI = w.CC + NP;
  w.T = w.PI + nSh;
  w.LAD = w.T + max(NP, nSh);
  w.AUG = w.X + b.cellRealsMixed;
  for (int k = L.gl; k < NP; k += kGroup) w.X[k] = (real)b.ion[(size_t)k * C1 + cell];
  if (L.gl == 0) b.nIterT[cell] = b.nIterT[cell] + 1;
  const double te = b.te[cell];
  const real teR = (real)te;
  double ne = b.ne[cell];
  const double hden = hdenG[cell];
  const real hdenR = (real)hden;
  // calcAlpha, one pair per lane
  for (int k = L.gl; k < NP; k += kGroup) {
    const int e = k / ns + 1, ion = k % ns + 1;
    const int elem = m.zOf[e];
#if MCX_BAL_EXACT
    w.AL[k] = ion <= min(ns - 1, elem) ? alphaOf(b, teR, elem, ion) : (real)0.;
#else
    w.AL[k] = ion <= min(ns - 1, elem) ? (b.alphaTab ? alphaLookup(b, k, teR, elem, ion) : alphaOf(b, teR, elem, ion))
                                       : (real)0.;
#endif
  }
  // photoionisation rates per shell
  for (int t = L.gl; t < nSh; t += kGroup) w.PI[t] = (real)b.gam[(size_t)t * C1 + cell];
  __syncwarp(L.mask);
  real xe = 0;
  for (int e = 1; e <= E; ++e) {
    const int elem = m.zOf[e];
    xe = xe + (real)xAt(b, m, w, elem, 1) * (real)m.abun[elem] * hdenR;
  }
  xe = (real)ne / xe;
  real heatef;
  if (xe > RF(0.95)) heatef = 1;
  else {
    if (xe < RF(1.e-4)) xe = RF(1.e-4);
    heatef = RF(0.9971) * ((real)1. - pow((real)1. - pow(xe, RF(0.2663)), RF(1.3163)));
  }
  // reverse charge exchange: deltaE_k > 1 only for N0 and O0
  if (L.gl == 0)
    for (int k = 0; k < 2; ++k) {
      const int elem = k == 0 ? 7 : 8;
      const real dE = k == 0 ? RF(10863.) : RF(2205.);
      if (!m.xref[elem] || ns - 1 < 1) continue;
      const int32_t* o = outerOf(b, elem, elem);
      const int nsh = m.nsh[(m.xref[elem] - 1) * 32];
      if (o[0] > nsh) continue;
      real cx = chexFit(b, elem, 1, teR);
      real rev = cx * ((real)1. - (real)xAt(b, m, w, 1, 1)) * hdenR * (real)2. * exp(-dE / teR) / ((real)o[1] / (real)o[2]);
      const int off = m.p0[(m.xref[elem] - 1) * 32] + o[0] - 1;
      w.PI[off] = w.PI[off] + rev;
    }
  // collisionalIonisation: the reference returns from the whole routine at the
  // first pair (element outer, ion inner) with u > 80, so that pair and every
  // later one keep 0
  {
    const real tev = teR * RF(8.617385e-05);
    int firstStop = NP;
    for (int k = L.gl; k < NP; k += kGroup) {
      const int e = k / ns + 1, ion = k % ns + 1;
      const int elem = m.zOf[e];
      w.CC[k] = 0;
      if (ion > min(ns - 1, elem - 1)) continue;
      const int elec = elem - ion + 1;
      const float* cf = b.CF + ((size_t)(elem - 1) * kNE + (elec - 1)) * 5;
      real u = (real)cf[0] / tev;
      if (u > (real)80.) { firstStop = min(firstStop, k); continue; }
      w.CC[k] = (real)cf[2] * ((real)1. + (real)cf[1] * sqrt(u)) / ((real)cf[3] + u) * pow(u, (real)cf[4]) * exp(-u);
    }
    for (int o = kGroup / 2; o > 0; o >>= 1) firstStop = min(firstStop, __shfl_xor_sync(L.mask, firstStop, o, kGroup));
    for (int k = L.gl; k < NP; k += kGroup)
      if (k >= firstStop) w.CC[k] = 0;
  }
  __syncwarp(L.mask);
  // compton, with the state before ionBalance
  if (b.lgCompton && L.gl == 0) {
    const real s1 = (real)b.comp[0 * (size_t)C1 + cell], s2 = (real)b.comp[1 * (size_t)C1 + cell];
    const real rhH = (real)b.comp[2 * (size_t)C1 + cell], rhHe = (real)b.comp[3 * (size_t)C1 + cell];
    real cool = (RF(6.65e-25) * RF(6.75e-10) * teR * s2) / hdenR;
    real heat = (RF(6.65e-25) * s1 / RF(8.184e-7)) / hdenR;
    real he = m.xref[2] ? rhHe * ((real)xAt(b, m, w, 2, 1) * (real)m.abun[2]) * (real)2. : (real)0.;
    real recoil = (rhH * (real)xAt(b, m, w, 1, 1) * (real)m.abun[1] + he) * kRyd2erg();
    b.compCool[cell] = cool;
    b.compHeat[cell] = heat;
    b.compRecoil[cell] = recoil;
  }
  const bool conv = ionBalanceWarp(b, m, w, L, te, ne, hden);
  __syncwarp(L.mask);
  for (int k = L.gl; k < NP; k += kGroup) b.ion[(size_t)k * C1 + cell] = (double)w.X[k];
  // photoIon(2) of every shell for the heating sum (secondary-ionisation tail times heatef)
  for (int t = L.gl; t < nSh; t += kGroup) {
    const size_t o = (size_t)t * C1 + cell;
    w.T[t] = b.shells[t].heavy ? (real)b.heatA[o] + (real)b.heatHi[o] * heatef : (real)b.heatA[o];
  }
  __syncwarp(L.mask);
  // thermBalance without forLines: the terms by lane, their sums in the
  // reference's order by the group's first lane
  const real neR = (real)ne;
  real* termFF = w.LAD;              // [E] free-free, then recombination, of H-like ions
  real* termRec = w.LAD + E;
  real* termFF2 = w.LAD + 2 * E;     // the same of He-like ions
  real* termRec2 = w.LAD + 3 * E;
  for (int l = L.gl; l < E; l += kGroup) {
    const int e = l + 1;
    const int i = m.zOf[e];
    termFF[l] = termRec[l] = termFF2[l] = termRec2[l] = 0;
    if (ns > i) {
      real L = log10(teR / (real)(i * i));
      real Np = (real)xAt(b, m, w, i, i + 1) * (real)m.abun[i];
      real betaFF = (real)i * (RF(1.0108464E-11) + RF(9.7930778E-13) * L - RF(6.6433144E-13) * L * L +
                               RF(2.4793747E-13) * L * L * L - RF(2.3938215E-14) * L * L * L * L);
      termFF[l] = Np * neR * betaFF * kBoltz() * teR / sqrt(teR);
      real betaRec = (real)i * (RF(9.4255985E-11) - RF(4.04794384E-12) * L - RF(1.0055237E-11) * L * L +
                                RF(1.99266862E-12) * L * L * L - RF(1.06681387E-13) * L * L * L * L);
      termRec[l] = Np * neR * betaRec * kBoltz() * teR / sqrt(teR);
      if (i >= 2) {
        L = log10((real)4. * teR / (real)(i * i));
        Np = (real)xAt(b, m, w, i, i) * (real)m.abun[i];
        betaFF = ((real)i / (real)2.) * (RF(1.070073e-11) - RF(2.5730207e-13) * L + RF(2.109134e-13) * L * L);
        termFF2[l] = Np * neR * betaFF * kBoltz() * teR / sqrt(teR);
        betaRec = ((real)i / (real)2.) * (RF(1.06926e-10) - RF(2.41756e-11) * L + RF(1.14542e-12) * L * L -
                                          RF(5.06535e-13) * L * L * L + RF(9.16745e-14) * L * L * L * L);
        termRec2[l] = Np * neR * betaRec * kBoltz() * teR / sqrt(teR);
      }
    }
  }
  // collisional ionisation cooling per pair into w.AL (alpha is not needed any more)
  for (int k = L.gl; k < NP; k += kGroup) {
    const int e = k / ns + 1, ion = k % ns + 1;
    const int elem = m.zOf[e];
    real v = 0;
    if (ion <= min(elem, ns - 1)) {
      const real c2 = (real)b.cionTherm[(elem - 1) * kNE + (ion - 1)] * w.CC[k] * kBoltz();
      v = (real)m.abun[elem] * xAt(b, m, w, elem, ion) * c2 * neR;
    }
    w.AL[k] = v;
  }
  // photoheating per shell into w.T (the photoIon(2) values staged above)
  for (int t = L.gl; t < nSh; t += kGroup) {
    const PhotoShell sh = b.shells[t];
    w.T[t] = w.T[t] * xAt(b, m, w, sh.elem, sh.ion) * (real)m.abun[sh.elem];
  }
  __syncwarp(L.mask);
  if (L.gl != 0) return;
  b.ibConv[cell] = conv ? 1 : 0;
  b.ne[cell] = ne;
#if !MCX_BAL_EXACT
  if (b.coolTab) b.coolAt[cell] = coolStencil(te, ne);
#endif
  real coolFF = 0, coolRec = 0;
  for (int e = 1; e <= E; ++e) {
    if (!(ns > m.zOf[e])) continue;
    real t = (real)termFF[e - 1];
    if (!isnan(t)) coolFF = coolFF + t;
    t = (real)termRec[e - 1];
    if (!isnan(t)) coolRec = coolRec + t;
  }
  for (int e = 1; e <= E; ++e) {
    const int i = m.zOf[e];
    if (i < 2 || !(ns > i)) continue;
    real t = (real)termFF2[e - 1];
    if (!isnan(t)) coolFF = coolFF + t;
    t = (real)termRec2[e - 1];
    if (!isnan(t)) coolRec = coolRec + t;
  }
  // Te4 as the He-like loop leaves it: 4 Te / (i^2 1e4) of the last element with nstages > i
  real Te4 = teR / RF(1.e4);
  for (int e = 1; e <= E; ++e) {
    const int i = m.zOf[e];
    if (i < 2 || !(ns > i)) continue;
    Te4 = (real)4. * teR / ((real)(i * i) * RF(1.e4));
  }
  real coolColl;
  if (teR > (real)5000.)
    coolColl = (RF(2.47e-8) * exp(-RF(118338.) / teR) * pow(Te4, RF(-0.228)) +
                RF(1.32e-8) * exp(-RF(140252.) / teR) * pow(Te4, RF(-0.460))) * kHcRyd() * (real)xAt(b, m, w, 1, 1) * neR;
  else
    coolColl = 0;
  real coolCollH = 0;
  for (int e = 1; e <= E; ++e) {
    const int elem = m.zOf[e];
    for (int ion = 1; ion <= min(elem, ns - 1); ++ion) coolCollH = coolCollH + (real)w.AL[(e - 1) * ns + (ion - 1)];
  }
  real heatSte = 0;
  for (int e = 1; e <= E; ++e) {
    const int elem = m.zOf[e];
    for (int ion = 1; ion <= min(elem, ns - 1); ++ion) {
      const int p0 = m.p0[(e - 1) * 32 + (ion - 1)];
      const int nsh = m.nsh[(e - 1) * 32 + (ion - 1)];
      for (int q = 0; q < nsh; ++q) heatSte = heatSte + (real)w.T[p0 + q];
    }
  }
  b.coolA[cell] = coolFF + coolRec;
  b.coolHex[cell] = coolColl;
  b.coolCollH[cell] = coolCollH;
  b.heat[cell] = heatSte;
}

__global__ void __launch_bounds__(128) ratesKernel(BalanceDev b, const float* __restrict__ hdenG, int round) {
  extern __shared__ double wsm[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, grp = lane / kGroup;
  const Lanes L{lane % kGroup, ((1u << kGroup) - 1u) << (grp * kGroup)};
  const int cellsPerBlock = (blockDim.x >> 5) * kCellsPerWarp;
  const int slot = wib * kCellsPerWarp + grp;
  const unsigned cnt = b.listCount[round];
  if ((unsigned)(blockIdx.x * cellsPerBlock) >= cnt) return;   // the whole block
  const int E = b.nElemUsed;
  // the element tables, then one slice per warp
  int32_t* sZ = reinterpret_cast<int32_t*>(wsm);
  int32_t* sX = sZ + 32;
  float* sA = reinterpret_cast<float*>(sX + 32);
  int16_t* sP0 = reinterpret_cast<int16_t*>(sA + 32);
  int16_t* sNs = sP0 + E * 32;
  for (int i = threadIdx.x; i < 32; i += blockDim.x) {
    sZ[i] = i <= 30 ? b.zOf[i] : 0;
    sX[i] = i <= 30 ? b.xref[i] : 0;
    sA[i] = i <= 30 ? b.abun[i] : 0.f;
  }
  for (int i = threadIdx.x; i < E * 32; i += blockDim.x) {
    sP0[i] = (int16_t)b.pairShell0[i];
    sNs[i] = (int16_t)b.pairNShell[i];
  }
  __syncthreads();
  const ElemMeta m{sZ, sX, sA, sP0, sNs};
  // the listed cells in strides of the grid (the grid is sized for the resident blocks)
  for (unsigned base = blockIdx.x * cellsPerBlock; base < cnt; base += gridDim.x * cellsPerBlock) {
    const unsigned li = base + slot;
    if (li < cnt) ratesCell(b, hdenG, round, (int)li, m, L, wsm, slot);
  }
}

// ------------------------------------------------------------- equilibrium

#if MCX_BAL_EXACT
__device__ __forceinline__ const real* atomTable(const BalanceDev& b) { return b.atomData; }
#else
__device__ __forceinline__ const real* atomTable(const BalanceDev& b) { return b.atomDataF; }
#endif

// splint with the interval search done once per atom: klo/khi and the
// weights depend only on x and the temperature points
struct SplineAt {
  int klo, khi;    // 1-based, 0 = below the table, -1 = above
  real a, bb, a3, b3, hh;
};

__device__ SplineAt splineAt(const real* xa, int n, real x) {
  SplineAt s{};
  if (x <= xa[0]) { s.klo = 0; return s; }
  if (x >= xa[n - 1]) { s.klo = -1; return s; }
  int klo = 1, khi = n;
  for (int i = 0; i < 1000; ++i) {
    if (khi - klo <= 1) break;
    int k = (khi + klo) / 2;
    if (xa[k - 1] > x) khi = k; else klo = k;
  }
  real h = xa[khi - 1] - xa[klo - 1];
  s.klo = klo;
  s.khi = khi;
  s.a = (xa[khi - 1] - x) / h;
  s.bb = (x - xa[klo - 1]) / h;
  s.a3 = s.a * s.a * s.a - s.a;
  s.b3 = s.bb * s.bb * s.bb - s.bb;
  s.hh = h * h;
  return s;
}

__device__ __forceinline__ real splineEval(const SplineAt& s, const real* ya, const real* y2a, int n) {
  if (s.klo == 0) return ya[0];
  if (s.klo < 0) return ya[n - 1];
  return s.a * ya[s.klo - 1] + s.bb * ya[s.khi - 1] + (s.a3 * y2a[s.klo - 1] + s.b3 * y2a[s.khi - 1]) * s.hh / (real)6.;
}

// The collision rate coefficients qeff of every level pair (source/emission_mod.f90:2884-2936):
// f(lo, up, qeff(lo,up), qeff(up,lo)) for lo < up, in the rate precision.
template <typename F>
__device__ __forceinline__ void collisionPairs(const BalanceDev& b, const int32_t* h, real TeR, real sqrTe,
                                               real log10Te, F f) {
  const real* D = atomTable(b);
  const double* eD = b.atomData + h[kAtOffE];
  const int nLev = h[kAtNLev], nT = h[kAtNTemp];
  const real* logT = D + h[kAtOffLogT];
  const real* qom = D + h[kAtOffQom];
  const real* y2 = D + h[kAtOffY2];
  const real* g = D + h[kAtOffG];
  const real* e = D + h[kAtOffE];
  const SplineAt sp = nT > 2 ? splineAt(logT, nT, log10Te) : SplineAt{};
  const real constant = (real)1.4388463, c863 = (real)8.63e-6;
  int p = 0;
  for (int i = 2; i <= nLev; ++i) {
    for (int j = i; j <= nLev; ++j, ++p) {
      const real* qq = qom + (size_t)p * nT;
      real cs;
      if (nT == 1) cs = qq[0];
      else if (nT == 2) cs = qq[0] + (qq[1] - qq[0]) / (logT[1] - logT[0]) * (log10Te - logT[0]);
      else cs = splineEval(sp, qq, y2 + (size_t)p * nT, nT);
      if (eD[i - 2] <= eD[j - 1]) {
        real expFac = exp((e[i - 2] - e[j - 1]) * constant / TeR);
        f(i - 1, j, c863 * cs * expFac / (g[i - 2] * sqrTe), c863 * cs / (g[j - 1] * sqrTe));
      } else {
        real expFac = exp((e[j - 1] - e[i - 2]) * constant / TeR);
        f(i - 1, j, c863 * cs / (g[j - 1] * sqrTe), c863 * cs * expFac / (g[i - 2] * sqrTe));
      }
    }
  }
}

#if !MCX_BAL_EXACT
// The same populations by state reduction in FP32 (Grassmann, Taksar & Heyman,
// Oper. Res. 33 (1985) 1107).  Rows 2..n of equilibrium's matrix are the
// balance of level i between the rates r(j->i) = Ne qeff(j,i) + a(j,i) into it,
// the rates out of it and, with rec, a recombination source
// s_i = Ne ionDenUp alpha_i; row 1 is the normalisation.  Eliminating levels
// n..2 redirects the flows through each removed level k in proportion to its
// exits r(k->j) / D_k, D_k = sum_{j<k} r(k->j), and back-substitution gives
// n_k = n_1 u_k + v_k with u_k the share fed from level 1 and v_k the share
// fed by the sources; the normalisation fixes n_1.  Every step adds or
// multiplies non-negative numbers, so each population keeps a relative error
// of a few FP32 ulps whatever the spread of the rates; the unpivoted LU of the
// reference cancels and needs FP64.  Returns false (the caller falls back to
// the FP64 LU) when a level has no exit to the levels below it.
__device__ __forceinline__ bool gthParts(const BalanceDev& b, const int32_t* h, double Ne, double srcMul, bool rec,
                                         const double* alphaTotal, real TeR, real sqrTe, real log10Te, float* u,
                                         float* v) {
  const int n = h[kAtNLev];
  const float* A = b.atomDataF + h[kAtOffA];
  const float NeF = (float)Ne;
  float R[kMaxLevels + 1][kMaxLevels + 1];   // R[a][c]: rate from level a to level c
  for (int i = 1; i <= n; ++i)
    for (int j = 1; j <= n; ++j) R[i][j] = 0.f;
  collisionPairs(b, h, TeR, sqrTe, log10Te, [&](int lo, int up, real qLoUp, real qUpLo) {
    R[lo][up] = NeF * qLoUp;
    R[up][lo] = NeF * qUpLo + A[(size_t)(up - 1) * n + (lo - 1)];
  });
  float src[kMaxLevels + 1], Dk[kMaxLevels + 1];
  for (int i = 1; i <= n; ++i) src[i] = (rec && i >= 2) ? (float)(srcMul * alphaTotal[i]) : 0.f;
  for (int k = n; k >= 2; --k) {
    float d = 0.f;
    for (int j = 1; j < k; ++j) d += R[k][j];
    if (!(d > 0.f) || !(d < 3.0e38f)) return false;
    Dk[k] = d;
    const float rd = 1.f / d;
    for (int i = 1; i < k; ++i) {
      const float fi = R[i][k] * rd;
      if (fi != 0.f)
        for (int j = 1; j < k; ++j) R[i][j] += fi * R[k][j];   // R[i][i] collects unused self-loops
    }
    if (rec) {
      const float fs = src[k] * rd;
      if (fs != 0.f)
        for (int j = 2; j < k; ++j) src[j] += fs * R[k][j];
    }
  }
  u[1] = 1.f;
  v[1] = 0.f;
  for (int k = 2; k <= n; ++k) {
    float a = 0.f, c = rec ? src[k] : 0.f;
    for (int i = 1; i < k; ++i) {
      a += u[i] * R[i][k];
      if (rec) c += v[i] * R[i][k];
    }
    u[k] = a / Dk[k];
    v[k] = c / Dk[k];
  }
  return true;
}

__device__ __forceinline__ bool gthPops(const BalanceDev& b, const int32_t* h, double Ne, double ionDenUp, bool rec,
                                        const double* alphaTotal, real TeR, real sqrTe, real log10Te, double* y) {
  float u[kMaxLevels + 1], v[kMaxLevels + 1];
  if (!gthParts(b, h, Ne, Ne * ionDenUp, rec, alphaTotal, TeR, sqrTe, log10Te, u, v)) return false;
  const int n = h[kAtNLev];
  float su = 0.f, sv = 0.f;
  for (int k = 2; k <= n; ++k) {
    su += u[k];
    sv += v[k];
  }
  const float n1 = (1.f - sv) / (1.f + su);
  y[1] = n1;
  for (int k = 2; k <= n; ++k) y[k] = (double)(n1 * u[k] + v[k]);
  return true;
}
#endif

// equilibrium of one atom: the normalised level populations y[1..nLev]
// (source/emission_mod.f90:2884-2984).  Collision rates in the rate
// precision; the FP64 path solves the rate matrix by the reference's
// unpivoted LU, the mixed path by FP32 state reduction (gthPops).
// the recombination coefficients of equilibrium's source term, alphaTotal[1..nLev]
// (source/emission_mod.f90:2836-2880)
__device__ __forceinline__ void recAlphas(const BalanceDev& b, const int32_t* h, real TeR, double* alphaTotal) {
  const double* DD = b.atomData;
  const int nLev = h[kAtNLev];
  for (int i = 0; i <= nLev; ++i) alphaTotal[i] = 0.;
  {
    const double* rr = DD + h[kAtOffRec];
    const real one = (real)1.;
    if (h[kAtRecType] == kRecPowerLaw) {
      for (int r = 0; r < h[kAtNRec]; ++r) {
        const double* v = rr + r * 11;
        const int j = r + 2;
        real br = (float)v[0], z = (float)v[1];
        real ar0 = (float)v[2], ar1 = (float)v[3], ar2 = (float)v[4], ar3 = (float)v[5];
        real ad0 = (float)v[6], ad1 = (float)v[7], ad2 = (float)v[8], ad3 = (float)v[9], ad4 = (float)v[10];
        if (z > (real)0.) {
          real tz = TeR * RF(1.e-4) / (z * z);
          real t4 = TeR * RF(1.e-4);
          alphaTotal[j] = RF(1.e-13) * br * z * ar0 * pow(tz, ar1) / (one + ar2 * pow(tz, ar3)) +
                          RF(1.0e-12) * br * (ad0 / t4 + ad1 + ad2 * TeR * RF(1.e-4) + ad3 * (t4 * t4)) *
                              pow(t4, (real)-1.5) * exp(-ad4 * RF(1.e4) / TeR);
        }
      }
    } else if (h[kAtRecType] == kRecChianti) {
      for (int r = 0; r < h[kAtNRec]; ++r) {
        const double* v = rr + r * 5;
        int jj = (int)v[0];
        real a = (float)v[1], bb = (float)v[2], cc = (float)v[3], d = (float)v[4];
        real L = log10(TeR);
        alphaTotal[jj] = pow((real)10., a + bb * L + cc * (L * L) + d * (L * L * L));
      }
    }
  }
}

__device__ __forceinline__ void equilibriumPops(const BalanceDev& b, int atom, double Te, double Ne, double ionDenUp,
                                                bool rec, double* y) {
  const int32_t* h = b.atomHdr + (size_t)atom * kAtHdrSize;
  const double* DD = b.atomData;
  const int nLev = h[kAtNLev];
  const double* A = DD + h[kAtOffA];
  const real TeR = (real)Te;
  const real sqrTe = sqrt(TeR), log10Te = log10(TeR);
  double alphaTotal[kMaxLevels + 1];
  if (rec) recAlphas(b, h, TeR, alphaTotal);
  else
    for (int i = 0; i <= nLev; ++i) alphaTotal[i] = 0.;
#if !MCX_BAL_EXACT
  if (gthPops(b, h, Ne, ionDenUp, rec, alphaTotal, TeR, sqrTe, log10Te, y)) return;
#endif
  real qeff[kMaxLevels + 1][kMaxLevels + 1];
  double x[kMaxLevels + 1][kMaxLevels + 1];
  for (int i = 1; i <= nLev; ++i) {
    y[i] = 0.;
    for (int j = 1; j <= nLev; ++j) { qeff[i][j] = 0; x[i][j] = 0.; }
  }
  collisionPairs(b, h, TeR, sqrTe, log10Te, [&](int lo, int up, real qLoUp, real qUpLo) {
    qeff[lo][up] = qLoUp;
    qeff[up][lo] = qUpLo;
  });
  for (int j = 1; j <= nLev; ++j) x[1][j] = 1.;
  y[1] = 1.;
  for (int i = 2; i <= nLev; ++i) {
    for (int j = 1; j <= nLev; ++j) {
      if (j != i) {
        x[i][j] = x[i][j] + Ne * (double)qeff[j][i];
        x[i][i] = x[i][i] - Ne * (double)qeff[i][j];
        if (j > i) x[i][j] = x[i][j] + A[(size_t)(j - 1) * nLev + (i - 1)];
        else x[i][i] = x[i][i] - A[(size_t)(i - 1) * nLev + (j - 1)];
      }
    }
    y[i] = -Ne * ionDenUp * alphaTotal[i];
  }
  const int n = nLev;
#if MCX_BAL_EXACT
  // lured + reslv as the reference writes them (no pivoting, multipliers recomputed)
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
#else
  // the same unpivoted elimination with one reciprocal per pivot and the
  // multipliers kept for the forward substitution (FP64)
  double rdiag[kMaxLevels + 1];
  for (int i = 1; i <= n - 1; ++i) {
    const double r = 1. / x[i][i];
    rdiag[i] = r;
    for (int k = i + 1; k <= n; ++k) {
      const double factor = x[k][i] * r;
      x[k][i] = factor;
      for (int j = i + 1; j <= n; ++j) x[k][j] = x[k][j] - x[i][j] * factor;
    }
  }
  rdiag[n] = 1. / x[n][n];
  for (int i = 1; i <= n - 1; ++i)
    for (int j = i + 1; j <= n; ++j) y[j] = y[j] - y[i] * x[j][i];
  y[n] = y[n] * rdiag[n];
  for (int k = n - 1; k >= 1; --k) {
    double acc = y[k];
    for (int j = k + 1; j <= n; ++j) acc = acc - y[j] * x[k][j];
    y[k] = acc * rdiag[k];
  }
#endif
  double sumN = 0.;
  for (int i = 1; i <= nLev; ++i) sumN = sumN + y[i];
  for (int i = 1; i <= nLev; ++i) y[i] = y[i] / sumN;
}

// equilibrium of one atom: the sum over its lines of a(j,i)*E_ji*n_j*m1*m2*m3
// that exceed 1e-35, lower level outer, upper level inner.
__device__ double equilibriumLines(const BalanceDev& b, int atom, double Te, double Ne, double ionDenUp, bool rec,
                                   double m1, double m2, double m3) {
  double y[kMaxLevels + 1];
  equilibriumPops(b, atom, Te, Ne, ionDenUp, rec, y);
  const int32_t* h = b.atomHdr + (size_t)atom * kAtHdrSize;
#if !MCX_BAL_EXACT
  // sum_j n_j sum_i a(j,i) E_ji with the line factors summed at set-up: the
  // per-line 1e-35 cut of the reference drops terms that are below 1e-12 of
  // any cooling rate the balance resolves
  {
    const double* P = b.linePow + (size_t)atom * (kMaxLevels + 1);
    const int n = h[kAtNLev];
    double acc = 0.;
    for (int j = 2; j <= n; ++j) acc = acc + y[j] * P[j];
    return acc * m1 * m2 * m3;
  }
#endif
  const double* DD = b.atomData;
  const int nLev = h[kAtNLev];
  const double* A = DD + h[kAtOffA];
  const double* eD = DD + h[kAtOffE];
  const double atp = DD[h[kAtOffAtp]];
  const int iup2p = h[kAtIup2p];
  double total = 0.;
  for (int i = 1; i <= nLev - 1; ++i)
    for (int j = i + 1; j <= nLev; ++j) {
      double aji = A[(size_t)(j - 1) * nLev + (i - 1)];
      if (aji != 0.) {
        double Eji = eD[j - 1] - eD[i - 1];
        if (j == iup2p && i == 1 && atp > 0.) aji = aji - atp;
        double f = aji * Eji * y[j] * m1 * m2 * m3;
        if (f > RD(1.e-35)) total = total + f;
      }
    }
  return total;
}

// forLines of update_mod: one thread per (cell, ion with data)
// Tight mode: a cell whose ladder has not converged in this round goes on at the same Te and its
// residual is not used (the secant step skips it), so its line cooling is not solved; the last round
// a cell can have still gets it (with Te held, the residual of that round is the result).
__device__ __forceinline__ bool coolingUnused(const BalanceDev& b, int round, int lastRound, int cell) {
  return b.converge && !b.ibConv[cell] && b.nIterT[cell] < b.maxIterT && round + 1 < kMaxRounds && !lastRound;
}

__global__ void __launch_bounds__(128) atomsKernel(BalanceDev b, int round, int lastRound) {
  const int li = blockIdx.x * blockDim.x + threadIdx.x;
  const int atom = blockIdx.y;
  if ((unsigned)li >= b.listCount[round]) return;
  const int cell = b.list[(size_t)(round & 1) * (b.nCells + 1) + li];
  if (coolingUnused(b, round, lastRound, cell)) return;
  const CellIdx c{cell, b.nCells + 1};
  const int32_t* h = b.atomHdr + (size_t)atom * kAtHdrSize;
  const int elem = h[kAtElem], ion = h[kAtIon];
  const int top = min(elem + 1, b.nstages);
  const double x = ionAt(b, c, elem, ion);
#if !MCX_BAL_EXACT
  // an ion below 1e-16 per H contributes < 1e-9 of the cooling: no solve
  if ((double)b.abun[elem] * x < kNegligibleIon) {
    b.forSum[(size_t)atom * c.C1 + cell] = 0.;
    return;
  }
#endif
  // forbiddenLines = fLineEm * elemAbun * ionDen * 1.9865e-16, summed where > 1e-35;
  // without the recombination term the ratio ionDen(ion+1)/ionDen(ion) is not used
  (void)top;
  b.forSum[(size_t)atom * c.C1 + cell] =
      equilibriumLines(b, atom, b.te[cell], b.ne[cell], 0., false, (double)b.abun[elem], x, RD(1.9865e-16));
}

// The emission phase's forLines (rec = .true., 1e-25 erg units): one thread
// per (cell, ion with data), each ion's line total into forSum[atom][cell].
__global__ void __launch_bounds__(128) forLinesAtomsKernel(BalanceDev b, const float* __restrict__ te,
                                                           const float* __restrict__ ne,
                                                           const float* __restrict__ ionDen,
                                                           const uint8_t* __restrict__ compute) {
  const int cell = blockIdx.x * blockDim.x + threadIdx.x;
  const int atom = blockIdx.y;
  const int C1 = b.nCells + 1;
  if (cell >= C1 || !compute[cell]) return;
  const int32_t* h = b.atomHdr + (size_t)atom * kAtHdrSize;
  const int elem = h[kAtElem], ion = h[kAtIon];
  const int top = min(elem + 1, b.nstages);
  const int e = b.xref[elem];
  const double x = ionDen[((size_t)(ion - 1) * b.nElemUsed + (e - 1)) * C1 + cell];
  double v = 0.;
#if !MCX_BAL_EXACT
  if ((double)b.abun[elem] * x >= kNegligibleIon)
#endif
  {
    double up = 0.;
    if (ion < top && x > 0.) up = (double)ionDen[((size_t)ion * b.nElemUsed + (e - 1)) * C1 + cell] / x;
    v = equilibriumLines(b, atom, te[cell], ne[cell], up, true, (double)b.abun[elem], x, RD(1.9865e9));
  }
  b.forSum[(size_t)atom * C1 + cell] = v;
}

#if !MCX_BAL_EXACT
// The emission phase's forLines from the surfaces: each cell placed on the
// grid once, then one thread per (cell, ion with data) forms
// (G + ionDenUp B) elemAbun ionDen 1.9865e9; cells outside the grid solve
// the ion directly.
__global__ void __launch_bounds__(128) surfaceStencilKernel(BalanceDev b, const float* __restrict__ te,
                                                            const float* __restrict__ ne,
                                                            const uint8_t* __restrict__ compute) {
  const int cell = blockIdx.x * blockDim.x + threadIdx.x;
  if (cell > b.nCells || !compute[cell]) return;
  b.coolAt[cell] = coolStencil((double)te[cell], (double)ne[cell]);
}

__global__ void __launch_bounds__(128) forLinesSurfaceKernel(BalanceDev b, const float* __restrict__ te,
                                                             const float* __restrict__ ne,
                                                             const float* __restrict__ ionDen,
                                                             const uint8_t* __restrict__ compute) {
  const int cell = blockIdx.x * blockDim.x + threadIdx.x;
  const int atom = blockIdx.y;
  const int C1 = b.nCells + 1;
  if (cell >= C1 || !compute[cell]) return;
  const int32_t* h = b.atomHdr + (size_t)atom * kAtHdrSize;
  const int elem = h[kAtElem], ion = h[kAtIon];
  const int top = min(elem + 1, b.nstages);
  const int e = b.xref[elem];
  const double x = ionDen[((size_t)(ion - 1) * b.nElemUsed + (e - 1)) * C1 + cell];
  double v = 0.;
  if ((double)b.abun[elem] * x >= kNegligibleIon) {
    double up = 0.;
    if (ion < top && x > 0.) up = (double)ionDen[((size_t)ion * b.nElemUsed + (e - 1)) * C1 + cell] / x;
    const CoolAt a = b.coolAt[cell];
    double L;
    if (a.iT >= 0) {
      const float2 g = surfaceAt(b.coolTab, atom, a);
      const float2 r = surfaceAt(b.recTab, atom, a);
      L = (double)expf(g.x) * (double)expf(g.y) + up * (double)(r.x + r.y);
    } else {
      L = equilibriumLines(b, atom, te[cell], ne[cell], up, true, 1., 1., 1.);
    }
    v = L * (double)b.abun[elem] * x * RD(1.9865e9);
  }
  b.forSum[(size_t)atom * C1 + cell] = v;
}
#endif

// normFor of emissionDriver: the ions' line totals summed in the reference's ion order
__global__ void forLinesSumKernel(BalanceDev b, const uint8_t* __restrict__ compute, float* forLines) {
  const int cell = blockIdx.x * blockDim.x + threadIdx.x;
  const int C1 = b.nCells + 1;
  if (cell >= C1 || !compute[cell]) return;
  double normFor = 0.;
  for (int atom = 0; atom < b.nAtoms; ++atom) normFor = normFor + b.forSum[(size_t)atom * C1 + cell];
  forLines[cell] = (float)normFor;
}

#if MCX_BAL_EXACT
// outputGas forbidden-line volume sums (source/output_mod.f90:410-432 with
// forLines at :1943-1984): per (cell, ion with data) the level populations of
// equilibrium(rec = .true.), weighted by elemAbun * ionDen * 1.9865e9 * Hden
// * dV over the cells with lgBlack < 1.  Each warp (32 consecutive cells)
// reduces level j into partial[group][forbBase[atom] + j - 1]; the line
// factors a(j,i) E_ji multiply the sums afterwards.
__global__ void __launch_bounds__(128) forbLevelSumsKernel(BalanceDev b, LineSumArgs a) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int group = t >> 5;
  if (group >= a.nGroups) return;   // whole warps only
  const int cell = a.cellBase + t + 1;
  const int atom = blockIdx.y;
  const int32_t* h = b.atomHdr + (size_t)atom * kAtHdrSize;
  const int elem = h[kAtElem], ion = h[kAtIon], nLev = h[kAtNLev];
  const int top = min(elem + 1, b.nstages);
  const size_t C1 = (size_t)b.nCells + 1;
  const int e = b.xref[elem];
  const bool valid = t + 1 <= a.nRange && a.black[cell] < 1;
  double y[kMaxLevels + 1];
  double w = 0.;
  if (valid) {
    const double x = a.ionDen[((size_t)(ion - 1) * b.nElemUsed + (e - 1)) * C1 + cell];
    double up = 0.;
    if (ion < top && x > 0.) up = (double)a.ionDen[((size_t)ion * b.nElemUsed + (e - 1)) * C1 + cell] / x;
    equilibriumPops(b, atom, a.te[cell], a.ne[cell], up, true, y);
    w = (double)b.abun[elem] * x * RD(1.9865e9) * (double)a.hden[cell] * a.vol[cell];
  } else {
    for (int j = 1; j <= nLev; ++j) y[j] = 0.;
  }
  double* row = a.partial + (size_t)group * a.nEntries + a.forbBase[atom];
  for (int j = 1; j <= nLev; ++j) {
    const double v = warpSumD(valid ? y[j] * w : 0.);
    if ((threadIdx.x & 31) == 0) row[j - 1] = v;
  }
}

// one thread per (cell, requested line): equilibrium with the recombination
// term, then the line's share (source/output_mod.f90:1943-1984, :410-432)
__global__ void __launch_bounds__(128) lineCellKernel(BalanceDev b, LineCellArgs a) {
  const int cell = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int k = blockIdx.y;
  if (cell > b.nCells) return;
  const size_t C1 = (size_t)b.nCells + 1;
  double v = 0.;
  if (a.black[cell] < 1) {
    const int atom = a.req[3 * k], lo = a.req[3 * k + 1], hi = a.req[3 * k + 2];
    const int32_t* h = b.atomHdr + (size_t)atom * kAtHdrSize;
    const int elem = h[kAtElem], ion = h[kAtIon], nLev = h[kAtNLev];
    const int top = min(elem + 1, b.nstages);
    const int e = b.xref[elem];
    const double x = a.ionDen[((size_t)(ion - 1) * b.nElemUsed + (e - 1)) * C1 + cell];
    double up = 0.;
    if (ion < top && x > 0.) up = (double)a.ionDen[((size_t)ion * b.nElemUsed + (e - 1)) * C1 + cell] / x;
    double y[kMaxLevels + 1];
    equilibriumPops(b, atom, a.te[cell], a.ne[cell], up, true, y);
    const double* A = b.atomData + h[kAtOffA];
    const double* E = b.atomData + h[kAtOffE];
    const double atp = b.atomData[h[kAtOffAtp]];
    double aji = A[(size_t)(hi - 1) * nLev + (lo - 1)];
    if (aji != 0.) {
      const double Eji = E[hi - 1] - E[lo - 1];
      if (hi == h[kAtIup2p] && lo == 1 && atp > 0.) aji = aji - atp;
      v = aji * Eji * y[hi] * (double)b.abun[elem] * x * RD(1.9865e9) * (double)a.hden[cell] * a.vol[cell];
    }
  }
  a.out[(size_t)k * C1 + cell] = v;
}

cudaError_t launchLineCells(BalanceData& bd, const LineCellArgs& a, cudaStream_t s) {
  if (a.nReq <= 0 || bd.dev.nCells <= 0) return cudaSuccess;
  lineCellKernel<<<dim3((bd.dev.nCells + 127) / 128, a.nReq), 128, 0, s>>>(bd.dev, a);
  return cudaGetLastError();
}

cudaError_t launchForbSums(BalanceData& bd, const LineSumArgs& a, cudaStream_t s) {
  BalanceDev& b = bd.dev;
  if (b.nAtoms <= 0 || a.nGroups <= 0) return cudaSuccess;
  const int T = 128, nb = (a.nGroups * 32 + T - 1) / T;
  forbLevelSumsKernel<<<dim3(nb, b.nAtoms), T, 0, s>>>(b, a);
  return cudaGetLastError();
}
#endif

#if !MCX_BAL_EXACT
// ------------------------------------------------------------- cooling surfaces

// G and B of one atom at (Te, Ne): forLines' line sum per ion without the
// recombination term (G) and its slope in ionDenUp with it (B), so that the
// sum with the term is G + ionDenUp B.  The state reduction gives both from
// one solve: with sources Ne alpha_i, n_k = n_1 u_k + ionDenUp w_k and
// n_1 = (1 - ionDenUp W) / (1 + U), U = sum u_k, W = sum w_k; a level without
// an exit below it falls back to two LU solves.
__device__ void surfaceValues(const BalanceDev& b, int atom, double Te, double Ne, double& G, double& B) {
  const int32_t* h = b.atomHdr + (size_t)atom * kAtHdrSize;
  const int n = h[kAtNLev];
  const real TeR = (real)Te;
  const real sqrTe = sqrt(TeR), log10Te = log10(TeR);
  double alphaTotal[kMaxLevels + 1];
  recAlphas(b, h, TeR, alphaTotal);
  float u[kMaxLevels + 1], v[kMaxLevels + 1];
  if (gthParts(b, h, Ne, Ne, true, alphaTotal, TeR, sqrTe, log10Te, u, v)) {
    const double* P = b.linePow + (size_t)atom * (kMaxLevels + 1);
    double U = 0., UP = 0., W = 0., WP = 0.;
    for (int k = 2; k <= n; ++k) {
      U += u[k];
      UP += (double)u[k] * P[k];
      W += v[k];
      WP += (double)v[k] * P[k];
    }
    G = UP / (1. + U);
    B = WP - W * G;
  } else {
    G = equilibriumLines(b, atom, Te, Ne, 0., false, 1., 1., 1.);
    B = equilibriumLines(b, atom, Te, Ne, 1., true, 1., 1., 1.) - G;
  }
}

// ln G and B of every atom at the grid nodes (see k_balance.cuh), one thread
// per node; G below 1e-37 is stored as 1e-37 (an ion that cools by less is
// below any cooling rate the balance resolves).
__global__ void __launch_bounds__(128) coolTableKernel(BalanceDev b, float* tab, float* rtab) {
  const size_t n = (size_t)b.nAtoms * kCoolNNe * kCoolNTe;
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n) return;
  const int iT = (int)(idx % kCoolNTe);
  const int iN = (int)((idx / kCoolNTe) % kCoolNNe);
  const int atom = (int)(idx / ((size_t)kCoolNTe * kCoolNNe));
  const double te = exp(kCoolLnTe0 + iT * ((kCoolLnTe1 - kCoolLnTe0) / (kCoolNTe - 1)));
  const double ne = exp(kCoolLnNe0 + iN * ((kCoolLnNe1 - kCoolLnNe0) / (kCoolNNe - 1)));
  double g, bb;
  surfaceValues(b, atom, te, ne, g, bb);
  tab[idx] = (float)log(fmax(g, 1e-37));
  rtab[idx] = (float)bb;
}

// weights of the 4-point Lagrange interpolant at nodes -1, 0, 1, 2 for t in [0, 1)
__device__ __forceinline__ void lagrange4(float t, float* w) {
  const float tm1 = t - 1.f, tm2 = t - 2.f, tp1 = t + 1.f;
  w[0] = -t * tm1 * tm2 * (1.f / 6.f);
  w[1] = tp1 * tm1 * tm2 * 0.5f;
  w[2] = -tp1 * t * tm2 * 0.5f;
  w[3] = tp1 * t * tm1 * (1.f / 6.f);
}

// Where a cell's (Te, Ne) sits on the cooling surfaces: the nodes iT, iN of
// the 4 x 4 stencil's second row and column and the fractions within the
// cell of the grid (iT = -1 outside it).
__device__ CoolAt coolStencil(double te, double ne) {
  const double sT = (log(te) - kCoolLnTe0) * ((kCoolNTe - 1) / (kCoolLnTe1 - kCoolLnTe0));
  const double sN = (log(ne) - kCoolLnNe0) * ((kCoolNNe - 1) / (kCoolLnNe1 - kCoolLnNe0));
  CoolAt a{-1, -1, 0.f, 0.f};
  if (sT >= 1. && sT < kCoolNTe - 2 && sN >= 1. && sN < kCoolNNe - 2) {
    a.iT = (int)sT;
    a.iN = (int)sN;
    a.tT = (float)(sT - a.iT);
    a.tN = (float)(sN - a.iN);
  }
  return a;
}

// A surface of atom `atom` ([nAtoms][kCoolNNe][kCoolNTe]) at the stencil a:
// 4-point Lagrange in both directions, summed as differences from the
// stencil's (iN, iT) node so that the FP32 sums keep the stored precision;
// returns the node value and the interpolated difference.
__device__ __forceinline__ float2 surfaceAt(const float* tab, int atom, const CoolAt& a) {
  float wT[4], wN[4];
  lagrange4(a.tT, wT);
  lagrange4(a.tN, wN);
  const float* t = tab + ((size_t)atom * kCoolNNe + (a.iN - 1)) * kCoolNTe + (a.iT - 1);
  const float ref = __ldg(t + kCoolNTe + 1);
  float acc = 0.f;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const float* row = t + (size_t)r * kCoolNTe;
    const float v = wT[0] * (__ldg(row) - ref) + wT[1] * (__ldg(row + 1) - ref) + wT[2] * (__ldg(row + 2) - ref) +
                    wT[3] * (__ldg(row + 3) - ref);
    acc += wN[r] * v;
  }
  return make_float2(ref, acc);
}

// forLines of update_mod with the cooling surfaces: one thread per (listed
// cell, ion with data), that ion's line cooling into forSum[atom][cell].  The
// stencil is interpolated as differences from its (iN, iT) node so that the
// FP32 sums keep the precision of the stored values; cells outside the grid
// solve the ion directly.
// one (listed cell, ion) of surfaceAtomsKernel
__device__ __forceinline__ void surfaceAtom(const BalanceDev& b, int round, int li, int atom) {
  const int cell = b.list[(size_t)(round & 1) * (b.nCells + 1) + li];
  const CellIdx c{cell, b.nCells + 1};
  const int32_t* h = b.atomHdr + (size_t)atom * kAtHdrSize;
  const int elem = h[kAtElem], ion = h[kAtIon];
  const double w = (double)b.abun[elem] * ionAt(b, c, elem, ion);
  double* out = b.forSum + (size_t)atom * c.C1 + cell;
  if (w < kNegligibleIon) {
    *out = 0.;
    return;
  }
  const CoolAt a = b.coolAt[cell];
  double g;
  if (a.iT >= 0) {
    // exp of the node value and of the interpolated difference apart: each is exact to an FP32 ulp
    const float2 r = surfaceAt(b.coolTab, atom, a);
    g = (double)expf(r.x) * (double)expf(r.y);
  } else {
    g = equilibriumLines(b, atom, b.te[cell], b.ne[cell], 0., false, 1., 1., 1.);
  }
  *out = w * RD(1.9865e-16) * g;
}

__global__ void __launch_bounds__(128) surfaceAtomsKernel(BalanceDev b, int round, int lastRound) {
  const int atom = blockIdx.y;
  const unsigned cnt = b.listCount[round];
  const int C1 = b.nCells + 1;
  for (unsigned li = blockIdx.x * blockDim.x + threadIdx.x; li < cnt; li += gridDim.x * blockDim.x)
    if (!coolingUnused(b, round, lastRound, b.list[(size_t)(round & 1) * C1 + li])) surfaceAtom(b, round, (int)li, atom);
}
#endif

// heating - cooling and the secant step of iterateT (FP64 in both precisions)
__device__ __forceinline__ void secantCell(const BalanceDev& b, int round, int lastRound, int li) {
  const int C1 = b.nCells + 1;
  const int cell = b.list[(size_t)(round & 1) * C1 + li];
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
  const bool tight = b.converge != 0;
  // tight mode: a residual whose ionisation ladder has not converged is evaluated again at the same Te
  // (the X-iterations go on from where they stopped) rather than taken as a bracket end
  const bool xPending = tight && !b.ibConv[cell];
  if (b.fixTe) {
    // Te held: the ladder goes on converging at this Te; the residual there is the result
    b.resid[cell] = res;
    if (xPending && nIterateT < b.maxIterT && round + 1 < kMaxRounds) {
      b.list[(size_t)((round + 1) & 1) * C1 + atomicAdd(&b.listCount[round + 1], 1u)] = cell;
    } else {
      b.state[cell] = 1;
      if (!b.ibConv[cell]) atomicAdd(&b.counters->noIonBal, 1ull);
    }
    return;
  }
  bool open = xPending || fabs(res) >= b.resTol * (fabs(cool) + fabs(heat)) / 2.;
  if (open && !xPending && tight && Thigh != 0. && Tlow != 0. && fabs(Thigh - Tlow) <= 1e-12 * (Thigh + Tlow)) {
    open = false;
    // closed on the rounding noise of the residual, or on a jump of heating - cooling (not a root)
    if (fabs(res) > 1e3 * b.resTol * (fabs(cool) + fabs(heat)) / 2.) b.side[cell] = 3;
  }
  if (open) {
    if (nIterateT < b.maxIterT) {
      if (xPending) {
      } else if (tight) {
        // Illinois: an end kept twice in a row has its residual halved
        const int8_t last = b.side[cell];
        if (res < 0.) {
          if (last == 1 && Thigh != 0.) resHigh = resHigh * 0.5;
          resLow = res;
          Tlow = te;
          b.side[cell] = 1;
        } else {
          if (last == 2 && Tlow != 0.) resLow = resLow * 0.5;
          resHigh = res;
          Thigh = te;
          b.side[cell] = 2;
        }
        if (Thigh != 0. && Tlow != 0.) {
          te = Tlow - (Thigh - Tlow) * resLow / (resHigh - resLow);
        } else {
          const double f = 1. + fmin(0.2, b.stepMin * ldexp(1., min(nIterateT, 60)));
          te = res < 0. ? te / f : te * f;
        }
      } else {
        if (res < 0.) {
          resLow = res;
          Tlow = te;
          if (Thigh != 0.) te = Tlow - (Thigh - Tlow) * resLow / (resHigh - resLow);
          else te = te / RD(1.2);
        } else {
          resHigh = res;
          Thigh = te;
          if (Tlow != 0.) te = Tlow - (Thigh - Tlow) * resLow / (resHigh - resLow);
          else te = te * RD(1.2);
        }
        if (nIterateT >= 6 && fabs(Thigh - Tlow) <= (RD(0.002) * (Thigh + Tlow))) {
          if (res < 0.) { te = Thigh - 100.; Thigh = 0.; }
          else { te = Tlow + 100.; Tlow = 0.; }
        }
      }
      if (te <= 0.) te = 1.;
      done = lastRound != 0;   // a caller-imposed round limit ends the cell here
    } else {
      // (tight mode: a cell whose ladder never converged was never bracketed and keeps its Te)
      if (Thigh == 0. && Tlow == 0.) {
      } else if (Thigh == 0.) te = Tlow;
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
  } else if (round + 1 < kMaxRounds) {
    b.list[(size_t)((round + 1) & 1) * C1 + atomicAdd(&b.listCount[round + 1], 1u)] = cell;
  }
}

__global__ void __launch_bounds__(128) secantKernel(BalanceDev b, int round, int lastRound) {
  const unsigned cnt = b.listCount[round];
  for (unsigned li = blockIdx.x * blockDim.x + threadIdx.x; li < cnt; li += gridDim.x * blockDim.x)
    secantCell(b, round, lastRound, (int)li);
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

#undef RF
#undef RD

size_t ratesSmem(const BalanceDev& b);
constexpr int kBuildL = MCX_BAL_EXACT ? 0 : 1;

cudaError_t launch(BalanceData& bd, const BalanceGrid& g, int maxRounds, cudaStream_t s, int atomSolves) {
  BalanceDev& b = bd.dev;
#if MCX_BAL_EXACT
  const int useSurfaces = 0;
  (void)atomSolves;
#else
  const int useSurfaces = atomSolves || b.coolTab == nullptr ? 0 : 1;
#endif
  const int C = b.nCells;
  if (C <= 0) return cudaSuccess;
  const int T = 128, nb = (C + T - 1) / T;
  cudaError_t e = cudaMemsetAsync(b.counters, 0, sizeof(BalanceCounters), s);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(b.listCount, 0, sizeof(unsigned) * (kMaxRounds + 1), s);
  if (e != cudaSuccess) return e;
  hitComptonKernel<<<nb, T, 0, s>>>(b, g.jste);
  if (b.nShellsTot > 0) shellIntegralsKernel<<<(unsigned)b.nShellsTot * (unsigned)nb, T, 0, s>>>(b, g.jste);
  loadStateKernel<<<nb, T, 0, s>>>(b, g.te, g.ne, g.ionDen);
  const int rounds = std::min(std::max(maxRounds, 1), (int)b.maxIterT);
  const int cellsPerBlock = b.ratesWarps[kBuildL] * kCellsPerWarp;
  // the per-round kernels stride over their lists with grids of resident size, so
  // the late rounds (few listed cells) do not launch a block per cell of the grid
  const int rGrid = std::max(1, std::min((C + cellsPerBlock - 1) / cellsPerBlock, b.ratesGrid[kBuildL]));
  const int aGrid = std::max(1, std::min(nb, 8 * b.smCount / std::max(1, b.nAtoms) + 1));
  const int sGrid = std::max(1, std::min(nb, 8 * b.smCount));
  // round r works on the cells listed for it (the first list holds every cell
  // a packet reached; each secant step lists the cells that go on)
  for (int r = 1; r <= rounds; ++r) {
    const int last = r == rounds && rounds < b.maxIterT ? 1 : 0;
    ratesKernel<<<rGrid, 32 * b.ratesWarps[kBuildL], ratesSmem(b), s>>>(b, g.hden, r - 1);
#if !MCX_BAL_EXACT
    if (b.nAtoms > 0 && useSurfaces) surfaceAtomsKernel<<<dim3(aGrid, b.nAtoms), T, 0, s>>>(b, r - 1, last);
    else
#endif
    if (b.nAtoms > 0) atomsKernel<<<dim3(nb, b.nAtoms), T, 0, s>>>(b, r - 1, last);
    secantKernel<<<sGrid, T, 0, s>>>(b, r - 1, last);
  }
  storeKernel<<<nb, T, 0, s>>>(b, g);
  return cudaGetLastError();
}

#if !MCX_BAL_EXACT
// the alphaTotal tables of every (element, ion) pair and their jump flags
cudaError_t buildAlphaTable(const BalanceData& bd, float* tab, uint8_t* jump, cudaStream_t s) {
  const int pairs = bd.dev.nElemUsed * bd.dev.nstages;
  if (pairs <= 0) return cudaSuccess;
  const dim3 grid((kAlphaN + 127) / 128, pairs);
  alphaTableKernel<<<grid, 128, 0, s>>>(bd.dev, tab);
  alphaJumpKernel<<<grid, 128, 0, s>>>(bd.dev, tab, jump);
  return cudaGetLastError();
}

// the surfaces of every atom into tab (ln G) and rtab (B), [nAtoms][kCoolNNe][kCoolNTe] floats each
cudaError_t buildCoolTable(const BalanceData& bd, float* tab, float* rtab, cudaStream_t s) {
  const size_t n = (size_t)bd.dev.nAtoms * kCoolNNe * kCoolNTe;
  if (n == 0) return cudaSuccess;
  coolTableKernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(bd.dev, tab, rtab);
  return cudaGetLastError();
}
#endif

constexpr int kBuild = MCX_BAL_EXACT ? 0 : 1;

// the rates kernel's dynamic shared memory for wps warps per block: the element
// tables and one slice per cell of the block
size_t ratesSmemFor(const BalanceDev& b, int wps) {
#if MCX_BAL_EXACT
  const size_t cell = (size_t)b.cellReals;
#else
  const size_t cell = (size_t)b.cellRealsMixed + (size_t)b.augReals;
#endif
  return (size_t)b.metaDoubles * sizeof(double) + (size_t)wps * kCellsPerWarp * cell * sizeof(real);
}
size_t ratesSmem(const BalanceDev& b) { return ratesSmemFor(b, b.ratesWarps[kBuild]); }

// the block size (4, 2 or 1 warps) that keeps the most warps resident with
// this build's shared memory per cell and registers
cudaError_t prepare(BalanceData& bd) {
  int best = 0, bestWarps = 0, bestBlocks = 0;
  for (int wps : {4, 2, 1}) {
    const size_t smem = ratesSmemFor(bd.dev, wps);
    if (smem > 200 * 1024) continue;
    cudaError_t e = cudaFuncSetAttribute(ratesKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int blocks = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, ratesKernel, 32 * wps, smem);
    if (e != cudaSuccess) return e;
    if (blocks * wps > bestWarps) {
      bestWarps = blocks * wps;
      best = wps;
      bestBlocks = blocks;
    }
  }
  if (!best) return cudaErrorInvalidValue;
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  bd.dev.smCount = sms;
  bd.dev.ratesWarps[kBuild] = best;
  bd.dev.ratesGrid[kBuild] = bestBlocks * sms;
  return cudaFuncSetAttribute(ratesKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ratesSmem(bd.dev));
}

cudaError_t launchForLines(BalanceData& bd, const float* te, const float* ne, const float* ionDen,
                           const uint8_t* compute, float* forLines, cudaStream_t s) {
  BalanceDev& b = bd.dev;
  const int C1 = b.nCells + 1, T = 128, nb = (C1 + T - 1) / T;
  if (b.nAtoms <= 0) return cudaSuccess;
#if !MCX_BAL_EXACT
  if (b.coolTab && b.recTab) {
    surfaceStencilKernel<<<nb, T, 0, s>>>(b, te, ne, compute);
    forLinesSurfaceKernel<<<dim3(nb, b.nAtoms), T, 0, s>>>(b, te, ne, ionDen, compute);
  } else
#endif
    forLinesAtomsKernel<<<dim3(nb, b.nAtoms), T, 0, s>>>(b, te, ne, ionDen, compute);
  forLinesSumKernel<<<nb, T, 0, s>>>(b, compute, forLines);
  return cudaGetLastError();
}

}  // namespace MCX_BAL_NS
}  // namespace mcx
