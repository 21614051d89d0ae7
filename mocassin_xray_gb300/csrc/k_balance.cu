// k_balance.cu - host side of the balance phase: the device tables of a
// set-up and the dispatch between the two compilations of the kernels
// (k_balance_f64.cu: FP64 throughout; k_balance_mixed.cu: FP32 rates with
// FP64 solves), see k_balance_impl.cuh.
#include "k_balance.cuh"
#include "setup_internal.h"

#include <algorithm>
#include <cstring>
#include <vector>

namespace mcx {

namespace bal_f64 {
cudaError_t launch(BalanceData& bd, const BalanceGrid& g, int maxRounds, cudaStream_t s, int atomSolves);
cudaError_t launchForLines(BalanceData& bd, const float* te, const float* ne, const float* ionDen,
                           const uint8_t* compute, float* forLines, cudaStream_t s);
cudaError_t launchForbSums(BalanceData& bd, const LineSumArgs& a, cudaStream_t s);
cudaError_t launchLineCells(BalanceData& bd, const LineCellArgs& a, cudaStream_t s);
cudaError_t prepare(BalanceData& bd);
}  // namespace bal_f64
namespace bal_mixed {
cudaError_t prepare(BalanceData& bd);
cudaError_t buildCoolTable(const BalanceData& bd, float* tab, float* rtab, cudaStream_t s);
cudaError_t buildAlphaTable(const BalanceData& bd, float* tab, uint8_t* jump, cudaStream_t s);
cudaError_t launch(BalanceData& bd, const BalanceGrid& g, int maxRounds, cudaStream_t s, int atomSolves);
cudaError_t launchForLines(BalanceData& bd, const float* te, const float* ne, const float* ionDen,
                           const uint8_t* compute, float* forLines, cudaStream_t s);
}  // namespace bal_mixed

namespace {

// charge-exchange coefficients (Z, ion, a, b, c, d) of ionBalance and
// photoionisation (source/update_mod.f90:1649-1701, :3727-3779); the "Ca"
// rows are written into Ar's, as in the reference
const float kChexRows[][6] = {
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
    {18, 2, 1.e-5f, 0.f, 0.f, 0.f},               {18, 3, 4.57f, 0.27f, -0.18f, -1.57f},
    {18, 4, 6.37f, 2.12f, 10.21f, -6.22f},        {18, 3, 3.17e-2f, 2.12f, 12.06f, -0.40f},
    {18, 4, 2.68f, 0.69f, -0.68f, -4.47f},        {26, 2, 1.26f, 7.72e-2f, -0.41f, -7.31f},
    {26, 3, 3.42f, 0.51f, -2.06f, -8.99f}};

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
  for (auto& g : graph)
    if (g) cudaGraphExecDestroy(g);
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
  d.converge = 0;
  d.fixTe = 0;
  d.maxIterT = kRefRounds;
  d.resTol = (double)0.02f;
  d.stepMin = 0.2;
  d.xTol = 0.01f;
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
  // the J-free tail of getPhotoRates (radField(IPnuP) times the cross-section sums above the
  // secondary-ionisation threshold), summed once for the mixed balance
  {
    std::vector<float> tail(2 * std::max<size_t>(sh.size(), 1), 0.f);
    const double hcRyd = (double)2.1799153e-11f;
    for (size_t k = 0; k < sh.size(); ++k) {
      const PhotoShell& p = sh[k];
      if (!p.heavy || p.ipNuP < 1 || p.ipNuP > s.nbins) continue;
      const int iup = std::min(p.highNuP, s.nbins), ilow = std::max(p.ipNuP + 1, s.secIonP);
      double g = 0., h = 0.;
      for (int i = ilow; i <= iup; ++i) {
        const double ph = s.xSec[(size_t)(i + p.xsecP - p.ipNuP - 1)];
        g += ph / (hcRyd * (double)s.nu[(size_t)(i - 1)]);
        h += ph;
      }
      tail[2 * k] = (float)g;
      tail[2 * k + 1] = (float)h;
    }
    d.shellTail = (const float*)up(tail.data(), tail.size() * sizeof(float));
  }
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
  {
    // the rows diRec would end on (dielectronic, source/update_mod.f90:3204-3305)
    std::vector<int16_t> rows((size_t)31 * 32 * 3, -1);
    const int nd = (int)t.diel.size() / 8, na = (int)t.aldro.size() / 6;
    for (int r = 0; r < nd; ++r) {
      const float* q = t.diel.data() + (size_t)r * 8;
      const int elem = (int)q[0], ion = (int)q[0] + 1 - (int)q[1], g = (int)q[7];
      if (elem < 1 || elem > 30 || ion < 1 || ion > 31) continue;
      int16_t* x = rows.data() + ((size_t)elem * 32 + ion) * 3;
      if (g == 0 || g == 1) x[0] = (int16_t)r;
      if (g == 0 || g == 2) x[1] = (int16_t)r;
    }
    for (int r = 0; r < na; ++r) {
      const float* q = t.aldro.data() + (size_t)r * 6;
      const int elem = (int)q[0], ion = (int)q[0] - (int)q[1] + 1;
      if (elem < 1 || elem > 30 || ion < 1 || ion > 31) continue;
      rows[((size_t)elem * 32 + ion) * 3 + 2] = (int16_t)r;
    }
    d.dielRow = (const int16_t*)up(rows.data(), rows.size() * sizeof(int16_t));
  }
  std::vector<float4> chex(31 * 32, make_float4(0.f, 0.f, 0.f, 0.f));
  for (const auto& r : kChexRows)   // in order: later rows overwrite earlier ones
    chex[(int)r[0] * 32 + (int)r[1]] = make_float4(r[2], r[3], r[4], r[5]);
  d.chex = (const float4*)up(chex.data(), chex.size() * sizeof(float4));
  d.atomHdr = (const int32_t*)up(t.atomHdr.data(), t.atomHdr.size() * sizeof(int32_t));
  d.atomData = (const double*)up(t.atomData.data(), t.atomData.size() * sizeof(double));
  std::vector<float> atomF(t.atomData.begin(), t.atomData.end());
  d.atomDataF = (const float*)up(atomF.data(), atomF.size() * sizeof(float));
  // per upper level j the summed line factors sum_i a(j,i) E_ji of its lines
  // that carry positive power (the mixed path's cooling; equilibrium's loop
  // drops the others)
  std::vector<double> pow_((size_t)std::max(t.nAtoms, 1) * (kMaxLevels + 1), 0.);
  for (int a = 0; a < t.nAtoms; ++a) {
    const int32_t* h = t.atomHdr.data() + (size_t)a * kAtHdrSize;
    const int n = h[kAtNLev];
    const double* A = t.atomData.data() + h[kAtOffA];
    const double* Ev = t.atomData.data() + h[kAtOffE];
    const double atp = t.atomData[h[kAtOffAtp]];
    for (int i = 1; i <= n - 1; ++i)
      for (int j = i + 1; j <= n; ++j) {
        double aji = A[(size_t)(j - 1) * n + (i - 1)];
        if (aji == 0.) continue;
        if (j == h[kAtIup2p] && i == 1 && atp > 0.) aji = aji - atp;
        const double f = aji * (Ev[j - 1] - Ev[i - 1]);
        if (f > 0.) pow_[(size_t)a * (kMaxLevels + 1) + j] += f;
      }
  }
  d.linePow = (const double*)up(pow_.data(), pow_.size() * sizeof(double));
  const size_t nPair = (size_t)E * ns;
  d.ion = carve<double>(blocks, nPair * C1, err);
  const size_t nSh = std::max<size_t>(sh.size(), 1);
  d.gam = carve<double>(blocks, nSh * C1, err);
  d.heatA = carve<double>(blocks, nSh * C1, err);
  d.heatHi = carve<double>(blocks, nSh * C1, err);
  d.comp = carve<double>(blocks, 4 * (size_t)C1, err);
  double** scal[] = {&d.te, &d.ne, &d.xOld, &d.tHigh, &d.tLow, &d.resHigh, &d.resLow, &d.heat, &d.coolA,
                     &d.coolHex, &d.coolCollH, &d.compHeat, &d.compRecoil, &d.compCool, &d.resid};
  for (double** p : scal) *p = carve<double>(blocks, C1, err);
  d.forSum = carve<double>(blocks, (size_t)std::max(t.nAtoms, 1) * C1, err);
  d.coolAt = carve<CoolAt>(blocks, C1, err);
  d.nIterT = carve<int32_t>(blocks, C1, err);
  d.state = carve<int8_t>(blocks, C1, err);
  d.ibConv = carve<int8_t>(blocks, C1, err);
  d.side = carve<int8_t>(blocks, C1, err);
  d.counters = carve<BalanceCounters>(blocks, 1, err);
  d.list = carve<int32_t>(blocks, 2 * C1, err);
  d.listCount = carve<unsigned int>(blocks, kMaxRounds + 1, err);
  if ((int)blocks.size() > (int)(sizeof(bd->blocks) / sizeof(bd->blocks[0]))) err = "balance: too many device blocks";
  for (size_t i = 0; i < blocks.size() && i < sizeof(bd->blocks) / sizeof(bd->blocks[0]); ++i) bd->blocks[i] = blocks[i];
  bd->nBlocks = (int)std::min(blocks.size(), sizeof(bd->blocks) / sizeof(bd->blocks[0]));
  if (!err.empty()) return err;
  // no photon hit until the J pass says otherwise
  cudaMemset(d.state, 2, C1);
  // the rates kernel's shared memory per cell: ionDen, alphaTot, coll1 per
  // (element, stage), the shell rates, an ordered-sum scratch and the ladders
  {
    const int NP = d.nElemUsed * ns, nSh = d.nShellsTot;
    int nHeavy = 0;
    for (int e = 1; e <= d.nElemUsed; ++e) nHeavy += d.zOf[e] >= 3 ? 1 : 0;
    d.cellReals = 3 * NP + nSh + std::max(NP, nSh) + std::max(nHeavy * 3 * (ns + 3), 4 * d.nElemUsed);
    // the mixed build's per-heavy-element sums of the photoionisation rates, Auger band and charge exchange
    d.augReals = nHeavy * 13 * (ns + 1);
    d.cellRealsMixed = 3 * NP + nSh + std::max(NP, nSh) + std::max(nHeavy * (ns + 3), 4 * d.nElemUsed);
    // zOf, xref, abun (3 x 32 words) and the (element, ion) shell offsets and counts (2 x E x 32 int16)
    d.metaDoubles = (3 * 32 * 4 + 2 * d.nElemUsed * 32 * 2 + 7) / 8;
    // one warp (4 cells) per block must fit 200 KB in both builds; prepare() picks the block size
    const size_t cellBytes = std::max((size_t)d.cellReals * sizeof(double),
                                      ((size_t)d.cellRealsMixed + (size_t)d.augReals) * sizeof(float));
    if ((size_t)d.metaDoubles * sizeof(double) + 4 * cellBytes > 200 * 1024)
      return "balance: too many ions for the rates kernel";
    if (nHeavy > 32) return "balance: more than 32 heavy elements";
    cudaError_t e1 = bal_f64::prepare(*bd), e2 = bal_mixed::prepare(*bd);
    if (e1 != cudaSuccess || e2 != cudaSuccess) return "balance: cannot reserve the rates kernel's shared memory";
  }
  out = std::move(bd);
  return "";
}

void invalidateBalanceGraphs(BalanceData& bd);

// the cooling surfaces (ln G and B of every atom), once per context and before
// any graph capture that bakes their pointers in
cudaError_t ensureSurfaces(BalanceData& bd, cudaStream_t s) {
  const int slots = (int)(sizeof(bd.blocks) / sizeof(bd.blocks[0]));
  if (!bd.dev.alphaTab && bd.dev.nElemUsed > 0) {
    // the recombination coefficients of the mixed rates kernel
    if (bd.nBlocks + 2 > slots) return cudaErrorMemoryAllocation;
    const size_t n = (size_t)bd.dev.nElemUsed * bd.dev.nstages * kAlphaN;
    void* p = nullptr;
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&p, n * sizeof(float));
    if (e != cudaSuccess) return e;
    bd.blocks[bd.nBlocks++] = p;
    e = cudaMalloc(&q, n);
    if (e != cudaSuccess) return e;
    bd.blocks[bd.nBlocks++] = q;
    e = bal_mixed::buildAlphaTable(bd, (float*)p, (uint8_t*)q, s);
    if (e != cudaSuccess) return e;
    invalidateBalanceGraphs(bd);
    bd.dev.alphaTab = (const float*)p;
    bd.dev.alphaJump = (const uint8_t*)q;
  }
  if (bd.dev.nAtoms <= 0 || bd.dev.coolTab) return cudaSuccess;
  if (bd.nBlocks + 2 > slots) return cudaErrorMemoryAllocation;
  const size_t bytes = (size_t)bd.dev.nAtoms * kCoolNNe * kCoolNTe * sizeof(float);
  void* p = nullptr;
  void* q = nullptr;
  cudaError_t e = cudaMalloc(&p, bytes);
  if (e != cudaSuccess) return e;
  bd.blocks[bd.nBlocks++] = p;
  e = cudaMalloc(&q, bytes);
  if (e != cudaSuccess) return e;
  bd.blocks[bd.nBlocks++] = q;
  e = bal_mixed::buildCoolTable(bd, (float*)p, (float*)q, s);
  if (e != cudaSuccess) return e;
  invalidateBalanceGraphs(bd);
  bd.dev.coolTab = (const float*)p;
  bd.dev.recTab = (const float*)q;
  return cudaSuccess;
}

namespace {
bool sameGrid(const BalanceGrid& a, const BalanceGrid& b) {
  return a.jste == b.jste && a.hden == b.hden && a.te == b.te && a.ne == b.ne && a.ionDen == b.ionDen &&
         a.converged == b.converged && a.black == b.black && a.nIterT == b.nIterT;
}
}  // namespace

cudaError_t launchBalance(BalanceData& bd, const BalanceGrid& g, int maxRounds, int precision, cudaStream_t s,
                          int atomSolves, int converge, int fixTe) {
  // Te held only with the tight stopping rules (the ladder converged at the held Te); a cell mask
  // only for those evaluations
  bd.dev.fixTe = fixTe && converge ? 1 : 0;
  if (!bd.dev.fixTe) bd.dev.evalMask = nullptr;
  {
    // the stopping rules: the reference's, or tight ones at the level the precision resolves
    BalanceDev& d = bd.dev;
    const int want = converge ? 1 : 0;
    const bool mixed = precision == kBalMixed;
    const double resTol = want ? (mixed ? 1e-6 : 1e-9) : (double)0.02f;
    // with Te held the ladder is converged to the end of FP64 (the adjoint differences its results
    // over steps of 1e-3, and its slow modes leave 1e-9-converged ladders off by up to 1e-5)
    const float xTol = want ? (mixed ? 1e-5f : (bd.dev.fixTe ? 1e-14f : 1e-9f)) : 0.01f;
    if (d.converge != want || d.resTol != resTol || d.xTol != xTol) {
      d.converge = want;
      d.maxIterT = want ? kMaxRounds : kRefRounds;
      d.resTol = resTol;
      d.xTol = xTol;
      d.stepMin = want ? 1e-4 : 0.2;
      invalidateBalanceGraphs(bd);
    }
  }
  if (precision == kBalMixed && !atomSolves) {
    cudaError_t e = ensureSurfaces(bd, s);
    if (e != cudaSuccess) return e;
  }
  auto direct = [&]() {
    return precision == kBalMixed ? bal_mixed::launch(bd, g, maxRounds, s, atomSolves)
                                  : bal_f64::launch(bd, g, maxRounds, s, 1);
  };
  if (maxRounds != kRefRounds || atomSolves || converge || bd.dev.fixTe) return direct();
  const int k = precision == kBalMixed ? 1 : 0;
  if (bd.graph[k] && !sameGrid(bd.graphGrid[k], g)) {
    cudaGraphExecDestroy(bd.graph[k]);
    bd.graph[k] = nullptr;
  }
  if (!bd.graph[k]) {
    // capture the launches of one balance once; replays skip their launch overhead
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return direct();
    cudaError_t le = direct();
    e = cudaStreamEndCapture(s, &graph);
    if (le != cudaSuccess || e != cudaSuccess || !graph) {
      if (graph) cudaGraphDestroy(graph);
      cudaGetLastError();
      return direct();
    }
    e = cudaGraphInstantiate(&bd.graph[k], graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
      bd.graph[k] = nullptr;
      cudaGetLastError();
      return direct();
    }
    bd.graphGrid[k] = g;
  }
  return cudaGraphLaunch(bd.graph[k], s);
}

cudaError_t launchForLinesEmission(BalanceData& bd, const float* te, const float* ne, const float* ionDen,
                                   const uint8_t* compute, float* forLines, int precision, cudaStream_t s) {
  if (precision == kBalMixed) {
    cudaError_t e = ensureSurfaces(bd, s);
    if (e != cudaSuccess) return e;
  }
  return precision == kBalMixed ? bal_mixed::launchForLines(bd, te, ne, ionDen, compute, forLines, s)
                                : bal_f64::launchForLines(bd, te, ne, ionDen, compute, forLines, s);
}

cudaError_t launchForbLevelSums(BalanceData& bd, const LineSumArgs& a, cudaStream_t s) {
  return bal_f64::launchForbSums(bd, a, s);
}

cudaError_t launchLineCellLuminosities(BalanceData& bd, const LineCellArgs& a, cudaStream_t s) {
  return bal_f64::launchLineCells(bd, a, s);
}

void invalidateBalanceGraphs(BalanceData& bd) {
  for (auto& g : bd.graph)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
}

}  // namespace mcx
