// setup_dust.cpp - grain data of a dust deck, read once:
//   makeDustXsec     source/ph_mod.f90:938-1720 (grain-species list, size
//                    distribution, 'Q'-type efficiency files mapped onto the
//                    frequency mesh, cross sections pi a^2 Q)
//   dustEmissionInt  source/dust_mod.f90:141-184 (emission integral of every
//                    species and size for T = 1..nTemps K)
//   getQs            source/ph_mod.f90:1601-1650 ('nk'-type files: optical
//                    constants, the efficiencies of every size and bin from a
//                    Mie calculation or geometric optics)
#include "list_reader.h"
#include "setup_internal.h"

#include <cmath>
#include <complex>
#include <fstream>
#include <sstream>
#include <stdexcept>

namespace mcx {

namespace {

[[noreturn]] void dfail(const std::string& msg) { throw std::runtime_error(msg); }

constexpr float kC = 2.9979250e10f;       // constants_mod.f90:12
constexpr float kFr1Ryd = 3.28984e15f;    // constants_mod.f90:13
constexpr float kHPlanckD = 6.6262e-27f;  // constants_mod.f90:14
constexpr float kPiD = 3.141592654f;

std::string joinDir(const std::string& dir, const std::string& f) {
  if (f.empty() || f[0] == '/' || dir.empty()) return f;
  return dir + "/" + f;
}

// one record's tokens (blank/comma separated, quotes stripped)
std::vector<std::string> tokensOf(const std::string& line) {
  std::vector<std::string> out;
  size_t i = 0;
  while (i < line.size()) {
    while (i < line.size() && (line[i] == ' ' || line[i] == '\t' || line[i] == ',' || line[i] == '\r')) ++i;
    if (i >= line.size()) break;
    if (line[i] == '\'' || line[i] == '"') {
      size_t j = line.find(line[i], i + 1);
      if (j == std::string::npos) j = line.size();
      out.push_back(line.substr(i + 1, j - i - 1));
      i = j + 1;
      continue;
    }
    size_t j = i;
    while (j < line.size() && !(line[j] == ' ' || line[j] == '\t' || line[j] == ',' || line[j] == '\r')) ++j;
    out.push_back(line.substr(i, j - i));
    i = j;
  }
  return out;
}

double num(const std::string& t, const std::string& what) {
  double v;
  if (!ListReader::number(t, v)) dfail("makeDustXsec: expected a number in " + what + ", got '" + t + "'");
  return v;
}

// linearMap (source/interpolation_mod.f90:111-131) with the reference's locate
void linearMap(const std::vector<float>& y, const std::vector<float>& x, const float* xNew, int nNew, float* yNew) {
  const int nx = (int)x.size();
  for (int i = 0; i < nNew; ++i) {
    int ii = locate(x.data(), nx, xNew[i]);
    if (ii == 0) yNew[i] = y[0];
    else if (ii == nx) yNew[i] = y[nx - 1];
    else yNew[i] = y[ii - 1] + (y[ii] - y[ii - 1]) * (xNew[i] - x[ii - 1]) / (x[ii] - x[ii - 1]);
  }
}

}  // namespace

float blackbodyFlux(float energy, float temperature) {
  const float hcRyd_k = 157893.94f;
  float constant = 0.5250229f / kHPlanckD;
  if (hcRyd_k * energy / temperature > 86.f)
    return constant * energy * energy * energy * expf(-hcRyd_k * energy / temperature);
  float denominator = expf(hcRyd_k * energy / temperature) - 1.f;
  if (denominator <= 0.f) return 3.32154e-6f * energy * energy * temperature / kHPlanckD;
  return constant * energy * energy * energy / denominator;
}

// Extinction, scattering and backscattering efficiencies of a homogeneous
// sphere of size parameter x and complex refractive index m: the series of
// Mie coefficients a_n, b_n as organised by Bohren & Huffman (1983,
// Absorption and Scattering of Light by Small Particles, appendix A):
// D_n(mx) = d/dz ln psi_n(z) by downward recurrence from n = max(nstop,
// |mx|) + 15, the Riccati-Bessel functions psi_n and chi_n of x by upward
// recurrence, summed to nstop = x + 4 x^(1/3) + 2 terms.
void mieEfficiencies(double x, std::complex<double> m, double& qext, double& qsca, double& qback) {
  using cd = std::complex<double>;
  const cd y = m * x;
  const double xstop = x + 4.0 * std::cbrt(x) + 2.0;
  const int nstop = (int)xstop;
  const int nmx = (int)std::max(xstop, std::abs(y)) + 15;
  std::vector<cd> D((size_t)nmx + 1, cd(0., 0.));
  for (int n = nmx; n >= 1; --n) {
    const double en = n;
    D[(size_t)n - 1] = en / y - 1.0 / (D[(size_t)n] + en / y);
  }
  double psi0 = std::cos(x), psi1 = std::sin(x);
  double chi0 = -std::sin(x), chi1 = std::cos(x);
  cd xi1(psi1, -chi1);
  double sumExt = 0., sumSca = 0.;
  cd sumBack(0., 0.);
  double sign = -1.;
  for (int n = 1; n <= nstop; ++n) {
    const double en = n, fn = 2. * en + 1.;
    const double psi = (2. * en - 1.) * psi1 / x - psi0;
    const double chi = (2. * en - 1.) * chi1 / x - chi0;
    const cd xi(psi, -chi);
    const cd da = D[(size_t)n] / m + en / x, db = m * D[(size_t)n] + en / x;
    const cd an = (da * psi - psi1) / (da * xi - xi1);
    const cd bn = (db * psi - psi1) / (db * xi - xi1);
    sumSca += fn * (std::norm(an) + std::norm(bn));
    sumExt += fn * (an.real() + bn.real());
    sumBack += fn * sign * (an - bn);
    sign = -sign;
    psi0 = psi1; psi1 = psi;
    chi0 = chi1; chi1 = chi;
    xi1 = cd(psi1, -chi1);
  }
  qsca = 2. / (x * x) * sumSca;
  qext = 2. / (x * x) * sumExt;
  qback = std::norm(sumBack) / (x * x);
}

// geometricOptics (source/ph_mod.f90:1700-1750): absorption by a sphere much
// larger than the wavelength, from the Fresnel reflectivities over 45
// incidence angles, and scattering from the Rayleigh-Gans efficiency
// saturated as Qrg / sqrt(1 + Qrg^2 / 4), minus the absorption.  The
// reference reads the refraction angle psi before the first angle sets it
// (taken as 0 here) and takes 1/m's permittivity as (epsre, -epsre) / |eps|^2.
void geometricOptics(float x, float a, float mre, float mim, float lambda, float& qa, float& qs) {
  const float pi = 3.141592654f;
  const float absmm1sq = (mre - 1.f) * (mre - 1.f) + mim * mim;
  const float epsre = mre * mre - mim * mim, epsim = mre * mim;
  const float epsrem1 = epsre / (epsre * epsre + epsim * epsim);
  const float epsimm1 = -(epsre / (epsre * epsre + epsim * epsim));
  qa = 0.f;
  float psi = 0.f;
  for (int i = 1; i <= 45; ++i) {
    const float t0 = (float)i * pi / 180.f, s0 = std::sin(t0), c0 = std::cos(t0);
    const float p20 = 0.5f * (s0 * s0 - epsre + std::sqrt((2.f * epsim) * (2.f * epsim) + (epsre - s0 * s0)));
    const float q20 = 0.5f * (-s0 * s0 + epsre + std::sqrt((2.f * epsim) * (2.f * epsim) + (epsre - s0 * s0)));
    const float sp = std::sin(psi);
    const float p21 = 0.5f * (sp * sp - epsrem1 + std::sqrt((2.f * epsimm1) * (2.f * epsimm1) + (epsrem1 - sp * sp)));
    const float q21 = 0.5f * (-sp * sp + epsrem1 + std::sqrt((2.f * epsimm1) * (2.f * epsimm1) + (epsrem1 - sp * sp)));
    const float rq20 = std::sqrt(q20);
    const float rperp0 = ((rq20 - c0) * (rq20 - c0) + p20) / ((rq20 + c0) * (rq20 + c0) + p20);
    const float rpara0 = rperp0 * ((rq20 - s0 * std::tan(t0)) * (rq20 - s0 * std::tan(t0)) + p20) /
                         ((rq20 + s0 * std::tan(t0)) * (rq20 + s0 * std::tan(t0)) + p20);
    psi = std::asin(s0 / ((q20 + s0 * s0) * (q20 + s0 * s0)));
    const float sps = std::sin(psi), cps = std::cos(psi), rq21 = std::sqrt(q21);
    const float rperp1 = ((rq21 - cps) * (rq21 - cps) + p21) / ((rq21 + cps) * (rq21 + cps) + p21);
    const float rpara1 = rperp1 * ((rq21 - sps * std::tan(psi)) * (rq21 - sps * std::tan(psi)) + p21) /
                         ((rq21 + sps * std::tan(psi)) * (rq21 + sps * std::tan(psi)) + p21);
    const float at = std::exp(-8.f * pi * a * mim * cps / lambda);
    qa = qa + s0 * c0 * (pi / 180.f) * (1.f - at) *
                  ((1.f - rperp0) / (1.f - at * rperp1) + (1.f - rpara0) / (1.f - at * rpara1));
  }
  const float qrg = (32.f * absmm1sq * x * x * x * x) / (27.f + 16.f * x * x) + (8.f / 3.f) * mim * x;
  qs = qrg / std::sqrt(1.f + 0.25f * qrg * qrg) - qa;
}

// getQs (source/ph_mod.f90:1601-1650): absorption and scattering efficiencies
// of every grain size in every frequency bin from the refractive index
// mapped onto the mesh.  Mie below |m| x = 1000 (x capped at 100), the
// Rayleigh-Gans limit when also |m - 1| x < 1e-3, geometric optics above.
void efficienciesFromIndex(const Setup& s, const std::vector<float>& ere, const std::vector<float>& eim,
                           float* qabs, float* qsca) {
  const DustTables& d = s.dust;
  const int nb = s.nbins;
  for (int i = 0; i < nb; ++i) {
    const float absM = std::sqrt(ere[i] * ere[i] + eim[i] * eim[i]);
    const float absMm1 = std::sqrt((ere[i] - 1.f) * (ere[i] - 1.f) + eim[i] * eim[i]);
    const float lam = 2.9979250e14f / (s.nu[i] * kFr1Ryd);
    for (int ai = 0; ai < d.nSizes; ++ai) {
      float x = 2.0f * 3.14159265f * d.grainRadius[ai] / lam;
      float qa, qs;
      if (absM * x < 1000.f) {
        if (x > 100.f) x = 100.f;
        double qe, qsc, qb;
        mieEfficiencies((double)x, std::complex<double>(ere[i], eim[i]), qe, qsc, qb);
        qa = (float)(qe - qsc);
        qs = (float)qsc;
      } else if (absMm1 * x < 0.001f) {
        qa = (8.f / 3.f) * eim[i] * x;
        qs = 32.f * absMm1 * absMm1 * x * x * x * x / (27.f + 16.f * x * x);
      } else {
        geometricOptics(x, d.grainRadius[ai], ere[i], eim[i], lam, qa, qs);
      }
      if (!s.p.lgDustScattering) qs = 0.f;
      qabs[(size_t)ai * nb + i] = qa;
      qsca[(size_t)ai * nb + i] = qs;
    }
  }
}

void buildDustTables(Setup& s) {
  DustTables& d = s.dust;
  const int nb = s.nbins;
  const float* nu = s.nu.data();
  // grain-species list and size distribution
  ListReader species(joinDir(s.p.baseDir, s.p.dustFile[0]));
  d.nSpecies = (int)species.need(1)[0];
  if (d.nSpecies < 1 || d.nSpecies > 64) dfail("makeDustXsec: invalid number of grain species");
  ListReader sizes(joinDir(s.p.baseDir, s.p.dustFile[1]));
  d.nSizes = (int)sizes.need(1)[0];
  if (d.nSizes < 1 || d.nSizes > 256) dfail("makeDustXsec: invalid nSizes");
  d.grainRadius.assign(d.nSizes, 0.f);
  d.grainWeight.assign(d.nSizes, 0.f);
  d.da.assign(d.nSizes, 0.f);
  for (int ai = 0; ai < d.nSizes; ++ai) {
    auto v = sizes.need(3);
    d.grainRadius[ai] = (float)v[1];
    d.grainWeight[ai] = (float)v[2];
  }
  if (d.nSizes > 1) {
    d.da[0] = d.grainRadius[1] - d.grainRadius[0];
    for (int ai = 1; ai < d.nSizes - 1; ++ai) d.da[ai] = (d.grainRadius[ai + 1] - d.grainRadius[ai - 1]) / 2.f;
    d.da[d.nSizes - 1] = d.grainRadius[d.nSizes - 1] - d.grainRadius[d.nSizes - 2];
    float normWeight = 0.f;
    for (int ai = 0; ai < d.nSizes; ++ai) normWeight = normWeight + d.grainWeight[ai] * d.da[ai];
    for (int ai = 0; ai < d.nSizes; ++ai) {
      d.grainWeight[ai] = (d.grainWeight[ai] * d.da[ai]) / normWeight;
      if (!(d.grainWeight[ai] >= 0.f)) dfail("makeDustXSec: invalid grain weight");
    }
  } else {
    d.grainWeight[0] = 1.f;
  }
  const size_t per = (size_t)d.nSizes * nb;
  d.Cabs.assign((size_t)d.nSpecies * per, 0.f);
  d.Csca.assign((size_t)d.nSpecies * per, 0.f);
  d.gCos.assign((size_t)d.nSpecies * per, 0.f);
  d.grainAbun.assign(d.nSpecies, 0.f);
  d.TdustSublime.assign(d.nSpecies, 0.f);
  d.grainLabel.assign(d.nSpecies, "");
  for (int n = 0; n < d.nSpecies; ++n) {
    auto t = tokensOf(species.record());
    while (t.empty()) t = tokensOf(species.record());
    if (t.size() < 2) dfail("makeDustXsec: species record needs a file name and an abundance");
    const std::string qfile = joinDir(s.p.baseDir, t[0]);
    d.grainAbun[n] = (float)num(t[1], "the grain-species file");
    ListReader q(qfile);
    auto head = tokensOf(q.record());
    if (head.empty()) dfail("makeDustXsec: empty extinction file " + qfile);
    if (head[0] == "nk") {
      // makeDustXsec's 'nk' branch (source/ph_mod.f90:1088-1230): label line, then
      // wavelength [um], n, k per record, wavelengths ascending
      auto lab = tokensOf(q.record());
      if (lab.size() < 5) dfail("makeDustXsec: species header of " + qfile + " needs label, Tsub, rho, Vn, Msurf");
      d.grainLabel[n] = lab[0];
      d.TdustSublime[n] = (float)num(lab[1], qfile);
      std::vector<float> wav, re, im;
      std::vector<double> v;
      while (!q.eof()) {
        const int got = q.readRecord(3, v);
        if (got < 0) break;
        if (v.size() < 3) continue;
        wav.push_back((float)v[0]); re.push_back((float)v[1]); im.push_back((float)v[2]);
      }
      const int nWav = (int)wav.size();
      if (nWav < 2) dfail("makeDustXsec: no optical constants in " + qfile);
      // wavelength [um] to energy [Ryd], reversed into ascending energy
      std::vector<float> e(nWav), r(nWav), k(nWav);
      for (int i = 0; i < nWav; ++i) {
        e[nWav - 1 - i] = kC / (wav[i] * kFr1Ryd * 1.e-4f);
        r[nWav - 1 - i] = re[i];
        k[nWav - 1 - i] = im[i];
      }
      std::vector<float> ere(nb), eim(nb);
      linearMap(r, e, nu, nb, ere.data());
      linearMap(k, e, nu, nb, eim.data());
      efficienciesFromIndex(s, ere, eim, &d.Cabs[(size_t)n * per], &d.Csca[(size_t)n * per]);
      continue;
    }
    if (head[0] != "Q") dfail("makeDustXsec: invalid dustFileType in " + qfile);
    auto lab = tokensOf(q.record());
    if (lab.size() < 5) dfail("makeDustXsec: species header of " + qfile + " needs label, Tsub, rho, Vn, Msurf");
    d.grainLabel[n] = lab[0];
    d.TdustSublime[n] = (float)num(lab[1], qfile);
    q.skip(2);
    const int nRadii = (int)q.need(1)[0];
    const int nWav = (int)q.need(1)[0];
    q.skip(1);
    if (nRadii < 1 || nWav < 2) dfail("makeDustXsec: invalid NRAD/NWAV in " + qfile);
    std::vector<float> agrain(nRadii), wav(nWav), qa(nWav), qs(nWav), gg(nWav);
    std::vector<float> t1((size_t)nRadii * nb), t2((size_t)nRadii * nb), t3((size_t)nRadii * nb);
    for (int i = 0; i < nRadii; ++i) {
      for (int j = 0; j < nWav; ++j) {
        auto v = q.need(5);
        agrain[i] = (float)v[0];
        wav[j] = (float)v[1];
        qa[j] = (float)v[2];
        qs[j] = (float)v[3];
        gg[j] = (float)v[4];
      }
      // wavelength [um] to energy [Ryd], same order as in the file
      for (int j = 0; j < nWav; ++j) wav[j] = kC / (wav[j] * kFr1Ryd * 1.e-4f);
      linearMap(qa, wav, nu, nb, &t1[(size_t)i * nb]);
      linearMap(qs, wav, nu, nb, &t2[(size_t)i * nb]);
      linearMap(gg, wav, nu, nb, &t3[(size_t)i * nb]);
    }
    for (int ai = 0; ai < d.nSizes; ++ai) {
      float* ca = &d.Cabs[(size_t)n * per + (size_t)ai * nb];
      float* cs = &d.Csca[(size_t)n * per + (size_t)ai * nb];
      float* cg = &d.gCos[(size_t)n * per + (size_t)ai * nb];
      const int iSize = locate(agrain.data(), nRadii, d.grainRadius[ai]);
      if (d.grainRadius[ai] < agrain[0]) {
        for (int j = 0; j < nb; ++j) { ca[j] = t1[j]; cs[j] = t2[j]; cg[j] = t3[j]; }
      } else if (d.grainRadius[ai] > agrain[nRadii - 1]) {
        const size_t o = (size_t)(nRadii - 1) * nb;
        for (int j = 0; j < nb; ++j) { ca[j] = t1[o + j]; cs[j] = t2[o + j]; cg[j] = t3[o + j]; }
      } else {
        const size_t o0 = (size_t)(iSize - 1) * nb, o1 = (size_t)iSize * nb;
        const float f = agrain[iSize - 1], g1 = iSize < nRadii ? agrain[iSize] : agrain[iSize - 1];
        for (int j = 0; j < nb; ++j) {
          if (iSize >= nRadii) { ca[j] = t1[o0 + j]; cs[j] = t2[o0 + j]; cg[j] = t3[o0 + j]; continue; }
          ca[j] = t1[o0 + j] + (d.grainRadius[ai] - f) * (t1[o1 + j] - t1[o0 + j]) / (g1 - f);
          cs[j] = t2[o0 + j] + (d.grainRadius[ai] - f) * (t2[o1 + j] - t2[o0 + j]) / (g1 - f);
          cg[j] = t3[o0 + j] + (d.grainRadius[ai] - f) * (t3[o1 + j] - t3[o0 + j]) / (g1 - f);
        }
      }
    }
  }
  // cross sections pi a^2 Q [cm^2] and their abundance- and size-weighted sums
  d.CTabs.assign(nb, 0.f);
  d.CTsca.assign(nb, 0.f);
  for (int i = 0; i < nb; ++i)
    for (int n = 0; n < d.nSpecies; ++n)
      for (int ai = 0; ai < d.nSizes; ++ai) {
        const size_t o = (size_t)n * per + (size_t)ai * nb + i;
        d.Csca[o] = d.Csca[o] * kPiD * d.grainRadius[ai] * d.grainRadius[ai] * 1.e-8f;
        d.Cabs[o] = d.Cabs[o] * kPiD * d.grainRadius[ai] * d.grainRadius[ai] * 1.e-8f;
        d.CTsca[i] = d.CTsca[i] + d.grainAbun[n] * d.Csca[o] * d.grainWeight[ai];
        d.CTabs[i] = d.CTabs[i] + d.grainAbun[n] * d.Cabs[o] * d.grainWeight[ai];
      }
  // dustEmissionInt
  d.emIntegral.assign((size_t)d.nSpecies * d.nSizes * kNTemps, 0.f);
  for (int n = 0; n < d.nSpecies; ++n)
    for (int ai = 0; ai < d.nSizes; ++ai)
      for (int nT = 1; nT <= kNTemps; ++nT) {
        float acc = 0.f;
        for (int i = 0; i < nb; ++i) {
          float bb = blackbodyFlux(nu[i], (float)nT);
          acc = acc + d.Cabs[(size_t)n * per + (size_t)ai * nb + i] * bb * kFr1Ryd * s.widFlx[i];
        }
        d.emIntegral[((size_t)n * d.nSizes + ai) * kNTemps + (nT - 1)] = acc * kHPlanckD * 4.f;
      }
}

}  // namespace mcx
