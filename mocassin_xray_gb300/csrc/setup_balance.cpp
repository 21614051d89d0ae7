// setup_balance.cpp - reads the tables of the per-cell balance once:
//   makeCollIonData   source/hydro_mod.f90:13-33  (cion.dat)
//   makeAugerData     source/hydro_mod.f90:35-53  (auger.dat)
//   initRRDR          source/hydro_mod.f90:334-418 (rrBadnell.dat, drBadnell.dat)
//   radRecFit         source/update_mod.f90:3094-3202 (radrec.dat and the Fe fit table)
//   dielectronic      source/update_mod.f90:3204-3305 (dielectronic.dat, aldrovandi.dat)
//   makeElements      source/hydro_mod.f90:676-764 (fileNames.dat, lgDataAvailable)
//   equilibrium       source/emission_mod.f90:2589-2880 (the multi-level ion files)
// The reference re-reads dielectronic.dat, aldrovandi.dat and every ion file
// on each call; they are read here once and kept in packed tables.
#include "list_reader.h"
#include "setup_internal.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <fstream>
#include <stdexcept>

namespace mcx {

namespace {

[[noreturn]] void bfail(const std::string& msg) { throw std::runtime_error(msg); }

std::string baseNameOf(const std::string& f) {
  size_t s = f.find_last_of('/');
  return s == std::string::npos ? f : f.substr(s + 1);
}

std::string trim(const std::string& s) {
  size_t a = s.find_first_not_of(" \t\r");
  if (a == std::string::npos) return "";
  size_t b = s.find_last_not_of(" \t\r");
  return s.substr(a, b - a + 1);
}

// Natural cubic spline second derivatives (spline with yp1 = ypn = 1e30,
// source/interpolation_mod.f90:207-278), in FP64.
void naturalSpline(const double* x, const double* y, int n, double* y2) {
  std::vector<double> u(n, 0.);
  y2[0] = 0.;
  u[0] = 0.;
  for (int i = 1; i < n - 1; ++i) {
    if (x[i + 1] - x[i - 1] == 0. || x[i + 1] - x[i] == 0. || x[i] - x[i - 1] == 0.)
      bfail("spline: bad temperature points in an ion file");
    double sig = (x[i] - x[i - 1]) / (x[i + 1] - x[i - 1]);
    double p = sig * y2[i - 1] + 2.;
    y2[i] = (sig - 1.) / p;
    double t = y[i + 1];
    t = t - y[i];
    t = t / (x[i + 1] - x[i]);
    t = t - (y[i] - y[i - 1]) / (x[i] - x[i - 1]);
    u[i] = (6. * t / (x[i + 1] - x[i - 1]) - sig * u[i - 1]) / p;
  }
  y2[n - 1] = (0. - 0. * u[n - 2]) / (0. * y2[n - 2] + 1.);
  for (int k = n - 2; k >= 0; --k) y2[k] = y2[k] * y2[k + 1] + u[k];
}

bool isPowerLawRecFile(const std::string& dataFile) {
  static const char* names[] = {"data/ci.dat",  "data/ciii.dat", "data/ni.dat",  "data/neiv.dat", "data/oii.dat",
                                "data/oiii.dat", "data/nii.dat", "data/nev.dat", "data/niv.dat"};
  for (auto n : names) if (dataFile == n) return true;
  return false;
}

// Reads one ion file in the order and with the quirks of equilibrium
// (source/emission_mod.f90:2589-2880) and appends it to the packed tables.
void parseAtom(BalanceTables& b, const std::string& path, const std::string& dataFile, int elem, int ion) {
  ListReader r(path);
  const int numLines = (int)r.need(1)[0];
  r.skip(numLines);
  auto nl = r.need(2);
  const int nLev = (int)nl[0], nTemp = (int)nl[1];
  if (nLev < 1 || nLev > kMaxLevels) bfail("equilibrium: unsupported number of levels in " + path);
  if (nTemp < 1 || nTemp > 64) bfail("equilibrium: unsupported number of temperature points in " + path);
  r.skip(nLev);                                     // labels, format (A20)
  std::vector<double> logT(nTemp);
  for (int i = 0; i < nTemp; ++i) logT[i] = std::log10(r.need(1)[0]);
  r.need(1);                                        // iRats
  // collision strengths: qom(k, ilow, iup), continuation lines carry "0 0"
  std::vector<double> qom((size_t)nTemp * nLev * nLev, 0.);
  auto Q = [&](int k, int l, int u) -> double& { return qom[((size_t)(l - 1) * nLev + (u - 1)) * nTemp + (k - 1)]; };
  int ilow1 = 0, iup1 = 0, k = 0;
  for (int it = 0; it < 10000; ++it) {
    auto v = r.need(3);
    int il = (int)v[0], iu = (int)v[1];
    double qx = v[2];
    if (qx == 0.) break;
    if (il == 0) { il = ilow1; ++k; } else { ilow1 = il; k = 1; }
    if (iu == 0) iu = iup1; else iup1 = iu;
    if (k < 1 || k > nTemp || il < 1 || il > nLev || iu < 1 || iu > nLev)
      bfail("equilibrium: collision strength index out of range in " + path);
    Q(k, il, iu) = qx;
  }
  // transition probabilities a(j,i), two-photon rows have negative indices
  std::vector<double> a((size_t)nLev * nLev, 0.);
  auto A = [&](int j, int i) -> double& { return a[(size_t)(j - 1) * nLev + (i - 1)]; };
  double atp = 0.;
  int iup2p = -1, jj = 0;
  for (int kk = 1; kk <= nLev - 1; ++kk) {
    for (int l = kk + 1; l <= nLev; ++l) {
      auto v = r.need(3);
      int i = (int)v[0], j = (int)v[1];
      double ax = v[2];
      if (i < 0 && j < 0) {
        atp = ax;
        iup2p = -j;
        i = -i;
        j = -j;
        if (i > nLev || j > nLev) bfail("equilibrium: transition index out of range in " + path);
        if (A(j, i) > 0.) ++jj;
        A(j, i) = A(j, i) + atp;
      } else if (i > 0 && j > 0) {
        if (i > nLev || j > nLev) bfail("equilibrium: transition index out of range in " + path);
        A(j, i) = ax;
      } else {
        bfail("equilibrium: insane transition probability in " + path);
      }
    }
  }
  for (int kk = 1; kk <= jj; ++kk) {
    auto v = r.need(3);
    int i = (int)v[0], j = (int)v[1];
    if (i < 1 || j < 1 || i > nLev || j > nLev) bfail("equilibrium: transition index out of range in " + path);
    A(j, i) = v[2];
  }
  // statistical weights and energies [1/cm]; equal neighbours are nudged by 0.1
  std::vector<double> g(nLev, 0.), e(nLev, 0.);
  for (int j = 1; j <= nLev; ++j) {
    auto v = r.need(3);
    int i = (int)v[0];
    if (i < 1 || i > nLev) bfail("equilibrium: level index out of range in " + path);
    g[i - 1] = (double)(int)v[1];
    e[i - 1] = v[2];
    if (i > 1 && e[i - 1] == e[i - 2]) e[i - 1] = e[i - 1] + 0.1;
  }
  // recombination-coefficient fits (read when rec = .true.)
  int recType = isPowerLawRecFile(dataFile) ? kRecPowerLaw : kRecChianti;
  std::vector<double> rec;
  int nRec = 0;
  if (recType == kRecPowerLaw) {
    std::vector<double> last(11, 0.);
    for (int j = 2; j <= nLev; ++j) {
      // one list-directed READ of br, z, a_r(4), a_d(5): blank records are
      // passed over, a record with a non-numeric item is a READ error that
      // leaves the eleven values as they were (gfortran), end of file leaves the loop
      std::vector<double> v;
      bool eofHit = false, err = false;
      while ((int)v.size() < 11) {
        if (r.eof()) { eofHit = true; break; }
        std::string line = r.record();
        size_t i = 0;
        while (i < line.size() && (int)v.size() < 11) {
          while (i < line.size() && (line[i] == ' ' || line[i] == '\t' || line[i] == ',' || line[i] == '\r')) ++i;
          if (i >= line.size()) break;
          size_t e = i;
          while (e < line.size() && !(line[e] == ' ' || line[e] == '\t' || line[e] == ',' || line[e] == '\r')) ++e;
          double x;
          if (!ListReader::number(line.substr(i, e - i), x)) { err = true; break; }
          v.push_back(x);
          i = e;
        }
        if (err) break;
      }
      if (eofHit) break;
      if (!err) last = v;
      rec.insert(rec.end(), last.begin(), last.end());
      ++nRec;
    }
  } else {
    for (int j = 2; j <= nLev; ++j) {
      std::vector<double> v;
      if (!r.read(5, v)) {
        // end of file before a complete record: the reference's READ of jj
        // meets end of file (or a partial last record) and leaves the loop
        break;
      }
      int jjr = (int)v[0];
      if (jjr == -9999) break;
      if (jjr > nLev) break;
      if (jjr < 1) bfail("equilibrium: bad level in the recombination fits of " + path);
      rec.insert(rec.end(), v.begin(), v.end());
      ++nRec;
    }
  }

  // pack
  const int nPairs = nLev * (nLev - 1) / 2;
  std::vector<int32_t> h(kAtHdrSize, 0);
  h[kAtElem] = elem; h[kAtIon] = ion; h[kAtNLev] = nLev; h[kAtNTemp] = nTemp;
  h[kAtIup2p] = iup2p; h[kAtRecType] = nRec > 0 ? recType : kRecNone; h[kAtNRec] = nRec;
  auto& d = b.atomData;
  h[kAtOffLogT] = (int32_t)d.size(); d.insert(d.end(), logT.begin(), logT.end());
  h[kAtOffQom] = (int32_t)d.size();
  for (int l = 1; l <= nLev - 1; ++l)
    for (int u = l + 1; u <= nLev; ++u)
      for (int kk = 1; kk <= nTemp; ++kk) d.push_back(Q(kk, l, u));
  h[kAtOffY2] = (int32_t)d.size();
  d.resize(d.size() + (size_t)nPairs * nTemp, 0.);
  if (nTemp > 2) {
    for (int p = 0; p < nPairs; ++p)
      naturalSpline(logT.data(), &d[h[kAtOffQom] + (size_t)p * nTemp], nTemp, &d[h[kAtOffY2] + (size_t)p * nTemp]);
  }
  h[kAtOffA] = (int32_t)d.size(); d.insert(d.end(), a.begin(), a.end());
  h[kAtOffG] = (int32_t)d.size(); d.insert(d.end(), g.begin(), g.end());
  h[kAtOffE] = (int32_t)d.size(); d.insert(d.end(), e.begin(), e.end());
  h[kAtOffRec] = (int32_t)d.size(); d.insert(d.end(), rec.begin(), rec.end());
  h[kAtOffAtp] = (int32_t)d.size(); d.push_back(atp);
  b.atomHdr.insert(b.atomHdr.end(), h.begin(), h.end());
  b.atomIndex[elem - 1][ion - 1] = b.nAtoms++;
  if (nLev > b.maxLev) b.maxLev = nLev;
}

}  // namespace

void buildBalanceTables(Setup& s) {
  BalanceTables& b = s.bal;
  const std::string& D = s.dataDir;
  for (auto& row : b.atomIndex) for (auto& v : row) v = -1;

  // makeCollIonData: CF(1:5, elem, nElec) for nElec = elem..1, then cionTherm
  {
    ListReader r(D + "/cion.dat");
    for (int elem = 1; elem <= kNElements; ++elem)
      for (int ne = elem; ne >= 1; --ne) {
        auto v = r.need(5);
        for (int i = 0; i < 5; ++i) b.CF[elem - 1][ne - 1][i] = (float)v[i];
      }
    r.skip(2);
    for (int elem = 3; elem <= kNElements; ++elem) {
      auto v = r.need(elem);
      for (int ion = 1; ion <= elem; ++ion) b.cionTherm[elem - 1][ion - 1] = (float)v[ion - 1];
    }
  }
  // makeAugerData: 1696 records of (elem, ion, shell, nelec) + 10 yields
  {
    ListReader r(D + "/auger.dat");
    for (int i = 0; i < 1696; ++i) {
      auto h = r.need(4);
      int elem = (int)h[0], ion = (int)h[1], shell = (int)h[2], nelec = (int)h[3];
      if (elem < 1 || elem > 30 || ion < 1 || ion > 30 || shell < 1 || shell > 10)
        bfail("makeAugerData: index out of range in auger.dat");
      b.nauger[elem - 1][ion - 1][shell - 1] = nelec;
      auto y = r.need(10);
      for (int j = 0; j < 10; ++j) b.auger[elem - 1][ion - 1][shell - 1][j] = (float)y[j];
    }
  }
  // initRRDR
  {
    ListReader r(D + "/rrBadnell.dat");
    r.skip(2);
    std::vector<double> v;
    for (int i = 0; i < 100000; ++i) {
      if (!r.read(10, v)) break;
      int z = (int)v[0], n = (int)v[1], m = (int)v[2];
      if (z <= 30 && m == 1) {
        if (z < 1 || n < 0 || n > 30) bfail("initRRDR: index out of range in rrBadnell.dat");
        for (int k = 0; k < 6; ++k) b.RRb[k][z - 1][n] = (float)v[4 + k];
      }
    }
  }
  {
    ListReader r(D + "/drBadnell.dat");
    r.skip(2);
    std::vector<double> v;
    for (int blk = 0; blk < 2; ++blk) {
      if (blk == 1) r.skip(1);
      for (int i = 0; i < 919; ++i) {
        if (!r.read(13, v)) break;
        int z = (int)v[0], n = (int)v[1], m = (int)v[2];
        if (z <= 30 && m == 1) {
          if (z < 1 || n < 0 || n > 30) bfail("initRRDR: index out of range in drBadnell.dat");
          for (int j = 0; j < 9; ++j) (blk == 0 ? b.DRbC : b.DRbE)[z - 1][n][j] = (float)v[4 + j];
        }
      }
    }
  }
  // radRecFit's first-call read of radrec.dat
  {
    ListReader r(D + "/radrec.dat");
    std::vector<double> v;
    auto rd = [&](float* dst, int n) {
      if (!r.read(n, v)) bfail("radRecFit: radrec.dat truncated");
      for (int i = 0; i < n; ++i) dst[i] = (float)v[i];
    };
    for (int ion = 4; ion <= 30; ++ion)
      if (ion != 11)
        for (int elem = ion; elem <= 30; ++elem)
          if (elem != 26 || ion >= 14) rd(b.rrec[elem - 1][ion - 1], 2);
    for (int ion = 1; ion <= 3; ++ion)
      for (int elem = ion; elem <= 30; ++elem) rd(b.rnew[elem - 1][ion - 1], 4);
    for (int elem = 11; elem <= 30; ++elem) rd(b.rnew[elem - 1][10], 4);
    for (int ion = 4; ion <= 10; ++ion) {
      for (int elem = std::max(6, ion); elem <= 8; ++elem) rd(b.rnew[elem - 1][ion - 1], 4);
      rd(b.rnew[9][ion - 1], 4);
    }
    for (int ion = 12; ion <= 26; ++ion) rd(b.rnew[25][ion - 1], 4);
  }
  // dielectronic: dielectronic.dat (elem, n, a, b, c, d, f, g) and aldrovandi.dat (elem, n, a, b, t0, t1)
  {
    ListReader r(D + "/dielectronic.dat");
    std::vector<double> v;
    for (int i = 0; i < 10000; ++i) {
      if (!r.read(8, v)) break;
      for (double x : v) b.diel.push_back((float)x);
    }
    ListReader ra(D + "/aldrovandi.dat");
    for (int i = 0; i < 100000; ++i) {
      if (!ra.read(6, v)) break;
      for (double x : v) b.aldro.push_back((float)x);
    }
  }
  // getOuterShell for every (z, nElec)
  for (int z = 1; z <= kNElements; ++z)
    for (int ne = 1; ne <= z; ++ne) {
      int os, g0, g1;
      getOuterShell(z, ne, os, g0, g1);
      b.outer[z - 1][ne - 1][0] = os;
      b.outer[z - 1][ne - 1][1] = g0;
      b.outer[z - 1][ne - 1][2] = g1;
    }
  // makeElements: ion file names, then lgDataAvailable = the file opens
  {
    std::ifstream in(D + "/fileNames.dat");
    if (!in) bfail("makeElements: can't open data/fileNames.dat");
    std::string line;
    const int nst = s.p.nstages;
    for (int elem = 3; elem <= kNElements; ++elem) {
      for (int ion = 1; ion <= std::min(elem + 1, 31); ++ion) {
        if (!std::getline(in, line)) bfail("makeElements: fileNames.dat truncated");
        std::string name = trim(line.substr(0, std::min<size_t>(20, line.size())));
        if (!s.elemOn[elem - 1] || ion > std::min(elem + 1, nst) || ion > kNElements + 1) continue;
        std::string path = D + "/" + baseNameOf(name);
        std::ifstream probe(path);
        if (!probe) continue;
        parseAtom(b, path, name, elem, ion);
      }
    }
  }
}

}  // namespace mcx
