// setup_emission.cpp - reads the tables of the emission phase once:
//   initGammaCont      source/ph_mod.f90:31-200 (gammaHI/HeI/HeII.dat, edge pointers)
//   initCartesianGrid  source/grid_mod.f90:59-93 (hydroLinesFiles.dat, gaussfitHb.dat,
//                      r1bEdge.dat, r2bEdge.dat, r2aEdge.dat)
//   readHeIRecLines    source/hydro_mod.f90:184-200 (HeIrecLines.dat)
//   HeI2photSub        source/emission_mod.f90:742-760 (HeI2phot.dat)
//   setDiffusePDF      source/emission_mod.f90:1644-1660 (r2a0100old.dat)
//   RecLinesEmission   source/emission_mod.f90:895-917 (the hydrogenic line files)
//   fb_ff              source/emission_mod.f90:550-614 (the heavy-ion free-bound terms)
// The reads follow Fortran list-directed semantics: each READ starts a new
// record, takes as many values as it needs across records, and drops the rest
// of its last record.
#include "setup_internal.h"
#include "list_reader.h"

#include <cmath>
#include <cstdlib>
#include <fstream>
#include <map>
#include <stdexcept>

namespace mcx {

namespace {

[[noreturn]] void efail(const std::string& msg) { throw std::runtime_error(msg); }

std::string baseName(const std::string& f) {
  size_t s = f.find_last_of('/');
  return s == std::string::npos ? f : f.substr(s + 1);
}

}  // namespace

void buildEmissionTables(Setup& s) {
  EmissionTables& em = s.em;
  const std::string& D = s.dataDir;
  const float* nu = s.nu.data();
  const int nb = s.nbins;

  // initGammaCont
  {
    const char* names[3] = {"gammaHI.dat", "gammaHeI.dat", "gammaHeII.dat"};
    std::vector<ListReader> r;
    for (auto n : names) r.emplace_back(D + "/" + n);
    int nt = 0;
    for (int k = 0; k < 3; ++k) {
      auto h = r[k].need(2);
      if (k > 0 && (int)h[0] != nt) efail("initGammaCont: the number of temperature points must be the same for all gammas");
      nt = (int)h[0];
      em.nlim[k] = (int)h[1];
      if (em.nlim[k] > 32) efail("initGammaCont: more than 32 edge points");
    }
    em.nTk = nt;
    for (int k = 0; k < 3; ++k) {
      auto t = r[k].need(nt);
      em.tk.assign(t.begin(), t.end());
    }
    em.edgeP.assign(3 * 32, 0);
    em.logGamma.assign((size_t)3 * nt * 32, 0.f);
    for (int k = 0; k < 3; ++k) {
      for (int i = 1; i <= em.nlim[k]; ++i) {
        auto row = r[k].need(1 + nt);
        float nuG = (float)row[0];
        int P = locate(nu, nb, nuG);
        if (P < nb && nuG > (nu[P - 1] + nu[P]) / 2.f) P = P + 1;
        em.edgeP[k * 32 + (i - 1)] = P;
        for (int itk = 1; itk <= nt; ++itk) {
          float v = (float)row[itk];
          em.logGamma[((size_t)k * nt + (itk - 1)) * 32 + (i - 1)] = v > 0.f ? log10f(v) : 0.f;
        }
      }
      em.edgeP[k * 32 + 0] = 1;
    }
  }

  // heavy-element free-bound terms: elements 3..19, ions 1..nstages-1 (fb_ff)
  em.fbHeavy.clear();
  for (int elem = 3; elem <= 19; ++elem) {
    if (!s.elemOn[elem - 1]) continue;
    for (int ion = 1; ion <= s.p.nstages - 1; ++ion) {
      if (ion > elem) break;
      int nElec = elem - ion + 1, outShell, g0, g1;
      getOuterShell(elem, nElec, outShell, g0, g1);
      const int* P = s.elementP[elem - 1][ion - 1][outShell - 1];
      if (P[1] > nb) efail("fb_ff: high frequency limit beyond grid limit. Increase frequency grid, or switch element off");
      if (P[0] > nb) efail("fb_ff: IP frequency beyond grid limit. Increase frequency grid, or switch element off");
      int rec[7] = {elem, ion, P[0], P[1], P[2], g0, g1};
      em.fbHeavy.insert(em.fbHeavy.end(), rec, rec + 7);
    }
  }

  // hydrogenic recombination-line tables
  {
    ListReader lf(D + "/hydroLinesFiles.dat");
    std::map<std::string, int> idx;
    std::vector<std::string> files;
    em.hydroFileMap.assign(9 * 12, 0);
    for (int i = 1; i <= 9; ++i)
      for (int j = 1; j <= 12; ++j) {
        std::string f = baseName(lf.readString());
        auto it = idx.find(f);
        if (it == idx.end()) { idx[f] = (int)files.size(); files.push_back(f); }
        em.hydroFileMap[(i - 1) * 12 + (j - 1)] = idx[f];
      }
    em.nHydroFiles = (int)files.size();
    em.hydroNDens.assign(files.size(), 0);
    em.hydroDens.assign(files.size() * 13, 0.f);
    em.hydroLines.assign(files.size() * 13 * 14 * 8, 0.f);
    for (size_t f = 0; f < files.size(); ++f) {
      ListReader r(D + "/" + files[f]);
      std::vector<double> v;
      int iden;
      for (iden = 1; iden <= 100; ++iden) {
        if (!r.read(1, v)) break;
        if (iden > 13) efail("RecLinesEmission: more than 13 densities in " + files[f]);
        em.hydroDens[f * 13 + (iden - 1)] = (float)v[0];
        for (int iup = 15; iup >= 2; --iup) {
          int n = std::min(8, iup - 1);
          auto row = r.need(n);
          for (int ilow = 1; ilow <= n; ++ilow)
            em.hydroLines[((f * 13 + (iden - 1)) * 14 + (iup - 2)) * 8 + (ilow - 1)] = (float)row[ilow - 1];
        }
      }
      em.hydroNDens[f] = iden - 1;
    }
  }
  {
    ListReader r(D + "/gaussfitHb.dat");
    for (int i = 0; i < 9; ++i) {
      auto v = r.need(8);
      for (int j = 0; j < 4; ++j) { em.HbCoeff[0][i][j] = (float)v[j]; em.HbCoeff[1][i][j] = (float)v[4 + j]; }
    }
    const char* eb[2] = {"r1bEdge.dat", "r2bEdge.dat"};
    for (int k = 0; k < 2; ++k) {
      ListReader re(D + "/" + eb[k]);
      for (int i = 0; i < 26; ++i) {
        auto v = re.need(3);
        for (int j = 0; j < 3; ++j) em.rbEdge[k][j][i] = (float)v[j];
      }
    }
    ListReader ra(D + "/r2aEdge.dat");
    for (int i = 0; i < 18; ++i) {
      auto v = ra.need(3);
      for (int j = 0; j < 3; ++j) em.r2aEdge[j][i] = (float)v[j];
    }
    const float temps[12] = {0.05f, 0.10f, 0.30f, 0.50f, 0.75f, 1.0f, 1.25f, 1.50f, 2.0f, 3.0f, 5.0f, 10.0f};
    for (int i = 0; i < 12; ++i) em.hydroLinesTemps[i] = temps[i];
  }
  {
    ListReader r(D + "/HeIrecLines.dat");
    for (int iden = 0; iden < 3; ++iden)
      for (int il = 0; il < 34; ++il) {
        auto v = r.need(4);
        for (int j = 0; j < 4; ++j) em.HeIrec[il][iden][j] = (float)v[j];
        em.HeIrec[il][iden][0] = em.HeIrec[il][iden][0] * 1.e25f;
      }
  }
  {
    ListReader r(D + "/HeI2phot.dat");
    for (int i = 0; i < 41; ++i) {
      auto v = r.need(2);
      em.HeI2phot[0][i] = (float)v[0];
      em.HeI2phot[1][i] = (float)v[1];
    }
  }
  {
    ListReader r(D + "/r2a0100old.dat");
    for (int i = 0; i < 4; ++i) {
      auto v = r.need(2);
      em.HeIILyman[0][i] = (float)v[0];
      em.HeIILyman[1][i] = (float)v[1];
      em.HeIILymanP[i] = locate(nu, nb, em.HeIILyman[1][i]);
    }
  }
  em.j2TsP = locate(nu, nb, 1.45673f);
}

}  // namespace mcx
