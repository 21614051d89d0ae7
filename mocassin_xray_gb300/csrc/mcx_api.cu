// mcx_api.cu - the C ABI of libmcx.so (declared in include/mcx.h): set-up
// objects, device contexts, array exchange in the reference's Fortran layout
// and the phase entry points (opacity, transport, J normalisation).
#include "../../include/mcx.h"
#include "k_emission.cuh"
#include "k_balance.cuh"
#include "k_lines.cuh"
#include "k_dust.cuh"
#include "k_opacity.cuh"
#include "k_transport_launch.h"
#include "mcx_device.cuh"
#include "setup_internal.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

using namespace mcx;

// ------------------------------------------------------------------ set-up
struct mcx_setup {
  Setup s;
};

namespace {
thread_local std::string g_setupError;

int copyRaw(const void* src, size_t size, void* dst, size_t nbytes) {
  if (nbytes != size) {
    g_setupError = "mcx_setup_get: size mismatch (expected " + std::to_string(size) + " bytes)";
    return MCX_ERR_INPUT;
  }
  std::memcpy(dst, src, nbytes);
  return MCX_OK;
}
template <typename T>
int copyOut(const std::vector<T>& v, void* dst, size_t nbytes) {
  if (nbytes != v.size() * sizeof(T)) {
    g_setupError = "mcx_setup_get: size mismatch (expected " + std::to_string(v.size() * sizeof(T)) + " bytes)";
    return MCX_ERR_INPUT;
  }
  if (nbytes) std::memcpy(dst, v.data(), nbytes);
  return MCX_OK;
}
template <typename T>
int copyIn(std::vector<T>& v, const void* src, size_t nbytes) {
  if (nbytes != v.size() * sizeof(T)) {
    g_setupError = "mcx_setup_set: size mismatch (expected " + std::to_string(v.size() * sizeof(T)) + " bytes)";
    return MCX_ERR_INPUT;
  }
  if (nbytes) std::memcpy(v.data(), src, nbytes);
  return MCX_OK;
}

// Cell volume in FP64 with the operation order of getVolume
// (source/grid_mod.f90:2887-2986) evaluated in double.
double volumeD(const Setup& s, int xP, int yP, int zP) {
  auto A = [](const std::vector<float>& a, int i) { return (double)a[i - 1]; };
  // half-width first cells with symmetric axes, first and last ones with a plane source
  const bool lo = s.p.lgSymmetricXYZ || s.p.lgPlaneIonization, hi = s.p.lgPlaneIonization;
  auto edge = [](double w, bool half) { return half ? w / 2. : w; };
  double dx = 0., dy = 0., dz = 0.;
  if (xP > 1 && xP < s.nx) dx = std::fabs(A(s.xAxis, xP + 1) - A(s.xAxis, xP - 1)) / 2.;
  else if (xP == 1) dx = edge(std::fabs(A(s.xAxis, 2) - A(s.xAxis, 1)), lo);
  else if (xP == s.nx) dx = edge(std::fabs(A(s.xAxis, xP) - A(s.xAxis, xP - 1)), hi);
  if (yP > 1 && yP < s.ny) dy = std::fabs(A(s.yAxis, yP + 1) - A(s.yAxis, yP - 1)) / 2.;
  else if (yP == 1) dy = edge(std::fabs(A(s.yAxis, 2) - A(s.yAxis, 1)), lo);
  else if (yP == s.ny) dy = edge(std::fabs(A(s.yAxis, yP) - A(s.yAxis, yP - 1)), hi);
  if (zP > 1 && zP < s.nz) dz = std::fabs(A(s.zAxis, zP + 1) - A(s.zAxis, zP - 1)) / 2.;
  else if (zP == 1) dz = edge(std::fabs(A(s.zAxis, 2) - A(s.zAxis, 1)), lo);
  else if (zP == s.nz) dz = edge(std::fabs(A(s.zAxis, zP) - A(s.zAxis, zP - 1)), hi);
  dx = dx / 1.e15; dy = dy / 1.e15; dz = dz / 1.e15;
  return dx * dy * dz;
}
}  // namespace

extern "C" int mcx_setup_from_input(const char* input_file, const char* data_dir, const mcx_setup_opts* opts,
                                    mcx_setup** out) {
  if (!input_file || !data_dir || !out) { g_setupError = "mcx_setup_from_input: null argument"; return MCX_ERR_INPUT; }
  *out = nullptr;
  auto* m = new (std::nothrow) mcx_setup();
  if (!m) { g_setupError = "mcx_setup_from_input: out of memory"; return MCX_ERR_NOMEM; }
  try {
    buildSetup(m->s, input_file, data_dir, opts ? opts->mesh_mode : 0);
  } catch (const std::exception& e) {
    g_setupError = e.what();
    delete m;
    std::string w = g_setupError;
    return (w.find("can't open") != std::string::npos || w.find("truncated") != std::string::npos) ? MCX_ERR_IO
                                                                                                 : MCX_ERR_INPUT;
  }
  *out = m;
  return MCX_OK;
}

extern "C" void mcx_setup_free(mcx_setup* s) { delete s; }

extern "C" const char* mcx_setup_last_error(void) { return g_setupError.c_str(); }

extern "C" int mcx_setup_info_get(const mcx_setup* m, mcx_setup_info* info) {
  if (!m || !info) { g_setupError = "mcx_setup_info_get: null argument"; return MCX_ERR_INPUT; }
  const Setup& s = m->s;
  std::memset(info, 0, sizeof(*info));
  info->nx = s.nx; info->ny = s.ny; info->nz = s.nz;
  info->n_angle_bins = s.p.nAngleBins;
  info->plane_ionization = s.p.lgPlaneIonization ? 1 : 0;
  info->n_stars = (int32_t)std::max<size_t>(s.stars.size(), 1);
  for (int j = 0; j < 2; ++j) { info->view_theta[j] = s.p.viewTheta[j]; info->view_phi[j] = s.p.viewPhi[j]; }
  info->n_cells = s.nCells;
  info->nbins = s.nbins;
  info->n_xsec = (int32_t)s.xSec.size();
  info->n_elem_used = s.nElemUsed;
  info->nstages = s.p.nstages;
  info->symmetric_xyz = s.p.lgSymmetricXYZ;
  info->lg_gas = s.p.lgGas; info->lg_dust = s.p.lgDust; info->lg_compton = s.p.lgCompton;
  for (int d = 0; d < 3; ++d) { info->star_idx[d] = s.starIdx[d]; info->star_pos[d] = s.starPos[d]; }
  info->lyman_p = s.lymanP;
  info->n_photons = s.p.nPhotons / std::max<int64_t>((int64_t)s.stars.size(), 1);
  info->max_iterate_mc = s.p.maxIterateMC;
  info->r_out = s.p.R_out; info->r_in = s.p.R_in;
  info->l_star = s.LStar; info->l_phot = s.LPhot;
  info->ion_edge1 = s.ionEdge.empty() ? 0.f : s.ionEdge[0];
  info->te_start = s.p.TeStart;
  info->min_convergence = s.p.minConvergence;
  info->xhi_limit = s.p.XHILimit;
  return MCX_OK;
}


static std::vector<int32_t> packedPointers(const Setup& s) {
  std::vector<int32_t> p(32, 0);
  p[0] = s.HlevXSecP[0]; p[1] = s.HlevNuP[0]; p[2] = s.HeISingXSecP[0]; p[3] = s.HeIlevNuP[0];
  p[4] = s.HeIIXSecP[0]; p[5] = s.HeIIlevNuP[0]; p[6] = s.bremsXSecP; p[7] = s.lymanP;
  p[8] = s.KshellLimitP; p[9] = s.secIonP; p[10] = s.cRecoilHP; p[11] = s.cRecoilHeP;
  p[12] = s.xrayP; p[13] = s.BjumpP;
  return p;
}

// The sources as MCX_SARR_STARS lays them out; source 1 from the single-source fields (which
// mcx_setup_set may have changed)
static std::vector<float> starTable(const Setup& s) {
  const size_t n = std::max<size_t>(s.stars.size(), 1);
  std::vector<float> t(8 * n, 0.f);
  for (size_t i = 0; i < n; ++i) {
    float* r = t.data() + 8 * i;
    const bool one = i == 0 || s.stars.size() <= i;
    r[0] = one ? s.LStar : s.stars[i].LStar;
    r[1] = one ? s.p.TStellar : s.stars[i].TStellar;
    for (int d = 0; d < 3; ++d) {
      r[2 + d] = one ? s.starPos[d] : s.stars[i].pos[d];
      r[5 + d] = (float)(one ? s.starIdx[d] : s.stars[i].idx[d]);
    }
  }
  return t;
}

// Every source's CDF, [nStars][nbins]; source 1's from srcCDF
static std::vector<float> sourceCDFs(const Setup& s) {
  std::vector<float> c(s.srcCDF);
  for (size_t i = 1; i < s.stars.size(); ++i) c.insert(c.end(), s.stars[i].cdf.begin(), s.stars[i].cdf.end());
  return c;
}

extern "C" int mcx_setup_get(const mcx_setup* m, int32_t id, void* dst, size_t nbytes) {
  if (!m || (!dst && nbytes)) { g_setupError = "mcx_setup_get: null argument"; return MCX_ERR_INPUT; }
  const Setup& s = m->s;
  switch (id) {
    case MCX_ARR_NU: return copyOut(s.nu, dst, nbytes);
    case MCX_ARR_WIDFLX: return copyOut(s.widFlx, dst, nbytes);
    case MCX_ARR_XSEC: return copyOut(s.xSec, dst, nbytes);
    case MCX_ARR_SRC_CDF: return copyOut(s.srcCDF, dst, nbytes);
    case MCX_ARR_KN_SIGMA_T: return copyOut(s.KNsigmaT, dst, nbytes);
    case MCX_ARR_KN_CDF: return copyOut(s.KNcdf, dst, nbytes);
    case MCX_ARR_PCOMP: return copyOut(s.Pcomp, dst, nbytes);
    case MCX_ARR_XAXIS: return copyOut(s.xAxis, dst, nbytes);
    case MCX_ARR_YAXIS: return copyOut(s.yAxis, dst, nbytes);
    case MCX_ARR_ZAXIS: return copyOut(s.zAxis, dst, nbytes);
    case MCX_ARR_ACTIVE: return copyOut(s.active, dst, nbytes);
    case MCX_ARR_HDEN: return copyOut(s.Hden, dst, nbytes);
    case MCX_ARR_TE: return copyOut(s.Te, dst, nbytes);
    case MCX_ARR_NE: return copyOut(s.Ne, dst, nbytes);
    case MCX_ARR_TEOLD: return copyOut(s.TeOld, dst, nbytes);
    case MCX_ARR_NEOLD: return copyOut(s.NeOld, dst, nbytes);
    case MCX_ARR_IONDEN: return copyOut(s.ionDen, dst, nbytes);
    case MCX_ARR_VOLUME: return copyOut(s.volume, dst, nbytes);
    case MCX_ARR_NDUST: return copyOut(s.Ndust, dst, nbytes);
    case MCX_ARR_ELEM_ABUN: {
      std::vector<float> v(s.elemAbun, s.elemAbun + kNElements);
      return copyOut(v, dst, nbytes);
    }
    case MCX_SARR_POINTERS: return copyOut(packedPointers(s), dst, nbytes);
    case MCX_SARR_ELEMENT_P: {
      std::vector<int32_t> v(&s.elementP[0][0][0][0], &s.elementP[0][0][0][0] + 30 * 30 * 7 * 3);
      return copyOut(v, dst, nbytes);
    }
    case MCX_SARR_N_SHELLS: {
      std::vector<int32_t> v(&s.nShells[0][0], &s.nShells[0][0] + 30 * 30);
      return copyOut(v, dst, nbytes);
    }
    case MCX_SARR_ELEM_XREF: {
      std::vector<int32_t> v(s.elemXref, s.elemXref + kNElements);
      return copyOut(v, dst, nbytes);
    }
    case MCX_SARR_ION_EDGE: return copyOut(s.ionEdge, dst, nbytes);
    case MCX_SARR_COMXSEC_H: return copyOut(s.comXSecH, dst, nbytes);
    case MCX_SARR_COMXSEC_C: return copyOut(s.comXSecC, dst, nbytes);
    case MCX_SARR_XSEC_RECOIL: return copyOut(s.xSecRecoil, dst, nbytes);
    case MCX_SARR_EM_DIMS: {
      const EmissionTables& em = s.em;
      std::vector<int32_t> v(16, 0);
      v[0] = em.nTk; v[1] = em.nlim[0]; v[2] = em.nlim[1]; v[3] = em.nlim[2];
      v[4] = (int32_t)(em.fbHeavy.size() / 7); v[5] = em.nHydroFiles; v[6] = em.j2TsP;
      for (int k = 0; k < 4; ++k) v[7 + k] = em.HeIILymanP[k];
      return copyOut(v, dst, nbytes);
    }
    case MCX_SARR_EM_TK: return copyOut(s.em.tk, dst, nbytes);
    case MCX_SARR_EM_EDGE_P: return copyOut(s.em.edgeP, dst, nbytes);
    case MCX_SARR_EM_LOG_GAMMA: return copyOut(s.em.logGamma, dst, nbytes);
    case MCX_SARR_EM_FB_HEAVY: return copyOut(s.em.fbHeavy, dst, nbytes);
    case MCX_SARR_EM_HYDRO_MAP: return copyOut(s.em.hydroFileMap, dst, nbytes);
    case MCX_SARR_EM_HYDRO_DENS: return copyOut(s.em.hydroDens, dst, nbytes);
    case MCX_SARR_EM_HYDRO_LINES: return copyOut(s.em.hydroLines, dst, nbytes);
    case MCX_SARR_EM_HYDRO_TEMPS: return copyOut(std::vector<float>(s.em.hydroLinesTemps, s.em.hydroLinesTemps + 12), dst, nbytes);
    case MCX_SARR_EM_HB_COEFF: return copyOut(std::vector<float>(&s.em.HbCoeff[0][0][0], &s.em.HbCoeff[0][0][0] + 72), dst, nbytes);
    case MCX_SARR_EM_RB_EDGE: return copyOut(std::vector<float>(&s.em.rbEdge[0][0][0], &s.em.rbEdge[0][0][0] + 156), dst, nbytes);
    case MCX_SARR_EM_R2A_EDGE: return copyOut(std::vector<float>(&s.em.r2aEdge[0][0], &s.em.r2aEdge[0][0] + 54), dst, nbytes);
    case MCX_SARR_EM_HEI_REC: return copyOut(std::vector<float>(&s.em.HeIrec[0][0][0], &s.em.HeIrec[0][0][0] + 408), dst, nbytes);
    case MCX_SARR_EM_HEI_2PHOT: return copyOut(std::vector<float>(&s.em.HeI2phot[0][0], &s.em.HeI2phot[0][0] + 82), dst, nbytes);
    case MCX_SARR_EM_HEII_LYMAN: return copyOut(std::vector<float>(&s.em.HeIILyman[0][0], &s.em.HeIILyman[0][0] + 8), dst, nbytes);
    case MCX_SARR_CION_CF: return copyRaw(&s.bal.CF[0][0][0], sizeof(s.bal.CF), dst, nbytes);
    case MCX_SARR_CION_THERM: return copyRaw(&s.bal.cionTherm[0][0], sizeof(s.bal.cionTherm), dst, nbytes);
    case MCX_SARR_NAUGER: return copyRaw(&s.bal.nauger[0][0][0], sizeof(s.bal.nauger), dst, nbytes);
    case MCX_SARR_AUGER: return copyRaw(&s.bal.auger[0][0][0][0], sizeof(s.bal.auger), dst, nbytes);
    case MCX_SARR_RR_BADNELL: return copyRaw(&s.bal.RRb[0][0][0], sizeof(s.bal.RRb), dst, nbytes);
    case MCX_SARR_DR_BADNELL_C: return copyRaw(&s.bal.DRbC[0][0][0], sizeof(s.bal.DRbC), dst, nbytes);
    case MCX_SARR_DR_BADNELL_E: return copyRaw(&s.bal.DRbE[0][0][0], sizeof(s.bal.DRbE), dst, nbytes);
    case MCX_SARR_RADREC_RREC: return copyRaw(&s.bal.rrec[0][0][0], sizeof(s.bal.rrec), dst, nbytes);
    case MCX_SARR_RADREC_RNEW: return copyRaw(&s.bal.rnew[0][0][0], sizeof(s.bal.rnew), dst, nbytes);
    case MCX_SARR_DIELEC: return copyOut(s.bal.diel, dst, nbytes);
    case MCX_SARR_ALDRO: return copyOut(s.bal.aldro, dst, nbytes);
    case MCX_SARR_OUTER_SHELL: return copyRaw(&s.bal.outer[0][0][0], sizeof(s.bal.outer), dst, nbytes);
    case MCX_SARR_ATOM_INDEX: return copyRaw(&s.bal.atomIndex[0][0], sizeof(s.bal.atomIndex), dst, nbytes);
    case MCX_SARR_ATOM_HDR: return copyOut(s.bal.atomHdr, dst, nbytes);
    case MCX_SARR_ATOM_DATA: return copyOut(s.bal.atomData, dst, nbytes);
    case MCX_SARR_DUST_DIMS: return copyOut(std::vector<int32_t>{s.dust.nSpecies, s.dust.nSizes, kNTemps, 0}, dst, nbytes);
    case MCX_SARR_DUST_CABS: return copyOut(s.dust.Cabs, dst, nbytes);
    case MCX_SARR_DUST_CSCA: return copyOut(s.dust.Csca, dst, nbytes);
    case MCX_SARR_DUST_CTABS: return copyOut(s.dust.CTabs, dst, nbytes);
    case MCX_SARR_DUST_CTSCA: return copyOut(s.dust.CTsca, dst, nbytes);
    case MCX_SARR_DUST_ABUN: return copyOut(s.dust.grainAbun, dst, nbytes);
    case MCX_SARR_DUST_TSUB: return copyOut(s.dust.TdustSublime, dst, nbytes);
    case MCX_SARR_DUST_RADIUS: return copyOut(s.dust.grainRadius, dst, nbytes);
    case MCX_SARR_DUST_WEIGHT: return copyOut(s.dust.grainWeight, dst, nbytes);
    case MCX_SARR_DUST_EMINT: return copyOut(s.dust.emIntegral, dst, nbytes);
    case MCX_ARR_TDUST: return copyOut(s.Tdust, dst, nbytes);
    case MCX_SARR_STARS: return copyOut(starTable(s), dst, nbytes);
    case MCX_SARR_SRC_CDFS: return copyOut(sourceCDFs(s), dst, nbytes);
    default: g_setupError = "mcx_setup_get: unknown array id " + std::to_string(id); return MCX_ERR_INPUT;
  }
}

extern "C" int mcx_setup_len(const mcx_setup* m, int32_t id, int64_t* count) {
  if (!m || !count) { g_setupError = "mcx_setup_len: null argument"; return MCX_ERR_INPUT; }
  const Setup& s = m->s;
  const int64_t C1 = (int64_t)s.nCells + 1, nb = s.nbins;
  switch (id) {
    case MCX_ARR_NU: case MCX_ARR_WIDFLX: case MCX_ARR_SRC_CDF: case MCX_ARR_KN_SIGMA_T:
    case MCX_SARR_COMXSEC_H: case MCX_SARR_COMXSEC_C: case MCX_SARR_XSEC_RECOIL: *count = nb; break;
    case MCX_ARR_XSEC: *count = (int64_t)s.xSec.size(); break;
    case MCX_ARR_KN_CDF: case MCX_ARR_PCOMP: *count = 180 * nb; break;
    case MCX_ARR_XAXIS: *count = s.nx; break;
    case MCX_ARR_YAXIS: *count = s.ny; break;
    case MCX_ARR_ZAXIS: *count = s.nz; break;
    case MCX_ARR_ACTIVE: *count = (int64_t)s.active.size(); break;
    case MCX_ARR_HDEN: case MCX_ARR_TE: case MCX_ARR_NE: case MCX_ARR_TEOLD: case MCX_ARR_NEOLD:
    case MCX_ARR_VOLUME: case MCX_ARR_NDUST: *count = C1; break;
    case MCX_ARR_IONDEN: *count = (int64_t)s.ionDen.size(); break;
    case MCX_ARR_ELEM_ABUN: case MCX_SARR_ELEM_XREF: *count = 30; break;
    case MCX_SARR_POINTERS: *count = 32; break;
    case MCX_SARR_ELEMENT_P: *count = 30 * 30 * 7 * 3; break;
    case MCX_SARR_N_SHELLS: *count = 30 * 30; break;
    case MCX_SARR_ION_EDGE: *count = (int64_t)s.ionEdge.size(); break;
    case MCX_SARR_EM_DIMS: *count = 16; break;
    case MCX_SARR_EM_TK: *count = (int64_t)s.em.tk.size(); break;
    case MCX_SARR_EM_EDGE_P: *count = (int64_t)s.em.edgeP.size(); break;
    case MCX_SARR_EM_LOG_GAMMA: *count = (int64_t)s.em.logGamma.size(); break;
    case MCX_SARR_EM_FB_HEAVY: *count = (int64_t)s.em.fbHeavy.size(); break;
    case MCX_SARR_EM_HYDRO_MAP: *count = (int64_t)s.em.hydroFileMap.size(); break;
    case MCX_SARR_EM_HYDRO_DENS: *count = (int64_t)s.em.hydroDens.size(); break;
    case MCX_SARR_EM_HYDRO_LINES: *count = (int64_t)s.em.hydroLines.size(); break;
    case MCX_SARR_EM_HYDRO_TEMPS: *count = 12; break;
    case MCX_SARR_EM_HB_COEFF: *count = 72; break;
    case MCX_SARR_EM_RB_EDGE: *count = 156; break;
    case MCX_SARR_EM_R2A_EDGE: *count = 54; break;
    case MCX_SARR_EM_HEI_REC: *count = 408; break;
    case MCX_SARR_EM_HEI_2PHOT: *count = 82; break;
    case MCX_SARR_EM_HEII_LYMAN: *count = 8; break;
    case MCX_SARR_CION_CF: *count = 30 * 30 * 5; break;
    case MCX_SARR_CION_THERM: *count = 30 * 30; break;
    case MCX_SARR_NAUGER: *count = 30 * 30 * 10; break;
    case MCX_SARR_AUGER: *count = 30 * 30 * 10 * 10; break;
    case MCX_SARR_RR_BADNELL: *count = 6 * 30 * 31; break;
    case MCX_SARR_DR_BADNELL_C: case MCX_SARR_DR_BADNELL_E: *count = 30 * 31 * 9; break;
    case MCX_SARR_RADREC_RREC: *count = 30 * 30 * 2; break;
    case MCX_SARR_RADREC_RNEW: *count = 30 * 30 * 4; break;
    case MCX_SARR_DIELEC: *count = (int64_t)s.bal.diel.size(); break;
    case MCX_SARR_ALDRO: *count = (int64_t)s.bal.aldro.size(); break;
    case MCX_SARR_OUTER_SHELL: *count = 30 * 30 * 3; break;
    case MCX_SARR_ATOM_INDEX: *count = 30 * 31; break;
    case MCX_SARR_ATOM_HDR: *count = (int64_t)s.bal.atomHdr.size(); break;
    case MCX_SARR_ATOM_DATA: *count = (int64_t)s.bal.atomData.size(); break;
    case MCX_SARR_DUST_DIMS: *count = 4; break;
    case MCX_SARR_DUST_CABS: case MCX_SARR_DUST_CSCA: *count = (int64_t)s.dust.Cabs.size(); break;
    case MCX_SARR_DUST_CTABS: case MCX_SARR_DUST_CTSCA: *count = (int64_t)s.dust.CTabs.size(); break;
    case MCX_SARR_DUST_ABUN: case MCX_SARR_DUST_TSUB: *count = s.dust.nSpecies; break;
    case MCX_SARR_DUST_RADIUS: case MCX_SARR_DUST_WEIGHT: *count = s.dust.nSizes; break;
    case MCX_SARR_DUST_EMINT: *count = (int64_t)s.dust.emIntegral.size(); break;
    case MCX_ARR_TDUST: *count = (int64_t)s.Tdust.size(); break;
    case MCX_SARR_STARS: *count = 8 * (int64_t)std::max<size_t>(s.stars.size(), 1); break;
    case MCX_SARR_SRC_CDFS: *count = nb * (int64_t)std::max<size_t>(s.stars.size(), 1); break;

    default: g_setupError = "mcx_setup_len: unknown array id " + std::to_string(id); return MCX_ERR_INPUT;
  }
  return MCX_OK;
}

extern "C" int mcx_setup_set(mcx_setup* m, int32_t id, const void* src, size_t nbytes) {
  if (!m || (!src && nbytes)) { g_setupError = "mcx_setup_set: null argument"; return MCX_ERR_INPUT; }
  Setup& s = m->s;
  switch (id) {
    case MCX_ARR_HDEN: return copyIn(s.Hden, src, nbytes);
    case MCX_ARR_TE: return copyIn(s.Te, src, nbytes);
    case MCX_ARR_NE: return copyIn(s.Ne, src, nbytes);
    case MCX_ARR_TEOLD: return copyIn(s.TeOld, src, nbytes);
    case MCX_ARR_NEOLD: return copyIn(s.NeOld, src, nbytes);
    case MCX_ARR_IONDEN: return copyIn(s.ionDen, src, nbytes);
    case MCX_ARR_SRC_CDF: return copyIn(s.srcCDF, src, nbytes);
    default: g_setupError = "mcx_setup_set: array id " + std::to_string(id) + " is not settable"; return MCX_ERR_INPUT;
  }
}

// ------------------------------------------------------------------ context
namespace {

// Trapped-packet hand-off: a history is parked for the trapped-packet kernel
// when it is about to be re-emitted for the kHandoffAt-th time (bulk histories
// end after a handful of emissions; a trapped one runs on to recursionLimit),
// in a buffer with room for kParkedCap histories (beyond it they stay in place).
constexpr int kHandoffAt = 256;
constexpr unsigned long long kParkedCap = 1ull << 16;

template <typename T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  DBuf() = default;
  // owns its allocation: moved, never copied (a copy would free it twice)
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  DBuf(DBuf&& o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
  DBuf& operator=(DBuf&& o) noexcept {
    if (this != &o) {
      if (p) cudaFree(p);
      p = o.p; n = o.n;
      o.p = nullptr; o.n = 0;
    }
    return *this;
  }
  ~DBuf() { if (p) cudaFree(p); }
  cudaError_t alloc(size_t count) {
    if (p) { cudaFree(p); p = nullptr; n = 0; }
    if (count == 0) return cudaSuccess;
    cudaError_t e = cudaMalloc((void**)&p, count * sizeof(T));
    if (e == cudaSuccess) n = count;
    return e;
  }
  size_t bytes() const { return n * sizeof(T); }
};

}  // namespace

struct mcx_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr, tev0 = nullptr, tev1 = nullptr;
  std::string err;
  bool loaded = false;
  int numSMs = 0;

  // model sizes and flags
  int nx = 0, ny = 0, nz = 0, nCells = 0, nbins = 0, nstages = 0, nElemUsed = 0, nXsec = 0;
  bool symmetric = false, lgDust = false, lgGas = false, lgCompton = false, radPress = false;
  float lStar = 0.f, ionEdge1 = 0.f, rOut = 0.f;
  int64_t nPhotons = 0;
  int starIdx[3] = {0, 0, 0};
  float starPos[3] = {0.f, 0.f, 0.f};
  int nStars = 1;                  // ionising sources; srcCDF holds their CDFs, [nStars][nbins]
  std::vector<float> stars;        // [nStars][8] as MCX_SARR_STARS
  std::vector<int32_t> activeHost;
  int activeFull = 0;        // active(i,j,k) == (i-1) ny nz + (j-1) nz + k for every cell
  int plane = 0;             // plane-parallel ionisation (lgPlaneIonization)
  float gauntTeOld = -1.f;   // BoltGaunt's saved TeOld2

  // tables
  DBuf<float> nu, log10nu, xsec, KNsigmaT, KNcdfT, PcompT, srcCDF, xAxis, yAxis, zAxis, volF;
  DBuf<double> volD;
  DBuf<int32_t> active;
  DBuf<int32_t> csrStart, slotPlane;
  DBuf<int2> csrTerm;
  DBuf<float> slotAbun, slotFFWeight;
  int nSlots = 0, bremsP0 = 0;
  // state
  DBuf<float> hden, te, ne, teOld, neOld, ionDen, ndust;
  // phase arrays
  DBuf<float> opacity, recPDF, recCDFT, totalLines, scaOpac, dustPDF, dustCDFT;
  DBuf<double> jste, jlo, escaped, hEst;   // jlo: the compensation of jste during a transport call
  // viewing angles (source/grid_mod.f90:570-601): escapedPackets' planes 1..nAngle
  int nAngle = 0, totPhi = 20;
  int8_t viewPTheta[21] = {}, viewPPhi[21] = {};
  // scratch
  DBuf<float> gauntTe;
  DBuf<uint8_t> computeMask;
  DBuf<DevTransportCounters> counters;
  // histories parked by the transport kernel for the trapped-packet kernel
  // (kParkedCap packets of the FP64 kernel, the larger of the two)
  DBuf<unsigned char> parked;
  std::unique_ptr<EmissionData> emission;
  std::unique_ptr<BalanceData> balance;
  std::unique_ptr<DustData> dust;
  DBuf<float> tdust;                 // [nSpecies+1][nSizes+1][nCells+1]
  DBuf<int32_t> lgConverged, lgBlack, nIterT;
  DBuf<float> forLines;
  // outputGas: per multi-level atom the line factors a(j,i) E_ji (two-photon
  // part removed) and wavelengths at [i-1][j-1], i lower, j upper level
  struct LineAtom {
    int elem = 0, ion = 0, nLev = 0;
    std::vector<double> fac, wav;
  };
  std::vector<LineAtom> lineAtoms;
  int xrefAll[30] = {};
  DBuf<double> linePartial, lineSums;
  DBuf<int32_t> lineForbBase;
  // batch of nebulae (mcx_load_batched); nNeb = 0 for a single grid
  int nNeb = 0;
  std::vector<int32_t> nebCellOff;                 // [nNeb+1]
  std::vector<NebulaDesc> nebDesc;                 // geometry; packet constants set per transport
  std::vector<float> nebLStar;
  std::vector<int32_t> nebSym, nebNx, nebNy, nebNz;
  std::vector<std::vector<int32_t>> nebActive;     // [nz][ny][nx] per nebula, batch-wide ids
  std::vector<float> nebGauntTeOld;                // each nebula's Gaunt cache temperature
  std::vector<float> nebGauntTemps;                // host staging of the Gaunt temperatures for the upload
  DBuf<float> nebGauntTeDev;
  DBuf<NebulaDesc> nebDescDev;
  DBuf<unsigned long long> nebPktBegin;
  DBuf<unsigned long long> nebStamps;             // [0] launch start, [1 + b] nebula b's last packet (global timer, ns)
  DBuf<float> nebAxes, nebCdf, nebFfK, jDiv;
  DBuf<int32_t> nebActiveDev;
  DBuf<int16_t> nebFfIdx;
  // mcx_state_save snapshots: everything an iteration carries into the next
  struct Snapshot {
    std::vector<DBuf<float>> f;       // the float arrays of snapshotArrays(), in order
    DBuf<int32_t> converged;
    float gauntTeOld = -1.f;
    std::vector<float> nebGauntTeOld;
    bool haveOpacity = false, haveRecPDF = false, haveDustPDF = false;
    bool valid = false;
  };
  std::vector<Snapshot> snaps;        // slot k at snaps[k]
  bool haveOpacity = false, haveRecPDF = false, haveDustPDF = false;
};

namespace {

int fail(mcx_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

int cudaFail(mcx_ctx* c, cudaError_t e, const char* what) {
  return fail(c, MCX_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define CK(call, what)                                   \
  do {                                                   \
    cudaError_t e_ = (call);                             \
    if (e_ != cudaSuccess) return cudaFail(c, e_, what); \
  } while (0)

__global__ void transposeKernel(const float* __restrict__ in, float* __restrict__ out, int rows, int cols) {
  // in: [rows][cols] -> out: [cols][rows]
  __shared__ float tile[32][33];
  int bx = blockIdx.x * 32, by = blockIdx.y * 32;
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    int r = by + j, cc = bx + threadIdx.x;
    if (r < rows && cc < cols) tile[j][threadIdx.x] = in[(size_t)r * cols + cc];
  }
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    int r = bx + j, cc = by + threadIdx.x;
    if (r < cols && cc < rows) out[(size_t)r * rows + cc] = tile[threadIdx.x][j];
  }
}

cudaError_t transpose(const float* in, float* out, int rows, int cols, cudaStream_t s) {
  dim3 b(32, 8), g((cols + 31) / 32, (rows + 31) / 32);
  transposeKernel<<<g, b, 0, s>>>(in, out, rows, cols);
  return cudaGetLastError();
}

// j = (j * mul) / div, two roundings as in source/iteration_mod.f90:1002-1031
// the same with the divisor of each cell's nebula (a batch mixing octant and full grids)
__global__ void scaleJCellKernel(double* j, size_t n, size_t C1, double mul, const float* __restrict__ div) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double v = j[i] * mul;
  const double d = (double)div[i % C1];
  if (d != 1.) v = v / d;
  j[i] = v;
}

// After a transport launch: J += Jlo (the exact rounding errors of its FP64
// atomics) and Jlo = 0, so J is the correctly rounded sum of the deposits.
__global__ void foldJKernel(double* __restrict__ j, double* __restrict__ lo, size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const double e = lo[i];
    if (e != 0.) {
      j[i] += e;
      lo[i] = 0.;
    }
  }
}

static cudaError_t foldJ(mcx_ctx* c) {
  foldJKernel<<<(unsigned)c->numSMs * 8, 256, 0, c->stream>>>(c->jste.p, c->jlo.p, c->jste.n);
  return cudaGetLastError();
}

// four entries per thread, one thread per four (a memory-bound pass over 331 MB
// wants every load in flight at once rather than a grid-stride loop)
__global__ void scaleJKernel(double* j, size_t n, double mul, double div) {
  const size_t i0 = (blockIdx.x * (size_t)blockDim.x + threadIdx.x) * 4;
  if (i0 >= n) return;
  double v[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) v[q] = i0 + q < n ? j[i0 + q] : 0.;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    v[q] = v[q] * mul;
    if (div != 1.) v[q] = v[q] / div;
  }
#pragma unroll
  for (int q = 0; q < 4; ++q)
    if (i0 + q < n) j[i0 + q] = v[q];
}

template <typename T>
cudaError_t upload(DBuf<T>& b, const std::vector<T>& v) {
  cudaError_t e = b.alloc(v.size());
  if (e != cudaSuccess) return e;
  if (v.empty()) return cudaSuccess;
  return cudaMemcpy(b.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
}

}  // namespace

extern "C" int mcx_ctx_create(int32_t device, mcx_ctx** out) {
  if (!out) return MCX_ERR_INPUT;
  *out = nullptr;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n <= device || device < 0) {
    g_setupError = std::string("mcx_ctx_create: no CUDA device ") + std::to_string(device) + ": " +
                   (e != cudaSuccess ? cudaGetErrorString(e) : "device index out of range");
    return MCX_ERR_CUDA;
  }
  auto* c = new (std::nothrow) mcx_ctx();
  if (!c) return MCX_ERR_NOMEM;
  c->device = device;
  if ((e = cudaSetDevice(device)) != cudaSuccess || (e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking)) != cudaSuccess ||
      (e = cudaEventCreate(&c->ev0)) != cudaSuccess || (e = cudaEventCreate(&c->ev1)) != cudaSuccess ||
      (e = cudaEventCreate(&c->tev0)) != cudaSuccess || (e = cudaEventCreate(&c->tev1)) != cudaSuccess) {
    g_setupError = std::string("mcx_ctx_create: ") + cudaGetErrorString(e);
    delete c;
    return MCX_ERR_CUDA;
  }
  cudaDeviceGetAttribute(&c->numSMs, cudaDevAttrMultiProcessorCount, device);
  *out = c;
  return MCX_OK;
}

extern "C" void mcx_ctx_destroy(mcx_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  if (c->tev0) cudaEventDestroy(c->tev0);
  if (c->tev1) cudaEventDestroy(c->tev1);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

extern "C" int mcx_last_error(const mcx_ctx* c, char* buf, size_t len) {
  if (!buf || len == 0) return MCX_ERR_INPUT;
  const std::string& m = c ? c->err : g_setupError;
  std::snprintf(buf, len, "%s", m.c_str());
  return MCX_OK;
}

// The float arrays of an iteration-boundary snapshot: the gas state and the
// phase outputs that the skip rule (source/iteration_mod.f90:131-149,
// :340-356) carries from one iteration into the next.
static std::vector<DBuf<float>*> snapshotArrays(mcx_ctx* c) {
  std::vector<DBuf<float>*> v = {&c->te, &c->ne, &c->teOld, &c->neOld, &c->ionDen, &c->opacity, &c->recPDF,
                                 &c->recCDFT, &c->totalLines, &c->forLines, &c->gauntTe};
  for (DBuf<float>* d : {&c->scaOpac, &c->dustPDF, &c->dustCDFT, &c->tdust})
    if (d->p) v.push_back(d);
  return v;
}

extern "C" int mcx_state_save_slot(mcx_ctx* c, int32_t slot) {
  if (!c) return MCX_ERR_INPUT;
  if (!c->loaded) return fail(c, MCX_ERR_STATE, "mcx_state_save: no model loaded");
  if (slot < 0 || slot >= MCX_STATE_SLOTS)
    return fail(c, MCX_ERR_INPUT, "mcx_state_save: slot out of range [0, MCX_STATE_SLOTS)");
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  if ((int)c->snaps.size() <= slot) c->snaps.resize(slot + 1);
  mcx_ctx::Snapshot& sn = c->snaps[slot];
  std::vector<DBuf<float>*> src = snapshotArrays(c);
  if (sn.f.size() != src.size()) sn.f = std::vector<DBuf<float>>(src.size());
  for (size_t k = 0; k < src.size(); ++k) {
    if (sn.f[k].n != src[k]->n) CK(sn.f[k].alloc(src[k]->n), "alloc snapshot");
    if (src[k]->n)
      CK(cudaMemcpyAsync(sn.f[k].p, src[k]->p, src[k]->bytes(), cudaMemcpyDeviceToDevice, c->stream), "snapshot");
  }
  if (sn.converged.n != c->lgConverged.n) CK(sn.converged.alloc(c->lgConverged.n), "alloc snapshot");
  CK(cudaMemcpyAsync(sn.converged.p, c->lgConverged.p, c->lgConverged.bytes(), cudaMemcpyDeviceToDevice, c->stream),
     "snapshot");
  sn.gauntTeOld = c->gauntTeOld;
  sn.nebGauntTeOld = c->nebGauntTeOld;
  sn.haveOpacity = c->haveOpacity; sn.haveRecPDF = c->haveRecPDF; sn.haveDustPDF = c->haveDustPDF;
  sn.valid = true;
  return MCX_OK;
}

extern "C" int mcx_state_restore_slot(mcx_ctx* c, int32_t slot) {
  if (!c) return MCX_ERR_INPUT;
  if (!c->loaded || slot < 0 || slot >= (int)c->snaps.size() || !c->snaps[slot].valid)
    return fail(c, MCX_ERR_STATE, "mcx_state_restore: no snapshot in this slot");
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  mcx_ctx::Snapshot& sn = c->snaps[slot];
  std::vector<DBuf<float>*> dst = snapshotArrays(c);
  if (dst.size() != sn.f.size()) return fail(c, MCX_ERR_STATE, "mcx_state_restore: snapshot of another model");
  for (size_t k = 0; k < dst.size(); ++k) {
    if (dst[k]->n != sn.f[k].n) return fail(c, MCX_ERR_STATE, "mcx_state_restore: snapshot of another model");
    if (dst[k]->n)
      CK(cudaMemcpyAsync(dst[k]->p, sn.f[k].p, sn.f[k].bytes(), cudaMemcpyDeviceToDevice, c->stream), "restore");
  }
  CK(cudaMemcpyAsync(c->lgConverged.p, sn.converged.p, sn.converged.bytes(), cudaMemcpyDeviceToDevice, c->stream),
     "restore");
  c->gauntTeOld = sn.gauntTeOld;
  c->nebGauntTeOld = sn.nebGauntTeOld;
  c->haveOpacity = sn.haveOpacity; c->haveRecPDF = sn.haveRecPDF; c->haveDustPDF = sn.haveDustPDF;
  return MCX_OK;
}

extern "C" int mcx_state_save(mcx_ctx* c) { return mcx_state_save_slot(c, 0); }
extern "C" int mcx_state_restore(mcx_ctx* c) { return mcx_state_restore_slot(c, 0); }

extern "C" int mcx_sync(mcx_ctx* c) {
  if (!c) return MCX_ERR_INPUT;
  CK(cudaStreamSynchronize(c->stream), "mcx_sync");
  return MCX_OK;
}

// Build the opacity kernel's per-bin CSR list of bound-free terms in the
// summation order of addOpacity (source/ionization_mod.f90:375-390).
static void buildOpacityTables(const Setup& s, std::vector<int32_t>& csrStart, std::vector<int2>& csrTerm,
                               std::vector<int32_t>& slotPlane, std::vector<float>& slotAbun,
                               std::vector<float>& slotFF) {
  const int nb = s.nbins, S = s.p.nstages, E = std::max(s.nElemUsed, 1);
  int slotOf[31][32];
  for (auto& r : slotOf) for (auto& x : r) x = -1;
  auto slot = [&](int n, int ion) {
    if (slotOf[n][ion] >= 0) return slotOf[n][ion];
    int id = (int)slotPlane.size();
    slotOf[n][ion] = id;
    int xr = s.elemXref[n - 1];
    slotPlane.push_back((xr - 1) + E * (ion - 1));
    slotAbun.push_back(s.elemAbun[n - 1]);
    // free-free electron sum: density(2,2) + sum_{n>=3} i^2 density(n,i+1)
    float w = 0.f;
    if (n == 2 && ion == 2) w = 1.f;
    else if (n >= 3 && ion >= 2 && ion - 1 <= std::min(n, S - 1)) w = (float)((ion - 1) * (ion - 1));
    slotFF.push_back(w);
    return id;
  };
  // all slots of ions with a filled density, in element order, so that every
  // free-free contributor has a slot
  for (int n = 1; n <= 30; ++n) {
    if (!s.elemOn[n - 1]) continue;
    for (int i = 1; i <= std::min(n, S); ++i) slot(n, i);
  }
  struct Range { int lo, hi, k, slot; };
  std::vector<Range> ranges;
  auto inOpacity = [&](int xSecP, int lo, int hi, int sl) {
    int iup = std::min(hi, nb);
    iup = std::max(lo, iup);
    ranges.push_back({lo, iup, xSecP - lo, sl});
  };
  if (s.elemOn[0]) inOpacity(s.HlevXSecP[0], s.HlevNuP[0], nb, slot(1, 1));
  if (s.elemOn[1]) {
    inOpacity(s.HeISingXSecP[0], s.HeIlevNuP[0], nb, slot(2, 1));
    inOpacity(s.HeIIXSecP[0], s.HeIIlevNuP[0], nb, slot(2, 2));
  }
  for (int n = 3; n <= 30; ++n) {
    if (!s.elemOn[n - 1]) continue;
    for (int ion = 1; ion <= std::min(n, S); ++ion)
      for (int sh = 1; sh <= s.nShells[n - 1][ion - 1]; ++sh) {
        const int* P = s.elementP[n - 1][ion - 1][sh - 1];
        inOpacity(P[2], P[0], P[1], slot(n, ion));
      }
  }
  std::vector<std::vector<int2>> per(nb + 1);
  for (const auto& r : ranges)
    for (int i = std::max(r.lo, 1); i <= std::min(r.hi, nb); ++i) per[i].push_back(make_int2(r.k, r.slot));
  // each term carries its cross section at the bin (xSecArray(i + k), 0 outside the table) as float bits
  csrStart.assign(nb + 1, 0);
  csrTerm.clear();
  const int nX = (int)s.xSec.size();
  for (int i = 1; i <= nb; ++i) {
    csrStart[i - 1] = (int32_t)csrTerm.size();
    for (const int2& t : per[i]) {
      const int xi = i + t.x;
      const float xs = (xi >= 1 && xi <= nX) ? s.xSec[(size_t)(xi - 1)] : 0.f;
      int32_t bits;
      std::memcpy(&bits, &xs, sizeof bits);
      csrTerm.push_back(make_int2(bits, t.y));
    }
  }
  csrStart[nb] = (int32_t)csrTerm.size();
}

static int loadSetup(mcx_ctx* c, const Setup& s);

extern "C" int mcx_load(mcx_ctx* c, const mcx_setup* m) {
  if (!c || !m) return fail(c, MCX_ERR_INPUT, "mcx_load: null argument");
  c->nNeb = 0;
  c->nebCellOff.clear();
  return loadSetup(c, m->s);
}

static int loadSetup(mcx_ctx* c, const Setup& s) {
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  c->loaded = false;
  c->nx = s.nx; c->ny = s.ny; c->nz = s.nz; c->nCells = s.nCells; c->nbins = s.nbins;
  c->nstages = s.p.nstages; c->nElemUsed = std::max(s.nElemUsed, 1); c->nXsec = (int)s.xSec.size();
  c->symmetric = s.p.lgSymmetricXYZ; c->lgDust = s.p.lgDust; c->lgGas = s.p.lgGas;
  c->lgCompton = s.p.lgCompton; c->radPress = s.p.lgRadPress;
  c->lStar = s.LStar; c->ionEdge1 = s.ionEdge.empty() ? 0.f : s.ionEdge[0]; c->rOut = s.p.R_out;
  c->nPhotons = s.p.nPhotons;
  for (int d = 0; d < 3; ++d) { c->starIdx[d] = s.starIdx[d]; c->starPos[d] = s.starPos[d]; }
  c->stars = starTable(s);
  c->nStars = (int)(c->stars.size() / 8);
  c->gauntTeOld = -1.f;
  // validate what the kernels index with
  for (int32_t a : s.active)
    if (a < 0 || a > s.nCells) return fail(c, MCX_ERR_INPUT, "mcx_load: active() holds ids outside [0, nCells] (sub-grids are not supported)");
  if (s.nbins < 2 || s.nCells < 1) return fail(c, MCX_ERR_INPUT, "mcx_load: empty grid or frequency mesh");
  for (int i = 0; i < c->nStars && !s.p.lgPlaneIonization; ++i) {
    const float* r = c->stars.data() + 8 * i;
    if (r[5] < 1.f || r[5] > (float)s.nx || r[6] < 1.f || r[6] > (float)s.ny || r[7] < 1.f || r[7] > (float)s.nz)
      return fail(c, MCX_ERR_INPUT, "mcx_load: source " + std::to_string(i + 1) + " must lie inside the grid");
  }
  c->plane = s.p.lgPlaneIonization ? 1 : 0;
  c->activeHost = s.active;
  c->activeFull = 1;
  for (int k = 0; k < s.nz && c->activeFull; ++k)
    for (int j = 0; j < s.ny && c->activeFull; ++j)
      for (int i = 0; i < s.nx; ++i)
        if (s.active[(size_t)i + (size_t)s.nx * ((size_t)j + (size_t)s.ny * k)] != (i * s.ny + j) * s.nz + k + 1) {
          c->activeFull = 0;
          break;
        }
  // viewing-angle bins (initCartesianGrid, source/grid_mod.f90:570-601): theta in 20 bins over
  // [0, pi], phi in 20 over [0, 2 pi) unless a view's phi is negative (no phi dependence)
  c->nAngle = s.p.nAngleBins;
  c->totPhi = 20;
  std::memset(c->viewPTheta, 0, sizeof c->viewPTheta);
  std::memset(c->viewPPhi, 0, sizeof c->viewPPhi);
  if (c->nAngle > 0) {
    float vphi[2] = {s.p.viewPhi[0], s.p.viewPhi[1]};
    for (int i = 0; i < c->nAngle; ++i)
      if (vphi[i] < 0.f) { c->totPhi = 1; vphi[0] = vphi[1] = -1.f; break; }
    const float pi = 3.141592654f, dTheta = pi / 20.f, dPhi = (2.f * pi) / (float)c->totPhi;
    for (int i = 0; i < c->nAngle; ++i) {
      const int kt = (int)(s.p.viewTheta[i] / dTheta) + 1, kp = (int)(vphi[i] / dPhi) + 1;
      if (kt < 0 || kt > 20 || kp < 0 || kp > c->totPhi)
        return fail(c, MCX_ERR_INPUT, "mcx_load: an inclination angle lies outside [0, pi] x [0, 2 pi)");
      c->viewPTheta[kt] = (int8_t)(i + 1);
      c->viewPPhi[kp] = (int8_t)(i + 1);
    }
  }

  const int nb = s.nbins;
  const size_t C1 = (size_t)s.nCells + 1;
  std::vector<float> l10(nb);
  for (int i = 0; i < nb; ++i) l10[i] = log10f(s.nu[i]);
  std::vector<float> knT((size_t)nb * 180), pcT((size_t)nb * 180);
  for (int i = 0; i < nb; ++i)
    for (int j = 0; j < 180; ++j) {
      knT[(size_t)i * 180 + j] = s.KNcdf[(size_t)j * nb + i];
      pcT[(size_t)i * 180 + j] = s.Pcomp[(size_t)j * nb + i];
    }
  std::vector<double> vd(C1, 1.0);
  std::vector<float> vf(C1, 1.f);
  for (int i = 1; i <= s.nx; ++i)
    for (int j = 1; j <= s.ny; ++j)
      for (int k = 1; k <= s.nz; ++k) {
        int cell = s.activeAt(i, j, k);
        if (cell > 0) { vd[cell] = volumeD(s, i, j, k); vf[cell] = s.volume[cell]; }
      }
  CK(upload(c->nu, s.nu), "upload nu");
  CK(upload(c->log10nu, l10), "upload log10nu");
  CK(upload(c->xsec, s.xSec.empty() ? std::vector<float>(1, 0.f) : s.xSec), "upload xsec");
  CK(upload(c->KNsigmaT, s.KNsigmaT), "upload KNsigmaT");
  CK(upload(c->KNcdfT, knT), "upload KN cdf");
  CK(upload(c->PcompT, pcT), "upload Pcomp");
  CK(upload(c->srcCDF, sourceCDFs(s)), "upload srcCDF");
  CK(upload(c->xAxis, s.xAxis), "upload xAxis");
  CK(upload(c->yAxis, s.yAxis), "upload yAxis");
  CK(upload(c->zAxis, s.zAxis), "upload zAxis");
  CK(upload(c->active, s.active), "upload active");
  CK(upload(c->volD, vd), "upload volume");
  CK(upload(c->volF, vf), "upload volume");
  std::vector<int32_t> cs, sp;
  std::vector<int2> ct;
  std::vector<float> sa, sf;
  buildOpacityTables(s, cs, ct, sp, sa, sf);
  c->nSlots = (int)sp.size();
  c->bremsP0 = s.bremsXSecP - 1;
  CK(upload(c->csrStart, cs), "upload csr");
  CK(upload(c->csrTerm, ct.empty() ? std::vector<int2>(1, make_int2(0, 0)) : ct), "upload csr");
  CK(upload(c->slotPlane, sp.empty() ? std::vector<int32_t>(1, 0) : sp), "upload slots");
  CK(upload(c->slotAbun, sa.empty() ? std::vector<float>(1, 0.f) : sa), "upload slots");
  CK(upload(c->slotFFWeight, sf.empty() ? std::vector<float>(1, 0.f) : sf), "upload slots");
  CK(upload(c->hden, s.Hden), "upload Hden");
  CK(upload(c->te, s.Te), "upload Te");
  CK(upload(c->ne, s.Ne), "upload Ne");
  CK(upload(c->teOld, s.TeOld), "upload TeOld");
  CK(upload(c->neOld, s.NeOld), "upload NeOld");
  CK(upload(c->ionDen, s.ionDen), "upload ionDen");
  CK(upload(c->ndust, s.Ndust), "upload Ndust");
  CK(c->opacity.alloc(C1 * nb), "alloc opacity");
  CK(c->recPDF.alloc(C1 * nb), "alloc recPDF");
  CK(c->recCDFT.alloc(C1 * nb), "alloc recCDF");
  CK(c->totalLines.alloc(C1), "alloc totalLines");
  CK(c->jste.alloc(C1 * nb), "alloc Jste");
  CK(c->jlo.alloc(C1 * nb), "alloc Jste compensation");
  CK(c->parked.alloc(kParkedCap * std::max(parkedPacketBytesF32(), parkedPacketBytesF64())), "alloc parked packets");
  CK(c->escaped.alloc(C1 * (nb + 1) * (size_t)(c->nAngle + 1)), "alloc escaped");
  if (c->radPress) CK(c->hEst.alloc(C1 * nb), "alloc H");
  if (c->lgDust) {
    CK(c->scaOpac.alloc(C1 * nb), "alloc scaOpac");
    CK(c->dustPDF.alloc(C1 * nb), "alloc dustPDF");
    CK(c->dustCDFT.alloc(C1 * nb), "alloc dustCDF");
  }
  CK(c->gauntTe.alloc(C1), "alloc gauntTe");
  CK(c->computeMask.alloc(C1), "alloc mask");
  CK(c->counters.alloc(1), "alloc counters");
  CK(cudaMemset(c->opacity.p, 0, c->opacity.bytes()), "memset");
  CK(cudaMemset(c->recPDF.p, 0, c->recPDF.bytes()), "memset");
  CK(cudaMemset(c->recCDFT.p, 0, c->recCDFT.bytes()), "memset");
  CK(cudaMemset(c->totalLines.p, 0, c->totalLines.bytes()), "memset");
  CK(cudaMemset(c->jste.p, 0, c->jste.bytes()), "memset");
  CK(cudaMemset(c->jlo.p, 0, c->jlo.bytes()), "memset");
  CK(cudaMemset(c->escaped.p, 0, c->escaped.bytes()), "memset");
  if (c->hEst.p) CK(cudaMemset(c->hEst.p, 0, c->hEst.bytes()), "memset");
  if (c->scaOpac.p) CK(cudaMemset(c->scaOpac.p, 0, c->scaOpac.bytes()), "memset");
  CK(c->lgConverged.alloc(C1), "alloc lgConverged");
  CK(c->lgBlack.alloc(C1), "alloc lgBlack");
  CK(c->nIterT.alloc(C1), "alloc nIterT");
  CK(c->forLines.alloc(C1), "alloc forLines");
  CK(cudaMemset(c->lgConverged.p, 0, c->lgConverged.bytes()), "memset");
  CK(cudaMemset(c->lgBlack.p, 0, c->lgBlack.bytes()), "memset");
  CK(cudaMemset(c->nIterT.p, 0, c->nIterT.bytes()), "memset");
  CK(cudaMemset(c->forLines.p, 0, c->forLines.bytes()), "memset");
  c->emission.reset();
  c->balance.reset();
  c->dust.reset();
  c->snaps.clear();
  if (c->lgDust) {
    std::string dm = dustDataCreate(s, c->dust);
    if (!dm.empty()) return fail(c, MCX_ERR_INPUT, "mcx_load: " + dm);
    CK(upload(c->tdust, s.Tdust), "upload Tdust");
  }
  if (c->lgGas) {
    std::string em = emissionDataCreate(s, c->emission);
    if (!em.empty()) return fail(c, MCX_ERR_INPUT, "mcx_load: " + em);
    std::string bl = balanceDataCreate(s, c->balance);
    if (!bl.empty()) return fail(c, MCX_ERR_INPUT, "mcx_load: " + bl);
    // the line factors of equilibrium (source/emission_mod.f90:2987-3004)
    c->lineAtoms.clear();
    for (int a = 0; a < s.bal.nAtoms; ++a) {
      const int32_t* h = s.bal.atomHdr.data() + (size_t)a * kAtHdrSize;
      const double* D = s.bal.atomData.data();
      mcx_ctx::LineAtom la;
      la.elem = h[kAtElem]; la.ion = h[kAtIon]; la.nLev = h[kAtNLev];
      const int n = la.nLev;
      la.fac.assign((size_t)n * n, 0.);
      la.wav.assign((size_t)n * n, 0.);
      const double* A = D + h[kAtOffA];
      const double* E = D + h[kAtOffE];
      const double atp = D[h[kAtOffAtp]];
      for (int i = 1; i <= n - 1; ++i)
        for (int j = i + 1; j <= n; ++j) {
          double aji = A[(size_t)(j - 1) * n + (i - 1)];
          if (aji == 0.) continue;
          const double Eji = E[j - 1] - E[i - 1];
          if (j == h[kAtIup2p] && i == 1 && atp > 0.) aji = aji - atp;
          la.fac[(size_t)(i - 1) * n + (j - 1)] = aji * Eji;
          la.wav[(size_t)(i - 1) * n + (j - 1)] = Eji > 0. ? 1.e8 / Eji : 0.;
        }
      c->lineAtoms.push_back(std::move(la));
    }
    for (int z = 0; z < 30; ++z) c->xrefAll[z] = s.elemXref[z];
  }
  CK(cudaDeviceSynchronize(), "mcx_load");
  c->haveOpacity = c->haveRecPDF = c->haveDustPDF = false;
  c->loaded = true;
  return MCX_OK;
}

// -------------------------------------------------------------- batches
extern "C" int mcx_load_batched(mcx_ctx* c, const mcx_setup* const* setups, int32_t n) {
  if (!c || !setups || n < 1) return fail(c, MCX_ERR_INPUT, "mcx_load_batched: null argument or empty batch");
  if (n > 32767) return fail(c, MCX_ERR_INPUT, "mcx_load_batched: at most 32767 nebulae");
  for (int b = 0; b < n; ++b)
    if (!setups[b]) return fail(c, MCX_ERR_INPUT, "mcx_load_batched: null set-up");
  const Setup& s0 = setups[0]->s;
  auto bad = [&](int b, const char* what) {
    return fail(c, MCX_ERR_INPUT, "mcx_load_batched: nebula " + std::to_string(b) + " differs from nebula 0 in " + what);
  };
  int64_t total = 0;
  for (int b = 0; b < n; ++b) {
    const Setup& s = setups[b]->s;
    if (!s.p.lgGas || s.p.lgDust) return fail(c, MCX_ERR_INPUT, "mcx_load_batched: a batch holds gas-only nebulae");
    if (s.p.nAngleBins > 0) return fail(c, MCX_ERR_INPUT, "mcx_load_batched: viewing angles (inclination) are not batched");
    if (s.p.lgPlaneIonization) return fail(c, MCX_ERR_INPUT, "mcx_load_batched: plane-parallel models are not batched");
    if (s.p.lgRadPress) return fail(c, MCX_ERR_INPUT, "mcx_load_batched: radiation pressure is not supported in a batch");
    if (s.nbins != s0.nbins || s.nu != s0.nu || s.widFlx != s0.widFlx) return bad(b, "the frequency mesh");
    if (s.p.nstages != s0.p.nstages || s.nElemUsed != s0.nElemUsed) return bad(b, "nstages or the elements");
    for (int z = 0; z < kNElements; ++z)
      if (s.elemXref[z] != s0.elemXref[z] || s.elemAbun[z] != s0.elemAbun[z]) return bad(b, "the abundances");
    if (s.p.lgCompton != s0.p.lgCompton) return bad(b, "the Compton switch");
    if (s.xSec != s0.xSec || s.ionEdge != s0.ionEdge) return bad(b, "the cross-section tables");
    for (int32_t a : s.active)
      if (a < 0 || a > s.nCells) return fail(c, MCX_ERR_INPUT, "mcx_load_batched: sub-grids are not supported");
    if (s.starIdx[0] < 1 || s.starIdx[0] > s.nx || s.starIdx[1] < 1 || s.starIdx[1] > s.ny || s.starIdx[2] < 1 ||
        s.starIdx[2] > s.nz)
      return fail(c, MCX_ERR_INPUT, "mcx_load_batched: a source lies outside its grid");
    if (s.stars.size() > 1) return fail(c, MCX_ERR_INPUT, "mcx_load_batched: one ionising source per nebula");
    total += s.nCells;
  }
  if (total > (int64_t)INT32_MAX - 1) return fail(c, MCX_ERR_INPUT, "mcx_load_batched: too many cells");
  // the concatenated per-cell state: nebula b owns cells off[b]+1 .. off[b+1]
  std::vector<int32_t> off(n + 1, 0);
  for (int b = 0; b < n; ++b) off[b + 1] = off[b] + setups[b]->s.nCells;
  const size_t C1 = (size_t)total + 1;
  const int S = s0.p.nstages, E = std::max(s0.nElemUsed, 1);
  Setup comb = s0;
  comb.nCells = (int)total;
  auto concat = [&](std::vector<float> Setup::*f, float fill0) {
    std::vector<float> v(C1, fill0);
    for (int b = 0; b < n; ++b) {
      const std::vector<float>& src = setups[b]->s.*f;
      for (int k = 1; k <= setups[b]->s.nCells; ++k) v[off[b] + k] = src[k];
    }
    comb.*f = std::move(v);
  };
  concat(&Setup::Hden, s0.Hden[0]);
  concat(&Setup::Te, s0.Te[0]);
  concat(&Setup::Ne, s0.Ne[0]);
  concat(&Setup::TeOld, s0.TeOld[0]);
  concat(&Setup::NeOld, s0.NeOld[0]);
  concat(&Setup::volume, 1.f);
  comb.Ndust.assign(C1, 0.f);
  comb.ionDen.assign((size_t)S * E * C1, 0.f);
  for (int b = 0; b < n; ++b) {
    const Setup& s = setups[b]->s;
    const size_t Cb1 = (size_t)s.nCells + 1;
    for (size_t plane = 0; plane < (size_t)S * E; ++plane) {
      comb.ionDen[plane * C1] = s0.ionDen[plane * ((size_t)s0.nCells + 1)];
      for (int k = 1; k <= s.nCells; ++k) comb.ionDen[plane * C1 + off[b] + k] = s.ionDen[plane * Cb1 + k];
    }
  }
  int rc = loadSetup(c, comb);
  if (rc != MCX_OK) return rc;
  c->loaded = false;
  // batch geometry
  std::vector<double> vd(C1, 1.0);
  std::vector<float> vf(C1, 1.f), axes, cdfs, jdiv(C1, 1.f);
  std::vector<int32_t> act;
  std::vector<int16_t> ffIdx(C1, 0);
  c->nebDesc.assign(n, NebulaDesc{});
  c->nebLStar.assign(n, 0.f);
  c->nebSym.assign(n, 0);
  c->nebNx.assign(n, 0); c->nebNy.assign(n, 0); c->nebNz.assign(n, 0);
  c->nebActive.assign(n, {});
  for (int b = 0; b < n; ++b) {
    const Setup& s = setups[b]->s;
    NebulaDesc& d = c->nebDesc[b];
    d.nx = s.nx; d.ny = s.ny; d.nz = s.nz; d.symmetric = s.p.lgSymmetricXYZ ? 1 : 0;
    d.axOff = (int32_t)axes.size();
    axes.insert(axes.end(), s.xAxis.begin(), s.xAxis.end());
    axes.insert(axes.end(), s.yAxis.begin(), s.yAxis.end());
    axes.insert(axes.end(), s.zAxis.begin(), s.zAxis.end());
    d.actOff = (int32_t)act.size();
    std::vector<int32_t> ab(s.active.size());
    for (size_t v = 0; v < s.active.size(); ++v) ab[v] = s.active[v] > 0 ? s.active[v] + off[b] : 0;
    act.insert(act.end(), ab.begin(), ab.end());
    c->nebActive[b] = std::move(ab);
    d.cdfOff = (int32_t)cdfs.size();
    cdfs.insert(cdfs.end(), s.srcCDF.begin(), s.srcCDF.end());
    for (int k = 0; k < 3; ++k) { d.starIdx[k] = s.starIdx[k]; d.starPos[k] = s.starPos[k]; }
    d.rOut = s.p.R_out;
    c->nebLStar[b] = s.LStar;
    c->nebSym[b] = d.symmetric;
    c->nebNx[b] = s.nx; c->nebNy[b] = s.ny; c->nebNz[b] = s.nz;
    for (int i = 1; i <= s.nx; ++i)
      for (int j = 1; j <= s.ny; ++j)
        for (int k = 1; k <= s.nz; ++k) {
          const int cell = s.activeAt(i, j, k);
          if (cell > 0) { vd[off[b] + cell] = volumeD(s, i, j, k); vf[off[b] + cell] = s.volume[cell]; }
        }
    for (int k = 1; k <= s.nCells; ++k) {
      ffIdx[off[b] + k] = (int16_t)b;
      jdiv[off[b] + k] = d.symmetric ? 8.f : 1.f;
    }
  }
  CK(upload(c->volD, vd), "upload volume");
  CK(upload(c->volF, vf), "upload volume");
  CK(upload(c->nebAxes, axes), "upload batch axes");
  CK(upload(c->nebActiveDev, act), "upload batch active");
  CK(upload(c->nebCdf, cdfs), "upload batch source CDFs");
  CK(upload(c->nebFfIdx, ffIdx), "upload batch Gaunt index");
  CK(upload(c->jDiv, jdiv), "upload batch octant factors");
  CK(c->nebFfK.alloc((size_t)n * 2 * c->nbins), "alloc batch Gaunt tables");
  CK(c->nebGauntTeDev.alloc(n), "alloc batch Gaunt temperatures");
  CK(c->nebDescDev.alloc(n), "alloc batch descriptors");
  CK(c->nebPktBegin.alloc((size_t)n + 1), "alloc batch packet offsets");
  CK(c->nebStamps.alloc((size_t)n + 1), "alloc batch timers");
  CK(cudaMemset(c->nebStamps.p, 0, c->nebStamps.bytes()), "memset");
  CK(cudaDeviceSynchronize(), "mcx_load_batched");
  c->nebGauntTeOld.assign(n, -1.f);
  c->nebCellOff = off;
  c->nNeb = n;
  c->loaded = true;
  return MCX_OK;
}

extern "C" int mcx_batch_info(mcx_ctx* c, int32_t* n_nebulae, int32_t* cell_offset) {
  if (!c || !n_nebulae) return fail(c, MCX_ERR_INPUT, "mcx_batch_info: null argument");
  if (!c->loaded) return fail(c, MCX_ERR_STATE, "mcx_batch_info: no model loaded");
  *n_nebulae = c->nNeb;
  if (cell_offset)
    for (int b = 0; b <= c->nNeb; ++b) cell_offset[b] = c->nebCellOff[b];
  return MCX_OK;
}

namespace {

struct ArrView {
  void* dev;
  size_t bytes;
};

ArrView viewOf(mcx_ctx* c, int id) {
  switch (id) {
    case MCX_ARR_NU: return {c->nu.p, c->nu.bytes()};
    case MCX_ARR_XSEC: return {c->xsec.p, c->xsec.bytes()};
    case MCX_ARR_SRC_CDF: return {c->srcCDF.p, (size_t)c->nbins * sizeof(float)};   // source 1's
    case MCX_ARR_KN_SIGMA_T: return {c->KNsigmaT.p, c->KNsigmaT.bytes()};
    case MCX_ARR_XAXIS: return {c->xAxis.p, c->xAxis.bytes()};
    case MCX_ARR_YAXIS: return {c->yAxis.p, c->yAxis.bytes()};
    case MCX_ARR_ZAXIS: return {c->zAxis.p, c->zAxis.bytes()};
    case MCX_ARR_ACTIVE: return {c->active.p, c->active.bytes()};
    case MCX_ARR_HDEN: return {c->hden.p, c->hden.bytes()};
    case MCX_ARR_TE: return {c->te.p, c->te.bytes()};
    case MCX_ARR_NE: return {c->ne.p, c->ne.bytes()};
    case MCX_ARR_TEOLD: return {c->teOld.p, c->teOld.bytes()};
    case MCX_ARR_NEOLD: return {c->neOld.p, c->neOld.bytes()};
    case MCX_ARR_IONDEN: return {c->ionDen.p, c->ionDen.bytes()};
    case MCX_ARR_OPACITY: return {c->opacity.p, c->opacity.bytes()};
    case MCX_ARR_RECPDF: return {c->recPDF.p, c->recPDF.bytes()};
    case MCX_ARR_TOTAL_LINES: return {c->totalLines.p, c->totalLines.bytes()};
    case MCX_ARR_JSTE: return {c->jste.p, c->jste.bytes()};
    case MCX_ARR_ESCAPED: return {c->escaped.p, c->escaped.bytes()};
    case MCX_ARR_VOLUME: return {c->volF.p, c->volF.bytes()};
    case MCX_ARR_GAUNT_TE: return {c->gauntTe.p, c->gauntTe.bytes()};
    case MCX_ARR_SCAOPAC: return {c->scaOpac.p, c->scaOpac.bytes()};
    case MCX_ARR_DUSTPDF: return {c->dustPDF.p, c->dustPDF.bytes()};
    case MCX_ARR_NDUST: return {c->ndust.p, c->ndust.bytes()};
    case MCX_ARR_H_EST: return {c->hEst.p, c->hEst.bytes()};
    case MCX_ARR_LG_CONVERGED: return {c->lgConverged.p, c->lgConverged.bytes()};
    case MCX_ARR_LG_BLACK: return {c->lgBlack.p, c->lgBlack.bytes()};
    case MCX_ARR_N_ITER_T: return {c->nIterT.p, c->nIterT.bytes()};
    case MCX_ARR_FOR_LINES: return {c->forLines.p, c->forLines.bytes()};
    case MCX_ARR_TDUST: return {c->tdust.p, c->tdust.bytes()};
    case MCX_ARR_BAL_RESID:
      if (!c->balance) return {nullptr, 0};
      return {c->balance->dev.resid, ((size_t)c->nCells + 1) * sizeof(double)};
    default: return {nullptr, 0};
  }
}

}  // namespace

extern "C" int mcx_get(mcx_ctx* c, int32_t id, void* host, size_t nbytes) {
  if (!c || (!host && nbytes)) return fail(c, MCX_ERR_INPUT, "mcx_get: null argument");
  if (!c->loaded) return fail(c, MCX_ERR_STATE, "mcx_get: no model loaded");
  ArrView v = viewOf(c, id);
  if (!v.dev) return fail(c, MCX_ERR_INPUT, "mcx_get: array id " + std::to_string(id) + " is not held by the context");
  if (v.bytes != nbytes) return fail(c, MCX_ERR_INPUT, "mcx_get: size mismatch, expected " + std::to_string(v.bytes) + " bytes");
  CK(cudaMemcpyAsync(host, v.dev, nbytes, cudaMemcpyDeviceToHost, c->stream), "mcx_get");
  CK(cudaStreamSynchronize(c->stream), "mcx_get");
  return MCX_OK;
}

extern "C" int mcx_put(mcx_ctx* c, int32_t id, const void* host, size_t nbytes) {
  if (!c || (!host && nbytes)) return fail(c, MCX_ERR_INPUT, "mcx_put: null argument");
  if (!c->loaded) return fail(c, MCX_ERR_STATE, "mcx_put: no model loaded");
  switch (id) {
    case MCX_ARR_NU: case MCX_ARR_XSEC: case MCX_ARR_XAXIS: case MCX_ARR_YAXIS: case MCX_ARR_ZAXIS:
    case MCX_ARR_ACTIVE: case MCX_ARR_VOLUME: case MCX_ARR_GAUNT_TE:
      return fail(c, MCX_ERR_INPUT, "mcx_put: geometry and tables are set by mcx_load");
    default: break;
  }
  ArrView v = viewOf(c, id);
  if (!v.dev) return fail(c, MCX_ERR_INPUT, "mcx_put: array id " + std::to_string(id) + " is not held by the context");
  if (v.bytes != nbytes) return fail(c, MCX_ERR_INPUT, "mcx_put: size mismatch, expected " + std::to_string(v.bytes) + " bytes");
  CK(cudaMemcpyAsync(v.dev, host, nbytes, cudaMemcpyHostToDevice, c->stream), "mcx_put");
  const int C1 = c->nCells + 1;
  if (id == MCX_ARR_RECPDF) { CK(transpose(c->recPDF.p, c->recCDFT.p, c->nbins, C1, c->stream), "transpose recPDF"); c->haveRecPDF = true; }
  if (id == MCX_ARR_DUSTPDF) { CK(transpose(c->dustPDF.p, c->dustCDFT.p, c->nbins, C1, c->stream), "transpose dustPDF"); c->haveDustPDF = true; }
  if (id == MCX_ARR_OPACITY) c->haveOpacity = true;
  CK(cudaStreamSynchronize(c->stream), "mcx_put");
  return MCX_OK;
}

extern "C" int mcx_device_ptr(mcx_ctx* c, int32_t id, void** dptr) {
  if (!c || !dptr) return fail(c, MCX_ERR_INPUT, "mcx_device_ptr: null argument");
  if (!c->loaded) return fail(c, MCX_ERR_STATE, "mcx_device_ptr: no model loaded");
  ArrView v = viewOf(c, id);
  if (!v.dev) return fail(c, MCX_ERR_INPUT, "mcx_device_ptr: unknown array id");
  *dptr = v.dev;
  return MCX_OK;
}

// ------------------------------------------------------------ opacity phase
// Skip rule of the opacity and emission loops (source/iteration_mod.f90:131-149,
// :340-356): for nIterateMC > 1, cells whose Te and Ne moved by less than 0.5 %
// keep last iteration's values.  Computed on the host from the device state.
static int skipMask(mcx_ctx* c, int it, std::vector<float>& te, std::vector<uint8_t>& mask, int64_t& computed,
                    int64_t& skipped) {
  const size_t C1 = (size_t)c->nCells + 1;
  std::vector<float> ne(C1), teOld(C1), neOld(C1);
  te.assign(C1, 0.f);
  mask.assign(C1, 0);
  CK(cudaMemcpyAsync(te.data(), c->te.p, C1 * 4, cudaMemcpyDeviceToHost, c->stream), "d2h Te");
  CK(cudaMemcpyAsync(ne.data(), c->ne.p, C1 * 4, cudaMemcpyDeviceToHost, c->stream), "d2h Ne");
  CK(cudaMemcpyAsync(teOld.data(), c->teOld.p, C1 * 4, cudaMemcpyDeviceToHost, c->stream), "d2h TeOld");
  CK(cudaMemcpyAsync(neOld.data(), c->neOld.p, C1 * 4, cudaMemcpyDeviceToHost, c->stream), "d2h NeOld");
  CK(cudaStreamSynchronize(c->stream), "skip rule");
  computed = skipped = 0;
  for (size_t cell = 1; cell < C1; ++cell) {
    bool skip = it > 1 && (std::fabs(te[cell] - teOld[cell]) / teOld[cell]) < 0.005f &&
                (std::fabs(ne[cell] - neOld[cell]) / neOld[cell]) < 0.005f;
    if (skip) ++skipped; else { mask[cell] = 1; ++computed; }
  }
  return MCX_OK;
}

extern "C" int mcx_emission(mcx_ctx* c, const mcx_phase_opts* opts, mcx_phase_stats* stats) {
  if (!c) return MCX_ERR_INPUT;
  if (!c->loaded) return fail(c, MCX_ERR_STATE, "mcx_emission: no model loaded");
  if (!c->lgGas && c->dust) {
    // dust-only grid: setDustPDF for every cell (source/emission_mod.f90:1921-1986)
    CK(cudaSetDevice(c->device), "cudaSetDevice");
    const int C1d = c->nCells + 1;
    CK(cudaEventRecord(c->ev0, c->stream), "event");
    CK(launchDustPDF(c->dust->dev, c->tdust.p, c->dustPDF.p, c->stream), "dust emission");
    CK(transpose(c->dustPDF.p, c->dustCDFT.p, c->nbins, C1d, c->stream), "transpose dustPDF");
    CK(cudaEventRecord(c->ev1, c->stream), "event");
    CK(cudaStreamSynchronize(c->stream), "mcx_emission");
    if (stats) {
      std::memset(stats, 0, sizeof(*stats));
      stats->cells_computed = c->nCells;
      cudaEventElapsedTime(&stats->kernel_ms, c->ev0, c->ev1);
    }
    c->haveDustPDF = true;
    return MCX_OK;
  }
  if (!c->lgGas || !c->emission) return fail(c, MCX_ERR_STATE, "mcx_emission: the grid holds no gas");
  if (c->gauntTeOld <= 0.f) return fail(c, MCX_ERR_STATE, "mcx_emission: run mcx_opacity first (its Gaunt factors are reused)");
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  const int it = opts ? opts->n_iterate_mc : 1;
  std::vector<float> te;
  std::vector<uint8_t> mask;
  int64_t computed = 0, skipped = 0;
  int rc = skipMask(c, it, te, mask, computed, skipped);
  if (rc != MCX_OK) return rc;
  const size_t C1 = (size_t)c->nCells + 1;
  CK(cudaMemcpyAsync(c->computeMask.p, mask.data(), C1, cudaMemcpyHostToDevice, c->stream), "h2d mask");
  CK(cudaEventRecord(c->ev0, c->stream), "event");
  EmissionDev ed = c->emission->dev;
  if (c->nNeb > 0) {
    // one Gaunt table per nebula, each at its own cache temperature
    c->nebGauntTemps.resize(c->nNeb);
    for (int b = 0; b < c->nNeb; ++b)
      c->nebGauntTemps[b] = c->nebGauntTeOld[b] > 0.f ? c->nebGauntTeOld[b] : c->gauntTeOld;
    CK(cudaMemcpyAsync(c->nebGauntTeDev.p, c->nebGauntTemps.data(), sizeof(float) * c->nNeb, cudaMemcpyHostToDevice,
                       c->stream), "h2d Gaunt temperatures");
    ed.ffK = c->nebFfK.p;
    CK(launchEmissionGauntBatched(ed, c->nebGauntTeDev.p, c->nNeb, c->stream), "emission gaunt");
    ed.ffIdx = c->nebFfIdx.p;
  } else {
    CK(launchEmissionGaunt(ed, c->gauntTeOld, c->stream), "emission gaunt");
  }
  const float* forLines = nullptr;
  if (c->balance && c->balance->dev.nAtoms > 0) {
    const int prec = (opts && opts->precision == MCX_PHASE_MIXED) ? kBalMixed : kBalFp64;
    CK(launchForLinesEmission(*c->balance, c->te.p, c->ne.p, c->ionDen.p, c->computeMask.p, c->forLines.p, prec,
                              c->stream),
       "emission forLines");
    forLines = c->forLines.p;
  }
  CK(launchEmission(ed, c->te.p, c->ne.p, c->ionDen.p, c->computeMask.p, forLines, c->recPDF.p, c->totalLines.p,
                    opts && opts->precision == MCX_PHASE_MIXED, c->stream), "emission kernel");
  CK(transpose(c->recPDF.p, c->recCDFT.p, c->nbins, (int)C1, c->stream), "transpose recPDF");
  CK(cudaEventRecord(c->ev1, c->stream), "event");
  CK(cudaStreamSynchronize(c->stream), "mcx_emission");
  if (stats) {
    std::memset(stats, 0, sizeof(*stats));
    stats->cells_computed = computed;
    stats->cells_skipped = skipped;
    cudaEventElapsedTime(&stats->kernel_ms, c->ev0, c->ev1);
  }
  c->haveRecPDF = true;
  return MCX_OK;
}

extern "C" int mcx_opacity(mcx_ctx* c, const mcx_phase_opts* opts, mcx_phase_stats* stats) {
  if (!c) return MCX_ERR_INPUT;
  if (!c->loaded) return fail(c, MCX_ERR_STATE, "mcx_opacity: no model loaded");
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  if (!c->lgGas) {
    // dust-only grid: the grain contribution of every cell is added to the
    // opacity, which the reference never resets on such a grid
    // (source/iteration_mod.f90:194-246)
    CK(cudaEventRecord(c->ev0, c->stream), "event");
    CK(launchDustOpacity(c->dust->dev, c->ndust.p, c->tdust.p, c->opacity.p, c->scaOpac.p, c->stream), "dust opacity");
    CK(cudaEventRecord(c->ev1, c->stream), "event");
    CK(cudaStreamSynchronize(c->stream), "mcx_opacity");
    if (stats) {
      std::memset(stats, 0, sizeof(*stats));
      stats->cells_computed = c->nCells;
      cudaEventElapsedTime(&stats->kernel_ms, c->ev0, c->ev1);
    }
    c->haveOpacity = true;
    return MCX_OK;
  }
  const int it = opts ? opts->n_iterate_mc : 1;
  const size_t C1 = (size_t)c->nCells + 1;
  // the skip rule and the Gaunt cache are sequential host logic over four
  // per-cell arrays (source/iteration_mod.f90:131-149, source/ionization_mod.f90:171-175)
  std::vector<float> te(C1), ne(C1), teOld(C1), neOld(C1), gte(C1, 0.f);
  std::vector<uint8_t> mask(C1, 0);
  CK(cudaMemcpyAsync(te.data(), c->te.p, C1 * 4, cudaMemcpyDeviceToHost, c->stream), "d2h Te");
  CK(cudaMemcpyAsync(ne.data(), c->ne.p, C1 * 4, cudaMemcpyDeviceToHost, c->stream), "d2h Ne");
  CK(cudaMemcpyAsync(teOld.data(), c->teOld.p, C1 * 4, cudaMemcpyDeviceToHost, c->stream), "d2h TeOld");
  CK(cudaMemcpyAsync(neOld.data(), c->neOld.p, C1 * 4, cudaMemcpyDeviceToHost, c->stream), "d2h NeOld");
  CK(cudaStreamSynchronize(c->stream), "mcx_opacity");
  int64_t computed = 0, skipped = 0;
  // each grid in its processing order (i, j, k nested, k fastest) with its own Gaunt cache
  auto replay = [&](int nx, int ny, int nz, const int32_t* act, float& gauntTeOld) {
    for (int i = 1; i <= nx; ++i)
      for (int j = 1; j <= ny; ++j)
        for (int k = 1; k <= nz; ++k) {
          int cell = act[(size_t)(i - 1) + (size_t)nx * ((size_t)(j - 1) + (size_t)ny * (size_t)(k - 1))];
          if (cell <= 0) continue;
          bool skip = it > 1 && (std::fabs(te[cell] - teOld[cell]) / teOld[cell]) < 0.005f &&
                      (std::fabs(ne[cell] - neOld[cell]) / neOld[cell]) < 0.005f;
          if (skip) { ++skipped; continue; }
          mask[cell] = 1;
          ++computed;
          if (std::fabs(1.f - gauntTeOld / te[cell]) > 0.10f) gauntTeOld = te[cell];
          gte[cell] = gauntTeOld;
        }
  };
  if (c->nNeb > 0) {
    for (int b = 0; b < c->nNeb; ++b)
      replay(c->nebNx[b], c->nebNy[b], c->nebNz[b], c->nebActive[b].data(), c->nebGauntTeOld[b]);
    c->gauntTeOld = c->nebGauntTeOld[0];
  } else {
    replay(c->nx, c->ny, c->nz, c->activeHost.data(), c->gauntTeOld);
  }
  CK(cudaMemcpyAsync(c->computeMask.p, mask.data(), C1, cudaMemcpyHostToDevice, c->stream), "h2d mask");
  CK(cudaMemcpyAsync(c->gauntTe.p, gte.data(), C1 * 4, cudaMemcpyHostToDevice, c->stream), "h2d gauntTe");
  OpacityDev t{};
  t.nbins = c->nbins; t.nCells = c->nCells; t.nXsec = c->nXsec; t.lgCompton = c->lgCompton;
  t.nSlots = c->nSlots; t.bremsP0 = c->bremsP0;
  t.nu = c->nu.p; t.log10nu = c->log10nu.p; t.xsec = c->xsec.p; t.KNsigmaT = c->KNsigmaT.p;
  t.csrStart = c->csrStart.p; t.csrTerm = c->csrTerm.p;
  t.slotPlane = c->slotPlane.p; t.slotAbun = c->slotAbun.p; t.slotFFWeight = c->slotFFWeight.p;
  CK(cudaEventRecord(c->ev0, c->stream), "event");
  CK(launchOpacity(t, c->hden.p, c->te.p, c->ne.p, c->ionDen.p, c->gauntTe.p, c->computeMask.p, c->opacity.p, c->stream),
     "opacity kernel");
  CK(cudaEventRecord(c->ev1, c->stream), "event");
  CK(cudaStreamSynchronize(c->stream), "mcx_opacity");
  if (stats) {
    std::memset(stats, 0, sizeof(*stats));
    stats->cells_computed = computed;
    stats->cells_skipped = skipped;
    cudaEventElapsedTime(&stats->kernel_ms, c->ev0, c->ev1);
  }
  c->haveOpacity = true;
  return MCX_OK;
}

// ---------------------------------------------------------- transport phase
// counters of the launch just queued (events ev0/ev1 around it) into stats
static int transportFinish(mcx_ctx* c, mcx_transport_stats* stats, const char* who) {
  DevTransportCounters h{};
  CK(cudaMemcpyAsync(&h, c->counters.p, sizeof(h), cudaMemcpyDeviceToHost, c->stream), "d2h counters");
  CK(cudaStreamSynchronize(c->stream), who);
  if (stats) {
    std::memset(stats, 0, sizeof(*stats));
    stats->crossings = (int64_t)h.crossings;
    stats->interactions = (int64_t)h.interactions;
    stats->absorptions = (int64_t)h.absorptions;
    stats->scatterings = (int64_t)h.scatterings;
    stats->escaped = (int64_t)h.escaped;
    stats->line_escapes = (int64_t)h.lineEscapes;
    stats->trapped = (int64_t)h.trapped;
    stats->emissions = (int64_t)h.emissions;
    stats->q_phot = h.qPhot;
    stats->handed_off = (int64_t)std::min<unsigned long long>(h.handoff, c->parked.p ? kParkedCap : 0);
    cudaEventElapsedTime(&stats->kernel_ms, c->ev0, c->ev1);
  }
  if (h.errors)
    return fail(c, MCX_ERR_INTERNAL,
                std::string(who) + ": " + std::to_string(h.errors) + " packet(s) reached a state where the reference stops");
  return MCX_OK;
}

extern "C" int mcx_transport(mcx_ctx* c, const mcx_transport_opts* o, mcx_transport_stats* stats) {
  if (!c || !o) return fail(c, MCX_ERR_INPUT, "mcx_transport: null argument");
  if (!c->loaded) return fail(c, MCX_ERR_STATE, "mcx_transport: no model loaded");
  if (o->istar < 1 || o->istar > c->nStars)
    return fail(c, MCX_ERR_INPUT, "mcx_transport: source " + std::to_string(o->istar) + " of " +
                                      std::to_string(c->nStars));
  if (o->n_packets < 0) return fail(c, MCX_ERR_INPUT, "mcx_transport: negative packet count");
  if (!c->haveOpacity) return fail(c, MCX_ERR_STATE, "mcx_transport: no opacity (call mcx_opacity or mcx_put(MCX_ARR_OPACITY))");
  if (c->lgGas && !c->haveRecPDF) return fail(c, MCX_ERR_STATE, "mcx_transport: no re-emission CDF (recPDF)");
  if (c->lgDust && !c->lgGas && !c->haveDustPDF) return fail(c, MCX_ERR_STATE, "mcx_transport: no dust emission CDF");
  if (o->precision != MCX_PREC_FP32_GEOM && o->precision != MCX_PREC_FP64)
    return fail(c, MCX_ERR_INPUT, "mcx_transport: unknown precision");
  if (c->nNeb > 0) return fail(c, MCX_ERR_STATE, "mcx_transport: the context holds a batch (use mcx_transport_batched)");
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  const int64_t norm = o->n_photons_norm > 0 ? o->n_photons_norm : o->n_packets;
  // source istar: its luminosity, position and CDF row (source 1: the context's, which mcx_put may change)
  const int si = o->istar - 1;
  const float* star = c->stars.data() + 8 * si;
  const double deltaE = norm > 0 ? (double)(si == 0 ? c->lStar : star[0]) / (double)norm : 0.;
  if (o->zero_estimators) {
    CK(cudaMemsetAsync(c->jste.p, 0, c->jste.bytes(), c->stream), "memset Jste");
    CK(cudaMemsetAsync(c->jlo.p, 0, c->jlo.bytes(), c->stream), "memset Jste compensation");
    CK(cudaMemsetAsync(c->escaped.p, 0, c->escaped.bytes(), c->stream), "memset escaped");
    if (c->hEst.p) CK(cudaMemsetAsync(c->hEst.p, 0, c->hEst.bytes(), c->stream), "memset H");
  }
  CK(cudaMemsetAsync(c->counters.p, 0, sizeof(DevTransportCounters), c->stream), "memset counters");

  DevGrid g{};
  g.nx = c->nx; g.ny = c->ny; g.nz = c->nz; g.nCells = c->nCells; g.nbins = c->nbins;
  g.symmetric = c->symmetric; g.lgDust = c->lgDust; g.lgGas = c->lgGas; g.lgCompton = c->lgCompton;
  g.radPress = c->radPress; g.activeFull = c->activeFull; g.plane = c->plane;
  for (int d = 0; d < 3; ++d) {
    g.starIdx[d] = si == 0 ? c->starIdx[d] : (int)star[5 + d];
    g.starPos[d] = si == 0 ? c->starPos[d] : star[2 + d];
  }
  g.ionEdge1 = c->ionEdge1; g.rOut = c->rOut;
  g.xAxis = c->xAxis.p; g.yAxis = c->yAxis.p; g.zAxis = c->zAxis.p; g.active = c->active.p;
  g.nu = c->nu.p; g.srcCDF = c->srcCDF.p + (size_t)si * c->nbins; g.KNsigmaT = c->KNsigmaT.p;
  g.KNcdfT = c->KNcdfT.p;
  g.PcompT = c->PcompT.p; g.volD = c->volD.p; g.volF = c->volF.p;
  g.nAngle = c->nAngle; g.totPhi = c->totPhi;
  std::memcpy(g.viewPTheta, c->viewPTheta, sizeof g.viewPTheta);
  std::memcpy(g.viewPPhi, c->viewPPhi, sizeof g.viewPPhi);
  DevTransportIn in{};
  in.opacity = c->opacity.p; in.scaOpac = c->scaOpac.p; in.recCDFT = c->recCDFT.p; in.dustCDFT = c->dustCDFT.p;
  in.totalLines = c->totalLines.p; in.ne = c->ne.p;
  DevTransportOut out{};
  out.jste = c->jste.p; out.jlo = c->jlo.p; out.escaped = c->escaped.p; out.hEst = c->hEst.p;

  TransportLaunch L{};
  L.emitBatch = o->emit_batch > 32 ? 32 : o->emit_batch;
  L.threads = o->block_size > 0 ? o->block_size : 256;
  if (L.threads % 32 != 0 || L.threads > 256) return fail(c, MCX_ERR_INPUT, "mcx_transport: block_size must be a multiple of 32 up to 256");
  L.smem = (size_t)(c->nx + c->ny + c->nz + 2 * c->nbins) * sizeof(float);
  int perSM = 0;
  CK(transportOccupancy(o->precision == MCX_PREC_FP64, L.threads, L.smem, &perSM, c->plane != 0), "occupancy");
  if (perSM < 1) perSM = 1;
  int mult = o->grid_mult > 0 ? std::min(o->grid_mult, perSM) : perSM;
  L.blocks = c->numSMs * mult;
  L.parked = c->parked.p;
  L.parkedCap = c->parked.p ? kParkedCap : 0;
  L.handoffAt = o->handoff_emissions < 0 ? 0 : (o->handoff_emissions > 0 ? o->handoff_emissions : kHandoffAt);
  L.numSMs = c->numSMs;
  const unsigned long long n = (unsigned long long)o->n_packets;
  if (n > 0) {
    const unsigned long long maxBlocks = (n + L.threads - 1) / L.threads;
    if ((unsigned long long)L.blocks > maxBlocks) L.blocks = (int)maxBlocks;
  }
  CK(cudaEventRecord(c->ev0, c->stream), "event");
  if (n > 0) {
    cudaError_t e = (o->precision == MCX_PREC_FP64)
                        ? launchTransportF64(g, in, out, c->counters.p, o->seed, o->counter_base, n, deltaE, L, c->stream)
                        : launchTransportF32(g, in, out, c->counters.p, o->seed, o->counter_base, n, deltaE, L, c->stream);
    if (e != cudaSuccess) return cudaFail(c, e, "transport kernel");
  }
  CK(cudaEventRecord(c->ev1, c->stream), "event");
  if (n > 0) CK(foldJ(c), "fold J compensation");
  return transportFinish(c, stats, "mcx_transport");
}

// transport of every nebula of a batch in one launch
extern "C" int mcx_transport_batched(mcx_ctx* c, const mcx_transport_opts* o, const mcx_batch_packets* pk,
                                     mcx_transport_stats* stats) {
  if (!c || !o || !pk || !pk->n_packets || !pk->seed || !pk->counter_base)
    return fail(c, MCX_ERR_INPUT, "mcx_transport_batched: null argument");
  if (!c->loaded) return fail(c, MCX_ERR_STATE, "mcx_transport_batched: no model loaded");
  if (c->nNeb <= 0) return fail(c, MCX_ERR_STATE, "mcx_transport_batched: the context holds no batch (mcx_load_batched)");
  if (o->istar != 1) return fail(c, MCX_ERR_INPUT, "mcx_transport_batched: only source 1 is supported");
  if (!c->haveOpacity || !c->haveRecPDF)
    return fail(c, MCX_ERR_STATE, "mcx_transport_batched: run mcx_opacity and mcx_emission first");
  if (o->precision != MCX_PREC_FP32_GEOM && o->precision != MCX_PREC_FP64)
    return fail(c, MCX_ERR_INPUT, "mcx_transport_batched: unknown precision");
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  const int n = c->nNeb;
  std::vector<unsigned long long> begin(n + 1, 0);
  std::vector<NebulaDesc> desc = c->nebDesc;
  for (int b = 0; b < n; ++b) {
    if (pk->n_packets[b] < 0) return fail(c, MCX_ERR_INPUT, "mcx_transport_batched: negative packet count");
    const int64_t norm = (pk->n_photons_norm && pk->n_photons_norm[b] > 0) ? pk->n_photons_norm[b] : pk->n_packets[b];
    desc[b].deltaE = norm > 0 ? (double)c->nebLStar[b] / (double)norm : 0.;
    desc[b].seed = pk->seed[b];
    desc[b].counterBase = pk->counter_base[b];
    begin[b + 1] = begin[b] + (unsigned long long)pk->n_packets[b];
  }
  if (o->zero_estimators) {
    CK(cudaMemsetAsync(c->jste.p, 0, c->jste.bytes(), c->stream), "memset Jste");
    CK(cudaMemsetAsync(c->jlo.p, 0, c->jlo.bytes(), c->stream), "memset Jste compensation");
    CK(cudaMemsetAsync(c->escaped.p, 0, c->escaped.bytes(), c->stream), "memset escaped");
  }
  CK(cudaMemsetAsync(c->counters.p, 0, sizeof(DevTransportCounters), c->stream), "memset counters");
  CK(cudaMemcpyAsync(c->nebDescDev.p, desc.data(), sizeof(NebulaDesc) * n, cudaMemcpyHostToDevice, c->stream),
     "h2d batch descriptors");
  CK(cudaMemcpyAsync(c->nebPktBegin.p, begin.data(), sizeof(unsigned long long) * (n + 1), cudaMemcpyHostToDevice,
                     c->stream), "h2d batch packet offsets");
  DevGrid g{};
  g.nCells = c->nCells; g.nbins = c->nbins;
  g.lgDust = 0; g.lgGas = 1; g.lgCompton = c->lgCompton; g.radPress = 0;
  g.ionEdge1 = c->ionEdge1;
  g.nu = c->nu.p; g.KNsigmaT = c->KNsigmaT.p; g.KNcdfT = c->KNcdfT.p; g.PcompT = c->PcompT.p;
  g.volD = c->volD.p; g.volF = c->volF.p;
  DevTransportIn in{};
  in.opacity = c->opacity.p; in.recCDFT = c->recCDFT.p; in.totalLines = c->totalLines.p; in.ne = c->ne.p;
  DevTransportOut out{};
  out.jste = c->jste.p; out.jlo = c->jlo.p; out.escaped = c->escaped.p;
  TransportLaunch L{};
  L.emitBatch = o->emit_batch > 32 ? 32 : o->emit_batch;
  L.threads = o->block_size > 0 ? o->block_size : 256;
  if (L.threads % 32 != 0 || L.threads > 256)
    return fail(c, MCX_ERR_INPUT, "mcx_transport_batched: block_size must be a multiple of 32 up to 256");
  L.smem = (size_t)c->nbins * sizeof(float);
  const bool fp64 = o->precision == MCX_PREC_FP64;
  int perSM = 0;
  CK(fp64 ? transportOccupancyBatchedF64(L.threads, L.smem, &perSM) : transportOccupancyBatchedF32(L.threads, L.smem, &perSM),
     "occupancy");
  if (perSM < 1) perSM = 1;
  L.blocks = c->numSMs * (o->grid_mult > 0 ? std::min(o->grid_mult, perSM) : perSM);
  const unsigned long long total = begin[n];
  if (total > 0) {
    const unsigned long long maxBlocks = (total + L.threads - 1) / L.threads;
    if ((unsigned long long)L.blocks > maxBlocks) L.blocks = (int)maxBlocks;
  }
  CK(cudaMemsetAsync(c->nebStamps.p, 0, c->nebStamps.bytes(), c->stream), "memset batch timers");
  CK(cudaEventRecord(c->ev0, c->stream), "event");
  if (total > 0) {
    cudaError_t e = fp64 ? launchTransportBatchedF64(g, in, out, c->counters.p, c->nebDescDev.p, c->nebPktBegin.p, n,
                                                     c->nebAxes.p, c->nebActiveDev.p, c->nebCdf.p, L,
                                                     c->nebStamps.p, c->stream)
                         : launchTransportBatchedF32(g, in, out, c->counters.p, c->nebDescDev.p, c->nebPktBegin.p, n,
                                                     c->nebAxes.p, c->nebActiveDev.p, c->nebCdf.p, L,
                                                     c->nebStamps.p, c->stream);
    if (e != cudaSuccess) return cudaFail(c, e, "batched transport kernel");
  }
  CK(cudaEventRecord(c->ev1, c->stream), "event");
  if (total > 0) CK(foldJ(c), "fold J compensation");
  return transportFinish(c, stats, "mcx_transport_batched");
}

extern "C" int mcx_batch_transport_ms(mcx_ctx* c, double* ms, int32_t n) {
  if (!c || !ms) return fail(c, MCX_ERR_INPUT, "mcx_batch_transport_ms: null argument");
  if (!c->loaded || c->nNeb <= 0) return fail(c, MCX_ERR_STATE, "mcx_batch_transport_ms: the context holds no batch");
  if (n != c->nNeb) return fail(c, MCX_ERR_INPUT, "mcx_batch_transport_ms: n must be the batch size");
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  std::vector<unsigned long long> t((size_t)n + 1);
  CK(cudaMemcpyAsync(t.data(), c->nebStamps.p, t.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                     c->stream), "d2h batch timers");
  CK(cudaStreamSynchronize(c->stream), "mcx_batch_transport_ms");
  for (int b = 0; b < n; ++b)
    ms[b] = (t[b + 1] > t[0]) ? (double)(t[b + 1] - t[0]) * 1e-6 : 0.;
  return MCX_OK;
}

extern "C" int mcx_normalize_j(mcx_ctx* c) {
  if (!c) return MCX_ERR_INPUT;
  if (!c->loaded) return fail(c, MCX_ERR_STATE, "mcx_normalize_j: no model loaded");
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  if (c->nNeb > 0) {
    const size_t C1 = (size_t)c->nCells + 1;
    scaleJCellKernel<<<(unsigned)((c->jste.n + 255) / 256), 256, 0, c->stream>>>(c->jste.p, c->jste.n, C1, 1.e-9,
                                                                               c->jDiv.p);
    CK(cudaGetLastError(), "scale J");
    scaleJCellKernel<<<(unsigned)((c->escaped.n + 255) / 256), 256, 0, c->stream>>>(c->escaped.p, c->escaped.n, C1, 1.,
                                                                                  c->jDiv.p);
    CK(cudaGetLastError(), "scale escaped");
    CK(cudaStreamSynchronize(c->stream), "mcx_normalize_j");
    return MCX_OK;
  }
  const double div = c->symmetric ? 8. : 1.;
  scaleJKernel<<<(unsigned)((c->jste.n + 1023) / 1024), 256, 0, c->stream>>>(c->jste.p, c->jste.n, 1.e-9, div);
  CK(cudaGetLastError(), "scale J");
  if (div != 1.) {
    scaleJKernel<<<(unsigned)((c->escaped.n + 1023) / 1024), 256, 0, c->stream>>>(c->escaped.p, c->escaped.n, 1., div);
    CK(cudaGetLastError(), "scale escaped");
  }
  CK(cudaStreamSynchronize(c->stream), "mcx_normalize_j");
  return MCX_OK;
}

extern "C" int mcx_balance(mcx_ctx* c, const mcx_balance_opts* opts, mcx_balance_stats* stats) {
  if (!c) return MCX_ERR_INPUT;
  if (!c->loaded) return fail(c, MCX_ERR_STATE, "mcx_balance: no model loaded");
  if (!c->lgGas && c->dust) {
    // dust-only grid: getDustT for every cell hit by a photon (source/update_mod.f90:234-265, :3346-3453)
    CK(cudaSetDevice(c->device), "cudaSetDevice");
    CK(cudaEventRecord(c->ev0, c->stream), "event");
    CK(launchDustT(c->dust->dev, c->jste.p, c->tdust.p, c->lgConverged.p, c->lgBlack.p, c->stream), "grain balance");
    CK(cudaEventRecord(c->ev1, c->stream), "event");
    DustCounters h{};
    CK(cudaMemcpyAsync(&h, c->dust->dev.counters, sizeof(h), cudaMemcpyDeviceToHost, c->stream), "d2h counters");
    CK(cudaStreamSynchronize(c->stream), "mcx_balance");
    if (stats) {
      std::memset(stats, 0, sizeof(*stats));
      stats->cells_updated = (int64_t)h.updated;
      stats->no_hit = (int64_t)h.noHit;
      stats->converged = (int64_t)h.converged;
      cudaEventElapsedTime(&stats->kernel_ms, c->ev0, c->ev1);
    }
    return MCX_OK;
  }
  if (!c->lgGas || !c->balance) return fail(c, MCX_ERR_STATE, "mcx_balance: the grid holds no gas");
  if (opts && opts->precision != MCX_BAL_FP64 && opts->precision != MCX_BAL_MIXED)
    return fail(c, MCX_ERR_INPUT, "mcx_balance: unknown precision");
  const int prec = (opts && opts->precision == MCX_BAL_MIXED) ? kBalMixed : kBalFp64;
  const int converge = opts && opts->converge ? 1 : 0;
  const int fixTe = opts && opts->fix_te ? 1 : 0;
  if (fixTe && !converge) return fail(c, MCX_ERR_INPUT, "mcx_balance: fix_te needs converge = 1");
  const int roundCap = converge ? kMaxRounds : kRefRounds;
  const int rounds = (opts && opts->max_rounds > 0) ? opts->max_rounds : roundCap;
  if (rounds > roundCap)
    return fail(c, MCX_ERR_INPUT, "mcx_balance: max_rounds above " + std::to_string(roundCap) +
                                      (converge ? " (tight convergence)" : " (maxIterateT)"));
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  const size_t C1 = (size_t)c->nCells + 1;
  CK(cudaEventRecord(c->ev0, c->stream), "event");
  // iterateMC saves the state the skip rule compares against (source/iteration_mod.f90:1136-1139)
  CK(cudaMemcpyAsync(c->teOld.p, c->te.p, C1 * sizeof(float), cudaMemcpyDeviceToDevice, c->stream), "TeOld");
  CK(cudaMemcpyAsync(c->neOld.p, c->ne.p, C1 * sizeof(float), cudaMemcpyDeviceToDevice, c->stream), "NeOld");
  BalanceGrid g{c->jste.p, c->hden.p, c->te.p, c->ne.p, c->ionDen.p, c->lgConverged.p, c->lgBlack.p, c->nIterT.p};
  CK(launchBalance(*c->balance, g, rounds, prec, c->stream, opts && opts->atom_solves ? 1 : 0, converge, fixTe),
     "balance kernels");
  CK(cudaEventRecord(c->ev1, c->stream), "event");
  BalanceCounters h{};
  CK(cudaMemcpyAsync(&h, c->balance->dev.counters, sizeof(h), cudaMemcpyDeviceToHost, c->stream), "d2h counters");
  CK(cudaStreamSynchronize(c->stream), "mcx_balance");
  if (stats) {
    std::memset(stats, 0, sizeof(*stats));
    stats->cells_updated = (int64_t)h.updated;
    stats->no_hit = (int64_t)h.noHit;
    stats->no_ion_bal = (int64_t)h.noIonBal;
    stats->no_te_bal = (int64_t)h.noTeBal;
    stats->converged = (int64_t)h.converged;
    stats->max_iter_t = (int32_t)h.maxIterT;
    cudaEventElapsedTime(&stats->kernel_ms, c->ev0, c->ev1);
  }
  return MCX_OK;
}

static int iterateImpl(mcx_ctx* c, const mcx_iterate_opts* o, const mcx_batch_packets* pk, mcx_iterate_stats* stats);

extern "C" int mcx_iterate(mcx_ctx* c, const mcx_iterate_opts* o, mcx_iterate_stats* stats) {
  if (!c || !o) return fail(c, MCX_ERR_INPUT, "mcx_iterate: null argument");
  if (!c->loaded) return fail(c, MCX_ERR_STATE, "mcx_iterate: no model loaded");
  if (o->n_packets <= 0) return fail(c, MCX_ERR_INPUT, "mcx_iterate: n_packets must be positive");
  if (c->nNeb > 0) return fail(c, MCX_ERR_STATE, "mcx_iterate: the context holds a batch (use mcx_iterate_batched)");
  return iterateImpl(c, o, nullptr, stats);
}

extern "C" int mcx_iterate_batched(mcx_ctx* c, const mcx_iterate_opts* o, const mcx_batch_packets* pk,
                                   mcx_iterate_stats* stats) {
  if (!c || !o || !pk) return fail(c, MCX_ERR_INPUT, "mcx_iterate_batched: null argument");
  if (!c->loaded) return fail(c, MCX_ERR_STATE, "mcx_iterate_batched: no model loaded");
  if (c->nNeb <= 0) return fail(c, MCX_ERR_STATE, "mcx_iterate_batched: the context holds no batch");
  return iterateImpl(c, o, pk, stats);
}

static int iterateImpl(mcx_ctx* c, const mcx_iterate_opts* o, const mcx_batch_packets* pk, mcx_iterate_stats* stats) {
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  mcx_iterate_stats st{};
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  CK(cudaEventCreate(&t0), "event");
  CK(cudaEventCreate(&t1), "event");
  CK(cudaEventRecord(t0, c->stream), "event");
  mcx_phase_opts po{};
  po.n_iterate_mc = o->n_iterate_mc;
  int rc = mcx_opacity(c, &po, &st.opacity);
  if (rc == MCX_OK) {
    po.precision = o->emission_precision;
    rc = mcx_emission(c, &po, &st.emission);
  }
  if (rc == MCX_OK) {
    mcx_transport_opts to{};
    to.istar = 1;
    to.precision = o->transport_precision;
    to.n_packets = o->n_packets;
    to.seed = o->seed;
    to.counter_base = o->counter_base;
    to.n_photons_norm = o->n_packets;
    to.zero_estimators = 1;
    to.block_size = o->transport_block_size;
    to.grid_mult = o->transport_grid_mult;
    to.emit_batch = o->transport_emit_batch;
    if (pk) {
      rc = mcx_transport_batched(c, &to, pk, &st.transport);
    } else {
      // the sources one after another (source/iteration_mod.f90:729-753): nPhotons / nStars packets each,
      // on consecutive counter ranges; J adds up, the escape tallies keep the last source's (the reference
      // zeroes escapedPackets before each source)
      const int64_t per = c->nStars > 1 ? o->n_packets / c->nStars : o->n_packets;
      mcx_transport_stats& ts = st.transport;
      for (int i = 1; i <= c->nStars && rc == MCX_OK; ++i) {
        to.istar = i;
        to.n_packets = per;
        to.n_photons_norm = per;
        to.counter_base = o->counter_base + (uint64_t)(i - 1) * (uint64_t)per;
        to.zero_estimators = i == 1 ? 1 : 0;
        if (i > 1) CK(cudaMemsetAsync(c->escaped.p, 0, c->escaped.bytes(), c->stream), "memset escaped");
        mcx_transport_stats one{};
        rc = mcx_transport(c, &to, &one);
        if (rc != MCX_OK) break;
        if (i == 1) { ts = one; continue; }
        ts.crossings += one.crossings; ts.interactions += one.interactions; ts.absorptions += one.absorptions;
        ts.scatterings += one.scatterings; ts.escaped += one.escaped; ts.line_escapes += one.line_escapes;
        ts.trapped += one.trapped; ts.emissions += one.emissions; ts.q_phot += one.q_phot;
        ts.kernel_ms += one.kernel_ms; ts.handed_off += one.handed_off;
      }
    }
  }
  if (rc == MCX_OK) rc = mcx_normalize_j(c);
  if (rc == MCX_OK) {
    mcx_balance_opts bo{};
    bo.precision = o->balance_precision;
    rc = mcx_balance(c, &bo, &st.balance);
  }
  if (rc == MCX_OK) {
    cudaEventRecord(t1, c->stream);
    cudaEventSynchronize(t1);
    cudaEventElapsedTime(&st.total_ms, t0, t1);
    if (stats) *stats = st;
  }
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  return rc;
}

static int lineLuminosities(mcx_ctx* c, int cellBase, int nRange, bool symmetric, mcx_lines* out);

extern "C" int mcx_line_luminosities(mcx_ctx* c, mcx_lines* out) {
  if (!c || !out) return fail(c, MCX_ERR_INPUT, "mcx_line_luminosities: null argument");
  if (!c->loaded) return fail(c, MCX_ERR_STATE, "mcx_line_luminosities: no model loaded");
  if (c->nNeb > 0)
    return fail(c, MCX_ERR_STATE, "mcx_line_luminosities: the context holds a batch (use mcx_line_luminosities_nebula)");
  return lineLuminosities(c, 0, c->nCells, c->symmetric, out);
}

extern "C" int mcx_line_luminosities_nebula(mcx_ctx* c, int32_t nebula, mcx_lines* out) {
  if (!c || !out) return fail(c, MCX_ERR_INPUT, "mcx_line_luminosities_nebula: null argument");
  if (!c->loaded) return fail(c, MCX_ERR_STATE, "mcx_line_luminosities_nebula: no model loaded");
  if (c->nNeb <= 0) return fail(c, MCX_ERR_STATE, "mcx_line_luminosities_nebula: the context holds no batch");
  if (nebula < 0 || nebula >= c->nNeb) return fail(c, MCX_ERR_INPUT, "mcx_line_luminosities_nebula: no such nebula");
  return lineLuminosities(c, c->nebCellOff[nebula], c->nebCellOff[nebula + 1] - c->nebCellOff[nebula],
                          c->nebSym[nebula] != 0, out);
}

static int lineLuminosities(mcx_ctx* c, int cellBase, int nRange, bool symmetric, mcx_lines* out) {
  if (!c->lgGas || !c->emission || !c->balance)
    return fail(c, MCX_ERR_STATE, "mcx_line_luminosities: the grid holds no gas");
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  const int S = c->nstages, C = c->nCells;
  // entry layout of the partial sums (k_lines.cuh)
  LineSumArgs a{};
  a.te = c->te.p; a.ne = c->ne.p; a.ionDen = c->ionDen.p; a.hden = c->hden.p;
  a.vol = c->volD.p; a.black = c->lgBlack.p;
  a.nCells = C;
  a.cellBase = cellBase;
  a.nRange = nRange;
  a.nGroups = (nRange + 31) / 32;
  int n = 1;
  a.hydroBase = n;
  for (int iz = 1; iz <= 30; ++iz)
    if (c->xrefAll[iz - 1] > 0 && S > iz) a.hydroIz[a.nHydro++] = iz;
  n += kHydroLinesPerElem * a.nHydro;
  a.heiBase = -1;
  if (c->xrefAll[1] > 0) { a.heiBase = n; n += 34; }
  a.ionBase = n;
  for (int z = 1; z <= 30; ++z)
    if (c->xrefAll[z - 1] > 0) {
      a.ionElem[a.nIonElem++] = z;
      n += 2 * std::min(z + 1, S);
    }
  std::vector<int32_t> forbBase(c->lineAtoms.size());
  for (size_t k = 0; k < c->lineAtoms.size(); ++k) { forbBase[k] = n; n += c->lineAtoms[k].nLev; }
  a.nEntries = n;
  const size_t partialCount = (size_t)a.nGroups * (size_t)n;
  if (c->linePartial.n < partialCount) CK(c->linePartial.alloc(partialCount), "alloc line sums");
  if (c->lineSums.n < (size_t)n) CK(c->lineSums.alloc(n), "alloc line sums");
  if (!forbBase.empty()) CK(upload(c->lineForbBase, forbBase), "upload line layout");
  a.partial = c->linePartial.p;
  a.forbBase = c->lineForbBase.p;

  CK(cudaEventRecord(c->ev0, c->stream), "event");
  CK(launchGasLineSums(c->emission->dev, a, c->stream), "line sums");
  if (!forbBase.empty()) CK(launchForbLevelSums(*c->balance, a, c->stream), "forbidden-line sums");
  CK(launchLineSumReduce(a.partial, a.nGroups, n, c->lineSums.p, c->stream), "line sum reduce");
  CK(cudaEventRecord(c->ev1, c->stream), "event");
  std::vector<double> sum(n);
  std::vector<int32_t> black((size_t)C + 1);
  CK(cudaMemcpyAsync(sum.data(), c->lineSums.p, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream), "d2h sums");
  CK(cudaMemcpyAsync(black.data(), c->lgBlack.p, black.size() * sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream),
     "d2h lgBlack");
  CK(cudaStreamSynchronize(c->stream), "mcx_line_luminosities");
  cudaEventElapsedTime(&out->kernel_ms, c->ev0, c->ev1);

  // normalisation and units (source/output_mod.f90:684-805)
  int nUsed = 0;
  for (int cell = cellBase + 1; cell <= cellBase + nRange; ++cell) nUsed += black[cell] < 1 ? 1 : 0;
  out->n_cells = nUsed;
  double hb = sum[0];
  const bool rel = hb > 0.;
  out->relative = rel ? 1 : 0;
  const double div = rel ? hb : 1.;
  if (out->hydro_vol) {
    std::fill(out->hydro_vol, out->hydro_vol + 30 * 14 * 8, 0.);
    for (int k = 0; k < a.nHydro; ++k) {
      const int iz = a.hydroIz[k];
      int l = 0;
      for (int iup = 2; iup <= 15; ++iup)
        for (int ilow = 1; ilow <= std::min(8, iup - 1); ++ilow, ++l)
          out->hydro_vol[(iz - 1) + 30 * (iup - 2) + 420 * (ilow - 1)] =
              sum[a.hydroBase + kHydroLinesPerElem * k + l] / div;
    }
  }
  if (out->hei_vol)
    for (int l = 0; l < 34; ++l) out->hei_vol[l] = a.heiBase >= 0 ? sum[a.heiBase + l] / div : 0.;
  const size_t forbN = (size_t)30 * S * 30 * 30;
  if (out->forb_vol) std::fill(out->forb_vol, out->forb_vol + forbN, 0.);
  if (out->wav) std::fill(out->wav, out->wav + forbN, 0.);
  for (size_t k = 0; k < c->lineAtoms.size(); ++k) {
    const auto& la = c->lineAtoms[k];
    if (la.ion > S) continue;
    const int nl = la.nLev;
    for (int i = 1; i <= nl; ++i)
      for (int j = 1; j <= nl; ++j) {
        const size_t at = (size_t)(la.elem - 1) + 30 * (size_t)(la.ion - 1) + (size_t)30 * S * (i - 1) +
                          (size_t)900 * S * (j - 1);
        const double f = la.fac[(size_t)(i - 1) * nl + (j - 1)];
        if (out->forb_vol && f != 0.) out->forb_vol[at] = f * sum[forbBase[k] + j - 1] / div;
        if (out->wav) out->wav[at] = la.wav[(size_t)(i - 1) * nl + (j - 1)];
      }
  }
  if (out->te_vol || out->ion_vol) {
    if (out->te_vol) std::fill(out->te_vol, out->te_vol + (size_t)30 * S, 0.);
    if (out->ion_vol) std::fill(out->ion_vol, out->ion_vol + (size_t)30 * S, 0.);
    int p = 0;
    for (int q = 0; q < a.nIonElem; ++q) {
      const int elem = a.ionElem[q], top = std::min(elem + 1, S);
      double denIon = 0.;
      for (int ion = 1; ion <= top; ++ion) denIon = denIon + sum[a.ionBase + 2 * (p + ion - 1) + 1];
      for (int ion = 1; ion <= top; ++ion, ++p) {
        const double num = sum[a.ionBase + 2 * p], den = sum[a.ionBase + 2 * p + 1];
        const size_t at = (size_t)(elem - 1) + 30 * (size_t)(ion - 1);
        if (out->te_vol) out->te_vol[at] = den <= 0. ? 0. : num / den;
        if (out->ion_vol) out->ion_vol[at] = denIon <= 0. ? 0. : den / denIon;
      }
    }
  }
  hb = hb * (double)1.e-16f;
  if (symmetric) hb = 8. * hb;
  out->hbeta_vol = hb;
  return MCX_OK;
}

// ------------------------------------------------ frozen-field sensitivities
namespace {

// the grid state a balance reads and writes
struct StateCopy {
  DBuf<float> te, ne, teOld, neOld, ionDen;
  DBuf<int32_t> conv, black, nIterT;
};

int copyState(mcx_ctx* c, StateCopy& d, bool save) {
  struct F { DBuf<float>* snap; DBuf<float>* live; } fs[] = {
      {&d.te, &c->te}, {&d.ne, &c->ne}, {&d.teOld, &c->teOld}, {&d.neOld, &c->neOld}, {&d.ionDen, &c->ionDen}};
  struct I { DBuf<int32_t>* snap; DBuf<int32_t>* live; } is[] = {
      {&d.conv, &c->lgConverged}, {&d.black, &c->lgBlack}, {&d.nIterT, &c->nIterT}};
  for (auto& f : fs) {
    if (save && f.snap->n != f.live->n) CK(f.snap->alloc(f.live->n), "alloc state copy");
    CK(cudaMemcpyAsync(save ? f.snap->p : f.live->p, save ? f.live->p : f.snap->p, f.live->bytes(),
                       cudaMemcpyDeviceToDevice, c->stream), "state copy");
  }
  for (auto& f : is) {
    if (save && f.snap->n != f.live->n) CK(f.snap->alloc(f.live->n), "alloc state copy");
    CK(cudaMemcpyAsync(save ? f.snap->p : f.live->p, save ? f.live->p : f.snap->p, f.live->bytes(),
                       cudaMemcpyDeviceToDevice, c->stream), "state copy");
  }
  return MCX_OK;
}

// The checks shared by the derivative calls and the requested lines as (atom slot, lower, upper).
int lineRequests(mcx_ctx* c, const mcx_sens_opts* o, bool haveOut, const std::string& who, std::vector<int32_t>& req) {
  if (!c || !o || !haveOut || (o->n_lines > 0 && !o->lines) || (o->n_abun > 0 && !o->abun_z))
    return fail(c, MCX_ERR_INPUT, who + ": null argument");
  if (!c->loaded) return fail(c, MCX_ERR_STATE, who + ": no model loaded");
  if (!c->lgGas || !c->balance) return fail(c, MCX_ERR_STATE, who + ": the grid holds no gas");
  if (c->nNeb > 0) return fail(c, MCX_ERR_STATE, who + ": not for a batch");
  if (o->n_lines < 1 || o->n_abun < 0) return fail(c, MCX_ERR_INPUT, who + ": no lines");
  const int nL = o->n_lines;
  req.assign(3 * (size_t)nL, 0);
  for (int k = 0; k < nL; ++k) {
    const mcx_line_ref& l = o->lines[k];
    int slot = -1;
    for (size_t a = 0; a < c->lineAtoms.size(); ++a)
      if (c->lineAtoms[a].elem == l.elem && c->lineAtoms[a].ion == l.ion) slot = (int)a;
    if (slot < 0) return fail(c, MCX_ERR_INPUT, who + ": no multi-level data for line " + std::to_string(k));
    const int n = c->lineAtoms[slot].nLev;
    if (l.lower < 1 || l.upper <= l.lower || l.upper > n ||
        c->lineAtoms[slot].fac[(size_t)(l.lower - 1) * n + (l.upper - 1)] == 0.)
      return fail(c, MCX_ERR_INPUT, who + ": line " + std::to_string(k) + " has no transition");
    req[3 * k] = slot; req[3 * k + 1] = l.lower; req[3 * k + 2] = l.upper;
  }
  for (int q = 0; q < o->n_abun; ++q)
    if (o->abun_z[q] < 1 || o->abun_z[q] > 30 || c->xrefAll[o->abun_z[q] - 1] <= 0)
      return fail(c, MCX_ERR_INPUT, who + ": element " + std::to_string(o->abun_z[q]) + " is not on");
  return MCX_OK;
}

}  // namespace

extern "C" int mcx_line_sensitivities(mcx_ctx* c, const mcx_sens_opts* o, mcx_sens_out* out) {
  std::vector<int32_t> req;
  if (int rc = lineRequests(c, o, out && out->L, "mcx_line_sensitivities", req)) return rc;
  const double h = o->h != 0. ? o->h : 1.e-3;
  const int nL = o->n_lines, C = c->nCells;
  const size_t C1 = (size_t)C + 1;
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  DBuf<int32_t> dReq;
  DBuf<double> cellL;
  CK(upload(dReq, req), "upload line requests");
  CK(cellL.alloc((size_t)nL * C1), "alloc line cells");
  LineCellArgs la{};
  la.te = c->te.p; la.ne = c->ne.p; la.ionDen = c->ionDen.p; la.hden = c->hden.p; la.vol = c->volD.p;
  la.black = c->lgBlack.p; la.req = dReq.p; la.out = cellL.p; la.nReq = nL;
  mcx_balance_opts bo{};
  bo.precision = o->precision;
  const bool tight = !o->reference_stopping;
  bo.converge = tight ? 1 : 0;
  std::vector<double> base((size_t)nL * C1), pert((size_t)nL * C1);
  std::vector<float> teBase(C1), tePert(C1);
  std::vector<int32_t> nitBase(C1), nitPert(C1);
  std::vector<int8_t> sideBase(C1), sidePert(C1);
  auto balanceAndLines = [&](std::vector<double>& dst, std::vector<float>& te, std::vector<int32_t>& nit,
                             std::vector<int8_t>& side) -> int {
    int rc = mcx_balance(c, &bo, nullptr);
    if (rc != MCX_OK) return rc;
    CK(launchLineCellLuminosities(*c->balance, la, c->stream), "line cells");
    CK(cudaMemcpyAsync(dst.data(), cellL.p, dst.size() * sizeof(double), cudaMemcpyDeviceToHost, c->stream), "d2h");
    CK(cudaMemcpyAsync(te.data(), c->te.p, C1 * sizeof(float), cudaMemcpyDeviceToHost, c->stream), "d2h Te");
    CK(cudaMemcpyAsync(nit.data(), c->nIterT.p, C1 * sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream), "d2h");
    CK(cudaMemcpyAsync(side.data(), c->balance->dev.side, C1, cudaMemcpyDeviceToHost, c->stream), "d2h");
    CK(cudaStreamSynchronize(c->stream), "mcx_line_sensitivities");
    return MCX_OK;
  };
  // tight mode: a cell left out of the differences did not converge in one of the two balances,
  // or ended one of them on a discontinuity of heating - cooling (its bracket closed on a jump),
  // or moved its Te by more than a smooth response to a step h can (it crossed a discontinuity)
  const double jump = std::max(5. * std::fabs(h), 1e-4);
  auto branched = [&](size_t cell) {
    return tight && (nitBase[cell] >= kMaxRounds || nitPert[cell] >= kMaxRounds || sideBase[cell] == 3 ||
                     sidePert[cell] == 3 ||
                     std::fabs((double)tePert[cell] - (double)teBase[cell]) > jump * (double)teBase[cell]);
  };
  // perturbed balances: continued from the converged unperturbed state (tight mode, whose first
  // steps are small), or from the state before the call (iterateT's own stopping rules)
  auto startPerturbed = [&](StateCopy& s0, StateCopy& s1) { return copyState(c, tight ? s1 : s0, false); };
  StateCopy s0, s1;
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  CK(cudaEventCreate(&t0), "event");
  CK(cudaEventCreate(&t1), "event");
  CK(cudaEventRecord(t0, c->stream), "event");
  out->branch_cells_hden = 0;
  out->branch_cells_abun = 0;
  int rc = copyState(c, s0, true);
  if (rc == MCX_OK) rc = balanceAndLines(base, teBase, nitBase, sideBase);
  if (rc == MCX_OK) rc = copyState(c, s1, true);
  if (rc == MCX_OK)
    for (int k = 0; k < nL; ++k) {
      double t = 0.;
      for (size_t cell = 1; cell < C1; ++cell) t += base[(size_t)k * C1 + cell];
      out->L[k] = t;
    }
  // every density at once: each cell answers for itself under the fixed J
  if (rc == MCX_OK && out->dL_dhden) {
    std::vector<float> hd(C1), hdp(C1);
    CK(cudaMemcpy(hd.data(), c->hden.p, C1 * sizeof(float), cudaMemcpyDeviceToHost), "d2h Hden");
    for (size_t cell = 0; cell < C1; ++cell) hdp[cell] = (float)((double)hd[cell] * (1. + h));
    CK(cudaMemcpy(c->hden.p, hdp.data(), C1 * sizeof(float), cudaMemcpyHostToDevice), "h2d Hden");
    rc = startPerturbed(s0, s1);
    if (rc == MCX_OK) rc = balanceAndLines(pert, tePert, nitPert, sidePert);
    CK(cudaMemcpy(c->hden.p, hd.data(), C1 * sizeof(float), cudaMemcpyHostToDevice), "h2d Hden");
    if (rc == MCX_OK)
      for (size_t cell = 0; cell < C1; ++cell) {
        const double dh = (double)hdp[cell] - (double)hd[cell];
        const bool skip = cell == 0 || dh == 0. || branched(cell);
        if (cell > 0 && branched(cell)) ++out->branch_cells_hden;
        for (int k = 0; k < nL; ++k)
          out->dL_dhden[(size_t)k * C1 + cell] =
              skip ? 0. : (pert[(size_t)k * C1 + cell] - base[(size_t)k * C1 + cell]) / dh;
      }
  }
  // one balance per abundance
  for (int q = 0; rc == MCX_OK && out->dL_dabun && q < o->n_abun; ++q) {
    const int z = o->abun_z[q];
    float& ab = c->balance->dev.abun[z];
    const float a0 = ab;
    ab = (float)((double)a0 * (1. + h));
    const double da = (double)ab - (double)a0;
    invalidateBalanceGraphs(*c->balance);
    rc = startPerturbed(s0, s1);
    if (rc == MCX_OK) rc = balanceAndLines(pert, tePert, nitPert, sidePert);
    ab = a0;
    invalidateBalanceGraphs(*c->balance);
    if (rc == MCX_OK) {
      std::vector<double> dsum(nL, 0.);
      for (size_t cell = 1; cell < C1; ++cell) {
        if (branched(cell)) {
          ++out->branch_cells_abun;
          continue;
        }
        for (int k = 0; k < nL; ++k) dsum[k] += pert[(size_t)k * C1 + cell] - base[(size_t)k * C1 + cell];
      }
      for (int k = 0; k < nL; ++k) out->dL_dabun[(size_t)k * o->n_abun + q] = dsum[k] / da;
    }
  }
  if (rc == MCX_OK) rc = copyState(c, s1, false);
  cudaEventRecord(t1, c->stream);
  cudaEventSynchronize(t1);
  cudaEventElapsedTime(&out->kernel_ms, t0, t1);
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  if (rc == MCX_OK) CK(cudaStreamSynchronize(c->stream), "mcx_line_sensitivities");
  return rc;
}

extern "C" int mcx_adjoint(mcx_ctx* c, const mcx_sens_opts* o, mcx_adjoint_out* out) {
  std::vector<int32_t> req;
  if (int rc = lineRequests(c, o, out && out->L, "mcx_adjoint", req)) return rc;
  if (o->reference_stopping)
    return fail(c, MCX_ERR_INPUT, "mcx_adjoint: needs the tightly converged balance (reference_stopping = 0)");
  const double h = o->h != 0. ? std::fabs(o->h) : 1.e-3;
  const int nL = o->n_lines, C = c->nCells;
  const size_t C1 = (size_t)C + 1, LC = (size_t)nL * C1;
  CK(cudaSetDevice(c->device), "cudaSetDevice");
  cudaStream_t st = c->stream;
  DBuf<int32_t> dReq;
  CK(upload(dReq, req), "upload line requests");
  // the evaluations: [0] the converged balance, [1, 2] Te(1 +- h), [3, 4] the stepped parameter
  DBuf<double> lum[5], res[5];
  for (int e = 0; e < 5; ++e) {
    CK(lum[e].alloc(LC), "alloc line cells");
    CK(res[e].alloc(C1), "alloc residuals");
  }
  DBuf<float> tP, tM, pP, pM;
  DBuf<double> dLdp, dTdp;
  DBuf<uint8_t> hold, maskRoot, maskSome;
  DBuf<unsigned long long> held;
  CK(tP.alloc(C1), "alloc"); CK(tM.alloc(C1), "alloc"); CK(pP.alloc(C1), "alloc"); CK(pM.alloc(C1), "alloc");
  CK(dLdp.alloc(LC), "alloc"); CK(dTdp.alloc(C1), "alloc"); CK(hold.alloc(C1), "alloc"); CK(held.alloc(1), "alloc");
  CK(maskRoot.alloc(C1), "alloc"); CK(maskSome.alloc(C1), "alloc");
  CK(cudaMemsetAsync(held.p, 0, sizeof(unsigned long long), st), "memset");
  LineCellArgs la{};
  la.te = c->te.p; la.ne = c->ne.p; la.ionDen = c->ionDen.p; la.hden = c->hden.p; la.vol = c->volD.p;
  la.black = c->lgBlack.p; la.req = dReq.p; la.nReq = nL;
  mcx_balance_opts bo{};
  bo.precision = o->precision;
  bo.converge = 1;
  auto lines = [&](int e) -> int {
    la.out = lum[e].p;
    CK(launchLineCellLuminosities(*c->balance, la, st), "line cells");
    return MCX_OK;
  };
  StateCopy s1;
  // R and L with every Te held, from the converged state, for the cells of `mask`; te (host) replaces
  // its Te where given
  auto held_eval = [&](int e, const std::vector<float>* te, const uint8_t* mask) -> int {
    if (int rc = copyState(c, s1, false)) return rc;
    if (te) CK(cudaMemcpyAsync(c->te.p, te->data(), C1 * sizeof(float), cudaMemcpyHostToDevice, st), "h2d Te");
    bo.fix_te = 1;
    c->balance->dev.evalMask = mask;
    int rc = mcx_balance(c, &bo, nullptr);
    c->balance->dev.evalMask = nullptr;
    bo.fix_te = 0;
    if (rc != MCX_OK) return rc;
    if ((rc = lines(e))) return rc;
    CK(cudaMemcpyAsync(res[e].p, c->balance->dev.resid, C1 * sizeof(double), cudaMemcpyDeviceToDevice, st), "d2d R");
    CK(cudaStreamSynchronize(st), "mcx_adjoint");
    return MCX_OK;
  };
  bool countHeld = true;   // the first combination counts the roots it cannot use
  AdjointArgs aa{};
  aa.rTp = res[1].p; aa.rTm = res[2].p; aa.lTp = lum[1].p; aa.lTm = lum[2].p; aa.teP = tP.p; aa.teM = tM.p;
  aa.rPp = res[3].p; aa.rPm = res[4].p; aa.lPp = lum[3].p; aa.lPm = lum[4].p;
  aa.hold = hold.p; aa.dLdp = dLdp.p; aa.nCells = C; aa.nL = nL;

  cudaEvent_t t0 = nullptr, t1 = nullptr;
  CK(cudaEventCreate(&t0), "event");
  CK(cudaEventCreate(&t1), "event");
  CK(cudaEventRecord(t0, st), "event");
  out->pinned_cells = 0;
  out->no_solution_cells = 0;
  // the converged balance (from the current state) and its line sums
  int rc = mcx_balance(c, &bo, nullptr);
  if (rc == MCX_OK) rc = lines(0);
  if (rc == MCX_OK) rc = copyState(c, s1, true);
  std::vector<float> te(C1), hd(C1), stepP(C1), stepM(C1);
  std::vector<int32_t> nit(C1), black(C1);
  std::vector<int8_t> side(C1);
  std::vector<double> hostL(LC);
  if (rc == MCX_OK) {
    CK(cudaMemcpyAsync(hostL.data(), lum[0].p, LC * sizeof(double), cudaMemcpyDeviceToHost, st), "d2h L");
    CK(cudaMemcpyAsync(te.data(), c->te.p, C1 * sizeof(float), cudaMemcpyDeviceToHost, st), "d2h Te");
    CK(cudaMemcpyAsync(hd.data(), c->hden.p, C1 * sizeof(float), cudaMemcpyDeviceToHost, st), "d2h Hden");
    CK(cudaMemcpyAsync(nit.data(), c->nIterT.p, C1 * sizeof(int32_t), cudaMemcpyDeviceToHost, st), "d2h");
    CK(cudaMemcpyAsync(black.data(), c->lgBlack.p, C1 * sizeof(int32_t), cudaMemcpyDeviceToHost, st), "d2h");
    CK(cudaMemcpyAsync(side.data(), c->balance->dev.side, C1, cudaMemcpyDeviceToHost, st), "d2h");
    CK(cudaStreamSynchronize(st), "mcx_adjoint");
    for (int k = 0; k < nL; ++k) {
      double t = 0.;
      for (size_t cell = 1; cell < C1; ++cell) t += hostL[(size_t)k * C1 + cell];
      out->L[k] = t;
    }
    // a cell without a root: its bracket closed on a jump (Te held); a cell whose balance did not
    // converge in 64 T-iterations has no converged state to differentiate (no derivative).  The
    // evaluations at Te(1 +- h) need the cells with a root, those at p(1 +- h) these and the held ones
    std::vector<uint8_t> hh(C1, 2), mr(C1, 0), ms(C1, 0);
    for (size_t cell = 1; cell < C1; ++cell) {
      hh[cell] = black[cell] >= 1 ? 2 : nit[cell] >= kMaxRounds ? 3 : side[cell] == 3 ? 1 : 0;
      mr[cell] = hh[cell] == 0;
      ms[cell] = hh[cell] <= 1;
      out->no_solution_cells += hh[cell] == 3;
      out->pinned_cells += hh[cell] == 1;
    }
    CK(cudaMemcpyAsync(hold.p, hh.data(), C1, cudaMemcpyHostToDevice, st), "h2d hold");
    CK(cudaMemcpyAsync(maskRoot.p, mr.data(), C1, cudaMemcpyHostToDevice, st), "h2d mask");
    CK(cudaMemcpyAsync(maskSome.p, ms.data(), C1, cudaMemcpyHostToDevice, st), "h2d mask");
    // Te(1 +- h)
    for (size_t cell = 0; cell < C1; ++cell) {
      stepP[cell] = (float)((double)te[cell] * (1. + h));
      stepM[cell] = (float)((double)te[cell] * (1. - h));
    }
    CK(cudaMemcpyAsync(tP.p, stepP.data(), C1 * sizeof(float), cudaMemcpyHostToDevice, st), "h2d");
    CK(cudaMemcpyAsync(tM.p, stepM.data(), C1 * sizeof(float), cudaMemcpyHostToDevice, st), "h2d");
    rc = held_eval(1, &stepP, maskRoot.p);
    if (rc == MCX_OK) rc = held_eval(2, &stepM, maskRoot.p);
  }
  // every cell's Hden (1 +- h) at once: at fixed J each cell answers for itself
  if (rc == MCX_OK && (out->dL_dhden || out->dte_dhden)) {
    for (size_t cell = 0; cell < C1; ++cell) {
      stepP[cell] = (float)((double)hd[cell] * (1. + h));
      stepM[cell] = (float)((double)hd[cell] * (1. - h));
    }
    CK(cudaMemcpyAsync(pP.p, stepP.data(), C1 * sizeof(float), cudaMemcpyHostToDevice, st), "h2d");
    CK(cudaMemcpyAsync(pM.p, stepM.data(), C1 * sizeof(float), cudaMemcpyHostToDevice, st), "h2d");
    CK(cudaMemcpyAsync(c->hden.p, stepP.data(), C1 * sizeof(float), cudaMemcpyHostToDevice, st), "h2d Hden");
    rc = held_eval(3, nullptr, maskSome.p);
    if (rc == MCX_OK) {
      CK(cudaMemcpyAsync(c->hden.p, stepM.data(), C1 * sizeof(float), cudaMemcpyHostToDevice, st), "h2d Hden");
      rc = held_eval(4, nullptr, maskSome.p);
    }
    CK(cudaMemcpyAsync(c->hden.p, hd.data(), C1 * sizeof(float), cudaMemcpyHostToDevice, st), "h2d Hden");
    if (rc == MCX_OK) {
      aa.pP = pP.p; aa.pM = pM.p; aa.dTdp = dTdp.p; aa.held = countHeld ? held.p : nullptr;
      countHeld = false;
      CK(launchAdjointCombine(aa, st), "adjoint kernel");
      if (out->dL_dhden)
        CK(cudaMemcpyAsync(out->dL_dhden, dLdp.p, LC * sizeof(double), cudaMemcpyDeviceToHost, st), "d2h");
      if (out->dte_dhden)
        CK(cudaMemcpyAsync(out->dte_dhden, dTdp.p, C1 * sizeof(double), cudaMemcpyDeviceToHost, st), "d2h");
      CK(cudaStreamSynchronize(st), "mcx_adjoint");
    }
  }
  // each abundance (1 +- h), one parameter shared by every cell
  for (int q = 0; rc == MCX_OK && out->dL_dabun && q < o->n_abun; ++q) {
    const int z = o->abun_z[q];
    float& ab = c->balance->dev.abun[z];
    const float a0 = ab, ap = (float)((double)a0 * (1. + h)), am = (float)((double)a0 * (1. - h));
    ab = ap;
    invalidateBalanceGraphs(*c->balance);
    rc = held_eval(3, nullptr, maskSome.p);
    ab = am;
    invalidateBalanceGraphs(*c->balance);
    if (rc == MCX_OK) rc = held_eval(4, nullptr, maskSome.p);
    ab = a0;
    invalidateBalanceGraphs(*c->balance);
    if (rc != MCX_OK) break;
    aa.pP = nullptr; aa.pM = nullptr; aa.dpScalar = (double)ap - (double)am; aa.dTdp = nullptr;
    aa.held = countHeld ? held.p : nullptr;
    countHeld = false;
    CK(launchAdjointCombine(aa, st), "adjoint kernel");
    CK(cudaMemcpyAsync(hostL.data(), dLdp.p, LC * sizeof(double), cudaMemcpyDeviceToHost, st), "d2h");
    CK(cudaStreamSynchronize(st), "mcx_adjoint");
    for (int k = 0; k < nL; ++k) {
      double t = 0.;
      for (size_t cell = 1; cell < C1; ++cell) t += hostL[(size_t)k * C1 + cell];
      out->dL_dabun[(size_t)k * o->n_abun + q] = t;
    }
  }
  if (rc == MCX_OK) {
    // roots whose dR/dTe (or dR/dp) the first combination found unusable also keep their Te
    unsigned long long nh = 0;
    CK(cudaMemcpyAsync(&nh, held.p, sizeof(nh), cudaMemcpyDeviceToHost, st), "d2h");
    CK(cudaStreamSynchronize(st), "mcx_adjoint");
    out->pinned_cells += (int64_t)nh;
    rc = copyState(c, s1, false);
  }
  cudaEventRecord(t1, st);
  cudaEventSynchronize(t1);
  cudaEventElapsedTime(&out->kernel_ms, t0, t1);
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  if (rc == MCX_OK) CK(cudaStreamSynchronize(st), "mcx_adjoint");
  return rc;
}

extern "C" int mcx_timer_start(mcx_ctx* c) {
  if (!c) return MCX_ERR_INPUT;
  CK(cudaEventRecord(c->tev0, c->stream), "timer");
  return MCX_OK;
}

extern "C" int mcx_timer_stop(mcx_ctx* c, float* ms) {
  if (!c || !ms) return MCX_ERR_INPUT;
  CK(cudaEventRecord(c->tev1, c->stream), "timer");
  CK(cudaEventSynchronize(c->tev1), "timer");
  CK(cudaEventElapsedTime(ms, c->tev0, c->tev1), "timer");
  return MCX_OK;
}

extern "C" const char* mcx_version(void) { return "mcx 0.1 (sm_103a)"; }
