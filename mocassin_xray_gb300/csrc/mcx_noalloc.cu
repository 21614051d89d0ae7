// mcx_noalloc.cu - mcx_transport_noalloc: the transport kernel run without
// any device allocation, for callers that cannot call cudaMalloc (see the
// declaration in include/mcx.h).  All scratch lives in one file-scope
// __device__ array; the caller owns every input and output buffer.
#include "../../include/mcx.h"
#include "k_transport_launch.h"
#include "mcx_device.cuh"

#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <string>

namespace {

constexpr size_t kScratchBytes = MCX_NOALLOC_SCRATCH_BYTES;
constexpr int kMaxDevices = 64;

// The scratch of every mcx_transport_noalloc call on this GPU.  Host code may
// not use this symbol as an address: it is resolved per device with
// cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_noallocScratch[kScratchBytes];

std::mutex g_mutex;
void* g_scratchAddr[kMaxDevices] = {};
thread_local std::string g_error;

int fail(int code, const std::string& msg) {
  g_error = msg;
  return code;
}

// Device address of g_noallocScratch on the current device (looked up once per device).
int scratchAddress(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(MCX_ERR_CUDA, std::string("mcx_transport_noalloc: cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return fail(MCX_ERR_CUDA, "mcx_transport_noalloc: device index out of range");
  std::lock_guard<std::mutex> lock(g_mutex);
  if (!g_scratchAddr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noallocScratch);
    if (e != cudaSuccess || !p)
      return fail(MCX_ERR_CUDA, std::string("mcx_transport_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    g_scratchAddr[dev] = p;
  }
  *out = g_scratchAddr[dev];
  return MCX_OK;
}

// out[cols][rows] = in[rows][cols]
__global__ void noallocTranspose(const float* __restrict__ in, float* __restrict__ out, int rows, int cols) {
  __shared__ float tile[32][33];
  int bx = blockIdx.x * 32, by = blockIdx.y * 32;
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    int r = by + j, c = bx + threadIdx.x;
    if (r < rows && c < cols) tile[j][threadIdx.x] = in[(size_t)r * cols + c];
  }
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    int r = bx + j, c = by + threadIdx.x;
    if (r < cols && c < rows) out[(size_t)r * rows + c] = tile[threadIdx.x][j];
  }
}

// Volumes of the active cells [e45 cm^3], getVolume (source/grid_mod.f90:2887-2986) in FP64 and FP32.
// The caller's active map is checked on the way: an id above nCells is
// counted in *badIds and its voxel skipped (the transport is then refused).
__global__ void noallocVolumes(const float* X, const float* Y, const float* Z, const int32_t* active, int nx, int ny,
                               int nz, int nCells, int sym, double* volD, float* volF, unsigned int* badIds) {
  const size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= (size_t)nx * ny * nz) return;
  const int cell = active[v];
  if (cell <= 0) return;
  if (cell > nCells) { atomicAdd(badIds, 1u); return; }
  const int xP = (int)(v % nx) + 1, yP = (int)((v / nx) % ny) + 1, zP = (int)(v / ((size_t)nx * ny)) + 1;
  double d[3];
  const float* A[3] = {X, Y, Z};
  const int P[3] = {xP, yP, zP}, N[3] = {nx, ny, nz};
  float f[3];
  for (int k = 0; k < 3; ++k) {
    const float* a = A[k];
    int p = P[k], n = N[k];
    double dd = 0.;
    float ff = 0.f;
    if (p > 1 && p < n) { dd = fabs((double)a[p] - (double)a[p - 2]) / 2.; ff = fabsf(a[p] - a[p - 2]) / 2.f; }
    else if (p == 1) {
      dd = sym ? fabs((double)a[1] - (double)a[0]) / 2. : fabs((double)a[1] - (double)a[0]);
      ff = sym ? fabsf(a[1] - a[0]) / 2.f : fabsf(a[1] - a[0]);
    } else if (p == n) { dd = fabs((double)a[p - 1] - (double)a[p - 2]); ff = fabsf(a[p - 1] - a[p - 2]); }
    d[k] = dd / 1.e15;
    f[k] = ff / 1.e15f;
  }
  volD[cell] = d[0] * d[1] * d[2];
  volF[cell] = f[0] * f[1] * f[2];
}

size_t roundUp(size_t x) { return (x + 255) & ~size_t(255); }

}  // namespace

extern "C" const char* mcx_noalloc_last_error(void) { return g_error.c_str(); }

extern "C" int mcx_transport_noalloc(const mcx_noalloc_transport_args* a, mcx_transport_stats* stats) {
  using namespace mcx;
  if (!a) return fail(MCX_ERR_INPUT, "mcx_transport_noalloc: null arguments");
  if (a->nx < 2 || a->ny < 2 || a->nz < 2 || a->n_cells < 1 || a->nbins < 2 || a->n_packets < 0)
    return fail(MCX_ERR_INPUT, "mcx_transport_noalloc: invalid sizes");
  if (a->precision != MCX_PREC_FP32_GEOM && a->precision != MCX_PREC_FP64)
    return fail(MCX_ERR_INPUT, "mcx_transport_noalloc: unknown precision");
  if (!a->x_axis || !a->y_axis || !a->z_axis || !a->active || !a->nu || !a->src_cdf || !a->kn_sigma_t ||
      !a->kn_cdf || !a->pcomp || !a->opacity || !a->rec_pdf || !a->total_lines || !a->ne || !a->jste || !a->escaped)
    return fail(MCX_ERR_INPUT, "mcx_transport_noalloc: a device pointer is null");
  for (int d = 0; d < 3; ++d) {
    const int n = d == 0 ? a->nx : (d == 1 ? a->ny : a->nz);
    if (a->star_idx[d] < 1 || a->star_idx[d] > n) return fail(MCX_ERR_INPUT, "mcx_transport_noalloc: the source must lie inside the grid");
  }
  const size_t C1 = (size_t)a->n_cells + 1, nb = (size_t)a->nbins;
  const size_t nvox = (size_t)a->nx * (size_t)a->ny * (size_t)a->nz;
  if (nvox > (size_t)0x7fffffff) return fail(MCX_ERR_INPUT, "mcx_transport_noalloc: grid above 2^31 - 1 voxels");
  // scratch layout: counters | active-map check | volD | volF | rec CDF rows | KN CDF rows | Pcomp rows
  const size_t offCnt = 0;
  const size_t offBad = roundUp(sizeof(DevTransportCounters));
  const size_t offVolD = offBad + roundUp(sizeof(unsigned int));
  const size_t offVolF = offVolD + roundUp(C1 * sizeof(double));
  const size_t offRec = offVolF + roundUp(C1 * sizeof(float));
  const size_t offKn = offRec + roundUp(C1 * nb * sizeof(float));
  const size_t offPc = offKn + roundUp(nb * 180 * sizeof(float));
  const size_t need = offPc + roundUp(nb * 180 * sizeof(float));
  if (need > kScratchBytes)
    return fail(MCX_ERR_INPUT, "mcx_transport_noalloc: the problem needs " + std::to_string(need) +
                                   " bytes of scratch, above the fixed limit of " + std::to_string(kScratchBytes) +
                                   " bytes (MCX_NOALLOC_SCRATCH_BYTES); use mcx_transport");
  void* base = nullptr;
  int rc = scratchAddress(&base);
  if (rc != MCX_OK) return rc;
  unsigned char* sb = static_cast<unsigned char*>(base);
  auto* cnt = reinterpret_cast<DevTransportCounters*>(sb + offCnt);
  auto* badIds = reinterpret_cast<unsigned int*>(sb + offBad);
  auto* volD = reinterpret_cast<double*>(sb + offVolD);
  auto* volF = reinterpret_cast<float*>(sb + offVolF);
  auto* recT = reinterpret_cast<float*>(sb + offRec);
  auto* knT = reinterpret_cast<float*>(sb + offKn);
  auto* pcT = reinterpret_cast<float*>(sb + offPc);
  cudaStream_t s = static_cast<cudaStream_t>(a->stream);
  cudaError_t e;
#define NA_CK(call, what) \
  if ((e = (call)) != cudaSuccess) return fail(MCX_ERR_CUDA, std::string("mcx_transport_noalloc: ") + what + ": " + cudaGetErrorString(e))
  int dev = 0, numSMs = 0;
  NA_CK(cudaGetDevice(&dev), "cudaGetDevice");
  NA_CK(cudaDeviceGetAttribute(&numSMs, cudaDevAttrMultiProcessorCount, dev), "multiprocessor count");
  NA_CK(cudaMemsetAsync(cnt, 0, sizeof(DevTransportCounters), s), "clear counters");
  NA_CK(cudaMemsetAsync(badIds, 0, sizeof(unsigned int), s), "clear the active-map check");
  NA_CK(cudaMemsetAsync(volD, 0, C1 * sizeof(double), s), "clear volumes");
  NA_CK(cudaMemsetAsync(volF, 0, C1 * sizeof(float), s), "clear volumes");
  if (a->zero_estimators) {
    NA_CK(cudaMemsetAsync(a->jste, 0, C1 * nb * sizeof(double), s), "clear jste");
    NA_CK(cudaMemsetAsync(a->escaped, 0, C1 * (nb + 1) * sizeof(double), s), "clear escaped");
  }
  noallocVolumes<<<(unsigned)((nvox + 255) / 256), 256, 0, s>>>(a->x_axis, a->y_axis, a->z_axis, a->active, a->nx,
                                                                 a->ny, a->nz, a->n_cells, a->symmetric_xyz, volD,
                                                                 volF, badIds);
  NA_CK(cudaGetLastError(), "volumes");
  unsigned int bad = 0;
  NA_CK(cudaMemcpyAsync(&bad, badIds, sizeof(bad), cudaMemcpyDeviceToHost, s), "read the active-map check");
  NA_CK(cudaStreamSynchronize(s), "synchronize");
  if (bad)
    return fail(MCX_ERR_INPUT, "mcx_transport_noalloc: " + std::to_string(bad) +
                                   " voxel(s) of the active map name a cell above n_cells");
  dim3 tb(32, 8);
  noallocTranspose<<<dim3((unsigned)((C1 + 31) / 32), (unsigned)((nb + 31) / 32)), tb, 0, s>>>(a->rec_pdf, recT, (int)nb, (int)C1);
  NA_CK(cudaGetLastError(), "transpose recPDF");
  noallocTranspose<<<dim3((unsigned)((nb + 31) / 32), (180 + 31) / 32), tb, 0, s>>>(a->kn_cdf, knT, 180, (int)nb);
  NA_CK(cudaGetLastError(), "transpose KN CDF");
  noallocTranspose<<<dim3((unsigned)((nb + 31) / 32), (180 + 31) / 32), tb, 0, s>>>(a->pcomp, pcT, 180, (int)nb);
  NA_CK(cudaGetLastError(), "transpose Pcomp");

  DevGrid g{};
  g.nx = a->nx; g.ny = a->ny; g.nz = a->nz; g.nCells = a->n_cells; g.nbins = a->nbins;
  g.symmetric = a->symmetric_xyz; g.lgDust = 0; g.lgGas = 1; g.lgCompton = a->lg_compton; g.radPress = 0;
  for (int d = 0; d < 3; ++d) { g.starIdx[d] = a->star_idx[d]; g.starPos[d] = a->star_pos[d]; }
  g.ionEdge1 = a->ion_edge1; g.rOut = a->r_out;
  g.xAxis = a->x_axis; g.yAxis = a->y_axis; g.zAxis = a->z_axis; g.active = a->active;
  g.nu = a->nu; g.srcCDF = a->src_cdf; g.KNsigmaT = a->kn_sigma_t; g.KNcdfT = knT; g.PcompT = pcT;
  g.volD = volD; g.volF = volF;
  DevTransportIn in{};
  in.opacity = a->opacity; in.scaOpac = nullptr; in.recCDFT = recT; in.dustCDFT = nullptr;
  in.totalLines = a->total_lines; in.ne = a->ne;
  DevTransportOut out{};
  out.jste = a->jste; out.escaped = a->escaped; out.hEst = nullptr;

  TransportLaunch L{};
  L.threads = 256;
  L.smem = (size_t)(a->nx + a->ny + a->nz + 2 * a->nbins) * sizeof(float);
  int perSM = 0;
  NA_CK(transportOccupancy(a->precision == MCX_PREC_FP64, L.threads, L.smem, &perSM, false), "occupancy");
  L.blocks = numSMs * (perSM < 1 ? 1 : perSM);
  const unsigned long long n = (unsigned long long)a->n_packets;
  if (n > 0) {
    const unsigned long long maxBlocks = (n + L.threads - 1) / L.threads;
    if ((unsigned long long)L.blocks > maxBlocks) L.blocks = (int)maxBlocks;
    e = (a->precision == MCX_PREC_FP64)
            ? launchTransportF64(g, in, out, cnt, a->seed, a->counter_base, n, a->delta_e, L, s)
            : launchTransportF32(g, in, out, cnt, a->seed, a->counter_base, n, a->delta_e, L, s);
    NA_CK(e, "transport kernel");
  }
  DevTransportCounters h{};
  NA_CK(cudaMemcpyAsync(&h, cnt, sizeof(h), cudaMemcpyDeviceToHost, s), "read counters");
  NA_CK(cudaStreamSynchronize(s), "synchronize");
#undef NA_CK
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
  }
  if (h.errors)
    return fail(MCX_ERR_INTERNAL, "mcx_transport_noalloc: " + std::to_string(h.errors) +
                                      " packet(s) reached a state where the reference stops");
  return MCX_OK;
}
