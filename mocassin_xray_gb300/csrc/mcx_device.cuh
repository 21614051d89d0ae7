// mcx_device.cuh - device-side data structures and helpers shared by the
// transport, opacity and balance kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace mcx {

// Frequency-independent grid description, passed by value to kernels.
struct DevGrid {
  int32_t nx, ny, nz, nCells, nbins;
  int32_t symmetric, lgDust, lgGas, lgCompton, radPress;
  // 1 when active(i,j,k) numbers every cell of the full grid in the
  // reference's order, (i-1) ny nz + (j-1) nz + k: the cell id is then
  // computed instead of loaded (one dependent global load less per event)
  int32_t activeFull;
  // 1 for plane-parallel ionisation (lgPlaneIonization): stellar packets start
  // on the plane y = 0 moving along +y, escape through the y planes only and
  // are reflected at the x and z planes
  int32_t plane;
  int32_t starIdx[3];
  float starPos[3];
  float ionEdge1, rOut;
  const float* xAxis;        // [nx]
  const float* yAxis;        // [ny]
  const float* zAxis;        // [nz]
  const int32_t* active;     // [nz][ny][nx]
  const float* nu;           // [nbins]
  const float* srcCDF;       // [nbins]
  const float* KNsigmaT;     // [nbins]
  const float* KNcdfT;       // [nbins][180]  (theta fastest, one row per frequency)
  const float* PcompT;       // [nbins][180]
  const double* volD;        // [nCells+1] cell volume [e45 cm^3] (FP64)
  const float* volF;         // [nCells+1] the same in FP32
  // viewing angles (the 'inclination' keyword): escapes are also binned into
  // plane k of escapedPackets when their direction falls in view k's bins
  int32_t nAngle, totPhi;            // nAngleBins; totAngleBinsPhi (20, or 1 without phi dependence)
  int8_t viewPTheta[21];             // viewPointPtheta(0:20)
  int8_t viewPPhi[21];               // viewPointPphi(0:totPhi)
};

// Per-cell fields the transport reads.
struct DevTransportIn {
  const float* opacity;      // [nbins][C+1]
  const float* scaOpac;      // [nbins][C+1] or null
  const float* recCDFT;      // [C+1][nbins]  re-emission CDF rows (frequency fastest)
  const float* dustCDFT;     // [C+1][nbins]  dust emission CDF rows or null
  const float* totalLines;   // [C+1]
  const float* ne;           // [C+1]
};

struct DevTransportOut {
  double* jste;              // [nbins][C+1]
  double* jlo;               // [nbins][C+1] rounding errors of the jste additions, or null (uncompensated)
  double* escaped;           // [nbins+1][C+1]
  double* hEst;              // [nbins][C+1] or null
};

// One nebula of a batch (mcx_load_batched): its geometry as slices of the
// batch's concatenated axes / active map / source CDFs, and the constants of
// its packets.
struct NebulaDesc {
  int32_t nx, ny, nz, symmetric;
  int32_t axOff, actOff, cdfOff, pad0;  // offsets into the batch's axes / active / source-CDF arrays
  int32_t starIdx[3];
  float starPos[3];
  float rOut, pad1;
  double deltaE;                        // L* / nPhotons of this nebula
  uint64_t seed, counterBase;           // Philox key and the global id of its first packet
};

// Counters accumulated by the transport kernel (device scratch).
struct DevTransportCounters {
  unsigned long long crossings, interactions, absorptions, scatterings;
  unsigned long long escaped, lineEscapes, trapped, emissions;
  unsigned long long errors;
  unsigned long long queue;            // work-queue head (next packet index)
  double qPhot;
  unsigned long long handoff;          // packets parked for the trapped-packet kernel (may exceed the capacity)
  unsigned long long parkedNext;       // the trapped-packet kernel's queue head (beyond its first wave)
  unsigned long long pad[3];
};

// Philox4x32-10 (Salmon et al., SC'11), round constants of the published algorithm.
__host__ __device__ inline void philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                              uint32_t k0, uint32_t k1, uint32_t out[4]) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
#ifdef __CUDA_ARCH__
    uint32_t lo0 = 0xD2511F53u * c0, hi0 = __umulhi(0xD2511F53u, c0);
    uint32_t lo1 = 0xCD9E8D57u * c2, hi1 = __umulhi(0xCD9E8D57u, c2);
#else
    uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t lo0 = (uint32_t)p0, hi0 = (uint32_t)(p0 >> 32), lo1 = (uint32_t)p1, hi1 = (uint32_t)(p1 >> 32);
#endif
    uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    if (r < 9) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

#ifdef __CUDACC__
// One Philox block, out of line and by value: inlined at every draw site the
// ten rounds would crowd the transport loop out of the instruction cache (a
// draw needs a new block once in four), and a value result keeps the caller's
// state in registers.
__device__ __noinline__ inline uint4 philoxBlock(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t k0, uint32_t k1) {
  uint32_t o[4];
  philox4x32_10(c0, c1, c2, 0u, k0, k1, o);
  return make_uint4(o[0], o[1], o[2], o[3]);
}
#endif

// Per-packet counter-based stream: draw k of packet pid is word k%4 of
// philox(key, (pid_lo, pid_hi, k/4, k>>34)).
struct PacketRng {
  uint32_t k0, k1, p0, p1;
  uint32_t buf[4];
  uint32_t k;        // draws taken so far (histories never take 2^32 draws)

  __device__ __forceinline__ void init(uint64_t seed, uint64_t pid) {
    k0 = (uint32_t)seed; k1 = (uint32_t)(seed >> 32);
    p0 = (uint32_t)pid; p1 = (uint32_t)(pid >> 32);
    k = 0;
  }
  __device__ __forceinline__ uint32_t next() {
    if ((k & 3u) == 0) {
      const uint4 b = philoxBlock(p0, p1, k >> 2, k0, k1);
      buf[0] = b.x; buf[1] = b.y; buf[2] = b.z; buf[3] = b.w;
    }
    uint32_t x;
    switch (k & 3u) { case 0: x = buf[0]; break; case 1: x = buf[1]; break; case 2: x = buf[2]; break; default: x = buf[3]; }
    ++k;
    return x;
  }
};

// Uniform in (0,1) in the geometry precision R.
template <typename R> __device__ __forceinline__ R uniformFrom(uint32_t x);
template <> __device__ __forceinline__ double uniformFrom<double>(uint32_t x) {
  return ((double)x + 0.5) * (1.0 / 4294967296.0);
}
template <> __device__ __forceinline__ float uniformFrom<float>(uint32_t x) {
  return ((float)(x >> 8) + 0.5f) * 5.9604644775390625e-08f;
}

}  // namespace mcx
