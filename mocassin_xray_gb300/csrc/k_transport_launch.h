// k_transport_launch.h - host-side launchers of the transport kernel
// instantiations (k_transport_f32.cu, k_transport_f64.cu).
#pragma once
#include "mcx_device.cuh"

namespace mcx {

struct TransportLaunch {
  int blocks;
  int threads;
  size_t smem;
  int emitBatch;   // 0 = the kernel's default
};

cudaError_t launchTransportF32(const DevGrid& g, const DevTransportIn& in, const DevTransportOut& out,
                               DevTransportCounters* cnt, uint64_t seed, uint64_t base, unsigned long long n,
                               double deltaE, const TransportLaunch& L, cudaStream_t s);
cudaError_t launchTransportF64(const DevGrid& g, const DevTransportIn& in, const DevTransportOut& out,
                               DevTransportCounters* cnt, uint64_t seed, uint64_t base, unsigned long long n,
                               double deltaE, const TransportLaunch& L, cudaStream_t s);
// The batch kernel: every nebula's packets in one launch (pktBegin[nNeb] = total).
cudaError_t launchTransportBatchedF32(const DevGrid& g, const DevTransportIn& in, const DevTransportOut& out,
                                      DevTransportCounters* cnt, const NebulaDesc* neb,
                                      const unsigned long long* pktBegin, int nNeb, const float* axes,
                                      const int32_t* active, const float* cdfs, const TransportLaunch& L,
                                      unsigned long long* stamps, cudaStream_t s);
cudaError_t launchTransportBatchedF64(const DevGrid& g, const DevTransportIn& in, const DevTransportOut& out,
                                      DevTransportCounters* cnt, const NebulaDesc* neb,
                                      const unsigned long long* pktBegin, int nNeb, const float* axes,
                                      const int32_t* active, const float* cdfs, const TransportLaunch& L,
                                      unsigned long long* stamps, cudaStream_t s);
cudaError_t transportOccupancyBatchedF32(int threads, size_t smem, int* blocksPerSM);
cudaError_t transportOccupancyBatchedF64(int threads, size_t smem, int* blocksPerSM);

// Resident blocks per SM of the FP64 (fp64 = true) or FP32 instantiation.
cudaError_t transportOccupancy(bool fp64, int threads, size_t smem, int* blocksPerSM);
cudaError_t transportOccupancyF32(int threads, size_t smem, int* blocksPerSM);
cudaError_t transportOccupancyF64(int threads, size_t smem, int* blocksPerSM);

inline cudaError_t transportOccupancy(bool fp64, int threads, size_t smem, int* blocksPerSM) {
  return fp64 ? transportOccupancyF64(threads, smem, blocksPerSM) : transportOccupancyF32(threads, smem, blocksPerSM);
}

}  // namespace mcx
