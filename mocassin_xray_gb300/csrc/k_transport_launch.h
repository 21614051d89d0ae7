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
  // Trapped-packet hand-off (single-grid kernel only): a packet about to be
  // re-emitted for the handoffAt-th time is parked in `parked` (room for
  // parkedCap packets) and continued by the trapped-packet kernel launched
  // right after; handoffAt = 0 or parked = null keeps every packet in place.
  void* parked;
  unsigned long long parkedCap;
  int handoffAt;
  int numSMs;
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

// Bytes of one parked packet of the FP32 / FP64 kernel.
size_t parkedPacketBytesF32();
size_t parkedPacketBytesF64();

// Resident blocks per SM of the FP64 (fp64 = true) or FP32 instantiation of
// the persistent kernel, with or without the plane-parallel source.
cudaError_t transportOccupancyF32(int threads, size_t smem, int* blocksPerSM, bool plane);
cudaError_t transportOccupancyF64(int threads, size_t smem, int* blocksPerSM, bool plane);

inline cudaError_t transportOccupancy(bool fp64, int threads, size_t smem, int* blocksPerSM, bool plane) {
  return fp64 ? transportOccupancyF64(threads, smem, blocksPerSM, plane)
              : transportOccupancyF32(threads, smem, blocksPerSM, plane);
}

}  // namespace mcx
