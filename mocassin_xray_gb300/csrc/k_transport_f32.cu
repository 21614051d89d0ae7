// k_transport_f32.cu - float-geometry instantiation of the transport kernel.
#include "k_transport.cuh"
#include "k_transport_launch.h"

namespace mcx {

cudaError_t launchTransportF32(const DevGrid& g, const DevTransportIn& in, const DevTransportOut& out,
                               DevTransportCounters* cnt, uint64_t seed, uint64_t base, unsigned long long n,
                               double deltaE, const TransportLaunch& L, cudaStream_t s) {
  return launchTransportImpl<float>(g, in, out, cnt, seed, base, n, deltaE, L, s);
}

size_t parkedPacketBytesF32() { return sizeof(Packet<float>); }

cudaError_t launchTransportBatchedF32(const DevGrid& g, const DevTransportIn& in, const DevTransportOut& out,
                                      DevTransportCounters* cnt, const NebulaDesc* neb,
                                      const unsigned long long* pktBegin, int nNeb, const float* axes,
                                      const int32_t* active, const float* cdfs, const TransportLaunch& L,
                                      unsigned long long* stamps, cudaStream_t s) {
  const size_t smem = packetStateOffset(L.smem) + packetStateBytes<float>(L.threads);
  cudaError_t e =
      cudaFuncSetAttribute(transportKernelBatched<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  // stamps[0]: the global timer at the start; stamps[1 + b]: when nebula b's last packet finished
  stampStartKernel<<<1, 1, 0, s>>>(stamps);
  transportKernelBatched<float><<<L.blocks, L.threads, smem, s>>>(g, in, out, cnt, neb, pktBegin, nNeb, axes, active,
                                                                  cdfs, L.emitBatch > 0 ? L.emitBatch : kEmitBatch,
                                                                  stamps + 1);
  return cudaGetLastError();
}

cudaError_t transportOccupancyBatchedF32(int threads, size_t smem, int* blocksPerSM) {
  const size_t all = packetStateOffset(smem) + packetStateBytes<float>(threads);
  cudaError_t e =
      cudaFuncSetAttribute(transportKernelBatched<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)all);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocksPerSM, transportKernelBatched<float>, threads, all);
}

template <bool kPlane>
static cudaError_t occupancyF32(int threads, size_t smem, int* blocksPerSM) {
  const size_t all = packetStateOffset(smem) + packetStateBytes<float>(threads);
  cudaError_t e =
      cudaFuncSetAttribute(transportKernel<float, kPlane>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)all);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocksPerSM, transportKernel<float, kPlane>, threads, all);
}

cudaError_t transportOccupancyF32(int threads, size_t smem, int* blocksPerSM, bool plane) {
  return plane ? occupancyF32<true>(threads, smem, blocksPerSM) : occupancyF32<false>(threads, smem, blocksPerSM);
}

}  // namespace mcx
