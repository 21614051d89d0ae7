// k_transport_f32.cu - float-geometry instantiation of the transport kernel.
#include "k_transport.cuh"
#include "k_transport_launch.h"

namespace mcx {

cudaError_t launchTransportF32(const DevGrid& g, const DevTransportIn& in, const DevTransportOut& out,
                               DevTransportCounters* cnt, uint64_t seed, uint64_t base, unsigned long long n,
                               double deltaE, const TransportLaunch& L, cudaStream_t s) {
  transportKernel<float><<<L.blocks, L.threads, L.smem, s>>>(g, in, out, cnt, seed, base, n, deltaE,
                                                         L.emitBatch > 0 ? L.emitBatch : kEmitBatch);
  return cudaGetLastError();
}

cudaError_t launchTransportBatchedF32(const DevGrid& g, const DevTransportIn& in, const DevTransportOut& out,
                                      DevTransportCounters* cnt, const NebulaDesc* neb,
                                      const unsigned long long* pktBegin, int nNeb, const float* axes,
                                      const int32_t* active, const float* cdfs, const TransportLaunch& L,
                                      cudaStream_t s) {
  transportKernelBatched<float><<<L.blocks, L.threads, L.smem, s>>>(g, in, out, cnt, neb, pktBegin, nNeb, axes, active,
                                                                  cdfs, L.emitBatch > 0 ? L.emitBatch : kEmitBatch);
  return cudaGetLastError();
}

cudaError_t transportOccupancyBatchedF32(int threads, size_t smem, int* blocksPerSM) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocksPerSM, transportKernelBatched<float>, threads, smem);
}

cudaError_t transportOccupancyF32(int threads, size_t smem, int* blocksPerSM) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocksPerSM, transportKernel<float>, threads, smem);
}

}  // namespace mcx
