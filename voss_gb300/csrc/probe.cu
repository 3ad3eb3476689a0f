// probe.cu -- shared-memory bandwidth microbenchmarks that give the sieve's
// roofline denominator on the running GPU.  Two rates:
//   * ld/st: each thread reads and writes its own 32-bit word per step
//     (conflict-free, 8 bytes per step): the shared-memory data-path roof;
//   * atomic: each thread applies atomicAnd to its own word per step
//     (conflict-free, counted as 8 bytes: a read and a write), the roof of the
//     operation the marking tiers issue.
#include <cuda_runtime.h>

#include <cstdint>

#include "engine.h"

namespace vg {

namespace {

constexpr int kProbeThreads = 1024;
constexpr int kProbeWords = 48 * 1024;      // 192 KiB of shared memory

__global__ void __launch_bounds__(kProbeThreads, 1) smem_ldst_kernel(uint32_t iters, uint32_t* sink) {
  extern __shared__ uint32_t s[];
  for (uint32_t i = threadIdx.x; i < kProbeWords; i += blockDim.x) s[i] = i;
  __syncthreads();
  uint32_t idx = threadIdx.x, acc = 0;
  volatile uint32_t* vs = s;
  for (uint32_t it = 0; it < iters; ++it) {
    const uint32_t v = vs[idx];
    vs[idx] = v + it;
    acc ^= v;
    idx += kProbeThreads;
    if (idx >= kProbeWords) idx -= kProbeWords;
  }
  if (acc == 0xFFFFFFFFu) sink[blockIdx.x] = acc;
}

__global__ void __launch_bounds__(kProbeThreads, 1) smem_atomic_kernel(uint32_t iters, uint32_t* sink) {
  extern __shared__ uint32_t s[];
  for (uint32_t i = threadIdx.x; i < kProbeWords; i += blockDim.x) s[i] = 0xFFFFFFFFu;
  __syncthreads();
  uint32_t idx = threadIdx.x;
  for (uint32_t it = 0; it < iters; ++it) {
    atomicAnd(s + idx, ~(1u << (it & 31)));
    idx += kProbeThreads;
    if (idx >= kProbeWords) idx -= kProbeWords;
  }
  __syncthreads();
  if (s[threadIdx.x] == 0x12345678u) sink[blockIdx.x] = 1;
}

template <class K>
double time_kernel(K kernel, uint32_t grid, uint32_t iters, uint32_t* sink, cudaStream_t s) {
  const size_t smem = kProbeWords * 4;
  check_cuda(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem), "probe attr");
  kernel<<<grid, kProbeThreads, smem, s>>>(iters / 8, sink);   // warm-up
  cudaEvent_t e0, e1;
  check_cuda(cudaEventCreate(&e0), "event");
  check_cuda(cudaEventCreate(&e1), "event");
  float best = 1e30f;
  for (int r = 0; r < 3; ++r) {
    check_cuda(cudaEventRecord(e0, s), "event");
    kernel<<<grid, kProbeThreads, smem, s>>>(iters, sink);
    check_cuda(cudaEventRecord(e1, s), "event");
    check_cuda(cudaEventSynchronize(e1), "probe run");
    float ms = 0;
    check_cuda(cudaEventElapsedTime(&ms, e0, e1), "event");
    if (ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  const double bytes = 8.0 * grid * kProbeThreads * (double)iters;
  return bytes / (best * 1e-3) / 1e9;
}

}  // namespace

void smem_peaks(Engine& E, double* ldst_gbs, double* atomic_gbs) {
  DevBuf sink;
  sink.reserve(4 * E.sm_count);
  const uint32_t iters = 1u << 16;
  if (ldst_gbs) *ldst_gbs = time_kernel(smem_ldst_kernel, E.sm_count, iters, sink.as<uint32_t>(), E.stream);
  if (atomic_gbs) *atomic_gbs = time_kernel(smem_atomic_kernel, E.sm_count, iters, sink.as<uint32_t>(), E.stream);
}

}  // namespace vg
