// probe.cu -- shared-memory bandwidth microbenchmarks that give the sieve's
// roofline denominator on the running GPU.  Two rates:
//   * ld/st: each thread reads and writes its own 32-bit word per step
//     (conflict-free, 8 bytes per step): the shared-memory data-path roof;
//   * atomic: each thread applies atomicAnd to its own word per step
//     (conflict-free, counted as 8 bytes: a read and a write), the roof of the
//     operation the marking tiers issue.
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

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

// Clocks per warp-wide shared atomicAnd when the lanes' banks collide k ways.
// Each lane holds one base address (row r_l of 32 words, bank b_l); op j of an
// unrolled block goes to base + 32 j words, an immediate offset, so every
// atomic is one instruction and every op of a lane stays on bank b_l.  Bases:
// rows (warp group * 32 + lane) * 5 mod 1280 (distinct within a warp), banks
// per pattern.  All addresses: < 1280 * 32 + 63 * 32 words < 48 Ki words.
constexpr uint32_t kCostRows = 1280;
constexpr uint32_t kCostOps = 64;
static_assert(kCostRows * 32u + (kCostOps - 1u) * 32u < (uint32_t)kProbeWords, "probe addresses in bounds");

__global__ void __launch_bounds__(kProbeThreads, 1)
smem_atomic_cost_kernel(uint32_t iters, uint32_t pattern, unsigned long long* cyc, uint32_t* sink) {
  extern __shared__ uint32_t s[];
  for (uint32_t i = threadIdx.x; i < kProbeWords; i += blockDim.x) s[i] = 0xFFFFFFFFu;
  __syncthreads();
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const uint32_t row = ((warp & 7u) * 32u + lane) * 5u % kCostRows;
  uint32_t bank = lane;                                   // pattern 0: distinct banks
  if (pattern == 1) bank = lane & 15u;                    // 2-way
  else if (pattern == 2) bank = lane & 7u;                // 4-way
  else if (pattern == 3) bank = lane & 3u;                // 8-way
  else if (pattern == 4) {                               // scattered: a hash of (warp, lane)
    uint32_t h = (lane + 1u) * 0x9E3779B9u ^ (warp + 1u) * 0x85EBCA6Bu;
    h ^= h >> 15; h *= 0x2C1B3C6Du; h ^= h >> 12; h *= 0x297A2D39u; h ^= h >> 15;
    bank = h >> 27;
  }
  uint32_t* p = s + row * 32u + bank;
  const uint32_t mask = ~(1u << lane);
  const unsigned long long t0 = clock64();
  for (uint32_t it = 0; it < iters; ++it) {
#pragma unroll
    for (uint32_t j = 0; j < kCostOps; ++j) atomicAnd(p + 32u * j, mask);
  }
  const unsigned long long t1 = clock64();
  __syncthreads();
  if (lane == 0) atomicMax(cyc + blockIdx.x, t1 - t0);
  if (threadIdx.x == 0 && s[0] == 0x12345678u) sink[blockIdx.x] = 1;
}

}  // namespace

void smem_atomic_cost(Engine& E, double clocks[5]) {
  DevBuf sink, cyc;
  sink.reserve(4 * E.sm_count);
  cyc.reserve(8 * E.sm_count);
  const size_t smem = kProbeWords * 4;
  check_cuda(cudaFuncSetAttribute(smem_atomic_cost_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
             "probe attr");
  const uint32_t iters = 256;
  std::vector<unsigned long long> h(E.sm_count);
  for (uint32_t pat = 0; pat < 5; ++pat) {
    for (int rep = 0; rep < 2; ++rep) {       // the first run warms the clocks up
      check_cuda(cudaMemsetAsync(cyc.ptr, 0, 8 * E.sm_count, E.stream), "probe memset");
      smem_atomic_cost_kernel<<<E.sm_count, kProbeThreads, smem, E.stream>>>(iters, pat, cyc.as<unsigned long long>(),
                                                                            sink.as<uint32_t>());
      check_cuda(cudaGetLastError(), "probe launch");
    }
    check_cuda(cudaMemcpyAsync(h.data(), cyc.ptr, 8 * E.sm_count, cudaMemcpyDeviceToHost, E.stream), "probe copy");
    check_cuda(cudaStreamSynchronize(E.stream), "probe run");
    double sum = 0;
    for (unsigned long long c : h) sum += (double)c;
    // per SM: (warps x iters x ops) warp-wide atomics
    clocks[pat] = sum / E.sm_count / ((double)(kProbeThreads / 32) * iters * kCostOps);
  }
}

void smem_peaks(Engine& E, double* ldst_gbs, double* atomic_gbs) {
  DevBuf sink;
  sink.reserve(4 * E.sm_count);
  const uint32_t iters = 1u << 16;
  if (ldst_gbs) *ldst_gbs = time_kernel(smem_ldst_kernel, E.sm_count, iters, sink.as<uint32_t>(), E.stream);
  if (atomic_gbs) *atomic_gbs = time_kernel(smem_atomic_kernel, E.sm_count, iters, sink.as<uint32_t>(), E.stream);
}

}  // namespace vg
