// goldbach.h -- consumers of a sieved wheel bitmap: Goldbach smallest-prime
// check, Sophie Germain count, sorted prime list.  Internal C++.
#pragma once
#include <cstdint>
#include <vector>

#include "engine.h"

namespace vg {

// Smallest odd primes used by the Goldbach kernel (all p < 65536).
constexpr uint32_t kGoldbachPrimes = 6541;
constexpr uint32_t kGoldbachHistBins = 65536;   // hist by p

struct GoldbachResult {
  uint32_t max_minp = 0;
  uint64_t sum_minp = 0;
  uint64_t n_counterexamples = 0;
  std::vector<uint64_t> counterexamples;   // at most max_ce, ascending
  std::vector<uint64_t> hist;              // kGoldbachHistBins, by p
};

// For every even n in [4, N]: the smallest prime p with n - p prime.
// minp_host (optional) receives (N-4)/2+1 entries, 0 for a counterexample.
GoldbachResult goldbach_run(Engine& E, uint64_t N, uint32_t* minp_host, uint64_t max_ce,
                            float* kernel_ms = nullptr);

// Device-resident Goldbach run for timing: the bitmap and outputs stay on the
// device; returns the min-p kernel's time in ms measured with CUDA events.
struct GoldbachPlan;
GoldbachPlan* goldbach_plan_create(Engine& E, uint64_t N);
void goldbach_plan_launch(GoldbachPlan* g, cudaStream_t s);
void goldbach_plan_fetch(GoldbachPlan* g, GoldbachResult* out, cudaStream_t s);
void goldbach_plan_free(GoldbachPlan* g);
uint64_t goldbach_plan_probes(GoldbachPlan* g);

// Primes p <= N with 2p+1 prime.
uint64_t sophie_germain_count(Engine& E, uint64_t N);

// Primes q with a <= q <= b, ascending; stops counting at max_count + 1.
std::vector<uint64_t> primes_in_range(Engine& E, uint64_t a, uint64_t b, uint64_t max_count);

}  // namespace vg
