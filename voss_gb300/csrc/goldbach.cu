// goldbach.cu -- kernels that read a sieved wheel bitmap.
//
//  * goldbach_minp_kernel: for every even n in [6, N] the smallest odd prime
//    p with n - p prime.  The reference walks the prime list per n and stops
//    at the first p whose partner is set in a 64-bit-per-64-numbers bitmap
//    (goldbach_upto.cu:25-46); it keeps only the counterexamples.  Here one
//    CTA holds 32768 even n as a bit set U of unresolved n; for p = 3, 5, 7...
//    the partners n - p of the whole tile are one shifted window of an
//    odd-number bitmap, so U & window resolves 32 n per word operation.  The
//    smallest p per n, its maximum and its histogram come out; the
//    counterexamples are the n left in U once p > n/2.
//  * sophie_germain_kernel: p <= N with 2p+1 prime (sophie_germain_upto.cu:
//    22-33), read straight from the wheel bitmap: only p = 11, 23, 29 mod 30
//    can qualify, and their 2p+1 falls on fixed bits of byte 2k or 2k+1.
//  * extract kernels: the sorted prime list of a range (range.cu:225-259),
//    by per-block popcount, an exclusive scan, and an ordered write.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <memory>
#include <vector>

#include "attr_cache.h"
#include "goldbach.h"
#include "voss/voss.h"

namespace vg {

namespace {


__device__ __forceinline__ uint64_t umin64(uint64_t x, uint64_t y) { return x < y ? x : y; }

__device__ __forceinline__ uint32_t wheel_bit(const uint32_t* __restrict__ wb, uint64_t k,
                                              uint32_t o) {
  return (__ldg(wb + (k >> 2)) >> ((uint32_t)((k & 3) << 3) + o)) & 1u;
}

// Odd-number bitmap: bit i of `odd` <-> 2i+1, for 2i+1 <= limit.  Byte k of
// the wheel bitmap holds the odd numbers 30k+1 .. 30k+29, which are odd bits
// 15k .. 15k+14, its class o at offset (W30[o]-1)/2 = 0,3,5,6,8,9,11,14; a
// 256-entry table spreads a byte to its 15-bit chunk, and an output word (odd
// bits 32w .. 32w+31) is at most four chunks shifted into place.  3 and 5 are
// not wheel residues and are set by hand.  Wheel bytes from kbytes on are 0.
__global__ void odd_bitmap_kernel(const uint32_t* __restrict__ wb, uint64_t kbytes,
                                  uint32_t* __restrict__ odd, uint64_t odd_words, uint64_t limit) {
  __shared__ uint16_t lut[256];
  constexpr uint32_t kOddOffsets = 0xEB986530u;      // (W30[o]-1)/2, 4 bits per class
  for (uint32_t v = threadIdx.x; v < 256; v += blockDim.x) {
    uint32_t c = 0;
    for (uint32_t o = 0; o < 8; ++o)
      if ((v >> o) & 1u) c |= 1u << ((kOddOffsets >> (4 * o)) & 15u);
    lut[v] = (uint16_t)c;
  }
  __syncthreads();
  const uint8_t* __restrict__ bytes = reinterpret_cast<const uint8_t*>(wb);
  for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < odd_words;
       w += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t b0 = 32 * w;
    const uint64_t k0 = b0 / 15;
    const uint32_t off = (uint32_t)(b0 - 15 * k0);
    uint64_t acc = 0;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const uint64_t k = k0 + c;
      if (k < kbytes) acc |= (uint64_t)lut[__ldg(bytes + k)] << (15 * c);
    }
    uint32_t out = (uint32_t)(acc >> off);
    if (w == 0) out |= (limit >= 3 ? 2u : 0u) | (limit >= 5 ? 4u : 0u);
    odd[w] = out;
  }
}

constexpr int kGbThreads = 256;
constexpr int kGbWords = 8;                                  // U words per thread
constexpr uint32_t kGbTile = kGbThreads * kGbWords * 32;     // even n per tile
constexpr uint32_t kGbSmemHist = 4096;                       // p < 4096 counted in smem
constexpr size_t kGbSmemBytes = kGbSmemHist * 4;
// The dense bit-set walk stops once at most this many n of a tile are open;
// the rest are tested a warp per n.
constexpr uint32_t kGbList = 256;
// Zero words before and after the odd-number bitmap: a thread's window words
// (floor(base/32) + kGbWords*tid .. + kGbWords) then never leave the buffer,
// with no bounds test (base >= -kGbTile/2 in the first tile, so at most
// kGbTile/64 words before it; the last tile's window ends at most
// kGbTile/32 + 1 words past the bitmap).
constexpr uint64_t kGbPad = kGbTile / 32 + 64;

// Does any of this thread's n wait for a prime?
__device__ __forceinline__ bool any_open(const uint32_t (&U)[kGbWords]) {
  uint32_t x = 0;
#pragma unroll
  for (int q = 0; q < kGbWords; ++q) x |= U[q];
  return x != 0;
}

struct GbOut {
  uint32_t* minp;                    // optional, index (n-4)/2
  unsigned long long* hist;          // by p
  unsigned int* max_minp;
  unsigned long long* sum_minp;
  unsigned long long* n_ce;
  unsigned long long* ce;
  uint64_t ce_cap;
  unsigned long long* probes;
  unsigned int* err;                 // 1: the prime list ran out before n/2
};

__global__ void __launch_bounds__(kGbThreads, 4)
goldbach_minp_kernel(const uint32_t* __restrict__ odd,
                     const uint32_t* __restrict__ oddp, uint32_t noddp, uint64_t N,
                     uint64_t ntiles, GbOut out) {
  extern __shared__ __align__(16) uint32_t gb_smem[];
  uint32_t* shist = gb_smem;                                          // kGbSmemHist
  __shared__ uint32_t s_list[kGbList];         // open n of the sparse phase (tile offsets)
  __shared__ uint32_t s_open[3], s_cnt;
  const uint32_t tid = threadIdx.x, lane = tid & 31u;
  const uint64_t n_last = N & ~1ull;           // largest even n
  uint32_t lmax = 0;
  uint32_t chk = 0;                            // checks so far (the same in every thread)
  unsigned long long lsum = 0, lprobes = 0;
  for (uint32_t i = tid; i < kGbSmemHist; i += kGbThreads) shist[i] = 0;
  if (tid < 3) s_open[tid] = 0;
  __syncthreads();

  for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const uint64_t n0 = 6 + tile * 2ull * kGbTile;
    const uint64_t nmax = umin64(n_last, n0 + 2ull * (kGbTile - 1));
    const uint32_t tcount = (uint32_t)((nmax - n0) / 2 + 1);
    const uint64_t obase = 1 + tile * (uint64_t)kGbTile;     // (n0 - 4) / 2
    uint32_t U[kGbWords];
#pragma unroll
    for (int q = 0; q < kGbWords; ++q) {
      const uint32_t t0 = 32u * (tid * kGbWords + q);
      U[q] = t0 >= tcount ? 0u : (tcount - t0 >= 32 ? 0xFFFFFFFFu : ((1u << (tcount - t0)) - 1u));
    }
    bool exhausted = true;
    bool sparse = false;
    uint32_t pi = 0;
    if (tid == 0) s_cnt = 0;                   // list of the sparse phase (ordered by the first check's barrier)
    for (; pi < noddp; ++pi) {
      const uint32_t p = __ldg(oddp + pi);
      if (2ull * p > nmax) { exhausted = false; break; }
      if ((pi & 7u) == 0) {
        // the tile's open n, summed over the block into one of three
        // counters taken in turn over all checks of all tiles (the next one
        // is cleared here: every thread read it two checks ago, and nobody
        // adds to it before this check's barrier)
        const uint32_t r = chk++ % 3u;
        uint32_t mine = 0;
#pragma unroll
        for (int q = 0; q < kGbWords; ++q) mine += __popc(U[q]);
        mine = __reduce_add_sync(0xFFFFFFFFu, mine);
        if (lane == 0 && mine) atomicAdd(&s_open[r], mine);
        if (tid == 0) s_open[(r + 1u) % 3u] = 0;
        __syncthreads();
        const uint32_t open = s_open[r];
        if (open == 0) { exhausted = false; break; }
        if (open <= kGbList) { sparse = true; break; }
      }
      // bit j of this thread's word q is n = n0 + 2*(32*(4*tid + q) + j); its
      // partner n - p is odd bit base + 32*(4*tid + q) + j, so the thread's
      // four windows are five consecutive bitmap words shifted by base mod 32
      const int64_t base = ((int64_t)n0 - (int64_t)p - 1) / 2;   // exact: n0 even, p odd
      uint32_t nres = 0;
      if (any_open(U)) {
        const uint32_t* wp = odd + ((base >> 5) + (int64_t)(kGbWords * tid));
        const uint32_t sh = (uint32_t)base & 31u;
        uint32_t a[kGbWords + 1];
#pragma unroll
        for (int q = 0; q <= kGbWords; ++q) a[q] = __ldg(wp + q);
#pragma unroll
        for (int q = 0; q < kGbWords; ++q) {
          if (!U[q]) continue;
          ++lprobes;
          uint32_t hit = U[q] & __funnelshift_r(a[q], a[q + 1], sh);
          if (!hit) continue;
          U[q] &= ~hit;
          nres += __popc(hit);
          if (out.minp) {
            const uint64_t o = obase + 32u * (tid * kGbWords + q);
            do {
              const uint32_t j = (uint32_t)__ffs(hit) - 1u;
              hit &= hit - 1u;
              out.minp[o + j] = p;
            } while (hit);
          }
        }
      }
      // the n resolved at p, per warp: one histogram update
      if (nres) { lmax = max(lmax, p); lsum += (unsigned long long)p * nres; }
      const uint32_t wres = __reduce_add_sync(0xFFFFFFFFu, nres);
      if (lane == 0 && wres) {
        if (p < kGbSmemHist) atomicAdd(&shist[p], wres);
        else atomicAdd(&out.hist[p], (unsigned long long)wres);
      }
    }
    if (sparse) {
      // Few n are left open: gather them into a shared list, then eight
      // lanes per n test eight primes at a time (from the first prime not
      // yet tried) and take the smallest hit by a ballot.  Same bound as
      // above (2p <= the tile's largest n), same outputs.
#pragma unroll
      for (int q = 0; q < kGbWords; ++q) {
        uint32_t u = U[q];
        U[q] = 0;
        while (u) {
          const uint32_t j = (uint32_t)__ffs(u) - 1u;
          u &= u - 1u;
          s_list[atomicAdd(&s_cnt, 1u)] = 32u * (tid * kGbWords + q) + j;
        }
      }
      __syncthreads();
      const uint32_t cnt = s_cnt;
      // four n per warp at a time, eight lanes (eight primes per step) each,
      // so that four chains of loads are in flight
      const uint32_t warp = tid >> 5, sub = lane >> 3, sl = lane & 7u;
      const uint32_t smask = 0xFFu << (8u * sub);
      constexpr uint32_t kSlots = 4u * (kGbThreads / 32);
      uint32_t e = 4u * warp + sub;
      bool active = e < cnt;
      uint32_t t = active ? s_list[e] : 0u;
      uint32_t pj = pi;
      while (__any_sync(0xFFFFFFFFu, active)) {
        const uint64_t n = n0 + 2ull * t;
        const uint32_t pk = pj + sl;
        const bool listed = active && pk < noddp;
        const uint32_t p = listed ? __ldg(oddp + pk) : 0xFFFFFFFFu;
        const bool in = listed && 2ull * p <= nmax;
        bool ok = false;
        if (in && p < n) {                                         // n - p <= 0 is no prime
          const uint64_t bi = (n - p - 1) / 2;                    // odd bit of n - p, < N / 2
          ok = (__ldg(odd + (bi >> 5)) >> (uint32_t)(bi & 31u)) & 1u;
        }
        const uint32_t hit = __ballot_sync(0xFFFFFFFFu, ok) & smask;
        const uint32_t oob = __ballot_sync(0xFFFFFFFFu, listed && !in) & smask;
        const uint32_t ool = __ballot_sync(0xFFFFFFFFu, active && pk >= noddp) & smask;
        const uint32_t pm = __shfl_sync(0xFFFFFFFFu, p, hit ? __ffs(hit) - 1u : lane);
        if (active) {
          bool done = true;
          if (hit) {
            if (sl == 0) {
              if (out.minp) out.minp[obase + t] = pm;
              lmax = max(lmax, pm);
              lsum += pm;
              if (pm < kGbSmemHist) atomicAdd(&shist[pm], 1u);
              else atomicAdd(&out.hist[pm], 1ull);
            }
          } else if (oob | ool) {
            if (sl == 0) {
              // primes past the bound first: a counterexample; the list ended first: an error
              if (oob && (!ool || __ffs(oob) < __ffs(ool))) {
                const unsigned long long slot = atomicAdd(out.n_ce, 1ull);
                if (slot < out.ce_cap) out.ce[slot] = n;
              } else {
                atomicOr(out.err, 1u);
              }
            }
          } else {
            done = false;
            pj += 8u;
          }
          if (sl == 0) ++lprobes;
          if (done) {
            e += kSlots;
            active = e < cnt;
            t = active ? s_list[e] : 0u;
            pj = pi;
          }
        }
      }
      __syncthreads();                           // the list is reused by the next tile
    }
    // Whatever is left: counterexamples, unless the prime list ran out first.
#pragma unroll
    for (int q = 0; q < kGbWords; ++q) {
      uint32_t u = U[q];
      if (!u) continue;
      if (exhausted) { atomicOr(out.err, 1u); continue; }
      while (u) {
        const uint32_t j = (uint32_t)__ffs(u) - 1u;
        u &= u - 1u;
        const uint64_t n = n0 + 2ull * (32u * (tid * kGbWords + q) + j);
        const unsigned long long slot = atomicAdd(out.n_ce, 1ull);
        if (slot < out.ce_cap) out.ce[slot] = n;
      }
    }
  }
  __syncthreads();
  for (uint32_t i = tid; i < kGbSmemHist; i += kGbThreads)
    if (shist[i]) atomicAdd(&out.hist[i], (unsigned long long)shist[i]);
  lmax = __reduce_max_sync(0xFFFFFFFFu, lmax);
  if (lane == 0) atomicMax(out.max_minp, lmax);
  atomicAdd(out.sum_minp, lsum);
  atomicAdd(out.probes, lprobes);
}

__global__ void sophie_germain_kernel(const uint32_t* __restrict__ wb, uint64_t N,
                                      unsigned long long* __restrict__ count) {
  // bytes k with 30k + 11 <= N
  const uint64_t kmax = N >= 11 ? (N - 11) / 30 : 0;
  unsigned long long c = 0;
  if (N >= 11) {
    for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k <= kmax;
         k += (uint64_t)gridDim.x * blockDim.x) {
      const uint64_t base = 30 * k;
      if (wheel_bit(wb, k, 2) && wheel_bit(wb, 2 * k, 6)) ++c;                         // 11 -> 23
      if (base + 23 <= N && wheel_bit(wb, k, 6) && wheel_bit(wb, 2 * k + 1, 4)) ++c;  // 23 -> 47
      if (base + 29 <= N && wheel_bit(wb, k, 7) && wheel_bit(wb, 2 * k + 1, 7)) ++c;  // 29 -> 59
    }
  }
  c = __reduce_add_sync(0xFFFFFFFFu, (unsigned)c);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(count, c);
}

constexpr int kExThreads = 512;
constexpr int kExWords = 8;
constexpr uint32_t kExBlockWords = kExThreads * kExWords;

__global__ void extract_count_kernel(const uint32_t* __restrict__ wb, uint64_t nwords,
                                     uint32_t* __restrict__ block_counts) {
  const uint64_t w0 = blockIdx.x * (uint64_t)kExBlockWords + threadIdx.x * (uint64_t)kExWords;
  uint32_t c = 0;
#pragma unroll
  for (int i = 0; i < kExWords; ++i)
    if (w0 + i < nwords) c += __popc(wb[w0 + i]);
  c = __reduce_add_sync(0xFFFFFFFFu, c);
  __shared__ uint32_t s[kExThreads / 32];
  if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t t = 0;
    for (int i = 0; i < kExThreads / 32; ++i) t += s[i];
    block_counts[blockIdx.x] = t;
  }
}

__global__ void extract_write_kernel(const uint32_t* __restrict__ wb, uint64_t nwords,
                                     uint64_t k_lo, const uint64_t* __restrict__ block_offsets,
                                     uint64_t* __restrict__ out) {
  const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint64_t w0 = blockIdx.x * (uint64_t)kExBlockWords + tid * (uint64_t)kExWords;
  uint32_t words[kExWords];
  uint32_t c = 0;
#pragma unroll
  for (int i = 0; i < kExWords; ++i) {
    words[i] = (w0 + i < nwords) ? wb[w0 + i] : 0u;
    c += __popc(words[i]);
  }
  // block exclusive scan of c
  uint32_t incl = c;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, incl, d);
    if ((int)lane >= d) incl += t;
  }
  __shared__ uint32_t s[kExThreads / 32];
  if (lane == 31) s[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    uint32_t v = lane < kExThreads / 32 ? s[lane] : 0u;
    uint32_t iv = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, iv, d);
      if ((int)lane >= d) iv += t;
    }
    if (lane < kExThreads / 32) s[lane] = iv - v;
  }
  __syncthreads();
  uint64_t pos = block_offsets[blockIdx.x] + s[warp] + (incl - c);
#pragma unroll
  for (int i = 0; i < kExWords; ++i) {
    uint32_t w = words[i];
    const uint64_t kb = k_lo + 4 * (w0 + i);
    while (w) {
      const uint32_t b = (uint32_t)__ffs(w) - 1u;
      w &= w - 1u;
      out[pos++] = 30 * (kb + (b >> 3)) + (uint32_t)((kW30Packed >> ((b & 7u) << 3)) & 0xFFu);
    }
  }
}

// Sieve [0, limit] (or [a, b]) into a wheel bitmap on the device.
const uint32_t* sieve_bitmap(Engine& E, Plan& plan, uint64_t a, uint64_t b_excl, uint64_t* nwords) {
  plan.eng = &E;
  plan.device = E.device;
  plan.load(1, &a, &b_excl, kFlagBitmap);
  plan.launch(E.stream);
  *nwords = (plan.host_reqs[0].k_hi - plan.host_reqs[0].k_lo + 3) / 4;
  return plan.bitmap.as<uint32_t>();
}

std::vector<uint32_t> odd_primes_below(uint32_t limit) {
  std::vector<uint8_t> comp(limit + 1, 0);
  std::vector<uint32_t> v;
  for (uint32_t i = 2; i <= limit; ++i) {
    if (comp[i]) continue;
    if (i > 2) v.push_back(i);
    for (uint64_t j = (uint64_t)i * i; j <= limit; j += i) comp[j] = 1;
  }
  return v;
}

}  // namespace

struct GoldbachPlan {
  Engine* eng = nullptr;
  uint64_t N = 0;
  Plan sieve;
  DevBuf odd, oddp, minp, hist, scalars, ce;
  uint64_t odd_words = 0, ntiles = 0, ce_cap = 0;
  uint32_t grid = 0;
  bool want_minp = false;
};

GoldbachPlan* goldbach_plan_create(Engine& E, uint64_t N) {
  std::unique_ptr<GoldbachPlan> g(new GoldbachPlan());
  g->eng = &E;
  g->N = N;
  const std::vector<uint32_t> op = odd_primes_below(65535);
  g->oddp.reserve(op.size() * 4);
  check_cuda(cudaMemcpy(g->oddp.ptr, op.data(), op.size() * 4, cudaMemcpyHostToDevice), "odd primes");
  g->odd_words = (N / 2 + 1 + 31) / 32 + 2;
  g->odd.reserve((g->odd_words + 2 * kGbPad) * 4);
  g->hist.reserve(sizeof(unsigned long long) * kGoldbachHistBins);
  g->scalars.reserve(64);
  g->ce_cap = 1024;
  g->ce.reserve(8 * g->ce_cap);
  g->ntiles = N >= 6 ? ((N & ~1ull) - 6) / (2ull * kGbTile) + 1 : 0;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, goldbach_minp_kernel, kGbThreads, kGbSmemBytes) !=
          cudaSuccess || per_sm < 1)
    per_sm = 1;
  g->grid = (uint32_t)std::min<uint64_t>(g->ntiles, (uint64_t)E.sm_count * per_sm);
  g->sieve.eng = &E;
  g->sieve.timed = false;
  return g.release();
}

void goldbach_plan_launch(GoldbachPlan* g, cudaStream_t s) {
  Engine& E = *g->eng;
  // wheel bitmap of [0, N] (sieve kernel on the same stream)
  {
    uint64_t a = 0, b = g->N + 1;
    if (!g->sieve.nreq || g->sieve.host_reqs[0].b != b) g->sieve.load(1, &a, &b, kFlagBitmap);
    g->sieve.launch(s);
  }
  const uint32_t* wb = g->sieve.bitmap.as<uint32_t>();
  uint32_t* odd = g->odd.as<uint32_t>() + kGbPad;
  const uint64_t kbytes = (g->N + 1 + 29) / 30;          // wheel bytes of [0, N]
  odd_bitmap_kernel<<<E.sm_count * 8, 256, 0, s>>>(wb, kbytes, odd, g->odd_words - 2, g->N);
  check_cuda(cudaGetLastError(), "odd_bitmap_kernel");
  check_cuda(cudaMemsetAsync(g->odd.as<uint32_t>(), 0, 4 * kGbPad, s), "odd pad");
  check_cuda(cudaMemsetAsync(odd + (g->odd_words - 2), 0, 4 * (2 + kGbPad), s), "odd pad");
  check_cuda(cudaMemsetAsync(g->hist.ptr, 0, sizeof(unsigned long long) * kGoldbachHistBins, s), "hist");
  check_cuda(cudaMemsetAsync(g->scalars.ptr, 0, 64, s), "scalars");
  // n never resolved (a counterexample) keep min p = 0
  if (g->want_minp)
    check_cuda(cudaMemsetAsync(g->minp.ptr, 0, 4 * ((g->N - 4) / 2 + 1), s), "minp");
  if (!g->ntiles) return;
  auto* sc = g->scalars.as<unsigned long long>();
  GbOut o;
  o.minp = g->want_minp ? g->minp.as<uint32_t>() : nullptr;
  o.hist = g->hist.as<unsigned long long>();
  o.max_minp = reinterpret_cast<unsigned int*>(sc + 0);
  o.sum_minp = sc + 1;
  o.n_ce = sc + 2;
  o.probes = sc + 3;
  o.err = reinterpret_cast<unsigned int*>(sc + 4);
  o.ce = g->ce.as<unsigned long long>();
  o.ce_cap = g->ce_cap;
  static AttrCache attr;          // per device, thread-safe
  int dev = 0;
  check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
  check_cuda((cudaError_t)attr.ensure(dev, kGbSmemBytes, [](size_t n) {
               return (int)cudaFuncSetAttribute(goldbach_minp_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                (int)n);
             }), "goldbach smem");
  goldbach_minp_kernel<<<g->grid, kGbThreads, kGbSmemBytes, s>>>(odd, g->oddp.as<uint32_t>(), kGoldbachPrimes,
                                                                  g->N, g->ntiles, o);
  check_cuda(cudaGetLastError(), "goldbach_minp_kernel");
}

void goldbach_plan_fetch(GoldbachPlan* g, GoldbachResult* r, cudaStream_t s) {
  unsigned long long sc[5] = {0, 0, 0, 0, 0};
  r->hist.assign(kGoldbachHistBins, 0);
  check_cuda(cudaMemcpyAsync(sc, g->scalars.ptr, sizeof(sc), cudaMemcpyDeviceToHost, s), "scalars");
  check_cuda(cudaMemcpyAsync(r->hist.data(), g->hist.ptr, 8ull * kGoldbachHistBins,
                             cudaMemcpyDeviceToHost, s), "hist");
  check_cuda(cudaStreamSynchronize(s), "goldbach run");
  if (sc[4]) throw Error(VOSS_ERR_INTERNAL, "Goldbach: no prime below 65536 resolved some n");
  const uint64_t nce = sc[2];
  r->n_counterexamples = nce;
  const uint64_t keep = std::min<uint64_t>(nce, g->ce_cap);
  std::vector<uint64_t> ce(keep);
  if (keep) {
    check_cuda(cudaMemcpy(ce.data(), g->ce.ptr, 8 * keep, cudaMemcpyDeviceToHost), "ce");
    std::sort(ce.begin(), ce.end());
  }
  r->counterexamples = ce;
  r->hist[0] = 0;
  // n = 4 = 2 + 2 is outside the kernel's tiles
  r->max_minp = std::max<uint32_t>((uint32_t)sc[0], g->N >= 4 ? 2u : 0u);
  r->sum_minp = sc[1] + (g->N >= 4 ? 2 : 0);
  if (g->N >= 4) r->hist[2] += 1;
}

uint64_t goldbach_plan_probes(GoldbachPlan* g) {
  unsigned long long sc[5];
  check_cuda(cudaMemcpy(sc, g->scalars.ptr, sizeof(sc), cudaMemcpyDeviceToHost), "probes");
  return sc[3];
}

void goldbach_plan_free(GoldbachPlan* g) { delete g; }

GoldbachResult goldbach_run(Engine& E, uint64_t N, uint32_t* minp_host, uint64_t max_ce,
                            float* kernel_ms) {
  std::unique_ptr<GoldbachPlan> g(goldbach_plan_create(E, N));
  const uint64_t nn = (N - 4) / 2 + 1;
  if (minp_host) {
    g->want_minp = true;
    g->minp.reserve(4 * nn);
  }
  g->ce_cap = std::max<uint64_t>(std::min<uint64_t>(max_ce, 1ull << 24), 1);
  g->ce.reserve(8 * g->ce_cap);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (kernel_ms) {
    check_cuda(cudaEventCreate(&e0), "event");
    check_cuda(cudaEventCreate(&e1), "event");
    check_cuda(cudaEventRecord(e0, E.stream), "event");
  }
  goldbach_plan_launch(g.get(), E.stream);
  if (kernel_ms) check_cuda(cudaEventRecord(e1, E.stream), "event");
  GoldbachResult r;
  goldbach_plan_fetch(g.get(), &r, E.stream);
  if (kernel_ms) {
    check_cuda(cudaEventElapsedTime(kernel_ms, e0, e1), "event");
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
  }
  if (minp_host) {
    check_cuda(cudaMemcpy(minp_host, g->minp.ptr, 4 * nn, cudaMemcpyDeviceToHost), "minp");
    minp_host[0] = 2;  // n = 4
  }
  if (r.counterexamples.size() > max_ce) r.counterexamples.resize(max_ce);
  return r;
}

uint64_t sophie_germain_count(Engine& E, uint64_t N) {
  uint64_t seeds = (N >= 2) + (N >= 3) + (N >= 5);
  if (N < 11) return seeds;
  Plan plan;
  uint64_t nw = 0;
  const uint32_t* wb = sieve_bitmap(E, plan, 0, 2 * N + 2, &nw);
  DevBuf cnt;
  cnt.reserve(8);
  check_cuda(cudaMemsetAsync(cnt.ptr, 0, 8, E.stream), "memset");
  sophie_germain_kernel<<<E.sm_count * 8, 256, 0, E.stream>>>(wb, N, cnt.as<unsigned long long>());
  check_cuda(cudaGetLastError(), "sophie_germain_kernel");
  unsigned long long c = 0;
  check_cuda(cudaMemcpyAsync(&c, cnt.ptr, 8, cudaMemcpyDeviceToHost, E.stream), "count");
  check_cuda(cudaStreamSynchronize(E.stream), "sophie germain");
  return seeds + c;
}

std::vector<uint64_t> primes_in_range(Engine& E, uint64_t a, uint64_t b, uint64_t max_count) {
  std::vector<uint64_t> seeds;
  for (uint64_t q : {2ull, 3ull, 5ull}) if (q >= a && q <= b) seeds.push_back(q);
  if (b < 7) return seeds;
  // count first, so an oversized request fails before any bitmap is built
  uint64_t aa = a, bb = b + 1;
  const uint64_t total = E.run(1, &aa, &bb, nullptr, false)[0].count;
  if (total > max_count) return std::vector<uint64_t>(max_count + 1, 0);
  Plan plan;
  uint64_t nw = 0;
  const uint32_t* wb = sieve_bitmap(E, plan, a, b + 1, &nw);
  const uint64_t nblocks = (nw + kExBlockWords - 1) / kExBlockWords;
  DevBuf bc, bo, outb;
  bc.reserve(4 * std::max<uint64_t>(nblocks, 1));
  bo.reserve(8 * std::max<uint64_t>(nblocks, 1));
  std::vector<uint64_t> res(seeds);
  if (nblocks) {
    extract_count_kernel<<<(unsigned)nblocks, kExThreads, 0, E.stream>>>(wb, nw, bc.as<uint32_t>());
    check_cuda(cudaGetLastError(), "extract_count_kernel");
    std::vector<uint32_t> counts(nblocks);
    check_cuda(cudaMemcpyAsync(counts.data(), bc.ptr, 4 * nblocks, cudaMemcpyDeviceToHost, E.stream), "counts");
    check_cuda(cudaStreamSynchronize(E.stream), "counts");
    std::vector<uint64_t> offs(nblocks);
    uint64_t t = 0;
    for (uint64_t i = 0; i < nblocks; ++i) { offs[i] = t; t += counts[i]; }
    if (t) {
      check_cuda(cudaMemcpyAsync(bo.ptr, offs.data(), 8 * nblocks, cudaMemcpyHostToDevice, E.stream), "offsets");
      outb.reserve(8 * t);
      extract_write_kernel<<<(unsigned)nblocks, kExThreads, 0, E.stream>>>(
          wb, nw, plan.host_reqs[0].k_lo, bo.as<uint64_t>(), outb.as<uint64_t>());
      check_cuda(cudaGetLastError(), "extract_write_kernel");
      res.resize(seeds.size() + t);
      check_cuda(cudaMemcpyAsync(res.data() + seeds.size(), outb.ptr, 8 * t, cudaMemcpyDeviceToHost, E.stream), "primes");
    }
    check_cuda(cudaStreamSynchronize(E.stream), "in_range");
  }
  return res;
}

}  // namespace vg
