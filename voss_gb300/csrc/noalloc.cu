// noalloc.cu -- range statistics without any device allocation.
//
// Some callers cannot allocate device memory once they are running: a
// process whose device memory is already owned by another framework's
// caching allocator (PyTorch, for one) and kept near full, or a
// latency-critical loop in which cudaMalloc / cudaFree would synchronize the
// device and stall every other stream.  voss_primes_range_stats_noalloc
// serves them: it runs the same sieve and finalize kernels as
// voss_primes_range_stats, but every byte of device memory it uses beyond
// the caller's output lives in file-scope static __device__ arrays below
// (about 29.9 MB per GPU that loads this library, held until the process
// exits: 24.1 MB of presieve tile copies, 3.6 MB of sieving-prime table and
// 2.2 MB of scratch).  It calls no cudaMalloc, cudaFree or allocating library
// routine.
//
// Limits (checked, VOSS_ERR_OUT_OF_RANGE beyond them): b <= 2^40, and at
// most kNaMaxSegs segments of 221184 bytes (30 integers each), i.e. a range
// width of at most about 4.3 * 10^11.
//
// The first call on a device sets that device up (tables copied into the
// static arrays, kernel attributes raised); make that first call before any
// stream capture.  Every call shares the one scratch array and leaves its
// contents behind; the init kernel clears what must start at zero, so calls
// in sequence are independent, but calls that overlap on the GPU (different
// streams, or different host threads at once) race on the scratch and give
// wrong results.
//
// Errors: the call returns once its kernels are enqueued.  A launch that is
// refused shows in its return code; a fault while the kernels run surfaces
// on the caller's next synchronisation of the stream.  An error already
// pending on the calling thread when the call starts is left in place for
// the caller to read, and the call returns VOSS_ERR_CUDA without launching.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>

#include "engine.h"
#include "voss/voss.h"
#include "voss/voss_gb300.h"

namespace vg {
namespace {

constexpr uint32_t kNaSegBytes = 221184;           // largest segment
constexpr uint32_t kNaMaxSegs = 65536;
constexpr uint64_t kNaMaxB = 1ull << 40;
constexpr uint32_t kNaPrimeLimit = 1u << 20;        // sieving primes, p*p < 2^40
constexpr uint32_t kNaPrimes = 82008;               // primes in [61, 2^20)
constexpr uint32_t kNaStride = 82016;               // kNaPrimes rounded up to 32
constexpr uint32_t kNaLargeCap = 4096;
// All tiles in one block: tile t is kTileShifts copies of
// tile_copy_stride(tile_period(t), kNaSegBytes) bytes, from byte
// na_tile_offset(t).
constexpr uint64_t na_tile_offset(int t) {
  uint64_t off = 0;
  for (int i = 0; i < t; ++i) off += (uint64_t)kTileShifts * tile_copy_stride(tile_period(i), kNaSegBytes);
  return off;
}
constexpr uint64_t kNaTileBytes = na_tile_offset(kTiles);

struct NaScratch {
  BatchHdr hdr;
  unsigned long long queue;
  unsigned int nlarge;
  unsigned int pad;
  ReqDesc req;
  ReqAccum acc;
  ReqResult res;
  LargeGapRec large[kNaLargeCap];
  SegRec segs[kNaMaxSegs];
};

// The scratch of every call (about 2.2 MB), the sieving-prime table (P, M
// and R: about 3.6 MB) and the presieve tile copies (about 24.1 MB).  In
// host code these names are host-side stand-ins; their device addresses
// come from cudaGetSymbolAddress at set-up.
static __device__ __align__(256) unsigned char g_na_scratch[sizeof(NaScratch)];
static __device__ __align__(256) uint32_t g_na_P[kNaStride];
static __device__ __align__(256) uint64_t g_na_M[kNaStride];
static __device__ __align__(256) uint32_t g_na_R[8 * kNaStride];
static __device__ __align__(256) uint32_t g_na_tiles[kNaTileBytes / 4];

// Host copies of the tables, built once per process in static storage.
static uint32_t h_P[kNaStride];
static uint64_t h_M[kNaStride];
static uint32_t h_R[8 * kNaStride];
static uint8_t h_tiles[kNaTileBytes];
static uint8_t h_tile_base[kMaxTilePeriod];    // one period of a tile
static uint8_t h_comp[kNaPrimeLimit];
static bool h_built = false;

struct NaDevice {
  bool ready = false;
  NaScratch* scratch = nullptr;
  uint32_t *P = nullptr, *R = nullptr, *tiles = nullptr;
  uint64_t* M = nullptr;
  uint32_t sms = 0;
};
static NaDevice g_dev[64];
static std::mutex g_mu;

const uint32_t kW30h[8] = {1, 7, 11, 13, 17, 19, 23, 29};

int64_t inv_mod(int64_t a, int64_t m) {
  int64_t t = 0, nt = 1, r = m, nr = a % m;
  while (nr) {
    const int64_t q = r / nr;
    int64_t x = nt; nt = t - q * nt; t = x;
    x = nr; nr = r - q * nr; r = x;
  }
  return t < 0 ? t + m : t;
}

void build_host_tables() {
  if (h_built) return;
  std::memset(h_comp, 0, sizeof(h_comp));
  for (uint32_t i = 2; (uint64_t)i * i < kNaPrimeLimit; ++i)
    if (!h_comp[i])
      for (uint32_t j = i * i; j < kNaPrimeLimit; j += i) h_comp[j] = 1;
  uint32_t n = 0;
  for (uint32_t i = kFirstTablePrime; i < kNaPrimeLimit; ++i) {
    if (h_comp[i]) continue;
    const uint64_t p = i;
    h_P[n] = i;
    h_M[n] = UINT64_MAX / p;
    const uint64_t inv30 = (uint64_t)inv_mod((int64_t)(30 % p), (int64_t)p);
    for (int o = 0; o < 8; ++o) h_R[8 * n + o] = (uint32_t)(((p - kW30h[o] % p) % p) * inv30 % p);
    ++n;
  }
  for (int t = 0; t < kTiles; ++t)
    build_tile_copies(kTilePrimes[t], kTilePrimes[t][3] ? 4 : 3, tile_period(t),
                      tile_copy_stride(tile_period(t), kNaSegBytes), h_tile_base, h_tiles + na_tile_offset(t));
  h_built = (n == kNaPrimes);
}

template <class T>
cudaError_t symbol_ptr(T** out, const void* sym) {
  return cudaGetSymbolAddress(reinterpret_cast<void**>(out), sym);
}

// Per-device set-up, with that device current.  Returns VOSS_OK or a code.
int setup(int dev) {
  std::lock_guard<std::mutex> g(g_mu);
  NaDevice& d = g_dev[dev];
  if (d.ready) return VOSS_OK;
  build_host_tables();
  if (!h_built) return VOSS_ERR_INTERNAL;
  if (symbol_ptr(&d.scratch, g_na_scratch) != cudaSuccess || symbol_ptr(&d.P, g_na_P) != cudaSuccess ||
      symbol_ptr(&d.M, g_na_M) != cudaSuccess || symbol_ptr(&d.R, g_na_R) != cudaSuccess ||
      symbol_ptr(&d.tiles, g_na_tiles) != cudaSuccess)
    return VOSS_ERR_CUDA;
  if (cudaMemcpyToSymbol(g_na_P, h_P, sizeof(h_P)) != cudaSuccess ||
      cudaMemcpyToSymbol(g_na_M, h_M, sizeof(h_M)) != cudaSuccess ||
      cudaMemcpyToSymbol(g_na_R, h_R, sizeof(h_R)) != cudaSuccess ||
      cudaMemcpyToSymbol(g_na_tiles, h_tiles, sizeof(h_tiles)) != cudaSuccess)
    return VOSS_ERR_CUDA;
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
    return VOSS_ERR_CUDA;
  d.sms = (uint32_t)sms;
  SieveParams prm{};
  prm.seg_bytes = kNaSegBytes;
  if (launch_sieve(prm, 0, 1024, nullptr) != cudaSuccess) return VOSS_ERR_CUDA;   // attributes only
  d.ready = true;
  return VOSS_OK;
}

// Writes the request and clears the accumulators of the shared scratch.
__global__ void na_init_kernel(NaScratch* s, ReqDesc r) {
  if (threadIdx.x == 0) {
    s->hdr.total_segs = r.nseg;
    s->hdr.nreq = 1;
    s->hdr.nfill = 0;
    s->hdr.nout = 0;
    s->queue = 0;
    s->nlarge = 0;
    s->req = r;
  }
  unsigned long long* acc = reinterpret_cast<unsigned long long*>(&s->acc);
  for (uint32_t i = threadIdx.x; i < sizeof(ReqAccum) / 8; i += blockDim.x) acc[i] = 0;
}

// ReqResult -> voss_range_stats_t (the host conversion of the other entry
// points, done on the device so the output can live anywhere the GPU writes).
__global__ void na_pack_kernel(const NaScratch* s, uint64_t a, uint64_t b, voss_range_stats_t* o) {
  const ReqResult& r = s->res;
  __shared__ unsigned long long over, large;
  if (threadIdx.x == 0) { over = 0; large = 0; }
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < (uint32_t)kHistBins; i += blockDim.x) {
    const uint64_t h = r.hist[i];
    if (i < VOSS_GAP_BINS - 1) o->gap_hist[i] = h;
    else if (h) atomicAdd(&over, (unsigned long long)h);
    if (i >= kLargeGap / 2 && h) atomicAdd(&large, (unsigned long long)h);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    o->a = a; o->b = b; o->count = r.count;
    o->twins = r.hist[1]; o->cousins = r.hist[2]; o->sexy = r.hist[3];
    o->pi_4_1 = r.c41; o->pi_4_3 = r.c43; o->pi_3_1 = r.c31; o->pi_3_2 = r.c32;
    o->first_prime = r.first; o->last_prime = r.last;
    o->max_gap = r.max_gap; o->max_gap_start = r.max_gap_start;
    o->num_gaps = r.num_gaps; o->large_gaps = large;
    o->gap_hist[VOSS_GAP_BINS - 1] = over;
  }
}

}  // namespace
}  // namespace vg

extern "C" int voss_primes_range_stats_noalloc(uint64_t a, uint64_t b, voss_range_stats_t* out,
                                               void* stream) {
  using namespace vg;
  if (!out) return VOSS_ERR_INVALID_ARG;
  if (b > kNaMaxB) return VOSS_ERR_OUT_OF_RANGE;
  // an error left by earlier work on this thread stays for its owner to
  // read (the launch checks below would otherwise take it as this call's)
  if (cudaPeekAtLastError() != cudaSuccess) return VOSS_ERR_CUDA;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return VOSS_ERR_NO_CUDA;
  const int rc = setup(dev);
  if (rc != VOSS_OK) return rc;
  const NaDevice& d = g_dev[dev];

  ReqDesc r{};
  r.a = a;
  r.b = b;
  r.rflags = kReqGaps;
  r.seg_bytes = kNaSegBytes;
  if (b > a) {
    r.k_lo = a / 30;
    r.k_hi = (b + 29) / 30;
    const uint64_t bytes = r.k_hi - r.k_lo;
    // whole waves of one CTA per SM, as the other entry points tune a range
    const uint64_t waves = (bytes + (uint64_t)d.sms * kNaSegBytes - 1) / ((uint64_t)d.sms * kNaSegBytes);
    uint64_t want = std::max<uint64_t>((bytes + waves * d.sms - 1) / (waves * d.sms), 16384);
    r.seg_bytes = (uint32_t)std::min<uint64_t>(kNaSegBytes, (want + 127) & ~127ull);
    r.nseg = (bytes + r.seg_bytes - 1) / r.seg_bytes;
    if (r.nseg > kNaMaxSegs) return VOSS_ERR_OUT_OF_RANGE;
    const uint64_t lim = isqrt_u64(b - 1);            // primes with p*p < b
    r.nprimes = (uint32_t)(std::upper_bound(h_P, h_P + kNaPrimes, (uint32_t)std::min<uint64_t>(lim, UINT32_MAX)) - h_P);
    const uint32_t split = std::max<uint32_t>(kFirstTablePrime, std::min<uint32_t>(6144, r.seg_bytes / 32));
    r.tier_split = (uint32_t)(std::lower_bound(h_P, h_P + kNaPrimes, split) - h_P);
    r.tier_huge = (uint32_t)(std::lower_bound(h_P, h_P + kNaPrimes, r.seg_bytes) - h_P);
  }
  r.bucket_idx = r.nprimes;          // no bucket lists on this path
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  NaScratch* sc = d.scratch;
  na_init_kernel<<<1, 256, 0, s>>>(sc, r);
  if (cudaGetLastError() != cudaSuccess) return VOSS_ERR_CUDA;

  SieveParams prm{};
  prm.reqs = &sc->req;
  prm.hdr = &sc->hdr;
  prm.queue = &sc->queue;
  prm.P = d.P;
  prm.M = d.M;
  prm.R = d.R;
  for (int t = 0; t < kTiles; ++t) {
    prm.tile[t] = d.tiles + na_tile_offset(t) / 4;
    prm.tile_stride16[t] = tile_copy_stride(tile_period(t), kNaSegBytes) / 16;
  }
  prm.seg_bytes = kNaSegBytes;
  prm.segs = sc->segs;
  prm.acc = &sc->acc;
  prm.large = sc->large;
  prm.n_large = &sc->nlarge;
  prm.large_cap = kNaLargeCap;
  prm.flags = 0;
  prm.bitmap = nullptr;
  const uint32_t grid = (uint32_t)std::min<uint64_t>(r.nseg, d.sms);
  if (grid && launch_sieve(prm, grid, 1024, s) != cudaSuccess) return VOSS_ERR_CUDA;
  if (launch_finalize(&sc->req, &sc->hdr, sc->segs, &sc->acc, sc->large, &sc->nlarge, kNaLargeCap,
                      &sc->res, 1, s) != cudaSuccess)
    return VOSS_ERR_CUDA;
  na_pack_kernel<<<1, 256, 0, s>>>(sc, a, b, out);
  if (cudaGetLastError() != cudaSuccess) return VOSS_ERR_CUDA;
  return VOSS_OK;
}
