// engine.cpp -- host side of the GB300 sieve.
//
// Replaces the reference's per-call host orchestration
// (library/src/primes/context.cu:212-559, prime_count.cu:141-293,
// range.cu:99-262).  Differences by design:
//   * the sieving-prime table (primes >= 61, with Barrett constants and the
//     eight residue-class starts of each prime) is built once per process and
//     stays resident on the device, growing on demand up to sqrt(10^14+10^10);
//   * a run is two kernel launches for any number of ranges and segments,
//     with no per-segment host work, no per-prime launches and no
//     synchronisation until the results are read;
//   * all buffers are reused across calls (grow-only).
#include "engine.h"

#include <algorithm>
#include <cstring>
#include <memory>
#include <numeric>

#include "voss/voss.h"

namespace vg {

void check_cuda(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    int code = (e == cudaErrorMemoryAllocation) ? VOSS_ERR_OUT_OF_MEMORY
             : (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) ? VOSS_ERR_NO_CUDA
             : VOSS_ERR_CUDA;
    throw Error(code, std::string(what) + ": " + cudaGetErrorString(e));
  }
}

uint64_t isqrt_u64(uint64_t x) {
  uint64_t lo = 0, hi = 1ull << 32;
  while (lo < hi) {
    const uint64_t mid = lo + (hi - lo + 1) / 2;
    if (mid <= x / mid) lo = mid; else hi = mid - 1;
  }
  return lo;
}

void DevBuf::reserve(size_t n) {
  if (n <= bytes && ptr) return;
  release();
  size_t want = std::max<size_t>(n, 256);
  check_cuda(cudaMalloc(&ptr, want), "cudaMalloc");
  bytes = want;
}

void DevBuf::release() {
  if (ptr) cudaFree(ptr);
  ptr = nullptr;
  bytes = 0;
}

void HostPinned::reserve(size_t n) {
  if (n <= bytes && ptr) return;
  if (ptr) cudaFreeHost(ptr);
  ptr = nullptr;
  bytes = 0;
  size_t want = std::max<size_t>(n, 256);
  check_cuda(cudaMallocHost(&ptr, want), "cudaMallocHost");
  bytes = want;
}

HostPinned::~HostPinned() {
  if (ptr) cudaFreeHost(ptr);
}

static const uint32_t kW30[8] = {1, 7, 11, 13, 17, 19, 23, 29};

static int64_t inverse_mod(int64_t a, int64_t m) {
  int64_t t = 0, nt = 1, r = m, nr = a % m;
  while (nr) {
    const int64_t q = r / nr;
    int64_t tmp = nt; nt = t - q * nt; t = tmp;
    tmp = nr; nr = r - q * nr; r = tmp;
  }
  return t < 0 ? t + m : t;
}

Engine& Engine::for_current_device() {
  static std::mutex reg_mu;
  static std::vector<std::unique_ptr<Engine>> engines;
  int dev = 0;
  check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
  std::lock_guard<std::mutex> g(reg_mu);
  if ((int)engines.size() <= dev) engines.resize(dev + 1);
  if (!engines[dev]) {
    std::unique_ptr<Engine> e(new Engine());
    e->device = dev;
    e->init();
    engines[dev] = std::move(e);
  }
  return *engines[dev];
}

void Engine::init() {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) throw Error(VOSS_ERR_NO_CUDA, "No CUDA device available");
  cudaDeviceProp prop;
  check_cuda(cudaGetDeviceProperties(&prop, device), "cudaGetDeviceProperties");
  sm_count = (uint32_t)prop.multiProcessorCount;
  // room for the sieve kernel's dynamic shared memory: the opt-in limit
  // less the kernel's own static shared memory
  max_smem_optin = prop.sharedMemPerBlockOptin - sieve_static_smem_bytes();
  name = prop.name;
  check_cuda(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "cudaStreamCreate");
  // Fit the default segment into what this device offers.
  while (sieve_smem_bytes(cfg.seg_bytes, cfg.threads) > max_smem_optin && cfg.seg_bytes > 16384)
    cfg.seg_bytes -= 8192;
  build_tiles();
  scratch.eng = this;
  scratch.device = device;
  scratch.timed = false;           // the one-call path reads no kernel times
  // the offset-regime table measured by voss_gb300/autotune.py on GB300
  static const TuneEntry kBuiltin[] = {
#include "tune_table.inc"
  };
  for (const TuneEntry& t : kBuiltin)
    if (t.seg_bytes) tuning.push_back(t);
  ensure_table(65536);
}

void Engine::build_tiles() {
  std::vector<uint8_t> base(kMaxTilePeriod);
  for (int t = 0; t < kTiles; ++t) {
    const uint32_t period = tile_period(t);
    const uint32_t stride = tile_copy_stride(period, kMaxSegBytes);
    const int nps = kTilePrimes[t][3] ? 4 : 3;
    std::vector<uint8_t> copies((size_t)kTileShifts * stride);
    build_tile_copies(kTilePrimes[t], nps, period, stride, base.data(), copies.data());
    tile[t].reserve(copies.size());
    check_cuda(cudaMemcpy(tile[t].ptr, copies.data(), copies.size(), cudaMemcpyHostToDevice), "tile upload");
  }
}

void Engine::ensure_table(uint64_t pmax) {
  if (pmax <= table_limit) return;
  uint64_t lim = std::max<uint64_t>(pmax, std::min<uint64_t>(2 * table_limit, isqrt_u64(kMaxB) + 64));
  lim = std::max<uint64_t>(lim, 4096);
  // plain byte sieve of [0, lim]
  std::vector<uint8_t> comp(lim + 1, 0);
  for (uint64_t i = 2; i * i <= lim; ++i)
    if (!comp[i])
      for (uint64_t j = i * i; j <= lim; j += i) comp[j] = 1;
  std::vector<uint32_t> P;
  P.reserve(lim / 10 + 16);
  for (uint64_t i = kFirstTablePrime; i <= lim; ++i)
    if (!comp[i]) P.push_back((uint32_t)i);
  const size_t n = P.size();
  std::vector<uint64_t> M(n);
  std::vector<uint32_t> R(8 * n, 0);        // the eight class residues of a prime together
  for (size_t i = 0; i < n; ++i) {
    const uint64_t p = P[i];
    M[i] = UINT64_MAX / p;
    const uint64_t inv30 = (uint64_t)inverse_mod((int64_t)(30 % p), (int64_t)p);
    for (int o = 0; o < 8; ++o)
      R[8 * i + o] = (uint32_t)(((p - kW30[o] % p) % p) * inv30 % p);
  }
  // The sieve kernel reads the first kConstPrimes entries from its own
  // compile-time copy; the two must agree.
  static constexpr ConstPrimeTable kConstTable = make_const_prime_table();
  for (size_t i = 0; i < std::min<size_t>(n, kConstPrimes); ++i)
    if (P[i] != kConstTable.p[i] || M[i] != kConstTable.m[i])
      throw Error(VOSS_ERR_INTERNAL, "prime table differs from the kernel's constant table");
  // Plans built earlier keep pointers to the current table: it is retired,
  // not freed, and stays valid for them.
  for (DevBuf* d : {&dP, &dM, &dR}) {
    if (!d->ptr) continue;
    std::unique_ptr<DevBuf> old(new DevBuf());
    old->ptr = d->ptr;
    old->bytes = d->bytes;
    d->ptr = nullptr;
    d->bytes = 0;
    retired_tables.push_back(std::move(old));
  }
  dP.reserve(std::max<size_t>(n, 1) * 4);
  dM.reserve(std::max<size_t>(n, 1) * 8);
  dR.reserve(std::max<size_t>(n, 1) * 8 * 4);
  if (n) {
    check_cuda(cudaMemcpy(dP.ptr, P.data(), n * 4, cudaMemcpyHostToDevice), "table P");
    check_cuda(cudaMemcpy(dM.ptr, M.data(), n * 8, cudaMemcpyHostToDevice), "table M");
    check_cuda(cudaMemcpy(dR.ptr, R.data(), R.size() * 4, cudaMemcpyHostToDevice), "table R");
  }
  hInvPrefix.assign(n + 1, 0.0);
  for (size_t i = 0; i < n; ++i) hInvPrefix[i + 1] = hInvPrefix[i] + 1.0 / (double)P[i];
  hP.swap(P);
  table_limit = lim;
}

uint32_t Engine::primes_below_sq(uint64_t b) const {
  if (b <= 1) return 0;
  const uint64_t r = isqrt_u64(b - 1);     // p*p < b  <=>  p <= isqrt(b-1)
  return (uint32_t)(std::upper_bound(hP.begin(), hP.end(), (uint64_t)std::min<uint64_t>(r, UINT32_MAX),
                                     [](uint64_t v, uint32_t p) { return v < p; }) - hP.begin());
}

uint32_t Engine::index_of(uint32_t p) const {
  return (uint32_t)(std::lower_bound(hP.begin(), hP.end(), p) - hP.begin());
}

Config Engine::tuned_for(uint64_t a, uint64_t b, bool batch) const {
  Config c = cfg;
  if (!cfg.auto_tune) return c;
  const uint64_t width = b > a ? b - a : 0;
  const uint64_t bytes = width / 30 + 1;
  // Offset regime: the table gives the largest segment and the tier split
  // measured best for ranges ending below b_max and no wider than width_max.
  uint32_t s = cfg.seg_bytes;
  uint32_t split = 0;
  c.bucket_split = 0;
  for (const TuneEntry& t : tuning) {
    if (b <= t.b_max && width <= t.width_max) {
      s = std::min<uint32_t>(std::max<uint32_t>(t.seg_bytes, 1024), cfg.seg_bytes) & ~127u;
      split = std::max<uint32_t>(kFirstTablePrime, t.tier_split);
      c.bucket_split = t.bucket_split;
      break;
    }
  }
  // Alone, a range should fill the GPU in whole waves: the segment shrinks
  // until the segments come in full waves of one CTA per SM (not below 16 KiB,
  // where the per-prime setup dominates).  In a batch other ranges fill the
  // GPU, so the largest segment is the cheapest.
  if (batch) {
    s = cfg.seg_bytes;
  } else {
    const uint64_t g = (uint64_t)sm_count * cfg.ctas_per_sm;
    const uint64_t waves = (bytes + g * s - 1) / (g * s);
    uint64_t want = (bytes + waves * g - 1) / (waves * g);
    want = std::max<uint64_t>(want, 16384);
    s = (uint32_t)std::min<uint64_t>(s, (want + 127) & ~127ull);
  }
  c.seg_bytes = s;
  // Without a table entry the warp-per-prime tier ends where a class has
  // about 32 hits per segment.
  c.tier_split = split ? split
                       : std::max<uint32_t>(kFirstTablePrime, std::min<uint32_t>(cfg.tier_split, s / 32));
  return c;
}

BucketPlan Engine::bucket_plan(const Config& c, uint64_t b, uint32_t nprimes, uint64_t nseg,
                               uint32_t seg_bytes) const {
  BucketPlan bp{nprimes, 0};
  // Lists pay off when most (prime, segment) pairs have no hit: primes well
  // above the segment, a request of several segments (one fill pass replaces
  // a setup per prime per segment), few enough segments for the fill
  // kernel's shared counts.
  if (!c.bucket_split || nseg < 2 || b < 2) return bp;
  const uint32_t from = std::max<uint32_t>(c.bucket_split, seg_bytes);
  const uint32_t idx = index_of(from);
  if (idx >= nprimes) return bp;
  // expected entries per segment: 8 * S * sum(1/p) over the bucket primes;
  // the capacity leaves a margin of many standard deviations
  const double mean = 8.0 * seg_bytes * (hInvPrefix[nprimes] - hInvPrefix[idx]);
  const double cap = (mean * 1.25 + 32.0 * std::sqrt(mean) + 1024.0) * cfg.bucket_cap_pct / 100.0;
  const uint32_t c32 = std::max<uint32_t>(32u, ((uint32_t)cap + 31u) & ~31u);
  // the fill kernel indexes a window's lists with 32-bit offsets
  if ((uint64_t)c32 * std::min<uint64_t>(nseg, kMaxBucketSegs) >= (1ull << 32)) return bp;
  bp.bucket_idx = idx;
  bp.cap = c32;
  return bp;
}

// ---------------------------------------------------------------------------
// Plan
// ---------------------------------------------------------------------------
static uint64_t round16(uint64_t bytes) { return (bytes + 15) & ~uint64_t(15); }

void Plan::reserve_capacity(uint32_t max_req, uint64_t max_segs, uint64_t max_bucket_entries) {
  cap_req = std::max<uint32_t>(max_req, 1);
  cap_segs = std::max<uint64_t>(max_segs, 1);
  if (share) {
    cap_out = cap_req;
    cap_req = 2 * cap_out;
    cap_segs += 4ull * cap_out;
    spans.reserve(sizeof(ReqSpan) * cap_out);
    apos.reserve(sizeof(uint32_t) * cap_req);
    rres.reserve(sizeof(ReqResult) * cap_out);
  }
  cap_bucket = max_bucket_entries;
  cap_fill = max_bucket_entries ? 65536u : 0u;
  if (cap_bucket) bucket.reserve(4 * cap_bucket);
  if (cap_fill) fills.reserve(sizeof(FillItem) * cap_fill);
  bcount.reserve(round16(4 * cap_segs));
  hdr.reserve(sizeof(BatchHdr) + sizeof(ReqDesc) * cap_req);
  ctl.reserve(sizeof(PlanCtl));
  segs.reserve(sizeof(SegRec) * cap_segs);
  acc.reserve(sizeof(ReqAccum) * cap_req);
  results.reserve(sizeof(ReqResult) * cap_req);
  stage.reserve(sizeof(BatchHdr) + sizeof(ReqDesc) * cap_req);
  host_results.reserve(sizeof(ReqResult) * cap_req);
}

uint64_t Plan::bucket_bytes_for(uint64_t a, uint64_t b) const {
  return allow_buckets ? list_bytes_for(a, b) : 0;
}

uint64_t Plan::list_bytes_for(uint64_t a, uint64_t b) const {
  if (b <= a) return 0;
  Engine& E = *eng;
  const Config c = E.tuned_for(a, b, batch_mode);
  const uint64_t bytes = (b + 29) / 30 - a / 30;
  const uint64_t nseg = (bytes + c.seg_bytes - 1) / c.seg_bytes;
  // plans of many requests hold every request's lists at once (no windows)
  if (nseg > kMaxBucketSegs) return 0;
  const BucketPlan bp = E.bucket_plan(c, b, E.primes_below_sq(b), nseg, c.seg_bytes);
  return bp.cap ? 4ull * bp.cap * nseg : 0;
}

uint32_t Plan::kernels_per_run() const {
  if (!nreq) return 0;
  const uint32_t fixed = kKernels + ((cap_req ? cap_out : nout) ? 1u : 0u);
  if (!wins.empty()) {
    uint32_t k = fixed - 1u;                 // zero + finalize (+ combine)
    for (const Window& W : wins) k += 1u + (W.fill_hi > W.fill_lo ? 1u : 0u);
    return k;
  }
  return fixed + ((cap_req ? cap_fill : nfill) ? 1u : 0u);
}

uint32_t Plan::fill_grid_max() const {
  return eng->sm_count * bucket_fill_ctas_per_sm();
}

bool Plan::overflowed() const {
  return nfill && host_flag.ptr && *static_cast<const unsigned int*>(host_flag.ptr) != 0;
}

uint64_t Plan::segments_for(uint64_t a, uint64_t b) const {
  if (b <= a) return 0;
  const Config c = eng->tuned_for(a, b, batch_mode);
  const uint64_t bytes = (b + 29) / 30 - a / 30;
  return (bytes + c.seg_bytes - 1) / c.seg_bytes;
}

void cut_ranges(uint32_t n, const uint64_t* a, const uint64_t* b, const uint32_t* rflags,
                std::vector<uint64_t>& atom_a, std::vector<uint64_t>& atom_b,
                std::vector<uint32_t>& atom_rf, std::vector<ReqSpan>& spans) {
  // every endpoint, once, in order; the elementary pieces lie between them
  std::vector<uint64_t> pts;
  pts.reserve(2 * (size_t)n);
  for (uint32_t i = 0; i < n; ++i)
    if (b[i] > a[i]) { pts.push_back(a[i]); pts.push_back(b[i]); }
  std::sort(pts.begin(), pts.end());
  pts.erase(std::unique(pts.begin(), pts.end()), pts.end());
  const size_t np = pts.size();
  // coverage of each piece (all requests, and those that want gaps) by
  // difference arrays over the endpoints
  std::vector<int32_t> cov(np + 1, 0), gcov(np + 1, 0);
  auto at = [&](uint64_t x) { return (size_t)(std::lower_bound(pts.begin(), pts.end(), x) - pts.begin()); };
  for (uint32_t i = 0; i < n; ++i) {
    if (b[i] <= a[i]) continue;
    const size_t ia = at(a[i]), ib = at(b[i]);
    ++cov[ia]; --cov[ib];
    if (!rflags || (rflags[i] & kReqGaps)) { ++gcov[ia]; --gcov[ib]; }
  }
  atom_a.clear(); atom_b.clear(); atom_rf.clear();
  std::vector<uint32_t> atom_of(np, UINT32_MAX);      // elementary piece k -> atom
  int32_t c = 0, g = 0;
  for (size_t k = 0; k + 1 < np; ++k) {
    c += cov[k];
    g += gcov[k];
    if (c > 0) {                                      // covered pieces become atoms
      atom_of[k] = (uint32_t)atom_a.size();
      atom_a.push_back(pts[k]);
      atom_b.push_back(pts[k + 1]);
      atom_rf.push_back(g > 0 ? kReqGaps : 0u);
    }
  }
  spans.assign(n, ReqSpan{0, 0, 0, 0});
  for (uint32_t i = 0; i < n; ++i) {
    spans[i].rflags = rflags ? rflags[i] : kReqGaps;
    if (b[i] <= a[i]) continue;
    // every piece inside the request is covered, so its atoms are contiguous
    spans[i].s = atom_of[at(a[i])];
    spans[i].e = atom_of[at(b[i]) - 1] + 1;
  }
}

void Plan::load(uint32_t n, const uint64_t* a, const uint64_t* b, uint32_t fl,
                const uint32_t* rflags) {
  nout = 0;
  if (!share || (fl & kFlagBitmap)) {
    load_requests(n, a, b, fl, rflags);
    return;
  }
  if (cap_out && n > cap_out) throw Error(VOSS_ERR_INVALID_ARG, "batch exceeds the plan's capacity");
  cut_ranges(n, a, b, rflags, atom_a, atom_b, atom_rf, host_spans);
  // A fixed-capacity plan takes the atoms only if they fit (narrow atoms may
  // be tuned to smaller segments than the requests they came from);
  // otherwise the batch runs unshared, which always fits.
  if (cap_out) {
    uint64_t segs_need = 0;
    for (size_t i = 0; i < atom_a.size(); ++i) segs_need += segments_for(atom_a[i], atom_b[i]);
    if (atom_a.size() > cap_req || segs_need > cap_segs) {
      load_requests(n, a, b, fl, rflags);
      return;
    }
  }
  load_requests((uint32_t)atom_a.size(), atom_a.data(), atom_b.data(), fl, atom_rf.data());
  host_apos.assign(nreq, 0);
  for (uint32_t d = 0; d < nreq; ++d) host_apos[order[d]] = d;   // position -> device index
  nout = n;
  static_cast<BatchHdr*>(stage.ptr)->nout = nout;
  if (!cap_out) {
    spans.reserve(sizeof(ReqSpan) * std::max<uint32_t>(n, 1));
    apos.reserve(sizeof(uint32_t) * std::max<uint32_t>(nreq, 1));
    rres.reserve(sizeof(ReqResult) * std::max<uint32_t>(n, 1));
    host_results.reserve(sizeof(ReqResult) * std::max<uint32_t>(std::max(n, nreq), 1));
  }
}

void Plan::load_requests(uint32_t n, const uint64_t* a, const uint64_t* b, uint32_t fl,
                         const uint32_t* rflags) {
  Engine& E = *eng;
  flags = fl;
  uint64_t max_b = 0;
  for (uint32_t i = 0; i < n; ++i) {
    if (b[i] > kMaxB) throw Error(VOSS_ERR_OUT_OF_RANGE, "range end exceeds 10^14 + 10^10 + 1");
    if (b[i] > a[i]) max_b = std::max(max_b, b[i]);
  }
  if (cap_req && n > cap_req) throw Error(VOSS_ERR_INVALID_ARG, "batch exceeds the plan's capacity");
  if (max_b > 1) E.ensure_table(isqrt_u64(max_b - 1));
  threads = E.cfg.threads;
  const bool many = n > 1 || batch_mode;

  struct Item { ReqDesc d; double cost; uint32_t idx; };
  std::vector<Item> items(n);
  uint32_t smax = 0;
  for (uint32_t i = 0; i < n; ++i) {
    ReqDesc r{};
    r.a = a[i];
    r.b = b[i];
    r.rflags = rflags ? rflags[i] : kReqGaps;
    double cost = 0;
    if (b[i] > a[i]) {
      const Config c = E.tuned_for(a[i], b[i], many);
      r.k_lo = a[i] / 30;
      r.k_hi = (b[i] + 29) / 30;
      r.seg_bytes = c.seg_bytes;
      r.nseg = (r.k_hi - r.k_lo + c.seg_bytes - 1) / c.seg_bytes;
      r.nprimes = E.primes_below_sq(b[i]);
      r.tier_split = E.index_of(c.tier_split);
      r.tier_huge = E.index_of(c.seg_bytes);
      smax = std::max(smax, c.seg_bytes);
      // per segment: fill and scan grow with the bytes, setup with the primes
      cost = (double)r.nseg * ((double)c.seg_bytes + 24.0 * r.nprimes);
    } else {
      r.seg_bytes = 128;
    }
    items[i] = Item{r, cost, i};
  }
  if (n > 1)
    std::stable_sort(items.begin(), items.end(),
                     [](const Item& x, const Item& y) { return x.cost > y.cost; });
  host_reqs.resize(n);
  order.resize(n);
  host_fills.clear();
  wins.clear();
  uint64_t base = 0, bbase = 0;
  for (uint32_t i = 0; i < n; ++i) {
    ReqDesc& r = host_reqs[i];
    r = items[i].d;
    r.seg_base = base;
    r.bucket_idx = r.nprimes;
    r.bucket_base = 0;
    r.bucket_cap = 0;
    order[i] = items[i].idx;
    base += r.nseg;
    // a lone request of a plan without fixed capacity may be windowed
    const bool windowed = !cap_req && n == 1 && r.nseg > kMaxBucketSegs;
    if (allow_buckets && r.nseg && !(fl & kFlagBitmap) && (windowed || r.nseg <= kMaxBucketSegs)) {
      const Config c = E.tuned_for(r.a, r.b, many);
      const BucketPlan bp = E.bucket_plan(c, r.b, r.nprimes, r.nseg, r.seg_bytes);
      const uint64_t wsegs = std::min<uint64_t>(r.nseg, kMaxBucketSegs);   // segments per window
      const uint64_t need = (uint64_t)bp.cap * wsegs;
      if (bp.cap) {
        // fill items, per window: runs of kFillPrimes primes; a run's hits
        // (8 per p bytes per prime) split over segment ranges so that every
        // item carries at most about kFillHits hits: items balance, and the
        // list blocks that the resident fill CTAs are writing at any time
        // (their items' entries) stay well inside L2, so lines leave it
        // complete
        item_buf.clear();
        std::vector<Window> rw;
        for (uint64_t w0 = 0; w0 < r.nseg; w0 += wsegs) {
          const uint32_t nseg = (uint32_t)std::min<uint64_t>(wsegs, r.nseg - w0);
          const uint64_t kw = r.k_lo + w0 * r.seg_bytes;
          const double per = 8.0 * (double)std::min<uint64_t>(r.k_hi - kw, (uint64_t)nseg * r.seg_bytes);
          const uint32_t f0 = (uint32_t)item_buf.size();
          for (uint32_t p0 = bp.bucket_idx; p0 < r.nprimes; p0 += kFillPrimes) {
            const uint32_t p1 = std::min<uint32_t>(p0 + kFillPrimes, r.nprimes);
            const double hits = per * (E.hInvPrefix[p1] - E.hInvPrefix[p0]);
            const uint32_t pieces = (uint32_t)std::min<double>(nseg, std::max(1.0, std::ceil(hits / kFillHits)));
            for (uint32_t j = 0; j < pieces; ++j) {
              const uint32_t g0 = (uint32_t)((uint64_t)nseg * j / pieces);
              const uint32_t g1 = (uint32_t)((uint64_t)nseg * (j + 1) / pieces);
              item_buf.push_back(FillItem{i, p0, p1, g0 | (g1 << 16)});
            }
          }
          rw.push_back(Window{r.seg_base + w0, r.seg_base + w0 + nseg, f0, (uint32_t)item_buf.size(),
                              (uint32_t)w0});
        }
        const bool fits = !cap_req || (bbase + need <= cap_bucket && host_fills.size() + item_buf.size() <= cap_fill);
        if (fits) {
          r.bucket_idx = bp.bucket_idx;
          r.bucket_cap = bp.cap;
          r.bucket_base = bbase;
          bbase += need;
          host_fills.insert(host_fills.end(), item_buf.begin(), item_buf.end());
          if (windowed) wins = std::move(rw);
        }
      }
    }
  }
  bucket_entries = bbase;
  nfill = (uint32_t)host_fills.size();
  nreq = n;
  total_segs = base;
  if (cap_req) {
    if (total_segs > cap_segs) throw Error(VOSS_ERR_INVALID_ARG, "batch exceeds the plan's segment capacity");
    seg_max = E.cfg.seg_bytes;     // fixed for graph replay
  } else {
    seg_max = std::max<uint32_t>(smax, 128);
    hdr.reserve(sizeof(BatchHdr) + sizeof(ReqDesc) * std::max<uint32_t>(n, 1));
    segs.reserve(sizeof(SegRec) * std::max<uint64_t>(total_segs, 1));
    acc.reserve(sizeof(ReqAccum) * std::max<uint32_t>(n, 1));
    results.reserve(sizeof(ReqResult) * std::max<uint32_t>(n, 1));
    stage.reserve(sizeof(BatchHdr) + sizeof(ReqDesc) * std::max<uint32_t>(n, 1));
    host_results.reserve(sizeof(ReqResult) * std::max<uint32_t>(n, 1));
  }
  if (flags & kFlagBitmap) {
    if (n != 1) throw Error(VOSS_ERR_INTERNAL, "bitmap output needs exactly one range");
    const uint64_t words = (host_reqs[0].k_hi - host_reqs[0].k_lo + 3) / 4 + 1;
    bitmap.reserve(words * 4);
  }
  if (!cap_req) {
    bucket.reserve(4 * std::max<uint64_t>(bucket_entries, 1));
    fills.reserve(sizeof(FillItem) * std::max<uint32_t>(nfill, 1));
    bcount.reserve(round16(4 * std::max<uint64_t>(total_segs, 1)));
  }
  ctl.reserve(sizeof(PlanCtl));
  large.reserve(sizeof(LargeGapRec) * large_cap);
  BatchHdr* h = static_cast<BatchHdr*>(stage.ptr);
  h->total_segs = total_segs;
  h->nreq = nreq;
  h->nfill = nfill;
  h->nout = 0;
  h->pad = 0;
  if (n) std::memcpy(h + 1, host_reqs.data(), sizeof(ReqDesc) * n);
  const uint64_t gcap = (uint64_t)E.sm_count * E.cfg.ctas_per_sm;
  grid = (uint32_t)(cap_req ? gcap : std::min<uint64_t>(total_segs, gcap));

  prm.reqs = dreqs();
  prm.hdr = hdr.as<BatchHdr>();
  prm.queue = &dctl()->queue;
  prm.P = E.dP.as<uint32_t>();
  prm.M = E.dM.as<uint64_t>();
  prm.R = E.dR.as<uint32_t>();
  for (int t = 0; t < kTiles; ++t) {
    prm.tile[t] = E.tile[t].as<uint32_t>();
    prm.tile_stride16[t] = tile_copy_stride(tile_period(t), kMaxSegBytes) / 16;
  }
  prm.seg_bytes = seg_max;
  prm.segs = segs.as<SegRec>();
  prm.acc = acc.as<ReqAccum>();
  prm.large = large.as<LargeGapRec>();
  prm.n_large = &dctl()->nlarge;
  prm.large_cap = large_cap;
  prm.flags = flags;
  prm.bitmap = bitmap.as<uint32_t>();
  prm.bucket = bucket.as<uint32_t>();
  prm.bcount = bcount.as<uint32_t>();
}

void Plan::prepare(uint32_t n, const uint64_t* a, const uint64_t* b, uint32_t fl) {
  load(n, a, b, fl);
}

void Plan::upload(cudaStream_t s) {
  const size_t bytes = sizeof(BatchHdr) + sizeof(ReqDesc) * nreq;
  check_cuda(cudaMemcpyAsync(hdr.ptr, stage.ptr, bytes, cudaMemcpyHostToDevice, s),
             "upload batch header and requests");
  if (nfill)
    check_cuda(cudaMemcpyAsync(fills.ptr, host_fills.data(), sizeof(FillItem) * nfill,
                               cudaMemcpyHostToDevice, s), "upload fill items");
  if (nout) {
    check_cuda(cudaMemcpyAsync(spans.ptr, host_spans.data(), sizeof(ReqSpan) * nout,
                               cudaMemcpyHostToDevice, s), "upload request spans");
    if (nreq)
      check_cuda(cudaMemcpyAsync(apos.ptr, host_apos.data(), sizeof(uint32_t) * nreq,
                                 cudaMemcpyHostToDevice, s), "upload atom order");
  }
}

Plan::~Plan() {
  for (cudaEvent_t& e : ev)
    if (e) cudaEventDestroy(e);
  if (graph_exec) cudaGraphExecDestroy(graph_exec);
  if (graph) cudaGraphDestroy(graph);
}

void Plan::capture(cudaStream_t s) {
  if (!cap_req) throw Error(VOSS_ERR_INTERNAL, "graph capture needs a fixed-capacity plan");
  if (graph_exec) return;
  // the kernels' attributes are raised outside the capture
  check_cuda(launch_sieve(prm, 0, threads, s), "sieve attributes");
  check_cuda(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "begin capture");
  try {
    run_device(s);
  } catch (...) {
    cudaGraph_t g = nullptr;
    cudaStreamEndCapture(s, &g);
    if (g) cudaGraphDestroy(g);
    throw;
  }
  check_cuda(cudaStreamEndCapture(s, &graph), "end capture");
  check_cuda(cudaGraphInstantiate(&graph_exec, graph, 0), "graph instantiate");
}

void Plan::launch_graph(cudaStream_t s) {
  if (!graph_exec) capture(s);
  check_cuda(cudaGraphLaunch(graph_exec, s), "graph launch");
}

void Plan::kernel_ms(float* sieve_ms, float* finalize_ms) {
  if (!ev[2]) throw Error(VOSS_ERR_INVALID_ARG, "plan has not been launched");
  check_cuda(cudaEventSynchronize(ev[2]), "plan events");
  if (sieve_ms) check_cuda(cudaEventElapsedTime(sieve_ms, ev[0], ev[1]), "event time");
  if (finalize_ms) check_cuda(cudaEventElapsedTime(finalize_ms, ev[1], ev[2]), "event time");
}

void Plan::run_device(cudaStream_t s) {
  for (cudaEvent_t& e : ev)
    if (!e) check_cuda(cudaEventCreate(&e), "cudaEventCreate");
  const uint32_t nacc = cap_req ? cap_req : nreq;
  if (nacc == 0) return;
  // accumulators, control words and bucket counts: one zeroing launch
  const uint64_t nsegs_dev = cap_req ? cap_segs : total_segs;
  check_cuda(launch_zero(ZeroSpan{acc.ptr, sizeof(ReqAccum) * nacc / 16},
                         ZeroSpan{ctl.ptr, sizeof(PlanCtl) / 16},
                         ZeroSpan{bcount.ptr, round16(4 * nsegs_dev) / 16}, eng->sm_count * 4, s),
             "zero_kernel");
  // the sieve's timed span covers the bucket fill that feeds it
  if (timed) check_cuda(cudaEventRecord(ev[0], s), "event");
  FillParams fp{};
  fp.reqs = dreqs();
  fp.hdr = hdr.as<BatchHdr>();
  fp.items = fills.as<FillItem>();
  fp.P = prm.P;
  fp.M = prm.M;
  fp.R = prm.R;
  fp.bucket = bucket.as<uint32_t>();
  fp.bcount = bcount.as<uint32_t>();
  fp.overflow = &dctl()->overflow;
  if (wins.empty()) {
    if (cap_req ? cap_fill : nfill) {
      const uint32_t fgrid = cap_req ? fill_grid_max() : std::min<uint32_t>(nfill, fill_grid_max());
      check_cuda(launch_bucket_fill(fp, fgrid, s), "bucket_fill_kernel");
    }
    check_cuda(launch_sieve(prm, grid, threads, s), "sieve_segments_kernel");
  } else {
    // one window at a time: fill its lists, then sieve its segments; each
    // sieve launch counts its own work queue from zero
    const uint64_t gcap = (uint64_t)eng->sm_count * eng->cfg.ctas_per_sm;
    for (size_t w = 0; w < wins.size(); ++w) {
      const Window& W = wins[w];
      if (w) check_cuda(cudaMemsetAsync(&dctl()->queue, 0, sizeof(unsigned long long), s), "reset work queue");
      fp.items = fills.as<FillItem>() + W.fill_lo;
      fp.nitems = W.fill_hi - W.fill_lo;
      fp.seg0 = W.seg0;
      if (fp.nitems)
        check_cuda(launch_bucket_fill(fp, std::min<uint32_t>(fp.nitems, fill_grid_max()), s), "bucket_fill_kernel");
      SieveParams wp = prm;
      wp.item_lo = W.item_lo;
      wp.item_hi = W.item_hi;
      wp.list_seg0 = W.seg0;
      check_cuda(launch_sieve(wp, (uint32_t)std::min<uint64_t>(W.item_hi - W.item_lo, gcap), threads, s),
                 "sieve_segments_kernel");
    }
  }
  if (timed) check_cuda(cudaEventRecord(ev[1], s), "event");
  check_cuda(launch_finalize(dreqs(), hdr.as<BatchHdr>(), segs.as<SegRec>(),
                             acc.as<ReqAccum>(), large.as<LargeGapRec>(),
                             &dctl()->nlarge, large_cap, results.as<ReqResult>(), nacc, s),
             "finalize_kernel");
  if (cap_req ? cap_out : nout)
    check_cuda(launch_combine(hdr.as<BatchHdr>(), spans.as<ReqSpan>(), apos.as<uint32_t>(),
                              results.as<ReqResult>(), rres.as<ReqResult>(), cap_req ? cap_out : nout, s),
               "combine_kernel");
  if (timed) check_cuda(cudaEventRecord(ev[2], s), "event");
}

void Plan::fetch_async(cudaStream_t s) {
  if (nout)
    check_cuda(cudaMemcpyAsync(host_results.ptr, rres.ptr, sizeof(ReqResult) * nout,
                               cudaMemcpyDeviceToHost, s), "download results");
  else if (nreq)
    check_cuda(cudaMemcpyAsync(host_results.ptr, results.ptr, sizeof(ReqResult) * nreq,
                               cudaMemcpyDeviceToHost, s), "download results");
  if (nfill) {
    host_flag.reserve(sizeof(unsigned int));
    check_cuda(cudaMemcpyAsync(host_flag.ptr, &dctl()->overflow, sizeof(unsigned int),
                               cudaMemcpyDeviceToHost, s), "download overflow flag");
  }
}

const ReqResult* Plan::finish() {
  const ReqResult* r = static_cast<const ReqResult*>(host_results.ptr);
  if (nout) {                          // combine_kernel wrote caller order
    out.assign(r, r + nout);
    return out.data();
  }
  out.resize(nreq);
  for (uint32_t i = 0; i < nreq; ++i) out[order[i]] = r[i];
  return out.data();
}

const ReqResult* Plan::fetch(cudaStream_t s) {
  fetch_async(s);
  check_cuda(cudaStreamSynchronize(s), "sieve run");
  return finish();
}

std::vector<LargeGapRec> Plan::fetch_large(cudaStream_t s) {
  unsigned int n = 0;
  check_cuda(cudaMemcpyAsync(&n, &dctl()->nlarge, sizeof(n), cudaMemcpyDeviceToHost, s), "large count");
  check_cuda(cudaStreamSynchronize(s), "large count");
  if (n > large_cap)
    throw Error(VOSS_ERR_INTERNAL, "large-gap buffer overflow (" + std::to_string(n) + " gaps)");
  std::vector<LargeGapRec> v(n);
  if (n) {
    check_cuda(cudaMemcpyAsync(v.data(), large.ptr, sizeof(LargeGapRec) * n,
                               cudaMemcpyDeviceToHost, s), "large gaps");
    check_cuda(cudaStreamSynchronize(s), "large gaps");
  }
  // device request index -> caller's index
  for (LargeGapRec& x : v) x.req = order[x.req];
  return v;
}

uint64_t Plan::wheel_bytes() const {
  uint64_t t = 0;
  for (const ReqDesc& r : host_reqs) t += r.k_hi - r.k_lo;
  return t;
}

uint64_t Plan::algorithmic_clears() const {
  // The algorithmic work of the sieve: the candidate clears of Eratosthenes
  // by every prime 17 < p with p*p < b (7..17 being the wheel-and-pattern
  // primes every wheel-30 sieve presieves): for each such p and class o, the
  // k in [k_lo, k_hi) with k = R (mod p) and 30k + W30[o] >= p*p.  The table
  // primes (>= 61) are cleared by the marking tiers, 19..59 by the presieve
  // tiles; the count is the same whichever does the work.
  const Engine& E = *eng;
  uint64_t total = 0;
  auto clears = [&](const ReqDesc& r, uint64_t p) {
    const int64_t inv30 = inverse_mod((int64_t)(30 % p), (int64_t)p);
    for (int o = 0; o < 8; ++o) {
      const uint64_t rr = ((p - kW30[o] % p) % p) * (uint64_t)inv30 % p;
      uint64_t k = r.k_lo + (rr + p - r.k_lo % p) % p;
      const uint64_t n = 30 * k + kW30[o];
      if (n < p * p) k += ((p * p - n + 30 * p - 1) / (30 * p)) * p;
      if (k < r.k_hi) total += (r.k_hi - 1 - k) / p + 1;
    }
  };
  for (const ReqDesc& r : host_reqs) {
    for (uint64_t p : {19ull, 23ull, 29ull, 31ull, 37ull, 41ull, 43ull, 47ull, 53ull, 59ull})
      if (p * p < r.b) clears(r, p);
    for (uint32_t i = 0; i < r.nprimes; ++i) clears(r, E.hP[i]);
  }
  return total;
}

const ReqResult* Engine::run(uint32_t n, const uint64_t* a, const uint64_t* b,
                             std::vector<LargeGapRec>* lg, bool gaps, bool share) {
  std::vector<uint32_t> rf(n, gaps ? kReqGaps : 0u);
  struct Unshare { Plan& p; ~Unshare() { p.share = false; } } unshare{scratch};
  scratch.share = share && !lg && n > 1;
  scratch.allow_buckets = true;
  scratch.load(n, a, b, 0, rf.data());
  scratch.launch(stream);
  const ReqResult* r = scratch.fetch(stream);
  if (scratch.overflowed()) {                // a bucket list ran out of room: redo without lists
    scratch.allow_buckets = false;
    scratch.load(n, a, b, 0, rf.data());
    scratch.launch(stream);
    scratch.allow_buckets = true;
    r = scratch.fetch(stream);
  }
  if (lg) *lg = scratch.fetch_large(stream);
  return r;
}

ReqResult merge_ordered(const ReqResult* parts, size_t n, bool gaps) {
  ReqResult m;
  std::memset(&m, 0, sizeof(m));
  uint64_t bg = 0, bs = 0;
  for (size_t i = 0; i < n; ++i) {
    const ReqResult& r = parts[i];
    m.count += r.count;
    m.c41 += r.c41; m.c43 += r.c43; m.c31 += r.c31; m.c32 += r.c32;
    if (!r.count) continue;
    if (gaps) {
      for (int b = 0; b < kHistBins; ++b) m.hist[b] += r.hist[b];
      if (m.last) {                               // the gap into this piece (its start is the earlier)
        const uint64_t g = r.first - m.last;
        m.hist[std::min<uint64_t>(g >> 1, kHistBins - 1)]++;
        if (g > bg) { bg = g; bs = m.last; }
      }
      if (r.max_gap > bg) { bg = r.max_gap; bs = r.max_gap_start; }
    }
    if (!m.first) m.first = r.first;
    m.last = r.last;
  }
  m.max_gap = bg;
  m.max_gap_start = bg ? bs : 0;
  m.num_gaps = m.count ? m.count - 1 : 0;
  return m;
}

void to_public(const ReqResult& r, uint64_t a, uint64_t b, voss_range_stats_t* o) {
  std::memset(o, 0, sizeof(*o));
  o->a = a;
  o->b = b;
  o->count = r.count;
  o->twins = r.hist[1];
  o->cousins = r.hist[2];
  o->sexy = r.hist[3];
  o->pi_4_1 = r.c41;
  o->pi_4_3 = r.c43;
  o->pi_3_1 = r.c31;
  o->pi_3_2 = r.c32;
  o->first_prime = r.first;
  o->last_prime = r.last;
  o->max_gap = r.max_gap;
  o->max_gap_start = r.max_gap_start;
  o->num_gaps = r.num_gaps;
  uint64_t over = 0, large = 0;
  for (int i = 0; i < kHistBins; ++i) {
    if (i < VOSS_GAP_BINS - 1) o->gap_hist[i] = r.hist[i];
    else over += r.hist[i];
    if (i >= (int)(kLargeGap / 2)) large += r.hist[i];
  }
  o->gap_hist[VOSS_GAP_BINS - 1] = over;
  o->large_gaps = large;
}

}  // namespace vg
