// capi.cpp -- the voss C ABI on top of the GB300 engine.
//
// Reference entry points keep the reference's validation order, error codes
// and messages (library/src/primes/context.cu:566-975,
// prime_count.cu:298-322, range.cu:267-323, goldbach_upto.cu:48-64,
// core/error.cpp, core/alloc.cpp, io/csv.cpp).  Compute failures inside a
// reference entry point map to VOSS_ERR_CUDA as the reference's catch
// blocks do (context.cu:628-634).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "engine.h"
#include "goldbach.h"
#include "serve.h"
#include "voss/voss.h"
#include "voss/voss_gb300.h"
#include "voss/voss_numbers.h"
#include "voss/voss_primes.h"

namespace {

thread_local std::string g_last_error;

void set_err(const std::string& m) { g_last_error = m; }

constexpr uint64_t kMaxN = 100000000000000ull;   // 10^14
// The smallest accepted tier split.  Splits below the first table prime (61)
// leave the warp-per-prime tier empty.
constexpr uint32_t kMinTierSplit = 37;

// Run f, converting exceptions to codes.  `compute_code` is the code the
// reference returns for a failure inside the computation.
template <class F>
int guarded(F&& f, int compute_code) {
  try {
    return f();
  } catch (const vg::Error& e) {
    set_err(e.what());
    return compute_code == VOSS_ERR_CUDA ? VOSS_ERR_CUDA : e.code;
  } catch (const std::bad_alloc&) {
    set_err("host allocation failed");
    return VOSS_ERR_OUT_OF_MEMORY;
  } catch (const std::exception& e) {
    set_err(e.what());
    return compute_code;
  } catch (...) {
    set_err("Unknown error");
    return VOSS_ERR_INTERNAL;
  }
}

// Statistics of [lo, hi) over several consecutive ranges, merged on the host.
struct Merged {
  uint64_t count = 0, c41 = 0, c43 = 0, first = 0, last = 0;
  std::vector<uint64_t> hist = std::vector<uint64_t>(vg::kHistBins, 0);
  std::vector<std::pair<uint64_t, uint32_t>> large;   // (second prime, gap)
};

void merge_into(Merged& m, const vg::ReqResult& r, const std::vector<vg::LargeGapRec>& lg,
                uint32_t req) {
  if (r.count) {
    if (m.last && r.first) {
      const uint64_t g = r.first - m.last;
      const uint64_t bin = std::min<uint64_t>(g >> 1, vg::kHistBins - 1);
      m.hist[bin]++;
      if (g >= vg::kLargeGap) m.large.emplace_back(r.first, (uint32_t)g);
    }
    if (!m.first) m.first = r.first;
    m.last = r.last;
  }
  m.count += r.count;
  m.c41 += r.c41;
  m.c43 += r.c43;
  for (int i = 0; i < vg::kHistBins; ++i) m.hist[i] += r.hist[i];
  for (const auto& x : lg)
    if (x.req == req) m.large.emplace_back(x.pos, x.gap);
}

}  // namespace

// ===========================================================================
// voss.h
// ===========================================================================
extern "C" const char* voss_get_last_error(void) { return g_last_error.c_str(); }

extern "C" const char* voss_strerror(int code) {
  switch (code) {
    case VOSS_OK: return "OK";
    case VOSS_ERR_INVALID_N: return "Invalid N";
    case VOSS_ERR_OUT_OF_RANGE: return "Out of range";
    case VOSS_ERR_NO_CUDA: return "No CUDA device";
    case VOSS_ERR_OUT_OF_MEMORY: return "Out of memory";
    case VOSS_ERR_CUDA: return "CUDA error";
    case VOSS_ERR_INVALID_ARG: return "Invalid argument";
    case VOSS_ERR_INTERNAL: return "Internal error";
    default: return "Unknown error";
  }
}

extern "C" void voss_free(void* ptr) { free(ptr); }

// ===========================================================================
// Context
// ===========================================================================
struct voss_primes_ctx {
  uint64_t N = 0;
  int profile = VOSS_PROFILE_STANDARD;
  bool has_count = false, has_full = false;
  uint64_t pi = 0;
  std::vector<uint64_t> hist;          // gap/2 bins (vg::kHistBins)
  uint64_t c41 = 0, c43 = 0;
  std::vector<std::pair<uint64_t, uint32_t>> large;   // sorted for the API
  bool has_sophie = false;
  uint64_t sophie = 0;
  voss_progress_cb cb = nullptr;
  void* user = nullptr;
};

namespace {

// Count of gaps of exactly g in a gap/2 histogram plus the exact large list.
uint64_t gap_count(const voss_primes_ctx* c, uint64_t g) {
  if (g == 1) return c->hist[0];
  if (g & 1) return 0;
  const uint64_t bin = g / 2;
  if (bin < (uint64_t)vg::kHistBins - 1) return c->hist[bin];
  uint64_t n = 0;
  for (const auto& x : c->large) n += (x.second == g);
  return n;
}

// Reference semantics of compute_full_impl (context.cu:212-559) on the GB300
// engine: primes in [1, N], chunked like the reference's segments when a
// progress callback is set.
void compute_ctx(voss_primes_ctx* c) {
  const uint64_t N = c->N;
  const bool gaps = c->profile != VOSS_PROFILE_MINIMAL;
  c->hist.assign(vg::kHistBins, 0);
  c->large.clear();
  c->c41 = c->c43 = 0;
  if (N < 7) {                          // context.cu:228-247
    c->pi = N < 3 ? 1 : N < 5 ? 2 : 3;
    if (N >= 3) c->hist[0] = 1;         // gap 2 -> 3
    if (N >= 5) c->hist[1] = 1;         // gap 3 -> 5
    c->has_count = true;
    c->has_full = gaps;
    return;
  }
  vg::Engine& E = vg::Engine::for_current_device();
  std::lock_guard<std::mutex> g(E.mu);
  const uint64_t kMaxSeg = 50000000010ull;
  const uint64_t segn = N < kMaxSeg ? ((N + 29) / 30) * 30 + 10 : kMaxSeg;
  const uint64_t nseg = (N + segn - 1) / segn;
  Merged m;
  if (!c->cb) {
    std::vector<vg::LargeGapRec> lg;
    uint64_t a = 0, b = N + 1;
    const vg::ReqResult* r = E.run(1, &a, &b, gaps ? &lg : nullptr, gaps);
    merge_into(m, r[0], lg, 0);
  } else {
    uint64_t cumulative = 3;
    for (uint64_t s = 0; s < nseg; ++s) {
      const uint64_t lo = s * segn + 1;
      const uint64_t hi = std::min<uint64_t>((s + 1) * segn, N);
      std::vector<vg::LargeGapRec> lg;
      uint64_t a = lo, b = hi + 1;
      const vg::ReqResult* r = E.run(1, &a, &b, gaps ? &lg : nullptr, gaps);
      vg::ReqResult copy = r[0];
      merge_into(m, copy, lg, 0);
      // primes >= 7 in the chunk (the reference's n_pos, context.cu:423-436)
      uint64_t seeds = 0;
      for (uint64_t q : {2ull, 3ull, 5ull}) seeds += (q >= lo && q <= hi);
      const uint64_t npos = copy.count - seeds;
      cumulative += npos;
      c->cb((int)(s + 1), (int)nseg, npos, cumulative, c->user);
    }
  }
  c->pi = m.count;
  c->has_count = true;
  if (gaps) {
    c->hist = m.hist;
    c->c41 = m.c41;
    c->c43 = m.c43;
    c->large = m.large;
    std::sort(c->large.begin(), c->large.end(), [](const auto& x, const auto& y) {
      return x.second != y.second ? x.second > y.second : x.first < y.first;
    });
    c->has_full = true;
  }
}

int ensure(voss_primes_ctx* c) {
  if (c->has_count && (c->has_full || c->profile == VOSS_PROFILE_MINIMAL)) return VOSS_OK;
  return guarded([&] { compute_ctx(c); return VOSS_OK; }, VOSS_ERR_CUDA);
}

int gap_query(voss_primes_ctx* ctx, uint64_t* out, uint64_t g) {
  if (!ctx) { set_err("ctx is null"); return VOSS_ERR_INVALID_ARG; }
  if (!out) { set_err("out pointer is null"); return VOSS_ERR_INVALID_ARG; }
  if (ctx->profile == VOSS_PROFILE_MINIMAL) {
    set_err("Profile MINIMAL does not compute gap histogram; use STANDARD or FULL");
    return VOSS_ERR_INVALID_ARG;
  }
  int rc = ensure(ctx);
  if (rc) return rc;
  *out = gap_count(ctx, g);
  return VOSS_OK;
}

}  // namespace

extern "C" int voss_primes_ctx_new(uint64_t N, int profile, voss_primes_ctx** out_ctx) {
  if (!out_ctx) { set_err("out_ctx pointer is null"); return VOSS_ERR_INVALID_ARG; }
  *out_ctx = nullptr;
  if (N < 2) { set_err("N must be >= 2"); return VOSS_ERR_INVALID_N; }
  if (N > kMaxN) { set_err("N exceeds maximum (10^14)"); return VOSS_ERR_OUT_OF_RANGE; }
  if (profile != VOSS_PROFILE_MINIMAL && profile != VOSS_PROFILE_STANDARD &&
      profile != VOSS_PROFILE_FULL) {
    set_err("invalid profile value");
    return VOSS_ERR_INVALID_ARG;
  }
  try {
    auto* c = new voss_primes_ctx();
    c->N = N;
    c->profile = profile;
    *out_ctx = c;
    return VOSS_OK;
  } catch (const std::exception& e) {
    set_err(std::string("ctx_new failed: ") + e.what());
    return VOSS_ERR_INTERNAL;
  }
}

extern "C" void voss_primes_ctx_free(voss_primes_ctx* ctx) { delete ctx; }

extern "C" int voss_primes_ctx_set_progress(voss_primes_ctx* ctx, voss_progress_cb cb, void* user) {
  if (!ctx) { set_err("ctx is null"); return VOSS_ERR_INVALID_ARG; }
  ctx->cb = cb;
  ctx->user = user;
  return VOSS_OK;
}

extern "C" int voss_primes_ctx_prime_count(voss_primes_ctx* ctx, uint64_t* out) {
  if (!ctx) { set_err("ctx is null"); return VOSS_ERR_INVALID_ARG; }
  if (!out) { set_err("out pointer is null"); return VOSS_ERR_INVALID_ARG; }
  if (!ctx->has_count) {
    int rc = ensure(ctx);
    if (rc) return rc;
  }
  *out = ctx->pi;
  return VOSS_OK;
}

extern "C" int voss_primes_ctx_twins(voss_primes_ctx* ctx, uint64_t* out) { return gap_query(ctx, out, 2); }
extern "C" int voss_primes_ctx_cousin(voss_primes_ctx* ctx, uint64_t* out) { return gap_query(ctx, out, 4); }
extern "C" int voss_primes_ctx_sexy(voss_primes_ctx* ctx, uint64_t* out) { return gap_query(ctx, out, 6); }

extern "C" int voss_primes_ctx_statistics(voss_primes_ctx* ctx, voss_primes_stats_t* out) {
  if (!ctx) { set_err("ctx is null"); return VOSS_ERR_INVALID_ARG; }
  if (!out) { set_err("out pointer is null"); return VOSS_ERR_INVALID_ARG; }
  if (ctx->profile == VOSS_PROFILE_MINIMAL) {
    set_err("Profile MINIMAL does not compute gap histogram; use STANDARD or FULL");
    return VOSS_ERR_INVALID_ARG;
  }
  int rc = ensure(ctx);
  if (rc) return rc;
  // Gap values ascending with their counts: bins below the overflow bin hold
  // one gap value each; the overflow bin is resolved from the exact list.
  std::vector<std::pair<uint64_t, uint64_t>> gc;
  for (int i = 0; i < vg::kHistBins - 1; ++i)
    if (ctx->hist[i]) gc.emplace_back(i == 0 ? 1 : 2ull * i, ctx->hist[i]);
  if (ctx->hist[vg::kHistBins - 1]) {
    std::vector<uint64_t> big;
    for (const auto& x : ctx->large) if (x.second >= 2ull * (vg::kHistBins - 1)) big.push_back(x.second);
    std::sort(big.begin(), big.end());
    for (size_t i = 0; i < big.size();) {
      size_t j = i;
      while (j < big.size() && big[j] == big[i]) ++j;
      gc.emplace_back(big[i], j - i);
      i = j;
    }
  }
  // Two passes in the reference's order and types (context.cu:716-753).
  int64_t total = 0, weighted = 0;
  for (const auto& x : gc) { total += (int64_t)x.second; weighted += (int64_t)x.first * (int64_t)x.second; }
  if (total == 0) {
    out->mean_gap = out->std_dev = out->skewness = out->kurtosis = 0.0;
    out->total_gaps = 0;
    return VOSS_OK;
  }
  const double mean = (double)weighted / (double)total;
  double var_sum = 0.0, m3 = 0.0, m4 = 0.0;
  for (const auto& x : gc) {
    const double d = (double)x.first - mean;
    const double d2 = d * d;
    var_sum += (double)x.second * d2;
    m3 += (double)x.second * d2 * d;
    m4 += (double)x.second * d2 * d2;
  }
  const double var = var_sum / (double)total;
  const double sd = std::sqrt(var);
  out->mean_gap = mean;
  out->std_dev = sd;
  out->skewness = sd > 0.0 ? (m3 / (double)total) / (var * sd) : 0.0;
  out->kurtosis = var > 0.0 ? (m4 / (double)total) / (var * var) - 3.0 : 0.0;
  out->total_gaps = (uint64_t)total;
  return VOSS_OK;
}

extern "C" int voss_primes_ctx_chebyshev_bias(voss_primes_ctx* ctx, uint64_t* p41, uint64_t* p43) {
  if (!ctx) { set_err("ctx is null"); return VOSS_ERR_INVALID_ARG; }
  if (!p41 || !p43) { set_err("out pointers must not be null"); return VOSS_ERR_INVALID_ARG; }
  if (ctx->profile == VOSS_PROFILE_MINIMAL) {
    set_err("Profile MINIMAL does not compute Chebyshev bias; use STANDARD or FULL");
    return VOSS_ERR_INVALID_ARG;
  }
  int rc = ensure(ctx);
  if (rc) return rc;
  *p41 = ctx->c41;
  *p43 = ctx->c43;
  return VOSS_OK;
}

extern "C" int voss_primes_ctx_large_gaps_count(voss_primes_ctx* ctx, uint64_t* out_count) {
  if (!ctx || !out_count) { set_err("null pointer"); return VOSS_ERR_INVALID_ARG; }
  if (ctx->profile == VOSS_PROFILE_MINIMAL) {
    set_err("Profile MINIMAL does not compute large gaps");
    return VOSS_ERR_INVALID_ARG;
  }
  int rc = ensure(ctx);
  if (rc) return rc;
  *out_count = ctx->large.size();
  return VOSS_OK;
}

extern "C" int voss_primes_ctx_large_gaps_get(voss_primes_ctx* ctx, uint64_t index,
                                              uint64_t* pos, uint32_t* gap) {
  if (!ctx || !pos || !gap) { set_err("null pointer"); return VOSS_ERR_INVALID_ARG; }
  if (ctx->profile == VOSS_PROFILE_MINIMAL) {
    set_err("Profile MINIMAL does not compute large gaps");
    return VOSS_ERR_INVALID_ARG;
  }
  int rc = ensure(ctx);
  if (rc) return rc;
  if (index >= ctx->large.size()) { set_err("index out of range"); return VOSS_ERR_INVALID_ARG; }
  *pos = ctx->large[index].first;
  *gap = ctx->large[index].second;
  return VOSS_OK;
}

extern "C" int voss_primes_ctx_export_csv(voss_primes_ctx* ctx, const char* prefix) {
  if (!ctx) { set_err("ctx is null"); return VOSS_ERR_INVALID_ARG; }
  if (!prefix) { set_err("prefix is null"); return VOSS_ERR_INVALID_ARG; }
  const std::string p(prefix);
  uint64_t c1 = 0, c3 = 0;
  int rc = voss_primes_ctx_chebyshev_bias(ctx, &c1, &c3);
  if (rc) return rc;
  auto open = [&](const std::string& path) -> FILE* {
    FILE* f = std::fopen(path.c_str(), "w");
    if (!f) set_err("failed to open " + path);
    return f;
  };
  {
    FILE* f = open(p + "_chebyshev.csv");
    if (!f) return VOSS_ERR_INTERNAL;
    std::fprintf(f, "pi_4_1,pi_4_3,difference\n%llu,%llu,%lld\n", (unsigned long long)c1,
                 (unsigned long long)c3, (long long)c3 - (long long)c1);
    std::fclose(f);
  }
  {
    uint64_t n = 0;
    rc = voss_primes_ctx_large_gaps_count(ctx, &n);
    if (rc) return rc;
    FILE* f = open(p + "_large_gaps.csv");
    if (!f) return VOSS_ERR_INTERNAL;
    std::fprintf(f, "position,gap\n");
    for (uint64_t i = 0; i < n; ++i)
      std::fprintf(f, "%llu,%u\n", (unsigned long long)ctx->large[i].first, (unsigned)ctx->large[i].second);
    std::fclose(f);
  }
  {
    voss_primes_stats_t s;
    rc = voss_primes_ctx_statistics(ctx, &s);
    if (rc) return rc;
    FILE* f = open(p + "_stats.csv");
    if (!f) return VOSS_ERR_INTERNAL;
    std::fprintf(f, "metric,value\nmean_gap,%.6f\nstd_dev,%.6f\nskewness,%.6f\nkurtosis,%.6f\ntotal_gaps,%llu\n",
                 s.mean_gap, s.std_dev, s.skewness, s.kurtosis, (unsigned long long)s.total_gaps);
    std::fclose(f);
  }
  return VOSS_OK;
}

extern "C" int voss_primes_ctx_sophie_germain_upto(voss_primes_ctx* ctx, uint64_t* out) {
  if (!ctx) { set_err("ctx is null"); return VOSS_ERR_INVALID_ARG; }
  if (!out) { set_err("out pointer is null"); return VOSS_ERR_INVALID_ARG; }
  if (ctx->profile == VOSS_PROFILE_MINIMAL) {
    set_err("Profile MINIMAL does not support sophie_germain; use STANDARD or FULL");
    return VOSS_ERR_INVALID_ARG;
  }
  if (ctx->has_sophie) { *out = ctx->sophie; return VOSS_OK; }
  return guarded([&] {
    vg::Engine& E = vg::Engine::for_current_device();
    std::lock_guard<std::mutex> g(E.mu);
    ctx->sophie = vg::sophie_germain_count(E, ctx->N);
    ctx->has_sophie = true;
    *out = ctx->sophie;
    return VOSS_OK;
  }, VOSS_ERR_INTERNAL);
}

extern "C" int voss_primes_ctx_sophie_germain(voss_primes_ctx* ctx, uint64_t* out) {
  return voss_primes_ctx_sophie_germain_upto(ctx, out);
}

// ===========================================================================
// Direct functions
// ===========================================================================
extern "C" int voss_primes_prime_count(uint64_t N, uint64_t* out) {
  if (N < 2) { set_err("N must be >= 2"); return VOSS_ERR_INVALID_N; }
  if (N > kMaxN) { set_err("N exceeds M0 maximum (10^14)"); return VOSS_ERR_OUT_OF_RANGE; }
  if (!out) { set_err("out pointer is null"); return VOSS_ERR_INVALID_ARG; }
  if (N < 7) { *out = N < 3 ? 1 : N < 5 ? 2 : 3; return VOSS_OK; }
  return guarded([&] {
    vg::Engine& E = vg::Engine::for_current_device();
    std::lock_guard<std::mutex> g(E.mu);
    uint64_t a = 0, b = N + 1;
    *out = E.run(1, &a, &b, nullptr, false)[0].count;
    return VOSS_OK;
  }, VOSS_ERR_CUDA);
}

extern "C" int voss_primes_in_range(uint64_t a, uint64_t b, uint64_t** arr, uint64_t* n) {
  return voss_primes_in_range_with_limit(a, b, 10000000ull, arr, n);
}

extern "C" int voss_primes_in_range_with_limit(uint64_t a, uint64_t b, uint64_t max_count,
                                               uint64_t** out_array, uint64_t* out_count) {
  if (!out_array || !out_count) { set_err("out pointer is null"); return VOSS_ERR_INVALID_ARG; }
  *out_array = nullptr;
  *out_count = 0;
  if (b > kMaxN) { set_err("b exceeds maximum (10^14)"); return VOSS_ERR_OUT_OF_RANGE; }
  if (max_count == 0) { set_err("max_count must be > 0"); return VOSS_ERR_INVALID_ARG; }
  return guarded([&] {
    if (a < 2) a = 2;
    if (b < a) return VOSS_OK;
    vg::Engine& E = vg::Engine::for_current_device();
    std::lock_guard<std::mutex> g(E.mu);
    std::vector<uint64_t> v = vg::primes_in_range(E, a, b, max_count);
    if (v.size() > max_count) {
      set_err("Range contains more primes than max_count");
      return VOSS_ERR_OUT_OF_MEMORY;
    }
    if (v.empty()) return VOSS_OK;
    auto* p = (uint64_t*)malloc(v.size() * sizeof(uint64_t));
    if (!p) { set_err("host malloc failed"); return VOSS_ERR_OUT_OF_MEMORY; }
    std::memcpy(p, v.data(), v.size() * sizeof(uint64_t));
    *out_array = p;
    *out_count = v.size();
    return VOSS_OK;
  }, VOSS_ERR_CUDA);
}

extern "C" int voss_primes_goldbach_test_upto(uint64_t N, uint64_t** out_ce, uint64_t* out_count,
                                              uint64_t max_ce) {
  if (!out_ce || !out_count) { set_err("null pointer"); return VOSS_ERR_INVALID_ARG; }
  *out_ce = nullptr;
  *out_count = 0;
  if (N < 4) { set_err("N must be >= 4"); return VOSS_ERR_INVALID_N; }
  if (max_ce == 0) return VOSS_OK;
  return guarded([&] {
    vg::Engine& E = vg::Engine::for_current_device();
    std::lock_guard<std::mutex> g(E.mu);
    vg::GoldbachResult r = vg::goldbach_run(E, N, nullptr, max_ce);
    if (!r.counterexamples.empty()) {
      auto* p = (uint64_t*)malloc(r.counterexamples.size() * sizeof(uint64_t));
      if (!p) { set_err("host malloc"); return VOSS_ERR_INTERNAL; }
      std::memcpy(p, r.counterexamples.data(), r.counterexamples.size() * sizeof(uint64_t));
      *out_ce = p;
      *out_count = r.counterexamples.size();
    }
    return VOSS_OK;
  }, VOSS_ERR_INTERNAL);
}

// Entry points outside the sieve: exported so the reference's binding loads.
#define VOSS_OUTSIDE(name) \
  set_err(std::string(name) + " is outside the sieve hot path and is not provided by this library"); \
  return VOSS_ERR_INTERNAL;

// nth / next / prev on the GPU sieve (the reference walks candidates with
// Miller-Rabin or a host vector<bool> sieve, nth.cu:40-103, next_prev.cu:22-83;
// same validation, limits and codes).  The sieve covers numbers below
// 10^14 + 10^10; beyond that these return VOSS_ERR_OUT_OF_RANGE.
namespace {

// smallest prime in [lo, hi), 0 if none (count-only run: first/last kept)
uint64_t first_prime_in(vg::Engine& E, uint64_t lo, uint64_t hi) {
  return E.run(1, &lo, &hi, nullptr, false)[0].first;
}
uint64_t last_prime_in(vg::Engine& E, uint64_t lo, uint64_t hi) {
  return E.run(1, &lo, &hi, nullptr, false)[0].last;
}
constexpr uint64_t kSearchMax = 100000000ull;   // the reference's MAX_SEARCH

}  // namespace

extern "C" int voss_primes_next(uint64_t x, uint64_t* out) {
  if (!out) { set_err("out pointer is null"); return VOSS_ERR_INVALID_ARG; }
  if (x < 2) { *out = 2; return VOSS_OK; }
  if (x >= vg::kMaxB - 1) { set_err("x exceeds the sieve's range (10^14 + 10^10)"); return VOSS_ERR_OUT_OF_RANGE; }
  return guarded([&] {
    vg::Engine& E = vg::Engine::for_current_device();
    std::lock_guard<std::mutex> g(E.mu);
    uint64_t w = 4096;
    for (uint64_t lo = x + 1; lo - (x + 1) < kSearchMax && lo < vg::kMaxB; lo += w, w *= 2) {
      const uint64_t hi = std::min<uint64_t>(lo + w, vg::kMaxB);
      const uint64_t p = first_prime_in(E, lo, hi);
      if (p) { *out = p; return VOSS_OK; }
    }
    set_err("no prime found within search limit");
    return VOSS_ERR_OUT_OF_RANGE;
  }, VOSS_ERR_CUDA);
}

extern "C" int voss_primes_prev(uint64_t x, uint64_t* out) {
  if (!out) { set_err("out pointer is null"); return VOSS_ERR_INVALID_ARG; }
  if (x <= 2) { set_err("no prime < " + std::to_string(x)); return VOSS_ERR_INVALID_N; }
  if (x == 3) { *out = 2; return VOSS_OK; }
  if (x > vg::kMaxB) { set_err("x exceeds the sieve's range (10^14 + 10^10)"); return VOSS_ERR_OUT_OF_RANGE; }
  return guarded([&] {
    vg::Engine& E = vg::Engine::for_current_device();
    std::lock_guard<std::mutex> g(E.mu);
    uint64_t w = 4096;
    for (uint64_t hi = x; hi > 2 && x - hi < kSearchMax; w *= 2) {
      const uint64_t lo = hi > w ? hi - w : 0;
      const uint64_t p = last_prime_in(E, lo, hi);
      if (p) { *out = p; return VOSS_OK; }
      hi = lo;
    }
    *out = 2;
    return VOSS_OK;
  }, VOSS_ERR_CUDA);
}

extern "C" int voss_primes_nth(uint64_t n, uint64_t* out) {
  if (!out) { set_err("out pointer is null"); return VOSS_ERR_INVALID_ARG; }
  if (n == 0) { set_err("n must be >= 1 (1-indexed)"); return VOSS_ERR_INVALID_N; }
  if (n > 50000000ull) { set_err("n exceeds maximum (50,000,000)"); return VOSS_ERR_OUT_OF_RANGE; }
  static const uint64_t first[6] = {0, 2, 3, 5, 7, 11};
  if (n <= 5) { *out = first[n]; return VOSS_OK; }
  return guarded([&] {
    vg::Engine& E = vg::Engine::for_current_device();
    std::lock_guard<std::mutex> g(E.mu);
    // estimate p_n ~ n (ln n + ln ln n - 1 + (ln ln n - 2) / ln n), count pi(est)
    // on the GPU, then list the primes between the estimate and p_n
    const double nf = (double)n, L = std::log(nf), LL = std::log(L);
    const uint64_t est = (uint64_t)(nf * (L + LL - 1.0 + (LL - 2.0) / L));
    uint64_t a = 0, b = est + 1;
    const uint64_t c = E.run(1, &a, &b, nullptr, false)[0].count;     // pi(est)
    const uint64_t span = (uint64_t)(L * 1.5 * (double)(c > n ? c - n : n - c) + 4096.0);
    if (c >= n) {                       // p_n <= est: the (c - n + 1)-th largest prime <= est
      const uint64_t lo = est > span ? est - span : 0;
      for (uint64_t lo2 = lo;; lo2 = lo2 > span ? lo2 - span : 0) {
        std::vector<uint64_t> v = vg::primes_in_range(E, lo2, est, ~0ull >> 1);
        if (v.size() >= c - n + 1) { *out = v[v.size() - (c - n + 1)]; return VOSS_OK; }
        if (lo2 == 0) break;
      }
    } else {                            // p_n > est: the (n - c)-th prime after est
      for (uint64_t hi = est + span;; hi += span) {
        std::vector<uint64_t> v = vg::primes_in_range(E, est + 1, hi, ~0ull >> 1);
        if (v.size() >= n - c) { *out = v[n - c - 1]; return VOSS_OK; }
      }
    }
    set_err("internal: could not locate the n-th prime");
    return VOSS_ERR_INTERNAL;
  }, VOSS_ERR_CUDA);
}
extern "C" int voss_primes_is_prime(uint64_t, int*) { VOSS_OUTSIDE("voss_primes_is_prime") }
extern "C" int voss_primes_factorize(uint64_t, uint64_t**, uint64_t*) { VOSS_OUTSIDE("voss_primes_factorize") }
extern "C" int voss_primes_is_mersenne_prime(uint32_t, int*) { VOSS_OUTSIDE("voss_primes_is_mersenne_prime") }
extern "C" int voss_primes_is_fermat_prime(uint32_t, int*) { VOSS_OUTSIDE("voss_primes_is_fermat_prime") }
extern "C" int voss_primes_goldbach_count(uint64_t, uint64_t*) { VOSS_OUTSIDE("voss_primes_goldbach_count") }
extern "C" int voss_primes_goldbach_partitions(uint64_t, uint64_t**, uint64_t*) { VOSS_OUTSIDE("voss_primes_goldbach_partitions") }
extern "C" int voss_numbers_phi(uint64_t, uint64_t*) { VOSS_OUTSIDE("voss_numbers_phi") }
extern "C" int voss_numbers_tau(uint64_t, uint64_t*) { VOSS_OUTSIDE("voss_numbers_tau") }
extern "C" int voss_numbers_sigma(uint64_t, uint64_t*) { VOSS_OUTSIDE("voss_numbers_sigma") }
extern "C" int voss_numbers_mu(uint64_t, int*) { VOSS_OUTSIDE("voss_numbers_mu") }
extern "C" int voss_numbers_gcd(uint64_t, uint64_t, uint64_t*) { VOSS_OUTSIDE("voss_numbers_gcd") }
extern "C" int voss_numbers_lcm(uint64_t, uint64_t, uint64_t*) { VOSS_OUTSIDE("voss_numbers_lcm") }
extern "C" int voss_numbers_fibonacci(uint64_t, uint64_t*) { VOSS_OUTSIDE("voss_numbers_fibonacci") }
extern "C" int voss_numbers_factorial(uint64_t, uint64_t*) { VOSS_OUTSIDE("voss_numbers_factorial") }

// ===========================================================================
// voss_gb300.h -- additive API
// ===========================================================================
extern "C" int voss_primes_range_stats_ex(uint64_t a, uint64_t b, voss_range_stats_t* out,
                                          uint64_t* hist_full) {
  if (!out) { set_err("out pointer is null"); return VOSS_ERR_INVALID_ARG; }
  if (b > vg::kMaxB) { set_err("b exceeds maximum (10^14 + 10^10 + 1)"); return VOSS_ERR_OUT_OF_RANGE; }
  return guarded([&] {
    vg::Engine& E = vg::Engine::for_current_device();
    std::lock_guard<std::mutex> g(E.mu);
    const vg::ReqResult* r = E.run(1, &a, &b);
    vg::to_public(r[0], a, b, out);
    if (hist_full) std::memcpy(hist_full, r[0].hist, sizeof(r[0].hist));
    return VOSS_OK;
  }, VOSS_ERR_INTERNAL);
}

extern "C" int voss_primes_range_stats(uint64_t a, uint64_t b, voss_range_stats_t* out) {
  return voss_primes_range_stats_ex(a, b, out, nullptr);
}

extern "C" int voss_primes_range_stats_batch(uint64_t n, const uint64_t* a, const uint64_t* b,
                                             voss_range_stats_t* out) {
  if (n && (!a || !b || !out)) { set_err("null pointer"); return VOSS_ERR_INVALID_ARG; }
  if (n > 0xFFFFFFFFull) { set_err("too many ranges"); return VOSS_ERR_INVALID_ARG; }
  for (uint64_t i = 0; i < n; ++i)
    if (b[i] > vg::kMaxB) { set_err("b exceeds maximum (10^14 + 10^10 + 1)"); return VOSS_ERR_OUT_OF_RANGE; }
  if (n == 0) return VOSS_OK;
  return guarded([&] {
    vg::Engine& E = vg::Engine::for_current_device();
    std::lock_guard<std::mutex> g(E.mu);
    // chunks bound the device memory of one launch (about 16 KB per range
    // with shared pieces); ranges share work within their chunk
    constexpr uint64_t kChunk = 32768;
    for (uint64_t i0 = 0; i0 < n; i0 += kChunk) {
      const uint64_t m = std::min<uint64_t>(kChunk, n - i0);
      const vg::ReqResult* r = E.run((uint32_t)m, a + i0, b + i0, nullptr, true, true);
      for (uint64_t i = 0; i < m; ++i) vg::to_public(r[i], a[i0 + i], b[i0 + i], out + i0 + i);
    }
    return VOSS_OK;
  }, VOSS_ERR_INTERNAL);
}

extern "C" int voss_gb300_cut_ranges(uint64_t n, const uint64_t* a, const uint64_t* b,
                                     const uint32_t* gaps_wanted, uint64_t cap, uint64_t* piece_a,
                                     uint64_t* piece_b, uint32_t* piece_gaps, uint64_t* npieces,
                                     uint32_t* first, uint32_t* last) {
  if (!npieces || (n && (!a || !b || !first || !last))) { set_err("null pointer"); return VOSS_ERR_INVALID_ARG; }
  if (n > 0x7FFFFFFFull) { set_err("too many ranges"); return VOSS_ERR_INVALID_ARG; }
  *npieces = 0;
  if (n == 0) return VOSS_OK;
  return guarded([&] {
    std::vector<uint32_t> rf;
    if (gaps_wanted) {
      rf.resize(n);
      for (uint64_t i = 0; i < n; ++i) rf[i] = gaps_wanted[i] ? vg::kReqGaps : 0u;
    }
    std::vector<uint64_t> pa, pb;
    std::vector<uint32_t> pr;
    std::vector<vg::ReqSpan> sp;
    vg::cut_ranges((uint32_t)n, a, b, gaps_wanted ? rf.data() : nullptr, pa, pb, pr, sp);
    *npieces = pa.size();
    if (pa.size() > cap) { set_err("piece arrays too small (2n - 1 always suffices)"); return VOSS_ERR_INVALID_ARG; }
    if (!pa.empty() && (!piece_a || !piece_b)) { set_err("null pointer"); return VOSS_ERR_INVALID_ARG; }
    for (size_t j = 0; j < pa.size(); ++j) {
      piece_a[j] = pa[j];
      piece_b[j] = pb[j];
      if (piece_gaps) piece_gaps[j] = (pr[j] & vg::kReqGaps) ? 1u : 0u;
    }
    for (uint64_t i = 0; i < n; ++i) { first[i] = sp[i].s; last[i] = sp[i].e; }
    return VOSS_OK;
  }, VOSS_ERR_INTERNAL);
}

extern "C" int voss_gb300_get_config(voss_gb300_config_t* out) {
  if (!out) { set_err("null pointer"); return VOSS_ERR_INVALID_ARG; }
  return guarded([&] {
    vg::Engine& E = vg::Engine::for_current_device();
    std::lock_guard<std::mutex> g(E.mu);
    out->seg_bytes = E.cfg.seg_bytes;
    out->threads = E.cfg.threads;
    out->tier_split = E.cfg.tier_split;
    out->ctas_per_sm = E.cfg.ctas_per_sm;
    out->auto_tune = E.cfg.auto_tune;
    out->bucket_split = E.cfg.bucket_split;
    out->bucket_cap_pct = E.cfg.bucket_cap_pct;
    return VOSS_OK;
  }, VOSS_ERR_INTERNAL);
}

extern "C" int voss_gb300_set_config(const voss_gb300_config_t* c) {
  if (!c) { set_err("null pointer"); return VOSS_ERR_INVALID_ARG; }
  if (c->seg_bytes && (c->seg_bytes % 128 || c->seg_bytes < 1024 || c->seg_bytes > vg::kMaxSegBytes)) {
    set_err("seg_bytes must be a multiple of 128 in [1024, " + std::to_string(vg::kMaxSegBytes) + "]");
    return VOSS_ERR_INVALID_ARG;
  }
  if (c->threads && (c->threads % 32 || c->threads > 1024 || c->threads < 64)) {
    set_err("threads must be a multiple of 32 in [64, 1024]");
    return VOSS_ERR_INVALID_ARG;
  }
  if (c->tier_split && c->tier_split < kMinTierSplit) {
    set_err("tier_split must be >= 37");
    return VOSS_ERR_INVALID_ARG;
  }
  if (c->ctas_per_sm > 8) { set_err("ctas_per_sm must be <= 8"); return VOSS_ERR_INVALID_ARG; }
  return guarded([&] {
    vg::Engine& E = vg::Engine::for_current_device();
    std::lock_guard<std::mutex> g(E.mu);
    if (E.servers) throw vg::Error(VOSS_ERR_INVALID_ARG, "a request server is running on this device");
    vg::Config n = E.cfg;
    if (c->seg_bytes) n.seg_bytes = c->seg_bytes;
    if (c->threads) n.threads = c->threads;
    if (c->tier_split) n.tier_split = c->tier_split;
    if (c->ctas_per_sm) n.ctas_per_sm = c->ctas_per_sm;
    n.auto_tune = c->auto_tune ? 1 : 0;
    n.bucket_split = c->bucket_split;
    if (c->bucket_cap_pct) n.bucket_cap_pct = c->bucket_cap_pct;
    if (vg::sieve_smem_bytes(n.seg_bytes, n.threads) > E.max_smem_optin)
      throw vg::Error(VOSS_ERR_INVALID_ARG, "segment does not fit in shared memory");
    E.cfg = n;
    return VOSS_OK;
  }, VOSS_ERR_INTERNAL);
}

extern "C" int voss_gb300_set_tuning(uint32_t n, const voss_gb300_tune_entry_t* e) {
  if (n && !e) { set_err("null pointer"); return VOSS_ERR_INVALID_ARG; }
  for (uint32_t i = 0; i < n; ++i)
    if (e[i].seg_bytes < 1024 || e[i].seg_bytes > vg::kMaxSegBytes || e[i].seg_bytes % 128 ||
        e[i].tier_split < kMinTierSplit) {
      set_err("tuning entry out of range (seg_bytes in [1024, " + std::to_string(vg::kMaxSegBytes) +
              "], multiple of 128; tier_split >= 37)");
      return VOSS_ERR_INVALID_ARG;
    }
  return guarded([&] {
    vg::Engine& E = vg::Engine::for_current_device();
    std::lock_guard<std::mutex> g(E.mu);
    if (E.servers) throw vg::Error(VOSS_ERR_INVALID_ARG, "a request server is running on this device");
    E.tuning.clear();
    for (uint32_t i = 0; i < n; ++i)
      E.tuning.push_back(vg::TuneEntry{e[i].b_max, e[i].width_max, e[i].seg_bytes, e[i].tier_split,
                                       e[i].bucket_split, 0});
    return VOSS_OK;
  }, VOSS_ERR_INTERNAL);
}

extern "C" int voss_gb300_get_tuning(uint32_t cap, voss_gb300_tune_entry_t* e, uint32_t* n) {
  if (!n || (cap && !e)) { set_err("null pointer"); return VOSS_ERR_INVALID_ARG; }
  return guarded([&] {
    vg::Engine& E = vg::Engine::for_current_device();
    std::lock_guard<std::mutex> g(E.mu);
    *n = (uint32_t)E.tuning.size();
    for (uint32_t i = 0; i < cap && i < E.tuning.size(); ++i)
      e[i] = voss_gb300_tune_entry_t{E.tuning[i].b_max, E.tuning[i].width_max, E.tuning[i].seg_bytes,
                                     E.tuning[i].tier_split, E.tuning[i].bucket_split};
    return VOSS_OK;
  }, VOSS_ERR_INTERNAL);
}

struct voss_gb300_plan {
  vg::Plan plan;
  std::vector<uint64_t> a, b;
};

extern "C" int voss_gb300_plan_create(uint64_t n, const uint64_t* a, const uint64_t* b,
                                      voss_gb300_plan** out) {
  if (!out || (n && (!a || !b))) { set_err("null pointer"); return VOSS_ERR_INVALID_ARG; }
  *out = nullptr;
  if (n > 0xFFFFFFFFull) { set_err("too many ranges"); return VOSS_ERR_INVALID_ARG; }
  return guarded([&] {
    vg::Engine& E = vg::Engine::for_current_device();
    std::lock_guard<std::mutex> g(E.mu);
    auto* p = new voss_gb300_plan();
    p->a.assign(a, a + n);
    p->b.assign(b, b + n);
    p->plan.eng = &E;
    p->plan.device = E.device;
    try {
      p->plan.prepare((uint32_t)n, p->a.data(), p->b.data(), 0);
    } catch (...) {
      delete p;
      throw;
    }
    *out = p;
    return VOSS_OK;
  }, VOSS_ERR_INTERNAL);
}

extern "C" int voss_gb300_plan_launch(voss_gb300_plan* p, void* stream) {
  if (!p) { set_err("null plan"); return VOSS_ERR_INVALID_ARG; }
  return guarded([&] {
    p->plan.launch((cudaStream_t)stream);
    return VOSS_OK;
  }, VOSS_ERR_INTERNAL);
}

extern "C" int voss_gb300_plan_results(voss_gb300_plan* p, voss_range_stats_t* out, void* stream) {
  if (!p || (!out && p->plan.nreq)) { set_err("null pointer"); return VOSS_ERR_INVALID_ARG; }
  return guarded([&] {
    const vg::ReqResult* r = p->plan.fetch((cudaStream_t)stream);
    for (uint32_t i = 0; i < p->plan.nreq; ++i) vg::to_public(r[i], p->a[i], p->b[i], out + i);
    return VOSS_OK;
  }, VOSS_ERR_INTERNAL);
}

extern "C" int voss_gb300_plan_info(voss_gb300_plan* p, uint64_t* total_segments, uint32_t* grid,
                                    uint32_t* kernels_per_run, uint32_t* smem_bytes,
                                    uint64_t* clears, uint64_t* wheel_bytes) {
  if (!p) { set_err("null plan"); return VOSS_ERR_INVALID_ARG; }
  return guarded([&] {
    if (total_segments) *total_segments = p->plan.total_segs;
    if (grid) *grid = p->plan.grid;
    if (kernels_per_run)
      *kernels_per_run = p->plan.kernels_per_run();
    if (smem_bytes) *smem_bytes = (uint32_t)vg::sieve_smem_bytes(p->plan.seg_max, p->plan.threads);
    if (clears) *clears = p->plan.algorithmic_clears();
    if (wheel_bytes) *wheel_bytes = p->plan.wheel_bytes();
    return VOSS_OK;
  }, VOSS_ERR_INTERNAL);
}

extern "C" void voss_gb300_plan_free(voss_gb300_plan* p) { delete p; }

extern "C" int voss_gb300_plan_kernel_ms(voss_gb300_plan* p, float* sieve_ms, float* finalize_ms) {
  if (!p) { set_err("null plan"); return VOSS_ERR_INVALID_ARG; }
  return guarded([&] { p->plan.kernel_ms(sieve_ms, finalize_ms); return VOSS_OK; }, VOSS_ERR_INTERNAL);
}

extern "C" int voss_gb300_smem_peak(double* ldst_gbs, double* atomic_gbs) {
  return guarded([&] {
    vg::Engine& E = vg::Engine::for_current_device();
    std::lock_guard<std::mutex> g(E.mu);
    vg::smem_peaks(E, ldst_gbs, atomic_gbs);
    return VOSS_OK;
  }, VOSS_ERR_INTERNAL);
}

extern "C" int voss_gb300_smem_atomic_cost(double* clocks) {
  if (!clocks) { set_err("null pointer"); return VOSS_ERR_INVALID_ARG; }
  return guarded([&] {
    vg::Engine& E = vg::Engine::for_current_device();
    std::lock_guard<std::mutex> g(E.mu);
    vg::smem_atomic_cost(E, clocks);
    return VOSS_OK;
  }, VOSS_ERR_INTERNAL);
}

extern "C" int voss_gb300_device_info(char* name, uint32_t name_len, uint32_t* sm_count) {
  return guarded([&] {
    vg::Engine& E = vg::Engine::for_current_device();
    if (name && name_len) {
      std::strncpy(name, E.name.c_str(), name_len - 1);
      name[name_len - 1] = 0;
    }
    if (sm_count) *sm_count = E.sm_count;
    return VOSS_OK;
  }, VOSS_ERR_INTERNAL);
}

// ---------------------------------------------------------------------------
// Goldbach smallest prime
// ---------------------------------------------------------------------------
static const uint64_t kMaxGoldbachN = 400000000000ull;

extern "C" int voss_primes_goldbach_minp(uint64_t N, uint32_t* minp, uint64_t* hist,
                                         uint32_t* max_minp, uint64_t* sum_minp,
                                         uint64_t* n_ce) {
  if (N < 4) { set_err("N must be >= 4"); return VOSS_ERR_INVALID_N; }
  if (N > kMaxGoldbachN) { set_err("N exceeds maximum (4*10^11)"); return VOSS_ERR_OUT_OF_RANGE; }
  return guarded([&] {
    vg::Engine& E = vg::Engine::for_current_device();
    std::lock_guard<std::mutex> g(E.mu);
    vg::GoldbachResult r = vg::goldbach_run(E, N, minp, 1);
    if (hist) std::memcpy(hist, r.hist.data(), 8 * r.hist.size());
    if (max_minp) *max_minp = r.max_minp;
    if (sum_minp) *sum_minp = r.sum_minp;
    if (n_ce) *n_ce = r.n_counterexamples;
    return VOSS_OK;
  }, VOSS_ERR_INTERNAL);
}

struct voss_gb300_goldbach {
  vg::GoldbachPlan* g = nullptr;
  ~voss_gb300_goldbach() { if (g) vg::goldbach_plan_free(g); }
};

extern "C" int voss_gb300_goldbach_create(uint64_t N, voss_gb300_goldbach** out) {
  if (!out) { set_err("null pointer"); return VOSS_ERR_INVALID_ARG; }
  *out = nullptr;
  if (N < 4) { set_err("N must be >= 4"); return VOSS_ERR_INVALID_N; }
  if (N > kMaxGoldbachN) { set_err("N exceeds maximum (4*10^11)"); return VOSS_ERR_OUT_OF_RANGE; }
  return guarded([&] {
    vg::Engine& E = vg::Engine::for_current_device();
    std::lock_guard<std::mutex> g(E.mu);
    auto* h = new voss_gb300_goldbach();
    h->g = vg::goldbach_plan_create(E, N);
    *out = h;
    return VOSS_OK;
  }, VOSS_ERR_INTERNAL);
}

extern "C" int voss_gb300_goldbach_launch(voss_gb300_goldbach* h, void* stream) {
  if (!h) { set_err("null handle"); return VOSS_ERR_INVALID_ARG; }
  return guarded([&] { vg::goldbach_plan_launch(h->g, (cudaStream_t)stream); return VOSS_OK; },
                 VOSS_ERR_INTERNAL);
}

extern "C" int voss_gb300_goldbach_results(voss_gb300_goldbach* h, uint32_t* max_minp,
                                           uint64_t* sum_minp, uint64_t* n_ce, uint64_t* hist,
                                           uint64_t* probes, void* stream) {
  if (!h) { set_err("null handle"); return VOSS_ERR_INVALID_ARG; }
  return guarded([&] {
    vg::GoldbachResult r;
    vg::goldbach_plan_fetch(h->g, &r, (cudaStream_t)stream);
    if (max_minp) *max_minp = r.max_minp;
    if (sum_minp) *sum_minp = r.sum_minp;
    if (n_ce) *n_ce = r.n_counterexamples;
    if (hist) std::memcpy(hist, r.hist.data(), 8 * r.hist.size());
    if (probes) *probes = vg::goldbach_plan_probes(h->g);
    return VOSS_OK;
  }, VOSS_ERR_INTERNAL);
}

extern "C" void voss_gb300_goldbach_free(voss_gb300_goldbach* h) { delete h; }

// ---------------------------------------------------------------------------
// Request server
// ---------------------------------------------------------------------------
struct voss_gb300_server {
  std::unique_ptr<vg::Server> s;
};

extern "C" int voss_gb300_server_create(const voss_gb300_server_config_t* c, voss_gb300_server** out) {
  if (!out) { set_err("null pointer"); return VOSS_ERR_INVALID_ARG; }
  *out = nullptr;
  return guarded([&] {
    vg::ServerConfig sc;
    if (c) {
      if (c->slots) sc.slots = c->slots;
      if (c->max_batch) sc.max_batch = c->max_batch;
      if (c->max_segments) sc.max_segs = c->max_segments;
      if (c->memory_budget) sc.mem_budget = c->memory_budget;
      if (c->bucket_bytes) sc.bucket_bytes = c->bucket_bytes;
      sc.use_graphs = c->use_graphs;
      sc.share = c->isolate_requests ? 0u : 1u;
    }
    vg::Engine& E = vg::Engine::for_current_device();
    auto* h = new voss_gb300_server();
    try {
      h->s.reset(new vg::Server(E, sc));
    } catch (...) {
      delete h;
      throw;
    }
    *out = h;
    return VOSS_OK;
  }, VOSS_ERR_INTERNAL);
}

extern "C" int voss_gb300_server_submit(voss_gb300_server* h, uint64_t a, uint64_t b, uint32_t op,
                                        uint64_t* ticket) {
  if (!h || !ticket) { set_err("null pointer"); return VOSS_ERR_INVALID_ARG; }
  return guarded([&] { *ticket = h->s->submit(a, b, op); return VOSS_OK; }, VOSS_ERR_INTERNAL);
}

extern "C" int voss_gb300_server_result(voss_gb300_server* h, uint64_t ticket, int wait,
                                        voss_range_stats_t* out, double* latency_us, int* ready) {
  if (!h) { set_err("null pointer"); return VOSS_ERR_INVALID_ARG; }
  return guarded([&] {
    const bool ok = h->s->result(ticket, wait != 0, out, latency_us);
    if (ready) *ready = ok ? 1 : 0;
    return VOSS_OK;
  }, VOSS_ERR_INTERNAL);
}

extern "C" int voss_gb300_server_drain(voss_gb300_server* h) {
  if (!h) { set_err("null pointer"); return VOSS_ERR_INVALID_ARG; }
  return guarded([&] { h->s->drain(); return VOSS_OK; }, VOSS_ERR_INTERNAL);
}

extern "C" int voss_gb300_server_metrics(voss_gb300_server* h, voss_gb300_server_metrics_t* out) {
  if (!h || !out) { set_err("null pointer"); return VOSS_ERR_INVALID_ARG; }
  return guarded([&] { h->s->metrics(out); return VOSS_OK; }, VOSS_ERR_INTERNAL);
}

extern "C" int voss_gb300_server_reset_metrics(voss_gb300_server* h) {
  if (!h) { set_err("null pointer"); return VOSS_ERR_INVALID_ARG; }
  return guarded([&] { h->s->reset_metrics(); return VOSS_OK; }, VOSS_ERR_INTERNAL);
}

extern "C" void voss_gb300_server_free(voss_gb300_server* h) { delete h; }
