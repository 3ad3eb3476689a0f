// engine.h -- host side of the GB300 sieve: resident prime table, presieve
// tiles, launch plans.  Internal C++ (throws vg::Error); the C ABI in
// capi.cpp turns errors into VOSS_* codes.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "sieve.cuh"
#include "voss/voss_gb300.h"

namespace vg {

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

void check_cuda(cudaError_t e, const char* what);

// Largest b (exclusive) a range may end at: 10^14 + 10^10 + 1.
constexpr uint64_t kMaxB = 100000000000000ull + 10000000000ull + 1ull;

uint64_t isqrt_u64(uint64_t x);

// Device buffer that only grows.
struct DevBuf {
  void* ptr = nullptr;
  size_t bytes = 0;
  void reserve(size_t n);
  void release();
  template <class T> T* as() const { return static_cast<T*>(ptr); }
  ~DevBuf() { release(); }
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
};

struct HostPinned {
  void* ptr = nullptr;
  size_t bytes = 0;
  void reserve(size_t n);
  ~HostPinned();
  HostPinned() = default;
  HostPinned(const HostPinned&) = delete;
  HostPinned& operator=(const HostPinned&) = delete;
};

struct Config {
  uint32_t seg_bytes = kMaxSegBytes;    // the largest that fits (227 KB of shared memory per CTA)
  uint32_t threads = 1024;
  uint32_t tier_split = 6144;    // primes below: a warp per prime; above: 4 per warp
  uint32_t ctas_per_sm = 1;
  uint32_t auto_tune = 1;
  uint32_t bucket_split = 0;   // with auto_tune off: bucket primes from here (0 = none)
  uint32_t bucket_cap_pct = 100;   // bucket list capacity, percent of the safe size
};

class Engine;

// A prepared batch of ranges with its device buffers.
//
// load() writes the request descriptors and the batch header into pinned
// staging memory; upload() copies them to the device; run_device() is the
// device part (memsets, sieve, finalize) with fixed pointers and sizes, so it
// can be captured into a CUDA graph once and replayed for every batch that
// fits the plan's capacity (the kernels read the batch size from the device
// header).  Requests are reordered by estimated cost, heaviest first, so the
// work queue ends on light items; results come back in the caller's order.
struct Plan {
  Engine* eng = nullptr;
  int device = 0;
  uint32_t nreq = 0;
  uint64_t total_segs = 0;
  uint32_t cap_req = 0;         // fixed capacity (graph-replayed plans); 0 = exact
  uint64_t cap_segs = 0;
  uint32_t seg_max = 0;         // shared-memory segment of the launch
  uint32_t threads = 1024;
  uint32_t grid = 0;
  bool batch_mode = false;      // tune for throughput of many ranges
  std::vector<ReqDesc> host_reqs;   // device order
  std::vector<uint32_t> order;      // host_reqs[i] is the caller's request order[i]
  DevBuf hdr;                   // BatchHdr followed by ReqDesc[] (one upload)
  DevBuf ctl;                   // PlanCtl: work queue, large-gap count, overflow flag
  DevBuf segs, acc, large, results, bitmap;
  DevBuf bucket, bcount, fills;   // bucket sieve lists, per-segment counts, fill items
  ReqDesc* dreqs() const { return reinterpret_cast<ReqDesc*>(static_cast<char*>(hdr.ptr) + sizeof(BatchHdr)); }
  PlanCtl* dctl() const { return ctl.as<PlanCtl>(); }
  uint64_t bucket_entries = 0;  // entries reserved by the current batch
  uint64_t cap_bucket = 0;      // fixed arena (graph-replayed plans); 0 = exact
  uint32_t nfill = 0;
  uint32_t cap_fill = 0;
  bool allow_buckets = true;
  // Shared atoms: a batch's ranges are cut at every endpoint into disjoint
  // atoms, each sieved once (with gap outputs if any request over it wants
  // them); combine_kernel then rebuilds each caller request from its atoms.
  bool share = false;
  uint32_t nout = 0;            // caller requests of a shared batch (0: not shared)
  uint32_t cap_out = 0;         // fixed capacity of caller requests (shared plans)
  DevBuf spans, apos, rres;     // ReqSpan per caller, atom device index by position, caller results
  std::vector<ReqSpan> host_spans;
  std::vector<uint32_t> host_apos;
  std::vector<uint64_t> atom_a, atom_b;
  std::vector<uint32_t> atom_rf;
  std::vector<FillItem> host_fills;
  std::vector<FillItem> item_buf;   // one request's fill items, before the capacity check
  // A lone request of more than kMaxBucketSegs segments with bucket lists
  // (plans without a fixed capacity only) runs in windows of kMaxBucketSegs
  // segments: per window a fill of its lists (host_fills[fill_lo, fill_hi),
  // segments counted from seg0) and a sieve launch over its work items, all
  // windows reusing one list arena.  Empty: one fill and one sieve launch.
  struct Window {
    uint64_t item_lo, item_hi;
    uint32_t fill_lo, fill_hi;
    uint32_t seg0;
  };
  std::vector<Window> wins;
  HostPinned stage;             // BatchHdr followed by ReqDesc[cap]
  HostPinned host_results;      // ReqResult[] in device order (caller order when shared)
  HostPinned host_flag;         // the overflow flag, copied with the results
  std::vector<ReqResult> out;   // caller order
  uint32_t large_cap = 1u << 16;
  uint32_t flags = 0;
  SieveParams prm{};
  cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};   // before sieve, after sieve, after finalize
  bool timed = true;            // record ev[] on each run (for kernel_ms)

  ~Plan();
  Plan() = default;
  Plan(const Plan&) = delete;
  Plan& operator=(const Plan&) = delete;

  // Kernels per run (zeroing + sieve + finalize; the bucket fill comes on top
  // when the run has lists, combine when it shares atoms).
  static constexpr uint32_t kKernels = 3;

  // Fix the capacity (requests, segments, bucket entries) of a
  // graph-replayed plan.  With share set, max_req and max_segs are the
  // caller's limits; the atoms get room for at most 2*max_req - 1 pieces,
  // each adding at most two partial segments.
  void reserve_capacity(uint32_t max_req, uint64_t max_segs, uint64_t max_bucket_entries = 0);
  // rflags: per request kReqGaps (NULL = all requests want gaps)
  void load(uint32_t n, const uint64_t* a, const uint64_t* b, uint32_t flags,
            const uint32_t* rflags = nullptr);
  // The device requests themselves (load() passes atoms here when sharing).
  void load_requests(uint32_t n, const uint64_t* a, const uint64_t* b, uint32_t flags,
                     const uint32_t* rflags);
  void upload(cudaStream_t s);
  void run_device(cudaStream_t s);
  void prepare(uint32_t n, const uint64_t* a, const uint64_t* b, uint32_t flags);
  void launch(cudaStream_t s) { upload(s); run_device(s); }
  // Capture run_device() into a CUDA graph (the plan must have a fixed
  // capacity); launch_graph() replays it for the currently loaded batch.
  void capture(cudaStream_t s);
  void launch_graph(cudaStream_t s);
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
  // Copy results of the last run to host memory (caller order).
  const ReqResult* fetch(cudaStream_t s);
  // Queue the device-to-host copy of the results without waiting; finish()
  // then reorders them (after the stream has reached that point).
  void fetch_async(cudaStream_t s);
  const ReqResult* finish();
  std::vector<LargeGapRec> fetch_large(cudaStream_t s);
  uint64_t algorithmic_clears() const;
  uint64_t wheel_bytes() const;
  // Durations of the sieve and finalize kernels of the last launch (CUDA
  // events recorded on the launching stream).
  void kernel_ms(float* sieve_ms, float* finalize_ms);
  // Segments a range needs under this plan's tuning (for admission).
  uint64_t segments_for(uint64_t a, uint64_t b) const;
  // Bucket-list bytes a range needs under this plan's tuning (for admission);
  // 0 while the plan runs without lists.
  uint64_t bucket_bytes_for(uint64_t a, uint64_t b) const;
  // The same when lists are allowed; reads no mutable plan state, so another
  // thread may call it while this plan runs.
  uint64_t list_bytes_for(uint64_t a, uint64_t b) const;
  // True if the last run's bucket lists overflowed (its results are then
  // invalid); valid once the stream has passed fetch_async().
  bool overflowed() const;
  // resident CTAs of the bucket fill kernel over the whole GPU
  uint32_t fill_grid_max() const;
  // kernel launches of one run
  uint32_t kernels_per_run() const;
};

// Bucket layout of one request: first bucket prime, list capacity per
// segment.  bucket_idx = nprimes when the request does not use buckets.
struct BucketPlan {
  uint32_t bucket_idx;
  uint32_t cap;
};

// One entry of the offset-regime tuning table: ranges with b <= b_max and
// width <= width_max use this segment size and tier split.
struct TuneEntry {
  uint64_t b_max;
  uint64_t width_max;
  uint32_t seg_bytes;
  uint32_t tier_split;
  uint32_t bucket_split;   // primes from here on go through bucket lists; 0 = none
  uint32_t pad;
};

class Engine {
 public:
  static Engine& for_current_device();

  std::mutex mu;     // one caller at a time per device
  int device = 0;
  uint32_t sm_count = 0;
  size_t max_smem_optin = 0;    // dynamic shared memory the sieve kernel may ask for
  std::string name;
  cudaStream_t stream = nullptr;
  Config cfg;
  // Request servers alive on this engine (guarded by mu).  Their threads read
  // cfg and tuning without mu, so neither may change while one runs.
  int servers = 0;

  // Resident sieving-prime table: primes >= 61 up to table_limit.
  std::vector<uint32_t> hP;
  std::vector<double> hInvPrefix;   // sum of 1/p over table primes [0, i)
  uint64_t table_limit = 0;
  DevBuf dP, dM, dR;            // primes, Barrett constants, class residues (8 per prime)
  // Earlier, smaller copies of the table.  Plans keep pointers to the table
  // they were built with, so a grown table leaves the old one allocated (its
  // primes are a prefix of the new one's) until the engine goes.
  std::vector<std::unique_ptr<DevBuf>> retired_tables;
  DevBuf tile[kTiles];        // presieve tiles, kTileShifts shifted copies each

  // Scratch plan reused by the synchronous entry points.
  Plan scratch;

  void ensure_table(uint64_t pmax);
  uint32_t primes_below_sq(uint64_t b) const;   // table primes p with p*p < b
  uint32_t index_of(uint32_t p) const;           // first table index with P >= p
  // Segment size and tier split for one range (offset-regime table, then the
  // built-in rule); batch = tune for the throughput of a batch rather than
  // the latency of this range alone.
  Config tuned_for(uint64_t a, uint64_t b, bool batch = false) const;
  // Bucket layout for a range with the given segment size and segment count.
  BucketPlan bucket_plan(const Config& c, uint64_t b, uint32_t nprimes, uint64_t nseg,
                         uint32_t seg_bytes) const;
  std::vector<TuneEntry> tuning;

  // Run ranges synchronously on the engine stream.  share: overlapping
  // ranges sieve their common integers once (not with large-gap output).
  const ReqResult* run(uint32_t n, const uint64_t* a, const uint64_t* b,
                       std::vector<LargeGapRec>* large = nullptr, bool gaps = true,
                       bool share = false);

 private:
  Engine() = default;
  void init();
  void build_tiles();
};

void smem_peaks(Engine& E, double* ldst_gbs, double* atomic_gbs);
// SM clocks per warp-wide shared atomicAnd with the lanes' banks distinct,
// 2-way, 4-way and 8-way shared, and scattered.
void smem_atomic_cost(Engine& E, double clocks[5]);

void to_public(const ReqResult& r, uint64_t a, uint64_t b, voss_range_stats_t* out);
// The result of a range from the results of its consecutive pieces (in order):
// counts add; with gaps, each junction between pieces that hold primes adds
// one gap, and the largest gap is the largest of the pieces' and the
// junctions' (the earliest on ties), as within one range.
ReqResult merge_ordered(const ReqResult* parts, size_t n, bool gaps);

// Launchers defined in sieve.cu.
size_t sieve_smem_bytes(uint32_t seg_bytes, uint32_t threads);
size_t sieve_static_smem_bytes();      // the sieve kernel's static shared memory
cudaError_t launch_sieve(const SieveParams& prm, uint32_t grid, uint32_t threads,
                         cudaStream_t stream);
cudaError_t launch_bucket_fill(const FillParams& fp, uint32_t grid, cudaStream_t stream);
uint32_t bucket_fill_ctas_per_sm();      // resident fill CTAs per SM (occupancy query, cached)
// Cut a batch's ranges at every endpoint into the disjoint pieces some range
// covers (ascending); a piece gets kReqGaps if a range over it asks for gaps
// (rflags NULL: all do).  spans[i] = the pieces [s, e) that tile range i.
void cut_ranges(uint32_t n, const uint64_t* a, const uint64_t* b, const uint32_t* rflags,
                std::vector<uint64_t>& atom_a, std::vector<uint64_t>& atom_b,
                std::vector<uint32_t>& atom_rf, std::vector<ReqSpan>& spans);

cudaError_t launch_zero(ZeroSpan z0, ZeroSpan z1, ZeroSpan z2, uint32_t max_grid, cudaStream_t stream);
cudaError_t launch_combine(const BatchHdr* hdr, const ReqSpan* spans, const uint32_t* apos,
                           const ReqResult* ares, ReqResult* out, uint32_t grid, cudaStream_t stream);
cudaError_t launch_finalize(const ReqDesc* reqs, const BatchHdr* hdr, const SegRec* segs,
                            ReqAccum* acc, LargeGapRec* large, unsigned int* n_large,
                            uint32_t large_cap, ReqResult* out, uint32_t grid,
                            cudaStream_t stream);

}  // namespace vg
