// sieve.cuh -- shared layouts of the wheel-30 segmented sieve (device + host).
//
// Bit layout (the reference's, src/voss_w30_v7.cu:38-39 and
// library/src/primes/context.cu:469-470): byte k of the wheel covers the 30
// integers 30k .. 30k+29; bit o of that byte stands for 30k + W30[o] with
// W30 = {1, 7, 11, 13, 17, 19, 23, 29}.  Four bytes form one little-endian
// uint32 word, so bit (k & 3) * 8 + o of word k / 4 is the same bit index
// k * 8 + o that the reference's uint32 `bits` array uses.
#pragma once
#include <cstdint>

namespace vg {

constexpr uint64_t kW30Packed = 0x1D1713110D0B0701ull;  // W30[o] = byte o
constexpr int kHistBins = 1025;       // gap/2 bins 0..1023, bin 1024 = gap >= 2048
constexpr int kSmemBins = 256;        // bins kept in shared memory (gap < 512)
constexpr int kSmemHistCopies = 4;    // one copy per 8 warps
constexpr int kSmemStride = kSmemBins + 4;   // + the overflow bin, padded
constexpr uint32_t kLargeGap = 500;   // the reference's large-gap threshold
// Largest segment: what one CTA's 227 KB of shared memory holds beside the
// histogram copies, the warp records and the byte table of the gap scan.
constexpr uint32_t kMaxSegBytes = 222848;
// The gap scan's byte table: for each value of a wheel byte, the gaps between
// its consecutive candidates (30k + W30[o] for its set bits o) counted per
// gap/2 - 1 = j (j = 0..13, gaps 2..28; at most 4 of one size) in 8-bit
// fields -- even j in .x/.y
// byte j/2, odd j in .z/.w byte (j-1)/2 -- with W30 of the byte's lowest set
// bit in the top byte of .y and of its highest in the top byte of .w.
constexpr uint32_t kByteTabEntries = 256;
constexpr uint32_t kInByteBins = 14;
__host__ __device__ constexpr uint64_t byte_gap_entry(uint32_t x, bool odd) {
  uint64_t e = 0;
  int prev = -1, lo = -1, hi = -1;
  for (int o = 0; o < 8; ++o) {
    if (!((x >> o) & 1u)) continue;
    const int v = (int)((kW30Packed >> (8 * o)) & 0xFFu);
    if (lo < 0) lo = v;
    hi = v;
    if (prev >= 0) {
      const int j = (v - prev) / 2 - 1;
      if ((j & 1) == (odd ? 1 : 0)) e += 1ull << (8 * (j >> 1));
    }
    prev = v;
  }
  const int top = odd ? hi : lo;
  return e | ((uint64_t)(top < 0 ? 0 : top) << 56);
}
// Presieve tiles: the wheel bytes with the multiples of a few small primes
// cleared are periodic, with period the product of those primes (in bytes).
// Four tiles cover the primes 7..59.
constexpr int kTiles = 4;
constexpr uint32_t kTilePrimes[kTiles][4] = {{7, 11, 13, 17}, {19, 23, 29, 31}, {37, 41, 43, 0}, {47, 53, 59, 0}};
__host__ __device__ constexpr uint32_t tile_period(int t) {
  return t == 0 ? 7u * 11u * 13u * 17u      // 17017 bytes
       : t == 1 ? 19u * 23u * 29u * 31u     // 392863 bytes
       : t == 2 ? 37u * 41u * 43u           // 65231 bytes
       :          47u * 53u * 59u;          // 146969 bytes
}
constexpr uint32_t kMaxTilePeriod = 19u * 23u * 29u * 31u;
constexpr uint32_t kFirstTablePrime = 61;   // smallest prime not in a tile

// The tile primes themselves (the tiles clear them as multiples of
// themselves) as bits of the wheel's first bytes, bit 8k + o for
// 30k + W30[o]: 7..29 in byte 0, 31..59 in byte 1.  All tile primes are
// below 90 (bytes 0..2), which the segment fix-ups rely on.
constexpr uint64_t tile_prime_bits() {
  uint64_t m = 0;
  for (int t = 0; t < kTiles; ++t)
    for (int i = 0; i < 4; ++i) {
      const uint32_t q = kTilePrimes[t][i];
      if (!q) continue;
      for (uint32_t o = 0; o < 8; ++o)
        if (((kW30Packed >> (8u * o)) & 0xFFu) == q % 30u) m |= 1ull << (8u * (q / 30u) + o);
    }
  return m;
}
constexpr uint64_t kTilePrimeBits = tile_prime_bits();
static_assert(kTilePrimeBits < (1ull << 24), "tile primes must lie in the wheel's first three bytes");
constexpr int kMaxThreads = 1024;

// The first kConstPrimes table primes (61, 67, 71, ...) with their Barrett
// constants floor((2^64-1)/p), computed at compile time.  Every prime table
// the sieve kernel is given starts with exactly these; the kernel reads them
// from constant memory, where a warp-uniform index is a broadcast.
constexpr uint32_t kConstPrimes = 1024;      // primes 61 .. 8293
struct ConstPrimeTable {
  uint32_t p[kConstPrimes];
  unsigned long long m[kConstPrimes];
};
constexpr ConstPrimeTable make_const_prime_table() {
  ConstPrimeTable t{};
  uint32_t n = 0;
  for (uint32_t c = kFirstTablePrime; n < kConstPrimes; c += 2) {
    bool prime = true;
    for (uint32_t d = 3; d * d <= c && prime; d += 2) prime = c % d != 0;
    if (prime) { t.p[n] = c; t.m[n] = ~0ull / c; ++n; }
  }
  return t;
}

// The presieve tiles are stored as kTileShifts copies, copy c starting c
// bytes into the periodic pattern, so that the pattern at any byte phase
// starts on a 16-byte boundary of one copy: the fill reads them with
// aligned 16-byte loads.
constexpr uint32_t kTileShifts = 16;

// Bytes of one copy of a tile with the given period, for segments of up to
// max_seg bytes (a multiple of 16).
constexpr uint32_t tile_copy_stride(uint32_t period, uint32_t max_seg) {
  return (period + max_seg + 32u + 15u) & ~15u;
}

// Host: the presieve tile of the primes ps (bit o of byte j set iff no p
// divides 30j + W30[o]) as kTileShifts copies of `stride` bytes each, copy c
// holding pattern bytes c, c+1, ...  base: scratch of `period` bytes; out:
// kTileShifts * stride bytes.
inline void build_tile_copies(const uint32_t* ps, int nps, uint32_t period, uint32_t stride,
                              uint8_t* base, uint8_t* out) {
  for (uint32_t j = 0; j < period; ++j) {
    uint8_t v = 0;
    for (uint32_t o = 0; o < 8; ++o) {
      const uint64_t x = 30ull * j + ((kW30Packed >> (8u * o)) & 0xFFu);
      bool comp = false;
      for (int i = 0; i < nps; ++i) comp = comp || x % ps[i] == 0;
      if (!comp) v = (uint8_t)(v | (1u << o));
    }
    base[j] = v;
  }
  for (uint32_t c = 0; c < kTileShifts; ++c) {
    uint8_t* dst = out + (size_t)c * stride;
    uint32_t j = c % period;
    for (uint32_t x = 0; x < stride; ++x) {
      dst[x] = base[j];
      if (++j == period) j = 0;
    }
  }
}

// Flags of one launch.
constexpr uint32_t kFlagBitmap = 1u;     // also write the sieved words out

// One range request, half-open [a, b), as the device sees it.  Each request
// carries its own segment size and tier boundaries (chosen per offset regime).
struct ReqDesc {
  uint64_t a, b;
  uint64_t k_lo, k_hi;      // wheel bytes [k_lo, k_hi) that cover [a, b)
  uint64_t seg_base;        // index of the request's first segment
  uint64_t nseg;
  uint32_t nprimes;         // table primes p (>= 61) with p*p < b
  uint32_t seg_bytes;       // this request's segment size (<= the launch's)
  uint32_t tier_split;      // table index of the first mid-tier prime
  uint32_t tier_huge;       // table index of the first prime >= seg_bytes
  uint32_t rflags;          // kReqGaps: gap histogram and largest gap wanted
  uint32_t bucket_idx;      // table index of the first bucket prime (= nprimes: none)
  uint64_t bucket_base;     // first entry of this request's bucket lists
  uint32_t bucket_cap;      // entries per segment list
  uint32_t pad;
};

constexpr uint32_t kReqGaps = 1u;
// Segments whose bucket lists are filled and held at once: a request of
// more segments is sieved in windows of this many, the lists of one window
// reusing the same memory (fill-kernel shared counts, 16-bit packing, and
// window offsets below 2^30 bytes).
constexpr uint32_t kMaxBucketSegs = 4096;
constexpr uint32_t kHugeHalf = 32;           // primes per half of a huge-tier work unit (one per lane)
constexpr uint32_t kBucketUnit = 1024;       // list entries per work unit of the sieve kernel
constexpr uint32_t kFillPrimes = 256;        // bucket primes per fill work item
constexpr uint32_t kFillHits = 16384;        // list entries per fill work item, about

// A bucket list entry: the segment-local bit index 8 * byte + class, so that
// entry / 32 is the word and entry mod 32 the bit within it.
__host__ __device__ constexpr uint32_t bucket_entry(uint32_t off, uint32_t o) { return (off << 3) | o; }

// One fill work item: the hits of bucket primes [p0, p1) (table indices) of
// request req that fall in its segments [g0, g1), packed g0 | g1 << 16.
struct FillItem {
  uint32_t req, p0, p1, segs;
};

// Batch header in device memory: a captured launch reads its size from here,
// so one CUDA graph serves every batch of a slot.
struct BatchHdr {
  uint64_t total_segs;
  uint32_t nreq;            // device requests (atoms, when requests share work)
  uint32_t nfill;           // bucket fill items
  uint32_t nout;            // caller requests rebuilt from atoms (0: none)
  uint32_t pad;
};

// Per-launch control words, zeroed together before each run.
struct PlanCtl {
  unsigned long long queue;   // work-queue head: next (request, segment) item
  unsigned int nlarge;        // large gaps recorded
  unsigned int overflow;      // a bucket list ran out of room
};

// A region to zero, in 16-byte units.
struct ZeroSpan {
  void* p;
  uint64_t n16;
};

// A caller request served from shared atoms: its atoms are [s, e) in
// position order.
struct ReqSpan {
  uint32_t s, e, rflags, pad;
};

// Per segment: first/last prime (absolute, 0 = none), the largest gap
// strictly inside the segment and its first prime, the prime count.
struct SegRec {
  uint64_t first, last;
  uint64_t max_gap_start;
  uint32_t max_gap;
  uint32_t count;
};

// Per request accumulators (global atomics).  Counts are of wheel primes
// (>= 7) only; the finalize step adds 2, 3, 5.
struct ReqAccum {
  unsigned long long count, c41, c31;
  unsigned long long hist[kHistBins];
};

// A gap >= kLargeGap: position = second prime (the reference's convention).
struct LargeGapRec {
  uint64_t pos;
  uint32_t gap;
  uint32_t req;
};

// Final per request result, written by the finalize kernel.
struct ReqResult {
  uint64_t count;
  uint64_t c41, c43, c31, c32;
  uint64_t first, last;
  uint64_t max_gap, max_gap_start;
  uint64_t num_gaps;
  uint64_t hist[kHistBins];
};

struct SieveParams {
  const ReqDesc* reqs;
  const BatchHdr* hdr;
  unsigned long long* queue;   // work-queue head: next (request, segment) item
  const uint32_t* P;         // table primes >= 61, ascending
  const uint64_t* M;         // floor((2^64-1)/p), for x mod p
  const uint32_t* R;         // R[8 * i + o]: k = R (mod p) <=> p | 30k+W30[o] (32 B per prime)
  const uint32_t* tile[kTiles];      // presieve tiles: kTileShifts shifted copies each
  uint32_t tile_stride16[kTiles];    // 16-byte units per copy
  uint32_t seg_bytes;        // the largest segment of the launch (shared memory)
  SegRec* segs;
  ReqAccum* acc;
  LargeGapRec* large;
  unsigned int* n_large;
  uint32_t large_cap;
  uint32_t flags;
  uint32_t* bitmap;          // kFlagBitmap: words of request 0, from k_lo
  const uint32_t* bucket;    // bucket list entries
  const uint32_t* bcount;    // entries written per segment (indexed like segs)
  // Work items of this launch: [item_lo, min(item_hi, total_segs)), item_hi
  // 0 standing for total_segs; a windowed plan launches once per window.  The bucket list of segment si of
  // a request sits at slot si - list_seg0 (the window's first segment).
  uint64_t item_lo, item_hi;
  uint64_t list_seg0;
};

struct FillParams {
  const ReqDesc* reqs;
  const BatchHdr* hdr;
  const FillItem* items;
  const uint32_t* P;
  const uint64_t* M;
  const uint32_t* R;
  uint32_t* bucket;
  uint32_t* bcount;
  unsigned int* overflow;
  uint32_t nitems;          // fill items of this launch (0: the batch header's nfill)
  uint32_t seg0;            // the window's first segment: item segments count from it
};

}  // namespace vg
