// sieve.cu -- wheel-30 segmented sieve with fused reductions, for sm_103a.
//
// One CTA owns one segment of S bytes (30*S integers) at a time, entirely in
// shared memory, and takes (request, segment) items from a device work queue
// (one global atomic per item; requests come heaviest first).  Per segment:
//   1. fill: AND of four presieve tiles (primes 7..17, 19..31, 37..43,
//      47..59) read at the segment's phase, 16 bytes per load from the tile
//      copy in which that phase is aligned -- replaces the reference's memset + per-prime
//      launches for the smallest primes (context.cu:404-414);
//   2. mark with shared-memory atomicAnd, in work units handed out heaviest
//      first by a shared counter: primes 61 <= p < split one warp each
//      (lane = residue class x stream, fixed bit mask per stream); split <=
//      p < S four per warp-round (lane = prime x class); p >= S two per
//      lane (at most one hit per class); primes from the request's bucket
//      split on come from the segment's bucket list, 1024 entries per unit,
//      read coalesced from HBM (filled by bucket_fill_kernel).  Each stream
//      starts at max(p^2, segment low), as the reference's
//      sieve_w30_seg_kernel does (sieve.cu:10-37, start offsets
//      context.cu:354-388);
//   3. reduce in the same CTA: popcount (count), masked popcount (p mod 4,
//      p mod 3), and an ordered gap scan with a warp max-scan carrying the
//      previous prime, histogram in shared memory -- replaces extract +
//      thrust::sort + mod4 + gaps kernels (extract.cu:10-39,
//      chebyshev.cu:11-25, gaps.cu:31-75).  Count-only requests skip the
//      gap scan.
// Segment boundaries, 2/3/5 and request totals are stitched by
// finalize_kernel (the reference does this on the host, context.cu:462-524);
// combine_kernel rebuilds requests that shared atoms of a batch.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "attr_cache.h"
#include "sieve.cuh"

namespace vg {

__device__ __forceinline__ uint32_t w30(uint32_t o) {
  return (uint32_t)((kW30Packed >> (o << 3)) & 0xFFu);
}

__constant__ ConstPrimeTable cTab = make_const_prime_table();

// x mod p by Barrett reduction with m = floor((2^64-1)/p).
__device__ __forceinline__ uint32_t mod_barrett(uint64_t x, uint32_t p, uint64_t m) {
  uint64_t q = __umul64hi(x, m);
  uint64_t r = x - q * (uint64_t)p;
  return (uint32_t)(r >= p ? r - p : r);
}

// First hit (segment-local byte) of class o of prime p, moved up so that the
// number it stands for is >= p*p.  Returns >= nbytes if there is none.
__device__ __forceinline__ uint32_t lift_to_square(uint32_t s, uint64_t k0, uint32_t p,
                                                   uint32_t o, uint32_t nbytes) {
  const uint64_t n = 30ull * (k0 + s) + w30(o);
  const uint64_t p2 = (uint64_t)p * p;
  if (n >= p2) return s;
  const uint64_t step = 30ull * p;
  const uint64_t add = ((p2 - n + step - 1) / step) * p;
  const uint64_t s2 = s + add;
  return s2 < nbytes ? (uint32_t)s2 : nbytes;
}

// Clear the candidate of byte j, class o, given keep = ~(1 << o): the mask
// is keep rotated to byte j & 3 of its word (a funnel shift uses its count
// mod 32, so 8 * j rotates by 8 * (j & 3)).
__device__ __forceinline__ void clear_bit(uint32_t* seg, uint32_t j, uint32_t keep) {
  atomicAnd(seg + (j >> 2), __funnelshift_l(keep, keep, j << 3));
}

// The eight class residues of table prime i (32 bytes, two vector loads).
__device__ __forceinline__ void load_residues(const uint32_t* __restrict__ R, uint32_t i, uint32_t r[8]) {
  const uint4 lo = __ldg(reinterpret_cast<const uint4*>(R) + 2u * i);
  const uint4 hi = __ldg(reinterpret_cast<const uint4*>(R) + 2u * i + 1u);
  r[0] = lo.x; r[1] = lo.y; r[2] = lo.z; r[3] = lo.w;
  r[4] = hi.x; r[5] = hi.y; r[6] = hi.z; r[7] = hi.w;
}

struct GapSink {
  uint32_t* shist;           // this warp's shared histogram copy
  ReqAccum* acc;             // this request's global accumulators
  LargeGapRec* large;
  unsigned int* n_large;
  uint32_t cap;
  uint32_t req;
  uint64_t base;             // 30 * k0: absolute value of relative 0
};

// Count the gap v - vprev.  Shared bins hold gap/2 < kSmemBins; one extra
// shared bin (never flushed) absorbs larger gaps, which take the rare path
// together with a new maximum and gaps >= kLargeGap.
__device__ __forceinline__ void record_gap(const GapSink& sk, uint32_t vprev, uint32_t v,
                                           uint32_t& maxg, uint32_t& maxgs) {
  const uint32_t g = v - vprev;
  const uint32_t bin = g >> 1;
  atomicAdd(sk.shist + min(bin, (uint32_t)kSmemBins), 1u);
  // rare: a new maximum, g >= kLargeGap, or g >= 2*kSmemBins (> kLargeGap)
  if (g > min(maxg, kLargeGap - 1u)) {
    if (g > maxg) { maxg = g; maxgs = vprev; }
    if (bin >= (uint32_t)kSmemBins)
      atomicAdd(&sk.acc->hist[bin < (uint32_t)kHistBins ? bin : kHistBins - 1], 1ull);
    if (g >= kLargeGap) {
      const unsigned idx = atomicAdd(sk.n_large, 1u);
      if (idx < sk.cap) {
        LargeGapRec r; r.pos = sk.base + v; r.gap = g; r.req = sk.req;
        sk.large[idx] = r;
      }
    }
  }
}

// A claimed (request, segment) work item with what the CTA needs of it.
// The edge masks fix the segment's first word, w = ((w & and0) | or0) &
// keep0, and its last word, w &= keepl: the tile primes themselves (7..29
// live in wheel byte 0, 31 in byte 1), 1, and the request's ends.
struct SegItem {
  uint64_t item, k0, bbase;
  uint32_t req, nbytes, np, split, huge, rflags, bcnt, valid;
  uint32_t and0, or0, keep0, keepl;
};

// Number of leading i in [0, n) for which pred(i) holds (pred holds on a
// prefix), by a 32-ary search of one warp: each step probes 32 evenly spaced
// points, so about log32(n) dependent loads instead of log2(n).
template <class Pred>
__device__ __forceinline__ uint32_t warp_count_leading(uint32_t n, uint32_t lane, Pred pred) {
  uint32_t lo = 0, hi = n;                      // the answer is in [lo, hi]
  while (lo < hi) {
    const uint32_t step = (hi - lo + 31u) / 32u;
    const uint32_t idx = lo + lane * step;
    const bool t = idx < hi && pred(idx);
    const uint32_t k = (uint32_t)__popc(__ballot_sync(0xFFFFFFFFu, t));
    if (k == 0) break;                          // pred(lo) fails: the answer is lo
    const uint32_t last_true = lo + (k - 1u) * step;
    hi = min(hi, lo + k * step);                // first probe that failed (or the end)
    lo = last_true + 1u;
  }
  return lo;
}

// Claim the next work item and look it up, by one whole warp: its request
// (the last with seg_base <= item), its bytes, the table primes with p*p
// below its upper end, and its bucket list.  Lane 0 writes d.
__device__ __noinline__ void claim_item(unsigned long long* queue, const ReqDesc* __restrict__ reqs,
                                        const uint32_t* __restrict__ P, const uint32_t* __restrict__ bcount,
                                        uint64_t item_lo, uint64_t item_end, uint64_t list_seg0,
                                        uint32_t nreq, SegItem& d, uint32_t lane) {
  unsigned long long it = 0;
  if (lane == 0) it = atomicAdd(queue, 1ull);
  const uint64_t item = item_lo + __shfl_sync(0xFFFFFFFFu, it, 0);
  if (item >= item_end) {
    if (lane == 0) { d.item = item; d.valid = 0; }
    return;
  }
  const uint32_t r = warp_count_leading(nreq, lane, [&](uint32_t i) { return reqs[i].seg_base <= item; }) - 1u;
  const ReqDesc& R = reqs[r];
  const uint64_t si = item - R.seg_base;
  const uint64_t k0 = R.k_lo + si * R.seg_bytes;
  const uint64_t left = R.k_hi - k0;
  const uint32_t nb = left < R.seg_bytes ? (uint32_t)left : R.seg_bytes;
  const uint64_t hi_num = 30ull * (k0 + nb);
  // only primes up to the bucket split matter (the rest come from the list)
  const uint32_t lim = R.bucket_idx < R.nprimes ? R.bucket_idx + 1u : R.nprimes;
  uint32_t a = warp_count_leading(lim, lane, [&](uint32_t i) {
    const uint64_t p = P[i];
    return p * p < hi_num;
  });
  if (lane == 0) {
    d.bcnt = 0;
    d.bbase = 0;
    if (R.bucket_idx < a) {
      a = R.bucket_idx;
      d.bcnt = min(bcount[item], R.bucket_cap);
      d.bbase = R.bucket_base + (si - list_seg0) * (uint64_t)R.bucket_cap;
    }
    d.item = item; d.valid = 1;
    d.req = r; d.k0 = k0; d.nbytes = nb; d.np = a;
    d.split = R.tier_split; d.huge = R.tier_huge; d.rflags = R.rflags;
    uint32_t and0 = ~0u, or0 = 0u, keep0 = ~0u, keepl = ~0u;
    if (k0 == 0) and0 = ~1u;                               // 1 is not prime
    if (k0 < 3) or0 = (uint32_t)(kTilePrimeBits >> (8u * k0));   // the tile primes are
    if (si == 0) {                                         // numbers below a
      for (uint32_t o = 0; o < 8; ++o)
        if (30ull * k0 + w30(o) < R.a) keep0 &= ~(1u << o);
    }
    if (k0 + nb == R.k_hi) {                               // numbers from b on
      const uint32_t lb = nb - 1;
      uint32_t m = 0;
      for (uint32_t o = 0; o < 8; ++o)
        if (30ull * (k0 + lb) + w30(o) >= R.b) m |= 1u << o;
      keepl = ~(m << ((lb & 3u) << 3));
      const uint32_t rem = nb & 3u;                        // bytes past the end
      if (rem) keepl &= (1u << (rem << 3)) - 1u;
    }
    d.and0 = and0; d.or0 = or0; d.keep0 = keep0; d.keepl = keepl;
  }
}

// Shared-memory per-warp record used to stitch warps inside a segment.
struct WarpRec {
  uint32_t first1, last1;    // relative value + 1 (0 = none)
  uint32_t cnt, c41, c31;
  uint32_t maxg, maxgs;
  uint32_t pad;
};

__global__ void __launch_bounds__(kMaxThreads, 1)
sieve_segments_kernel(const SieveParams prm) {
  extern __shared__ __align__(16) uint32_t smem[];
  uint32_t* seg = smem;
  uint32_t* shist = seg + (prm.seg_bytes >> 2);
  WarpRec* wrec = reinterpret_cast<WarpRec*>(shist + kSmemHistCopies * kSmemStride);
  uint4* btab = reinterpret_cast<uint4*>(wrec + kMaxThreads / 32);   // the gap scan's byte table

  // the segment in hand, s_item[cur], and the next one, s_item[cur ^ 1],
  // claimed and looked up by warp 0 while the others mark (so no thread
  // waits on that lookup)
  __shared__ SegItem s_item[2];
  __shared__ uint32_t s_ctr;
  __shared__ uint32_t s_vtab[32];      // bit b of a word -> 30*(b/8) + W30[b%8]

  const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  const uint32_t nthr = blockDim.x, nwarps = nthr >> 5;

  for (uint32_t i = tid; i < kSmemHistCopies * kSmemStride; i += nthr) shist[i] = 0;
  if (tid < 32) s_vtab[tid] = 30u * (tid >> 3) + w30(tid & 7u);
  for (uint32_t i = tid; i < kByteTabEntries; i += nthr) {
    const uint64_t e = byte_gap_entry(i, false), od = byte_gap_entry(i, true);
    btab[i] = make_uint4((uint32_t)e, (uint32_t)(e >> 32), (uint32_t)od, (uint32_t)(od >> 32));
  }
  if (tid == 0) s_ctr = 0;
  int cur_req = -1;

  const uint64_t total_segs = prm.hdr->total_segs;
  const uint64_t item_end = prm.item_hi ? min(total_segs, prm.item_hi) : total_segs;
  const uint32_t nreq = prm.hdr->nreq;
  uint32_t cur = 0;
  if (warp == 0) claim_item(prm.queue, prm.reqs, prm.P, prm.bcount, prm.item_lo, item_end, prm.list_seg0, nreq, s_item[0], lane);
  __syncthreads();
  // Three barriers per segment: after the fill, after the marking, before
  // the warps are stitched.  No thread reads the segment after the last one,
  // so the next fill follows it directly.
  for (;; cur ^= 1u) {
    // work queue: the next (request, segment) item, heaviest requests first
    const SegItem& S = s_item[cur];
    if (!S.valid) break;
    const uint64_t item = S.item;
    const uint32_t req = S.req;
    const uint64_t k0 = S.k0;
    const uint32_t nbytes = S.nbytes;
    const uint32_t nwords = (nbytes + 3u) >> 2;
    const uint32_t np = S.np;

    if ((int)req != cur_req) {
      if (cur_req >= 0) {                           // flush the previous request's bins
        __syncthreads();                            // after warp 0's last stitching gaps
        for (uint32_t bn = tid; bn < (uint32_t)kSmemBins; bn += nthr) {
          uint32_t s = 0;
#pragma unroll
          for (int c = 0; c < kSmemHistCopies; ++c) { s += shist[c * kSmemStride + bn]; shist[c * kSmemStride + bn] = 0; }
          if (s) atomicAdd(&prm.acc[cur_req].hist[bn], (unsigned long long)s);
        }
      }
      cur_req = (int)req;
    }

    // 1. presieve fill
    {
      // copy (phase mod 16) of each tile holds the phase on a 16-byte boundary
      uint32_t toff[kTiles];                       // 16-byte units from each tile's start
#pragma unroll
      for (int t = 0; t < kTiles; ++t) {
        const uint32_t ph = (uint32_t)(k0 % tile_period(t));
        toff[t] = (ph & 15u) * prm.tile_stride16[t] + (ph >> 4);
      }
      uint4* seg4 = reinterpret_cast<uint4*>(seg);
      const uint32_t n16 = (nbytes + 15u) >> 4;    // up to 3 words past the end: never read
#pragma unroll 4
      for (uint32_t v = tid; v < n16; v += nthr) {
        uint4 x = __ldg(reinterpret_cast<const uint4*>(prm.tile[0]) + toff[0] + v);
#pragma unroll
        for (int t = 1; t < kTiles; ++t) {
          const uint4 y = __ldg(reinterpret_cast<const uint4*>(prm.tile[t]) + toff[t] + v);
          x.x &= y.x; x.y &= y.y; x.z &= y.z; x.w &= y.w;
        }
        seg4[v] = x;
      }
    }
    __syncthreads();

    // 2. marking.  Work units, heaviest first, handed out by a shared counter:
    //    units [0, nsmall): one prime each, p < split: a warp per prime, lane
    //      = (class o, stream h of 4); a stream steps 4p bytes = p words, so
    //      its bit mask never changes;
    //    then 32 primes each, split <= p < S: lanes = (prime q of 4, class
    //      o), eight rounds of four primes, loads of all rounds issued before
    //      any marking so their latency overlaps;
    //    then 64 primes each, p >= S (two per lane), then the bucket units.
    {
      // unit layout: [0, nsmall) small primes, then 32-prime units of the mid
      // tier (split <= p < S), then 64-prime units of the huge tier (p >= S),
      // then kBucketUnit-entry units of the segment's bucket list
      const uint32_t nsmall = S.split < np ? S.split : np;
      const uint32_t hbeg = S.huge < np ? max(S.huge, nsmall) : np;
      const uint32_t nmidu = (hbeg - nsmall + 31u) / 32u;
      const uint32_t nhugeu = (np - hbeg + 2u * kHugeHalf - 1u) / (2u * kHugeHalf);
      const uint32_t nscan = nsmall + nmidu + nhugeu;
      const uint32_t bcnt = S.bcnt;
      const uint64_t bbase = S.bbase;
      if (warp == 0)                                // overlaps the marking
        claim_item(prm.queue, prm.reqs, prm.P, prm.bcount, prm.item_lo, item_end, prm.list_seg0, nreq,
                   s_item[cur ^ 1u], lane);
      const uint32_t nunits = nscan + (bcnt + kBucketUnit - 1) / kBucketUnit;
      const uint32_t o = lane & 7u, h = lane >> 3;
      for (;;) {
        uint32_t u = 0;
        if (lane == 0) u = atomicAdd(&s_ctr, 1u);
        u = __shfl_sync(0xFFFFFFFFu, u, 0);
        if (u >= nunits) break;
        if (u < nsmall) {
          const bool cst = u < kConstPrimes;
          const uint32_t p = cst ? cTab.p[u] : __ldg(prm.P + u);
          const uint32_t m = mod_barrett(k0, p, cst ? (uint64_t)cTab.m[u] : __ldg(prm.M + u));
          const uint32_t r = __ldg(prm.R + 8u * u + o);
          uint32_t s = r >= m ? r - m : r + p - m;
          if (30ull * k0 < (uint64_t)p * p) s = lift_to_square(s, k0, p, o, nbytes);
          // This lane's stream: bytes j0 + 4 p i = words w0 + p i with one
          // mask, n of them in the segment.  All 32 streams step p words, so
          // their banks shift alike: a lane that starts at the step rot
          // where its stream is in bank `lane` (w0 + p rot = lane mod 32)
          // stays on a bank of its own while every lane walks on, and each
          // atomic of the warp takes one shared-memory wavefront instead of
          // one per lane sharing a bank.  A lane walks steps rot .. n-1,
          // then wraps to 0 .. rot-1 (wrapped lanes may meet one other lane
          // on a bank).  With fewer than 32 steps the rotation is taken mod n.
          const uint32_t j0 = s + h * p;
          const uint32_t c = j0 & 3u;
          const uint32_t mask = ~(1u << ((c << 3) | o));
          const uint32_t lim = (nbytes - c + 3u) >> 2;      // word w holds byte 4w + c < nbytes
          const uint32_t w0 = j0 >> 2;
          const uint32_t n = w0 < lim ? (lim - w0 + p - 1u) / p : 0u;
          const uint32_t pinv = p * (2u - p * p);           // p^-1 mod 64 (p odd, p*p = 1 mod 8)
          uint32_t rot = ((lane - w0) * pinv) & 31u;
          if (rot >= n) rot = n ? rot % n : 0u;
          const uint32_t first = n - rot;                    // steps before the wrap
          const uint32_t k1 = __reduce_min_sync(0xFFFFFFFFu, first);
          const uint32_t kmax = __reduce_max_sync(0xFFFFFFFFu, n);
          uint32_t* q = seg + w0 + p * rot;
          uint32_t k = 0;
#pragma unroll 8
          for (; k < k1; ++k, q += p) atomicAnd(q, mask);
          for (; k < kmax; ++k, q += p) {
            if (k == first) q -= n * p;                      // wrap to step 0
            if (k < n) atomicAnd(q, mask);
          }
        } else if (u >= nscan) {
          // bucket list of this segment: primes >= the bucket split whose
          // hits were listed by bucket_fill_kernel; entries read coalesced
          const uint64_t base = bbase + (uint64_t)(u - nscan) * kBucketUnit;
          const uint32_t lim = min(kBucketUnit, bcnt - (u - nscan) * kBucketUnit);
#pragma unroll 8
          for (uint32_t e = lane; e < lim; e += 32) {
            // entry = bit index: word v / 32, and ~(1 << (v mod 32)) is
            // 0xFFFFFFFE rotated by v (a funnel shift takes its count mod 32)
            const uint32_t v = __ldg(prm.bucket + base + e);
            atomicAnd(seg + (v >> 5), __funnelshift_l(0xFFFFFFFEu, 0xFFFFFFFEu, v));
          }
        } else if (u >= nsmall + nmidu) {
          // huge tier: p >= S, at most one hit per class; 64-prime units, a
          // lane per prime in each of two halves whose table loads are all
          // issued first; the eight classes unrolled, clears predicated.
          const uint32_t ib = hbeg + 2u * kHugeHalf * (u - nsmall - nmidu) + lane;
          uint32_t pq[2], rq[2][8];
          uint64_t mq[2];
#pragma unroll
          for (uint32_t q = 0; q < 2; ++q) {
            // past the table end a lane repeats the last prime: its clears
            // are the same bits again
            const uint32_t i = min(ib + kHugeHalf * q, np - 1u);
            pq[q] = __ldg(prm.P + i);
            mq[q] = __ldg(prm.M + i);
            load_residues(prm.R, i, rq[q]);
          }
#pragma unroll
          for (uint32_t q = 0; q < 2; ++q) {
            const uint32_t p = pq[q];
            const uint32_t m = mod_barrett(k0, p, mq[q]);
            const uint64_t p2 = (uint64_t)p * p;
            const bool low = 30ull * k0 < p2;
            uint32_t sv[8];
#pragma unroll
            for (uint32_t t = 0; t < 8; ++t) sv[t] = rq[q][t] >= m ? rq[q][t] - m : rq[q][t] + p - m;
            // p >= the segment: sv[t] is the class's only candidate here, so
            // below p*p there is none (the next one is sv[t] + p).  The test
            // sits apart from the clears, under one branch taken by few
            // segments.
            if (low) {
#pragma unroll
              for (uint32_t t = 0; t < 8; ++t)
                if (30ull * (k0 + sv[t]) + w30(t) < p2) sv[t] = nbytes;
            }
#pragma unroll
            for (uint32_t t = 0; t < 8; ++t)
              if (sv[t] < nbytes) clear_bit(seg, sv[t], ~(1u << t));
          }
        } else {
          // mid tier: p and k0 mod p once per prime (lane = prime), then
          // shuffled to the (prime, class) lanes of each round.
          const uint32_t base = nsmall + 32u * (u - nsmall);
          const uint32_t im = base + lane;
          const bool okm = im < hbeg;
          const uint32_t pm = okm ? __ldg(prm.P + im) : 0u;
          const uint32_t mm = okm ? mod_barrett(k0, pm, __ldg(prm.M + im)) : 0u;
          const bool low_any = __any_sync(0xFFFFFFFFu, okm && 30ull * k0 < (uint64_t)pm * pm);
          const uint32_t keep = ~(1u << o);
          uint32_t rr[8];
#pragma unroll
          for (int t = 0; t < 8; ++t) {
            const uint32_t i = base + 4u * t + h;
            rr[t] = i < hbeg ? __ldg(prm.R + 8u * i + o) : 0u;
          }
#pragma unroll
          for (int t = 0; t < 8; ++t) {
            const uint32_t p = __shfl_sync(0xFFFFFFFFu, pm, 4 * t + h);
            const uint32_t m = __shfl_sync(0xFFFFFFFFu, mm, 4 * t + h);
            if (!p) continue;
            uint32_t s = rr[t] >= m ? rr[t] - m : rr[t] + p - m;
            if (low_any && 30ull * k0 < (uint64_t)p * p) s = lift_to_square(s, k0, p, o, nbytes);
#pragma unroll 8
            for (uint32_t j = s; j < nbytes; j += p) clear_bit(seg, j, keep);
          }
        }
      }
    }
    __syncthreads();
    if (tid == 0) s_ctr = 0;                        // every unit is taken: reset for the next segment

    // 3. reductions: each thread scans one contiguous run of words (odd
    //    length, so the lanes of a warp hit distinct banks); lanes are
    //    stitched with a warp max-scan of their last prime, warps by warp 0.
    {
      const uint32_t run = ((nwords + nthr - 1) / nthr) | 1u;
      const uint32_t wbeg = min(tid * run, nwords);
      const uint32_t wend = min(wbeg + run, nwords);
      // edge fix-ups, each by the thread whose run holds the word
      if (wbeg == 0 && wend > 0) seg[0] = ((seg[0] & S.and0) | S.or0) & S.keep0;
      if (wbeg < wend && wend == nwords) seg[nwords - 1u] &= S.keepl;
      if (prm.flags & kFlagBitmap) {
        __syncthreads();
        uint32_t* dst = prm.bitmap + ((k0 - prm.reqs[0].k_lo) >> 2);
        for (uint32_t w = tid; w < nwords; w += nthr) dst[w] = seg[w];
      }
      GapSink sk;
      sk.shist = shist + (warp % kSmemHistCopies) * kSmemStride;
      sk.acc = prm.acc + req;
      sk.large = prm.large; sk.n_large = prm.n_large; sk.cap = prm.large_cap;
      sk.req = req; sk.base = 30ull * k0;
      const uint32_t m41 = (k0 & 1ull) ? 0x99669966u : 0x66996699u;
      uint32_t first1 = 0, last1 = 0, cnt = 0, c41 = 0, c31 = 0, maxg = 0, maxgs = 0;
      const bool gaps = (S.rflags & kReqGaps) != 0;
      if (gaps) {
        // Byte by byte, four fixed steps per word, so the lanes of a warp
        // stay in step whatever their primes: the gaps inside a wheel byte
        // (2..28) come from the byte table and are summed in packed 8-bit
        // counters (accE: gap/2 - 1 even, accO: odd), flushed warp-reduced
        // into the shared histogram every kFlushWords words; the gap into a
        // byte from the previous prime goes to the histogram directly, and
        // to the rare path when it may be a new largest gap, a large gap or
        // beyond the shared bins.  The run's first prime arrives as a gap
        // from kNoPrev, which the rare path takes as "no gap, first prime".
        constexpr uint32_t kNoPrev = 0x80000000u;
        constexpr uint32_t kFlushWords = 15;      // 15 words * 4 bytes * 4 gaps of one size < 256
        uint64_t accE = 0, accO = 0;
        uint32_t pv = kNoPrev, thr = 0;
        const uint32_t nsteps = run;              // the same for every lane
        for (uint32_t i = 0; i < nsteps; ++i) {
          const uint32_t wi = wbeg + i;
          const uint32_t w = wi < wend ? seg[wi] : 0u;
          if (w) {
            cnt += __popc(w);
            c41 += __popc(w & m41);
            c31 += __popc(w & 0x2B2B2B2Bu);
            const uint32_t vb = 120u * wi;
#pragma unroll
            for (uint32_t b = 0; b < 4; ++b) {
              const uint32_t x = (w >> (8u * b)) & 0xFFu;
              if (x) {
                const uint4 t = btab[x];
                accE += ((uint64_t)t.y << 32) | t.x;
                accO += ((uint64_t)t.w << 32) | t.z;
                const uint32_t v = vb + 30u * b + (t.y >> 24);
                const uint32_t g = v - pv;
                if (g <= thr) {
                  atomicAdd(sk.shist + (g >> 1), 1u);
                } else if (g & kNoPrev) {
                  first1 = v + 1u;                  // the run's first prime
                } else {
                  const uint32_t bin = g >> 1;
                  if (bin < (uint32_t)kSmemBins) atomicAdd(sk.shist + bin, 1u);
                  else atomicAdd(&sk.acc->hist[bin < (uint32_t)kHistBins ? bin : kHistBins - 1], 1ull);
                  if (g > maxg) { maxg = g; maxgs = pv; }
                  if (g >= kLargeGap) {
                    const unsigned idx = atomicAdd(sk.n_large, 1u);
                    if (idx < sk.cap) {
                      LargeGapRec r; r.pos = sk.base + v; r.gap = g; r.req = sk.req;
                      sk.large[idx] = r;
                    }
                  }
                  thr = min(maxg, kLargeGap - 1u);
                }
                pv = vb + 30u * b + (t.w >> 24);
              }
            }
          }
          if ((i + 1u) % kFlushWords == 0u || i + 1u == nsteps) {
            // 16-bit pairs of the 8-bit counters, summed over the warp; lane
            // k < 7 adds pair k (bins 2k+1, 2k+3 from accE; k >= 4 accO)
            const uint32_t eL = (uint32_t)accE, eH = (uint32_t)(accE >> 32);
            const uint32_t oL = (uint32_t)accO, oH = (uint32_t)(accO >> 32);
            const uint32_t q0 = __reduce_add_sync(0xFFFFFFFFu, __byte_perm(eL, 0u, 0x5150));   // bins 1, 3
            const uint32_t q1 = __reduce_add_sync(0xFFFFFFFFu, __byte_perm(eL, 0u, 0x5352));   // bins 5, 7
            const uint32_t q2 = __reduce_add_sync(0xFFFFFFFFu, __byte_perm(eH, 0u, 0x5150));   // bins 9, 11
            const uint32_t q3 = __reduce_add_sync(0xFFFFFFFFu, __byte_perm(eH, 0u, 0x4442));   // bin 13
            const uint32_t q4 = __reduce_add_sync(0xFFFFFFFFu, __byte_perm(oL, 0u, 0x5150));   // bins 2, 4
            const uint32_t q5 = __reduce_add_sync(0xFFFFFFFFu, __byte_perm(oL, 0u, 0x5352));   // bins 6, 8
            const uint32_t q6 = __reduce_add_sync(0xFFFFFFFFu, __byte_perm(oH, 0u, 0x5150));   // bins 10, 12
            const uint32_t q7 = __reduce_add_sync(0xFFFFFFFFu, __byte_perm(oH, 0u, 0x4442));   // bin 14
            accE = 0;
            accO = 0;
            if (lane < 8u) {
              const uint32_t q = lane == 0 ? q0 : lane == 1 ? q1 : lane == 2 ? q2 : lane == 3 ? q3
                               : lane == 4 ? q4 : lane == 5 ? q5 : lane == 6 ? q6 : q7;
              // pair k of accE holds bins 4k'+1.. : lane 0 -> 1,3; 1 -> 5,7; 2 -> 9,11; 3 -> 13
              // accO: lane 4 -> 2,4; 5 -> 6,8; 6 -> 10,12; 7 -> 14
              const uint32_t b0 = lane < 4u ? 4u * lane + 1u : 4u * (lane - 4u) + 2u;
              if (q & 0xFFFFu) atomicAdd(sk.shist + b0, q & 0xFFFFu);
              if (q >> 16) atomicAdd(sk.shist + b0 + 2u, q >> 16);
            }
          }
        }
        // A largest gap inside a byte (at most 28) is not tracked above:
        // where no gap between bytes exceeds 28, the run is walked prime by
        // prime for its exact largest gap (the earliest one on ties).
        if (first1 && maxg <= 28u) {
          maxg = 0; maxgs = 0;
          uint32_t q = first1 - 1u;
          for (uint32_t wi = wbeg; wi < wend; ++wi) {
            uint32_t w = seg[wi];
            const uint32_t vb = 120u * wi;
            while (w) {
              const uint32_t v = vb + s_vtab[__ffs(w) - 1];
              w &= w - 1u;
              if (v - q > maxg) { maxg = v - q; maxgs = q; }
              q = v;
            }
          }
        }
        last1 = first1 ? pv + 1u : 0u;
      } else {
        for (uint32_t wi = wbeg; wi < wend; ++wi) {
          const uint32_t w = seg[wi];
          if (!w) continue;
          cnt += __popc(w);
          c41 += __popc(w & m41);
          c31 += __popc(w & 0x2B2B2B2Bu);
          const uint32_t vb = 120u * wi;
          if (!first1) first1 = vb + s_vtab[__ffs(w) - 1] + 1u;
          last1 = vb + s_vtab[31 - __clz(w)] + 1u;
        }
      }
      // lane stitching: previous lane's last prime (values grow with the lane)
      uint32_t sc = last1;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, sc, d);
        if ((int)lane >= d) sc = max(sc, t);
      }
      uint32_t prev1 = __shfl_up_sync(0xFFFFFFFFu, sc, 1);
      if (lane == 0) prev1 = 0;
      if (gaps && first1 && prev1) record_gap(sk, prev1 - 1u, first1 - 1u, maxg, maxgs);
      const uint32_t wlast = __shfl_sync(0xFFFFFFFFu, sc, 31);
      const uint32_t wfirst = __reduce_min_sync(0xFFFFFFFFu, first1 ? first1 : 0xFFFFFFFFu);
      cnt = __reduce_add_sync(0xFFFFFFFFu, cnt);
      c41 = __reduce_add_sync(0xFFFFFFFFu, c41);
      c31 = __reduce_add_sync(0xFFFFFFFFu, c31);
      const uint32_t gm = __reduce_max_sync(0xFFFFFFFFu, maxg);
      const uint32_t gs = __reduce_min_sync(0xFFFFFFFFu, (maxg == gm && gm) ? maxgs : 0xFFFFFFFFu);
      if (lane == 0) {
        WarpRec r;
        r.first1 = wfirst == 0xFFFFFFFFu ? 0u : wfirst;
        r.last1 = wlast; r.cnt = cnt; r.c41 = c41; r.c31 = c31;
        r.maxg = gm; r.maxgs = gs; r.pad = 0;
        wrec[warp] = r;
      }
      __syncthreads();
      // warps are stitched like lanes, lane = warp: the gap from the last
      // prime before a warp to its first prime, the largest gap (ties: the
      // first), the sums
      if (warp == 0) {
        WarpRec r = {0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u};
        if (lane < nwarps) r = wrec[lane];
        uint32_t sw = r.last1;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
          const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, sw, d);
          if ((int)lane >= d) sw = max(sw, t);
        }
        uint32_t before = __shfl_up_sync(0xFFFFFFFFu, sw, 1);
        if (lane == 0) before = 0;
        uint32_t bg = 0, bs = 0;
        if (gaps && r.first1 && before) record_gap(sk, before - 1u, r.first1 - 1u, bg, bs);
        if (r.maxg > bg) { bg = r.maxg; bs = r.maxgs; }   // on a tie the joining gap starts first
        const uint32_t gm = __reduce_max_sync(0xFFFFFFFFu, bg);
        const uint32_t gs = __reduce_min_sync(0xFFFFFFFFu, (bg == gm && gm) ? bs : 0xFFFFFFFFu);
        const uint32_t fst1 = __reduce_min_sync(0xFFFFFFFFu, r.first1 ? r.first1 : 0xFFFFFFFFu);
        const uint32_t run1 = __shfl_sync(0xFFFFFFFFu, sw, 31);
        const uint32_t tc = __reduce_add_sync(0xFFFFFFFFu, r.cnt);
        const uint32_t t41 = __reduce_add_sync(0xFFFFFFFFu, r.c41);
        const uint32_t t31 = __reduce_add_sync(0xFFFFFFFFu, r.c31);
        if (lane == 0) {
          SegRec sr;
          sr.first = fst1 != 0xFFFFFFFFu ? sk.base + fst1 - 1u : 0;
          sr.last = run1 ? sk.base + run1 - 1u : 0;
          sr.max_gap = gm;
          sr.max_gap_start = gm ? sk.base + gs : 0;
          sr.count = tc;
          prm.segs[item] = sr;
          if (tc) {
            atomicAdd(&sk.acc->count, (unsigned long long)tc);
            atomicAdd(&sk.acc->c41, (unsigned long long)t41);
            atomicAdd(&sk.acc->c31, (unsigned long long)t31);
          }
        }
      }
    }
  }
  __syncthreads();
  if (cur_req >= 0) {
    for (uint32_t bn = tid; bn < (uint32_t)kSmemBins; bn += nthr) {
      uint32_t s = 0;
#pragma unroll
      for (int c = 0; c < kSmemHistCopies; ++c) s += shist[c * kSmemStride + bn];
      if (s) atomicAdd(&prm.acc[cur_req].hist[bn], (unsigned long long)s);
    }
  }
}

// One CTA per request: seeds 2, 3, 5, gaps across segment boundaries, the
// largest gap, and the final counts (the reference's host-side conventions,
// context.cu:321-322,462-524, restated for a half-open [a, b)).
__global__ void __launch_bounds__(256)
finalize_kernel(const ReqDesc* __restrict__ reqs, const BatchHdr* __restrict__ hdr,
                const SegRec* __restrict__ segs, ReqAccum* __restrict__ acc, LargeGapRec* large,
                unsigned int* n_large, uint32_t large_cap, ReqResult* __restrict__ out) {
  const uint32_t r = blockIdx.x, tid = threadIdx.x;
  if (r >= hdr->nreq) return;       // fixed-size launches (graph replay) cover capacity
  const ReqDesc R = reqs[r];
  ReqAccum* A = acc + r;
  const SegRec* S = segs + R.seg_base;
  __shared__ uint64_t s_bg[256], s_bs[256];

  const bool in2 = R.a <= 2 && 2 < R.b, in3 = R.a <= 3 && 3 < R.b, in5 = R.a <= 5 && 5 < R.b;
  const uint64_t seed_first = in2 ? 2 : in3 ? 3 : in5 ? 5 : 0;
  const uint64_t seed_last = in5 ? 5 : in3 ? 3 : in2 ? 2 : 0;

  uint64_t bg = 0, bs = 0;
  auto consider = [&](uint64_t g, uint64_t st) {
    if (g > bg || (g == bg && g && st < bs)) { bg = g; bs = st; }
  };
  if (tid == 0 && (R.rflags & kReqGaps)) {
    if (in2 && in3) { atomicAdd(&A->hist[0], 1ull); consider(1, 2); }
    if (in3 && in5) { atomicAdd(&A->hist[1], 1ull); consider(2, 3); }
  }
  const bool want_gaps = (R.rflags & kReqGaps) != 0;
  for (uint64_t i = want_gaps ? tid : R.nseg; i < R.nseg; i += blockDim.x) {
    const SegRec s = S[i];
    if (s.max_gap) consider(s.max_gap, s.max_gap_start);
    if (!s.first) continue;
    uint64_t prev = 0;
    for (uint64_t j = i; j-- > 0;) {
      if (S[j].first) { prev = S[j].last; break; }
    }
    if (!prev) prev = seed_last;
    if (!prev) continue;
    const uint64_t g = s.first - prev;
    const uint64_t bin = g >> 1;
    atomicAdd(&A->hist[bin < (uint64_t)kHistBins ? bin : kHistBins - 1], 1ull);
    consider(g, prev);
    if (g >= kLargeGap) {
      const unsigned idx = atomicAdd(n_large, 1u);
      if (idx < large_cap) {
        LargeGapRec lr; lr.pos = s.first; lr.gap = (uint32_t)g; lr.req = r;
        large[idx] = lr;
      }
    }
  }
  s_bg[tid] = bg; s_bs[tid] = bs;
  __syncthreads();
  for (uint32_t w = blockDim.x / 2; w > 0; w >>= 1) {
    if (tid < w) {
      const uint64_t g2 = s_bg[tid + w], t2 = s_bs[tid + w];
      if (g2 > s_bg[tid] || (g2 == s_bg[tid] && g2 && t2 < s_bs[tid])) { s_bg[tid] = g2; s_bs[tid] = t2; }
    }
    __syncthreads();
  }
  ReqResult* O = out + r;
  for (uint32_t b = tid; b < (uint32_t)kHistBins; b += blockDim.x) O->hist[b] = A->hist[b];
  if (tid == 0) {
    const uint64_t ns = (uint64_t)in2 + in3 + in5;
    const uint64_t wc = A->count;
    O->count = wc + ns;
    O->c41 = A->c41 + (in5 ? 1 : 0);
    O->c43 = (wc - A->c41) + (in3 ? 1 : 0);
    O->c31 = A->c31;
    O->c32 = (wc - A->c31) + (in2 ? 1 : 0) + (in5 ? 1 : 0);
    uint64_t f = seed_first, l = seed_last;
    if (!f) {
      for (uint64_t i = 0; i < R.nseg; ++i) if (S[i].first) { f = S[i].first; break; }
    }
    for (uint64_t i = R.nseg; i-- > 0;) if (S[i].last) { l = S[i].last; break; }
    O->first = f;
    O->last = l;
    O->max_gap = s_bg[0];
    O->max_gap_start = s_bg[0] ? s_bs[0] : 0;
    O->num_gaps = O->count ? O->count - 1 : 0;
  }
}

// Bucket fill: one CTA per work item (a request, a run of its bucket primes
// and a run of its segments; heavy runs of small primes are split over
// several items so that items carry similar numbers of hits), a thread per
// prime walking its eight classes.  Pass 1 counts the hits per segment in
// shared memory; one global atomic per segment reserves room in that
// segment's list and leaves the reserved base in the shared counter; pass 2
// walks the hits again and writes each entry at the counter's next slot.  A
// hit's segment and offset advance by p = pq*S + pr without a division.  A
// list that would overflow its capacity raises *overflow and drops the entry
// (the host then reruns without lists).
//
// The walk takes the eight classes together, eight independent chains of
// atomic-then-store per thread: all step unconditionally while all have hits
// left (each chain's count of hits is known up front), then each finishes
// under its own predicate.  (Lanes of a warp hold primes of nearly the same size
// and walk in step, so many of them meet on one segment counter at a time;
// the counter then hands them consecutive slots and their entries leave in
// shared sectors.  Spreading the lanes over segments removes the atomic
// conflicts but scatters the stores, and measured slower.)
struct FillChain {
  uint32_t sg, off, n;       // segment (relative to the item's first), offset, hits left
};

template <bool kWrite>
__device__ __forceinline__ void fill_step(FillChain& c, uint32_t o, uint32_t* cnt, uint32_t* list,
                                          uint32_t cap, unsigned int* overflow, uint32_t S,
                                          uint32_t pq, uint32_t pr) {
  if (kWrite) {
    const uint32_t pos = atomicAdd(&cnt[c.sg], 1u);
    if (pos < cap) list[c.sg * cap + pos] = bucket_entry(c.off, o);
    else atomicOr(overflow, 1u);
  } else {
    atomicAdd(&cnt[c.sg], 1u);
  }
  c.off += pr;
  const uint32_t carry = c.off >= S ? 1u : 0u;
  c.off -= carry ? S : 0u;
  c.sg += pq + carry;
}

template <bool kWrite>
__device__ __forceinline__ void fill_pass(const FillChain (&start)[8], uint32_t* cnt, uint32_t* list,
                                          uint32_t cap, unsigned int* overflow, uint32_t S,
                                          uint32_t pq, uint32_t pr) {
  FillChain c[8];
  uint32_t all = start[0].n, most = start[0].n;
#pragma unroll
  for (int o = 0; o < 8; ++o) { c[o] = start[o]; all = min(all, c[o].n); most = max(most, c[o].n); }
  for (uint32_t t = 0; t < all; ++t) {
#pragma unroll
    for (uint32_t o = 0; o < 8; ++o) fill_step<kWrite>(c[o], o, cnt, list, cap, overflow, S, pq, pr);
  }
  for (uint32_t t = all; t < most; ++t) {
#pragma unroll
    for (uint32_t o = 0; o < 8; ++o)
      if (t < c[o].n) fill_step<kWrite>(c[o], o, cnt, list, cap, overflow, S, pq, pr);
  }
}

__global__ void __launch_bounds__(kFillPrimes)
bucket_fill_kernel(const FillParams fp) {
  __shared__ uint32_t cnt[kMaxBucketSegs];
  const uint32_t tid = threadIdx.x;
  const uint32_t nitems = fp.nitems ? fp.nitems : fp.hdr->nfill;
  for (uint32_t it = blockIdx.x; it < nitems; it += gridDim.x) {
    const FillItem item = fp.items[it];
    const ReqDesc R = fp.reqs[item.req];
    // segments g0..g1 of the window that starts at segment seg0 of the
    // request; byte offsets below are relative to the window's start k0
    const uint32_t g0 = item.segs & 0xFFFFu, g1 = item.segs >> 16;
    const uint32_t nseg = g1 - g0;
    const uint32_t S = R.seg_bytes;
    const uint64_t k0 = R.k_lo + (uint64_t)fp.seg0 * S;
    const uint32_t total = (uint32_t)min(R.k_hi - k0, (uint64_t)kMaxBucketSegs * S);
    const uint32_t lo = g0 * S;
    const uint32_t hi = min(total, g1 * S);
    const uint32_t cap = R.bucket_cap;
    // the item's lists, segment g at g * cap (the host keeps a window's
    // entries below 2^32)
    uint32_t* const list = fp.bucket + R.bucket_base + (uint64_t)g0 * cap;
    unsigned int* const gcount = fp.bcount + R.seg_base + fp.seg0 + g0;
    const float inv_s = 1.0f / (float)S;
    // q = x / S, r = x % S for x < 2^30: a float estimate, corrected once
    auto divmod_s = [&](uint32_t x, uint32_t& r) {
      uint32_t q = __float2uint_rz((float)x * inv_s);
      int32_t d = (int32_t)(x - q * S);
      if (d < 0) { --q; d += (int32_t)S; } else if (d >= (int32_t)S) { ++q; d -= (int32_t)S; }
      r = (uint32_t)d;
      return q;
    };
    for (uint32_t g = tid; g < nseg; g += blockDim.x) cnt[g] = 0;
    __syncthreads();
    const uint32_t i = item.p0 + tid;
    const bool valid = i < item.p1;
    uint32_t p = 0, m = 0, pq = 0, pr = 0;
    bool low = false;
    if (valid) {
      p = __ldg(fp.P + i);
      m = mod_barrett(k0, p, __ldg(fp.M + i));
      low = 30ull * k0 < (uint64_t)p * p;
      pq = divmod_s(p, pr);
    }
    // first hit at or after byte lo of each class and the number of hits
    // below hi, kept for both passes; the eight residue loads issue together
    uint32_t r8[8];
    if (valid) load_residues(fp.R, i, r8);
    FillChain ch[8];
#pragma unroll
    for (int o = 0; o < 8; ++o) {
      ch[o].sg = 0; ch[o].off = 0; ch[o].n = 0;
      if (valid) {
        const uint32_t r = r8[o];
        uint32_t k = r >= m ? r - m : r + p - m;
        if (low) k = lift_to_square(k, k0, p, o, total);
        if (k < lo) k += ((lo - k + p - 1) / p) * p;
        if (k < hi) {
          ch[o].n = (hi - 1u - k) / p + 1u;
          ch[o].sg = divmod_s(k, ch[o].off) - g0;
        }
      }
    }
    fill_pass<false>(ch, cnt, list, cap, fp.overflow, S, pq, pr);
    __syncthreads();
    for (uint32_t g = tid; g < nseg; g += blockDim.x) {
      const uint32_t c = cnt[g];
      cnt[g] = c ? atomicAdd(gcount + g, c) : 0u;
    }
    __syncthreads();
    fill_pass<true>(ch, cnt, list, cap, fp.overflow, S, pq, pr);
    __syncthreads();
  }
}

// Rebuild caller requests from shared atoms (disjoint pieces of the batch's
// ranges, each sieved once).  A request is the ordered run of its atoms:
// counts add; its gaps are the atoms' inner gaps plus one junction gap
// between each atom holding primes and the next such atom; the maximal gap
// is the largest of those, the earliest on ties, as within one range.  Each
// thread folds a contiguous run of atoms, thread 0 joins the runs in order.
// A request that asked for counts only gets no gap outputs even where its
// atoms were scanned for another request's gaps, so its result is the one
// it gets alone.
__global__ void __launch_bounds__(256)
combine_kernel(const BatchHdr* __restrict__ hdr, const ReqSpan* __restrict__ spans,
               const uint32_t* __restrict__ apos, const ReqResult* __restrict__ ares,
               ReqResult* __restrict__ out) {
  const uint32_t r = blockIdx.x, tid = threadIdx.x;
  if (r >= hdr->nout) return;
  const ReqSpan sp = spans[r];
  const bool gaps = (sp.rflags & kReqGaps) != 0;
  __shared__ uint32_t jh[kHistBins];
  __shared__ uint64_t t_first[256], t_last[256], t_bg[256], t_bs[256];
  __shared__ uint64_t t_sum[5][256];
  for (uint32_t b = tid; b < (uint32_t)kHistBins; b += blockDim.x) jh[b] = 0;
  __syncthreads();

  auto add_gap = [&](uint64_t g, uint64_t st, uint64_t& bg, uint64_t& bs) {
    const uint64_t bin = g >> 1;
    atomicAdd(&jh[bin < (uint64_t)kHistBins ? bin : kHistBins - 1], 1u);
    if (g > bg || (g == bg && st < bs)) { bg = g; bs = st; }
  };
  const uint32_t n = sp.e - sp.s;
  const uint32_t per = (n + blockDim.x - 1) / blockDim.x;
  const uint32_t j0 = sp.s + min(n, tid * per), j1 = sp.s + min(n, (tid + 1) * per);
  uint64_t c[5] = {0, 0, 0, 0, 0};
  uint64_t first = 0, last = 0, bg = 0, bs = 0;
  for (uint32_t j = j0; j < j1; ++j) {
    const ReqResult* A = ares + apos[j];
    const uint64_t ac = A->count;
    c[0] += ac; c[1] += A->c41; c[2] += A->c43; c[3] += A->c31; c[4] += A->c32;
    if (!ac) continue;
    if (!first) first = A->first;
    if (gaps) {
      if (last) add_gap(A->first - last, last, bg, bs);
      const uint64_t mg = A->max_gap;
      if (mg && (mg > bg || (mg == bg && A->max_gap_start < bs))) { bg = mg; bs = A->max_gap_start; }
    }
    last = A->last;
  }
  t_first[tid] = first; t_last[tid] = last; t_bg[tid] = bg; t_bs[tid] = bs;
#pragma unroll
  for (int q = 0; q < 5; ++q) t_sum[q][tid] = c[q];
  __syncthreads();
  ReqResult* O = out + r;
  if (tid == 0) {
    uint64_t s5[5] = {0, 0, 0, 0, 0};
    uint64_t f = 0, l = 0, g = 0, gs = 0;
    for (uint32_t t = 0; t < blockDim.x; ++t) {
#pragma unroll
      for (int q = 0; q < 5; ++q) s5[q] += t_sum[q][t];
      if (!t_first[t]) continue;
      if (!f) f = t_first[t];
      if (gaps) {
        if (l) add_gap(t_first[t] - l, l, g, gs);
        if (t_bg[t] && (t_bg[t] > g || (t_bg[t] == g && t_bs[t] < gs))) { g = t_bg[t]; gs = t_bs[t]; }
      }
      l = t_last[t];
    }
    O->count = s5[0]; O->c41 = s5[1]; O->c43 = s5[2]; O->c31 = s5[3]; O->c32 = s5[4];
    O->first = f;
    O->last = l;
    O->max_gap = g;
    O->max_gap_start = g ? gs : 0;
    O->num_gaps = s5[0] ? s5[0] - 1 : 0;
  }
  __syncthreads();
  for (uint32_t b = tid; b < (uint32_t)kHistBins; b += blockDim.x) {
    uint64_t h = 0;
    if (gaps) {
      h = jh[b];
      for (uint32_t j = sp.s; j < sp.e; ++j) h += ares[apos[j]].hist[b];
    }
    O->hist[b] = h;
  }
}

// Zero up to three regions in one launch (a plan's accumulators, control
// words and bucket counts, before each run).
__global__ void zero_kernel(ZeroSpan z0, ZeroSpan z1, ZeroSpan z2) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t t0 = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const uint4 zero = make_uint4(0u, 0u, 0u, 0u);
  for (uint64_t i = t0; i < z0.n16; i += stride) static_cast<uint4*>(z0.p)[i] = zero;
  for (uint64_t i = t0; i < z1.n16; i += stride) static_cast<uint4*>(z1.p)[i] = zero;
  for (uint64_t i = t0; i < z2.n16; i += stride) static_cast<uint4*>(z2.p)[i] = zero;
}

// ---------------------------------------------------------------------------
// host-side launchers (called by the engine)
// ---------------------------------------------------------------------------
size_t sieve_smem_bytes(uint32_t seg_bytes, uint32_t /*threads*/) {
  // segment, histogram copies, warp records (room for 32 warps), byte table
  return (size_t)seg_bytes + sizeof(uint32_t) * kSmemHistCopies * kSmemStride +
         sizeof(WarpRec) * (kMaxThreads / 32) + sizeof(uint4) * kByteTabEntries;
}

size_t sieve_static_smem_bytes() {
  cudaFuncAttributes a{};
  return cudaFuncGetAttributes(&a, sieve_segments_kernel) == cudaSuccess ? a.sharedSizeBytes : 1024;
}

cudaError_t launch_sieve(const SieveParams& prm, uint32_t grid, uint32_t threads,
                         cudaStream_t stream) {
  const size_t smem = sieve_smem_bytes(prm.seg_bytes, threads);
  // the attribute is per device: raised once per (device, size), outside
  // stream capture (plans raise it before they capture)
  static AttrCache attr;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const int rc = attr.ensure(dev, smem, [](size_t n) {
    return (int)cudaFuncSetAttribute(sieve_segments_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)n);
  });
  if (rc) return (cudaError_t)rc;
  if (grid == 0) return cudaSuccess;
  sieve_segments_kernel<<<grid, threads, smem, stream>>>(prm);
  return cudaGetLastError();
}

cudaError_t launch_combine(const BatchHdr* hdr, const ReqSpan* spans, const uint32_t* apos,
                           const ReqResult* ares, ReqResult* out, uint32_t grid, cudaStream_t stream) {
  if (grid == 0) return cudaSuccess;
  combine_kernel<<<grid, 256, 0, stream>>>(hdr, spans, apos, ares, out);
  return cudaGetLastError();
}

cudaError_t launch_zero(ZeroSpan z0, ZeroSpan z1, ZeroSpan z2, uint32_t max_grid, cudaStream_t stream) {
  const uint64_t n = std::max(z0.n16, std::max(z1.n16, z2.n16));
  if (n == 0) return cudaSuccess;
  const uint32_t grid = (uint32_t)std::min<uint64_t>((n + 255) / 256, max_grid);
  zero_kernel<<<grid, 256, 0, stream>>>(z0, z1, z2);
  return cudaGetLastError();
}

uint32_t bucket_fill_ctas_per_sm() {
  static int n = 0;
  if (!n && (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, bucket_fill_kernel, kFillPrimes, 0) != cudaSuccess || n < 1))
    n = 1;
  return (uint32_t)n;
}

cudaError_t launch_bucket_fill(const FillParams& fp, uint32_t grid, cudaStream_t stream) {
  if (grid == 0) return cudaSuccess;
  bucket_fill_kernel<<<grid, kFillPrimes, 0, stream>>>(fp);
  return cudaGetLastError();
}

cudaError_t launch_finalize(const ReqDesc* reqs, const BatchHdr* hdr, const SegRec* segs,
                            ReqAccum* acc, LargeGapRec* large, unsigned int* n_large,
                            uint32_t large_cap, ReqResult* out, uint32_t grid,
                            cudaStream_t stream) {
  if (grid == 0) return cudaSuccess;
  finalize_kernel<<<grid, 256, 0, stream>>>(reqs, hdr, segs, acc, large, n_large, large_cap, out);
  return cudaGetLastError();
}

}  // namespace vg
