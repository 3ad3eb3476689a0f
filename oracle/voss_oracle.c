/*
 * voss_oracle.c -- CPU restatement of voss's wheel-30 sieve and the
 * statistics it feeds.  TEST INFRASTRUCTURE ONLY: the parity tests, the
 * smoke check and bench.py's CPU-baseline leg call this as the checker.
 * The shipped library never links or calls it.
 *
 * What it restates (reference file:line, paths inside the voss project):
 *   - bit layout: byte k, bit o  <->  30*k + W30[o], W30 = {1,7,11,13,17,19,
 *     23,29}                                         src/voss_w30_v7.cu:38-39
 *   - base primes by a plain Eratosthenes sieve, primes >= 7
 *                                             library/src/primes/context.cu:107-121
 *   - start of each (prime, residue class) stream: k0 = (-r mod p)*inv30 mod p,
 *     advanced by 30p to max(p^2, segment low)     context.cu:123-138,354-388
 *   - gap = difference of consecutive primes, counted per gap value;
 *     boundary gaps between segments stitched in order, 2,3,5 seeded by hand
 *                                                  context.cu:321-322,462-524
 *   - Chebyshev class of p by p mod 4                 chebyshev.cu:11-25
 *   - Goldbach: for even n, primes ascending, first p with n-p prime
 *                                                  goldbach_upto.cu:25-46
 *   - primes in [a,b] inclusive, sorted                  range.cu:99-262
 *
 * The range statistics here are over the half-open interval [a, b) of
 * integers: every prime q with a <= q < b, and every gap between two
 * consecutive primes that both lie in [a, b).  2, 3 and 5 are outside the
 * wheel and are added explicitly, as the reference does.
 *
 * Pinned by tests/test_oracle_golden.py against vectors produced by the
 * reference's own sympy oracle (library/tests/reference.py) and against the
 * known answers in the reference's tests.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "voss_oracle.h"

static const uint32_t W30[8] = {1, 7, 11, 13, 17, 19, 23, 29};

/* Plain Eratosthenes on a byte array: primes >= 7 and <= limit. */
static uint32_t* base_primes(uint64_t limit, uint64_t* count) {
    *count = 0;
    if (limit < 7) return NULL;
    uint8_t* comp = (uint8_t*)calloc(limit + 1, 1);
    if (!comp) return NULL;
    for (uint64_t i = 2; i * i <= limit; i++)
        if (!comp[i])
            for (uint64_t j = i * i; j <= limit; j += i) comp[j] = 1;
    uint64_t n = 0;
    for (uint64_t i = 7; i <= limit; i++) n += !comp[i];
    uint32_t* out = (uint32_t*)malloc((n ? n : 1) * sizeof(uint32_t));
    uint64_t c = 0;
    for (uint64_t i = 7; i <= limit; i++)
        if (!comp[i]) out[c++] = (uint32_t)i;
    free(comp);
    *count = n;
    return out;
}

static uint64_t isqrt_u64(uint64_t x) {
    uint64_t r = 0;
    uint64_t lo = 0, hi = 1ull << 32;
    while (lo < hi) {
        uint64_t mid = lo + (hi - lo + 1) / 2;
        if (mid <= x / mid) lo = mid; else hi = mid - 1;
    }
    r = lo;
    return r;
}

static int64_t inverse_mod(int64_t a, int64_t m) {
    int64_t t = 0, nt = 1, r = m, nr = a % m;
    while (nr) {
        int64_t q = r / nr, tmp;
        tmp = nt; nt = t - q * nt; t = tmp;
        tmp = nr; nr = r - q * nr; r = tmp;
    }
    return t < 0 ? t + m : t;
}

/* Sieve the bytes [k_lo, k_lo + nbytes) of the wheel.  After the call, bit o
 * of byte i is set iff 30*(k_lo+i) + W30[o] is prime (1 is cleared).  */
static void sieve_bytes(uint8_t* seg, uint64_t k_lo, uint64_t nbytes,
                        const uint32_t* bp, uint64_t nbp) {
    memset(seg, 0xFF, nbytes);
    uint64_t low = 30 * k_lo;                    /* smallest number covered */
    uint64_t high = 30 * (k_lo + nbytes) - 1;    /* largest number covered  */
    for (uint64_t i = 0; i < nbp; i++) {
        uint64_t p = bp[i];
        uint64_t p2 = p * p;
        if (p2 > high) break;
        int64_t inv30 = inverse_mod(30 % (int64_t)p, (int64_t)p);
        uint64_t lb = p2 > low ? p2 : low;
        for (int o = 0; o < 8; o++) {
            uint64_t r = W30[o];
            uint64_t k0 = (uint64_t)(((int64_t)((p - r % p) % p) * inv30) % (int64_t)p);
            uint64_t n = 30 * k0 + r;              /* first n = r mod 30, p | n */
            if (n < lb) {
                uint64_t step = 30 * p;
                n += ((lb - n + step - 1) / step) * step;
            }
            if (n > high) continue;
            uint64_t j = (n - r) / 30 - k_lo;
            uint8_t m = (uint8_t)~(1u << o);
            for (; j < nbytes; j += p) seg[j] &= m;
        }
    }
    if (k_lo == 0) seg[0] &= 0xFE;               /* 1 is not prime */
}

static inline uint64_t bitval(uint64_t k, int o) { return 30 * k + W30[o]; }

/* Per-chunk partial result (chunks processed in parallel, merged in order). */
typedef struct {
    uint64_t count, c41, c31, first, last, max_gap, max_gap_start;
    uint64_t hist[ORACLE_HBINS];
    uint64_t nlarge;
    uint64_t* large_pos;   /* second prime of each gap >= large threshold */
    uint32_t* large_gap;
    uint64_t large_cap;
} chunk_t;

static void record_gap(chunk_t* c, uint64_t prev, uint64_t cur, uint64_t thr) {
    uint64_t g = cur - prev;
    uint64_t bin = g >> 1;
    c->hist[bin < ORACLE_HBINS - 1 ? bin : ORACLE_HBINS - 1]++;
    if (g > c->max_gap || (g == c->max_gap && prev < c->max_gap_start)) {
        c->max_gap = g;
        c->max_gap_start = prev;
    }
    if (thr && g >= thr) {
        if (c->nlarge == c->large_cap) {
            c->large_cap = c->large_cap ? 2 * c->large_cap : 16;
            c->large_pos = (uint64_t*)realloc(c->large_pos, c->large_cap * 8);
            c->large_gap = (uint32_t*)realloc(c->large_gap, c->large_cap * 4);
        }
        c->large_pos[c->nlarge] = cur;
        c->large_gap[c->nlarge] = (uint32_t)g;
        c->nlarge++;
    }
}

#define CHUNK_BYTES 65536u

int oracle_range_stats(uint64_t a, uint64_t b, int nthreads,
                       uint64_t large_threshold, oracle_stats_t* out,
                       uint64_t* large_pos, uint32_t* large_gap,
                       uint64_t large_cap) {
    if (!out) return 1;
    memset(out, 0, sizeof(*out));
    out->a = a; out->b = b;
    if (b <= a) return 0;

    /* Wheel part: numbers >= 7 that are coprime to 30.  */
    uint64_t k_lo = a / 30;
    uint64_t k_hi = (b + 29) / 30;
    uint64_t nbp = 0;
    uint32_t* bp = base_primes(b > 1 ? isqrt_u64(b - 1) : 0, &nbp);
    uint64_t nchunks = (k_hi - k_lo + CHUNK_BYTES - 1) / CHUNK_BYTES;
    chunk_t* ch = (chunk_t*)calloc(nchunks ? nchunks : 1, sizeof(chunk_t));
    if (!ch) { free(bp); return 2; }

#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel
#endif
    {
        uint8_t* seg = (uint8_t*)malloc(CHUNK_BYTES);
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
        for (int64_t ci = 0; ci < (int64_t)nchunks; ci++) {
            chunk_t* c = &ch[ci];
            uint64_t k0 = k_lo + (uint64_t)ci * CHUNK_BYTES;
            uint64_t nb = k_hi - k0 < CHUNK_BYTES ? k_hi - k0 : CHUNK_BYTES;
            sieve_bytes(seg, k0, nb, bp, nbp);
            uint64_t have = 0, prev = 0;
            for (uint64_t i = 0; i < nb; i++) {
                uint8_t v = seg[i];
                if (!v) continue;
                uint64_t k = k0 + i;
                for (int o = 0; o < 8; o++) {
                    if (!((v >> o) & 1)) continue;
                    uint64_t q = bitval(k, o);
                    if (q < a || q >= b || q < 7) continue;
                    c->count++;
                    if ((q & 3) == 1) c->c41++;
                    if (q % 3 == 1) c->c31++;
                    if (have) record_gap(c, prev, q, large_threshold);
                    else { c->first = q; have = 1; }
                    prev = q;
                }
            }
            c->last = have ? prev : 0;
        }
        free(seg);
    }

    /* Seeds 2, 3, 5 in order, then the chunks in order (stitching). */
    chunk_t acc;
    memset(&acc, 0, sizeof(acc));
    uint64_t have = 0, last = 0;
    static const uint64_t seeds[3] = {2, 3, 5};
    for (int s = 0; s < 3; s++) {
        uint64_t q = seeds[s];
        if (q < a || q >= b) continue;
        acc.count++;
        if ((q & 3) == 1) acc.c41++;
        if (q % 3 == 1) acc.c31++;
        if (have) record_gap(&acc, last, q, large_threshold);
        else { acc.first = q; have = 1; }
        last = q;
    }
    uint64_t c43 = 0, c32 = 0;
    /* mod-4 / mod-3 complements for the seeds: 3 is 3 mod 4; 2, 5 are 2 mod 3 */
    if (a <= 3 && 3 < b) c43++;
    if (a <= 2 && 2 < b) c32++;
    if (a <= 5 && 5 < b) c32++;
    for (uint64_t ci = 0; ci < nchunks; ci++) {
        chunk_t* c = &ch[ci];
        if (c->count) {
            if (have) record_gap(&acc, last, c->first, large_threshold);
            else { acc.first = c->first; have = 1; }
            last = c->last;
            acc.count += c->count;
            acc.c41 += c->c41;
            acc.c31 += c->c31;
            c43 += c->count - c->c41;    /* wheel primes are odd: 1 or 3 mod 4 */
            c32 += c->count - c->c31;    /* and never 0 mod 3 */
            for (int h = 0; h < ORACLE_HBINS; h++) acc.hist[h] += c->hist[h];
            if (c->max_gap > acc.max_gap ||
                (c->max_gap == acc.max_gap && c->max_gap && c->max_gap_start < acc.max_gap_start)) {
                acc.max_gap = c->max_gap;
                acc.max_gap_start = c->max_gap_start;
            }
            for (uint64_t j = 0; j < c->nlarge; j++) {
                if (acc.nlarge == acc.large_cap) {
                    acc.large_cap = acc.large_cap ? 2 * acc.large_cap : 16;
                    acc.large_pos = (uint64_t*)realloc(acc.large_pos, acc.large_cap * 8);
                    acc.large_gap = (uint32_t*)realloc(acc.large_gap, acc.large_cap * 4);
                }
                acc.large_pos[acc.nlarge] = c->large_pos[j];
                acc.large_gap[acc.nlarge] = c->large_gap[j];
                acc.nlarge++;
            }
        }
        free(c->large_pos);
        free(c->large_gap);
    }
    free(ch);
    free(bp);

    out->count = acc.count;
    out->pi_4_1 = acc.c41;
    out->pi_4_3 = c43;
    out->pi_3_1 = acc.c31;
    out->pi_3_2 = c32;
    out->first = have ? acc.first : 0;
    out->last = have ? last : 0;
    out->max_gap = acc.max_gap;
    out->max_gap_start = acc.max_gap_start;
    memcpy(out->hist, acc.hist, sizeof(acc.hist));
    out->num_gaps = acc.count ? acc.count - 1 : 0;
    out->n_large = acc.nlarge;
    uint64_t ncopy = acc.nlarge < large_cap ? acc.nlarge : large_cap;
    for (uint64_t j = 0; j < ncopy; j++) {
        if (large_pos) large_pos[j] = acc.large_pos[j];
        if (large_gap) large_gap[j] = acc.large_gap[j];
    }
    free(acc.large_pos);
    free(acc.large_gap);
    return 0;
}

int64_t oracle_primes_in_range(uint64_t a, uint64_t b, uint64_t* out,
                               uint64_t cap) {
    /* primes q with a <= q <= b, ascending (range.cu:99-262 semantics) */
    if (b < a) return 0;
    uint64_t n = 0;
    static const uint64_t seeds[3] = {2, 3, 5};
    for (int s = 0; s < 3; s++)
        if (seeds[s] >= a && seeds[s] <= b) {
            if (n < cap && out) out[n] = seeds[s];
            n++;
        }
    if (b < 7) return (int64_t)n;
    uint64_t k_lo = a / 30, k_hi = b / 30 + 1;
    uint64_t nbp = 0;
    uint32_t* bp = base_primes(isqrt_u64(b), &nbp);
    uint8_t* seg = (uint8_t*)malloc(CHUNK_BYTES);
    for (uint64_t k0 = k_lo; k0 < k_hi; k0 += CHUNK_BYTES) {
        uint64_t nb = k_hi - k0 < CHUNK_BYTES ? k_hi - k0 : CHUNK_BYTES;
        sieve_bytes(seg, k0, nb, bp, nbp);
        for (uint64_t i = 0; i < nb; i++) {
            uint8_t v = seg[i];
            for (int o = 0; v && o < 8; o++) {
                if (!((v >> o) & 1)) continue;
                uint64_t q = bitval(k0 + i, o);
                if (q < a || q > b || q < 7) continue;
                if (n < cap && out) out[n] = q;
                n++;
            }
        }
    }
    free(seg);
    free(bp);
    return (int64_t)n;
}

/* Odd-number primality bitmap for [0, limit]: bit i <-> 2i+1.  */
static uint64_t* odd_prime_bits(uint64_t limit, uint64_t* nwords_out) {
    uint64_t nodd = limit / 2 + 1;
    uint64_t nwords = (nodd + 63) / 64;
    uint64_t* bits = (uint64_t*)calloc(nwords, 8);
    uint64_t nbp = 0;
    uint32_t* bp = base_primes(isqrt_u64(limit), &nbp);
    uint8_t* seg = (uint8_t*)malloc(CHUNK_BYTES);
    uint64_t k_hi = limit / 30 + 1;
    for (uint64_t k0 = 0; k0 < k_hi; k0 += CHUNK_BYTES) {
        uint64_t nb = k_hi - k0 < CHUNK_BYTES ? k_hi - k0 : CHUNK_BYTES;
        sieve_bytes(seg, k0, nb, bp, nbp);
        for (uint64_t i = 0; i < nb; i++) {
            uint8_t v = seg[i];
            for (int o = 0; v && o < 8; o++) {
                if (!((v >> o) & 1)) continue;
                uint64_t q = bitval(k0 + i, o);
                if (q > limit) continue;
                bits[(q >> 1) >> 6] |= 1ull << ((q >> 1) & 63);
            }
        }
    }
    if (limit >= 3) bits[0] |= 1ull << 1;   /* 3 */
    if (limit >= 5) bits[0] |= 1ull << 2;   /* 5 */
    free(seg);
    free(bp);
    *nwords_out = nwords;
    return bits;
}

int oracle_goldbach_minp(uint64_t N, int nthreads, uint32_t* minp,
                         uint64_t* hist, uint64_t hist_bins,
                         uint32_t* max_minp, uint64_t* n_counterexamples,
                         uint64_t* sum_minp) {
    /* For every even n in [4, N]: the smallest prime p with n - p prime
     * (goldbach_upto.cu:38-43 stops at exactly that p).  minp[(n-4)/2] = p
     * (0 for a counterexample) when minp is given.  hist[p] counts the n
     * whose smallest p is p (p < hist_bins); sum_minp is the sum of all p. */
    if (N < 4) return 1;
    uint64_t nw = 0;
    uint64_t* bits = odd_prime_bits(N, &nw);
    uint64_t nn = (N - 4) / 2 + 1;
    uint64_t np = 0;
    uint32_t* plist = base_primes(N / 2, &np);   /* odd primes >= 7 */
    const uint32_t small[2] = {3, 5};
    uint32_t mx = 0;
    uint64_t nce = 0, sum = 0;
    if (hist) memset(hist, 0, hist_bins * 8);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel reduction(max:mx) reduction(+:nce, sum)
#endif
    {
        uint64_t* lh = hist ? (uint64_t*)calloc(hist_bins, 8) : NULL;
#ifdef _OPENMP
#pragma omp for schedule(static, 65536)
#endif
        for (int64_t i = 0; i < (int64_t)nn; i++) {
            uint64_t n = 4 + 2 * (uint64_t)i;
            uint32_t found = 0;
            if (n == 4) {
                found = 2;
            } else {
                for (uint64_t j = 0; j < 2 + np && !found; j++) {
                    uint64_t p = j < 2 ? small[j] : plist[j - 2];
                    if (p > n / 2) break;
                    uint64_t m = n - p;            /* odd */
                    if ((bits[(m >> 1) >> 6] >> ((m >> 1) & 63)) & 1) found = (uint32_t)p;
                }
            }
            if (minp) minp[i] = found;
            if (!found) nce++;
            if (found > mx) mx = found;
            sum += found;
            if (lh && found && found < hist_bins) lh[found]++;
        }
        if (lh) {
#ifdef _OPENMP
#pragma omp critical
#endif
            for (uint64_t h = 0; h < hist_bins; h++) hist[h] += lh[h];
            free(lh);
        }
    }
    free(plist);
    free(bits);
    if (max_minp) *max_minp = mx;
    if (n_counterexamples) *n_counterexamples = nce;
    if (sum_minp) *sum_minp = sum;
    return 0;
}

int oracle_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
