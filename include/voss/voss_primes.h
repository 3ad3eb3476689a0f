/* voss_primes.h -- the prime-sieve part of the voss C ABI.
 *
 * Same declarations as the reference's library/include/voss/voss_primes.h
 * (lines cited per entry), so its ctypes binding (bindings/python/voss/
 * _capi.py) and C callers bind this library unchanged.  The sieve behind
 * them is the GB300 segmented sieve of this project; results are the
 * reference's, bit for bit, on the same inputs.
 *
 * Entry points outside the sieve (Miller-Rabin, factorisation, Mersenne /
 * Fermat tests, single-n Goldbach partitions) are exported so that the
 * binding loads, and return VOSS_ERR_INTERNAL with a message.
 */
#ifndef VOSS_PRIMES_H
#define VOSS_PRIMES_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* pi(N): primes <= N; 2 <= N <= 10^14 (voss_primes.h:13, prime_count.cu:298). */
int voss_primes_prime_count(uint64_t N, uint64_t* out);

/* Profiles (voss_primes.h:18-20).  MINIMAL counts only; STANDARD and FULL
 * compute counts, gap histogram, Chebyshev counts and large gaps. */
#define VOSS_PROFILE_MINIMAL   0
#define VOSS_PROFILE_STANDARD  1
#define VOSS_PROFILE_FULL      2

/* Opaque, caller-owned handle over [1, N] (voss_primes.h:25-28). */
typedef struct voss_primes_ctx voss_primes_ctx;

int voss_primes_ctx_new(uint64_t N, int profile, voss_primes_ctx** out_ctx);
void voss_primes_ctx_free(voss_primes_ctx* ctx);

/* Queries (voss_primes.h:31-34).  The first query runs the sieve once; later
 * queries read the cached result.  Twins / cousin / sexy are the numbers of
 * consecutive primes <= N that differ by 2 / 4 / 6. */
int voss_primes_ctx_prime_count(voss_primes_ctx* ctx, uint64_t* out);
int voss_primes_ctx_twins(voss_primes_ctx* ctx, uint64_t* out);
int voss_primes_ctx_cousin(voss_primes_ctx* ctx, uint64_t* out);
int voss_primes_ctx_sexy(voss_primes_ctx* ctx, uint64_t* out);

/* Sophie Germain primes p <= N (p and 2p+1 prime) (voss_primes.h:43-47). */
int voss_primes_ctx_sophie_germain(voss_primes_ctx* ctx, uint64_t* out);
int voss_primes_ctx_sophie_germain_upto(voss_primes_ctx* ctx, uint64_t* out);

/* Gap moments over the histogram (voss_primes.h:52-62). */
typedef struct {
    double   mean_gap;
    double   std_dev;
    double   skewness;
    double   kurtosis;     /* excess */
    uint64_t total_gaps;
} voss_primes_stats_t;

int voss_primes_ctx_statistics(voss_primes_ctx* ctx, voss_primes_stats_t* out);

/* Primes <= N that are 1 and 3 mod 4 (voss_primes.h:68-70). */
int voss_primes_ctx_chebyshev_bias(voss_primes_ctx* ctx,
                                   uint64_t* out_pi_4_1,
                                   uint64_t* out_pi_4_3);

/* Gaps >= 500, largest first; position = the second prime of the gap
 * (voss_primes.h:76-81). */
int voss_primes_ctx_large_gaps_count(voss_primes_ctx* ctx, uint64_t* out_count);
int voss_primes_ctx_large_gaps_get(voss_primes_ctx* ctx, uint64_t index,
                                   uint64_t* out_position, uint32_t* out_gap);

/* <prefix>_chebyshev.csv, <prefix>_large_gaps.csv, <prefix>_stats.csv
 * (voss_primes.h:94; csv.cpp:17-115). */
int voss_primes_ctx_export_csv(voss_primes_ctx* ctx, const char* prefix);

/* Primes in [a, b] inclusive, ascending, in a malloc'd array released by
 * voss_free; more than max_count primes -> VOSS_ERR_OUT_OF_MEMORY
 * (voss_primes.h:101-106, range.cu:267-323; the default limit is 10^7). */
int voss_primes_in_range(uint64_t a, uint64_t b,
                         uint64_t** out_array, uint64_t* out_count);
int voss_primes_in_range_with_limit(uint64_t a, uint64_t b, uint64_t max_count,
                                    uint64_t** out_array, uint64_t* out_count);

/* n-th prime (1-based, n <= 5*10^7), smallest prime > x, largest prime < x,
 * all on the GPU sieve (voss_primes.h:109-116; nth.cu:40-103,
 * next_prev.cu:22-83 validate the same way).  x must stay below
 * 10^14 + 10^10, the sieve's range; beyond it VOSS_ERR_OUT_OF_RANGE. */
int voss_primes_nth(uint64_t n, uint64_t* out_prime);
int voss_primes_next(uint64_t x, uint64_t* out_prime);
int voss_primes_prev(uint64_t x, uint64_t* out_prime);

/* Outside the sieve; exported for the binding (voss_primes.h:121-147). */
int voss_primes_is_prime(uint64_t x, int* out);
int voss_primes_factorize(uint64_t x, uint64_t** out_array, uint64_t* out_count);
int voss_primes_is_mersenne_prime(uint32_t p, int* out);
int voss_primes_is_fermat_prime(uint32_t n, int* out);

/* Called synchronously after each chunk of a Context computation with the
 * chunk number (1-based), the chunk total, the primes >= 7 found in the chunk
 * and the running pi (voss_primes.h:152-159).  Chunks are the reference's
 * segments: [i*S+1, (i+1)*S] with S = 30*ceil(N/30)+10 below 5*10^10, else
 * S = 5*10^10 + 10 (context.cu:260-269). */
typedef void (*voss_progress_cb)(int seg, int total,
                                 uint64_t primes_in_seg,
                                 uint64_t cumulative,
                                 void* user);

int voss_primes_ctx_set_progress(voss_primes_ctx* ctx,
                                 voss_progress_cb cb,
                                 void* user);

/* Outside the sieve; exported for the binding (voss_primes.h:165-170). */
int voss_primes_goldbach_count(uint64_t n, uint64_t* out);
int voss_primes_goldbach_partitions(uint64_t n,
                                    uint64_t** out_array,
                                    uint64_t* out_count);

/* Every even n in [4, N]: the n with no p such that p and n - p are prime,
 * at most max_counterexamples of them, malloc'd (voss_primes.h:178-181,
 * goldbach_upto.cu:48-150).  N < 4 -> VOSS_ERR_INVALID_N; max == 0 -> OK,
 * nothing done. */
int voss_primes_goldbach_test_upto(uint64_t N,
                                   uint64_t** out_counterexamples,
                                   uint64_t* out_count,
                                   uint64_t max_counterexamples);

#ifdef __cplusplus
}
#endif

#endif /* VOSS_PRIMES_H */
