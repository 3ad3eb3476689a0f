/* voss_oracle.h -- CPU restatement of voss's sieve statistics (test
 * infrastructure only; see voss_oracle.c for what it restates). */
#ifndef VOSS_ORACLE_H
#define VOSS_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Gap histogram bins by gap/2: bin 0 holds the gap 1 (2 -> 3), bin i the gap
 * 2i for 1 <= i < ORACLE_HBINS-1, the last bin every gap >= 2*(HBINS-1). */
#define ORACLE_HBINS 1025

typedef struct {
    uint64_t a, b;             /* the half-open range [a, b) */
    uint64_t count;            /* primes in [a, b) */
    uint64_t pi_4_1, pi_4_3;   /* primes = 1, 3 (mod 4) */
    uint64_t pi_3_1, pi_3_2;   /* primes = 1, 2 (mod 3) */
    uint64_t first, last;      /* smallest / largest prime, 0 if none */
    uint64_t max_gap;          /* largest gap, 0 if fewer than two primes */
    uint64_t max_gap_start;    /* first prime of the earliest largest gap */
    uint64_t num_gaps;         /* count - 1, or 0 */
    uint64_t n_large;          /* gaps >= the large threshold */
    uint64_t hist[ORACLE_HBINS];
} oracle_stats_t;

int oracle_range_stats(uint64_t a, uint64_t b, int nthreads,
                       uint64_t large_threshold, oracle_stats_t* out,
                       uint64_t* large_pos, uint32_t* large_gap,
                       uint64_t large_cap);

int64_t oracle_primes_in_range(uint64_t a, uint64_t b, uint64_t* out,
                               uint64_t cap);

int oracle_goldbach_minp(uint64_t N, int nthreads, uint32_t* minp,
                         uint64_t* hist, uint64_t hist_bins,
                         uint32_t* max_minp, uint64_t* n_counterexamples,
                         uint64_t* sum_minp);

int oracle_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif
