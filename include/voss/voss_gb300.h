/* voss_gb300.h -- additions to the voss C ABI made by the GB300 build.
 *
 * Everything here is additive: the reference has no counterpart for range
 * statistics over an arbitrary [a, b), batches, reusable launch plans, the
 * smallest-Goldbach-prime output or the request server.  The reference
 * functions these build on are cited per entry.  All functions return a
 * VOSS_* code from voss.h and set voss_get_last_error() on failure.
 */
#ifndef VOSS_GB300_H
#define VOSS_GB300_H

#include <stdint.h>
#include "voss/voss.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Gap histogram of a range, indexed by gap/2: bin 0 is the gap 1 (2 -> 3),
 * bin i (1 <= i <= 200) the gap 2i, bin 201 every gap above 400. */
#define VOSS_GAP_BINS 202
/* The full histogram: bins 0..1023 as above (gaps up to 2046), bin 1024
 * every gap >= 2048. */
#define VOSS_GAP_BINS_FULL 1025

/* Statistics of the primes q with a <= q < b.  Gaps are between consecutive
 * primes that both lie in [a, b).  twins/cousins/sexy count gaps of 2/4/6
 * between consecutive primes, as the reference's ctx_twins/cousin/sexy do
 * (context.cu:965-975).  Chebyshev classes: pi_4_1 / pi_4_3 primes = 1 / 3
 * mod 4 (2 in neither), pi_3_1 / pi_3_2 primes = 1 / 2 mod 3 (3 in neither).
 * max_gap_start is the first prime of the earliest largest gap.
 * large_gaps counts gaps >= 500 (the reference's threshold, context.cu:64). */
typedef struct {
    uint64_t a, b;
    uint64_t count;
    uint64_t twins, cousins, sexy;
    uint64_t pi_4_1, pi_4_3, pi_3_1, pi_3_2;
    uint64_t first_prime, last_prime;      /* 0 if there is no prime */
    uint64_t max_gap, max_gap_start;       /* 0 if fewer than two primes */
    uint64_t num_gaps;
    uint64_t large_gaps;
    uint64_t gap_hist[VOSS_GAP_BINS];
} voss_range_stats_t;

/* One range [a, b), b <= 10^14 + 10^10 + 1.  Replaces the reference's
 * in_range_with_limit + host reduction for offset ranges (range.cu:99-262). */
int voss_primes_range_stats(uint64_t a, uint64_t b, voss_range_stats_t* out);

/* As above, plus the full gap/2 histogram (VOSS_GAP_BINS_FULL entries) when
 * hist_full is not NULL. */
int voss_primes_range_stats_ex(uint64_t a, uint64_t b, voss_range_stats_t* out,
                               uint64_t* hist_full);

/* n independent ranges in one launch (one persistent kernel over all their
 * segments).  out[i] is the result of [a[i], b[i]).  Ranges that overlap
 * sieve their common integers once: the ranges are cut at every endpoint
 * into disjoint pieces, each piece is sieved once and each range is rebuilt
 * from its pieces, gaps stitched where they meet; results are the same as
 * one call per range.  Batches of more than 32768 ranges run in chunks of
 * that size (sharing within a chunk). */
int voss_primes_range_stats_batch(uint64_t n, const uint64_t* a, const uint64_t* b,
                                  voss_range_stats_t* out);

/* How a batch shares work (voss_primes_range_stats_batch and the server):
 * the ranges [a[i], b[i]) cut at every endpoint into the disjoint pieces
 * that some range covers, ascending.  Writes *npieces, the pieces
 * [piece_a[j], piece_b[j]) and piece_gaps[j] (1 if a range over the piece
 * has gaps_wanted[i] != 0, or gaps_wanted is NULL), and for each range the
 * pieces [first[i], last[i]) that tile it (0, 0 for an empty range).  cap is
 * the room in the piece arrays; 2n - 1 always suffices.  Host only: runs
 * without a GPU. */
int voss_gb300_cut_ranges(uint64_t n, const uint64_t* a, const uint64_t* b,
                          const uint32_t* gaps_wanted, uint64_t cap, uint64_t* piece_a,
                          uint64_t* piece_b, uint32_t* piece_gaps, uint64_t* npieces,
                          uint32_t* first, uint32_t* last);

/* voss_primes_range_stats for callers that cannot allocate device memory
 * while they run -- for instance a process whose device memory belongs to
 * another framework's caching allocator, or a latency-critical loop where
 * cudaMalloc / cudaFree would synchronize the device.  The reference has no
 * counterpart.  The call allocates nothing: its scratch, sieving-prime table
 * and presieve tiles live in static device arrays of this library (about
 * 29.9 MB per GPU that loads it, held until the process exits).  The caller
 * passes the range and `out`, device-accessible memory that receives the
 * result in stream order on `stream` (a cudaStream_t, NULL = legacy default
 * stream); the call returns once the work is enqueued.
 * Limits: b <= 2^40 and a width of at most 65536 segments of 221184 bytes
 * (about 4.3 * 10^11 integers); beyond them VOSS_ERR_OUT_OF_RANGE.
 * The first call on a device sets that device up; make it before any stream
 * capture.  All calls share one scratch array and leave their contents
 * behind: calls in sequence are independent, calls that overlap on the GPU
 * race and give wrong results.
 * Errors: a refused launch shows in the return code; a fault while the
 * kernels run surfaces on the caller's next synchronisation of `stream`.
 * If a CUDA error is already pending on the calling thread, the call
 * returns VOSS_ERR_CUDA without launching and leaves that error in place. */
int voss_primes_range_stats_noalloc(uint64_t a, uint64_t b, voss_range_stats_t* out,
                                    void* stream);

/* Tunables of the segmented sieve.  seg_bytes: shared-memory segment in
 * bytes (30 integers each), a multiple of 128, at most 222848.  threads: CTA
 * size (multiple of 32, <= 1024).  tier_split: primes below it are marked a
 * warp per prime, primes from it on four primes per warp.  ctas_per_sm: resident
 * CTAs per SM used to size the persistent grid.  Zero fields keep the
 * current value; auto_tune = 1 lets the library pick per range.
 * set_config and set_tuning return VOSS_ERR_INVALID_ARG while a request
 * server runs on the device (its thread reads both). */
typedef struct {
    uint32_t seg_bytes;
    uint32_t threads;
    uint32_t tier_split;
    uint32_t ctas_per_sm;
    uint32_t auto_tune;
    uint32_t bucket_split;   /* with auto_tune = 0: primes from here on (and >= the
                                segment) go through bucket lists; 0 = none */
    uint32_t bucket_cap_pct; /* bucket list capacity in percent of the default
                                (many standard deviations above the mean); a
                                list that overflows makes the run repeat
                                without lists, so results never change */
} voss_gb300_config_t;

int voss_gb300_get_config(voss_gb300_config_t* out);
int voss_gb300_set_config(const voss_gb300_config_t* cfg);

/* Offset-regime tuning table (written by voss_gb300/autotune.py, a built-in
 * copy ships in the library): a range [a, b) uses the first entry with
 * b <= b_max and b - a <= width_max.  n = 0 clears the table (the built-in
 * rule then applies).  Bucket lists are used for ranges of 2 to 4096
 * segments. */
typedef struct {
    uint64_t b_max;
    uint64_t width_max;
    uint32_t seg_bytes;
    uint32_t tier_split;
    uint32_t bucket_split;   /* primes from here on (and >= the segment) are
                                marked from per-segment bucket lists; 0 = none */
} voss_gb300_tune_entry_t;

int voss_gb300_set_tuning(uint32_t n, const voss_gb300_tune_entry_t* entries);
int voss_gb300_get_tuning(uint32_t cap, voss_gb300_tune_entry_t* entries, uint32_t* n);

/* A launch plan: the requests, their segment list and all device buffers,
 * prepared once and launched any number of times on a caller's stream (also
 * inside stream capture, after the first launch).  Used to time the device
 * part alone and by the request server. */
typedef struct voss_gb300_plan voss_gb300_plan;

int voss_gb300_plan_create(uint64_t n, const uint64_t* a, const uint64_t* b,
                           voss_gb300_plan** out);
/* Enqueue one full run (reset, sieve, finalize) on `stream` (a cudaStream_t;
 * NULL = the legacy default stream).  Does not synchronise. */
int voss_gb300_plan_launch(voss_gb300_plan* plan, void* stream);
/* Copy the results of the last run to the host (synchronises `stream`). */
int voss_gb300_plan_results(voss_gb300_plan* plan, voss_range_stats_t* out, void* stream);
/* Segments, grid size, kernels per run, shared bytes per CTA, and the
 * algorithmic work of one run: the candidate clears of Eratosthenes by the
 * primes 17 < p <= sqrt(b) of each range (whether the presieve tiles or the
 * marking does them), and the wheel bytes covered. */
int voss_gb300_plan_info(voss_gb300_plan* plan, uint64_t* total_segments, uint32_t* grid,
                         uint32_t* kernels_per_run, uint32_t* smem_bytes,
                         uint64_t* clears, uint64_t* wheel_bytes);
void voss_gb300_plan_free(voss_gb300_plan* plan);
/* Durations in ms of the sieve (the bucket fill kernel, when the run uses
 * bucket lists, plus the sieve kernel) and of the finalize kernel of the
 * plan's last launch, from CUDA events recorded on the launching stream
 * (waits for that launch to finish). */
int voss_gb300_plan_kernel_ms(voss_gb300_plan* plan, float* sieve_ms, float* finalize_ms);

/* Every even n in [4, N], N <= 4*10^11: the smallest prime p with n - p prime
 * (the p at which the reference's goldbach_check_kernel stops,
 * goldbach_upto.cu:38-43; the reference does not output it).
 * minp: NULL or (N-4)/2+1 entries, minp[(n-4)/2] = p, 0 for a counterexample.
 * hist: NULL or VOSS_GOLDBACH_HIST_BINS entries, hist[p] = number of n.
 * max_minp, sum_minp, n_counterexamples: NULL or outputs. */
#define VOSS_GOLDBACH_HIST_BINS 65536
int voss_primes_goldbach_minp(uint64_t N, uint32_t* minp, uint64_t* hist,
                              uint32_t* max_minp, uint64_t* sum_minp,
                              uint64_t* n_counterexamples);

/* Device-resident Goldbach run (sieve, odd-number bitmap, min-p kernel) that
 * can be launched repeatedly on a stream; used to time the device part. */
typedef struct voss_gb300_goldbach voss_gb300_goldbach;
int voss_gb300_goldbach_create(uint64_t N, voss_gb300_goldbach** out);
int voss_gb300_goldbach_launch(voss_gb300_goldbach* g, void* stream);
int voss_gb300_goldbach_results(voss_gb300_goldbach* g, uint32_t* max_minp,
                                uint64_t* sum_minp, uint64_t* n_counterexamples,
                                uint64_t* hist, uint64_t* probes, void* stream);
void voss_gb300_goldbach_free(voss_gb300_goldbach* g);

/* Request server with continuous batching.  Requests (a range and what is
 * asked of it) are submitted at any time; a scheduler thread packs the
 * pending ones into batches, FIFO, while batch slots and device memory
 * (segment records, accumulators, results of every batch in flight) allow,
 * and runs each batch as one replayed CUDA graph on its slot's stream, so
 * batches overlap on the device.  Admission counts each request's segment
 * records, accumulators, results and bucket lists.  The reference has no counterpart: it
 * serves one Context at a time (context.cu:212-559).  Every request gets the
 * full voss_range_stats_t; for COUNT and CHEBYSHEV requests the gap fields
 * are not computed (zero).  A request wider than half a batch runs as
 * consecutive pieces of at most half a batch, interleaved with other requests'
 * batches, and its result is merged from theirs; any range with b up to
 * 10^14 + 10^10 + 1 is accepted. */
#define VOSS_OP_COUNT      0
#define VOSS_OP_TWINS      1
#define VOSS_OP_GAP_HIST   2
#define VOSS_OP_CHEBYSHEV  3

typedef struct {
    uint32_t slots;               /* batches in flight (default 4) */
    uint32_t max_batch;           /* requests per batch (default 1024) */
    uint64_t max_segments;        /* segments per batch (default 65536) */
    uint64_t memory_budget;       /* device bytes over all batches in flight */
    uint32_t use_graphs;          /* replay a captured CUDA graph per batch */
    uint64_t bucket_bytes;        /* bucket-list arena per slot (default 256 MiB) */
    uint32_t isolate_requests;    /* nonzero: each request of a batch is sieved on
                                     its own; default (0): overlapping requests of
                                     a batch share the sieving of their common
                                     integers (results are the same either way) */
} voss_gb300_server_config_t;

typedef struct {
    uint64_t submitted, completed, pending, batches;
    uint64_t max_inflight_batches, peak_admitted_bytes;
    double p50_us, p99_us, mean_us;   /* submit -> result ready */
    double req_per_s;                 /* completed / (last completion - first submit) */
    double mean_batch;
} voss_gb300_server_metrics_t;

typedef struct voss_gb300_server voss_gb300_server;

/* cfg may be NULL (defaults); zero fields take the defaults. */
int voss_gb300_server_create(const voss_gb300_server_config_t* cfg, voss_gb300_server** out);
int voss_gb300_server_submit(voss_gb300_server* s, uint64_t a, uint64_t b, uint32_t op,
                             uint64_t* ticket);
/* wait = 0: *ready = 0 if the result is not there yet.  On ready, *out gets
 * the result and the ticket is released. */
int voss_gb300_server_result(voss_gb300_server* s, uint64_t ticket, int wait,
                             voss_range_stats_t* out, double* latency_us, int* ready);
int voss_gb300_server_drain(voss_gb300_server* s);
int voss_gb300_server_metrics(voss_gb300_server* s, voss_gb300_server_metrics_t* out);
int voss_gb300_server_reset_metrics(voss_gb300_server* s);
void voss_gb300_server_free(voss_gb300_server* s);

/* Shared-memory bandwidth of this GPU in GB/s, measured by two
 * microbenchmarks (conflict-free 32-bit load+store, and atomicAnd; 8 bytes
 * per step each): the denominators of the sieve's roofline. */
int voss_gb300_smem_peak(double* ldst_gbs, double* atomic_gbs);

/* SM clocks per warp-wide shared-memory atomicAnd on this GPU when the 32
 * lanes' banks are distinct, shared 2, 4 or 8 ways, and scattered (clocks[0..4]):
 * the cost model of the sieve's marking (one wavefront per bank conflict).
 * No counterpart in the reference. */
int voss_gb300_smem_atomic_cost(double* clocks);

/* Name of the device the library runs on, and its SM count. */
int voss_gb300_device_info(char* name, uint32_t name_len, uint32_t* sm_count);

#ifdef __cplusplus
}
#endif

#endif /* VOSS_GB300_H */
