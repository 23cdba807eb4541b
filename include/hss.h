/*
 * hss.h - C ABI of the GB300 (sm_103a) square-sided Heronian triangle search.
 *
 * The reference has no library interface: its GPU search is one CUDA program
 * whose kernel signature and host object are the in-process boundary
 * (src/gpu_search_v42.cu:292-297 `search_kernel(n, first_l, info, fourth,
 * has_inert, prime_offsets, values, factor_info, cached, hits, hit_count,
 * candidate_total)`, owned by `Search::prepare` :354 and `Search::run` :393),
 * and its process boundary is the command line `gpu_search_v42 LIMIT FIRST_L
 * LAST_L RESULTS_FILE [GPU [STATE_FILE]]` (:610-632).  This header replaces
 * the in-process boundary; the command-line drop-in (gpu_search_v42) is built
 * on top of it.
 *
 * Conventions: plain C types, caller-owned output buffers, opaque handles,
 * status 0 on success and a negative HSS_ERR_* code on failure (message via
 * hss_last_error).  A handle is not thread-safe; the serving calls are
 * serialised internally.
 */
#ifndef HSS_H
#define HSS_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HSS_OK 0
#define HSS_ERR_ARGUMENT (-1)  /* invalid argument (range, null pointer) */
#define HSS_ERR_CUDA (-2)      /* CUDA runtime error (message has the detail) */
#define HSS_ERR_MEMORY (-3)    /* host or device allocation failed */
#define HSS_ERR_LIMIT (-4)     /* limit beyond what the cache layout indexes */
#define HSS_ERR_STATE (-5)     /* checkpoint does not match the request */
#define HSS_ERR_OVERFLOW (-6)  /* an internal capacity was exceeded */
#define HSS_ERR_NOT_FOUND (-7) /* unknown request id */
#define HSS_ERR_BUSY (-8)      /* request still running */
#define HSS_ERR_NO_DEVICE (-9) /* no CUDA device / wrong architecture */

#define HSS_MAX_LIMIT 30000000ULL  /* every segment (<= 4063 values) fits a work item */

/* Enumeration paths.  PLAIN mirrors the reference's launch shape (one block
 * per (root, slice), one thread per pair, gpu_search_v42.cu:298-304);
 * BATCHED is the persistent kernel draining a work queue of (root, m-range)
 * items weighted by Gaussian divisor count.  Both give identical counts. */
#define HSS_MODE_PLAIN 0
#define HSS_MODE_BATCHED 1

typedef struct hss_ctx hss_t;

typedef struct {
    uint32_t prep_threads;    /* host threads for the cache build (0: all cores) */
    uint32_t hit_capacity;    /* device hit buffer per launch (0: 4096, as
                                 gpu_search_v42.cu:177-178) */
    uint32_t block_threads;   /* batched CTA size: 128, 256 or 512 (0: 256) */
    uint32_t item_target;     /* batched item weight in alpha*beta evaluations
                                 (0: 1<<23) */
    uint32_t ctas_per_sm;     /* batched kernel variant: minimum CTAs per SM it is
                                 compiled for (128 threads: 4 or 6; 256: 2 or 3;
                                 512: 1); 0 picks 4 / 2 / 1 */
    uint32_t use_graph;       /* 1: capture each batched launch sequence in a
                                 CUDA graph */
    uint32_t host_build;      /* 1: build the factor cache with host threads
                                 and upload it; 0 (default): build it with
                                 kernels on the device (same arrays and values,
                                 about 10x faster) */
    uint32_t exact_capacity;  /* initial exact-work queue items (0: 1<<24); a
                                 launch group that outgrows the queue makes the
                                 call grow it 4x (up to 1<<28) and run again */
    uint32_t serve_state_kb;  /* serving: device memory for the admitted
                                 requests' row records, 80 bytes per root row
                                 (0: 1/16 of free HBM at serve start, at most
                                 256 MiB); admission waits for room in it */
} hss_opts;

/* Counters of one search call.  `pairs` and `candidates` are the reference's
 * counters (search_v18.cpp:322, gpu_search_v42.cu:160); the rest are the
 * work figures the kernels export: processed pairs (not both even, no
 * shared p = 3 mod 4 prime, some split prime), Gaussian products tested,
 * candidates whose z = l^4+m^4-D passes mod 16, products settled by the
 * exact 128-bit path, pairs sharing a split prime, and hits found. */
typedef struct {
    uint64_t pairs;
    uint64_t processed;
    uint64_t products;
    uint64_t candidates;
    uint64_t r16;
    uint64_t exact;
    uint64_t merged;
    uint64_t hits;
    double kernel_ms;   /* device time of the whole call (CUDA events on its stream) */
    double main_ms;     /* device time of the batched / plain kernels */
    double merged_ms;   /* device time of the shared-prime kernels */
    uint64_t merged_products;    /* products, candidates and mod-16 survivors of */
    uint64_t merged_candidates;  /* the pairs sharing a split prime (included in */
    uint64_t merged_r16;         /* the totals above) */
    uint64_t h2d_bytes;          /* host-to-device bytes copied by the call */
    uint64_t d2h_bytes;          /* device-to-host bytes copied by the call */
    uint32_t launches;           /* kernels launched by the call */
    uint32_t graph_launches;     /* CUDA graph launches of the call (opts.use_graph) */
    uint32_t reruns;             /* times the call ran again after growing the
                                    exact-work or big-pair queue */
    uint32_t reserved;
} hss_counts;

/* A hit (l <= m <= n, gcd 1), with the signed 4A of the representation that
 * produced it; area = |4A| / 4.  heron_ok is the device's 256-bit Heron
 * recheck (all four Heron factors positive, product equal to (4A)^2). */
typedef struct {
    uint64_t l, m, n;
    uint64_t area4_lo;
    int64_t area4_hi;
    uint32_t heron_ok;
    uint32_t reserved;
} hss_hit;

/* Version string of the library. */
const char* hss_version(void);

/* Text for a status code. */
const char* hss_strerror(int status);

/* Last error message recorded on the handle (never NULL). */
const char* hss_last_error(const hss_t* h);

/* Builds the Gaussian factor cache for LIMIT resident on `device`, by
 * kernels on the device or (opts->host_build) on the host and uploaded
 * (replaces Search::prepare and the uploads of Search::run,
 * gpu_search_v42.cu:354-432).  1 <= limit <= HSS_MAX_LIMIT. */
int hss_open(uint64_t limit, int device, const hss_opts* opts, hss_t** out);

/* Releases the device cache and the handle (gpu_search_v42.cu:496-505). */
void hss_close(hss_t* h);

/* Limit of the handle and sizes of its cache: records (free + central
 * values), and the sizes the reference's preparation prints on stderr,
 * "flattened N Gaussian values" and "cached N Gaussian pair values"
 * (gpu_search_v42.cu:606, 567), recomputed for this limit. */
int hss_info(const hss_t* h, uint64_t* limit, uint64_t* records, uint64_t* flattened,
             uint64_t* cached, double* prep_seconds);

/* Measures the device's 32-bit integer instruction throughput with a probe
 * kernel (independent multiply-add and shift/logic chains on every SM);
 * used as the denominator of the integer roofline. */
int hss_int32_peak(int device, double* ops_per_second, double* ms);

/* Host-only inspection of the factor cache layout for LIMIT (no device is
 * touched): the number of records (free + central values) and the two sizes
 * the reference's preparation reports.  If x != 0, the segment of x (its free
 * set followed by the central value x^2) is copied to re/im (up to cap
 * values) and its length stored in *count. */
int hss_cache_inspect(uint64_t limit, uint64_t x, uint64_t* records, uint64_t* flattened,
                      uint64_t* cached, int64_t* re, int64_t* im, uint32_t cap, uint32_t* count);

/* Builds the factor cache for LIMIT both ways - kernels on `device` (the
 * default of hss_open) and host threads (hss_opts.host_build) - and compares
 * every array entry by entry: smallest prime factors, segment offsets, hot
 * and exact records, record owners, the prime-power index and both
 * prime-power tables, and the reported sizes.  *mismatches receives the
 * number of differing entries (0: identical); *host_seconds and
 * *device_seconds (when not NULL) the two build times.  A verification entry
 * point: no counterpart in the reference. */
int hss_cache_check(uint64_t limit, int device, uint64_t* mismatches, double* host_seconds,
                    double* device_seconds);

/* Searches root rows first..last (1 <= first <= last <= limit) against all
 * m in [l, limit] with the given mode (one reference "batch" when last-first
 * < 512, gpu_search_v42.cu:456-482).  Counters go to *out.  row_candidates,
 * if not NULL, receives last-first+1 per-row candidate counts.  Up to
 * hit_cap hits are copied to `hits`, sorted by (l, m, n) and deduplicated;
 * *nhits receives the number found (which may exceed hit_cap). */
int hss_search(hss_t* h, uint64_t first, uint64_t last, int mode, hss_counts* out,
               uint64_t* row_candidates, hss_hit* hits, uint32_t hit_cap, uint32_t* nhits);

/* Autotuner: times the batched path on rows first..last (a sample of the
 * intended workload) for every compiled kernel variant (CTA size and minimum
 * CTAs per SM, which caps registers per thread) and item weight, keeps the
 * fastest configuration in the handle's options and returns it in *best.
 * `trials` receives up to max_trials (threads, ctas_per_sm, item_target,
 * milliseconds) records when not NULL. */
typedef struct {
    uint32_t block_threads, ctas_per_sm, item_target;
    float ms;
} hss_tune_trial;

int hss_autotune(hss_t* h, uint64_t first, uint64_t last, hss_opts* best, hss_tune_trial* trials,
                 uint32_t max_trials, uint32_t* ntrials);

/* The same search as hss_search (batched path), for callers that cannot
 * allocate memory while searching - processes whose device memory is owned
 * by a pool or an embedding runtime fixed at start-up, or loops that cannot
 * take the synchronisation an allocation implies.  hss_search grows its
 * per-call buffers with cudaMalloc / cudaMallocHost; this call allocates
 * nothing: its device scratch is one array of about 23 MiB that is static in
 * the library (every GPU that loads the library holds it until the process
 * exits), its host staging is static too, and the handle's cache, stream and
 * tables (made by hss_open) are the inputs.  Limit per call: at most 64 root
 * rows (HSS_ERR_LIMIT beyond that); up to 4096 hits kept.  The array holds
 * 2^20 pairs sharing a split prime, 2^16 exact-work items and 2^13 big
 * shared-prime pairs at a time, so a call runs as several launch groups
 * when its rows need more (a row at LIMIT 10^7 has about 85,000 such pairs:
 * about 12 rows per group), and a group whose exact-work or big-pair queue
 * fills is run again in smaller pieces (down to 64 roots of one row, then
 * HSS_ERR_OVERFLOW).  The first call on a device looks up the
 * array's device address (cudaGetSymbolAddress) and should come before any
 * stream capture.  Calls share the array: they are serialised within the
 * process, clear what must start at zero, and calls that overlap on the GPU
 * race.  Errors are reported by status only (hss_last_error is not updated).
 * No counterpart in the reference. */
int hss_search_noalloc(hss_t* h, uint64_t first, uint64_t last, hss_counts* out, hss_hit* hits,
                       uint32_t hit_cap, uint32_t* nhits);

/* Batched search of several intervals in one persistent launch sequence:
 * intervals i = [firsts[i], lasts[i]].  per_interval (count entries) receives
 * each interval's counters; hits of all intervals are returned together. */
int hss_search_many(hss_t* h, const uint64_t* firsts, const uint64_t* lasts, uint32_t count,
                    hss_counts* per_interval, hss_counts* total, hss_hit* hits,
                    uint32_t hit_cap, uint32_t* nhits);

/* ---- serving: continuous admission of interval requests ----
 * Requests are queued by hss_submit and advanced by a background loop that
 * launches waves of batched work: each wave takes wave_mpairs x 2^20 logical
 * pairs from the oldest admitted request and one root row from every younger
 * one, so requests that arrive while others run join at the next wave, short
 * ones finish within a few waves, and large ones finish in arrival order.  Waves alternate between two launch lanes (a stream and launch
 * buffers each), so one runs while the previous one is harvested.  Every
 * admitted request keeps its per-row counters in a device arena sized at
 * hss_serve_start (hss_opts.serve_state_kb, else 1/16 of free device memory
 * up to 256 MiB; 80 bytes per root row): a request is admitted when a slot
 * (max_active) and room for its rows are free, and hss_submit refuses one
 * larger than the whole arena (HSS_ERR_MEMORY).  Results are the same as
 * hss_search on the same interval.  No counterpart in the reference. */
typedef struct {
    uint64_t first, last;
    uint64_t submitted_ns;  /* CLOCK_MONOTONIC at submit */
    uint64_t admitted_ns;   /* when the request first joined a wave */
    uint64_t finished_ns;   /* when its last wave completed (0 if running) */
    hss_counts counts;
    uint32_t nhits;
    int32_t status;         /* HSS_OK when done, HSS_ERR_BUSY while running */
} hss_request_info;

/* max_active: requests admitted at once (0: 64).  wave_mpairs: logical pairs
 * per wave in units of 2^20 (0: 256), shared among the admitted requests. */
int hss_serve_start(hss_t* h, uint32_t max_active, uint32_t wave_mpairs);
int hss_submit(hss_t* h, uint64_t first, uint64_t last, uint64_t* request_id);
int hss_poll(hss_t* h, uint64_t request_id, hss_request_info* info, hss_hit* hits,
             uint32_t hit_cap);
int hss_wait(hss_t* h, uint64_t request_id, hss_request_info* info, hss_hit* hits,
             uint32_t hit_cap);
int hss_serve_stop(hss_t* h);

#ifdef __cplusplus
}
#endif

#endif /* HSS_H */
