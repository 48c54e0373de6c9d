/*
 * gbsort.h -- C ABI of the GB300 histogram sort (libgbsort.so).
 *
 * Plain pointers and sizes only.  Every entry point returns a gbsort_status;
 * none of them aborts the process.  Device entry points take device
 * pointers and a cudaStream_t passed as `void *` (NULL = the library's own
 * stream of the current device, a blocking stream: it orders after work
 * issued earlier on the legacy default stream, as the legacy stream itself
 * would) and return once the work is enqueued on that stream, except where
 * stated.  Host entry points copy to the current
 * CUDA device, sort there, copy back and return when the result is in host
 * memory.
 *
 * Sort semantics are those of MP-sort (mpsort.h:1-12): records of `elsize`
 * bytes ordered ascending by their radix, stably (the reference's merge
 * sort keeps ties in input order, stdlib/msort.c:76-167, and so does every
 * path here).  The drop-in `radix_sort` / `mpsort_omp` symbols are declared
 * in mpsort.h.
 */
#ifndef GBSORT_H
#define GBSORT_H

#include <stddef.h>
#include <stdint.h>

#include "gbsort_key.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef enum gbsort_status {
    GBSORT_OK = 0,
    GBSORT_ERR_BAD_ARG = 1,      /* NULL pointer, bad key descriptor, size out of range */
    GBSORT_ERR_OOM = 2,          /* device or pinned host memory could not be allocated */
    GBSORT_ERR_CUDA = 3,         /* a CUDA call failed (message: gbsort_last_error) */
    GBSORT_ERR_NO_DEVICE = 4,    /* no CUDA device is visible */
    GBSORT_ERR_INTERNAL = 5,     /* a device-side consistency check failed */
    GBSORT_ERR_UNSUPPORTED = 6   /* this method cannot take this record layout */
} gbsort_status;

typedef enum gbsort_method {
    GBSORT_AUTO = 0,             /* histogram sort with the learned lookup where it applies, else LSD */
    GBSORT_HISTOGRAM_PLAIN = 1,  /* splitters by bisection + binary-search bucket lookup */
    GBSORT_HISTOGRAM_LEARNED = 2,/* splitters and bucket lookup from the trained CDF model */
    GBSORT_LSD = 3               /* stable LSD radix sort of key words + one record permutation */
} gbsort_method;

/* Statistics of the most recent sort on the calling thread's device. */
typedef struct gbsort_stats {
    int32_t method;              /* gbsort_method that ran (never GBSORT_AUTO) */
    uint32_t nbuckets;           /* level-1 buckets */
    uint32_t sample;             /* sampled keys */
    uint32_t splitter_rounds;    /* bisection rounds (plain) or training steps (learned) */
    uint32_t local_sorts;        /* shared-memory bucket sorts */
    uint32_t splits;             /* buckets split once more on device */
    uint32_t copies;             /* single-key buckets copied without sorting */
    uint32_t resplits;           /* sub-buckets over capacity sent to another split round */
    uint32_t bigbin_passes;      /* extra local passes on clustered keys */
    uint32_t window_misses;      /* learned lookups that fell back to the full search */
    uint32_t max_bucket;         /* largest level-1 bucket (records) */
    uint32_t lsd_passes;         /* digit passes of the LSD path */
    uint32_t widest_window;      /* widest learned search window (buckets) */
    float model_loss;            /* final training loss of the learned model */
    /* device time (ms, CUDA events) of the histogram sort's stages: splitter
     * search (sample, sort, bisection or training), bucket counts, count
     * scan, bucket scatter, bucket splits, local sorts */
    float stage_ms[6];
    uint32_t launches;           /* kernels this sort enqueued */
    uint32_t splitter_fallback;  /* 1: the model's splitters failed the sample check and the
                                    sample quantiles (the plain splitters) were used */
    uint32_t heavy_keys;         /* keys owning a single-key bucket worth three splitters or more,
                                    looked up by hash before the bucket search */
    uint32_t refined_splits;     /* bucket splits whose crowded bins were cut into finer bins */
    uint32_t pipelined;          /* 1: a host sort sent its input up in pieces, sorting as they landed */
    uint32_t region_overflow;    /* pipelined: 0, or 1 + the first level-1 bucket that outgrew the
                                    region reserved for it from the sample (level 1 was then redone) */
    uint32_t engine;             /* 1: level 2 (bucket splits, local sorts, copies) ran as one
                                    persistent launch over a device task queue; stage_ms[4] then
                                    holds all of level 2 and stage_ms[5] is 0 */
    uint32_t uniform_splits;     /* level-1 buckets of 8-16 byte records split into equal key ranges
                                    without a histogram pass (smooth keys) */
    uint32_t uniform_fallbacks;  /* such attempts in which a group outgrew its region: the bucket was
                                    then split by its histogram (same result) */
    uint32_t deep_splits;        /* records of 8-16 bytes: splits in the third split round or later */
} gbsort_stats;

/* OR into `method`: hash the records (gbsort_multiset_hash_device) before
 * and after the sort and return GBSORT_ERR_INTERNAL if the output is not a
 * permutation of the input -- the reference's self-check
 * (mpsort-mpi.c:148-159, 324-330).  The call then waits for the sort. */
#define GBSORT_VERIFY 0x100

/* Sort nmemb records of elsize bytes from d_in into d_out (device memory;
 * d_out may equal d_in).  `key` describes the radix; `method` a
 * gbsort_method, optionally with GBSORT_VERIFY.  nmemb is a full size_t
 * (radixsort.c:35): below 2^32 records every layout is taken; from 2^32 on
 * the records are first cut into at most 15 key ranges of under 2^32 each
 * by one stable partition pass (64-bit offsets, scratch of nmemb * elsize
 * bytes, host synchronisation between the stages), which needs a one-word
 * key at a 4-byte offset and 8-64 byte records (else
 * GBSORT_ERR_UNSUPPORTED) and at most about 2.2e10 records (else
 * GBSORT_ERR_BAD_ARG). */
GBSORT_API int gbsort_sort_device(const void *d_in, void *d_out, size_t nmemb, size_t elsize,
                       const gbsort_key_desc *key, int method, void *stream);

/* out[i] = source[index[i]] for nindex records of elsize bytes (device
 * memory; int64 indices): mpsort.take / mpsort.permute of one process
 * (reference mpsort/__init__.py:116-204, which needs two or three sorts
 * across MPI ranks to do the same).  Indices outside [0, nsource) are not
 * read: the call returns GBSORT_ERR_BAD_ARG (message: the first such
 * position).  Waits for the gather. */
GBSORT_API int gbsort_take_device(const void *d_source, size_t nsource, size_t elsize, const int64_t *d_index,
                                  size_t nindex, void *d_out, void *stream);

/* Order-independent 64-bit hash of the multiset of nmemb records of elsize
 * bytes (device memory): the sum, modulo 2^64, of a 64-bit mix of every
 * record's bytes, written to *d_hash (device memory) on `stream`.  Equal
 * multisets give equal hashes whatever their order; a changed, lost or
 * duplicated record changes the hash except with probability about 2^-64.
 * Replaces the reference's byte-sum checksum (mpsort-mpi.c:148-159). */
GBSORT_API int gbsort_multiset_hash_device(const void *d_records, size_t nmemb, size_t elsize,
                                           uint64_t *d_hash, void *stream);

/* gbsort_sort_device for host memory: in and out may be equal.  Blocks
 * until done. */
GBSORT_API int gbsort_sort_host(const void *in, void *out, size_t nmemb, size_t elsize,
                     const gbsort_key_desc *key, int method);

/* Sort host records in place by a host radix() callback producing rsize
 * bytes per record (compared as a little-endian unsigned integer, which is
 * what radixsort.c:47-194 does on a little-endian host).  The callback runs
 * on the host, once per record; the sort runs on the GPU.  Blocks. */
GBSORT_API int gbsort_sort_radix_host(void *base, size_t nmemb, size_t elsize,
                           void (*radix)(const void *ptr, void *radix, void *arg),
                           size_t rsize, void *arg);

/* Batched sort of nseg independent segments in one pipeline: segment i is
 * records [seg_offsets[i], seg_offsets[i+1]) of d_in (device memory; the
 * offsets array is in host memory, nseg + 1 entries, non-decreasing from 0,
 * below 2^32 - 1 records in all).  Each segment comes out sorted in place of
 * its range in d_out.  With a histogram-sort layout, segments above a size
 * threshold (default 2^22 records, or the segment tuning entry's) take the
 * whole-GPU sort one after the other and the rest share one level-2 pipeline
 * (the persistent engine, or split rounds, as tuned) fed with one task per
 * segment; otherwise each segment is sorted by the LSD path.  Waits. */
GBSORT_API int gbsort_sort_segments_device(const void *d_in, void *d_out, const uint64_t *seg_offsets,
                                size_t nseg, size_t elsize, const gbsort_key_desc *key,
                                int method, void *stream);

/* Join of two segments sorted by the same key (device memory): for every
 * key present in both, the pair of record indices (ia into a, ib into b).
 * Keys must be unique within each side.  *d_npairs (device memory) receives
 * the pair count; d_pairs_a / d_pairs_b need min(na, nb) entries. */
GBSORT_API int gbsort_merge_join_device(const void *d_a, size_t na, const void *d_b, size_t nb,
                             size_t elsize, const gbsort_key_desc *key, uint64_t *d_pairs_a,
                             uint64_t *d_pairs_b, uint64_t *d_npairs, void *stream);

/* Learned-model pieces, exposed for checking: one forward and backward pass
 * of the piecewise-linear CDF over sorted keys x (host arrays of s keys,
 * knots y of (1 << lbits) + 1 floats).  Outputs the mean squared loss, the
 * predictions (s floats) and the gradient (same size as y). */
GBSORT_API int gbsort_cdf_forward_backward(const uint64_t *x, uint32_t s, uint64_t kmin, uint64_t kmax,
                                int lbits, const float *y, float *loss, float *pred,
                                float *grad);

/* The gradient the model's training steps use, at knots y (host arrays as
 * above): T y - b, where the tridiagonal T and the vector b come from one
 * pass of the statistics kernel over the sorted keys (the loss is quadratic
 * in the knots, so this equals the backward pass's gradient; the training
 * runs all its steps from T and b without reading the keys again).
 * lbits <= 13.  For checking against the CPU oracle. */
GBSORT_API int gbsort_cdf_train_gradient(const uint64_t *x, uint32_t s, uint64_t kmin, uint64_t kmax, int lbits,
                                         const float *y, float *grad);

/* Learned-lookup probe (host arrays): trains the CDF model on the sample,
 * derives its splitters (nbuckets - 1 of them, returned in `splitters`) and
 * looks every key up twice -- with the model plus its search window, and
 * with a full binary search over the same splitters.  The two bucket arrays
 * must be identical; widest_window receives the widest window in buckets.
 * Used by tests. */
GBSORT_API int gbsort_debug_buckets(const uint64_t *sample, uint32_t s, int nbuckets, const uint64_t *keys,
                         uint32_t nkeys, uint32_t *bucket_search, uint32_t *bucket_learned,
                         uint64_t *splitters, uint32_t *widest_window);

/* What the trained model gains (host arrays): trains the model on the
 * sample for `epochs` gradient steps (0 = the initial fit of the empirical
 * CDF at the knots), looks every key up with the model and with the full
 * binary search over the same splitters, and reports the final training
 * loss, the splitters read by each lookup in total (reads[0] learned,
 * reads[1] full search) and the widest window.  Used by tests. */
GBSORT_API int gbsort_debug_model(const uint64_t *sample, uint32_t s, int nbuckets, int epochs,
                       const uint64_t *keys, uint32_t nkeys, uint32_t *bucket_search,
                       uint32_t *bucket_learned, float *loss, uint64_t *reads,
                       uint32_t *widest_window);

/* Plain splitter search alone (host arrays): the reference's bisection
 * (internal-parallel.h:128-248) for nsplit splitters over a sorted run of
 * s keys with targets C[i+1] = s*(i+1)/(nsplit+1).  Outputs the splitters
 * before single-key bucket shaping, the per-splitter CLT/CLE counts and the
 * number of rounds. */
GBSORT_API int gbsort_debug_bisect(const uint64_t *sorted, uint32_t s, int nsplit, uint64_t *splitters,
                        int64_t *clt, int64_t *cle, uint32_t *rounds);

/* Test of the bounded look-back wait of the LSD pass: one pass over n
 * pseudo-random keys in which tile `withhold_tile` (of n / 4096) never
 * publishes its counts, and every wait polls at most spin_limit times.
 * Returns GBSORT_ERR_INTERNAL (message: the wait gave up) when a wait ran
 * out, GBSORT_OK when none did (withhold_tile beyond the last tile).  The
 * wait's limit in sorts is about a second.  No counterpart in the
 * reference (its waits are MPI barriers). */
GBSORT_API int gbsort_debug_lookback(uint32_t n, uint32_t withhold_tile, uint32_t spin_limit);

/* Largest sort (nmemb * elsize bytes) gbsort_sort_device_noalloc accepts. */
#define GBSORT_NOALLOC_MAX_BYTES (8u << 20)

/* The histogram sort without any allocation, for callers that cannot call
 * cudaMalloc: code running inside a framework whose caching allocator owns
 * the device memory budget, code on a latency-critical path where an
 * allocation would synchronise the device, or code that must not run out
 * of memory half-way.  No counterpart in the reference, which always
 * allocates its temporaries.  Its scratch space is one fixed device array
 * of 22 MiB inside libgbsort; sorts larger than GBSORT_NOALLOC_MAX_BYTES
 * return GBSORT_ERR_BAD_ARG.  Same layouts as the histogram sort (one-word
 * key at a 4-byte offset, 8-64 byte records); the result is the same stable
 * order.
 * Set-up: the CUDA driver creates the array on a GPU when it loads the
 * library's device code there -- at context creation under eager module
 * loading, else (lazy loading, CUDA's default) at the first call of this
 * entry point on that GPU, which looks the array's address up with that GPU
 * current.  That first call may therefore allocate device memory (the array,
 * and the library's kernels if no other gbsort call has loaded them) and
 * must not run while any thread captures a stream in global mode; every
 * later call on that GPU allocates nothing.  The array then stays until the
 * process exits.
 * All calls share the array and leave their data in it, so calls whose work
 * overlaps on the GPU (different streams or unordered host threads) race.
 * Waits for its work on `stream` to finish before returning. */
GBSORT_API int gbsort_sort_device_noalloc(const void *d_in, void *d_out, size_t nmemb, size_t elsize,
                                          const gbsort_key_desc *key, void *stream);

GBSORT_API int gbsort_last_stats(gbsort_stats *out);
GBSORT_API const char *gbsort_status_string(int status);
GBSORT_API const char *gbsort_last_error(void);
GBSORT_API int gbsort_device_count(void);
/* Frees the cached device workspace and pinned staging of the current device. */
GBSORT_API int gbsort_release(void);
/* Version string of this library. */
GBSORT_API const char *gbsort_version(void);

/* ---- autotuner --------------------------------------------------------------
 * gbsort_autotune times every candidate configuration -- the LSD path, and
 * the plain and learned histogram sorts at level-1 bucket caps of 512, 1024,
 * 2048 and 4096, each with level 2 as split rounds and (records of 8-16
 * bytes) as the persistent engine -- on nmemb records of this layout (the
 * caller's device records, read only, or pseudo-random ones when d_records
 * is NULL), returns the fastest and stores it in the tuning table under
 * (elsize, key width, size class = bit length of nmemb).  Sorts with
 * GBSORT_AUTO use the table entry of the nearest size class within a factor
 * of 4.  The table can be set by hand, saved to and loaded from a text file
 * (one entry per line: elsize key_width size_class method max_buckets
 * sample_per_bucket ms level2; files without the level2 column load too).
 * No counterpart in the reference. */
/* How level 2 of the histogram sort (bucket splits and local sorts) runs:
 * as split rounds (one launch per round, then one for the local sorts) or as
 * one persistent launch over a device task queue (records of 8-16 bytes). */
enum { GBSORT_LEVEL2_DEFAULT = 0, GBSORT_LEVEL2_ROUNDS = 1, GBSORT_LEVEL2_ENGINE = 2 };

typedef struct gbsort_tuning {
    int32_t method;              /* GBSORT_HISTOGRAM_PLAIN, _LEARNED or GBSORT_LSD */
    uint32_t max_buckets;        /* level-1 bucket cap: a power of two, 2..4096 (0: default) */
    uint32_t sample_per_bucket;  /* sampled keys per level-1 bucket, 16..1024 (0: 128) */
    float ms;                    /* measured time of this configuration */
    uint32_t level2;             /* GBSORT_LEVEL2_* */
    uint32_t reserved[3];
} gbsort_tuning;
GBSORT_API int gbsort_autotune(size_t nmemb, size_t elsize, const gbsort_key_desc *key,
                    const void *d_records, gbsort_tuning *best);
GBSORT_API int gbsort_tuning_set(size_t nmemb, size_t elsize, const gbsort_key_desc *key,
                      const gbsort_tuning *t);
/* GBSORT_ERR_UNSUPPORTED when the table has no entry for this shape. */
GBSORT_API int gbsort_tuning_get(size_t nmemb, size_t elsize, const gbsort_key_desc *key,
                      gbsort_tuning *t);
GBSORT_API int gbsort_tuning_clear(void);
/* gbsort_autotune_segments times segmented sorts of this batch (the
 * caller's device records, read only, or pseudo-random ones) with level 2
 * as split rounds and as the engine and with segment-size thresholds of
 * 2^20, 2^22 and the largest segment (records of larger segments take the
 * whole-GPU sort), returns the fastest and stores it under the batch's size
 * class in a key space of its own (size_class + 128 in the tuning file, with
 * the threshold in reserved[0], the file's ninth column).  Segmented sorts
 * and segmented plans use that entry. */
GBSORT_API int gbsort_autotune_segments(const uint64_t *seg_offsets, size_t nseg, size_t elsize,
                             const gbsort_key_desc *key, const void *d_records, gbsort_tuning *best);
GBSORT_API int gbsort_tuning_get_segments(size_t nmemb, size_t elsize, const gbsort_key_desc *key,
                               gbsort_tuning *t);
GBSORT_API int gbsort_tuning_save(const char *path);
GBSORT_API int gbsort_tuning_load(const char *path);

/* ---- graph plans ----------------------------------------------------------
 * The whole device pipeline of one sort shape -- sample, splitter search or
 * model training, bucket count, scan, scatter, bucket splits and local
 * sorts -- captured once into a CUDA graph and replayed with one graph
 * launch and no host synchronisation.  No counterpart in the reference
 * (its sort is a synchronous call).
 *
 *   gbsort_plan_create   fixes nmemb, elsize, key and method (GBSORT_AUTO
 *                        resolves at the first capture); owns its scratch.
 *   gbsort_plan_sort     enqueues the sort of d_in into d_out on `stream`
 *                        (NULL: the plan's own stream) and returns at once;
 *                        the graph is captured on first use and again when
 *                        the buffers change.  One launch per plan at a time:
 *                        a second call first waits for the previous one.
 *   gbsort_plan_wait     waits for the launch, then returns its status (the
 *                        device error word) and fills gbsort_last_stats
 *                        (without stage times).
 *   gbsort_plan_destroy  waits and frees everything. */
typedef struct gbsort_plan gbsort_plan;
GBSORT_API int gbsort_plan_create(gbsort_plan **plan, size_t nmemb, size_t elsize,
                       const gbsort_key_desc *key, int method);
/* A plan for gbsort_sort_segments_device of a fixed batch (the offsets are
 * copied; method GBSORT_AUTO, _HISTOGRAM_PLAIN or _LEARNED for the segments
 * sorted on their own); needs a histogram-sort layout. */
GBSORT_API int gbsort_plan_create_segments(gbsort_plan **plan, const uint64_t *seg_offsets, size_t nseg,
                                size_t elsize, const gbsort_key_desc *key, int method);
GBSORT_API int gbsort_plan_sort(gbsort_plan *plan, const void *d_in, void *d_out, void *stream);
GBSORT_API int gbsort_plan_wait(gbsort_plan *plan);
GBSORT_API int gbsort_plan_destroy(gbsort_plan *plan);

#ifdef __cplusplus
}
#endif

#endif /* GBSORT_H */
