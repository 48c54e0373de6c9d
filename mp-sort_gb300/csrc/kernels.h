// kernels.h -- host-side launch wrappers for the gbsort kernels.
//
// Every wrapper enqueues work on `stream` and returns the launch's
// cudaError_t; none of them synchronises.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "../../include/gbsort_key.h"

namespace gb {

// Count of kernels this library has enqueued (every wrapper below adds the
// launches it made); read before and after a sort for its launch count.
void note_launches(int k);
unsigned long long launch_count();

// Streaming multiprocessors of the current device.
int num_sms();

// ---- verify.cu: multiset hash, and the first partition of huge sorts ------
// *out = sum over the n records of a 64-bit mix of each record's bytes
// (order-independent; equal multisets of records give equal sums).
cudaError_t multiset_hash(const void* rec, uint64_t n, uint32_t elsize, unsigned long long* out, cudaStream_t st);
// s keys at evenly spaced records i * n / s of n (64-bit) records.
cudaError_t sample_keys64(const uint8_t* rec, uint64_t n, uint32_t elsize, gbsort_key_word key, uint32_t s,
                          uint64_t* out, cudaStream_t st);
// Chunks of the partition kernels; counts are [part][chunk].
int part_grid();
// Records per (part, chunk) for nsplit <= 14 sorted splitters (part =
// #{splitters <= key}).
cudaError_t part_count(const uint8_t* rec, uint64_t n, uint32_t elsize, gbsort_key_word key, const uint64_t* S,
                       int nsplit, uint32_t* counts, cudaStream_t st);
// Stable scatter of every record to offsets[part][chunk] + its rank among
// its chunk's records of that part.
cudaError_t part_scatter(const uint8_t* rec, uint8_t* out, uint64_t n, uint32_t elsize, gbsort_key_word key,
                         const uint64_t* S, int nsplit, const unsigned long long* offsets, uint32_t* err,
                         cudaStream_t st);

// ---- take.cu --------------------------------------------------------------
// out[i] = src[index[i]] for nidx records of elsize bytes; *bad receives the
// first position whose index lies outside [0, nsrc), plus one (0: none).
cudaError_t take_records(const void* src, uint64_t nsrc, uint32_t elsize, const int64_t* index, uint64_t nidx,
                         void* out, unsigned long long* bad, cudaStream_t st);

// ---- scan.cu --------------------------------------------------------------
// Exclusive prefix sum of n uint32 values (n <= 2^24); `tmp` needs
// scan_tmp_words(n) words.  out may alias in.
size_t scan_tmp_words(size_t n);
cudaError_t exclusive_scan_u32(const uint32_t* in, uint32_t* out, size_t n, uint32_t* tmp,
                               cudaStream_t stream);

// ---- lsd.cu: the generic path (any key width, any record size) -------------
// Key words of every record into word-major arrays keys[w * n + i], and the
// identity permutation into idx (if not null).
cudaError_t extract_keys(const void* rec, uint32_t n, uint32_t elsize, const gbsort_key_desc& key,
                         uint64_t* keys, uint32_t* idx, cudaStream_t stream);
// rsize little-endian radix bytes per record (from a host radix() callback)
// into nwords = ceil(rsize / 8) key words.
cudaError_t radix_bytes_to_keys(const uint8_t* radix, uint32_t n, uint32_t rsize, uint64_t* keys,
                                uint32_t* idx, cudaStream_t stream);
// 256-bin histograms of all 8 * nwords digits in one read ([digit][256]).
cudaError_t lsd_digit_histograms(const uint64_t* keys, uint32_t n, int nwords, uint32_t* hist,
                                 cudaStream_t stream);
// Exclusive scans of those histograms: the first output slot of every bin.
cudaError_t lsd_digit_starts(const uint32_t* hist, int nwords, uint32_t* starts, cudaStream_t stream);
// Tiles of one LSD pass over n keys (status words needed: 256 per tile).
uint32_t lsd_tiles(uint32_t n);
// Record-carrying LSD passes (records of 8-32 bytes in 4-byte words, key
// words at 4-byte offsets, buffers aligned to the record's vector size):
// the digit histograms of every key word read from the records, and one
// stable pass that moves whole records by one digit.  Tiles of 2048 or
// 4096 records; status holds lsd_record_tiles(n, elsize) * 256 words.
bool lsd_records_supported(uint32_t elsize, const void* in, const void* out, const gbsort_key_desc& key);
uint32_t lsd_record_tiles(uint32_t n, uint32_t elsize);
cudaError_t lsd_record_histograms(const void* in, uint32_t n, uint32_t elsize, const gbsort_key_desc& key,
                                  uint32_t* hist, cudaStream_t stream);
cudaError_t lsd_record_pass(const void* in, void* out, uint32_t n, uint32_t elsize, const gbsort_key_desc& key,
                            int word, int shift, const uint32_t* starts, unsigned long long* status,
                            uint32_t* ticket, uint32_t* err, cudaStream_t stream);
// One one-sweep LSD pass on digit (word, shift): stable scatter of all key
// words (and idx, if not null) with offsets from starts (256 entries of this
// digit) plus a decoupled look-back over the tiles; status and ticket are
// scratch (zeroed here); err receives DEV_ERR_TIMEOUT if a wait gave up.
// spin_limit: polls of one look-back wait before it gives up (0: about a
// second's worth); withhold_tile: a tile that never publishes its counts
// (tests of the bounded wait only; ~0u otherwise).
cudaError_t lsd_onesweep(const uint64_t* keys_in, const uint32_t* idx_in, uint64_t* keys_out, uint32_t* idx_out,
                         uint32_t n, int nwords, int word, int shift, const uint32_t* starts,
                         unsigned long long* status, uint32_t* ticket, uint32_t* err, cudaStream_t stream,
                         uint32_t spin_limit = 0, uint32_t withhold_tile = ~0u);
// Pseudo-random contents for the first nbytes / 4 words of p (synthetic
// inputs of the autotuner).
cudaError_t fill_hash(void* p, size_t nbytes, uint64_t seed, cudaStream_t stream);
// out[i] = in[idx[i]] for records of elsize bytes.
cudaError_t gather_records(const void* in, void* out, const uint32_t* idx, uint32_t n,
                           uint32_t elsize, cudaStream_t stream);

// ---- hsort.cu: the histogram sort ----------------------------------------
// Device statistics slots filled by the histogram sort.
enum StatSlot : int {
  STAT_LOCAL = 0,        // shared-memory local sorts
  STAT_SPLIT = 1,        // bucket splits
  STAT_COPY = 2,         // single-key copy tasks
  STAT_PUSHED = 3,       // sub-buckets re-split in a further round
  STAT_BIGBIN = 4,       // extra local MSD passes on clustered bins
  STAT_WINDOW_MISS = 5,  // learned lookups whose window missed (full search ran)
  STAT_MAX_BUCKET = 6,   // largest level-1 bucket
  STAT_REFINED = 7,      // splits whose crowded bins were cut finer
  STAT_DEEP = 8,         // splits of a third round or later (with areas: A to the output and back)
  STAT_SLOTS = 9
};

enum Lookup : int { LOOKUP_PLAIN = 0, LOOKUP_LEARNED = 1 };

struct SortTask {        // one bucket or sub-bucket of the level-2 task engine
  uint32_t start;        // first record in the destination buffers (the other scratch buffer, the output)
  uint32_t count;        // records
  uint64_t lo, hi;       // key range [lo, hi] of the records
  uint32_t from;         // first record in the source buffer: start, except for the level-1
                         // buckets of a scatter into reserved (gapped) bucket regions
  uint32_t flags;        // TASK_* below
};
enum TaskFlags : uint32_t {
  TASK_SRC_B = 1,    // the records are in scratch B (else scratch A)
  TASK_COPY = 2,     // one key: copied, not sorted
  TASK_SRC_OUT = 4,  // the records are in the output buffer, at their final positions
  TASK_L1 = 8,       // a level-1 bucket (round 0 of the split rounds)
};
__host__ __device__ inline SortTask make_task(uint32_t start, uint32_t count, uint64_t lo, uint64_t hi, bool in_b,
                                              bool copy) {
  return SortTask{start, count, lo, hi, start, (in_b ? (uint32_t)TASK_SRC_B : 0u) | (copy ? (uint32_t)TASK_COPY : 0u)};
}
// A task whose records lie at `from` of the buffer `flags` names, bound for
// `start` of the next buffer (or the output).
__host__ __device__ inline SortTask make_task_at(uint32_t start, uint32_t from, uint32_t count, uint64_t lo,
                                                 uint64_t hi, uint32_t flags) {
  return SortTask{start, count, lo, hi, from, flags};
}

// Keys heavy enough to own a single-key level-1 bucket worth three
// splitters or more: a run of equal splitters k becomes [k, k+1) followed by
// copies of k + 1 (finalize_splitters), so bucket i + 1 holds exactly the key
// S[i] when S[i] + 1 == S[i + 1] == S[i + 2].  The level-1 kernels probe
// this open-addressing table before the bucket lookup: a learned window
// spans a heavy key's whole run, and a binary search every heavy record.
constexpr int kHeavyLog2 = 11;
constexpr int kHeavySlots = 1 << kHeavyLog2;
constexpr int kHeavyProbes = 8;  // longest probe sequence an insert may take
struct HeavySlot {
  uint64_t key;
  uint32_t bucket1;  // bucket + 1; 0 marks an empty slot
  uint32_t weight;   // (splitters the key spans) << 14 | bucket: larger is heavier
};
struct HeavyTable {
  uint32_t n;       // keys held
  uint32_t probes;  // longest probe sequence of an insert (0: table empty)
  uint32_t pad[2];
  HeavySlot slot[kHeavySlots];
};

struct HsortParams {
  const uint8_t* in;
  uint8_t* out;
  uint8_t* bufA;
  uint8_t* bufB;
  uint32_t n;
  uint32_t elsize;
  gbsort_key_word key;
  uint32_t a_cap;      // records scratch A holds (n, or more for reserved bucket regions)
  uint32_t chunks;     // count chunks of the input (0: hsort_grid(n))
  const HeavyTable* heavy;  // heavy keys of the level-1 splitters (null: none)
  // level-1 bucket of every record: written by the count, read by the
  // scatter (n entries; the scatter's scratch B is free during level 1)
  uint16_t* bkt;
  // Uniform splits (records of 8-16 bytes, split rounds): a level-1 bucket
  // may be cut into equal key ranges and scattered into regions of scratch B
  // sized for them, without the histogram pass.  uniform: device words
  // [tried, failed] (null: never); gate_words: the model's widest window and
  // the heavy-key count, both zero for keys this suits.
  uint32_t* uniform;
  const uint32_t* gate_widest;
  const uint32_t* gate_heavy;
  // 1: the split rounds of records of 8-16 bytes give each level-1 bucket an
  // area of scratch B (split_area) and ping-pong later rounds through A and
  // the output; scratch B then holds split_area(n) records
  uint32_t areas;
};

// Scratch B position of a level-1 bucket's area in the split rounds of
// records of 8-16 bytes: bucket [start, start + m) owns B records
// [split_area(start), split_area(start + m)), a quarter more than it holds,
// so a split may give each group a region with room to spare.
__host__ __device__ inline uint32_t split_area(uint32_t start) { return (uint32_t)((uint64_t)start + (start >> 2)); }
// Largest n whose areas fit 32-bit record offsets.
constexpr uint32_t kSplitAreaMaxN = 3435973836u;  // 0.8 * 2^32

bool hsort_supported(uint32_t elsize);
int hsort_grid(uint32_t n);
cudaError_t sample_keys(const uint8_t* rec, uint32_t n, uint32_t elsize, gbsort_key_word key,
                        uint32_t s, uint64_t* out, cudaStream_t stream);
// Plain splitter search: for every splitter, the reference's bisection over
// the sorted sample (internal-parallel.h piter_* with CLT < C <= CLE), then
// equal runs turned into single-key buckets.
cudaError_t plain_splitters(const uint64_t* sorted_sample, uint32_t s, int nsplit,
                            uint64_t* splitters, uint32_t* iters, int64_t* clt, int64_t* cle,
                            cudaStream_t stream);
// The heavy-key table of sorted splitters S (one CTA); *held receives the
// number of keys it holds.
cudaError_t heavy_table(const uint64_t* splitters, int nsplit, HeavyTable* table, uint32_t* held,
                        cudaStream_t stream);
cudaError_t finalize_splitters(uint64_t* splitters, int nsplit, cudaStream_t stream, const uint32_t* only_if = nullptr);
// Level-1 bucket counts per chunk ([nbuckets][grid]) and the stable scatter.
// `model` points to a host copy of the ModelDev (cdf.cuh) for the learned
// lookup, else null.  `stats` is the device statistics array (Stat indices).
// The input is cut into p.chunks count chunks (hsort_grid(n) when 0);
// l1_count counts chunks [c0, c1) (c1 < 0: all) into counts[bucket][chunk].
cudaError_t l1_count(const HsortParams& p, int lookup, const uint64_t* splitters, int nbuckets,
                     const void* model, uint32_t* counts, uint32_t* stats, cudaStream_t stream, int c0 = 0,
                     int c1 = -1);
// First record of chunk c of `chunks` (n for c >= chunks).
uint32_t hsort_chunk_begin(uint32_t n, int c, int chunks);
// Reserved bucket regions from the sorted sample: a bucket holding c of the
// s sampled keys gets cap[b] = (c + sigmas sqrt(c + 1) + spare) * n / s
// records (at most n) plus pad; the caller scans cap into starts.
cudaError_t bucket_caps(const uint64_t* sorted_sample, uint32_t s, const uint64_t* splitters, int nbuckets,
                        uint32_t n, double sigmas, double spare, uint32_t pad, uint32_t* cap, cudaStream_t stream);
// Scatter offsets of chunks [c0, c1) into reserved regions: counts of those
// chunks become region start + the bucket's running total (kept in total[]);
// if a bucket outgrows its region, overflow[0] becomes the first such bucket
// + 1 and overflow[1], [2] its capacity and count.
cudaError_t region_offsets(uint32_t* counts, int chunks, int nbuckets, const uint32_t* region, const uint32_t* cap,
                           uint32_t* total, int c0, int c1, uint32_t* overflow, cudaStream_t stream);
// Scatter of chunks [c0, c1) (c1 < 0: all) to offsets[bucket][chunk], each
// record to the bucket l1_count wrote for it in p.bkt; does nothing if
// *skip_if is set (a region overflow).
cudaError_t l1_scatter(const HsortParams& p, int nbuckets, const uint32_t* offsets, uint32_t* stats,
                       cudaStream_t stream, int c0 = 0, int c1 = -1, const uint32_t* skip_if = nullptr);
// Level-2 task lists (device memory).  A split round consumes split_in and
// appends to split_out and local; build_tasks appends to split_out and local.
struct TaskListsHost {
  const SortTask* split_in;
  const uint32_t* nsplit_in;
  SortTask* split_out;
  uint32_t* nsplit_out;
  SortTask* local;
  uint32_t* nlocal;
  uint32_t cap_split;
  uint32_t cap_local;
};
// Tasks of level-1 buckets [b0, b1) (b1 < 0: all), largest split first.
cudaError_t build_tasks(const uint32_t* offsets, int grid, const uint64_t* splitters, int nbuckets,
                        uint32_t n, const TaskListsHost& lists, uint32_t* err, uint32_t* stats,
                        cudaStream_t stream, int b0 = 0, int b1 = -1);
// Tasks of buckets [b0, b1) that still lie in their reserved regions: the
// bucket at region[b], `total[b]` records, going to out_start[b]; every one
// goes to the split list (single-key buckets in copy pieces).
cudaError_t build_region_tasks(const uint32_t* region, const uint32_t* total, const uint32_t* out_start,
                               const uint64_t* splitters, int nbuckets, const TaskListsHost& lists, uint32_t* err,
                               uint32_t* stats, cudaStream_t stream, int b0, int b1);
// err gets DEV_ERR_LEVELS unless *count is zero.
cudaError_t require_zero(const uint32_t* count, uint32_t* err, cudaStream_t stream);
cudaError_t run_split_round(const HsortParams& p, const TaskListsHost& lists, uint32_t* work_counter,
                            uint32_t* stats, uint32_t* err, cudaStream_t stream);
cudaError_t run_local(const HsortParams& p, const SortTask* tasks, const uint32_t* ntasks, uint32_t cap,
                      uint32_t* work_counter, uint32_t* stats, cudaStream_t stream);
// The persistent level-2 engine (records of 8, 12 or 16 bytes): the tasks of
// seed.split_in (count *seed.nsplit_in, largest first) then seed.local go
// into the device queue (qtask / qready of qcap entries, qctl 3 words), and
// one launch runs every split, local sort and copy, including the ones the
// splits produce.  Tasks must lie at their final positions (no reserved
// regions).  err: task overflow or a wait that ran out.
bool engine_supported(uint32_t elsize);
// qctl: tail, head and pending, kEngineCtlStride words apart (one cache line each).
constexpr uint32_t kEngineCtlStride = 32;
cudaError_t run_engine(const HsortParams& p, const TaskListsHost& seed, SortTask* qtask, uint32_t* qready,
                       uint32_t* qctl, uint32_t qcap, uint32_t* stats, uint32_t* err, cudaStream_t stream);

}  // namespace gb
