// gbsort.cu -- host side of libgbsort: device workspace, the sort pipelines
// and every entry point of include/gbsort.h and include/mpsort.h.
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/gbsort.h"
#include "../../include/mpsort.h"
#include "cdf.cuh"
#include "cdf_api.h"
#include "kernels.h"

namespace gb {
cudaError_t join_count(const uint8_t* a, uint32_t na, const uint8_t* b, uint32_t nb, uint32_t elsize,
                       gbsort_key_word key, uint32_t* counts, int grid, cudaStream_t st);
cudaError_t join_write(const uint8_t* a, uint32_t na, const uint8_t* b, uint32_t nb, uint32_t elsize,
                       gbsort_key_word key, const uint32_t* offsets, int grid, uint64_t* pa, uint64_t* pb,
                       uint64_t* npairs, cudaStream_t st);
int join_grid(uint32_t na);
cudaError_t segment_ranges(const uint8_t* rec, uint32_t elsize, gbsort_key_word key, const uint64_t* offsets,
                           uint32_t nseg, uint64_t skip_above, SortTask* tasks, uint32_t* ntasks, uint32_t cap,
                           uint32_t* err, cudaStream_t st);
cudaError_t probe_buckets(const uint64_t* keys, uint32_t nkeys, const uint64_t* S, const void* model,
                          uint32_t* learned, uint32_t* search, uint32_t* misses, unsigned long long* reads,
                          cudaStream_t st);
}  // namespace gb

namespace {

using namespace gb;

thread_local char g_err[512] = "";
thread_local int g_mpsort_status = GBSORT_OK;
thread_local gbsort_stats g_stats = {};
int g_mpi_options = 0;
std::mutex g_opt_mu;

void set_err(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

#define GB_CUDA(call)                                                                  \
  do {                                                                                 \
    cudaError_t e_ = (call);                                                           \
    if (e_ != cudaSuccess) {                                                           \
      set_err("%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_));      \
      return e_ == cudaErrorMemoryAllocation ? GBSORT_ERR_OOM : GBSORT_ERR_CUDA;       \
    }                                                                                  \
  } while (0)

// A grow-only device allocation.
struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
  cudaError_t ensure(size_t bytes) {
    if (bytes <= cap) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    size_t want = bytes + bytes / 16;
    cudaError_t e = cudaMalloc(&p, want);
    if (e != cudaSuccess) {
      cudaGetLastError();
      e = cudaMalloc(&p, bytes);
      if (e != cudaSuccess) {
        cudaGetLastError();
        p = nullptr;
        return e;
      }
      want = bytes;
    }
    cap = want;
    return cudaSuccess;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
  template <typename T>
  T* as() const {
    return reinterpret_cast<T*>(p);
  }
};

// Bump allocator over one device buffer for the small arrays of a run.
struct Bump {
  uint8_t* base;
  size_t off = 0;
  template <typename T>
  T* take(size_t count) {
    off = (off + 255) & ~(size_t)255;
    T* r = reinterpret_cast<T*>(base + off);
    off += sizeof(T) * count;
    return r;
  }
};

// Device counters of a histogram-sort run (one 64-word array), in order.
enum CounterSlot : int {
  CNT_ERR = STAT_SLOTS,  // kernels given the statistics find the error word next to them
  CNT_ITERS = 21,        // bisection rounds
  CNT_WIDEST = 22,       // widest learned window
  CNT_LOSS = 23,         // final training loss (float)
  CNT_L2 = 24,           // level-2 task counters: nsplit[2], nlocal, work
  CNT_FALLBACK = 28,     // the learned splitters were rejected
  CNT_HEAVY = 30,        // keys in the heavy-key table
  CNT_UNIFORM = 36,      // uniform bucket splits: tried, then failed (2 words)
  CNT_OVERFLOW = 31,     // a bucket outgrew its reserved region (pipelined host sort): bucket + 1,
                         // then its capacity and count (3 words)
  CNT_ENGINE = 48,       // the level-2 engine's queue: tail, head, pending, kEngineCtlStride apart
  CNT_WORDS = 128
};

// Bytes past the records of each scratch buffer: the staged local sorts copy
// a task's byte range rounded out to 16 bytes.
constexpr size_t kScratchSlack = 256;
constexpr int kMaxPieces = 16;  // host -> device pieces of a pipelined host sort
// Reserved bucket regions of the pipelined host sort.  A bucket holding c
// of the s sampled keys gets (c + 5 sqrt(c + 1) + 10) * n / s records plus
// 256: its count is c * n / s give or take sqrt(c + 1) * n / s, so the
// region covers five standard deviations plus ten sampled keys' worth --
// which matters for buckets the sample barely saw (after a heavy key's run
// of equal splitters, the next bucket may hold no sampled key at all).  By
// Cauchy-Schwarz, sum_b sqrt(c_b + 1) <= sqrt(nb (s + nb)), which bounds the
// total reserved.
constexpr double kRegionSigmas = 5.0;
constexpr double kRegionSpare = 10.0;
constexpr uint32_t kRegionPad = 256;
constexpr int kMaxWaves = 16;   // level-2 waves (and device -> host pieces)

struct HostCounters {  // pinned: the device counters of the last run are copied here
  uint32_t c[CNT_WORDS];
  uint32_t starts[kMaxWaves + 1];  // first output record of each wave
};

// A host sort whose copies overlap the device work: the input goes up in
// pieces aligned to the count kernel's chunks (each piece counted as it
// lands), and level 2 runs in waves of level-1 buckets, each wave's output
// range going down while the next wave sorts.
struct HostPipe {
  const uint8_t* h_in;
  uint8_t* h_out;
  int pieces;
  int waves;
};

struct Context {
  int device = -1;
  cudaStream_t stream = nullptr;
  DevBuf A, B;             // record scratch
  DevBuf hin, hout;        // staging of the host entry points
  DevBuf keysA, keysB;     // generic path key words
  DevBuf idxA, idxB;       // generic path permutation
  DevBuf small;            // splitters, counts, tasks, model, counters
  DevBuf radix;            // host radix bytes (callback path)
  DevBuf part;             // first partition of sorts of 2^32 records or more
  DevBuf seg;              // segment offsets and error words of a segmented sort
  DevBuf vh;               // multiset hashes of a self-checked sort
  HostCounters* hc = nullptr;
  cudaEvent_t ev[8] = {};  // stage boundaries of the histogram sort
  cudaStream_t cstream = nullptr;                // copies of a pipelined host sort
  cudaEvent_t pev[kMaxPieces] = {}, wev[kMaxWaves] = {}, sev = nullptr, dev_done = nullptr;
  std::mutex mu;
  // shape of the last enqueued histogram sort (for hsort_collect)
  uint32_t run_nbuckets = 0, run_sample = 0, run_lsd_passes = 0;
  bool run_learned = false, run_timing = false, run_pipelined = false, run_engine = false;
};

std::mutex g_ctx_mu;
Context* g_ctx[64] = {};

// blocking: the library's own streams of a device (the `NULL` stream of the
// device entry points) order after work on the legacy default stream, so a
// caller's earlier kernels there (filling the input, say) finish first; a
// graph plan's capture streams do not.
int ctx_init(Context& c, int dev, bool blocking) {
  c.device = dev;
  const unsigned flags = blocking ? cudaStreamDefault : cudaStreamNonBlocking;
  GB_CUDA(cudaStreamCreateWithFlags(&c.stream, flags));
  GB_CUDA(cudaStreamCreateWithFlags(&c.cstream, flags));
  GB_CUDA(cudaMallocHost(&c.hc, sizeof(HostCounters)));
  for (cudaEvent_t& e : c.ev) GB_CUDA(cudaEventCreate(&e));
  for (cudaEvent_t& e : c.pev) GB_CUDA(cudaEventCreate(&e));
  for (cudaEvent_t& e : c.wev) GB_CUDA(cudaEventCreate(&e));
  GB_CUDA(cudaEventCreate(&c.sev));
  GB_CUDA(cudaEventCreate(&c.dev_done));
  return GBSORT_OK;
}

void ctx_destroy(Context& c) {
  if (c.stream) cudaStreamSynchronize(c.stream);
  DevBuf* bufs[] = {&c.A, &c.B, &c.hin, &c.hout, &c.keysA, &c.keysB, &c.idxA, &c.idxB, &c.small, &c.radix, &c.part, &c.vh, &c.seg};
  for (DevBuf* b : bufs) b->release();
  if (c.cstream) cudaStreamSynchronize(c.cstream);
  for (cudaEvent_t& e : c.ev)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t& e : c.pev)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t& e : c.wev)
    if (e) cudaEventDestroy(e);
  if (c.sev) cudaEventDestroy(c.sev);
  if (c.dev_done) cudaEventDestroy(c.dev_done);
  if (c.hc) cudaFreeHost(c.hc);
  if (c.stream) cudaStreamDestroy(c.stream);
  if (c.cstream) cudaStreamDestroy(c.cstream);
  c.cstream = nullptr;
  c.hc = nullptr;
  c.stream = nullptr;
}

int get_ctx(Context** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_err("no CUDA device: %s", cudaGetErrorString(e));
    return GBSORT_ERR_NO_DEVICE;
  }
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
    cudaGetLastError();
    set_err("no CUDA device visible");
    return GBSORT_ERR_NO_DEVICE;
  }
  if (dev < 0 || dev >= 64) return GBSORT_ERR_BAD_ARG;
  std::lock_guard<std::mutex> lk(g_ctx_mu);
  if (!g_ctx[dev]) {
    Context* c = new Context();
    int rc = ctx_init(*c, dev, true);
    if (rc) {
      delete c;
      return rc;
    }
    g_ctx[dev] = c;
  }
  *out = g_ctx[dev];
  return GBSORT_OK;
}

bool key_ok(const gbsort_key_desc* key, size_t elsize) {
  if (!key || key->nwords < 1 || key->nwords > GBSORT_MAX_KEY_WORDS) return false;
  for (uint32_t w = 0; w < key->nwords; ++w) {
    const gbsort_key_word& k = key->word[w];
    if (k.width != 4 && k.width != 8) return false;
    if (k.is_signed > 1) return false;
    if ((size_t)k.offset + k.width > elsize) return false;
  }
  return true;
}

uint32_t pow2_ceil(uint64_t x) {
  uint32_t p = 1;
  while (p < x && p < (1u << 30)) p <<= 1;
  return p;
}

// ------------------------------------------------------------ LSD path --
// Scratch of lsd_sort_keys for n keys of nwords words.
size_t lsd_scratch_bytes(uint32_t n, int nwords) {
  return (size_t)2 * 8 * 256 * 4 * nwords + (size_t)lsd_tiles(n) * 256 * 8 + 4096;
}

// The LSD digits (word, shift) a sort runs, least significant first: all
// of them, or (with the histograms on the host) those whose histogram does
// not put every key in one bin.
void lsd_pass_list(int nwords, uint32_t n, const std::vector<uint32_t>* h, std::vector<int>& pass_word,
                   std::vector<int>& pass_shift) {
  for (int w = 0; w < nwords; ++w)
    for (int d = 0; d < 8; ++d) {
      bool trivial = false;
      if (h)
        for (int b = 0; b < 256; ++b)
          if ((*h)[((size_t)w * 8 + d) * 256 + b] == n) trivial = true;
      if (!trivial) {
        pass_word.push_back(w);
        pass_shift.push_back(8 * d);
      }
    }
}

// Sorts key words (and idx) in place in keys / idx, ping-ponging through
// keys2 / idx2, one one-sweep pass per 8-bit digit.  With skip_trivial the
// digit histograms are read back (one synchronisation) and digits whose
// histogram puts every key in one bin are skipped.  Returns the number of
// passes run (the result is in the first buffer either way).
int lsd_sort_keys(Bump& bump, uint64_t* keys, uint64_t* keys2, uint32_t* idx, uint32_t* idx2, uint32_t n,
                  int nwords, bool skip_trivial, int* passes_out, uint32_t* err, cudaStream_t st) {
  uint32_t* hist = bump.take<uint32_t>((size_t)8 * 256 * nwords);
  uint32_t* starts = bump.take<uint32_t>((size_t)8 * 256 * nwords);
  unsigned long long* status = bump.take<unsigned long long>((size_t)lsd_tiles(n) * 256 + 1);
  uint32_t* ticket = reinterpret_cast<uint32_t*>(status + (size_t)lsd_tiles(n) * 256);  // cleared with the status
  GB_CUDA(lsd_digit_histograms(keys, n, nwords, hist, st));
  GB_CUDA(lsd_digit_starts(hist, nwords, starts, st));
  std::vector<int> pass_word, pass_shift;
  std::vector<uint32_t> h;
  if (skip_trivial) {
    h.resize((size_t)8 * 256 * nwords);
    GB_CUDA(cudaMemcpyAsync(h.data(), hist, h.size() * 4, cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
  }
  lsd_pass_list(nwords, n, skip_trivial ? &h : nullptr, pass_word, pass_shift);
  uint64_t* kin = keys;
  uint64_t* kout = keys2;
  uint32_t* iin = idx;
  uint32_t* iout = idx2;
  for (size_t p = 0; p < pass_word.size(); ++p) {
    const uint32_t* st_d = starts + ((size_t)pass_word[p] * 8 + pass_shift[p] / 8) * 256;
    GB_CUDA(lsd_onesweep(kin, iin, kout, iout, n, nwords, pass_word[p], pass_shift[p], st_d, status, ticket, err,
                         st));
    std::swap(kin, kout);
    std::swap(iin, iout);
  }
  if (kin != keys) {  // odd number of passes: move the result home
    GB_CUDA(cudaMemcpyAsync(keys, kin, sizeof(uint64_t) * n * nwords, cudaMemcpyDeviceToDevice, st));
    if (idx) GB_CUDA(cudaMemcpyAsync(idx, iin, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, st));
  }
  if (passes_out) *passes_out = (int)pass_word.size();
  return GBSORT_OK;
}

// LSD over records of 8-32 bytes that carry themselves through the digit
// passes (lsd_record_pass), ping-ponging through scratch A / B so that the
// last pass writes d_out.
int lsd_records_enqueue(Context& c, const void* d_in, void* d_out, uint32_t n, uint32_t elsize,
                        const gbsort_key_desc* key, bool skip_trivial, cudaStream_t st) {
  const int nwords = (int)key->nwords;
  const size_t bytes = (size_t)n * elsize;
  GB_CUDA(c.A.ensure(bytes + kScratchSlack));
  GB_CUDA(c.B.ensure(bytes + kScratchSlack));
  GB_CUDA(c.small.ensure((size_t)2 * 8 * 256 * 4 * nwords + (size_t)lsd_record_tiles(n, elsize) * 256 * 8 +
                         CNT_WORDS * 4 + 8192));
  Bump bump{c.small.as<uint8_t>()};
  uint32_t* counters = bump.take<uint32_t>(CNT_WORDS);
  uint32_t* err = counters + CNT_ERR;
  uint32_t* hist = bump.take<uint32_t>((size_t)8 * 256 * nwords);
  uint32_t* starts = bump.take<uint32_t>((size_t)8 * 256 * nwords);
  unsigned long long* status = bump.take<unsigned long long>((size_t)lsd_record_tiles(n, elsize) * 256);
  uint32_t* ticket = bump.take<uint32_t>(1);
  GB_CUDA(cudaMemsetAsync(counters, 0, CNT_WORDS * sizeof(uint32_t), st));
  GB_CUDA(lsd_record_histograms(d_in, n, elsize, *key, hist, st));
  GB_CUDA(lsd_digit_starts(hist, nwords, starts, st));
  std::vector<uint32_t> h;
  if (skip_trivial) {
    h.resize((size_t)8 * 256 * nwords);
    GB_CUDA(cudaMemcpyAsync(h.data(), hist, h.size() * 4, cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
  }
  std::vector<int> pass_word, pass_shift;
  lsd_pass_list(nwords, n, skip_trivial ? &h : nullptr, pass_word, pass_shift);
  const size_t P = pass_word.size();
  const void* src = d_in;
  for (size_t p = 0; p < P; ++p) {
    void* dst = p + 1 == P ? d_out : (p % 2 == 0 ? c.A.p : c.B.p);
    if (dst == src) dst = c.A.p;  // one pass, in place: through A, then home
    const uint32_t* st_d = starts + ((size_t)pass_word[p] * 8 + pass_shift[p] / 8) * 256;
    GB_CUDA(lsd_record_pass(src, dst, n, elsize, *key, pass_word[p], pass_shift[p], st_d, status, ticket, err,
                            st));
    src = dst;
  }
  if (src != d_out) GB_CUDA(cudaMemcpyAsync(d_out, src, bytes, cudaMemcpyDeviceToDevice, st));
  GB_CUDA(cudaMemcpyAsync(c.hc->c, counters, CNT_WORDS * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  c.run_lsd_passes = (uint32_t)P;
  return GBSORT_OK;
}

// Generic path over device records: keys from the descriptor (or from radix
// bytes already on the device), LSD, then one gather into d_out -- or, with
// GBSORT_LSD_RECORDS=1 and records of 8-32 bytes, passes that carry the
// records themselves (fewer bytes, more time on this GPU: opt-in).  With
// skip_trivial, constant digits are found on the host (one synchronisation)
// and skipped; without, nothing waits for the host (graph capture).
int lsd_enqueue(Context& c, const void* d_in, void* d_out, uint32_t n, uint32_t elsize, const gbsort_key_desc* key,
                const uint8_t* d_radix, uint32_t rsize, bool skip_trivial, cudaStream_t st) {
  static const bool records = [] {
    const char* e = getenv("GBSORT_LSD_RECORDS");
    return e && atoi(e) == 1;
  }();
  if (!d_radix && records && lsd_records_supported(elsize, d_in, d_out, *key))
    return lsd_records_enqueue(c, d_in, d_out, n, elsize, key, skip_trivial, st);
  const int nwords = d_radix ? (int)((rsize + 7) / 8) : (int)key->nwords;
  GB_CUDA(c.keysA.ensure(sizeof(uint64_t) * (size_t)n * nwords));
  GB_CUDA(c.keysB.ensure(sizeof(uint64_t) * (size_t)n * nwords));
  GB_CUDA(c.idxA.ensure(sizeof(uint32_t) * (size_t)n));
  GB_CUDA(c.idxB.ensure(sizeof(uint32_t) * (size_t)n));
  if (d_in == d_out) GB_CUDA(c.A.ensure((size_t)n * elsize));
  GB_CUDA(c.small.ensure(lsd_scratch_bytes(n, nwords) + CNT_WORDS * 4 + 4096));
  Bump bump{c.small.as<uint8_t>()};
  uint32_t* counters = bump.take<uint32_t>(CNT_WORDS);
  uint32_t* err = counters + CNT_ERR;
  GB_CUDA(cudaMemsetAsync(counters, 0, CNT_WORDS * sizeof(uint32_t), st));
  if (d_radix) GB_CUDA(radix_bytes_to_keys(d_radix, n, rsize, c.keysA.as<uint64_t>(), c.idxA.as<uint32_t>(), st));
  else GB_CUDA(extract_keys(d_in, n, elsize, *key, c.keysA.as<uint64_t>(), c.idxA.as<uint32_t>(), st));
  int passes = 0;
  int rc = lsd_sort_keys(bump, c.keysA.as<uint64_t>(), c.keysB.as<uint64_t>(), c.idxA.as<uint32_t>(),
                         c.idxB.as<uint32_t>(), n, nwords, skip_trivial, &passes, err, st);
  if (rc) return rc;
  const void* src = d_in;
  if (d_in == d_out) {  // the gather needs an untouched copy of the input
    GB_CUDA(cudaMemcpyAsync(c.A.p, d_in, (size_t)n * elsize, cudaMemcpyDeviceToDevice, st));
    src = c.A.p;
  }
  GB_CUDA(gather_records(src, d_out, c.idxA.as<uint32_t>(), n, elsize, st));
  GB_CUDA(cudaMemcpyAsync(c.hc->c, counters, CNT_WORDS * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  c.run_lsd_passes = (uint32_t)passes;
  return GBSORT_OK;
}

int lsd_collect(Context& c) {
  if (c.hc->c[CNT_ERR]) {
    set_err("device check failed in the LSD path: code %u", c.hc->c[CNT_ERR]);
    return GBSORT_ERR_INTERNAL;
  }
  g_stats = gbsort_stats{};
  g_stats.method = GBSORT_LSD;
  g_stats.lsd_passes = c.run_lsd_passes;
  return GBSORT_OK;
}

int run_lsd(Context& c, const void* d_in, void* d_out, uint32_t n, uint32_t elsize, const gbsort_key_desc* key,
            const uint8_t* d_radix, uint32_t rsize, cudaStream_t st) {
  // the constant-digit check costs a host round trip: worth it for large sorts only
  int rc = lsd_enqueue(c, d_in, d_out, n, elsize, key, d_radix, rsize, n >= (1u << 22), st);
  if (rc) return rc;
  GB_CUDA(cudaStreamSynchronize(st));
  return lsd_collect(c);
}

// --------------------------------------------------------- hsort path ----
bool hsort_layout_ok(const void* d_in, const void* d_out, uint32_t elsize, const gbsort_key_desc* key) {
  if (key->nwords != 1 || !hsort_supported(elsize)) return false;
  if (key->word[0].offset % 4) return false;
  uintptr_t a = (uintptr_t)d_in | (uintptr_t)d_out;
  uint32_t need = elsize % 16 == 0 ? 16 : (elsize % 8 == 0 ? 8 : 4);
  return a % need == 0;
}

struct HsortRun {
  uint32_t nbuckets = 1;
  uint32_t sample = 0;
};

// Run-time shape of a histogram sort (the autotuner's choices).
struct Knobs {
  int max_buckets = 0;        // level-1 bucket cap, a power of two up to 4096 (0: default)
  int sample_per_bucket = 0;  // sampled keys per level-1 bucket (0: 128)
  int level2 = 0;             // GBSORT_LEVEL2_*: split rounds or the persistent engine (0: default)
};

// Level-1 bucket count: about 2048 records per bucket, at most the cap --
// the knob, else GBSORT_MAX_BUCKETS (a power of two up to 4096), else 2048.
// Fewer, larger buckets keep the scatter's runs long enough to fill whole
// DRAM sectors; the bucket splits then carry more of the work.  4096
// buckets (1e9 x 16 B) help uniform keys (44.5 against 46.6 ms: smaller
// splits) but not sorted-with-swaps (36.2 / 34.3 ms), Zipf (62.8 / 55.7 ms)
// or 40-byte records (69.3 / 60.1 ms): the 16-byte scatter's ranking table
// and held sectors then leave room for one CTA per SM only.
int choose_buckets(uint32_t n, uint32_t elsize, const Knobs& k) {
  if (n <= 4096) return 1;
  static int env_cap = -1;
  if (env_cap < 0) {
    const char* e = getenv("GBSORT_MAX_BUCKETS");
    int v = e ? atoi(e) : 0;
    env_cap = (v >= 2 && v <= 4096 && (v & (v - 1)) == 0) ? v : 0;
  }
  (void)elsize;
  const int cap = k.max_buckets ? k.max_buckets : env_cap ? env_cap : 2048;
  uint64_t want = ((uint64_t)n + 2047) / 2048;
  uint32_t nb = pow2_ceil(want);
  return (int)std::min<uint32_t>(nb, (uint32_t)cap);
}

// ------------------------------------------------------ tuning table ----
// Winning configurations of gbsort_autotune per (record size, key width,
// size class = bit length of n); sorts with GBSORT_AUTO look here first.
std::mutex g_tune_mu;
std::map<uint64_t, gbsort_tuning> g_tune;

uint64_t tune_key(uint32_t elsize, uint32_t width, uint32_t cls) {
  return ((uint64_t)elsize << 16) | ((uint64_t)width << 8) | cls;
}
uint32_t size_class(uint64_t n) {
  uint32_t b = 0;
  while (n) {
    ++b;
    n >>= 1;
  }
  return b;
}
bool tuning_ok(const gbsort_tuning& t) {
  if (t.method != GBSORT_HISTOGRAM_PLAIN && t.method != GBSORT_HISTOGRAM_LEARNED && t.method != GBSORT_LSD)
    return false;
  if (t.max_buckets && (t.max_buckets < 2 || t.max_buckets > 4096 || (t.max_buckets & (t.max_buckets - 1))))
    return false;
  if (t.level2 > GBSORT_LEVEL2_ENGINE) return false;
  return t.sample_per_bucket == 0 || (t.sample_per_bucket >= 16 && t.sample_per_bucket <= 1024);
}
// The entry of the nearest size class (within a factor of 4) for this layout.
bool tune_lookup(uint32_t elsize, uint32_t width, uint64_t n, gbsort_tuning* out) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  if (g_tune.empty()) return false;
  const uint32_t cls = size_class(n);
  for (uint32_t d = 0; d <= 2; ++d)
    for (int sgn = 0; sgn < 2; ++sgn) {
      if (d == 0 && sgn) continue;
      uint32_t c = sgn ? cls + d : cls - d;
      if (c > 64) continue;
      auto it = g_tune.find(tune_key(elsize, width, c));
      if (it != g_tune.end()) {
        *out = it->second;
        return true;
      }
    }
  return false;
}

// Device task lists of level 2 and their counters.
struct Level2 {
  SortTask* split[2];
  SortTask* local;
  uint32_t* nsplit;  // [2]
  uint32_t* nlocal;
  uint32_t* work;
  uint32_t cap_split, cap_local;
  SortTask* qtask;   // the persistent engine's queue (every task of level 2)
  uint32_t* qready;
  uint32_t* qctl;    // tail, head, pending
  uint32_t qcap;
  static size_t bytes(uint32_t cap_split, uint32_t cap_local) {
    const size_t q = (size_t)cap_split + cap_local;
    return ((size_t)cap_split * 2 + cap_local) * sizeof(SortTask) + q * (sizeof(SortTask) + 4) + 8192;
  }
  // counters: the run's counter array (CNT_WORDS)
  void carve(Bump& bump, uint32_t* counters, uint32_t cs, uint32_t cl) {
    cap_split = cs;
    cap_local = cl;
    split[0] = bump.take<SortTask>(cs);
    split[1] = bump.take<SortTask>(cs);
    local = bump.take<SortTask>(cl);
    nsplit = counters + CNT_L2;
    nlocal = counters + CNT_L2 + 2;
    work = counters + CNT_L2 + 3;
    qcap = cs + cl;
    qtask = bump.take<SortTask>(qcap);
    qready = bump.take<uint32_t>(qcap);
    qctl = counters + CNT_ENGINE;
  }
  TaskListsHost round(int r) const {  // round r reads split[r&1], appends to split[(r+1)&1]
    TaskListsHost L;
    L.split_in = split[r & 1];
    L.nsplit_in = nsplit + (r & 1);
    L.split_out = split[(r + 1) & 1];
    L.nsplit_out = nsplit + ((r + 1) & 1);
    L.local = local;
    L.nlocal = nlocal;
    L.cap_split = cap_split;
    L.cap_local = cap_local;
    return L;
  }
};

constexpr uint64_t kAutoLsdMax = (uint64_t)1 << 23;  // method auto, untuned: LSD up to this many records
constexpr int kSplitRounds = 16;  // every round narrows each re-split range; 64-bit keys need few
constexpr int kCdfEpochs = 8;     // gradient steps of the CDF model

// Level 2 as the persistent engine or as split rounds.  The engine takes
// records of 8-16 bytes with their tasks at final positions.  By default
// batched segments use it (their uneven tasks leave rounds half idle:
// configuration 3, 1.74e10 -> 2.05e10 records/s) and a single array keeps
// the rounds (uniform keys, 1e9 x 16 B: rounds 24.8 ms, engine 28.0 ms --
// the engine kernel holds both task bodies in one register budget); a
// tuning entry or GBSORT_LEVEL2=rounds|engine overrides the default.
bool use_engine(uint32_t elsize, int level2, bool segments) {
  static const int env = [] {
    const char* e = getenv("GBSORT_LEVEL2");
    if (!e) return 0;
    return strcmp(e, "engine") == 0 ? (int)GBSORT_LEVEL2_ENGINE
                                    : (strcmp(e, "rounds") == 0 ? (int)GBSORT_LEVEL2_ROUNDS : 0);
  }();
  if (!engine_supported(elsize)) return false;
  const int choice = env ? env : level2;
  if (choice == GBSORT_LEVEL2_ENGINE) return true;
  if (choice == GBSORT_LEVEL2_ROUNDS) return false;
  return segments;
}

uint32_t hsort_sample_size(uint32_t n, int nb, const Knobs& knobs) {
  const uint64_t spb = knobs.sample_per_bucket ? (uint64_t)knobs.sample_per_bucket : 128;
  return nb > 1 ? (uint32_t)std::min<uint64_t>(n, std::max<uint64_t>(4096, (uint64_t)nb * spb)) : 0;
}

// Leaves of the learned CDF model of the histogram sort: 2^12.  Finer
// leaves narrow the lookup windows of clustered keys (5e8 x 40 B Morton
// keys: count 3.62 ms with 2^11 leaves, 3.40 ms with 2^12); uniform and
// Zipf keys count in the same time either way.  The count holds 12 bytes
// per leaf in shared memory.
constexpr int kModelLeafBits = 12;

// Bytes of the small device buffer a histogram sort of n records uses
// (G: count chunks).
size_t hsort_small_bytes(uint32_t n, uint32_t elsize, const Knobs& knobs, int G) {
  const int nb = choose_buckets(n, elsize, knobs);
  const uint32_t s = hsort_sample_size(n, nb, knobs);
  const uint32_t cap_split = (uint32_t)nb + n / 4096 + 4096;
  const uint32_t cap_local = 4u * (uint32_t)nb + n / 512 + 65536;
  const int nleaf = 1 << kModelLeafBits;
  return (size_t)s * 16 + (size_t)nb * 8 + (size_t)nb * G * 8 + Level2::bytes(cap_split, cap_local) +
         lsd_scratch_bytes(std::max<uint32_t>(s, 1), 1) + (size_t)nleaf * 64 + (size_t)nb * 24 + sizeof(HeavyTable) +
         (4 << 20);
}

// Enqueues the whole histogram sort on `st` without waiting for the host
// anywhere (so it can be captured into a CUDA graph); the device counters
// end up in c.hc once the stream reaches the end.  hsort_collect reads them.
int hsort_enqueue(Context& c, const void* d_in, void* d_out, uint32_t n, uint32_t elsize, const gbsort_key_desc* key,
                  bool learned, bool timing, const Knobs& knobs, cudaStream_t st, const HostPipe* hp = nullptr) {
  const int nb = choose_buckets(n, elsize, knobs);
  const int grid = hsort_grid(n);
  const uint32_t s = hsort_sample_size(n, nb, knobs);
  // pipelined: the input goes up in pieces, each cut into `grid` count
  // chunks, and is scattered as it lands into bucket regions reserved from
  // the sample (kRegion*); scratch A holds the regions
  const int pieces = hp ? std::min(hp->pieces, kMaxPieces) : 1;
  const int G = grid * pieces;  // count chunks
  uint64_t a_cap64 = n;
  bool region_fit = false;  // the reserved regions fit 32-bit record offsets
  if (hp && s > 0) {
    const double per = (double)n / (double)s, snb = (double)s + nb;
    const double reserved = ((double)s + kRegionSigmas * std::sqrt((double)nb * snb) + kRegionSpare * nb) * per +
                            (double)nb * (kRegionPad + 2);
    region_fit = reserved < 4294967295.0;
    if (region_fit) a_cap64 = (uint64_t)reserved;
  }
  const uint32_t a_cap = (uint32_t)std::max<uint64_t>(a_cap64, n);
  // areas: the split rounds of records of 8-16 bytes give each level-1
  // bucket an area of scratch B a quarter larger than the bucket (uniform
  // splits scatter into regions there); the persistent engine does not
  bool areas = elsize % 4 == 0 && elsize >= 8 && elsize <= 16 && n <= kSplitAreaMaxN &&
               (hp || !use_engine(elsize, knobs.level2, false));
  GB_CUDA(c.A.ensure((size_t)a_cap * elsize + kScratchSlack));
  if (areas && c.B.ensure((size_t)split_area(n) * elsize + kScratchSlack) != cudaSuccess) {
    cudaGetLastError();  // no room for the areas: the splits write at final positions
    areas = false;
  }
  GB_CUDA(c.B.ensure((size_t)(areas ? split_area(n) : n) * elsize + kScratchSlack));
  const uint32_t cap_split = (uint32_t)nb + n / 4096 + 4096;
  const uint32_t cap_local = 4u * (uint32_t)nb + n / 512 + 65536;
  const int lbits = kModelLeafBits;
  const int nleaf = 1 << lbits;
  GB_CUDA(c.small.ensure(hsort_small_bytes(n, elsize, knobs, G)));
  Bump bump{c.small.as<uint8_t>()};
  uint32_t* counters = bump.take<uint32_t>(CNT_WORDS);
  uint32_t* stats = counters;
  uint32_t* err = counters + CNT_ERR;
  uint32_t* iters = counters + CNT_ITERS;
  uint32_t* widest = counters + CNT_WIDEST;
  float* loss = reinterpret_cast<float*>(counters + CNT_LOSS);
  uint32_t* fallback = counters + CNT_FALLBACK;
  GB_CUDA(cudaMemsetAsync(counters, 0, CNT_WORDS * sizeof(uint32_t), st));
  uint64_t* S = bump.take<uint64_t>((size_t)std::max(nb, 2));
  uint32_t* counts = bump.take<uint32_t>((size_t)nb * G);
  uint32_t* scan_tmp = bump.take<uint32_t>(scan_tmp_words((size_t)nb * G));
  Level2 l2;
  l2.carve(bump, counters, cap_split, cap_local);

  HsortParams p{};
  p.in = (const uint8_t*)d_in;
  p.out = (uint8_t*)d_out;
  p.bufA = c.A.as<uint8_t>();
  p.bufB = c.B.as<uint8_t>();
  p.n = n;
  p.elsize = elsize;
  p.key = key->word[0];
  p.a_cap = a_cap;
  p.chunks = (uint32_t)G;
  p.areas = areas ? 1u : 0u;
  p.bkt = c.B.as<uint16_t>();  // scratch B is free during level 1
  static const bool uniform_off = getenv("GBSORT_UNIFORM_SPLITS") && atoi(getenv("GBSORT_UNIFORM_SPLITS")) == 0;
  p.uniform = areas && !uniform_off ? counters + CNT_UNIFORM : nullptr;
  p.gate_widest = counters + CNT_WIDEST;
  p.gate_heavy = counters + CNT_HEAVY;

  ModelDev model{};
  int lookup = LOOKUP_PLAIN;
  if (hp)
    for (int i = 0; i < pieces; ++i) {
      const uint32_t r0 = hsort_chunk_begin(n, i * grid, G), r1 = hsort_chunk_begin(n, (i + 1) * grid, G);
      GB_CUDA(cudaMemcpyAsync((uint8_t*)d_in + (size_t)r0 * elsize, hp->h_in + (size_t)r0 * elsize,
                              (size_t)(r1 - r0) * elsize, cudaMemcpyHostToDevice, c.cstream));
      GB_CUDA(cudaEventRecord(c.pev[i], c.cstream));
    }
  if (timing) GB_CUDA(cudaEventRecord(c.ev[0], st));
  uint64_t* bump_sample = nullptr;  // the sorted sample (for the reserved regions)
  if (nb > 1) {
    uint64_t* sA = bump.take<uint64_t>(s);
    uint64_t* sB = bump.take<uint64_t>(s);
    bump_sample = sA;
    // pipelined: the sample is read from the pinned host array itself by the
    // sampling kernel (over the host link, without waiting for the copy
    // engine, which is busy with the pieces)
    GB_CUDA(sample_keys(hp ? hp->h_in : p.in, n, elsize, p.key, s, sA, st));
    int rc = lsd_sort_keys(bump, sA, sB, nullptr, nullptr, s, 1, false, nullptr, err, st);
    if (rc) return rc;
    if (!learned) {
      GB_CUDA(plain_splitters(sA, s, nb - 1, S, iters, nullptr, nullptr, st));
      GB_CUDA(finalize_splitters(S, nb - 1, st));
    } else {
      CdfShape* dshape = bump.take<CdfShape>(1);
      GB_CUDA(cdf_shape_device(sA, s, lbits, dshape, st));
      const CdfShape sh = cdf_shape_ref(dshape, lbits);
      CdfWork w{};
      w.y = bump.take<float>(nleaf + 1);
      w.grad = bump.take<float>(nleaf + 1);
      w.h = bump.take<float>(nleaf + 1);
      w.off = bump.take<float>(nleaf + 1);
      w.knots = bump.take<float2>(nleaf);
      w.loss = loss;
      uint32_t* win = bump.take<uint32_t>(nleaf);
      uint32_t* wlo = bump.take<uint32_t>(nleaf);
      uint32_t* whi = bump.take<uint32_t>(nleaf);
      GB_CUDA(cdf_train(sA, s, sh, kCdfEpochs, 0.5f, w, st));
      GB_CUDA(cdf_splitters(sA, s, sh, nb, w.knots, S, st));
      GB_CUDA(finalize_splitters(S, nb - 1, st));
      // the plain splitters vet the model's: if the sample shows a heavy
      // key outside a single-key bucket or an overfull bucket, the sample's
      // own quantiles (what the bisection converges to) replace them, on the
      // device; the model still serves the lookup, its knots then set from
      // the final splitters, with windows for them
      uint32_t* jcounts = bump.take<uint32_t>(nb);
      GB_CUDA(vet_splitters(sA, s, S, nb, jcounts, fallback, st));
      GB_CUDA(quantile_splitters(sA, s, nb - 1, S, fallback, st));
      GB_CUDA(finalize_splitters(S, nb - 1, st, fallback));
      GB_CUDA(refit_knots(sh, nb, S, w.knots, fallback, st));
      GB_CUDA(cdf_windows(sh, nb, w.knots, S, win, wlo, whi, widest, st));
      model.lbits = lbits;
      model.nbuckets = nb;
      model.knots = w.knots;
      model.win = win;
      model.shape = dshape;
      lookup = LOOKUP_LEARNED;
    }
    HeavyTable* heavy = bump.take<HeavyTable>(1);
    GB_CUDA(heavy_table(S, nb - 1, heavy, counters + CNT_HEAVY, st));
    p.heavy = heavy;
  }
  if (timing) GB_CUDA(cudaEventRecord(c.ev[1], st));
  const ModelDev* mp = lookup == LOOKUP_LEARNED ? &model : nullptr;
  // the level-1 scatter: each record to the bucket the count wrote for it
  auto scatter = [&](int c0, int c1, const uint32_t* skip) -> cudaError_t {
    return l1_scatter(p, nb, counts, stats, st, c0, c1, skip);
  };

  // pipelined: each piece is counted and scattered into the reserved bucket
  // regions as soon as it has landed; if a bucket outgrows its region the
  // scatters stop and level 1 is redone exactly from the complete input
  bool regions = false;
  uint32_t *region = nullptr, *total = nullptr, *out_start = nullptr;
  const int waves = hp ? std::max(1, std::min(std::min(hp->waves, kMaxWaves), nb)) : 1;
  if (hp) {
    uint32_t* cap = bump.take<uint32_t>(nb);
    region = bump.take<uint32_t>(nb);
    total = bump.take<uint32_t>(nb);
    out_start = bump.take<uint32_t>(nb);
    uint32_t* overflow = counters + CNT_OVERFLOW;
    c.hc->c[CNT_OVERFLOW] = 0;
    if (region_fit) {
      GB_CUDA(bucket_caps(bump_sample, s, S, nb, n, kRegionSigmas, kRegionSpare, kRegionPad, cap, st));
      GB_CUDA(exclusive_scan_u32(cap, region, (size_t)nb, scan_tmp, st));
      GB_CUDA(cudaMemsetAsync(total, 0, sizeof(uint32_t) * nb, st));
      for (int i = 0; i < pieces; ++i) {
        GB_CUDA(cudaStreamWaitEvent(st, c.pev[i], 0));
        GB_CUDA(l1_count(p, lookup, S, nb, mp, counts, stats, st, i * grid, (i + 1) * grid));
        GB_CUDA(region_offsets(counts, G, nb, region, cap, total, i * grid, (i + 1) * grid, overflow, st));
        GB_CUDA(scatter(i * grid, (i + 1) * grid, overflow));
      }
      GB_CUDA(cudaMemcpyAsync(&c.hc->c[CNT_OVERFLOW], overflow, 12, cudaMemcpyDeviceToHost, st));
    } else {  // regions would not fit 32-bit offsets: level 1 waits for the whole input
      for (int i = 0; i < pieces; ++i) GB_CUDA(cudaStreamWaitEvent(st, c.pev[i], 0));
    }
    GB_CUDA(cudaEventRecord(c.sev, st));
    GB_CUDA(cudaEventSynchronize(c.sev));
    regions = region_fit && c.hc->c[CNT_OVERFLOW] == 0 && !getenv("GBSORT_NO_REGIONS");
    if (regions) {
      GB_CUDA(exclusive_scan_u32(total, out_start, (size_t)nb, scan_tmp, st));
    } else {  // exact level 1 over the complete input
      p.a_cap = n;
      GB_CUDA(l1_count(p, lookup, S, nb, mp, counts, stats, st));
      GB_CUDA(exclusive_scan_u32(counts, counts, (size_t)nb * G, scan_tmp, st));
      GB_CUDA(scatter(0, -1, nullptr));
    }
    // the first output record of every wave of level-1 buckets
    for (int j = 0; j < waves; ++j) {
      const uint32_t* at = regions ? out_start + (size_t)(j * nb / waves) : counts + (size_t)(j * nb / waves) * G;
      GB_CUDA(cudaMemcpyAsync(&c.hc->starts[j], at, 4, cudaMemcpyDeviceToHost, st));
    }
    c.hc->starts[waves] = n;
    GB_CUDA(cudaEventRecord(c.sev, st));
  } else {
    GB_CUDA(l1_count(p, lookup, S, nb, mp, counts, stats, st));
    if (timing) GB_CUDA(cudaEventRecord(c.ev[2], st));
    GB_CUDA(exclusive_scan_u32(counts, counts, (size_t)nb * G, scan_tmp, st));
    if (timing) GB_CUDA(cudaEventRecord(c.ev[3], st));
    GB_CUDA(scatter(0, -1, nullptr));
  }
  if (timing) GB_CUDA(cudaEventRecord(c.ev[4], st));
  static const bool trace = getenv("GBSORT_TRACE") != nullptr;
  for (int j = 0; j < waves; ++j) {
    if (hp) {  // the wave's lists start empty
      GB_CUDA(cudaMemsetAsync(l2.nsplit, 0, sizeof(uint32_t), st));
      GB_CUDA(cudaMemsetAsync(l2.nlocal, 0, sizeof(uint32_t), st));
    }
    {
      TaskListsHost L = l2.round(-1);  // appends to split[0]
      if (regions)
        GB_CUDA(build_region_tasks(region, total, out_start, S, nb, L, err, stats, st, j * nb / waves,
                                   (j + 1) * nb / waves));
      else
        GB_CUDA(build_tasks(counts, G, S, nb, n, L, err, stats, st, j * nb / waves, (j + 1) * nb / waves));
    }
    if (!hp && use_engine(elsize, knobs.level2, false)) {  // one persistent launch (a host sort's waves keep the rounds)
      GB_CUDA(run_engine(p, l2.round(0), l2.qtask, l2.qready, l2.qctl, l2.qcap, stats, err, st));
      if (timing) GB_CUDA(cudaEventRecord(c.ev[5], st));
      continue;
    }
    for (int r = 0; r < kSplitRounds; ++r) {
      TaskListsHost L = l2.round(r);
      GB_CUDA(cudaMemsetAsync(L.nsplit_out, 0, sizeof(uint32_t), st));
      GB_CUDA(run_split_round(p, L, l2.work, stats, err, st));
      if (trace && timing) {  // debugging aid: split tasks per round (synchronises)
        uint32_t h[3];
        GB_CUDA(cudaMemcpyAsync(h, l2.nsplit, 12, cudaMemcpyDeviceToHost, st));
        GB_CUDA(cudaStreamSynchronize(st));
        fprintf(stderr, "gbsort trace: round %d in %u out %u local %u\n", r, h[r & 1], h[(r + 1) & 1], h[2]);
      }
    }
    if (timing) GB_CUDA(cudaEventRecord(c.ev[5], st));
    GB_CUDA(run_local(p, l2.local, l2.nlocal, l2.cap_local, l2.work, stats, st));
    if (hp) {
      GB_CUDA(require_zero(l2.nsplit + (kSplitRounds & 1), err, st));
      GB_CUDA(cudaEventRecord(c.wev[j], st));
    }
  }
  if (timing) GB_CUDA(cudaEventRecord(c.ev[6], st));
  GB_CUDA(cudaMemcpyAsync(c.hc->c, counters, CNT_WORDS * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  if (hp) {  // each wave's output range goes down as soon as the wave is sorted
    GB_CUDA(cudaEventSynchronize(c.sev));
    for (int j = 0; j < waves; ++j) {
      const uint32_t r0 = c.hc->starts[j], r1 = c.hc->starts[j + 1];
      if (r1 < r0 || r1 > n) {
        set_err("wave bounds out of order");
        return GBSORT_ERR_INTERNAL;
      }
      GB_CUDA(cudaStreamWaitEvent(c.cstream, c.wev[j], 0));
      if (r1 > r0)
        GB_CUDA(cudaMemcpyAsync(hp->h_out + (size_t)r0 * elsize, (const uint8_t*)d_out + (size_t)r0 * elsize,
                                (size_t)(r1 - r0) * elsize, cudaMemcpyDeviceToHost, c.cstream));
    }
    GB_CUDA(cudaEventRecord(c.dev_done, c.cstream));
    static const bool ptrace = getenv("GBSORT_PIPE_TRACE") != nullptr;
    if (ptrace) {  // debugging aid: the pipeline's timeline (synchronises)
      GB_CUDA(cudaEventSynchronize(c.dev_done));
      float t;
      cudaEventElapsedTime(&t, c.pev[0], c.pev[pieces - 1]);
      fprintf(stderr, "gbsort pipe: pieces up by %.2f ms (after the first)\n", t);
      cudaEventElapsedTime(&t, c.pev[0], c.sev);
      fprintf(stderr, "gbsort pipe: counts scanned at %.2f\n", t);
      if (c.hc->c[CNT_OVERFLOW])
        fprintf(stderr, "gbsort pipe: bucket %u outgrew its region (%u records reserved, %u counted)\n",
                c.hc->c[CNT_OVERFLOW] - 1, c.hc->c[CNT_OVERFLOW + 1], c.hc->c[CNT_OVERFLOW + 2]);
      for (int j = 0; j < waves; ++j) {
        cudaEventElapsedTime(&t, c.pev[0], c.wev[j]);
        fprintf(stderr, "gbsort pipe: wave %d sorted at %.2f\n", j, t);
      }
      cudaEventElapsedTime(&t, c.pev[0], c.dev_done);
      fprintf(stderr, "gbsort pipe: last piece down at %.2f\n", t);
    }
  }
  c.run_nbuckets = (uint32_t)nb;
  c.run_sample = s;
  c.run_learned = learned;
  c.run_engine = !hp && use_engine(elsize, knobs.level2, false);
  c.run_timing = timing;
  c.run_pipelined = hp != nullptr;
  return GBSORT_OK;
}

// Status and statistics of the last enqueued histogram sort, once its
// stream has reached the end.
int hsort_collect(Context& c) {
  const uint32_t* h = c.hc->c;
  if (h[CNT_ERR]) {
    set_err("device check failed: code %u", h[CNT_ERR]);
    return GBSORT_ERR_INTERNAL;
  }
  // the last round's output list, or the engine's pending tasks, must be empty
  const uint32_t left = c.run_engine ? h[CNT_ENGINE + 2 * kEngineCtlStride] : h[CNT_L2 + (kSplitRounds & 1)];
  if (left != 0) {
    set_err("level 2 did not finish: %u tasks left", left);
    return GBSORT_ERR_INTERNAL;
  }
  g_stats = gbsort_stats{};
  g_stats.method = c.run_learned ? GBSORT_HISTOGRAM_LEARNED : GBSORT_HISTOGRAM_PLAIN;
  g_stats.nbuckets = c.run_nbuckets;
  g_stats.sample = c.run_sample;
  g_stats.splitter_rounds = c.run_learned ? (uint32_t)kCdfEpochs : h[CNT_ITERS];
  g_stats.local_sorts = h[STAT_LOCAL];
  g_stats.splits = h[STAT_SPLIT];
  g_stats.copies = h[STAT_COPY];
  g_stats.resplits = h[STAT_PUSHED];
  g_stats.bigbin_passes = h[STAT_BIGBIN];
  g_stats.window_misses = h[STAT_WINDOW_MISS];
  g_stats.max_bucket = h[STAT_MAX_BUCKET];
  g_stats.widest_window = h[CNT_WIDEST];
  float loss;
  memcpy(&loss, &h[CNT_LOSS], 4);
  g_stats.model_loss = c.run_learned ? loss : 0.f;
  g_stats.splitter_fallback = c.run_learned && h[CNT_FALLBACK] ? 1u : 0u;
  g_stats.heavy_keys = h[CNT_HEAVY];
  g_stats.refined_splits = h[STAT_REFINED];
  g_stats.pipelined = c.run_pipelined ? 1u : 0u;
  g_stats.region_overflow = c.run_pipelined ? h[CNT_OVERFLOW] : 0u;
  g_stats.engine = c.run_engine ? 1u : 0u;
  g_stats.uniform_splits = h[CNT_UNIFORM] - h[CNT_UNIFORM + 1];
  g_stats.uniform_fallbacks = h[CNT_UNIFORM + 1];
  g_stats.deep_splits = h[STAT_DEEP];
  if (c.run_timing)
    for (int i = 0; i < 6; ++i) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, c.ev[i], c.ev[i + 1]);
      g_stats.stage_ms[i] = ms;
    }
  return GBSORT_OK;
}

int run_hsort(Context& c, const void* d_in, void* d_out, uint32_t n, uint32_t elsize, const gbsort_key_desc* key,
              int method, const Knobs& knobs, cudaStream_t st) {
  int rc = hsort_enqueue(c, d_in, d_out, n, elsize, key, method == GBSORT_HISTOGRAM_LEARNED, true, knobs, st);
  if (rc) return rc;
  GB_CUDA(cudaStreamSynchronize(st));
  return hsort_collect(c);
}

int sort_device_dispatch(Context& c, const void* d_in, void* d_out, size_t nmemb, size_t elsize,
                         const gbsort_key_desc* key, int method, cudaStream_t st);

// GBSORT_AUTO: the tuned configuration for this layout and size when there
// is one (a histogram method only where the layout allows it), else the
// learned histogram sort where possible and LSD otherwise.
int resolve_auto(uint32_t elsize, const gbsort_key_desc* key, uint64_t n, bool hs_ok, Knobs* knobs) {
  gbsort_tuning t;
  if (key->nwords == 1 && tune_lookup(elsize, key->word[0].width, n, &t)) {
    if (t.method == GBSORT_LSD) return GBSORT_LSD;
    if (hs_ok) {
      knobs->max_buckets = (int)t.max_buckets;
      knobs->sample_per_bucket = (int)t.sample_per_bucket;
      knobs->level2 = (int)t.level2;
      return t.method;
    }
  }
  // untuned: below about 8M records the LSD path's few full passes beat the
  // histogram sort's fixed costs (measured crossover 8M-16M, 16 B records)
  return hs_ok && n > kAutoLsdMax ? GBSORT_HISTOGRAM_LEARNED : GBSORT_LSD;
}

// Sorts of 2^32 records or more (64-bit counts): the splitters of P - 1
// sample quantiles cut the records into P key ranges of under 2^32 records
// each (P <= 15, about 1.5e9 records per range), one stable partition pass
// moves every range into its place in a scratch copy, and each range is
// then sorted into the output by the 32-bit pipeline.  A range of one key
// (a key owning 2^32 records or more) is copied, not sorted.  Synchronises
// with the host between the stages.
int run_partitioned(Context& c, const void* d_in, void* d_out, uint64_t n, uint32_t E, const gbsort_key_desc* key,
                    int method, cudaStream_t st) {
  constexpr uint64_t kPartTarget = 1500000000ull;
  constexpr uint64_t kPartMax = 0xfffffffeull;
  const int P = (int)std::min<uint64_t>(15, (n + kPartTarget - 1) / kPartTarget);
  if ((uint64_t)P * kPartTarget * 2 < n) {
    set_err("%llu records exceed the partitioned sort's range (about 2.2e10)", (unsigned long long)n);
    return GBSORT_ERR_BAD_ARG;
  }
  const int nsplit = P - 1;
  const uint32_t s = 1u << 20;
  const int g = part_grid();
  GB_CUDA(c.part.ensure((size_t)n * E + kScratchSlack));
  GB_CUDA(c.small.ensure((size_t)s * 16 + lsd_scratch_bytes(s, 1) + (size_t)g * 16 * 12 + (1 << 16)));
  Bump bump{c.small.as<uint8_t>()};
  uint32_t* counters = bump.take<uint32_t>(CNT_WORDS);
  uint32_t* err = counters + CNT_ERR;
  uint64_t* sA = bump.take<uint64_t>(s);
  uint64_t* sB = bump.take<uint64_t>(s);
  uint64_t* S = bump.take<uint64_t>(16);
  uint32_t* counts = bump.take<uint32_t>((size_t)16 * g);
  unsigned long long* offs = bump.take<unsigned long long>((size_t)16 * g);
  GB_CUDA(cudaMemsetAsync(counters, 0, CNT_WORDS * sizeof(uint32_t), st));
  GB_CUDA(sample_keys64((const uint8_t*)d_in, n, E, key->word[0], s, sA, st));
  int rc = lsd_sort_keys(bump, sA, sB, nullptr, nullptr, s, 1, false, nullptr, err, st);
  if (rc) return rc;
  GB_CUDA(plain_splitters(sA, s, nsplit, S, counters + CNT_ITERS, nullptr, nullptr, st));
  GB_CUDA(finalize_splitters(S, nsplit, st));
  GB_CUDA(part_count((const uint8_t*)d_in, n, E, key->word[0], S, nsplit, counts, st));
  std::vector<uint32_t> hc((size_t)P * g);
  std::vector<uint64_t> hS(16, 0);
  uint32_t herr = 0;
  GB_CUDA(cudaMemcpyAsync(hc.data(), counts, hc.size() * 4, cudaMemcpyDeviceToHost, st));
  if (nsplit) GB_CUDA(cudaMemcpyAsync(hS.data(), S, (size_t)nsplit * 8, cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaMemcpyAsync(&herr, err, 4, cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  if (herr) {
    set_err("device check failed in the partition's splitter search: code %u", herr);
    return GBSORT_ERR_INTERNAL;
  }
  std::vector<unsigned long long> ho((size_t)P * g);
  std::vector<uint64_t> pstart(P + 1, 0);
  uint64_t run = 0;
  for (int q = 0; q < P; ++q) {
    pstart[q] = run;
    for (int ch = 0; ch < g; ++ch) {
      ho[(size_t)q * g + ch] = run;
      run += hc[(size_t)q * g + ch];
    }
  }
  pstart[P] = run;
  if (run != n) {
    set_err("partition counts %llu records of %llu", (unsigned long long)run, (unsigned long long)n);
    return GBSORT_ERR_INTERNAL;
  }
  auto range_of = [&](int q, uint64_t& lo, uint64_t& hi) {
    lo = q == 0 ? 0ull : hS[q - 1];
    hi = q == nsplit ? ~0ull : hS[q] - 1;
  };
  for (int q = 0; q < P; ++q) {
    uint64_t lo, hi;
    range_of(q, lo, hi);
    if (pstart[q + 1] - pstart[q] > kPartMax && lo != hi) {
      set_err("a key range of the partition holds %llu records (2^32 or more) of more than one key",
              (unsigned long long)(pstart[q + 1] - pstart[q]));
      return GBSORT_ERR_UNSUPPORTED;
    }
  }
  GB_CUDA(cudaMemcpyAsync(offs, ho.data(), ho.size() * 8, cudaMemcpyHostToDevice, st));
  GB_CUDA(part_scatter((const uint8_t*)d_in, c.part.as<uint8_t>(), n, E, key->word[0], S, nsplit, offs, err, st));
  GB_CUDA(cudaMemcpyAsync(&herr, err, 4, cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  if (herr) {
    set_err("device check failed in the partition scatter: code %u", herr);
    return GBSORT_ERR_INTERNAL;
  }
  for (int q = 0; q < P; ++q) {
    const uint64_t a = pstart[q], m = pstart[q + 1] - pstart[q];
    if (m == 0) continue;
    uint64_t lo, hi;
    range_of(q, lo, hi);
    const uint8_t* src = c.part.as<uint8_t>() + (size_t)a * E;
    uint8_t* dst = (uint8_t*)d_out + (size_t)a * E;
    if (lo == hi) {  // one key: the partition kept input order, which is the stable order
      GB_CUDA(cudaMemcpyAsync(dst, src, (size_t)m * E, cudaMemcpyDeviceToDevice, st));
      continue;
    }
    rc = sort_device_dispatch(c, src, dst, m, E, key, method, st);
    if (rc) return rc;
  }
  GB_CUDA(cudaStreamSynchronize(st));
  return GBSORT_OK;
}

int sort_device_locked(Context& c, const void* d_in, void* d_out, size_t nmemb, size_t elsize,
                       const gbsort_key_desc* key, int method, cudaStream_t st) {
  const unsigned long long l0 = launch_count();
  // GBSORT_VERIFY: multiset hashes of the input before and the output after
  // the sort must agree (the reference's checksum, mpsort-mpi.c:148-159)
  const bool verify = (method & GBSORT_VERIFY) != 0 && nmemb > 0;
  method &= ~GBSORT_VERIFY;
  unsigned long long* vh = nullptr;
  if (verify) {
    GB_CUDA(c.vh.ensure(2 * sizeof(unsigned long long)));
    vh = c.vh.as<unsigned long long>();
    GB_CUDA(multiset_hash(d_in, nmemb, (uint32_t)elsize, vh, st));
  }
  int rc = sort_device_dispatch(c, d_in, d_out, nmemb, elsize, key, method, st);
  if (rc == GBSORT_OK && verify) {
    unsigned long long h[2];
    GB_CUDA(multiset_hash(d_out, nmemb, (uint32_t)elsize, vh + 1, st));
    GB_CUDA(cudaMemcpyAsync(h, vh, sizeof h, cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
    if (h[0] != h[1]) {
      set_err("self-check failed: the output is not a permutation of the input records (multiset hash %016llx, "
              "input %016llx)", h[1], h[0]);
      rc = GBSORT_ERR_INTERNAL;
    }
  }
  if (rc == GBSORT_OK) g_stats.launches = (uint32_t)(launch_count() - l0);
  return rc;
}

int sort_device_dispatch(Context& c, const void* d_in, void* d_out, size_t nmemb, size_t elsize,
                         const gbsort_key_desc* key, int method, cudaStream_t st) {
  if (nmemb == 0) {
    g_stats = gbsort_stats{};
    return GBSORT_OK;
  }
  if (elsize == 0 || elsize > (1u << 20)) {
    set_err("elsize must be in [1, 2^20]");
    return GBSORT_ERR_BAD_ARG;
  }
  if (!key_ok(key, elsize)) {
    set_err("bad key descriptor");
    return GBSORT_ERR_BAD_ARG;
  }
  if (nmemb >= 0xffffffffull) {  // 64-bit record counts: a first stable partition into key ranges
    if (!hsort_layout_ok(d_in, d_out, (uint32_t)elsize, key)) {
      set_err("sorts of 2^32 records or more need a one-word key at a 4-byte offset and a record size of 8-64 bytes");
      return GBSORT_ERR_UNSUPPORTED;
    }
    return run_partitioned(c, d_in, d_out, nmemb, (uint32_t)elsize, key, method, st);
  }
  const uint32_t n = (uint32_t)nmemb, E = (uint32_t)elsize;
  bool hs_ok = hsort_layout_ok(d_in, d_out, E, key);
  Knobs knobs;
  if (method == GBSORT_AUTO) method = resolve_auto(E, key, n, hs_ok, &knobs);
  if (method == GBSORT_HISTOGRAM_PLAIN || method == GBSORT_HISTOGRAM_LEARNED) {
    if (!hs_ok) {
      set_err("histogram sort needs a one-word key at a 4-byte offset and a record size of 8-64 bytes");
      return GBSORT_ERR_UNSUPPORTED;
    }
    return run_hsort(c, d_in, d_out, n, E, key, method, knobs, st);
  }
  if (method == GBSORT_LSD) return run_lsd(c, d_in, d_out, n, E, key, nullptr, 0, st);
  set_err("unknown method %d", method);
  return GBSORT_ERR_BAD_ARG;
}

}  // namespace

// ============================================================== C ABI ====
extern "C" {

int gbsort_sort_device(const void* d_in, void* d_out, size_t nmemb, size_t elsize, const gbsort_key_desc* key,
                       int method, void* stream) {
  if (nmemb && (!d_in || !d_out)) return GBSORT_ERR_BAD_ARG;
  Context* c = nullptr;
  int rc = get_ctx(&c);
  if (rc) return rc;
  std::lock_guard<std::mutex> lk(c->mu);
  cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
  return sort_device_locked(*c, d_in, d_out, nmemb, elsize, key, method, st);
}

namespace {
constexpr size_t kPipelineMin = (size_t)1 << 22;  // records; smaller host sorts copy in one piece each way
// An integer setting from the environment, within [lo, hi], else dflt.
int env_int(const char* name, int dflt, int lo, int hi) {
  const char* e = getenv(name);
  if (!e) return dflt;
  const int v = atoi(e);
  return v >= lo && v <= hi ? v : dflt;
}
bool is_pinned(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeHost;
}
}  // namespace

int gbsort_sort_host(const void* in, void* out, size_t nmemb, size_t elsize, const gbsort_key_desc* key,
                     int method) {
  if (nmemb == 0) return GBSORT_OK;
  if (!in || !out) return GBSORT_ERR_BAD_ARG;
  if (!key_ok(key, elsize)) {
    set_err("bad key descriptor");
    return GBSORT_ERR_BAD_ARG;
  }
  Context* c = nullptr;
  int rc = get_ctx(&c);
  if (rc) return rc;
  std::lock_guard<std::mutex> lk(c->mu);
  const size_t bytes = nmemb * elsize;
  GB_CUDA(c->hin.ensure(bytes));
  GB_CUDA(c->hout.ensure(bytes));
  // large sorts of pinned host arrays overlap their copies with the device
  // work (pieces up, waves down); pageable arrays would make every copy
  // synchronous, so they take the plain path
  if (nmemb >= kPipelineMin && nmemb < 0xffffffffull && is_pinned(in) && is_pinned(out)) {
    const uint32_t n = (uint32_t)nmemb, E = (uint32_t)elsize;
    const bool hs_ok = hsort_layout_ok(c->hin.p, c->hout.p, E, key);
    Knobs knobs;
    int m = method == GBSORT_AUTO ? resolve_auto(E, key, n, hs_ok, &knobs) : method;
    if (hs_ok && (m == GBSORT_HISTOGRAM_PLAIN || m == GBSORT_HISTOGRAM_LEARNED)) {
      static const int pieces = env_int("GBSORT_PIPE_PIECES", 16, 1, kMaxPieces);
      static const int waves = env_int("GBSORT_PIPE_WAVES", 16, 1, kMaxWaves);
      HostPipe hp{(const uint8_t*)in, (uint8_t*)out, pieces, waves};
      const unsigned long long l0 = launch_count();
      rc = hsort_enqueue(*c, c->hin.p, c->hout.p, n, E, key, m == GBSORT_HISTOGRAM_LEARNED, false, knobs, c->stream,
                         &hp);
      cudaError_t e1 = cudaStreamSynchronize(c->stream), e2 = cudaStreamSynchronize(c->cstream);
      if (rc) return rc;
      if (e1 != cudaSuccess || e2 != cudaSuccess) {
        set_err("pipelined host sort: %s", cudaGetErrorString(e1 != cudaSuccess ? e1 : e2));
        return GBSORT_ERR_CUDA;
      }
      rc = hsort_collect(*c);
      if (rc == GBSORT_OK) g_stats.launches = (uint32_t)(launch_count() - l0);
      return rc;
    }
  }
  GB_CUDA(cudaMemcpyAsync(c->hin.p, in, bytes, cudaMemcpyHostToDevice, c->stream));
  rc = sort_device_locked(*c, c->hin.p, c->hout.p, nmemb, elsize, key, method, c->stream);
  if (rc) return rc;
  GB_CUDA(cudaMemcpyAsync(out, c->hout.p, bytes, cudaMemcpyDeviceToHost, c->stream));
  GB_CUDA(cudaStreamSynchronize(c->stream));
  return GBSORT_OK;
}

int gbsort_sort_radix_host(void* base, size_t nmemb, size_t elsize,
                           void (*radix)(const void* ptr, void* radix, void* arg), size_t rsize, void* arg) {
  if (nmemb <= 1) return GBSORT_OK;
  if (!base || !radix || rsize == 0 || rsize > 8 * GBSORT_MAX_KEY_WORDS || elsize == 0) {
    set_err("bad arguments");
    return GBSORT_ERR_BAD_ARG;
  }
  if (nmemb >= 0xffffffffull) return GBSORT_ERR_BAD_ARG;
  Context* c = nullptr;
  int rc = get_ctx(&c);
  if (rc) return rc;
  std::lock_guard<std::mutex> lk(c->mu);
  // radix bytes on the host, in parallel slices (radix() must be re-entrant,
  // as the reference's mpsort_omp also calls it from every thread)
  std::vector<uint8_t> rb(nmemb * rsize);
  unsigned nth = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
  if (nmemb < 65536) nth = 1;
  std::vector<std::thread> th;
  for (unsigned t = 0; t < nth; ++t) {
    th.emplace_back([&, t]() {
      size_t lo = nmemb * t / nth, hi = nmemb * (t + 1) / nth;
      for (size_t i = lo; i < hi; ++i) radix((const uint8_t*)base + i * elsize, rb.data() + i * rsize, arg);
    });
  }
  for (auto& x : th) x.join();
  const size_t bytes = nmemb * elsize;
  GB_CUDA(c->hin.ensure(bytes));
  GB_CUDA(c->hout.ensure(bytes));
  GB_CUDA(c->radix.ensure(rb.size()));
  GB_CUDA(cudaMemcpyAsync(c->hin.p, base, bytes, cudaMemcpyHostToDevice, c->stream));
  GB_CUDA(cudaMemcpyAsync(c->radix.p, rb.data(), rb.size(), cudaMemcpyHostToDevice, c->stream));
  rc = run_lsd(*c, c->hin.p, c->hout.p, (uint32_t)nmemb, (uint32_t)elsize, nullptr, c->radix.as<uint8_t>(),
               (uint32_t)rsize, c->stream);
  if (rc) return rc;
  GB_CUDA(cudaMemcpyAsync(base, c->hout.p, bytes, cudaMemcpyDeviceToHost, c->stream));
  GB_CUDA(cudaStreamSynchronize(c->stream));
  return GBSORT_OK;
}

}  // extern "C"

namespace {

// ------------------------------------------------------ segmented sorts ----
// Shape of a batched segmented sort (its tuning entry: method / max_buckets
// for the segments sorted on their own, level2 for the shared pipeline,
// reserved[0] the size above which a segment is sorted on its own).
struct SegKnobs {
  int big_method = GBSORT_HISTOGRAM_LEARNED;
  Knobs big;
  int level2 = GBSORT_LEVEL2_DEFAULT;
  uint64_t big_above = (uint64_t)1 << 22;  // records: a segment this large fills the GPU on its own
};

uint64_t seg_tune_key(uint32_t elsize, uint32_t width, uint64_t n) {
  return tune_key(elsize, width, 0x80u | size_class(n));  // a key space of its own
}

SegKnobs seg_knobs(uint32_t elsize, const gbsort_key_desc* key, uint64_t n, int method) {
  SegKnobs k;
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(seg_tune_key(elsize, key->word[0].width, n));
    if (it != g_tune.end()) {
      const gbsort_tuning& t = it->second;
      if (t.method == GBSORT_HISTOGRAM_PLAIN || t.method == GBSORT_HISTOGRAM_LEARNED) k.big_method = t.method;
      k.big.max_buckets = (int)t.max_buckets;
      k.level2 = (int)t.level2;
      if (t.reserved[0]) k.big_above = t.reserved[0];
    }
  }
  if (method == GBSORT_HISTOGRAM_PLAIN || method == GBSORT_HISTOGRAM_LEARNED) k.big_method = method;
  return k;
}

// Device work of a segmented sort of the histogram-sort layouts, enqueued
// on st without waiting for the host anywhere (graph plans capture it):
// segments above k.big_above records take the whole-GPU histogram sort one
// after the other; the rest share one level-2 pipeline (the persistent
// engine by default) fed by one task per segment.  d_offs: the nseg + 1
// offsets on the device; errs: 1 + (segments sorted on their own) device
// words that receive each part's error word.  Buffers are sized once,
// before anything is enqueued.
int segments_enqueue(Context& c, const void* d_in, void* d_out, const std::vector<uint64_t>& offs,
                     const uint64_t* d_offs, uint32_t E, const gbsort_key_desc* key, const SegKnobs& k,
                     uint32_t* errs, cudaStream_t st) {
  const size_t nseg = offs.size() - 1;
  const uint32_t N = (uint32_t)offs[nseg];
  const uint32_t cap_split = (uint32_t)nseg * 2 + N / 4096 + 4096;
  const uint32_t cap_local = 4u * (uint32_t)nseg + N / 512 + 65536;
  // the largest small-buffer layout of any part, before any work is enqueued
  size_t small_need = Level2::bytes(cap_split, cap_local) + (1 << 20);
  uint32_t nbig = 0;
  for (size_t i = 0; i < nseg; ++i) {
    const uint64_t m = offs[i + 1] - offs[i];
    if (m > k.big_above) {
      ++nbig;
      small_need = std::max(small_need, hsort_small_bytes((uint32_t)m, E, k.big, hsort_grid((uint32_t)m)));
    }
  }
  GB_CUDA(c.small.ensure(small_need));
  GB_CUDA(c.A.ensure((size_t)N * E + kScratchSlack));
  // (the areas of a segment sorted on its own fit too: no growth later)
  GB_CUDA(c.B.ensure((size_t)(E >= 8 && E <= 16 && N <= kSplitAreaMaxN ? split_area(N) : N) * E + kScratchSlack));
  uint32_t bi = 0;
  uint64_t nbig_records = 0;
  for (size_t i = 0; i < nseg; ++i) {
    const uint64_t a = offs[i], m = offs[i + 1] - offs[i];
    if (m <= k.big_above) continue;
    int rc = hsort_enqueue(c, (const uint8_t*)d_in + a * E, (uint8_t*)d_out + a * E, (uint32_t)m, E, key,
                           k.big_method == GBSORT_HISTOGRAM_LEARNED, false, k.big, st);
    if (rc) return rc;
    // this part's error word, and its unfinished tasks as an error, kept before the next part
    uint32_t* cnt = c.small.as<uint32_t>();  // hsort_enqueue's counters come first in the small buffer
    GB_CUDA(require_zero(c.run_engine ? cnt + CNT_ENGINE + 2 * kEngineCtlStride : cnt + CNT_L2 + (kSplitRounds & 1),
                         cnt + CNT_ERR, st));
    GB_CUDA(cudaMemcpyAsync(errs + 1 + bi, cnt + CNT_ERR, 4, cudaMemcpyDeviceToDevice, st));
    ++bi;
    nbig_records += m;
  }
  Bump bump{c.small.as<uint8_t>()};
  uint32_t* counters = bump.take<uint32_t>(CNT_WORDS);
  uint32_t* stats = counters;
  uint32_t* err = counters + CNT_ERR;
  Level2 l2;
  l2.carve(bump, counters, cap_split, cap_local);
  GB_CUDA(cudaMemsetAsync(counters, 0, CNT_WORDS * sizeof(uint32_t), st));
  if (nbig_records < N) {
    GB_CUDA(cudaMemcpyAsync(c.A.p, d_in, (size_t)N * E, cudaMemcpyDeviceToDevice, st));
    GB_CUDA(segment_ranges(c.A.as<uint8_t>(), E, key->word[0], d_offs, (uint32_t)nseg, k.big_above, l2.split[0],
                           l2.nsplit, cap_split, err, st));
    HsortParams p{};
    p.in = (const uint8_t*)d_in;
    p.out = (uint8_t*)d_out;
    p.bufA = c.A.as<uint8_t>();
    p.bufB = c.B.as<uint8_t>();
    p.n = N;
    p.elsize = E;
    p.key = key->word[0];
    p.a_cap = N;
    const bool engine = use_engine(E, k.level2, true);
    if (engine) {
      GB_CUDA(run_engine(p, l2.round(0), l2.qtask, l2.qready, l2.qctl, l2.qcap, stats, err, st));
      GB_CUDA(require_zero(l2.qctl + 2 * kEngineCtlStride, err, st));
    } else {
      for (int r = 0; r < kSplitRounds; ++r) {
        TaskListsHost L = l2.round(r);
        GB_CUDA(cudaMemsetAsync(L.nsplit_out, 0, sizeof(uint32_t), st));
        GB_CUDA(run_split_round(p, L, l2.work, stats, err, st));
      }
      GB_CUDA(run_local(p, l2.local, l2.nlocal, l2.cap_local, l2.work, stats, st));
      GB_CUDA(require_zero(l2.nsplit + (kSplitRounds & 1), err, st));
    }
    c.run_engine = engine;
  } else {
    c.run_engine = false;
  }
  GB_CUDA(cudaMemcpyAsync(errs, err, 4, cudaMemcpyDeviceToDevice, st));
  GB_CUDA(cudaMemcpyAsync(c.hc->c, counters, CNT_WORDS * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  c.run_nbuckets = (uint32_t)nseg;
  c.run_sample = nbig;
  return GBSORT_OK;
}

// Status and statistics of a segmented sort once its stream reached the
// end: the error words (h_errs, 1 + segments sorted on their own) and the
// shared pipeline's counters.
int segments_collect(Context& c, const uint32_t* h_errs, uint32_t nerrs) {
  for (uint32_t i = 0; i < nerrs; ++i)
    if (h_errs[i]) {
      set_err("segmented sort device check failed: code %u (part %u)", h_errs[i], i);
      return GBSORT_ERR_INTERNAL;
    }
  const uint32_t* h = c.hc->c;
  g_stats = gbsort_stats{};
  g_stats.method = GBSORT_HISTOGRAM_PLAIN;
  g_stats.nbuckets = c.run_nbuckets;
  g_stats.sample = c.run_sample;  // segments sorted on their own
  g_stats.local_sorts = h[STAT_LOCAL];
  g_stats.splits = h[STAT_SPLIT];
  g_stats.copies = h[STAT_COPY];
  g_stats.resplits = h[STAT_PUSHED];
  g_stats.bigbin_passes = h[STAT_BIGBIN];
  g_stats.engine = c.run_engine ? 1u : 0u;
  g_stats.uniform_splits = h[CNT_UNIFORM] - h[CNT_UNIFORM + 1];
  g_stats.uniform_fallbacks = h[CNT_UNIFORM + 1];
  g_stats.deep_splits = h[STAT_DEEP];
  return GBSORT_OK;
}

bool segments_args_ok(const uint64_t* seg_offsets, size_t nseg) {
  if (!seg_offsets || seg_offsets[0] != 0 || seg_offsets[nseg] >= 0xffffffffull) return false;
  for (size_t i = 0; i < nseg; ++i)
    if (seg_offsets[i + 1] < seg_offsets[i]) return false;
  return true;
}

// One segmented sort from start to finish on `st` (synchronises).
int segments_run(Context& c, const void* d_in, void* d_out, const uint64_t* seg_offsets, size_t nseg, uint32_t E,
                 const gbsort_key_desc* key, const SegKnobs& k, cudaStream_t st) {
  std::vector<uint64_t> offs(seg_offsets, seg_offsets + nseg + 1);
  uint32_t nbig = 0;
  for (size_t i = 0; i < nseg; ++i) nbig += offs[i + 1] - offs[i] > k.big_above;
  GB_CUDA(c.seg.ensure((nseg + 1) * 8 + (size_t)(nbig + 1) * 4 + 256));
  uint64_t* d_offs = c.seg.as<uint64_t>();
  uint32_t* errs = reinterpret_cast<uint32_t*>(d_offs + nseg + 1);
  GB_CUDA(cudaMemcpyAsync(d_offs, offs.data(), (nseg + 1) * 8, cudaMemcpyHostToDevice, st));
  GB_CUDA(cudaMemsetAsync(errs, 0, (size_t)(nbig + 1) * 4, st));
  int rc = segments_enqueue(c, d_in, d_out, offs, d_offs, E, key, k, errs, st);
  if (rc) return rc;
  std::vector<uint32_t> h_errs(nbig + 1);
  GB_CUDA(cudaMemcpyAsync(h_errs.data(), errs, h_errs.size() * 4, cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  return segments_collect(c, h_errs.data(), nbig + 1);
}

}  // namespace

extern "C" {

int gbsort_sort_segments_device(const void* d_in, void* d_out, const uint64_t* seg_offsets, size_t nseg,
                                size_t elsize, const gbsort_key_desc* key, int method, void* stream) {
  if (nseg == 0) return GBSORT_OK;
  if (!d_in || !d_out || !segments_args_ok(seg_offsets, nseg)) return GBSORT_ERR_BAD_ARG;
  if (seg_offsets[nseg] == 0) return GBSORT_OK;
  if (!key_ok(key, elsize)) return GBSORT_ERR_BAD_ARG;
  Context* c = nullptr;
  int rc = get_ctx(&c);
  if (rc) return rc;
  std::lock_guard<std::mutex> lk(c->mu);
  cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
  const uint32_t E = (uint32_t)elsize;
  if (!hsort_layout_ok(d_in, d_out, E, key) || method == GBSORT_LSD) {
    // generic path: one LSD sort per segment
    for (size_t i = 0; i < nseg; ++i) {
      uint64_t a = seg_offsets[i], b = seg_offsets[i + 1];
      if (b == a) continue;
      rc = sort_device_locked(*c, (const uint8_t*)d_in + a * E, (uint8_t*)d_out + a * E, b - a, E, key,
                              GBSORT_LSD, st);
      if (rc) return rc;
    }
    return GBSORT_OK;
  }
  const unsigned long long l0 = launch_count();
  rc = segments_run(*c, d_in, d_out, seg_offsets, nseg, E, key, seg_knobs(E, key, seg_offsets[nseg], method), st);
  if (rc == GBSORT_OK) g_stats.launches = (uint32_t)(launch_count() - l0);
  return rc;
}

int gbsort_autotune_segments(const uint64_t* seg_offsets, size_t nseg, size_t elsize, const gbsort_key_desc* key,
                             const void* d_records, gbsort_tuning* best) {
  if (!best || nseg == 0 || !segments_args_ok(seg_offsets, nseg) || seg_offsets[nseg] == 0 ||
      !key_ok(key, elsize) || key->nwords != 1)
    return GBSORT_ERR_BAD_ARG;
  Context* c = nullptr;
  int rc = get_ctx(&c);
  if (rc) return rc;
  std::lock_guard<std::mutex> lk(c->mu);
  cudaStream_t st = c->stream;
  const uint32_t E = (uint32_t)elsize;
  const uint64_t n = seg_offsets[nseg];
  const size_t bytes = (size_t)n * E;
  GB_CUDA(c->hout.ensure(bytes));
  const void* in = d_records;
  if (!in) {
    GB_CUDA(c->hin.ensure(bytes));
    GB_CUDA(fill_hash(c->hin.p, bytes, 0x5eed5eedull, st));
    in = c->hin.p;
  }
  if (!hsort_layout_ok(in, c->hout.p, E, key)) {
    set_err("segment tuning needs a histogram-sort layout");
    return GBSORT_ERR_UNSUPPORTED;
  }
  uint64_t largest = 0;
  for (size_t i = 0; i < nseg; ++i) largest = std::max(largest, seg_offsets[i + 1] - seg_offsets[i]);
  gbsort_tuning win{};
  win.ms = -1.f;
  for (int level2 : {GBSORT_LEVEL2_ROUNDS, GBSORT_LEVEL2_ENGINE}) {
    if (level2 == GBSORT_LEVEL2_ENGINE && !engine_supported(E)) continue;
    for (uint64_t above : {(uint64_t)1 << 20, (uint64_t)1 << 22, largest}) {
      SegKnobs k;
      k.level2 = level2;
      k.big_above = std::max<uint64_t>(above, 4096);
      float best_ms = -1.f;
      for (int rep = 0; rep < 3; ++rep) {  // a warm-up, then the best of two
        GB_CUDA(cudaEventRecord(c->ev[7], st));
        const int r = segments_run(*c, in, c->hout.p, seg_offsets, nseg, E, key, k, st);
        if (r) return r;
        GB_CUDA(cudaEventRecord(c->ev[6], st));
        GB_CUDA(cudaEventSynchronize(c->ev[6]));
        float ms = 0.f;
        GB_CUDA(cudaEventElapsedTime(&ms, c->ev[7], c->ev[6]));
        if (rep > 0 && (best_ms < 0.f || ms < best_ms)) best_ms = ms;
      }
      if (win.ms < 0.f || best_ms < win.ms) {
        win.method = GBSORT_HISTOGRAM_LEARNED;
        win.max_buckets = 0;
        win.level2 = (uint32_t)level2;
        win.reserved[0] = (uint32_t)std::min<uint64_t>(k.big_above, 0xffffffffull);
        win.ms = best_ms;
      }
    }
  }
  *best = win;
  std::lock_guard<std::mutex> tl(g_tune_mu);
  g_tune[seg_tune_key(E, key->word[0].width, n)] = win;
  return GBSORT_OK;
}

int gbsort_merge_join_device(const void* d_a, size_t na, const void* d_b, size_t nb, size_t elsize,
                             const gbsort_key_desc* key, uint64_t* d_pairs_a, uint64_t* d_pairs_b, uint64_t* d_npairs,
                             void* stream) {
  if (!d_npairs || !key_ok(key, elsize) || key->nwords != 1 || key->word[0].offset % 4 || elsize % 4)
    return GBSORT_ERR_BAD_ARG;
  if (na >= 0xffffffffull || nb >= 0xffffffffull) return GBSORT_ERR_BAD_ARG;
  Context* c = nullptr;
  int rc = get_ctx(&c);
  if (rc) return rc;
  std::lock_guard<std::mutex> lk(c->mu);
  cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
  if (na == 0 || nb == 0) {
    GB_CUDA(cudaMemsetAsync(d_npairs, 0, 8, st));
    return GBSORT_OK;
  }
  const int g = join_grid((uint32_t)na);
  GB_CUDA(c->small.ensure((size_t)g * 8 + (1 << 20)));
  Bump bump{c->small.as<uint8_t>()};
  uint32_t* counts = bump.take<uint32_t>(g + 1);
  uint32_t* tmp = bump.take<uint32_t>(scan_tmp_words(g + 1));
  GB_CUDA(join_count((const uint8_t*)d_a, (uint32_t)na, (const uint8_t*)d_b, (uint32_t)nb, (uint32_t)elsize,
                     key->word[0], counts, g, st));
  GB_CUDA(exclusive_scan_u32(counts, counts, (size_t)g + 1, tmp, st));
  GB_CUDA(join_write((const uint8_t*)d_a, (uint32_t)na, (const uint8_t*)d_b, (uint32_t)nb, (uint32_t)elsize,
                     key->word[0], counts, g, d_pairs_a, d_pairs_b, d_npairs, st));
  return GBSORT_OK;
}

int gbsort_cdf_forward_backward(const uint64_t* x, uint32_t s, uint64_t kmin, uint64_t kmax, int lbits,
                                const float* y, float* loss, float* pred, float* grad) {
  if (!x || !y || s == 0 || lbits < 0 || lbits > 16) return GBSORT_ERR_BAD_ARG;
  Context* c = nullptr;
  int rc = get_ctx(&c);
  if (rc) return rc;
  std::lock_guard<std::mutex> lk(c->mu);
  const int nk = (1 << lbits) + 1;
  GB_CUDA(c->small.ensure((size_t)s * 12 + (size_t)nk * 8 + (1 << 16)));
  Bump bump{c->small.as<uint8_t>()};
  uint64_t* dx = bump.take<uint64_t>(s);
  float* dy = bump.take<float>(nk);
  float* dg = bump.take<float>(nk);
  float* dp = bump.take<float>(s);
  float* dl = bump.take<float>(1);
  cudaStream_t st = c->stream;
  GB_CUDA(cudaMemcpyAsync(dx, x, (size_t)s * 8, cudaMemcpyHostToDevice, st));
  GB_CUDA(cudaMemcpyAsync(dy, y, (size_t)nk * 4, cudaMemcpyHostToDevice, st));
  CdfShape sh = cdf_shape(kmin, kmax, lbits);
  GB_CUDA(cdf_forward(dx, s, sh, dy, dp, dl, st));
  GB_CUDA(cdf_backward(dx, s, sh, dy, dg, st));
  if (loss) GB_CUDA(cudaMemcpyAsync(loss, dl, 4, cudaMemcpyDeviceToHost, st));
  if (pred) GB_CUDA(cudaMemcpyAsync(pred, dp, (size_t)s * 4, cudaMemcpyDeviceToHost, st));
  if (grad) GB_CUDA(cudaMemcpyAsync(grad, dg, (size_t)nk * 4, cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  return GBSORT_OK;
}

int gbsort_cdf_train_gradient(const uint64_t* x, uint32_t s, uint64_t kmin, uint64_t kmax, int lbits,
                              const float* y, float* grad) {
  if (!x || !y || !grad || s == 0 || lbits < 0 || lbits > 13) return GBSORT_ERR_BAD_ARG;
  Context* c = nullptr;
  int rc = get_ctx(&c);
  if (rc) return rc;
  std::lock_guard<std::mutex> lk(c->mu);
  const int nk = (1 << lbits) + 1;
  GB_CUDA(c->small.ensure((size_t)s * 8 + (size_t)nk * 24 + (1 << 16)));
  Bump bump{c->small.as<uint8_t>()};
  uint64_t* dx = bump.take<uint64_t>(s);
  float* dy = bump.take<float>(nk);
  float* dg = bump.take<float>(nk);
  CdfWork w{};
  w.h = bump.take<float>(nk);
  w.off = bump.take<float>(nk);
  w.grad = bump.take<float>(nk);
  cudaStream_t st = c->stream;
  GB_CUDA(cudaMemcpyAsync(dx, x, (size_t)s * 8, cudaMemcpyHostToDevice, st));
  GB_CUDA(cudaMemcpyAsync(dy, y, (size_t)nk * 4, cudaMemcpyHostToDevice, st));
  GB_CUDA(cdf_train_gradient(dx, s, cdf_shape(kmin, kmax, lbits), dy, dg, w, st));
  GB_CUDA(cudaMemcpyAsync(grad, dg, (size_t)nk * 4, cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  return GBSORT_OK;
}

int gbsort_debug_bisect(const uint64_t* sorted, uint32_t s, int nsplit, uint64_t* splitters, int64_t* clt,
                        int64_t* cle, uint32_t* rounds) {
  if (!sorted || s == 0 || nsplit <= 0) return GBSORT_ERR_BAD_ARG;
  Context* c = nullptr;
  int rc = get_ctx(&c);
  if (rc) return rc;
  std::lock_guard<std::mutex> lk(c->mu);
  GB_CUDA(c->small.ensure((size_t)s * 8 + (size_t)nsplit * 24 + (1 << 16)));
  Bump bump{c->small.as<uint8_t>()};
  uint64_t* dx = bump.take<uint64_t>(s);
  uint64_t* dS = bump.take<uint64_t>(nsplit);
  int64_t* dlt = bump.take<int64_t>(nsplit);
  int64_t* dle = bump.take<int64_t>(nsplit);
  uint32_t* dit = bump.take<uint32_t>(1);
  cudaStream_t st = c->stream;
  GB_CUDA(cudaMemcpyAsync(dx, sorted, (size_t)s * 8, cudaMemcpyHostToDevice, st));
  GB_CUDA(plain_splitters(dx, s, nsplit, dS, dit, dlt, dle, st));
  GB_CUDA(cudaMemcpyAsync(splitters, dS, (size_t)nsplit * 8, cudaMemcpyDeviceToHost, st));
  if (clt) GB_CUDA(cudaMemcpyAsync(clt, dlt, (size_t)nsplit * 8, cudaMemcpyDeviceToHost, st));
  if (cle) GB_CUDA(cudaMemcpyAsync(cle, dle, (size_t)nsplit * 8, cudaMemcpyDeviceToHost, st));
  if (rounds) GB_CUDA(cudaMemcpyAsync(rounds, dit, 4, cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  return GBSORT_OK;
}

int gbsort_debug_lookback(uint32_t n, uint32_t withhold_tile, uint32_t spin_limit) {
  if (n == 0 || spin_limit == 0) return GBSORT_ERR_BAD_ARG;
  Context* c = nullptr;
  int rc = get_ctx(&c);
  if (rc) return rc;
  std::lock_guard<std::mutex> lk(c->mu);
  GB_CUDA(c->small.ensure((size_t)n * 16 + lsd_scratch_bytes(n, 1) + (1 << 16)));
  Bump bump{c->small.as<uint8_t>()};
  uint32_t* counters = bump.take<uint32_t>(CNT_WORDS);
  uint64_t* kin = bump.take<uint64_t>(n);
  uint64_t* kout = bump.take<uint64_t>(n);
  uint32_t* hist = bump.take<uint32_t>(8 * 256);
  uint32_t* starts = bump.take<uint32_t>(8 * 256);
  unsigned long long* status = bump.take<unsigned long long>((size_t)lsd_tiles(n) * 256 + 1);
  uint32_t* ticket = reinterpret_cast<uint32_t*>(status + (size_t)lsd_tiles(n) * 256);
  uint32_t* err = counters + CNT_ERR;
  cudaStream_t st = c->stream;
  GB_CUDA(cudaMemsetAsync(counters, 0, CNT_WORDS * sizeof(uint32_t), st));
  GB_CUDA(fill_hash(kin, (size_t)n * 8, 0x10cbac4ull, st));
  GB_CUDA(lsd_digit_histograms(kin, n, 1, hist, st));
  GB_CUDA(lsd_digit_starts(hist, 1, starts, st));
  GB_CUDA(lsd_onesweep(kin, nullptr, kout, nullptr, n, 1, 0, 0, starts, status, ticket, err, st, spin_limit,
                       withhold_tile));
  uint32_t herr = 0;
  GB_CUDA(cudaMemcpyAsync(&herr, err, 4, cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  if (herr == DEV_ERR_TIMEOUT) {
    set_err("a look-back wait gave up after %u polls (device code %u)", spin_limit, herr);
    return GBSORT_ERR_INTERNAL;
  }
  if (herr) {
    set_err("device check failed: code %u", herr);
    return GBSORT_ERR_INTERNAL;
  }
  return GBSORT_OK;
}

namespace {
// Trains the model on the sample for `epochs` steps and looks every key up
// with the model (window search) and with the full search; see
// gbsort_debug_buckets and gbsort_debug_model.
int debug_model(const uint64_t* sample, uint32_t s, int nbuckets, int epochs, const uint64_t* keys, uint32_t nkeys,
                uint32_t* bucket_search, uint32_t* bucket_learned, uint64_t* splitters, uint32_t* widest_window,
                float* loss, uint64_t* reads) {
  if (!sample || s == 0 || nbuckets < 2 || nbuckets > 8192 || !keys || epochs < 0 || epochs > 1000)
    return GBSORT_ERR_BAD_ARG;
  Context* c = nullptr;
  int rc = get_ctx(&c);
  if (rc) return rc;
  std::lock_guard<std::mutex> lk(c->mu);
  const int lbits = 11, nleaf = 1 << lbits;
  GB_CUDA(c->small.ensure((size_t)s * 8 + (size_t)nkeys * 16 + (size_t)nbuckets * 8 + (size_t)nleaf * 64 +
                          (1 << 20)));
  Bump bump{c->small.as<uint8_t>()};
  uint64_t* dx = bump.take<uint64_t>(s);
  uint64_t* dk = bump.take<uint64_t>(nkeys);
  uint32_t* dl = bump.take<uint32_t>(nkeys);
  uint32_t* ds = bump.take<uint32_t>(nkeys);
  uint64_t* S = bump.take<uint64_t>(nbuckets);
  uint32_t* misc = bump.take<uint32_t>(4);
  unsigned long long* dreads = bump.take<unsigned long long>(2);
  CdfWork w{};
  w.y = bump.take<float>(nleaf + 1);
  w.grad = bump.take<float>(nleaf + 1);
  w.h = bump.take<float>(nleaf + 1);
  w.off = bump.take<float>(nleaf + 1);
  w.knots = bump.take<float2>(nleaf);
  w.loss = bump.take<float>(1);
  uint32_t* win = bump.take<uint32_t>(nleaf);
  uint32_t* wlo = bump.take<uint32_t>(nleaf);
  uint32_t* whi = bump.take<uint32_t>(nleaf);
  cudaStream_t st = c->stream;
  std::vector<uint64_t> hs(sample, sample + s);
  std::sort(hs.begin(), hs.end());
  GB_CUDA(cudaMemcpyAsync(dx, hs.data(), (size_t)s * 8, cudaMemcpyHostToDevice, st));
  GB_CUDA(cudaMemcpyAsync(dk, keys, (size_t)nkeys * 8, cudaMemcpyHostToDevice, st));
  GB_CUDA(cudaMemsetAsync(misc, 0, 16, st));
  GB_CUDA(cudaMemsetAsync(dreads, 0, 16, st));
  CdfShape sh = cdf_shape(hs.front(), hs.back(), lbits);
  GB_CUDA(cdf_train(dx, s, sh, epochs, 0.5f, w, st));
  GB_CUDA(cdf_splitters(dx, s, sh, nbuckets, w.knots, S, st));
  GB_CUDA(finalize_splitters(S, nbuckets - 1, st));
  GB_CUDA(cdf_windows(sh, nbuckets, w.knots, S, win, wlo, whi, misc, st));
  ModelDev m{};
  m.kmin = sh.kmin;
  m.lshift = sh.lshift;
  m.lbits = sh.lbits;
  m.nbuckets = nbuckets;
  m.knots = w.knots;
  m.win = win;
  GB_CUDA(probe_buckets(dk, nkeys, S, &m, dl, ds, misc + 1, dreads, st));
  if (bucket_learned) GB_CUDA(cudaMemcpyAsync(bucket_learned, dl, (size_t)nkeys * 4, cudaMemcpyDeviceToHost, st));
  if (bucket_search) GB_CUDA(cudaMemcpyAsync(bucket_search, ds, (size_t)nkeys * 4, cudaMemcpyDeviceToHost, st));
  if (splitters) GB_CUDA(cudaMemcpyAsync(splitters, S, (size_t)(nbuckets - 1) * 8, cudaMemcpyDeviceToHost, st));
  uint32_t hm[2] = {0, 0};
  unsigned long long hr[2] = {0, 0};
  float hl = 0.f;
  GB_CUDA(cudaMemcpyAsync(hm, misc, 8, cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaMemcpyAsync(hr, dreads, 16, cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaMemcpyAsync(&hl, w.loss, 4, cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  if (widest_window) *widest_window = hm[0];
  if (loss) *loss = hl;
  if (reads) {
    reads[0] = hr[0];
    reads[1] = hr[1];
  }
  g_stats.window_misses = hm[1];
  return GBSORT_OK;
}
}  // namespace

int gbsort_debug_buckets(const uint64_t* sample, uint32_t s, int nbuckets, const uint64_t* keys, uint32_t nkeys,
                         uint32_t* bucket_search, uint32_t* bucket_learned, uint64_t* splitters,
                         uint32_t* widest_window) {
  return debug_model(sample, s, nbuckets, 8, keys, nkeys, bucket_search, bucket_learned, splitters, widest_window,
                     nullptr, nullptr);
}

int gbsort_debug_model(const uint64_t* sample, uint32_t s, int nbuckets, int epochs, const uint64_t* keys,
                       uint32_t nkeys, uint32_t* bucket_search, uint32_t* bucket_learned, float* loss,
                       uint64_t* reads, uint32_t* widest_window) {
  return debug_model(sample, s, nbuckets, epochs, keys, nkeys, bucket_search, bucket_learned, nullptr,
                     widest_window, loss, reads);
}

int gbsort_last_stats(gbsort_stats* out) {
  if (!out) return GBSORT_ERR_BAD_ARG;
  *out = g_stats;
  return GBSORT_OK;
}

const char* gbsort_status_string(int status) {
  switch (status) {
    case GBSORT_OK: return "ok";
    case GBSORT_ERR_BAD_ARG: return "bad argument";
    case GBSORT_ERR_OOM: return "out of memory";
    case GBSORT_ERR_CUDA: return "CUDA error";
    case GBSORT_ERR_NO_DEVICE: return "no CUDA device";
    case GBSORT_ERR_INTERNAL: return "device consistency check failed";
    case GBSORT_ERR_UNSUPPORTED: return "unsupported layout for this method";
    default: return "unknown status";
  }
}

const char* gbsort_last_error(void) { return g_err; }

int gbsort_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

int gbsort_release(void) {
  Context* c = nullptr;
  int rc = get_ctx(&c);
  if (rc) return rc;
  std::lock_guard<std::mutex> lk(c->mu);
  cudaStreamSynchronize(c->stream);
  DevBuf* bufs[] = {&c->A, &c->B, &c->hin, &c->hout, &c->keysA, &c->keysB, &c->idxA, &c->idxB, &c->small, &c->radix,
                    &c->part, &c->vh, &c->seg};
  for (DevBuf* b : bufs) b->release();
  return GBSORT_OK;
}

const char* gbsort_version(void) { return "gbsort 0.1.0 (sm_103a)"; }

// ----------------------------------------------------------- autotuner --
int gbsort_autotune(size_t nmemb, size_t elsize, const gbsort_key_desc* key, const void* d_records,
                    gbsort_tuning* best) {
  if (!best || nmemb < 2 || nmemb >= 0xffffffffull || elsize == 0 || elsize > (1u << 20) || !key_ok(key, elsize))
    return GBSORT_ERR_BAD_ARG;
  Context* c = nullptr;
  int rc = get_ctx(&c);
  if (rc) return rc;
  std::lock_guard<std::mutex> lk(c->mu);
  cudaStream_t st = c->stream;
  const uint32_t n = (uint32_t)nmemb, E = (uint32_t)elsize;
  const size_t bytes = (size_t)n * E;
  // inputs: the caller's records, or pseudo-random ones; the sorts write to
  // the host-staging buffer so the caller's data is never modified
  GB_CUDA(c->hout.ensure(bytes));
  const void* in = d_records;
  if (!in) {
    GB_CUDA(c->hin.ensure(bytes));
    GB_CUDA(fill_hash(c->hin.p, bytes, 0x5eed5eedull, st));
    in = c->hin.p;
  }
  void* out = c->hout.p;
  const bool hs_ok = hsort_layout_ok(in, out, E, key);
  struct Cand {
    int method;
    int cap;
    int level2;
  };
  std::vector<Cand> cands;
  cands.push_back({GBSORT_LSD, 0, GBSORT_LEVEL2_DEFAULT});
  if (hs_ok)
    for (int m : {GBSORT_HISTOGRAM_LEARNED, GBSORT_HISTOGRAM_PLAIN})
      for (int cap : {512, 1024, 2048, 4096}) {
        cands.push_back({m, cap, GBSORT_LEVEL2_ROUNDS});
        if (engine_supported(E)) cands.push_back({m, cap, GBSORT_LEVEL2_ENGINE});
      }
  gbsort_tuning win{};
  win.ms = -1.f;
  for (const Cand& cd : cands) {
    Knobs k;
    k.max_buckets = cd.cap;
    k.level2 = cd.level2;
    float ms_best = -1.f;
    for (int rep = 0; rep < 3; ++rep) {  // a warm-up, then the best of two
      GB_CUDA(cudaEventRecord(c->ev[7], st));
      int r = cd.method == GBSORT_LSD ? run_lsd(*c, in, out, n, E, key, nullptr, 0, st)
                                      : run_hsort(*c, in, out, n, E, key, cd.method, k, st);
      if (r) {
        ms_best = -1.f;
        break;
      }
      // run_* returned after synchronising, so the end event is already due
      GB_CUDA(cudaEventRecord(c->ev[6], st));
      GB_CUDA(cudaEventSynchronize(c->ev[6]));
      float ms = 0.f;
      GB_CUDA(cudaEventElapsedTime(&ms, c->ev[7], c->ev[6]));
      if (rep > 0 && (ms_best < 0.f || ms < ms_best)) ms_best = ms;
    }
    if (ms_best >= 0.f && (win.ms < 0.f || ms_best < win.ms)) {
      win.method = cd.method;
      win.max_buckets = (uint32_t)cd.cap;
      win.sample_per_bucket = 0;
      win.level2 = (uint32_t)cd.level2;
      win.ms = ms_best;
    }
  }
  if (win.ms < 0.f) {
    set_err("autotune: no candidate ran");
    return GBSORT_ERR_INTERNAL;
  }
  *best = win;
  if (key->nwords == 1) {
    std::lock_guard<std::mutex> tl(g_tune_mu);
    g_tune[tune_key(E, key->word[0].width, size_class(n))] = win;
  }
  return GBSORT_OK;
}

int gbsort_tuning_set(size_t nmemb, size_t elsize, const gbsort_key_desc* key, const gbsort_tuning* t) {
  if (!t || !key_ok(key, elsize) || key->nwords != 1 || !tuning_ok(*t)) return GBSORT_ERR_BAD_ARG;
  std::lock_guard<std::mutex> tl(g_tune_mu);
  g_tune[tune_key((uint32_t)elsize, key->word[0].width, size_class(nmemb))] = *t;
  return GBSORT_OK;
}

int gbsort_tuning_get(size_t nmemb, size_t elsize, const gbsort_key_desc* key, gbsort_tuning* t) {
  if (!t || !key_ok(key, elsize)) return GBSORT_ERR_BAD_ARG;
  if (key->nwords != 1 || !tune_lookup((uint32_t)elsize, key->word[0].width, nmemb, t)) return GBSORT_ERR_UNSUPPORTED;
  return GBSORT_OK;
}

int gbsort_tuning_get_segments(size_t nmemb, size_t elsize, const gbsort_key_desc* key, gbsort_tuning* t) {
  if (!t || !key_ok(key, elsize)) return GBSORT_ERR_BAD_ARG;
  if (key->nwords != 1) return GBSORT_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> tl(g_tune_mu);
  auto it = g_tune.find(seg_tune_key((uint32_t)elsize, key->word[0].width, nmemb));
  if (it == g_tune.end()) return GBSORT_ERR_UNSUPPORTED;
  *t = it->second;
  return GBSORT_OK;
}

int gbsort_tuning_clear(void) {
  std::lock_guard<std::mutex> tl(g_tune_mu);
  g_tune.clear();
  return GBSORT_OK;
}

// One line per entry: elsize width class method max_buckets sample_per_bucket ms
int gbsort_tuning_save(const char* path) {
  if (!path) return GBSORT_ERR_BAD_ARG;
  FILE* f = fopen(path, "w");
  if (!f) {
    set_err("cannot write %s", path);
    return GBSORT_ERR_BAD_ARG;
  }
  std::lock_guard<std::mutex> tl(g_tune_mu);
  fprintf(f, "# gbsort tuning: elsize key_width size_class method max_buckets sample_per_bucket ms level2 "
             "big_above (size_class + 128: segmented sorts)\n");
  for (const auto& kv : g_tune)
    fprintf(f, "%u %u %u %d %u %u %.4f %u %u\n", (unsigned)(kv.first >> 16), (unsigned)((kv.first >> 8) & 0xff),
            (unsigned)(kv.first & 0xff), kv.second.method, kv.second.max_buckets, kv.second.sample_per_bucket,
            kv.second.ms, kv.second.level2, kv.second.reserved[0]);
  fclose(f);
  return GBSORT_OK;
}

int gbsort_tuning_load(const char* path) {
  if (!path) return GBSORT_ERR_BAD_ARG;
  FILE* f = fopen(path, "r");
  if (!f) {
    set_err("cannot read %s", path);
    return GBSORT_ERR_BAD_ARG;
  }
  char line[256];
  std::map<uint64_t, gbsort_tuning> loaded;
  int rc = GBSORT_OK;
  while (fgets(line, sizeof line, f)) {
    if (line[0] == '#' || line[0] == '\n') continue;
    unsigned el, wd, cls, mb, spb, l2 = 0, big = 0;
    int m;
    float ms;
    const int got = sscanf(line, "%u %u %u %d %u %u %f %u %u", &el, &wd, &cls, &m, &mb, &spb, &ms, &l2, &big);
    if (got < 7 || (wd != 4 && wd != 8) || (cls & 0x7f) > 64 || cls > 0xff || el == 0 || el > (1u << 20)) {
      rc = GBSORT_ERR_BAD_ARG;
      break;
    }
    gbsort_tuning t{};
    t.method = m;
    t.max_buckets = mb;
    t.sample_per_bucket = spb;
    t.level2 = l2;
    t.ms = ms;
    t.reserved[0] = big;
    if (!tuning_ok(t)) {
      rc = GBSORT_ERR_BAD_ARG;
      break;
    }
    loaded[tune_key(el, wd, cls)] = t;
  }
  fclose(f);
  if (rc) {
    set_err("malformed tuning file %s", path);
    return rc;
  }
  std::lock_guard<std::mutex> tl(g_tune_mu);
  for (const auto& kv : loaded) g_tune[kv.first] = kv.second;
  return GBSORT_OK;
}

// ------------------------------------------------------- graph plans ----
struct gbsort_plan {
  Context ctx;                       // the plan's own scratch, counters and capture stream
  size_t nmemb = 0, elsize = 0;
  gbsort_key_desc key{};
  int method = GBSORT_AUTO;          // as requested; resolved per capture
  int resolved = GBSORT_AUTO;
  const void* in = nullptr;          // buffers the graph was captured with
  void* out = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaEvent_t done = nullptr;
  uint32_t kernels = 0;              // kernel launches in the graph
  bool pending = false;
  // segmented plans: the segment offsets (their device copy sits at the
  // front of ctx.seg, the error words after it) and the pinned host copy of
  // the error words
  std::vector<uint64_t> segs;
  uint32_t nerrs = 0;
  uint32_t* herrs = nullptr;
};

static int plan_new(gbsort_plan** plan, size_t nmemb, size_t elsize, const gbsort_key_desc* key, int method) {
  Context* probe = nullptr;
  int rc = get_ctx(&probe);  // checks for a device
  if (rc) return rc;
  gbsort_plan* p = new gbsort_plan();
  rc = ctx_init(p->ctx, probe->device, false);
  if (rc == GBSORT_OK && cudaEventCreateWithFlags(&p->done, cudaEventDisableTiming) != cudaSuccess) {
    cudaGetLastError();
    rc = GBSORT_ERR_CUDA;
  }
  if (rc) {
    ctx_destroy(p->ctx);
    delete p;
    return rc;
  }
  p->nmemb = nmemb;
  p->elsize = elsize;
  p->key = *key;
  p->method = method;
  *plan = p;
  return GBSORT_OK;
}

int gbsort_plan_create(gbsort_plan** plan, size_t nmemb, size_t elsize, const gbsort_key_desc* key, int method) {
  if (!plan) return GBSORT_ERR_BAD_ARG;
  *plan = nullptr;
  if (nmemb == 0 || nmemb >= 0xffffffffull || elsize == 0 || elsize > (1u << 20) || !key_ok(key, elsize) ||
      method < GBSORT_AUTO || method > GBSORT_LSD) {
    set_err("bad plan arguments");
    return GBSORT_ERR_BAD_ARG;
  }
  return plan_new(plan, nmemb, elsize, key, method);
}

int gbsort_plan_create_segments(gbsort_plan** plan, const uint64_t* seg_offsets, size_t nseg, size_t elsize,
                                const gbsort_key_desc* key, int method) {
  if (!plan) return GBSORT_ERR_BAD_ARG;
  *plan = nullptr;
  if (nseg == 0 || !segments_args_ok(seg_offsets, nseg) || seg_offsets[nseg] == 0 || elsize == 0 ||
      elsize > (1u << 20) || !key_ok(key, elsize) || key->nwords != 1 ||
      (method != GBSORT_AUTO && method != GBSORT_HISTOGRAM_PLAIN && method != GBSORT_HISTOGRAM_LEARNED)) {
    set_err("bad segmented plan arguments");
    return GBSORT_ERR_BAD_ARG;
  }
  int rc = plan_new(plan, seg_offsets[nseg], elsize, key, method);
  if (rc) return rc;
  gbsort_plan* p = *plan;
  p->segs.assign(seg_offsets, seg_offsets + nseg + 1);
  // one error word for the shared pipeline and one per segment that may be
  // sorted on its own (any segment above 4096 records, whatever the tuning)
  uint32_t nbig = 0;
  for (size_t i = 0; i < nseg; ++i) nbig += seg_offsets[i + 1] - seg_offsets[i] > 4096;
  p->nerrs = nbig + 1;
  Context& c = p->ctx;
  if (c.seg.ensure((nseg + 1) * 8 + (size_t)p->nerrs * 4 + 256) != cudaSuccess ||
      cudaMallocHost(&p->herrs, (size_t)p->nerrs * 4) != cudaSuccess ||
      cudaMemcpy(c.seg.p, p->segs.data(), (nseg + 1) * 8, cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaGetLastError();
    gbsort_plan_destroy(p);
    *plan = nullptr;
    set_err("segmented plan set-up failed");
    return GBSORT_ERR_CUDA;
  }
  return GBSORT_OK;
}

constexpr int kResolvedSegments = -1;  // gbsort_plan::resolved of a segmented plan

// Captures the pipeline for (in, out) into the plan's graph.
static int plan_capture(gbsort_plan* p, const void* in, void* out) {
  Context& c = p->ctx;
  const uint32_t n = (uint32_t)p->nmemb, E = (uint32_t)p->elsize;
  const bool hs_ok = hsort_layout_ok(in, out, E, &p->key);
  Knobs knobs;
  int m;
  SegKnobs sk;
  if (!p->segs.empty()) {
    m = kResolvedSegments;
    sk = seg_knobs(E, &p->key, n, p->method);
    sk.big_above = std::max<uint64_t>(sk.big_above, 4096);  // the plan holds error words for these
  } else {
    m = p->method == GBSORT_AUTO ? resolve_auto(E, &p->key, n, hs_ok, &knobs) : p->method;
  }
  if (m != GBSORT_LSD && !hs_ok) {
    set_err("histogram sort needs a one-word key at a 4-byte offset and a record size of 8-64 bytes");
    return GBSORT_ERR_UNSUPPORTED;
  }
  // relaxed capture: buffer growth (cudaMalloc) may happen while capturing
  GB_CUDA(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeRelaxed));
  const unsigned long long l0 = launch_count();
  int rc;
  if (m == kResolvedSegments) {
    const uint64_t* d_offs = c.seg.as<uint64_t>();
    uint32_t* errs = reinterpret_cast<uint32_t*>(c.seg.as<uint64_t>() + p->segs.size());
    rc = cudaMemsetAsync(errs, 0, (size_t)p->nerrs * 4, c.stream) == cudaSuccess ? GBSORT_OK : GBSORT_ERR_CUDA;
    if (!rc) rc = segments_enqueue(c, in, out, p->segs, d_offs, E, &p->key, sk, errs, c.stream);
    if (!rc && cudaMemcpyAsync(p->herrs, errs, (size_t)p->nerrs * 4, cudaMemcpyDeviceToHost, c.stream) != cudaSuccess)
      rc = GBSORT_ERR_CUDA;
  } else {
    rc = m == GBSORT_LSD ? lsd_enqueue(c, in, out, n, E, &p->key, nullptr, 0, false, c.stream)
                         : hsort_enqueue(c, in, out, n, E, &p->key, m == GBSORT_HISTOGRAM_LEARNED, false, knobs,
                                         c.stream);
  }
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(c.stream, &g);
  if (rc || e != cudaSuccess) {
    cudaGetLastError();
    if (g) cudaGraphDestroy(g);
    if (!rc) set_err("graph capture failed: %s", cudaGetErrorString(e));
    return rc ? rc : GBSORT_ERR_CUDA;
  }
  p->kernels = (uint32_t)(launch_count() - l0);
  if (p->exec) {
    cudaGraphExecUpdateResultInfo info;
    if (cudaGraphExecUpdate(p->exec, g, &info) != cudaSuccess) {
      cudaGetLastError();
      cudaGraphExecDestroy(p->exec);
      p->exec = nullptr;
    }
  }
  if (!p->exec) {
    e = cudaGraphInstantiate(&p->exec, g, 0);
    if (e != cudaSuccess) {
      cudaGetLastError();
      cudaGraphDestroy(g);
      p->exec = nullptr;
      set_err("graph instantiation failed: %s", cudaGetErrorString(e));
      return GBSORT_ERR_CUDA;
    }
  }
  if (p->graph) cudaGraphDestroy(p->graph);
  p->graph = g;
  p->in = in;
  p->out = out;
  p->resolved = m;
  return GBSORT_OK;
}

int gbsort_plan_sort(gbsort_plan* p, const void* d_in, void* d_out, void* stream) {
  if (!p || !d_in || !d_out) return GBSORT_ERR_BAD_ARG;
  if (p->pending) {  // the previous launch must be collected first
    int rc = gbsort_plan_wait(p);
    if (rc) return rc;
  }
  if (!p->exec || d_in != p->in || d_out != p->out) {
    int rc = plan_capture(p, d_in, d_out);
    if (rc) return rc;
  }
  cudaStream_t st = stream ? (cudaStream_t)stream : p->ctx.stream;
  GB_CUDA(cudaGraphLaunch(p->exec, st));
  GB_CUDA(cudaEventRecord(p->done, st));
  note_launches(p->kernels);
  p->pending = true;
  return GBSORT_OK;
}

int gbsort_plan_wait(gbsort_plan* p) {
  if (!p) return GBSORT_ERR_BAD_ARG;
  if (!p->pending) return GBSORT_OK;
  p->pending = false;
  GB_CUDA(cudaEventSynchronize(p->done));
  int rc = p->resolved == kResolvedSegments ? segments_collect(p->ctx, p->herrs, p->nerrs)
           : p->resolved == GBSORT_LSD       ? lsd_collect(p->ctx)
                                             : hsort_collect(p->ctx);
  if (rc == GBSORT_OK) g_stats.launches = p->kernels;
  return rc;
}

int gbsort_plan_destroy(gbsort_plan* p) {
  if (!p) return GBSORT_OK;
  if (p->pending) cudaEventSynchronize(p->done);
  if (p->exec) cudaGraphExecDestroy(p->exec);
  if (p->graph) cudaGraphDestroy(p->graph);
  if (p->done) cudaEventDestroy(p->done);
  if (p->herrs) cudaFreeHost(p->herrs);
  ctx_destroy(p->ctx);
  delete p;
  return GBSORT_OK;
}

// ---------------------------------------------------------- drop-ins ----
void mpsort_radix_desc(const void* ptr, void* radix, void* arg) {
  const gbsort_key_desc* d = (const gbsort_key_desc*)arg;
  const uint8_t* rec = (const uint8_t*)ptr;
  uint8_t* out = (uint8_t*)radix;
  for (uint32_t i = 0; i < d->nwords; ++i) {
    const gbsort_key_word& w = d->word[i];
    uint64_t v;
    if (w.width == 8) {
      memcpy(&v, rec + w.offset, 8);
      if (w.is_signed) v += 0x8000000000000000ull;
    } else {
      uint32_t u;
      memcpy(&u, rec + w.offset, 4);
      v = w.is_signed ? (uint64_t)(int64_t)(int32_t)u + 0x8000000000000000ull : (uint64_t)u;
    }
    memcpy(out + 8 * i, &v, 8);
  }
}

static void dropin_sort(void* base, size_t nmemb, size_t size, void (*radix)(const void*, void*, void*),
                        size_t rsize, void* arg, const char* who) {
  int rc;
  if (nmemb == 0) {
    g_mpsort_status = GBSORT_OK;
    return;
  }
  if (radix == mpsort_radix_desc) {
    const gbsort_key_desc* d = (const gbsort_key_desc*)arg;
    if (!d || rsize != 8u * d->nwords) rc = GBSORT_ERR_BAD_ARG;
    else rc = gbsort_sort_host(base, base, nmemb, size, d, GBSORT_AUTO);
  } else {
    rc = gbsort_sort_radix_host(base, nmemb, size, radix, rsize, arg);
  }
  g_mpsort_status = rc;
  if (rc != GBSORT_OK)
    fprintf(stderr, "%s: GPU sort failed (%s): %s; data left unsorted\n", who, gbsort_status_string(rc), g_err);
}

void radix_sort(void* base, size_t nmemb, size_t size, void (*radix)(const void* ptr, void* radix, void* arg),
                size_t rsize, void* arg) {
  dropin_sort(base, nmemb, size, radix, rsize, arg, "radix_sort");
}

void mpsort_omp(void* base, size_t nmemb, size_t size, void (*radix)(const void* ptr, void* radix, void* arg),
                size_t rsize, void* arg) {
  dropin_sort(base, nmemb, size, radix, rsize, arg, "mpsort_omp");
}

int mpsort_last_status(void) { return g_mpsort_status; }

// One-process forms of the reference's MPI entry points: the communicator is
// not read.  As in the reference with one rank, `base` ends sorted (its
// first, local sort) and so does `out` (outnmemb must equal nmemb).  With
// the descriptor radix the sort is self-checked like the reference's: a
// multiset hash of the records before and after, in place of its byte sum.
void mpsort_mpi_newarray_impl(void* base, size_t nmemb, void* out, size_t outnmemb, size_t elsize,
                              void (*radix)(const void* ptr, void* radix, void* arg), size_t rsize, void* arg,
                              intptr_t comm, int line, const char* file) {
  (void)comm;
  int rc = GBSORT_OK;
  if (outnmemb != nmemb) {
    set_err("input and output size mismatch: %zu (in) != %zu (out)", nmemb, outnmemb);
    rc = GBSORT_ERR_BAD_ARG;
  } else if (nmemb > 0) {
    if (radix == mpsort_radix_desc) {
      const gbsort_key_desc* d = (const gbsort_key_desc*)arg;
      if (!d || rsize != 8u * d->nwords) rc = GBSORT_ERR_BAD_ARG;
      else rc = gbsort_sort_host(base, base, nmemb, elsize, d, GBSORT_AUTO | GBSORT_VERIFY);
    } else {
      rc = gbsort_sort_radix_host(base, nmemb, elsize, radix, rsize, arg);
    }
    if (rc == GBSORT_OK && out != base) memcpy(out, base, nmemb * elsize);
  }
  g_mpsort_status = rc;
  if (rc != GBSORT_OK)
    fprintf(stderr, "mpsort_mpi (%s:%d): GPU sort failed (%s): %s\n", file ? file : "?", line,
            gbsort_status_string(rc), g_err);
}

void mpsort_mpi_impl(void* base, size_t nmemb, size_t elsize, void (*radix)(const void* ptr, void* radix, void* arg),
                     size_t rsize, void* arg, intptr_t comm, int line, const char* file) {
  mpsort_mpi_newarray_impl(base, nmemb, base, nmemb, elsize, radix, rsize, arg, comm, line, file);
}

void mpsort_mpi_report_last_run(void) {
  static const char* names[6] = {"splitters", "count", "scan", "scatter", "split", "local"};
  const gbsort_stats& st = g_stats;
  printf("mpsort (GB300) last run: method %d, %u buckets, %u launches\n", st.method, st.nbuckets, st.launches);
  for (int i = 0; i < 6; ++i) printf("%s %.4f ms\n", names[i], st.stage_ms[i]);
}

int gbsort_take_device(const void* d_source, size_t nsource, size_t elsize, const int64_t* d_index, size_t nindex,
                       void* d_out, void* stream) {
  if (elsize == 0 || elsize > (1u << 20) || (nindex && (!d_index || !d_out || (nsource && !d_source))))
    return GBSORT_ERR_BAD_ARG;
  Context* c = nullptr;
  int rc = get_ctx(&c);
  if (rc) return rc;
  std::lock_guard<std::mutex> lk(c->mu);
  cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
  GB_CUDA(c->vh.ensure(2 * sizeof(unsigned long long)));
  unsigned long long* bad = c->vh.as<unsigned long long>();
  GB_CUDA(take_records(d_source, nsource, (uint32_t)elsize, d_index, nindex, d_out, bad, st));
  unsigned long long hb = 0;
  GB_CUDA(cudaMemcpyAsync(&hb, bad, sizeof hb, cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  if (hb) {
    set_err("index %llu is out of range for %zu source records", hb - 1, nsource);
    return GBSORT_ERR_BAD_ARG;
  }
  return GBSORT_OK;
}

int gbsort_multiset_hash_device(const void* d_records, size_t nmemb, size_t elsize, uint64_t* d_hash, void* stream) {
  if (!d_hash || (nmemb && !d_records) || elsize == 0 || elsize > (1u << 20)) return GBSORT_ERR_BAD_ARG;
  Context* c = nullptr;
  int rc = get_ctx(&c);
  if (rc) return rc;
  cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
  GB_CUDA(multiset_hash(d_records, nmemb, (uint32_t)elsize, (unsigned long long*)d_hash, st));
  return GBSORT_OK;
}

void mpsort_mpi_set_options(int options) {
  std::lock_guard<std::mutex> lk(g_opt_mu);
  g_mpi_options |= options;
}
int mpsort_mpi_has_options(int options) {
  std::lock_guard<std::mutex> lk(g_opt_mu);
  return (g_mpi_options & options) == options;
}
void mpsort_mpi_unset_options(int options) {
  std::lock_guard<std::mutex> lk(g_opt_mu);
  g_mpi_options &= ~options;
}

}  // extern "C"
