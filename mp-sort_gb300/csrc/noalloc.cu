// noalloc.cu -- gbsort_sort_device_noalloc: the histogram sort for callers
// that must not allocate device memory.
//
// Some callers cannot call cudaMalloc: code that runs while a framework's
// caching allocator owns the device memory budget, code on a latency-critical
// path where an allocation would synchronise the device, or code that must
// behave the same on every call with no chance of running out of memory
// half-way.  This entry point takes its scratch space (the two record
// buffers and the small count / task / splitter arrays of the pipeline)
// from one file-scope device array of fixed size instead of allocating it.
//
// Limits and rules:
//   * records * elsize <= GBSORT_NOALLOC_MAX_BYTES (8 MiB); larger sorts are
//     rejected with GBSORT_ERR_BAD_ARG before any work is enqueued;
//   * the plain (bisection) splitters are used; the result is the same
//     stable order every other method produces;
//   * all calls share the one array and each call leaves its contents
//     behind (the counters are cleared at the start of every call): two
//     calls whose work overlaps on the GPU (different streams, or different
//     host threads without ordering) race on it;
//   * set-up, once per device: the driver creates the array when it loads
//     this file's device code on that device -- at context creation under
//     eager module loading, else at the first cudaGetSymbolAddress below,
//     made by the first call on that device with the device current.  That
//     first call may allocate (the array, and the library's kernels if no
//     other call loaded them) and must not run during a global-mode stream
//     capture; later calls allocate nothing;
//   * the call waits for the work on `stream` to finish (it reads the
//     device-side consistency word back).
#include <cuda_runtime.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <mutex>

#include "../../include/gbsort.h"
#include "kernels.h"

namespace {

using namespace gb;

constexpr size_t kRecordBytesMax = GBSORT_NOALLOC_MAX_BYTES;
// two record buffers plus the pipeline's small arrays for the largest sort
constexpr size_t kScratchBytes = 2 * kRecordBytesMax + (6u << 20);

static __device__ __align__(256) uint8_t g_noalloc_scratch[kScratchBytes];

std::mutex g_mu;
void* g_scratch_addr[64] = {};

struct Carve {
  uint8_t* base;
  size_t off = 0;
  size_t cap = 0;
  template <typename T>
  T* take(size_t count) {
    off = (off + 255) & ~(size_t)255;
    T* r = reinterpret_cast<T*>(base + off);
    off += sizeof(T) * count;
    return r;
  }
  bool ok() const { return off <= cap; }
};

int fail(const char* what, cudaError_t e) {
  fprintf(stderr, "gbsort_sort_device_noalloc: %s: %s\n", what, cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? GBSORT_ERR_OOM : GBSORT_ERR_CUDA;
}

#define NA_CUDA(call)                                \
  do {                                               \
    cudaError_t e_ = (call);                         \
    if (e_ != cudaSuccess) return fail(#call, e_);   \
  } while (0)

// Device address of the scratch array on the current device (looked up once).
int scratch_address(uint8_t** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail("cudaGetDevice", e);
  if (dev < 0 || dev >= 64) return GBSORT_ERR_BAD_ARG;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return fail("cudaGetSymbolAddress", e);
    g_scratch_addr[dev] = p;
  }
  *out = reinterpret_cast<uint8_t*>(g_scratch_addr[dev]);
  return GBSORT_OK;
}

}  // namespace

extern "C" GBSORT_API int gbsort_sort_device_noalloc(const void* d_in, void* d_out, size_t nmemb, size_t elsize,
                                                     const gbsort_key_desc* key, void* stream) {
  if (nmemb == 0) return GBSORT_OK;
  if (!d_in || !d_out || !key || elsize == 0) return GBSORT_ERR_BAD_ARG;
  if (nmemb > kRecordBytesMax / elsize) {
    fprintf(stderr, "gbsort_sort_device_noalloc: %zu records of %zu bytes exceed the %zu-byte limit\n", nmemb,
            elsize, (size_t)kRecordBytesMax);
    return GBSORT_ERR_BAD_ARG;
  }
  if (key->nwords != 1 || key->word[0].offset % 4 || (key->word[0].width != 4 && key->word[0].width != 8) ||
      key->word[0].is_signed > 1 || (size_t)key->word[0].offset + key->word[0].width > elsize ||
      !hsort_supported((uint32_t)elsize)) {
    fprintf(stderr, "gbsort_sort_device_noalloc: needs a one-word key at a 4-byte offset and 8-64 byte records\n");
    return GBSORT_ERR_UNSUPPORTED;
  }
  {
    uintptr_t a = (uintptr_t)d_in | (uintptr_t)d_out;
    size_t need = elsize % 16 == 0 ? 16 : (elsize % 8 == 0 ? 8 : 4);
    if (a % need) return GBSORT_ERR_UNSUPPORTED;
  }
  uint8_t* scratch = nullptr;
  int rc = scratch_address(&scratch);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  const uint32_t n = (uint32_t)nmemb, E = (uint32_t)elsize;

  // pipeline shape (as the allocating entry point chooses it)
  int nb = 1;
  if (n > 4096) {
    uint64_t want = ((uint64_t)n + 2047) / 2048;
    while ((uint64_t)nb < want && nb < 4096) nb <<= 1;
  }
  const int grid = hsort_grid(n);
  const uint32_t s_eff = nb > 1 ? (uint32_t)std::min<uint64_t>(n, std::max<uint64_t>(4096, (uint64_t)nb * 128)) : 0;
  const uint32_t cap_split = (uint32_t)nb + n / 4096 + 4096;
  const uint32_t cap_local = 4u * (uint32_t)nb + n / 512 + 65536;

  Carve cv{scratch, 0, kScratchBytes};
  uint8_t* A = cv.take<uint8_t>((size_t)n * E);
  uint8_t* B = cv.take<uint8_t>((size_t)n * E);
  uint32_t* counters = cv.take<uint32_t>(64);
  uint64_t* S = cv.take<uint64_t>((size_t)(nb > 2 ? nb : 2));
  uint32_t* counts = cv.take<uint32_t>((size_t)nb * grid);
  uint32_t* scan_tmp = cv.take<uint32_t>(scan_tmp_words((size_t)nb * grid));
  SortTask* split0 = cv.take<SortTask>(cap_split);
  SortTask* split1 = cv.take<SortTask>(cap_split);
  SortTask* local = cv.take<SortTask>(cap_local);
  uint64_t* sA = cv.take<uint64_t>(s_eff);
  uint64_t* sB = cv.take<uint64_t>(s_eff);
  uint32_t* shist = cv.take<uint32_t>(8 * 256);
  uint32_t* sstarts = cv.take<uint32_t>(8 * 256);
  unsigned long long* sstatus = cv.take<unsigned long long>((size_t)lsd_tiles(s_eff > 0 ? s_eff : 1) * 256 + 1);
  uint32_t* sticket = reinterpret_cast<uint32_t*>(sstatus + (size_t)lsd_tiles(s_eff > 0 ? s_eff : 1) * 256);
  if (!cv.ok()) {
    fprintf(stderr, "gbsort_sort_device_noalloc: scratch layout exceeds the static array\n");
    return GBSORT_ERR_BAD_ARG;
  }
  uint32_t* stats = counters;
  uint32_t* err = counters + STAT_SLOTS;
  uint32_t* iters = counters + 21;
  uint32_t* nsplit = counters + 24;
  uint32_t* nlocal = counters + 26;
  uint32_t* work = counters + 27;
  // every call starts from zeroed counters: the array keeps the last call's
  NA_CUDA(cudaMemsetAsync(counters, 0, 64 * sizeof(uint32_t), st));

  HsortParams p{};
  p.in = (const uint8_t*)d_in;
  p.out = (uint8_t*)d_out;
  p.bufA = A;
  p.bufB = B;
  p.n = n;
  p.elsize = E;
  p.key = key->word[0];
  p.a_cap = n;
  p.bkt = reinterpret_cast<uint16_t*>(B);  // level-1 bucket ids (B is free until level 2)

  if (nb > 1) {
    NA_CUDA(sample_keys(p.in, n, E, p.key, s_eff, sA, st));
    uint64_t* kin = sA;
    uint64_t* kout = sB;
    NA_CUDA(lsd_digit_histograms(sA, s_eff, 1, shist, st));
    NA_CUDA(lsd_digit_starts(shist, 1, sstarts, st));
    for (int d = 0; d < 8; ++d) {  // LSD sort of the sample, 8 one-sweep digit passes
      NA_CUDA(lsd_onesweep(kin, nullptr, kout, nullptr, s_eff, 1, 0, 8 * d, sstarts + 256 * d, sstatus, sticket,
                           err, st));
      uint64_t* t = kin;
      kin = kout;
      kout = t;
    }
    NA_CUDA(plain_splitters(kin, s_eff, nb - 1, S, iters, nullptr, nullptr, st));
    NA_CUDA(finalize_splitters(S, nb - 1, st));
  }
  NA_CUDA(l1_count(p, LOOKUP_PLAIN, S, nb, nullptr, counts, stats, st));
  NA_CUDA(exclusive_scan_u32(counts, counts, (size_t)nb * grid, scan_tmp, st));
  NA_CUDA(l1_scatter(p, nb, counts, stats, st));
  SortTask* lists[2] = {split0, split1};
  {
    TaskListsHost L{lists[1], nsplit + 1, lists[0], nsplit, local, nlocal, cap_split, cap_local};
    NA_CUDA(build_tasks(counts, grid, S, nb, n, L, err, stats, st));
  }
  const int rounds = 16;
  for (int r = 0; r < rounds; ++r) {
    TaskListsHost L{lists[r & 1], nsplit + (r & 1), lists[(r + 1) & 1], nsplit + ((r + 1) & 1),
                    local, nlocal, cap_split, cap_local};
    NA_CUDA(cudaMemsetAsync(L.nsplit_out, 0, sizeof(uint32_t), st));
    NA_CUDA(run_split_round(p, L, work, stats, err, st));
  }
  NA_CUDA(run_local(p, local, nlocal, cap_local, work, stats, st));
  uint32_t host_err = 0, host_left = 0;
  NA_CUDA(cudaMemcpyAsync(&host_err, err, 4, cudaMemcpyDeviceToHost, st));
  NA_CUDA(cudaMemcpyAsync(&host_left, nsplit + (rounds & 1), 4, cudaMemcpyDeviceToHost, st));
  NA_CUDA(cudaStreamSynchronize(st));
  if (host_err || host_left) {
    fprintf(stderr, "gbsort_sort_device_noalloc: device check failed (code %u, %u tasks left)\n", host_err,
            host_left);
    return GBSORT_ERR_INTERNAL;
  }
  return GBSORT_OK;
}
