// segments.cu -- batched segments, the sorted-key join and a lookup probe.
//
//  * segment_ranges: one task per segment (its key range from a min/max
//    reduction) for the task engine of hsort.cu, so many arrays of uneven
//    size are sorted by one persistent launch per round.
//  * join_count / join_write: pairs of equal keys of two key-sorted record
//    arrays with unique keys per side, in key order (two-snapshot ID
//    matching).  Per tile of `a`, the matching window of `b` is staged in
//    shared memory and every key is found there by binary search.
//  * k_probe_buckets: learned and full-search lookups of the same keys
//    against the same splitters, for the checks.
#include "cdf.cuh"
#include "cdf_api.h"
#include "common.cuh"
#include "kernels.h"

namespace gb {

int num_sms();

namespace {

constexpr uint32_t kCopyPieceSeg = 1u << 16;
constexpr int kJoinTile = 2048;
constexpr int kJoinWindow = 4096;

__global__ void __launch_bounds__(kThreads) k_segment_ranges(const uint8_t* __restrict__ rec, uint32_t elsize,
                                                              gbsort_key_word kw,
                                                              const uint64_t* __restrict__ offs, uint32_t nseg,
                                                              uint64_t skip_above, SortTask* __restrict__ tasks,
                                                              uint32_t* ntasks, uint32_t cap, uint32_t* err) {
  __shared__ uint64_t red[2 * kWarps];
  for (uint32_t sg = blockIdx.x; sg < nseg; sg += gridDim.x) {
    const uint64_t a = offs[sg], b = offs[sg + 1];
    if (b == a || b - a > skip_above) continue;  // empty, or sorted on its own
    uint64_t mn = ~0ull, mx = 0;
    for (uint64_t i = a + threadIdx.x; i < b; i += kThreads) {
      uint64_t k = load_key_aligned4(rec + i * elsize, kw);
      mn = k < mn ? k : mn;
      mx = k > mx ? k : mx;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      uint64_t x = __shfl_xor_sync(GB_FULL_MASK, mn, o), y = __shfl_xor_sync(GB_FULL_MASK, mx, o);
      mn = x < mn ? x : mn;
      mx = y > mx ? y : mx;
    }
    if (lane_id() == 0) {
      red[warp_id()] = mn;
      red[kWarps + warp_id()] = mx;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int i = 0; i < kWarps; ++i) {
        mn = red[i] < mn ? red[i] : mn;
        mx = red[kWarps + i] > mx ? red[kWarps + i] : mx;
      }
      const uint32_t cnt = (uint32_t)(b - a);
      if (mn == mx || cnt == 1) {
        uint32_t pieces = (cnt + kCopyPieceSeg - 1) / kCopyPieceSeg;
        uint32_t at = atomicAdd(ntasks, pieces);
        if (at + pieces > cap) set_error(err, DEV_ERR_TASK_OVERFLOW);
        else
          for (uint32_t i = 0; i < pieces; ++i) {
            uint32_t s0 = i * kCopyPieceSeg;
            tasks[at + i] = make_task((uint32_t)a + s0, min(kCopyPieceSeg, cnt - s0), mn, mx, false, true);
          }
      } else {
        uint32_t at = atomicAdd(ntasks, 1u);
        if (at >= cap) set_error(err, DEV_ERR_TASK_OVERFLOW);
        else tasks[at] = make_task((uint32_t)a, cnt, mn, mx, false, false);
      }
    }
    __syncthreads();
  }
}

__device__ __forceinline__ uint32_t lower_bound_keys(const uint8_t* rec, uint32_t elsize, const gbsort_key_word& kw,
                                                     uint32_t lo, uint32_t hi, uint64_t key) {
  while (lo < hi) {
    uint32_t m = (lo + hi) >> 1;
    if (load_key_aligned4(rec + (size_t)m * elsize, kw) < key) lo = m + 1;
    else hi = m;
  }
  return lo;
}

// Matches of a's tile [t0, t1) in b: returns per-item match index (or -1).
// `win` (kJoinWindow keys) caches b's window [w0, w1) when it fits.
__device__ __forceinline__ void join_tile(const uint8_t* a, uint32_t t0, uint32_t t1, const uint8_t* b, uint32_t nb,
                                          uint32_t elsize, const gbsort_key_word& kw, uint64_t* win, uint32_t* wlim,
                                          int64_t (&match)[kJoinTile / kThreads]) {
  constexpr int PER = kJoinTile / kThreads;
  if (threadIdx.x == 0) {
    uint64_t k0 = load_key_aligned4(a + (size_t)t0 * elsize, kw);
    uint64_t k1 = load_key_aligned4(a + (size_t)(t1 - 1) * elsize, kw);
    uint32_t w0 = lower_bound_keys(b, elsize, kw, 0, nb, k0);
    uint32_t w1 = k1 == ~0ull ? nb : lower_bound_keys(b, elsize, kw, w0, nb, k1 + 1);
    wlim[0] = w0;
    wlim[1] = w1;
  }
  __syncthreads();
  const uint32_t w0 = wlim[0], w1 = wlim[1];
  const bool cached = w1 - w0 <= (uint32_t)kJoinWindow;
  if (cached)
    for (uint32_t i = w0 + threadIdx.x; i < w1; i += kThreads) win[i - w0] = load_key_aligned4(b + (size_t)i * elsize, kw);
  __syncthreads();
#pragma unroll
  for (int r = 0; r < PER; ++r) {
    uint32_t i = t0 + threadIdx.x * PER + r;
    match[r] = -1;
    if (i < t1) {
      uint64_t k = load_key_aligned4(a + (size_t)i * elsize, kw);
      uint32_t pos;
      bool hit;
      if (cached) {
        uint32_t lo = 0, hi = w1 - w0;
        while (lo < hi) {
          uint32_t m = (lo + hi) >> 1;
          if (win[m] < k) lo = m + 1; else hi = m;
        }
        hit = lo < w1 - w0 && win[lo] == k;
        pos = w0 + lo;
      } else {
        pos = lower_bound_keys(b, elsize, kw, w0, w1, k);
        hit = pos < w1 && load_key_aligned4(b + (size_t)pos * elsize, kw) == k;
      }
      if (hit) match[r] = pos;
    }
  }
  __syncthreads();
}

__host__ __device__ __forceinline__ uint32_t jchunk(uint32_t n, uint32_t c, uint32_t g) {
  return (uint32_t)((uint64_t)n * c / g);
}

__global__ void __launch_bounds__(kThreads) k_join_count(const uint8_t* a, uint32_t na, const uint8_t* b, uint32_t nb,
                                                          uint32_t elsize, gbsort_key_word kw, uint32_t* counts) {
  __shared__ uint64_t win[kJoinWindow];
  __shared__ uint32_t wlim[2];
  __shared__ uint32_t tmp[kWarps];
  const uint32_t c0 = jchunk(na, blockIdx.x, gridDim.x), c1 = jchunk(na, blockIdx.x + 1, gridDim.x);
  uint32_t total = 0;
  for (uint32_t t0 = c0; t0 < c1; t0 += kJoinTile) {
    uint32_t t1 = min(c1, t0 + kJoinTile);
    int64_t match[kJoinTile / kThreads];
    join_tile(a, t0, t1, b, nb, elsize, kw, win, wlim, match);
    uint32_t cnt = 0;
#pragma unroll
    for (int r = 0; r < kJoinTile / kThreads; ++r) cnt += match[r] >= 0;
    uint32_t sum;
    block_exclusive_scan<uint32_t>(cnt, tmp, &sum);
    total += sum;
  }
  if (threadIdx.x == 0) counts[blockIdx.x] = total;
  if (blockIdx.x == 0 && threadIdx.x == 0) counts[gridDim.x] = 0;
}

__global__ void __launch_bounds__(kThreads) k_join_write(const uint8_t* a, uint32_t na, const uint8_t* b, uint32_t nb,
                                                          uint32_t elsize, gbsort_key_word kw,
                                                          const uint32_t* __restrict__ offsets, uint64_t* pa,
                                                          uint64_t* pb, uint64_t* npairs) {
  __shared__ uint64_t win[kJoinWindow];
  __shared__ uint32_t wlim[2];
  __shared__ uint32_t tmp[kWarps];
  const uint32_t c0 = jchunk(na, blockIdx.x, gridDim.x), c1 = jchunk(na, blockIdx.x + 1, gridDim.x);
  uint32_t base = offsets[blockIdx.x];
  for (uint32_t t0 = c0; t0 < c1; t0 += kJoinTile) {
    uint32_t t1 = min(c1, t0 + kJoinTile);
    int64_t match[kJoinTile / kThreads];
    join_tile(a, t0, t1, b, nb, elsize, kw, win, wlim, match);
    uint32_t cnt = 0;
#pragma unroll
    for (int r = 0; r < kJoinTile / kThreads; ++r) cnt += match[r] >= 0;
    uint32_t sum;
    uint32_t pre = block_exclusive_scan<uint32_t>(cnt, tmp, &sum);
    uint32_t at = base + pre;
#pragma unroll
    for (int r = 0; r < kJoinTile / kThreads; ++r)
      if (match[r] >= 0) {
        pa[at] = t0 + threadIdx.x * (kJoinTile / kThreads) + r;
        pb[at] = (uint64_t)match[r];
        ++at;
      }
    base += sum;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) *npairs = offsets[gridDim.x];
}

// Splitter reads of upper_bound_in(S, lo, hi, key): one per halving step.
__device__ __forceinline__ uint32_t search_reads(const uint64_t* S, uint32_t lo, uint32_t hi, uint64_t key) {
  uint32_t r = 0;
  while (lo < hi) {
    uint32_t mid = (lo + hi) >> 1;
    ++r;
    if (S[mid] <= key) lo = mid + 1;
    else hi = mid;
  }
  return r;
}

__global__ void k_probe_buckets(const uint64_t* __restrict__ keys, uint32_t nkeys, const uint64_t* __restrict__ S,
                                ModelDev m, uint32_t* __restrict__ learned, uint32_t* __restrict__ search,
                                uint32_t* misses, unsigned long long* reads) {
  m = resolve_model(m);
  const uint32_t nsplit = (uint32_t)(m.nbuckets - 1);
  unsigned long long rl = 0, rp = 0;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nkeys; i += gridDim.x * blockDim.x) {
    const uint64_t k = keys[i];
    const uint32_t bl = bucket_learned(S, m, m.knots, m.win, k, misses);
    const uint32_t bs = bucket_plain(S, m.nbuckets, k);
    learned[i] = bl;
    search[i] = bs;
    if (reads) {
      // splitters the learned lookup reads: none for a zero window, else the
      // two window bounds and the search inside the window
      uint32_t leaf, g;
      model_predict(k, m.kmin, m.lshift, m.lbits, m.nbuckets, m.knots, leaf, g);
      const uint32_t w = m.win[leaf];
      if (w != 0) {
        uint32_t lo = g > (w >> 16) ? g - (w >> 16) : 0u;
        uint32_t hi = min(g + (w & 0xffffu), nsplit);
        rl += (lo > 0) + (hi < nsplit) + search_reads(S, lo, hi, k);
      }
      rp += search_reads(S, 0, nsplit, k);
    }
  }
  if (reads) {
    atomicAdd(reads, rl);
    atomicAdd(reads + 1, rp);
  }
}

}  // namespace

cudaError_t segment_ranges(const uint8_t* rec, uint32_t elsize, gbsort_key_word key, const uint64_t* offsets,
                           uint32_t nseg, uint64_t skip_above, SortTask* tasks, uint32_t* ntasks, uint32_t cap,
                           uint32_t* err, cudaStream_t st) {
  uint32_t g = nseg < (uint32_t)num_sms() * 8 ? nseg : (uint32_t)num_sms() * 8;
  k_segment_ranges<<<g, kThreads, 0, st>>>(rec, elsize, key, offsets, nseg, skip_above, tasks, ntasks, cap, err);
  note_launches(1);
  return cudaGetLastError();
}

int join_grid(uint32_t na) {
  uint32_t g = (na + kJoinTile - 1) / kJoinTile;
  uint32_t cap = (uint32_t)num_sms() * 4;
  return (int)(g < 1 ? 1 : (g > cap ? cap : g));
}

cudaError_t join_count(const uint8_t* a, uint32_t na, const uint8_t* b, uint32_t nb, uint32_t elsize,
                       gbsort_key_word key, uint32_t* counts, int grid, cudaStream_t st) {
  k_join_count<<<grid, kThreads, 0, st>>>(a, na, b, nb, elsize, key, counts);
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t join_write(const uint8_t* a, uint32_t na, const uint8_t* b, uint32_t nb, uint32_t elsize,
                       gbsort_key_word key, const uint32_t* offsets, int grid, uint64_t* pa, uint64_t* pb,
                       uint64_t* npairs, cudaStream_t st) {
  k_join_write<<<grid, kThreads, 0, st>>>(a, na, b, nb, elsize, key, offsets, pa, pb, npairs);
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t probe_buckets(const uint64_t* keys, uint32_t nkeys, const uint64_t* S, const void* model,
                          uint32_t* learned, uint32_t* search, uint32_t* misses, unsigned long long* reads,
                          cudaStream_t st) {
  const ModelDev m = *(const ModelDev*)model;
  unsigned g = (nkeys + 255) / 256;
  if (g > 4096) g = 4096;
  if (g == 0) return cudaSuccess;
  k_probe_buckets<<<g, 256, 0, st>>>(keys, nkeys, S, m, learned, search, misses, reads);
  note_launches(1);
  return cudaGetLastError();
}

}  // namespace gb
