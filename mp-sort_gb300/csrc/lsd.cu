// lsd.cu -- the generic path: stable LSD radix sort of key words + index,
// then one record permutation.
//
// Serves every key the histogram sort does not take (multi-word radix,
// records whose size or alignment is not a multiple of 4 bytes, keys from a
// host radix() callback) and sorts the sample of the histogram sort.  It
// reproduces the reference's ordering -- a stable sort by the radix as a
// little-endian unsigned integer (radixsort.c:19-44, stdlib/msort.c:52-174)
// -- with 8-bit digit passes:
//   * one read of the keys builds the histograms of every digit, so passes
//     whose digit is constant are skipped by the host;
//   * per pass, each CTA counts digits over its contiguous chunk, the
//     (digit x chunk) matrix is scanned, and each CTA re-reads its chunk and
//     scatters stably: tile ranks come from warp match ranking, chunk order
//     from the scanned offsets.
#include "common.cuh"
#include "kernels.h"

namespace gb {

namespace {

constexpr int kLsdRpt = 8;                      // items per thread per tile
constexpr int kLsdTile = kThreads * kLsdRpt;    // 4096

__host__ __device__ __forceinline__ uint32_t chunk_begin(uint32_t n, uint32_t c, uint32_t g) {
  return (uint32_t)(((uint64_t)n * c / g) & ~(uint64_t)31);
}
__host__ __device__ __forceinline__ uint32_t chunk_end(uint32_t n, uint32_t c, uint32_t g) {
  return c + 1 == g ? n : chunk_begin(n, c + 1, g);
}

__global__ void k_extract_keys(const uint8_t* __restrict__ rec, uint32_t n, uint32_t elsize,
                               gbsort_key_desc key, int aligned4, uint64_t* __restrict__ keys,
                               uint32_t* __restrict__ idx) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint8_t* r = rec + (size_t)i * elsize;
    for (uint32_t w = 0; w < key.nwords; ++w) {
      uint64_t v = aligned4 ? load_key_aligned4(r, key.word[w]) : load_key_bytes(r, key.word[w]);
      keys[(size_t)w * n + i] = v;
    }
    if (idx) idx[i] = i;
  }
}

__global__ void k_radix_bytes(const uint8_t* __restrict__ radix, uint32_t n, uint32_t rsize,
                              uint64_t* __restrict__ keys, uint32_t* __restrict__ idx) {
  const uint32_t nw = (rsize + 7) / 8;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint8_t* r = radix + (size_t)i * rsize;
    for (uint32_t w = 0; w < nw; ++w) {
      uint64_t v = 0;
      for (uint32_t b = 0; b < 8 && 8 * w + b < rsize; ++b) v |= (uint64_t)r[8 * w + b] << (8 * b);
      keys[(size_t)w * n + i] = v;
    }
    if (idx) idx[i] = i;
  }
}

// Histograms of all 8 digits of one key word, 256 bins each.
__global__ void __launch_bounds__(kThreads) k_digit_hist(const uint64_t* __restrict__ keys, uint32_t n,
                                                          uint32_t* __restrict__ hist) {
  __shared__ uint32_t h[8 * 256];
  for (int i = threadIdx.x; i < 8 * 256; i += kThreads) h[i] = 0;
  __syncthreads();
  for (uint32_t i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    uint64_t k = keys[i];
#pragma unroll
    for (int d = 0; d < 8; ++d) atomicAdd(&h[d * 256 + ((k >> (8 * d)) & 255)], 1u);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < 8 * 256; i += kThreads)
    if (h[i]) atomicAdd(&hist[i], h[i]);
}

__global__ void __launch_bounds__(kThreads) k_lsd_count(const uint64_t* __restrict__ keys, uint32_t n,
                                                         int shift, uint32_t* __restrict__ counts) {
  __shared__ uint32_t h[256];
  const uint32_t c = blockIdx.x, g = gridDim.x;
  const uint32_t b = chunk_begin(n, c, g), e = chunk_end(n, c, g);
  for (int i = threadIdx.x; i < 256; i += kThreads) h[i] = 0;
  __syncthreads();
  for (uint32_t i0 = b; i0 < e; i0 += kThreads) {
    uint32_t i = i0 + threadIdx.x;
    bool v = i < e;
    uint32_t d = v ? (uint32_t)(keys[i] >> shift) & 255u : 0xffffffffu;
    uint32_t peers = __match_any_sync(GB_FULL_MASK, d);
    if (v && (peers & lanemask_lt()) == 0) atomicAdd(&h[d], (uint32_t)__popc(peers));
  }
  __syncthreads();
  for (int d = threadIdx.x; d < 256; d += kThreads) counts[(size_t)d * g + c] = h[d];
}

template <int NW, bool IDX>
__global__ void __launch_bounds__(kThreads) k_lsd_scatter(const uint64_t* __restrict__ keys_in,
                                                           const uint32_t* __restrict__ idx_in,
                                                           uint64_t* __restrict__ keys_out,
                                                           uint32_t* __restrict__ idx_out, uint32_t n,
                                                           int word, int shift,
                                                           const uint32_t* __restrict__ offsets) {
  using Rank = BlockRank<kLsdRpt, 8>;
  __shared__ uint16_t hist[Rank::kCounters];
  __shared__ uint32_t scan_tmp[kWarps];
  __shared__ uint32_t start[257];
  __shared__ uint32_t cursor[256];
  const uint32_t c = blockIdx.x, g = gridDim.x;
  const uint32_t cb = chunk_begin(n, c, g), ce = chunk_end(n, c, g);
  for (int d = threadIdx.x; d < 256; d += kThreads) cursor[d] = offsets[(size_t)d * g + c];
  __syncthreads();
  const uint32_t w = warp_id(), lane = lane_id();
  for (uint32_t t = cb; t < ce; t += kLsdTile) {
    uint64_t k[NW][kLsdRpt];
    uint32_t ix[kLsdRpt];
    uint32_t digit[kLsdRpt], pos[kLsdRpt];
    uint32_t nvalid = min((uint32_t)kLsdTile, ce - t);
#pragma unroll
    for (int r = 0; r < kLsdRpt; ++r) {
      uint32_t e = w * 32 * kLsdRpt + r * 32 + lane;
      bool valid = e < nvalid;
#pragma unroll
      for (int q = 0; q < NW; ++q) k[q][r] = valid ? keys_in[(size_t)q * n + t + e] : 0;
      if (IDX) ix[r] = valid ? idx_in[t + e] : 0;
      uint64_t kw = 0;
#pragma unroll
      for (int q = 0; q < NW; ++q) kw = (q == word) ? k[q][r] : kw;
      digit[r] = valid ? (uint32_t)(kw >> shift) & 255u : 255u;
    }
    Rank::rank(digit, pos, hist, scan_tmp, start);
#pragma unroll
    for (int r = 0; r < kLsdRpt; ++r) {
      uint32_t e = w * 32 * kLsdRpt + r * 32 + lane;
      if (e < nvalid) {
        uint32_t d = digit[r];
        uint32_t dest = cursor[d] + pos[r] - start[d];
#pragma unroll
        for (int q = 0; q < NW; ++q) keys_out[(size_t)q * n + dest] = k[q][r];
        if (IDX) idx_out[dest] = ix[r];
      }
    }
    __syncthreads();
    for (int d = threadIdx.x; d < 256; d += kThreads) {
      uint32_t cnt = start[d + 1] - start[d];
      if (d == 255) cnt -= (uint32_t)kLsdTile - nvalid;  // the padding items sit at the end
      cursor[d] += cnt;
    }
    __syncthreads();
  }
}

// out[i] = in[idx[i]], copied in units of VB bytes (VB divides elsize and
// both base addresses are VB-aligned).
template <typename V>
__global__ void k_gather(const uint8_t* __restrict__ in, uint8_t* __restrict__ out,
                         const uint32_t* __restrict__ idx, uint32_t n, uint32_t elsize) {
  const uint32_t vpr = elsize / sizeof(V);
  const uint64_t total = (uint64_t)n * vpr;
  for (uint64_t f = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; f < total;
       f += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t i = (uint32_t)(f / vpr), v = (uint32_t)(f % vpr);
    const V* src = reinterpret_cast<const V*>(in + (size_t)idx[i] * elsize) + v;
    V* dst = reinterpret_cast<V*>(out + (size_t)i * elsize) + v;
    *dst = *src;
  }
}

}  // namespace

int num_sms() {
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 148;
  }
  return sms;
}

static unsigned blocks_for(uint64_t n, int threads) {
  uint64_t b = (n + threads - 1) / threads;
  uint64_t cap = (uint64_t)num_sms() * 8;
  return (unsigned)(b < 1 ? 1 : (b > cap ? cap : b));
}


cudaError_t extract_keys(const void* rec, uint32_t n, uint32_t elsize, const gbsort_key_desc& key,
                         uint64_t* keys, uint32_t* idx, cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  int aligned4 = ((uintptr_t)rec % 4 == 0) && (elsize % 4 == 0);
  for (uint32_t w = 0; w < key.nwords; ++w) aligned4 &= (key.word[w].offset % 4 == 0);
  k_extract_keys<<<blocks_for(n, 256), 256, 0, stream>>>((const uint8_t*)rec, n, elsize, key, aligned4,
                                                          keys, idx);
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t radix_bytes_to_keys(const uint8_t* radix, uint32_t n, uint32_t rsize, uint64_t* keys,
                                uint32_t* idx, cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  k_radix_bytes<<<blocks_for(n, 256), 256, 0, stream>>>(radix, n, rsize, keys, idx);
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t lsd_digit_histograms(const uint64_t* keys, uint32_t n, int nwords, uint32_t* hist,
                                 cudaStream_t stream) {
  cudaError_t e = cudaMemsetAsync(hist, 0, sizeof(uint32_t) * 8 * 256 * nwords, stream);
  if (e != cudaSuccess || n == 0) return e;
  for (int w = 0; w < nwords; ++w)
    k_digit_hist<<<blocks_for(n, kThreads), kThreads, 0, stream>>>(keys + (size_t)w * n, n,
                                                                    hist + (size_t)w * 8 * 256);
  note_launches(1);
  return cudaGetLastError();
}

int lsd_grid(uint32_t n) {
  uint64_t g = ((uint64_t)n + kLsdTile - 1) / kLsdTile;
  uint64_t cap = (uint64_t)num_sms() * 2;
  return (int)(g < 1 ? 1 : (g > cap ? cap : g));
}

cudaError_t lsd_count(const uint64_t* keys_word, uint32_t n, int shift, uint32_t* counts,
                      cudaStream_t stream) {
  k_lsd_count<<<lsd_grid(n), kThreads, 0, stream>>>(keys_word, n, shift, counts);
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t lsd_scatter(const uint64_t* keys_in, const uint32_t* idx_in, uint64_t* keys_out,
                        uint32_t* idx_out, uint32_t n, int nwords, int word, int shift,
                        const uint32_t* offsets, cudaStream_t stream) {
  int g = lsd_grid(n);
#define GB_LSD_CASE(NWV)                                                                            \
  case NWV:                                                                                         \
    if (idx_in)                                                                                     \
      k_lsd_scatter<NWV, true><<<g, kThreads, 0, stream>>>(keys_in, idx_in, keys_out, idx_out, n,   \
                                                           word, shift, offsets);                   \
    else                                                                                            \
      k_lsd_scatter<NWV, false><<<g, kThreads, 0, stream>>>(keys_in, idx_in, keys_out, idx_out, n,  \
                                                            word, shift, offsets);                  \
    break;
  switch (nwords) {
    GB_LSD_CASE(1)
    GB_LSD_CASE(2)
    GB_LSD_CASE(3)
    GB_LSD_CASE(4)
    default:
      return cudaErrorInvalidValue;
  }
#undef GB_LSD_CASE
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t gather_records(const void* in, void* out, const uint32_t* idx, uint32_t n, uint32_t elsize,
                           cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  uintptr_t a = (uintptr_t)in | (uintptr_t)out;
  const uint8_t* i8 = (const uint8_t*)in;
  uint8_t* o8 = (uint8_t*)out;
  if (elsize % 16 == 0 && a % 16 == 0)
    k_gather<uint4><<<blocks_for((uint64_t)n * (elsize / 16), 256), 256, 0, stream>>>(i8, o8, idx, n, elsize);
  else if (elsize % 8 == 0 && a % 8 == 0)
    k_gather<uint2><<<blocks_for((uint64_t)n * (elsize / 8), 256), 256, 0, stream>>>(i8, o8, idx, n, elsize);
  else if (elsize % 4 == 0 && a % 4 == 0)
    k_gather<uint32_t><<<blocks_for((uint64_t)n * (elsize / 4), 256), 256, 0, stream>>>(i8, o8, idx, n, elsize);
  else
    k_gather<uint8_t><<<blocks_for((uint64_t)n * elsize, 256), 256, 0, stream>>>(i8, o8, idx, n, elsize);
  note_launches(1);
  return cudaGetLastError();
}

}  // namespace gb
