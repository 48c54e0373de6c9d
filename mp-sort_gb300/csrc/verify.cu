// verify.cu -- the multiset hash of a record array (the sort's self-check)
// and the first partition of sorts of 2^32 records or more.
//
// Self-check.  The reference checksums the records before and after its
// MPI sort and aborts on a mismatch (mpsort-mpi.c:148-159, 193, 324-330,
// a byte sum).  Here the check is an order-independent hash of the multiset
// of records: the sum, modulo 2^64, of a 64-bit mix of every record's
// bytes.  Equal multisets hash equally in any order; a changed, lost or
// duplicated record changes the sum except with probability about 2^-64.
//
// Large sorts.  The histogram sort indexes records with 32-bit offsets.  A
// sort of 2^32 records or more is first cut into P < 16 key ranges of
// under 2^32 records each by one stable partition pass with 64-bit offsets
// (the splitters are sample quantiles, as for the level-1 buckets); every
// range is then an independent sort.
#include "common.cuh"
#include "kernels.h"

namespace gb {

namespace {

// The 64-bit finaliser of MurmurHash3 (fmix64, a published mixing function).
__device__ __forceinline__ uint64_t fmix64(uint64_t z) {
  z ^= z >> 33;
  z *= 0xff51afd7ed558ccdull;
  z ^= z >> 33;
  z *= 0xc4ceb9fe1a85ec53ull;
  z ^= z >> 33;
  return z;
}

// Hash of one record: FNV-1a-style multiply chain over its 32-bit words
// (or bytes), finalised by fmix64.
__device__ __forceinline__ uint64_t record_hash_words(const uint32_t* w, uint32_t nw) {
  uint64_t h = 0xcbf29ce484222325ull ^ nw;
  for (uint32_t j = 0; j < nw; ++j) h = (h ^ w[j]) * 0x100000001b3ull;
  return fmix64(h);
}
__device__ __forceinline__ uint64_t record_hash_bytes(const uint8_t* b, uint32_t nb) {
  uint64_t h = 0xcbf29ce484222325ull ^ nb;
  for (uint32_t j = 0; j < nb; ++j) h = (h ^ b[j]) * 0x100000001b3ull;
  return fmix64(h);
}

__global__ void __launch_bounds__(256) k_multiset_hash(const uint8_t* __restrict__ rec, uint64_t n, uint32_t elsize,
                                                        int words, unsigned long long* __restrict__ out) {
  __shared__ unsigned long long part[8];
  unsigned long long sum = 0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint8_t* r = rec + i * elsize;
    sum += words ? record_hash_words(reinterpret_cast<const uint32_t*>(r), elsize / 4) : record_hash_bytes(r, elsize);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(GB_FULL_MASK, sum, o);
  if (lane_id() == 0) part[warp_id()] = sum;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long t = 0;
    for (int i = 0; i < 8; ++i) t += part[i];
    atomicAdd(out, t);
  }
}

// ---------------------------------------------------------- partition ----
constexpr int kPartThreads = 512;
constexpr int kPartRpt = 4;
constexpr int kPartTile = kPartThreads * kPartRpt;

__host__ __device__ __forceinline__ uint64_t part_chunk_begin(uint64_t n, uint32_t c, uint32_t g) {
  return (n / g) * c + (c < n % g ? c : n % g);
}

// Part of a key among nsplit (< 16) sorted splitters: #{S[j] <= key}.
__device__ __forceinline__ uint32_t part_of(const uint64_t* S, int nsplit, uint64_t key) {
  uint32_t p = 0;
  for (int j = 0; j < nsplit; ++j) p += S[j] <= key;
  return p;
}

__global__ void k_sample64(const uint8_t* __restrict__ rec, uint64_t n, uint32_t elsize, gbsort_key_word kw,
                           uint32_t s, uint64_t* __restrict__ out) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < s; i += gridDim.x * blockDim.x) {
    const uint64_t j = (n / s) * i + ((n % s) * i) / s;  // i * n / s without overflow (i < s < 2^32)
    out[i] = load_key_aligned4(rec + j * elsize, kw);
  }
}

__global__ void __launch_bounds__(kPartThreads) k_part_count(const uint8_t* __restrict__ rec, uint64_t n,
                                                              uint32_t elsize, gbsort_key_word kw,
                                                              const uint64_t* __restrict__ S, int nsplit,
                                                              uint32_t* __restrict__ counts, uint32_t g) {
  __shared__ uint64_t s_split[16];
  __shared__ uint32_t hist[16];
  if (threadIdx.x < 16) {
    hist[threadIdx.x] = 0;
    if ((int)threadIdx.x < nsplit) s_split[threadIdx.x] = S[threadIdx.x];
  }
  __syncthreads();
  const uint64_t cb = part_chunk_begin(n, blockIdx.x, g), ce = part_chunk_begin(n, blockIdx.x + 1, g);
  for (uint64_t i = cb + threadIdx.x; i < ce; i += kPartThreads)
    atomicAdd(&hist[part_of(s_split, nsplit, load_key_aligned4(rec + i * elsize, kw))], 1u);
  __syncthreads();
  if ((int)threadIdx.x <= nsplit) counts[(size_t)threadIdx.x * g + blockIdx.x] = hist[threadIdx.x];
}

template <int EW>
struct PartIO {
  static constexpr uint32_t E = EW * 4;
  using V = typename std::conditional<EW % 4 == 0, uint4,
                                      typename std::conditional<EW % 2 == 0, uint2, uint32_t>::type>::type;
  static constexpr int VPR = E / sizeof(V);
};

// Stable partition of each chunk: every tile is ranked by part (block
// ranking over 4-bit digits), records go to cursor[part] + their rank in
// the part's run of the tile; runs are long, so the stores coalesce.
template <int EW>
__global__ void __launch_bounds__(kPartThreads) k_part_scatter(const uint8_t* __restrict__ rec, uint8_t* __restrict__ out,
                                                                uint64_t n, gbsort_key_word kw,
                                                                const uint64_t* __restrict__ S, int nsplit,
                                                                const unsigned long long* __restrict__ offsets,
                                                                uint32_t g, uint32_t* err) {
  using IO = PartIO<EW>;
  using V = typename IO::V;
  constexpr uint32_t E = IO::E;
  using Rank = BlockRank<kPartRpt, 4, kPartThreads>;
  __shared__ uint64_t s_split[16];
  __shared__ unsigned long long cursor[16];
  __shared__ uint16_t hist[Rank::kCounters];
  __shared__ uint32_t scan_tmp[kPartThreads / 32];
  __shared__ uint32_t start[17];
  if (threadIdx.x < 16) {
    if ((int)threadIdx.x < nsplit) s_split[threadIdx.x] = S[threadIdx.x];
    cursor[threadIdx.x] = (int)threadIdx.x <= nsplit ? offsets[(size_t)threadIdx.x * g + blockIdx.x] : 0ull;
  }
  __syncthreads();
  const uint64_t cb = part_chunk_begin(n, blockIdx.x, g), ce = part_chunk_begin(n, blockIdx.x + 1, g);
  const uint32_t w = warp_id(), lane = lane_id();
  for (uint64_t t0 = cb; t0 < ce; t0 += kPartTile) {
    const uint32_t nvalid = (uint32_t)min((uint64_t)kPartTile, ce - t0);
    uint32_t digit[kPartRpt], pos[kPartRpt];
    V v[kPartRpt][IO::VPR];
#pragma unroll
    for (int r = 0; r < kPartRpt; ++r) {
      const uint32_t e = w * 32 * kPartRpt + r * 32 + lane;
      digit[r] = 15;  // padding ranks after every real item
      if (e < nvalid) {
        const uint8_t* src = rec + (t0 + e) * E;
#pragma unroll
        for (int q = 0; q < IO::VPR; ++q) v[r][q] = reinterpret_cast<const V*>(src)[q];
        digit[r] = part_of(s_split, nsplit, load_key_aligned4(src, kw));
      }
    }
    Rank::rank(digit, pos, hist, scan_tmp, start);
#pragma unroll
    for (int r = 0; r < kPartRpt; ++r) {
      const uint32_t e = w * 32 * kPartRpt + r * 32 + lane;
      if (e >= nvalid) continue;
      const unsigned long long dest = cursor[digit[r]] + (pos[r] - start[digit[r]]);
      if (dest >= n) {
        set_error(err, DEV_ERR_COUNT_MISMATCH);
        continue;
      }
      uint8_t* d = out + dest * E;
#pragma unroll
      for (int q = 0; q < IO::VPR; ++q) reinterpret_cast<V*>(d)[q] = v[r][q];
    }
    __syncthreads();
    if ((int)threadIdx.x <= nsplit) cursor[threadIdx.x] += start[threadIdx.x + 1] - start[threadIdx.x];
    __syncthreads();
  }
}

template <typename F>
bool dispatch_part_ew(uint32_t elsize, F&& f) {
  switch (elsize / 4) {
    case 2: f(std::integral_constant<int, 2>()); return true;
    case 3: f(std::integral_constant<int, 3>()); return true;
    case 4: f(std::integral_constant<int, 4>()); return true;
    case 6: f(std::integral_constant<int, 6>()); return true;
    case 8: f(std::integral_constant<int, 8>()); return true;
    case 10: f(std::integral_constant<int, 10>()); return true;
    case 12: f(std::integral_constant<int, 12>()); return true;
    case 16: f(std::integral_constant<int, 16>()); return true;
    default: return false;
  }
}

}  // namespace

cudaError_t multiset_hash(const void* rec, uint64_t n, uint32_t elsize, unsigned long long* out, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(out, 0, sizeof(unsigned long long), st);
  if (e != cudaSuccess || n == 0) return e;
  const int words = elsize % 4 == 0 && (uintptr_t)rec % 4 == 0;
  uint64_t blocks = (n + 255) / 256;
  const uint64_t cap = (uint64_t)num_sms() * 8;
  if (blocks > cap) blocks = cap;
  k_multiset_hash<<<(unsigned)blocks, 256, 0, st>>>((const uint8_t*)rec, n, elsize, words, out);
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t sample_keys64(const uint8_t* rec, uint64_t n, uint32_t elsize, gbsort_key_word key, uint32_t s,
                          uint64_t* out, cudaStream_t st) {
  k_sample64<<<(s + 255) / 256, 256, 0, st>>>(rec, n, elsize, key, s, out);
  note_launches(1);
  return cudaGetLastError();
}

int part_grid() { return num_sms() * 4; }

cudaError_t part_count(const uint8_t* rec, uint64_t n, uint32_t elsize, gbsort_key_word key, const uint64_t* S,
                       int nsplit, uint32_t* counts, cudaStream_t st) {
  if (nsplit < 0 || nsplit > 15) return cudaErrorInvalidValue;
  const int g = part_grid();
  k_part_count<<<g, kPartThreads, 0, st>>>(rec, n, elsize, key, S, nsplit, counts, (uint32_t)g);
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t part_scatter(const uint8_t* rec, uint8_t* out, uint64_t n, uint32_t elsize, gbsort_key_word key,
                         const uint64_t* S, int nsplit, const unsigned long long* offsets, uint32_t* err,
                         cudaStream_t st) {
  if (nsplit < 0 || nsplit > 15) return cudaErrorInvalidValue;
  const int g = part_grid();
  cudaError_t e = cudaSuccess;
  const bool ok = dispatch_part_ew(elsize, [&](auto ewc) {
    constexpr int EW = decltype(ewc)::value;
    k_part_scatter<EW><<<g, kPartThreads, 0, st>>>(rec, out, n, key, S, nsplit, offsets, (uint32_t)g, err);
    note_launches(1);
    e = cudaGetLastError();
  });
  return ok ? e : cudaErrorInvalidValue;
}

}  // namespace gb
