// lsd.cu -- the generic path: stable LSD radix sort of key words + index,
// then one record permutation.
//
// Serves every key the histogram sort does not take (multi-word radix,
// records whose size or alignment is not a multiple of 4 bytes, keys from a
// host radix() callback) and sorts the sample of the histogram sort.  It
// reproduces the reference's ordering -- a stable sort by the radix as a
// little-endian unsigned integer (radixsort.c:19-44, stdlib/msort.c:52-174)
// -- with 8-bit digit passes in a one-sweep design:
//   * one read of the keys builds the histograms of every digit; their
//     exclusive scans give each digit's first output slot in every pass
//     (and passes whose digit is constant can be skipped by the host);
//   * each pass is then ONE kernel: a CTA takes the next tile by ticket,
//     ranks its digits stably (warp match ranking), publishes the tile's
//     per-digit counts and looks back over the previous tiles' published
//     counts for its global offsets (decoupled look-back, bounded spins),
//     stages the tile in digit order in shared memory and writes it out in
//     runs, so every key is read once and written once per pass.
#include "common.cuh"
#include "kernels.h"

namespace gb {

namespace {

#ifndef GB_LSD_THREADS
#define GB_LSD_THREADS 512
#endif
// Key + index passes: 512-thread CTAs (tiles of 4096) measured 5% faster on
// 1e9 x 16 B than 256-thread ones (tiles of 2048).
constexpr int kLsdThreads = GB_LSD_THREADS;
constexpr int kLsdRpt = 8;                          // items per thread per tile
constexpr int kLsdTile = kLsdThreads * kLsdRpt;     // 4096

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

// Exclusive scans of the 256-bin histograms: one block per (word, digit).
__global__ void __launch_bounds__(256) k_digit_starts(const uint32_t* __restrict__ hist,
                                                      uint32_t* __restrict__ starts) {
  __shared__ uint32_t tmp[8];
  const uint32_t v = hist[blockIdx.x * 256 + threadIdx.x];
  starts[blockIdx.x * 256 + threadIdx.x] = block_exclusive_scan<uint32_t, 256>(v, tmp, nullptr);
}

// Look-back status word of (tile, digit): a 2-bit flag over a 62-bit count.
constexpr unsigned long long kStatAgg = 1ull << 62;     // the tile's own count
constexpr unsigned long long kStatPrefix = 2ull << 62;  // count of every tile up to this one
constexpr unsigned long long kStatValue = (1ull << 62) - 1;
constexpr uint32_t kLookbackSpins = 1u << 22;           // ~1 s of polling, then an error

__device__ __forceinline__ void st_relaxed(unsigned long long* p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ld_relaxed(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

// One LSD pass on digit (word, shift).  starts[d] = first output slot of
// digit d; status holds ntiles * 256 zeroed words; *ticket starts at 0.
template <int NW, bool IDX>
__global__ void __launch_bounds__(kLsdThreads) k_lsd_onesweep(const uint64_t* __restrict__ keys_in,
                                                            const uint32_t* __restrict__ idx_in,
                                                            uint64_t* __restrict__ keys_out,
                                                            uint32_t* __restrict__ idx_out, uint32_t n, int word,
                                                            int shift, const uint32_t* __restrict__ starts,
                                                            unsigned long long* status, uint32_t* ticket,
                                                            uint32_t* err, uint32_t spin_limit,
                                                            uint32_t withhold_tile) {
  using Rank = BlockRank<kLsdRpt, 8, kLsdThreads>;
  static_assert(kLsdThreads >= 256, "one thread per digit in the look-back");
  __shared__ uint16_t hist[Rank::kCounters];
  __shared__ uint32_t scan_tmp[kLsdThreads / 32];
  __shared__ uint32_t start[257];
  __shared__ uint32_t base[256];
  __shared__ uint32_t tile_s;
  extern __shared__ __align__(16) uint8_t smem[];
  uint64_t* skeys = reinterpret_cast<uint64_t*>(smem);  // [NW][kLsdTile], digit order
  uint32_t* sidx = reinterpret_cast<uint32_t*>(skeys + NW * kLsdTile);

  // tiles go out in ticket order, so every tile a CTA looks back at belongs
  // to a CTA that is already running
  if (threadIdx.x == 0) tile_s = atomicAdd(ticket, 1u);
  __syncthreads();
  const uint32_t tile = tile_s;
  const uint32_t t = tile * (uint32_t)kLsdTile;
  const uint32_t nvalid = min((uint32_t)kLsdTile, n - t);
  const uint32_t w = warp_id(), lane = lane_id();
  // only the digit's word stays in registers across the ranking; the other
  // words (and the index) are read after it, straight into place
  const uint64_t* kdig = keys_in + (size_t)word * n + t;
  uint64_t k[kLsdRpt];
  uint32_t digit[kLsdRpt], pos[kLsdRpt];
#pragma unroll
  for (int r = 0; r < kLsdRpt; ++r) {
    uint32_t e = w * 32 * kLsdRpt + r * 32 + lane;
    bool valid = e < nvalid;
    k[r] = valid ? kdig[e] : 0;
    // padding items take the last digit and, being last in the tile, rank
    // after every real item
    digit[r] = valid ? (uint32_t)(k[r] >> shift) & 255u : 255u;
  }
  Rank::rank(digit, pos, hist, scan_tmp, start);
#pragma unroll
  for (int r = 0; r < kLsdRpt; ++r) {
    const uint32_t e = w * 32 * kLsdRpt + r * 32 + lane;
    if (pos[r] < nvalid) {
#pragma unroll
      for (int q = 0; q < NW; ++q)
        skeys[q * kLsdTile + pos[r]] = q == word ? k[r] : keys_in[(size_t)q * n + t + e];
      if (IDX) sidx[pos[r]] = idx_in[t + e];
    }
  }
  if (threadIdx.x < 256) {
    const uint32_t d = threadIdx.x;
    uint32_t cnt = start[d + 1] - start[d];
    if (d == 255) cnt -= (uint32_t)kLsdTile - nvalid;
    unsigned long long* mine = status + (size_t)tile * 256 + d;
    unsigned long long excl = 0;
    // withhold_tile (a test of the bounded wait) never publishes, so the
    // next tile's wait runs out; it is ~0u in every sort
    const bool publish = tile != withhold_tile;
    if (tile == 0) {
      if (publish) st_relaxed(mine, kStatPrefix | cnt);
    } else {
      if (publish) st_relaxed(mine, kStatAgg | cnt);
      uint32_t j = tile - 1, spins = 0;
      for (;;) {
        const unsigned long long v = ld_relaxed(status + (size_t)j * 256 + d);
        const unsigned long long f = v & ~kStatValue;
        if (f == 0) {  // tile j has not published yet
          if (++spins > spin_limit) {
            set_error(err, DEV_ERR_TIMEOUT);
            break;
          }
          __nanosleep(spins < 32 ? 32 : 256);
          continue;
        }
        excl += v & kStatValue;
        if (f == kStatPrefix || j == 0) break;
        --j;
      }
      if (publish) st_relaxed(mine, kStatPrefix | (excl + cnt));
    }
    base[d] = starts[d] + (uint32_t)excl - start[d];
  }
  __syncthreads();
  // runs of equal digits go to consecutive output slots
  for (uint32_t i = threadIdx.x; i < nvalid; i += kLsdThreads) {
    const uint32_t d = (uint32_t)(skeys[word * kLsdTile + i] >> shift) & 255u;
    const uint32_t dest = base[d] + i;
    if (dest >= n) {
      set_error(err, DEV_ERR_COUNT_MISMATCH);
      continue;
    }
#pragma unroll
    for (int q = 0; q < NW; ++q) keys_out[(size_t)q * n + dest] = skeys[q * kLsdTile + i];
    if (IDX) idx_out[dest] = sidx[i];
  }
}

// ------------------------------------------------ record-carrying passes --
// Records of 8-32 bytes (4-byte words, key words at 4-byte offsets) can be
// moved by the digit passes themselves: each pass reads whole records in
// input order, ranks them by the digit of one key word taken from the
// registers, stages them in digit order in shared memory and writes them
// out in runs.  No key arrays, no index, no final gather (whose reads by
// index are random and fetch about a DRAM line per record): 2E bytes per
// record per pass.  Measured on 16-byte records the passes still take
// longer than key + index passes plus the gather (the one-tile-per-CTA
// passes are latency-bound, not bandwidth-bound), so this form is opt-in
// (GBSORT_LSD_RECORDS=1).
template <int EW, int NT = 256>
struct RecPass {
  static constexpr int kRpt = EW <= 4 ? 8 : 4;
  static constexpr int kTile = NT * kRpt;
  using V = typename std::conditional<EW % 4 == 0, uint4, typename std::conditional<EW % 2 == 0, uint2,
                                                                                  uint32_t>::type>::type;
  static constexpr int kVw = sizeof(V) / 4;       // words per vector
  static constexpr int kVpr = EW / kVw;           // vectors per record
  static constexpr size_t kSmem = (size_t)kTile * (EW * 4 + 1);
};

template <int EW>
__device__ __forceinline__ void rec_load(const uint8_t* p, uint32_t (&r)[EW]) {
  using V = typename RecPass<EW>::V;
  constexpr int VW = RecPass<EW>::kVw;
#pragma unroll
  for (int i = 0; i < RecPass<EW>::kVpr; ++i) {
    const V v = reinterpret_cast<const V*>(p)[i];
    const uint32_t* w = reinterpret_cast<const uint32_t*>(&v);
#pragma unroll
    for (int j = 0; j < VW; ++j) r[i * VW + j] = w[j];
  }
}

template <int EW>
__device__ __forceinline__ void rec_store(uint8_t* p, const uint32_t (&r)[EW]) {
  using V = typename RecPass<EW>::V;
  constexpr int VW = RecPass<EW>::kVw;
#pragma unroll
  for (int i = 0; i < RecPass<EW>::kVpr; ++i) {
    V v;
    uint32_t* w = reinterpret_cast<uint32_t*>(&v);
#pragma unroll
    for (int j = 0; j < VW; ++j) w[j] = r[i * VW + j];
    reinterpret_cast<V*>(p)[i] = v;
  }
}

// Histograms of all 8 digits of every key word, read from the records.
template <int EW>
__global__ void __launch_bounds__(kThreads) k_record_digit_hist(const uint8_t* __restrict__ in, uint32_t n,
                                                                 gbsort_key_desc key,
                                                                 uint32_t* __restrict__ hist) {
  __shared__ uint32_t h[4 * 8 * 256];
  const int nw = (int)key.nwords;
  for (int i = threadIdx.x; i < nw * 8 * 256; i += kThreads) h[i] = 0;
  __syncthreads();
  for (uint32_t i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
    uint32_t r[EW];
    rec_load<EW>(in + (size_t)i * (EW * 4), r);
    for (int w = 0; w < nw; ++w) {
      const uint64_t k = key_from_regs<EW>(r, key.word[w]);
#pragma unroll
      for (int d = 0; d < 8; ++d) atomicAdd(&h[(w * 8 + d) * 256 + ((k >> (8 * d)) & 255)], 1u);
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nw * 8 * 256; i += kThreads)
    if (h[i]) atomicAdd(&hist[i], h[i]);
}

// One record-carrying pass on digit (word, shift); status holds
// tiles * 256 zeroed words, *ticket starts at 0 (as k_lsd_onesweep).
template <int EW, int NT>
__global__ void __launch_bounds__(NT, 3) k_lsd_records(const uint8_t* __restrict__ in,
                                                                     uint8_t* __restrict__ out, uint32_t n,
                                                                     gbsort_key_word kw, int shift,
                                                                     const uint32_t* __restrict__ starts,
                                                                     unsigned long long* status, uint32_t* ticket,
                                                                     uint32_t* err, uint32_t spin_limit) {
  static_assert(NT >= 256, "one thread per digit in the look-back");
  constexpr int RPT = RecPass<EW, NT>::kRpt, T = RecPass<EW, NT>::kTile;
  constexpr uint32_t E = EW * 4;
  using Rank = BlockRank<RPT, 8, NT>;
  using V = typename RecPass<EW, NT>::V;
  constexpr int VPR = RecPass<EW, NT>::kVpr;
  __shared__ uint16_t hist[Rank::kCounters];
  __shared__ uint32_t scan_tmp[NT / 32];
  __shared__ uint32_t start[257];
  __shared__ uint32_t base[256];
  __shared__ uint32_t tile_s;
  extern __shared__ __align__(16) uint8_t smem[];
  uint8_t* stage = smem;                     // [T] records, digit order
  uint8_t* sdig = smem + (size_t)T * E;      // [T] their digits

  if (threadIdx.x == 0) tile_s = atomicAdd(ticket, 1u);
  __syncthreads();
  const uint32_t tile = tile_s;
  const uint32_t t = tile * (uint32_t)T;
  const uint32_t nvalid = min((uint32_t)T, n - t);
  const uint32_t w = warp_id(), lane = lane_id();
  uint32_t rec[RPT][EW];
  uint32_t digit[RPT], pos[RPT];
#pragma unroll
  for (int r = 0; r < RPT; ++r) {
    const uint32_t e = w * 32 * RPT + r * 32 + lane;
    digit[r] = 255u;  // padding items take the last digit and rank after every real item
    if (e < nvalid) {
      rec_load<EW>(in + (size_t)(t + e) * E, rec[r]);
      digit[r] = (uint32_t)(key_from_regs<EW>(rec[r], kw) >> shift) & 255u;
    }
  }
  Rank::rank(digit, pos, hist, scan_tmp, start);
#pragma unroll
  for (int r = 0; r < RPT; ++r)
    if (pos[r] < nvalid) {
      rec_store<EW>(stage + (size_t)pos[r] * E, rec[r]);
      sdig[pos[r]] = (uint8_t)digit[r];
    }
  if (threadIdx.x < 256) {
    const uint32_t d = threadIdx.x;
    uint32_t cnt = start[d + 1] - start[d];
    if (d == 255) cnt -= (uint32_t)T - nvalid;
    unsigned long long* mine = status + (size_t)tile * 256 + d;
    unsigned long long excl = 0;
    if (tile == 0) {
      st_relaxed(mine, kStatPrefix | cnt);
    } else {
      st_relaxed(mine, kStatAgg | cnt);
      uint32_t j = tile - 1, spins = 0;
      for (;;) {
        const unsigned long long v = ld_relaxed(status + (size_t)j * 256 + d);
        const unsigned long long f = v & ~kStatValue;
        if (f == 0) {  // tile j has not published yet
          if (++spins > spin_limit) {
            set_error(err, DEV_ERR_TIMEOUT);
            break;
          }
          __nanosleep(spins < 32 ? 32 : 256);
          continue;
        }
        excl += v & kStatValue;
        if (f == kStatPrefix || j == 0) break;
        --j;
      }
      st_relaxed(mine, kStatPrefix | (excl + cnt));
    }
    base[d] = starts[d] + (uint32_t)excl - start[d];
  }
  __syncthreads();
  // runs of equal digits go to consecutive output slots; consecutive threads
  // take consecutive vectors of consecutive records
  for (uint32_t f = threadIdx.x; f < nvalid * VPR; f += NT) {
    const uint32_t i = f / VPR, q = f % VPR;
    const uint32_t dest = base[sdig[i]] + i;
    if (dest >= n) {
      set_error(err, DEV_ERR_COUNT_MISMATCH);
      continue;
    }
    reinterpret_cast<V*>(out + (size_t)dest * E)[q] = reinterpret_cast<const V*>(stage + (size_t)i * E)[q];
  }
}

// Pseudo-random bytes: word i of the buffer is a 64-bit mix of (i, seed).
__global__ void k_fill_hash(uint32_t* __restrict__ p, uint64_t nwords, uint64_t seed) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nwords;
       i += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t z = (i + 1) * 0x9E3779B97F4A7C15ull ^ seed;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    p[i] = (uint32_t)((z ^ (z >> 31)) >> 16);
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

cudaError_t lsd_digit_starts(const uint32_t* hist, int nwords, uint32_t* starts, cudaStream_t stream) {
  k_digit_starts<<<8 * nwords, 256, 0, stream>>>(hist, starts);
  note_launches(1);
  return cudaGetLastError();
}

uint32_t lsd_tiles(uint32_t n) { return (uint32_t)(((uint64_t)n + kLsdTile - 1) / kLsdTile); }

template <typename F>
static bool dispatch_rec_ew(uint32_t elsize, F&& f) {
  switch (elsize / 4) {
    case 2: f(std::integral_constant<int, 2>()); return true;
    case 3: f(std::integral_constant<int, 3>()); return true;
    case 4: f(std::integral_constant<int, 4>()); return true;
    case 5: f(std::integral_constant<int, 5>()); return true;
    case 6: f(std::integral_constant<int, 6>()); return true;
    case 7: f(std::integral_constant<int, 7>()); return true;
    case 8: f(std::integral_constant<int, 8>()); return true;
    default: return false;
  }
}

bool lsd_records_supported(uint32_t elsize, const void* in, const void* out, const gbsort_key_desc& key) {
  if (elsize % 4 || elsize < 8 || elsize > 32 || key.nwords < 1 || key.nwords > 4) return false;
  for (uint32_t w = 0; w < key.nwords; ++w)
    if (key.word[w].offset % 4 || key.word[w].offset + key.word[w].width > elsize) return false;
  const uint32_t vec = elsize % 16 == 0 ? 16 : (elsize % 8 == 0 ? 8 : 4);
  return ((uintptr_t)in | (uintptr_t)out) % vec == 0;
}

// Threads per CTA of the record passes: 256 (tiles of 8 or 4 records per
// thread; four CTAs per SM) beat 512 (two per SM) by 1.3x on 1e9 x 16 B.
constexpr int kRecThreads = 256;

uint32_t lsd_record_tiles(uint32_t n, uint32_t elsize) {
  uint32_t tile = 0;
  dispatch_rec_ew(elsize, [&](auto ewc) { tile = RecPass<decltype(ewc)::value, kRecThreads>::kTile; });
  return tile ? (uint32_t)(((uint64_t)n + tile - 1) / tile) : 0;
}

cudaError_t lsd_record_histograms(const void* in, uint32_t n, uint32_t elsize, const gbsort_key_desc& key,
                                  uint32_t* hist, cudaStream_t stream) {
  cudaError_t e = cudaMemsetAsync(hist, 0, sizeof(uint32_t) * 8 * 256 * key.nwords, stream);
  if (e != cudaSuccess || n == 0) return e;
  const bool ok = dispatch_rec_ew(elsize, [&](auto ewc) {
    constexpr int EW = decltype(ewc)::value;
    k_record_digit_hist<EW><<<blocks_for(n, kThreads), kThreads, 0, stream>>>((const uint8_t*)in, n, key, hist);
  });
  if (!ok) return cudaErrorInvalidValue;
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t lsd_record_pass(const void* in, void* out, uint32_t n, uint32_t elsize, const gbsort_key_desc& key,
                            int word, int shift, const uint32_t* starts, unsigned long long* status,
                            uint32_t* ticket, uint32_t* err, cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  const uint32_t tiles = lsd_record_tiles(n, elsize);
  cudaError_t e = cudaMemsetAsync(status, 0, sizeof(unsigned long long) * 256 * (size_t)tiles, stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(ticket, 0, sizeof(uint32_t), stream);
  if (e != cudaSuccess) return e;
  auto launch = [&](auto kern, size_t smem, int nt) {
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess)
      kern<<<tiles, nt, smem, stream>>>((const uint8_t*)in, (uint8_t*)out, n, key.word[word], shift, starts, status,
                                        ticket, err, kLookbackSpins);
  };
  const bool ok = dispatch_rec_ew(elsize, [&](auto ewc) {
    constexpr int EW = decltype(ewc)::value;
    launch(k_lsd_records<EW, kRecThreads>, RecPass<EW, kRecThreads>::kSmem, kRecThreads);
  });
  if (!ok) return cudaErrorInvalidValue;
  if (e != cudaSuccess) return e;
  note_launches(1);
  return cudaGetLastError();
}

template <int NW, bool IDX>
static cudaError_t launch_onesweep(const uint64_t* keys_in, const uint32_t* idx_in, uint64_t* keys_out,
                                   uint32_t* idx_out, uint32_t n, int word, int shift, const uint32_t* starts,
                                   unsigned long long* status, uint32_t* ticket, uint32_t* err,
                                   uint32_t spin_limit, uint32_t withhold_tile, cudaStream_t stream) {
  const size_t smem = (size_t)NW * kLsdTile * 8 + (IDX ? (size_t)kLsdTile * 4 : 0);
  cudaError_t e = cudaFuncSetAttribute(k_lsd_onesweep<NW, IDX>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  k_lsd_onesweep<NW, IDX><<<lsd_tiles(n), kLsdThreads, smem, stream>>>(keys_in, idx_in, keys_out, idx_out, n, word,
                                                                     shift, starts, status, ticket, err,
                                                                     spin_limit, withhold_tile);
  return cudaGetLastError();
}

cudaError_t lsd_onesweep(const uint64_t* keys_in, const uint32_t* idx_in, uint64_t* keys_out, uint32_t* idx_out,
                         uint32_t n, int nwords, int word, int shift, const uint32_t* starts,
                         unsigned long long* status, uint32_t* ticket, uint32_t* err, cudaStream_t stream,
                         uint32_t spin_limit, uint32_t withhold_tile) {
  if (n == 0) return cudaSuccess;
  if (spin_limit == 0) spin_limit = kLookbackSpins;
  const size_t words = (size_t)256 * lsd_tiles(n);
  cudaError_t e;
  if ((void*)ticket == (void*)(status + words)) {  // the usual layout: one clear for both
    e = cudaMemsetAsync(status, 0, sizeof(unsigned long long) * words + sizeof(uint32_t), stream);
  } else {
    e = cudaMemsetAsync(status, 0, sizeof(unsigned long long) * words, stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(ticket, 0, sizeof(uint32_t), stream);
  }
  if (e != cudaSuccess) return e;
#define GB_LSD_CASE(NWV)                                                                                       \
  case NWV:                                                                                                    \
    e = idx_in ? launch_onesweep<NWV, true>(keys_in, idx_in, keys_out, idx_out, n, word, shift, starts, status,  \
                                            ticket, err, spin_limit, withhold_tile, stream)                    \
               : launch_onesweep<NWV, false>(keys_in, idx_in, keys_out, idx_out, n, word, shift, starts,       \
                                             status, ticket, err, spin_limit, withhold_tile, stream);          \
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
  return e;
}

cudaError_t fill_hash(void* p, size_t nbytes, uint64_t seed, cudaStream_t stream) {
  const uint64_t nw = nbytes / 4;
  if (nw == 0) return cudaSuccess;
  k_fill_hash<<<blocks_for(nw, 256), 256, 0, stream>>>((uint32_t*)p, nw, seed);
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
