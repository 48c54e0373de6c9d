// hsort.cu -- the histogram sort: the GB300 form of mpsort_omp's
// sample / split / exchange / local-sort pipeline for single-word keys.
//
//   reference stage (mpsort-omp.c)          device stage (this file)
//   ------------------------------------    ----------------------------------
//   radix_sort of each chunk (:247)          sample_keys + LSD sort of a sample
//   Pmin/Pmax, piter bisection (:251-295)    k_plain_splitters / learned model
//   _histogram + _reduce_sum (:286-289)      k_l1_count: (bucket x chunk) counts
//   _solve_for_layout (:331)                 scan of the count matrix
//   memcpy exchange (:338-369)               k_l1_scatter: stable bucket scatter
//   radix_sort of each chunk again (:389)    k_tasks: split + shared-memory sort
//
// Records stay whole (any size that is a multiple of 4 bytes, up to 64) and
// the result is the stable order by key, record for record.  The buffers:
// input -> scratch A (level 1), A -> scratch B (bucket splits), and every
// final local sort writes the output, so the output may alias the input.
#include "cdf.cuh"
#include "common.cuh"
#include "kernels.h"

#include <type_traits>

namespace gb {

int num_sms();

namespace {

// Local-sort shape (overridable at build time for tuning sweeps).
#ifndef GB_LOCAL_MAX
#define GB_LOCAL_MAX 2048
#endif
#ifndef GB_LOCAL_THREADS
#define GB_LOCAL_THREADS 256
#endif
#ifndef GB_LOCAL_CTAS
#define GB_LOCAL_CTAS 3
#endif
#ifndef GB_STAGED_THREADS
#define GB_STAGED_THREADS 512
#endif
constexpr int kLocalMax = GB_LOCAL_MAX;          // records a local sort holds in shared memory
constexpr int kLocalThreads = GB_LOCAL_THREADS;  // threads of a local-sort CTA
constexpr int kLocalCtasPerSm = GB_LOCAL_CTAS;
constexpr int kStagedThreads = GB_STAGED_THREADS;  // threads of a staged local-sort CTA (two per SM)
// Three CTAs per SM give 80 registers a thread: the local sort's pass calls
// then need almost no stack (at four CTAs, 64 registers, the saves around
// every call doubled the kernel's L2 stores; 1e9 x 16 B: 14.1 against 15.2
// ms), and records above 16 bytes keep L1 room for the gather's reads of the
// group (5e8 x 40 B: 13.1 ms with three, 18.4 ms with four).
template <int EW>
constexpr int local_ctas_per_sm() {
  return kLocalCtasPerSm;
}
constexpr int kLocalBits = 11;         // bins of the local counting pass (about one record each)
constexpr int kInsertMax = 24;         // bins up to this size use insertion sort
#ifndef GB_SPLIT_BITS
#define GB_SPLIT_BITS 12
#endif
constexpr int kSplitBits = GB_SPLIT_BITS;  // bins of a bucket split
constexpr int kSplitBins = 1 << kSplitBits;
constexpr int kFineBins = 2 * kSplitBins;  // bins of a split after crowded bins are refined
#ifndef GB_SPLIT_CROWDED
#define GB_SPLIT_CROWDED 512
#endif
constexpr uint32_t kCrowded = GB_SPLIT_CROWDED;  // records of a split bin that get it refined (at least)
// Buckets below this many records are not refined: their second histogram
// read costs more than the re-splits it saves (small segments sit in L2).
constexpr uint32_t kRefineMin = 1u << 17;
constexpr int kMaxGroups = 512;        // sub-buckets per split
constexpr int kGroupBits = 9;          // bits of a group id
static_assert((1 << kGroupBits) == kMaxGroups, "group ids fill kGroupBits");
constexpr int kMaxBucketBits = 12;     // bits of a level-1 bucket id (at most 4096 buckets)
constexpr uint32_t kCopyPiece = 1u << 16;

__host__ __device__ __forceinline__ uint32_t chunk_begin(uint32_t n, uint32_t c, uint32_t g) {
  return (uint32_t)(((uint64_t)n * c / g) & ~(uint64_t)31);
}
__host__ __device__ __forceinline__ uint32_t chunk_end(uint32_t n, uint32_t c, uint32_t g) {
  return c + 1 == g ? n : chunk_begin(n, c + 1, g);
}

// ------------------------------------------------------------ record I/O --
// A record of EW 32-bit words moved with the widest vector that divides it.
template <int EW>
struct RecIO {
  __device__ __forceinline__ static void load(const uint8_t* p, uint32_t (&r)[EW]) {
    if constexpr (EW % 4 == 0) {
#pragma unroll
      for (int i = 0; i < EW / 4; ++i) {
        uint4 v = reinterpret_cast<const uint4*>(p)[i];
        r[4 * i] = v.x; r[4 * i + 1] = v.y; r[4 * i + 2] = v.z; r[4 * i + 3] = v.w;
      }
    } else if constexpr (EW % 2 == 0) {
#pragma unroll
      for (int i = 0; i < EW / 2; ++i) {
        uint2 v = reinterpret_cast<const uint2*>(p)[i];
        r[2 * i] = v.x; r[2 * i + 1] = v.y;
      }
    } else {
#pragma unroll
      for (int i = 0; i < EW; ++i) r[i] = reinterpret_cast<const uint32_t*>(p)[i];
    }
  }
  // Same, for data read exactly once: evict-first, so the stream does not
  // push out of L2 the partly written bucket lines of the scatter.
  __device__ __forceinline__ static void load_stream(const uint8_t* p, uint32_t (&r)[EW]) {
    if constexpr (EW % 4 == 0) {
#pragma unroll
      for (int i = 0; i < EW / 4; ++i) {
        uint4 v = __ldcs(reinterpret_cast<const uint4*>(p) + i);
        r[4 * i] = v.x; r[4 * i + 1] = v.y; r[4 * i + 2] = v.z; r[4 * i + 3] = v.w;
      }
    } else if constexpr (EW % 2 == 0) {
#pragma unroll
      for (int i = 0; i < EW / 2; ++i) {
        uint2 v = __ldcs(reinterpret_cast<const uint2*>(p) + i);
        r[2 * i] = v.x; r[2 * i + 1] = v.y;
      }
    } else {
#pragma unroll
      for (int i = 0; i < EW; ++i) r[i] = __ldcs(reinterpret_cast<const unsigned int*>(p) + i);
    }
  }
  __device__ __forceinline__ static void store(uint8_t* p, const uint32_t (&r)[EW]) {
    if constexpr (EW % 4 == 0) {
#pragma unroll
      for (int i = 0; i < EW / 4; ++i)
        reinterpret_cast<uint4*>(p)[i] = make_uint4(r[4 * i], r[4 * i + 1], r[4 * i + 2], r[4 * i + 3]);
    } else if constexpr (EW % 2 == 0) {
#pragma unroll
      for (int i = 0; i < EW / 2; ++i) reinterpret_cast<uint2*>(p)[i] = make_uint2(r[2 * i], r[2 * i + 1]);
    } else {
#pragma unroll
      for (int i = 0; i < EW; ++i) reinterpret_cast<uint32_t*>(p)[i] = r[i];
    }
  }
};

// Block copy of `count` records of EW words from src to dst (distinct).
template <int EW>
__device__ __forceinline__ void block_copy(const uint8_t* src, uint8_t* dst, uint32_t count) {
  constexpr int E = EW * 4;
  if constexpr (EW % 4 == 0) {
    const uint64_t nv = (uint64_t)count * (E / 16);
    for (uint64_t f = threadIdx.x; f < nv; f += kThreads)
      reinterpret_cast<uint4*>(dst)[f] = reinterpret_cast<const uint4*>(src)[f];
  } else if constexpr (EW % 2 == 0) {
    const uint64_t nv = (uint64_t)count * (E / 8);
    for (uint64_t f = threadIdx.x; f < nv; f += kThreads)
      reinterpret_cast<uint2*>(dst)[f] = reinterpret_cast<const uint2*>(src)[f];
  } else {
    const uint64_t nv = (uint64_t)count * EW;
    for (uint64_t f = threadIdx.x; f < nv; f += kThreads)
      reinterpret_cast<uint32_t*>(dst)[f] = reinterpret_cast<const uint32_t*>(src)[f];
  }
}

__device__ __forceinline__ uint64_t key_at(const uint8_t* base, uint32_t i, uint32_t elsize,
                                           const gbsort_key_word& kw) {
  return load_key_aligned4(base + (size_t)i * elsize, kw);
}

// --------------------------------------------------------------- sample --
__global__ void k_sample(const uint8_t* __restrict__ rec, uint32_t n, uint32_t elsize,
                         gbsort_key_word kw, uint32_t s, uint64_t* __restrict__ out) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < s; i += gridDim.x * blockDim.x) {
    uint32_t j = (uint32_t)((uint64_t)i * n / s);
    out[i] = key_at(rec, j, elsize, kw);
  }
}

// ----------------------------------------------------- plain splitters --
// One thread per splitter runs the reference's bisection for that splitter
// (piter_bisect / _histogram / piter_accept, internal-parallel.h:150-248)
// against the sorted sample, which plays the role of the locally sorted
// chunks.  The splitters never interact, so running each one's rounds to
// completion independently gives the same values as the reference's
// lock-step rounds; `iters` receives the number of rounds of the slowest.
__device__ __forceinline__ uint32_t count_lt(const uint64_t* a, uint32_t n, uint64_t p) {
  uint32_t lo = 0, hi = n;
  while (lo < hi) {
    uint32_t m = (lo + hi) >> 1;
    if (a[m] < p) lo = m + 1; else hi = m;
  }
  return lo;
}
__device__ __forceinline__ uint32_t count_le(const uint64_t* a, uint32_t n, uint64_t p) {
  uint32_t lo = 0, hi = n;
  while (lo < hi) {
    uint32_t m = (lo + hi) >> 1;
    if (a[m] <= p) lo = m + 1; else hi = m;
  }
  return lo;
}

__global__ void k_plain_splitters(const uint64_t* __restrict__ sample, uint32_t s, int nsplit,
                                  uint64_t* __restrict__ P, uint32_t* iters, int64_t* clt,
                                  int64_t* cle) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nsplit) return;
  const int64_t C = (int64_t)((uint64_t)s * (uint64_t)(i + 1) / (uint64_t)(nsplit + 1));
  uint64_t left = sample[0], right = sample[s - 1], p = left;
  bool narrow = false;
  uint32_t it = 0;
  for (;;) {
    ++it;
    if (narrow) {           // last round: test right itself, then stop
      p = right;
      break;
    }
    p = left + ((right - left) >> 1);
    if (p <= left) narrow = true;
    int64_t lt = count_lt(sample, s, p), le = count_le(sample, s, p);
    if (lt < C && C <= le) break;
    if (lt >= C) right = p; else left = p;
    if (it > 200) break;    // cannot happen for 64-bit keys; keeps the loop bounded
  }
  P[i] = p;
  atomicMax(iters, it);
  if (clt) clt[i] = count_lt(sample, s, p);
  if (cle) cle[i] = count_le(sample, s, p);
}

// Runs of equal splitters become single-key buckets: [.., k, k, k, ..] ->
// [.., k, k+1, k+1, ..], so every record of a heavy key k lands in the bucket
// [k, k+1) and needs no sort at all.
__global__ void __launch_bounds__(1024) k_finalize_splitters(uint64_t* S, int nsplit, const uint32_t* only_if) {
  constexpr int PER = 8;  // nsplit <= 8192
  if (only_if && *only_if == 0) return;
  uint64_t cur[PER], prev[PER];
#pragma unroll
  for (int j = 0; j < PER; ++j) {
    int i = threadIdx.x + j * 1024;
    cur[j] = i < nsplit ? S[i] : 0;
    prev[j] = (i > 0 && i < nsplit) ? S[i - 1] : 0;
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < PER; ++j) {
    int i = threadIdx.x + j * 1024;
    if (i > 0 && i < nsplit && cur[j] == prev[j] && cur[j] != ~0ull) S[i] = cur[j] + 1;
  }
}

// ------------------------------------------------------- heavy keys ------
__device__ __forceinline__ uint32_t heavy_hash(uint64_t key) {
  return (uint32_t)((key * 0x9E3779B97F4A7C15ull) >> (64 - kHeavyLog2));
}

__global__ void __launch_bounds__(1024) k_heavy_table(const uint64_t* __restrict__ S, int nsplit,
                                                      HeavyTable* __restrict__ t, uint32_t* held) {
  for (int i = threadIdx.x; i < kHeavySlots; i += blockDim.x) t->slot[i].bucket1 = 0;
  if (threadIdx.x == 0) t->n = t->probes = 0;
  __syncthreads();
  for (int i = threadIdx.x; i + 2 < nsplit; i += blockDim.x) {
    const uint64_t a = S[i], b = S[i + 1];
    if (a + 1 != b || S[i + 2] != b) continue;  // bucket i + 1 is not [a, a + 1) worth two splitters
    const uint32_t h = heavy_hash(a);
    // copies of b from i + 1 on: at least two, below 2^13; bucket i + 1 < 2^14
    const uint32_t m = upper_bound_in(S, (uint32_t)i + 1, (uint32_t)nsplit, b) - ((uint32_t)i + 1);
    for (int j = 0; j < kHeavyProbes; ++j) {  // a key that finds no slot keeps the ordinary lookup
      HeavySlot& sl = t->slot[(h + j) & (kHeavySlots - 1)];
      if (atomicCAS(&sl.bucket1, 0u, (uint32_t)i + 2) == 0) {
        sl.key = a;
        sl.weight = (m << 14) | ((uint32_t)i + 1);
        atomicAdd(&t->n, 1u);
        atomicMax(&t->probes, (uint32_t)j + 1);
        break;
      }
    }
  }
  __syncthreads();
  if (threadIdx.x == 0 && held) *held = t->n;
}

// The weight word of `key` if the table holds it (its bucket in the low 14
// bits), else 0.  probes: the table's longest probe sequence, 0 for an empty
// or absent table.
constexpr uint32_t kHeavyBucketMask = 0x3fffu;  // level-1 buckets are at most 8192 (k_finalize_splitters)
__device__ __forceinline__ uint32_t heavy_lookup(const HeavyTable* t, uint32_t probes, uint64_t key) {
  const uint32_t h = heavy_hash(key);
  for (uint32_t j = 0; j < probes; ++j) {
    const uint4 s = __ldg(reinterpret_cast<const uint4*>(&t->slot[(h + j) & (kHeavySlots - 1)]));
    if (s.z == 0) break;
    if ((((uint64_t)s.y << 32) | s.x) == key) return s.w;
  }
  return 0;
}
// ---------------------------------------------------------- lookups ------
struct LookupSmem {
  uint64_t* S;
  float2* knots;
  uint32_t* win;
};

template <int LK>
__device__ __forceinline__ uint32_t lookup(const LookupSmem& L, const ModelDev& m, int nbuckets,
                                           uint64_t key, uint32_t* misses) {
  if constexpr (LK == LOOKUP_PLAIN) return bucket_plain(L.S, nbuckets, key);
  else return bucket_learned(L.S, m, L.knots, L.win, key, misses);
}

// Loads the lookup tables into shared memory at `smem` and returns the first
// free byte.  The plain lookup binary-searches every splitter, so they go to
// shared memory; the learned lookup touches at most a couple of splitters
// per key (its window), so it reads them through the L1 cache and keeps
// only the model's knots and windows in shared memory -- which leaves room
// for more resident CTAs.
template <int LK>
__device__ __forceinline__ uint8_t* load_lookup(uint8_t* smem, const uint64_t* S, int nbuckets,
                                                const ModelDev& m, LookupSmem& L) {
  if constexpr (LK == LOOKUP_PLAIN) {
    L.S = reinterpret_cast<uint64_t*>(smem);
    for (int i = threadIdx.x; i < nbuckets - 1; i += blockDim.x) L.S[i] = S[i];
    smem += 8 * (size_t)((nbuckets + 1) & ~1);
  } else {
    L.S = const_cast<uint64_t*>(S);
  }
  if constexpr (LK == LOOKUP_LEARNED) {
    const int nl = 1 << m.lbits;
    L.knots = reinterpret_cast<float2*>(smem);
    for (int i = threadIdx.x; i < nl; i += blockDim.x) L.knots[i] = m.knots[i];
    smem += 8 * (size_t)nl;
    L.win = reinterpret_cast<uint32_t*>(smem);
    for (int i = threadIdx.x; i < nl; i += blockDim.x) L.win[i] = m.win[i];
    smem += 4 * (size_t)nl;
  }
  return smem;
}

template <int LK>
size_t lookup_smem_bytes(int nbuckets, const ModelDev* m) {
  if (LK == LOOKUP_LEARNED) return 12 * ((size_t)1 << m->lbits);
  return 8 * (size_t)((nbuckets + 1) & ~1);
}

// ----------------------------------------------------- level-1 count ------
// Counts of records [cb, ce) per bucket into hist.  HEAVY: probe the
// heavy-key table (hprobes > 0) first.
template <int LK, bool HEAVY>
__device__ __forceinline__ void count_range(const HsortParams& p, const LookupSmem& L, const ModelDev& model,
                                            int nbuckets, uint32_t* hist, uint32_t* stats, uint32_t cb, uint32_t ce,
                                            uint32_t hprobes) {
  constexpr int U = 8;
  // keys of the next batch are loaded while the current batch is counted
  uint64_t k[U], kn[U];
#pragma unroll
  for (int u = 0; u < U; ++u) {
    uint32_t i = cb + u * kThreads + threadIdx.x;
    kn[u] = i < ce ? key_at(p.in, i, p.elsize, p.key) : 0;
  }
  for (uint32_t base = cb; base < ce; base += kThreads * U) {
#pragma unroll
    for (int u = 0; u < U; ++u) {
      k[u] = kn[u];
      uint32_t i = base + kThreads * U + u * kThreads + threadIdx.x;
      kn[u] = i < ce ? key_at(p.in, i, p.elsize, p.key) : 0;
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      uint32_t i = base + u * kThreads + threadIdx.x;
      const bool v = i < ce;
      if constexpr (!HEAVY) {
        if (v) {
          const uint32_t b = lookup<LK>(L, model, nbuckets, k[u], stats + STAT_WINDOW_MISS);
          atomicAdd(&hist[b], 1u);
          if (p.bkt) p.bkt[i] = (uint16_t)b;
        }
        continue;
      }
      uint32_t hw = v ? heavy_lookup(p.heavy, hprobes, k[u]) : 0;
      uint32_t b = hw & kHeavyBucketMask;
      if (v && !hw) {
        b = lookup<LK>(L, model, nbuckets, k[u], stats + STAT_WINDOW_MISS);
        atomicAdd(&hist[b], 1u);
      }
      if (v && p.bkt) p.bkt[i] = (uint16_t)b;
      // records of heavy keys: one match over the warp groups them, one
      // atomic per distinct key (many lanes adding to one counter
      // serialise; Zipf keys at 1e9 x 16 B: count 10.0 -> 8.7 ms against
      // atomics for the warp's two heaviest keys and one per other record)
      if (__any_sync(GB_FULL_MASK, hw != 0)) {
        const uint32_t peers = __match_any_sync(GB_FULL_MASK, hw);
        if (hw && lane_id() == (uint32_t)(__ffs(peers) - 1)) atomicAdd(&hist[hw & kHeavyBucketMask], __popc(peers));
      }
    }
  }
}

template <int LK>
__global__ void __launch_bounds__(kThreads, 2) k_l1_count(HsortParams p, const uint64_t* __restrict__ S,
                                                        int nbuckets, ModelDev model,
                                                        uint32_t* __restrict__ counts,
                                                        uint32_t* __restrict__ stats, uint32_t c0, uint32_t nchunks) {
  model = resolve_model(model);
  extern __shared__ __align__(16) uint8_t smem[];
  LookupSmem L;
  uint32_t* hist = reinterpret_cast<uint32_t*>(load_lookup<LK>(smem, S, nbuckets, model, L));
  if constexpr (LK == LOOKUP_LEARNED) {
    // the learned lookup's window searches read splitters from shared
    // memory here too (the count has room for them): keys next to heavy-key
    // steps have wide windows (Zipf keys, 1e9 x 16 B: count 8.7 -> 7.9 ms;
    // 5e8 x 40 B Morton keys 3.8 -> 3.4 ms)
    uint64_t* Ss = reinterpret_cast<uint64_t*>(hist + ((nbuckets + 1) & ~1));
    for (int i = threadIdx.x; i < nbuckets - 1; i += kThreads) Ss[i] = S[i];
    L.S = Ss;
  }
  for (int i = threadIdx.x; i < nbuckets; i += kThreads) hist[i] = 0;
  __syncthreads();
  const uint32_t hprobes = p.heavy ? p.heavy->probes : 0;
  const uint32_t c = c0 + blockIdx.x, g = nchunks;  // this CTA's chunk of the nchunks
  const uint32_t cb = chunk_begin(p.n, c, g), ce = chunk_end(p.n, c, g);
  if (hprobes) count_range<LK, true>(p, L, model, nbuckets, hist, stats, cb, ce, hprobes);
  else count_range<LK, false>(p, L, model, nbuckets, hist, stats, cb, ce, 0);
  __syncthreads();
  for (int b = threadIdx.x; b < nbuckets; b += kThreads) counts[(size_t)b * g + c] = hist[b];
}

// --------------------------------------------------- warp-row ranking ---
// Stable ranking of a tile by a bucket id without a block-wide sort.  Items
// are in warp-chunk order (item r of lane l in warp w is element
// w * 32 * RPT + r * 32 + l); cnt is a shared [buckets][kWarps] byte table
// (a warp holds at most 32 * RPT <= 128 items of one bucket), all zero on
// entry.
//   warp_ranks (then a barrier):  each warp ranks its items with ballot
//       matches and adds its per-bucket counts to its column of cnt;
//   tile_rank (then a barrier):   an item's rank in its bucket's run of the
//       tile is the counts of the warps before its own plus its rank in its
//       warp; `all` is the run's length;
//   clear_rows (then a barrier):  the warps zero the entries they touched.
// kNoBucket marks padding items.
constexpr uint32_t kNoBucket = 0xffffffffu;
static_assert(kWarps == 16, "a table row is one 16-byte vector");

// Ids are below 2^BITS (BITS unrolled ballots match them).  Padding items
// sit above every real item of their row (the valid items of a tile are a
// prefix), so they may share a label with real items: they are masked out
// of every count.
template <int RPT, int BITS>
__device__ __forceinline__ void warp_ranks(const uint32_t (&bkt)[RPT], uint32_t (&rank)[RPT], uint32_t (&lead)[RPT],
                                           uint8_t* cnt) {
  static_assert(RPT <= 7, "per-warp counts must fit a byte");
  const uint32_t w = warp_id(), lane = lane_id();
#pragma unroll
  for (int r = 0; r < RPT; ++r) {
    const uint32_t valid = __ballot_sync(GB_FULL_MASK, bkt[r] != kNoBucket);
    const uint32_t peers = match_bits<BITS>(bkt[r]) & valid;
    const uint32_t leader = __ffs(peers) - 1;
    uint32_t old = 0;
    if (lane == leader && bkt[r] != kNoBucket) {
      uint8_t* slot = cnt + (size_t)bkt[r] * kWarps + w;
      old = *slot;
      *slot = (uint8_t)(old + __popc(peers));
    }
    old = __shfl_sync(GB_FULL_MASK, old, leader);
    rank[r] = old + __popc(peers & lanemask_lt());
    lead[r] = lane == leader;
    __syncwarp();
  }
}

// Selectors of the earlier warps' bytes of a table row: entry w has byte j
// set to 1 for j < w (warp-uniform reads of the constant bank).
#define GB_EARLIER(n) ((n) <= 0 ? 0u : (n) >= 4 ? 0x01010101u : (0x01010101u >> (8 * (4 - (n)))))
#define GB_EARLIER_ROW(w) {GB_EARLIER(w), GB_EARLIER((w) - 4), GB_EARLIER((w) - 8), GB_EARLIER((w) - 12)}
__constant__ uint4 kEarlierWarps[kWarps] = {
    GB_EARLIER_ROW(0),  GB_EARLIER_ROW(1),  GB_EARLIER_ROW(2),  GB_EARLIER_ROW(3),
    GB_EARLIER_ROW(4),  GB_EARLIER_ROW(5),  GB_EARLIER_ROW(6),  GB_EARLIER_ROW(7),
    GB_EARLIER_ROW(8),  GB_EARLIER_ROW(9),  GB_EARLIER_ROW(10), GB_EARLIER_ROW(11),
    GB_EARLIER_ROW(12), GB_EARLIER_ROW(13), GB_EARLIER_ROW(14), GB_EARLIER_ROW(15)};
#undef GB_EARLIER_ROW
#undef GB_EARLIER

__device__ __forceinline__ uint32_t tile_rank(uint32_t b, uint32_t rank, const uint8_t* cnt, uint32_t& all) {
  const uint4 x = *reinterpret_cast<const uint4*>(cnt + (size_t)b * kWarps);
  const uint4 k = kEarlierWarps[warp_id()];
  // byte dot products: with 0x01 selectors the row's total, with this
  // warp's selectors the counts of the warps before it
  all = __dp4a(x.w, 0x01010101u, __dp4a(x.z, 0x01010101u, __dp4a(x.y, 0x01010101u, __dp4a(x.x, 0x01010101u, 0u))));
  return __dp4a(x.w, k.w, __dp4a(x.z, k.z, __dp4a(x.y, k.y, __dp4a(x.x, k.x, rank))));
}

template <int RPT>
__device__ __forceinline__ void clear_rows(const uint32_t (&bkt)[RPT], const uint32_t (&lead)[RPT], uint8_t* cnt) {
#pragma unroll
  for (int r = 0; r < RPT; ++r)
    if (lead[r] && bkt[r] != kNoBucket) cnt[(size_t)bkt[r] * kWarps + warp_id()] = 0;
}

// --------------------------------------------------- level-1 scatter ------
template <int EW>
struct Tile {
  static constexpr int kRpt = (16 / EW) < 1 ? 1 : ((16 / EW) > 4 ? 4 : (16 / EW));
  static constexpr int kSize = kThreads * kRpt;
};
#ifndef GB_SCATTER_RPT
#define GB_SCATTER_RPT 16
#endif
// Records of 20 bytes and more: each thread also holds the next tile's
// records in registers (loaded while the current tile is ranked; 5e8 x 40 B
// scatter 22.1 ms against 23.9 ms without).  Records of 8-16 bytes come
// from L2 instead (each tile is prefetched two tiles ahead): with the
// register copy the kernel spills at 64 registers, and 1e9 x 16 B scatters
// in 17.38 ms against 17.19 ms without.  GB_SCATTER_PREFETCH=0 / 1 forces
// either form.
#ifndef GB_SCATTER_PREFETCH
#define GB_SCATTER_PREFETCH -1
#endif
// Tiles between a scatter tile's L2 prefetch and its loads (1e9 x 16 B: 1
// and 2 scatter in the same 17.2 ms).
#ifndef GB_SCATTER_L2_AHEAD
#define GB_SCATTER_L2_AHEAD 2
#endif
#ifndef GB_SCATTER_CTAS
#define GB_SCATTER_CTAS 2  // level-1 scatter CTAs per SM (the register budget follows)
#endif
// Tile of the level-1 scatter: up to GB_SCATTER_RPT / EW records per thread.
template <int EW>
struct ScatterTile {
  // records of 24-40 bytes: two per thread (a tile of 1024; the staged tile
  // still leaves room for two CTAs per SM)
  static constexpr int kRpt = (EW >= 6 && EW <= 10) ? 2
                              : (GB_SCATTER_RPT / EW) < 1 ? 1
                              : ((GB_SCATTER_RPT / EW) > 7 ? 7 : (GB_SCATTER_RPT / EW));
  static constexpr int kSize = kThreads * kRpt;
  static constexpr bool kPrefetch = GB_SCATTER_PREFETCH < 0 ? EW >= 5 : GB_SCATTER_PREFETCH != 0;
};

// u16 entries of one bucket-id buffer of the scatter: a tile's ids plus the
// 16-byte rounding of a bulk copy.
template <int EW>
__host__ __device__ constexpr uint32_t scatter_id_buf() {
  return (ScatterTile<EW>::kSize * 2 + 32 + 15) / 16 * 8;
}

// One 32-byte store (a whole DRAM sector, one memory request; two 16-byte
// stores to scattered places cost a request each).  p is 32-byte aligned.
// No memory clobber: the kernels that use it never read the sectors they
// write, so the loads around it may move across it.
__device__ __forceinline__ void store_sector(uint8_t* p, const uint4& a, const uint4& b) {
  asm volatile("st.global.v8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"l"(p), "r"(a.x), "r"(a.y), "r"(a.z),
               "r"(a.w), "r"(b.x), "r"(b.y), "r"(b.z), "r"(b.w));
}

// Unrolled iterations of a staged split's write-out loop: four at 12 and 16
// bytes a record (no spills), two at 8 (four would spill).
template <int EW>
__host__ __device__ constexpr int split_outs_unroll() {
  return EW >= 3 ? 4 : 2;
}

// Global stores with no memory clobber, for write-outs whose destinations
// the kernel never reads back: the shared-memory loads of the following
// records may move above them (a store through a plain pointer, which might
// address shared memory, keeps every later shared-memory load below it).
__device__ __forceinline__ void st_global(uint4* p, const uint4& v) {
  asm volatile("st.global.v4.b32 [%0], {%1, %2, %3, %4};" ::"l"(__cvta_generic_to_global(p)), "r"(v.x), "r"(v.y),
               "r"(v.z), "r"(v.w));
}
__device__ __forceinline__ void st_global(uint2* p, const uint2& v) {
  asm volatile("st.global.v2.b32 [%0], {%1, %2};" ::"l"(__cvta_generic_to_global(p)), "r"(v.x), "r"(v.y));
}
__device__ __forceinline__ void st_global(uint32_t* p, uint32_t v) {
  asm volatile("st.global.b32 [%0], %1;" ::"l"(__cvta_generic_to_global(p)), "r"(v));
}

// Stable scatter of each chunk into its buckets.  Per tile of T records
// (RPT per thread, in warp-chunk order), without a block-wide sort:
//   1. each warp ranks its own records by bucket (warp_ranks);
//   2. after one barrier, every record's rank in its bucket's run of the
//      tile gives its destination cursor[bucket] + rank (tile_rank);
//   3. after a second barrier, the last record of each run advances the
//      cursor and each warp clears the table entries it touched.
// Cursors start at the scanned (bucket, chunk) offsets, so chunk order and
// tile order are both preserved.
//
// Write combining (16-byte records): a 32-byte DRAM sector holds two
// records.  Two neighbours in the same run are written in the same phase
// and meet in L2; but a run usually has one record, and its sector partner
// comes a tile later -- a half-written sector that L2 may evict, costing
// an ECC read-modify-write in DRAM.  So the last record of a run whose
// destination starts a sector is held in shared memory (one slot per
// bucket) and written together with its partner, the next tile's first
// record of that bucket; slots still held at the chunk's end are flushed.
template <int EW>
__global__ void __launch_bounds__(kThreads, GB_SCATTER_CTAS) k_l1_scatter(HsortParams p, int nbuckets,
                                                                           const uint32_t* __restrict__ offsets,
                                                                           int nchunks, uint32_t* __restrict__ stats,
                                                                           uint32_t c0, uint32_t c1,
                                                                           const uint32_t* __restrict__ skip_if) {
  if (skip_if && *skip_if) return;  // a reserved region overflowed: the exact path redoes level 1
  uint32_t* err = stats + STAT_SLOTS;  // the error word follows the statistics
  constexpr int RPT = ScatterTile<EW>::kRpt, T = ScatterTile<EW>::kSize;
  constexpr bool kPre = ScatterTile<EW>::kPrefetch;
  constexpr uint32_t kAhead = GB_SCATTER_L2_AHEAD;  // tiles between a tile's L2 prefetch and its loads
  constexpr bool kCombine = EW == 4;
  constexpr uint32_t E = EW * 4;
  constexpr uint32_t kNoSlot = 0xffffffffu;
  extern __shared__ __align__(16) uint8_t smem[];
  uint8_t* q = smem;
  uint32_t* cursor = reinterpret_cast<uint32_t*>(q);
  q += 4 * (size_t)((nbuckets + 3) & ~3);
  uint32_t* held_at = reinterpret_cast<uint32_t*>(q);  // destination of the held record, or kNoSlot
  if (kCombine) q += 4 * (size_t)((nbuckets + 3) & ~3);
  uint4* held = reinterpret_cast<uint4*>(q);  // the held record of each bucket
  if (kCombine) q += 16 * (size_t)nbuckets;
  // other record sizes: the tile and its destinations, written out by
  // consecutive threads taking consecutive words of a record (one memory
  // request per record or two, not one per word)
  uint8_t* stage = q;
  if (!kCombine) q += (size_t)T * E;
  uint32_t* wdest = reinterpret_cast<uint32_t*>(q);
  if (!kCombine) q += 4 * (size_t)T;
  uint8_t* cnt = q;  // [nbuckets][kWarps]
  q += (size_t)nbuckets * kWarps;
  // the bucket ids of the next two tiles come into shared memory by bulk
  // asynchronous copies (no registers held for them)
  uint16_t* idbuf = reinterpret_cast<uint16_t*>(q);  // [2][kIdBuf]
  constexpr uint32_t kIdBuf = scatter_id_buf<EW>();
  uint64_t* ibar = reinterpret_cast<uint64_t*>(q + 4 * (size_t)kIdBuf);
  for (int i = threadIdx.x; i < nbuckets * kWarps / 16; i += kThreads)
    reinterpret_cast<uint4*>(cnt)[i] = make_uint4(0, 0, 0, 0);
  uint32_t ipar = 0;  // next completion parity of each id buffer
  if (threadIdx.x == 0) {
    mbar_init(&ibar[0], 1);
    mbar_init(&ibar[1], 1);
    mbar_init_fence();
  }
  // ids of the tile starting at record t (chunk end ce) into buffer b
  auto issue_ids = [&](uint32_t t, uint32_t ce_, int b) {
    const uint32_t cnt_ = min((uint32_t)T, ce_ - t);
    bulk_load(idbuf + (size_t)b * kIdBuf, p.bkt + t, (cnt_ * 2 + 15) & ~15u, &ibar[b]);
  };

  const uint32_t w = warp_id(), lane = lane_id();
  // the count kernel's chunks, several per CTA
  for (uint32_t c = c0 + blockIdx.x; c < c1; c += gridDim.x) {
  const uint32_t g = (uint32_t)nchunks;
  const uint32_t cb = chunk_begin(p.n, c, g), ce = chunk_end(p.n, c, g);
  __syncthreads();
  for (int b = threadIdx.x; b < nbuckets; b += kThreads) {
    cursor[b] = offsets[(size_t)b * g + c];
    if (kCombine) held_at[b] = kNoSlot;
  }
  __syncthreads();

  if (threadIdx.x == 0) {  // (the barrier above ended every read of both buffers)
    fence_proxy_async_smem();
    if (cb < ce) issue_ids(cb, ce, 0);
    if (cb + T < ce) issue_ids(cb + T, ce, 1);
  }
  // the next tile's records are loaded while the current tile is ranked
  uint32_t nxt[kPre ? RPT : 1][EW];
  if constexpr (kPre) {
#pragma unroll
    for (int r = 0; r < RPT; ++r) {
      uint32_t e = w * 32 * RPT + r * 32 + lane;
      if (cb + e < ce) RecIO<EW>::load_stream(p.in + (size_t)(cb + e) * E, nxt[r]);
    }
  }
  for (uint32_t t0 = cb, tk = 0; t0 < ce; t0 += T, ++tk) {
    const int ib = (int)(tk & 1);
    const bool id_ok = mbar_wait_bounded(&ibar[ib], (ipar >> ib) & 1u, kBulkWaitPolls);
    ipar ^= 1u << ib;
    const uint32_t nvalid = min((uint32_t)T, ce - t0);
    if (threadIdx.x == 0 && t0 + kAhead * T < ce)
      prefetch_l2_range(p.in + (size_t)(t0 + kAhead * T) * E, min((uint32_t)T, ce - t0 - kAhead * T) * E);
    uint32_t rec[RPT][EW];
    uint32_t bkt[RPT], rank[RPT];
#pragma unroll
    for (int r = 0; r < RPT; ++r) {
      const uint32_t et = w * 32 * RPT + r * 32 + lane;  // in the tile
      bkt[r] = kNoBucket;
      if (et < nvalid) bkt[r] = min((uint32_t)idbuf[(size_t)ib * kIdBuf + et], (uint32_t)nbuckets - 1);
      if constexpr (kPre) {
#pragma unroll
        for (int q2 = 0; q2 < EW; ++q2) rec[r][q2] = nxt[r][q2];
        uint32_t e = t0 + T + et;
        if (e < ce) RecIO<EW>::load_stream(p.in + (size_t)e * E, nxt[r]);
      } else {
        uint32_t e = t0 + et;
        if (e < ce) RecIO<EW>::load_stream(p.in + (size_t)e * E, rec[r]);
      }
    }
    // 1. ranks within the warp, in (r, lane) order (a wait for ids that ran
    // out leaves in-range ids behind: the CTA stops at the barrier)
    uint32_t lead[RPT];
    warp_ranks<RPT, kMaxBucketBits>(bkt, rank, lead, cnt);
    if (!__syncthreads_and(id_ok)) {
      if (threadIdx.x == 0) set_error(err, DEV_ERR_TIMEOUT);
      mbar_wait_bounded(&ibar[ib], ((ipar >> ib) & 1u) ^ 1u, kBulkWaitPolls);  // (the parity flipped above)
      if (t0 + T < ce) mbar_wait_bounded(&ibar[ib ^ 1], (ipar >> (ib ^ 1)) & 1u, kBulkWaitPolls);
      return;
    }
    // every thread has read this tile's ids: the buffer takes the tile after next
    if (threadIdx.x == 0 && t0 + 2 * T < ce) {
      fence_proxy_async_smem();
      issue_ids(t0 + 2 * T, ce, ib);
    }
    // 2. rank in the tile = counts of the earlier warps + rank in the warp
    uint32_t tot[RPT];
    uint32_t holds = 0;  // bit r: row r starts a sector whose partner comes later
    if constexpr (!kCombine) {  // each record to the staged tile, its destination beside it
#pragma unroll
      for (int r = 0; r < RPT; ++r) {
        tot[r] = 0;
        const uint32_t e = w * 32 * RPT + r * 32 + lane;
        wdest[e] = kNoSlot;
        if (bkt[r] == kNoBucket) continue;
        uint32_t all;
        const uint32_t at = tile_rank(bkt[r], rank[r], cnt, all);
        const uint32_t dest = cursor[bkt[r]] + at;
        tot[r] = at + 1 == all ? all : 0;  // the run's last record advances the cursor
        if (dest >= p.a_cap) {
          set_error(err, DEV_ERR_COUNT_MISMATCH);
          continue;
        }
        RecIO<EW>::store(stage + (size_t)e * E, rec[r]);
        wdest[e] = dest;
      }
    } else {
      // 16-byte records, stored from registers: every row's table reads
      // come first (they are independent, so they are in flight together),
      // then the stores; rank[] becomes the destination
      uint32_t completes = 0;  // bit r: row r completes its bucket's held sector
#pragma unroll
      for (int r = 0; r < RPT; ++r) {
        tot[r] = 0;
        if (bkt[r] == kNoBucket) continue;
        uint32_t all;
        const uint32_t at = tile_rank(bkt[r], rank[r], cnt, all);
        rank[r] = cursor[bkt[r]] + at;
        tot[r] = at + 1 == all ? all : 0;
        if ((rank[r] & 1u) && at == 0 && held_at[bkt[r]] == rank[r] - 1) completes |= 1u << r;
      }
#pragma unroll
      for (int r = 0; r < RPT; ++r) {
        if (bkt[r] == kNoBucket) continue;
        const uint32_t dest = rank[r];
        if (dest >= p.a_cap) {
          set_error(err, DEV_ERR_COUNT_MISMATCH);
          continue;
        }
        uint8_t* to = p.bufA + (size_t)dest * E;
        if ((dest & 1u) == 0 && tot[r]) {
          holds |= 1u << r;
          continue;
        }
        if ((completes >> r) & 1u) {
          store_sector(to - 16, held[bkt[r]], make_uint4(rec[r][0], rec[r][1], rec[r][2], rec[r][3]));
          continue;
        }
        RecIO<EW>::store(to, rec[r]);
      }
    }
    __syncthreads();
    if constexpr (!kCombine) {
      using V = typename std::conditional<E % 16 == 0, uint4,
                                          typename std::conditional<E % 8 == 0, uint2, uint32_t>::type>::type;
      constexpr uint32_t VPR = E / sizeof(V);
      for (uint32_t f = threadIdx.x; f < nvalid * VPR; f += kThreads) {
        const uint32_t i = f / VPR, qw = f % VPR;
        const uint32_t d = wdest[i];
        if (d != kNoSlot)
          reinterpret_cast<V*>(p.bufA + (size_t)d * E)[qw] = reinterpret_cast<const V*>(stage + (size_t)i * E)[qw];
      }
    }
    // 3. advance the cursors, hold the open sectors, clear the rows
#pragma unroll
    for (int r = 0; r < RPT; ++r) {
      if (tot[r]) cursor[bkt[r]] += tot[r];
      if constexpr (kCombine) {
        if ((holds >> r) & 1u) {
          held[bkt[r]] = make_uint4(rec[r][0], rec[r][1], rec[r][2], rec[r][3]);
          held_at[bkt[r]] = rank[r];
        } else if (bkt[r] != kNoBucket && tot[r]) {
          held_at[bkt[r]] = kNoSlot;  // the run ended on a completed sector
        }
      }
    }
    clear_rows<RPT>(bkt, lead, cnt);
    __syncthreads();
  }
  if constexpr (kCombine) {  // the chunk's open sectors
    for (int b = threadIdx.x; b < nbuckets; b += kThreads)
      if (held_at[b] != kNoSlot) reinterpret_cast<uint4*>(p.bufA)[held_at[b]] = held[b];
  }
  }
}

template <int EW>
size_t l1_scatter_smem(int nbuckets) {
  const size_t words = 4 * (size_t)((nbuckets + 3) & ~3);
  const size_t combine = EW == 4 ? words + 16 * (size_t)nbuckets : 0;
  const size_t stage = EW == 4 ? 0 : (size_t)ScatterTile<EW>::kSize * (EW * 4 + 4);
  const size_t ids = 4 * (size_t)scatter_id_buf<EW>() + 16;  // two id buffers and their mbarriers
  return words + combine + stage + (size_t)nbuckets * kWarps + ids;
}

// ------------------------------------------------------------- tasks -----
// Level 2 runs as two kinds of persistent kernels over device task lists:
//   k_split  -- one CTA per SM takes buckets larger than kLocalMax, splits
//               each by a histogram of its key range and appends the pieces
//               to the local list (small), the next split list (still
//               large) or as copies (one key);
//   k_local  -- two CTAs per SM drain the local list: shared-memory sorts
//               and copies, all writing the final output.
// Local tasks only read their own ranges of A / B, which later splits never
// touch, so one k_local launch after the last split round serves them all.
struct TaskLists {
  const SortTask* split_in;
  const uint32_t* nsplit_in;
  SortTask* split_out;
  uint32_t* nsplit_out;
  SortTask* local;
  uint32_t* nlocal;
  uint32_t cap_split;
  uint32_t cap_local;
};

__device__ __forceinline__ void push(SortTask* list, uint32_t* n, uint32_t cap, const SortTask& t, uint32_t* err) {
  uint32_t at = atomicAdd(n, 1u);
  if (at < cap) list[at] = t;
  else set_error(err, DEV_ERR_TASK_OVERFLOW);
}

// Copies of single-key ranges go to the local list in pieces of kCopyPiece:
// records [from, from + cnt) of the buffer `flags` names to output
// positions [start, start + cnt).
__device__ __forceinline__ void push_copy(const TaskLists& L, uint32_t start, uint32_t from, uint32_t cnt,
                                          uint64_t lo, uint64_t hi, uint32_t flags, uint32_t* err) {
  for (uint32_t s0 = 0; s0 < cnt; s0 += kCopyPiece)
    push(L.local, L.nlocal, L.cap_local,
         make_task_at(start + s0, from + s0, min(kCopyPiece, cnt - s0), lo, hi, flags | TASK_COPY), err);
}

__global__ void k_build_tasks(const uint32_t* __restrict__ offsets, int grid,
                              const uint64_t* __restrict__ S, int nbuckets, uint32_t n, TaskLists L,
                              uint32_t* err, uint32_t* stats, int b0, int b1) {
  int b = b0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= b1) return;
  uint32_t start = offsets[(size_t)b * grid];
  uint32_t end = b + 1 < nbuckets ? offsets[(size_t)(b + 1) * grid] : n;
  uint32_t cnt = end - start;
  if (cnt == 0) return;
  atomicMax(stats + STAT_MAX_BUCKET, cnt);
  uint64_t lo = b == 0 ? 0ull : S[b - 1];
  uint64_t hi = b == nbuckets - 1 ? ~0ull : S[b] - 1;
  if (lo == hi || cnt == 1) push_copy(L, start, start, cnt, lo, hi, 0u, err);
  else if (cnt <= (uint32_t)kLocalMax) push(L.local, L.nlocal, L.cap_local, make_task(start, cnt, lo, hi, false, false), err);
  else push(L.split_out, L.nsplit_out, L.cap_split, make_task_at(start, start, cnt, lo, hi, TASK_L1), err);
}

// Largest split task first: the level-1 buckets differ in size by tens of
// percent and each is one CTA's work, so handing out the large ones first
// shortens the round's tail (longest-processing-time order).  One block
// sorts (~count, index) keys by a bitonic network and permutes the list in
// place; lists above kOrderMax tasks are left as they are.
constexpr int kOrderMax = 4096;
__global__ void __launch_bounds__(1024) k_order_tasks(SortTask* list, const uint32_t* n_ptr) {
  __shared__ unsigned long long key[kOrderMax];
  const uint32_t n = *n_ptr;
  if (n < 2 || n > (uint32_t)kOrderMax) return;
  uint32_t np = 1;
  while (np < n) np <<= 1;
  for (uint32_t i = threadIdx.x; i < np; i += blockDim.x)
    key[i] = i < n ? ((unsigned long long)(~list[i].count) << 32) | i : ~0ull;
  __syncthreads();
  for (uint32_t k = 2; k <= np; k <<= 1)
    for (uint32_t j = k >> 1; j > 0; j >>= 1) {
      for (uint32_t i = threadIdx.x; i < np; i += blockDim.x) {
        const uint32_t l = i ^ j;
        if (l > i) {
          const unsigned long long a = key[i], b = key[l];
          const bool up = (i & k) == 0;
          if ((a > b) == up) {
            key[i] = b;
            key[l] = a;
          }
        }
      }
      __syncthreads();
    }
  SortTask mine[kOrderMax / 1024];
#pragma unroll
  for (int q = 0; q < kOrderMax / 1024; ++q) {
    const uint32_t i = threadIdx.x + q * 1024;
    if (i < n) mine[q] = list[(uint32_t)key[i]];
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < kOrderMax / 1024; ++q) {
    const uint32_t i = threadIdx.x + q * 1024;
    if (i < n) list[i] = mine[q];
  }
}

// Block copy with four independent vector loads in flight per thread.
template <int EW>
__device__ __forceinline__ void block_copy_ilp(const uint8_t* src, uint8_t* dst, uint32_t count, int nthreads) {
  constexpr int E = EW * 4;
  using V = typename std::conditional<EW % 4 == 0, uint4, typename std::conditional<EW % 2 == 0, uint2, uint32_t>::type>::type;
  const uint64_t nv = (uint64_t)count * E / sizeof(V);
  const V* s = reinterpret_cast<const V*>(src);
  V* d = reinterpret_cast<V*>(dst);
  constexpr int U = sizeof(V) >= 16 ? 2 : 4;
  for (uint64_t f0 = threadIdx.x; f0 < nv; f0 += (uint64_t)nthreads * U) {
    V v[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      uint64_t f = f0 + (uint64_t)u * nthreads;
      if (f < nv) v[u] = s[f];
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      uint64_t f = f0 + (uint64_t)u * nthreads;
      if (f < nv) d[f] = v[u];
    }
  }
}

template <int NT>
struct LocalSmemT {
  static constexpr int kNW = NT / 32;
  uint64_t keyA[kLocalMax];  // keys in input order (then staging of big bins)
  uint64_t keyB[kLocalMax];  // keys in sorted order
  uint16_t idxA[kLocalMax];
  uint16_t idxB[kLocalMax];
  uint32_t cnt[(1 << kLocalBits) + 1];    // bin counts, then (scanned in place) bin starts and the end
  uint16_t big[kLocalMax / (kInsertMax + 1) + 2];  // start of pending bins
  uint16_t bigsz[kLocalMax / (kInsertMax + 1) + 2];
  uint32_t nbig;
  uint64_t red[2 * kNW];
  uint32_t scan_tmp[kNW];
  uint32_t task_id;
  SortTask next;
  uint32_t pend_id;  // the task claimed for after the next one, and its descriptor
  SortTask pend;
};
constexpr int kSplitTileBytes = kThreads * 64;  // a scatter tile: kThreads * RPT records of <= 16 / RPT words
static_assert(kFineBins * 4 <= kSplitTileBytes, "the fine histogram fits the staging tile");
// Staged splits (records of 8-16 bytes): the bucket streams through two
// tile buffers filled by bulk asynchronous copies, each a tile's bytes plus
// the 16-byte rounding of both its ends.
constexpr int kSplitBufBytes = 24576 + 128;
constexpr int kSplitStageBytes = 2 * kSplitBufBytes;
static_assert(kSplitStageBytes >= kSplitTileBytes, "the staging area holds an unstaged tile");
template <int EW>
__host__ __device__ constexpr bool split_staged() {
  return EW >= 2 && EW <= 4;
}
// Records per staged tile: 24 KB of 16-byte records, 2048 smaller ones.
template <int EW>
__host__ __device__ constexpr int staged_split_tile() {
  return EW == 4 ? 1536 : 2048;
}
// Shared memory of a split; SB: bytes of the staging area (kSplitTileBytes,
// or kSplitStageBytes for staged splits -- the unstaged splits and the
// engine keep the smaller one, which leaves L1 more room for their loads).
template <int SB>
struct SplitSmemT {
  static constexpr bool kStaged = SB > kSplitTileBytes;
  __align__(128) uint8_t stage[SB];  // the tile in group order, or two staged tiles
  uint16_t sgrp[kThreads * 4];                // group of each record in group order
  uint16_t perm[kStaged ? kThreads * 4 : 1];  // staged: input slot of each record in group order
  uint32_t goff[kMaxGroups];                     // first staged slot of each group
  uint32_t hist[kSplitBins];  // bin counts; for refined bins then (first fine bin << 4 | sub-bin bits)
  uint16_t gmap[kFineBins];
  uint32_t cursor[kMaxGroups];
  __align__(16) uint8_t gcnt[kMaxGroups * kWarps];  // warp-row ranking table, zero between tiles
  uint64_t red[2 * kWarps];
  uint32_t gstart[kMaxGroups + 1];
  uint32_t gfirst[kMaxGroups + 1];
  uint32_t scan_tmp[kWarps];
  uint32_t task_id;
  SortTask next;
  uint32_t emit_base;  // the engine's reservation for this split's groups
  uint64_t bar[2];     // staged tiles: completion of each buffer's copy
  uint32_t uflag;      // uniform splits: attempt decision, then a group outgrew its region
};
using SplitSmem = SplitSmemT<kSplitTileBytes>;
using SplitSmemStaged = SplitSmemT<kSplitStageBytes>;
template <int EW>
using SplitSmemOf = typename std::conditional<split_staged<EW>(), SplitSmemStaged, SplitSmem>::type;

template <int NT = kThreads>
__device__ __forceinline__ void block_minmax(uint64_t& mn, uint64_t& mx, uint64_t* red) {
  constexpr int NW = NT / 32;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    uint64_t a = __shfl_xor_sync(GB_FULL_MASK, mn, o), b = __shfl_xor_sync(GB_FULL_MASK, mx, o);
    mn = a < mn ? a : mn;
    mx = b > mx ? b : mx;
  }
  if (lane_id() == 0) {
    red[warp_id()] = mn;
    red[NW + warp_id()] = mx;
  }
  __syncthreads();
  mn = red[0];
  mx = red[NW];
#pragma unroll
  for (int i = 1; i < NW; ++i) {
    mn = red[i] < mn ? red[i] : mn;
    mx = red[NW + i] > mx ? red[NW + i] : mx;
  }
  __syncthreads();
}

// Places the packed words at positions [a, a+s) of keyA in order when they
// span fewer than 2^kLocalBits values from mn -- a run of equal keys, whose
// words differ only in their input indices: each word sets its bit in a
// bitmap of the span, and its rank is the number of set bits below it (the
// words are distinct).  As many barriers as a counting pass over the span,
// but 64 bitmap words to clear and prefix-count where the pass clears and
// scans 2048 bin counters.  sm.cnt holds the bitmap and its prefix counts;
// the words go through keyB.
template <int NT, typename SM>
__device__ __forceinline__ void local_bitmap_place(SM& sm, uint32_t a, uint32_t s, uint64_t mn) {
  constexpr int PER = kLocalMax / NT;
  constexpr int kWords = (1 << kLocalBits) / 32;
  static_assert(kWords == 64, "two bitmap words per lane of one warp");
  uint32_t* bits = sm.cnt;
  uint32_t* below = sm.cnt + kWords;  // set bits in the words before each word
  for (int i = threadIdx.x; i < kWords; i += NT) bits[i] = 0;
  __syncthreads();
#pragma unroll
  for (int r = 0; r < PER; ++r) {
    const uint32_t e = r * NT + threadIdx.x;
    if (e < s) {
      const uint32_t d = (uint32_t)(sm.keyA[a + e] - mn);
      atomicOr(&bits[d >> 5], 1u << (d & 31));
    }
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    const uint32_t lane = threadIdx.x;
    const uint32_t c0 = __popc(bits[2 * lane]), c1 = __popc(bits[2 * lane + 1]);
    uint32_t inc = c0 + c1;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(GB_FULL_MASK, inc, o);
      if (lane >= (uint32_t)o) inc += t;
    }
    below[2 * lane] = inc - c0 - c1;
    below[2 * lane + 1] = inc - c1;
  }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < PER; ++r) {
    const uint32_t e = r * NT + threadIdx.x;
    if (e < s) {
      const uint64_t kv = sm.keyA[a + e];
      const uint32_t d = (uint32_t)(kv - mn), wd = d >> 5;
      const uint32_t at = below[wd] + __popc(bits[wd] & ((1u << (d & 31)) - 1u));
      sm.keyB[a + min(at, s - 1)] = kv;
    }
  }
  __syncthreads();
  for (uint32_t e = threadIdx.x; e < s; e += NT) sm.keyA[a + e] = sm.keyB[a + e];
  __syncthreads();
}

// One counting pass over positions [a, a+s) of keyA / idxA, in place: every
// element takes a slot in its bin, (key - mn) >> shift, by a shared-memory
// atomic (the order inside a bin is arbitrary), lands in keyB / idxB at its
// bin's start plus that slot, and then -- in a small bin -- takes its final
// place by counting the bin's members with a smaller (key, input index):
// that comparison, not the pass, makes the result stable.  Bins above
// kInsertMax go back unchanged and are queued for another pass.  With
// by_idx the bins are the input indices themselves (a bin of equal keys is
// put back in input order; indices are distinct and below kLocalMax).
// PACKED: the keys are ((key - min) << kLocalBits) | input index, distinct
// and ordered as (key, index); the index arrays are not used.
template <int NT, bool PACKED, typename SM>
__device__ __noinline__ void local_msd_pass(SM& sm, uint32_t a, uint32_t s, uint64_t mn, uint64_t mx, bool by_idx) {
  constexpr int kBins = 1 << kLocalBits;
  constexpr int PER = kLocalMax / NT;
  static_assert(kLocalMax <= kBins, "input indices must fit the bins");
  if constexpr (PACKED) {
    if (mx - mn < (uint64_t)kBins) {  // (block-wide bounds: every thread takes this branch)
      local_bitmap_place<NT>(sm, a, s, mn);
      return;
    }
  }
  const int bits = bitlen64(mx - mn);
  const int shift = bits > kLocalBits ? bits - kLocalBits : 0;
  for (int i = threadIdx.x; i < kBins; i += NT) sm.cnt[i] = 0;
  __syncthreads();
  uint32_t bin[PER], slot[PER];
#pragma unroll
  for (int r = 0; r < PER; ++r) {
    const uint32_t e = r * NT + threadIdx.x;
    if (e < s) {
      if constexpr (PACKED) bin[r] = (uint32_t)((sm.keyA[a + e] - mn) >> shift);
      else bin[r] = by_idx ? (uint32_t)sm.idxA[a + e] : (uint32_t)((sm.keyA[a + e] - mn) >> shift);
      slot[r] = atomicAdd(&sm.cnt[bin[r]], 1u);
    }
  }
  __syncthreads();
  {  // exclusive scan of the bin counts
    constexpr int BPT = kBins / NT;
    uint32_t loc[BPT], sum = 0;
#pragma unroll
    for (int i = 0; i < BPT; ++i) {
      loc[i] = sm.cnt[threadIdx.x * BPT + i];
      sum += loc[i];
    }
    uint32_t pre = block_exclusive_scan<uint32_t, NT>(sum, sm.scan_tmp, nullptr);
#pragma unroll
    for (int i = 0; i < BPT; ++i) {
      sm.cnt[threadIdx.x * BPT + i] = pre;
      pre += loc[i];
    }
    if (threadIdx.x == NT - 1) sm.cnt[kBins] = pre;
  }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < PER; ++r) {
    const uint32_t e = r * NT + threadIdx.x;
    if (e < s) {
      const uint32_t pos = sm.cnt[bin[r]] + slot[r];
      sm.keyB[a + pos] = sm.keyA[a + e];
      if constexpr (!PACKED) sm.idxB[a + pos] = sm.idxA[a + e];
    }
  }
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < s; i += NT) {
    const uint64_t kv = sm.keyB[a + i];
    uint16_t iv = 0;
    if constexpr (!PACKED) iv = sm.idxB[a + i];
    const uint32_t d = !PACKED && by_idx ? (uint32_t)iv : (uint32_t)((kv - mn) >> shift);
    const uint32_t b0 = sm.cnt[d], b1 = sm.cnt[d + 1];
    const uint32_t sz = b1 - b0;
    uint32_t at = i;
    if (sz <= (uint32_t)kInsertMax) {
      uint32_t r = 0;
      for (uint32_t j = b0; j < b1; ++j) {
        const uint64_t kj = sm.keyB[a + j];
        if constexpr (PACKED) r += kj < kv;
        else r += (kj < kv) || (kj == kv && sm.idxB[a + j] < iv);
      }
      at = b0 + r;
    } else if (i == b0) {
      uint32_t q = atomicAdd(&sm.nbig, 1u);
      sm.big[q] = (uint16_t)(a + b0);
      sm.bigsz[q] = (uint16_t)sz;
    }
    sm.keyA[a + at] = kv;
    if constexpr (!PACKED) sm.idxA[a + at] = iv;
  }
  __syncthreads();
}

// Further passes over the bins too large to place by counting.
template <int NT, bool PACKED, typename SM>
__device__ void local_big_bins(SM& sm, uint32_t* stats) {
  for (;;) {
    uint32_t nb = sm.nbig;
    __syncthreads();
    if (nb == 0) break;
    uint32_t a = sm.big[nb - 1], s = sm.bigsz[nb - 1];
    __syncthreads();
    if (threadIdx.x == 0) sm.nbig = nb - 1;
    uint64_t bmn = ~0ull, bmx = 0;
    for (uint32_t e = threadIdx.x; e < s; e += NT) {
      uint64_t kv = sm.keyA[a + e];
      bmn = kv < bmn ? kv : bmn;
      bmx = kv > bmx ? kv : bmx;
    }
    block_minmax<NT>(bmn, bmx, sm.red);
    if (threadIdx.x == 0) atomicAdd(stats + STAT_BIGBIN, 1u);
    // equal keys: back into input order (their bin filled in any order);
    // packed keys are never equal
    local_msd_pass<NT, PACKED>(sm, a, s, bmn, bmx, !PACKED && bmn == bmx);
  }
}

// Stable sort of `m` <= kLocalMax records of src by key into dst (distinct).
template <int EW, int NT>
__device__ void local_sort(LocalSmemT<NT>& sm, const uint8_t* src, uint8_t* dst, uint32_t m,
                           const gbsort_key_word& kw, uint32_t* stats) {
  constexpr int kLocalRpt = kLocalMax / NT;
  constexpr uint32_t E = EW * 4;
  const uint32_t w = warp_id(), lane = lane_id();
  uint64_t mn = ~0ull, mx = 0;
  uint64_t k[kLocalRpt];
#pragma unroll
  for (int r = 0; r < kLocalRpt; ++r) {
    uint32_t e = w * 32 * kLocalRpt + r * 32 + lane;
    k[r] = e < m ? key_at(src, e, E, kw) : 0;
    if (e < m) {
      mn = k[r] < mn ? k[r] : mn;
      mx = k[r] > mx ? k[r] : mx;
    }
  }
  if (threadIdx.x == 0) sm.nbig = 0;
  block_minmax<NT>(mn, mx, sm.red);
  if (mn == mx) {  // one key: the input order is the stable order
    block_copy_ilp<EW>(src, dst, m, NT);
    __syncthreads();
    return;
  }
  // a key range of at most 64 - kLocalBits bits leaves room for the input
  // index below the key: one distinct 64-bit word per record
  const bool packed = bitlen64(mx - mn) <= 64 - kLocalBits;
#pragma unroll
  for (int r = 0; r < kLocalRpt; ++r) {
    uint32_t e = w * 32 * kLocalRpt + r * 32 + lane;
    if (e < m) {
      sm.keyA[e] = packed ? ((k[r] - mn) << kLocalBits) | e : k[r];
      if (!packed) sm.idxA[e] = (uint16_t)e;
    }
  }
  __syncthreads();
  using V = typename std::conditional<EW % 4 == 0, uint4,
                                      typename std::conditional<EW % 2 == 0, uint2, uint32_t>::type>::type;
  constexpr int VPR = E / sizeof(V);
  // the input index of each sorted record is the low bits of its key word;
  // records of several vectors read it once into idxA
  const bool idx_in_key = packed && VPR == 1;
  if (packed) {
    local_msd_pass<NT, true>(sm, 0, m, 0, ((mx - mn) << kLocalBits) | (kLocalMax - 1), false);
    local_big_bins<NT, true>(sm, stats);
    if (!idx_in_key) {
      for (uint32_t i = threadIdx.x; i < m; i += NT) sm.idxA[i] = (uint16_t)(sm.keyA[i] & (kLocalMax - 1));
      __syncthreads();
    }
  } else {
    local_msd_pass<NT, false>(sm, 0, m, mn, mx, false);
    local_big_bins<NT, false>(sm, stats);
  }
  // gather the records into dst in sorted order, four loads in flight
  {
    constexpr int U = sizeof(V) >= 16 ? 2 : 4;
    const uint32_t nv = m * VPR;
    for (uint32_t f0 = threadIdx.x; f0 < nv; f0 += NT * U) {
      V v[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        uint32_t f = f0 + u * NT;
        if (f < nv) {
          const uint32_t i = f / VPR;
          const uint32_t from = idx_in_key ? (uint32_t)(sm.keyA[i] & (kLocalMax - 1)) : sm.idxA[i];
          v[u] = reinterpret_cast<const V*>(src + (size_t)from * E)[f % VPR];
        }
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        uint32_t f = f0 + u * NT;
        if (f < nv) reinterpret_cast<V*>(dst + (size_t)(f / VPR) * E)[f % VPR] = v[u];
      }
    }
  }
  __syncthreads();
}

// ------------------------------------------------ staged local sorts ----
// Records of up to 16 bytes: a task's records come into shared memory with
// one bulk asynchronous copy, issued while the previous task sorts (two
// buffers), so no thread waits on DRAM; keys are read there, sorted as
// packed words ((key - min) << 11 | input index, distinct and ordered as
// (key, index)), and the records leave in sorted order by coalesced stores.
// Without index arrays the shared memory of two CTAs per SM holds both
// buffers: a task whose key range is wider than the 53 bits a packed word
// keeps is packed by its top 53 bits and runs of equal prefixes are sorted
// again by their full keys (local_refine_runs).
template <int NT>
struct LocalSmemP {
  static constexpr int kNW = NT / 32;
  static constexpr int kLongRuns = kLocalMax / (kInsertMax + 1) + 2;
  uint64_t keyA[kLocalMax];  // packed keys (sorted order at the end)
  uint64_t keyB[kLocalMax];
  uint32_t cnt[(1 << kLocalBits) + 1];
  uint16_t big[kLongRuns];  // pending bins of the MSD passes
  uint16_t bigsz[kLongRuns];
  uint16_t run[kLongRuns];  // long runs of equal prefixes (wide key ranges)
  uint16_t runsz[kLongRuns];
  uint32_t nbig, nrun;
  uint64_t red[2 * kNW];
  uint32_t scan_tmp[kNW];
  uint32_t task_id[2], pend_staged;
  SortTask task[2];  // the current task and the next one, alternating
  uint64_t bar[2];   // completion of the two record buffers' copies
};
// One record buffer: kLocalMax records plus the 16-byte rounding of a start.
template <int EW>
__host__ __device__ constexpr uint32_t staged_buf_bytes() {
  return (uint32_t)((kLocalMax * EW * 4 + 32 + 127) & ~127);
}
template <int EW, int NT>
constexpr size_t staged_smem_bytes() {
  return 2 * (size_t)staged_buf_bytes<EW>() + sizeof(LocalSmemP<NT>);
}

// Runs of equal packed prefixes (keys that differ only in the bits dropped
// from a wide range) put back in (full key, index) order: short runs by one
// thread's insertion sort, long ones re-packed relative to their own least
// key (they differ only in the dropped bits, at most kLocalBits of them)
// and sorted by the MSD pass.
template <int EW, int NT>
__device__ __noinline__ void local_refine_runs(LocalSmemP<NT>& sm, const uint8_t* rb, uint32_t m,
                                               const gbsort_key_word& kw, uint32_t* stats) {
  constexpr uint32_t E = EW * 4;
  constexpr uint64_t kIdx = kLocalMax - 1;
  bool any = false;
  for (uint32_t i = threadIdx.x; i + 1 < m; i += NT) any |= (sm.keyA[i] >> kLocalBits) == (sm.keyA[i + 1] >> kLocalBits);
  if (!__syncthreads_or(any)) return;
  if (threadIdx.x == 0) sm.nrun = 0;
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < m; i += NT) {
    // the prefix is the same for every member of a run, whatever order
    // another thread's insertion sort has them in
    const uint64_t pre = sm.keyA[i] >> kLocalBits;
    if (i > 0 && (sm.keyA[i - 1] >> kLocalBits) == pre) continue;
    uint32_t len = 1;
    while (i + len < m && (sm.keyA[i + len] >> kLocalBits) == pre) ++len;
    if (len == 1) continue;
    if (len <= (uint32_t)kInsertMax) {
      for (uint32_t a = i + 1; a < i + len; ++a) {
        const uint64_t v = sm.keyA[a];
        const uint32_t vi = (uint32_t)(v & kIdx);
        const uint64_t vk = load_key_aligned4(rb + (size_t)vi * E, kw);
        uint32_t b = a;
        while (b > i) {
          const uint64_t u = sm.keyA[b - 1];
          const uint32_t ui = (uint32_t)(u & kIdx);
          const uint64_t uk = load_key_aligned4(rb + (size_t)ui * E, kw);
          if (uk < vk || (uk == vk && ui < vi)) break;
          sm.keyA[b] = u;
          --b;
        }
        sm.keyA[b] = v;
      }
    } else {
      const uint32_t q = atomicAdd(&sm.nrun, 1u);
      sm.run[q] = (uint16_t)i;
      sm.runsz[q] = (uint16_t)len;
    }
  }
  __syncthreads();
  for (;;) {
    const uint32_t nr = sm.nrun;
    __syncthreads();
    if (nr == 0) break;
    const uint32_t a = sm.run[nr - 1], s = sm.runsz[nr - 1];
    __syncthreads();
    if (threadIdx.x == 0) sm.nrun = nr - 1;
    uint64_t rmn = ~0ull, rmx = 0;
    for (uint32_t e = threadIdx.x; e < s; e += NT) {
      const uint64_t kk = load_key_aligned4(rb + (size_t)(sm.keyA[a + e] & kIdx) * E, kw);
      rmn = kk < rmn ? kk : rmn;
      rmx = kk > rmx ? kk : rmx;
    }
    block_minmax<NT>(rmn, rmx, sm.red);
    for (uint32_t e = threadIdx.x; e < s; e += NT) {
      const uint64_t v = sm.keyA[a + e];
      const uint64_t kk = load_key_aligned4(rb + (size_t)(v & kIdx) * E, kw);
      sm.keyA[a + e] = ((kk - rmn) << kLocalBits) | (v & kIdx);
    }
    __syncthreads();
    if (threadIdx.x == 0) atomicAdd(stats + STAT_BIGBIN, 1u);
    local_msd_pass<NT, true>(sm, a, s, 0, ((rmx - rmn) << kLocalBits) | kIdx, false);
    local_big_bins<NT, true>(sm, stats);
  }
}

// In-place exclusive scan of the 2^kLocalBits bin counts of a staged local
// sort (cnt[kBins] receives the total), one barrier inside; the caller
// synchronises before reading the result.
template <int NT>
__device__ __forceinline__ void scan_local_bins(uint32_t* cnt, uint32_t* wtot) {
  constexpr int kBins = 1 << kLocalBits;
  constexpr int BPT = kBins / NT;
  const uint32_t lane = lane_id(), w = warp_id();
  uint32_t loc[BPT], sum = 0;
#pragma unroll
  for (int i = 0; i < BPT; ++i) {
    loc[i] = cnt[threadIdx.x * BPT + i];
    sum += loc[i];
  }
  uint32_t x = sum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(GB_FULL_MASK, x, o);
    if (lane >= (uint32_t)o) x += y;
  }
  if (lane == 31) wtot[w] = x;
  __syncthreads();
  uint32_t pre = x - sum;
  for (uint32_t q = 0; q < w; ++q) pre += wtot[q];
#pragma unroll
  for (int i = 0; i < BPT; ++i) {
    cnt[threadIdx.x * BPT + i] = pre;
    pre += loc[i];
  }
  if (threadIdx.x == NT - 1) cnt[kBins] = pre;
}

// Stable sort of m <= kLocalMax records held in shared memory at rb into
// dst (global memory).  The keys lie in [lo, hi], the task's range, which
// fixes the packing without a reduction: a key's packed word is
// ((key - lo) >> drop) << kLocalBits | its input index, and its bin the
// word's top kLocalBits bits.  One pass places every word in its bin (a
// slot by a shared-memory atomic), each word of a bin of up to kInsertMax
// counts the smaller words of its bin -- distinct words, so this is the
// stable (key, index) order -- and its record goes straight to that output
// position; larger bins take further MSD passes, and a range wider than a
// packed word (drop > 0) is finished by local_refine_runs before any record
// leaves.  cnt is zero on entry and on return.
template <int EW, int NT>
__device__ void local_sort_staged(LocalSmemP<NT>& sm, const uint8_t* rb, uint8_t* dst, uint32_t m, uint64_t lo,
                                  uint64_t hi, const gbsort_key_word& kw, uint32_t* stats, uint32_t* err) {
  constexpr int PER = kLocalMax / NT;
  constexpr int kBins = 1 << kLocalBits;
  constexpr uint32_t E = EW * 4;
  constexpr uint64_t kIdx = kLocalMax - 1;
  using V = typename std::conditional<EW % 4 == 0, uint4,
                                      typename std::conditional<EW % 2 == 0, uint2, uint32_t>::type>::type;
  constexpr uint32_t VPR = E / sizeof(V);
  auto put = [&](uint32_t at, uint32_t from) {  // record `from` of rb to output position `at`
#pragma unroll
    for (uint32_t q = 0; q < VPR; ++q)
      st_global(reinterpret_cast<V*>(dst + (size_t)at * E) + q, reinterpret_cast<const V*>(rb + (size_t)from * E)[q]);
  };
  const uint64_t range = hi - lo;
  const int rbits = bitlen64(range);
  const int drop = rbits > 64 - kLocalBits ? rbits - (64 - kLocalBits) : 0;
  const int pbits = bitlen64(((range >> drop) << kLocalBits) | kIdx);
  const int shift = pbits > kLocalBits ? pbits - kLocalBits : 0;
  uint64_t pk[PER];
  uint32_t bin[PER], slot[PER];
  bool bad = false;
#pragma unroll
  for (int r = 0; r < PER; ++r) {
    const uint32_t e = r * NT + threadIdx.x;
    if (e < m) {
      const uint64_t k = load_key_aligned4(rb + (size_t)e * E, kw);
      bad |= k < lo || k > hi;
      const uint64_t off = k < lo ? 0 : (k > hi ? range : k - lo);
      pk[r] = ((off >> drop) << kLocalBits) | e;
      bin[r] = (uint32_t)(pk[r] >> shift);
      slot[r] = atomicAdd(&sm.cnt[bin[r]], 1u);
    }
  }
  if (bad) set_error(err, DEV_ERR_COUNT_MISMATCH);  // a key outside its task's range (never expected)
  if (threadIdx.x == 0) sm.nbig = 0;
  __syncthreads();
  scan_local_bins<NT>(sm.cnt, sm.scan_tmp);
  __syncthreads();
#pragma unroll
  for (int r = 0; r < PER; ++r) {
    const uint32_t e = r * NT + threadIdx.x;
    if (e < m) sm.keyB[sm.cnt[bin[r]] + slot[r]] = pk[r];
  }
  __syncthreads();
  // each thread's PER positions in bin order, their loads batched so that
  // the chains keyB -> bin bounds -> record of the PER positions overlap
  uint64_t vv[PER];
  uint32_t lo_[PER], hi_[PER];
#pragma unroll
  for (int r = 0; r < PER; ++r) {
    const uint32_t i = r * NT + threadIdx.x;
    vv[r] = i < m ? sm.keyB[i] : 0;
  }
#pragma unroll
  for (int r = 0; r < PER; ++r) {
    const uint32_t d = (uint32_t)(vv[r] >> shift);
    lo_[r] = sm.cnt[d];
    hi_[r] = sm.cnt[d + 1];
  }
#pragma unroll
  for (int r = 0; r < PER; ++r) {
    const uint32_t i = r * NT + threadIdx.x;
    if (i >= m) continue;
    const uint64_t v = vv[r];
    const uint32_t b0 = lo_[r], b1 = hi_[r];
    if (b1 - b0 > (uint32_t)kInsertMax) {  // a crowded bin: further passes below
      if (i == b0) {
        const uint32_t q = atomicAdd(&sm.nbig, 1u);
        sm.big[q] = (uint16_t)b0;
        sm.bigsz[q] = (uint16_t)(b1 - b0);
      }
      sm.keyA[i] = v;
      continue;
    }
    uint32_t at = i;
    if (b1 - b0 > 1) {
      uint32_t rk = 0;
      for (uint32_t j = b0; j < b1; ++j) rk += sm.keyB[j] < v;
      at = b0 + rk;
    }
    if (drop) sm.keyA[at] = v;
    else put(at, (uint32_t)(v & kIdx));
  }
  __syncthreads();
  const uint32_t nb = sm.nbig;
  if (nb) {  // crowded bins (clustered keys): MSD passes over their packed words in keyA
    if (!drop)
      for (uint32_t q = threadIdx.x; q < nb; q += NT) {
        sm.run[q] = sm.big[q];
        sm.runsz[q] = sm.bigsz[q];
      }
    __syncthreads();
    local_big_bins<NT, true>(sm, stats);
    if (!drop) {  // their records, now in order
      for (uint32_t q = 0; q < nb; ++q) {
        const uint32_t a = sm.run[q], s = sm.runsz[q];
        for (uint32_t i = threadIdx.x; i < s; i += NT) put(a + i, (uint32_t)(sm.keyA[a + i] & kIdx));
      }
    }
  }
  if (drop) {  // a range wider than a packed word: equal prefixes sorted by full keys, then every record
    local_refine_runs<EW, NT>(sm, rb, m, kw, stats);
    for (uint32_t f = threadIdx.x; f < m * VPR; f += NT) {
      const uint32_t i = f / VPR;
      const uint32_t from = (uint32_t)(sm.keyA[i] & kIdx);
      reinterpret_cast<V*>(dst)[f] = reinterpret_cast<const V*>(rb + (size_t)from * E)[f % VPR];
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i <= kBins; i += NT) sm.cnt[i] = 0;  // zero for the next task
}

// Fine bins of a split with refined (crowded) bins: cm[b] = first fine bin
// of bin b << 4 | r, bin b being cut into 2^r sub-bins of its key range.
__device__ __forceinline__ uint32_t fine_bin(const uint32_t* cm, uint64_t key, uint64_t blo, int shift,
                                             uint32_t nbins) {
  const uint64_t x = key > blo ? key - blo : 0;
  const uint32_t b = (uint32_t)min(x >> shift, (uint64_t)(nbins - 1));
  const uint32_t c = cm[b], r = c & 15u;
  const uint32_t sub = r ? (uint32_t)(x >> (shift - (int)r)) & ((1u << r) - 1u) : 0u;
  return (c >> 4) + sub;
}
// Least key of fine bin f (f below the number of fine bins).
__device__ __forceinline__ uint64_t fine_bin_lo(const uint32_t* cm, uint32_t f, uint64_t blo, int shift,
                                                uint32_t nbins) {
  uint32_t lo = 0, hi = nbins;  // the last bin whose first fine bin is <= f
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if ((cm[mid] >> 4) <= f) lo = mid;
    else hi = mid;
  }
  const uint32_t r = cm[lo] & 15u, sub = f - (cm[lo] >> 4);
  return blo + ((uint64_t)lo << shift) + ((uint64_t)sub << (shift - (int)r));
}
// In-place exclusive scan of PER * kThreads bin counts (PER per thread).
template <int PER>
__device__ __forceinline__ void scan_bins(uint32_t* a, uint32_t* scan_tmp) {
  uint32_t loc[PER], s = 0;
#pragma unroll
  for (int i = 0; i < PER; ++i) {
    loc[i] = a[threadIdx.x * PER + i];
    s += loc[i];
  }
  uint32_t pre = block_exclusive_scan<uint32_t>(s, scan_tmp, nullptr);
#pragma unroll
  for (int i = 0; i < PER; ++i) {
    a[threadIdx.x * PER + i] = pre;
    pre += loc[i];
  }
  __syncthreads();
}

// Split of one large bucket: 4096 bins of its key range, grouped into at most
// 256 runs of consecutive bins, a stable scatter src -> other by group, and
// one task per group (local sort, copy, or another split).
// ---- the persistent engine's queue (the engine itself is further down) ----
struct EngineQueue {
  SortTask* task;     // [cap]
  uint32_t* ready;    // [cap], zero before the launch
  uint32_t* tail;     // tasks pushed
  uint32_t* head;     // tasks claimed
  uint32_t* pending;  // tasks pushed and not finished
  uint32_t cap;       // (the three counters sit in separate cache lines)
};

__device__ __forceinline__ uint32_t ld_acquire_u32(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_u32(uint32_t* p, uint32_t v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

struct EngineSink {  // the persistent engine's queue: a split publishes its groups by engine_emit
  const EngineQueue& q;
};

constexpr uint32_t kEngineWaitPolls = 1u << 24;

// A split publishes all its groups with one reservation: a block scan of
// every thread's task count, one atomic each on pending and tail, then the
// tasks and their ready flags (instead of two atomics and a fence per task).
// Every thread calls it with its own tasks: n of them, the i-th from make(i).
template <typename Make>
__device__ __forceinline__ void engine_emit(const EngineQueue& q, uint32_t n, Make&& make, uint32_t* base_slot,
                                            uint32_t* scan_tmp, uint32_t* err) {
  uint32_t total;
  const uint32_t off = block_exclusive_scan<uint32_t>(n, scan_tmp, &total);
  if (total == 0) return;
  if (threadIdx.x == 0) {
    atomicAdd(q.pending, total);  // before any flag: pending never undercounts
    const uint32_t base = atomicAdd(q.tail, total);
    *base_slot = base;
    if (base + total > q.cap || base + total < base) {
      set_error(err, DEV_ERR_TASK_OVERFLOW);
      atomicSub(q.pending, base >= q.cap ? total : base + total - q.cap);
    }
  }
  __syncthreads();
  const uint32_t base = *base_slot;
  for (uint32_t i = 0; i < n; ++i)
    if (base + off + i < q.cap) q.task[base + off + i] = make(i);
  __threadfence();
  for (uint32_t i = 0; i < n; ++i)
    if (base + off + i < q.cap) st_release_u32(&q.ready[base + off + i], 1u);
  __syncthreads();
}

enum EngineState : uint32_t { ENGINE_HAVE = 0, ENGINE_DONE = 1 };

// Where the tasks of a split go: the next round's lists (RoundSink) or the
// persistent engine's queue (EngineSink, below).
struct RoundSink {
  const TaskLists& L;
  __device__ void copy(uint32_t start, uint32_t from, uint32_t cnt, uint64_t lo, uint64_t hi, uint32_t flags,
                       uint32_t* err) const {
    push_copy(L, start, from, cnt, lo, hi, flags, err);
  }
  __device__ void local(const SortTask& t, uint32_t* err) const { push(L.local, L.nlocal, L.cap_local, t, err); }
  __device__ void split(const SortTask& t, uint32_t* err) const {
    push(L.split_out, L.nsplit_out, L.cap_split, t, err);
  }
};

// A bucket's records streamed through the split's two staging buffers:
// thread 0 keeps the next two tiles in flight (bulk asynchronous copies of
// the tiles' 16-byte aligned byte ranges; the rounding reads at most 15
// bytes on either side, inside the scratch allocation), every thread waits
// for each tile in turn.  par holds each buffer's next completion parity,
// the same in every thread (every thread waits for every tile).
template <int EW>
struct SplitTiles {
  static constexpr uint32_t E = EW * 4;
  static constexpr uint32_t T = staged_split_tile<EW>();
  static_assert(T * E + 32 <= (uint32_t)kSplitBufBytes, "a staged tile fits its buffer");
  const uint8_t* src;
  uint32_t m;
  SplitSmemStaged& sm;
  uint32_t& par;

  __device__ __forceinline__ void issue(uint32_t i) const {  // thread 0: tile i into buffer i & 1
    const uint32_t t0 = i * T;
    const uint32_t cnt = min(T, m - t0);
    const uintptr_t a = (uintptr_t)(src + (size_t)t0 * E);
    const uintptr_t a0 = a & ~(uintptr_t)15;
    const uint32_t bytes = (uint32_t)(((a - a0) + (uintptr_t)cnt * E + 15) & ~(uintptr_t)15);
    bulk_load(sm.stage + (size_t)(i & 1) * kSplitBufBytes, (const void*)a0, bytes, &sm.bar[i & 1]);
  }
  // After a barrier that ends every thread's use of both buffers.
  __device__ __forceinline__ void start() const {
    if (threadIdx.x == 0) {
      fence_proxy_async_smem();
      issue(0);
      if (T < m) issue(1);
    }
  }
  // Waits for tile i (with a barrier); its first record, or nullptr if the
  // wait ran out -- then DEV_ERR_TIMEOUT is set and the CTA's copies still
  // in flight have been waited for, and the caller must leave.
  __device__ __forceinline__ const uint8_t* wait(uint32_t i, uint32_t* err) const {
    const uint32_t b = i & 1;
    const bool ok = __syncthreads_and(mbar_wait_bounded(&sm.bar[b], (par >> b) & 1u, kBulkWaitPolls));
    if (!ok) {
      if (threadIdx.x == 0) set_error(err, DEV_ERR_TIMEOUT);
      mbar_wait_bounded(&sm.bar[b], (par >> b) & 1u, kBulkWaitPolls);
      if ((i + 1) * T < m) mbar_wait_bounded(&sm.bar[b ^ 1], (par >> (b ^ 1)) & 1u, kBulkWaitPolls);
      return nullptr;
    }
    par ^= 1u << b;
    return sm.stage + (size_t)b * kSplitBufBytes + ((uintptr_t)src & 15);
  }
  // After a barrier that ends every thread's use of tile i: its buffer takes tile i + 2.
  __device__ __forceinline__ void release(uint32_t i) const {
    if (threadIdx.x == 0 && (i + 2) * T < m) {
      fence_proxy_async_smem();
      issue(i + 2);
    }
  }
};

// Uniform split of a level-1 bucket (records of 8-16 bytes, split rounds
// with areas).  Its key range [lo, hi] is cut into G = ceil(m / kUniformTarget)
// groups of equal width -- group g holds the keys whose offset x = key - lo
// has floor(x G / S) = g, S = hi - lo + 1 -- and each group is scattered
// into its own region of the bucket's area of scratch B (cap = area / G
// records, a quarter above the mean), with no histogram pass: the regions
// need no exact counts.  Keys this suits (the model's widest window and the
// heavy-key count both zero: the sample saw a smooth distribution, and few
// earlier attempts in this sort overflowed) fill the groups like a binomial
// draw, so a region about five standard deviations above its mean size does
// not fill; if one does, the attempt is void.  Returns 1 when the groups are
// emitted, 0 to run the exact split instead (not attempted, or a region
// overflowed), -1 if a staged wait ran out (the CTA must leave).
// Mean records of a uniform group (local sorts hold 2048).  1e9 x 16 B,
// uniform keys: 1600 / 1800 / 1950 give 43.6 / 42.8 / 43.1 ms (1950 sends
// 5414 groups past 2048 records round the split again).
constexpr uint32_t kUniformTarget = 1800;

template <int EW, typename SM, typename Sink>
__device__ int split_uniform(SM& sm, const HsortParams& p, const SortTask& task, const uint8_t* src, uint8_t* oth,
                             uint32_t dpos, const Sink& L, uint32_t* stats, uint32_t* err, uint32_t& par) {
  constexpr uint32_t E = EW * 4;
  constexpr int SRPT = staged_split_tile<EW>() / kThreads;
  const uint32_t m = task.count;
  const uint32_t G = (m + kUniformTarget - 1) / kUniformTarget;
  const uint32_t cap = (split_area(task.start + m) - split_area(task.start)) / max(G, 1u);
  const uint32_t w = warp_id(), lane = lane_id();
  uint64_t* glo = reinterpret_cast<uint64_t*>(sm.hist);  // G + 1 key offsets from lo, group starts
  if (threadIdx.x == 0) {
    bool go = p.uniform != nullptr && G >= 2 && G <= (uint32_t)kMaxGroups && task.hi - task.lo >= 16ull * G;
    if (go) {
      const uint32_t mean = (m + G - 1) / G;
      // (without these gates, Zipf keys void 298 attempts before the failure
      // count stops them: split 11.8 -> 13.1 ms)
      go = *p.gate_widest == 0 && *p.gate_heavy == 0 && cap >= mean + 5 * (uint32_t)sqrtf((float)mean) + 16;
    }
    if (go) {
      const uint32_t tried = *(volatile uint32_t*)&p.uniform[0], failed = *(volatile uint32_t*)&p.uniform[1];
      go = 8ull * failed <= (uint64_t)tried + 8;
    }
    if (go) {
      atomicAdd(&p.uniform[0], 1u);
      const unsigned __int128 S = (unsigned __int128)(task.hi - task.lo) + 1;
      sm.red[0] = (uint64_t)((((unsigned __int128)G) << 64) / S);  // M: floor(x M / 2^64) is g or g - 1
    }
    sm.uflag = go ? 1u : 0u;
  }
  __syncthreads();
  if (!sm.uflag) return 0;
  const uint64_t M = sm.red[0];
  for (uint32_t g = threadIdx.x; g <= G; g += kThreads) {
    const unsigned __int128 S = (unsigned __int128)(task.hi - task.lo) + 1;
    const unsigned __int128 v = ((unsigned __int128)g * S + (G - 1)) / G;  // ceil(g S / G)
    glo[g] = (v >> 64) ? ~0ull : (uint64_t)v;
  }
  const uint32_t g_me = threadIdx.x;
  if (g_me < G) sm.cursor[g_me] = g_me * cap;
  __syncthreads();
  auto group_of = [&](uint64_t key) -> uint32_t {
    const uint64_t x = key > task.lo ? key - task.lo : 0;
    const unsigned long long q = __umul64hi(x, M);
    uint32_t g = q < G ? (uint32_t)q : G - 1;
    if (g + 1 < G && x >= glo[g + 1]) ++g;
    return g;
  };
  using V = typename std::conditional<E % 16 == 0, uint4,
                                      typename std::conditional<E % 8 == 0, uint2, uint32_t>::type>::type;
  constexpr uint32_t VPR = E / sizeof(V);
  const SplitTiles<EW> tiles{src, m, sm, par};
  tiles.start();
  for (uint32_t i = 0; i * tiles.T < m; ++i) {
    const uint32_t nvalid = min(tiles.T, m - i * tiles.T);
    const uint8_t* rb = tiles.wait(i, err);  // (a barrier: the last tile's rows are clear)
    if (!rb) return -1;
    uint32_t grp[SRPT], rank[SRPT], lead[SRPT];
#pragma unroll
    for (int r = 0; r < SRPT; ++r) {
      const uint32_t e = w * 32 * SRPT + r * 32 + lane;
      grp[r] = e < nvalid ? group_of(load_key_aligned4(rb + (size_t)e * E, p.key)) : kNoBucket;
    }
    warp_ranks<SRPT, kGroupBits>(grp, rank, lead, sm.gcnt);
    __syncthreads();
    uint32_t gtot;
    tile_rank(g_me, 0, sm.gcnt, gtot);
    const uint32_t goff = block_exclusive_scan<uint32_t>(gtot, sm.scan_tmp, nullptr);
    sm.goff[g_me] = goff;
    __syncthreads();
#pragma unroll
    for (int r = 0; r < SRPT; ++r) {
      if (grp[r] == kNoBucket) continue;
      uint32_t all;
      const uint32_t slot = sm.goff[grp[r]] + tile_rank(grp[r], rank[r], sm.gcnt, all);
      if (slot >= nvalid) {  // impossible with consistent ranks
        set_error(err, DEV_ERR_COUNT_MISMATCH);
        continue;
      }
      sm.perm[slot] = (uint16_t)(w * 32 * SRPT + r * 32 + lane);
      sm.sgrp[slot] = (uint16_t)grp[r];
    }
    __syncthreads();
    bool over = false;
#pragma unroll (split_outs_unroll<EW>())
    for (uint32_t k = 0; k < (SplitTiles<EW>::T * VPR + kThreads - 1) / kThreads; ++k) {
      const uint32_t f = threadIdx.x + k * kThreads;
      if (f >= nvalid * VPR) break;
      const uint32_t j = f / VPR, qw = f % VPR;
      const uint32_t g = sm.sgrp[j] & (kMaxGroups - 1);
      const uint32_t from = min((uint32_t)sm.perm[j], nvalid - 1);
      const uint32_t dest = sm.cursor[g] + (j - sm.goff[g]);
      if (g < G && dest < (g + 1) * cap)
        st_global(reinterpret_cast<V*>(oth + (size_t)dest * E) + qw, reinterpret_cast<const V*>(rb + (size_t)from * E)[qw]);
      else over = true;
    }
    if (over) sm.uflag = 2;  // a group outgrew its region: the attempt is void
    __syncthreads();
    tiles.release(i);
    if (g_me < G) sm.cursor[g_me] += gtot;
    clear_rows<SRPT>(grp, lead, sm.gcnt);
  }
  __syncthreads();
  if (sm.uflag != 1) {
    if (threadIdx.x == 0) atomicAdd(&p.uniform[1], 1u);
    __syncthreads();
    return 0;
  }
  // each group's records: a task from its region to its place in the output
  const uint32_t cnt = g_me < G ? sm.cursor[g_me] - g_me * cap : 0;
  uint32_t total;
  const uint32_t off = block_exclusive_scan<uint32_t>(cnt, sm.scan_tmp, &total);
  if (threadIdx.x == 0 && total != m) set_error(err, DEV_ERR_COUNT_MISMATCH);
  if (cnt) {
    const uint64_t klo = task.lo + glo[g_me];
    const uint64_t khi = g_me + 1 < G ? task.lo + glo[g_me + 1] - 1 : task.hi;
    const uint32_t from = dpos + g_me * cap, start = task.start + off;
    if (klo == khi || cnt == 1) {
      L.copy(start, from, cnt, klo, khi, TASK_SRC_B, err);
    } else if (cnt <= (uint32_t)kLocalMax) {
      L.local(make_task_at(start, from, cnt, klo, khi, TASK_SRC_B), err);
    } else {
      atomicAdd(stats + STAT_PUSHED, 1u);
      L.split(make_task_at(start, from, cnt, klo, khi, TASK_SRC_B), err);
    }
  }
  __syncthreads();
  return 1;
}

// One bucket split.  STAGED: the histogram and scatter passes stream the
// bucket through shared memory (SplitTiles) instead of loading records
// into registers; false if a staged wait ran out (the CTA must leave).
template <int EW, bool STAGED, typename Sink, typename SM>
__device__ bool split_task(SM& sm, const HsortParams& p, const SortTask& task, const Sink& L,
                           uint32_t* stats, uint32_t* err, uint32_t& par) {
  constexpr uint32_t E = EW * 4;
  constexpr int RPT = Tile<EW>::kRpt, T = Tile<EW>::kSize;
  const bool in_b = (task.flags & TASK_SRC_B) != 0, in_out = (task.flags & TASK_SRC_OUT) != 0;
  const uint8_t* src = (in_b ? p.bufB : in_out ? p.out : p.bufA) + (size_t)task.from * E;
  // where the groups go: by default the other scratch buffer at their final
  // positions; with areas, a level-1 bucket goes to its area of B, and later
  // rounds go from B or the output to A and from A to the output
  uint8_t* dbuf = in_b ? p.bufA : p.bufB;
  uint32_t dpos = task.start;
  uint32_t dflags = in_b ? 0u : (uint32_t)TASK_SRC_B;  // where the emitted tasks' records lie
  const bool areas = STAGED && p.areas != 0;
  if (areas && threadIdx.x == 0 && !(task.flags & TASK_L1) && !in_b) atomicAdd(stats + STAT_DEEP, 1u);
  if (areas) {
    if (task.flags & TASK_L1) {
      dbuf = p.bufB;
      dpos = split_area(task.start);
      dflags = TASK_SRC_B;
    } else if (in_b || in_out) {
      dbuf = p.bufA;
      dflags = 0;
    } else {
      dbuf = p.out;
      dflags = TASK_SRC_OUT;
    }
  }
  uint8_t* oth = dbuf + (size_t)dpos * E;
  const uint32_t m = task.count;
  if constexpr (STAGED) {
    if (areas && (task.flags & TASK_L1)) {
      const int u = split_uniform<EW>(sm, p, task, src, oth, dpos, L, stats, err, par);
      if (u < 0) return false;
      if (u > 0) return true;
    }
  }
  int bits = bitlen64(task.hi - task.lo);
  int shift = bits > kSplitBits ? bits - kSplitBits : 0;
  uint32_t nbins = (uint32_t)((task.hi - task.lo) >> shift) + 1;
  const uint32_t w = warp_id(), lane = lane_id();

  // Histogram over the task's key range; if the keys actually present span
  // far fewer bits, histogram again over their own range so that the bins
  // split them finely.
  uint64_t blo = task.lo, bhi = task.hi;
  for (int pass = 0; pass < 2; ++pass) {
    for (int i = threadIdx.x; i < kSplitBins; i += kThreads) sm.hist[i] = 0;
    __syncthreads();
    uint64_t mn = ~0ull, mx = 0;
    auto add = [&](uint64_t key) {
      mn = key < mn ? key : mn;
      mx = key > mx ? key : mx;
      const uint64_t x = key > blo ? key - blo : 0;
      atomicAdd(&sm.hist[(uint32_t)min(x >> shift, (uint64_t)(nbins - 1))], 1u);
    };
    if constexpr (STAGED) {
      const SplitTiles<EW> tiles{src, m, sm, par};
      tiles.start();
      for (uint32_t i = 0; i * tiles.T < m; ++i) {
        const uint8_t* rb = tiles.wait(i, err);
        if (!rb) return false;
        const uint32_t nvalid = min(tiles.T, m - i * tiles.T);
        for (uint32_t e = threadIdx.x; e < nvalid; e += kThreads) add(load_key_aligned4(rb + (size_t)e * E, p.key));
        __syncthreads();
        tiles.release(i);
      }
    } else {
      constexpr int U = 8;  // keys in flight per thread
      for (uint32_t i0 = 0; i0 < m; i0 += kThreads * U) {
        uint64_t kk[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          uint32_t i = i0 + u * kThreads + threadIdx.x;
          kk[u] = i < m ? key_at(src, i, E, p.key) : 0;
        }
#pragma unroll
        for (int u = 0; u < U; ++u)
          if (i0 + u * kThreads + threadIdx.x < m) add(kk[u]);
      }
    }
    block_minmax(mn, mx, sm.red);
    if (pass == 1 || bitlen64(mx - mn) + 4 > bits) break;
    blo = mn;
    bhi = mx;
    bits = bitlen64(bhi - blo);
    shift = bits > kSplitBits ? bits - kSplitBits : 0;
    nbins = (uint32_t)((bhi - blo) >> shift) + 1;
  }
  // Crowded bins (clustered keys): in a bucket of kRefineMin records or
  // more, a bin of more than kCrowded records and four times the mean is
  // cut into 2^r sub-bins of its key range (r up to
  // kSplitBits, at most kFineBins bins in all) and the bucket is
  // histogrammed once more over these fine bins, so that it splits in one
  // round rather than sending every crowded bin round the split again.  Fine
  // bins keep key order: those of bin b follow those of bin b - 1.
  const uint32_t crowd = (uint32_t)max((unsigned long long)kCrowded, 4ull * (m / nbins));
  bool crowded = false;
  for (uint32_t b = threadIdx.x; b < nbins; b += kThreads) crowded |= sm.hist[b] > crowd;
  const bool refined = __syncthreads_or(crowded) && shift > 0 && m >= kRefineMin;
  uint32_t* counts = sm.hist;  // bins the groups are formed from
  uint32_t nfine = nbins;
  if (refined) {
    // sub-bin bits: about 128 records per fine bin, fewer bits for all
    // while the total exceeds kFineBins
    auto rbits = [&](uint32_t c, int cut) -> uint32_t {
      if (c <= crowd) return 0;
      const int r = min(min(bitlen64(c - 1) - 7, kSplitBits), shift) - cut;
      return r > 0 ? (uint32_t)r : 0u;
    };
    constexpr int PER = kSplitBins / kThreads;
    int cut = 0;
    uint32_t total = 0, pre = 0;
    for (;;) {
      uint32_t s = 0;
#pragma unroll
      for (int i = 0; i < PER; ++i) {
        const uint32_t b = threadIdx.x * PER + i;
        if (b < nbins) s += 1u << rbits(sm.hist[b], cut);
      }
      pre = block_exclusive_scan<uint32_t>(s, sm.scan_tmp, &total);
      if (total <= (uint32_t)kFineBins) break;
      ++cut;  // all-zero bits give nbins <= kSplitBins fine bins, so this ends
    }
    uint32_t cm[PER];
#pragma unroll
    for (int i = 0; i < PER; ++i) {
      const uint32_t b = threadIdx.x * PER + i;
      const uint32_t r = b < nbins ? rbits(sm.hist[b], cut) : 0;
      cm[i] = (pre << 4) | r;
      pre += b < nbins ? 1u << r : 0u;
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < PER; ++i) sm.hist[threadIdx.x * PER + i] = cm[i];
    // the fine histogram lives in the staging tile until the scatter
    counts = reinterpret_cast<uint32_t*>(sm.stage);
    for (int i = threadIdx.x; i < kFineBins; i += kThreads) counts[i] = 0;
    __syncthreads();
    constexpr int U = 8;
    for (uint32_t i0 = 0; i0 < m; i0 += kThreads * U) {
      uint64_t kk[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        uint32_t i = i0 + u * kThreads + threadIdx.x;
        kk[u] = i < m ? key_at(src, i, E, p.key) : 0;
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        uint32_t i = i0 + u * kThreads + threadIdx.x;
        if (i < m) atomicAdd(&counts[fine_bin(sm.hist, kk[u], blo, shift, nbins)], 1u);
      }
    }
    nfine = total;
    if (threadIdx.x == 0) atomicAdd(stats + STAT_REFINED, 1u);
    __syncthreads();
  }
  // exclusive scan of the bins, then the group of every bin
  const uint32_t nscan = refined ? (uint32_t)kFineBins : (uint32_t)kSplitBins;
  if (refined) scan_bins<kFineBins / kThreads>(counts, sm.scan_tmp);
  else scan_bins<kSplitBins / kThreads>(counts, sm.scan_tmp);
  // group of a bin = slot of its midpoint: a bin holding most of the records
  // never shares a group with the empty bins on either side, so every group
  // that is split again covers a strictly narrower key range
  // target <= m / 2 keeps the first and the last bin's midpoints at least a
  // target apart, so no group spans every bin: each re-split narrows
  const uint32_t target = min(max((uint32_t)(kLocalMax - kLocalMax / 8), (m + kMaxGroups - 1) / kMaxGroups), m / 2);
  for (uint32_t b = threadIdx.x; b < nscan; b += kThreads) {
    uint32_t gb_ = kMaxGroups - 1;
    if (b < nfine) {
      uint64_t incl = b + 1 < nscan ? counts[b + 1] : m;
      unsigned long long mid2 = (unsigned long long)counts[b] + incl;
      gb_ = (uint32_t)min(mid2 / (2ull * target), (unsigned long long)(kMaxGroups - 1));
    }
    sm.gmap[b] = (uint16_t)gb_;
  }
  __syncthreads();
  for (uint32_t b = threadIdx.x; b < nfine; b += kThreads) {
    int gcur = sm.gmap[b];
    int gprev = b ? (int)sm.gmap[b - 1] : -1;
    for (int g = gprev + 1; g <= gcur; ++g) {
      sm.gstart[g] = counts[b];
      sm.gfirst[g] = b;
    }
    if (b == nfine - 1) {
      for (int g = gcur + 1; g <= kMaxGroups; ++g) {
        sm.gstart[g] = m;
        sm.gfirst[g] = nfine;
      }
    }
  }
  __syncthreads();
  for (int g = threadIdx.x; g < kMaxGroups; g += kThreads) sm.cursor[g] = sm.gstart[g];
  __syncthreads();
  // stable scatter src -> other by group: each tile is ranked by group
  // (warp-row ranking), placed in shared memory in group order and written
  // out by consecutive threads, so the runs of a group leave as coalesced
  // stores rather than one memory request per record
  static_assert(kMaxGroups == kThreads, "one group per thread in the tile scan");
  static_assert(T <= kThreads * 4 && T * E <= kSplitTileBytes, "tile staging size");
  const uint32_t g_me = threadIdx.x;
  if constexpr (STAGED) {
    // the tile arrives in input order; its records leave from there in group
    // order through perm (input slot of each group-ordered record)
    constexpr int SRPT = staged_split_tile<EW>() / kThreads;
    static_assert(SRPT * kThreads == staged_split_tile<EW>() && SRPT <= 4, "staged tile shape");
    using V = typename std::conditional<E % 16 == 0, uint4,
                                        typename std::conditional<E % 8 == 0, uint2, uint32_t>::type>::type;
    constexpr uint32_t VPR = E / sizeof(V);
    const SplitTiles<EW> tiles{src, m, sm, par};
    tiles.start();
    for (uint32_t i = 0; i * tiles.T < m; ++i) {
      const uint32_t nvalid = min(tiles.T, m - i * tiles.T);
      const uint8_t* rb = tiles.wait(i, err);  // (a barrier: the last tile's rows are clear)
      if (!rb) return false;
      uint32_t grp[SRPT], rank[SRPT], lead[SRPT];
#pragma unroll
      for (int r = 0; r < SRPT; ++r) {
        const uint32_t e = w * 32 * SRPT + r * 32 + lane;
        grp[r] = kNoBucket;
        if (e < nvalid) {
          const uint64_t key = load_key_aligned4(rb + (size_t)e * E, p.key);
          uint32_t bin;
          if (refined) {
            bin = fine_bin(sm.hist, key, blo, shift, nbins);
          } else {
            const uint64_t x = key > blo ? key - blo : 0;
            bin = (uint32_t)min(x >> shift, (uint64_t)(nbins - 1));
          }
          grp[r] = sm.gmap[bin];
        }
      }
      warp_ranks<SRPT, kGroupBits>(grp, rank, lead, sm.gcnt);
      __syncthreads();
      uint32_t gtot;
      tile_rank(g_me, 0, sm.gcnt, gtot);
      const uint32_t goff = block_exclusive_scan<uint32_t>(gtot, sm.scan_tmp, nullptr);
      sm.goff[g_me] = goff;
      __syncthreads();
#pragma unroll
      for (int r = 0; r < SRPT; ++r) {
        if (grp[r] == kNoBucket) continue;
        uint32_t all;
        const uint32_t slot = sm.goff[grp[r]] + tile_rank(grp[r], rank[r], sm.gcnt, all);
        if (slot >= nvalid) {  // impossible with consistent ranks
          set_error(err, DEV_ERR_COUNT_MISMATCH);
          continue;
        }
        sm.perm[slot] = (uint16_t)(w * 32 * SRPT + r * 32 + lane);
        sm.sgrp[slot] = (uint16_t)grp[r];
      }
      __syncthreads();
      bool bad = false;
#pragma unroll (split_outs_unroll<EW>())
      for (uint32_t k = 0; k < (SplitTiles<EW>::T * VPR + kThreads - 1) / kThreads; ++k) {
        const uint32_t f = threadIdx.x + k * kThreads;
        if (f >= nvalid * VPR) break;
        const uint32_t j = f / VPR, qw = f % VPR;
        const uint32_t g = sm.sgrp[j] & (kMaxGroups - 1);
        const uint32_t from = min((uint32_t)sm.perm[j], nvalid - 1);
        const uint32_t dest = sm.cursor[g] + (j - sm.goff[g]);
        if (dest < m)
          st_global(reinterpret_cast<V*>(oth + (size_t)dest * E) + qw, reinterpret_cast<const V*>(rb + (size_t)from * E)[qw]);
        else bad = true;
      }
      if (bad) set_error(err, DEV_ERR_COUNT_MISMATCH);
      __syncthreads();
      tiles.release(i);
      sm.cursor[g_me] += gtot;
      clear_rows<SRPT>(grp, lead, sm.gcnt);
    }
    __syncthreads();
  } else
  for (uint32_t t0 = 0; t0 < m; t0 += T) {
    const uint32_t nvalid = min((uint32_t)T, m - t0);
    // the tile after next heads for L2 (its loads below then wait on L2, not DRAM)
    if (threadIdx.x == 0 && t0 + 2 * T < m) prefetch_l2_range(src + (size_t)(t0 + 2 * T) * E, min((uint32_t)T, m - t0 - 2 * T) * E);
    uint32_t rec[RPT][EW];
    uint32_t grp[RPT], rank[RPT], lead[RPT];
#pragma unroll
    for (int r = 0; r < RPT; ++r) {
      uint32_t e = w * 32 * RPT + r * 32 + lane;
      grp[r] = kNoBucket;
      if (e < nvalid) {
        RecIO<EW>::load(src + (size_t)(t0 + e) * E, rec[r]);
        uint64_t key = key_from_regs<EW>(rec[r], p.key);
        uint32_t bin;
        if (refined) {
          bin = fine_bin(sm.hist, key, blo, shift, nbins);
        } else {
          uint64_t x = key > blo ? key - blo : 0;
          bin = (uint32_t)min(x >> shift, (uint64_t)(nbins - 1));
        }
        grp[r] = sm.gmap[bin];
      }
    }
    warp_ranks<RPT, kGroupBits>(grp, rank, lead, sm.gcnt);
    __syncthreads();
    uint32_t gtot;
    tile_rank(g_me, 0, sm.gcnt, gtot);  // this thread's group: records in the tile
    const uint32_t goff = block_exclusive_scan<uint32_t>(gtot, sm.scan_tmp, nullptr);
    sm.goff[g_me] = goff;
    __syncthreads();
#pragma unroll
    for (int r = 0; r < RPT; ++r) {
      if (grp[r] == kNoBucket) continue;
      uint32_t all;
      const uint32_t slot = sm.goff[grp[r]] + tile_rank(grp[r], rank[r], sm.gcnt, all);
      if (slot >= nvalid) {  // impossible with consistent ranks; never write past the tile
        set_error(err, DEV_ERR_COUNT_MISMATCH);
        continue;
      }
      RecIO<EW>::store(sm.stage + (size_t)slot * E, rec[r]);
      sm.sgrp[slot] = (uint16_t)grp[r];
    }
    __syncthreads();
    {  // consecutive threads take consecutive words of consecutive records
      using V = typename std::conditional<E % 16 == 0, uint4,
                                          typename std::conditional<E % 8 == 0, uint2, uint32_t>::type>::type;
      constexpr uint32_t VPR = E / sizeof(V);
      bool bad = false;
#pragma unroll 1
      for (uint32_t k = 0; k < (T * VPR + kThreads - 1) / kThreads; ++k) {
        const uint32_t f = threadIdx.x + k * kThreads;
        if (f >= nvalid * VPR) break;
        const uint32_t i = f / VPR, qw = f % VPR;
        const uint32_t g = sm.sgrp[i];
        const uint32_t dest = sm.cursor[g] + (i - sm.goff[g]);
        if (dest < m)
          st_global(reinterpret_cast<V*>(oth + (size_t)dest * E) + qw, reinterpret_cast<const V*>(sm.stage + (size_t)i * E)[qw]);
        else bad = true;
      }
      if (bad) set_error(err, DEV_ERR_COUNT_MISMATCH);
    }
    __syncthreads();
    sm.cursor[g_me] += gtot;
    clear_rows<RPT>(grp, lead, sm.gcnt);
    __syncthreads();
  }
  __threadfence_block();
  // one task per group
  if constexpr (std::is_same<Sink, EngineSink>::value) {
    // the groups go to the engine's queue in one reservation
    static_assert(kMaxGroups == kThreads, "one group per thread");
    const uint32_t g = threadIdx.x;
    const uint32_t g0 = sm.gstart[g], g1 = sm.gstart[g + 1];
    uint32_t n = 0, s = 0;
    uint64_t glo = 0, ghi = 0;
    bool cp = false;
    if (g1 > g0) {
      const uint32_t b0 = sm.gfirst[g], b1 = sm.gfirst[g + 1];
      s = g1 - g0;
      glo = refined ? fine_bin_lo(sm.hist, b0, blo, shift, nbins) : blo + ((uint64_t)b0 << shift);
      ghi = b1 >= sm.gfirst[kMaxGroups] ? bhi
            : (refined ? fine_bin_lo(sm.hist, b1, blo, shift, nbins) : blo + ((uint64_t)b1 << shift)) - 1;
      cp = glo == ghi || s == 1;
      n = cp ? (s + kCopyPiece - 1) / kCopyPiece : 1;
      if (!cp && s > (uint32_t)kLocalMax) atomicAdd(stats + STAT_PUSHED, 1u);
    }
    const bool nsrc_b = !in_b;
    const uint32_t start = task.start + g0;
    engine_emit(L.q, n,
                [&](uint32_t i) {
                  return cp ? make_task(start + i * kCopyPiece, min(kCopyPiece, s - i * kCopyPiece), glo, ghi,
                                        nsrc_b, true)
                            : make_task(start, s, glo, ghi, nsrc_b, false);
                },
                &sm.emit_base, sm.scan_tmp, err);
    return true;
  } else {
    for (int g = threadIdx.x; g < kMaxGroups; g += kThreads) {
      const uint32_t g0 = sm.gstart[g], g1 = sm.gstart[g + 1];
      if (g1 == g0) continue;
      const uint32_t b0 = sm.gfirst[g], b1 = sm.gfirst[g + 1];
      const uint32_t s = g1 - g0;
      const uint64_t glo = refined ? fine_bin_lo(sm.hist, b0, blo, shift, nbins) : blo + ((uint64_t)b0 << shift);
      const uint64_t ghi = b1 >= sm.gfirst[kMaxGroups] ? bhi  // (the number of bins there)
                           : (refined ? fine_bin_lo(sm.hist, b1, blo, shift, nbins) : blo + ((uint64_t)b1 << shift)) - 1;
      if (glo == ghi || s == 1) {
        L.copy(task.start + g0, dpos + g0, s, glo, ghi, dflags, err);
      } else if (s <= (uint32_t)kLocalMax) {
        L.local(make_task_at(task.start + g0, dpos + g0, s, glo, ghi, dflags), err);
      } else {
        atomicAdd(stats + STAT_PUSHED, 1u);
        L.split(make_task_at(task.start + g0, dpos + g0, s, glo, ghi, dflags), err);
      }
    }
    __syncthreads();
  }
  return true;
}

template <int EW>
__global__ void __launch_bounds__(kThreads, 2) k_split(HsortParams p, TaskLists L, uint32_t* __restrict__ work,
                                                        uint32_t* __restrict__ stats, uint32_t* __restrict__ err) {
  extern __shared__ __align__(128) uint8_t smem_raw[];
  SplitSmemOf<EW>& sm = *reinterpret_cast<SplitSmemOf<EW>*>(smem_raw);
  const uint32_t nt = min(*L.nsplit_in, L.cap_split);
  for (int i = threadIdx.x; i < kMaxGroups * kWarps; i += kThreads) sm.gcnt[i] = 0;
  if (threadIdx.x == 0) {
    mbar_init(&sm.bar[0], 1);
    mbar_init(&sm.bar[1], 1);
    mbar_init_fence();
  }
  uint32_t par = 0;  // next completion parity of each staging buffer
  for (;;) {
    if (threadIdx.x == 0) {
      uint32_t id = atomicAdd(work, 1u);
      sm.task_id = id;
      if (id < nt) sm.next = L.split_in[id];
    }
    __syncthreads();
    const uint32_t t = sm.task_id;
    const SortTask task = sm.next;
    __syncthreads();
    if (t >= nt) break;
    // forwarded as is (a task still in a reserved bucket region is split, so
    // that its records move out of the region in the first round)
    if (task.from == task.start && ((task.flags & TASK_COPY) || task.count <= (uint32_t)kLocalMax)) {
      if (threadIdx.x == 0) push(L.local, L.nlocal, L.cap_local, task, err);
      continue;
    }
    if (task.from != task.start && ((task.flags & TASK_COPY) || task.count <= (uint32_t)kLocalMax)) {
      // a small bucket or a copy piece still in its reserved region: moved
      // out now (later rounds write scratch A at final positions, which may
      // cover a region); a copy piece is final, a small bucket becomes a
      // local task in scratch B
      // (with areas, a small bucket goes to its area of B)
      constexpr uint32_t E = EW * 4;
      const bool copy = (task.flags & TASK_COPY) != 0;
      const uint32_t to = split_staged<EW>() && p.areas ? split_area(task.start) : task.start;
      block_copy_ilp<EW>(p.bufA + (size_t)task.from * E, copy ? p.out + (size_t)task.start * E : p.bufB + (size_t)to * E,
                         task.count, kThreads);
      if (!copy && threadIdx.x == 0) {
        __threadfence();
        push(L.local, L.nlocal, L.cap_local, make_task_at(task.start, to, task.count, task.lo, task.hi, TASK_SRC_B),
             err);
      }
      __syncthreads();
      continue;
    }
    if (threadIdx.x == 0) atomicAdd(stats + STAT_SPLIT, 1u);
    if (!split_task<EW, split_staged<EW>()>(sm, p, task, RoundSink{L}, stats, err, par)) return;
  }
}

template <int EW, int NT = kLocalThreads>
__global__ void __launch_bounds__(NT, local_ctas_per_sm<EW>()) k_local(HsortParams p, const SortTask* __restrict__ tasks,
                                                        const uint32_t* __restrict__ ntasks, uint32_t cap,
                                                        uint32_t* __restrict__ work, uint32_t* __restrict__ stats) {
  extern __shared__ __align__(128) uint8_t smem_raw[];
  LocalSmemT<NT>& sm = *reinterpret_cast<LocalSmemT<NT>*>(smem_raw);
  constexpr uint32_t E = EW * 4;
  const uint32_t nt = min(*ntasks, cap);
  // thread 0 claims the next task while the current one is sorted, so the
  // claim (a global atomic) and the descriptor load overlap with work
  if (threadIdx.x == 0) {
    uint32_t id = atomicAdd(work, 1u);
    sm.task_id = id;
    if (id < nt) sm.next = tasks[id];
  }
  __syncthreads();
  for (;;) {
    const uint32_t t = sm.task_id;
    if (t >= nt) break;
    const SortTask task = sm.next;
    __syncthreads();
    if (warp_id() == 0) {
      // the claim and its descriptor wait in shared memory: registers live
      // across the sort would be saved to the stack around every pass call
      const uint32_t lane = lane_id();
      uint32_t nid = 0;
      SortTask nxt{};
      if (lane == 0) {
        nid = atomicAdd(work, 1u);
        if (nid < nt) nxt = tasks[nid];
        sm.pend_id = nid;
        sm.pend = nxt;
      }
      // the next task's records head for L2 while this one sorts; the
      // warp's lanes share the lines
      const uint32_t id = __shfl_sync(GB_FULL_MASK, nid, 0);
      if (id < nt) {
        const uint32_t from = __shfl_sync(GB_FULL_MASK, nxt.from, 0);
        const uint32_t cnt = __shfl_sync(GB_FULL_MASK, nxt.count, 0);
        const uint32_t flags = __shfl_sync(GB_FULL_MASK, nxt.flags, 0);
        const uint8_t* ns = ((flags & TASK_SRC_B) ? p.bufB : (flags & TASK_SRC_OUT) ? p.out : p.bufA) + (size_t)from * E;
        const uint8_t* ne = ns + (size_t)cnt * E;
        for (const uint8_t* q = (const uint8_t*)((uintptr_t)ns & ~(uintptr_t)127) + 128 * lane; q < ne;
             q += 128 * 32)
          asm volatile("prefetch.global.L2 [%0];" ::"l"(q));
      }
    }
    const uint8_t* src =
        ((task.flags & TASK_SRC_B) ? p.bufB : (task.flags & TASK_SRC_OUT) ? p.out : p.bufA) + (size_t)task.from * E;
    uint8_t* out = p.out + (size_t)task.start * E;
    if ((task.flags & TASK_COPY) || task.count == 1) {
      block_copy_ilp<EW>(src, out, task.count, NT);
      if (threadIdx.x == 0) atomicAdd(stats + STAT_COPY, 1u);
      __syncthreads();
    } else {
      local_sort<EW, NT>(sm, src, out, task.count, p.key, stats);
      if (threadIdx.x == 0) atomicAdd(stats + STAT_LOCAL, 1u);
    }
    if (threadIdx.x == 0) {
      sm.task_id = sm.pend_id;
      sm.next = sm.pend;
    }
    __syncthreads();
  }
}

// Local sorts of records up to 16 bytes, two CTAs per SM.  Thread 0 claims
// the next task while the current one sorts and, if it is a sort task,
// starts the bulk copy of its records into the other buffer; copy tasks and
// single records go straight from global memory to the output.  Task
// descriptors alternate between two shared slots, so one barrier per task
// separates a claim from its use.  A copy whose wait runs out (about a
// second) records DEV_ERR_TIMEOUT; the CTA then waits once more (bounded)
// for the copies it has in flight and stops.
template <int EW, int NT>
__global__ void __launch_bounds__(NT, 2) k_local_staged(HsortParams p, const SortTask* __restrict__ tasks,
                                                         const uint32_t* __restrict__ ntasks, uint32_t cap,
                                                         uint32_t* __restrict__ work, uint32_t* __restrict__ stats) {
  constexpr uint32_t E = EW * 4;
  constexpr uint32_t kBuf = staged_buf_bytes<EW>();
  extern __shared__ __align__(128) uint8_t smem_raw[];
  uint8_t* rbuf = smem_raw;  // [2][kBuf]
  LocalSmemP<NT>& sm = *reinterpret_cast<LocalSmemP<NT>*>(smem_raw + 2 * kBuf);
  uint32_t* err = stats + STAT_SLOTS;
  const uint32_t nt = min(*ntasks, cap);
  auto staged = [](const SortTask& t) { return !(t.flags & TASK_COPY) && t.count > 1 && t.count <= (uint32_t)kLocalMax; };
  auto source = [&](const SortTask& t) {
    return ((t.flags & TASK_SRC_B) ? p.bufB : (t.flags & TASK_SRC_OUT) ? p.out : p.bufA) + (size_t)t.from * E;
  };
  // the task's byte range rounded out to 16 bytes (the slack lies inside
  // the scratch allocations) into buffer `slot`
  auto issue = [&](const SortTask& t, int slot) {
    const uintptr_t a = (uintptr_t)source(t);
    const uintptr_t a0 = a & ~(uintptr_t)15;
    const uint32_t bytes = (uint32_t)(((a - a0) + (uintptr_t)t.count * E + 15) & ~(uintptr_t)15);
    bulk_load(rbuf + (size_t)slot * kBuf, (const void*)a0, bytes, &sm.bar[slot]);
  };
  for (int i = threadIdx.x; i <= (1 << kLocalBits); i += NT) sm.cnt[i] = 0;
  if (threadIdx.x == 0) {
    mbar_init(&sm.bar[0], 1);
    mbar_init(&sm.bar[1], 1);
    mbar_init_fence();
    const uint32_t id = atomicAdd(work, 1u);
    sm.task_id[0] = id;
    if (id < nt) {
      sm.task[0] = tasks[id];
      if (staged(sm.task[0])) issue(sm.task[0], 0);
    }
  }
  __syncthreads();
  uint32_t parity = 0;  // bit s: parity of the next completion of buffer s
  for (int it = 0;; ++it) {
    const int slot = it & 1;  // buffer and descriptor slot of this task; the next one takes the other
    const uint32_t t = sm.task_id[slot];
    if (t >= nt) break;
    const SortTask task = sm.task[slot];
    if (threadIdx.x == 0) {
      const uint32_t nid = atomicAdd(work, 1u);
      uint32_t st = 0;
      if (nid < nt) {
        const SortTask nxt = tasks[nid];
        sm.task[slot ^ 1] = nxt;
        if (staged(nxt)) {
          fence_proxy_async_smem();
          issue(nxt, slot ^ 1);
          st = 1;
        }
      }
      sm.task_id[slot ^ 1] = nid;
      sm.pend_staged = st;
    }
    uint8_t* out = p.out + (size_t)task.start * E;
    if (!staged(task)) {
      block_copy_ilp<EW>(source(task), out, task.count, NT);
      if (threadIdx.x == 0) atomicAdd(stats + STAT_COPY, 1u);
    } else {
      bool ok = mbar_wait_bounded(&sm.bar[slot], (parity >> slot) & 1u, kBulkWaitPolls);
      ok = __syncthreads_and(ok);
      if (!ok) {  // stop: wait once more for this CTA's copies, then leave
        if (threadIdx.x == 0) set_error(err, DEV_ERR_TIMEOUT);
        mbar_wait_bounded(&sm.bar[slot], (parity >> slot) & 1u, kBulkWaitPolls);
        if (sm.pend_staged) mbar_wait_bounded(&sm.bar[slot ^ 1], (parity >> (slot ^ 1)) & 1u, kBulkWaitPolls);
        return;
      }
      parity ^= 1u << slot;
      const uint8_t* rb = rbuf + (size_t)slot * kBuf + ((uintptr_t)source(task) & 15);
      local_sort_staged<EW, NT>(sm, rb, out, task.count, task.lo, task.hi, p.key, stats, err);
      if (threadIdx.x == 0) atomicAdd(stats + STAT_LOCAL, 1u);
    }
    __syncthreads();
  }
}

// ---------------------------------------------- persistent level-2 engine --
// Level 2 as ONE persistent launch: two CTAs per SM take tasks from a device
// queue in push order -- bucket splits, shared-memory local sorts and
// single-key copies alike -- and a split appends its groups to the same
// queue, so there are no rounds and no launch per round: a local task runs
// as soon as a CTA is free after its split has published it.
//   * a task becomes visible through its ready flag (written after the task,
//     with release order); a CTA claims the next index with an atomic and
//     waits for that flag;
//   * `pending` counts tasks pushed and not finished; a split adds its
//     children before it finishes, so pending reaches zero only when no task
//     is left and none can come: a CTA waiting on a flag then stops;
//   * every wait is bounded (about four seconds of polling, far above any
//     task) and records DEV_ERR_TIMEOUT if it runs out;
//   * shared memory: the split's and the local sort's arrays overlay each
//     other; a local task's records come in by a bulk copy, started for the
//     next task while the current local task sorts when that task is ready.
// Tasks always lie at their final positions (no reserved regions), so the
// order in which they run does not matter: their ranges are disjoint.
// Control words of a CTA, outside the overlaid arrays.  The task to run
// alternates between two slots (the running one is read by every thread
// while thread 0 fills the other), so one barrier per task separates them.
struct EngineCtl {
  uint64_t bar[2];      // completion of the two record buffers' copies
  SortTask task[2];     // the task to run
  uint32_t state[2];    // ENGINE_*
  uint32_t loaded[2];   // 1: the task's records are on their way into its buffer
  uint32_t slot[2];     // the task's record buffer
  SortTask next;        // the task claimed ahead, if it was ready
  uint32_t next_idx;    // index claimed ahead (kNoClaim: none)
  uint32_t next_ready;  // 1: `next` holds it
  uint32_t next_loaded; // 1: its records are on their way
  uint32_t parity;      // bit b: parity of the next completion of buffer b
  uint32_t dirty;       // kDirty* below
};
// The overlaid arrays that must be zero when a task starts: the local
// sort's bin counts (a split may have overwritten them) and the split's
// warp-row ranking table (a local sort may have).
constexpr uint32_t kDirtyBins = 1, kDirtyTable = 2;
constexpr uint32_t kNoClaim = 0xffffffffu;

template <int EW>
__host__ __device__ constexpr size_t engine_ctl_offset() {
  return ((sizeof(SplitSmem) > 2 * (size_t)staged_buf_bytes<EW>() + sizeof(LocalSmemP<kThreads>)
               ? sizeof(SplitSmem)
               : 2 * (size_t)staged_buf_bytes<EW>() + sizeof(LocalSmemP<kThreads>)) +
          127) & ~(size_t)127;
}
template <int EW>
constexpr size_t engine_smem_bytes() {
  return engine_ctl_offset<EW>() + sizeof(EngineCtl);
}

// Thread 0: waits until task i is ready; false (and *state DONE) when it
// will never come (pending reached zero first, or the wait ran out).
__device__ __forceinline__ bool engine_wait(const EngineQueue& q, uint32_t i, uint32_t* err) {
  if (i >= q.cap) return false;
  for (uint32_t k = 0; k < kEngineWaitPolls; ++k) {
    if (ld_acquire_u32(&q.ready[i])) return true;
    if (ld_acquire_u32(q.pending) == 0) return ld_acquire_u32(&q.ready[i]) != 0;
    __nanosleep(k < 64 ? 64 : 256);
  }
  set_error(err, DEV_ERR_TIMEOUT);
  return false;
}

template <int EW>
__device__ __forceinline__ bool engine_staged(const SortTask& t) {
  return !(t.flags & TASK_COPY) && t.count > 1 && t.count <= (uint32_t)kLocalMax;
}

template <int EW>
__global__ void __launch_bounds__(kThreads, 2) k_engine(HsortParams p, EngineQueue q, uint32_t* __restrict__ stats) {
  constexpr uint32_t E = EW * 4;
  constexpr uint32_t kBuf = staged_buf_bytes<EW>();
  extern __shared__ __align__(128) uint8_t smem_raw[];
  SplitSmem& ssm = *reinterpret_cast<SplitSmem*>(smem_raw);
  uint8_t* rbuf = smem_raw;
  LocalSmemP<kThreads>& lsm = *reinterpret_cast<LocalSmemP<kThreads>*>(smem_raw + 2 * kBuf);
  EngineCtl& c = *reinterpret_cast<EngineCtl*>(smem_raw + engine_ctl_offset<EW>());
  uint32_t* err = stats + STAT_SLOTS;
  const EngineSink sink{q};
  auto source = [&](const SortTask& t) {
    return ((t.flags & TASK_SRC_B) ? p.bufB : (t.flags & TASK_SRC_OUT) ? p.out : p.bufA) + (size_t)t.from * E;
  };
  auto issue = [&](const SortTask& t, uint32_t slot) {  // thread 0
    const uintptr_t a = (uintptr_t)source(t);
    const uintptr_t a0 = a & ~(uintptr_t)15;
    const uint32_t bytes = (uint32_t)(((a - a0) + (uintptr_t)t.count * E + 15) & ~(uintptr_t)15);
    fence_proxy_async_smem();
    bulk_load(rbuf + (size_t)slot * kBuf, (const void*)a0, bytes, &c.bar[slot]);
  };
  for (int i = threadIdx.x; i < kMaxGroups * kWarps; i += kThreads) ssm.gcnt[i] = 0;
  if (threadIdx.x == 0) {
    mbar_init(&c.bar[0], 1);
    mbar_init(&c.bar[1], 1);
    mbar_init_fence();
    c.parity = 0;
    c.dirty = kDirtyBins;  // the table is zeroed above; the bins are not
    c.next_idx = kNoClaim;
    c.next_ready = 0;
    c.next_loaded = 0;
    c.slot[0] = 0;
    c.loaded[0] = 0;
    const uint32_t i = atomicAdd(q.head, 1u);
    c.state[0] = engine_wait(q, i, err) ? ENGINE_HAVE : ENGINE_DONE;
    if (c.state[0] == ENGINE_HAVE) {
      c.task[0] = q.task[i];
      if (engine_staged<EW>(c.task[0])) {
        issue(c.task[0], 0);
        c.loaded[0] = 1;
      }
    }
  }
  __syncthreads();
  for (uint32_t it = 0;; ++it) {
    const uint32_t cur = it & 1u;
    if (c.state[cur] == ENGINE_DONE) break;
    const SortTask& task = c.task[cur];  // read where used (thread 0 fills the other slot meanwhile)
    const uint32_t slot = c.slot[cur], loaded = c.loaded[cur];
    const bool staged = engine_staged<EW>(task);
    const bool copy = (task.flags & TASK_COPY) || task.count == 1;
    const bool split = !staged && !copy;
    if (staged && threadIdx.x == 0) {  // claim the next task now; its records come in during this sort
      const uint32_t n = atomicAdd(q.head, 1u);
      c.next_idx = n;
      if (n < q.cap && ld_acquire_u32(&q.ready[n])) {
        c.next = q.task[n];
        c.next_ready = 1;
        if (engine_staged<EW>(c.next)) {
          issue(c.next, slot ^ 1);
          c.next_loaded = 1;
        }
      }
    }
    uint8_t* out = p.out + (size_t)task.start * E;
    if (copy) {
      block_copy_ilp<EW>(source(task), out, task.count, kThreads);
      if (threadIdx.x == 0) atomicAdd(stats + STAT_COPY, 1u);
    } else if (split) {
      if (c.dirty & kDirtyTable)  // the ranking table starts at zero (split_task's first barriers follow)
        for (int i = threadIdx.x; i < kMaxGroups * kWarps / 16; i += kThreads)
          reinterpret_cast<uint4*>(ssm.gcnt)[i] = make_uint4(0, 0, 0, 0);
      if (threadIdx.x == 0) atomicAdd(stats + STAT_SPLIT, 1u);
      uint32_t unused_par = 0;
      split_task<EW, false>(ssm, p, task, sink, stats, err, unused_par);
      if (threadIdx.x == 0) c.dirty = kDirtyBins;
    } else {
      if (c.dirty & kDirtyBins)  // the local sort expects zero bins (the barrier below follows)
        for (int i = threadIdx.x; i <= (1 << kLocalBits); i += kThreads) lsm.cnt[i] = 0;
      const uint32_t par = (c.parity >> slot) & 1u;
      bool ok = loaded ? mbar_wait_bounded(&c.bar[slot], par, kBulkWaitPolls) : false;
      ok = __syncthreads_and(ok);
      if (!ok) {  // the copy never completed: record it, wait once more for the copies in flight, stop
        if (threadIdx.x == 0) set_error(err, DEV_ERR_TIMEOUT);
        mbar_wait_bounded(&c.bar[slot], par, kBulkWaitPolls);
        if (c.next_loaded) mbar_wait_bounded(&c.bar[slot ^ 1], (c.parity >> (slot ^ 1)) & 1u, kBulkWaitPolls);
        return;
      }
      const uint8_t* rb = rbuf + (size_t)slot * kBuf + ((uintptr_t)source(task) & 15);
      local_sort_staged<EW, kThreads>(lsm, rb, out, task.count, task.lo, task.hi, p.key, stats, err);
      if (threadIdx.x == 0) {
        c.parity ^= 1u << slot;
        c.dirty = kDirtyTable;
        atomicAdd(stats + STAT_LOCAL, 1u);
      }
    }
    if (threadIdx.x == 0) {
      // a split's children were pushed before it counts as finished (their
      // pending increments come first, so pending cannot reach zero early)
      if (split) __threadfence();
      atomicSub(&*q.pending, 1u);
      uint32_t n = c.next_idx;
      bool have;
      SortTask nt{};
      if (n != kNoClaim && c.next_ready) {
        nt = c.next;
        have = true;
      } else {
        if (n == kNoClaim) n = atomicAdd(q.head, 1u);
        have = engine_wait(q, n, err);
        if (have) nt = q.task[n];
      }
      const uint32_t nxt = cur ^ 1u;
      const uint32_t nslot = staged ? (slot ^ 1) : slot;  // after a local task, the other buffer
      c.state[nxt] = have ? ENGINE_HAVE : ENGINE_DONE;
      c.task[nxt] = nt;
      c.slot[nxt] = nslot;
      c.loaded[nxt] = c.next_loaded;
      if (have && engine_staged<EW>(nt) && !c.next_loaded) {
        issue(nt, nslot);
        c.loaded[nxt] = 1;
      }
      c.next_idx = kNoClaim;
      c.next_ready = 0;
      c.next_loaded = 0;
    }
    __syncthreads();
  }
}

__global__ void k_engine_seed(const SortTask* __restrict__ split, const uint32_t* __restrict__ nsplit,
                              const SortTask* __restrict__ local, const uint32_t* __restrict__ nlocal,
                              uint32_t cap_split, uint32_t cap_local, EngineQueue q, uint32_t* err) {
  const uint32_t ns = min(*nsplit, cap_split), nl = min(*nlocal, cap_local);
  const uint32_t total = ns + nl;
  if (total > q.cap) {
    if (blockIdx.x == 0 && threadIdx.x == 0) set_error(err, DEV_ERR_TASK_OVERFLOW);
    return;
  }
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
    q.task[i] = i < ns ? split[i] : local[i - ns];
    q.ready[i] = 1u;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    *q.tail = total;
    *q.head = 0;
    *q.pending = total;
  }
}

// ------------------------------------------------------------ dispatch --
template <typename F>
bool dispatch_ew(uint32_t elsize, F&& f) {
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

bool hsort_supported(uint32_t elsize) {
  if (elsize % 4) return false;
  switch (elsize / 4) {
    case 2: case 3: case 4: case 6: case 8: case 10: case 12: case 16: return true;
    default: return false;
  }
}

int hsort_grid(uint32_t n) {
  int g = num_sms() * 2;  // chunks of the count matrix: two CTAs per SM count them
  uint64_t maxg = ((uint64_t)n + 4095) / 4096;
  if ((uint64_t)g > maxg) g = (int)(maxg < 1 ? 1 : maxg);
  return g;
}

cudaError_t sample_keys(const uint8_t* rec, uint32_t n, uint32_t elsize, gbsort_key_word key, uint32_t s,
                        uint64_t* out, cudaStream_t stream) {
  if (s == 0) return cudaSuccess;
  unsigned blocks = (s + 255) / 256;
  if (blocks > 4096) blocks = 4096;
  k_sample<<<blocks, 256, 0, stream>>>(rec, n, elsize, key, s, out);
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t plain_splitters(const uint64_t* sorted_sample, uint32_t s, int nsplit, uint64_t* splitters,
                            uint32_t* iters, int64_t* clt, int64_t* cle, cudaStream_t stream) {
  if (nsplit <= 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(iters, 0, sizeof(uint32_t), stream);
  if (e != cudaSuccess) return e;
  k_plain_splitters<<<(nsplit + 127) / 128, 128, 0, stream>>>(sorted_sample, s, nsplit, splitters, iters,
                                                               clt, cle);
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t heavy_table(const uint64_t* splitters, int nsplit, HeavyTable* table, uint32_t* held,
                        cudaStream_t stream) {
  k_heavy_table<<<1, 1024, 0, stream>>>(splitters, nsplit, table, held);
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t finalize_splitters(uint64_t* splitters, int nsplit, cudaStream_t stream, const uint32_t* only_if) {
  if (nsplit <= 1) return cudaSuccess;
  if (nsplit > 8192) return cudaErrorInvalidValue;
  k_finalize_splitters<<<1, 1024, 0, stream>>>(splitters, nsplit, only_if);
  note_launches(1);
  return cudaGetLastError();
}

// Opt the kernel in to `bytes` of dynamic shared memory (needed above 48 KB
// of dynamic plus static shared memory; harmless below).
static cudaError_t set_smem(const void* fn, size_t bytes) {
  return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

cudaError_t l1_count(const HsortParams& p, int lookup_kind, const uint64_t* splitters, int nbuckets,
                     const void* model, uint32_t* counts, uint32_t* stats, cudaStream_t stream, int c0, int c1) {
  const ModelDev m = model ? *(const ModelDev*)model : ModelDev{};
  const int g = p.chunks ? (int)p.chunks : hsort_grid(p.n);
  if (c1 < 0) c1 = g;
  if (c1 <= c0) return cudaSuccess;
  cudaError_t e;
  if (lookup_kind == LOOKUP_LEARNED) {
    size_t sm = lookup_smem_bytes<LOOKUP_LEARNED>(nbuckets, &m) + 4 * (size_t)((nbuckets + 1) & ~1) +
                8 * (size_t)nbuckets;
    if ((e = set_smem((const void*)k_l1_count<LOOKUP_LEARNED>, sm)) != cudaSuccess) return e;
    k_l1_count<LOOKUP_LEARNED><<<c1 - c0, kThreads, sm, stream>>>(p, splitters, nbuckets, m, counts, stats,
                                                                  (uint32_t)c0, (uint32_t)g);
    note_launches(1);
  } else {
    size_t sm = lookup_smem_bytes<LOOKUP_PLAIN>(nbuckets, &m) + 4 * (size_t)nbuckets;
    if ((e = set_smem((const void*)k_l1_count<LOOKUP_PLAIN>, sm)) != cudaSuccess) return e;
    k_l1_count<LOOKUP_PLAIN><<<c1 - c0, kThreads, sm, stream>>>(p, splitters, nbuckets, m, counts, stats,
                                                                (uint32_t)c0, (uint32_t)g);
    note_launches(1);
  }
  return cudaGetLastError();
}

uint32_t hsort_chunk_begin(uint32_t n, int c, int chunks) {
  return c >= chunks ? n : chunk_begin(n, (uint32_t)c, (uint32_t)chunks);
}

cudaError_t l1_scatter(const HsortParams& p, int nbuckets, const uint32_t* offsets, uint32_t* stats,
                       cudaStream_t stream, int c0, int c1, const uint32_t* skip_if) {
  if (nbuckets < 1 || nbuckets > (1 << kMaxBucketBits)) return cudaErrorInvalidValue;  // ids rank in 12 bits
  if (!p.bkt) return cudaErrorInvalidValue;  // the count writes the bucket ids the scatter reads
  const int g = p.chunks ? (int)p.chunks : hsort_grid(p.n);
  if (c1 < 0) c1 = g;
  if (c1 <= c0) return cudaSuccess;
  const int ctas = std::min(std::min(hsort_grid(p.n), num_sms() * GB_SCATTER_CTAS), c1 - c0);
  cudaError_t e = cudaSuccess;
  bool ok = dispatch_ew(p.elsize, [&](auto ewc) {
    constexpr int EW = decltype(ewc)::value;
    size_t sm = l1_scatter_smem<EW>(nbuckets);
    e = set_smem((const void*)k_l1_scatter<EW>, sm);
    if (e == cudaSuccess)
      k_l1_scatter<EW><<<ctas, kThreads, sm, stream>>>(p, nbuckets, offsets, g, stats, (uint32_t)c0, (uint32_t)c1,
                                                        skip_if);
    note_launches(1);
  });
  if (!ok) return cudaErrorInvalidValue;
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

static TaskLists lists_of(const TaskListsHost& h) {
  TaskLists L;
  L.split_in = h.split_in;
  L.nsplit_in = h.nsplit_in;
  L.split_out = h.split_out;
  L.nsplit_out = h.nsplit_out;
  L.local = h.local;
  L.nlocal = h.nlocal;
  L.cap_split = h.cap_split;
  L.cap_local = h.cap_local;
  return L;
}

__global__ void k_require_zero(const uint32_t* count, uint32_t* err) {
  if (threadIdx.x == 0 && *count != 0) set_error(err, DEV_ERR_LEVELS);
}

// cap[b] = ceil(sample share of bucket b * n * slack) + pad.
__global__ void k_bucket_caps(const uint64_t* __restrict__ x, uint32_t s, const uint64_t* __restrict__ S,
                              int nbuckets, uint32_t n, double sigmas, double spare, uint32_t pad,
                              uint32_t* __restrict__ cap) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nbuckets) return;
  // sample keys in [S[b-1], S[b]): lower bounds of the two splitters
  auto lower = [&](uint64_t k) {
    uint32_t lo = 0, hi = s;
    while (lo < hi) {
      uint32_t mid = (lo + hi) >> 1;
      if (x[mid] < k) lo = mid + 1;
      else hi = mid;
    }
    return lo;
  };
  const uint32_t i0 = b == 0 ? 0u : lower(S[b - 1]);
  const uint32_t i1 = b == nbuckets - 1 ? s : lower(S[b]);
  const double c = (double)(i1 - i0);
  const double want = (c + sigmas * sqrt(c + 1.0) + spare) * (double)n / (double)s;
  cap[b] = (uint32_t)min(want + 1.0, (double)n) + pad;
}

__global__ void k_region_offsets(uint32_t* __restrict__ counts, int chunks, int nbuckets,
                                 const uint32_t* __restrict__ region, const uint32_t* __restrict__ cap,
                                 uint32_t* __restrict__ total, int c0, int c1, uint32_t* overflow) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nbuckets) return;
  uint32_t run = total[b];
  uint32_t* row = counts + (size_t)b * chunks;
  for (int c = c0; c < c1; ++c) {
    const uint32_t x = row[c];
    row[c] = region[b] + run;
    run += x;
  }
  total[b] = run;
  // overflow[0] = first bucket that outgrew its region + 1; [1], [2] its
  // capacity and count (for the pipeline trace)
  if (run > cap[b] && atomicCAS(overflow, 0u, (uint32_t)b + 1) == 0) {
    overflow[1] = cap[b];
    overflow[2] = run;
  }
}

__global__ void k_build_region_tasks(const uint32_t* __restrict__ region, const uint32_t* __restrict__ total,
                                     const uint32_t* __restrict__ out_start, const uint64_t* __restrict__ S,
                                     int nbuckets, TaskLists L, uint32_t* err, uint32_t* stats, int b0, int b1) {
  const int b = b0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= b1) return;
  const uint32_t cnt = total[b];
  if (cnt == 0) return;
  atomicMax(stats + STAT_MAX_BUCKET, cnt);
  const uint64_t lo = b == 0 ? 0ull : S[b - 1];
  const uint64_t hi = b == nbuckets - 1 ? ~0ull : S[b] - 1;
  if (lo == hi || cnt == 1) {  // copy pieces, each moved by one CTA of the first split round
    for (uint32_t s0 = 0; s0 < cnt; s0 += kCopyPiece) {
      SortTask t = make_task_at(out_start[b] + s0, region[b] + s0, min(kCopyPiece, cnt - s0), lo, hi,
                                TASK_COPY | TASK_L1);
      push(L.split_out, L.nsplit_out, L.cap_split, t, err);
    }
  } else {
    SortTask t = make_task_at(out_start[b], region[b], cnt, lo, hi, TASK_L1);
    push(L.split_out, L.nsplit_out, L.cap_split, t, err);
  }
}

cudaError_t bucket_caps(const uint64_t* sorted_sample, uint32_t s, const uint64_t* splitters, int nbuckets,
                        uint32_t n, double sigmas, double spare, uint32_t pad, uint32_t* cap, cudaStream_t stream) {
  k_bucket_caps<<<(nbuckets + 255) / 256, 256, 0, stream>>>(sorted_sample, s, splitters, nbuckets, n, sigmas, spare,
                                                            pad, cap);
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t region_offsets(uint32_t* counts, int chunks, int nbuckets, const uint32_t* region, const uint32_t* cap,
                           uint32_t* total, int c0, int c1, uint32_t* overflow, cudaStream_t stream) {
  k_region_offsets<<<(nbuckets + 127) / 128, 128, 0, stream>>>(counts, chunks, nbuckets, region, cap, total, c0, c1,
                                                               overflow);
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t build_region_tasks(const uint32_t* region, const uint32_t* total, const uint32_t* out_start,
                               const uint64_t* splitters, int nbuckets, const TaskListsHost& lists, uint32_t* err,
                               uint32_t* stats, cudaStream_t stream, int b0, int b1) {
  if (b1 <= b0) return cudaSuccess;
  k_build_region_tasks<<<(b1 - b0 + 255) / 256, 256, 0, stream>>>(region, total, out_start, splitters, nbuckets,
                                                                  lists_of(lists), err, stats, b0, b1);
  k_order_tasks<<<1, 1024, 0, stream>>>(lists.split_out, lists.nsplit_out);
  note_launches(2);
  return cudaGetLastError();
}

cudaError_t require_zero(const uint32_t* count, uint32_t* err, cudaStream_t stream) {
  k_require_zero<<<1, 32, 0, stream>>>(count, err);
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t build_tasks(const uint32_t* offsets, int grid, const uint64_t* splitters, int nbuckets, uint32_t n,
                        const TaskListsHost& lists, uint32_t* err, uint32_t* stats, cudaStream_t stream, int b0,
                        int b1) {
  if (b1 < 0) b1 = nbuckets;
  if (b1 <= b0) return cudaSuccess;
  k_build_tasks<<<(b1 - b0 + 255) / 256, 256, 0, stream>>>(offsets, grid, splitters, nbuckets, n, lists_of(lists),
                                                           err, stats, b0, b1);
  k_order_tasks<<<1, 1024, 0, stream>>>(lists.split_out, lists.nsplit_out);
  note_launches(2);
  return cudaGetLastError();
}

int split_grid() { return num_sms() * 2; }
template <int EW>
int local_grid() { return num_sms() * local_ctas_per_sm<EW>(); }

cudaError_t run_split_round(const HsortParams& p, const TaskListsHost& lists, uint32_t* work_counter,
                            uint32_t* stats, uint32_t* err, cudaStream_t stream) {
  cudaError_t e = cudaMemsetAsync(work_counter, 0, sizeof(uint32_t), stream);
  if (e != cudaSuccess) return e;
  bool ok = dispatch_ew(p.elsize, [&](auto ewc) {
    constexpr int EW = decltype(ewc)::value;
    size_t sm = sizeof(SplitSmemOf<EW>);
    e = set_smem((const void*)k_split<EW>, sm);
    if (e == cudaSuccess)
      k_split<EW><<<split_grid(), kThreads, sm, stream>>>(p, lists_of(lists), work_counter, stats, err);
    note_launches(1);
  });
  if (!ok) return cudaErrorInvalidValue;
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

cudaError_t run_local(const HsortParams& p, const SortTask* tasks, const uint32_t* ntasks, uint32_t cap,
                      uint32_t* work_counter, uint32_t* stats, cudaStream_t stream) {
  cudaError_t e = cudaMemsetAsync(work_counter, 0, sizeof(uint32_t), stream);
  if (e != cudaSuccess) return e;
  bool ok = dispatch_ew(p.elsize, [&](auto ewc) {
    constexpr int EW = decltype(ewc)::value;
    if constexpr (EW <= 4) {  // records up to 16 bytes: staged in shared memory by bulk copies
      const size_t sm = staged_smem_bytes<EW, kStagedThreads>();
      e = set_smem((const void*)k_local_staged<EW, kStagedThreads>, sm);
      if (e == cudaSuccess)
        k_local_staged<EW, kStagedThreads><<<num_sms() * 2, kStagedThreads, sm, stream>>>(p, tasks, ntasks, cap,
                                                                                           work_counter, stats);
    } else {
      const size_t sm = sizeof(LocalSmemT<kLocalThreads>);
      e = set_smem((const void*)k_local<EW>, sm);
      if (e == cudaSuccess)
        k_local<EW><<<local_grid<EW>(), kLocalThreads, sm, stream>>>(p, tasks, ntasks, cap, work_counter, stats);
    }
    note_launches(1);
  });
  if (!ok) return cudaErrorInvalidValue;
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

bool engine_supported(uint32_t elsize) { return elsize % 4 == 0 && elsize / 4 >= 2 && elsize / 4 <= 4; }

cudaError_t run_engine(const HsortParams& p, const TaskListsHost& seed, SortTask* qtask, uint32_t* qready,
                       uint32_t* qctl, uint32_t qcap, uint32_t* stats, uint32_t* err, cudaStream_t stream) {
  EngineQueue q{qtask, qready, qctl, qctl + kEngineCtlStride, qctl + 2 * kEngineCtlStride, qcap};
  cudaError_t e = cudaMemsetAsync(qready, 0, sizeof(uint32_t) * qcap, stream);
  if (e != cudaSuccess) return e;
  k_engine_seed<<<num_sms() * 2, 256, 0, stream>>>(seed.split_in, seed.nsplit_in, seed.local, seed.nlocal,
                                                   seed.cap_split, seed.cap_local, q, err);
  note_launches(1);
  bool ok = dispatch_ew(p.elsize, [&](auto ewc) {
    constexpr int EW = decltype(ewc)::value;
    if constexpr (EW >= 2 && EW <= 4) {
      const size_t sm = engine_smem_bytes<EW>();
      e = set_smem((const void*)k_engine<EW>, sm);
      if (e == cudaSuccess) k_engine<EW><<<num_sms() * 2, kThreads, sm, stream>>>(p, q, stats);
      note_launches(1);
    } else {
      e = cudaErrorInvalidValue;
    }
  });
  if (!ok) return cudaErrorInvalidValue;
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

}  // namespace gb
