// common.cuh -- device helpers shared by every gbsort kernel (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/gbsort_key.h"

#define GB_FULL_MASK 0xffffffffu

namespace gb {

// Launch shape of the record-streaming kernels: one CTA of 512 threads per
// SM slot, 16 warps.
constexpr int kThreads = 512;
constexpr int kWarps = kThreads / 32;

// Device error word: kernels never trap; they record the first error here and
// return.  The host reads it after the pipeline and maps it to a status code.
enum DevError : uint32_t {
  DEV_OK = 0,
  DEV_ERR_TASK_OVERFLOW = 1,   // a task list ran out of room
  DEV_ERR_LEVELS = 2,          // more split rounds than the key width allows
  DEV_ERR_COUNT_MISMATCH = 3,  // a scatter wrote a different count than counted
  DEV_ERR_WINDOW = 4,          // learned search window missed (never expected)
  DEV_ERR_TIMEOUT = 5,         // a bounded spin-wait gave up
};

__device__ __forceinline__ void set_error(uint32_t* err, uint32_t code) {
  if (err) atomicCAS(err, 0u, code);
}

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31; }
__device__ __forceinline__ uint32_t warp_id() { return threadIdx.x >> 5; }
__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Lanes of the warp whose label has the same low `bits` bits as this lane's:
// one ballot per bit.  Runs on the integer pipes at a fixed cost, where the
// native match instruction serialises over the distinct values in the warp
// (and ranking tiles of thousands of buckets has up to 32 of them).
template <int BITS>
__device__ __forceinline__ uint32_t match_bits(uint32_t label) {
  uint32_t m = GB_FULL_MASK;
#pragma unroll
  for (int b = 0; b < BITS; ++b) {
    const uint32_t bit = (label >> b) & 1u;
    const uint32_t v = __ballot_sync(GB_FULL_MASK, bit);
    m &= bit ? v : ~v;
  }
  return m;
}
__device__ __forceinline__ uint32_t match_bits_rt(uint32_t label, int bits) {
  uint32_t m = GB_FULL_MASK;
  for (int b = 0; b < bits; ++b) {
    const uint32_t bit = (label >> b) & 1u;
    const uint32_t v = __ballot_sync(GB_FULL_MASK, bit);
    m &= bit ? v : ~v;
  }
  return m;
}

// Order-preserving 64-bit word of a key field held as raw bits (binding.pyx
// radix_func_*: u8 as is, u4 zero-extended, i8/i4 sign-extended plus 2^63).
__device__ __forceinline__ uint64_t map_key(uint64_t raw, uint32_t width, uint32_t is_signed) {
  if (width == 8) return is_signed ? (raw ^ 0x8000000000000000ull) : raw;
  uint32_t v = (uint32_t)raw;
  if (is_signed) return (uint64_t)(int64_t)(int32_t)v ^ 0x8000000000000000ull;
  return (uint64_t)v;
}

// Load one key word from a record whose address is 4-byte aligned.
__device__ __forceinline__ uint64_t load_key_aligned4(const uint8_t* rec, const gbsort_key_word& w) {
  const uint32_t* p = reinterpret_cast<const uint32_t*>(rec + w.offset);
  uint64_t raw = p[0];
  if (w.width == 8) raw |= (uint64_t)p[1] << 32;
  return map_key(raw, w.width, w.is_signed);
}

// Load one key word from a record at any byte alignment.
__device__ __forceinline__ uint64_t load_key_bytes(const uint8_t* rec, const gbsort_key_word& w) {
  uint64_t raw = 0;
  for (uint32_t b = 0; b < w.width; ++b) raw |= (uint64_t)rec[w.offset + b] << (8 * b);
  return map_key(raw, w.width, w.is_signed);
}

// Select word `idx` of a register array without dynamic indexing.
template <int N>
__device__ __forceinline__ uint32_t reg_select(const uint32_t (&a)[N], uint32_t idx) {
  uint32_t v = 0;
#pragma unroll
  for (int i = 0; i < N; ++i) v = (i == (int)idx) ? a[i] : v;
  return v;
}

// Key of a record held in registers as E_WORDS 32-bit words.
// A 64-bit key first in the record takes a branch of its own (uniform over
// the grid): no word selection (measured on the level-1 scatter when it
// still looked keys up: 1e9 x 16 B, 17.9 -> 17.5 ms).
template <int E_WORDS>
__device__ __forceinline__ uint64_t key_from_regs(const uint32_t (&r)[E_WORDS], const gbsort_key_word& w) {
  if constexpr (E_WORDS >= 2) {
    if (w.offset == 0 && w.width == 8) {
      const uint64_t raw = (uint64_t)r[0] | ((uint64_t)r[1] << 32);
      return w.is_signed ? raw ^ 0x8000000000000000ull : raw;
    }
  }
  uint32_t k = w.offset >> 2;
  uint64_t raw = reg_select<E_WORDS>(r, k);
  if (w.width == 8) raw |= (uint64_t)reg_select<E_WORDS>(r, k + 1) << 32;
  return map_key(raw, w.width, w.is_signed);
}

__device__ __forceinline__ int bitlen64(uint64_t x) { return x ? 64 - __clzll(x) : 0; }

// ---------------------------------------------------------------------------
// Bulk asynchronous copies global -> shared memory (cp.async.bulk, the
// untiled TMA form) completing on an mbarrier.  Addresses and sizes are
// multiples of 16 bytes.  Waits are bounded: a wait that runs out returns
// false and the caller records DEV_ERR_TIMEOUT.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
// Makes initialised mbarriers visible to the async proxy (before a barrier).
__device__ __forceinline__ void mbar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
// Orders this thread's earlier shared-memory accesses before later async
// copies into the same memory.
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// One arrival that also expects `bytes` of transaction, then the copy.
__device__ __forceinline__ void bulk_load(void* dst_smem, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst_smem)),
               "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}

__device__ __forceinline__ bool mbar_test(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{ .reg .pred p; mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Waits for the completion of the mbarrier phase of the given parity, polling
// at most `limit` times with a short back-off; false if it ran out.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint32_t limit) {
  for (uint32_t i = 0; i < limit; ++i) {
    if (mbar_test(bar, parity)) return true;
    __nanosleep(i < 64 ? 20 : 200);
  }
  return mbar_test(bar, parity);
}
constexpr uint32_t kBulkWaitPolls = 1u << 22;  // about a second of polling

// Bulk prefetch into L2 of the 16-byte aligned part of [p, p + bytes).
__device__ __forceinline__ void prefetch_l2_range(const void* p, uint32_t bytes) {
  const uintptr_t a = ((uintptr_t)p + 15) & ~(uintptr_t)15;
  const uintptr_t b = ((uintptr_t)p + bytes) & ~(uintptr_t)15;
  if (b > a)
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(a), "r"((uint32_t)(b - a)) : "memory");
}

// Block-wide exclusive scan of one value per thread (NT threads).
// `tmp` holds NT / 32 entries.  Returns the exclusive prefix; *total gets the sum.
template <typename T, int NT = kThreads>
__device__ __forceinline__ T block_exclusive_scan(T v, T* tmp, T* total) {
  constexpr int NW = NT / 32;
  const uint32_t lane = lane_id(), w = warp_id();
  T x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T y = __shfl_up_sync(GB_FULL_MASK, x, o);
    if (lane >= (uint32_t)o) x += y;
  }
  if (lane == 31) tmp[w] = x;
  __syncthreads();
  if (w == 0) {
    T s = lane < (uint32_t)NW ? tmp[lane] : T(0);
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      T y = __shfl_up_sync(GB_FULL_MASK, s, o);
      if (lane >= (uint32_t)o) s += y;
    }
    if (lane < (uint32_t)NW) tmp[lane] = s;
  }
  __syncthreads();
  T warp_prefix = w ? tmp[w - 1] : T(0);
  T result = warp_prefix + x - v;
  if (total) *total = tmp[NW - 1];
  __syncthreads();
  return result;
}

// ---------------------------------------------------------------------------
// Stable block ranking by a small digit (the warp match/ballot ranking).
//
// Items are in "warp-chunk" order: item r of lane l in warp w is tile element
//   w * 32 * RPT + r * 32 + l,
// so each warp owns a contiguous run of the tile.  Ranks are positions in the
// tile stably sorted by digit.  `hist` holds kWarps << DIGIT_BITS uint16
// counters, warp-major (hist[w][d]), so the lanes of a warp touching
// different digits touch different banks.  Items with valid == false must
// carry the largest digit; they then land after every valid item.
// ---------------------------------------------------------------------------
template <int RPT, int DIGIT_BITS, int NT = kThreads>
struct BlockRank {
  static constexpr int kNW = NT / 32;
  static constexpr int kDigits = 1 << DIGIT_BITS;
  static constexpr int kCounters = kDigits * kNW;
  static constexpr int kDigitsPerThread = (kDigits + NT - 1) / NT;

  // ranks[r] receives the position of item r; digit_start (optional, kDigits
  // + 1 entries in shared memory) receives the start of every digit's run.
  __device__ __forceinline__ static void rank(const uint32_t (&digit)[RPT], uint32_t (&ranks)[RPT],
                                              uint16_t* hist, uint32_t* scan_tmp,
                                              uint32_t* digit_start) {
    const uint32_t lane = lane_id(), w = warp_id();
    for (int i = threadIdx.x; i < kCounters; i += NT) hist[i] = 0;
    __syncthreads();
    const uint32_t lt = lanemask_lt();
    uint16_t* wh = hist + w * kDigits;
#pragma unroll
    for (int r = 0; r < RPT; ++r) {
      const uint32_t d = digit[r];
      const uint32_t peers = match_bits<DIGIT_BITS>(d);
      const uint32_t before = wh[d];
      ranks[r] = before + __popc(peers & lt);
      __syncwarp();
      if ((peers & lt) == 0) wh[d] = (uint16_t)(before + __popc(peers));
      __syncwarp();
    }
    __syncthreads();
    // per digit: exclusive prefix over the warps, then over the digits
    uint32_t total;
    if constexpr (kDigits >= NT) {
      uint32_t tot[kDigitsPerThread];
      uint32_t sum = 0;
#pragma unroll
      for (int j = 0; j < kDigitsPerThread; ++j) {
        const int d = threadIdx.x * kDigitsPerThread + j;
        uint32_t run = 0;
        if (d < kDigits) {
#pragma unroll
          for (int q = 0; q < kNW; ++q) {
            uint32_t c = hist[q * kDigits + d];
            hist[q * kDigits + d] = (uint16_t)run;
            run += c;
          }
        }
        tot[j] = run;
        sum += run;
      }
      uint32_t base = block_exclusive_scan<uint32_t, NT>(sum, scan_tmp, &total);
#pragma unroll
      for (int j = 0; j < kDigitsPerThread; ++j) {
        const int d = threadIdx.x * kDigitsPerThread + j;
        if (d < kDigits) {
#pragma unroll
          for (int q = 0; q < kNW; ++q) hist[q * kDigits + d] = (uint16_t)(hist[q * kDigits + d] + base);
          if (digit_start) digit_start[d] = base;
        }
        base += tot[j];
      }
    } else {
      // fewer digits than threads: TPD adjacent lanes share a digit, each
      // summing kNW / TPD warps, combined with shuffles
      constexpr int TPD = NT / kDigits;
      constexpr int WPS = kNW / TPD > 0 ? kNW / TPD : 1;
      static_assert(TPD <= 32 && (32 % TPD) == 0, "digit groups must tile a warp");
      const int d = threadIdx.x / TPD, qq = threadIdx.x % TPD;
      uint32_t run = 0;
      if (qq * WPS < kNW) {
#pragma unroll
        for (int q = 0; q < WPS; ++q) {
          const int wq = qq * WPS + q;
          uint32_t c = hist[wq * kDigits + d];
          hist[wq * kDigits + d] = (uint16_t)run;
          run += c;
        }
      }
      uint32_t incl = run;
#pragma unroll
      for (int o = 1; o < TPD; o <<= 1) {
        uint32_t y = __shfl_up_sync(GB_FULL_MASK, incl, o);
        if (qq >= o) incl += y;
      }
      const uint32_t excl = incl - run;
      const uint32_t dtot = __shfl_sync(GB_FULL_MASK, incl, (lane | (TPD - 1)));
      uint32_t scan = block_exclusive_scan<uint32_t, NT>(qq == 0 ? dtot : 0u, scan_tmp, &total);
      const uint32_t base = __shfl_sync(GB_FULL_MASK, scan, lane & ~(uint32_t)(TPD - 1)) + excl;
      if (qq * WPS < kNW) {
#pragma unroll
        for (int q = 0; q < WPS; ++q) {
          const int wq = qq * WPS + q;
          hist[wq * kDigits + d] = (uint16_t)(hist[wq * kDigits + d] + base);
        }
      }
      if (digit_start && qq == 0) digit_start[d] = base;
    }
    if (digit_start && threadIdx.x == 0) digit_start[kDigits] = total;
    __syncthreads();
#pragma unroll
    for (int r = 0; r < RPT; ++r) ranks[r] += wh[digit[r]];
    __syncthreads();
  }
};

}  // namespace gb
