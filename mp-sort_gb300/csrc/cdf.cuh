// cdf.cuh -- the learned CDF model of the key and the bucket lookups.
//
// The histogram sort assigns every record to the bucket
//     t(key) = #{ j : S[j] <= key }          (S = nsplit sorted splitters)
// which is the device form of the reference's CLT/CLE counting
// (internal-parallel.h:85-126).  Two lookups compute exactly this t:
//
//   plain   -- binary search over all splitters (the reference's
//              _bsearch_last_le, internal-parallel.h:40-83);
//   learned -- a monotone piecewise-linear CDF F of the key predicts
//              g = floor(F(key) * nbuckets); a per-leaf window [g-dlo, g+dhi],
//              computed exactly from the splitters, brackets t, and a short
//              search inside it finishes (no search at all for a zero window).
//              If a window ever misses, the full search runs and a counter
//              records it; the result is t either way.
//
// The model: L = 2^lbits leaves uniform in (key - kmin) >> lshift; leaf j
// interpolates linearly between knots y[j] and y[j+1] (fp32, trained on
// (key, rank) pairs).  Every step is a monotone operation, so g is
// non-decreasing in the key.
#pragma once

#include "cdf_api.h"
#include "common.cuh"

namespace gb {

struct ModelDev {
  uint64_t kmin;
  int lshift;          // leaf = (key - kmin) >> lshift
  int lbits;           // leaves = 1 << lbits
  int nbuckets;        // splitters = nbuckets - 1
  int pad;
  const float2* knots; // [leaves]: (y[j], y[j+1])
  const uint32_t* win; // [leaves]: (dlo << 16) | dhi
  const CdfShape* shape;  // if set, kmin and lshift come from this device copy
};


// kmin / lshift from the device copy of the shape, when there is one.
__device__ __forceinline__ CdfShape resolve_shape(CdfShape sh) {
  if (sh.dev) {
    const CdfShape d = *sh.dev;
    sh.kmin = d.kmin;
    sh.lshift = d.lshift;
  }
  return sh;
}
__device__ __forceinline__ ModelDev resolve_model(ModelDev m) {
  if (m.shape) {
    const CdfShape d = *m.shape;
    m.kmin = d.kmin;
    m.lshift = d.lshift;
  }
  return m;
}

// Fraction of the way through the leaf, in [0, 1): the top 23 bits of the
// offset in the leaf placed in a float's mantissa (1.m - 1 = m / 2^23), so
// no integer-to-float conversion (those run on the slow 64-bit pipe here).
__device__ __forceinline__ float leaf_frac(uint64_t x, int lshift) {
  if (lshift == 0) return 0.f;
  const uint64_t m = x & ((1ull << lshift) - 1ull);
  const uint32_t top = lshift >= 23 ? (uint32_t)(m >> (lshift - 23)) : (uint32_t)(m << (23 - lshift));
  return __int_as_float(0x3f800000 | top) - 1.0f;
}

// floor(v) for v in [0, 2^23): adding 2^23 with round-toward-zero leaves
// the integer part in the low mantissa bits.
__device__ __forceinline__ int floor_small(float v) {
  return __float_as_int(__fadd_rz(v, 8388608.0f)) - 0x4b000000;
}

// (leaf, predicted bucket) for a key.
__device__ __forceinline__ void model_predict(uint64_t key, uint64_t kmin, int lshift, int lbits,
                                              int nbuckets, const float2* knots, uint32_t& leaf,
                                              uint32_t& g) {
  const uint32_t nleaf = 1u << lbits;
  float f;
  if (key < kmin) {
    leaf = 0;
    f = knots[0].x;
  } else {
    uint64_t x = key - kmin;
    uint64_t l = lshift >= 64 ? 0 : (x >> lshift);
    if (l >= nleaf) {
      leaf = nleaf - 1;
      f = knots[leaf].y;
    } else {
      leaf = (uint32_t)l;
      float2 k = knots[leaf];
      f = fmaf(leaf_frac(x, lshift), k.y - k.x, k.x);
      f = fminf(fmaxf(f, k.x), k.y);
    }
  }
  const float v = fmaxf(f * (float)nbuckets, 0.f);
  const int b = floor_small(fminf(v, 8388607.f));
  g = (uint32_t)min(b, nbuckets - 1);
}

// t = #{ j in [lo, hi) : S[j] <= key } + lo, valid when S[lo-1] <= key < S[hi].
__device__ __forceinline__ uint32_t upper_bound_in(const uint64_t* S, uint32_t lo, uint32_t hi,
                                                   uint64_t key) {
  while (lo < hi) {
    uint32_t mid = (lo + hi) >> 1;
    if (S[mid] <= key) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ uint32_t bucket_plain(const uint64_t* S, int nbuckets, uint64_t key) {
  return upper_bound_in(S, 0, (uint32_t)(nbuckets - 1), key);
}

__device__ __forceinline__ uint32_t bucket_learned(const uint64_t* S, const ModelDev& m,
                                                   const float2* knots, const uint32_t* win,
                                                   uint64_t key, uint32_t* misses) {
  uint32_t leaf, g;
  model_predict(key, m.kmin, m.lshift, m.lbits, m.nbuckets, knots, leaf, g);
  const uint32_t w = win[leaf];
  // a zero window means the prediction equals the true bucket at every key
  // of the leaf (the windows are exact maxima over the leaf), so no splitter
  // needs to be read
  if (w == 0) return g;
  const uint32_t nsplit = (uint32_t)(m.nbuckets - 1);
  uint32_t lo = g > (w >> 16) ? g - (w >> 16) : 0u;
  uint32_t hi = min(g + (w & 0xffffu), nsplit);
  bool ok = (lo == 0 || S[lo - 1] <= key) && (hi == nsplit || S[hi] > key);
  if (!ok) {
    if (misses) atomicAdd(misses, 1u);
    return upper_bound_in(S, 0, nsplit, key);
  }
  return upper_bound_in(S, lo, hi, key);
}

}  // namespace gb
