// cdf.cu -- training and use of the learned CDF model (see cdf.cuh).
//
// Data: the sorted sample x_0 <= ... <= x_{s-1} with targets r_i = i / s,
// i.e. (key, exact rank) pairs of the sample that the plain bisection also
// works on.  Model: knots y_0 .. y_L (fp32) of a piecewise-linear F over L
// uniform leaves of (key - kmin) >> lshift.  Loss: mean (F(x_i) - r_i)^2.
//
//   k_cdf_forward   -- F(x_i) and the loss
//   k_cdf_backward  -- dLoss/dy_j (each sample feeds its two knots)
//   k_cdf_stats     -- the tridiagonal normal matrix T and vector b of the
//                      least-squares fit, so that dLoss/dy = T y - b
//   k_cdf_epochs    -- every damped Jacobi-preconditioned gradient step in
//                      one CTA from T and b (no further pass over the sample)
//   k_cdf_project   -- non-decreasing knots in [0, 1] (cumulative max)
//   k_cdf_splitters -- S_j = least key with predicted bucket >= j + 1
//   k_cdf_heavy     -- keys covering a whole bucket of the sample get their
//                      own single-key bucket [k, k + 1)
//   k_cdf_windows   -- exact per-leaf [g - dlo, g + dhi] bracket of the true
//                      bucket, evaluated at the points where either the
//                      prediction or the true bucket can reach its extreme
#include "cdf.cuh"
#include "cdf_api.h"
#include "common.cuh"
#include "kernels.h"

namespace gb {

namespace {

__device__ __forceinline__ void features(uint64_t key, uint64_t kmin, int lshift, int lbits, uint32_t& leaf,
                                         float& frac) {
  const uint32_t nleaf = 1u << lbits;
  if (key < kmin) {
    leaf = 0;
    frac = 0.f;
    return;
  }
  uint64_t x = key - kmin;
  uint64_t l = lshift >= 64 ? 0 : (x >> lshift);
  if (l >= nleaf) {
    leaf = nleaf - 1;
    frac = 1.f;
    return;
  }
  leaf = (uint32_t)l;
  frac = leaf_frac(x, lshift);
}

__global__ void k_cdf_forward(const uint64_t* __restrict__ x, uint32_t s, CdfShape sh,
                              const float* __restrict__ y, float* __restrict__ pred, float* __restrict__ loss) {
  sh = resolve_shape(sh);
  __shared__ float red[32];
  float acc = 0.f;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < s; i += gridDim.x * blockDim.x) {
    uint32_t leaf;
    float frac;
    features(x[i], sh.kmin, sh.lshift, sh.lbits, leaf, frac);
    float f = fmaf(frac, y[leaf + 1] - y[leaf], y[leaf]);
    float r = (float)i / (float)s;
    if (pred) pred[i] = f;
    float e = f - r;
    acc += e * e;
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(GB_FULL_MASK, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    float v = threadIdx.x < blockDim.x / 32 ? red[threadIdx.x] : 0.f;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(GB_FULL_MASK, v, o);
    if (threadIdx.x == 0) atomicAdd(loss, v / (float)s);
  }
}

// grad[j] += sum_i 2 (F(x_i) - r_i) * dF/dy_j / s, with dF/dy_leaf = 1 - frac,
// dF/dy_{leaf+1} = frac.  Neighbouring samples share leaves (the sample is
// sorted), so lanes with the same leaf combine before the atomic.
__global__ void k_cdf_backward(const uint64_t* __restrict__ x, uint32_t s, CdfShape sh,
                               const float* __restrict__ y, float* __restrict__ grad) {
  sh = resolve_shape(sh);
  for (uint32_t i0 = blockIdx.x * blockDim.x; i0 < s; i0 += gridDim.x * blockDim.x) {
    uint32_t i = i0 + threadIdx.x;
    bool v = i < s;
    uint32_t leaf = 0xffffffffu;
    float g0 = 0.f, g1 = 0.f;
    if (v) {
      float frac;
      features(x[i], sh.kmin, sh.lshift, sh.lbits, leaf, frac);
      float f = fmaf(frac, y[leaf + 1] - y[leaf], y[leaf]);
      float e = 2.f * (f - (float)i / (float)s) / (float)s;
      g0 = e * (1.f - frac);
      g1 = e * frac;
    }
    uint32_t peers = __match_any_sync(GB_FULL_MASK, leaf);
    // reduce within the peer group (leader = lowest lane)
    float a0 = 0.f, a1 = 0.f;
    for (uint32_t m = peers; m; m &= m - 1) {
      int l = __ffs(m) - 1;
      a0 += __shfl_sync(peers, g0, l);
      a1 += __shfl_sync(peers, g1, l);
    }
    if (v && (peers & lanemask_lt()) == 0) {
      atomicAdd(&grad[leaf], a0);
      atomicAdd(&grad[leaf + 1], a1);
    }
  }
}

// Sufficient statistics of the fit.  The loss is quadratic in the knots:
// with a_i = (1 - frac_i) e_leaf + frac_i e_{leaf+1},
//   dLoss/dy = T y - b,  T = (2/s) sum_i a_i a_i^T,  b = (2/s) sum_i r_i a_i,
// T tridiagonal (diag[j]; off[j] couples knots j and j + 1) and its diagonal
// the Gauss-Newton curvature a training step divides by.  One pass over the
// sample gives T and b; every training step after it touches only the
// knots (k_cdf_epochs), with the same gradient k_cdf_backward computes
// from the sample.
__global__ void k_cdf_stats(const uint64_t* __restrict__ x, uint32_t s, CdfShape sh, float* __restrict__ diag,
                            float* __restrict__ off, float* __restrict__ b) {
  sh = resolve_shape(sh);
  const float c = 2.f / (float)s;
  for (uint32_t i0 = blockIdx.x * blockDim.x; i0 < s; i0 += gridDim.x * blockDim.x) {
    const uint32_t i = i0 + threadIdx.x;
    const bool v = i < s;
    uint32_t leaf = 0xffffffffu;
    float d0 = 0.f, d1 = 0.f, o = 0.f, b0 = 0.f, b1 = 0.f;
    if (v) {
      float f;
      features(x[i], sh.kmin, sh.lshift, sh.lbits, leaf, f);
      const float r = (float)i / (float)s;
      d0 = c * (1.f - f) * (1.f - f);
      d1 = c * f * f;
      o = c * (1.f - f) * f;
      b0 = c * r * (1.f - f);
      b1 = c * r * f;
    }
    // lanes of one leaf add up before the atomics (the sample is sorted)
    const uint32_t peers = __match_any_sync(GB_FULL_MASK, leaf);
    float a[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
    for (uint32_t m = peers; m; m &= m - 1) {
      const int l = __ffs(m) - 1;
      a[0] += __shfl_sync(peers, d0, l);
      a[1] += __shfl_sync(peers, d1, l);
      a[2] += __shfl_sync(peers, o, l);
      a[3] += __shfl_sync(peers, b0, l);
      a[4] += __shfl_sync(peers, b1, l);
    }
    if (v && (peers & lanemask_lt()) == 0) {
      atomicAdd(&diag[leaf], a[0]);
      atomicAdd(&diag[leaf + 1], a[1]);
      atomicAdd(&off[leaf], a[2]);
      atomicAdd(&b[leaf], a[3]);
      atomicAdd(&b[leaf + 1], a[4]);
    }
  }
}

// (T y - b)_j from the statistics; off has nknots - 1 entries.
__device__ __forceinline__ float stat_gradient(const float* y, const float* diag, const float* off, const float* b,
                                               int j, int nknots) {
  float g = diag[j] * y[j] - b[j];
  if (j > 0) g += off[j - 1] * y[j - 1];
  if (j + 1 < nknots) g += off[j] * y[j + 1];
  return g;
}

// `epochs` damped Jacobi-preconditioned gradient steps on the knots in one
// CTA: the end knots stay fixed (F(kmin) = 0, F(end) = 1), every other
// knot moves by -lr * g_j / diag_j, all from the previous epoch's knots.
__global__ void __launch_bounds__(1024) k_cdf_epochs(float* __restrict__ y, const float* __restrict__ diag,
                                                     const float* __restrict__ off, const float* __restrict__ b,
                                                     int nknots, int epochs, float lr) {
  extern __shared__ float sy[];
  for (int j = threadIdx.x; j < nknots; j += blockDim.x) sy[j] = y[j];
  __syncthreads();
  constexpr int kMaxPer = 8;  // knots per thread: nknots <= 8 * 1024 + 1
  for (int e = 0; e < epochs; ++e) {
    float nv[kMaxPer];
#pragma unroll
    for (int q = 0; q < kMaxPer; ++q) {
      const int j = threadIdx.x + q * blockDim.x;
      nv[q] = 0.f;
      if (j > 0 && j < nknots - 1) nv[q] = sy[j] - lr * stat_gradient(sy, diag, off, b, j, nknots) / (diag[j] + 1e-12f);
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < kMaxPer; ++q) {
      const int j = threadIdx.x + q * blockDim.x;
      if (j > 0 && j < nknots - 1) sy[j] = nv[q];
    }
    __syncthreads();
  }
  for (int j = threadIdx.x; j < nknots; j += blockDim.x) y[j] = sy[j];
}

__global__ void k_cdf_stat_grad(const float* __restrict__ y, const float* __restrict__ diag,
                                const float* __restrict__ off, const float* __restrict__ b, int nknots,
                                float* __restrict__ grad) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < nknots) grad[j] = stat_gradient(y, diag, off, b, j, nknots);
}

// Initial knots: the empirical CDF of the sample at every knot.
__global__ void k_cdf_init(const uint64_t* __restrict__ x, uint32_t s, CdfShape sh, float* __restrict__ y) {
  sh = resolve_shape(sh);
  const int nk = (1 << sh.lbits) + 1;
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < nk; j += gridDim.x * blockDim.x) {
    // knot j sits at key kmin + (j << lshift): count samples below it
    uint64_t kj;
    bool beyond = false;
    if (sh.lshift >= 64) beyond = j > 0;
    else {
      uint64_t off = (uint64_t)j << sh.lshift;
      if (sh.lshift > 0 && (off >> sh.lshift) != (uint64_t)j) beyond = true;
      kj = sh.kmin + off;
      if (kj < sh.kmin) beyond = true;  // wrapped past 2^64
    }
    uint32_t c;
    if (beyond) c = s;
    else {
      uint32_t lo = 0, hi = s;
      while (lo < hi) {
        uint32_t m = (lo + hi) >> 1;
        if (x[m] < kj) lo = m + 1; else hi = m;
      }
      c = lo;
    }
    y[j] = (float)c / (float)s;
  }
}

// Cumulative max, clamp to [0, 1], y_0 = 0, y_L = 1; knots[j] = (y_j, y_{j+1}).
__global__ void __launch_bounds__(1024) k_cdf_project(float* __restrict__ y, int nknots, float2* __restrict__ knots) {
  __shared__ float tmp[1024];
  const int per = (nknots + 1023) / 1024;
  const int b = threadIdx.x * per;
  float m = 0.f;
  for (int i = 0; i < per; ++i) {
    int j = b + i;
    if (j < nknots) {
      float v = fminf(fmaxf(y[j], 0.f), 1.f);
      if (j == 0) v = 0.f;
      if (j == nknots - 1) v = 1.f;
      y[j] = v;
      m = fmaxf(m, v);
    }
  }
  tmp[threadIdx.x] = m;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    float v = threadIdx.x >= (unsigned)o ? tmp[threadIdx.x - o] : 0.f;
    __syncthreads();
    tmp[threadIdx.x] = fmaxf(tmp[threadIdx.x], v);
    __syncthreads();
  }
  float run = threadIdx.x ? tmp[threadIdx.x - 1] : 0.f;
  for (int i = 0; i < per; ++i) {
    int j = b + i;
    if (j < nknots) {
      run = fmaxf(run, y[j]);
      y[j] = run;
    }
  }
  __syncthreads();
  for (int j = threadIdx.x; j + 1 < nknots; j += 1024) knots[j] = make_float2(y[j], y[j + 1]);
}

__device__ __forceinline__ uint32_t predict(uint64_t key, const CdfShape& sh, int nbuckets, const float2* knots) {
  uint32_t leaf, g;
  model_predict(key, sh.kmin, sh.lshift, sh.lbits, nbuckets, knots, leaf, g);
  return g;
}

// S_j = least key with predicted bucket >= j + 1 (all keys above if none).
__global__ void k_cdf_splitters(CdfShape sh, int nbuckets, const float2* __restrict__ knots,
                                uint64_t* __restrict__ S) {
  sh = resolve_shape(sh);
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nbuckets - 1) return;
  uint64_t lo = 0, hi = ~0ull;
  if (predict(hi, sh, nbuckets, knots) < (uint32_t)(j + 1)) {
    S[j] = ~0ull;
    return;
  }
  while (lo < hi) {  // smallest key with predict >= j + 1
    uint64_t mid = lo + ((hi - lo) >> 1);
    if (predict(mid, sh, nbuckets, knots) >= (uint32_t)(j + 1)) hi = mid;
    else lo = mid + 1;
  }
  S[j] = lo;
}

// Keys whose run in the sorted sample is at least one bucket long get the
// single-key bucket [k, k + 1): S at lower_bound(S, k) becomes k, the next
// splitter k + 1 (a later cumulative max restores the order).
__global__ void k_cdf_heavy(const uint64_t* __restrict__ x, uint32_t s, int nbuckets, uint64_t* __restrict__ S) {
  const uint32_t need = (s + nbuckets - 1) / nbuckets;
  const int nsplit = nbuckets - 1;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < s; i += gridDim.x * blockDim.x) {
    if (i > 0 && x[i - 1] == x[i]) continue;  // only run starts
    if (i + need > s || x[i + need - 1] != x[i]) continue;
    uint64_t k = x[i];
    uint32_t lo = 0, hi = nsplit;
    while (lo < hi) {
      uint32_t m = (lo + hi) >> 1;
      if (S[m] < k) lo = m + 1; else hi = m;
    }
    if (lo < (uint32_t)nsplit) S[lo] = k;
    if (lo + 1 < (uint32_t)nsplit && k != ~0ull) S[lo + 1] = k + 1;
  }
}

__global__ void __launch_bounds__(1024) k_cummax_u64(uint64_t* S, int n) {
  // single block: per-thread segments, then a max-scan of the segment maxima
  __shared__ uint64_t tmp[1024];
  const int per = (n + 1023) / 1024;
  const int b = threadIdx.x * per;
  uint64_t m = 0;
  for (int i = 0; i < per; ++i)
    if (b + i < n) m = S[b + i] > m ? S[b + i] : m;
  tmp[threadIdx.x] = m;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    uint64_t v = threadIdx.x >= o ? tmp[threadIdx.x - o] : 0;
    __syncthreads();
    if (v > tmp[threadIdx.x]) tmp[threadIdx.x] = v;
    __syncthreads();
  }
  uint64_t run = threadIdx.x ? tmp[threadIdx.x - 1] : 0;
  for (int i = 0; i < per; ++i)
    if (b + i < n) {
      run = S[b + i] > run ? S[b + i] : run;
      S[b + i] = run;
    }
}

__device__ __forceinline__ uint32_t true_bucket(const uint64_t* S, int nsplit, uint64_t key) {
  return upper_bound_in(S, 0, (uint32_t)nsplit, key);
}

__device__ __forceinline__ void window_update(uint32_t* win_lo, uint32_t* win_hi, uint64_t key, const CdfShape& sh,
                                              int nbuckets, const float2* knots, const uint64_t* S) {
  uint32_t leaf, g;
  model_predict(key, sh.kmin, sh.lshift, sh.lbits, nbuckets, knots, leaf, g);
  uint32_t t = true_bucket(S, nbuckets - 1, key);
  if (g > t) atomicMax(&win_lo[leaf], g - t);
  if (t > g) atomicMax(&win_hi[leaf], t - g);
}

// Extremes of g - t sit at the last key before each true step (S_j - 1) and
// at a leaf's last key; extremes of t - g at each S_j and at a leaf's first
// key.  Both lists are evaluated; first/last keys of a leaf are clamped to
// the key range.
__global__ void k_cdf_windows(CdfShape sh, int nbuckets, const float2* __restrict__ knots,
                              const uint64_t* __restrict__ S, uint32_t* __restrict__ win_lo,
                              uint32_t* __restrict__ win_hi) {
  sh = resolve_shape(sh);
  const int nleaf = 1 << sh.lbits;
  const int nsplit = nbuckets - 1;
  const int total = nsplit + nleaf;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
    if (i < nsplit) {
      uint64_t k = S[i];
      window_update(win_lo, win_hi, k, sh, nbuckets, knots, S);
      if (k > 0) window_update(win_lo, win_hi, k - 1, sh, nbuckets, knots, S);
    } else {
      int l = i - nsplit;
      uint64_t first, last;
      if (l == 0) first = 0;
      else first = sh.kmin + ((uint64_t)l << sh.lshift);
      if (l == nleaf - 1) last = ~0ull;
      else {
        uint64_t nx = sh.kmin + ((uint64_t)(l + 1) << sh.lshift);
        last = nx - 1;
      }
      if (sh.lshift >= 64) {  // a single leaf spans everything
        first = 0;
        last = ~0ull;
      }
      window_update(win_lo, win_hi, first, sh, nbuckets, knots, S);
      window_update(win_lo, win_hi, last, sh, nbuckets, knots, S);
      if (l == 0 && sh.kmin > 0) window_update(win_lo, win_hi, sh.kmin - 1, sh, nbuckets, knots, S);
    }
  }
}

// Knot pair of leaf l from the buckets of its first and last key: bucket + 1/2
// over nbuckets, so that the floor of the prediction is that bucket at both
// ends (nbuckets is a power of two: the quotients are exact).
__global__ void k_refit_knots(CdfShape sh, int nbuckets, const uint64_t* __restrict__ S, float2* __restrict__ knots,
                              const uint32_t* __restrict__ only_if) {
  if (only_if && *only_if == 0) return;
  sh = resolve_shape(sh);
  const int nleaf = 1 << sh.lbits;
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= nleaf) return;
  uint64_t first = sh.kmin + ((uint64_t)l << sh.lshift), last;
  if (l == nleaf - 1) last = ~0ull;
  else last = sh.kmin + ((uint64_t)(l + 1) << sh.lshift) - 1;
  if (sh.lshift >= 64) {  // a single leaf spans everything
    first = sh.kmin;
    last = ~0ull;
  }
  const float inv = 1.f / (float)nbuckets;
  const uint32_t bx = true_bucket(S, nbuckets - 1, first), by = true_bucket(S, nbuckets - 1, last);
  knots[l] = make_float2(((float)bx + 0.5f) * inv, ((float)by + 0.5f) * inv);
}

__global__ void k_pack_windows(const uint32_t* __restrict__ lo, const uint32_t* __restrict__ hi, int nleaf,
                               uint32_t* __restrict__ win, uint32_t* wide) {
  int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= nleaf) return;
  uint32_t a = min(lo[l], 0xffffu), b = min(hi[l], 0xffffu);
  win[l] = (a << 16) | b;
  atomicMax(wide, max(lo[l], hi[l]));
}

// S[i] = x_(C_i), the C_i-th smallest sample key, C_i = s (i+1) / (nsplit+1):
// the value the reference's bisection converges to (CLT < C <= CLE holds at
// the C-th order statistic and nowhere else), read directly.
__global__ void k_quantile_splitters(const uint64_t* __restrict__ x, uint32_t s, int nsplit, uint64_t* __restrict__ S,
                                     const uint32_t* __restrict__ only_if) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nsplit || (only_if && *only_if == 0)) return;
  uint64_t c = (uint64_t)s * (uint64_t)(i + 1) / (uint64_t)(nsplit + 1);
  S[i] = x[c > 0 ? c - 1 : 0];
}

// Check of a splitter set on the sorted sample: every key with a bucket's
// worth of sample copies must own a single-key bucket [k, k+1), and no
// other bucket may hold more than `limit` sample keys.  flags[0] != 0 means
// rejected; counts (nbuckets) must start at zero.
__global__ void k_vet_count(const uint64_t* __restrict__ x, uint32_t s, const uint64_t* __restrict__ S, int nbuckets,
                              uint32_t* __restrict__ counts, uint32_t* __restrict__ flags) {
  const uint32_t need = (s + nbuckets - 1) / nbuckets;
  const uint32_t nsplit = (uint32_t)(nbuckets - 1);
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < s; i += gridDim.x * blockDim.x) {
    const uint64_t k = x[i];
    const uint32_t t = upper_bound_in(S, 0, nsplit, k);
    const bool pure = t > 0 && S[t - 1] == k && (t == nsplit || S[t] == k + 1);
    if (!pure) atomicAdd(&counts[t], 1u);
    const bool run_start = i == 0 || x[i - 1] != k;
    if (run_start && i + need <= s && x[i + need - 1] == k && !pure) atomicOr(flags, 1u);
  }
}

__global__ void k_vet_max(const uint32_t* __restrict__ counts, int nbuckets, uint32_t limit, uint32_t* __restrict__ flags) {
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < nbuckets; b += gridDim.x * blockDim.x)
    if (counts[b] > limit) atomicOr(flags, 2u);
}

// Leaves of 2^lshift keys from kmin, lshift the least that covers kmax.
__host__ __device__ CdfShape make_shape(uint64_t kmin, uint64_t kmax, int lbits) {
  CdfShape sh{};
  sh.kmin = kmin;
  sh.lbits = lbits;
  int bits = 0;
  for (uint64_t d = kmax > kmin ? kmax - kmin : 0; d; d >>= 1) ++bits;
  sh.lshift = bits > lbits ? bits - lbits : 0;
  sh.dev = nullptr;
  return sh;
}

__global__ void k_cdf_shape(const uint64_t* __restrict__ x, uint32_t s, int lbits, CdfShape* out) {
  if (threadIdx.x == 0) *out = make_shape(x[0], x[s - 1], lbits);
}

unsigned grid_for(uint32_t n, int threads) {
  uint32_t b = (n + threads - 1) / threads;
  return b < 1 ? 1 : (b > 1184 ? 1184 : b);
}

}  // namespace

CdfShape cdf_shape(uint64_t kmin, uint64_t kmax, int lbits) { return make_shape(kmin, kmax, lbits); }

CdfShape cdf_shape_ref(const CdfShape* dev, int lbits) {
  CdfShape sh{};
  sh.lbits = lbits;
  sh.dev = dev;
  return sh;
}

cudaError_t cdf_shape_device(const uint64_t* x, uint32_t s, int lbits, CdfShape* out, cudaStream_t st) {
  k_cdf_shape<<<1, 32, 0, st>>>(x, s, lbits, out);
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t cdf_forward(const uint64_t* x, uint32_t s, const CdfShape& sh, const float* y, float* pred, float* loss,
                        cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(loss, 0, sizeof(float), st);
  if (e != cudaSuccess) return e;
  k_cdf_forward<<<grid_for(s, 256), 256, 0, st>>>(x, s, sh, y, pred, loss);
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t cdf_backward(const uint64_t* x, uint32_t s, const CdfShape& sh, const float* y, float* grad,
                         cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(grad, 0, sizeof(float) * ((1u << sh.lbits) + 1), st);
  if (e != cudaSuccess) return e;
  k_cdf_backward<<<grid_for(s, 256), 256, 0, st>>>(x, s, sh, y, grad);
  note_launches(1);
  return cudaGetLastError();
}

// Statistics T, b of the sample into w.h (diag), w.off, w.grad (b).
static cudaError_t cdf_stats(const uint64_t* x, uint32_t s, const CdfShape& sh, CdfWork& w, cudaStream_t st) {
  const int nk = (1 << sh.lbits) + 1;
  cudaError_t e;
  if ((e = cudaMemsetAsync(w.h, 0, sizeof(float) * nk, st)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(w.off, 0, sizeof(float) * nk, st)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(w.grad, 0, sizeof(float) * nk, st)) != cudaSuccess) return e;
  k_cdf_stats<<<grid_for(s, 256), 256, 0, st>>>(x, s, sh, w.h, w.off, w.grad);
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t cdf_train(const uint64_t* x, uint32_t s, const CdfShape& sh, int epochs, float lr, CdfWork& w,
                      cudaStream_t st) {
  const int nk = (1 << sh.lbits) + 1;
  if (nk > 8 * 1024 + 1) return cudaErrorInvalidValue;
  cudaError_t e;
  k_cdf_init<<<grid_for(nk, 256), 256, 0, st>>>(x, s, sh, w.y);
  note_launches(1);
  if ((e = cdf_stats(x, s, sh, w, st)) != cudaSuccess) return e;
  if (epochs > 0) {
    k_cdf_epochs<<<1, 1024, sizeof(float) * nk, st>>>(w.y, w.h, w.off, w.grad, nk, epochs, lr);
    note_launches(1);
  }
  if (w.loss && (e = cdf_forward(x, s, sh, w.y, nullptr, w.loss, st)) != cudaSuccess) return e;
  k_cdf_project<<<1, 1024, 0, st>>>(w.y, nk, w.knots);
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t cdf_train_gradient(const uint64_t* x, uint32_t s, const CdfShape& sh, const float* y, float* grad,
                               CdfWork& w, cudaStream_t st) {
  const int nk = (1 << sh.lbits) + 1;
  cudaError_t e;
  if ((e = cdf_stats(x, s, sh, w, st)) != cudaSuccess) return e;
  k_cdf_stat_grad<<<grid_for(nk, 256), 256, 0, st>>>(y, w.h, w.off, w.grad, nk, grad);
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t cdf_splitters(const uint64_t* x, uint32_t s, const CdfShape& sh, int nbuckets, const float2* knots,
                          uint64_t* S, cudaStream_t st) {
  const int nsplit = nbuckets - 1;
  if (nsplit <= 0) return cudaSuccess;
  k_cdf_splitters<<<grid_for(nsplit, 128), 128, 0, st>>>(sh, nbuckets, knots, S);
  k_cdf_heavy<<<grid_for(s, 256), 256, 0, st>>>(x, s, nbuckets, S);
  k_cummax_u64<<<1, 1024, 0, st>>>(S, nsplit);
  note_launches(3);
  return cudaGetLastError();
}

cudaError_t cdf_windows(const CdfShape& sh, int nbuckets, const float2* knots, const uint64_t* S, uint32_t* win,
                        uint32_t* tmp_lo, uint32_t* tmp_hi, uint32_t* widest, cudaStream_t st) {
  const int nleaf = 1 << sh.lbits;
  cudaError_t e;
  if ((e = cudaMemsetAsync(tmp_lo, 0, sizeof(uint32_t) * nleaf, st)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(tmp_hi, 0, sizeof(uint32_t) * nleaf, st)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(widest, 0, sizeof(uint32_t), st)) != cudaSuccess) return e;
  k_cdf_windows<<<grid_for(nbuckets + nleaf, 128), 128, 0, st>>>(sh, nbuckets, knots, S, tmp_lo, tmp_hi);
  k_pack_windows<<<grid_for(nleaf, 256), 256, 0, st>>>(tmp_lo, tmp_hi, nleaf, win, widest);
  note_launches(2);
  return cudaGetLastError();
}

cudaError_t refit_knots(const CdfShape& sh, int nbuckets, const uint64_t* S, float2* knots, const uint32_t* only_if,
                        cudaStream_t st) {
  const int nleaf = 1 << sh.lbits;
  if (nbuckets < 2) return cudaSuccess;
  k_refit_knots<<<grid_for(nleaf, 256), 256, 0, st>>>(sh, nbuckets, S, knots, only_if);
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t quantile_splitters(const uint64_t* x, uint32_t s, int nsplit, uint64_t* S, const uint32_t* only_if,
                               cudaStream_t st) {
  if (nsplit <= 0) return cudaSuccess;
  k_quantile_splitters<<<grid_for(nsplit, 256), 256, 0, st>>>(x, s, nsplit, S, only_if);
  note_launches(1);
  return cudaGetLastError();
}

cudaError_t vet_splitters(const uint64_t* x, uint32_t s, const uint64_t* S, int nbuckets, uint32_t* counts,
                            uint32_t* flags, cudaStream_t st) {
  cudaError_t e;
  if ((e = cudaMemsetAsync(counts, 0, sizeof(uint32_t) * nbuckets, st)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(flags, 0, sizeof(uint32_t), st)) != cudaSuccess) return e;
  // a bucket may hold up to 2.5x its share of the sample before the plain
  // splitters take over
  const uint32_t limit = (uint32_t)(2.5 * (double)s / (double)nbuckets) + 8;
  k_vet_count<<<grid_for(s, 256), 256, 0, st>>>(x, s, S, nbuckets, counts, flags);
  k_vet_max<<<grid_for(nbuckets, 256), 256, 0, st>>>(counts, nbuckets, limit, flags);
  note_launches(2);
  return cudaGetLastError();
}

}  // namespace gb
