// cdf_api.h -- host entry points of the learned CDF model (cdf.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace gb {

struct CdfShape {
  uint64_t kmin;  // key of leaf 0's left edge
  int lshift;     // leaf = (key - kmin) >> lshift
  int lbits;      // 1 << lbits leaves, (1 << lbits) + 1 knots
  // When set, kmin and lshift are read from this device copy at kernel start
  // (computed on the device from the sorted sample, so the pipeline never
  // waits for the host); lbits must match it.
  const CdfShape* dev;
};

struct CdfWork {   // device buffers of one training run
  float* y;        // knots, (1 << lbits) + 1
  float* grad;     // same size: b of the fit's statistics (dLoss/dy = T y - b)
  float* h;        // same size: diagonal of T (the Gauss-Newton curvature)
  float* off;      // same size: off-diagonal of T
  float2* knots;   // 1 << lbits pairs (y_j, y_{j+1}) after projection
  float* loss;     // 1 float (may be null)
};

CdfShape cdf_shape(uint64_t kmin, uint64_t kmax, int lbits);
// The shape of a sorted sample x[0..s) computed on the device into *out, and
// a host-side CdfShape that refers to it.
cudaError_t cdf_shape_device(const uint64_t* x, uint32_t s, int lbits, CdfShape* out, cudaStream_t st);
CdfShape cdf_shape_ref(const CdfShape* dev, int lbits);
cudaError_t cdf_forward(const uint64_t* x, uint32_t s, const CdfShape& sh, const float* y, float* pred,
                        float* loss, cudaStream_t st);
cudaError_t cdf_backward(const uint64_t* x, uint32_t s, const CdfShape& sh, const float* y, float* grad,
                         cudaStream_t st);
cudaError_t cdf_train(const uint64_t* x, uint32_t s, const CdfShape& sh, int epochs, float lr, CdfWork& w,
                      cudaStream_t st);
// The training's gradient at knots y (device, (1 << lbits) + 1 floats) into
// grad: T y - b from one statistics pass over x (uses w's h, off, grad).
cudaError_t cdf_train_gradient(const uint64_t* x, uint32_t s, const CdfShape& sh, const float* y, float* grad,
                               CdfWork& w, cudaStream_t st);
cudaError_t cdf_splitters(const uint64_t* x, uint32_t s, const CdfShape& sh, int nbuckets,
                          const float2* knots, uint64_t* S, cudaStream_t st);
cudaError_t cdf_windows(const CdfShape& sh, int nbuckets, const float2* knots, const uint64_t* S,
                        uint32_t* win, uint32_t* tmp_lo, uint32_t* tmp_hi, uint32_t* widest,
                        cudaStream_t st);

// Splitters read directly from the sorted sample at the bisection's targets
// (only when *only_if != 0, if only_if is given).
cudaError_t quantile_splitters(const uint64_t* x, uint32_t s, int nsplit, uint64_t* S, const uint32_t* only_if,
                               cudaStream_t st);
// Knots of every leaf set from the splitters S instead of the training (only
// when *only_if != 0): the model then predicts, at each leaf's first and last
// key, the true bucket, and in between no more splitters away than the leaf
// holds.  Used when the sample quantiles replaced the model's splitters,
// which the trained knots do not predict.
cudaError_t refit_knots(const CdfShape& sh, int nbuckets, const uint64_t* S, float2* knots, const uint32_t* only_if,
                        cudaStream_t st);
// Rejects (flags[0] != 0) a splitter set that leaves a heavy sample key out
// of a single-key bucket or puts more than 2.5x its share in any bucket.
cudaError_t vet_splitters(const uint64_t* x, uint32_t s, const uint64_t* S, int nbuckets, uint32_t* counts,
                            uint32_t* flags, cudaStream_t st);

}  // namespace gb
