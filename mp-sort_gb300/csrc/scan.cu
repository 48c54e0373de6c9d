// scan.cu -- exclusive prefix sum of uint32 counts (reduce, then scan).
//
// Used for the (bucket x chunk) count matrices of the histogram sort and the
// (digit x chunk) matrices of the LSD passes: the device counterpart of the
// reference's count reductions (mpsort-omp.c:110-121) and displacement
// arithmetic (mpsort-mpi.c:483-510).
#include <atomic>

#include "common.cuh"
#include "kernels.h"

namespace gb {

static std::atomic<unsigned long long> g_launches{0};
void note_launches(int k) { g_launches.fetch_add((unsigned long long)k, std::memory_order_relaxed); }
unsigned long long launch_count() { return g_launches.load(std::memory_order_relaxed); }

namespace {

constexpr int kSeg = 4096;  // elements per segment (8 per thread)
constexpr int kPer = kSeg / kThreads;

__global__ void __launch_bounds__(kThreads) k_segment_sums(const uint32_t* __restrict__ in, size_t n,
                                                            uint32_t* __restrict__ sums) {
  __shared__ uint32_t tmp[kWarps];
  size_t base = (size_t)blockIdx.x * kSeg;
  uint32_t s = 0;
#pragma unroll
  for (int i = 0; i < kPer; ++i) {
    size_t j = base + (size_t)i * kThreads + threadIdx.x;
    if (j < n) s += in[j];
  }
  uint32_t total;
  block_exclusive_scan<uint32_t>(s, tmp, &total);
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// Scans the segment sums in place (one block; nseg <= kSeg).
__global__ void __launch_bounds__(kThreads) k_scan_sums(uint32_t* sums, int nseg) {
  __shared__ uint32_t tmp[kWarps];
  uint32_t v[kPer];
  uint32_t s = 0;
  const int base = threadIdx.x * kPer;
#pragma unroll
  for (int i = 0; i < kPer; ++i) {
    v[i] = (base + i < nseg) ? sums[base + i] : 0u;
    s += v[i];
  }
  uint32_t pre = block_exclusive_scan<uint32_t>(s, tmp, nullptr);
#pragma unroll
  for (int i = 0; i < kPer; ++i) {
    if (base + i < nseg) sums[base + i] = pre;
    pre += v[i];
  }
}

__global__ void __launch_bounds__(kThreads) k_segment_scan(const uint32_t* in, uint32_t* out, size_t n,
                                                            const uint32_t* __restrict__ seg_base) {
  __shared__ uint32_t tmp[kWarps];
  size_t base = (size_t)blockIdx.x * kSeg + (size_t)threadIdx.x * kPer;
  uint32_t v[kPer];
  uint32_t s = 0;
#pragma unroll
  for (int i = 0; i < kPer; ++i) {
    v[i] = (base + i < n) ? in[base + i] : 0u;
    s += v[i];
  }
  uint32_t pre = block_exclusive_scan<uint32_t>(s, tmp, nullptr) + seg_base[blockIdx.x];
#pragma unroll
  for (int i = 0; i < kPer; ++i) {
    if (base + i < n) out[base + i] = pre;
    pre += v[i];
  }
}

}  // namespace

// Words of scratch for a scan of n elements: the segment sums, plus (above
// kSeg segments) the scratch of scanning those sums the same way.
size_t scan_tmp_words(size_t n) {
  const size_t nseg = (n + kSeg - 1) / kSeg;
  return nseg <= (size_t)kSeg ? nseg + 1 : nseg + scan_tmp_words(nseg);
}

// Exclusive scan of n counts (out may alias in): segment sums, a scan of the
// sums (one block, or the same scan again over the sums when there are more
// than kSeg of them), then each segment scanned from its base.
cudaError_t exclusive_scan_u32(const uint32_t* in, uint32_t* out, size_t n, uint32_t* tmp,
                               cudaStream_t stream) {
  if (n == 0) return cudaSuccess;
  const size_t nseg = (n + kSeg - 1) / kSeg;
  if (nseg > (size_t)0x7fffffff) return cudaErrorInvalidValue;
  k_segment_sums<<<(unsigned)nseg, kThreads, 0, stream>>>(in, n, tmp);
  note_launches(2);
  if (nseg <= (size_t)kSeg) {
    k_scan_sums<<<1, kThreads, 0, stream>>>(tmp, (int)nseg);
    note_launches(1);
  } else {
    const cudaError_t e = exclusive_scan_u32(tmp, tmp, nseg, tmp + nseg, stream);
    if (e != cudaSuccess) return e;
  }
  k_segment_scan<<<(unsigned)nseg, kThreads, 0, stream>>>(in, out, n, tmp);
  return cudaGetLastError();
}

}  // namespace gb
