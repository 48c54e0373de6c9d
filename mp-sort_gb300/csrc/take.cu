// take.cu -- out[i] = source[index[i]] for records of any size (device).
//
// The GB300 form of mpsort.take / mpsort.permute for one process
// (mpsort/__init__.py:116-204 reaches the same result over MPI ranks with
// two or three distributed sorts; with every record in one GPU's memory a
// gather reads each requested record once and writes the output in order).
// Indices outside [0, nsource) are not read: the call reports them.
#include "common.cuh"
#include "kernels.h"

namespace gb {

namespace {

template <typename V>
__global__ void k_take(const uint8_t* __restrict__ src, uint64_t nsrc, uint32_t elsize,
                       const int64_t* __restrict__ index, uint64_t nidx, uint8_t* __restrict__ out,
                       unsigned long long* __restrict__ bad) {
  const uint32_t vpr = elsize / sizeof(V);
  const uint64_t total = nidx * vpr;
  for (uint64_t f = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; f < total;
       f += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t i = f / vpr;
    const uint32_t v = (uint32_t)(f % vpr);
    const int64_t j = __ldg(index + i);
    V* dst = reinterpret_cast<V*>(out + i * elsize) + v;
    if (j < 0 || (uint64_t)j >= nsrc) {  // out of range: first bad position + 1, output left as is
      if (v == 0) atomicCAS(bad, 0ull, (unsigned long long)i + 1);
      continue;
    }
    *dst = reinterpret_cast<const V*>(src + (uint64_t)j * elsize)[v];
  }
}

}  // namespace

cudaError_t take_records(const void* src, uint64_t nsrc, uint32_t elsize, const int64_t* index, uint64_t nidx,
                         void* out, unsigned long long* bad, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(bad, 0, sizeof(unsigned long long), st);
  if (e != cudaSuccess || nidx == 0) return e;
  const uintptr_t a = (uintptr_t)src | (uintptr_t)out;
  const uint8_t* s8 = (const uint8_t*)src;
  uint8_t* o8 = (uint8_t*)out;
  auto blocks = [&](uint64_t work) {
    uint64_t b = (work + 255) / 256, cap = (uint64_t)num_sms() * 16;
    return (unsigned)(b < 1 ? 1 : (b > cap ? cap : b));
  };
  if (elsize % 16 == 0 && a % 16 == 0)
    k_take<uint4><<<blocks(nidx * (elsize / 16)), 256, 0, st>>>(s8, nsrc, elsize, index, nidx, o8, bad);
  else if (elsize % 8 == 0 && a % 8 == 0)
    k_take<uint2><<<blocks(nidx * (elsize / 8)), 256, 0, st>>>(s8, nsrc, elsize, index, nidx, o8, bad);
  else if (elsize % 4 == 0 && a % 4 == 0)
    k_take<uint32_t><<<blocks(nidx * (elsize / 4)), 256, 0, st>>>(s8, nsrc, elsize, index, nidx, o8, bad);
  else
    k_take<uint8_t><<<blocks(nidx * elsize), 256, 0, st>>>(s8, nsrc, elsize, index, nidx, o8, bad);
  note_launches(1);
  return cudaGetLastError();
}

}  // namespace gb
