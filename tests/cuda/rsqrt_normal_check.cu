// rsqrt_normal (csrc/common.cuh) against CUDA's rsqrtf on every positive
// normal float: prints the number of bit patterns whose results differ.
#include <cstdint>
#include <cstdio>

#include "../../galactic-tides_gb300/csrc/common.cuh"

__global__ void k_compare(uint32_t lo, uint32_t hi, unsigned long long *bad, uint32_t *first) {
  for (uint64_t b = lo + blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; b < hi;
       b += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
    const float x = __uint_as_float(static_cast<uint32_t>(b));
    if (__float_as_uint(rsqrtf(x)) != __float_as_uint(gtc::rsqrt_normal(x))) {
      atomicAdd(bad, 1ull);
      atomicMin(first, static_cast<uint32_t>(b));
    }
  }
}

int main() {
  unsigned long long *bad = nullptr;
  uint32_t *first = nullptr;
  if (cudaMalloc(&bad, sizeof *bad) != cudaSuccess || cudaMalloc(&first, sizeof *first) != cudaSuccess)
    return 2;
  cudaMemset(bad, 0, sizeof *bad);
  cudaMemset(first, 0xff, sizeof *first);
  const uint32_t lo = 0x00800000u, hi = 0x7f800000u;  // smallest normal .. FLT_MAX
  k_compare<<<1216, 256>>>(lo, hi, bad, first);
  const cudaError_t e = cudaDeviceSynchronize();
  unsigned long long nbad = 0;
  uint32_t f = 0;
  cudaMemcpy(&nbad, bad, sizeof nbad, cudaMemcpyDeviceToHost);
  cudaMemcpy(&f, first, sizeof f, cudaMemcpyDeviceToHost);
  std::printf("checked %u mismatches %llu first 0x%08x status %s\n", hi - lo, nbad, f,
              cudaGetErrorString(e));
  cudaFree(bad);
  cudaFree(first);
  return e == cudaSuccess ? 0 : 1;
}
