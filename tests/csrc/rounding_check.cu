// Exhaustive check of the engine's correctly rounded reciprocal and square root
// (jdem_device.cuh) against IEEE division and sqrtf, over every positive
// normal float, and of inv_norm against where(d == 0, 0, 1 / sqrt(max(d, 1e-16)))
// over every non-negative finite float.  Prints the three mismatch counts and
// the smallest and largest float (as bits) where the square roots differ.
#include <cstdio>
#include "jdem_device.cuh"

using namespace jdem;

__global__ void k_check(unsigned long long* bad, unsigned int* sqrt_range) {
  unsigned long long n_rcp = 0, n_sqrt = 0, n_inv = 0;
  for (unsigned long long b = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; b <= 0x7F7FFFFFull;
       b += (unsigned long long)gridDim.x * blockDim.x) {
    const float x = __uint_as_float((unsigned int)b);
    const float ref_inv = x == 0.0f ? 0.0f : 1.0f / sqrtf(fmaxf(x, 1e-16f));
    n_inv += __float_as_uint(inv_norm(x)) != __float_as_uint(ref_inv);
    if (b < 0x00800000ull) continue;  // zero and subnormals: inv_norm only
    if (__float_as_uint(sqrt_rn_above_1e16(x)) != __float_as_uint(sqrtf(x))) {
      ++n_sqrt;
      atomicMin(&sqrt_range[0], (unsigned int)b);
      atomicMax(&sqrt_range[1], (unsigned int)b);
    }
    const float q = 1.0f / x;
    if (q >= 1.17549435e-38f) n_rcp += __float_as_uint(rcp_rn_normal(x)) != __float_as_uint(q);
  }
  atomicAdd(&bad[0], n_rcp);
  atomicAdd(&bad[1], n_sqrt);
  atomicAdd(&bad[2], n_inv);
}

int main() {
  unsigned long long* d = nullptr;
  unsigned int* r = nullptr;
  unsigned long long h[3] = {~0ull, ~0ull, ~0ull};
  unsigned int hr[2] = {0xFFFFFFFFu, 0u};
  if (cudaMalloc(&d, sizeof(h)) != cudaSuccess || cudaMemset(d, 0, sizeof(h)) != cudaSuccess) return 2;
  if (cudaMalloc(&r, sizeof(hr)) != cudaSuccess || cudaMemcpy(r, hr, sizeof(hr), cudaMemcpyHostToDevice) != cudaSuccess)
    return 2;
  k_check<<<152 * 8, 256>>>(d, r);
  if (cudaDeviceSynchronize() != cudaSuccess || cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost) != cudaSuccess ||
      cudaMemcpy(hr, r, sizeof(hr), cudaMemcpyDeviceToHost) != cudaSuccess)
    return 3;
  printf("rcp %llu sqrt %llu inv_norm %llu sqrt_lo %u sqrt_hi %u\n", h[0], h[1], h[2], hr[0], hr[1]);
  cudaFree(d);
  cudaFree(r);
  return 0;
}
