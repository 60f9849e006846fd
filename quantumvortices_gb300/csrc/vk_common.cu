// vk_common.cu -- small kernels shared by both precisions.
#include "vk_kernels.cuh"

namespace vk {

// Fixed-order sum of per-CTA partials part[i*3 + j] -> out[j], j = 0..2.
// One block; each thread strides the partial list, then a fixed-shape tree.
__global__ void k_reduce_partials3(const double* __restrict__ part, int nblk, double* __restrict__ out) {
  __shared__ double sh[3][256];
  double a = 0.0, b = 0.0, c = 0.0;
  for (int i = threadIdx.x; i < nblk; i += blockDim.x) {
    a += part[3 * i + 0];
    b += part[3 * i + 1];
    c += part[3 * i + 2];
  }
  sh[0][threadIdx.x] = a;
  sh[1][threadIdx.x] = b;
  sh[2][threadIdx.x] = c;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) {
      sh[0][threadIdx.x] += sh[0][threadIdx.x + s];
      sh[1][threadIdx.x] += sh[1][threadIdx.x + s];
      sh[2][threadIdx.x] += sh[2][threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = sh[0][0];
    out[1] = sh[1][0];
    out[2] = sh[2][0];
  }
}

}  // namespace vk
