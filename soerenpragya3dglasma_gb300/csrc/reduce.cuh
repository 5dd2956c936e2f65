// reduce.cuh -- deterministic FP64 block reductions shared by the measurement kernels.
#pragma once

#include <cuda_runtime.h>

namespace glasma {
namespace red {

constexpr int kThreads = 256;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ double warp_min(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_down_sync(0xffffffffu, v, o));
  return v;
}

// op[k]: 0 sum, 1 max, 2 min.  Thread 0 writes out[k].  blockDim.x == kThreads.
template <int K>
__device__ __forceinline__ void block_reduce_store(double (&v)[K], const int (&op)[K], double* out) {
  __shared__ double sh[K][kThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < K; k++) {
    const double r = op[k] == 1 ? warp_max(v[k]) : (op[k] == 2 ? warp_min(v[k]) : warp_sum(v[k]));
    if (lane == 0) sh[k][warp] = r;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
#pragma unroll
    for (int k = 0; k < K; k++) {
      const double neutral = op[k] == 1 ? -1.0e300 : (op[k] == 2 ? 1.0e300 : 0.0);
      double r = (lane < kThreads / 32) ? sh[k][lane] : neutral;
      r = op[k] == 1 ? warp_max(r) : (op[k] == 2 ? warp_min(r) : warp_sum(r));
      if (lane == 0) out[k] = r;
    }
  }
  __syncthreads();
}

// out[k] = reduction over b of partials[b*K + k], fixed order; launch with one block of kThreads.
template <int K>
__global__ void finish_kernel(const double* __restrict__ partials, int nblocks, int op_code, double* out) {
  int op[K];
  double v[K];
#pragma unroll
  for (int k = 0; k < K; k++) {
    op[k] = (op_code >> (2 * k)) & 3;
    v[k] = 0.0;
  }
  bool first = true;
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
#pragma unroll
    for (int k = 0; k < K; k++) {
      const double x = partials[(long long)b * K + k];
      if (first)
        v[k] = x;
      else
        v[k] = op[k] == 1 ? fmax(v[k], x) : (op[k] == 2 ? fmin(v[k], x) : v[k] + x);
    }
    first = false;
  }
  if (first) {  // this thread saw no block: neutral elements
#pragma unroll
    for (int k = 0; k < K; k++) v[k] = op[k] == 2 ? 1.0e300 : (op[k] == 1 ? -1.0e300 : 0.0);
  }
  block_reduce_store<K>(v, op, out);
}

}  // namespace red
}  // namespace glasma
