// pm_reduce.h -- deterministic reductions shared by the Krylov kernels.
//
// A grid reduction writes one partial per block; the last block to arrive
// (atomic ticket) sums the partials in block order, so the result does not
// depend on the order in which blocks run.
#pragma once
#include <cuda_runtime.h>

namespace pm {

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block sum of v (blockDim multiple of 32, <= 1024); result valid in thread 0.
static __device__ double block_sum(double v, double* sh) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  if (wid == 0) {
    v = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : 0.0;
    v = warp_sum(v);
  }
  return v;
}

// Grid reduction of up to NV values: each block writes its partial sums; the
// last block to arrive sums all partials in block order.  Returns true in the
// last block; tot[] valid in its thread 0.  partial holds NV * gridDim.x
// doubles; counter is zero on entry and is reset by the last block.
template <int NV>
static __device__ bool grid_reduce(const double (&v)[NV], double* partial, unsigned* counter,
                                   double (&tot)[NV]) {
  __shared__ double sh[32];
  __shared__ bool last;
  double bs[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) bs[k] = block_sum(v[k], sh);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) partial[(size_t)k * gridDim.x + blockIdx.x] = bs[k];
    __threadfence();
    const unsigned t = atomicAdd(counter, 1u);
    last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    double s = 0.0;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x)
      s += __ldcg(&partial[(size_t)k * gridDim.x + i]);
    tot[k] = block_sum(s, sh);
  }
  if (threadIdx.x == 0) *counter = 0u;
  return true;
}

}  // namespace pm
