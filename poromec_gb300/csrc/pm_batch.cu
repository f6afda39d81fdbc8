// pm_batch.cu -- independent diagonal-PCG solves of a batch of meshes held
// as one union mesh (a block-diagonal operator).
//
// Each instance keeps its own PCG scalars (pcg, Iters.f:299-595), stopping
// test and iteration count, exactly as if it were solved alone; only the
// launches are shared.  The per-instance dot products are segmented
// reductions over the instance's contiguous equation range (the layout in
// BatchView), summed in block order.  An instance that has converged is
// marked done: the SpMV skips its nodes and the vector kernels return at
// once for its blocks, so a batch of uneven meshes costs what its
// unconverged instances need.
#include <cuda_runtime.h>

#include "pm_krylov.h"
#include "pm_reduce.h"

namespace pm {
namespace {

// The block's instance and equation range [e0, e1).
__device__ __forceinline__ int seg_range(const BatchView& B, int& e0, int& e1) {
  const int inst = B.blk_inst[blockIdx.x];
  const int k = (int)blockIdx.x - B.blk_ptr[inst];
  e0 = B.eq_ptr[inst] + k * B.chunk;
  e1 = min(e0 + B.chunk, B.eq_ptr[inst + 1]);
  return inst;
}

// Segmented sum of up to two values; true in the last block of the instance,
// with tot[] valid in its thread 0.
template <int NV>
__device__ bool seg_reduce(const BatchView& B, int inst, const double (&v)[NV],
                           double (&tot)[NV]) {
  __shared__ double sh[32];
  __shared__ bool last;
  double bs[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) bs[k] = block_sum(v[k], sh);
  const int b0 = B.blk_ptr[inst], b1 = B.blk_ptr[inst + 1];
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) B.partial[(size_t)k * B.nblk + blockIdx.x] = bs[k];
    __threadfence();
    const unsigned t = atomicAdd(&B.counter[inst], 1u);
    last = (t == (unsigned)(b1 - b0 - 1));
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    double s = 0.0;
    for (int i = b0 + threadIdx.x; i < b1; i += blockDim.x)
      s += __ldcg(&B.partial[(size_t)k * B.nblk + i]);
    tot[k] = block_sum(s, sh);
  }
  if (threadIdx.x == 0) B.counter[inst] = 0u;
  return true;
}

__device__ __forceinline__ void pair_store(double v, float2* pr, int i) {
  pr[i] = split_pair(v);
}

// x = 0, r = b, z = m r, p = z, d = (r, z); conv = tol sqrt|d| (pcg's test)
// or conv_abs[inst] (a refinement sweep aims at the first sweep's target).
// Instances outside the sweep are marked done by their first block.
__global__ void __launch_bounds__(256)
    k_bpcg_init(BatchView B, const double* __restrict__ b, const double* __restrict__ m,
                double* __restrict__ r, double* __restrict__ z, double* __restrict__ p,
                double* __restrict__ x, float2* __restrict__ pair, double tol,
                const double* __restrict__ conv_abs, const int* __restrict__ insweep,
                int maxit) {
  int e0, e1;
  const int inst = seg_range(B, e0, e1);
  if (insweep && !insweep[inst]) {
    if ((int)blockIdx.x == B.blk_ptr[inst] && threadIdx.x == 0) B.done[inst] = 1;
    return;
  }
  double acc = 0.0;
  for (int i = e0 + threadIdx.x; i < e1; i += blockDim.x) {
    const double bi = b[i], zi = bi * m[i];
    x[i] = 0.0;
    r[i] = bi;
    z[i] = zi;
    p[i] = zi;
    if (pair) pair_store(zi, pair, i);
    acc += bi * zi;
  }
  double in[1] = {acc}, tot[1];
  if (seg_reduce<1>(B, inst, in, tot) && threadIdx.x == 0) {
    BatchScalars& S = B.bs[inst];
    S.d = tot[0];
    S.bmb = tot[0];
    S.conv = conv_abs ? conv_abs[inst] : tol * sqrt(fabs(tot[0]));
    S.iter = 0;
    S.maxit = maxit;
    if (tot[0] == 0.0) {  // b = 0 (or no equations): x = 0 is the solution
      S.conv_flag = 1;
      B.done[inst] = 1;
    } else {
      S.conv_flag = 0;
      B.done[inst] = 0;
      atomicAdd(B.nactive, 1);
    }
  }
}

// alpha = d / (p, q)
__global__ void __launch_bounds__(256)
    k_bpcg_alpha(BatchView B, const double* __restrict__ p, const double* __restrict__ q) {
  int e0, e1;
  const int inst = seg_range(B, e0, e1);
  if (B.done[inst]) return;
  double acc = 0.0;
  for (int i = e0 + threadIdx.x; i < e1; i += blockDim.x) acc += p[i] * q[i];
  double in[1] = {acc}, tot[1];
  if (seg_reduce<1>(B, inst, in, tot) && threadIdx.x == 0) {
    BatchScalars& S = B.bs[inst];
    S.pq = tot[0];
    S.alpha = S.d / tot[0];
  }
}

// x += alpha p, r -= alpha q, z = m r, di = (r, z), beta = di / d, d = di;
// converged when sqrt|d| < conv (Iters.f:446-497)
__global__ void __launch_bounds__(256)
    k_bpcg_update(BatchView B, double* __restrict__ x, const double* __restrict__ p,
                  double* __restrict__ r, const double* __restrict__ q,
                  const double* __restrict__ m, double* __restrict__ z) {
  int e0, e1;
  const int inst = seg_range(B, e0, e1);
  if (B.done[inst]) return;
  const double alpha = B.bs[inst].alpha;
  double acc = 0.0;
  for (int i = e0 + threadIdx.x; i < e1; i += blockDim.x) {
    x[i] = x[i] + alpha * p[i];
    const double ri = r[i] - alpha * q[i];
    r[i] = ri;
    const double zi = ri * m[i];
    z[i] = zi;
    acc += ri * zi;
  }
  double in[1] = {acc}, tot[1];
  if (seg_reduce<1>(B, inst, in, tot) && threadIdx.x == 0) {
    BatchScalars& S = B.bs[inst];
    const double di = tot[0];
    S.beta = di / S.d;
    S.d = di;
    S.iter += 1;
    if (sqrt(fabs(di)) < S.conv) S.conv_flag = 1;
    else if (!isfinite(di)) S.conv_flag = 3;
    else if (S.iter >= S.maxit) S.conv_flag = 2;
    if (S.conv_flag) {
      B.done[inst] = 1;
      atomicSub(B.nactive, 1);
    }
  }
}

// p = z + beta p (and its FP32 pair for the compensated operator)
__global__ void __launch_bounds__(256)
    k_bpcg_dir(BatchView B, const double* __restrict__ z, double* __restrict__ p,
               float2* __restrict__ pair) {
  int e0, e1;
  const int inst = seg_range(B, e0, e1);
  if (B.done[inst]) return;
  const double beta = B.bs[inst].beta;
  for (int i = e0 + threadIdx.x; i < e1; i += blockDim.x) {
    const double pi = z[i] + beta * p[i];
    p[i] = pi;
    if (pair) pair_store(pi, pair, i);
  }
}

// per instance: sums of squares of the displacement and pressure entries
__global__ void __launch_bounds__(256)
    k_bresnorms(BatchView B, const double* __restrict__ b, const int32_t* __restrict__ kind,
                double* __restrict__ out) {
  int e0, e1;
  const int inst = seg_range(B, e0, e1);
  double au = 0.0, ap = 0.0;
  for (int i = e0 + threadIdx.x; i < e1; i += blockDim.x) {
    const double bi = b[i];
    if (kind[i]) ap += bi * bi;
    else au += bi * bi;
  }
  double in[2] = {au, ap}, tot[2];
  if (seg_reduce<2>(B, inst, in, tot) && threadIdx.x == 0) {
    out[2 * inst] = tot[0];
    out[2 * inst + 1] = tot[1];
  }
}

// r = b - q, out[inst] = (r, m r): the FP64 outer residual of the refinement
__global__ void __launch_bounds__(256)
    k_btrue_residual(BatchView B, const double* __restrict__ b, const double* __restrict__ q,
                     const double* __restrict__ m, double* __restrict__ r,
                     double* __restrict__ out) {
  int e0, e1;
  const int inst = seg_range(B, e0, e1);
  double acc = 0.0;
  for (int i = e0 + threadIdx.x; i < e1; i += blockDim.x) {
    const double ri = b[i] - q[i];
    r[i] = ri;
    acc += ri * ri * m[i];
  }
  double in[1] = {acc}, tot[1];
  if (seg_reduce<1>(B, inst, in, tot) && threadIdx.x == 0) out[inst] = tot[0];
}

__global__ void __launch_bounds__(256)
    k_baxpy(BatchView B, double* __restrict__ y, const double* __restrict__ x,
            const int* __restrict__ mask) {
  int e0, e1;
  const int inst = seg_range(B, e0, e1);
  if (mask && !mask[inst]) return;
  for (int i = e0 + threadIdx.x; i < e1; i += blockDim.x) y[i] += x[i];
}

}  // namespace

cudaError_t bpcg_init(const BatchView& B, const double* b, const double* m, KrylovVecs& V,
                      float2* pair, double tol, const double* conv_abs, const int* insweep,
                      int maxit, cudaStream_t s) {
  k_bpcg_init<<<B.nblk, 256, 0, s>>>(B, b, m, V.r, V.z, V.p, V.x, pair, tol, conv_abs, insweep,
                                      maxit);
  return cudaGetLastError();
}

cudaError_t bpcg_iteration(const PanelView& P, const double* val64, const CompVals* C,
                           const BatchView& B, const double* m, KrylovVecs& V, float2* pair,
                           cudaStream_t s) {
  cudaError_t e = C ? spmvc(P, *C, pair, V.q, s)
                    : spmv(P, val64, V.p, V.q, 0, nullptr, nullptr, nullptr, s);
  if (e != cudaSuccess) return e;
  k_bpcg_alpha<<<B.nblk, 256, 0, s>>>(B, V.p, V.q);
  k_bpcg_update<<<B.nblk, 256, 0, s>>>(B, V.x, V.p, V.r, V.q, m, V.z);
  k_bpcg_dir<<<B.nblk, 256, 0, s>>>(B, V.z, V.p, C ? pair : nullptr);
  return cudaGetLastError();
}

cudaError_t bresnorms(const BatchView& B, const double* b, const int32_t* kind, double* out,
                      cudaStream_t s) {
  k_bresnorms<<<B.nblk, 256, 0, s>>>(B, b, kind, out);
  return cudaGetLastError();
}

cudaError_t btrue_residual(const BatchView& B, const double* b, const double* q,
                           const double* m, double* r, double* out, cudaStream_t s) {
  k_btrue_residual<<<B.nblk, 256, 0, s>>>(B, b, q, m, r, out);
  return cudaGetLastError();
}

cudaError_t baxpy(const BatchView& B, double* y, const double* x, const int* mask,
                  cudaStream_t s) {
  k_baxpy<<<B.nblk, 256, 0, s>>>(B, y, x, mask);
  return cudaGetLastError();
}

}  // namespace pm
