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

#include "../../include/poromec_gb300.h"
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
// With sweep (the device-driven step): b and pcg's test on sweep 0, b_refine
// and conv_abs on the later sweeps.
__global__ void __launch_bounds__(256)
    k_bpcg_init(BatchView B, const double* __restrict__ b, const double* __restrict__ m,
                double* __restrict__ r, double* __restrict__ z, double* __restrict__ p,
                double* __restrict__ x, float2* __restrict__ pair, double tol,
                const double* __restrict__ conv_abs, const int* __restrict__ insweep,
                int maxit, const double* __restrict__ b_refine, const int* __restrict__ sweep) {
  int e0, e1;
  const int inst = seg_range(B, e0, e1);
  if (insweep && !insweep[inst]) {
    if ((int)blockIdx.x == B.blk_ptr[inst] && threadIdx.x == 0) B.done[inst] = 1;
    return;
  }
  if (sweep) {
    const bool refine = *sweep > 0;
    if (refine) b = b_refine;
    else conv_abs = nullptr;
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
  // x, r and q streamed (evict-first): L2 keeps p (or its pair), m and z
  double acc = 0.0;
  for (int i = e0 + threadIdx.x; i < e1; i += blockDim.x) {
    __stcs(&x[i], __ldcs(&x[i]) + alpha * p[i]);
    const double ri = __ldcs(&r[i]) - alpha * __ldcs(&q[i]);
    __stcs(&r[i], ri);
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
    const double pi = __ldcs(&z[i]) + beta * p[i];
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

// ---- control kernels of the device-driven batch step ------------------------
// One block of kCtlThreads threads each, between the conditional nodes of the
// step's graph: they keep the host loop's per-instance bookkeeping in device
// memory and set the loop conditions.  Instance loops are strided, sums and
// minima are block reductions, so the decisions are the host loop's.
constexpr int kCtlThreads = 256;

__device__ int ctl_sum(int v, int* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  int t = 0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sh[w];
  return t;
}

__device__ int ctl_min(int v, int* sh) {
  for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  int t = v;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t = min(t, sh[w]);
  return t;
}

__device__ double ctl_max(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = v;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t = fmax(t, sh[w]);
  return t;
}

__global__ void __launch_bounds__(kCtlThreads) k_bs_begin(BatchCtl* c, BatchStepArrays A, int ni) {
  for (int i = threadIdx.x; i < ni; i += blockDim.x) {
    A.active[i] = 1;
    A.iters[i] = 0;
    A.nlit[i] = 0;
  }
  if (threadIdx.x == 0) *c = BatchCtl{};
  if (threadIdx.x == 0) c->it = 1;
}

// cal_residuo_pm (Residuo.f:39-276) per active instance at iteration c->it;
// the nonlinear loop goes on while an instance is left and no error is set.
__global__ void __launch_bounds__(kCtlThreads)
    k_bs_stop(BatchCtl* c, BatchStepArrays A, int ni, int stop_crit, double tol,
              cudaGraphConditionalHandle cond) {
  __shared__ int shi[32];
  __shared__ double shd[32];
  const int it = c->it;
  int left = 0;
  double rmax = 0.0;
  for (int i = threadIdx.x; i < ni; i += blockDim.x) {
    if (!A.active[i]) continue;
    bool done;
    if (stop_crit == 1) {
      const double res = sqrt(A.nr[2 * i] + A.nr[2 * i + 1]);
      if (it == 1) A.res0[i] = res;
      else if (it == 2) A.res0[i] = fmax(A.res0[i], res);
      rmax = fmax(rmax, res);
      done = A.res0[i] > 0.0 ? res / A.res0[i] < tol : true;
    } else {
      const double gresu = sqrt(A.nr[2 * i]), gresp = sqrt(A.nr[2 * i + 1]);
      if (it == 1) {
        A.resu0[i] = gresu;
        A.resp0[i] = gresp;
      } else if (it == 2) {
        A.resu0[i] = fmax(A.resu0[i], gresu);
        A.resp0[i] = fmax(A.resp0[i], gresu);  // as the reference
      }
      int istop = 0;
      if (gresu / A.resu0[i] < tol) istop += 1;
      if (gresp / A.resp0[i] < tol) istop += 1;
      done = istop == 2;
    }
    if (done) {
      A.active[i] = 0;
      A.nlit[i] = it;
    } else {
      ++left;
    }
  }
  left = ctl_sum(left, shi);
  rmax = ctl_max(rmax, shd);
  if (threadIdx.x == 0) {
    c->res_max = fmax(c->res_max, rmax);
    cudaGraphSetConditional(cond, (left > 0 && c->err == 0) ? 1u : 0u);
  }
}

// a solve of the active instances: sweep 0, no iterations yet (none after a
// zero diagonal)
__global__ void __launch_bounds__(kCtlThreads)
    k_bs_solve_start(BatchCtl* c, BatchStepArrays A, int ni, cudaGraphConditionalHandle cond) {
  for (int i = threadIdx.x; i < ni; i += blockDim.x) {
    A.insweep[i] = A.active[i];
    A.total[i] = 0;
  }
  if (threadIdx.x == 0) {
    c->sweeps = 0;
    if (c->zdiag && c->err == 0) c->err = PM_E_ZERO_DIAG;
    cudaGraphSetConditional(cond, c->err == 0 ? 1u : 0u);
  }
}

__global__ void k_bs_loop_start(const int* nactive, BatchCtl* c,
                                cudaGraphConditionalHandle cond) {
  if (threadIdx.x == 0) {
    c->trips = 0;
    cudaGraphSetConditional(cond, *nactive > 0 ? 1u : 0u);
  }
}

// after a trip of iters_per_trip iterations: go on while instances are
// active; every instance stops at maxit, so a trip count past it is an error
__global__ void k_bs_loop_next(const int* nactive, BatchCtl* c, int maxit, int iters_per_trip,
                               cudaGraphConditionalHandle cond) {
  if (threadIdx.x == 0) {
    const int t = ++c->trips;
    c->runs_pcg += 1;
    bool go = *nactive > 0;
    if (go && (long long)t * iters_per_trip > (long long)maxit + iters_per_trip) {
      if (c->err == 0) {
        c->err = PM_E_NOCONV;
        c->err_inst = -1;
      }
      go = false;
    }
    cudaGraphSetConditional(cond, go ? 1u : 0u);
  }
}

// the end of a sweep: iterations, the first failed instance (in index
// order), the first sweep's targets; without refinement the solve ends here
__global__ void __launch_bounds__(kCtlThreads)
    k_bs_sweep_end(BatchCtl* c, const BatchScalars* __restrict__ bs, BatchStepArrays A, int ni,
                   int comp, cudaGraphConditionalHandle cond) {
  __shared__ int shi[32];
  const int sw = c->sweeps;
  int bad = ni;
  for (int i = threadIdx.x; i < ni; i += blockDim.x) {
    if (!A.insweep[i]) continue;
    A.total[i] += bs[i].iter;
    if (bs[i].conv_flag == 3 || bs[i].conv_flag == 2) bad = min(bad, i);
    else if (sw == 0) A.conv0[i] = bs[i].conv;
  }
  bad = ctl_min(bad, shi);
  if (threadIdx.x == 0) {
    c->sweeps = sw + 1;
    c->runs_sweep += 1;
    if (bad < ni && c->err == 0) {
      c->err = PM_E_NOCONV;
      c->err_inst = bad;
      c->err_flag = bs[bad].conv_flag;
      c->err_iters = A.total[bad];
    }
    if (c->err != 0 || !comp) cudaGraphSetConditional(cond, 0u);
  }
}

// refinement: the instances whose FP64 residual (r, m r) = rn2 is still
// above the first sweep's target take another sweep, at most max_sweeps
__global__ void __launch_bounds__(kCtlThreads)
    k_bs_sweep_next(BatchCtl* c, BatchStepArrays A, int ni, int max_sweeps,
                    cudaGraphConditionalHandle cond) {
  __shared__ int shi[32];
  int again = 0;
  for (int i = threadIdx.x; i < ni; i += blockDim.x) {
    const int in = A.insweep[i] && !(sqrt(fabs(A.rn2[i])) < A.conv0[i]) && A.conv0[i] > 0.0;
    A.insweep[i] = in;
    again += in;
  }
  again = ctl_sum(again, shi);
  if (threadIdx.x == 0) {
    bool go = c->err == 0 && again > 0;
    if (go && c->sweeps >= max_sweeps) {
      c->err = PM_E_NOCONV;
      c->err_inst = -2;
      go = false;
    }
    cudaGraphSetConditional(cond, go ? 1u : 0u);
  }
}

// after a solve: per-instance iterations of the step, the solve's largest
__global__ void __launch_bounds__(kCtlThreads)
    k_bs_solve_end(BatchCtl* c, BatchStepArrays A, int ni, int comp) {
  __shared__ int shi[32];
  int mx = 0;
  for (int i = threadIdx.x; i < ni; i += blockDim.x) {
    if (A.active[i]) A.iters[i] += A.total[i];
    mx = max(mx, A.total[i]);
  }
  mx = -ctl_min(-mx, shi);
  if (threadIdx.x == 0) {
    c->iters_max = max(c->iters_max, mx);
    c->refine = comp ? c->sweeps : 0;
  }
}

// the nonlinear iteration count: an error past maxnlit
__global__ void k_bs_nl_next(BatchCtl* c, int maxnlit) {
  if (threadIdx.x == 0) {
    c->runs_nl += 1;
    if (c->err != 0) return;
    if (c->it >= maxnlit) c->err = PM_E_NLNOCONV;
    else c->it += 1;
  }
}

// the closing passes run when the step met its test without an error
__global__ void k_bs_finish(BatchCtl* c, const int* elem_err, cudaGraphConditionalHandle cond) {
  if (threadIdx.x == 0) {
    c->ok = c->err == 0 && c->zdiag == 0 && *elem_err == 0;
    cudaGraphSetConditional(cond, c->ok ? 1u : 0u);
  }
}

}  // namespace

cudaError_t bpcg_init(const BatchView& B, const double* b, const double* m, KrylovVecs& V,
                      float2* pair, double tol, const double* conv_abs, const int* insweep,
                      int maxit, cudaStream_t s) {
  k_bpcg_init<<<B.nblk, 256, 0, s>>>(B, b, m, V.r, V.z, V.p, V.x, pair, tol, conv_abs, insweep,
                                      maxit, nullptr, nullptr);
  return cudaGetLastError();
}

cudaError_t bpcg_init_sweep(const BatchView& B, const double* b, const double* b_refine,
                            const double* m, KrylovVecs& V, float2* pair, double tol,
                            const double* conv_abs, const int* insweep, int maxit,
                            const int* sweep, cudaStream_t s) {
  k_bpcg_init<<<B.nblk, 256, 0, s>>>(B, b, m, V.r, V.z, V.p, V.x, pair, tol, conv_abs, insweep,
                                      maxit, b_refine, sweep);
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

cudaError_t bs_begin(BatchCtl* c, const BatchStepArrays& A, int ni, cudaStream_t s) {
  k_bs_begin<<<1, kCtlThreads, 0, s>>>(c, A, ni);
  return cudaGetLastError();
}
cudaError_t bs_stop(BatchCtl* c, const BatchStepArrays& A, int ni, int stop_crit, double tol,
                    cudaGraphConditionalHandle cond, cudaStream_t s) {
  k_bs_stop<<<1, kCtlThreads, 0, s>>>(c, A, ni, stop_crit, tol, cond);
  return cudaGetLastError();
}
cudaError_t bs_solve_start(BatchCtl* c, const BatchStepArrays& A, int ni,
                           cudaGraphConditionalHandle cond, cudaStream_t s) {
  k_bs_solve_start<<<1, kCtlThreads, 0, s>>>(c, A, ni, cond);
  return cudaGetLastError();
}
cudaError_t bs_loop_start(const BatchView& B, BatchCtl* c, cudaGraphConditionalHandle cond,
                          cudaStream_t s) {
  k_bs_loop_start<<<1, 32, 0, s>>>(B.nactive, c, cond);
  return cudaGetLastError();
}
cudaError_t bs_loop_next(const BatchView& B, BatchCtl* c, int maxit, int iters_per_trip,
                         cudaGraphConditionalHandle cond, cudaStream_t s) {
  k_bs_loop_next<<<1, 32, 0, s>>>(B.nactive, c, maxit, iters_per_trip, cond);
  return cudaGetLastError();
}
cudaError_t bs_sweep_end(BatchCtl* c, const BatchView& B, const BatchStepArrays& A, int ni,
                         bool comp, cudaGraphConditionalHandle cond, cudaStream_t s) {
  k_bs_sweep_end<<<1, kCtlThreads, 0, s>>>(c, B.bs, A, ni, comp ? 1 : 0, cond);
  return cudaGetLastError();
}
cudaError_t bs_sweep_next(BatchCtl* c, const BatchStepArrays& A, int ni, int max_sweeps,
                          cudaGraphConditionalHandle cond, cudaStream_t s) {
  k_bs_sweep_next<<<1, kCtlThreads, 0, s>>>(c, A, ni, max_sweeps, cond);
  return cudaGetLastError();
}
cudaError_t bs_solve_end(BatchCtl* c, const BatchStepArrays& A, int ni, bool comp,
                         cudaStream_t s) {
  k_bs_solve_end<<<1, kCtlThreads, 0, s>>>(c, A, ni, comp ? 1 : 0);
  return cudaGetLastError();
}
cudaError_t bs_nl_next(BatchCtl* c, int maxnlit, cudaStream_t s) {
  k_bs_nl_next<<<1, 32, 0, s>>>(c, maxnlit);
  return cudaGetLastError();
}
cudaError_t bs_finish(BatchCtl* c, const int* elem_err, cudaGraphConditionalHandle cond,
                      cudaStream_t s) {
  k_bs_finish<<<1, 32, 0, s>>>(c, elem_err, cond);
  return cudaGetLastError();
}

}  // namespace pm
