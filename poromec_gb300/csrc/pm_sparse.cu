// pm_sparse.cu -- SpMV and Krylov kernels of the Biot hot path on sm_103a.
//
// SpMV over node panels (see Panels in pm_internal.h): one warp per node,
// the lanes stride along the panel width, so every value row of the panel
// is read as one coalesced stream and each gathered x value (L2 resident)
// serves all d rows of the node.  The reduction of the d <= 4 row sums is a
// warp shuffle tree.  The PCG / MINRES dot products that follow an SpMV are
// fused into it; every reduction ends with a last-block pass that sums the
// per-block partials in block order, so results do not depend on scheduling.
//
// The Krylov recurrences are those of pcg (Iters.f:299-595) and pminres
// (Iters.f:3987-4305, sym_ortho :6595).  Each kernel first reads the
// solver's done flag so a CUDA graph of many iterations can run past
// convergence without changing the result.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>

#include "../../include/poromec_gb300.h"
#include "pm_krylov.h"
#include "pm_reduce.h"

namespace pm {
namespace {

// Early exit shared by the per-iteration kernels.  conv_flag is set by the
// reduction that detects convergence; the first kernel of the next
// iteration turns it into done, which every later kernel reads.
__device__ __forceinline__ bool krylov_skip(KrylovScalars* ks, bool first) {
  if (ks->done) return true;
  if (first && ks->conv_flag) {
    if (blockIdx.x == 0 && threadIdx.x == 0) ks->done = 1;
    return true;
  }
  return false;
}

// v as an FP32 pair (split_pair), interleaved so that one 8-byte gather of
// the compensated operator fetches both halves.
__device__ __forceinline__ void split_store(double v, float2* pr, int i) {
  pr[i] = split_pair(v);
}

// ---- SpMV over panels ------------------------------------------------------
// A sub-warp of 8 lanes per node: lane t of the sub-warp accumulates columns
// t, t+8, ... of the node's d <= 4 panel rows (coalesced 64-byte runs per
// row), then the 4 row sums are reduced across the 8 lanes with a
// transposed butterfly (each lane keeps half of its values at every level:
// 4 adds per lane instead of 4 x 3).  On GB300 the FP64 pipe issues 2
// DFMA per clock per SM, so for T = double the kernel is bound by FP64
// instructions, not HBM: the count is one FMA per stored value plus 4 adds
// per lane and node.  T = float is the FP32 inner operator of the refinement.
//
// MODE 0: y = A x.   MODE 1: PCG, also alpha = d / (y . x).
// MODE 2: MINRES, also alpha = |x . y| / beta^2.   MODE 3: y = A x and
// ks->xkx = x . y (energy norm of the solver log).   MODE 4: mixed PCG,
// FP32 operator, alpha = d / (y . xd) with the FP64 direction xd.
//
// Nodes are visited in P.order, sorted by (d, W): the 4 sub-warps of a warp
// then run the same loop, so FP64 instructions issue with full lane masks
// (on GB300 a partial-mask FP64 instruction costs the full pipe time).
constexpr int kSub = 8;

template <typename T>
__device__ __forceinline__ T shfl(T v, int m) {
  return __shfl_xor_sync(0xffffffffu, v, m);
}

template <typename T, int MODE>
__global__ void __launch_bounds__(256)
    k_spmv(PanelView P, const T* __restrict__ val, const T* __restrict__ x,
           T* __restrict__ y, KrylovScalars* ks, double* partial, unsigned* counter,
           const double* __restrict__ xd = nullptr) {
  if (MODE == 1 || MODE == 2 || MODE == 4)
    if (krylov_skip(ks, true)) return;
  const int lane = threadIdx.x & 31;
  const int t = lane & (kSub - 1);
  const int warp = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int nwarp = (int)((gridDim.x * blockDim.x) >> 5);
  constexpr int kNodesPerWarp = 32 / kSub;
  double dsum = 0.0;
  for (int base = warp * kNodesPerWarp; base < P.nact; base += nwarp * kNodesPerWarp) {
    const NodeRef nr = node_ref(P, base + (lane >> 3));
    int e0 = 0, d = 0, W = 0;
    T a0 = T(0), a1 = T(0), a2 = T(0), a3 = T(0);
    if (nr.on) {
      e0 = nr.e0;
      d = nr.d;
      W = nr.W;
      const T* v = val + nr.vo;
      const int32_t* cols = P.cols + nr.co;
      if (d == 4) {
        for (int c = t; c < W; c += kSub) {
          const T xv = x[cols[c]];
          a0 += v[c] * xv;
          a1 += v[W + c] * xv;
          a2 += v[2 * W + c] * xv;
          a3 += v[3 * W + c] * xv;
        }
      } else if (d == 3) {
        for (int c = t; c < W; c += kSub) {
          const T xv = x[cols[c]];
          a0 += v[c] * xv;
          a1 += v[W + c] * xv;
          a2 += v[2 * W + c] * xv;
        }
      } else {
        for (int c = t; c < W; c += kSub) {
          const T xv = x[cols[c]];
          a0 += v[c] * xv;
          if (d > 1) a1 += v[W + c] * xv;
        }
      }
    }
    // transposed butterfly over the 8 lanes of the sub-warp
    const bool h4 = (t & 4) != 0, h2 = (t & 2) != 0;
    T k0 = h4 ? a2 : a0, k1 = h4 ? a3 : a1;
    k0 += shfl(h4 ? a0 : a2, 4);
    k1 += shfl(h4 ? a1 : a3, 4);
    T k = h2 ? k1 : k0;
    k += shfl(h2 ? k0 : k1, 2);
    k += shfl(k, 1);
    const int r = (h4 ? 2 : 0) + (h2 ? 1 : 0);
    if ((t & 1) == 0 && r < d) {
      y[e0 + r] = k;
      if (MODE == 4) dsum += double(k) * xd[e0 + r];
      else if (MODE != 0) dsum += double(k * x[e0 + r]);
    }
  }
  if (MODE != 0) {
    double in[1] = {dsum}, tot[1];
    if (grid_reduce<1>(in, partial, counter, tot) && threadIdx.x == 0) {
      if (MODE == 1 || MODE == 4) {
        ks->pq = tot[0];
        ks->alpha = ks->d / tot[0];
      } else if (MODE == 2) {
        ks->alpha = fabs(tot[0]) * (1.0 / (ks->beta * ks->beta));
      } else {
        ks->xkx = tot[0];
      }
    }
  }
}

// ---- PCG -------------------------------------------------------------------
// r = b, z = m r, p = z, d = (r, z); conv = tol sqrt|(b, m b)|  (x0 = 0, so
// b - A x0 = b exactly)
__global__ void __launch_bounds__(256)
    k_pcg_init(int n, const double* __restrict__ b, const double* __restrict__ m,
               double* __restrict__ r, double* __restrict__ z, double* __restrict__ p,
               double* __restrict__ x, KrylovScalars* ks, double tol, int maxit,
               double* partial, unsigned* counter) {
  double acc = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double bi = b[i], zi = bi * m[i];
    x[i] = 0.0;
    r[i] = bi;
    z[i] = zi;
    p[i] = zi;
    acc += bi * zi;
  }
  double in[1] = {acc}, tot[1];
  if (grid_reduce<1>(in, partial, counter, tot) && threadIdx.x == 0) {
    ks->d = tot[0];
    ks->bmb = tot[0];
    ks->conv = tol * sqrt(fabs(tot[0]));
    ks->done = 0;
    ks->conv_flag = 0;
    ks->iter = 0;
    ks->maxit = maxit;
  }
}

// x += alpha p, r -= alpha q, z = m r, di = (r, z), beta = di / d, d = di;
// converged when sqrt|d| < conv (Iters.f:446-497).
__global__ void __launch_bounds__(256)
    k_pcg_update(int n, double* __restrict__ x, const double* __restrict__ p,
                 double* __restrict__ r, const double* __restrict__ q,
                 const double* __restrict__ m, double* __restrict__ z,
                 KrylovScalars* ks, double* partial, unsigned* counter) {
  if (krylov_skip(ks, false)) return;
  const double alpha = ks->alpha;
  if (!isfinite(alpha)) {
    // breakdown ((p, A p) = 0): stop with x at the last finite iterate
    if (blockIdx.x == 0 && threadIdx.x == 0) ks->conv_flag = 3;
    return;
  }
  // x, r and q are streamed (evict-first), so that L2 keeps the operand of
  // the next product (p, or its FP32 pair), m and z
  double acc = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    __stcs(&x[i], __ldcs(&x[i]) + alpha * p[i]);
    const double ri = __ldcs(&r[i]) - alpha * __ldcs(&q[i]);
    __stcs(&r[i], ri);
    const double zi = ri * m[i];
    z[i] = zi;
    acc += ri * zi;
  }
  double in[1] = {acc}, tot[1];
  if (grid_reduce<1>(in, partial, counter, tot) && threadIdx.x == 0) {
    const double di = tot[0];
    ks->beta = di / ks->d;
    ks->d = di;
    ks->iter += 1;
    if (sqrt(fabs(di)) < ks->conv) ks->conv_flag = 1;
    else if (!isfinite(di)) ks->conv_flag = 3;  // breakdown: stop instead of iterating on NaN
    else if (ks->iter >= ks->maxit) ks->conv_flag = 2;
  }
}

__global__ void __launch_bounds__(256)
    k_pcg_dir(int n, const double* __restrict__ z, double* __restrict__ p,
              KrylovScalars* ks) {
  if (krylov_skip(ks, false)) return;
  const double beta = ks->beta;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    p[i] = __ldcs(&z[i]) + beta * p[i];  // p stays in L2 for the product
}

// ---- mixed-precision PCG (inner solve of the FP64 refinement) ----------------
// The recurrences of pcg on FP64 vectors and scalars; only the product
// q = A p uses the FP32 panel values and FP32 copies of p and q.
__global__ void __launch_bounds__(256)
    k_pcgm_init(int n, const double* __restrict__ b, const double* __restrict__ m,
                double* __restrict__ r, double* __restrict__ z, double* __restrict__ p,
                float* __restrict__ p32, double* __restrict__ x, KrylovScalars* ks, double tol,
                int maxit, double* partial, unsigned* counter) {
  double acc = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double bi = b[i], zi = bi * m[i];
    x[i] = 0.0;
    r[i] = bi;
    z[i] = zi;
    p[i] = zi;
    p32[i] = float(zi);
    acc += bi * zi;
  }
  double in[1] = {acc}, tot[1];
  if (grid_reduce<1>(in, partial, counter, tot) && threadIdx.x == 0) {
    ks->d = tot[0];
    ks->bmb = tot[0];
    ks->conv = tol * sqrt(fabs(tot[0]));
    ks->done = 0;
    ks->conv_flag = 0;
    ks->iter = 0;
    ks->maxit = maxit;
  }
}

__global__ void __launch_bounds__(256)
    k_pcgm_update(int n, double* __restrict__ x, const double* __restrict__ p,
                  double* __restrict__ r, const float* __restrict__ q32,
                  const double* __restrict__ m, double* __restrict__ z, KrylovScalars* ks,
                  double* partial, unsigned* counter) {
  if (krylov_skip(ks, false)) return;
  const double alpha = ks->alpha;
  double acc = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    x[i] = x[i] + alpha * p[i];
    const double ri = r[i] - alpha * double(q32[i]);
    r[i] = ri;
    const double zi = ri * m[i];
    z[i] = zi;
    acc += ri * zi;
  }
  double in[1] = {acc}, tot[1];
  if (grid_reduce<1>(in, partial, counter, tot) && threadIdx.x == 0) {
    const double di = tot[0];
    ks->beta = di / ks->d;
    ks->d = di;
    ks->iter += 1;
    if (sqrt(fabs(di)) < ks->conv) ks->conv_flag = 1;
    else if (!isfinite(di)) ks->conv_flag = 3;
    else if (ks->iter >= ks->maxit) ks->conv_flag = 2;
  }
}

__global__ void __launch_bounds__(256)
    k_pcgm_dir(int n, const double* __restrict__ z, double* __restrict__ p,
               float* __restrict__ p32, KrylovScalars* ks) {
  if (krylov_skip(ks, false)) return;
  const double beta = ks->beta;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double pi = z[i] + beta * p[i];
    p[i] = pi;
    p32[i] = float(pi);
  }
}

// ---- MINRES ----------------------------------------------------------------
__device__ double sign1(double a) { return a > 0.0 ? 1.0 : (a < 0.0 ? -1.0 : 0.0); }

// sym_ortho (Iters.f:6595-6640); c, s, r keep their values in the branch the
// reference leaves uncovered (b != 0, a > 0, |b| == a).
__device__ void sym_ortho(double a, double b, double& c, double& s, double& r) {
  const double ma = fabs(a), mb = fabs(b), sa = sign1(a), sb = sign1(b);
  if (b == 0.0) {
    s = 0.0;
    r = ma;
    c = (a == 0.0) ? 1.0 : sa;
  } else if (a == 0.0) {
    c = 0.0;
    s = sb;
    r = mb;
  } else if (mb > a) {
    const double t = a / b;
    s = sb / sqrt(1.0 + t * t);
    c = s * t;
    r = b / s;
  } else if (ma > mb) {
    const double t = b / a;
    c = sa / sqrt(1.0 + t * t);
    s = c * t;
    r = a / c;
  }
}

// conv = tol * || M^(1/2) b || with M = |m| (Iters.f:4082-4088)
__global__ void __launch_bounds__(256)
    k_minres_conv(int n, const double* __restrict__ b, const double* __restrict__ m,
                  KrylovScalars* ks, double tol, double* partial, unsigned* counter) {
  double acc = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double zi = b[i] * sqrt(fabs(m[i]));
    acc += zi * zi;
  }
  double in[1] = {acc}, tot[1];
  if (grid_reduce<1>(in, partial, counter, tot) && threadIdx.x == 0)
    ks->conv = tol * sqrt(fabs(tot[0]));
}

// (Re)start: v = b - A x (q = A x), v0 = w0 = w00 = 0, z0 = m v,
// beta = sqrt|(v, z0)| (Iters.f:4100-4131)
__global__ void __launch_bounds__(256)
    k_minres_start(int n, const double* __restrict__ b, const double* __restrict__ q,
                   const double* __restrict__ m, double* __restrict__ v,
                   double* __restrict__ v0, double* __restrict__ w0,
                   double* __restrict__ w00, double* __restrict__ z0, KrylovScalars* ks,
                   int maxit, double* partial, unsigned* counter, float2* __restrict__ zc) {
  double acc = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double vi = b[i] - q[i];
    v[i] = vi;
    v0[i] = 0.0;
    w0[i] = 0.0;
    w00[i] = 0.0;
    const double zi = vi * m[i];
    z0[i] = zi;
    if (zc) split_store(zi, zc, i);
    acc += vi * zi;
  }
  double in[1] = {acc}, tot[1];
  if (grid_reduce<1>(in, partial, counter, tot) && threadIdx.x == 0) {
    const double beta = sqrt(fabs(tot[0]));
    ks->beta = beta;
    ks->normr = beta;
    ks->neta = beta;
    ks->beta_old = beta;
    ks->c_old = 1.0;
    ks->c = 1.0;
    ks->s_old = 0.0;
    ks->s = 0.0;
    ks->done = 0;
    ks->conv_flag = 0;
    ks->jcycle = 0;
    ks->maxit = maxit;
  }
}

// p = (A z0)/beta - alpha v/beta - beta v0/beta_old, z = m p,
// beta_new = sqrt|(z, p)|, then the QR update of the tridiagonal
// (Iters.f:4143-4200).
__global__ void __launch_bounds__(256)
    k_minres_lanczos(int n, double* __restrict__ p, const double* __restrict__ v,
                     const double* __restrict__ v0, const double* __restrict__ m,
                     double* __restrict__ z, KrylovScalars* ks, double* partial,
                     unsigned* counter, float2* __restrict__ zc) {
  if (krylov_skip(ks, false)) return;
  const double beta = ks->beta;
  const double t1 = 1.0 / beta, t2 = -ks->alpha / beta, t3 = -beta / ks->beta_old;
  double acc = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double pi = t1 * p[i] + t2 * v[i] + t3 * v0[i];
    p[i] = pi;
    const double zi = pi * m[i];
    z[i] = zi;
    if (zc) split_store(zi, zc, i);
    acc += zi * pi;
  }
  double in[1] = {acc}, tot[1];
  if (grid_reduce<1>(in, partial, counter, tot) && threadIdx.x == 0) {
    const double alpha = ks->alpha;
    const double beta_old = beta;
    const double beta_new = sqrt(fabs(tot[0]));
    double c = ks->c, s = ks->s;
    const double c_old = ks->c_old, s_old = ks->s_old;
    const double delta = c * alpha - c_old * s * beta_old;
    const double ro2 = s * alpha + c_old * c * beta_old;
    const double ro3 = s_old * beta_old;
    ks->c_old = c;
    ks->s_old = s;
    double ro1 = ks->ro1;
    sym_ortho(delta, beta_new, c, s, ro1);
    ks->c = c;
    ks->s = s;
    ks->ro1 = ro1;
    ks->beta_old = beta_old;
    ks->beta = beta_new;
    ks->t1 = 1.0 / (beta_old * ro1);
    ks->t2 = -ro2 / ro1;
    ks->t3 = -ro3 / ro1;
    ks->t4 = c * ks->neta;
    ks->normr = fabs(s) * ks->normr;
    ks->iter += 1;
    ks->jcycle += 1;
    if (ks->normr < ks->conv) {
      ks->conv_flag = 1;
    } else if (!isfinite(ks->normr)) {
      ks->conv_flag = 3;
    } else {
      ks->neta = -s * ks->neta;
      if (ks->jcycle >= ks->maxit) ks->conv_flag = 2;
    }
  }
}

// w = t1 z0 + t2 w0 + t3 w00, x += t4 w, then the shifts v0 = v, v = p,
// z0 = z, w00 = w0, w0 = w (Iters.f:4202-4222).
__global__ void __launch_bounds__(256)
    k_minres_update(int n, double* __restrict__ x, double* __restrict__ z0,
                    double* __restrict__ w0, double* __restrict__ w00,
                    double* __restrict__ v0, double* __restrict__ v,
                    const double* __restrict__ p, const double* __restrict__ z,
                    KrylovScalars* ks) {
  if (krylov_skip(ks, false)) return;
  const double t1 = ks->t1, t2 = ks->t2, t3 = ks->t3, t4 = ks->t4;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double wi = t1 * z0[i] + t2 * w0[i] + t3 * w00[i];
    x[i] = x[i] + t4 * wi;
    v0[i] = v[i];
    v[i] = p[i];
    z0[i] = z[i];
    w00[i] = w0[i];
    w0[i] = wi;
  }
}

// ---- compensated FP32 operator (PM_FP32C_REFINE) -----------------------------
// Each FP64 panel value v is stored as hi = fl32(v) and an int8 relative
// correction q = round((v - hi) / hi * 2^31), |q| <= 127 (5 bytes; v is
// represented as hi (1 + q 2^-31) within 2^-32 |v|, hi's own rounding being
// at most 2^-24 |hi|).  The operand vector is an FP32 pair (xh, xl).
// Products and sums use error-free FP32 transformations: t = hi*xh and its
// rounding error e = fma(hi, xh, -t) (TwoProd), the cross terms hi*xl and
// t*q*2^-31 (= (v - hi)*xh to 2^-24 relative) go to a correction, and the
// running sum is a (sum, correction) pair updated with TwoSum.  The FP32
// pipe issues 128 lanes per clock per SM against 2 for FP64, so this
// operator is bound by HBM, with an error of ~2e-10 per entry where plain
// FP32 storage (2^-24) is amplified by the conditioning of this indefinite
// system beyond what refinement recovers.
struct F2 {
  float s, c;
};

__device__ __forceinline__ void two_sum_acc(F2& a, float t) {
  const float s = a.s + t;
  const float bp = s - a.s;
  const float err = (a.s - (s - bp)) + (t - bp);
  a.s = s;
  a.c += err;
}

__device__ __forceinline__ F2 f2_add(F2 a, F2 b) {
  F2 r{a.s, a.c + b.c};
  two_sum_acc(r, b.s);
  return r;
}

// q * 2^-31 for an int8 q, exactly: 1.5 * 2^23 + q is a float whose low
// mantissa bits are q; scaling by 2^-31 and removing 1.5 * 2^-8 is exact.
__device__ __forceinline__ float q_scale(int q) {
  return fmaf(__int_as_float(0x4B400000 + q), 0x1p-31f, -0x1.8p-8f);
}

__device__ __forceinline__ void f2_fma(F2& acc, float vh, int q, float xh, float xl) {
  const float t = vh * xh;
  const float e = fmaf(vh, xh, -t);
  const float c = fmaf(vh, xl, fmaf(t, q_scale(q), e));
  two_sum_acc(acc, t);
  acc.c += c;
}

// Packed two-lane FP32 arithmetic of sm_100+ (fma/add/sub/mul .rn.f32x2):
// two rows of a node, which share the column's x pair, in one instruction.
// Each lane is an IEEE round-to-nearest FP32 operation, so the error-free
// transformations below hold lane by lane.
typedef unsigned long long f2x;
__device__ __forceinline__ f2x pk2(float a, float b) {
  f2x r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ float2 up2(f2x r) {
  float2 a;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a.x), "=f"(a.y) : "l"(r));
  return a;
}
__device__ __forceinline__ f2x fma2(f2x a, f2x b, f2x c) {
  f2x d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}
__device__ __forceinline__ f2x add2(f2x a, f2x b) {
  f2x d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f2x sub2(f2x a, f2x b) {
  f2x d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f2x mul2(f2x a, f2x b) {
  f2x d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}

// Compensated accumulation of two rows at once.  sn holds minus the running
// sum of the rounded products t (so that the product can be formed as
// tn = hi * (-xh) = -t and its error as fma(hi, xh, tn) without negations),
// cn minus the TwoSum errors, cp the product corrections
// e + hi*xl + t*q*2^-31; the row value is -sn + (cp - cn).
struct P2 {
  f2x sn, cn, cp;
};

__device__ __forceinline__ void p2_fma(P2& a, f2x vh, f2x nqs, f2x xh, f2x nxh, f2x xl) {
  const f2x tn = mul2(vh, nxh);
  const f2x e = fma2(vh, xh, tn);
  const f2x s = add2(a.sn, tn);
  const f2x bp = sub2(s, a.sn);
  const f2x err = add2(sub2(a.sn, sub2(s, bp)), sub2(tn, bp));
  a.sn = s;
  a.cn = add2(a.cn, err);
  a.cp = fma2(vh, xl, fma2(tn, nqs, add2(a.cp, e)));
}

// -q0 2^-31, -q1 2^-31 for two int8 corrections (the magic-number
// conversion of q_scale, with the sign folded into the constants)
__device__ __forceinline__ f2x p2_nqs(int q0, int q1) {
  const f2x f = pk2(__int_as_float(0x4B400000 + q0), __int_as_float(0x4B400000 + q1));
  return fma2(f, pk2(-0x1p-31f, -0x1p-31f), pk2(0x1.8p-8f, 0x1.8p-8f));
}

__device__ __forceinline__ F2 f2_shfl(F2 a, int m) {
  return F2{__shfl_xor_sync(0xffffffffu, a.s, m), __shfl_xor_sync(0xffffffffu, a.c, m)};
}

// Rows of one node panel on the compensated operator: lane t of the S-lane
// sub-warp takes columns t, t + S, ...; U columns per trip.  The column
// indices of the next trip are loaded one trip ahead, so each trip issues its
// U gathers of x pairs together with its U * D value loads instead of after
// a dependent index load.  Values and column indices are read once per
// product and loaded with the evict-first hint, which leaves L2 to the
// gathered operand.  The last trip is masked.
template <int D, int S, int U, bool PK>
__device__ __forceinline__ void cf_rows(const float* __restrict__ h,
                                        const int8_t* __restrict__ l,
                                        const int32_t* __restrict__ cols,
                                        const float2* __restrict__ xp, int W, int t,
                                        F2 (&a)[4]) {
  // PK: rows 2k, 2k+1 in packed two-lane arithmetic (an odd last row scalar)
  P2 pa[2] = {{0ull, 0ull, 0ull}, {0ull, 0ull, 0ull}};
  int cn[U];
#pragma unroll
  for (int u = 0; u < U; ++u) cn[u] = (t + u * S < W) ? __ldcs(&cols[t + u * S]) : -1;
  for (int c = t; c < W; c += U * S) {
    float2 xv[U];
    float hv[U][D];
    int lv[U][D];
#pragma unroll
    for (int u = 0; u < U; ++u) xv[u] = cn[u] >= 0 ? xp[cn[u]] : make_float2(0.f, 0.f);
#pragma unroll
    for (int u = 0; u < U; ++u)
#pragma unroll
      for (int r = 0; r < D; ++r) {
        const bool ok = c + u * S < W;
        hv[u][r] = ok ? __ldcs(&h[r * W + c + u * S]) : 0.f;
        lv[u][r] = ok ? int(__ldcs(&l[r * W + c + u * S])) : 0;
      }
    const int cnext = c + U * S;
#pragma unroll
    for (int u = 0; u < U; ++u)
      cn[u] = (cnext + u * S < W) ? __ldcs(&cols[cnext + u * S]) : -1;
    if (PK) {
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const f2x xh = pk2(xv[u].x, xv[u].x), nxh = pk2(-xv[u].x, -xv[u].x);
        const f2x xl = pk2(xv[u].y, xv[u].y);
#pragma unroll
        for (int k = 0; k < D / 2; ++k)
          p2_fma(pa[k], pk2(hv[u][2 * k], hv[u][2 * k + 1]),
                 p2_nqs(lv[u][2 * k], lv[u][2 * k + 1]), xh, nxh, xl);
        if (D & 1) f2_fma(a[D - 1], hv[u][D - 1], lv[u][D - 1], xv[u].x, xv[u].y);
      }
    } else {
#pragma unroll
      for (int u = 0; u < U; ++u)
#pragma unroll
        for (int r = 0; r < D; ++r)
          f2_fma(a[r], hv[u][r], lv[u][r], xv[u].x, xv[u].y);
    }
  }
  if (PK) {
#pragma unroll
    for (int k = 0; k < D / 2; ++k) {
      const float2 sn = up2(pa[k].sn), cn2 = up2(pa[k].cn), cp = up2(pa[k].cp);
      a[2 * k] = F2{-sn.x, cp.x - cn2.x};
      a[2 * k + 1] = F2{-sn.y, cp.y - cn2.y};
    }
  }
}

// MODE 0: y = A x.  MODE 1: PCG, alpha = d / (y . xd).  MODE 2: MINRES,
// alpha = |xd . y| / beta^2.  xd is the FP64 operand whose pair is xp; y is
// FP64.  S: lanes per node (8, 16 or 32), U: columns per lane and trip; both
// chosen per matrix by the autotuner.  With S = 32 a warp reads each panel
// row as full 128-byte lines; with S = 8 four nodes share a warp and each
// load instruction touches four lines.
template <int MODE, int S, int U, bool PK, int MINB>
__global__ void __launch_bounds__(256, MINB)
    k_spmv_cf(PanelView P, const float* __restrict__ vh, const int8_t* __restrict__ vl,
              const float2* __restrict__ xp, double* __restrict__ y, const double* __restrict__ xd,
              KrylovScalars* ks, double* partial, unsigned* counter) {
  if (MODE != 0)
    if (krylov_skip(ks, true)) return;
  const int lane = threadIdx.x & 31;
  const int t = lane & (S - 1);
  const int warp = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int nwarp = (int)((gridDim.x * blockDim.x) >> 5);
  constexpr int kNodesPerWarp = 32 / S;
  const int stride = nwarp * kNodesPerWarp;
  double dsum = 0.0;
  for (int base = warp * kNodesPerWarp; base < P.nact; base += stride) {
    const NodeRef nr = node_ref(P, base + lane / S);
    int e0 = 0, d = 0, W = 0;
    F2 a[4] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
    if (nr.on) {
      e0 = nr.e0;
      d = nr.d;
      W = nr.W;
      const float* h = vh + nr.vo;
      const int8_t* l = vl + nr.vo;
      const int32_t* cols = P.cols + nr.co;
      if (d == 4) cf_rows<4, S, U, PK>(h, l, cols, xp, W, t, a);
      else if (d == 3) cf_rows<3, S, U, PK>(h, l, cols, xp, W, t, a);
      else if (d == 2) cf_rows<2, S, U, PK>(h, l, cols, xp, W, t, a);
      else cf_rows<1, S, U, PK>(h, l, cols, xp, W, t, a);
    }
    // transposed butterfly on (sum, correction) pairs over the S lanes: the
    // first two levels halve the rows each lane carries, the rest add
    constexpr int o1 = S / 2, o2 = S / 4;
    const bool h1 = (t & o1) != 0, h2 = (t & o2) != 0;
    F2 k0 = h1 ? a[2] : a[0], k1 = h1 ? a[3] : a[1];
    k0 = f2_add(k0, f2_shfl(h1 ? a[0] : a[2], o1));
    k1 = f2_add(k1, f2_shfl(h1 ? a[1] : a[3], o1));
    F2 k = h2 ? k1 : k0;
    k = f2_add(k, f2_shfl(h2 ? k0 : k1, o2));
#pragma unroll
    for (int o = S / 8; o > 0; o >>= 1) k = f2_add(k, f2_shfl(k, o));
    const int r = (h1 ? 2 : 0) + (h2 ? 1 : 0);
    if ((t & (o2 - 1)) == 0 && r < d) {
      const double v = double(k.s) + double(k.c);
      y[e0 + r] = v;
      if (MODE != 0) dsum += v * __ldcs(&xd[e0 + r]);
    }
  }
  if (MODE != 0) {
    double in[1] = {dsum}, tot[1];
    if (grid_reduce<1>(in, partial, counter, tot) && threadIdx.x == 0) {
      if (MODE == 1) {
        ks->pq = tot[0];
        ks->alpha = ks->d / tot[0];
      } else {
        ks->alpha = fabs(tot[0]) * (1.0 / (ks->beta * ks->beta));
      }
    }
  }
}

// ---- record kernel: node records streamed into shared memory by cp.async ----
// Each warp takes nodes gw, gw + nw, ... of the visiting order (gw its global
// warp index, nw the warps of the grid) and keeps two record buffers in
// shared memory: while it computes node i from one, the 16-byte cp.async
// copies of node i + nw stream into the other.  The bytes in flight per SM
// are then set by the buffers (about a record per warp), not by the loads a
// thread holds in registers, which bounds the register kernels above at
// the read bandwidth of one 16-byte load per thread in flight.  The copies
// complete through cp.async.wait_group, so the kernel contains no
// spin-wait of its own.
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// (qb_k - 128) * 2^-31 for byte k of a packed word of biased corrections,
// exactly: the byte permute builds the float 1.5 * 2^23 + qb_k; scaling by
// 2^-31 and removing (1.5 * 2^23 + 128) * 2^-31 = 0x1.8001p-8 is exact.
__device__ __forceinline__ float qb_scale(unsigned w, int k) {
  const float f = __int_as_float((int)__byte_perm(w, 0x4B400000u, 0x7640u | (unsigned)k));
  return fmaf(f, 0x1p-31f, -0x1.8001p-8f);
}

__device__ __forceinline__ void f2_fma_s(F2& acc, float vh, float qs, float xh, float xl) {
  const float t = vh * xh;
  const float e = fmaf(vh, xh, -t);
  const float c = fmaf(vh, xl, fmaf(t, qs, e));
  two_sum_acc(acc, t);
  acc.c += c;
}

__device__ __forceinline__ int rec_bytes(int d, int Wp) {
  return 4 * d * Wp + ((d * Wp + 15) & ~15) + 4 * Wp;
}

// Rows of one node from its record in shared memory: lane t takes column
// quads t, t + 32, t + 64 per trip, issues the 12 gathers of x pairs for
// them, then the compensated products of the d rows.
template <int D>
__device__ __forceinline__ void ca_rows(const float4* __restrict__ h4,
                                        const unsigned* __restrict__ q4,
                                        const int4* __restrict__ c4,
                                        const float2* __restrict__ xp, int nq, int lane,
                                        F2 (&a)[4]) {
  for (int j0 = lane; j0 < nq; j0 += 96) {
    float2 xv[3][4];
#pragma unroll
    for (int u = 0; u < 3; ++u) {
      const int j = j0 + 32 * u;
      const int4 cc = j < nq ? c4[j] : make_int4(0, 0, 0, 0);
      xv[u][0] = xp[cc.x];
      xv[u][1] = xp[cc.y];
      xv[u][2] = xp[cc.z];
      xv[u][3] = xp[cc.w];
    }
#pragma unroll
    for (int u = 0; u < 3; ++u) {
      const int j = j0 + 32 * u;
      if (j < nq) {
#pragma unroll
        for (int r = 0; r < D; ++r) {
          const float4 hv = h4[r * nq + j];
          const unsigned qv = q4[r * nq + j];
          f2_fma_s(a[r], hv.x, qb_scale(qv, 0), xv[u][0].x, xv[u][0].y);
          f2_fma_s(a[r], hv.y, qb_scale(qv, 1), xv[u][1].x, xv[u][1].y);
          f2_fma_s(a[r], hv.z, qb_scale(qv, 2), xv[u][2].x, xv[u][2].y);
          f2_fma_s(a[r], hv.w, qb_scale(qv, 3), xv[u][3].x, xv[u][3].y);
        }
      }
    }
  }
}

// MODE as k_spmv_cf.  Shared memory: per warp two buffers of C.rec_max
// bytes, then per warp 32 staged row results (float2) and their equations.
// Row results leave the butterfly in 4 lanes; they are staged and converted
// to FP64 (and dotted with xd) 32 at a time, so the FP64 instructions, which
// cost a full warp's pipe time whatever their mask, run with all lanes on.
template <int MODE>
__global__ void __launch_bounds__(512, 1)
    k_spmv_ca(PanelView P, CompVals C, const float2* __restrict__ xp, double* __restrict__ y,
              const double* __restrict__ xd, KrylovScalars* ks, double* partial,
              unsigned* counter) {
  if (MODE != 0)
    if (krylov_skip(ks, true)) return;
  extern __shared__ __align__(16) unsigned char ca_smem[];
  const int lane = threadIdx.x & 31, w = (int)(threadIdx.x >> 5);
  const int nwb = (int)(blockDim.x >> 5);
  const size_t rmax = (size_t)C.rec_max;
  unsigned char* buf = ca_smem + (size_t)w * 2 * rmax;
  float2* o_sc = reinterpret_cast<float2*>(ca_smem + (size_t)nwb * 2 * rmax) + w * 32;
  int* o_eq = reinterpret_cast<int*>(ca_smem + (size_t)nwb * 2 * rmax +
                                     (size_t)nwb * 32 * sizeof(float2)) + w * 32;
  const int gw = (int)blockIdx.x * nwb + w, nw = (int)gridDim.x * nwb;
  auto issue = [&](int i, int b) {
    const int k = P.order[i];
    const int R = rec_bytes(P.d[k], (P.W[k] + 3) & ~3);
    const unsigned char* src = C.rec + C.rec_off[k];
    unsigned char* dst = buf + (size_t)b * rmax;
    for (int c = lane * 16; c < R; c += 32 * 16) cp_async16(dst + c, src + c);
  };
  double dsum = 0.0;
  int count = 0;  // staged rows of this warp (warp-uniform)
  auto flush = [&]() {
    __syncwarp();
    if (lane < count) {
      const float2 sc = o_sc[lane];
      const int e = o_eq[lane];
      const double v = double(sc.x) + double(sc.y);
      y[e] = v;
      if (MODE != 0) dsum += v * xd[e];
    }
    __syncwarp();
    count = 0;
  };
  if (gw < P.nact) issue(gw, 0);
  cp_async_commit();
  int it = 0;
  for (int i = gw; i < P.nact; i += nw, ++it) {
    if (i + nw < P.nact) issue(i + nw, (it + 1) & 1);
    cp_async_commit();
    cp_async_wait<1>();  // this lane's copies of node i have landed
    __syncwarp();        // ... and every other lane's
    const int k = P.order[i];
    const int d = P.d[k], e0 = P.eq0[k];
    const int Wp = (P.W[k] + 3) & ~3, nq = Wp >> 2;
    const unsigned char* b = buf + (size_t)(it & 1) * rmax;
    const float4* h4 = reinterpret_cast<const float4*>(b);
    const unsigned* q4 = reinterpret_cast<const unsigned*>(b + 4 * d * Wp);
    const int4* c4 = reinterpret_cast<const int4*>(b + 4 * d * Wp + ((d * Wp + 15) & ~15));
    F2 a[4] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
    if (d == 4) ca_rows<4>(h4, q4, c4, xp, nq, lane, a);
    else if (d == 3) ca_rows<3>(h4, q4, c4, xp, nq, lane, a);
    else if (d == 2) ca_rows<2>(h4, q4, c4, xp, nq, lane, a);
    else ca_rows<1>(h4, q4, c4, xp, nq, lane, a);
    __syncwarp();  // the buffer is read; the next trip refills it
    // transposed butterfly over the 32 lanes (as in k_spmv_cf)
    const bool h1 = (lane & 16) != 0, h2 = (lane & 8) != 0;
    F2 k0 = h1 ? a[2] : a[0], k1 = h1 ? a[3] : a[1];
    k0 = f2_add(k0, f2_shfl(h1 ? a[0] : a[2], 16));
    k1 = f2_add(k1, f2_shfl(h1 ? a[1] : a[3], 16));
    F2 kk = h2 ? k1 : k0;
    kk = f2_add(kk, f2_shfl(h2 ? k0 : k1, 8));
    kk = f2_add(kk, f2_shfl(kk, 4));
    kk = f2_add(kk, f2_shfl(kk, 2));
    kk = f2_add(kk, f2_shfl(kk, 1));
    const int r = (h1 ? 2 : 0) + (h2 ? 1 : 0);
    if (count + d > 32) flush();
    if ((lane & 7) == 0 && r < d) {
      o_sc[count + r] = make_float2(kk.s, kk.c);
      o_eq[count + r] = e0 + r;
    }
    count += d;
  }
  cp_async_wait<0>();
  flush();
  if (MODE != 0) {
    double in[1] = {dsum}, tot[1];
    if (grid_reduce<1>(in, partial, counter, tot) && threadIdx.x == 0) {
      if (MODE == 1) {
        ks->pq = tot[0];
        ks->alpha = ks->d / tot[0];
      } else {
        ks->alpha = fabs(tot[0]) * (1.0 / (ks->beta * ks->beta));
      }
    }
  }
}

// ---- streamed record kernel: batches of node records moved by TMA ---------
// The records of the visiting order are cut on the host into batches of up
// to kCsNodes consecutive nodes, each one contiguous 16-byte aligned byte
// range, and each CTA owns a run of batches balanced by estimated time.  The
// batches stream through C.cs_nstage shared-memory stages: a producer warp
// issues one cp.async.bulk per batch, completing on the stage's mbarrier, and
// each half-warp of the kCsWarps consumer warps computes one node of the
// batch from shared memory.  The bytes in flight per SM are the stages ahead,
// independent of the registers.  Every mbarrier wait is bounded: a warp whose
// wait gives up sets *C.fault, the producer then waits with the same bound
// for its copies in flight, and every thread still takes part in the grid
// reduction, so the reduction counter stays consistent.
//
// Measured on the 56^3 cube (2.35 M equations) it takes 1.04 ms against
// 0.63 ms for the register kernels: shared memory holds two stages of 16
// whole node records (104 KB each), i.e. 16 node streams per SM, while the
// register kernels keep 48 streams of 4-column chunks in the larger register
// file; the gather latency of the x pairs is then what the streamed kernel
// cannot hide.  It stays an autotuner candidate.
__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes,
                                         unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ bool mbar_test(unsigned long long* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
// a non-blocking poll with a short sleep, given up after 2^30 clock cycles
// (about half a second; a batch lands in microseconds)
constexpr long long kCsWaitCycles = 1ll << 30;
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, unsigned parity) {
  if (mbar_test(bar, parity)) return true;
  const long long t0 = clock64();
  while (clock64() - t0 < kCsWaitCycles) {
    if (mbar_test(bar, parity)) return true;
    __nanosleep(32);
  }
  return mbar_test(bar, parity);
}

// Rows of one node from its record in shared memory by a 16-lane half-warp:
// lane t takes column quads t, t + 16, ... ; the 4 x-pair gathers of the next
// quad are issued before the products of the current one.
template <int D>
__device__ __forceinline__ void cs_rows(const float4* __restrict__ h4,
                                        const unsigned* __restrict__ q4,
                                        const int4* __restrict__ c4,
                                        const float2* __restrict__ xp, int nq, int t,
                                        F2 (&a)[4]) {
  float2 xn[4];
  int j = t;
  if (j < nq) {
    const int4 cc = c4[j];
    xn[0] = xp[cc.x];
    xn[1] = xp[cc.y];
    xn[2] = xp[cc.z];
    xn[3] = xp[cc.w];
  }
  for (; j < nq; j += 16) {
    const float2 x0 = xn[0], x1 = xn[1], x2 = xn[2], x3 = xn[3];
    const int jn = j + 16;
    if (jn < nq) {
      const int4 cc = c4[jn];
      xn[0] = xp[cc.x];
      xn[1] = xp[cc.y];
      xn[2] = xp[cc.z];
      xn[3] = xp[cc.w];
    }
#pragma unroll
    for (int r = 0; r < D; ++r) {
      const float4 hv = h4[r * nq + j];
      const unsigned qv = q4[r * nq + j];
      f2_fma_s(a[r], hv.x, qb_scale(qv, 0), x0.x, x0.y);
      f2_fma_s(a[r], hv.y, qb_scale(qv, 1), x1.x, x1.y);
      f2_fma_s(a[r], hv.z, qb_scale(qv, 2), x2.x, x2.y);
      f2_fma_s(a[r], hv.w, qb_scale(qv, 3), x3.x, x3.y);
    }
  }
}

__device__ __forceinline__ void mbar_arrive(unsigned long long* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// kCsNodes consumer warps (one node of each batch each) and one producer
// warp, whose lane 0 issues the copies.  Per stage two mbarriers: full (the
// batch landed: one arrival with the byte count, completed by the copy) and
// empty (the kCsNodes consumer warps are done with it).  The warps never
// wait for each other, only for their data, so the gather latency of one
// warp overlaps the arithmetic of the others.
template <int MODE>
__global__ void __launch_bounds__((kCsWarps + 1) * 32)
    k_spmv_cs(PanelView P, CompVals C, const float2* __restrict__ xp, double* __restrict__ y,
              const double* __restrict__ xd, KrylovScalars* ks, double* partial,
              unsigned* counter) {
  if (MODE != 0)
    if (krylov_skip(ks, true)) return;
  extern __shared__ __align__(128) unsigned char cs_smem[];
  unsigned long long* full = reinterpret_cast<unsigned long long*>(cs_smem);
  unsigned long long* empty = full + kCsMaxStages;
  const int nst = C.cs_nstage, sbytes = C.cs_stage_bytes;
  unsigned char* stages = cs_smem + 128;
  const int lane = threadIdx.x & 31, w = (int)(threadIdx.x >> 5);
  const int half = lane >> 4, t = lane & 15;
  const bool producer = w == kCsWarps;
  float2* o_sc = reinterpret_cast<float2*>(stages + (size_t)nst * sbytes) + w * 32;
  int* o_eq = reinterpret_cast<int*>(stages + (size_t)nst * sbytes +
                                     (size_t)(kCsWarps + 1) * 32 * sizeof(float2)) + w * 32;
  const int b0 = C.cs_cta_batch[blockIdx.x], b1 = C.cs_cta_batch[blockIdx.x + 1];
  if (threadIdx.x == 0) {
    for (int k = 0; k < nst; ++k) {
      mbar_init(&full[k], 1);
      mbar_init(&empty[k], kCsWarps);
    }
    mbar_fence_init();
  }
  __syncthreads();
  double dsum = 0.0;
  int count = 0;  // staged rows of this warp (warp-uniform)
  auto flush = [&]() {
    __syncwarp();
    if (lane < count) {
      const float2 sc = o_sc[lane];
      const int e = o_eq[lane];
      const double v = double(sc.x) + double(sc.y);
      y[e] = v;
      if (MODE != 0) dsum += v * xd[e];
    }
    __syncwarp();
    count = 0;
  };
  if (producer) {
    if (lane == 0) {
      int j = b0;
      bool ok = true;
      for (; j < b1 && ok; ++j) {
        const int k = (j - b0) % nst, use = (j - b0) / nst;
        // the consumers' release of the batch that used this stage before
        if (use > 0) ok = mbar_wait_bounded(&empty[k], (unsigned)((use - 1) & 1));
        if (!ok) break;
        fence_proxy_async();
        const unsigned bytes = (unsigned)C.cs_batch_bytes[j];
        mbar_expect_tx(&full[k], bytes);
        bulk_g2s(stages + (size_t)k * sbytes, C.rec + C.cs_batch_off[j], bytes, &full[k]);
      }
      if (!ok) {
        atomicExch(C.fault, 1);
        // the copies issued and maybe not consumed land before the CTA leaves
        for (int i = std::max(b0, j - nst); i < j; ++i)
          mbar_wait_bounded(&full[(i - b0) % nst], (unsigned)(((i - b0) / nst) & 1));
      }
    }
  } else {
    for (int j = b0; j < b1; ++j) {
      const int k = (j - b0) % nst;
      const int s0 = C.cs_batch_slot[j], s1 = C.cs_batch_slot[j + 1];
      const int slot = s0 + 2 * w + half;
      const bool has = slot < s1;
      const int4 dd = has ? C.cs_desc[slot] : make_int4(0, 0, 0, 0);
      const bool ok = mbar_wait_bounded(&full[k], (unsigned)(((j - b0) / nst) & 1));
      if (!__all_sync(0xffffffffu, ok)) {
        if (lane == 0) atomicExch(C.fault, 1);
        break;
      }
      const int d = dd.y;
      F2 a[4] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
      if (has) {
        const int Wp = (dd.z + 3) & ~3, nq = Wp >> 2;
        const unsigned char* b = stages + (size_t)k * sbytes + dd.w;
        const float4* h4 = reinterpret_cast<const float4*>(b);
        const unsigned* q4 = reinterpret_cast<const unsigned*>(b + 4 * d * Wp);
        const int4* c4 = reinterpret_cast<const int4*>(b + 4 * d * Wp + ((d * Wp + 15) & ~15));
        if (d == 4) cs_rows<4>(h4, q4, c4, xp, nq, t, a);
        else if (d == 3) cs_rows<3>(h4, q4, c4, xp, nq, t, a);
        else if (d == 2) cs_rows<2>(h4, q4, c4, xp, nq, t, a);
        else cs_rows<1>(h4, q4, c4, xp, nq, t, a);
      }
      __syncwarp();  // this warp has read stage k
      if (lane == 0) mbar_arrive(&empty[k]);
      // transposed butterfly within each half-warp (as k_spmv_cf with S = 16)
      const bool h1 = (t & 8) != 0, h2 = (t & 4) != 0;
      F2 k0 = h1 ? a[2] : a[0], k1 = h1 ? a[3] : a[1];
      k0 = f2_add(k0, f2_shfl(h1 ? a[0] : a[2], 8));
      k1 = f2_add(k1, f2_shfl(h1 ? a[1] : a[3], 8));
      F2 kk = h2 ? k1 : k0;
      kk = f2_add(kk, f2_shfl(h2 ? k0 : k1, 4));
      kk = f2_add(kk, f2_shfl(kk, 2));
      kk = f2_add(kk, f2_shfl(kk, 1));
      const int r = (h1 ? 2 : 0) + (h2 ? 1 : 0);
      // rows of both halves: half 0's d0 rows, then half 1's
      const int d0 = __shfl_sync(0xffffffffu, d, 0), d1 = __shfl_sync(0xffffffffu, d, 16);
      if (count + d0 + d1 > 32) flush();
      if ((t & 3) == 0 && r < d) {
        o_sc[count + (half ? d0 : 0) + r] = make_float2(kk.s, kk.c);
        o_eq[count + (half ? d0 : 0) + r] = dd.x + r;
      }
      count += d0 + d1;
    }
    flush();
  }
  if (MODE != 0) {
    double in[1] = {dsum}, tot[1];
    if (grid_reduce<1>(in, partial, counter, tot) && threadIdx.x == 0) {
      if (MODE == 1) {
        ks->pq = tot[0];
        ks->alpha = ks->d / tot[0];
      } else {
        ks->alpha = fabs(tot[0]) * (1.0 / (ks->beta * ks->beta));
      }
    }
  }
}

// FP64 panel values (rows of W) -> node records (layout in CompVals): one
// warp per node, coalesced on both sides.  hi = fl32(v), qb = 128 +
// round((v - hi) / hi * 2^31) clamped to [1, 255]; pad columns get hi = 0,
// qb = 128 and repeat the last column index.
__global__ void __launch_bounds__(256)
    k_split_records(PanelView P, const double* __restrict__ val, uint8_t* __restrict__ rec,
                    const int64_t* __restrict__ rec_off) {
  const int lane = threadIdx.x & 31;
  const int nwarp = (int)((gridDim.x * blockDim.x) >> 5);
  for (int k = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); k < P.nact; k += nwarp) {
    const int d = P.d[k], W = P.W[k], Wp = (W + 3) & ~3;
    const double* v = val + P.val_off[k];
    uint8_t* base = rec + rec_off[k];
    float* hi = reinterpret_cast<float*>(base);
    uint8_t* qb = base + 4 * d * Wp;
    const int qpad = (d * Wp + 15) & ~15;
    int32_t* cols = reinterpret_cast<int32_t*>(base + 4 * d * Wp + qpad);
    for (int r = 0; r < d; ++r)
      for (int c = lane; c < Wp; c += 32) {
        float h = 0.f, q = 0.f;
        if (c < W) {
          const double a = v[(size_t)r * W + c];
          h = float(a);
          // a - h is exact in FP64; the quotient in FP32 moves q by < 1e-5
          if (h != 0.f && isfinite(h)) q = rintf(float(a - double(h)) / h * 2147483648.0f);
        }
        hi[r * Wp + c] = h;
        qb[r * Wp + c] = (uint8_t)(128 + (int)fminf(fmaxf(q, -127.f), 127.f));
      }
    for (int c = d * Wp + lane; c < qpad; c += 32) qb[c] = 128;
    const int32_t* src = P.cols + P.col_off[k];
    for (int c = lane; c < Wp; c += 32) cols[c] = src[c < W ? c : W - 1];
  }
}

// FP64 panel values -> (hi = fl32(v), q = round((v - hi) / hi * 2^31)),
// |q| clamped to 127 (a tie at the rounding bound costs one unit, 2^-31).
__global__ void k_split_values(int64_t n, const double* __restrict__ v, float* __restrict__ hi,
                               int8_t* __restrict__ lo) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double a = v[i];
    const float h = float(a);
    hi[i] = h;
    // a - h is exact in FP64; the quotient is formed in FP32 (its 2^-24
    // relative error moves q by less than 1e-5), which keeps the FP64 pipe,
    // 1/64 of the FP32 rate on this part, to two operations per value
    float q = 0.f;
    if (h != 0.f && isfinite(h)) q = rintf(float(a - double(h)) / h * 2147483648.0f);
    lo[i] = (int8_t)fminf(fmaxf(q, -127.f), 127.f);
  }
}

__global__ void k_split_pair(int n, const double* __restrict__ v, float2* __restrict__ pr) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    split_store(v[i], pr, i);
}

// PCG start on the compensated operator: x = 0, r = b, z = m r, p = z (with
// its FP32 pair), d = (r, z); conv = tol sqrt|d| as in pcg, or conv_abs when
// positive (a refinement sweep aims at the first sweep's absolute target).
__global__ void __launch_bounds__(256)
    k_pcgc_init(int n, const double* __restrict__ b, const double* __restrict__ m,
                double* __restrict__ r, double* __restrict__ z, double* __restrict__ p,
                float2* __restrict__ pc, double* __restrict__ x,
                KrylovScalars* ks, double tol, double conv_abs, int maxit, double* partial,
                unsigned* counter) {
  double acc = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double bi = b[i], zi = bi * m[i];
    x[i] = 0.0;
    r[i] = bi;
    z[i] = zi;
    p[i] = zi;
    split_store(zi, pc, i);
    acc += bi * zi;
  }
  double in[1] = {acc}, tot[1];
  if (grid_reduce<1>(in, partial, counter, tot) && threadIdx.x == 0) {
    ks->d = tot[0];
    ks->bmb = tot[0];
    ks->conv = conv_abs > 0.0 ? conv_abs : tol * sqrt(fabs(tot[0]));
    ks->done = 0;
    ks->conv_flag = 0;
    ks->iter = 0;
    ks->maxit = maxit;
  }
}

__global__ void __launch_bounds__(256)
    k_pcgc_dir(int n, const double* __restrict__ z, double* __restrict__ p,
               float2* __restrict__ pc, KrylovScalars* ks) {
  if (krylov_skip(ks, false)) return;
  const double beta = ks->beta;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double pi = __ldcs(&z[i]) + beta * __ldcs(&p[i]);
    __stcs(&p[i], pi);
    split_store(pi, pc, i);  // the product's operand: kept in L2
  }
}

// Residual replacement in the PCG on the compensated operator (van der Vorst
// and Ye, "Residual replacement strategies for Krylov subspace iterative
// methods for the convergence of true residuals", SIAM J. Sci. Comput. 22,
// 2000): the recursive residual, updated with the compensated products,
// drifts from b - A x by the operator's error times the change of x; it is
// replaced by r = b - q (q = A x by the FP64 operator), z = m r,
// d = (r, z), while x and the search direction p are kept, so the Krylov
// iteration goes on instead of restarting.  The flags are re-decided from
// the replaced residual: converged only when it meets pcg's test.
__global__ void __launch_bounds__(256)
    k_pcgc_replace(int n, const double* __restrict__ b, const double* __restrict__ q,
                   const double* __restrict__ m, double* __restrict__ r,
                   double* __restrict__ z, KrylovScalars* ks, double* partial,
                   unsigned* counter) {
  double acc = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double ri = b[i] - q[i];
    const double zi = ri * m[i];
    r[i] = ri;
    z[i] = zi;
    acc += ri * zi;
  }
  double in[1] = {acc}, tot[1];
  if (grid_reduce<1>(in, partial, counter, tot) && threadIdx.x == 0) {
    const double di = tot[0];
    ks->d = di;
    ks->done = 0;
    if (sqrt(fabs(di)) < ks->conv) ks->conv_flag = 1;
    else if (!isfinite(di)) ks->conv_flag = 3;
    else if (ks->iter >= ks->maxit) ks->conv_flag = 2;
    else ks->conv_flag = 0;
  }
}

// The FP64 outer residual of the refinement: r = b - q (q = A x by the FP64
// operator) and out = (r, m r), with |m| when absval.
__global__ void __launch_bounds__(256)
    k_true_residual(int n, const double* __restrict__ b, const double* __restrict__ q,
                    const double* __restrict__ m, int absval, double* __restrict__ r,
                    double* out, double* partial, unsigned* counter) {
  double acc = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double ri = b[i] - q[i];
    r[i] = ri;
    acc += ri * ri * (absval == 2 ? 1.0 : absval ? fabs(m[i]) : m[i]);
  }
  double in[1] = {acc}, tot[1];
  if (grid_reduce<1>(in, partial, counter, tot) && threadIdx.x == 0) out[0] = tot[0];
}

// ---- rpsqmr (Iters.f:6100-6439) ---------------------------------------------
// Symmetric QMR, diagonal preconditioner on the right.  Vectors: q = V.p
// (direction, the SpMV operand), t = V.q (A q, then M r), r = V.r,
// d = V.z, x = V.x.  Scalars: ks->d = rho, ks->pq = sigma (written by the
// SpMV), ks->normr = tau, ks->neta = v(j-1), ks->t1/t2 the d-update
// coefficients, ks->ro1 = ||r||.  Breakdowns (sigma = 0, rho = 0: stop_mef
// in the reference) set conv_flag 3; maxit sets 2 (fsqmr: the reference then
// switches to GMRES(l)).

// x = 0, r = b (- A 0), q = M r, d = 0; conv = tol ||b||, tau = ||r||,
// rho = (r, q)
// qc (compensated operator): the FP32 pair of q as well; conv_abs > 0
// replaces tol ||b|| (a correction sweep of the refinement aims at the
// original target)
__global__ void __launch_bounds__(256)
    k_sqmr_init(int n, const double* __restrict__ b, const double* __restrict__ m,
                double* __restrict__ r, double* __restrict__ q, double* __restrict__ dv,
                double* __restrict__ x, float2* __restrict__ qc, KrylovScalars* ks, double tol,
                double conv_abs, int maxit, double* partial, unsigned* counter) {
  double bb = 0.0, rq = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double bi = b[i];
    x[i] = 0.0;
    r[i] = bi;
    const double qi = bi * m[i];
    q[i] = qi;
    if (qc) split_store(qi, qc, i);
    dv[i] = 0.0;
    bb += bi * bi;
    rq += bi * qi;
  }
  double in[2] = {bb, rq}, tot[2];
  if (grid_reduce<2>(in, partial, counter, tot) && threadIdx.x == 0) {
    ks->conv = conv_abs > 0.0 ? conv_abs : tol * sqrt(fabs(tot[0]));
    ks->normr = sqrt(tot[0]);
    ks->d = tot[1];
    ks->neta = 0.0;
    ks->ro1 = sqrt(tot[0]);
    ks->done = 0;
    ks->conv_flag = 0;
    ks->iter = 0;
    ks->maxit = maxit;
  }
}

// r -= alpha t; v = ||r|| / tau, c = 1 / sqrt(1 + v^2), tau = tau v c,
// the d-update coefficients c^2 v(j-1)^2 and c^2 alpha; test ||r|| < conv
__global__ void __launch_bounds__(256)
    k_sqmr_r(int n, double* __restrict__ r, const double* __restrict__ t, KrylovScalars* ks,
             double* partial, unsigned* counter) {
  if (krylov_skip(ks, false)) return;
  const double alpha = ks->alpha;
  double acc = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double ri = r[i] - alpha * t[i];
    r[i] = ri;
    acc += ri * ri;
  }
  double in[1] = {acc}, tot[1];
  if (grid_reduce<1>(in, partial, counter, tot) && threadIdx.x == 0) {
    const double nr = sqrt(tot[0]);
    const double vn = nr / ks->normr;
    const double cn = 1.0 / sqrt(1.0 + vn * vn);
    ks->normr = ks->normr * vn * cn;
    ks->t1 = cn * cn * ks->neta * ks->neta;
    ks->t2 = cn * cn * alpha;
    ks->neta = vn;
    ks->ro1 = nr;
    ks->iter += 1;
    if (ks->pq == 0.0 || !isfinite(alpha)) ks->conv_flag = 3;
    else if (nr < ks->conv) ks->conv_flag = 1;
    else if (!isfinite(nr)) ks->conv_flag = 3;
    else if (ks->iter >= ks->maxit) ks->conv_flag = 2;
  }
}

// d = c^2 v(j-1)^2 d + c^2 alpha q, x += d, t = M r; beta = (r, t) / rho,
// rho = (r, t)
__global__ void __launch_bounds__(256)
    k_sqmr_x(int n, double* __restrict__ dv, const double* __restrict__ q,
             double* __restrict__ x, const double* __restrict__ r,
             const double* __restrict__ m, double* __restrict__ t, KrylovScalars* ks,
             double* partial, unsigned* counter) {
  if (krylov_skip(ks, false)) return;
  const double t1 = ks->t1, t2 = ks->t2;
  double acc = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double di = t1 * dv[i] + t2 * q[i];
    dv[i] = di;
    x[i] = x[i] + di;
    const double ti = r[i] * m[i];
    t[i] = ti;
    acc += r[i] * ti;
  }
  double in[1] = {acc}, tot[1];
  if (grid_reduce<1>(in, partial, counter, tot) && threadIdx.x == 0) {
    if (ks->d == 0.0) {
      ks->conv_flag = 3;
    } else {
      ks->beta = tot[0] / ks->d;
      ks->d = tot[0];
    }
  }
}

// q = t + beta q
__global__ void __launch_bounds__(256)
    k_sqmr_dir(int n, const double* __restrict__ t, double* __restrict__ q,
               float2* __restrict__ qc, KrylovScalars* ks) {
  if (krylov_skip(ks, false)) return;
  const double beta = ks->beta;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double qi = t[i] + beta * q[i];
    q[i] = qi;
    if (qc) split_store(qi, qc, i);
  }
}

// ---- reference CSRD layout --------------------------------------------------
// y = (D + L + L^T) x for the lower CSR of Matvec.f:1504-1598 (1-based ia,
// ja); the transposed part is scattered with FP64 atomics.  y must be zero.
__global__ void __launch_bounds__(256)
    k_csrd_spmv(int neq, const int64_t* __restrict__ ia, const int32_t* __restrict__ ja,
                const double* __restrict__ ad, const double* __restrict__ al,
                const double* __restrict__ x, double* __restrict__ y) {
  const int lane = threadIdx.x & 31;
  const int nw = (int)((gridDim.x * blockDim.x) >> 5);
  for (int i = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); i < neq; i += nw) {
    const double xi = x[i];
    double t = 0.0;
    for (int64_t k = ia[i] - 1 + lane; k < ia[i + 1] - 1; k += 32) {
      const int j = ja[k] - 1;
      const double s = al[k];
      t += s * x[j];
      atomicAdd(&y[j], s * xi);
    }
    t = warp_sum(t);
    if (lane == 0) atomicAdd(&y[i], t + ad[i] * xi);
  }
}

// ---- small vector kernels --------------------------------------------------
__global__ void k_precond(int n, const double* __restrict__ ad, double* __restrict__ m,
                          int absval, int* zero_diag) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double a = ad[i];
    if (a == 0.0) atomicOr(zero_diag, 1);
    const double v = 1.0 / a;
    m[i] = absval ? fabs(v) : v;
  }
}

// Panel diagonal -> ad (the diagonal of the node's own block).
template <typename TV>
__global__ void k_diag(PanelView P, const TV* __restrict__ val, double* __restrict__ ad) {
  for (int node = blockIdx.x * blockDim.x + threadIdx.x; node < P.nact;
       node += gridDim.x * blockDim.x) {
    const int e0 = P.eq0[node], d = P.d[node], W = P.W[node], low = P.low[node];
    const TV* v = val + P.val_off[node];
    for (int r = 0; r < d; ++r) ad[e0 + r] = double(v[(int64_t)r * W + low + r]);
  }
}

// Residual norms of cal_residuo_pm: sum of squares of b over displacement
// and pressure equations (stop_crit 2) and over all (stop_crit 1).
__global__ void __launch_bounds__(256)
    k_resnorms(int n, const double* __restrict__ b, const int32_t* __restrict__ kind,
               double* out, double* partial, unsigned* counter) {
  double au = 0.0, ap = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double bi = b[i];
    if (kind[i]) ap += bi * bi;
    else au += bi * bi;
  }
  double in[2] = {au, ap}, tot[2];
  if (grid_reduce<2>(in, partial, counter, tot) && threadIdx.x == 0) {
    out[0] = tot[0];
    out[1] = tot[1];
  }
}

// sum |m_i| r_i^2 (the refinement loop's residual norm)
__global__ void __launch_bounds__(256)
    k_wnorm2(int n, const double* __restrict__ r, const double* __restrict__ m, double* out,
             double* partial, unsigned* counter) {
  double acc = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    acc += fabs(m[i]) * r[i] * r[i];
  double in[1] = {acc}, tot[1];
  if (grid_reduce<1>(in, partial, counter, tot) && threadIdx.x == 0) out[0] = tot[0];
}

__global__ void k_axpy_into(int n, double* __restrict__ y, const double* __restrict__ x,
                            double a) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    y[i] = y[i] + a * x[i];
}

__global__ void k_sub(int n, double* __restrict__ y, const double* __restrict__ a,
                      const double* __restrict__ b) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    y[i] = a[i] - b[i];
}

// FP64 panel values -> FP32 copy (PM_FP32_REFINE with FP64 assembly).
__global__ void k_to_f32(int64_t n, const double* __restrict__ a, float* __restrict__ b) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    b[i] = float(a[i]);
}

}  // namespace

int vec_grid(int n) {
  int g = (n + 255) / 256;
  return g < 1 ? 1 : (g > kRedBlocks ? kRedBlocks : g);
}

cudaError_t spmv(const PanelView& P, const double* val64, const double* x, double* y,
                 int mode, KrylovScalars* ks, double* partial, unsigned* counter,
                 cudaStream_t s) {
  // 32 nodes per CTA (8 warps of 4 sub-warps), at most kRedBlocks CTAs: a
  // small mesh launches only the CTAs it fills, and its fused dot sums that
  // many partials
  const int grid = std::max(1, std::min(kRedBlocks, (P.nact + 31) / 32));
  switch (mode) {
    case 0: k_spmv<double, 0><<<grid, 256, 0, s>>>(P, val64, x, y, ks, partial, counter); break;
    case 1: k_spmv<double, 1><<<grid, 256, 0, s>>>(P, val64, x, y, ks, partial, counter); break;
    case 2: k_spmv<double, 2><<<grid, 256, 0, s>>>(P, val64, x, y, ks, partial, counter); break;
    default: k_spmv<double, 3><<<grid, 256, 0, s>>>(P, val64, x, y, ks, partial, counter); break;
  }
  return cudaGetLastError();
}

cudaError_t pcgm_init(int n, const double* b, const double* m, KrylovVecs& V,
                      KrylovVecs32& V32, KrylovScalars* ks, double tol, int maxit,
                      double* partial, unsigned* counter, cudaStream_t s) {
  k_pcgm_init<<<vec_grid(n), 256, 0, s>>>(n, b, m, V.r, V.z, V.p, V32.p, V.x, ks, tol, maxit,
                                           partial, counter);
  return cudaGetLastError();
}

cudaError_t pcgm_iteration(const PanelView& P, const float* val32, int n, const double* m,
                           KrylovVecs& V, KrylovVecs32& V32, KrylovScalars* ks,
                           double* partial, unsigned* counter, cudaStream_t s) {
  k_spmv<float, 4><<<kRedBlocks, 256, 0, s>>>(P, val32, V32.p, V32.q, ks, partial, counter,
                                               V.p);
  k_pcgm_update<<<vec_grid(n), 256, 0, s>>>(n, V.x, V.p, V.r, V32.q, m, V.z, ks, partial,
                                             counter);
  k_pcgm_dir<<<vec_grid(n), 256, 0, s>>>(n, V.z, V.p, V32.p, ks);
  return cudaGetLastError();
}

cudaError_t pcg_init(int n, const double* b, const double* m, KrylovVecs& V,
                     KrylovScalars* ks, double tol, int maxit, double* partial,
                     unsigned* counter, cudaStream_t s) {
  k_pcg_init<<<vec_grid(n), 256, 0, s>>>(n, b, m, V.r, V.z, V.p, V.x, ks, tol, maxit,
                                          partial, counter);
  return cudaGetLastError();
}

cudaError_t pcg_iteration(const PanelView& P, const double* val64, int n, const double* m,
                          KrylovVecs& V, KrylovScalars* ks, double* partial,
                          unsigned* counter, cudaStream_t s) {
  cudaError_t e = spmv(P, val64, V.p, V.q, 1, ks, partial, counter, s);
  if (e != cudaSuccess) return e;
  k_pcg_update<<<vec_grid(n), 256, 0, s>>>(n, V.x, V.p, V.r, V.q, m, V.z, ks, partial,
                                            counter);
  k_pcg_dir<<<vec_grid(n), 256, 0, s>>>(n, V.z, V.p, ks);
  return cudaGetLastError();
}

cudaError_t sqmr_init(int n, const double* b, const double* m, KrylovVecs& V, float2* qc,
                      KrylovScalars* ks, double tol, double conv_abs, int maxit,
                      double* partial, unsigned* counter, cudaStream_t s) {
  k_sqmr_init<<<vec_grid(n), 256, 0, s>>>(n, b, m, V.r, V.p, V.z, V.x, qc, ks, tol, conv_abs,
                                           maxit, partial, counter);
  return cudaGetLastError();
}

cudaError_t sqmr_iteration(const PanelView& P, const double* val64, int n, const double* m,
                           KrylovVecs& V, KrylovScalars* ks, double* partial,
                           unsigned* counter, cudaStream_t s) {
  // t = A q with sigma = (q, t) and alpha = rho / sigma fused (PCG's mode)
  cudaError_t e = spmv(P, val64, V.p, V.q, 1, ks, partial, counter, s);
  if (e != cudaSuccess) return e;
  k_sqmr_r<<<vec_grid(n), 256, 0, s>>>(n, V.r, V.q, ks, partial, counter);
  k_sqmr_x<<<vec_grid(n), 256, 0, s>>>(n, V.z, V.p, V.x, V.r, m, V.q, ks, partial, counter);
  k_sqmr_dir<<<vec_grid(n), 256, 0, s>>>(n, V.q, V.p, nullptr, ks);
  return cudaGetLastError();
}

cudaError_t minres_conv(int n, const double* b, const double* m, KrylovScalars* ks,
                        double tol, double* partial, unsigned* counter, cudaStream_t s) {
  k_minres_conv<<<vec_grid(n), 256, 0, s>>>(n, b, m, ks, tol, partial, counter);
  return cudaGetLastError();
}

cudaError_t minres_start(const PanelView& P, const double* val64, int n, const double* b,
                         const double* m, KrylovVecs& V, const KrylovVecs32* pair,
                         KrylovScalars* ks, int maxit, bool zero_x, double* partial,
                         unsigned* counter, cudaStream_t s) {
  if (zero_x) {
    cudaMemsetAsync(V.x, 0, sizeof(double) * n, s);
    cudaMemsetAsync(V.q, 0, sizeof(double) * n, s);
  } else {
    cudaError_t e = spmv(P, val64, V.x, V.q, 0, ks, partial, counter, s);
    if (e != cudaSuccess) return e;
  }
  k_minres_start<<<vec_grid(n), 256, 0, s>>>(n, b, V.q, m, V.v, V.v0, V.w0, V.w00, V.z0,
                                              ks, maxit, partial, counter,
                                              pair ? pair->c : nullptr);
  return cudaGetLastError();
}

cudaError_t minres_iteration(const PanelView& P, const double* val64, int n, const double* m,
                             KrylovVecs& V, KrylovScalars* ks, double* partial,
                             unsigned* counter, cudaStream_t s) {
  cudaError_t e = spmv(P, val64, V.z0, V.p, 2, ks, partial, counter, s);
  if (e != cudaSuccess) return e;
  k_minres_lanczos<<<vec_grid(n), 256, 0, s>>>(n, V.p, V.v, V.v0, m, V.z, ks, partial,
                                                counter, nullptr);
  k_minres_update<<<vec_grid(n), 256, 0, s>>>(n, V.x, V.z0, V.w0, V.w00, V.v0, V.v, V.p,
                                               V.z, ks);
  return cudaGetLastError();
}

cudaError_t csrd_spmv(int neq, const int64_t* ia, const int32_t* ja, const double* ad,
                      const double* al, const double* x, double* y, cudaStream_t s) {
  cudaMemsetAsync(y, 0, sizeof(double) * neq, s);
  int grid = (neq + 7) / 8;
  if (grid > 8 * kRedBlocks) grid = 8 * kRedBlocks;
  if (grid < 1) grid = 1;
  k_csrd_spmv<<<grid, 256, 0, s>>>(neq, ia, ja, ad, al, x, y);
  return cudaGetLastError();
}

cudaError_t precond(int n, const double* ad, double* m, int absval, int* zero_diag,
                    cudaStream_t s) {
  k_precond<<<vec_grid(n), 256, 0, s>>>(n, ad, m, absval, zero_diag);
  return cudaGetLastError();
}

cudaError_t panel_diag(const PanelView& P, const double* val64, const float* val32,
                       double* ad, cudaStream_t s) {
  const int g = vec_grid(P.nact);
  if (val32) k_diag<float><<<g, 256, 0, s>>>(P, val32, ad);
  else k_diag<double><<<g, 256, 0, s>>>(P, val64, ad);
  return cudaGetLastError();
}

cudaError_t resnorms(int n, const double* b, const int32_t* kind, double* out,
                     double* partial, unsigned* counter, cudaStream_t s) {
  k_resnorms<<<vec_grid(n), 256, 0, s>>>(n, b, kind, out, partial, counter);
  return cudaGetLastError();
}

cudaError_t wnorm2(int n, const double* r, const double* m, double* out, double* partial,
                   unsigned* counter, cudaStream_t s) {
  k_wnorm2<<<vec_grid(n), 256, 0, s>>>(n, r, m, out, partial, counter);
  return cudaGetLastError();
}

cudaError_t axpy_into(int n, double* y, const double* x, double a, cudaStream_t s) {
  k_axpy_into<<<vec_grid(n), 256, 0, s>>>(n, y, x, a);
  return cudaGetLastError();
}

cudaError_t vsub(int n, double* y, const double* a, const double* b, cudaStream_t s) {
  k_sub<<<vec_grid(n), 256, 0, s>>>(n, y, a, b);
  return cudaGetLastError();
}

cudaError_t to_f32(int64_t n, const double* a, float* b, cudaStream_t s) {
  int64_t g = (n + 255) / 256;
  if (g > 8 * kRedBlocks) g = 8 * kRedBlocks;
  k_to_f32<<<(int)g, 256, 0, s>>>(n, a, b);
  return cudaGetLastError();
}

// ---- compensated operator launchers ------------------------------------------
cudaError_t split_values(int64_t n, const double* v, float* hi, int8_t* lo, cudaStream_t s) {
  int64_t g = (n + 255) / 256;
  if (g > 8 * kRedBlocks) g = 8 * kRedBlocks;
  if (g < 1) g = 1;
  k_split_values<<<(int)g, 256, 0, s>>>(n, v, hi, lo);
  return cudaGetLastError();
}

cudaError_t split_records(const PanelView& P, const double* v, CompVals C, cudaStream_t s) {
  k_split_records<<<8 * kRedBlocks, 256, 0, s>>>(P, v, const_cast<uint8_t*>(C.rec), C.rec_off);
  return cudaGetLastError();
}

cudaError_t split_pair(int n, const double* v, float2* pr, cudaStream_t s) {
  k_split_pair<<<vec_grid(n), 256, 0, s>>>(n, v, pr);
  return cudaGetLastError();
}

// One wave: the SMs times the CTAs of this variant resident per SM (at
// most kRedBlocks, the size of the reduction partials), so no CTA waits for
// a second, partly filled wave.
template <typename K>
int resident_grid(K kernel) {
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  }
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 256, 0) != cudaSuccess ||
      per_sm < 1)
    return kRedBlocks;
  const int g = sms * per_sm;
  return g < kRedBlocks ? g : kRedBlocks;
}

template <int MODE, int S, int U, bool PK = false, int MINB = 1>
void launch_cf(const PanelView& P, CompVals C, const float2* xp, double* y, const double* xd,
               KrylovScalars* ks, double* partial, unsigned* counter, cudaStream_t s) {
  static const int grid = resident_grid(k_spmv_cf<MODE, S, U, PK, MINB>);
  k_spmv_cf<MODE, S, U, PK, MINB><<<grid, 256, 0, s>>>(
      P, C.hi, C.lo, xp, y, xd, ks, partial, counter);
}

int cs_smem_bytes(int nstage, int stage_bytes) {
  return 128 + nstage * stage_bytes + (kCsWarps + 1) * 32 * (int)(sizeof(float2) + sizeof(int));
}

// Stages of the streamed kernel and CTAs per SM (*ctas); fewer than 2
// stages leaves the kernel out.  The
// launch attribute is the whole opt-in size less the static shared memory,
// so that meshes with different stage sizes can share the kernel.
cudaError_t cs_configure(int stage_bytes, int* nstage, int* ctas) {
  int dev = 0, optin = 0, per_sm = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess)
    e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e == cudaSuccess)
    e = cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
  if (e != cudaSuccess) return e;
  // the dynamic part is what is left after the static shared memory of the
  // kernel variants (the reduction scratch) and the per-CTA reservation
  int stat = 0;
  for (const void* k : {(const void*)k_spmv_cs<0>, (const void*)k_spmv_cs<1>,
                        (const void*)k_spmv_cs<2>}) {
    cudaFuncAttributes fa;
    if ((e = cudaFuncGetAttributes(&fa, k)) != cudaSuccess) return e;
    stat = std::max(stat, (int)fa.sharedSizeBytes);
  }
  const int dyn = optin - stat;
  const int reserve = 1024;
  *nstage = 0;
  *ctas = 0;
  // one CTA per SM with as many stages as fit (a deeper pipeline); two CTAs
  // of two stages where one CTA holds fewer than three
  int n = kCsMaxStages;
  while (n > 0 && cs_smem_bytes(n, stage_bytes) > dyn) --n;
  if (n >= 3) {
    *nstage = n;
    *ctas = 1;
  } else if (2 * (cs_smem_bytes(2, stage_bytes) + stat + reserve) <= per_sm) {
    *nstage = 2;
    *ctas = 2;
  } else if (n == 2) {
    *nstage = 2;
    *ctas = 1;
  }
  if (*nstage == 0) return cudaSuccess;
  static std::once_flag once;
  static cudaError_t ae = cudaSuccess;
  std::call_once(once, [&]() {
    for (const void* k : {(const void*)k_spmv_cs<0>, (const void*)k_spmv_cs<1>,
                          (const void*)k_spmv_cs<2>}) {
      if (ae == cudaSuccess)
        ae = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn);
      if (ae == cudaSuccess)
        ae = cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout,
                                  cudaSharedmemCarveoutMaxShared);
    }
  });
  if (ae != cudaSuccess) return ae;
  // two CTAs only if they are resident together
  if (*ctas == 2) {
    int nb = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_spmv_cs<1>, (kCsWarps + 1) * 32,
                                                      cs_smem_bytes(2, stage_bytes));
    if (e != cudaSuccess) return e;
    if (nb < 2) {
      int n = kCsMaxStages;
      while (n > 0 && cs_smem_bytes(n, stage_bytes) > dyn) --n;
      *nstage = n >= 2 ? n : 0;
      *ctas = n >= 2 ? 1 : 0;
    }
  }
  return cudaSuccess;
}

int ca_smem_bytes(int rec_max, int warps) {
  return warps * (2 * rec_max + 32 * (int)(sizeof(float2) + sizeof(int)));
}

// Warps per CTA of the record kernel: as many as the opt-in shared memory
// holds two records each for, at most 16; grid: the CTAs resident on all SMs.
cudaError_t ca_configure(int rec_max, int* warps, int* grid) {
  int dev = 0, smem = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  int wn = 16;
  while (wn > 0 && ca_smem_bytes(rec_max, wn) > smem) --wn;
  *warps = wn;
  *grid = 0;
  if (wn == 0) return cudaSuccess;
  const int bytes = ca_smem_bytes(rec_max, wn);
  e = cudaFuncSetAttribute(k_spmv_ca<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_spmv_ca<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_spmv_ca<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_spmv_ca<1>, wn * 32, bytes);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  *grid = sms * per_sm < kRedBlocks ? sms * per_sm : kRedBlocks;
  return cudaSuccess;
}

// C.shape = 10 * lanes-per-node code (0: 8, 1: 16, 2: 32) + columns per trip,
// or kCaShape for the record kernel
template <int MODE>
void launch_spmv_cf(const PanelView& P, CompVals C, const float2* xp, double* y,
                    const double* xd, KrylovScalars* ks, double* partial, unsigned* counter,
                    cudaStream_t s) {
  switch (C.shape) {
    case kCaShape:
      k_spmv_ca<MODE><<<C.ca_grid, C.ca_warps * 32, ca_smem_bytes(C.rec_max, C.ca_warps), s>>>(
          P, C, xp, y, xd, ks, partial, counter);
      break;
    case kCsShape:
      k_spmv_cs<MODE><<<C.cs_grid, (kCsWarps + 1) * 32,
                        cs_smem_bytes(C.cs_nstage, C.cs_stage_bytes), s>>>(P, C, xp, y, xd, ks,
                                                                           partial, counter);
      break;
    case 2: launch_cf<MODE, 8, 2>(P, C, xp, y, xd, ks, partial, counter, s); break;
    case 4: launch_cf<MODE, 8, 4>(P, C, xp, y, xd, ks, partial, counter, s); break;
    case 11: launch_cf<MODE, 16, 1>(P, C, xp, y, xd, ks, partial, counter, s); break;
    case 12: launch_cf<MODE, 16, 2>(P, C, xp, y, xd, ks, partial, counter, s); break;
    case 14: launch_cf<MODE, 16, 4>(P, C, xp, y, xd, ks, partial, counter, s); break;
    case 21: launch_cf<MODE, 32, 1>(P, C, xp, y, xd, ks, partial, counter, s); break;
    case 22: launch_cf<MODE, 32, 2>(P, C, xp, y, xd, ks, partial, counter, s); break;
    case 24: launch_cf<MODE, 32, 4>(P, C, xp, y, xd, ks, partial, counter, s); break;
    case 104: launch_cf<MODE, 8, 4, true>(P, C, xp, y, xd, ks, partial, counter, s); break;
    case 112: launch_cf<MODE, 16, 2, true>(P, C, xp, y, xd, ks, partial, counter, s); break;
    case 114: launch_cf<MODE, 16, 4, true>(P, C, xp, y, xd, ks, partial, counter, s); break;
    case 124: launch_cf<MODE, 32, 4, true>(P, C, xp, y, xd, ks, partial, counter, s); break;
    case 214: launch_cf<MODE, 16, 4, false, 4>(P, C, xp, y, xd, ks, partial, counter, s); break;
    case 314: launch_cf<MODE, 16, 4, true, 3>(P, C, xp, y, xd, ks, partial, counter, s); break;
    case 312: launch_cf<MODE, 16, 2, true, 4>(P, C, xp, y, xd, ks, partial, counter, s); break;
    default: launch_cf<MODE, 8, 1>(P, C, xp, y, xd, ks, partial, counter, s); break;
  }
}

cudaError_t spmvc(const PanelView& P, CompVals C, const float2* xp, double* y, cudaStream_t s) {
  launch_spmv_cf<0>(P, C, xp, y, nullptr, nullptr, nullptr, nullptr, s);
  return cudaGetLastError();
}

cudaError_t spmvc_pcg(const PanelView& P, CompVals C, const float2* xp, double* y,
                      const double* xd, KrylovScalars* ks, double* partial, unsigned* counter,
                      cudaStream_t s) {
  launch_spmv_cf<1>(P, C, xp, y, xd, ks, partial, counter, s);
  return cudaGetLastError();
}

cudaError_t pcgc_init(int n, const double* b, const double* m, KrylovVecs& V,
                      KrylovVecs32& V32, KrylovScalars* ks, double tol, double conv_abs,
                      int maxit, double* partial, unsigned* counter, cudaStream_t s) {
  k_pcgc_init<<<vec_grid(n), 256, 0, s>>>(n, b, m, V.r, V.z, V.p, V32.c, V.x, ks, tol,
                                           conv_abs, maxit, partial, counter);
  return cudaGetLastError();
}

cudaError_t pcgc_iteration(const PanelView& P, CompVals C, int n, const double* m,
                           KrylovVecs& V, KrylovVecs32& V32, KrylovScalars* ks,
                           double* partial, unsigned* counter, cudaStream_t s) {
  launch_spmv_cf<1>(P, C, V32.c, V.q, V.p, ks, partial, counter, s);
  k_pcg_update<<<vec_grid(n), 256, 0, s>>>(n, V.x, V.p, V.r, V.q, m, V.z, ks, partial,
                                            counter);
  k_pcgc_dir<<<vec_grid(n), 256, 0, s>>>(n, V.z, V.p, V32.c, ks);
  return cudaGetLastError();
}

// rpsqmr on the compensated operator: the product of the FP32 pair of q
// (same fused sigma and alpha), the FP64 updates, and the direction writing
// the pair of the new q
cudaError_t sqmrc_iteration(const PanelView& P, CompVals C, int n, const double* m,
                            KrylovVecs& V, KrylovVecs32& V32, KrylovScalars* ks,
                            double* partial, unsigned* counter, cudaStream_t s) {
  launch_spmv_cf<1>(P, C, V32.c, V.q, V.p, ks, partial, counter, s);
  k_sqmr_r<<<vec_grid(n), 256, 0, s>>>(n, V.r, V.q, ks, partial, counter);
  k_sqmr_x<<<vec_grid(n), 256, 0, s>>>(n, V.z, V.p, V.x, V.r, m, V.q, ks, partial, counter);
  k_sqmr_dir<<<vec_grid(n), 256, 0, s>>>(n, V.q, V.p, V32.c, ks);
  return cudaGetLastError();
}

cudaError_t minresc_iteration(const PanelView& P, CompVals C, int n, const double* m,
                              KrylovVecs& V, KrylovVecs32& V32, KrylovScalars* ks,
                              double* partial, unsigned* counter, cudaStream_t s) {
  launch_spmv_cf<2>(P, C, V32.c, V.p, V.z0, ks, partial, counter, s);
  k_minres_lanczos<<<vec_grid(n), 256, 0, s>>>(n, V.p, V.v, V.v0, m, V.z, ks, partial,
                                                counter, V32.c);
  k_minres_update<<<vec_grid(n), 256, 0, s>>>(n, V.x, V.z0, V.w0, V.w00, V.v0, V.v, V.p,
                                               V.z, ks);
  return cudaGetLastError();
}

namespace {
__global__ void k_loop_start(int* trips, cudaGraphConditionalHandle cond) {
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    *trips = 0;
    cudaGraphSetConditional(cond, 1u);
  }
}

__global__ void k_loop_next(const KrylovScalars* ks, int* trips,
                            cudaGraphConditionalHandle cond, int iters_per_trip) {
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    const int t = ++*trips;
    const int cap = ks->maxit / iters_per_trip + 4;
    cudaGraphSetConditional(cond, (ks->conv_flag == 0 && t < cap) ? 1u : 0u);
  }
}
}  // namespace

cudaError_t loop_start(int* trips, cudaGraphConditionalHandle cond, cudaStream_t s) {
  k_loop_start<<<1, 32, 0, s>>>(trips, cond);
  return cudaGetLastError();
}

cudaError_t loop_next(const KrylovScalars* ks, int* trips, cudaGraphConditionalHandle cond,
                      int iters_per_trip, cudaStream_t s) {
  k_loop_next<<<1, 32, 0, s>>>(ks, trips, cond, iters_per_trip);
  return cudaGetLastError();
}

cudaError_t pcgc_replace(int n, const double* b, const double* q, const double* m,
                         KrylovVecs& V, KrylovScalars* ks, double* partial, unsigned* counter,
                         cudaStream_t s) {
  k_pcgc_replace<<<vec_grid(n), 256, 0, s>>>(n, b, q, m, V.r, V.z, ks, partial, counter);
  return cudaGetLastError();
}

cudaError_t true_residual(int n, const double* b, const double* q, const double* m, int absval,
                          double* r, double* out, double* partial, unsigned* counter,
                          cudaStream_t s) {
  k_true_residual<<<vec_grid(n), 256, 0, s>>>(n, b, q, m, absval, r, out, partial, counter);
  return cudaGetLastError();
}


// ---- solve without device allocation ---------------------------------------
// pm_pcg_csrd_noalloc: the diagonal-preconditioned PCG of pm_solve, on the
// reference CSRD arrays the caller already holds on the device, taking every
// scratch vector and reduction buffer from one fixed array compiled into the
// library.  It exists for callers that may not allocate device memory while
// they solve: a Fortran driver whose memory is owned by its own arena (the
// reference's Malloc.f style), code running inside a framework that has
// reserved the device memory pool, or a step that must not pay the latency
// of cudaMalloc.  The array is a file-scope __device__ symbol: every GPU that
// loads the library holds PM_NOALLOC_MAX_NEQ * 5 doubles plus the reduction
// buffers (about 10.5 MB) until the process exits.
namespace {

constexpr int kNoAllocMaxNeq = PM_NOALLOC_MAX_NEQ;
constexpr size_t kNoAllocVec = (size_t)kNoAllocMaxNeq;
// layout (doubles): m, r, z, p, q (kNoAllocVec each), partials (2 * kRedBlocks),
// solver scalars (KrylovScalars), counter + zero-diagonal flag
constexpr size_t kNoAllocPartial = 5 * kNoAllocVec;
constexpr size_t kNoAllocScalars = kNoAllocPartial + 2 * (size_t)kRedBlocks;
constexpr size_t kNoAllocFlags = kNoAllocScalars + 64;
constexpr size_t kNoAllocDoubles = kNoAllocFlags + 8;
static_assert(sizeof(KrylovScalars) <= 64 * sizeof(double), "scalars region too small");

static __device__ __align__(256) double g_noalloc_scratch[kNoAllocDoubles];

// Device address of g_noalloc_scratch per device, looked up once per device
// (cudaGetSymbolAddress with that device current).
constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mutex;
double* g_noalloc_ptr[kNoAllocMaxDevices] = {nullptr};

// alpha = d / (p, q) for the CSRD product q = A p
__global__ void __launch_bounds__(256)
    k_noalloc_alpha(int n, const double* __restrict__ p, const double* __restrict__ q,
                    KrylovScalars* ks, double* partial, unsigned* counter) {
  if (krylov_skip(ks, true)) return;
  double acc = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    acc += p[i] * q[i];
  double in[1] = {acc}, tot[1];
  if (grid_reduce<1>(in, partial, counter, tot) && threadIdx.x == 0) {
    ks->pq = tot[0];
    ks->alpha = ks->d / tot[0];
  }
}

// q = A p on the CSRD layout, skipped once the solve has converged
__global__ void __launch_bounds__(256)
    k_noalloc_csrd(int neq, const int64_t* __restrict__ ia, const int32_t* __restrict__ ja,
                   const double* __restrict__ ad, const double* __restrict__ al,
                   const double* __restrict__ x, double* __restrict__ y,
                   const KrylovScalars* ks) {
  if (ks->done || ks->conv_flag) return;
  const int lane = threadIdx.x & 31;
  const int nw = (int)((gridDim.x * blockDim.x) >> 5);
  for (int i = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); i < neq; i += nw) {
    const double xi = x[i];
    double t = 0.0;
    for (int64_t k = ia[i] - 1 + lane; k < ia[i + 1] - 1; k += 32) {
      const int j = ja[k] - 1;
      const double s = al[k];
      t += s * x[j];
      atomicAdd(&y[j], s * xi);
    }
    t = warp_sum(t);
    if (lane == 0) atomicAdd(&y[i], t + ad[i] * xi);
  }
}

__global__ void k_noalloc_zero(int n, double* __restrict__ y, const KrylovScalars* ks) {
  if (ks->done || ks->conv_flag) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    y[i] = 0.0;
}

}  // namespace

}  // namespace pm

extern "C" int pm_pcg_csrd_noalloc(int neq, const int64_t* d_ia, const int32_t* d_ja,
                                   const double* d_ad, const double* d_al, const double* d_b,
                                   double* d_x, double tol, int maxit, int* iters,
                                   void* stream) {
  using namespace pm;
  if (neq > kNoAllocMaxNeq) return PM_E_TOO_LARGE;
  if (neq <= 0 || !d_ia || !d_ja || !d_ad || !d_al || !d_b || !d_x || maxit < 1 || !(tol >= 0.0))
    return PM_E_ARG;
  // an error left by the caller's earlier launches is theirs: report it
  // before launching anything (without clearing it), so that errors of this
  // solve are not confused with it
  if (cudaPeekAtLastError() != cudaSuccess) return PM_E_CUDA;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNoAllocMaxDevices)
    return PM_E_CUDA;
  double* base = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev]) {
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return PM_E_CUDA;
      g_noalloc_ptr[dev] = static_cast<double*>(p);
    }
    base = g_noalloc_ptr[dev];
  }
  cudaStream_t s = (cudaStream_t)stream;
  double* m = base;
  KrylovVecs V{};
  V.x = d_x;
  V.r = base + kNoAllocVec;
  V.z = base + 2 * kNoAllocVec;
  V.p = base + 3 * kNoAllocVec;
  V.q = base + 4 * kNoAllocVec;
  double* partial = base + kNoAllocPartial;
  KrylovScalars* ks = reinterpret_cast<KrylovScalars*>(base + kNoAllocScalars);
  unsigned* counter = reinterpret_cast<unsigned*>(base + kNoAllocFlags);
  int* zero_diag = reinterpret_cast<int*>(base + kNoAllocFlags + 1);
  // the array keeps the previous call's contents: the counter and the flag
  // must start at zero; every vector is written before it is read
  if (cudaMemsetAsync(base + kNoAllocFlags, 0, 2 * sizeof(double), s) != cudaSuccess)
    return PM_E_CUDA;
  const int g = vec_grid(neq);
  k_precond<<<g, 256, 0, s>>>(neq, d_ad, m, 0, zero_diag);
  k_pcg_init<<<g, 256, 0, s>>>(neq, d_b, m, V.r, V.z, V.p, V.x, ks, tol, maxit, partial,
                                counter);
  if (cudaGetLastError() != cudaSuccess) return PM_E_CUDA;
  int zd = 0;
  if (cudaMemcpyAsync(&zd, zero_diag, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return PM_E_CUDA;
  if (zd) return PM_E_ZERO_DIAG;
  int sgrid = (neq + 7) / 8;
  if (sgrid > 8 * kRedBlocks) sgrid = 8 * kRedBlocks;
  KrylovScalars h{};
  for (;;) {
    for (int k = 0; k < 16; ++k) {
      k_noalloc_zero<<<g, 256, 0, s>>>(neq, V.q, ks);
      k_noalloc_csrd<<<sgrid, 256, 0, s>>>(neq, d_ia, d_ja, d_ad, d_al, V.p, V.q, ks);
      k_noalloc_alpha<<<g, 256, 0, s>>>(neq, V.p, V.q, ks, partial, counter);
      k_pcg_update<<<g, 256, 0, s>>>(neq, V.x, V.p, V.r, V.q, m, V.z, ks, partial, counter);
      k_pcg_dir<<<g, 256, 0, s>>>(neq, V.z, V.p, ks);
    }
    if (cudaGetLastError() != cudaSuccess) return PM_E_CUDA;
    if (cudaMemcpyAsync(&h, ks, sizeof(h), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      return PM_E_CUDA;
    if (h.conv_flag) break;
  }
  if (iters) *iters = h.iter;
  return h.conv_flag == 1 ? PM_OK : PM_E_NOCONV;
}
