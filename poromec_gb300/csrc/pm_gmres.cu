// pm_gmres.cu -- vector kernels of GMRES(l) (gmres2, Iters.f:1411-1700).
//
// The Krylov basis g(:, 1..k+1) is one (k+1) x n column-major block in HBM.
// Modified Gram-Schmidt keeps the reference's order: for j = 1..i,
// beta_j = (w, g_j) on the current w, then w -= beta_j g_j.  Each MGS kernel
// does the update of step j and the dot product of step j+1 (or |w|^2 after
// the last step) in one pass, so a step reads w, g_j and g_(j+1) once.  The
// scalars land in a small device array that the host reads once per Arnoldi
// step; the (k+1) x k Hessenberg matrix, its Givens rotations and the back
// substitution are host work in the reference's formulas.
#include <cuda_runtime.h>

#include "pm_krylov.h"
#include "pm_reduce.h"

namespace pm {
namespace {

// g1 = (b - ax) m (ax null: x = 0); out[0] = (g1, g1)
__global__ void __launch_bounds__(256)
    k_gm_resid(int n, const double* __restrict__ b, const double* ax, const double* __restrict__ m,
               double* g1, double* out, double* partial, unsigned* counter) {
  double acc = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double v = (b[i] - (ax ? ax[i] : 0.0)) * m[i];
    g1[i] = v;
    acc += v * v;
  }
  double in[1] = {acc}, tot[1];
  if (grid_reduce<1>(in, partial, counter, tot) && threadIdx.x == 0) out[0] = tot[0];
}

__global__ void __launch_bounds__(256) k_gm_scale(int n, double* __restrict__ g, double sc) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    g[i] = g[i] * sc;
}

// w = (A g_i) m; out[0] = (w, w), out[1] = (w, g_1)
__global__ void __launch_bounds__(256)
    k_gm_first(int n, double* __restrict__ w, const double* __restrict__ m,
               const double* __restrict__ g1, double* out, double* partial, unsigned* counter) {
  double ww = 0.0, wg = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double v = w[i] * m[i];
    w[i] = v;
    ww += v * v;
    wg += v * g1[i];
  }
  double in[2] = {ww, wg}, tot[2];
  if (grid_reduce<2>(in, partial, counter, tot) && threadIdx.x == 0) {
    out[0] = tot[0];
    out[1] = tot[1];
  }
}

// w -= (*bin) g_j; *out = (w, gnext), or (w, w) when gnext is null
__global__ void __launch_bounds__(256)
    k_gm_mgs(int n, double* __restrict__ w, const double* __restrict__ gj,
             const double* __restrict__ gnext, const double* bin, double* out, double* partial,
             unsigned* counter) {
  const double beta = *bin;
  double acc = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double v = w[i] - beta * gj[i];
    w[i] = v;
    acc += v * (gnext ? gnext[i] : v);
  }
  double in[1] = {acc}, tot[1];
  if (grid_reduce<1>(in, partial, counter, tot) && threadIdx.x == 0) *out = tot[0];
}

// *out = (a, b)
__global__ void __launch_bounds__(256)
    k_gm_dot(int n, const double* __restrict__ a, const double* __restrict__ b, double* out,
             double* partial, unsigned* counter) {
  double acc = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    acc += a[i] * b[i];
  double in[1] = {acc}, tot[1];
  if (grid_reduce<1>(in, partial, counter, tot) && threadIdx.x == 0) *out = tot[0];
}

// x += sum_j y_j g_j, j = 1..ni in order for every entry (Iters.f:1590-1595)
__global__ void __launch_bounds__(256)
    k_gm_update(int n, double* __restrict__ x, const double* __restrict__ G,
                const double* __restrict__ y, int ni) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double xi = x[i];
    for (int j = 0; j < ni; ++j) xi = xi + y[j] * G[(size_t)j * n + i];
    x[i] = xi;
  }
}

}  // namespace

cudaError_t gm_resid(int n, const double* b, const double* ax, const double* m, double* g1,
                     double* out, double* partial, unsigned* counter, cudaStream_t s) {
  k_gm_resid<<<vec_grid(n), 256, 0, s>>>(n, b, ax, m, g1, out, partial, counter);
  return cudaGetLastError();
}

cudaError_t gm_scale(int n, double* g, double sc, cudaStream_t s) {
  k_gm_scale<<<vec_grid(n), 256, 0, s>>>(n, g, sc);
  return cudaGetLastError();
}

cudaError_t gm_first(int n, double* w, const double* m, const double* g1, double* out,
                     double* partial, unsigned* counter, cudaStream_t s) {
  k_gm_first<<<vec_grid(n), 256, 0, s>>>(n, w, m, g1, out, partial, counter);
  return cudaGetLastError();
}

cudaError_t gm_mgs(int n, double* w, const double* gj, const double* gnext, const double* bin,
                   double* out, double* partial, unsigned* counter, cudaStream_t s) {
  k_gm_mgs<<<vec_grid(n), 256, 0, s>>>(n, w, gj, gnext, bin, out, partial, counter);
  return cudaGetLastError();
}

cudaError_t gm_dot(int n, const double* a, const double* b, double* out, double* partial,
                   unsigned* counter, cudaStream_t s) {
  k_gm_dot<<<vec_grid(n), 256, 0, s>>>(n, a, b, out, partial, counter);
  return cudaGetLastError();
}

cudaError_t gm_update(int n, double* x, const double* G, const double* y, int ni,
                      cudaStream_t s) {
  k_gm_update<<<vec_grid(n), 256, 0, s>>>(n, x, G, y, ni);
  return cudaGetLastError();
}

}  // namespace pm
