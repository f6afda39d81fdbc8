// pm_loads.h -- scalar time loads of tload (Pload.f:220-377) at a node, for
// the device step (pload_pm) and for the deck reader's initial values
// (bound_nodalloads, Rdata.f:4067-4090).
#pragma once
#include <cmath>
#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

#include "../../include/poromec_gb300.h"

namespace pm {

// interpol (Interpolation.f:1-32): piecewise-linear table lookup, clamped
__host__ __device__ inline double load_interp(const double* xs, const double* ys, double xi,
                                              int n) {
  if (xi <= xs[0]) return ys[0];
  if (xi >= xs[n - 1]) return ys[n - 1];
  for (int i = 0; i < n - 1; ++i) {
    const double x1 = xs[i], x2 = xs[i + 1], y1 = ys[i], y2 = ys[i + 1];
    if (xi >= x1 && xi <= x2) return y1 + (y2 - y1) * (xi - x1) / (x2 - x1);
  }
  return 0.0;
}

// Scalar loads of tload (Pload.f:220-377) evaluated at a node.
__host__ __device__ inline double nodal_load(const int32_t* load, const double* fload, int maxt,
                                             int nc, double t, const double* x, double u,
                                             double gmod) {
  const int ty = load[3 * (nc - 1)];
  const int nparc = load[3 * (nc - 1) + 1];
  const int nt = load[3 * (nc - 1) + 2];
  const double* F = fload + (size_t)maxt * PM_NFLOAD * (nc - 1);
  auto col = [&](int k) { return F + (size_t)maxt * (k - 1); };
  const double DOISPI = 6.283185307;
  switch (ty) {
    case 1: return F[0];
    case 2: return F[0] + F[1] * t;
    case 3: return (F[0] - u) * col(2)[0];
    case 4:
    case 5: {
      double c = 0.0;
      for (int i = 1; i <= nparc; ++i) {
        const double a = col(i)[0], w = 1.0 / col(i)[1], t0 = col(i)[2];
        const double ti = fmax(t - t0, 0.0);
        c += a * (ty == 4 ? sin(DOISPI * w * ti) : cos(DOISPI * w * ti));
      }
      return c;
    }
    case 39:
    case 41:
    case 43: return load_interp(col(1), col(2), t, nt);
    case 42: {
      const double a = load_interp(col(1), col(2), t, nt), b = load_interp(col(1), col(3), t, nt);
      const double w = load_interp(col(1), col(4), t, nt), t0 = load_interp(col(1), col(5), t, nt);
      return t0 * (b + a * (w - x[2]) * gmod);
    }
    default: return 0.0;
  }
}

}  // namespace pm
