// pm_elements.cu -- element kernels of the Biot hot path on sm_103a.
//
// One CTA per element (64 threads for hexa20, 32 for tetra10).  Phase 1 maps
// the integration points to threads: each thread builds the subparametric
// geometry of its point (vertex Jacobian, determinant, inverse; the
// quadratic derivatives mapped with that same inverse, as jacob3d_m does in
// Elmlib.f:2301-2396) into shared memory.  Phase 2 maps the element matrix
// (or vector) entries to threads and reduces over the points.
//
// The element matrix of elmt17_pm / elmt15_pm (Elmlib03.f:2022-2200,
// :258-434) is formed from node-pair blocks:
//   Kuu(i,j) = a [ b P_kl + c P_lk ]           (k != l)
//   Kuu(i,j) = a [ P_kk + c (tr P - P_kk) ]     (k == l)
//   P_kl     = sum_g w_g dN_i/dx_k dN_j/dx_l
//   Kpu(l,j) = -alpha sum_g w_g Np_l dN_j/dx_k,   Kup = Kpu^T
//   Kpp(l,m) = -sum_g w_g (Np_l Np_m / M + dt perm grad Np_l . grad Np_m)
// which is the reference's per-point 9-entry update regrouped (the same
// products, summed in a different order).  The blocks are added straight
// into the node panels; elements of one colour share no node, so the adds
// need no atomics.  The hexa's shape functions at its 64 points come from a
// table filled once per device (ensure_shape_tables); each point's values
// are scaled by sqrt(w_g) before the pair loops, so these need no w_g.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <type_traits>
#include <utility>
#include <vector>

#include "pm_internal.h"

namespace pm {
namespace {

// Gauss tables of the reference block data (Elmlib.f:3780-3962), digits as
// typed there.
__constant__ double cPG4[4] = {-.861136311594053, -.339981043584856,
                               .339981043584856, .861136311594053};
__constant__ double cWG4[4] = {.347854845137454, .652145154862546,
                               .652145154862546, .347854845137454};
__constant__ double cPG3[3] = {-.774596669241483, 0.0, .774596669241483};
__constant__ double cWG3[3] = {.555555555555556, .888888888888889,
                               .555555555555556};
__constant__ double cPRI4[4] = {0.58541020, 0.13819660, 0.13819660, 0.13819660};
__constant__ double cPSI4[4] = {0.13819660, 0.58541020, 0.13819660, 0.13819660};
__constant__ double cPTI4[4] = {0.13819660, 0.13819660, 0.58541020, 0.13819660};
__constant__ double cPRI2[3] = {.5, 0.0, .5};
__constant__ double cPSI2[3] = {.5, .5, 0.0};
__constant__ double cWF2 = .333333333333333;
constexpr double kDiv6 = 0.166666666666667;

__constant__ int cHexaFace[6][8] = {{1, 2, 3, 4, 9, 10, 11, 12},
                                    {5, 6, 7, 8, 13, 14, 15, 16},
                                    {1, 5, 6, 2, 17, 13, 18, 9},
                                    {4, 3, 7, 8, 11, 19, 15, 20},
                                    {1, 4, 8, 5, 12, 20, 16, 17},
                                    {2, 6, 7, 3, 18, 14, 19, 10}};
__constant__ int cTetraFace[4][6] = {{2, 3, 4, 8, 9, 10},
                                     {1, 4, 3, 7, 9, 6},
                                     {1, 2, 4, 5, 10, 7},
                                     {1, 3, 2, 6, 8, 5}};

template <bool HEXA>
struct ET;
template <>
struct ET<true> {
  static constexpr int NEN = 20, NV = 8, NGP = 64, NT = 64;
};
template <>
struct ET<false> {
  static constexpr int NEN = 10, NV = 4, NGP = 4, NT = 32;
};

// ---- shape functions (sfhexa8_m, sfhexa20_m, sftetra4, sftetra10) ---------
template <typename T>
__device__ __forceinline__ void sf_hexa8(T r, T s, T t, T* h, T* hr, T* hs,
                                         T* ht) {
  const T pR = 1 + r, pS = 1 + s, pT = 1 + t, mR = 1 - r, mS = 1 - s, mT = 1 - t;
  const T e = T(0.125);
  h[0] = pR * pS * pT * e; h[1] = mR * pS * pT * e; h[2] = mR * mS * pT * e;
  h[3] = pR * mS * pT * e; h[4] = pR * pS * mT * e; h[5] = mR * pS * mT * e;
  h[6] = mR * mS * mT * e; h[7] = pR * mS * mT * e;
  hr[0] = pS * pT * e; hr[1] = -pS * pT * e; hr[2] = -mS * pT * e; hr[3] = mS * pT * e;
  hr[4] = pS * mT * e; hr[5] = -pS * mT * e; hr[6] = -mS * mT * e; hr[7] = mS * mT * e;
  hs[0] = pR * pT * e; hs[1] = mR * pT * e; hs[2] = -mR * pT * e; hs[3] = -pR * pT * e;
  hs[4] = pR * mT * e; hs[5] = mR * mT * e; hs[6] = -mR * mT * e; hs[7] = -pR * mT * e;
  ht[0] = pR * pS * e; ht[1] = mR * pS * e; ht[2] = mR * mS * e; ht[3] = pR * mS * e;
  ht[4] = -pR * pS * e; ht[5] = -mR * pS * e; ht[6] = -mR * mS * e; ht[7] = -pR * mS * e;
}

template <typename T>
__device__ __forceinline__ void sf_hexa20_d(T r, T s, T t, T* hr, T* hs, T* ht) {
  const T pR = 1 + r, pS = 1 + s, pT = 1 + t, mR = 1 - r, mS = 1 - s, mT = 1 - t;
  const T mRr = 1 - r * r, mSs = 1 - s * s, mTt = 1 - t * t;
  const T e = T(0.125), q = T(0.25), hf = T(0.5);
  hr[0] = pS * pT * (2 * r + s + t - 1) * e;
  hr[1] = pS * pT * (2 * r - s - t + 1) * e;
  hr[2] = mS * pT * (2 * r + s - t + 1) * e;
  hr[3] = mS * pT * (2 * r - s + t - 1) * e;
  hr[4] = pS * mT * (2 * r + s - t - 1) * e;
  hr[5] = pS * mT * (2 * r - s + t + 1) * e;
  hr[6] = mS * mT * (2 * r + s + t + 1) * e;
  hr[7] = mS * mT * (2 * r - s - t - 1) * e;
  hr[8] = -r * pS * pT * hf; hr[9] = -mSs * pT * q; hr[10] = -r * mS * pT * hf;
  hr[11] = mSs * pT * q; hr[12] = -r * pS * mT * hf; hr[13] = -mSs * mT * q;
  hr[14] = -r * mS * mT * hf; hr[15] = mSs * mT * q; hr[16] = pS * mTt * q;
  hr[17] = -pS * mTt * q; hr[18] = -mS * mTt * q; hr[19] = mS * mTt * q;
  hs[0] = pR * pT * (r + 2 * s + t - 1) * e;
  hs[1] = mR * pT * (-r + 2 * s + t - 1) * e;
  hs[2] = mR * pT * (r + 2 * s - t + 1) * e;
  hs[3] = pR * pT * (-r + 2 * s - t + 1) * e;
  hs[4] = pR * mT * (r + 2 * s - t - 1) * e;
  hs[5] = mR * mT * (-r + 2 * s - t - 1) * e;
  hs[6] = mR * mT * (r + 2 * s + t + 1) * e;
  hs[7] = pR * mT * (-r + 2 * s + t + 1) * e;
  hs[8] = mRr * pT * q; hs[9] = -s * mR * pT * hf; hs[10] = -mRr * pT * q;
  hs[11] = -s * pR * pT * hf; hs[12] = mRr * mT * q; hs[13] = -s * mR * mT * hf;
  hs[14] = -mRr * mT * q; hs[15] = -s * pR * mT * hf; hs[16] = pR * mTt * q;
  hs[17] = mR * mTt * q; hs[18] = -mR * mTt * q; hs[19] = -pR * mTt * q;
  ht[0] = pR * pS * (r + s + 2 * t - 1) * e;
  ht[1] = mR * pS * (-r + s + 2 * t - 1) * e;
  ht[2] = mR * mS * (-r - s + 2 * t - 1) * e;
  ht[3] = pR * mS * (r - s + 2 * t - 1) * e;
  ht[4] = pR * pS * (-r - s + 2 * t + 1) * e;
  ht[5] = mR * pS * (r - s + 2 * t + 1) * e;
  ht[6] = mR * mS * (r + s + 2 * t + 1) * e;
  ht[7] = pR * mS * (-r + s + 2 * t + 1) * e;
  ht[8] = mRr * pS * q; ht[9] = mR * mSs * q; ht[10] = mRr * mS * q;
  ht[11] = pR * mSs * q; ht[12] = -mRr * pS * q; ht[13] = -mR * mSs * q;
  ht[14] = -mRr * mS * q; ht[15] = -pR * mSs * q; ht[16] = -t * pR * pS * hf;
  ht[17] = -t * mR * pS * hf; ht[18] = -t * mR * mS * hf; ht[19] = -t * pR * mS * hf;
}

template <typename T>
__device__ __forceinline__ void sf_hexa20_v(T r, T s, T t, T* h) {
  const T pR = 1 + r, pS = 1 + s, pT = 1 + t, mR = 1 - r, mS = 1 - s, mT = 1 - t;
  const T mRr = 1 - r * r, mSs = 1 - s * s, mTt = 1 - t * t;
  const T e = T(0.125), q = T(0.25);
  h[0] = pR * pS * pT * (r + s + t - 2) * e;
  h[1] = mR * pS * pT * (-r + s + t - 2) * e;
  h[2] = mR * mS * pT * (-r - s + t - 2) * e;
  h[3] = pR * mS * pT * (r - s + t - 2) * e;
  h[4] = pR * pS * mT * (r + s - t - 2) * e;
  h[5] = mR * pS * mT * (-r + s - t - 2) * e;
  h[6] = mR * mS * mT * (-r - s - t - 2) * e;
  h[7] = pR * mS * mT * (r - s - t - 2) * e;
  h[8] = mRr * pS * pT * q; h[9] = mR * mSs * pT * q; h[10] = mRr * mS * pT * q;
  h[11] = pR * mSs * pT * q; h[12] = mRr * pS * mT * q; h[13] = mR * mSs * mT * q;
  h[14] = mRr * mS * mT * q; h[15] = pR * mSs * mT * q; h[16] = pR * pS * mTt * q;
  h[17] = mR * pS * mTt * q; h[18] = mR * mS * mTt * q; h[19] = pR * mS * mTt * q;
}

template <typename T>
__device__ __forceinline__ void sf_tetra4(T r, T s, T t, T* h, T* hr, T* hs, T* ht) {
  h[0] = r; h[1] = s; h[2] = t; h[3] = 1 - r - s - t;
  hr[0] = 1; hr[1] = 0; hr[2] = 0; hr[3] = -1;
  hs[0] = 0; hs[1] = 1; hs[2] = 0; hs[3] = -1;
  ht[0] = 0; ht[1] = 0; ht[2] = 1; ht[3] = -1;
}

template <typename T>
__device__ __forceinline__ void sf_tetra10_d(T r, T s, T t, T* hr, T* hs, T* ht) {
  const T u = 1 - r - s - t;
  hr[0] = 4 * r - 1; hr[1] = 0; hr[2] = 0; hr[3] = 1 - 4 * u; hr[4] = 4 * s;
  hr[5] = 4 * t; hr[6] = 4 * (u - r); hr[7] = 0; hr[8] = -4 * t; hr[9] = -4 * s;
  hs[0] = 0; hs[1] = 4 * s - 1; hs[2] = 0; hs[3] = 1 - 4 * u; hs[4] = 4 * r;
  hs[5] = 0; hs[6] = -4 * r; hs[7] = 4 * t; hs[8] = -4 * t; hs[9] = 4 * (u - s);
  ht[0] = 0; ht[1] = 0; ht[2] = 4 * t - 1; ht[3] = 1 - 4 * u; ht[4] = 0;
  ht[5] = 4 * r; ht[6] = -4 * r; ht[7] = 4 * s; ht[8] = 4 * (u - t); ht[9] = -4 * s;
}

template <typename T>
__device__ __forceinline__ void sf_tetra10_v(T r, T s, T t, T* h) {
  const T u = 1 - r - s - t;
  h[0] = r * (2 * r - 1); h[1] = s * (2 * s - 1); h[2] = t * (2 * t - 1);
  h[3] = u * (2 * u - 1); h[4] = 4 * r * s; h[5] = 4 * r * t; h[6] = 4 * r * u;
  h[7] = 4 * s * t; h[8] = 4 * t * u; h[9] = 4 * s * u;
}

// Shared geometry of one element: per integration point the weight
// w = w_q det, the physical quadratic derivatives g[node][3], the linear
// functions and their physical derivatives.
template <bool HEXA, typename T>
struct Geo {
  static constexpr int NEN = ET<HEXA>::NEN, NV = ET<HEXA>::NV, NGP = ET<HEXA>::NGP;
  T w[NGP];
  T g[NGP][NEN][3];
  T hp[NGP][NV];
  T gp[NGP][NV][3];
  T xv[NV][3];
};

// Shape functions of the hexa at its 64 integration points are the same for
// every element: a table filled once per device by k_fill_shape_tables from
// the sf_* functions above, so its values are theirs bit for bit.  Row k
// holds one function at the 64 points, so a warp's loads are coalesced.
constexpr int kTabH8 = 0;     // rows 0..31: h, hr, hs, ht of sfhexa8 (8 each)
constexpr int kTabH20D = 32;  // rows 32..91: hr, hs, ht of sfhexa20 (20 each)
constexpr int kTabH20V = 92;  // rows 92..111: h of sfhexa20
constexpr int kTabRows = 112;
constexpr int kHexaGp = 64;
__device__ double gShapeHexa[kTabRows * kHexaGp];

__global__ void k_fill_shape_tables() {
  const int gq = threadIdx.x;
  if (gq >= kHexaGp) return;
  const int lz = gq >> 4, ly = (gq >> 2) & 3, lx = gq & 3;
  const double r = cPG4[lx], s = cPG4[ly], t = cPG4[lz];
  double h[8], hr[8], hs[8], ht[8], ur[20], us[20], ut[20], hv[20];
  sf_hexa8<double>(r, s, t, h, hr, hs, ht);
  sf_hexa20_d<double>(r, s, t, ur, us, ut);
  sf_hexa20_v<double>(r, s, t, hv);
  double* tb = gShapeHexa + gq;
  for (int k = 0; k < 8; ++k) {
    tb[(kTabH8 + k) * kHexaGp] = h[k];
    tb[(kTabH8 + 8 + k) * kHexaGp] = hr[k];
    tb[(kTabH8 + 16 + k) * kHexaGp] = hs[k];
    tb[(kTabH8 + 24 + k) * kHexaGp] = ht[k];
  }
  for (int k = 0; k < 20; ++k) {
    tb[(kTabH20D + k) * kHexaGp] = ur[k];
    tb[(kTabH20D + 20 + k) * kHexaGp] = us[k];
    tb[(kTabH20D + 40 + k) * kHexaGp] = ut[k];
    tb[(kTabH20V + k) * kHexaGp] = hv[k];
  }
}

// Integration point geometry (thread-per-point).  Returns false when the
// determinant is <= 1e-14, the condition jacob3d_m stops on.
template <bool HEXA, typename T>
__device__ bool point_geometry_rst(Geo<HEXA, T>& G, int gq, T r, T s, T t, T wq, T* huv);

// The hexa's point geometry from the shape tables: the Jacobian from the
// vertices, its inverse by one reciprocal of the determinant, and the
// physical derivatives, with the table rows streamed from L1.
template <typename T>
__device__ bool point_geometry_hexa_tab(Geo<true, T>& G, int gq, T* huv) {
  constexpr int NEN = 20, NV = 8;
  const double* tb = gShapeHexa + gq;
  auto tab = [tb](int row) { return T(__ldg(tb + row * kHexaGp)); };
  T J[3][3];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    T a0 = 0, a1 = 0, a2 = 0;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      const T xk = G.xv[k][j];
      a0 += tab(kTabH8 + 8 + k) * xk;
      a1 += tab(kTabH8 + 16 + k) * xk;
      a2 += tab(kTabH8 + 24 + k) * xk;
    }
    J[0][j] = a0; J[1][j] = a1; J[2][j] = a2;
  }
  const T det = J[0][0] * J[1][1] * J[2][2] + J[0][1] * J[1][2] * J[2][0] +
                J[0][2] * J[1][0] * J[2][1] - J[2][0] * J[1][1] * J[0][2] -
                J[1][0] * J[0][1] * J[2][2] - J[0][0] * J[2][1] * J[1][2];
  if (!(det > T(1.0e-14))) return false;
  const T rd = T(1) / det;
  T Ji[3][3];
  Ji[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) * rd;
  Ji[1][0] = -(J[1][0] * J[2][2] - J[1][2] * J[2][0]) * rd;
  Ji[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) * rd;
  Ji[0][1] = -(J[0][1] * J[2][2] - J[0][2] * J[2][1]) * rd;
  Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * rd;
  Ji[2][1] = -(J[0][0] * J[2][1] - J[0][1] * J[2][0]) * rd;
  Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * rd;
  Ji[1][2] = -(J[0][0] * J[1][2] - J[0][2] * J[1][0]) * rd;
  Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * rd;
  const int lz = gq >> 4, ly = (gq >> 2) & 3, lx = gq & 3;
  G.w[gq] = T(cWG4[lx] * cWG4[ly] * cWG4[lz]) * det;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    const T hr = tab(kTabH8 + 8 + k), hs = tab(kTabH8 + 16 + k), ht = tab(kTabH8 + 24 + k);
    G.hp[gq][k] = tab(kTabH8 + k);
    G.gp[gq][k][0] = Ji[0][0] * hr + Ji[0][1] * hs + Ji[0][2] * ht;
    G.gp[gq][k][1] = Ji[1][0] * hr + Ji[1][1] * hs + Ji[1][2] * ht;
    G.gp[gq][k][2] = Ji[2][0] * hr + Ji[2][1] * hs + Ji[2][2] * ht;
  }
#pragma unroll 4
  for (int k = 0; k < NEN; ++k) {
    const T ur = tab(kTabH20D + k), us = tab(kTabH20D + 20 + k), ut = tab(kTabH20D + 40 + k);
    G.g[gq][k][0] = Ji[0][0] * ur + Ji[0][1] * us + Ji[0][2] * ut;
    G.g[gq][k][1] = Ji[1][0] * ur + Ji[1][1] * us + Ji[1][2] * ut;
    G.g[gq][k][2] = Ji[2][0] * ur + Ji[2][1] * us + Ji[2][2] * ut;
  }
  if (huv)
    for (int k = 0; k < NEN; ++k) huv[k] = tab(kTabH20V + k);
  return true;
}

template <bool HEXA, typename T>
__device__ bool point_geometry(Geo<HEXA, T>& G, int gq, T* huv) {
  if constexpr (HEXA) {
    return point_geometry_hexa_tab<T>(G, gq, huv);
  } else {
    return point_geometry_rst<HEXA, T>(G, gq, T(cPRI4[gq]), T(cPSI4[gq]), T(cPTI4[gq]),
                                       T(0.25), huv);
  }
}

// The geometry of point (r, s, t) with quadrature weight wq into slot gq of G
// (slots are the integration points, or the vertices for isw 3).
template <bool HEXA, typename T>
__device__ bool point_geometry_rst(Geo<HEXA, T>& G, int gq, T r, T s, T t, T wq, T* huv) {
  constexpr int NEN = ET<HEXA>::NEN, NV = ET<HEXA>::NV;
  T h[NV], hr[NV], hs[NV], ht[NV];
  if (HEXA) sf_hexa8<T>(r, s, t, h, hr, hs, ht);
  else sf_tetra4<T>(r, s, t, h, hr, hs, ht);
  T J[3][3];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    T a0 = 0, a1 = 0, a2 = 0;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      const T xk = G.xv[k][j];
      a0 += hr[k] * xk; a1 += hs[k] * xk; a2 += ht[k] * xk;
    }
    J[0][j] = a0; J[1][j] = a1; J[2][j] = a2;
  }
  const T det = J[0][0] * J[1][1] * J[2][2] + J[0][1] * J[1][2] * J[2][0] +
                J[0][2] * J[1][0] * J[2][1] - J[2][0] * J[1][1] * J[0][2] -
                J[1][0] * J[0][1] * J[2][2] - J[0][0] * J[2][1] * J[1][2];
  if (!(det > T(1.0e-14))) return false;
  T Ji[3][3];
  Ji[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) / det;
  Ji[1][0] = -(J[1][0] * J[2][2] - J[1][2] * J[2][0]) / det;
  Ji[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) / det;
  Ji[0][1] = -(J[0][1] * J[2][2] - J[0][2] * J[2][1]) / det;
  Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det;
  Ji[2][1] = -(J[0][0] * J[2][1] - J[0][1] * J[2][0]) / det;
  Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;
  Ji[1][2] = -(J[0][0] * J[1][2] - J[0][2] * J[1][0]) / det;
  Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
  T w = wq * det;
  if (!HEXA) w = w * T(kDiv6);
  G.w[gq] = w;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    G.hp[gq][k] = h[k];
    G.gp[gq][k][0] = Ji[0][0] * hr[k] + Ji[0][1] * hs[k] + Ji[0][2] * ht[k];
    G.gp[gq][k][1] = Ji[1][0] * hr[k] + Ji[1][1] * hs[k] + Ji[1][2] * ht[k];
    G.gp[gq][k][2] = Ji[2][0] * hr[k] + Ji[2][1] * hs[k] + Ji[2][2] * ht[k];
  }
  T ur[NEN], us[NEN], ut[NEN];
  if (HEXA) sf_hexa20_d<T>(r, s, t, ur, us, ut);
  else sf_tetra10_d<T>(r, s, t, ur, us, ut);
#pragma unroll
  for (int k = 0; k < NEN; ++k) {
    G.g[gq][k][0] = Ji[0][0] * ur[k] + Ji[0][1] * us[k] + Ji[0][2] * ut[k];
    G.g[gq][k][1] = Ji[1][0] * ur[k] + Ji[1][1] * us[k] + Ji[1][2] * ut[k];
    G.g[gq][k][2] = Ji[2][0] * ur[k] + Ji[2][1] * us[k] + Ji[2][2] * ut[k];
  }
  if (huv) {
    if (HEXA) sf_hexa20_v<T>(r, s, t, huv);
    else sf_tetra10_v<T>(r, s, t, huv);
  }
  return true;
}

struct ElemCtx {
  int nodes[kMaxNen];
  int mat;
};

template <bool HEXA, typename T>
__device__ void load_element(const ElemLaunch& L, int el, ElemCtx& E,
                             Geo<HEXA, T>& G) {
  constexpr int NEN = ET<HEXA>::NEN, NV = ET<HEXA>::NV;
  const int32_t* ixe = L.ix + (size_t)(NEN + 1) * (el - 1);
  for (int k = threadIdx.x; k <= NEN; k += blockDim.x) {
    if (k < NEN) E.nodes[k] = ixe[k];
    else E.mat = ixe[NEN];
  }
  __syncthreads();
  for (int k = threadIdx.x; k < NV * 3; k += blockDim.x) {
    const int n = E.nodes[k / 3];
    G.xv[k / 3][k % 3] = T(L.x[(size_t)3 * (n - 1) + (k % 3)]);
  }
  __syncthreads();
}

// Equation of local dof k (0..3) of node n, 0 when prescribed/absent.
__device__ __forceinline__ int eq_of(const ElemLaunch& L, int n, int k) {
  return L.eq[(size_t)kNdf * (n - 1) + k];
}

template <typename T>
__device__ __forceinline__ void add_val(double* v64, float* v32, int64_t a, T v) {
  if (v64) v64[a] += double(v);
  else v32[a] += float(v);
}

// ---------------------------------------------------------------------------
// isw = 2, lhs: element matrix into the panels.
// ---------------------------------------------------------------------------
// The weight a pair loop still applies at point gq: none for the hexa, whose
// point values k_assemble_K scales by sqrt(w); w for the tetra.
template <bool HEXA, typename T>
__device__ __forceinline__ T pair_weight(const Geo<HEXA, T>& G, int gq) {
  if constexpr (HEXA) return T(1);
  else return G.w[gq];
}

template <bool HEXA, typename T>
struct SmK {
  static constexpr int NEN = ET<HEXA>::NEN, NV = ET<HEXA>::NV, NST = 3 * NEN + NV,
                       NSLOT = NEN + NV;
  Geo<HEXA, T> G;
  ElemCtx E;
  int sEq[NEN][kNdf];  // equation numbers of the local dofs
  int sE0[NEN];        // first equation of each node
  int sFail;
  // with RHS: the element's dof values, and (tetra) the contribution slots;
  // the hexa's slots reuse G.g once the pair loops have read it
  double ul[NST];
  double Cx[HEXA ? 1 : NST * NSLOT];
};

// Element matrix into the panels; with RHS also b -= K_e u_e from the same
// blocks (p = s.u, the product the reference forms in lku for isw 2 with
// rhs), one pass instead of a second matrix-free element pass.  The product
// is deterministic: every block writes its share of a row into a slot of its
// own (row r of the element vector: slot j for node j's u columns, slot
// NEN + l for vertex l's p column) and each row sums its slots in order.
template <bool HEXA, typename T, bool RHS>
__global__ void __launch_bounds__(ET<HEXA>::NT)
    k_assemble_K(ElemLaunch L, double* val64, float* val32, const double* __restrict__ u,
                 double* __restrict__ bvec) {
  constexpr int NEN = ET<HEXA>::NEN, NV = ET<HEXA>::NV, NGP = ET<HEXA>::NGP,
                NT = ET<HEXA>::NT;
  constexpr int NST = SmK<HEXA, T>::NST, NSLOT = SmK<HEXA, T>::NSLOT;
  static_assert(!RHS || std::is_same<T, double>::value, "the fused product is FP64");
  static_assert(!HEXA || NST * NSLOT <= NGP * NEN * 3, "hexa slots fit in G.g");
  extern __shared__ __align__(16) unsigned char smem[];
  SmK<HEXA, T>& S = *reinterpret_cast<SmK<HEXA, T>*>(smem);
  Geo<HEXA, T>& G = S.G;
  ElemCtx& E = S.E;
  auto& sEq = S.sEq;
  auto& sE0 = S.sE0;
  int& sFail = S.sFail;
  const double* ul = S.ul;
  const int el = L.elems[blockIdx.x];
  if (threadIdx.x == 0) sFail = 0;
  load_element<HEXA, T>(L, el, E, G);
  for (int k = threadIdx.x; k < NEN; k += NT) {
    const int n = E.nodes[k];
    int e0 = 0x7fffffff;
    for (int q = 0; q < kNdf; ++q) {
      const int e = eq_of(L, n, q);
      sEq[k][q] = e;
      if (e > 0 && e < e0) e0 = e;
    }
    sE0[k] = e0;
  }
  if constexpr (RHS) {
    for (int k = threadIdx.x; k < NST; k += NT) {
      const int n = k < 3 * NEN ? E.nodes[k / 3] : E.nodes[k - 3 * NEN];
      const int q = k < 3 * NEN ? k % 3 : 3;
      S.ul[k] = u[(size_t)kNdf * (n - 1) + q];
    }
  }
  for (int gq = threadIdx.x; gq < NGP; gq += NT) {
    if (!point_geometry<HEXA, T>(G, gq, nullptr)) {
      sFail = 1;
      continue;
    }
    // every entry below is a sum over points of w times a product of two
    // point values: for the hexa's 64 points, scale the point's values by
    // sqrt(w) (w > 0 here) and the pair loops need no multiply by w; the
    // tetra's 4-point loops keep the per-pair weight
    if constexpr (HEXA) {
      const T sw = sqrt(G.w[gq]);
#pragma unroll
      for (int k = 0; k < NEN; ++k) {
        G.g[gq][k][0] *= sw; G.g[gq][k][1] *= sw; G.g[gq][k][2] *= sw;
      }
#pragma unroll
      for (int k = 0; k < NV; ++k) {
        G.hp[gq][k] *= sw;
        G.gp[gq][k][0] *= sw; G.gp[gq][k][1] *= sw; G.gp[gq][k][2] *= sw;
      }
    }
  }
  __syncthreads();
  if (sFail) {
    if (threadIdx.x == 0) atomicOr(L.err, 1);
    return;
  }
  const MatConst mc = L.mat[E.mat - 1];
  const T a = T(mc.a), b = T(mc.b), c = T(mc.c);
  const int32_t* slot = L.slot + (size_t)NEN * NEN * blockIdx.x;
  // ---- Kuu: node pairs (i >= j) -------------------------------------------
  constexpr int NPAIR = NEN * (NEN + 1) / 2, QUU = (NPAIR + NT - 1) / NT;
  // RHS: per pair, row (i, k) gets K_ij u_j (slot j) and, for i != j, row
  // (j, l) gets K_ij^T u_i (slot i); held here until G.g is free
  double ru[RHS ? QUU : 1][6];
#pragma unroll
  for (int q = 0; q < QUU; ++q) {
    const int pr = threadIdx.x + q * NT;
    if (pr >= NPAIR) break;
    // decode pr -> (i, j), i >= j
    int i = int((sqrtf(8.0f * pr + 1.0f) - 1.0f) * 0.5f);
    while ((i + 1) * (i + 2) / 2 <= pr) ++i;
    while (i * (i + 1) / 2 > pr) --i;
    const int j = pr - i * (i + 1) / 2;
    T P[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
#pragma unroll 4
    for (int gq = 0; gq < NGP; ++gq) {
      const T w = pair_weight(G, gq);
      const T gi0 = w * G.g[gq][i][0], gi1 = w * G.g[gq][i][1], gi2 = w * G.g[gq][i][2];
      const T gj0 = G.g[gq][j][0], gj1 = G.g[gq][j][1], gj2 = G.g[gq][j][2];
      P[0][0] += gi0 * gj0; P[0][1] += gi0 * gj1; P[0][2] += gi0 * gj2;
      P[1][0] += gi1 * gj0; P[1][1] += gi1 * gj1; P[1][2] += gi1 * gj2;
      P[2][0] += gi2 * gj0; P[2][1] += gi2 * gj1; P[2][2] += gi2 * gj2;
    }
    const T tr = P[0][0] + P[1][1] + P[2][2];
    T K[3][3];
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
      for (int l = 0; l < 3; ++l)
        K[k][l] = (k == l) ? a * (P[k][k] + c * (tr - P[k][k]))
                           : a * (b * P[k][l] + c * P[l][k]);
    if constexpr (RHS) {
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        ru[q][k] = K[k][0] * ul[3 * j] + K[k][1] * ul[3 * j + 1] + K[k][2] * ul[3 * j + 2];
        ru[q][3 + k] = K[0][k] * ul[3 * i] + K[1][k] * ul[3 * i + 1] + K[2][k] * ul[3 * i + 2];
      }
    }
    const int ni = E.nodes[i], nj = E.nodes[j];
    const int64_t offi = L.node_val_off[ni - 1], offj = L.node_val_off[nj - 1];
    const int Wi = L.node_W[ni - 1], Wj = L.node_W[nj - 1];
    const int sij = slot[i * NEN + j], sji = slot[j * NEN + i];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const int er = sEq[i][k];
      if (er == 0) continue;
      const int64_t rowi = offi + (int64_t)(er - sE0[i]) * Wi + sij - sE0[j];
#pragma unroll
      for (int l = 0; l < 3; ++l) {
        const int ec = sEq[j][l];
        if (ec == 0) continue;
        add_val<T>(val64, val32, rowi + ec, K[k][l]);
        if (i != j) {
          // transposed entry in node j's panel: row ec, column er
          add_val<T>(val64, val32,
                     offj + (int64_t)(ec - sE0[j]) * Wj + sji - sE0[i] + er, K[k][l]);
        }
      }
    }
  }
  // ---- Kpu / Kup: (vertex l, node j) ---------------------------------------
  const T alpha = T(mc.coef_biot);
  constexpr int NPU = NV * NEN, QPU = (NPU + NT - 1) / NT;
  // RHS: p row l gets Kpu_lj . u_j (slot j), rows (j, k) get Kup_jl p_l
  // (slot NEN + l)
  double rk[RHS ? QPU : 1][4];
#pragma unroll
  for (int q = 0; q < QPU; ++q) {
    const int pr = threadIdx.x + q * NT;
    if (pr >= NPU) break;
    const int l = pr / NEN, j = pr % NEN;
    T A0 = 0, A1 = 0, A2 = 0;
#pragma unroll 4
    for (int gq = 0; gq < NGP; ++gq) {
      const T wh = pair_weight(G, gq) * G.hp[gq][l];
      A0 += wh * G.g[gq][j][0]; A1 += wh * G.g[gq][j][1]; A2 += wh * G.g[gq][j][2];
    }
    const T Kv[3] = {-alpha * A0, -alpha * A1, -alpha * A2};
    if constexpr (RHS) {
      const double pl = ul[3 * NEN + l];
      rk[q][0] = Kv[0] * ul[3 * j] + Kv[1] * ul[3 * j + 1] + Kv[2] * ul[3 * j + 2];
      rk[q][1] = Kv[0] * pl; rk[q][2] = Kv[1] * pl; rk[q][3] = Kv[2] * pl;
    }
    const int er = sEq[l][3];
    if (er == 0) continue;
    const int nl = E.nodes[l], nj = E.nodes[j];
    const int64_t offl = L.node_val_off[nl - 1], offj = L.node_val_off[nj - 1];
    const int Wl = L.node_W[nl - 1], Wj = L.node_W[nj - 1];
    const int slj = slot[l * NEN + j], sjl = slot[j * NEN + l];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const int ec = sEq[j][k];
      if (ec == 0) continue;
      add_val<T>(val64, val32, offl + (int64_t)(er - sE0[l]) * Wl + slj - sE0[j] + ec, Kv[k]);
      add_val<T>(val64, val32, offj + (int64_t)(ec - sE0[j]) * Wj + sjl - sE0[l] + er, Kv[k]);
    }
  }
  double* C = nullptr;
  if constexpr (RHS) {
    // every read of G.g is done: the hexa's slots may overwrite it
    __syncthreads();
    if constexpr (HEXA) C = reinterpret_cast<double*>(&G.g[0][0][0]);
    else C = S.Cx;
#pragma unroll
    for (int q = 0; q < QUU; ++q) {
      const int pr = threadIdx.x + q * NT;
      if (pr >= NPAIR) break;
      int i = int((sqrtf(8.0f * pr + 1.0f) - 1.0f) * 0.5f);
      while ((i + 1) * (i + 2) / 2 <= pr) ++i;
      while (i * (i + 1) / 2 > pr) --i;
      const int j = pr - i * (i + 1) / 2;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        C[(3 * i + k) * NSLOT + j] = ru[q][k];
        if (i != j) C[(3 * j + k) * NSLOT + i] = ru[q][3 + k];
      }
    }
#pragma unroll
    for (int q = 0; q < QPU; ++q) {
      const int pr = threadIdx.x + q * NT;
      if (pr >= NPU) break;
      const int l = pr / NEN, j = pr % NEN;
      C[(3 * NEN + l) * NSLOT + j] = rk[q][0];
#pragma unroll
      for (int k = 0; k < 3; ++k) C[(3 * j + k) * NSLOT + NEN + l] = rk[q][1 + k];
    }
  }
  // ---- Kpp: vertex pairs (l >= m) ------------------------------------------
  const T imod = T(mc.imod_biot), dtp = T(mc.perm * L.dt);
  constexpr int NPP = NV * (NV + 1) / 2;
  for (int pr = threadIdx.x; pr < NPP; pr += NT) {
    int l = 0;
    while ((l + 1) * (l + 2) / 2 <= pr) ++l;
    const int m = pr - l * (l + 1) / 2;
    T acc = 0, am = 0, ak = 0;
#pragma unroll 4
    for (int gq = 0; gq < NGP; ++gq) {
      if constexpr (HEXA) {  // values carry sqrt(w)
        am += G.hp[gq][l] * G.hp[gq][m];
        ak += G.gp[gq][l][0] * G.gp[gq][m][0] + G.gp[gq][l][1] * G.gp[gq][m][1] +
              G.gp[gq][l][2] * G.gp[gq][m][2];
      } else {
        const T w = G.w[gq];
        acc += w * imod * G.hp[gq][l] * G.hp[gq][m] +
               w * dtp * (G.gp[gq][l][0] * G.gp[gq][m][0] + G.gp[gq][l][1] * G.gp[gq][m][1] +
                          G.gp[gq][l][2] * G.gp[gq][m][2]);
      }
    }
    if constexpr (HEXA) acc = imod * am + dtp * ak;
    if constexpr (RHS) {
      C[(3 * NEN + l) * NSLOT + NEN + m] = -acc * ul[3 * NEN + m];
      if (l != m) C[(3 * NEN + m) * NSLOT + NEN + l] = -acc * ul[3 * NEN + l];
    }
    const int er = sEq[l][3], ec = sEq[m][3];
    if (er == 0 || ec == 0) continue;
    const int nl = E.nodes[l], nm = E.nodes[m];
    add_val<T>(val64, val32,
               L.node_val_off[nl - 1] + (int64_t)(er - sE0[l]) * L.node_W[nl - 1] +
                   slot[l * NEN + m] - sE0[m] + ec, -acc);
    if (l != m)
      add_val<T>(val64, val32,
                 L.node_val_off[nm - 1] + (int64_t)(ec - sE0[m]) * L.node_W[nm - 1] +
                     slot[m * NEN + l] - sE0[l] + er, -acc);
  }
  if constexpr (RHS) {
    __syncthreads();
    for (int r = threadIdx.x; r < NST; r += NT) {
      const int e = r < 3 * NEN ? sEq[r / 3][r % 3] : sEq[r - 3 * NEN][3];
      if (e == 0) continue;
      double sum = 0;
      for (int k = 0; k < NSLOT; ++k) sum += C[r * NSLOT + k];
      bvec[e - 1] -= sum;
    }
  }
}

// ---------------------------------------------------------------------------
// isw = 2, rhs: b -= K_e u_e, matrix free (FP64).  K_e u_e is, per point,
//   u rows: w [ B_i^T sigma(u) - alpha g_i (Np . u_p) ]
//   p rows: -w [ alpha Np_l div u + Np_l (Np . u_p)/M + dt perm grad Np_l . grad p ]
// with sigma = stress3d(deform3d(u)) -- the rows of s.u in lku_m.
// ---------------------------------------------------------------------------
template <bool HEXA>
struct SmR {
  Geo<HEXA, double> G;
  double ul[3 * ET<HEXA>::NEN + ET<HEXA>::NV];
  double S6[ET<HEXA>::NGP][6];  // w (sigma - alpha p I)
  double Q4[ET<HEXA>::NGP][4];  // w (alpha div + p/M), w dt perm grad p
  ElemCtx E;
  int sFail;
};

template <bool HEXA>
__global__ void __launch_bounds__(ET<HEXA>::NT)
    k_residual(ElemLaunch L, const double* __restrict__ u, double* __restrict__ bvec) {
  constexpr int NEN = ET<HEXA>::NEN, NV = ET<HEXA>::NV, NGP = ET<HEXA>::NGP,
                NT = ET<HEXA>::NT, NST = 3 * NEN + NV;
  extern __shared__ __align__(16) unsigned char smem[];
  SmR<HEXA>& S = *reinterpret_cast<SmR<HEXA>*>(smem);
  Geo<HEXA, double>& G = S.G;
  ElemCtx& E = S.E;
  auto& ul = S.ul;
  auto& S6 = S.S6;
  auto& Q4 = S.Q4;
  int& sFail = S.sFail;
  const int el = L.elems[blockIdx.x];
  if (threadIdx.x == 0) sFail = 0;
  load_element<HEXA, double>(L, el, E, G);
  for (int k = threadIdx.x; k < NST; k += NT) {
    const int n = k < 3 * NEN ? E.nodes[k / 3] : E.nodes[k - 3 * NEN];
    const int q = k < 3 * NEN ? k % 3 : 3;
    ul[k] = u[(size_t)kNdf * (n - 1) + q];
  }
  __syncthreads();
  const MatConst mc = L.mat[E.mat - 1];
  for (int gq = threadIdx.x; gq < NGP; gq += NT) {
    if (!point_geometry<HEXA, double>(G, gq, nullptr)) {
      sFail = 1;
      continue;
    }
    double ux = 0, uy = 0, uz = 0, vx = 0, vy = 0, vz = 0, wx = 0, wy = 0, wz = 0;
#pragma unroll
    for (int i = 0; i < NEN; ++i) {
      const double gx = G.g[gq][i][0], gy = G.g[gq][i][1], gz = G.g[gq][i][2];
      const double a0 = ul[3 * i], a1 = ul[3 * i + 1], a2 = ul[3 * i + 2];
      ux += gx * a0; uy += gy * a0; uz += gz * a0;
      vx += gx * a1; vy += gy * a1; vz += gz * a1;
      wx += gx * a2; wy += gy * a2; wz += gz * a2;
    }
    const double e0 = ux, e1 = vy, e2 = wz, e3 = uy + vx, e4 = vz + wy, e5 = uz + wx;
    const double A = mc.a, B = mc.b, C = mc.c;
    double pg = 0, px = 0, py = 0, pz = 0;
#pragma unroll
    for (int l = 0; l < NV; ++l) {
      const double pl = ul[3 * NEN + l];
      pg += G.hp[gq][l] * pl;
      px += G.gp[gq][l][0] * pl; py += G.gp[gq][l][1] * pl; pz += G.gp[gq][l][2] * pl;
    }
    const double w = G.w[gq];
    const double ap = mc.coef_biot * pg;
    S6[gq][0] = w * ((e0 + B * e1 + B * e2) * A - ap);
    S6[gq][1] = w * ((B * e0 + e1 + B * e2) * A - ap);
    S6[gq][2] = w * ((B * e0 + B * e1 + e2) * A - ap);
    S6[gq][3] = w * (e3 * C * A);
    S6[gq][4] = w * (e4 * C * A);
    S6[gq][5] = w * (e5 * C * A);
    Q4[gq][0] = w * (mc.coef_biot * (e0 + e1 + e2) + mc.imod_biot * pg);
    const double wdp = w * mc.perm * L.dt;
    Q4[gq][1] = wdp * px; Q4[gq][2] = wdp * py; Q4[gq][3] = wdp * pz;
  }
  __syncthreads();
  if (sFail) {
    if (threadIdx.x == 0) atomicOr(L.err, 1);
    return;
  }
  for (int k = threadIdx.x; k < NST; k += NT) {
    double acc = 0;
    int n, q;
    if (k < 3 * NEN) {
      const int i = k / 3;
      q = k % 3;
      n = E.nodes[i];
      for (int gq = 0; gq < NGP; ++gq) {
        const double gx = G.g[gq][i][0], gy = G.g[gq][i][1], gz = G.g[gq][i][2];
        if (q == 0) acc += gx * S6[gq][0] + gy * S6[gq][3] + gz * S6[gq][5];
        else if (q == 1) acc += gx * S6[gq][3] + gy * S6[gq][1] + gz * S6[gq][4];
        else acc += gx * S6[gq][5] + gy * S6[gq][4] + gz * S6[gq][2];
      }
    } else {
      const int l = k - 3 * NEN;
      q = 3;
      n = E.nodes[l];
      for (int gq = 0; gq < NGP; ++gq)
        acc -= G.hp[gq][l] * Q4[gq][0] + G.gp[gq][l][0] * Q4[gq][1] +
               G.gp[gq][l][1] * Q4[gq][2] + G.gp[gq][l][2] * Q4[gq][3];
    }
    const int e = eq_of(L, n, q);
    if (e > 0) bvec[e - 1] -= acc;
  }
}

// ---------------------------------------------------------------------------
// isw = 4: b0 -= p with p the previous-state internal force, body forces,
// Darcy gravity term and face loads (Elmlib03.f:2263-2526 / 497-752).
// ---------------------------------------------------------------------------
__device__ double d_interpol(const double* xs, const double* ys, double xi, int n) {
  if (xi <= xs[0]) return ys[0];
  if (xi >= xs[n - 1]) return ys[n - 1];
  for (int i = 0; i < n - 1; ++i) {
    const double x1 = xs[i], x2 = xs[i + 1], y1 = ys[i], y2 = ys[i + 1];
    if (xi >= x1 && xi <= x2) return y1 + (y2 - y1) * (xi - x1) / (x2 - x1);
  }
  return 0.0;
}

// tload (Pload.f:220-377) for the load types the elastic path uses.
__device__ void d_tload(const int32_t* load, const double* fload, int maxt, int nc,
                        double t, const double* x, double gmod, double& c,
                        double* vc) {
  c = 0.0;
  if (nc <= 0) return;
  const int ty = load[3 * (nc - 1)];
  const int nt = load[3 * (nc - 1) + 2];
  const double* F = fload + (size_t)maxt * PM_NFLOAD * (nc - 1);
  auto col = [&](int k) { return F + (size_t)maxt * (k - 1); };
  if (ty == 1) c = F[0];
  else if (ty == 2) c = F[0] + F[1] * t;
  else if (ty == 39 || ty == 41 || ty == 43) c = d_interpol(col(1), col(2), t, nt);
  else if (ty == 40) {
    vc[0] = d_interpol(col(1), col(2), t, nt);
    vc[1] = d_interpol(col(1), col(3), t, nt);
    vc[2] = d_interpol(col(1), col(4), t, nt);
  } else if (ty == 42) {
    const double a = d_interpol(col(1), col(2), t, nt);
    const double b = d_interpol(col(1), col(3), t, nt);
    const double w = d_interpol(col(1), col(4), t, nt);
    const double t0 = d_interpol(col(1), col(5), t, nt);
    c = t0 * (b + a * (w - x[2]) * gmod);
  }
}

__device__ void d_rotate_face(double* xf, int nfv) {
  const double v1x = xf[3] - xf[0], v1y = xf[4] - xf[1], v1z = xf[5] - xf[2];
  double v2x = xf[6] - xf[0], v2y = xf[7] - xf[1], v2z = xf[8] - xf[2];
  const double v3x = v1y * v2z - v1z * v2y, v3y = v1z * v2x - v1x * v2z,
               v3z = v1x * v2y - v1y * v2x;
  v2x = v1z * v3y - v1y * v3z; v2y = v1x * v3z - v1z * v3x; v2z = v1y * v3x - v1x * v3y;
  const double n1 = sqrt(v1x * v1x + v1y * v1y + v1z * v1z);
  const double n2 = sqrt(v2x * v2x + v2y * v2y + v2z * v2z);
  const double n3 = sqrt(v3x * v3x + v3y * v3y + v3z * v3z);
  const double R[3][3] = {{v1x / n1, v1y / n1, v1z / n1},
                          {v2x / n2, v2y / n2, v2z / n2},
                          {v3x / n3, v3y / n3, v3z / n3}};
  for (int i = 0; i < nfv; ++i) {
    double* p = xf + 3 * i;
    const double a = R[0][0] * p[0] + R[0][1] * p[1] + R[0][2] * p[2];
    const double b = R[1][0] * p[0] + R[1][1] * p[1] + R[1][2] * p[2];
    const double c = R[2][0] * p[0] + R[2][1] * p[1] + R[2][2] * p[2];
    p[0] = a; p[1] = b; p[2] = c;
  }
}

__device__ double d_det2(const double* hx, const double* hy, const double* xf, int n) {
  double j00 = 0, j01 = 0, j10 = 0, j11 = 0;
  for (int k = 0; k < n; ++k) {
    j00 += hx[k] * xf[3 * k]; j01 += hx[k] * xf[3 * k + 1];
    j10 += hy[k] * xf[3 * k]; j11 += hy[k] * xf[3 * k + 1];
  }
  return j00 * j11 - j10 * j01;
}

// Face tractions (types 40/41/42) and normal fluxes (43), single thread.
template <bool HEXA>
__device__ void face_loads(const ElemLaunch& L, const int* iqm, const int* iqh,
                           const double xv[][3], const int32_t* load,
                           const double* fload, int maxt, double* p, int* fail) {
  constexpr int NEN = ET<HEXA>::NEN;
  const int nface = HEXA ? 6 : 4, nfv = HEXA ? 4 : 3, nfn = HEXA ? 8 : 6;
  for (int j = 1; j <= nface; ++j) {
    if (!(iqm[j - 1] > 0 || iqh[j - 1] > 0)) continue;
    const int* fn = HEXA ? cHexaFace[j - 1] : cTetraFace[j - 1];
    double xf[12];
    for (int i = 0; i < nfv; ++i)
      for (int k = 0; k < 3; ++k) xf[3 * i + k] = xv[fn[i] - 1][k];
    const int cargm = iqm[j - 1] != 0 ? load[3 * (iqm[j - 1] - 1)] : 0;
    const int cargh = iqh[j - 1] != 0 ? load[3 * (iqh[j - 1] - 1)] : 0;
    double ff[3] = {0, 0, 0}, mp[3] = {0, 0, 0}, nc = 0, dd;
    if (cargm == 40 || cargm == 41 || cargm == 42) {
      const bool normal = HEXA ? (cargm == 41) : (cargm == 41 || cargm == 42);
      if (normal) {
        const double v1[3] = {xf[3] - xf[0], xf[4] - xf[1], xf[5] - xf[2]};
        const double v2[3] = {xf[6] - xf[0], xf[7] - xf[1], xf[8] - xf[2]};
        ff[0] = v2[1] * v1[2] - v2[2] * v1[1];
        ff[1] = v2[2] * v1[0] - v2[0] * v1[2];
        ff[2] = v2[0] * v1[1] - v2[1] * v1[0];
        const double tmp = 1.0 / sqrt(ff[0] * ff[0] + ff[1] * ff[1] + ff[2] * ff[2]);
        ff[0] *= tmp; ff[1] *= tmp; ff[2] *= tmp;
        if (HEXA && j != 2) { ff[0] = -ff[0]; ff[1] = -ff[1]; ff[2] = -ff[2]; }
        if (!HEXA && cargm == 42)
          for (int k = 0; k < 3; ++k) mp[k] = (xf[k] + xf[3 + k] + xf[6 + k]) / 3;
      }
      d_rotate_face(xf, nfv);
      if (cargm == 41 || cargm == 42) {
        d_tload(load, fload, maxt, iqm[j - 1], L.t, mp, L.gmod, nc, &dd);
        ff[0] *= nc; ff[1] *= nc; ff[2] *= nc;
      } else {
        d_tload(load, fload, maxt, iqm[j - 1], L.t, mp, L.gmod, dd, ff);
      }
      if (HEXA) {
        for (int ly = 0; ly < 3; ++ly)
          for (int lx = 0; lx < 3; ++lx) {
            const double r = cPG3[lx], s = cPG3[ly];
            const double pr = 1 + r, ps = 1 + s, mr = 1 - r, ms = 1 - s;
            const double hx[4] = {ps * 0.25, -ps * 0.25, -ms * 0.25, ms * 0.25};
            const double hy[4] = {pr * 0.25, mr * 0.25, -mr * 0.25, -pr * 0.25};
            const double det = d_det2(hx, hy, xf, 4);
            if (!(det > 1.0e-14)) *fail = 1;
            const double w = cWG3[lx] * cWG3[ly] * det;
            double h[8];
            const double mrr = 1 - r * r, mss = 1 - s * s;
            h[4] = mrr * ps * 0.5; h[5] = mss * mr * 0.5; h[6] = mrr * ms * 0.5;
            h[7] = mss * pr * 0.5;
            h[0] = pr * ps * 0.25 - h[4] * 0.5 - h[7] * 0.5;
            h[1] = mr * ps * 0.25 - h[4] * 0.5 - h[5] * 0.5;
            h[2] = mr * ms * 0.25 - h[5] * 0.5 - h[6] * 0.5;
            h[3] = pr * ms * 0.25 - h[6] * 0.5 - h[7] * 0.5;
            for (int i = 0; i < nfn; ++i) {
              const int no = fn[i];
              const double wt1 = h[i] * w;
              p[3 * no - 3] -= ff[0] * wt1;
              p[3 * no - 2] -= ff[1] * wt1;
              p[3 * no - 1] -= ff[2] * wt1;
            }
          }
      } else {
        for (int lx = 0; lx < 3; ++lx) {
          const double r = cPRI2[lx], s = cPSI2[lx], t = 1 - r - s;
          const double hx[3] = {1, 0, -1}, hy[3] = {0, 1, -1};
          const double det = d_det2(hx, hy, xf, 3);
          if (!(det > 1.0e-14)) *fail = 1;
          const double w = 0.5 * (cWF2 * det);
          const double h[6] = {r * (2 * r - 1), s * (2 * s - 1), t * (2 * t - 1),
                               4 * r * s, 4 * s * t, 4 * t * r};
          for (int i = 0; i < nfn; ++i) {
            const int no = fn[i];
            const double wt1 = h[i] * w;
            p[3 * no - 3] -= ff[0] * wt1;
            p[3 * no - 2] -= ff[1] * wt1;
            p[3 * no - 1] -= ff[2] * wt1;
          }
        }
      }
    }
    if (cargh == 43) {
      d_rotate_face(xf, nfv);
      d_tload(load, fload, maxt, iqh[j - 1], L.t, mp, L.gmod, nc, &dd);
      if (HEXA) {
        for (int ly = 0; ly < 3; ++ly)
          for (int lx = 0; lx < 3; ++lx) {
            const double r = cPG3[lx], s = cPG3[ly];
            const double pr = 1 + r, ps = 1 + s, mr = 1 - r, ms = 1 - s;
            const double hx[4] = {ps * 0.25, -ps * 0.25, -ms * 0.25, ms * 0.25};
            const double hy[4] = {pr * 0.25, mr * 0.25, -mr * 0.25, -pr * 0.25};
            const double h[4] = {pr * ps * 0.25, mr * ps * 0.25, mr * ms * 0.25, pr * ms * 0.25};
            const double det = d_det2(hx, hy, xf, 4);
            if (!(det > 1.0e-14)) *fail = 1;
            const double w = cWG3[lx] * cWG3[ly] * det * L.dt * nc;
            for (int i = 0; i < 4; ++i) p[3 * NEN + fn[i] - 1] -= h[i] * w;
          }
      } else {
        for (int lx = 0; lx < 3; ++lx) {
          const double r = cPRI2[lx], s = cPSI2[lx];
          const double hx[3] = {1, 0, -1}, hy[3] = {0, 1, -1};
          const double h[3] = {r, s, 1 - r - s};
          const double det = d_det2(hx, hy, xf, 3);
          if (!(det > 1.0e-14)) *fail = 1;
          const double w = 0.5 * (cWF2 * det) * L.dt * nc;
          for (int i = 0; i < 3; ++i) p[3 * NEN + fn[i] - 1] -= h[i] * w;
        }
      }
    }
  }
}

template <bool HEXA>
struct SmF {
  Geo<HEXA, double> G;
  double ul[3 * ET<HEXA>::NEN + ET<HEXA>::NV];
  double dpl[ET<HEXA>::NV];
  double S6[ET<HEXA>::NGP][6];
  double Q4[ET<HEXA>::NGP][4];
  double HU[ET<HEXA>::NGP][ET<HEXA>::NEN];  // w pm_d N_i
  double pf[3 * ET<HEXA>::NEN + ET<HEXA>::NV];  // face-load contributions
  ElemCtx E;
  int iqm[7], iqh[7];
  int sFail, sAny;
};

template <bool HEXA>
__global__ void __launch_bounds__(ET<HEXA>::NT)
    k_rhs4(ElemLaunch L, const double* __restrict__ u, const double* __restrict__ dp,
           const int32_t* __restrict__ eload, const int32_t* __restrict__ eloadp,
           const int32_t* __restrict__ load, const double* __restrict__ fload, int maxt,
           double* __restrict__ bvec) {
  constexpr int NEN = ET<HEXA>::NEN, NV = ET<HEXA>::NV, NGP = ET<HEXA>::NGP,
                NT = ET<HEXA>::NT, NST = 3 * NEN + NV;
  extern __shared__ __align__(16) unsigned char smem[];
  SmF<HEXA>& S = *reinterpret_cast<SmF<HEXA>*>(smem);
  Geo<HEXA, double>& G = S.G;
  ElemCtx& E = S.E;
  auto& ul = S.ul;
  auto& dpl = S.dpl;
  auto& S6 = S.S6;
  auto& Q4 = S.Q4;
  auto& HU = S.HU;
  auto& pf = S.pf;
  auto& iqm = S.iqm;
  auto& iqh = S.iqh;
  int& sFail = S.sFail;
  int& sAny = S.sAny;
  const int el = L.elems[blockIdx.x];
  if (threadIdx.x == 0) { sFail = 0; sAny = 0; }
  load_element<HEXA, double>(L, el, E, G);
  for (int k = threadIdx.x; k < NST; k += NT) {
    const int n = k < 3 * NEN ? E.nodes[k / 3] : E.nodes[k - 3 * NEN];
    const int q = k < 3 * NEN ? k % 3 : 3;
    ul[k] = u[(size_t)kNdf * (n - 1) + q];
    pf[k] = 0.0;
  }
  for (int k = threadIdx.x; k < NV; k += NT) dpl[k] = dp[E.nodes[k] - 1];
  for (int k = threadIdx.x; k < 7; k += NT) {
    iqm[k] = eload ? eload[(size_t)7 * (el - 1) + k] : 0;
    iqh[k] = eloadp ? eloadp[(size_t)7 * (el - 1) + k] : 0;
    if (iqm[k] > 0 || iqh[k] > 0) atomicOr(&sAny, 1);
  }
  __syncthreads();
  const MatConst mc = L.mat[E.mat - 1];
  for (int gq = threadIdx.x; gq < NGP; gq += NT) {
    double huv[NEN];
    if (!point_geometry<HEXA, double>(G, gq, huv)) {
      sFail = 1;
      continue;
    }
    double ux = 0, uy = 0, uz = 0, vx = 0, vy = 0, vz = 0, wx = 0, wy = 0, wz = 0;
#pragma unroll
    for (int i = 0; i < NEN; ++i) {
      const double gx = G.g[gq][i][0], gy = G.g[gq][i][1], gz = G.g[gq][i][2];
      const double a0 = ul[3 * i], a1 = ul[3 * i + 1], a2 = ul[3 * i + 2];
      ux += gx * a0; uy += gy * a0; uz += gz * a0;
      vx += gx * a1; vy += gy * a1; vz += gz * a1;
      wx += gx * a2; wy += gy * a2; wz += gz * a2;
    }
    const double e0 = ux, e1 = vy, e2 = wz, e3 = uy + vx, e4 = vz + wy, e5 = uz + wx;
    const double A = mc.a, B = mc.b, C = mc.c;
    double dpm = 0, px = 0, py = 0, pz = 0;
#pragma unroll
    for (int l = 0; l < NV; ++l) {
      dpm += G.hp[gq][l] * dpl[l];
      const double pl = ul[3 * NEN + l];
      px += G.gp[gq][l][0] * pl; py += G.gp[gq][l][1] * pl; pz += G.gp[gq][l][2] * pl;
    }
    dpm = mc.coef_biot * dpm;
    const double w = G.w[gq];
    S6[gq][0] = w * ((e0 + B * e1 + B * e2) * A - dpm);
    S6[gq][1] = w * ((B * e0 + e1 + B * e2) * A - dpm);
    S6[gq][2] = w * ((B * e0 + B * e1 + e2) * A - dpm);
    S6[gq][3] = w * (e3 * C * A);
    S6[gq][4] = w * (e4 * C * A);
    S6[gq][5] = w * (e5 * C * A);
    // p rows: + w dt perm [rho_f g - grad p]
    const double wdp = w * mc.perm * L.dt;
    Q4[gq][1] = wdp * (mc.fluid_d * L.g0 - px);
    Q4[gq][2] = wdp * (mc.fluid_d * L.g1 - py);
    Q4[gq][3] = wdp * (mc.fluid_d * L.g2 - pz);
    const double wpm = w * mc.pm_d;
#pragma unroll
    for (int i = 0; i < NEN; ++i) HU[gq][i] = wpm * huv[i];
  }
  __syncthreads();
  if (sAny && threadIdx.x == 0) {
    int f = 0;
    face_loads<HEXA>(L, iqm, iqh, G.xv, load, fload, maxt, pf, &f);
    if (f) sFail = 1;
  }
  __syncthreads();
  if (sFail) {
    if (threadIdx.x == 0) atomicOr(L.err, 1);
    return;
  }
  const double gl[3] = {L.g0, L.g1, L.g2};
  for (int k = threadIdx.x; k < NST; k += NT) {
    double acc = 0;
    int n, q;
    if (k < 3 * NEN) {
      const int i = k / 3;
      q = k % 3;
      n = E.nodes[i];
      for (int gq = 0; gq < NGP; ++gq) {
        const double gx = G.g[gq][i][0], gy = G.g[gq][i][1], gz = G.g[gq][i][2];
        if (q == 0) acc += gx * S6[gq][0] + gy * S6[gq][3] + gz * S6[gq][5];
        else if (q == 1) acc += gx * S6[gq][3] + gy * S6[gq][1] + gz * S6[gq][4];
        else acc += gx * S6[gq][5] + gy * S6[gq][4] + gz * S6[gq][2];
        acc -= HU[gq][i] * gl[q];
      }
    } else {
      const int l = k - 3 * NEN;
      q = 3;
      n = E.nodes[l];
      for (int gq = 0; gq < NGP; ++gq)
        acc += G.gp[gq][l][0] * Q4[gq][1] + G.gp[gq][l][1] * Q4[gq][2] +
               G.gp[gq][l][2] * Q4[gq][3];
    }
    acc += pf[k];
    const int e = eq_of(L, n, q);
    if (e > 0) bvec[e - 1] -= acc;
  }
}

// ---------------------------------------------------------------------------
// Adjoint of the time-stepped solve.  Each step solves K du = F - A s - g0
// with s = (u, dp) the previous state, where (from k_rhs4 and k_residual)
//   A s = [Kuu u_u + Kup dp ; Kpp_perm u_p],   g0 = [-body ; G_k],
//   Kpp_perm = -dt perm int(grad N grad N),  G_k = dt perm rho_f int(grad N . g),
// and then s += (du, du_p).  Every block is linear in one element parameter:
// Kuu in E, Kpp_perm and G_k in the permeability k, the storage block
// -(1/M) int(N N) of Kpp in 1/M.
//
// MODE 0 (apply), for the adjoint state: mu -= [Kuu lam_u ; Kpp_perm lam_p],
//   nu -= Kpu lam_u (p rows), element by element (one colour per launch, so
//   no two elements of a launch share an equation).
// MODE 1 (grad): per element the contractions of d(F - A s - g0 - K du)
//   with lam for the log parameters:
//   d/dlog E:  -lam_u^T Kuu u_n          (u_n = s + du, the step's new state)
//   d/dlog k:  -lam_p^T (Kpp_perm p_n + G_k)
//   d/dlog M:   lam_p^T Kstor du_p,  Kstor = -(1/M) int(N N)
//   accumulated into grad[3 (el - 1) + {0, 1, 2}].
// ---------------------------------------------------------------------------
template <bool HEXA>
struct SmA {
  Geo<HEXA, double> G;
  double ll[3 * ET<HEXA>::NEN + ET<HEXA>::NV];  // lam on the element dofs
  double ul[3 * ET<HEXA>::NEN + ET<HEXA>::NV];  // u_n (MODE 1)
  double dl[ET<HEXA>::NV];                      // du_p (MODE 1)
  double S6[ET<HEXA>::NGP][6];
  double Q4[ET<HEXA>::NGP][4];
  double gsum[3][ET<HEXA>::NT / 32];
  ElemCtx E;
  int sFail;
};

template <bool HEXA, int MODE>
__global__ void __launch_bounds__(ET<HEXA>::NT)
    k_adjoint(ElemLaunch L, const double* __restrict__ lam, const double* __restrict__ un,
              const double* __restrict__ dun, double* __restrict__ mu, double* __restrict__ nu,
              double* __restrict__ grad) {
  constexpr int NEN = ET<HEXA>::NEN, NV = ET<HEXA>::NV, NGP = ET<HEXA>::NGP,
                NT = ET<HEXA>::NT, NST = 3 * NEN + NV;
  extern __shared__ __align__(16) unsigned char smem[];
  SmA<HEXA>& S = *reinterpret_cast<SmA<HEXA>*>(smem);
  Geo<HEXA, double>& G = S.G;
  ElemCtx& E = S.E;
  const int el = L.elems[blockIdx.x];
  if (threadIdx.x == 0) S.sFail = 0;
  load_element<HEXA, double>(L, el, E, G);
  for (int k = threadIdx.x; k < NST; k += NT) {
    const int n = k < 3 * NEN ? E.nodes[k / 3] : E.nodes[k - 3 * NEN];
    const int q = k < 3 * NEN ? k % 3 : 3;
    S.ll[k] = lam[(size_t)kNdf * (n - 1) + q];
    if (MODE == 1) S.ul[k] = un[(size_t)kNdf * (n - 1) + q];
  }
  if (MODE == 1)
    for (int k = threadIdx.x; k < NV; k += NT) S.dl[k] = dun[(size_t)kNdf * (E.nodes[k] - 1) + 3];
  __syncthreads();
  const MatConst mc = L.mat[E.mat - 1];
  double gE = 0.0, gK = 0.0, gM = 0.0;
  for (int gq = threadIdx.x; gq < NGP; gq += NT) {
    if (!point_geometry<HEXA, double>(G, gq, nullptr)) {
      S.sFail = 1;
      continue;
    }
    // strains, pressure value and gradient of lam (and of u_n)
    double le[6], ue[6];
    {
      double ux = 0, uy = 0, uz = 0, vx = 0, vy = 0, vz = 0, wx = 0, wy = 0, wz = 0;
      double Ux = 0, Uy = 0, Uz = 0, Vx = 0, Vy = 0, Vz = 0, Wx = 0, Wy = 0, Wz = 0;
#pragma unroll
      for (int i = 0; i < NEN; ++i) {
        const double gx = G.g[gq][i][0], gy = G.g[gq][i][1], gz = G.g[gq][i][2];
        const double a0 = S.ll[3 * i], a1 = S.ll[3 * i + 1], a2 = S.ll[3 * i + 2];
        ux += gx * a0; uy += gy * a0; uz += gz * a0;
        vx += gx * a1; vy += gy * a1; vz += gz * a1;
        wx += gx * a2; wy += gy * a2; wz += gz * a2;
        if (MODE == 1) {
          const double b0 = S.ul[3 * i], b1 = S.ul[3 * i + 1], b2 = S.ul[3 * i + 2];
          Ux += gx * b0; Uy += gy * b0; Uz += gz * b0;
          Vx += gx * b1; Vy += gy * b1; Vz += gz * b1;
          Wx += gx * b2; Wy += gy * b2; Wz += gz * b2;
        }
      }
      le[0] = ux; le[1] = vy; le[2] = wz; le[3] = uy + vx; le[4] = vz + wy; le[5] = uz + wx;
      ue[0] = Ux; ue[1] = Vy; ue[2] = Wz; ue[3] = Uy + Vx; ue[4] = Vz + Wy; ue[5] = Uz + Wx;
    }
    double lp = 0, lpx = 0, lpy = 0, lpz = 0, upx = 0, upy = 0, upz = 0, dpv = 0;
#pragma unroll
    for (int l = 0; l < NV; ++l) {
      const double pl = S.ll[3 * NEN + l];
      lp += G.hp[gq][l] * pl;
      lpx += G.gp[gq][l][0] * pl; lpy += G.gp[gq][l][1] * pl; lpz += G.gp[gq][l][2] * pl;
      if (MODE == 1) {
        const double ql = S.ul[3 * NEN + l];
        upx += G.gp[gq][l][0] * ql; upy += G.gp[gq][l][1] * ql; upz += G.gp[gq][l][2] * ql;
        dpv += G.hp[gq][l] * S.dl[l];
      }
    }
    const double w = G.w[gq];
    const double A = mc.a, B = mc.b, C = mc.c;
    const double wdp = w * mc.perm * L.dt;
    if (MODE == 0) {
      // w D eps(lam) (no coupling term), w dt perm grad lam_p, w alpha div lam_u
      S.S6[gq][0] = w * (le[0] + B * le[1] + B * le[2]) * A;
      S.S6[gq][1] = w * (B * le[0] + le[1] + B * le[2]) * A;
      S.S6[gq][2] = w * (B * le[0] + B * le[1] + le[2]) * A;
      S.S6[gq][3] = w * le[3] * C * A;
      S.S6[gq][4] = w * le[4] * C * A;
      S.S6[gq][5] = w * le[5] * C * A;
      S.Q4[gq][0] = w * mc.coef_biot * (le[0] + le[1] + le[2]);
      S.Q4[gq][1] = wdp * lpx; S.Q4[gq][2] = wdp * lpy; S.Q4[gq][3] = wdp * lpz;
    } else {
      const double s0 = (ue[0] + B * ue[1] + B * ue[2]) * A;
      const double s1 = (B * ue[0] + ue[1] + B * ue[2]) * A;
      const double s2 = (B * ue[0] + B * ue[1] + ue[2]) * A;
      gE -= w * (le[0] * s0 + le[1] * s1 + le[2] * s2 +
                 C * A * (le[3] * ue[3] + le[4] * ue[4] + le[5] * ue[5]));
      gK += wdp * (lpx * (upx - mc.fluid_d * L.g0) + lpy * (upy - mc.fluid_d * L.g1) +
                   lpz * (upz - mc.fluid_d * L.g2));
      gM -= w * mc.imod_biot * lp * dpv;
    }
  }
  __syncthreads();
  if (S.sFail) {
    if (threadIdx.x == 0) atomicOr(L.err, 1);
    return;
  }
  if (MODE == 1) {
    double v[3] = {gE, gK, gM};
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      double x = v[k];
      for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
      if (lane == 0) S.gsum[k][wid] = x;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
      double t = 0.0;
      for (int i = 0; i < NT / 32; ++i) t += S.gsum[threadIdx.x][i];
      grad[(size_t)3 * (el - 1) + threadIdx.x] += t;
    }
    return;
  }
  for (int k = threadIdx.x; k < NST; k += NT) {
    int n, q;
    double am = 0.0, an = 0.0;
    if (k < 3 * NEN) {
      const int i = k / 3;
      q = k % 3;
      n = E.nodes[i];
      for (int gq = 0; gq < NGP; ++gq) {
        const double gx = G.g[gq][i][0], gy = G.g[gq][i][1], gz = G.g[gq][i][2];
        if (q == 0) am += gx * S.S6[gq][0] + gy * S.S6[gq][3] + gz * S.S6[gq][5];
        else if (q == 1) am += gx * S.S6[gq][3] + gy * S.S6[gq][1] + gz * S.S6[gq][4];
        else am += gx * S.S6[gq][5] + gy * S.S6[gq][4] + gz * S.S6[gq][2];
      }
    } else {
      const int l = k - 3 * NEN;
      q = 3;
      n = E.nodes[l];
      for (int gq = 0; gq < NGP; ++gq) {
        am -= G.gp[gq][l][0] * S.Q4[gq][1] + G.gp[gq][l][1] * S.Q4[gq][2] +
              G.gp[gq][l][2] * S.Q4[gq][3];
        an -= G.hp[gq][l] * S.Q4[gq][0];
      }
    }
    const int e = eq_of(L, n, q);
    if (e > 0) {
      mu[e - 1] -= am;
      if (q == 3) nu[e - 1] -= an;
    }
  }
}

// ---------------------------------------------------------------------------
// isw = 3: stresses and Darcy fluxes at the vertices (Elmlib03.f:2206-2256
// hexa20, :440-495 tetra10), accumulated per vertex node for tform_pm's
// average (Pform.f:433-640).  At vertex i (natural coordinates of the
// element's vertex table): total stress D eps(u) - alpha dp_i, Biot stress
// total + alpha p_i (normal components), flux perm (rho_f g - grad p) with
// the linear pressure gradient.  One thread per vertex; one colour per
// launch, so no two elements of a launch share a vertex.  MODE 7 is the
// porosity change of porosity_form (Pform.f:969-1175; Elmlib03.f:2605-2631):
// alpha tr(eps(du)) + dp_i / M at vertex i, with u the step's increments.
// ---------------------------------------------------------------------------
__constant__ double cRNH[8] = {1, -1, -1, 1, 1, -1, -1, 1};
__constant__ double cSNH[8] = {1, 1, -1, -1, 1, 1, -1, -1};
__constant__ double cTNH[8] = {1, 1, 1, 1, -1, -1, -1, -1};
__constant__ double cRNT[4] = {1, 0, 0, 0};
__constant__ double cSNT[4] = {0, 1, 0, 0};
__constant__ double cTNT[4] = {0, 0, 1, 0};

template <bool HEXA>
struct Sm3 {
  Geo<HEXA, double> G;
  double ul[3 * ET<HEXA>::NEN + ET<HEXA>::NV];
  double dpl[ET<HEXA>::NV];
  ElemCtx E;
  int sFail;
};

template <bool HEXA, int MODE>
__global__ void __launch_bounds__(ET<HEXA>::NT)
    k_vertex(ElemLaunch L, const double* __restrict__ u, const double* __restrict__ dp,
             double* __restrict__ tx, double* __restrict__ txb, double* __restrict__ flux) {
  constexpr int NEN = ET<HEXA>::NEN, NV = ET<HEXA>::NV, NT = ET<HEXA>::NT,
                NST = 3 * NEN + NV;
  extern __shared__ __align__(16) unsigned char smem[];
  Sm3<HEXA>& S = *reinterpret_cast<Sm3<HEXA>*>(smem);
  Geo<HEXA, double>& G = S.G;
  ElemCtx& E = S.E;
  const int el = L.elems[blockIdx.x];
  if (threadIdx.x == 0) S.sFail = 0;
  load_element<HEXA, double>(L, el, E, G);
  for (int k = threadIdx.x; k < NST; k += NT) {
    const int n = k < 3 * NEN ? E.nodes[k / 3] : E.nodes[k - 3 * NEN];
    const int q = k < 3 * NEN ? k % 3 : 3;
    S.ul[k] = u[(size_t)kNdf * (n - 1) + q];
  }
  if (MODE == 3)
    for (int k = threadIdx.x; k < NV; k += NT) S.dpl[k] = dp[E.nodes[k] - 1];
  __syncthreads();
  const int i = threadIdx.x;
  if (i < NV) {
    const double r = HEXA ? cRNH[i] : cRNT[i], sv = HEXA ? cSNH[i] : cSNT[i],
                 tv = HEXA ? cTNH[i] : cTNT[i];
    if (!point_geometry_rst<HEXA, double>(G, i, r, sv, tv, 1.0, nullptr)) S.sFail = 1;
  }
  __syncthreads();
  if (S.sFail) {
    if (threadIdx.x == 0) atomicOr(L.err, 1);
    return;
  }
  if (i >= NV) return;
  const MatConst mc = L.mat[E.mat - 1];
  double ux = 0, uy = 0, uz = 0, vx = 0, vy = 0, vz = 0, wx = 0, wy = 0, wz = 0;
#pragma unroll
  for (int k = 0; k < NEN; ++k) {
    const double gx = G.g[i][k][0], gy = G.g[i][k][1], gz = G.g[i][k][2];
    const double a0 = S.ul[3 * k], a1 = S.ul[3 * k + 1], a2 = S.ul[3 * k + 2];
    ux += gx * a0; uy += gy * a0; uz += gz * a0;
    vx += gx * a1; vy += gy * a1; vz += gz * a1;
    wx += gx * a2; wy += gy * a2; wz += gz * a2;
  }
  const int no = E.nodes[i] - 1;
  if (MODE == 7) {
    // tx is the porosity change accumulator here
    tx[no] += mc.coef_biot * (ux + vy + wz) + mc.imod_biot * S.ul[3 * NEN + i];
    return;
  }
  const double e0 = ux, e1 = vy, e2 = wz, e3 = uy + vx, e4 = vz + wy, e5 = uz + wx;
  const double A = mc.a, B = mc.b, C = mc.c;
  const double dpm = mc.coef_biot * S.dpl[i];
  const double pm = mc.coef_biot * S.ul[3 * NEN + i];
  double t[6];
  t[0] = (e0 + B * e1 + B * e2) * A - dpm;
  t[1] = (B * e0 + e1 + B * e2) * A - dpm;
  t[2] = (B * e0 + B * e1 + e2) * A - dpm;
  t[3] = e3 * C * A;
  t[4] = e4 * C * A;
  t[5] = e5 * C * A;
  double px = 0, py = 0, pz = 0;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    const double pk = S.ul[3 * NEN + k];
    px += G.gp[i][k][0] * pk; py += G.gp[i][k][1] * pk; pz += G.gp[i][k][2] * pk;
  }
  double* T6 = tx + (size_t)6 * no;
  double* B6 = txb + (size_t)6 * no;
  for (int j = 0; j < 6; ++j) {
    T6[j] += t[j];
    B6[j] += t[j] + (j < 3 ? pm : 0.0);
  }
  double* F3 = flux + (size_t)3 * no;
  F3[0] += mc.perm * (mc.fluid_d * L.g0 - px);
  F3[1] += mc.perm * (mc.fluid_d * L.g1 - py);
  F3[2] += mc.perm * (mc.fluid_d * L.g2 - pz);
}

// isw = 5: initial stress, b -= int(B^T sigma0) with sigma0 interpolated by
// the linear functions from the vertex values (Elmlib03.f:2528-2590).
template <bool HEXA>
struct Sm5 {
  Geo<HEXA, double> G;
  double S6[ET<HEXA>::NGP][6];
  ElemCtx E;
  int sFail;
};

template <bool HEXA>
__global__ void __launch_bounds__(ET<HEXA>::NT)
    k_stress5(ElemLaunch L, const double* __restrict__ tx0, double* __restrict__ bvec) {
  constexpr int NEN = ET<HEXA>::NEN, NV = ET<HEXA>::NV, NGP = ET<HEXA>::NGP,
                NT = ET<HEXA>::NT;
  extern __shared__ __align__(16) unsigned char smem[];
  Sm5<HEXA>& S = *reinterpret_cast<Sm5<HEXA>*>(smem);
  Geo<HEXA, double>& G = S.G;
  ElemCtx& E = S.E;
  auto& S6 = S.S6;
  int& sFail = S.sFail;
  const int el = L.elems[blockIdx.x];
  if (threadIdx.x == 0) sFail = 0;
  load_element<HEXA, double>(L, el, E, G);
  for (int gq = threadIdx.x; gq < NGP; gq += NT) {
    if (!point_geometry<HEXA, double>(G, gq, nullptr)) {
      sFail = 1;
      continue;
    }
    double tx[6] = {0, 0, 0, 0, 0, 0};
    for (int j = 0; j < NV; ++j)
      for (int k = 0; k < 6; ++k) tx[k] += G.hp[gq][j] * tx0[(size_t)6 * (E.nodes[j] - 1) + k];
    for (int k = 0; k < 6; ++k) S6[gq][k] = G.w[gq] * tx[k];
  }
  __syncthreads();
  if (sFail) {
    if (threadIdx.x == 0) atomicOr(L.err, 1);
    return;
  }
  for (int k = threadIdx.x; k < 3 * NEN; k += NT) {
    const int i = k / 3, q = k % 3;
    double acc = 0;
    for (int gq = 0; gq < NGP; ++gq) {
      const double gx = G.g[gq][i][0], gy = G.g[gq][i][1], gz = G.g[gq][i][2];
      if (q == 0) acc += gx * S6[gq][0] + gy * S6[gq][3] + gz * S6[gq][5];
      else if (q == 1) acc += gx * S6[gq][3] + gy * S6[gq][1] + gz * S6[gq][4];
      else acc += gx * S6[gq][5] + gy * S6[gq][4] + gz * S6[gq][2];
    }
    const int e = eq_of(L, E.nodes[i], q);
    if (e > 0) bvec[e - 1] -= acc;
  }
}

// Launch helper: dynamic shared memory sized by the kernel's struct, with the
// opt-in above 48 KB set once per kernel.
template <typename Sm, typename Kern, typename... Args>
cudaError_t launch_elem(Kern k, int n, int nt, cudaStream_t s, Args... args) {
  // kernels of one signature and shared-memory struct (k_assemble_K with and
  // without the fused product) share this instantiation: key on the kernel
  static std::mutex mu;
  static std::vector<std::pair<const void*, int>> opted;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  {
    std::lock_guard<std::mutex> lock(mu);
    const std::pair<const void*, int> key(reinterpret_cast<const void*>(k), dev);
    if (std::find(opted.begin(), opted.end(), key) == opted.end()) {
      e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(Sm));
      if (e != cudaSuccess) return e;
      opted.push_back(key);
    }
  }
  k<<<n, nt, sizeof(Sm), s>>>(args...);
  return cudaGetLastError();
}

}  // namespace

cudaError_t ensure_shape_tables() {
  static std::mutex mu;
  static bool filled[kMaxDevices] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(mu);
  if (filled[dev]) return cudaSuccess;
  cudaStream_t s;
  if ((e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking)) != cudaSuccess) return e;
  k_fill_shape_tables<<<1, kHexaGp, 0, s>>>();
  e = cudaGetLastError();
  const cudaError_t e2 = cudaStreamSynchronize(s);
  cudaStreamDestroy(s);
  if (e == cudaSuccess) e = e2;
  if (e == cudaSuccess) filled[dev] = true;
  return e;
}

cudaError_t launch_assemble_K(const ElemLaunch& L, bool hexa, double* val, cudaStream_t s,
                              const double* u, double* b) {
  if (L.nelem <= 0) return cudaSuccess;
  float* no32 = nullptr;
  if (b) {
    if (hexa)
      return launch_elem<SmK<true, double>>(k_assemble_K<true, double, true>, L.nelem, 64, s,
                                            L, val, no32, u, b);
    return launch_elem<SmK<false, double>>(k_assemble_K<false, double, true>, L.nelem, 32, s,
                                           L, val, no32, u, b);
  }
  const double* nu = nullptr;
  double* nb = nullptr;
  if (hexa)
    return launch_elem<SmK<true, double>>(k_assemble_K<true, double, false>, L.nelem, 64, s, L,
                                          val, no32, nu, nb);
  return launch_elem<SmK<false, double>>(k_assemble_K<false, double, false>, L.nelem, 32, s, L,
                                         val, no32, nu, nb);
}

cudaError_t launch_residual(const ElemLaunch& L, bool hexa, const double* u,
                            double* b, cudaStream_t s) {
  if (L.nelem <= 0) return cudaSuccess;
  if (hexa) return launch_elem<SmR<true>>(k_residual<true>, L.nelem, 64, s, L, u, b);
  return launch_elem<SmR<false>>(k_residual<false>, L.nelem, 32, s, L, u, b);
}

cudaError_t launch_rhs4(const ElemLaunch& L, bool hexa, const double* u,
                        const double* dp, const int32_t* eload,
                        const int32_t* eloadp, const int32_t* load,
                        const double* fload, int maxt, double* b, cudaStream_t s) {
  if (L.nelem <= 0) return cudaSuccess;
  if (hexa)
    return launch_elem<SmF<true>>(k_rhs4<true>, L.nelem, 64, s, L, u, dp, eload, eloadp,
                                  load, fload, maxt, b);
  return launch_elem<SmF<false>>(k_rhs4<false>, L.nelem, 32, s, L, u, dp, eload, eloadp,
                                 load, fload, maxt, b);
}

// (the shared-memory opt-in is set per kernel: the two modes share a
// signature, so launch_elem's per-instantiation flag would cover only one)
template <bool HEXA, int MODE>
cudaError_t launch_adjoint_t(const ElemLaunch& L, const double* lam, const double* un,
                             const double* dun, double* mu, double* nu, double* grad,
                             cudaStream_t s) {
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k_adjoint<HEXA, MODE>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)sizeof(SmA<HEXA>));
    if (e != cudaSuccess) return e;
    attr = true;
  }
  k_adjoint<HEXA, MODE><<<L.nelem, ET<HEXA>::NT, sizeof(SmA<HEXA>), s>>>(L, lam, un, dun, mu,
                                                                          nu, grad);
  return cudaGetLastError();
}

cudaError_t launch_adjoint(const ElemLaunch& L, bool hexa, int mode, const double* lam,
                           const double* un, const double* dun, double* mu, double* nu,
                           double* grad, cudaStream_t s) {
  if (L.nelem <= 0) return cudaSuccess;
  if (hexa)
    return mode == 0 ? launch_adjoint_t<true, 0>(L, lam, un, dun, mu, nu, grad, s)
                     : launch_adjoint_t<true, 1>(L, lam, un, dun, mu, nu, grad, s);
  return mode == 0 ? launch_adjoint_t<false, 0>(L, lam, un, dun, mu, nu, grad, s)
                   : launch_adjoint_t<false, 1>(L, lam, un, dun, mu, nu, grad, s);
}

cudaError_t launch_stress3(const ElemLaunch& L, bool hexa, const double* u,
                           const double* dp, double* tx, double* txb, double* flux,
                           cudaStream_t s) {
  if (L.nelem <= 0) return cudaSuccess;
  if (hexa)
    return launch_elem<Sm3<true>>(k_vertex<true, 3>, L.nelem, 64, s, L, u, dp, tx, txb, flux);
  return launch_elem<Sm3<false>>(k_vertex<false, 3>, L.nelem, 32, s, L, u, dp, tx, txb, flux);
}

cudaError_t launch_poro7(const ElemLaunch& L, bool hexa, const double* du, double* dporo,
                         cudaStream_t s) {
  if (L.nelem <= 0) return cudaSuccess;
  if (hexa)
    return launch_elem<Sm3<true>>(k_vertex<true, 7>, L.nelem, 64, s, L, du,
                                  (const double*)nullptr, dporo, (double*)nullptr,
                                  (double*)nullptr);
  return launch_elem<Sm3<false>>(k_vertex<false, 7>, L.nelem, 32, s, L, du,
                                 (const double*)nullptr, dporo, (double*)nullptr,
                                 (double*)nullptr);
}

cudaError_t launch_stress5(const ElemLaunch& L, bool hexa, const double* tx0,
                           double* b, cudaStream_t s) {
  if (L.nelem <= 0) return cudaSuccess;
  if (hexa) return launch_elem<Sm5<true>>(k_stress5<true>, L.nelem, 64, s, L, tx0, b);
  return launch_elem<Sm5<false>>(k_stress5<false>, L.nelem, 32, s, L, tx0, b);
}

}  // namespace pm
