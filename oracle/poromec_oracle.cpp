// poromec_oracle.cpp -- CPU oracle: C++ restatement of poroMec's Biot hot
// path.  TEST INFRASTRUCTURE ONLY (see poromec_oracle.h): used by tests/,
// __graft_entry__.smoke() and bench.py's CPU baseline, never by the product.
//
// Every routine cites the Fortran routine it restates (file:line in
// lmn-labest/poroMec).  Loop order and operation order follow the Fortran so
// that, compiled without FMA contraction (-ffp-contract=off), the arithmetic
// matches the reference's x86-64 gfortran -O2 build operation for operation.
#include "poromec_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <cstdio>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---------------------------------------------------------------------------
// Quadrature tables: the literal values of the reference's block data
// (Elmlib.f:3780-3962).  The digits are kept exactly as typed there (15
// digits for Gauss-Legendre, 8 for the tetra rule, div6 = 0.166666666666667)
// because they set the last digits of every element matrix.
// ---------------------------------------------------------------------------
const double PG4[4] = {-.861136311594053, -.339981043584856, .339981043584856,
                       .861136311594053};
const double WG4[4] = {.347854845137454, .652145154862546, .652145154862546,
                       .347854845137454};
const double PG3[3] = {-.774596669241483, 0.0, .774596669241483};
const double WG3[3] = {.555555555555556, .888888888888889, .555555555555556};
// tetra rule of degree 2 (npint4(2) = 4): pri4/psi4/pti4/wf4(.,2)
const double PRI4[4] = {0.58541020, 0.13819660, 0.13819660, 0.13819660};
const double PSI4[4] = {0.13819660, 0.58541020, 0.13819660, 0.13819660};
const double PTI4[4] = {0.13819660, 0.13819660, 0.58541020, 0.13819660};
const double WF4[4] = {0.25, 0.25, 0.25, 0.25};
// triangle rule of degree 2 (npint(2) = 3): pri/psi/wf(.,2)
const double PRI2[3] = {.5, 0.0, .5};
const double PSI2[3] = {.5, .5, 0.0};
const double WF2[3] = {.333333333333333, .333333333333333, .333333333333333};
const double DIV6 = 0.166666666666667;  // Elmlib03.f elmt15_pm parameter
const double SCALE = 1.0e-06;           // density scale, Elmlib03.f

// Face node tables (Elmlib03.f: hexa_face_node20 in elmt17_pm,
// tetra_face_node10 in elmt15_pm), 1-based local node numbers.
const int HEXA_FACE[6][8] = {{1, 2, 3, 4, 9, 10, 11, 12},
                             {5, 6, 7, 8, 13, 14, 15, 16},
                             {1, 5, 6, 2, 17, 13, 18, 9},
                             {4, 3, 7, 8, 11, 19, 15, 20},
                             {1, 4, 8, 5, 12, 20, 16, 17},
                             {2, 6, 7, 3, 18, 14, 19, 10}};
const int TETRA_FACE[4][6] = {{2, 3, 4, 8, 9, 10},
                              {1, 4, 3, 7, 9, 6},
                              {1, 2, 4, 5, 10, 7},
                              {1, 3, 2, 6, 8, 5}};

struct DetError {};

// ---------------------------------------------------------------------------
// Shape functions (Elmlib.f).
// ---------------------------------------------------------------------------
// sfhexa8_m (Elmlib.f:1510-1618)
void sfhexa8_m(double* h, double* hx, double* hy, double* hz, double r,
               double s, double t, bool afl, bool bfl) {
  const double pR = 1.0 + r, pS = 1.0 + s, pT = 1.0 + t;
  const double mR = 1.0 - r, mS = 1.0 - s, mT = 1.0 - t;
  if (afl) {
    h[0] = pR * pS * pT * 0.125;
    h[1] = mR * pS * pT * 0.125;
    h[2] = mR * mS * pT * 0.125;
    h[3] = pR * mS * pT * 0.125;
    h[4] = pR * pS * mT * 0.125;
    h[5] = mR * pS * mT * 0.125;
    h[6] = mR * mS * mT * 0.125;
    h[7] = pR * mS * mT * 0.125;
  }
  if (bfl) {
    hx[0] = pS * pT * 0.125;
    hx[1] = -pS * pT * 0.125;
    hx[2] = -mS * pT * 0.125;
    hx[3] = mS * pT * 0.125;
    hx[4] = pS * mT * 0.125;
    hx[5] = -pS * mT * 0.125;
    hx[6] = -mS * mT * 0.125;
    hx[7] = mS * mT * 0.125;
    hy[0] = pR * pT * 0.125;
    hy[1] = mR * pT * 0.125;
    hy[2] = -mR * pT * 0.125;
    hy[3] = -pR * pT * 0.125;
    hy[4] = pR * mT * 0.125;
    hy[5] = mR * mT * 0.125;
    hy[6] = -mR * mT * 0.125;
    hy[7] = -pR * mT * 0.125;
    hz[0] = pR * pS * 0.125;
    hz[1] = mR * pS * 0.125;
    hz[2] = mR * mS * 0.125;
    hz[3] = pR * mS * 0.125;
    hz[4] = -pR * pS * 0.125;
    hz[5] = -mR * pS * 0.125;
    hz[6] = -mR * mS * 0.125;
    hz[7] = -pR * mS * 0.125;
  }
}

// sfhexa20_m (Elmlib.f:1619-1808)
void sfhexa20_m(double* h, double* hx, double* hy, double* hz, double r,
                double s, double t, bool afl, bool bfl) {
  const double pR = 1.0 + r, pS = 1.0 + s, pT = 1.0 + t;
  const double mR = 1.0 - r, mS = 1.0 - s, mT = 1.0 - t;
  const double mRr = 1.0 - r * r, mSs = 1.0 - s * s, mTt = 1.0 - t * t;
  if (afl) {
    h[0] = pR * pS * pT * (r + s + t - 2.0) * 0.125;
    h[1] = mR * pS * pT * (-r + s + t - 2.0) * 0.125;
    h[2] = mR * mS * pT * (-r - s + t - 2.0) * 0.125;
    h[3] = pR * mS * pT * (r - s + t - 2.0) * 0.125;
    h[4] = pR * pS * mT * (r + s - t - 2.0) * 0.125;
    h[5] = mR * pS * mT * (-r + s - t - 2.0) * 0.125;
    h[6] = mR * mS * mT * (-r - s - t - 2.0) * 0.125;
    h[7] = pR * mS * mT * (r - s - t - 2.0) * 0.125;
    h[8] = mRr * pS * pT * 0.25;
    h[9] = mR * mSs * pT * 0.25;
    h[10] = mRr * mS * pT * 0.25;
    h[11] = pR * mSs * pT * 0.25;
    h[12] = mRr * pS * mT * 0.25;
    h[13] = mR * mSs * mT * 0.25;
    h[14] = mRr * mS * mT * 0.25;
    h[15] = pR * mSs * mT * 0.25;
    h[16] = pR * pS * mTt * 0.25;
    h[17] = mR * pS * mTt * 0.25;
    h[18] = mR * mS * mTt * 0.25;
    h[19] = pR * mS * mTt * 0.25;
  }
  if (bfl) {
    hx[0] = pS * pT * (2.0 * r + s + t - 1.0) * 0.125;
    hx[1] = pS * pT * (2.0 * r - s - t + 1.0) * 0.125;
    hx[2] = mS * pT * (2.0 * r + s - t + 1.0) * 0.125;
    hx[3] = mS * pT * (2.0 * r - s + t - 1.0) * 0.125;
    hx[4] = pS * mT * (2.0 * r + s - t - 1.0) * 0.125;
    hx[5] = pS * mT * (2.0 * r - s + t + 1.0) * 0.125;
    hx[6] = mS * mT * (2.0 * r + s + t + 1.0) * 0.125;
    hx[7] = mS * mT * (2.0 * r - s - t - 1.0) * 0.125;
    hx[8] = -r * pS * pT * 0.50;
    hx[9] = -mSs * pT * 0.25;
    hx[10] = -r * mS * pT * 0.50;
    hx[11] = mSs * pT * 0.25;
    hx[12] = -r * pS * mT * 0.50;
    hx[13] = -mSs * mT * 0.25;
    hx[14] = -r * mS * mT * 0.50;
    hx[15] = mSs * mT * 0.25;
    hx[16] = pS * mTt * 0.25;
    hx[17] = -pS * mTt * 0.25;
    hx[18] = -mS * mTt * 0.25;
    hx[19] = mS * mTt * 0.25;

    hy[0] = pR * pT * (r + 2.0 * s + t - 1.0) * 0.125;
    hy[1] = mR * pT * (-r + 2.0 * s + t - 1.0) * 0.125;
    hy[2] = mR * pT * (r + 2.0 * s - t + 1.0) * 0.125;
    hy[3] = pR * pT * (-r + 2.0 * s - t + 1.0) * 0.125;
    hy[4] = pR * mT * (r + 2.0 * s - t - 1.0) * 0.125;
    hy[5] = mR * mT * (-r + 2.0 * s - t - 1.0) * 0.125;
    hy[6] = mR * mT * (r + 2.0 * s + t + 1.0) * 0.125;
    hy[7] = pR * mT * (-r + 2.0 * s + t + 1.0) * 0.125;
    hy[8] = mRr * pT * 0.25;
    hy[9] = -s * mR * pT * 0.50;
    hy[10] = -mRr * pT * 0.25;
    hy[11] = -s * pR * pT * 0.50;
    hy[12] = mRr * mT * 0.25;
    hy[13] = -s * mR * mT * 0.50;
    hy[14] = -mRr * mT * 0.25;
    hy[15] = -s * pR * mT * 0.50;
    hy[16] = pR * mTt * 0.25;
    hy[17] = mR * mTt * 0.25;
    hy[18] = -mR * mTt * 0.25;
    hy[19] = -pR * mTt * 0.25;

    hz[0] = pR * pS * (r + s + 2.0 * t - 1.0) * 0.125;
    hz[1] = mR * pS * (-r + s + 2.0 * t - 1.0) * 0.125;
    hz[2] = mR * mS * (-r - s + 2.0 * t - 1.0) * 0.125;
    hz[3] = pR * mS * (r - s + 2.0 * t - 1.0) * 0.125;
    hz[4] = pR * pS * (-r - s + 2.0 * t + 1.0) * 0.125;
    hz[5] = mR * pS * (r - s + 2.0 * t + 1.0) * 0.125;
    hz[6] = mR * mS * (r + s + 2.0 * t + 1.0) * 0.125;
    hz[7] = pR * mS * (-r + s + 2.0 * t + 1.0) * 0.125;
    hz[8] = mRr * pS * 0.25;
    hz[9] = mR * mSs * 0.25;
    hz[10] = mRr * mS * 0.25;
    hz[11] = pR * mSs * 0.25;
    hz[12] = -mRr * pS * 0.25;
    hz[13] = -mR * mSs * 0.25;
    hz[14] = -mRr * mS * 0.25;
    hz[15] = -pR * mSs * 0.25;
    hz[16] = -t * pR * pS * 0.50;
    hz[17] = -t * mR * pS * 0.50;
    hz[18] = -t * mR * mS * 0.50;
    hz[19] = -t * pR * mS * 0.50;
  }
}

// sftetra4 (Elmlib.f:942-1012)
void sftetra4(double* h, double* hr, double* hs, double* ht, double r,
              double s, double t, bool afl, bool bfl) {
  const double u = 1.0 - r - s - t;
  if (afl) {
    h[0] = r;
    h[1] = s;
    h[2] = t;
    h[3] = u;
  }
  if (bfl) {
    hr[0] = 1.0; hr[1] = 0.0; hr[2] = 0.0; hr[3] = -1.0;
    hs[0] = 0.0; hs[1] = 1.0; hs[2] = 0.0; hs[3] = -1.0;
    ht[0] = 0.0; ht[1] = 0.0; ht[2] = 1.0; ht[3] = -1.0;
  }
}

// sftetra10 (Elmlib.f:1013-1113)
void sftetra10(double* h, double* hr, double* hs, double* ht, double r,
               double s, double t, bool afl, bool bfl) {
  const double u = 1.0 - r - s - t;
  if (afl) {
    h[0] = r * (2.0 * r - 1.0);
    h[1] = s * (2.0 * s - 1.0);
    h[2] = t * (2.0 * t - 1.0);
    h[3] = u * (2.0 * u - 1.0);
    h[4] = 4.0 * r * s;
    h[5] = 4.0 * r * t;
    h[6] = 4.0 * r * u;
    h[7] = 4.0 * s * t;
    h[8] = 4.0 * t * u;
    h[9] = 4.0 * s * u;
  }
  if (bfl) {
    hr[0] = 4.0 * r - 1.0; hr[1] = 0.0; hr[2] = 0.0;
    hr[3] = 1.0 - 4.0 * u; hr[4] = 4.0 * s; hr[5] = 4.0 * t;
    hr[6] = 4.0 * (u - r); hr[7] = 0.0; hr[8] = -4.0 * t; hr[9] = -4.0 * s;
    hs[0] = 0.0; hs[1] = 4.0 * s - 1.0; hs[2] = 0.0;
    hs[3] = 1.0 - 4.0 * u; hs[4] = 4.0 * r; hs[5] = 0.0;
    hs[6] = -4.0 * r; hs[7] = 4.0 * t; hs[8] = -4.0 * t;
    hs[9] = 4.0 * (u - s);
    ht[0] = 0.0; ht[1] = 0.0; ht[2] = 4.0 * t - 1.0;
    ht[3] = 1.0 - 4.0 * u; ht[4] = 0.0; ht[5] = 4.0 * r;
    ht[6] = -4.0 * r; ht[7] = 4.0 * s; ht[8] = 4.0 * (u - t);
    ht[9] = -4.0 * s;
  }
}

// sftria3 (Elmlib.f:823-877)
void sftria3(double* h, double* hr, double* hs, double r, double s, bool afl,
             bool bfl) {
  const double t = 1.0 - r - s;
  if (afl) {
    h[0] = r; h[1] = s; h[2] = t;
  }
  if (bfl) {
    hr[0] = 1.0; hr[1] = 0.0; hr[2] = -1.0;
    hs[0] = 0.0; hs[1] = 1.0; hs[2] = -1.0;
  }
}

// sftria6 (Elmlib.f:878-941)
void sftria6(double* h, double* hr, double* hs, double r, double s, bool afl,
             bool bfl) {
  const double t = 1.0 - r - s;
  if (afl) {
    h[0] = r * (2.0 * r - 1.0);
    h[1] = s * (2.0 * s - 1.0);
    h[2] = t * (2.0 * t - 1.0);
    h[3] = 4.0 * r * s;
    h[4] = 4.0 * s * t;
    h[5] = 4.0 * t * r;
  }
  if (bfl) {
    hr[0] = 4.0 * r - 1.0; hr[1] = 0.0; hr[2] = 1.0 - 4.0 * t;
    hr[3] = 4.0 * s; hr[4] = -4.0 * s; hr[5] = 4.0 * (t - r);
    hs[0] = 0.0; hs[1] = 4.0 * s - 1.0; hs[2] = 1.0 - 4.0 * t;
    hs[3] = 4.0 * r; hs[4] = 4.0 * (t - s); hs[5] = -4.0 * r;
  }
}

// sfquad4_m (Elmlib.f:1174-1245)
void sfquad4_m(double* h, double* hx, double* hy, double r, double s, bool afl,
               bool bfl) {
  const double pr = 1.0 + r, ps = 1.0 + s, mr = 1.0 - r, ms = 1.0 - s;
  if (afl) {
    h[0] = pr * ps * 0.25;
    h[1] = mr * ps * 0.25;
    h[2] = mr * ms * 0.25;
    h[3] = pr * ms * 0.25;
  }
  if (bfl) {
    hx[0] = ps * 0.25; hx[1] = -ps * 0.25; hx[2] = -ms * 0.25; hx[3] = ms * 0.25;
    hy[0] = pr * 0.25; hy[1] = mr * 0.25; hy[2] = -mr * 0.25; hy[3] = -pr * 0.25;
  }
}

// sfquad8_m (Elmlib.f:1318-1427)
void sfquad8_m(double* h, double* hx, double* hy, double r, double s, bool afl,
               bool bfl) {
  const double pr = 1.0 + r, ps = 1.0 + s, mr = 1.0 - r, ms = 1.0 - s;
  const double mrr = 1.0 - r * r, mss = 1.0 - s * s;
  if (afl) {
    h[4] = mrr * ps * 0.5;
    h[5] = mss * mr * 0.5;
    h[6] = mrr * ms * 0.5;
    h[7] = mss * pr * 0.5;
    const double a5 = h[4] * 0.5, a6 = h[5] * 0.5, a7 = h[6] * 0.5,
                 a8 = h[7] * 0.5;
    h[0] = pr * ps * 0.25 - a5 - a8;
    h[1] = mr * ps * 0.25 - a5 - a6;
    h[2] = mr * ms * 0.25 - a6 - a7;
    h[3] = pr * ms * 0.25 - a7 - a8;
  }
  if (bfl) {
    hx[4] = -r * ps;
    hx[5] = -0.5 * mss;
    hx[6] = -r * ms;
    hx[7] = 0.5 * mss;
    double a5 = hx[4] * 0.5, a6 = hx[5] * 0.5, a7 = hx[6] * 0.5,
           a8 = hx[7] * 0.5;
    hx[0] = ps * 0.25 - a5 - a8;
    hx[1] = -ps * 0.25 - a5 - a6;
    hx[2] = -ms * 0.25 - a6 - a7;
    hx[3] = ms * 0.25 - a7 - a8;
    hy[4] = mrr * 0.5;
    hy[5] = -s * mr;
    hy[6] = -mrr * 0.5;
    hy[7] = -s * pr;
    a5 = hy[4] * 0.5; a6 = hy[5] * 0.5; a7 = hy[6] * 0.5; a8 = hy[7] * 0.5;
    hy[0] = pr * 0.25 - a5 - a8;
    hy[1] = mr * 0.25 - a5 - a6;
    hy[2] = -mr * 0.25 - a6 - a7;
    hy[3] = -pr * 0.25 - a7 - a8;
  }
}

// jacob3d_m (Elmlib.f:2301-2396).  x is (3, nen) column-major.  With afl the
// Jacobian, its determinant (det <= 1e-14 is fatal in the reference) and its
// explicit inverse are formed; the derivatives are always mapped to x,y,z.
void jacob3d_m(double* hx, double* hy, double* hz, double xj[3][3],
               double xji[3][3], const double* x, double& det, int nen,
               bool afl) {
  if (afl) {
    for (int j = 0; j < 3; ++j) {
      xj[0][j] = 0.0;
      xj[1][j] = 0.0;
      xj[2][j] = 0.0;
      for (int k = 0; k < nen; ++k) {
        xj[0][j] = xj[0][j] + hx[k] * x[3 * k + j];
        xj[1][j] = xj[1][j] + hy[k] * x[3 * k + j];
        xj[2][j] = xj[2][j] + hz[k] * x[3 * k + j];
      }
    }
    det = xj[0][0] * xj[1][1] * xj[2][2] + xj[0][1] * xj[1][2] * xj[2][0] +
          xj[0][2] * xj[1][0] * xj[2][1] - xj[2][0] * xj[1][1] * xj[0][2] -
          xj[1][0] * xj[0][1] * xj[2][2] - xj[0][0] * xj[2][1] * xj[1][2];
    if (det <= 1.0e-14) throw DetError();
    xji[0][0] = (xj[1][1] * xj[2][2] - xj[1][2] * xj[2][1]) / det;
    xji[1][0] = -(xj[1][0] * xj[2][2] - xj[1][2] * xj[2][0]) / det;
    xji[2][0] = (xj[1][0] * xj[2][1] - xj[1][1] * xj[2][0]) / det;
    xji[0][1] = -(xj[0][1] * xj[2][2] - xj[0][2] * xj[2][1]) / det;
    xji[1][1] = (xj[0][0] * xj[2][2] - xj[0][2] * xj[2][0]) / det;
    xji[2][1] = -(xj[0][0] * xj[2][1] - xj[0][1] * xj[2][0]) / det;
    xji[0][2] = (xj[0][1] * xj[1][2] - xj[0][2] * xj[1][1]) / det;
    xji[1][2] = -(xj[0][0] * xj[1][2] - xj[0][2] * xj[1][0]) / det;
    xji[2][2] = (xj[0][0] * xj[1][1] - xj[0][1] * xj[1][0]) / det;
  }
  for (int k = 0; k < nen; ++k) {
    const double hxk = hx[k], hyk = hy[k], hzk = hz[k];
    hx[k] = xji[0][0] * hxk + xji[0][1] * hyk + xji[0][2] * hzk;
    hy[k] = xji[1][0] * hxk + xji[1][1] * hyk + xji[1][2] * hzk;
    hz[k] = xji[2][0] * hxk + xji[2][1] * hyk + xji[2][2] * hzk;
  }
}

// jacob2d_m (Elmlib.f:2128-2211) on the first two (rotated) coordinates of
// x(3, nen); only det is used by the callers.
void jacob2d_m(const double* hx, const double* hy, const double* x,
               double& det, int nen) {
  double xj[2][2];
  for (int j = 0; j < 2; ++j) {
    xj[0][j] = 0.0;
    xj[1][j] = 0.0;
    for (int k = 0; k < nen; ++k) {
      xj[0][j] = xj[0][j] + hx[k] * x[3 * k + j];
      xj[1][j] = xj[1][j] + hy[k] * x[3 * k + j];
    }
  }
  det = xj[0][0] * xj[1][1] - xj[1][0] * xj[0][1];
  if (det <= 1.0e-14) throw DetError();
}

// rotmatrix (Elmlib.f:2397-2446)
void rotmatrix(const double* x, double r[3][3]) {
  const double v1x = x[3] - x[0], v1y = x[4] - x[1], v1z = x[5] - x[2];
  double v2x = x[6] - x[0], v2y = x[7] - x[1], v2z = x[8] - x[2];
  const double v3x = v1y * v2z - v1z * v2y;
  const double v3y = v1z * v2x - v1x * v2z;
  const double v3z = v1x * v2y - v1y * v2x;
  v2x = v1z * v3y - v1y * v3z;
  v2y = v1x * v3z - v1z * v3x;
  v2z = v1y * v3x - v1x * v3y;
  const double n1 = std::sqrt(v1x * v1x + v1y * v1y + v1z * v1z);
  const double n2 = std::sqrt(v2x * v2x + v2y * v2y + v2z * v2z);
  const double n3 = std::sqrt(v3x * v3x + v3y * v3y + v3z * v3z);
  r[0][0] = v1x / n1; r[0][1] = v1y / n1; r[0][2] = v1z / n1;
  r[1][0] = v2x / n2; r[1][1] = v2y / n2; r[1][2] = v2z / n2;
  r[2][0] = v3x / n3; r[2][1] = v3y / n3; r[2][2] = v3z / n3;
}

// rotate (Elmlib.f:2518-2544), transp = .false., in place
void rotate(double* x, const double r[3][3]) {
  const double x1 = r[0][0] * x[0] + r[0][1] * x[1] + r[0][2] * x[2];
  const double x2 = r[1][0] * x[0] + r[1][1] * x[1] + r[1][2] * x[2];
  const double x3 = r[2][0] * x[0] + r[2][1] * x[1] + r[2][2] * x[2];
  x[0] = x1; x[1] = x2; x[2] = x3;
}

// face_normal_vector (Elmlib.f:3678-3728): normal = (x3-x1) x (x2-x1), unit
void face_normal_vector(const double* xf, double* nrm) {
  const double v1[3] = {xf[3] - xf[0], xf[4] - xf[1], xf[5] - xf[2]};
  const double v2[3] = {xf[6] - xf[0], xf[7] - xf[1], xf[8] - xf[2]};
  nrm[0] = v2[1] * v1[2] - v2[2] * v1[1];
  nrm[1] = v2[2] * v1[0] - v2[0] * v1[2];
  nrm[2] = v2[0] * v1[1] - v2[1] * v1[0];
  double tmp = std::sqrt(nrm[0] * nrm[0] + nrm[1] * nrm[1] + nrm[2] * nrm[2]);
  tmp = 1.0 / tmp;
  nrm[0] *= tmp; nrm[1] *= tmp; nrm[2] *= tmp;
}

// face_ponto_medio (Elmlib.f:3729)
void face_midpoint(const double* xf, int n, double* mp) {
  mp[0] = mp[1] = mp[2] = 0.0;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < 3; ++j) mp[j] = mp[j] + xf[3 * i + j];
  for (int j = 0; j < 3; ++j) mp[j] = mp[j] / n;
}

// deform3d (Elmlib.f:2774-2836)
void deform3d(const double* hx, const double* hy, const double* hz,
              const double* u, double* eps, int nen) {
  double ux = 0, uy = 0, uz = 0, vx = 0, vy = 0, vz = 0, wx = 0, wy = 0, wz = 0;
  for (int i = 0; i < nen; ++i) {
    const double a = u[3 * i], b = u[3 * i + 1], c = u[3 * i + 2];
    ux = ux + hx[i] * a; uy = uy + hy[i] * a; uz = uz + hz[i] * a;
    vx = vx + hx[i] * b; vy = vy + hy[i] * b; vz = vz + hz[i] * b;
    wx = wx + hx[i] * c; wy = wy + hy[i] * c; wz = wz + hz[i] * c;
  }
  eps[0] = ux; eps[1] = vy; eps[2] = wz;
  eps[3] = uy + vx; eps[4] = vz + wy; eps[5] = uz + wx;
}

// stress3d (Elmlib.f:2906-2939)
void stress3d(double a, double b, double c, const double* eps, double* t) {
  t[0] = (eps[0] + b * eps[1] + b * eps[2]) * a;
  t[1] = (b * eps[0] + eps[1] + b * eps[2]) * a;
  t[2] = (b * eps[0] + b * eps[1] + eps[2]) * a;
  t[3] = eps[3] * c * a;
  t[4] = eps[4] * c * a;
  t[5] = eps[5] * c * a;
}

// interpol (Interpolation.f:1-32)
double interpol(const double* xs, const double* ys, double xi, int n) {
  if (xi <= xs[0]) return ys[0];
  if (xi >= xs[n - 1]) return ys[n - 1];
  for (int i = 0; i < n - 1; ++i) {
    const double x1 = xs[i], x2 = xs[i + 1], y1 = ys[i], y2 = ys[i + 1];
    if (xi >= x1 && xi <= x2) return y1 + (y2 - y1) * (xi - x1) / (x2 - x1);
  }
  return 0.0;
}

struct Loads {
  int nloads = 0, maxt = 1;
  std::vector<int32_t> load;   // (3, nloads): type, nparc, ntime
  std::vector<double> fload;   // (maxt, OR_NFLOAD, nloads)
  double f(int l, int k, int nc) const {  // Fortran fload(l,k,nc), 1-based
    return fload[(size_t)(l - 1) + (size_t)maxt * ((k - 1) + OR_NFLOAD * (size_t)(nc - 1))];
  }
  const double* col(int k, int nc) const {
    return &fload[(size_t)maxt * ((k - 1) + OR_NFLOAD * (size_t)(nc - 1))];
  }
  int type(int nc) const { return load[3 * (nc - 1)]; }
};

// tload (Pload.f:220-377): value c (scalar loads) or vc (vector load 40) at
// time t; x is the point used by the hydrostatic type 42.
void tload(const Loads& L, int nc, double t, const double* x, double u,
           double& c, double* vc, double gravity_mod) {
  c = 0.0;
  if (nc <= 0) return;
  const int itype = L.load[3 * (nc - 1)];
  int nparc = L.load[3 * (nc - 1) + 1];
  const double DOISPI = 6.283185307;
  if (itype == 1) {
    c = L.f(1, 1, nc);
  } else if (itype == 2) {
    c = L.f(1, 1, nc) + L.f(2, 1, nc) * t;
  } else if (itype == 3) {
    c = (L.f(1, 1, nc) - u) * L.f(2, 1, nc);
  } else if (itype == 4 || itype == 5) {
    for (int i = 1; i <= nparc; ++i) {
      const double a = L.f(1, i, nc), w = 1.0 / L.f(2, i, nc), t0 = L.f(3, i, nc);
      const double ti = std::max(t - t0, 0.0);
      c = c + a * (itype == 4 ? std::sin(DOISPI * w * ti) : std::cos(DOISPI * w * ti));
    }
  } else if (itype == 39) {
    nparc = L.load[3 * (nc - 1) + 2];
    c = interpol(L.col(1, nc), L.col(2, nc), t, nparc);
  } else if (itype == 40) {
    nparc = L.load[3 * (nc - 1) + 2];
    vc[0] = interpol(L.col(1, nc), L.col(2, nc), t, nparc);
    vc[1] = interpol(L.col(1, nc), L.col(3, nc), t, nparc);
    vc[2] = interpol(L.col(1, nc), L.col(4, nc), t, nparc);
  } else if (itype == 41 || itype == 43) {
    nparc = L.load[3 * (nc - 1) + 2];
    c = interpol(L.col(1, nc), L.col(2, nc), t, nparc);
  } else if (itype == 42) {
    nparc = L.load[3 * (nc - 1) + 2];
    const double a = interpol(L.col(1, nc), L.col(2, nc), t, nparc);
    const double b = interpol(L.col(1, nc), L.col(3, nc), t, nparc);
    const double w = interpol(L.col(1, nc), L.col(4, nc), t, nparc);
    const double t0 = interpol(L.col(1, nc), L.col(5, nc), t, nparc);
    const double hh = (w - x[2]);
    c = t0 * (b + a * hh * gravity_mod);
  }
}

struct Env {
  double gravity[3] = {0.0, 0.0, -9.81};
  double gravity_mod = 9.81;
  double dt = 1.0, t = 0.0;
  int istep = 0;
};

// ---------------------------------------------------------------------------
// Elastic Biot elements: elmt17_pm (hexa20, Elmlib03.f:1822-2636) and
// elmt15_pm (tetra10, Elmlib03.f:59-854) for isw = 2, 4, 5.
// s(nst,nst) column-major; u, p, dp local.  txn(6,nen) nodal initial stress.
// ---------------------------------------------------------------------------
struct Mat {
  double a, b, c, coef_biot, imod_biot, dt_perm, dt_fluid_perm, pm_d, fluid_d,
      perm;
};

Mat material(const double* e, const Env& env) {
  Mat m;
  m.pm_d = e[5] * SCALE;
  m.fluid_d = e[6] * SCALE;
  const double fluid_sw = m.fluid_d * env.gravity_mod;
  const double ym = e[0], ps = e[1];
  m.perm = e[2] / fluid_sw;
  m.imod_biot = 1.0 / e[3];
  m.coef_biot = e[4];
  m.dt_perm = m.perm * env.dt;
  m.dt_fluid_perm = m.fluid_d * m.dt_perm;
  const double a1 = 1.0 - ps, a2 = 1.0 - 2.0 * ps, a3 = 1.0 + ps;
  m.a = (ym * a1) / (a3 * a2);
  m.b = ps / a1;
  m.c = 0.5 * (a2 / a1);
  return m;
}

// lku_m (Elmlib.f:695-728)
void lku_m(const double* s, const double* u, double* p, int nst) {
  for (int i = 0; i < nst; ++i) p[i] = 0.0;
  for (int j = 0; j < nst; ++j)
    for (int i = 0; i < nst; ++i) p[i] = p[i] + s[i + (size_t)nst * j] * u[j];
}

// Kuu, Kpu, Kpp accumulation shared by the two elements (Elmlib03.f
// 2079-2137 / 297-369), nu = number of displacement nodes, np = vertices.
inline void kuu_gp(double* s, int nst, int nu, const double* hux,
                   const double* huy, const double* huz, double w,
                   const Mat& m) {
  const double wt1 = w * m.a, b = m.b, c = m.c;
#define S(l, k) s[(l) - 1 + (size_t)nst * ((k) - 1)]
  for (int i = 1; i <= nu; ++i) {
    const int l1 = 3 * i - 2, l2 = l1 + 1, l3 = l2 + 1;
    const double hxi = hux[i - 1], hyi = huy[i - 1], hzi = huz[i - 1];
    for (int j = 1; j <= nu; ++j) {
      const int k1 = 3 * j - 2, k2 = k1 + 1, k3 = k2 + 1;
      const double hxj = hux[j - 1], hyj = huy[j - 1], hzj = huz[j - 1];
      S(l1, k1) = S(l1, k1) + (hxi * hxj + c * (hyi * hyj + hzi * hzj)) * wt1;
      S(l1, k2) = S(l1, k2) + (b * hxi * hyj + c * hyi * hxj) * wt1;
      S(l1, k3) = S(l1, k3) + (b * hxi * hzj + c * hzi * hxj) * wt1;
      S(l2, k1) = S(l2, k1) + (b * hyi * hxj + c * hxi * hyj) * wt1;
      S(l2, k2) = S(l2, k2) + (hyi * hyj + c * (hxi * hxj + hzi * hzj)) * wt1;
      S(l2, k3) = S(l2, k3) + (b * hyi * hzj + c * hzi * hyj) * wt1;
      S(l3, k1) = S(l3, k1) + (b * hzi * hxj + c * hxi * hzj) * wt1;
      S(l3, k2) = S(l3, k2) + (b * hzi * hyj + c * hyi * hzj) * wt1;
      S(l3, k3) = S(l3, k3) + (hzi * hzj + c * (hyi * hyj + hxi * hxj)) * wt1;
    }
  }
}

inline void kpu_kpp_gp(double* s, int nst, int nu, int np, const double* hux,
                       const double* huy, const double* huz, const double* hp,
                       const double* hpx, const double* hpy, const double* hpz,
                       double w, const Mat& m) {
  const int off = 3 * nu;
  double wt2 = w * m.coef_biot;
  for (int i = 1; i <= np; ++i) {
    const int l = i + off;
    const double wt1 = hp[i - 1] * wt2;
    for (int j = 1; j <= nu; ++j) {
      const int k1 = 3 * j - 2, k2 = k1 + 1, k3 = k2 + 1;
      S(l, k1) = S(l, k1) - hux[j - 1] * wt1;
      S(l, k2) = S(l, k2) - huy[j - 1] * wt1;
      S(l, k3) = S(l, k3) - huz[j - 1] * wt1;
    }
  }
  const double wt1 = w * m.imod_biot;
  wt2 = w * m.dt_perm;
  for (int i = 1; i <= np; ++i) {
    const int l = i + off;
    for (int j = 1; j <= np; ++j) {
      const int k = j + off;
      S(l, k) = S(l, k) - wt1 * hp[i - 1] * hp[j - 1] -
                wt2 * (hpx[i - 1] * hpx[j - 1] + hpy[i - 1] * hpy[j - 1] +
                       hpz[i - 1] * hpz[j - 1]);
    }
  }
}

inline void kup_copy(double* s, int nst, int nu, int np) {
  const int off = 3 * nu;
  for (int i = 1; i <= np; ++i) {
    const int l = i + off;
    for (int j = 1; j <= nu; ++j) {
      const int k1 = 3 * j - 2, k2 = k1 + 1, k3 = k2 + 1;
      S(k1, l) = S(l, k1);
      S(k2, l) = S(l, k2);
      S(k3, l) = S(l, k3);
    }
  }
}
#undef S

// isw = 4 contribution at one integration point (Elmlib03.f:2263-2350 /
// 497-585): internal force of the previous state and body forces.
inline void rhs_gp(double* p, int nu, int np, const double* hu,
                   const double* hux, const double* huy, const double* huz,
                   const double* hp, const double* hpx, const double* hpy,
                   const double* hpz, const double* u, const double* dp,
                   double w, const Mat& m, const Env& env) {
  const double* gl = env.gravity;
  const int off = 3 * nu;
  double epsi[6], txi[6];
  deform3d(hux, huy, huz, u, epsi, nu);
  stress3d(m.a, m.b, m.c, epsi, txi);
  double dpm = 0.0;
  if (np == 8) {
    dpm = hp[0] * dp[0] + hp[1] * dp[1] + hp[2] * dp[2] + hp[3] * dp[3] +
          hp[4] * dp[4] + hp[5] * dp[5] + hp[6] * dp[6] + hp[7] * dp[7];
  } else {
    dpm = hp[0] * dp[0] + hp[1] * dp[1] + hp[2] * dp[2] + hp[3] * dp[3];
  }
  dpm = m.coef_biot * dpm;
  txi[0] = txi[0] - dpm;
  txi[1] = txi[1] - dpm;
  txi[2] = txi[2] - dpm;
  double wt1 = w, wt2 = w * m.pm_d;
  for (int i = 1; i <= nu; ++i) {
    const int l1 = 3 * i - 2, l2 = l1 + 1, l3 = l2 + 1;
    const double hxi = hux[i - 1], hyi = huy[i - 1], hzi = huz[i - 1];
    p[l1 - 1] = p[l1 - 1] + wt1 * (hxi * txi[0] + hyi * txi[3] + hzi * txi[5]);
    p[l2 - 1] = p[l2 - 1] + wt1 * (hxi * txi[3] + hyi * txi[1] + hzi * txi[4]);
    p[l3 - 1] = p[l3 - 1] + wt1 * (hxi * txi[5] + hyi * txi[4] + hzi * txi[2]);
    const double wt3 = hu[i - 1] * wt2;
    p[l1 - 1] = p[l1 - 1] - wt3 * gl[0];
    p[l2 - 1] = p[l2 - 1] - wt3 * gl[1];
    p[l3 - 1] = p[l3 - 1] - wt3 * gl[2];
  }
  wt1 = w * m.dt_fluid_perm;
  wt2 = w * m.dt_perm;
  for (int i = 1; i <= np; ++i) {
    const int l = i + off;
    p[l - 1] = p[l - 1] + wt1 * (hpx[i - 1] * gl[0] + hpy[i - 1] * gl[1] +
                                 hpz[i - 1] * gl[2]);
    double tmp = 0.0;
    for (int j = 1; j <= np; ++j) {
      const int k = j + off;
      tmp = tmp + wt2 * u[k - 1] *
                      (hpx[i - 1] * hpx[j - 1] + hpy[i - 1] * hpy[j - 1] +
                       hpz[i - 1] * hpz[j - 1]);
    }
    p[l - 1] = p[l - 1] - tmp;
  }
}

// Face tractions and fluxes of isw = 4 (Elmlib03.f:2352-2520 hexa20,
// :587-752 tetra10).
void face_loads(double* p, bool hexa, const int* iqm, const int* iqh,
                const double* x, const Loads& L, const Env& env) {
  const int nface = hexa ? 6 : 4;
  const int nfv = hexa ? 4 : 3;      // face vertices
  const int nfn = hexa ? 8 : 6;      // face nodes
  const int nu = hexa ? 20 : 10;
  int tpm = 0, tph = 0;
  for (int i = 0; i < nface; ++i) {
    tpm += iqm[i];
    tph += iqh[i];
  }
  if (!(tpm > 0 || tph > 0)) return;
  for (int j = 1; j <= nface; ++j) {
    if (!(iqm[j - 1] > 0 || iqh[j - 1] > 0)) continue;
    const int* fnode = hexa ? HEXA_FACE[j - 1] : TETRA_FACE[j - 1];
    double xf[12];
    for (int i = 0; i < nfv; ++i) {
      const int no = fnode[i];
      xf[3 * i + 0] = x[3 * (no - 1) + 0];
      xf[3 * i + 1] = x[3 * (no - 1) + 1];
      xf[3 * i + 2] = x[3 * (no - 1) + 2];
    }
    const int cargm = iqm[j - 1] != 0 ? L.type(iqm[j - 1]) : 0;
    const int cargh = iqh[j - 1] != 0 ? L.type(iqh[j - 1]) : 0;
    double face_f[3] = {0.0, 0.0, 0.0}, mp[3] = {0.0, 0.0, 0.0};
    double n_carg = 0.0, ddum = 0.0, face_u = 0.0, rr[3][3];
    if (cargm == 40 || cargm == 41 || cargm == 42) {
      if (hexa) {
        if (cargm == 41) {
          face_normal_vector(xf, face_f);
          if (j != 2) {
            face_f[0] = -face_f[0]; face_f[1] = -face_f[1]; face_f[2] = -face_f[2];
          }
        }
      } else {
        if (cargm == 41 || cargm == 42) {
          face_normal_vector(xf, face_f);
          if (cargm == 42) face_midpoint(xf, 3, mp);
        }
      }
      rotmatrix(xf, rr);
      for (int i = 0; i < nfv; ++i) rotate(&xf[3 * i], rr);
      if (cargm == 41 || cargm == 42) {
        tload(L, iqm[j - 1], env.t, mp, face_u, n_carg, &ddum, env.gravity_mod);
        face_f[0] = n_carg * face_f[0];
        face_f[1] = n_carg * face_f[1];
        face_f[2] = n_carg * face_f[2];
      } else {
        tload(L, iqm[j - 1], env.t, mp, face_u, ddum, face_f, env.gravity_mod);
      }
      double hp[8], hpx[8], hpy[8], hu[8], hux[8], huy[8], det;
      if (hexa) {
        for (int ly = 0; ly < 3; ++ly) {
          const double si = PG3[ly];
          for (int lx = 0; lx < 3; ++lx) {
            const double ri = PG3[lx];
            sfquad4_m(hp, hpx, hpy, ri, si, false, true);
            jacob2d_m(hpx, hpy, xf, det, 4);
            const double w = WG3[lx] * WG3[ly] * det;
            sfquad8_m(hu, hux, huy, ri, si, true, false);
            for (int i = 0; i < nfn; ++i) {
              const int no = fnode[i];
              const double wt1 = hu[i] * w;
              const int l1 = 3 * no - 2;
              p[l1 - 1] = p[l1 - 1] - face_f[0] * wt1;
              p[l1] = p[l1] - face_f[1] * wt1;
              p[l1 + 1] = p[l1 + 1] - face_f[2] * wt1;
            }
          }
        }
      } else {
        for (int lx = 0; lx < 3; ++lx) {
          const double ri = PRI2[lx], si = PSI2[lx];
          sftria3(hp, hpx, hpy, ri, si, false, true);
          jacob2d_m(hpx, hpy, xf, det, 3);
          double w = WF2[lx] * det;
          w = 0.5 * w;
          sftria6(hu, hux, huy, ri, si, true, false);
          for (int i = 0; i < nfn; ++i) {
            const int no = fnode[i];
            const double wt1 = hu[i] * w;
            const int l1 = 3 * no - 2;
            p[l1 - 1] = p[l1 - 1] - face_f[0] * wt1;
            p[l1] = p[l1] - face_f[1] * wt1;
            p[l1 + 1] = p[l1 + 1] - face_f[2] * wt1;
          }
        }
      }
    }
    if (cargh == 43) {
      // the reference rotates xf again here (a second rotation of already
      // rotated points when a mechanical load was applied on the same face)
      rotmatrix(xf, rr);
      for (int i = 0; i < nfv; ++i) rotate(&xf[3 * i], rr);
      tload(L, iqh[j - 1], env.t, mp, face_u, n_carg, &ddum, env.gravity_mod);
      double hp[8], hpx[8], hpy[8], det;
      if (hexa) {
        for (int ly = 0; ly < 3; ++ly) {
          const double si = PG3[ly];
          for (int lx = 0; lx < 3; ++lx) {
            const double ri = PG3[lx];
            sfquad4_m(hp, hpx, hpy, ri, si, true, true);
            jacob2d_m(hpx, hpy, xf, det, 4);
            double w = WG3[lx] * WG3[ly] * det;
            w = w * env.dt * n_carg;
            for (int i = 0; i < 4; ++i) {
              const int no = fnode[i];
              const double wt1 = hp[i] * w;
              p[3 * nu + no - 1] = p[3 * nu + no - 1] - wt1;
            }
          }
        }
      } else {
        for (int lx = 0; lx < 3; ++lx) {
          const double ri = PRI2[lx], si = PSI2[lx];
          sftria3(hp, hpx, hpy, ri, si, true, true);
          jacob2d_m(hpx, hpy, xf, det, 3);
          double w = WF2[lx] * det;
          w = 0.5 * w * env.dt * n_carg;
          for (int i = 0; i < 3; ++i) {
            const int no = fnode[i];
            const double wt1 = hp[i] * w;
            p[3 * nu + no - 1] = p[3 * nu + no - 1] - wt1;
          }
        }
      }
    }
  }
}

// One element call.  hexa: elmt17_pm, else elmt15_pm.  x(3,nenv) vertex
// coordinates; txn(6,nenv) nodal initial stress for isw = 5.
void element(bool hexa, const double* e, const int* iqm, const int* iqh,
             const double* x, const double* u, const double* dp, double* p,
             double* s, const double* txn, int isw, const Loads& L,
             const Env& env) {
  const int nu = hexa ? 20 : 10, np = hexa ? 8 : 4;
  const int nst = 3 * nu + np;
  const Mat m = material(e, env);
  double hu[20], hux[20], huy[20], huz[20], hp[8], hpx[8], hpy[8], hpz[8];
  double xj[3][3], xji[3][3], det;
  const int ngp = hexa ? 64 : 4;
  auto gauss_point = [&](int g, double& ri, double& si, double& ti,
                         double& wq) {
    if (hexa) {
      const int lz = g / 16, ly = (g / 4) % 4, lx = g % 4;
      ri = PG4[lx]; si = PG4[ly]; ti = PG4[lz];
      wq = WG4[lx] * WG4[ly] * WG4[lz];
    } else {
      ri = PRI4[g]; si = PSI4[g]; ti = PTI4[g];
      wq = WF4[g];
    }
  };
  if (isw == 2) {
    for (int i = 0; i < nst * nst; ++i) s[i] = 0.0;
    for (int i = 0; i < nst; ++i) p[i] = 0.0;
    for (int g = 0; g < ngp; ++g) {
      double ri, si, ti, wq, w;
      gauss_point(g, ri, si, ti, wq);
      if (hexa) {
        sfhexa8_m(hp, hpx, hpy, hpz, ri, si, ti, true, true);
        jacob3d_m(hpx, hpy, hpz, xj, xji, x, det, 8, true);
        w = wq * det;
        sfhexa20_m(hu, hux, huy, huz, ri, si, ti, false, true);
        jacob3d_m(hux, huy, huz, xj, xji, x, det, 20, false);
      } else {
        sftetra4(hp, hpx, hpy, hpz, ri, si, ti, true, true);
        jacob3d_m(hpx, hpy, hpz, xj, xji, x, det, 4, true);
        w = wq * det;
        w = w * DIV6;
        sftetra10(hu, hux, huy, huz, ri, si, ti, false, true);
        jacob3d_m(hux, huy, huz, xj, xji, x, det, 10, false);
      }
      kuu_gp(s, nst, nu, hux, huy, huz, w, m);
      kpu_kpp_gp(s, nst, nu, np, hux, huy, huz, hp, hpx, hpy, hpz, w, m);
    }
    kup_copy(s, nst, nu, np);
    lku_m(s, u, p, nst);
  } else if (isw == 4) {
    for (int g = 0; g < ngp; ++g) {
      double ri, si, ti, wq, w;
      gauss_point(g, ri, si, ti, wq);
      if (hexa) {
        sfhexa8_m(hp, hpx, hpy, hpz, ri, si, ti, true, true);
        jacob3d_m(hpx, hpy, hpz, xj, xji, x, det, 8, true);
        w = wq * det;
        sfhexa20_m(hu, hux, huy, huz, ri, si, ti, true, true);
        jacob3d_m(hux, huy, huz, xj, xji, x, det, 20, false);
      } else {
        sftetra4(hp, hpx, hpy, hpz, ri, si, ti, true, true);
        jacob3d_m(hpx, hpy, hpz, xj, xji, x, det, 4, true);
        w = wq * det;
        w = w * DIV6;
        sftetra10(hu, hux, huy, huz, ri, si, ti, true, true);
        jacob3d_m(hux, huy, huz, xj, xji, x, det, 10, false);
      }
      rhs_gp(p, nu, np, hu, hux, huy, huz, hp, hpx, hpy, hpz, u, dp, w, m, env);
    }
    face_loads(p, hexa, iqm, iqh, x, L, env);
  } else if (isw == 3) {
    // stresses and fluxes at the vertices (Elmlib03.f:2206-2256 hexa20,
    // :440-495 tetra10): p(6 i ..) total stress D eps - alpha dp, then
    // p(6 np + 6 i ..) the Biot effective stress (total + alpha p), then
    // p(12 np + 3 i ..) the Darcy flux perm (rho_f g - grad p)
    static const double RNH[8] = {1, -1, -1, 1, 1, -1, -1, 1};
    static const double SNH[8] = {1, 1, -1, -1, 1, 1, -1, -1};
    static const double TNH[8] = {1, 1, 1, 1, -1, -1, -1, -1};
    static const double RNT[4] = {1, 0, 0, 0}, SNT[4] = {0, 1, 0, 0}, TNT[4] = {0, 0, 1, 0};
    for (int i = 0; i < np; ++i) {
      const double ri = hexa ? RNH[i] : RNT[i], si = hexa ? SNH[i] : SNT[i],
                   ti = hexa ? TNH[i] : TNT[i];
      if (hexa) {
        sfhexa8_m(hp, hpx, hpy, hpz, ri, si, ti, false, true);
        jacob3d_m(hpx, hpy, hpz, xj, xji, x, det, 8, true);
        sfhexa20_m(hu, hux, huy, huz, ri, si, ti, false, true);
        jacob3d_m(hux, huy, huz, xj, xji, x, det, 20, false);
      } else {
        sftetra4(hp, hpx, hpy, hpz, ri, si, ti, false, true);
        jacob3d_m(hpx, hpy, hpz, xj, xji, x, det, 4, true);
        sftetra10(hu, hux, huy, huz, ri, si, ti, false, true);
        jacob3d_m(hux, huy, huz, xj, xji, x, det, 10, false);
      }
      double epsi[6];
      double* t = p + 6 * i;
      double* tb = p + 6 * np + 6 * i;
      deform3d(hux, huy, huz, u, epsi, nu);
      stress3d(m.a, m.b, m.c, epsi, t);
      const double dpm = m.coef_biot * dp[i];
      const double pm = m.coef_biot * u[3 * nu + i];
      t[0] = t[0] - dpm;
      t[1] = t[1] - dpm;
      t[2] = t[2] - dpm;
      tb[0] = t[0] + pm;
      tb[1] = t[1] + pm;
      tb[2] = t[2] + pm;
      tb[3] = t[3];
      tb[4] = t[4];
      tb[5] = t[5];
    }
    for (int i = 0; i < np; ++i) {
      const double ri = hexa ? RNH[i] : RNT[i], si = hexa ? SNH[i] : SNT[i],
                   ti = hexa ? TNH[i] : TNT[i];
      if (hexa) {
        sfhexa8_m(hp, hpx, hpy, hpz, ri, si, ti, true, true);
        jacob3d_m(hpx, hpy, hpz, xj, xji, x, det, 8, true);
      } else {
        sftetra4(hp, hpx, hpy, hpz, ri, si, ti, true, true);
        jacob3d_m(hpx, hpy, hpz, xj, xji, x, det, 4, true);
      }
      // darcy_flux (Elmlib.f:3178-3200)
      double* q = p + 12 * np + 3 * i;
      q[0] = m.fluid_d * env.gravity[0];
      q[1] = m.fluid_d * env.gravity[1];
      q[2] = m.fluid_d * env.gravity[2];
      for (int k = 0; k < np; ++k) {
        q[0] = q[0] - hpx[k] * u[3 * nu + k];
        q[1] = q[1] - hpy[k] * u[3 * nu + k];
        q[2] = q[2] - hpz[k] * u[3 * nu + k];
      }
      q[0] = m.perm * q[0];
      q[1] = m.perm * q[1];
      q[2] = m.perm * q[2];
    }
  } else if (isw == 7) {
    // porosity change at the vertices (Elmlib03.f:2605-2631 hexa20, the
    // tetra10 twin in elmt15_pm): p(i) = alpha tr(eps(du)) + dp_i / M with u
    // the step's increments
    static const double RNH[8] = {1, -1, -1, 1, 1, -1, -1, 1};
    static const double SNH[8] = {1, 1, -1, -1, 1, 1, -1, -1};
    static const double TNH[8] = {1, 1, 1, 1, -1, -1, -1, -1};
    static const double RNT[4] = {1, 0, 0, 0}, SNT[4] = {0, 1, 0, 0}, TNT[4] = {0, 0, 1, 0};
    for (int i = 0; i < np; ++i) {
      const double ri = hexa ? RNH[i] : RNT[i], si = hexa ? SNH[i] : SNT[i],
                   ti = hexa ? TNH[i] : TNT[i];
      if (hexa) {
        sfhexa8_m(hp, hpx, hpy, hpz, ri, si, ti, false, true);
        jacob3d_m(hpx, hpy, hpz, xj, xji, x, det, 8, true);
        sfhexa20_m(hu, hux, huy, huz, ri, si, ti, false, true);
        jacob3d_m(hux, huy, huz, xj, xji, x, det, 20, false);
      } else {
        sftetra4(hp, hpx, hpy, hpz, ri, si, ti, false, true);
        jacob3d_m(hpx, hpy, hpz, xj, xji, x, det, 4, true);
        sftetra10(hu, hux, huy, huz, ri, si, ti, false, true);
        jacob3d_m(hux, huy, huz, xj, xji, x, det, 10, false);
      }
      double epsi[6];
      deform3d(hux, huy, huz, u, epsi, nu);
      const double pi = m.imod_biot * u[3 * nu + i];
      p[i] = m.coef_biot * (epsi[0] + epsi[1] + epsi[2]) + pi;
    }
  } else if (isw == 5) {
    for (int g = 0; g < ngp; ++g) {
      double ri, si, ti, wq, w;
      gauss_point(g, ri, si, ti, wq);
      if (hexa) {
        sfhexa8_m(hp, hpx, hpy, hpz, ri, si, ti, true, true);
        jacob3d_m(hpx, hpy, hpz, xj, xji, x, det, 8, true);
        w = wq * det;
        sfhexa20_m(hu, hux, huy, huz, ri, si, ti, false, true);
        jacob3d_m(hux, huy, huz, xj, xji, x, det, 20, false);
      } else {
        sftetra4(hp, hpx, hpy, hpz, ri, si, ti, true, true);
        jacob3d_m(hpx, hpy, hpz, xj, xji, x, det, 4, true);
        w = wq * det;
        w = w * DIV6;
        sftetra10(hu, hux, huy, huz, ri, si, ti, false, true);
        jacob3d_m(hux, huy, huz, xj, xji, x, det, 10, false);
      }
      double txi[6] = {0, 0, 0, 0, 0, 0};
      for (int j = 0; j < np; ++j)
        for (int k = 0; k < 6; ++k) txi[k] = txi[k] + hp[j] * txn[6 * j + k];
      for (int i = 1; i <= nu; ++i) {
        const int l1 = 3 * i - 2;
        const double hxi = hux[i - 1], hyi = huy[i - 1], hzi = huz[i - 1];
        p[l1 - 1] = p[l1 - 1] + w * (hxi * txi[0] + hyi * txi[3] + hzi * txi[5]);
        p[l1] = p[l1] + w * (hxi * txi[3] + hyi * txi[1] + hzi * txi[4]);
        p[l1 + 1] = p[l1 + 1] + w * (hxi * txi[5] + hyi * txi[4] + hzi * txi[2]);
      }
    }
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// Handle
// ---------------------------------------------------------------------------
struct or_handle_s {
  int nnode, nnodev, numel, nen, nenv, ndf, nst;
  std::vector<int32_t> ix, idr, fnno, ie, num;  // idr: equation numbers
  std::vector<double> x, e;
  int numat;
  bool hexa;
  int neq = 0;
  int64_t nad = 0;
  std::vector<int64_t> ia;  // 1-based values, size neq+1
  std::vector<int32_t> ja;  // 1-based columns
  std::vector<double> ad, al;
  std::vector<int32_t> eload, eloadp, nload;
  std::vector<double> f;  // (ndf, nnode) nodal values
  Loads L;
  Env env;
  std::vector<double> u, u0, dp, b0, b, x0, m, bst0;
  std::vector<double> poro;  // nodal porosity (vertex nodes)
  int nkrylov = 150;         // GMRES(l) basis size, ngram (Main.f:274)
  bool fstress0 = false;
  int numcolors = 0;
  std::vector<int32_t> color_ptr, color_elems;  // elements grouped by colour
  std::vector<int32_t> thr_begin, thr_end, thr_height;  // SpMV partition
  int thr_n = 0;
  double resu0 = 0.0, resp0 = 0.0, res0 = 0.0;  // 'save' variables of cal_residuo_pm
};

namespace {

// Element colouring by vertex incidence (the semantics of Colormsh.f:160-254:
// no two elements of one colour share a vertex; greedy in element order).
void colour_mesh(or_handle_s* h) {
  std::vector<std::vector<int>> node_colours(h->nnode + 1);
  std::vector<int> col(h->numel, -1);
  int ncol = 0;
  for (int el = 0; el < h->numel; ++el) {
    const int32_t* nodes = &h->ix[(size_t)(h->nen + 1) * el];
    std::vector<char> used(ncol + 1, 0);
    for (int k = 0; k < h->nenv; ++k)
      for (int c : node_colours[nodes[k]]) used[c] = 1;
    int c = 0;
    while (c < ncol && used[c]) ++c;
    if (c == ncol) ++ncol;
    col[el] = c;
    for (int k = 0; k < h->nenv; ++k) node_colours[nodes[k]].push_back(c);
  }
  h->numcolors = ncol;
  h->color_ptr.assign(ncol + 1, 0);
  for (int el = 0; el < h->numel; ++el) h->color_ptr[col[el] + 1]++;
  for (int c = 0; c < ncol; ++c) h->color_ptr[c + 1] += h->color_ptr[c];
  h->color_elems.resize(h->numel);
  std::vector<int32_t> pos(h->color_ptr.begin(), h->color_ptr.end() - 1);
  for (int el = 0; el < h->numel; ++el) h->color_elems[pos[col[el]]++] = el + 1;
}

// partition_csrc_bynonzeros (Matrix_partition.f:125-178): rows split so that
// each thread gets about (2*nad+neq)/nth weighted entries.
void partition_rows(or_handle_s* h, int nth) {
  if (h->thr_n == nth) return;
  h->thr_n = nth;
  h->thr_begin.assign(nth + 1, 0);
  h->thr_end.assign(nth + 1, 0);
  h->thr_height.assign(nth + 1, 0);
  const int neq = h->neq;
  const int64_t mean = (2 * h->nad + neq) / nth + 1;
  int line = 2;
  h->thr_begin[1] = 1;
  for (int i = 1; i <= nth - 1; ++i) {
    int64_t size = 0;
    h->thr_end[i] = h->thr_begin[i] - 1;
    while (line <= neq + 1) {
      const int64_t tam = 2 * (h->ia[line - 1] - h->ia[line - 2]) + 1;
      if (size + tam <= mean) {
        size += tam;
        h->thr_end[i] = line - 1;
        h->thr_begin[i + 1] = line;
        ++line;
      } else {
        break;
      }
    }
    if (h->thr_begin[i + 1] == 0) h->thr_begin[i + 1] = h->thr_end[i] + 1;
  }
  h->thr_end[nth] = neq;
  // lowest column written by each thread (thread_height)
  for (int t = 1; t <= nth; ++t) {
    int lo = h->thr_begin[t];
    for (int i = h->thr_begin[t]; i <= h->thr_end[t]; ++i)
      if (h->ia[i] > h->ia[i - 1]) lo = std::min(lo, h->ja[h->ia[i - 1] - 1]);
    h->thr_height[t] = lo;
  }
}

// csr (Assbly.f:218-304): b -= p, ad += s_ii, al(kk) += s_ij with the linear
// search of the row for column ld(j).
void csr_assemble(or_handle_s* h, const double* s, const double* p,
                  const int* ld, int nst, bool lhs, bool rhs, double* b) {
  const int neq = h->neq;
  for (int i = 0; i < nst; ++i) {
    const int k = ld[i];
    if (k <= 0 || k > neq) continue;
    if (rhs) b[k - 1] = b[k - 1] - p[i];
    if (lhs) {
      h->ad[k - 1] = h->ad[k - 1] + s[i + (size_t)nst * i];
      for (int j = 0; j < nst; ++j) {
        const int l = ld[j];
        if (l <= 0) continue;
        for (int64_t kk = h->ia[k - 1]; kk <= h->ia[k] - 1; ++kk)
          if (l == h->ja[kk - 1]) h->al[kk - 1] = h->al[kk - 1] + s[i + (size_t)nst * j];
      }
    }
  }
}

void gather_element(const or_handle_s* h, int nel, const double* u, int* ld,
                    double* ul, double* xl, double* dpl, int* iqm, int* iqh,
                    double* txn, const double* tx0) {
  const int32_t* nodes = &h->ix[(size_t)(h->nen + 1) * (nel - 1)];
  const int ndf = h->ndf;
  int kk = 0;
  for (int i = 0; i < h->nen; ++i) {
    const int no = nodes[i];
    for (int j = 0; j < ndf - 1; ++j) {
      ld[kk] = h->idr[(size_t)ndf * (no - 1) + j];
      ul[kk] = u[(size_t)ndf * (no - 1) + j];
      ++kk;
    }
  }
  for (int i = 0; i < h->nenv; ++i) {
    const int no = nodes[i];
    ld[kk] = h->idr[(size_t)ndf * (no - 1) + ndf - 1];
    ul[kk] = u[(size_t)ndf * (no - 1) + ndf - 1];
    ++kk;
    dpl[i] = h->dp[no - 1];
    for (int j = 0; j < 3; ++j) xl[3 * i + j] = h->x[(size_t)3 * (no - 1) + j];
    if (tx0)
      for (int j = 0; j < 6; ++j) txn[6 * i + j] = tx0[(size_t)6 * (no - 1) + j];
  }
  for (int j = 0; j < 7; ++j) {
    iqm[j] = h->eload.empty() ? 0 : h->eload[(size_t)7 * (nel - 1) + j];
    iqh[j] = h->eloadp.empty() ? 0 : h->eloadp[(size_t)7 * (nel - 1) + j];
  }
}

int element_type_ok(const or_handle_s* h, int nel) {
  const int ma = h->ix[(size_t)(h->nen + 1) * (nel - 1) + h->nen];
  if (ma < 1 || ma > h->numat) return 0;
  const int iel = h->ie[ma - 1];
  return (iel == 17 && h->hexa) || (iel == 15 && !h->hexa);
}

int pform(or_handle_s* h, int isw, bool lhs, bool rhs, const double* u,
          double* b, int nthreads, const double* tx0, int e_begin = 1,
          int e_end = -1, bool zero = true) {
  if (e_end < 0) e_end = h->numel + 1;
  if (lhs && zero) {
    std::fill(h->al.begin(), h->al.end(), 0.0);
    std::fill(h->ad.begin(), h->ad.end(), 0.0);
  }
  const int nst = h->nst;
  int status = OR_OK;
  auto body = [&](int nel, std::vector<double>& s, std::vector<double>& p) {
    int ld[68], iqm[7], iqh[7];
    double ul[68], xl[24], dpl[8], txn[48];
    gather_element(h, nel, u, ld, ul, xl, dpl, iqm, iqh, txn, tx0);
    if (!element_type_ok(h, nel)) return OR_E_ELTYPE;
    const int ma = h->ix[(size_t)(h->nen + 1) * (nel - 1) + h->nen];
    for (int i = 0; i < nst; ++i) p[i] = 0.0;
    try {
      element(h->hexa, &h->e[(size_t)OR_PROP * (ma - 1)], iqm, iqh, xl, ul, dpl,
              p.data(), s.data(), txn, isw, h->L, h->env);
    } catch (DetError&) {
      return OR_E_DET;
    }
    csr_assemble(h, s.data(), p.data(), ld, nst, lhs && isw == 2, rhs, b);
    return OR_OK;
  };
  if (nthreads <= 1) {
    std::vector<double> s((size_t)nst * nst), p(nst);
    for (int nel = e_begin; nel < e_end; ++nel) {
      const int st = body(nel, s, p);
      if (st != OR_OK) return st;
    }
  } else {
#pragma omp parallel num_threads(nthreads)
    {
      std::vector<double> s((size_t)nst * nst), p(nst);
      for (int c = 0; c < h->numcolors; ++c) {
        // a colour lists its elements in increasing order: the elements of
        // a timing sample [e_begin, e_end) are one contiguous part of it,
        // shared among the threads like a whole colour
        const int* first = h->color_elems.data() + h->color_ptr[c];
        const int* last = h->color_elems.data() + h->color_ptr[c + 1];
        const int j0 = h->color_ptr[c] + (int)(std::lower_bound(first, last, e_begin) - first);
        const int j1 = h->color_ptr[c] + (int)(std::lower_bound(first, last, e_end) - first);
#pragma omp for schedule(static)
        for (int jc = j0; jc < j1; ++jc) {
          const int nel = h->color_elems[jc];
          const int st = body(nel, s, p);
          if (st != OR_OK) {
#pragma omp critical
            status = st;
          }
        }
      }
    }
  }
  return status;
}

void matvec(or_handle_s* h, const double* x, double* y, int nthreads) {
  const int neq = h->neq;
  const int64_t* ia = h->ia.data();
  const int32_t* ja = h->ja.data();
  const double* ad = h->ad.data();
  const double* al = h->al.data();
  if (nthreads <= 1) {
    // matvec_csrc_sym_pm (Matvec.f:1560-1589); y is written in row order, so
    // y(ja(k)), ja(k) < i, always already holds its row value.
    for (int i = 1; i <= neq; ++i) {
      const double xi = x[i - 1];
      double t = ad[i - 1] * xi;
      for (int64_t k = ia[i - 1]; k <= ia[i] - 1; ++k) {
        const int jak = ja[k - 1];
        const double s = al[k - 1];
        t = t + s * x[jak - 1];
        y[jak - 1] = y[jak - 1] + s * xi;
      }
      y[i - 1] = t;
    }
    return;
  }
  // matvec_csrc_sym_pm_omp (Matvec_omp.f:461-587)
  partition_rows(h, nthreads);
  std::vector<double> ty((size_t)nthreads * neq);
#pragma omp parallel num_threads(nthreads)
  {
#ifdef _OPENMP
    const int tid = omp_get_thread_num() + 1;
#else
    const int tid = 1;
#endif
    double* buf = &ty[(size_t)(tid - 1) * neq];
    for (int j = h->thr_height[tid]; j <= h->thr_begin[tid] - 1; ++j) buf[j - 1] = 0.0;
#pragma omp barrier
    for (int i = h->thr_begin[tid]; i <= h->thr_end[tid]; ++i) {
      y[i - 1] = 0.0;
      const double xi = x[i - 1];
      double t = ad[i - 1] * xi;
      for (int64_t k = ia[i - 1]; k <= ia[i] - 1; ++k) {
        const int jak = ja[k - 1];
        const double s = al[k - 1];
        t = t + s * x[jak - 1];
        buf[jak - 1] = buf[jak - 1] + s * xi;
      }
      buf[i - 1] = t;
    }
#pragma omp barrier
    for (int t = 1; t <= nthreads; ++t) {
      const double* tb = &ty[(size_t)(t - 1) * neq];
#pragma omp for schedule(static)
      for (int j = h->thr_height[t]; j <= h->thr_end[t]; ++j) y[j - 1] = y[j - 1] + tb[j - 1];
    }
  }
}

double dot(const double* a, const double* b, int n, int nthreads) {
  if (nthreads <= 1) {
    double tmp = 0.0;  // dot_par (Matvec.f:1714-1743)
    for (int i = 0; i < n; ++i) tmp = tmp + a[i] * b[i];
    return tmp;
  }
  double tmp = 0.0;
#pragma omp parallel for reduction(+ : tmp) num_threads(nthreads) schedule(static)
  for (int i = 0; i < n; ++i) tmp += a[i] * b[i];
  return tmp;
}

// pcg (Iters.f:299-595)
int pcg(or_handle_s* h, const double* m, const double* b, double* x, double tol,
        int maxit, int nth, or_step_info* info) {
  const int neq = h->neq;
  for (int i = 0; i < neq; ++i)
    if (h->ad[i] == 0.0) return OR_E_ZERO_DIAG;
  std::vector<double> z(neq), r(neq), p(neq);
  for (int i = 0; i < neq; ++i) x[i] = 0.0;
  for (int i = 0; i < neq; ++i) z[i] = b[i] * m[i];
  double d = dot(b, z.data(), neq, nth);
  const double conv = tol * std::sqrt(std::fabs(d));
  matvec(h, x, z.data(), nth);
  for (int i = 0; i < neq; ++i) {
    r[i] = b[i] - z[i];
    z[i] = r[i] * m[i];
    p[i] = z[i];
  }
  d = dot(r.data(), z.data(), neq, nth);
  int j;
  bool converged = false;
  for (j = 1; j <= maxit; ++j) {
    matvec(h, p.data(), z.data(), nth);
    const double alpha = d / dot(z.data(), p.data(), neq, nth);
    for (int i = 0; i < neq; ++i) {
      x[i] = x[i] + alpha * p[i];
      r[i] = r[i] - alpha * z[i];
      z[i] = r[i] * m[i];
    }
    const double di = dot(r.data(), z.data(), neq, nth);
    const double beta = di / d;
    for (int i = 0; i < neq; ++i) p[i] = z[i] + beta * p[i];
    d = di;
    if (std::sqrt(std::fabs(d)) < conv) {
      converged = true;
      break;
    }
  }
  if (info) {
    info->iters = converged ? j : maxit;
    info->conv = conv;
  }
  if (!converged) return OR_E_NOCONV;
  matvec(h, x, z.data(), nth);
  if (info) info->xkx = dot(x, z.data(), neq, nth);
  return OR_OK;
}

// sign1 / sym_ortho (Iters.f:6595-6660); c, s, r keep their previous values
// in the branch the reference leaves uncovered.
double sign1(double a) { return a > 0.0 ? 1.0 : (a < 0.0 ? -1.0 : 0.0); }
void sym_ortho(double a, double b, double& c, double& s, double& r) {
  const double ma = std::fabs(a), mb = std::fabs(b), sa = sign1(a), sb = sign1(b);
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
    s = sb / std::sqrt(1.0 + t * t);
    c = s * t;
    r = b / s;
  } else if (ma > mb) {
    const double t = b / a;
    c = sa / std::sqrt(1.0 + t * t);
    s = c * t;
    r = a / c;
  }
}

// pminres (Iters.f:3987-4305), nrestart = 10 (call_minres, Solv.f:1727)
int pminres(or_handle_s* h, const double* m, const double* b, double* x,
            double tol, int maxit, int nth, or_step_info* info) {
  const int neq = h->neq;
  for (int i = 0; i < neq; ++i)
    if (h->ad[i] == 0.0) return OR_E_ZERO_DIAG;
  std::vector<double> v0(neq), v(neq), w(neq), w0(neq), w00(neq), z(neq), z0(neq),
      p(neq);
  int it = 0, nrestart = 10;
  for (int i = 0; i < neq; ++i) x[i] = 0.0;
  for (int i = 0; i < neq; ++i) z[i] = b[i] * std::sqrt(std::fabs(m[i]));
  double tmp1 = dot(z.data(), z.data(), neq, nth);
  const double conv = tol * std::sqrt(std::fabs(tmp1));
  bool converged = false;
  for (;;) {
    matvec(h, x, z.data(), nth);
    for (int i = 0; i < neq; ++i) {
      v[i] = b[i] - z[i];
      v0[i] = 0.0;
      w0[i] = 0.0;
      w00[i] = 0.0;
      z0[i] = v[i] * m[i];
    }
    double beta = std::sqrt(std::fabs(dot(v.data(), z0.data(), neq, nth)));
    double normr = beta;
    double neta = beta, beta_old = beta, c_old = 1.0, c = 1.0, s_old = 0.0,
           s = 0.0, ro1 = 0.0;
    for (int j = 1; j <= maxit; ++j) {
      ++it;
      matvec(h, z0.data(), p.data(), nth);
      tmp1 = 1.0 / (beta * beta);
      const double alpha = std::fabs(dot(z0.data(), p.data(), neq, nth)) * tmp1;
      tmp1 = 1.0 / beta;
      double tmp2 = -alpha / beta;
      double tmp3 = -beta / beta_old;
      for (int i = 0; i < neq; ++i) {
        p[i] = tmp1 * p[i] + tmp2 * v[i] + tmp3 * v0[i];
        z[i] = p[i] * m[i];
      }
      beta_old = beta;
      tmp1 = dot(z.data(), p.data(), neq, nth);
      beta = std::sqrt(std::fabs(tmp1));
      const double delta = c * alpha - c_old * s * beta_old;
      const double ro2 = s * alpha + c_old * c * beta_old;
      const double ro3 = s_old * beta_old;
      c_old = c;
      s_old = s;
      sym_ortho(delta, beta, c, s, ro1);
      tmp1 = 1.0 / (beta_old * ro1);
      tmp2 = -ro2 / ro1;
      tmp3 = -ro3 / ro1;
      const double tmp4 = c * neta;
      for (int i = 0; i < neq; ++i) {
        w[i] = tmp1 * z0[i] + tmp2 * w0[i] + tmp3 * w00[i];
        x[i] = x[i] + tmp4 * w[i];
        v0[i] = v[i];
        v[i] = p[i];
        z0[i] = z[i];
        w00[i] = w0[i];
        w0[i] = w[i];
      }
      normr = std::fabs(s) * normr;
      if (normr < conv) {
        converged = true;
        break;
      }
      neta = -s * neta;
    }
    if (converged) break;
    if (nrestart != 0) {
      --nrestart;
      continue;
    }
    break;
  }
  if (info) {
    info->iters = it;
    info->conv = conv;
  }
  if (!converged) return OR_E_NOCONV;
  matvec(h, x, z.data(), nth);
  if (info) info->xkx = dot(x, z.data(), neq, nth);
  return OR_OK;
}

// ---- reverse Cuthill-McKee (Reord.f) ---------------------------------------
// The routines keep the reference's 1-based arrays: xadj(nnode+1) int64 and
// adjncy of graph_v1, mask, xls, perm; the level structures live in perm.

// rootls_v1 (Reord.f:282-345)
void rootls(int root, int64_t* xadj, const int32_t* adjncy, int32_t* mask, int& nlvl,
            int32_t* xls, int32_t* ls) {
  mask[root] = 0;
  ls[1] = root;
  nlvl = 0;
  int lvlend = 0, ccsize = 1;
  for (;;) {
    const int lbegin = lvlend + 1;
    lvlend = ccsize;
    nlvl = nlvl + 1;
    xls[nlvl] = lbegin;
    for (int i = lbegin; i <= lvlend; ++i) {
      const int node = ls[i];
      const int64_t jstrt = xadj[node], jstop = xadj[node + 1] - 1;
      for (int64_t j = jstrt; j <= jstop; ++j) {
        const int nbr = adjncy[j];
        if (mask[nbr] == 0) continue;
        ccsize = ccsize + 1;
        ls[ccsize] = nbr;
        mask[nbr] = 0;
      }
    }
    if (ccsize - lvlend <= 0) break;
  }
  xls[nlvl + 1] = lvlend + 1;
  for (int i = 1; i <= ccsize; ++i) mask[ls[i]] = 1;
}

// fnroot_v1 (Reord.f:96-164)
void fnroot(int& root, int64_t* xadj, const int32_t* adjncy, int32_t* mask, int& nlvl,
            int32_t* xls, int32_t* ls) {
  rootls(root, xadj, adjncy, mask, nlvl, xls, ls);
  const int ccsize = xls[nlvl + 1] - 1;
  if (nlvl == 1 || nlvl == ccsize) return;
  for (;;) {
    const int jstrt = xls[nlvl];
    int mindeg = ccsize;
    root = ls[jstrt];
    if (ccsize != jstrt) {
      for (int j = jstrt; j <= ccsize; ++j) {
        const int node = ls[j];
        int ndeg = 0;
        for (int64_t k = xadj[node]; k <= xadj[node + 1] - 1; ++k)
          if (mask[adjncy[k]] > 0) ndeg = ndeg + 1;
        if (ndeg >= mindeg) continue;
        root = node;
        mindeg = ndeg;
      }
    }
    int nunlvl = 0;
    rootls(root, xadj, adjncy, mask, nunlvl, xls, ls);
    if (nunlvl <= nlvl) return;
    nlvl = nunlvl;
    if (nlvl >= ccsize) return;
  }
}

// degree_v1 (Reord.f:346-430): xadj's sign marks the nodes already queued
void degree(int root, int64_t* xadj, const int32_t* adjncy, const int32_t* mask, int32_t* deg,
            int& ccsize, int32_t* ls) {
  ls[1] = root;
  xadj[root] = -xadj[root];
  int lvlend = 0;
  ccsize = 1;
  for (;;) {
    const int lbegin = lvlend + 1;
    lvlend = ccsize;
    for (int i = lbegin; i <= lvlend; ++i) {
      const int node = ls[i];
      const int64_t jstrt = -xadj[node];
      const int64_t jstop = std::llabs(xadj[node + 1]) - 1;
      int ideg = 0;
      for (int64_t j = jstrt; j <= jstop; ++j) {
        const int nbr = adjncy[j];
        if (mask[nbr] == 0) continue;
        ideg = ideg + 1;
        if (xadj[nbr] < 0) continue;
        xadj[nbr] = -xadj[nbr];
        ccsize = ccsize + 1;
        ls[ccsize] = nbr;
      }
      deg[node] = ideg;
    }
    if (ccsize - lvlend <= 0) break;
  }
  for (int i = 1; i <= ccsize; ++i) xadj[ls[i]] = -xadj[ls[i]];
}

// rcm_v1 (Reord.f:165-281)
void rcm(int root, int64_t* xadj, const int32_t* adjncy, int32_t* mask, int32_t* perm,
         int& ccsize, int32_t* deg) {
  degree(root, xadj, adjncy, mask, deg, ccsize, perm);
  mask[root] = 0;
  if (ccsize <= 1) return;
  int lvlend = 0, lnbr = 1;
  while (true) {
    const int lbegin = lvlend + 1;
    lvlend = lnbr;
    for (int i = lbegin; i <= lvlend; ++i) {
      const int node = perm[i];
      const int fnbr = lnbr + 1;
      for (int64_t j = xadj[node]; j <= xadj[node + 1] - 1; ++j) {
        const int nbr = adjncy[j];
        if (mask[nbr] == 0) continue;
        lnbr = lnbr + 1;
        mask[nbr] = 0;
        perm[lnbr] = nbr;
      }
      if (fnbr >= lnbr) continue;
      // linear insertion by increasing degree
      int k = fnbr;
      do {
        int l = k;
        k = k + 1;
        const int nbr = perm[k];
        while (l >= fnbr && deg[perm[l]] > deg[nbr]) {
          perm[l + 1] = perm[l];
          l = l - 1;
        }
        perm[l + 1] = nbr;
      } while (k < lnbr);
    }
    if (lnbr <= lvlend) break;
  }
  for (int i = 1, l = ccsize; i <= ccsize / 2; ++i, --l) std::swap(perm[l], perm[i]);
}

}  // namespace

// ---------------------------------------------------------------------------
// C API
// ---------------------------------------------------------------------------
extern "C" {

// reord (Reord.f:1-44) with graph_v1 (Graph.f:72-133) and genrcm_v1
// (Reord.f:45-95); afl = 0 gives the identity.
int or_reord(int nnode, int numel, int nen, const int32_t* ix, int afl, int32_t* iperm) {
  if (nnode < 1 || numel < 0 || nen < 1 || !iperm || (numel > 0 && !ix)) return OR_E_ARG;
  if (!afl) {
    for (int i = 0; i < nnode; ++i) iperm[i] = i + 1;
    return OR_OK;
  }
  // graph_v1: every node of an element is a neighbour of the others, lists
  // sorted by node number without repeats (1-based xadj / adjncy)
  std::vector<std::vector<int32_t>> nb(nnode + 1);
  for (int el = 0; el < numel; ++el) {
    const int32_t* nodes = ix + (size_t)(nen + 1) * el;
    for (int j = 0; j < nen; ++j) {
      const int noj = nodes[j];
      if (noj == 0 || noj > nnode) continue;
      for (int k = 0; k < nen; ++k) {
        const int nok = nodes[k];
        if (nok == 0 || nok > nnode || nok == noj) continue;
        nb[noj].push_back(nok);
      }
    }
  }
  std::vector<int64_t> xadj(nnode + 2, 0);
  xadj[1] = 1;
  for (int n = 1; n <= nnode; ++n) {
    std::sort(nb[n].begin(), nb[n].end());
    nb[n].erase(std::unique(nb[n].begin(), nb[n].end()), nb[n].end());
    xadj[n + 1] = xadj[n] + (int64_t)nb[n].size();
  }
  std::vector<int32_t> adjncy(xadj[nnode + 1] + 1, 0);
  for (int n = 1; n <= nnode; ++n)
    std::copy(nb[n].begin(), nb[n].end(), adjncy.begin() + xadj[n]);
  // genrcm_v1
  std::vector<int32_t> perm(nnode + 2, 0), mask(nnode + 1, 1), xls(nnode + 2, 0);
  int num = 1;
  for (int i = 1; i <= nnode; ++i) {
    if (mask[i] == 0) continue;
    int root = i, nlvl = 0, ccsize = 0;
    fnroot(root, xadj.data(), adjncy.data(), mask.data(), nlvl, xls.data(), perm.data() + num - 1);
    rcm(root, xadj.data(), adjncy.data(), mask.data(), perm.data() + num - 1, ccsize, xls.data());
    num = num + ccsize;
    if (num > nnode) break;
  }
  for (int i = 1; i <= nnode; ++i) iperm[i - 1] = perm[i];
  return OR_OK;
}

static void initial_porosity(or_handle_s* h);

int or_create(int nnode, int nnodev, int numel, int nen, int nenv, int ndf,
              const int32_t* ix, const int32_t* id, const int32_t* fnno,
              const double* x, int numat, const int32_t* ie, const double* e,
              const int32_t* num, or_handle* out) {
  if (!out || nnode <= 0 || numel <= 0 || ndf != 4 ||
      !((nen == 20 && nenv == 8) || (nen == 10 && nenv == 4)))
    return OR_E_ARG;
  or_handle_s* h = new or_handle_s();
  h->nnode = nnode; h->nnodev = nnodev; h->numel = numel; h->nen = nen;
  h->nenv = nenv; h->ndf = ndf; h->numat = numat; h->hexa = (nen == 20);
  h->nst = 3 * nen + nenv;
  h->ix.assign(ix, ix + (size_t)(nen + 1) * numel);
  h->fnno.assign(fnno, fnno + nnode);
  h->x.assign(x, x + (size_t)3 * nnode);
  h->ie.assign(ie, ie + numat);
  h->e.assign(e, e + (size_t)OR_PROP * numat);
  h->num.resize(nnode);
  for (int i = 0; i < nnode; ++i) h->num[i] = num ? num[i] : i + 1;
  // numeqpmec2 (Numeq.f:86-151); pressure only on vertex nodes.
  h->idr.assign((size_t)ndf * nnode, 0);
  int neq = 0;
  for (int i = 0; i < nnode; ++i) {
    const int n = h->num[i];
    const int ndfn = (h->fnno[n - 1] == 1) ? ndf : ndf - 1;
    for (int j = 0; j < ndfn; ++j) {
      const int k = id[(size_t)ndf * (n - 1) + j];
      if (k == 0) {
        ++neq;
        h->idr[(size_t)ndf * (n - 1) + j] = neq;
      } else {
        h->idr[(size_t)ndf * (n - 1) + j] = 0;
      }
    }
  }
  h->neq = neq;
  // graph_v1 (Graph.f:72-133, graph0_v1/graph1_v1): all nen nodes of each
  // element are neighbours, duplicates removed.
  std::vector<std::vector<int32_t>> nb(nnode + 1);
  for (int el = 0; el < numel; ++el) {
    const int32_t* nodes = &h->ix[(size_t)(nen + 1) * el];
    for (int j = 0; j < nen; ++j) {
      const int noj = nodes[j];
      if (noj == 0 || noj > nnode) continue;
      for (int k = 0; k < nen; ++k) {
        const int nok = nodes[k];
        if (nok == 0 || nok > nnode || nok == noj) continue;
        nb[noj].push_back(nok);
      }
    }
  }
  for (int n = 1; n <= nnode; ++n) {
    std::sort(nb[n].begin(), nb[n].end());
    nb[n].erase(std::unique(nb[n].begin(), nb[n].end()), nb[n].end());
  }
  // csria_v1 / csrja_v1 (Csr.f:631-870) lower part, then sort_graph_csr.
  h->ia.assign(neq + 1, 0);
  std::vector<int64_t> cnt(neq + 2, 0);
  auto for_row = [&](int i, auto&& fn) {
    for (int ii = 0; ii < ndf; ++ii) {
      const int neqi = h->idr[(size_t)ndf * (i - 1) + ii];
      if (!(neqi > 0 && neqi <= neq)) continue;
      for (int kk = 0; kk < ndf; ++kk) {
        const int neqj = h->idr[(size_t)ndf * (i - 1) + kk];
        if (neqj <= 0) continue;
        if (neqj < neqi) fn(neqi, neqj);
      }
      for (int j : nb[i])
        for (int jj = 0; jj < ndf; ++jj) {
          const int neqj = h->idr[(size_t)ndf * (j - 1) + jj];
          if (neqj <= 0) continue;
          if (neqj < neqi) fn(neqi, neqj);
        }
    }
  };
  for (int no = 1; no <= nnode; ++no)
    for_row(h->num[no - 1], [&](int r, int) { cnt[r]++; });
  h->ia[0] = 1;
  for (int i = 1; i <= neq; ++i) h->ia[i] = h->ia[i - 1] + cnt[i];
  h->nad = h->ia[neq] - 1;
  h->ja.assign(h->nad, 0);
  std::vector<int64_t> fill(neq + 1);
  for (int i = 1; i <= neq; ++i) fill[i] = h->ia[i - 1] - 1;
  for (int no = 1; no <= nnode; ++no)
    for_row(h->num[no - 1], [&](int r, int c) { h->ja[fill[r]++] = c; });
  for (int i = 1; i <= neq; ++i)
    std::sort(h->ja.begin() + (h->ia[i - 1] - 1), h->ja.begin() + (h->ia[i] - 1));
  h->ad.assign(neq, 0.0);
  h->al.assign(h->nad, 0.0);
  h->u.assign((size_t)ndf * nnode, 0.0);
  h->u0.assign((size_t)ndf * nnode, 0.0);
  h->dp.assign(nnode, 0.0);
  h->f.assign((size_t)ndf * nnode, 0.0);
  h->b0.assign(neq, 0.0);
  h->b.assign(neq, 0.0);
  h->x0.assign(neq, 0.0);
  h->m.assign(neq, 0.0);
  h->bst0.assign(neq, 0.0);
  h->env.gravity_mod = std::sqrt(h->env.gravity[0] * h->env.gravity[0] +
                                 h->env.gravity[1] * h->env.gravity[1] +
                                 h->env.gravity[2] * h->env.gravity[2]);
  colour_mesh(h);
  initial_porosity(h);
  *out = h;
  return OR_OK;
}

void or_destroy(or_handle h) { delete h; }

int or_set_loads(or_handle h, const int32_t* eload, const int32_t* eloadp,
                 const int32_t* nload, const double* f, int nloads, int maxt,
                 const int32_t* load, const double* fload) {
  if (!h) return OR_E_ARG;
  if (eload) h->eload.assign(eload, eload + (size_t)7 * h->numel);
  if (eloadp) h->eloadp.assign(eloadp, eloadp + (size_t)7 * h->numel);
  if (nload) h->nload.assign(nload, nload + (size_t)h->ndf * h->nnode);
  if (f) h->f.assign(f, f + (size_t)h->ndf * h->nnode);
  h->L.nloads = nloads;
  h->L.maxt = maxt > 0 ? maxt : 1;
  if (nloads > 0) {
    h->L.load.assign(load, load + (size_t)3 * nloads);
    h->L.fload.assign(fload, fload + (size_t)h->L.maxt * OR_NFLOAD * nloads);
  }
  return OR_OK;
}

int or_set_env(or_handle h, const double* gravity, double dt, double t, int istep) {
  if (!h) return OR_E_ARG;
  if (gravity) {
    for (int i = 0; i < 3; ++i) h->env.gravity[i] = gravity[i];
    h->env.gravity_mod = std::sqrt(h->env.gravity[0] * h->env.gravity[0] +
                                   h->env.gravity[1] * h->env.gravity[1] +
                                   h->env.gravity[2] * h->env.gravity[2]);
  }
  h->env.dt = dt;
  h->env.t = t;
  h->env.istep = istep;
  return OR_OK;
}

int or_set_state(or_handle h, const double* u, const double* u0, const double* dp) {
  if (!h) return OR_E_ARG;
  const size_t n = (size_t)h->ndf * h->nnode;
  if (u) h->u.assign(u, u + n);
  if (u0) h->u0.assign(u0, u0 + n);
  if (dp) h->dp.assign(dp, dp + h->nnode);
  return OR_OK;
}

int or_get_state(or_handle h, double* u, double* u0, double* dp) {
  if (!h) return OR_E_ARG;
  if (u) std::copy(h->u.begin(), h->u.end(), u);
  if (u0) std::copy(h->u0.begin(), h->u0.end(), u0);
  if (dp) std::copy(h->dp.begin(), h->dp.end(), dp);
  return OR_OK;
}

int or_set_initial_stress(or_handle h, const double* tx0) {
  if (!h || !tx0) return OR_E_ARG;
  std::fill(h->bst0.begin(), h->bst0.end(), 0.0);
  h->fstress0 = true;
  // tform with isw = 5 (Main.f:840-846): bstress0 -= int(B^T sigma0)
  return pform(h, 5, false, true, h->u0.data(), h->bst0.data(), 1, tx0);
}

int or_sizes(or_handle h, int* neq, int64_t* nad, int* numcolors) {
  if (!h) return OR_E_ARG;
  if (neq) *neq = h->neq;
  if (nad) *nad = h->nad;
  if (numcolors) *numcolors = h->numcolors;
  return OR_OK;
}

int or_get_id(or_handle h, int32_t* id) {
  if (!h || !id) return OR_E_ARG;
  std::copy(h->idr.begin(), h->idr.end(), id);
  return OR_OK;
}

int or_get_csrd(or_handle h, int64_t* ia, int32_t* ja, double* ad, double* al) {
  if (!h) return OR_E_ARG;
  if (ia) std::copy(h->ia.begin(), h->ia.end(), ia);
  if (ja) std::copy(h->ja.begin(), h->ja.end(), ja);
  if (ad) std::copy(h->ad.begin(), h->ad.end(), ad);
  if (al) std::copy(h->al.begin(), h->al.end(), al);
  return OR_OK;
}

int or_set_csrd_values(or_handle h, const double* ad, const double* al) {
  if (!h) return OR_E_ARG;
  if (ad) h->ad.assign(ad, ad + h->neq);
  if (al) h->al.assign(al, al + h->nad);
  return OR_OK;
}

int or_element(or_handle h, int nel, int isw, const double* ul,
               const double* dpl, double* s, double* p) {
  if (!h || nel < 1 || nel > h->numel) return OR_E_ARG;
  int ld[68], iqm[7], iqh[7];
  double ulx[68], xl[24], dpx[8], txn[48];
  gather_element(h, nel, h->u.data(), ld, ulx, xl, dpx, iqm, iqh, txn, nullptr);
  const int ma = h->ix[(size_t)(h->nen + 1) * (nel - 1) + h->nen];
  for (int i = 0; i < h->nst; ++i) p[i] = 0.0;
  try {
    element(h->hexa, &h->e[(size_t)OR_PROP * (ma - 1)], iqm, iqh, xl, ul, dpl, p,
            s, txn, isw, h->L, h->env);
  } catch (DetError&) {
    return OR_E_DET;
  }
  return OR_OK;
}

// tform_pm (Pform.f:433-640) with isw 3, then effective_stress
// (Pform.f:2487-2505): vertex values of every element accumulated in element
// order and averaged over the elements sharing the vertex; mid-side nodes
// keep zeros.  tx, txb, txe (6, nnode), flux (3, nnode), from the current u
// and dp.
// initial_porosity (Pform.f:1343-1432): e(8) of the elements sharing a
// vertex, averaged
static void initial_porosity(or_handle_s* h) {
  const int nnode = h->nnode, nenv = h->nenv, nen = h->nen;
  std::vector<int> ic(nnode, 0);
  h->poro.assign(nnode, 0.0);
  for (int nel = 1; nel <= h->numel; ++nel) {
    const int ma = h->ix[(size_t)(nen + 1) * (nel - 1) + nen];
    const double poro = h->e[(size_t)OR_PROP * (ma - 1) + 7];
    for (int i = 0; i < nenv; ++i) {
      const int no = h->ix[(size_t)(nen + 1) * (nel - 1) + i];
      if (no <= 0) continue;
      ic[no - 1] += 1;
      h->poro[no - 1] = h->poro[no - 1] + poro;
    }
  }
  for (int i = 0; i < nnode; ++i)
    if (h->fnno[i] == 1) h->poro[i] = h->poro[i] / ic[i];
}

// porosity_form (Pform.f:969-1175) with u = h->u
static int porosity_form(or_handle_s* h) {
  const int nnode = h->nnode, nenv = h->nenv, nen = h->nen;
  std::vector<int> ic(nnode, 0);
  std::vector<double> dporo(nnode, 0.0);
  int ld[68], iqm[7], iqh[7];
  double ul[68], xl[24], dpl[8], txn[48], pl[120], sdum[1];
  for (int nel = 1; nel <= h->numel; ++nel) {
    gather_element(h, nel, h->u.data(), ld, ul, xl, dpl, iqm, iqh, txn, nullptr);
    const int ma = h->ix[(size_t)(nen + 1) * (nel - 1) + nen];
    for (int i = 0; i < nenv; ++i) pl[i] = 0.0;
    try {
      element(h->hexa, &h->e[(size_t)OR_PROP * (ma - 1)], iqm, iqh, xl, ul, dpl, pl, sdum,
              txn, 7, h->L, h->env);
    } catch (DetError&) {
      return OR_E_DET;
    }
    for (int i = 0; i < nenv; ++i) {
      const int no = h->ix[(size_t)(nen + 1) * (nel - 1) + i];
      if (no <= 0) continue;
      ic[no - 1] += 1;
      dporo[no - 1] = dporo[no - 1] + pl[i];
    }
  }
  for (int i = 0; i < nnode; ++i)
    if (h->fnno[i] == 1) h->poro[i] = h->poro[i] + dporo[i] / ic[i];
  return OR_OK;
}

int or_set_nkrylov(or_handle h, int nkrylov) {
  if (!h || nkrylov < 1) return OR_E_ARG;
  h->nkrylov = nkrylov;
  return OR_OK;
}

int or_get_porosity(or_handle h, double* poro) {
  if (!h || !poro) return OR_E_ARG;
  std::copy(h->poro.begin(), h->poro.end(), poro);
  return OR_OK;
}

int or_set_porosity(or_handle h, const double* poro) {
  if (!h || !poro) return OR_E_ARG;
  h->poro.assign(poro, poro + h->nnode);
  return OR_OK;
}

int or_stress(or_handle h, double* tx, double* txb, double* txe, double* flux) {
  if (!h || !tx || !txb || !txe || !flux) return OR_E_ARG;
  const int nnode = h->nnode, nenv = h->nenv, nen = h->nen;
  std::vector<int> ic(nnode, 0);
  std::fill(tx, tx + (size_t)6 * nnode, 0.0);
  std::fill(txb, txb + (size_t)6 * nnode, 0.0);
  std::fill(flux, flux + (size_t)3 * nnode, 0.0);
  int ld[68], iqm[7], iqh[7];
  double ul[68], xl[24], dpl[8], txn[48], pl[120], sdum[1];
  for (int nel = 1; nel <= h->numel; ++nel) {
    gather_element(h, nel, h->u.data(), ld, ul, xl, dpl, iqm, iqh, txn, nullptr);
    const int ma = h->ix[(size_t)(nen + 1) * (nel - 1) + nen];
    for (int i = 0; i < 15 * nenv; ++i) pl[i] = 0.0;
    try {
      element(h->hexa, &h->e[(size_t)OR_PROP * (ma - 1)], iqm, iqh, xl, ul, dpl, pl, sdum,
              txn, 3, h->L, h->env);
    } catch (DetError&) {
      return OR_E_DET;
    }
    for (int i = 0; i < nenv; ++i) {
      const int no = h->ix[(size_t)(nen + 1) * (nel - 1) + i];
      if (no <= 0) continue;
      ic[no - 1] += 1;
      for (int j = 0; j < 6; ++j) {
        tx[(size_t)6 * (no - 1) + j] += pl[6 * i + j];
        txb[(size_t)6 * (no - 1) + j] += pl[6 * nenv + 6 * i + j];
      }
      for (int j = 0; j < 3; ++j) flux[(size_t)3 * (no - 1) + j] += pl[12 * nenv + 3 * i + j];
    }
  }
  for (int i = 0; i < nnode; ++i) {
    if (h->fnno[i] == 1 && ic[i] > 0) {
      for (int j = 0; j < 6; ++j) {
        tx[(size_t)6 * i + j] = tx[(size_t)6 * i + j] / ic[i];
        txb[(size_t)6 * i + j] = txb[(size_t)6 * i + j] / ic[i];
      }
      for (int j = 0; j < 3; ++j) flux[(size_t)3 * i + j] = flux[(size_t)3 * i + j] / ic[i];
    }
  }
  for (int i = 0; i < nnode; ++i) {
    const double pi = h->u[(size_t)h->ndf * i + h->ndf - 1];
    txe[(size_t)6 * i + 0] = tx[(size_t)6 * i + 0] + pi;
    txe[(size_t)6 * i + 1] = tx[(size_t)6 * i + 1] + pi;
    txe[(size_t)6 * i + 2] = tx[(size_t)6 * i + 2] + pi;
    for (int j = 3; j < 6; ++j) txe[(size_t)6 * i + j] = tx[(size_t)6 * i + j];
  }
  return OR_OK;
}

int or_pform(or_handle h, int isw, int lhs, int rhs, const double* u, double* b,
             int nthreads) {
  if (!h || !u || !b) return OR_E_ARG;
  return pform(h, isw, lhs != 0, rhs != 0, u, b, nthreads, nullptr);
}

int or_pform_range(or_handle h, int isw, int lhs, int rhs, const double* u,
                   double* b, int nthreads, int e_begin, int e_end) {
  if (!h || !u || !b || e_begin < 1 || e_end > h->numel + 1 || e_begin > e_end)
    return OR_E_ARG;
  // a timing sample of the element loop: ad/al are not zeroed first
  return pform(h, isw, lhs != 0, rhs != 0, u, b, nthreads, nullptr, e_begin, e_end, false);
}

// rpsqmr (Iters.f:6100-6439): symmetric QMR with the diagonal
// preconditioner applied on the right, for symmetric indefinite systems.
// conv = tol ||b||; the loop stops when ||r|| < conv; a non-converged run
// returns OR_E_NOCONV (where the reference sets fsqmr and switches to
// GMRES(l), Solv.f:707-766); sigma = 0 or rho = 0 are breakdowns
// (stop_mef in the reference).
int rpsqmr(or_handle_s* h, const double* m, const double* b, double* x, double tol,
           int maxit, int nth, or_step_info* info, bool* reached_maxit = nullptr) {
  const int neq = h->neq;
  for (int i = 0; i < neq; ++i)
    if (h->ad[i] == 0.0) return OR_E_ZERO_DIAG;
  std::vector<double> t(neq), r(neq), q(neq), d(neq);
  for (int i = 0; i < neq; ++i) x[i] = 0.0;
  const double norm_b = dot(b, b, neq, nth);
  const double conv = tol * std::sqrt(std::fabs(norm_b));
  matvec(h, x, t.data(), nth);
  for (int i = 0; i < neq; ++i) {
    r[i] = b[i] - t[i];
    q[i] = r[i] * m[i];
    d[i] = 0.0;
  }
  double tau = std::sqrt(dot(r.data(), r.data(), neq, nth));
  double ro = dot(r.data(), q.data(), neq, nth);
  double v0 = 0.0;
  int j;
  bool converged = false;
  for (j = 1; j <= maxit; ++j) {
    matvec(h, q.data(), t.data(), nth);
    const double sigma = dot(q.data(), t.data(), neq, nth);
    if (sigma == 0.0) return OR_E_NOCONV;
    const double alpha = ro / sigma;
    for (int i = 0; i < neq; ++i) r[i] = r[i] - alpha * t[i];
    const double vn = std::sqrt(dot(r.data(), r.data(), neq, nth)) / tau;
    const double cn = 1.0 / std::sqrt(1.0 + vn * vn);
    tau = tau * vn * cn;
    const double tmp1 = cn * cn * v0 * v0;
    const double tmp2 = cn * cn * alpha;
    for (int i = 0; i < neq; ++i) {
      d[i] = tmp1 * d[i] + tmp2 * q[i];
      x[i] = x[i] + d[i];
      t[i] = r[i] * m[i];
    }
    v0 = vn;
    if (ro == 0.0) return OR_E_NOCONV;
    const double rt = dot(r.data(), t.data(), neq, nth);
    const double beta = rt / ro;
    ro = rt;
    for (int i = 0; i < neq; ++i) q[i] = t[i] + beta * q[i];
    const double norm_r = std::sqrt(dot(r.data(), r.data(), neq, nth));
    if (norm_r < conv) {
      converged = true;
      break;
    }
  }
  if (info) {
    info->iters = converged ? j : maxit;
    info->conv = conv;
  }
  if (!converged) {
    if (reached_maxit) *reached_maxit = true;
    return OR_E_NOCONV;
  }
  matvec(h, x, t.data(), nth);
  if (info) info->xkx = dot(x, t.data(), neq, nth);
  return OR_OK;
}

// sym_ortho2 (Iters.f:6718-6745): the Givens rotation of GMRES
static void sym_ortho2(double a, double b, double& c, double& s, double& r) {
  const double ma = std::fabs(a), mb = std::fabs(b);
  c = 1.0;
  s = 0.0;
  r = a;
  if (b != 0.0) {
    if (mb > ma) {
      const double t = a / b;
      s = 1.0 / std::sqrt(1.0 + t * t);
      c = s * t;
      r = b / s;
    } else {
      const double t = b / a;
      c = 1.0 / std::sqrt(1.0 + t * t);
      s = c * t;
      r = a / c;
    }
  }
}

// gmres2 (Iters.f:1411-1700): restarted GMRES(k) with the diagonal
// preconditioner on the left, modified Gram-Schmidt with one more pass when
// the norm drops below kesp = 0.25 of its value before orthogonalisation,
// Givens QR of the Hessenberg matrix.  maxit counts cycles.  x starts at 0
// (fnew); conv = tol ||M b||; a run that ends its cycles above conv is the
// reference's stop_mef (OR_E_NOCONV here).  A zero right-hand side returns
// x = 0 (the reference divides by the zero residual norm there).
int gmres2(or_handle_s* h, const double* m, const double* b, double* x, double tol,
           int maxit, int k, int nth, or_step_info* info) {
  const int neq = h->neq;
  const double kesp = 0.25;
  std::vector<double> g((size_t)neq * (k + 1)), hm((size_t)(k + 1) * k, 0.0);
  std::vector<double> y(k), c(k), sv(k), e(k + 1);
  auto G = [&](int j) { return g.data() + (size_t)neq * (j - 1); };  // g(1, j)
  auto H = [&](int i, int j) -> double& { return hm[(size_t)(k + 1) * (j - 1) + (i - 1)]; };
  for (int i = 0; i < neq; ++i) {
    x[i] = 0.0;
    G(1)[i] = b[i] * m[i];
  }
  double norm = std::sqrt(dot(G(1), G(1), neq, nth));
  const double econv = tol * norm;
  if (info) info->conv = econv;
  if (norm == 0.0) {
    if (info) info->iters = 0;
    return OR_OK;
  }
  int nit = 0, ni = 0;
  bool converged = false;
  for (int l = 1; l <= maxit; ++l) {
    matvec(h, x, G(1), nth);
    for (int i = 0; i < neq; ++i) G(1)[i] = (b[i] - G(1)[i]) * m[i];
    e[0] = std::sqrt(dot(G(1), G(1), neq, nth));
    double inorm = 1.0 / e[0];
    for (int i = 0; i < neq; ++i) G(1)[i] = G(1)[i] * inorm;
    ni = 0;
    for (int i = 1; i <= k; ++i) {
      ++nit;
      ++ni;
      double* w = G(i + 1);
      matvec(h, G(i), w, nth);
      for (int j = 0; j < neq; ++j) w[j] = w[j] * m[j];
      const double tau = std::sqrt(dot(w, w, neq, nth));
      for (int j = 1; j <= i; ++j) {
        const double beta = dot(w, G(j), neq, nth);
        const double* gj = G(j);
        for (int ic = 0; ic < neq; ++ic) w[ic] = w[ic] - beta * gj[ic];
        H(j, i) = beta;
      }
      norm = std::sqrt(dot(w, w, neq, nth));
      if (norm <= kesp * tau) {
        for (int j = 1; j <= i; ++j) {
          const double beta = dot(w, G(j), neq, nth);
          const double* gj = G(j);
          for (int ic = 0; ic < neq; ++ic) w[ic] = w[ic] - beta * gj[ic];
          H(j, i) = H(j, i) + beta;
        }
      }
      norm = std::sqrt(dot(w, w, neq, nth));
      H(i + 1, i) = norm;
      inorm = 1.0 / norm;
      for (int ic = 0; ic < neq; ++ic) w[ic] = w[ic] * inorm;
      for (int j = 1; j <= i - 1; ++j) {
        const double aux1 = c[j - 1] * H(j, i) + sv[j - 1] * H(j + 1, i);
        const double aux2 = -sv[j - 1] * H(j, i) + c[j - 1] * H(j + 1, i);
        H(j, i) = aux1;
        H(j + 1, i) = aux2;
      }
      double r;
      sym_ortho2(H(i, i), H(i + 1, i), c[i - 1], sv[i - 1], r);
      H(i, i) = r;
      H(i + 1, i) = 0.0;
      e[i] = -sv[i - 1] * e[i - 1];
      e[i - 1] = c[i - 1] * e[i - 1];
      if (std::fabs(e[i]) <= econv) break;
    }
    // back substitution R y = e
    for (int j = 1; j <= ni; ++j) y[j - 1] = e[j - 1];
    for (int j = ni; j >= 2; --j) {
      y[j - 1] = y[j - 1] / H(j, j);
      const double r = y[j - 1];
      for (int i = 1; i <= j - 1; ++i) y[i - 1] = y[i - 1] - H(i, j) * r;
    }
    y[0] = y[0] / H(1, 1);
    for (int j = 1; j <= ni; ++j) {
      const double r = y[j - 1];
      const double* gj = G(j);
      for (int i = 0; i < neq; ++i) x[i] = x[i] + r * gj[i];
    }
    if (std::fabs(e[ni]) <= econv) {
      converged = true;
      break;
    }
  }
  if (info) info->iters = nit;
  if (!converged) return OR_E_NOCONV;
  std::vector<double> t(neq);
  matvec(h, x, t.data(), nth);
  if (info) info->xkx = dot(x, t.data(), neq, nth);
  return OR_OK;
}

int or_matvec(or_handle h, const double* x, double* y, int nthreads) {
  if (!h || !x || !y) return OR_E_ARG;
  matvec(h, x, y, nthreads);
  return OR_OK;
}

int or_solve(or_handle h, int solver, int precond, const double* b, double* x,
             double tol, int maxit, int nthreads, or_step_info* info) {
  if (!h || !b || !x) return OR_E_ARG;
  // cal_precond (Precond.f:1601-1721) -> pre_diag (Precond.f:22-79)
  for (int i = 0; i < h->neq; ++i) {
    if (precond == 5)
      h->m[i] = std::fabs(1.0 / h->ad[i]);
    else
      h->m[i] = 1.0 / h->ad[i];
  }
  if (solver == 1) return pcg(h, h->m.data(), b, x, tol, maxit, nthreads, info);
  if (solver == 7) return pminres(h, h->m.data(), b, x, tol, maxit, nthreads, info);
  if (solver == 2) return gmres2(h, h->m.data(), b, x, tol, maxit, h->nkrylov, nthreads, info);
  if (solver == 11) {
    // Solv.f:707-766: rpsqmr, and GMRES(l) from x = 0 when it reaches maxit
    bool fallback = false;
    const int st = rpsqmr(h, h->m.data(), b, x, tol, maxit, nthreads, info, &fallback);
    if (!fallback) return st;
    const int its = info ? info->iters : 0;
    const int st2 = gmres2(h, h->m.data(), b, x, tol, maxit, h->nkrylov, nthreads, info);
    if (info) info->iters += its;
    return st2;
  }
  return OR_E_ARG;
}

int or_step(or_handle h, int maxnlit, double tol, int stop_crit, int solver,
            int precond, double solvtol, int maxit, int nthreads,
            or_step_info* info) {
  if (!h) return OR_E_ARG;
  const int ndf = h->ndf, nnode = h->nnode;
  h->env.istep += 1;
  h->env.t = h->env.t + h->env.dt;
  // pload_pm (Pload.f:1-92)
  for (int i = 1; i <= nnode; ++i)
    for (int j = 1; j <= ndf - 1; ++j) {
      const int nc = h->nload.empty() ? 0 : h->nload[(size_t)ndf * (i - 1) + j - 1];
      if (nc > 0) {
        double c, vc[3];
        tload(h->L, nc, h->env.t, &h->x[(size_t)3 * (i - 1)],
              h->u[(size_t)ndf * (i - 1) + j - 1], c, vc, h->env.gravity_mod);
        h->f[(size_t)ndf * (i - 1) + j - 1] = c;
      }
    }
  for (int i = 1; i <= nnode; ++i)
    if (h->fnno[i - 1] == 1) {
      const int nc = h->nload.empty() ? 0 : h->nload[(size_t)ndf * (i - 1) + ndf - 1];
      if (nc > 0) {
        double c, vc[3];
        tload(h->L, nc, h->env.t, &h->x[(size_t)3 * (i - 1)],
              h->u[(size_t)ndf * (i - 1) + ndf - 1], c, vc, h->env.gravity_mod);
        h->f[(size_t)ndf * (i - 1) + ndf - 1] = c;
      }
    }
  for (int i = 1; i <= nnode; ++i)
    for (int j = 1; j <= ndf - 1; ++j) {
      const size_t q = (size_t)ndf * (i - 1) + j - 1;
      const int k = h->idr[q];
      if (k > 0) h->b0[k - 1] = h->f[q];
      else h->u[q] = h->f[q];
    }
  for (int i = 1; i <= nnode; ++i)
    if (h->fnno[i - 1] == 1) {
      const size_t q = (size_t)ndf * (i - 1) + ndf - 1;
      const int k = h->idr[q];
      if (k > 0) h->b0[k - 1] = -h->env.dt * h->f[q];
      else h->u[q] = h->f[q];
    }
  // element loop isw = 4 with u = u(n) (Main.f:908-926)
  int st = pform(h, 4, false, true, h->u.data(), h->b0.data(), nthreads, nullptr);
  if (st != OR_OK) return st;
  if (h->fstress0)
    for (int i = 0; i < h->neq; ++i) h->b0[i] = h->b0[i] + h->bst0[i];
  // delta_predict_pm (Predict.f:117-158)
  for (int i = 1; i <= nnode; ++i) {
    for (int j = 1; j <= ndf - 1; ++j) {
      const size_t q = (size_t)ndf * (i - 1) + j - 1;
      h->u[q] = h->u[q] - h->u0[q];
    }
    if (h->fnno[i - 1] == 1) {
      const size_t q = (size_t)ndf * (i - 1) + ndf - 1;
      h->u[q] = h->u[q] - h->u0[q];
    }
  }
  // nonlinear loop (Main.f:946-1060)
  bool lhs = true;
  double& resu0 = h->resu0;
  double& resp0 = h->resp0;
  int it = 1;
  or_step_info loc{};
  for (;;) {
    h->b = h->b0;
    st = pform(h, 2, lhs, true, h->u.data(), h->b.data(), nthreads, nullptr);
    if (st != OR_OK) return st;
    if (stop_crit == 1) {
      // cal_residuo_pm, stop_crit 1: |R|/|R0| over all equations
      const double res = std::sqrt(dot(h->b.data(), h->b.data(), h->neq, 1));
      if (it == 1) h->res0 = res;
      else if (it == 2) h->res0 = std::max(h->res0, res);
      loc.res_u = res;
      loc.res_p = 0.0;
      if (res / h->res0 < tol) break;
    } else if (stop_crit == 2) {
      // cal_residuo_pm (Residuo.f:39-276), stop_crit 2
      double resu = 0.0, resp = 0.0;
      for (int i = 1; i <= nnode; ++i)
        for (int j = 1; j <= ndf - 1; ++j) {
          const int neqi = h->idr[(size_t)ndf * (i - 1) + j - 1];
          if (neqi != 0) resu = resu + h->b[neqi - 1] * h->b[neqi - 1];
        }
      for (int i = 1; i <= nnode; ++i) {
        const int neqi = h->idr[(size_t)ndf * (i - 1) + ndf - 1];
        if (neqi != 0) resp = resp + h->b[neqi - 1] * h->b[neqi - 1];
      }
      const double gresu = std::sqrt(resu), gresp = std::sqrt(resp);
      if (getenv("OR_DEBUG")) fprintf(stderr, "nlit %d resu %.6e resp %.6e\n", it, gresu, gresp);
      if (it == 1) {
        resu0 = gresu;
        resp0 = gresp;
      } else if (it == 2) {
        resu0 = std::max(resu0, gresu);
        resp0 = std::max(resp0, gresu);  // the reference compares with gresu here
      }
      loc.res_u = gresu;
      loc.res_p = gresp;
      int istop = 0;
      if (gresu / resu0 < tol) istop += 1;
      if (gresp / resp0 < tol) istop += 1;
      if (istop == 2) break;
    }
    st = or_solve(h, solver, precond, h->b.data(), h->x0.data(), solvtol, maxit,
                  nthreads, &loc);
    if (st != OR_OK) return st;
    // delta_update_pm (Predict.f:159-215)
    for (int i = 1; i <= nnode; ++i)
      for (int j = 1; j <= ndf - 1; ++j) {
        const size_t q = (size_t)ndf * (i - 1) + j - 1;
        const int k = h->idr[q];
        if (k > 0) h->u[q] = h->u[q] + h->x0[k - 1];
      }
    for (int i = 1; i <= nnode; ++i)
      if (h->fnno[i - 1] == 1) {
        const size_t q = (size_t)ndf * (i - 1) + ndf - 1;
        const int k = h->idr[q];
        if (k > 0) h->u[q] = h->u[q] + h->x0[k - 1];
      }
    if (it >= maxnlit) return OR_E_NLNOCONV;
    ++it;
    lhs = false;
  }
  loc.nlit = it;
  // porosity_form (Pform.f:969-1175, elastic: no variable properties), on the
  // increments before they are added to the state (Main.f:1086)
  st = porosity_form(h);
  if (st != OR_OK) return st;
  // update_res_v2 (Pload.f:483-540)
  for (int i = 1; i <= nnode; ++i) {
    for (int j = 1; j <= ndf - 1; ++j) {
      const size_t q = (size_t)ndf * (i - 1) + j - 1;
      h->u[q] = h->u0[q] + h->u[q];
      h->u0[q] = h->u[q];
    }
    if (h->fnno[i - 1] == 1) {
      const size_t q = (size_t)ndf * (i - 1) + ndf - 1;
      h->dp[i - 1] = h->dp[i - 1] + h->u[q];
      h->u[q] = h->u0[q] + h->u[q];
      h->u0[q] = h->u[q];
    }
  }
  if (info) *info = loc;
  return OR_OK;
}

double or_element_flops(int nen, int isw) {
  // Counted from the restated loops of elmt17_pm / elmt15_pm, isw = 2:
  // per integration point Kuu = nu*nu*66, Kpu = np*(1 + 6*nu) + 1,
  // Kpp = np*np*10 + 2; geometry (shape functions, Jacobian, inverse and the
  // two derivative mappings) as coded; plus lku_m = 2*nst^2.
  if (isw != 2) return 0.0;
  const bool hexa = (nen == 20);
  const int nu = hexa ? 20 : 10, np = hexa ? 8 : 4, ngp = hexa ? 64 : 4;
  const int nst = 3 * nu + np;
  const double sf_lin = hexa ? (6 + 8 * 3 + 24 * 2) : 1;
  const double sf_quad = hexa ? 20 * 3 * 6.0 : 10 * 3 * 2.0;
  const double jac = 9.0 * np * 2 + 17 + 9 * 4;
  const double map = (np + nu) * 15.0;
  const double geom = sf_lin + sf_quad + jac + map + (hexa ? 3 : 2);
  const double per_gp = nu * nu * 66.0 + np * (1.0 + 6.0 * nu) + 1 +
                        np * np * 10.0 + 2 + geom;
  return ngp * per_gp + 2.0 * nst * nst;
}

}  // extern "C"
