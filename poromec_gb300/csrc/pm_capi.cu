// pm_capi.cu -- C ABI of the GB300 Biot hot path: handle management, the
// pform_pm / matvec / solv_pm replacements and the 'solv' macro step driver.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <type_traits>

#include "pm_internal.h"
#include "pm_loads.h"

using pm::Handle;

namespace {

constexpr int kGraphIters = 16;  // Krylov iterations per captured graph

#define PM_CUDA(call)                                                        \
  do {                                                                       \
    cudaError_t e_ = (call);                                                 \
    if (e_ != cudaSuccess) {                                                 \
      h->err = std::string(#call) + ": " + cudaGetErrorString(e_);           \
      return PM_E_CUDA;                                                      \
    }                                                                        \
  } while (0)

#define PM_TRY(call)              \
  do {                            \
    int st_ = (call);             \
    if (st_ != PM_OK) return st_; \
  } while (0)

// pload_pm (Pload.f:1-92): nodal loads and prescribed values at t.
__global__ void k_pload(int nnode, const int32_t* __restrict__ eq, const int32_t* __restrict__ fnno,
                        const int32_t* __restrict__ nload, double* __restrict__ f,
                        double* __restrict__ u, double* __restrict__ b0,
                        const int32_t* __restrict__ load, const double* __restrict__ fload,
                        int maxt, const double* __restrict__ x, double t, double dt,
                        double gmod) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nnode; i += gridDim.x * blockDim.x) {
    const int nj = fnno[i] == 1 ? 4 : 3;
    for (int j = 0; j < nj; ++j) {
      const size_t q = (size_t)4 * i + j;
      const int nc = nload ? nload[q] : 0;
      if (nc > 0) f[q] = pm::nodal_load(load, fload, maxt, nc, t, x + 3 * i, u[q], gmod);
      const int k = eq[q];
      if (k > 0) b0[k - 1] = (j < 3) ? f[q] : -dt * f[q];
      else u[q] = f[q];
    }
  }
}

// delta_predict_pm (Predict.f:117-158): u = u - u0
__global__ void k_predict(int nnode, const int32_t* __restrict__ fnno, double* __restrict__ u,
                          const double* __restrict__ u0) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nnode; i += gridDim.x * blockDim.x) {
    const int nj = fnno[i] == 1 ? 4 : 3;
    for (int j = 0; j < nj; ++j) u[4 * i + j] -= u0[4 * i + j];
  }
}

// delta_update_pm (Predict.f:159-215): du += x on free dofs (nothing when
// *skip is set: a device-driven step whose solve failed)
__global__ void k_delta_update(int nnode, const int32_t* __restrict__ eq,
                               const int32_t* __restrict__ fnno, double* __restrict__ u,
                               const double* __restrict__ x, const int* skip = nullptr) {
  if (skip && *skip) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nnode; i += gridDim.x * blockDim.x) {
    const int nj = fnno[i] == 1 ? 4 : 3;
    for (int j = 0; j < nj; ++j) {
      const int k = eq[4 * i + j];
      if (k > 0) u[4 * i + j] += x[k - 1];
    }
  }
}

// tform_pm's average over the elements that share a vertex node (mid-side
// nodes keep zeros) and effective_stress (Pform.f:2487-2505): txe = tx + p
// on the normal components
__global__ void k_stress_finish(int nnode, const int32_t* __restrict__ fnno,
                                const int32_t* __restrict__ cnt, const double* __restrict__ u,
                                double* __restrict__ tx, double* __restrict__ txb,
                                double* __restrict__ txe, double* __restrict__ flux) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nnode; i += gridDim.x * blockDim.x) {
    if (fnno[i] == 1 && cnt[i] > 0) {
      const double c = (double)cnt[i];
      for (int j = 0; j < 6; ++j) {
        tx[6 * (size_t)i + j] = tx[6 * (size_t)i + j] / c;
        txb[6 * (size_t)i + j] = txb[6 * (size_t)i + j] / c;
      }
      for (int j = 0; j < 3; ++j) flux[3 * (size_t)i + j] = flux[3 * (size_t)i + j] / c;
    }
    const double p = u[4 * (size_t)i + 3];
    for (int j = 0; j < 6; ++j) txe[6 * (size_t)i + j] = tx[6 * (size_t)i + j] + (j < 3 ? p : 0.0);
  }
}

// porosity_form's average (Pform.f:1150-1170, elastic: the change is added)
__global__ void k_poro_finish(int nnode, const int32_t* __restrict__ fnno,
                              const int32_t* __restrict__ cnt, const double* __restrict__ dporo,
                              double* __restrict__ poro) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nnode; i += gridDim.x * blockDim.x)
    if (fnno[i] == 1 && cnt[i] > 0) poro[i] = poro[i] + dporo[i] / (double)cnt[i];
}

// equation-space vector -> nodal layout (4 per node), zero on restrained dofs
__global__ void k_eq_to_nodal(int nnode, const int32_t* __restrict__ eq,
                              const double* __restrict__ v, double* __restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 4 * nnode;
       i += gridDim.x * blockDim.x) {
    const int k = eq[i];
    out[i] = k > 0 ? v[k - 1] : 0.0;
  }
}

// update_res_v2 (Pload.f:483-540): u = u0 + du, u0 = u, dp += du_p
__global__ void k_update_res(int nnode, const int32_t* __restrict__ fnno, double* __restrict__ u,
                             double* __restrict__ u0, double* __restrict__ dp) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nnode; i += gridDim.x * blockDim.x) {
    for (int j = 0; j < 3; ++j) {
      const double v = u0[4 * i + j] + u[4 * i + j];
      u[4 * i + j] = v;
      u0[4 * i + j] = v;
    }
    if (fnno[i] == 1) {
      dp[i] += u[4 * i + 3];
      const double v = u0[4 * i + 3] + u[4 * i + 3];
      u[4 * i + 3] = v;
      u0[4 * i + 3] = v;
    }
  }
}

int grid_for(int n) {
  int g = (n + 255) / 256;
  return std::max(1, std::min(g, 4 * pm::kRedBlocks));
}

pm::ElemLaunch elem_launch(Handle* h, int c) {
  pm::ElemLaunch L;
  L.ix = h->D.ix;
  L.eq = h->D.eq;
  L.x = h->D.x;
  L.mat = h->D.mat;
  L.slot = h->D.slot + (size_t)h->nen * h->nen * h->color_ptr[c];
  L.elems = h->D.color_elems + h->color_ptr[c];
  L.nelem = h->color_ptr[c + 1] - h->color_ptr[c];
  L.nen = h->nen;
  L.node_val_off = h->P.node_val_off;
  L.node_W = h->P.node_W;
  L.dt = h->dt;
  L.t = h->t;
  L.g0 = h->gravity[0];
  L.g1 = h->gravity[1];
  L.g2 = h->gravity[2];
  L.gmod = h->gravity_mod;
  L.err = h->D.err;
  return L;
}

int check_elem_err(Handle* h) {
  int e = 0;
  PM_CUDA(cudaMemcpyAsync(&e, h->D.err, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  PM_CUDA(cudaStreamSynchronize(h->stream));
  if (e) {
    PM_CUDA(cudaMemsetAsync(h->D.err, 0, sizeof(int), h->stream));
    h->err = "element Jacobian determinant <= 1e-14";
    return PM_E_DET;
  }
  return PM_OK;
}

// isw 2 with lhs: K into the FP64 panels (the FP32 and compensated copies
// are rounded from them); with b also rhs (b -= K_e u_e) in the same element
// launch.
int assemble_K(Handle* h, const double* u = nullptr, double* b = nullptr) {
  PM_CUDA(cudaMemsetAsync(h->P.val, 0, sizeof(double) * (size_t)h->P.nnz, h->stream));
  h->launches += h->numcolors;
  for (int c = 0; c < h->numcolors; ++c)
    PM_CUDA(pm::launch_assemble_K(elem_launch(h, c), h->hexa, h->P.val, h->stream, u, b));
  h->assembled = true;
  h->assembled32 = h->assembledC = false;
  h->assembled_dt = h->dt;
  return PM_OK;
}

int residual(Handle* h, const double* du, double* b) {
  h->launches += h->numcolors;
  for (int c = 0; c < h->numcolors; ++c)
    PM_CUDA(pm::launch_residual(elem_launch(h, c), h->hexa, du, b, h->stream));
  return PM_OK;
}

int rhs4(Handle* h, const double* u, double* b) {
  h->launches += h->numcolors;
  for (int c = 0; c < h->numcolors; ++c)
    PM_CUDA(pm::launch_rhs4(elem_launch(h, c), h->hexa, u, h->D.dp, h->D.eload, h->D.eloadp,
                            h->D.load, h->D.fload, h->maxt, b, h->stream));
  return PM_OK;
}

// Preconditioner of cal_precond (Precond.f:1601-1721) from the FP64 diagonal.
int build_precond(Handle* h, int precond) {
  if (precond != 2 && precond != 5) {
    h->err = "precond must be 2 (diag) or 5 (|diag|)";
    return PM_E_ARG;
  }
  h->launches += 2;
  PM_CUDA(pm::panel_diag(h->P.view(), h->P.val, nullptr, h->D.ad, h->stream));
  PM_CUDA(cudaMemsetAsync(h->D.err, 0, sizeof(int), h->stream));
  PM_CUDA(pm::precond(h->neq, h->D.ad, h->D.m, precond == 5, h->D.err, h->stream));
  int z = 0;
  PM_CUDA(cudaMemcpyAsync(&z, h->D.err, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  PM_CUDA(cudaStreamSynchronize(h->stream));
  if (z) {
    PM_CUDA(cudaMemsetAsync(h->D.err, 0, sizeof(int), h->stream));
    h->err = "zero diagonal coefficient";
    return PM_E_ZERO_DIAG;
  }
  return PM_OK;
}

int read_scalars(Handle* h, pm::KrylovScalars* ks) {
  PM_CUDA(cudaMemcpyAsync(ks, h->D.ks, sizeof(pm::KrylovScalars), cudaMemcpyDeviceToHost,
                          h->stream));
  PM_CUDA(cudaStreamSynchronize(h->stream));
  return PM_OK;
}

// Captures kGraphIters Krylov iterations into an executable graph.
template <typename Body>
int capture(Handle* h, cudaGraphExec_t* exec, Body body) {
  if (*exec) {
    cudaGraphExecDestroy(*exec);
    *exec = nullptr;
  }
  cudaGraph_t g;
  PM_CUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
  cudaError_t be = cudaSuccess;
  for (int k = 0; k < kGraphIters && be == cudaSuccess; ++k) be = body();
  cudaError_t ee = cudaStreamEndCapture(h->stream, &g);
  if (be != cudaSuccess || ee != cudaSuccess) {
    h->err = std::string("graph capture: ") +
             cudaGetErrorString(be != cudaSuccess ? be : ee);
    return PM_E_CUDA;
  }
  cudaError_t ie = cudaGraphInstantiate(exec, g, 0);
  cudaGraphDestroy(g);
  if (ie != cudaSuccess) {
    h->err = std::string("graph instantiate: ") + cudaGetErrorString(ie);
    return PM_E_CUDA;
  }
  return PM_OK;
}

// A whole FP64 PCG solve as one graph: a conditional while node whose body
// is kGraphIters iterations followed by loop_next, which keeps the loop going
// while the solve runs (and bounds its trips by maxit), so the host waits
// once per solve instead of once per kGraphIters iterations.  Built on the
// first solve; if the driver refuses any part, the solve keeps the polled
// graphs (run_graph).
int build_pcg_loop(Handle* h) {
  if (h->pcg_loop || h->pcg_loop_failed) return PM_OK;
  if (std::getenv("PM_POLLED_GRAPHS")) {  // the host-polled graphs instead
    h->pcg_loop_failed = true;
    return PM_OK;
  }
  const pm::PanelView P = h->P.view();
  pm::KrylovVecs& V = h->D.kv;
  const int n = h->neq;
  cudaGraph_t g = nullptr;
  cudaGraphExec_t exec = nullptr;
  bool ok = cudaGraphCreate(&g, 0) == cudaSuccess;
  cudaGraphConditionalHandle cond{};
  cudaGraphNodeParams np{};
  cudaGraphNode_t node{};
  if (ok && !h->D.trips) ok = cudaMalloc(&h->D.trips, sizeof(int)) == cudaSuccess;
  // the handle is 0 at every launch; the start kernel sets it to 1
  if (ok) ok = cudaGraphConditionalHandleCreate(&cond, g, 0, cudaGraphCondAssignDefault) ==
               cudaSuccess;
  cudaGraphNode_t start{};
  if (ok) {
    ok = cudaStreamBeginCaptureToGraph(h->stream, g, nullptr, nullptr, 0,
                                       cudaStreamCaptureModeThreadLocal) == cudaSuccess;
    if (ok) {
      const cudaError_t le = pm::loop_start(h->D.trips, cond, h->stream);
      cudaGraph_t out = nullptr;
      ok = cudaStreamEndCapture(h->stream, &out) == cudaSuccess && le == cudaSuccess;
    }
    size_t nn = 1;
    if (ok) ok = cudaGraphGetNodes(g, &start, &nn) == cudaSuccess && nn == 1;
  }
  if (ok) {
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = cond;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    ok = cudaGraphAddNode(&node, g, &start, nullptr, 1, &np) == cudaSuccess;
  }
  if (ok) {
    cudaGraph_t body = np.conditional.phGraph_out[0];
    ok = cudaStreamBeginCaptureToGraph(h->stream, body, nullptr, nullptr, 0,
                                       cudaStreamCaptureModeThreadLocal) == cudaSuccess;
    if (ok) {
      cudaError_t be = cudaSuccess;
      for (int k = 0; k < kGraphIters && be == cudaSuccess; ++k)
        be = pm::pcg_iteration(P, h->P.val, n, h->D.m, V, h->D.ks, h->D.partial, h->D.counter,
                               h->stream);
      if (be == cudaSuccess) be = pm::loop_next(h->D.ks, h->D.trips, cond, kGraphIters, h->stream);
      cudaGraph_t out = nullptr;
      const cudaError_t ee = cudaStreamEndCapture(h->stream, &out);
      ok = be == cudaSuccess && ee == cudaSuccess;
    }
  }
  if (ok) ok = cudaGraphInstantiate(&exec, g, 0) == cudaSuccess;
  if (g) cudaGraphDestroy(g);
  if (!ok) {
    cudaGetLastError();  // the refusal is not this solve's error
    h->pcg_loop_failed = true;
    if (h->debug) fprintf(stderr, "device-side PCG loop unavailable: polled graphs\n");
    return PM_OK;
  }
  h->pcg_loop = exec;
  return PM_OK;
}

// Runs graphs of kGraphIters iterations until the solve's flag is set.
int run_graph(Handle* h, cudaGraphExec_t g, pm::KrylovScalars* ks) {
  for (;;) {
    PM_CUDA(cudaGraphLaunch(g, h->stream));
    h->launches += 3 * kGraphIters;
    PM_TRY(read_scalars(h, ks));
    if (ks->conv_flag) return PM_OK;
  }
}

// sym_ortho2 (Iters.f:6718-6745)
void sym_ortho2(double a, double b, double& c, double& s, double& r) {
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

// gmres2 (Iters.f:1411-1700) on the device: restarted GMRES(k), diagonal
// preconditioner on the left, modified Gram-Schmidt with a second pass when
// |w| drops to kesp = 0.25 of its value before orthogonalisation, Givens QR.
// maxit counts cycles; x (device) starts at 0; conv = tol |M b|.  The basis
// and scalars live in HBM; the host keeps H, the rotations and e (k + 1
// values) and reads the step's dot products once per Arnoldi step (twice
// with the second pass).
int gmres_run(Handle* h, const double* d_b, double* x, double tol, int maxit, int* nit_out,
              double* econv_out) {
  const int n = h->neq, k = h->nkrylov;
  pm::Dev& D = h->D;
  cudaStream_t st = h->stream;
  if (h->gm_alloc_k < k) {
    for (double** p : {&D.gm_basis, &D.gm_scal, &D.gm_y})
      if (*p) {
        cudaFree(*p);
        *p = nullptr;
      }
    h->gm_alloc_k = 0;
    if (cudaMalloc(&D.gm_basis, sizeof(double) * (size_t)(k + 1) * n) != cudaSuccess ||
        cudaMalloc(&D.gm_scal, sizeof(double) * (size_t)(2 * k + 4)) != cudaSuccess ||
        cudaMalloc(&D.gm_y, sizeof(double) * (size_t)k) != cudaSuccess) {
      cudaGetLastError();
      h->err = "GMRES(l): cannot allocate the Krylov basis ((nkrylov + 1) x neq doubles)";
      return PM_E_NOMEM;
    }
    h->gm_alloc_k = k;
  }
  const pm::PanelView P = h->P.view();
  const double* val64 = h->P.val;
  double* G = D.gm_basis;
  double* gs = D.gm_scal;
  auto g = [&](int j) { return G + (size_t)(j - 1) * n; };
  std::vector<double> H((size_t)(k + 1) * k, 0.0), c(k), sn(k), e(k + 1), y(k), hs(2 * k + 4);
  auto Hm = [&](int i, int j) -> double& { return H[(size_t)(k + 1) * (j - 1) + (i - 1)]; };
  auto read = [&](int a, int cnt) -> int {
    PM_CUDA(cudaMemcpyAsync(hs.data() + a, gs + a, sizeof(double) * cnt,
                            cudaMemcpyDeviceToHost, st));
    PM_CUDA(cudaStreamSynchronize(st));
    return PM_OK;
  };
  const double kesp = 0.25;
  PM_CUDA(cudaMemsetAsync(x, 0, sizeof(double) * n, st));
  PM_CUDA(pm::gm_resid(n, d_b, nullptr, D.m, g(1), gs, D.partial, D.counter, st));
  PM_TRY(read(0, 1));
  h->launches += 1;
  double norm = std::sqrt(hs[0]);
  const double econv = tol * norm;
  *econv_out = econv;
  *nit_out = 0;
  if (norm == 0.0) return PM_OK;
  int nit = 0, ni = 0;
  for (int l = 1; l <= maxit; ++l) {
    PM_CUDA(pm::spmv(P, val64, x, g(1), 0, nullptr, nullptr, nullptr, st));
    PM_CUDA(pm::gm_resid(n, d_b, g(1), D.m, g(1), gs, D.partial, D.counter, st));
    PM_TRY(read(0, 1));
    e[0] = std::sqrt(hs[0]);
    if (!(e[0] > 0.0) || !std::isfinite(e[0])) {
      if (e[0] == 0.0) break;  // x solves the system exactly
      h->err = "GMRES(l): non-finite residual";
      *nit_out = nit;
      return PM_E_NOCONV;
    }
    PM_CUDA(pm::gm_scale(n, g(1), 1.0 / e[0], st));
    h->launches += 3;
    ni = 0;
    for (int i = 1; i <= k; ++i) {
      ++nit;
      ++ni;
      double* w = g(i + 1);
      PM_CUDA(pm::spmv(P, val64, g(i), w, 0, nullptr, nullptr, nullptr, st));
      PM_CUDA(pm::gm_first(n, w, D.m, g(1), gs, D.partial, D.counter, st));
      for (int j = 1; j <= i; ++j)
        PM_CUDA(pm::gm_mgs(n, w, g(j), j < i ? g(j + 1) : nullptr, gs + j,
                           j < i ? gs + j + 1 : gs + k + 1, D.partial, D.counter, st));
      h->launches += 2 + i;
      PM_TRY(read(0, k + 2));
      const double tau = std::sqrt(hs[0]);
      for (int j = 1; j <= i; ++j) Hm(j, i) = hs[j];
      norm = std::sqrt(hs[k + 1]);
      if (norm <= kesp * tau) {
        PM_CUDA(pm::gm_dot(n, w, g(1), gs + k + 3, D.partial, D.counter, st));
        for (int j = 1; j <= i; ++j)
          PM_CUDA(pm::gm_mgs(n, w, g(j), j < i ? g(j + 1) : nullptr, gs + k + 2 + j,
                             j < i ? gs + k + 3 + j : gs + 2 * k + 3, D.partial, D.counter,
                             st));
        h->launches += 1 + i;
        PM_TRY(read(k + 2, k + 2));
        for (int j = 1; j <= i; ++j) Hm(j, i) = Hm(j, i) + hs[k + 2 + j];
        norm = std::sqrt(hs[2 * k + 3]);
      }
      Hm(i + 1, i) = norm;
      if (norm != 0.0) {
        PM_CUDA(pm::gm_scale(n, w, 1.0 / norm, st));
        h->launches += 1;
      }
      for (int j = 1; j <= i - 1; ++j) {
        const double aux1 = c[j - 1] * Hm(j, i) + sn[j - 1] * Hm(j + 1, i);
        const double aux2 = -sn[j - 1] * Hm(j, i) + c[j - 1] * Hm(j + 1, i);
        Hm(j, i) = aux1;
        Hm(j + 1, i) = aux2;
      }
      double r;
      sym_ortho2(Hm(i, i), Hm(i + 1, i), c[i - 1], sn[i - 1], r);
      Hm(i, i) = r;
      Hm(i + 1, i) = 0.0;
      e[i] = -sn[i - 1] * e[i - 1];
      e[i - 1] = c[i - 1] * e[i - 1];
      if (!std::isfinite(e[i])) {
        h->err = "GMRES(l): breakdown (non-finite Givens rotation) after " +
                 std::to_string(nit) + " iterations";
        *nit_out = nit;
        return PM_E_NOCONV;
      }
      if (std::fabs(e[i]) <= econv) break;
    }
    // R y = e (Iters.f:1575-1585), then x += sum_j y_j g_j
    for (int j = 1; j <= ni; ++j) y[j - 1] = e[j - 1];
    for (int j = ni; j >= 2; --j) {
      y[j - 1] = y[j - 1] / Hm(j, j);
      const double r = y[j - 1];
      for (int i = 1; i <= j - 1; ++i) y[i - 1] = y[i - 1] - Hm(i, j) * r;
    }
    y[0] = y[0] / Hm(1, 1);
    PM_CUDA(cudaMemcpyAsync(D.gm_y, y.data(), sizeof(double) * ni, cudaMemcpyHostToDevice, st));
    PM_CUDA(pm::gm_update(n, x, G, D.gm_y, ni, st));
    h->launches += 1;
    if (h->debug)
      fprintf(stderr, "gmres cycle %d: %d its, |e| %.3e conv %.3e\n", l, nit, std::fabs(e[ni]),
              econv);
    if (std::fabs(e[ni]) <= econv) {
      *nit_out = nit;
      PM_CUDA(cudaStreamSynchronize(st));
      return PM_OK;
    }
  }
  *nit_out = nit;
  if (e[0] == 0.0) return PM_OK;
  h->err = "GMRES(l): no convergence reached after " + std::to_string(maxit) + " cycles (" +
           std::to_string(nit) + " iterations, nkrylov " + std::to_string(k) + ")";
  return PM_E_NOCONV;
}

int check_cs_fault(Handle* h);

// One Krylov solve of K x = b on the device (solv_pm, Solv.f:27-780).
//
// comp = false: the reference's FP64 iteration on the FP64 panels.
// comp = true (PM_FP32C_REFINE): the same recurrences with FP64 vectors,
// scalars and dots, whose operator products run on the compensated FP32
// values (pm_krylov.h), inside an FP64 iterative-refinement loop:
//   PCG:    solve to the reference's test sqrt|(r, m r)| < tol sqrt|(b, m b)|;
//           then r = b - A64 x in FP64; while sqrt|(r, m r)| is above that
//           target, solve A dx = r to the same absolute target, x += dx.
//   MINRES: a restart computes v = b - A64 x in FP64 (Iters.f:4100-4131), so
//           a converged cycle is followed by one such restart whose FP64
//           residual norm beta must also meet the target, else the cycle
//           continues from there (within the reference's 10 restarts).
int krylov(Handle* h, int solver, const double* d_b, double* d_x, double tol, int maxit,
           bool comp, pm_step_info* info) {
  const int n = h->neq;
  pm::KrylovVecs& V = h->D.kv;
  pm::KrylovVecs32& V32 = h->D.kv32;
  const pm::PanelView P = h->P.view();
  const double* val64 = h->P.val;
  const pm::CompVals C = h->P.comp(h->shape);
  pm::KrylovScalars ks{};
  int sweeps = 0;
  double final_target = -1.0;  // compensated MINRES: the target its cycles refine to
  cudaEvent_t e0 = h->ev[0], e1 = h->ev[1];
  PM_CUDA(cudaEventRecord(e0, h->stream));
  if (solver == 1) {
    cudaGraphExec_t* g = comp ? &h->pcgc_graph : &h->pcg_graph;
    if (!*g) {
      PM_TRY(capture(h, g, [&]() {
        return comp ? pm::pcgc_iteration(P, C, n, h->D.m, V, V32, h->D.ks, h->D.partial,
                                         h->D.counter, h->stream)
                    : pm::pcg_iteration(P, val64, n, h->D.m, V, h->D.ks, h->D.partial,
                                        h->D.counter, h->stream);
      }));
    }
    h->launches += 1;
    if (comp)
      PM_CUDA(pm::pcgc_init(n, d_b, h->D.m, V, V32, h->D.ks, tol, -1.0, maxit, h->D.partial,
                            h->D.counter, h->stream));
    else
      PM_CUDA(pm::pcg_init(n, d_b, h->D.m, V, h->D.ks, tol, maxit, h->D.partial, h->D.counter,
                           h->stream));
    if (!comp) {
      PM_TRY(build_pcg_loop(h));
      if (h->pcg_loop) {
        PM_CUDA(cudaGraphLaunch(h->pcg_loop, h->stream));
        PM_TRY(read_scalars(h, &ks));
        h->launches += 1 + (3 * kGraphIters + 1) * ((ks.iter + kGraphIters - 1) / kGraphIters);
        if (ks.conv_flag == 0) {
          // the loop ended without the solve's flag (its condition was not
          // honoured): finish with the polled graphs from where it stopped,
          // and use those from now on
          h->pcg_loop_failed = true;
          cudaGraphExecDestroy(h->pcg_loop);
          h->pcg_loop = nullptr;
          PM_TRY(run_graph(h, *g, &ks));
        }
      } else {
        PM_TRY(run_graph(h, *g, &ks));
      }
    } else {
      // The compensated products (2^-32 per value) make the recursive
      // residual drift from b - A x.  Every time it has fallen by a factor
      // drop (in (r, m r)) since the last replacement, and when it meets
      // pcg's test, it is replaced by the FP64 residual of the current x;
      // the iteration then goes on with the same search direction until the
      // replaced residual itself meets the test (the refinement of the FP64
      // solve, without restarting the Krylov space).  Once the recursive
      // test is met, the search direction has done its work: if the FP64
      // residual misses the test there (or the recurrence breaks down, as it
      // can on small systems whose Krylov space is exhausted), the remaining
      // correction is solved by restarted sweeps with the FP64 operator,
      // A dx = b - A x to the same absolute target, x += dx.  The same
      // sweeps take over when the compensated iteration stalls: a
      // replacement is also made after kForce iterations without one, and
      // when the replaced (r, m r) has not fallen below kProgress times its
      // value at the previous replacement, the compensated operator has
      // reached its own error level (|A| |x| large against |b|: the small
      // increments late in a load history), so the iteration stops there.
      double drop = 1e-4;  // PM_RR_DROP overrides (a tuning knob)
      if (const char* e = std::getenv("PM_RR_DROP")) drop = std::atof(e);
      constexpr int kMaxReplace = 256, kMaxSweeps = 8, kForce = 1024;
      constexpr double kProgress = 0.5;
      double d_ref = -1.0, d_true = -1.0;
      int it_ref = 0;
      bool restart = false;
      for (;;) {
        PM_CUDA(cudaGraphLaunch(*g, h->stream));
        h->launches += 3 * kGraphIters;
        PM_TRY(read_scalars(h, &ks));
        if (d_ref < 0.0) d_ref = d_true = std::fabs(ks.bmb);
        if (ks.conv_flag == 2) break;
        if (ks.conv_flag == 3) {  // x holds the last finite iterate
          restart = d_x != V.x;
          break;
        }
        const bool met = ks.conv_flag == 1;
        const bool force = ks.iter - it_ref >= kForce;
        if (!met && !force && std::fabs(ks.d) > drop * d_ref) continue;
        h->launches += 2;
        PM_CUDA(pm::spmv(P, val64, V.x, h->D.dx, 0, nullptr, nullptr, nullptr, h->stream));
        PM_CUDA(pm::pcgc_replace(n, d_b, h->D.dx, h->D.m, V, h->D.ks, h->D.partial,
                                 h->D.counter, h->stream));
        PM_TRY(read_scalars(h, &ks));
        ++sweeps;
        if (h->debug)
          fprintf(stderr, "residual replacement %d after %d its: sqrt|(r, m r)| %.3e target %.3e\n",
                  sweeps, ks.iter, std::sqrt(std::fabs(ks.d)), ks.conv);
        d_ref = std::fabs(ks.d);
        it_ref = ks.iter;
        if (ks.conv_flag != 0) break;
        const bool stalled = d_ref > kProgress * d_true;
        d_true = d_ref;
        if (met || stalled || sweeps >= kMaxReplace) {
          if (h->debug && stalled && !met)
            fprintf(stderr, "compensated iteration stalled: FP64 correction sweeps\n");
          restart = d_x != V.x;
          if (!restart) ks.conv_flag = 2;
          break;
        }
      }
      if (d_x != V.x)
        PM_CUDA(cudaMemcpyAsync(d_x, V.x, sizeof(double) * n, cudaMemcpyDeviceToDevice,
                                h->stream));
      int total = ks.iter, restarts = 0;
      const double conv = ks.conv;
      while (restart) {
        h->launches += 2;
        PM_CUDA(pm::spmv(P, val64, d_x, h->D.dx, 0, nullptr, nullptr, nullptr, h->stream));
        PM_CUDA(pm::true_residual(n, d_b, h->D.dx, h->D.m, 0, h->D.rr, h->D.norms,
                                  h->D.partial, h->D.counter, h->stream));
        double rn2 = 0.0;
        PM_CUDA(cudaMemcpyAsync(&rn2, h->D.norms, sizeof(double), cudaMemcpyDeviceToHost,
                                h->stream));
        PM_CUDA(cudaStreamSynchronize(h->stream));
        if (h->debug)
          fprintf(stderr, "restarted sweep %d after %d its: sqrt|(r, m r)| %.3e target %.3e\n",
                  restarts, total, std::sqrt(std::fabs(rn2)), conv);
        if (std::sqrt(std::fabs(rn2)) < conv) {
          ks.conv_flag = 1;
          break;
        }
        if (++restarts > kMaxSweeps || total >= maxit) {
          ks.conv_flag = 2;
          break;
        }
        // the correction sits at the compensated operator's noise level:
        // it is solved with the FP64 operator (pcg to the same absolute
        // target, the tolerance rescaled to this right-hand side)
        if (!h->pcg_graph) {
          PM_TRY(capture(h, &h->pcg_graph, [&]() {
            return pm::pcg_iteration(P, val64, n, h->D.m, V, h->D.ks, h->D.partial,
                                     h->D.counter, h->stream);
          }));
        }
        h->launches += 1;
        PM_CUDA(pm::pcg_init(n, h->D.rr, h->D.m, V, h->D.ks, conv / std::sqrt(std::fabs(rn2)),
                             maxit - total, h->D.partial, h->D.counter, h->stream));
        PM_TRY(run_graph(h, h->pcg_graph, &ks));
        total += ks.iter;
        ++sweeps;
        if (ks.conv_flag != 1) break;
        h->launches += 1;
        PM_CUDA(pm::axpy_into(n, d_x, V.x, 1.0, h->stream));
      }
      ks.iter = total;
    }
    if (ks.conv_flag != 1) {
      h->err = ks.conv_flag == 3
                   ? "PCG: breakdown (non-finite recurrence) after " + std::to_string(ks.iter) +
                         " iterations"
                   : "PCG: no convergence reached after " + std::to_string(ks.iter) +
                         " iterations";
      if (info) info->iters = ks.iter;
      return PM_E_NOCONV;
    }
  } else if (solver == 7) {
    cudaGraphExec_t* g = comp ? &h->minresc_graph : &h->minres_graph;
    if (!*g) {
      PM_TRY(capture(h, g, [&]() {
        return comp ? pm::minresc_iteration(P, C, n, h->D.m, V, V32, h->D.ks, h->D.partial,
                                            h->D.counter, h->stream)
                    : pm::minres_iteration(P, val64, n, h->D.m, V, h->D.ks, h->D.partial,
                                           h->D.counter, h->stream);
      }));
    }
    PM_CUDA(cudaMemsetAsync(h->D.ks, 0, sizeof(pm::KrylovScalars), h->stream));
    PM_CUDA(pm::minres_conv(n, d_b, h->D.m, h->D.ks, tol, h->D.partial, h->D.counter,
                            h->stream));
    int nrestart = 10;  // call_minres, Solv.f:1727
    bool zero_x = true, converged = false;
    double conv_final = -1.0;
    for (;;) {
      h->launches += zero_x ? 1 : 2;
      PM_CUDA(pm::minres_start(P, val64, n, d_b, h->D.m, V, comp ? &V32 : nullptr, h->D.ks,
                               maxit, zero_x, h->D.partial, h->D.counter, h->stream));
      if (comp) {
        // beta = the FP64 residual norm ||M^(1/2) (b - A64 x)|| of the restart
        PM_TRY(read_scalars(h, &ks));
        if (conv_final < 0.0) conv_final = final_target = ks.conv;
        if (converged) {
          ++sweeps;
          if (h->debug)
            fprintf(stderr, "refine sweep %d: |b-A64x| %.3e target %.3e after %d its\n",
                    sweeps, ks.beta, conv_final, ks.iter);
          if (ks.beta < conv_final) break;
          if (sweeps >= 8) {
            h->err = "MINRES: the FP64 residual stayed above the target after " +
                     std::to_string(sweeps) + " refinement sweeps";
            if (info) info->iters = ks.iter;
            return PM_E_NOCONV;
          }
        }
        // A compensated cycle aims at a relative reduction inner_tol of its
        // starting FP64 residual (never below the final target): the
        // recursive residual estimate of MINRES can stall near the
        // operator's rounding level (~2^-32 per entry, amplified by the
        // conditioning) before a tight target, while the FP64 restart that
        // follows the cycle carries the refinement.
        h->cycle_conv = std::max(conv_final, h->inner_tol * ks.beta);
        PM_CUDA(cudaMemcpy(&h->D.ks->conv, &h->cycle_conv, sizeof(double),
                           cudaMemcpyHostToDevice));
      }
      zero_x = false;
      PM_TRY(run_graph(h, *g, &ks));
      if (ks.conv_flag == 1) {
        if (!comp) break;
        converged = true;
        continue;
      }
      if (ks.conv_flag == 3) {
        h->err = "MINRES: breakdown (non-finite recurrence) after " + std::to_string(ks.iter) +
                 " iterations";
        return PM_E_NOCONV;
      }
      if (nrestart == 0) {
        h->err = "MINRES: no convergence reached after " + std::to_string(ks.iter) +
                 " iterations";
        if (info) info->iters = ks.iter;
        return PM_E_NOCONV;
      }
      --nrestart;
    }
  } else if (solver == 2) {
    if (comp) {
      h->err = "GMRES(l) (solver 2) runs on the FP64 operator (PM_FP64)";
      return PM_E_ARG;
    }
    int nit = 0;
    PM_TRY(gmres_run(h, d_b, V.x, tol, maxit, &nit, &final_target));
    ks.iter = nit;
  } else if (solver == 11) {
    cudaGraphExec_t* g = comp ? &h->sqmrc_graph : &h->sqmr_graph;
    if (!*g) {
      PM_TRY(capture(h, g, [&]() {
        return comp ? pm::sqmrc_iteration(P, C, n, h->D.m, V, V32, h->D.ks, h->D.partial,
                                          h->D.counter, h->stream)
                    : pm::sqmr_iteration(P, val64, n, h->D.m, V, h->D.ks, h->D.partial,
                                         h->D.counter, h->stream);
      }));
    }
    auto run_sqmr = [&]() -> int {
      for (;;) {
        PM_CUDA(cudaGraphLaunch(*g, h->stream));
        h->launches += 4 * kGraphIters;
        PM_TRY(read_scalars(h, &ks));
        if (ks.conv_flag) return PM_OK;
      }
    };
    h->launches += 1;
    PM_CUDA(pm::sqmr_init(n, d_b, h->D.m, V, comp ? V32.c : nullptr, h->D.ks, tol, -1.0, maxit,
                          h->D.partial, h->D.counter, h->stream));
    PM_TRY(run_sqmr());
    int total = ks.iter;
    const double conv = ks.conv;
    // compensated operator: the FP64 residual b - A64 x (rpsqmr's 2-norm
    // test, conv = tol ||b||) decides; a correction sweep solves for it
    while (comp && ks.conv_flag == 1) {
      h->launches += 3;
      if (sweeps == 0) {
        if (d_x != V.x)
          PM_CUDA(cudaMemcpyAsync(d_x, V.x, sizeof(double) * n, cudaMemcpyDeviceToDevice,
                                  h->stream));
      } else {
        PM_CUDA(pm::axpy_into(n, d_x, V.x, 1.0, h->stream));
      }
      PM_CUDA(pm::spmv(P, val64, d_x, h->D.dx, 0, nullptr, nullptr, nullptr, h->stream));
      PM_CUDA(pm::true_residual(n, d_b, h->D.dx, nullptr, 2, h->D.rr, h->D.norms, h->D.partial,
                                h->D.counter, h->stream));
      double rn2 = 0.0;
      PM_CUDA(cudaMemcpyAsync(&rn2, h->D.norms, sizeof(double), cudaMemcpyDeviceToHost,
                              h->stream));
      PM_CUDA(cudaStreamSynchronize(h->stream));
      ++sweeps;
      if (h->debug)
        fprintf(stderr, "refine sweep %d: |b-A64x| %.3e target %.3e after %d its\n", sweeps,
                std::sqrt(std::fabs(rn2)), conv, total);
      if (std::sqrt(std::fabs(rn2)) < conv) break;
      if (sweeps >= 8 || total >= maxit) {
        ks.conv_flag = 2;
        break;
      }
      h->launches += 1;
      PM_CUDA(pm::sqmr_init(n, h->D.rr, h->D.m, V, V32.c, h->D.ks, tol, conv, maxit - total,
                            h->D.partial, h->D.counter, h->stream));
      PM_TRY(run_sqmr());
      total += ks.iter;
    }
    ks.iter = total;
    if (ks.conv_flag == 2) {
      // Solv.f:765: rpsqmr reached maxit; GMRES(l) from x = 0 (FP64 operator)
      const int its = ks.iter;
      int nit = 0;
      if (h->debug) fprintf(stderr, "rpsqmr: maxit reached, switching to GMRES(l)\n");
      const int st2 = gmres_run(h, d_b, comp ? d_x : V.x, tol, maxit, &nit, &final_target);
      if (st2 != PM_OK) {
        if (info) info->iters = its + nit;
        return st2;
      }
      ks.iter = its + nit;
      ks.conv_flag = 1;
    }
    if (ks.conv_flag != 1) {
      h->err = "rpsqmr: breakdown (sigma or rho zero, or non-finite) after " +
               std::to_string(ks.iter) + " iterations";
      if (info) info->iters = ks.iter;
      return PM_E_NOCONV;
    }
  } else {
    h->err = "solver must be 1 (pcg), 2 (gmres), 7 (minres) or 11 (rpsqmr)";
    return PM_E_ARG;
  }
  if (comp && h->shape == pm::kCsShape) PM_TRY(check_cs_fault(h));
  PM_CUDA(cudaEventRecord(e1, h->stream));
  // x.Kx of the solver log (one more product with the converged x)
  const double* xs = (comp && (solver == 1 || solver == 11)) ? d_x : V.x;
  h->launches += 1;
  PM_CUDA(pm::spmv(P, val64, xs, V.q, 3, h->D.ks, h->D.partial, h->D.counter, h->stream));
  if (d_x != xs)
    PM_CUDA(cudaMemcpyAsync(d_x, xs, sizeof(double) * n, cudaMemcpyDeviceToDevice, h->stream));
  const int iters = ks.iter;
  PM_TRY(read_scalars(h, &ks));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  h->timers[5] = ms;
  h->timers[6] = iters;
  if (info) {
    info->iters = iters;
    info->refine = sweeps;
    info->conv = final_target > 0.0 ? final_target : ks.conv;
    info->xkx = ks.xkx;
  }
  return PM_OK;
}

// FP32 values + FP64 iterative refinement (PM_FP32_REFINE):
//   x = 0, r = b
//   repeat: if ||r||_|M| <= tol ||b||_|M|: done
//           solve A32 dx = r by PCG (Iters.f:299-595 recurrences) whose
//             products use the FP32 panel values and FP32 copies of the
//             direction, everything else (vectors, dots, scalars) FP64,
//             to a relative tolerance inner_tol
//           x += dx;  r = b - A64 x  (FP64 panels, FP64 arithmetic)
// ||.||_|M| = sqrt(sum |m_i| r_i^2) is a norm also on this indefinite
// system.  An inner solve that stalls at the FP32 operator's rounding floor
// stops at its iteration cap and hands its progress to the next sweep.
int solve_mixed(Handle* h, int solver, const double* d_b, double* d_x, double tol, int maxit,
                pm_step_info* info) {
  if (solver != 1) {
    h->err = "the FP32 + FP64-refinement mode is implemented for PCG (solver 1)";
    return PM_E_ARG;
  }
  const int n = h->neq;
  const pm::PanelView P = h->P.view();
  pm::KrylovVecs& V = h->D.kv;
  pm::KrylovVecs32& V32 = h->D.kv32;
  double* r = h->D.rr;
  if (!h->pcgm_graph) {
    PM_TRY(capture(h, &h->pcgm_graph, [&]() {
      return pm::pcgm_iteration(P, h->P.val32, n, h->D.m, V, V32, h->D.ks, h->D.partial,
                                h->D.counter, h->stream);
    }));
  }
  cudaEvent_t e0 = h->ev[0], e1 = h->ev[1];
  PM_CUDA(cudaEventRecord(e0, h->stream));
  PM_CUDA(cudaMemsetAsync(d_x, 0, sizeof(double) * n, h->stream));
  PM_CUDA(cudaMemcpyAsync(r, d_b, sizeof(double) * n, cudaMemcpyDeviceToDevice, h->stream));
  double bnorm = -1.0;
  int total = 0, sweep = 0, cap = maxit;
  const int kMaxSweeps = 30;
  for (sweep = 0; sweep < kMaxSweeps; ++sweep) {
    double rn2 = 0.0;
    h->launches += 1;
    PM_CUDA(pm::wnorm2(n, r, h->D.m, h->D.norms, h->D.partial, h->D.counter, h->stream));
    PM_CUDA(cudaMemcpyAsync(&rn2, h->D.norms, sizeof(double), cudaMemcpyDeviceToHost,
                            h->stream));
    PM_CUDA(cudaStreamSynchronize(h->stream));
    const double rn = std::sqrt(rn2);
    if (bnorm < 0) bnorm = rn;
    if (rn <= tol * bnorm || rn == 0.0) break;
    const double itol = std::max(h->inner_tol, 0.3 * tol * bnorm / rn);
    pm::KrylovScalars ks{};
    h->launches += 1;
    PM_CUDA(pm::pcgm_init(n, r, h->D.m, V, V32, h->D.ks, itol, std::min(cap, maxit),
                          h->D.partial, h->D.counter, h->stream));
    for (;;) {
      PM_CUDA(cudaGraphLaunch(h->pcgm_graph, h->stream));
      h->launches += 3 * kGraphIters;
      PM_TRY(read_scalars(h, &ks));
      if (ks.conv_flag) break;
    }
    if (h->debug)
      fprintf(stderr, "refine sweep %d: |r|_|M| %.3e / %.3e, inner tol %.1e, its %d, flag %d\n",
              sweep, rn, bnorm, itol, ks.iter, ks.conv_flag);
    if (ks.conv_flag == 3) {
      h->err = "refinement: inner PCG breakdown (non-finite recurrence)";
      return PM_E_NOCONV;
    }
    total += ks.iter;
    if (sweep == 0) cap = std::max(200, 3 * ks.iter);
    if (total > maxit) {
      h->err = "refinement: no convergence after " + std::to_string(total) + " inner iterations";
      if (info) info->iters = total;
      return PM_E_NOCONV;
    }
    // x += dx;  r = b - A64 x
    h->launches += 3;
    PM_CUDA(pm::axpy_into(n, d_x, V.x, 1.0, h->stream));
    PM_CUDA(pm::spmv(P, h->P.val, d_x, h->D.by, 0, nullptr, nullptr, nullptr, h->stream));
    PM_CUDA(pm::vsub(n, r, d_b, h->D.by, h->stream));
  }
  if (sweep == kMaxSweeps) {
    h->err = "refinement: no convergence after " + std::to_string(kMaxSweeps) + " sweeps";
    return PM_E_NOCONV;
  }
  PM_CUDA(cudaEventRecord(e1, h->stream));
  PM_CUDA(cudaEventSynchronize(e1));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  h->timers[5] = ms;
  h->timers[6] = total;
  if (info) {
    info->iters = total;
    info->refine = sweep;
    info->conv = tol * bnorm;
  }
  return PM_OK;
}

// Autotuner of the compensated SpMV: times each shape (lanes per node 8, 16,
// 32 x columns per lane and trip 1, 2, 4, and the record kernel) on this matrix, 3 launches each
// after one warm-up, with CUDA events on the launching stream, and keeps the
// fastest for the handle's lifetime (graphs captured later bake it in).
// PM_SPMV_SHAPE=<code> in the environment fixes the choice instead.
// The streamed SpMV's fault flag (a bounded pipeline wait gave up): cleared
// and reported once.
int check_cs_fault(Handle* h) {
  if (!h->P.fault) return PM_OK;
  int f = 0;
  PM_CUDA(cudaMemcpyAsync(&f, h->P.fault, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  PM_CUDA(cudaStreamSynchronize(h->stream));
  if (!f) return PM_OK;
  PM_CUDA(cudaMemsetAsync(h->P.fault, 0, sizeof(int), h->stream));
  h->err = "streamed SpMV: a pipeline wait gave up (results of that product are invalid)";
  return PM_E_CUDA;
}

int tune_spmvc(Handle* h, cudaStream_t s) {
  if (h->shape) return PM_OK;
  if (const char* env = std::getenv("PM_SPMV_SHAPE")) {
    const int u = std::atoi(env);
    for (int c : pm::kCfShapes)
      if (u == c && !(c == pm::kCaShape && (h->P.ca_warps == 0 || h->ninst > 0)) &&
          !(c == pm::kCsShape && (h->P.cs_nstage == 0 || h->ninst > 0))) {
        h->shape = u;
        return PM_OK;
      }
  }
  const pm::PanelView P = h->P.view();
  PM_CUDA(cudaMemsetAsync(h->D.kv32.c, 0, sizeof(float2) * std::max(h->neq, 1), s));
  // the PCG form (product fused with p.Ap), as the solver runs it: it writes
  // only ks->pq and ks->alpha, which every solver's init sets again
  PM_CUDA(cudaMemsetAsync(h->D.ks, 0, sizeof(pm::KrylovScalars), s));
  constexpr int kReps = 5, kPasses = 2, kWarm = 10;
  std::vector<int> cand;
  for (int c : pm::kCfShapes)
    // the record kernel: only where two records per warp fit in shared
    // memory, and not for batches (it does not skip converged instances)
    if (!(c == pm::kCaShape && (h->P.ca_warps == 0 || h->ninst > 0)) &&
        !(c == pm::kCsShape && (h->P.cs_nstage == 0 || h->ninst > 0)))
      cand.push_back(c);
  auto run = [&](int c) {
    const pm::CompVals C = h->P.comp(c);
    return h->ninst > 0 ? pm::spmvc(P, C, h->D.kv32.c, h->D.dx, s)
                        : pm::spmvc_pcg(P, C, h->D.kv32.c, h->D.dx, h->D.xs, h->D.ks,
                                        h->D.partial, h->D.counter, s);
  };
  // clocks settle before the first timing
  for (int k = 0; k < kWarm; ++k) PM_CUDA(run(cand[0]));
  h->launches += kWarm;
  std::vector<float> best_ms(cand.size(), 1e30f);
  for (int pass = 0; pass < kPasses; ++pass)
    for (size_t i = 0; i < cand.size(); ++i) {
      PM_CUDA(run(cand[i]));
      PM_CUDA(cudaEventRecord(h->ev[0], s));
      for (int k = 0; k < kReps; ++k) PM_CUDA(run(cand[i]));
      PM_CUDA(cudaEventRecord(h->ev[1], s));
      PM_CUDA(cudaEventSynchronize(h->ev[1]));
      float ms = 0.f;
      PM_CUDA(cudaEventElapsedTime(&ms, h->ev[0], h->ev[1]));
      best_ms[i] = std::min(best_ms[i], ms / kReps);
      h->launches += 1 + kReps;
    }
  // a shape whose pipeline reported a fault is not chosen
  if (check_cs_fault(h) != PM_OK)
    for (size_t i = 0; i < cand.size(); ++i)
      if (cand[i] == pm::kCsShape) best_ms[i] = 1e30f;
  size_t bi = 0;
  for (size_t i = 0; i < cand.size(); ++i) {
    if (h->debug) fprintf(stderr, "spmv autotune: shape %3d  %.4f ms\n", cand[i], best_ms[i]);
    if (best_ms[i] < best_ms[bi]) bi = i;
  }
  h->shape = cand[bi];
  return PM_OK;
}

// Compensated copies of the current FP64 panel values (PM_FP32C_REFINE).
// Until the autotuner has chosen, both layouts are written; afterwards only
// the one its shape reads.
int ensure_comp(Handle* h, cudaStream_t s) {
  if (h->assembledC) return PM_OK;
  if (!h->P.valh) {
    PM_CUDA(cudaMalloc(&h->P.valh, sizeof(float) * (size_t)h->P.nnz));
    PM_CUDA(cudaMalloc(&h->P.vall, sizeof(int8_t) * (size_t)h->P.nnz));
    if (h->ninst == 0) PM_TRY(pm::build_rec_layout(h));  // batches do not use records
  }
  if (h->shape != pm::kCaShape) {
    h->launches += 1;
    PM_CUDA(pm::split_values(h->P.nnz, h->P.val, h->P.valh, h->P.vall, s));
  }
  if (h->P.rec && (h->shape == 0 || h->shape == pm::kCaShape || h->shape == pm::kCsShape)) {
    h->launches += 1;
    PM_CUDA(pm::split_records(h->P.view(), h->P.val, h->P.comp(h->shape), s));
  }
  h->assembledC = true;
  return tune_spmvc(h, s);
}

// y = A x by the handle's operator: FP64 panels, or in PM_FP32C_REFINE the
// compensated one (x split into its FP32 pair first).
int spmv_op(Handle* h, const double* d_x, double* d_y, cudaStream_t s) {
  if (h->precision == PM_FP32C_REFINE) {
    PM_TRY(ensure_comp(h, s));
    h->launches += 2;
    PM_CUDA(pm::split_pair(h->neq, d_x, h->D.kv32.c, s));
    PM_CUDA(pm::spmvc(h->P.view(), h->P.comp(h->shape), h->D.kv32.c,
                      d_y, s));
    return PM_OK;
  }
  h->launches += 1;
  PM_CUDA(pm::spmv(h->P.view(), h->P.val, d_x, d_y, 0, nullptr, nullptr, nullptr, s));
  return PM_OK;
}

// ---- batches of independent meshes -------------------------------------------
// Device tables of the segmented layout (BatchView) from the equation
// ranges of the instances; equations are numbered in node order, so each
// instance's equations are one contiguous range.
int batch_setup(Handle* h) {
  const int ni = h->ninst;
  std::vector<int32_t> lo(ni, 0x7fffffff), hi(ni, -1);
  for (int i = 0; i < ni; ++i)
    for (int n = h->h_inst_node[i]; n < h->h_inst_node[i + 1]; ++n)
      for (int j = 0; j < 4; ++j) {
        const int e = h->h_eq[(size_t)4 * n + j];
        if (e > 0) {
          lo[i] = std::min(lo[i], e - 1);
          hi[i] = std::max(hi[i], e);
        }
      }
  h->h_inst_eq.assign(ni + 1, 0);
  for (int i = 0; i < ni; ++i) {
    if (hi[i] < 0) {  // no free equation
      lo[i] = h->h_inst_eq[i];
      hi[i] = h->h_inst_eq[i];
    }
    if (lo[i] != h->h_inst_eq[i]) {
      h->err = "batch: the equations of an instance are not one contiguous range";
      return PM_E_ARG;
    }
    h->h_inst_eq[i + 1] = hi[i];
  }
  if (h->h_inst_eq[ni] != h->neq) {
    h->err = "batch: equation ranges do not cover the system";
    return PM_E_ARG;
  }
  pm::BatchView& B = h->B;
  B.ninst = ni;
  B.chunk = 2048;
  std::vector<int32_t> bptr(ni + 1, 0), binst;
  for (int i = 0; i < ni; ++i) {
    const int cnt = h->h_inst_eq[i + 1] - h->h_inst_eq[i];
    const int nb = std::max(1, (cnt + B.chunk - 1) / B.chunk);
    bptr[i + 1] = bptr[i] + nb;
    for (int k = 0; k < nb; ++k) binst.push_back(i);
  }
  B.nblk = bptr[ni];
  auto up = [&](auto** dst, const auto* src, size_t n) -> int {
    using T = std::remove_pointer_t<std::remove_reference_t<decltype(*dst)>>;
    if (cudaMalloc((void**)dst, sizeof(T) * std::max<size_t>(n, 1)) != cudaSuccess) {
      h->err = "cudaMalloc failed";
      return PM_E_NOMEM;
    }
    if (src) {
      if (cudaMemcpy(*dst, src, sizeof(T) * n, cudaMemcpyHostToDevice) != cudaSuccess) {
        h->err = "cudaMemcpy failed";
        return PM_E_CUDA;
      }
    } else {
      cudaMemset(*dst, 0, sizeof(T) * std::max<size_t>(n, 1));
    }
    return PM_OK;
  };
  int32_t *eq_ptr, *blk_ptr, *blk_inst;
  PM_TRY(up(&eq_ptr, h->h_inst_eq.data(), (size_t)ni + 1));
  PM_TRY(up(&blk_ptr, bptr.data(), (size_t)ni + 1));
  PM_TRY(up(&blk_inst, binst.data(), binst.size()));
  B.eq_ptr = eq_ptr;
  B.blk_ptr = blk_ptr;
  B.blk_inst = blk_inst;
  PM_TRY(up(&B.bs, (pm::BatchScalars*)nullptr, (size_t)ni));
  PM_TRY(up(&B.done, (int*)nullptr, (size_t)ni));
  PM_TRY(up(&B.nactive, (int*)nullptr, 1));
  PM_TRY(up(&B.partial, (double*)nullptr, (size_t)2 * B.nblk));
  PM_TRY(up(&B.counter, (unsigned*)nullptr, (size_t)ni));
  PM_TRY(up(&h->P.node_inst, h->h_inst_act.data(), h->h_inst_act.size()));
  h->P.inst_done = B.done;
  PM_TRY(pm::build_meta(h, h->h_inst_act.data()));
  PM_TRY(up(&h->d_insweep, (int*)nullptr, (size_t)ni));
  PM_TRY(up(&h->d_conv0, (double*)nullptr, (size_t)ni));
  PM_TRY(up(&h->d_bnorms, (double*)nullptr, (size_t)2 * ni));
  pm::BatchStepArrays& A = h->bsa;
  PM_TRY(up(&h->d_bctl, (pm::BatchCtl*)nullptr, 1));
  PM_TRY(up(&A.active, (int*)nullptr, (size_t)ni));
  PM_TRY(up(&A.total, (int*)nullptr, (size_t)ni));
  PM_TRY(up(&A.iters, (int*)nullptr, (size_t)ni));
  PM_TRY(up(&A.nlit, (int*)nullptr, (size_t)ni));
  PM_TRY(up(&A.res0, (double*)nullptr, (size_t)ni));
  PM_TRY(up(&A.resu0, (double*)nullptr, (size_t)ni));
  PM_TRY(up(&A.resp0, (double*)nullptr, (size_t)ni));
  PM_TRY(up(&A.nr, (double*)nullptr, (size_t)2 * ni));
  PM_TRY(up(&A.rn2, (double*)nullptr, (size_t)ni));
  A.insweep = h->d_insweep;
  A.conv0 = h->d_conv0;
  h->b_iters.assign(ni, 0);
  h->b_nlit.assign(ni, 0);
  return PM_OK;
}

// Independent PCG solves of the active instances (active[i] != 0) on the
// union system; inactive instances get x = 0.  comp: the compensated FP32
// operator inside the FP64 refinement of krylov(), per instance: after the
// sweep, r = b - A64 x in FP64, and the instances whose sqrt|(r, m r)| is
// still above their first sweep's target solve A dx = r to that target.
constexpr int kMaxBatchSweeps = 8;  // refinement sweeps of a batch solve

int krylov_batch(Handle* h, const double* d_b, double* d_x, double tol, int maxit, bool comp,
                 const std::vector<int>& active, pm_step_info* info) {
  const int n = h->neq, ni = h->ninst;
  pm::KrylovVecs& V = h->D.kv;
  float2* pair = h->D.kv32.c;
  const pm::PanelView PB = h->P.bview();
  const pm::PanelView P = h->P.view();
  const pm::CompVals C = h->P.comp(h->shape);
  const pm::BatchView& B = h->B;
  cudaStream_t s = h->stream;
  cudaGraphExec_t* g = comp ? &h->bpcgc_graph : &h->bpcg_graph;
  if (!*g) {
    PM_TRY(capture(h, g, [&]() {
      return pm::bpcg_iteration(PB, h->P.val, comp ? &C : nullptr, B, h->D.m, V, pair, s);
    }));
  }
  cudaEvent_t e0 = h->ev[0], e1 = h->ev[1];
  PM_CUDA(cudaEventRecord(e0, s));
  PM_CUDA(cudaMemsetAsync(d_x, 0, sizeof(double) * n, s));
  std::vector<int> insweep(active);
  std::vector<double> conv0(ni, 0.0), rn2(ni, 0.0);
  std::vector<pm::BatchScalars> bs(ni);
  std::vector<int> total(ni, 0);
  int sweeps = 0;
  for (;;) {
    PM_CUDA(cudaMemcpyAsync(h->d_insweep, insweep.data(), sizeof(int) * ni,
                            cudaMemcpyHostToDevice, s));
    PM_CUDA(cudaMemsetAsync(B.nactive, 0, sizeof(int), s));
    h->launches += 1;
    PM_CUDA(pm::bpcg_init(B, sweeps == 0 ? d_b : h->D.rr, h->D.m, V, comp ? pair : nullptr, tol,
                          sweeps == 0 ? nullptr : h->d_conv0, h->d_insweep, maxit, s));
    for (int launched = 0;; launched += kGraphIters) {
      int nact = 0;
      PM_CUDA(cudaMemcpyAsync(&nact, B.nactive, sizeof(int), cudaMemcpyDeviceToHost, s));
      PM_CUDA(cudaStreamSynchronize(s));
      if (nact == 0) break;
      if (launched > maxit + kGraphIters) {  // every instance stops at maxit
        h->err = "batch PCG: iteration count past maxit with instances still active";
        return PM_E_NOCONV;
      }
      PM_CUDA(cudaGraphLaunch(*g, s));
      h->launches += 4 * kGraphIters;
    }
    PM_CUDA(cudaMemcpyAsync(bs.data(), B.bs, sizeof(pm::BatchScalars) * ni,
                            cudaMemcpyDeviceToHost, s));
    PM_CUDA(cudaStreamSynchronize(s));
    for (int i = 0; i < ni; ++i) {
      if (!insweep[i]) continue;
      total[i] += bs[i].iter;
      if (bs[i].conv_flag == 3 || bs[i].conv_flag == 2) {
        h->err = "batch PCG, instance " + std::to_string(i) +
                 (bs[i].conv_flag == 3 ? ": breakdown (non-finite recurrence)"
                                       : ": no convergence reached after " +
                                             std::to_string(total[i]) + " iterations");
        if (info) info->iters = total[i];
        return PM_E_NOCONV;
      }
      if (sweeps == 0) conv0[i] = bs[i].conv;
    }
    h->launches += 1;
    PM_CUDA(pm::baxpy(B, d_x, V.x, h->d_insweep, s));
    ++sweeps;
    if (!comp) break;
    // FP64 outer residual of every instance in the sweep
    h->launches += 2;
    PM_CUDA(pm::spmv(P, h->P.val, d_x, h->D.dx, 0, nullptr, nullptr, nullptr, s));
    PM_CUDA(pm::btrue_residual(B, d_b, h->D.dx, h->D.m, h->D.rr, h->d_bnorms, s));
    PM_CUDA(cudaMemcpyAsync(rn2.data(), h->d_bnorms, sizeof(double) * ni,
                            cudaMemcpyDeviceToHost, s));
    PM_CUDA(cudaStreamSynchronize(s));
    int again = 0;
    for (int i = 0; i < ni; ++i) {
      insweep[i] = insweep[i] && !(std::sqrt(std::fabs(rn2[i])) < conv0[i]) && conv0[i] > 0.0;
      again += insweep[i];
    }
    if (h->debug)
      fprintf(stderr, "batch refine sweep %d: %d instances above target\n", sweeps, again);
    if (again == 0) break;
    if (sweeps >= kMaxBatchSweeps) {
      h->err = "batch refinement: FP64 residual above target after " +
               std::to_string(sweeps) + " sweeps";
      return PM_E_NOCONV;
    }
    PM_CUDA(cudaMemcpyAsync(h->d_conv0, conv0.data(), sizeof(double) * ni,
                            cudaMemcpyHostToDevice, s));
  }
  PM_CUDA(cudaEventRecord(e1, s));
  PM_CUDA(cudaEventSynchronize(e1));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  int mx = 0;
  for (int i = 0; i < ni; ++i) {
    h->b_iters[i] = total[i];
    mx = std::max(mx, total[i]);
  }
  h->timers[5] = ms;
  h->timers[6] = mx;
  if (info) {
    info->iters = mx;
    info->refine = comp ? sweeps : 0;
    info->conv = 0.0;
    info->xkx = 0.0;
  }
  return PM_OK;
}

int solve_dev(Handle* h, int solver, int precond, const double* d_b, double* d_x, double tol,
              int maxit, pm_step_info* info) {
  if (!h->assembled) {
    h->err = "solve before assembly";
    return PM_E_STATE;
  }
  PM_TRY(build_precond(h, precond));
  if (h->ninst > 0) {
    if (solver != 1 || h->precision == PM_FP32_REFINE) {
      h->err = "a batch of meshes is solved by PCG (solver 1) in PM_FP64 or PM_FP32C_REFINE";
      return PM_E_ARG;
    }
    const bool comp = h->precision == PM_FP32C_REFINE;
    if (comp) PM_TRY(ensure_comp(h, h->stream));
    return krylov_batch(h, d_b, d_x, tol, maxit, comp, std::vector<int>(h->ninst, 1), info);
  }
  if (h->precision == PM_FP32_REFINE) {
    if (!h->assembled32) {
      if (!h->P.val32) {
        PM_CUDA(cudaMalloc(&h->P.val32, sizeof(float) * (size_t)h->P.nnz));
        if (h->pcgm_graph) {
          cudaGraphExecDestroy(h->pcgm_graph);
          h->pcgm_graph = nullptr;
        }
      }
      h->launches += 1;
      PM_CUDA(pm::to_f32(h->P.nnz, h->P.val, h->P.val32, h->stream));
      h->assembled32 = true;
    }
    return solve_mixed(h, solver, d_b, d_x, tol, maxit, info);
  }
  if (h->precision == PM_FP32C_REFINE) {
    PM_TRY(ensure_comp(h, h->stream));
    return krylov(h, solver, d_b, d_x, tol, maxit, true, info);
  }
  return krylov(h, solver, d_b, d_x, tol, maxit, false, info);
}

int alloc_state(Handle* h) {
  const size_t nn = (size_t)4 * h->nnode, n = h->neq;
  auto A = [&](double** p, size_t m) -> int {
    if (cudaMalloc((void**)p, sizeof(double) * std::max<size_t>(m, 1)) != cudaSuccess) {
      h->err = "cudaMalloc failed";
      return PM_E_NOMEM;
    }
    cudaMemset(*p, 0, sizeof(double) * std::max<size_t>(m, 1));
    return PM_OK;
  };
  pm::Dev& D = h->D;
  PM_TRY(A(&D.u, nn));
  PM_TRY(A(&D.u0, nn));
  PM_TRY(A(&D.f, nn));
  PM_TRY(A(&D.dp, h->nnode));
  PM_TRY(A(&D.poro, h->nnode));
  PM_TRY(A(&D.dporo, h->nnode));
  PM_CUDA(cudaMalloc(&D.vcnt, sizeof(int32_t) * std::max(h->nnode, 1)));
  PM_TRY(A(&D.b0, n));
  PM_TRY(A(&D.b, n));
  PM_TRY(A(&D.bst0, n));
  PM_TRY(A(&D.ad, n));
  PM_TRY(A(&D.m, n));
  PM_TRY(A(&D.bx, std::max(n, nn)));
  PM_TRY(A(&D.by, std::max(n, nn)));
  PM_TRY(A(&D.rr, n));
  PM_TRY(A(&D.dx, n));
  PM_TRY(A(&D.xs, n));
  pm::KrylovVecs& V = D.kv;
  for (double** p : {&V.x, &V.r, &V.z, &V.p, &V.q, &V.v, &V.v0, &V.w0, &V.w00, &V.z0})
    PM_TRY(A(p, n));
  PM_CUDA(cudaMalloc(&D.ks, sizeof(pm::KrylovScalars)));
  PM_CUDA(cudaMemset(D.ks, 0, sizeof(pm::KrylovScalars)));
  pm::KrylovVecs32& V32 = D.kv32;
  for (float** p : {&V32.p, &V32.q}) {
    if (cudaMalloc((void**)p, sizeof(float) * std::max<size_t>(n, 1)) != cudaSuccess) {
      h->err = "cudaMalloc failed";
      return PM_E_NOMEM;
    }
    cudaMemset(*p, 0, sizeof(float) * std::max<size_t>(n, 1));
  }
  if (cudaMalloc((void**)&V32.c, sizeof(float2) * std::max<size_t>(n, 1)) != cudaSuccess) {
    h->err = "cudaMalloc failed";
    return PM_E_NOMEM;
  }
  PM_TRY(A(&D.partial, 4 * (size_t)pm::kRedBlocks));
  PM_CUDA(cudaMalloc(&D.counter, sizeof(unsigned) * 4));
  PM_CUDA(cudaMemset(D.counter, 0, sizeof(unsigned) * 4));
  PM_TRY(A(&D.norms, 4));
  PM_CUDA(cudaMalloc(&D.err, sizeof(int)));
  PM_CUDA(cudaMemset(D.err, 0, sizeof(int)));
  return PM_OK;
}

void free_all(Handle* h) {
  pm::Dev& D = h->D;
  pm::Panels& P = h->P;
  void* ptrs[] = {D.ix, D.eq, D.x, D.mat, D.slot, D.color_elems, D.eload, D.eloadp, D.nload,
                  D.load, D.fload, D.dofkind, D.fnno, D.u, D.u0, D.dp, D.poro, D.dporo, D.vcnt, D.gm_basis, D.gm_scal,
                  D.gm_y, D.f, D.b0, D.b, D.bst0,
                  D.ad, D.m, D.bx, D.by, D.rr, D.dx, D.xs, D.kv.x, D.kv.r, D.kv.z, D.kv.p, D.kv.q,
                  D.kv.v, D.kv.v0, D.kv.w0, D.kv.w00, D.kv.z0, D.ks, D.partial, D.counter,
                  D.norms, D.err, P.eq0, P.d, P.W, P.low, P.val_off, P.col_off, P.cols, P.val,
                  P.val32, P.valh, P.vall, P.rec, P.rec_off, P.node_val_off, P.node_W,
                  P.order, P.cs_desc, P.cs_batch_slot, P.cs_batch_off, P.cs_batch_bytes,
                  P.cs_cta_batch, P.fault, P.meta};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  for (void* p : {(void*)D.kv32.p, (void*)D.kv32.q, (void*)D.kv32.c})
    if (p) cudaFree(p);
  if (h->pcg_graph) cudaGraphExecDestroy(h->pcg_graph);
  if (h->pcg_loop) cudaGraphExecDestroy(h->pcg_loop);
  if (h->D.trips) cudaFree(h->D.trips);
  if (h->pcgm_graph) cudaGraphExecDestroy(h->pcgm_graph);
  if (h->minres_graph) cudaGraphExecDestroy(h->minres_graph);
  if (h->pcgc_graph) cudaGraphExecDestroy(h->pcgc_graph);
  if (h->sqmr_graph) cudaGraphExecDestroy(h->sqmr_graph);
  if (h->sqmrc_graph) cudaGraphExecDestroy(h->sqmrc_graph);
  if (h->bpcg_graph) cudaGraphExecDestroy(h->bpcg_graph);
  if (h->bpcgc_graph) cudaGraphExecDestroy(h->bpcgc_graph);
  for (void* p : {(void*)h->B.eq_ptr, (void*)h->B.blk_ptr, (void*)h->B.blk_inst, (void*)h->B.bs,
                  (void*)h->B.done, (void*)h->B.nactive, (void*)h->B.partial,
                  (void*)h->B.counter, (void*)h->P.node_inst, (void*)h->d_insweep,
                  (void*)h->d_conv0, (void*)h->d_bnorms})
    if (p) cudaFree(p);
  if (h->minresc_graph) cudaGraphExecDestroy(h->minresc_graph);
  if (h->bstep_exec) cudaGraphExecDestroy(h->bstep_exec);
  const pm::BatchStepArrays& A = h->bsa;
  for (void* p : {(void*)h->d_bctl, (void*)A.active, (void*)A.total, (void*)A.iters,
                  (void*)A.nlit, (void*)A.res0, (void*)A.resu0, (void*)A.resp0, (void*)A.nr,
                  (void*)A.rn2})
    if (p) cudaFree(p);
  for (auto& e : h->ev)
    if (e) cudaEventDestroy(e);
  if (h->stream) cudaStreamDestroy(h->stream);
}

pm::MatConst mat_const(const double* e, double gmod) {
  pm::MatConst m;
  m.pm_d = e[5] * 1.0e-06;
  m.fluid_d = e[6] * 1.0e-06;
  const double ym = e[0], ps = e[1];
  m.perm = e[2] / (m.fluid_d * gmod);
  m.imod_biot = 1.0 / e[3];
  m.coef_biot = e[4];
  const double a1 = 1.0 - ps, a2 = 1.0 - 2.0 * ps, a3 = 1.0 + ps;
  m.a = (ym * a1) / (a3 * a2);
  m.b = ps / a1;
  m.c = 0.5 * (a2 / a1);
  return m;
}

int upload_materials(Handle* h) {
  h->h_mat.resize(h->numat);
  for (int k = 0; k < h->numat; ++k) h->h_mat[k] = mat_const(&h->h_e[(size_t)PM_PROP * k], h->gravity_mod);
  if (!h->D.mat) PM_CUDA(cudaMalloc(&h->D.mat, sizeof(pm::MatConst) * h->numat));
  PM_CUDA(cudaMemcpy(h->D.mat, h->h_mat.data(), sizeof(pm::MatConst) * h->numat,
                     cudaMemcpyHostToDevice));
  h->assembled = h->assembled32 = h->assembledC = false;
  return PM_OK;
}

template <typename T>
int set_dev_array(Handle* h, T** dst, const T* src, size_t n) {
  if (!src) {
    if (*dst) {
      cudaFree(*dst);
      *dst = nullptr;
    }
    return PM_OK;
  }
  if (!*dst) PM_CUDA(cudaMalloc((void**)dst, sizeof(T) * n));
  PM_CUDA(cudaMemcpy(*dst, src, sizeof(T) * n, cudaMemcpyHostToDevice));
  return PM_OK;
}

// One step of every instance of a batch: the 'solv' macro of pm_step with
// each instance's own nonlinear test (cal_residuo_pm per instance: its own
// reference norms, its own decision); instances that have met their test
// take no further solve (their correction is zero), the others solve
// together in one batched PCG.
// porosity_form (Pform.f:969-1175) on the step's increments held in D.u
// (Main.f:1086 runs it after the nonlinear loop, before update_res_v2)
int porosity_pass(Handle* h, cudaStream_t s) {
  pm::Dev& D = h->D;
  PM_CUDA(cudaMemsetAsync(D.dporo, 0, sizeof(double) * h->nnode, s));
  for (int c = 0; c < h->numcolors; ++c)
    PM_CUDA(pm::launch_poro7(elem_launch(h, c), h->hexa, D.u, D.dporo, s));
  k_poro_finish<<<grid_for(h->nnode), 256, 0, s>>>(h->nnode, D.fnno, D.vcnt, D.dporo, D.poro);
  PM_CUDA(cudaGetLastError());
  h->launches += h->numcolors + 1;
  return PM_OK;
}

// ---- a batch time step as one CUDA graph ---------------------------------------
// Launches captured from the handle's stream into graph g after node dep,
// and conditional nodes added between the captures.
struct GraphCap {
  cudaStream_t s;
  cudaGraph_t g;
  bool ok;
  cudaGraphNode_t dep = nullptr;  // the node the next capture or node follows

  template <typename Fn>
  void seg(Fn fn) {
    if (!ok) return;
    ok = cudaStreamBeginCaptureToGraph(s, g, dep ? &dep : nullptr, nullptr, dep ? 1 : 0,
                                       cudaStreamCaptureModeRelaxed) == cudaSuccess;
    if (!ok) return;
    const int rc = fn();
    cudaStreamCaptureStatus st{};
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    const bool info =
        cudaStreamGetCaptureInfo(s, &st, nullptr, nullptr, &deps, nullptr, &nd) == cudaSuccess;
    const cudaGraphNode_t leaf = (info && nd == 1) ? deps[0] : nullptr;
    cudaGraph_t out = nullptr;
    const bool ended = cudaStreamEndCapture(s, &out) == cudaSuccess;
    ok = rc == PM_OK && leaf != nullptr && ended;
    if (ok) dep = leaf;
  }
  // a conditional node after dep; returns its body graph
  cudaGraph_t cond(cudaGraphConditionalHandle c, cudaGraphConditionalNodeType type) {
    if (!ok) return nullptr;
    cudaGraphNodeParams np{};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = c;
    np.conditional.type = type;
    np.conditional.size = 1;
    cudaGraphNode_t node{};
    ok = cudaGraphAddNode(&node, g, dep ? &dep : nullptr, nullptr, dep ? 1 : 0, &np) ==
         cudaSuccess;
    if (!ok) return nullptr;
    dep = node;
    return np.conditional.phGraph_out[0];
  }
  cudaGraphConditionalHandle handle() {
    cudaGraphConditionalHandle c{};
    if (ok) ok = cudaGraphConditionalHandleCreate(&c, g, 0, 0) == cudaSuccess;
    return c;
  }
};

int kernel_nodes(cudaGraph_t g) {
  if (!g) return 0;
  size_t n = 0;
  if (cudaGraphGetNodes(g, nullptr, &n) != cudaSuccess) return 0;
  std::vector<cudaGraphNode_t> v(n);
  if (n && cudaGraphGetNodes(g, v.data(), &n) != cudaSuccess) return 0;
  int k = 0;
  for (cudaGraphNode_t x : v) {
    cudaGraphNodeType t{};
    if (cudaGraphNodeGetType(x, &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++k;
  }
  return k;
}

// The batch step of step_batch as one CUDA graph, captured every step (the
// step's t, dt and settings are kernel arguments) and launched once:
//   load, isw 4 and predictor passes; b = b0 - K u (assembly or residual);
//   per-instance stop test;
//   WHILE an instance is left: preconditioner;
//     WHILE a refinement sweep is wanted: bpcg_init;
//       WHILE an instance is iterating: kGraphIters PCG iterations;
//       sweep bookkeeping, x += dx, [compensated: FP64 residual, next sweep];
//     du += x; b = b0 - K u; stop test;
//   IF no error: porosity and state updates.
// The loop conditions are set by the control kernels of pm_batch.cu from
// device-side state (BatchCtl, BatchStepArrays) that the host reads once,
// after the graph.  *ran is false when the graph was not built (the step's
// settings need the host loop, or the driver refused a part): step_batch's
// host loop then runs the step.
int step_batch_graph(Handle* h, int maxnlit, double tol, int stop_crit, int precond,
                     double solvtol, int maxit, int reassemble, pm_step_info* info, bool* ran) {
  *ran = false;
  const bool comp = h->precision == PM_FP32C_REFINE;
  if (h->bstep_failed || std::getenv("PM_BATCH_HOST_STEP") || !h->d_bctl ||
      (stop_crit != 1 && stop_crit != 2) || (precond != 2 && precond != 5) ||
      (comp && (!h->P.valh || h->shape == 0)))
    return PM_OK;
  cudaStream_t s = h->stream;
  pm::Dev& D = h->D;
  const int ni = h->ninst, n = h->neq;
  // host bookkeeping that the capture advances; put back if the graph is not run
  const int istep0 = h->istep;
  const double t0 = h->t, adt0 = h->assembled_dt;
  const bool asm0 = h->assembled, asm32 = h->assembled32, asmC = h->assembledC;
  const int64_t launches0 = h->launches;
  h->istep += 1;
  h->t = h->t + h->dt;
  const bool need_K = reassemble || !h->assembled || h->assembled_dt != h->dt;
  const bool split = comp && (need_K || !h->assembledC);
  pm::BatchCtl* c = h->d_bctl;
  const pm::BatchStepArrays A = h->bsa;
  const pm::BatchView& B = h->B;
  pm::KrylovVecs& V = D.kv;
  float2* pair = D.kv32.c;
  const pm::PanelView PB = h->P.bview(), P = h->P.view();
  const pm::CompVals C = h->P.comp(h->shape);
  const int nb = grid_for(h->nnode);

  cudaGraph_t g = nullptr;
  GraphCap top{s, nullptr, cudaGraphCreate(&g, 0) == cudaSuccess};
  top.g = g;
  const cudaGraphConditionalHandle c_nl = top.handle(), c_ok = top.handle();
  top.seg([&]() -> int {
    PM_CUDA(pm::bs_begin(c, A, ni, s));
    k_pload<<<nb, 256, 0, s>>>(h->nnode, D.eq, D.fnno, D.nload, D.f, D.u, D.b0, D.load,
                               D.fload, h->maxt, D.x, h->t, h->dt, h->gravity_mod);
    PM_CUDA(cudaGetLastError());
    PM_TRY(rhs4(h, D.u, D.b0));
    if (h->fstress0) PM_CUDA(pm::axpy_into(n, D.b0, D.bst0, 1.0, s));
    k_predict<<<nb, 256, 0, s>>>(h->nnode, D.fnno, D.u, D.u0);
    PM_CUDA(cudaGetLastError());
    PM_CUDA(cudaMemcpyAsync(D.b, D.b0, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
    if (need_K) PM_TRY(assemble_K(h, D.u, D.b));  // b -= K u in the same launch
    else PM_TRY(residual(h, D.u, D.b));
    if (split) PM_CUDA(pm::split_values(h->P.nnz, h->P.val, h->P.valh, h->P.vall, s));
    PM_CUDA(pm::bresnorms(B, D.b, D.dofkind, A.nr, s));
    PM_CUDA(pm::bs_stop(c, A, ni, stop_crit, tol, c_nl, s));
    return PM_OK;
  });
  const cudaGraph_t g_nl = top.cond(c_nl, cudaGraphCondTypeWhile);
  GraphCap nl{s, g_nl, top.ok};
  const cudaGraphConditionalHandle c_sw = nl.handle();
  nl.seg([&]() -> int {
    PM_CUDA(pm::panel_diag(P, h->P.val, nullptr, D.ad, s));
    PM_CUDA(pm::precond(n, D.ad, D.m, precond == 5, &c->zdiag, s));
    PM_CUDA(cudaMemsetAsync(D.xs, 0, sizeof(double) * n, s));
    PM_CUDA(pm::bs_solve_start(c, A, ni, c_sw, s));
    return PM_OK;
  });
  const cudaGraph_t g_sw = nl.cond(c_sw, cudaGraphCondTypeWhile);
  GraphCap sw{s, g_sw, nl.ok};
  const cudaGraphConditionalHandle c_pcg = sw.handle();
  sw.seg([&]() -> int {
    PM_CUDA(cudaMemsetAsync(B.nactive, 0, sizeof(int), s));
    PM_CUDA(pm::bpcg_init_sweep(B, D.b, D.rr, D.m, V, comp ? pair : nullptr, solvtol, A.conv0,
                                A.insweep, maxit, &c->sweeps, s));
    PM_CUDA(pm::bs_loop_start(B, c, c_pcg, s));
    return PM_OK;
  });
  const cudaGraph_t g_pcg = sw.cond(c_pcg, cudaGraphCondTypeWhile);
  GraphCap pcg{s, g_pcg, sw.ok};
  pcg.seg([&]() -> int {
    for (int k = 0; k < kGraphIters; ++k)
      PM_CUDA(pm::bpcg_iteration(PB, h->P.val, comp ? &C : nullptr, B, D.m, V, pair, s));
    PM_CUDA(pm::bs_loop_next(B, c, maxit, kGraphIters, c_pcg, s));
    return PM_OK;
  });
  sw.ok = sw.ok && pcg.ok;
  sw.seg([&]() -> int {
    PM_CUDA(pm::bs_sweep_end(c, B, A, ni, comp, c_sw, s));
    PM_CUDA(pm::baxpy(B, D.xs, V.x, A.insweep, s));
    if (comp) {
      PM_CUDA(pm::spmv(P, h->P.val, D.xs, D.dx, 0, nullptr, nullptr, nullptr, s));
      PM_CUDA(pm::btrue_residual(B, D.b, D.dx, D.m, D.rr, A.rn2, s));
      PM_CUDA(pm::bs_sweep_next(c, A, ni, kMaxBatchSweeps, c_sw, s));
    }
    return PM_OK;
  });
  nl.ok = nl.ok && sw.ok;
  nl.seg([&]() -> int {
    PM_CUDA(pm::bs_solve_end(c, A, ni, comp, s));
    k_delta_update<<<nb, 256, 0, s>>>(h->nnode, D.eq, D.fnno, D.u, D.xs, &c->err);
    PM_CUDA(cudaGetLastError());
    PM_CUDA(pm::bs_nl_next(c, maxnlit, s));
    PM_CUDA(cudaMemcpyAsync(D.b, D.b0, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
    PM_TRY(residual(h, D.u, D.b));
    PM_CUDA(pm::bresnorms(B, D.b, D.dofkind, A.nr, s));
    PM_CUDA(pm::bs_stop(c, A, ni, stop_crit, tol, c_nl, s));
    return PM_OK;
  });
  top.ok = top.ok && nl.ok;
  top.seg([&]() -> int {
    PM_CUDA(pm::bs_finish(c, D.err, c_ok, s));
    return PM_OK;
  });
  const cudaGraph_t g_ok = top.cond(c_ok, cudaGraphCondTypeIf);
  GraphCap fin{s, g_ok, top.ok};
  fin.seg([&]() -> int {
    PM_TRY(porosity_pass(h, s));
    k_update_res<<<nb, 256, 0, s>>>(h->nnode, D.fnno, D.u, D.u0, D.dp);
    PM_CUDA(cudaGetLastError());
    return PM_OK;
  });
  bool ok = top.ok && fin.ok;
  const int kn_top = ok ? kernel_nodes(g) : 0, kn_nl = ok ? kernel_nodes(g_nl) : 0;
  const int kn_sw = ok ? kernel_nodes(g_sw) : 0, kn_pcg = ok ? kernel_nodes(g_pcg) : 0;
  const int kn_ok = ok ? kernel_nodes(g_ok) : 0;
  if (ok) {
    if (h->bstep_exec) cudaGraphExecDestroy(h->bstep_exec);
    h->bstep_exec = nullptr;
    ok = cudaGraphInstantiate(&h->bstep_exec, g, 0) == cudaSuccess;
  }
  if (g) cudaGraphDestroy(g);
  h->launches = launches0;
  if (!ok) {
    cudaGetLastError();  // the refusal is not this step's error
    h->bstep_failed = true;
    h->istep = istep0;
    h->t = t0;
    h->assembled = asm0;
    h->assembled32 = asm32;
    h->assembledC = asmC;
    h->assembled_dt = adt0;
    if (h->debug) fprintf(stderr, "batch step graph unavailable: host loop\n");
    return PM_OK;
  }
  *ran = true;
  if (split) h->assembledC = true;
  PM_CUDA(cudaEventRecord(h->ev[0], s));
  PM_CUDA(cudaGraphLaunch(h->bstep_exec, s));
  PM_CUDA(cudaEventRecord(h->ev[1], s));
  pm::BatchCtl ctl{};
  int elem_err = 0;
  std::vector<int> iters(ni), nlit(ni);
  PM_CUDA(cudaMemcpyAsync(&ctl, c, sizeof(ctl), cudaMemcpyDeviceToHost, s));
  PM_CUDA(cudaMemcpyAsync(&elem_err, D.err, sizeof(int), cudaMemcpyDeviceToHost, s));
  PM_CUDA(cudaMemcpyAsync(iters.data(), A.iters, sizeof(int) * ni, cudaMemcpyDeviceToHost, s));
  PM_CUDA(cudaMemcpyAsync(nlit.data(), A.nlit, sizeof(int) * ni, cudaMemcpyDeviceToHost, s));
  PM_CUDA(cudaStreamSynchronize(s));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, h->ev[0], h->ev[1]);
  h->launches += kn_top + (int64_t)kn_nl * ctl.runs_nl + (int64_t)kn_sw * ctl.runs_sweep +
                 (int64_t)kn_pcg * ctl.runs_pcg + (ctl.ok ? kn_ok : 0);
  h->timers[0] = h->timers[1] = h->timers[2] = 0.0;
  h->timers[3] = ms;
  h->timers[7] = (double)(h->launches - launches0);
  if (elem_err) {
    PM_CUDA(cudaMemsetAsync(D.err, 0, sizeof(int), s));
    h->err = "element Jacobian determinant <= 1e-14";
    return PM_E_DET;
  }
  if (ctl.err == PM_E_ZERO_DIAG) {
    h->err = "zero diagonal coefficient";
    return PM_E_ZERO_DIAG;
  }
  if (ctl.err == PM_E_NOCONV) {
    if (ctl.err_inst >= 0) {
      h->err = "batch PCG, instance " + std::to_string(ctl.err_inst) +
               (ctl.err_flag == 3 ? ": breakdown (non-finite recurrence)"
                                  : ": no convergence reached after " +
                                        std::to_string(ctl.err_iters) + " iterations");
      if (info) info->iters = ctl.err_iters;
    } else if (ctl.err_inst == -1) {
      h->err = "batch PCG: iteration count past maxit with instances still active";
    } else {
      h->err = "batch refinement: FP64 residual above target after " +
               std::to_string(kMaxBatchSweeps) + " sweeps";
    }
    return PM_E_NOCONV;
  }
  if (ctl.err == PM_E_NLNOCONV) {
    h->err = "nonlinear iteration: no convergence after " + std::to_string(ctl.it) +
             " iterations (batch)";
    return PM_E_NLNOCONV;
  }
  h->b_iters = iters;
  h->b_nlit = nlit;
  if (info) {
    pm_step_info loc{};
    loc.res_u = ctl.res_max;
    loc.iters = ctl.iters_max;
    loc.refine = ctl.refine;
    loc.nlit = ctl.it;
    *info = loc;
  }
  return PM_OK;
}

int step_batch(Handle* h, int maxnlit, double tol, int stop_crit, int solver, int precond,
               double solvtol, int maxit, int reassemble, pm_step_info* info) {
  if (solver != 1 || h->precision == PM_FP32_REFINE) {
    h->err = "a batch of meshes is solved by PCG (solver 1) in PM_FP64 or PM_FP32C_REFINE";
    return PM_E_ARG;
  }
  {
    bool ran = false;
    const int rc = step_batch_graph(h, maxnlit, tol, stop_crit, precond, solvtol, maxit,
                                    reassemble, info, &ran);
    if (ran || rc != PM_OK) return rc;
  }
  cudaStream_t s = h->stream;
  pm::Dev& D = h->D;
  const int ni = h->ninst;
  const int64_t launches0 = h->launches;
  cudaEvent_t ev[4];
  for (auto& e : ev) PM_CUDA(cudaEventCreate(&e));
  struct EvGuard {
    cudaEvent_t* e;
    ~EvGuard() {
      for (int i = 0; i < 4; ++i) cudaEventDestroy(e[i]);
    }
  } guard{ev};
  h->istep += 1;
  h->t = h->t + h->dt;
  PM_CUDA(cudaEventRecord(ev[0], s));
  h->launches += 2 + (h->fstress0 ? 1 : 0);
  k_pload<<<grid_for(h->nnode), 256, 0, s>>>(h->nnode, D.eq, D.fnno, D.nload, D.f, D.u, D.b0,
                                              D.load, D.fload, h->maxt, D.x, h->t, h->dt,
                                              h->gravity_mod);
  PM_CUDA(cudaGetLastError());
  PM_TRY(rhs4(h, D.u, D.b0));
  if (h->fstress0) PM_CUDA(pm::axpy_into(h->neq, D.b0, D.bst0, 1.0, s));
  k_predict<<<grid_for(h->nnode), 256, 0, s>>>(h->nnode, D.fnno, D.u, D.u0);
  PM_CUDA(cudaGetLastError());
  PM_CUDA(cudaEventRecord(ev[1], s));
  std::vector<int> active(ni, 1);
  std::vector<double> nr(2 * (size_t)ni);
  h->b_res0.resize(ni);
  h->b_resu0.resize(ni);
  h->b_resp0.resize(ni);
  h->b_nlit.assign(ni, 0);
  std::fill(h->b_iters.begin(), h->b_iters.end(), 0);
  std::vector<int> iters(ni, 0);
  bool lhs = true;
  int it = 1;
  pm_step_info loc{};
  double t_asm = 0, t_res = 0, t_sol = 0;
  for (;;) {
    PM_CUDA(cudaMemcpyAsync(D.b, D.b0, sizeof(double) * h->neq, cudaMemcpyDeviceToDevice, s));
    PM_CUDA(cudaEventRecord(ev[2], s));
    const bool need_K = lhs && (reassemble || !h->assembled || h->assembled_dt != h->dt);
    if (need_K) {
      PM_TRY(assemble_K(h, D.u, D.b));  // b -= K u in the same launch
      h->assembled32 = h->assembledC = false;
    } else {
      PM_TRY(residual(h, D.u, D.b));
    }
    PM_CUDA(cudaEventRecord(ev[3], s));
    PM_TRY(check_elem_err(h));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ev[2], ev[3]);
    t_asm += ms;
    if (stop_crit == 1 || stop_crit == 2) {
      h->launches += 1;
      PM_CUDA(pm::bresnorms(h->B, D.b, D.dofkind, h->d_bnorms, s));
      PM_CUDA(cudaMemcpyAsync(nr.data(), h->d_bnorms, sizeof(double) * 2 * ni,
                              cudaMemcpyDeviceToHost, s));
      PM_CUDA(cudaStreamSynchronize(s));
      int left = 0;
      for (int i = 0; i < ni; ++i) {
        if (!active[i]) continue;
        bool done = false;
        if (stop_crit == 1) {  // cal_residuo_pm (Residuo.f:39-276), per instance
          const double res = std::sqrt(nr[2 * i] + nr[2 * i + 1]);
          if (it == 1) h->b_res0[i] = res;
          else if (it == 2) h->b_res0[i] = std::max(h->b_res0[i], res);
          loc.res_u = std::max(loc.res_u, res);
          done = h->b_res0[i] > 0.0 ? res / h->b_res0[i] < tol : true;
        } else {
          const double gresu = std::sqrt(nr[2 * i]), gresp = std::sqrt(nr[2 * i + 1]);
          if (it == 1) {
            h->b_resu0[i] = gresu;
            h->b_resp0[i] = gresp;
          } else if (it == 2) {
            h->b_resu0[i] = std::max(h->b_resu0[i], gresu);
            h->b_resp0[i] = std::max(h->b_resp0[i], gresu);  // as the reference
          }
          int istop = 0;
          if (gresu / h->b_resu0[i] < tol) istop += 1;
          if (gresp / h->b_resp0[i] < tol) istop += 1;
          done = istop == 2;
        }
        if (done) {
          active[i] = 0;
          h->b_nlit[i] = it;
        } else {
          ++left;
        }
      }
      if (left == 0) break;
    }
    PM_CUDA(cudaEventRecord(ev[2], s));
    PM_TRY(build_precond(h, precond));
    const bool comp = h->precision == PM_FP32C_REFINE;
    if (comp) PM_TRY(ensure_comp(h, s));
    pm_step_info si{};
    PM_TRY(krylov_batch(h, D.b, D.xs, solvtol, maxit, comp, active, &si));
    for (int i = 0; i < ni; ++i)
      if (active[i]) iters[i] += h->b_iters[i];
    loc.iters = std::max(loc.iters, si.iters);
    loc.refine = si.refine;
    h->launches += 1;
    k_delta_update<<<grid_for(h->nnode), 256, 0, s>>>(h->nnode, D.eq, D.fnno, D.u, D.xs);
    PM_CUDA(cudaGetLastError());
    PM_CUDA(cudaEventRecord(ev[3], s));
    PM_CUDA(cudaEventSynchronize(ev[3]));
    cudaEventElapsedTime(&ms, ev[2], ev[3]);
    t_sol += ms;
    if (it >= maxnlit) {
      h->err = "nonlinear iteration: no convergence after " + std::to_string(it) +
               " iterations (batch)";
      return PM_E_NLNOCONV;
    }
    ++it;
    lhs = false;
  }
  h->b_iters = iters;
  loc.nlit = it;
  PM_TRY(porosity_pass(h, s));
  h->launches += 1;
  k_update_res<<<grid_for(h->nnode), 256, 0, s>>>(h->nnode, D.fnno, D.u, D.u0, D.dp);
  PM_CUDA(cudaGetLastError());
  PM_CUDA(cudaStreamSynchronize(s));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, ev[0], ev[1]);
  h->timers[0] = ms;
  h->timers[1] = t_asm;
  h->timers[2] = 0.0;
  h->timers[3] = t_sol;
  h->timers[7] = (double)(h->launches - launches0);
  if (info) *info = loc;
  return PM_OK;
}

}  // namespace

extern "C" {

const char* pm_status_string(int s) {
  switch (s) {
    case PM_OK: return "ok";
    case PM_E_ARG: return "invalid argument";
    case PM_E_DET: return "element Jacobian determinant <= 1e-14";
    case PM_E_ZERO_DIAG: return "zero diagonal coefficient";
    case PM_E_NOCONV: return "Krylov solver did not converge";
    case PM_E_NLNOCONV: return "nonlinear iteration did not converge";
    case PM_E_ELTYPE: return "unsupported element type";
    case PM_E_CUDA: return "CUDA error";
    case PM_E_NOMEM: return "device allocation failed";
    case PM_E_STATE: return "call out of order";
    case PM_E_TOO_LARGE: return "problem larger than the fixed scratch of pm_pcg_csrd_noalloc";
    default: return "unknown status";
  }
}

const char* pm_last_error(pm_handle hh) {
  Handle* h = reinterpret_cast<Handle*>(hh);
  return h ? h->err.c_str() : "null handle";
}

static int mesh_create(int nnode, int nnodev, int numel, int nen, int nenv, int ndm, int ndf,
                       const int32_t* ix, const int32_t* id, const int32_t* fnno,
                       const double* x, int numat, const int32_t* ie, const double* e,
                       const int32_t* num, int ninst, const int32_t* inst_node_ptr,
                       pm_handle* out) {
  if (!out || !ix || !id || !fnno || !x || !ie || !e || nnode <= 0 || numel <= 0 ||
      numat <= 0 || ndm != 3 || ndf != 4 ||
      !((nen == 20 && nenv == 8) || (nen == 10 && nenv == 4)))
    return PM_E_ARG;
  *out = nullptr;
  for (int k = 0; k < numat; ++k)
    if (!((nen == 20 && ie[k] == 17) || (nen == 10 && ie[k] == 15))) return PM_E_ELTYPE;
  for (int el = 0; el < numel; ++el) {
    const int ma = ix[(size_t)(nen + 1) * el + nen];
    if (ma < 1 || ma > numat) return PM_E_ARG;
  }
  if (ninst > 0) {
    // node ranges 0 = p[0] <= ... <= p[ninst] = nnode; every element inside one range
    if (!inst_node_ptr || num || inst_node_ptr[0] != 0 || inst_node_ptr[ninst] != nnode)
      return PM_E_ARG;
    for (int i = 0; i < ninst; ++i)
      if (inst_node_ptr[i + 1] < inst_node_ptr[i]) return PM_E_ARG;
    const int32_t* pe = inst_node_ptr + ninst + 1;
    for (int el = 0; el < numel; ++el) {
      const int32_t* nd = ix + (size_t)(nen + 1) * el;
      const int i0 = (int)(std::upper_bound(inst_node_ptr, pe, nd[0] - 1) - inst_node_ptr) - 1;
      for (int a = 0; a < nen; ++a)
        if (nd[a] - 1 < inst_node_ptr[i0] || nd[a] - 1 >= inst_node_ptr[i0 + 1]) return PM_E_ARG;
    }
  }
  Handle* h = new (std::nothrow) Handle();
  if (!h) return PM_E_NOMEM;
  h->nnode = nnode;
  h->nnodev = nnodev;
  h->numel = numel;
  h->nen = nen;
  h->nenv = nenv;
  h->numat = numat;
  h->hexa = (nen == 20);
  h->h_e.assign(e, e + (size_t)PM_PROP * numat);
  h->h_ie.assign(ie, ie + numat);
  if (ninst > 0) {
    h->ninst = ninst;
    h->h_inst_node.assign(inst_node_ptr, inst_node_ptr + ninst + 1);
  }
  int st = PM_OK;
  auto fail = [&](int s) {
    free_all(h);
    delete h;
    return s;
  };
  if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess)
    return fail(PM_E_CUDA);
  if (pm::ensure_shape_tables() != cudaSuccess) return fail(PM_E_CUDA);
  for (auto& ev : h->ev)
    if (cudaEventCreate(&ev) != cudaSuccess) return fail(PM_E_CUDA);
  if ((st = pm::build_structure(h, ix, id, fnno, x, num)) != PM_OK) return fail(st);
  if ((st = alloc_state(h)) != PM_OK) return fail(st);
  if ((st = upload_materials(h)) != PM_OK) return fail(st);
  {
    // initial_porosity (Pform.f:1343-1432): e(8) averaged over the elements
    // sharing a vertex; the counts are tform_pm's and porosity_form's ic
    std::vector<int32_t> ic(nnode, 0);
    std::vector<double> poro(nnode, 0.0);
    for (int el = 0; el < numel; ++el) {
      const int32_t* nd = ix + (size_t)(nen + 1) * el;
      const double p0 = e[(size_t)PM_PROP * (nd[nen] - 1) + 7];
      for (int a = 0; a < nenv; ++a)
        if (nd[a] > 0) {
          ic[nd[a] - 1] += 1;
          poro[nd[a] - 1] += p0;
        }
    }
    for (int i = 0; i < nnode; ++i)
      if (fnno[i] == 1 && ic[i] > 0) poro[i] = poro[i] / ic[i];
    if (cudaMemcpy(h->D.vcnt, ic.data(), sizeof(int32_t) * nnode, cudaMemcpyHostToDevice) !=
            cudaSuccess ||
        cudaMemcpy(h->D.poro, poro.data(), sizeof(double) * nnode, cudaMemcpyHostToDevice) !=
            cudaSuccess)
      return fail(PM_E_CUDA);
  }
  if (ninst > 0 && (st = batch_setup(h)) != PM_OK) return fail(st);
  h->debug = getenv("PM_DEBUG") != nullptr;
  *out = reinterpret_cast<pm_handle>(h);
  return PM_OK;
}

int pm_mesh_create(int nnode, int nnodev, int numel, int nen, int nenv, int ndm, int ndf,
                   const int32_t* ix, const int32_t* id, const int32_t* fnno, const double* x,
                   int numat, const int32_t* ie, const double* e, const int32_t* num,
                   pm_handle* out) {
  return mesh_create(nnode, nnodev, numel, nen, nenv, ndm, ndf, ix, id, fnno, x, numat, ie, e,
                     num, 0, nullptr, out);
}

int pm_batch_create(int nnode, int nnodev, int numel, int nen, int nenv, int ndm, int ndf,
                    const int32_t* ix, const int32_t* id, const int32_t* fnno, const double* x,
                    int numat, const int32_t* ie, const double* e, int ninst,
                    const int32_t* inst_node_ptr, pm_handle* out) {
  if (ninst < 1) return PM_E_ARG;
  return mesh_create(nnode, nnodev, numel, nen, nenv, ndm, ndf, ix, id, fnno, x, numat, ie, e,
                     nullptr, ninst, inst_node_ptr, out);
}

int pm_get_batch_iters(pm_handle hh, int* iters, int* nlit, int n) {
  Handle* h = reinterpret_cast<Handle*>(hh);
  if (!h || h->ninst == 0 || n < h->ninst) return PM_E_ARG;
  for (int i = 0; i < h->ninst; ++i) {
    if (iters) iters[i] = h->b_iters[i];
    if (nlit) nlit[i] = h->b_nlit[i];
  }
  return PM_OK;
}

void pm_destroy(pm_handle hh) {
  Handle* h = reinterpret_cast<Handle*>(hh);
  if (!h) return;
  if (h->stream) cudaStreamSynchronize(h->stream);
  free_all(h);
  delete h;
}

int pm_set_loads(pm_handle hh, const int32_t* eload, const int32_t* eloadp,
                 const int32_t* nload, const double* f, int nloads, int maxt,
                 const int32_t* load, const double* fload) {
  Handle* h = reinterpret_cast<Handle*>(hh);
  if (!h || nloads < 0 || (nloads > 0 && (!load || !fload || maxt < 1))) return PM_E_ARG;
  PM_TRY(set_dev_array(h, &h->D.eload, eload, (size_t)7 * h->numel));
  PM_TRY(set_dev_array(h, &h->D.eloadp, eloadp, (size_t)7 * h->numel));
  PM_TRY(set_dev_array(h, &h->D.nload, nload, (size_t)4 * h->nnode));
  if (f) PM_CUDA(cudaMemcpy(h->D.f, f, sizeof(double) * 4 * h->nnode, cudaMemcpyHostToDevice));
  else PM_CUDA(cudaMemset(h->D.f, 0, sizeof(double) * 4 * h->nnode));
  h->nloads = nloads;
  h->maxt = maxt > 0 ? maxt : 1;
  PM_TRY(set_dev_array(h, &h->D.load, nloads ? load : nullptr, (size_t)3 * nloads));
  PM_TRY(set_dev_array(h, &h->D.fload, nloads ? fload : nullptr,
                       (size_t)h->maxt * PM_NFLOAD * nloads));
  return PM_OK;
}

int pm_set_env(pm_handle hh, const double* gravity, double dt, double t, int istep) {
  Handle* h = reinterpret_cast<Handle*>(hh);
  if (!h || !(dt > 0.0)) return PM_E_ARG;
  if (gravity) {
    for (int i = 0; i < 3; ++i) h->gravity[i] = gravity[i];
    h->gravity_mod = std::sqrt(gravity[0] * gravity[0] + gravity[1] * gravity[1] +
                               gravity[2] * gravity[2]);
    PM_TRY(upload_materials(h));
  }
  if (dt != h->dt) h->assembled = h->assembled32 = h->assembledC = false;
  h->dt = dt;
  h->t = t;
  h->istep = istep;
  return PM_OK;
}

int pm_set_state(pm_handle hh, const double* u, const double* u0, const double* dp) {
  Handle* h = reinterpret_cast<Handle*>(hh);
  if (!h) return PM_E_ARG;
  const size_t nn = (size_t)4 * h->nnode;
  if (u) PM_CUDA(cudaMemcpy(h->D.u, u, sizeof(double) * nn, cudaMemcpyHostToDevice));
  if (u0) PM_CUDA(cudaMemcpy(h->D.u0, u0, sizeof(double) * nn, cudaMemcpyHostToDevice));
  if (dp) PM_CUDA(cudaMemcpy(h->D.dp, dp, sizeof(double) * h->nnode, cudaMemcpyHostToDevice));
  return PM_OK;
}

int pm_get_state(pm_handle hh, double* u, double* u0, double* dp) {
  Handle* h = reinterpret_cast<Handle*>(hh);
  if (!h) return PM_E_ARG;
  PM_CUDA(cudaStreamSynchronize(h->stream));
  const size_t nn = (size_t)4 * h->nnode;
  if (u) PM_CUDA(cudaMemcpy(u, h->D.u, sizeof(double) * nn, cudaMemcpyDeviceToHost));
  if (u0) PM_CUDA(cudaMemcpy(u0, h->D.u0, sizeof(double) * nn, cudaMemcpyDeviceToHost));
  if (dp) PM_CUDA(cudaMemcpy(dp, h->D.dp, sizeof(double) * h->nnode, cudaMemcpyDeviceToHost));
  return PM_OK;
}

int pm_set_initial_stress(pm_handle hh, const double* tx0) {
  Handle* h = reinterpret_cast<Handle*>(hh);
  if (!h || !tx0) return PM_E_ARG;
  double* d_tx0 = nullptr;
  PM_CUDA(cudaMalloc(&d_tx0, sizeof(double) * 6 * h->nnode));
  PM_CUDA(cudaMemcpy(d_tx0, tx0, sizeof(double) * 6 * h->nnode, cudaMemcpyHostToDevice));
  PM_CUDA(cudaMemsetAsync(h->D.bst0, 0, sizeof(double) * h->neq, h->stream));
  int st = PM_OK;
  for (int c = 0; c < h->numcolors && st == PM_OK; ++c) {
    cudaError_t e = pm::launch_stress5(elem_launch(h, c), h->hexa, d_tx0, h->D.bst0, h->stream);
    if (e != cudaSuccess) {
      h->err = cudaGetErrorString(e);
      st = PM_E_CUDA;
    }
  }
  if (st == PM_OK) st = check_elem_err(h);
  cudaStreamSynchronize(h->stream);
  cudaFree(d_tx0);
  if (st == PM_OK) h->fstress0 = true;
  return st;
}

int pm_set_precision(pm_handle hh, int mode) {
  Handle* h = reinterpret_cast<Handle*>(hh);
  if (!h || (mode != PM_FP64 && mode != PM_FP32_REFINE && mode != PM_FP32C_REFINE))
    return PM_E_ARG;
  h->precision = mode;
  return PM_OK;
}

int pm_tune_spmv(pm_handle hh, int* shape) {
  Handle* h = reinterpret_cast<Handle*>(hh);
  if (!h || !shape) return PM_E_ARG;
  if (!h->assembled) {
    h->err = "matrix not assembled";
    return PM_E_STATE;
  }
  PM_TRY(ensure_comp(h, h->stream));
  *shape = h->shape;
  return PM_OK;
}

int pm_set_refine(pm_handle hh, double inner_tol) {
  Handle* h = reinterpret_cast<Handle*>(hh);
  if (!h || !(inner_tol > 0.0 && inner_tol < 1.0)) return PM_E_ARG;
  h->inner_tol = inner_tol;
  return PM_OK;
}

int pm_get_sizes(pm_handle hh, int* neq, int64_t* nad, int* numcolors, int64_t* nnz_panel) {
  Handle* h = reinterpret_cast<Handle*>(hh);
  if (!h) return PM_E_ARG;
  if (neq) *neq = h->neq;
  if (nad) *nad = h->nad;
  if (numcolors) *numcolors = h->numcolors;
  if (nnz_panel) *nnz_panel = h->P.nnz;
  return PM_OK;
}

int pm_get_id(pm_handle hh, int32_t* id) {
  Handle* h = reinterpret_cast<Handle*>(hh);
  if (!h || !id) return PM_E_ARG;
  std::memcpy(id, h->h_eq.data(), sizeof(int32_t) * h->h_eq.size());
  return PM_OK;
}

int pm_get_csrd(pm_handle hh, int64_t* ia, int32_t* ja, double* ad, double* al) {
  Handle* h = reinterpret_cast<Handle*>(hh);
  if (!h) return PM_E_ARG;
  std::vector<double> val;
  if (ad || al) {
    if (!h->assembled) {
      h->err = "matrix not assembled";
      return PM_E_STATE;
    }
    val.resize(h->P.nnz);
    PM_CUDA(cudaStreamSynchronize(h->stream));
    PM_CUDA(cudaMemcpy(val.data(), h->P.val, sizeof(double) * h->P.nnz, cudaMemcpyDeviceToHost));
  }
  int64_t pos = 0;
  int row = 0;
  if (ia) ia[0] = 1;
  for (int k = 0; k < h->P.nact; ++k) {
    const int d = h->h_d[k], W = h->h_W[k], low = h->h_low[k];
    const int64_t vo = h->h_val_off[k], co = h->h_col_off[k];
    for (int q = 0; q < d; ++q, ++row) {
      const int len = low + q;
      for (int c = 0; c < len; ++c) {
        if (ja) ja[pos + c] = h->h_cols[co + c] + 1;
        if (al) al[pos + c] = val[vo + (int64_t)q * W + c];
      }
      if (ad) ad[row] = val[vo + (int64_t)q * W + low + q];
      pos += len;
      if (ia) ia[row + 1] = pos + 1;
    }
  }
  return PM_OK;
}

int pm_assemble(pm_handle hh, int isw, int lhs, int rhs, const double* u, double* b) {
  Handle* h = reinterpret_cast<Handle*>(hh);
  if (!h || !u || (rhs && !b) || (isw != 2 && isw != 4)) return PM_E_ARG;
  const size_t nn = (size_t)4 * h->nnode;
  PM_CUDA(cudaMemcpyAsync(h->D.bx, u, sizeof(double) * nn, cudaMemcpyHostToDevice, h->stream));
  if (rhs)
    PM_CUDA(cudaMemcpyAsync(h->D.by, b, sizeof(double) * h->neq, cudaMemcpyHostToDevice,
                            h->stream));
  if (isw == 2) {
    if (lhs && rhs) {
      PM_TRY(assemble_K(h, h->D.bx, h->D.by));
    } else if (lhs) {
      PM_TRY(assemble_K(h));
    } else if (rhs) {
      PM_TRY(residual(h, h->D.bx, h->D.by));
    }
  } else if (rhs) {
    PM_TRY(rhs4(h, h->D.bx, h->D.by));
  }
  PM_TRY(check_elem_err(h));
  if (rhs)
    PM_CUDA(cudaMemcpyAsync(b, h->D.by, sizeof(double) * h->neq, cudaMemcpyDeviceToHost,
                            h->stream));
  PM_CUDA(cudaStreamSynchronize(h->stream));
  return PM_OK;
}

int pm_spmv_dev(pm_handle hh, const double* d_x, double* d_y, void* stream) {
  Handle* h = reinterpret_cast<Handle*>(hh);
  if (!h || !d_x || !d_y) return PM_E_ARG;
  if (!h->assembled) {
    h->err = "matrix not assembled";
    return PM_E_STATE;
  }
  cudaStream_t s = stream ? (cudaStream_t)stream : h->stream;
  return spmv_op(h, d_x, d_y, s);
}

int pm_spmv(pm_handle hh, const double* x, double* y) {
  Handle* h = reinterpret_cast<Handle*>(hh);
  if (!h || !x || !y) return PM_E_ARG;
  if (!h->assembled) {
    h->err = "matrix not assembled";
    return PM_E_STATE;
  }
  PM_CUDA(cudaMemcpyAsync(h->D.bx, x, sizeof(double) * h->neq, cudaMemcpyHostToDevice, h->stream));
  PM_TRY(spmv_op(h, h->D.bx, h->D.by, h->stream));
  PM_CUDA(cudaMemcpyAsync(y, h->D.by, sizeof(double) * h->neq, cudaMemcpyDeviceToHost, h->stream));
  PM_CUDA(cudaStreamSynchronize(h->stream));
  if (h->precision == PM_FP32C_REFINE && h->shape == pm::kCsShape) PM_TRY(check_cs_fault(h));
  return PM_OK;
}

int pm_solve_dev(pm_handle hh, int solver, int precond, const double* d_b, double* d_x,
                 double tol, int maxit, pm_step_info* info, void* stream) {
  Handle* h = reinterpret_cast<Handle*>(hh);
  if (!h || !d_b || !d_x || maxit < 1) return PM_E_ARG;
  if (stream && (cudaStream_t)stream != h->stream) {
    // order the handle's stream after the caller's
    PM_CUDA(cudaEventRecord(h->ev[0], (cudaStream_t)stream));
    PM_CUDA(cudaStreamWaitEvent(h->stream, h->ev[0], 0));
  }
  int st = solve_dev(h, solver, precond, d_b, d_x, tol, maxit, info);
  if (stream && (cudaStream_t)stream != h->stream) {
    PM_CUDA(cudaEventRecord(h->ev[1], h->stream));
    PM_CUDA(cudaStreamWaitEvent((cudaStream_t)stream, h->ev[1], 0));
  }
  return st;
}

int pm_solve(pm_handle hh, int solver, int precond, const double* b, double* x, double tol,
             int maxit, pm_step_info* info) {
  Handle* h = reinterpret_cast<Handle*>(hh);
  if (!h || !b || !x || maxit < 1) return PM_E_ARG;
  PM_CUDA(cudaMemcpyAsync(h->D.bx, b, sizeof(double) * h->neq, cudaMemcpyHostToDevice, h->stream));
  PM_TRY(solve_dev(h, solver, precond, h->D.bx, h->D.by, tol, maxit, info));
  PM_CUDA(cudaMemcpyAsync(x, h->D.by, sizeof(double) * h->neq, cudaMemcpyDeviceToHost, h->stream));
  PM_CUDA(cudaStreamSynchronize(h->stream));
  return PM_OK;
}

int pm_matvec_csrd_dev(int neq, const int64_t* d_ia, const int32_t* d_ja, const double* d_ad,
                       const double* d_al, const double* d_x, double* d_y, void* stream) {
  if (neq <= 0 || !d_ia || !d_ja || !d_ad || !d_al || !d_x || !d_y) return PM_E_ARG;
  cudaError_t e = pm::csrd_spmv(neq, d_ia, d_ja, d_ad, d_al, d_x, d_y, (cudaStream_t)stream);
  return e == cudaSuccess ? PM_OK : PM_E_CUDA;
}

int pm_step(pm_handle hh, int maxnlit, double tol, int stop_crit, int solver, int precond,
            double solvtol, int maxit, int reassemble, pm_step_info* info) {
  Handle* h = reinterpret_cast<Handle*>(hh);
  if (!h || maxnlit < 1 || maxit < 1) return PM_E_ARG;
  if (h->ninst > 0)
    return step_batch(h, maxnlit, tol, stop_crit, solver, precond, solvtol, maxit, reassemble,
                      info);
  cudaStream_t s = h->stream;
  pm::Dev& D = h->D;
  cudaEvent_t ev[6];
  for (auto& e : ev) PM_CUDA(cudaEventCreate(&e));
  struct EvGuard {
    cudaEvent_t* e;
    ~EvGuard() {
      for (int i = 0; i < 6; ++i) cudaEventDestroy(e[i]);
    }
  } guard{ev};
  const int64_t launches0 = h->launches;
  h->istep += 1;
  h->t = h->t + h->dt;
  PM_CUDA(cudaEventRecord(ev[0], s));
  h->launches += 2 + (h->fstress0 ? 1 : 0);  // pload, predict, initial stress
  k_pload<<<grid_for(h->nnode), 256, 0, s>>>(h->nnode, D.eq, D.fnno, D.nload, D.f, D.u, D.b0,
                                              D.load, D.fload, h->maxt, D.x, h->t, h->dt,
                                              h->gravity_mod);
  PM_CUDA(cudaGetLastError());
  PM_TRY(rhs4(h, D.u, D.b0));
  if (h->fstress0) PM_CUDA(pm::axpy_into(h->neq, D.b0, D.bst0, 1.0, s));
  k_predict<<<grid_for(h->nnode), 256, 0, s>>>(h->nnode, D.fnno, D.u, D.u0);
  PM_CUDA(cudaGetLastError());
  PM_CUDA(cudaEventRecord(ev[1], s));
  bool lhs = true;
  int it = 1;
  long tot_iters = 0;
  pm_step_info loc{};
  double t_asm = 0, t_res = 0, t_sol = 0;
  for (;;) {
    PM_CUDA(cudaMemcpyAsync(D.b, D.b0, sizeof(double) * h->neq, cudaMemcpyDeviceToDevice, s));
    PM_CUDA(cudaEventRecord(ev[2], s));
    const bool need_K = lhs && (reassemble || !h->assembled || h->assembled_dt != h->dt);
    if (need_K) {
      PM_TRY(assemble_K(h, D.u, D.b));  // b -= K u in the same launch
      h->assembled32 = h->assembledC = false;
    }
    PM_CUDA(cudaEventRecord(ev[3], s));
    if (!need_K) PM_TRY(residual(h, D.u, D.b));
    PM_CUDA(cudaEventRecord(ev[4], s));
    PM_TRY(check_elem_err(h));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ev[2], ev[3]);
    t_asm += ms;
    cudaEventElapsedTime(&ms, ev[3], ev[4]);
    t_res += ms;
    if (stop_crit == 1 || stop_crit == 2) {
      h->launches += 1;
      PM_CUDA(pm::resnorms(h->neq, D.b, D.dofkind, D.norms, D.partial, D.counter, s));
      double nr[2];
      PM_CUDA(cudaMemcpyAsync(nr, D.norms, sizeof(nr), cudaMemcpyDeviceToHost, s));
      PM_CUDA(cudaStreamSynchronize(s));
      // cal_residuo_pm (Residuo.f:39-276)
      if (stop_crit == 1) {
        const double res = std::sqrt(nr[0] + nr[1]);
        if (it == 1) h->res0 = res;
        else if (it == 2) h->res0 = std::max(h->res0, res);
        loc.res_u = res;
        if (res / h->res0 < tol) break;
      } else {
        const double gresu = std::sqrt(nr[0]), gresp = std::sqrt(nr[1]);
        if (it == 1) {
          h->resu0 = gresu;
          h->resp0 = gresp;
        } else if (it == 2) {
          h->resu0 = std::max(h->resu0, gresu);
          h->resp0 = std::max(h->resp0, gresu);  // the reference compares with gresu here
        }
        loc.res_u = gresu;
        loc.res_p = gresp;
        int istop = 0;
        if (gresu / h->resu0 < tol) istop += 1;
        if (gresp / h->resp0 < tol) istop += 1;
        if (istop == 2) break;
      }
    }
    PM_CUDA(cudaEventRecord(ev[2], s));
    pm_step_info si{};
    PM_TRY(solve_dev(h, solver, precond, D.b, D.xs, solvtol, maxit, &si));
    PM_CUDA(cudaEventRecord(ev[3], s));
    loc.iters = si.iters;
    tot_iters += si.iters;
    loc.refine = si.refine;
    loc.conv = si.conv;
    loc.xkx = si.xkx;
    h->launches += 1;
    k_delta_update<<<grid_for(h->nnode), 256, 0, s>>>(h->nnode, D.eq, D.fnno, D.u, D.xs);
    PM_CUDA(cudaGetLastError());
    PM_CUDA(cudaEventSynchronize(ev[3]));
    cudaEventElapsedTime(&ms, ev[2], ev[3]);
    t_sol += ms;
    if (it >= maxnlit) {
      h->err = "nonlinear iteration: no convergence after " + std::to_string(it) + " iterations";
      return PM_E_NLNOCONV;
    }
    ++it;
    lhs = false;
  }
  loc.nlit = it;
  PM_CUDA(cudaEventRecord(ev[5], s));
  PM_TRY(porosity_pass(h, s));
  k_update_res<<<grid_for(h->nnode), 256, 0, s>>>(h->nnode, D.fnno, D.u, D.u0, D.dp);
  PM_CUDA(cudaGetLastError());
  PM_CUDA(cudaStreamSynchronize(s));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, ev[0], ev[1]);
  h->timers[0] = ms;
  h->timers[1] = t_asm;
  h->timers[2] = t_res;
  h->timers[3] = t_sol;
  h->timers[4] = (double)tot_iters;
  h->launches += 1;  // update_res
  h->timers[7] = (double)(h->launches - launches0);
  if (info) *info = loc;
  return PM_OK;
}

int pm_set_nkrylov(pm_handle hh, int nkrylov) {
  Handle* h = reinterpret_cast<Handle*>(hh);
  if (!h || nkrylov < 1) return PM_E_ARG;
  h->nkrylov = nkrylov;
  return PM_OK;
}

int pm_get_porosity(pm_handle hh, double* poro) {
  Handle* h = reinterpret_cast<Handle*>(hh);
  if (!h || !poro) return PM_E_ARG;
  PM_CUDA(cudaStreamSynchronize(h->stream));
  PM_CUDA(cudaMemcpy(poro, h->D.poro, sizeof(double) * h->nnode, cudaMemcpyDeviceToHost));
  return PM_OK;
}

int pm_set_porosity(pm_handle hh, const double* poro) {
  Handle* h = reinterpret_cast<Handle*>(hh);
  if (!h || !poro) return PM_E_ARG;
  PM_CUDA(cudaStreamSynchronize(h->stream));
  PM_CUDA(cudaMemcpy(h->D.poro, poro, sizeof(double) * h->nnode, cudaMemcpyHostToDevice));
  return PM_OK;
}

int pm_stress_dev(pm_handle hh, double* d_tx, double* d_txb, double* d_txe, double* d_flux,
                  void* stream) {
  Handle* h = reinterpret_cast<Handle*>(hh);
  if (!h || !d_tx || !d_txb || !d_txe || !d_flux) return PM_E_ARG;
  cudaStream_t s = stream ? (cudaStream_t)stream : h->stream;
  // the state and the scratch belong to the handle's stream
  if (stream) PM_CUDA(cudaStreamSynchronize(h->stream));
  const size_t nn = (size_t)h->nnode;
  PM_CUDA(cudaMemsetAsync(d_tx, 0, sizeof(double) * 6 * nn, s));
  PM_CUDA(cudaMemsetAsync(d_txb, 0, sizeof(double) * 6 * nn, s));
  PM_CUDA(cudaMemsetAsync(d_flux, 0, sizeof(double) * 3 * nn, s));
  h->launches += h->numcolors + 1;
  for (int c = 0; c < h->numcolors; ++c)
    PM_CUDA(pm::launch_stress3(elem_launch(h, c), h->hexa, h->D.u, h->D.dp, d_tx, d_txb, d_flux,
                               s));
  k_stress_finish<<<grid_for(h->nnode), 256, 0, s>>>(h->nnode, h->D.fnno, h->D.vcnt, h->D.u, d_tx,
                                                      d_txb, d_txe, d_flux);
  PM_CUDA(cudaGetLastError());
  if (stream) PM_CUDA(cudaStreamSynchronize(s));
  return check_elem_err(h);
}

int pm_stress(pm_handle hh, double* tx, double* txb, double* txe, double* flux) {
  Handle* h = reinterpret_cast<Handle*>(hh);
  if (!h || !tx || !txb || !txe || !flux) return PM_E_ARG;
  const size_t nn = (size_t)h->nnode;
  double* d = nullptr;
  PM_CUDA(cudaMalloc(&d, sizeof(double) * 21 * nn));
  int st = pm_stress_dev(hh, d, d + 6 * nn, d + 12 * nn, d + 18 * nn, nullptr);
  if (st == PM_OK) {
    cudaMemcpy(tx, d, sizeof(double) * 6 * nn, cudaMemcpyDeviceToHost);
    cudaMemcpy(txb, d + 6 * nn, sizeof(double) * 6 * nn, cudaMemcpyDeviceToHost);
    cudaMemcpy(txe, d + 12 * nn, sizeof(double) * 6 * nn, cudaMemcpyDeviceToHost);
    if (cudaMemcpy(flux, d + 18 * nn, sizeof(double) * 3 * nn, cudaMemcpyDeviceToHost) !=
        cudaSuccess) {
      h->err = "cudaMemcpy failed";
      st = PM_E_CUDA;
    }
  }
  cudaFree(d);
  return st;
}

int pm_set_materials(pm_handle hh, const double* e, int numat) {
  Handle* h = reinterpret_cast<Handle*>(hh);
  if (!h || !e || numat != h->numat) return PM_E_ARG;
  h->h_e.assign(e, e + (size_t)PM_PROP * numat);
  return upload_materials(h);
}

static int adjoint_launch(Handle* h, int mode, const double* d_lam, const double* d_un,
                          const double* d_dun, double* d_mu, double* d_nu, double* d_grad,
                          void* stream) {
  if (!h->assembled) {
    h->err = "adjoint before assembly (the element passes use the step's dt)";
    return PM_E_STATE;
  }
  cudaStream_t s = stream ? (cudaStream_t)stream : h->stream;
  h->launches += 1 + h->numcolors;
  k_eq_to_nodal<<<grid_for(4 * h->nnode), 256, 0, s>>>(h->nnode, h->D.eq, d_lam, h->D.bx);
  PM_CUDA(cudaGetLastError());
  for (int c = 0; c < h->numcolors; ++c)
    PM_CUDA(pm::launch_adjoint(elem_launch(h, c), h->hexa, mode, h->D.bx, d_un, d_dun, d_mu,
                               d_nu, d_grad, s));
  if (stream) PM_CUDA(cudaStreamSynchronize(s));
  return check_elem_err(h);
}

int pm_adjoint_apply_dev(pm_handle hh, const double* d_lam, double* d_mu, double* d_nu,
                         void* stream) {
  Handle* h = reinterpret_cast<Handle*>(hh);
  if (!h || !d_lam || !d_mu || !d_nu) return PM_E_ARG;
  return adjoint_launch(h, 0, d_lam, nullptr, nullptr, d_mu, d_nu, nullptr, stream);
}

int pm_adjoint_grad_dev(pm_handle hh, const double* d_lam, const double* d_un,
                        const double* d_dun, double* d_grad, void* stream) {
  Handle* h = reinterpret_cast<Handle*>(hh);
  if (!h || !d_lam || !d_un || !d_dun || !d_grad) return PM_E_ARG;
  return adjoint_launch(h, 1, d_lam, d_un, d_dun, nullptr, nullptr, d_grad, stream);
}

int pm_get_timers(pm_handle hh, double* t, int n) {
  Handle* h = reinterpret_cast<Handle*>(hh);
  if (!h || !t) return PM_E_ARG;
  for (int i = 0; i < n && i < 8; ++i) t[i] = h->timers[i];
  return PM_OK;
}

}  // extern "C"
