// pm_internal.h -- handle, device data layout and kernel interfaces of the
// GB300 Biot hot path.  Shared by the host set-up (pm_setup.cpp), the
// element kernels (pm_elements.cu) and the C ABI (pm_capi.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/poromec_gb300.h"
#include "pm_krylov.h"

namespace pm {

constexpr int kMaxNen = 20;
constexpr int kNdf = 4;

// Per-material constants of the elastic Biot elements (elmt17_pm,
// Elmlib03.f:1950-2000; elmt15_pm :190-240), from e(1..7) and |g|.
struct MatConst {
  double a, b, c;        // a = E(1-nu)/((1+nu)(1-2nu)), b = nu/(1-nu), c = (1-2nu)/(2(1-nu))
  double coef_biot;      // alpha
  double imod_biot;      // 1/M
  double perm;           // K_h / (rho_f 1e-6 |g|)
  double pm_d, fluid_d;  // densities * 1e-6
};

// Node-panel storage of the assembled symmetric matrix (both triangles).
// The free dofs of a node carry consecutive equation numbers (numeqpmec2),
// and all rows of a node have the same columns: the free dofs of every node
// sharing an element with it.  Node I owns a dense d_I x W_I panel stored
// row-major; its W_I columns are listed once.  The reference CSRD row r of
// node I (local dof q) is the first low_I + q entries of panel row q.
struct Panels {
  int nact = 0;           // nodes with at least one free dof
  int64_t nnz = 0;        // sum d_I W_I
  int64_t ncols = 0;      // sum W_I
  int32_t* order = nullptr;  // active nodes sorted by (d, W) for the SpMV
  int32_t* eq0 = nullptr;
  int32_t* d = nullptr;
  int32_t* W = nullptr;
  int32_t* low = nullptr;
  int64_t* val_off = nullptr;
  int64_t* col_off = nullptr;
  int32_t* cols = nullptr;
  double* val = nullptr;   // FP64 values
  float* val32 = nullptr;  // FP32 values (PM_FP32_REFINE)
  float* valh = nullptr;      // compensated values (PM_FP32C_REFINE): fl32(v)
  int8_t* vall = nullptr;     //   and round((v - fl32(v)) / fl32(v) * 2^31)
  // the same values as node records for the record kernel (CompVals)
  uint8_t* rec = nullptr;
  int64_t* rec_off = nullptr;
  int rec_max = 0, ca_warps = 0, ca_grid = 0;
  int4* cs_desc = nullptr;
  int32_t *cs_batch_slot = nullptr, *cs_batch_bytes = nullptr, *cs_cta_batch = nullptr;
  int64_t* cs_batch_off = nullptr;
  int cs_grid = 0, cs_nstage = 0, cs_stage_bytes = 0;
  int* fault = nullptr;
  // batches: instance of each active node, done flag of each instance
  int32_t* node_inst = nullptr;
  int* inst_done = nullptr;
  // indexed by node id - 1
  int64_t* node_val_off = nullptr;
  int32_t* node_W = nullptr;
  int4* meta = nullptr;  // per visiting slot (PanelView::meta), or null
  PanelView view() const {
    return PanelView{nact, order, eq0, d, W, low, val_off, col_off, cols, nullptr, nullptr, meta};
  }
  // the view of the batched iteration: rows of converged instances skipped
  PanelView bview() const {
    return PanelView{nact,   order,    eq0,  d,         W,        low,
                     val_off, col_off, cols, node_inst, inst_done, meta};
  }
  CompVals comp(int shape) const {
    return CompVals{valh,          vall,          rec,          rec_off,        rec_max,
                    ca_warps,      ca_grid,       cs_desc,      cs_batch_slot,  cs_batch_off,
                    cs_batch_bytes, cs_cta_batch, cs_grid,      cs_nstage,      cs_stage_bytes,
                    fault,         shape};
  }
};

struct ElemLaunch {
  const int32_t* ix;     // (nen+1, numel)
  const int32_t* eq;     // (ndf, nnode), 1-based equation numbers
  const double* x;       // (3, nnode)
  const MatConst* mat;   // numat
  const int32_t* slot;   // (nen, nen) per element of the launched colour
  const int32_t* elems;  // 1-based element ids of the colour
  int nelem;
  int nen;
  const int64_t* node_val_off;
  const int32_t* node_W;
  double dt, t;
  double g0, g1, g2, gmod;
  int* err;
};

// The hexa shape-function table of the element kernels, filled once per
// device; called before a handle's first element launch.
constexpr int kMaxDevices = 64;
cudaError_t ensure_shape_tables();
// Element matrices into the FP64 panels; with b the same launch also does
// b -= K_e u_e (isw 2 with lhs and rhs) from the blocks it assembles.
cudaError_t launch_assemble_K(const ElemLaunch& L, bool hexa, double* val, cudaStream_t s,
                              const double* u = nullptr, double* b = nullptr);
cudaError_t launch_residual(const ElemLaunch& L, bool hexa, const double* u,
                            double* b, cudaStream_t s);
cudaError_t launch_rhs4(const ElemLaunch& L, bool hexa, const double* u,
                        const double* dp, const int32_t* eload,
                        const int32_t* eloadp, const int32_t* load,
                        const double* fload, int maxt, double* b,
                        cudaStream_t s);
cudaError_t launch_adjoint(const ElemLaunch& L, bool hexa, int mode, const double* lam,
                           const double* un, const double* dun, double* mu, double* nu,
                           double* grad, cudaStream_t s);
cudaError_t launch_stress3(const ElemLaunch& L, bool hexa, const double* u,
                           const double* dp, double* tx, double* txb, double* flux,
                           cudaStream_t s);
cudaError_t launch_poro7(const ElemLaunch& L, bool hexa, const double* du, double* dporo,
                         cudaStream_t s);
cudaError_t launch_stress5(const ElemLaunch& L, bool hexa, const double* tx0,
                           double* b, cudaStream_t s);
// Nodal kernels of the step driver (pm_capi.cu).
struct Handle;

struct Dev {
  int32_t* ix = nullptr;
  int32_t* eq = nullptr;
  double* x = nullptr;
  MatConst* mat = nullptr;
  int32_t* slot = nullptr;         // (nen*nen) per element, elements in colour order
  int32_t* color_elems = nullptr;  // 1-based element ids, colour by colour
  int32_t* eload = nullptr;
  int32_t* eloadp = nullptr;
  int32_t* nload = nullptr;
  int32_t* load = nullptr;
  double* fload = nullptr;
  int32_t* dofkind = nullptr;      // per equation: 0 displacement, 1 pressure
  int32_t* fnno = nullptr;
  double *u = nullptr, *u0 = nullptr, *dp = nullptr, *f = nullptr;
  double *poro = nullptr, *dporo = nullptr;  // nodal porosity and its step change
  int32_t* vcnt = nullptr;                    // elements sharing each vertex node
  double* gm_basis = nullptr;  // GMRES(l): (k+1) x neq Krylov basis, allocated on first use
  double* gm_scal = nullptr;   // GMRES(l): per-step dot products (2k + 4)
  double* gm_y = nullptr;      // GMRES(l): the cycle's coefficients (k)
  double *b0 = nullptr, *b = nullptr, *bst0 = nullptr;
  double *ad = nullptr, *m = nullptr;
  double *bx = nullptr, *by = nullptr;   // staging vectors for host calls
  double *rr = nullptr, *dx = nullptr;   // refinement residual / correction
  double* xs = nullptr;                  // solution of the step's solve
  KrylovVecs kv{};
  KrylovVecs32 kv32{};
  KrylovScalars* ks = nullptr;
  double* partial = nullptr;
  unsigned* counter = nullptr;
  double* norms = nullptr;
  int* err = nullptr;
  int* trips = nullptr;  // trips of the device-side solve loop (pcg_loop)
};

struct Handle {
  int nnode = 0, nnodev = 0, numel = 0, nen = 0, nenv = 0, ndf = 4, numat = 0;
  bool hexa = true;
  int neq = 0;
  int64_t nad = 0;
  int numcolors = 0;
  int precision = PM_FP64;
  double inner_tol = 1.0e-5;   // inner tolerance of the FP32 refinement sweeps
                               // (and of a compensated MINRES cycle)
  double cycle_conv = 0.0;     // the current compensated MINRES cycle's target
  int nkrylov = 150;           // GMRES(l) basis size (ngram, Main.f:274)
  int gm_alloc_k = 0;          // basis size of the allocated D.gm_basis
  bool debug = false;          // PM_DEBUG set: solver progress on stderr
  std::vector<int32_t> color_ptr;
  std::vector<int32_t> h_eq;       // (ndf, nnode)
  std::vector<int32_t> h_fnno;
  std::vector<MatConst> h_mat;
  std::vector<double> h_e;
  std::vector<int32_t> h_ie;
  // host copies of the panel structure (pm_get_csrd)
  std::vector<int32_t> h_eq0, h_d, h_W, h_low, h_cols;
  std::vector<int32_t> h_order;    // SpMV visiting order of the active nodes
  // batch of independent meshes (pm_batch_create); ninst = 0 for one mesh
  int ninst = 0;
  std::vector<int32_t> h_inst_node;  // ninst + 1 node ranges (0-based)
  std::vector<int32_t> h_inst_act;   // instance of each active node
  std::vector<int32_t> h_inst_eq;    // ninst + 1 equation ranges (0-based)
  BatchView B{};
  int* d_insweep = nullptr;
  double* d_conv0 = nullptr;
  double* d_bnorms = nullptr;
  std::vector<double> b_res0, b_resu0, b_resp0;
  std::vector<int> b_iters;          // Krylov iterations of the last solve, per instance
  std::vector<int> b_nlit;           // nonlinear iterations of the last step, per instance
  std::vector<int64_t> h_val_off, h_col_off;
  int nloads = 0, maxt = 1;
  double gravity[3] = {0.0, 0.0, -9.81};
  double gravity_mod = 9.81;
  double dt = 1.0, t = 0.0;
  int istep = 0;
  bool fstress0 = false;
  bool assembled = false;      // FP64 panel values valid
  bool assembled32 = false;    // FP32 panel values valid
  bool assembledC = false;     // compensated panel values valid
  int shape = 0;               // compensated SpMV shape code (0 = not tuned)
  double assembled_dt = -1.0;
  double resu0 = 0.0, resp0 = 0.0, res0 = 0.0;
  Panels P;
  Dev D;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  // graphs of kGraphIters iterations (pointers baked in are fixed for the
  // handle's lifetime)
  cudaGraphExec_t pcg_graph = nullptr, minres_graph = nullptr, pcgm_graph = nullptr;
  cudaGraphExec_t pcgc_graph = nullptr, minresc_graph = nullptr;
  cudaGraphExec_t bpcg_graph = nullptr, bpcgc_graph = nullptr;
  cudaGraphExec_t sqmr_graph = nullptr;
  cudaGraphExec_t sqmrc_graph = nullptr;
  // a whole FP64 PCG solve in one graph: a conditional while node around
  // kGraphIters iterations (built on the first solve; not used if the
  // driver cannot build it)
  cudaGraphExec_t pcg_loop = nullptr;
  bool pcg_loop_failed = false;
  // a batch time step as one graph (step_batch_graph): control state and
  // per-instance arrays on the device, the executable graph of the last step
  pm::BatchCtl* d_bctl = nullptr;
  pm::BatchStepArrays bsa{};
  cudaGraphExec_t bstep_exec = nullptr;
  bool bstep_failed = false;
  double timers[8] = {0};
  int64_t launches = 0;        // kernels launched by the library (all calls)
  std::string err;
};

// pm_setup.cpp
int build_structure(Handle* h, const int32_t* ix, const int32_t* idflag,
                    const int32_t* fnno, const double* x, const int32_t* num);
int build_rec_layout(Handle* h);
// PanelView::meta from the host panel arrays (inst: the instance of each
// active node, or null for one mesh); leaves it null when a field does not fit
int build_meta(Handle* h, const int32_t* inst);

}  // namespace pm
