// pm_krylov.h -- interfaces of the SpMV and Krylov kernels (pm_sparse.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace pm {

#ifdef __CUDACC__
// v as an unevaluated FP32 pair (hi, lo), the operand format of the
// compensated operator, split by truncation on the integer pipe: hi keeps
// the top 24 significand bits of v and lo the top 24 of the exact remainder
// v - hi, so |v - hi - lo| < 2^-46 |v|.  For 2^-78 <= |v| < 2^127 both are
// built from v's bits (lo = 0 where the remainder is below float's normal
// range, an error under 2^-47 |v|), with no FP64 conversion; other values
// take the rounded conversions.
__device__ __forceinline__ float2 split_pair(double v) {
  const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(v));
  const unsigned e = unsigned(b >> 52) & 0x7ffu;  // biased FP64 exponent
  if (e - 945u <= 1150u - 945u) {
    const unsigned sign = unsigned(b >> 32) & 0x80000000u;
    const float hi = __uint_as_float(sign | ((e - 896u) << 23) | (unsigned(b >> 29) & 0x7fffffu));
    const unsigned m = unsigned(b) & 0x1fffffffu;  // the 29 significand bits below hi
    float lo = 0.f;
    if (m != 0u) {
      const int k = 31 - __clz(static_cast<int>(m));  // leading bit of m, 0..28
      const int ef = int(e) - 948 + k;                 // float exponent field of lo
      if (ef >= 1) {
        const unsigned mant = k >= 23 ? (m >> (k - 23)) : (m << (23 - k));
        lo = __uint_as_float(sign | (unsigned(ef) << 23) | (mant & 0x7fffffu));
      }
    }
    return make_float2(hi, lo);
  }
  const float h = float(v);
  return make_float2(h, float(v - double(h)));
}
#endif

// Grid of the SpMV and reduction kernels: 8 CTAs of 256 threads per SM on
// the 152 SMs of a GB300, so the last-block reductions sum at most 1216
// partials.
constexpr int kRedBlocks = 1216;

// Read-only view of the node panels passed by value to kernels.
struct PanelView {
  int nact;
  const int32_t* order;    // SpMV visiting order: active nodes sorted by (d, W)
  const int32_t* eq0;      // first equation (0-based) per active node
  const int32_t* d;        // free dofs per active node
  const int32_t* W;        // panel width
  const int32_t* low;      // columns left of the node's own dofs
  const int64_t* val_off;  // value offset
  const int64_t* col_off;  // column list offset
  const int32_t* cols;     // 0-based column equations
  // batches of independent meshes: the instance of each active node, and the
  // instances whose solve has converged (their rows are skipped); both null
  // for a single mesh
  const int32_t* node_inst;
  const int* inst_done;
  // the same per visiting slot as one 16-byte record, so that a node's panel
  // is located by one load: x eq0, y d | W << 3 | instance << 16,
  // z val_off, w col_off (unsigned); null when a field does not fit
  // (W >= 8192, 65536 instances or more, 2^32 panel values or columns)
  const int4* meta;
};

// A node's panel located from its visiting slot: meta record or the separate
// arrays; on = false past the last slot or for a converged instance.
struct NodeRef {
  int e0, d, W;
  int64_t vo, co;
  bool on;
};
// the node of a meta record m already loaded for slot
__device__ __forceinline__ NodeRef node_from_meta(const PanelView& P, const int4& m, int slot) {
  NodeRef r{0, 0, 0, 0, 0, false};
  if (slot >= P.nact) return r;
  if (P.inst_done && P.inst_done[(unsigned)m.y >> 16]) return r;
  r.e0 = m.x;
  r.d = m.y & 7;
  r.W = (m.y >> 3) & 8191;
  r.vo = (int64_t)(unsigned)m.z;
  r.co = (int64_t)(unsigned)m.w;
  r.on = true;
  return r;
}
__device__ __forceinline__ NodeRef node_ref(const PanelView& P, int slot) {
  NodeRef r{0, 0, 0, 0, 0, false};
  if (slot >= P.nact) return r;
  if (P.meta) {
    return node_from_meta(P, P.meta[slot], slot);
  } else {
    const int node = P.order[slot];
    if (P.inst_done && P.inst_done[P.node_inst[node]]) return r;
    r.e0 = P.eq0[node];
    r.d = P.d[node];
    r.W = P.W[node];
    r.vo = P.val_off[node];
    r.co = P.col_off[node];
  }
  r.on = true;
  return r;
}

// Scalars of one Krylov solve, kept in device memory so that a captured
// graph of iterations runs without host round trips.
struct KrylovScalars {
  double d, bmb, conv, alpha, beta, pq, xkx;
  double beta_old, normr, neta, c, c_old, s, s_old, ro1, t1, t2, t3, t4;
  int done;       // set by the first kernel of the iteration after conv_flag
  int conv_flag;  // 1 converged, 2 iteration limit, 3 breakdown (non-finite)
  int iter;       // iterations completed (all restarts)
  int jcycle;     // iterations of the current MINRES cycle
  int maxit;
};

struct KrylovVecs {
  double *x, *r, *z, *p, *q;        // PCG
  double *v, *v0, *w0, *w00, *z0;   // MINRES (also uses x, z, p, q)
};

// FP32 copies used by the mixed-precision PCG: the search direction and
// its product with the FP32 matrix (PM_FP32_REFINE); the operand of the
// compensated product as interleaved (hi, lo) pairs (PM_FP32C_REFINE).
struct KrylovVecs32 {
  float *p, *q;
  float2* c;
};

int vec_grid(int n);
cudaError_t pcgm_init(int n, const double* b, const double* m, KrylovVecs& V,
                      KrylovVecs32& V32, KrylovScalars* ks, double tol, int maxit,
                      double* partial, unsigned* counter, cudaStream_t s);
cudaError_t pcgm_iteration(const PanelView& P, const float* val32, int n, const double* m,
                           KrylovVecs& V, KrylovVecs32& V32, KrylovScalars* ks,
                           double* partial, unsigned* counter, cudaStream_t s);
cudaError_t spmv(const PanelView& P, const double* val64, const double* x, double* y,
                 int mode, KrylovScalars* ks, double* partial, unsigned* counter,
                 cudaStream_t s);
cudaError_t pcg_init(int n, const double* b, const double* m, KrylovVecs& V,
                     KrylovScalars* ks, double tol, int maxit, double* partial,
                     unsigned* counter, cudaStream_t s);
cudaError_t pcg_iteration(const PanelView& P, const double* val64, int n, const double* m,
                          KrylovVecs& V, KrylovScalars* ks, double* partial,
                          unsigned* counter, cudaStream_t s);
// rpsqmr (Iters.f:6100-6439): init and one iteration (4 launches)
cudaError_t sqmr_init(int n, const double* b, const double* m, KrylovVecs& V, float2* qc,
                      KrylovScalars* ks, double tol, double conv_abs, int maxit,
                      double* partial, unsigned* counter, cudaStream_t s);
cudaError_t sqmr_iteration(const PanelView& P, const double* val64, int n, const double* m,
                           KrylovVecs& V, KrylovScalars* ks, double* partial,
                           unsigned* counter, cudaStream_t s);
// GMRES(l) vector kernels (pm_gmres.cu)
cudaError_t gm_resid(int n, const double* b, const double* ax, const double* m, double* g1,
                     double* out, double* partial, unsigned* counter, cudaStream_t s);
cudaError_t gm_scale(int n, double* g, double sc, cudaStream_t s);
cudaError_t gm_first(int n, double* w, const double* m, const double* g1, double* out,
                     double* partial, unsigned* counter, cudaStream_t s);
cudaError_t gm_mgs(int n, double* w, const double* gj, const double* gnext, const double* bin,
                   double* out, double* partial, unsigned* counter, cudaStream_t s);
cudaError_t gm_dot(int n, const double* a, const double* b, double* out, double* partial,
                   unsigned* counter, cudaStream_t s);
cudaError_t gm_update(int n, double* x, const double* G, const double* y, int ni,
                      cudaStream_t s);
cudaError_t minres_conv(int n, const double* b, const double* m, KrylovScalars* ks,
                        double tol, double* partial, unsigned* counter, cudaStream_t s);
// pair != nullptr also writes the FP32 pair of z0 (compensated iteration)
cudaError_t minres_start(const PanelView& P, const double* val64, int n, const double* b,
                         const double* m, KrylovVecs& V, const KrylovVecs32* pair,
                         KrylovScalars* ks, int maxit, bool zero_x, double* partial,
                         unsigned* counter, cudaStream_t s);
cudaError_t minres_iteration(const PanelView& P, const double* val64, int n, const double* m,
                             KrylovVecs& V, KrylovScalars* ks, double* partial,
                             unsigned* counter, cudaStream_t s);
cudaError_t csrd_spmv(int neq, const int64_t* ia, const int32_t* ja, const double* ad,
                      const double* al, const double* x, double* y, cudaStream_t s);
cudaError_t precond(int n, const double* ad, double* m, int absval, int* zero_diag,
                    cudaStream_t s);
cudaError_t panel_diag(const PanelView& P, const double* val64, const float* val32,
                       double* ad, cudaStream_t s);
cudaError_t resnorms(int n, const double* b, const int32_t* kind, double* out,
                     double* partial, unsigned* counter, cudaStream_t s);
cudaError_t wnorm2(int n, const double* r, const double* m, double* out, double* partial,
                   unsigned* counter, cudaStream_t s);
cudaError_t axpy_into(int n, double* y, const double* x, double a, cudaStream_t s);
cudaError_t vsub(int n, double* y, const double* a, const double* b, cudaStream_t s);
cudaError_t to_f32(int64_t n, const double* a, float* b, cudaStream_t s);

// Compensated FP32 operator (PM_FP32C_REFINE).  Each FP64 panel value v is
// held as hi = fl32(v) and an int8 relative correction q (v = hi (1 + q 2^-31)
// within 2^-32 |v|), 5 bytes; the operand vector as interleaved FP32 pairs
// (KrylovVecs32::c); products and sums in compensated FP32 arithmetic, the
// result in FP64.
struct CompVals {
  const float* hi;
  const int8_t* lo;
  // Record layout (shape kCaShape): per active node one 16-byte aligned record
  // at rec + rec_off[node]: d rows of Wp = W rounded up to 4 FP32 hi values,
  // then d * Wp biased corrections qb = q + 128 (padded to 16 bytes), then
  // the Wp column indices (pad columns repeat the last one, with zero values).
  // Records follow the SpMV visiting order, so the product streams them.
  const uint8_t* rec;
  const int64_t* rec_off;
  int rec_max;   // bytes of the largest record
  int ca_warps;  // warps per CTA of the record kernel (two records each in smem)
  int ca_grid;   // its CTAs (resident on all SMs)
  // Streamed record kernel (shape kCsShape): the records cut into batches of
  // up to kCsNodes consecutive nodes (one contiguous byte range each), runs
  // of batches per CTA, and per visiting slot (eq0, d, W, byte offset of the
  // node's record in its batch).
  const int4* cs_desc;
  const int32_t* cs_batch_slot;   // first slot of each batch (+ end)
  const int64_t* cs_batch_off;    // byte offset of each batch in rec
  const int32_t* cs_batch_bytes;  // bytes of each batch
  const int32_t* cs_cta_batch;    // first batch of each CTA (+ end)
  int cs_grid, cs_nstage, cs_stage_bytes;
  int* fault;  // set when a pipeline wait of the streamed kernel gave up
  int shape;  // SpMV shape: 10 * (0: 8, 1: 16, 2: 32 lanes per node) + columns
              // per lane and trip (1, 2, 4), + 100 for packed two-row FP32
              // arithmetic; 214: shape 14 held to 64 registers (4 CTAs per
              // SM), 312 / 314: shapes 112 / 114 held to 4 / 3 CTAs per SM;
              // kCaShape: the record kernel; kCsShape: the streamed record
              // kernel
};
constexpr int kCaShape = 90, kCsShape = 91;
constexpr int kCsWarps = 8;                // consumer warps of the streamed kernel
constexpr int kCsNodes = 2 * kCsWarps;     // nodes per batch (one per half-warp)
constexpr int kCsMaxStages = 4;
constexpr int kCfShapes[] = {1,   2,   4,   11,  12,  14,  21,  22,  24,
                              104, 112, 114, 124, 214, 312, 314, kCaShape, kCsShape};
cudaError_t split_values(int64_t n, const double* v, float* hi, int8_t* lo, cudaStream_t s);
cudaError_t split_records(const PanelView& P, const double* v, CompVals C, cudaStream_t s);
// Dynamic shared memory of the record kernel for a given record size and
// warp count, and the set-up of its launch attributes (once per process).
int ca_smem_bytes(int rec_max, int warps);
cudaError_t ca_configure(int rec_max, int* warps, int* grid);
// Shared memory of the streamed kernel for nstage stages of stage_bytes, and
// the stage count that fits (0: the kernel is not available for this mesh).
int cs_smem_bytes(int nstage, int stage_bytes);
cudaError_t cs_configure(int stage_bytes, int* nstage, int* ctas);
cudaError_t split_pair(int n, const double* v, float2* pr, cudaStream_t s);
cudaError_t spmvc(const PanelView& P, CompVals C, const float2* xp, double* y, cudaStream_t s);
// the PCG form of the compensated product: y = A x and ks->alpha = ks->d / (y . xd)
cudaError_t spmvc_pcg(const PanelView& P, CompVals C, const float2* xp, double* y,
                      const double* xd, KrylovScalars* ks, double* partial, unsigned* counter,
                      cudaStream_t s);
cudaError_t pcgc_init(int n, const double* b, const double* m, KrylovVecs& V,
                      KrylovVecs32& V32, KrylovScalars* ks, double tol, double conv_abs,
                      int maxit, double* partial, unsigned* counter, cudaStream_t s);
cudaError_t pcgc_iteration(const PanelView& P, CompVals C, int n, const double* m,
                           KrylovVecs& V, KrylovVecs32& V32, KrylovScalars* ks,
                           double* partial, unsigned* counter, cudaStream_t s);
// A device-side solve loop: loop_start, before the conditional while node,
// resets *trips and opens the loop (the handle's launch value is 0, so a
// loop whose condition is never set does not run); loop_next, the last
// kernel of the body, keeps it going while the solve has neither converged
// nor stopped (ks->conv_flag == 0), at most ks->maxit / iters_per_trip + 4
// trips.
cudaError_t loop_start(int* trips, cudaGraphConditionalHandle cond, cudaStream_t s);
cudaError_t loop_next(const KrylovScalars* ks, int* trips, cudaGraphConditionalHandle cond,
                      int iters_per_trip, cudaStream_t s);
// residual replacement of the compensated PCG: r = b - q (q = A x in FP64),
// z = m r, d = (r, z), flags re-decided; x and p kept
cudaError_t pcgc_replace(int n, const double* b, const double* q, const double* m,
                         KrylovVecs& V, KrylovScalars* ks, double* partial, unsigned* counter,
                         cudaStream_t s);
cudaError_t minresc_iteration(const PanelView& P, CompVals C, int n, const double* m,
                              KrylovVecs& V, KrylovVecs32& V32, KrylovScalars* ks,
                              double* partial, unsigned* counter, cudaStream_t s);
cudaError_t sqmrc_iteration(const PanelView& P, CompVals C, int n, const double* m,
                            KrylovVecs& V, KrylovVecs32& V32, KrylovScalars* ks,
                            double* partial, unsigned* counter, cudaStream_t s);
cudaError_t true_residual(int n, const double* b, const double* q, const double* m, int absval,
                          double* r, double* out, double* partial, unsigned* counter,
                          cudaStream_t s);

// ---- batches of independent meshes (pm_batch.cu) ------------------------------
// The instances are held as one union mesh; their equations are contiguous
// ranges.  Per-instance dot products are segmented reductions: each block
// takes a chunk of one instance's range, and the last block of an instance
// sums the instance's block partials in block order (deterministic).
struct BatchScalars {
  double d, bmb, conv, alpha, beta, pq;
  int iter, conv_flag, maxit, pad;
};

struct BatchView {
  int ninst;
  int nblk;                 // blocks of the segmented layout
  int chunk;                // equations per block
  const int32_t* eq_ptr;    // ninst + 1 equation ranges
  const int32_t* blk_ptr;   // ninst + 1 block ranges
  const int32_t* blk_inst;  // instance of each block
  BatchScalars* bs;         // per instance
  int* done;                // per instance: solve finished (or not in this sweep)
  int* nactive;             // instances still iterating
  double* partial;          // 2 * nblk
  unsigned* counter;        // per instance
};

cudaError_t bpcg_init(const BatchView& B, const double* b, const double* m, KrylovVecs& V,
                      float2* pair, double tol, const double* conv_abs, const int* insweep,
                      int maxit, cudaStream_t s);
// one iteration: q = A p (FP64 panels, or the compensated operator when
// C != nullptr), then the per-instance alpha, update and direction
cudaError_t bpcg_iteration(const PanelView& P, const double* val64, const CompVals* C,
                           const BatchView& B, const double* m, KrylovVecs& V, float2* pair,
                           cudaStream_t s);
// bpcg_init for a refinement sweep decided on the device: b and pcg's test
// when *sweep = 0, b_refine and conv_abs after
cudaError_t bpcg_init_sweep(const BatchView& B, const double* b, const double* b_refine,
                            const double* m, KrylovVecs& V, float2* pair, double tol,
                            const double* conv_abs, const int* insweep, int maxit,
                            const int* sweep, cudaStream_t s);
cudaError_t bresnorms(const BatchView& B, const double* b, const int32_t* kind, double* out,
                      cudaStream_t s);
cudaError_t btrue_residual(const BatchView& B, const double* b, const double* q,
                           const double* m, double* r, double* out, cudaStream_t s);
cudaError_t baxpy(const BatchView& B, double* y, const double* x, const int* mask,
                  cudaStream_t s);

// ---- a batch time step driven on the device (one CUDA graph per step) ----
// Control state, set by the control kernels between the graph's
// conditional nodes and read by the host once the step's graph has run.
struct BatchCtl {
  int it;          // nonlinear iteration (1-based)
  int sweeps;      // refinement sweeps of the current solve
  int trips;       // PCG loop trips of the current sweep
  int err;         // 0 or the step's status (PM_E_NOCONV, PM_E_NLNOCONV, PM_E_ZERO_DIAG)
  int err_inst;    // Krylov failure: its instance (-1 the trip bound, -2 the sweeps)
  int err_flag;    //   and the instance's conv_flag
  int err_iters;   //   and its iterations
  int zdiag;       // zero diagonal seen by the preconditioner
  int refine;      // sweeps of the last solve (compensated operator)
  int iters_max;   // the largest per-instance iteration count of a solve
  int runs_nl, runs_sweep, runs_pcg, ok;  // trips of each loop, closing passes run
  double res_max;  // the largest residual norm of the stop test (stop_crit 1)
};

// per-instance device arrays of the step (ni each; nr 2 ni)
struct BatchStepArrays {
  int *active, *insweep, *total, *iters, *nlit;
  double *conv0, *res0, *resu0, *resp0, *nr, *rn2;
};

cudaError_t bs_begin(BatchCtl* c, const BatchStepArrays& A, int ni, cudaStream_t s);
cudaError_t bs_stop(BatchCtl* c, const BatchStepArrays& A, int ni, int stop_crit, double tol,
                    cudaGraphConditionalHandle cond, cudaStream_t s);
cudaError_t bs_solve_start(BatchCtl* c, const BatchStepArrays& A, int ni,
                           cudaGraphConditionalHandle cond, cudaStream_t s);
cudaError_t bs_loop_start(const BatchView& B, BatchCtl* c, cudaGraphConditionalHandle cond,
                          cudaStream_t s);
cudaError_t bs_loop_next(const BatchView& B, BatchCtl* c, int maxit, int iters_per_trip,
                         cudaGraphConditionalHandle cond, cudaStream_t s);
cudaError_t bs_sweep_end(BatchCtl* c, const BatchView& B, const BatchStepArrays& A, int ni,
                         bool comp, cudaGraphConditionalHandle cond, cudaStream_t s);
cudaError_t bs_sweep_next(BatchCtl* c, const BatchStepArrays& A, int ni, int max_sweeps,
                          cudaGraphConditionalHandle cond, cudaStream_t s);
cudaError_t bs_solve_end(BatchCtl* c, const BatchStepArrays& A, int ni, bool comp,
                         cudaStream_t s);
cudaError_t bs_nl_next(BatchCtl* c, int maxnlit, cudaStream_t s);
cudaError_t bs_finish(BatchCtl* c, const int* elem_err, cudaGraphConditionalHandle cond,
                      cudaStream_t s);

}  // namespace pm
