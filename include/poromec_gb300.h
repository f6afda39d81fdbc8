/*
 * poromec_gb300.h -- C ABI of the GB300 (sm_103a) implementation of the
 * poroMec per-time-step Biot hot path.
 *
 * The reference (lmn-labest/poroMec, Fortran 77/90) has no FFI layer: its
 * "operator API" is the set of subroutines Main.f calls.  Each entry point
 * below replaces one of them and keeps its argument meaning; the Fortran
 * driver binds them with ISO_C_BINDING interfaces.
 *
 * Conventions
 *  - Arrays are the Fortran arrays, column-major, leading dimension first:
 *    ix(nen+1,numel), id(ndf,nnode), x(ndm,nnode), e(PM_PROP,numat),
 *    u(ndf,nnode).  Node, element, material and equation numbers are
 *    1-based; ia is int64 and ja int32 as in Datastruct.f.
 *  - Host pointers are read (or written) only during the call; device state
 *    lives in the handle.  Entry points with the _dev suffix take device
 *    pointers and a cudaStream_t (passed as void*).
 *  - Every call returns a pm_status.  Where the reference stops the program
 *    (stop_mef, Paralelo.f:1158-1165) the library returns an error instead.
 *  - One handle per host thread; each handle owns one CUDA stream.
 */
#ifndef POROMEC_GB300_H
#define POROMEC_GB300_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PM_PROP 15   /* rows of e(prop,numat); e(1..7) = E, nu, K_h, M, alpha, rho, rho_f */
#define PM_NFLOAD 6  /* second dimension of fload(maxt, PM_NFLOAD, nloads) */

typedef struct pm_handle_s* pm_handle;

typedef enum {
  PM_OK = 0,
  PM_E_ARG = 1,        /* invalid argument or inconsistent sizes */
  PM_E_DET = 2,        /* Jacobian determinant <= 1e-14 (jacob3d_m, Elmlib.f:2301) */
  PM_E_ZERO_DIAG = 3,  /* zero diagonal entry (pcg, Iters.f:401-406) */
  PM_E_NOCONV = 4,     /* Krylov solver reached maxit (Iters.f:499-501) */
  PM_E_NLNOCONV = 5,   /* nonlinear loop reached maxnlit (Main.f:1046-1053) */
  PM_E_ELTYPE = 6,     /* element type other than 15 (tetra10) / 17 (hexa20) */
  PM_E_CUDA = 7,       /* CUDA runtime error (message in pm_last_error) */
  PM_E_NOMEM = 8,      /* device allocation failed */
  PM_E_STATE = 9,      /* call out of order (e.g. solve before assembly) */
  PM_E_TOO_LARGE = 10  /* larger than the fixed scratch of pm_pcg_csrd_noalloc */
} pm_status;

typedef struct {
  int iters;      /* Krylov iterations of the last solve */
  int nlit;       /* nonlinear iterations of the step */
  int refine;     /* outer refinement sweeps (mixed precision), else 0 */
  double conv;    /* tol * ||b||_M of the last solve */
  double xkx;     /* x.Kx of the last solve (the reference's solver log) */
  double res_u;   /* last residual norms of cal_residuo_pm */
  double res_p;
} pm_step_info;

/* Precision modes (pm_set_precision). */
#define PM_FP64 0          /* plain FP64: values, vectors and arithmetic */
#define PM_FP32_REFINE 1   /* FP32 matrix values and FP32 SpMV in the inner PCG
                              of an FP64 iterative-refinement loop */
#define PM_FP32C_REFINE 2  /* matrix values as FP32 + an int8 relative correction
                              (5 bytes, 2^-32 relative) and compensated FP32
                              SpMV inside PCG / MINRES with FP64 vectors and
                              dots, in an FP64 iterative-refinement loop (outer
                              b - Ax in FP64) */

/* Mesh set-up: the 'mesh' macro (Main.f:481-870): equation numbering
 * numeqpmec2 (Numeq.f:86-151), CSRD structure datastruct_pm/csrstruct_pm
 * (Datastruct.f:1-278, Csr.f:18-307) and element colouring coloredmesh
 * (Colormsh.f:9-71).
 *  id:  restraint flags as read by 'constrainpmec' (1 = prescribed, 0 = free)
 *  fnno: 1 for vertex nodes (pressure dof), 0 for mid-side nodes
 *  ie:  element type per material: 17 hexa20 (nen 20), 15 tetra10 (nen 10)
 *  num: node visiting order (reord, Reord.f:1-44), NULL = natural order. */
int pm_mesh_create(int nnode, int nnodev, int numel, int nen, int nenv, int ndm,
                   int ndf, const int32_t* ix, const int32_t* id,
                   const int32_t* fnno, const double* x, int numat,
                   const int32_t* ie, const double* e, const int32_t* num,
                   pm_handle* out);

/* Node order of the 'mesh' macro: reord (Reord.f:1-44, Main.f:585-590), the
 * reverse Cuthill-McKee permutation of the node graph (genrcm_v1, fnroot_v1,
 * rcm_v1, Reord.f:45-430) that the reference computes before numbering the
 * equations when reordf is true, its default (Main.f:255).  ix(nen+1,numel)
 * as for pm_mesh_create; num(nnode) receives the 1-based node visited i-th,
 * to be passed as pm_mesh_create's num.  Host computation: no GPU needed. */
int pm_reord(int nnode, int numel, int nen, const int32_t* ix, int32_t* num);

/* A batch of independent meshes in one handle (the reference runs one mesh
 * per process; this has no single counterpart there).  The arrays are those
 * of pm_mesh_create for the union of the meshes, node ids and element
 * connectivities offset so that instance i owns nodes
 * inst_node_ptr[i] .. inst_node_ptr[i+1]-1 (0-based, inst_node_ptr[0] = 0,
 * inst_node_ptr[ninst] = nnode) and each element lies inside one instance.
 * pm_solve and pm_step then solve every instance independently, as if each
 * were its own handle (own PCG scalars, stopping test, nonlinear test), in
 * shared launches: PCG (solver 1) only, in PM_FP64 or PM_FP32C_REFINE.
 * pm_step on a batch captures the whole time step into one CUDA graph whose
 * loops (nonlinear iterations, refinement sweeps, PCG iterations) are decided
 * on the device, and launches it once; with PM_BATCH_HOST_STEP set in the
 * environment, on stop_crit other than 1 or 2, and on the first compensated
 * step (SpMV shape tuning) the host drives the same kernels instead. */
int pm_batch_create(int nnode, int nnodev, int numel, int nen, int nenv, int ndm, int ndf,
                    const int32_t* ix, const int32_t* id, const int32_t* fnno,
                    const double* x, int numat, const int32_t* ie, const double* e,
                    int ninst, const int32_t* inst_node_ptr, pm_handle* h);

/* Per instance of a batch: Krylov iterations of the last pm_solve or
 * pm_step (summed over its nonlinear iterations) and the nonlinear iteration
 * at which the last pm_step met its test; n >= ninst. */
int pm_get_batch_iters(pm_handle h, int* iters, int* nlit, int n);
void pm_destroy(pm_handle h);
const char* pm_last_error(pm_handle h);
const char* pm_status_string(int status);

/* Loads: eload/eloadp(7,numel) face load ids (elmtloads), nload(ndf,nnode)
 * nodal time-load ids, f(ndf,nnode) nodal values, load(3,nloads) = type,
 * number of components, number of time points; fload(maxt,PM_NFLOAD,nloads)
 * the load tables read by rload (Rdata.f:1487) and evaluated by tload
 * (Pload.f:220-377).  Any pointer may be NULL (= zero). */
int pm_set_loads(pm_handle h, const int32_t* eload, const int32_t* eloadp,
                 const int32_t* nload, const double* f, int nloads, int maxt,
                 const int32_t* load, const double* fload);
/* gravity(3), dt, t, istep: the transiente/gravity common blocks. */
int pm_set_env(pm_handle h, const double* gravity, double dt, double t, int istep);
/* Nodal state u(ndf,nnode), u0(ndf,nnode), dp(nnode); NULL leaves it unchanged. */
int pm_set_state(pm_handle h, const double* u, const double* u0, const double* dp);
int pm_get_state(pm_handle h, double* u, double* u0, double* dp);
/* Initial stress tx0(6,nnode): bstress0 by the element routine isw = 5
 * (initial_stress, Pform.f:679), added to b0 every step (Main.f:931-933). */
int pm_set_initial_stress(pm_handle h, const double* tx0);
int pm_set_precision(pm_handle h, int mode);
/* PM_FP32_REFINE: relative tolerance of each inner FP32-operator PCG sweep
 * (default 1e-5). */
int pm_set_refine(pm_handle h, double inner_tol);

int pm_get_sizes(pm_handle h, int* neq, int64_t* nad, int* numcolors,
                 int64_t* nnz_panel);
/* Equation numbers id(ndf,nnode) after numeqpmec2 (0 = no equation). */
int pm_get_id(pm_handle h, int32_t* id);
/* CSRD arrays in the reference layout: ia(neq+1) int64, ja(nad) int32,
 * ad(neq), al(nad) (strict lower triangle by rows).  Any pointer may be NULL. */
int pm_get_csrd(pm_handle h, int64_t* ia, int32_t* ja, double* ad, double* al);

/* pform_pm (Pform.f:1-429): element loop plus assembly.
 *  isw 2: element matrix and internal force p = s.u; lhs assembles K
 *         (ad/al zeroed first), rhs does b -= p.   u = du(ndf,nnode).
 *  isw 4: body forces, previous-state internal forces and face loads, b -= p.
 *         u = u(n) (ndf,nnode); dp taken from the handle state.
 *  b(neq) is read and written (host array). */
int pm_assemble(pm_handle h, int isw, int lhs, int rhs, const double* u, double* b);

/* matvec_csrc_sym_pm (Matvec.f:1504-1598): y = (D + L + L^T) x with the
 * assembled matrix.  x, y host arrays of length neq.  Under PM_FP32C_REFINE
 * the product is the compensated FP32 operator of the solver. */
int pm_spmv(pm_handle h, const double* x, double* y);

/* solv_pm (Solv.f:27-780): solver 1 = PCG (Iters.f:299-595),
 * 2 = GMRES(l) (gmres2, Iters.f:1411-1700; FP64 only; maxit counts cycles of
 * nkrylov iterations, see pm_set_nkrylov),
 * 7 = preconditioned MINRES (Iters.f:3987-4305, 10 restarts),
 * 11 = rpsqmr (Iters.f:6100-6439, the reference's default; PM_FP64 or
 * PM_FP32C_REFINE; where
 * it does not converge in maxit it switches to GMRES(l) from x = 0 with maxit
 * cycles, Solv.f:765, and info->iters counts both); precond 2 = diag 1/ad,
 * 5 = |1/ad|
 * (Precond.f:22-79).  x is set to 0 first (fnew = .true.).  b, x host arrays
 * of length neq. */
int pm_solve(pm_handle h, int solver, int precond, const double* b, double* x,
             double tol, int maxit, pm_step_info* info);

/* GMRES(l) basis size (ngram, default 150, Main.f:274; solver-file key
 * nkrylov, Rdata.f:3222-3229).  The (nkrylov + 1) x neq basis is allocated on
 * the first GMRES solve. */
int pm_set_nkrylov(pm_handle h, int nkrylov);

/* One 'solv' macro step (Main.f:876-1123) on the device-resident state:
 * pload_pm, isw 4 loop, predictor, nonlinear loop (isw 2, residual check
 * cal_residuo_pm with stop_crit 1/2, solve, delta_update_pm), update_res_v2.
 * reassemble = 0 keeps K from the previous step (valid for linear elastic
 * elements with unchanged dt and materials); the reference reassembles. */
int pm_step(pm_handle h, int maxnlit, double tol, int stop_crit, int solver,
            int precond, double solvtol, int maxit, int reassemble,
            pm_step_info* info);

/* Device-pointer variants (cudaStream_t passed as void*; NULL = the handle's
 * stream).  Vectors are FP64 of length neq in equation order. */
int pm_spmv_dev(pm_handle h, const double* d_x, double* d_y, void* stream);
int pm_solve_dev(pm_handle h, int solver, int precond, const double* d_b,
                 double* d_x, double tol, int maxit, pm_step_info* info,
                 void* stream);
/* The reference CSRD layout on the device, standalone (no handle):
 * y = (D + L + L^T) x for ia(neq+1) int64 1-based, ja(nad) int32 1-based. */
int pm_matvec_csrd_dev(int neq, const int64_t* d_ia, const int32_t* d_ja,
                       const double* d_ad, const double* d_al,
                       const double* d_x, double* d_y, void* stream);

/* Solve without device allocation.  No counterpart in the reference: it
 * serves callers that must not allocate device memory while they solve (a
 * driver whose memory belongs to its own arena, a framework that owns the
 * device pool, a latency-bound step).  It runs the PCG of pm_solve (solver 1,
 * precond 2: m = 1/ad) on the reference CSRD arrays the caller already holds
 * on the device (d_ia int64 1-based, d_ja int32 1-based, d_ad, d_al), with
 * right-hand side d_b and solution d_x (set to 0 first), length neq.  All
 * scratch comes from one array compiled into the library: each GPU that
 * loads the library holds about 10.5 MB for it until the process exits, and
 * neq above PM_NOALLOC_MAX_NEQ returns PM_E_TOO_LARGE.  The first call on a
 * device looks up that array's device address, so make it before any stream
 * capture.  Calls share the array and it keeps the last call's contents:
 * two calls that run at the same time on one GPU (two streams, two host
 * threads) race, so serialise them.  stream may be NULL (legacy stream).
 * The matrix is scattered into the scratch with atomic adds, so unlike the
 * rest of the library its results can differ in the last bits from run to
 * run (within the solve tolerance).  The looked-up address is kept for the
 * life of the process: do not call it after cudaDeviceReset on that device. */
#define PM_NOALLOC_MAX_NEQ 262144
int pm_pcg_csrd_noalloc(int neq, const int64_t* d_ia, const int32_t* d_ja,
                        const double* d_ad, const double* d_al, const double* d_b,
                        double* d_x, double tol, int maxit, int* iters, void* stream);

/* Autotuner of the PM_FP32C_REFINE SpMV (no counterpart in the reference,
 * whose SpMV has no tunable shape): builds the compensated values of the
 * assembled matrix if needed, times the kernel shapes (8, 16 or 32 lanes per
 * node x 1, 2 or 4 columns per lane and trip) on it and keeps the fastest;
 * *shape receives its code, 10 * (0, 1, 2 for 8, 16, 32 lanes) + columns.
 * The first compensated solve or product runs it implicitly. */
int pm_tune_spmv(pm_handle h, int* shape);

/* tform_pm (Pform.f:433-640) with the element stress pass isw 3
 * (Elmlib03.f:2206-2256 hexa20, 440-495 tetra10) and effective_stress
 * (Pform.f:2487-2505): from the current state, per node (6, nnode) the total
 * stress, the Biot effective stress (total + alpha p) and the effective stress
 * (total + p), and (3, nnode) the Darcy flux; vertex nodes average the values
 * of the elements that share them, mid-side nodes are zero.  The '_dev' form
 * takes device arrays (stream as pm_spmv_dev). */
/* Nodal porosity (nnode; vertex nodes carry it): initial_porosity
 * (Pform.f:1343-1432, material column 8 averaged over the elements sharing a
 * vertex) at creation; every pm_step adds porosity_form's change
 * (Pform.f:969-1175, Elmlib03.f:2605-2631 isw 7): the average over the
 * elements at the vertex of alpha tr(eps(du)) + dp/M of the step's increments. */
int pm_get_porosity(pm_handle h, double* poro);
int pm_set_porosity(pm_handle h, const double* poro);
int pm_stress(pm_handle h, double* tx, double* txb, double* txe, double* flux);
int pm_stress_dev(pm_handle h, double* d_tx, double* d_txb, double* d_txe, double* d_flux,
                  void* stream);

/* Material table (e, PM_PROP per material) replaced, same numat as at
 * creation; the next step re-assembles.  With one material per element
 * (numat = numel) this sets per-element parameters. */
int pm_set_materials(pm_handle h, const double* e, int numat);

/* Adjoint of the time-stepped solve (no counterpart in the reference).  A
 * step solves K du = F - A s - g0 for the previous state s = (u, dp), with
 * A s = [Kuu u_u + Kup dp ; Kpp_perm u_p] and g0 = [-body ; G_k] (the
 * previous-state terms of pform isw 4), then s += (du, du_p).  The reverse
 * sweep of a misfit J(u_N) is, for n = N..1, with mu = dJ/du and nu = dJ/ddp
 * in equation space (mu_N from J, nu_N = 0):
 *   lam_n = K^-1 (mu_n + nu_n)                       (pm_solve_dev: K = K^T)
 *   mu_{n-1} = mu_n - [Kuu lam_u ; Kpp_perm lam_p],  nu_{n-1} = nu_n - Kpu lam_u
 *   grad += contractions of lam_n with the parameter derivatives
 * Device pointers; stream NULL = the handle's stream (a non-NULL stream is
 * synchronised before return).  The matrix must be assembled for the step's
 * dt and materials. */
/* mu -= [Kuu lam_u ; Kpp_perm lam_p], nu -= Kpu lam_u (lam, mu, nu: neq) */
int pm_adjoint_apply_dev(pm_handle h, const double* d_lam, double* d_mu, double* d_nu,
                         void* stream);
/* grad[3 e + {0, 1, 2}] += d/dlog E, d/dlog k, d/dlog M of the element e
 * contribution lam^T (F - A s - g0 - K du): -lam_u^T Kuu u_n,
 * -lam_p^T (Kpp_perm p_n + G_k), lam_p^T Kstor du_p (Kstor = -(1/M) int NN),
 * with u_n = s + du the step's new state and du its increment, both in the
 * nodal layout (4 per node); lam: neq; grad: 3 numel (per element when
 * numat = numel, each element's material parameters). */
int pm_adjoint_grad_dev(pm_handle h, const double* d_lam, const double* d_un,
                        const double* d_dun, double* d_grad, void* stream);

/* Timing of the last pm_step phases in milliseconds (CUDA events):
 * [0] pload+isw4, [1] assembly (isw2 lhs), [2] isw2 residual passes,
 * [3] solve (a batch step run as one graph: the whole step, [0]-[2] are 0),
 * [4] Krylov iterations of all the solves of the last single-mesh
 * pm_step (the step's info->iters counts its last solve only; 0 for a batch),
 * [5] device time of the last Krylov solve,
 * [6] Krylov iterations of the last solve, [7] kernels launched by the step. */
int pm_get_timers(pm_handle h, double* t, int n);

/* ---- input decks ---------------------------------------------------------
 * pm_deck_read parses a deck of the reference: the macro program of Main.f
 * (config, pcg / solver, gravity, mesh, setpnode, maxnlit / nl, dt, loop,
 * solv, next, pnup, pnsf, pgeo, stop) and the mesh macro of rdat_pm
 * (Rdata.f:1-1037: parameters, materials, fmaterials, hexa8 / tetra4 /
 * hexa20 / tetra10, coordinates, constrainpmec, nodalforces, elmtloads,
 * elmtpresloads, nodalloads, loads, initialpres, initialdisp, initialstress,
 * hydrostatic, hydrostress, insert, return, end).  Linear elements with
 * maxno 20 / 10 become hexa20 / tetra10 by mk_elconn_quad_v1
 * (Adjacency.f:583-700), with the restraints, forces and initial stresses of
 * the mid-side nodes from their edge's vertices (Rdata.f:2337-2544).  Older
 * decks (element codes 7 / 6, "pcg", "maxnlit", inline type-40 loads) are
 * read too.  Files named in the deck are relative to its directory.  On
 * failure pm_deck_error() gives the message with file and line (per thread;
 * also for the output files of pm_deck_run and the writers; a failure of a
 * library call inside pm_deck_run is in pm_last_error(h)). */
typedef struct pm_deck_s* pm_deck;
int pm_deck_read(const char* path, pm_deck* d);
const char* pm_deck_error(void);
void pm_deck_free(pm_deck d);
/* Scalars by name: nnode nnodev numel numat nen nenv nloads maxt fstress0
 * mk_quad, reord (1 unless the config block sets it false), the settings in
 * force at the first solv (solver precond maxit
 * solvtol maxnlit tol stop_crit nkrylov dt gravity_x gravity_y gravity_z),
 * nprint, nops, unknown_macros. */
int pm_deck_value(pm_deck d, const char* name, double* v);
/* Arrays owned by the deck, in the layouts of pm_mesh_create / pm_set_loads:
 * int32 ix id nload eload eloadp fnno load print_nodes; double e x f u0 tx0
 * fload (u0 after boundc and bound_nodalloads; tx0(6, nnode)). */
int pm_deck_int_array(pm_deck d, const char* name, const int32_t** p, int64_t* n);
int pm_deck_real_array(pm_deck d, const char* name, const double** p, int64_t* n);
/* A handle with the deck's mesh, loads, gravity, dt, initial state and
 * initial stress; the equations are numbered in pm_reord's node order unless
 * the deck's config block sets reord false (the reference's default is
 * true, Main.f:255). */
int pm_deck_create(pm_deck d, pm_handle* h);
/* Runs the macro program on h (from pm_deck_create): solv steps with the
 * settings in force, pnup / pnsf writing <prefix>_<up|stress|stressE|stressB|
 * flux|poro>_node_<n>.txt for the setpnode nodes (printnode, Pdata.f:733-790;
 * pnsf adds the initial stress as Main.f does), pgeo and pres writing the VTK
 * files of pm_deck_write_geo / pm_deck_write_res (pres with every field), and
 * the solver log <prefix>_log_1.txt (one line per solv: iterations, energy
 * norm x.Kx and tolerance in D20.10, seconds; the layout of the shipped golden
 * logs) and, at the end, <prefix>_t_1.txt (phase seconds ELMT / TFORM / SOLVR /
 * TOTAL and the sizes neq, nad, nnode, numel, colors, as write_log_file).  format 0 writes printnode's
 * (i9,10e18.10) rows; format 1 the column layout of the golden runs shipped
 * with the reference (i9, f30.6, f30.10 ...).  *nsteps = steps run. */
int pm_deck_run(pm_deck d, pm_handle h, const char* prefix, int format, int* nsteps);
/* Legacy ASCII VTK (Vtk.f, Write_vtk.f).  pm_deck_write_geo: the mesh as
 * read (write_mesh_geo_pm, the pgeo macro), <prefix>_bc.vtk: node ids and one
 * field per node macro of the deck (restraint flags, forces, nodal loads,
 * initial pressure, initial stress) in read order, cell materials, ids and
 * element loads; quad = 0 writes the vertex mesh of a linear deck.
 * pm_deck_write_res: the state of h (write_mesh_res_pm, the pres macro),
 * <prefix>_istep_<istep>.vtk: desloc, pressao, and by the bits of fields
 * 1 deltaPressao, 2 totalStress, 4 terzaghiStress, 8 BiotStress,
 * 16 darcyFlux, 32 porosity; mid-side pressures are the edge averages. */
int pm_deck_write_geo(pm_deck d, const char* prefix, int quad);
int pm_deck_write_res(pm_deck d, pm_handle h, const char* prefix, int istep, double t, int quad,
                      int fields);

#ifdef __cplusplus
}
#endif
#endif
