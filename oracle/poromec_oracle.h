/*
 * poromec_oracle.h -- CPU oracle for the poroMec Biot hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is a line-by-line C++ restatement
 * of the reference Fortran routines (lmn-labest/poroMec, mef/src Fortran files) that
 * the GPU library replaces.  It exists to check the GPU library (tests/,
 * __graft_entry__.smoke) and to time the reference algorithm on the host
 * cores (bench.py cpu_baseline / --impl reference).  Nothing in the product
 * path (poromec_gb300/) links, loads or calls it.
 *
 * Parity pin: the restatement is checked against the reference's own golden
 * runs (output/poro_mec/elastico/{hexa,tetra}: node histories printed with 10
 * decimals, neq/nad counts), converted into tests/golden/ by
 * tests/golden/make_golden.py.
 *
 * Conventions follow the Fortran call surface: arrays are column-major with
 * the leading dimension first (ix(nen+1,numel), id(ndf,nnode), u(ndf,nnode),
 * x(ndm,nnode), e(OR_PROP,numat)); node, element, material and equation
 * numbers are 1-based; ia is int64, ja int32 as in Datastruct.f.
 */
#ifndef POROMEC_ORACLE_H
#define POROMEC_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OR_PROP 15      /* e(prop,numat): e(1..7) used by the elastic Biot elements */
#define OR_NFLOAD 6     /* second dimension of fload(maxt, OR_NFLOAD, nloads) */

typedef struct or_handle_s* or_handle;

typedef struct {
  int iters;          /* Krylov iterations of the last solve */
  int nlit;           /* nonlinear iterations taken by the step */
  double conv;        /* tol * ||b||_M of the last solve */
  double xkx;         /* energy norm x.Kx logged by the solver */
  double res_u, res_p;/* last residual norms (cal_residuo_pm, stop_crit 2) */
} or_step_info;

/* Status codes (the reference calls stop_mef instead of returning). */
enum { OR_OK = 0, OR_E_ARG = 1, OR_E_DET = 2, OR_E_ZERO_DIAG = 3,
       OR_E_NOCONV = 4, OR_E_NLNOCONV = 5, OR_E_ELTYPE = 6 };

/* Mesh macro: numeqpmec2 (Numeq.f:86-151), graph_v1 + csria_v1/csrja_v1 +
 * sort_graph_csr (Graph.f:72, Csr.f:631-870,2149), element colouring.
 * id is the restraint flag array as read by constrainpmec (1 = prescribed).
 * num: node permutation (1-based, num(i) = i-th node visited), or NULL for
 * identity (reord false). */
/* reord (Reord.f:1-44): reverse Cuthill-McKee permutation of the node graph
 * of graph_v1 (Graph.f:72-133) by genrcm_v1 / fnroot_v1 / rcm_v1 /
 * rootls_v1 / degree_v1 (Reord.f:45-430); iperm(i) is the node visited
 * i-th (1-based), the num argument of or_create.  afl = 0: identity. */
int or_reord(int nnode, int numel, int nen, const int32_t* ix, int afl, int32_t* iperm);

int or_create(int nnode, int nnodev, int numel, int nen, int nenv, int ndf,
              const int32_t* ix, const int32_t* id, const int32_t* fnno,
              const double* x, int numat, const int32_t* ie, const double* e,
              const int32_t* num, or_handle* out);
void or_destroy(or_handle h);

int or_set_loads(or_handle h, const int32_t* eload, const int32_t* eloadp,
                 const int32_t* nload, const double* f, int nloads, int maxt,
                 const int32_t* load, const double* fload);
int or_set_env(or_handle h, const double* gravity, double dt, double t, int istep);
int or_set_state(or_handle h, const double* u, const double* u0, const double* dp);
int or_get_state(or_handle h, double* u, double* u0, double* dp);
/* Initial stress tx0(6,nnode) -> bstress0 via element isw=5 (Main.f:840-846). */
int or_set_initial_stress(or_handle h, const double* tx0);

int or_sizes(or_handle h, int* neq, int64_t* nad, int* numcolors);
int or_get_id(or_handle h, int32_t* id);
int or_get_csrd(or_handle h, int64_t* ia, int32_t* ja, double* ad, double* al);
int or_set_csrd_values(or_handle h, const double* ad, const double* al);

/* One element call elmlib_pm (Elmlib.f:1-214) for element nel (1-based):
 * u(nst), dp(nenv) local; returns s(nst,nst) column-major and p(nst). */
int or_element(or_handle h, int nel, int isw, const double* ul,
               const double* dpl, double* s, double* p);

/* pform_pm (Pform.f:1-429): element loop + csr assembly (Assbly.f:218-304).
 * u is the (ndf,nnode) nodal array passed as 'u' (u_n for isw 4, du for
 * isw 2); b (neq) is updated in place (b -= p) when rhs != 0; ad/al are
 * zeroed and assembled when lhs != 0.  nthreads > 1 runs the coloured
 * OpenMP loop (Pform.f:172-303). */
int or_pform(or_handle h, int isw, int lhs, int rhs, const double* u,
             double* b, int nthreads);

/* The element loop of or_pform restricted to elements [e_begin, e_end)
 * (1-based), without zeroing ad/al: a bounded timing sample of pform_pm. */
int or_pform_range(or_handle h, int isw, int lhs, int rhs, const double* u,
                   double* b, int nthreads, int e_begin, int e_end);

/* matvec_csrc_sym_pm (Matvec.f:1504-1598); nthreads > 1 runs the
 * row-partitioned variant with per-thread buffers (Matvec_omp.f:461-587). */
int or_matvec(or_handle h, const double* x, double* y, int nthreads);

/* tform_pm (Pform.f:433-640, element isw 3: Elmlib03.f:2206-2256 /
 * 440-495) and effective_stress (Pform.f:2487-2505): nodal total, Biot and
 * effective stress (6 per node) and Darcy flux (3 per node) at the vertices
 * from the current u and dp; mid-side nodes zero. */
int or_stress(or_handle h, double* tx, double* txb, double* txe, double* flux);
/* nodal porosity: initial_porosity (Pform.f:1343-1432) at creation, updated by
 * porosity_form (Pform.f:969-1175) at the end of every or_step */
/* GMRES(l) basis size (ngram, default 150, Main.f:274; solver file key
 * nkrylov, Rdata.f:3222-3229) used by solver 2 and by the rpsqmr fallback */
int or_set_nkrylov(or_handle h, int nkrylov);
int or_get_porosity(or_handle h, double* poro);
int or_set_porosity(or_handle h, const double* poro);

/* solv_pm (Solv.f:27-780): solver 1 = pcg (Iters.f:299-595), 2 = gmres2
 * (Iters.f:1411-1700, maxit = cycles of nkrylov iterations), 7 = pminres
 * (Iters.f:3987-4305, 10 restarts), 11 = rpsqmr (Iters.f:6100-6439), which
 * switches to gmres2 from x = 0 when it reaches maxit (Solv.f:765; info->iters
 * then counts both); precond 2 = 1/ad, 5 = |1/ad|
 * (Precond.f:22-79).  x is zeroed first (fnew = .true.). */
int or_solve(or_handle h, int solver, int precond, const double* b, double* x,
             double tol, int maxit, int nthreads, or_step_info* info);

/* One 'solv' macro step (Main.f:876-1123), state held in the handle. */
int or_step(or_handle h, int maxnlit, double tol, int stop_crit, int solver,
            int precond, double solvtol, int maxit, int nthreads,
            or_step_info* info);

/* Flop count of the element routines (isw=2) measured by instrumenting the
 * restatement: multiply-adds counted as 2 flops. */
double or_element_flops(int nen, int isw);

#ifdef __cplusplus
}
#endif
#endif
