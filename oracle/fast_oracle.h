/*
 * fast_oracle.h -- CPU oracle for the FastS structured solve step.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is a plain-C, FP64 restatement of
 * the FastS Fortran kernels named in each function comment.  It is used by
 * tests/, by __graft_entry__.smoke() and by bench.py's CPU-baseline leg as the
 * checker; it is never linked into, loaded by, or called from the product
 * path (fast_gb300/), which runs only on the GPU and fails loudly without it.
 *
 * Parity status: unpinned by reference data.  The reference ships no golden
 * vectors (its Data reference files are not distributed) and cannot be built here
 * (no Fortran compiler, Cassiopee absent).  Correspondence to the reference is
 * by line-by-line restatement of the cited routines plus the known-answer
 * tests in tests/ (free-stream preservation, conservation, Roe flux = physical
 * flux for equal states, LU-SGS against a dense solve of the same splitting).
 *
 * Conventions (identical to FastS): arrays are structure-of-arrays
 * rop[v*NDIMDX + l], l = inddm(i,j,k) - 1 with Fortran cell indices
 * i in [1-ng, ni+ng]; param_int / param_real use the FastS index map
 * (FastS/FastS/param_solver.h).  All integers are int64.
 */
#ifndef FAST_ORACLE_H
#define FAST_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* One zone as the step driver sees it (mirrors the pointer set that
 * FastS/FastS/Compute/computePT.cpp:44-500 extracts for each zone). */
typedef struct {
  const int64_t* param_int;
  const double*  param_real;
  double* ro;     /* time level n   (primitive: ro,u,v,w,T[,nutilde])     */
  double* ro_m1;  /* time level n-1                                        */
  double* ro_p1;  /* time level n+1 / RK work array (rop_tmp)              */
  double* xmut;   /* laminar (+turbulent) viscosity, NDIMDX; with SA        */
                  /* (IFLOW 3) followed by the wall distance, 2*NDIMDX     */
  double* drodm;  /* residual / increment, NEQ*NDIMDX                      */
  double* coe;    /* dt/vol, spectral radii, LU diagonal: NEQ_COE*NDIMDX   */
  const double* ti; const double* tj; const double* tk; const double* vol;
  double* rdm;    /* Newton residual per LU block: nssiter*neq*2*ndim_rdm  */
  double* wig;    /* senseur wiggle flags (KFLUDOM = 2), then o3sc weights  */
  double* cfl;    /* CFL max, min, mean of the last verified step (3)      */
} or_zone;

/* Interface transfer: rcv_zone cells <- dnr_zone cells.  types = NULL: the
 * 1-to-1 (type 0) copy.  Otherwise per point an interpolation type (0 / 1
 * one donor, 2 trilinear, 22 bilinear in (i, j), 3 and 5 tensor-product
 * Lagrange) whose molecule starts at dnr_idx, with its coefficients
 * concatenated in coefs (1, 1, 8, 4, 9, 15 per point). */
typedef struct {
  int64_t dnr_zone, rcv_zone, n;
  const int64_t* dnr_idx;  /* 0-based cell indices in the donor zone     */
  const int64_t* rcv_idx;  /* 0-based cell indices in the receiver zone  */
  const int64_t* types;
  const double* coefs;
} or_transfer;

int  or_version(void);
void or_set_threads(int n);
void or_set_lu_tiles(int n);

/* individual kernels (ind = 6 Fortran indices imin,imax,jmin,jmax,kmin,kmax) */
void or_invist(const int64_t* pi, const double* pr, const int64_t* ind,
               const double* rop, double* xmut);
/* SA/vispalart.for: SA eddy viscosity (IFLOW 3) */
void or_vispalart(const int64_t* pi, const double* pr, const int64_t* ind,
                  const double* rop, double* xmut);
/* SA/spsource_SA.for: SA source term into drodm(:,6), coe(:,6) when
 * implicit on the first sub-step; dist = wall distance (NDIMDX) */
void or_spsource(const int64_t* pi, const double* pr, int nitcfg, const int64_t* ind,
                 const double* rop, double* coe, const double* ti, const double* tj,
                 const double* tk, const double* vol, const double* dist, double* drodm);
void or_tstb3_global(const int64_t* pi, const double* pr, const int64_t* ind,
                     double* coe, const double* vol);
void or_tstb3c(const int64_t* pi, const double* pr, int first_it, const int64_t* ind,
               const double* rop, double* coe, const double* xmut,
               const double* ti, const double* tj, const double* tk, const double* vol);
void or_init_rhs(const int64_t* pi, int nitcfg, const int64_t* ind, double* drodm);
void or_flux(const int64_t* pi, const double* pr, const int64_t* ind,
             const double* rop, double* drodm, const double* xmut,
             const double* ti, const double* tj, const double* tk, const double* vol,
             const double* wig);
/* BC/correct_flux.for for wall BCs with the Roe scheme (lapply = 4) */
void or_correct_flux(const int64_t* pi, const double* pr, const double* rop, double* drodm,
                     const double* xmut, const double* ti, const double* tj, const double* tk,
                     const double* vol, const double* wig);
/* SENSOR/sciacovelli.for: o3sc shock-sensor weights wig[sl + d*NDIMDX + l]
 * (sl = 3*NDIMDX for the senseur scheme, else 0) */
void or_shock_sensor(const int64_t* pi, const double* pr, const int64_t* ind, const double* rop,
                     const double* ti, const double* tj, const double* tk, const double* vol,
                     double* wig);
/* SENSOR/wiggle2001.for: wig[d*NDIMDX + l] = 1 where a slope product of
 * any variable changes sign across the d-face of cell l, else 0 */
void or_wiggle(const int64_t* pi, const int64_t* ind, const double* rop, double* wig);
void or_core3ark3(const int64_t* pi, const double* pr, int nitcfg, const int64_t* ind,
                  double* rop_1, const double* rop, const double* drodm, const double* coe);
void or_core3as2(const int64_t* pi, const double* pr, int nitcfg, int first_it,
                 const int64_t* ind, const double* rop, const double* rop_n,
                 const double* rop_n1, double* drodm, const double* coe);
void or_invlu(const int64_t* pi, const double* pr, const int64_t* ind_lu,
              double* rotmp, double* rop_ssiter, const double* drodm_in,
              double* drodm_out, const double* ti, const double* tj, const double* tk,
              const double* coe, int mjrnewton);
void or_cprdu3s1(const int64_t* pi, int it_bloc, int nssiter,
                 const double* drodm, double* rdm);
void or_bc_zone(const int64_t* pi, const double* pr, const double* ti, const double* tj,
                const double* tk, int lrhs, double* rop);
/* cp_tijk.for + cp_vol.for: face normals * areas and volumes of a zone */
void or_metric(const int64_t* pi, const double* x, const double* y, const double* z, double* ti,
               double* tj, double* tk, double* vol);
void or_correct_coins(const int64_t* pi, const int64_t* ind, double* rop);
void or_transfers(or_zone* zones, const or_transfer* tr, int ntr, int use_p1);
double or_cfl_dt(const int64_t* pi, const double* pr, const double* rop,
                 const double* xmut, const double* ti, const double* tj,
                 const double* tk, const double* vol, double cfl);

/* The whole solve step: FastS/FastS/Compute/computePT.cpp:534-680 (loops
 * nit_c x nstep, sub-iteration flags, time-level rotation).  first_it is
 * read and updated (FastS HOOK["FIRST_IT"]).  Returns 0 on success. */
int or_compute(or_zone* zones, int nzones, const or_transfer* tr, int ntr,
               int nitrun, int nstep_deb, int nstep_fin, int nit_c,
               int modulo_verif, int* first_it);

/* display_ss_iteration reduction (FastS/FastS/DISPLAY/display_ss_iteration.cpp:112-145):
 * out[ne*nit + it] = L2, out[(neq+ne)*nit + it] = Loo. */
void or_residual_norms(const int64_t* pi, const double* pr, const double* rdm,
                       int nssiter, int it_bloc, double* out);

#ifdef __cplusplus
}
#endif
#endif
