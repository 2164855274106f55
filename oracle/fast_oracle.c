/*
 * fast_oracle.c -- CPU oracle (FP64 restatement) of the FastS solve step.
 *
 * TEST INFRASTRUCTURE ONLY: loaded by tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py as the checker.  The product path never loads
 * or calls it.  Parity status: unpinned by reference data (the reference ships
 * no golden vectors and cannot be compiled here); see fast_oracle.h.
 *
 * Every routine restates the FastS Fortran routine cited in its comment
 * (paths relative to the Fast/ project directory).  Compiled with
 * -ffp-contract=off so that every multiply and add rounds separately, and
 * written with the reference's left-to-right evaluation order, so that the
 * result is the reference's arithmetic with one thread and one cache block
 * per zone (cache_blocking_I/J/K >= zone size).  With FastS's default cache
 * blocking the only difference is the order of the last two face-flux
 * summands of cells on a cache-block boundary (one rounding of drodm).
 */
#include "fast_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ---- FastS/FastS/param_solver.h index map (the subset used here) ---- */
enum { NIJK = 0, NIJK_MTR = 5, NIJK_XYZ = 10, IJKV = 20, ITYPZONE = 25, IFLOW = 27, ILES = 28,
       ITYPCP = 29, SIZE_SSDOM = 30, KFLUDOM = 33, LALE = 34, NEQ = 36,
       NEQ_IJ = 37, NEQ_K = 38, NEQ_COE = 39, NDIMDX = 41, NDIMDX_MTR = 43,
       DTLOC = 46, RK = 52, LEVEL = 53, EXPLOC = 54, NSSITER = 58, SLOPE = 64,
       PT_BC = 70, NB_RELAX = 71, LU_MATCH = 75, SENSORTYPE = 85 };
enum { DTC = 0, GAMMA = 1, CVINF = 2, ROINF = 3, PINF = 4, VINF = 5, TINF = 6,
       PRANDT = 10, XMUL0 = 11, TEMP0 = 12, CS = 13, EPSI_NEWTON = 14,
       PSIROE = 34, WIG_AMP = 72, VXINF = 19, VYINF = 20, VZINF = 21,
       RONUTILDEINF = 8, SA_RATIOM_R = 18, PRANDT_TUR = 38, CFL = 15 };
enum { BC_TYPE = 0, BC_IDIR = 1, BC_FEN = 2, BC_NBDATA = 8 };

#define OMAX(a, b) ((a) > (b) ? (a) : (b))
#define OMIN(a, b) ((a) < (b) ? (a) : (b))
/* Fortran SIGN(a,b): |a| with the sign of b */
static inline double fsign(double a, double b) { return copysign(fabs(a), b); }

static int g_threads = 1;
static int g_lu_tiles = 1;
void or_set_threads(int n) { g_threads = n > 0 ? n : 1; }
/* LU-SGS tiles (FastS with OMP_NUM_THREADS = n: one LU block per thread,
 * block-Jacobi between them, lhs.cpp ipt_shift_lu).  1 = one tile per zone. */
void or_set_lu_tiles(int n) { g_lu_tiles = n > 0 ? n : 1; }
int or_version(void) { return 3; }

/* formule_param.h: inddm (returned 0-based) */
static inline int64_t inddm(const int64_t* p, int64_t i, int64_t j, int64_t k) {
  return (i + p[NIJK + 3] - 1) + (j + p[NIJK + 3] - 1) * p[NIJK] +
         (k + p[NIJK + 4] - 1) * p[NIJK] * p[NIJK + 1];
}
/* formule_mtr_param.h: indmtr (returned 0-based) */
static inline int64_t indmtr(const int64_t* p, int64_t i, int64_t j, int64_t k) {
  return (i + p[NIJK_MTR + 3] - 1) * p[NIJK_MTR] + (j + p[NIJK_MTR + 3] - 1) * p[NIJK_MTR + 1] +
         (k + p[NIJK_MTR + 4] - 1) * p[NIJK_MTR + 2];
}

/* ======================================================================
 * invist -- FastS/FastS/Compute/invist.for:28-36 (Sutherland law)
 * ====================================================================== */
void or_invist(const int64_t* pi, const double* pr, const int64_t* ind,
               const double* rop, double* xmut) {
  double cmus1 = pr[CS];
  double temp01 = 1. / pr[TEMP0];
  double coesut = pr[XMUL0] * (1. + cmus1 * temp01) * sqrt(temp01);
  int64_t v5 = 4 * pi[NDIMDX];
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int64_t k = ind[4]; k <= ind[5]; k++)
    for (int64_t j = ind[2]; j <= ind[3]; j++)
      for (int64_t i = ind[0]; i <= ind[1]; i++) {
        int64_t l = inddm(pi, i, j, k);
        double t1 = rop[l + v5];
        xmut[l] = coesut * sqrt(t1) * t1 / (t1 + cmus1);
      }
}

/* ======================================================================
 * Spalart-Allmaras -- constants of FastS/FastS/param_solver.h:315-327
 * ====================================================================== */
#define SA_CKARM 0.41
#define SA_CB1 0.1355
#define SA_CB2 0.622
#define SA_CV1 357.911
#define SA_CW2 0.3
#define SA_CW3 64.
#define SA_CW4 0.21
#define SA_CW5 1.5
#define SA_SIGMA (2. / 3.)
#define SA_CROT 2.0

/* mulam.for: Sutherland law in the form the SA routines use */
static inline double sa_mulam(double coesut, double temp01, double cmus1, double t) {
  return coesut * sqrt(t * temp01) / (1. + cmus1 / t);
}
/* SA/chi.for (anutild = max(nutilde, 1e-27), chi = max(anutild*ro/mu, 1e-7)) */
static inline double sa_fv1(double s) { return 1. / (1. + SA_CV1 / (s * s * s)); }

/* SA/vispalart.for (SA branch, SA_IDES <= 1) with mulam.for, chi.for and
 * xmut.for: mu_t = ro nutilde fv1(chi), clipped to [0, ratiom mu]. */
void or_vispalart(const int64_t* pi, const double* pr, const int64_t* ind,
                  const double* rop, double* xmut) {
  const double cmus1 = pr[CS], temp01 = 1. / pr[TEMP0];
  const double coesut = pr[XMUL0] * (1. + cmus1 * temp01);
  const int64_t nd = pi[NDIMDX];
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int64_t k = ind[4]; k <= ind[5]; k++)
    for (int64_t j = ind[2]; j <= ind[3]; j++)
      for (int64_t i = ind[0]; i <= ind[1]; i++) {
        int64_t l = inddm(pi, i, j, k);
        double amulam = sa_mulam(coesut, temp01, cmus1, rop[l + 4 * nd]);
        double anulam = rop[l] / amulam;
        double anutild = OMAX(rop[l + 5 * nd], 1.e-27);
        double chi = OMAX(anutild * anulam, 1.e-7);
        double fvv1 = sa_fv1(chi);
        double amut = rop[l] * anutild * fvv1;
        double xmuprov = OMAX(amut, 0.);
        xmut[l] = amulam + OMIN(xmuprov, pr[SA_RATIOM_R] * amulam);
      }
}

/* SA/spsource_SA.for with sourceSA_grad_3dcart.for / sourceSA_grad_3d.for
 * (velocity and nutilde gradients from face sums), sourceSA_prod_dest.for
 * (production, destruction, cross-diffusion) and sourceSA_LU.for (implicit:
 * coe6 = coe5 - min(dS/d(ro nutilde), 0) coe1 on the first sub-step).
 * The reference also evaluates the term on the first ghost ring
 * (ind_ssa = [0, n+1]); those ghost residuals are never read, so the
 * interior range is enough.  dist = wall distance (xmut(1+NDIMDX) there).
 * rot_corr / low_re = param_int SA_ROT_CORR / SA_LOW_RE. */
void or_spsource(const int64_t* pi, const double* pr, int nitcfg, const int64_t* ind,
                 const double* rop, double* coe, const double* ti, const double* tj,
                 const double* tk, const double* vol, const double* dist_in, double* drodm) {
  const int64_t nd = pi[NDIMDX], ndm = pi[NDIMDX_MTR];
  const double sw_low_re = (double)pi[130], sw_rot = (double)pi[131];
  const double cmus1 = pr[CS], temp01 = 1. / pr[TEMP0];
  const double coesut = pr[XMUL0] * (1. + cmus1 * temp01);
  const double c1 = SA_CB2 / SA_SIGMA;
  const double cw1 = (SA_CB1 / SA_CKARM / SA_CKARM) + (1. + SA_CB2) / SA_SIGMA;
  const int typ = (int)pi[ITYPZONE];
  const int lu = pi[ITYPCP] <= 1 && nitcfg <= 1;
  const int64_t incj = pi[NIJK], inck = pi[NIJK] * pi[NIJK + 1];
  const int64_t mi = pi[NIJK_MTR], mj = pi[NIJK_MTR + 1], mk = pi[NIJK_MTR + 2];
  const double *r_ = rop, *nu_ = rop + 5 * nd;
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int64_t k = ind[4]; k <= ind[5]; k++)
    for (int64_t j = ind[2]; j <= ind[3]; j++)
      for (int64_t i = ind[0]; i <= ind[1]; i++) {
        const int64_t l = inddm(pi, i, j, k);
        const int64_t lt = typ == 2 ? 0 : indmtr(pi, i, j, k);
        const int64_t l1 = l + 1, l2 = l - 1, l3 = l + incj, l4 = l - incj, l5 = l + inck, l6 = l - inck;
        const double xvol = 0.5 / vol[lt];
        double g[3][3], gn[3], gr[3];   /* g[v][x]: d(u,v,w)/dx, gn: d nutilde, gr: d ro nutilde */
        double rot, St, anvisc;
        if (typ == 3) {   /* sourceSA_grad_2d.for: i and j faces, u and v */
          const double* T[2] = {ti, tj};
          const int64_t lt1[2] = {lt + mi, lt + mj};
          double t0[2][2], t1[2][2];
          for (int x = 0; x < 2; x++)
            for (int d = 0; d < 2; d++) {
              t0[x][d] = T[d][lt + x * ndm];
              t1[x][d] = T[d][lt1[d] + x * ndm];
            }
          for (int v = 0; v < 3; v++) {
            const double* q = v < 2 ? rop + (v + 1) * nd : nu_;
            double u1 = (q[l] + q[l2]), u2 = (q[l] + q[l3]), u3 = (q[l] + q[l1]);
            double u4 = (q[l] + q[l4]);
            double* o = v < 2 ? g[v] : gn;
            for (int x = 0; x < 2; x++)
              o[x] = (u3 * t1[x][0] - u1 * t0[x][0] + u2 * t1[x][1] - u4 * t0[x][1]);
          }
          double a = nu_[l] * r_[l];
          double u1 = a + nu_[l2] * r_[l2], u2 = a + nu_[l3] * r_[l3], u3 = a + nu_[l1] * r_[l1];
          double u4 = a + nu_[l4] * r_[l4];
          for (int x = 0; x < 2; x++)
            gr[x] = (u3 * t1[x][0] - u1 * t0[x][0] + u2 * t1[x][1] - u4 * t0[x][1]);
          const double rotz = g[1][0] - g[0][1];
          rot = fabs(rotz) * xvol;
          const double S11 = g[0][0], S22 = g[1][1], S12 = 0.5 * (g[0][1] + g[1][0]);
          St = S11 * S11 + S22 * S22 + 2. * (S12 * S12);
          St = sqrt(2. * St) * xvol;
          anvisc = c1 * (gn[0] * gr[0] + gn[1] * gr[1]) * xvol * xvol;
        } else {
        if (typ == 2) {   /* sourceSA_grad_3dcart.for */
          const double tix = ti[0], tjy = tj[0], tkz = tk[0];
          for (int v = 0; v < 3; v++) {
            const double* q = rop + (v + 1) * nd;
            double u1 = (q[l] + q[l2]), u2 = (q[l] + q[l3]), u3 = (q[l] + q[l1]);
            double u4 = (q[l] + q[l4]), u5 = (q[l] + q[l5]), u6 = (q[l] + q[l6]);
            g[v][0] = (u3 - u1) * tix;
            g[v][1] = (u2 - u4) * tjy;
            g[v][2] = (u5 - u6) * tkz;
          }
          {
            const double* q = nu_;
            double u1 = (q[l] + q[l2]), u2 = (q[l] + q[l3]), u3 = (q[l] + q[l1]);
            double u4 = (q[l] + q[l4]), u5 = (q[l] + q[l5]), u6 = (q[l] + q[l6]);
            gn[0] = (u3 - u1) * tix;
            gn[1] = (u2 - u4) * tjy;
            gn[2] = (u5 - u6) * tkz;
          }
          {
            double a = nu_[l] * r_[l];
            double u1 = a + nu_[l2] * r_[l2], u2 = a + nu_[l3] * r_[l3], u3 = a + nu_[l1] * r_[l1];
            double u4 = a + nu_[l4] * r_[l4], u5 = a + nu_[l5] * r_[l5], u6 = a + nu_[l6] * r_[l6];
            gr[0] = (u3 - u1) * tix;
            gr[1] = (u2 - u4) * tjy;
            gr[2] = (u5 - u6) * tkz;
          }
        } else {          /* sourceSA_grad_3d.for */
          const double* T[3] = {ti, tj, tk};
          const int64_t lt1[3] = {lt + mi, lt + mj, lt + mk};
          /* t0[x][d] = t_d(lt, x), t1[x][d] = t_d(lt + inc_d, x) */
          double t0[3][3], t1[3][3];
          for (int x = 0; x < 3; x++)
            for (int d = 0; d < 3; d++) {
              t0[x][d] = T[d][lt + x * ndm];
              t1[x][d] = T[d][lt1[d] + x * ndm];
            }
          for (int v = 0; v < 4; v++) {
            const double* q = v < 3 ? rop + (v + 1) * nd : nu_;
            double u1 = (q[l] + q[l2]), u2 = (q[l] + q[l3]), u3 = (q[l] + q[l1]);
            double u4 = (q[l] + q[l4]), u5 = (q[l] + q[l5]), u6 = (q[l] + q[l6]);
            double* o = v < 3 ? g[v] : gn;
            for (int x = 0; x < 3; x++)
              o[x] = (u3 * t1[x][0] - u1 * t0[x][0] + u2 * t1[x][1] - u4 * t0[x][1] +
                      u5 * t1[x][2] - u6 * t0[x][2]);
          }
          double a = nu_[l] * r_[l];
          double u1 = a + nu_[l2] * r_[l2], u2 = a + nu_[l3] * r_[l3], u3 = a + nu_[l1] * r_[l1];
          double u4 = a + nu_[l4] * r_[l4], u5 = a + nu_[l5] * r_[l5], u6 = a + nu_[l6] * r_[l6];
          for (int x = 0; x < 3; x++)
            gr[x] = (u3 * t1[x][0] - u1 * t0[x][0] + u2 * t1[x][1] - u4 * t0[x][1] +
                     u5 * t1[x][2] - u6 * t0[x][2]);
        }
        const double dudx = g[0][0], dudy = g[0][1], dudz = g[0][2];
        const double dvdx = g[1][0], dvdy = g[1][1], dvdz = g[1][2];
        const double dwdx = g[2][0], dwdy = g[2][1], dwdz = g[2][2];
        const double rotx = dwdy - dvdz, roty = dudz - dwdx, rotz = dvdx - dudy;
        rot = sqrt(rotx * rotx + roty * roty + rotz * rotz) * xvol;
        const double S11 = dudx, S22 = dvdy, S33 = dwdz;
        const double S12 = 0.5 * (dudy + dvdx), S13 = 0.5 * (dudz + dwdx), S23 = 0.5 * (dvdz + dwdy);
        St = S11 * S11 + S22 * S22 + S33 * S33 + 2. * (S12 * S12) + 2. * (S13 * S13) +
             2. * (S23 * S23);
        St = sqrt(2. * St) * xvol;
        anvisc = c1 * (gn[0] * gr[0] + gn[1] * gr[1] + gn[2] * gr[2]) * xvol * xvol;
        }
        /* mulam.for, chi.for */
        const double amulam = sa_mulam(coesut, temp01, cmus1, rop[l + 4 * nd]);
        const double anulam = r_[l] / amulam;
        const double anutild = OMAX(nu_[l], 1.e-27);
        const double chi = OMAX(anutild * anulam, 1.e-7);
        /* sourceSA_prod_dest.for */
        const double f1 = sa_fv1(chi);
        const double f2 = 1. - chi / (1. + chi * f1);
        const double dist = OMAX(dist_in[l], 1.e-27);
        double stild = rot + (anutild * f2) / (SA_CKARM * SA_CKARM * dist * dist);
        stild = stild + sw_rot * SA_CROT * OMIN(0.00000000000000000001, St - rot);
        const double prod = r_[l] * SA_CB1 * stild * anutild;
        stild = OMAX(stild, 0.00000000000000000001);
        double r = anutild / (stild * SA_CKARM * SA_CKARM * dist * dist);
        r = OMIN(r, 10.);
        const double r5 = r * r * r * r * r - 1.;
        double gg = r * (1. + SA_CW2 * r5);
        const double lre = 1. + chi / 40.;
        const double cw2_lre = SA_CW4 + SA_CW5 / (lre * lre);
        gg = sw_low_re * r * (1. + cw2_lre * r5) + (1. - sw_low_re) * gg;
        /* fw(g) = g ((1 + cw3) / (g^6 + cw3))^(1/6); g**6 is expanded by
         * the Fortran compiler as (g^3)^2 with g^3 = g^2 g */
        const double g3 = gg * gg * gg, g6 = g3 * g3;
        const double fwg = gg * pow((1. + SA_CW3) / (g6 + SA_CW3), 1. / 6.);
        const double destruc = r_[l] * cw1 * fwg * (anutild / dist) * (anutild / dist);
        const double tsource = (prod + anvisc - destruc);
        if (lu) {         /* sourceSA_LU.for */
          const double tsourceb = prod - destruc;
          double amutild = anutild * r_[l];
          amutild = OMAX(amutild, 0.0000000000000001);
          const double tsourcenu = vol[lt] * tsourceb / amutild;
          coe[l + 5 * nd] = coe[l + 4 * nd] - OMIN(tsourcenu, 0.) * coe[l];
        }
        drodm[l + 5 * nd] = drodm[l + 5 * nd] + vol[lt] * tsource;
      }
}

/* ======================================================================
 * tstb3_global -- FastS/FastS/Compute/tstb3_global.for:43-66 (coe1 = dt/vol)
 * ====================================================================== */
void or_tstb3_global(const int64_t* pi, const double* pr, const int64_t* ind,
                     double* coe, const double* vol) {
  double volinv = pr[DTC] / vol[0];
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int64_t k = ind[4]; k <= ind[5]; k++)
    for (int64_t j = ind[2]; j <= ind[3]; j++)
      for (int64_t i = ind[0]; i <= ind[1]; i++) {
        int64_t l = inddm(pi, i, j, k);
        if (pi[ITYPZONE] != 2) coe[l] = pr[DTC] / vol[indmtr(pi, i, j, k)];
        else coe[l] = volinv;
      }
}

/* ======================================================================
 * tstb3c -- FastS/FastS/Compute/tstb3c.for:121-171 (3d general),
 *           :300-345 (3d cartesian), :346-390 (2d): spectral radii coe2..4
 *           and the scalar LU diagonal coe5.
 * ====================================================================== */
void or_tstb3c(const int64_t* pi, const double* pr, int first_it, const int64_t* ind,
               const double* rop, double* coe, const double* xmut,
               const double* ti, const double* tj, const double* tk, const double* vol) {
  if (pi[ITYPCP] > 1) return;
  const int64_t nd = pi[NDIMDX], ndm = pi[NDIMDX_MTR];
  const double cut0x = 1e-20;
  double gamma = pr[GAMMA];
  double rgp = pr[CVINF] * (gamma - 1.);
  double prandt = pr[PRANDT];
  double xid = 1.5;
  if (first_it == 0) xid = 1.;
  double gam1 = gamma / prandt;
  if (pi[IFLOW] == 1) gam1 = 0.;
  double gam2 = gamma * rgp;
  const double *r_ = rop, *u_ = rop + nd, *v_ = rop + 2 * nd, *w_ = rop + 3 * nd, *t_ = rop + 4 * nd;
  double *c1 = coe, *c2 = coe + nd, *c3 = coe + 2 * nd, *c4 = coe + 3 * nd, *c5 = coe + 4 * nd;
  int typ = (int)pi[ITYPZONE];

  if (typ == 2) {
    double tcxi = ti[0], tcyj = tj[0], tczk = tk[0];
    double tc2i = sqrt(tcxi * tcxi), tc2j = sqrt(tcyj * tcyj), tc2k = sqrt(tczk * tczk);
#pragma omp parallel for num_threads(g_threads) schedule(static)
    for (int64_t k = ind[4]; k <= ind[5]; k++)
      for (int64_t j = ind[2]; j <= ind[3]; j++)
        for (int64_t i = ind[0]; i <= ind[1]; i++) {
          int64_t l = inddm(pi, i, j, k);
          double r = r_[l];
          double detj = OMAX(vol[0], cut0x);
          double u = u_[l], v = v_[l], w = w_[l];
          double c = sqrt(gam2 * t_[l]);
          double vmu = gam1 * xmut[l];
          double volu = detj * r;
          double xmvis = vmu / volu;
          double qni = tcxi * u, cni = c * tc2i, vmi = fabs(qni) + cni;
          c2[l] = vmi * 2. + xmvis * tc2i * tc2i * 4.;
          double qnj = tcyj * v, cnj = c * tc2j, vmj = fabs(qnj) + cnj;
          c3[l] = vmj * 2. + xmvis * tc2j * tc2j * 4.;
          double qnk = tczk * w, cnk = c * tc2k, vmk = fabs(qnk) + cnk;
          c4[l] = vmk * 2. + xmvis * tc2k * tc2k * 4.;
          c5[l] = xid + c1[l] * (c2[l] + c3[l] + c4[l]) * 0.5;
        }
    return;
  }
  const int64_t mi = pi[NIJK_MTR], mj = pi[NIJK_MTR + 1], mk = pi[NIJK_MTR + 2];
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int64_t k = ind[4]; k <= ind[5]; k++)
    for (int64_t j = ind[2]; j <= ind[3]; j++)
      for (int64_t i = ind[0]; i <= ind[1]; i++) {
        int64_t l = inddm(pi, i, j, k);
        int64_t lt = indmtr(pi, i, j, k);
        int64_t li = lt + mi, lj = lt + mj, lk = lt + mk;
        double r = r_[l];
        double detj = OMAX(vol[lt], cut0x);
        double u = u_[l], v = v_[l];
        double c = sqrt(gam2 * t_[l]);
        double vmu = gam1 * xmut[l], volu = detj * r, xmvis = vmu / volu;
        if (typ == 0) {
          double w = w_[l];
          const double *tix = ti, *tiy = ti + ndm, *tiz = ti + 2 * ndm;
          const double *tjx = tj, *tjy = tj + ndm, *tjz = tj + 2 * ndm;
          const double *tkx = tk, *tky = tk + ndm, *tkz = tk + 2 * ndm;
          double tcxi = .5 * (tix[lt] + tix[li]);
          double tcyi = .5 * (tiy[lt] + tiy[li]);
          double tczi = .5 * (tiz[lt] + tiz[li]);
          double tc2i = .5 * (sqrt(tix[lt] * tix[lt] + tiy[lt] * tiy[lt] + tiz[lt] * tiz[lt]) +
                              sqrt(tix[li] * tix[li] + tiy[li] * tiy[li] + tiz[li] * tiz[li]));
          double qni = tcxi * u + tcyi * v + tczi * w;
          double vmi = fabs(qni) + c * tc2i;
          c2[l] = vmi * 2. + xmvis * tc2i * tc2i * 4.;
          double tcxj = .5 * (tjx[lt] + tjx[lj]);
          double tcyj = .5 * (tjy[lt] + tjy[lj]);
          double tczj = .5 * (tjz[lt] + tjz[lj]);
          double tc2j = .5 * (sqrt(tjx[lt] * tjx[lt] + tjy[lt] * tjy[lt] + tjz[lt] * tjz[lt]) +
                              sqrt(tjx[lj] * tjx[lj] + tjy[lj] * tjy[lj] + tjz[lj] * tjz[lj]));
          double qnj = tcxj * u + tcyj * v + tczj * w;
          double vmj = fabs(qnj) + c * tc2j;
          c3[l] = vmj * 2. + xmvis * tc2j * tc2j * 4.;
          double tcxk = .5 * (tkx[lt] + tkx[lk]);
          double tcyk = .5 * (tky[lt] + tky[lk]);
          double tczk = .5 * (tkz[lt] + tkz[lk]);
          double tc2k = .5 * (sqrt(tkx[lt] * tkx[lt] + tky[lt] * tky[lt] + tkz[lt] * tkz[lt]) +
                              sqrt(tkx[lk] * tkx[lk] + tky[lk] * tky[lk] + tkz[lk] * tkz[lk]));
          double qnk = tcxk * u + tcyk * v + tczk * w;
          double vmk = fabs(qnk) + c * tc2k;
          c4[l] = vmk * 2. + xmvis * tc2k * tc2k * 4.;
          c5[l] = xid + c1[l] * (c2[l] + c3[l] + c4[l]) * 0.5;
        } else { /* 2d */
          const double *tix = ti, *tiy = ti + ndm;
          const double *tjx = tj, *tjy = tj + ndm;
          double tcxi = .5 * (tix[lt] + tix[li]);
          double tcyi = .5 * (tiy[lt] + tiy[li]);
          double tc2i = .5 * (sqrt(tix[lt] * tix[lt] + tiy[lt] * tiy[lt]) +
                              sqrt(tix[li] * tix[li] + tiy[li] * tiy[li]));
          double qni = tcxi * u + tcyi * v;
          double vmi = fabs(qni) + c * tc2i;
          c2[l] = vmi * 2. + xmvis * tc2i * tc2i * 4.;
          double tcxj = .5 * (tjx[lt] + tjx[lj]);
          double tcyj = .5 * (tjy[lt] + tjy[lj]);
          double tc2j = .5 * (sqrt(tjx[lt] * tjx[lt] + tjy[lt] * tjy[lt]) +
                              sqrt(tjx[lj] * tjx[lj] + tjy[lj] * tjy[lj]));
          double qnj = tcxj * u + tcyj * v;
          double vmj = fabs(qnj) + c * tc2j;
          c3[l] = vmj * 2. + xmvis * tc2j * tc2j * 4.;
          c5[l] = xid + c1[l] * (c2[l] + c3[l]) * 0.5;
        }
      }
}

/* ======================================================================
 * tstb3_impli -- FastS/FastS/Compute/tstb3_impli.for (implicit, local time
 * step: DTLOC = 1): the spectral radii coe2..4 as tstb3c computes them, then
 * FastS/FastS/Compute/dtloc.for: coe1 = CFL min(dtconv, dtvis) with
 * d = 1 / sum tc2^2, dtvis = 0.5 detj d / gam1 / xmut ro,
 * dtconv = sqrt(d) / (|u| + c), and coe5 = 1 + coe1 sum / 2.  Euler: gam1 is
 * 1e-30 (not 0), and the volume floor is 1e-30.
 * ====================================================================== */
static void or_local_dt(const int64_t* pi, const double* pr, const int64_t* ind, int lu,
                        const double* rop, double* coe, const double* xmut,
                        const double* ti, const double* tj, const double* tk, const double* vol);

/* explicit: FastS/FastS/Compute/tstb3_expli.for, the same time step, coe1 only */
void or_tstb3_expli(const int64_t* pi, const double* pr, const int64_t* ind,
                    const double* rop, double* coe, const double* xmut,
                    const double* ti, const double* tj, const double* tk, const double* vol) {
  or_local_dt(pi, pr, ind, 0, rop, coe, xmut, ti, tj, tk, vol);
}

void or_tstb3_impli(const int64_t* pi, const double* pr, const int64_t* ind,
                    const double* rop, double* coe, const double* xmut,
                    const double* ti, const double* tj, const double* tk, const double* vol) {
  or_local_dt(pi, pr, ind, 1, rop, coe, xmut, ti, tj, tk, vol);
}

static void or_local_dt(const int64_t* pi, const double* pr, const int64_t* ind, int lu,
                        const double* rop, double* coe, const double* xmut,
                        const double* ti, const double* tj, const double* tk, const double* vol) {
  const int64_t nd = pi[NDIMDX], ndm = pi[NDIMDX_MTR];
  const double cut0x = 1e-30;
  double gamma = pr[GAMMA];
  double rgp = pr[CVINF] * (gamma - 1.);
  double prandt = pr[PRANDT];
  double xid = 1.;
  double gam1 = gamma / prandt;
  if (pi[IFLOW] == 1) gam1 = cut0x;
  double gam1_1 = 1. / gam1;
  double gam2 = gamma * rgp;
  double cfl = pr[CFL];
  const double *r_ = rop, *u_ = rop + nd, *v_ = rop + 2 * nd, *w_ = rop + 3 * nd, *t_ = rop + 4 * nd;
  double *c1 = coe, *c2 = coe + nd, *c3 = coe + 2 * nd, *c4 = coe + 3 * nd, *c5 = coe + 4 * nd;
  int typ = (int)pi[ITYPZONE];
  const int64_t mi = pi[NIJK_MTR], mj = pi[NIJK_MTR + 1], mk = pi[NIJK_MTR + 2];
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int64_t k = ind[4]; k <= ind[5]; k++)
    for (int64_t j = ind[2]; j <= ind[3]; j++)
      for (int64_t i = ind[0]; i <= ind[1]; i++) {
        int64_t l = inddm(pi, i, j, k);
        double r = r_[l];
        double u = u_[l], v = v_[l], w = typ == 3 ? 0. : w_[l];
        double c = sqrt(gam2 * t_[l]);
        double vmu = gam1 * xmut[l];
        double tc2i, tc2j, tc2k, detj, C2 = 0., C3 = 0., C4 = 0.;
        if (typ == 2) {   /* cartesian */
          double tcxi = ti[0], tcyj = tj[0], tczk = tk[0];
          tc2i = sqrt(tcxi * tcxi); tc2j = sqrt(tcyj * tcyj); tc2k = sqrt(tczk * tczk);
          detj = OMAX(vol[0], cut0x);
          double volu = detj * r, xmvis = vmu / volu;
          double vmi = fabs(tcxi * u) + c * tc2i;
          C2 = vmi * 2. + xmvis * tc2i * tc2i * 4.;
          double vmj = fabs(tcyj * v) + c * tc2j;
          C3 = vmj * 2. + xmvis * tc2j * tc2j * 4.;
          double vmk = fabs(tczk * w) + c * tc2k;
          C4 = vmk * 2. + xmvis * tc2k * tc2k * 4.;
        } else {
          int64_t lt = indmtr(pi, i, j, k);
          int64_t li = lt + mi, lj = lt + mj, lk = lt + mk;
          detj = OMAX(vol[lt], cut0x);
          double volu = detj * r, xmvis = vmu / volu;
          if (typ != 3) {
            const double *tix = ti, *tiy = ti + ndm, *tiz = ti + 2 * ndm;
            const double *tjx = tj, *tjy = tj + ndm, *tjz = tj + 2 * ndm;
            const double *tkx = tk, *tky = tk + ndm, *tkz = tk + 2 * ndm;
            double tcxi = .5 * (tix[lt] + tix[li]), tcyi = .5 * (tiy[lt] + tiy[li]), tczi = .5 * (tiz[lt] + tiz[li]);
            tc2i = .5 * (sqrt(tix[lt] * tix[lt] + tiy[lt] * tiy[lt] + tiz[lt] * tiz[lt]) +
                         sqrt(tix[li] * tix[li] + tiy[li] * tiy[li] + tiz[li] * tiz[li]));
            double vmi = fabs(tcxi * u + tcyi * v + tczi * w) + c * tc2i;
            C2 = vmi * 2. + xmvis * tc2i * tc2i * 4.;
            double tcxj = .5 * (tjx[lt] + tjx[lj]), tcyj = .5 * (tjy[lt] + tjy[lj]), tczj = .5 * (tjz[lt] + tjz[lj]);
            tc2j = .5 * (sqrt(tjx[lt] * tjx[lt] + tjy[lt] * tjy[lt] + tjz[lt] * tjz[lt]) +
                         sqrt(tjx[lj] * tjx[lj] + tjy[lj] * tjy[lj] + tjz[lj] * tjz[lj]));
            double vmj = fabs(tcxj * u + tcyj * v + tczj * w) + c * tc2j;
            C3 = vmj * 2. + xmvis * tc2j * tc2j * 4.;
            double tcxk = .5 * (tkx[lt] + tkx[lk]), tcyk = .5 * (tky[lt] + tky[lk]), tczk = .5 * (tkz[lt] + tkz[lk]);
            tc2k = .5 * (sqrt(tkx[lt] * tkx[lt] + tky[lt] * tky[lt] + tkz[lt] * tkz[lt]) +
                         sqrt(tkx[lk] * tkx[lk] + tky[lk] * tky[lk] + tkz[lk] * tkz[lk]));
            double vmk = fabs(tcxk * u + tcyk * v + tczk * w) + c * tc2k;
            C4 = vmk * 2. + xmvis * tc2k * tc2k * 4.;
          } else {   /* 2d: tc2k = 0, w = 0 */
            const double *tix = ti, *tiy = ti + ndm;
            const double *tjx = tj, *tjy = tj + ndm;
            double tcxi = .5 * (tix[lt] + tix[li]), tcyi = .5 * (tiy[lt] + tiy[li]);
            tc2i = .5 * (sqrt(tix[lt] * tix[lt] + tiy[lt] * tiy[lt]) + sqrt(tix[li] * tix[li] + tiy[li] * tiy[li]));
            double vmi = fabs(tcxi * u + tcyi * v) + c * tc2i;
            C2 = vmi * 2. + xmvis * tc2i * tc2i * 4.;
            double tcxj = .5 * (tjx[lt] + tjx[lj]), tcyj = .5 * (tjy[lt] + tjy[lj]);
            tc2j = .5 * (sqrt(tjx[lt] * tjx[lt] + tjy[lt] * tjy[lt]) + sqrt(tjx[lj] * tjx[lj] + tjy[lj] * tjy[lj]));
            double vmj = fabs(tcxj * u + tcyj * v) + c * tc2j;
            C3 = vmj * 2. + xmvis * tc2j * tc2j * 4.;
            tc2k = 0.;
          }
        }
        /* dtloc.for */
        double d = 1. / (tc2i * tc2i + tc2j * tc2j + tc2k * tc2k);
        double dtvis = 0.5 * detj * d * gam1_1 / xmut[l] * r;
        double sp = sqrt(u * u + v * v + w * w) + c;
        double dtconv = sqrt(d) / sp;
        c1[l] = cfl * OMIN(dtconv, dtvis);
        if (!lu) continue;   /* explicit: coe1 only */
        c2[l] = C2;
        c3[l] = C3;
        if (typ != 3) c4[l] = C4;
        if (typ == 3) c5[l] = xid + c1[l] * (c2[l] + c3[l]) * 0.5;
        else c5[l] = xid + c1[l] * (c2[l] + c3[l] + c4[l]) * 0.5;
      }
}

/* ======================================================================
 * init_rhs -- FastS/FastS/Compute/init_rhs.for:49-129 (RK low-storage A)
 * ====================================================================== */
void or_init_rhs(const int64_t* pi, int nitcfg, const int64_t* ind, double* drodm) {
  const double cxsi1 = -0.6830127018922193, cxsi2 = -4. / 3.;
  int64_t b = pi[RK], nd = pi[NDIMDX], neq = pi[NEQ];
  double coefH = 0.;
  if (b == 3) {
    if (nitcfg == 2) coefH = cxsi1;
    else if (nitcfg == 3) coefH = cxsi2;
    else if (nitcfg == 1) coefH = 0.;
  } else if (b == 2) {
    if (nitcfg == 2) coefH = -1.;
    else if (nitcfg == 1) coefH = 0.;
  }
  int zero = (pi[ITYPCP] <= 1 || nitcfg == 1);
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int64_t k = ind[4]; k <= ind[5]; k++)
    for (int64_t j = ind[2]; j <= ind[3]; j++)
      for (int64_t i = ind[0]; i <= ind[1]; i++) {
        int64_t l = inddm(pi, i, j, k);
        for (int64_t ne = 0; ne < neq; ne++) {
          if (zero) drodm[l + ne * nd] = 0.;
          else drodm[l + ne * nd] = drodm[l + ne * nd] * coefH;
        }
      }
}

/* ======================================================================
 * Face fluxes -- FastS/FastS/Compute/template_FluxAndBalance.for:192-271
 * (generated per scheme under ROE/, AUSM/): face "dir" of cell l is the
 * face between l-inc and l; assemble_drodm_plus_vec1.for adds it to l and
 * subtracts it from l-inc.
 * ====================================================================== */
static void bc_window(const int64_t* pi, const int64_t* fen, int idir, int64_t* cl);
static void bc_normal(const int64_t* pi, const double* ti, const double* tj, const double* tk,
                      int idir, int64_t i, int64_t j, int64_t k, double t[3]);

typedef struct {
  const int64_t* pi; const double* pr;
  const double *rop, *xmut, *ti, *tj, *tk, *vol;
  int64_t inc[3], nd, ndm, inc_mtr[3];
  int typ, iflow, kflu, slope;
  double gam, rgp, gam1, gam3, c1, c2, c3, c4, c5, c6, cvisq, psiroe, wig_cte, tmin_1;
  double c50, c51, c52, c53, c54;           /* o5 (template_FluxAndBalance.for:149-154) */
  double tcx, tcy, tcz, si, sj, sk, volinv; /* 3d cartesian constants */
  const double* wig; double opt0;           /* senseur (KFLUDOM = 2) */
  int neq;                                  /* 6: Spalart-Allmaras (IFLOW = 3) */
  double gam4, coesut_sa, temp01, cmus1, sigma_1;
} fctx;

static void fctx_init(fctx* c, const int64_t* pi, const double* pr, const double* rop,
                      const double* xmut, const double* ti, const double* tj,
                      const double* tk, const double* vol) {
  c->pi = pi; c->pr = pr; c->rop = rop; c->xmut = xmut; c->ti = ti; c->tj = tj; c->tk = tk; c->vol = vol;
  c->inc[0] = 1; c->inc[1] = pi[NIJK]; c->inc[2] = pi[NIJK] * pi[NIJK + 1];
  c->inc_mtr[0] = pi[NIJK_MTR]; c->inc_mtr[1] = pi[NIJK_MTR + 1]; c->inc_mtr[2] = pi[NIJK_MTR + 2];
  c->nd = pi[NDIMDX]; c->ndm = pi[NDIMDX_MTR];
  c->typ = (int)pi[ITYPZONE]; c->iflow = (int)pi[IFLOW]; c->kflu = (int)pi[KFLUDOM];
  c->slope = (int)pi[SLOPE];
  /* template_FluxAndBalance.for:108-156 */
  c->tcx = ti[0]; c->tcy = tj[0]; c->tcz = pi[NEQ_K] > 0 ? tk[0] : 0.;  /* a 2-d zone has no tk */
  c->si = fabs(c->tcx); c->sj = fabs(c->tcy); c->sk = fabs(c->tcz);
  c->volinv = 0.5 / vol[0];
  c->gam = pr[GAMMA];
  c->rgp = pr[CVINF] * (c->gam - 1.);
  c->gam1 = c->gam / (c->gam - 1.);
  c->gam3 = c->gam1 / pr[PRANDT] * c->rgp;
  c->psiroe = pr[PSIROE];
  c->wig_cte = pr[WIG_AMP];
  c->tmin_1 = 100. / pr[TINF];
  double uref = pr[VINF], roref = pr[ROINF];
  c->c1 = 0.02 * uref;
  c->c2 = 0.02 / (uref * roref);
  c->c3 = -2.;
  double c6 = 1. / 6.;
  c->c4 = 5. * c6;
  c->c5 = 2. * c6;
  c->c6 = -1. * c6;
  c->cvisq = 1. / 3;
  c->c50 = 1. / 60;
  c->c51 = 27. * c->c50;
  c->c52 = -13. * c->c50;
  c->c53 = -3. * c->c50;
  c->c54 = 2. * c->c50;
  c->c50 = 47. * c->c50;
  c->wig = NULL;
  c->opt0 = (double)pi[SENSORTYPE];
  /* SA drivers (e.g. AUSM/3dcart/fluausm_SA_o3_3dcart.for:114-127) */
  c->neq = (int)pi[NEQ];
  c->gam4 = c->gam1 / pr[PRANDT_TUR] * c->rgp;
  c->cmus1 = pr[CS];
  c->temp01 = 1. / pr[TEMP0];
  c->coesut_sa = pr[XMUL0] * (1. + c->cmus1 * c->temp01);
  c->sigma_1 = 1. / (2. / 3.);
}

/* Slope/minmod_slope_var.for:1-17 limiter */
static inline double avmin(double c, double r) {
  return fsign(1., c) * OMAX(0., OMIN(fabs(c), fsign(1., c) * r));
}

/* van Albada's smooth limiter (slope = 8; not a FastS slope): the averaged
 * slope ((y^2 + e) x + (x^2 + e) y) / (x^2 + y^2 + 2 e), e = 1e-12, of the
 * backward / forward differences x, y (van Albada, van Leer & Roberts,
 * Astron. Astrophys. 108, 1982); differentiable everywhere. */
static inline double vanalbada(double x, double y) {
  const double e2 = 1e-12;
  return ((y * y + e2) * x + (x * x + e2) * y) / (x * x + y * y + 2. * e2);
}

/* Slope/{o1,o3,o3sc,minmod}_slope_var.for: qm = right state, qp = left
 * state of the d-face of cell l.  o3sc (slope 6) blends the o3 states with
 * the first-order ones by the shock-sensor weight of the face,
 * wig(l + sl_d) (e.g. AUSM/3dcart/fluFaceEuler_o3sc_3dcart_i.for:10,
 * sl_d = d * NDIMDX, shifted by 3 * NDIMDX for the senseur scheme). */
static void slopes(const fctx* c, int64_t l, int d, double qm[6], double qp[6]) {
  const double* rop = c->rop;
  const int64_t inc = c->inc[d];
  int64_t nd = c->nd, nm = l - inc, nm2 = l - 2 * inc, np = l + inc;
  int64_t nm3 = l - 3 * inc, np2 = l + 2 * inc;   /* o5: three ghost layers */
  double csc = 0.;
  if (c->slope == 6 || c->slope == 7) csc = c->wig[l + d * nd + (c->kflu == 2 ? 3 * nd : 0)];
  for (int v = 0; v < c->neq; v++) {
    if (c->typ == 3 && v == 3) { qm[v] = 0.; qp[v] = 0.; continue; }
    int64_t vs = v * nd;
    if (c->slope == 1) {
      qm[v] = rop[l + vs];
      qp[v] = rop[nm + vs];
    } else if (c->slope == 2 || c->slope == 6) {
      qm[v] = c->c4 * rop[l + vs] + c->c5 * rop[nm + vs] + c->c6 * rop[np + vs];
      qp[v] = c->c4 * rop[nm + vs] + c->c6 * rop[nm2 + vs] + c->c5 * rop[l + vs];
      if (c->slope == 6) {   /* Slope/o3sc_slope_var.for:5-6 */
        qm[v] = rop[l + vs] * (1. - csc) + qm[v] * csc;
        qp[v] = rop[nm + vs] * (1. - csc) + qp[v] * csc;
      }
    } else if (c->slope == 5 || c->slope == 7) {   /* Slope/o5_slope_var.for */
      qm[v] = c->c50 * rop[l + vs] + c->c51 * rop[nm + vs] + c->c52 * rop[np + vs] +
              c->c53 * rop[nm2 + vs] + c->c54 * rop[np2 + vs];
      qp[v] = c->c50 * rop[nm + vs] + c->c52 * rop[nm2 + vs] + c->c51 * rop[l + vs] +
              c->c53 * rop[np + vs] + c->c54 * rop[nm3 + vs];
      if (c->slope == 7) {   /* Slope/o5sc_slope_var.for */
        qm[v] = rop[l + vs] * (1. - csc) + qm[v] * csc;
        qp[v] = rop[nm + vs] * (1. - csc) + qp[v] * csc;
      }
    } else if (c->slope == 8) { /* van Albada MUSCL */
      double d1 = rop[nm + vs] - rop[nm2 + vs], d2 = rop[l + vs] - rop[nm + vs];
      double d3 = rop[np + vs] - rop[l + vs];
      qm[v] = rop[l + vs] - 0.5 * vanalbada(d2, d3);
      qp[v] = rop[nm + vs] + 0.5 * vanalbada(d1, d2);
    } else { /* minmod */
      double roff = .5 * OMAX(0., OMIN(rop[l + 4 * nd] * c->tmin_1 - .5, 1.));
      double delm = rop[l + vs] - rop[nm + vs];
      double delp = rop[np + vs] - rop[l + vs];
      double delq = rop[nm + vs] - rop[nm2 + vs];
      double slp = roff * avmin(delm, delp);
      double slq = roff * avmin(delq, delm);
      qm[v] = rop[l + vs] - slp;
      qp[v] = rop[nm + vs] + slq;
    }
  }
}

/* face normal for direction d at metric index lt (Normale/normale_*.for) */
static void face_normal(const fctx* c, int d, int64_t lt, double* tcx, double* tcy,
                        double* tcz, double* s) {
  if (c->typ == 2) {
    *tcx = c->tcx; *tcy = c->tcy; *tcz = c->tcz;
    *s = d == 0 ? c->si : (d == 1 ? c->sj : c->sk);
    return;
  }
  const double* t = d == 0 ? c->ti : (d == 1 ? c->tj : c->tk);
  *tcx = t[lt];
  *tcy = t[lt + c->ndm];
  if (c->typ == 3) { *tcz = 0.; *s = sqrt(*tcx * *tcx + *tcy * *tcy); return; }
  *tcz = t[lt + 2 * c->ndm];
  *s = sqrt(*tcx * *tcx + *tcy * *tcy + *tcz * *tcz);
}


/* Roe flux with Harten entropy fix -- etat_roe_GD.for:1-20,
 * Vit_ent/qn_3dfull_*.for, Vit_ent/fludiffer_3dfull_i.for:1-61.
 * The general (3d full) form is used for every zone type: for a cartesian
 * face the normal has exact zeros in its two tangential components
 * (tcx,0,0), so every extra product is an exact zero and the result is the
 * cartesian files' (Vit_ent/fludiffer_3dcart_*.for) bit for bit, up to the
 * sign of zero results. */
static void roe_face(const fctx* c, const double qm[5], const double qp[5],
                     double tcx, double tcy, double tcz, double s, double flu[5]) {
  double gam = c->gam, rgp = c->rgp, gam1 = c->gam1, psiroe = c->psiroe;
  double qp1 = qp[0], qp2 = qp[1], qp3 = qp[2], qp4 = qp[3], qp5 = qp[4];
  double qm1 = qm[0], qm2 = qm[1], qm3 = qm[2], qm4 = qm[3], qm5 = qm[4];
  double r1 = qp1;
  double p1 = r1 * qp5 * rgp;
  double h1 = gam1 * qp5 * rgp + .5 * (qp2 * qp2 + qp3 * qp3 + qp4 * qp4);
  double r2 = qm1;
  double p2 = r2 * qm5 * rgp;
  double h2 = gam1 * qm5 * rgp + .5 * (qm2 * qm2 + qm3 * qm3 + qm4 * qm4);
  qp1 = sqrt(r1);
  qm1 = sqrt(r2);
  double r = qp1 * qm1;
  double r_1 = 1. / (qp1 + qm1);
  double u = (qp1 * qp2 + qm1 * qm2) * r_1;
  double v = (qp1 * qp3 + qm1 * qm3) * r_1;
  double w = (qp1 * qp4 + qm1 * qm4) * r_1;
  double h = (qp1 * h1 + qm1 * h2) * r_1;
  double q = .5 * (u * u + v * v + w * w);
  double cc = sqrt((gam - 1.) * fabs(h - q));
  double qn1 = qp2 * tcx + qp3 * tcy + qp4 * tcz;
  double qn2 = qm2 * tcx + qm3 * tcy + qm4 * tcz;
  double du = (qm2 - qp2) * s, dv = (qm3 - qp3) * s, dw = (qm4 - qp4) * s;
  double dp = p2 - p1;
  double dqn = qn2 - qn1;
  double s_1 = 1.0 / OMAX(s, 1.E-30);
  double nx = tcx * s_1, ny = tcy * s_1, nz = tcz * s_1;
  double qn = u * nx + v * ny + w * nz;
  double f1 = qn;
  double f4 = psiroe * (fabs(f1) + cc);
  double f2 = 0.5 + fsign(0.5, fabs(f1) - f4);
  double f3 = (f2 - 1.0) * (f1 * f1 / f4 + f4) * 0.5 - f2 * fabs(f1);
  f1 = (r2 - r1 - dp / (cc * cc)) * s;
  double flu1 = f3 * (f1);
  double flu2 = f3 * (f1 * u + r * (du - nx * dqn));
  double flu3 = f3 * (f1 * v + r * (dv - ny * dqn));
  double flu4 = f3 * (f1 * w + r * (dw - nz * dqn));
  double flu5 = f3 * (f1 * q + r * (u * du + v * dv + w * dw - qn * dqn));
  f1 = qn + cc;
  f2 = 0.5 + fsign(0.5, fabs(f1) - f4);
  f3 = (f2 - 1.) * (f1 * f1 / f4 + f4) * 0.5 - f2 * fabs(f1);
  f1 = (dp + r * cc * dqn * s_1) / (2. * cc * cc) * s * f3;
  flu1 = flu1 + f1;
  flu2 = flu2 + f1 * (u + nx * cc);
  flu3 = flu3 + f1 * (v + ny * cc);
  flu4 = flu4 + f1 * (w + nz * cc);
  flu5 = flu5 + f1 * (h + qn * cc);
  f1 = qn - cc;
  f2 = 0.5 + fsign(0.5, fabs(f1) - f4);
  f3 = (f2 - 1.) * (f1 * f1 / f4 + f4) * 0.5 - f2 * fabs(f1);
  f1 = (dp - r * cc * dqn * s_1) / (2. * cc * cc) * f3 * s;
  flu1 = flu1 + f1;
  flu2 = flu2 + f1 * (u - nx * cc);
  flu3 = flu3 + f1 * (v - ny * cc);
  flu4 = flu4 + f1 * (w - nz * cc);
  flu5 = flu5 + f1 * (h - qn * cc);
  double rou1 = r1 * qn1, rou2 = r2 * qn2, p1p2 = p1 + p2;
  flu[0] = (flu1 + rou1 + rou2) * 0.5;
  flu[1] = (flu2 + rou1 * qp2 + rou2 * qm2 + tcx * p1p2) * 0.5;
  flu[2] = (flu3 + rou1 * qp3 + rou2 * qm3 + tcy * p1p2) * 0.5;
  flu[3] = (flu4 + rou1 * qp4 + rou2 * qm4 + tcz * p1p2) * 0.5;
  flu[4] = (flu5 + rou1 * h1 + rou2 * h2) * 0.5;
}

/* AUSM+(P) -- etat_GD.for:1-15, AUSM/fluFaceEuler.for:36-57,
 * Vit_ent/fluvector_3dfull_i.for:1-5.  Same general-form remark as Roe.
 * tl = temperature of cell l (the right cell), used for the sound speed. */
static void ausm_face(const fctx* c, const double qm[6], const double qp[6], double tl,
                      double tcx, double tcy, double tcz, double s, double wg, double flu[6]) {
  double rgp = c->rgp, gam1 = c->gam1;
  double r1 = qp[0], rou1 = r1 * qp[1], rov1 = r1 * qp[2], row1 = r1 * qp[3];
  double p1 = r1 * qp[4] * rgp;
  double h1 = gam1 * p1 + .5 * (rou1 * qp[1] + rov1 * qp[2] + row1 * qp[3]);
  double r2 = qm[0], rou2 = r2 * qm[1], rov2 = r2 * qm[2], row2 = r2 * qm[3];
  double p2 = r2 * qm[4] * rgp;
  double h2 = gam1 * p2 + .5 * (rou2 * qm[1] + rov2 * qm[2] + row2 * qm[3]);
  double qn1 = qp[1] * tcx + qp[2] * tcy + qp[3] * tcz;
  double qn2 = qm[1] * tcx + qm[2] * tcy + qm[3] * tcz;
  double cc = rgp * c->gam * tl;
  double u, tdu;
  if (c->kflu == 2) {  /* SENSOR/fluFaceEuler.for: Rhie-Chow term and dissipation switched by wig */
    u = 0.25 * (qn1 + qn2) - c->c2 * s * (p2 - p1) * (c->opt0 * wg + 1. - c->opt0);
    tdu = OMAX(fabs(u), c->c1 * s) * wg;
  } else {
    double son = sqrt(qn1 * qn1 / cc);
    double tam = c->c3 * son + s;
    double tam1 = OMAX(0., tam) * c->c2;
    u = 0.25 * (qn1 + qn2) - tam1 * (p2 - p1);
    tdu = OMAX(fabs(u), c->c1 * s) * c->wig_cte;
  }
  double p1p2 = (p1 + p2) * 0.5;
  flu[0] = u * (r1 + r2) - tdu * (r2 - r1);
  flu[1] = u * (rou1 + rou2) - tdu * (rou2 - rou1) + tcx * p1p2;
  flu[2] = u * (rov1 + rov2) - tdu * (rov2 - rov1) + tcy * p1p2;
  flu[3] = u * (row1 + row2) - tdu * (row2 - row1) + tcz * p1p2;
  flu[4] = u * (h1 + h2) - tdu * (h2 - h1);
  if (c->neq == 6) {   /* AUSM/fluFaceSA.for: flux of ro * nutilde */
    double qm6 = qm[5] * qm[0], qp6 = qp[5] * qp[0];
    flu[5] = u * (qm6 + qp6) - tdu * (qm6 - qp6);
  }
}

/* SA/mut_prandtltb_interface.for: laminar viscosity of the two cells (their
 * sum), total mu and the laminar + turbulent conductivity; SA/mut_interface:
 * nutilde diffusion coefficient. */
static void sa_mut(const fctx* c, int64_t il, int64_t ir, double volinv, double* xmutvol,
                   double* xktvol, double* xmutvol_sa) {
  const double* rop = c->rop;
  const int64_t nd = c->nd;
  double xmulam = c->coesut_sa * sqrt(rop[il + 4 * nd] * c->temp01) / (1. + c->cmus1 / rop[il + 4 * nd]);
  xmulam = xmulam + c->coesut_sa * sqrt(rop[ir + 4 * nd] * c->temp01) / (1. + c->cmus1 / rop[ir + 4 * nd]);
  double xmutot = c->xmut[ir] + c->xmut[il];
  double xmutur = xmutot - xmulam;
  *xktvol = (xmulam * c->gam3 + xmutur * c->gam4) * volinv;
  *xmutvol = xmutot * volinv;
  double x = xmulam + rop[il + 5 * nd] * rop[il] + rop[ir + 5 * nd] * rop[ir];
  *xmutvol_sa = x * volinv * c->sigma_1;
}

/* Viscous face flux on a 3d cartesian zone: fluvisq_3dcart_{i,j,k}.for and
 * mut_interface.for (xmutvol = (mu_r + mu_l) * 0.5/vol, xktvol = xmutvol*gam3). */
static void visc_cart(const fctx* c, int d, int64_t l, double flu[6]) {
  const double* rop = c->rop;
  int64_t nd = c->nd, inci = c->inc[0], incj = c->inc[1], inck = c->inc[2];
  int64_t v2 = nd, v3 = 2 * nd, v4 = 3 * nd, v5 = 4 * nd;
  double tcx = c->tcx, tcy = c->tcy, tcz = c->tcz, cvisq = c->cvisq;
  double f1, f2, f3, f4, f5, f6, fv, fv5, div;
  int64_t il, ir = l;
  if (d == 0) {
    il = l - inci;
    int64_t l220 = l - inci - incj, l020 = l - incj, l210 = l - inci + incj, l010 = l + incj;
    int64_t l202 = l - inci - inck, l002 = l - inck, l201 = l - inci + inck, l001 = l + inck;
    double tix = tcx, tjy = .25 * tcy, tkz = .25 * tcz;
    f1 = rop[il + v2]; f2 = rop[ir + v2]; fv = f1 + f2;
    f3 = fv + rop[l220 + v2] + rop[l020 + v2];
    f4 = fv + rop[l210 + v2] + rop[l010 + v2];
    f5 = fv + rop[l202 + v2] + rop[l002 + v2];
    f6 = fv + rop[l201 + v2] + rop[l001 + v2];
    double gradU_nx = (f2 - f1) * tix, gradU_ny = (f4 - f3) * tjy, gradU_nz = (f6 - f5) * tkz;
    f1 = rop[il + v3]; f2 = rop[ir + v3]; fv = f1 + f2;
    f3 = fv + rop[l220 + v3] + rop[l020 + v3];
    f4 = fv + rop[l210 + v3] + rop[l010 + v3];
    double gradV_nx = (f2 - f1) * tix, gradV_ny = (f4 - f3) * tjy;
    f1 = rop[il + v4]; f2 = rop[ir + v4]; fv = f1 + f2;
    f5 = fv + rop[l202 + v4] + rop[l002 + v4];
    f6 = fv + rop[l201 + v4] + rop[l001 + v4];
    double gradW_nx = (f2 - f1) * tix, gradW_nz = (f6 - f5) * tkz;
    f1 = rop[il + v5]; f2 = rop[ir + v5];
    double gradT_nx = (f2 - f1) * tix;
    div = (gradU_nx + gradV_ny + gradW_nz) * cvisq;
    f1 = gradU_nx - div;
    f2 = gradU_ny + gradV_nx;
    f3 = gradU_nz + gradW_nx;
    double xmutvol, xktvol, xmutvol_sa = 0.;
    if (c->neq == 6) {
      sa_mut(c, il, ir, c->volinv, &xmutvol, &xktvol, &xmutvol_sa);
    } else {
      xmutvol = (c->xmut[ir] + c->xmut[il]) * c->volinv;
      xktvol = xmutvol * c->gam3;
    }
    fv = -(2. * f1 * tcx) * xmutvol;
    fv5 = fv * (rop[ir + v2] + rop[il + v2]);
    flu[1] = flu[1] + fv;
    fv = -(f2 * tcx) * xmutvol;
    fv5 = fv5 + fv * (rop[ir + v3] + rop[il + v3]);
    flu[2] = flu[2] + fv;
    fv = -(f3 * tcx) * xmutvol;
    fv5 = fv5 + fv * (rop[ir + v4] + rop[il + v4]);
    flu[3] = flu[3] + fv;
    fv = fv5 * 0.5 - (gradT_nx * tcx) * xktvol;
    flu[4] = flu[4] + fv;
    if (c->neq == 6) {   /* SA/fluvisq_SA_3dcart_i.for */
      double gn = (rop[ir + 5 * nd] - rop[il + 5 * nd]) * tix;
      flu[5] = flu[5] - xmutvol_sa * gn * tcx;
    }
  } else if (d == 1) {
    il = l - incj;
    int64_t l022 = l - incj - inck, l002 = l - inck, l021 = l - incj + inck, l001 = l + inck;
    int64_t l220 = l - inci - incj, l200 = l - inci, l120 = l + inci - incj, l100 = l + inci;
    double tiy = tcy, tjz = .25 * tcz, tkx = .25 * tcx;
    f1 = rop[il + v2]; f2 = rop[ir + v2]; fv = f1 + f2;
    f5 = fv + rop[l220 + v2] + rop[l200 + v2];
    f6 = fv + rop[l120 + v2] + rop[l100 + v2];
    double gradU_nx = (f6 - f5) * tkx, gradU_ny = (f2 - f1) * tiy;
    f1 = rop[il + v3]; f2 = rop[ir + v3]; fv = f1 + f2;
    f3 = fv + rop[l022 + v3] + rop[l002 + v3];
    f4 = fv + rop[l021 + v3] + rop[l001 + v3];
    f5 = fv + rop[l220 + v3] + rop[l200 + v3];
    f6 = fv + rop[l120 + v3] + rop[l100 + v3];
    double gradV_nx = (f6 - f5) * tkx, gradV_ny = (f2 - f1) * tiy, gradV_nz = (f4 - f3) * tjz;
    f1 = rop[il + v4]; f2 = rop[ir + v4]; fv = f1 + f2;
    f3 = fv + rop[l022 + v4] + rop[l002 + v4];
    f4 = fv + rop[l021 + v4] + rop[l001 + v4];
    double gradW_ny = (f2 - f1) * tiy, gradW_nz = (f4 - f3) * tjz;
    f1 = rop[il + v5]; f2 = rop[ir + v5];
    double gradT_ny = (f2 - f1) * tiy;
    div = (gradU_nx + gradV_ny + gradW_nz) * cvisq;
    f2 = gradU_ny + gradV_nx;
    f4 = gradV_ny - div;
    f5 = gradV_nz + gradW_ny;
    double xmutvol, xktvol, xmutvol_sa = 0.;
    if (c->neq == 6) {
      sa_mut(c, il, ir, c->volinv, &xmutvol, &xktvol, &xmutvol_sa);
    } else {
      xmutvol = (c->xmut[ir] + c->xmut[il]) * c->volinv;
      xktvol = xmutvol * c->gam3;
    }
    fv = -(f2 * tcy) * xmutvol;
    fv5 = fv * (rop[ir + v2] + rop[il + v2]);
    flu[1] = flu[1] + fv;
    fv = -(2. * f4 * tcy) * xmutvol;
    fv5 = fv5 + fv * (rop[ir + v3] + rop[il + v3]);
    flu[2] = flu[2] + fv;
    fv = -(f5 * tcy) * xmutvol;
    fv5 = fv5 + fv * (rop[ir + v4] + rop[il + v4]);
    flu[3] = flu[3] + fv;
    fv = fv5 * 0.5 - (gradT_ny * tcy) * xktvol;
    flu[4] = flu[4] + fv;
    if (c->neq == 6) {   /* SA/fluvisq_SA_3dcart_j.for */
      double gn = (rop[ir + 5 * nd] - rop[il + 5 * nd]) * tiy;
      flu[5] = flu[5] - xmutvol_sa * (gn * tcy);
    }
  } else {
    il = l - inck;
    int64_t l200 = l - inci, l202 = l - inci - inck, l102 = l + inci - inck, l100 = l + inci;
    int64_t l022 = l - incj - inck, l020 = l - incj, l012 = l + incj - inck, l010 = l + incj;
    double tiz = tcz, tky = 0.25 * tcy, tjx = 0.25 * tcx;
    f1 = rop[il + v2]; f2 = rop[ir + v2]; fv = f1 + f2;
    f3 = fv + rop[l202 + v2] + rop[l200 + v2];
    f4 = fv + rop[l102 + v2] + rop[l100 + v2];
    double gradU_nx = (f4 - f3) * tjx, gradU_nz = (f2 - f1) * tiz;
    f1 = rop[il + v3]; f2 = rop[ir + v3]; fv = f1 + f2;
    f5 = fv + rop[l022 + v3] + rop[l020 + v3];
    f6 = fv + rop[l012 + v3] + rop[l010 + v3];
    double gradV_ny = (f6 - f5) * tky, gradV_nz = (f2 - f1) * tiz;
    f1 = rop[il + v4]; f2 = rop[l + v4]; fv = f1 + f2;
    f3 = fv + rop[l202 + v4] + rop[l200 + v4];
    f4 = fv + rop[l102 + v4] + rop[l100 + v4];
    f5 = fv + rop[l022 + v4] + rop[l020 + v4];
    f6 = fv + rop[l012 + v4] + rop[l010 + v4];
    double gradW_nx = (f4 - f3) * tjx, gradW_ny = (f6 - f5) * tky, gradW_nz = (f2 - f1) * tiz;
    f1 = rop[il + v5]; f2 = rop[ir + v5];
    double gradT_nz = (f2 - f1) * tiz;
    div = (gradU_nx + gradV_ny + gradW_nz) * cvisq;
    f3 = gradU_nz + gradW_nx;
    f5 = gradV_nz + gradW_ny;
    f6 = gradW_nz - div;
    double xmutvol, xktvol, xmutvol_sa = 0.;
    if (c->neq == 6) {
      sa_mut(c, il, ir, c->volinv, &xmutvol, &xktvol, &xmutvol_sa);
    } else {
      xmutvol = (c->xmut[ir] + c->xmut[il]) * c->volinv;
      xktvol = xmutvol * c->gam3;
    }
    fv = -f3 * tcz * xmutvol;
    fv5 = fv * (rop[ir + v2] + rop[il + v2]);
    flu[1] = flu[1] + fv;
    fv = -f5 * tcz * xmutvol;
    fv5 = fv5 + fv * (rop[ir + v3] + rop[il + v3]);
    flu[2] = flu[2] + fv;
    fv = -2. * f6 * tcz * xmutvol;
    fv5 = fv5 + fv * (rop[ir + v4] + rop[il + v4]);
    flu[3] = flu[3] + fv;
    fv = fv5 * 0.5 - gradT_nz * tcz * xktvol;
    flu[4] = flu[4] + fv;
    if (c->neq == 6) {   /* SA/fluvisq_SA_3dcart_k.for */
      double gn = (rop[ir + 5 * nd] - rop[il + 5 * nd]) * tiz;
      flu[5] = flu[5] - xmutvol_sa * gn * tcz;
    }
  }
}

/* Viscous face flux on a 3d general zone: Compute/fluvisq_3dfull_{i,j,k}.for
 * + mut_interface.for.  Green-Gauss gradient over the cell joining il =
 * l - inc_d and ir = l: faces normal to d at the two cell centres (mean of
 * two face vectors), faces along the transverse directions a = d+1, b = d+2
 * (mod 3) from four-cell means (factor 1/8 = 1/4 x 1/2).  The three files
 * are this routine with (d, a, b) = (i, j, k), (j, k, i), (k, i, j). */
static void visc_full(const fctx* c, int d, int64_t l, int64_t lt, double tcx, double tcy,
                      double tcz, double flu[6]) {
  const double* rop = c->rop;
  const int64_t nd = c->nd, ndm = c->ndm;
  const int a = (d + 1) % 3, b = (d + 2) % 3;
  const double* T3[3] = {c->ti, c->tj, c->tk};
  const double *TD = T3[d], *TA = T3[a], *TB = T3[b];
  const int64_t mD = c->inc_mtr[d], mA = c->inc_mtr[a], mB = c->inc_mtr[b];
  const int64_t iA = c->inc[a], iB = c->inc[b];
  const int64_t ltm = lt - mD, ltp = lt + mD, ltA = lt + mA, ltAm = lt + mA - mD,
                ltB = lt + mB, ltBm = lt + mB - mD;
  double t0[3], t1[3], ta0[3], ta1[3], tb0[3], tb1[3];
  for (int m = 0; m < 3; m++) {
    const int64_t o = m * ndm;
    t0[m] = .5 * (TD[lt + o] + TD[ltm + o]);
    t1[m] = .5 * (TD[lt + o] + TD[ltp + o]);
    ta0[m] = .125 * (TA[lt + o] + TA[ltm + o]);
    ta1[m] = .125 * (TA[ltA + o] + TA[ltAm + o]);
    tb0[m] = .125 * (TB[lt + o] + TB[ltm + o]);
    tb1[m] = .125 * (TB[ltB + o] + TB[ltBm + o]);
  }
  const int64_t il = l - c->inc[d], ir = l;
  double g[5][3];
  const int ng = c->neq == 6 ? 5 : 4;    /* u, v, w, T (, nutilde) */
  for (int v = 0; v < ng; v++) {
    const double* q = rop + (v + 1) * nd;
    double f1 = q[il], f2 = q[ir];
    double f3 = q[ir] + q[il] + q[il - iA] + q[ir - iA];
    double f4 = q[ir] + q[il] + q[il + iA] + q[ir + iA];
    double f5 = q[ir] + q[il] + q[il - iB] + q[ir - iB];
    double f6 = q[ir] + q[il] + q[il + iB] + q[ir + iB];
    for (int m = 0; m < 3; m++)
      g[v][m] = (f2 * t1[m] - f1 * t0[m]) + (f4 * ta1[m] - f3 * ta0[m]) + (f6 * tb1[m] - f5 * tb0[m]);
  }
  const double div = (g[0][0] + g[1][1] + g[2][2]) * c->cvisq;
  const double f1 = g[0][0] - div, f2 = g[0][1] + g[1][0], f3 = g[0][2] + g[2][0];
  const double f4 = g[1][1] - div, f5 = g[1][2] + g[2][1], f6 = g[2][2] - div;
  const double volinv = 1. / (c->vol[lt] + c->vol[ltm]);
  double xmutvol, xktvol, xmutvol_sa = 0.;
  if (c->neq == 6) {
    sa_mut(c, il, ir, volinv, &xmutvol, &xktvol, &xmutvol_sa);
  } else {
    xmutvol = (c->xmut[ir] + c->xmut[il]) * volinv;
    xktvol = xmutvol * c->gam3;
  }
  double fv, fv5;
  fv = -(2. * f1 * tcx + f2 * tcy + f3 * tcz) * xmutvol;
  fv5 = fv * (rop[ir + nd] + rop[il + nd]);
  flu[1] = flu[1] + fv;
  fv = -(f2 * tcx + 2. * f4 * tcy + f5 * tcz) * xmutvol;
  fv5 = fv5 + fv * (rop[ir + 2 * nd] + rop[il + 2 * nd]);
  flu[2] = flu[2] + fv;
  fv = -(f3 * tcx + f5 * tcy + 2. * f6 * tcz) * xmutvol;
  fv5 = fv5 + fv * (rop[ir + 3 * nd] + rop[il + 3 * nd]);
  flu[3] = flu[3] + fv;
  fv = fv5 * 0.5 - (g[3][0] * tcx + g[3][1] * tcy + g[3][2] * tcz) * xktvol;
  flu[4] = flu[4] + fv;
  if (c->neq == 6)   /* SA/fluvisq_SA_3dfull_*.for + assemble_tauij_3dfull.for */
    flu[5] = flu[5] - xmutvol_sa * (g[4][0] * tcx + g[4][1] * tcy + g[4][2] * tcz);
}

/* Viscous face flux on a 2-d zone: Compute/fluvisq_2d_i.for and
 * fluvisq_2d_j.for + mut_interface.for.  The 2-d Green-Gauss gradient of
 * the 3-d general routine without its k faces: faces normal to d at the two
 * cell centres (means of two face vectors) and the faces along the single
 * transverse direction a (four-cell means, factor 1/8); two velocity
 * components, no w row. */
static void visc_2d(const fctx* c, int d, int64_t l, int64_t lt, double tcx, double tcy,
                    double flu[6]) {
  const double* rop = c->rop;
  const int64_t nd = c->nd, ndm = c->ndm;
  const int a = 1 - d;
  const double *TD = d == 0 ? c->ti : c->tj, *TA = d == 0 ? c->tj : c->ti;
  const int64_t mD = c->inc_mtr[d], mA = c->inc_mtr[a], iA = c->inc[a];
  const int64_t ltm = lt - mD, ltp = lt + mD, ltA = lt + mA, ltAm = lt + mA - mD;
  double t0[2], t1[2], ta0[2], ta1[2];
  for (int m = 0; m < 2; m++) {
    const int64_t o = m * ndm;
    t0[m] = .5 * (TD[lt + o] + TD[ltm + o]);
    t1[m] = .5 * (TD[lt + o] + TD[ltp + o]);
    ta0[m] = .125 * (TA[lt + o] + TA[ltm + o]);
    ta1[m] = .125 * (TA[ltA + o] + TA[ltAm + o]);
  }
  const int64_t il = l - c->inc[d], ir = l;
  double g[3][2];                         /* u, v, T */
  const int var[3] = {1, 2, 4};
  for (int v = 0; v < 3; v++) {
    const double* q = rop + var[v] * nd;
    double f1 = q[il], f2 = q[ir];
    double f3 = q[ir] + q[il] + q[il - iA] + q[ir - iA];
    double f4 = q[ir] + q[il] + q[il + iA] + q[ir + iA];
    for (int m = 0; m < 2; m++) g[v][m] = (f2 * t1[m] - f1 * t0[m]) + (f4 * ta1[m] - f3 * ta0[m]);
  }
  const double div = (g[0][0] + g[1][1]) * c->cvisq;
  const double f1 = g[0][0] - div, f2 = g[0][1] + g[1][0], f4 = g[1][1] - div;
  const double volinv = 1. / (c->vol[lt] + c->vol[ltm]);
  double xmutvol, xktvol, xmutvol_sa = 0.;
  if (c->neq == 6) {   /* SA/fluvisq_2d_*.for: mut_prandtltb_interface.for */
    sa_mut(c, il, ir, volinv, &xmutvol, &xktvol, &xmutvol_sa);
  } else {
    xmutvol = (c->xmut[ir] + c->xmut[il]) * volinv;
    xktvol = xmutvol * c->gam3;
  }
  double fv, fv5;
  fv = -(2. * f1 * tcx + f2 * tcy) * xmutvol;
  fv5 = fv * (rop[ir + nd] + rop[il + nd]);
  flu[1] = flu[1] + fv;
  fv = -(f2 * tcx + 2. * f4 * tcy) * xmutvol;
  fv5 = fv5 + fv * (rop[ir + 2 * nd] + rop[il + 2 * nd]);
  flu[2] = flu[2] + fv;
  fv = fv5 * 0.5 - (g[2][0] * tcx + g[2][1] * tcy) * xktvol;
  flu[4] = flu[4] + fv;
  if (c->neq == 6) {   /* SA/fluvisq_SA_2d_*.for: diffusion of nutilde */
    const double* q = rop + 5 * nd;
    double f1n = q[il], f2n = q[ir];
    double f3n = q[ir] + q[il] + q[il - iA] + q[ir - iA];
    double f4n = q[ir] + q[il] + q[il + iA] + q[ir + iA];
    double gx = (f2n * t1[0] - f1n * t0[0]) + (f4n * ta1[0] - f3n * ta0[0]);
    double gy = (f2n * t1[1] - f1n * t0[1]) + (f4n * ta1[1] - f3n * ta0[1]);
    flu[5] = flu[5] - xmutvol_sa * (gx * tcx + gy * tcy);
  }
}

/* Roe flux of ro * nutilde (ROE/3dfull/fluFaceSA_*_3dfull_i.for and the
 * 3dcart variants): first-order states (cells nm = l - inc and l, no slope),
 * upwinding by the Roe-averaged normal velocity with the floor c1 |S|:
 * flu6 = (qm6 + qp6 - tdu (nu_l ro_l - nu_nm ro_nm)) / 2.  Cartesian faces
 * take the normal velocity from their one component (Vit_ent/qn_3dcart_*). */
static double roe_sa_flux(const fctx* c, int d, int64_t l, int64_t nm, double tcx, double tcy,
                          double tcz, double s) {
  const double* rop = c->rop;
  const int64_t nd = c->nd;
  const double t[3] = {tcx, tcy, tcz};
  double qp[3] = {rop[nm + nd], rop[nm + 2 * nd], rop[nm + 3 * nd]};
  const double qm[3] = {rop[l + nd], rop[l + 2 * nd], rop[l + 3 * nd]};
  const int cart = c->typ == 2, two_d = c->typ == 3;
  double qn1 = cart ? qp[d] * t[d] : (two_d ? qp[0] * tcx + qp[1] * tcy : qp[0] * tcx + qp[1] * tcy + qp[2] * tcz);
  const double qn2 = cart ? qm[d] * t[d] : (two_d ? qm[0] * tcx + qm[1] * tcy : qm[0] * tcx + qm[1] * tcy + qm[2] * tcz);
  double qp1 = rop[nm], qm1 = rop[l];
  const double qm6 = rop[l + 5 * nd] * qm1 * qn2;
  const double qp6 = rop[nm + 5 * nd] * qp1 * qn1;
  qp1 = sqrt(qp1);
  qm1 = sqrt(qm1);
  const double r_1 = 1. / (qp1 + qm1);
  for (int m = 0; m < 3; m++) qp[m] = r_1 * (qp1 * qp[m] + qm1 * qm[m]);
  qn1 = cart ? qp[d] * t[d] : (two_d ? qp[0] * tcx + qp[1] * tcy : qp[0] * tcx + qp[1] * tcy + qp[2] * tcz);
  const double s_1 = 1.0 / OMAX(s, 1.e-30);
  const double tdu = OMAX(c->c1 / s_1, fabs(qn1));
  return 0.5 * (qm6 + qp6 - tdu * (rop[l + 5 * nd] * rop[l] - rop[nm + 5 * nd] * rop[nm]));
}

/* One face flux (convective + viscous) of direction d at cell (i,j,k). */
static void face_flux(const fctx* c, int d, int64_t i, int64_t j, int64_t k, double flu[6]) {
  int64_t l = inddm(c->pi, i, j, k);
  int64_t lt = indmtr(c->pi, i, j, k);
  double qm[6], qp[6], tcx, tcy, tcz, s;
  slopes(c, l, d, qm, qp);
  if (c->typ == 2) {
    tcx = d == 0 ? c->tcx : 0.; tcy = d == 1 ? c->tcy : 0.; tcz = d == 2 ? c->tcz : 0.;
    s = d == 0 ? c->si : (d == 1 ? c->sj : c->sk);
  } else {
    face_normal(c, d, lt, &tcx, &tcy, &tcz, &s);
  }
  if (c->kflu == 5) {
    roe_face(c, qm, qp, tcx, tcy, tcz, s, flu);
    if (c->neq == 6) flu[5] = roe_sa_flux(c, d, l, l - c->inc[d], tcx, tcy, tcz, s);
  } else ausm_face(c, qm, qp, c->rop[l + 4 * c->nd], tcx, tcy, tcz, s,
                 c->wig ? c->wig[l + d * c->nd] : 0., flu);
  if (c->iflow >= 2) {
    if (c->typ == 2) visc_cart(c, d, l, flu);
    else if (c->typ == 3) visc_2d(c, d, l, lt, tcx, tcy, flu);
    else visc_full(c, d, l, lt, tcx, tcy, tcz, flu);
  }
}

/* BC/correct_flux.for with lapply = 4 (wall BCs with the Roe scheme), in
 * BC order, for each face of the wall window (the face between the first
 * interior cell l0 and its ghost): drodm(l0) += F_roe * sens_c + 0 with the
 * Euler Roe flux of that face (corr_fluroe_euler_*: the balance's flux
 * removed), then drodm(l0) += F_wall * sens_w (CL_correction_flu.for:
 * bflwallslip.for for BCWallInviscid / BCSymmetryPlane, bflwall.for for
 * BCWall / BCWallViscous). */
void or_correct_flux(const int64_t* pi, const double* pr, const double* rop, double* drodm,
                     const double* xmut, const double* ti, const double* tj, const double* tk,
                     const double* vol, const double* wig) {
  if (pi[KFLUDOM] != 5) return;
  int64_t pt_bcs = pi[PT_BC];
  if (pt_bcs <= 0) return;
  fctx c;
  fctx_init(&c, pi, pr, rop, xmut, ti, tj, tk, vol);
  c.wig = wig;   /* o3sc: the shock-sensor weights of the wall faces */
  c.iflow = 1;   /* Euler part only */
  const int64_t nd = pi[NDIMDX];
  const double rgp = pr[CVINF] * (pr[GAMMA] - 1.), gam2 = pr[GAMMA] / (pr[GAMMA] - 1.);
  for (int64_t n = 0; n < pi[pt_bcs]; n++) {
    const int64_t pt = pi[pt_bcs + 1 + n], type = pi[pt + BC_TYPE];
    if (type != 3 && type != 4 && type != 6) continue;
    const int idir = (int)pi[pt + BC_IDIR];
    int64_t cl[6];
    bc_window(pi, pi + pt + BC_FEN, idir, cl);
    const int d = (idir - 1) / 2, low = idir % 2;
    /* the face layer: cell 1 (low faces) or the first ghost n_d + 1 (high) */
    const int64_t fc = low ? 1 : pi[IJKV + d] + 1;
    cl[2 * d] = fc; cl[2 * d + 1] = fc;
    const int64_t inc = c.inc[d];
    const double sens_c = low ? -1. : 1., sens_w = low ? 1. : -1.;
    for (int64_t k = cl[4]; k <= cl[5]; k++)
      for (int64_t j = cl[2]; j <= cl[3]; j++)
        for (int64_t i = cl[0]; i <= cl[1]; i++) {
          const int64_t l = inddm(pi, i, j, k), iadrf = l - inc, l0 = low ? l : l - inc;
          double flu[6];
          face_flux(&c, d, i, j, k, flu);
          for (int v = 0; v < 5; v++) drodm[l0 + v * nd] = drodm[l0 + v * nd] + (flu[v] * sens_c + 0.);
          double t[3];
          bc_normal(pi, ti, tj, tk, idir, i, j, k, t);
          const double qen = 0.;
          const double r = 0.5 * (rop[l] + rop[iadrf]);
          const double u = 0.5 * (rop[l + nd] + rop[iadrf + nd]);
          const double v = 0.5 * (rop[l + 2 * nd] + rop[iadrf + 2 * nd]);
          const double w = 0.5 * (rop[l + 3 * nd] + rop[iadrf + 3 * nd]);
          const double u_int = t[0] * u + t[1] * v + t[2] * w - qen;
          double fw[5];
          if (type == 3) {    /* bflwallslip.for */
            double p = rop[iadrf + 4 * nd] * rop[iadrf] * rgp;
            const double h = gam2 * p + r * (u * u + v * v + w * w) * 0.5;
            p = 0.5 * (rop[l + 4 * nd] * rop[l] + rop[iadrf + 4 * nd] * rop[iadrf]) * rgp;
            fw[0] = u_int * r;
            fw[1] = t[0] * p + u_int * r * u;
            fw[2] = t[1] * p + u_int * r * v;
            fw[3] = t[2] * p + u_int * r * w;
            fw[4] = u_int * h + p * qen;
          } else {            /* bflwall.for */
            const double p = 0.5 * (rop[l + 4 * nd] * rop[l] + rop[iadrf + 4 * nd] * rop[iadrf]) * rgp;
            fw[0] = 0.;
            fw[1] = t[0] * p + u_int * u * r;
            fw[2] = t[1] * p + u_int * v * r;
            fw[3] = t[2] * p + u_int * w * r;
            fw[4] = p * qen;
          }
          for (int m = 0; m < 5; m++) drodm[l0 + m * nd] = drodm[l0 + m * nd] + fw[m] * sens_w;
        }
  }
}

/* Flux balance of template_FluxAndBalance.for:192-271 for one zone: every
 * face flux is computed once; each interior cell then receives, in the
 * order the reference's k/j/i loop nest produces, drodm + F_k(lo) + F_j(lo)
 * + F_i(lo) - F_i(hi) - F_j(hi) - F_k(hi). */
/* SENSOR/wiggle2001.for + wiggle.for (3-d): for the d-face of cell l,
 * f_v = sign(1, (q_{l-1}-q_{l-2})(q_l-q_{l-1})) + sign(1, (q_l-q_{l-1})(q_{l+1}-q_l))
 * for the 5 variables; wig = 1 if min_v f_v < -1e-12.  Cells of ind plus
 * the imax+1 / jmax+1 / kmax+1 planes of the last faces. */
static double wig_face(const int64_t* pi, const double* rop, int64_t l, int64_t inc) {
  const int64_t nd = pi[NDIMDX], nm = l - inc, nm2 = l - 2 * inc, np = l + inc;
  const int two_d = pi[ITYPZONE] == 3;   /* wiggle2d_{i,j}.for: min(f1, f2, f3, f5) */
  double test = 0.;
  for (int v = 0; v < 5; v++) {
    if (two_d && v == 3) continue;
    const double* q = rop + v * nd;
    double qm = (q[nm] - q[nm2]) * (q[l] - q[nm]);
    double qp = (q[l] - q[nm]) * (q[np] - q[l]);
    double f = fsign(1., qm) + fsign(1., qp);
    test = v == 0 ? f : OMIN(test, f);
  }
  return test < -1e-12 ? 1. : 0.;
}

void or_wiggle(const int64_t* pi, const int64_t* ind, const double* rop, double* wig) {
  const int64_t nd = pi[NDIMDX];
  const int64_t inc[3] = {1, pi[NIJK], pi[NIJK] * pi[NIJK + 1]};
  const int64_t hi[3] = {ind[1], ind[3], ind[5]};
  const int64_t corr[3] = {ind[1] == pi[IJKV], ind[3] == pi[IJKV + 1], ind[5] == pi[IJKV + 2]};
  const int ndir = pi[ITYPZONE] == 3 ? 2 : 3;   /* 2-d: i and j faces */
  for (int d = 0; d < ndir; d++)
    for (int64_t k = ind[4]; k <= ind[5] + (d == 2 ? corr[2] : 0); k++)
      for (int64_t j = ind[2]; j <= ind[3] + (d == 1 ? corr[1] : 0); j++)
        for (int64_t i = ind[0]; i <= ind[1] + (d == 0 ? corr[0] : 0); i++) {
          const int64_t l = inddm(pi, i, j, k);
          wig[l + d * nd] = wig_face(pi, rop, l, inc[d]);
        }
  (void)hi;
}

/* The velocity divergence and the squared vorticity of cell (i,j,k) from
 * the face-averaged velocities (SA/div_rot_3dcart.for, SA/div_rot_3dfull.for,
 * SA/div_rot_2d.for) and the cell's face-metric norms tc[d]
 * (SENSOR/sciacovelli.for:186-200 for cartesian zones, SA/metric_3dfull.for,
 * SA/metric_2d.for). */
static void div_rot(const int64_t* pi, const double* rop, const double* ti, const double* tj,
                    const double* tk, const double* vol, int64_t i, int64_t j, int64_t k,
                    double* div, double* rot, double tc[3]) {
  const int64_t nd = pi[NDIMDX], l = inddm(pi, i, j, k);
  const int typ = (int)pi[ITYPZONE];
  const int64_t incj = pi[NIJK], inck = pi[NIJK] * pi[NIJK + 1];
  const int64_t l1 = l + 1, l2 = l - 1, l3 = l + incj, l4 = l - incj, l5 = l + inck, l6 = l - inck;
  double u1[3], u2[3], u3[3], u4[3], u5[3], u6[3];
  const int nvel = typ == 3 ? 2 : 3;
  for (int m = 0; m < nvel; m++) {
    const double* q = rop + (m + 1) * nd;
    u1[m] = q[l] + q[l2]; u2[m] = q[l] + q[l3]; u3[m] = q[l] + q[l1]; u4[m] = q[l] + q[l4];
    if (typ != 3) { u5[m] = q[l] + q[l5]; u6[m] = q[l] + q[l6]; }
  }
  double dudx, rotx = 0., roty = 0., rotz;
  if (typ == 2) {
    const double tix = ti[0], tjy = tj[0], tkz = tk[0], xvol = 0.5 / vol[0];
    tc[0] = fabs(tix); tc[1] = fabs(tjy); tc[2] = fabs(tkz);
    dudx = (u3[0] - u1[0]) * tix;
    rotz = -(u2[0] - u4[0]) * tjy;
    roty = (u5[0] - u6[0]) * tkz;
    *div = dudx * xvol;
    dudx = (u3[1] - u1[1]) * tix;
    rotz = (rotz + dudx) * xvol;
    dudx = (u2[1] - u4[1]) * tjy;
    *div = *div + dudx * xvol;
    dudx = (u5[1] - u6[1]) * tkz;
    rotx = -dudx;
    dudx = (u3[2] - u1[2]) * tix;
    roty = (roty - dudx) * xvol;
    dudx = (u2[2] - u4[2]) * tjy;
    rotx = (rotx + dudx) * xvol;
    dudx = (u5[2] - u6[2]) * tkz;
    *div = *div + dudx * xvol;
    *rot = rotx * rotx + roty * roty + rotz * rotz;
    return;
  }
  const int64_t lt = indmtr(pi, i, j, k), ndm = pi[NDIMDX_MTR];
  const int64_t im = pi[NIJK_MTR], jm = pi[NIJK_MTR + 1], km = pi[NIJK_MTR + 2];
  const double xvol = 0.5 / vol[lt];
  if (typ == 3) {
    const double tix = ti[lt], tiy = ti[lt + ndm], tix1 = ti[lt + im], tiy1 = ti[lt + im + ndm];
    const double tjx = tj[lt], tjy = tj[lt + ndm], tjx1 = tj[lt + jm], tjy1 = tj[lt + jm + ndm];
    double t = sqrt(tix * tix + tiy * tiy);
    t = t + sqrt(tix1 * tix1 + tiy1 * tiy1);
    tc[0] = OMAX(.5 * t, 1.e-27);
    t = sqrt(tjx * tjx + tjy * tjy);
    t = t + sqrt(tjx1 * tjx1 + tjy1 * tjy1);
    tc[1] = OMAX(.5 * t, 1.e-27);
    tc[2] = 1.;
#define G2(m, x) (u3[m] * ti##x##1 - u1[m] * ti##x + u2[m] * tj##x##1 - u4[m] * tj##x)
    dudx = G2(0, x);
    *div = dudx * xvol;
    rotz = -G2(0, y);
    dudx = G2(1, x);
    rotz = (rotz + dudx) * xvol;
    dudx = G2(1, y);
    *div = *div + dudx * xvol;
#undef G2
    *rot = rotz * rotz;
    return;
  }
  const double tix = ti[lt], tiy = ti[lt + ndm], tiz = ti[lt + 2 * ndm];
  const double tix1 = ti[lt + im], tiy1 = ti[lt + im + ndm], tiz1 = ti[lt + im + 2 * ndm];
  const double tjx = tj[lt], tjy = tj[lt + ndm], tjz = tj[lt + 2 * ndm];
  const double tjx1 = tj[lt + jm], tjy1 = tj[lt + jm + ndm], tjz1 = tj[lt + jm + 2 * ndm];
  const double tkx = tk[lt], tky = tk[lt + ndm], tkz = tk[lt + 2 * ndm];
  const double tkx1 = tk[lt + km], tky1 = tk[lt + km + ndm], tkz1 = tk[lt + km + 2 * ndm];
  double t = sqrt(tix * tix + tiy * tiy + tiz * tiz);
  t = t + sqrt(tix1 * tix1 + tiy1 * tiy1 + tiz1 * tiz1);
  tc[0] = OMAX(.5 * t, 1.e-27);
  t = sqrt(tjx * tjx + tjy * tjy + tjz * tjz);
  t = t + sqrt(tjx1 * tjx1 + tjy1 * tjy1 + tjz1 * tjz1);
  tc[1] = OMAX(.5 * t, 1.e-27);
  t = sqrt(tkx * tkx + tky * tky + tkz * tkz);
  t = t + sqrt(tkx1 * tkx1 + tky1 * tky1 + tkz1 * tkz1);
  tc[2] = OMAX(.5 * t, 1.e-27);
#define G3(m, x) (u3[m] * ti##x##1 - u1[m] * ti##x + u2[m] * tj##x##1 - u4[m] * tj##x + \
                  u5[m] * tk##x##1 - u6[m] * tk##x)
  dudx = G3(0, x);
  *div = dudx * xvol;
  rotz = -G3(0, y);
  roty = G3(0, z);
  dudx = G3(1, x);
  rotz = (rotz + dudx) * xvol;
  dudx = G3(1, y);
  *div = *div + dudx * xvol;
  dudx = G3(1, z);
  rotx = -dudx;
  dudx = G3(2, x);
  roty = (roty - dudx) * xvol;
  dudx = G3(2, y);
  rotx = (rotx + dudx) * xvol;
  dudx = G3(2, z);
  *div = *div + dudx * xvol;
#undef G3
  *rot = rotx * rotx + roty * roty + rotz * rotz;
}

/* SENSOR/sciacovelli.for + SENSOR/shock_sensor.for: the directional shock
 * sensor of the o3sc slope, wig(l + sl_d) = 1 - min(2 div^2 / (div^2 + rot
 * + 1e-15) * J_d * M, 1), with Jameson's pressure switch J_d =
 * |p(l-inc) - 2 p(l) + p(l+inc)| / |p(l-inc) + 2 p(l) + p(l+inc)| (p = rho T)
 * and the dilatation weight M = (1 - tanh(2.5 + 10 div / (tc_d c))) / 2.
 * Cells of ind plus, at the zone's high edges, the next cell layer of the
 * direction (its faces close the zone), as the loopPlan corrections do.
 * sl_d = d * NDIMDX, shifted by 3 * NDIMDX when the senseur scheme keeps its
 * wiggle flags in the first three. */
void or_shock_sensor(const int64_t* pi, const double* pr, const int64_t* ind, const double* rop,
                     const double* ti, const double* tj, const double* tk, const double* vol,
                     double* wig) {
  const int64_t nd = pi[NDIMDX];
  const double gam = pr[GAMMA], rgp = pr[CVINF] * (gam - 1.);
  const int64_t inc[3] = {1, pi[NIJK], pi[NIJK] * pi[NIJK + 1]};
  const int64_t corr[3] = {ind[1] == pi[IJKV], ind[3] == pi[IJKV + 1], ind[5] == pi[IJKV + 2]};
  const int ndir = pi[ITYPZONE] == 3 ? 2 : 3;
  const int64_t shift = pi[KFLUDOM] == 2 ? 3 * nd : 0;
  if (ind[0] > ind[1] || ind[2] > ind[3] || ind[4] > ind[5]) return;
  for (int64_t k = ind[4]; k <= ind[5] + (ndir == 3 ? corr[2] : 0); k++)
    for (int64_t j = ind[2]; j <= ind[3] + corr[1]; j++)
      for (int64_t i = ind[0]; i <= ind[1] + corr[0]; i++) {
        const int out[3] = {i > ind[1], j > ind[3], k > ind[5]};
        if (out[0] + out[1] + out[2] > 1) continue;
        const int64_t l = inddm(pi, i, j, k);
        double div, rot, tc[3];
        div_rot(pi, rop, ti, tj, tk, vol, i, j, k, &div, &rot, tc);
        for (int d = 0; d < ndir; d++) {
          if (out[(d + 1) % 3] || out[(d + 2) % 3]) continue;   /* only the d-layer extends */
          double mach = sqrt(gam * rgp * rop[l + 4 * nd]);
          mach = 10.0 * (1.0 / tc[d]) * (1.0 / mach) * div;
          mach = 0.5 * (1.0 - tanh(2.5 + mach));
          const int64_t n = inc[d];
          const double p2 = rop[l - n] * rop[l - n + 4 * nd];
          const double p0 = rop[l] * rop[l + 4 * nd];
          const double p1 = rop[l + n] * rop[l + n + 4 * nd];
          double w = fabs(p2 - 2. * p0 + p1) / fabs(p2 + 2. * p0 + p1);
          w = OMIN(2.0 * div * div / (div * div + rot + 1e-15) * w * mach, 1.0);
          wig[l + d * nd + shift] = 1.0 - w;
        }
      }
}

void or_flux(const int64_t* pi, const double* pr, const int64_t* ind,
             const double* rop, double* drodm, const double* xmut,
             const double* ti, const double* tj, const double* tk, const double* vol,
             const double* wig) {
  fctx c;
  fctx_init(&c, pi, pr, rop, xmut, ti, tj, tk, vol);
  c.wig = wig;
  int64_t ni = ind[1] - ind[0] + 1, nj = ind[3] - ind[2] + 1, nk = ind[5] - ind[4] + 1;
  int two_d = (c.typ == 3);
  int64_t fi = (ni + 1) * nj * nk, fj = ni * (nj + 1) * nk, fk = ni * nj * (nk + 1);
  const int neq = c.neq;
  double* Fi = (double*)malloc(sizeof(double) * neq * fi);
  double* Fj = (double*)malloc(sizeof(double) * neq * fj);
  double* Fk = two_d ? NULL : (double*)malloc(sizeof(double) * neq * fk);
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int64_t kk = 0; kk < nk + 1; kk++) {
    double flu[6];
    int64_t k = ind[4] + kk;
    for (int64_t jj = 0; jj < nj + 1; jj++)
      for (int64_t ii = 0; ii < ni + 1; ii++) {
        int64_t i = ind[0] + ii, j = ind[2] + jj;
        if (kk < nk && jj < nj) {
          face_flux(&c, 0, i, j, k, flu);
          for (int v = 0; v < neq; v++) Fi[v * fi + ii + (ni + 1) * (jj + nj * kk)] = flu[v];
        }
        if (kk < nk && ii < ni) {
          face_flux(&c, 1, i, j, k, flu);
          for (int v = 0; v < neq; v++) Fj[v * fj + ii + ni * (jj + (nj + 1) * kk)] = flu[v];
        }
        if (!two_d && jj < nj && ii < ni) {
          face_flux(&c, 2, i, j, k, flu);
          for (int v = 0; v < neq; v++) Fk[v * fk + ii + ni * (jj + nj * kk)] = flu[v];
        }
      }
  }
  int64_t nd = pi[NDIMDX];
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int64_t kk = 0; kk < nk; kk++)
    for (int64_t jj = 0; jj < nj; jj++)
      for (int64_t ii = 0; ii < ni; ii++) {
        int64_t l = inddm(pi, ind[0] + ii, ind[2] + jj, ind[4] + kk);
        int64_t ai = ii + (ni + 1) * (jj + nj * kk);
        int64_t aj = ii + ni * (jj + (nj + 1) * kk);
        int64_t ak = ii + ni * (jj + nj * kk);
        for (int v = 0; v < neq; v++) {
          double x = drodm[l + v * nd];
          if (!two_d) x = x + Fk[v * fk + ak];
          x = x + Fj[v * fj + aj];
          x = x + Fi[v * fi + ai];
          x = x - Fi[v * fi + ai + 1];
          x = x - Fj[v * fj + aj + ni];
          if (!two_d) x = x - Fk[v * fk + ak + ni * nj];
          drodm[l + v * nd] = x;
        }
      }
  free(Fi); free(Fj); free(Fk);
}

/* ======================================================================
 * core3ark3 -- FastS/FastS/Compute/core3ark3.for:6-150 (RK3 low storage,
 * B = 0.5, 0.9106836025229591, 0.3660254037844387; prim <-> cons update)
 * ====================================================================== */
void or_core3ark3(const int64_t* pi, const double* pr, int nitcfg, const int64_t* ind,
                  double* rop_1, const double* rop, const double* drodm, const double* coe) {
  const double cgamma1 = 0.5, cgamma2 = 0.9106836025229591, cgamma3 = 0.3660254037844387;
  int64_t nd = pi[NDIMDX];
  double cv = pr[CVINF], cvinv = 1. / cv, cvinv2 = 0.5 * cvinv;
  int64_t b = pi[RK];
  double coefW = 0.;
  if (b == 1) { if (nitcfg == 1) coefW = 1.; }
  else if (b == 2) { if (nitcfg == 1) coefW = 1.; else if (nitcfg == 2) coefW = 0.5; }
  else if (b == 3) {
    if (nitcfg == 1) coefW = cgamma1;
    else if (nitcfg == 2) coefW = cgamma2;
    else if (nitcfg == 3) coefW = cgamma3;
  }
  int two_d = pi[ITYPZONE] == 3;
  const int sa = pi[NEQ] == 6;
  const double cmus1 = pr[CS], temp01 = 1. / pr[TEMP0];
  const double coesut = pr[XMUL0] * (1. + cmus1 * temp01);
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int64_t k = ind[4]; k <= ind[5]; k++)
    for (int64_t j = ind[2]; j <= ind[3]; j++)
      for (int64_t i = ind[0]; i <= ind[1]; i++) {
        int64_t l = inddm(pi, i, j, k);
        double r_1 = coefW * coe[l];
        double tab1 = drodm[l] * r_1, tab2 = drodm[l + nd] * r_1, tab3 = drodm[l + 2 * nd] * r_1;
        double tab4 = drodm[l + 3 * nd] * r_1, tab5 = drodm[l + 4 * nd] * r_1;
        double ro_old = rop[l], u_old = rop[l + nd], v_old = rop[l + 2 * nd];
        double w_old = rop[l + 3 * nd], t_old = rop[l + 4 * nd];
        rop_1[l] = rop[l] + tab1;
        r_1 = 1. / rop_1[l];
        rop_1[l + nd] = (ro_old * u_old + tab2) * r_1;
        rop_1[l + 2 * nd] = (ro_old * v_old + tab3) * r_1;
        if (!two_d) {
          rop_1[l + 3 * nd] = (ro_old * w_old + tab4) * r_1;
          double roe_old = ro_old * (cv * t_old + 0.5 * (u_old * u_old + v_old * v_old + w_old * w_old));
          rop_1[l + 4 * nd] = (roe_old + tab5) * r_1 * cvinv -
              cvinv2 * (rop_1[l + nd] * rop_1[l + nd] + rop_1[l + 2 * nd] * rop_1[l + 2 * nd] +
                        rop_1[l + 3 * nd] * rop_1[l + 3 * nd]);
          if (sa) {   /* core3ark3.for:188-236: nutilde limited to [0, ratiom nu_lam] */
            double tab6 = drodm[l + 5 * nd] * (coefW * coe[l]);
            double anulam = sa_mulam(coesut, temp01, cmus1, rop_1[l + 4 * nd]);
            anulam = anulam * r_1 * pr[SA_RATIOM_R];
            double t6 = (ro_old * rop[l + 5 * nd] + tab6) * r_1;
            t6 = OMIN(t6, anulam);
            rop_1[l + 5 * nd] = OMAX(t6, 0.);
          }
        } else {
          rop_1[l + 3 * nd] = 0.;
          double roe_old = ro_old * (cv * t_old + 0.5 * (u_old * u_old + v_old * v_old));
          rop_1[l + 4 * nd] = (roe_old + tab5) * r_1 * cvinv -
              cvinv2 * (rop_1[l + nd] * rop_1[l + nd] + rop_1[l + 2 * nd] * rop_1[l + 2 * nd]);
          if (sa) {   /* core3ark3.for:238-276 (2-d) */
            double tab6 = drodm[l + 5 * nd] * (coefW * coe[l]);
            double anulam = sa_mulam(coesut, temp01, cmus1, rop_1[l + 4 * nd]);
            anulam = anulam * r_1 * pr[SA_RATIOM_R];
            double t6 = (ro_old * rop[l + 5 * nd] + tab6) * r_1;
            t6 = OMIN(t6, anulam);
            rop_1[l + 5 * nd] = OMAX(t6, 0.);
          }
        }
      }
}

/* ======================================================================
 * core3as2 -- FastS/FastS/Compute/core3as2.for:233-374 (5 eq.): dual time
 * Newton residual; BDF1 on the first physical step, BDF2 after.
 * ====================================================================== */
void or_core3as2(const int64_t* pi, const double* pr, int nitcfg, int first_it,
                 const int64_t* ind, const double* rop, const double* rop_n,
                 const double* rop_n1, double* drodm, const double* coe) {
  int64_t nd = pi[NDIMDX];
  double cv = pr[CVINF];
  double c1, c2, c3;
  if (first_it == 0 || pi[DTLOC] == 1) { c1 = -1.; c2 = 1.; c3 = 0.; }
  else { c1 = -1.5; c2 = 2.; c3 = -0.5; }
  int two_d = pi[ITYPZONE] == 3;
  const int sa = pi[NEQ] == 6;
  double c4 = c1 + c2;
#pragma omp parallel for num_threads(g_threads) schedule(static)
  for (int64_t k = ind[4]; k <= ind[5]; k++)
    for (int64_t j = ind[2]; j <= ind[3]; j++)
      for (int64_t i = ind[0]; i <= ind[1]; i++) {
        int64_t l = inddm(pi, i, j, k);
        const double *a = rop, *b = rop_n, *m = rop_n1;
        double cf = coe[l];
        if (nitcfg == 1 && sa && pi[DTLOC] == 1) {   /* core3as2.for:57-66, 106-114 */
          for (int v = 0; v < 6; v++) {
            if (two_d && v == 3) continue;
            drodm[l + v * nd] = cf * drodm[l + v * nd];
          }
        } else if (nitcfg == 1) {
          drodm[l] = cf * drodm[l] + c4 * a[l] + c3 * m[l];
          for (int v = 1; v <= 3; v++) {
            if (two_d && v == 3) continue;
            int64_t o = v * nd;
            drodm[l + o] = cf * drodm[l + o] + c4 * a[l + o] * a[l] + c3 * m[l + o] * m[l];
          }
          double roe, roe_n1;
          if (!two_d) {
            roe = a[l] * (cv * a[l + 4 * nd] + 0.5 * (a[l + nd] * a[l + nd] + a[l + 2 * nd] * a[l + 2 * nd] + a[l + 3 * nd] * a[l + 3 * nd]));
            roe_n1 = m[l] * (cv * m[l + 4 * nd] + 0.5 * (m[l + nd] * m[l + nd] + m[l + 2 * nd] * m[l + 2 * nd] + m[l + 3 * nd] * m[l + 3 * nd]));
          } else {
            roe = a[l] * (cv * a[l + 4 * nd] + 0.5 * (a[l + nd] * a[l + nd] + a[l + 2 * nd] * a[l + 2 * nd]));
            roe_n1 = m[l] * (cv * m[l + 4 * nd] + 0.5 * (m[l + nd] * m[l + nd] + m[l + 2 * nd] * m[l + 2 * nd]));
          }
          drodm[l + 4 * nd] = cf * drodm[l + 4 * nd] + c4 * roe + c3 * roe_n1;
          if (sa) {   /* core3as2.for:97-99 */
            int64_t o = 5 * nd;
            drodm[l + o] = cf * drodm[l + o] + c4 * a[l + o] * a[l] + c3 * m[l + o] * m[l];
          }
        } else {
          drodm[l] = cf * drodm[l] + c1 * a[l] + c2 * b[l] + c3 * m[l];
          for (int v = 1; v <= 3; v++) {
            if (two_d && v == 3) continue;
            int64_t o = v * nd;
            drodm[l + o] = cf * drodm[l + o] + c1 * a[l + o] * a[l] + c2 * b[l + o] * b[l] + c3 * m[l + o] * m[l];
          }
          double roe, roe_n, roe_n1;
          if (!two_d) {
            roe = a[l] * (cv * a[l + 4 * nd] + 0.5 * (a[l + nd] * a[l + nd] + a[l + 2 * nd] * a[l + 2 * nd] + a[l + 3 * nd] * a[l + 3 * nd]));
            roe_n = b[l] * (cv * b[l + 4 * nd] + 0.5 * (b[l + nd] * b[l + nd] + b[l + 2 * nd] * b[l + 2 * nd] + b[l + 3 * nd] * b[l + 3 * nd]));
            roe_n1 = m[l] * (cv * m[l + 4 * nd] + 0.5 * (m[l + nd] * m[l + nd] + m[l + 2 * nd] * m[l + 2 * nd] + m[l + 3 * nd] * m[l + 3 * nd]));
          } else {
            roe = a[l] * (cv * a[l + 4 * nd] + 0.5 * (a[l + nd] * a[l + nd] + a[l + 2 * nd] * a[l + 2 * nd]));
            roe_n = b[l] * (cv * b[l + 4 * nd] + 0.5 * (b[l + nd] * b[l + nd] + b[l + 2 * nd] * b[l + 2 * nd]));
            roe_n1 = m[l] * (cv * m[l + 4 * nd] + 0.5 * (m[l + nd] * m[l + nd] + m[l + 2 * nd] * m[l + 2 * nd]));
          }
          drodm[l + 4 * nd] = cf * drodm[l + 4 * nd] + c1 * roe + c2 * roe_n + c3 * roe_n1;
          if (sa) {   /* core3as2.for:187-190 */
            int64_t o = 5 * nd;
            drodm[l + o] = cf * drodm[l + o] + c1 * a[l + o] * a[l] + c2 * b[l + o] * b[l] + c3 * m[l + o] * m[l];
          }
        }
      }
}

/* ======================================================================
 * LU-SGS -- FastS/FastS/Compute/LU/invlu_l.for (lower), invlu_u.for
 * (upper + mjr_newton.for), neighbour terms lu_{i,j,k}_{3dcart,3dfull,2d}.for.
 * ====================================================================== */
typedef struct {
  const int64_t* pi; const double *rop, *coe, *ti, *tj, *tk;
  int64_t nd, ndm, inc[3], inc_mtr[3];
  int typ, neq;
  double gam1, gamm1, cp, gam2;
} luctx;

/* b = B(W_nb) . out_nb for direction d, neighbour l1 (= l - inc for the
 * lower sweep, l + inc for the upper).  signe = +-0.5.  For the 3d full /
 * 2d zones the normal is the mean of the neighbour's two faces in d. */
static void lu_nb(const luctx* c, int d, int64_t l1, int64_t ltnb1, int64_t ltnb2,
                  double signe, const double* out, double b[6]) {
  int64_t nd = c->nd;
  double tcx = 0., tcy = 0., tcz = 0.;
  if (c->typ == 2) {
    if (d == 0) tcx = c->ti[0]; else if (d == 1) tcy = c->tj[0]; else tcz = c->tk[0];
  } else {
    const double* t = d == 0 ? c->ti : (d == 1 ? c->tj : c->tk);
    tcx = 0.5 * (t[ltnb2] + t[ltnb1]);
    tcy = 0.5 * (t[ltnb2 + c->ndm] + t[ltnb1 + c->ndm]);
    if (c->typ == 0) tcz = 0.5 * (t[ltnb2 + 2 * c->ndm] + t[ltnb1 + 2 * c->ndm]);
  }
  double u = c->rop[l1 + nd], v = c->rop[l1 + 2 * nd], w = c->rop[l1 + 3 * nd], t = c->rop[l1 + 4 * nd];
  double gam1 = c->gam1, gamm1 = c->gamm1, gam2 = c->gam2;
  double o1 = out[l1], o2 = out[l1 + nd], o3 = out[l1 + 2 * nd], o4 = out[l1 + 3 * nd], o5 = out[l1 + 4 * nd];
  double cs = c->coe[l1 + (d + 1) * nd] * signe;
  const double o6 = c->neq == 6 ? out[l1 + 5 * nd] : 0.;
  if (c->typ == 2) {
    double q2 = .5 * (u * u + v * v + w * w);
    double h = c->cp * t + q2;
    double ph2 = gamm1 * q2;
    if (d == 0) { /* lu_i_3dcart.for */
      double qn = tcx * u;
      double b11 = cs, b12 = tcx;
      double b21 = (tcx * ph2 - u * qn), b22 = (qn - tcx * gam2 * u) + cs, b23 = (-tcx * gamm1 * v), b24 = (-tcx * gamm1 * w), b25 = tcx * gamm1;
      double b31 = (-v * qn), b32 = (tcx * v), b33 = (qn) + cs;
      double b41 = (-w * qn), b42 = (tcx * w), b44 = (qn) + cs;
      double b51 = qn * (ph2 - h), b52 = (tcx * h - gamm1 * u * qn), b53 = (-gamm1 * v * qn), b54 = (-gamm1 * w * qn), b55 = (gam1 * qn) + cs;
      b[0] = b11 * o1 + b12 * o2;
      b[1] = b21 * o1 + b22 * o2 + b23 * o3 + b24 * o4 + b25 * o5;
      b[2] = b31 * o1 + b32 * o2 + b33 * o3;
      b[3] = b41 * o1 + b42 * o2 + b44 * o4;
      b[4] = b51 * o1 + b52 * o2 + b53 * o3 + b54 * o4 + b55 * o5;
    } else if (d == 1) { /* lu_j_3dcart.for */
      double qn = tcy * v;
      double b11 = cs, b13 = tcy;
      double b21 = (-u * qn), b22 = qn + cs, b23 = tcy * u;
      double b31 = (tcy * ph2 - v * qn), b32 = (-tcy * gamm1 * u), b33 = (qn - tcy * gam2 * v) + cs, b34 = (-tcy * gamm1 * w), b35 = tcy * gamm1;
      double b41 = (-w * qn), b43 = (tcy * w), b44 = (qn) + cs;
      double b51 = qn * (ph2 - h), b52 = (-gamm1 * u * qn), b53 = (tcy * h - gamm1 * v * qn), b54 = (-gamm1 * w * qn), b55 = (gam1 * qn) + cs;
      b[0] = b11 * o1 + b13 * o3;
      b[1] = b21 * o1 + b22 * o2 + b23 * o3;
      b[2] = b31 * o1 + b32 * o2 + b33 * o3 + b34 * o4 + b35 * o5;
      b[3] = b41 * o1 + b43 * o3 + b44 * o4;
      b[4] = b51 * o1 + b52 * o2 + b53 * o3 + b54 * o4 + b55 * o5;
    } else { /* lu_k_3dcart.for */
      double qn = tcz * w;
      double b11 = cs, b14 = tcz;
      double b21 = -u * qn, b22 = qn + cs, b24 = tcz * u;
      double b31 = -v * qn, b33 = qn + cs, b34 = tcz * v;
      double b41 = tcz * ph2 - w * qn, b42 = -tcz * gamm1 * u, b43 = -tcz * gamm1 * v, b44 = (qn - tcz * gam2 * w) + cs, b45 = tcz * gamm1;
      double b51 = qn * (ph2 - h), b52 = -gamm1 * u * qn, b53 = -gamm1 * v * qn, b54 = tcz * h - gamm1 * w * qn, b55 = gam1 * qn + cs;
      b[0] = b11 * o1 + b14 * o4;
      b[1] = b21 * o1 + b22 * o2 + b24 * o4;
      b[2] = b31 * o1 + b33 * o3 + b34 * o4;
      b[3] = b41 * o1 + b42 * o2 + b43 * o3 + b44 * o4 + b45 * o5;
      b[4] = b51 * o1 + b52 * o2 + b53 * o3 + b54 * o4 + b55 * o5;
    }
    /* lu_{i,j,k}_3dcart_SA.for: scalar convection of ro nutilde */
    if (c->neq == 6) {
      double qn = d == 0 ? tcx * u : (d == 1 ? tcy * v : tcz * w);
      b[5] = (qn + cs) * o6;
    }
    return;
  }
  if (c->typ == 0) { /* lu_{i,j,k}_3dfull.for */
    double q2 = .5 * (u * u + v * v + w * w);
    double h = c->cp * t + q2;
    double ph2 = gamm1 * q2;
    double qn = tcx * u + tcy * v + tcz * w;
    double b11 = cs, b12 = tcx, b13 = tcy, b14 = tcz;
    double b21 = (tcx * ph2 - u * qn), b22 = (qn - tcx * gam2 * u) + cs, b23 = (tcy * u - tcx * gamm1 * v), b24 = (tcz * u - tcx * gamm1 * w), b25 = tcx * gamm1;
    double b31 = (tcy * ph2 - v * qn), b32 = (tcx * v - tcy * gamm1 * u), b33 = (qn - tcy * gam2 * v) + cs, b34 = (tcz * v - tcy * gamm1 * w), b35 = tcy * gamm1;
    double b41 = (tcz * ph2 - w * qn), b42 = (tcx * w - tcz * gamm1 * u), b43 = (tcy * w - tcz * gamm1 * v), b44 = (qn - tcz * gam2 * w) + cs, b45 = tcz * gamm1;
    double b51 = qn * (ph2 - h), b52 = (tcx * h - gamm1 * u * qn), b53 = (tcy * h - gamm1 * v * qn), b54 = (tcz * h - gamm1 * w * qn), b55 = (gam1 * qn) + cs;
    b[0] = b11 * o1 + b12 * o2 + b13 * o3 + b14 * o4;
    b[1] = b21 * o1 + b22 * o2 + b23 * o3 + b24 * o4 + b25 * o5;
    b[2] = b31 * o1 + b32 * o2 + b33 * o3 + b34 * o4 + b35 * o5;
    b[3] = b41 * o1 + b42 * o2 + b43 * o3 + b44 * o4 + b45 * o5;
    b[4] = b51 * o1 + b52 * o2 + b53 * o3 + b54 * o4 + b55 * o5;
    if (c->neq == 6) b[5] = (qn + cs) * o6;   /* lu_{i,j,k}_3dfull_SA.for */
    return;
  }
  { /* lu_{i,j}_2d.for */
    double q2 = .5 * (u * u + v * v);
    double h = c->cp * t + q2;
    double ph2 = gamm1 * q2;
    double qn = tcx * u + tcy * v;
    double b11 = cs, b12 = tcx, b13 = tcy;
    double b21 = (tcx * ph2 - u * qn), b22 = (qn - tcx * gam2 * u) + cs, b23 = (tcy * u - tcx * gamm1 * v), b25 = tcx * gamm1;
    double b31 = (tcy * ph2 - v * qn), b32 = (tcx * v - tcy * gamm1 * u), b33 = (qn - tcy * gam2 * v) + cs, b35 = tcy * gamm1;
    double b51 = qn * (ph2 - h), b52 = (tcx * h - gamm1 * u * qn), b53 = (tcy * h - gamm1 * v * qn), b55 = (gam1 * qn) + cs;
    b[0] = b11 * o1 + b12 * o2 + b13 * o3;
    b[1] = b21 * o1 + b22 * o2 + b23 * o3 + b25 * o5;
    b[2] = b31 * o1 + b32 * o2 + b33 * o3 + b35 * o5;
    b[3] = 0.;
    b[4] = b51 * o1 + b52 * o2 + b53 * o3 + b55 * o5;
    if (c->neq == 6) b[5] = (qn + cs) * o6;   /* lu_{i,j}_2d_SA.for */
  }
}

/* mjr_newton.for: W^{p+1} = prim(cons(W^p) + dW) */
static void mjr_newton(const int64_t* pi, const double* pr, int64_t l, const double* rop,
                       double* rop_1, const double* out) {
  int64_t nd = pi[NDIMDX];
  double cvinv = 1. / pr[CVINF], cvinv2 = 0.5 * cvinv;
  double ro_old = rop[l], u_old = rop[l + nd], v_old = rop[l + 2 * nd], w_old = rop[l + 3 * nd], t_old = rop[l + 4 * nd];
  double n1 = rop[l] + out[l];
  double r_1 = 1. / n1;
  double n2 = (ro_old * u_old + out[l + nd]) * r_1;
  double n3 = (ro_old * v_old + out[l + 2 * nd]) * r_1;
  const double nu_old = pi[NEQ] == 6 ? rop[l + 5 * nd] : 0.;
  if (pi[ITYPZONE] == 3) {
    double roe_old = ro_old * (pr[CVINF] * t_old + 0.5 * (u_old * u_old + v_old * v_old));
    double n5 = (roe_old + out[l + 4 * nd]) * r_1 * cvinv - cvinv2 * (n2 * n2 + n3 * n3);
    rop_1[l] = n1; rop_1[l + nd] = n2; rop_1[l + 2 * nd] = n3; rop_1[l + 3 * nd] = 0.; rop_1[l + 4 * nd] = n5;
    if (pi[NEQ] == 6) {   /* mjr_newton_2d_SA.for */
      const double cmus1 = pr[CS], temp01 = 1. / pr[TEMP0];
      const double coesut = pr[XMUL0] * (1. + cmus1 * temp01);
      double anulam = sa_mulam(coesut, temp01, cmus1, n5);
      anulam = anulam * r_1 * pr[SA_RATIOM_R];
      double t6 = (ro_old * nu_old + out[l + 5 * nd]) * r_1;
      t6 = OMIN(t6, anulam);
      rop_1[l + 5 * nd] = OMAX(t6, 0.);
    }
    return;
  }
  double n4 = (ro_old * w_old + out[l + 3 * nd]) * r_1;
  double roe_old = ro_old * (pr[CVINF] * t_old + 0.5 * (u_old * u_old + v_old * v_old + w_old * w_old));
  double n5 = (roe_old + out[l + 4 * nd]) * r_1 * cvinv - cvinv2 * (n2 * n2 + n3 * n3 + n4 * n4);
  rop_1[l] = n1; rop_1[l + nd] = n2; rop_1[l + 2 * nd] = n3; rop_1[l + 3 * nd] = n4; rop_1[l + 4 * nd] = n5;
  if (pi[NEQ] == 6) {   /* mjr_newton_SA.for */
    const double cmus1 = pr[CS], temp01 = 1. / pr[TEMP0];
    const double coesut = pr[XMUL0] * (1. + cmus1 * temp01);
    double anulam = sa_mulam(coesut, temp01, cmus1, n5);
    anulam = anulam * r_1 * pr[SA_RATIOM_R];
    double t6 = (ro_old * nu_old + out[l + 5 * nd]) * r_1;
    t6 = OMIN(t6, anulam);
    rop_1[l + 5 * nd] = OMAX(t6, 0.);
  }
}

void or_invlu(const int64_t* pi, const double* pr, const int64_t* ind,
              double* rotmp, double* rop_ssiter, const double* drodm_in,
              double* drodm_out, const double* ti, const double* tj, const double* tk,
              const double* coe, int mjrnewton) {
  if (ind[1] < ind[0]) return;
  luctx c;
  c.pi = pi; c.rop = rop_ssiter; c.coe = coe; c.ti = ti; c.tj = tj; c.tk = tk;
  c.nd = pi[NDIMDX]; c.ndm = pi[NDIMDX_MTR]; c.typ = (int)pi[ITYPZONE];
  c.inc[0] = 1; c.inc[1] = pi[NIJK]; c.inc[2] = pi[NIJK] * pi[NIJK + 1];
  c.inc_mtr[0] = pi[NIJK_MTR]; c.inc_mtr[1] = pi[NIJK_MTR + 1]; c.inc_mtr[2] = pi[NIJK_MTR + 2];
  c.gam1 = pr[GAMMA]; c.gamm1 = c.gam1 - 1.; c.cp = pr[GAMMA] * pr[CVINF]; c.gam2 = c.gamm1 - 1.;
  int64_t nd = c.nd;
  int neq = (int)pi[NEQ];
  c.neq = neq;
  int two_d = c.typ == 3;
  /* lower sweep: invlu_l.for, lexicographic k, j, i.  The neighbour terms
   * present at a cell are those whose neighbour lies inside the LU range;
   * their order is j, k, i on a 3d cartesian zone (invlu_l.for 3dcart
   * section) and k, j, i otherwise. */
  for (int64_t k = ind[4]; k <= ind[5]; k++)
    for (int64_t j = ind[2]; j <= ind[3]; j++)
      for (int64_t i = ind[0]; i <= ind[1]; i++) {
        int64_t l = inddm(pi, i, j, k), lt = indmtr(pi, i, j, k);
        double xal = coe[l] * 0.5;
        double x[6], b[6];
        int first = 1;
        int hasj = j > ind[2], hask = (!two_d) && k > ind[4], hasi = i > ind[0];
        int order[2] = {2, 1};
        if (c.typ == 2) { order[0] = 1; order[1] = 2; }
        for (int v = 0; v < neq; v++) x[v] = drodm_in[l + v * nd];
        for (int o = 0; o < 2; o++) {
          int d = order[o];
          if ((d == 1 && !hasj) || (d == 2 && !hask)) continue;
          lu_nb(&c, d, l - c.inc[d], lt - c.inc_mtr[d], lt, 0.5, drodm_out, b);
          for (int v = 0; v < neq; v++) x[v] = x[v] + b[v] * xal;
          first = 0;
        }
        if (hasi) {
          lu_nb(&c, 0, l - 1, lt - c.inc_mtr[0], lt, 0.5, drodm_out, b);
          for (int v = 0; v < neq; v++) x[v] = x[v] + b[v] * xal;
        }
        (void)first;
        double diag = 1. / coe[l + 4 * nd];
        for (int v = 0; v < 5; v++) drodm_out[l + v * nd] = x[v] * diag;
        if (neq == 6) drodm_out[l + 5 * nd] = x[5] / coe[l + 5 * nd];   /* lu_dinv_SA.for */
        if (two_d) drodm_out[l + 3 * nd] = drodm_in[l + 3 * nd] * diag;
      }
  /* upper sweep: invlu_u.for, reverse lexicographic; out = D^-1 (D out_L
   * + terms k, j, i), then mjr_newton plane by plane (k descending).  When
   * rotmp and rop_ssiter are the same array the k+1 neighbour is read after
   * its plane has been Newton-updated, as in the reference. */
  for (int64_t k = ind[5]; k >= ind[4]; k--) {
    for (int64_t j = ind[3]; j >= ind[2]; j--)
      for (int64_t i = ind[1]; i >= ind[0]; i--) {
        int64_t l = inddm(pi, i, j, k), lt = indmtr(pi, i, j, k);
        double xal = coe[l] * (-0.5);
        double x[6], b[6];
        double dg = coe[l + 4 * nd];
        for (int v = 0; v < 5; v++) x[v] = drodm_out[l + v * nd] * dg;
        if (neq == 6) x[5] = drodm_out[l + 5 * nd] * coe[l + 5 * nd];   /* lu_d_SA.for */
        int hasj = j < ind[3], hask = (!two_d) && k < ind[5], hasi = i < ind[1];
        if (hask) {
          lu_nb(&c, 2, l + c.inc[2], lt + c.inc_mtr[2], lt + 2 * c.inc_mtr[2], -0.5, drodm_out, b);
          for (int v = 0; v < neq; v++) x[v] = x[v] + b[v] * xal;
        }
        if (hasj) {
          lu_nb(&c, 1, l + c.inc[1], lt + c.inc_mtr[1], lt + 2 * c.inc_mtr[1], -0.5, drodm_out, b);
          for (int v = 0; v < neq; v++) x[v] = x[v] + b[v] * xal;
        }
        if (hasi) {
          lu_nb(&c, 0, l + 1, lt + c.inc_mtr[0], lt + 2 * c.inc_mtr[0], -0.5, drodm_out, b);
          for (int v = 0; v < neq; v++) x[v] = x[v] + b[v] * xal;
        }
        double diag = 1. / coe[l + 4 * nd];
        for (int v = 0; v < 5; v++) drodm_out[l + v * nd] = x[v] * diag;
        if (neq == 6) drodm_out[l + 5 * nd] = x[5] / coe[l + 5 * nd];
      }
    if (mjrnewton == 1)
      for (int64_t j = ind[2]; j <= ind[3]; j++)
        for (int64_t i = ind[0]; i <= ind[1]; i++)
          mjr_newton(pi, pr, inddm(pi, i, j, k), rop_ssiter, rotmp, drodm_out);
  }
}

/* ======================================================================
 * cprdu3s1 -- FastS/FastS/Compute/cprdu3s1_incl.for:14-135: per LU block
 * (SIZE_SSDOM cells, the last block of a direction takes the remainder)
 * sum of squares and max |drodm| for each equation, stored at sub-iteration
 * it_bloc: rdm(it_bloc, ne, 1:2, no_rdm) (Fortran order).
 * ====================================================================== */
void or_cprdu3s1(const int64_t* pi, int it_bloc, int nssiter, const double* drodm, double* rdm) {
  int64_t ijkv_lu[3];
  for (int d = 0; d < 3; d++) {
    int64_t q = pi[IJKV + d] / pi[SIZE_SSDOM + d];
    ijkv_lu[d] = q > 1 ? q : 1;
  }
  int64_t neq = pi[NEQ], nd = pi[NDIMDX];
  int64_t nrdm = ijkv_lu[0] * ijkv_lu[1] * ijkv_lu[2];
  for (int64_t no = 0; no < nrdm; no++) {
    int64_t k_lu = no / (ijkv_lu[0] * ijkv_lu[1]);
    int64_t j_lu = (no - ijkv_lu[0] * ijkv_lu[1] * k_lu) / ijkv_lu[0];
    int64_t i_lu = no - j_lu * ijkv_lu[0] - k_lu * ijkv_lu[0] * ijkv_lu[1];
    int64_t lo[3] = {i_lu, j_lu, k_lu}, a[3], b[3];
    for (int d = 0; d < 3; d++) {
      a[d] = 1 + lo[d] * pi[SIZE_SSDOM + d];
      b[d] = (lo[d] + 1) * pi[SIZE_SSDOM + d];
      if (lo[d] == ijkv_lu[d] - 1) b[d] = pi[IJKV + d];
    }
    double xs[6] = {0, 0, 0, 0, 0, 0}, xm[6] = {0, 0, 0, 0, 0, 0};
    for (int64_t k = a[2]; k <= b[2]; k++)
      for (int64_t j = a[1]; j <= b[1]; j++)
        for (int64_t i = a[0]; i <= b[0]; i++) {
          int64_t l = inddm(pi, i, j, k);
          for (int64_t ne = 0; ne < neq; ne++) {
            double dv = drodm[l + ne * nd];
            double xp = fabs(dv);
            if (xp > xm[ne]) xm[ne] = xp;
            xs[ne] = xs[ne] + dv * dv;
          }
        }
    for (int64_t ne = 0; ne < neq; ne++) {
      rdm[(it_bloc - 1) + ne * nssiter + 0 * neq * nssiter + no * neq * 2 * nssiter] = xs[ne];
      rdm[(it_bloc - 1) + ne * nssiter + 1 * neq * nssiter + no * neq * 2 * nssiter] = xm[ne];
    }
  }
}

/* display_ss_iteration.cpp:112-145 */
void or_residual_norms(const int64_t* pi, const double* pr, const double* rdm,
                       int nssiter, int it_bloc, double* out) {
  int64_t ijkv_lu[3];
  for (int d = 0; d < 3; d++) {
    int64_t q = pi[IJKV + d] / pi[SIZE_SSDOM + d];
    ijkv_lu[d] = q > 1 ? q : 1;
  }
  int64_t neq = pi[NEQ];
  double xpt_1 = 1. / (double)(pi[IJKV] * pi[IJKV + 1] * pi[IJKV + 2]);
  for (int64_t ne = 0; ne < neq; ne++)
    for (int i = 0; i < it_bloc; i++) {
      double rmax = 0., rmoy = 0.;
      for (int64_t k_lu = 0; k_lu < ijkv_lu[2]; k_lu++)
        for (int64_t j_lu = 0; j_lu < ijkv_lu[1]; j_lu++)
          for (int64_t i_lu = 0; i_lu < ijkv_lu[0]; i_lu++) {
            int64_t no = i_lu + j_lu * ijkv_lu[0] + k_lu * ijkv_lu[0] * ijkv_lu[1];
            int64_t ind1 = i + ne * nssiter + no * neq * 2 * nssiter;
            int64_t ind2 = i + (ne + neq) * nssiter + no * neq * 2 * nssiter;
            rmax = OMAX(rmax, rdm[ind2]);
            rmoy = rmoy + rdm[ind1];
          }
      out[it_bloc * ne + i] = sqrt(rmoy * xpt_1) / pr[DTC];
      out[it_bloc * (ne + neq) + i] = rmax / pr[DTC];
    }
}

/* ======================================================================
 * Ghost cells: BC/BCzone.cpp:60-865 dispatch with FastC/FastC/BC/
 * indice_cl_sdm.for windows (npass = 0), bvbs_periodique.for (tag 11,
 * ghost <- cell shifted by the zone size), bvbs_extrapolate.for (tag 0,
 * zeroth order); then correct_coins.for for edges and corners.
 * ====================================================================== */
/* ----------------------------------------------------------- metrics
 * FastC/FastC/Metric/cp_tijk.for (faces: normal * area) and cp_vol.for
 * (volumes) for 3-d general (ITYPZONE 0) and 3-d cartesian (2) zones, over
 * every cell including ghosts (indice_omp1.h ind_mtr), plus the last
 * imax+1 / jmax+1 / kmax+1 faces.  x, y, z: vertex coordinates, Fortran
 * order, NIJK_XYZ dimensions.  General zones index the metric on the
 * vertex grid (NIJK_MTR strides 1, nvi, nvi*nvj). */
static void face_i(const double* x, const double* y, const double* z, int64_t l0, int64_t l1,
                   int64_t l2, int64_t l3, double t[3]) {
  double tix10 = (y[l1] - y[l0]) * (z[l3] - z[l0]) - (z[l1] - z[l0]) * (y[l3] - y[l0]);
  double tiy10 = (z[l1] - z[l0]) * (x[l3] - x[l0]) - (x[l1] - x[l0]) * (z[l3] - z[l0]);
  double tiz10 = (x[l1] - x[l0]) * (y[l3] - y[l0]) - (y[l1] - y[l0]) * (x[l3] - x[l0]);
  double tix11 = (y[l2] - y[l3]) * (z[l0] - z[l2]) - (z[l2] - z[l3]) * (y[l0] - y[l2]);
  double tiy11 = (z[l2] - z[l3]) * (x[l0] - x[l2]) - (x[l2] - x[l3]) * (z[l0] - z[l2]);
  double tiz11 = (x[l2] - x[l3]) * (y[l0] - y[l2]) - (y[l2] - y[l3]) * (x[l0] - x[l2]);
  t[0] = .5 * (tix10 + tix11); t[1] = .5 * (tiy10 + tiy11); t[2] = .5 * (tiz10 + tiz11);
}
static void face_j(const double* x, const double* y, const double* z, int64_t l0, int64_t l4,
                   int64_t l2, int64_t l6, double t[3]) {
  double tjx10 = (y[l0] - y[l4]) * (z[l2] - z[l0]) - (z[l0] - z[l4]) * (y[l2] - y[l0]);
  double tjy10 = (z[l0] - z[l4]) * (x[l2] - x[l0]) - (x[l0] - x[l4]) * (z[l2] - z[l0]);
  double tjz10 = (x[l0] - x[l4]) * (y[l2] - y[l0]) - (y[l0] - y[l4]) * (x[l2] - x[l0]);
  double tjx11 = (y[l6] - y[l2]) * (z[l4] - z[l6]) - (z[l6] - z[l2]) * (y[l4] - y[l6]);
  double tjy11 = (z[l6] - z[l2]) * (x[l4] - x[l6]) - (x[l6] - x[l2]) * (z[l4] - z[l6]);
  double tjz11 = (x[l6] - x[l2]) * (y[l4] - y[l6]) - (y[l6] - y[l2]) * (x[l4] - x[l6]);
  t[0] = .5 * (tjx10 + tjx11); t[1] = .5 * (tjy10 + tjy11); t[2] = .5 * (tjz10 + tjz11);
}
static void face_k(const double* x, const double* y, const double* z, int64_t l0, int64_t l4,
                   int64_t l1, int64_t l5, double t[3]) {
  double tkx10 = (y[l4] - y[l0]) * (z[l5] - z[l4]) - (z[l4] - z[l0]) * (y[l5] - y[l4]);
  double tky10 = (z[l4] - z[l0]) * (x[l5] - x[l4]) - (x[l4] - x[l0]) * (z[l5] - z[l4]);
  double tkz10 = (x[l4] - x[l0]) * (y[l5] - y[l4]) - (y[l4] - y[l0]) * (x[l5] - x[l4]);
  double tkx11 = (y[l1] - y[l5]) * (z[l0] - z[l1]) - (z[l1] - z[l5]) * (y[l0] - y[l1]);
  double tky11 = (z[l1] - z[l5]) * (x[l0] - x[l1]) - (x[l1] - x[l5]) * (z[l0] - z[l1]);
  double tkz11 = (x[l1] - x[l5]) * (y[l0] - y[l1]) - (y[l1] - y[l5]) * (x[l0] - x[l1]);
  t[0] = .5 * (tkx10 + tkx11); t[1] = .5 * (tky10 + tky11); t[2] = .5 * (tkz10 + tkz11);
}

void or_metric(const int64_t* pi, const double* x, const double* y, const double* z, double* ti,
               double* tj, double* tk, double* vol) {
  const int64_t nvi = pi[NIJK_XYZ], nvj = pi[NIJK_XYZ + 1], nvk = pi[NIJK_XYZ + 2];
  const int64_t ng = pi[NIJK_XYZ + 3], ngk = pi[NIJK_XYZ + 4];
  const int64_t inci = 1, incj = nvi, inck = nvi * nvj;
#define VX(i, j, k) (((i) + ng - 1) + ((j) + ng - 1) * nvi + ((k) + ngk - 1) * nvi * nvj)
  double t[3];
  if (pi[ITYPZONE] == 2) {
    const int64_t l0 = VX(1, 1, 1), l1 = l0 + incj, l2 = l0 + inck, l3 = l1 + inck;
    const int64_t l4 = l0 + inci, l5 = l1 + inci, l6 = l2 + inci, l7 = l3 + inci;
    face_i(x, y, z, l0, l1, l2, l3, t); ti[0] = t[0];
    face_j(x, y, z, l0, l4, l2, l6, t); tj[0] = t[1];
    face_k(x, y, z, l0, l4, l1, l5, t); tk[0] = t[2];
    double ax = .25 * ((x[l4] + x[l5] + x[l7] + x[l6]) * ti[0] - (x[l0] + x[l1] + x[l3] + x[l2]) * ti[0]);
    double ay = .25 * ((y[l1] + y[l3] + y[l5] + y[l7]) * tj[0] - (y[l0] + y[l2] + y[l4] + y[l6]) * tj[0]);
    double az = .25 * ((z[l2] + z[l3] + z[l6] + z[l7]) * tk[0] - (z[l0] + z[l1] + z[l4] + z[l5]) * tk[0]);
    vol[0] = OMAX((ax + ay + az) / 3., 1.e-30);
    return;
  }
  const int64_t iv = pi[IJKV], jv = pi[IJKV + 1], kv = pi[IJKV + 2];
  const int64_t ngc = pi[NIJK + 3], ngkc = pi[NIJK + 4];
  if (pi[ITYPZONE] == 3) {   /* 2-d: cp_tijk.for / cp_vol.for "Domaine 2D" branches, k = 1 */
    const int64_t ndm2 = nvi * nvj;
#define VT(i, j) (((i) + ng - 1) + ((j) + ng - 1) * nvi)
    for (int64_t j = 1 - ngc; j <= jv + ngc + 1; j++)
      for (int64_t i = 1 - ngc; i <= iv + ngc + 1; i++) {
        const int64_t lt = VT(i, j), l0 = VX(i, j, 1), l1 = l0 + incj, l2 = l0 + inck, l3 = l1 + inck;
        const int64_t l4 = l0 + inci, l6 = l2 + inci;
        if (j <= jv + ngc) {
          face_i(x, y, z, l0, l1, l2, l3, t);
          ti[lt] = t[0]; ti[lt + ndm2] = t[1];
        }
        if (i <= iv + ngc) {
          face_j(x, y, z, l0, l4, l2, l6, t);
          tj[lt] = t[0]; tj[lt + ndm2] = t[1];
        }
      }
    for (int64_t j = 1 - ngc; j <= jv + ngc; j++)
      for (int64_t i = 1 - ngc; i <= iv + ngc; i++) {
        const int64_t lt = VT(i, j), l0 = VX(i, j, 1), l1 = l0 + incj, l2 = l0 + inck, l3 = l1 + inck;
        const int64_t l4 = l0 + inci, l5 = l1 + inci, l6 = l2 + inci, l7 = l3 + inci;
        const int64_t lip = lt + 1, ljp = lt + nvi;
        double a[2];
        const double* c2[2] = {x, y};
        for (int c = 0; c < 2; c++) {
          const double* q = c2[c];
          const int64_t o = c * ndm2;
          a[c] = .25 * ((q[l4] + q[l5] + q[l7] + q[l6]) * ti[lip + o] - (q[l0] + q[l1] + q[l3] + q[l2]) * ti[lt + o] +
                        (q[l1] + q[l3] + q[l5] + q[l7]) * tj[ljp + o] - (q[l0] + q[l2] + q[l4] + q[l6]) * tj[lt + o]);
        }
        double tkz10 = (x[l4] - x[l0]) * (y[l5] - y[l4]) - (y[l4] - y[l0]) * (x[l5] - x[l4]);
        double tkz11 = (x[l1] - x[l5]) * (y[l0] - y[l1]) - (y[l1] - y[l5]) * (x[l0] - x[l1]);
        double tk1 = .5 * (tkz10 + tkz11);
        double az = .25 * (z[l2] + z[l3] + z[l6] + z[l7] - z[l0] - z[l1] - z[l4] - z[l5]) * tk1;
        vol[lt] = OMAX((a[0] + a[1] + az) / 3., 1.e-30);
      }
#undef VT
    return;
  }
  const int64_t ndm = nvi * nvj * nvk;
  for (int64_t k = 1 - ngkc; k <= kv + ngkc; k++)
    for (int64_t j = 1 - ngc; j <= jv + ngc; j++)
      for (int64_t i = 1 - ngc; i <= iv + ngc; i++) {
        const int64_t lt = VX(i, j, k), l0 = lt, l1 = l0 + incj, l2 = l0 + inck, l3 = l1 + inck;
        const int64_t l4 = l0 + inci, l5 = l1 + inci, l6 = l2 + inci;
        face_i(x, y, z, l0, l1, l2, l3, t);
        for (int c = 0; c < 3; c++) ti[lt + c * ndm] = t[c];
        face_j(x, y, z, l0, l4, l2, l6, t);
        for (int c = 0; c < 3; c++) tj[lt + c * ndm] = t[c];
        face_k(x, y, z, l0, l4, l1, l5, t);
        for (int c = 0; c < 3; c++) tk[lt + c * ndm] = t[c];
      }
  for (int64_t k = 1 - ngkc; k <= kv + ngkc; k++)   /* i = imax + 1 faces */
    for (int64_t j = 1 - ngc; j <= jv + ngc; j++) {
      const int64_t lt = VX(iv + ngc + 1, j, k), l1 = lt + incj, l2 = lt + inck, l3 = l1 + inck;
      face_i(x, y, z, lt, l1, l2, l3, t);
      for (int c = 0; c < 3; c++) ti[lt + c * ndm] = t[c];
    }
  for (int64_t k = 1 - ngkc; k <= kv + ngkc; k++)   /* j = jmax + 1 faces */
    for (int64_t i = 1 - ngc; i <= iv + ngc; i++) {
      const int64_t lt = VX(i, jv + ngc + 1, k), l2 = lt + inck, l4 = lt + inci, l6 = l2 + inci;
      face_j(x, y, z, lt, l4, l2, l6, t);
      for (int c = 0; c < 3; c++) tj[lt + c * ndm] = t[c];
    }
  for (int64_t j = 1 - ngc; j <= jv + ngc; j++)     /* k = kmax + 1 faces */
    for (int64_t i = 1 - ngc; i <= iv + ngc; i++) {
      const int64_t lt = VX(i, j, kv + ngkc + 1), l1 = lt + incj, l4 = lt + inci, l5 = l1 + inci;
      face_k(x, y, z, lt, l4, l1, l5, t);
      for (int c = 0; c < 3; c++) tk[lt + c * ndm] = t[c];
    }
  for (int64_t k = 1 - ngkc; k <= kv + ngkc; k++)
    for (int64_t j = 1 - ngc; j <= jv + ngc; j++)
      for (int64_t i = 1 - ngc; i <= iv + ngc; i++) {
        const int64_t lt = VX(i, j, k), l0 = lt, l1 = l0 + incj, l2 = l0 + inck, l3 = l1 + inck;
        const int64_t l4 = l0 + inci, l5 = l1 + inci, l6 = l2 + inci, l7 = l3 + inci;
        const int64_t lip = lt + inci, ljp = lt + incj, lkp = lt + inck;
        const double* c3[3] = {x, y, z};
        double a[3];
        for (int c = 0; c < 3; c++) {
          const double* q = c3[c];
          const int64_t o = c * ndm;
          a[c] = .25 * ((q[l4] + q[l5] + q[l7] + q[l6]) * ti[lip + o] - (q[l0] + q[l1] + q[l3] + q[l2]) * ti[lt + o] +
                        (q[l1] + q[l3] + q[l5] + q[l7]) * tj[ljp + o] - (q[l0] + q[l2] + q[l4] + q[l6]) * tj[lt + o] +
                        (q[l2] + q[l3] + q[l6] + q[l7]) * tk[lkp + o] - (q[l0] + q[l1] + q[l4] + q[l5]) * tk[lt + o]);
        }
        vol[lt] = OMAX((a[0] + a[1] + a[2]) / 3., 1.e-30);
      }
#undef VX
}

static void bc_window(const int64_t* pi, const int64_t* fen, int idir, int64_t* cl) {
  int64_t ng = pi[NIJK + 3], ngk = pi[NIJK + 4];
  int64_t sdm[6] = {1, pi[IJKV], 1, pi[IJKV + 1], 1, pi[IJKV + 2]};
  for (int d = 0; d < 3; d++) {
    cl[2 * d] = OMAX(fen[2 * d], sdm[2 * d]);
    cl[2 * d + 1] = OMIN(fen[2 * d + 1], sdm[2 * d + 1]);
  }
  if (idir == 1) { cl[1] = cl[0] - 1; cl[0] = cl[0] - ng; }
  else if (idir == 2) { cl[1] = cl[0] + ng; cl[0] = cl[0] + 1; }
  else if (idir == 3) { cl[3] = cl[2] - 1; cl[2] = cl[2] - ng; }
  else if (idir == 4) { cl[3] = cl[2] + ng; cl[2] = cl[2] + 1; }
  else if (idir == 5) { cl[5] = cl[4] - 1; cl[4] = cl[4] - ngk; }
  else { cl[5] = cl[4] + ngk; cl[4] = cl[4] + 1; }
}

/* Raw face normal of a BC window at the boundary face of ghost line
 * (i, j, k): tijk(lmtr, ic..kc) * c_mtr (shape_tab_mtr.for), lmtr at the
 * first interior cell (low faces) or the first ghost (high faces). */
static void bc_normal(const int64_t* pi, const double* ti, const double* tj, const double* tk,
                      int idir, int64_t i, int64_t j, int64_t k, double t[3]) {
  int d = (idir - 1) / 2, low = idir % 2;
  int64_t c[3] = {i, j, k};
  c[d] = low ? 1 : pi[IJKV + d] + 1;
  const double* T = d == 0 ? ti : (d == 1 ? tj : tk);
  const int64_t neq_mtr = d < 2 ? pi[NEQ_IJ] : pi[NEQ_K], ndm = pi[NDIMDX_MTR];
  const int64_t lm = indmtr(pi, c[0], c[1], c[2]);
  if (neq_mtr == 3) {
    t[0] = T[lm] * 1.; t[1] = T[lm + ndm] * 1.; t[2] = T[lm + 2 * ndm] * 1.;
  } else if (neq_mtr == 2) {   /* ic = 1, jc = 2, kc = 2, ck_mtr = 0 */
    t[0] = T[lm] * 1.; t[1] = T[lm + ndm] * 1.; t[2] = T[lm + ndm] * 0.;
  } else {
    double ci = d == 0 ? 1. : 0., cj = d == 1 ? 1. : 0., ck = d == 2 ? 1. : 0.;
    t[0] = T[lm] * ci; t[1] = T[lm] * cj; t[2] = T[lm] * ck;
  }
}

/* BC/non_reflection.for: characteristic state between the exterior state
 * (roe, rue, rve, rwe, ete) and interior cell l1; t = normal * snorm. */
typedef struct { double r, u, v, w, qn, sn, svar[5], qvar5; } nr_out;
static void non_reflection(const double* pr, const double t[3], const double* rop, int64_t nd,
                           int64_t l1, const double ext[5], nr_out* o) {
  const double gam = pr[GAMMA], gam1 = pr[GAMMA] - 1., gam1_1 = 1. / gam1;
  const double tcx = t[0], tcy = t[1], tcz = t[2];
  const double sn = sqrt(tcx * tcx + tcy * tcy + tcz * tcz);
  const double roi = rop[l1], rui = rop[l1 + nd] * roi, rvi = rop[l1 + 2 * nd] * roi,
               rwi = rop[l1 + 3 * nd] * roi;
  const double eti = rop[l1 + 4 * nd] * pr[CVINF] * roi + .5 * (rui * rui + rvi * rvi + rwi * rwi) / roi;
  const double qen = 0.;  /* (vent . n) * c_ale: no mesh motion */
  const double qref1 = .5 * (ext[0] + roi), qref2 = .5 * (ext[1] + rui), qref3 = .5 * (ext[2] + rvi),
               qref4 = .5 * (ext[3] + rwi), qref5 = .5 * (ext[4] + eti);
  const double r = qref1, ri = 1. / r;
  const double u = qref2 * ri, v = qref3 * ri, w = qref4 * ri;
  const double p = gam1 * (qref5 - .5 * r * (u * u + v * v + w * w));
  const double c = sqrt(gam * p * ri), ci = 1. / c, s_1 = 1. / sn;
  const double qn = tcx * u + tcy * v + tcz * w - qen;
  double tnx, tny;
  if (sn == 0.) { tnx = 1.; tny = 0.; } else { tnx = tcx / sn; tny = tcy / sn; }
  const double eig[5] = {qn, qn, qn, qn + sn * c, qn - sn * c};
  double rv[2][5];
  const double qv[2][5] = {{ext[0], ext[1], ext[2], ext[3], ext[4]}, {roi, rui, rvi, rwi, eti}};
  for (int side = 0; side < 2; side++) {
    const double* q = qv[side];
    double sv1 = q[0], sv2 = (q[1] - u * q[0]) * ri, sv3 = (q[2] - v * q[0]) * ri,
           sv4 = (q[3] - w * q[0]) * ri;
    double sv5 = gam1 * (.5 * (u * u + v * v + w * w) * q[0] - u * q[1] - v * q[2] - w * q[3] + q[4]);
    rv[side][0] = sv1 - ci * ci * sv5;
    rv[side][1] = tcz * s_1 * (tnx * sv2 + tny * sv3) - sv4;
    rv[side][2] = -tny * sv2 + tnx * sv3;
    rv[side][3] = .5 * s_1 * (tcx * sv2 + tcy * sv3 + tcz * sv4) + .5 * ri * ci * sv5;
    rv[side][4] = -.5 * s_1 * (tcx * sv2 + tcy * sv3 + tcz * sv4) + .5 * ri * ci * sv5;
  }
  double rvar[5];
  for (int m = 0; m < 5; m++) rvar[m] = eig[m] < 0. ? rv[0][m] : rv[1][m];
  o->svar[0] = rvar[0] + r * ci * (rvar[3] + rvar[4]);
  o->svar[1] = tcz * s_1 * tnx * rvar[1] - tny * rvar[2] + tcx * s_1 * (rvar[3] - rvar[4]);
  o->svar[2] = tcz * s_1 * tny * rvar[1] + tnx * rvar[2] + tcy * s_1 * (rvar[3] - rvar[4]);
  o->svar[3] = -rvar[1] + tcz * s_1 * (rvar[3] - rvar[4]);
  o->svar[4] = r * c * (rvar[3] + rvar[4]);
  o->qvar5 = .5 * (u * u + v * v + w * w) * o->svar[0] + r * (u * o->svar[1] + v * o->svar[2] + w * o->svar[3]) +
             gam1_1 * o->svar[4];
  o->r = r; o->u = u; o->v = v; o->w = w; o->qn = qn; o->sn = sn;
}

/* BCzone.cpp DEFAULT_STATE with nbdata = 0: the free stream. */
static void bc_default_state(const double* pr, double st[5]) {
  st[0] = pr[ROINF];
  st[1] = pr[VXINF] * pr[ROINF];
  st[2] = pr[VYINF] * pr[ROINF];
  st[3] = pr[VZINF] * pr[ROINF];
  st[4] = pr[PINF] / (pr[GAMMA] - 1.) + 0.5 * (pr[VXINF] * st[1] + pr[VYINF] * st[2] + pr[VZINF] * st[3]);
}

/* BCzone.cpp:255-865 for the types of the path, with the ghost windows of
 * indice_cl_sdm.for (npass = 0).  Ghost cells of the first rank (next to
 * the face) are filled before the next ranks of the same line, which the
 * farfield / inflow / outflow next ranks read. */
void or_bc_zone(const int64_t* pi, const double* pr, const double* ti, const double* tj,
                const double* tk, int lrhs, double* rop) {
  int64_t pt_bcs = pi[PT_BC];
  if (pt_bcs <= 0) goto coins;
  {
    int64_t nb_bc = pi[pt_bcs];
    int64_t nd = pi[NDIMDX], neq = pi[NEQ];
    double c1 = lrhs == 1 ? 0. : 1.;
    const double cvinv = 1. / pr[CVINF];
    const double c4 = 5. / 6., c5 = 2. / 6., c6 = -1. / 6.;
    const double k0 = 1. / c6, k1 = -(c4 + c5) * k0, k2 = -c6 * k0, k3 = (2. - c5 - c4) * k0;
    const int sa = neq == 6;
    const double nue = pr[RONUTILDEINF] / pr[ROINF];   /* BCFarfield_init.for: state(6)/state(1) */
    for (int64_t n = 0; n < nb_bc; n++) {
      int64_t pt = pi[pt_bcs + 1 + n];
      int64_t type = pi[pt + BC_TYPE];
      int idir = (int)pi[pt + BC_IDIR];
      int64_t cl[6];
      bc_window(pi, pi + pt + BC_FEN, idir, cl);
      int d = (idir - 1) / 2;
      int low = (idir % 2) == 1;
      int64_t n_d = pi[IJKV + d];
      if (type == 11 || type == 0) {
        for (int64_t k = cl[4]; k <= cl[5]; k++)
          for (int64_t j = cl[2]; j <= cl[3]; j++)
            for (int64_t i = cl[0]; i <= cl[1]; i++) {
              int64_t idx[3] = {i, j, k};
              int64_t l = inddm(pi, i, j, k);
              int64_t src[3] = {i, j, k};
              if (type == 11) { src[d] = low ? idx[d] + n_d : idx[d] - n_d; }
              else { src[d] = low ? cl[2 * d + 1] + 1 : cl[2 * d] - 1; }
              int64_t l1 = inddm(pi, src[0], src[1], src[2]);
              for (int64_t v = 0; v < neq; v++) {
                if (type == 11) rop[l + v * nd] = rop[l1 + v * nd] * c1;
                else rop[l + v * nd] = OMAX(-1.e30, rop[l1 + v * nd]) * c1;
              }
            }
        continue;
      }
      /* the other types: ghost lines normal to the face */
      int64_t first = low ? cl[2 * d + 1] : cl[2 * d];       /* rank next to the face */
      int64_t step = low ? -1 : 1;                            /* towards the next ranks */
      int64_t ir = low ? first + 1 : first - 1;               /* first interior cell */
      int64_t iref = low ? 2 * first + 1 : 2 * first - 1;     /* mirror: iref - i */
      int64_t a0 = d == 0 ? 1 : 0, a1 = d == 2 ? 1 : 2;      /* tangential directions */
      int64_t ta = a0, tb = a1;
      if (d == 1) { ta = 0; tb = 2; }
      double snorm = low ? -1. : 1.;
      double st[5];
      bc_default_state(pr, st);
      double nue_bc = nue;
      /* BC data (BCzone.cpp:324-325 and DEFAULT_STATE): nbdata arrays in
       * param_real at param_int[pt_bcs + 1 + nb_bc + n], cumulative sizes at
       * param_int[pt + BC_NBDATA + 1 ...] */
      int64_t nbdata = pi[pt + BC_NBDATA];
      const double* bdata = nbdata > 0 ? pr + pi[pt_bcs + 1 + nb_bc + n] : 0;
      if (nbdata > 0 && (type == 1 || type == 13 || type == 10)) {
        if (nbdata == 21) {
          for (int m = 0; m < 5; m++) st[m] = bdata[3 + m];
          nue_bc = bdata[16] / st[0];
        } else {
          for (int m = 0; m < 5; m++) st[m] = bdata[m];
          if (sa) nue_bc = bdata[5] / st[0];
        }
      }
      const double* pext = 0;  /* BCOutpres: per-face pressure (bvbs_outpres.for) */
      if (type == 16) pext = pi[pt + BC_NBDATA + 1] == 1 ? bdata + 1 : bdata;
      const int64_t* fen = pi + pt + BC_FEN;
      for (int64_t b = cl[2 * tb]; b <= cl[2 * tb + 1]; b++)
        for (int64_t a = cl[2 * ta]; a <= cl[2 * ta + 1]; a++) {
          int64_t c[3];
          c[ta] = a; c[tb] = b;
          double t[3];
          c[d] = first;
          bc_normal(pi, ti, tj, tk, idir, c[0], c[1], c[2], t);
          for (int64_t rank = 0; rank < (d == 2 ? pi[NIJK + 4] : pi[NIJK + 3]); rank++) {
            c[d] = first + step * rank;
            int64_t l = inddm(pi, c[0], c[1], c[2]);
            int64_t cm[3] = {c[0], c[1], c[2]};
            cm[d] = iref - c[d];
            int64_t ldjr = inddm(pi, cm[0], cm[1], cm[2]);
            int64_t ci1[3] = {c[0], c[1], c[2]};
            ci1[d] = ir;
            int64_t l1 = inddm(pi, ci1[0], ci1[1], ci1[2]);
            int slip = type == 3 || type == 5 || (type == 4 && pi[IFLOW] == 1);
            int noslip = (type == 6 || type == 4) && pi[IFLOW] > 1;
            if (slip) {             /* BCWallInviscid.for */
              double tcx = t[0], tcy = t[1], tcz = t[2];
              double surf = sqrt(tcx * tcx + tcy * tcy + tcz * tcz);
              surf = OMAX(surf, 1e-30);
              double s_1 = 1. / surf;
              tcx = tcx * s_1; tcy = tcy * s_1; tcz = tcz * s_1;
              double u = rop[ldjr + nd] - 0., v = rop[ldjr + 2 * nd] - 0., w = rop[ldjr + 3 * nd] - 0.;
              double qn = u * tcx + v * tcy + w * tcz;
              double ut = u - qn * tcx, vt = v - qn * tcy, wt = w - qn * tcz;
              double ua = 2. * ut - u, va = 2. * vt - v, wa = 2. * wt - w;
              rop[l] = rop[ldjr];
              rop[l + nd] = 0. + ua; rop[l + 2 * nd] = 0. + va; rop[l + 3 * nd] = 0. + wa;
              rop[l + 4 * nd] = rop[ldjr + 4 * nd];
              if (sa) rop[l + 5 * nd] = rop[ldjr + 5 * nd];   /* BCWallInviscidSA_*.for */
            } else if (noslip) {    /* BCWallViscous.for (adiabatic) */
              double u = rop[ldjr + nd], v = rop[ldjr + 2 * nd], w = rop[ldjr + 3 * nd];
              rop[l] = rop[ldjr];
              rop[l + nd] = 0. - u; rop[l + 2 * nd] = 0. - v; rop[l + 3 * nd] = 0. - w;
              rop[l + 4 * nd] = rop[ldjr + 4 * nd];
              if (sa) rop[l + 5 * nd] = -rop[ldjr + 5 * nd];  /* BCWallViscous_SA.for */
            } else if (rank == 0 && (type == 1 || type == 13)) {   /* BCFarfield.for / BCInflow_i.for */
              double tn[3] = {t[0] * snorm, t[1] * snorm, t[2] * snorm};
              nr_out o;
              non_reflection(pr, tn, rop, nd, l1, st, &o);
              double roinv = 1. / o.svar[0];
              double u = o.u + o.r * o.svar[1] * roinv, v = o.v + o.r * o.svar[2] * roinv,
                     w = o.w + o.r * o.svar[3] * roinv;
              rop[l] = o.svar[0];
              rop[l + nd] = u; rop[l + 2 * nd] = v; rop[l + 3 * nd] = w;
              rop[l + 4 * nd] = (o.qvar5 * roinv - .5 * (u * u + v * v + w * w)) * cvinv;
              /* BCFarfield_firstrank_SA.for (eigv1 = qn) / BCInflow_firstrank_SA.for */
              if (sa) rop[l + 5 * nd] = (type == 13 || o.qn < 0.) ? nue_bc : rop[l1 + 5 * nd];
            } else if (rank == 0 && type == 16) {   /* BCOutpres_i.for + linearization_state.for */
              const double rgp = pr[CVINF] * (pr[GAMMA] - 1.), gam = pr[GAMMA];
              int64_t li = (a - fen[2 * ta]) + (b - fen[2 * tb]) * (fen[2 * ta + 1] - fen[2 * ta] + 1);
              double tcx = t[0] * snorm, tcy = t[1] * snorm, tcz = t[2] * snorm;
              double sn = sqrt(tcx * tcx + tcy * tcy + tcz * tcz);
              double s_1 = 1. / sn, tnx, tny, tnz;
              if (sn == 0.) { tnx = 1.; tny = 0.; tnz = 0.; }
              else { tnx = tcx * s_1; tny = tcy * s_1; tnz = tcz * s_1; }
              double roi = rop[l1], ui = rop[l1 + nd], vi = rop[l1 + 2 * nd], wi = rop[l1 + 3 * nd],
                     Ti = rop[l1 + 4 * nd];
              double pin = roi * rgp * Ti;
              double ro0 = rop[l1], T0 = rop[l1 + 4 * nd];
              double p0 = ro0 * rgp * T0;
              double roc0 = sqrt(ro0 * gam * p0);
              double dqn = (pext[li] - pin) / roc0;
              double rog = roi + ro0 * ro0 * dqn / roc0;   /* ro0**2. */
              rop[l] = rog;
              rop[l + nd] = ui - dqn * tnx;
              rop[l + 2 * nd] = vi - dqn * tny;
              rop[l + 3 * nd] = wi - dqn * tnz;
              rop[l + 4 * nd] = pext[li] / (rog * rgp);
              if (sa) rop[l + 5 * nd] = rop[l1 + 5 * nd];   /* BCOutpresSA_i.for */
            } else if (rank == 0 && type == 10) {                  /* BCOutflow.for */
              double roe = rop[l1], rue = rop[l1 + nd] * roe, rve = rop[l1 + 2 * nd] * roe,
                     rwe = rop[l1 + 3 * nd] * roe;
              double roe_inv = 1. / st[0];
              double ete = st[4] - 0.5 * (st[1] * st[1] + st[2] * st[2] + st[3] * st[3]) * roe_inv +
                           0.5 * (rue * rop[l1 + nd] + rve * rop[l1 + 2 * nd] + rwe * rop[l1 + 3 * nd]);
              double ext[5] = {roe, rue, rve, rwe, ete};
              double tn[3] = {t[0] * snorm, t[1] * snorm, t[2] * snorm};
              nr_out o;
              non_reflection(pr, tn, rop, nd, l1, ext, &o);
              rop[l] = rop[l1];
              double roinv = 1. / rop[l];
              if (o.qn < 0.) {
                for (int m = 0; m < 3; m++)
                  rop[l + (m + 1) * nd] = rop[l1 + (m + 1) * nd] - o.qn / (o.sn * o.sn) * tn[m];
              } else {
                for (int m = 0; m < 3; m++) rop[l + (m + 1) * nd] = rop[l1 + (m + 1) * nd];
              }
              rop[l + 4 * nd] = (o.qvar5 * roinv - .5 * (rop[l + nd] * rop[l + nd] + rop[l + 2 * nd] * rop[l + 2 * nd] +
                                                         rop[l + 3 * nd] * rop[l + 3 * nd])) * cvinv;
              if (sa) rop[l + 5 * nd] = rop[l1 + 5 * nd];   /* BCOutflow_firstrank_SA.for */
            } else if (type == 1 || type == 13) {  /* BC_nextrank.for */
              int64_t inc = d == 0 ? 1 : (d == 1 ? pi[NIJK] : pi[NIJK] * pi[NIJK + 1]);
              int64_t dl = -step * inc;            /* towards the interior */
              int64_t q0 = l + dl, q1 = l + 2 * dl, q2 = l + 3 * dl;
              rop[l] = rop[q0] * k3 + rop[q1] * k1 + rop[q2] * k2;
              /* BC_nextrankSA.for tests ro <= 0.3 ro0 instead */
              int keep = sa ? rop[l] <= 0.3 * rop[q0] : fabs(rop[l] / rop[q0] - 1.) >= 0.7;
              if (keep) {
                for (int v = 0; v < neq; v++) rop[l + v * nd] = rop[q0 + v * nd];
              } else {
                for (int v = 1; v < neq; v++)
                  rop[l + v * nd] = rop[q0 + v * nd] * k3 + rop[q1 + v * nd] * k1 + rop[q2 + v * nd] * k2;
              }
            } else if (type == 10 || type == 16) {  /* BC_extrap.for: copy of the first ghost */
              int64_t cf[3] = {c[0], c[1], c[2]};
              cf[d] = first;
              int64_t q0 = inddm(pi, cf[0], cf[1], cf[2]);
              for (int v = 0; v < neq; v++) rop[l + v * nd] = rop[q0 + v * nd];   /* BC_extrap(SA) */
            }
          }
        }
    }
  }
coins:
  if (lrhs == 0) {
    int64_t ind[6] = {1, pi[IJKV], 1, pi[IJKV + 1], 1, pi[IJKV + 2]};
    or_correct_coins(pi, ind, rop);
  }
}

/* correct_coins.for: edges = mean of the two adjacent face ghosts, corners
 * = mean of the three. */
void or_correct_coins(const int64_t* pi, const int64_t* ind_loop, double* rop) {
  int64_t ng = pi[NIJK + 3], ngk = pi[NIJK + 4], nd = pi[NDIMDX], neq = pi[NEQ];
  int64_t il[6];
  il[0] = OMAX(1, ind_loop[0]); il[2] = OMAX(1, ind_loop[2]); il[4] = OMAX(1, ind_loop[4]);
  il[1] = OMIN(pi[IJKV], ind_loop[1]); il[3] = OMIN(pi[IJKV + 1], ind_loop[3]); il[5] = OMIN(pi[IJKV + 2], ind_loop[5]);
  int64_t itest[4] = {1, pi[IJKV], 1, pi[IJKV + 1]};
  /* faces I: edges along j and k */
  for (int idir = 1; idir <= 2; idir++) {
    int64_t is = idir == 1 ? -1 : 1;
    int64_t i0 = il[idir - 1];
    if (i0 != itest[idir - 1]) continue;
    if (il[2] == 1)
      for (int64_t ne = 0; ne < neq; ne++) for (int64_t k = il[4]; k <= il[5]; k++)
        for (int64_t j = 1; j <= ng; j++) for (int64_t i = 1; i <= ng; i++) {
          int64_t i1 = OMIN(ng, i + 1), j1 = OMIN(ng, j + 1);
          int64_t l1 = inddm(pi, i0 + i * is, il[2] - j, k);
          int64_t l11 = inddm(pi, i0 + i1 * is, il[2], k), l12 = inddm(pi, i0, il[2] - j1, k);
          rop[l1 + ne * nd] = (rop[l11 + ne * nd] + rop[l12 + ne * nd]) * 0.5;
        }
    if (il[3] == pi[IJKV + 1])
      for (int64_t ne = 0; ne < neq; ne++) for (int64_t k = il[4]; k <= il[5]; k++)
        for (int64_t j = 1; j <= ng; j++) for (int64_t i = 1; i <= ng; i++) {
          int64_t i1 = OMIN(ng, i + 1), j1 = OMIN(ng, j + 1);
          int64_t l1 = inddm(pi, i0 + i * is, il[3] + j, k);
          int64_t l11 = inddm(pi, i0 + i1 * is, il[3], k), l12 = inddm(pi, i0, il[3] + j1, k);
          rop[l1 + ne * nd] = (rop[l11 + ne * nd] + rop[l12 + ne * nd]) * 0.5;
        }
    if (il[4] == 1)
      for (int64_t ne = 0; ne < neq; ne++) for (int64_t k = 1; k <= ngk; k++)
        for (int64_t j = il[2]; j <= il[3]; j++) for (int64_t i = 1; i <= ng; i++) {
          int64_t k1 = OMIN(ngk, k + 1), i1 = OMIN(ng, i + 1);
          int64_t l1 = inddm(pi, i0 + i * is, j, il[4] - k);
          int64_t l11 = inddm(pi, i0, j, il[4] - k1), l12 = inddm(pi, i0 + i1 * is, j, il[4]);
          rop[l1 + ne * nd] = (rop[l11 + ne * nd] + rop[l12 + ne * nd]) * 0.5;
        }
    if (il[5] == pi[IJKV + 2])
      for (int64_t ne = 0; ne < neq; ne++) for (int64_t k = 1; k <= ngk; k++)
        for (int64_t j = il[2]; j <= il[3]; j++) for (int64_t i = 1; i <= ng; i++) {
          int64_t k1 = OMIN(ngk, k + 1), i1 = OMIN(ng, i + 1);
          int64_t l1 = inddm(pi, i0 + i * is, j, il[5] + k);
          int64_t l11 = inddm(pi, i0, j, il[5] + k1), l12 = inddm(pi, i0 + i1 * is, j, il[5]);
          rop[l1 + ne * nd] = (rop[l11 + ne * nd] + rop[l12 + ne * nd]) * 0.5;
        }
  }
  /* faces J: edges along k */
  for (int idir = 3; idir <= 4; idir++) {
    int64_t is = idir == 3 ? -1 : 1;
    int64_t j0 = il[idir - 1];
    if (j0 != itest[idir - 1]) continue;
    if (il[4] == 1)
      for (int64_t ne = 0; ne < neq; ne++) for (int64_t k = 1; k <= ngk; k++)
        for (int64_t j = 1; j <= ng; j++) for (int64_t i = il[0]; i <= il[1]; i++) {
          int64_t k1 = OMIN(ngk, k + 1), j1 = OMIN(ng, j + 1);
          int64_t l1 = inddm(pi, i, j0 + j * is, il[4] - k);
          int64_t l11 = inddm(pi, i, j0, il[4] - k1), l12 = inddm(pi, i, j0 + j1 * is, il[4]);
          rop[l1 + ne * nd] = (rop[l11 + ne * nd] + rop[l12 + ne * nd]) * 0.5;
        }
    if (il[5] == pi[IJKV + 2])
      for (int64_t ne = 0; ne < neq; ne++) for (int64_t k = 1; k <= ngk; k++)
        for (int64_t j = 1; j <= ng; j++) for (int64_t i = il[0]; i <= il[1]; i++) {
          int64_t k1 = OMIN(ngk, k + 1), j1 = OMIN(ng, j + 1);
          int64_t l1 = inddm(pi, i, j0 + j * is, il[5] + k);
          int64_t l11 = inddm(pi, i, j0, il[5] + k1), l12 = inddm(pi, i, j0 + j1 * is, il[5]);
          rop[l1 + ne * nd] = (rop[l11 + ne * nd] + rop[l12 + ne * nd]) * 0.5;
        }
  }
  /* corners */
  double c3 = 1. / 3.;
  for (int corner = 0; corner < 8; corner++) {
    int hi_i = corner & 1, hi_j = (corner >> 1) & 1, hi_k = (corner >> 2) & 1;
    int64_t i0 = hi_i ? il[1] : il[0], j0 = hi_j ? il[3] : il[2], k0 = hi_k ? il[5] : il[4];
    int64_t ti_ = hi_i ? pi[IJKV] : 1, tj_ = hi_j ? pi[IJKV + 1] : 1, tk_ = hi_k ? pi[IJKV + 2] : 1;
    if (i0 != ti_ || j0 != tj_ || k0 != tk_) continue;
    int64_t si = hi_i ? 1 : -1, sj = hi_j ? 1 : -1, sk = hi_k ? 1 : -1;
    for (int64_t ne = 0; ne < neq; ne++) for (int64_t k = 1; k <= ngk; k++)
      for (int64_t j = 1; j <= ng; j++) for (int64_t i = 1; i <= ng; i++) {
        int64_t i1 = OMIN(ng, i + 1), j1 = OMIN(ng, j + 1), k1 = OMIN(ngk, k + 1);
        int64_t l = inddm(pi, i0 + si * i, j0 + sj * j, k0 + sk * k);
        int64_t l11 = inddm(pi, i0, j0, k0 + sk * k1);
        int64_t l12 = inddm(pi, i0 + si * i1, j0, k0);
        int64_t l13 = inddm(pi, i0, j0 + sj * j1, k0);
        rop[l + ne * nd] = (rop[l11 + ne * nd] + rop[l12 + ne * nd] + rop[l13 + ne * nd]) * c3;
      }
  }
}

/* FastC/FastC/Com/setInterpTransfersFast.cpp:852-883, interpolation type 0
 * (1-to-1 match): receiver ghost cell <- donor cell, every variable. */
void or_transfers(or_zone* zones, const or_transfer* tr, int ntr, int use_p1) {
  for (int t = 0; t < ntr; t++) {
    or_zone* dz = &zones[tr[t].dnr_zone];
    or_zone* rz = &zones[tr[t].rcv_zone];
    const double* src = use_p1 ? dz->ro_p1 : dz->ro;
    double* dst = use_p1 ? rz->ro_p1 : rz->ro;
    int64_t ndd = dz->param_int[NDIMDX], ndr = rz->param_int[NDIMDX];
    int64_t neq = rz->param_int[NEQ];
    if (!tr[t].types) {
      for (int64_t n = 0; n < tr[t].n; n++)
        for (int64_t v = 0; v < neq; v++)
          dst[tr[t].rcv_idx[n] + v * ndr] = src[tr[t].dnr_idx[n] + v * ndd];
      continue;
    }
    /* interpolation molecules: the tensor-product formulas (trilinear /
     * bilinear weights, i fastest; separable Lagrange factors, i then j then
     * k), summed with i fastest */
    const int64_t si = 1, sj = dz->param_int[NIJK], sk = dz->param_int[NIJK] * dz->param_int[NIJK + 1];
    int64_t co = 0;
    for (int64_t n = 0; n < tr[t].n; n++) {
      const int64_t ty = tr[t].types[n], d0 = tr[t].dnr_idx[n], r = tr[t].rcv_idx[n];
      const double* c = tr[t].coefs + co;
      for (int64_t v = 0; v < neq; v++) {
        const double* f = src + v * ndd;
        double val = 0.;
        if (ty == 0 || ty == 1) {
          val = c[0] * f[d0];
        } else if (ty == 2 || ty == 22) {
          const int nk = ty == 2 ? 2 : 1;
          for (int kk = 0; kk < nk; kk++)
            for (int jj = 0; jj < 2; jj++)
              for (int ii = 0; ii < 2; ii++)
                val += c[ii + 2 * jj + 4 * kk] * f[d0 + ii * si + jj * sj + kk * sk];
        } else {
          const int w = ty == 3 ? 3 : 5;
          for (int kk = 0; kk < w; kk++)
            for (int jj = 0; jj < w; jj++)
              for (int ii = 0; ii < w; ii++)
                val += c[ii] * c[w + jj] * c[2 * w + kk] * f[d0 + ii * si + jj * sj + kk * sk];
        }
        dst[r + v * ndr] = val;
      }
      co += ty <= 1 ? 1 : (ty == 2 ? 8 : (ty == 22 ? 4 : (ty == 3 ? 9 : 15)));
    }
  }
}

/* cpcfl3.for (non-ALE branches, called by cptst3.for on the first
 * sub-step of a verified iteration): per interior cell the CFL number
 * dt / min(vis, conv) (Navier-Stokes) or dt / conv (Euler), with the face
 * areas of the cell's faces; cfl = (max, min, sum) in the i-fastest loop
 * order (the driver divides the sum by the cell count, computePT.cpp:643). */
void or_cpcfl3(const int64_t* pi, const double* pr, const double* rop, const double* xmut,
               const double* ti, const double* tj, const double* tk, const double* vol,
               double cfl[3]) {
  const int64_t nd = pi[NDIMDX], ndm = pi[NDIMDX_MTR];
  const double rgp = pr[CVINF] * (pr[GAMMA] - 1.);
  const double gam1 = pr[GAMMA] / pr[PRANDT], gam2 = pr[GAMMA] * rgp;
  const double dt = pr[DTC];
  const int typ = (int)pi[ITYPZONE], visc = pi[IFLOW] >= 2;
  const int64_t inc[3] = {pi[NIJK_MTR], pi[NIJK_MTR + 1], pi[NIJK_MTR + 2]};
  cfl[0] = 0.; cfl[1] = 100000000.; cfl[2] = 0.;
  double surf_c = 0.;
  if (typ == 2) {
    const double ddi = 2. * sqrt(ti[0] * ti[0]), ddj = 2. * sqrt(tj[0] * tj[0]),
                 ddk = 2. * sqrt(tk[0] * tk[0]);
    surf_c = 1. / OMAX(OMAX(ddi, ddj), ddk);
  }
  for (int64_t k = 1; k <= pi[IJKV + 2]; k++)
    for (int64_t j = 1; j <= pi[IJKV + 1]; j++)
      for (int64_t i = 1; i <= pi[IJKV]; i++) {
        const int64_t l = inddm(pi, i, j, k);
        const int64_t lvo = typ == 2 ? 0 : indmtr(pi, i, j, k);
        double surf = surf_c;
        if (typ == 0) {
          const double* T[3] = {ti, tj, tk};
          double dd[3];
          for (int d = 0; d < 3; d++) {
            const double* t = T[d];
            const int64_t a = lvo + inc[d], b = lvo;
            dd[d] = sqrt(t[a] * t[a] + t[a + ndm] * t[a + ndm] + t[a + 2 * ndm] * t[a + 2 * ndm]);
            dd[d] = dd[d] + sqrt(t[b] * t[b] + t[b + ndm] * t[b + ndm] + t[b + 2 * ndm] * t[b + 2 * ndm]);
          }
          surf = 1. / OMAX(OMAX(dd[0], dd[1]), dd[2]);
        } else if (typ == 3) {
          const double* T[2] = {ti, tj};
          double dd[2];
          for (int d = 0; d < 2; d++) {
            const double* t = T[d];
            const int64_t a = lvo + inc[d], b = lvo;
            dd[d] = sqrt(t[a] * t[a] + t[a + ndm] * t[a + ndm]);
            dd[d] = dd[d] + sqrt(t[b] * t[b] + t[b + ndm] * t[b + ndm]);
          }
          surf = 1. / OMAX(dd[0], dd[1]);
        }
        const double u = rop[l + nd], v = rop[l + 2 * nd], w = rop[l + 3 * nd], r = rop[l];
        const double c = sqrt(gam2 * rop[l + 4 * nd]);
        const double ur2 = typ == 3 ? u * u + v * v : u * u + v * v + w * w;
        const double sp = sqrt(ur2);
        const double xinvspc = 1. / (sp + c);
        const double conv = 2. * vol[lvo] * surf * xinvspc;
        double cfloc;
        if (visc) {
          const double xinvkt = gam1 / xmut[l];
          const double vis = 2. * r * vol[lvo] * vol[lvo] * surf * surf * xinvkt;
          cfloc = dt / OMIN(vis, conv);
        } else {
          cfloc = dt / conv;
        }
        cfl[0] = OMAX(cfl[0], cfloc);
        cfl[1] = OMIN(cfl[1], cfloc);
        cfl[2] = cfl[2] + cfloc;
      }
}

/* cpcfl3.for (non-ALE branches): the largest stable dt for the given CFL,
 * i.e. cfl * min over interior cells of comp = min(vis, conv). */
double or_cfl_dt(const int64_t* pi, const double* pr, const double* rop,
                 const double* xmut, const double* ti, const double* tj,
                 const double* tk, const double* vol, double cfl) {
  int64_t nd = pi[NDIMDX];
  double gam = pr[GAMMA], rgp = pr[CVINF] * (gam - 1.);
  double gam1 = gam / pr[PRANDT], gam2 = gam * rgp;
  double best = 1e300;
  for (int64_t k = 1; k <= pi[IJKV + 2]; k++)
    for (int64_t j = 1; j <= pi[IJKV + 1]; j++)
      for (int64_t i = 1; i <= pi[IJKV]; i++) {
        int64_t l = inddm(pi, i, j, k);
        double surf, vv;
        if (pi[ITYPZONE] == 2) {
          double ddi = 2. * sqrt(ti[0] * ti[0]), ddj = 2. * sqrt(tj[0] * tj[0]), ddk = 2. * sqrt(tk[0] * tk[0]);
          surf = 1. / OMAX(OMAX(ddi, ddj), ddk);
          vv = vol[0];
        } else {
          int64_t lt = indmtr(pi, i, j, k);
          int64_t ndm = pi[NDIMDX_MTR];
          double dd[3];
          const double* t3[3] = {ti, tj, tk};
          for (int d = 0; d < 3; d++) {
            int64_t lo = lt, hi = lt + pi[NIJK_MTR + d];
            const double* t = t3[d];
            if (pi[ITYPZONE] == 3 && d == 2) { dd[d] = 0.; continue; }
            double a = sqrt(t[hi] * t[hi] + t[hi + ndm] * t[hi + ndm] + (pi[ITYPZONE] == 3 ? 0. : t[hi + 2 * ndm] * t[hi + 2 * ndm]));
            double b = sqrt(t[lo] * t[lo] + t[lo + ndm] * t[lo + ndm] + (pi[ITYPZONE] == 3 ? 0. : t[lo + 2 * ndm] * t[lo + 2 * ndm]));
            dd[d] = a + b;
          }
          surf = 1. / OMAX(OMAX(dd[0], dd[1]), dd[2]);
          vv = vol[lt];
        }
        double u = rop[l + nd], v = rop[l + 2 * nd], w = rop[l + 3 * nd], r = rop[l];
        double c = sqrt(gam2 * rop[l + 4 * nd]);
        double sp = sqrt(u * u + v * v + w * w);
        double conv = 2. * vv * surf / (sp + c);
        double comp = conv;
        if (pi[IFLOW] >= 2) {
          double vis = 2. * r * vv * vv * surf * surf * (gam1 / xmut[l]);
          comp = OMIN(vis, conv);
        }
        if (comp < best) best = comp;
      }
  return cfl * best;
}

/* ======================================================================
 * The solve step -- computePT.cpp:534-680 with gsdr3.cpp:152-173 (choice
 * of the sub-step arrays), souszones_list.cpp:31-97 (verification flags),
 * navier_stokes_struct.for:6 (per-zone sub-step), lhs.cpp (residual + LU),
 * transfert_multiblock.cpp / bcs.cpp (ghost fill), computePT.cpp:675-679
 * (time-level rotation M1 <- N <- P1).
 * ====================================================================== */
int or_compute(or_zone* zones, int nzones, const or_transfer* tr, int ntr,
               int nitrun, int nstep_deb, int nstep_fin, int nit_c,
               int modulo_verif, int* first_it) {
  if (nzones < 1) return 1;
  const int64_t* p0 = zones[0].param_int;
  int64_t nssiter = p0[NSSITER];
  int implicit = p0[ITYPCP] <= 1;
  for (int it = 0; it < nit_c; it++) {
    int64_t nitrun_loc = (int64_t)nitrun * nit_c + it;
    for (int nstep = nstep_deb; nstep <= nstep_fin; nstep++) {
      int lssiter_verif = 0, lexit_lu = 0;
      if (modulo_verif > 0 && nitrun_loc % modulo_verif == 0) {
        lssiter_verif = 1;
        if (nstep == nssiter && implicit) lexit_lu = 1;
      }
      int skip = (lssiter_verif == 0 && nstep == nssiter && p0[ITYPCP] == 1);
      if (skip) continue;
      for (int z = 0; z < nzones; z++) {
        or_zone* Z = &zones[z];
        const int64_t* pi = Z->param_int;
        const double* pr = Z->param_real;
        int64_t ni = pi[IJKV], nj = pi[IJKV + 1], nk = pi[IJKV + 2];
        int64_t ng = pi[NIJK + 3], ngk = pi[NIJK + 4];
        int64_t sdm[6] = {1, ni, 1, nj, 1, nk};
        int64_t coe_r[6] = {1 - ng, ni + ng, 1 - ng, nj + ng, 1 - ngk, nk + ngk};
        int64_t grad_r[6] = {0, ni + 1, 0, nj + 1, 1 - (ngk ? 1 : 0), nk + (ngk ? 1 : 0)};
        double *ssiter, *out;
        if (nstep == 1) { ssiter = Z->ro; out = Z->ro_p1; }
        else if (implicit) { ssiter = Z->ro_p1; out = Z->ro_p1; }
        else if (nstep % 2 == 0) { ssiter = Z->ro_p1; out = Z->ro; }
        else { ssiter = Z->ro; out = Z->ro_p1; }
        if (nstep == 1) {
          if (pi[IFLOW] == 2) or_invist(pi, pr, implicit ? coe_r : grad_r, ssiter, Z->xmut);
          /* navier_stokes_struct.for:258-266: SA viscosity on ind_coe */
          if (pi[IFLOW] == 3) or_vispalart(pi, pr, coe_r, ssiter, Z->xmut);
          if (implicit && pi[DTLOC] == 1) {   /* cptst3.for: local time step */
            or_tstb3_impli(pi, pr, coe_r, ssiter, Z->coe, Z->xmut, Z->ti, Z->tj, Z->tk, Z->vol);
          } else if (implicit) {
            or_tstb3_global(pi, pr, coe_r, Z->coe, Z->vol);
            or_tstb3c(pi, pr, *first_it, coe_r, ssiter, Z->coe, Z->xmut, Z->ti, Z->tj, Z->tk, Z->vol);
          } else if (pi[DTLOC] == 1) {   /* cptst3.for: local time step, explicit */
            or_tstb3_expli(pi, pr, sdm, ssiter, Z->coe, Z->xmut, Z->ti, Z->tj, Z->tk, Z->vol);
          } else {
            or_tstb3_global(pi, pr, sdm, Z->coe, Z->vol);
          }
          /* cptst3.for:115-120: CFL statistics of a verified iteration */
          if (lssiter_verif && Z->cfl) {
            or_cpcfl3(pi, pr, ssiter, Z->xmut, Z->ti, Z->tj, Z->tk, Z->vol, Z->cfl);
            Z->cfl[2] = Z->cfl[2] / (double)(pi[IJKV] * pi[IJKV + 1] * pi[IJKV + 2]);
          }
        }
        or_init_rhs(pi, nstep, sdm, Z->drodm);
        /* src_term.for:86-97: SA source (after the coefficients of the
         * first sub-step, which coe6 reads) */
        if (pi[IFLOW] == 3)
          or_spsource(pi, pr, nstep, sdm, ssiter, Z->coe, Z->ti, Z->tj, Z->tk, Z->vol,
                      Z->xmut + pi[NDIMDX], Z->drodm);
        /* src_term.for:246-255: o3sc / o5sc shock sensor on every sub-step */
        if (pi[SLOPE] == 6 || pi[SLOPE] == 7)
          or_shock_sensor(pi, pr, sdm, ssiter, Z->ti, Z->tj, Z->tk, Z->vol, Z->wig);
        /* src_term.for:257-266: senseur wiggle on the first sub-step */
        if (pi[KFLUDOM] == 2 && nstep == 1) or_wiggle(pi, sdm, ssiter, Z->wig);
        or_flux(pi, pr, sdm, ssiter, Z->drodm, Z->xmut, Z->ti, Z->tj, Z->tk, Z->vol, Z->wig);
        /* navier_stokes_struct.for:378: wall-face correction (Roe) */
        or_correct_flux(pi, pr, ssiter, Z->drodm, Z->xmut, Z->ti, Z->tj, Z->tk, Z->vol, Z->wig);
        if (implicit) {
          or_core3as2(pi, pr, nstep, *first_it, sdm, ssiter, Z->ro, Z->ro_m1, Z->drodm, Z->coe);
          if (lssiter_verif) or_cprdu3s1(pi, nstep, (int)nssiter, Z->drodm, Z->rdm);
          if (!lexit_lu) {
            int nt = g_lu_tiles;
            if (nt <= 1) {
              or_invlu(pi, pr, sdm, Z->ro_p1, ssiter, Z->drodm, Z->drodm, Z->ti, Z->tj, Z->tk, Z->coe, 1);
            } else {
              /* k-slab tiles; a tile never reads outside its own range */
#pragma omp parallel for num_threads(g_threads) schedule(static)
              for (int tt = 0; tt < nt; tt++) {
                int64_t k0 = 1 + (nk * tt) / nt, k1 = (nk * (tt + 1)) / nt;
                int64_t tl[6] = {1, ni, 1, nj, k0, k1};
                if (k1 >= k0)
                  or_invlu(pi, pr, tl, Z->ro_p1, ssiter, Z->drodm, Z->drodm, Z->ti, Z->tj, Z->tk, Z->coe, 1);
              }
            }
          }
        } else {
          or_core3ark3(pi, pr, nstep, sdm, out, ssiter, Z->drodm, Z->coe);
        }
      }
      /* ghost fill of the array just written: 1-to-1 transfers, then BCs */
      int use_p1 = implicit || (nstep % 2 == 1);
      if (ntr > 0) or_transfers(zones, tr, ntr, use_p1);
      for (int z = 0; z < nzones; z++) {
        or_zone* Z = &zones[z];
        or_bc_zone(Z->param_int, Z->param_real, Z->ti, Z->tj, Z->tk, 0, use_p1 ? Z->ro_p1 : Z->ro);
      }
    }
    *first_it = 1;
    /* FastS/FastS/PyTree.py:226-228: switchPointers__(zones, case, nitmax%2+2)
     * for an explicit step -- order 2 (an even stage count, RK2, whose last
     * stage wrote ro) leaves the levels in place */
    if (!implicit && nssiter % 2 == 0) continue;
    for (int z = 0; z < nzones; z++) {
      double* save = zones[z].ro_m1;
      zones[z].ro_m1 = zones[z].ro;
      zones[z].ro = zones[z].ro_p1;
      zones[z].ro_p1 = save;
    }
  }
  return 0;
}
