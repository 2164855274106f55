// fgb_flux.cu -- face-flux residual and fused stage updates (sm_103a).
//
// Replaces the per-tile loop nest of FastS/FastS/Compute/template_FluxAndBalance.for
// (generated as ROE/*/fluroe_*.for and AUSM/*/fluausm_*.for) and the update
// routines core3ark3.for / core3as2.for / init_rhs.for.
//
// GPU design.  On GB300 these FP64 kernels are bound by the FP64 pipe, not by
// HBM, so each face flux is computed exactly once:
//   * face_flux<D,...>: one thread per face of direction D writes the 5 flux
//     components to a face array (SoA).  Threads run along i, so every stencil
//     load is coalesced; reconstruction stencils are re-read through L1.
//   * assemble<...>: one thread per interior cell adds its six face fluxes in
//     the reference's accumulation order (+F_k lo, +F_j lo, +F_i lo, -F_i hi,
//     -F_j hi, -F_k hi) and applies, in the same kernel, the RK3 low-storage
//     stage update (explicit) or the BDF Newton residual (implicit).
// The cartesian face kernels are specialised per direction at compile time:
// products with the zero tangential metric components of a cartesian face are
// not issued at all, which is exact (they are exact zeros in the general form).
#include <type_traits>
#include "fgb_kernels.cuh"

namespace fgb {

// ---------------------------------------------------------------- slopes
// Slope/o1_slope_var.for, o3_slope_var.for, o3sc_slope_var.for,
// minmod_slope_var.for.  a = q(l-2*inc), b = q(l-inc), c = q(l),
// d = q(l+inc); qm = right state of the face (cell l side), qp = left state.
// roff: minmod's low-temperature cut-off, or o3sc's shock-sensor weight of
// the face (the o3 states blended with the first-order ones).
// van Albada's smooth averaged slope of the differences x, y (VANALBADA;
// differentiable, for the adjoint): ((y^2 + e) x + (x^2 + e) y) / (x^2 + y^2 + 2e)
__device__ __forceinline__ double vanalbada(double x, double y) {
  const double e2 = 1e-12;
  return ((y * y + e2) * x + (x * x + e2) * y) / (x * x + y * y + 2. * e2);
}

template <int SL>
__device__ __forceinline__ void reconstruct(const Zone& z, double a, double b, double c, double d,
                                            double roff, double& qm, double& qp) {
  if (SL == VANALBADA) {
    qm = c - mul_pow2<-1>(vanalbada(c - b, d - c));
    qp = b + mul_pow2<-1>(vanalbada(b - a, c - b));
  } else if (SL == O1) {
    qm = c;
    qp = b;
  } else if (SL == O3 || SL == O3SC) {
    qm = z.c4 * c + z.c5 * b + z.c6 * d;
    qp = z.c4 * b + z.c6 * a + z.c5 * c;
    if (SL == O3SC) {
      qm = c * (1. - roff) + qm * roff;
      qp = b * (1. - roff) + qp * roff;
    }
  } else {  // minmod with the low-temperature cut-off roff
    double delm = c - b, delp = d - c, delq = b - a;
    double sm = fsignF(1., delm);
    double slp = roff * (sm * fmaxF(0., fminF(fabs(delm), sm * delp)));
    double sq = fsignF(1., delq);
    double slq = roff * (sq * fmaxF(0., fminF(fabs(delq), sq * delm)));
    qm = c - slp;
    qp = b + slq;
  }
}

// ------------------------------------------------------------- Roe (cart)
// Roe average + Harten-fixed dissipation for a cartesian face of direction D
// (Vit_ent/fludiffer_3dcart_{i,j,k}.for, etat_roe_GD.for).
template <int D>
__device__ __forceinline__ void roe_cart(const Zone& z, const double qm[5], const double qp[5],
                                         double F[5]) {
  const double tc = D == 0 ? z.tcx : (D == 1 ? z.tcy : z.tcz);
  const double s = D == 0 ? z.si : (D == 1 ? z.sj : z.sk);
  const double rgp = z.rgp, gam1 = z.gam1;
  double r1 = qp[0];
  double p1 = r1 * qp[4] * rgp;
  double h1 = gam1 * qp[4] * rgp + mul_pow2<-1>(qp[1] * qp[1] + qp[2] * qp[2] + qp[3] * qp[3]);
  double r2 = qm[0];
  double p2 = r2 * qm[4] * rgp;
  double h2 = gam1 * qm[4] * rgp + mul_pow2<-1>(qm[1] * qm[1] + qm[2] * qm[2] + qm[3] * qm[3]);
  double s1 = sqrt(r1), s2 = sqrt(r2);
  double r = s1 * s2;
  double r_1 = 1. / (s1 + s2);
  double vel[3], dvel[3];
#pragma unroll
  for (int m = 0; m < 3; m++) vel[m] = (s1 * qp[m + 1] + s2 * qm[m + 1]) * r_1;
  double h = (s1 * h1 + s2 * h2) * r_1;
  double q = mul_pow2<-1>(vel[0] * vel[0] + vel[1] * vel[1] + vel[2] * vel[2]);
  double c = sqrt((z.gam - 1.) * fabs(h - q));
  double qn1 = qp[D + 1] * tc, qn2 = qm[D + 1] * tc;
#pragma unroll
  for (int m = 0; m < 3; m++) dvel[m] = (qm[m + 1] - qp[m + 1]) * s;
  double dp = p2 - p1, dqn = qn2 - qn1;
  double s_1 = 1. / fmaxF(s, 1.e-30);
  double nn = tc * s_1;
  double qn = vel[D] * nn;
  double f1 = qn;
  double f4 = z.psiroe * (fabs(f1) + c);
  double f2 = .5 + fsignF(.5, fabs(f1) - f4);
  double f3 = mul_pow2<-1>((f2 - 1.) * (f1 * f1 / f4 + f4)) - f2 * fabs(f1);
  f1 = (r2 - r1 - dp / (c * c)) * s;
  double fl[5];
  fl[0] = f3 * (f1);
#pragma unroll
  for (int m = 0; m < 3; m++)
    fl[m + 1] = (m == D) ? f3 * (f1 * vel[m] + r * (dvel[m] - nn * dqn))
                         : f3 * (f1 * vel[m] + r * (dvel[m]));
  fl[4] = f3 * (f1 * q + r * (vel[0] * dvel[0] + vel[1] * dvel[1] + vel[2] * dvel[2] - qn * dqn));
  // lambda4 = qn + c
  f1 = qn + c;
  f2 = .5 + fsignF(.5, fabs(f1) - f4);
  f3 = mul_pow2<-1>((f2 - 1.) * (f1 * f1 / f4 + f4)) - f2 * fabs(f1);
  f1 = (dp + r * c * dqn * s_1) / (mul_pow2<1>(c) * c) * s * f3;
  fl[0] = fl[0] + f1;
#pragma unroll
  for (int m = 0; m < 3; m++) fl[m + 1] = fl[m + 1] + f1 * ((m == D) ? (vel[m] + nn * c) : vel[m]);
  fl[4] = fl[4] + f1 * (h + qn * c);
  // lambda5 = qn - c
  f1 = qn - c;
  f2 = .5 + fsignF(.5, fabs(f1) - f4);
  f3 = mul_pow2<-1>((f2 - 1.) * (f1 * f1 / f4 + f4)) - f2 * fabs(f1);
  f1 = (dp - r * c * dqn * s_1) / (mul_pow2<1>(c) * c) * f3 * s;
  fl[0] = fl[0] + f1;
#pragma unroll
  for (int m = 0; m < 3; m++) fl[m + 1] = fl[m + 1] + f1 * ((m == D) ? (vel[m] - nn * c) : vel[m]);
  fl[4] = fl[4] + f1 * (h - qn * c);
  double rou1 = r1 * qn1, rou2 = r2 * qn2, p1p2 = p1 + p2;
  F[0] = mul_pow2<-1>(fl[0] + rou1 + rou2);
#pragma unroll
  for (int m = 0; m < 3; m++)
    F[m + 1] = (m == D) ? mul_pow2<-1>(fl[m + 1] + rou1 * qp[m + 1] + rou2 * qm[m + 1] + tc * p1p2)
                        : mul_pow2<-1>(fl[m + 1] + rou1 * qp[m + 1] + rou2 * qm[m + 1]);
  F[4] = mul_pow2<-1>(fl[4] + rou1 * h1 + rou2 * h2);
}

// ----------------------------------------------------------- Roe (general)
// Vit_ent/fludiffer_3dfull_i.for with the face normal (tcx,tcy,tcz), |S| = s.
// TAPE: also store, at tp[k * ts] for k = 1..8, the square roots and
// quotients that a reverse pass of this flux needs (s1, s2, 1/(s1+s2), c,
// 1/|S|, and the reciprocals 1/f4, 1/c^2, 1/(s1 s2)); F is unchanged.
template <bool TAPE = false>
__device__ __forceinline__ void roe_full(const Zone& z, const double qm[5], const double qp[5],
                                         double tcx, double tcy, double tcz, double s, double F[5],
                                         double* tp = nullptr, int64_t ts = 0) {
  const double rgp = z.rgp, gam1 = z.gam1;
  double r1 = qp[0], p1 = r1 * qp[4] * rgp;
  double h1 = gam1 * qp[4] * rgp + mul_pow2<-1>(qp[1] * qp[1] + qp[2] * qp[2] + qp[3] * qp[3]);
  double r2 = qm[0], p2 = r2 * qm[4] * rgp;
  double h2 = gam1 * qm[4] * rgp + mul_pow2<-1>(qm[1] * qm[1] + qm[2] * qm[2] + qm[3] * qm[3]);
  double s1 = sqrt(r1), s2 = sqrt(r2);
  double r = s1 * s2, r_1 = 1. / (s1 + s2);
  double u = (s1 * qp[1] + s2 * qm[1]) * r_1;
  double v = (s1 * qp[2] + s2 * qm[2]) * r_1;
  double w = (s1 * qp[3] + s2 * qm[3]) * r_1;
  double h = (s1 * h1 + s2 * h2) * r_1;
  double q = mul_pow2<-1>(u * u + v * v + w * w);
  double c = sqrt((z.gam - 1.) * fabs(h - q));
  double qn1 = qp[1] * tcx + qp[2] * tcy + qp[3] * tcz;
  double qn2 = qm[1] * tcx + qm[2] * tcy + qm[3] * tcz;
  double du = (qm[1] - qp[1]) * s, dv = (qm[2] - qp[2]) * s, dw = (qm[3] - qp[3]) * s;
  double dp = p2 - p1, dqn = qn2 - qn1;
  double s_1 = 1.0 / fmaxF(s, 1.E-30);
  double nx = tcx * s_1, ny = tcy * s_1, nz = tcz * s_1;
  double qn = u * nx + v * ny + w * nz;
  double f1 = qn;
  double f4 = z.psiroe * (fabs(f1) + c);
  if (TAPE) {
    tp[ts] = s1; tp[2 * ts] = s2; tp[3 * ts] = r_1; tp[4 * ts] = c; tp[5 * ts] = s_1;
    tp[6 * ts] = 1. / f4; tp[7 * ts] = 1. / (c * c); tp[8 * ts] = 1. / r;
  }
  double f2 = 0.5 + fsignF(0.5, fabs(f1) - f4);
  double f3 = mul_pow2<-1>((f2 - 1.0) * (f1 * f1 / f4 + f4)) - f2 * fabs(f1);
  f1 = (r2 - r1 - dp / (c * c)) * s;
  double fl1 = f3 * (f1);
  double fl2 = f3 * (f1 * u + r * (du - nx * dqn));
  double fl3 = f3 * (f1 * v + r * (dv - ny * dqn));
  double fl4 = f3 * (f1 * w + r * (dw - nz * dqn));
  double fl5 = f3 * (f1 * q + r * (u * du + v * dv + w * dw - qn * dqn));
  f1 = qn + c;
  f2 = 0.5 + fsignF(0.5, fabs(f1) - f4);
  f3 = mul_pow2<-1>((f2 - 1.) * (f1 * f1 / f4 + f4)) - f2 * fabs(f1);
  f1 = (dp + r * c * dqn * s_1) / (mul_pow2<1>(c) * c) * s * f3;
  fl1 = fl1 + f1;
  fl2 = fl2 + f1 * (u + nx * c);
  fl3 = fl3 + f1 * (v + ny * c);
  fl4 = fl4 + f1 * (w + nz * c);
  fl5 = fl5 + f1 * (h + qn * c);
  f1 = qn - c;
  f2 = 0.5 + fsignF(0.5, fabs(f1) - f4);
  f3 = mul_pow2<-1>((f2 - 1.) * (f1 * f1 / f4 + f4)) - f2 * fabs(f1);
  f1 = (dp - r * c * dqn * s_1) / (mul_pow2<1>(c) * c) * f3 * s;
  fl1 = fl1 + f1;
  fl2 = fl2 + f1 * (u - nx * c);
  fl3 = fl3 + f1 * (v - ny * c);
  fl4 = fl4 + f1 * (w - nz * c);
  fl5 = fl5 + f1 * (h - qn * c);
  double rou1 = r1 * qn1, rou2 = r2 * qn2, p1p2 = p1 + p2;
  F[0] = mul_pow2<-1>(fl1 + rou1 + rou2);
  F[1] = mul_pow2<-1>(fl2 + rou1 * qp[1] + rou2 * qm[1] + tcx * p1p2);
  F[2] = mul_pow2<-1>(fl3 + rou1 * qp[2] + rou2 * qm[2] + tcy * p1p2);
  F[3] = mul_pow2<-1>(fl4 + rou1 * qp[3] + rou2 * qm[3] + tcz * p1p2);
  F[4] = mul_pow2<-1>(fl5 + rou1 * h1 + rou2 * h2);
}

// ---------------------------------------------------------- Roe (SA row)
// ROE/3dfull/fluFaceSA_*_3dfull_{i,j,k}.for (3dcart: Vit_ent/qn_3dcart_*):
// the ro nutilde flux from the first-order states of cells nm = l - inc and
// l, upwinded by the Roe-averaged normal velocity with the floor c1 |S|.
template <int D, bool CART, bool TWO_D = false>
__device__ __forceinline__ double roe_sa_flux(const Zone& z, const double* __restrict__ q,
                                              int64_t l, int64_t nm, double tcx, double tcy,
                                              double tcz, double s) {
  const int64_t nd = z.nd;
  const double t[3] = {tcx, tcy, tcz};
  double qp[3] = {q[nm + nd], q[nm + 2 * nd], q[nm + 3 * nd]};
  const double qm[3] = {q[l + nd], q[l + 2 * nd], q[l + 3 * nd]};
  double qn1 = CART ? qp[D] * t[D] : (TWO_D ? qp[0] * tcx + qp[1] * tcy : qp[0] * tcx + qp[1] * tcy + qp[2] * tcz);
  const double qn2 = CART ? qm[D] * t[D] : (TWO_D ? qm[0] * tcx + qm[1] * tcy : qm[0] * tcx + qm[1] * tcy + qm[2] * tcz);
  double qp1 = q[nm], qm1 = q[l];
  const double qm6 = q[l + 5 * nd] * qm1 * qn2;
  const double qp6 = q[nm + 5 * nd] * qp1 * qn1;
  qp1 = sqrt(qp1);
  qm1 = sqrt(qm1);
  const double r_1 = 1. / (qp1 + qm1);
#pragma unroll
  for (int m = 0; m < 3; m++) qp[m] = r_1 * (qp1 * qp[m] + qm1 * qm[m]);
  qn1 = CART ? qp[D] * t[D] : (TWO_D ? qp[0] * tcx + qp[1] * tcy : qp[0] * tcx + qp[1] * tcy + qp[2] * tcz);
  const double s_1 = 1.0 / fmaxF(s, 1.E-30);
  const double tdu = fmaxF(z.c1 / s_1, fabs(qn1));
  return mul_pow2<-1>(qm6 + qp6 - tdu * (q[l + 5 * nd] * q[l] - q[nm + 5 * nd] * q[nm]));
}

// ------------------------------------------------------------- AUSM+(P)
// AUSM/fluFaceEuler.for:36-57 + etat_GD.for + Vit_ent/fluvector_*.for.
// NX = number of non-zero normal components the face can have (1: cartesian
// face of direction D, 3: general).
// NV = 6: Spalart-Allmaras, the ro nutilde flux of AUSM/fluFaceSA.for with
// the same interface velocity and dissipation.
template <int D, bool CART, bool SENS = false, int NV = 5>
__device__ __forceinline__ void ausm_face(const Zone& z, const double qm[NV], const double qp[NV],
                                          double tl, double tcx, double tcy, double tcz,
                                          double s, double F[NV], double wg = 0.) {
  const double rgp = z.rgp, gam1 = z.gam1;
  double r1 = qp[0], rou1 = r1 * qp[1], rov1 = r1 * qp[2], row1 = r1 * qp[3];
  double p1 = r1 * qp[4] * rgp;
  double h1 = gam1 * p1 + mul_pow2<-1>(rou1 * qp[1] + rov1 * qp[2] + row1 * qp[3]);
  double r2 = qm[0], rou2 = r2 * qm[1], rov2 = r2 * qm[2], row2 = r2 * qm[3];
  double p2 = r2 * qm[4] * rgp;
  double h2 = gam1 * p2 + mul_pow2<-1>(rou2 * qm[1] + rov2 * qm[2] + row2 * qm[3]);
  double qn1, qn2;
  if (CART) {
    const double tc = D == 0 ? tcx : (D == 1 ? tcy : tcz);
    qn1 = qp[D + 1] * tc;
    qn2 = qm[D + 1] * tc;
  } else {
    qn1 = qp[1] * tcx + qp[2] * tcy + qp[3] * tcz;
    qn2 = qm[1] * tcx + qm[2] * tcy + qm[3] * tcz;
  }
  double u, tdu;
  if (SENS) {  // SENSOR/fluFaceEuler.for: Rhie-Chow term and dissipation switched by wig
    u = mul_pow2<-2>(qn1 + qn2) - z.c2 * s * (p2 - p1) * (z.opt0 * wg + 1. - z.opt0);
    tdu = fmaxF(fabs(u), z.c1 * s) * wg;
  } else {
    double cc = z.rgpgam * tl;  // c^2 = (rgp gam) T of cell l
    double son = sqrt(qn1 * qn1 / cc);
    double tam = z.c3 * son + s;
    double tam1 = fmaxF(0., tam) * z.c2;
    u = mul_pow2<-2>(qn1 + qn2) - tam1 * (p2 - p1);
    tdu = fmaxF(fabs(u), z.c1 * s) * z.wig_cte;
  }
  double p1p2 = mul_pow2<-1>(p1 + p2);
  F[0] = u * (r1 + r2) - tdu * (r2 - r1);
  F[1] = u * (rou1 + rou2) - tdu * (rou2 - rou1);
  F[2] = u * (rov1 + rov2) - tdu * (rov2 - rov1);
  F[3] = u * (row1 + row2) - tdu * (row2 - row1);
  F[4] = u * (h1 + h2) - tdu * (h2 - h1);
  if (NV == 6) {
    const double qm6 = qm[NV - 1] * qm[0], qp6 = qp[NV - 1] * qp[0];
    F[NV - 1] = u * (qm6 + qp6) - tdu * (qm6 - qp6);
  }
  if (CART) {
    const double tc = D == 0 ? tcx : (D == 1 ? tcy : tcz);
    F[D + 1] = F[D + 1] + tc * p1p2;
  } else {
    F[1] = F[1] + tcx * p1p2;
    F[2] = F[2] + tcy * p1p2;
    F[3] = F[3] + tcz * p1p2;
  }
}

// ------------------------------------------------- viscosity at a face
// mut_interface.for (laminar: xmutvol = (mu_r + mu_l) volinv, xktvol =
// xmutvol gam3) or, with Spalart-Allmaras, mut_prandtltb_interface.for
// (laminar and turbulent conductivities apart) and SA/mut_interface.for
// (xsa: diffusion coefficient of nutilde).
template <int NV>
__device__ __forceinline__ void mut_face(const Zone& z, const double* __restrict__ q,
                                         const double* __restrict__ xmut, int64_t il, int64_t ir,
                                         double volinv, double& xmutvol, double& xktvol,
                                         double& xsa) {
  if (NV == 6) {
    const int64_t nd = z.nd;
    double xmulam = sa_mulam(z, q[il + 4 * nd]);
    xmulam = xmulam + sa_mulam(z, q[ir + 4 * nd]);
    const double xmutot = xmut[ir] + xmut[il];
    const double xmutur = xmutot - xmulam;
    xktvol = (xmulam * z.gam3 + xmutur * z.gam4) * volinv;
    xmutvol = xmutot * volinv;
    const double x = xmulam + q[il + 5 * nd] * q[il] + q[ir + 5 * nd] * q[ir];
    xsa = x * volinv * z.sigma_1;
  } else {
    xmutvol = (xmut[ir] + xmut[il]) * volinv;
    xktvol = xmutvol * z.gam3;
    xsa = 0.;
  }
}

// ------------------------------------------------------ viscous (cart)
// fluvisq_3dcart_{i,j,k}.for + mut_interface.for (SA: fluvisq_SA_3dcart_*,
// nutilde diffusion).  Face D of cell l.
template <int D, int NV = 5>
__device__ __forceinline__ void visc_cart(const Zone& z, const double* __restrict__ q,
                                          const double* __restrict__ xmut, int64_t l, double F[NV]) {
  const int64_t nd = z.nd;
  const double* U = q + nd;
  const double* V = q + 2 * nd;
  const double* W = q + 3 * nd;
  const double* T = q + 4 * nd;
  const int64_t ii = z.inc[0], ij = z.inc[1], ik = z.inc[2];
  const double tcx = z.tcx, tcy = z.tcy, tcz = z.tcz, cvisq = z.cvisq;
  // neighbours of the two cells (il = l - inc_D, ir = l) in the two
  // transverse directions; a = first transverse, b = second transverse
  const int64_t inD = D == 0 ? ii : (D == 1 ? ij : ik);
  const int64_t il = l - inD, ir = l;
  double fv, fv5;
  if (D == 0) {
    const double tix = tcx, tjy = mul_pow2<-2>(tcy), tkz = mul_pow2<-2>(tcz);
    double f1 = U[il], f2 = U[ir], s = f1 + f2;
    double f3 = s + U[l - ii - ij] + U[l - ij];
    double f4 = s + U[l - ii + ij] + U[l + ij];
    double f5 = s + U[l - ii - ik] + U[l - ik];
    double f6 = s + U[l - ii + ik] + U[l + ik];
    double gUx = (f2 - f1) * tix, gUy = (f4 - f3) * tjy, gUz = (f6 - f5) * tkz;
    f1 = V[il]; f2 = V[ir]; s = f1 + f2;
    f3 = s + V[l - ii - ij] + V[l - ij];
    f4 = s + V[l - ii + ij] + V[l + ij];
    double gVx = (f2 - f1) * tix, gVy = (f4 - f3) * tjy;
    f1 = W[il]; f2 = W[ir]; s = f1 + f2;
    f5 = s + W[l - ii - ik] + W[l - ik];
    f6 = s + W[l - ii + ik] + W[l + ik];
    double gWx = (f2 - f1) * tix, gWz = (f6 - f5) * tkz;
    double gTx = (T[ir] - T[il]) * tix;
    double div = (gUx + gVy + gWz) * cvisq;
    double e1 = gUx - div, e2 = gUy + gVx, e3 = gUz + gWx;
    double xmutvol, xktvol, xsa;
    mut_face<NV>(z, q, xmut, il, ir, z.volinv, xmutvol, xktvol, xsa);
    fv = -(mul_pow2<1>(e1) * tcx) * xmutvol;
    fv5 = fv * (U[ir] + U[il]);
    F[1] = F[1] + fv;
    fv = -(e2 * tcx) * xmutvol;
    fv5 = fv5 + fv * (V[ir] + V[il]);
    F[2] = F[2] + fv;
    fv = -(e3 * tcx) * xmutvol;
    fv5 = fv5 + fv * (W[ir] + W[il]);
    F[3] = F[3] + fv;
    fv = mul_pow2<-1>(fv5) - (gTx * tcx) * xktvol;
    F[4] = F[4] + fv;
    if (NV == 6) {
      const double gn = (q[ir + 5 * nd] - q[il + 5 * nd]) * tix;
      F[NV - 1] = F[NV - 1] - xsa * gn * tcx;
    }
  } else if (D == 1) {
    const double tiy = tcy, tjz = mul_pow2<-2>(tcz), tkx = mul_pow2<-2>(tcx);
    double f1 = U[il], f2 = U[ir], s = f1 + f2;
    double f5 = s + U[l - ii - ij] + U[l - ii];
    double f6 = s + U[l + ii - ij] + U[l + ii];
    double gUx = (f6 - f5) * tkx, gUy = (f2 - f1) * tiy;
    f1 = V[il]; f2 = V[ir]; s = f1 + f2;
    double f3 = s + V[l - ij - ik] + V[l - ik];
    double f4 = s + V[l - ij + ik] + V[l + ik];
    f5 = s + V[l - ii - ij] + V[l - ii];
    f6 = s + V[l + ii - ij] + V[l + ii];
    double gVx = (f6 - f5) * tkx, gVy = (f2 - f1) * tiy, gVz = (f4 - f3) * tjz;
    f1 = W[il]; f2 = W[ir]; s = f1 + f2;
    f3 = s + W[l - ij - ik] + W[l - ik];
    f4 = s + W[l - ij + ik] + W[l + ik];
    double gWy = (f2 - f1) * tiy, gWz = (f4 - f3) * tjz;
    double gTy = (T[ir] - T[il]) * tiy;
    double div = (gUx + gVy + gWz) * cvisq;
    double e2 = gUy + gVx, e4 = gVy - div, e5 = gVz + gWy;
    double xmutvol, xktvol, xsa;
    mut_face<NV>(z, q, xmut, il, ir, z.volinv, xmutvol, xktvol, xsa);
    fv = -(e2 * tcy) * xmutvol;
    fv5 = fv * (U[ir] + U[il]);
    F[1] = F[1] + fv;
    fv = -(mul_pow2<1>(e4) * tcy) * xmutvol;
    fv5 = fv5 + fv * (V[ir] + V[il]);
    F[2] = F[2] + fv;
    fv = -(e5 * tcy) * xmutvol;
    fv5 = fv5 + fv * (W[ir] + W[il]);
    F[3] = F[3] + fv;
    fv = mul_pow2<-1>(fv5) - (gTy * tcy) * xktvol;
    F[4] = F[4] + fv;
    if (NV == 6) {
      const double gn = (q[ir + 5 * nd] - q[il + 5 * nd]) * tiy;
      F[NV - 1] = F[NV - 1] - xsa * (gn * tcy);
    }
  } else {
    const double tiz = tcz, tky = mul_pow2<-2>(tcy), tjx = mul_pow2<-2>(tcx);
    double f1 = U[il], f2 = U[ir], s = f1 + f2;
    double f3 = s + U[l - ii - ik] + U[l - ii];
    double f4 = s + U[l + ii - ik] + U[l + ii];
    double gUx = (f4 - f3) * tjx, gUz = (f2 - f1) * tiz;
    f1 = V[il]; f2 = V[ir]; s = f1 + f2;
    double f5 = s + V[l - ij - ik] + V[l - ij];
    double f6 = s + V[l + ij - ik] + V[l + ij];
    double gVy = (f6 - f5) * tky, gVz = (f2 - f1) * tiz;
    f1 = W[il]; f2 = W[ir]; s = f1 + f2;
    f3 = s + W[l - ii - ik] + W[l - ii];
    f4 = s + W[l + ii - ik] + W[l + ii];
    f5 = s + W[l - ij - ik] + W[l - ij];
    f6 = s + W[l + ij - ik] + W[l + ij];
    double gWx = (f4 - f3) * tjx, gWy = (f6 - f5) * tky, gWz = (f2 - f1) * tiz;
    double gTz = (T[ir] - T[il]) * tiz;
    double div = (gUx + gVy + gWz) * cvisq;
    double e3 = gUz + gWx, e5 = gVz + gWy, e6 = gWz - div;
    double xmutvol, xktvol, xsa;
    mut_face<NV>(z, q, xmut, il, ir, z.volinv, xmutvol, xktvol, xsa);
    fv = -e3 * tcz * xmutvol;
    fv5 = fv * (U[ir] + U[il]);
    F[1] = F[1] + fv;
    fv = -e5 * tcz * xmutvol;
    fv5 = fv5 + fv * (V[ir] + V[il]);
    F[2] = F[2] + fv;
    fv = mul_pow2<1, true>(e6) * tcz * xmutvol;
    fv5 = fv5 + fv * (W[ir] + W[il]);
    F[3] = F[3] + fv;
    fv = mul_pow2<-1>(fv5) - gTz * tcz * xktvol;
    F[4] = F[4] + fv;
    if (NV == 6) {
      const double gn = (q[ir + 5 * nd] - q[il + 5 * nd]) * tiz;
      F[NV - 1] = F[NV - 1] - xsa * gn * tcz;
    }
  }
}

// ------------------------------------------------------ viscous (full)
// fluvisq_3dfull_{i,j,k}.for + mut_interface.for on a 3d general zone, face
// D of cell l: Green-Gauss gradient over the cell joining il = l - inc_D and
// ir = l, with the transverse directions A = D+1, B = D+2 (mod 3) -- the
// three reference files are this routine for (D, A, B) = (i,j,k), (j,k,i),
// (k,i,j).
template <int D, int NV = 5>
__device__ __forceinline__ void visc_full(const Zone& z, const double* __restrict__ q,
                                          const double* __restrict__ xmut, int64_t l, int64_t lt,
                                          double tcx, double tcy, double tcz, double F[NV]) {
  constexpr int A = (D + 1) % 3, B = (D + 2) % 3;
  const int64_t nd = z.nd, ndm = z.ndm;
  const double* TD = D == 0 ? z.ti : (D == 1 ? z.tj : z.tk);
  const double* TA = A == 0 ? z.ti : (A == 1 ? z.tj : z.tk);
  const double* TB = B == 0 ? z.ti : (B == 1 ? z.tj : z.tk);
  const int64_t mD = z.minc[D], mA = z.minc[A], mB = z.minc[B];
  const int64_t iA = z.inc[A], iB = z.inc[B];
  const int64_t ltm = lt - mD, ltp = lt + mD, ltA = lt + mA, ltAm = lt + mA - mD, ltB = lt + mB,
                ltBm = lt + mB - mD;
  double t0[3], t1[3], ta0[3], ta1[3], tb0[3], tb1[3];
#pragma unroll
  for (int m = 0; m < 3; m++) {
    const int64_t o = m * ndm;
    t0[m] = mul_pow2<-1>(TD[lt + o] + TD[ltm + o]);
    t1[m] = mul_pow2<-1>(TD[lt + o] + TD[ltp + o]);
    ta0[m] = .125 * (TA[lt + o] + TA[ltm + o]);
    ta1[m] = .125 * (TA[ltA + o] + TA[ltAm + o]);
    tb0[m] = .125 * (TB[lt + o] + TB[ltm + o]);
    tb1[m] = .125 * (TB[ltB + o] + TB[ltBm + o]);
  }
  const int64_t il = l - z.inc[D], ir = l;
  constexpr int NG = NV == 6 ? 5 : 4;   // u, v, w, T (, nutilde: fluvisq_SA_3dfull_*)
  double g[NG][3];
#pragma unroll
  for (int v = 0; v < NG; v++) {
    const double* Q = q + (v + 1) * nd;
    const double f1 = Q[il], f2 = Q[ir];
    const double f3 = Q[ir] + Q[il] + Q[il - iA] + Q[ir - iA];
    const double f4 = Q[ir] + Q[il] + Q[il + iA] + Q[ir + iA];
    const double f5 = Q[ir] + Q[il] + Q[il - iB] + Q[ir - iB];
    const double f6 = Q[ir] + Q[il] + Q[il + iB] + Q[ir + iB];
#pragma unroll
    for (int m = 0; m < 3; m++)
      g[v][m] = (f2 * t1[m] - f1 * t0[m]) + (f4 * ta1[m] - f3 * ta0[m]) + (f6 * tb1[m] - f5 * tb0[m]);
  }
  const double div = (g[0][0] + g[1][1] + g[2][2]) * z.cvisq;
  const double e1 = g[0][0] - div, e2 = g[0][1] + g[1][0], e3 = g[0][2] + g[2][0];
  const double e4 = g[1][1] - div, e5 = g[1][2] + g[2][1], e6 = g[2][2] - div;
  const double volinv = 1. / (z.vol[lt] + z.vol[ltm]);
  double xmutvol, xktvol, xsa;
  mut_face<NV>(z, q, xmut, il, ir, volinv, xmutvol, xktvol, xsa);
  double fv, fv5;
  fv = -(mul_pow2<1>(e1) * tcx + e2 * tcy + e3 * tcz) * xmutvol;
  fv5 = fv * (q[ir + nd] + q[il + nd]);
  F[1] = F[1] + fv;
  fv = -(e2 * tcx + mul_pow2<1>(e4) * tcy + e5 * tcz) * xmutvol;
  fv5 = fv5 + fv * (q[ir + 2 * nd] + q[il + 2 * nd]);
  F[2] = F[2] + fv;
  fv = -(e3 * tcx + e5 * tcy + mul_pow2<1>(e6) * tcz) * xmutvol;
  fv5 = fv5 + fv * (q[ir + 3 * nd] + q[il + 3 * nd]);
  F[3] = F[3] + fv;
  fv = mul_pow2<-1>(fv5) - (g[3][0] * tcx + g[3][1] * tcy + g[3][2] * tcz) * xktvol;
  F[4] = F[4] + fv;
  if (NV == 6)   // SA/assemble_tauij_3dfull.for
    F[NV - 1] = F[NV - 1] - xsa * (g[NG - 1][0] * tcx + g[NG - 1][1] * tcy + g[NG - 1][2] * tcz);
}

// ------------------------------------------------------- viscous (2-d)
// fluvisq_2d_{i,j}.for + mut_interface.for: visc_full without the k faces,
// one transverse direction A, two velocity components (no w row).  NV = 6:
// SA/fluvisq_2d_* (mut_prandtltb_interface.for) + SA/fluvisq_SA_2d_*.
template <int D, int NV = 5>
__device__ __forceinline__ void visc_2d(const Zone& z, const double* __restrict__ q,
                                        const double* __restrict__ xmut, int64_t l, int64_t lt,
                                        double tcx, double tcy, double F[NV]) {
  constexpr int A = 1 - D;
  const int64_t nd = z.nd, ndm = z.ndm;
  const double* TD = D == 0 ? z.ti : z.tj;
  const double* TA = A == 0 ? z.ti : z.tj;
  const int64_t mD = z.minc[D], mA = z.minc[A], iA = z.inc[A];
  const int64_t ltm = lt - mD, ltp = lt + mD, ltA = lt + mA, ltAm = lt + mA - mD;
  double t0[2], t1[2], ta0[2], ta1[2];
#pragma unroll
  for (int m = 0; m < 2; m++) {
    const int64_t o = m * ndm;
    t0[m] = mul_pow2<-1>(TD[lt + o] + TD[ltm + o]);
    t1[m] = mul_pow2<-1>(TD[lt + o] + TD[ltp + o]);
    ta0[m] = .125 * (TA[lt + o] + TA[ltm + o]);
    ta1[m] = .125 * (TA[ltA + o] + TA[ltAm + o]);
  }
  const int64_t il = l - z.inc[D], ir = l;
  double g[3][2];   // u, v, T
#pragma unroll
  for (int v = 0; v < 3; v++) {
    const double* Q = q + (v == 2 ? 4 : v + 1) * nd;
    const double f1 = Q[il], f2 = Q[ir];
    const double f3 = Q[ir] + Q[il] + Q[il - iA] + Q[ir - iA];
    const double f4 = Q[ir] + Q[il] + Q[il + iA] + Q[ir + iA];
#pragma unroll
    for (int m = 0; m < 2; m++) g[v][m] = (f2 * t1[m] - f1 * t0[m]) + (f4 * ta1[m] - f3 * ta0[m]);
  }
  const double div = (g[0][0] + g[1][1]) * z.cvisq;
  const double e1 = g[0][0] - div, e2 = g[0][1] + g[1][0], e4 = g[1][1] - div;
  const double volinv = 1. / (z.vol[lt] + z.vol[ltm]);
  double xmutvol, xktvol, xsa;
  mut_face<NV>(z, q, xmut, il, ir, volinv, xmutvol, xktvol, xsa);
  double fv, fv5;
  fv = -(mul_pow2<1>(e1) * tcx + e2 * tcy) * xmutvol;
  fv5 = fv * (q[ir + nd] + q[il + nd]);
  F[1] = F[1] + fv;
  fv = -(e2 * tcx + mul_pow2<1>(e4) * tcy) * xmutvol;
  fv5 = fv5 + fv * (q[ir + 2 * nd] + q[il + 2 * nd]);
  F[2] = F[2] + fv;
  fv = mul_pow2<-1>(fv5) - (g[2][0] * tcx + g[2][1] * tcy) * xktvol;
  F[4] = F[4] + fv;
  if (NV == 6) {   // diffusion of nutilde
    const double* Q = q + 5 * nd;
    const double f1 = Q[il], f2 = Q[ir];
    const double f3 = Q[ir] + Q[il] + Q[il - iA] + Q[ir - iA];
    const double f4 = Q[ir] + Q[il] + Q[il + iA] + Q[ir + iA];
    const double gx = (f2 * t1[0] - f1 * t0[0]) + (f4 * ta1[0] - f3 * ta0[0]);
    const double gy = (f2 * t1[1] - f1 * t0[1]) + (f4 * ta1[1] - f3 * ta0[1]);
    F[NV - 1] = F[NV - 1] - xsa * (gx * tcx + gy * tcy);
  }
}

// ------------------------------------------------------------- face kernel
// One thread per face of direction D; faces of direction D are indexed
// f = ii + NI*(jj + NJ*kk) over the interior face box (NI = ni+1 for D=0 ...).
// NV = 6: Spalart-Allmaras (AUSM+(P): nutilde takes the o3 slope; Roe:
// first-order nutilde flux, no reconstruction).
template <int D, int TYP, int KF, int SL, bool VISC, int NV = 5>
__device__ __forceinline__ void face_flux_at(const Zone& z, const double* __restrict__ q,
                                             const double* __restrict__ xmut,
                                             double* __restrict__ Fo, const int64_t f) {
  const int64_t NI = z.ni + (D == 0), NJ = z.nj + (D == 1), NK = z.nk + (D == 2);
  const int64_t nf = NI * NJ * NK;
  if (f >= nf) return;
  const int64_t ii = f % NI;
  const int64_t r = f / NI;
  const int64_t jj = r % NJ, kk = r / NJ;
  const int64_t l = inddm(z, ii + 1, jj + 1, kk + 1);
  const int64_t inc = z.inc[D];
  const int64_t nd = z.nd;
  double qm[NV], qp[NV];
  double roff = 0.;
  if (SL == MINMOD) roff = mul_pow2<-1>(fmaxF(0., fminF(q[l + 4 * nd] * z.tmin_1 - .5, 1.)));
  if (SL == O3SC || SL == O5SC) roff = z.wig[l + D * nd + (KF == SENSEUR ? 3 * nd : 0)];
#pragma unroll
  for (int v = 0; v < NV; v++) {
    if (TYP == Z2D && v == 3) { qm[v] = 0.; qp[v] = 0.; continue; }   // 2-d: no w slope
    if (KF == ROE && v == 5) { qm[v] = 0.; qp[v] = 0.; continue; }    // Roe SA: unreconstructed
    const double* Q = q + v * nd;
    double a = (SL == O1) ? 0. : Q[l - 2 * inc];
    double b = Q[l - inc], c = Q[l];
    double d = (SL == O1) ? 0. : Q[l + inc];
    if (SL == O5 || SL == O5SC) {   // Slope/o5_slope_var.for, o5sc_slope_var.for
      const double e = Q[l - 3 * inc], g = Q[l + 2 * inc];
      qm[v] = z.c50 * c + z.c51 * b + z.c52 * d + z.c53 * a + z.c54 * g;
      qp[v] = z.c50 * b + z.c52 * a + z.c51 * c + z.c53 * d + z.c54 * e;
      if (SL == O5SC) {
        qm[v] = c * (1. - roff) + qm[v] * roff;
        qp[v] = b * (1. - roff) + qp[v] * roff;
      }
      continue;
    }
    reconstruct<SL>(z, a, b, c, d, roff, qm[v], qp[v]);
  }
  double F[NV];
  if (TYP == Z2D) {
    // *_2d_{i,j}.for: the 3-d general face with tcz = 0 and w = 0 (the
    // w terms vanish exactly), w flux = 0
    const int64_t lt = indmtr(z, ii + 1, jj + 1, kk + 1);
    const double* t = D == 0 ? z.ti : z.tj;
    double tcx = t[lt], tcy = t[lt + z.ndm];
    double s = sqrt(tcx * tcx + tcy * tcy);
    if (KF == ROE) {
      roe_full(z, qm, qp, tcx, tcy, 0., s, F);
      if (NV == 6) F[NV - 1] = roe_sa_flux<D, false, true>(z, q, l, l - inc, tcx, tcy, 0., s);
    } else {
      ausm_face<D, false, KF == SENSEUR, NV>(z, qm, qp, q[l + 4 * nd], tcx, tcy, 0., s, F,
                                            KF == SENSEUR ? z.wig[l + D * nd] : 0.);
    }
    F[3] = 0.;
    if (VISC) visc_2d<D, NV>(z, q, xmut, l, lt, tcx, tcy, F);
  } else if (TYP == Z3DCART) {
    if (KF == ROE) {
      roe_cart<D>(z, qm, qp, F);
      if (NV == 6)
        F[NV - 1] = roe_sa_flux<D, true>(z, q, l, l - inc, z.tcx, z.tcy, z.tcz,
                                        D == 0 ? z.si : (D == 1 ? z.sj : z.sk));
    }
    else ausm_face<D, true, KF == SENSEUR, NV>(z, qm, qp, q[l + 4 * nd], z.tcx, z.tcy, z.tcz,
                                              D == 0 ? z.si : (D == 1 ? z.sj : z.sk), F,
                                              KF == SENSEUR ? z.wig[l + D * nd] : 0.);
    if (VISC) visc_cart<D, NV>(z, q, xmut, l, F);
  } else {
    const int64_t lt = indmtr(z, ii + 1, jj + 1, kk + 1);
    const double* t = D == 0 ? z.ti : (D == 1 ? z.tj : z.tk);
    double tcx = t[lt], tcy = t[lt + z.ndm], tcz = t[lt + 2 * z.ndm];
    double s = sqrt(tcx * tcx + tcy * tcy + tcz * tcz);
    if (KF == ROE) {
      roe_full(z, qm, qp, tcx, tcy, tcz, s, F);
      if (NV == 6) F[NV - 1] = roe_sa_flux<D, false>(z, q, l, l - inc, tcx, tcy, tcz, s);
    } else ausm_face<D, false, KF == SENSEUR, NV>(z, qm, qp, q[l + 4 * nd], tcx, tcy, tcz, s, F,
                                               KF == SENSEUR ? z.wig[l + D * nd] : 0.);
    if (VISC) visc_full<D, NV>(z, q, xmut, l, lt, tcx, tcy, tcz, F);
  }
#pragma unroll
  for (int v = 0; v < NV; v++) Fo[v * nf + f] = F[v];
}

template <int D, int TYP, int KF, int SL, bool VISC, int NV = 5>
__global__ void __launch_bounds__(128) face_flux(Zone z, const double* __restrict__ q,
                                                 const double* __restrict__ xmut,
                                                 double* __restrict__ Fo) {
  face_flux_at<D, TYP, KF, SL, VISC, NV>(z, q, xmut, Fo, (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
}

// Zone batches: one launch for the same kernel over several zones of the
// same kind.  The zones' descriptors and arguments travel in the kernel
// parameter (__grid_constant__, read in place); block b belongs to the zone
// m with bstart[m] <= b < bstart[m + 1], and every thread of a block reads
// the same entry (a uniform constant-bank access).
__device__ __forceinline__ int batch_zone(const int64_t* bstart, int nz, int64_t b) {
  int lo = 0, hi = nz - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (bstart[mid] <= b) lo = mid; else hi = mid - 1;
  }
  return lo;
}

template <int D, int TYP, int KF, int SL, bool VISC, int NV = 5>
__global__ void __launch_bounds__(256) face_flux_batch(const __grid_constant__ FaceBatch b) {
  const int m = batch_zone(b.bstart, b.nz, blockIdx.x);
  const FaceEntry& e = b.e[m];
  face_flux_at<D, TYP, KF, SL, VISC, NV>(e.z, e.q, e.xmut, e.F[D],
                                         (int64_t)(blockIdx.x - b.bstart[m]) * blockDim.x + threadIdx.x);
}

// --------------------------------------------------------- assemble+update
// cons energy of a primitive state (core3ark3.for:127-150 / core3as2.for)
__device__ __forceinline__ double roe_of(double cv, double r, double u, double v, double w,
                                         double t) {
  return r * (cv * t + mul_pow2<-1>(u * u + v * v + w * w));
}

// NV = 6 (Spalart-Allmaras): the ro nutilde balance starts from drodm(:,6),
// which sa_source has initialised and given the source term; the updates
// are core3ark3.for's nutilde branch (clipped to [0, ratiom nu_lam]) and
// core3as2.for's sixth residual.
template <bool IMPL, int NV = 5>
__device__ __forceinline__ void assemble_at(const Zone& z, const StageArgs& a, const int64_t t) {
  const int64_t n = z.ni * z.nj * z.nk;
  if (t >= n) return;
  const int64_t ii = t % z.ni;
  const int64_t r = t / z.ni;
  const int64_t jj = r % z.nj, kk = r / z.nj;
  const int64_t l = inddm(z, ii + 1, jj + 1, kk + 1);
  const int64_t nd = z.nd;
  const int64_t nfi = (z.ni + 1) * z.nj * z.nk, nfj = z.ni * (z.nj + 1) * z.nk,
                nfk = z.ni * z.nj * (z.nk + 1);
  const int64_t ai = ii + (z.ni + 1) * (jj + z.nj * kk);
  const int64_t aj = ii + z.ni * (jj + (z.nj + 1) * kk);
  const int64_t ak = ii + z.ni * (jj + z.nj * kk);
  double x[NV];
  if (a.mode == 2) {  // balance already in drodm (corrected by wall_corr)
#pragma unroll
    for (int v = 0; v < NV; v++) x[v] = a.drodm[l + v * nd];
  } else {
    const bool two_d = z.typ == Z2D;   // no k faces
#pragma unroll
    for (int v = 0; v < NV; v++) {
      double s = v == 5 ? a.drodm[l + v * nd] : (a.zero_init ? 0. : a.drodm[l + v * nd] * a.coefH);
      if (!two_d) s = s + a.Fk[v * nfk + ak];
      s = s + a.Fj[v * nfj + aj];
      s = s + a.Fi[v * nfi + ai];
      s = s - a.Fi[v * nfi + ai + 1];
      s = s - a.Fj[v * nfj + aj + z.ni];
      if (!two_d) s = s - a.Fk[v * nfk + ak + z.ni * z.nj];
      x[v] = s;
    }
    if (a.mode == 1) {
#pragma unroll
      for (int v = 0; v < NV; v++) a.drodm[l + v * nd] = x[v];
      return;
    }
  }
  const double cv = z.cv;
  if (!IMPL) {
#pragma unroll
    for (int v = 0; v < NV; v++) a.drodm[l + v * nd] = x[v];
    // core3ark3.for:99-125
    const double* R = a.rop_in;
    double r_1 = a.coefW * a.coe[l];
    double tab1 = x[0] * r_1, tab2 = x[1] * r_1, tab3 = x[2] * r_1, tab4 = x[3] * r_1,
           tab5 = x[4] * r_1;
    double ro = R[l], u = R[l + nd], v = R[l + 2 * nd], w = R[l + 3 * nd], tt = R[l + 4 * nd];
    double n1 = ro + tab1;
    double rr = 1. / n1;
    double n2 = (ro * u + tab2) * rr;
    double n3 = (ro * v + tab3) * rr;
    double cvinv = 1. / cv, cvinv2 = mul_pow2<-1>(cvinv);
    double n4, n5;
    if (z.typ == Z2D) {  // core3ark3.for 2-d branch: w = 0
      n4 = 0.;
      double roe_old = ro * (cv * tt + mul_pow2<-1>(u * u + v * v));
      n5 = (roe_old + tab5) * rr * cvinv - cvinv2 * (n2 * n2 + n3 * n3);
    } else {
      n4 = (ro * w + tab4) * rr;
      double roe_old = ro * (cv * tt + mul_pow2<-1>(u * u + v * v + w * w));
      n5 = (roe_old + tab5) * rr * cvinv - cvinv2 * (n2 * n2 + n3 * n3 + n4 * n4);
    }
    double* O = a.rop_out;
    O[l] = n1; O[l + nd] = n2; O[l + 2 * nd] = n3; O[l + 3 * nd] = n4; O[l + 4 * nd] = n5;
    if (NV == 6) {   // core3ark3.for:188-236
      const double tab6 = x[NV - 1] * r_1;
      double anulam = sa_mulam(z, n5);
      anulam = anulam * rr * z.ratiom;
      double t6 = (ro * R[l + 5 * nd] + tab6) * rr;
      t6 = fminF(t6, anulam);
      O[l + 5 * nd] = fmaxF(t6, 0.);
    }
  } else {
    // core3as2.for:233-330 (5 equations, 3d)
    const double* P = a.rop_in;   // W^p (rop_ssiter)
    const double* N = a.rop_n;    // W^n
    const double* M = a.rop_n1;   // W^{n-1}
    const double cf = a.coe[l];
    double pr_ = P[l], pu = P[l + nd], pv = P[l + 2 * nd], pw = P[l + 3 * nd], pt = P[l + 4 * nd];
    double mr = M[l], mu = M[l + nd], mv = M[l + 2 * nd], mw = M[l + 3 * nd], mt = M[l + 4 * nd];
    double y[NV];
    // BDF2 (c1, c2, c3) = (-1.5, 2, -0.5): the products by c2, c3 and
    // c1 + c2 = 0.5 are products by powers of two (mul_pow2, the same bits);
    // other coefficients (BDF1) take the FP64 multiplies
    auto balance = [&](auto bdf2_tag) {
      constexpr bool B2 = decltype(bdf2_tag)::value;
      auto c2m = [&](double v) { return B2 ? mul_pow2<1>(v) : a.c2 * v; };
      auto c3m = [&](double v) { return B2 ? mul_pow2<-1, true>(v) : a.c3 * v; };
      if (a.first_sub && NV == 6 && z.dtloc == 1) {   // core3as2.for:57-66, 106-114
#pragma unroll
        for (int v = 0; v < NV; v++) y[v] = cf * x[v];
      } else if (a.first_sub) {
        double c4 = a.c1 + a.c2;
        auto c4m = [&](double v) { return B2 ? mul_pow2<-1>(v) : c4 * v; };
        y[0] = cf * x[0] + c4m(pr_) + c3m(mr);
        y[1] = cf * x[1] + c4m(pu) * pr_ + c3m(mu) * mr;
        y[2] = cf * x[2] + c4m(pv) * pr_ + c3m(mv) * mr;
        y[3] = cf * x[3] + c4m(pw) * pr_ + c3m(mw) * mr;
        double roe = roe_of(cv, pr_, pu, pv, pw, pt);
        double roe1 = roe_of(cv, mr, mu, mv, mw, mt);
        y[4] = cf * x[4] + c4m(roe) + c3m(roe1);
        if (NV == 6)   // core3as2.for:97-99
          y[NV - 1] = cf * x[NV - 1] + c4m(P[l + 5 * nd]) * pr_ + c3m(M[l + 5 * nd]) * mr;
      } else {
        double nr = N[l], nu = N[l + nd], nv = N[l + 2 * nd], nw = N[l + 3 * nd], nt = N[l + 4 * nd];
        y[0] = cf * x[0] + a.c1 * pr_ + c2m(nr) + c3m(mr);
        y[1] = cf * x[1] + a.c1 * pu * pr_ + c2m(nu) * nr + c3m(mu) * mr;
        y[2] = cf * x[2] + a.c1 * pv * pr_ + c2m(nv) * nr + c3m(mv) * mr;
        y[3] = cf * x[3] + a.c1 * pw * pr_ + c2m(nw) * nr + c3m(mw) * mr;
        double roe = roe_of(cv, pr_, pu, pv, pw, pt);
        double roen = roe_of(cv, nr, nu, nv, nw, nt);
        double roe1 = roe_of(cv, mr, mu, mv, mw, mt);
        y[4] = cf * x[4] + a.c1 * roe + c2m(roen) + c3m(roe1);
        if (NV == 6)   // core3as2.for:187-190
          y[NV - 1] = cf * x[NV - 1] + a.c1 * P[l + 5 * nd] * pr_ + c2m(N[l + 5 * nd]) * nr +
                      c3m(M[l + 5 * nd]) * mr;
      }
    };
    if (a.c1 == -1.5 && a.c2 == 2. && a.c3 == -0.5) balance(std::true_type{});
    else balance(std::false_type{});
    // core3as2.for 2-d branch: the w residual is left as the balance, and
    // the energies have no w term (w = 0 in a 2-d state: the same values)
    if (z.typ == Z2D) y[3] = x[3];
#pragma unroll
    for (int v = 0; v < NV; v++) a.drodm[l + v * nd] = y[v];
  }
}

template <bool IMPL, int NV = 5>
__global__ void __launch_bounds__(256) assemble(Zone z, StageArgs a) {
  assemble_at<IMPL, NV>(z, a, (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
}

template <bool IMPL, int NV = 5>
__global__ void __launch_bounds__(256) assemble_batch(const __grid_constant__ StageBatch b) {
  const int m = batch_zone(b.bstart, b.nz, blockIdx.x);
  assemble_at<IMPL, NV>(b.e[m].z, b.e[m].a,
                        (int64_t)(blockIdx.x - b.bstart[m]) * blockDim.x + threadIdx.x);
}

// -------------------------------------------------- Spalart-Allmaras source
// SA/spsource_SA.for with sourceSA_grad_3dcart.for / sourceSA_grad_3d.for,
// sourceSA_prod_dest.for and sourceSA_LU.for, fused with init_rhs.for for
// the sixth equation: drodm(l,6) = init + vol * (production + cross
// diffusion - destruction); on the first implicit sub-step also
// coe(l,6) = coe(l,5) - min(d source / d(ro nutilde), 0) coe(l,1).  One
// thread per interior cell (the reference's first ghost ring is never read).
template <int TYP>
__device__ __forceinline__ void sa_source_at(const Zone& z, const double* __restrict__ q,
                                             double* __restrict__ drodm, double* __restrict__ coe,
                                             double coefH, int zero_init, int lu, const int64_t t) {
  const int64_t n = z.ni * z.nj * z.nk;
  if (t >= n) return;
  const int64_t ii = t % z.ni, r0 = t / z.ni, jj = r0 % z.nj, kk = r0 / z.nj;
  const int64_t l = inddm(z, ii + 1, jj + 1, kk + 1);
  const int64_t lt = TYP == Z3DCART ? 0 : indmtr(z, ii + 1, jj + 1, kk + 1);
  const int64_t nd = z.nd, ndm = z.ndm;
  const int64_t l1 = l + 1, l2 = l - 1, l3 = l + z.inc[1], l4 = l - z.inc[1], l5 = l + z.inc[2],
                l6 = l - z.inc[2];
  const double* Rr = q;
  const double* Nu = q + 5 * nd;
  const double vol = z.vol[lt];
  const double xvol = 0.5 / vol;
  double g[3][3], gn[3], gr[3];
  if (TYP == Z2D) {       // sourceSA_grad_2d.for: i and j faces, u and v
    const double* TT[2] = {z.ti, z.tj};
    double t0[2][2], t1[2][2];
#pragma unroll
    for (int x = 0; x < 2; x++)
#pragma unroll
      for (int d = 0; d < 2; d++) {
        t0[x][d] = TT[d][lt + x * ndm];
        t1[x][d] = TT[d][lt + z.minc[d] + x * ndm];
      }
#pragma unroll
    for (int v = 0; v < 3; v++) {
      const double* Q = v < 2 ? q + (v + 1) * nd : Nu;
      const double u1 = (Q[l] + Q[l2]), u2 = (Q[l] + Q[l3]), u3 = (Q[l] + Q[l1]);
      const double u4 = (Q[l] + Q[l4]);
      double* o = v < 2 ? g[v] : gn;
#pragma unroll
      for (int x = 0; x < 2; x++) o[x] = (u3 * t1[x][0] - u1 * t0[x][0] + u2 * t1[x][1] - u4 * t0[x][1]);
    }
    const double a = Nu[l] * Rr[l];
    const double u1 = a + Nu[l2] * Rr[l2], u2 = a + Nu[l3] * Rr[l3], u3 = a + Nu[l1] * Rr[l1];
    const double u4 = a + Nu[l4] * Rr[l4];
#pragma unroll
    for (int x = 0; x < 2; x++) gr[x] = (u3 * t1[x][0] - u1 * t0[x][0] + u2 * t1[x][1] - u4 * t0[x][1]);
  } else if (TYP == Z3DCART) {   // sourceSA_grad_3dcart.for
    const double tix = z.ti[0], tjy = z.tj[0], tkz = z.tk[0];
#pragma unroll
    for (int v = 0; v < 4; v++) {
      const double* Q = v < 3 ? q + (v + 1) * nd : Nu;
      const double u1 = (Q[l] + Q[l2]), u2 = (Q[l] + Q[l3]), u3 = (Q[l] + Q[l1]);
      const double u4 = (Q[l] + Q[l4]), u5 = (Q[l] + Q[l5]), u6 = (Q[l] + Q[l6]);
      double* o = v < 3 ? g[v] : gn;
      o[0] = (u3 - u1) * tix;
      o[1] = (u2 - u4) * tjy;
      o[2] = (u5 - u6) * tkz;
    }
    const double a = Nu[l] * Rr[l];
    const double u1 = a + Nu[l2] * Rr[l2], u2 = a + Nu[l3] * Rr[l3], u3 = a + Nu[l1] * Rr[l1];
    const double u4 = a + Nu[l4] * Rr[l4], u5 = a + Nu[l5] * Rr[l5], u6 = a + Nu[l6] * Rr[l6];
    gr[0] = (u3 - u1) * tix;
    gr[1] = (u2 - u4) * tjy;
    gr[2] = (u5 - u6) * tkz;
  } else {                // sourceSA_grad_3d.for
    const double* TT[3] = {z.ti, z.tj, z.tk};
    double t0[3][3], t1[3][3];   // [component][face family]: faces lt and lt + inc_d
#pragma unroll
    for (int x = 0; x < 3; x++)
#pragma unroll
      for (int d = 0; d < 3; d++) {
        t0[x][d] = TT[d][lt + x * ndm];
        t1[x][d] = TT[d][lt + z.minc[d] + x * ndm];
      }
#pragma unroll
    for (int v = 0; v < 4; v++) {
      const double* Q = v < 3 ? q + (v + 1) * nd : Nu;
      const double u1 = (Q[l] + Q[l2]), u2 = (Q[l] + Q[l3]), u3 = (Q[l] + Q[l1]);
      const double u4 = (Q[l] + Q[l4]), u5 = (Q[l] + Q[l5]), u6 = (Q[l] + Q[l6]);
      double* o = v < 3 ? g[v] : gn;
#pragma unroll
      for (int x = 0; x < 3; x++)
        o[x] = (u3 * t1[x][0] - u1 * t0[x][0] + u2 * t1[x][1] - u4 * t0[x][1] +
                u5 * t1[x][2] - u6 * t0[x][2]);
    }
    const double a = Nu[l] * Rr[l];
    const double u1 = a + Nu[l2] * Rr[l2], u2 = a + Nu[l3] * Rr[l3], u3 = a + Nu[l1] * Rr[l1];
    const double u4 = a + Nu[l4] * Rr[l4], u5 = a + Nu[l5] * Rr[l5], u6 = a + Nu[l6] * Rr[l6];
#pragma unroll
    for (int x = 0; x < 3; x++)
      gr[x] = (u3 * t1[x][0] - u1 * t0[x][0] + u2 * t1[x][1] - u4 * t0[x][1] +
               u5 * t1[x][2] - u6 * t0[x][2]);
  }
  // vorticity and strain magnitudes
  const double c1 = SA_CB2 / SA_SIGMA;
  const double cw1 = (SA_CB1 / SA_CKARM / SA_CKARM) + (1. + SA_CB2) / SA_SIGMA;
  double rot, St, anvisc;
  if (TYP == Z2D) {
    const double rotz = g[1][0] - g[0][1];
    rot = fabs(rotz) * xvol;
    const double S11 = g[0][0], S22 = g[1][1], S12 = mul_pow2<-1>(g[0][1] + g[1][0]);
    St = S11 * S11 + S22 * S22 + mul_pow2<1>(S12 * S12);
    St = sqrt(mul_pow2<1>(St)) * xvol;
    anvisc = c1 * (gn[0] * gr[0] + gn[1] * gr[1]) * xvol * xvol;
  } else {
    const double rotx = g[2][1] - g[1][2], roty = g[0][2] - g[2][0], rotz = g[1][0] - g[0][1];
    rot = sqrt(rotx * rotx + roty * roty + rotz * rotz) * xvol;
    const double S11 = g[0][0], S22 = g[1][1], S33 = g[2][2];
    const double S12 = mul_pow2<-1>(g[0][1] + g[1][0]), S13 = mul_pow2<-1>(g[0][2] + g[2][0]),
                 S23 = mul_pow2<-1>(g[1][2] + g[2][1]);
    St = S11 * S11 + S22 * S22 + S33 * S33 + mul_pow2<1>(S12 * S12) + mul_pow2<1>(S13 * S13) +
         mul_pow2<1>(S23 * S23);
    St = sqrt(mul_pow2<1>(St)) * xvol;
    anvisc = c1 * (gn[0] * gr[0] + gn[1] * gr[1] + gn[2] * gr[2]) * xvol * xvol;
  }
  // mulam.for, SA/chi.for
  const double amulam = sa_mulam(z, q[l + 4 * nd]);
  const double anulam = Rr[l] / amulam;
  const double anutild = fmaxF(Nu[l], 1.e-27);
  const double chi = fmaxF(anutild * anulam, 1.e-7);
  // sourceSA_prod_dest.for
  const double f1 = 1. / (1. + SA_CV1 / (chi * chi * chi));
  const double f2 = 1. - chi / (1. + chi * f1);
  const double dist = fmaxF(z.dist[l], 1.e-27);
  double stild = rot + (anutild * f2) / (SA_CKARM * SA_CKARM * dist * dist);
  stild = stild + z.sa_rot * SA_CROT * fminF(0.00000000000000000001, St - rot);
  const double prod = Rr[l] * SA_CB1 * stild * anutild;
  stild = fmaxF(stild, 0.00000000000000000001);
  double rr = anutild / (stild * SA_CKARM * SA_CKARM * dist * dist);
  rr = fminF(rr, 10.);
  const double r5 = rr * rr * rr * rr * rr - 1.;
  double gg = rr * (1. + SA_CW2 * r5);
  const double lre = 1. + chi / 40.;
  const double cw2_lre = SA_CW4 + SA_CW5 / (lre * lre);
  gg = z.sa_low_re * rr * (1. + cw2_lre * r5) + (1. - z.sa_low_re) * gg;
  const double g3 = gg * gg * gg, g6 = g3 * g3;   // g**6 as the Fortran compiler expands it
  const double fwg = gg * pow((1. + SA_CW3) / (g6 + SA_CW3), 1. / 6.);
  const double destruc = Rr[l] * cw1 * fwg * (anutild / dist) * (anutild / dist);
  const double tsource = (prod + anvisc - destruc);
  if (lu) {   // sourceSA_LU.for
    const double tsourceb = prod - destruc;
    double amutild = anutild * Rr[l];
    amutild = fmaxF(amutild, 0.0000000000000001);
    const double tsourcenu = vol * tsourceb / amutild;
    coe[l + 5 * nd] = coe[l + 4 * nd] - fminF(tsourcenu, 0.) * coe[l];
  }
  const double init = zero_init ? 0. : drodm[l + 5 * nd] * coefH;
  drodm[l + 5 * nd] = init + vol * tsource;
}

template <int TYP>
__global__ void __launch_bounds__(256) sa_source(Zone z, const double* __restrict__ q,
                                                 double* __restrict__ drodm, double* __restrict__ coe,
                                                 double coefH, int zero_init, int lu) {
  sa_source_at<TYP>(z, q, drodm, coe, coefH, zero_init, lu, (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
}

template <int TYP>
__global__ void __launch_bounds__(256) sa_source_batch(const __grid_constant__ SaBatch b) {
  const int m = batch_zone(b.bstart, b.nz, blockIdx.x);
  const SaEntry& e = b.e[m];
  sa_source_at<TYP>(e.z, e.q, e.drodm, e.coe, b.coefH, b.zero_init, b.lu,
                    (int64_t)(blockIdx.x - b.bstart[m]) * blockDim.x + threadIdx.x);
}

cudaError_t launch_sa_source(const Zone& z, const double* q, double* drodm, double* coe,
                             double coefH, int zero_init, int lu, cudaStream_t st) {
  const int B = 256;
  const int64_t n = z.ni * z.nj * z.nk;
  const unsigned g = (unsigned)((n + B - 1) / B);
  if (z.typ == Z3DCART) sa_source<Z3DCART><<<g, B, 0, st>>>(z, q, drodm, coe, coefH, zero_init, lu);
  else if (z.typ == Z3DFULL) sa_source<Z3DFULL><<<g, B, 0, st>>>(z, q, drodm, coe, coefH, zero_init, lu);
  else if (z.typ == Z2D) sa_source<Z2D><<<g, B, 0, st>>>(z, q, drodm, coe, coefH, zero_init, lu);
  else return cudaErrorNotSupported;
  return cudaGetLastError();
}

// ------------------------------------------------- taped faces (adjoint)
// face_flux<D, Z2D, ROE, VANALBADA, false> that also writes, per face, the
// values a reverse pass needs and would otherwise recompute with square
// roots and divisions (FACE_TAPE doubles, face-major stride nf): |S|, the
// Roe-flux values of roe_full<true>, and per variable (ro, u, v, T) and
// side the van Albada slope va and the reciprocal of its denominator.  The
// flux is computed by the same expressions as face_flux: F is the same.
template <int D>
__global__ void __launch_bounds__(128) face_flux_tape(Zone z, const double* __restrict__ q,
                                                      double* __restrict__ Fo,
                                                      double* __restrict__ tape) {
  const int64_t NI = z.ni + (D == 0), NJ = z.nj + (D == 1);
  const int64_t nf = NI * NJ;
  const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  const int64_t ii = f % NI, jj = f / NI;
  const int64_t l = inddm(z, ii + 1, jj + 1, 1);
  const int64_t inc = z.inc[D], nd = z.nd;
  double* T = tape + f;
  double qm[5], qp[5];
#pragma unroll
  for (int v = 0; v < 5; v++) {
    if (v == 3) { qm[v] = 0.; qp[v] = 0.; continue; }
    const double* Q = q + v * nd;
    const double a = Q[l - 2 * inc], b = Q[l - inc], c = Q[l], d = Q[l + inc];
    const double x1 = c - b, y1 = d - c, x2 = b - a, y2 = c - b;
    const double vm = vanalbada(x1, y1), vp = vanalbada(x2, y2);
    qm[v] = c - mul_pow2<-1>(vm);
    qp[v] = b + mul_pow2<-1>(vp);
    const int m = v == 4 ? 3 : v;
    T[(TAPE_VA + 2 * m) * nf] = vm;
    T[(TAPE_VA + 2 * m + 1) * nf] = vp;
    T[(TAPE_ID + 2 * m) * nf] = 1. / (x1 * x1 + y1 * y1 + 2. * 1e-12);
    T[(TAPE_ID + 2 * m + 1) * nf] = 1. / (x2 * x2 + y2 * y2 + 2. * 1e-12);
  }
  const int64_t lt = indmtr(z, ii + 1, jj + 1, 1);
  const double* t = D == 0 ? z.ti : z.tj;
  const double tcx = t[lt], tcy = t[lt + z.ndm];
  const double s = sqrt(tcx * tcx + tcy * tcy);
  T[0] = s;
  double F[5];
  roe_full<true>(z, qm, qp, tcx, tcy, 0., s, F, T, nf);
  F[3] = 0.;
#pragma unroll
  for (int v = 0; v < 5; v++) Fo[v * nf + f] = F[v];
}

cudaError_t launch_faces_tape(const Zone& z, const double* q, double* Fi, double* Fj, double* tape,
                              cudaStream_t st) {
  if (z.typ != Z2D || z.kflu != ROE || z.slope != VANALBADA || z.iflow != 1)
    return cudaErrorNotSupported;
  const int B = 128;
  const int64_t nfi = (z.ni + 1) * z.nj, nfj = z.ni * (z.nj + 1);
  face_flux_tape<0><<<(unsigned)((nfi + B - 1) / B), B, 0, st>>>(z, q, Fi, tape);
  face_flux_tape<1><<<(unsigned)((nfj + B - 1) / B), B, 0, st>>>(z, q, Fj, tape + FACE_TAPE * nfi);
  return cudaGetLastError();
}

// ------------------------------------------------------------ host glue
#define FGB_CHECK_LAUNCH() \
  do { cudaError_t e_ = cudaGetLastError(); if (e_ != cudaSuccess) return e_; } while (0)

template <int TYP, int KF, int SL, bool VISC, int NV = 5>
static cudaError_t launch_faces_t(const Zone& z, const double* q, const double* xmut, double* Fi,
                                  double* Fj, double* Fk, cudaStream_t st) {
  const int B = 128;
  int64_t nfi = (z.ni + 1) * z.nj * z.nk, nfj = z.ni * (z.nj + 1) * z.nk,
          nfk = z.ni * z.nj * (z.nk + 1);
  face_flux<0, TYP, KF, SL, VISC, NV><<<(unsigned)((nfi + B - 1) / B), B, 0, st>>>(z, q, xmut, Fi);
  FGB_CHECK_LAUNCH();
  face_flux<1, TYP, KF, SL, VISC, NV><<<(unsigned)((nfj + B - 1) / B), B, 0, st>>>(z, q, xmut, Fj);
  FGB_CHECK_LAUNCH();
  if (TYP != Z2D) {
    face_flux<2, TYP, KF, SL, VISC, NV><<<(unsigned)((nfk + B - 1) / B), B, 0, st>>>(z, q, xmut, Fk);
    FGB_CHECK_LAUNCH();
  }
  return cudaSuccess;
}

// *_o3sc_*: the o3 slope blended by the shock sensor; Euler / laminar /
// Spalart-Allmaras, AUSM+(P), senseur and Roe.
template <int TYP, class Op>
static cudaError_t faces_o3sc(const Zone& z, Op& op) {
  if (z.neq == 6) {
    if (z.kflu == ROE) return op.template run<TYP, ROE, O3SC, true, 6>();
    if (z.kflu == AUSM) return op.template run<TYP, AUSM, O3SC, true, 6>();
    if (z.kflu == SENSEUR) return op.template run<TYP, SENSEUR, O3SC, true, 6>();
    return cudaErrorNotSupported;
  }
  const bool visc = z.iflow >= 2;
  if (z.kflu == ROE) return visc ? op.template run<TYP, ROE, O3SC, true>()
                                 : op.template run<TYP, ROE, O3SC, false>();
  if (z.kflu == AUSM) return visc ? op.template run<TYP, AUSM, O3SC, true>()
                                  : op.template run<TYP, AUSM, O3SC, false>();
  if (z.kflu == SENSEUR) return visc ? op.template run<TYP, SENSEUR, O3SC, true>()
                                     : op.template run<TYP, SENSEUR, O3SC, false>();
  return cudaErrorNotSupported;
}

// Dispatch over the (zone type, scheme, slope, viscous) combinations that the
// reference generates for 3d zones.  Returns cudaErrorNotSupported for the
// others (host code reports it as an argument error, never falls back).
// o5 / o5sc: AUSM+(P) only (the reference's senseur o5 variant needs the
// time-dependent wiggle2023 sensor)
template <int TYP, int SL, class Op>
static cudaError_t faces_o5(const Zone& z, Op& op) {
  if (z.kflu != AUSM) return cudaErrorNotSupported;
  if (z.neq == 6) return op.template run<TYP, AUSM, SL, true, 6>();
  return z.iflow >= 2 ? op.template run<TYP, AUSM, SL, true>() : op.template run<TYP, AUSM, SL, false>();
}

template <class Op>
static cudaError_t faces_dispatch(const Zone& z, Op& op) {
  const bool visc = z.iflow >= 2;
  if (z.slope == O5 || z.slope == O5SC) {
    const bool sc = z.slope == O5SC;
    if (z.typ == Z3DCART) return sc ? faces_o5<Z3DCART, O5SC>(z, op) : faces_o5<Z3DCART, O5>(z, op);
    if (z.typ == Z3DFULL) return sc ? faces_o5<Z3DFULL, O5SC>(z, op) : faces_o5<Z3DFULL, O5>(z, op);
    if (z.typ == Z2D) return sc ? faces_o5<Z2D, O5SC>(z, op) : faces_o5<Z2D, O5>(z, op);
    return cudaErrorNotSupported;
  }
  if (z.slope == O3SC) {
    if (z.typ == Z3DCART) return faces_o3sc<Z3DCART>(z, op);
    if (z.typ == Z3DFULL) return faces_o3sc<Z3DFULL>(z, op);
    if (z.typ == Z2D) return faces_o3sc<Z2D>(z, op);
    return cudaErrorNotSupported;
  }
  if (z.neq == 6 && z.typ == Z2D) {   // Spalart-Allmaras on 2-d zones
    if (z.kflu == AUSM && z.slope == O3) return op.template run<Z2D, AUSM, O3, true, 6>();
    if (z.kflu == SENSEUR && z.slope == O3) return op.template run<Z2D, SENSEUR, O3, true, 6>();
    if (z.kflu == ROE && z.slope == O1) return op.template run<Z2D, ROE, O1, true, 6>();
    if (z.kflu == ROE && z.slope == O3) return op.template run<Z2D, ROE, O3, true, 6>();
    if (z.kflu == ROE && z.slope == MINMOD) return op.template run<Z2D, ROE, MINMOD, true, 6>();
    return cudaErrorNotSupported;
  }
  if (z.neq == 6) {   // Spalart-Allmaras: AUSM+(P) o3 or Roe o1 / o3 / minmod, 3d zones
    const bool cart = z.typ == Z3DCART;
    if (z.typ != Z3DCART && z.typ != Z3DFULL) return cudaErrorNotSupported;
    if (z.kflu == AUSM && z.slope == O3)
      return cart ? op.template run<Z3DCART, AUSM, O3, true, 6>()
                  : op.template run<Z3DFULL, AUSM, O3, true, 6>();
    if (z.kflu == SENSEUR && z.slope == O3)   // SENSOR/*/fluFaceSA_o3_*: the AUSM form, sensor u / tdu
      return cart ? op.template run<Z3DCART, SENSEUR, O3, true, 6>()
                  : op.template run<Z3DFULL, SENSEUR, O3, true, 6>();
    if (z.kflu == ROE && z.slope == O1)
      return cart ? op.template run<Z3DCART, ROE, O1, true, 6>()
                  : op.template run<Z3DFULL, ROE, O1, true, 6>();
    if (z.kflu == ROE && z.slope == O3)
      return cart ? op.template run<Z3DCART, ROE, O3, true, 6>()
                  : op.template run<Z3DFULL, ROE, O3, true, 6>();
    if (z.kflu == ROE && z.slope == MINMOD)
      return cart ? op.template run<Z3DCART, ROE, MINMOD, true, 6>()
                  : op.template run<Z3DFULL, ROE, MINMOD, true, 6>();
    return cudaErrorNotSupported;
  }
  if (z.typ == Z3DCART) {
    if (z.kflu == ROE) {
      if (z.slope == O1) return visc ? op.template run<Z3DCART, ROE, O1, true>()
                                     : op.template run<Z3DCART, ROE, O1, false>();
      if (z.slope == O3) return visc ? op.template run<Z3DCART, ROE, O3, true>()
                                     : op.template run<Z3DCART, ROE, O3, false>();
      if (z.slope == MINMOD) return visc ? op.template run<Z3DCART, ROE, MINMOD, true>()
                                         : op.template run<Z3DCART, ROE, MINMOD, false>();
      if (z.slope == VANALBADA && !visc) return op.template run<Z3DCART, ROE, VANALBADA, false>();
    } else if (z.kflu == AUSM && z.slope == O3) {
      return visc ? op.template run<Z3DCART, AUSM, O3, true>()
                  : op.template run<Z3DCART, AUSM, O3, false>();
    } else if (z.kflu == SENSEUR && z.slope == O3) {
      return visc ? op.template run<Z3DCART, SENSEUR, O3, true>()
                  : op.template run<Z3DCART, SENSEUR, O3, false>();
    }
  } else if (z.typ == Z3DFULL) {
    if (z.kflu == ROE) {
      if (z.slope == O1) return visc ? op.template run<Z3DFULL, ROE, O1, true>()
                                     : op.template run<Z3DFULL, ROE, O1, false>();
      if (z.slope == O3) return visc ? op.template run<Z3DFULL, ROE, O3, true>()
                                     : op.template run<Z3DFULL, ROE, O3, false>();
      if (z.slope == MINMOD) return visc ? op.template run<Z3DFULL, ROE, MINMOD, true>()
                                         : op.template run<Z3DFULL, ROE, MINMOD, false>();
      if (z.slope == VANALBADA && !visc) return op.template run<Z3DFULL, ROE, VANALBADA, false>();
    } else if (z.kflu == AUSM && z.slope == O3) {
      return visc ? op.template run<Z3DFULL, AUSM, O3, true>()
                  : op.template run<Z3DFULL, AUSM, O3, false>();
    } else if (z.kflu == SENSEUR && z.slope == O3) {
      return visc ? op.template run<Z3DFULL, SENSEUR, O3, true>()
                  : op.template run<Z3DFULL, SENSEUR, O3, false>();
    }
  }
  if (z.typ == Z2D) {   // 2-d zones: Euler / laminar, Roe o1 / o3 / minmod, AUSM+(P) o3
    if (z.kflu == ROE) {
      if (z.slope == O1) return visc ? op.template run<Z2D, ROE, O1, true>()
                                     : op.template run<Z2D, ROE, O1, false>();
      if (z.slope == O3) return visc ? op.template run<Z2D, ROE, O3, true>()
                                     : op.template run<Z2D, ROE, O3, false>();
      if (z.slope == MINMOD) return visc ? op.template run<Z2D, ROE, MINMOD, true>()
                                         : op.template run<Z2D, ROE, MINMOD, false>();
      if (z.slope == VANALBADA && !visc) return op.template run<Z2D, ROE, VANALBADA, false>();
    } else if (z.kflu == AUSM && z.slope == O3) {
      return visc ? op.template run<Z2D, AUSM, O3, true>()
                  : op.template run<Z2D, AUSM, O3, false>();
    } else if (z.kflu == SENSEUR && z.slope == O3) {
      return visc ? op.template run<Z2D, SENSEUR, O3, true>()
                  : op.template run<Z2D, SENSEUR, O3, false>();
    }
  }
  return cudaErrorNotSupported;
}

struct FacesOne {
  const Zone& z; const double* q; const double* xmut; double *Fi, *Fj, *Fk; cudaStream_t st;
  template <int TYP, int KF, int SL, bool VISC, int NV = 5>
  cudaError_t run() { return launch_faces_t<TYP, KF, SL, VISC, NV>(z, q, xmut, Fi, Fj, Fk, st); }
};

cudaError_t launch_faces(const Zone& z, const double* q, const double* xmut, double* Fi,
                         double* Fj, double* Fk, cudaStream_t st) {
  FacesOne op{z, q, xmut, Fi, Fj, Fk, st};
  return faces_dispatch(z, op);
}

// A batch of zones of one kind: the faces of direction D of every zone in
// one launch, blocks of b.block threads.
struct FacesBatchOp {
  FaceBatch& b; cudaStream_t st;
  template <int TYP, int KF, int SL, bool VISC, int NV = 5>
  cudaError_t run() {
    const int B = b.block;
    for (int D = 0; D < (TYP == Z2D ? 2 : 3); D++) {
      b.bstart[0] = 0;
      for (int m = 0; m < b.nz; m++) {
        const Zone& z = b.e[m].z;
        const int64_t nf = (z.ni + (D == 0)) * (z.nj + (D == 1)) * (z.nk + (D == 2));
        b.bstart[m + 1] = b.bstart[m] + (nf + B - 1) / B;
      }
      const unsigned g = (unsigned)b.bstart[b.nz];
      if (D == 0) face_flux_batch<0, TYP, KF, SL, VISC, NV><<<g, B, 0, st>>>(b);
      else if (D == 1) face_flux_batch<1, TYP, KF, SL, VISC, NV><<<g, B, 0, st>>>(b);
      else face_flux_batch<2, TYP, KF, SL, VISC, NV><<<g, B, 0, st>>>(b);
      cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
  }
};

cudaError_t launch_faces_batch(FaceBatch& b, cudaStream_t st) {
  if (b.nz <= 0) return cudaSuccess;
  if (b.block != 64 && b.block != 128 && b.block != 256) return cudaErrorInvalidValue;
  FacesBatchOp op{b, st};
  return faces_dispatch(b.e[0].z, op);
}

int faces_batch_blocks(int* out, int nmax) {
  const int c[3] = {64, 128, 256};
  int n = 0;
  for (int k = 0; k < 3 && n < nmax; k++) out[n++] = c[k];
  return n;
}

// the template instance a zone's faces use
int64_t faces_kind_key(const Zone& z) {
  return (int64_t)z.typ | ((int64_t)z.kflu << 4) | ((int64_t)z.slope << 8) |
         ((int64_t)(z.iflow >= 2) << 12) | ((int64_t)z.neq << 13);
}

cudaError_t launch_assemble_batch(StageBatch& b, bool implicit, cudaStream_t st) {
  if (b.nz <= 0) return cudaSuccess;
  const int B = 256;
  b.bstart[0] = 0;
  for (int m = 0; m < b.nz; m++) {
    const Zone& z = b.e[m].z;
    b.bstart[m + 1] = b.bstart[m] + (z.ni * z.nj * z.nk + B - 1) / B;
  }
  const unsigned g = (unsigned)b.bstart[b.nz];
  const bool sa = b.e[0].z.neq == 6;
  if (implicit) {
    if (sa) assemble_batch<true, 6><<<g, B, 0, st>>>(b);
    else assemble_batch<true, 5><<<g, B, 0, st>>>(b);
  } else {
    if (sa) assemble_batch<false, 6><<<g, B, 0, st>>>(b);
    else assemble_batch<false, 5><<<g, B, 0, st>>>(b);
  }
  return cudaGetLastError();
}

cudaError_t launch_sa_source_batch(SaBatch& b, cudaStream_t st) {
  if (b.nz <= 0) return cudaSuccess;
  const int B = 256;
  b.bstart[0] = 0;
  for (int m = 0; m < b.nz; m++) {
    const Zone& z = b.e[m].z;
    b.bstart[m + 1] = b.bstart[m] + (z.ni * z.nj * z.nk + B - 1) / B;
  }
  const unsigned g = (unsigned)b.bstart[b.nz];
  const int typ = b.e[0].z.typ;
  if (typ == Z3DCART) sa_source_batch<Z3DCART><<<g, B, 0, st>>>(b);
  else if (typ == Z3DFULL) sa_source_batch<Z3DFULL><<<g, B, 0, st>>>(b);
  else if (typ == Z2D) sa_source_batch<Z2D><<<g, B, 0, st>>>(b);
  else return cudaErrorNotSupported;
  return cudaGetLastError();
}

// --------------------------------------------------- wall correction (Roe)
// BC/correct_flux.for, lapply = 4: for each face of a wall window, remove
// the Euler Roe flux of the face from the balance of its interior cell
// (corr_fluroe_euler_*: the same reconstruction and Roe flux as face_flux),
// then add the wall flux (CL_correction_flu.for: bflwallslip.for /
// bflwall.for) built from the face-averaged state.  One thread per face;
// the windows of one BC have distinct cells, BCs run one after another.
template <int D, int TYP, int SL>
__global__ void __launch_bounds__(128) wall_corr(Zone z, const double* __restrict__ q,
                                                 double* __restrict__ drodm, WallCorrArgs a) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= a.n) return;
  const int64_t l = a.l[e], l0 = a.l0[e], nd = z.nd, inc = z.inc[D];
  double qm[5], qp[5];
  double roff = 0.;
  if (SL == MINMOD) roff = mul_pow2<-1>(fmaxF(0., fminF(q[l + 4 * nd] * z.tmin_1 - .5, 1.)));
  if (SL == O3SC) roff = z.wig[l + D * nd];
#pragma unroll
  for (int v = 0; v < 5; v++) {
    if (TYP == Z2D && v == 3) { qm[v] = 0.; qp[v] = 0.; continue; }
    const double* Q = q + v * nd;
    double aa = (SL == O1) ? 0. : Q[l - 2 * inc];
    double bb = Q[l - inc], cc = Q[l];
    double dd = (SL == O1) ? 0. : Q[l + inc];
    reconstruct<SL>(z, aa, bb, cc, dd, roff, qm[v], qp[v]);
  }
  double F[5];
  if (TYP == Z3DCART) {
    roe_cart<D>(z, qm, qp, F);
  } else if (TYP == Z2D) {
    const int64_t lt = a.lt[e];
    const double* t = D == 0 ? z.ti : z.tj;
    double tcx = t[lt], tcy = t[lt + z.ndm];
    double s = sqrt(tcx * tcx + tcy * tcy);
    roe_full(z, qm, qp, tcx, tcy, 0., s, F);
    F[3] = 0.;
  } else {
    const int64_t lt = a.lt[e];
    const double* t = D == 0 ? z.ti : (D == 1 ? z.tj : z.tk);
    double tcx = t[lt], tcy = t[lt + z.ndm], tcz = t[lt + 2 * z.ndm];
    double s = sqrt(tcx * tcx + tcy * tcy + tcz * tcz);
    roe_full(z, qm, qp, tcx, tcy, tcz, s, F);
  }
  double x[5];
#pragma unroll
  for (int v = 0; v < 5; v++) x[v] = drodm[l0 + v * nd] + (F[v] * a.sens_c + 0.);
  const int64_t ia = l - inc;   // iadrf
  const double t0 = a.nrm[3 * e], t1 = a.nrm[3 * e + 1], t2 = a.nrm[3 * e + 2];
  const double qen = 0.;
  const double r = mul_pow2<-1>(q[l] + q[ia]);
  const double u = mul_pow2<-1>(q[l + nd] + q[ia + nd]);
  const double v = mul_pow2<-1>(q[l + 2 * nd] + q[ia + 2 * nd]);
  const double w = mul_pow2<-1>(q[l + 3 * nd] + q[ia + 3 * nd]);
  const double u_int = t0 * u + t1 * v + t2 * w - qen;
  double fw[5];
  if (a.slip) {
    double p = q[ia + 4 * nd] * q[ia] * a.rgp;
    const double h = a.gam2 * p + mul_pow2<-1>(r * (u * u + v * v + w * w));
    p = mul_pow2<-1>(q[l + 4 * nd] * q[l] + q[ia + 4 * nd] * q[ia]) * a.rgp;
    fw[0] = u_int * r;
    fw[1] = t0 * p + u_int * r * u;
    fw[2] = t1 * p + u_int * r * v;
    fw[3] = t2 * p + u_int * r * w;
    fw[4] = u_int * h + p * qen;
  } else {
    const double p = mul_pow2<-1>(q[l + 4 * nd] * q[l] + q[ia + 4 * nd] * q[ia]) * a.rgp;
    fw[0] = 0.;
    fw[1] = t0 * p + u_int * u * r;
    fw[2] = t1 * p + u_int * v * r;
    fw[3] = t2 * p + u_int * w * r;
    fw[4] = p * qen;
  }
#pragma unroll
  for (int m = 0; m < 5; m++) drodm[l0 + m * nd] = x[m] + fw[m] * a.sens_w;
}

template <int D, int TYP>
static void wall_corr_sl(const Zone& z, const double* q, double* drodm, const WallCorrArgs& a,
                         cudaStream_t st) {
  const unsigned g = (unsigned)((a.n + 127) / 128);
  if (z.slope == O1) wall_corr<D, TYP, O1><<<g, 128, 0, st>>>(z, q, drodm, a);
  else if (z.slope == O3) wall_corr<D, TYP, O3><<<g, 128, 0, st>>>(z, q, drodm, a);
  else if (z.slope == O3SC) wall_corr<D, TYP, O3SC><<<g, 128, 0, st>>>(z, q, drodm, a);
  else if (z.slope == VANALBADA) wall_corr<D, TYP, VANALBADA><<<g, 128, 0, st>>>(z, q, drodm, a);
  else wall_corr<D, TYP, MINMOD><<<g, 128, 0, st>>>(z, q, drodm, a);
}

cudaError_t launch_wall_corr(const Zone& z, const double* q, double* drodm, const WallCorrArgs& a,
                             cudaStream_t st) {
  if (a.n <= 0) return cudaSuccess;
  if (z.kflu != ROE) return cudaErrorNotSupported;
  if (z.typ == Z2D) {
    if (a.dir == 0) wall_corr_sl<0, Z2D>(z, q, drodm, a, st);
    else if (a.dir == 1) wall_corr_sl<1, Z2D>(z, q, drodm, a, st);
    else return cudaErrorNotSupported;
    return cudaGetLastError();
  }
  if (z.typ != Z3DCART && z.typ != Z3DFULL) return cudaErrorNotSupported;
  const bool cart = z.typ == Z3DCART;
  if (a.dir == 0) cart ? wall_corr_sl<0, Z3DCART>(z, q, drodm, a, st) : wall_corr_sl<0, Z3DFULL>(z, q, drodm, a, st);
  else if (a.dir == 1) cart ? wall_corr_sl<1, Z3DCART>(z, q, drodm, a, st) : wall_corr_sl<1, Z3DFULL>(z, q, drodm, a, st);
  else cart ? wall_corr_sl<2, Z3DCART>(z, q, drodm, a, st) : wall_corr_sl<2, Z3DFULL>(z, q, drodm, a, st);
  return cudaGetLastError();
}

// ------------------------------------------------------- shock sensor
// SENSOR/sciacovelli.for + shock_sensor.for: weights of the o3sc slope.
// One thread per cell of the box [1, ni+1] x [1, nj+1] x [1, nk+1]; a cell
// beyond the interior in direction d writes only its d-weight (the faces
// that close the zone, as the reference's loopPlan corrections), and cells
// beyond it in two directions write nothing.  Per cell the velocity
// divergence and squared vorticity from face-averaged velocities
// (SA/div_rot_{3dcart,3dfull,2d}.for) and the face-metric norms tc_d
// (SA/metric_{3dfull,2d}.for), then, per direction,
//   M = (1 - tanh(2.5 + 10 div / (tc_d c))) / 2,
//   J = |p_- - 2 p + p_+| / |p_- + 2 p + p_+|   (p = rho T),
//   wig = 1 - min(2 div^2 / (div^2 + rot + 1e-15) * J * M, 1),
// at wig[l + d*nd + shift], shift = 3*nd for the senseur scheme (its wiggle
// flags hold the first three).
template <int TYP>
__global__ void __launch_bounds__(128) shock_sensor(Zone z, const double* __restrict__ q,
                                                    double* __restrict__ wig) {
  const int64_t NI = z.ni + 1, NJ = z.nj + 1, NK = z.nk + (TYP == Z2D ? 0 : 1);
  const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= NI * NJ * NK) return;
  const int64_t ii = f % NI, r = f / NI, jj = r % NJ, kk = r / NJ;
  const int o0 = ii == z.ni, o1 = jj == z.nj, o2 = (TYP != Z2D) && kk == z.nk;
  if (o0 + o1 + o2 > 1) return;
  const int64_t nd = z.nd, l = inddm(z, ii + 1, jj + 1, kk + 1);
  const int64_t incj = z.inc[1], inck = z.inc[2];
  const int64_t l1 = l + 1, l2 = l - 1, l3 = l + incj, l4 = l - incj, l5 = l + inck, l6 = l - inck;
  double u1[3], u2[3], u3[3], u4[3], u5[3], u6[3];
#pragma unroll
  for (int m = 0; m < (TYP == Z2D ? 2 : 3); m++) {
    const double* Q = q + (m + 1) * nd;
    const double c0 = Q[l];
    u1[m] = c0 + Q[l2]; u2[m] = c0 + Q[l3]; u3[m] = c0 + Q[l1]; u4[m] = c0 + Q[l4];
    if (TYP != Z2D) { u5[m] = c0 + Q[l5]; u6[m] = c0 + Q[l6]; }
  }
  double div, rot, tc[3], dudx, rotx, roty, rotz;
  if (TYP == Z3DCART) {
    const double tix = z.tcx, tjy = z.tcy, tkz = z.tcz, xvol = z.volinv;
    tc[0] = z.si; tc[1] = z.sj; tc[2] = z.sk;
    dudx = (u3[0] - u1[0]) * tix;
    rotz = -(u2[0] - u4[0]) * tjy;
    roty = (u5[0] - u6[0]) * tkz;
    div = dudx * xvol;
    dudx = (u3[1] - u1[1]) * tix;
    rotz = (rotz + dudx) * xvol;
    dudx = (u2[1] - u4[1]) * tjy;
    div = div + dudx * xvol;
    dudx = (u5[1] - u6[1]) * tkz;
    rotx = -dudx;
    dudx = (u3[2] - u1[2]) * tix;
    roty = (roty - dudx) * xvol;
    dudx = (u2[2] - u4[2]) * tjy;
    rotx = (rotx + dudx) * xvol;
    dudx = (u5[2] - u6[2]) * tkz;
    div = div + dudx * xvol;
    rot = rotx * rotx + roty * roty + rotz * rotz;
  } else {
    const int64_t lt = indmtr(z, ii + 1, jj + 1, kk + 1), ndm = z.ndm;
    const double xvol = 0.5 / z.vol[lt];
    const int64_t im = z.minc[0], jm = z.minc[1], km = z.minc[2];
    const double tix = z.ti[lt], tiy = z.ti[lt + ndm], tix1 = z.ti[lt + im], tiy1 = z.ti[lt + im + ndm];
    const double tjx = z.tj[lt], tjy = z.tj[lt + ndm], tjx1 = z.tj[lt + jm], tjy1 = z.tj[lt + jm + ndm];
    if (TYP == Z2D) {
      double t = sqrt(tix * tix + tiy * tiy);
      t = t + sqrt(tix1 * tix1 + tiy1 * tiy1);
      tc[0] = fmaxF(mul_pow2<-1>(t), 1.e-27);
      t = sqrt(tjx * tjx + tjy * tjy);
      t = t + sqrt(tjx1 * tjx1 + tjy1 * tjy1);
      tc[1] = fmaxF(mul_pow2<-1>(t), 1.e-27);
      tc[2] = 1.;
      dudx = u3[0] * tix1 - u1[0] * tix + u2[0] * tjx1 - u4[0] * tjx;
      div = dudx * xvol;
      rotz = -(u3[0] * tiy1 - u1[0] * tiy + u2[0] * tjy1 - u4[0] * tjy);
      dudx = u3[1] * tix1 - u1[1] * tix + u2[1] * tjx1 - u4[1] * tjx;
      rotz = (rotz + dudx) * xvol;
      dudx = u3[1] * tiy1 - u1[1] * tiy + u2[1] * tjy1 - u4[1] * tjy;
      div = div + dudx * xvol;
      rot = rotz * rotz;
    } else {
      const double tiz = z.ti[lt + 2 * ndm], tiz1 = z.ti[lt + im + 2 * ndm];
      const double tjz = z.tj[lt + 2 * ndm], tjz1 = z.tj[lt + jm + 2 * ndm];
      const double tkx = z.tk[lt], tky = z.tk[lt + ndm], tkz = z.tk[lt + 2 * ndm];
      const double tkx1 = z.tk[lt + km], tky1 = z.tk[lt + km + ndm], tkz1 = z.tk[lt + km + 2 * ndm];
      double t = sqrt(tix * tix + tiy * tiy + tiz * tiz);
      t = t + sqrt(tix1 * tix1 + tiy1 * tiy1 + tiz1 * tiz1);
      tc[0] = fmaxF(mul_pow2<-1>(t), 1.e-27);
      t = sqrt(tjx * tjx + tjy * tjy + tjz * tjz);
      t = t + sqrt(tjx1 * tjx1 + tjy1 * tjy1 + tjz1 * tjz1);
      tc[1] = fmaxF(mul_pow2<-1>(t), 1.e-27);
      t = sqrt(tkx * tkx + tky * tky + tkz * tkz);
      t = t + sqrt(tkx1 * tkx1 + tky1 * tky1 + tkz1 * tkz1);
      tc[2] = fmaxF(mul_pow2<-1>(t), 1.e-27);
#define FGB_G(m, x) (u3[m] * ti##x##1 - u1[m] * ti##x + u2[m] * tj##x##1 - u4[m] * tj##x + \
                     u5[m] * tk##x##1 - u6[m] * tk##x)
      dudx = FGB_G(0, x);
      div = dudx * xvol;
      rotz = -FGB_G(0, y);
      roty = FGB_G(0, z);
      dudx = FGB_G(1, x);
      rotz = (rotz + dudx) * xvol;
      dudx = FGB_G(1, y);
      div = div + dudx * xvol;
      dudx = FGB_G(1, z);
      rotx = -dudx;
      dudx = FGB_G(2, x);
      roty = (roty - dudx) * xvol;
      dudx = FGB_G(2, y);
      rotx = (rotx + dudx) * xvol;
      dudx = FGB_G(2, z);
      div = div + dudx * xvol;
#undef FGB_G
      rot = rotx * rotx + roty * roty + rotz * rotz;
    }
  }
  const int64_t shift = z.kflu == SENSEUR ? 3 * nd : 0;
  const int out[3] = {o0, o1, o2};
  // the factors that do not depend on the direction are formed once (same
  // operations, same order: ((10 (1/tc)) (1/c)) div and ((2 div div) / den)
  // J M), and M is reused when tc_d equals the previous direction's (cubic
  // cartesian cells): the FP64 pipe, with tanh the largest part, bounds it
  const double isnd = 1.0 / sqrt(z.gam * z.rgp * q[l + 4 * nd]);
  const double ratio = 2.0 * div * div / (div * div + rot + 1e-15);
  const double p0 = q[l] * q[l + 4 * nd];
  double tc_prev = -1., m_prev = 0.;
#pragma unroll
  for (int d = 0; d < (TYP == Z2D ? 2 : 3); d++) {
    if (out[(d + 1) % 3] || out[(d + 2) % 3]) continue;
    double mach = m_prev;
    if (tc[d] != tc_prev) {
      mach = 10.0 * (1.0 / tc[d]) * isnd * div;
      mach = mul_pow2<-1>(1.0 - tanh(2.5 + mach));
      tc_prev = tc[d];
      m_prev = mach;
    }
    const int64_t n = z.inc[d];
    const double p2 = q[l - n] * q[l - n + 4 * nd];
    const double p1 = q[l + n] * q[l + n + 4 * nd];
    double w = fabs(p2 - mul_pow2<1>(p0) + p1) / fabs(p2 + mul_pow2<1>(p0) + p1);
    w = fminF(ratio * w * mach, 1.0);
    wig[l + d * nd + shift] = 1.0 - w;
  }
}

cudaError_t launch_shock_sensor(const Zone& z, const double* q, double* wig, cudaStream_t st) {
  const int B = 128;
  const int64_t n = (z.ni + 1) * (z.nj + 1) * (z.nk + (z.typ == Z2D ? 0 : 1));
  const unsigned g = (unsigned)((n + B - 1) / B);
  if (z.typ == Z3DCART) shock_sensor<Z3DCART><<<g, B, 0, st>>>(z, q, wig);
  else if (z.typ == Z3DFULL) shock_sensor<Z3DFULL><<<g, B, 0, st>>>(z, q, wig);
  else if (z.typ == Z2D) shock_sensor<Z2D><<<g, B, 0, st>>>(z, q, wig);
  else return cudaErrorNotSupported;
  return cudaGetLastError();
}

// ------------------------------------------------------------ wiggle
// SENSOR/wiggle2001.for + wiggle.for (3-d): flag of the D-face of cell l
// (faces indexed like face_flux, so the last imax+1 / jmax+1 / kmax+1
// planes are included): 1 if, for some variable, both slope products
// (q_{l-1}-q_{l-2})(q_l-q_{l-1}) and (q_l-q_{l-1})(q_{l+1}-q_l) are
// negative (min of sign sums < -1e-12), else 0.
template <int D, bool TWO_D = false>
__global__ void __launch_bounds__(128) wiggle(Zone z, const double* __restrict__ q,
                                              double* __restrict__ wig) {
  const int64_t NI = z.ni + (D == 0), NJ = z.nj + (D == 1), NK = z.nk + (D == 2);
  const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= NI * NJ * NK) return;
  const int64_t ii = f % NI, r = f / NI, jj = r % NJ, kk = r / NJ;
  const int64_t l = inddm(z, ii + 1, jj + 1, kk + 1), inc = z.inc[D], nd = z.nd;
  const int64_t nm = l - inc, nm2 = l - 2 * inc, np = l + inc;
  double test = 0.;
#pragma unroll
  for (int v = 0; v < 5; v++) {
    if (TWO_D && v == 3) continue;   // wiggle2d_{i,j}.for: min(f1, f2, f3, f5)
    const double* Q = q + v * nd;
    const double qm = (Q[nm] - Q[nm2]) * (Q[l] - Q[nm]);
    const double qp = (Q[l] - Q[nm]) * (Q[np] - Q[l]);
    const double fv = fsignF(1., qm) + fsignF(1., qp);
    test = v == 0 ? fv : fminF(test, fv);
  }
  wig[l + D * nd] = test < -1e-12 ? 1. : 0.;
}

cudaError_t launch_wiggle(const Zone& z, const double* q, double* wig, cudaStream_t st) {
  const int B = 128;
  const int64_t nfi = (z.ni + 1) * z.nj * z.nk, nfj = z.ni * (z.nj + 1) * z.nk,
                nfk = z.ni * z.nj * (z.nk + 1);
  if (z.typ == Z2D) {
    wiggle<0, true><<<(unsigned)((nfi + B - 1) / B), B, 0, st>>>(z, q, wig);
    wiggle<1, true><<<(unsigned)((nfj + B - 1) / B), B, 0, st>>>(z, q, wig);
    return cudaGetLastError();
  }
  wiggle<0><<<(unsigned)((nfi + B - 1) / B), B, 0, st>>>(z, q, wig);
  wiggle<1><<<(unsigned)((nfj + B - 1) / B), B, 0, st>>>(z, q, wig);
  wiggle<2><<<(unsigned)((nfk + B - 1) / B), B, 0, st>>>(z, q, wig);
  return cudaGetLastError();
}

cudaError_t launch_assemble(const Zone& z, const StageArgs& a, bool implicit, cudaStream_t st) {
  const int B = 256;
  int64_t n = z.ni * z.nj * z.nk;
  const unsigned g = (unsigned)((n + B - 1) / B);
  if (z.neq == 6) {
    if (implicit) assemble<true, 6><<<g, B, 0, st>>>(z, a);
    else assemble<false, 6><<<g, B, 0, st>>>(z, a);
  } else {
    if (implicit) assemble<true><<<g, B, 0, st>>>(z, a);
    else assemble<false><<<g, B, 0, st>>>(z, a);
  }
  return cudaGetLastError();
}

}  // namespace fgb
