// fgb_adjoint.cu -- tangent and adjoint of the explicit 2-d Euler step
// (Roe + van Albada MUSCL, RK3 low storage, slip-wall / characteristic
// farfield BCs, 1-to-1 copies, corner averages) on sm_103a.
//
// The step is a composition of local maps: one face flux per face, one BC
// formula per ghost cell, one stage update per cell.  Each local map is
// restated here as a template over the scalar type and evaluated with
// forward-mode dual numbers at the linearisation state, which gives its
// exact local Jacobian; the tangent kernels multiply the Jacobian by the
// input perturbations, the adjoint kernels multiply its transpose by the
// output adjoints and scatter-add the result (FP64 atomics) into the adjoint
// of every input: neighbouring cells, face normals (metric), cell volumes
// and the farfield state.  The restated formulas are those of face_flux
// (2-d branch, VANALBADA), bc_face (BCF_SLIP, BCF_FARFIELD with
// non_reflection), bc_next, gather_copy, coins and assemble<false> (2-d
// branch): the derivative is that of the product kernels' arithmetic.
#include "fgb_kernels.cuh"

namespace fgb {

// ------------------------------------------------------------ dual numbers
template <int N>
struct Dual {
  double v;
  double d[N];
  __device__ Dual() {}
  __device__ Dual(double x) : v(x) {
#pragma unroll
    for (int k = 0; k < N; k++) d[k] = 0.;
  }
};
template <int N>
__device__ __forceinline__ Dual<N> var(double x, int k) {
  Dual<N> r(x);
  r.d[k] = 1.;
  return r;
}
#define DUAL_BIN(OP, DV, DA, DB)                                                             \
  template <int N>                                                                          \
  __device__ __forceinline__ Dual<N> operator OP(const Dual<N>& a, const Dual<N>& b) {      \
    Dual<N> r;                                                                              \
    r.v = a.v OP b.v;                                                                       \
    _Pragma("unroll") for (int k = 0; k < N; k++) r.d[k] = DV;                              \
    return r;                                                                               \
  }                                                                                         \
  template <int N>                                                                          \
  __device__ __forceinline__ Dual<N> operator OP(const Dual<N>& a, double b) {              \
    return a OP Dual<N>(b);                                                                 \
  }                                                                                         \
  template <int N>                                                                          \
  __device__ __forceinline__ Dual<N> operator OP(double a, const Dual<N>& b) {              \
    return Dual<N>(a) OP b;                                                                 \
  }
DUAL_BIN(+, a.d[k] + b.d[k], , )
DUAL_BIN(-, a.d[k] - b.d[k], , )
DUAL_BIN(*, a.d[k] * b.v + a.v * b.d[k], , )
#undef DUAL_BIN
// quotient: the value as the primal computes it, the derivatives through one
// reciprocal (N + 1 divisions -> 2)
template <int N>
__device__ __forceinline__ Dual<N> operator/(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r;
  r.v = a.v / b.v;
  const double ib = 1. / b.v;
#pragma unroll
  for (int k = 0; k < N; k++) r.d[k] = (a.d[k] - r.v * b.d[k]) * ib;
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator/(const Dual<N>& a, double b) {
  return a / Dual<N>(b);
}
template <int N>
__device__ __forceinline__ Dual<N> operator/(double a, const Dual<N>& b) {
  return Dual<N>(a) / b;
}
template <int N> __device__ __forceinline__ Dual<N> operator-(const Dual<N>& a) {
  Dual<N> r;
  r.v = -a.v;
#pragma unroll
  for (int k = 0; k < N; k++) r.d[k] = -a.d[k];
  return r;
}
template <int N> __device__ __forceinline__ Dual<N> sqrt(const Dual<N>& a) {
  Dual<N> r;
  r.v = ::sqrt(a.v);
  const double h = 0.5 / r.v;
#pragma unroll
  for (int k = 0; k < N; k++) r.d[k] = a.d[k] * h;
  return r;
}
template <int N> __device__ __forceinline__ Dual<N> fabs(const Dual<N>& a) {
  return a.v < 0. ? -a : a;
}
__device__ __forceinline__ double val(double x) { return x; }
template <int N> __device__ __forceinline__ double val(const Dual<N>& x) { return x.v; }
// Fortran max / min: the selected argument (its derivative)
template <typename T> __device__ __forceinline__ T tmax(const T& a, double b) { return val(a) > b ? a : T(b); }
// SIGN(c, x) with a constant magnitude: piecewise constant
template <typename T> __device__ __forceinline__ double tsign(double c, const T& x) {
  return copysign(::fabs(c), val(x));
}

// Input seeding of a local Jacobian: N > 1 -- input idx is direction idx
// (the whole Jacobian); N == 1 -- only input col is seeded (its column, one
// lane per column)
template <int N>
__device__ __forceinline__ Dual<N> seed(double x, int idx, int col) {
  Dual<N> r(x);
  if (N == 1) {
    if (idx == col) r.d[0] = 1.;
  } else {
    r.d[idx] = 1.;
  }
  return r;
}

// ------------------------------------------------------ restated formulas
template <typename T>
__device__ __forceinline__ T vanalbada_t(const T& x, const T& y) {
  const double e2 = 1e-12;
  return ((y * y + e2) * x + (x * x + e2) * y) / (x * x + y * y + 2. * e2);
}

// gradient of vanalbada_t: va = N / Dn, N = (y^2 + e) x + (x^2 + e) y,
// Dn = x^2 + y^2 + 2e; d va / dx = (y^2 + e + 2xy - 2x va) / Dn and
// symmetrically in y (one reciprocal)
__device__ __forceinline__ void vanalbada_grad(double x, double y, double& gx, double& gy) {
  const double e2 = 1e-12;
  const double xx = x * x, yy = y * y, xy2 = 2. * x * y;
  const double iD = 1. / (xx + yy + 2. * e2);
  const double va = ((yy + e2) * x + (xx + e2) * y) * iD;
  gx = (yy + e2 + xy2 - 2. * x * va) * iD;
  gy = (xx + e2 + xy2 - 2. * y * va) * iD;
}

// the same gradient given va and iD = 1 / Dn (from the face tape)
__device__ __forceinline__ void vanalbada_grad_v(double x, double y, double va, double iD, double& gx,
                                                 double& gy) {
  const double e2 = 1e-12;
  const double xx = x * x, yy = y * y, xy2 = 2. * x * y;
  gx = (yy + e2 + xy2 - 2. * x * va) * iD;
  gy = (xx + e2 + xy2 - 2. * y * va) * iD;
}

// roe_full (fgb_flux.cu) for a 2-d face: tcz = 0, w = 0 (those terms vanish
// exactly in the primal), s = |(tcx, tcy)|; F[3] = 0
template <typename T>
__device__ __forceinline__ void roe2d(const Zone& z, const T qm[5], const T qp[5], const T& tcx,
                                      const T& tcy, T F[5]) {
  const double rgp = z.rgp, gam1 = z.gam1;
  const T s = sqrt(tcx * tcx + tcy * tcy);
  T r1 = qp[0], p1 = r1 * qp[4] * rgp;
  T h1 = gam1 * qp[4] * rgp + .5 * (qp[1] * qp[1] + qp[2] * qp[2]);
  T r2 = qm[0], p2 = r2 * qm[4] * rgp;
  T h2 = gam1 * qm[4] * rgp + .5 * (qm[1] * qm[1] + qm[2] * qm[2]);
  T s1 = sqrt(r1), s2 = sqrt(r2);
  T r = s1 * s2, r_1 = 1. / (s1 + s2);
  T u = (s1 * qp[1] + s2 * qm[1]) * r_1;
  T v = (s1 * qp[2] + s2 * qm[2]) * r_1;
  T h = (s1 * h1 + s2 * h2) * r_1;
  T q = .5 * (u * u + v * v);
  T c = sqrt((z.gam - 1.) * fabs(h - q));
  T qn1 = qp[1] * tcx + qp[2] * tcy;
  T qn2 = qm[1] * tcx + qm[2] * tcy;
  T du = (qm[1] - qp[1]) * s, dv = (qm[2] - qp[2]) * s;
  T dp = p2 - p1, dqn = qn2 - qn1;
  T s_1 = 1.0 / tmax(s, 1.E-30);
  T nx = tcx * s_1, ny = tcy * s_1;
  T qn = u * nx + v * ny;
  T f1 = qn;
  T f4 = z.psiroe * (fabs(f1) + c);
  double f2 = 0.5 + tsign(0.5, fabs(f1) - f4);
  T f3 = (f2 - 1.0) * (f1 * f1 / f4 + f4) * 0.5 - f2 * fabs(f1);
  f1 = (r2 - r1 - dp / (c * c)) * s;
  T fl1 = f3 * (f1);
  T fl2 = f3 * (f1 * u + r * (du - nx * dqn));
  T fl3 = f3 * (f1 * v + r * (dv - ny * dqn));
  T fl5 = f3 * (f1 * q + r * (u * du + v * dv - qn * dqn));
  f1 = qn + c;
  f2 = 0.5 + tsign(0.5, fabs(f1) - f4);
  f3 = (f2 - 1.) * (f1 * f1 / f4 + f4) * 0.5 - f2 * fabs(f1);
  f1 = (dp + r * c * dqn * s_1) / (2. * c * c) * s * f3;
  fl1 = fl1 + f1;
  fl2 = fl2 + f1 * (u + nx * c);
  fl3 = fl3 + f1 * (v + ny * c);
  fl5 = fl5 + f1 * (h + qn * c);
  f1 = qn - c;
  f2 = 0.5 + tsign(0.5, fabs(f1) - f4);
  f3 = (f2 - 1.) * (f1 * f1 / f4 + f4) * 0.5 - f2 * fabs(f1);
  f1 = (dp - r * c * dqn * s_1) / (2. * c * c) * f3 * s;
  fl1 = fl1 + f1;
  fl2 = fl2 + f1 * (u - nx * c);
  fl3 = fl3 + f1 * (v - ny * c);
  fl5 = fl5 + f1 * (h - qn * c);
  T rou1 = r1 * qn1, rou2 = r2 * qn2, p1p2 = p1 + p2;
  F[0] = (fl1 + rou1 + rou2) * 0.5;
  F[1] = (fl2 + rou1 * qp[1] + rou2 * qm[1] + tcx * p1p2) * 0.5;
  F[2] = (fl3 + rou1 * qp[2] + rou2 * qm[2] + tcy * p1p2) * 0.5;
  F[3] = T(0.);
  F[4] = (fl5 + rou1 * h1 + rou2 * h2) * 0.5;
}

// Reverse mode of roe2d, written out: given the output adjoints Fb (F[3]
// unused), adds d(Fb . F)/d(input) to qmb, qpb (variables 0, 1, 2, 4) and
// tb[0..1] (tcx, tcy).  Forward pass with every intermediate kept, then the
// chain rule in reverse order; |x| and the entropy-fix switches take the
// derivative of the branch the value selects (the dual numbers' rule).
__device__ __forceinline__ double sgn1(double x) { return x < 0. ? -1. : 1.; }

// TAPED: the square roots and quotients of the forward pass come from the
// face tape of the recomputation (roe_full<true>: tp[k * ts], k = 0..8)
template <bool TAPED>
__device__ void roe2d_rev(const Zone& z, const double qm[5], const double qp[5], double tcx,
                          double tcy, const double Fb[5], double qmb[5], double qpb[5], double tb[2],
                          const double* tp = nullptr, int64_t ts = 0) {
  const double rgp = z.rgp, gam1 = z.gam1, g_ = z.gam - 1., psi = z.psiroe;
  // ---- forward
  const double ss = tcx * tcx + tcy * tcy, s = TAPED ? tp[0] : ::sqrt(ss);
  const double r1 = qp[0], p1 = r1 * qp[4] * rgp;
  const double h1 = gam1 * qp[4] * rgp + .5 * (qp[1] * qp[1] + qp[2] * qp[2]);
  const double r2 = qm[0], p2 = r2 * qm[4] * rgp;
  const double h2 = gam1 * qm[4] * rgp + .5 * (qm[1] * qm[1] + qm[2] * qm[2]);
  const double s1 = TAPED ? tp[ts] : ::sqrt(r1), s2 = TAPED ? tp[2 * ts] : ::sqrt(r2);
  const double r = s1 * s2, r_1 = TAPED ? tp[3 * ts] : 1. / (s1 + s2);
  const double i_r = TAPED ? tp[8 * ts] : 1. / r;
  const double t7u = s1 * qp[1] + s2 * qm[1], t7v = s1 * qp[2] + s2 * qm[2];
  const double u = t7u * r_1, v = t7v * r_1;
  const double t8 = s1 * h1 + s2 * h2, h = t8 * r_1;
  const double q = .5 * (u * u + v * v);
  const double hq = h - q, c = TAPED ? tp[4 * ts] : ::sqrt(g_ * ::fabs(hq));
  const double qn1 = qp[1] * tcx + qp[2] * tcy, qn2 = qm[1] * tcx + qm[2] * tcy;
  const double du = (qm[1] - qp[1]) * s, dv = (qm[2] - qp[2]) * s;
  const double dp = p2 - p1, dqn = qn2 - qn1;
  const bool smax_on = s > 1.E-30;
  const double s_1 = TAPED ? tp[5 * ts] : 1.0 / (smax_on ? s : 1.E-30);
  const double nx = tcx * s_1, ny = tcy * s_1;
  const double qn = u * nx + v * ny;
  const double A1 = ::fabs(qn), f4 = psi * (A1 + c), i_f4 = TAPED ? tp[6 * ts] : 1. / f4;
  const double f2a = 0.5 + copysign(0.5, A1 - f4);
  const double f3a = (f2a - 1.0) * (qn * qn * i_f4 + f4) * 0.5 - f2a * A1;
  const double c2 = c * c, i_c2 = TAPED ? tp[7 * ts] : 1. / c2;
  const double Z = r2 - r1 - dp * i_c2, f1a = Z * s;
  const double X2 = f1a * u + r * (du - nx * dqn), X3 = f1a * v + r * (dv - ny * dqn);
  const double Y5 = u * du + v * dv - qn * dqn, X5 = f1a * q + r * Y5;
  const double l4 = qn + c, A4 = ::fabs(l4);
  const double f2b = 0.5 + copysign(0.5, A4 - f4);
  const double f3b = (f2b - 1.) * (l4 * l4 * i_f4 + f4) * 0.5 - f2b * A4;
  const double N4 = dp + r * c * dqn * s_1, K4 = N4 * 0.5 * i_c2, f1b = K4 * s * f3b;
  const double l5 = qn - c, A5 = ::fabs(l5);
  const double f2c = 0.5 + copysign(0.5, A5 - f4);
  const double f3c = (f2c - 1.) * (l5 * l5 * i_f4 + f4) * 0.5 - f2c * A5;
  const double N5 = dp - r * c * dqn * s_1, K5 = N5 * 0.5 * i_c2, f1c = K5 * f3c * s;
  const double rou1 = r1 * qn1, rou2 = r2 * qn2, p1p2 = p1 + p2;
  // ---- reverse
  double r1b = 0., r2b = 0., qn1b = 0., qn2b = 0., p1b = 0., p2b = 0., h1b = 0., h2b = 0.;
  double ub = 0., vb = 0., hb = 0., qb = 0., cb = 0., rb = 0., nxb = 0., nyb = 0., qnb = 0.;
  double dub = 0., dvb = 0., dpb = 0., dqnb = 0., sb = 0., s_1b = 0., f4b = 0., c2b = 0.;
  double tcxb = 0., tcyb = 0.;
  const double b0 = 0.5 * Fb[0], b1 = 0.5 * Fb[1], b2 = 0.5 * Fb[2], b4 = 0.5 * Fb[4];
  const double fl1b = b0, fl2b = b1, fl3b = b2, fl5b = b4;
  const double rou1b = b0 + b1 * qp[1] + b2 * qp[2] + b4 * h1;
  const double rou2b = b0 + b1 * qm[1] + b2 * qm[2] + b4 * h2;
  qpb[1] += b1 * rou1; qmb[1] += b1 * rou2; qpb[2] += b2 * rou1; qmb[2] += b2 * rou2;
  tcxb += b1 * p1p2; tcyb += b2 * p1p2;
  const double p1p2b = b1 * tcx + b2 * tcy;
  h1b += b4 * rou1; h2b += b4 * rou2;
  r1b += rou1b * qn1; qn1b += rou1b * r1; r2b += rou2b * qn2; qn2b += rou2b * r2;
  p1b += p1p2b; p2b += p1p2b;
  // wave 5 (qn - c)
  {
    const double f1cb = fl1b + fl2b * (u - nx * c) + fl3b * (v - ny * c) + fl5b * (h - qn * c);
    ub += fl2b * f1c; nxb -= fl2b * f1c * c; cb -= fl2b * f1c * nx;
    vb += fl3b * f1c; nyb -= fl3b * f1c * c; cb -= fl3b * f1c * ny;
    hb += fl5b * f1c; qnb -= fl5b * f1c * c; cb -= fl5b * f1c * qn;
    const double K5b = f1cb * f3c * s, f3cb = f1cb * K5 * s;
    sb += f1cb * K5 * f3c;
    const double N5b = K5b * 0.5 * i_c2;
    c2b -= K5b * K5 * i_c2;
    dpb += N5b; rb -= N5b * c * dqn * s_1; cb -= N5b * r * dqn * s_1;
    dqnb -= N5b * r * c * s_1; s_1b -= N5b * r * c * dqn;
    double l5b = f3cb * (f2c - 1.) * l5 * i_f4;
    f4b += f3cb * (f2c - 1.) * 0.5 * (1. - l5 * l5 * i_f4 * i_f4);
    l5b += -f3cb * f2c * sgn1(l5);
    qnb += l5b; cb -= l5b;
  }
  // wave 4 (qn + c)
  {
    const double f1bb = fl1b + fl2b * (u + nx * c) + fl3b * (v + ny * c) + fl5b * (h + qn * c);
    ub += fl2b * f1b; nxb += fl2b * f1b * c; cb += fl2b * f1b * nx;
    vb += fl3b * f1b; nyb += fl3b * f1b * c; cb += fl3b * f1b * ny;
    hb += fl5b * f1b; qnb += fl5b * f1b * c; cb += fl5b * f1b * qn;
    const double K4b = f1bb * s * f3b, f3bb = f1bb * K4 * s;
    sb += f1bb * K4 * f3b;
    const double N4b = K4b * 0.5 * i_c2;
    c2b -= K4b * K4 * i_c2;
    dpb += N4b; rb += N4b * c * dqn * s_1; cb += N4b * r * dqn * s_1;
    dqnb += N4b * r * c * s_1; s_1b += N4b * r * c * dqn;
    double l4b = f3bb * (f2b - 1.) * l4 * i_f4;
    f4b += f3bb * (f2b - 1.) * 0.5 * (1. - l4 * l4 * i_f4 * i_f4);
    l4b += -f3bb * f2b * sgn1(l4);
    qnb += l4b; cb += l4b;
  }
  // wave 1 (qn)
  {
    const double f3ab = fl1b * f1a + fl2b * X2 + fl3b * X3 + fl5b * X5;
    double f1ab = fl1b * f3a;
    const double X2b = fl2b * f3a, X3b = fl3b * f3a, X5b = fl5b * f3a;
    f1ab += X2b * u; ub += X2b * f1a; rb += X2b * (du - nx * dqn); dub += X2b * r;
    nxb -= X2b * r * dqn; dqnb -= X2b * r * nx;
    f1ab += X3b * v; vb += X3b * f1a; rb += X3b * (dv - ny * dqn); dvb += X3b * r;
    nyb -= X3b * r * dqn; dqnb -= X3b * r * ny;
    f1ab += X5b * q; qb += X5b * f1a; rb += X5b * Y5;
    ub += X5b * r * du; dub += X5b * r * u; vb += X5b * r * dv; dvb += X5b * r * v;
    qnb -= X5b * r * dqn; dqnb -= X5b * r * qn;
    const double Zb = f1ab * s;
    sb += f1ab * Z;
    r2b += Zb; r1b -= Zb; dpb -= Zb * i_c2; c2b += Zb * dp * i_c2 * i_c2;
    qnb += f3ab * (f2a - 1.) * qn * i_f4;
    f4b += f3ab * (f2a - 1.) * 0.5 * (1. - qn * qn * i_f4 * i_f4);
    const double A1b = -f3ab * f2a + f4b * psi;
    cb += f4b * psi;
    qnb += A1b * sgn1(qn);
  }
  cb += 2. * c * c2b;
  ub += qnb * nx; nxb += qnb * u; vb += qnb * ny; nyb += qnb * v;
  tcxb += nxb * s_1; s_1b += nxb * tcx; tcyb += nyb * s_1; s_1b += nyb * tcy;
  if (smax_on) sb += -s_1b * s_1 * s_1;
  p2b += dpb; p1b -= dpb; qn2b += dqnb; qn1b -= dqnb;
  qmb[1] += dub * s; qpb[1] -= dub * s; sb += dub * (qm[1] - qp[1]);
  qmb[2] += dvb * s; qpb[2] -= dvb * s; sb += dvb * (qm[2] - qp[2]);
  qpb[1] += qn1b * tcx; tcxb += qn1b * qp[1]; qpb[2] += qn1b * tcy; tcyb += qn1b * qp[2];
  qmb[1] += qn2b * tcx; tcxb += qn2b * qm[1]; qmb[2] += qn2b * tcy; tcyb += qn2b * qm[2];
  {
    const double gb = cb * 0.5 * c * i_c2;   // d / d(g_ |hq|) = cb / (2c)
    const double hqb = gb * g_ * sgn1(hq);
    hb += hqb; qb -= hqb;
  }
  ub += qb * u; vb += qb * v;
  const double t8b = hb * r_1;
  double r_1b = hb * t8;
  double s1b = t8b * h1, s2b = t8b * h2;
  h1b += t8b * s1; h2b += t8b * s2;
  const double t7ub = ub * r_1, t7vb = vb * r_1;
  r_1b += ub * t7u + vb * t7v;
  s1b += t7ub * qp[1] + t7vb * qp[2]; s2b += t7ub * qm[1] + t7vb * qm[2];
  qpb[1] += t7ub * s1; qmb[1] += t7ub * s2; qpb[2] += t7vb * s1; qmb[2] += t7vb * s2;
  s1b += rb * s2; s2b += rb * s1;
  const double denb = -r_1b * r_1 * r_1;
  s1b += denb; s2b += denb;
  r1b += s1b * 0.5 * s2 * i_r; r2b += s2b * 0.5 * s1 * i_r;   // 1 / s1 = s2 / r
  qmb[4] += h2b * gam1 * rgp; qmb[1] += h2b * qm[1]; qmb[2] += h2b * qm[2];
  r2b += p2b * qm[4] * rgp; qmb[4] += p2b * r2 * rgp;
  qpb[4] += h1b * gam1 * rgp; qpb[1] += h1b * qp[1]; qpb[2] += h1b * qp[2];
  r1b += p1b * qp[4] * rgp; qpb[4] += p1b * r1 * rgp;
  qpb[0] += r1b; qmb[0] += r2b;
  const double ssb = sb * 0.5 * s_1;
  tcxb += 2. * tcx * ssb; tcyb += 2. * tcy * ssb;
  tb[0] += tcxb; tb[1] += tcyb;
}

// adjoint of one face: mu = d J / d F (per component) -> cells and normal.
// The reconstructed states first (values only), the reverse Roe pass, then
// per variable the reconstruction derivatives (vanalbada_grad, recomputed:
// they are not live across the Roe pass) and the scatter.
// TAPED: the slopes and their reciprocal denominators, and the Roe values,
// from the face tape (face-major, stride ts) instead of recomputed
template <int D, bool TAPED = false>
__device__ __forceinline__ void face_adjoint(const Zone& z, const double* __restrict__ q,
                                             int64_t l, int64_t lt, const double mu[5],
                                             double* __restrict__ lamQ, double* __restrict__ lamT,
                                             const double* __restrict__ tp = nullptr, int64_t ts = 0) {
  const int64_t inc = z.inc[D], nd = z.nd;
  double qm[5], qp[5];
#pragma unroll
  for (int v = 0; v < 5; v++) {
    if (v == 3) { qm[v] = 0.; qp[v] = 0.; continue; }
    const double* Q = q + v * nd;
    const double a = Q[l - 2 * inc], b = Q[l - inc], c = Q[l], d = Q[l + inc];
    const int m = v == 4 ? 3 : v;
    qm[v] = c - 0.5 * (TAPED ? tp[(TAPE_VA + 2 * m) * ts] : vanalbada_t(c - b, d - c));
    qp[v] = b + 0.5 * (TAPED ? tp[(TAPE_VA + 2 * m + 1) * ts] : vanalbada_t(b - a, c - b));
  }
  const double* M = D == 0 ? z.ti : z.tj;
  double qmb[5] = {0, 0, 0, 0, 0}, qpb[5] = {0, 0, 0, 0, 0}, tb[2] = {0, 0};
  roe2d_rev<TAPED>(z, qm, qp, M[lt], M[lt + z.ndm], mu, qmb, qpb, tb, tp, ts);
#pragma unroll
  for (int m = 0; m < 4; m++) {
    const int v = m == 3 ? 4 : m;
    const double* Q = q + v * nd;
    const double a = Q[l - 2 * inc], b = Q[l - inc], c = Q[l], d = Q[l + inc];
    // qm = c - va(c - b, d - c) / 2, qp = b + va(b - a, c - b) / 2
    double mx, my, px, py;
    if (TAPED) {
      vanalbada_grad_v(c - b, d - c, tp[(TAPE_VA + 2 * m) * ts], tp[(TAPE_ID + 2 * m) * ts], mx, my);
      vanalbada_grad_v(b - a, c - b, tp[(TAPE_VA + 2 * m + 1) * ts], tp[(TAPE_ID + 2 * m + 1) * ts], px, py);
    } else {
      vanalbada_grad(c - b, d - c, mx, my);
      vanalbada_grad(b - a, c - b, px, py);
    }
    const int64_t o = v * nd;
    const double gm = qmb[v], gp = qpb[v];
    atomicAdd(lamQ + l - 2 * inc + o, -0.5 * px * gp);
    atomicAdd(lamQ + l - inc + o, 0.5 * mx * gm + (1. + 0.5 * (px - py)) * gp);
    atomicAdd(lamQ + l + o, (1. - 0.5 * (mx - my)) * gm + 0.5 * py * gp);
    atomicAdd(lamQ + l + inc + o, -0.5 * my * gm);
  }
  atomicAdd(lamT + lt, tb[0]);
  atomicAdd(lamT + lt + z.ndm, tb[1]);
}

// the four primitive variables of a 2-d state (w = 0 throughout)
__device__ __constant__ const int V4[4] = {0, 1, 2, 4};

// ---------------------------------------------------------------- faces
// Face of direction D of cell l (2-d: D = 0, 1): F(qm, qp, t) with
// qm = c - va(c - b, d - c) / 2, qp = b + va(b - a, c - b) / 2 per variable
// (a, b, c, d = cells l - 2 inc, l - inc, l, l + inc).  The Roe Jacobian is
// taken over (qm, qp, tcx, tcy) (10 duals), the reconstruction's over its
// three cells per variable (3 duals).
struct FaceLin {
  double JF[5][10];    // dF_v / d(qm[0..3], qp[0..3], tcx, tcy)
  double gm[4][3];     // d qm_v / d(b, c, d)
  double gp[4][3];     // d qp_v / d(a, b, c)
};

template <int D>
__device__ __forceinline__ void face_lin(const Zone& z, const double* __restrict__ q, int64_t l,
                                         int64_t lt, FaceLin& L) {
  const int64_t inc = z.inc[D], nd = z.nd;
  Dual<10> qm[5], qp[5];
#pragma unroll
  for (int m = 0; m < 4; m++) {
    const double* Q = q + V4[m] * nd;
    const double a = Q[l - 2 * inc], b = Q[l - inc], c = Q[l], d = Q[l + inc];
    {
      Dual<3> B = var<3>(b, 0), C = var<3>(c, 1), Dd = var<3>(d, 2);
      Dual<3> r = C - 0.5 * vanalbada_t(C - B, Dd - C);
      qm[V4[m]] = var<10>(r.v, m);
#pragma unroll
      for (int k = 0; k < 3; k++) L.gm[m][k] = r.d[k];
    }
    {
      Dual<3> A = var<3>(a, 0), B = var<3>(b, 1), C = var<3>(c, 2);
      Dual<3> r = B + 0.5 * vanalbada_t(B - A, C - B);
      qp[V4[m]] = var<10>(r.v, 4 + m);
#pragma unroll
      for (int k = 0; k < 3; k++) L.gp[m][k] = r.d[k];
    }
  }
  qm[3] = Dual<10>(0.);
  qp[3] = Dual<10>(0.);
  const double* M = D == 0 ? z.ti : z.tj;
  Dual<10> tcx = var<10>(M[lt], 8), tcy = var<10>(M[lt + z.ndm], 9);
  Dual<10> F[5];
  roe2d(z, qm, qp, tcx, tcy, F);
#pragma unroll
  for (int v = 0; v < 5; v++)
#pragma unroll
    for (int k = 0; k < 10; k++) L.JF[v][k] = F[v].d[k];
}

// adjoint: mu = lamD(l) [l interior] - lamD(l - inc) [l - inc interior]
// (register-bounded to 3 blocks of 128 per SM: faster than the unbounded
// 255-register build, measured on GB300)
template <int D, bool TAPED>
__global__ void __launch_bounds__(128, 3) adj_faces(Zone z, const double* __restrict__ q,
                                                 const double* __restrict__ tape,
                                                 const double* __restrict__ lamD,
                                                 double* __restrict__ lamQ,
                                                 double* __restrict__ lamT) {
  const int64_t NI = z.ni + (D == 0), NJ = z.nj + (D == 1);
  const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= NI * NJ) return;
  const int64_t ii = f % NI, jj = f / NI;
  const int64_t l = inddm(z, ii + 1, jj + 1, 1), lt = indmtr(z, ii + 1, jj + 1, 1);
  const int64_t inc = z.inc[D], nd = z.nd;
  const int64_t idx = D == 0 ? ii : jj, n = D == 0 ? z.ni : z.nj;
  const bool hi_in = idx < n, lo_in = idx >= 1;
  double mu[5];
#pragma unroll
  for (int v = 0; v < 5; v++)
    mu[v] = (hi_in ? lamD[l + v * nd] : 0.) - (lo_in ? lamD[l - inc + v * nd] : 0.);
  face_adjoint<D, TAPED>(z, q, l, lt, mu, lamQ, lamT, TAPED ? tape + f : nullptr, NI * NJ);
}

// tangent: dF = J (dq, dt) into the face array (SoA, 5 x faces)
template <int D>
__global__ void __launch_bounds__(128) tan_faces(Zone z, const double* __restrict__ q,
                                                 const double* __restrict__ dq,
                                                 const double* __restrict__ dT,
                                                 double* __restrict__ dF) {
  const int64_t NI = z.ni + (D == 0), NJ = z.nj + (D == 1);
  const int64_t nf = NI * NJ;
  const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  const int64_t ii = f % NI, jj = f / NI;
  const int64_t l = inddm(z, ii + 1, jj + 1, 1), lt = indmtr(z, ii + 1, jj + 1, 1);
  const int64_t inc = z.inc[D], nd = z.nd;
  FaceLin L;
  face_lin<D>(z, q, l, lt, L);
  double din[10];
#pragma unroll
  for (int m = 0; m < 4; m++) {
    const double* Q = dq + V4[m] * nd;
    const double a = Q[l - 2 * inc], b = Q[l - inc], c = Q[l], d = Q[l + inc];
    din[m] = L.gm[m][0] * b + L.gm[m][1] * c + L.gm[m][2] * d;
    din[4 + m] = L.gp[m][0] * a + L.gp[m][1] * b + L.gp[m][2] * c;
  }
  din[8] = dT[lt];
  din[9] = dT[lt + z.ndm];
#pragma unroll
  for (int v = 0; v < 5; v++) {
    double s = 0.;
#pragma unroll
    for (int k = 0; k < 10; k++) s += L.JF[v][k] * din[k];
    dF[v * nf + f] = s;
  }
}

cudaError_t launch_adj_faces(const Zone& z, const double* q, const double* tape,
                             const double* lamD, double* lamQ,
                             double* lamTi, double* lamTj, cudaStream_t st) {
  if (z.typ != Z2D) return cudaErrorNotSupported;
  const int B = 128;
  const int64_t nfi = (z.ni + 1) * z.nj, nfj = z.ni * (z.nj + 1);
  const unsigned gi = (unsigned)((nfi + B - 1) / B), gj = (unsigned)((nfj + B - 1) / B);
  if (tape) {
    adj_faces<0, true><<<gi, B, 0, st>>>(z, q, tape, lamD, lamQ, lamTi);
    adj_faces<1, true><<<gj, B, 0, st>>>(z, q, tape + FACE_TAPE * nfi, lamD, lamQ, lamTj);
  } else {
    adj_faces<0, false><<<gi, B, 0, st>>>(z, q, nullptr, lamD, lamQ, lamTi);
    adj_faces<1, false><<<gj, B, 0, st>>>(z, q, nullptr, lamD, lamQ, lamTj);
  }
  return cudaGetLastError();
}

cudaError_t launch_tan_faces(const Zone& z, const double* q, const double* dq, const double* dTi,
                             const double* dTj, double* dFi, double* dFj, cudaStream_t st) {
  if (z.typ != Z2D) return cudaErrorNotSupported;
  const int B = 128;
  const int64_t nfi = (z.ni + 1) * z.nj, nfj = z.ni * (z.nj + 1);
  tan_faces<0><<<(unsigned)((nfi + B - 1) / B), B, 0, st>>>(z, q, dq, dTi, dFi);
  tan_faces<1><<<(unsigned)((nfj + B - 1) / B), B, 0, st>>>(z, q, dq, dTj, dFj);
  return cudaGetLastError();
}

// --------------------------------------------------------- stage update
// assemble<false> 2-d branch (core3ark3.for): W_out = prim(cons(W_in) +
// coefW dtc / vol D); Jacobian over (ro, u, v, T of W_in; D0, D1, D2, D4;
// vol) = 9 duals, outputs ro, u, v, T of W_out (w stays 0).
__device__ __forceinline__ void update_lin(const Zone& z, const double* __restrict__ q,
                                           const double* __restrict__ D, int64_t l, int64_t lt,
                                           double coefW, double J[4][9]) {
  const int64_t nd = z.nd;
  Dual<9> ro = var<9>(q[l], 0), u = var<9>(q[l + nd], 1), v = var<9>(q[l + 2 * nd], 2),
          tt = var<9>(q[l + 4 * nd], 3);
  Dual<9> x0 = var<9>(D[l], 4), x1 = var<9>(D[l + nd], 5), x2 = var<9>(D[l + 2 * nd], 6),
          x4 = var<9>(D[l + 4 * nd], 7);
  Dual<9> vol = var<9>(z.vol[lt], 8);
  const double cv = z.cv;
  Dual<9> coe = z.dtc / vol;   // tstb3_global.for
  Dual<9> r_1 = coefW * coe;
  Dual<9> tab1 = x0 * r_1, tab2 = x1 * r_1, tab3 = x2 * r_1, tab5 = x4 * r_1;
  Dual<9> n1 = ro + tab1;
  Dual<9> rr = 1. / n1;
  Dual<9> n2 = (ro * u + tab2) * rr;
  Dual<9> n3 = (ro * v + tab3) * rr;
  const double cvinv = 1. / cv, cvinv2 = 0.5 * cvinv;
  Dual<9> roe_old = ro * (cv * tt + 0.5 * (u * u + v * v));
  Dual<9> n5 = (roe_old + tab5) * rr * cvinv - cvinv2 * (n2 * n2 + n3 * n3);
  const Dual<9>* o[4] = {&n1, &n2, &n3, &n5};
#pragma unroll
  for (int m = 0; m < 4; m++)
#pragma unroll
    for (int k = 0; k < 9; k++) J[m][k] = o[m]->d[k];
}

// adjoint of one stage update: lamIn += J_W^T lamOut, lamD += J_D^T lamOut,
// lamVol += J_vol^T lamOut; lamOut (interior) is consumed (zeroed)
__global__ void __launch_bounds__(128) adj_update(Zone z, const double* __restrict__ q,
                                                  const double* __restrict__ D, double coefW,
                                                  double* __restrict__ lamOut,
                                                  double* __restrict__ lamIn,
                                                  double* __restrict__ lamD,
                                                  double* __restrict__ lamVol) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= z.ni * z.nj) return;
  const int64_t ii = t % z.ni, jj = t / z.ni;
  const int64_t l = inddm(z, ii + 1, jj + 1, 1), lt = indmtr(z, ii + 1, jj + 1, 1), nd = z.nd;
  double lo[4];
#pragma unroll
  for (int m = 0; m < 4; m++) { lo[m] = lamOut[l + V4[m] * nd]; lamOut[l + V4[m] * nd] = 0.; }
  lamOut[l + 3 * nd] = 0.;
  // forward values of update_lin's formula, then its reverse pass
  const double ro = q[l], u = q[l + nd], v = q[l + 2 * nd], tt = q[l + 4 * nd];
  const double x0 = D[l], x1 = D[l + nd], x2 = D[l + 2 * nd], x4 = D[l + 4 * nd];
  const double vol = z.vol[lt], cv = z.cv, cvinv = 1. / cv;
  const double r_1 = coefW * (z.dtc / vol);
  const double n1 = ro + x0 * r_1, rr = 1. / n1;
  const double B2 = ro * u + x1 * r_1, B3 = ro * v + x2 * r_1;
  const double n2 = B2 * rr, n3 = B3 * rr;
  const double E = cv * tt + 0.5 * (u * u + v * v), A5 = ro * E + x4 * r_1;
  // n5 = A5 rr / cv - (n2^2 + n3^2) / (2 cv)
  const double A5b = lo[3] * rr * cvinv;
  const double n2b = lo[1] - lo[3] * cvinv * n2, n3b = lo[2] - lo[3] * cvinv * n3;
  const double B2b = n2b * rr, B3b = n3b * rr;
  const double rrb = lo[3] * A5 * cvinv + n2b * B2 + n3b * B3;
  const double n1b = lo[0] - rrb * rr * rr;
  const double g[9] = {n1b + B2b * u + B3b * v + A5b * E, (B2b + A5b * u) * ro,
                       (B3b + A5b * v) * ro, A5b * ro * cv,
                       n1b * r_1, B2b * r_1, B3b * r_1, A5b * r_1,
                       -(n1b * x0 + B2b * x1 + B3b * x2 + A5b * x4) * r_1 / vol};
#pragma unroll
  for (int m = 0; m < 4; m++) {
    lamIn[l + V4[m] * nd] += g[m];       // one thread per cell: no race
    lamD[l + V4[m] * nd] += g[4 + m];
  }
  atomicAdd(lamVol + lt, g[8]);
}

// tangent of one stage's balance: dD = (zero ? 0 : coefH dD) + sum of the
// face tangents (the wall-face corrections are added after it)
__global__ void __launch_bounds__(128) tan_balance(Zone z, double coefH, int zero,
                                                   const double* __restrict__ dFi,
                                                   const double* __restrict__ dFj,
                                                   double* __restrict__ dD) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= z.ni * z.nj) return;
  const int64_t ii = t % z.ni, jj = t / z.ni;
  const int64_t l = inddm(z, ii + 1, jj + 1, 1), nd = z.nd;
  const int64_t nfi = (z.ni + 1) * z.nj, nfj = z.ni * (z.nj + 1);
  const int64_t ai = ii + (z.ni + 1) * jj, aj = ii + z.ni * jj;
#pragma unroll
  for (int v = 0; v < 5; v++) {
    double s = zero ? 0. : dD[l + v * nd] * coefH;
    s = s + dFj[v * nfj + aj] + dFi[v * nfi + ai] - dFi[v * nfi + ai + 1] - dFj[v * nfj + aj + z.ni];
    dD[l + v * nd] = s;
  }
}

// tangent of one stage's update: dOut = J (dIn, dD, dvol)
__global__ void __launch_bounds__(128) tan_apply(Zone z, const double* __restrict__ q,
                                                 const double* __restrict__ D, double coefW,
                                                 const double* __restrict__ dIn,
                                                 const double* __restrict__ dD,
                                                 const double* __restrict__ dVol,
                                                 double* __restrict__ dOut) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= z.ni * z.nj) return;
  const int64_t ii = t % z.ni, jj = t / z.ni;
  const int64_t l = inddm(z, ii + 1, jj + 1, 1), lt = indmtr(z, ii + 1, jj + 1, 1), nd = z.nd;
  double J[4][9];
  update_lin(z, q, D, l, lt, coefW, J);
  const double din[9] = {dIn[l], dIn[l + nd], dIn[l + 2 * nd], dIn[l + 4 * nd],
                         dD[l], dD[l + nd], dD[l + 2 * nd], dD[l + 4 * nd], dVol[lt]};
#pragma unroll
  for (int m = 0; m < 4; m++) {
    double s = 0.;
#pragma unroll
    for (int k = 0; k < 9; k++) s += J[m][k] * din[k];
    dOut[l + V4[m] * nd] = s;
  }
  dOut[l + 3 * nd] = 0.;
}

cudaError_t launch_adj_update(const Zone& z, const double* q, const double* D, double coefW,
                              double* lamOut, double* lamIn, double* lamD, double* lamVol,
                              cudaStream_t st) {
  const int64_t n = z.ni * z.nj;
  adj_update<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(z, q, D, coefW, lamOut, lamIn, lamD, lamVol);
  return cudaGetLastError();
}

cudaError_t launch_tan_balance(const Zone& z, double coefH, int zero, const double* dFi,
                               const double* dFj, double* dD, cudaStream_t st) {
  const int64_t n = z.ni * z.nj;
  tan_balance<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(z, coefH, zero, dFi, dFj, dD);
  return cudaGetLastError();
}

cudaError_t launch_tan_apply(const Zone& z, const double* q, const double* D, double coefW,
                             const double* dIn, const double* dD, const double* dVol, double* dOut,
                             cudaStream_t st) {
  const int64_t n = z.ni * z.nj;
  tan_apply<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(z, q, D, coefW, dIn, dD, dVol, dOut);
  return cudaGetLastError();
}

// ------------------------------------------------- Roe wall-face correction
// wall_corr (correct_flux.for, lapply = 4) at a slip wall (bflwallslip.for):
// D(l0) += F_roe(face) sens_c + fw sens_w, fw from the face average of the
// interior cell l and its ghost ia = l - inc and the raw face normal
// (t0, t1; t2 = 0 in 2-d) -- 10 duals over (l: ro, u, v, T; ia: ro, u, v,
// T; t0, t1).  The Roe term is the face flux of face_lin with the sign
// sens_c: it cancels the face's contribution to D(l0) of the balance.
template <int N>
__device__ __forceinline__ void wallslip_eval(const double* __restrict__ q, int64_t nd, int64_t l,
                                              int64_t ia, double t0v, double t1v, double rgp,
                                              double gam2, int col, double J[4][N]) {
  typedef Dual<N> T;
  const T rl = seed<N>(q[l], 0, col), ul = seed<N>(q[l + nd], 1, col),
          vl = seed<N>(q[l + 2 * nd], 2, col), Tl = seed<N>(q[l + 4 * nd], 3, col);
  const T ra = seed<N>(q[ia], 4, col), ua = seed<N>(q[ia + nd], 5, col),
          va = seed<N>(q[ia + 2 * nd], 6, col), Ta = seed<N>(q[ia + 4 * nd], 7, col);
  const T t0 = seed<N>(t0v, 8, col), t1 = seed<N>(t1v, 9, col);
  const T r = 0.5 * (rl + ra), u = 0.5 * (ul + ua), v = 0.5 * (vl + va);
  const T u_int = t0 * u + t1 * v - 0.;
  T p = Ta * ra * rgp;
  const T h = gam2 * p + r * (u * u + v * v) * 0.5;
  p = 0.5 * (Tl * rl + Ta * ra) * rgp;
  const T f0 = u_int * r, f1 = t0 * p + u_int * r * u, f2 = t1 * p + u_int * r * v;
  const T f4 = u_int * h + p * 0.;
  const T* o[4] = {&f0, &f1, &f2, &f4};
#pragma unroll
  for (int m = 0; m < 4; m++)
#pragma unroll
    for (int k = 0; k < N; k++) J[m][k] = o[m]->d[k];
}
__device__ __forceinline__ void wallslip_lin(const double* __restrict__ q, int64_t nd, int64_t l,
                                             int64_t ia, double t0v, double t1v, double rgp,
                                             double gam2, double J[4][10]) {
  wallslip_eval<10>(q, nd, l, ia, t0v, t1v, rgp, gam2, -1, J);
}

// the Roe part of the wall correction: the face adjoint with mu = sens_c
// lamD(l0); the wall face is a face of the stage's face tape (direction D,
// face (ii, jj) of its high-side cell l), read when a tape is given
template <int D>
__global__ void __launch_bounds__(128) adj_wall_roe(Zone z, const double* __restrict__ q,
                                                    const double* __restrict__ tape,
                                                    const double* __restrict__ lamD,
                                                    double* __restrict__ lamQ,
                                                    double* __restrict__ lamT, WallCorrArgs a) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= a.n) return;
  const int64_t l = a.l[e], l0 = a.l0[e], lt = a.lt[e], nd = z.nd;
  double mu[5];
#pragma unroll
  for (int v = 0; v < 5; v++) mu[v] = lamD[l0 + v * nd] * a.sens_c;
  if (tape) {
    const int64_t NI = z.ni + (D == 0), NJ = z.nj + (D == 1);
    const int64_t ii = l % z.nip - z.ng, jj = l / z.nip - z.ng;
    face_adjoint<D, true>(z, q, l, lt, mu, lamQ, lamT, tape + ii + NI * jj, NI * NJ);
  } else {
    face_adjoint<D>(z, q, l, lt, mu, lamQ, lamT);
  }
}

// the wall-flux part: sixteen lanes per face, lane k < 10 the column of input k
template <int D>
__global__ void __launch_bounds__(128) adj_wall_flux(Zone z, const double* __restrict__ q,
                                                     const double* __restrict__ lamD,
                                                     double* __restrict__ lamQ,
                                                     double* __restrict__ lamT, WallCorrArgs a) {
  const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t e = gid >> 4;
  const int k = (int)(gid & 15);
  if (e >= a.n || k >= 10) return;
  const int64_t l = a.l[e], l0 = a.l0[e], lt = a.lt[e], nd = z.nd, inc = z.inc[D];
  double J[4][1];
  wallslip_eval<1>(q, nd, l, l - inc, a.nrm[3 * e], a.nrm[3 * e + 1], a.rgp, a.gam2, k, J);
  double w = 0.;
#pragma unroll
  for (int m = 0; m < 4; m++) w += lamD[l0 + V4[m] * nd] * a.sens_w * J[m][0];
  if (k < 4) atomicAdd(lamQ + l + V4[k] * nd, w);
  else if (k < 8) atomicAdd(lamQ + l - inc + V4[k - 4] * nd, w);
  else atomicAdd(lamT + lt + (k == 8 ? 0 : z.ndm), w);
}

template <int D>
__global__ void __launch_bounds__(128) tan_wall(Zone z, const double* __restrict__ q,
                                                const double* __restrict__ dq,
                                                const double* __restrict__ dT,
                                                double* __restrict__ dD, WallCorrArgs a) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= a.n) return;
  const int64_t l = a.l[e], l0 = a.l0[e], lt = a.lt[e], nd = z.nd, inc = z.inc[D];
  FaceLin L;
  face_lin<D>(z, q, l, lt, L);
  double din[10];
#pragma unroll
  for (int m = 0; m < 4; m++) {
    const double* Q = dq + V4[m] * nd;
    din[m] = L.gm[m][0] * Q[l - inc] + L.gm[m][1] * Q[l] + L.gm[m][2] * Q[l + inc];
    din[4 + m] = L.gp[m][0] * Q[l - 2 * inc] + L.gp[m][1] * Q[l - inc] + L.gp[m][2] * Q[l];
  }
  din[8] = dT[lt];
  din[9] = dT[lt + z.ndm];
  double J[4][10];
  wallslip_lin(q, nd, l, l - inc, a.nrm[3 * e], a.nrm[3 * e + 1], a.rgp, a.gam2, J);
  const double dw[10] = {dq[l], dq[l + nd], dq[l + 2 * nd], dq[l + 4 * nd],
                         dq[l - inc], dq[l - inc + nd], dq[l - inc + 2 * nd], dq[l - inc + 4 * nd],
                         dT[lt], dT[lt + z.ndm]};
#pragma unroll
  for (int v = 0; v < 5; v++) {
    double f = 0.;
#pragma unroll
    for (int k = 0; k < 10; k++) f += L.JF[v][k] * din[k];
    double x = f * a.sens_c;
    const int m = v == 0 ? 0 : (v == 1 ? 1 : (v == 2 ? 2 : (v == 4 ? 3 : -1)));
    if (m >= 0) {
      double w = 0.;
#pragma unroll
      for (int k = 0; k < 10; k++) w += J[m][k] * dw[k];
      x = x + w * a.sens_w;
    }
    atomicAdd(dD + l0 + v * nd, x);
  }
}

cudaError_t launch_adj_wall(const Zone& z, const double* q, const double* tape,
                            const double* lamD, double* lamQ,
                            double* lamTi, double* lamTj, const WallCorrArgs& a, cudaStream_t st) {
  if (a.n <= 0) return cudaSuccess;
  if (z.typ != Z2D || !a.slip || a.dir > 1) return cudaErrorNotSupported;
  const unsigned g = (unsigned)((a.n + 127) / 128), g16 = (unsigned)((16 * a.n + 127) / 128);
  if (a.dir == 0) {
    adj_wall_roe<0><<<g, 128, 0, st>>>(z, q, tape, lamD, lamQ, lamTi, a);
    adj_wall_flux<0><<<g16, 128, 0, st>>>(z, q, lamD, lamQ, lamTi, a);
  } else {
    adj_wall_roe<1><<<g, 128, 0, st>>>(z, q, tape ? tape + FACE_TAPE * (z.ni + 1) * z.nj : nullptr,
                                       lamD, lamQ, lamTj, a);
    adj_wall_flux<1><<<g16, 128, 0, st>>>(z, q, lamD, lamQ, lamTj, a);
  }
  return cudaGetLastError();
}

cudaError_t launch_tan_wall(const Zone& z, const double* q, const double* dq, const double* dTi,
                            const double* dTj, double* dD, const WallCorrArgs& a, cudaStream_t st) {
  if (a.n <= 0) return cudaSuccess;
  if (z.typ != Z2D || !a.slip || a.dir > 1) return cudaErrorNotSupported;
  const unsigned g = (unsigned)((a.n + 127) / 128);
  if (a.dir == 0) tan_wall<0><<<g, 128, 0, st>>>(z, q, dq, dTi, dD, a);
  else tan_wall<1><<<g, 128, 0, st>>>(z, q, dq, dTj, dD, a);
  return cudaGetLastError();
}

// ------------------------------------------------------------ ghost cells
// bc_face BCF_SLIP: ghost(ro, u, v, T) of mirror cell s and face normal
// (tcx, tcy) -- 6 inputs
template <int N>
__device__ __forceinline__ void slip_eval(const double* __restrict__ q, int64_t nd, int64_t s,
                                          double t0, double t1, int col, double J[4][N]) {
  Dual<N> ro = seed<N>(q[s], 0, col), u = seed<N>(q[s + nd], 1, col),
          v = seed<N>(q[s + 2 * nd], 2, col), tt = seed<N>(q[s + 4 * nd], 3, col),
          tcx = seed<N>(t0, 4, col), tcy = seed<N>(t1, 5, col);
  Dual<N> surf = sqrt(tcx * tcx + tcy * tcy);
  surf = tmax(surf, 1e-30);
  Dual<N> s_1 = 1. / surf;
  tcx = tcx * s_1;
  tcy = tcy * s_1;
  Dual<N> uu = u - 0., vv = v - 0.;
  Dual<N> qn = uu * tcx + vv * tcy;
  Dual<N> ut = uu - qn * tcx, vt = vv - qn * tcy;
  Dual<N> ua = 2. * ut - uu, va = 2. * vt - vv;
  Dual<N> o1 = 0. + ua, o2 = 0. + va;
  const Dual<N>* o[4] = {&ro, &o1, &o2, &tt};
#pragma unroll
  for (int m = 0; m < 4; m++)
#pragma unroll
    for (int k = 0; k < N; k++) J[m][k] = o[m]->d[k];
}
__device__ __forceinline__ void slip_lin(const double* __restrict__ q, int64_t nd, int64_t s,
                                         double t0, double t1, double J[4][6]) {
  slip_eval<6>(q, nd, s, t0, t1, -1, J);
}

// bc_face BCF_FARFIELD (non_reflection.for, 2-d: t[2] = 0): ghost(ro, u, v,
// T) of interior cell s (ro, u, v, T) and the exterior state (st0, st1, st2,
// st4; st3 = 0) -- 8 duals; the normal t (x snorm) is held fixed
template <int N>
__device__ __forceinline__ void farfield_eval(const BcFaceArgs& a, const double* __restrict__ q,
                                              int64_t s, const double t[3], int col,
                                              double J[4][N]) {
  const int64_t nd = a.nd;
  typedef Dual<N> T;
  const T roi = seed<N>(q[s], 0, col), ui = seed<N>(q[s + nd], 1, col),
          vi = seed<N>(q[s + 2 * nd], 2, col), ti = seed<N>(q[s + 4 * nd], 3, col);
  const T e0 = seed<N>(a.st[0], 4, col), e1 = seed<N>(a.st[1], 5, col),
          e2 = seed<N>(a.st[2], 6, col), e3 = T(0.), e4 = seed<N>(a.st[4], 7, col);
  const double gam1 = a.gam1, gam1_1 = a.gam1_1;
  const double tcx = t[0], tcy = t[1], tcz = 0.;
  const double sn = ::sqrt(tcx * tcx + tcy * tcy + tcz * tcz);
  const T rui = ui * roi, rvi = vi * roi, rwi = T(0.) * roi;
  const T eti = ti * a.cv * roi + .5 * (rui * rui + rvi * rvi + rwi * rwi) / roi;
  const T qref1 = .5 * (e0 + roi), qref2 = .5 * (e1 + rui), qref3 = .5 * (e2 + rvi),
          qref4 = .5 * (e3 + rwi), qref5 = .5 * (e4 + eti);
  const T r = qref1, ri = 1. / r;
  const T u = qref2 * ri, v = qref3 * ri, w = qref4 * ri;
  const T p = gam1 * (qref5 - .5 * r * (u * u + v * v + w * w));
  const T c = sqrt(a.gam * p * ri), ci = 1. / c;
  const double s_1 = 1. / sn;
  const T qn = tcx * u + tcy * v + tcz * w - 0.;
  double tnx, tny;
  if (sn == 0.) { tnx = 1.; tny = 0.; } else { tnx = tcx / sn; tny = tcy / sn; }
  const T eig[5] = {qn, qn, qn, qn + sn * c, qn - sn * c};
  T rv[2][5];
  const T qv[2][5] = {{e0, e1, e2, e3, e4}, {roi, rui, rvi, rwi, eti}};
#pragma unroll
  for (int side = 0; side < 2; side++) {
    const T* x = qv[side];
    const T sv1 = x[0], sv2 = (x[1] - u * x[0]) * ri, sv3 = (x[2] - v * x[0]) * ri,
            sv4 = (x[3] - w * x[0]) * ri;
    const T sv5 = gam1 * (.5 * (u * u + v * v + w * w) * x[0] - u * x[1] - v * x[2] - w * x[3] + x[4]);
    rv[side][0] = sv1 - ci * ci * sv5;
    rv[side][1] = tcz * s_1 * (tnx * sv2 + tny * sv3) - sv4;
    rv[side][2] = -tny * sv2 + tnx * sv3;
    rv[side][3] = .5 * s_1 * (tcx * sv2 + tcy * sv3 + tcz * sv4) + .5 * ri * ci * sv5;
    rv[side][4] = -.5 * s_1 * (tcx * sv2 + tcy * sv3 + tcz * sv4) + .5 * ri * ci * sv5;
  }
  T rvar[5];
#pragma unroll
  for (int m = 0; m < 5; m++) rvar[m] = eig[m].v < 0. ? rv[0][m] : rv[1][m];
  T sv[5];
  sv[0] = rvar[0] + r * ci * (rvar[3] + rvar[4]);
  sv[1] = tcz * s_1 * tnx * rvar[1] - tny * rvar[2] + tcx * s_1 * (rvar[3] - rvar[4]);
  sv[2] = tcz * s_1 * tny * rvar[1] + tnx * rvar[2] + tcy * s_1 * (rvar[3] - rvar[4]);
  sv[3] = -rvar[1] + tcz * s_1 * (rvar[3] - rvar[4]);
  sv[4] = r * c * (rvar[3] + rvar[4]);
  const T qvar5 = .5 * (u * u + v * v + w * w) * sv[0] + r * (u * sv[1] + v * sv[2] + w * sv[3]) +
                  gam1_1 * sv[4];
  const T roinv = 1. / sv[0];
  const T uo = u + r * sv[1] * roinv, vo = v + r * sv[2] * roinv, wo = w + r * sv[3] * roinv;
  const T to = (qvar5 * roinv - .5 * (uo * uo + vo * vo + wo * wo)) * a.cvinv;
  const T* o[4] = {&sv[0], &uo, &vo, &to};
#pragma unroll
  for (int m = 0; m < 4; m++)
#pragma unroll
    for (int k = 0; k < N; k++) J[m][k] = o[m]->d[k];
}
__device__ __forceinline__ void farfield_lin(const BcFaceArgs& a, const double* __restrict__ q,
                                             int64_t s, const double t[3], double J[4][8]) {
  farfield_eval<8>(a, q, s, t, -1, J);
}

// Adjoint of the face-BC windows of a zone (all windows in one launch):
// lam[src] += J^T lam[dst], lam[dst] = 0; slip: the window direction's
// metric adjoint (face of the entry) += d/d normal; farfield: lamSt += d/d
// st.  Eight lanes per ghost cell, lane k the Jacobian column of input k
// (one seeded input each); no lane leaves before the warp barrier that
// orders the reads of lam[dst] before its reset.  The tangent kernel applies
// the full local Jacobian (window parameters from c.lp per entry).
__global__ void __launch_bounds__(128) adj_bc_face_cat(const double* __restrict__ q,
                                                       double* __restrict__ lam, BcFaceCat c,
                                                       int64_t ndm, double* __restrict__ lamTi,
                                                       double* __restrict__ lamTj,
                                                       double* __restrict__ lamSt) {
  const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t e = gid >> 3;
  const int k = (int)(gid & 7);
  const bool act = e < c.n;
  int64_t l = 0, s = 0;
  const BcFaceArgs* a = nullptr;
  double lo[4] = {0., 0., 0., 0.};
  if (act) {
    a = c.lp + c.lid[e];
    l = c.dst[e];
    s = c.src[e];
#pragma unroll
    for (int m = 0; m < 4; m++) lo[m] = lam[l + V4[m] * a->nd];
  }
  __syncwarp();
  if (act && k == 0) {
#pragma unroll
    for (int v = 0; v < 5; v++) lam[l + v * a->nd] = 0.;
  }
  if (!act) return;
  const int64_t nd = a->nd;
  double J[4][1];
  if (a->op == BCF_SLIP) {
    if (k >= 6) return;
    slip_eval<1>(q, nd, s, c.nrm[3 * e], c.nrm[3 * e + 1], k, J);
  } else {
    const double t[3] = {c.nrm[3 * e], c.nrm[3 * e + 1], c.nrm[3 * e + 2]};
    farfield_eval<1>(*a, q, s, t, k, J);
  }
  double g = 0.;
#pragma unroll
  for (int m = 0; m < 4; m++) g += lo[m] * J[m][0];
  if (k < 4) atomicAdd(lam + s + V4[k] * nd, g);
  else if (a->op == BCF_SLIP) atomicAdd((a->dir == 0 ? lamTi : lamTj) + c.mt[e] + (k == 4 ? 0 : ndm), g);
  else atomicAdd(lamSt + (k == 7 ? 4 : k - 4), g);
}

__global__ void __launch_bounds__(128) tan_bc_face_cat(const double* __restrict__ q,
                                                       double* __restrict__ dq, BcFaceCat c,
                                                       int64_t ndm, const double* __restrict__ dTi,
                                                       const double* __restrict__ dTj,
                                                       const double* __restrict__ dSt) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= c.n) return;
  const BcFaceArgs& a = c.lp[c.lid[e]];
  const int64_t nd = a.nd, l = c.dst[e], s = c.src[e];
  const double* dT = a.dir == 0 ? dTi : dTj;
  double out[4];
  if (a.op == BCF_SLIP) {
    double J[4][6];
    slip_lin(q, nd, s, c.nrm[3 * e], c.nrm[3 * e + 1], J);
    const double din[6] = {dq[s], dq[s + nd], dq[s + 2 * nd], dq[s + 4 * nd], dT[c.mt[e]],
                           dT[c.mt[e] + ndm]};
#pragma unroll
    for (int m = 0; m < 4; m++) {
      double x = 0.;
#pragma unroll
      for (int k = 0; k < 6; k++) x += J[m][k] * din[k];
      out[m] = x;
    }
  } else {
    const double t[3] = {c.nrm[3 * e], c.nrm[3 * e + 1], c.nrm[3 * e + 2]};
    double J[4][8];
    farfield_lin(a, q, s, t, J);
    const double din[8] = {dq[s], dq[s + nd], dq[s + 2 * nd], dq[s + 4 * nd],
                           dSt[0], dSt[1], dSt[2], dSt[4]};
#pragma unroll
    for (int m = 0; m < 4; m++) {
      double x = 0.;
#pragma unroll
      for (int k = 0; k < 8; k++) x += J[m][k] * din[k];
      out[m] = x;
    }
  }
#pragma unroll
  for (int m = 0; m < 4; m++) dq[l + V4[m] * nd] = out[m];
  dq[l + 3 * nd] = 0.;
}

cudaError_t launch_adj_bc_face_cat(const double* q, double* lam, const BcFaceCat& c, int64_t ndm,
                                   double* lamTi, double* lamTj, double* lamSt, cudaStream_t st) {
  if (c.n <= 0) return cudaSuccess;
  adj_bc_face_cat<<<(unsigned)((8 * c.n + 127) / 128), 128, 0, st>>>(q, lam, c, ndm, lamTi, lamTj, lamSt);
  return cudaGetLastError();
}

cudaError_t launch_tan_bc_face_cat(const double* q, double* dq, const BcFaceCat& c, int64_t ndm,
                                   const double* dTi, const double* dTj, const double* dSt,
                                   cudaStream_t st) {
  if (c.n <= 0) return cudaSuccess;
  tan_bc_face_cat<<<(unsigned)((c.n + 127) / 128), 128, 0, st>>>(q, dq, c, ndm, dTi, dTj, dSt);
  return cudaGetLastError();
}

// bc_next: linear in (q0, q1, q2) with the branch taken at the primal state
__global__ void __launch_bounds__(128) lin_bc_next(const double* __restrict__ q,
                                                   double* __restrict__ x, BcNextArgs a,
                                                   int adjoint, int nv) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= a.n) return;
  const int64_t nd = a.nd, l = a.dst[e], q0 = a.q0[e], q1 = a.q1[e], q2 = a.q2[e];
  const double r = q[q0] * a.k3 + q[q1] * a.k1 + q[q2] * a.k2;
  const bool keep = ::fabs(r / q[q0] - 1.) >= 0.7;
  for (int v = 0; v < nv; v++) {
    const int64_t o = v * nd;
    if (adjoint) {
      const double g = x[l + o];
      x[l + o] = 0.;
      if (keep) {
        atomicAdd(x + q0 + o, g);
      } else {
        atomicAdd(x + q0 + o, a.k3 * g);
        atomicAdd(x + q1 + o, a.k1 * g);
        atomicAdd(x + q2 + o, a.k2 * g);
      }
    } else {
      x[l + o] = keep ? x[q0 + o] : x[q0 + o] * a.k3 + x[q1 + o] * a.k1 + x[q2 + o] * a.k2;
    }
  }
}

cudaError_t launch_lin_bc_next(const double* q, double* x, const BcNextArgs& a, int adjoint, int nv,
                               cudaStream_t st) {
  if (a.n <= 0) return cudaSuccess;
  lin_bc_next<<<(unsigned)((a.n + 127) / 128), 128, 0, st>>>(q, x, a, adjoint, nv);
  return cudaGetLastError();
}

// adjoint of gather_copy (copy or extrapolation, c = 1): lam[src] += lam[dst]
__global__ void __launch_bounds__(256) adj_gather(double* __restrict__ lam, int64_t nd,
                                                  const int32_t* __restrict__ d_idx,
                                                  const int32_t* __restrict__ s_idx, int64_t n,
                                                  int nv) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int64_t d = d_idx[t], s = s_idx[t];
  for (int v = 0; v < nv; v++) {
    const double g = lam[d + v * nd];
    lam[d + v * nd] = 0.;
    atomicAdd(lam + s + v * nd, g);
  }
}

cudaError_t launch_adj_gather(double* lam, int64_t nd, const int32_t* d_idx, const int32_t* s_idx,
                              int64_t n, int nv, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  adj_gather<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(lam, nd, d_idx, s_idx, n, nv);
  return cudaGetLastError();
}

// adjoint of coins: edge (a + b) / 2, corner (a + b + c) / 3
__global__ void __launch_bounds__(256) adj_coins(double* __restrict__ lam, int64_t nd,
                                                 const int32_t* __restrict__ dst,
                                                 const int32_t* __restrict__ a,
                                                 const int32_t* __restrict__ b,
                                                 const int32_t* __restrict__ c, int64_t n_edge,
                                                 int64_t n, int nv) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const double c3 = 1. / 3.;
  for (int v = 0; v < nv; v++) {
    const int64_t o = v * nd;
    const double g = lam[dst[t] + o];
    lam[dst[t] + o] = 0.;
    if (t < n_edge) {
      atomicAdd(lam + a[t] + o, g * 0.5);
      atomicAdd(lam + b[t] + o, g * 0.5);
    } else {
      atomicAdd(lam + a[t] + o, g * c3);
      atomicAdd(lam + b[t] + o, g * c3);
      atomicAdd(lam + c[t] + o, g * c3);
    }
  }
}

cudaError_t launch_adj_coins(double* lam, int64_t nd, const int32_t* dst, const int32_t* a,
                             const int32_t* b, const int32_t* c, int64_t n_edge, int64_t n, int nv,
                             cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  adj_coins<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(lam, nd, dst, a, b, c, n_edge, n, nv);
  return cudaGetLastError();
}

__global__ void __launch_bounds__(256) scale(double* __restrict__ x, int64_t n, double c) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) x[t] = x[t] * c;
}

cudaError_t launch_scale(double* x, int64_t n, double c, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  scale<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(x, n, c);
  return cudaGetLastError();
}

}  // namespace fgb
