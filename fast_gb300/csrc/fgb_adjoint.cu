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
DUAL_BIN(/, (a.d[k] - r.v * b.d[k]) / b.v, , )
#undef DUAL_BIN
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

// ------------------------------------------------------ restated formulas
template <typename T>
__device__ __forceinline__ T vanalbada_t(const T& x, const T& y) {
  const double e2 = 1e-12;
  return ((y * y + e2) * x + (x * x + e2) * y) / (x * x + y * y + 2. * e2);
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
template <int D>
__global__ void __launch_bounds__(128) adj_faces(Zone z, const double* __restrict__ q,
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
  FaceLin L;
  face_lin<D>(z, q, l, lt, L);
  double g[10];
#pragma unroll
  for (int k = 0; k < 10; k++) {
    double s = 0.;
#pragma unroll
    for (int v = 0; v < 5; v++) s += mu[v] * L.JF[v][k];
    g[k] = s;
  }
#pragma unroll
  for (int m = 0; m < 4; m++) {
    const int64_t o = V4[m] * nd;
    const double gm = g[m], gp = g[4 + m];
    atomicAdd(lamQ + l - 2 * inc + o, gp * L.gp[m][0]);
    atomicAdd(lamQ + l - inc + o, gm * L.gm[m][0] + gp * L.gp[m][1]);
    atomicAdd(lamQ + l + o, gm * L.gm[m][1] + gp * L.gp[m][2]);
    atomicAdd(lamQ + l + inc + o, gm * L.gm[m][2]);
  }
  atomicAdd(lamT + lt, g[8]);
  atomicAdd(lamT + lt + z.ndm, g[9]);
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

cudaError_t launch_adj_faces(const Zone& z, const double* q, const double* lamD, double* lamQ,
                             double* lamTi, double* lamTj, cudaStream_t st) {
  if (z.typ != Z2D) return cudaErrorNotSupported;
  const int B = 128;
  const int64_t nfi = (z.ni + 1) * z.nj, nfj = z.ni * (z.nj + 1);
  adj_faces<0><<<(unsigned)((nfi + B - 1) / B), B, 0, st>>>(z, q, lamD, lamQ, lamTi);
  adj_faces<1><<<(unsigned)((nfj + B - 1) / B), B, 0, st>>>(z, q, lamD, lamQ, lamTj);
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
  double J[4][9];
  update_lin(z, q, D, l, lt, coefW, J);
  double lo[4];
#pragma unroll
  for (int m = 0; m < 4; m++) { lo[m] = lamOut[l + V4[m] * nd]; lamOut[l + V4[m] * nd] = 0.; }
  lamOut[l + 3 * nd] = 0.;
  double g[9];
#pragma unroll
  for (int k = 0; k < 9; k++) {
    double s = 0.;
#pragma unroll
    for (int m = 0; m < 4; m++) s += lo[m] * J[m][k];
    g[k] = s;
  }
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
__device__ __forceinline__ void wallslip_lin(const double* __restrict__ q, int64_t nd, int64_t l,
                                             int64_t ia, double t0v, double t1v, double rgp,
                                             double gam2, double J[4][10]) {
  typedef Dual<10> T;
  const T rl = var<10>(q[l], 0), ul = var<10>(q[l + nd], 1), vl = var<10>(q[l + 2 * nd], 2),
          Tl = var<10>(q[l + 4 * nd], 3);
  const T ra = var<10>(q[ia], 4), ua = var<10>(q[ia + nd], 5), va = var<10>(q[ia + 2 * nd], 6),
          Ta = var<10>(q[ia + 4 * nd], 7);
  const T t0 = var<10>(t0v, 8), t1 = var<10>(t1v, 9);
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
    for (int k = 0; k < 10; k++) J[m][k] = o[m]->d[k];
}

template <int D>
__global__ void __launch_bounds__(128) adj_wall(Zone z, const double* __restrict__ q,
                                                const double* __restrict__ lamD,
                                                double* __restrict__ lamQ,
                                                double* __restrict__ lamT, WallCorrArgs a) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= a.n) return;
  const int64_t l = a.l[e], l0 = a.l0[e], lt = a.lt[e], nd = z.nd, inc = z.inc[D];
  double mu[5];
#pragma unroll
  for (int v = 0; v < 5; v++) mu[v] = lamD[l0 + v * nd] * a.sens_c;
  FaceLin L;
  face_lin<D>(z, q, l, lt, L);
  double g[10];
#pragma unroll
  for (int k = 0; k < 10; k++) {
    double s = 0.;
#pragma unroll
    for (int v = 0; v < 5; v++) s += mu[v] * L.JF[v][k];
    g[k] = s;
  }
#pragma unroll
  for (int m = 0; m < 4; m++) {
    const int64_t o = V4[m] * nd;
    const double gm = g[m], gp = g[4 + m];
    atomicAdd(lamQ + l - 2 * inc + o, gp * L.gp[m][0]);
    atomicAdd(lamQ + l - inc + o, gm * L.gm[m][0] + gp * L.gp[m][1]);
    atomicAdd(lamQ + l + o, gm * L.gm[m][1] + gp * L.gp[m][2]);
    atomicAdd(lamQ + l + inc + o, gm * L.gm[m][2]);
  }
  atomicAdd(lamT + lt, g[8]);
  atomicAdd(lamT + lt + z.ndm, g[9]);
  // the wall flux
  double J[4][10];
  wallslip_lin(q, nd, l, l - inc, a.nrm[3 * e], a.nrm[3 * e + 1], a.rgp, a.gam2, J);
  double w[10];
#pragma unroll
  for (int k = 0; k < 10; k++) {
    double s = 0.;
#pragma unroll
    for (int m = 0; m < 4; m++) s += lamD[l0 + V4[m] * nd] * a.sens_w * J[m][k];
    w[k] = s;
  }
#pragma unroll
  for (int m = 0; m < 4; m++) {
    atomicAdd(lamQ + l + V4[m] * nd, w[m]);
    atomicAdd(lamQ + l - inc + V4[m] * nd, w[4 + m]);
  }
  atomicAdd(lamT + lt, w[8]);
  atomicAdd(lamT + lt + z.ndm, w[9]);
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

cudaError_t launch_adj_wall(const Zone& z, const double* q, const double* lamD, double* lamQ,
                            double* lamTi, double* lamTj, const WallCorrArgs& a, cudaStream_t st) {
  if (a.n <= 0) return cudaSuccess;
  if (z.typ != Z2D || !a.slip || a.dir > 1) return cudaErrorNotSupported;
  const unsigned g = (unsigned)((a.n + 127) / 128);
  if (a.dir == 0) adj_wall<0><<<g, 128, 0, st>>>(z, q, lamD, lamQ, lamTi, a);
  else adj_wall<1><<<g, 128, 0, st>>>(z, q, lamD, lamQ, lamTj, a);
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
// (tcx, tcy) -- 6 duals
__device__ __forceinline__ void slip_lin(const double* __restrict__ q, int64_t nd, int64_t s,
                                         double t0, double t1, double J[4][6]) {
  Dual<6> ro = var<6>(q[s], 0), u = var<6>(q[s + nd], 1), v = var<6>(q[s + 2 * nd], 2),
          tt = var<6>(q[s + 4 * nd], 3), tcx = var<6>(t0, 4), tcy = var<6>(t1, 5);
  Dual<6> surf = sqrt(tcx * tcx + tcy * tcy);
  surf = tmax(surf, 1e-30);
  Dual<6> s_1 = 1. / surf;
  tcx = tcx * s_1;
  tcy = tcy * s_1;
  Dual<6> uu = u - 0., vv = v - 0.;
  Dual<6> qn = uu * tcx + vv * tcy;
  Dual<6> ut = uu - qn * tcx, vt = vv - qn * tcy;
  Dual<6> ua = 2. * ut - uu, va = 2. * vt - vv;
  Dual<6> o1 = 0. + ua, o2 = 0. + va;
  const Dual<6>* o[4] = {&ro, &o1, &o2, &tt};
#pragma unroll
  for (int m = 0; m < 4; m++)
#pragma unroll
    for (int k = 0; k < 6; k++) J[m][k] = o[m]->d[k];
}

// bc_face BCF_FARFIELD (non_reflection.for, 2-d: t[2] = 0): ghost(ro, u, v,
// T) of interior cell s (ro, u, v, T) and the exterior state (st0, st1, st2,
// st4; st3 = 0) -- 8 duals; the normal t (x snorm) is held fixed
__device__ __forceinline__ void farfield_lin(const BcFaceArgs& a, const double* __restrict__ q,
                                             int64_t s, const double t[3], double J[4][8]) {
  const int64_t nd = a.nd;
  typedef Dual<8> T;
  const T roi = var<8>(q[s], 0), ui = var<8>(q[s + nd], 1), vi = var<8>(q[s + 2 * nd], 2),
          ti = var<8>(q[s + 4 * nd], 3);
  const T e0 = var<8>(a.st[0], 4), e1 = var<8>(a.st[1], 5), e2 = var<8>(a.st[2], 6), e3 = T(0.),
          e4 = var<8>(a.st[4], 7);
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
    for (int k = 0; k < 8; k++) J[m][k] = o[m]->d[k];
}

// adjoint of one face-BC list: lam[src] += J^T lam[dst], lam[dst] = 0;
// slip: lamT[mt] (metric of the face) += d/d normal; farfield: lamSt += d/d st
__global__ void __launch_bounds__(128) adj_bc_face(const double* __restrict__ q,
                                                   double* __restrict__ lam, BcFaceArgs a,
                                                   const int32_t* __restrict__ mt, int64_t ndm,
                                                   double* __restrict__ lamT,
                                                   double* __restrict__ lamSt) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= a.n) return;
  const int64_t nd = a.nd, l = a.dst[e], s = a.src[e];
  double lo[4];
#pragma unroll
  for (int m = 0; m < 4; m++) { lo[m] = lam[l + V4[m] * nd]; lam[l + V4[m] * nd] = 0.; }
  lam[l + 3 * nd] = 0.;
  if (a.op == BCF_SLIP) {
    double J[4][6];
    slip_lin(q, nd, s, a.nrm[3 * e], a.nrm[3 * e + 1], J);
    double g[6];
#pragma unroll
    for (int k = 0; k < 6; k++) {
      double x = 0.;
#pragma unroll
      for (int m = 0; m < 4; m++) x += lo[m] * J[m][k];
      g[k] = x;
    }
#pragma unroll
    for (int m = 0; m < 4; m++) atomicAdd(lam + s + V4[m] * nd, g[m]);
    atomicAdd(lamT + mt[e], g[4]);
    atomicAdd(lamT + mt[e] + ndm, g[5]);
  } else {   // BCF_FARFIELD
    const double t[3] = {a.nrm[3 * e], a.nrm[3 * e + 1], a.nrm[3 * e + 2]};
    double J[4][8];
    farfield_lin(a, q, s, t, J);
    double g[8];
#pragma unroll
    for (int k = 0; k < 8; k++) {
      double x = 0.;
#pragma unroll
      for (int m = 0; m < 4; m++) x += lo[m] * J[m][k];
      g[k] = x;
    }
#pragma unroll
    for (int m = 0; m < 4; m++) atomicAdd(lam + s + V4[m] * nd, g[m]);
    atomicAdd(lamSt + 0, g[4]);
    atomicAdd(lamSt + 1, g[5]);
    atomicAdd(lamSt + 2, g[6]);
    atomicAdd(lamSt + 4, g[7]);
  }
}

// tangent of one face-BC list: dq[dst] = J (dq[src], dnormal | dst)
__global__ void __launch_bounds__(128) tan_bc_face(const double* __restrict__ q,
                                                   double* __restrict__ dq, BcFaceArgs a,
                                                   const int32_t* __restrict__ mt, int64_t ndm,
                                                   const double* __restrict__ dT,
                                                   const double* __restrict__ dSt) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= a.n) return;
  const int64_t nd = a.nd, l = a.dst[e], s = a.src[e];
  double out[4];
  if (a.op == BCF_SLIP) {
    double J[4][6];
    slip_lin(q, nd, s, a.nrm[3 * e], a.nrm[3 * e + 1], J);
    const double din[6] = {dq[s], dq[s + nd], dq[s + 2 * nd], dq[s + 4 * nd], dT[mt[e]],
                           dT[mt[e] + ndm]};
#pragma unroll
    for (int m = 0; m < 4; m++) {
      double x = 0.;
#pragma unroll
      for (int k = 0; k < 6; k++) x += J[m][k] * din[k];
      out[m] = x;
    }
  } else {
    const double t[3] = {a.nrm[3 * e], a.nrm[3 * e + 1], a.nrm[3 * e + 2]};
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

cudaError_t launch_adj_bc_face(const double* q, double* lam, const BcFaceArgs& a, const int32_t* mt,
                               int64_t ndm, double* lamT, double* lamSt, cudaStream_t st) {
  if (a.n <= 0) return cudaSuccess;
  if (a.op != BCF_SLIP && a.op != BCF_FARFIELD) return cudaErrorNotSupported;
  adj_bc_face<<<(unsigned)((a.n + 127) / 128), 128, 0, st>>>(q, lam, a, mt, ndm, lamT, lamSt);
  return cudaGetLastError();
}

cudaError_t launch_tan_bc_face(const double* q, double* dq, const BcFaceArgs& a, const int32_t* mt,
                               int64_t ndm, const double* dT, const double* dSt, cudaStream_t st) {
  if (a.n <= 0) return cudaSuccess;
  if (a.op != BCF_SLIP && a.op != BCF_FARFIELD) return cudaErrorNotSupported;
  tan_bc_face<<<(unsigned)((a.n + 127) / 128), 128, 0, st>>>(q, dq, a, mt, ndm, dT, dSt);
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
