// fgb_lu.cu -- implicit-path kernels: time-step / LU coefficients and the
// scalar-diagonal LU-SGS sweeps (sm_103a).
//
// Replaces FastS/FastS/Compute/{invist,tstb3_global,tstb3c}.for (coefficients)
// and FastS/FastS/Compute/LU/{invlu_l,invlu_u,lu_*,mjr_newton}.for (sweeps).
//
// The reference sweeps a zone lexicographically (k, j, i), each cell using the
// already-updated i-1, j-1, k-1 neighbours (lower) or i+1, j+1, k+1 (upper).
// All cells with the same i+j+k only depend on the previous hyperplane, so
// the GPU processes one hyperplane per step: the arithmetic and the data each
// cell sees are exactly the reference's, only the schedule differs.  The
// upper sweep of the reference Newton-updates plane k right after sweeping
// it; when the state array is updated in place (sub-iterations >= 2) the k+1
// neighbour is therefore read after its update while the i+1 / j+1
// neighbours are read before theirs.  The kernels reproduce that by writing
// the updated state to a separate buffer and reading the k+1 neighbour from it.
#include "fgb_kernels.cuh"

namespace fgb {

// ----------------------------------------------------------- coefficients
__global__ void __launch_bounds__(256) coefficients(Zone z, CoeArgs a) {
  const int64_t nx = a.hi[0] - a.lo[0] + 1, ny = a.hi[1] - a.lo[1] + 1, nz = a.hi[2] - a.lo[2] + 1;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nx * ny * nz) return;
  const int64_t i = a.lo[0] + t % nx;
  const int64_t r = t / nx;
  const int64_t j = a.lo[1] + r % ny, k = a.lo[2] + r / ny;
  const int64_t l = inddm(z, i, j, k);
  const int64_t nd = z.nd;
  const double* R = a.rop;
  double xm = 0.;
  if (a.do_invist) {  // invist.for:33-35
    double t1 = R[l + 4 * nd];
    xm = a.coesut * sqrt(t1) * t1 / (t1 + a.cmus1);
    a.xmut[l] = xm;
  } else {
    xm = a.xmut_in[l];
  }
  // tstb3_global.for:58-64
  double c1;
  if (z.typ != Z3DCART) c1 = z.dtc / z.vol[indmtr(z, i, j, k)];
  else c1 = z.dtc / z.vol[0];
  a.coe[l] = c1;
  if (!a.do_lu) return;
  // tstb3c.for
  const double cut0x = 1e-20;
  const double gamma = z.gam;
  const double rgp = z.cv * (gamma - 1.);
  double gam1 = gamma / z.prandt;
  if (z.iflow == 1) gam1 = 0.;
  const double gam2 = gamma * rgp;
  const double xid = a.first_it == 0 ? 1. : 1.5;
  double rr = R[l], u = R[l + nd], v = R[l + 2 * nd], w = R[l + 3 * nd];
  double c = sqrt(gam2 * R[l + 4 * nd]);
  double vmu = gam1 * xm;
  double c2, c3, c4;
  if (z.typ == Z3DCART) {
    double detj = fmaxF(z.vol[0], cut0x);
    double volu = detj * rr;
    double xmvis = vmu / volu;
    double tcxi = z.ti[0], tcyj = z.tj[0], tczk = z.tk[0];
    double tc2i = sqrt(tcxi * tcxi), tc2j = sqrt(tcyj * tcyj), tc2k = sqrt(tczk * tczk);
    double vmi = fabs(tcxi * u) + c * tc2i;
    c2 = vmi * 2. + xmvis * tc2i * tc2i * 4.;
    double vmj = fabs(tcyj * v) + c * tc2j;
    c3 = vmj * 2. + xmvis * tc2j * tc2j * 4.;
    double vmk = fabs(tczk * w) + c * tc2k;
    c4 = vmk * 2. + xmvis * tc2k * tc2k * 4.;
  } else {
    const int64_t lt = indmtr(z, i, j, k), m = z.ndm;
    double detj = fmaxF(z.vol[lt], cut0x);
    double volu = detj * rr;
    double xmvis = vmu / volu;
    const double* T3[3] = {z.ti, z.tj, z.tk};
    double cc[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
      const double* T = T3[d];
      int64_t l2 = lt + z.minc[d];
      double tx = .5 * (T[lt] + T[l2]);
      double ty = .5 * (T[lt + m] + T[l2 + m]);
      double tz = .5 * (T[lt + 2 * m] + T[l2 + 2 * m]);
      double tc2 = .5 * (sqrt(T[lt] * T[lt] + T[lt + m] * T[lt + m] + T[lt + 2 * m] * T[lt + 2 * m]) +
                         sqrt(T[l2] * T[l2] + T[l2 + m] * T[l2 + m] + T[l2 + 2 * m] * T[l2 + 2 * m]));
      double qn = tx * u + ty * v + tz * w;
      double vm = fabs(qn) + c * tc2;
      cc[d] = vm * 2. + xmvis * tc2 * tc2 * 4.;
    }
    c2 = cc[0]; c3 = cc[1]; c4 = cc[2];
  }
  a.coe[l + nd] = c2;
  a.coe[l + 2 * nd] = c3;
  a.coe[l + 3 * nd] = c4;
  a.coe[l + 4 * nd] = xid + c1 * (c2 + c3 + c4) * 0.5;
}

cudaError_t launch_coefficients(const Zone& z, const CoeArgs& a, cudaStream_t st) {
  int64_t n = (a.hi[0] - a.lo[0] + 1) * (a.hi[1] - a.lo[1] + 1) * (a.hi[2] - a.lo[2] + 1);
  coefficients<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(z, a);
  return cudaGetLastError();
}

// ------------------------------------------------------- neighbour term
// b = B_d(W_nb) . dW_nb  (LU/lu_{i,j,k}_3dcart.for, lu_{i,j,k}_3dfull.for).
// signe = +0.5 (lower) / -0.5 (upper); cs = coe_{d+2}(nb) * signe.
template <int TYP, int D, typename T>
__device__ __forceinline__ void nb_term(const Zone& z, const T* __restrict__ R, int64_t l1,
                                        T tcx, T tcy, T tcz, T cs, const T o[5], T b[5],
                                        T gam1, T gamm1, T gam2, T cp) {
  const int64_t nd = z.nd;
  T u = R[l1 + nd], v = R[l1 + 2 * nd], w = R[l1 + 3 * nd], t = R[l1 + 4 * nd];
  T q2 = T(.5) * (u * u + v * v + w * w);
  T h = cp * t + q2;
  T ph2 = gamm1 * q2;
  if (TYP == Z3DCART) {
    if (D == 0) {
      T qn = tcx * u;
      T b21 = (tcx * ph2 - u * qn), b22 = (qn - tcx * gam2 * u) + cs, b23 = (-tcx * gamm1 * v),
        b24 = (-tcx * gamm1 * w), b25 = tcx * gamm1;
      T b31 = (-v * qn), b32 = (tcx * v), b33 = (qn) + cs;
      T b41 = (-w * qn), b42 = (tcx * w), b44 = (qn) + cs;
      T b51 = qn * (ph2 - h), b52 = (tcx * h - gamm1 * u * qn), b53 = (-gamm1 * v * qn),
        b54 = (-gamm1 * w * qn), b55 = (gam1 * qn) + cs;
      b[0] = cs * o[0] + tcx * o[1];
      b[1] = b21 * o[0] + b22 * o[1] + b23 * o[2] + b24 * o[3] + b25 * o[4];
      b[2] = b31 * o[0] + b32 * o[1] + b33 * o[2];
      b[3] = b41 * o[0] + b42 * o[1] + b44 * o[3];
      b[4] = b51 * o[0] + b52 * o[1] + b53 * o[2] + b54 * o[3] + b55 * o[4];
    } else if (D == 1) {
      T qn = tcy * v;
      T b21 = (-u * qn), b22 = qn + cs, b23 = tcy * u;
      T b31 = (tcy * ph2 - v * qn), b32 = (-tcy * gamm1 * u), b33 = (qn - tcy * gam2 * v) + cs,
        b34 = (-tcy * gamm1 * w), b35 = tcy * gamm1;
      T b41 = (-w * qn), b43 = (tcy * w), b44 = (qn) + cs;
      T b51 = qn * (ph2 - h), b52 = (-gamm1 * u * qn), b53 = (tcy * h - gamm1 * v * qn),
        b54 = (-gamm1 * w * qn), b55 = (gam1 * qn) + cs;
      b[0] = cs * o[0] + tcy * o[2];
      b[1] = b21 * o[0] + b22 * o[1] + b23 * o[2];
      b[2] = b31 * o[0] + b32 * o[1] + b33 * o[2] + b34 * o[3] + b35 * o[4];
      b[3] = b41 * o[0] + b43 * o[2] + b44 * o[3];
      b[4] = b51 * o[0] + b52 * o[1] + b53 * o[2] + b54 * o[3] + b55 * o[4];
    } else {
      T qn = tcz * w;
      T b21 = -u * qn, b22 = qn + cs, b24 = tcz * u;
      T b31 = -v * qn, b33 = qn + cs, b34 = tcz * v;
      T b41 = tcz * ph2 - w * qn, b42 = -tcz * gamm1 * u, b43 = -tcz * gamm1 * v,
        b44 = (qn - tcz * gam2 * w) + cs, b45 = tcz * gamm1;
      T b51 = qn * (ph2 - h), b52 = -gamm1 * u * qn, b53 = -gamm1 * v * qn,
        b54 = tcz * h - gamm1 * w * qn, b55 = gam1 * qn + cs;
      b[0] = cs * o[0] + tcz * o[3];
      b[1] = b21 * o[0] + b22 * o[1] + b24 * o[3];
      b[2] = b31 * o[0] + b33 * o[2] + b34 * o[3];
      b[3] = b41 * o[0] + b42 * o[1] + b43 * o[2] + b44 * o[3] + b45 * o[4];
      b[4] = b51 * o[0] + b52 * o[1] + b53 * o[2] + b54 * o[3] + b55 * o[4];
    }
  } else {
    T qn = tcx * u + tcy * v + tcz * w;
    T b21 = (tcx * ph2 - u * qn), b22 = (qn - tcx * gam2 * u) + cs,
      b23 = (tcy * u - tcx * gamm1 * v), b24 = (tcz * u - tcx * gamm1 * w), b25 = tcx * gamm1;
    T b31 = (tcy * ph2 - v * qn), b32 = (tcx * v - tcy * gamm1 * u),
      b33 = (qn - tcy * gam2 * v) + cs, b34 = (tcz * v - tcy * gamm1 * w), b35 = tcy * gamm1;
    T b41 = (tcz * ph2 - w * qn), b42 = (tcx * w - tcz * gamm1 * u),
      b43 = (tcy * w - tcz * gamm1 * v), b44 = (qn - tcz * gam2 * w) + cs, b45 = tcz * gamm1;
    T b51 = qn * (ph2 - h), b52 = (tcx * h - gamm1 * u * qn), b53 = (tcy * h - gamm1 * v * qn),
      b54 = (tcz * h - gamm1 * w * qn), b55 = (gam1 * qn) + cs;
    b[0] = cs * o[0] + tcx * o[1] + tcy * o[2] + tcz * o[3];
    b[1] = b21 * o[0] + b22 * o[1] + b23 * o[2] + b24 * o[3] + b25 * o[4];
    b[2] = b31 * o[0] + b32 * o[1] + b33 * o[2] + b34 * o[3] + b35 * o[4];
    b[3] = b41 * o[0] + b42 * o[1] + b43 * o[2] + b44 * o[3] + b45 * o[4];
    b[4] = b51 * o[0] + b52 * o[1] + b53 * o[2] + b54 * o[3] + b55 * o[4];
  }
}

// metric normal of the neighbour cell in direction d (mean of its two faces)
template <int TYP, typename T>
__device__ __forceinline__ void nb_normal(const Zone& z, int d, int64_t lta, int64_t ltb, T& tx,
                                          T& ty, T& tz) {
  if (TYP == Z3DCART) {
    tx = d == 0 ? T(z.tcx) : T(0);
    ty = d == 1 ? T(z.tcy) : T(0);
    tz = d == 2 ? T(z.tcz) : T(0);
  } else {
    const double* M = d == 0 ? z.ti : (d == 1 ? z.tj : z.tk);
    const int64_t m = z.ndm;
    tx = T(0.5 * (M[ltb] + M[lta]));
    ty = T(0.5 * (M[ltb + m] + M[lta + m]));
    tz = T(0.5 * (M[ltb + 2 * m] + M[lta + 2 * m]));
  }
}

template <int D> struct DirT { static constexpr int value = D; };

template <int TYP>
__global__ void __launch_bounds__(128) lu_lower(Zone z, LuArgs a) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= a.nbj * a.nbk) return;
  const int64_t jj = a.jlo + t % a.nbj, kk = a.klo + t / a.nbj;
  const int64_t ii = a.s - jj - kk;
  if (ii < 0 || ii >= z.ni) return;
  const int64_t l = inddm(z, ii + 1, jj + 1, kk + 1);
  const int64_t lt = TYP == Z3DCART ? 0 : indmtr(z, ii + 1, jj + 1, kk + 1);
  const int64_t nd = z.nd;
  const double gam1 = z.gam, gamm1 = gam1 - 1., cp = z.gam * z.cv, gam2 = gamm1 - 1.;
  const double xal = a.coe[l] * 0.5;
  double x[5], o[5], b[5];
#pragma unroll
  for (int v = 0; v < 5; v++) x[v] = a.din[l + v * nd];
  auto term = [&](auto dc, int64_t l1) {
    constexpr int D = decltype(dc)::value;
    double tx, ty, tz;
    nb_normal<TYP, double>(z, D, lt - z.minc[D], lt, tx, ty, tz);
#pragma unroll
    for (int v = 0; v < 5; v++) o[v] = a.dout[l1 + v * nd];
    double cs = a.coe[l1 + (D + 1) * nd] * 0.5;
    nb_term<TYP, D, double>(z, a.rop_old, l1, tx, ty, tz, cs, o, b, gam1, gamm1, gam2, cp);
#pragma unroll
    for (int v = 0; v < 5; v++) x[v] = x[v] + b[v] * xal;
  };
  if (TYP == Z3DCART) {  // invlu_l.for cartesian section: j, then k, then i
    if (jj > 0) term(DirT<1>{}, l - z.inc[1]);
    if (kk > 0) term(DirT<2>{}, l - z.inc[2]);
  } else {               // general section: k, then j, then i
    if (kk > 0) term(DirT<2>{}, l - z.inc[2]);
    if (jj > 0) term(DirT<1>{}, l - z.inc[1]);
  }
  if (ii > 0) term(DirT<0>{}, l - 1);
  const double diag = 1. / a.coe[l + 4 * nd];
#pragma unroll
  for (int v = 0; v < 5; v++) a.dout[l + v * nd] = x[v] * diag;
}

template <int TYP>
__global__ void __launch_bounds__(128) lu_upper(Zone z, LuArgs a) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= a.nbj * a.nbk) return;
  const int64_t jj = a.jlo + t % a.nbj, kk = a.klo + t / a.nbj;
  const int64_t ii = a.s - jj - kk;
  if (ii < 0 || ii >= z.ni) return;
  const int64_t l = inddm(z, ii + 1, jj + 1, kk + 1);
  const int64_t lt = TYP == Z3DCART ? 0 : indmtr(z, ii + 1, jj + 1, kk + 1);
  const int64_t nd = z.nd;
  const double gam1 = z.gam, gamm1 = gam1 - 1., cp = z.gam * z.cv, gam2 = gamm1 - 1.;
  const double xal = a.coe[l] * (-0.5);
  const double dg = a.coe[l + 4 * nd];
  double x[5], o[5], b[5];
#pragma unroll
  for (int v = 0; v < 5; v++) x[v] = a.dout[l + v * nd] * dg;  // lu_d.for
  auto term = [&](auto dc, int64_t l1, const double* R) {
    constexpr int D = decltype(dc)::value;
    double tx, ty, tz;
    nb_normal<TYP, double>(z, D, lt + z.minc[D], lt + 2 * z.minc[D], tx, ty, tz);
#pragma unroll
    for (int v = 0; v < 5; v++) o[v] = a.dout[l1 + v * nd];
    double cs = a.coe[l1 + (D + 1) * nd] * (-0.5);
    nb_term<TYP, D, double>(z, R, l1, tx, ty, tz, cs, o, b, gam1, gamm1, gam2, cp);
#pragma unroll
    for (int v = 0; v < 5; v++) x[v] = x[v] + b[v] * xal;
  };
  if (kk < z.nk - 1) term(DirT<2>{}, l + z.inc[2], a.rop_knb);
  if (jj < z.nj - 1) term(DirT<1>{}, l + z.inc[1], a.rop_old);
  if (ii < z.ni - 1) term(DirT<0>{}, l + 1, a.rop_old);
  const double diag = 1. / a.coe[l + 4 * nd];
#pragma unroll
  for (int v = 0; v < 5; v++) x[v] = x[v] * diag;
#pragma unroll
  for (int v = 0; v < 5; v++) a.dout[l + v * nd] = x[v];
  // mjr_newton.for: W^{p+1} = prim(cons(W^p) + dW)
  const double* R = a.rop_old;
  const double cv = z.cv, cvinv = 1. / cv, cvinv2 = 0.5 * cvinv;
  double ro = R[l], u = R[l + nd], v = R[l + 2 * nd], w = R[l + 3 * nd], tt = R[l + 4 * nd];
  double n1 = ro + x[0];
  double r_1 = 1. / n1;
  double n2 = (ro * u + x[1]) * r_1;
  double n3 = (ro * v + x[2]) * r_1;
  double n4 = (ro * w + x[3]) * r_1;
  double roe_old = ro * (cv * tt + 0.5 * (u * u + v * v + w * w));
  double n5 = (roe_old + x[4]) * r_1 * cvinv - cvinv2 * (n2 * n2 + n3 * n3 + n4 * n4);
  double* O = a.rop_new;
  O[l] = n1; O[l + nd] = n2; O[l + 2 * nd] = n3; O[l + 3 * nd] = n4; O[l + 4 * nd] = n5;
}

// One full LU-SGS solve (lower, then upper + Newton update) as a sequence of
// hyperplane launches on stream st.
cudaError_t launch_lusgs(const Zone& z, LuArgs a, cudaStream_t st) {
  const int B = 128;
  const int64_t smax = (z.ni - 1) + (z.nj - 1) + (z.nk - 1);
  auto box = [&](int64_t s) {
    int64_t jlo = s - (z.ni - 1) - (z.nk - 1); if (jlo < 0) jlo = 0;
    int64_t jhi = s < z.nj - 1 ? s : z.nj - 1;
    int64_t klo = s - (z.ni - 1) - (z.nj - 1); if (klo < 0) klo = 0;
    int64_t khi = s < z.nk - 1 ? s : z.nk - 1;
    a.s = s; a.jlo = jlo; a.klo = klo; a.nbj = jhi - jlo + 1; a.nbk = khi - klo + 1;
  };
  for (int64_t s = 0; s <= smax; s++) {
    box(s);
    unsigned g = (unsigned)((a.nbj * a.nbk + B - 1) / B);
    if (z.typ == Z3DCART) lu_lower<Z3DCART><<<g, B, 0, st>>>(z, a);
    else lu_lower<Z3DFULL><<<g, B, 0, st>>>(z, a);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  for (int64_t s = smax; s >= 0; s--) {
    box(s);
    unsigned g = (unsigned)((a.nbj * a.nbk + B - 1) / B);
    if (z.typ == Z3DCART) lu_upper<Z3DCART><<<g, B, 0, st>>>(z, a);
    else lu_upper<Z3DFULL><<<g, B, 0, st>>>(z, a);
  }
  return cudaGetLastError();
}

}  // namespace fgb
