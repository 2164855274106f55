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
#include <algorithm>
#include "fgb_kernels.cuh"

namespace fgb {

// ----------------------------------------------------------- coefficients
// tstb3_impli.for with dtloc.for (implicit, local time step, DTLOC = 1): the
// spectral radii coe2..4 as tstb3c.for forms them, then coe1 = CFL x
// min(dtconv, dtvis) per cell (d = 1 / sum tc2^2, dtvis = 0.5 detj d / gam1
// / xmut ro, dtconv = sqrt(d) / (|u| + c)) and coe5 = 1 + coe1 sum / 2.
// Euler: gam1 = 1e-30 (tstb3c.for takes 0); volume floor 1e-30.
// Explicit (tstb3_expli.for): the same time step, coe1 only.
__device__ __forceinline__ void coefficients_local(const Zone& z, const CoeArgs& a, int64_t l,
                                                   int64_t i, int64_t j, int64_t k, double xm) {
  const bool lu = a.do_lu;
  const int64_t nd = z.nd;
  const double* R = a.rop;
  const double cut0x = 1e-30;
  const double gamma = z.gam;
  const double rgp = z.cv * (gamma - 1.);
  double gam1 = gamma / z.prandt;
  if (z.iflow == 1) gam1 = cut0x;
  const double gam1_1 = 1. / gam1;
  const double gam2 = gamma * rgp;
  const double r = R[l], u = R[l + nd], v = R[l + 2 * nd], w = z.typ == Z2D ? 0. : R[l + 3 * nd];
  const double c = sqrt(gam2 * R[l + 4 * nd]);
  const double vmu = gam1 * xm;
  double tc2[3], cc[3] = {0., 0., 0.}, detj;
  if (z.typ == Z3DCART) {
    detj = fmaxF(z.vol[0], cut0x);
    const double xmvis = vmu / (detj * r);
    const double tc[3] = {z.ti[0], z.tj[0], z.tk[0]}, q[3] = {u, v, w};
#pragma unroll
    for (int d = 0; d < 3; d++) {
      tc2[d] = z.ctc2[d];   // sqrt(tc^2), once per zone
      if (lu) {
        const double vm = fabs(tc[d] * q[d]) + c * tc2[d];
        cc[d] = mul_pow2<1>(vm) + mul_pow2<2>(xmvis * tc2[d] * tc2[d]);
      }
    }
  } else {
    const int64_t lt = indmtr(z, i, j, k), m = z.ndm;
    detj = fmaxF(z.vol[lt], cut0x);
    const double xmvis = vmu / (detj * r);
    const double* T3[3] = {z.ti, z.tj, z.tk};
    const int nd3 = z.typ == Z2D ? 2 : 3;
    tc2[2] = 0.; cc[2] = 0.;
    for (int d = 0; d < nd3; d++) {
      const double* T = T3[d];
      const int64_t l2 = lt + z.minc[d];
      const double tx = mul_pow2<-1>(T[lt] + T[l2]);
      const double ty = mul_pow2<-1>(T[lt + m] + T[l2 + m]);
      double qn;
      if (z.typ == Z2D) {
        tc2[d] = mul_pow2<-1>(sqrt(T[lt] * T[lt] + T[lt + m] * T[lt + m]) +
                              sqrt(T[l2] * T[l2] + T[l2 + m] * T[l2 + m]));
        qn = tx * u + ty * v;
      } else {
        const double tz = mul_pow2<-1>(T[lt + 2 * m] + T[l2 + 2 * m]);
        tc2[d] = mul_pow2<-1>(sqrt(T[lt] * T[lt] + T[lt + m] * T[lt + m] + T[lt + 2 * m] * T[lt + 2 * m]) +
                              sqrt(T[l2] * T[l2] + T[l2 + m] * T[l2 + m] + T[l2 + 2 * m] * T[l2 + 2 * m]));
        qn = tx * u + ty * v + tz * w;
      }
      if (lu) {
        const double vm = fabs(qn) + c * tc2[d];
        cc[d] = mul_pow2<1>(vm) + mul_pow2<2>(xmvis * tc2[d] * tc2[d]);
      }
    }
  }
  // dtloc.for
  const double dd = 1. / (tc2[0] * tc2[0] + tc2[1] * tc2[1] + tc2[2] * tc2[2]);
  const double dtvis = mul_pow2<-1>(detj) * dd * gam1_1 / xm * r;
  const double sp = sqrt(u * u + v * v + w * w) + c;
  const double dtconv = sqrt(dd) / sp;
  const double c1 = z.cfl * fminF(dtconv, dtvis);
  a.coe[l] = c1;
  if (!lu) return;
  a.coe[l + nd] = cc[0];
  a.coe[l + 2 * nd] = cc[1];
  if (z.typ == Z2D) {
    a.coe[l + 4 * nd] = 1. + mul_pow2<-1>(c1 * (cc[0] + cc[1]));
  } else {
    a.coe[l + 3 * nd] = cc[2];
    a.coe[l + 4 * nd] = 1. + mul_pow2<-1>(c1 * (cc[0] + cc[1] + cc[2]));
  }
}

__device__ __forceinline__ void coefficients_at(const Zone& z, const CoeArgs& a, const int64_t t) {
  const int64_t nx = a.hi[0] - a.lo[0] + 1, ny = a.hi[1] - a.lo[1] + 1, nz = a.hi[2] - a.lo[2] + 1;
  if (t >= nx * ny * nz) return;
  const int64_t i = a.lo[0] + t % nx;
  const int64_t r = t / nx;
  const int64_t j = a.lo[1] + r % ny, k = a.lo[2] + r / ny;
  const int64_t l = inddm(z, i, j, k);
  const int64_t nd = z.nd;
  const double* R = a.rop;
  double xm = 0.;
  if (a.do_sa) {      // SA/vispalart.for with mulam.for, chi.for, xmut.for
    const double amulam = sa_mulam(z, R[l + 4 * nd]);
    const double anulam = R[l] / amulam;
    const double anutild = fmaxF(R[l + 5 * nd], 1.e-27);
    const double chi = fmaxF(anutild * anulam, 1.e-7);
    const double fvv1 = 1. / (1. + SA_CV1 / (chi * chi * chi));
    const double amut = R[l] * anutild * fvv1;
    const double xmuprov = fmaxF(amut, 0.);
    xm = amulam + fminF(xmuprov, z.ratiom * amulam);
    a.xmut[l] = xm;
  } else if (a.do_invist) {  // invist.for:33-35
    double t1 = R[l + 4 * nd];
    xm = a.coesut * sqrt(t1) * t1 / (t1 + a.cmus1);
    a.xmut[l] = xm;
  } else {
    xm = a.xmut_in[l];
  }
  if (z.dtloc == 1) {   // cptst3.for: local time step (tstb3_impli.for / tstb3_expli.for)
    coefficients_local(z, a, l, i, j, k, xm);
    return;
  }
  // tstb3_global.for:58-64
  double c1;
  if (z.typ != Z3DCART) c1 = z.dtc / z.vol[indmtr(z, i, j, k)];
  else c1 = z.cdtv;   // dtc / vol[0], once per zone
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
    const double tc2i = z.ctc2[0], tc2j = z.ctc2[1], tc2k = z.ctc2[2];   // sqrt(tc^2), once per zone
    double vmi = fabs(tcxi * u) + c * tc2i;
    c2 = mul_pow2<1>(vmi) + mul_pow2<2>(xmvis * tc2i * tc2i);
    double vmj = fabs(tcyj * v) + c * tc2j;
    c3 = mul_pow2<1>(vmj) + mul_pow2<2>(xmvis * tc2j * tc2j);
    double vmk = fabs(tczk * w) + c * tc2k;
    c4 = mul_pow2<1>(vmk) + mul_pow2<2>(xmvis * tc2k * tc2k);
  } else if (z.typ == Z2D) {  // tstb3c.for 2-d branch: i and j only
    const int64_t lt = indmtr(z, i, j, k), m = z.ndm;
    double detj = fmaxF(z.vol[lt], cut0x);
    double volu = detj * rr;
    double xmvis = vmu / volu;
    const double* T2[2] = {z.ti, z.tj};
    double cc[2];
#pragma unroll
    for (int d = 0; d < 2; d++) {
      const double* T = T2[d];
      int64_t l2 = lt + z.minc[d];
      double tx = mul_pow2<-1>(T[lt] + T[l2]);
      double ty = mul_pow2<-1>(T[lt + m] + T[l2 + m]);
      double tc2 = mul_pow2<-1>(sqrt(T[lt] * T[lt] + T[lt + m] * T[lt + m]) + sqrt(T[l2] * T[l2] + T[l2 + m] * T[l2 + m]));
      double qn = tx * u + ty * v;
      double vm = fabs(qn) + c * tc2;
      cc[d] = mul_pow2<1>(vm) + mul_pow2<2>(xmvis * tc2 * tc2);
    }
    a.coe[l + nd] = cc[0];
    a.coe[l + 2 * nd] = cc[1];
    a.coe[l + 4 * nd] = xid + mul_pow2<-1>(c1 * (cc[0] + cc[1]));
    return;
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
      double tx = mul_pow2<-1>(T[lt] + T[l2]);
      double ty = mul_pow2<-1>(T[lt + m] + T[l2 + m]);
      double tz = mul_pow2<-1>(T[lt + 2 * m] + T[l2 + 2 * m]);
      double tc2 = mul_pow2<-1>(sqrt(T[lt] * T[lt] + T[lt + m] * T[lt + m] + T[lt + 2 * m] * T[lt + 2 * m]) +
                         sqrt(T[l2] * T[l2] + T[l2 + m] * T[l2 + m] + T[l2 + 2 * m] * T[l2 + 2 * m]));
      double qn = tx * u + ty * v + tz * w;
      double vm = fabs(qn) + c * tc2;
      cc[d] = mul_pow2<1>(vm) + mul_pow2<2>(xmvis * tc2 * tc2);
    }
    c2 = cc[0]; c3 = cc[1]; c4 = cc[2];
  }
  a.coe[l + nd] = c2;
  a.coe[l + 2 * nd] = c3;
  a.coe[l + 3 * nd] = c4;
  a.coe[l + 4 * nd] = xid + mul_pow2<-1>(c1 * (c2 + c3 + c4));
}

__global__ void __launch_bounds__(256) coefficients(Zone z, CoeArgs a) {
  coefficients_at(z, a, (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
}

__device__ __forceinline__ int batch_zone_lu(const int64_t* bstart, int nz, int64_t b) {
  int lo = 0, hi = nz - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (bstart[mid] <= b) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__global__ void __launch_bounds__(256) coefficients_batch(const __grid_constant__ CoeBatch b) {
  const int m = batch_zone_lu(b.bstart, b.nz, blockIdx.x);
  coefficients_at(b.e[m].z, b.e[m].a, (int64_t)(blockIdx.x - b.bstart[m]) * blockDim.x + threadIdx.x);
}

cudaError_t launch_coefficients_batch(const CoeBatch& b, cudaStream_t st) {
  if (b.nz <= 0) return cudaSuccess;
  coefficients_batch<<<(unsigned)b.bstart[b.nz], 256, 0, st>>>(b);
  return cudaGetLastError();
}

cudaError_t launch_coefficients(const Zone& z, const CoeArgs& a, cudaStream_t st) {
  int64_t n = (a.hi[0] - a.lo[0] + 1) * (a.hi[1] - a.lo[1] + 1) * (a.hi[2] - a.lo[2] + 1);
  coefficients<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(z, a);
  return cudaGetLastError();
}

// ------------------------------------------------------- neighbour term
// b = B_d(W_nb) . dW_nb  (LU/lu_{i,j,k}_3dcart.for, lu_{i,j,k}_3dfull.for).
// (u,v,w,t) = neighbour state, cs = coe_{d+2}(nb) * signe with signe = +0.5
// in the lower sweep and -0.5 in the upper sweep.
template <int TYP, int D, typename T>
__device__ __forceinline__ void nb_term(T u, T v, T w, T t, T tcx, T tcy, T tcz, T cs,
                                        const T o[5], T b[5], T gam1, T gamm1, T gam2, T cp) {
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
    constexpr bool F32 = sizeof(T) == 4;
    tx = d == 0 ? (F32 ? T(z.ftc[0]) : T(z.tcx)) : T(0);
    ty = d == 1 ? (F32 ? T(z.ftc[1]) : T(z.tcy)) : T(0);
    tz = d == 2 ? (F32 ? T(z.ftc[2]) : T(z.tcz)) : T(0);
  } else if (TYP == Z2D) {   // lu_{i,j}_2d.for: two components
    const double* M = d == 0 ? z.ti : z.tj;
    const int64_t m = z.ndm;
    tx = T(0.5 * (M[ltb] + M[lta]));
    ty = T(0.5 * (M[ltb + m] + M[lta + m]));
    tz = T(0);
  } else {
    const double* M = d == 0 ? z.ti : (d == 1 ? z.tj : z.tk);
    const int64_t m = z.ndm;
    tx = T(0.5 * (M[ltb] + M[lta]));
    ty = T(0.5 * (M[ltb + m] + M[lta + m]));
    tz = T(0.5 * (M[ltb + 2 * m] + M[lta + 2 * m]));
  }
}

// Loads of values that other CTAs of the same launch write (increments, the
// updated state) bypass L1 (ld.global.cg): L1 is not coherent across SMs.
template <typename T> __device__ __forceinline__ T ldcg(const T* p) { return __ldcg(p); }


// ------------------------------------------------------ B-coefficient table
// The neighbour terms of a sweep are B_d(W_nb) . dW_nb.  B_d(W_nb) depends on
// the neighbour's state and metric only, which are known before the sweep,
// so a fully parallel pre-pass evaluates every entry (the same expressions
// in the same order as lu_{i,j,k}_*.for) and the sweep keeps only the
// matrix-vector product on its critical path.  Entries that carry the
// spectral radius (b11, b22, b33, b44, b55) are stored without it; the sweep
// adds coe_{d+2}(nb)*signe exactly as the reference expression does.
constexpr int NB_CART = 14;   // entries per direction, 3d cartesian zone
constexpr int NB_FULL = 25;   // entries per direction, 3d general zone
constexpr int QN_FULL = 23;   // general layout: qn (entries 0..22 are the B matrix)
template <int TYP> struct NBE { static constexpr int n = TYP == Z3DCART ? NB_CART : NB_FULL; };
// Entries that the sweeps only use as (entry + cs), cs = coe_{d+2}(nb) * signe:
// the diagonal of B and qn (the Spalart-Allmaras row).  The stored table
// holds them with the lower sweep's cs added (in place) and, after the NB
// entries, with the upper sweep's (-cs), so the sweeps do not add them.
constexpr int NS_CART = 3, NS_FULL = 5;
template <int TYP> struct NSE { static constexpr int n = TYP == Z3DCART ? NS_CART : NS_FULL; };
template <int TYP>
__host__ __device__ constexpr int sum_index(int d, int m) {
  // cartesian: direction 0 {b22, b33 = b44 = qn, b55}, 1 {b22 = b44 = qn, b33,
  // b55}, 2 {b22 = b33 = qn, b44, b55}; general: b22, b33, b44, b55, qn
  return TYP == Z3DCART ? (m == 2 ? 13 : (m == 0 ? 1 : (d == 0 ? 6 : (d == 1 ? 5 : 8))))
                        : (m == 0 ? 4 : (m == 1 ? 10 : (m == 2 ? 16 : (m == 3 ? 22 : QN_FULL))));
}
template <int TYP, int D>
__host__ __device__ constexpr int qn_slot() {   // the slot of qn + cs
  return TYP == Z3DCART ? (D == 0 ? 1 : 0) : 4;
}
// 2-d zones use the general entries with tz = 0 and w = 0 (lu_{i,j}_2d.for
// is lu_{i,j}_3dfull.for without the w / tz terms, which vanish exactly)

template <int TYP, typename T>
__device__ __forceinline__ void bentries(const Zone& z, int d, T u, T v, T w, T t, T tcx, T tcy,
                                         T tcz, T* e) {
  constexpr bool F32 = sizeof(T) == 4;   // FP32: the zone's FP32 constants, no conversion
  const T gam1 = F32 ? T(z.fgam) : T(z.gam), gamm1 = F32 ? T(z.fgm1) : T(z.gam - 1.),
          cp = F32 ? T(z.fcp) : T(z.gam * z.cv), gam2 = F32 ? T(z.fgm2) : T((z.gam - 1.) - 1.);
  T q2 = T(.5) * (u * u + v * v + w * w);
  T h = cp * t + q2;
  T ph2 = gamm1 * q2;
  if (TYP == Z3DCART) {
    if (d == 0) {
      T qn = tcx * u;
      e[0] = (tcx * ph2 - u * qn); e[1] = (qn - tcx * gam2 * u); e[2] = (-tcx * gamm1 * v);
      e[3] = (-tcx * gamm1 * w); e[4] = (-v * qn); e[5] = (tcx * v); e[6] = qn;
      e[7] = (-w * qn); e[8] = (tcx * w); e[9] = qn * (ph2 - h);
      e[10] = (tcx * h - gamm1 * u * qn); e[11] = (-gamm1 * v * qn);
      e[12] = (-gamm1 * w * qn); e[13] = (gam1 * qn);
    } else if (d == 1) {
      T qn = tcy * v;
      e[0] = (-u * qn); e[1] = qn; e[2] = tcy * u; e[3] = (tcy * ph2 - v * qn);
      e[4] = (-tcy * gamm1 * u); e[5] = (qn - tcy * gam2 * v); e[6] = (-tcy * gamm1 * w);
      e[7] = (-w * qn); e[8] = (tcy * w); e[9] = qn * (ph2 - h); e[10] = (-gamm1 * u * qn);
      e[11] = (tcy * h - gamm1 * v * qn); e[12] = (-gamm1 * w * qn); e[13] = (gam1 * qn);
    } else {
      T qn = tcz * w;
      e[0] = -u * qn; e[1] = qn; e[2] = tcz * u; e[3] = -v * qn; e[4] = tcz * v;
      e[5] = tcz * ph2 - w * qn; e[6] = -tcz * gamm1 * u; e[7] = -tcz * gamm1 * v;
      e[8] = (qn - tcz * gam2 * w); e[9] = qn * (ph2 - h); e[10] = -gamm1 * u * qn;
      e[11] = -gamm1 * v * qn; e[12] = tcz * h - gamm1 * w * qn; e[13] = gam1 * qn;
    }
  } else {
    T qn = tcx * u + tcy * v + tcz * w;
    e[0] = tcx; e[1] = tcy; e[2] = tcz;
    e[3] = (tcx * ph2 - u * qn); e[4] = (qn - tcx * gam2 * u);
    e[5] = (tcy * u - tcx * gamm1 * v); e[6] = (tcz * u - tcx * gamm1 * w); e[7] = tcx * gamm1;
    e[8] = (tcy * ph2 - v * qn); e[9] = (tcx * v - tcy * gamm1 * u);
    e[10] = (qn - tcy * gam2 * v); e[11] = (tcz * v - tcy * gamm1 * w); e[12] = tcy * gamm1;
    e[13] = (tcz * ph2 - w * qn); e[14] = (tcx * w - tcz * gamm1 * u);
    e[15] = (tcy * w - tcz * gamm1 * v); e[16] = (qn - tcz * gam2 * w); e[17] = tcz * gamm1;
    e[18] = qn * (ph2 - h); e[19] = (tcx * h - gamm1 * u * qn);
    e[20] = (tcy * h - gamm1 * v * qn); e[21] = (tcz * h - gamm1 * w * qn); e[22] = (gam1 * qn);
    e[QN_FULL] = qn;   // read by the Spalart-Allmaras row only
  }
}


// b = B . o from the entries e (cs = coe_{d+2}(nb) * signe).  MODE 0: raw
// entries (the sums formed here); 1: a stored table, lower sweep (sums in
// place); 2: a stored table, upper sweep (sums after the NB entries).
template <int TYP, int D, typename T, int MODE>
__device__ __forceinline__ T bsum(const T* e, T cs, int idx, int slot) {
  return MODE == 0 ? e[idx] + cs : (MODE == 1 ? e[idx] : e[NBE<TYP>::n + slot]);
}
template <int TYP, int D, typename T, int MODE>
__device__ __forceinline__ void bmatvec(const Zone& z, const T* e, T cs, const T o[5], T b[5]) {
  // cartesian: tc_D (gam - 1), a zone constant (FP64: evaluated once on the
  // host; FP32: the product of the two FP32 roundings)
  constexpr bool F32 = sizeof(T) == 4;
  auto tcg = [&](double) -> T { return F32 ? T(z.ftc[D]) * T(z.fgm1) : T(z.ctcg[D]); };
  auto S = [&](int m) { return bsum<TYP, D, T, MODE>(e, cs, sum_index<TYP>(D, m), m); };
  if (TYP == Z3DCART) {
    if (D == 0) {
      const T tcx = F32 ? T(z.ftc[0]) : T(z.tcx), b25 = tcg(z.tcx);
      const T s22 = S(0), s33 = S(1), s55 = S(2);
      b[0] = cs * o[0] + tcx * o[1];
      b[1] = e[0] * o[0] + s22 * o[1] + e[2] * o[2] + e[3] * o[3] + b25 * o[4];
      b[2] = e[4] * o[0] + e[5] * o[1] + s33 * o[2];
      b[3] = e[7] * o[0] + e[8] * o[1] + s33 * o[3];
      b[4] = e[9] * o[0] + e[10] * o[1] + e[11] * o[2] + e[12] * o[3] + s55 * o[4];
    } else if (D == 1) {
      const T tcy = F32 ? T(z.ftc[1]) : T(z.tcy), b35 = tcg(z.tcy);
      const T s22 = S(0), s33 = S(1), s55 = S(2);
      b[0] = cs * o[0] + tcy * o[2];
      b[1] = e[0] * o[0] + s22 * o[1] + e[2] * o[2];
      b[2] = e[3] * o[0] + e[4] * o[1] + s33 * o[2] + e[6] * o[3] + b35 * o[4];
      b[3] = e[7] * o[0] + e[8] * o[2] + s22 * o[3];
      b[4] = e[9] * o[0] + e[10] * o[1] + e[11] * o[2] + e[12] * o[3] + s55 * o[4];
    } else {
      const T tcz = F32 ? T(z.ftc[2]) : T(z.tcz), b45 = tcg(z.tcz);
      const T s22 = S(0), s44 = S(1), s55 = S(2);
      b[0] = cs * o[0] + tcz * o[3];
      b[1] = e[0] * o[0] + s22 * o[1] + e[2] * o[3];
      b[2] = e[3] * o[0] + s22 * o[2] + e[4] * o[3];
      b[3] = e[5] * o[0] + e[6] * o[1] + e[7] * o[2] + s44 * o[3] + b45 * o[4];
      b[4] = e[9] * o[0] + e[10] * o[1] + e[11] * o[2] + e[12] * o[3] + s55 * o[4];
    }
  } else if (TYP == Z2D) {   // lu_{i,j}_2d.for: no w row
    b[0] = cs * o[0] + e[0] * o[1] + e[1] * o[2];
    b[1] = e[3] * o[0] + S(0) * o[1] + e[5] * o[2] + e[7] * o[4];
    b[2] = e[8] * o[0] + e[9] * o[1] + S(1) * o[2] + e[12] * o[4];
    b[3] = T(0);
    b[4] = e[18] * o[0] + e[19] * o[1] + e[20] * o[2] + S(3) * o[4];
  } else {
    b[0] = cs * o[0] + e[0] * o[1] + e[1] * o[2] + e[2] * o[3];
    b[1] = e[3] * o[0] + S(0) * o[1] + e[5] * o[2] + e[6] * o[3] + e[7] * o[4];
    b[2] = e[8] * o[0] + e[9] * o[1] + S(1) * o[2] + e[11] * o[3] + e[12] * o[4];
    b[3] = e[13] * o[0] + e[14] * o[1] + e[15] * o[2] + S(2) * o[3] + e[17] * o[4];
    b[4] = e[18] * o[0] + e[19] * o[1] + e[20] * o[2] + e[21] * o[3] + S(3) * o[4];
  }
}

template <int D> struct DirT { static constexpr int value = D; };

// ------------------------------------------------------- plane-ordered data
// The sweeps visit cells hyperplane by hyperplane, which has no locality in
// the natural (i,j,k) layout.  Every value the sweeps read is therefore
// gathered once per solve into hyperplane order (index g = position in the
// plane table), as one contiguous record per cell: a warp working on
// consecutive cells of a plane, and on their neighbours in the previous
// plane, then reads a few contiguous spans instead of one scattered word per
// array (which thrashed the TLB and sector caches).
//   rec[g] : coe1 / 2, 1/coe5, coe5, coe6 (SA), coe_{2..4} / 2, W^p (5), B entries
//            (3 x NBS: NB entries with the lower sweep's sums, the upper sums)
//   dio[g] : residual in / increment out (5 words, 6 with SA, stride 6)
//   nst[g] : in-place upper sweep: W^{p+1} u, v, w, T (stride 4)
template <int TYP, typename T> struct Rec {
  // FP32 sweeps in cartesian zones rebuild B from the neighbour's state
  // instead of reading a stored table: the same float arithmetic on the same
  // float inputs as the pre-pass, so the same values, in 12 words a cell.
  static constexpr bool HAS_B = !(TYP == Z3DCART && sizeof(T) == 4);
  static constexpr int NB = NBE<TYP>::n;
  static constexpr int NBS = NB + NSE<TYP>::n;   // per direction: entries, then upper sums
  static constexpr int COE1 = 0, DIAG = 1, COE5 = 2, COE6 = 3, COEN = 4, ST = 7, B = 12;
  static constexpr int SIZE = HAS_B ? ((B + 3 * NBS) + 3) / 4 * 4 : B;   // whole 16-byte vectors
};
constexpr int DIO = 6;

template <typename T>
struct PlaneData {
  T* rec;              // [G][Rec::SIZE]
  T* dio;              // [G][DIO]
  T* nst;              // [G][4]
  const int32_t* nbl;  // [3][G] plane index of the i-1 / j-1 / k-1 neighbour, -1 if none
  const int32_t* nbu;  // [3][G] plane index of the i+1 / j+1 / k+1 neighbour, -1 if none
  const uint32_t* cells;  // [G] packed (i, j, k) of each plane index
  const int64_t* plane;   // plane s = [plane[s], plane[s+1])
  int64_t G;
  int64_t smax;           // last plane
  const int32_t* zid;     // [G] zone of each plane index (several zones)
  const LuZone* zt;       // zone table
};

__device__ __forceinline__ void unpack(uint32_t c, int64_t& ii, int64_t& jj, int64_t& kk) {
  ii = c & 2047u; jj = (c >> 11) & 2047u; kk = c >> 22;
}

// neighbour tables of a group (static): the neighbours of a cell are in
// its own zone
__global__ void __launch_bounds__(256) lu_neighbours(const LuZone* __restrict__ zt,
                                                     const int32_t* __restrict__ zid,
                                                     const uint32_t* __restrict__ cells,
                                                     int32_t* __restrict__ nbl,
                                                     int32_t* __restrict__ nbu, int64_t G) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= G) return;
  const LuZone& Z = zt[zid[g]];
  const Zone& z = Z.z;
  int64_t ii, jj, kk;
  unpack(cells[g], ii, jj, kk);
  const int64_t l = inddm(z, ii + 1, jj + 1, kk + 1);
  const int64_t idx[3] = {ii, jj, kk}, n[3] = {z.ni, z.nj, z.nk};
#pragma unroll
  for (int d = 0; d < 3; d++) {
    nbl[d * G + g] = idx[d] > 0 ? Z.f.posmap[l - z.inc[d]] : -1;
    nbu[d * G + g] = idx[d] < n[d] - 1 ? Z.f.posmap[l + z.inc[d]] : -1;
  }
}

// Record stores: whole 16-byte vectors, so that a thread fills its record
// with SIZE/2 (FP64) or SIZE/4 (FP32) stores instead of SIZE scalar ones.
template <int N>
__device__ __forceinline__ void store_rec(double* dst, const double (&r)[N]) {
  static_assert(N % 2 == 0, "FP64 records are whole double2 vectors");
  double2* d = reinterpret_cast<double2*>(dst);
#pragma unroll
  for (int m = 0; m < N / 2; m++) d[m] = make_double2(r[2 * m], r[2 * m + 1]);
}
template <int N>
__device__ __forceinline__ void store_rec(float* dst, const float (&r)[N]) {
  static_assert(N % 4 == 0, "FP32 records are whole float4 vectors");
  float4* d = reinterpret_cast<float4*>(dst);
#pragma unroll
  for (int m = 0; m < N / 4; m++) d[m] = make_float4(r[4 * m], r[4 * m + 1], r[4 * m + 2], r[4 * m + 3]);
}
template <int NV>
__device__ __forceinline__ void store_dio(double* dst, const double (&x)[NV]) {
  double2* d = reinterpret_cast<double2*>(dst);   // DIO = 6 words: 48-byte slots
  d[0] = make_double2(x[0], x[1]); d[1] = make_double2(x[2], x[3]);
  d[2] = make_double2(x[4], NV == 6 ? x[NV - 1] : 0.);
}
template <int NV>
__device__ __forceinline__ void store_dio(float* dst, const float (&x)[NV]) {
  float2* d = reinterpret_cast<float2*>(dst);     // 24-byte slots
  d[0] = make_float2(x[0], x[1]); d[1] = make_float2(x[2], x[3]);
  d[2] = make_float2(x[4], NV == 6 ? x[NV - 1] : 0.f);
}

// Per-solve gather into plane-ordered records + B entries (fully parallel).
// A CTA takes a tile of GT_I x GT_J cells (i, j) at one k.  Reads of
// din / coe / W^p run along i (coalesced).  In the plane table, cells of
// one plane and one k follow each other by increasing j, so the cells of a
// tile anti-diagonal (i + j constant) have consecutive plane indices: the
// CTA stages its records in shared memory ordered by anti-diagonal and then
// writes each anti-diagonal as one contiguous span of records.
constexpr int GT_I = 16, GT_J = 8, GT_N = GT_I * GT_J;

template <int TYP, typename T>
struct GatherSmem {
  static constexpr int CH = Rec<TYP, T>::SIZE * (int)sizeof(T) / 16;   // 16-byte chunks per record
  static constexpr int STRIDE = (CH | 1) * (16 / (int)sizeof(T));   // odd chunk stride: no bank conflicts
  static constexpr size_t bytes = sizeof(T) * (size_t)GT_N * (STRIDE + DIO) + 4 * GT_N;
};

// slot of tile cell (ti, tj): anti-diagonal a = ti + tj first, then tj
__device__ __forceinline__ int tile_slot(int ti, int tj) {
  const int a = ti + tj;
  int q = 0;
  for (int b = 0; b < a; b++) q += min(min(b + 1, GT_J), GT_I + GT_J - 1 - b);
  return q + tj - max(0, a - (GT_I - 1));
}

template <typename T> struct Vec2;
template <> struct Vec2<double> { using t = double2; };
template <> struct Vec2<float> { using t = float2; };

template <int TYP, typename T, int NV>
__global__ void __launch_bounds__(GT_N) lu_gather(Zone z, LuFields f, PlaneData<T> p) {
  using R = Rec<TYP, T>;
  using S = GatherSmem<TYP, T>;
  extern __shared__ __align__(16) unsigned char smem[];
  T* s_rec = reinterpret_cast<T*>(smem);
  T* s_dio = s_rec + GT_N * S::STRIDE;
  int32_t* s_g = reinterpret_cast<int32_t*>(s_dio + GT_N * DIO);
  const int ti = threadIdx.x % GT_I, tj = threadIdx.x / GT_I;
  const int64_t ii = (int64_t)blockIdx.x * GT_I + ti, jj = (int64_t)blockIdx.y * GT_J + tj;
  const int64_t kk = blockIdx.z;
  const int q = tile_slot(ti, tj);
  if (ii < z.ni && jj < z.nj) {
    const int64_t l = inddm(z, ii + 1, jj + 1, kk + 1);
    const int64_t lt = TYP == Z3DCART ? 0 : indmtr(z, ii + 1, jj + 1, kk + 1);
    const int64_t nd = z.nd;
    T x[NV];
#pragma unroll
    for (int v = 0; v < NV; v++) x[v] = T(f.din[l + v * nd]);
    T r[R::SIZE];
    const T c5 = T(f.coe[l + 4 * nd]);
    // coe1 and coe_{d+2} halved here, off the sweeps' critical path: the
    // sweeps use coe * (+-0.5), and x * -0.5 = -(x * 0.5) exactly
    r[R::COE1] = T(f.coe[l]) * T(0.5);
    r[R::DIAG] = T(1.) / c5;
    r[R::COE5] = c5;
    r[R::COE6] = NV == 6 ? T(f.coe[l + 5 * nd]) : T(0);
#pragma unroll
    for (int d = 0; d < 3; d++) r[R::COEN + d] = T(f.coe[l + (d + 1) * nd]) * T(0.5);
#pragma unroll
    for (int v = 0; v < 5; v++) r[R::ST + v] = T(f.rop_old[l + v * nd]);
#pragma unroll
    for (int m = R::B; m < R::SIZE; m++) r[m] = T(0);   // padding and unused entries
    if (R::HAS_B) {
#pragma unroll
      for (int d = 0; d < 3; d++) {
        T tx, ty, tz;
        nb_normal<TYP, T>(z, d, lt, lt + z.minc[d], tx, ty, tz);
        T* e = r + R::B + d * R::NBS;
        bentries<TYP, T>(z, d, r[R::ST + 1], r[R::ST + 2], r[R::ST + 3], r[R::ST + 4], tx, ty, tz, e);
        // the sums the sweeps use: entry + cs (lower), entry + (-cs) (upper)
        const T cs = r[R::COEN + d];
#pragma unroll
        for (int m = 0; m < NSE<TYP>::n; m++) {
          const int idx = sum_index<TYP>(d, m);
          e[R::NB + m] = e[idx] + (-cs);
          e[idx] = e[idx] + cs;
        }
      }
    }
    s_g[q] = f.posmap[l];
    store_rec(s_rec + q * S::STRIDE, r);
    store_dio(s_dio + q * DIO, x);
  } else {
    s_g[q] = -1;
  }
  __syncthreads();
  for (int c = threadIdx.x; c < GT_N * S::CH; c += GT_N) {
    const int qq = c / S::CH, m = c - qq * S::CH;
    const int32_t g = s_g[qq];
    if (g < 0) continue;
    reinterpret_cast<int4*>(p.rec + (int64_t)g * R::SIZE)[m] =
        reinterpret_cast<const int4*>(s_rec + qq * S::STRIDE)[m];
  }
  using V2 = typename Vec2<T>::t;
  for (int c = threadIdx.x; c < GT_N * (DIO / 2); c += GT_N) {
    const int qq = c / (DIO / 2), m = c - qq * (DIO / 2);
    const int32_t g = s_g[qq];
    if (g < 0) continue;
    reinterpret_cast<V2*>(p.dio + (int64_t)g * DIO)[m] =
        reinterpret_cast<const V2*>(s_dio + qq * DIO)[m];
  }
}

// ---------------------------------------------------------------- cells
// Precision T: double for the plain FP64 path; float for the mixed path
// (FP32 sweeps and approximate Jacobians; the Newton update stays FP64).
template <int NV, typename T>
__device__ __forceinline__ void load_dio(const T* __restrict__ dio, int64_t g, T o[NV]) {
  const T* q = dio + g * DIO;
#pragma unroll
  for (int v = 0; v < NV; v++) o[v] = __ldcg(q + v);
}

// mjr_newton_SA.for: ro nutilde updated, nutilde clipped to
// [0, ratiom nu_lam(T^{p+1})]; r_1 = 1 / ro^{p+1}, t_new = T^{p+1}
__device__ __forceinline__ double newton_sa(const Zone& z, double ro_old, double nu_old, double d6,
                                            double r_1, double t_new) {
  double anulam = sa_mulam(z, t_new);
  anulam = anulam * r_1 * z.ratiom;
  double t6 = (ro_old * nu_old + d6) * r_1;
  t6 = fminF(t6, anulam);
  return fmaxF(t6, 0.);
}

// mjr_newton.for: W^{p+1} = prim(cons(W^p) + dW) in precision T; cvinv =
// 1/cv in precision T (the FP64 quotient is the host's: the same IEEE value)
template <typename T, bool TWO_D = false>
__device__ __forceinline__ void newton(T cv, T cvinv, T ro, T u, T v, T w, T tt, const T d[5],
                                       T n[5]) {
  const T cvinv2 = T(0.5) * cvinv;
  n[0] = ro + d[0];
  const T r_1 = T(1.) / n[0];
  n[1] = (ro * u + d[1]) * r_1;
  n[2] = (ro * v + d[2]) * r_1;
  if (TWO_D) {  // mjr_newton.for 2-d branch: w = 0
    n[3] = T(0);
    const T roe_old = ro * (cv * tt + T(0.5) * (u * u + v * v));
    n[4] = (roe_old + d[4]) * r_1 * cvinv - cvinv2 * (n[1] * n[1] + n[2] * n[2]);
    return;
  }
  n[3] = (ro * w + d[3]) * r_1;
  const T roe_old = ro * (cv * tt + T(0.5) * (u * u + v * v + w * w));
  n[4] = (roe_old + d[4]) * r_1 * cvinv - cvinv2 * (n[1] * n[1] + n[2] * n[2] + n[3] * n[3]);
}

// ------------------------------------------------------------ cell operands
// Everything a cell of a sweep reads except what the previous hyperplane
// produces (the neighbours' increments and, in place, the k+1 neighbour's
// new state).  FP32 sweeps load these for the next cell between arriving at
// the grid barrier and waiting on it, so only the increments' loads stay
// between two hyperplanes; without a stored B table (FP32, cartesian) the
// neighbours' states are held instead (3 x 4 values).
template <int TYP, typename T, int NV = 5>
struct CellOps {
  static constexpr bool HOLD_W = !Rec<TYP, T>::HAS_B;
  static constexpr int NW = HOLD_W ? 4 : 1;
  int32_t n[3];   // neighbour plane indices (-1: none)
  T x[NV];        // lower: residual; upper: lower result x coe5 (lu_d.for; x coe6 for SA)
  T xal, diag;
  T c6;           // SA: coe6 of the cell (its sixth diagonal, divided by)
  T cs[3];        // coe_{d+2}(neighbour) x (+-1/2)
  T wn[3][NW];    // neighbours' u, v, w, T (no stored B table)
  T st[5];        // upper: W^p of the cell (in-place Newton)
};

// upper sweep: the cell's own lower result times coe5 (lu_d.for; x coe6 for SA)
template <int TYP, typename T, int NV>
__device__ __forceinline__ void load_x_upper(const PlaneData<T>& p, int64_t g, CellOps<TYP, T, NV>& o) {
  using R = Rec<TYP, T>;
  load_dio<NV>(p.dio, g, o.x);
  const T dg = p.rec[g * R::SIZE + R::COE5];
#pragma unroll
  for (int v = 0; v < 5; v++) o.x[v] = o.x[v] * dg;
  if (NV == 6) o.x[NV - 1] = o.x[NV - 1] * o.c6;   // lu_d_SA.for
}

// with_x false: everything but the upper sweep's own lower result (which
// the caller loads after waiting for it, load_x_upper)
template <int TYP, typename T, bool UPPER, int NV>
__device__ __forceinline__ void load_ops(const PlaneData<T>& p, bool inplace, int64_t g,
                                         CellOps<TYP, T, NV>& o, bool with_x = true) {
  using R = Rec<TYP, T>;
  const T* me = p.rec + g * R::SIZE;
  const int32_t* nbt = UPPER ? p.nbu : p.nbl;
#pragma unroll
  for (int d = 0; d < 3; d++) o.n[d] = nbt[d * p.G + g];
  if (!UPPER) load_dio<NV>(p.dio, g, o.x);
  if (NV == 6) o.c6 = me[R::COE6];
  if (UPPER) {
    if (with_x) load_x_upper<TYP, T, NV>(p, g, o);
    o.xal = -me[R::COE1];
#pragma unroll
    for (int v = 0; v < 5; v++) o.st[v] = me[R::ST + v];
  } else {
    o.xal = me[R::COE1];
  }
  o.diag = me[R::DIAG];
#pragma unroll
  for (int d = 0; d < 3; d++) {
    if (o.n[d] < 0) continue;
    const T* rn = p.rec + (int64_t)o.n[d] * R::SIZE;
    o.cs[d] = UPPER ? -rn[R::COEN + d] : rn[R::COEN + d];
    if (CellOps<TYP, T, NV>::HOLD_W && !(UPPER && d == 2 && inplace)) {
#pragma unroll
      for (int m = 0; m < CellOps<TYP, T, NV>::NW; m++) o.wn[d][m] = rn[R::ST + 1 + m];
    }
  }
}

// invlu_l.for / invlu_u.for for one cell: out = (x + sum_d B_d(nb).out_nb *
// (+-coe1/2)) / coe5 in the reference's direction order; in place (upper
// sweep of a sub-iteration that updates W^{p+1} over W^p) the k+1 term uses
// the neighbour's new state and the cell's own Newton update follows.
template <int TYP, typename T, bool UPPER, int NV>
__device__ __forceinline__ void run_cell(const Zone& z, const PlaneData<T>& p, const LuFields& f,
                                         int64_t g, const CellOps<TYP, T, NV>& o) {
  using R = Rec<TYP, T>;
  using C = CellOps<TYP, T, NV>;
  constexpr int NB = R::NB;
  T x[NV], od[NV], b[5];
#pragma unroll
  for (int v = 0; v < NV; v++) x[v] = o.x[v];
  auto term = [&](auto dc, bool fresh) {
    constexpr int D = decltype(dc)::value;
    const int32_t n = o.n[D];
    if (n < 0) return;
    load_dio<NV>(p.dio, n, od);
    T qcs = T(0);   // SA row: qn + cs of the neighbour
    if (fresh) {  // k+1 neighbour updated in place: B from its new state
      T e[NB];
      const T* q = p.nst + (int64_t)n * 4;
      T u = __ldcg(q), vv = __ldcg(q + 1), w = __ldcg(q + 2), t = __ldcg(q + 3);
      T tx, ty, tz;
      if (TYP == Z3DCART) {
        tx = T(0); ty = T(0); tz = sizeof(T) == 4 ? T(z.ftc[2]) : T(z.tcz);
      } else {
        int64_t ii, jj, kk;
        unpack(p.cells[n], ii, jj, kk);
        const int64_t lt = indmtr(z, ii + 1, jj + 1, kk + 1);
        nb_normal<TYP, T>(z, D, lt, lt + z.minc[D], tx, ty, tz);
      }
      bentries<TYP, T>(z, D, u, vv, w, t, tx, ty, tz, e);
      bmatvec<TYP, D, T, 0>(z, e, o.cs[D], od, b);
      if (NV == 6) qcs = bsum<TYP, D, T, 0>(e, o.cs[D], sum_index<TYP>(D, qn_slot<TYP, D>()), 0);
    } else if (C::HOLD_W) {  // cartesian: B from the held state
      T e[NB];
      T tx, ty, tz;
      nb_normal<TYP, T>(z, D, 0, 0, tx, ty, tz);
      bentries<TYP, T>(z, D, o.wn[D][0], o.wn[D][C::NW > 1 ? 1 : 0],
                       o.wn[D][C::NW > 2 ? 2 : 0], o.wn[D][C::NW > 3 ? 3 : 0],
                       tx, ty, tz, e);
      bmatvec<TYP, D, T, 0>(z, e, o.cs[D], od, b);
      if (NV == 6) qcs = bsum<TYP, D, T, 0>(e, o.cs[D], sum_index<TYP>(D, qn_slot<TYP, D>()), 0);
    } else {
      constexpr int MODE = UPPER ? 2 : 1;
      const T* e = p.rec + (int64_t)n * R::SIZE + R::B + D * R::NBS;
      bmatvec<TYP, D, T, MODE>(z, e, o.cs[D], od, b);
      if (NV == 6)
        qcs = bsum<TYP, D, T, MODE>(e, o.cs[D], sum_index<TYP>(D, qn_slot<TYP, D>()), qn_slot<TYP, D>());
    }
#pragma unroll
    for (int v = 0; v < 5; v++) x[v] = x[v] + b[v] * o.xal;
    if (NV == 6) {   // lu_*_SA.for: b6 = (qn + coe_{d+2}(nb) signe) dW6_nb
      const T b6 = qcs * od[NV - 1];
      x[NV - 1] = x[NV - 1] + b6 * o.xal;
    }
  };
  if (UPPER) {                 // invlu_u.for: k, then j, then i
    term(DirT<2>{}, f.inplace != 0);
    term(DirT<1>{}, false);
    term(DirT<0>{}, false);
  } else if (TYP == Z3DCART) { // invlu_l.for cartesian section: j, then k, then i
    term(DirT<1>{}, false);
    term(DirT<2>{}, false);
    term(DirT<0>{}, false);
  } else {                     // general section: k, then j, then i
    term(DirT<2>{}, false);
    term(DirT<1>{}, false);
    term(DirT<0>{}, false);
  }
#pragma unroll
  for (int v = 0; v < 5; v++) x[v] = x[v] * o.diag;
  if (NV == 6) x[NV - 1] = x[NV - 1] / o.c6;   // lu_dinv_SA.for
  T* io = p.dio + g * DIO;
#pragma unroll
  for (int v = 0; v < NV; v++) io[v] = x[v];
  if (!UPPER || !f.inplace) return;  // otherwise the Newton update runs after the sweep
  // in place: the k-1 neighbour needs this cell's new state in the next plane
  T nw[5];
  const T cvinv = sizeof(T) == 8 ? T(z.cvinv) : T(z.fcvinv);
  newton<T, TYP == Z2D>(sizeof(T) == 8 ? T(z.cv) : T(z.fcv), cvinv, o.st[0], o.st[1], o.st[2], o.st[3],
                        o.st[4], x, nw);
  T* q = p.nst + g * 4;
#pragma unroll
  for (int v = 0; v < 4; v++) q[v] = nw[v + 1];
  if (sizeof(T) == 8) {  // FP64 path: this is the update itself
    int64_t ii, jj, kk;
    unpack(p.cells[g], ii, jj, kk);
    const int64_t l = inddm(z, ii + 1, jj + 1, kk + 1);
#pragma unroll
    for (int v = 0; v < 5; v++) f.rop_new[l + v * z.nd] = double(nw[v]);
    if (NV == 6)
      f.rop_new[l + 5 * z.nd] = newton_sa(z, double(o.st[0]), f.rop_old[l + 5 * z.nd],
                                          double(x[NV - 1]), 1. / double(nw[0]), double(nw[4]));
  }
}

// ------------------------------------------------------- grid barrier
// Cooperative launch guarantees that every CTA is resident.  One monotone
// counter per launch (zeroed before it): round r is complete when the
// counter reaches (r + 1) * gridDim.x.  Arrive (after the CTA's writes) is a
// release add by thread 0; wait is an acquire poll by the CTA's last thread
// (the one least likely to own a cell of the next plane, so its poll does
// not queue behind operand loads) followed by a CTA barrier, so the CTA can
// do independent work in between.  The wait is
// bounded: past 2^24 polls it sets the error word and the kernel returns;
// the host reports FGB_ERR_DEVICE.
struct GridBar { unsigned int* count; int* err; long long limit; unsigned int skew; };

__device__ __forceinline__ void bar_arrive(const GridBar& g) {
  __syncthreads();
  if (threadIdx.x == 0)
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(g.count), "r"(1u) : "memory");
}

__device__ __forceinline__ bool bar_wait(const GridBar& g, unsigned int target) {
  if (threadIdx.x == blockDim.x - 1) {
    long long spins = 0;
    while (true) {
      unsigned int cur;
      asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(cur) : "l"(g.count) : "memory");
      if ((int)(cur - target) >= 0) break;
      if ((++spins & 63) == 0) {
        if (*(volatile int*)g.err) break;
        if (spins > g.limit) { atomicExch(g.err, 1); break; }
      }
    }
  }
  __syncthreads();
  return *(volatile int*)g.err == 0;
}

// L2 prefetch of everything plane s keeps in plane order (records,
// increments, neighbour tables): contiguous spans, spread over the grid.
__device__ __forceinline__ void prefetch_span_l2(const void* base, int64_t bytes) {
  const char* b = static_cast<const char*>(base);
  const int64_t nt = (int64_t)gridDim.x * blockDim.x;
  for (int64_t o = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * 128; o < bytes; o += nt * 128)
    asm volatile("prefetch.global.L2 [%0];" ::"l"(b + o));
}

template <int TYP, typename T>
__device__ __forceinline__ void prefetch_plane(const PlaneData<T>& p, int64_t s, bool upper) {
  const int64_t c0 = p.plane[s], n = p.plane[s + 1] - c0;
  prefetch_span_l2(p.rec + c0 * Rec<TYP, T>::SIZE, n * Rec<TYP, T>::SIZE * (int64_t)sizeof(T));
  prefetch_span_l2(p.dio + c0 * DIO, n * DIO * (int64_t)sizeof(T));
  const int32_t* nb = upper ? p.nbu : p.nbl;
#pragma unroll
  for (int d = 0; d < 3; d++) prefetch_span_l2(nb + d * p.G + c0, n * 4);
}

// Cells of plane s spread over every CTA: cell c of the plane goes to CTA
// c mod gridDim, so each CTA's share is packed into its first warps.  With
// PRE, a thread's first cell of the plane comes with its operands already
// loaded (FP32 sweeps: they are latency-bound); FP64 sweeps, bound by the
// FP64 pipe, load them here.
// MULTI: the cells of a plane belong to several zones, whose descriptor and
// fields come from the group's zone table
template <int TYP, typename T, bool UPPER, int NV, bool MULTI>
__device__ __forceinline__ void run_cell_of(const Zone& z, const PlaneData<T>& p, const LuFields& f,
                                            int64_t g, const CellOps<TYP, T, NV>& o) {
  if (MULTI) {
    const LuZone& Z = p.zt[p.zid[g]];
    run_cell<TYP, T, UPPER, NV>(Z.z, p, Z.f, g, o);
  } else {
    run_cell<TYP, T, UPPER, NV>(z, p, f, g, o);
  }
}

template <int TYP, typename T, bool UPPER, bool PRE, int NV, bool MULTI>
__device__ __forceinline__ void do_plane(const Zone& z, const PlaneData<T>& p, const LuFields& f,
                                         int64_t s, CellOps<TYP, T, NV>& first) {
  const int64_t c0 = p.plane[s], n = p.plane[s + 1] - c0;
  int64_t c = (int64_t)threadIdx.x * gridDim.x + blockIdx.x;
  if (c >= n) return;
  if (!PRE) load_ops<TYP, T, UPPER, NV>(p, f.inplace != 0, c0 + c, first);
  run_cell_of<TYP, T, UPPER, NV, MULTI>(z, p, f, c0 + c, first);
  for (c += (int64_t)gridDim.x * blockDim.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
    CellOps<TYP, T, NV> o;
    load_ops<TYP, T, UPPER, NV>(p, f.inplace != 0, c0 + c, o);
    run_cell_of<TYP, T, UPPER, NV, MULTI>(z, p, f, c0 + c, o);
  }
}

template <int TYP, typename T, bool UPPER, int NV>
__device__ __forceinline__ void load_first(const PlaneData<T>& p, const LuFields& f, int64_t s,
                                           CellOps<TYP, T, NV>& o) {
  const int64_t c0 = p.plane[s], n = p.plane[s + 1] - c0;
  const int64_t c = (int64_t)threadIdx.x * gridDim.x + blockIdx.x;
  if (c < n) load_ops<TYP, T, UPPER, NV>(p, f.inplace != 0, c0 + c, o);
}

template <typename T> struct LuThreads { static constexpr int n = 512; };

template <int TYP, typename T, int NV, bool MULTI>
__global__ void __launch_bounds__(LuThreads<T>::n, 1)
    lusgs_persistent(Zone z, PlaneData<T> p, LuFields f, GridBar gb) {
  const int64_t smax = p.smax;
  // traversal step t: lower planes 0..smax, then upper planes smax..0
  auto plane_of = [&](int64_t t) { return t <= smax ? t : 2 * smax + 1 - t; };
  const int64_t nsteps = 2 * smax + 2;
  prefetch_plane<TYP, T>(p, 0, false);
  if (nsteps > 1) prefetch_plane<TYP, T>(p, plane_of(1), 1 > smax);
  constexpr bool PRE = sizeof(T) == 4;
  CellOps<TYP, T, NV> o;
  if (PRE) load_first<TYP, T, false, NV>(p, f, 0, o);
  unsigned int round = 0;
  for (int64_t t = 0; t < nsteps; t++) {
    const int64_t s = plane_of(t);
    if (t <= smax) do_plane<TYP, T, false, PRE, NV, MULTI>(z, p, f, s, o);
    else do_plane<TYP, T, true, PRE, NV, MULTI>(z, p, f, s, o);
    if (t == nsteps - 1) break;
    bar_arrive(gb);
    if (t + 2 < nsteps) prefetch_plane<TYP, T>(p, plane_of(t + 2), t + 2 > smax);
    if (PRE) {
      if (t + 1 <= smax) load_first<TYP, T, false, NV>(p, f, plane_of(t + 1), o);
      else load_first<TYP, T, true, NV>(p, f, plane_of(t + 1), o);
    }
    round++;
    if (!bar_wait(gb, round * gridDim.x + gb.skew)) return;
  }
}

// ------------------------------------------------------- dataflow sweep
// Lower and upper sweeps as one launch of independent warps, with no grid
// barrier.  Each hyperplane's cells (contiguous in plane order) are cut into
// chunks of 32; a warp takes chunks in order from a global ticket counter
// (all lower chunks by increasing plane, then all upper chunks by decreasing
// plane), waits until the chunks holding its cells' neighbours in the
// previous plane of the sweep have published their completion mark, sweeps
// its 32 cells (one per lane, the cell code of the other schedules) and
// publishes its own mark.  A warp only ever waits on chunks with smaller
// tickets, which running warps already hold, so the launch cannot deadlock
// whatever the number of resident CTAs.  Its dependencies are the chunks of
// the previous plane that hold its cells' neighbours, as at most two ranges
// of chunk indices per sweep (the i-1 / j-1 and the k-1 neighbours); a
// plane starts as soon as the
// cells it needs are done instead of after the whole previous plane, and the
// FP64 pipes stay busy across plane boundaries.  An upper chunk also waits on
// its own lower mark (its cells' lower results).  Marks are 2 e + 1 (lower)
// and 2 e + 2 (upper) of the solve's epoch e, so the flags are never
// cleared.  Waits are bounded: past poll_limit polls a lane sets the error
// word and every warp returns.
constexpr int FLOW_CHUNK = 32;
constexpr int FLOW_THREADS = 256;

__device__ __forceinline__ bool flow_poll(const FlowArgs& a, int64_t c, int mark) {
  long long spins = 0;
  while (true) {
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(a.flag + c) : "memory");
    if (v >= mark) return true;
    if ((++spins & 63) == 0) {
      if (*(volatile int*)a.err) return false;
      if (spins > a.poll_limit) { atomicExch(a.err, 2); return false; }
    }
  }
}

// L2 prefetch of what a chunk reads that no earlier plane produced (its
// cells' records, residuals / lower results and neighbour indices), issued
// before the dependency wait: those lines are cold in L2 (the records are
// written by the gather and read once per sweep), so without it the DRAM
// latency lands between the wait and the cell work.  Lane m takes every
// 32nd 128-byte line of each span.
__device__ __forceinline__ void prefetch_span_chunk(const void* base, int64_t bytes, int lane) {
  const char* b = static_cast<const char*>(base);
  const int64_t a0 = (int64_t)((uintptr_t)b & 127u);
  for (int64_t o = (int64_t)lane * 128 - a0; o < bytes; o += 32 * 128)
    asm volatile("prefetch.global.L2 [%0];" ::"l"(b + (o < 0 ? 0 : o)));
}
template <int TYP, typename T>
__device__ __forceinline__ void prefetch_chunk(const PlaneData<T>& p, int64_t g0, int64_t n,
                                               bool upper, int lane) {
  using R = Rec<TYP, T>;
  prefetch_span_chunk(p.rec + g0 * R::SIZE, n * R::SIZE * (int64_t)sizeof(T), lane);
  prefetch_span_chunk(p.dio + g0 * DIO, n * DIO * (int64_t)sizeof(T), lane);
  const int32_t* nb = upper ? p.nbu : p.nbl;
#pragma unroll
  for (int d = 0; d < 3; d++) prefetch_span_chunk(nb + d * p.G + g0, n * 4, lane);
  if (upper) prefetch_span_chunk(p.cells + g0, n * 4, lane);   // the in-place Newton update's cells
}

// (Loading the cells' static operands before the wait was measured slower:
// the operands held across the wait raise the register count to 154 and
// halve the resident warps; so was splitting the neighbours' wait and the
// upper chunk's own-lower wait into two rounds.)
template <int TYP, typename T, int NV, bool MULTI, bool UPPER>
__device__ __forceinline__ void flow_chunk(const Zone& z, const PlaneData<T>& p, const LuFields& f,
                                           int64_t g0, int64_t n, int lane) {
  if (lane < n) {
    CellOps<TYP, T, NV> o;
    load_ops<TYP, T, UPPER, NV>(p, f.inplace != 0, g0 + lane, o);
    run_cell_of<TYP, T, UPPER, NV, MULTI>(z, p, f, g0 + lane, o);
  }
}

// FP32 sweeps (bound by the latency of the hyperplane chain, not by
// arithmetic): the chunk's static operands -- its records, its neighbours'
// coefficients and held states, its residual -- are loaded before the
// dependency wait, so that only the neighbours' increments (and, upper, the
// cell's own lower result) are read after it.  (FP64 sweeps load them after
// the wait: held across it they cost registers the FP64 sweep needs.)
template <int TYP, typename T, int NV, bool MULTI, bool UPPER>
__device__ __forceinline__ void flow_pre(const PlaneData<T>& p, const LuFields& f, int64_t g0,
                                         int64_t n, int lane, CellOps<TYP, T, NV>& o) {
  if (lane < n) load_ops<TYP, T, UPPER, NV>(p, f.inplace != 0, g0 + lane, o, false);
}
template <int TYP, typename T, int NV, bool MULTI, bool UPPER>
__device__ __forceinline__ void flow_run(const Zone& z, const PlaneData<T>& p, const LuFields& f,
                                         int64_t g0, int64_t n, int lane, CellOps<TYP, T, NV>& o) {
  if (lane < n) {
    if (UPPER) load_x_upper<TYP, T, NV>(p, g0 + lane, o);
    run_cell_of<TYP, T, UPPER, NV, MULTI>(z, p, f, g0 + lane, o);
  }
}

template <int TYP, typename T, int NV, bool MULTI>
__global__ void __launch_bounds__(FLOW_THREADS)
    lusgs_flow(Zone z, PlaneData<T> p, LuFields f, FlowArgs a) {
  const int lane = threadIdx.x & 31;
  const int64_t nc = a.nchunk;
  while (true) {
    unsigned long long t = 0;
    if (lane == 0) t = atomicAdd(a.ticket, 1ull);
    t = __shfl_sync(0xffffffffu, t, 0);
    if (t >= (unsigned long long)(2 * nc)) return;
    if (*(volatile int*)a.err) return;
    const bool upper = t >= (unsigned long long)nc;
    const int64_t ch = upper ? 2 * nc - 1 - (int64_t)t : (int64_t)t;
    const int32_t* dp = a.dep + FLOW_DEP * ch + (upper ? 4 : 0);
    const int64_t lo1 = dp[0], n1 = dp[1] - lo1 + 1, lo2 = dp[2], n2 = dp[3] - lo2 + 1;
    const int mark = upper ? a.upper_mark : a.lower_mark;
    const int s = a.cplane[ch];
    const int64_t g0 = p.plane[s] + (ch - a.cbase[s]) * FLOW_CHUNK;
    const int64_t n = p.plane[s + 1] - g0;
    if (a.prefetch) prefetch_chunk<TYP, T>(p, g0, n < FLOW_CHUNK ? n : FLOW_CHUNK, upper, lane);
    constexpr bool PRE = sizeof(T) == 4;
    CellOps<TYP, T, NV> o;
    if (PRE) {
      if (upper) flow_pre<TYP, T, NV, MULTI, true>(p, f, g0, n, lane, o);
      else flow_pre<TYP, T, NV, MULTI, false>(p, f, g0, n, lane, o);
    }
    bool ok = true;
    for (int64_t m = lane; m < n1 + n2; m += 32)
      ok = ok && flow_poll(a, m < n1 ? lo1 + m : lo2 + (m - n1), mark + a.wait_skew);
    if (upper && lane == 0) ok = ok && flow_poll(a, ch, a.lower_mark + a.wait_skew);
    if (!__all_sync(0xffffffffu, ok)) return;
    if (PRE) {
      if (upper) flow_run<TYP, T, NV, MULTI, true>(z, p, f, g0, n, lane, o);
      else flow_run<TYP, T, NV, MULTI, false>(z, p, f, g0, n, lane, o);
    } else {
      if (upper) flow_chunk<TYP, T, NV, MULTI, true>(z, p, f, g0, n, lane);
      else flow_chunk<TYP, T, NV, MULTI, false>(z, p, f, g0, n, lane);
    }
    __syncwarp();
    if (lane == 0)
      asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(a.flag + ch), "r"(mark) : "memory");
  }
}

// one launch per hyperplane (no inter-CTA waits): cross-check of the
// persistent kernel
template <int TYP, typename T, bool UPPER, int NV, bool MULTI>
__global__ void __launch_bounds__(128) lusgs_plane(Zone z, PlaneData<T> p, LuFields f, int64_t s) {
  const int64_t c0 = p.plane[s], n = p.plane[s + 1] - c0;
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  CellOps<TYP, T, NV> o;
  load_ops<TYP, T, UPPER, NV>(p, f.inplace != 0, c0 + c, o);
  run_cell_of<TYP, T, UPPER, NV, MULTI>(z, p, f, c0 + c, o);
}

// FP64 Newton update of every interior cell after the sweeps.  Tiles of
// GT_I x GT_J cells at one k as in lu_gather: the increments of a tile
// anti-diagonal are contiguous in plane order, so the CTA reads them as
// spans into shared memory, then updates its cells in natural order.
template <typename T, bool TWO_D, int NV>
__global__ void __launch_bounds__(GT_N) lu_newton(Zone z, LuFields f, const T* __restrict__ dio) {
  __shared__ __align__(16) T s_dio[GT_N * DIO];
  __shared__ int32_t s_g[GT_N];
  const int ti = threadIdx.x % GT_I, tj = threadIdx.x / GT_I;
  const int64_t ii = (int64_t)blockIdx.x * GT_I + ti, jj = (int64_t)blockIdx.y * GT_J + tj;
  const int64_t kk = blockIdx.z;
  const int q = tile_slot(ti, tj);
  const bool in = ii < z.ni && jj < z.nj;
  const int64_t l = in ? inddm(z, ii + 1, jj + 1, kk + 1) : 0;
  s_g[q] = in ? f.posmap[l] : -1;
  __syncthreads();
  using V2 = typename Vec2<T>::t;
  for (int c = threadIdx.x; c < GT_N * (DIO / 2); c += GT_N) {
    const int qq = c / (DIO / 2), m = c - qq * (DIO / 2);
    const int32_t g = s_g[qq];
    if (g < 0) continue;
    reinterpret_cast<V2*>(s_dio + qq * DIO)[m] = reinterpret_cast<const V2*>(dio + (int64_t)g * DIO)[m];
  }
  __syncthreads();
  if (!in) return;
  const int64_t nd = z.nd;
  const double* R = f.rop_old;
  if (sizeof(T) == 8) {  // mjr_newton.for, FP64
    double d[5], nw[5];
#pragma unroll
    for (int v = 0; v < 5; v++) d[v] = double(s_dio[q * DIO + v]);
    newton<double, TWO_D>(z.cv, z.cvinv, R[l], R[l + nd], R[l + 2 * nd], R[l + 3 * nd], R[l + 4 * nd],
                          d, nw);
#pragma unroll
    for (int v = 0; v < 5; v++) f.rop_new[l + v * nd] = nw[v];
    if (NV == 6)
      f.rop_new[l + 5 * nd] = newton_sa(z, R[l], R[l + 5 * nd], double(s_dio[q * DIO + NV - 1]),
                                        1. / nw[0], nw[4]);
    return;
  }
  // Mixed precision: the same map written as W^{p+1} = W^p + delta with the
  // increments in cancellation-free form,
  //   ro' = ro + d0,  du = (d1 - u d0) / ro'  (likewise v, w),
  //   de = (d4 - e d0) / ro'  with e = cv T + |u|^2 / 2,
  //   dT = (de - (du (2u + du) + dv (2v + dv) + dw (2w + dw)) / 2) / cv,
  // evaluated in FP32 (their relative FP32 error vanishes with delta) and
  // added to the FP64 state.
  const double ro = R[l], u = R[l + nd], v = R[l + 2 * nd], w = R[l + 3 * nd], tt = R[l + 4 * nd];
  const float d0 = float(s_dio[q * DIO]), d1 = float(s_dio[q * DIO + 1]),
              d2 = float(s_dio[q * DIO + 2]), d3 = float(s_dio[q * DIO + 3]),
              d4 = float(s_dio[q * DIO + 4]);
  const double ron = ro + double(d0);
  const float r1 = 1.f / float(ron);
  const float fu = float(u), fv = float(v), fw = float(w), cv = z.fcv;
  const float e = cv * float(tt) + 0.5f * (fu * fu + fv * fv + fw * fw);
  const float du = (d1 - fu * d0) * r1, dv = (d2 - fv * d0) * r1;
  const float dw = TWO_D ? 0.f : (d3 - fw * d0) * r1;   // 2-d: w = 0
  const float de = (d4 - e * d0) * r1;
  const float dT = (de - 0.5f * (du * (2.f * fu + du) + dv * (2.f * fv + dv) + dw * (2.f * fw + dw))) / cv;
  f.rop_new[l] = ron;
  f.rop_new[l + nd] = u + double(du);
  f.rop_new[l + 2 * nd] = v + double(dv);
  f.rop_new[l + 3 * nd] = TWO_D ? 0. : w + double(dw);
  f.rop_new[l + 4 * nd] = tt + double(dT);
  if (NV == 6)   // the SA update (mjr_newton_SA.for) on the FP64 state
    f.rop_new[l + 5 * nd] = newton_sa(z, ro, R[l + 5 * nd], double(s_dio[q * DIO + NV - 1]), 1. / ron,
                                      tt + double(dT));
}

template <int TYP, typename T, int NV>
static cudaError_t gather_t(const Zone& z, const LuFields& f, const PlaneData<T>& p, cudaStream_t st) {
  using S = GatherSmem<TYP, T>;
  static bool smem_set[64] = {};   // per device
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  if (!smem_set[dev]) {
    cudaError_t e0 = cudaFuncSetAttribute(lu_gather<TYP, T, NV>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::bytes);
    if (e0 != cudaSuccess) return e0;
    smem_set[dev] = true;
  }
  lu_gather<TYP, T, NV><<<dim3((unsigned)((z.ni + GT_I - 1) / GT_I), (unsigned)((z.nj + GT_J - 1) / GT_J),
                           (unsigned)z.nk), GT_N, S::bytes, st>>>(z, f, p);
  return cudaGetLastError();
}

template <int TYP, typename T, int NV, bool MULTI>
static cudaError_t sweep_t(const Zone& z, const LuFields& f, const PlaneData<T>& p, const LuGroup& L,
                           cudaStream_t st) {
  cudaError_t e;
  if (L.persistent == 2) {
    // CTA size: L.flow_threads (the autotuner's choice, a whole number of
    // warps), by default FLOW_THREADS
    const int threads = L.flow_threads > 0 ? L.flow_threads : FLOW_THREADS;
    if (threads % 32 != 0 || threads > FLOW_THREADS) return cudaErrorInvalidValue;
    const int wpc = threads / 32;
    static int per_sm[64][FLOW_THREADS / 32 + 1] = {};   // per instantiation, device, CTA size
    int dev = 0;
    e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    if (per_sm[dev][wpc] == 0) {
      int per = 0;
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, lusgs_flow<TYP, T, NV, MULTI>, threads, 0);
      if (e != cudaSuccess) return e;
      if (per < 1) return cudaErrorLaunchOutOfResources;
      per_sm[dev][wpc] = per;
    }
    // CTAs per SM: L.flow_per_sm (the autotuner's choice), by default one
    // (8 warps), measured faster than filling every resident slot on one
    // large zone (256^3 Taylor-Green, FP64: 98 vs 105 ms of LU-SGS per step)
    int nsm_ = 0;
    e = cudaDeviceGetAttribute(&nsm_, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    const int per_use = L.flow_per_sm > 0 ? std::min(L.flow_per_sm, per_sm[dev][wpc]) : 1;
    int grid = nsm_ * per_use;
    if (L.grid_cap > 0 && L.grid_cap < grid) grid = L.grid_cap;
    e = cudaMemsetAsync(L.flow.ticket, 0, sizeof(unsigned long long), st);
    if (e != cudaSuccess) return e;
    lusgs_flow<TYP, T, NV, MULTI><<<grid, threads, 0, st>>>(z, p, f, L.flow);
    return cudaGetLastError();
  }
  if (L.persistent) {
    static int grids[64] = {};   // per instantiation and device: resident CTAs of the sweep
    int dev = 0;
    e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    if (grids[dev] == 0) {
      int nsm = 0, per = 0;
      e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
      if (e != cudaSuccess) return e;
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, lusgs_persistent<TYP, T, NV, MULTI>,
                                                        LuThreads<T>::n, 0);
      if (e != cudaSuccess) return e;
      grids[dev] = nsm * (per > 0 ? per : 1);
    }
    int grid = grids[dev];
    if (L.grid_cap > 0 && L.grid_cap < grid) grid = L.grid_cap;
    e = cudaMemsetAsync(L.bar, 0, sizeof(unsigned int), st);
    if (e != cudaSuccess) return e;
    GridBar gb{L.bar, L.err, L.flow.poll_limit << 2, (unsigned int)L.flow.wait_skew};
    Zone zz = z;
    LuFields ff = f;
    PlaneData<T> pp = p;
    void* args[] = {(void*)&zz, (void*)&pp, (void*)&ff, (void*)&gb};
    e = cudaLaunchCooperativeKernel((void*)lusgs_persistent<TYP, T, NV, MULTI>, dim3(grid),
                                    dim3(LuThreads<T>::n), args, 0, st);
  } else {
    const int B = 128;
    for (int64_t s = 0; s <= p.smax; s++) {
      int64_t n = L.plane_host[s + 1] - L.plane_host[s];
      if (n > 0)
        lusgs_plane<TYP, T, false, NV, MULTI><<<(unsigned)((n + B - 1) / B), B, 0, st>>>(z, p, f, s);
    }
    for (int64_t s = p.smax; s >= 0; s--) {
      int64_t n = L.plane_host[s + 1] - L.plane_host[s];
      if (n > 0)
        lusgs_plane<TYP, T, true, NV, MULTI><<<(unsigned)((n + B - 1) / B), B, 0, st>>>(z, p, f, s);
    }
    e = cudaGetLastError();
  }
  return e;
}

template <int TYP, typename T, int NV>
static cudaError_t group_t(const LuZone* zh, const PlaneData<T>& p, const LuGroup& L, cudaStream_t st) {
  cudaError_t e;
  for (int m = 0; m < L.nz; m++) {
    e = gather_t<TYP, T, NV>(zh[m].z, zh[m].f, p, st);
    if (e != cudaSuccess) return e;
  }
  // a single zone runs with its descriptor as a kernel parameter; several
  // zones read theirs from the table (per cell)
  e = L.nz == 1 ? sweep_t<TYP, T, NV, false>(zh[0].z, zh[0].f, p, L, st)
                : sweep_t<TYP, T, NV, true>(zh[0].z, zh[0].f, p, L, st);
  if (e != cudaSuccess) return e;
  for (int m = 0; m < L.nz; m++) {
    const Zone& z = zh[m].z;
    if (zh[m].f.inplace && sizeof(T) == 8) continue;   // updated by the upper sweep
    lu_newton<T, TYP == Z2D, NV><<<dim3((unsigned)((z.ni + GT_I - 1) / GT_I),
                                        (unsigned)((z.nj + GT_J - 1) / GT_J), (unsigned)z.nk),
                                   GT_N, 0, st>>>(z, zh[m].f, p.dio);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

template <typename T>
static PlaneData<T> plane_data(const LuGroup& L, int rec_size) {
  PlaneData<T> p;
  const int64_t G = L.GG;
  T* w = (T*)L.work;
  p.rec = w; w += (int64_t)rec_size * G;
  p.dio = w; w += (int64_t)DIO * G;
  p.nst = w; w += 4 * G;
  p.nbl = L.nbl; p.nbu = L.nbu; p.cells = L.cells; p.plane = L.plane; p.G = G;
  p.smax = L.smax; p.zid = L.zid; p.zt = L.ztab;
  return p;
}

int lusgs_flow_chunk() { return FLOW_CHUNK; }

// words of LU work per interior cell (the caller allocates G * this * 8 bytes)
int64_t lusgs_work_words(int typ) {
  return (typ == Z3DCART ? Rec<Z3DCART, double>::SIZE : Rec<Z3DFULL, double>::SIZE) + DIO + 4;
  // (2-d zones use the general record layout)
}

cudaError_t launch_lu_neighbours(const LuGroup& L, cudaStream_t st) {
  lu_neighbours<<<(unsigned)((L.GG + 255) / 256), 256, 0, st>>>(L.ztab, L.zid, L.cells, L.nbl, L.nbu,
                                                                L.GG);
  return cudaGetLastError();
}

// One LU-SGS solve (lower, upper, Newton update) of a group of zones of one
// kind (zone type, equation count, sweep precision).
cudaError_t launch_lusgs(const LuZone* zh, const LuGroup& L, cudaStream_t st) {
  if (L.nz < 1) return cudaSuccess;
  const Zone& z = zh[0].z;
  const bool sa = z.neq == 6;   // Spalart-Allmaras: 3d zones
  if (L.fp32) {
    const int rs = z.typ == Z3DCART ? Rec<Z3DCART, float>::SIZE : Rec<Z3DFULL, float>::SIZE;
    PlaneData<float> p = plane_data<float>(L, rs);
    if (z.typ == Z3DCART)
      return sa ? group_t<Z3DCART, float, 6>(zh, p, L, st) : group_t<Z3DCART, float, 5>(zh, p, L, st);
    if (z.typ == Z2D) return sa ? group_t<Z2D, float, 6>(zh, p, L, st) : group_t<Z2D, float, 5>(zh, p, L, st);
    return sa ? group_t<Z3DFULL, float, 6>(zh, p, L, st) : group_t<Z3DFULL, float, 5>(zh, p, L, st);
  }
  const int rs = z.typ == Z3DCART ? Rec<Z3DCART, double>::SIZE : Rec<Z3DFULL, double>::SIZE;
  PlaneData<double> p = plane_data<double>(L, rs);
  if (z.typ == Z3DCART)
    return sa ? group_t<Z3DCART, double, 6>(zh, p, L, st) : group_t<Z3DCART, double, 5>(zh, p, L, st);
  if (z.typ == Z2D) return sa ? group_t<Z2D, double, 6>(zh, p, L, st) : group_t<Z2D, double, 5>(zh, p, L, st);
  return sa ? group_t<Z3DFULL, double, 6>(zh, p, L, st) : group_t<Z3DFULL, double, 5>(zh, p, L, st);
}

}  // namespace fgb
