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
template <int TYP> struct NBE { static constexpr int n = TYP == Z3DCART ? NB_CART : NB_FULL; };

template <int TYP, typename T>
__device__ __forceinline__ void bentries(const Zone& z, int d, T u, T v, T w, T t, T tcx, T tcy,
                                         T tcz, T* e) {
  const T gam1 = T(z.gam), gamm1 = T(z.gam - 1.), cp = T(z.gam * z.cv),
          gam2 = T((z.gam - 1.) - 1.);
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
  }
}

// b = B . o from the stored entries (cs = coe_{d+2}(nb) * signe)
template <int TYP, int D, typename T>
__device__ __forceinline__ void bmatvec(const Zone& z, const T* e, T cs, const T o[5], T b[5]) {
  const T gamm1 = T(z.gam - 1.);
  if (TYP == Z3DCART) {
    if (D == 0) {
      const T tcx = T(z.tcx), b25 = tcx * gamm1;
      b[0] = cs * o[0] + tcx * o[1];
      b[1] = e[0] * o[0] + (e[1] + cs) * o[1] + e[2] * o[2] + e[3] * o[3] + b25 * o[4];
      b[2] = e[4] * o[0] + e[5] * o[1] + ((e[6]) + cs) * o[2];
      b[3] = e[7] * o[0] + e[8] * o[1] + ((e[6]) + cs) * o[3];
      b[4] = e[9] * o[0] + e[10] * o[1] + e[11] * o[2] + e[12] * o[3] + (e[13] + cs) * o[4];
    } else if (D == 1) {
      const T tcy = T(z.tcy), b35 = tcy * gamm1;
      b[0] = cs * o[0] + tcy * o[2];
      b[1] = e[0] * o[0] + (e[1] + cs) * o[1] + e[2] * o[2];
      b[2] = e[3] * o[0] + e[4] * o[1] + (e[5] + cs) * o[2] + e[6] * o[3] + b35 * o[4];
      b[3] = e[7] * o[0] + e[8] * o[2] + ((e[1]) + cs) * o[3];
      b[4] = e[9] * o[0] + e[10] * o[1] + e[11] * o[2] + e[12] * o[3] + (e[13] + cs) * o[4];
    } else {
      const T tcz = T(z.tcz), b45 = tcz * gamm1;
      b[0] = cs * o[0] + tcz * o[3];
      b[1] = e[0] * o[0] + (e[1] + cs) * o[1] + e[2] * o[3];
      b[2] = e[3] * o[0] + (e[1] + cs) * o[2] + e[4] * o[3];
      b[3] = e[5] * o[0] + e[6] * o[1] + e[7] * o[2] + (e[8] + cs) * o[3] + b45 * o[4];
      b[4] = e[9] * o[0] + e[10] * o[1] + e[11] * o[2] + e[12] * o[3] + (e[13] + cs) * o[4];
    }
  } else {
    b[0] = cs * o[0] + e[0] * o[1] + e[1] * o[2] + e[2] * o[3];
    b[1] = e[3] * o[0] + (e[4] + cs) * o[1] + e[5] * o[2] + e[6] * o[3] + e[7] * o[4];
    b[2] = e[8] * o[0] + e[9] * o[1] + (e[10] + cs) * o[2] + e[11] * o[3] + e[12] * o[4];
    b[3] = e[13] * o[0] + e[14] * o[1] + e[15] * o[2] + (e[16] + cs) * o[3] + e[17] * o[4];
    b[4] = e[18] * o[0] + e[19] * o[1] + e[20] * o[2] + e[21] * o[3] + (e[22] + cs) * o[4];
  }
}

template <int D> struct DirT { static constexpr int value = D; };

// ---------------------------------------------------------------- cells
// Precision T: double for the plain FP64 path; float for the mixed path
// (FP32 sweeps and approximate Jacobians; the Newton update stays FP64).
template <typename T>
struct LuCellArgs {
  const T* st;            // W^p in precision T
  const T* coe;           // coe in precision T
  T* dio;                 // increment, in place over the residual
  const T* bt;            // B entries: bt[(d*NB + m)*nd + l]
  const double* rop_old;  // FP64 W^p (Newton update)
  double* rop_new;        // FP64 W^{p+1}
  T* stn;                 // mixed path, in place: W^{p+1} in precision T (k+1 neighbours)
  int inplace;            // upper sweep: k+1 neighbour taken after its update
  const uint32_t* cells;  // cells ordered by hyperplane, packed i | j<<11 | k<<22
  const int64_t* plane;   // plane s holds cells[plane[s] .. plane[s+1])
};

__device__ __forceinline__ void unpack(uint32_t c, int64_t& ii, int64_t& jj, int64_t& kk) {
  ii = c & 2047u; jj = (c >> 11) & 2047u; kk = c >> 22;
}

template <int TYP, typename T>
__device__ __forceinline__ void lower_cell(const Zone& z, const LuCellArgs<T>& a, int64_t ii,
                                           int64_t jj, int64_t kk) {
  const int64_t l = inddm(z, ii + 1, jj + 1, kk + 1);
  const int64_t nd = z.nd;
  constexpr int NB = NBE<TYP>::n;
  const T xal = a.coe[l] * T(0.5);
  T x[5], o[5], b[5], e[NB];
#pragma unroll
  for (int v = 0; v < 5; v++) x[v] = ldcg(a.dio + l + v * nd);
  auto term = [&](auto dc, int64_t l1) {
    constexpr int D = decltype(dc)::value;
#pragma unroll
    for (int v = 0; v < 5; v++) o[v] = ldcg(a.dio + l1 + v * nd);
#pragma unroll
    for (int m = 0; m < NB; m++) e[m] = a.bt[(D * NB + m) * nd + l1];
    T cs = a.coe[l1 + (D + 1) * nd] * T(0.5);
    bmatvec<TYP, D, T>(z, e, cs, o, b);
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
  const T diag = T(1.) / a.coe[l + 4 * nd];
#pragma unroll
  for (int v = 0; v < 5; v++) a.dio[l + v * nd] = x[v] * diag;
}

// mjr_newton.for: W^{p+1} = prim(cons(W^p) + dW), FP64
__device__ __forceinline__ void newton64(const Zone& z, const double* R, double* O, int64_t l,
                                         double d0, double d1, double d2, double d3, double d4) {
  const int64_t nd = z.nd;
  const double cv = z.cv, cvinv = 1. / cv, cvinv2 = 0.5 * cvinv;
  double ro = R[l], u = R[l + nd], v = R[l + 2 * nd], w = R[l + 3 * nd], tt = R[l + 4 * nd];
  double n1 = ro + d0;
  double r_1 = 1. / n1;
  double n2 = (ro * u + d1) * r_1;
  double n3 = (ro * v + d2) * r_1;
  double n4 = (ro * w + d3) * r_1;
  double roe_old = ro * (cv * tt + 0.5 * (u * u + v * v + w * w));
  double n5 = (roe_old + d4) * r_1 * cvinv - cvinv2 * (n2 * n2 + n3 * n3 + n4 * n4);
  O[l] = n1; O[l + nd] = n2; O[l + 2 * nd] = n3; O[l + 3 * nd] = n4; O[l + 4 * nd] = n5;
}

template <int TYP, typename T>
__device__ __forceinline__ void upper_cell(const Zone& z, const LuCellArgs<T>& a, int64_t ii,
                                           int64_t jj, int64_t kk) {
  const int64_t l = inddm(z, ii + 1, jj + 1, kk + 1);
  const int64_t lt = TYP == Z3DCART ? 0 : indmtr(z, ii + 1, jj + 1, kk + 1);
  const int64_t nd = z.nd;
  constexpr int NB = NBE<TYP>::n;
  const T xal = a.coe[l] * T(-0.5);
  const T dg = a.coe[l + 4 * nd];
  T x[5], o[5], b[5], e[NB];
#pragma unroll
  for (int v = 0; v < 5; v++) x[v] = ldcg(a.dio + l + v * nd) * dg;  // lu_d.for
  auto term = [&](auto dc, int64_t l1, bool fresh) {
    constexpr int D = decltype(dc)::value;
#pragma unroll
    for (int v = 0; v < 5; v++) o[v] = ldcg(a.dio + l1 + v * nd);
    T cs = a.coe[l1 + (D + 1) * nd] * T(-0.5);
    if (fresh) {  // neighbour already updated: B from its new state
      T u, vv, w, t;
      if (sizeof(T) == 8) {
        u = T(ldcg(a.rop_new + l1 + nd)); vv = T(ldcg(a.rop_new + l1 + 2 * nd));
        w = T(ldcg(a.rop_new + l1 + 3 * nd)); t = T(ldcg(a.rop_new + l1 + 4 * nd));
      } else {
        u = ldcg(a.stn + l1 + nd); vv = ldcg(a.stn + l1 + 2 * nd);
        w = ldcg(a.stn + l1 + 3 * nd); t = ldcg(a.stn + l1 + 4 * nd);
      }
      T tx, ty, tz;
      nb_normal<TYP, T>(z, D, lt + z.minc[D], lt + 2 * z.minc[D], tx, ty, tz);
      bentries<TYP, T>(z, D, u, vv, w, t, tx, ty, tz, e);
    } else {
#pragma unroll
      for (int m = 0; m < NB; m++) e[m] = a.bt[(D * NB + m) * nd + l1];
    }
    bmatvec<TYP, D, T>(z, e, cs, o, b);
#pragma unroll
    for (int v = 0; v < 5; v++) x[v] = x[v] + b[v] * xal;
  };
  if (kk < z.nk - 1) term(DirT<2>{}, l + z.inc[2], a.inplace != 0);
  if (jj < z.nj - 1) term(DirT<1>{}, l + z.inc[1], false);
  if (ii < z.ni - 1) term(DirT<0>{}, l + 1, false);
  const T diag = T(1.) / a.coe[l + 4 * nd];
#pragma unroll
  for (int v = 0; v < 5; v++) x[v] = x[v] * diag;
#pragma unroll
  for (int v = 0; v < 5; v++) a.dio[l + v * nd] = x[v];
  if (!a.inplace) return;  // the Newton update runs after the sweep
  if (sizeof(T) == 8) {
    // the k-1 neighbour reads this cell's new state in the next plane
    newton64(z, a.rop_old, a.rop_new, l, double(x[0]), double(x[1]), double(x[2]),
             double(x[3]), double(x[4]));
  } else {
    // mixed path: the new state in precision T for the neighbour's Jacobian;
    // the FP64 update itself runs after the sweep
    const T* R = a.st;
    const T cv = T(z.cv), cvinv = T(1.) / cv, cvinv2 = T(0.5) * cvinv;
    T ro = R[l], u = R[l + nd], v = R[l + 2 * nd], w = R[l + 3 * nd], tt = R[l + 4 * nd];
    T n1 = ro + x[0], r_1 = T(1.) / n1;
    T n2 = (ro * u + x[1]) * r_1, n3 = (ro * v + x[2]) * r_1, n4 = (ro * w + x[3]) * r_1;
    T roe_old = ro * (cv * tt + T(0.5) * (u * u + v * v + w * w));
    T n5 = (roe_old + x[4]) * r_1 * cvinv - cvinv2 * (n2 * n2 + n3 * n3 + n4 * n4);
    a.stn[l + nd] = n2; a.stn[l + 2 * nd] = n3; a.stn[l + 3 * nd] = n4; a.stn[l + 4 * nd] = n5;
  }
}

// ------------------------------------------------------- grid barrier
// Cooperative launch guarantees that every CTA is resident.  The wait is
// bounded: past ~1 s it sets the error word, leaves the barrier and the
// kernel returns; the host reports FGB_ERR_DEVICE.
struct GridBar { unsigned int* count; unsigned int* gen; int* err; };

__device__ __forceinline__ bool grid_sync(const GridBar& g, unsigned int nblocks,
                                          unsigned int& my_gen) {
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned int target = my_gen + 1;
    __threadfence();
    unsigned int arrived = atomicAdd(g.count, 1u);
    if (arrived == nblocks - 1) {
      atomicExch(g.count, 0u);
      __threadfence();
      atomicExch(g.gen, target);
    } else {
      long long spins = 0;
      while (true) {
        unsigned int cur;
        asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(cur) : "l"(g.gen) : "memory");
        if (cur == target) break;
        if (*(volatile int*)g.err) break;
        if (++spins > (1ll << 24)) { atomicExch(g.err, 1); break; }
        __nanosleep(32);
      }
    }
    __threadfence();
    my_gen = target;
  }
  __syncthreads();
  return *(volatile int*)g.err == 0;
}

// cells of plane s spread over every CTA: cell c of the plane goes to CTA
// c mod gridDim, so each CTA's share is packed into its first warps
template <int TYP, typename T, bool UPPER>
__device__ __forceinline__ void do_plane(const Zone& z, const LuCellArgs<T>& a, int64_t s) {
  const int64_t c0 = a.plane[s], n = a.plane[s + 1] - c0;
  for (int64_t c = (int64_t)threadIdx.x * gridDim.x + blockIdx.x; c < n;
       c += (int64_t)gridDim.x * blockDim.x) {
    int64_t ii, jj, kk;
    unpack(a.cells[c0 + c], ii, jj, kk);
    if (UPPER) upper_cell<TYP, T>(z, a, ii, jj, kk);
    else lower_cell<TYP, T>(z, a, ii, jj, kk);
  }
}

template <int TYP, typename T>
__global__ void __launch_bounds__(256) lusgs_persistent(Zone z, LuCellArgs<T> a, GridBar g) {
  const int64_t smax = (z.ni - 1) + (z.nj - 1) + (z.nk - 1);
  unsigned int my_gen = 0;
  for (int64_t s = 0; s <= smax; s++) {   // lower sweep, ascending hyperplanes
    do_plane<TYP, T, false>(z, a, s);
    if (!grid_sync(g, gridDim.x, my_gen)) return;
  }
  for (int64_t s = smax; s >= 0; s--) {   // upper sweep
    do_plane<TYP, T, true>(z, a, s);
    if (s > 0 && !grid_sync(g, gridDim.x, my_gen)) return;
  }
}

// one launch per hyperplane (no inter-CTA waits): cross-check of the
// persistent kernel
template <int TYP, typename T, bool UPPER>
__global__ void __launch_bounds__(128) lusgs_plane(Zone z, LuCellArgs<T> a, int64_t s) {
  const int64_t c0 = a.plane[s], n = a.plane[s + 1] - c0;
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  int64_t ii, jj, kk;
  unpack(a.cells[c0 + c], ii, jj, kk);
  if (UPPER) upper_cell<TYP, T>(z, a, ii, jj, kk);
  else lower_cell<TYP, T>(z, a, ii, jj, kk);
}

// B-coefficient pre-pass over every interior cell
template <int TYP, typename T>
__global__ void __launch_bounds__(256) lu_bprep(Zone z, const T* __restrict__ st,
                                                T* __restrict__ bt) {
  const int64_t n = z.ni * z.nj * z.nk;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int64_t ii = t % z.ni, r = t / z.ni, jj = r % z.nj, kk = r / z.nj;
  const int64_t l = inddm(z, ii + 1, jj + 1, kk + 1);
  const int64_t lt = TYP == Z3DCART ? 0 : indmtr(z, ii + 1, jj + 1, kk + 1);
  const int64_t nd = z.nd;
  constexpr int NB = NBE<TYP>::n;
  T u = st[l + nd], v = st[l + 2 * nd], w = st[l + 3 * nd], tt = st[l + 4 * nd];
  T e[NB];
#pragma unroll
  for (int d = 0; d < 3; d++) {
    T tx, ty, tz;
    nb_normal<TYP, T>(z, d, lt, lt + z.minc[d], tx, ty, tz);
    bentries<TYP, T>(z, d, u, v, w, tt, tx, ty, tz, e);
#pragma unroll
    for (int m = 0; m < NB; m++) bt[(d * NB + m) * nd + l] = e[m];
  }
}

// FP64 Newton update of every interior cell after the sweeps
template <typename T>
__global__ void __launch_bounds__(256) lu_newton(Zone z, const double* __restrict__ R,
                                                 double* __restrict__ O, const T* __restrict__ d) {
  const int64_t n = z.ni * z.nj * z.nk;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int64_t ii = t % z.ni, r = t / z.ni, jj = r % z.nj, kk = r / z.nj;
  const int64_t l = inddm(z, ii + 1, jj + 1, kk + 1), nd = z.nd;
  newton64(z, R, O, l, double(d[l]), double(d[l + nd]), double(d[l + 2 * nd]),
           double(d[l + 3 * nd]), double(d[l + 4 * nd]));
}

// FP32 copies of the state, the coefficients and the residual for the
// mixed-precision sweeps (one pass per sub-iteration)
__global__ void __launch_bounds__(256) to_float(int64_t n, const double* __restrict__ a,
                                                float* __restrict__ b) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) b[t] = (float)a[t];
}

template <int TYP, typename T>
static cudaError_t launch_t(const Zone& z, const LuCellArgs<T>& a, const LuLaunch& L,
                            cudaStream_t st) {
  const int64_t ncell = z.ni * z.nj * z.nk;
  const unsigned gc = (unsigned)((ncell + 255) / 256);
  lu_bprep<TYP, T><<<gc, 256, 0, st>>>(z, a.st, const_cast<T*>(a.bt));
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  if (L.persistent) {
    static int grid_cache[2][2] = {{0, 0}, {0, 0}};
    int& grid = grid_cache[TYP == Z3DCART][sizeof(T) == 4];
    if (grid == 0) {
      int dev = 0, nsm = 0, per = 0;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, lusgs_persistent<TYP, T>, 256, 0);
      grid = nsm * (per > 0 ? per : 1);
    }
    e = cudaMemsetAsync(L.bar, 0, 2 * sizeof(unsigned int), st);
    if (e != cudaSuccess) return e;
    GridBar g{L.bar, L.bar + 1, L.err};
    void* args[] = {(void*)&z, (void*)&a, (void*)&g};
    e = cudaLaunchCooperativeKernel((void*)lusgs_persistent<TYP, T>, dim3(grid), dim3(256), args,
                                    0, st);
  } else {
    const int B = 128;
    const int64_t smax = (z.ni - 1) + (z.nj - 1) + (z.nk - 1);
    for (int64_t s = 0; s <= smax; s++) {
      int64_t n = L.plane_host[s + 1] - L.plane_host[s];
      lusgs_plane<TYP, T, false><<<(unsigned)((n + B - 1) / B), B, 0, st>>>(z, a, s);
    }
    for (int64_t s = smax; s >= 0; s--) {
      int64_t n = L.plane_host[s + 1] - L.plane_host[s];
      lusgs_plane<TYP, T, true><<<(unsigned)((n + B - 1) / B), B, 0, st>>>(z, a, s);
    }
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) return e;
  if (!a.inplace || sizeof(T) == 4) {
    lu_newton<T><<<gc, 256, 0, st>>>(z, a.rop_old, a.rop_new, a.dio);
    e = cudaGetLastError();
  }
  return e;
}

// One LU-SGS solve (lower, upper, Newton update) of one zone.
cudaError_t launch_lusgs(const Zone& z, const LuArgs& a, const LuLaunch& L, cudaStream_t st) {
  const int inplace = a.rop_knb == a.rop_new;
  if (L.fp32) {
    const int64_t n = 5 * z.nd;
    const unsigned g = (unsigned)((n + 255) / 256);
    to_float<<<g, 256, 0, st>>>(n, a.rop_old, L.st32);
    to_float<<<g, 256, 0, st>>>(n, a.coe, L.coe32);
    to_float<<<g, 256, 0, st>>>(n, a.din, L.d32);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    LuCellArgs<float> c{L.st32, L.coe32, L.d32, (const float*)L.bt, a.rop_old, a.rop_new,
                        L.stn32, inplace, L.cells, L.plane};
    return z.typ == Z3DCART ? launch_t<Z3DCART, float>(z, c, L, st)
                            : launch_t<Z3DFULL, float>(z, c, L, st);
  }
  LuCellArgs<double> c{a.rop_old, a.coe, a.dout, (const double*)L.bt, a.rop_old, a.rop_new,
                       nullptr, inplace, L.cells, L.plane};
  return z.typ == Z3DCART ? launch_t<Z3DCART, double>(z, c, L, st)
                          : launch_t<Z3DFULL, double>(z, c, L, st);
}

}  // namespace fgb
