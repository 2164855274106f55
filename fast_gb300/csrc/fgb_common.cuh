// fgb_common.cuh -- zone descriptor, index maps and FP64 helpers shared by
// the sm_103a kernels of the FastS solve step.
//
// Memory layout in HBM is FastS's own (FastS/FastS/formule_param.h):
// structure-of-arrays, one contiguous block per variable,
//   q[v*nd + l],  l = (i+ng-1) + (j+ng-1)*nip + (k+ngk-1)*nip*njp
// with Fortran cell indices i in [1-ng, ni+ng] (ng = 2 ghost layers, ngk = 0
// for a 2-d zone).  Keeping the reference layout makes every host<->device
// copy a single memcpy of the pyTree's compacted time-level array.
//
// All FP64 kernels are compiled with --fmad=false and evaluate expressions in
// the reference's left-to-right order, so their results are the reference
// arithmetic bit for bit (checked against the CPU oracle in tests/).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace fgb {

// FastS param_int / param_real index map (FastS/FastS/param_solver.h)
enum PI : int {
  NIJK = 0, NIJK_MTR = 5, NIJK_XYZ = 10, IJKV = 20, MXSSDOM_LU = 24, ITYPZONE = 25,
  IFLOW = 27, ILES = 28, ITYPCP = 29, SIZE_SSDOM = 30, KFLUDOM = 33, LALE = 34, NEQ = 36,
  NEQ_IJ = 37, NEQ_K = 38, NEQ_COE = 39, NDIMDX = 41, NDIMDX_MTR = 43, DTLOC = 46, SA_INT = 47,
  RK = 52, LEVEL = 53, EXPLOC = 54, NSSITER = 58, SLOPE = 64, PT_BC = 70, NB_RELAX = 71,
  LU_MATCH = 75, SENSORTYPE = 85
};
enum PR : int {
  DTC = 0, GAMMA = 1, CVINF = 2, ROINF = 3, PINF = 4, VINF = 5, TINF = 6, MINF = 7,
  RONUTILDEINF = 8, PRANDT = 10, XMUL0 = 11, TEMP0 = 12, CS = 13, EPSI_NEWTON = 14, CFL = 15,
  SA_RATIOM = 18, VXINF = 19, VYINF = 20, VZINF = 21, PSIROE = 34, PRANDT_TUR = 38, WIG_AMP = 72
};
enum PI_SA : int { SA_LOW_RE = 130, SA_ROT_CORR = 131 };
enum ZoneType : int { Z3DFULL = 0, Z3DHOMO = 1, Z3DCART = 2, Z2D = 3 };
enum Scheme : int { AUSM = 1, SENSEUR = 2, ROE = 5 };
enum Slope : int { O1 = 1, O3 = 2, MINMOD = 3, O5 = 5, O3SC = 6, O5SC = 7, VANALBADA = 8 };   // 8: not a FastS slope

// Everything a kernel needs about one zone; passed by value.
struct Zone {
  int64_t ni, nj, nk;        // interior cells (IJKV)
  int64_t ng, ngk;           // ghost layers (i/j, k)
  int64_t nip, njp, nkp;     // cells incl. ghosts (NIJK)
  int64_t nd;                // NDIMDX
  int64_t inc[3];            // cell strides i, j, k
  int64_t minc[3];           // metric strides (NIJK_MTR)
  int64_t mg, mgk;           // metric ghost offsets
  int64_t ndm;               // NDIMDX_MTR
  int typ, iflow, kflu, slope, neq, itypcp, rk, dtloc;
  // constants of template_FluxAndBalance.for:108-156 and friends
  double gam, rgp, gam1, gam3, cv, dtc, psiroe, wig_cte, tmin_1;
  double cvinv;   // 1/cv (mjr_newton.for computes it once per call)
  const double* wig;   // senseur wiggle flags, 3 x NDIMDX (KFLUDOM = 2)
  double opt0;         // float(SENSORTYPE)
  double c1, c2, c3, c4, c5, c6, cvisq;
  double c50, c51, c52, c53, c54;   // o5 reconstruction (template_FluxAndBalance.for:149-154)
  double tcx, tcy, tcz, si, sj, sk, volinv;  // 3d cartesian metric
  // cell-independent terms of a 3d cartesian zone's coefficients (the same
  // IEEE operations as per cell, evaluated once on the host): sqrt(tc^2) of
  // each direction and dtc / vol
  double ctc2[3], cdtv;
  double ctcg[3];  // tc_d (gam - 1) of each direction (LU-SGS B entries)
  // FP32 roundings of the constants of the LU-SGS B entries (lu_*.for) and
  // of the Newton update -- gam, gam - 1, gam cv, (gam - 1) - 1, tc_d, cv,
  // 1/cv -- evaluated once on the host with the device's IEEE operations, for
  // the FP32 sweeps (a conversion from FP64 runs on the FP64 pipe, one warp
  // instruction per 64 cycles, on the sweep's critical path)
  float fgam, fgm1, fcp, fgm2, ftc[3], fcv, fcvinv, fpad;
  double rgpgam;   // rgp * gam (the sound speed squared is rgp gam T)
  double cfl;      // CFL number of the local time step (DTLOC = 1)
  double prandt, xmul0, temp0, cs;
  const double *ti, *tj, *tk, *vol;
  // Spalart-Allmaras (IFLOW 3, neq 6): Sutherland constants in the form of
  // the SA routines (coesut without sqrt(temp01)), turbulent conductivity,
  // 1/sigma, the mu_t / mu clip, the rotation / low-Re switches and the wall
  // distance (NDIMDX, natural layout)
  double sa_coesut, sa_temp01, sa_cmus1, gam4, sigma_1, ratiom, sa_rot, sa_low_re;
  const double* dist;
};

// Spalart-Allmaras constants (FastS/FastS/param_solver.h:315-327)
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

// mulam.for: laminar viscosity as the SA routines write it
__device__ __forceinline__ double sa_mulam(const Zone& z, double t) {
  return z.sa_coesut * sqrt(t * z.sa_temp01) / (1. + z.sa_cmus1 / t);
}

__host__ __device__ inline int64_t inddm(const Zone& z, int64_t i, int64_t j, int64_t k) {
  return (i + z.ng - 1) + (j + z.ng - 1) * z.nip + (k + z.ngk - 1) * z.nip * z.njp;
}
__host__ __device__ inline int64_t indmtr(const Zone& z, int64_t i, int64_t j, int64_t k) {
  return (i + z.mg - 1) * z.minc[0] + (j + z.mg - 1) * z.minc[1] + (k + z.mgk - 1) * z.minc[2];
}

// Fortran intrinsics with the semantics the reference relies on
__device__ __forceinline__ double fmaxF(double a, double b) { return a > b ? a : b; }
__device__ __forceinline__ double fminF(double a, double b) { return a < b ? a : b; }
__device__ __forceinline__ double fsignF(double a, double b) { return copysign(fabs(a), b); }

// x * (+-2^K) with the bits of the FP64 product, without an FP64 instruction
// in the common case.  GB300 issues one FP64 warp instruction per 64 cycles
// per SM sub-partition, so the FP64-bound kernels take products by powers
// of two off that pipe: when x and the product are normal numbers the
// product is x with its exponent field moved by K (exact, and so equal to
// the rounded product), an integer add on the integer pipe; zero, subnormal,
// infinite or NaN x, or a product leaving the normal range, take the FP64
// multiply in an out-of-line call (a real branch: an inlined multiply would
// be predicated and still occupy the FP64 pipe).
static __device__ __noinline__ double mul_pow2_slow(double x, double f) { return x * f; }
template <int K, bool NEG = false>
__device__ __forceinline__ double mul_pow2(double x) {
  static_assert(K >= -4 && K <= 4 && K != 0, "small power of two");
  constexpr unsigned lo = K < 0 ? 1u - K : 1u, hi = K > 0 ? 2046u - K : 2046u;
  const long long b = __double_as_longlong(x);
  const unsigned e = (unsigned)(b >> 52) & 0x7ffu;
  if (e - lo <= hi - lo) {
    long long r = K > 0 ? b + ((long long)K << 52) : b - ((long long)(-K) << 52);
    if (NEG) r ^= (long long)0x8000000000000000ull;
    return __longlong_as_double(r);
  }
  const double f = K < 0 ? 1.0 / (double)(1 << -K) : (double)(1 << K);
  return mul_pow2_slow(x, NEG ? -f : f);
}
template <int K, bool NEG = false>
__device__ __forceinline__ float mul_pow2(float x) {   // FP32: the multiply itself
  const float f = K < 0 ? 1.0f / (float)(1 << -K) : (float)(1 << K);
  return x * (NEG ? -f : f);
}

// Device error word shared by all kernels of a solver (bounded waits set it).
struct DevStatus { int code; int where; };

}  // namespace fgb
