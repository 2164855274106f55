// fgb_ghost.cu -- ghost-cell fill and residual-norm reduction (sm_103a).
//
// Ghost fill replaces FastS/FastS/BC/BCzone.cpp (periodic tag 11 through
// bvbs_periodique.for, extrapolation tag 0 through bvbs_extrapolate.for),
// FastS/FastS/BC/correct_coins.for (edges/corners) and the 1-to-1 branch of
// FastC/FastC/Com/setInterpTransfersFast.cpp:852-883.  All of these are pure
// gathers once the index arithmetic is done, so the host resolves every
// window to (destination, source) cell lists once per zone and the device
// runs one gather kernel per list: coalesced on the destination side, no
// atomics, no ordering constraints inside a list.  The lists run in the
// reference's order: transfers, then face BCs, then edges/corners (which read
// only face ghosts).
//
// The residual norms replace FastS/FastS/Compute/cprdu3s1_incl.for: one CTA
// per LU block reduces sum(drodm^2) and max|drodm| per equation with warp
// shuffles.
#include "../../include/fast_gb300.h"
#include "fgb_kernels.cuh"

namespace fgb {

// dst[v*nd_dst + d_idx[t]] = op(src[v*nd_src + s_idx[t]])
// op: 0 = copy, 1 = zeroth-order extrapolation max(-1e30, x), 2 = scale by c
__global__ void __launch_bounds__(256) gather_copy(double* __restrict__ dst, int64_t nd_dst,
                                                   const double* __restrict__ src, int64_t nd_src,
                                                   const int32_t* __restrict__ d_idx,
                                                   const int32_t* __restrict__ s_idx, int64_t n,
                                                   int neq, int op, double c) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int64_t d = d_idx[t], s = s_idx[t];
  for (int v = 0; v < neq; v++) {
    double x = src[s + v * nd_src];
    if (op == 1) x = fmaxF(-1.e30, x);
    if (op != 0) x = x * c;
    dst[d + v * nd_dst] = x;
  }
}

// correct_coins.for: edge = (a + b) * 0.5, corner = (a + b + c) * (1/3)
__global__ void __launch_bounds__(256) coins(double* __restrict__ q, int64_t nd,
                                             const int32_t* __restrict__ dst,
                                             const int32_t* __restrict__ a,
                                             const int32_t* __restrict__ b,
                                             const int32_t* __restrict__ c, int64_t n_edge,
                                             int64_t n, int neq) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const double c3 = 1. / 3.;
  for (int v = 0; v < neq; v++) {
    const double* Q = q + v * nd;
    double x;
    if (t < n_edge) x = (Q[a[t]] + Q[b[t]]) * 0.5;
    else x = (Q[a[t]] + Q[b[t]] + Q[c[t]]) * c3;
    q[dst[t] + v * nd] = x;
  }
}

cudaError_t launch_gather(double* dst, int64_t nd_dst, const double* src, int64_t nd_src,
                          const int32_t* d_idx, const int32_t* s_idx, int64_t n, int neq,
                          int op, double c, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  gather_copy<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(dst, nd_dst, src, nd_src, d_idx, s_idx,
                                                           n, neq, op, c);
  return cudaGetLastError();
}

cudaError_t launch_coins(double* q, int64_t nd, const int32_t* dst, const int32_t* a,
                         const int32_t* b, const int32_t* c, int64_t n_edge, int64_t n, int neq,
                         cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  coins<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(q, nd, dst, a, b, c, n_edge, n, neq);
  return cudaGetLastError();
}

// ------------------------------------------------------------ norms
// One CTA per LU block (cprdu3s1_incl.for:14-135 block decomposition).
__global__ void __launch_bounds__(256) block_norms(Zone z, NormArgs a) {
  const int64_t no = blockIdx.x;
  const int64_t k_lu = no / (a.ijkv_lu[0] * a.ijkv_lu[1]);
  const int64_t j_lu = (no - a.ijkv_lu[0] * a.ijkv_lu[1] * k_lu) / a.ijkv_lu[0];
  const int64_t i_lu = no - j_lu * a.ijkv_lu[0] - k_lu * a.ijkv_lu[0] * a.ijkv_lu[1];
  const int64_t N[3] = {z.ni, z.nj, z.nk};
  const int64_t L[3] = {i_lu, j_lu, k_lu};
  int64_t lo[3], ext[3];
#pragma unroll
  for (int d = 0; d < 3; d++) {
    lo[d] = 1 + L[d] * a.size[d];
    int64_t hi = (L[d] + 1) * a.size[d];
    if (L[d] == a.ijkv_lu[d] - 1) hi = N[d];
    ext[d] = hi - lo[d] + 1;
  }
  double s[6] = {0, 0, 0, 0, 0, 0}, m[6] = {0, 0, 0, 0, 0, 0};
  const int64_t n = ext[0] * ext[1] * ext[2];
  for (int64_t t = threadIdx.x; t < n; t += blockDim.x) {
    int64_t i = lo[0] + t % ext[0];
    int64_t r = t / ext[0];
    int64_t j = lo[1] + r % ext[1], k = lo[2] + r / ext[1];
    int64_t l = inddm(z, i, j, k);
    for (int ne = 0; ne < a.neq; ne++) {
      double x = a.drodm[l + ne * z.nd];
      s[ne] += x * x;
      m[ne] = fmaxF(m[ne], fabs(x));
    }
  }
  __shared__ double ss[8][6], sm[8][6];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int ne = 0; ne < a.neq; ne++) {
    double x = s[ne], y = m[ne];
    for (int o = 16; o > 0; o >>= 1) {
      x += __shfl_down_sync(0xffffffffu, x, o);
      y = fmaxF(y, __shfl_down_sync(0xffffffffu, y, o));
    }
    if (lane == 0) { ss[warp][ne] = x; sm[warp][ne] = y; }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const int nw = (blockDim.x + 31) / 32;
    for (int ne = 0; ne < a.neq; ne++) {
      double x = 0., y = 0.;
      for (int w = 0; w < nw; w++) { x += ss[w][ne]; y = fmaxF(y, sm[w][ne]); }
      const int64_t base = (a.it_bloc - 1) + ne * a.nssiter + no * a.neq * 2 * a.nssiter;
      a.rdm[base] = x;
      a.rdm[base + a.neq * a.nssiter] = y;
    }
  }
}

cudaError_t launch_norms(const Zone& z, const NormArgs& a, cudaStream_t st) {
  unsigned nb = (unsigned)(a.ijkv_lu[0] * a.ijkv_lu[1] * a.ijkv_lu[2]);
  block_norms<<<nb, 256, 0, st>>>(z, a);
  return cudaGetLastError();
}

// ------------------------------------------- norms into a fixed scratch
// fgb_residual_norms_noalloc keeps its per-block partials here instead of in
// an allocation: a module global, so one array per device, created with the
// library's device image.  Slots [no * 2 * neq, (no + 1) * 2 * neq) belong to
// LU block no; block_norms writes all of them before norms_finish reads them,
// so nothing has to start at zero.
static __device__ __align__(256) double g_norm_partials[FGB_NORM_PARTIALS_MAX];

cudaError_t norm_partials_address(double** p) {
  return cudaGetSymbolAddress((void**)p, g_norm_partials);
}

// Sum (L2^2) and maximum (Loo) of the partials over the blocks, in block
// order, then the scaling of display_ss_iteration.cpp:112-145: one thread
// per equation, the same operations in the same order as fgb_residuals'
// host loop.
__global__ void __launch_bounds__(32) norms_finish(const double* __restrict__ part, int64_t nblocks,
                                                   int neq, double xpt_1, double dtc,
                                                   double* __restrict__ out) {
  const int ne = threadIdx.x;
  if (ne >= neq) return;
  double rmoy = 0., rmax = 0.;
  for (int64_t no = 0; no < nblocks; no++) {
    const double* q = part + no * 2 * neq;
    const double m = q[neq + ne];
    rmax = rmax < m ? m : rmax;
    rmoy = rmoy + q[ne];
  }
  out[ne] = sqrt(rmoy * xpt_1) / dtc;
  out[neq + ne] = rmax / dtc;
}

cudaError_t launch_norms_finish(const double* part, int64_t nblocks, int neq, double xpt_1,
                                double dtc, double* out, cudaStream_t st) {
  norms_finish<<<1, 32, 0, st>>>(part, nblocks, neq, xpt_1, dtc, out);
  return cudaGetLastError();
}

}  // namespace fgb

namespace fgb {
// FP64 FMA throughput probe: 8 independent FMA chains per thread, grid =
// 8 CTAs of 256 threads per SM.  __fma_rn is an explicit FMA (unaffected by
// --fmad=false).  The result is written so the chains are not removed.
__global__ void __launch_bounds__(256) fp64_fma_probe(double* out, int iters, double a, double b) {
  double x[8];
#pragma unroll
  for (int i = 0; i < 8; i++) x[i] = threadIdx.x * 1e-9 + i;
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int i = 0; i < 8; i++) x[i] = __fma_rn(x[i], a, b);
  }
  double s = 0.;
#pragma unroll
  for (int i = 0; i < 8; i++) s += x[i];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

cudaError_t run_fp64_probe(int nsm, int iters, double* out, cudaStream_t st) {
  fp64_fma_probe<<<nsm * 8, 256, 0, st>>>(out, iters, 0.999999, 1e-7);
  return cudaGetLastError();
}
}  // namespace fgb
