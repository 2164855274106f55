// fgb_kernels.cuh -- launch interfaces of the solve-step kernels, shared by
// the kernel translation units and the host orchestration (fgb_capi.cu).
#pragma once
#include "fgb_common.cuh"

namespace fgb {

// fgb_flux.cu: face fluxes + fused init_rhs / RK3 stage / BDF residual
struct StageArgs {
  const double* Fi; const double* Fj; const double* Fk;
  double* drodm;
  const double* coe;
  // explicit: rop_out = RK stage of rop_in; implicit: BDF residual from
  // rop_in (W^p), rop_n (W^n), rop_n1 (W^{n-1})
  const double* rop_in; double* rop_out;
  const double* rop_n; const double* rop_n1;
  double coefH; int zero_init;       // init_rhs.for
  double coefW;                      // core3ark3.for
  double c1, c2, c3; int first_sub;  // core3as2.for
  int mode;   // 0: balance + update, 1: balance into drodm only, 2: update from drodm only
};
// BC/correct_flux.for, wall BCs with the Roe scheme: one wall BC window
struct WallCorrArgs {
  const int32_t* l;      // cell on the high side of the wall face
  const int32_t* l0;     // interior cell receiving the correction
  const int32_t* lt;     // metric index of the face
  const double* nrm;     // [n][3] raw face normal (tijk * c_mtr)
  int64_t n;
  int dir, slip;         // face direction; bflwallslip (1) or bflwall (0)
  double sens_c, sens_w, rgp, gam2;
};
cudaError_t launch_wall_corr(const Zone& z, const double* q, double* drodm, const WallCorrArgs& a,
                             cudaStream_t st);

// Zone batches: one launch of a kernel over up to BATCH_MAX zones of one
// kind (the same template instance).  The entries travel in the kernel
// parameter (__grid_constant__, at most 32 KB); block b of the launch works
// on zone m with bstart[m] <= b < bstart[m + 1] (bstart[nz] = grid size).
constexpr int BATCH_MAX = 40;
struct FaceEntry { Zone z; const double* q; const double* xmut; double* F[3]; };
struct FaceBatch { int nz; int block; int64_t bstart[BATCH_MAX + 1]; FaceEntry e[BATCH_MAX]; };
struct StageEntry { Zone z; StageArgs a; };
struct StageBatch { int nz; int64_t bstart[BATCH_MAX + 1]; StageEntry e[BATCH_MAX]; };
struct SaEntry { Zone z; const double* q; double* drodm; double* coe; };
struct SaBatch { int nz; double coefH; int zero_init, lu; int64_t bstart[BATCH_MAX + 1]; SaEntry e[BATCH_MAX]; };
// faces of every direction of a batch (block: threads per block, chosen by
// the autotuner; the caller fills z, q, xmut, F of each entry); the zones
// share the kind of e[0].z (zone type, scheme, slope, viscosity, NEQ)
cudaError_t launch_faces_batch(FaceBatch& b, cudaStream_t st);
// the block sizes launch_faces_batch may use, and a key of the kind of zone z
int faces_batch_blocks(int* out, int nmax);
int64_t faces_kind_key(const Zone& z);
cudaError_t launch_assemble_batch(StageBatch& b, bool implicit, cudaStream_t st);
cudaError_t launch_sa_source_batch(SaBatch& b, cudaStream_t st);
cudaError_t launch_faces(const Zone& z, const double* q, const double* xmut, double* Fi,
                         double* Fj, double* Fk, cudaStream_t st);
cudaError_t launch_wiggle(const Zone& z, const double* q, double* wig, cudaStream_t st);
cudaError_t launch_shock_sensor(const Zone& z, const double* q, double* wig, cudaStream_t st);
cudaError_t launch_assemble(const Zone& z, const StageArgs& a, bool implicit, cudaStream_t st);
// Spalart-Allmaras source of the sub-step (init_rhs of equation 6 fused in);
// lu: also coe(:,6) for the LU-SGS sweeps (first implicit sub-step)
cudaError_t launch_sa_source(const Zone& z, const double* q, double* drodm, double* coe,
                             double coefH, int zero_init, int lu, cudaStream_t st);

// fgb_lu.cu: coefficients and LU-SGS
struct CoeArgs {
  const double* rop; const double* xmut_in; double* xmut; double* coe;
  int64_t lo[3], hi[3];      // Fortran index range (may include ghosts)
  int do_invist, do_lu, first_it;
  int do_sa;                 // SA/vispalart.for instead of invist.for
  double coesut, cmus1;      // invist.for constants
};
// natural-order fields of one zone's LU solve
struct LuFields {
  const double* rop_old;    // W^p
  double* rop_new;          // W^{p+1}
  const double* coe;        // coefficients
  const double* din;        // Newton residual
  const int32_t* posmap;    // natural index -> group plane index (-1 outside the LU range)
  int inplace;              // upper sweep reads the k+1 neighbour after its update
};
// one zone of an LU group as the sweep kernels see it
struct LuZone { Zone z; LuFields f; };

// One LU-SGS solve of a group of zones of one kind (zone type, equation
// count).  The plane-ordered arrays hold every interior cell of every zone
// of the group: plane s = the cells with i+j+k = s of zone 0, then of zone 1,
// ...  One persistent cooperative launch (one bounded grid barrier per
// plane) or one launch per plane sweeps all zones together, so a group of
// small blocks costs the barriers of its largest block, not of their sum.
// FP64 or FP32 sweeps (mixed precision; the Newton update stays FP64).
// Dataflow schedule of the sweeps (lusgs_flow): chunks of 32 consecutive
// cells of a hyperplane, their completion marks and dependency ranges.
constexpr int FLOW_DEP = 8;     // dependency table entries per dataflow chunk
struct FlowArgs {
  unsigned long long* ticket;   // zeroed before each launch
  int* flag;                    // [nchunk] completion mark of each chunk (never cleared)
  const int32_t* cplane;        // [nchunk] hyperplane of each chunk
  const int64_t* cbase;         // [smax + 2] first chunk of each hyperplane
  const int32_t* dep;           // [nchunk][FLOW_DEP]: the chunks holding the lower
                                // neighbours (plane s-1) as two ranges [lo, hi], then
                                // the upper ones (plane s+1); an empty range is [0, -1]
  int64_t nchunk;
  int lower_mark, upper_mark;   // 2 epoch + 1, 2 epoch + 2 (published)
  int wait_skew;                // added to the marks a wait expects (0; > 0 only in tests)
  int* err;                     // device error word (2: a wait gave up)
  long long poll_limit;
  int prefetch;                 // 1: L2 prefetch of a chunk's cold operands before its wait
};
int lusgs_flow_chunk();

struct LuGroup {
  int persistent;           // 0 one launch per plane, 1 grid barrier, 2 dataflow
  int flow_per_sm;          // dataflow: CTAs per SM (0: one)
  int flow_threads;         // dataflow: threads per CTA (0: 256; a multiple of 32, at most 256)
  FlowArgs flow;
  int grid_cap;             // > 0: at most this many CTAs in the persistent sweep
  int fp32;
  unsigned int* bar;        // barrier counter (zeroed by the launcher)
  int* err;                 // device error word (barrier time-out)
  void* work;               // GG * lusgs_work_words(typ) words of the sweep precision
  int64_t GG;               // interior cells of the group
  int64_t smax;             // last hyperplane over the group
  const uint32_t* cells;    // packed i | j<<11 | k<<22 per group plane index
  const int32_t* zid;       // zone (position in the group) per group plane index
  const int64_t* plane;     // device plane offsets (smax + 2)
  const int64_t* plane_host;
  int32_t* nbl;             // [3][GG] lower neighbours (group plane index or -1)
  int32_t* nbu;             // [3][GG] upper neighbours
  LuZone* ztab;             // device zone table of this solve (nz entries)
  int nz;
};
int64_t lusgs_work_words(int typ);
// neighbour tables of a group (ztab must hold every zone's z and f.posmap)
cudaError_t launch_lu_neighbours(const LuGroup& G, cudaStream_t st);
cudaError_t launch_coefficients(const Zone& z, const CoeArgs& a, cudaStream_t st);
struct CoeEntry { Zone z; CoeArgs a; };
struct CoeBatch { int nz; int64_t bstart[BATCH_MAX + 1]; CoeEntry e[BATCH_MAX]; };
cudaError_t launch_coefficients_batch(const CoeBatch& b, cudaStream_t st);
// gather of every zone, sweeps, Newton update; ztab_host = the nz entries
// already copied to G.ztab on the stream
cudaError_t launch_lusgs(const LuZone* ztab_host, const LuGroup& G, cudaStream_t st);

// fgb_ghost.cu: ghost fill and residual norms
struct NormArgs {
  const double* drodm;
  double* rdm;
  int64_t ijkv_lu[3];   // number of LU blocks per direction
  int64_t size[3];      // SIZE_SSDOM
  int64_t nssiter;
  int it_bloc;          // 1-based sub-iteration slot
  int neq;
};
cudaError_t launch_gather(double* dst, int64_t nd_dst, const double* src, int64_t nd_src,
                          const int32_t* d_idx, const int32_t* s_idx, int64_t n, int neq,
                          int op, double c, cudaStream_t st);
enum { BCF_SLIP = 0, BCF_NOSLIP = 1, BCF_FARFIELD = 2, BCF_OUTFLOW = 3, BCF_OUTPRES = 4 };
struct BcFaceArgs {            // one face BC window (bc_face)
  const int32_t* dst;          // ghost cells
  const int32_t* src;          // mirror cell (walls) or first interior cell
  const double* nrm;           // [n][3] raw face normal (x snorm for farfield / outflow)
  int64_t n, nd;
  int op;
  double gam, gam1, gam1_1, cv, cvinv;
  double st[5];                // exterior state (conservative)
  int sa, inflow;              // Spalart-Allmaras zone; BCInflow (nutilde imposed)
  double nue;                  // exterior nutilde (state(6) / state(1))
  int dir;                     // face direction of the window (0 i, 1 j, 2 k)
};
// All face-BC windows of a zone as one list: per entry its ghost cell,
// source cell, raw normal, face metric index and window (lid), the
// window's parameters in lp[lid] (device memory)
struct BcFaceCat {
  const int32_t *dst, *src, *lid, *mt;
  const double* nrm;
  int64_t n;
  const BcFaceArgs* lp;
  const double* aux;           // per entry: imposed pressure (BCOutpres), else 0
};
// All gather windows of a zone (periodic, extrapolation) as one list with
// the operation of each entry (0 copy, 1 max(-1e30, x))
struct GatherCat {
  const int32_t *dst, *src, *op;
  int64_t n;
};
struct BcNextArgs {            // farfield / inflow ghost ranks past the first
  const int32_t *dst, *q0, *q1, *q2;   // one entry per ghost line: its second rank
  int64_t n, nd;
  double k1, k2, k3;
  int sa;
  int nrank;                   // ranks past the first (ghost layers - 1), one after the other
};
cudaError_t launch_bc_face_cat(double* q, const BcFaceCat& c, cudaStream_t st);
// Every 1-to-1 transfer of a solver in one launch: entry t copies cell
// di[t] of zone dz[t] into ghost cell ri[t] of zone rz[t] (all variables);
// the zones' current level pointers travel as a kernel parameter
constexpr int ZT_MAX = 64;
struct ZoneLevels { double* q[ZT_MAX]; int64_t nd[ZT_MAX]; int neq[ZT_MAX]; int ng[ZT_MAX]; };
cudaError_t launch_transfer_all(const ZoneLevels& zl, const int32_t* rz, const int32_t* ri,
                                const int32_t* dz, const int32_t* di, int64_t n, cudaStream_t st);
// Interpolated transfers of one donor / receiver zone pair (sj, sk: the
// donor's j and k cell strides; coff: first coefficient of each point)
cudaError_t launch_transfer_interp(double* dst, int64_t nd_dst, const double* src, int64_t nd_src,
                                   int64_t sj, int64_t sk, const int32_t* ri, const int32_t* di,
                                   const int32_t* ty, const int64_t* coff, const double* coef,
                                   int64_t n, int neq, cudaStream_t st);
cudaError_t launch_gather_cat(double* q, int64_t nd, const GatherCat& c, int neq, cudaStream_t st);
// The BC lists of every zone of a solver concatenated with the zone of each
// entry (zface, zgat, znext, zcoin); corners: cc < 0 marks an edge
struct FillAll {
  BcFaceCat face; const int32_t* zface;
  GatherCat gat; const int32_t* zgat;
  BcNextArgs next; const int32_t* znext;
  const int32_t *cdst, *ca, *cb, *cc, *zcoin; int64_t ncoin;
};
cudaError_t launch_fill_all(const ZoneLevels& zl, const FillAll& f, cudaStream_t st);
cudaError_t launch_bc_next(double* q, const BcNextArgs& a, cudaStream_t st);
cudaError_t launch_coins(double* q, int64_t nd, const int32_t* dst, const int32_t* a,
                         const int32_t* b, const int32_t* c, int64_t n_edge, int64_t n, int neq,
                         cudaStream_t st);
// cpcfl3.for: (max, min, mean) CFL of a zone into out[3]; part holds
// 3 * cfl_partial_blocks(z) doubles
int64_t cfl_partial_blocks(const Zone& z);
cudaError_t launch_cfl(const Zone& z, const double* q, const double* xmut, double* part,
                       double* out, cudaStream_t st);
cudaError_t launch_norms(const Zone& z, const NormArgs& a, cudaStream_t st);
cudaError_t norm_partials_address(double** p);   // the fixed partials array of this device
cudaError_t launch_norms_finish(const double* part, int64_t nblocks, int neq, double xpt_1,
                                double dtc, double* out, cudaStream_t st);
cudaError_t run_fp64_probe(int nsm, int iters, double* out, cudaStream_t st);

// fgb_adjoint.cu: tangent / adjoint of the explicit 2-d Euler step (Roe +
// van Albada), from local Jacobians of the face flux, BC and update formulas
// Face tape of the adjoint's recomputation (2-d Roe + van Albada faces):
// FACE_TAPE doubles per face, face-major; slots 0..8 = |S| and the Roe
// values of roe_full<true>, TAPE_VA.. = van Albada slopes (variable m, side
// qm / qp), TAPE_ID.. = reciprocals of their denominators.  A stage's tape =
// FACE_TAPE * (i faces + j faces) doubles, the i faces first.
constexpr int FACE_TAPE = 25, TAPE_VA = 9, TAPE_ID = 17;
cudaError_t launch_faces_tape(const Zone& z, const double* q, double* Fi, double* Fj, double* tape,
                              cudaStream_t st);
cudaError_t launch_adj_faces(const Zone& z, const double* q, const double* tape,
                             const double* lamD, double* lamQ,
                             double* lamTi, double* lamTj, cudaStream_t st);
cudaError_t launch_tan_faces(const Zone& z, const double* q, const double* dq, const double* dTi,
                             const double* dTj, double* dFi, double* dFj, cudaStream_t st);
cudaError_t launch_adj_update(const Zone& z, const double* q, const double* D, double coefW,
                              double* lamOut, double* lamIn, double* lamD, double* lamVol,
                              cudaStream_t st);
cudaError_t launch_tan_balance(const Zone& z, double coefH, int zero, const double* dFi,
                               const double* dFj, double* dD, cudaStream_t st);
cudaError_t launch_tan_apply(const Zone& z, const double* q, const double* D, double coefW,
                             const double* dIn, const double* dD, const double* dVol, double* dOut,
                             cudaStream_t st);
cudaError_t launch_adj_wall(const Zone& z, const double* q, const double* tape,
                            const double* lamD, double* lamQ,
                            double* lamTi, double* lamTj, const WallCorrArgs& a, cudaStream_t st);
cudaError_t launch_tan_wall(const Zone& z, const double* q, const double* dq, const double* dTi,
                            const double* dTj, double* dD, const WallCorrArgs& a, cudaStream_t st);
cudaError_t launch_adj_bc_face_cat(const double* q, double* lam, const BcFaceCat& c, int64_t ndm,
                                   double* lamTi, double* lamTj, double* lamSt, cudaStream_t st);
cudaError_t launch_tan_bc_face_cat(const double* q, double* dq, const BcFaceCat& c, int64_t ndm,
                                   const double* dTi, const double* dTj, const double* dSt,
                                   cudaStream_t st);
cudaError_t launch_lin_bc_next(const double* q, double* x, const BcNextArgs& a, int adjoint, int nv,
                               cudaStream_t st);
cudaError_t launch_adj_gather(double* lam, int64_t nd, const int32_t* d_idx, const int32_t* s_idx,
                              int64_t n, int nv, cudaStream_t st);
cudaError_t launch_scale(double* x, int64_t n, double c, cudaStream_t st);
cudaError_t launch_adj_coins(double* lam, int64_t nd, const int32_t* dst, const int32_t* a,
                             const int32_t* b, const int32_t* c, int64_t n_edge, int64_t n, int nv,
                             cudaStream_t st);

}  // namespace fgb
