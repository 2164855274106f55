/*
 * fast_gb300.h -- C ABI of the GB300 implementation of the FastS structured
 * solve step.  Plain pointers and sizes only; every call returns an int
 * status (FGB_OK = 0) and never exits the process; fgb_last_error() gives the
 * message of the last failure on the calling thread.
 *
 * The reference crosses the Python/C boundary in the CPython module `fasts`
 * (FastS/FastS/fastS.cpp:25-67).  Each entry point below names the reference
 * interface it replaces.  Arrays keep the reference layout
 * (FastS/FastS/formule_param.h): structure-of-arrays q[v*NDIMDX + l] with
 * ghost cells, param_int / param_real with the FastS index map
 * (FastS/FastS/param_solver.h).  Host buffers are only read or written during
 * the call; device state lives in the solver handle.
 */
#ifndef FAST_GB300_H
#define FAST_GB300_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  FGB_OK = 0,
  FGB_ERR_ARG = 1,      /* invalid argument / unsupported numerics         */
  FGB_ERR_CUDA = 2,     /* CUDA runtime error (message has the CUDA text)  */
  FGB_ERR_DEVICE = 3,   /* a kernel reported an error through its status   */
  FGB_ERR_STATE = 4     /* call out of sequence (e.g. compute before data) */
};

typedef struct fgb_solver fgb_solver;

/* Message of the last failed call on this thread ("" if none). */
const char* fgb_last_error(void);

/* Library version and the compute capability it was built for. */
int fgb_version(int* major, int* minor, int* sm);

/* Create / destroy a solver on CUDA device `device` (one stream per solver).
 * Replaces the work dictionary built by FastC.createWorkArrays__
 * (FastC/FastC/PyTree.py:2064) and the device side of FastS.PyTree.warmup
 * (FastS/FastS/PyTree.py:341). */
int fgb_create(int device, fgb_solver** out);
int fgb_destroy(fgb_solver* s);

/* Add one structured zone.  param_int / param_real: the zone's
 * .Solver#ownData/Parameter_int|real (FastC/FastC/PyTree.py:1817-2030, with
 * the BC block appended by _BCcompact, FastC/FastC/PyTree.py:2788).
 * ti, tj, tk, vol: the metric of fasts.allocate_metric
 * (FastS/FastS/Metric/allocate_metric.cpp, list slot METRIC_TI).
 * The returned zone id is the zone's position in the solver (0, 1, ...).
 * Refused with FGB_ERR_ARG: explicit schemes other than RK1 / RK2 / RK3
 * with nssiter = rk, explicit local time stepping (EXPLOC != 0, which the
 * reference's C layer refuses too) and moving meshes (LALE != 0), DTLOC
 * other than 0 / 1, LU-SGS with nb_relax > 1 or lu_match, and zones or
 * schemes the kernels do not cover (the message names them). */
int fgb_add_zone(fgb_solver* s, const int64_t* param_int, int64_t n_int,
                 const double* param_real, int64_t n_real,
                 const double* ti, const double* tj, const double* tk,
                 const double* vol, int* zone_id);

/* Add a 1-to-1 interface (interpolation type 0 of
 * FastC/FastC/Com/setInterpTransfersFast.cpp:852-883): for t < n, receiver
 * cell rcv_idx[t] of zone rcv_zone takes the value of donor cell dnr_idx[t]
 * of zone dnr_zone (0-based cell indices into the zone arrays). */
int fgb_add_transfer(fgb_solver* s, int dnr_zone, int rcv_zone, int64_t n,
                     const int64_t* dnr_idx, const int64_t* rcv_idx);

/* Add an interpolated (overset) interface: the non-type-0 transfers of
 * FastC/FastC/Com/setInterpTransfersFast.cpp:804-960, whose arithmetic lives
 * in Cassiopee Connector (commonInterpTransfers*.h, not part of the
 * reference tree: the tensor-product formulas are restated, parity
 * unpinned).  For t < n, receiver cell rcv_idx[t] of zone rcv_zone takes
 * the sum over the donor molecule of type types[t] whose first cell is
 * dnr_idx[t] of coefficient x donor value, for every variable: type 0 / 1
 * one donor (1 coefficient), 2 trilinear 2x2x2 (8, i fastest), 22 bilinear
 * 2x2 in (i, j) (4), 3 tensor-product Lagrange 3x3x3 (3 + 3 + 3 factors for
 * i, j, k), 5 Lagrange 5x5x5 (5 + 5 + 5).  coefs: the coefficients of every
 * point one after the other (ncoefs in all).  The tc tree's ID_ subregions
 * carry exactly these arrays (PointList, PointListDonor, InterpolantsType,
 * InterpolantsDonor). */
int fgb_add_interp_transfer(fgb_solver* s, int dnr_zone, int rcv_zone, int64_t n,
                            const int64_t* dnr_idx, const int64_t* rcv_idx, const int64_t* types,
                            const double* coefs, int64_t ncoefs);

/* Wall distance of a Spalart-Allmaras zone (IFLOW 3, NEQ 6): NDIMDX doubles
 * at cell centres, ghosts included -- the FlowSolution#Centers
 * "TurbulentDistance" field that FastS reads behind the viscosity array
 * (navier_stokes_struct.for passes xmut(1+NDIMDX) to spsource_SA.for).
 * Required before the first fgb_compute of such a zone. */
int fgb_set_wall_distance(fgb_solver* s, int zone, const double* dist);

/* Solver options.  "lu_precision": 64 (default) or 32 -- FP32 LU-SGS sweeps
 * inside the FP64 defect-correction loop; "modulo_verif": residual check
 * period (FastC numerics key modulo_verif, default 200); "first_it": the
 * HOOK["FIRST_IT"] flag (0 = BDF1 step); "profile": 1 to time every kernel
 * group with CUDA events (see fgb_kernel_stats); "graph": 1 (default) to
 * replay the loops of fgb_adjoint_forward / _backward as CUDA graphs, 0 for
 * stream launches (profiling always uses stream launches); "compute_graph":
 * 1 (default) to record an fgb_compute call as a CUDA graph the second time
 * its signature comes (step range, the verification flags of its step
 * numbers, first_it, sweep precision, and the level buffers every zone's
 * time levels are in) and to replay the graph from then on, with the host
 * side of the call (level rotation) redone -- same results; calls with an
 * asynchronous upload pending, profiled calls and per-zone side-stream
 * launches run as stream launches; any state-changing call (a changed
 * option, a zone, a transfer, a wall distance, a BC state, the adjoint)
 * drops the recorded graphs; fgb_get_option("step_graphs") counts them;
 * "zone_streams":
 * 1 (default) to run the per-zone kernels of several zones on 8 side streams
 * (zone m on stream m mod 8, joined before each LU-SGS solve and after each
 * ghost fill), 0 for the solver stream alone (profiling uses it alone);
 * "lu_grid": 0 (default) for one persistent LU-SGS sweep CTA per resident
 * slot of the device, n > 0 for at most n CTAs (each CTA then takes more
 * cells of a hyperplane: same results, a schedule for testing);
 * "lu_mode": 2 (default) dataflow LU-SGS sweeps (chunks of 32 cells of a
 * hyperplane, point-to-point completion marks), 1 persistent sweeps with a
 * grid barrier per hyperplane, 0 one launch per hyperplane (same results);
 * "lu_poll_limit": polls before a dataflow wait gives up (default 2^22; a
 * grid-barrier wait gives up after 4 times as many), after which
 * fgb_synchronize reports FGB_ERR_DEVICE; "lu_wait_skew": test support, 0
 * (raises the marks and barrier targets the waits expect, so that they run
 * out); "lu_prefetch": 1 (default) to prefetch into L2 the operands of a
 * dataflow chunk that no earlier plane produced before its dependency wait,
 * 0 not to (same results);
 * "batch": 1 (default) to run the coefficient, Spalart-Allmaras source,
 * face and balance / update kernels of several zones as one launch per kind
 * of zone (zone type, scheme, slope, viscosity, NEQ; up to 40 zones a
 * launch), 0 for per-zone launches (same results); "autotune": 1 (default)
 * to pick the batched face kernels' block size by timing the candidates on
 * the first batch of each kind (kept per device for the process), and the
 * LU-SGS schedule of each zone group and sweep precision by timing the
 * grid-barrier sweep and the dataflow sweep (CTAs of 8 warps, 1, 2 or 4 per
 * SM; CTAs of 4 warps, 1 or 2 per SM) on its first solve.  fgb_get_option
 * also reads "lu_tuned" / "lu_tuned32": the first group's FP64 / FP32
 * choice as 1000 x warps per CTA (dataflow) + 10 x lu_mode + CTAs per SM
 * (-1 before the first solve). */
int fgb_set_option(fgb_solver* s, const char* key, double value);
int fgb_get_option(fgb_solver* s, const char* key, double* value);

/* Host <-> device copies of one time level of one zone (NEQ*NDIMDX doubles).
 * level 0 = n (FlowSolution#Centers "Density"... compacted), 1 = n-1
 * ("..._M1"), 2 = n+1 ("..._P1").  These are the arrays the reference's
 * _computePT reads in place through K_PYTREE::getValueAF
 * (FastS/FastS/Compute/computePT.cpp:140-260). */
int fgb_upload_state(fgb_solver* s, int zone, int level, const double* host);
/* As fgb_upload_state, without waiting for the copy: when the host buffer
 * lies in memory page-locked by fgb_pin_host, the copy runs on a side stream
 * after the solver's work so far, and the solver stream waits for it before
 * the level's first use (level n-1 of an implicit step: the balance of the
 * first sub-step, after its coefficients and face fluxes); every other call
 * waits for it first.  The buffer must not change until a call that
 * synchronizes (fgb_synchronize, fgb_download_state).  Other buffers: the
 * synchronous upload. */
int fgb_upload_state_async(fgb_solver* s, int zone, int level, const double* host);
int fgb_download_state(fgb_solver* s, int zone, int level, double* host);

/* Work arrays for inspection: which = "drodm" (NEQ*NDIMDX), "coe"
 * (NEQ*NDIMDX), "xmut" (NDIMDX), "dist" (NDIMDX, Spalart-Allmaras zones),
 * "rdm" (nssiter*NEQ*2*n_lu_blocks). */
int fgb_download_work(fgb_solver* s, int zone, const char* which, double* host,
                      int64_t n);

/* One call of the solve step: replaces fasts._computePT(zones, metrics,
 * nitrun, nstep_deb, nstep_fin, layer_mode, nit_c, hook)
 * (FastS/FastS/Compute/computePT.cpp:44-721): nit_c physical steps of
 * sub-steps nstep_deb..nstep_fin, each followed by the time-level rotation
 * M1 <- N <- P1.  layer_mode must be 1 (the "c" layer).  Asynchronous on the
 * solver stream; errors of the kernels are reported by fgb_synchronize. */
int fgb_compute(fgb_solver* s, int nitrun, int nstep_deb, int nstep_fin,
                int layer_mode, int nit_c);

/* Ghost-cell fill of one time level of every zone: replaces
 * fasts._applyBC(zones, metrics, hook, nstep, var) (FastS/FastS/BC/applyBC.cpp)
 * together with the 1-to-1 transfers of FastS.PyTree._fillGhostcells
 * (FastS/FastS/PyTree.py:1162). */
int fgb_apply_bc(fgb_solver* s, int level);

/* Newton residual history of the last verified step, reduced over LU blocks
 * as in fasts.display_ss_iteration (FastS/FastS/DISPLAY/
 * display_ss_iteration.cpp:112-145): out[ne*nit + it] = L2,
 * out[(neq+ne)*nit + it] = Loo for it < nit (nit = number of sub-iterations
 * recorded); returns nit through *nit_out. */
int fgb_residuals(fgb_solver* s, int zone, double* out, int64_t n, int* nit_out);

/* CFL statistics of the last verified iteration (the first sub-step of an
 * iteration with nitrun % modulo_verif == 0), as cptst3.for -> cpcfl3.for
 * computes them and FastS/FastS/Compute/computePT.cpp:629-644 reduces them
 * into the zone's CFL_minmaxmoy node: out[0] = max, out[1] = min, out[2] =
 * mean over the interior cells of dt / min(viscous, convective) time step
 * (the convective one for Euler).  Waits for the solver stream. */
int fgb_cfl(fgb_solver* s, int zone, double* out);

/* Page-lock a host buffer (cudaHostRegister) that fgb_upload_state /
 * fgb_download_state copy, so that those copies run as DMA at the link's
 * bandwidth.  The buffer must stay allocated until fgb_destroy, which
 * unregisters it.  Registering the same pointer twice is a no-op. */
int fgb_pin_host(fgb_solver* s, void* ptr, int64_t bytes);

/* Exterior state (conservative ro, ro u, ro v, ro w, ro E) of every farfield
 * / inflow / outflow BC of a zone, replacing the free stream (BCzone.cpp
 * DEFAULT_STATE, or the nbdata = 21 per-BC state). */
int fgb_set_bc_state(fgb_solver* s, int zone, const double* st);

/* Differentiation of the explicit solve of a 2-d Euler zone (RK3, Roe +
 * van Albada MUSCL, slip walls, characteristic farfield, self 1-to-1
 * interfaces); no reference counterpart.
 * fgb_adjoint_forward: from the state at level 0 (its ghosts filled here),
 *   nsteps RK3 steps, keeping every ckpt-th state; the final state replaces
 *   level 0.
 * fgb_adjoint_backward: given dJ/dW_final (NEQ*NDIMDX, host), the gradient
 *   of J with respect to the initial state (NEQ*NDIMDX), the metric arrays ti
 *   and tj (2*NDIMDX_MTR each), vol (NDIMDX_MTR) and the farfield state (5),
 *   by the discrete adjoint of every stage (segments recomputed from their
 *   checkpoints, then swept in reverse).
 * fgb_tangent: the forward-mode derivative dW_final of the same run for
 *   perturbations of the initial state, ti, tj, vol and the farfield state. */
int fgb_adjoint_forward(fgb_solver* s, int zone, int nsteps, int ckpt);
int fgb_adjoint_backward(fgb_solver* s, int zone, const double* lam_final, double* lam_w0,
                         double* lam_ti, double* lam_tj, double* lam_vol, double* lam_st);
int fgb_tangent(fgb_solver* s, int zone, int nsteps, const double* dw0, const double* dti,
                const double* dtj, const double* dvol, const double* dst, double* dw_final);

/* Size, in doubles, of the fixed device array that holds the per-block
 * partials of fgb_residual_norms_noalloc (256 KB): a zone qualifies when
 * 2 * neq * (its number of LU blocks) <= FGB_NORM_PARTIALS_MAX, i.e. up to
 * 3276 blocks of SIZE_SSDOM cells for neq = 5. */
#define FGB_NORM_PARTIALS_MAX 32768

/* Residual norms of a zone's current right-hand side, reduced on the device
 * into the caller's device buffer, with no memory allocated:
 *   out_dev[ne] = L2,  out_dev[neq + ne] = Loo   (ne < neq)
 * with the LU-block decomposition, summation order and 1/DTC scaling of
 * fgb_residuals, so on the same state the values equal the last column that
 * entry reports.  Implicit (dual time, LU-SGS) zones only: an explicit zone's
 * right-hand-side array holds the RK3 stage combination, not a residual, and
 * is rejected with FGB_ERR_ARG.  out_dev: 2*neq doubles of device memory on the solver's
 * device.  Asynchronous on the solver stream; fgb_synchronize waits for it.
 *
 * For callers that cannot allocate: a convergence monitor that runs between
 * solves on a stream shared with other work (a device allocation or free can
 * synchronize the whole device, and fgb_residuals also allocates host memory,
 * copies the full block table back and waits for the stream), or a process
 * that reserved all of its device memory up front.  No device memory and, on
 * success, no host memory is allocated; the per-block partials go to one
 * fixed array per device of FGB_NORM_PARTIALS_MAX doubles that is part of the
 * library's device image.  Zones that need more are rejected with
 * FGB_ERR_ARG.  Nothing in that array has to start at zero: each call writes
 * every slot it reads.
 *
 * The first call on a device does a one-time set-up (it looks up the array's
 * device address, which may load the library's device code); make that first
 * call before any stream capture.  The array is shared by every solver on the
 * device, so calls whose work can overlap in time (solvers on different
 * streams, calls from several host threads) race on it: serialize them.
 *
 * No counterpart in the reference (its norms are reduced on the host, in
 * display_ss_iteration.cpp). */
int fgb_residual_norms_noalloc(fgb_solver* s, int zone, double* out_dev);

/* Wait for the solver stream and report any kernel error. */
int fgb_synchronize(fgb_solver* s);

/* Per-kernel timing (option "profile" = 1): CUDA events recorded on the
 * solver stream around each kernel group.  index >= 0: name, number of
 * timed groups and total milliseconds of group `index` (count = 0 past the
 * last group); index < 0: clear the records, *count = number of groups. */
int fgb_kernel_stats(fgb_solver* s, int index, char* name, int name_len, int64_t* count,
                     double* total_ms);

/* Kernel launches issued by the solver since creation (for launch counts). */
int fgb_launch_count(fgb_solver* s, int64_t* count);

/* Device time of a region of the solver stream: op = 0 records the start
 * event, op = 1 records the stop event, waits for it and returns the elapsed
 * milliseconds in *ms.  (Measurement support; no reference counterpart.) */
int fgb_stream_timer(fgb_solver* s, int op, double* ms);

/* Measured FP64 FMA throughput of device `device` in GFLOP/s (2 flops per
 * FMA): the compute roof of the FP64 kernels.  (Measurement support; no
 * reference counterpart.) */
int fgb_fp64_peak(int device, double* gflops);


#ifdef __cplusplus
}
#endif
#endif
