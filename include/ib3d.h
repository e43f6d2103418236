/*
 * ib3d.h -- C ABI of the GB300 hot path of the IB3D sharp-interface immersed-
 * boundary Navier-Stokes solver.
 *
 * The reference (Fortran 90 + OpenACC) runs its per-step hot path as
 * argument-less subroutines over the module `global` (modGlobal.f90:1-106),
 * called from PROGRAM main (main.f90:5-67). Each entry point below replaces one
 * of those calls; the comment beside it names the reference interface
 * (file:line) it stands in for. A Fortran driver binds them with ISO_C_BINDING
 * (`bind(C)` interfaces) and replaces `CALL nsMomentum` by
 * `ierr = ib3d_ns_momentum(ctx)`, and so on.
 *
 * Types: int64_t is Fortran INTEGER(KIND=8), double is REAL(KIND=8).
 * 3-D arrays are the address of element (1,1,1) of a Fortran array with
 * dimensions (nx+2, ny+2, nz+2), column-major (i fastest). Index lists are
 * (n,3) INTEGER(8) column-major, 1-based.
 *
 * Ownership: the context owns all device memory; host pointers are only read or
 * written for the duration of the call. Errors: every int-returning call
 * returns IB3D_OK (0) or a negative IB3D_ERR_* code, and ib3d_last_error()
 * describes it; nothing aborts, traps or loops forever. Threading: one context
 * per host thread; work is ordered on the context's CUDA stream and a call
 * synchronises only when it returns host data.
 */
#ifndef IB3D_H
#define IB3D_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define IB3D_OK 0
#define IB3D_ERR_ARG (-1)       /* bad argument / call order */
#define IB3D_ERR_CUDA (-2)      /* CUDA runtime error or missing device */
#define IB3D_ERR_MESH (-3)      /* bad triangle index or degenerate mesh */
#define IB3D_ERR_PROBE (-4)     /* a ghost-point or drag probe left the grid */
#define IB3D_ERR_NOCONV (-5)    /* SOR hit max_sweeps; fields stay valid */
#define IB3D_ERR_NONFINITE (-6) /* NaN or Inf in a convergence scalar */
#define IB3D_ERR_MEMORY (-7)    /* device allocation failed */
#define IB3D_ERR_TOO_LARGE (-8) /* grid larger than ib3d_pressure_solve_noalloc's fixed scratch */
#define IB3D_ERR_IO (-9)        /* a restart file could not be opened, read or written */

/* SOR stopping test. */
#define IB3D_CRIT_UPDATE 0   /* max |pc - pco| over fluid cells (subPcorVcor.f90:193-210) */
#define IB3D_CRIT_RESIDUAL 1 /* max |b/dt - A pc| over fluid cells */

/* Pressure-solve arithmetic. */
#define IB3D_PREC_FP64 0     /* reference arithmetic, bit-identical to the FP64 oracle */
#define IB3D_PREC_FP32DC 1   /* FP32 red-black sweeps inside an FP64 defect-correction loop */
#define IB3D_PREC_FP64_FAST 2 /* plain FP64 method (FP64 sweeps, the reference's iteration) with
                                 contracted multiply-adds, a precomputed omega/diag per cell instead
                                 of the division, and reciprocal spacings in the divergence and the
                                 predictor: differs from IB3D_PREC_FP64 by rounding only */

/* Initial guess of the pressure correction pc at each step. */
#define IB3D_WARM_ZERO 0     /* pc = 0, as subPcorVcor.f90:19-28 */
#define IB3D_WARM_PREV 1     /* pc = previous step's pc (linear extrapolation of p) */
#define IB3D_WARM_LEARNED 2  /* pc = prediction of the attached network (ib3d_attach_net) */

/* ib3d_params.inner_schedule */
#define IB3D_INNER_FIXED 0
#define IB3D_INNER_ADAPTIVE 1
#define IB3D_INNER_TAIL 2
/* ib3d_params.outlet */
#define IB3D_OUTLET_ZERO_GRADIENT 0
#define IB3D_OUTLET_CONVECTIVE 1
/* ib3d_params.momentum */
#define IB3D_MOMENTUM_EULER 0
#define IB3D_MOMENTUM_AB2 1

typedef struct ib3d_params {
  double re;            /* Reynolds number (inputdata line 2; rev = 1/re, subReadInput.f90:22) */
  double deltat;        /* time step (subReadInput.f90:24) */
  double omega;         /* SOR relaxation factor (reference hard-codes 1.99, subPcorVcor.f90:158) */
  double eps;           /* SOR tolerance (inputdata eps1) */
  int64_t max_sweeps;   /* sweep cap; the reference has none (pcItaMax is read but unused) */
  int32_t criterion;    /* IB3D_CRIT_* */
  int32_t precision;    /* IB3D_PREC_* */
  int32_t warm_start;   /* IB3D_WARM_* */
  int32_t check_every;  /* sweeps between residual checks (IB3D_CRIT_RESIDUAL); >= 1 */
  int32_t inner_sweeps; /* FP32 sweeps per defect-correction pass (IB3D_PREC_FP32DC) */
  int32_t sweep_kernel; /* FP32 sweep kernel: 0 colour-packed arrays (even nx), one launch per colour
                           pass, two rows per thread (as 3 where the packed arrays exceed L2);
                           1 the padded field layout; 2 colour-packed arrays, the red and black
                           passes fused into one z-wavefront launch per sweep (even nx <= 512); 3
                           and 4 colour-packed arrays, one row per thread, the loads without (3)
                           or behind (4) branches. All give the same results. */
  double omega_inner;   /* relaxation factor of the FP32 inner sweeps (0: use omega). The FP64
                           defect correction fixes the final accuracy, so the inner solve may use
                           its own factor. */
  int32_t inner_schedule; /* IB3D_INNER_FIXED: every pass runs inner_sweeps; IB3D_INNER_ADAPTIVE:
                             the first pass runs inner_sweeps, later passes as many as the measured
                             residual reduction per sweep predicts are needed to reach eps (at most
                             four decades per FP32 solve), so fewer FP64 residual passes run and the
                             last pass overshoots less; IB3D_INNER_TAIL: every pass runs inner_sweeps
                             except the last, which runs as many as the previous pass's reduction
                             per sweep predicts are needed to reach eps (+8 % and 8 sweeps) */
  int32_t outlet;         /* IB3D_OUTLET_ZERO_GRADIENT (the reference's active outlet,
                             subBoundaryConditions.f90:149-151) or IB3D_OUTLET_CONVECTIVE (Orlanski,
                             the commented :153-155, with the speed uc of calculateUc,
                             subCalculateuc.f90:2-38, taken after each step's pressure forcing) */
  int32_t momentum;       /* IB3D_MOMENTUM_EULER (nsMomentum) or IB3D_MOMENTUM_AB2: ib3d_step uses
                             nsMomentumAB (subNavierStokes.f90:1128-1628) after the first step */
  int32_t smooth_sweeps;  /* FP32 form only: the first pass of each pressure solve begins with this
                             many red-black sweeps at relaxation 1 (Gauss-Seidel), counted among the
                             pass's sweeps. Over-relaxed sweeps (omega near 2) damp the
                             high-frequency part of the initial error by only |omega - 1| per sweep;
                             a few Gauss-Seidel sweeps remove what a coarse-grid guess (the learned
                             warm start) or the new right-hand side adds there. 0: none */
  int32_t ramp_sweeps;    /* FP32 form only: after the smoothing sweeps, the first pass raises the
                             relaxation linearly from 1 to omega_inner over this many sweeps. 0: none */
} ib3d_params;

/* Per-call statistics of the pressure solve (subPcorVcor.f90:60-65 logs the same). */
typedef struct ib3d_solve_stats {
  int64_t sweeps;        /* nIterPcor: SOR sweeps (FP64 sweeps, or FP32 inner sweeps) */
  int64_t outer;         /* defect-correction passes (0 for IB3D_PREC_FP64) */
  double divmax;         /* max |div u*| over fluid cells before the solve */
  double derr_std_st;    /* max |u_new - u_old| / dt over fluid cells */
  double final_err;      /* last value of the stopping test */
  double solve_seconds;  /* device time of the SOR loop (cpu_time pair at :33,:37) */
  double initial_err;    /* IB3D_PREC_FP32DC: FP64 residual L-inf of the initial guess */
} ib3d_solve_stats;

typedef struct ib3d_ctx ib3d_ctx;

/* Fills p with the reference's defaults (omega 1.99, eps 1e-5, update criterion). */
void ib3d_default_params(ib3d_params* p);

/* Grid and solver set-up: replaces readInput (subReadInput.f90:2-133), allocateArrays
 * (subAllocateArrays.f90:1-15), coefficientMatrix (subCoefficientMatrix.f90:1-59) and
 * non_uni_coeff (subNavierStokes.f90:3-619). x1n/y1n/z1n are the nx+1/ny+1/nz+1 node
 * coordinates of gridx/y/z.dat. Selects device 0 if no device is current. */
int ib3d_create(ib3d_ctx** out, const ib3d_params* prm, int64_t nx, int64_t ny, int64_t nz,
                const double* x1n, const double* y1n, const double* z1n);
void ib3d_destroy(ib3d_ctx* ctx);
const char* ib3d_last_error(const ib3d_ctx* ctx);
/* Replaces the solver options of a live context (for example to switch precision). */
int ib3d_set_params(ib3d_ctx* ctx, const ib3d_params* prm);

/* Surface mesh: the arrays readSurfaceMeshGmsh fills (subReadInput.f90:137-176), then
 * shiftSurfaceNodesInitial (subSearch.f90:2-39) and computeSurfaceNorm (subSearch.f90:80-131).
 * e1/e2/e3 are 1-based node indices; inor is the normal orientation (+1 outward). */
int ib3d_set_mesh(ib3d_ctx* ctx, int64_t nnodes, const double* xn, const double* yn, const double* zn,
                  int64_t nelems, const int64_t* e1, const int64_t* e2, const int64_t* e3,
                  double xshift, double yshift, double zshift, int64_t inor);

/* ---- Surface-mesh files --------------------------------------------------------
 * readSurfaceMeshGmsh (subReadInput.f90:137-176, Gmsh 2 ASCII, the first
 * sur_geo_points element lines skipped) and readSurfaceMeshGambit (:180-213, Gambit
 * .neu). ib3d_read_surface_mesh returns the counts when any array pointer is NULL,
 * and fills the arrays (sized by *nnodes, *nelems on entry) otherwise;
 * ib3d_set_mesh_file reads and calls ib3d_set_mesh. IB3D_ERR_IO on a short or
 * malformed file. */
#define IB3D_MESH_GMSH 0
#define IB3D_MESH_GAMBIT 1
int ib3d_read_surface_mesh(const char* path, int32_t format, int64_t sur_geo_points, int64_t* nnodes, double* xn,
                           double* yn, double* zn, int64_t* nelems, int64_t* e1, int64_t* e2, int64_t* e3);
int ib3d_set_mesh_file(ib3d_ctx* ctx, const char* path, int32_t format, int64_t sur_geo_points, double xshift,
                       double yshift, double zshift, int64_t inor);

/* Replaces the Poisson coefficient tables that ib3d_create builds as
 * coefficientMatrix does (subCoefficientMatrix.f90:1-59: the 1-D three-point
 * coefficients with the inlet/wall Neumann and outlet Dirichlet rows folded in).
 * acx is (nx,3) column-major like Acx (acy, acz likewise), for boundary conditions
 * the reference does not fold in, e.g. Neumann on all six faces. Both the FP64
 * tables and the FP32 copies of the mixed-precision solve are replaced. */
int ib3d_set_poisson_coefficients(ib3d_ctx* ctx, const double* acx, const double* acy, const double* acz);

/* Prescribed body motion (replaces shiftSurfaceNodesMovingbody, subSearch.f90:41-76,
 * whose shift is integrated from the force; here the caller gives it). Shifts every
 * surface node by (dx, dy, dz) (xnode1 = xr + xmove, :64-73), recomputes the
 * surface normals (computeSurfaceNorm, :80-131), and makes (us, vs, ws) the
 * surface velocity of the velocity forcing (the reference's commented hooks
 * usurf = u_curr etc., subForcing.f90:144, 228, 312, 397, 482, 566) and, with the
 * previous call's velocity, the acceleration in the pressure forcing's
 * dpdn = (-(v_curr - v_prev)/deltat)*cosBeta (hook at :20, summed over the three
 * axes). The search results describe the old position afterwards: call
 * ib3d_search before the next forcing. A context never moved keeps the reference's
 * fixed-body forcing (surface velocity 0, dpdn = 0). */
int ib3d_move_body(ib3d_ctx* ctx, double dx, double dy, double dz, double us, double vs, double ws);

/* Force-driven motion, shiftSurfaceNodesMovingbody (subSearch.f90:41-76):
 * u_final = F/(vol*1)*deltat + u_init per axis (vol = pi/6, a unit-diameter sphere of
 * density 1; u_init the previous call's u_final, 0 before the first), then
 * ib3d_move_body by u_final*deltat with surface velocity u_final. The reference
 * never computes Total_Force, so the caller passes the force (e.g. from the drag and
 * lift of ib3d_stress). vel (may be NULL) receives u_final. */
int ib3d_move_body_free(ib3d_ctx* ctx, double fx, double fy, double fz, double vel[3]);

/* tagging (subSearch.f90:134-321), cellCount (subSearch.f90:515-596) and
 * computeNormDistance (subSearch.f90:599-678), plus the ghost-point schedule.
 * box = {i_start, i_end, j_start, j_end, k_start, k_end} (inputdata lines 8-10).
 * counts (may be NULL) = {fluid, solid, ib, red, black}. */
int ib3d_search(ib3d_ctx* ctx, const int64_t box[6], int64_t counts[5]);

/* selectiveRetagging (subSearch.f90:327-512), for a body that moves a little each step:
 * the tagging test runs only on the 6x6x6 neighbourhood i-2..i+3, j-2..j+3, k-2..k+3
 * of every cell of the current IB list (clipped to the interior); every other cell
 * keeps its flag. Then cellCount, computeNormDistance and the ghost-point schedule as
 * ib3d_search runs them. Call it after ib3d_move_body in place of ib3d_search; it
 * needs the IB list of an earlier ib3d_search (or ib3d_selective_retag) of the same
 * mesh. Its flags equal a full search's whenever every cell whose flag changes lies
 * within those neighbourhoods (a body moving less than about two cells per call).
 * counts (may be NULL) as ib3d_search. */
int ib3d_selective_retag(ib3d_ctx* ctx, int64_t counts[5]);

/* Parity read-back of the search: cell flags (nx+2,ny+2,nz+2) int64 as in `cell`
 * (modGlobal.f90:25), interceptedIndexPtr (nib,3), nelp (nib) and the seven normal
 * distances (7 x nib: p, u1, u2, v1, v2, w1, w2). Any pointer may be NULL. */
int ib3d_get_search(ib3d_ctx* ctx, int64_t* cell, int64_t* ib_list, int64_t* nelp, double* normdis);

/* initialConditions (subInitialConditions.f90:2-48): all fields 0, u = 1 on fluid cells. */
int ib3d_initial_conditions(ib3d_ctx* ctx);

/* `!$acc update device` of the fields (subInitialConditions.f90:44, subLastConditions.f90:40).
 * Any pointer may be NULL to leave that field unchanged. ut/vt/wt are set equal to u/v/w. */
int ib3d_upload_fields(ib3d_ctx* ctx, const double* u, const double* v, const double* w, const double* p);
/* `!$acc update host (u, v, w, ut, vt, wt, p, cell)` (main.f90:55). Any pointer may be NULL. */
int ib3d_download_fields(ib3d_ctx* ctx, double* u, double* v, double* w, double* ut, double* vt,
                         double* wt, double* p);
/* The same download without waiting for it (the host side of main.f90:55 overlapped with the next
 * step): the fields as they stand after the work queued so far are copied to a device snapshot on
 * the context's stream (544 MB at 256x192x192, allocated on the first call), and the host copies
 * run from the snapshot on separate streams while the caller queues the next step. The host
 * buffers must stay valid, and unread, until ib3d_download_wait returns; pinned host memory lets
 * the copies run asynchronously. A second call first waits, on the device, for the previous
 * call's copies to leave the snapshot. */
int ib3d_download_fields_async(ib3d_ctx* ctx, double* u, double* v, double* w, double* ut, double* vt,
                               double* wt, double* p);
/* Blocks until the host copies of the last ib3d_download_fields_async have landed. */
int ib3d_download_wait(ib3d_ctx* ctx);
/* Read back one device field: 0 u,1 v,2 w,3 ut,4 vt,5 wt,6 p,7 pc,8 b. */
int ib3d_get_field(ib3d_ctx* ctx, int which, double* out);
/* Write one device field (same numbering); for tests that start a routine from a given state. */
int ib3d_set_field(ib3d_ctx* ctx, int which, const double* in);

/* Per-step routines, in main.f90's order (:46-52). */
int ib3d_ns_momentum(ib3d_ctx* ctx);      /* nsMomentum, subNavierStokes.f90:622-1122 */
/* nsMomentumAB (subNavierStokes.f90:1128-1628): nsMomentum's discretisation with the
 * second-order Adams-Bashforth update ut = u + dt*(0.5*(3*resid - resi_u) + dpdx)
 * (:1400, 1509, 1619), resi_u the previous call's resid (zero after
 * ib3d_initial_conditions or an upload, subInitialConditions.f90:24,
 * subLastConditions.f90:16). Both momentum calls store resid once the arrays exist
 * (IB3D_MOMENTUM_AB2 in the parameters, or the first call of this function). */
int ib3d_ns_momentum_ab(ib3d_ctx* ctx);
/* calculateUc (subCalculateuc.f90:2-38): the outlet convection speed
 * uc = max(mean ut(nx-4,:,:) over that plane's fluid cells, 0), summed in serial order,
 * used by the convective outlet; ib3d_step calls it after the pressure forcing when
 * ib3d_params.outlet is IB3D_OUTLET_CONVECTIVE. uc (may be NULL) receives the value. */
int ib3d_calculate_uc(ib3d_ctx* ctx, double* uc);
int ib3d_velocity_bc(ib3d_ctx* ctx);      /* velocityBC, subBoundaryConditions.f90:2-195 */
int ib3d_solid_cell_bc(ib3d_ctx* ctx);    /* solidCellBC, subBoundaryConditions.f90:199-217 */
int ib3d_velocity_forcing(ib3d_ctx* ctx); /* velocityForcing1, subForcing.f90:107-652 */
int ib3d_pressure_forcing(ib3d_ctx* ctx); /* pressureForcing1, subForcing.f90:2-103 */
/* poissonSolver, subPcorVcor.f90:2-80 (computeDiv, REDBLACKSOR, correctPressure,
 * correctVelocity, velocityBC, steady-state indicator, u = ut). stats may be NULL. */
int ib3d_poisson_solver(ib3d_ctx* ctx, ib3d_solve_stats* stats);
/* REDBLACKSOR alone (subPcorVcor.f90:148-212): solves A pc = b/deltat on the fluid
 * cells for the b already in the context (ib3d_set_field field 8), with the
 * context's precision, stopping test and warm start (IB3D_WARM_ZERO starts from
 * pc = 0 as poissonSolver does, :19-28); no divergence and no corrections. */
int ib3d_redblack_sor(ib3d_ctx* ctx, ib3d_solve_stats* stats);

/* stressCal1 (first != 0, subStressCal1.f90:2-460) or stressCal2 (subStressCal2.f90:2-381):
 * coef = {Cd viscous, Cd pressure, Cl viscous, Cl pressure} (dragcoff.dat / liftcoff.dat). */
int ib3d_stress(ib3d_ctx* ctx, int first, double coef[4]);
/* The whole step of main.f90:42-66 (first selects stressCal1). stats/coef may be NULL. */
int ib3d_step(ib3d_ctx* ctx, int first, ib3d_solve_stats* stats, double coef[4]);

/* Phase timers (the reference times only its SOR loop with cpu_time,
 * subPcorVcor.f90:33-37, and logs it to iter.dat :60-65). When enabled, every
 * phase records CUDA events on the context's stream; reading synchronizes.
 * ms[]: 0 momentum, 1 boundary conditions, 2 forcing, 3 divergence, 4 FP64 sweeps,
 * 5 FP32 sweeps, 6 residual + accumulation, 7 corrections + copy, 8 drag/lift,
 * 9 network warm start. */
typedef struct ib3d_timers {
  double ms[10];
  int64_t sweeps64;   /* FP64 red-black sweeps run */
  int64_t sweeps32;   /* FP32 red-black sweeps run */
  int64_t outer;      /* defect-correction passes */
  int64_t launches;   /* kernels launched by the library */
  int64_t steps;      /* ib3d_step calls */
  int64_t launches32; /* launches of the FP32 sweep kernel (one per colour pass, or one per
                         group of fused sweeps) */
} ib3d_timers;
/* on != 0 clears and starts the timers; on == 0 stops them (counts are kept). */
int ib3d_timers_enable(ib3d_ctx* ctx, int on);
int ib3d_timers_read(ib3d_ctx* ctx, ib3d_timers* out);
/* The context's CUDA stream (a cudaStream_t), for callers that order their own work
 * with the library's or record events on it. */
void* ib3d_stream(ib3d_ctx* ctx);

/* Device pointer of a field (same numbering as ib3d_get_field), for callers that keep
 * data on the GPU; valid until ib3d_destroy. */
void* ib3d_device_field(ib3d_ctx* ctx, int which);
/* Blocks until the context's stream is idle. */
int ib3d_synchronize(ib3d_ctx* ctx);

/* ---- Restart files -------------------------------------------------------------
 * writeResult (subWriteOutput.f90:62-72) saves u, v, w, p and totime, ita, ita1
 * every 1000 steps as formatted text; lastConditions (subLastConditions.f90:2-42)
 * reads them back and sets ut = u, vt = v, wt = w. ib3d_write_restart and
 * ib3d_read_restart do the same straight from and into device memory in a binary
 * file (64-byte header "IB3DRST1", nx, ny, nz, totime, ita, ita1, nfields = 4, then
 * u, v, w, p in the Fortran layout), so the Fortran driver no longer needs the per-step
 * download of main.f90:55 to keep a restart. The text pair reads and writes the
 * reference's own `result` file (one "u v w p totime ita ita1" record per cell, k
 * outer), for runs that move between the two codes. A file for another grid size
 * returns IB3D_ERR_ARG; an unreadable or short file IB3D_ERR_IO. */
int ib3d_write_restart(ib3d_ctx* ctx, const char* path, double totime, int64_t ita, int64_t ita1);
int ib3d_read_restart(ib3d_ctx* ctx, const char* path, double* totime, int64_t* ita, int64_t* ita1);
int ib3d_write_result_text(ib3d_ctx* ctx, const char* path, double totime, int64_t ita, int64_t ita1);
int ib3d_read_result_text(ib3d_ctx* ctx, const char* path, double* totime, int64_t* ita, int64_t* ita1);

/* ---- Learned warm start (no counterpart in the reference) -------------------------
 * A 3-level 3-D U-Net (16/32/64 channels, 3x3x3 convolutions, BF16 weights and
 * activations, FP32 accumulation), applied to the coarsened domain (see
 * ib3d_net_set_coarsening), predicts the change of the pressure correction
 * from one step to the next, pc^n - pc^{n-1}, from four inputs per cell: the
 * previous correction (p^{n-1} - p^{n-2}), b/dt, p^{n-1}, and the FP64 residual of
 * the previous correction against this step's b/dt divided by the diagonal of A.
 * pc^{n-1} plus the prediction is the SOR initial guess; the FP64 stopping test is
 * unchanged, so the previous correction (IB3D_WARM_PREV) is both the fallback and
 * the yardstick. The network is trained on the GPU by this library's own forward,
 * backward and Adam kernels on patches captured from solver runs. */
typedef struct ib3d_net ib3d_net;
int ib3d_net_create(ib3d_net** out, uint64_t seed);   /* He-initialised weights */
void ib3d_net_destroy(ib3d_net* net);
const char* ib3d_net_last_error(const ib3d_net* net);
int64_t ib3d_net_num_params(const ib3d_net* net);
int ib3d_net_get_params(ib3d_net* net, float* out);
int ib3d_net_set_params(ib3d_net* net, const float* in);
/* Loss (mean squared error) and gradient of one batch given on the host: x is
 * [B][S^3][4] FP32 (the four inputs above, x fastest within a patch), target
 * [B][S^3]; S a multiple of 4.
 * out (may be NULL) receives the prediction. No parameter update. */
int ib3d_net_loss_grad(ib3d_net* net, int B, int S, const float* x, const float* target, double* loss, float* grad,
                       float* out);
/* Training set: room for `capacity` patches of S^3 cells; ib3d_net_capture adds
 * random patches of a context's last step (after ib3d_step), ib3d_net_train runs
 * Adam steps on random batches of it. */
int ib3d_net_dataset_reserve(ib3d_net* net, int S, int64_t capacity);
int64_t ib3d_net_dataset_size(const ib3d_net* net);
int ib3d_net_capture(ib3d_net* net, ib3d_ctx* ctx, int npatches, uint64_t seed);
/* The network sees the domain coarsened by f = 1, 2 or 4 (default 2): each voxel holds
 * the average of the f^3 cells it covers, and the prediction is taken back to the
 * cells by trilinear interpolation between voxel centres -- a learned coarse-grid
 * correction of the smooth error that red-black SOR removes slowest, at 1/f^3 of the
 * inference cost (ib3d_params.smooth_sweeps removes the rough error the
 * interpolation leaves). Capture (S^3 voxels = (fS)^3 cells per patch) and
 * inference use the same f; changing it clears the training set. */
int ib3d_net_set_coarsening(ib3d_net* net, int f);
int ib3d_net_train(ib3d_net* net, int steps, int batch, double lr, uint64_t seed, double* last_loss);
/* Weight gradients of the convolutions: on the tensor cores (on != 0, the default:
 * an implicit GEMM over the voxels with tcgen05.mma) or on the CUDA cores in FP32
 * (on == 0, the reference the tensor-core form is checked against). */
int ib3d_net_set_wgrad_tensor_cores(ib3d_net* net, int on);
/* Keeps the two previous pressures and the previous correction's residual in ctx
 * (needed by capture and by the learned warm start); ib3d_attach_net calls it. */
int ib3d_enable_history(ib3d_ctx* ctx);
/* Network used by IB3D_WARM_LEARNED (NULL detaches). */
int ib3d_attach_net(ib3d_ctx* ctx, ib3d_net* net);

/* Mixed-precision pressure solve that allocates no memory. No counterpart in the
 * reference: it serves host codes that cannot call cudaMalloc -- a solver whose
 * device memory belongs to another runtime (an OpenACC data region, a framework's
 * caching allocator, a fixed pool sized at start-up) or one that must not allocate
 * inside its time loop. It needs no context: the caller passes every array as a
 * device pointer it owns, and the FP32 work arrays and control block live in one
 * static device array built into the library, which each GPU that loads the library
 * holds until the process exits.
 *
 * Solves A pc = b/deltat on the fluid cells (cell == 0) by FP64 defect correction
 * around inner_sweeps FP32 red-black sweeps per pass, from the pc given, until the
 * FP64 residual L-inf drops below eps (IB3D_ERR_NOCONV after max_sweeps). acx/acy/acz
 * are the (n,3) column-major Poisson coefficients of coefficientMatrix
 * (subCoefficientMatrix.f90:1-59); cell, b and pc are (nx+2,ny+2,nz+2) arrays in the
 * reference's layout (cell as uint8). stream is a cudaStream_t or NULL.
 *
 * Limit: (nx+2)*(ny+2)*(nz+2) <= 2^21 cells (two 8 MiB FP32 arrays); larger grids
 * (and any extent above 2^21) return IB3D_ERR_TOO_LARGE before any CUDA call. The
 * first call on a device looks up the scratch's device address (cudaGetSymbolAddress)
 * and caches it; make that first call before any stream capture. A call that meets a
 * CUDA error drops the cached address, so the next call looks it up again. The call
 * waits on the stream once per defect-correction pass to read the convergence
 * decision. Every call uses the same scratch and clears what must start at zero, so
 * calls that overlap on the GPU (other streams, other host threads) race: serialise
 * them. */
int ib3d_pressure_solve_noalloc(int64_t nx, int64_t ny, int64_t nz, const double* acx, const double* acy,
                                const double* acz, const unsigned char* cell, const double* b, double deltat,
                                double* pc, double omega, double eps, int64_t max_sweeps, int32_t inner_sweeps,
                                void* stream, int64_t* sweeps, double* residual);

#ifdef __cplusplus
}
#endif
#endif
