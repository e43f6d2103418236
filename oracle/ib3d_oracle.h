/*
 * IB3D CPU oracle: a serial FP64 restatement of the reference solver's per-step
 * hot path (Fortran 90 + OpenACC), used ONLY as test infrastructure: the
 * checker for the CUDA library, and the timed CPU baseline in bench.py.
 * It is never linked into, called by, or shipped with the product path.
 *
 * Parity status: UNPINNED by the reference itself. The reference ships no
 * tests, golden vectors or fixtures, its surface mesh is missing, and no
 * Fortran compiler exists in the build container or on the GPU host, so the
 * reference cannot be run. This file restates its arithmetic operation by
 * operation (left-to-right Fortran evaluation, every literal double as under
 * -Mr8, x**n with integral n as repeated multiplication, no FMA contraction:
 * build with -ffp-contract=off) and is pinned by analytic known-answer tests
 * instead (see tests/test_oracle.py).
 *
 * Array conventions follow the reference: 3-D fields are Fortran column-major
 * (nx+2, ny+2, nz+2) with i fastest and 1-based indices; index lists are
 * (n,3) int64 column-major.
 */
#ifndef IB3D_ORACLE_H
#define IB3D_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct OrState OrState;

/* Grid set-up: restates readInput (subReadInput.f90:2-133). x1n/y1n/z1n hold the
 * nx+1 / ny+1 / nz+1 node coordinates of the grid files (x1(2..nx+2)). */
OrState* or_create(int64_t nx, int64_t ny, int64_t nz, const double* x1n, const double* y1n,
                   const double* z1n, double re, double deltat);
void or_destroy(OrState* s);

/* Solver options that the reference hard-codes. omega: subPcorVcor.f90:158 (1.99);
 * eps: inputdata eps1; criterion 0 = update L-inf (subPcorVcor.f90:193-210),
 * 1 = residual L-inf of b/dt - A pc over fluid cells (added), tested every
 * check_every sweeps; max_sweeps caps the sweep loop (the reference has none). */
void or_set_solver(OrState* s, double omega, double eps, int criterion, int64_t max_sweeps,
                   int check_every);

/* Surface mesh: readSurfaceMeshGmsh's arrays (subReadInput.f90:137-176), then
 * shiftSurfaceNodesInitial (subSearch.f90:2-39) and computeSurfaceNorm (80-131). */
int or_set_mesh(OrState* s, int64_t nnodes, const double* xn, const double* yn, const double* zn,
                int64_t nelems, const int64_t* e1, const int64_t* e2, const int64_t* e3,
                double xshift, double yshift, double zshift, int64_t inor);

/* Prescribed motion: shift every surface node by (dx, dy, dz) as
 * shiftSurfaceNodesMovingbody does (subSearch.f90:64-73), recompute the surface
 * normals (80-131), and make (us, vs, ws) the surface velocity of the forcing
 * (usurf/vsurf/wsurf, subForcing.f90:144-145 etc.) and of dpdn (:20). Call
 * or_search afterwards. */
int or_move_body(OrState* s, double dx, double dy, double dz, double us, double vs, double ws);

/* Force-driven motion (shiftSurfaceNodesMovingbody, subSearch.f90:41-76) with the
 * surface force given: the body velocity integrates F/(pi/6) over deltat. */
int or_move_body_free(OrState* s, double fx, double fy, double fz, double vel[3]);

/* tagging (subSearch.f90:134-321) + cellCount (515-596) + computeNormDistance (599-678).
 * box = {i_start, i_end, j_start, j_end, k_start, k_end} (1-based, inclusive). */
int or_search(OrState* s, const int64_t box[6]);

/* selectiveRetagging (subSearch.f90:327-512): re-tags the 6x6x6 neighbourhood of every
 * IB cell of the current list (after a small move of the body), then cellCount and
 * computeNormDistance. Returns 0, or -1 with no IB cells to start from. */
int or_selective_retag(OrState* s);

/* No body at all: every interior cell fluid, lists built as cellCount does. */
void or_no_body(OrState* s);

/* Setup routines run once before the time loop (main.f90:15-18). */
void or_initial_conditions(OrState* s);   /* subInitialConditions.f90:2-48 */
void or_coefficient_matrix(OrState* s);   /* subCoefficientMatrix.f90:1-59 */
void or_non_uni_coeff(OrState* s);        /* subNavierStokes.f90:3-619 */
/* Replaces the Acx/Acy/Acz tables ((n,3) column-major) after or_coefficient_matrix. */
void or_set_coefficients(OrState* s, const double* acx, const double* acy, const double* acz);

/* Per-step routines (main.f90:29-39 and 42-66). */
void or_ns_momentum(OrState* s);                        /* subNavierStokes.f90:622-1122 */
void or_ns_momentum_ab(OrState* s);                     /* nsMomentumAB, subNavierStokes.f90:1128-1628 */
/* 0: or_step uses nsMomentum every step; 1: nsMomentumAB after the first step. */
void or_set_momentum(OrState* s, int momentum);
void or_velocity_bc(OrState* s);                        /* subBoundaryConditions.f90:2-195 (active branch) */
void or_solid_cell_bc(OrState* s);                      /* subBoundaryConditions.f90:199-217 */
int or_velocity_forcing(OrState* s);                    /* subForcing.f90:107-652 */
int or_pressure_forcing(OrState* s);                    /* subForcing.f90:2-103 */
int or_poisson_solver(OrState* s, int64_t* nsweeps, double* divmax, double* derrStdSt,
                      double* final_err);               /* subPcorVcor.f90:2-80 */
int or_stress(OrState* s, int first, double coef[4]);   /* subStressCal1/2.f90 */
/* REDBLACKSOR alone (subPcorVcor.f90:148-212) on the b set by the caller (field 8),
 * pc starting from 0. */
int or_redblack_sor(OrState* s, int64_t* nsweeps, double* final_err);
/* Outlet of velocityBC: 0 zero-gradient (subBoundaryConditions.f90:149-151, the
 * reference's active branch), 1 Orlanski convective (:153-155) with the speed uc that
 * or_calculate_uc (calculateUc, subCalculateuc.f90:2-38) sets after each step's
 * pressure forcing; uc starts at 1 (subReadInput.f90:28). */
void or_set_outlet(OrState* s, int outlet);
void or_calculate_uc(OrState* s);
double or_uc(const OrState* s);
/* One full time step as main.f90:42-66 sequences it; first selects stressCal1. */
int or_step(OrState* s, int first, int64_t* nsweeps, double coef[4]);

/* Accessors (pointers into oracle-owned storage). */
double* or_field(OrState* s, int which);  /* 0 u,1 v,2 w,3 ut,4 vt,5 wt,6 p,7 pc,8 b */
int64_t* or_cell(OrState* s);
void or_counts(OrState* s, int64_t out[5]); /* fluid, solid, ib, red, black */
int64_t* or_list(OrState* s, int which);    /* 0 fluid,1 solid,2 ib,3 red,4 black: (n,3) col-major */
double* or_surface(OrState* s, int which);  /* 0..2 cent, 3..5 cos, 6..8 alpha3.. */
double* or_normdis(OrState* s, int which);  /* 0 p,1 u1,2 u2,3 v1,4 v2,5 w1,6 w2 */
int64_t* or_nelp(OrState* s);
double* or_acoef(OrState* s, int axis);     /* (n,3) col-major Acx/Acy/Acz */
/* Convection coefficient tables: fam 0 uu,1 vv,2 ww,3 uv(=uw),4 vu(=vw),5 wu(=wv);
 * m 0..5 = ca1..ca6, 6..11 = ck1..ck6. Length n+2, 1-based storage at [1..n+2]. */
double* or_conv_coef(OrState* s, int fam, int m);
double* or_grid1d(OrState* s, int which);   /* 0 x1,1 y1,2 z1,3 dx,4 dy,5 dz, 6.. xu yu zu xv yv zv xw yw zw xp yp zp */
void or_set_threads(int n);
/* Row form of the sweep loop (on != 0): structured loops over the field's rows with a
 * fluid mask instead of the red/black index lists, bit-identical results; the timed
 * CPU baseline uses it. */
void or_set_sweep_rows(OrState* s, int on);
/* writeResult (subWriteOutput.f90:62-72) and lastConditions (subLastConditions.f90:2-42):
 * the reference's formatted restart file `result`. Return 0, or 1 on an I/O error or a
 * short or malformed file. */
int or_write_result_text(OrState* s, const char* path, double totime, int64_t ita, int64_t ita1);
int or_read_result_text(OrState* s, const char* path, double* totime, int64_t* ita, int64_t* ita1);

#ifdef __cplusplus
}
#endif
#endif
