/*
 * IB3D CPU oracle (test infrastructure only; see ib3d_oracle.h).
 *
 * Each routine restates one reference subroutine; the citation above it names
 * the reference file and lines it follows. Loop order, list order, clamps and
 * the operation order of every expression follow the Fortran. Build with
 * -ffp-contract=off so that no multiply-add is fused.
 */
#include "ib3d_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define SQ(x) ((x) * (x))

struct OrState {
  int64_t nx, ny, nz;
  double re, rev, deltat;
  double omega, eps;
  int criterion, check_every;
  int64_t max_sweeps;
  /* 1-D grid arrays, 1-based (element 0 unused) */
  double *x1, *y1, *z1, *deltax, *deltay, *deltaz;
  double *xu, *yu, *zu, *xv, *yv, *zv, *xw, *yw, *zw, *xp, *yp, *zp;
  double *Acx, *Acy, *Acz; /* (n,3) col-major */
  double *cc[6][12];       /* convection tables, 1-based */
  /* 3-D fields, Fortran column-major */
  double *u, *v, *w, *ut, *vt, *wt, *p, *pc, *pco, *b;
  int64_t *cell, *minElemcell;
  /* surface */
  int64_t nnodes, nelems, inor;
  double *xnode1, *ynode1, *znode1;
  int64_t *e1, *e2, *e3;
  double *xcent, *ycent, *zcent, *cosA, *cosB, *cosG, *alpha3, *beta3, *gamma3;
  /* outlet: 0 zero-gradient (the reference's active branch), 1 Orlanski convective
   * with the convection speed uc of calculateUc (initial value subReadInput.f90:28) */
  int outlet;
  double uc;
  /* nsMomentumAB: resi_u/v/w, the previous momentum call's residual
   * (allocateArrays, zeroed by initialConditions, subInitialConditions.f90:24) */
  int momentum;                 /* 0 nsMomentum every step, 1 nsMomentumAB after the first */
  double *resi_u, *resi_v, *resi_w;
  /* body motion: surface velocity now and one step earlier (0 for a fixed body) */
  int moving;
  double bvel[3], bprev[3];
  /* cell lists, (n,3) col-major, 1-based rows */
  int64_t nfluid, nsolid, nib, nred, nblack;
  int64_t *fluid, *solid, *ib, *red, *black;
  /* immersed-boundary geometry per IB cell */
  double *nd[7];  /* pNormDis, u1, u2, v1, v2, w1, w2 */
  int64_t *nelp;
  /* stress probe caches: Elemcell, ucell, vcell, wcell, pcell (ibElems,3) */
  int64_t *scache[5];
  int have_scache;
  /* throughput form of the sweep loop (or_set_sweep_rows): fluid mask in the field
   * layout (1 = fluid, from cellCount) and b/deltat of the running solve */
  int sweep_rows;
  unsigned char* fmask;
  double* bdt;
};

/* Fortran-style accessors. */
#define NX2 (s->nx + 2)
#define NY2 (s->ny + 2)
#define F3(a, i, j, k) (a)[((i)-1) + NX2 * (((j)-1) + NY2 * ((int64_t)(k)-1))]
#define L(a, n, r, c) (a)[((r)-1) + (n) * ((c)-1)]

static double* alloc1(int64_t n) { return (double*)calloc((size_t)(n + 4), sizeof(double)); }

void or_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

/* readInput, subReadInput.f90:2-133 (grid part). */
OrState* or_create(int64_t nx, int64_t ny, int64_t nz, const double* x1n, const double* y1n,
                   const double* z1n, double re, double deltat) {
  OrState* s = (OrState*)calloc(1, sizeof(OrState));
  s->nx = nx; s->ny = ny; s->nz = nz;
  s->re = re;
  s->rev = 1.0 / re;                       /* :22 */
  s->deltat = deltat;                      /* :24 deltat = dt_order*1e-3 (given directly) */
  s->omega = 1.99; s->eps = 1e-5; s->criterion = 0; s->max_sweeps = 1000000; s->check_every = 1;
  s->uc = 1.0;                             /* :28 */
  s->x1 = alloc1(nx + 3); s->y1 = alloc1(ny + 3); s->z1 = alloc1(nz + 3);
  s->deltax = alloc1(nx + 2); s->deltay = alloc1(ny + 2); s->deltaz = alloc1(nz + 2);
  s->xu = alloc1(nx + 3); s->yu = alloc1(ny + 2); s->zu = alloc1(nz + 2);
  s->xv = alloc1(nx + 2); s->yv = alloc1(ny + 3); s->zv = alloc1(nz + 2);
  s->xw = alloc1(nx + 2); s->yw = alloc1(ny + 2); s->zw = alloc1(nz + 3);
  s->xp = alloc1(nx + 2); s->yp = alloc1(ny + 2); s->zp = alloc1(nz + 2);
  for (int64_t i = 2; i <= nx + 2; ++i) s->x1[i] = x1n[i - 2];   /* :56-58 */
  for (int64_t i = 2; i <= nx + 1; ++i) s->deltax[i] = s->x1[i + 1] - s->x1[i]; /* :61-63 */
  s->deltax[1] = s->deltax[2];
  s->deltax[nx + 2] = s->deltax[nx + 1];
  s->x1[1] = s->x1[2] - s->deltax[1];
  s->x1[nx + 3] = s->x1[nx + 2] + s->deltax[nx + 2];            /* :65-68 */
  for (int64_t i = 2; i <= ny + 2; ++i) s->y1[i] = y1n[i - 2];
  for (int64_t i = 2; i <= ny + 1; ++i) s->deltay[i] = s->y1[i + 1] - s->y1[i];
  s->deltay[1] = s->deltay[2];
  s->deltay[ny + 2] = s->deltay[ny + 1];
  s->y1[1] = s->y1[2] - s->deltay[1];
  s->y1[ny + 3] = s->y1[ny + 2] + s->deltay[ny + 2];            /* :70-83 */
  for (int64_t i = 2; i <= nz + 2; ++i) s->z1[i] = z1n[i - 2];
  for (int64_t i = 2; i <= nz + 1; ++i) s->deltaz[i] = s->z1[i + 1] - s->z1[i];
  s->deltaz[1] = s->deltaz[2];
  s->deltaz[nz + 2] = s->deltaz[nz + 1];
  s->z1[1] = s->z1[2] - s->deltaz[1];
  s->z1[nz + 3] = s->z1[nz + 2] + s->deltaz[nz + 2];            /* :86-99 */
  for (int64_t i = 1; i <= nx + 3; ++i) s->xu[i] = s->x1[i];     /* :101-103 */
  for (int64_t i = 1; i <= ny + 3; ++i) s->yv[i] = s->y1[i];
  for (int64_t i = 1; i <= nz + 3; ++i) s->zw[i] = s->z1[i];
  for (int64_t i = 1; i <= ny + 2; ++i) {                        /* :113-117 */
    s->yu[i] = 0.5 * (s->y1[i] + s->y1[i + 1]);
    s->yw[i] = s->yu[i];
    s->yp[i] = s->yu[i];
  }
  for (int64_t i = 1; i <= nx + 2; ++i) {                        /* :119-123 */
    s->xv[i] = 0.5 * (s->x1[i] + s->x1[i + 1]);
    s->xw[i] = s->xv[i];
    s->xp[i] = s->xv[i];
  }
  for (int64_t i = 1; i <= nz + 2; ++i) {                        /* :125-129 */
    s->zu[i] = 0.5 * (s->z1[i] + s->z1[i + 1]);
    s->zv[i] = s->zu[i];
    s->zp[i] = s->zu[i];
  }
  const int64_t n3 = (nx + 2) * (ny + 2) * (nz + 2);
  double** f[] = {&s->u, &s->v, &s->w, &s->ut, &s->vt, &s->wt, &s->p, &s->pc, &s->pco, &s->b};
  for (size_t q = 0; q < sizeof(f) / sizeof(f[0]); ++q) *f[q] = (double*)calloc((size_t)n3, sizeof(double));
  s->cell = (int64_t*)calloc((size_t)n3, sizeof(int64_t));
  s->resi_u = (double*)calloc((size_t)n3, sizeof(double));
  s->resi_v = (double*)calloc((size_t)n3, sizeof(double));
  s->resi_w = (double*)calloc((size_t)n3, sizeof(double));
  s->minElemcell = (int64_t*)calloc((size_t)n3, sizeof(int64_t));
  s->Acx = (double*)calloc((size_t)(3 * nx), sizeof(double));
  s->Acy = (double*)calloc((size_t)(3 * ny), sizeof(double));
  s->Acz = (double*)calloc((size_t)(3 * nz), sizeof(double));
  for (int fam = 0; fam < 6; ++fam) {
    int64_t n = (fam % 3 == 0) ? nx : (fam % 3 == 1) ? ny : nz;
    for (int m = 0; m < 12; ++m) s->cc[fam][m] = alloc1(n + 2);
  }
  return s;
}

void or_set_solver(OrState* s, double omega, double eps, int criterion, int64_t max_sweeps,
                   int check_every) {
  s->omega = omega; s->eps = eps; s->criterion = criterion; s->max_sweeps = max_sweeps;
  s->check_every = check_every < 1 ? 1 : check_every;
}

void or_destroy(OrState* s) {
  if (!s) return;
  double* d[] = {s->x1, s->y1, s->z1, s->deltax, s->deltay, s->deltaz, s->xu, s->yu, s->zu,
                 s->xv, s->yv, s->zv, s->xw, s->yw, s->zw, s->xp, s->yp, s->zp, s->Acx, s->Acy,
                 s->Acz, s->u, s->v, s->w, s->ut, s->vt, s->wt, s->p, s->pc, s->pco, s->b,
                 s->xnode1, s->ynode1, s->znode1, s->xcent, s->ycent, s->zcent, s->cosA, s->cosB,
                 s->cosG, s->alpha3, s->beta3, s->gamma3};
  for (size_t q = 0; q < sizeof(d) / sizeof(d[0]); ++q) free(d[q]);
  for (int fam = 0; fam < 6; ++fam) for (int m = 0; m < 12; ++m) free(s->cc[fam][m]);
  for (int q = 0; q < 7; ++q) free(s->nd[q]);
  for (int q = 0; q < 5; ++q) free(s->scache[q]);
  free(s->cell); free(s->minElemcell); free(s->e1); free(s->e2); free(s->e3);
  free(s->fluid); free(s->solid); free(s->ib); free(s->red); free(s->black); free(s->nelp);
  free(s->resi_u); free(s->resi_v); free(s->resi_w);
  free(s->fmask); free(s->bdt);
  free(s);
}

/* computeSurfaceNorm (subSearch.f90:80-131): centroids, cross-product normals,
 * unit normals times inor. */
static void surface_norm(OrState* s) {
  const int64_t nelems = s->nelems;
  const double dinor = (double)s->inor;
  for (int64_t n = 1; n <= nelems; ++n) {      /* subSearch.f90:95-125 */
    double p1x = s->xnode1[s->e1[n]], p1y = s->ynode1[s->e1[n]], p1z = s->znode1[s->e1[n]];
    double p2x = s->xnode1[s->e2[n]], p2y = s->ynode1[s->e2[n]], p2z = s->znode1[s->e2[n]];
    double p3x = s->xnode1[s->e3[n]], p3y = s->ynode1[s->e3[n]], p3z = s->znode1[s->e3[n]];
    s->xcent[n] = ((p2x + p1x) + p3x) / 3.0;
    s->ycent[n] = ((p2y + p1y) + p3y) / 3.0;
    s->zcent[n] = ((p2z + p1z) + p3z) / 3.0;
    double ca = (p2y - p1y) * (p3z - p1z) - (p3y - p1y) * (p2z - p1z);
    double cb = (p2z - p1z) * (p3x - p1x) - (p3z - p1z) * (p2x - p1x);
    double cg = (p2x - p1x) * (p3y - p1y) - (p3x - p1x) * (p2y - p1y);
    s->alpha3[n] = ca; s->beta3[n] = cb; s->gamma3[n] = cg;
    double len = sqrt((SQ(ca) + SQ(cb)) + SQ(cg));
    s->cosA[n] = (ca / len) * dinor;
    s->cosB[n] = (cb / len) * dinor;
    s->cosG[n] = (cg / len) * dinor;
  }
}

/* shiftSurfaceNodesInitial (subSearch.f90:2-39) + computeSurfaceNorm (80-131). */
int or_set_mesh(OrState* s, int64_t nnodes, const double* xn, const double* yn, const double* zn,
                int64_t nelems, const int64_t* e1, const int64_t* e2, const int64_t* e3,
                double xshift, double yshift, double zshift, int64_t inor) {
  for (int64_t n = 0; n < nelems; ++n) {
    if (e1[n] < 1 || e1[n] > nnodes || e2[n] < 1 || e2[n] > nnodes || e3[n] < 1 || e3[n] > nnodes)
      return -3;
  }
  s->nnodes = nnodes; s->nelems = nelems; s->inor = inor;
  s->xnode1 = alloc1(nnodes); s->ynode1 = alloc1(nnodes); s->znode1 = alloc1(nnodes);
  for (int64_t i = 1; i <= nnodes; ++i) {      /* subSearch.f90:28-35 */
    s->xnode1[i] = xn[i - 1] + xshift;
    s->ynode1[i] = yn[i - 1] + yshift;
    s->znode1[i] = zn[i - 1] + zshift;
  }
  s->e1 = (int64_t*)calloc((size_t)nelems + 1, sizeof(int64_t));
  s->e2 = (int64_t*)calloc((size_t)nelems + 1, sizeof(int64_t));
  s->e3 = (int64_t*)calloc((size_t)nelems + 1, sizeof(int64_t));
  for (int64_t n = 1; n <= nelems; ++n) { s->e1[n] = e1[n - 1]; s->e2[n] = e2[n - 1]; s->e3[n] = e3[n - 1]; }
  double** a[] = {&s->xcent, &s->ycent, &s->zcent, &s->cosA, &s->cosB, &s->cosG, &s->alpha3, &s->beta3, &s->gamma3};
  for (int q = 0; q < 9; ++q) *a[q] = alloc1(nelems);
  surface_norm(s);
  return 0;
}

/* Prescribed body motion: the node shift of shiftSurfaceNodesMovingbody
 * (subSearch.f90:64-73, xnode1 = xr + xmove) with (xmove, ymove, zmove) given
 * instead of integrated from the force, then computeSurfaceNorm again. (us, vs, ws)
 * becomes the surface velocity of the velocity forcing (the commented hooks
 * usurf = u_curr etc., subForcing.f90:144, 228, 312, 397, 482, 566) and, with the
 * previous call's velocity, the body acceleration in dpdn (hook at :20). The
 * search must be run again before the next forcing. */
int or_move_body(OrState* s, double dx, double dy, double dz, double us, double vs, double ws) {
  if (!s->xnode1) return -2;
  for (int64_t i = 1; i <= s->nnodes; ++i) {
    const double xr = s->xnode1[i], yr = s->ynode1[i], zr = s->znode1[i];
    s->xnode1[i] = xr + dx;
    s->ynode1[i] = yr + dy;
    s->znode1[i] = zr + dz;
  }
  surface_norm(s);
  if (s->moving) {
    s->bprev[0] = s->bvel[0]; s->bprev[1] = s->bvel[1]; s->bprev[2] = s->bvel[2];
  } else {
    s->bprev[0] = us; s->bprev[1] = vs; s->bprev[2] = ws;   /* no acceleration on the first move */
  }
  s->bvel[0] = us; s->bvel[1] = vs; s->bvel[2] = ws;
  s->moving = 1;
  s->have_scache = 0;
  return 0;
}

/* Replaces the tables coefficientMatrix built (subCoefficientMatrix.f90:1-59), for
 * boundary conditions the reference does not fold in (all-Neumann, say); each
 * array is (n,3) column-major like Acx. */
void or_set_coefficients(OrState* s, const double* acx, const double* acy, const double* acz) {
  memcpy(s->Acx, acx, (size_t)(3 * s->nx) * sizeof(double));
  memcpy(s->Acy, acy, (size_t)(3 * s->ny) * sizeof(double));
  memcpy(s->Acz, acz, (size_t)(3 * s->nz) * sizeof(double));
}

/* shiftSurfaceNodesMovingbody (subSearch.f90:41-76) with the force given:
 * vol = (pi*(1.0)**3)/6. (:53, pi = 4*atan(1), subReadInput.f90:23),
 * u_final = (F/(vol*1.))*deltat + u_init, move = u_final*deltat. */
int or_move_body_free(OrState* s, double fx, double fy, double fz, double vel[3]) {
  const double pi = 4.0 * atan(1.0);
  const double vol = (pi * (1.0 * 1.0 * 1.0)) / 6.0;
  const double f[3] = {fx, fy, fz};
  double v[3];
  for (int q = 0; q < 3; ++q) {
    const double init = s->moving ? s->bvel[q] : 0.0;
    v[q] = (f[q] / (vol * 1.0)) * s->deltat + init;
  }
  const int rc = or_move_body(s, v[0] * s->deltat, v[1] * s->deltat, v[2] * s->deltat, v[0], v[1], v[2]);
  if (vel) { vel[0] = v[0]; vel[1] = v[1]; vel[2] = v[2]; }
  return rc;
}

/* Signed distance of a corner to the plane of element m (subSearch.f90:204-234). */
static inline double corner_dot(const OrState* s, int64_t m, double x, double y, double z) {
  return ((x - s->xcent[m]) * s->cosA[m] + (y - s->ycent[m]) * s->cosB[m]) + (z - s->zcent[m]) * s->cosG[m];
}

/* cellCount (subSearch.f90:515-596): lexicographic compaction of the flags into the
 * fluid, solid and IB lists, and the fluid list into red and black. */
static void cell_count(OrState* s) {
  const int64_t nx = s->nx, ny = s->ny, nz = s->nz;
  int64_t nf = 0, ns = 0, nb = 0;
  for (int64_t k = 2; k <= nz + 1; ++k)
    for (int64_t j = 2; j <= ny + 1; ++j)
      for (int64_t i = 2; i <= nx + 1; ++i) {
        int64_t c = F3(s->cell, i, j, k);
        if (c == 0) ++nf; else if (c == 1) ++ns; else if (c == 2) ++nb;
      }
  free(s->fluid); free(s->solid); free(s->ib); free(s->red); free(s->black);
  s->nfluid = nf; s->nsolid = ns; s->nib = nb;
  s->fluid = (int64_t*)malloc((size_t)(3 * nf + 3) * sizeof(int64_t));
  s->solid = (int64_t*)malloc((size_t)(3 * ns + 3) * sizeof(int64_t));
  s->ib = (int64_t*)malloc((size_t)(3 * nb + 3) * sizeof(int64_t));
  int64_t a = 0, bq = 0, c2 = 0;
  for (int64_t k = 2; k <= nz + 1; ++k)
    for (int64_t j = 2; j <= ny + 1; ++j)
      for (int64_t i = 2; i <= nx + 1; ++i) {
        int64_t c = F3(s->cell, i, j, k);
        if (c == 0) { ++a; L(s->fluid, nf, a, 1) = i; L(s->fluid, nf, a, 2) = j; L(s->fluid, nf, a, 3) = k; }
        else if (c == 1) { ++bq; L(s->solid, ns, bq, 1) = i; L(s->solid, ns, bq, 2) = j; L(s->solid, ns, bq, 3) = k; }
        else if (c == 2) { ++c2; L(s->ib, nb, c2, 1) = i; L(s->ib, nb, c2, 2) = j; L(s->ib, nb, c2, 3) = k; }
      }
  int64_t nr = 0, nk = 0;
  for (int64_t n = 1; n <= nf; ++n) {
    int64_t sum = L(s->fluid, nf, n, 1) + L(s->fluid, nf, n, 2) + L(s->fluid, nf, n, 3);
    if (sum % 2 == 1) ++nr; else ++nk;                      /* :562 */
  }
  s->nred = nr; s->nblack = nk;
  s->red = (int64_t*)malloc((size_t)(3 * nr + 3) * sizeof(int64_t));
  s->black = (int64_t*)malloc((size_t)(3 * nk + 3) * sizeof(int64_t));
  int64_t ir = 0, ik = 0;
  for (int64_t n = 1; n <= nf; ++n) {
    int64_t i = L(s->fluid, nf, n, 1), j = L(s->fluid, nf, n, 2), k = L(s->fluid, nf, n, 3);
    if ((i + j + k) % 2 == 1) { ++ir; L(s->red, nr, ir, 1) = i; L(s->red, nr, ir, 2) = j; L(s->red, nr, ir, 3) = k; }
    else { ++ik; L(s->black, nk, ik, 1) = i; L(s->black, nk, ik, 2) = j; L(s->black, nk, ik, 3) = k; }
  }
  /* the same fluid set as a mask in the field layout, for the row form of the sweeps */
  const int64_t n3 = NX2 * NY2 * (nz + 2);
  if (!s->fmask) s->fmask = (unsigned char*)malloc((size_t)n3);
  memset(s->fmask, 0, (size_t)n3);
  for (int64_t n = 1; n <= nf; ++n)
    F3(s->fmask, L(s->fluid, nf, n, 1), L(s->fluid, nf, n, 2), L(s->fluid, nf, n, 3)) = 1;
}

/* No body: every interior cell fluid (the flags tagging leaves outside its box). */
void or_no_body(OrState* s) {
  const int64_t n3 = NX2 * NY2 * (s->nz + 2);
  memset(s->cell, 0, (size_t)n3 * sizeof(int64_t));
  cell_count(s);
  for (int q = 0; q < 7; ++q) { free(s->nd[q]); s->nd[q] = alloc1(0); }
  free(s->nelp);
  s->nelp = (int64_t*)calloc(1, sizeof(int64_t));
}

/* The tagging test of one cell (subSearch.f90:166-247, and the same lines of
 * selectiveRetagging, :361-435): the nearest surface centroid of the cell centre
 * (dsqrt of the squared distances in y, x, z order; strict '<', so the first minimum
 * wins), then the signs of the eight corner distances to that element's plane
 * against -1e-16: all <= solid (1), all > fluid (0), else IB (2). */
static void tag_cell(OrState* s, int64_t i, int64_t j, int64_t k) {
  const double thr = -1e-16;
  double minDis = 1e14;
  int64_t nel = 0;
  const double n1x = s->xp[i], n1y = s->yp[j], n1z = s->zp[k];
  const double n2x = s->x1[i], n3x = s->x1[i + 1];
  const double n2y = s->y1[j], n3y = s->y1[j + 1];
  const double n2z = s->z1[k], n3z = s->z1[k + 1];
  for (int64_t m = 1; m <= s->nelems; ++m) {          /* :187-196 */
    double dis = sqrt((SQ(n1y - s->ycent[m]) + SQ(n1x - s->xcent[m])) + SQ(n1z - s->zcent[m]));
    if (dis < minDis) { minDis = dis; nel = m; }
  }
  F3(s->minElemcell, i, j, k) = nel;                   /* :198 */
  double d[8];
  d[0] = corner_dot(s, nel, n2x, n2y, n2z);            /* n2dotn :204 */
  d[1] = corner_dot(s, nel, n2x, n3y, n2z);            /* n3dotn :208 */
  d[2] = corner_dot(s, nel, n3x, n2y, n2z);            /* n4dotn :212 */
  d[3] = corner_dot(s, nel, n3x, n3y, n2z);            /* n5dotn :216 */
  d[4] = corner_dot(s, nel, n2x, n2y, n3z);            /* n6dotn :220 */
  d[5] = corner_dot(s, nel, n2x, n3y, n3z);            /* n7dotn :224 */
  d[6] = corner_dot(s, nel, n3x, n2y, n3z);            /* n8dotn :228 */
  d[7] = corner_dot(s, nel, n3x, n3y, n3z);            /* n9dotn :232 */
  int all_in = 1, all_out = 1;
  for (int q = 0; q < 8; ++q) {
    if (!(d[q] <= thr)) all_in = 0;
    if (!(d[q] > thr)) all_out = 0;
  }
  F3(s->cell, i, j, k) = all_in ? 1 : (all_out ? 0 : 2);   /* :238-247 */
}

static void norm_distance(OrState* s);

/* tagging (subSearch.f90:134-321), cellCount (515-596), computeNormDistance (599-678). */
int or_search(OrState* s, const int64_t box[6]) {
  const int64_t nx = s->nx, ny = s->ny, nz = s->nz;
  const int64_t n3 = NX2 * NY2 * (nz + 2);
  memset(s->cell, 0, (size_t)n3 * sizeof(int64_t));         /* :150; out-of-box cells read as 0 */
  memset(s->minElemcell, 0, (size_t)n3 * sizeof(int64_t));  /* :151 */
  if (box[0] < 1 || box[1] > nx + 2 || box[2] < 1 || box[3] > ny + 2 || box[4] < 1 || box[5] > nz + 2)
    return -2;
#pragma omp parallel for collapse(2) schedule(static)
  for (int64_t k = box[4]; k <= box[5]; ++k)
    for (int64_t j = box[2]; j <= box[3]; ++j)
      for (int64_t i = box[0]; i <= box[1]; ++i) tag_cell(s, i, j, k);
  cell_count(s);
  norm_distance(s);
  return 0;
}

/* selectiveRetagging (subSearch.f90:327-512): minElemcell = 0 (:339), then the
 * tagging test on the 6x6x6 neighbourhood i1-2..i1+3, j1-2..j1+3, k1-2..k1+3 of every
 * IB cell (i1, j1, k1) of the current list (:355-435); every other cell keeps its
 * flag. Neighbourhoods overlap, but the test depends on the cell alone, so the order
 * does not matter. The neighbourhood is clipped to the interior cells (a body kept
 * three cells from the walls never reaches the clip). Then cellCount (:515-596; the
 * reference recounts at :445-463) and computeNormDistance (:599-678), as after
 * tagging. Returns 0, or -1 when no IB cell exists to start from. */
int or_selective_retag(OrState* s) {
  const int64_t nx = s->nx, ny = s->ny, nz = s->nz;
  const int64_t n3 = NX2 * NY2 * (nz + 2);
  const int64_t nb = s->nib;
  if (nb < 1) return -1;
  memset(s->minElemcell, 0, (size_t)n3 * sizeof(int64_t));
  /* the neighbourhoods' cells, each once, so that the OpenMP loop writes each cell once */
  unsigned char* mark = (unsigned char*)calloc((size_t)n3, 1);
  for (int64_t nn = 1; nn <= nb; ++nn) {
    const int64_t i1 = L(s->ib, nb, nn, 1), j1 = L(s->ib, nb, nn, 2), k1 = L(s->ib, nb, nn, 3);
    for (int64_t k = k1 - 2; k <= k1 + 3; ++k)
      for (int64_t j = j1 - 2; j <= j1 + 3; ++j)
        for (int64_t i = i1 - 2; i <= i1 + 3; ++i)
          if (i >= 2 && i <= nx + 1 && j >= 2 && j <= ny + 1 && k >= 2 && k <= nz + 1) F3(mark, i, j, k) = 1;
  }
#pragma omp parallel for collapse(2) schedule(dynamic, 4)
  for (int64_t k = 2; k <= nz + 1; ++k)
    for (int64_t j = 2; j <= ny + 1; ++j)
      for (int64_t i = 2; i <= nx + 1; ++i)
        if (F3(mark, i, j, k)) tag_cell(s, i, j, k);
  free(mark);
  cell_count(s);
  norm_distance(s);
  return 0;
}

/* computeNormDistance (subSearch.f90:599-678) over the IB list cellCount built. */
static void norm_distance(OrState* s) {
  const int64_t nb = s->nib;
  /* computeNormDistance (subSearch.f90:621-672). */
  for (int q = 0; q < 7; ++q) { free(s->nd[q]); s->nd[q] = alloc1(nb); }
  free(s->nelp);
  s->nelp = (int64_t*)calloc((size_t)nb + 1, sizeof(int64_t));
  for (int64_t n = 1; n <= nb; ++n) {
    int64_t i = L(s->ib, nb, n, 1), j = L(s->ib, nb, n, 2), k = L(s->ib, nb, n, 3);
    double n1x = s->xp[i], n2x = s->x1[i], n3x = s->x1[i + 1];
    double n1y = s->yp[j], n2y = s->y1[j], n3y = s->y1[j + 1];
    double n1z = s->zp[k], n2z = s->z1[k], n3z = s->z1[k + 1];
    int64_t m = F3(s->minElemcell, i, j, k);
    s->nelp[n] = m;
    s->nd[0][n] = corner_dot(s, m, n1x, n1y, n1z);   /* pNormDis :645 */
    s->nd[1][n] = corner_dot(s, m, n2x, n1y, n1z);   /* u1NormDis :649 */
    s->nd[2][n] = corner_dot(s, m, n3x, n1y, n1z);   /* u2NormDis :653 */
    s->nd[3][n] = corner_dot(s, m, n1x, n2y, n1z);   /* v1NormDis :657 */
    s->nd[4][n] = corner_dot(s, m, n1x, n3y, n1z);   /* v2NormDis :661 */
    s->nd[5][n] = corner_dot(s, m, n1x, n1y, n2z);   /* w1NormDis :665 */
    s->nd[6][n] = corner_dot(s, m, n1x, n1y, n3z);   /* w2NormDis :669 */
  }
  s->have_scache = 0;
}

/* initialConditions (subInitialConditions.f90:2-48). */
void or_initial_conditions(OrState* s) {
  const int64_t n3 = NX2 * NY2 * (s->nz + 2);
  double* f[] = {s->u, s->ut, s->v, s->vt, s->w, s->wt, s->p, s->resi_u, s->resi_v, s->resi_w};
  for (int q = 0; q < 10; ++q) memset(f[q], 0, (size_t)n3 * sizeof(double));   /* :19-24 */
  for (int64_t n = 1; n <= s->nfluid; ++n) {
    int64_t i = L(s->fluid, s->nfluid, n, 1), j = L(s->fluid, s->nfluid, n, 2), k = L(s->fluid, s->nfluid, n, 3);
    F3(s->u, i, j, k) = 1.0;
  }
}

/* coefficientMatrix (subCoefficientMatrix.f90:1-59). */
void or_coefficient_matrix(OrState* s) {
  const int64_t nx = s->nx, ny = s->ny, nz = s->nz;
  for (int64_t j = 2; j <= ny + 1; ++j) {
    double r1 = s->yp[j] - s->yp[j - 1], r2 = s->yp[j + 1] - s->yp[j], rs = r1 + r2;
    L(s->Acy, ny, j - 1, 1) = 2.0 / (r1 * rs);
    L(s->Acy, ny, j - 1, 2) = -2.0 / (r1 * r2);
    L(s->Acy, ny, j - 1, 3) = 2.0 / (r2 * rs);
  }
  for (int64_t i = 2; i <= nx + 1; ++i) {
    double r1 = s->xp[i] - s->xp[i - 1], r2 = s->xp[i + 1] - s->xp[i], rs = r1 + r2;
    L(s->Acx, nx, i - 1, 1) = 2.0 / (r1 * rs);
    L(s->Acx, nx, i - 1, 2) = -2.0 / (r1 * r2);
    L(s->Acx, nx, i - 1, 3) = 2.0 / (r2 * rs);
  }
  for (int64_t i = 2; i <= nz + 1; ++i) {
    double r1 = s->zp[i] - s->zp[i - 1], r2 = s->zp[i + 1] - s->zp[i], rs = r1 + r2;
    L(s->Acz, nz, i - 1, 1) = 2.0 / (r1 * rs);
    L(s->Acz, nz, i - 1, 2) = -2.0 / (r1 * r2);
    L(s->Acz, nz, i - 1, 3) = 2.0 / (r2 * rs);
  }
  L(s->Acx, nx, 1, 2) = L(s->Acx, nx, 1, 2) + L(s->Acx, nx, 1, 1);     /* :36-53 */
  L(s->Acx, nx, 1, 1) = 0.0;
  L(s->Acx, nx, nx, 2) = L(s->Acx, nx, nx, 2) - L(s->Acx, nx, nx, 3);
  L(s->Acx, nx, nx, 3) = 0.0;
  L(s->Acy, ny, 1, 2) = L(s->Acy, ny, 1, 2) + L(s->Acy, ny, 1, 1);
  L(s->Acy, ny, 1, 1) = 0.0;
  L(s->Acy, ny, ny, 2) = L(s->Acy, ny, ny, 2) + L(s->Acy, ny, ny, 3);
  L(s->Acy, ny, ny, 3) = 0.0;
  L(s->Acz, nz, 1, 2) = L(s->Acz, nz, 1, 2) + L(s->Acz, nz, 1, 1);
  L(s->Acz, nz, 1, 1) = 0.0;
  L(s->Acz, nz, nz, 2) = L(s->Acz, nz, nz, 2) + L(s->Acz, nz, nz, 3);
  L(s->Acz, nz, nz, 3) = 0.0;
}

/* One station of non_uni_coeff: the 12 coefficients from three spacing ratios
 * (subNavierStokes.f90:41-116; the same block repeats for every family). */
static void conv_coeffs(double t1, double t2, double t3, double out[12]) {
  const double t3_2 = t3 * t3, t3_3 = t3 * t3 * t3, t3_4 = t3 * t3 * t3 * t3;
  const double t1_2 = t1 * t1, t1_3 = t1 * t1 * t1, t1_4 = t1 * t1 * t1 * t1;
  const double t2_2 = t2 * t2, t2_3 = t2 * t2 * t2, t2_4 = t2 * t2 * t2 * t2;
  double f1 = t3;
  double f2 = 2.0 * t3 + t3_2;
  double f3 = 3.0 * t3 + 3.0 * t3_2 + t3_3;
  double f4 = 4.0 * t3 + 6.0 * t3_2 + 4.0 * t3_3 + t3_4;
  double f5 = 1.0 / (t1 * t2);
  double f6 = (2.0 * t1 + 1.0) / (t1_2 * t2_2);
  double f7 = (3.0 * t1_2 + 3.0 * t1 + 1.0) / (t1_3 * t2_3);
  double f8 = (4.0 * t1_3 + 6.0 * t1_2 + 4.0 * t1 + 1.0) / (t1_4 * t2_4);
  double s51 = -1.0 / t2_4, s52 = f4, s53 = f4, s54 = s51;
  double s55 = -(f1 / t2_4 + f4 / t2);
  double s56 = (f4 / t2_2 - f2 / t2_4);
  double s57 = -(f3 / t2_4 + f4 / t2_3);
  double s61 = -1.0, s62 = f8, s63 = f8, s64 = -1.0;
  double s65 = (f5 + f8), s66 = (f8 - f6), s67 = (f7 + f8);
  double s71 = -1.0, s72 = (1.0 + f4), s73 = f4, s74 = (f4 - f1), s75 = (f4 - f2), s76 = (f4 - f3);
  double s81 = -1.0 / t2_4;
  double s82 = (f8 + (1.0 / t2_4));
  double s83 = f8;
  double s84 = (f5 / t2_4 - f8 / t2);
  double s85 = (f8 / t2_2 - f6 / t2_4);
  double s86 = (f7 / t2_4 - f8 / t2_3);
  double s91 = -s66 * s51;
  double s92 = s56 * s61;
  double s93 = -(s54 * s66 + s56 * s62);
  double s94 = (s56 * s64 + s66 * s52);
  double s95 = (s56 * s63 - s66 * s53);
  double s96 = (s56 * s65 - s66 * s55);
  double s97 = (s56 * s67 - s66 * s57);
  double s101 = -s85 * s71;
  double s102 = -s85 * s72;
  double s103 = s75 * s81;
  double s104 = s75 * s82;
  double s105 = (s75 * s83 - s85 * s73);
  double s106 = (s75 * s84 - s85 * s74);
  double s107 = (s75 * s86 - s85 * s76);
  out[0] = (s97 * s101 - s107 * s91);
  out[1] = (s97 * s102 + s107 * s93);
  out[2] = (s95 * s107 - s105 * s97);
  out[3] = (s94 * s107 + s104 * s97);
  out[4] = (s97 * s103 - s107 * s92);
  out[5] = (s97 * s106 - s107 * s96);
  double ak1 = (1.0 + 2.0 * t1) * (t3 + t3_2) * t2;
  double ak2 = (1.0 + t1) * (2.0 * t3 + t3_2);
  double ak3 = (1.0 + t1);
  double ak4 = (1.0 + t1) * ((1.0 + t3) * (1.0 + t3));
  double ak5 = ((1.0 + t1) * (1.0 + t1)) * (t3 + t3_2) * t2;
  double ak6 = t1_2 * t2 * (t3 + t3_2);
  double ak7 = (1.0 + t1) * (t3 + t3_2) * t2;
  out[6] = ak3;
  out[7] = -ak4;
  out[8] = (ak1 + ak2);
  out[9] = -ak5;
  out[10] = ak6;
  out[11] = ak7;
}

/* non_uni_coeff (subNavierStokes.f90:3-619). */
void or_non_uni_coeff(OrState* s) {
  const double* del[3] = {s->deltax, s->deltay, s->deltaz};
  const int64_t nn[3] = {s->nx, s->ny, s->nz};
  double c[12];
  for (int ax = 0; ax < 3; ++ax) {
    const double* d = del[ax];
    for (int64_t i = 2; i <= nn[ax]; ++i) {   /* uu/vv/ww: lines 36-283 */
      double t1 = d[i] / d[i - 1], t2 = d[i + 1] / d[i], t3 = d[i + 2] / d[i + 1];
      conv_coeffs(t1, t2, t3, c);
      for (int m = 0; m < 12; ++m) s->cc[ax][m][i] = c[m];
    }
    for (int64_t i = 2; i <= nn[ax]; ++i) {   /* uv/vu/wu: lines 285-595 */
      double h1 = (i == 2) ? d[i - 1] : 0.5 * (d[i - 1] + d[i - 2]);
      double h2 = 0.5 * (d[i] + d[i - 1]);
      double h3 = 0.5 * (d[i] + d[i + 1]);
      double h4 = 0.5 * (d[i + 1] + d[i + 2]);
      conv_coeffs(h2 / h1, h3 / h2, h4 / h3, c);
      for (int m = 0; m < 12; ++m) s->cc[3 + ax][m][i] = c[m];
    }
  }
}

/* nsMomentum (subNavierStokes.f90:622-1122) and nsMomentumAB (1128-1628): the same
 * discretisation, Euler or second-order Adams-Bashforth update (:1400, 1509, 1619);
 * both store resid in resi_* (:897, 1006, 1115 and 1403, 1512, 1622). */
static void ns_momentum(OrState* s, int ab2);
void or_ns_momentum(OrState* s) { ns_momentum(s, 0); }
void or_ns_momentum_ab(OrState* s) { ns_momentum(s, 1); }
void or_set_momentum(OrState* s, int momentum) { s->momentum = momentum; }

/* velocityBC active branch (subBoundaryConditions.f90:350-406). */
void or_velocity_bc(OrState* s) {
  const int64_t nx = s->nx, ny = s->ny, nz = s->nz;
  for (int64_t k = 2; k <= nz + 1; ++k)
    for (int64_t j = 2; j <= ny + 1; ++j) {
      F3(s->ut, 1, j, k) = 1.0;
      F3(s->vt, 1, j, k) = -F3(s->vt, 2, j, k);
      F3(s->wt, 1, j, k) = -F3(s->wt, 2, j, k);
      if (s->outlet == 1) {        /* Orlanski: the commented lines :153-155 (active at :131-133) */
        const double uc = s->uc, dt = s->deltat;
        F3(s->ut, nx + 1, j, k) = F3(s->u, nx + 1, j, k) - (dt / s->deltax[nx + 1]) * uc *
                                  (F3(s->u, nx + 1, j, k) - F3(s->u, nx, j, k));
        F3(s->vt, nx + 2, j, k) = -F3(s->vt, nx + 1, j, k) + F3(s->v, nx + 2, j, k) + F3(s->v, nx + 1, j, k) -
                                  (2.0 * dt / s->deltax[nx + 2]) * uc * (F3(s->v, nx + 2, j, k) - F3(s->v, nx + 1, j, k));
        F3(s->wt, nx + 2, j, k) = -F3(s->wt, nx + 1, j, k) + F3(s->w, nx + 2, j, k) + F3(s->w, nx + 1, j, k) -
                                  (2.0 * dt / s->deltax[nx + 2]) * uc * (F3(s->w, nx + 2, j, k) - F3(s->w, nx + 1, j, k));
      } else {                                                    /* zero gradient, :149-151 */
        F3(s->ut, nx + 1, j, k) = F3(s->ut, nx, j, k);
        F3(s->vt, nx + 2, j, k) = F3(s->vt, nx + 1, j, k);
        F3(s->wt, nx + 2, j, k) = F3(s->wt, nx + 1, j, k);
      }
    }
  for (int64_t k = 2; k <= nz + 1; ++k)
    for (int64_t i = 2; i <= nx + 1; ++i) {
      F3(s->ut, i, 1, k) = F3(s->ut, i, 2, k);
      F3(s->wt, i, 1, k) = F3(s->wt, i, 2, k);
      F3(s->vt, i, 1, k) = 0.0;
      F3(s->ut, i, ny + 2, k) = F3(s->ut, i, ny + 1, k);
      F3(s->wt, i, ny + 2, k) = F3(s->wt, i, ny + 1, k);
      F3(s->vt, i, ny + 1, k) = 0.0;
    }
  for (int64_t j = 2; j <= ny + 1; ++j)
    for (int64_t i = 2; i <= nx + 1; ++i) {
      F3(s->ut, i, j, 1) = F3(s->ut, i, j, 2);
      F3(s->vt, i, j, 1) = F3(s->vt, i, j, 2);
      F3(s->wt, i, j, 1) = 0.0;
      F3(s->ut, i, j, nz + 2) = F3(s->ut, i, j, nz + 1);
      F3(s->vt, i, j, nz + 2) = F3(s->vt, i, j, nz + 1);
      F3(s->wt, i, j, nz + 1) = 0.0;
    }
}

/* solidCellBC (subBoundaryConditions.f90:199-217). */
void or_solid_cell_bc(OrState* s) {
  for (int64_t n = 1; n <= s->nsolid; ++n) {
    int64_t i = L(s->solid, s->nsolid, n, 1), j = L(s->solid, s->nsolid, n, 2), k = L(s->solid, s->nsolid, n, 3);
    F3(s->ut, i, j, k) = 0.0; F3(s->vt, i, j, k) = 0.0; F3(s->wt, i, j, k) = 0.0; F3(s->p, i, j, k) = 0.0;
  }
}

/* Third-order upwind convection term (subNavierStokes.f90:812-817 and its
 * analogues): ((adv*Sa)/(ca6*dA)) + ((|adv|*Sk)/((2*ck6)*dK)). */
static inline double up3(double adv, double* const* c, int64_t m, double q2, double q1, double q0,
                         double qm1, double qm2, double dA, double dK) {
  double sa = (((c[0][m] * q2 + c[1][m] * q1) + c[2][m] * q0) + c[3][m] * qm1) + c[4][m] * qm2;
  double sk = (((c[6][m] * q2 + c[7][m] * q1) + c[8][m] * q0) + c[9][m] * qm1) + c[10][m] * qm2;
  return (adv * sa) / (c[5][m] * dA) + (fabs(adv) * sk) / (2.0 * c[11][m] * dK);
}

/* First-order upwind convection term (subNavierStokes.f90:847-852 and analogues),
 * al = 1 (:643). */
static inline double up1(double adv, double dA, double r, double qm, double q0, double qp) {
  const double al = 1.0;
  double t1 = (adv / dA) * (((-1.0 / (r * (r + 1.0))) * qm - (1.0 - 1.0 / r) * q0) + (r / (r + 1.0)) * qp);
  double t2 = al * fabs(adv) * (1.0 / (2.0 * dA)) * ((2.0 / (r * (r + 1.0)) * qm - 2.0 / r * q0) + 2.0 / (r + 1.0) * qp);
  return t1 - t2;
}

/* nsMomentum (subNavierStokes.f90:622-1122): explicit Euler predictor per fluid cell. */
static void ns_momentum(OrState* s, int ab2) {
  const int64_t nx = s->nx, ny = s->ny, nz = s->nz;
  const double rev = s->rev, deltat = s->deltat;
  const double *DX = s->deltax, *DY = s->deltay, *DZ = s->deltaz;
  const double *U = s->u, *V = s->v, *W = s->w, *P = s->p;
  const int64_t* C = s->cell;
  double* const* cuu = s->cc[0];
  double* const* cvv = s->cc[1];
  double* const* cww = s->cc[2];
  double* const* cuv = s->cc[3];
  double* const* cvu = s->cc[4];
  double* const* cwu = s->cc[5];
  const int64_t nf = s->nfluid;
#pragma omp parallel for schedule(static)
  for (int64_t n = 1; n <= nf; ++n) {
    const int64_t i = L(s->fluid, nf, n, 1), j = L(s->fluid, nf, n, 2), k = L(s->fluid, nf, n, 3);
    const double dxr = DX[i + 1], dx = DX[i], dxl = DX[i - 1];
    const double dye = DY[j + 1], dy = DY[j], dyw = DY[j - 1];
    const double dzt = DZ[k + 1], dz = DZ[k], dzb = DZ[k - 1];
    const double u0 = F3(U, i, j, k), v0 = F3(V, i, j, k), w0 = F3(W, i, j, k);
    const double u22 = F3(U, i - 1, j, k) - u0, u4 = u0 - F3(U, i + 1, j, k);
    const double u6 = F3(U, i, j - 1, k) - u0, u8 = u0 - F3(U, i, j + 1, k);
    const double u10 = F3(U, i, j, k - 1) - u0, u12 = u0 - F3(U, i, j, k + 1);
    const double v4 = F3(V, i - 1, j, k) - v0, v6 = v0 - F3(V, i + 1, j, k);
    const double v8 = F3(V, i, j - 1, k) - v0, v10 = v0 - F3(V, i, j + 1, k);
    const double v12 = F3(V, i, j, k - 1) - v0, v14 = v0 - F3(V, i, j, k + 1);
    const double w6 = F3(W, i - 1, j, k) - w0, w8 = w0 - F3(W, i + 1, j, k);
    const double w10 = F3(W, i, j - 1, k) - w0, w12 = w0 - F3(W, i, j + 1, k);
    const double w14 = F3(W, i, j, k - 1) - w0, w16 = w0 - F3(W, i, j, k + 1);
    const double p0 = F3(P, i, j, k);
    const double dpdx = (p0 - F3(P, i + 1, j, k)) / (0.5 * (dxr + dx));   /* :779-781 */
    const double dpdy = (p0 - F3(P, i, j + 1, k)) / (0.5 * (dye + dy));
    const double dpdz = (p0 - F3(P, i, j, k + 1)) / (0.5 * (dzt + dz));
    const double dx2xr = dx + dxr, dx2xl = dx + dxl, dy2ye = dy + dye, dy2yw = dy + dyw;
    const double dz2zt = dz + dzt, dz2zb = dz + dzb;
    const int noib = F3(C, i + 1, j, k) != 2 && F3(C, i - 1, j, k) != 2 && F3(C, i, j + 1, k) != 2 &&
                     F3(C, i, j - 1, k) != 2 && F3(C, i, j, k + 1) != 2 && F3(C, i, j, k - 1) != 2;
    const double ddx = 0.5 * (DX[i] + DX[i - 1]), ddxr = 0.5 * (DX[i] + DX[i + 1]);
    const double ddy = 0.5 * (DY[j] + DY[j - 1]), ddye = 0.5 * (DY[j] + DY[j + 1]);
    const double ddz = 0.5 * (DZ[k] + DZ[k - 1]), ddzr = 0.5 * (DZ[k] + DZ[k + 1]);
    double cx, cy, cz;

    /* ---- u momentum (:792-897) ---- */
    {
      double vu_e = F3(V, i + 1, j, k) + (dxr / dx2xr) * (F3(V, i, j, k) - F3(V, i + 1, j, k));
      double vu_w = F3(V, i + 1, j - 1, k) + (dxr / dx2xr) * (F3(V, i, j - 1, k) - F3(V, i + 1, j - 1, k));
      double vin = 0.5 * (vu_e + vu_w);
      double wu_n = F3(W, i + 1, j, k) + (dxr / dx2xr) * (F3(W, i, j, k) - F3(W, i + 1, j, k));
      double wu_s = F3(W, i + 1, j, k - 1) + (dxr / dx2xr) * (F3(W, i, j, k - 1) - F3(W, i + 1, j, k - 1));
      double win = 0.5 * (wu_n + wu_s);
      if (i != 2 && i < nx && j != 2 && j < ny + 1 && k != 2 && k < nz + 1 && noib) {
        cx = up3(u0, cuu, i, F3(U, i + 2, j, k), F3(U, i + 1, j, k), u0, F3(U, i - 1, j, k), F3(U, i - 2, j, k), DX[i + 1], DX[i]);
        cy = up3(vin, cvu, j, F3(U, i, j + 2, k), F3(U, i, j + 1, k), u0, F3(U, i, j - 1, k), F3(U, i, j - 2, k), ddye, ddy);
        cz = up3(win, cwu, k, F3(U, i, j, k + 2), F3(U, i, j, k + 1), u0, F3(U, i, j, k - 1), F3(U, i, j, k - 2), ddzr, ddz);
      } else {
        double r1x = DX[i] / DX[i + 1];
        double r1yn = 0.5 * (DY[j] + DY[j - 1]), r1yd = 0.5 * (DY[j] + DY[j + 1]), r1y = r1yn / r1yd;
        double r1zn = 0.5 * (DZ[k] + DZ[k - 1]), r1zd = 0.5 * (DZ[k] + DZ[k + 1]), r1z = r1zn / r1zd;
        cx = up1(u0, DX[i + 1], r1x, F3(U, i - 1, j, k), u0, F3(U, i + 1, j, k));
        cy = up1(vin, r1yd, r1y, F3(U, i, j - 1, k), u0, F3(U, i, j + 1, k));
        cz = up1(win, r1zd, r1z, F3(U, i, j, k - 1), u0, F3(U, i, j, k + 1));
      }
      double d2x = (2.0 / dx2xr) * ((-u4 / dxr) + (u22 / dx));
      double d2y = (2.0 / (0.5 * (dy2ye + dy2yw))) * ((-u8 / (0.5 * dy2ye)) + (u6 / (0.5 * dy2yw)));
      double d2z = (2.0 / (0.5 * (dz2zt + dz2zb))) * ((-u12 / (0.5 * dz2zt)) + (u10 / (0.5 * dz2zb)));
      double xtt2 = rev * (d2x + d2y + d2z);
      double resid = -cx - cy - cz + xtt2;
      if (ab2) F3(s->ut, i, j, k) = u0 + deltat * (0.5 * (3.0 * resid - F3(s->resi_u, i, j, k)) + dpdx);
      else F3(s->ut, i, j, k) = u0 + deltat * (resid + dpdx);
      F3(s->resi_u, i, j, k) = resid;                               /* :897 (1403) */
    }
    /* ---- v momentum (:901-1006) ---- */
    {
      double uv_e = F3(U, i, j + 1, k) + (dye / dy2ye) * (F3(U, i, j, k) - F3(U, i, j + 1, k));
      double uv_w = F3(U, i - 1, j + 1, k) + (dye / dy2ye) * (F3(U, i - 1, j, k) - F3(U, i - 1, j + 1, k));
      double uin = 0.5 * (uv_e + uv_w);
      double wv_n = F3(W, i, j + 1, k) + (dye / dy2ye) * (F3(W, i, j, k) - F3(W, i, j + 1, k));
      double wv_s = F3(W, i, j + 1, k - 1) + (dye / dy2ye) * (F3(W, i, j, k - 1) - F3(W, i, j + 1, k - 1));
      double win = 0.5 * (wv_n + wv_s);
      if (i != 2 && i < nx + 1 && j != 2 && j < ny && k != 2 && k < nz + 1 && noib) {
        cx = up3(uin, cuv, i, F3(V, i + 2, j, k), F3(V, i + 1, j, k), v0, F3(V, i - 1, j, k), F3(V, i - 2, j, k), ddxr, ddx);
        cy = up3(v0, cvv, j, F3(V, i, j + 2, k), F3(V, i, j + 1, k), v0, F3(V, i, j - 1, k), F3(V, i, j - 2, k), DY[j + 1], DY[j]);
        cz = up3(win, cwu, k, F3(V, i, j, k + 2), F3(V, i, j, k + 1), v0, F3(V, i, j, k - 1), F3(V, i, j, k - 2), ddzr, ddz);
      } else {
        double r1xn = 0.5 * (DX[i] + DX[i - 1]), r1xd = 0.5 * (DX[i] + DX[i + 1]), r1x = r1xn / r1xd;
        double r1y = DY[j] / DY[j + 1];
        double r1zn = 0.5 * (DZ[k] + DZ[k - 1]), r1zd = 0.5 * (DZ[k] + DZ[k + 1]), r1z = r1zn / r1zd;
        cx = up1(uin, r1xd, r1x, F3(V, i - 1, j, k), v0, F3(V, i + 1, j, k));
        cy = up1(v0, DY[j + 1], r1y, F3(V, i, j - 1, k), v0, F3(V, i, j + 1, k));
        cz = up1(win, r1zd, r1z, F3(V, i, j, k - 1), v0, F3(V, i, j, k + 1));
      }
      double d2x = (2.0 / (0.5 * (dx2xr + dx2xl))) * ((-v6 / (0.5 * dx2xr)) + (v4 / (0.5 * dx2xl)));
      double d2y = (2.0 / dy2ye) * ((-v10 / dye) + (v8 / dy));
      double d2z = (2.0 / (0.5 * (dz2zt + dz2zb))) * ((-v14 / (0.5 * dz2zt)) + (v12 / (0.5 * dz2zb)));
      double ytt2 = rev * (d2x + d2y + d2z);
      double resid = -cx - cy - cz + ytt2;
      if (ab2) F3(s->vt, i, j, k) = v0 + deltat * (0.5 * (3.0 * resid - F3(s->resi_v, i, j, k)) + dpdy);
      else F3(s->vt, i, j, k) = v0 + deltat * (resid + dpdy);
      F3(s->resi_v, i, j, k) = resid;                               /* :897 (1403) */
    }
    /* ---- w momentum (:1010-1116) ---- */
    {
      double uw_e = F3(U, i, j, k + 1) + (dzt / dz2zt) * (F3(U, i, j, k) - F3(U, i, j, k + 1));
      double uw_w = F3(U, i - 1, j, k + 1) + (dzt / dz2zt) * (F3(U, i - 1, j, k) - F3(U, i - 1, j, k + 1));
      double uin = 0.5 * (uw_e + uw_w);
      double vw_n = F3(V, i, j, k + 1) + (dzt / dz2zt) * (F3(V, i, j, k) - F3(V, i, j, k + 1));
      double vw_s = F3(V, i, j - 1, k + 1) + (dzt / dz2zt) * (F3(V, i, j - 1, k) - F3(V, i, j - 1, k + 1));
      double vin = 0.5 * (vw_n + vw_s);
      if (i != 2 && i < nx + 1 && j != 2 && j < ny + 1 && k != 2 && k < nz && noib) {
        cx = up3(uin, cuv, i, F3(W, i + 2, j, k), F3(W, i + 1, j, k), w0, F3(W, i - 1, j, k), F3(W, i - 2, j, k), ddxr, ddx);
        cy = up3(vin, cvu, j, F3(W, i, j + 2, k), F3(W, i, j + 1, k), w0, F3(W, i, j - 1, k), F3(W, i, j - 2, k), ddye, ddy);
        cz = up3(w0, cww, k, F3(W, i, j, k + 2), F3(W, i, j, k + 1), w0, F3(W, i, j, k - 1), F3(W, i, j, k - 2), DZ[k + 1], DZ[k]);
      } else {
        double r1xn = 0.5 * (DX[i] + DX[i - 1]), r1xd = 0.5 * (DX[i] + DX[i + 1]), r1x = r1xn / r1xd;
        double r1yn = 0.5 * (DY[j] + DY[j - 1]), r1yd = 0.5 * (DY[j] + DY[j + 1]), r1y = r1yn / r1yd;
        double r1z = DZ[k] / DZ[k + 1];
        cx = up1(uin, r1xd, r1x, F3(W, i - 1, j, k), w0, F3(W, i + 1, j, k));
        cy = up1(vin, r1yd, r1y, F3(W, i, j - 1, k), w0, F3(W, i, j + 1, k));
        cz = up1(w0, DZ[k + 1], r1z, F3(W, i, j, k - 1), w0, F3(W, i, j, k + 1));
      }
      double d2x = (2.0 / (0.5 * (dx2xr + dx2xl))) * ((-w8 / (0.5 * dx2xr)) + (w6 / (0.5 * dx2xl)));
      double d2y = (2.0 / (0.5 * (dy2ye + dy2yw))) * ((-w12 / (0.5 * dy2ye)) + (w10 / (0.5 * dy2yw)));
      double d2z = (2.0 / dz2zt) * ((-w16 / dzt) + (w14 / dz));
      double ztt2 = rev * (d2x + d2y + d2z);
      double resid = -cx - cy - cz + ztt2;
      if (ab2) F3(s->wt, i, j, k) = w0 + deltat * (0.5 * (3.0 * resid - F3(s->resi_w, i, j, k)) + dpdz);
      else F3(s->wt, i, j, k) = w0 + deltat * (resid + dpdz);
      F3(s->resi_w, i, j, k) = resid;                               /* :897 (1403) */
    }
  }
}

/* Linear bracket scan that keeps the last match, as every forcing and stress
 * routine does (e.g. subForcing.f90:36-38). Returns 0 when no bracket exists. */
static int64_t bracket(const double* A, int64_t lo, int64_t hi, double pos) {
  int64_t r = 0;
  for (int64_t l = lo; l <= hi; ++l)
    if (pos >= A[l] && pos < A[l + 1]) r = l;
  return r;
}

/* Trilinear probe value and one-sided quadratic derivative estimates of a
 * staggered field (the common block of subForcing.f90:175-215 and its
 * analogues). (ox,oy,oz) is the field-index offset of the coordinate index:
 * -1 along a velocity component's own direction, 0 otherwise. */
static void probe_eval(const OrState* s, const double* F, const double* X, const double* Y,
                       const double* Z, int ox, int oy, int oz, int64_t ix, int64_t iy, int64_t iz,
                       double px, double py, double pz, double out[4]) {
  const int64_t a0 = ix + ox, a1 = ix + 1 + ox, b0 = iy + oy, b1 = iy + 1 + oy, c0 = iz + oz, c1 = iz + 1 + oz;
  const double f000 = F3(F, a0, b0, c0), f100 = F3(F, a1, b0, c0), f010 = F3(F, a0, b1, c0), f110 = F3(F, a1, b1, c0);
  const double f001 = F3(F, a0, b0, c1), f101 = F3(F, a1, b0, c1), f011 = F3(F, a0, b1, c1), f111 = F3(F, a1, b1, c1);
  const double tx = px - X[ix], dX = X[ix + 1] - X[ix];
  const double ty = py - Y[iy], dY = Y[iy + 1] - Y[iy];
  const double tz = pz - Z[iz], dZ = Z[iz + 1] - Z[iz];
  double x1z1 = f000 + (f100 - f000) * tx / dX;
  double x2z1 = f010 + (f110 - f010) * tx / dX;
  double x1z2 = f001 + (f101 - f001) * tx / dX;
  double x2z2 = f011 + (f111 - f011) * tx / dX;
  double z1 = x1z1 + (x2z1 - x1z1) * ty / dY;
  double z2 = x1z2 + (x2z2 - x1z2) * ty / dY;
  double y1 = x1z1 + (x1z2 - x1z1) * tz / dZ;
  double y2 = x2z1 + (x2z2 - x2z1) * tz / dZ;
  double z1x1 = f000 + (f001 - f000) * tz / dZ;
  double z2x1 = f010 + (f011 - f010) * tz / dZ;
  double z1x2 = f100 + (f101 - f100) * tz / dZ;
  double z2x2 = f110 + (f111 - f110) * tz / dZ;
  double x1 = z1x1 + (z2x1 - z1x1) * ty / dY;
  double x2 = z1x2 + (z2x2 - z1x2) * ty / dY;
  double pos = x1 + (x2 - x1) * tx / dX;
  double h2 = fabs(X[ix + 1] - px), h1 = fabs(X[ix] - px);
  out[1] = (SQ(h1) * x2 - SQ(h2) * x1 + (SQ(h2) - SQ(h1)) * pos) / (h1 * h2 * (h1 + h2) + 1e-16);
  h2 = fabs(Y[iy + 1] - py); h1 = fabs(Y[iy] - py);
  out[2] = (SQ(h1) * y2 - SQ(h2) * y1 + (SQ(h2) - SQ(h1)) * pos) / (h1 * h2 * (h1 + h2) + 1e-16);
  h2 = fabs(Z[iz + 1] - pz); h1 = fabs(Z[iz] - pz);
  out[3] = (SQ(h1) * z2 - SQ(h2) * z1 + (SQ(h2) - SQ(h1)) * pos) / (h1 * h2 * (h1 + h2) + 1e-16);
  out[0] = pos;
}

/* Ghost-point blocks of velocityForcing1 in their serial order
 * (subForcing.f90:143-224, 227-308, 311-393, 396-478, 481-562, 565-646). */
typedef struct {
  int field;          /* 0 ut, 1 vt, 2 wt */
  int nd;             /* index into nd[] */
  int node_off[3];    /* node coordinate index offset: X[i+node_off[0]] */
  int scan_extra[3];  /* scan upper bound = n+1+scan_extra */
  int clamp_axis;     /* axis of the clamp */
  int clamp_hi;       /* 1: if idx==n+2 -> n+1 ; 0: if idx==1 -> 2 */
  int tgt[3];         /* write target offset */
} GhostBlock;

static const GhostBlock kGhost[6] = {
    {0, 2, {1, 0, 0}, {1, 0, 0}, 0, 1, {0, 0, 0}},    /* U(i,j,k)   :143-224 */
    {0, 1, {0, 0, 0}, {0, 0, 0}, 0, 0, {-1, 0, 0}},   /* U(i-1,j,k) :227-308 */
    {1, 4, {0, 1, 0}, {0, 1, 0}, 1, 1, {0, 0, 0}},    /* V(i,j,k)   :311-393 */
    {1, 3, {0, 0, 0}, {0, 0, 0}, 1, 0, {0, -1, 0}},   /* V(i,j-1,k) :396-478 */
    {2, 6, {0, 0, 1}, {0, 0, 1}, 2, 1, {0, 0, 0}},    /* W(i,j,k)   :481-562 */
    {2, 5, {0, 0, 0}, {0, 0, 0}, 2, 0, {0, 0, -1}},   /* W(i,j,k-1) :565-646 */
};

/* velocityForcing1 (subForcing.f90:107-652). Serial over IB cells and blocks:
 * later writes win and later probes read earlier writes, as on a CPU. */
int or_velocity_forcing(OrState* s) {
  const int64_t nx = s->nx, ny = s->ny, nz = s->nz, nb = s->nib;
  const int64_t nn[3] = {nx, ny, nz};
  for (int64_t n = 1; n <= nb; ++n) {
    const int64_t ijk[3] = {L(s->ib, nb, n, 1), L(s->ib, nb, n, 2), L(s->ib, nb, n, 3)};
    const int64_t i = ijk[0], j = ijk[1], k = ijk[2];
    const int64_t nel = s->nelp[n];
    const double diag = sqrt((SQ(s->deltax[i]) + SQ(s->deltay[j])) + SQ(s->deltaz[k]));
    for (int b = 0; b < 6; ++b) {
      const GhostBlock* g = &kGhost[b];
      double* F = g->field == 0 ? s->ut : g->field == 1 ? s->vt : s->wt;
      const double* X = g->field == 0 ? s->xu : g->field == 1 ? s->xv : s->xw;
      const double* Y = g->field == 0 ? s->yu : g->field == 1 ? s->yv : s->yw;
      const double* Z = g->field == 0 ? s->zu : g->field == 1 ? s->zv : s->zw;
      const double* A3[3] = {X, Y, Z};
      const double surf = s->moving ? s->bvel[g->field] : 0.0;   /* usurf = u_curr (:144) */
      const double sd = s->nd[g->nd][n];
      const double pt1 = 1.5 * diag + (fabs(sd) - sd) * 0.5;
      const double pos[3] = {X[i + g->node_off[0]] + pt1 * s->cosA[nel],
                             Y[j + g->node_off[1]] + pt1 * s->cosB[nel],
                             Z[k + g->node_off[2]] + pt1 * s->cosG[nel]};
      int64_t br[3];
      for (int a = 0; a < 3; ++a) {
        br[a] = bracket(A3[a], 1, nn[a] + 1 + g->scan_extra[a], pos[a]);
        if (br[a] == 0) return -4;
      }
      const int ca = g->clamp_axis;
      if (g->clamp_hi) { if (br[ca] == nn[ca] + 2) br[ca] = nn[ca] + 1; }
      else { if (br[ca] == 1) br[ca] = 2; }
      double pe[4];
      probe_eval(s, F, X, Y, Z, g->field == 0 ? -1 : 0, g->field == 1 ? -1 : 0, g->field == 2 ? -1 : 0,
                 br[0], br[1], br[2], pos[0], pos[1], pos[2], pe);
      const double dndn = pe[1] * s->cosA[nel] + pe[2] * s->cosB[nel] + pe[3] * s->cosG[nel];
      const double n1 = pt1 + sd;
      const double cval = surf;
      const double bval = 2.0 / n1 * (pe[0] - surf) - dndn;
      const double aval = dndn / n1 - (pe[0] - surf) / SQ(n1);
      F3(F, i + g->tgt[0], j + g->tgt[1], k + g->tgt[2]) = aval * SQ(sd) + bval * sd + cval;
    }
  }
  return 0;
}

/* pressureForcing1 (subForcing.f90:2-103). dpdn = 0 for a fixed body (:11); for a
 * moving one the hook at :20, dpdn = (-(v_curr-v_prev)/deltat)*cosBeta(nelp(n)),
 * summed over the three axes in x, y, z order. */
int or_pressure_forcing(OrState* s) {
  const int64_t nx = s->nx, ny = s->ny, nz = s->nz, nb = s->nib;
  const double acc[3] = {-(s->bvel[0] - s->bprev[0]) / s->deltat, -(s->bvel[1] - s->bprev[1]) / s->deltat,
                         -(s->bvel[2] - s->bprev[2]) / s->deltat};
  for (int64_t n = 1; n <= nb; ++n) {
    const int64_t i = L(s->ib, nb, n, 1), j = L(s->ib, nb, n, 2), k = L(s->ib, nb, n, 3);
    const int64_t nel = s->nelp[n];
    const double dpdn = s->moving ? (acc[0] * s->cosA[nel] + acc[1] * s->cosB[nel]) + acc[2] * s->cosG[nel] : 0.0;
    const double sd = s->nd[0][n];
    const double pt1 = 1.5 * sqrt((SQ(s->deltax[i]) + SQ(s->deltay[j])) + SQ(s->deltaz[k])) + (fabs(sd) - sd) * 0.5;
    const double px = s->xp[i] + pt1 * s->cosA[nel];
    const double py = s->yp[j] + pt1 * s->cosB[nel];
    const double pz = s->zp[k] + pt1 * s->cosG[nel];
    int64_t ix = bracket(s->xp, 1, nx + 1, px), iy = bracket(s->yp, 1, ny + 1, py), iz = bracket(s->zp, 1, nz + 1, pz);
    if (!ix || !iy || !iz) return -4;
    double pe[4];
    probe_eval(s, s->p, s->xp, s->yp, s->zp, 0, 0, 0, ix, iy, iz, px, py, pz, pe);
    const double dpdn_e = pe[1] * s->cosA[nel] + pe[2] * s->cosB[nel] + pe[3] * s->cosG[nel];
    const double n1 = pt1 + sd;
    const double bval = dpdn;
    const double aval = (dpdn_e - dpdn) / (2.0 * n1);
    const double cval = pe[0] - (dpdn_e + dpdn) * n1 * 0.5;
    F3(s->p, i, j, k) = aval * SQ(sd) + bval * sd + cval;
  }
  return 0;
}

/* calculateUc (subCalculateuc.f90:2-38): uc = max(mean of ut(nx-4,j,k) over the
 * fluid cells of that plane, 0), summed serially k outer, j inner. */
void or_calculate_uc(OrState* s) {
  const int64_t i = s->nx - 4;
  double uc1 = 0.0;
  int64_t count = 0;
  for (int64_t k = 2; k <= s->nz + 1; ++k)
    for (int64_t j = 2; j <= s->ny + 1; ++j)
      if (F3(s->cell, i, j, k) == 0) {
        uc1 = uc1 + F3(s->ut, i, j, k);
        count = count + 1;
      }
  uc1 = uc1 / (double)count;
  s->uc = uc1 > 0.0 ? uc1 : 0.0;   /* dmax1(uc1, uc0) */
}

void or_set_outlet(OrState* s, int outlet) { s->outlet = outlet; }
double or_uc(const OrState* s) { return s->uc; }

/* Residual of the pressure-correction system at one fluid cell:
 * b/dt - sum(A_nb pc_nb) - diag pc, in the order the SOR numerator uses. */
static inline double cell_residual(const OrState* s, int64_t i, int64_t j, int64_t k, double bdt) {
  const int64_t nx = s->nx, ny = s->ny, nz = s->nz;
  const double* pc = s->pc;
  double num = bdt - L(s->Acx, nx, i - 1, 1) * F3(pc, i - 1, j, k) - L(s->Acx, nx, i - 1, 3) * F3(pc, i + 1, j, k)
               - L(s->Acy, ny, j - 1, 1) * F3(pc, i, j - 1, k) - L(s->Acy, ny, j - 1, 3) * F3(pc, i, j + 1, k)
               - L(s->Acz, nz, k - 1, 1) * F3(pc, i, j, k - 1) - L(s->Acz, nz, k - 1, 3) * F3(pc, i, j, k + 1);
  double diag = L(s->Acx, nx, i - 1, 2) + L(s->Acy, ny, j - 1, 2) + L(s->Acz, nz, k - 1, 2);
  return num - diag * F3(pc, i, j, k);
}

static int red_black_sor_rows(OrState* s, int64_t* isum_out, double* err_out);

/* REDBLACKSOR (subPcorVcor.f90:148-212). Returns 0 on convergence, 1 when
 * max_sweeps ran out (the reference loops forever instead). */
static int red_black_sor(OrState* s, int64_t* isum_out, double* err_out) {
  if (s->sweep_rows) return red_black_sor_rows(s, isum_out, err_out);
  const int64_t nx = s->nx, ny = s->ny, nz = s->nz;
  const double omega = s->omega, deltat = s->deltat;
  double* pc = s->pc;
  double* pco = s->pco;
  const double* b = s->b;
  int64_t isum = 0;
  double err = 0.0;
  for (;;) {
    ++isum;                                                     /* :159 */
    const int64_t nr = s->nred, nk = s->nblack, nf = s->nfluid;
#pragma omp parallel for schedule(static)
    for (int64_t n = 1; n <= nr; ++n) {                          /* :165-175 */
      const int64_t i = L(s->red, nr, n, 1), j = L(s->red, nr, n, 2), k = L(s->red, nr, n, 3);
      double g = (F3(b, i, j, k) / deltat
                  - L(s->Acx, nx, i - 1, 1) * F3(pco, i - 1, j, k) - L(s->Acx, nx, i - 1, 3) * F3(pco, i + 1, j, k)
                  - L(s->Acy, ny, j - 1, 1) * F3(pco, i, j - 1, k) - L(s->Acy, ny, j - 1, 3) * F3(pco, i, j + 1, k)
                  - L(s->Acz, nz, k - 1, 1) * F3(pco, i, j, k - 1) - L(s->Acz, nz, k - 1, 3) * F3(pco, i, j, k + 1))
                 / (L(s->Acx, nx, i - 1, 2) + L(s->Acy, ny, j - 1, 2) + L(s->Acz, nz, k - 1, 2));
      F3(pc, i, j, k) = (1.0 - omega) * F3(pco, i, j, k) + omega * g;
    }
#pragma omp parallel for schedule(static)
    for (int64_t n = 1; n <= nk; ++n) {                          /* :179-190 */
      const int64_t i = L(s->black, nk, n, 1), j = L(s->black, nk, n, 2), k = L(s->black, nk, n, 3);
      double g = (F3(b, i, j, k) / deltat
                  - L(s->Acx, nx, i - 1, 1) * F3(pc, i - 1, j, k) - L(s->Acx, nx, i - 1, 3) * F3(pc, i + 1, j, k)
                  - L(s->Acy, ny, j - 1, 1) * F3(pc, i, j - 1, k) - L(s->Acy, ny, j - 1, 3) * F3(pc, i, j + 1, k)
                  - L(s->Acz, nz, k - 1, 1) * F3(pc, i, j, k - 1) - L(s->Acz, nz, k - 1, 3) * F3(pc, i, j, k + 1))
                 / (L(s->Acx, nx, i - 1, 2) + L(s->Acy, ny, j - 1, 2) + L(s->Acz, nz, k - 1, 2));
      F3(pc, i, j, k) = (1.0 - omega) * F3(pco, i, j, k) + omega * g;
    }
    double derr2 = 0.0;
#pragma omp parallel for schedule(static) reduction(max : derr2)
    for (int64_t n = 1; n <= nf; ++n) {                          /* :194-201 */
      const int64_t i = L(s->fluid, nf, n, 1), j = L(s->fluid, nf, n, 2), k = L(s->fluid, nf, n, 3);
      double d = fabs(F3(pc, i, j, k) - F3(pco, i, j, k));
      if (d > derr2) derr2 = d;
      F3(pco, i, j, k) = F3(pc, i, j, k);
    }
    if (s->criterion == 0) {
      err = derr2;
      if (!(derr2 >= s->eps)) break;                            /* :210 */
    } else if (isum % s->check_every == 0) {
      double rmax = 0.0;
#pragma omp parallel for schedule(static) reduction(max : rmax)
      for (int64_t n = 1; n <= nf; ++n) {
        const int64_t i = L(s->fluid, nf, n, 1), j = L(s->fluid, nf, n, 2), k = L(s->fluid, nf, n, 3);
        double r = fabs(cell_residual(s, i, j, k, F3(b, i, j, k) / deltat));
        if (r > rmax) rmax = r;
      }
      err = rmax;
      if (!(rmax >= s->eps)) break;
    }
    if (isum >= s->max_sweeps) { *isum_out = isum; *err_out = err; return 1; }
  }
  *isum_out = isum;
  *err_out = err;
  return 0;
}

/* The same sweep loop as red_black_sor, for the timed CPU baseline: each colour pass
 * walks the rows (j,k) of the field and updates that colour's fluid cells (the mask
 * cellCount built) instead of gathering through the int64 red/black lists, so the
 * OpenMP threads stream contiguous memory. Every cell's arithmetic is the list form's,
 * expression for expression, and the values it reads are the same: a red cell's
 * neighbours are black or non-fluid, so pco there equals pc; a cell's own pco equals
 * its pc until its colour pass writes it, so the update-norm max |pc - pco| is taken
 * as each cell is written, and the pco copy pass drops out. b/deltat is divided once
 * per solve (the same quotient the list form rounds in every sweep). Results, sweep
 * counts included, are bit-identical to red_black_sor's (tests/test_oracle.py). */
static int red_black_sor_rows(OrState* s, int64_t* isum_out, double* err_out) {
  const int64_t nx = s->nx, ny = s->ny, nz = s->nz;
  const int64_t sy = NX2, sz = NX2 * NY2, n3 = sz * (nz + 2);
  const double omega = s->omega, deltat = s->deltat;
  double* pc = s->pc;
  const unsigned char* fm = s->fmask;
  if (!s->bdt) s->bdt = (double*)malloc((size_t)n3 * sizeof(double));
  double* bdt = s->bdt;
#pragma omp parallel for schedule(static)
  for (int64_t q = 0; q < n3; ++q) bdt[q] = s->b[q] / deltat;
  const double *ax1 = s->Acx, *ax2 = s->Acx + nx, *ax3 = s->Acx + 2 * nx;
  const double *ay1 = s->Acy, *ay2 = s->Acy + ny, *ay3 = s->Acy + 2 * ny;
  const double *az1 = s->Acz, *az2 = s->Acz + nz, *az3 = s->Acz + 2 * nz;
  int64_t isum = 0;
  double err = 0.0;
  for (;;) {
    ++isum;
    double derr2 = 0.0;
    for (int colour = 1; colour >= 0; --colour) {   /* red ((i+j+k) odd) first, then black */
#pragma omp parallel for collapse(2) schedule(static) reduction(max : derr2)
      for (int64_t k = 2; k <= nz + 1; ++k)
        for (int64_t j = 2; j <= ny + 1; ++j) {
          const int64_t i0 = ((2 + j + k) % 2 == colour) ? 2 : 3;
          const int64_t row = (j - 1) * sy + (k - 1) * sz;
          const double ya = ay1[j - 2], yc = ay3[j - 2], za = az1[k - 2], zc = az3[k - 2];
          const double dyz2 = ay2[j - 2], dz2 = az2[k - 2];
          double dmax = derr2;
          for (int64_t i = i0; i <= nx + 1; i += 2) {
            const int64_t o = row + (i - 1);
            if (!fm[o]) continue;
            const double g = (bdt[o] - ax1[i - 2] * pc[o - 1] - ax3[i - 2] * pc[o + 1] - ya * pc[o - sy] -
                              yc * pc[o + sy] - za * pc[o - sz] - zc * pc[o + sz]) /
                             (ax2[i - 2] + dyz2 + dz2);
            const double old = pc[o];
            const double nv = (1.0 - omega) * old + omega * g;
            pc[o] = nv;
            const double d = fabs(nv - old);
            if (d > dmax) dmax = d;
          }
          derr2 = dmax;
        }
    }
    if (s->criterion == 0) {
      err = derr2;
      if (!(derr2 >= s->eps)) break;                            /* :210 */
    } else if (isum % s->check_every == 0) {
      double rmax = 0.0;
#pragma omp parallel for collapse(2) schedule(static) reduction(max : rmax)
      for (int64_t k = 2; k <= nz + 1; ++k)
        for (int64_t j = 2; j <= ny + 1; ++j) {
          double m = rmax;
          for (int64_t i = 2; i <= nx + 1; ++i) {
            if (!F3(fm, i, j, k)) continue;
            const double r = fabs(cell_residual(s, i, j, k, F3(bdt, i, j, k)));
            if (r > m) m = r;
          }
          rmax = m;
        }
      err = rmax;
      if (!(rmax >= s->eps)) break;
    }
    if (isum >= s->max_sweeps) { *isum_out = isum; *err_out = err; return 1; }
  }
  *isum_out = isum;
  *err_out = err;
  return 0;
}

void or_set_sweep_rows(OrState* s, int on) { s->sweep_rows = on ? 1 : 0; }

/* writeResult (subWriteOutput.f90:62-72): one list-directed record
 * "u v w p totime ita ita1" per cell, k outer, j, i inner. Values are written with
 * 17 significant digits, so every double reads back exactly. */
int or_write_result_text(OrState* s, const char* path, double totime, int64_t ita, int64_t ita1) {
  FILE* fp = fopen(path, "w");
  if (!fp) return 1;
  int ok = 1;
  for (int64_t k = 1; k <= s->nz + 2 && ok; ++k)
    for (int64_t j = 1; j <= s->ny + 2 && ok; ++j)
      for (int64_t i = 1; i <= s->nx + 2 && ok; ++i)
        ok = fprintf(fp, " %.17g %.17g %.17g %.17g %.17g %lld %lld\n", F3(s->u, i, j, k), F3(s->v, i, j, k),
                     F3(s->w, i, j, k), F3(s->p, i, j, k), totime, (long long)ita, (long long)ita1) > 0;
  if (fclose(fp) != 0) ok = 0;
  return ok ? 0 : 1;
}

/* Next value of a list-directed record: blanks, tabs, line ends and at most one
 * comma separate values, so a record may continue on the following lines. */
static int list_value(FILE* fp, double* out) {
  int ch, comma = 0;
  while ((ch = fgetc(fp)) != EOF) {
    if (ch == ' ' || ch == '\t' || ch == '\n' || ch == '\r') continue;
    if (ch == ',' && !comma) { comma = 1; continue; }
    break;
  }
  if (ch == EOF) return 0;
  char buf[64];
  int n = 0;
  while (ch != EOF && ch != ' ' && ch != '\t' && ch != '\n' && ch != '\r' && ch != ',' && n < 63) {
    buf[n++] = (char)ch;
    ch = fgetc(fp);
  }
  if (ch != EOF) ungetc(ch, fp);
  buf[n] = 0;
  char* end = NULL;
  *out = strtod(buf, &end);
  return n > 0 && end == buf + n;
}

/* lastConditions (subLastConditions.f90:2-42): resi_u/v/w = 0 (:15-17), then
 * READ(1,*) u, v, w, p, totime, ita, ita1 for every cell in the order writeResult
 * wrote them (:23-29; each READ starts a new record and drops what is left of the
 * line), then ut = u, vt = v, wt = w (:32-38). Returns 1 on a short or malformed file. */
int or_read_result_text(OrState* s, const char* path, double* totime, int64_t* ita, int64_t* ita1) {
  FILE* fp = fopen(path, "r");
  if (!fp) return 1;
  const int64_t n3 = NX2 * NY2 * (s->nz + 2);
  memset(s->resi_u, 0, (size_t)n3 * sizeof(double));
  memset(s->resi_v, 0, (size_t)n3 * sizeof(double));
  memset(s->resi_w, 0, (size_t)n3 * sizeof(double));
  double t = 0.0, it = 0.0, it1 = 0.0;
  int ok = 1;
  for (int64_t k = 1; k <= s->nz + 2 && ok; ++k)
    for (int64_t j = 1; j <= s->ny + 2 && ok; ++j)
      for (int64_t i = 1; i <= s->nx + 2 && ok; ++i) {
        ok = list_value(fp, &F3(s->u, i, j, k)) && list_value(fp, &F3(s->v, i, j, k)) &&
             list_value(fp, &F3(s->w, i, j, k)) && list_value(fp, &F3(s->p, i, j, k)) && list_value(fp, &t) &&
             list_value(fp, &it) && list_value(fp, &it1);
        int ch;
        while (ok && (ch = fgetc(fp)) != EOF && ch != '\n') {
        }
      }
  fclose(fp);
  if (!ok) return 1;
  memcpy(s->ut, s->u, (size_t)n3 * sizeof(double));
  memcpy(s->vt, s->v, (size_t)n3 * sizeof(double));
  memcpy(s->wt, s->w, (size_t)n3 * sizeof(double));
  if (totime) *totime = t;
  if (ita) *ita = (int64_t)it;
  if (ita1) *ita1 = (int64_t)it1;
  return 0;
}

/* poissonSolver (subPcorVcor.f90:2-80) with computeDiv (82-101), correctPressure
 * (105-120), correctVelocity (125-142), velocityBC and the steady-state
 * indicator (45-58). */
/* REDBLACKSOR alone (subPcorVcor.f90:148-212) on the b already in place, from pc = 0
 * as poissonSolver starts it (:19-28); no divergence, no corrections. */
int or_redblack_sor(OrState* s, int64_t* nsweeps, double* final_err) {
  const int64_t n3 = NX2 * NY2 * (s->nz + 2);
  memset(s->pc, 0, (size_t)n3 * sizeof(double));
  memset(s->pco, 0, (size_t)n3 * sizeof(double));
  int64_t isum = 0;
  double err = 0.0;
  const int rc = red_black_sor(s, &isum, &err);
  if (nsweeps) *nsweeps = isum;
  if (final_err) *final_err = err;
  return rc;
}

int or_poisson_solver(OrState* s, int64_t* nsweeps, double* divmax_out, double* derrStdSt_out,
                      double* final_err) {
  const int64_t n3 = NX2 * NY2 * (s->nz + 2);
  const double deltat = s->deltat;
  memset(s->b, 0, (size_t)n3 * sizeof(double));                 /* :19-28 */
  memset(s->pc, 0, (size_t)n3 * sizeof(double));
  memset(s->pco, 0, (size_t)n3 * sizeof(double));
  const int64_t nf = s->nfluid;
  double divmax = 0.0;
#pragma omp parallel for schedule(static) reduction(max : divmax)
  for (int64_t n = 1; n <= nf; ++n) {                            /* :91-99 */
    const int64_t i = L(s->fluid, nf, n, 1), j = L(s->fluid, nf, n, 2), k = L(s->fluid, nf, n, 3);
    double bb = (F3(s->ut, i, j, k) - F3(s->ut, i - 1, j, k)) / s->deltax[i] +
                (F3(s->vt, i, j, k) - F3(s->vt, i, j - 1, k)) / s->deltay[j] +
                (F3(s->wt, i, j, k) - F3(s->wt, i, j, k - 1)) / s->deltaz[k];
    F3(s->b, i, j, k) = bb;
    if (fabs(bb) > divmax) divmax = fabs(bb);
  }
  int64_t isum = 0;
  double err = 0.0;
  int rc = red_black_sor(s, &isum, &err);
#pragma omp parallel for schedule(static)
  for (int64_t n = 1; n <= nf; ++n) {                            /* :113-118 */
    const int64_t i = L(s->fluid, nf, n, 1), j = L(s->fluid, nf, n, 2), k = L(s->fluid, nf, n, 3);
    F3(s->p, i, j, k) = F3(s->p, i, j, k) + F3(s->pc, i, j, k);
  }
#pragma omp parallel for schedule(static)
  for (int64_t n = 1; n <= nf; ++n) {                            /* :132-140 */
    const int64_t i = L(s->fluid, nf, n, 1), j = L(s->fluid, nf, n, 2), k = L(s->fluid, nf, n, 3);
    const double* pc = s->pc;
    F3(s->ut, i, j, k) = F3(s->ut, i, j, k) - deltat / (0.5 * (s->deltax[i + 1] + s->deltax[i])) * (F3(pc, i + 1, j, k) - F3(pc, i, j, k));
    F3(s->vt, i, j, k) = F3(s->vt, i, j, k) - deltat / (0.5 * (s->deltay[j + 1] + s->deltay[j])) * (F3(pc, i, j + 1, k) - F3(pc, i, j, k));
    F3(s->wt, i, j, k) = F3(s->wt, i, j, k) - deltat / (0.5 * (s->deltaz[k + 1] + s->deltaz[k])) * (F3(pc, i, j, k + 1) - F3(pc, i, j, k));
  }
  or_velocity_bc(s);                                             /* :43 */
  double dss = 0.0;
#pragma omp parallel for schedule(static) reduction(max : dss)
  for (int64_t n = 1; n <= nf; ++n) {                            /* :49-57 */
    const int64_t i = L(s->fluid, nf, n, 1), j = L(s->fluid, nf, n, 2), k = L(s->fluid, nf, n, 3);
    double du = fabs(F3(s->ut, i, j, k) - F3(s->u, i, j, k)) / deltat;
    double dv = fabs(F3(s->vt, i, j, k) - F3(s->v, i, j, k)) / deltat;
    double dw = fabs(F3(s->wt, i, j, k) - F3(s->w, i, j, k)) / deltat;
    double m = dss;
    if (du > m) m = du;
    if (dv > m) m = dv;
    if (dw > m) m = dw;
    dss = m;
  }
  memcpy(s->u, s->ut, (size_t)n3 * sizeof(double));              /* :67-77 */
  memcpy(s->v, s->vt, (size_t)n3 * sizeof(double));
  memcpy(s->w, s->wt, (size_t)n3 * sizeof(double));
  if (nsweeps) *nsweeps = isum;
  if (divmax_out) *divmax_out = divmax;
  if (derrStdSt_out) *derrStdSt_out = dss;
  if (final_err) *final_err = err;
  return rc;
}

/* stressCal1 (subStressCal1.f90:2-460) when first != 0 or no cache exists,
 * else stressCal2 (subStressCal2.f90:2-381), which reuses the cached probe cells.
 * coef = {Cd viscous, Cd pressure, Cl viscous, Cl pressure}. */
int or_stress(OrState* s, int first, double coef[4]) {
  const int64_t nx = s->nx, ny = s->ny, nz = s->nz, ne = s->nelems;
  if (first || !s->have_scache) {
    for (int q = 0; q < 5; ++q) { free(s->scache[q]); s->scache[q] = (int64_t*)calloc((size_t)(3 * ne + 3), sizeof(int64_t)); }
  }
  const int use_cache = !(first || !s->have_scache);
  double viscousDrag = 0.0, pressureDrag = 0.0, viscousLift = 0.0, pressureLift = 0.0;
  double surf_area = 0.0, area_Sx = 0.0, area_Sy = 0.0;
  const double* XS[4][3] = {{s->xu, s->yu, s->zu}, {s->xv, s->yv, s->zv}, {s->xw, s->yw, s->zw}, {s->xp, s->yp, s->zp}};
  const double* FS[3] = {s->ut, s->vt, s->wt};
  for (int64_t e = 1; e <= ne; ++e) {
    int64_t ic, jc, kc;
    if (use_cache) {
      ic = L(s->scache[0], ne, e, 1); jc = L(s->scache[0], ne, e, 2); kc = L(s->scache[0], ne, e, 3);
    } else {                                                     /* :89-109 */
      ic = bracket(s->x1, 2, nx + 1, s->xcent[e]);
      jc = bracket(s->y1, 2, ny + 1, s->ycent[e]);
      kc = bracket(s->z1, 2, nz + 1, s->zcent[e]);
      if (!ic || !jc || !kc) return -4;
      L(s->scache[0], ne, e, 1) = ic; L(s->scache[0], ne, e, 2) = jc; L(s->scache[0], ne, e, 3) = kc;
    }
    const double xs = s->xcent[e], ys = s->ycent[e], zs = s->zcent[e];
    const double dX = s->x1[ic + 1] - s->x1[ic], dY = s->y1[jc + 1] - s->y1[jc], dZ = s->z1[kc + 1] - s->z1[kc];
    const double diagdis = sqrt((SQ(dX) + SQ(dY)) + SQ(dZ));        /* :119 */
    const double normdis = diagdis;
    const double ca = s->cosA[e], cb = s->cosB[e], cg = s->cosG[e];
    const double px = xs + normdis * ca, py = ys + normdis * cb, pz = zs + normdis * cg;
    double dnds[3];
    for (int c = 0; c < 3; ++c) {                                /* u :134-195, v :198-260, w :263-324 */
      int64_t ix, iy, iz;
      if (use_cache) {
        ix = L(s->scache[1 + c], ne, e, 1); iy = L(s->scache[1 + c], ne, e, 2); iz = L(s->scache[1 + c], ne, e, 3);
      } else {
        ix = bracket(XS[c][0], 2, nx + 1, px);
        iy = bracket(XS[c][1], 2, ny + 1, py);
        iz = bracket(XS[c][2], 2, nz + 1, pz);
        if (!ix || !iy || !iz) return -4;
        L(s->scache[1 + c], ne, e, 1) = ix; L(s->scache[1 + c], ne, e, 2) = iy; L(s->scache[1 + c], ne, e, 3) = iz;
      }
      double pe[4];
      probe_eval(s, FS[c], XS[c][0], XS[c][1], XS[c][2], c == 0 ? -1 : 0, c == 1 ? -1 : 0, c == 2 ? -1 : 0,
                 ix, iy, iz, px, py, pz, pe);
      const double dn_e = pe[1] * ca + pe[2] * cb + pe[3] * cg;
      dnds[c] = (2.0 / normdis) * (pe[0] - 0.0) - dn_e;
    }
    const double a3 = s->alpha3[e], b3 = s->beta3[e], g3 = s->gamma3[e];
    const double alen = sqrt((SQ(a3) + SQ(b3)) + SQ(g3));          /* :327-331 */
    const double area = alen / 2.0;
    const double area_yz = 0.5 * fabs(a3);
    const double area_xz = 0.5 * fabs(b3);
    const double dot = dnds[0] * ca + dnds[1] * cb + dnds[2] * cg;
    const double stx1 = dnds[0] - dot * ca;                         /* :335-339 */
    const double sty1 = dnds[1] - dot * cb;
    const double shear_x = (1.0 / s->re) * stx1 * area;             /* :341-345 */
    const double shear_y = (1.0 / s->re) * sty1 * area;
    int64_t ix, iy, iz;
    if (use_cache) {
      ix = L(s->scache[4], ne, e, 1); iy = L(s->scache[4], ne, e, 2); iz = L(s->scache[4], ne, e, 3);
    } else {                                                     /* :352-367 */
      ix = bracket(s->xp, 2, nx + 1, px);
      iy = bracket(s->yp, 2, ny + 1, py);
      iz = bracket(s->zp, 2, nz + 1, pz);
      if (!ix || !iy || !iz) return -4;
      L(s->scache[4], ne, e, 1) = ix; L(s->scache[4], ne, e, 2) = iy; L(s->scache[4], ne, e, 3) = iz;
    }
    double pe[4];
    probe_eval(s, s->p, s->xp, s->yp, s->zp, 0, 0, 0, ix, iy, iz, px, py, pz, pe);
    const double dpdn_e = pe[1] * ca + pe[2] * cb + pe[3] * cg;
    const double dpdn = 0.0;
    const double cval = pe[0] - (dpdn_e + dpdn) * diagdis * 0.5;    /* :413-415 */
    const double f_surf = cval * area;
    const double fx = -f_surf * ca, fy = -f_surf * cb;
    viscousDrag = viscousDrag + shear_x;                           /* :428-434 */
    pressureDrag = pressureDrag + fx;
    viscousLift = viscousLift + shear_y;
    pressureLift = pressureLift + fy;
    surf_area = surf_area + area;
    area_Sx = area_Sx + area_xz;
    area_Sy = area_Sy + area_yz;
  }
  s->have_scache = 1;
  area_Sx = 0.5 * area_Sx;                                       /* :441-450 */
  area_Sy = 0.5 * area_Sy;
  coef[0] = 2.0 * (viscousDrag / area_Sx);
  coef[1] = 2.0 * (pressureDrag / area_Sy);
  coef[2] = 2.0 * (viscousLift / area_Sy);
  coef[3] = 2.0 * (pressureLift / area_Sx);
  (void)surf_area;
  return 0;
}

/* One time step in main.f90's order (:42-66; step 1 at :26-39). */
int or_step(OrState* s, int first, int64_t* nsweeps, double coef[4]) {
  if (s->momentum == 1 && !first) or_ns_momentum_ab(s);        /* main.f90:45 */
  else or_ns_momentum(s);                                      /* main.f90:46 (30) */
  or_velocity_bc(s);
  or_solid_cell_bc(s);
  int rc = or_velocity_forcing(s);
  if (rc) return rc;
  or_velocity_bc(s);
  double divmax, dss, err;
  int nc = or_poisson_solver(s, nsweeps, &divmax, &dss, &err);
  rc = or_pressure_forcing(s);
  if (rc) return rc;
  if (s->outlet == 1) or_calculate_uc(s);                       /* main.f90:53-54 hook */
  rc = or_stress(s, first, coef);
  if (rc) return rc;
  return nc;
}

double* or_field(OrState* s, int which) {
  double* f[] = {s->u, s->v, s->w, s->ut, s->vt, s->wt, s->p, s->pc, s->b};
  return (which >= 0 && which < 9) ? f[which] : NULL;
}
int64_t* or_cell(OrState* s) { return s->cell; }
void or_counts(OrState* s, int64_t out[5]) {
  out[0] = s->nfluid; out[1] = s->nsolid; out[2] = s->nib; out[3] = s->nred; out[4] = s->nblack;
}
int64_t* or_list(OrState* s, int which) {
  int64_t* l[] = {s->fluid, s->solid, s->ib, s->red, s->black};
  return (which >= 0 && which < 5) ? l[which] : NULL;
}
double* or_surface(OrState* s, int which) {
  double* a[] = {s->xcent, s->ycent, s->zcent, s->cosA, s->cosB, s->cosG, s->alpha3, s->beta3, s->gamma3};
  return (which >= 0 && which < 9) ? a[which] + 1 : NULL;
}
double* or_normdis(OrState* s, int which) { return (which >= 0 && which < 7 && s->nd[which]) ? s->nd[which] + 1 : NULL; }
int64_t* or_nelp(OrState* s) { return s->nelp ? s->nelp + 1 : NULL; }
double* or_acoef(OrState* s, int axis) { return axis == 0 ? s->Acx : axis == 1 ? s->Acy : s->Acz; }
double* or_conv_coef(OrState* s, int fam, int m) { return s->cc[fam][m]; }
double* or_grid1d(OrState* s, int which) {
  double* a[] = {s->x1, s->y1, s->z1, s->deltax, s->deltay, s->deltaz, s->xu, s->yu, s->zu,
                 s->xv, s->yv, s->zv, s->xw, s->yw, s->zw, s->xp, s->yp, s->zp};
  return (which >= 0 && which < 18) ? a[which] : NULL;
}
