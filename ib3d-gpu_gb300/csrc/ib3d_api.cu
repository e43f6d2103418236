// C ABI of the GB300 IB3D hot path (declared in include/ib3d.h): context set-up,
// host-side grid tables, device residency and the per-step entry points that
// replace the reference's Fortran subroutine calls.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>

#include "ib3d_internal.cuh"

namespace ib3d {

int cuda_fail(ib3d_ctx* c, cudaError_t e, const char* where) {
  if (c) {
    char buf[512];
    snprintf(buf, sizeof(buf), "CUDA error %d (%s) at %s", (int)e, cudaGetErrorString(e), where);
    c->err = buf;
  }
  return IB3D_ERR_CUDA;
}

void free_ib(ib3d_ctx* c);

cudaEvent_t timer_event(ib3d_ctx* c) {
  if (!c->pool.empty()) {
    cudaEvent_t e = c->pool.back();
    c->pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

namespace {
// Resolves the recorded event pairs into per-phase milliseconds.
void timer_fold(ib3d_ctx* c) {
  if (c->pending.empty()) return;
  cudaStreamSynchronize(c->st);
  for (auto& pr : c->pending) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, pr.a, pr.b) == cudaSuccess) c->tms[pr.phase] += ms;
    c->pool.push_back(pr.a);
    c->pool.push_back(pr.b);
  }
  c->pending.clear();
}
}  // namespace

void timer_push(ib3d_ctx* c, int phase, cudaEvent_t a, cudaEvent_t b) {
  c->pending.push_back({phase, a, b});
  if (c->pending.size() > 4096) timer_fold(c);
}

namespace {

// One station of non_uni_coeff (subNavierStokes.f90:37-116): the 12 coefficients of
// the non-uniform third-order upwind stencil from three spacing ratios. Integral
// powers x**2.0, x**3.0, x**4.0 are products evaluated left to right.
void conv_station(double t1, double t2, double t3, double out[12]) {
  const double t3_2 = t3 * t3, t3_3 = t3 * t3 * t3, t3_4 = t3 * t3 * t3 * t3;
  const double t1_2 = t1 * t1, t1_3 = t1 * t1 * t1, t1_4 = t1 * t1 * t1 * t1;
  const double t2_2 = t2 * t2, t2_3 = t2 * t2 * t2, t2_4 = t2 * t2 * t2 * t2;
  const double f1 = t3;
  const double f2 = 2.0 * t3 + t3_2;
  const double f3 = 3.0 * t3 + 3.0 * t3_2 + t3_3;
  const double f4 = 4.0 * t3 + 6.0 * t3_2 + 4.0 * t3_3 + t3_4;
  const double f5 = 1.0 / (t1 * t2);
  const double f6 = (2.0 * t1 + 1.0) / (t1_2 * t2_2);
  const double f7 = (3.0 * t1_2 + 3.0 * t1 + 1.0) / (t1_3 * t2_3);
  const double f8 = (4.0 * t1_3 + 6.0 * t1_2 + 4.0 * t1 + 1.0) / (t1_4 * t2_4);
  const double s51 = -1.0 / t2_4, s52 = f4, s53 = f4, s54 = s51;
  const double s55 = -(f1 / t2_4 + f4 / t2);
  const double s56 = (f4 / t2_2 - f2 / t2_4);
  const double s57 = -(f3 / t2_4 + f4 / t2_3);
  const double s61 = -1.0, s62 = f8, s63 = f8, s64 = -1.0;
  const double s65 = (f5 + f8), s66 = (f8 - f6), s67 = (f7 + f8);
  const double s71 = -1.0, s72 = (1.0 + f4), s73 = f4, s74 = (f4 - f1), s75 = (f4 - f2), s76 = (f4 - f3);
  const double s81 = -1.0 / t2_4;
  const double s82 = (f8 + (1.0 / t2_4));
  const double s83 = f8;
  const double s84 = (f5 / t2_4 - f8 / t2);
  const double s85 = (f8 / t2_2 - f6 / t2_4);
  const double s86 = (f7 / t2_4 - f8 / t2_3);
  const double s91 = -s66 * s51;
  const double s92 = s56 * s61;
  const double s93 = -(s54 * s66 + s56 * s62);
  const double s94 = (s56 * s64 + s66 * s52);
  const double s95 = (s56 * s63 - s66 * s53);
  const double s96 = (s56 * s65 - s66 * s55);
  const double s97 = (s56 * s67 - s66 * s57);
  const double s101 = -s85 * s71;
  const double s102 = -s85 * s72;
  const double s103 = s75 * s81;
  const double s104 = s75 * s82;
  const double s105 = (s75 * s83 - s85 * s73);
  const double s106 = (s75 * s84 - s85 * s74);
  const double s107 = (s75 * s86 - s85 * s76);
  out[0] = (s97 * s101 - s107 * s91);
  out[1] = (s97 * s102 + s107 * s93);
  out[2] = (s95 * s107 - s105 * s97);
  out[3] = (s94 * s107 + s104 * s97);
  out[4] = (s97 * s103 - s107 * s92);
  out[5] = (s97 * s106 - s107 * s96);
  const double ak1 = (1.0 + 2.0 * t1) * (t3 + t3_2) * t2;
  const double ak2 = (1.0 + t1) * (2.0 * t3 + t3_2);
  const double ak3 = (1.0 + t1);
  const double ak4 = (1.0 + t1) * ((1.0 + t3) * (1.0 + t3));
  const double ak5 = ((1.0 + t1) * (1.0 + t1)) * (t3 + t3_2) * t2;
  const double ak6 = t1_2 * t2 * (t3 + t3_2);
  const double ak7 = (1.0 + t1) * (t3 + t3_2) * t2;
  out[6] = ak3;
  out[7] = -ak4;
  out[8] = (ak1 + ak2);
  out[9] = -ak5;
  out[10] = ak6;
  out[11] = ak7;
}

// readInput's grid part (subReadInput.f90:55-129) for one axis: node coordinates
// x1(1..n+3), spacings d(1..n+2), face and centre coordinates.
bool axis_tables(int n, const double* nodes, std::vector<double>& x1, std::vector<double>& dd,
                 std::vector<double>& face, std::vector<double>& centre) {
  x1.assign((size_t)n + 4, 0.0);
  dd.assign((size_t)n + 3, 0.0);
  for (int i = 2; i <= n + 2; ++i) x1[i] = nodes[i - 2];
  for (int i = 2; i <= n + 1; ++i) dd[i] = x1[i + 1] - x1[i];
  dd[1] = dd[2];
  dd[n + 2] = dd[n + 1];
  x1[1] = x1[2] - dd[1];
  x1[n + 3] = x1[n + 2] + dd[n + 2];
  face = x1;                                   // xu = x1 (:101-103)
  centre.assign((size_t)n + 3, 0.0);
  for (int i = 1; i <= n + 2; ++i) centre[i] = 0.5 * (x1[i] + x1[i + 1]);   // :119-123
  for (int i = 1; i <= n + 2; ++i)
    if (!(dd[i] > 0.0) || !std::isfinite(dd[i])) return false;
  return true;
}

// coefficientMatrix for one axis (subCoefficientMatrix.f90:8-33), boundary rows
// folded in as :36-53 do: low end Neumann; high end Neumann, or Dirichlet (outlet).
void poisson_axis(int n, const std::vector<double>& c, bool dirichlet_hi, std::vector<double> a[3]) {
  for (int q = 0; q < 3; ++q) a[q].assign((size_t)n + 1, 0.0);
  for (int i = 2; i <= n + 1; ++i) {
    const double r1 = c[i] - c[i - 1], r2 = c[i + 1] - c[i], rs = r1 + r2;
    a[0][i - 1] = 2.0 / (r1 * rs);
    a[1][i - 1] = -2.0 / (r1 * r2);
    a[2][i - 1] = 2.0 / (r2 * rs);
  }
  a[1][1] = a[1][1] + a[0][1];
  a[0][1] = 0.0;
  if (dirichlet_hi) a[1][n] = a[1][n] - a[2][n];
  else a[1][n] = a[1][n] + a[2][n];
  a[2][n] = 0.0;
}

// 1-D tables of the fast momentum kernel (k_momentum_fast.cu lists them): the
// quotients of nsMomentum whose divisors depend only on the grid.
void fast_tables(const std::vector<double>& d, int n, int axis, const std::vector<double> cc[6][12], int S,
                 std::vector<double>& out) {
  auto put = [&](int t, int m, double v) { out[(size_t)(axis * kFastTables + t) * S + m] = std::isfinite(v) ? v : 0.0; };
  for (int m = 2; m <= n + 1; ++m) {
    const double dm = d[m], dp = d[m + 1], dl = d[m - 1];
    put(0, m, dp / (dm + dp));
    put(1, m, 1.0 / (cc[axis][5][m] * dp));
    put(2, m, 1.0 / (2.0 * cc[axis][11][m] * dm));
    put(3, m, 1.0 / (cc[3 + axis][5][m] * (0.5 * (dm + dp))));
    put(4, m, 1.0 / (2.0 * cc[3 + axis][11][m] * (0.5 * (dm + dl))));
    const double rn[2] = {dm / dp, (0.5 * (dm + dl)) / (0.5 * (dm + dp))};
    const double da[2] = {dp, 0.5 * (dm + dp)};
    for (int f = 0; f < 2; ++f) {
      const double r = rn[f];
      const int b = 5 + 8 * f;
      put(b + 0, m, -1.0 / (r * (r + 1.0)));
      put(b + 1, m, 1.0 - 1.0 / r);
      put(b + 2, m, r / (r + 1.0));
      put(b + 3, m, 2.0 / (r * (r + 1.0)));
      put(b + 4, m, 2.0 / r);
      put(b + 5, m, 2.0 / (r + 1.0));
      put(b + 6, m, 1.0 / da[f]);
      put(b + 7, m, 1.0 / (2.0 * da[f]));
    }
    put(21, m, 2.0 / ((dm + dp) * dp));
    put(22, m, 2.0 / ((dm + dp) * dm));
    const double hs = 0.5 * ((dm + dp) + (dm + dl));
    put(23, m, 2.0 / (hs * (0.5 * (dm + dp))));
    put(24, m, 2.0 / (hs * (0.5 * (dm + dl))));
    put(25, m, 1.0 / dm);
    // third-order upwind folded: adv*sa*ra + |adv|*sk*rk = adv * sum_q (ca*ra +- ck*rk) q,
    // + for adv >= 0 and - for adv < 0, for the own-axis family (ra, rk of tables 1, 2)
    // and the transverse one (tables 3, 4)
    const double ro[2] = {1.0 / (cc[axis][5][m] * dp), 1.0 / (cc[3 + axis][5][m] * (0.5 * (dm + dp)))};
    const double rk[2] = {1.0 / (2.0 * cc[axis][11][m] * dm), 1.0 / (2.0 * cc[3 + axis][11][m] * (0.5 * (dm + dl)))};
    for (int h = 0; h < 2; ++h) {
      const int fam = h == 0 ? axis : 3 + axis;
      for (int q = 0; q < 5; ++q) {
        const double a = cc[fam][q][m] * ro[h], k = cc[fam][6 + q][m] * rk[h];
        put(26 + 10 * h + q, m, a + k);
        put(31 + 10 * h + q, m, a - k);
      }
    }
  }
}

struct Packer {
  std::vector<double> host;
  std::vector<std::pair<const double**, size_t>> fix;
  void add(const std::vector<double>& v, const double** slot) {
    fix.push_back({slot, host.size()});
    host.insert(host.end(), v.begin(), v.end());
    while (host.size() % 4) host.push_back(0.0);   // 32-byte alignment of each table
  }
};

int alloc_fields(ib3d_ctx* c) {
  const size_t n3 = (size_t)c->d.n3;
  double** f[] = {&c->u, &c->v, &c->w, &c->ut, &c->vt, &c->wt, &c->p, &c->pc, &c->b, &c->bdt};
  for (double** q : f) {
    if (cudaMalloc(q, n3 * sizeof(double)) != cudaSuccess) return IB3D_ERR_MEMORY;
    if (cudaMemsetAsync(*q, 0, n3 * sizeof(double), c->st) != cudaSuccess) return IB3D_ERR_CUDA;
  }
  if (cudaMalloc(&c->e32, n3 * sizeof(float)) != cudaSuccess) return IB3D_ERR_MEMORY;
  if (cudaMalloc(&c->r32, n3 * sizeof(float)) != cudaSuccess) return IB3D_ERR_MEMORY;
  if (c->d.nx % 2 == 0) {   // colour-packed arrays of the FP32 inner solve (even nx)
    c->packed_lp = packed_row_length(c->d.nx);
    const size_t np = (size_t)c->packed_lp * (size_t)c->d.NY2 * (size_t)c->d.NZ2;
    if (np >= ((size_t)1 << 31)) return IB3D_ERR_TOO_LARGE;   // the sweep kernels use 32-bit offsets
    for (int q = 0; q < 2; ++q) {
      if (cudaMalloc(&c->ep[q], np * sizeof(float)) != cudaSuccess) return IB3D_ERR_MEMORY;
      if (cudaMalloc(&c->rp[q], np * sizeof(float)) != cudaSuccess) return IB3D_ERR_MEMORY;
      cudaMemsetAsync(c->ep[q], 0, np * sizeof(float), c->st);
      cudaMemsetAsync(c->rp[q], 0xff, np * sizeof(float), c->st);   // all-ones bits: NaN
    }
  }
  if (cudaMalloc(&c->cell, n3) != cudaSuccess) return IB3D_ERR_MEMORY;
  if (cudaMalloc(&c->ibmap, n3 * sizeof(int)) != cudaSuccess) return IB3D_ERR_MEMORY;
  cudaMemsetAsync(c->e32, 0, n3 * sizeof(float), c->st);
  cudaMemsetAsync(c->r32, 0, n3 * sizeof(float), c->st);
  cudaMemsetAsync(c->cell, 0, n3, c->st);
  cudaMemsetAsync(c->ibmap, 0xff, n3 * sizeof(int), c->st);
  if (cudaMalloc(&c->ctl, sizeof(SolveCtl)) != cudaSuccess) return IB3D_ERR_MEMORY;
  if (cudaMallocHost(&c->h_ctl, sizeof(SolveCtl)) != cudaSuccess) return IB3D_ERR_MEMORY;
  if (cudaMalloc(&c->d_flag, sizeof(int)) != cudaSuccess) return IB3D_ERR_MEMORY;
  if (cudaMalloc(&c->d_coef, 8 * sizeof(double)) != cudaSuccess) return IB3D_ERR_MEMORY;
  {
    const double uc0 = 1.0;   // uc = 1 (subReadInput.f90:28); d_coef[6] holds the outlet speed
    if (cudaMemcpy(c->d_coef + 6, &uc0, sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess) return IB3D_ERR_CUDA;
  }
  c->scan_cap = 64;
  if (cudaMalloc(&c->d_scan, c->scan_cap * sizeof(long long)) != cudaSuccess) return IB3D_ERR_MEMORY;
  cudaMemsetAsync(c->ctl, 0, sizeof(SolveCtl), c->st);
  return IB3D_OK;
}

bool valid_params(const ib3d_params* p) {
  return p && p->re > 0 && std::isfinite(p->re) && p->deltat > 0 && std::isfinite(p->deltat) && p->omega > 0 &&
         p->omega < 2 && p->eps > 0 && p->max_sweeps >= 1 && (p->criterion == 0 || p->criterion == 1) &&
         (p->precision >= IB3D_PREC_FP64 && p->precision <= IB3D_PREC_FP64_FAST) && (p->warm_start >= 0 && p->warm_start <= 2) &&
         p->check_every >= 1 && p->inner_sweeps >= 1 && (p->sweep_kernel >= 0 && p->sweep_kernel <= 4) &&
         (p->omega_inner == 0.0 || (p->omega_inner > 0.0 && p->omega_inner < 2.0)) &&
         (p->inner_schedule >= IB3D_INNER_FIXED && p->inner_schedule <= IB3D_INNER_TAIL) && p->smooth_sweeps >= 0 && p->ramp_sweeps >= 0 &&
         (p->outlet == IB3D_OUTLET_ZERO_GRADIENT || p->outlet == IB3D_OUTLET_CONVECTIVE) &&
         (p->momentum == IB3D_MOMENTUM_EULER || p->momentum == IB3D_MOMENTUM_AB2);
}

// The sweep loop of the context's precision mode.
int run_sor(ib3d_ctx* c, ib3d_solve_stats* st) {
  if (c->prm.precision == IB3D_PREC_FP32DC) return run_sor_fp32dc(c, st);
  if (c->prm.precision == IB3D_PREC_FP64_FAST) return run_sor_fp64_fast(c, st);
  return run_sor_fp64(c, st);
}

int fail(ib3d_ctx* c, int code, const char* msg) {
  if (c) c->err = msg;
  return code;
}

}  // namespace
}  // namespace ib3d

using namespace ib3d;

// FP32 copies of the nine Poisson tables (each padded to 8 floats; off32[3*axis+col]
// is each table's offset) and, for even nx, the x tables regrouped for the
// colour-packed sweep: hp[((s*3 + col)*nq + g)*4 + e] = Acx(i-1, col) at
// i = 2 + s + 8g + 2e (0 beyond the row), columns 1 and 3 (col 0, 2) negated: the
// sweep subtracts their products with fused multiply-adds, fma(-a, x, num).
static void poisson32_host(const ib3d_ctx* c, std::vector<float>& h32, std::vector<size_t>& off32,
                           std::vector<float>& hp) {
  h32.clear(); off32.clear(); hp.clear();
  for (int ax = 0; ax < 3; ++ax)
    for (int q = 0; q < 3; ++q) {
      off32.push_back(h32.size());
      for (double x : c->hac[ax][q]) h32.push_back((float)x);
      while (h32.size() % 8) h32.push_back(0.0f);
    }
  const int nx = c->d.nx;
  if (nx % 2 == 0) {
    const int nq = ((nx >> 1) + 3) >> 2;
    hp.assign((size_t)2 * 3 * nq * 4, 0.0f);
    for (int s = 0; s < 2; ++s)
      for (int q = 0; q < 3; ++q)
        for (int g = 0; g < nq; ++g)
          for (int e = 0; e < 4; ++e) {
            const long long i = 2 + s + 8ll * g + 2 * e;
            if (i <= nx + 1) {
              const float a = (float)c->hac[0][q][i - 1];
              hp[(((size_t)s * 3 + q) * nq + g) * 4 + e] = q == 1 ? a : -a;
            }
          }
    // then the three z coefficients of each plane as one float4 (Grid1D::acz4)
    for (size_t m = 0; m < c->hac[2][0].size(); ++m)
      for (int q = 0; q < 4; ++q) hp.push_back(q < 3 ? (float)c->hac[2][q][m] : 0.0f);
  }
}

static int upload_poisson32(ib3d_ctx* c, const std::vector<float>& h32, const std::vector<float>& hp) {
  if (cudaMemcpy(c->d_tables32, h32.data(), h32.size() * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess)
    return IB3D_ERR_CUDA;
  if (!hp.empty() && cudaMemcpy(c->d_axp, hp.data(), hp.size() * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess)
    return IB3D_ERR_CUDA;
  return IB3D_OK;
}

extern "C" {

void ib3d_default_params(ib3d_params* p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->re = 100.0;
  p->deltat = 0.75e-3;
  p->omega = 1.99;
  p->eps = 1e-5;
  p->max_sweeps = 1000000;
  p->criterion = IB3D_CRIT_UPDATE;
  p->precision = IB3D_PREC_FP64;
  p->warm_start = IB3D_WARM_ZERO;
  p->check_every = 1;
  p->inner_sweeps = 64;
}

const char* ib3d_last_error(const ib3d_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

// resi_u/v/w of nsMomentumAB, allocated (zeroed, subInitialConditions.f90:24) the
// first time the Adams-Bashforth scheme is selected
static int ensure_resi(ib3d_ctx* c, bool need) {
  if (!need || c->resi[0]) return IB3D_OK;
  for (int q = 0; q < 3; ++q) {
    if (cudaMalloc(&c->resi[q], (size_t)c->d.n3 * sizeof(double)) != cudaSuccess)
      return fail(c, IB3D_ERR_MEMORY, "nsMomentumAB residual arrays");
    if (cudaMemsetAsync(c->resi[q], 0, (size_t)c->d.n3 * sizeof(double), c->st) != cudaSuccess)
      return fail(c, IB3D_ERR_CUDA, "nsMomentumAB residual arrays");
  }
  return IB3D_OK;
}

static int zero_resi(ib3d_ctx* c) {
  for (int q = 0; q < 3; ++q)
    if (c->resi[q]) IB3D_CUDA(c, cudaMemsetAsync(c->resi[q], 0, (size_t)c->d.n3 * sizeof(double), c->st));
  return IB3D_OK;
}

int ib3d_set_params(ib3d_ctx* ctx, const ib3d_params* prm) {
  if (!ctx) return IB3D_ERR_ARG;
  if (!valid_params(prm)) return fail(ctx, IB3D_ERR_ARG, "ib3d_set_params: invalid parameters");
  ctx->prm = *prm;
  if (int rc = ensure_resi(ctx, prm->momentum == IB3D_MOMENTUM_AB2)) return rc;
  // the velocity-correction factors depend on deltat: rebuild them
  const double dt = prm->deltat;
  std::vector<double> cx((size_t)ctx->d.nx + 3, 0.0), cy((size_t)ctx->d.ny + 3, 0.0), cz((size_t)ctx->d.nz + 3, 0.0);
  for (int i = 1; i <= ctx->d.nx + 1; ++i) cx[i] = dt / (0.5 * (ctx->hdx[i + 1] + ctx->hdx[i]));
  for (int j = 1; j <= ctx->d.ny + 1; ++j) cy[j] = dt / (0.5 * (ctx->hdy[j + 1] + ctx->hdy[j]));
  for (int k = 1; k <= ctx->d.nz + 1; ++k) cz[k] = dt / (0.5 * (ctx->hdz[k + 1] + ctx->hdz[k]));
  IB3D_CUDA(ctx, cudaMemcpyAsync((void*)ctx->g.corx, cx.data(), cx.size() * sizeof(double), cudaMemcpyHostToDevice, ctx->st));
  IB3D_CUDA(ctx, cudaMemcpyAsync((void*)ctx->g.cory, cy.data(), cy.size() * sizeof(double), cudaMemcpyHostToDevice, ctx->st));
  IB3D_CUDA(ctx, cudaMemcpyAsync((void*)ctx->g.corz, cz.data(), cz.size() * sizeof(double), cudaMemcpyHostToDevice, ctx->st));
  IB3D_CUDA(ctx, cudaStreamSynchronize(ctx->st));
  return IB3D_OK;
}

int ib3d_create(ib3d_ctx** out, const ib3d_params* prm, int64_t nx, int64_t ny, int64_t nz, const double* x1n,
                const double* y1n, const double* z1n) {
  if (!out) return IB3D_ERR_ARG;
  *out = nullptr;
  if (!valid_params(prm) || nx < 4 || ny < 4 || nz < 4 || !x1n || !y1n || !z1n) return IB3D_ERR_ARG;
  if ((nx + 2) * (ny + 2) * (nz + 2) >= (1ll << 31)) return IB3D_ERR_ARG;
  if (nz > 65535) return IB3D_ERR_ARG;   // bounds the FP32 sweep launch's grid z-dimension
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return IB3D_ERR_CUDA;
  ib3d_ctx* c = new ib3d_ctx();
  c->prm = *prm;
  cudaGetDevice(&c->device);
  c->d.nx = (int)nx; c->d.ny = (int)ny; c->d.nz = (int)nz;
  c->d.NX2 = (int)nx + 2; c->d.NY2 = (int)ny + 2; c->d.NZ2 = (int)nz + 2;
  c->d.n3 = (long long)c->d.NX2 * c->d.NY2 * c->d.NZ2;
  if (!axis_tables((int)nx, x1n, c->hx1, c->hdx, c->hxu, c->hxp) ||
      !axis_tables((int)ny, y1n, c->hy1, c->hdy, c->hyv, c->hyp) ||
      !axis_tables((int)nz, z1n, c->hz1, c->hdz, c->hzw, c->hzp)) {
    delete c;
    return IB3D_ERR_ARG;
  }
  // staggered copies (subReadInput.f90:101-129): the u grid is (x1, yp, zp), etc.
  c->hxv = c->hxp; c->hxw = c->hxp;
  c->hyu = c->hyp; c->hyw = c->hyp;
  c->hzu = c->hzp; c->hzv = c->hzp;
  poisson_axis((int)nx, c->hxp, true, c->hac[0]);
  poisson_axis((int)ny, c->hyp, false, c->hac[1]);
  poisson_axis((int)nz, c->hzp, false, c->hac[2]);
  // non_uni_coeff (subNavierStokes.f90:36-595)
  const std::vector<double>* del[3] = {&c->hdx, &c->hdy, &c->hdz};
  const int nn[3] = {(int)nx, (int)ny, (int)nz};
  double cs[12];
  for (int ax = 0; ax < 3; ++ax) {
    const std::vector<double>& dd = *del[ax];
    for (int m = 0; m < 12; ++m) {
      c->hcc[ax][m].assign((size_t)nn[ax] + 3, 0.0);
      c->hcc[3 + ax][m].assign((size_t)nn[ax] + 3, 0.0);
    }
    for (int i = 2; i <= nn[ax]; ++i) {
      conv_station(dd[i] / dd[i - 1], dd[i + 1] / dd[i], dd[i + 2] / dd[i + 1], cs);
      for (int m = 0; m < 12; ++m) c->hcc[ax][m][i] = cs[m];
      const double h1 = (i == 2) ? dd[i - 1] : 0.5 * (dd[i - 1] + dd[i - 2]);
      const double h2 = 0.5 * (dd[i] + dd[i - 1]);
      const double h3 = 0.5 * (dd[i] + dd[i + 1]);
      const double h4 = 0.5 * (dd[i + 1] + dd[i + 2]);
      conv_station(h2 / h1, h3 / h2, h4 / h3, cs);
      for (int m = 0; m < 12; ++m) c->hcc[3 + ax][m][i] = cs[m];
    }
  }
  if (cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return IB3D_ERR_CUDA;
  }
  // pack and upload the FP64 tables
  Packer pk;
  std::vector<double> corx((size_t)nx + 3, 0.0), cory((size_t)ny + 3, 0.0), corz((size_t)nz + 3, 0.0);
  pk.add(c->hx1, &c->g.x1); pk.add(c->hy1, &c->g.y1); pk.add(c->hz1, &c->g.z1);
  pk.add(c->hdx, &c->g.dx); pk.add(c->hdy, &c->g.dy); pk.add(c->hdz, &c->g.dz);
  pk.add(c->hxu, &c->g.xu); pk.add(c->hyu, &c->g.yu); pk.add(c->hzu, &c->g.zu);
  pk.add(c->hxv, &c->g.xv); pk.add(c->hyv, &c->g.yv); pk.add(c->hzv, &c->g.zv);
  pk.add(c->hxw, &c->g.xw); pk.add(c->hyw, &c->g.yw); pk.add(c->hzw, &c->g.zw);
  pk.add(c->hxp, &c->g.xp); pk.add(c->hyp, &c->g.yp); pk.add(c->hzp, &c->g.zp);
  for (int q = 0; q < 3; ++q) {
    pk.add(c->hac[0][q], &c->g.acx[q]);
    pk.add(c->hac[1][q], &c->g.acy[q]);
    pk.add(c->hac[2][q], &c->g.acz[q]);
  }
  for (int f = 0; f < 6; ++f)
    for (int m = 0; m < 12; ++m) pk.add(c->hcc[f][m], &c->g.cc[f][m]);
  pk.add(corx, &c->g.corx); pk.add(cory, &c->g.cory); pk.add(corz, &c->g.corz);
  int rc = IB3D_OK;
  if (cudaMalloc(&c->d_tables, pk.host.size() * sizeof(double)) != cudaSuccess) rc = IB3D_ERR_MEMORY;
  if (!rc && cudaMemcpy(c->d_tables, pk.host.data(), pk.host.size() * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess)
    rc = IB3D_ERR_CUDA;
  if (!rc)
    for (auto& f : pk.fix) *f.first = c->d_tables + f.second;
  // FP32 copies of the Poisson coefficients for the inner solve, and the x
  // coefficients of the colour-packed FP32 sweep grouped by four cells of one colour
  if (!rc) {
    std::vector<float> h32, hp;
    std::vector<size_t> off32;
    poisson32_host(c, h32, off32, hp);
    if (cudaMalloc(&c->d_tables32, h32.size() * sizeof(float)) != cudaSuccess) rc = IB3D_ERR_MEMORY;
    if (!rc && !hp.empty() && cudaMalloc(&c->d_axp, hp.size() * sizeof(float)) != cudaSuccess) rc = IB3D_ERR_MEMORY;
    if (!rc) {
      for (int ax = 0; ax < 3; ++ax)
        for (int q = 0; q < 3; ++q) {
          const float** slot = ax == 0 ? &c->g.acx32[q] : ax == 1 ? &c->g.acy32[q] : &c->g.acz32[q];
          *slot = c->d_tables32 + off32[3 * ax + q];
        }
      if (!hp.empty()) {
        const int nq = (int)(((nx >> 1) + 3) >> 2);
        for (int s = 0; s < 2; ++s)
          for (int q = 0; q < 3; ++q)
            c->g.axp[s][q] = reinterpret_cast<const float4*>(c->d_axp) + ((size_t)s * 3 + q) * nq;
        c->g.acz4 = reinterpret_cast<const float4*>(c->d_axp) + (size_t)6 * nq;
      }
      rc = upload_poisson32(c, h32, hp);
    }
  }
  if (!rc) {
    const int S = (int)std::max(nx, std::max(ny, nz)) + 3;
    std::vector<double> ft((size_t)3 * kFastTables * S, 0.0);
    fast_tables(c->hdx, (int)nx, 0, c->hcc, S, ft);
    fast_tables(c->hdy, (int)ny, 1, c->hcc, S, ft);
    fast_tables(c->hdz, (int)nz, 2, c->hcc, S, ft);
    c->fast_stride = S;
    if (cudaMalloc(&c->d_fast, ft.size() * sizeof(double)) != cudaSuccess) rc = IB3D_ERR_MEMORY;
    if (!rc && cudaMemcpy(c->d_fast, ft.data(), ft.size() * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess)
      rc = IB3D_ERR_CUDA;
  }
  if (!rc) rc = alloc_fields(c);
  if (!rc) rc = ensure_resi(c, prm->momentum == IB3D_MOMENTUM_AB2);
  if (!rc) rc = ib3d_set_params(c, prm);
  if (!rc && cudaStreamSynchronize(c->st) != cudaSuccess) rc = IB3D_ERR_CUDA;
  if (rc) {
    ib3d_destroy(c);
    return rc;
  }
  *out = c;
  return IB3D_OK;
}

void ib3d_destroy(ib3d_ctx* c) {
  if (!c) return;
  if (c->st) cudaStreamSynchronize(c->st);
  timer_fold(c);
  for (cudaEvent_t e : c->pool) cudaEventDestroy(e);
  free_ib(c);
  void* ptrs[] = {c->d_tables, c->d_tables32, c->d_fast, c->d_axp, c->u, c->v, c->w, c->ut, c->vt, c->wt, c->p, c->pc, c->b, c->bdt,
                  c->e32, c->r32, c->ep[0], c->ep[1], c->rp[0], c->rp[1], c->cell, c->ibmap, c->ctl, c->d_nodes, c->d_tri, c->d_surf, c->d_iblist,
                  c->d_nelp, c->d_nd, c->d_minel, c->d_scache, c->d_contrib, c->d_coef, c->d_flag, c->d_scan,
                  c->hist[0], c->hist[1], c->r_hist, c->d_norm, c->d_norm_part, c->resi[0], c->resi[1], c->resi[2],
                  c->wdiag, c->epn[0], c->epn[1], c->d_retag_mask, c->d_retag_list};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (c->h_ctl) cudaFreeHost(c->h_ctl);
  if (c->sweep_exec) cudaGraphExecDestroy(c->sweep_exec);
  for (cudaStream_t x : c->xfer)
    if (x) {
      cudaStreamSynchronize(x);
      cudaStreamDestroy(x);
    }
  if (c->stage) cudaFree(c->stage);
  if (c->xfer_ready) cudaEventDestroy(c->xfer_ready);
  if (c->staged) cudaEventDestroy(c->staged);
  for (cudaEvent_t e : c->xfer_done)
    if (e) cudaEventDestroy(e);
  if (c->st) cudaStreamDestroy(c->st);
  delete c;
}

int ib3d_set_poisson_coefficients(ib3d_ctx* c, const double* acx, const double* acy, const double* acz) {
  if (!c || !acx || !acy || !acz) return IB3D_ERR_ARG;
  const int n[3] = {c->d.nx, c->d.ny, c->d.nz};
  const double* src[3] = {acx, acy, acz};
  for (int ax = 0; ax < 3; ++ax)
    for (int q = 0; q < 3; ++q)
      for (int i = 1; i <= n[ax]; ++i)
        if (!std::isfinite(src[ax][(size_t)q * n[ax] + (i - 1)]))
          return fail(c, IB3D_ERR_ARG, "ib3d_set_poisson_coefficients: non-finite coefficient");
  IB3D_CUDA(c, cudaStreamSynchronize(c->st));
  for (int ax = 0; ax < 3; ++ax)
    for (int q = 0; q < 3; ++q) {
      std::vector<double>& h = c->hac[ax][q];
      for (int i = 1; i <= n[ax]; ++i) h[i] = src[ax][(size_t)q * n[ax] + (i - 1)];   // (n,3) column-major
      const double* dev = ax == 0 ? c->g.acx[q] : ax == 1 ? c->g.acy[q] : c->g.acz[q];
      IB3D_CUDA(c, cudaMemcpy(const_cast<double*>(dev), h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice));
    }
  std::vector<float> h32, hp;
  std::vector<size_t> off32;
  poisson32_host(c, h32, off32, hp);
  return upload_poisson32(c, h32, hp);
}

int ib3d_set_mesh(ib3d_ctx* c, int64_t nnodes, const double* xn, const double* yn, const double* zn, int64_t nelems,
                  const int64_t* e1, const int64_t* e2, const int64_t* e3, double xshift, double yshift,
                  double zshift, int64_t inor) {
  if (!c) return IB3D_ERR_ARG;
  if (nnodes < 3 || nelems < 1 || !xn || !yn || !zn || !e1 || !e2 || !e3 || nnodes > (1ll << 30) ||
      nelems > (1ll << 30))
    return fail(c, IB3D_ERR_ARG, "ib3d_set_mesh: bad sizes or null arrays");
  std::vector<int> tri((size_t)3 * nelems);
  for (int64_t e = 0; e < nelems; ++e) {
    const int64_t v[3] = {e1[e], e2[e], e3[e]};
    for (int q = 0; q < 3; ++q) {
      if (v[q] < 1 || v[q] > nnodes) return fail(c, IB3D_ERR_MESH, "ib3d_set_mesh: triangle node index out of range");
      tri[(size_t)q * nelems + e] = (int)v[q];
    }
  }
  std::vector<double> nodes((size_t)3 * nnodes);
  for (int64_t i = 0; i < nnodes; ++i) {       // shiftSurfaceNodesInitial (subSearch.f90:28-35)
    nodes[i] = xn[i] + xshift;
    nodes[nnodes + i] = yn[i] + yshift;
    nodes[2 * nnodes + i] = zn[i] + zshift;
  }
  cudaFree(c->d_nodes); cudaFree(c->d_tri); cudaFree(c->d_surf); cudaFree(c->d_scache); cudaFree(c->d_contrib);
  c->d_nodes = nullptr; c->d_tri = nullptr; c->d_surf = nullptr; c->d_scache = nullptr; c->d_contrib = nullptr;
  c->nnodes = nnodes; c->nelems = nelems; c->inor = inor;
  IB3D_CUDA(c, cudaMalloc(&c->d_nodes, nodes.size() * sizeof(double)));
  IB3D_CUDA(c, cudaMalloc(&c->d_tri, tri.size() * sizeof(int)));
  IB3D_CUDA(c, cudaMalloc(&c->d_surf, (size_t)9 * nelems * sizeof(double)));
  IB3D_CUDA(c, cudaMalloc(&c->d_scache, (size_t)15 * nelems * sizeof(int)));
  IB3D_CUDA(c, cudaMalloc(&c->d_contrib, (size_t)7 * nelems * sizeof(double)));
  IB3D_CUDA(c, cudaMemcpy(c->d_nodes, nodes.data(), nodes.size() * sizeof(double), cudaMemcpyHostToDevice));
  IB3D_CUDA(c, cudaMemcpy(c->d_tri, tri.data(), tri.size() * sizeof(int), cudaMemcpyHostToDevice));
  int rc = run_surface_norm(c);
  if (rc) return rc;
  std::vector<double> cosv((size_t)3 * nelems);
  IB3D_CUDA(c, cudaMemcpyAsync(cosv.data(), c->d_surf + 3 * nelems, cosv.size() * sizeof(double),
                               cudaMemcpyDeviceToHost, c->st));
  IB3D_CUDA(c, cudaStreamSynchronize(c->st));
  for (double x : cosv)
    if (!std::isfinite(x)) return fail(c, IB3D_ERR_MESH, "ib3d_set_mesh: degenerate triangle (zero area)");
  c->searched = false;
  c->retag_ok = false;
  c->have_scache = false;
  return IB3D_OK;
}

int ib3d_move_body(ib3d_ctx* c, double dx, double dy, double dz, double us, double vs, double ws) {
  if (!c) return IB3D_ERR_ARG;
  if (!c->d_surf) return fail(c, IB3D_ERR_ARG, "ib3d_move_body: call ib3d_set_mesh first");
  const double v[6] = {dx, dy, dz, us, vs, ws};
  for (double x : v)
    if (!std::isfinite(x)) return fail(c, IB3D_ERR_ARG, "ib3d_move_body: non-finite shift or velocity");
  int rc = run_move_body(c, dx, dy, dz);
  if (rc) return rc;
  const double now[3] = {us, vs, ws};
  for (int q = 0; q < 3; ++q) {
    // the first move has no previous velocity: no acceleration term
    c->bprev[q] = c->motion.moving ? c->motion.vel[q] : now[q];
    c->motion.vel[q] = now[q];
  }
  c->motion.moving = 1;
  c->searched = false;     // the flags and ghost points belong to the old position
  c->have_scache = false;  // and so do the drag probes
  return IB3D_OK;
}

int ib3d_search(ib3d_ctx* c, const int64_t box[6], int64_t counts[5]) {
  if (!c || !box) return IB3D_ERR_ARG;
  if (!c->d_surf) return fail(c, IB3D_ERR_ARG, "ib3d_search: call ib3d_set_mesh first");
  const int64_t hi[3] = {c->d.nx + 2, c->d.ny + 2, c->d.nz + 2};
  for (int a = 0; a < 3; ++a)
    if (box[2 * a] < 1 || box[2 * a + 1] > hi[a] || box[2 * a] > box[2 * a + 1])
      return fail(c, IB3D_ERR_ARG, "ib3d_search: search box outside the padded grid");
  for (int q = 0; q < 6; ++q) c->box[q] = box[q];
  c->retag_ok = false;
  int rc = run_search(c);
  if (rc) return rc;
  c->searched = true;
  c->retag_ok = true;
  if (counts)
    for (int q = 0; q < 5; ++q) counts[q] = c->counts[q];
  return IB3D_OK;
}

int ib3d_selective_retag(ib3d_ctx* c, int64_t counts[5]) {
  if (!c) return IB3D_ERR_ARG;
  if (!c->retag_ok || c->nib < 1)
    return fail(c, IB3D_ERR_ARG, "ib3d_selective_retag: needs the IB cells of an earlier search of this mesh");
  c->retag_ok = false;
  int rc = run_selective_retag(c);
  if (rc) return rc;
  c->searched = true;
  c->retag_ok = c->nib > 0;
  if (counts)
    for (int q = 0; q < 5; ++q) counts[q] = c->counts[q];
  return IB3D_OK;
}

int ib3d_get_search(ib3d_ctx* c, int64_t* cell, int64_t* ib_list, int64_t* nelp, double* normdis) {
  if (!c) return IB3D_ERR_ARG;
  if (!c->searched) return fail(c, IB3D_ERR_ARG, "ib3d_get_search: call ib3d_search first");
  const size_t n3 = (size_t)c->d.n3, nib = (size_t)c->nib;
  if (cell) {
    std::vector<unsigned char> h(n3);
    IB3D_CUDA(c, cudaMemcpyAsync(h.data(), c->cell, n3, cudaMemcpyDeviceToHost, c->st));
    IB3D_CUDA(c, cudaStreamSynchronize(c->st));
    for (size_t q = 0; q < n3; ++q) cell[q] = h[q];
  }
  if (nib && (ib_list || nelp)) {
    std::vector<int> h(3 * nib), hn(nib);
    IB3D_CUDA(c, cudaMemcpyAsync(h.data(), c->d_iblist, 3 * nib * sizeof(int), cudaMemcpyDeviceToHost, c->st));
    IB3D_CUDA(c, cudaMemcpyAsync(hn.data(), c->d_nelp, nib * sizeof(int), cudaMemcpyDeviceToHost, c->st));
    IB3D_CUDA(c, cudaStreamSynchronize(c->st));
    if (ib_list)
      for (size_t q = 0; q < 3 * nib; ++q) ib_list[q] = h[q];
    if (nelp)
      for (size_t q = 0; q < nib; ++q) nelp[q] = hn[q];
  }
  if (nib && normdis) {
    IB3D_CUDA(c, cudaMemcpyAsync(normdis, c->d_nd, 7 * nib * sizeof(double), cudaMemcpyDeviceToHost, c->st));
    IB3D_CUDA(c, cudaStreamSynchronize(c->st));
  }
  return IB3D_OK;
}

int ib3d_initial_conditions(ib3d_ctx* c) {
  if (!c) return IB3D_ERR_ARG;
  if (int rc = zero_resi(c)) return rc;   // resi_u = 0 (subInitialConditions.f90:24)
  launch_initial(c);
  IB3D_CUDA(c, cudaGetLastError());
  return IB3D_OK;
}

static double* field_ptr(ib3d_ctx* c, int which) {
  double* f[] = {c->u, c->v, c->w, c->ut, c->vt, c->wt, c->p, c->pc, c->b};
  return (which >= 0 && which < 9) ? f[which] : nullptr;
}

int ib3d_upload_fields(ib3d_ctx* c, const double* u, const double* v, const double* w, const double* p) {
  if (!c) return IB3D_ERR_ARG;
  if (int rc = zero_resi(c)) return rc;   // lastConditions: resi_u = 0 (subLastConditions.f90:16)
  const size_t bytes = (size_t)c->d.n3 * sizeof(double);
  const double* src[3] = {u, v, w};
  double* dst[3] = {c->u, c->v, c->w};
  double* dst2[3] = {c->ut, c->vt, c->wt};
  for (int q = 0; q < 3; ++q) {
    if (!src[q]) continue;
    IB3D_CUDA(c, cudaMemcpyAsync(dst[q], src[q], bytes, cudaMemcpyHostToDevice, c->st));
    IB3D_CUDA(c, cudaMemcpyAsync(dst2[q], dst[q], bytes, cudaMemcpyDeviceToDevice, c->st));
  }
  if (p) IB3D_CUDA(c, cudaMemcpyAsync(c->p, p, bytes, cudaMemcpyHostToDevice, c->st));
  IB3D_CUDA(c, cudaStreamSynchronize(c->st));
  return IB3D_OK;
}

// The transfer streams of the host downloads and their events, created on first use.
static int ensure_xfer(ib3d_ctx* c) {
  if (c->xfer_ready) return IB3D_OK;
  IB3D_CUDA(c, cudaEventCreateWithFlags(&c->xfer_ready, cudaEventDisableTiming));
  IB3D_CUDA(c, cudaEventCreateWithFlags(&c->staged, cudaEventDisableTiming));
  for (auto& e : c->xfer_done) IB3D_CUDA(c, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  for (auto& x : c->xfer) IB3D_CUDA(c, cudaStreamCreateWithFlags(&x, cudaStreamNonBlocking));
  return IB3D_OK;
}

int ib3d_download_fields(ib3d_ctx* c, double* u, double* v, double* w, double* ut, double* vt, double* wt,
                         double* p) {
  if (!c) return IB3D_ERR_ARG;
  const size_t bytes = (size_t)c->d.n3 * sizeof(double);
  double* dst[7] = {u, v, w, ut, vt, wt, p};
  const double* src[7] = {c->u, c->v, c->w, c->ut, c->vt, c->wt, c->p};
  // the copies go round-robin over the context's stream and three more, which start
  // once the work queued on the context's stream is done, so that several copy engines
  // share the host link; the call returns when all of them have landed
  int rc = ensure_xfer(c);
  if (rc) return rc;
  IB3D_CUDA(c, cudaEventRecord(c->xfer_ready, c->st));
  for (auto& x : c->xfer) IB3D_CUDA(c, cudaStreamWaitEvent(x, c->xfer_ready, 0));
  int n = 0;
  for (int q = 0; q < 7; ++q)
    if (dst[q]) {
      cudaStream_t s = n % 4 == 0 ? c->st : c->xfer[n % 4 - 1];
      IB3D_CUDA(c, cudaMemcpyAsync(dst[q], src[q], bytes, cudaMemcpyDeviceToHost, s));
      ++n;
    }
  IB3D_CUDA(c, cudaStreamSynchronize(c->st));
  for (auto& x : c->xfer) IB3D_CUDA(c, cudaStreamSynchronize(x));
  c->async_pending = false;
  return IB3D_OK;
}

int ib3d_download_fields_async(ib3d_ctx* c, double* u, double* v, double* w, double* ut, double* vt, double* wt,
                               double* p) {
  if (!c) return IB3D_ERR_ARG;
  const size_t n3 = (size_t)c->d.n3, bytes = n3 * sizeof(double);
  double* dst[7] = {u, v, w, ut, vt, wt, p};
  const double* src[7] = {c->u, c->v, c->w, c->ut, c->vt, c->wt, c->p};
  int rc = ensure_xfer(c);
  if (rc) return rc;
  if (!c->stage && cudaMalloc(&c->stage, 7 * bytes) != cudaSuccess) {
    cudaGetLastError();
    return fail(c, IB3D_ERR_MEMORY, "ib3d_download_fields_async: no device memory for the snapshot");
  }
  // the snapshot may be overwritten only once the previous call's host copies have read it
  if (c->async_pending)
    for (auto& e : c->xfer_done) IB3D_CUDA(c, cudaStreamWaitEvent(c->st, e, 0));
  for (int q = 0; q < 7; ++q)
    if (dst[q]) IB3D_CUDA(c, cudaMemcpyAsync(c->stage + q * n3, src[q], bytes, cudaMemcpyDeviceToDevice, c->st));
  IB3D_CUDA(c, cudaEventRecord(c->staged, c->st));
  int n = 0;
  for (int q = 0; q < 7; ++q)
    if (dst[q]) {
      cudaStream_t x = c->xfer[n % 3];
      if (n < 3) IB3D_CUDA(c, cudaStreamWaitEvent(x, c->staged, 0));
      IB3D_CUDA(c, cudaMemcpyAsync(dst[q], c->stage + q * n3, bytes, cudaMemcpyDeviceToHost, x));
      ++n;
    }
  for (int i = 0; i < 3; ++i) IB3D_CUDA(c, cudaEventRecord(c->xfer_done[i], c->xfer[i]));
  c->async_pending = true;
  return IB3D_OK;
}

int ib3d_download_wait(ib3d_ctx* c) {
  if (!c) return IB3D_ERR_ARG;
  if (!c->async_pending) return IB3D_OK;
  for (auto& e : c->xfer_done) IB3D_CUDA(c, cudaEventSynchronize(e));
  c->async_pending = false;
  return IB3D_OK;
}

int ib3d_get_field(ib3d_ctx* c, int which, double* out) {
  if (!c || !out) return IB3D_ERR_ARG;
  double* f = field_ptr(c, which);
  if (!f) return fail(c, IB3D_ERR_ARG, "ib3d_get_field: unknown field");
  IB3D_CUDA(c, cudaMemcpyAsync(out, f, (size_t)c->d.n3 * sizeof(double), cudaMemcpyDeviceToHost, c->st));
  IB3D_CUDA(c, cudaStreamSynchronize(c->st));
  return IB3D_OK;
}

int ib3d_set_field(ib3d_ctx* c, int which, const double* in) {
  if (!c || !in) return IB3D_ERR_ARG;
  double* f = field_ptr(c, which);
  if (!f) return fail(c, IB3D_ERR_ARG, "ib3d_set_field: unknown field");
  IB3D_CUDA(c, cudaMemcpyAsync(f, in, (size_t)c->d.n3 * sizeof(double), cudaMemcpyHostToDevice, c->st));
  IB3D_CUDA(c, cudaStreamSynchronize(c->st));
  return IB3D_OK;
}

void* ib3d_device_field(ib3d_ctx* c, int which) { return c ? (void*)field_ptr(c, which) : nullptr; }

void* ib3d_stream(ib3d_ctx* c) { return c ? (void*)c->st : nullptr; }

int ib3d_timers_enable(ib3d_ctx* c, int on) {
  if (!c) return IB3D_ERR_ARG;
  timer_fold(c);
  if (on) {
    for (double& x : c->tms) x = 0.0;
    c->t_sweeps64 = c->t_sweeps32 = c->t_outer = c->t_steps = c->t_launches32 = 0;
    c->launches = 0;
  }
  c->timing = on != 0;
  return IB3D_OK;
}

int ib3d_timers_read(ib3d_ctx* c, ib3d_timers* out) {
  if (!c || !out) return IB3D_ERR_ARG;
  timer_fold(c);
  IB3D_CUDA(c, cudaStreamSynchronize(c->st));
  for (int q = 0; q < 10; ++q) out->ms[q] = c->tms[q];
  out->sweeps64 = c->t_sweeps64;
  out->sweeps32 = c->t_sweeps32;
  out->outer = c->t_outer;
  out->launches = c->launches;
  out->launches32 = c->t_launches32;
  out->steps = c->t_steps;
  return IB3D_OK;
}

int ib3d_synchronize(ib3d_ctx* c) {
  if (!c) return IB3D_ERR_ARG;
  IB3D_CUDA(c, cudaStreamSynchronize(c->st));
  return IB3D_OK;
}

int ib3d_ns_momentum(ib3d_ctx* c) {
  if (!c) return IB3D_ERR_ARG;
  if (c->prm.precision != IB3D_PREC_FP64) launch_momentum_fast(c, false);
  else launch_momentum(c, false);
  IB3D_CUDA(c, cudaGetLastError());
  return IB3D_OK;
}

int ib3d_ns_momentum_ab(ib3d_ctx* c) {
  if (!c) return IB3D_ERR_ARG;
  if (int rc = ensure_resi(c, true)) return rc;
  if (c->prm.precision != IB3D_PREC_FP64) launch_momentum_fast(c, true);
  else launch_momentum(c, true);
  IB3D_CUDA(c, cudaGetLastError());
  return IB3D_OK;
}

int ib3d_calculate_uc(ib3d_ctx* c, double* uc) {
  if (!c) return IB3D_ERR_ARG;
  launch_calculate_uc(c);
  IB3D_CUDA(c, cudaGetLastError());
  if (uc) {
    IB3D_CUDA(c, cudaMemcpyAsync(uc, c->d_coef + 6, sizeof(double), cudaMemcpyDeviceToHost, c->st));
    IB3D_CUDA(c, cudaStreamSynchronize(c->st));
  }
  return IB3D_OK;
}

int ib3d_velocity_bc(ib3d_ctx* c) {
  if (!c) return IB3D_ERR_ARG;
  launch_velocity_bc(c);
  IB3D_CUDA(c, cudaGetLastError());
  return IB3D_OK;
}

int ib3d_solid_cell_bc(ib3d_ctx* c) {
  if (!c) return IB3D_ERR_ARG;
  launch_solid_bc(c);
  IB3D_CUDA(c, cudaGetLastError());
  return IB3D_OK;
}

int ib3d_velocity_forcing(ib3d_ctx* c) {
  if (!c) return IB3D_ERR_ARG;
  if (!c->searched) return fail(c, IB3D_ERR_ARG, "ib3d_velocity_forcing: call ib3d_search first");
  return run_velocity_forcing(c);
}

int ib3d_pressure_forcing(ib3d_ctx* c) {
  if (!c) return IB3D_ERR_ARG;
  if (!c->searched) return fail(c, IB3D_ERR_ARG, "ib3d_pressure_forcing: call ib3d_search first");
  return run_pressure_forcing(c);
}

int ib3d_enable_history(ib3d_ctx* c) {
  if (!c) return IB3D_ERR_ARG;
  for (int q = 0; q < 2; ++q)
    if (!c->hist[q]) {
      IB3D_CUDA(c, cudaMalloc(&c->hist[q], (size_t)c->d.n3 * sizeof(double)));
      IB3D_CUDA(c, cudaMemsetAsync(c->hist[q], 0, (size_t)c->d.n3 * sizeof(double), c->st));
    }
  if (!c->r_hist) {
    IB3D_CUDA(c, cudaMalloc(&c->r_hist, (size_t)c->d.n3 * sizeof(float)));
    IB3D_CUDA(c, cudaMemsetAsync(c->r_hist, 0, (size_t)c->d.n3 * sizeof(float), c->st));
  }
  if (!c->d_norm) {
    IB3D_CUDA(c, cudaMalloc(&c->d_norm, sizeof(NetNorm)));
    IB3D_CUDA(c, cudaMemsetAsync(c->d_norm, 0, sizeof(NetNorm), c->st));   // valid = 0
    IB3D_CUDA(c, cudaMalloc(&c->d_norm_part, (size_t)net_norm_blocks(c) * 5 * sizeof(double)));
  }
  c->hist_valid = 0;
  return IB3D_OK;
}

int ib3d_poisson_solver(ib3d_ctx* c, ib3d_solve_stats* stats) {
  if (!c) return IB3D_ERR_ARG;
  ib3d_solve_stats st{};
  if (c->hist[0]) {   // p still holds p^{n-1}: keep it and the one before
    double* t = c->hist[1];
    c->hist[1] = c->hist[0];
    c->hist[0] = t;
    IB3D_CUDA(c, cudaMemcpyAsync(c->hist[0], c->p, (size_t)c->d.n3 * sizeof(double), cudaMemcpyDeviceToDevice, c->st));
    c->hist_valid = std::min(c->hist_valid + 1, 2);
  }
  unsigned long long* red = reinterpret_cast<unsigned long long*>(c->d_coef + 4);  // divmax, derrStdSt
  IB3D_CUDA(c, cudaMemsetAsync(red, 0, 2 * sizeof(unsigned long long), c->st));
  // divergence writes its max into ctl->aux; copy it aside before the SOR resets ctl
  IB3D_CUDA(c, cudaMemsetAsync(c->ctl, 0, sizeof(SolveCtl), c->st));
  if (c->prm.precision != IB3D_PREC_FP64) launch_divergence_fast(c, c->prm.warm_start == IB3D_WARM_ZERO);
  else launch_divergence(c, c->prm.warm_start == IB3D_WARM_ZERO);
  if (c->r_hist) {
    PhaseScope ps(c, PH_NET);
    net_hist_residual(c);   // the current guess's residual: a network input and a capture input
  }
  if (c->prm.warm_start == IB3D_WARM_LEARNED) {
    PhaseScope ps(c, PH_NET);
    net_predict_pc(c);   // until two previous pressures exist, pc keeps the previous step's value
  }
  IB3D_CUDA(c, cudaMemcpyAsync(red, &c->ctl->aux, sizeof(unsigned long long), cudaMemcpyDeviceToDevice, c->st));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, c->st);
  int rc = run_sor(c, &st);
  cudaEventRecord(e1, c->st);
  if (rc == IB3D_OK || rc == IB3D_ERR_NOCONV) {
    launch_correct(c);
    launch_velocity_bc(c);
    IB3D_CUDA(c, cudaMemsetAsync(&c->ctl->aux, 0, sizeof(unsigned long long), c->st));
    launch_dss_copy(c);
    IB3D_CUDA(c, cudaMemcpyAsync(red + 1, &c->ctl->aux, sizeof(unsigned long long), cudaMemcpyDeviceToDevice, c->st));
    unsigned long long h[2];
    IB3D_CUDA(c, cudaMemcpyAsync(h, red, sizeof(h), cudaMemcpyDeviceToHost, c->st));
    IB3D_CUDA(c, cudaStreamSynchronize(c->st));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    st.solve_seconds = ms * 1e-3;
    std::memcpy(&st.divmax, &h[0], sizeof(double));
    double dmax = 0.0;   // max |ut-u| over the fluid cells (k_dss_copy)
    std::memcpy(&dmax, &h[1], sizeof(double));
    st.derr_std_st = dmax / c->prm.deltat;
    if (c->prm.warm_start == IB3D_WARM_LEARNED) net_note_failure(c);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (stats) *stats = st;
  if (rc == IB3D_ERR_NOCONV) c->err = "ib3d_poisson_solver: SOR reached max_sweeps";
  if (rc == IB3D_ERR_NONFINITE) c->err = "ib3d_poisson_solver: non-finite SOR error measure";
  if (rc == IB3D_OK && (!std::isfinite(st.divmax) || !std::isfinite(st.derr_std_st))) {
    c->err = "ib3d_poisson_solver: non-finite divergence or steady-state indicator";
    return IB3D_ERR_NONFINITE;
  }
  return rc;
}

int ib3d_redblack_sor(ib3d_ctx* c, ib3d_solve_stats* stats) {
  if (!c) return IB3D_ERR_ARG;
  ib3d_solve_stats st{};
  IB3D_CUDA(c, cudaMemsetAsync(c->ctl, 0, sizeof(SolveCtl), c->st));
  launch_bdt(c, c->prm.warm_start == IB3D_WARM_ZERO);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, c->st);
  const int rc = run_sor(c, &st);
  cudaEventRecord(e1, c->st);
  const cudaError_t ce = cudaStreamSynchronize(c->st);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (ce != cudaSuccess) return fail(c, IB3D_ERR_CUDA, cudaGetErrorString(ce));
  st.solve_seconds = ms * 1e-3;
  if (stats) *stats = st;
  if (rc == IB3D_ERR_NOCONV) c->err = "ib3d_redblack_sor: SOR reached max_sweeps";
  if (rc == IB3D_ERR_NONFINITE) c->err = "ib3d_redblack_sor: non-finite SOR error measure";
  return rc;
}

int ib3d_stress(ib3d_ctx* c, int first, double coef[4]) {
  if (!c) return IB3D_ERR_ARG;
  if (!c->searched) return fail(c, IB3D_ERR_ARG, "ib3d_stress: call ib3d_search first");
  return run_stress(c, first, coef);
}

int ib3d_step(ib3d_ctx* c, int first, ib3d_solve_stats* stats, double coef[4]) {
  if (!c) return IB3D_ERR_ARG;
  if (!c->searched) return fail(c, IB3D_ERR_ARG, "ib3d_step: call ib3d_search first");
  int rc;
  c->t_steps += 1;
  if (c->prm.momentum == IB3D_MOMENTUM_AB2 && !first) {
    if ((rc = ib3d_ns_momentum_ab(c))) return rc;   // main.f90:45 (nsMomentumAB)
  } else if ((rc = ib3d_ns_momentum(c))) {         // main.f90:46 (30 on the first step)
    return rc;
  }
  if ((rc = ib3d_velocity_bc(c))) return rc;        // :47
  if ((rc = ib3d_solid_cell_bc(c))) return rc;      // :48
  if ((rc = ib3d_velocity_forcing(c))) return rc;   // :49
  if ((rc = ib3d_velocity_bc(c))) return rc;        // :50
  const int prc = ib3d_poisson_solver(c, stats);    // :51
  if (prc && prc != IB3D_ERR_NOCONV) return prc;
  if ((rc = ib3d_pressure_forcing(c))) return rc;   // :52
  if (c->prm.outlet == IB3D_OUTLET_CONVECTIVE)      // the calculateUc hook, :53-54
    if ((rc = ib3d_calculate_uc(c, nullptr))) return rc;
  if ((rc = ib3d_stress(c, first, coef))) return rc;  // :64 (stressCal1 at :39)
  return prc;
}

}  // extern "C"
