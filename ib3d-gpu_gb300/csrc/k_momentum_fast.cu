// Momentum predictor, fast FP64 form (used with IB3D_PREC_FP32DC).
//
// Same discretisation as k_momentum (nsMomentum, subNavierStokes.f90:622-1122),
// but every quotient whose divisor depends only on the grid is read from a 1-D
// table of reciprocals and weights built once on the host, and multiply-adds may
// contract (this file is compiled with -fmad=true). There is no division left in
// the kernel; results differ from the reference arithmetic by rounding only
// (~1e-16 relative per operation). The FP64 path (IB3D_PREC_FP64) keeps the
// bit-identical kernel.
//
// Table layout (built by build_fast_tables in ib3d_api.cu): ft[(axis*kFT + t)*S + m],
// m the 1-based cell index along the axis, S the table stride. Per axis, with d the
// spacings, "node" the component's own axis and "half" a transverse axis:
//   0 w     d[m+1]/(d[m]+d[m+1])                 interpolation weight (dxr/dx2xr)
//   1 ran   1/(ca6_own[m]*d[m+1])   2 rkn 1/(2*ck6_own[m]*d[m])
//   3 rah   1/(ca6_half[m]*0.5(d[m]+d[m+1]))     4 rkh 1/(2*ck6_half[m]*0.5(d[m]+d[m-1]))
//   5..12   first-order node: c1,c2,c3,d1,d2,d3, 1/dA, 1/(2dA) (r = d[m]/d[m+1], dA = d[m+1])
//   13..20  first-order half: same with r = 0.5(d[m]+d[m-1])/(0.5(d[m]+d[m+1])), dA = 0.5(d[m]+d[m+1])
//   21 cna  2/((d[m]+d[m+1]) d[m+1])   22 cnb 2/((d[m]+d[m+1]) d[m])       node diffusion
//   23 cha  2/(0.5(2d[m]+d[m+1]+d[m-1]) 0.5(d[m]+d[m+1]))  24 chb  .../0.5(d[m]+d[m-1])  half diffusion
//   25 rd   1/d[m]                                reciprocal spacing (divergence, k_fast.cu)
//   26..30  third-order upwind of the own-axis family for adv >= 0: ca[q]*ran + ck[q]*rkn, q = 0..4
//   31..35  the same for adv < 0: ca[q]*ran - ck[q]*rkn
//   36..45  the same for the transverse family with rah, rkh
#include "ib3d_internal.cuh"

namespace ib3d {

namespace {

struct Ft {
  const double* t;
  int S;
  __device__ __forceinline__ double operator()(int axis, int tab, int m) const {
    return t[(axis * kFastTables + tab) * S + m];
  }
};

// third-order upwind: adv * ca.q * ra + |adv| * ck.q * rk = adv * (ca*ra +- ck*rk).q, the
// folded coefficients read from the tables of adv's sign (OWN: the component's own
// axis, else a transverse one)
template <bool OWN>
__device__ __forceinline__ double up3f(const Ft& F, int axis, int m, double adv, double q2, double q1, double q0,
                                       double qm1, double qm2) {
  const int b = (OWN ? 26 : 36) + (adv < 0.0 ? 5 : 0);
  const double s = fma(F(axis, b + 4, m), qm2,
                       fma(F(axis, b + 3, m), qm1, fma(F(axis, b + 2, m), q0, fma(F(axis, b + 1, m), q1, F(axis, b, m) * q2))));
  return adv * s;
}

// first-order upwind; base = 5 (node) or 13 (half)
__device__ __forceinline__ double up1f(const Ft& F, int axis, int base, int m, double adv, double qm, double q0,
                                       double qp) {
  const double c1 = F(axis, base + 0, m), c2 = F(axis, base + 1, m), c3 = F(axis, base + 2, m);
  const double d1 = F(axis, base + 3, m), d2 = F(axis, base + 4, m), d3 = F(axis, base + 5, m);
  const double rA = F(axis, base + 6, m), rA2 = F(axis, base + 7, m);
  const double t1 = adv * rA * fma(c3, qp, fma(c1, qm, -c2 * q0));
  const double t2 = fabs(adv) * rA2 * fma(d3, qp, fma(d1, qm, -d2 * q0));
  return t1 - t2;
}

}  // namespace

__global__ void __launch_bounds__(128) k_momentum_fast(Dims d, Grid1D g, const double* __restrict__ ftab, int S,
                                                       const double* __restrict__ U, const double* __restrict__ V,
                                                       const double* __restrict__ W, const double* __restrict__ P,
                                                       const unsigned char* __restrict__ C, double* __restrict__ UT,
                                                       double* __restrict__ VT, double* __restrict__ WT, double rev,
                                                       double deltat, double* __restrict__ RU,
                                                       double* __restrict__ RV, double* __restrict__ RW, int ab2) {
  const unsigned tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= (unsigned)d.nx * (unsigned)d.ny * (unsigned)d.nz) return;
  const int i = (int)(tid % (unsigned)d.nx) + 2;
  const unsigned t = tid / (unsigned)d.nx;
  const int j = (int)(t % (unsigned)d.ny) + 2, k = (int)(t / (unsigned)d.ny) + 2;
  const long long o = d.at(i, j, k);
  if (C[o] != 0) return;
  const Ft F{ftab, S};
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const long long sx = 1, sy = d.NX2, sz = (long long)d.NX2 * d.NY2;
  const bool noib = C[o + sx] != 2 && C[o - sx] != 2 && C[o + sy] != 2 && C[o - sy] != 2 && C[o + sz] != 2 &&
                    C[o - sz] != 2;
  const double u0 = U[o], v0 = V[o], w0 = W[o], p0 = P[o];
  const int m3[3] = {i, j, k};

  // ---- u: own axis x
  {
    const double wx = F(0, 0, i);
    const double vin = 0.5 * (fma(wx, V[o] - V[o + sx], V[o + sx]) + fma(wx, V[o - sy] - V[o + sx - sy], V[o + sx - sy]));
    const double win = 0.5 * (fma(wx, W[o] - W[o + sx], W[o + sx]) + fma(wx, W[o - sz] - W[o + sx - sz], W[o + sx - sz]));
    double cx, cy, cz;
    if (i != 2 && i < nx && j != 2 && j < ny + 1 && k != 2 && k < nz + 1 && noib) {
      cx = up3f<true>(F, 0, i, u0, U[o + 2 * sx], U[o + sx], u0, U[o - sx], U[o - 2 * sx]);
      cy = up3f<false>(F, 1, j, vin, U[o + 2 * sy], U[o + sy], u0, U[o - sy], U[o - 2 * sy]);
      cz = up3f<false>(F, 2, k, win, U[o + 2 * sz], U[o + sz], u0, U[o - sz], U[o - 2 * sz]);
    } else {
      cx = up1f(F, 0, 5, i, u0, U[o - sx], u0, U[o + sx]);
      cy = up1f(F, 1, 13, j, vin, U[o - sy], u0, U[o + sy]);
      cz = up1f(F, 2, 13, k, win, U[o - sz], u0, U[o + sz]);
    }
    const double d2 = F(0, 22, i) * (U[o - sx] - u0) - F(0, 21, i) * (u0 - U[o + sx]) +
                      F(1, 24, j) * (U[o - sy] - u0) - F(1, 23, j) * (u0 - U[o + sy]) +
                      F(2, 24, k) * (U[o - sz] - u0) - F(2, 23, k) * (u0 - U[o + sz]);
    const double resid = fma(rev, d2, -cx - cy - cz);
    const double rhs = ab2 ? 0.5 * (3.0 * resid - RU[o]) : resid;   // nsMomentumAB or nsMomentum
    UT[o] = fma(deltat, rhs, u0) + g.corx[i] * (p0 - P[o + sx]);
    if (RU) RU[o] = resid;
  }
  // ---- v: own axis y
  {
    const double wy = F(1, 0, j);
    const double uin = 0.5 * (fma(wy, U[o] - U[o + sy], U[o + sy]) + fma(wy, U[o - sx] - U[o - sx + sy], U[o - sx + sy]));
    const double win = 0.5 * (fma(wy, W[o] - W[o + sy], W[o + sy]) + fma(wy, W[o - sz] - W[o + sy - sz], W[o + sy - sz]));
    double cx, cy, cz;
    if (i != 2 && i < nx + 1 && j != 2 && j < ny && k != 2 && k < nz + 1 && noib) {
      cx = up3f<false>(F, 0, i, uin, V[o + 2 * sx], V[o + sx], v0, V[o - sx], V[o - 2 * sx]);
      cy = up3f<true>(F, 1, j, v0, V[o + 2 * sy], V[o + sy], v0, V[o - sy], V[o - 2 * sy]);
      cz = up3f<false>(F, 2, k, win, V[o + 2 * sz], V[o + sz], v0, V[o - sz], V[o - 2 * sz]);
    } else {
      cx = up1f(F, 0, 13, i, uin, V[o - sx], v0, V[o + sx]);
      cy = up1f(F, 1, 5, j, v0, V[o - sy], v0, V[o + sy]);
      cz = up1f(F, 2, 13, k, win, V[o - sz], v0, V[o + sz]);
    }
    const double d2 = F(0, 24, i) * (V[o - sx] - v0) - F(0, 23, i) * (v0 - V[o + sx]) +
                      F(1, 22, j) * (V[o - sy] - v0) - F(1, 21, j) * (v0 - V[o + sy]) +
                      F(2, 24, k) * (V[o - sz] - v0) - F(2, 23, k) * (v0 - V[o + sz]);
    const double resid = fma(rev, d2, -cx - cy - cz);
    const double rhs = ab2 ? 0.5 * (3.0 * resid - RV[o]) : resid;   // nsMomentumAB or nsMomentum
    VT[o] = fma(deltat, rhs, v0) + g.cory[j] * (p0 - P[o + sy]);
    if (RV) RV[o] = resid;
  }
  // ---- w: own axis z
  {
    const double wz = F(2, 0, k);
    const double uin = 0.5 * (fma(wz, U[o] - U[o + sz], U[o + sz]) + fma(wz, U[o - sx] - U[o - sx + sz], U[o - sx + sz]));
    const double vin = 0.5 * (fma(wz, V[o] - V[o + sz], V[o + sz]) + fma(wz, V[o - sy] - V[o - sy + sz], V[o - sy + sz]));
    double cx, cy, cz;
    if (i != 2 && i < nx + 1 && j != 2 && j < ny + 1 && k != 2 && k < nz && noib) {
      cx = up3f<false>(F, 0, i, uin, W[o + 2 * sx], W[o + sx], w0, W[o - sx], W[o - 2 * sx]);
      cy = up3f<false>(F, 1, j, vin, W[o + 2 * sy], W[o + sy], w0, W[o - sy], W[o - 2 * sy]);
      cz = up3f<true>(F, 2, k, w0, W[o + 2 * sz], W[o + sz], w0, W[o - sz], W[o - 2 * sz]);
    } else {
      cx = up1f(F, 0, 13, i, uin, W[o - sx], w0, W[o + sx]);
      cy = up1f(F, 1, 13, j, vin, W[o - sy], w0, W[o + sy]);
      cz = up1f(F, 2, 5, k, w0, W[o - sz], w0, W[o + sz]);
    }
    const double d2 = F(0, 24, i) * (W[o - sx] - w0) - F(0, 23, i) * (w0 - W[o + sx]) +
                      F(1, 24, j) * (W[o - sy] - w0) - F(1, 23, j) * (w0 - W[o + sy]) +
                      F(2, 22, k) * (W[o - sz] - w0) - F(2, 21, k) * (w0 - W[o + sz]);
    const double resid = fma(rev, d2, -cx - cy - cz);
    const double rhs = ab2 ? 0.5 * (3.0 * resid - RW[o]) : resid;   // nsMomentumAB or nsMomentum
    WT[o] = fma(deltat, rhs, w0) + g.corz[k] * (p0 - P[o + sz]);
    if (RW) RW[o] = resid;
  }
  (void)m3;
}

void launch_momentum_fast(ib3d_ctx* c, bool ab2) {
  PhaseScope ps(c, PH_MOMENTUM);
  c->launches += 1;
  const long long n = (long long)c->d.nx * c->d.ny * c->d.nz;
  k_momentum_fast<<<(unsigned)((n + 127) / 128), 128, 0, c->st>>>(c->d, c->g, c->d_fast, c->fast_stride, c->u, c->v,
                                                                   c->w, c->p, c->cell, c->ut, c->vt, c->wt,
                                                                   1.0 / c->prm.re, c->prm.deltat, c->resi[0],
                                                                   c->resi[1], c->resi[2], ab2 ? 1 : 0);
}

}  // namespace ib3d
