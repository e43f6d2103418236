// Momentum predictor: nsMomentum (subNavierStokes.f90:622-1122).
//
// One thread per interior cell of the padded grid; non-fluid cells return at once
// (the reference gathers fluid cells through fluidIndexPtr instead). Per fluid cell:
// staggered transverse-velocity interpolation, third-order upwind convection on
// non-uniform spacing away from walls and immersed-boundary neighbours (else the
// first-order form), second-order diffusion and the explicit pressure gradient,
// then ut = u + dt*(resid + dp/dx) for each component.
//
// Compiled with -fmad=false; each expression keeps the reference's left-to-right
// evaluation so that results are bit-identical to the FP64 oracle.
#include "ib3d_internal.cuh"

namespace ib3d {

namespace {

// Third-order upwind term (subNavierStokes.f90:812-817 and analogues):
// adv*(sum ca*q)/(ca6*dA) + |adv|*(sum ck*q)/(2*ck6*dK). FAM selects the table
// family at compile time so the table pointers stay in the parameter bank.
template <int FAM>
__device__ __forceinline__ double up3(const Grid1D& g, double adv, int m, double q2, double q1, double q0,
                                      double qm1, double qm2, double dA, double dK) {
  const double* const* c = g.cc[FAM];
  const double sa = (((c[0][m] * q2 + c[1][m] * q1) + c[2][m] * q0) + c[3][m] * qm1) + c[4][m] * qm2;
  const double sk = (((c[6][m] * q2 + c[7][m] * q1) + c[8][m] * q0) + c[9][m] * qm1) + c[10][m] * qm2;
  return (adv * sa) / (c[5][m] * dA) + (fabs(adv) * sk) / (2.0 * c[11][m] * dK);
}

// First-order upwind term (subNavierStokes.f90:847-852 and analogues), al = 1.
__device__ __forceinline__ double up1(double adv, double dA, double r, double qm, double q0, double qp) {
  const double t1 = (adv / dA) * (((-1.0 / (r * (r + 1.0))) * qm - (1.0 - 1.0 / r) * q0) + (r / (r + 1.0)) * qp);
  const double t2 = 1.0 * fabs(adv) * (1.0 / (2.0 * dA)) *
                    ((2.0 / (r * (r + 1.0)) * qm - 2.0 / r * q0) + 2.0 / (r + 1.0) * qp);
  return t1 - t2;
}

}  // namespace

__global__ void __launch_bounds__(128) k_momentum(Dims d, Grid1D g, const double* __restrict__ U,
                                                  const double* __restrict__ V, const double* __restrict__ W,
                                                  const double* __restrict__ P,
                                                  const unsigned char* __restrict__ C, double* __restrict__ UT,
                                                  double* __restrict__ VT, double* __restrict__ WT, double rev,
                                                  double deltat, double* __restrict__ RU, double* __restrict__ RV,
                                                  double* __restrict__ RW, int ab2) {
  const unsigned tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= (unsigned)d.nx * (unsigned)d.ny * (unsigned)d.nz) return;
  const int i = (int)(tid % (unsigned)d.nx) + 2;
  const unsigned t = tid / (unsigned)d.nx;
  const int j = (int)(t % (unsigned)d.ny) + 2, k = (int)(t / (unsigned)d.ny) + 2;
  const long long o = d.at(i, j, k);
  if (C[o] != 0) return;
  const int nx = d.nx, ny = d.ny, nz = d.nz;
  const long long sx = 1, sy = d.NX2, sz = (long long)d.NX2 * d.NY2;
  const double* DX = g.dx;
  const double* DY = g.dy;
  const double* DZ = g.dz;
  const double dxr = DX[i + 1], dx = DX[i], dxl = DX[i - 1];
  const double dye = DY[j + 1], dy = DY[j], dyw = DY[j - 1];
  const double dzt = DZ[k + 1], dz = DZ[k], dzb = DZ[k - 1];
  const double u0 = U[o], v0 = V[o], w0 = W[o];
  const double u22 = U[o - sx] - u0, u4 = u0 - U[o + sx];
  const double u6 = U[o - sy] - u0, u8 = u0 - U[o + sy];
  const double u10 = U[o - sz] - u0, u12 = u0 - U[o + sz];
  const double v4 = V[o - sx] - v0, v6 = v0 - V[o + sx];
  const double v8 = V[o - sy] - v0, v10 = v0 - V[o + sy];
  const double v12 = V[o - sz] - v0, v14 = v0 - V[o + sz];
  const double w6 = W[o - sx] - w0, w8 = w0 - W[o + sx];
  const double w10 = W[o - sy] - w0, w12 = w0 - W[o + sy];
  const double w14 = W[o - sz] - w0, w16 = w0 - W[o + sz];
  const double p0 = P[o];
  const double dpdx = (p0 - P[o + sx]) / (0.5 * (dxr + dx));   // :779-781
  const double dpdy = (p0 - P[o + sy]) / (0.5 * (dye + dy));
  const double dpdz = (p0 - P[o + sz]) / (0.5 * (dzt + dz));
  const double dx2xr = dx + dxr, dx2xl = dx + dxl, dy2ye = dy + dye, dy2yw = dy + dyw;
  const double dz2zt = dz + dzt, dz2zb = dz + dzb;
  const bool noib = C[o + sx] != 2 && C[o - sx] != 2 && C[o + sy] != 2 && C[o - sy] != 2 && C[o + sz] != 2 &&
                    C[o - sz] != 2;
  const double ddx = 0.5 * (DX[i] + DX[i - 1]), ddxr = 0.5 * (DX[i] + DX[i + 1]);
  const double ddy = 0.5 * (DY[j] + DY[j - 1]), ddye = 0.5 * (DY[j] + DY[j + 1]);
  const double ddz = 0.5 * (DZ[k] + DZ[k - 1]), ddzr = 0.5 * (DZ[k] + DZ[k + 1]);
  double cx, cy, cz;

  // ---- u momentum (:792-897)
  {
    const double vu_e = V[o + sx] + (dxr / dx2xr) * (V[o] - V[o + sx]);
    const double vu_w = V[o + sx - sy] + (dxr / dx2xr) * (V[o - sy] - V[o + sx - sy]);
    const double vin = 0.5 * (vu_e + vu_w);
    const double wu_n = W[o + sx] + (dxr / dx2xr) * (W[o] - W[o + sx]);
    const double wu_s = W[o + sx - sz] + (dxr / dx2xr) * (W[o - sz] - W[o + sx - sz]);
    const double win = 0.5 * (wu_n + wu_s);
    if (i != 2 && i < nx && j != 2 && j < ny + 1 && k != 2 && k < nz + 1 && noib) {
      cx = up3<0>(g, u0, i, U[o + 2 * sx], U[o + sx], u0, U[o - sx], U[o - 2 * sx], DX[i + 1], DX[i]);
      cy = up3<4>(g, vin, j, U[o + 2 * sy], U[o + sy], u0, U[o - sy], U[o - 2 * sy], ddye, ddy);
      cz = up3<5>(g, win, k, U[o + 2 * sz], U[o + sz], u0, U[o - sz], U[o - 2 * sz], ddzr, ddz);
    } else {
      const double r1x = DX[i] / DX[i + 1];
      const double r1yn = 0.5 * (DY[j] + DY[j - 1]), r1yd = 0.5 * (DY[j] + DY[j + 1]), r1y = r1yn / r1yd;
      const double r1zn = 0.5 * (DZ[k] + DZ[k - 1]), r1zd = 0.5 * (DZ[k] + DZ[k + 1]), r1z = r1zn / r1zd;
      cx = up1(u0, DX[i + 1], r1x, U[o - sx], u0, U[o + sx]);
      cy = up1(vin, r1yd, r1y, U[o - sy], u0, U[o + sy]);
      cz = up1(win, r1zd, r1z, U[o - sz], u0, U[o + sz]);
    }
    const double d2x = (2.0 / dx2xr) * ((-u4 / dxr) + (u22 / dx));
    const double d2y = (2.0 / (0.5 * (dy2ye + dy2yw))) * ((-u8 / (0.5 * dy2ye)) + (u6 / (0.5 * dy2yw)));
    const double d2z = (2.0 / (0.5 * (dz2zt + dz2zb))) * ((-u12 / (0.5 * dz2zt)) + (u10 / (0.5 * dz2zb)));
    const double xtt2 = rev * (d2x + d2y + d2z);
    const double resid = -cx - cy - cz + xtt2;
    if (ab2) UT[o] = u0 + deltat * (0.5 * (3.0 * resid - RU[o]) + dpdx);   // nsMomentumAB
    else UT[o] = u0 + deltat * (resid + dpdx);
    if (RU) RU[o] = resid;
  }
  // ---- v momentum (:901-1006)
  {
    const double uv_e = U[o + sy] + (dye / dy2ye) * (U[o] - U[o + sy]);
    const double uv_w = U[o - sx + sy] + (dye / dy2ye) * (U[o - sx] - U[o - sx + sy]);
    const double uin = 0.5 * (uv_e + uv_w);
    const double wv_n = W[o + sy] + (dye / dy2ye) * (W[o] - W[o + sy]);
    const double wv_s = W[o + sy - sz] + (dye / dy2ye) * (W[o - sz] - W[o + sy - sz]);
    const double win = 0.5 * (wv_n + wv_s);
    if (i != 2 && i < nx + 1 && j != 2 && j < ny && k != 2 && k < nz + 1 && noib) {
      cx = up3<3>(g, uin, i, V[o + 2 * sx], V[o + sx], v0, V[o - sx], V[o - 2 * sx], ddxr, ddx);
      cy = up3<1>(g, v0, j, V[o + 2 * sy], V[o + sy], v0, V[o - sy], V[o - 2 * sy], DY[j + 1], DY[j]);
      cz = up3<5>(g, win, k, V[o + 2 * sz], V[o + sz], v0, V[o - sz], V[o - 2 * sz], ddzr, ddz);
    } else {
      const double r1xn = 0.5 * (DX[i] + DX[i - 1]), r1xd = 0.5 * (DX[i] + DX[i + 1]), r1x = r1xn / r1xd;
      const double r1y = DY[j] / DY[j + 1];
      const double r1zn = 0.5 * (DZ[k] + DZ[k - 1]), r1zd = 0.5 * (DZ[k] + DZ[k + 1]), r1z = r1zn / r1zd;
      cx = up1(uin, r1xd, r1x, V[o - sx], v0, V[o + sx]);
      cy = up1(v0, DY[j + 1], r1y, V[o - sy], v0, V[o + sy]);
      cz = up1(win, r1zd, r1z, V[o - sz], v0, V[o + sz]);
    }
    const double d2x = (2.0 / (0.5 * (dx2xr + dx2xl))) * ((-v6 / (0.5 * dx2xr)) + (v4 / (0.5 * dx2xl)));
    const double d2y = (2.0 / dy2ye) * ((-v10 / dye) + (v8 / dy));
    const double d2z = (2.0 / (0.5 * (dz2zt + dz2zb))) * ((-v14 / (0.5 * dz2zt)) + (v12 / (0.5 * dz2zb)));
    const double ytt2 = rev * (d2x + d2y + d2z);
    const double resid = -cx - cy - cz + ytt2;
    if (ab2) VT[o] = v0 + deltat * (0.5 * (3.0 * resid - RV[o]) + dpdy);   // nsMomentumAB
    else VT[o] = v0 + deltat * (resid + dpdy);
    if (RV) RV[o] = resid;
  }
  // ---- w momentum (:1010-1116)
  {
    const double uw_e = U[o + sz] + (dzt / dz2zt) * (U[o] - U[o + sz]);
    const double uw_w = U[o - sx + sz] + (dzt / dz2zt) * (U[o - sx] - U[o - sx + sz]);
    const double uin = 0.5 * (uw_e + uw_w);
    const double vw_n = V[o + sz] + (dzt / dz2zt) * (V[o] - V[o + sz]);
    const double vw_s = V[o - sy + sz] + (dzt / dz2zt) * (V[o - sy] - V[o - sy + sz]);
    const double vin = 0.5 * (vw_n + vw_s);
    if (i != 2 && i < nx + 1 && j != 2 && j < ny + 1 && k != 2 && k < nz && noib) {
      cx = up3<3>(g, uin, i, W[o + 2 * sx], W[o + sx], w0, W[o - sx], W[o - 2 * sx], ddxr, ddx);
      cy = up3<4>(g, vin, j, W[o + 2 * sy], W[o + sy], w0, W[o - sy], W[o - 2 * sy], ddye, ddy);
      cz = up3<2>(g, w0, k, W[o + 2 * sz], W[o + sz], w0, W[o - sz], W[o - 2 * sz], DZ[k + 1], DZ[k]);
    } else {
      const double r1xn = 0.5 * (DX[i] + DX[i - 1]), r1xd = 0.5 * (DX[i] + DX[i + 1]), r1x = r1xn / r1xd;
      const double r1yn = 0.5 * (DY[j] + DY[j - 1]), r1yd = 0.5 * (DY[j] + DY[j + 1]), r1y = r1yn / r1yd;
      const double r1z = DZ[k] / DZ[k + 1];
      cx = up1(uin, r1xd, r1x, W[o - sx], w0, W[o + sx]);
      cy = up1(vin, r1yd, r1y, W[o - sy], w0, W[o + sy]);
      cz = up1(w0, DZ[k + 1], r1z, W[o - sz], w0, W[o + sz]);
    }
    const double d2x = (2.0 / (0.5 * (dx2xr + dx2xl))) * ((-w8 / (0.5 * dx2xr)) + (w6 / (0.5 * dx2xl)));
    const double d2y = (2.0 / (0.5 * (dy2ye + dy2yw))) * ((-w12 / (0.5 * dy2ye)) + (w10 / (0.5 * dy2yw)));
    const double d2z = (2.0 / dz2zt) * ((-w16 / dzt) + (w14 / dz));
    const double ztt2 = rev * (d2x + d2y + d2z);
    const double resid = -cx - cy - cz + ztt2;
    if (ab2) WT[o] = w0 + deltat * (0.5 * (3.0 * resid - RW[o]) + dpdz);   // nsMomentumAB
    else WT[o] = w0 + deltat * (resid + dpdz);
    if (RW) RW[o] = resid;
  }
}

void launch_momentum(ib3d_ctx* c, bool ab2) {
  PhaseScope ps(c, PH_MOMENTUM);
  c->launches += 1;
  const long long n = (long long)c->d.nx * c->d.ny * c->d.nz;
  const unsigned nb = (unsigned)((n + 127) / 128);
  k_momentum<<<nb, 128, 0, c->st>>>(c->d, c->g, c->u, c->v, c->w, c->p, c->cell, c->ut, c->vt, c->wt,
                                     1.0 / c->prm.re, c->prm.deltat, c->resi[0], c->resi[1], c->resi[2],
                                     ab2 ? 1 : 0);
}

}  // namespace ib3d
