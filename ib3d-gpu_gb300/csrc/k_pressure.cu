// Pressure path of one time step: divergence RHS, red-black SOR (FP64 reference
// arithmetic, or FP32 sweeps inside an FP64 defect-correction loop), pressure and
// velocity correction, boundary conditions and the steady-state indicator.
//
// Reference: poissonSolver / computeDiv / correctPressure / correctVelocity /
// REDBLACKSOR (subPcorVcor.f90:2-212), velocityBC and solidCellBC
// (subBoundaryConditions.f90:2-217), initialConditions (subInitialConditions.f90).
//
// This file is compiled with -fmad=false: every FP64 product and sum is rounded
// separately, in the reference's left-to-right order, so the FP64 path is
// bit-identical to the serial oracle. Kernels address the reference's padded
// Fortran layout directly and mask by the uint8 cell flags instead of gathering
// through int64 index lists.
#include <algorithm>
#include <cmath>

#include "ib3d_internal.cuh"

namespace ib3d {

namespace {

__device__ __forceinline__ void decode(const Dims& d, unsigned idx, int& i, int& j, int& k) {
  const unsigned nx2 = (unsigned)d.NX2, ny2 = (unsigned)d.NY2;
  i = (int)(idx % nx2) + 1;
  const unsigned t = idx / nx2;
  j = (int)(t % ny2) + 1;
  k = (int)(t / ny2) + 1;
}
__device__ __forceinline__ bool interior(const Dims& d, int i, int j, int k) {
  return i >= 2 && i <= d.nx + 1 && j >= 2 && j <= d.ny + 1 && k >= 2 && k <= d.nz + 1;
}
inline unsigned nblocks(long long n) { return (unsigned)((n + kBlock - 1) / kBlock); }

}  // namespace

// computeDiv (subPcorVcor.f90:82-101) fused with the zeroing of b and pc
// (subPcorVcor.f90:19-28). Also stores bdt = b/deltat, the quotient every SOR
// sweep of the reference recomputes (:170, :184) -- the same rounded value.
__global__ void k_divergence(Dims d, Grid1D g, const double* __restrict__ ut, const double* __restrict__ vt,
                             const double* __restrict__ wt, const unsigned char* __restrict__ cell,
                             double* __restrict__ b, double* __restrict__ bdt, double* __restrict__ pc,
                             double deltat, int zero_pc, unsigned long long* divmax) {
  const unsigned idx = blockIdx.x * blockDim.x + threadIdx.x;
  double m = 0.0;
  if (idx < (unsigned)d.n3) {
    int i, j, k;
    decode(d, idx, i, j, k);
    double bb = 0.0;
    if (interior(d, i, j, k) && cell[idx] == 0) {
      const long long pl = (long long)d.NX2 * d.NY2;
      bb = (ut[idx] - ut[idx - 1]) / g.dx[i] + (vt[idx] - vt[idx - d.NX2]) / g.dy[j] +
           (wt[idx] - wt[idx - pl]) / g.dz[k];
      m = fabs(bb);
    }
    b[idx] = bb;
    bdt[idx] = bb / deltat;
    if (zero_pc) pc[idx] = 0.0;
  }
  block_max_atomic(m, divmax);
}

// One colour of a red-black SOR sweep in FP64 (subPcorVcor.f90:164-191).
// Red cells are (i+j+k) odd (subSearch.f90:562). Because the reference's pco
// equals pc at every fluid cell when a sweep starts and non-fluid pc stays 0, the
// red pass's pco neighbours and both passes' pco(i,j,k) are the current pc values,
// so one in-place kernel per colour reproduces it exactly. Each thread owns one
// (i, i+1) pair of a row and updates the member of the active colour; the max
// update |pc_new - pc_old| (the reference's derr2, :193-201) is reduced on chip.
template <int COLOR>
__global__ void __launch_bounds__(kBlock) k_sor64(Dims d, Grid1D g, const double* __restrict__ bdt,
                                                  double* __restrict__ pc, const unsigned char* __restrict__ cell,
                                                  double omega, double om1, SolveCtl* ctl, long long sweep,
                                                  int decide_mode, double eps, long long max_sweeps) {
  if (ctl->done) return;
  const unsigned tid = blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned npairs = (unsigned)(d.nx + 1) >> 1;
  double delta = 0.0;
  if (tid < npairs * (unsigned)d.ny * (unsigned)d.nz) {
    const int ip = (int)(tid % npairs);
    const unsigned t = tid / npairs;
    const int j = (int)(t % (unsigned)d.ny) + 2, k = (int)(t / (unsigned)d.ny) + 2;
    const int i0 = 2 + 2 * ip;
    const int i = i0 + ((i0 + j + k + 1 + COLOR) & 1);
    if (i <= d.nx + 1) {
      const long long idx = d.at(i, j, k);
      if (cell[idx] == 0) {
        const long long sy = d.NX2, sz = (long long)d.NX2 * d.NY2;
        const double num = bdt[idx] - g.acx[0][i - 1] * pc[idx - 1] - g.acx[2][i - 1] * pc[idx + 1] -
                           g.acy[0][j - 1] * pc[idx - sy] - g.acy[2][j - 1] * pc[idx + sy] -
                           g.acz[0][k - 1] * pc[idx - sz] - g.acz[2][k - 1] * pc[idx + sz];
        const double diag = g.acx[1][i - 1] + g.acy[1][j - 1] + g.acz[1][k - 1];
        const double gs = num / diag;
        const double old = pc[idx];
        const double nw = om1 * old + omega * gs;
        pc[idx] = nw;
        delta = fabs(nw - old);
      }
    }
  }
  block_max_atomic(delta, &ctl->upd);
  if (COLOR == 1) finish_block(ctl, &ctl->upd, decide_mode, sweep, eps, max_sweeps);
}

// Residual r = b/dt - A pc at fluid cells, in the SOR numerator's order followed by
// "- diag*pc"; max |r| feeds the residual stopping test or the defect-correction
// loop, and r (rounded to FP32) is the right-hand side of the FP32 inner solve.
__global__ void __launch_bounds__(kBlock) k_residual64(Dims d, Grid1D g, const double* __restrict__ bdt,
                                                       const double* __restrict__ pc,
                                                       const unsigned char* __restrict__ cell,
                                                       float* __restrict__ r32, float* __restrict__ rp_red,
                                                       float* __restrict__ rp_black, int Lp, SolveCtl* ctl,
                                                       long long sweep, int decide_mode, double eps,
                                                       long long max_sweeps) {
  if (decide_mode != 2 && ctl->done) return;
  const unsigned tid = blockIdx.x * blockDim.x + threadIdx.x;
  double m = 0.0;
  if (tid < (unsigned)d.nx * (unsigned)d.ny * (unsigned)d.nz) {
    const int i = (int)(tid % (unsigned)d.nx) + 2;
    const unsigned t = tid / (unsigned)d.nx;
    const int j = (int)(t % (unsigned)d.ny) + 2, k = (int)(t / (unsigned)d.ny) + 2;
    const long long idx = d.at(i, j, k);
    float rr = __int_as_float(0x7fc00000);   // NaN marks a non-fluid cell for the FP32 sweep
    if (cell[idx] == 0) {
      const long long sy = d.NX2, sz = (long long)d.NX2 * d.NY2;
      const double num = bdt[idx] - g.acx[0][i - 1] * pc[idx - 1] - g.acx[2][i - 1] * pc[idx + 1] -
                         g.acy[0][j - 1] * pc[idx - sy] - g.acy[2][j - 1] * pc[idx + sy] -
                         g.acz[0][k - 1] * pc[idx - sz] - g.acz[2][k - 1] * pc[idx + sz];
      const double diag = g.acx[1][i - 1] + g.acy[1][j - 1] + g.acz[1][k - 1];
      const double r = num - diag * pc[idx];
      m = fabs(r);
      rr = (float)r;
    }
    if (rp_red) {   // colour-packed right-hand side (k_sor32.cu)
      const long long s = ((long long)(k - 1) * d.NY2 + (j - 1)) * Lp + ((i - 2) >> 1) + 4;
      (((i + j + k) & 1) ? rp_red : rp_black)[s] = rr;
    } else if (r32) {
      r32[idx] = rr;
    }
  }
  block_max_atomic(m, &ctl->res);
  finish_block(ctl, &ctl->res, decide_mode == 2 ? 0 : decide_mode, sweep, eps, max_sweeps);
}

// One colour of an FP32 red-black sweep on A e = r (the inner solve of the
// defect-correction loop). Same stencil and colouring as k_sor64; e and r are FP32,
// the coefficients are the FP64 tables rounded once to FP32.
template <int COLOR>
__global__ void __launch_bounds__(kBlock) k_sor32(Dims d, Grid1D g, const float* __restrict__ r32,
                                                  float* __restrict__ e, const unsigned char* __restrict__ cell,
                                                  float omega, float om1) {
  const unsigned tid = blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned npairs = (unsigned)(d.nx + 1) >> 1;
  if (tid >= npairs * (unsigned)d.ny * (unsigned)d.nz) return;
  const int ip = (int)(tid % npairs);
  const unsigned t = tid / npairs;
  const int j = (int)(t % (unsigned)d.ny) + 2, k = (int)(t / (unsigned)d.ny) + 2;
  const int i0 = 2 + 2 * ip;
  const int i = i0 + ((i0 + j + k + 1 + COLOR) & 1);
  if (i > d.nx + 1) return;
  const long long idx = d.at(i, j, k);
  if (cell[idx] != 0) return;
  const long long sy = d.NX2, sz = (long long)d.NX2 * d.NY2;
  float num = r32[idx];
  num = fmaf(-g.acx32[0][i - 1], e[idx - 1], num);
  num = fmaf(-g.acx32[2][i - 1], e[idx + 1], num);
  num = fmaf(-g.acy32[0][j - 1], e[idx - sy], num);
  num = fmaf(-g.acy32[2][j - 1], e[idx + sy], num);
  num = fmaf(-g.acz32[0][k - 1], e[idx - sz], num);
  num = fmaf(-g.acz32[2][k - 1], e[idx + sz], num);
  const float diag = g.acx32[1][i - 1] + g.acy32[1][j - 1] + g.acz32[1][k - 1];
  e[idx] = sor32_update(e[idx], num, diag, omega, om1);
}

// pc += e (FP64 accumulation of the FP32 correction), then e = 0.
__global__ void k_accumulate(long long n3, double* __restrict__ pc, float* __restrict__ e) {
  const unsigned idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (unsigned)n3) return;
  const float x = e[idx];
  if (x != 0.0f) {
    pc[idx] = pc[idx] + (double)x;
    e[idx] = 0.0f;
  }
}

// correctPressure + correctVelocity (subPcorVcor.f90:105-142) in one pass over the
// fluid cells. cor*[i] = deltat/(0.5*(d(i+1)+d(i))), the 1-D quotient of :137-139.
__global__ void __launch_bounds__(kBlock) k_correct(Dims d, Grid1D g, const double* __restrict__ pc,
                                                    const unsigned char* __restrict__ cell, double* __restrict__ p,
                                                    double* __restrict__ ut, double* __restrict__ vt,
                                                    double* __restrict__ wt) {
  const unsigned tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= (unsigned)d.nx * (unsigned)d.ny * (unsigned)d.nz) return;
  const int i = (int)(tid % (unsigned)d.nx) + 2;
  const unsigned t = tid / (unsigned)d.nx;
  const int j = (int)(t % (unsigned)d.ny) + 2, k = (int)(t / (unsigned)d.ny) + 2;
  const long long idx = d.at(i, j, k);
  if (cell[idx] != 0) return;
  const long long sy = d.NX2, sz = (long long)d.NX2 * d.NY2;
  const double c = pc[idx];
  p[idx] = p[idx] + c;
  ut[idx] = ut[idx] - g.corx[i] * (pc[idx + 1] - c);
  vt[idx] = vt[idx] - g.cory[j] * (pc[idx + sy] - c);
  wt[idx] = wt[idx] - g.corz[k] * (pc[idx + sz] - c);
}

// velocityBC, active branch (subBoundaryConditions.f90:350-406): x faces (inlet
// u = 1, v/w reflected; outlet zero gradient), then y and z faces (slip).
__global__ void k_bc_x(Dims d, Grid1D g, double* ut, double* vt, double* wt, const double* __restrict__ u,
                       const double* __restrict__ v, const double* __restrict__ w, const double* __restrict__ ucp,
                       double deltat, int convective) {
  const unsigned tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= (unsigned)d.ny * (unsigned)d.nz) return;
  const int j = (int)(tid % (unsigned)d.ny) + 2, k = (int)(tid / (unsigned)d.ny) + 2;
  const int nx = d.nx;
  ut[d.at(1, j, k)] = 1.0;
  vt[d.at(1, j, k)] = -vt[d.at(2, j, k)];
  wt[d.at(1, j, k)] = -wt[d.at(2, j, k)];
  if (convective) {   // Orlanski (the commented :153-155), uc from calculateUc
    const double uc = *ucp;
    const long long a = d.at(nx + 1, j, k), b2 = d.at(nx + 2, j, k), a0 = d.at(nx, j, k);
    ut[a] = u[a] - (deltat / g.dx[nx + 1]) * uc * (u[a] - u[a0]);
    vt[b2] = -vt[a] + v[b2] + v[a] - (2.0 * deltat / g.dx[nx + 2]) * uc * (v[b2] - v[a]);
    wt[b2] = -wt[a] + w[b2] + w[a] - (2.0 * deltat / g.dx[nx + 2]) * uc * (w[b2] - w[a]);
  } else {            // zero gradient (:149-151)
    ut[d.at(nx + 1, j, k)] = ut[d.at(nx, j, k)];
    vt[d.at(nx + 2, j, k)] = vt[d.at(nx + 1, j, k)];
    wt[d.at(nx + 2, j, k)] = wt[d.at(nx + 1, j, k)];
  }
}

// calculateUc (subCalculateuc.f90:2-38): uc = max(mean of ut(nx-4,j,k) over the
// plane's fluid cells, 0). One warp; the sum runs in the serial order k outer, j
// inner (lane 0 adds the warp's 32 loaded values one by one), so it matches a
// serial build of the reference bit for bit.
__global__ void k_calculate_uc(Dims d, const double* __restrict__ ut, const unsigned char* __restrict__ cell,
                               double* ucp) {
  const int lane = threadIdx.x;
  const int i = d.nx - 4;
  double sum = 0.0;
  long long count = 0;
  for (int k = 2; k <= d.nz + 1; ++k)
    for (int j0 = 2; j0 <= d.ny + 1; j0 += 32) {
      const int j = j0 + lane;
      double x = 0.0;
      int fl = 0;
      if (j <= d.ny + 1) {
        const long long o = d.at(i, j, k);
        fl = cell[o] == 0;
        x = fl ? ut[o] : 0.0;
      }
      for (int l = 0; l < 32; ++l) {
        const double xl = __shfl_sync(0xffffffffu, x, l);
        const int fll = __shfl_sync(0xffffffffu, fl, l);
        if (fll) { sum = sum + xl; ++count; }
      }
    }
  if (lane == 0) {
    const double uc1 = sum / (double)count;
    *ucp = uc1 > 0.0 ? uc1 : 0.0;
  }
}

void launch_calculate_uc(ib3d_ctx* c) {
  PhaseScope ps(c, PH_BC);
  c->launches += 1;
  k_calculate_uc<<<1, 32, 0, c->st>>>(c->d, c->ut, c->cell, c->d_coef + 6);
}
__global__ void k_bc_y(Dims d, double* ut, double* vt, double* wt) {
  const unsigned tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= (unsigned)d.nx * (unsigned)d.nz) return;
  const int i = (int)(tid % (unsigned)d.nx) + 2, k = (int)(tid / (unsigned)d.nx) + 2;
  const int ny = d.ny;
  ut[d.at(i, 1, k)] = ut[d.at(i, 2, k)];
  wt[d.at(i, 1, k)] = wt[d.at(i, 2, k)];
  vt[d.at(i, 1, k)] = 0.0;
  ut[d.at(i, ny + 2, k)] = ut[d.at(i, ny + 1, k)];
  wt[d.at(i, ny + 2, k)] = wt[d.at(i, ny + 1, k)];
  vt[d.at(i, ny + 1, k)] = 0.0;
}
__global__ void k_bc_z(Dims d, double* ut, double* vt, double* wt) {
  const unsigned tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= (unsigned)d.nx * (unsigned)d.ny) return;
  const int i = (int)(tid % (unsigned)d.nx) + 2, j = (int)(tid / (unsigned)d.nx) + 2;
  const int nz = d.nz;
  ut[d.at(i, j, 1)] = ut[d.at(i, j, 2)];
  vt[d.at(i, j, 1)] = vt[d.at(i, j, 2)];
  wt[d.at(i, j, 1)] = 0.0;
  ut[d.at(i, j, nz + 2)] = ut[d.at(i, j, nz + 1)];
  vt[d.at(i, j, nz + 2)] = vt[d.at(i, j, nz + 1)];
  wt[d.at(i, j, nz + 1)] = 0.0;
}

// solidCellBC (subBoundaryConditions.f90:199-217), flag-masked.
__global__ void k_solid_bc(Dims d, const unsigned char* __restrict__ cell, double* ut, double* vt, double* wt,
                           double* p) {
  const unsigned idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (unsigned)d.n3) return;
  if (cell[idx] != 1) return;
  int i, j, k;
  decode(d, idx, i, j, k);
  if (!interior(d, i, j, k)) return;
  ut[idx] = 0.0; vt[idx] = 0.0; wt[idx] = 0.0; p[idx] = 0.0;
}

// Steady-state indicator derrStdSt = max |ut-u|/dt (subPcorVcor.f90:45-58) over fluid
// cells, fused with the copy u = ut, v = vt, w = wt of the whole array (:67-77). The
// kernel reduces max |ut-u| and the caller divides the maximum by dt once: rounded
// division by a positive number is monotone, so the quotient of the maximum is the
// maximum of the per-cell quotients, bit for bit, without three FP64 divisions per
// cell.
__global__ void k_dss_copy(Dims d, const unsigned char* __restrict__ cell, double* __restrict__ u,
                           double* __restrict__ v, double* __restrict__ w, const double* __restrict__ ut,
                           const double* __restrict__ vt, const double* __restrict__ wt,
                           unsigned long long* acc) {
  const unsigned idx = blockIdx.x * blockDim.x + threadIdx.x;
  double m = 0.0;
  if (idx < (unsigned)d.n3) {
    const double a = ut[idx], bb = vt[idx], c = wt[idx];
    int i, j, k;
    decode(d, idx, i, j, k);
    if (interior(d, i, j, k) && cell[idx] == 0) {
      const double du = fabs(a - u[idx]);
      const double dv = fabs(bb - v[idx]);
      const double dw = fabs(c - w[idx]);
      m = nan_max(nan_max(du, dv), dw);
    }
    u[idx] = a; v[idx] = bb; w[idx] = c;
  }
  block_max_atomic(m, acc);
}

// initialConditions (subInitialConditions.f90:22-56): every field 0, u = 1 on fluid cells.
__global__ void k_initial(Dims d, const unsigned char* __restrict__ cell, double* u, double* v, double* w,
                          double* ut, double* vt, double* wt, double* p, double* pc) {
  const unsigned idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (unsigned)d.n3) return;
  int i, j, k;
  decode(d, idx, i, j, k);
  u[idx] = (interior(d, i, j, k) && cell[idx] == 0) ? 1.0 : 0.0;
  v[idx] = 0.0; w[idx] = 0.0; ut[idx] = 0.0; vt[idx] = 0.0; wt[idx] = 0.0; p[idx] = 0.0; pc[idx] = 0.0;
}

// ---------------------------------------------------------------- launchers

void launch_divergence(ib3d_ctx* c, bool zero_pc) {
  PhaseScope ps(c, PH_DIVERGENCE);
  c->launches += 1;
  k_divergence<<<nblocks(c->d.n3), kBlock, 0, c->st>>>(c->d, c->g, c->ut, c->vt, c->wt, c->cell, c->b, c->bdt,
                                                        c->pc, c->prm.deltat, zero_pc ? 1 : 0, &c->ctl->aux);
}

// b/dt from a b set by the caller (the quotient the sweeps use), and pc = 0 for a
// zero initial guess.
__global__ void k_bdt(long long n3, const double* __restrict__ b, double* __restrict__ bdt,
                      double* __restrict__ pc, double deltat, int zero_pc) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n3) return;
  bdt[idx] = b[idx] / deltat;
  if (zero_pc) pc[idx] = 0.0;
}

void launch_bdt(ib3d_ctx* c, bool zero_pc) {
  PhaseScope ps(c, PH_DIVERGENCE);
  c->launches += 1;
  k_bdt<<<nblocks(c->d.n3), kBlock, 0, c->st>>>(c->d.n3, c->b, c->bdt, c->pc, c->prm.deltat, zero_pc ? 1 : 0);
}

void launch_correct(ib3d_ctx* c) {
  PhaseScope ps(c, PH_CORRECT);
  c->launches += 1;
  const long long n = (long long)c->d.nx * c->d.ny * c->d.nz;
  k_correct<<<nblocks(n), kBlock, 0, c->st>>>(c->d, c->g, c->pc, c->cell, c->p, c->ut, c->vt, c->wt);
}

void launch_velocity_bc(ib3d_ctx* c) {
  PhaseScope ps(c, PH_BC);
  c->launches += 3;
  const Dims& d = c->d;
  k_bc_x<<<nblocks((long long)d.ny * d.nz), kBlock, 0, c->st>>>(d, c->g, c->ut, c->vt, c->wt, c->u, c->v, c->w,
                                                                 c->d_coef + 6, c->prm.deltat,
                                                                 c->prm.outlet == IB3D_OUTLET_CONVECTIVE ? 1 : 0);
  k_bc_y<<<nblocks((long long)d.nx * d.nz), kBlock, 0, c->st>>>(d, c->ut, c->vt, c->wt);
  k_bc_z<<<nblocks((long long)d.nx * d.ny), kBlock, 0, c->st>>>(d, c->ut, c->vt, c->wt);
}

void launch_solid_bc(ib3d_ctx* c) {
  PhaseScope ps(c, PH_BC);
  c->launches += 1;
  k_solid_bc<<<nblocks(c->d.n3), kBlock, 0, c->st>>>(c->d, c->cell, c->ut, c->vt, c->wt, c->p);
}

void launch_dss_copy(ib3d_ctx* c) {
  PhaseScope ps(c, PH_CORRECT);
  c->launches += 1;
  k_dss_copy<<<nblocks(c->d.n3), kBlock, 0, c->st>>>(c->d, c->cell, c->u, c->v, c->w, c->ut, c->vt, c->wt,
                                                      &c->ctl->aux);
}

void launch_initial(ib3d_ctx* c) {
  c->launches += 1;
  k_initial<<<nblocks(c->d.n3), kBlock, 0, c->st>>>(c->d, c->cell, c->u, c->v, c->w, c->ut, c->vt, c->wt, c->p,
                                                     c->pc);
}

namespace {
int read_ctl(ib3d_ctx* c) {
  IB3D_CUDA(c, cudaMemcpyAsync(c->h_ctl, c->ctl, sizeof(SolveCtl), cudaMemcpyDeviceToHost, c->st));
  IB3D_CUDA(c, cudaStreamSynchronize(c->st));
  return IB3D_OK;
}
int reset_ctl(ib3d_ctx* c) {
  IB3D_CUDA(c, cudaMemsetAsync(c->ctl, 0, sizeof(SolveCtl), c->st));
  return IB3D_OK;
}
}  // namespace

// REDBLACKSOR (subPcorVcor.f90:148-212) in FP64. Sweeps are enqueued in growing
// batches; the sweep that meets the stopping test raises ctl->done from the device
// and every later kernel of the batch returns at once, so the stopping sweep is the
// one the reference's per-sweep host test would pick, with one host round trip per
// batch instead of per sweep.
int run_sor_fp64(ib3d_ctx* c, ib3d_solve_stats* st) {
  const Dims& d = c->d;
  const ib3d_params& P = c->prm;
  const unsigned ncol = (unsigned)((((long long)d.nx + 1) / 2) * d.ny * d.nz);
  const unsigned gcol = (ncol + kBlock - 1) / kBlock;
  const long long ncell = (long long)d.nx * d.ny * d.nz;
  const double om1 = 1.0 - P.omega;
  const bool resid = P.criterion == IB3D_CRIT_RESIDUAL;
  const int every = P.check_every < 1 ? 1 : P.check_every;
  int rc = reset_ctl(c);
  if (rc) return rc;
  long long sweep = 0;
  long long batch = 4;
  for (;;) {
    {
    PhaseScope ps(c, PH_SOR64);
    for (long long q = 0; q < batch; ++q) {
      ++sweep;
      c->launches += (resid && (sweep % every) == 0) ? 3 : 2;
      int mode_black = resid ? ((sweep % every) ? 1 : 2) : 0;
      k_sor64<0><<<gcol, kBlock, 0, c->st>>>(d, c->g, c->bdt, c->pc, c->cell, P.omega, om1, c->ctl, sweep, 2,
                                             P.eps, P.max_sweeps);
      k_sor64<1><<<gcol, kBlock, 0, c->st>>>(d, c->g, c->bdt, c->pc, c->cell, P.omega, om1, c->ctl, sweep,
                                             mode_black, P.eps, P.max_sweeps);
      if (resid && (sweep % every) == 0)
        k_residual64<<<nblocks(ncell), kBlock, 0, c->st>>>(d, c->g, c->bdt, c->pc, c->cell, nullptr, nullptr,
                                                            nullptr, 0, c->ctl, sweep, 0, P.eps, P.max_sweeps);
    }
    }
    IB3D_CUDA(c, cudaGetLastError());
    rc = read_ctl(c);
    if (rc) return rc;
    if (c->h_ctl->done) break;
    if (batch < 256) batch *= 2;
  }
  st->sweeps = c->h_ctl->nsweeps;
  st->outer = 0;
  c->t_sweeps64 += st->sweeps;
  st->final_err = c->h_ctl->final_err;
  if (c->h_ctl->final_err != c->h_ctl->final_err) return IB3D_ERR_NONFINITE;
  return c->h_ctl->done == 2 ? IB3D_ERR_NOCONV : IB3D_OK;
}

// Mixed precision: FP64 defect correction around FP32 red-black sweeps.
//   repeat: r = b/dt - A pc (FP64); stop when max|r| < eps;
//           solve A e = r approximately with inner_sweeps FP32 sweeps from e = 0;
//           pc += e (FP64).
// The residual, right-hand side and the accumulated pc stay FP64, so the loop stops
// at the same FP64 residual tolerance as the FP64 path.
int run_sor_fp32dc(ib3d_ctx* c, ib3d_solve_stats* st) {
  const Dims& d = c->d;
  const ib3d_params& P = c->prm;
  const unsigned ncol = (unsigned)((((long long)d.nx + 1) / 2) * d.ny * d.nz);
  const unsigned gcol = (ncol + kBlock - 1) / kBlock;
  const double wi = P.omega_inner > 0.0 ? P.omega_inner : P.omega;
  const float om = (float)wi, om1 = (float)(1.0 - wi);
  const int inner = P.inner_sweeps < 1 ? 1 : P.inner_sweeps;
  const bool fused = P.sweep_kernel == 2;
  const bool packed = P.sweep_kernel != 1 && c->ep[0] != nullptr;
  if (fused) {
    if (!packed || !fused_sweep_fits(d.nx)) {
      c->err = "sweep_kernel 2 (fused sweep) needs an even nx whose packed rows fit its blocks (nx <= 512)";
      return IB3D_ERR_ARG;
    }
    if (!c->epn[0]) {
      const size_t np = (size_t)c->packed_lp * (size_t)d.NY2 * (size_t)d.NZ2;
      for (int q = 0; q < 2; ++q) {
        if (cudaMalloc(&c->epn[q], np * sizeof(float)) != cudaSuccess) return IB3D_ERR_MEMORY;
        IB3D_CUDA(c, cudaMemsetAsync(c->epn[q], 0, np * sizeof(float), c->st));
      }
    }
  }
  int rc = reset_ctl(c);
  if (rc) return rc;
  if (!packed) IB3D_CUDA(c, cudaMemsetAsync(c->e32, 0, sizeof(float) * (size_t)d.n3, c->st));
  long long sweeps = 0, outer = 0;
  int batch = inner, prev_batch = inner;
  double prev_res = 0.0;
  for (;;) {
    {
      PhaseScope ps(c, PH_RESIDUAL);
      launch_residual_fast(c, sweeps);
    }
    IB3D_CUDA(c, cudaGetLastError());
    rc = read_ctl(c);
    if (rc) return rc;
    if (c->h_ctl->stage_err) {
      c->err = "fused FP32 sweep: a shared-memory stage never arrived (bounded wait gave up)";
      return IB3D_ERR_CUDA;
    }
    const double res = c->h_ctl->last_res;
    if (outer == 0) st->initial_err = res;
    if (c->h_ctl->done) break;
    if (P.inner_schedule == IB3D_INNER_ADAPTIVE && outer > 0 && res > 0.0 && res < prev_res) {
      // log residual reduction per sweep over the last pass, and the sweeps that
      // rate needs to reach eps (with a margin), at most four decades per pass
      const double rate = std::log(res / prev_res) / batch;
      const double need = std::log(P.eps / res) / rate;
      const double cap = std::log(1e-4) / rate;
      batch = (int)std::min(std::max(std::min(1.08 * need + 8.0, cap), 16.0), 65536.0);
    }
    if (P.inner_schedule == IB3D_INNER_TAIL) {
      // passes of `inner` sweeps; the one the last pass's rate says will reach eps is cut
      // to the sweeps it needs (a prediction that falls short costs one more pass)
      batch = inner;
      if (outer > 0 && res > 0.0 && res < prev_res) {
        const double rate = std::log(res / prev_res) / prev_batch;
        const double need = std::log(P.eps / res) / rate;
        batch = (int)std::min(std::max(1.08 * need + 8.0, 16.0), (double)inner);
      }
    }
    if (sweeps + batch > P.max_sweeps) batch = (int)std::max(1ll, P.max_sweeps - sweeps);
    prev_batch = batch;
    prev_res = res;
    {
      PhaseScope ps(c, PH_SOR32);
      c->launches += fused ? batch : 2 * batch;
      c->t_launches32 += fused ? batch : 2 * batch;
      // the solve's first sweeps run at relaxation 1 (smooth_sweeps: Gauss-Seidel damps the
      // high-frequency error that the over-relaxed sweeps barely touch), the next
      // ramp_sweeps with the relaxation rising linearly from 1 to omega_inner; the
      // colour-packed kernels run the sweeps after those through run_sor32_sweeps
      const int special = outer == 0 ? P.smooth_sweeps + P.ramp_sweeps : 0;
      const int direct = packed && !fused ? std::min(batch, special) : batch;
      for (int q = 0; q < direct; ++q) {
        const bool smooth = outer == 0 && q < P.smooth_sweeps;
        float w = smooth ? 1.0f : om, w1 = smooth ? 0.0f : om1;
        if (outer == 0 && q >= P.smooth_sweeps && q < P.smooth_sweeps + P.ramp_sweeps) {
          const double wr = 1.0 + (double)(q - P.smooth_sweeps + 1) / (P.ramp_sweeps + 1) * (wi - 1.0);
          w = (float)wr;
          w1 = (float)(1.0 - wr);
        }
        if (fused) {
          launch_sor32_fused(c, w, w1);
        } else if (packed) {
          launch_sor32_sweep(c, w, w1);
        } else {
          k_sor32<0><<<gcol, kBlock, 0, c->st>>>(d, c->g, c->r32, c->e32, c->cell, w, w1);
          k_sor32<1><<<gcol, kBlock, 0, c->st>>>(d, c->g, c->r32, c->e32, c->cell, w, w1);
        }
      }
      if (direct < batch) run_sor32_sweeps(c, batch - direct, om, om1);
    }
    {
      PhaseScope ps(c, PH_RESIDUAL);
      c->launches += 1;
      if (packed) launch_accumulate_packed(c);
      else k_accumulate<<<nblocks(d.n3), kBlock, 0, c->st>>>(d.n3, c->pc, c->e32);
    }
    sweeps += batch;
    ++outer;
  }
  st->sweeps = c->h_ctl->nsweeps;
  st->outer = outer;
  c->t_sweeps32 += sweeps;
  c->t_outer += outer;
  st->final_err = c->h_ctl->final_err;
  if (c->h_ctl->final_err != c->h_ctl->final_err) return IB3D_ERR_NONFINITE;
  return c->h_ctl->done == 2 ? IB3D_ERR_NOCONV : IB3D_OK;
}

}  // namespace ib3d
