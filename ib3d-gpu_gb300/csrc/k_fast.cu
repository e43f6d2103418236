// FMA-contracted FP64 kernels of the mixed-precision path (IB3D_PREC_FP32DC): the
// divergence right-hand side and the FP64 defect of the defect-correction loop.
//
// Same quantities as k_divergence and k_residual64 (k_pressure.cu): computeDiv
// (subPcorVcor.f90:82-101) and r = b/dt - A pc over the fluid cells, both still in
// FP64, but compiled with -fmad=true and with the divisions by the grid spacing and
// by dt replaced by products with reciprocals (1-D table 25 of the fast tables,
// 1/d[m]). They differ from the reference arithmetic by rounding only; the FP64
// path (IB3D_PREC_FP64) keeps the bit-identical kernels. The residual is FP64-bound
// (about 15 FP64 operations per cell without contraction, 9 with it).
#include "ib3d_internal.cuh"

namespace ib3d {

namespace {

inline unsigned nblk(long long n) { return (unsigned)((n + kBlock - 1) / kBlock); }

__device__ __forceinline__ double rtab(const double* ft, int S, int axis, int m) {
  return ft[(axis * kFastTables + 25) * S + m];
}

// b = div(ut, vt, wt) at fluid cells (0 elsewhere), b/dt, optional pc = 0, max |b|.
__global__ void __launch_bounds__(kBlock) k_divergence_fast(Dims d, const double* __restrict__ ft, int S,
                                                            const double* __restrict__ ut,
                                                            const double* __restrict__ vt,
                                                            const double* __restrict__ wt,
                                                            const unsigned char* __restrict__ cell,
                                                            double* __restrict__ b, double* __restrict__ bdt,
                                                            double* __restrict__ pc, double rdt, int zero_pc,
                                                            unsigned long long* divmax) {
  const unsigned idx = blockIdx.x * blockDim.x + threadIdx.x;
  double m = 0.0;
  if (idx < (unsigned)d.n3) {
    const unsigned nx2 = (unsigned)d.NX2, ny2 = (unsigned)d.NY2;
    const int i = (int)(idx % nx2) + 1;
    const unsigned t = idx / nx2;
    const int j = (int)(t % ny2) + 1, k = (int)(t / ny2) + 1;
    double bb = 0.0;
    if (i >= 2 && i <= d.nx + 1 && j >= 2 && j <= d.ny + 1 && k >= 2 && k <= d.nz + 1 && cell[idx] == 0) {
      const long long pl = (long long)d.NX2 * d.NY2;
      bb = (ut[idx] - ut[idx - 1]) * rtab(ft, S, 0, i);
      bb = fma(vt[idx] - vt[idx - d.NX2], rtab(ft, S, 1, j), bb);
      bb = fma(wt[idx] - wt[idx - pl], rtab(ft, S, 2, k), bb);
      m = fabs(bb);
    }
    b[idx] = bb;
    bdt[idx] = bb * rdt;
    if (zero_pc) pc[idx] = 0.0;
  }
  block_max_atomic(m, divmax);
}

// r = b/dt - A pc at fluid cells, written as the FP32 right-hand side of the inner
// solve (colour-packed arrays, or the padded r32), NaN off the fluid cells; max |r|
// decides convergence (finish_block, mode 0).
__global__ void __launch_bounds__(kBlock) k_residual_fast(Dims d, Grid1D g, const double* __restrict__ bdt,
                                                          const double* __restrict__ pc,
                                                          const unsigned char* __restrict__ cell,
                                                          float* __restrict__ r32, float* __restrict__ rp_red,
                                                          float* __restrict__ rp_black, int Lp, SolveCtl* ctl,
                                                          long long sweep, double eps, long long max_sweeps) {
  if (ctl->done) return;
  const unsigned tid = blockIdx.x * blockDim.x + threadIdx.x;
  double m = 0.0;
  if (tid < (unsigned)d.nx * (unsigned)d.ny * (unsigned)d.nz) {
    const int i = (int)(tid % (unsigned)d.nx) + 2;
    const unsigned t = tid / (unsigned)d.nx;
    const int j = (int)(t % (unsigned)d.ny) + 2, k = (int)(t / (unsigned)d.ny) + 2;
    const long long idx = d.at(i, j, k);
    float rr = __int_as_float(0x7fc00000);
    if (cell[idx] == 0) {
      const long long sy = d.NX2, sz = (long long)d.NX2 * d.NY2;
      double s = g.acx[0][i - 1] * pc[idx - 1];
      s = fma(g.acx[2][i - 1], pc[idx + 1], s);
      s = fma(g.acy[0][j - 1], pc[idx - sy], s);
      s = fma(g.acy[2][j - 1], pc[idx + sy], s);
      s = fma(g.acz[0][k - 1], pc[idx - sz], s);
      s = fma(g.acz[2][k - 1], pc[idx + sz], s);
      s = fma(g.acx[1][i - 1] + g.acy[1][j - 1] + g.acz[1][k - 1], pc[idx], s);
      const double r = bdt[idx] - s;
      m = fabs(r);
      rr = (float)r;
    }
    if (rp_red) {
      const long long sp = ((long long)(k - 1) * d.NY2 + (j - 1)) * Lp + ((i - 2) >> 1) + 4;
      (((i + j + k) & 1) ? rp_red : rp_black)[sp] = rr;
    } else {
      r32[idx] = rr;
    }
  }
  block_max_atomic(m, &ctl->res);
  finish_block(ctl, &ctl->res, 0, sweep, eps, max_sweeps);
}

// r = ((b/dt) - A pc) / diag(A) at the fluid cells (the FP64 residual of the defect
// correction, scaled as one Jacobi update and rounded to FP32), 0 elsewhere: the
// previous correction's residual against this step's right-hand side, taken before
// the guess is replaced; an input of the learned warm start (unet.cu). Dividing by
// the diagonal takes out the local grid spacing (A ~ 1/h^2), so the input means the
// same on the fine core and the stretched far field.
__global__ void __launch_bounds__(kBlock) k_hist_residual(Dims d, Grid1D g, const double* __restrict__ bdt,
                                                          const double* __restrict__ pc,
                                                          const unsigned char* __restrict__ cell,
                                                          float* __restrict__ r) {
  const unsigned tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= (unsigned)d.n3) return;
  const int i = (int)(tid % (unsigned)d.NX2);
  const unsigned t = tid / (unsigned)d.NX2;
  const int j = (int)(t % (unsigned)d.NY2), k = (int)(t / (unsigned)d.NY2);
  float out = 0.f;
  if (i >= 1 && i <= d.nx && j >= 1 && j <= d.ny && k >= 1 && k <= d.nz && cell[tid] == 0) {
    // padded index (i, j, k) 0-based is the 1-based cell (i+1, j+1, k+1)
    const long long idx = tid, sy = d.NX2, sz = (long long)d.NX2 * d.NY2;
    const double diag = g.acx[1][i] + g.acy[1][j] + g.acz[1][k];
    double s = g.acx[0][i] * pc[idx - 1];
    s = fma(g.acx[2][i], pc[idx + 1], s);
    s = fma(g.acy[0][j], pc[idx - sy], s);
    s = fma(g.acy[2][j], pc[idx + sy], s);
    s = fma(g.acz[0][k], pc[idx - sz], s);
    s = fma(g.acz[2][k], pc[idx + sz], s);
    s = fma(diag, pc[idx], s);
    out = (float)(bdt[idx] - s) / (float)diag;
  }
  r[tid] = out;
}

}  // namespace

void net_hist_residual(ib3d_ctx* c) {
  k_hist_residual<<<nblk(c->d.n3), kBlock, 0, c->st>>>(c->d, c->g, c->bdt, c->pc, c->cell, c->r_hist);
  c->launches += 1;
}

void launch_divergence_fast(ib3d_ctx* c, bool zero_pc) {
  PhaseScope ps(c, PH_DIVERGENCE);
  c->launches += 1;
  k_divergence_fast<<<nblk(c->d.n3), kBlock, 0, c->st>>>(c->d, c->d_fast, c->fast_stride, c->ut, c->vt, c->wt,
                                                         c->cell, c->b, c->bdt, c->pc, 1.0 / c->prm.deltat,
                                                         zero_pc ? 1 : 0, &c->ctl->aux);
}

void launch_residual_fast(ib3d_ctx* c, long long sweep) {
  const Dims& d = c->d;
  const bool packed = c->prm.sweep_kernel == 0 && c->ep[0] != nullptr;
  c->launches += 1;
  k_residual_fast<<<nblk((long long)d.nx * d.ny * d.nz), kBlock, 0, c->st>>>(
      d, c->g, c->bdt, c->pc, c->cell, packed ? nullptr : c->r32, packed ? c->rp[0] : nullptr,
      packed ? c->rp[1] : nullptr, c->packed_lp, c->ctl, sweep, c->prm.eps, c->prm.max_sweeps);
}

}  // namespace ib3d
