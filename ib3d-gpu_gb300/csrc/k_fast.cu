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
    } else if (r32) {   // neither: a convergence check of the fast plain FP64 path
      r32[idx] = rr;
    }
  }
  block_max_atomic(m, &ctl->res);
  finish_block(ctl, &ctl->res, 0, sweep, eps, max_sweeps);
}

// omega/diag(A) at the fluid cells, 0 elsewhere: the factor of the fast plain FP64
// sweep, one IEEE division per cell per solve instead of one per cell per sweep.
__global__ void __launch_bounds__(kBlock) k_wdiag(Dims d, Grid1D g, const unsigned char* __restrict__ cell,
                                                  double omega, double* __restrict__ wd) {
  const unsigned tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= (unsigned)d.n3) return;
  const int i = (int)(tid % (unsigned)d.NX2) + 1;
  const unsigned t = tid / (unsigned)d.NX2;
  const int j = (int)(t % (unsigned)d.NY2) + 1, k = (int)(t / (unsigned)d.NY2) + 1;
  double w = 0.0;
  if (i >= 2 && i <= d.nx + 1 && j >= 2 && j <= d.ny + 1 && k >= 2 && k <= d.nz + 1 && cell[tid] == 0)
    w = omega / (g.acx[1][i - 1] + g.acy[1][j - 1] + g.acz[1][k - 1]);
  wd[tid] = w;
}

// One colour of the fast plain FP64 sweep (IB3D_PREC_FP64_FAST): REDBLACKSOR's
// update (subPcorVcor.f90:164-191), pc <- (1-omega) pc + omega (b/dt - sum A_nb
// pc_nb) / diag, as six contracted multiply-adds, one product and one multiply-add
// with wd = omega/diag (8 FP64 operations a cell against the reference
// arithmetic's ~18 and a division). Red cells are (i+j+k) odd (subSearch.f90:562);
// each thread owns one (i, i+1) pair of a row. DELTA: the update norm max |pc_new -
// pc_old| (IB3D_CRIT_UPDATE) is reduced on chip and decided after the black pass;
// the residual test needs no update norm, so that form skips it.
template <int COLOR, bool DELTA>
__global__ void __launch_bounds__(kBlock) k_sor64_fast(Dims d, Grid1D g, const double* __restrict__ bdt,
                                                       const double* __restrict__ wd, double* __restrict__ pc,
                                                       double om1, SolveCtl* ctl, long long sweep,
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
      const double w = wd[idx];
      if (w != 0.0) {
        const long long sy = d.NX2, sz = (long long)d.NX2 * d.NY2;
        double num = fma(-g.acx[0][i - 1], pc[idx - 1], bdt[idx]);
        num = fma(-g.acx[2][i - 1], pc[idx + 1], num);
        num = fma(-g.acy[0][j - 1], pc[idx - sy], num);
        num = fma(-g.acy[2][j - 1], pc[idx + sy], num);
        num = fma(-g.acz[0][k - 1], pc[idx - sz], num);
        num = fma(-g.acz[2][k - 1], pc[idx + sz], num);
        const double old = pc[idx];
        const double nw = fma(w, num, om1 * old);
        pc[idx] = nw;
        if (DELTA) delta = fabs(nw - old);
      }
    }
  }
  if (DELTA) block_max_atomic(delta, &ctl->upd);
  if (COLOR == 1) finish_block(ctl, &ctl->upd, decide_mode, sweep, eps, max_sweeps);
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

// Sums over the fluid cells of (h1-h2)^2, (b/dt)^2, h1^2, (r/diag)^2 and their
// count, for the network inputs' RMS. Grid (ceil(nx/256), ny, ceil(nz/kNormPlanes)):
// a thread accumulates kNormPlanes cells of one column in FP64 (one FMA per sum and
// cell), the warp adds its threads' sums in FP32 and the block its warps' in FP64,
// one partial row per block, in a fixed order.
constexpr int kNormPlanes = 8;
__global__ void __launch_bounds__(kBlock) k_norm_sums(Dims d, const unsigned char* __restrict__ cell,
                                                      const double* __restrict__ h1, const double* __restrict__ h2,
                                                      const double* __restrict__ bdt, const float* __restrict__ r,
                                                      double* __restrict__ partial) {
  static_assert(kBlock == 256, "the block reduction below assumes 8 warps");
  __shared__ double sm[8][5];
  const int i = blockIdx.x * kBlock + threadIdx.x + 2, j = blockIdx.y + 2, k0 = blockIdx.z * kNormPlanes + 2;
  double a0 = 0.0, a1 = 0.0, a2 = 0.0;
  float a3 = 0.f, a4 = 0.f;
  if (i <= d.nx + 1) {
#pragma unroll
    for (int kk = 0; kk < kNormPlanes; ++kk) {
      const int k = k0 + kk;
      if (k > d.nz + 1) break;
      const long long o = d.at(i, j, k);
      if (cell[o] == 0) {
        const double p1 = h1[o], b = bdt[o], dp = p1 - h2[o];
        const float rr = r[o];
        a0 = fma(dp, dp, a0);
        a1 = fma(b, b, a1);
        a2 = fma(p1, p1, a2);
        a3 = fmaf(rr, rr, a3);
        a4 += 1.f;
      }
    }
  }
  float q[5] = {(float)a0, (float)a1, (float)a2, a3, a4};
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int c = 0; c < 5; ++c) {
    float x = q[c];
    for (int off = 16; off > 0; off >>= 1) x += __shfl_down_sync(0xffffffffu, x, off);
    if (lane == 0) sm[wid][c] = (double)x;
  }
  __syncthreads();
  if (threadIdx.x < 5) {
    double x = 0.0;
    for (int w = 0; w < 8; ++w) x += sm[w][threadIdx.x];
    const size_t b = ((size_t)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
    partial[b * 5 + threadIdx.x] = x;
  }
}

// Adds the per-block partial sums in a fixed order (each thread a strided set of
// rows, four at a time, then a tree over the threads), so the normalisation does not
// depend on scheduling, and writes NetNorm.
constexpr int kNormThreads = 1024;
__global__ void __launch_bounds__(kNormThreads) k_norm_final(const double* __restrict__ partial, int nblocks,
                                                             NetNorm* __restrict__ out) {
  __shared__ double sm[5][kNormThreads];
  const int t = threadIdx.x;
  double x[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  int b = t;
  for (; b + 3 * kNormThreads < nblocks; b += 4 * kNormThreads) {
    double v[4][5];
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int c = 0; c < 5; ++c) v[u][c] = partial[(size_t)(b + u * kNormThreads) * 5 + c];
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int c = 0; c < 5; ++c) x[c] += v[u][c];
  }
  for (; b < nblocks; b += kNormThreads)
#pragma unroll
    for (int c = 0; c < 5; ++c) x[c] += partial[(size_t)b * 5 + c];
#pragma unroll
  for (int c = 0; c < 5; ++c) sm[c][t] = x[c];
  __syncthreads();
  for (int s = kNormThreads / 2; s > 0; s >>= 1) {
    if (t < s)
#pragma unroll
      for (int c = 0; c < 5; ++c) sm[c][t] += sm[c][t + s];
    __syncthreads();
  }
  if (t == 0) {
    const double tot[5] = {sm[0][0], sm[1][0], sm[2][0], sm[3][0], sm[4][0]};
    NetNorm nm{};
    nm.valid = tot[0] > 0.0 && tot[1] > 0.0 && tot[2] > 0.0 && tot[3] > 0.0 && tot[4] > 0.0;
    if (nm.valid) {
      nm.s1 = sqrt(tot[0] / tot[4]);
      nm.s2 = sqrt(tot[1] / tot[4]);
      nm.s3 = sqrt(tot[2] / tot[4]);
      nm.s4 = sqrt(tot[3] / tot[4]);
      nm.r1 = 1.0 / nm.s1;
      nm.r2 = 1.0 / nm.s2;
      nm.r3 = 1.0 / nm.s3;
      nm.r4 = 1.0 / nm.s4;
    }
    *out = nm;
  }
}

}  // namespace

static dim3 norm_grid(const Dims& d) {
  return dim3((unsigned)((d.nx + kBlock - 1) / kBlock), (unsigned)d.ny,
              (unsigned)((d.nz + kNormPlanes - 1) / kNormPlanes));
}

long long net_norm_blocks(const ib3d_ctx* c) {
  const dim3 g = norm_grid(c->d);
  return (long long)g.x * g.y * g.z;
}

void net_hist_residual(ib3d_ctx* c) {
  k_hist_residual<<<nblk(c->d.n3), kBlock, 0, c->st>>>(c->d, c->g, c->bdt, c->pc, c->cell, c->r_hist);
  const dim3 g = norm_grid(c->d);
  k_norm_sums<<<g, kBlock, 0, c->st>>>(c->d, c->cell, c->hist[0], c->hist[1], c->bdt, c->r_hist, c->d_norm_part);
  k_norm_final<<<1, kNormThreads, 0, c->st>>>(c->d_norm_part, (int)(g.x * g.y * g.z), c->d_norm);
  c->launches += 3;
}

void launch_divergence_fast(ib3d_ctx* c, bool zero_pc) {
  PhaseScope ps(c, PH_DIVERGENCE);
  c->launches += 1;
  k_divergence_fast<<<nblk(c->d.n3), kBlock, 0, c->st>>>(c->d, c->d_fast, c->fast_stride, c->ut, c->vt, c->wt,
                                                         c->cell, c->b, c->bdt, c->pc, 1.0 / c->prm.deltat,
                                                         zero_pc ? 1 : 0, &c->ctl->aux);
}

// REDBLACKSOR in the fast plain FP64 form: the loop of run_sor_fp64 (batches of
// sweeps between host reads of the device-side decision; the residual test every
// check_every sweeps, or the update norm every sweep) around k_sor64_fast.
int run_sor_fp64_fast(ib3d_ctx* c, ib3d_solve_stats* st) {
  const Dims& d = c->d;
  const ib3d_params& P = c->prm;
  const unsigned gcol = nblk((((long long)d.nx + 1) / 2) * d.ny * d.nz);
  const long long ncell = (long long)d.nx * d.ny * d.nz;
  const bool resid = P.criterion == IB3D_CRIT_RESIDUAL;
  const int every = P.check_every < 1 ? 1 : P.check_every;
  if (!c->wdiag) IB3D_CUDA(c, cudaMalloc(&c->wdiag, (size_t)d.n3 * sizeof(double)));
  c->launches += 1;
  k_wdiag<<<nblk(d.n3), kBlock, 0, c->st>>>(d, c->g, c->cell, P.omega, c->wdiag);
  IB3D_CUDA(c, cudaMemsetAsync(c->ctl, 0, sizeof(SolveCtl), c->st));
  const double om1 = 1.0 - P.omega;
  long long sweep = 0, batch = 4;
  for (;;) {
    {
      PhaseScope ps(c, PH_SOR64);
      for (long long q = 0; q < batch; ++q) {
        ++sweep;
        const bool check = resid && (sweep % every) == 0;
        c->launches += check ? 3 : 2;
        if (resid) {
          k_sor64_fast<0, false><<<gcol, kBlock, 0, c->st>>>(d, c->g, c->bdt, c->wdiag, c->pc, om1, c->ctl, sweep, 2,
                                                             P.eps, P.max_sweeps);
          k_sor64_fast<1, false><<<gcol, kBlock, 0, c->st>>>(d, c->g, c->bdt, c->wdiag, c->pc, om1, c->ctl, sweep,
                                                             check ? 2 : 1, P.eps, P.max_sweeps);
          if (check)
            k_residual_fast<<<nblk(ncell), kBlock, 0, c->st>>>(d, c->g, c->bdt, c->pc, c->cell, nullptr, nullptr,
                                                               nullptr, 0, c->ctl, sweep, P.eps, P.max_sweeps);
        } else {
          k_sor64_fast<0, true><<<gcol, kBlock, 0, c->st>>>(d, c->g, c->bdt, c->wdiag, c->pc, om1, c->ctl, sweep, 2,
                                                            P.eps, P.max_sweeps);
          k_sor64_fast<1, true><<<gcol, kBlock, 0, c->st>>>(d, c->g, c->bdt, c->wdiag, c->pc, om1, c->ctl, sweep, 0,
                                                            P.eps, P.max_sweeps);
        }
      }
    }
    IB3D_CUDA(c, cudaGetLastError());
    IB3D_CUDA(c, cudaMemcpyAsync(c->h_ctl, c->ctl, sizeof(SolveCtl), cudaMemcpyDeviceToHost, c->st));
    IB3D_CUDA(c, cudaStreamSynchronize(c->st));
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

void launch_residual_fast(ib3d_ctx* c, long long sweep) {
  const Dims& d = c->d;
  // the colour-packed sweeps (kernels 0 and 2) read the packed right-hand side
  const bool packed = c->prm.sweep_kernel != 1 && c->ep[0] != nullptr;
  c->launches += 1;
  k_residual_fast<<<nblk((long long)d.nx * d.ny * d.nz), kBlock, 0, c->st>>>(
      d, c->g, c->bdt, c->pc, c->cell, packed ? nullptr : c->r32, packed ? c->rp[0] : nullptr,
      packed ? c->rp[1] : nullptr, c->packed_lp, c->ctl, sweep, c->prm.eps, c->prm.max_sweeps);
}

}  // namespace ib3d
