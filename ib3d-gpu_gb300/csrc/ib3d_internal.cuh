// Internal declarations shared by the IB3D CUDA translation units.
//
// Device layout (one context = one grid on one GPU, everything resident in HBM):
//   * 3-D FP64 fields u,v,w,ut,vt,wt,p,pc,b,bdt in the reference's Fortran layout
//     (nx+2, ny+2, nz+2), i fastest, so that upload/download are plain copies.
//   * cell flags as uint8 (0 fluid, 1 solid, 2 immersed-boundary) in the same layout,
//     and an int32 map from a cell to its immersed-boundary index (-1 elsewhere).
//   * 1-D grid tables (coordinates, spacings, Poisson and convection coefficients,
//     plus 1-D quotients the kernels would otherwise recompute per cell).
//   * FP32 scratch e32/r32 for the mixed-precision pressure solve.
//   * per-immersed-boundary-cell geometry and the ghost-point schedule.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/ib3d.h"

namespace ib3d {

constexpr int kBlock = 256;
constexpr int kFastTables = 46;   // 1-D tables per axis of the fast kernels (k_momentum_fast.cu, k_fast.cu)

// Index helpers: 1-based Fortran (i,j,k) into the padded column-major array.
struct Dims {
  int nx, ny, nz;      // interior cells
  int NX2, NY2, NZ2;   // padded extents
  long long n3;        // padded cell count
  __host__ __device__ __forceinline__ long long at(int i, int j, int k) const {
    return (long long)(i - 1) + (long long)NX2 * ((long long)(j - 1) + (long long)NY2 * (long long)(k - 1));
  }
};

// 1-D device tables; every pointer is 1-based (element 0 unused) unless noted.
struct Grid1D {
  const double *x1, *y1, *z1, *dx, *dy, *dz;
  const double *xu, *yu, *zu, *xv, *yv, *zv, *xw, *yw, *zw, *xp, *yp, *zp;
  // Poisson coefficients, 1-based by interior index (Acx(i-1,c) of the reference
  // is acx[c][i-1]); [0..2] = columns 1..3.
  const double *acx[3], *acy[3], *acz[3];
  const float *acx32[3], *acy32[3], *acz32[3];
  // x coefficients regrouped for the colour-packed sweep: axp[s][c][q] holds column c
  // of Acx at the four cells i = (2+s) + 8q + {0,2,4,6} (s = 0 rows whose colour
  // starts at i = 2, s = 1 at i = 3), as FP32 float4; columns c = 0 and 2 (the
  // off-diagonal ones) are stored negated
  const float4* axp[2][3];
  // acz32[0..2][m] as one float4 per plane (w = 0), for the colour-packed sweep
  const float4* acz4;
  // convection tables cc[fam][m], fam 0 uu,1 vv,2 ww,3 uv(=uw),4 vu(=vw),5 wu(=wv)
  const double* cc[6][12];
  // velocity-correction factor deltat/(0.5*(d(i+1)+d(i))) per axis
  const double *corx, *cory, *corz;
};

// RMS over the fluid cells of each network input -- pc^{n-1} = p^{n-1} - p^{n-2},
// b/dt, p^{n-1}, r/diag -- and their reciprocals; valid = 0 while any of them is 0
// (then the network is not used and pc keeps the previous correction).
struct NetNorm {
  double s1, s2, s3, s4;
  double r1, r2, r3, r4;
  int valid;
};

// Shared control block of the sweep loop; lives in device memory.
struct SolveCtl {
  unsigned long long upd;     // max |delta pc| of the running sweep (bit pattern, >= 0)
  unsigned long long res;     // max |residual| of the running check (bit pattern)
  unsigned long long aux;     // divmax / derrStdSt accumulator (bit pattern)
  unsigned int tickets;       // finished-block counter of the deciding kernel
  int done;                   // 0 running, 1 converged, 2 sweep cap reached
  long long nsweeps;          // sweep at which the loop stopped
  double final_err;           // stopping-test value at that sweep
  double last_res;            // last residual measured
  int stage_err;              // a staged sweep's bulk-copy wait gave up (the pass's results are invalid)
};

// Body motion seen by the forcing: the surface velocity (usurf, vsurf, wsurf of
// subForcing.f90:144-145, 228-229, 312-313, 397-398, 482-483, 566-567, set to the
// body velocity instead of 0) and the acceleration term of dpdn (:20), per axis
// acc[q] = -(v_curr - v_prev)/deltat. moving = 0 keeps the reference's fixed body.
struct Motion {
  int moving;
  double vel[3];
  double acc[3];
};

// Per-op data of the ghost-point schedule. An op is one ghost value: six per
// immersed-boundary cell for the velocity (blocks U2,U1,V2,V1,W2,W1 in
// subForcing.f90's order) and one for the pressure.
struct ForceSched {
  int nops;
  int nlevels;
  int* order;        // op ids sorted by level (device)
  std::vector<int> level_off;  // host: start of each level in `order`, size nlevels+1
  int* rd_idx;       // 8 linear read indices per op (device)
  int* rd_src;       // 8 sources per op: op id that wrote it earlier, or -1 (device)
  int* tgt;          // linear target index per op (device)
  int* brk;          // 3 bracket indices per op (device)
  unsigned char* fin;// 1 if the op is the last writer of its target (device)
  double* out;       // ghost value per op (device)
  int* final_ops;    // ops with fin = 1 (device)
  int nfinal;
};

}  // namespace ib3d

struct ib3d_net;

struct ib3d_ctx {
  ib3d::Dims d;
  ib3d_params prm;
  cudaStream_t st = nullptr;
  // streams the host transfers of ib3d_download_fields spread over (created on first
  // use), and the event that orders them after the work on st
  cudaStream_t xfer[3] = {nullptr, nullptr, nullptr};
  cudaEvent_t xfer_ready = nullptr;
  // ib3d_download_fields_async: device snapshot of the seven fields (allocated on first
  // use), the event after the snapshot, one event per transfer stream after its host
  // copies, and whether such copies may still be in flight
  double* stage = nullptr;
  cudaEvent_t staged = nullptr;
  cudaEvent_t xfer_done[3] = {nullptr, nullptr, nullptr};
  bool async_pending = false;
  int device = 0;
  std::string err;

  // host copies of the 1-D tables (1-based std::vectors)
  std::vector<double> hx1, hy1, hz1, hdx, hdy, hdz;
  std::vector<double> hxu, hyu, hzu, hxv, hyv, hzv, hxw, hyw, hzw, hxp, hyp, hzp;
  std::vector<double> hac[3][3];
  std::vector<double> hcc[6][12];

  // device storage
  double* d_tables = nullptr;  // all 1-D FP64 tables in one allocation
  double* d_fast = nullptr;    // 3 x kFastTables 1-D tables of the fast momentum kernel
  int fast_stride = 0;
  float* d_tables32 = nullptr;
  float* d_axp = nullptr;      // grouped x coefficients of the colour-packed sweep
  ib3d::Grid1D g{};
  double *u = nullptr, *v = nullptr, *w = nullptr, *ut = nullptr, *vt = nullptr, *wt = nullptr;
  double *p = nullptr, *pc = nullptr, *b = nullptr, *bdt = nullptr;
  // resi_u/v/w: the previous step's convection-diffusion residual (nsMomentumAB), kept
  // only when ib3d_params.momentum is IB3D_MOMENTUM_AB2
  double* resi[3] = {nullptr, nullptr, nullptr};
  float *e32 = nullptr, *r32 = nullptr;
  // omega/diag(A) per fluid cell (0 elsewhere) for the fast plain FP64 sweep
  // (IB3D_PREC_FP64_FAST); allocated on its first solve, refilled at every solve
  double* wdiag = nullptr;
  // colour-packed FP32 arrays of the inner solve ([0] red, [1] black); see k_sor32.cu
  float* ep[2] = {nullptr, nullptr};
  float* rp[2] = {nullptr, nullptr};
  // second pair of colour-packed corrections for the fused sweep (sweep_kernel 2): each
  // sweep reads ep[] and writes epn[], then the pairs swap
  float* epn[2] = {nullptr, nullptr};
  // CUDA graph of kGraphSweeps FP32 sweeps of the colour-packed kernels (k_sor32.cu),
  // with the tables, relaxation and kernel choice it was captured with
  cudaGraphExec_t sweep_exec = nullptr;
  ib3d::Grid1D sweep_g{};
  float sweep_w = 0.f, sweep_w1 = 0.f;
  int sweep_kern = -1;
  bool sweep_graph_failed = false;   // capture refused once: the sweeps launch one by one
  int packed_lp = 0;
  unsigned char* cell = nullptr;
  int* ibmap = nullptr;
  ib3d::SolveCtl* ctl = nullptr;
  ib3d::SolveCtl* h_ctl = nullptr;  // pinned mirror

  // surface mesh
  long long nnodes = 0, nelems = 0, inor = 1;
  double* d_nodes = nullptr;  // 3*nnodes shifted node coordinates (x block, y block, z block)
  int* d_tri = nullptr;       // 3*nelems 1-based node ids
  double* d_surf = nullptr;   // 9*nelems: xc,yc,zc,cosA,cosB,cosG,alpha3,beta3,gamma3
  ib3d::Motion motion{};      // prescribed body motion (ib3d_move_body)
  double bprev[3] = {0, 0, 0};

  // search results
  bool searched = false;
  bool retag_ok = false;            // an IB list of this mesh exists (ib3d_selective_retag may run)
  unsigned char* d_retag_mask = nullptr;  // selectiveRetagging: neighbourhood mask over their bounding box
  int* d_retag_list = nullptr;            // and the marked cells (i, j, k blocks)
  size_t retag_cap = 0;
  long long retagged = 0;                 // cells tagged by the last selective retag
  long long counts[5] = {0, 0, 0, 0, 0};
  int nib = 0;
  int* d_iblist = nullptr;    // 3*nib (i block, j block, k block), 1-based
  int* d_nelp = nullptr;      // nib, 1-based element ids
  double* d_nd = nullptr;     // 7*nib normal distances (p,u1,u2,v1,v2,w1,w2)
  int* d_minel = nullptr;     // box-sized nearest element
  long long box[6] = {0, 0, 0, 0, 0, 0};

  ib3d::ForceSched fv{};  // velocity ghost points
  ib3d::ForceSched fp{};  // pressure ghost points

  // drag/lift
  bool have_scache = false;
  int* d_scache = nullptr;     // 15*nelems: cell, u, v, w, p brackets (3 each)
  double* d_contrib = nullptr; // 7*nelems per-element terms
  double* d_coef = nullptr;    // 4 coefficients
  int* d_flag = nullptr;       // device error flag (probe out of grid)

  // reduction / scan scratch
  long long* d_scan = nullptr;
  size_t scan_cap = 0;

  // previous pressures for the learned warm start: hist[0] = p^{n-1}, hist[1] = p^{n-2}
  double* hist[2] = {nullptr, nullptr};
  int hist_valid = 0;
  // residual of the previous correction against this step's right-hand side divided
  // by the diagonal (FP32, padded layout, 0 off the fluid cells), kept for the
  // network and for capture
  float* r_hist = nullptr;
  // the network inputs' normalisation of this step (device; written with r_hist) and
  // the per-block partial sums it is reduced from
  ib3d::NetNorm* d_norm = nullptr;
  double* d_norm_part = nullptr;
  ib3d_net* net = nullptr;

  // phase timers (ib3d_timers_*) and the launch counter
  bool timing = false;
  struct EvPair {
    int phase;
    cudaEvent_t a, b;
  };
  std::vector<EvPair> pending;
  std::vector<cudaEvent_t> pool;
  double tms[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  long long t_sweeps64 = 0, t_sweeps32 = 0, t_outer = 0, t_steps = 0, t_launches32 = 0;
  long long launches = 0;
};

// ---- kernel launchers (defined in the .cu files) ----
namespace ib3d {
// k_pressure.cu
void launch_divergence(ib3d_ctx* c, bool zero_pc);
// k_fast.cu: FMA-contracted FP64 kernels of the IB3D_PREC_FP32DC path
void launch_divergence_fast(ib3d_ctx* c, bool zero_pc);
void launch_residual_fast(ib3d_ctx* c, long long sweep);
void launch_bdt(ib3d_ctx* c, bool zero_pc);
int run_sor_fp64(ib3d_ctx* c, ib3d_solve_stats* st);
int run_sor_fp64_fast(ib3d_ctx* c, ib3d_solve_stats* st);
int run_sor_fp32dc(ib3d_ctx* c, ib3d_solve_stats* st);
void launch_correct(ib3d_ctx* c);
void launch_velocity_bc(ib3d_ctx* c);
void launch_calculate_uc(ib3d_ctx* c);
void launch_solid_bc(ib3d_ctx* c);
void launch_dss_copy(ib3d_ctx* c);
void launch_initial(ib3d_ctx* c);
// k_momentum.cu, k_momentum_fast.cu
void launch_momentum(ib3d_ctx* c, bool ab2);
void launch_momentum_fast(ib3d_ctx* c, bool ab2);
// k_sor32.cu
int packed_row_length(int nx);
void launch_sor32_packed(ib3d_ctx* c, int color, float omega, float om1);
void launch_sor32_sweep(ib3d_ctx* c, float omega, float om1);
void run_sor32_sweeps(ib3d_ctx* c, int n, float omega, float om1);
void launch_accumulate_packed(ib3d_ctx* c);
void launch_sor32_fused(ib3d_ctx* c, float omega, float om1);
bool fused_sweep_fits(int nx);
// k_ib.cu
int run_surface_norm(ib3d_ctx* c);
int run_search(ib3d_ctx* c);
int run_selective_retag(ib3d_ctx* c);
int run_velocity_forcing(ib3d_ctx* c);
int run_pressure_forcing(ib3d_ctx* c);
int run_stress(ib3d_ctx* c, int first, double coef[4]);

int run_move_body(ib3d_ctx* c, double dx, double dy, double dz);
// unet.cu: pc = the attached network's prediction; nonzero when not available yet
int net_predict_pc(ib3d_ctx* c);
// unet.cu: after a step's synchronisation, records a convolution that gave up (the
// step then used the previous correction) in the network's error string
void net_note_failure(ib3d_ctx* c);
// k_fast.cu: r_hist = ((b/dt) - A pc) / diag(A) for the current pc, and the inputs'
// normalisation (NetNorm) from it, both on the device
void net_hist_residual(ib3d_ctx* c);
// blocks of the k_hist_residual launch (one partial-sum row each)
long long net_norm_blocks(const ib3d_ctx* c);

// error helper: records the message and returns IB3D_ERR_CUDA
int cuda_fail(ib3d_ctx* c, cudaError_t e, const char* where);

// Phase indices of ib3d_timers.ms
enum Phase { PH_MOMENTUM = 0, PH_BC, PH_FORCING, PH_DIVERGENCE, PH_SOR64, PH_SOR32, PH_RESIDUAL, PH_CORRECT,
             PH_STRESS, PH_NET };
cudaEvent_t timer_event(ib3d_ctx* c);
void timer_push(ib3d_ctx* c, int phase, cudaEvent_t a, cudaEvent_t b);
// Records a start event on construction and an end event on destruction when the
// context's timers are on; otherwise does nothing.
struct PhaseScope {
  ib3d_ctx* c;
  int ph;
  cudaEvent_t a = nullptr;
  PhaseScope(ib3d_ctx* c_, int ph_) : c(c_), ph(ph_) {
    if (c->timing) {
      a = timer_event(c);
      cudaEventRecord(a, c->st);
    }
  }
  ~PhaseScope() {
    if (a) {
      cudaEvent_t b = timer_event(c);
      cudaEventRecord(b, c->st);
      timer_push(c, ph, a, b);
    }
  }
};
}  // namespace ib3d

#define IB3D_CUDA(c, expr)                                            \
  do {                                                                \
    cudaError_t _e = (expr);                                          \
    if (_e != cudaSuccess) return ib3d::cuda_fail((c), _e, #expr);    \
  } while (0)

// ---- device helpers ----
namespace ib3d {
// max that keeps a NaN (fmax would drop it), so that a NaN in a convergence
// scalar reaches the host check instead of reading as "converged".
__device__ __forceinline__ double nan_max(double a, double b) {
  return (a != a) ? a : ((b > a || b != b) ? b : a);
}
// Block-wide max of a non-negative double (an fabs result, or a NaN from one), then
// one atomicMax on its bit pattern. For non-negative IEEE doubles the unsigned order
// of the bit patterns is the numeric order, and a NaN with the sign bit clear orders
// above +inf, so the max is exact, a NaN still reaches the host check, and the
// reduction runs on the integer units rather than the FP64 pipe (on this part the
// FP64 compares of a floating-point reduction cost as much as a stencil's FMAs).
__device__ __forceinline__ unsigned long long warp_max_bits(unsigned long long v) {
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long w = __shfl_down_sync(0xffffffffu, v, o);
    v = w > v ? w : v;
  }
  return v;
}
__device__ __forceinline__ void block_max_atomic(double v, unsigned long long* slot) {
  __shared__ unsigned long long sm[32];
  const unsigned long long b = warp_max_bits((unsigned long long)__double_as_longlong(v));
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) sm[wid] = b;
  __syncthreads();
  if (wid == 0) {
    const int nw = (int)((blockDim.x * blockDim.y * blockDim.z + 31) >> 5);
    unsigned long long x = lane < nw ? sm[lane] : 0ull;
    x = warp_max_bits(x);
    if (lane == 0 && x != 0ull) atomicMax(slot, x);
  }
}
__device__ __forceinline__ double bits_to_double(unsigned long long b) { return __longlong_as_double((long long)b); }

// The finishing step shared by every kernel that ends a sweep or a check: the
// last block to retire reads the accumulated maximum, applies the stopping test
// (continue while err >= eps, subPcorVcor.f90:210) and the sweep cap, and resets
// the accumulator. Returns nothing; the decision lands in ctl for the next kernel
// and for the host.
__device__ __forceinline__ void finish_block(SolveCtl* ctl, unsigned long long* acc, int mode, long long sweep,
                                             double eps, long long max_sweeps) {
  // mode 0: test acc against eps, then the cap; 1: only the cap; 2: no decision
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned nb = gridDim.x * gridDim.y * gridDim.z;
    const unsigned ticket = atomicAdd(&ctl->tickets, 1u);
    if (ticket == nb - 1) {
      __threadfence();
      const double err = bits_to_double(atomicExch(acc, 0ull));
      ctl->tickets = 0;
      if (mode == 0) {
        ctl->last_res = err;
        if (!(err >= eps)) {
          ctl->done = 1; ctl->nsweeps = sweep; ctl->final_err = err;
        } else if (sweep >= max_sweeps) {
          ctl->done = 2; ctl->nsweeps = sweep; ctl->final_err = err;
        }
      } else if (mode == 1) {
        if (sweep >= max_sweeps) { ctl->done = 2; ctl->nsweeps = sweep; ctl->final_err = ctl->last_res; }
      }
      __threadfence();
    }
  }
}

// The FP32 SOR update shared by every FP32 sweep kernel: e <- (1-omega) e +
// omega num / diag, the quotient as a product with the hardware's approximate
// reciprocal (rcp.approx.ftz.f32, one instruction) instead of the IEEE division's
// sequence. diag is the sum of three positive Poisson diagonal entries, a normal
// number far from the range limits, so the reciprocal needs no range handling. The
// FP32 sweeps only precondition the FP64 defect correction, whose FP64 residual
// decides convergence, so the quotient's last-bit rounding does not reach the result.
__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ float sor32_update(float e, float num, float diag, float omega, float om1) {
  return fmaf(om1, e, (omega * num) * rcp_approx(diag));
}
}  // namespace ib3d
