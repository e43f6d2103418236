// Pressure solve that allocates no memory.
//
// Some host codes that would call this library cannot call cudaMalloc: a Fortran
// or C++ solver whose device memory is owned by another runtime (an OpenACC data
// region, a framework's caching allocator, a fixed memory pool sized at start-up),
// a code that must not allocate inside its time loop for latency or fragmentation
// reasons, or one that runs where allocation is forbidden. They hold their arrays
// already and only need the solve. ib3d_pressure_solve_noalloc takes every input
// and output as a device pointer the caller owns, and keeps its own scratch (the
// FP32 right-hand side and correction of the inner sweeps, and the loop's control
// block) in one file-scope __device__ array that the library image carries, so the
// call performs no allocation of any kind.
//
// The solve is the library's mixed-precision pressure solve: FP64 defect
// correction around FP32 red-black sweeps, stopped at an FP64 residual L-inf
// tolerance, with the same arithmetic as ib3d_poisson_solver's IB3D_PREC_FP32DC
// mode (two-launch sweep form).
#include <mutex>

#include "ib3d_internal.cuh"

namespace ib3d {
namespace {

// Largest padded grid, (nx+2)*(ny+2)*(nz+2), the scratch can hold: 2^21 cells
// (for example 126^3), i.e. two FP32 arrays of 8 MiB each plus the control block.
constexpr long long kMaxCells = 1ll << 21;
constexpr size_t kArrayBytes = (size_t)kMaxCells * sizeof(float);
constexpr size_t kCtlOffset = 2 * kArrayBytes;
constexpr size_t kScratchBytes = kCtlOffset + 256;

// The scratch itself. Every GPU that loads the library holds it until the process
// exits. In host code this name is only a host-side stand-in for the device
// object, so host code never passes it to a kernel: it passes the device address
// obtained once per device with cudaGetSymbolAddress (below).
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_mu;
constexpr int kMaxDevices = 64;
unsigned char* g_addr[kMaxDevices] = {};

// Device address of the scratch on the current device, looked up on the first
// call made on that device and cached. A call that meets any CUDA error drops the
// cached address (forget_scratch_address), so the next call looks it up again.
cudaError_t scratch_on_current_device(unsigned char** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_addr[dev] = static_cast<unsigned char*>(p);
  }
  *out = g_addr[dev];
  return cudaSuccess;
}

void forget_scratch_address() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return;
  std::lock_guard<std::mutex> lock(g_mu);
  g_addr[dev] = nullptr;
}

struct Coefs {  // the caller's (n,3) column-major Acx/Acy/Acz (device)
  const double *ax, *ay, *az;
  int nx, ny, nz;
  __device__ __forceinline__ double x(int c, int m) const { return ax[(m - 1) + nx * c]; }
  __device__ __forceinline__ double y(int c, int m) const { return ay[(m - 1) + ny * c]; }
  __device__ __forceinline__ double z(int c, int m) const { return az[(m - 1) + nz * c]; }
};

__device__ __forceinline__ void decide(SolveCtl* ctl, long long sweeps, double eps, long long max_sweeps) {
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned ticket = atomicAdd(&ctl->tickets, 1u);
    if (ticket == gridDim.x - 1) {
      __threadfence();
      const double err = bits_to_double(atomicExch(&ctl->res, 0ull));
      ctl->tickets = 0;
      ctl->last_res = err;
      if (!(err >= eps)) { ctl->done = 1; ctl->nsweeps = sweeps; ctl->final_err = err; }
      else if (sweeps >= max_sweeps) { ctl->done = 2; ctl->nsweeps = sweeps; ctl->final_err = err; }
      __threadfence();
    }
  }
}

// r = b/dt - A pc on fluid cells (FP64), its maximum, and r rounded to FP32.
__global__ void k_na_residual(Dims d, Coefs A, const double* __restrict__ b, double deltat,
                              const double* __restrict__ pc, const unsigned char* __restrict__ cell,
                              float* __restrict__ r32, SolveCtl* ctl, long long sweeps, double eps,
                              long long max_sweeps) {
  const unsigned tid = blockIdx.x * blockDim.x + threadIdx.x;
  double m = 0.0;
  if (tid < (unsigned)d.nx * (unsigned)d.ny * (unsigned)d.nz) {
    const int i = (int)(tid % (unsigned)d.nx) + 2;
    const unsigned t = tid / (unsigned)d.nx;
    const int j = (int)(t % (unsigned)d.ny) + 2, k = (int)(t / (unsigned)d.ny) + 2;
    const long long idx = d.at(i, j, k);
    float rr = 0.0f;
    if (cell[idx] == 0) {
      const long long sy = d.NX2, sz = (long long)d.NX2 * d.NY2;
      const double bdt = b[idx] / deltat;
      const double num = bdt - A.x(0, i - 1) * pc[idx - 1] - A.x(2, i - 1) * pc[idx + 1] -
                         A.y(0, j - 1) * pc[idx - sy] - A.y(2, j - 1) * pc[idx + sy] -
                         A.z(0, k - 1) * pc[idx - sz] - A.z(2, k - 1) * pc[idx + sz];
      const double diag = A.x(1, i - 1) + A.y(1, j - 1) + A.z(1, k - 1);
      const double r = num - diag * pc[idx];
      m = fabs(r);
      rr = (float)r;
    }
    r32[idx] = rr;
  }
  block_max_atomic(m, &ctl->res);
  decide(ctl, sweeps, eps, max_sweeps);
}

// One colour of the FP32 red-black sweep on A e = r, in place.
template <int COLOR>
__global__ void k_na_sor32(Dims d, Coefs A, const float* __restrict__ r32, float* __restrict__ e,
                           const unsigned char* __restrict__ cell, float omega, float om1) {
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
  num = fmaf(-(float)A.x(0, i - 1), e[idx - 1], num);
  num = fmaf(-(float)A.x(2, i - 1), e[idx + 1], num);
  num = fmaf(-(float)A.y(0, j - 1), e[idx - sy], num);
  num = fmaf(-(float)A.y(2, j - 1), e[idx + sy], num);
  num = fmaf(-(float)A.z(0, k - 1), e[idx - sz], num);
  num = fmaf(-(float)A.z(2, k - 1), e[idx + sz], num);
  const float diag = (float)A.x(1, i - 1) + (float)A.y(1, j - 1) + (float)A.z(1, k - 1);
  e[idx] = sor32_update(e[idx], num, diag, omega, om1);
}

__global__ void k_na_accumulate(long long n3, double* __restrict__ pc, float* __restrict__ e) {
  const unsigned idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (unsigned)n3) return;
  const float x = e[idx];
  if (x != 0.0f) {
    pc[idx] = pc[idx] + (double)x;
    e[idx] = 0.0f;
  }
}


int run_noalloc(int64_t nx, int64_t ny, int64_t nz, const double* acx, const double* acy, const double* acz,
                const unsigned char* cell, const double* b, double deltat, double* pc, double omega, double eps,
                int64_t max_sweeps, int32_t inner_sweeps, cudaStream_t st, unsigned char* base,
                int64_t* sweeps_out, double* residual_out) {
  const long long n3 = (nx + 2) * (ny + 2) * (nz + 2);
  float* r32 = reinterpret_cast<float*>(base);
  float* e32 = reinterpret_cast<float*>(base + kArrayBytes);
  SolveCtl* ctl = reinterpret_cast<SolveCtl*>(base + kCtlOffset);
  Dims d;
  d.nx = (int)nx; d.ny = (int)ny; d.nz = (int)nz;
  d.NX2 = d.nx + 2; d.NY2 = d.ny + 2; d.NZ2 = d.nz + 2;
  d.n3 = n3;
  const Coefs A{acx, acy, acz, d.nx, d.ny, d.nz};
  // the scratch keeps the previous call's contents: the correction must start at
  // zero and the control block must be cleared
  if (cudaMemsetAsync(e32, 0, (size_t)n3 * sizeof(float), st) != cudaSuccess) return IB3D_ERR_CUDA;
  if (cudaMemsetAsync(ctl, 0, sizeof(SolveCtl), st) != cudaSuccess) return IB3D_ERR_CUDA;
  const long long ncell = (long long)nx * ny * nz;
  const unsigned gres = (unsigned)((ncell + kBlock - 1) / kBlock);
  const unsigned gcol = (unsigned)((((nx + 1) / 2) * ny * nz + kBlock - 1) / kBlock);
  const unsigned gall = (unsigned)((n3 + kBlock - 1) / kBlock);
  const float om = (float)omega, om1 = (float)(1.0 - omega);
  SolveCtl h{};
  long long sweeps = 0;
  for (;;) {
    k_na_residual<<<gres, kBlock, 0, st>>>(d, A, b, deltat, pc, cell, r32, ctl, sweeps, eps, max_sweeps);
    if (cudaGetLastError() != cudaSuccess) return IB3D_ERR_CUDA;
    if (cudaMemcpyAsync(&h, ctl, sizeof(SolveCtl), cudaMemcpyDeviceToHost, st) != cudaSuccess) return IB3D_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return IB3D_ERR_CUDA;
    if (h.done) break;
    for (int q = 0; q < inner_sweeps; ++q) {
      k_na_sor32<0><<<gcol, kBlock, 0, st>>>(d, A, r32, e32, cell, om, om1);
      k_na_sor32<1><<<gcol, kBlock, 0, st>>>(d, A, r32, e32, cell, om, om1);
    }
    k_na_accumulate<<<gall, kBlock, 0, st>>>(n3, pc, e32);
    sweeps += inner_sweeps;
  }
  if (sweeps_out) *sweeps_out = h.nsweeps;
  if (residual_out) *residual_out = h.final_err;
  if (h.final_err != h.final_err) return IB3D_ERR_NONFINITE;
  return h.done == 2 ? IB3D_ERR_NOCONV : IB3D_OK;
}
}  // namespace
}  // namespace ib3d

using namespace ib3d;

extern "C" int ib3d_pressure_solve_noalloc(int64_t nx, int64_t ny, int64_t nz, const double* acx, const double* acy,
                                           const double* acz, const unsigned char* cell, const double* b,
                                           double deltat, double* pc, double omega, double eps,
                                           int64_t max_sweeps, int32_t inner_sweeps, void* stream,
                                           int64_t* sweeps_out, double* residual_out) {
  if (nx < 4 || ny < 4 || nz < 4 || !acx || !acy || !acz || !cell || !b || !pc || !(deltat > 0) ||
      !(omega > 0 && omega < 2) || !(eps > 0) || max_sweeps < 1 || inner_sweeps < 1)
    return IB3D_ERR_ARG;
  // each extent is bounded before the product is formed, so the product cannot overflow
  if (nx > kMaxCells || ny > kMaxCells || nz > kMaxCells) return IB3D_ERR_TOO_LARGE;
  if ((nx + 2) * (ny + 2) > kMaxCells) return IB3D_ERR_TOO_LARGE;
  const long long n3 = (nx + 2) * (ny + 2) * (nz + 2);
  if (n3 > kMaxCells) return IB3D_ERR_TOO_LARGE;
  unsigned char* base = nullptr;
  if (scratch_on_current_device(&base) != cudaSuccess) {
    forget_scratch_address();
    return IB3D_ERR_CUDA;
  }
  const int rc = run_noalloc(nx, ny, nz, acx, acy, acz, cell, b, deltat, pc, omega, eps, max_sweeps, inner_sweeps,
                             static_cast<cudaStream_t>(stream), base, sweeps_out, residual_out);
  if (rc == IB3D_ERR_CUDA) forget_scratch_address();
  return rc;
}
