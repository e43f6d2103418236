// Learned warm start of the pressure solve: a 3-level 3-D U-Net (16/32/64
// channels, 3x3x3 convolutions, 2x2x2 average pooling, nearest upsampling, skip
// concatenations, 1x1 head; 0.36 M parameters) in BF16 with FP32 accumulation,
// trained with Adam on snapshots the solver generates.
//
// Inputs per cell: (p^{n-1} - p^{n-2})/s1 (the previous correction pc^{n-1}),
// (b/dt)^n/s2, p^{n-1}/s3, and r/s4 with r = ((b/dt)^n - A pc^{n-1})/diag(A) the FP64
// residual of the previous correction against this step's right-hand side;
// s1..s4 are the RMS of each over the fluid cells. Differences are taken in FP64
// before the cast to BF16, which would otherwise erase them (b/dt and A pc^{n-1}
// agree to several digits). Output: the change of the correction,
// (pc^n - pc^{n-1})/s1, so that the guess is pc^{n-1} + s1 * output: a network
// with a zero head reproduces the previous-correction warm start exactly, and the
// FP64 defect-correction loop still stops at the same FP64 residual, so a poor
// guess only costs sweeps.
#include <algorithm>
#include <cmath>
#include <random>
#include <vector>

#include "ib3d_internal.cuh"
#include "unet.cuh"

using namespace ib3d;
using namespace ib3d::unet;

namespace {

struct Layer {
  int N, K, Kreal;
  size_t w, b;   // offsets of the FP32 weights [N][27][K] and biases [N] in the parameter vector
};
constexpr int kInputs = 4;   // input channels per cell (see the file header)
// conv1a conv1b | conv2a conv2b | conv3a conv3b | conv4a conv4b | conv5a conv5b
constexpr int kL = 10;
const int kN[kL] = {16, 16, 32, 32, 64, 64, 32, 32, 16, 16};
const int kK[kL] = {16, 16, 16, 32, 32, 64, 96, 32, 48, 16};
const int kKreal[kL] = {kInputs, 16, 16, 32, 32, 64, 96, 32, 48, 16};

struct Buffers {
  Vol v1{}, v2{}, v3{};
  bool grads = false;
  std::vector<void*> owned;
  // level 1
  bf16 *in0, *a1, *cat5, *a5, *d1;
  float *out, *gout, *tgt;
  bf16 *g_a1, *g_cat5, *g_a5, *g_d1;
  // level 2
  bf16 *p1, *a2, *cat4, *a4, *d2;
  bf16 *g_p1, *g_a2, *g_cat4, *g_a4, *g_d2;
  // level 3
  bf16 *p2, *a3, *b;
  bf16 *g_p2, *g_a3, *g_b;
};

}  // namespace

struct ib3d_net {
  cudaStream_t st = nullptr;
  std::string err;
  Layer L[kL];
  size_t head = 0;     // offset of the head weights (16) and bias (1)
  size_t nparam = 0;
  float *p = nullptr, *g = nullptr, *m1 = nullptr, *m2 = nullptr;
  bf16 *wf = nullptr, *wt = nullptr;   // BF16 copies: forward [N][27][K], transposed [K][27][N]
  int step = 0;
  Buffers buf;
  int coarsen = 2;     // fine cells per coarse voxel edge (1: full resolution)
  // training set
  int S = 0;
  long long cap = 0, count = 0;
  bf16* ds_in = nullptr;   // [patch][S^3][4]
  float* ds_t = nullptr;   // [patch][S^3]
  double* d_loss = nullptr;
  int* d_err = nullptr;    // set by a convolution whose tensor-core wait gave up
  bool wgrad_cuda_cores = false;   // weight gradients on the CUDA cores (the tensor-core form's reference)
};

namespace {

int fail(ib3d_net* n, int code, const char* msg) {
  if (n) n->err = msg;
  return code;
}

// After a synchronisation: a convolution whose tensor-core wait gave up leaves its
// output invalid; report it (and keep reporting it).
int check_conv(ib3d_net* n) {
  int h = 0;
  if (cudaMemcpy(&h, n->d_err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
    return fail(n, IB3D_ERR_CUDA, "ib3d_net: reading the convolution status failed");
  return h ? fail(n, IB3D_ERR_CUDA, "ib3d_net: a tensor-core wait timed out") : IB3D_OK;
}
#define NET_CUDA(n, expr)                                                              \
  do {                                                                                 \
    cudaError_t _e = (expr);                                                           \
    if (_e != cudaSuccess) return fail((n), IB3D_ERR_CUDA, cudaGetErrorString(_e));    \
  } while (0)

void free_buffers(Buffers& b) {
  for (void* q : b.owned) cudaFree(q);
  b = Buffers{};
}

// Activation (and, for training, gradient) buffers for one input volume.
int ensure_buffers(ib3d_net* n, const Vol& v1, bool grads) {
  Buffers& b = n->buf;
  if (b.v1.B == v1.B && b.v1.D == v1.D && b.v1.H == v1.H && b.v1.W == v1.W && (b.grads || !grads)) return IB3D_OK;
  free_buffers(b);
  b.v1 = v1;
  b.v2 = {v1.B, v1.D / 2, v1.H / 2, v1.W / 2};
  b.v3 = {v1.B, v1.D / 4, v1.H / 4, v1.W / 4};
  b.grads = grads;
  const long long m1 = b.v1.voxels(), m2 = b.v2.voxels(), m3 = b.v3.voxels();
  auto alloc_bf = [&](bf16** q, long long vox, int c) -> bool {
    if (cudaMalloc(q, (size_t)vox * c * sizeof(bf16)) != cudaSuccess) return false;
    cudaMemsetAsync(*q, 0, (size_t)vox * c * sizeof(bf16), n->st);
    b.owned.push_back(*q);
    return true;
  };
  auto alloc_f = [&](float** q, long long vox) -> bool {
    if (cudaMalloc(q, (size_t)vox * sizeof(float)) != cudaSuccess) return false;
    b.owned.push_back(*q);
    return true;
  };
  bool ok = alloc_bf(&b.in0, m1, 16) && alloc_bf(&b.a1, m1, 16) && alloc_bf(&b.cat5, m1, 48) &&
            alloc_bf(&b.a5, m1, 16) && alloc_bf(&b.d1, m1, 16) && alloc_f(&b.out, m1) && alloc_bf(&b.p1, m2, 16) &&
            alloc_bf(&b.a2, m2, 32) && alloc_bf(&b.cat4, m2, 96) && alloc_bf(&b.a4, m2, 32) &&
            alloc_bf(&b.d2, m2, 32) && alloc_bf(&b.p2, m3, 32) && alloc_bf(&b.a3, m3, 64) && alloc_bf(&b.b, m3, 64);
  if (ok && grads)
    ok = alloc_f(&b.gout, m1) && alloc_f(&b.tgt, m1) && alloc_bf(&b.g_a1, m1, 16) && alloc_bf(&b.g_cat5, m1, 48) &&
         alloc_bf(&b.g_a5, m1, 16) && alloc_bf(&b.g_d1, m1, 16) && alloc_bf(&b.g_p1, m2, 16) &&
         alloc_bf(&b.g_a2, m2, 32) && alloc_bf(&b.g_cat4, m2, 96) && alloc_bf(&b.g_a4, m2, 32) &&
         alloc_bf(&b.g_d2, m2, 32) && alloc_bf(&b.g_p2, m3, 32) && alloc_bf(&b.g_a3, m3, 64) &&
         alloc_bf(&b.g_b, m3, 64);
  if (!ok) {
    free_buffers(b);
    return fail(n, IB3D_ERR_MEMORY, "ib3d_net: activation buffers");
  }
  return IB3D_OK;
}

Act A(bf16* p, int cs, int co = 0) { return Act{p, cs, co}; }

const bf16* wf(ib3d_net* n, int l) { return n->wf + n->L[l].w; }
const bf16* wt(ib3d_net* n, int l) { return n->wt + n->L[l].w; }
const float* bias(ib3d_net* n, int l) { return n->p + n->L[l].b; }

void forward(ib3d_net* n) {
  Buffers& b = n->buf;
  cudaStream_t st = n->st;
  conv(st, b.v1, A(b.in0, 16), 16, wf(n, 0), bias(n, 0), 1, 1, A(b.a1, 16), 16, n->d_err);
  conv(st, b.v1, A(b.a1, 16), 16, wf(n, 1), bias(n, 1), 1, 1, A(b.cat5, 48, 32), 16, n->d_err);   // e1
  pool_fwd(st, b.v2, 16, A(b.cat5, 48, 32), A(b.p1, 16));
  conv(st, b.v2, A(b.p1, 16), 16, wf(n, 2), bias(n, 2), 1, 1, A(b.a2, 32), 32, n->d_err);
  conv(st, b.v2, A(b.a2, 32), 32, wf(n, 3), bias(n, 3), 1, 1, A(b.cat4, 96, 64), 32, n->d_err);   // e2
  pool_fwd(st, b.v3, 32, A(b.cat4, 96, 64), A(b.p2, 32));
  conv(st, b.v3, A(b.p2, 32), 32, wf(n, 4), bias(n, 4), 1, 1, A(b.a3, 64), 64, n->d_err);
  conv(st, b.v3, A(b.a3, 64), 64, wf(n, 5), bias(n, 5), 1, 1, A(b.b, 64), 64, n->d_err);
  up_fwd(st, b.v2, 64, A(b.b, 64), A(b.cat4, 96, 0));
  conv(st, b.v2, A(b.cat4, 96), 96, wf(n, 6), bias(n, 6), 1, 1, A(b.a4, 32), 32, n->d_err);
  conv(st, b.v2, A(b.a4, 32), 32, wf(n, 7), bias(n, 7), 1, 1, A(b.d2, 32), 32, n->d_err);
  up_fwd(st, b.v1, 32, A(b.d2, 32), A(b.cat5, 48, 0));
  conv(st, b.v1, A(b.cat5, 48), 48, wf(n, 8), bias(n, 8), 1, 1, A(b.a5, 16), 16, n->d_err);
  conv(st, b.v1, A(b.a5, 16), 16, wf(n, 9), bias(n, 9), 1, 1, A(b.d1, 16), 16, n->d_err);
  head_fwd(st, b.v1.voxels(), 16, A(b.d1, 16), n->p + n->head, b.out);
}

// Backward of conv layer l with output Y (gradient gY, overwritten by the ReLU
// mask) and input X; writes the input gradient to gX unless gX.p is null.
void conv_bwd(ib3d_net* n, int l, const Vol& v, Act X, Act Y, Act gY, Act gX) {
  const Layer& ly = n->L[l];
  const long long M = v.voxels();
  relu_bwd(n->st, M, ly.N, gY, Y);
  bias_grad(n->st, M, gY, ly.N, n->g + ly.b);
  if (n->wgrad_cuda_cores) wgrad_cuda_cores(n->st, v, gY, ly.N, X, ly.K, n->g + ly.w);
  else wgrad(n->st, v, gY, ly.N, X, ly.K, n->g + ly.w, n->d_err);
  if (gX.p) conv(n->st, v, gY, ly.N, wt(n, l), nullptr, 0, -1, gX, ly.K, n->d_err);
}

void backward(ib3d_net* n) {
  Buffers& b = n->buf;
  cudaStream_t st = n->st;
  head_bwd(st, b.v1.voxels(), 16, A(b.d1, 16), n->p + n->head, b.gout, A(b.g_d1, 16), n->g + n->head);
  conv_bwd(n, 9, b.v1, A(b.a5, 16), A(b.d1, 16), A(b.g_d1, 16), A(b.g_a5, 16));
  conv_bwd(n, 8, b.v1, A(b.cat5, 48), A(b.a5, 16), A(b.g_a5, 16), A(b.g_cat5, 48));
  up_bwd(st, b.v2, 32, A(b.g_cat5, 48, 0), A(b.g_d2, 32));
  conv_bwd(n, 7, b.v2, A(b.a4, 32), A(b.d2, 32), A(b.g_d2, 32), A(b.g_a4, 32));
  conv_bwd(n, 6, b.v2, A(b.cat4, 96), A(b.a4, 32), A(b.g_a4, 32), A(b.g_cat4, 96));
  up_bwd(st, b.v3, 64, A(b.g_cat4, 96, 0), A(b.g_b, 64));
  conv_bwd(n, 5, b.v3, A(b.a3, 64), A(b.b, 64), A(b.g_b, 64), A(b.g_a3, 64));
  conv_bwd(n, 4, b.v3, A(b.p2, 32), A(b.a3, 64), A(b.g_a3, 64), A(b.g_p2, 32));
  pool_bwd(st, b.v3, 32, A(b.g_p2, 32), A(b.g_cat4, 96, 64), 1);
  conv_bwd(n, 3, b.v2, A(b.a2, 32), A(b.cat4, 96, 64), A(b.g_cat4, 96, 64), A(b.g_a2, 32));
  conv_bwd(n, 2, b.v2, A(b.p1, 16), A(b.a2, 32), A(b.g_a2, 32), A(b.g_p1, 16));
  pool_bwd(st, b.v2, 16, A(b.g_p1, 16), A(b.g_cat5, 48, 32), 1);
  conv_bwd(n, 1, b.v1, A(b.a1, 16), A(b.cat5, 48, 32), A(b.g_cat5, 48, 32), A(b.g_a1, 16));
  conv_bwd(n, 0, b.v1, A(b.in0, 16), A(b.a1, 16), A(b.g_a1, 16), Act{nullptr, 0, 0});
}

void cast_weights(ib3d_net* n) {
  for (int l = 0; l < kL; ++l) cast_conv_weights(n->st, n->L[l].N, n->L[l].K, n->p + n->L[l].w, n->wf + n->L[l].w,
                                                   n->wt + n->L[l].w);
}

// ------------------------------------------------------------- data kernels

// Input channels of one cell (see the file header); channels kInputs..15 are zero.
// The difference of the pressures is taken in FP64; the scaling in FP32 (sc holds
// the reciprocal RMS values r1..r4 of NetNorm).
__device__ __forceinline__ void cell_inputs(long long o, const double* h1, const double* h2, const double* bdt,
                                            const float* r, const float sc[kInputs], float in[kInputs]) {
  in[0] = (float)(h1[o] - h2[o]) * sc[0];
  in[1] = (float)bdt[o] * sc[1];
  in[2] = (float)h1[o] * sc[2];
  in[3] = r[o] * sc[3];
}

// Inputs of one coarse voxel: the average of cell_inputs over the f^3 fine cells it
// covers that lie in the domain (x0..x0+f-1 etc., 1-based interior cells from 2);
// non-fluid cells count as zero inputs.
__device__ __forceinline__ void coarse_inputs(const Dims& d, const unsigned char* cell, int f, int i0, int j0,
                                              int k0, const double* h1, const double* h2, const double* bdt,
                                              const float* r, const NetNorm& nm, float in[kInputs]) {
  const float sc[kInputs] = {(float)nm.r1, (float)nm.r2, (float)nm.r3, (float)nm.r4};
  float acc[kInputs] = {};
  int n = 0;
  for (int dz = 0; dz < f; ++dz)
    for (int dy = 0; dy < f; ++dy)
      for (int dx = 0; dx < f; ++dx) {
        const int i = i0 + dx, j = j0 + dy, k = k0 + dz;
        if (i > d.nx + 1 || j > d.ny + 1 || k > d.nz + 1) continue;
        ++n;
        const long long o = d.at(i, j, k);
        if (cell[o] != 0) continue;
        float c[kInputs];
        cell_inputs(o, h1, h2, bdt, r, sc, c);
#pragma unroll
        for (int q = 0; q < kInputs; ++q) acc[q] += c[q];
      }
#pragma unroll
  for (int q = 0; q < kInputs; ++q) in[q] = n ? acc[q] / (float)n : 0.f;
}

// Full-domain input volume at coarsening f: voxel (x,y,z) covers fine cells
// 2+f*x .. 2+f*x+f-1 (and likewise in y, z); 1 x D x H x W with D, H, W the coarse
// extents rounded up to multiples of 4, zero outside the domain.
__global__ void k_pack_domain(Dims d, Vol v, int f, const unsigned char* __restrict__ cell,
                              const double* __restrict__ h1, const double* __restrict__ h2,
                              const double* __restrict__ bdt, const float* __restrict__ r,
                              const NetNorm* __restrict__ nmp, bf16* __restrict__ in0) {
  const long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= v.voxels()) return;
  const int x = (int)(m % v.W), y = (int)((m / v.W) % v.H), z = (int)(m / ((long long)v.W * v.H));
  float in[kInputs] = {};
  const NetNorm nm = *nmp;
  if (nm.valid && f * x < d.nx && f * y < d.ny && f * z < d.nz)
    coarse_inputs(d, cell, f, 2 + f * x, 2 + f * y, 2 + f * z, h1, h2, bdt, r, nm, in);
  bf16* dst = in0 + m * 16;
#pragma unroll
  for (int c = 0; c < kInputs; ++c) dst[c] = __float2bfloat16(in[c]);
}

// pc = (p^{n-1} - p^{n-2}) + s1 * out on fluid cells, 0 elsewhere, out taken back
// from the coarse voxels by trilinear interpolation between their centres (a
// piecewise-constant prolongation leaves jumps at voxel faces whose high-frequency
// error the over-relaxed sweeps remove slowly: 5 % more sweeps). Without a valid
// normalisation, or after a convolution gave up (err), pc is left as it is: the
// previous correction.
__global__ void k_unpack_domain(Dims d, Vol v, int f, const float* __restrict__ out,
                                const unsigned char* __restrict__ cell, const double* __restrict__ h1,
                                const double* __restrict__ h2, const NetNorm* __restrict__ nmp,
                                const int* __restrict__ err, double* __restrict__ pc) {
  const unsigned tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= (unsigned)d.n3 || !nmp->valid || *err != 0) return;
  const double s1 = nmp->s1;
  const int i = (int)(tid % (unsigned)d.NX2);
  const unsigned t = tid / (unsigned)d.NX2;
  const int j = (int)(t % (unsigned)d.NY2), k = (int)(t / (unsigned)d.NY2);
  double val = 0.0;
  if (i >= 1 && i <= d.nx && j >= 1 && j <= d.ny && k >= 1 && k <= d.nz && cell[tid] == 0) {
    // trilinear interpolation between voxel centres (voxel x covers cells f*x .. f*x+f-1,
    // centre at f*x + (f-1)/2), clamped at the ends of the coarse extents in use
    const int cxn = (d.nx + f - 1) / f, cyn = (d.ny + f - 1) / f, czn = (d.nz + f - 1) / f;
    const float fx = fminf(fmaxf(((float)(i - 1) - 0.5f * (f - 1)) / f, 0.f), (float)(cxn - 1));
    const float fy = fminf(fmaxf(((float)(j - 1) - 0.5f * (f - 1)) / f, 0.f), (float)(cyn - 1));
    const float fz = fminf(fmaxf(((float)(k - 1) - 0.5f * (f - 1)) / f, 0.f), (float)(czn - 1));
    const int x0 = min((int)fx, cxn - 1), y0 = min((int)fy, cyn - 1), z0 = min((int)fz, czn - 1);
    const int x1 = min(x0 + 1, cxn - 1), y1 = min(y0 + 1, cyn - 1), z1 = min(z0 + 1, czn - 1);
    const float wx = fx - x0, wy = fy - y0, wz = fz - z0;
    auto O = [&](int z, int y, int x) { return out[((long long)z * v.H + y) * v.W + x]; };
    const float c00 = O(z0, y0, x0) * (1.f - wx) + O(z0, y0, x1) * wx;
    const float c01 = O(z0, y1, x0) * (1.f - wx) + O(z0, y1, x1) * wx;
    const float c10 = O(z1, y0, x0) * (1.f - wx) + O(z1, y0, x1) * wx;
    const float c11 = O(z1, y1, x0) * (1.f - wx) + O(z1, y1, x1) * wx;
    const float o = (c00 * (1.f - wy) + c01 * wy) * (1.f - wz) + (c10 * (1.f - wy) + c11 * wy) * wz;
    val = (h1[tid] - h2[tid]) + s1 * (double)o;
  }
  pc[tid] = val;
}

// One training patch of S^3 coarse voxels at coarsening f, covering the fine cells
// from (i0,j0,k0) (1-based interior cells): the averaged inputs and the averaged
// change of the correction over the fluid cells (0 where a voxel has none).
__global__ void k_capture(Dims d, int S, int f, int i0, int j0, int k0, const double* __restrict__ h1,
                          const double* __restrict__ h2, const double* __restrict__ bdt,
                          const float* __restrict__ r, const double* __restrict__ pc,
                          const unsigned char* __restrict__ cell, const NetNorm* __restrict__ nmp,
                          bf16* __restrict__ din, float* __restrict__ dt) {
  const long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= (long long)S * S * S) return;
  const NetNorm nm = *nmp;
  const int x = (int)(m % S), y = (int)((m / S) % S), z = (int)(m / ((long long)S * S));
  const int ci = i0 + f * x, cj = j0 + f * y, ck = k0 + f * z;
  float in[kInputs];
  coarse_inputs(d, cell, f, ci, cj, ck, h1, h2, bdt, r, nm, in);
#pragma unroll
  for (int c = 0; c < kInputs; ++c) din[m * kInputs + c] = __float2bfloat16(in[c]);
  double t = 0.0;
  int n = 0;
  for (int dz = 0; dz < f; ++dz)
    for (int dy = 0; dy < f; ++dy)
      for (int dx = 0; dx < f; ++dx) {
        const long long o = d.at(ci + dx, cj + dy, ck + dz);
        if (cell[o] != 0) continue;
        t += (pc[o] - (h1[o] - h2[o])) * nm.r1;
        ++n;
      }
  dt[m] = n ? (float)(t / n) : 0.f;
}

// Gathers a batch of patches into the 16-channel input and the target.
__global__ void k_gather(long long per, int B, const int* __restrict__ ids, const bf16* __restrict__ ds_in,
                         const float* __restrict__ ds_t, bf16* __restrict__ in0, float* __restrict__ tgt) {
  const long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= per * B) return;
  const int bi = (int)(m / per);
  const long long v = m % per;
  const long long src = (long long)ids[bi] * per + v;
  bf16* dst = in0 + m * 16;
  for (int c = 0; c < kInputs; ++c) dst[c] = ds_in[src * kInputs + c];
  tgt[m] = ds_t[src];
}

// Host-side copy of a batch given as FP32 [B][S^3][kInputs] into the 16-channel input.
__global__ void k_set_input(long long M, const float* __restrict__ x, bf16* __restrict__ in0) {
  const long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= M) return;
  for (int c = 0; c < kInputs; ++c) in0[m * 16 + c] = __float2bfloat16(x[m * kInputs + c]);
}

}  // namespace

namespace ib3d {
// Called by the pressure solve: pc = network prediction (returns nonzero when the
// history or the normalisation is not available yet; pc is then left unchanged).
int net_predict_pc(ib3d_ctx* c) {
  ib3d_net* n = c->net;
  if (!n || c->hist_valid < 2 || !c->d_norm) return 1;
  // no host synchronisation here: the normalisation (k_hist_residual, this step) and
  // the convolutions' status are read on the device by the pack and unpack kernels
  const int f = n->coarsen;
  const int cz = (c->d.nz + f - 1) / f, cy = (c->d.ny + f - 1) / f, cx = (c->d.nx + f - 1) / f;
  const Vol v{1, (cz + 3) / 4 * 4, (cy + 3) / 4 * 4, (cx + 3) / 4 * 4};
  cudaStream_t saved = n->st;
  n->st = c->st;
  int rc = ensure_buffers(n, v, false);
  if (rc) { n->st = saved; return rc; }
  k_pack_domain<<<(unsigned)((v.voxels() + 255) / 256), 256, 0, c->st>>>(c->d, v, f, c->cell, c->hist[0],
                                                                         c->hist[1], c->bdt, c->r_hist, c->d_norm,
                                                                         n->buf.in0);
  forward(n);
  k_unpack_domain<<<(unsigned)((c->d.n3 + 255) / 256), 256, 0, c->st>>>(c->d, v, f, n->buf.out, c->cell,
                                                                        c->hist[0], c->hist[1], c->d_norm, n->d_err,
                                                                        c->pc);
  n->st = saved;
  c->launches += 17;
  return cudaGetLastError() == cudaSuccess ? 0 : 1;
}

void net_note_failure(ib3d_ctx* c) {
  if (!c->net) return;
  int h = 0;
  if (cudaMemcpy(&h, c->net->d_err, sizeof(int), cudaMemcpyDeviceToHost) == cudaSuccess && h)
    c->net->err = "ib3d_net: a tensor-core wait timed out; the steps since used the previous correction";
}
}  // namespace ib3d

extern "C" {

int ib3d_net_create(ib3d_net** out, uint64_t seed) {
  if (!out) return IB3D_ERR_ARG;
  *out = nullptr;
  ib3d_net* n = new ib3d_net();
  size_t off = 0;
  for (int l = 0; l < kL; ++l) {
    n->L[l] = {kN[l], kK[l], kKreal[l], off, off + (size_t)kN[l] * 27 * kK[l]};
    off = n->L[l].b + kN[l];
    off = (off + 7) & ~(size_t)7;    // keep every block 32-byte aligned
  }
  n->head = off;
  n->nparam = off + 17;
  std::vector<float> hp(n->nparam, 0.0f);
  std::mt19937_64 rng(seed);
  for (int l = 0; l < kL; ++l) {
    std::normal_distribution<float> nd(0.0f, std::sqrt(2.0f / (27.0f * kKreal[l])));
    for (int o = 0; o < kN[l]; ++o)
      for (int t = 0; t < 27; ++t)
        for (int k = 0; k < kK[l]; ++k)
          hp[n->L[l].w + ((size_t)o * 27 + t) * kK[l] + k] = k < kKreal[l] ? nd(rng) : 0.0f;
  }
  std::normal_distribution<float> nh(0.0f, 0.01f);
  for (int q = 0; q < 16; ++q) hp[n->head + q] = nh(rng);
  bool ok = cudaStreamCreateWithFlags(&n->st, cudaStreamNonBlocking) == cudaSuccess;
  float** fb[] = {&n->p, &n->g, &n->m1, &n->m2};
  for (float** q : fb) ok = ok && cudaMalloc(q, n->nparam * sizeof(float)) == cudaSuccess;
  ok = ok && cudaMalloc(&n->wf, n->nparam * sizeof(bf16)) == cudaSuccess &&
       cudaMalloc(&n->wt, n->nparam * sizeof(bf16)) == cudaSuccess &&
       cudaMalloc(&n->d_loss, sizeof(double)) == cudaSuccess &&
       cudaMalloc(&n->d_err, sizeof(int)) == cudaSuccess && cudaMemset(n->d_err, 0, sizeof(int)) == cudaSuccess;
  if (!ok) {
    ib3d_net_destroy(n);
    return IB3D_ERR_MEMORY;
  }
  cudaMemcpy(n->p, hp.data(), n->nparam * sizeof(float), cudaMemcpyHostToDevice);
  cudaMemset(n->m1, 0, n->nparam * sizeof(float));
  cudaMemset(n->m2, 0, n->nparam * sizeof(float));
  cast_weights(n);
  if (cudaStreamSynchronize(n->st) != cudaSuccess) {
    ib3d_net_destroy(n);
    return IB3D_ERR_CUDA;
  }
  *out = n;
  return IB3D_OK;
}

void ib3d_net_destroy(ib3d_net* n) {
  if (!n) return;
  if (n->st) cudaStreamSynchronize(n->st);
  free_buffers(n->buf);
  void* ptrs[] = {n->p, n->g, n->m1, n->m2, n->wf, n->wt, n->ds_in, n->ds_t, n->d_loss, n->d_err};
  for (void* q : ptrs)
    if (q) cudaFree(q);
  if (n->st) cudaStreamDestroy(n->st);
  delete n;
}

const char* ib3d_net_last_error(const ib3d_net* n) { return n ? n->err.c_str() : "null network"; }

int64_t ib3d_net_num_params(const ib3d_net* n) { return n ? (int64_t)n->nparam : 0; }

int ib3d_net_get_params(ib3d_net* n, float* out) {
  if (!n || !out) return IB3D_ERR_ARG;
  NET_CUDA(n, cudaMemcpy(out, n->p, n->nparam * sizeof(float), cudaMemcpyDeviceToHost));
  return IB3D_OK;
}

int ib3d_net_set_params(ib3d_net* n, const float* in) {
  if (!n || !in) return IB3D_ERR_ARG;
  NET_CUDA(n, cudaMemcpy(n->p, in, n->nparam * sizeof(float), cudaMemcpyHostToDevice));
  cast_weights(n);
  NET_CUDA(n, cudaStreamSynchronize(n->st));
  return IB3D_OK;
}

// Loss and parameter gradient of one batch given on the host (x: [B][S^3][kInputs] FP32,
// target: [B][S^3]); no update. out (may be NULL) receives the network output.
int ib3d_net_loss_grad(ib3d_net* n, int B, int S, const float* x, const float* target, double* loss, float* grad,
                       float* out) {
  if (!n || B < 1 || S < 4 || S % 4 || !x || !target) return IB3D_ERR_ARG;
  const Vol v{B, S, S, S};
  int rc = ensure_buffers(n, v, true);
  if (rc) return rc;
  const long long M = v.voxels();
  float* dx = nullptr;
  NET_CUDA(n, cudaMalloc(&dx, (size_t)M * kInputs * sizeof(float)));
  cudaMemcpyAsync(dx, x, (size_t)M * kInputs * sizeof(float), cudaMemcpyHostToDevice, n->st);
  cudaMemcpyAsync(n->buf.tgt, target, (size_t)M * sizeof(float), cudaMemcpyHostToDevice, n->st);
  k_set_input<<<(unsigned)((M + 255) / 256), 256, 0, n->st>>>(M, dx, n->buf.in0);
  cudaMemsetAsync(n->g, 0, n->nparam * sizeof(float), n->st);
  cudaMemsetAsync(n->d_loss, 0, sizeof(double), n->st);
  forward(n);
  mse(n->st, M, n->buf.out, n->buf.tgt, n->buf.gout, n->d_loss);
  backward(n);
  if (loss) cudaMemcpyAsync(loss, n->d_loss, sizeof(double), cudaMemcpyDeviceToHost, n->st);
  if (grad) cudaMemcpyAsync(grad, n->g, n->nparam * sizeof(float), cudaMemcpyDeviceToHost, n->st);
  if (out) cudaMemcpyAsync(out, n->buf.out, (size_t)M * sizeof(float), cudaMemcpyDeviceToHost, n->st);
  NET_CUDA(n, cudaStreamSynchronize(n->st));
  cudaFree(dx);
  NET_CUDA(n, cudaGetLastError());
  return check_conv(n);
}

// Reserves room for `capacity` training patches of edge S (S a multiple of 4).
int ib3d_net_dataset_reserve(ib3d_net* n, int S, int64_t capacity) {
  if (!n || S < 4 || S % 4 || capacity < 1) return IB3D_ERR_ARG;
  if (n->ds_in) cudaFree(n->ds_in);
  if (n->ds_t) cudaFree(n->ds_t);
  n->ds_in = nullptr;
  n->ds_t = nullptr;
  const size_t per = (size_t)S * S * S;
  NET_CUDA(n, cudaMalloc(&n->ds_in, (size_t)capacity * per * kInputs * sizeof(bf16)));
  NET_CUDA(n, cudaMalloc(&n->ds_t, (size_t)capacity * per * sizeof(float)));
  n->S = S;
  n->cap = capacity;
  n->count = 0;
  return IB3D_OK;
}

int64_t ib3d_net_dataset_size(const ib3d_net* n) { return n ? n->count : 0; }

// Coarsening of capture and inference: 1 (full resolution), 2 (the default: 2x2x2
// cells per voxel) or 4. Clears the training set, whose patches used the old one.
int ib3d_net_set_coarsening(ib3d_net* n, int f) {
  if (!n || (f != 1 && f != 2 && f != 4)) return IB3D_ERR_ARG;
  n->coarsen = f;
  n->count = 0;
  return IB3D_OK;
}

int ib3d_net_set_wgrad_tensor_cores(ib3d_net* n, int on) {
  if (!n) return IB3D_ERR_ARG;
  n->wgrad_cuda_cores = on == 0;
  return IB3D_OK;
}

// Adds up to npatches random S^3 patches of the context's last step (inputs from
// the two previous pressures and this step's b/dt, target this step's pc).
int ib3d_net_capture(ib3d_net* n, ib3d_ctx* c, int npatches, uint64_t seed) {
  if (!n || !c || npatches < 1 || !n->ds_in) return IB3D_ERR_ARG;
  if (c->hist_valid < 2) return fail(n, IB3D_ERR_ARG, "ib3d_net_capture: fewer than two previous pressures");
  const int S = n->S, f = n->coarsen, F = S * f;   // F fine cells per patch edge
  if (F > c->d.nx || F > c->d.ny || F > c->d.nz) return fail(n, IB3D_ERR_ARG, "ib3d_net_capture: patch larger than grid");
  NetNorm nm{};
  if (!c->d_norm || cudaMemcpy(&nm, c->d_norm, sizeof(nm), cudaMemcpyDeviceToHost) != cudaSuccess || !nm.valid)
    return fail(n, IB3D_ERR_ARG, "ib3d_net_capture: zero normalisation");
  std::mt19937_64 rng(seed);
  const size_t per = (size_t)S * S * S;
  for (int q = 0; q < npatches && n->count < n->cap; ++q) {
    const int i0 = 2 + (int)(rng() % (uint64_t)(c->d.nx - F + 1));
    const int j0 = 2 + (int)(rng() % (uint64_t)(c->d.ny - F + 1));
    const int k0 = 2 + (int)(rng() % (uint64_t)(c->d.nz - F + 1));
    k_capture<<<(unsigned)((per + 255) / 256), 256, 0, c->st>>>(c->d, S, f, i0, j0, k0, c->hist[0], c->hist[1],
                                                                c->bdt, c->r_hist, c->pc, c->cell, c->d_norm,
                                                                n->ds_in + n->count * per * kInputs,
                                                                n->ds_t + n->count * per);
    n->count++;
  }
  NET_CUDA(n, cudaStreamSynchronize(c->st));
  NET_CUDA(n, cudaGetLastError());
  return IB3D_OK;
}

// `steps` Adam steps (lr, default moments) on random batches of the captured set.
int ib3d_net_train(ib3d_net* n, int steps, int batch, double lr, uint64_t seed, double* last_loss) {
  if (!n || steps < 1 || batch < 1 || n->count < 1) return IB3D_ERR_ARG;
  const int S = n->S;
  const Vol v{batch, S, S, S};
  int rc = ensure_buffers(n, v, true);
  if (rc) return rc;
  const long long per = (long long)S * S * S, M = v.voxels();
  int* ids = nullptr;
  NET_CUDA(n, cudaMalloc(&ids, batch * sizeof(int)));
  std::mt19937_64 rng(seed);
  std::vector<int> hid(batch);
  double loss = 0.0;
  for (int s = 0; s < steps; ++s) {
    for (int q = 0; q < batch; ++q) hid[q] = (int)(rng() % (uint64_t)n->count);
    cudaMemcpyAsync(ids, hid.data(), batch * sizeof(int), cudaMemcpyHostToDevice, n->st);
    k_gather<<<(unsigned)((M + 255) / 256), 256, 0, n->st>>>(per, batch, ids, n->ds_in, n->ds_t, n->buf.in0,
                                                            n->buf.tgt);
    cudaMemsetAsync(n->g, 0, n->nparam * sizeof(float), n->st);
    cudaMemsetAsync(n->d_loss, 0, sizeof(double), n->st);
    forward(n);
    mse(n->st, M, n->buf.out, n->buf.tgt, n->buf.gout, n->d_loss);
    backward(n);
    n->step++;
    adam(n->st, (int)n->nparam, n->p, n->g, n->m1, n->m2, (float)lr, n->step);
    cast_weights(n);
    if (s == steps - 1) cudaMemcpyAsync(&loss, n->d_loss, sizeof(double), cudaMemcpyDeviceToHost, n->st);
    // hid is rewritten next step: wait for the async copy of this step's ids
    cudaStreamSynchronize(n->st);
  }
  cudaFree(ids);
  NET_CUDA(n, cudaGetLastError());
  if (int rc = check_conv(n)) return rc;
  if (last_loss) *last_loss = loss;
  return IB3D_OK;
}

// Uses the network as the warm start of ctx's pressure solves (IB3D_WARM_LEARNED).
int ib3d_attach_net(ib3d_ctx* c, ib3d_net* n) {
  if (!c) return IB3D_ERR_ARG;
  c->net = n;
  return ib3d_enable_history(c);
}

}  // extern "C"
