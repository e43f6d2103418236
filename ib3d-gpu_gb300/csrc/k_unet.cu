// Kernels of the learned warm start: a small 3-D U-Net in BF16 with FP32
// accumulation (forward, backward, Adam). Host orchestration is in unet.cu.
//
// Activations are channels-last BF16 tensors [voxel][channel] over B x D x H x W
// voxels; a tensor can be a channel slice of a wider buffer (channel stride cs,
// offset co), which is how the U-Net's skip concatenations are stored. Channel
// counts are multiples of 16.
//
// 3x3x3 convolutions (zero padding) are implicit GEMMs on the fifth-generation
// tensor cores (tcgen05.mma kind::f16, BF16 operands from shared memory, FP32
// accumulator in tensor memory): rows are 128 voxels of a block, columns the
// output channels, and the reduction runs over 27 taps x input channels in steps of
// 16 channels. The threads gather four steps' A tiles (the 128 voxels' neighbours,
// 16 channels each) and B tiles (the weights) into one of two shared-memory stages
// in the canonical no-swizzle K-major layout, one thread issues the stage's four
// MMAs, and a tcgen05.commit to the stage's mbarrier frees it for the stage after
// next; the next stage's loads are in flight meanwhile. The
// same kernel computes the input gradient with mirrored taps and transposed
// weights, and k_wgrad_tc the weight gradients as a second implicit GEMM over voxels.
#include <cuda_bf16.h>

#include <algorithm>

#include "ib3d_internal.cuh"
#include "unet.cuh"

namespace ib3d {
namespace unet {

namespace {

__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor, no swizzle, K-major: core matrices of 8 rows x 16
// bytes; lbo = byte distance between core matrices along K, sbo = along M/N.
__device__ __forceinline__ unsigned long long smem_desc(const void* p, unsigned lbo, unsigned sbo) {
  unsigned long long d = (unsigned long long)((smem_addr(p) & 0x3FFFF) >> 4);
  d |= (unsigned long long)((lbo >> 4) & 0x3FFF) << 16;
  d |= (unsigned long long)((sbo >> 4) & 0x3FFF) << 32;
  d |= 1ull << 46;   // descriptor version; base offset 0, no swizzle
  return d;
}

// Bounded wait on an mbarrier phase (true when it completed).
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned phase, int limit) {
  for (int it = 0; it < limit; ++it) {
    unsigned ok;
    asm volatile("{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
                 : "=r"(ok) : "r"(smem_addr(bar)), "r"(phase) : "memory");
    if (ok) return true;
  }
  return false;
}

__device__ __forceinline__ void decode(long long m, const Vol& v, int& b, int& z, int& y, int& x) {
  x = (int)(m % v.W);
  long long t = m / v.W;
  y = (int)(t % v.H);
  t /= v.H;
  z = (int)(t % v.D);
  b = (int)(t / v.D);
}

}  // namespace

// Y[v][n] = act( sum_{tap,k} X[v + sign*off(tap)][k] * Wt[n][tap][k] + bias[n] ),
// N output channels (a multiple of 16, at most 128). Block: 128 threads, 128
// consecutive voxels; D in tensor memory (128 lanes x N FP32 columns).
//
// The reduction runs in steps of 16 (tap, channel) pairs, kSub steps per stage: a
// stage is kSub A tiles (128 x 16) and kSub B tiles (N x 16) in shared memory, and
// one thread issues its kSub MMAs back to back and commits them to the stage's
// mbarrier. Two stages alternate, and every thread loads the next stage's
// neighbour values into registers before the current stage's MMAs are issued, so
// the global-load latency overlaps the tensor-core work; the registers go to shared
// memory once the MMAs that last read that stage have completed.
//
// Every wait is bounded and decided for the whole block: a barrier that does not
// complete sets *err, and the kernel still waits (bounded) for its issued MMAs
// before it frees the tensor memory.
constexpr int kSub = 4;

template <int N>
constexpr size_t conv_smem_bytes() {
  return (size_t)2 * kSub * (128 * 16 + N * 16) * sizeof(bf16);
}

template <int N>
__global__ void __launch_bounds__(128) k_conv3(Vol vol, Act X, int K, const bf16* __restrict__ Wt,
                                               const float* __restrict__ bias, int relu, int sign, Act Y, int* err) {
  static_assert(N % 16 == 0 && N >= 16 && N <= 128, "tcgen05 N");
  extern __shared__ __align__(1024) unsigned char smraw[];
  bf16* sA = reinterpret_cast<bf16*>(smraw);             // [2][kSub][128 * 16]
  bf16* sB = sA + 2 * kSub * 128 * 16;                     // [2][kSub][N * 16]
  __shared__ __align__(8) unsigned long long bar[3];
  __shared__ unsigned tmem_base;
  constexpr unsigned kCols = N <= 32 ? 32 : (N <= 64 ? 64 : 128);   // power of two >= N
  const int t = threadIdx.x, warp = t >> 5;
  const long long M = vol.voxels();
  const long long m = (long long)blockIdx.x * 128 + t;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 :: "r"(smem_addr(&tmem_base)), "r"(kCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (t == 0) {
    for (int q = 0; q < 3; ++q) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_addr(&bar[q])));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const unsigned tmem = tmem_base;
  int vb = 0, vz = 0, vy = 0, vx = 0;
  const bool vok = m < M;
  if (vok) decode(m, vol, vb, vz, vy, vx);
  // instruction descriptor: D FP32, A and B BF16, both K-major, N, M = 128
  const unsigned idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((unsigned)(N >> 3) << 17) | ((128u >> 4) << 24);
  const int kchunks = K / 16, steps = 27 * kchunks, nst = (steps + kSub - 1) / kSub;
  const int g = t >> 3, rr = t & 7;   // core-matrix row group and row of this thread's A (and B) row
  uint4 ra[kSub][2], rb[kSub][2];
  // registers of stage q: this voxel's neighbour and this thread's weight row, per step
  auto gather = [&](int q) {
#pragma unroll
    for (int j = 0; j < kSub; ++j) {
      const int s = q * kSub + j;
      ra[j][0] = ra[j][1] = rb[j][0] = rb[j][1] = make_uint4(0, 0, 0, 0);
      if (s < steps) {
        const int tap = s / kchunks, kc = (s % kchunks) * 16;
        const int z = vz + sign * (tap / 9 - 1), y = vy + sign * ((tap / 3) % 3 - 1), x = vx + sign * (tap % 3 - 1);
        if (vok && z >= 0 && z < vol.D && y >= 0 && y < vol.H && x >= 0 && x < vol.W) {
          const long long sv = (((long long)vb * vol.D + z) * vol.H + y) * vol.W + x;
          const uint4* src = reinterpret_cast<const uint4*>(X.p + sv * X.cs + X.co + kc);
          ra[j][0] = src[0];
          ra[j][1] = src[1];
        }
        if (t < N) {
          const uint4* w = reinterpret_cast<const uint4*>(Wt + ((size_t)t * 27 + tap) * K + kc);
          rb[j][0] = w[0];
          rb[j][1] = w[1];
        }
      }
    }
  };
  auto store = [&](int buf) {
#pragma unroll
    for (int j = 0; j < kSub; ++j) {
      char* a = reinterpret_cast<char*>(sA + (buf * kSub + j) * 128 * 16);
      *reinterpret_cast<uint4*>(a + (g * 2 + 0) * 128 + rr * 16) = ra[j][0];
      *reinterpret_cast<uint4*>(a + (g * 2 + 1) * 128 + rr * 16) = ra[j][1];
      if (t < N) {
        char* b = reinterpret_cast<char*>(sB + (buf * kSub + j) * N * 16);
        *reinterpret_cast<uint4*>(b + (g * 2 + 0) * 128 + rr * 16) = rb[j][0];
        *reinterpret_cast<uint4*>(b + (g * 2 + 1) * 128 + rr * 16) = rb[j][1];
      }
    }
  };
  gather(0);
  store(0);
  unsigned phase[2] = {0, 0};
  bool ok = true;
  for (int q = 0; q < nst; ++q) {
    const int buf = q & 1;
    if (q + 1 < nst) gather(q + 1);   // in flight while this stage's MMAs are issued and run
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");   // make the stage visible to the tensor core
    __syncthreads();
    if (t == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
      for (int j = 0; j < kSub; ++j) {
        const int s = q * kSub + j;
        if (s < steps) {
          const unsigned long long ad = smem_desc(sA + (buf * kSub + j) * 128 * 16, 128, 256);
          const unsigned long long bd = smem_desc(sB + (buf * kSub + j) * N * 16, 128, 256);
          asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                       " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
                       :: "r"(tmem), "l"(ad), "l"(bd), "r"(idesc), "r"(s > 0 ? 1u : 0u) : "memory");
        }
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                   :: "r"(smem_addr(&bar[buf])) : "memory");
    }
    if (q + 1 < nst) {
      const int nb = buf ^ 1;
      if (q >= 1) {   // stage nb was last read by the MMAs of stage q - 1
        ok = __syncthreads_and(mbar_wait(&bar[nb], phase[nb], 1 << 20)) != 0;
        phase[nb] ^= 1;
        if (!ok) break;
      }
      store(nb);
    }
  }
  // a commit after the last MMA arrives once every MMA of this thread is done
  if (t == 0)
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                 :: "r"(smem_addr(&bar[2])) : "memory");
  bool done = __syncthreads_and(mbar_wait(&bar[2], 0, 1 << 20)) != 0;
  if (ok && done) {
    // the last one or two stages' own arrivals, so that none is left pending at exit
    for (int q = nst >= 2 ? nst - 2 : 0; q < nst; ++q) {
      const int b = q & 1;
      done = __syncthreads_and(mbar_wait(&bar[b], phase[b], 1 << 20)) != 0 && done;
      phase[b] ^= 1;
    }
  }
  if (!ok || !done) {
    if (t == 0) atomicExch(err, 1);
    mbar_wait(&bar[2], 0, 1 << 20);   // let the issued MMAs finish before freeing the columns
  } else {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
    for (int c0 = 0; c0 < N; c0 += 16) {
      unsigned r[16];
      const unsigned addr = tmem + ((unsigned)(warp * 32) << 16) + (unsigned)c0;   // this warp's 32 lanes
      asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                   : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                     "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
                     "=r"(r[14]), "=r"(r[15])
                   : "r"(addr));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (vok) {
        bf16* dst = Y.p + m * Y.cs + Y.co + c0;
#pragma unroll
        for (int q = 0; q < 16; q += 2) {
          float v0 = __uint_as_float(r[q]), v1 = __uint_as_float(r[q + 1]);
          if (bias) { v0 += bias[c0 + q]; v1 += bias[c0 + q + 1]; }
          if (relu) { v0 = fmaxf(v0, 0.f); v1 = fmaxf(v1, 0.f); }
          *reinterpret_cast<__nv_bfloat162*>(dst + q) = __floats2bfloat162_rn(v0, v1);
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem), "r"(kCols));
}

// 8x8 transpose of BF16 values across the eight lanes of an octet (lanes 8m..8m+7):
// on entry lane l holds row l (eight values, the first in the low half of v.x); on
// return it holds column l. Three exchange rounds (lane distance 4, 2, 1), each
// swapping the off-diagonal blocks of the next-smaller block size.
__device__ __forceinline__ uint4 transpose8(uint4 v, int l8) {
  unsigned w0 = v.x, w1 = v.y, w2 = v.z, w3 = v.w;
  {
    const bool up = l8 & 4;
    const unsigned r0 = __shfl_xor_sync(0xffffffffu, up ? w0 : w2, 4);
    const unsigned r1 = __shfl_xor_sync(0xffffffffu, up ? w1 : w3, 4);
    if (up) { w0 = r0; w1 = r1; } else { w2 = r0; w3 = r1; }
  }
  {
    const bool up = l8 & 2;
    const unsigned r0 = __shfl_xor_sync(0xffffffffu, up ? w0 : w1, 2);
    const unsigned r1 = __shfl_xor_sync(0xffffffffu, up ? w2 : w3, 2);
    if (up) { w0 = r0; w2 = r1; } else { w1 = r0; w3 = r1; }
  }
  {
    const bool up = l8 & 1;
    const unsigned s0 = up ? __byte_perm(w0, w1, 0x5410) : __byte_perm(w0, w1, 0x7632);
    const unsigned s1 = up ? __byte_perm(w2, w3, 0x5410) : __byte_perm(w2, w3, 0x7632);
    const unsigned r0 = __shfl_xor_sync(0xffffffffu, s0, 1);
    const unsigned r1 = __shfl_xor_sync(0xffffffffu, s1, 1);
    if (up) {
      w0 = __byte_perm(r0, w0, 0x7610); w1 = __byte_perm(r0, w1, 0x7632);
      w2 = __byte_perm(r1, w2, 0x7610); w3 = __byte_perm(r1, w3, 0x7632);
    } else {
      w0 = __byte_perm(w0, r0, 0x5410); w1 = __byte_perm(w1, r0, 0x7610);
      w2 = __byte_perm(w2, r1, 0x5410); w3 = __byte_perm(w3, r1, 0x7610);
    }
  }
  return make_uint4(w0, w1, w2, w3);
}

// dW[n][tap][k] += sum_v dZ[v][n] * X[v + off(tap)][k] on the tensor cores: an
// implicit GEMM D[r][n] = sum_v A[r][v] B[n][v] with the 27 K (tap, channel) pairs as
// rows (128 per block, grid.x), the N output channels as columns and the voxels as the
// reduction (a chunk of them per block, grid.y). A[r][v] = X[v + off(tap)][k] and
// B[n][v] = dZ[v][n]; both tensors are channels-last, so an octet of threads loads
// eight channels of eight consecutive voxels and transposes them (transpose8) into the
// K-major core matrices the MMA reads. The pipeline is k_conv3's: kSub steps of 16
// voxels per stage, two stages, one thread issuing tcgen05.mma kind::f16 into an FP32
// accumulator in tensor memory, bounded mbarrier waits decided for the whole block. The
// block adds its 128 x N partial sums to dW with FP32 atomics.
template <int N>
constexpr size_t wgrad_smem_bytes() {
  return (size_t)2 * kSub * (128 * 16 + N * 16) * sizeof(bf16);
}

template <int N>
__global__ void __launch_bounds__(128) k_wgrad_tc(Vol vol, Act dZ, Act X, int K, float* __restrict__ dW,
                                                  long long chunk, int* err) {
  static_assert(N % 16 == 0 && N >= 16 && N <= 64, "output channels");
  extern __shared__ __align__(1024) unsigned char smraw[];
  bf16* sA = reinterpret_cast<bf16*>(smraw);             // [2][kSub][128 * 16]
  bf16* sB = sA + 2 * kSub * 128 * 16;                     // [2][kSub][N * 16]
  __shared__ __align__(8) unsigned long long bar[3];
  __shared__ unsigned tmem_base;
  constexpr unsigned kCols = N <= 32 ? 32 : 64;
  const int t = threadIdx.x, warp = t >> 5, oct = t >> 3, l8 = t & 7;
  const long long M = vol.voxels();
  const long long v0 = (long long)blockIdx.y * chunk, v1 = min(M, v0 + chunk);
  const int rows = 27 * K;
  const int R0 = blockIdx.x * 128 + 8 * oct;      // first (tap, channel) row of this octet
  const bool rok = R0 < rows;
  const int tap = rok ? R0 / K : 0, k0 = rok ? R0 % K : 0;   // K % 16 == 0: an octet's rows share the tap
  const int dz = tap / 9 - 1, dy = (tap / 3) % 3 - 1, dx = tap % 3 - 1;
  const bool bok = oct < N / 8;                   // this octet also stages eight rows of B
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 :: "r"(smem_addr(&tmem_base)), "r"(kCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (t == 0) {
    for (int q = 0; q < 3; ++q) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_addr(&bar[q])));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const unsigned tmem = tmem_base;
  // instruction descriptor: D FP32, A and B BF16, both K-major, N, M = 128
  const unsigned idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((unsigned)(N >> 3) << 17) | ((128u >> 4) << 24);
  const int steps = (int)((v1 - v0 + 15) / 16), nst = (steps + kSub - 1) / kSub;
  uint4 ra[kSub][2], rb[kSub][2];
  auto gather = [&](int q) {
#pragma unroll
    for (int j = 0; j < kSub; ++j)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        ra[j][h] = rb[j][h] = make_uint4(0, 0, 0, 0);
        const int s = q * kSub + j;
        const long long v = v0 + 16ll * s + 8 * h + l8;
        if (s < steps && v < v1) {
          int vb, z, y, x;
          decode(v, vol, vb, z, y, x);
          if (bok) rb[j][h] = *reinterpret_cast<const uint4*>(dZ.p + v * dZ.cs + dZ.co + 8 * oct);
          z += dz; y += dy; x += dx;
          if (rok && z >= 0 && z < vol.D && y >= 0 && y < vol.H && x >= 0 && x < vol.W) {
            const long long sv = (((long long)vb * vol.D + z) * vol.H + y) * vol.W + x;
            ra[j][h] = *reinterpret_cast<const uint4*>(X.p + sv * X.cs + X.co + k0);
          }
        }
      }
  };
  auto store = [&](int buf) {
#pragma unroll
    for (int j = 0; j < kSub; ++j)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const uint4 a = transpose8(ra[j][h], l8);   // row: channel k0+l8, voxels 8h..8h+7 of the step
        const uint4 b = transpose8(rb[j][h], l8);   // row: channel 8 oct + l8
        char* ap = reinterpret_cast<char*>(sA + (buf * kSub + j) * 128 * 16);
        *reinterpret_cast<uint4*>(ap + (oct * 2 + h) * 128 + l8 * 16) = a;
        if (bok) {
          char* bp = reinterpret_cast<char*>(sB + (buf * kSub + j) * N * 16);
          *reinterpret_cast<uint4*>(bp + (oct * 2 + h) * 128 + l8 * 16) = b;
        }
      }
  };
  gather(0);
  store(0);
  unsigned phase[2] = {0, 0};
  bool ok = true;
  for (int q = 0; q < nst; ++q) {
    const int buf = q & 1;
    if (q + 1 < nst) gather(q + 1);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (t == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
      for (int j = 0; j < kSub; ++j) {
        const int s = q * kSub + j;
        if (s < steps) {
          const unsigned long long ad = smem_desc(sA + (buf * kSub + j) * 128 * 16, 128, 256);
          const unsigned long long bd = smem_desc(sB + (buf * kSub + j) * N * 16, 128, 256);
          asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                       " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
                       :: "r"(tmem), "l"(ad), "l"(bd), "r"(idesc), "r"(s > 0 ? 1u : 0u) : "memory");
        }
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                   :: "r"(smem_addr(&bar[buf])) : "memory");
    }
    if (q + 1 < nst) {
      const int nb = buf ^ 1;
      if (q >= 1) {   // stage nb was last read by the MMAs of stage q - 1
        ok = __syncthreads_and(mbar_wait(&bar[nb], phase[nb], 1 << 20)) != 0;
        phase[nb] ^= 1;
        if (!ok) break;
      }
      store(nb);
    }
  }
  if (t == 0)
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                 :: "r"(smem_addr(&bar[2])) : "memory");
  bool done = __syncthreads_and(mbar_wait(&bar[2], 0, 1 << 20)) != 0;
  if (ok && done) {
    for (int q = nst >= 2 ? nst - 2 : 0; q < nst; ++q) {
      const int b = q & 1;
      done = __syncthreads_and(mbar_wait(&bar[b], phase[b], 1 << 20)) != 0 && done;
      phase[b] ^= 1;
    }
  }
  if (!ok || !done) {
    if (t == 0) atomicExch(err, 1);
    mbar_wait(&bar[2], 0, 1 << 20);   // let the issued MMAs finish before freeing the columns
  } else if (steps > 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const int R = blockIdx.x * 128 + t;   // this thread's accumulator row (lane t of tensor memory)
#pragma unroll
    for (int c0 = 0; c0 < N; c0 += 16) {
      unsigned r[16];
      const unsigned addr = tmem + ((unsigned)(warp * 32) << 16) + (unsigned)c0;
      asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                   : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                     "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
                     "=r"(r[14]), "=r"(r[15])
                   : "r"(addr));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (R < rows) {
        const int tp = R / K, k = R % K;
#pragma unroll
        for (int c = 0; c < 16; ++c) atomicAdd(&dW[((size_t)(c0 + c) * 27 + tp) * K + k], __uint_as_float(r[c]));
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem), "r"(kCols));
}

// dW[n][tap][k] += sum_v dZ[v][n] * X[v + off(tap)][k]   (FP32, CUDA cores): the
// reference form of k_wgrad_tc, kept for the gradient check of the tensor-core form.
// grid: (voxel chunks, 27 taps); each block reduces kWgTile voxels at a time through
// shared memory and adds its partial sums to dW with atomics.
constexpr int kWgTile = 32;
__global__ void __launch_bounds__(256) k_wgrad(Vol vol, Act dZ, int N, Act X, int K, float* __restrict__ dW,
                                               long long chunk) {
  extern __shared__ float sm[];
  float* sZ = sm;                    // [kWgTile][N]
  float* sX = sm + kWgTile * N;      // [kWgTile][K]
  const int tap = blockIdx.y;
  const int dz = tap / 9 - 1, dy = (tap / 3) % 3 - 1, dx = tap % 3 - 1;
  const long long M = vol.voxels();
  const long long v0 = (long long)blockIdx.x * chunk, v1 = min(M, v0 + chunk);
  const int NK = N * K;
  float acc[24];
#pragma unroll
  for (int q = 0; q < 24; ++q) acc[q] = 0.f;
  for (long long vt = v0; vt < v1; vt += kWgTile) {
    for (int e = threadIdx.x; e < kWgTile * N; e += blockDim.x) {
      const int lv = e / N, n = e % N;
      const long long m = vt + lv;
      sZ[e] = m < v1 ? __bfloat162float(dZ.p[m * dZ.cs + dZ.co + n]) : 0.f;
    }
    for (int e = threadIdx.x; e < kWgTile * K; e += blockDim.x) {
      const int lv = e / K, k = e % K;
      const long long m = vt + lv;
      float val = 0.f;
      if (m < v1) {
        int b, z, y, x;
        decode(m, vol, b, z, y, x);
        z += dz; y += dy; x += dx;
        if (z >= 0 && z < vol.D && y >= 0 && y < vol.H && x >= 0 && x < vol.W) {
          const long long sv = (((long long)b * vol.D + z) * vol.H + y) * vol.W + x;
          val = __bfloat162float(X.p[sv * X.cs + X.co + k]);
        }
      }
      sX[e] = val;
    }
    __syncthreads();
    for (int q = 0; q < 24; ++q) {
      const int pidx = threadIdx.x + q * 256;
      if (pidx >= NK) break;
      const int n = pidx / K, k = pidx % K;
      float s = acc[q];
#pragma unroll 8
      for (int lv = 0; lv < kWgTile; ++lv) s = fmaf(sZ[lv * N + n], sX[lv * K + k], s);
      acc[q] = s;
    }
    __syncthreads();
  }
  for (int q = 0; q < 24; ++q) {
    const int pidx = threadIdx.x + q * 256;
    if (pidx >= NK) break;
    const int n = pidx / K, k = pidx % K;
    atomicAdd(&dW[((size_t)n * 27 + tap) * K + k], acc[q]);
  }
}

// db[n] += sum_v dZ[v][n]
__global__ void k_bias_grad(long long M, Act dZ, int N, float* __restrict__ db) {
  __shared__ float s[64];
  if (threadIdx.x < N) s[threadIdx.x] = 0.f;
  __syncthreads();
  float acc[4] = {0.f, 0.f, 0.f, 0.f};
  const int n = threadIdx.x % N, lane_group = threadIdx.x / N, groups = blockDim.x / N;
  for (long long m = (long long)blockIdx.x * groups + lane_group; m < M; m += (long long)gridDim.x * groups)
    acc[0] += __bfloat162float(dZ.p[m * dZ.cs + dZ.co + n]);
  if (lane_group < groups) atomicAdd(&s[n], acc[0]);
  __syncthreads();
  if (threadIdx.x < N) atomicAdd(&db[threadIdx.x], s[threadIdx.x]);
}

// dY *= (Y > 0): ReLU backward through the layer's own output, in place.
__global__ void k_relu_bwd(long long M, int C, Act dY, Act Y) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= M * C) return;
  const long long m = e / C;
  const int c = (int)(e % C);
  if (!(__bfloat162float(Y.p[m * Y.cs + Y.co + c]) > 0.f)) dY.p[m * dY.cs + dY.co + c] = __float2bfloat16(0.f);
}

// 2x2x2 average pooling: out has half the extent of in along each axis.
__global__ void k_pool_fwd(Vol out, int C, Act in, Act o) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= out.voxels() * C) return;
  const long long m = e / C;
  const int c = (int)(e % C);
  int b, z, y, x;
  decode(m, out, b, z, y, x);
  const int D2 = out.D * 2, H2 = out.H * 2, W2 = out.W * 2;
  float s = 0.f;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const long long sv = (((long long)b * D2 + 2 * z + (q >> 2)) * H2 + 2 * y + ((q >> 1) & 1)) * W2 + 2 * x + (q & 1);
    s += __bfloat162float(in.p[sv * in.cs + in.co + c]);
  }
  o.p[m * o.cs + o.co + c] = __float2bfloat16(0.125f * s);
}

// gin[child] (+)= gout[parent] / 8
__global__ void k_pool_bwd(Vol out, int C, Act gout, Act gin, int accumulate) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= out.voxels() * C) return;
  const long long m = e / C;
  const int c = (int)(e % C);
  int b, z, y, x;
  decode(m, out, b, z, y, x);
  const int D2 = out.D * 2, H2 = out.H * 2, W2 = out.W * 2;
  const float g = 0.125f * __bfloat162float(gout.p[m * gout.cs + gout.co + c]);
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const long long sv = (((long long)b * D2 + 2 * z + (q >> 2)) * H2 + 2 * y + ((q >> 1) & 1)) * W2 + 2 * x + (q & 1);
    bf16* d = gin.p + sv * gin.cs + gin.co + c;
    *d = __float2bfloat16(accumulate ? __bfloat162float(*d) + g : g);
  }
}

// nearest-neighbour upsampling x2: fine voxel takes its parent's value.
__global__ void k_up_fwd(Vol fine, int C, Act in, Act o) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= fine.voxels() * C) return;
  const long long m = e / C;
  const int c = (int)(e % C);
  int b, z, y, x;
  decode(m, fine, b, z, y, x);
  const long long pv = (((long long)b * (fine.D / 2) + z / 2) * (fine.H / 2) + y / 2) * (fine.W / 2) + x / 2;
  o.p[m * o.cs + o.co + c] = in.p[pv * in.cs + in.co + c];
}

// parent gradient = sum of its eight children's gradients.
__global__ void k_up_bwd(Vol coarse, int C, Act gfine, Act gout) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= coarse.voxels() * C) return;
  const long long m = e / C;
  const int c = (int)(e % C);
  int b, z, y, x;
  decode(m, coarse, b, z, y, x);
  const int D2 = coarse.D * 2, H2 = coarse.H * 2, W2 = coarse.W * 2;
  float s = 0.f;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const long long sv = (((long long)b * D2 + 2 * z + (q >> 2)) * H2 + 2 * y + ((q >> 1) & 1)) * W2 + 2 * x + (q & 1);
    s += __bfloat162float(gfine.p[sv * gfine.cs + gfine.co + c]);
  }
  gout.p[m * gout.cs + gout.co + c] = __float2bfloat16(s);
}

// 1x1 head: out[v] = sum_c w[c] * in[v][c] + b   (FP32 output)
__global__ void k_head_fwd(long long M, int C, Act in, const float* __restrict__ w, float* __restrict__ out) {
  const long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= M) return;
  float s = w[C];
  for (int c = 0; c < C; ++c) s = fmaf(w[c], __bfloat162float(in.p[m * in.cs + in.co + c]), s);
  out[m] = s;
}

// gin[v][c] = gout[v] * w[c]; dw[c] += sum_v gout[v] * in[v][c]; dw[C] += sum_v gout[v]
__global__ void k_head_bwd(long long M, int C, Act in, const float* __restrict__ w, const float* __restrict__ gout,
                           Act gin, float* __restrict__ dw) {
  __shared__ float s[33];
  if (threadIdx.x <= C) s[threadIdx.x] = 0.f;
  __syncthreads();
  const long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (m < M) {
    const float g = gout[m];
    for (int c = 0; c < C; ++c) {
      gin.p[m * gin.cs + gin.co + c] = __float2bfloat16(g * w[c]);
      atomicAdd(&s[c], g * __bfloat162float(in.p[m * in.cs + in.co + c]));
    }
    atomicAdd(&s[C], g);
  }
  __syncthreads();
  if (threadIdx.x <= C) atomicAdd(&dw[threadIdx.x], s[threadIdx.x]);
}

// mean squared error: g = 2 (out - t) / M, loss += sum (out - t)^2 / M
__global__ void k_mse(long long M, const float* __restrict__ out, const float* __restrict__ t, float* __restrict__ g,
                      double* loss) {
  const long long m = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  float d = 0.f;
  if (m < M) {
    d = out[m] - t[m];
    g[m] = 2.f * d / (float)M;
  }
  float s = d * d;
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0 && s != 0.f) atomicAdd(loss, (double)s / (double)M);
}

// Adam (FP32 master weights) and the BF16 copies the kernels read: the forward
// layout [n][tap][k] and the transposed input-gradient layout [k][tap][n].
__global__ void k_adam(int n, float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m1,
                       float* __restrict__ m2, float lr, float b1, float b2, float c1, float c2, float eps) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const float gg = g[e];
  const float a = b1 * m1[e] + (1.f - b1) * gg;
  const float b = b2 * m2[e] + (1.f - b2) * gg * gg;
  m1[e] = a;
  m2[e] = b;
  p[e] -= lr * (a / c1) / (sqrtf(b / c2) + eps);
}

__global__ void k_cast_conv_weights(int N, int K, const float* __restrict__ w, bf16* __restrict__ wf,
                                    bf16* __restrict__ wt) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= N * 27 * K) return;
  const int k = e % K, tap = (e / K) % 27, n = e / (27 * K);
  const bf16 v = __float2bfloat16(w[e]);
  wf[e] = v;
  wt[((size_t)k * 27 + tap) * N + n] = v;
}

// ------------------------------------------------------------ launch helpers

template <int N>
void launch_conv3(cudaStream_t st, unsigned nb, const Vol& vol, Act X, int K, const bf16* W, const float* bias,
                  int relu, int sign, Act Y, int* err) {
  constexpr size_t smem = conv_smem_bytes<N>();
  static bool attr = false;   // the stages need more than the default 48 KB of dynamic shared memory
  if (!attr) {
    cudaFuncSetAttribute(k_conv3<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    attr = true;
  }
  k_conv3<N><<<nb, 128, smem, st>>>(vol, X, K, W, bias, relu, sign, Y, err);
}

void conv(cudaStream_t st, const Vol& vol, Act X, int K, const bf16* W, const float* bias, int relu, int sign, Act Y,
          int N, int* err) {
  const long long M = vol.voxels();
  const unsigned nb = (unsigned)((M + 127) / 128);
  switch (N) {
    case 16: launch_conv3<16>(st, nb, vol, X, K, W, bias, relu, sign, Y, err); break;
    case 32: launch_conv3<32>(st, nb, vol, X, K, W, bias, relu, sign, Y, err); break;
    case 48: launch_conv3<48>(st, nb, vol, X, K, W, bias, relu, sign, Y, err); break;
    case 64: launch_conv3<64>(st, nb, vol, X, K, W, bias, relu, sign, Y, err); break;
    case 96: launch_conv3<96>(st, nb, vol, X, K, W, bias, relu, sign, Y, err); break;
    default: break;
  }
}

template <int N>
void launch_wgrad_tc(cudaStream_t st, const Vol& vol, Act dZ, Act X, int K, float* dW, int* err) {
  constexpr size_t smem = wgrad_smem_bytes<N>();
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_wgrad_tc<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    attr = true;
  }
  const long long M = vol.voxels();
  const int rowblocks = (27 * K + 127) / 128;
  // about two blocks per SM: split the voxels into chunks of whole stages (64 voxels)
  long long chunks = std::max(1ll, std::min((304ll + rowblocks - 1) / rowblocks, (M + 255) / 256));
  long long chunk = (M + chunks - 1) / chunks;
  chunk = (chunk + 63) / 64 * 64;
  chunks = (M + chunk - 1) / chunk;
  k_wgrad_tc<N><<<dim3((unsigned)rowblocks, (unsigned)chunks), 128, smem, st>>>(vol, dZ, X, K, dW, chunk, err);
}

void wgrad(cudaStream_t st, const Vol& vol, Act dZ, int N, Act X, int K, float* dW, int* err) {
  switch (N) {
    case 16: launch_wgrad_tc<16>(st, vol, dZ, X, K, dW, err); break;
    case 32: launch_wgrad_tc<32>(st, vol, dZ, X, K, dW, err); break;
    case 64: launch_wgrad_tc<64>(st, vol, dZ, X, K, dW, err); break;
    default: wgrad_cuda_cores(st, vol, dZ, N, X, K, dW); break;
  }
}

void wgrad_cuda_cores(cudaStream_t st, const Vol& vol, Act dZ, int N, Act X, int K, float* dW) {
  const long long M = vol.voxels();
  const long long chunk = 4096;
  dim3 grid((unsigned)((M + chunk - 1) / chunk), 27);
  const size_t smem = (size_t)kWgTile * (N + K) * sizeof(float);
  k_wgrad<<<grid, 256, smem, st>>>(vol, dZ, N, X, K, dW, chunk);
}

void bias_grad(cudaStream_t st, long long M, Act dZ, int N, float* db) {
  k_bias_grad<<<256, 256, 0, st>>>(M, dZ, N, db);
}

void relu_bwd(cudaStream_t st, long long M, int C, Act dY, Act Y) {
  k_relu_bwd<<<(unsigned)((M * C + 255) / 256), 256, 0, st>>>(M, C, dY, Y);
}

void pool_fwd(cudaStream_t st, const Vol& out, int C, Act in, Act o) {
  k_pool_fwd<<<(unsigned)((out.voxels() * C + 255) / 256), 256, 0, st>>>(out, C, in, o);
}

void pool_bwd(cudaStream_t st, const Vol& out, int C, Act gout, Act gin, int accumulate) {
  k_pool_bwd<<<(unsigned)((out.voxels() * C + 255) / 256), 256, 0, st>>>(out, C, gout, gin, accumulate);
}

void up_fwd(cudaStream_t st, const Vol& fine, int C, Act in, Act o) {
  k_up_fwd<<<(unsigned)((fine.voxels() * C + 255) / 256), 256, 0, st>>>(fine, C, in, o);
}

void up_bwd(cudaStream_t st, const Vol& coarse, int C, Act gfine, Act gout) {
  k_up_bwd<<<(unsigned)((coarse.voxels() * C + 255) / 256), 256, 0, st>>>(coarse, C, gfine, gout);
}

void head_fwd(cudaStream_t st, long long M, int C, Act in, const float* w, float* out) {
  k_head_fwd<<<(unsigned)((M + 255) / 256), 256, 0, st>>>(M, C, in, w, out);
}

void head_bwd(cudaStream_t st, long long M, int C, Act in, const float* w, const float* gout, Act gin, float* dw) {
  k_head_bwd<<<(unsigned)((M + 255) / 256), 256, 0, st>>>(M, C, in, w, gout, gin, dw);
}

void mse(cudaStream_t st, long long M, const float* out, const float* t, float* g, double* loss) {
  k_mse<<<(unsigned)((M + 255) / 256), 256, 0, st>>>(M, out, t, g, loss);
}

void adam(cudaStream_t st, int n, float* p, const float* g, float* m1, float* m2, float lr, int step) {
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
  k_adam<<<(n + 255) / 256, 256, 0, st>>>(n, p, g, m1, m2, lr, b1, b2, c1, c2, 1e-8f);
}

void cast_conv_weights(cudaStream_t st, int N, int K, const float* w, bf16* wf, bf16* wt) {
  k_cast_conv_weights<<<(N * 27 * K + 255) / 256, 256, 0, st>>>(N, K, w, wf, wt);
}

}  // namespace unet
}  // namespace ib3d
