// Fused FP32 red-black SOR sweep: both colours of one sweep in a single pass over
// memory (the inner solve of the FP64 defect-correction loop).
//
// A two-kernel sweep (red pass, then black pass) moves each array through the
// memory system twice per sweep. Here each block owns a 64 x 8 (x,y) tile and a
// chunk of z planes and marches through z: at plane step kk it computes the new
// red values of plane kk on the tile plus a one-cell ring, then the new black
// values of plane kk-1 on the tile (which need the new red values of planes
// kk-2..kk), and stores plane kk-1. Old values are read from one buffer and new
// ones written to another, and the red ring is recomputed by every block that needs
// it, so no block reads another block's results within a sweep: the update is
// exactly the red-then-black sweep (red reads old black, black reads new red)
// with the two-kernel form's FP32 operation order, hence the same bits.
//
// Non-fluid cells carry a NaN right-hand side (written by the residual kernel), so
// no flag array is read: a NaN r keeps the cell at its old value, 0.
//
// Shared memory per block: four e planes (tile + 2-cell ring), three r planes and
// three new-red planes (tile + 1-cell ring) = 28.8 KB.
#include "ib3d_internal.cuh"

namespace ib3d {

namespace {
constexpr int TX = 64, TY = 8, NT = 256;
constexpr int EX = TX + 4, EY = TY + 4;   // e tile with a 2-cell ring
constexpr int RX = TX + 2, RY = TY + 2;   // r / new-red tile with a 1-cell ring
__device__ __forceinline__ int mod3(int k) { return ((k % 3) + 3) % 3; }
__device__ __forceinline__ float qnan() { return __int_as_float(0x7fc00000); }
}  // namespace

__global__ void __launch_bounds__(NT) k_sor32_fused(Dims d, Grid1D g, const float* __restrict__ r,
                                                    const float* __restrict__ ein, float* __restrict__ eout,
                                                    float omega, float om1, int lz) {
  __shared__ float se[4][EY][EX];
  __shared__ float sr[3][RY][RX];
  __shared__ float sn[3][RY][RX];
  const int tid = threadIdx.x;
  const int x0 = 2 + blockIdx.x * TX, y0 = 2 + blockIdx.y * TY;
  const int k0 = 2 + blockIdx.z * lz, k1 = min(k0 + lz - 1, d.nz + 1);

  auto load_e = [&](int kk) {
    float(*dst)[EX] = se[kk & 3];
    const bool plane_ok = kk >= 1 && kk <= d.nz + 2;
    for (int q = tid; q < EX * EY; q += NT) {
      const int lx = q % EX - 2, ly = q / EX - 2;
      const int i = x0 + lx, j = y0 + ly;
      float v = 0.f;
      if (plane_ok && i >= 1 && i <= d.nx + 2 && j >= 1 && j <= d.ny + 2) v = ein[d.at(i, j, kk)];
      dst[ly + 2][lx + 2] = v;
    }
  };
  auto load_r = [&](int kk) {
    float(*dst)[RX] = sr[mod3(kk)];
    const bool plane_ok = kk >= 2 && kk <= d.nz + 1;
    for (int q = tid; q < RX * RY; q += NT) {
      const int lx = q % RX - 1, ly = q / RX - 1;
      const int i = x0 + lx, j = y0 + ly;
      float v = qnan();
      if (plane_ok && i >= 2 && i <= d.nx + 1 && j >= 2 && j <= d.ny + 1) v = r[d.at(i, j, kk)];
      dst[ly + 1][lx + 1] = v;
    }
  };

  load_e(k0 - 2);
  load_e(k0 - 1);
  for (int kk = k0 - 1; kk <= k1 + 1; ++kk) {
    load_e(kk + 1);
    load_r(kk);
    __syncthreads();
    // new red values of plane kk on the tile and its one-cell ring
    {
      const float(*em)[EX] = se[(kk - 1) & 3];
      const float(*e0)[EX] = se[kk & 3];
      const float(*ep)[EX] = se[(kk + 1) & 3];
      const float(*rr)[RX] = sr[mod3(kk)];
      float(*dn)[RX] = sn[mod3(kk)];
      for (int q = tid; q < (RX / 2) * RY; q += NT) {
        const int ly = q / (RX / 2) - 1, m = q % (RX / 2);
        const int j = y0 + ly;
        const int base = -1 + 2 * m;
        const int lx = base + ((x0 + base + j + kk + 1) & 1);   // (i+j+kk) odd: red
        const int i = x0 + lx;
        const int ex = lx + 2, ey = ly + 2;
        float val = e0[ey][ex];
        const float rv = rr[ly + 1][lx + 1];
        if (rv == rv) {
          float num = rv;
          num = fmaf(-g.acx32[0][i - 1], e0[ey][ex - 1], num);
          num = fmaf(-g.acx32[2][i - 1], e0[ey][ex + 1], num);
          num = fmaf(-g.acy32[0][j - 1], e0[ey - 1][ex], num);
          num = fmaf(-g.acy32[2][j - 1], e0[ey + 1][ex], num);
          num = fmaf(-g.acz32[0][kk - 1], em[ey][ex], num);
          num = fmaf(-g.acz32[2][kk - 1], ep[ey][ex], num);
          const float diag = g.acx32[1][i - 1] + g.acy32[1][j - 1] + g.acz32[1][kk - 1];
          val = fmaf(om1, val, omega * __fdiv_rn(num, diag));
        }
        dn[ly + 1][lx + 1] = val;
      }
    }
    __syncthreads();
    // new black values of plane kk-1 on the tile; store plane kk-1
    const int km = kk - 1;
    if (km >= k0) {
      const int ly = tid >> 5, m = tid & 31;
      const int j = y0 + ly;
      const int lxa = 2 * m;
      const int ia = x0 + lxa;
      const int lxb = lxa + ((ia + j + km) & 1);    // (i+j+km) even: black
      const int lxr = 2 * lxa + 1 - lxb;
      const float(*nm)[RX] = sn[mod3(km - 1)];
      const float(*n0)[RX] = sn[mod3(km)];
      const float(*np)[RX] = sn[mod3(km + 1)];
      const int ib = x0 + lxb;
      const int bx = lxb + 1, by = ly + 1;
      float bval = se[km & 3][ly + 2][lxb + 2];
      const float rv = sr[mod3(km)][by][bx];
      if (rv == rv) {
        float num = rv;
        num = fmaf(-g.acx32[0][ib - 1], n0[by][bx - 1], num);
        num = fmaf(-g.acx32[2][ib - 1], n0[by][bx + 1], num);
        num = fmaf(-g.acy32[0][j - 1], n0[by - 1][bx], num);
        num = fmaf(-g.acy32[2][j - 1], n0[by + 1][bx], num);
        num = fmaf(-g.acz32[0][km - 1], nm[by][bx], num);
        num = fmaf(-g.acz32[2][km - 1], np[by][bx], num);
        const float diag = g.acx32[1][ib - 1] + g.acy32[1][j - 1] + g.acz32[1][km - 1];
        bval = fmaf(om1, bval, omega * __fdiv_rn(num, diag));
      }
      const float rval = n0[by][lxr + 1];
      if (j <= d.ny + 1) {
        const int ir = x0 + lxr;
        if (ib <= d.nx + 1) eout[d.at(ib, j, km)] = bval;
        if (ir <= d.nx + 1) eout[d.at(ir, j, km)] = rval;
      }
    }
  }
}

void launch_sor32_fused(ib3d_ctx* c, const float* ein, float* eout, float omega, float om1) {
  const Dims& d = c->d;
  const int lz = 32;
  dim3 grid((unsigned)((d.nx + TX - 1) / TX), (unsigned)((d.ny + TY - 1) / TY), (unsigned)((d.nz + lz - 1) / lz));
  k_sor32_fused<<<grid, NT, 0, c->st>>>(d, c->g, c->r32, ein, eout, omega, om1, lz);
}

}  // namespace ib3d
