// FP32 red-black SOR sweep on colour-packed arrays (the inner solve of the FP64
// defect-correction loop).
//
// In the padded Fortran layout a colour pass touches every cache line of e, r and
// the flags although it updates half the cells. Here each colour lives in its own
// array: the cells of colour c in row (j,k) are i = i_c + 2m, m = 0..nx/2-1, with
// i_c = 2 if cell (2,j,k) has colour c, else 3 (red is (i+j+k) odd,
// subSearch.f90:562). The y and z neighbours of (c, m) are the other colour's
// entries with the same m in rows j+-1, k+-1; the x neighbours are its entries m-1
// and m (i_c = 2) or m and m+1 (i_c = 3). Rows carry zero ghost entries on both
// sides and the arrays carry zero ghost rows, standing in for the grid's ghost
// layer. Entry m of a row is stored at m + 4 (rows are 16-byte aligned), so a
// thread updates four consecutive cells of its colour with float4 loads and
// stores; the x coefficients of those four cells come regrouped as float4 (Grid1D::axp)
// so that the warp reads them without strided scalar loads. A non-fluid cell carries
// a NaN right-hand side and keeps its value, 0, so no flag array is read.
//
// Per cell the arithmetic and its order are those of the one-array form (k_sor32
// in k_pressure.cu), so both give the same bits.
#include <utility>

#include "ib3d_internal.cuh"

namespace ib3d {

// Row length of a packed colour array: the row's cells rounded up to whole float4
// groups, plus 4 entries of left padding (ghost at 3) and 4 of right padding.
int packed_row_length(int nx) { return 4 * (((nx >> 1) + 3) >> 2) + 8; }

// Updates the four cells of one thread. FIRST: the row starts (i = 2) with the
// colour being updated, so cell c's x neighbours are other-colour entries c-1 and c
// (else c and c+1) of the row, ox[] holding entries -1..4.
template <bool FIRST>
__device__ __forceinline__ void update4(const float (&rv)[4], float (&ev)[4], const float (&ox)[6],
                                        const float (&sv)[4], const float (&nv)[4], const float (&bv)[4],
                                        const float (&tv)[4], const float4 a0, const float4 a1, const float4 a2,
                                        float ay0, float ay1, float ay2, float az0, float az1, float az2,
                                        float omega, float om1) {
  const float ax0[4] = {a0.x, a0.y, a0.z, a0.w};
  const float ax1[4] = {a1.x, a1.y, a1.z, a1.w};
  const float ax2[4] = {a2.x, a2.y, a2.z, a2.w};
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const float r = rv[c];
    if (r == r) {   // fluid cell (NaN marks the others, including the row's padding)
      const float W = FIRST ? ox[c] : ox[c + 1];
      const float E = FIRST ? ox[c + 1] : ox[c + 2];
      float num = r;
      num = fmaf(-ax0[c], W, num);
      num = fmaf(-ax2[c], E, num);
      num = fmaf(-ay0, sv[c], num);
      num = fmaf(-ay2, nv[c], num);
      num = fmaf(-az0, bv[c], num);
      num = fmaf(-az2, tv[c], num);
      const float diag = ax1[c] + ay1 + az1;
      ev[c] = sor32_update(ev[c], num, diag, omega, om1);
    }
  }
}

// One colour pass. Block (32, kRows): a warp covers 32 float4 groups of one row
// (j, k), so the row's colour phase is uniform across the warp; grid (ceil(nq/32),
// ceil(ny/kRows), ceil(nz/kPlanes)) maps the rest without integer division. A
// thread updates its four cells in kPlanes consecutive planes, carrying the other
// colour's centre and upper plane over to the next plane instead of loading them
// again. The x neighbours beyond the thread's own four cells (the other colour's
// last entry of group q-1 and first of group q+1) come from the neighbouring
// lanes' centre values by shuffles; only the lanes at the ends of a warp's span
// load them. The kernel is held to 64 registers (8 blocks of 128 threads per SM):
// the pass is bound by the L1 data pipe with the arrays resident in L2, and the
// warps that fit hide the load latency better than a longer unroll would.
// Offsets are 32-bit (a packed array holds fewer than 2^31 entries, checked at
// allocation).
constexpr int kPlanes = 8;
constexpr int kRows = 4;

template <int COLOR>
__global__ void __launch_bounds__(32 * kRows, 8) k_sor32p(Dims d, Grid1D g, const float* __restrict__ r_own,
                                                          float* __restrict__ e_own, const float* __restrict__ e_oth,
                                                          int Lp, float omega, float om1) {
  // launched with programmatic dependent launch: the blocks may start while the
  // previous pass drains; wait for it (and its writes) before touching memory
  asm volatile("griddepcontrol.wait;" ::: "memory");
  const int nq = ((d.nx >> 1) + 3) >> 2;
  const int lane = threadIdx.x;
  const int q = blockIdx.x * 32 + lane;
  const int j = blockIdx.y * kRows + threadIdx.y + 2;
  const int k0 = blockIdx.z * kPlanes + 2;
  if (j <= d.ny + 1) {   // uniform across the warp, so the shuffles see all lanes
    const bool active = q < nq;
    const bool load_left = lane == 0, load_right = lane == 31 || q + 1 >= nq;
    const int plane = (d.ny + 2) * Lp;
    const int sj = (j - 1) * Lp + 4 * q + 4;
    const float ay0 = g.acy32[0][j - 1], ay1 = g.acy32[1][j - 1], ay2 = g.acy32[2][j - 1];
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    float4 ob = active ? *reinterpret_cast<const float4*>(e_oth + (k0 - 2) * plane + sj) : z4;
    float4 ox = active ? *reinterpret_cast<const float4*>(e_oth + (k0 - 1) * plane + sj) : z4;
#pragma unroll
    for (int kk = 0; kk < kPlanes; ++kk) {
      const int k = k0 + kk;
      if (k > d.nz + 1) break;
      const int s0 = (k - 1) * plane + sj;
      // does this row start (i = 2) with the colour being updated?
      const bool own_first = (COLOR == 0) == (((j + k) & 1) == 1);
      float4 rr = z4, eo = z4, os = z4, on = z4, ot = z4;
      if (active) {
        rr = *reinterpret_cast<const float4*>(r_own + s0);
        eo = *reinterpret_cast<const float4*>(e_own + s0);
        os = *reinterpret_cast<const float4*>(e_oth + s0 - Lp);
        on = *reinterpret_cast<const float4*>(e_oth + s0 + Lp);
        ot = *reinterpret_cast<const float4*>(e_oth + s0 + plane);
      }
      float left = __shfl_up_sync(0xffffffffu, ox.w, 1);
      float right = __shfl_down_sync(0xffffffffu, ox.x, 1);
      if (active && load_left) left = e_oth[s0 - 1];
      if (active && load_right) right = e_oth[s0 + 4];
      const float oxa[6] = {left, ox.x, ox.y, ox.z, ox.w, right};
      const float rv[4] = {rr.x, rr.y, rr.z, rr.w};
      const float sv[4] = {os.x, os.y, os.z, os.w};
      const float nv[4] = {on.x, on.y, on.z, on.w};
      const float bv[4] = {ob.x, ob.y, ob.z, ob.w};
      const float tv[4] = {ot.x, ot.y, ot.z, ot.w};
      float ev[4] = {eo.x, eo.y, eo.z, eo.w};
      const float az0 = g.acz32[0][k - 1], az1 = g.acz32[1][k - 1], az2 = g.acz32[2][k - 1];
      if (active) {
        const int sp = own_first ? 0 : 1;
        const float4 a0 = g.axp[sp][0][q], a1 = g.axp[sp][1][q], a2 = g.axp[sp][2][q];
        if (own_first)
          update4<true>(rv, ev, oxa, sv, nv, bv, tv, a0, a1, a2, ay0, ay1, ay2, az0, az1, az2, omega, om1);
        else
          update4<false>(rv, ev, oxa, sv, nv, bv, tv, a0, a1, a2, ay0, ay1, ay2, az0, az1, az2, omega, om1);
        *reinterpret_cast<float4*>(e_own + s0) = make_float4(ev[0], ev[1], ev[2], ev[3]);
      }
      ob = ox;
      ox = ot;
    }
  }
  // the next pass may launch now; its griddepcontrol.wait still waits for this grid
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// One whole red-black sweep per launch: the red pass and the black pass fused into a
// z-wavefront. A block owns kFY rows (j) by kFZ planes (k) over the full x extent of
// the packed rows (blockDim.x = 32 x warps, one float4 group per thread; blockDim.y
// = kFY + 2 rows) and marches k upward. At plane k every row thread updates the red
// cells of its row from the black values before the sweep (planes k-1, k, k+1 kept in
// registers, the rows j+-1 loaded), puts the new red row into a three-plane ring in
// shared memory, and after one barrier the inner rows update their black cells of
// plane k-1 from the new red values (rows j+-1 from the ring, planes k-2 and k from
// registers). Black at the block's edges needs new red values one row and one plane
// beyond the block, so those are computed by this block too (the neighbouring blocks
// compute the same values). Every block therefore reads the values before the sweep
// from one pair of arrays (e_red, e_black) and writes the new values to a second pair
// (n_red, n_black): no block overwrites what another still has to read, and the
// caller swaps the pairs after each sweep. Every fluid cell is written by exactly one
// block; the other entries hold 0 in both pairs. Per cell the arithmetic is
// update4's, in the same order, so the results are bit-identical to two k_sor32p
// passes. Each array is read once per sweep (plus the halo rows and planes), against
// the other colour's array twice in the two-pass form.
constexpr int kFY = 8;
constexpr int kFZ = 16;

template <bool FIRST>
__device__ __forceinline__ void update_group(const float4 r4, float4& e4, const float (&ox)[6], const float4 s4,
                                             const float4 n4, const float4 b4, const float4 t4, const float4 a0,
                                             const float4 a1, const float4 a2, float ay0, float ay1, float ay2,
                                             float az0, float az1, float az2, float omega, float om1) {
  const float rv[4] = {r4.x, r4.y, r4.z, r4.w};
  const float sv[4] = {s4.x, s4.y, s4.z, s4.w};
  const float nv[4] = {n4.x, n4.y, n4.z, n4.w};
  const float bv[4] = {b4.x, b4.y, b4.z, b4.w};
  const float tv[4] = {t4.x, t4.y, t4.z, t4.w};
  float ev[4] = {e4.x, e4.y, e4.z, e4.w};
  update4<FIRST>(rv, ev, ox, sv, nv, bv, tv, a0, a1, a2, ay0, ay1, ay2, az0, az1, az2, omega, om1);
  e4 = make_float4(ev[0], ev[1], ev[2], ev[3]);
}

__global__ void __launch_bounds__(640) k_sor32f(Dims d, Grid1D g, const float* __restrict__ r_red,
                                                 const float* __restrict__ r_black,
                                                 const float* __restrict__ e_red, const float* __restrict__ e_black,
                                                 float* __restrict__ n_red, float* __restrict__ n_black, int Lp,
                                                 float omega, float om1) {
  extern __shared__ float4 ring[];   // [3][kFY + 2][blockDim.x]
  asm volatile("griddepcontrol.wait;" ::: "memory");
  const int nq = ((d.nx >> 1) + 3) >> 2;
  const int nqp = blockDim.x;
  const int q = threadIdx.x, lane = q & 31;
  const int tr = threadIdx.y;                       // 0 and kFY + 1: halo rows
  const int j = blockIdx.x * kFY + 1 + tr;          // row of this thread
  const int k0 = blockIdx.y * kFZ + 2;              // first plane the block owns
  const int k1 = min(k0 + kFZ, d.nz + 2);           // one past the last
  const bool row_cell = j >= 2 && j <= d.ny + 1;    // the row holds cells (not a ghost row)
  const bool row_in = j <= d.ny + 2;                // the row exists in the arrays
  const bool inner = tr >= 1 && tr <= kFY && row_cell;
  const bool active = q < nq && row_in;
  const bool load_left = lane == 0, load_right = lane == 31 || q + 1 >= nq;
  const int plane = (d.ny + 2) * Lp;
  const int sj = (j - 1) * Lp + 4 * q + 4;
  const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
  float ay0 = 0.f, ay1 = 0.f, ay2 = 0.f;
  if (row_cell) {
    ay0 = g.acy32[0][j - 1];
    ay1 = g.acy32[1][j - 1];
    ay2 = g.acy32[2][j - 1];
  }
  float4* ringp = ring + tr * nqp + q;
  const int ring_plane = (kFY + 2) * nqp;
  // black values before the sweep at planes k-1 and k of this row (registers), for
  // the first red plane k0-1 (the ghost plane when k0 = 2: no red update there)
  const int kr0 = k0 - 1;
  float4 bm = z4, b0 = z4;
  if (active && kr0 >= 2) {
    bm = *reinterpret_cast<const float4*>(e_black + (kr0 - 2) * plane + sj);
    b0 = *reinterpret_cast<const float4*>(e_black + (kr0 - 1) * plane + sj);
  } else if (active) {
    b0 = *reinterpret_cast<const float4*>(e_black + (kr0 - 1) * plane + sj);
  }
  float4 rm2 = z4, rm1 = z4;   // new red values at planes k-2, k-1 of this row
  for (int k = kr0; k <= k1; ++k) {
    // ---- red cells of plane k
    const bool plane_cell = k >= 2 && k <= d.nz + 1;
    const int s0 = (k - 1) * plane + sj;
    float4 bp = z4;   // black before the sweep at plane k+1
    if (active && k + 1 <= d.nz + 2) bp = *reinterpret_cast<const float4*>(e_black + s0 + plane);
    float4 rn = z4;
    const bool red_here = plane_cell && row_cell;   // warp-uniform
    if (red_here) {
      float left = __shfl_up_sync(0xffffffffu, b0.w, 1);
      float right = __shfl_down_sync(0xffffffffu, b0.x, 1);
      if (active) {
        if (load_left) left = e_black[s0 - 1];
        if (load_right) right = e_black[s0 + 4];
        const float4 rr = *reinterpret_cast<const float4*>(r_red + s0);
        rn = *reinterpret_cast<const float4*>(e_red + s0);
        const float4 os = *reinterpret_cast<const float4*>(e_black + s0 - Lp);
        const float4 on = *reinterpret_cast<const float4*>(e_black + s0 + Lp);
        const float oxa[6] = {left, b0.x, b0.y, b0.z, b0.w, right};
        const float az0 = g.acz32[0][k - 1], az1 = g.acz32[1][k - 1], az2 = g.acz32[2][k - 1];
        const bool own_first = ((j + k) & 1) == 1;   // red is (i+j+k) odd: does the row start with red?
        const int sp = own_first ? 0 : 1;
        const float4 a0 = g.axp[sp][0][q], a1 = g.axp[sp][1][q], a2 = g.axp[sp][2][q];
        if (own_first)
          update_group<true>(rr, rn, oxa, os, on, bm, bp, a0, a1, a2, ay0, ay1, ay2, az0, az1, az2, omega, om1);
        else
          update_group<false>(rr, rn, oxa, os, on, bm, bp, a0, a1, a2, ay0, ay1, ay2, az0, az1, az2, omega, om1);
        if (inner && k >= k0 && k < k1) *reinterpret_cast<float4*>(n_red + s0) = rn;
      }
    }
    const int slot = (k - kr0) % 3;
    ringp[slot * ring_plane] = rn;
    __syncthreads();
    // ---- black cells of plane k-1, from the new red values
    const int kb = k - 1;
    if (inner && kb >= k0 && kb < k1) {   // warp-uniform
      const int slot_b = (kb - kr0) % 3;
      const float4* rb_row = ring + slot_b * ring_plane + tr * nqp;
      float left = __shfl_up_sync(0xffffffffu, rm1.w, 1);
      float right = __shfl_down_sync(0xffffffffu, rm1.x, 1);
      if (active) {
        if (load_left) left = q > 0 ? rb_row[q - 1].w : 0.f;
        if (load_right) right = q + 1 < nqp ? rb_row[q + 1].x : 0.f;
        const int sb = s0 - plane;
        const float4 rr = *reinterpret_cast<const float4*>(r_black + sb);
        float4 en = bm;   // black before the sweep at plane k-1
        const float4 os = rb_row[q - nqp], on = rb_row[q + nqp];
        const float oxa[6] = {left, rm1.x, rm1.y, rm1.z, rm1.w, right};
        const float az0 = g.acz32[0][kb - 1], az1 = g.acz32[1][kb - 1], az2 = g.acz32[2][kb - 1];
        const bool own_first = ((j + kb) & 1) == 0;   // black is (i+j+k) even
        const int sp = own_first ? 0 : 1;
        const float4 a0 = g.axp[sp][0][q], a1 = g.axp[sp][1][q], a2 = g.axp[sp][2][q];
        if (own_first)
          update_group<true>(rr, en, oxa, os, on, rm2, rn, a0, a1, a2, ay0, ay1, ay2, az0, az1, az2, omega, om1);
        else
          update_group<false>(rr, en, oxa, os, on, rm2, rn, a0, a1, a2, ay0, ay1, ay2, az0, az1, az2, omega, om1);
        *reinterpret_cast<float4*>(n_black + sb) = en;
      }
    }
    bm = b0;
    b0 = bp;
    rm2 = rm1;
    rm1 = rn;
  }
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// pc += e at every interior cell, reading e from its colour's packed array, then
// zero e (the next inner solve starts from e = 0).
__global__ void k_accumulate_packed(Dims d, double* __restrict__ pc, float* __restrict__ e_red,
                                    float* __restrict__ e_black, int Lp) {
  const unsigned tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= (unsigned)d.nx * (unsigned)d.ny * (unsigned)d.nz) return;
  const int i = (int)(tid % (unsigned)d.nx) + 2;
  const unsigned t = tid / (unsigned)d.nx;
  const int j = (int)(t % (unsigned)d.ny) + 2, k = (int)(t / (unsigned)d.ny) + 2;
  const long long s = ((long long)(k - 1) * (d.ny + 2) + (j - 1)) * Lp + ((i - 2) >> 1) + 4;
  float* e = ((i + j + k) & 1) ? e_red : e_black;
  const float x = e[s];
  if (x != 0.0f) {
    const long long o = d.at(i, j, k);
    pc[o] = pc[o] + (double)x;
    e[s] = 0.0f;
  }
}

void launch_sor32_packed(ib3d_ctx* c, int color, float omega, float om1) {
  const Dims& d = c->d;
  const int nq = ((d.nx >> 1) + 3) >> 2;
  const dim3 grid((unsigned)((nq + 31) / 32), (unsigned)((d.ny + kRows - 1) / kRows),
                  (unsigned)((d.nz + kPlanes - 1) / kPlanes)),
      block(32, kRows);
  // programmatic dependent launch: the colour passes run back to back, and the launch
  // and block start-up of one overlap the tail of the previous one
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = 0;
  cfg.stream = c->st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  const float* r = c->rp[color];
  float* e = c->ep[color];
  const float* o = c->ep[1 - color];
  if (color == 0)
    cudaLaunchKernelEx(&cfg, k_sor32p<0>, d, c->g, r, e, o, c->packed_lp, omega, om1);
  else
    cudaLaunchKernelEx(&cfg, k_sor32p<1>, d, c->g, r, e, o, c->packed_lp, omega, om1);
}

// One fused sweep: reads the sweep's input from ep[], writes its result to epn[] and
// swaps the two pairs, so ep[] holds the current correction afterwards.
void launch_sor32_fused(ib3d_ctx* c, float omega, float om1) {
  const Dims& d = c->d;
  const int nq = ((d.nx >> 1) + 3) >> 2;
  const int wx = (nq + 31) / 32;
  const dim3 grid((unsigned)((d.ny + kFY - 1) / kFY), (unsigned)((d.nz + kFZ - 1) / kFZ)),
      block((unsigned)(32 * wx), (unsigned)(kFY + 2));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = sizeof(float4) * 3 * (kFY + 2) * 32 * wx;
  cfg.stream = c->st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, k_sor32f, d, c->g, (const float*)c->rp[0], (const float*)c->rp[1],
                     (const float*)c->ep[0], (const float*)c->ep[1], c->epn[0], c->epn[1], c->packed_lp, omega, om1);
  std::swap(c->ep[0], c->epn[0]);
  std::swap(c->ep[1], c->epn[1]);
}

// Largest nx the fused sweep takes: its block spans a whole packed row.
bool fused_sweep_fits(int nx) { return ((((nx >> 1) + 3) >> 2) + 31) / 32 * 32 * (kFY + 2) <= 640; }

void launch_accumulate_packed(ib3d_ctx* c) {
  const long long n = (long long)c->d.nx * c->d.ny * c->d.nz;
  k_accumulate_packed<<<(unsigned)((n + kBlock - 1) / kBlock), kBlock, 0, c->st>>>(c->d, c->pc, c->ep[0], c->ep[1],
                                                                                   c->packed_lp);
}

}  // namespace ib3d
