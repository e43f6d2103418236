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
#include <algorithm>
#include <cstring>
#include <utility>

#include "ib3d_internal.cuh"

namespace ib3d {

// Row length of a packed colour array: the row's cells rounded up to whole float4
// groups, plus 4 entries of left padding (ghost at 3) and 4 of right padding.
int packed_row_length(int nx) { return 4 * (((nx >> 1) + 3) >> 2) + 8; }

// Two FP32 values in one 64-bit register for the packed FP32 instructions of
// sm_100 and later (fma/add/mul.rn.f32x2): each lane is rounded as the scalar
// instruction rounds it (round to nearest, subnormals kept), so an update computed
// on a pair has the bits of the two scalar updates, in half the instructions.
typedef unsigned long long f32x2;
__device__ __forceinline__ f32x2 pk2(float lo, float hi) {
  f32x2 v;
  asm("mov.b64 %0, {%1, %2};" : "=l"(v) : "f"(lo), "f"(hi));
  return v;
}
__device__ __forceinline__ void up2(f32x2 v, float& lo, float& hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ f32x2 fma2(f32x2 a, f32x2 b, f32x2 c) {
  f32x2 d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}
__device__ __forceinline__ f32x2 add2(f32x2 a, f32x2 b) {
  f32x2 d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f32x2 mul2(f32x2 a, f32x2 b) {
  f32x2 d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}

// Updates the four cells of one thread, as two pairs of cells. FIRST: the row
// starts (i = 2) with the colour being updated, so cell c's x neighbours are
// other-colour entries c-1 and c (else c and c+1) of the row, ox[] holding entries
// -1..4. a0 and a2 hold the negated x off-diagonal coefficients (Grid1D::axp), so
// fma(a0, W, num) is the scalar form's fma(-Acx(.,1), W, num); per cell the
// operations and their order are those of the one-array kernel (k_sor32).
template <bool FIRST>
__device__ __forceinline__ void update4(const float (&rv)[4], float (&ev)[4], const float (&ox)[6],
                                        const float (&sv)[4], const float (&nv)[4], const float (&bv)[4],
                                        const float (&tv)[4], const float4 a0, const float4 a1, const float4 a2,
                                        float ay0, float ay1, float ay2, float az0, float az1, float az2,
                                        float omega, float om1) {
  const float ax0[4] = {a0.x, a0.y, a0.z, a0.w};
  const float ax1[4] = {a1.x, a1.y, a1.z, a1.w};
  const float ax2[4] = {a2.x, a2.y, a2.z, a2.w};
  const f32x2 nay0 = pk2(-ay0, -ay0), nay2 = pk2(-ay2, -ay2), ay1p = pk2(ay1, ay1);
  const f32x2 naz0 = pk2(-az0, -az0), naz2 = pk2(-az2, -az2), az1p = pk2(az1, az1);
  const f32x2 om = pk2(omega, omega), om1p = pk2(om1, om1);
  // every cell is computed and a NaN right-hand side (a non-fluid cell, or the row's
  // padding) selects the old value, so the four updates run without branches
#pragma unroll
  for (int c = 0; c < 4; c += 2) {
    const int w = FIRST ? c : c + 1;   // ox index of the first cell's W neighbour
    f32x2 num = pk2(rv[c], rv[c + 1]);
    num = fma2(pk2(ax0[c], ax0[c + 1]), pk2(ox[w], ox[w + 1]), num);
    num = fma2(pk2(ax2[c], ax2[c + 1]), pk2(ox[w + 1], ox[w + 2]), num);
    num = fma2(nay0, pk2(sv[c], sv[c + 1]), num);
    num = fma2(nay2, pk2(nv[c], nv[c + 1]), num);
    num = fma2(naz0, pk2(bv[c], bv[c + 1]), num);
    num = fma2(naz2, pk2(tv[c], tv[c + 1]), num);
    float d0, d1;
    up2(add2(add2(pk2(ax1[c], ax1[c + 1]), ay1p), az1p), d0, d1);
    // sor32_update on the pair: fma(om1, e, (omega * num) * rcp(diag))
    const f32x2 q = mul2(mul2(om, num), pk2(rcp_approx(d0), rcp_approx(d1)));
    float u0, u1;
    up2(fma2(om1p, pk2(ev[c], ev[c + 1]), q), u0, u1);
    ev[c] = rv[c] == rv[c] ? u0 : ev[c];
    ev[c + 1] = rv[c + 1] == rv[c + 1] ? u1 : ev[c + 1];
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
//
// ALL_LOAD: lanes past the end of a row (when the row's groups do not fill whole
// warps) load the row's last group instead of skipping their loads, and skip only the
// store, so no branch guards the loads. The compiler then schedules the plane's loads
// earlier, which costs registers (a few spill at the 64-register cap) but keeps more
// bytes in flight: 5 % faster on arrays larger than L2 (384x256x256: 81.9 against 86.0
// us per sweep), 6 % slower where they sit in L2 (256x192x192: 24.4 against 23.0), so
// the launcher picks it by the arrays' size. Both forms give the same bits.
constexpr int kPlanes = 8;
constexpr int kRows = 4;

template <int COLOR, bool ALL_LOAD>
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
    const bool lds = ALL_LOAD || active;                // this lane loads
    const int qa = ALL_LOAD && !active ? nq - 1 : q;   // the group it loads
    const bool load_left = lane == 0, load_right = lane == 31 || q + 1 >= nq;
    const int plane = (d.ny + 2) * Lp;
    const int sj = (j - 1) * Lp + 4 * qa + 4;
    const float ay0 = g.acy32[0][j - 1], ay1 = g.acy32[1][j - 1], ay2 = g.acy32[2][j - 1];
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    float4 ob = lds ? *reinterpret_cast<const float4*>(e_oth + (k0 - 2) * plane + sj) : z4;
    float4 ox = lds ? *reinterpret_cast<const float4*>(e_oth + (k0 - 1) * plane + sj) : z4;
#pragma unroll
    for (int kk = 0; kk < kPlanes; ++kk) {
      const int k = k0 + kk;
      if (k > d.nz + 1) break;
      const int s0 = (k - 1) * plane + sj;
      // does this row start (i = 2) with the colour being updated?
      const bool own_first = (COLOR == 0) == (((j + k) & 1) == 1);
      float4 rr = z4, eo = z4, os = z4, on = z4, ot = z4;
      if (lds) {
        rr = *reinterpret_cast<const float4*>(r_own + s0);
        eo = *reinterpret_cast<const float4*>(e_own + s0);
        os = *reinterpret_cast<const float4*>(e_oth + s0 - Lp);
        on = *reinterpret_cast<const float4*>(e_oth + s0 + Lp);
        ot = *reinterpret_cast<const float4*>(e_oth + s0 + plane);
      }
      float left = __shfl_up_sync(0xffffffffu, ox.w, 1);
      float right = __shfl_down_sync(0xffffffffu, ox.x, 1);
      if (lds && load_left) left = e_oth[s0 - 1];
      if (lds && load_right) right = e_oth[s0 + 4];
      const float oxa[6] = {left, ox.x, ox.y, ox.z, ox.w, right};
      const float rv[4] = {rr.x, rr.y, rr.z, rr.w};
      const float sv[4] = {os.x, os.y, os.z, os.w};
      const float nv[4] = {on.x, on.y, on.z, on.w};
      const float bv[4] = {ob.x, ob.y, ob.z, ob.w};
      const float tv[4] = {ot.x, ot.y, ot.z, ot.w};
      float ev[4] = {eo.x, eo.y, eo.z, eo.w};
      const float az0 = g.acz32[0][k - 1], az1 = g.acz32[1][k - 1], az2 = g.acz32[2][k - 1];
      if (lds) {
        const int sp = own_first ? 0 : 1;
        const float4 a0 = g.axp[sp][0][qa], a1 = g.axp[sp][1][qa], a2 = g.axp[sp][2][qa];
        if (own_first)
          update4<true>(rv, ev, oxa, sv, nv, bv, tv, a0, a1, a2, ay0, ay1, ay2, az0, az1, az2, omega, om1);
        else
          update4<false>(rv, ev, oxa, sv, nv, bv, tv, a0, a1, a2, ay0, ay1, ay2, az0, az1, az2, omega, om1);
        if (active) *reinterpret_cast<float4*>(e_own + s0) = make_float4(ev[0], ev[1], ev[2], ev[3]);
      }
      ob = ox;
      ox = ot;
    }
  }
  // the next pass may launch now; its griddepcontrol.wait still waits for this grid
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// One colour pass with two rows per thread. A warp owns rows a = j (even) and
// b = j + 1 over kPlanes2 planes from an even plane k0, so the row phase of each
// row at each plane is fixed by the colour: row a starts with the updated colour
// at even planes exactly when COLOR is 1, row b at odd planes. The thread keeps
// the x coefficients of both phases in registers for all its planes instead of
// loading them per plane, and each row's other-colour centre values serve as the
// other row's y neighbour, so a plane of two rows loads eight float4 groups
// (r and e of both rows, the other colour at row a-1, row b+1 and both rows of
// plane k+1) against ten plus six coefficient groups for two rows of k_sor32p.
// Row b may be the top ghost row (odd ny): its other-colour values (zero) are
// read as row a's neighbours, and its own update is neither loaded nor stored.
// Per cell the arithmetic is update4's, so the bits are those of k_sor32p.
constexpr int kRows2 = 4;
constexpr int kPlanes2 = 8;
static_assert(kPlanes2 % 2 == 0, "blocks start at even planes");

__device__ __forceinline__ float4 ld4(const float* p) { return *reinterpret_cast<const float4*>(p); }

template <int COLOR>
__global__ void __launch_bounds__(32 * kRows2, 4) k_sor32p2(Dims d, Grid1D g, const float* __restrict__ r_own,
                                                                    float* __restrict__ e_own,
                                                                    const float* __restrict__ e_oth, int Lp, float omega,
                                                                    float om1) {
  const int nq = ((d.nx >> 1) + 3) >> 2;
  const int lane = threadIdx.x;
  const int q = blockIdx.x * 32 + lane;
  const int ja = blockIdx.y * (2 * kRows2) + 2 * threadIdx.y + 2;
  const int k0 = blockIdx.z * kPlanes2 + 2;
  const bool live = ja <= d.ny + 1;   // uniform across the warp, so the shuffles see all lanes
  const bool lds = live && q < nq;
  const bool rowb = ja + 1 <= d.ny + 1;
  const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
  // the coefficient tables are written by the host before the solve, never by a
  // kernel, so they load before the wait for the previous pass
  const float ya0 = live ? g.acy32[0][ja - 1] : 0.f, ya1 = live ? g.acy32[1][ja - 1] : 0.f,
              ya2 = live ? g.acy32[2][ja - 1] : 0.f;
  const float yb0 = rowb ? g.acy32[0][ja] : 0.f, yb1 = rowb ? g.acy32[1][ja] : 0.f,
              yb2 = rowb ? g.acy32[2][ja] : 0.f;
  // P: the phase of row a at even planes (and of row b at odd ones); Q the other
  const float4 p0 = lds ? g.axp[1 - COLOR][0][q] : z4, p1 = lds ? g.axp[1 - COLOR][1][q] : z4,
               p2 = lds ? g.axp[1 - COLOR][2][q] : z4;
  const float4 q0 = lds ? g.axp[COLOR][0][q] : z4, q1 = lds ? g.axp[COLOR][1][q] : z4,
               q2 = lds ? g.axp[COLOR][2][q] : z4;
  asm volatile("griddepcontrol.wait;" ::: "memory");
  if (live) {
    const bool load_left = lane == 0, load_right = lane == 31 || q + 1 >= nq;
    const int plane = (d.ny + 2) * Lp;
    const int sa = (ja - 1) * Lp + 4 * q + 4;
    float4 oba = lds ? ld4(e_oth + (k0 - 2) * plane + sa) : z4, obb = lds ? ld4(e_oth + (k0 - 2) * plane + sa + Lp) : z4;
    float4 oxa = lds ? ld4(e_oth + (k0 - 1) * plane + sa) : z4, oxb = lds ? ld4(e_oth + (k0 - 1) * plane + sa + Lp) : z4;
#pragma unroll
    for (int kk = 0; kk < kPlanes2; ++kk) {
      const int k = k0 + kk;
      if (k > d.nz + 1) break;
      const int s0 = (k - 1) * plane + sa;
      float4 ra = z4, ea = z4, rb = z4, eb = z4, osa = z4, onb = z4, ota = z4, otb = z4;
      if (lds) {
        ra = ld4(r_own + s0);
        ea = ld4(e_own + s0);
        osa = ld4(e_oth + s0 - Lp);
        ota = ld4(e_oth + s0 + plane);
        otb = ld4(e_oth + s0 + Lp + plane);
        if (rowb) {
          rb = ld4(r_own + s0 + Lp);
          eb = ld4(e_own + s0 + Lp);
          onb = ld4(e_oth + s0 + 2 * Lp);
        }
      }
      float la = __shfl_up_sync(0xffffffffu, oxa.w, 1), ra_ = __shfl_down_sync(0xffffffffu, oxa.x, 1);
      float lb = __shfl_up_sync(0xffffffffu, oxb.w, 1), rb_ = __shfl_down_sync(0xffffffffu, oxb.x, 1);
      if (lds && load_left) {
        la = e_oth[s0 - 1];
        lb = e_oth[s0 + Lp - 1];
      }
      if (lds && load_right) {
        ra_ = e_oth[s0 + 4];
        rb_ = e_oth[s0 + Lp + 4];
      }
      const float4 zc = g.acz4[k - 1];
      const float z0 = zc.x, z1 = zc.y, z2 = zc.z;
      if (lds) {
        const float xa[6] = {la, oxa.x, oxa.y, oxa.z, oxa.w, ra_};
        const float xb[6] = {lb, oxb.x, oxb.y, oxb.z, oxb.w, rb_};
        const float rva[4] = {ra.x, ra.y, ra.z, ra.w}, rvb[4] = {rb.x, rb.y, rb.z, rb.w};
        const float sva[4] = {osa.x, osa.y, osa.z, osa.w}, nva[4] = {oxb.x, oxb.y, oxb.z, oxb.w};
        const float svb[4] = {oxa.x, oxa.y, oxa.z, oxa.w}, nvb[4] = {onb.x, onb.y, onb.z, onb.w};
        const float bva[4] = {oba.x, oba.y, oba.z, oba.w}, tva[4] = {ota.x, ota.y, ota.z, ota.w};
        const float bvb[4] = {obb.x, obb.y, obb.z, obb.w}, tvb[4] = {otb.x, otb.y, otb.z, otb.w};
        float eva[4] = {ea.x, ea.y, ea.z, ea.w}, evb[4] = {eb.x, eb.y, eb.z, eb.w};
        if ((kk & 1) == 0) {
          update4<COLOR != 0>(rva, eva, xa, sva, nva, bva, tva, p0, p1, p2, ya0, ya1, ya2, z0, z1, z2, omega, om1);
          update4<COLOR == 0>(rvb, evb, xb, svb, nvb, bvb, tvb, q0, q1, q2, yb0, yb1, yb2, z0, z1, z2, omega, om1);
        } else {
          update4<COLOR == 0>(rva, eva, xa, sva, nva, bva, tva, q0, q1, q2, ya0, ya1, ya2, z0, z1, z2, omega, om1);
          update4<COLOR != 0>(rvb, evb, xb, svb, nvb, bvb, tvb, p0, p1, p2, yb0, yb1, yb2, z0, z1, z2, omega, om1);
        }
        *reinterpret_cast<float4*>(e_own + s0) = make_float4(eva[0], eva[1], eva[2], eva[3]);
        if (rowb) *reinterpret_cast<float4*>(e_own + s0 + Lp) = make_float4(evb[0], evb[1], evb[2], evb[3]);
      }
      oba = oxa;
      oxa = ota;
      obb = oxb;
      oxb = otb;
    }
  }
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// One whole red-black sweep per launch: the red pass and the black pass fused into a
// z-wavefront over planes staged in shared memory.
//
// A block owns FY rows (j) by kFZ planes (k) over the full x extent of the packed
// rows (blockDim.x = 32 x warps, one float4 group per thread; blockDim.y = FY + 2
// row threads, the outer two for halo rows) and marches k upward. For every plane p
// one thread copies the block's rows of the four arrays into a shared-memory stage
// with 1-D bulk asynchronous copies (cp.async.bulk, completion counted on the
// stage's mbarrier): black before the sweep on rows j0-2..j0+FY+1, red before the
// sweep and the red right-hand side on rows j0-1..j0+FY, the black right-hand side
// on rows j0..j0+FY-1. S stages rotate, so the copies of planes up to k+S-2 are in
// flight while plane k is computed, and the threads read only shared memory: the
// load path serves hits, with no cache misses to fill.
//
// At plane k every row thread updates the red cells of its row from the black values
// before the sweep (planes k-1 and k carried in registers, k+1 and the rows j+-1
// read from the stages) and puts the new red row into a three-plane ring; after one
// barrier the inner rows update their black cells of plane k-1 from the new red
// values (rows j+-1 from the ring, planes k-2 and k from registers). Black at the
// block's edges needs new red values one row and one plane beyond the block, so those
// are computed by this block too (the neighbouring blocks compute the same values).
// Every block therefore reads the values before the sweep from one pair of arrays
// (e_red, e_black) and writes the new values to a second pair (n_red, n_black): no
// block overwrites what another still has to read, and the caller swaps the pairs
// after each sweep. Every fluid cell is written by exactly one block; the other
// entries hold 0 in both pairs. Per cell the arithmetic is update4's, in the same
// order, so the results are bit-identical to two k_sor32p passes.
//
// Every mbarrier wait is bounded and decided for the whole block: a wait that gives
// up sets ctl->stage_err (the host fails the solve), stops the issue of copies, and
// the block waits (bounded) for the copies it has issued before it exits.
constexpr int kFZ = 16;
constexpr int kMaxStages = 6;

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

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

// Bounded wait on an mbarrier phase (true when it completed).
__device__ __forceinline__ bool stage_wait(unsigned long long* bar, unsigned parity) {
  for (int it = 0; it < (1 << 22); ++it) {
    unsigned ok;
    asm volatile("{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
                 : "=r"(ok) : "r"(smem_u32(bar)), "r"(parity) : "memory");
    if (ok) return true;
  }
  return false;
}

__device__ __forceinline__ void bulk_copy(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
               :: "r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar)) : "memory");
}

template <int FY, int S>
__global__ void __launch_bounds__(640) k_sor32t(Dims d, Grid1D g, const float* __restrict__ r_red,
                                                 const float* __restrict__ r_black,
                                                 const float* __restrict__ e_red, const float* __restrict__ e_black,
                                                 float* __restrict__ n_red, float* __restrict__ n_black, int Lp,
                                                 float omega, float om1, SolveCtl* ctl) {
  static_assert(S >= 4 && S <= kMaxStages, "a stage is refilled two planes after it is last read");
  extern __shared__ __align__(128) float smf[];   // [S][(4 FY + 8) Lp] stages, then the ring
  __shared__ __align__(8) unsigned long long bar[kMaxStages];
  asm volatile("griddepcontrol.wait;" ::: "memory");
  const int nq = ((d.nx >> 1) + 3) >> 2;
  const int nqp = blockDim.x;
  const int q = threadIdx.x, lane = q & 31;
  const int tr = threadIdx.y;                       // 0 and FY + 1: halo rows
  const bool lead = q == 0 && tr == 0;
  const int j0 = blockIdx.x * FY + 2;               // first row the block owns
  const int j = j0 - 1 + tr;                        // row of this thread
  const int k0 = blockIdx.y * kFZ + 2;              // first plane the block owns
  const int k1 = min(k0 + kFZ, d.nz + 2);           // one past the last
  const int kr0 = k0 - 1;                           // first red plane (a halo plane, or the ghost plane)
  const bool row_cell = j >= 2 && j <= d.ny + 1;    // the row holds cells (not a ghost row)
  const bool inner = tr >= 1 && tr <= FY && row_cell;
  const bool active = q < nq && j <= d.ny + 2;
  const bool load_left = lane == 0, load_right = lane == 31 || q + 1 >= nq;
  const int plane = (d.ny + 2) * Lp;
  const int e = 4 * q + 4;                          // this thread's first entry within a row
  const int stage_floats = (4 * FY + 8) * Lp;
  float4* ring = reinterpret_cast<float4*>(smf + S * stage_floats);   // [3][FY + 2][nqp]
  // rows copied into a stage (clipped to the arrays' rows 1..ny+2; rows outside are never read)
  const int eb_lo = max(1, j0 - 2), eb_hi = min(d.ny + 2, j0 + FY + 1);
  const int er_lo = max(1, j0 - 1), er_hi = min(d.ny + 2, j0 + FY);
  const int rb_lo = j0, rb_hi = min(d.ny + 1, j0 + FY - 1);
  // this thread's entries within a stage: black row j, red and r_red row j, r_black row j
  const int o_eb = (tr + 1) * Lp + e, o_er = (FY + 4 + tr) * Lp + e, o_rr = (2 * FY + 6 + tr) * Lp + e,
            o_rb = (3 * FY + 8 + tr - 1) * Lp + e;
  const unsigned stage_bytes =
      (unsigned)((eb_hi - eb_lo + 1) + 2 * (er_hi - er_lo + 1) + (rb_hi - rb_lo + 1)) * (unsigned)Lp * 4u;
  const int pbase = kr0 - 1, plast = k1 + 1;        // planes the block reads
  if (lead) {
    for (int s = 0; s < S; ++s) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_u32(&bar[s])));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  // Planes pbase..plast pass through the stages in order (plane p in stage (p - pbase)
  // mod S), each once through its stage's mbarrier, so that the n-th use of a stage is
  // the barrier's phase n: a plane outside the arrays (the ghost-side halo planes 0 and
  // nz+3) only arrives, and its stage is never read.
  int istage = 0;   // stage of the next plane to issue (lead thread)
  auto issue = [&](int p) {
    float* st = smf + istage * stage_floats;
    unsigned long long* b = &bar[istage];
    istage = istage + 1 == S ? 0 : istage + 1;
    if (p < 1 || p > d.nz + 2) {
      asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" :: "r"(smem_u32(b)) : "memory");
      return;
    }
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(smem_u32(b)), "r"(stage_bytes)
                 : "memory");
    const long long pl = (long long)(p - 1) * plane;
    bulk_copy(st + (eb_lo - (j0 - 2)) * Lp, e_black + pl + (long long)(eb_lo - 1) * Lp,
              (unsigned)(eb_hi - eb_lo + 1) * Lp * 4u, b);
    bulk_copy(st + (FY + 4 + er_lo - (j0 - 1)) * Lp, e_red + pl + (long long)(er_lo - 1) * Lp,
              (unsigned)(er_hi - er_lo + 1) * Lp * 4u, b);
    bulk_copy(st + (2 * FY + 6 + er_lo - (j0 - 1)) * Lp, r_red + pl + (long long)(er_lo - 1) * Lp,
              (unsigned)(er_hi - er_lo + 1) * Lp * 4u, b);
    bulk_copy(st + (3 * FY + 8 + rb_lo - j0) * Lp, r_black + pl + (long long)(rb_lo - 1) * Lp,
              (unsigned)(rb_hi - rb_lo + 1) * Lp * 4u, b);
  };
  // block-uniform wait for the next plane in order; false when it gave up
  int wstage = 0;
  unsigned wparity = 0;   // bit s: parity of the next phase of stage s
  auto wait_next = [&]() {
    const bool ok = stage_wait(&bar[wstage], (wparity >> wstage) & 1u);
    wparity ^= 1u << wstage;
    wstage = wstage + 1 == S ? 0 : wstage + 1;
    return __syncthreads_and(ok) != 0;
  };
  int issued = pbase - 1, waited = pbase - 1;       // last plane issued / waited for (block-uniform)
  for (int p = pbase; p < pbase + S && p <= plast; ++p) {
    if (lead) issue(p);
    issued = p;
  }
  // x coefficients of this thread's four cells in both row phases
  float4 axc[2][3];
#pragma unroll
  for (int sp = 0; sp < 2; ++sp)
#pragma unroll
    for (int c = 0; c < 3; ++c) axc[sp][c] = q < nq ? g.axp[sp][c][q] : make_float4(0.f, 0.f, 0.f, 0.f);
  float ay0 = 0.f, ay1 = 0.f, ay2 = 0.f;
  if (row_cell) {
    ay0 = g.acy32[0][j - 1];
    ay1 = g.acy32[1][j - 1];
    ay2 = g.acy32[2][j - 1];
  }
  bool ok = true;
  // planes kr0-1 and kr0 before the first red plane
  for (int p = pbase; p <= kr0 && ok; ++p) {
    ok = wait_next();
    waited = p;
  }
  const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
  float4 bm = z4, b0 = z4, rm2 = z4, rm1 = z4;
  if (ok && row_cell && active) {
    if (kr0 - 1 >= 1) bm = *reinterpret_cast<const float4*>(smf + o_eb);                 // stage 0
    if (kr0 >= 1) b0 = *reinterpret_cast<const float4*>(smf + stage_floats + o_eb);     // stage 1
  }
  // stages of planes k-1, k, k+1 and ring slots of planes k-1, k, rotated each plane
  int s_m = 0, s_0 = 1, s_p = 2 % S;
  int ring_m = 2, ring_0 = 0;
  float4* ringp = ring + tr * nqp + q;
  const int ring_plane = (FY + 2) * nqp;
  for (int k = kr0; k <= k1 && ok; ++k) {
    ok = wait_next();   // plane k+1
    if (!ok) break;
    waited = k + 1;
    const float* st_p = smf + s_p * stage_floats;
    const float* st_0 = smf + s_0 * stage_floats;
    // ---- red cells of plane k
    const bool plane_cell = k >= 2 && k <= d.nz + 1;
    const int s0 = (k - 1) * plane + (j - 1) * Lp + e;
    float4 bp = z4;   // black before the sweep at plane k+1
    if (row_cell && active && k + 1 <= d.nz + 2) bp = *reinterpret_cast<const float4*>(st_p + o_eb);
    float4 rn = z4;
    if (plane_cell && row_cell) {   // warp-uniform
      float left = __shfl_up_sync(0xffffffffu, b0.w, 1);
      float right = __shfl_down_sync(0xffffffffu, b0.x, 1);
      if (active) {
        const float* rowb = st_0 + o_eb;
        if (load_left) left = rowb[-1];
        if (load_right) right = rowb[4];
        const float4 rr = *reinterpret_cast<const float4*>(st_0 + o_rr);
        rn = *reinterpret_cast<const float4*>(st_0 + o_er);
        const float4 os = *reinterpret_cast<const float4*>(rowb - Lp);
        const float4 on = *reinterpret_cast<const float4*>(rowb + Lp);
        const float oxa[6] = {left, b0.x, b0.y, b0.z, b0.w, right};
        const float az0 = g.acz32[0][k - 1], az1 = g.acz32[1][k - 1], az2 = g.acz32[2][k - 1];
        if (((j + k) & 1) == 1)   // red is (i+j+k) odd: the row starts with red
          update_group<true>(rr, rn, oxa, os, on, bm, bp, axc[0][0], axc[0][1], axc[0][2], ay0, ay1, ay2, az0, az1,
                             az2, omega, om1);
        else
          update_group<false>(rr, rn, oxa, os, on, bm, bp, axc[1][0], axc[1][1], axc[1][2], ay0, ay1, ay2, az0,
                              az1, az2, omega, om1);
        if (inner && k >= k0 && k < k1) *reinterpret_cast<float4*>(n_red + s0) = rn;
      }
    }
    ringp[ring_0 * ring_plane] = rn;
    __syncthreads();
    // every thread is past plane k-1's red update and plane k-2's black update: the
    // stage of plane k-2 is free for plane k-2+S
    if (k >= kr0 + 1) {
      const int pn = k - 2 + S;
      if (pn <= plast) {
        if (lead) issue(pn);
        issued = pn;
      }
    }
    // ---- black cells of plane k-1, from the new red values
    const int kb = k - 1;
    if (inner && kb >= k0 && kb < k1) {   // warp-uniform
      const float4* rb_row = ring + ring_m * ring_plane + tr * nqp;
      float left = __shfl_up_sync(0xffffffffu, rm1.w, 1);
      float right = __shfl_down_sync(0xffffffffu, rm1.x, 1);
      if (active) {
        if (load_left) left = q > 0 ? rb_row[q - 1].w : 0.f;
        if (load_right) right = q + 1 < nqp ? rb_row[q + 1].x : 0.f;
        const float4 rr = *reinterpret_cast<const float4*>(smf + s_m * stage_floats + o_rb);
        float4 en = bm;   // black before the sweep at plane k-1
        const float4 os = rb_row[q - nqp], on = rb_row[q + nqp];
        const float oxa[6] = {left, rm1.x, rm1.y, rm1.z, rm1.w, right};
        const float az0 = g.acz32[0][kb - 1], az1 = g.acz32[1][kb - 1], az2 = g.acz32[2][kb - 1];
        if (((j + kb) & 1) == 0)   // black is (i+j+k) even: the row starts with black
          update_group<true>(rr, en, oxa, os, on, rm2, rn, axc[0][0], axc[0][1], axc[0][2], ay0, ay1, ay2, az0, az1,
                             az2, omega, om1);
        else
          update_group<false>(rr, en, oxa, os, on, rm2, rn, axc[1][0], axc[1][1], axc[1][2], ay0, ay1, ay2, az0,
                              az1, az2, omega, om1);
        *reinterpret_cast<float4*>(n_black + s0 - plane) = en;
      }
    }
    bm = b0;
    b0 = bp;
    rm2 = rm1;
    rm1 = rn;
    s_m = s_0;
    s_0 = s_p;
    s_p = s_p + 1 == S ? 0 : s_p + 1;
    ring_m = ring_0;
    ring_0 = ring_0 == 2 ? 0 : ring_0 + 1;
  }
  if (!ok) {
    if (lead) atomicExch(&ctl->stage_err, 1);
    // let the copies still in flight land before the block's shared memory is released
    for (int p = waited + 1; p <= issued; ++p) {
      stage_wait(&bar[wstage], (wparity >> wstage) & 1u);
      wparity ^= 1u << wstage;
      wstage = wstage + 1 == S ? 0 : wstage + 1;
    }
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
  // the loads without branches (sweep_kernel 0 beyond L2, and 3) or behind branches (4)
  if (c->prm.sweep_kernel != 4) {
    if (color == 0) cudaLaunchKernelEx(&cfg, k_sor32p<0, true>, d, c->g, r, e, o, c->packed_lp, omega, om1);
    else cudaLaunchKernelEx(&cfg, k_sor32p<1, true>, d, c->g, r, e, o, c->packed_lp, omega, om1);
  } else {
    if (color == 0) cudaLaunchKernelEx(&cfg, k_sor32p<0, false>, d, c->g, r, e, o, c->packed_lp, omega, om1);
    else cudaLaunchKernelEx(&cfg, k_sor32p<1, false>, d, c->g, r, e, o, c->packed_lp, omega, om1);
  }
}

// Where the four packed arrays fit in L2 with room to spare, one colour pass per
// launch of the two-row kernel; beyond 96 MB the one-row kernel with branch-free
// loads, which keeps more DRAM requests in flight (at 384x256x256, 213 MB: 79.7 us
// per sweep against 82.5-85.2 for the two-row kernel; at 256^3, 145 MB, the two are
// within 2 %).
constexpr size_t kTwoRowMaxBytes = (size_t)96 << 20;
static bool two_row_kernel(const ib3d_ctx* c) {
  const Dims& d = c->d;
  const size_t packed = 4 * sizeof(float) * (size_t)c->packed_lp * (size_t)d.NY2 * (size_t)d.NZ2;
  return c->prm.sweep_kernel == 0 && packed <= kTwoRowMaxBytes;
}

// One colour pass of the two-row kernel.
static void launch_pass2(ib3d_ctx* c, int color, float omega, float om1) {
  const Dims& d = c->d;
  const int nq = ((d.nx >> 1) + 3) >> 2;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)((nq + 31) / 32), (unsigned)((d.ny + 2 * kRows2 - 1) / (2 * kRows2)),
                     (unsigned)((d.nz + kPlanes2 - 1) / kPlanes2));
  cfg.blockDim = dim3(32, kRows2);
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
  if (color == 0) cudaLaunchKernelEx(&cfg, k_sor32p2<0>, d, c->g, r, e, o, c->packed_lp, omega, om1);
  else cudaLaunchKernelEx(&cfg, k_sor32p2<1>, d, c->g, r, e, o, c->packed_lp, omega, om1);
}

// One red-black sweep with the colour-packed two-pass kernels.
void launch_sor32_sweep(ib3d_ctx* c, float omega, float om1) {
  if (two_row_kernel(c)) {
    launch_pass2(c, 0, omega, om1);
    launch_pass2(c, 1, omega, om1);
  } else {
    launch_sor32_packed(c, 0, omega, om1);
    launch_sor32_packed(c, 1, omega, om1);
  }
}

// Sweeps per replay of the captured sweep graph: the host issues one graph launch
// per kGraphSweeps sweeps instead of two kernel launches per sweep (a pass takes
// about 8 us), so the sweep loop does not depend on the host's launch rate.
constexpr int kGraphSweeps = 32;

// Captures kGraphSweeps sweeps at (omega, om1) as a CUDA graph on the context's
// stream, unless the cached one was captured with the same tables, relaxation and
// kernel choice. Returns false when capture or instantiation fails (the caller then
// launches the sweeps one by one).
static bool ensure_sweep_graph(ib3d_ctx* c, float omega, float om1) {
  if (c->sweep_exec && c->sweep_w == omega && c->sweep_w1 == om1 && c->sweep_kern == c->prm.sweep_kernel &&
      std::memcmp(&c->sweep_g, &c->g, sizeof(Grid1D)) == 0)
    return true;
  if (c->sweep_exec) {
    cudaGraphExecDestroy(c->sweep_exec);
    c->sweep_exec = nullptr;
  }
  if (cudaStreamBeginCapture(c->st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  for (int q = 0; q < kGraphSweeps; ++q) launch_sor32_sweep(c, omega, om1);
  cudaGraph_t graph = nullptr;
  const cudaError_t e = cudaStreamEndCapture(c->st, &graph);
  bool ok = e == cudaSuccess && graph != nullptr &&
            cudaGraphInstantiate(&c->sweep_exec, graph, 0) == cudaSuccess;
  if (graph) cudaGraphDestroy(graph);
  if (!ok) {
    c->sweep_exec = nullptr;
    cudaGetLastError();
    return false;
  }
  c->sweep_w = omega;
  c->sweep_w1 = om1;
  c->sweep_kern = c->prm.sweep_kernel;
  c->sweep_g = c->g;
  return true;
}

// n red-black sweeps at (omega, om1) with the colour-packed kernels: whole groups of
// kGraphSweeps as replays of the captured graph, the rest launched directly.
void run_sor32_sweeps(ib3d_ctx* c, int n, float omega, float om1) {
  if (n >= kGraphSweeps && !c->sweep_graph_failed) {
    if (ensure_sweep_graph(c, omega, om1)) {
      for (; n >= kGraphSweeps; n -= kGraphSweeps) cudaGraphLaunch(c->sweep_exec, c->st);
    } else {
      c->sweep_graph_failed = true;
    }
  }
  for (; n > 0; --n) launch_sor32_sweep(c, omega, om1);
}

// Rows per block and stages of the staged sweep for a row of nq float4 groups: 16 rows
// with up to five stages where the shared memory holds them, else 8 rows.
struct StagedShape {
  int fy, stages, wx;
  size_t smem;
};
static size_t staged_smem(int fy, int S, int Lp, int wx) {
  return (size_t)S * (4 * fy + 8) * Lp * sizeof(float) + (size_t)3 * (fy + 2) * 32 * wx * sizeof(float4);
}
static bool staged_shape(int nx, StagedShape& out) {
  const int nq = ((nx >> 1) + 3) >> 2, wx = (nq + 31) / 32, Lp = packed_row_length(nx);
  const size_t cap = 227 * 1024 - 256;   // shared memory per block, less the static barriers
  // one block per SM with the deepest staging that fits: tried at 256x192x192, two
  // blocks of 8 rows and 4 stages per SM ran 35.6 us per sweep against 28.5 us for one
  // block of 16 rows and 5 stages
  for (size_t share : {cap})
    for (int fy : {16, 8}) {
      if (32 * wx * (fy + 2) > 640) continue;
      for (int S = 5; S >= 4; --S)
        if (staged_smem(fy, S, Lp, wx) <= share) {
          out = {fy, S, wx, staged_smem(fy, S, Lp, wx)};
          return true;
        }
    }
  return false;
}

// Largest nx the fused sweep takes: its block spans a whole packed row, and four
// stages of it fit in shared memory.
bool fused_sweep_fits(int nx) {
  StagedShape sh;
  return staged_shape(nx, sh);
}

// One fused sweep: reads the sweep's input from ep[], writes its result to epn[] and
// swaps the two pairs, so ep[] holds the current correction afterwards.
void launch_sor32_fused(ib3d_ctx* c, float omega, float om1) {
  const Dims& d = c->d;
  StagedShape sh;
  if (!staged_shape(d.nx, sh)) return;   // checked before the solve starts
  const dim3 grid((unsigned)((d.ny + sh.fy - 1) / sh.fy), (unsigned)((d.nz + kFZ - 1) / kFZ)),
      block((unsigned)(32 * sh.wx), (unsigned)(sh.fy + 2));
  static bool smem_set = false;   // more than the default 48 KB of dynamic shared memory
  if (!smem_set) {
    const int mx = 227 * 1024 - 256;
    cudaFuncSetAttribute(k_sor32t<16, 5>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(k_sor32t<16, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(k_sor32t<8, 5>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(k_sor32t<8, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    smem_set = true;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = sh.smem;
  cfg.stream = c->st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  const float *rr = c->rp[0], *rb = c->rp[1], *er = c->ep[0], *eb = c->ep[1];
  float *nr = c->epn[0], *nb = c->epn[1];
  const int Lp = c->packed_lp;
  if (sh.fy == 16 && sh.stages == 5)
    cudaLaunchKernelEx(&cfg, k_sor32t<16, 5>, d, c->g, rr, rb, er, eb, nr, nb, Lp, omega, om1, c->ctl);
  else if (sh.fy == 16)
    cudaLaunchKernelEx(&cfg, k_sor32t<16, 4>, d, c->g, rr, rb, er, eb, nr, nb, Lp, omega, om1, c->ctl);
  else if (sh.stages == 5)
    cudaLaunchKernelEx(&cfg, k_sor32t<8, 5>, d, c->g, rr, rb, er, eb, nr, nb, Lp, omega, om1, c->ctl);
  else
    cudaLaunchKernelEx(&cfg, k_sor32t<8, 4>, d, c->g, rr, rb, er, eb, nr, nb, Lp, omega, om1, c->ctl);
  std::swap(c->ep[0], c->epn[0]);
  std::swap(c->ep[1], c->epn[1]);
}

void launch_accumulate_packed(ib3d_ctx* c) {
  const long long n = (long long)c->d.nx * c->d.ny * c->d.nz;
  k_accumulate_packed<<<(unsigned)((n + kBlock - 1) / kBlock), kBlock, 0, c->st>>>(c->d, c->pc, c->ep[0], c->ep[1],
                                                                                   c->packed_lp);
}

}  // namespace ib3d
