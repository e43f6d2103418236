// Immersed-boundary geometry, ghost-point forcing and drag/lift.
//
// Reference: computeSurfaceNorm, tagging, cellCount, computeNormDistance
// (subSearch.f90:80-678), pressureForcing1 / velocityForcing1 (subForcing.f90:2-652),
// stressCal1 / stressCal2 (subStressCal1.f90, subStressCal2.f90).
//
// Compiled with -fmad=false (bit-identical FP64 arithmetic to the serial oracle).
//
// Serial semantics of the forcing. velocityForcing1 reads and writes the same
// arrays: each immersed-boundary (IB) cell writes six ghost faces and its probe
// stencils read faces that earlier cells (or earlier blocks of the same cell) may
// have written, and adjacent IB cells write the same face (the later one wins).
// On a CPU the loop order decides the result; the reference's OpenACC loop races.
// Here every ghost value is an "op" with a serial number (6n + block, or n for the
// pressure). At search time each of an op's eight stencil reads is resolved to
// either the pre-forcing field value or the op that last wrote that face before it
// in serial order (a face of field u has at most two writers: the U(i,j,k) block of
// IB cell (i,j,k) and the U(i-1,j,k) block of IB cell (i+1,j,k)); ops are grouped
// into dependency levels; each level runs as one launch writing to a per-op buffer;
// finally the last writer of each face stores its value. The result equals the
// serial loop's exactly, with no race.
#include <algorithm>

#include "ib3d_internal.cuh"

namespace ib3d {

namespace {

inline unsigned nblk(long long n, int b = kBlock) { return (unsigned)((n + b - 1) / b); }

// l in [lo,hi] with A[l] <= pos < A[l+1], or 0. A is strictly increasing, so this
// is the unique match the reference's linear "keep the last match" scans find.
__device__ __forceinline__ int bracket(const double* A, int lo, int hi, double pos) {
  if (!(pos >= A[lo]) || !(pos < A[hi + 1])) return 0;
  int a = lo, b = hi;
  while (a < b) {
    const int m = (a + b + 1) >> 1;
    if (A[m] <= pos) a = m; else b = m - 1;
  }
  return a;
}

// Trilinear probe value and one-sided quadratic derivative estimates, the common
// block of subForcing.f90:175-215 (and its analogues in subStressCal1.f90).
// f = values at (x0|x1, y0|y1, z0|z1) with x fastest: f[q], q = xbit + 2*ybit + 4*zbit.
__device__ __forceinline__ void probe_eval(const double f[8], const double* X, const double* Y, const double* Z,
                                           int ix, int iy, int iz, double px, double py, double pz,
                                           double out[4]) {
  const double f000 = f[0], f100 = f[1], f010 = f[2], f110 = f[3];
  const double f001 = f[4], f101 = f[5], f011 = f[6], f111 = f[7];
  const double tx = px - X[ix], dX = X[ix + 1] - X[ix];
  const double ty = py - Y[iy], dY = Y[iy + 1] - Y[iy];
  const double tz = pz - Z[iz], dZ = Z[iz + 1] - Z[iz];
  const double x1z1 = f000 + (f100 - f000) * tx / dX;
  const double x2z1 = f010 + (f110 - f010) * tx / dX;
  const double x1z2 = f001 + (f101 - f001) * tx / dX;
  const double x2z2 = f011 + (f111 - f011) * tx / dX;
  const double z1 = x1z1 + (x2z1 - x1z1) * ty / dY;
  const double z2 = x1z2 + (x2z2 - x1z2) * ty / dY;
  const double y1 = x1z1 + (x1z2 - x1z1) * tz / dZ;
  const double y2 = x2z1 + (x2z2 - x2z1) * tz / dZ;
  const double z1x1 = f000 + (f001 - f000) * tz / dZ;
  const double z2x1 = f010 + (f011 - f010) * tz / dZ;
  const double z1x2 = f100 + (f101 - f100) * tz / dZ;
  const double z2x2 = f110 + (f111 - f110) * tz / dZ;
  const double x1 = z1x1 + (z2x1 - z1x1) * ty / dY;
  const double x2 = z1x2 + (z2x2 - z1x2) * ty / dY;
  const double pos = x1 + (x2 - x1) * tx / dX;
  double h2 = fabs(X[ix + 1] - px), h1 = fabs(X[ix] - px);
  out[1] = (h1 * h1 * x2 - h2 * h2 * x1 + (h2 * h2 - h1 * h1) * pos) / (h1 * h2 * (h1 + h2) + 1e-16);
  h2 = fabs(Y[iy + 1] - py); h1 = fabs(Y[iy] - py);
  out[2] = (h1 * h1 * y2 - h2 * h2 * y1 + (h2 * h2 - h1 * h1) * pos) / (h1 * h2 * (h1 + h2) + 1e-16);
  h2 = fabs(Z[iz + 1] - pz); h1 = fabs(Z[iz] - pz);
  out[3] = (h1 * h1 * z2 - h2 * h2 * z1 + (h2 * h2 - h1 * h1) * pos) / (h1 * h2 * (h1 + h2) + 1e-16);
  out[0] = pos;
}

// Velocity ghost-point blocks in subForcing.f90's order (U(i,j,k) :143-224,
// U(i-1,j,k) :227-308, V(i,j,k) :311-393, V(i,j-1,k) :396-478, W(i,j,k) :481-562,
// W(i,j,k-1) :565-646): field, normal-distance slot, node offset, scan extension,
// clamp (+1: idx == n+2 -> n+1 ; -1: idx == 1 -> 2), write-target offset.
struct GhostBlock {
  int field, nd, node[3], scan[3], clamp_axis, clamp_dir, tgt[3];
};
__constant__ GhostBlock c_ghost[6] = {
    {0, 2, {1, 0, 0}, {1, 0, 0}, 0, +1, {0, 0, 0}},
    {0, 1, {0, 0, 0}, {0, 0, 0}, 0, -1, {-1, 0, 0}},
    {1, 4, {0, 1, 0}, {0, 1, 0}, 1, +1, {0, 0, 0}},
    {1, 3, {0, 0, 0}, {0, 0, 0}, 1, -1, {0, -1, 0}},
    {2, 6, {0, 0, 1}, {0, 0, 1}, 2, +1, {0, 0, 0}},
    {2, 5, {0, 0, 0}, {0, 0, 0}, 2, -1, {0, 0, -1}},
};

struct StagCoords {
  const double *X, *Y, *Z;
};
__device__ __forceinline__ StagCoords stag(const Grid1D& g, int field) {
  if (field == 0) return {g.xu, g.yu, g.zu};
  if (field == 1) return {g.xv, g.yv, g.zv};
  if (field == 2) return {g.xw, g.yw, g.zw};
  return {g.xp, g.yp, g.zp};
}

// Geometry of velocity op q = 6n + blk: probe point and pt1, normal distance, nel.
struct OpGeom {
  int i, j, k, nel;
  double sd, pt1, pos[3];
};
__device__ __forceinline__ OpGeom vel_geom(const Grid1D& g, const int* iblist, const int* nelp, const double* nd,
                                           const double* surf, int nib, int nel_tot, int n, int blk) {
  const GhostBlock& gb = c_ghost[blk];
  OpGeom o;
  o.i = iblist[n]; o.j = iblist[nib + n]; o.k = iblist[2 * nib + n];
  o.nel = nelp[n];
  o.sd = nd[gb.nd * nib + n];
  const double diag = sqrt((g.dx[o.i] * g.dx[o.i] + g.dy[o.j] * g.dy[o.j]) + g.dz[o.k] * g.dz[o.k]);
  o.pt1 = 1.5 * diag + (fabs(o.sd) - o.sd) * 0.5;                       // :148
  const StagCoords sc = stag(g, gb.field);
  const int e = o.nel - 1;
  o.pos[0] = sc.X[o.i + gb.node[0]] + o.pt1 * surf[3 * nel_tot + e];    // :151-153
  o.pos[1] = sc.Y[o.j + gb.node[1]] + o.pt1 * surf[4 * nel_tot + e];
  o.pos[2] = sc.Z[o.k + gb.node[2]] + o.pt1 * surf[5 * nel_tot + e];
  return o;
}

}  // namespace

// ------------------------------------------------------------- surface and search

// computeSurfaceNorm (subSearch.f90:95-125).
__global__ void k_surface_norm(const double* __restrict__ nodes, const int* __restrict__ tri, int nn, int ne,
                               double inor, double* __restrict__ surf) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  const int a = tri[e] - 1, b = tri[ne + e] - 1, c = tri[2 * ne + e] - 1;
  const double p1x = nodes[a], p1y = nodes[nn + a], p1z = nodes[2 * nn + a];
  const double p2x = nodes[b], p2y = nodes[nn + b], p2z = nodes[2 * nn + b];
  const double p3x = nodes[c], p3y = nodes[nn + c], p3z = nodes[2 * nn + c];
  surf[e] = ((p2x + p1x) + p3x) / 3.0;
  surf[ne + e] = ((p2y + p1y) + p3y) / 3.0;
  surf[2 * ne + e] = ((p2z + p1z) + p3z) / 3.0;
  const double ca = (p2y - p1y) * (p3z - p1z) - (p3y - p1y) * (p2z - p1z);
  const double cb = (p2z - p1z) * (p3x - p1x) - (p3z - p1z) * (p2x - p1x);
  const double cg = (p2x - p1x) * (p3y - p1y) - (p3x - p1x) * (p2y - p1y);
  surf[6 * ne + e] = ca; surf[7 * ne + e] = cb; surf[8 * ne + e] = cg;
  const double len = sqrt((ca * ca + cb * cb) + cg * cg);
  surf[3 * ne + e] = (ca / len) * inor;
  surf[4 * ne + e] = (cb / len) * inor;
  surf[5 * ne + e] = (cg / len) * inor;
}

__device__ __forceinline__ double corner_dot(const double* surf, int ne, int e, double x, double y, double z) {
  return ((x - surf[e]) * surf[3 * ne + e] + (y - surf[ne + e]) * surf[4 * ne + e]) +
         (z - surf[2 * ne + e]) * surf[5 * ne + e];
}

// tagging (subSearch.f90:166-249): nearest centroid of each box cell's centre, then
// the signs of the eight corner distances to that element's plane. The reference
// compares dsqrt((dy)^2+(dx)^2+(dz)^2) with strict '<'. Since sqrt is monotone, an
// element whose squared distance is not below the current best's squared distance
// cannot have a strictly smaller rounded root, so the root is only taken for
// candidates that improve the squared distance: the same argmin, bit for bit.
// Centroids are staged through shared memory in tiles. The cells tagged are the
// box's (list == nullptr), or the nlist cells of a list inside the box (the
// neighbourhoods of selectiveRetagging); minel is indexed by the cell's position in
// the box either way.
constexpr int kTagTile = 512;
__global__ void __launch_bounds__(kBlock) k_tagging(Dims d, Grid1D g, const double* __restrict__ surf, int ne,
                                                    int bi0, int bj0, int bk0, int bni, int bnj, int bnk,
                                                    const int* __restrict__ list, int nlist,
                                                    unsigned char* __restrict__ cell, int* __restrict__ minel) {
  __shared__ double sx[kTagTile], sy[kTagTile], sz[kTagTile];
  const unsigned tid = blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned ncell = list ? (unsigned)nlist : (unsigned)bni * (unsigned)bnj * (unsigned)bnk;
  const bool active = tid < ncell;
  int i = 0, j = 0, k = 0;
  double n1x = 0, n1y = 0, n1z = 0;
  if (active) {
    if (list) {
      i = list[tid];
      j = list[nlist + tid];
      k = list[2 * nlist + tid];
    } else {
      i = bi0 + (int)(tid % (unsigned)bni);
      const unsigned t = tid / (unsigned)bni;
      j = bj0 + (int)(t % (unsigned)bnj);
      k = bk0 + (int)(t / (unsigned)bnj);
    }
    n1x = g.xp[i]; n1y = g.yp[j]; n1z = g.zp[k];
  }
  double best = 1e14, best2 = 1e300;
  int nel = 0;
  for (int base = 0; base < ne; base += kTagTile) {
    const int cnt = min(kTagTile, ne - base);
    __syncthreads();
    for (int q = threadIdx.x; q < cnt; q += blockDim.x) {
      sx[q] = surf[base + q]; sy[q] = surf[ne + base + q]; sz[q] = surf[2 * ne + base + q];
    }
    __syncthreads();
    if (active) {
      for (int q = 0; q < cnt; ++q) {
        const double ay = n1y - sy[q], ax = n1x - sx[q], az = n1z - sz[q];
        const double d2 = (ay * ay + ax * ax) + az * az;
        if (d2 < best2) {
          const double dis = sqrt(d2);
          if (dis < best) { best = dis; best2 = d2; nel = base + q + 1; }
        }
      }
    }
  }
  if (!active) return;
  const double n2x = g.x1[i], n3x = g.x1[i + 1], n2y = g.y1[j], n3y = g.y1[j + 1];
  const double n2z = g.z1[k], n3z = g.z1[k + 1];
  const int e = nel - 1;
  const double thr = -1e-16;
  double dd[8];
  dd[0] = corner_dot(surf, ne, e, n2x, n2y, n2z);
  dd[1] = corner_dot(surf, ne, e, n2x, n3y, n2z);
  dd[2] = corner_dot(surf, ne, e, n3x, n2y, n2z);
  dd[3] = corner_dot(surf, ne, e, n3x, n3y, n2z);
  dd[4] = corner_dot(surf, ne, e, n2x, n2y, n3z);
  dd[5] = corner_dot(surf, ne, e, n2x, n3y, n3z);
  dd[6] = corner_dot(surf, ne, e, n3x, n2y, n3z);
  dd[7] = corner_dot(surf, ne, e, n3x, n3y, n3z);
  bool all_in = true, all_out = true;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    if (!(dd[q] <= thr)) all_in = false;
    if (!(dd[q] > thr)) all_out = false;
  }
  cell[d.at(i, j, k)] = all_in ? 1 : (all_out ? 0 : 2);
  minel[(i - bi0) + bni * ((j - bj0) + bnj * (k - bk0))] = nel;
}

// Bounding box of the IB list: {min i, max i, min j, max j, min k, max k}, out[] set
// to {INT_MAX, INT_MIN, ...} before the launch.
__global__ void k_ib_bounds(const int* __restrict__ iblist, int nib, int* __restrict__ out) {
  int lo[3] = {0x7fffffff, 0x7fffffff, 0x7fffffff}, hi[3] = {-0x7fffffff, -0x7fffffff, -0x7fffffff};
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < nib; n += gridDim.x * blockDim.x)
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const int v = iblist[a * nib + n];
      lo[a] = min(lo[a], v);
      hi[a] = max(hi[a], v);
    }
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    for (int o = 16; o > 0; o >>= 1) {
      lo[a] = min(lo[a], __shfl_down_sync(0xffffffffu, lo[a], o));
      hi[a] = max(hi[a], __shfl_down_sync(0xffffffffu, hi[a], o));
    }
    if ((threadIdx.x & 31) == 0) {
      atomicMin(&out[2 * a], lo[a]);
      atomicMax(&out[2 * a + 1], hi[a]);
    }
  }
}

// selectiveRetagging's neighbourhoods (subSearch.f90:355-358): cells i1-2..i1+3,
// j1-2..j1+3, k1-2..k1+3 of every IB cell (i1,j1,k1), clipped to the box (the
// neighbourhoods' bounding box clipped to the interior), marked in a box-shaped mask.
// Overlapping neighbourhoods write the same value.
__global__ void k_mark_neighbourhoods(const int* __restrict__ iblist, int nib, int bi0, int bj0, int bk0, int bni,
                                      int bnj, int bnk, unsigned char* __restrict__ mask) {
  const unsigned tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= (unsigned)nib * 216u) return;
  const int n = (int)(tid / 216u), o = (int)(tid % 216u);
  const int i = iblist[n] - 2 + o % 6, j = iblist[nib + n] - 2 + (o / 6) % 6, k = iblist[2 * nib + n] - 2 + o / 36;
  const int li = i - bi0, lj = j - bj0, lk = k - bk0;
  if (li >= 0 && li < bni && lj >= 0 && lj < bnj && lk >= 0 && lk < bnk) mask[li + bni * (lj + bnj * lk)] = 1;
}

// Compaction of the marked cells of a box-shaped mask into a list (i block, j block,
// k block); same three passes as the IB compaction below.
__global__ void k_mask_blockcount(const unsigned char* __restrict__ mask, unsigned nbox, long long* bcount) {
  __shared__ int s;
  if (threadIdx.x == 0) s = 0;
  __syncthreads();
  const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
  const bool f = t < nbox && mask[t];
  const unsigned bal = __ballot_sync(0xffffffffu, f);
  if ((threadIdx.x & 31) == 0 && bal) atomicAdd(&s, __popc(bal));
  __syncthreads();
  if (threadIdx.x == 0) bcount[blockIdx.x] = s;
}
__global__ void k_mask_scatter(const unsigned char* __restrict__ mask, unsigned nbox, int bi0, int bj0, int bk0,
                               int bni, int bnj, const long long* __restrict__ boff, int nlist,
                               int* __restrict__ list) {
  __shared__ int wsum[kBlock / 32];
  const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
  const bool f = t < nbox && mask[t];
  const unsigned bal = __ballot_sync(0xffffffffu, f);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) wsum[wid] = __popc(bal);
  __syncthreads();
  int before = 0;
  for (int q = 0; q < wid; ++q) before += wsum[q];
  before += __popc(bal & ((1u << lane) - 1u));
  if (f) {
    const long long n = boff[blockIdx.x] + before;
    if (n < nlist) {
      list[n] = bi0 + (int)(t % (unsigned)bni);
      const unsigned r = t / (unsigned)bni;
      list[nlist + n] = bj0 + (int)(r % (unsigned)bnj);
      list[2 * nlist + n] = bk0 + (int)(r / (unsigned)bnj);
    }
  }
}

// Cell counts over the interior (subSearch.f90:259-270) and the red/black split of
// the fluid cells (subSearch.f90:557-567): {fluid, solid, ib, red, black}.
__global__ void k_count(Dims d, const unsigned char* __restrict__ cell, unsigned long long* counts) {
  __shared__ unsigned int sc[5];
  if (threadIdx.x < 5) sc[threadIdx.x] = 0;
  __syncthreads();
  const unsigned tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid < (unsigned)d.nx * (unsigned)d.ny * (unsigned)d.nz) {
    const int i = (int)(tid % (unsigned)d.nx) + 2;
    const unsigned t = tid / (unsigned)d.nx;
    const int j = (int)(t % (unsigned)d.ny) + 2, k = (int)(t / (unsigned)d.ny) + 2;
    const unsigned char c = cell[d.at(i, j, k)];
    if (c == 0) {
      atomicAdd(&sc[0], 1u);
      atomicAdd(&sc[((i + j + k) & 1) ? 3 : 4], 1u);
    } else if (c == 1) {
      atomicAdd(&sc[1], 1u);
    } else if (c == 2) {
      atomicAdd(&sc[2], 1u);
    }
  }
  __syncthreads();
  if (threadIdx.x < 5 && sc[threadIdx.x]) atomicAdd(&counts[threadIdx.x], (unsigned long long)sc[threadIdx.x]);
}

// Lexicographic compaction of the IB cells (cellCount, subSearch.f90:532-553): the
// box is scanned with i fastest, then j, then k, which is the reference's loop
// order. Pass 1 counts per block, pass 2 scans the block counts, pass 3 writes.
__device__ __forceinline__ bool box_is_ib(const Dims& d, const unsigned char* cell, unsigned tid, int bi0, int bj0,
                                          int bk0, int bni, int bnj, unsigned nbox, int& i, int& j, int& k) {
  if (tid >= nbox) return false;
  i = bi0 + (int)(tid % (unsigned)bni);
  const unsigned t = tid / (unsigned)bni;
  j = bj0 + (int)(t % (unsigned)bnj);
  k = bk0 + (int)(t / (unsigned)bnj);
  if (i < 2 || i > d.nx + 1 || j < 2 || j > d.ny + 1 || k < 2 || k > d.nz + 1) return false;
  return cell[d.at(i, j, k)] == 2;
}
__global__ void k_ib_blockcount(Dims d, const unsigned char* __restrict__ cell, int bi0, int bj0, int bk0, int bni,
                                int bnj, unsigned nbox, long long* bcount) {
  __shared__ int s;
  if (threadIdx.x == 0) s = 0;
  __syncthreads();
  int i, j, k;
  const bool f = box_is_ib(d, cell, blockIdx.x * blockDim.x + threadIdx.x, bi0, bj0, bk0, bni, bnj, nbox, i, j, k);
  const unsigned bal = __ballot_sync(0xffffffffu, f);
  if ((threadIdx.x & 31) == 0 && bal) atomicAdd(&s, __popc(bal));
  __syncthreads();
  if (threadIdx.x == 0) bcount[blockIdx.x] = s;
}
__global__ void k_exclusive_scan(long long* a, int n, long long* total) {
  // single block; a sequential carry over 1024-wide chunks
  __shared__ long long buf[1024];
  __shared__ long long carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < n; base += 1024) {
    const int q = base + threadIdx.x;
    const long long x = q < n ? a[q] : 0;
    buf[threadIdx.x] = x;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
      const long long y = threadIdx.x >= off ? buf[threadIdx.x - off] : 0;
      __syncthreads();
      buf[threadIdx.x] += y;
      __syncthreads();
    }
    if (q < n) a[q] = carry + buf[threadIdx.x] - x;
    __syncthreads();
    if (threadIdx.x == 1023) carry += buf[1023];
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = carry;
}
__global__ void k_ib_scatter(Dims d, const unsigned char* __restrict__ cell, int bi0, int bj0, int bk0, int bni,
                             int bnj, unsigned nbox, const long long* __restrict__ boff, int nib,
                             int* __restrict__ iblist) {
  __shared__ int wsum[kBlock / 32];
  int i = 0, j = 0, k = 0;
  const bool f = box_is_ib(d, cell, blockIdx.x * blockDim.x + threadIdx.x, bi0, bj0, bk0, bni, bnj, nbox, i, j, k);
  const unsigned bal = __ballot_sync(0xffffffffu, f);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) wsum[wid] = __popc(bal);
  __syncthreads();
  int before = 0;
  for (int q = 0; q < wid; ++q) before += wsum[q];
  before += __popc(bal & ((1u << lane) - 1u));
  if (f) {
    const long long n = boff[blockIdx.x] + before;
    if (n < nib) { iblist[n] = i; iblist[nib + n] = j; iblist[2 * nib + n] = k; }
  }
}

// computeNormDistance (subSearch.f90:621-672) plus the IB index map.
__global__ void k_normdist(Dims d, Grid1D g, const double* __restrict__ surf, int ne, const int* __restrict__ iblist,
                           int nib, const int* __restrict__ minel, int bi0, int bj0, int bk0, int bni, int bnj,
                           int* __restrict__ nelp, double* __restrict__ nd, int* __restrict__ ibmap) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nib) return;
  const int i = iblist[n], j = iblist[nib + n], k = iblist[2 * nib + n];
  const double n1x = g.xp[i], n2x = g.x1[i], n3x = g.x1[i + 1];
  const double n1y = g.yp[j], n2y = g.y1[j], n3y = g.y1[j + 1];
  const double n1z = g.zp[k], n2z = g.z1[k], n3z = g.z1[k + 1];
  const int m = minel[(i - bi0) + bni * ((j - bj0) + bnj * (k - bk0))];
  nelp[n] = m;
  const int e = m - 1;
  nd[0 * nib + n] = corner_dot(surf, ne, e, n1x, n1y, n1z);
  nd[1 * nib + n] = corner_dot(surf, ne, e, n2x, n1y, n1z);
  nd[2 * nib + n] = corner_dot(surf, ne, e, n3x, n1y, n1z);
  nd[3 * nib + n] = corner_dot(surf, ne, e, n1x, n2y, n1z);
  nd[4 * nib + n] = corner_dot(surf, ne, e, n1x, n3y, n1z);
  nd[5 * nib + n] = corner_dot(surf, ne, e, n1x, n1y, n2z);
  nd[6 * nib + n] = corner_dot(surf, ne, e, n1x, n1y, n3z);
  ibmap[d.at(i, j, k)] = n;
}

// --------------------------------------------------------------- forcing schedule

// Serial number of the op that writes face (a,b,c) of `field` through IB cell
// (ci,cj,ck) with block blk, or -1 when that cell is not an IB cell.
__device__ __forceinline__ long long writer(const Dims& d, const int* ibmap, int ci, int cj, int ck, int blk) {
  if (ci < 2 || ci > d.nx + 1 || cj < 2 || cj > d.ny + 1 || ck < 2 || ck > d.nz + 1) return -1;
  const int n = ibmap[d.at(ci, cj, ck)];
  return n < 0 ? -1 : 6ll * n + blk;
}
// The two possible writers of face (a,b,c) of a velocity field: the "own" block of
// IB cell (a,b,c) and the "minus" block of the next IB cell along the field's axis.
__device__ __forceinline__ void face_writers(const Dims& d, const int* ibmap, int field, int a, int b, int c,
                                             long long w[2]) {
  w[0] = writer(d, ibmap, a, b, c, 2 * field);
  w[1] = writer(d, ibmap, a + (field == 0), b + (field == 1), c + (field == 2), 2 * field + 1);
}

// Builds the velocity ops: brackets, clamps, the eight read indices with their
// sources, the target and whether the op is its target's last writer.
__global__ void k_sched_vel(Dims d, Grid1D g, const int* __restrict__ iblist, const int* __restrict__ nelp,
                            const double* __restrict__ nd, const double* __restrict__ surf, int nib, int ne,
                            const int* __restrict__ ibmap, int* __restrict__ brk, int* __restrict__ rd_idx,
                            int* __restrict__ rd_src, int* __restrict__ tgt, unsigned char* __restrict__ fin,
                            int* err) {
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= 6ll * nib) return;
  const int n = (int)(q / 6), blk = (int)(q % 6);
  const GhostBlock& gb = c_ghost[blk];
  const OpGeom o = vel_geom(g, iblist, nelp, nd, surf, nib, ne, n, blk);
  const StagCoords sc = stag(g, gb.field);
  const int nn[3] = {d.nx, d.ny, d.nz};
  const double* A[3] = {sc.X, sc.Y, sc.Z};
  int br[3];
  for (int a = 0; a < 3; ++a) {
    br[a] = bracket(A[a], 1, nn[a] + 1 + gb.scan[a], o.pos[a]);
    if (br[a] == 0) { atomicExch(err, 1); br[a] = 2; }
  }
  const int ca = gb.clamp_axis;
  if (gb.clamp_dir > 0) { if (br[ca] == nn[ca] + 2) br[ca] = nn[ca] + 1; }    // e.g. :171
  else { if (br[ca] == 1) br[ca] = 2; }                                       // e.g. :252
  // A bracket in the first ghost layer would address field index 0 (the reference
  // would read outside its array): report the probe as off the grid and use a safe cell.
  if (br[gb.field] < 2) { atomicExch(err, 1); br[gb.field] = 2; }
  brk[3 * q] = br[0]; brk[3 * q + 1] = br[1]; brk[3 * q + 2] = br[2];
  const int a0 = br[0] - (gb.field == 0), b0 = br[1] - (gb.field == 1), c0 = br[2] - (gb.field == 2);
  for (int r = 0; r < 8; ++r) {
    const int a = a0 + (r & 1), b = b0 + ((r >> 1) & 1), c = c0 + (r >> 2);
    rd_idx[8 * q + r] = (int)d.at(a, b, c);
    long long w[2];
    face_writers(d, ibmap, gb.field, a, b, c, w);
    long long src = -1;
    for (int s = 0; s < 2; ++s)
      if (w[s] >= 0 && w[s] < q && w[s] > src) src = w[s];
    rd_src[8 * q + r] = (int)src;
  }
  const int ta = o.i + gb.tgt[0], tb = o.j + gb.tgt[1], tc = o.k + gb.tgt[2];
  tgt[q] = (int)d.at(ta, tb, tc);
  long long w[2];
  face_writers(d, ibmap, gb.field, ta, tb, tc, w);
  fin[q] = (w[0] > q || w[1] > q) ? 0 : 1;
}

// Pressure ops: one per IB cell (subForcing.f90:18-98); p(a,b,c) has one writer,
// the IB cell (a,b,c) itself.
__global__ void k_sched_p(Dims d, Grid1D g, const int* __restrict__ iblist, const int* __restrict__ nelp,
                          const double* __restrict__ nd, const double* __restrict__ surf, int nib, int ne,
                          const int* __restrict__ ibmap, int* __restrict__ brk, int* __restrict__ rd_idx,
                          int* __restrict__ rd_src, int* __restrict__ tgt, unsigned char* __restrict__ fin,
                          int* err) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= nib) return;
  const int i = iblist[n], j = iblist[nib + n], k = iblist[2 * nib + n];
  const int e = nelp[n] - 1;
  const double sd = nd[n];
  const double pt1 = 1.5 * sqrt((g.dx[i] * g.dx[i] + g.dy[j] * g.dy[j]) + g.dz[k] * g.dz[k]) + (fabs(sd) - sd) * 0.5;
  const double pos[3] = {g.xp[i] + pt1 * surf[3 * ne + e], g.yp[j] + pt1 * surf[4 * ne + e],
                         g.zp[k] + pt1 * surf[5 * ne + e]};
  const double* A[3] = {g.xp, g.yp, g.zp};
  const int nn[3] = {d.nx, d.ny, d.nz};
  int br[3];
  for (int a = 0; a < 3; ++a) {
    br[a] = bracket(A[a], 1, nn[a] + 1, pos[a]);
    if (br[a] == 0) { atomicExch(err, 1); br[a] = 2; }
  }
  brk[3 * n] = br[0]; brk[3 * n + 1] = br[1]; brk[3 * n + 2] = br[2];
  for (int r = 0; r < 8; ++r) {
    const int a = br[0] + (r & 1), b = br[1] + ((r >> 1) & 1), c = br[2] + (r >> 2);
    const long long L = d.at(a, b, c);
    rd_idx[8 * n + r] = (int)L;
    int src = -1;
    if (a >= 2 && a <= d.nx + 1 && b >= 2 && b <= d.ny + 1 && c >= 2 && c <= d.nz + 1) {
      const int m = ibmap[L];
      if (m >= 0 && m < n) src = m;
    }
    rd_src[8 * n + r] = src;
  }
  tgt[n] = (int)d.at(i, j, k);
  fin[n] = 1;
}

// ------------------------------------------------------------ forcing execution

// One dependency level of velocityForcing1 (subForcing.f90:143-646 per op).
__global__ void k_force_vel(Grid1D g, const int* __restrict__ order, int off, int cnt,
                            const int* __restrict__ iblist, const int* __restrict__ nelp,
                            const double* __restrict__ nd, const double* __restrict__ surf, int nib, int ne,
                            const int* __restrict__ brk, const int* __restrict__ rd_idx,
                            const int* __restrict__ rd_src, const double* __restrict__ ut,
                            const double* __restrict__ vt, const double* __restrict__ wt, Motion mo,
                            double* out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= cnt) return;
  const int q = order[off + t];
  const int n = q / 6, blk = q % 6;
  const GhostBlock& gb = c_ghost[blk];
  const OpGeom o = vel_geom(g, iblist, nelp, nd, surf, nib, ne, n, blk);
  const StagCoords sc = stag(g, gb.field);
  const double* F = gb.field == 0 ? ut : gb.field == 1 ? vt : wt;
  double f[8];
#pragma unroll
  for (int r = 0; r < 8; ++r) {
    const int s = rd_src[8 * q + r];
    f[r] = s >= 0 ? out[s] : F[rd_idx[8 * q + r]];
  }
  double pe[4];
  probe_eval(f, sc.X, sc.Y, sc.Z, brk[3 * q], brk[3 * q + 1], brk[3 * q + 2], o.pos[0], o.pos[1], o.pos[2], pe);
  const int e = o.nel - 1;
  const double dndn = pe[1] * surf[3 * ne + e] + pe[2] * surf[4 * ne + e] + pe[3] * surf[5 * ne + e];
  const double n1 = o.pt1 + o.sd;
  const double surfv = mo.moving ? mo.vel[gb.field] : 0.0;           // usurf = u_curr (:144) or 0 (:145)
  const double cval = surfv;
  const double bval = 2.0 / n1 * (pe[0] - surfv) - dndn;              // :222
  const double aval = dndn / n1 - (pe[0] - surfv) / (n1 * n1);        // :223
  out[q] = aval * (o.sd * o.sd) + bval * o.sd + cval;                 // :224
}

// One dependency level of pressureForcing1 (subForcing.f90:18-98); dpdn = 0 for a
// fixed body (:11), the body acceleration along the normal for a moving one (:20).
__global__ void k_force_p(Grid1D g, const int* __restrict__ order, int off, int cnt, const int* __restrict__ iblist,
                          const int* __restrict__ nelp, const double* __restrict__ nd,
                          const double* __restrict__ surf, int nib, int ne, const int* __restrict__ brk,
                          const int* __restrict__ rd_idx, const int* __restrict__ rd_src,
                          const double* __restrict__ p, Motion mo, double* out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= cnt) return;
  const int n = order[off + t];
  const int i = iblist[n], j = iblist[nib + n], k = iblist[2 * nib + n];
  const int e = nelp[n] - 1;
  const double sd = nd[n];
  const double pt1 = 1.5 * sqrt((g.dx[i] * g.dx[i] + g.dy[j] * g.dy[j]) + g.dz[k] * g.dz[k]) + (fabs(sd) - sd) * 0.5;
  const double px = g.xp[i] + pt1 * surf[3 * ne + e];
  const double py = g.yp[j] + pt1 * surf[4 * ne + e];
  const double pz = g.zp[k] + pt1 * surf[5 * ne + e];
  double f[8];
#pragma unroll
  for (int r = 0; r < 8; ++r) {
    const int s = rd_src[8 * n + r];
    f[r] = s >= 0 ? out[s] : p[rd_idx[8 * n + r]];
  }
  double pe[4];
  probe_eval(f, g.xp, g.yp, g.zp, brk[3 * n], brk[3 * n + 1], brk[3 * n + 2], px, py, pz, pe);
  const double dpdn = mo.moving ? (mo.acc[0] * surf[3 * ne + e] + mo.acc[1] * surf[4 * ne + e]) +
                                      mo.acc[2] * surf[5 * ne + e]
                                : 0.0;
  const double dpdn_e = pe[1] * surf[3 * ne + e] + pe[2] * surf[4 * ne + e] + pe[3] * surf[5 * ne + e];
  const double n1 = pt1 + sd;
  const double bval = dpdn;
  const double aval = (dpdn_e - dpdn) / (2.0 * n1);                  // :95
  const double cval = pe[0] - (dpdn_e + dpdn) * n1 * 0.5;            // :96
  out[n] = aval * (sd * sd) + bval * sd + cval;                      // :98
}

// Stores each face's last-writer value (after every level has run).
__global__ void k_force_scatter(const int* __restrict__ final_ops, int nfinal, const int* __restrict__ tgt,
                                const double* __restrict__ out, int vel, double* f0, double* f1, double* f2) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nfinal) return;
  const int q = final_ops[t];
  double* F = f0;
  if (vel) {
    const int field = (q % 6) >> 1;
    F = field == 0 ? f0 : field == 1 ? f1 : f2;
  }
  F[tgt[q]] = out[q];
}

// ------------------------------------------------------------------- drag / lift

// Per-element terms of stressCal1/2 (subStressCal1.f90:85-434): viscous traction and
// pressure force from the probe at one cell diagonal along the normal. Probe cells
// are found on the first call and cached (stressCal2 reuses them, :81-83 etc.).
__global__ void k_stress_elem(Dims d, Grid1D g, const double* __restrict__ surf, int ne, int first,
                              int* __restrict__ scache, const double* __restrict__ ut,
                              const double* __restrict__ vt, const double* __restrict__ wt,
                              const double* __restrict__ p, double inv_re, double* __restrict__ contrib, int* err) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  const int nn[3] = {d.nx, d.ny, d.nz};
  const double xs = surf[e], ys = surf[ne + e], zs = surf[2 * ne + e];
  const double ca = surf[3 * ne + e], cb = surf[4 * ne + e], cg = surf[5 * ne + e];
  if (first) {
    const double cpos[3] = {xs, ys, zs};
    const double* A1[3] = {g.x1, g.y1, g.z1};
    for (int a = 0; a < 3; ++a) {
      int b = bracket(A1[a], 2, nn[a] + 1, cpos[a]);                   // :89-105
      if (!b) { atomicExch(err, 1); b = 2; }
      scache[15 * e + a] = b;
    }
  }
  const int ic = scache[15 * e], jc = scache[15 * e + 1], kc = scache[15 * e + 2];
  const double dX = g.x1[ic + 1] - g.x1[ic], dY = g.y1[jc + 1] - g.y1[jc], dZ = g.z1[kc + 1] - g.z1[kc];
  const double diagdis = sqrt((dX * dX + dY * dY) + dZ * dZ);           // :119
  const double px = xs + diagdis * ca, py = ys + diagdis * cb, pz = zs + diagdis * cg;
  const double ppos[3] = {px, py, pz};
  double dnds[3];
  for (int c = 0; c < 4; ++c) {
    const StagCoords sc = stag(g, c);
    const double* A[3] = {sc.X, sc.Y, sc.Z};
    if (first) {
      for (int a = 0; a < 3; ++a) {
        int b = bracket(A[a], 2, nn[a] + 1, ppos[a]);                  // e.g. :135-145
        if (!b) { atomicExch(err, 1); b = 2; }
        scache[15 * e + 3 + 3 * c + a] = b;
      }
    }
    const int ix = scache[15 * e + 3 + 3 * c], iy = scache[15 * e + 4 + 3 * c], iz = scache[15 * e + 5 + 3 * c];
    const double* F = c == 0 ? ut : c == 1 ? vt : c == 2 ? wt : p;
    const int a0 = ix - (c == 0), b0 = iy - (c == 1), c0 = iz - (c == 2);
    double f[8];
#pragma unroll
    for (int r = 0; r < 8; ++r) f[r] = F[d.at(a0 + (r & 1), b0 + ((r >> 1) & 1), c0 + (r >> 2))];
    double pe[4];
    probe_eval(f, sc.X, sc.Y, sc.Z, ix, iy, iz, px, py, pz, pe);
    const double dn_e = pe[1] * ca + pe[2] * cb + pe[3] * cg;
    if (c < 3) {
      dnds[c] = (2.0 / diagdis) * (pe[0] - 0.0) - dn_e;                // :195, :260, :324
    } else {
      const double a3 = surf[6 * ne + e], b3 = surf[7 * ne + e], g3 = surf[8 * ne + e];
      const double alen = sqrt((a3 * a3 + b3 * b3) + g3 * g3);         // :327-331
      const double area = alen / 2.0;
      const double dot = dnds[0] * ca + dnds[1] * cb + dnds[2] * cg;
      const double stx1 = dnds[0] - dot * ca;                         // :335-337
      const double sty1 = dnds[1] - dot * cb;
      const double dpdn = 0.0;
      const double cval = pe[0] - (dn_e + dpdn) * diagdis * 0.5;      // :415
      const double f_surf = cval * area;
      contrib[0 * ne + e] = inv_re * stx1 * area;                     // shear_x_force :341
      contrib[1 * ne + e] = -f_surf * ca;                             // f_surf_x :421
      contrib[2 * ne + e] = inv_re * sty1 * area;                     // shear_y_force :343
      contrib[3 * ne + e] = -f_surf * cb;                             // f_surf_y :423
      contrib[4 * ne + e] = area;
      contrib[5 * ne + e] = 0.5 * fabs(b3);                           // area_xz :330
      contrib[6 * ne + e] = 0.5 * fabs(a3);                           // area_yz :329
    }
  }
}

// Element-order sums (the serial order of the reference's loop, so the sums are
// bit-identical to the oracle) and the coefficients (subStressCal1.f90:428-450).
__global__ void k_stress_sum(const double* __restrict__ contrib, int ne, double* coef) {
  __shared__ double s[7];
  if (threadIdx.x < 7) {
    const double* c = contrib + (long long)threadIdx.x * ne;
    double acc = 0.0;
    for (int e = 0; e < ne; ++e) acc = acc + c[e];
    s[threadIdx.x] = acc;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const double area_Sx = 0.5 * s[5], area_Sy = 0.5 * s[6];
    coef[0] = 2.0 * (s[0] / area_Sx);
    coef[1] = 2.0 * (s[1] / area_Sy);
    coef[2] = 2.0 * (s[2] / area_Sy);
    coef[3] = 2.0 * (s[3] / area_Sx);
  }
}

// ------------------------------------------------------------------- host side

// shiftSurfaceNodesMovingbody's node loop (subSearch.f90:64-73): x = xr + xmove.
__global__ void k_shift_nodes(double* __restrict__ nodes, int nn, double dx, double dy, double dz) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nn) return;
  const double xr = nodes[i], yr = nodes[nn + i], zr = nodes[2 * nn + i];
  nodes[i] = xr + dx;
  nodes[nn + i] = yr + dy;
  nodes[2 * nn + i] = zr + dz;
}

int run_move_body(ib3d_ctx* c, double dx, double dy, double dz) {
  k_shift_nodes<<<nblk(c->nnodes), kBlock, 0, c->st>>>(c->d_nodes, (int)c->nnodes, dx, dy, dz);
  IB3D_CUDA(c, cudaGetLastError());
  c->launches += 2;
  return run_surface_norm(c);
}

int run_surface_norm(ib3d_ctx* c) {
  k_surface_norm<<<nblk(c->nelems), kBlock, 0, c->st>>>(c->d_nodes, c->d_tri, (int)c->nnodes, (int)c->nelems,
                                                        (double)c->inor, c->d_surf);
  IB3D_CUDA(c, cudaGetLastError());
  return IB3D_OK;
}

namespace {
void free_sched(ForceSched& s) {
  cudaFree(s.order); cudaFree(s.rd_idx); cudaFree(s.rd_src); cudaFree(s.tgt); cudaFree(s.brk);
  cudaFree(s.fin); cudaFree(s.out); cudaFree(s.final_ops);
  s = ForceSched{};
}

// Dependency levels (level = 1 + max level of the sources; sources precede the op in
// serial order) and the level-sorted op list.
int build_levels(ib3d_ctx* c, ForceSched& s) {
  const int n = s.nops;
  std::vector<int> src((size_t)8 * n), lvl(n, 0);
  std::vector<unsigned char> fin(n);
  if (n > 0) {
    IB3D_CUDA(c, cudaMemcpyAsync(src.data(), s.rd_src, sizeof(int) * 8 * (size_t)n, cudaMemcpyDeviceToHost, c->st));
    IB3D_CUDA(c, cudaMemcpyAsync(fin.data(), s.fin, (size_t)n, cudaMemcpyDeviceToHost, c->st));
    IB3D_CUDA(c, cudaStreamSynchronize(c->st));
  }
  int maxl = -1;
  for (int q = 0; q < n; ++q) {
    int l = 0;
    for (int r = 0; r < 8; ++r) {
      const int sidx = src[8 * (size_t)q + r];
      if (sidx >= 0) l = std::max(l, lvl[sidx] + 1);
    }
    lvl[q] = l;
    maxl = std::max(maxl, l);
  }
  s.nlevels = maxl + 1;
  s.level_off.assign((size_t)s.nlevels + 1, 0);
  for (int q = 0; q < n; ++q) s.level_off[lvl[q] + 1]++;
  for (int l = 0; l < s.nlevels; ++l) s.level_off[l + 1] += s.level_off[l];
  std::vector<int> order(n), pos(s.level_off.begin(), s.level_off.end() - 1), finals;
  for (int q = 0; q < n; ++q) order[pos[lvl[q]]++] = q;
  for (int q = 0; q < n; ++q)
    if (fin[q]) finals.push_back(q);
  s.nfinal = (int)finals.size();
  IB3D_CUDA(c, cudaMalloc(&s.order, sizeof(int) * (size_t)std::max(n, 1)));
  IB3D_CUDA(c, cudaMalloc(&s.final_ops, sizeof(int) * (size_t)std::max(s.nfinal, 1)));
  if (n > 0)
    IB3D_CUDA(c, cudaMemcpyAsync(s.order, order.data(), sizeof(int) * (size_t)n, cudaMemcpyHostToDevice, c->st));
  if (s.nfinal > 0)
    IB3D_CUDA(c, cudaMemcpyAsync(s.final_ops, finals.data(), sizeof(int) * (size_t)s.nfinal,
                                 cudaMemcpyHostToDevice, c->st));
  IB3D_CUDA(c, cudaStreamSynchronize(c->st));
  return IB3D_OK;
}

int alloc_sched(ib3d_ctx* c, ForceSched& s, int nops) {
  free_sched(s);
  s.nops = nops;
  const size_t n = (size_t)std::max(nops, 1);
  IB3D_CUDA(c, cudaMalloc(&s.rd_idx, sizeof(int) * 8 * n));
  IB3D_CUDA(c, cudaMalloc(&s.rd_src, sizeof(int) * 8 * n));
  IB3D_CUDA(c, cudaMalloc(&s.tgt, sizeof(int) * n));
  IB3D_CUDA(c, cudaMalloc(&s.brk, sizeof(int) * 3 * n));
  IB3D_CUDA(c, cudaMalloc(&s.fin, n));
  IB3D_CUDA(c, cudaMalloc(&s.out, sizeof(double) * n));
  return IB3D_OK;
}
}  // namespace

void free_ib(ib3d_ctx* c) {
  free_sched(c->fv);
  free_sched(c->fp);
}

namespace {
// Scratch of at least `n` long longs in c->d_scan (counts at 0..7, block offsets from 8).
int ensure_scan(ib3d_ctx* c, size_t n) {
  if (n + 9 > c->scan_cap) {
    cudaFree(c->d_scan);
    c->d_scan = nullptr;
    c->scan_cap = n + 64;
    IB3D_CUDA(c, cudaMalloc(&c->d_scan, sizeof(long long) * c->scan_cap));
  }
  return IB3D_OK;
}
int finish_search(ib3d_ctx* c, int bi0, int bj0, int bk0, int bni, int bnj, int bnk);
}  // namespace

int run_search(ib3d_ctx* c) {
  const Dims& d = c->d;
  const int bi0 = (int)c->box[0], bj0 = (int)c->box[2], bk0 = (int)c->box[4];
  const int bni = (int)(c->box[1] - c->box[0] + 1), bnj = (int)(c->box[3] - c->box[2] + 1),
            bnk = (int)(c->box[5] - c->box[4] + 1);
  const unsigned nbox = (unsigned)bni * bnj * bnk;
  const int ne = (int)c->nelems;
  // fresh flags and maps
  IB3D_CUDA(c, cudaMemsetAsync(c->cell, 0, (size_t)d.n3, c->st));
  cudaFree(c->d_minel);
  c->d_minel = nullptr;
  IB3D_CUDA(c, cudaMalloc(&c->d_minel, sizeof(int) * (size_t)nbox));
  k_tagging<<<nblk(nbox), kBlock, 0, c->st>>>(d, c->g, c->d_surf, ne, bi0, bj0, bk0, bni, bnj, bnk, nullptr, 0,
                                               c->cell, c->d_minel);
  IB3D_CUDA(c, cudaGetLastError());
  return finish_search(c, bi0, bj0, bk0, bni, bnj, bnk);
}

// selectiveRetagging (subSearch.f90:327-512): the tagging test on the 6x6x6
// neighbourhood of every cell of the current IB list, every other cell keeping its
// flag; then the counts, the IB list, the normal distances and the ghost-point
// schedules as after a full search. The neighbourhoods' cells are marked in a mask
// over their bounding box (clipped to the interior), compacted into a list, and only
// those are tagged.
int run_selective_retag(ib3d_ctx* c) {
  const Dims& d = c->d;
  const int nib = c->nib, ne = (int)c->nelems;
  int* dbound = reinterpret_cast<int*>(c->d_scan);
  const int init[6] = {0x7fffffff, -0x7fffffff, 0x7fffffff, -0x7fffffff, 0x7fffffff, -0x7fffffff};
  IB3D_CUDA(c, cudaMemcpyAsync(dbound, init, sizeof(init), cudaMemcpyHostToDevice, c->st));
  k_ib_bounds<<<std::min(nblk(nib), 64u), kBlock, 0, c->st>>>(c->d_iblist, nib, dbound);
  int hb[6];
  IB3D_CUDA(c, cudaMemcpyAsync(hb, dbound, sizeof(hb), cudaMemcpyDeviceToHost, c->st));
  IB3D_CUDA(c, cudaStreamSynchronize(c->st));
  const int bi0 = std::max(hb[0] - 2, 2), bi1 = std::min(hb[1] + 3, d.nx + 1);
  const int bj0 = std::max(hb[2] - 2, 2), bj1 = std::min(hb[3] + 3, d.ny + 1);
  const int bk0 = std::max(hb[4] - 2, 2), bk1 = std::min(hb[5] + 3, d.nz + 1);
  const int bni = bi1 - bi0 + 1, bnj = bj1 - bj0 + 1, bnk = bk1 - bk0 + 1;
  const unsigned nbox = (unsigned)bni * bnj * bnk;
  cudaFree(c->d_minel);
  c->d_minel = nullptr;
  IB3D_CUDA(c, cudaMalloc(&c->d_minel, sizeof(int) * (size_t)nbox));
  IB3D_CUDA(c, cudaMemsetAsync(c->d_minel, 0, sizeof(int) * (size_t)nbox, c->st));
  if ((size_t)nbox > c->retag_cap) {
    cudaFree(c->d_retag_mask);
    cudaFree(c->d_retag_list);
    c->d_retag_mask = nullptr;
    c->d_retag_list = nullptr;
    c->retag_cap = (size_t)nbox + (size_t)nbox / 4;
    IB3D_CUDA(c, cudaMalloc(&c->d_retag_mask, c->retag_cap));
    IB3D_CUDA(c, cudaMalloc(&c->d_retag_list, 3 * sizeof(int) * c->retag_cap));
  }
  IB3D_CUDA(c, cudaMemsetAsync(c->d_retag_mask, 0, nbox, c->st));
  k_mark_neighbourhoods<<<nblk(216ll * nib), kBlock, 0, c->st>>>(c->d_iblist, nib, bi0, bj0, bk0, bni, bnj, bnk,
                                                                  c->d_retag_mask);
  const unsigned nb = nblk(nbox);
  if (int rc = ensure_scan(c, nb)) return rc;
  long long* boff = c->d_scan + 8;
  k_mask_blockcount<<<nb, kBlock, 0, c->st>>>(c->d_retag_mask, nbox, boff);
  k_exclusive_scan<<<1, 1024, 0, c->st>>>(boff, (int)nb, c->d_scan);
  long long nlist = 0;
  IB3D_CUDA(c, cudaMemcpyAsync(&nlist, c->d_scan, sizeof(long long), cudaMemcpyDeviceToHost, c->st));
  IB3D_CUDA(c, cudaStreamSynchronize(c->st));
  // the list is sized for the whole box: the three index blocks start nlist apart
  k_mask_scatter<<<nb, kBlock, 0, c->st>>>(c->d_retag_mask, nbox, bi0, bj0, bk0, bni, bnj, boff, (int)nlist,
                                           c->d_retag_list);
  if (nlist > 0)
    k_tagging<<<nblk(nlist), kBlock, 0, c->st>>>(d, c->g, c->d_surf, ne, bi0, bj0, bk0, bni, bnj, bnk,
                                                 c->d_retag_list, (int)nlist, c->cell, c->d_minel);
  IB3D_CUDA(c, cudaGetLastError());
  c->retagged = nlist;
  return finish_search(c, bi0, bj0, bk0, bni, bnj, bnk);
}

namespace {
// The part of the search after the flags are set: counts, the lexicographic IB list
// over the box (every IB cell lies in it), the normal distances and the ghost-point
// schedules.
int finish_search(ib3d_ctx* c, int bi0, int bj0, int bk0, int bni, int bnj, int bnk) {
  const Dims& d = c->d;
  const unsigned nbox = (unsigned)bni * bnj * bnk;
  const int ne = (int)c->nelems;
  IB3D_CUDA(c, cudaMemsetAsync(c->ibmap, 0xff, sizeof(int) * (size_t)d.n3, c->st));
  // counts
  unsigned long long* dcount = reinterpret_cast<unsigned long long*>(c->d_scan);
  IB3D_CUDA(c, cudaMemsetAsync(dcount, 0, 5 * sizeof(unsigned long long), c->st));
  k_count<<<nblk((long long)d.nx * d.ny * d.nz), kBlock, 0, c->st>>>(d, c->cell, dcount);
  unsigned long long hc[5];
  IB3D_CUDA(c, cudaMemcpyAsync(hc, dcount, sizeof(hc), cudaMemcpyDeviceToHost, c->st));
  IB3D_CUDA(c, cudaStreamSynchronize(c->st));
  for (int q = 0; q < 5; ++q) c->counts[q] = (long long)hc[q];
  c->nib = (int)hc[2];
  const int nib = c->nib;
  // compaction of the IB cells
  cudaFree(c->d_iblist); cudaFree(c->d_nelp); cudaFree(c->d_nd);
  c->d_iblist = nullptr; c->d_nelp = nullptr; c->d_nd = nullptr;
  IB3D_CUDA(c, cudaMalloc(&c->d_iblist, sizeof(int) * 3 * (size_t)std::max(nib, 1)));
  IB3D_CUDA(c, cudaMalloc(&c->d_nelp, sizeof(int) * (size_t)std::max(nib, 1)));
  IB3D_CUDA(c, cudaMalloc(&c->d_nd, sizeof(double) * 7 * (size_t)std::max(nib, 1)));
  const unsigned nb = nblk(nbox);
  if (int rc = ensure_scan(c, nb)) return rc;
  long long* boff = c->d_scan + 8;
  k_ib_blockcount<<<nb, kBlock, 0, c->st>>>(d, c->cell, bi0, bj0, bk0, bni, bnj, nbox, boff);
  k_exclusive_scan<<<1, 1024, 0, c->st>>>(boff, (int)nb, c->d_scan);
  k_ib_scatter<<<nb, kBlock, 0, c->st>>>(d, c->cell, bi0, bj0, bk0, bni, bnj, nbox, boff, nib, c->d_iblist);
  if (nib > 0)
    k_normdist<<<nblk(nib), kBlock, 0, c->st>>>(d, c->g, c->d_surf, ne, c->d_iblist, nib, c->d_minel, bi0, bj0,
                                                bk0, bni, bnj, c->d_nelp, c->d_nd, c->ibmap);
  IB3D_CUDA(c, cudaGetLastError());
  // ghost-point schedules
  IB3D_CUDA(c, cudaMemsetAsync(c->d_flag, 0, sizeof(int), c->st));
  int rc = alloc_sched(c, c->fv, 6 * nib);
  if (rc) return rc;
  rc = alloc_sched(c, c->fp, nib);
  if (rc) return rc;
  if (nib > 0) {
    k_sched_vel<<<nblk(6ll * nib), kBlock, 0, c->st>>>(d, c->g, c->d_iblist, c->d_nelp, c->d_nd, c->d_surf, nib, ne,
                                                       c->ibmap, c->fv.brk, c->fv.rd_idx, c->fv.rd_src, c->fv.tgt,
                                                       c->fv.fin, c->d_flag);
    k_sched_p<<<nblk(nib), kBlock, 0, c->st>>>(d, c->g, c->d_iblist, c->d_nelp, c->d_nd, c->d_surf, nib, ne,
                                               c->ibmap, c->fp.brk, c->fp.rd_idx, c->fp.rd_src, c->fp.tgt, c->fp.fin,
                                               c->d_flag);
    IB3D_CUDA(c, cudaGetLastError());
  }
  rc = build_levels(c, c->fv);
  if (rc) return rc;
  rc = build_levels(c, c->fp);
  if (rc) return rc;
  int flag = 0;
  IB3D_CUDA(c, cudaMemcpy(&flag, c->d_flag, sizeof(int), cudaMemcpyDeviceToHost));
  c->have_scache = false;
  if (flag) {
    c->err = "ib3d_search: a ghost-point probe fell outside the grid";
    return IB3D_ERR_PROBE;
  }
  return IB3D_OK;
}
}  // namespace

int run_velocity_forcing(ib3d_ctx* c) {
  PhaseScope ps(c, PH_FORCING);
  ForceSched& s = c->fv;
  c->launches += s.nlevels + (s.nfinal > 0 ? 1 : 0);
  for (int l = 0; l < s.nlevels; ++l) {
    const int off = s.level_off[l], cnt = s.level_off[l + 1] - off;
    if (cnt <= 0) continue;
    k_force_vel<<<nblk(cnt), kBlock, 0, c->st>>>(c->g, s.order, off, cnt, c->d_iblist, c->d_nelp, c->d_nd, c->d_surf,
                                                 c->nib, (int)c->nelems, s.brk, s.rd_idx, s.rd_src, c->ut, c->vt,
                                                 c->wt, c->motion, s.out);
  }
  if (s.nfinal > 0)
    k_force_scatter<<<nblk(s.nfinal), kBlock, 0, c->st>>>(s.final_ops, s.nfinal, s.tgt, s.out, 1, c->ut, c->vt,
                                                          c->wt);
  IB3D_CUDA(c, cudaGetLastError());
  return IB3D_OK;
}

int run_pressure_forcing(ib3d_ctx* c) {
  PhaseScope ps(c, PH_FORCING);
  ForceSched& s = c->fp;
  for (int q = 0; q < 3; ++q) c->motion.acc[q] = -(c->motion.vel[q] - c->bprev[q]) / c->prm.deltat;   // :20
  c->launches += s.nlevels + (s.nfinal > 0 ? 1 : 0);
  for (int l = 0; l < s.nlevels; ++l) {
    const int off = s.level_off[l], cnt = s.level_off[l + 1] - off;
    if (cnt <= 0) continue;
    k_force_p<<<nblk(cnt), kBlock, 0, c->st>>>(c->g, s.order, off, cnt, c->d_iblist, c->d_nelp, c->d_nd, c->d_surf,
                                               c->nib, (int)c->nelems, s.brk, s.rd_idx, s.rd_src, c->p, c->motion,
                                               s.out);
  }
  if (s.nfinal > 0)
    k_force_scatter<<<nblk(s.nfinal), kBlock, 0, c->st>>>(s.final_ops, s.nfinal, s.tgt, s.out, 0, c->p, nullptr,
                                                          nullptr);
  IB3D_CUDA(c, cudaGetLastError());
  return IB3D_OK;
}

int run_stress(ib3d_ctx* c, int first, double coef[4]) {
  const int ne = (int)c->nelems;
  const int do_first = (first || !c->have_scache) ? 1 : 0;
  if (do_first) IB3D_CUDA(c, cudaMemsetAsync(c->d_flag, 0, sizeof(int), c->st));
  PhaseScope ps(c, PH_STRESS);
  c->launches += 2;
  k_stress_elem<<<nblk(ne), kBlock, 0, c->st>>>(c->d, c->g, c->d_surf, ne, do_first, c->d_scache, c->ut, c->vt,
                                                c->wt, c->p, 1.0 / c->prm.re, c->d_contrib, c->d_flag);
  k_stress_sum<<<1, 32, 0, c->st>>>(c->d_contrib, ne, c->d_coef);
  IB3D_CUDA(c, cudaGetLastError());
  if (do_first) {
    int flag = 0;
    IB3D_CUDA(c, cudaMemcpyAsync(&flag, c->d_flag, sizeof(int), cudaMemcpyDeviceToHost, c->st));
    IB3D_CUDA(c, cudaStreamSynchronize(c->st));
    if (flag) {
      c->err = "ib3d_stress: a drag probe fell outside the grid";
      return IB3D_ERR_PROBE;
    }
    c->have_scache = true;
  }
  if (coef) {
    IB3D_CUDA(c, cudaMemcpyAsync(coef, c->d_coef, 4 * sizeof(double), cudaMemcpyDeviceToHost, c->st));
    IB3D_CUDA(c, cudaStreamSynchronize(c->st));
  }
  return IB3D_OK;
}

}  // namespace ib3d
