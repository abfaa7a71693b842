// 3D parallel-beam X-ray projector: XRayTransform3D.project / back_project
// (scico/linop/xray/_xray3d.py:95-266) for sm_103a.
//
// Weight model (_calc_weights, :206-266).  Voxel (i0, i1, i2) has its centre
// at x = (i0+0.5, i1+0.5, i2+0.5) and lands on the detector at
//   Px_r = ((M[r][0]*x0 + M[r][1]*x1) + M[r][2]*x2) + M[r][3]      (r = 0, 1)
// in float32, each operation rounded.  left = Px - 0.25,
// to_next t = min(ceil(left) - left, 0.5), ul = floor(left), and the four taps
//   (ul0,   ul1)   t0*t1*4          (ul0+1, ul1)   (0.5-t0)*t1*4
//   (ul0,   ul1+1) t0*(0.5-t1)*4    (ul0+1, ul1+1) (0.5-t0)*(0.5-t1)*4
// each zeroed when its detector pixel is out of range.  Every kernel here
// evaluates these expressions with the same float32 operations in the same
// order (no contraction), so forward and adjoint use bit-identical weights.
//
// Two geometry kinds (ct_proj3d_views classifies):
//  * AXIS0 -- rotation about volume axis 0, slice i on detector row
//    i + row_offset with t0 = 0.5.  Then ul = 2*t1, ll = 2*(0.5-t1) (both
//    exact) and the two other taps are zero, and the column weights of pixel
//    (i1, i2) are the same for every slice.  The kernels compute each column
//    weight once per view and tile and apply it to 32 slices at a time:
//      forward  k_p3_ax0_fwd: lanes = slice pairs; a warp walks a 16x16 pixel
//               tile (staged in shared memory, [pixel][slice]) in the per-view
//               detector order of the order table, carrying the two open bins
//               in registers; each completed bin is added into the warp's own
//               slice of a [group][view][col][slice] accumulator in global
//               memory (old values loaded three bins ahead), which
//               k_p3_ax0_rows transposes into the sinogram.
//      adjoint  k_p3_ax0_adj: lanes = pixels along axis 2, 32 slices of
//               accumulators per thread; the view's detector rows of the
//               CTA's slices are staged as (y[c], y[c+1]) pairs, read with
//               one 8-byte shared load per slice.
//  * GENERAL -- any matrices.  The adjoint is voxel-driven (four gathers per
//    view, as the reference's _back_project_single).  The forward is
//    detector-driven: each detector pixel marches along the axis on which
//    the ray direction is largest and, in each plane, visits the voxels whose
//    footprint can cover it (an exact membership test on the rounded ul
//    decides), so each output has a single owner and no atomics are needed.
#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "kernels.cuh"

namespace ct {
namespace {

constexpr int kVT = CT_VIEW3D_STRIDE;
constexpr int kOrd = CT_PROJ3D_ORDER;
constexpr int kTileJ = 16, kTileK = 16;  // AXIS0 forward pixel tile (axis 1 x axis 2)
constexpr int kFwdSlices = 64;  // slices per forward CTA: two per lane
constexpr int kSvStride = 66;   // shared [pixel][slice] row stride (floats, even: float2 reads)
constexpr int kWalkGroup = 8;   // walk entries whose loads are issued together
constexpr int kFwdViewsPerCta = 16;
constexpr int kFwdViewsPerWarp = kFwdViewsPerCta / 8;
constexpr int kAdjRows = 16;  // AXIS0 adjoint tile: 16 (axis 1) x 32 (axis 2) pixels
constexpr int kAdjTargetCtas = 304;
constexpr int kGenViewChunk = 64;

static_assert(kTileJ * kTileK == kOrd, "order table covers one tile");

// Device error word of the 3D kernels' internal checks (bit 0: forward
// accumulator span, bit 1: adjoint window span).
__device__ int g_proj3d_err = 0;

int* errflag3_ptr() {
  static int* cached[64] = {nullptr};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  if (!cached[dev]) {
    int* p = nullptr;
    if (cudaGetSymbolAddress((void**)&p, g_proj3d_err) != cudaSuccess) return nullptr;
    cached[dev] = p;
  }
  return cached[dev];
}

// Detector coordinate of voxel centre (x0, x1, x2) on detector axis r of a
// view (_xray3d.py:214-219), rounded like the reference's float32 expression.
__device__ __forceinline__ float px3(float m0, float m1, float m2, float m3, float x0, float x1,
                                     float x2) {
  return fadd(fadd(fadd(fmul(m0, x0), fmul(m1, x1)), fmul(m2, x2)), m3);
}

// left = Px - w/2, to_next = min(ceil(left) - left, w), ul = floor(left)
// with w = 0.5 (:222-225).
__device__ __forceinline__ void edge3(float px, int& ul, float& t) {
  const float left = fsub(px, 0.25f);
  t = fminf(fsub(ceilf(left), left), 0.5f);
  ul = (int)floorf(left);
}

// 4-byte global -> shared copy that bypasses registers; zero-fills when
// `valid` is false (source size 0, nothing is read).
__device__ __forceinline__ void cp_async4(uint32_t dst, const float* src, bool valid) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(dst), "l"(src),
               "r"(valid ? 4 : 0)
               : "memory");
}

__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;" ::: "memory");
}

// ---------------------------------------------------------------------------
// AXIS0 forward
// ---------------------------------------------------------------------------
struct Ax0FwdArgs {
  const float* vol;  // (S, NJ, NK)
  float* acc_out;    // [G][V][C][Spad]
  const float* views;
  const uint16_t* order;
  int S, NJ, NK, V, C, Spad;
  int tiles_k, n_tiles, G;
  int vpc;   // views per CTA
  int* errflag;
  const double* skip;  // device flag: return at once when non-zero (may be null)
};

// Bin range of one 16x32 tile for one view.  Every operation of the rounded
// Px is monotone in each pixel index, so the tile's extremes are at corner
// pixels; floor(left) of those, widened by one bin below and two above
// (room for the second tap and the carried bin), gives [lo, hi).
__device__ __forceinline__ void tile_bins(float m11, float m12, float m13, int j0, int k0,
                                          int& lo, int& hi) {
  const float ja = (float)j0 + 0.5f, jb = (float)(j0 + kTileJ - 1) + 0.5f;
  const float ka = (float)k0 + 0.5f, kb = (float)(k0 + kTileK - 1) + 0.5f;
  const float a0 = fmul(m11, ja), a1 = fmul(m11, jb);
  const float b0 = fmul(m12, ka), b1 = fmul(m12, kb);
  const float pmin = fadd(fminf(a0, a1) + fminf(b0, b1), m13);
  const float pmax = fadd(fmaxf(a0, a1) + fmaxf(b0, b1), m13);
  lo = (int)floorf(pmin - 0.25f) - 1;
  hi = (int)floorf(pmax - 0.25f) + 3;
}

// Tile order of the forward: Z-order (Morton) over the tile grid's
// power-of-two bounding box, axis-2 tile bit lowest, the longer side's
// surplus bits on top.  A tile group takes a run of consecutive tiles in this
// order, a compact patch of the image, so that for every view the tiles it
// visits one after another touch overlapping detector columns and the
// accumulator's read-modify-write stays in L2.
__device__ __forceinline__ int bit_len(int n) {  // bits of n - 1 (0 for n <= 1)
  return n <= 1 ? 0 : 32 - __clz(n - 1);
}
__device__ __forceinline__ void zorder_decode(int code, int bj, int bk, int& tj, int& tk) {
  const int m = min(bj, bk);
  tj = 0;
  tk = 0;
  for (int b = 0; b < m; ++b) {
    tk |= ((code >> (2 * b)) & 1) << b;
    tj |= ((code >> (2 * b + 1)) & 1) << b;
  }
  const int rest = code >> (2 * m);
  if (bj > m) tj |= rest << m;
  else tk |= rest << m;
}
// Tiles of the grid [0, nj) x [0, nk) inside the box [j, j + sj) x [k, k + sk).
__device__ __forceinline__ int tiles_in(int j, int sj, int k, int sk, int nj, int nk) {
  return max(0, min(nj, j + sj) - j) * max(0, min(nk, k + sk) - k);
}
// Code of the r-th tile of the grid in Z-order (r < nj * nk): descend the
// surplus blocks, then the quadrants, counting the grid tiles each holds.
__device__ int zorder_select(int r, int nj, int nk) {
  const int bj = bit_len(nj), bk = bit_len(nk), m = min(bj, bk);
  const int sq = 1 << m;
  int code = 0, j = 0, k = 0;
  const int nblk = 1 << (max(bj, bk) - m);
  for (int blk = 0; blk < nblk; ++blk) {
    const int jb = bj > m ? blk * sq : 0, kb = bj > m ? 0 : blk * sq;
    const int c = tiles_in(jb, sq, kb, sq, nj, nk);
    if (r < c) {
      code = blk << (2 * m);
      j = jb;
      k = kb;
      break;
    }
    r -= c;
  }
  for (int l = m - 1; l >= 0; --l) {
    const int s = 1 << l;
    for (int q = 0; q < 4; ++q) {
      const int dj = q >> 1, dk = q & 1;
      const int c = tiles_in(j + dj * s, s, k + dk * s, s, nj, nk);
      if (r < c || q == 3) {
        code |= q << (2 * l);
        j += dj * s;
        k += dk * s;
        break;
      }
      r -= c;
    }
  }
  return code;
}

__global__ void __launch_bounds__(256, 2) k_p3_ax0_fwd(const Ax0FwdArgs a) {
  if (a.skip && *a.skip != 0.0) return;
  extern __shared__ __align__(16) float smem[];
  float* sv = smem;                                           // [kOrd][kSvStride]
  float2* tab = reinterpret_cast<float2*>(sv + kOrd * kSvStride);  // [8][kOrd]
  __shared__ float vpar[kFwdViewsPerCta][4];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int g = blockIdx.x, i0 = blockIdx.y * kFwdSlices, v0 = blockIdx.z * a.vpc;
  const int nvh = min(a.vpc, a.V - v0);
  float2* tabw = tab + warp * kOrd;
  const uint32_t sv_s = (uint32_t)__cvta_generic_to_shared(sv);

  // zero this CTA's slices of the output accumulator; fetch the CTA's view
  // parameters (M[1][1..3]) and each warp's walk orders (entry 32u + lane),
  // which do not depend on the tile
  for (int v = 0; v < nvh; ++v) {
    float* o = a.acc_out + ((size_t)g * a.V + v0 + v) * a.C * a.Spad + i0;
    for (int e = tid; e < a.C * kFwdSlices; e += 256)
      o[(size_t)(e / kFwdSlices) * a.Spad + (e % kFwdSlices)] = 0.0f;
  }
  if (tid < 3 * nvh) vpar[tid / 3][tid % 3] = a.views[(size_t)(v0 + tid / 3) * kVT + 5 + tid % 3];
  int ordr[kFwdViewsPerWarp][kOrd / 32];
#pragma unroll
  for (int w = 0; w < kFwdViewsPerWarp; ++w) {
    const int vi = warp + 8 * w;
    const uint16_t* ord = a.order + (size_t)(v0 + min(vi, nvh - 1)) * kOrd;
#pragma unroll
    for (int u = 0; u < kOrd / 32; ++u) ordr[w][u] = __ldg(ord + 32 * u + lane);
  }
  __syncthreads();

  // this group's run of tiles in Z-order, ranks [g per, (g + 1) per): each
  // thread looks up one rank, 256 tiles at a time
  __shared__ int2 tlist[256];  // tile origins (j0, k0)
  const int nrun = min((a.n_tiles + a.G - 1) / a.G, a.n_tiles - g * ((a.n_tiles + a.G - 1) / a.G));
  for (int q = 0; q < nrun; ++q) {
    if ((q & 255) == 0) {
      if (q + tid < nrun) {
        const int tiles_j = a.n_tiles / a.tiles_k, per = (a.n_tiles + a.G - 1) / a.G;
        int tj, tk;
        zorder_decode(zorder_select(g * per + q + tid, tiles_j, a.tiles_k), bit_len(tiles_j),
                      bit_len(a.tiles_k), tj, tk);
        tlist[tid] = make_int2(tj * kTileJ, tk * kTileK);
      }
      __syncthreads();
    }
    const int2 t0 = tlist[q & 255];
    const int j0 = t0.x, k0 = t0.y;
    // stage vol[i0+s][j0+j][k0+k] as sv[(j*16+k)*66 + s] with register-free
    // 4-byte async copies, all in flight at once.  A warp copies two
    // 16-float rows, slices s and s+1 of one j (lanes = k, then the second
    // half-warp): shared banks 2k + s and 2k + s + 1 are all distinct
#pragma unroll 8
    for (int q = 0; q < kOrd * kFwdSlices / 256; ++q) {
      const int row = 2 * (q * 8 + warp) + (lane >> 4);  // (s, j) = (row % 64, row / 64)
      const int s = row % kFwdSlices, j = row / kFwdSlices, k = lane & 15;
      const int gi = i0 + s, gj = j0 + j, gk = k0 + k;
      const bool ok = gi < a.S && gj < a.NJ && gk < a.NK;
      const float* src = ok ? a.vol + ((size_t)gi * a.NJ + gj) * a.NK + gk : a.vol;
      cp_async4(sv_s + (uint32_t)((j * kTileK + k) * kSvStride + s) * 4u, src, ok);
    }
    cp_async_wait_all();
    __syncthreads();

#pragma unroll 1
    for (int w = 0; w < kFwdViewsPerWarp; ++w) {
      const int vi = warp + 8 * w;
      if (vi >= nvh) break;
      const int v = v0 + vi;
      const float m11 = vpar[vi][0], m12 = vpar[vi][1], m13 = vpar[vi][2];
      int lo, hi;
      tile_bins(m11, m12, m13, j0, k0, lo, hi);
      const int nb = hi - lo;
      // table entries: (w0, bin << 16 | pixel*66).  The second tap's weight
      // is 1 - w0 = 2*(0.5 - t1) exactly; taps on columns off the detector
      // are accumulated and never written out, so no masks here
      int po[kOrd / 32];  // this view's order entries (register select, no local memory)
#pragma unroll
      for (int u = 0; u < kOrd / 32; ++u) {
        po[u] = ordr[0][u];
#pragma unroll
        for (int w2 = 1; w2 < kFwdViewsPerWarp; ++w2) po[u] = w == w2 ? ordr[w2][u] : po[u];
      }
#pragma unroll
      for (int u = 0; u < kOrd / 32; ++u) {
        const int p = po[u];
        const float x1 = (float)(j0 + p / kTileK) + 0.5f, x2 = (float)(k0 + p % kTileK) + 0.5f;
        // Px_1 with M[1][0] = 0: the x0 term is an exact zero
        const float px = fadd(fadd(fmul(m11, x1), fmul(m12, x2)), m13);
        int ul;
        float t1;
        edge3(px, ul, t1);
        const int rel = min(max(ul - lo, 0), nb - 2);  // in range: extremes at corners
        tabw[32 * u + lane] = make_float2(fmul(2.0f, t1), __int_as_float((rel << 16) | (p * kSvStride)));
      }
      __syncwarp();
      // this warp's slices of the output accumulator: column c at o[c * Spad]
      float2* o = reinterpret_cast<float2*>(a.acc_out + (((size_t)g * a.V + v) * a.C) * a.Spad + i0) + lane;
      const size_t ostride = (size_t)a.Spad / 2;
      auto old_at = [&](int c) {
        return (c >= 0 && c < a.C) ? o[(size_t)c * ostride] : make_float2(0.f, 0.f);
      };
      auto put = [&](int c, float2 val) {
        if (c >= 0 && c < a.C) o[(size_t)c * ostride] = val;
      };
      // Open bin cb (tile-relative): its total is cin + sum w0*x over its
      // own pixels (a); the next bin receives sum (1-w0)*x = s - a.  r0..r2
      // hold the accumulator's values of bins cb..cb+2, loaded ahead.
      int cb = 0;
      float2 cin = make_float2(0.f, 0.f), av = cin, sx = cin;
      float2 r0 = old_at(lo), r1 = old_at(lo + 1), r2 = old_at(lo + 2);
      for (int e0 = 0; e0 < kOrd; e0 += kWalkGroup) {
        float2 T[kWalkGroup], x[kWalkGroup];
#pragma unroll
        for (int u = 0; u < kWalkGroup; ++u) T[u] = tabw[e0 + u];
#pragma unroll
        for (int u = 0; u < kWalkGroup; ++u)
          x[u] = *reinterpret_cast<const float2*>(sv + (__float_as_int(T[u].y) & 0xffff) + 2 * lane);
#pragma unroll
        for (int u = 0; u < kWalkGroup; ++u) {
          const int rb = __float_as_int(T[u].y) >> 16;
          if (__builtin_expect(rb != cb, 0)) {  // warp-uniform: every lane reads the same entry
            put(lo + cb, make_float2(r0.x + (cin.x + av.x), r0.y + (cin.y + av.y)));
            const float2 nxt = make_float2(sx.x - av.x, sx.y - av.y);
            if (rb == cb + 1) {
              r0 = r1;
              r1 = r2;
              r2 = old_at(lo + cb + 3);
              cin = nxt;
            } else {  // a jump (rare: rounding at near-ties of the order)
              put(lo + cb + 1, make_float2(r1.x + nxt.x, r1.y + nxt.y));
              r0 = old_at(lo + rb);
              r1 = old_at(lo + rb + 1);
              r2 = old_at(lo + rb + 2);
              cin = make_float2(0.f, 0.f);
            }
            av = make_float2(0.f, 0.f);
            sx = av;
            cb = rb;
          }
          av.x = fmaf(T[u].x, x[u].x, av.x);
          av.y = fmaf(T[u].x, x[u].y, av.y);
          sx.x += x[u].x;
          sx.y += x[u].y;
        }
      }
      put(lo + cb, make_float2(r0.x + (cin.x + av.x), r0.y + (cin.y + av.y)));
      put(lo + cb + 1, make_float2(r1.x + (sx.x - av.x), r1.y + (sx.y - av.y)));
      __syncwarp();
    }
    __syncthreads();
  }
}

// proj[v][r][c] = sum_g acc_out[g][v][c][r - row_offset] (0 where no slice
// lands on row r).  32x32 (col, row) tiles through shared memory.
__global__ void k_p3_ax0_rows(const float* __restrict__ acc, float* __restrict__ proj, int V,
                              int R, int C, int S, int Spad, int G, int row_offset,
                              const double* skip) {
  if (skip && *skip != 0.0) return;
  __shared__ float t[32][33];
  const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32, v = blockIdx.z;
  const int lx = threadIdx.x, ly = threadIdx.y;  // 32 x 8
  for (int q = 0; q < 4; ++q) {
    const int cl = ly + 8 * q, c = c0 + cl;
    const int i = r0 + lx - row_offset;
    float s = 0.f;
    if (c < C && i >= 0 && i < S) {
      for (int gg = 0; gg < G; ++gg) s += acc[(((size_t)gg * V + v) * C + c) * Spad + i];
    }
    t[cl][lx] = s;
  }
  __syncthreads();
  for (int q = 0; q < 4; ++q) {
    const int rl = ly + 8 * q, r = r0 + rl, c = c0 + lx;
    if (r < R && c < C) proj[((size_t)v * R + r) * C + c] = t[lx][rl];
  }
}

// ---------------------------------------------------------------------------
// AXIS0 adjoint
// ---------------------------------------------------------------------------
struct Ax0AdjArgs {
  const float* proj;  // (V, R, C)
  float* out;         // (S, NJ, NK), or split partials
  const float* views;
  int S, NJ, NK, V, R, C, row_offset;
  int per_split;
  size_t split_stride;
  int* errflag;
  const double* skip;
};

// staged detector columns per slice row of the 16 x 32 adjoint tile:
// 15|m11| + 31|m12| + 5 <= 51 for |m11|, |m12| <= 1
constexpr int kAW = (kAdjRows - 1) + 31 + 6;
constexpr int kAdjStage = (32 * kAW + 255) / 256;  // staging slots per thread

__device__ __forceinline__ float2 ld_shared_f2(uint32_t addr) {
  float2 v;
  asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(addr));
  return v;
}

// Window [lo, lo + nb) of detector columns that the 16x32 tile at (j0, k0)
// reads in one view (corner bound as tile_bins, two extra columns above).
__device__ __forceinline__ void adj_window(float m11, float m12, float m13, int j0, int k0,
                                           int& lo, int& nb) {
  const float ja = (float)j0 + 0.5f, jb = (float)(j0 + kAdjRows - 1) + 0.5f;
  const float ka = (float)k0 + 0.5f, kb = (float)(k0 + 31) + 0.5f;
  const float a0 = fmul(m11, ja), a1 = fmul(m11, jb), b0 = fmul(m12, ka), b1 = fmul(m12, kb);
  lo = (int)floorf(fadd(fminf(a0, a1) + fminf(b0, b1), m13) - 0.25f) - 1;
  nb = (int)floorf(fadd(fmaxf(a0, a1) + fmaxf(b0, b1), m13) - 0.25f) + 3 - lo;
}

__global__ void __launch_bounds__(256, 2) k_p3_ax0_adj(const Ax0AdjArgs a) {
  if (a.skip && *a.skip != 0.0) return;
  // [2][32][kAW] pairs (y[c], y[c+1]) of the slice rows, double-buffered
  __shared__ __align__(16) float2 sy[2 * 32 * kAW];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int k0 = blockIdx.x * 32, j0 = blockIdx.y * kAdjRows;
  const int nsg = (a.S + 31) / 32;
  const int sg = blockIdx.z % nsg, split = blockIdx.z / nsg;
  const int i0 = sg * 32;
  const int k = k0 + lane;
  const int jj[2] = {j0 + warp, j0 + warp + 8};
  const int vs = split * a.per_split, ve = min(a.V, vs + a.per_split);
  const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(sy);

  // issue the copies of view v's window into buffer `buf`
  auto stage = [&](int v, int buf, int lo, int nb) {
    const float* src = a.proj + (size_t)v * a.R * a.C;
#pragma unroll
    for (int it = 0; it < kAdjStage; ++it) {
      const int e = tid + 256 * it;
      if (e < 32 * kAW) {
        const int s = e / kAW, bl = e - s * kAW;
        const int r = i0 + s + a.row_offset, c = lo + bl;
        const bool row_ok = bl < nb && i0 + s < a.S && r >= 0 && r < a.R;
        const float* row = src + (size_t)(row_ok ? r : 0) * a.C;
        const bool ok0 = row_ok && c >= 0 && c < a.C;
        const bool ok1 = row_ok && c + 1 >= 0 && c + 1 < a.C;
        const uint32_t d = sbase + (uint32_t)(buf * 32 * kAW + e) * 8u;
        cp_async4(d, ok0 ? row + c : a.proj, ok0);
        cp_async4(d + 4, ok1 ? row + c + 1 : a.proj, ok1);
      }
    }
  };

  float acc[2][32];
#pragma unroll
  for (int q = 0; q < 2; ++q)
#pragma unroll
    for (int s = 0; s < 32; ++s) acc[q][s] = 0.f;

  int lo = 0, nb = 0;
  if (vs < ve) {
    const float* m = a.views + (size_t)vs * kVT;
    adj_window(m[5], m[6], m[7], j0, k0, lo, nb);
    stage(vs, 0, lo, min(nb, kAW));
    cp_async_wait_all();
  }
  __syncthreads();
  for (int v = vs; v < ve; ++v) {
    const int buf = (v - vs) & 1;
    const float* m = a.views + (size_t)v * kVT;
    const float m11 = m[5], m12 = m[6], m13 = m[7];
    if (nb > kAW && tid == 0) atomicOr(a.errflag, 2);  // cannot happen for |m| <= 1
    const int nbc = min(nb, kAW);
    // next view's copies run while this view is computed
    int lo_n = 0, nb_n = 0;
    if (v + 1 < ve) {
      const float* mn = a.views + (size_t)(v + 1) * kVT;
      adj_window(mn[5], mn[6], mn[7], j0, k0, lo_n, nb_n);
      stage(v + 1, buf ^ 1, lo_n, min(nb_n, kAW));
    }
    const uint32_t vbase = sbase + (uint32_t)(buf * 32 * kAW) * 8u;
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const float x1 = (float)jj[q] + 0.5f, x2 = (float)k + 0.5f;
      const float px = fadd(fadd(fmul(m11, x1), fmul(m12, x2)), m13);
      int ul;
      float t1;
      edge3(px, ul, t1);
      float w0 = (ul >= 0 && ul < a.C) ? fmul(2.0f, t1) : 0.0f;
      float w1 = (ul + 1 >= 0 && ul + 1 < a.C) ? fmul(2.0f, fsub(0.5f, t1)) : 0.0f;
      int rel = ul - lo;
      if (rel < 0 || rel >= nbc - 1) {  // outside the staged window (cannot happen)
        rel = 0;
        w0 = 0.f;
        w1 = 0.f;
      }
      const uint32_t addr = vbase + (uint32_t)rel * 8u;
#pragma unroll
      for (int s = 0; s < 32; ++s) {
        const float2 y = ld_shared_f2(addr + (uint32_t)(s * kAW * 8));
        acc[q][s] = fmaf(w0, y.x, acc[q][s]);
        acc[q][s] = fmaf(w1, y.y, acc[q][s]);
      }
    }
    cp_async_wait_all();
    __syncthreads();
    lo = lo_n;
    nb = nb_n;
  }
  float* out = a.out + (size_t)split * a.split_stride;
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    if (jj[q] >= a.NJ || k >= a.NK) continue;
#pragma unroll
    for (int s = 0; s < 32; ++s) {
      if (i0 + s < a.S) out[((size_t)(i0 + s) * a.NJ + jj[q]) * a.NK + k] = acc[q][s];
    }
  }
}

// ---------------------------------------------------------------------------
// GENERAL adjoint: one voxel per thread, views in order, four gathers each
// (_back_project_single, :192-204).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_p3_gen_adj(const float* __restrict__ proj,
                                                    float* __restrict__ out,
                                                    const float* __restrict__ views, int n0,
                                                    int n1, int n2, int V, int R, int C,
                                                    int per_split, size_t split_stride,
                                                    const double* skip) {
  if (skip && *skip != 0.0) return;
  __shared__ float sm[kGenViewChunk * 8];
  const size_t n = (size_t)n0 * n1 * n2;
  const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int split = blockIdx.y;
  const int vs = split * per_split, ve = min(V, vs + per_split);
  int i0 = 0, i1 = 0, i2 = 0;
  if (e < n) {
    i2 = (int)(e % n2);
    const size_t r = e / n2;
    i1 = (int)(r % n1);
    i0 = (int)(r / n1);
  }
  const float x0 = (float)i0 + 0.5f, x1 = (float)i1 + 0.5f, x2 = (float)i2 + 0.5f;
  float acc = 0.f;
  for (int vc = vs; vc < ve; vc += kGenViewChunk) {
    const int nvc = min(kGenViewChunk, ve - vc);
    __syncthreads();
    for (int q = threadIdx.x; q < nvc * 8; q += blockDim.x)
      sm[q] = views[(size_t)(vc + q / 8) * kVT + (q & 7)];
    __syncthreads();
    if (e >= n) continue;
    for (int vi = 0; vi < nvc; ++vi) {
      const float* m = sm + vi * 8;
      int u0, u1;
      float t0, t1;
      edge3(px3(m[0], m[1], m[2], m[3], x0, x1, x2), u0, t0);
      edge3(px3(m[4], m[5], m[6], m[7], x0, x1, x2), u1, t1);
      const float s0 = fsub(0.5f, t0), s1 = fsub(0.5f, t1);
      const bool r0 = u0 >= 0 && u0 < R, r1 = u0 + 1 >= 0 && u0 + 1 < R;
      const bool c0 = u1 >= 0 && u1 < C, c1 = u1 + 1 >= 0 && u1 + 1 < C;
      const float* y = proj + (size_t)(vc + vi) * R * C;
      if (r0 && c0) acc = fmaf(__ldg(y + (size_t)u0 * C + u1), fmul(fmul(t0, t1), 4.0f), acc);
      if (r1 && c0) acc = fmaf(__ldg(y + (size_t)(u0 + 1) * C + u1), fmul(fmul(s0, t1), 4.0f), acc);
      if (r0 && c1) acc = fmaf(__ldg(y + (size_t)u0 * C + u1 + 1), fmul(fmul(t0, s1), 4.0f), acc);
      if (r1 && c1)
        acc = fmaf(__ldg(y + (size_t)(u0 + 1) * C + u1 + 1), fmul(fmul(s0, s1), 4.0f), acc);
    }
  }
  if (e < n) out[(size_t)split * split_stride + e] = acc;
}

// ---------------------------------------------------------------------------
// GENERAL forward: one detector pixel per thread.
// ---------------------------------------------------------------------------
// x range [lo, hi] of voxel centres along one axis allowed by the detector
// window [wlo, whi] on one detector axis, given Px = beta + mq * x.
__device__ __forceinline__ void narrow(float beta, float mq, float wlo, float whi, float& lo,
                                       float& hi) {
  if (fabsf(mq) > 1e-20f) {
    const float u = (wlo - beta) / mq, w = (whi - beta) / mq;
    lo = fmaxf(lo, fminf(u, w));
    hi = fminf(hi, fmaxf(u, w));
  } else if (beta < wlo || beta > whi) {
    lo = 1.0f;
    hi = 0.0f;
  }
}

__global__ void __launch_bounds__(256) k_p3_gen_fwd(const float* __restrict__ vol,
                                                    float* __restrict__ proj,
                                                    const float* __restrict__ views, int n0,
                                                    int n1, int n2, int V, int R, int C,
                                                    const double* skip) {
  if (skip && *skip != 0.0) return;
  const int v = blockIdx.y;
  const int pix = blockIdx.x * blockDim.x + threadIdx.x;
  if (pix >= R * C) return;
  const int r = pix / C, c = pix - (pix / C) * C;
  const float* m = views + (size_t)v * kVT;
  float mm[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) mm[q] = m[q];
  const int ax = (int)m[8];
  // the other two axes, ascending: p = ax==0 ? 1 : 0, q = ax==2 ? 1 : 2
  auto pick = [ax](float a0, float a1, float a2, int which) {
    // which: 0 = the marching axis, 1 = p, 2 = q
    const int k = which == 0 ? ax : (which == 1 ? (ax == 0 ? 1 : 0) : (ax == 2 ? 1 : 2));
    return k == 0 ? a0 : (k == 1 ? a1 : a2);
  };
  const float na_f = pick((float)n0, (float)n1, (float)n2, 0);
  const int na = (int)na_f, np = (int)pick((float)n0, (float)n1, (float)n2, 1),
            nq = (int)pick((float)n0, (float)n1, (float)n2, 2);
  const float ma0 = pick(mm[0], mm[1], mm[2], 0), mp0 = pick(mm[0], mm[1], mm[2], 1),
              mq0 = pick(mm[0], mm[1], mm[2], 2);
  const float ma1 = pick(mm[4], mm[5], mm[6], 0), mp1 = pick(mm[4], mm[5], mm[6], 1),
              mq1 = pick(mm[4], mm[5], mm[6], 2);
  // taps reaching (r, c) come from voxels with floor(left) in {r-1, r} x
  // {c-1, c}: Px in [r-0.75, r+1.25) x [c-0.75, c+1.25); widened by a margin
  // far above the rounding of the range arithmetic (the exact test decides)
  const float mg = 0.05f;
  const float w0lo = (float)r - 0.75f - mg, w0hi = (float)r + 1.25f + mg;
  const float w1lo = (float)c - 0.75f - mg, w1hi = (float)c + 1.25f + mg;
  // |x_p - centre_p| <= e_p from the 2x2 system of the (p, q) plane
  const float det = mp0 * mq1 - mq0 * mp1;
  const float h0 = 0.5f * (w0hi - w0lo), h1 = 0.5f * (w1hi - w1lo);
  const float ep = (fabsf(mq1) * h0 + fabsf(mq0) * h1) / fabsf(det);
  // voxel strides of the marching, p and q axes
  const size_t sa = (size_t)pick((float)((size_t)n1 * n2), (float)n2, 1.0f, 0);
  const size_t sp = ax == 0 ? (size_t)n2 : (size_t)n1 * n2;
  const size_t sq = ax == 2 ? (size_t)n2 : 1;
  float acc = 0.f;
  for (int ia = 0; ia < na; ++ia) {
    const float xa = (float)ia + 0.5f;
    const float al0 = ma0 * xa + mm[3], al1 = ma1 * xa + mm[7];
    const float cr0 = 0.5f * (w0lo + w0hi) - al0, cr1 = 0.5f * (w1lo + w1hi) - al1;
    const float cp = (mq1 * cr0 - mq0 * cr1) / det;
    const float plo = fmaxf(0.5f, cp - ep - mg), phi = fminf((float)np - 0.5f, cp + ep + mg);
    if (!(plo <= phi)) continue;
    const int ip0 = max(0, (int)ceilf(plo - 0.5f)), ip1 = min(np - 1, (int)floorf(phi - 0.5f));
    for (int ip = ip0; ip <= ip1; ++ip) {
      const float xp = (float)ip + 0.5f;
      float qlo = 0.5f, qhi = (float)nq - 0.5f;
      narrow(al0 + mp0 * xp, mq0, w0lo, w0hi, qlo, qhi);
      narrow(al1 + mp1 * xp, mq1, w1lo, w1hi, qlo, qhi);
      if (!(qlo <= qhi)) continue;
      const int iq0 = max(0, (int)ceilf(qlo - 0.5f - mg)), iq1 = min(nq - 1, (int)floorf(qhi - 0.5f + mg));
      for (int iq = iq0; iq <= iq1; ++iq) {
        const int i0 = ax == 0 ? ia : ip;
        const int i1 = ax == 0 ? ip : (ax == 1 ? ia : iq);
        const int i2 = ax == 2 ? ia : iq;
        const float x0 = (float)i0 + 0.5f, x1 = (float)i1 + 0.5f, x2 = (float)i2 + 0.5f;
        int u0, u1;
        float t0, t1;
        edge3(px3(mm[0], mm[1], mm[2], mm[3], x0, x1, x2), u0, t0);
        edge3(px3(mm[4], mm[5], mm[6], mm[7], x0, x1, x2), u1, t1);
        const int d0 = r - u0, d1 = c - u1;
        if ((unsigned)d0 > 1u || (unsigned)d1 > 1u) continue;
        const float f0 = d0 ? fsub(0.5f, t0) : t0;
        const float f1 = d1 ? fsub(0.5f, t1) : t1;
        const float w = fmul(fmul(f0, f1), 4.0f);
        acc = fmaf(w, __ldg(vol + ia * sa + ip * sp + iq * sq), acc);
      }
    }
  }
  proj[((size_t)v * R + r) * C + c] = acc;
}

__global__ void k_p3_sum_splits(const float* __restrict__ part, float* __restrict__ out, size_t n,
                                int nsplit, size_t stride) {
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n;
       e += (size_t)gridDim.x * blockDim.x) {
    float s = 0.0f;
    for (int k = 0; k < nsplit; ++k) s += part[(size_t)k * stride + e];
    out[e] = s;
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// Host planning and launchers
// ---------------------------------------------------------------------------

ct_status proj3d_check(const ct_geom3d* g, const char* who) {
  if (!g) return fail(CT_ERR_INVALID_ARG, "%s: null geometry", who);
  for (int q = 0; q < 3; ++q)
    if (g->shape[q] <= 0) return fail(CT_ERR_SHAPE, "%s: shape[%d]=%d", who, q, g->shape[q]);
  if (g->det_shape[0] <= 0 || g->det_shape[1] <= 0)
    return fail(CT_ERR_SHAPE, "%s: det_shape=(%d, %d)", who, g->det_shape[0], g->det_shape[1]);
  if (g->n_views <= 0) return fail(CT_ERR_SHAPE, "%s: n_views=%d", who, g->n_views);
  if (!g->views) return fail(CT_ERR_INVALID_ARG, "%s: null view table", who);
  if (g->kind != CT_PROJ3D_GENERAL && g->kind != CT_PROJ3D_AXIS0)
    return fail(CT_ERR_INVALID_ARG, "%s: kind=%d", who, g->kind);
  if (g->kind == CT_PROJ3D_AXIS0 && !g->order)
    return fail(CT_ERR_INVALID_ARG, "%s: AXIS0 geometry without an order table", who);
  const double n = (double)g->shape[0] * g->shape[1] * g->shape[2];
  if (n > 2147483647.0 || (double)g->det_shape[0] * g->det_shape[1] > 2147483647.0)
    return fail(CT_ERR_UNSUPPORTED, "%s: volume or detector above 2^31 elements", who);
  return CT_OK;
}

// Largest schedule values the tuner tries: AXIS0 forward tile groups and
// adjoint view splits.
constexpr int kMaxGroups = 8;
constexpr int kMaxSplits3d = 4;

// The AXIS0 span bounds need max |M[1][1]| and |M[1][2]|; ct_proj3d_views
// guarantees both <= 1, so the bounds are fixed.
Proj3dPlan proj3d_plan_sched(const ct_geom3d* g, Sched3d sc) {
  Proj3dPlan p;
  const int S = g->shape[0], NJ = g->shape[1], NK = g->shape[2], V = g->n_views;
  const int C = g->det_shape[1];
  const int sms = std::max(1, sm_count());
  int ns = 1, ns_max = 1;
  if (g->kind == CT_PROJ3D_AXIS0) {
    p.Spad = (S + kFwdSlices - 1) / kFwdSlices * kFwdSlices;
    p.tiles_k = (NK + kTileK - 1) / kTileK;
    p.n_tiles = p.tiles_k * ((NJ + kTileJ - 1) / kTileJ);
    const long base = (long)(p.Spad / kFwdSlices) * ((V + p.vpc - 1) / p.vpc);
    const int g_max = std::min(kMaxGroups, p.n_tiles);
    if (sc.G > 0) {
      p.G = std::min(sc.G, g_max);
    } else {
      // tile groups: fill the GPU (two CTAs per SM) with a small last wave
      const long slots = 2L * sms;
      double best = -1.0;
      for (int G = 1; G <= g_max; ++G) {
        const double waves = (double)(base * G) / (double)slots;
        const double score = std::min(1.0, waves) * waves / std::ceil(waves);
        if (score > best + 1e-9) {
          best = score;
          p.G = G;
        }
      }
    }
    p.fwd_smem = sizeof(float) * (size_t)kOrd * kSvStride + sizeof(float2) * 8 * kOrd;
    p.fwd_bytes = round_up(sizeof(float) * (size_t)p.G * V * C * p.Spad, 256);
    p.fwd_ws_bytes = round_up(sizeof(float) * (size_t)g_max * V * C * p.Spad, 256);
    const long ctas = (long)((NK + 31) / 32) * ((NJ + kAdjRows - 1) / kAdjRows) * (p.Spad / 32);
    if (ctas < kAdjTargetCtas) ns = (int)((kAdjTargetCtas + ctas - 1) / ctas);
    ns_max = std::max(1, V / 16);
  } else {
    const double n = (double)S * NJ * NK;
    const long ctas = (long)((n + 255) / 256);
    if (ctas < 4L * sms) ns = (int)((4L * sms + ctas - 1) / ctas);
    ns_max = std::max(1, V / 8);
  }
  ns = std::min(ns, ns_max);
  const int ns_ws = std::max(ns, std::min(kMaxSplits3d, ns_max));
  if (sc.ns > 0) ns = std::min(sc.ns, ns_max);
  p.per_split = (V + ns - 1) / ns;
  p.nsplit = (V + p.per_split - 1) / p.per_split;
  p.adj_bytes = p.nsplit > 1 ? round_up(sizeof(float) * (size_t)p.nsplit * S * NJ * NK, 256) : 0;
  p.adj_ws_bytes = ns_ws > 1 ? round_up(sizeof(float) * (size_t)ns_ws * S * NJ * NK, 256) : 0;
  p.adj_ws_bytes = std::max(p.adj_ws_bytes, p.adj_bytes);
  return p;
}

// Schedules recorded by ct_proj3d_autotune, keyed by the geometry's sizes
// and kind.
using Sched3dKey = std::tuple<int, int, int, int, int, int, int>;
struct Sched3dVal {
  Sched3d s;
  float fwd_us = 0.0f, adj_us = 0.0f;
};
std::mutex g_sched3_mu;
std::map<Sched3dKey, Sched3dVal> g_sched3;

Sched3dKey sched3_key(const ct_geom3d* g) {
  return Sched3dKey(g->shape[0], g->shape[1], g->shape[2], g->n_views, g->det_shape[0], g->det_shape[1], g->kind);
}

bool sched3_lookup(const ct_geom3d* g, Sched3dVal& out) {
  std::lock_guard<std::mutex> lk(g_sched3_mu);
  const auto it = g_sched3.find(sched3_key(g));
  if (it == g_sched3.end()) return false;
  out = it->second;
  return true;
}

Proj3dPlan proj3d_plan(const ct_geom3d* g, int batch) {
  (void)batch;  // one volume per launch; a batch runs the same plan per volume
  Sched3dVal v;
  return proj3d_plan_sched(g, sched3_lookup(g, v) ? v.s : Sched3d{});
}

ct_status need_ws(const char* who, size_t need, void* ws, size_t bytes) {
  if (need == 0) return CT_OK;
  if (!ws || bytes < need || !aligned(ws, 256))
    return fail(CT_ERR_WORKSPACE, "%s: need %zu bytes (256-B aligned), got %zu", who, need, bytes);
  return CT_OK;
}

ct_status proj3d_prepare(const ct_geom3d* g, const Proj3dPlan& p) {
  if (!errflag3_ptr()) return fail(CT_ERR_CUDA, "proj3d: error-word address unavailable");
  if (g->kind != CT_PROJ3D_AXIS0) return CT_OK;
  return cuda_check(cudaFuncSetAttribute(k_p3_ax0_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)p.fwd_smem),
                    "k_p3_ax0_fwd smem attribute");
}

ct_status proj3d_fwd_launch(const ct_geom3d* g, const Proj3dPlan& p, const float* vol, float* proj,
                            void* ws, cudaStream_t s, const double* skip) {
  const int S = g->shape[0], NJ = g->shape[1], NK = g->shape[2], V = g->n_views;
  const int R = g->det_shape[0], C = g->det_shape[1];
  if (g->kind == CT_PROJ3D_AXIS0) {
    Ax0FwdArgs a;
    a.vol = vol;
    a.acc_out = static_cast<float*>(ws);
    a.views = g->views;
    a.order = g->order;
    a.S = S;
    a.NJ = NJ;
    a.NK = NK;
    a.V = V;
    a.C = C;
    a.Spad = p.Spad;
    a.tiles_k = p.tiles_k;
    a.n_tiles = p.n_tiles;
    a.G = p.G;
    a.vpc = p.vpc;
    a.errflag = errflag3_ptr();
    a.skip = skip;
    dim3 grid(p.G, p.Spad / kFwdSlices, (V + p.vpc - 1) / p.vpc);
    k_p3_ax0_fwd<<<grid, 256, p.fwd_smem, s>>>(a);
    ct_status st = launch_check("k_p3_ax0_fwd");
    if (st != CT_OK) return st;
    dim3 g2((C + 31) / 32, (R + 31) / 32, V);
    k_p3_ax0_rows<<<g2, dim3(32, 8), 0, s>>>(a.acc_out, proj, V, R, C, S, p.Spad, p.G,
                                             g->row_offset, skip);
    return launch_check("k_p3_ax0_rows");
  }
  dim3 grid((R * C + 255) / 256, V);
  k_p3_gen_fwd<<<grid, 256, 0, s>>>(vol, proj, g->views, S, NJ, NK, V, R, C, skip);
  return launch_check("k_p3_gen_fwd");
}

ct_status proj3d_adj_launch(const ct_geom3d* g, const Proj3dPlan& p, const float* proj, float* out,
                            float* part, cudaStream_t s, const double* skip) {
  const int S = g->shape[0], NJ = g->shape[1], NK = g->shape[2], V = g->n_views;
  const int R = g->det_shape[0], C = g->det_shape[1];
  const size_t vol_n = (size_t)S * NJ * NK;
  float* dst = p.nsplit > 1 ? part : out;
  if (g->kind == CT_PROJ3D_AXIS0) {
    Ax0AdjArgs a;
    a.proj = proj;
    a.out = dst;
    a.views = g->views;
    a.S = S;
    a.NJ = NJ;
    a.NK = NK;
    a.V = V;
    a.R = R;
    a.C = C;
    a.row_offset = g->row_offset;
    a.per_split = p.per_split;
    a.split_stride = vol_n;
    a.errflag = errflag3_ptr();
    a.skip = skip;
    dim3 grid((NK + 31) / 32, (NJ + kAdjRows - 1) / kAdjRows, ((S + 31) / 32) * p.nsplit);
    k_p3_ax0_adj<<<grid, 256, 0, s>>>(a);
    return launch_check("k_p3_ax0_adj");
  }
  dim3 grid((unsigned)((vol_n + 255) / 256), p.nsplit);
  k_p3_gen_adj<<<grid, 256, 0, s>>>(proj, dst, g->views, S, NJ, NK, V, R, C, p.per_split, vol_n,
                                    skip);
  return launch_check("k_p3_gen_adj");
}

}  // namespace ct

extern "C" {

ct_status ct_proj3d_views(const float* matrices, int32_t n_views, const int32_t* shape,
                          const int32_t* det_shape, float* views_out, uint16_t* order_out,
                          int32_t* kind_out, int32_t* row_offset_out) {
  using ct::fail;
  if (!matrices || !shape || !det_shape || !views_out || !kind_out || !row_offset_out)
    return fail(CT_ERR_INVALID_ARG, "ct_proj3d_views: null argument");
  if (n_views <= 0) return fail(CT_ERR_SHAPE, "ct_proj3d_views: n_views=%d", n_views);
  for (int q = 0; q < 3; ++q)
    if (shape[q] <= 0) return fail(CT_ERR_SHAPE, "ct_proj3d_views: shape[%d]=%d", q, shape[q]);
  if (det_shape[0] <= 0 || det_shape[1] <= 0)
    return fail(CT_ERR_SHAPE, "ct_proj3d_views: det_shape=(%d, %d)", det_shape[0], det_shape[1]);
  for (int v = 0; v < n_views; ++v) {
    const float* m = matrices + (size_t)v * 8;
    float* t = views_out + (size_t)v * CT_VIEW3D_STRIDE;
    for (int q = 0; q < 8; ++q) {
      if (!std::isfinite(m[q]))
        return fail(CT_ERR_NONFINITE, "ct_proj3d_views: matrix %d has a non-finite entry", v);
      t[q] = m[q];
    }
    const double d[3] = {(double)m[1] * m[6] - (double)m[2] * m[5],
                         (double)m[2] * m[4] - (double)m[0] * m[6],
                         (double)m[0] * m[5] - (double)m[1] * m[4]};
    int ax = 0;
    for (int q = 1; q < 3; ++q)
      if (std::fabs(d[q]) > std::fabs(d[ax])) ax = q;
    const double n0 = std::sqrt((double)m[0] * m[0] + (double)m[1] * m[1] + (double)m[2] * m[2]);
    const double n1 = std::sqrt((double)m[4] * m[4] + (double)m[5] * m[5] + (double)m[6] * m[6]);
    if (!(std::fabs(d[ax]) > 1e-6 * n0 * n1))
      return fail(CT_ERR_UNSUPPORTED,
                  "ct_proj3d_views: matrix %d maps the volume onto a line (parallel rows)", v);
    t[8] = (float)ax;
    t[9] = t[10] = t[11] = 0.0f;
  }
  // AXIS0: rows of axis 0 only, shared by all views, each slice on one row
  // with to_next 0.5 (float32 arithmetic as the reference's; the zero terms
  // of Px_0 are exact)
  bool ax0 = order_out != nullptr;
  int32_t off = 0;
  for (int v = 0; ax0 && v < n_views; ++v) {
    const float* m = matrices + (size_t)v * 8;
    ax0 = m[1] == 0.0f && m[2] == 0.0f && m[4] == 0.0f && std::fabs(m[5]) <= 1.0f &&
          std::fabs(m[6]) <= 1.0f;
    // every view must put slice i on row i + off with to_next 0.5 (the
    // translation may differ between views by amounts below one ulp)
    for (int i = 0; ax0 && i < shape[0]; ++i) {
      const float x0 = (float)i + 0.5f;
      const float px = m[0] * x0 + m[3];  // two roundings; host code is not contracted
      const float left = px - 0.25f;
      const float tn = std::fmin(std::ceil(left) - left, 0.5f);
      const int ul = (int)std::floor(left);
      if (v == 0 && i == 0) off = ul;
      ax0 = tn == 0.5f && ul == i + off;
    }
  }
  *kind_out = ax0 ? CT_PROJ3D_AXIS0 : CT_PROJ3D_GENERAL;
  *row_offset_out = ax0 ? off : 0;
  if (ax0) {
    std::vector<std::pair<double, int>> key(CT_PROJ3D_ORDER);
    for (int v = 0; v < n_views; ++v) {
      const float* m = matrices + (size_t)v * 8;
      for (int p = 0; p < CT_PROJ3D_ORDER; ++p)
        key[p] = {(double)m[5] * (p / ct::kTileK) + (double)m[6] * (p % ct::kTileK), p};
      std::stable_sort(key.begin(), key.end(),
                       [](const std::pair<double, int>& a, const std::pair<double, int>& b) {
                         return a.first < b.first;
                       });
      for (int p = 0; p < CT_PROJ3D_ORDER; ++p)
        order_out[(size_t)v * CT_PROJ3D_ORDER + p] = (uint16_t)key[p].second;
    }
  }
  return CT_OK;
}

ct_status ct_proj3d_workspace(const ct_geom3d* g, int32_t batch, size_t* fwd_bytes,
                              size_t* adj_bytes) {
  ct_status st = ct::proj3d_check(g, "ct_proj3d_workspace");
  if (st != CT_OK) return st;
  if (batch <= 0) return ct::fail(CT_ERR_INVALID_ARG, "ct_proj3d_workspace: batch=%d", batch);
  const ct::Proj3dPlan p = ct::proj3d_plan(g, batch);
  if (fwd_bytes) *fwd_bytes = p.fwd_ws_bytes;  // fit any schedule the autotuner may record
  if (adj_bytes) *adj_bytes = p.adj_ws_bytes;
  return CT_OK;
}

ct_status ct_proj3d_fwd(const ct_geom3d* g, const float* vol, float* proj, int32_t batch,
                        void* workspace, size_t workspace_bytes, ct_stream_t stream) {
  using namespace ct;
  ct_status st = proj3d_check(g, "ct_proj3d_fwd");
  if (st != CT_OK) return st;
  if (!vol || !proj) return fail(CT_ERR_INVALID_ARG, "ct_proj3d_fwd: null array");
  if (batch <= 0) return fail(CT_ERR_INVALID_ARG, "ct_proj3d_fwd: batch=%d", batch);
  const Proj3dPlan p = proj3d_plan(g, batch);
  st = need_ws("ct_proj3d_fwd", p.fwd_bytes, workspace, workspace_bytes);
  if (st != CT_OK) return st;
  st = proj3d_prepare(g, p);
  if (st != CT_OK) return st;
  const size_t vol_n = (size_t)g->shape[0] * g->shape[1] * g->shape[2];
  const size_t proj_n = (size_t)g->n_views * g->det_shape[0] * g->det_shape[1];
  for (int b = 0; b < batch; ++b) {
    st = proj3d_fwd_launch(g, p, vol + b * vol_n, proj + b * proj_n, workspace, as_stream(stream),
                           nullptr);
    if (st != CT_OK) return st;
  }
  return CT_OK;
}

ct_status ct_proj3d_adj(const ct_geom3d* g, const float* proj, float* vol, int32_t batch,
                        void* workspace, size_t workspace_bytes, ct_stream_t stream) {
  using namespace ct;
  ct_status st = proj3d_check(g, "ct_proj3d_adj");
  if (st != CT_OK) return st;
  if (!vol || !proj) return fail(CT_ERR_INVALID_ARG, "ct_proj3d_adj: null array");
  if (batch <= 0) return fail(CT_ERR_INVALID_ARG, "ct_proj3d_adj: batch=%d", batch);
  const Proj3dPlan p = proj3d_plan(g, batch);
  st = need_ws("ct_proj3d_adj", p.adj_bytes, workspace, workspace_bytes);
  if (st != CT_OK) return st;
  st = proj3d_prepare(g, p);
  if (st != CT_OK) return st;
  cudaStream_t s = as_stream(stream);
  const size_t vol_n = (size_t)g->shape[0] * g->shape[1] * g->shape[2];
  const size_t proj_n = (size_t)g->n_views * g->det_shape[0] * g->det_shape[1];
  float* part = static_cast<float*>(workspace);
  for (int b = 0; b < batch; ++b) {
    st = proj3d_adj_launch(g, p, proj + b * proj_n, vol + b * vol_n, part, s, nullptr);
    if (st != CT_OK) return st;
    if (p.nsplit > 1) {
      const int blocks = (int)std::min<size_t>((vol_n + 255) / 256, 4096);
      k_p3_sum_splits<<<blocks, 256, 0, s>>>(part, vol + b * vol_n, vol_n, p.nsplit, vol_n);
      st = launch_check("k_p3_sum_splits");
      if (st != CT_OK) return st;
    }
  }
  return CT_OK;
}

ct_status ct_proj3d_autotune(const ct_geom3d* g, float* vol, float* proj, void* workspace,
                             size_t workspace_bytes, int32_t reps, ct_stream_t stream,
                             ct_proj3d_schedule* chosen) {
  using namespace ct;
  const char* who = "ct_proj3d_autotune";
  ct_status st = proj3d_check(g, who);
  if (st != CT_OK) return st;
  if (!vol || !proj) return fail(CT_ERR_INVALID_ARG, "%s: null array", who);
  if (reps <= 0) return fail(CT_ERR_INVALID_ARG, "%s: reps=%d", who, reps);
  cudaStream_t s = as_stream(stream);
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  st = cuda_check(cudaStreamIsCapturing(s, &cap), "stream capture query");
  if (st != CT_OK) return st;
  if (cap != cudaStreamCaptureStatusNone) return fail(CT_ERR_INVALID_ARG, "%s: cannot measure inside a stream capture", who);
  const Proj3dPlan p0 = proj3d_plan_sched(g, Sched3d{});
  const size_t need = std::max(p0.fwd_ws_bytes, p0.adj_ws_bytes);
  st = need_ws(who, need, workspace, workspace_bytes);
  if (st != CT_OK) return st;
  st = proj3d_prepare(g, p0);
  if (st != CT_OK) return st;
  const size_t vol_n = (size_t)g->shape[0] * g->shape[1] * g->shape[2];
  float* part = static_cast<float*>(workspace);

  auto timed = [&](auto&& fn, float& us) {
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    ct_status r = cuda_check(cudaEventCreate(&e0), "autotune event");
    if (r == CT_OK) r = cuda_check(cudaEventCreate(&e1), "autotune event");
    if (r == CT_OK) r = fn();
    if (r == CT_OK) r = cuda_check(cudaEventRecord(e0, s), "autotune event record");
    for (int k = 0; k < reps && r == CT_OK; ++k) r = fn();
    if (r == CT_OK) r = cuda_check(cudaEventRecord(e1, s), "autotune event record");
    if (r == CT_OK) r = cuda_check(cudaEventSynchronize(e1), "autotune event sync");
    float ms = 0.0f;
    if (r == CT_OK) r = cuda_check(cudaEventElapsedTime(&ms, e0, e1), "autotune elapsed time");
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    us = 1000.0f * ms / (float)reps;
    return r;
  };

  // Ties (within kTie of the fastest) go to the smaller count: both counts set
  // a summation order, so the choice should not flip between runs on noise.
  constexpr float kTie = 1.03f;
  auto pick = [&](const std::vector<std::pair<int, float>>& cand, int& val, float& us) {
    float fastest = cand.front().second;
    for (const auto& c : cand) fastest = std::min(fastest, c.second);
    for (const auto& c : cand)
      if (c.second <= kTie * fastest) {
        val = c.first;
        us = c.second;
        return;
      }
  };
  Sched3d best;
  float best_f = 0.0f, best_a = 0.0f;
  if (g->kind == CT_PROJ3D_AXIS0) {
    std::vector<std::pair<int, float>> cand;
    for (int G = 1; G <= std::min(kMaxGroups, p0.n_tiles); ++G) {
      const Proj3dPlan p = proj3d_plan_sched(g, Sched3d{G, 0});
      float us = 0.0f;
      st = timed([&] { return proj3d_fwd_launch(g, p, vol, proj, workspace, s, nullptr); }, us);
      if (st != CT_OK) return st;
      cand.emplace_back(p.G, us);
    }
    pick(cand, best.G, best_f);
  }
  {
    std::vector<std::pair<int, float>> cand;
    int last = 0;
    for (int ns = 1; ns <= kMaxSplits3d; ns *= 2) {
      const Proj3dPlan p = proj3d_plan_sched(g, Sched3d{0, ns});
      if (p.nsplit == last) continue;
      last = p.nsplit;
      float us = 0.0f;
      st = timed(
          [&] {
            ct_status r = proj3d_adj_launch(g, p, proj, vol, part, s, nullptr);
            if (r != CT_OK || p.nsplit == 1) return r;
            const int blocks = (int)std::min<size_t>((vol_n + 255) / 256, 4096);
            k_p3_sum_splits<<<blocks, 256, 0, s>>>(part, vol, vol_n, p.nsplit, vol_n);
            return launch_check("k_p3_sum_splits");
          },
          us);
      if (st != CT_OK) return st;
      cand.emplace_back(p.nsplit, us);
    }
    pick(cand, best.ns, best_a);
  }
  {
    std::lock_guard<std::mutex> lk(g_sched3_mu);
    g_sched3[sched3_key(g)] = Sched3dVal{best, best_f, best_a};
  }
  if (chosen) {
    const Proj3dPlan p = proj3d_plan_sched(g, best);
    chosen->tile_groups = g->kind == CT_PROJ3D_AXIS0 ? p.G : 0;
    chosen->adj_splits = p.nsplit;
    chosen->fwd_us = best_f;
    chosen->adj_us = best_a;
    chosen->tuned = 1;
  }
  return CT_OK;
}

ct_status ct_proj3d_schedule_get(const ct_geom3d* g, ct_proj3d_schedule* out) {
  using namespace ct;
  ct_status st = proj3d_check(g, "ct_proj3d_schedule_get");
  if (st != CT_OK) return st;
  if (!out) return fail(CT_ERR_INVALID_ARG, "ct_proj3d_schedule_get: null output");
  Sched3dVal v{};
  const bool tuned = sched3_lookup(g, v);
  const Proj3dPlan p = proj3d_plan_sched(g, tuned ? v.s : Sched3d{});
  out->tile_groups = g->kind == CT_PROJ3D_AXIS0 ? p.G : 0;
  out->adj_splits = p.nsplit;
  out->fwd_us = tuned ? v.fwd_us : 0.0f;
  out->adj_us = tuned ? v.adj_us : 0.0f;
  out->tuned = tuned ? 1 : 0;
  return CT_OK;
}

void ct_proj3d_schedule_clear(void) {
  std::lock_guard<std::mutex> lk(ct::g_sched3_mu);
  ct::g_sched3.clear();
}

// Diagnostic: returns (and clears) the 3D projector's internal check word.
int ct_proj3d_errflag(void) {
  int v = 0;
  if (cudaMemcpyFromSymbol(&v, ct::g_proj3d_err, sizeof(int)) != cudaSuccess) return -1;
  if (v != 0) {  // clear only a set word (no copy on the common path)
    const int zero = 0;
    cudaMemcpyToSymbol(ct::g_proj3d_err, &zero, sizeof(int));
  }
  return v;
}

}  // extern "C"
