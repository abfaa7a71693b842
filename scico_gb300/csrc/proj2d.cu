// 2D parallel-beam projector (scico XRayTransform2D) for sm_103a.
//
// Model (scico/linop/xray/_xray2d.py:308-351): pixel (i, j) projects for
// view v to Px = (Pxmin + Pdx0 i) + Pdx1 j; with k = floor(Px) and
// w = min(1 - (Px - k), width)/width it adds w*x to bin k and (1-w)*x to bin
// k+1 (bins outside [0, det) dropped).
//
// Forward (A), tile-owned pixel-driven sweep, two kernels:
//   k_proj2d_fwd_strips  A CTA owns a strip of 32 image rows x 256 columns,
//     loaded once as eight 32x32 tensor-map boxes (TMA, 128-B swizzle, zero
//     fill outside the image), and a run of views.  For each view the 8
//     warps take the strip's 8 tiles; lane r holds tile row r in registers
//     and walks its 32 pixels in the direction in which k never decreases,
//     carrying the running sums of the current bin and the next in registers
//     and storing finished bins in its shared-memory partial row.  The 32 partial rows are summed in row
//     order into the tile's bins; the warps need no barrier until every view
//     of the run is done, then the 8 tiles are summed in tile order into the
//     strip's bins of each view.
//   k_proj2d_fwd_gather  sums, per detector bin, the strips that cover it in
//     strip order.
//   No atomics: the result is bit-reproducible.
// Adjoint (A^T), k_proj2d_adj: pixel-driven gather with the same weights.  A
//   CTA owns a 64x64 pixel tile; per run of 32 views it stages the tile's
//   detector windows in shared memory as (y[k], y[k+1]) pairs (zero outside
//   the detector), then each thread accumulates its 4 x 4 pixels over the
//   views in view order.  Small images split the views into a fixed number
//   of runs whose partial images are summed in run order.
//
// floor(Px) is taken with one round-down float add of 1.5*2^23 (exact for
// |Px| < 2^22, checked per tile and view, with a floorf path otherwise):
// full-rate FP32 operations instead of conversion instructions.
#include <algorithm>
#include <atomic>
#include <cstring>
#include <map>
#include <tuple>
#include <vector>
#include <mutex>

#include <cuda.h>  // CUtensorMap and the tensor-map encoder's types

#include "common.cuh"
#include "tma.cuh"

namespace {

constexpr int kT = 32;          // forward tile edge: rows = lanes, columns = registers
constexpr int kCW = 256;        // forward strip width (8 tiles)
constexpr int kFW = 8;          // warps of a forward CTA (one tile each)
constexpr int kFwdTargetCtas = 1824;
constexpr int kLSDefault = 47;  // partial-row stride when projected pixels are at most one bin wide
constexpr int kGL = 16;         // strips read per round by a forward gather warp
constexpr int kAI = 64;         // adjoint tile rows
constexpr int kAJ = 64;         // adjoint tile columns
constexpr int kAPX = 4;         // columns per adjoint thread
constexpr int kAR = 4;          // rows per adjoint thread
constexpr int kAdjThreads = 256;  // adjoint CTA: 64 x 64 pixels = kAdjThreads x kAR x kAPX
constexpr int kAVC = 32;        // views staged per adjoint run
constexpr int kAdjTargetCtas = 1216;  // 152 SMs x 8: view splits until the CTAs balance over the SMs
constexpr int kAdjMinViewsPerSplit = 16;
constexpr uint32_t kMaxPolls = 1u << 24;
// Poll limit of the forward's strip-copy wait, read when a call launches
// (ct_set_wait_poll_limit); a solver graph keeps the value it was captured
// with.
std::atomic<uint32_t> g_wait_polls{kMaxPolls};

constexpr float kMagic = 12582912.0f;  // 1.5 * 2^23
constexpr int kMagicBits = 0x4B400000;
constexpr float kFastLimit = 2097152.0f;  // 2^21

struct ViewParams {
  float pxmin, pd0, pd1, width, inv_width;
};

__device__ __forceinline__ ViewParams load_view(const float* __restrict__ views, int v) {
  const float4 a = __ldg(reinterpret_cast<const float4*>(views) + 2 * v);
  const float4 b = __ldg(reinterpret_cast<const float4*>(views) + 2 * v + 1);
  return ViewParams{a.x, a.y, a.z, a.w, b.x};
}

// Extreme Px over the pixel rectangle [i0, i1] x [j0, j1]: px2d is
// non-decreasing in i where Pdx0 >= 0 and non-increasing where Pdx0 < 0 (each
// operation is a monotone rounding), and likewise in j, so the extremes are
// at the two corners the signs select.
__device__ __forceinline__ void rect_px(const ViewParams& p, int i0, int i1, int j0, int j1, float& lo,
                                        float& hi) {
  const bool ui = p.pd0 >= 0.0f, uj = p.pd1 >= 0.0f;
  lo = ct::px2d(p.pxmin, p.pd0, p.pd1, ui ? i0 : i1, uj ? j0 : j1);
  hi = ct::px2d(p.pxmin, p.pd0, p.pd1, ui ? i1 : i0, uj ? j1 : j0);
}

// key = floor(px) - kbias and w = min(1 - (px - floor(px)), width) * inv_width
// (the general path, used where |Px| may reach 2^21).
__device__ __forceinline__ void weight_floor(float px, float width, float inv_width, int kbias, int& key,
                                             float& w) {
  const float fl = floorf(px);
  key = (int)fl - kbias;
  const float dist = ct::fsub(1.0f, ct::fsub(px, fl));
  w = ct::fmul(fminf(dist, width), inv_width);
}

__device__ __forceinline__ void st_shared(uint32_t addr, float v) {
  asm volatile("st.shared.f32 [%0], %1;" ::"r"(addr), "f"(v) : "memory");
}

// Reads a shared float and leaves 0 in its place (one instruction).
__device__ __forceinline__ float xchg_zero_shared(uint32_t addr) {
  uint32_t r;
  asm volatile("atom.shared.exch.b32 %0, [%1], 0;" : "=r"(r) : "r"(addr) : "memory");
  return __uint_as_float(r);
}

__device__ __forceinline__ float2 ld_shared2(uint32_t addr) {
  float2 r;
  asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(r.x), "=f"(r.y) : "r"(addr) : "memory");
  return r;
}

// Paired float32 arithmetic (sm_100+ f32x2): each element is rounded exactly
// as the scalar operation of the same name.  A paired multiply feeding a
// paired add is contracted into one fused multiply-add by the assembler even
// with explicit rounding modifiers (measured: identical to fma.rn.f32x2), so
// products that must be rounded on their own stay scalar (__fmul_rn).
__device__ __forceinline__ unsigned long long pk2(float lo, float hi) {
  unsigned long long r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
  return r;
}
__device__ __forceinline__ void upk2(unsigned long long v, float& lo, float& hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ unsigned long long fadd2(unsigned long long a, unsigned long long b) {
  unsigned long long r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ unsigned long long fadd2_rd(unsigned long long a, unsigned long long b) {
  unsigned long long r;
  asm("add.rm.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ unsigned long long fsub2(unsigned long long a, unsigned long long b) {
  unsigned long long r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}

// ---------------------------------------------------------------------------
// Forward
// ---------------------------------------------------------------------------

// Walk one tile row for one view.  REV walks j downwards (Pdx1 < 0) so that
// the bin key never decreases.  Bin b receives, in walk order, the (1-w) x of
// the pixels with key b-1 followed by the w x of the pixels with key b.
//
// Fast floor for |px| < 2^22: t = magic + floor(px) exactly (one round-down
// add), dist = (floor(px) + 1) - px and w = sat(dist * inv_width), which is
// min(1 - (px - floor(px)), width) / width up to one rounding of the product
// (dist is the reference's 1 - (px - floor(px)) exactly for px >= 0; below
// the detector's first bin it may differ by one rounding).
//
// walk_row_fast: |Pdx1| < 0.999 and |Px| < 2^21, so consecutive keys differ
// by 0 or 1.  The Px, floor, distance and 1 - w steps of two consecutive
// pixels run as paired instructions (each element rounded as the scalar
// step), then the two pixels enter the carry in
// walk order: when the key advances, the current bin's sum is complete and
// the next bin's (1-w) x sum becomes the current one.  The floor uses the
// lane's own magic number kMagic + lane LS (an integer below 2^24, so
// t = magic + floor(px) is still exact), which makes the float bits of t the
// lane's partial-row index plus a constant: the store address is
// row_addr + 4 bits(t) with row_addr = warp_rows_addr - 4 (kMagicBits + base),
// the same for every lane of the warp.  pj[j] = Pdx1 * (j0 + j), the
// rounded column products of the warp's tile (a per-warp shared table, read
// by broadcast 16-byte loads).
template <bool REV>
__device__ __forceinline__ void walk_row_fast(const float (&xr)[kT], uint32_t row_addr, float magic,
                                              const float* __restrict__ pj, float R, float inv_width) {
  const unsigned long long R2 = pk2(R, R);
  const unsigned long long M2 = pk2(magic, magic), M12 = pk2(magic - 1.0f, magic - 1.0f);
  const unsigned long long one2 = pk2(1.0f, 1.0f);
  float A = 0.0f, B = 0.0f;
  int tbp = 0;
  auto step = [&](int tb, float w, float omw, float x, bool first) {
    if (first) tbp = tb;
    const bool next = tb != tbp;  // the key advanced by one bin: bin tbp is complete
    if (next) st_shared(row_addr + 4u * (uint32_t)tbp, A);
    const float a0 = next ? B : A;
    const float b0 = next ? 0.0f : B;
    A = fmaf(w, x, a0);
    B = fmaf(omw, x, b0);
    tbp = tb;
  };
  // Columns (2h, 2h+1) are evaluated as one pair (lower column in the low
  // half); REV steps the pair's upper column first.
#pragma unroll
  for (int q = 0; q < kT / 4; ++q) {
    const int qq = REV ? kT / 4 - 1 - q : q;
    const float4 p4 = *reinterpret_cast<const float4*>(pj + 4 * qq);
#pragma unroll
    for (int hh = 0; hh < 2; ++hh) {
      const int h = REV ? 1 - hh : hh;
      const int jl = 4 * qq + 2 * h;
      const unsigned long long px2 = fadd2(R2, h ? pk2(p4.z, p4.w) : pk2(p4.x, p4.y));
      const unsigned long long t2 = fadd2_rd(px2, M2);
      const unsigned long long d2 = fsub2(fsub2(t2, M12), px2);
      float tl, th, dl, dh;
      upk2(t2, tl, th);
      upk2(d2, dl, dh);
      const float wl = __saturatef(ct::fmul(dl, inv_width)), wh = __saturatef(ct::fmul(dh, inv_width));
      float ol, oh;
      upk2(fsub2(one2, pk2(wl, wh)), ol, oh);
      const bool first = q == 0 && hh == 0;
      if (!REV) {
        step(__float_as_int(tl), wl, ol, xr[jl], first);
        step(__float_as_int(th), wh, oh, xr[jl + 1], false);
      } else {
        step(__float_as_int(th), wh, oh, xr[jl + 1], first);
        step(__float_as_int(tl), wl, ol, xr[jl], false);
      }
    }
  }
  st_shared(row_addr + 4u * (uint32_t)tbp, A);
  st_shared(row_addr + 4u * (uint32_t)tbp + 4u, B);
}

// General walk (any step, floorf when |Px| may be large): bins skipped when
// the key advances by 2 or more keep their zero.
template <bool REV>
__device__ __forceinline__ void walk_row_gen(const float (&xr)[kT], float* __restrict__ mp, const ViewParams& p,
                                             float R, float fj0, int base) {
  int cur = 0;
  float A = 0.0f, B = 0.0f;
#pragma unroll
  for (int t = 0; t < kT; ++t) {
    const int jj = REV ? kT - 1 - t : t;
    const float px = ct::fadd(R, ct::fmul(p.pd1, fj0 + (float)jj));
    int key;
    float w;
    weight_floor(px, p.width, p.inv_width, base, key, w);
    const float omw = ct::fsub(1.0f, w);
    if (t == 0) cur = key;
    const int d = key - cur;
    if (d >= 2) mp[cur + 1] = B;
    const float a0 = d == 0 ? A : (d == 1 ? B : 0.0f);
    const float b0 = d == 0 ? B : 0.0f;
    A = fmaf(w, xr[jj], a0);
    B = fmaf(omw, xr[jj], b0);
    cur = key;
    mp[cur] = A;
  }
  mp[cur + 1] = B;
}

struct FwdArgs {
  const float* img;
  float* part;          // [batch][strip][view][cspan]
  const float* views;
  int rows, cols, nv;
  int L, LS, cspan;
  int n_chunks, vpc;
  int tensor;           // 1 = strip tiles by tensor-map loads (the kernel's map parameter)
  uint32_t max_polls;   // poll limit of the strip-copy wait
  int* errflag;
  const double* skip;
};

// Strip bins of one view: base = floor(min Px) and span = the bins the strip
// can touch, floor(max Px) - base + 2 (both kernels use this).
__device__ __forceinline__ void strip_bins(const ViewParams& p, int i0, int c0, int& base, int& span) {
  float lo, hi;
  rect_px(p, i0, i0 + kT - 1, c0, c0 + kCW - 1, lo, hi);
  base = (int)floorf(lo);
  span = (int)floorf(hi) - base + 2;
}

// Shared memory of k_proj2d_fwd_strips, from the first 1024-B boundary of the
// dynamic allocation: one region used twice, first the strip as kFW 32x32
// tiles (4 KB each, 128-B swizzled: the 16-B chunk q of tile row r sits at
// chunk q ^ (r & 7) of the row's 128 bytes), then, once every lane holds its
// tile row in registers, the partial rows [kFW][32][LS]; then the tiles' bins
// of every view of the CTA's run [kMaxVpc][kFW][L]; then the per-view
// parameters of the run (FwdViewSmem); then the copy barrier.
__host__ __device__ constexpr size_t fwd_region_floats(int LS) {
  return (size_t)kFW * kT * kT > (size_t)kFW * kT * LS ? (size_t)kFW * kT * kT : (size_t)kFW * kT * LS;
}
// Float offset of element (r, c) of a 32x32 tile in the swizzled layout.
__host__ __device__ constexpr int swz(int r, int c) { return r * kT + ((((c >> 2) ^ (r & 7)) << 2) | (c & 3)); }
constexpr int kMaxVpc = 16;  // views per forward CTA (upper bound of the plan's vpc)
__host__ __device__ constexpr size_t fwd_tbins_floats(int L) { return (size_t)kMaxVpc * kFW * L; }
struct FwdViewSmem {
  float4 pv[kMaxVpc];          // pxmin, Pdx0, Pdx1, 1/width
  float width[kMaxVpc];
  int2 strip[kMaxVpc];         // strip base bin, strip span
  int4 tile[kMaxVpc][kFW];     // per tile: base bin, span (0 = nothing to do), strip offset, fast floor
  float pj[kFW][kT];           // per warp: Pdx1 * j over its tile's columns for the current view
};

// Per-view parameters of a forward CTA's run of views, one lane per (view,
// tile): the view's table entry, the strip's bins and each tile's base bin,
// span, offset in the strip and floor path (every lane of a warp would
// otherwise compute the same values for its tile).  A span that does not fit
// the partial rows or the strip's bins (impossible for a table from
// ct_proj2d_views) sets bit 0 of the error word and skips the tile.
__device__ __forceinline__ void fwd_view_params(const FwdArgs& a, FwdViewSmem* vs, int i0, int c0, int ch) {
  const int vbeg = blockIdx.y * a.vpc;
  const int nvw = min(a.nv, vbeg + a.vpc) - vbeg;
  const int t = threadIdx.x;
  if (t >= nvw * kFW) return;
  const int vi = t / kFW, w = t - vi * kFW;
  const ViewParams p = load_view(a.views, vbeg + vi);
  int cb, ssp;
  strip_bins(p, i0, c0, cb, ssp);
  int base = 0, span = 0, off = 0, fast = 0;
  const int j0 = (ch * (kCW / kT) + w) * kT;
  if (j0 < a.cols && i0 < a.rows) {
    float lo, hi;
    rect_px(p, i0, i0 + kT - 1, j0, j0 + kT - 1, lo, hi);
    base = (int)floorf(lo);
    span = (int)floorf(hi) - base + 2;
    off = base - cb;
    fast = (fmaxf(fabsf(lo), fabsf(hi)) < kFastLimit && fabsf(p.pd1) < 0.999f) ? 1 : 0;
    if (span > a.L || off < 0 || off + span > a.cspan) {
      atomicOr(a.errflag, 1);
      span = 0;
    }
  }
  vs->tile[vi][w] = make_int4(base, span, off, fast);
  if (w == 0) {
    vs->pv[vi] = make_float4(p.pxmin, p.pd0, p.pd1, p.inv_width);
    vs->width[vi] = p.width;
    vs->strip[vi] = make_int2(cb, ssp);
  }
}

// grid = (n_strips, view groups, batch), block = 256.  LSC: the partial-row
// stride as a compile-time constant (its default-geometry value, so the row
// sums address with immediates), or 0 for a.LS.
template <int LSC>
__global__ void __launch_bounds__(kFW * 32, 3)
    k_proj2d_fwd_strips(const FwdArgs a, const __grid_constant__ CUtensorMap tmap) {
  ct::grid_dep_wait();  // before any global access (dependent launch)
  ct::grid_dep_trigger();
  const int LS = LSC ? LSC : a.LS;
  if (a.skip && *a.skip != 0.0) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const uint32_t sbase = ct::smem_u32(smem_raw);
  float* tiles = reinterpret_cast<float*>(smem_raw + (((sbase + 1023u) & ~1023u) - sbase));  // [kFW][32][32]
  float* part = tiles;                                               // [kFW][32][LS]
  float* tbins = tiles + fwd_region_floats(LS);                      // [kMaxVpc][kFW][L]
  FwdViewSmem* vs = reinterpret_cast<FwdViewSmem*>(tbins + fwd_tbins_floats(a.L));
  uint64_t* bar = reinterpret_cast<uint64_t*>(vs + 1);

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int s = blockIdx.x;
  const int ti = s / a.n_chunks, ch = s - ti * a.n_chunks;
  const int i0 = ti * kT, c0 = ch * kCW;
  const int b = blockIdx.z;

  const int vbeg = blockIdx.y * a.vpc;
  const int vend = min(a.nv, vbeg + a.vpc);

  // ---- stage the strip's tiles (zero outside the image) ---------------------
  // Tiles that start right of the image are not loaded: their warps have
  // nothing to do (span 0 in every view).
  const int ntl = min(kFW, (a.cols - c0 + kT - 1) / kT);
  int timed_out = 0;
  if (a.tensor) {
    if (tid == 0) {
      ct::mbar_init(bar, 1);
      ct::fence_barrier_init();
    }
    __syncthreads();
    if (tid == 0) {
      ct::mbar_arrive_expect_tx(bar, (uint32_t)(ntl * kT * kT * 4));
      for (int w = 0; w < ntl; ++w) ct::tensor_g2s_3d(tiles + w * kT * kT, &tmap, c0 + w * kT, i0, b, bar);
    }
    fwd_view_params(a, vs, i0, c0, ch);
    if (!ct::mbar_wait_bounded(bar, 0, a.max_polls)) {
      timed_out = 1;
      if (tid == 0) atomicOr(a.errflag, 2);
      // the copies were issued: let them land (default limit) before the
      // CTA's shared memory is released
      ct::mbar_wait_bounded(bar, 0, kMaxPolls);
    }
  } else {
    // the same layout by plain loads (rows not 16-B strided or image not
    // 16-B aligned): consecutive threads read consecutive columns
    const float* im = a.img + (size_t)b * a.rows * a.cols;
    for (int e = tid; e < ntl * kT * kT; e += kFW * 32) {
      const int w = e >> 10, r = (e >> 5) & 31, c = e & 31;
      const int gi = i0 + r, gj = c0 + w * kT + c;
      tiles[w * kT * kT + swz(r, c)] = (gi < a.rows && gj < a.cols) ? __ldg(im + (size_t)gi * a.cols + gj) : 0.0f;
    }
    fwd_view_params(a, vs, i0, c0, ch);
  }
  if (__syncthreads_or(timed_out)) {
    // The strip is not known to be complete: skip the work and leave zeros
    // in this CTA's strip bins, so the gather reads defined values.
    for (int vi = warp; vi < vend - vbeg; vi += kFW) {
      float* po = a.part + (((size_t)b * gridDim.x + s) * a.nv + vbeg + vi) * a.cspan;
      const int n = min(vs->strip[vi].y, a.cspan);
      for (int k = lane; k < n; k += 32) po[k] = 0.0f;
    }
    return;
  }

  const int tj = ch * (kCW / kT) + warp;  // this warp's tile column
  const int j0 = tj * kT;
  const float fi = (float)(i0 + lane);
  const float fj0 = (float)j0;
  // this lane's tile row, kept in registers for all the CTA's views
  float xr[kT];
  {
    const float* row = tiles + warp * kT * kT + lane * kT;
#pragma unroll
    for (int q = 0; q < kT / 4; ++q) {
      const float4 f = *reinterpret_cast<const float4*>(row + ((q ^ (lane & 7)) << 2));
      xr[4 * q] = f.x;
      xr[4 * q + 1] = f.y;
      xr[4 * q + 2] = f.z;
      xr[4 * q + 3] = f.w;
    }
  }
  __syncthreads();  // the tiles are dead from here: their bytes become partial rows
  // From here to the combine every warp works alone on its tile: its partial
  // rows, its column products and its rows of the tile bins.
  float* wpart = part + warp * kT * LS;
  {
    float4* z4 = reinterpret_cast<float4*>(wpart);  // kT * LS floats per warp: whole float4s (kT = 32)
    for (int e = lane; e < kT * LS / 4; e += 32) z4[e] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  }
  __syncwarp();

  float* mp = wpart + lane * LS;
  const float magic = kMagic + (float)(lane * LS);  // exact: an integer below 2^24
  for (int v = vbeg; v < vend; ++v) {
    const int vi = v - vbeg;
    const int4 tp = vs->tile[vi][warp];
    const int span = tp.y;
    if (span == 0) continue;  // warp-uniform
    const float4 pv = vs->pv[vi];
    const int base = tp.x;
    const float R = ct::fadd(pv.x, ct::fmul(pv.y, fi));
    if (tp.w) {
      const uint32_t row_addr = ct::smem_u32(wpart) - 4u * (uint32_t)(kMagicBits + base);
      // the tile's column products, one lane per column (the previous
      // view's reads ended before the warp barrier that closed it)
      float* pj = vs->pj[warp];
      pj[lane] = ct::fmul(pv.z, fj0 + (float)lane);
      __syncwarp();
      if (pv.z >= 0.0f)
        walk_row_fast<false>(xr, row_addr, magic, pj, R, pv.w);
      else
        walk_row_fast<true>(xr, row_addr, magic, pj, R, pv.w);
    } else {
      const ViewParams p{pv.x, pv.y, pv.z, vs->width[vi], pv.w};
      if (p.pd1 >= 0.0f)
        walk_row_gen<false>(xr, mp, p, R, fj0, base);
      else
        walk_row_gen<true>(xr, mp, p, R, fj0, base);
    }
    __syncwarp();
    // The tile's bins for this view: lane = bin, rows summed in row order;
    // each entry is read and zeroed by one shared exchange.
    float* tb = tbins + ((size_t)vi * kFW + warp) * a.L;
    if (lane < span) {
      float acc = 0.0f;
      const uint32_t q = ct::smem_u32(wpart + lane);
#pragma unroll
      for (int r = 0; r < kT; ++r) acc += xchg_zero_shared(q + 4u * (uint32_t)(r * LS));
      tb[lane] = acc;
    }
    if (span > 32) {
      if (span <= 35) {
        // at most 3 more bins: lane = row, then a fixed butterfly over rows
        const uint32_t q = ct::smem_u32(mp + 32);
#pragma unroll
        for (int e = 0; e < 3; ++e) {
          if (32 + e < span) {  // warp-uniform
            float t = xchg_zero_shared(q + 4u * (uint32_t)e);
#pragma unroll
            for (int d = 16; d > 0; d >>= 1) t += __shfl_xor_sync(0xffffffffu, t, d);
            if (lane == 0) tb[32 + e] = t;
          }
        }
      } else {
        for (int k = 32 + lane; k < span; k += 32) {
          float acc = 0.0f;
          const uint32_t q = ct::smem_u32(wpart + k);
#pragma unroll 8
          for (int r = 0; r < kT; ++r) acc += xchg_zero_shared(q + 4u * (uint32_t)(r * LS));
          tb[k] = acc;
        }
      }
    }
    __syncwarp();  // rows zeroed (lane = bin) before the next walk writes them (lane = row)
  }
  __syncthreads();
  // ---- combine the 8 tiles in tile order into the strip's bins, every view
  // of the run: warp w takes views w, w + 8 and adds the tiles' bins one
  // tile after the other into a row of the (now dead) partial-row region
  // (32 LS >= cspan floats per warp), lane = bin; bin k of the strip is
  // 0 + the covering tiles in tile order ------------------------------------
  float* acc = part + warp * kT * LS;
  for (int vi = warp; vi < vend - vbeg; vi += kFW) {
    const float* tb = tbins + (size_t)vi * kFW * a.L;
    float* po = a.part + (((size_t)b * gridDim.x + s) * a.nv + vbeg + vi) * a.cspan;
    const int n = min(vs->strip[vi].y, a.cspan);
    for (int k = lane; k < n; k += 32) acc[k] = 0.0f;
    __syncwarp();
#pragma unroll 1
    for (int w = 0; w < kFW; ++w) {
      const int4 tp = vs->tile[vi][w];  // base, span, offset in the strip, floor path
      for (int k = lane; k < tp.y; k += 32) acc[tp.z + k] += tb[w * a.L + k];
      __syncwarp();  // the next tile may add to the same bins
    }
    for (int k = lane; k < n; k += 32) po[k] = acc[k];
    __syncwarp();  // read before the next view zeroes the row
  }
}

// sino[b, v, bin] = sum over strips (strip order) of the strip bins covering
// bin.  A warp takes 64 consecutive bins of one view (lane: bins k0 + lane
// and k0 + 32 + lane): its lanes compute the strips' bin ranges (lane =
// strip), a ballot lists the strips that meet the warp's bins, and the
// listed strips are read kGL at a time (loads first, then the sums in strip
// order, zero where a strip misses the bin).
// grid = (n_views, ceil(det / 256), batch), block = 128.
__global__ void __launch_bounds__(128)
    k_proj2d_fwd_gather(const float* __restrict__ part, float* __restrict__ sino,
                        const float* __restrict__ views, int nv, int det, int cspan, int n_chunks,
                        int n_strips, const double* __restrict__ skip) {
  ct::grid_dep_wait();  // before any global access (dependent launch)
  ct::grid_dep_trigger();
  if (skip && *skip != 0.0) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int v = blockIdx.x, b = blockIdx.z;
  const int k0 = blockIdx.y * 256 + warp * 64;
  if (k0 >= det) return;  // whole warp
  const ViewParams p = load_view(views, v);
  const int bin0 = k0 + lane, bin1 = k0 + 32 + lane;
  const float* pb = part + ((size_t)b * n_strips * nv + v) * cspan;
  const size_t sstride = (size_t)nv * cspan;
  float acc0 = 0.0f, acc1 = 0.0f;
  for (int c = 0; c < n_strips; c += 32) {
    const int s = c + lane;
    int base = 0, span = 0;
    if (s < n_strips) {
      const int ti = s / n_chunks, ch = s - ti * n_chunks;
      strip_bins(p, ti * kT, ch * kCW, base, span);
      span = min(span, cspan);
    }
    unsigned mask = __ballot_sync(0xffffffffu, s < n_strips && base < k0 + 64 && base + span > k0);
    while (mask) {
      float v0[kGL], v1[kGL];
#pragma unroll
      for (int u = 0; u < kGL; ++u) {
        v0[u] = 0.0f;
        v1[u] = 0.0f;
        if (mask) {
          const int sl = __ffs(mask) - 1;
          mask &= mask - 1u;
          const int bs = __shfl_sync(0xffffffffu, base, sl);
          const int sp = __shfl_sync(0xffffffffu, span, sl);
          const float* q = pb + (size_t)(c + sl) * sstride;
          const int o0 = bin0 - bs, o1 = bin1 - bs;
          if ((unsigned)o0 < (unsigned)sp) v0[u] = __ldg(q + o0);
          if ((unsigned)o1 < (unsigned)sp) v1[u] = __ldg(q + o1);
        }
      }
#pragma unroll
      for (int u = 0; u < kGL; ++u) {
        acc0 += v0[u];
        acc1 += v1[u];
      }
    }
  }
  float* so = sino + ((size_t)b * nv + v) * det;
  if (bin0 < det) so[bin0] = acc0;
  if (bin1 < det) so[bin1] = acc1;
}

// ---------------------------------------------------------------------------
// Adjoint
// ---------------------------------------------------------------------------

struct AdjArgs {
  const float* sino;
  float* out;
  const float* views;
  int rows, cols, nv, det;
  int nsplit, per_split;
  size_t split_stride;
  int W;  // window length (bins) per staged view
  int* errflag;
  const double* skip;
};

// One view's contribution to this thread's pixels.  Fast path: the window
// pair of key k lives at shared address off + 8 (kMagicBits + k) for the
// float bits kMagicBits + k of kMagic + k.

// adj_view_fast with the Px, floor, distance and 1 - w steps of two pixels
// per paired instruction (bit-identical to the scalar form); the column
// products Pdx1 * j are shared by the thread's rows.
__device__ __forceinline__ void adj_view_fast2(const float4 pv, uint32_t off, const float (&fi)[kAR],
                                               const float (&fj)[kAPX], float (&acc)[kAR][kAPX]) {
  const unsigned long long M2 = pk2(kMagic, kMagic), M12 = pk2(kMagic - 1.0f, kMagic - 1.0f);
  const unsigned long long one2 = pk2(1.0f, 1.0f);
  float pj[kAPX];
#pragma unroll
  for (int q = 0; q < kAPX; ++q) pj[q] = ct::fmul(pv.z, fj[q]);
#pragma unroll
  for (int r = 0; r < kAR; ++r) {
    const float R = ct::fadd(pv.x, ct::fmul(pv.y, fi[r]));
    const unsigned long long R2 = pk2(R, R);
#pragma unroll
    for (int h = 0; h < kAPX / 2; ++h) {
      const unsigned long long px2 = fadd2(R2, pk2(pj[2 * h], pj[2 * h + 1]));
      const unsigned long long t2 = fadd2_rd(px2, M2);
      const unsigned long long d2 = fsub2(fsub2(t2, M12), px2);
      float t0, t1, d0, d1;
      upk2(t2, t0, t1);
      upk2(d2, d0, d1);
      const float w0 = __saturatef(ct::fmul(d0, pv.w)), w1 = __saturatef(ct::fmul(d1, pv.w));
      float o0, o1;
      upk2(fsub2(one2, pk2(w0, w1)), o0, o1);
      const float2 y0 = ld_shared2(off + 8u * (uint32_t)__float_as_int(t0));
      const float2 y1 = ld_shared2(off + 8u * (uint32_t)__float_as_int(t1));
      acc[r][2 * h] = fmaf(y0.x, w0, acc[r][2 * h]);
      acc[r][2 * h] = fmaf(y0.y, o0, acc[r][2 * h]);
      acc[r][2 * h + 1] = fmaf(y1.x, w1, acc[r][2 * h + 1]);
      acc[r][2 * h + 1] = fmaf(y1.y, o1, acc[r][2 * h + 1]);
    }
  }
}

__device__ __forceinline__ void adj_view_gen(const float4 pv, float width, int base, const float2* __restrict__ wy,
                                             const float (&fi)[kAR], const float (&fj)[kAPX],
                                             float (&acc)[kAR][kAPX]) {
#pragma unroll
  for (int r = 0; r < kAR; ++r) {
    const float R = ct::fadd(pv.x, ct::fmul(pv.y, fi[r]));
#pragma unroll
    for (int q = 0; q < kAPX; ++q) {
      const float px = ct::fadd(R, ct::fmul(pv.z, fj[q]));
      int key;
      float w;
      weight_floor(px, width, pv.w, base, key, w);
      const float2 y = wy[key];
      acc[r][q] = fmaf(y.x, w, acc[r][q]);
      acc[r][q] = fmaf(y.y, ct::fsub(1.0f, w), acc[r][q]);
    }
  }
}

// grid = (ceil(cols/64), ceil(rows/64), batch*nsplit), block = 256: thread
// (ty, tx) owns rows ty + 16 r (r < kAR) at columns tx + 16 q (q < kAPX) of
// the 64 x 64 tile.
__global__ void __launch_bounds__(kAdjThreads) k_proj2d_adj(const AdjArgs a) {
  ct::grid_dep_wait();  // before any global access (dependent launch)
  ct::grid_dep_trigger();
  if (a.skip && *a.skip != 0.0) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* sy = reinterpret_cast<float2*>(smem_raw);          // [kAVC][W]
  float4* sp = reinterpret_cast<float4*>(sy + kAVC * a.W);   // [kAVC] pxmin, pd0, pd1, 1/width
  float* sw = reinterpret_cast<float*>(sp + kAVC);           // [kAVC] width
  int* sb = reinterpret_cast<int*>(sw + kAVC);               // [kAVC] window base
  int* sf = sb + kAVC;                                       // [kAVC] 1 = fast floor, -1 = skip
  uint32_t* so = reinterpret_cast<uint32_t*>(sf + kAVC);     // [kAVC] fast-path address offset

  constexpr int kWarps = kAdjThreads / 32;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int z = blockIdx.z;
  const int b = z / a.nsplit, sidx = z - b * a.nsplit;
  const int vbeg = sidx * a.per_split, vend = min(a.nv, vbeg + a.per_split);
  const int i0 = blockIdx.y * kAI, j0 = blockIdx.x * kAJ;
  const int ty = tid >> 4, tx = tid & 15;
  float fi[kAR];
#pragma unroll
  for (int r = 0; r < kAR; ++r) fi[r] = (float)(i0 + ty + (kAI / kAR) * r);
  float fj[kAPX];
#pragma unroll
  for (int q = 0; q < kAPX; ++q) fj[q] = (float)(j0 + tx + 16 * q);
  float acc[kAR][kAPX];
#pragma unroll
  for (int r = 0; r < kAR; ++r)
#pragma unroll
    for (int q = 0; q < kAPX; ++q) acc[r][q] = 0.0f;
  const float* yb = a.sino + (size_t)b * a.nv * a.det;

  for (int a0 = vbeg; a0 < vend; a0 += kAVC) {
    const int n = min(kAVC, vend - a0);
    __syncthreads();
    if (tid < n) {
      const ViewParams p = load_view(a.views, a0 + tid);
      float lo, hi;
      rect_px(p, i0, i0 + kAI - 1, j0, j0 + kAJ - 1, lo, hi);
      const int base = (int)floorf(lo);
      const int span = (int)floorf(hi) - base + 2;
      sp[tid] = make_float4(p.pxmin, p.pd0, p.pd1, p.inv_width);
      sw[tid] = p.width;
      sb[tid] = base;
      int f = fmaxf(fabsf(lo), fabsf(hi)) < kFastLimit ? 1 : 0;
      if (span > a.W) {  // cannot happen for a table from ct_proj2d_views
        atomicOr(a.errflag, 4);
        f = -1;
      }
      sf[tid] = f;
      so[tid] = ct::smem_u32(sy + tid * a.W) - 8u * (uint32_t)(kMagicBits + base);
    }
    __syncthreads();
    for (int v = warp; v < n; v += kWarps) {
      const float* yr = yb + (size_t)(a0 + v) * a.det;
      const int base = sb[v];
      float2* wy = sy + v * a.W;
      for (int k = lane; k < a.W; k += 32) {
        const int bin = base + k;
        const float y0 = ((unsigned)bin < (unsigned)a.det) ? __ldg(yr + bin) : 0.0f;
        const float y1 = ((unsigned)(bin + 1) < (unsigned)a.det) ? __ldg(yr + bin + 1) : 0.0f;
        wy[k] = make_float2(y0, y1);
      }
    }
    __syncthreads();
    for (int v = 0; v < n; ++v) {
      const int f = sf[v];
      if (f == 1)
        adj_view_fast2(sp[v], so[v], fi, fj, acc);
      else if (f == 0)
        adj_view_gen(sp[v], sw[v], sb[v], sy + v * a.W, fi, fj, acc);
    }
  }
#pragma unroll
  for (int r = 0; r < kAR; ++r) {
    const int i = i0 + ty + (kAI / kAR) * r;
    if (i < a.rows) {
      float* o = a.out + (size_t)sidx * a.split_stride + (size_t)b * a.rows * a.cols + (size_t)i * a.cols;
#pragma unroll
      for (int q = 0; q < kAPX; ++q) {
        const int j = j0 + tx + 16 * q;
        if (j < a.cols) o[j] = acc[r][q];
      }
    }
  }
}

// out[e] = sum_s part[s*stride + e] in split order.
__global__ void k_sum_splits(const float* __restrict__ part, float* __restrict__ out, size_t n,
                             int nsplit, size_t stride) {
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n;
       e += (size_t)gridDim.x * blockDim.x) {
    float s = 0.0f;
    for (int k = 0; k < nsplit; ++k) s += part[(size_t)k * stride + e];
    out[e] = s;
  }
}

// Device error word of the library's device checks (bit 0: forward tile
// span, bit 1: strip copy wait, bit 2: adjoint window span, bit 3: a grid
// barrier wait of the solver's fast-forward kernel).
__device__ int g_proj2d_err = 0;

int* errflag_ptr() {
  static int* cached[64] = {nullptr};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  if (!cached[dev]) {
    int* p = nullptr;
    if (cudaGetSymbolAddress((void**)&p, g_proj2d_err) != cudaSuccess) return nullptr;
    cached[dev] = p;
  }
  return cached[dev];
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against the driver library); null where the driver does not provide it.
using TensorMapEncodeFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                       const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                       CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
TensorMapEncodeFn tensor_map_encoder() {
  static const TensorMapEncodeFn fn = []() -> TensorMapEncodeFn {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    return reinterpret_cast<TensorMapEncodeFn>(p);
  }();
  return fn;
}

// Tensor map of a float32 image batch [batch][rows][cols] read as 32x32 boxes
// with 128-B swizzle and zero fill outside the image.  Needs 16-B strided
// rows and a 16-B aligned base; false where the map cannot be made.
bool encode_image_map(CUtensorMap* m, const float* img, int rows, int cols, int batch) {
  if ((cols & 3) != 0 || !ct::aligned(img, 16)) return false;
  const TensorMapEncodeFn enc = tensor_map_encoder();
  if (!enc) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)cols, (cuuint64_t)rows, (cuuint64_t)batch};
  const cuuint64_t strides[2] = {(cuuint64_t)cols * 4u, (cuuint64_t)rows * cols * 4u};
  const cuuint32_t box[3] = {(cuuint32_t)kT, (cuuint32_t)kT, 1u};
  const cuuint32_t estr[3] = {1u, 1u, 1u};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(img), dims, strides, box, estr,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

size_t fwd_smem_bytes(int LS, int L) {
  // up to 1008 bytes to the first 1024-B boundary (the allocation starts
  // 16-B aligned), then the region, tile bins, view parameters and barrier
  return 1008 + sizeof(float) * (fwd_region_floats(LS) + fwd_tbins_floats(L)) + sizeof(FwdViewSmem) + 16;
}

size_t adj_smem_bytes(int W) {
  return sizeof(float2) * (size_t)kAVC * W + sizeof(float4) * kAVC + sizeof(float) * kAVC +
         3 * sizeof(int) * kAVC;
}

}  // namespace

#include "kernels.cuh"

namespace ct {

int* proj2d_errflag_ptr() { return errflag_ptr(); }

ct_status proj2d_check(const ct_geom2d* g, const char* who) {
  if (!g) return fail(CT_ERR_INVALID_ARG, "%s: null geometry", who);
  if (g->rows <= 0 || g->cols <= 0 || g->n_views <= 0 || g->det_count <= 0)
    return fail(CT_ERR_SHAPE, "%s: bad geometry rows=%d cols=%d views=%d det=%d", who, g->rows,
                g->cols, g->n_views, g->det_count);
  if (!g->views) return fail(CT_ERR_INVALID_ARG, "%s: null view table", who);
  if (!aligned(g->views, 16)) return fail(CT_ERR_INVALID_ARG, "%s: view table not 16-B aligned", who);
  if (!(g->max_width > 0.0f) || g->max_width > 16.0f)
    return fail(CT_ERR_UNSUPPORTED, "%s: max projected pixel width %g outside (0, 16]", who,
                (double)g->max_width);
  const Proj2dPlan p = proj2d_plan(g, 1);
  if (p.fwd_smem > 200 * 1024 || p.adj_smem > 200 * 1024)
    return fail(CT_ERR_UNSUPPORTED, "%s: tile spans of %d / %d bins too large", who, p.L, p.W);
  return CT_OK;
}

// Largest adjoint split count a schedule may use: up to twice the splits
// that fill the GPU, at least 16 views per split.
int max_splits(const ct_geom2d* g, long ctas) {
  int ns = ctas < 2L * kAdjTargetCtas ? (int)((2L * kAdjTargetCtas + ctas - 1) / ctas) : 1;
  return std::max(1, std::min(ns, std::max(1, g->n_views / kAdjMinViewsPerSplit)));
}

Proj2dPlan proj2d_plan_sched(const ct_geom2d* g, int batch, Sched2d sc) {
  Proj2dPlan p;
  const float mw = g->max_width * 1.0001f;
  // Keys inside an a x b pixel rectangle differ by at most
  // (a-1)|Pdx0| + (b-1)|Pdx1| <= max(a-1, b-1) * max_width (plus rounding),
  // and the rectangle needs the bins [base, top + 1].
  p.tiles_i = (g->rows + kT - 1) / kT;
  p.n_chunks = (g->cols + kCW - 1) / kCW;
  p.n_strips = p.tiles_i * p.n_chunks;
  p.L = (int)floorf((float)(kT - 1) * mw + 1.01f) + 3;
  // Row stride: the smallest value >= L that is 15 or 17 modulo 32.  Lane r
  // stores to bank (r LS + key_r) mod 32 with key_r ~ r Pdx0 + c, and these
  // strides spread the 32 lanes over the banks best (modelled over the views
  // of a 360-angle scan: 2.08 wavefronts per store against 2.38 for stride 35).
  p.LS = p.L;
  while ((p.LS & 31) != 15 && (p.LS & 31) != 17) ++p.LS;
  p.cspan = (int)floorf((float)(kCW - 1) * mw + 1.01f) + 3;
  const long work = (long)p.n_strips * g->n_views * batch;
  p.vpc = sc.vpc > 0 ? std::min(sc.vpc, kMaxVpc)
                     : (int)std::min<long>(kMaxVpc, std::max<long>(2, (work + kFwdTargetCtas - 1) / kFwdTargetCtas));
  p.fwd_groups = (g->n_views + p.vpc - 1) / p.vpc;
  p.fwd_bytes = round_up((size_t)batch * p.n_strips * g->n_views * p.cspan * sizeof(float), 256);
  p.fwd_smem = fwd_smem_bytes(p.LS, p.L);
  p.W = (int)floorf((float)(std::max(kAI, kAJ) - 1) * mw + 1.01f) + 3;
  p.adj_smem = adj_smem_bytes(p.W);
  p.adj_gx = (g->cols + kAJ - 1) / kAJ;
  p.adj_gy = (g->rows + kAI - 1) / kAI;
  const long ctas = (long)p.adj_gx * p.adj_gy * batch;
  const int ns_max = max_splits(g, ctas);
  int ns = 1;
  if (sc.ns > 0) {
    ns = std::min(sc.ns, ns_max);
  } else {
    if (ctas < kAdjTargetCtas) ns = (int)((kAdjTargetCtas + ctas - 1) / ctas);
    ns = std::min(ns, std::max(1, g->n_views / kAdjMinViewsPerSplit));
  }
  p.per_split = (g->n_views + ns - 1) / ns;
  p.nsplit = (g->n_views + p.per_split - 1) / p.per_split;
  const size_t img = (size_t)batch * g->rows * g->cols * sizeof(float);
  p.adj_bytes = p.nsplit > 1 ? round_up((size_t)p.nsplit * img, 256) : 0;
  const int ws_splits = std::max(p.nsplit, ns_max);
  p.adj_ws_bytes = ws_splits > 1 ? round_up((size_t)ws_splits * img, 256) : 0;
  return p;
}

// ---- recorded schedules ------------------------------------------------------
struct SchedKey {
  int rows, cols, nv, det, batch;
  uint32_t width_bits;
  bool operator<(const SchedKey& o) const {
    return std::tie(rows, cols, nv, det, batch, width_bits) <
           std::tie(o.rows, o.cols, o.nv, o.det, o.batch, o.width_bits);
  }
};
struct SchedVal {
  Sched2d s;
  float fwd_us, adj_us;
};
std::mutex g_sched_mu;
std::map<SchedKey, SchedVal> g_sched;

SchedKey sched_key(const ct_geom2d* g, int batch) {
  uint32_t wb;
  memcpy(&wb, &g->max_width, sizeof(wb));
  return SchedKey{g->rows, g->cols, g->n_views, g->det_count, batch, wb};
}

bool sched_lookup(const ct_geom2d* g, int batch, SchedVal& out) {
  std::lock_guard<std::mutex> lk(g_sched_mu);
  const auto it = g_sched.find(sched_key(g, batch));
  if (it == g_sched.end()) return false;
  out = it->second;
  return true;
}

uint32_t proj2d_wait_polls() { return g_wait_polls.load(std::memory_order_relaxed); }

ct_status proj2d_sum_splits(const float* part, float* out, size_t n, int nsplit, cudaStream_t s) {
  const int blocks = (int)std::min<size_t>((n + 255) / 256, 4096);
  k_sum_splits<<<blocks, 256, 0, s>>>(part, out, n, nsplit, n);
  return launch_check("k_sum_splits");
}

Proj2dPlan proj2d_plan(const ct_geom2d* g, int batch) {
  SchedVal v;
  return proj2d_plan_sched(g, batch, sched_lookup(g, batch, v) ? v.s : Sched2d{});
}

ct_status proj2d_prepare(const Proj2dPlan& p) {
  if (!errflag_ptr()) return fail(CT_ERR_CUDA, "proj2d: error-word address unavailable");
  ct_status st = cuda_check(cudaFuncSetAttribute(k_proj2d_fwd_strips<kLSDefault>,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 (int)p.fwd_smem),
                            "fwd smem attribute");
  if (st != CT_OK) return st;
  st = cuda_check(cudaFuncSetAttribute(k_proj2d_fwd_strips<0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)p.fwd_smem),
                  "fwd smem attribute");
  if (st != CT_OK) return st;
  return cuda_check(cudaFuncSetAttribute(k_proj2d_adj, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)p.adj_smem),
                    "adj smem attribute");
}

ct_status proj2d_fwd_launch(const ct_geom2d* g, const Proj2dPlan& p, const float* img, float* sino,
                            int batch, float* part, cudaStream_t s, const double* skip, bool dependent) {
  FwdArgs a;
  a.img = img;
  a.part = part;
  a.views = g->views;
  a.rows = g->rows;
  a.cols = g->cols;
  a.nv = g->n_views;
  a.L = p.L;
  a.LS = p.LS;
  a.cspan = p.cspan;
  a.n_chunks = p.n_chunks;
  a.vpc = p.vpc;
  CUtensorMap tmap;
  memset(&tmap, 0, sizeof(tmap));
  a.tensor = encode_image_map(&tmap, img, g->rows, g->cols, batch) ? 1 : 0;
  a.max_polls = g_wait_polls.load(std::memory_order_relaxed);
  a.errflag = errflag_ptr();
  a.skip = skip;
  if (!a.errflag) return fail(CT_ERR_CUDA, "proj2d: error-word address unavailable");
  dim3 g1(p.n_strips, p.fwd_groups, batch);
  auto strips = p.LS == kLSDefault ? k_proj2d_fwd_strips<kLSDefault> : k_proj2d_fwd_strips<0>;
  ct_status st = cuda_check(launch_k(strips, g1, dim3(kFW * 32), p.fwd_smem, s, dependent, a, tmap),
                            "k_proj2d_fwd_strips");
  if (st != CT_OK) return st;
  // the gather follows the strips kernel: a dependent launch
  dim3 g2(g->n_views, (g->det_count + 255) / 256, batch);
  return cuda_check(launch_k(k_proj2d_fwd_gather, g2, dim3(128), 0, s, true, (const float*)part, sino,
                             (const float*)g->views, (int)g->n_views, (int)g->det_count, p.cspan, p.n_chunks,
                             p.n_strips, skip),
                    "k_proj2d_fwd_gather");
}

ct_status proj2d_adj_launch(const ct_geom2d* g, const Proj2dPlan& p, const float* sino, float* out,
                            float* part, int batch, cudaStream_t s, const double* skip, bool dependent) {
  AdjArgs a;
  a.sino = sino;
  a.out = p.nsplit > 1 ? part : out;
  a.views = g->views;
  a.rows = g->rows;
  a.cols = g->cols;
  a.nv = g->n_views;
  a.det = g->det_count;
  a.nsplit = p.nsplit;
  a.per_split = p.per_split;
  a.split_stride = p.nsplit > 1 ? (size_t)batch * g->rows * g->cols : 0;
  a.W = p.W;
  a.errflag = errflag_ptr();
  a.skip = skip;
  if (!a.errflag) return fail(CT_ERR_CUDA, "proj2d: error-word address unavailable");
  dim3 grid(p.adj_gx, p.adj_gy, batch * p.nsplit);
  return cuda_check(launch_k(k_proj2d_adj, grid, dim3(kAdjThreads), p.adj_smem, s, dependent, a),
                    "k_proj2d_adj");
}

}  // namespace ct

extern "C" {

ct_status ct_proj2d_workspace(const ct_geom2d* g, int32_t batch, size_t* fwd_bytes,
                              size_t* adj_bytes) {
  ct_status st = ct::proj2d_check(g, "ct_proj2d_workspace");
  if (st != CT_OK) return st;
  if (batch <= 0) return ct::fail(CT_ERR_INVALID_ARG, "ct_proj2d_workspace: batch=%d", batch);
  const ct::Proj2dPlan p = ct::proj2d_plan(g, batch);
  if (fwd_bytes) *fwd_bytes = p.fwd_bytes;
  if (adj_bytes) *adj_bytes = p.adj_ws_bytes;  // fits any schedule the autotuner may record
  return CT_OK;
}

ct_status ct_proj2d_fwd(const ct_geom2d* g, const float* img, float* sino, int32_t batch,
                        void* workspace, size_t workspace_bytes, ct_stream_t stream) {
  ct_status st = ct::proj2d_check(g, "ct_proj2d_fwd");
  if (st != CT_OK) return st;
  if (!img || !sino) return ct::fail(CT_ERR_INVALID_ARG, "ct_proj2d_fwd: null array");
  if (batch <= 0) return ct::fail(CT_ERR_INVALID_ARG, "ct_proj2d_fwd: batch=%d", batch);
  const ct::Proj2dPlan p = ct::proj2d_plan(g, batch);
  if (!workspace || workspace_bytes < p.fwd_bytes || !ct::aligned(workspace, 256))
    return ct::fail(CT_ERR_WORKSPACE, "ct_proj2d_fwd: need %zu bytes (256-B aligned), got %zu",
                    p.fwd_bytes, workspace_bytes);
  st = ct::proj2d_prepare(p);
  if (st != CT_OK) return st;
  return ct::proj2d_fwd_launch(g, p, img, sino, batch, static_cast<float*>(workspace),
                               ct::as_stream(stream), nullptr);
}

ct_status ct_proj2d_adj(const ct_geom2d* g, const float* sino, float* img, int32_t batch,
                        void* workspace, size_t workspace_bytes, ct_stream_t stream) {
  ct_status st = ct::proj2d_check(g, "ct_proj2d_adj");
  if (st != CT_OK) return st;
  if (!img || !sino) return ct::fail(CT_ERR_INVALID_ARG, "ct_proj2d_adj: null array");
  if (batch <= 0) return ct::fail(CT_ERR_INVALID_ARG, "ct_proj2d_adj: batch=%d", batch);
  const ct::Proj2dPlan p = ct::proj2d_plan(g, batch);
  cudaStream_t s = ct::as_stream(stream);
  if (p.nsplit > 1) {
    if (!workspace || workspace_bytes < p.adj_bytes || !ct::aligned(workspace, 256))
      return ct::fail(CT_ERR_WORKSPACE, "ct_proj2d_adj: need %zu bytes (256-B aligned), got %zu",
                      p.adj_bytes, workspace_bytes);
  }
  st = ct::proj2d_prepare(p);
  if (st != CT_OK) return st;
  float* part = static_cast<float*>(workspace);
  st = ct::proj2d_adj_launch(g, p, sino, img, part, batch, s, nullptr);
  if (st != CT_OK || p.nsplit == 1) return st;
  const size_t n = (size_t)batch * g->rows * g->cols;
  const int blocks = (int)std::min<size_t>((n + 255) / 256, 4096);
  k_sum_splits<<<blocks, 256, 0, s>>>(part, img, n, p.nsplit, n);
  return ct::launch_check("k_sum_splits");
}

}  // extern "C"

// ---- autotuning ------------------------------------------------------------------
namespace {

// Device time of `reps` calls of fn (after one untimed call), per call, in µs.
template <class F>
ct_status time_calls(F&& fn, int reps, cudaStream_t s, float& us) {
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  ct_status st = ct::cuda_check(cudaEventCreate(&e0), "autotune event");
  if (st == CT_OK) st = ct::cuda_check(cudaEventCreate(&e1), "autotune event");
  if (st == CT_OK) st = fn();
  if (st == CT_OK) st = ct::cuda_check(cudaEventRecord(e0, s), "autotune event record");
  for (int r = 0; r < reps && st == CT_OK; ++r) st = fn();
  if (st == CT_OK) st = ct::cuda_check(cudaEventRecord(e1, s), "autotune event record");
  if (st == CT_OK) st = ct::cuda_check(cudaEventSynchronize(e1), "autotune event sync");
  float ms = 0.0f;
  if (st == CT_OK) st = ct::cuda_check(cudaEventElapsedTime(&ms, e0, e1), "autotune elapsed time");
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  us = 1000.0f * ms / (float)reps;
  return st;
}

}  // namespace

extern "C" {

ct_status ct_proj2d_autotune(const ct_geom2d* g, int32_t batch, float* img, float* sino, void* workspace,
                             size_t workspace_bytes, int32_t reps, ct_stream_t stream,
                             ct_proj2d_schedule* chosen) {
  const char* who = "ct_proj2d_autotune";
  ct_status st = ct::proj2d_check(g, who);
  if (st != CT_OK) return st;
  if (!img || !sino) return ct::fail(CT_ERR_INVALID_ARG, "%s: null array", who);
  if (batch <= 0 || reps <= 0) return ct::fail(CT_ERR_INVALID_ARG, "%s: batch=%d reps=%d", who, batch, reps);
  cudaStream_t s = ct::as_stream(stream);
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  st = ct::cuda_check(cudaStreamIsCapturing(s, &cap), "stream capture query");
  if (st != CT_OK) return st;
  if (cap != cudaStreamCaptureStatusNone)
    return ct::fail(CT_ERR_INVALID_ARG, "%s: cannot measure inside a stream capture", who);
  const ct::Proj2dPlan p0 = ct::proj2d_plan_sched(g, batch, ct::Sched2d{});
  const size_t need = std::max(p0.fwd_bytes, p0.adj_ws_bytes);
  if (!workspace || workspace_bytes < need || !ct::aligned(workspace, 256))
    return ct::fail(CT_ERR_WORKSPACE, "%s: need %zu bytes (256-B aligned), got %zu", who, need, workspace_bytes);
  st = ct::proj2d_prepare(p0);
  if (st != CT_OK) return st;
  float* ws = static_cast<float*>(workspace);

  // forward: views per CTA
  static const int kVpcCand[] = {2, 3, 4, 5, 6, 7, 8, 10, 12, 16};
  ct::Sched2d best;
  float best_f = 0.0f;
  for (int vpc : kVpcCand) {
    if (vpc > kMaxVpc) continue;
    const ct::Proj2dPlan p = ct::proj2d_plan_sched(g, batch, ct::Sched2d{vpc, 0});
    float us = 0.0f;
    st = time_calls([&] { return ct::proj2d_fwd_launch(g, p, img, sino, batch, ws, s, nullptr); }, reps, s, us);
    if (st != CT_OK) return st;
    if (best.vpc == 0 || us < best_f) {
      best.vpc = p.vpc;
      best_f = us;
    }
  }
  // adjoint: view splits (the split sum included, as ct_proj2d_adj runs it)
  const long ctas = (long)p0.adj_gx * p0.adj_gy * batch;
  const int ns_max = ct::max_splits(g, ctas);
  const size_t n = (size_t)batch * g->rows * g->cols;
  // Split counts 1, 2, 4, 8, ...: neighbours far enough apart in time that
  // the choice does not flip between runs on noise (the split count sets the
  // adjoint's summation order, and with it the rounding a caller sees).
  // Timings within kTie of the fastest count as ties and go to the fewest
  // splits (less split memory).
  constexpr float kTie = 1.03f;
  std::vector<std::pair<int, float>> cand;
  int last = 0;
  for (int ns = 1; ns <= ns_max; ns *= 2) {
    const ct::Proj2dPlan p = ct::proj2d_plan_sched(g, batch, ct::Sched2d{0, ns});
    if (p.nsplit == last) continue;  // same split count as the previous candidate
    last = p.nsplit;
    float us = 0.0f;
    st = time_calls(
        [&] {
          ct_status r = ct::proj2d_adj_launch(g, p, sino, img, ws, batch, s, nullptr);
          if (r != CT_OK || p.nsplit == 1) return r;
          const int blocks = (int)std::min<size_t>((n + 255) / 256, 4096);
          k_sum_splits<<<blocks, 256, 0, s>>>(ws, img, n, p.nsplit, n);
          return ct::launch_check("k_sum_splits");
        },
        reps, s, us);
    if (st != CT_OK) return st;
    cand.emplace_back(p.nsplit, us);
  }
  float fastest = cand.front().second;
  for (const auto& c : cand) fastest = std::min(fastest, c.second);
  float best_a = 0.0f;
  for (const auto& c : cand) {
    if (c.second <= kTie * fastest) {
      best.ns = c.first;
      best_a = c.second;
      break;
    }
  }
  {
    std::lock_guard<std::mutex> lk(ct::g_sched_mu);
    ct::g_sched[ct::sched_key(g, batch)] = ct::SchedVal{best, best_f, best_a};
  }
  if (chosen) {
    chosen->views_per_cta = best.vpc;
    chosen->adj_splits = best.ns;
    chosen->fwd_us = best_f;
    chosen->adj_us = best_a;
    chosen->tuned = 1;
  }
  return CT_OK;
}

ct_status ct_proj2d_schedule_get(const ct_geom2d* g, int32_t batch, ct_proj2d_schedule* out) {
  ct_status st = ct::proj2d_check(g, "ct_proj2d_schedule_get");
  if (st != CT_OK) return st;
  if (!out || batch <= 0) return ct::fail(CT_ERR_INVALID_ARG, "ct_proj2d_schedule_get: out=%p batch=%d",
                                          (void*)out, batch);
  ct::SchedVal v{};
  const bool tuned = ct::sched_lookup(g, batch, v);
  const ct::Proj2dPlan p = ct::proj2d_plan(g, batch);
  out->views_per_cta = p.vpc;
  out->adj_splits = p.nsplit;
  out->fwd_us = tuned ? v.fwd_us : 0.0f;
  out->adj_us = tuned ? v.adj_us : 0.0f;
  out->tuned = tuned ? 1 : 0;
  return CT_OK;
}

void ct_proj2d_schedule_clear(void) {
  std::lock_guard<std::mutex> lk(ct::g_sched_mu);
  ct::g_sched.clear();
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free forward projection.
//
// Some callers cannot allocate device memory when they project: code that
// runs inside a stream capture it does not own, plugin hosts that hand a
// custom call no allocator and no scratch buffer, and real-time loops that
// forbid allocation once they are running.  ct_proj2d_fwd_noalloc gives them
// the forward projection with its scratch in a fixed array in the library's
// own device memory (kNoallocScratchBytes, held by every GPU that loads the
// library until the process exits).
// ---------------------------------------------------------------------------
namespace {

constexpr size_t kNoallocScratchBytes = 16u << 20;  // 16 MiB
static __device__ __align__(256) unsigned char g_fwd_scratch[kNoallocScratchBytes];

// Device address of g_fwd_scratch, looked up once per device with that
// device current (host code only has a stand-in for the symbol).
float* noalloc_scratch() {
  static std::mutex m;
  static float* cached[64] = {nullptr};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  std::lock_guard<std::mutex> lock(m);
  if (!cached[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_fwd_scratch) != cudaSuccess) return nullptr;
    cached[dev] = static_cast<float*>(p);
  }
  return cached[dev];
}

}  // namespace

extern "C" {

ct_status ct_proj2d_fwd_noalloc(const ct_geom2d* g, const float* img, float* sino, int32_t batch,
                                ct_stream_t stream) {
  ct_status st = ct::proj2d_check(g, "ct_proj2d_fwd_noalloc");
  if (st != CT_OK) return st;
  if (!img || !sino) return ct::fail(CT_ERR_INVALID_ARG, "ct_proj2d_fwd_noalloc: null array");
  if (batch <= 0) return ct::fail(CT_ERR_INVALID_ARG, "ct_proj2d_fwd_noalloc: batch=%d", batch);
  const ct::Proj2dPlan p = ct::proj2d_plan(g, batch);
  if (p.fwd_bytes > kNoallocScratchBytes)
    return ct::fail(CT_ERR_UNSUPPORTED,
                    "ct_proj2d_fwd_noalloc: this projection needs %zu bytes of scratch, more than the "
                    "%zu-byte built-in array; use ct_proj2d_fwd with a workspace",
                    p.fwd_bytes, kNoallocScratchBytes);
  float* scratch = noalloc_scratch();
  if (!scratch) return ct::fail(CT_ERR_CUDA, "ct_proj2d_fwd_noalloc: scratch address lookup failed");
  st = ct::proj2d_prepare(p);
  if (st != CT_OK) return st;
  // Every scratch element the second pass reads is written by the first
  // pass of the same call, so nothing needs clearing between calls.
  return ct::proj2d_fwd_launch(g, p, img, sino, batch, scratch, ct::as_stream(stream), nullptr);
}

void ct_set_wait_poll_limit(uint32_t polls) { g_wait_polls.store(polls, std::memory_order_relaxed); }

uint32_t ct_wait_poll_limit(void) { return g_wait_polls.load(std::memory_order_relaxed); }

ct_status ct_proj2d_check(ct_stream_t stream) {
  ct_status st = ct::cuda_check(cudaStreamSynchronize(ct::as_stream(stream)), "ct_proj2d_check: synchronize");
  if (st != CT_OK) return st;
  int v = 0;
  st = ct::cuda_check(cudaMemcpyFromSymbol(&v, g_proj2d_err, sizeof(int)), "ct_proj2d_check: read");
  if (st != CT_OK) return st;
  if (v == 0) return CT_OK;
  const int zero = 0;
  st = ct::cuda_check(cudaMemcpyToSymbol(g_proj2d_err, &zero, sizeof(int)), "ct_proj2d_check: clear");
  if (st != CT_OK) return st;
  if (v & 8)
    return ct::fail(CT_ERR_TIMEOUT, "ct_proj2d_check: a solver grid barrier wait ran out (error word 0x%x); "
                    "the solve's results are void", v);
  if (v & 2)
    return ct::fail(CT_ERR_TIMEOUT, "ct_proj2d_check: a forward strip copy wait ran out (error word 0x%x); "
                    "the CTAs concerned skipped their work and wrote zeros", v);
  return ct::fail(CT_ERR_UNSUPPORTED, "ct_proj2d_check: a %s span exceeded the plan (error word 0x%x); "
                  "the work concerned was skipped", (v & 1) ? "forward tile" : "adjoint window", v);
}

// Diagnostic: returns (and clears) the projector's internal check word.
int ct_proj2d_errflag(void) {
  int v = 0;
  if (cudaMemcpyFromSymbol(&v, g_proj2d_err, sizeof(int)) != cudaSuccess) return -1;
  if (v != 0) {  // clear only a set word (no copy on the common path)
    const int zero = 0;
    cudaMemcpyToSymbol(g_proj2d_err, &zero, sizeof(int));
  }
  return v;
}

}  // extern "C"
