// 2D parallel-beam projector (scico XRayTransform2D) for sm_103a.
//
// Model (scico/linop/xray/_xray2d.py:308-351): pixel (i, j) projects for
// view v to Px = (Pxmin + Pdx0 i) + Pdx1 j; with k = floor(Px) and
// w = min(1 - (Px - k), width)/width it adds w*x to bin k and (1-w)*x to bin
// k+1 (bins outside [0, det) dropped).
//
// Forward (A):  tile-owned pixel-driven sweep.  A CTA owns a 32x32 image
//   tile and a run of views; lane r of a warp holds tile row r in registers
//   and walks its 32 pixels in the direction in which k is non-decreasing,
//   carrying the running sums of the current bin and the next one in
//   registers.  Each row's bin sums go to the warp's shared-memory partial
//   rows, which are then summed over the 32 rows in a fixed order.  The
//   per-(tile, view) partial bins are written to the workspace and a second
//   kernel sums the tiles covering each bin in tile order.  No atomics; the
//   result is bit-reproducible.
// Adjoint (A^T): pixel-driven gather over all views with the same weights,
//   views summed in a fixed order (optionally in fixed view splits reduced
//   by a second kernel), no atomics.
#include <algorithm>

#include "common.cuh"

namespace {

constexpr int kTile = 32;       // forward tile edge (rows = lanes, cols = registers)
constexpr int kFwdWarps = 8;    // views processed concurrently by one forward CTA
constexpr int kFwdViewsPerCta = 24;
constexpr int kAdjRows = 8;     // adjoint CTA: 8 rows x (32*kAdjPx) cols
constexpr int kAdjPx = 2;
constexpr int kAdjTargetCtas = 304;
constexpr int kAdjMinViewsPerSplit = 16;

struct ViewParams {
  float pxmin, pd0, pd1, width, inv_width;
};

__device__ __forceinline__ ViewParams load_view(const float* __restrict__ views, int v) {
  const float4 a = __ldg(reinterpret_cast<const float4*>(views) + 2 * v);
  const float4 b = __ldg(reinterpret_cast<const float4*>(views) + 2 * v + 1);
  return ViewParams{a.x, a.y, a.z, a.w, b.x};
}

// Bin range [base, top] of the pixel keys of the 32x32 tile at (i0, j0).
// Px is monotone in i and in j separately (every operation of px2d is a
// monotone rounding), so the extremes are at the tile corners.
__device__ __forceinline__ void tile_keys(const ViewParams& p, int i0, int j0, int& base, int& top) {
  const float a = ct::px2d(p.pxmin, p.pd0, p.pd1, i0, j0);
  const float b = ct::px2d(p.pxmin, p.pd0, p.pd1, i0 + kTile - 1, j0);
  const float c = ct::px2d(p.pxmin, p.pd0, p.pd1, i0, j0 + kTile - 1);
  const float d = ct::px2d(p.pxmin, p.pd0, p.pd1, i0 + kTile - 1, j0 + kTile - 1);
  base = (int)floorf(fminf(fminf(a, b), fminf(c, d)));
  top = (int)floorf(fmaxf(fmaxf(a, b), fmaxf(c, d)));
}

// Walk one tile row for one view.  REV walks j downwards (Pdx1 < 0) so that
// the bin key never decreases.  mp: this lane's partial row, indexed by
// key - base.  Bin b receives, in j order, the (1-w) x of the pixels with
// key b-1 followed by the w x of the pixels with key b.
template <bool REV>
__device__ __forceinline__ void walk_row(const float (&xr)[kTile], float* __restrict__ mp,
                                         const ViewParams& p, float R, int j0, int base) {
  int cur = 0;
  float A = 0.0f, B = 0.0f;
#pragma unroll
  for (int t = 0; t < kTile; ++t) {
    const int jj = REV ? kTile - 1 - t : t;
    const float px = ct::fadd(R, ct::fmul(p.pd1, (float)(j0 + jj)));
    int key;
    float w;
    ct::boxcar2d(px, p.width, p.inv_width, key, w);
    const float omw = ct::fsub(1.0f, w);
    if (t == 0) cur = key;
    const int d = key - cur;
    if (d >= 2) mp[cur + 1 - base] = B;  // bin cur+1 complete, bins between stay 0
    const float a0 = d == 0 ? A : (d == 1 ? B : 0.0f);
    const float b0 = d == 0 ? B : 0.0f;
    A = fmaf(w, xr[jj], a0);
    B = fmaf(omw, xr[jj], b0);
    cur = key;
    mp[cur - base] = A;
  }
  mp[cur + 1 - base] = B;
}

// Forward pass 1.  grid = (n_tiles, view groups, batch), block = 256.
// part layout: [batch][tile][view][L].
__global__ void __launch_bounds__(kFwdWarps * 32)
    k_proj2d_fwd_tiles(const float* __restrict__ img, float* __restrict__ part,
                       const float* __restrict__ views, int rows, int cols, int nv, int L,
                       int LS, int tiles_j, int n_tiles, int* __restrict__ errflag,
                       const double* __restrict__ skip) {
  if (skip && *skip != 0.0) return;
  extern __shared__ float smem[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int tile = blockIdx.x;
  const int ti = tile / tiles_j, tj = tile - ti * tiles_j;
  const int b = blockIdx.z;
  const int i0 = ti * kTile, j0 = tj * kTile;
  const int i = i0 + lane;

  float xr[kTile];
  {
    const float* im = img + (size_t)b * rows * cols;
    if (i < rows) {
      const float* rp = im + (size_t)i * cols + j0;
      const bool vec = ((cols & 3) == 0) && (j0 + kTile <= cols) && ct::aligned(rp, 16);
      if (vec) {
#pragma unroll
        for (int q = 0; q < kTile / 4; ++q) {
          const float4 f = __ldg(reinterpret_cast<const float4*>(rp) + q);
          xr[4 * q] = f.x;
          xr[4 * q + 1] = f.y;
          xr[4 * q + 2] = f.z;
          xr[4 * q + 3] = f.w;
        }
      } else {
#pragma unroll
        for (int jj = 0; jj < kTile; ++jj) xr[jj] = (j0 + jj < cols) ? __ldg(rp + jj) : 0.0f;
      }
    } else {
#pragma unroll
      for (int jj = 0; jj < kTile; ++jj) xr[jj] = 0.0f;
    }
  }

  float* wpart = smem + (size_t)warp * kTile * LS;
  float* mp = wpart + (size_t)lane * LS;
  const int vbeg = blockIdx.y * kFwdViewsPerCta;
  const int vend = min(nv, vbeg + kFwdViewsPerCta);
  for (int v = vbeg + warp; v < vend; v += kFwdWarps) {
    const ViewParams p = load_view(views, v);
    int base, top;
    tile_keys(p, i0, j0, base, top);
    float* po = part + (((size_t)b * n_tiles + tile) * nv + v) * L;
    if (top - base + 2 > L) {  // cannot happen for a table from ct_proj2d_views
      if (lane == 0) atomicOr(errflag, 1);
      for (int k = lane; k < L; k += 32) po[k] = 0.0f;
      continue;
    }
    for (int k = 0; k < L; ++k) mp[k] = 0.0f;
    const float R = ct::fadd(p.pxmin, ct::fmul(p.pd0, (float)i));
    if (p.pd1 >= 0.0f)
      walk_row<false>(xr, mp, p, R, j0, base);
    else
      walk_row<true>(xr, mp, p, R, j0, base);
    __syncwarp();
    for (int k = lane; k < L; k += 32) {
      float s = 0.0f;
      const float* q = wpart + k;
#pragma unroll 8
      for (int r = 0; r < kTile; ++r) s += q[(size_t)r * LS];
      po[k] = s;
    }
    __syncwarp();
  }
}

// Forward pass 2: sino[b, v, bin] = sum over tiles (in tile order) of the
// tile partials covering bin.  grid = (n_views, batch), block = 256,
// dynamic smem = n_tiles ints.
__global__ void __launch_bounds__(256)
    k_proj2d_fwd_gather(const float* __restrict__ part, float* __restrict__ sino,
                        const float* __restrict__ views, int nv, int det, int L, int tiles_j,
                        int n_tiles, const double* __restrict__ skip) {
  if (skip && *skip != 0.0) return;
  extern __shared__ int sbase[];
  const int v = blockIdx.x, b = blockIdx.y;
  const ViewParams p = load_view(views, v);
  for (int t = threadIdx.x; t < n_tiles; t += blockDim.x) {
    const int ti = t / tiles_j, tj = t - ti * tiles_j;
    int base, top;
    tile_keys(p, ti * kTile, tj * kTile, base, top);
    sbase[t] = base;
  }
  __syncthreads();
  const float* pb = part + ((size_t)b * n_tiles * nv + v) * L;
  const size_t tstride = (size_t)nv * L;
  float* out = sino + ((size_t)b * nv + v) * det;
  for (int bin = threadIdx.x; bin < det; bin += blockDim.x) {
    float acc = 0.0f;
    for (int t = 0; t < n_tiles; ++t) {
      const int off = bin - sbase[t];
      if ((unsigned)off < (unsigned)L) acc += __ldg(pb + t * tstride + off);
    }
    out[bin] = acc;
  }
}

// Adjoint.  grid = (ceil(cols/64), ceil(rows/8), batch*nsplit),
// block = (32, 8).  With nsplit > 1, split s sums views
// [s*per, (s+1)*per) into out + s*split_stride.
__global__ void __launch_bounds__(256)
    k_proj2d_adj(const float* __restrict__ sino, float* __restrict__ out,
                 const float* __restrict__ views, int rows, int cols, int nv, int det,
                 int nsplit, int per_split, size_t split_stride, const double* __restrict__ skip) {
  if (skip && *skip != 0.0) return;
  __shared__ float4 sv[256];
  __shared__ float sinv[256];
  const int z = blockIdx.z;
  const int b = z / nsplit, s = z - b * nsplit;
  const int vbeg = s * per_split, vend = min(nv, vbeg + per_split);
  const int i = blockIdx.y * kAdjRows + threadIdx.y;
  const int jb = blockIdx.x * 32 * kAdjPx + threadIdx.x;
  const int tid = threadIdx.y * 32 + threadIdx.x;
  const float* yb = sino + (size_t)b * nv * det;
  float acc[kAdjPx];
#pragma unroll
  for (int q = 0; q < kAdjPx; ++q) acc[q] = 0.0f;
  const float fi = (float)i;

  for (int a0 = vbeg; a0 < vend; a0 += 256) {
    const int n = min(256, vend - a0);
    __syncthreads();
    if (tid < n) {
      const ViewParams p = load_view(views, a0 + tid);
      sv[tid] = make_float4(p.pxmin, p.pd0, p.pd1, p.width);
      sinv[tid] = p.inv_width;
    }
    __syncthreads();
    for (int k = 0; k < n; ++k) {
      const float4 pv = sv[k];
      const float invw = sinv[k];
      const float* yr = yb + (size_t)(a0 + k) * det;
      const float R = ct::fadd(pv.x, ct::fmul(pv.y, fi));
#pragma unroll
      for (int q = 0; q < kAdjPx; ++q) {
        const int j = jb + 32 * q;
        const float px = ct::fadd(R, ct::fmul(pv.z, (float)j));
        int key;
        float w;
        ct::boxcar2d(px, pv.w, invw, key, w);
        const float omw = ct::fsub(1.0f, w);
        const float y0 = ((unsigned)key < (unsigned)det) ? __ldg(yr + key) : 0.0f;
        const float y1 = ((unsigned)(key + 1) < (unsigned)det) ? __ldg(yr + key + 1) : 0.0f;
        acc[q] = fmaf(y0, w, acc[q]);
        acc[q] = fmaf(y1, omw, acc[q]);
      }
    }
  }
  if (i < rows) {
    float* o = out + (size_t)s * split_stride + (size_t)b * rows * cols + (size_t)i * cols;
#pragma unroll
    for (int q = 0; q < kAdjPx; ++q) {
      const int j = jb + 32 * q;
      if (j < cols) o[j] = acc[q];
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


// Device error word for the forward's internal span check.
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

}  // namespace

#include "kernels.cuh"

namespace ct {

ct_status proj2d_check(const ct_geom2d* g, const char* who) {
  if (!g) return fail(CT_ERR_INVALID_ARG, "%s: null geometry", who);
  if (g->rows <= 0 || g->cols <= 0 || g->n_views <= 0 || g->det_count <= 0)
    return fail(CT_ERR_SHAPE, "%s: bad geometry rows=%d cols=%d views=%d det=%d", who, g->rows,
                g->cols, g->n_views, g->det_count);
  if (!g->views) return fail(CT_ERR_INVALID_ARG, "%s: null view table", who);
  if (!aligned(g->views, 16)) return fail(CT_ERR_INVALID_ARG, "%s: view table not 16-B aligned", who);
  if (!(g->max_width > 0.0f) || g->max_width > 64.0f)
    return fail(CT_ERR_UNSUPPORTED, "%s: max projected pixel width %g outside (0, 64]", who,
                (double)g->max_width);
  const Proj2dPlan p = proj2d_plan(g, 1);
  if (p.fwd_smem > 200 * 1024)
    return fail(CT_ERR_UNSUPPORTED, "%s: tile span of %d bins too large", who, p.L);
  if ((size_t)p.n_tiles * sizeof(int) > 200 * 1024)
    return fail(CT_ERR_UNSUPPORTED, "%s: %d image tiles too many", who, p.n_tiles);
  return CT_OK;
}

Proj2dPlan proj2d_plan(const ct_geom2d* g, int batch) {
  Proj2dPlan p;
  p.tiles_i = (g->rows + kTile - 1) / kTile;
  p.tiles_j = (g->cols + kTile - 1) / kTile;
  p.n_tiles = p.tiles_i * p.tiles_j;
  // Keys inside a tile differ by at most 31*(|Pdx0|+|Pdx1|) + 1 (plus
  // rounding); the tile needs bins [base, top + 1].
  p.L = (int)floorf(31.0f * g->max_width * 1.0001f + 1.01f) + 3;
  p.LS = p.L | 1;  // odd row stride: lanes of one column hit distinct banks
  p.view_groups = (g->n_views + kFwdViewsPerCta - 1) / kFwdViewsPerCta;
  p.fwd_bytes = round_up((size_t)batch * p.n_tiles * g->n_views * p.L * sizeof(float), 256);
  p.fwd_smem = (size_t)kFwdWarps * kTile * p.LS * sizeof(float);
  p.adj_gx = (g->cols + 32 * kAdjPx - 1) / (32 * kAdjPx);
  p.adj_gy = (g->rows + kAdjRows - 1) / kAdjRows;
  const long ctas = (long)p.adj_gx * p.adj_gy * batch;
  int ns = 1;
  if (ctas < kAdjTargetCtas) ns = (int)((kAdjTargetCtas + ctas - 1) / ctas);
  ns = std::min(ns, std::max(1, g->n_views / kAdjMinViewsPerSplit));
  p.per_split = (g->n_views + ns - 1) / ns;
  p.nsplit = (g->n_views + p.per_split - 1) / p.per_split;
  p.adj_bytes =
      p.nsplit > 1 ? round_up((size_t)p.nsplit * batch * g->rows * g->cols * sizeof(float), 256) : 0;
  return p;
}

ct_status proj2d_prepare(const Proj2dPlan& p) {
  if (!errflag_ptr()) return fail(CT_ERR_CUDA, "proj2d: error-word address unavailable");
  if (p.fwd_smem > 48 * 1024) {
    ct_status st = cuda_check(cudaFuncSetAttribute(k_proj2d_fwd_tiles,
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   (int)p.fwd_smem),
                              "fwd smem attribute");
    if (st != CT_OK) return st;
  }
  const size_t smem2 = (size_t)p.n_tiles * sizeof(int);
  if (smem2 > 48 * 1024) {
    ct_status st = cuda_check(cudaFuncSetAttribute(k_proj2d_fwd_gather,
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   (int)smem2),
                              "gather smem attribute");
    if (st != CT_OK) return st;
  }
  return CT_OK;
}

ct_status proj2d_fwd_launch(const ct_geom2d* g, const Proj2dPlan& p, const float* img, float* sino,
                            int batch, float* part, cudaStream_t s, const double* skip) {
  int* errflag = errflag_ptr();
  if (!errflag) return fail(CT_ERR_CUDA, "proj2d: error-word address unavailable");
  dim3 g1(p.n_tiles, p.view_groups, batch);
  k_proj2d_fwd_tiles<<<g1, kFwdWarps * 32, p.fwd_smem, s>>>(img, part, g->views, g->rows, g->cols,
                                                            g->n_views, p.L, p.LS, p.tiles_j,
                                                            p.n_tiles, errflag, skip);
  ct_status st = launch_check("k_proj2d_fwd_tiles");
  if (st != CT_OK) return st;
  dim3 g2(g->n_views, batch);
  k_proj2d_fwd_gather<<<g2, 256, (size_t)p.n_tiles * sizeof(int), s>>>(
      part, sino, g->views, g->n_views, g->det_count, p.L, p.tiles_j, p.n_tiles, skip);
  return launch_check("k_proj2d_fwd_gather");
}

ct_status proj2d_adj_launch(const ct_geom2d* g, const Proj2dPlan& p, const float* sino, float* out,
                            float* part, int batch, cudaStream_t s, const double* skip) {
  const size_t n = (size_t)batch * g->rows * g->cols;
  dim3 grid(p.adj_gx, p.adj_gy, batch * p.nsplit);
  float* dst = p.nsplit > 1 ? part : out;
  k_proj2d_adj<<<grid, dim3(32, kAdjRows), 0, s>>>(sino, dst, g->views, g->rows, g->cols,
                                                   g->n_views, g->det_count, p.nsplit, p.per_split,
                                                   p.nsplit > 1 ? n : 0, skip);
  return launch_check("k_proj2d_adj");
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
  if (adj_bytes) *adj_bytes = p.adj_bytes;
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
  float* part = static_cast<float*>(workspace);
  st = ct::proj2d_adj_launch(g, p, sino, img, part, batch, s, nullptr);
  if (st != CT_OK || p.nsplit == 1) return st;
  const size_t n = (size_t)batch * g->rows * g->cols;
  const int blocks = (int)std::min<size_t>((n + 255) / 256, 4096);
  k_sum_splits<<<blocks, 256, 0, s>>>(part, img, n, p.nsplit, n);
  return ct::launch_check("k_sum_splits");
}

// Diagnostic: returns (and clears) the forward's internal span-check word.
int ct_proj2d_errflag(void) {
  int v = 0;
  if (cudaMemcpyFromSymbol(&v, g_proj2d_err, sizeof(int)) != cudaSuccess) return -1;
  const int zero = 0;
  cudaMemcpyToSymbol(g_proj2d_err, &zero, sizeof(int));
  return v;
}

}  // extern "C"
