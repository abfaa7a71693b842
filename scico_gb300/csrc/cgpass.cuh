// The element passes of the CG vector steps (scico/solver.py:378-400),
// shared by the separate kernels (vec.cu) and the solver's fused CG step
// (admm.cu), so that both compute the same bits.  Grid-stride loops over a
// grid of kReduceBlocks x kReduceThreads threads; with vec (n % 4 == 0 and
// 16-B aligned arrays) a thread moves four consecutive elements per 128-bit
// access, two quads per step so that more loads are in flight; per element
// the arithmetic is the scalar code's.
#pragma once

#include "common.cuh"

namespace ct {

__device__ __forceinline__ float4 cgp_ld4(const float* p, size_t e) { return *reinterpret_cast<const float4*>(p + e); }
__device__ __forceinline__ void cgp_st4(float* p, size_t e, float4 v) { *reinterpret_cast<float4*>(p + e) = v; }
__device__ __forceinline__ float cgp_at4(const float4& v, int j) {
  return j == 0 ? v.x : (j == 1 ? v.y : (j == 2 ? v.z : v.w));
}

// x += af p; r -= af Ap; returns this thread's share of <r, r> (float64).
__device__ __forceinline__ double cg_update_pass(float* x, float* r, const float* p, const float* Ap, size_t n,
                                                 float af, int vec) {
  constexpr int NT = kReduceThreads;
  double rr = 0.0;
  if (vec) {
    const size_t stride = 4 * (size_t)gridDim.x * NT;
    auto quad = [&](size_t e0, float4 x4, float4 r4, float4 p4, float4 a4) {
      float xv[4], rv[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        xv[j] = fadd(cgp_at4(x4, j), fmul(af, cgp_at4(p4, j)));
        rv[j] = fsub(cgp_at4(r4, j), fmul(af, cgp_at4(a4, j)));
        rr += (double)rv[j] * (double)rv[j];
      }
      cgp_st4(x, e0, make_float4(xv[0], xv[1], xv[2], xv[3]));
      cgp_st4(r, e0, make_float4(rv[0], rv[1], rv[2], rv[3]));
    };
    for (size_t e0 = 4 * ((size_t)blockIdx.x * NT + threadIdx.x); e0 < n; e0 += 2 * stride) {
      const bool two = e0 + stride < n;
      const float4 x0 = cgp_ld4(x, e0), r0 = cgp_ld4(r, e0), p0 = cgp_ld4(p, e0), a0 = cgp_ld4(Ap, e0);
      float4 x1 = x0, r1 = r0, p1 = p0, a1 = a0;
      if (two) {
        x1 = cgp_ld4(x, e0 + stride);
        r1 = cgp_ld4(r, e0 + stride);
        p1 = cgp_ld4(p, e0 + stride);
        a1 = cgp_ld4(Ap, e0 + stride);
      }
      quad(e0, x0, r0, p0, a0);
      if (two) quad(e0 + stride, x1, r1, p1, a1);
    }
  } else {
    for (size_t e = (size_t)blockIdx.x * NT + threadIdx.x; e < n; e += (size_t)gridDim.x * NT) {
      const float pe = p[e];
      x[e] = fadd(x[e], fmul(af, pe));
      const float re = fsub(r[e], fmul(af, Ap[e]));
      r[e] = re;
      rr += (double)re * (double)re;
    }
  }
  return rr;
}

// p = r + bf p.
__device__ __forceinline__ void cg_direction_pass(float* p, const float* r, size_t n, float bf, int vec) {
  constexpr int NT = kReduceThreads;
  if (vec) {
    const size_t stride = 4 * (size_t)gridDim.x * NT;
    auto quad = [&](size_t e0, float4 r4, float4 p4) {
      cgp_st4(p, e0, make_float4(fadd(r4.x, fmul(bf, p4.x)), fadd(r4.y, fmul(bf, p4.y)),
                                 fadd(r4.z, fmul(bf, p4.z)), fadd(r4.w, fmul(bf, p4.w))));
    };
    for (size_t e0 = 4 * ((size_t)blockIdx.x * NT + threadIdx.x); e0 < n; e0 += 2 * stride) {
      const bool two = e0 + stride < n;
      const float4 r0 = cgp_ld4(r, e0), p0 = cgp_ld4(p, e0);
      float4 r1 = r0, p1 = p0;
      if (two) {
        r1 = cgp_ld4(r, e0 + stride);
        p1 = cgp_ld4(p, e0 + stride);
      }
      quad(e0, r0, p0);
      if (two) quad(e0 + stride, r1, p1);
    }
  } else {
    for (size_t e = (size_t)blockIdx.x * NT + threadIdx.x; e < n; e += (size_t)gridDim.x * NT)
      p[e] = fadd(r[e], fmul(bf, p[e]));
  }
}

}  // namespace ct
