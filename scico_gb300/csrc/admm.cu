// Fused ADMM-TV solver for 2D and 3D parallel-beam CT.
//
// Solves  min_x scale ||A x - y||^2 + lam21 ||D x||_{2,1} + lam1 ||D x||_1
// with scico's ADMM + LinearSubproblemSolver (scico/optimize/_admm.py:334-378,
// _admmaux.py:205-269, scico/solver.py:326-405), D = FiniteDifference over
// all image axes with append=0 (stacked (ND, *shape), ND = 2 for a slice
// with XRayTransform2D, 3 for a volume with XRayTransform3D).  One g_i per
// non-zero lambda, L2,1 first, each with its own z_i and u_i, all sharing D
// and rho.  The elementwise kernels are templated on ND; A is whichever
// projector the descriptor names.
//
// Per outer iteration (each kernel below is one launch; with graphs the
// whole solve is captured once into a CUDA graph -- set-up, the iterations
// as a conditional WHILE node that k_zu keeps running for maxiter
// iterations, the statistics epilogue -- and launched once per call; a batch
// of scans is one graph with one such branch per scan):
//   k_rhs         rhs = c A^T y + sum_i rho D^T(z_i - u_i); also the dual
//                 residual ||sum_i rho D^T(z_i - z_i_old)|| of the previous
//                 iteration
//   A x           forward projection of the current x, k_resid2 gives
//                 ||A x - y||^2 for the previous iteration's objective, then
//                 A^T (A x); in the graph these three form a conditional IF
//                 node that k_rhs opens only when CG moved x
//   k_lhs_finish<INIT>   writes the previous iteration's itstat record, then
//                 lhs(x) = c A^T A x + rho D^T D x, r = rhs - lhs(x), p = r,
//                 CG scalars (num, ||b||, tolerance) in float64
//   CG loop       A p, A^T, k_lhs_finish<PAP> (Ap, <p,Ap>), CG update,
//                 direction.  In the graph the loop is a conditional WHILE
//                 node whose condition the device sets (CG start and each
//                 update), so it runs exactly the reference's number of CG
//                 iterations; without a graph, cg_maxiter copies are launched
//                 and become no-ops once CG has converged
//   k_zu          Dx, z_i = prox(Dx + u_i), u_i += Dx - z_i, primal residual
//                 and g_i(z_i) partial sums; in the graph its last block
//                 counts the iteration and sets the iteration loop's
//                 condition
// lhs(x) and A x are kept from the last CG start while x is unchanged (no CG
// step ran since): the deterministic kernels would recompute the same bits,
// so the projections of x are skipped then.
// The reference evaluates the itstat quantities with extra operator
// applications after each step; here they are fused into the kernels that
// already read the operands, and the x-dependent ones are taken from the
// next iteration's first projection of the same x (an epilogue covers the
// last iteration).
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <mutex>
#include <vector>

#include "cgpass.cuh"
#include "kernels.cuh"

namespace {

constexpr int NT = ct::kReduceThreads;
constexpr int NB = ct::kReduceBlocks;

// Scalar slots (double) of the solver state block.
enum Slot {
  S_RESID2 = 0,   // ||A x - y||^2 of the current x
  S_DUAL2 = 1,    // ||sum rho D^T dz||^2 of the previous iteration
  S_PRIMAL2 = 2,  // sum_i rho ||D x - z_i||^2 of the last z/u update
  S_G21 = 3,      // ||z_l21||_{2,1} of the last z/u update
  S_G1 = 4,       // ||z_l1||_1 of the last z/u update
  S_HAVE_PREV = 5,
  S_REC = 6,      // records written in this call
  S_XCLEAN = 7,   // 1 while lhs(x) and A x in the workspace belong to the current x
  S_ITER = 8,     // ADMM iterations run in this call (the graph's device-side loop)
  S_ZU_DONE = 9,  // 1: the fast-forward kernel ran the last iteration's z/u update
  S_CG = 16,      // CT_CG_NSCALARS doubles
  S_COUNT = 32
};

struct TermParams {
  int ng;          // number of g terms (1 or 2)
  int kind[2];     // 0 = L2,1, 1 = L1
  float thr[2];    // prox threshold lam_i / rho
  float rho;       // rho (float32, as the reference multiplies arrays)
  float alpha;     // relaxation
  float c;         // 2 * loss scale
};

// Image shape (n[0..ND-1], C order) of the fused kernels: ND = 2 for 2D
// slices, 3 for volumes.
struct Shape3 {
  int n[3];
};

// Loads of the state arrays in the fused passes.  LdPlain: ordinary loads
// (the separate kernels read only what earlier kernels wrote).  LdL2: loads
// through L2 only (ld.global.cg) for the cooperative fast-forward kernel,
// whose blocks read, after a grid barrier, elements that other blocks wrote
// earlier in the same launch.  The arithmetic is the same either way.
struct LdPlain {
  static __device__ __forceinline__ float4 q(const float* p) { return *reinterpret_cast<const float4*>(p); }
  static __device__ __forceinline__ float s(const float* p) { return *p; }
};
struct LdL2 {
  static __device__ __forceinline__ float4 q(const float* p) { return __ldcg(reinterpret_cast<const float4*>(p)); }
  static __device__ __forceinline__ float s(const float* p) { return __ldcg(p); }
};

template <int ND>
__device__ __forceinline__ void coords(size_t e, const Shape3& sh, int (&c)[ND]) {
  if (ND == 2) {
    c[0] = (int)(e / (size_t)sh.n[1]);
    c[ND - 1] = (int)(e % (size_t)sh.n[1]);
  } else {
    const size_t r = e / (size_t)sh.n[ND - 1];
    c[ND - 1] = (int)(e - r * (size_t)sh.n[ND - 1]);
    c[1] = (int)(r % (size_t)sh.n[1]);
    c[0] = (int)(r / (size_t)sh.n[1]);
  }
}

// C-order element stride of axis k.
template <int ND>
__device__ __forceinline__ size_t axis_stride(const Shape3& sh, int k) {
  size_t st = 1;
  for (int q = ND - 1; q > k; --q) st *= (size_t)sh.n[q];
  return st;
}

// D^T applied at element e to a stacked (ND, *shape) field f = a - b (b may
// be null): sum over axes of (f_k[e - st_k] - f_k[e]) with the append=0
// boundaries, axes added in order (linop/_stack.py:71-72).
template <int ND, class LD = LdPlain>
__device__ __forceinline__ float dT_at(const float* a, const float* b, const int (&c)[ND], size_t e,
                                       const Shape3& sh, size_t N) {
  auto f = [&](int comp, size_t idx) -> float {
    const float av = LD::s(a + comp * N + idx);
    return b ? ct::fsub(av, LD::s(b + comp * N + idx)) : av;
  };
  float tot = 0.0f;
#pragma unroll
  for (int k = 0; k < ND; ++k) {
    const size_t st = axis_stride<ND>(sh, k);
    const float lo = c[k] >= 1 ? f(k, e - st) : 0.0f;
    const float hi = c[k] <= sh.n[k] - 2 ? f(k, e) : 0.0f;
    const float term = ct::fsub(lo, hi);
    tot = k == 0 ? term : ct::fadd(tot, term);
  }
  return tot;
}

// (D^T D q) at element e, append=0 differences over all axes.
template <int ND>
__device__ __forceinline__ float dtd_at(const float* __restrict__ q, const int (&c)[ND], size_t e,
                                        const Shape3& sh) {
  const float qc = q[e];
  float tot = 0.0f;
#pragma unroll
  for (int k = 0; k < ND; ++k) {
    const size_t st = axis_stride<ND>(sh, k);
    const float lo = c[k] >= 1 ? ct::fsub(qc, q[e - st]) : 0.0f;
    const float hi = c[k] <= sh.n[k] - 2 ? ct::fsub(q[e + st], qc) : 0.0f;
    const float term = ct::fsub(lo, hi);
    tot = k == 0 ? term : ct::fadd(tot, term);
  }
  return tot;
}

// D x at element e: x[e + st_k] - x[e] per axis; the appended last
// difference along an axis is x - x.
template <int ND>
__device__ __forceinline__ void d_at(const float* __restrict__ x, const int (&c)[ND], size_t e,
                                     const Shape3& sh, float (&d)[ND]) {
  const float xc = x[e];
#pragma unroll
  for (int k = 0; k < ND; ++k) {
    const size_t st = axis_stride<ND>(sh, k);
    d[k] = ct::fsub(c[k] <= sh.n[k] - 2 ? x[e + st] : xc, xc);
  }
}

// ---------------------------------------------------------------------------
// Quad path: a thread takes four consecutive elements e0..e0+3 along the
// last axis (used when n[ND-1] % 4 == 0 and every array is 16-B aligned, so
// the quad shares its row and each axis' neighbours are quads too).  The
// per-element arithmetic is the scalar code's, in the same order; only the
// loads are 128-bit.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float4 ld4(const float* __restrict__ p, size_t e) {
  return *reinterpret_cast<const float4*>(p + e);
}
__device__ __forceinline__ void st4(float* __restrict__ p, size_t e, const float (&v)[4]) {
  *reinterpret_cast<float4*>(p + e) = make_float4(v[0], v[1], v[2], v[3]);
}
__device__ __forceinline__ void unpack4(const float4 a, float (&v)[4]) {
  v[0] = a.x;
  v[1] = a.y;
  v[2] = a.z;
  v[3] = a.w;
}

// dT_at for the quad at e0 (coordinates c of e0).
template <int ND, class LD = LdPlain>
__device__ __forceinline__ void dT_at4(const float* a, const float* b, const int (&c)[ND], size_t e0,
                                       const Shape3& sh, size_t N, float (&tot)[4]) {
  auto f4 = [&](int comp, size_t idx, float (&v)[4]) {
    unpack4(LD::q(a + comp * N + idx), v);
    if (b) {
      float w[4];
      unpack4(LD::q(b + comp * N + idx), w);
#pragma unroll
      for (int j = 0; j < 4; ++j) v[j] = ct::fsub(v[j], w[j]);
    }
  };
  auto f1 = [&](int comp, size_t idx) -> float {
    const float av = LD::s(a + comp * N + idx);
    return b ? ct::fsub(av, LD::s(b + comp * N + idx)) : av;
  };
#pragma unroll
  for (int k = 0; k < ND; ++k) {
    float fc[4], lo[4], hi[4];
    f4(k, e0, fc);
    if (k < ND - 1) {
      const size_t st = axis_stride<ND>(sh, k);
      if (c[k] >= 1) {
        f4(k, e0 - st, lo);
      } else {
#pragma unroll
        for (int j = 0; j < 4; ++j) lo[j] = 0.0f;
      }
      const bool h = c[k] <= sh.n[k] - 2;
#pragma unroll
      for (int j = 0; j < 4; ++j) hi[j] = h ? fc[j] : 0.0f;
    } else {
      const int cl = c[ND - 1], nl = sh.n[ND - 1];
      lo[0] = cl >= 1 ? f1(k, e0 - 1) : 0.0f;
      lo[1] = fc[0];
      lo[2] = fc[1];
      lo[3] = fc[2];
#pragma unroll
      for (int j = 0; j < 4; ++j) hi[j] = cl + j <= nl - 2 ? fc[j] : 0.0f;
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const float term = ct::fsub(lo[j], hi[j]);
      tot[j] = k == 0 ? term : ct::fadd(tot[j], term);
    }
  }
}

// dtd_at for the quad at e0; qc = q at e0..e0+3.
template <int ND>
__device__ __forceinline__ void dtd_at4(const float* __restrict__ q, const float (&qc)[4], const int (&c)[ND],
                                        size_t e0, const Shape3& sh, float (&tot)[4]) {
#pragma unroll
  for (int k = 0; k < ND; ++k) {
    float lo[4], hi[4];
    if (k < ND - 1) {
      const size_t st = axis_stride<ND>(sh, k);
      float ql[4], qh[4];
      const bool hl = c[k] >= 1, hh = c[k] <= sh.n[k] - 2;
      if (hl) unpack4(ld4(q, e0 - st), ql);
      if (hh) unpack4(ld4(q, e0 + st), qh);
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        lo[j] = hl ? ct::fsub(qc[j], ql[j]) : 0.0f;
        hi[j] = hh ? ct::fsub(qh[j], qc[j]) : 0.0f;
      }
    } else {
      const int cl = c[ND - 1], nl = sh.n[ND - 1];
      const float qm = cl >= 1 ? q[e0 - 1] : 0.0f;
      const float qp = cl + 3 <= nl - 2 ? q[e0 + 4] : 0.0f;
      const float prev[4] = {qm, qc[0], qc[1], qc[2]};
      const float next[4] = {qc[1], qc[2], qc[3], qp};
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        lo[j] = cl + j >= 1 ? ct::fsub(qc[j], prev[j]) : 0.0f;
        hi[j] = cl + j <= nl - 2 ? ct::fsub(next[j], qc[j]) : 0.0f;
      }
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const float term = ct::fsub(lo[j], hi[j]);
      tot[j] = k == 0 ? term : ct::fadd(tot[j], term);
    }
  }
}

// d_at for the quad at e0; xc = x at e0..e0+3.
template <int ND>
__device__ __forceinline__ void d_at4(const float* __restrict__ x, const float (&xc)[4], const int (&c)[ND],
                                      size_t e0, const Shape3& sh, float (&d)[ND][4]) {
#pragma unroll
  for (int k = 0; k < ND; ++k) {
    float nx[4];
    if (k < ND - 1) {
      const size_t st = axis_stride<ND>(sh, k);
      if (c[k] <= sh.n[k] - 2) {
        unpack4(ld4(x, e0 + st), nx);
      } else {
#pragma unroll
        for (int j = 0; j < 4; ++j) nx[j] = xc[j];
      }
    } else {
      const int cl = c[ND - 1], nl = sh.n[ND - 1];
      nx[0] = xc[1];
      nx[1] = xc[2];
      nx[2] = xc[3];
      nx[3] = cl + 3 <= nl - 2 ? x[e0 + 4] : xc[3];
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) d[k][j] = ct::fsub(nx[j], xc[j]);
  }
}

template <int ND>
__global__ void __launch_bounds__(NT) k_init_state(const float* __restrict__ x, float* __restrict__ z,
                                                   float* __restrict__ u, float* __restrict__ dz,
                                                   Shape3 sh, size_t N, int ng, int vec) {
  if (vec) {
    for (size_t e0 = 4 * ((size_t)blockIdx.x * NT + threadIdx.x); e0 < N; e0 += 4 * (size_t)gridDim.x * NT) {
      int c[ND];
      coords<ND>(e0, sh, c);
      float xc[4], d[ND][4];
      unpack4(ld4(x, e0), xc);
      d_at4<ND>(x, xc, c, e0, sh, d);
      const float zero[4] = {0.0f, 0.0f, 0.0f, 0.0f};
      for (int t = 0; t < ng; ++t) {
        const size_t o = (size_t)t * ND * N;
#pragma unroll
        for (int k = 0; k < ND; ++k) {
          st4(z + o + k * N, e0, d[k]);
          st4(u + o + k * N, e0, zero);
          st4(dz + o + k * N, e0, zero);
        }
      }
    }
    return;
  }
  for (size_t e = (size_t)blockIdx.x * NT + threadIdx.x; e < N; e += (size_t)gridDim.x * NT) {
    int c[ND];
    coords<ND>(e, sh, c);
    float d[ND];
    d_at<ND>(x, c, e, sh, d);
    for (int t = 0; t < ng; ++t) {
      const size_t o = (size_t)t * ND * N;
#pragma unroll
      for (int k = 0; k < ND; ++k) {
        z[o + k * N + e] = d[k];
        u[o + k * N + e] = 0.0f;
        dz[o + k * N + e] = 0.0f;
      }
    }
  }
}

// out = c * (sum of the adjoint split partials), plain (used once for A^T y).
__global__ void __launch_bounds__(NT) k_scale_splits(const float* __restrict__ src, float* __restrict__ out,
                                                     size_t n, int nsplit, float c, int vec) {
  if (vec) {
    for (size_t e0 = 4 * ((size_t)blockIdx.x * NT + threadIdx.x); e0 < n; e0 += 4 * (size_t)gridDim.x * NT) {
      float4 a = ld4(src, e0);
      for (int k = 1; k < nsplit; ++k) {
        const float4 w = ld4(src + (size_t)k * n, e0);
        a = make_float4(ct::fadd(a.x, w.x), ct::fadd(a.y, w.y), ct::fadd(a.z, w.z), ct::fadd(a.w, w.w));
      }
      *reinterpret_cast<float4*>(out + e0) =
          make_float4(ct::fmul(c, a.x), ct::fmul(c, a.y), ct::fmul(c, a.z), ct::fmul(c, a.w));
    }
    return;
  }
  for (size_t e = (size_t)blockIdx.x * NT + threadIdx.x; e < n; e += (size_t)gridDim.x * NT) {
    float s = src[e];
    for (int k = 1; k < nsplit; ++k) s = ct::fadd(s, src[(size_t)k * n + e]);
    out[e] = ct::fmul(c, s);
  }
}

// k_rhs's pass over the elements: rhs = c A^T y + sum_i rho D^T (z_i - u_i)
// and this thread's share of the dual residual ||sum_i rho D^T dz_i||^2.
template <int ND, class LD>
__device__ __forceinline__ ct::KSum rhs_pass(const float* atyc, const float* z, const float* u, const float* dz,
                                            float* rhs, const Shape3& sh, size_t N, const TermParams& tp,
                                            int vec) {
  ct::KSum ks;  // dual residual
  if (vec) {
    for (size_t e0 = 4 * ((size_t)blockIdx.x * NT + threadIdx.x); e0 < N; e0 += 4 * (size_t)gridDim.x * NT) {
      int c[ND];
      coords<ND>(e0, sh, c);
      float val[4], dv[4];
      unpack4(LD::q(atyc + e0), val);
      for (int t = 0; t < tp.ng; ++t) {
        const size_t o = (size_t)t * ND * N;
        float g[4], h[4];
        dT_at4<ND, LD>(z + o, u + o, c, e0, sh, N, g);
        dT_at4<ND, LD>(dz + o, nullptr, c, e0, sh, N, h);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          val[j] = ct::fadd(val[j], ct::fmul(tp.rho, g[j]));
          const float w = ct::fmul(tp.rho, h[j]);
          dv[j] = (t == 0) ? w : ct::fadd(dv[j], w);
        }
      }
      st4(rhs, e0, val);
#pragma unroll
      for (int j = 0; j < 4; ++j) ks.add(ct::fmul(dv[j], dv[j]));
    }
  } else {
  for (size_t e = (size_t)blockIdx.x * NT + threadIdx.x; e < N; e += (size_t)gridDim.x * NT) {
    int c[ND];
    coords<ND>(e, sh, c);
    float val = LD::s(atyc + e);
    float dv = 0.0f;
    for (int t = 0; t < tp.ng; ++t) {
      const size_t o = (size_t)t * ND * N;
      val = ct::fadd(val, ct::fmul(tp.rho, dT_at<ND, LD>(z + o, u + o, c, e, sh, N)));
      const float w = ct::fmul(tp.rho, dT_at<ND, LD>(dz + o, nullptr, c, e, sh, N));
      dv = (t == 0) ? w : ct::fadd(dv, w);
    }
    rhs[e] = val;
    ks.add(ct::fmul(dv, dv));
  }
  }
  return ks;
}

// In the solve graph (use_dirty != 0) k_rhs also sets the condition of the
// iteration's projection node (a conditional IF node): run the projections of
// x only when CG moved x since lhs(x) and A x were last computed.
template <int ND>
__global__ void __launch_bounds__(NT)
    k_rhs(const float* __restrict__ atyc, const float* __restrict__ z, const float* __restrict__ u,
          const float* __restrict__ dz, float* __restrict__ rhs, Shape3 sh, size_t N, TermParams tp,
          double* __restrict__ slots, double* __restrict__ partials, unsigned int* __restrict__ ticket,
          int vec, cudaGraphConditionalHandle dirty, int use_dirty, unsigned int* __restrict__ bar_reset) {
  ct::grid_dep_wait();  // before any global access (dependent launch)
  ct::grid_dep_trigger();
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    if (use_dirty) cudaGraphSetConditional(dirty, slots[S_XCLEAN] == 0.0 ? 1u : 0u);
    if (bar_reset) {  // the grid barrier counters of this iteration's cooperative kernels
      bar_reset[0] = 0u;  // k_init_ffwd
      bar_reset[1] = 0u;  // k_cg_step: counter and the next launch's base
      bar_reset[2] = 0u;
    }
  }
  ct::KSum ks = rhs_pass<ND, LdPlain>(atyc, z, u, dz, rhs, sh, N, tp, vec);
  double acc[1] = {ks.value()};
  double tot[1];
  if (ct::grid_sumk_last<NT, 1>(acc, partials, ticket, tot)) slots[S_DUAL2] = tot[0];
}

__global__ void __launch_bounds__(NT)
    k_resid2(const float* __restrict__ sino, const float* __restrict__ y, size_t n,
             double* __restrict__ slots, double* __restrict__ partials, unsigned int* __restrict__ ticket,
             int vec) {
  ct::grid_dep_wait();  // before any global access (dependent launch)
  ct::grid_dep_trigger();
  if (slots[S_XCLEAN] != 0.0) return;  // x unchanged: S_RESID2 is current
  ct::KSum ks;
  if (vec) {
    // two quads per step for more loads in flight
    const size_t stride = 4 * (size_t)gridDim.x * NT;
    for (size_t e0 = 4 * ((size_t)blockIdx.x * NT + threadIdx.x); e0 < n; e0 += 2 * stride) {
      const bool two = e0 + stride < n;
      float a[4], b[4], a2[4], b2[4];
      unpack4(ld4(y, e0), a);
      unpack4(ld4(sino, e0), b);
      if (two) {
        unpack4(ld4(y, e0 + stride), a2);
        unpack4(ld4(sino, e0 + stride), b2);
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const float d = ct::fsub(a[j], b[j]);
        ks.add(ct::fmul(d, d));
      }
      if (two) {
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const float d = ct::fsub(a2[j], b2[j]);
          ks.add(ct::fmul(d, d));
        }
      }
    }
  } else {
    for (size_t e = (size_t)blockIdx.x * NT + threadIdx.x; e < n; e += (size_t)gridDim.x * NT) {
      const float d = ct::fsub(y[e], sino[e]);
      ks.add(ct::fmul(d, d));
    }
  }
  double acc[1] = {ks.value()};
  double tot[1];
  if (ct::grid_sumk_last<NT, 1>(acc, partials, ticket, tot)) slots[S_RESID2] = tot[0];
}

// Where and how the itstat records are written.
struct RecParams {
  double* itstat;
  int max_records;
  double scale, lam21, lam1;
};

// Writes the itstat record of the previous iteration (if there is one), from
// the slots and the CG scalars as that iteration left them (one thread).
__device__ __forceinline__ void write_record(const RecParams& rp, double* __restrict__ slots) {
  if (slots[S_HAVE_PREV] == 0.0) return;
  const int rec = (int)slots[S_REC];
  if (rp.itstat && rec < rp.max_records) {
    double* o = rp.itstat + (size_t)rec * CT_ITSTAT_FIELDS;
    const double* cg = slots + S_CG;
    o[CT_ITSTAT_OBJECTIVE] = rp.scale * slots[S_RESID2] + rp.lam21 * slots[S_G21] + rp.lam1 * slots[S_G1];
    o[CT_ITSTAT_PRIMAL] = sqrt(slots[S_PRIMAL2]);
    o[CT_ITSTAT_DUAL] = sqrt(slots[S_DUAL2]);
    o[CT_ITSTAT_CG_ITERS] = cg[CT_CG_ITERS];
    o[CT_ITSTAT_CG_RELRES] = sqrt(cg[CT_CG_NUM]) / cg[CT_CG_BNORM];
    o[5] = 0.0;
    o[6] = 0.0;
    o[7] = 0.0;
  }
  slots[S_REC] = (double)(rec + 1);
}

// The last record of a call (the statistics epilogue).
__global__ void k_itstat_final(RecParams rp, double* __restrict__ slots) {
  ct::grid_dep_wait();  // before any global access (dependent launch)
  ct::grid_dep_trigger();
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  write_record(rp, slots);
  slots[S_HAVE_PREV] = 0.0;
}

// k_lhs_finish's pass over the elements (see there); acc: this thread's
// shares of ||r||^2, ||rhs||^2 (INIT) or <q, Ap> (acc[0]).
template <int ND, bool INIT, class LD>
__device__ __forceinline__ void lhs_pass(const float* adj, int nsplit, const float* q, const Shape3& sh, size_t N,
                                         const TermParams& tp, float* out, const float* rhs, float* p, float* lhsx,
                                         bool cached, int vec, double (&acc)[2]) {
  if (vec) {
    for (size_t e0 = 4 * ((size_t)blockIdx.x * NT + threadIdx.x); e0 < N; e0 += 4 * (size_t)gridDim.x * NT) {
      float v[4], qc[4];
      if (!INIT || !cached) unpack4(LD::q(q + e0), qc);
      if (cached) {
        unpack4(LD::q(lhsx + e0), v);
      } else {
        float4 a4 = LD::q(adj + e0);
        for (int k = 1; k < nsplit; ++k) {
          const float4 w = LD::q(adj + (size_t)k * N + e0);
          a4 = make_float4(ct::fadd(a4.x, w.x), ct::fadd(a4.y, w.y), ct::fadd(a4.z, w.z), ct::fadd(a4.w, w.w));
        }
        float a[4];
        unpack4(a4, a);
        int c[ND];
        coords<ND>(e0, sh, c);
        float g[4];
        dtd_at4<ND>(q, qc, c, e0, sh, g);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          float vj = ct::fmul(tp.rho, g[j]);
          for (int t = 1; t < tp.ng; ++t) vj = ct::fadd(vj, ct::fmul(tp.rho, g[j]));
          v[j] = ct::fadd(vj, ct::fmul(tp.c, a[j]));
        }
        if (INIT) st4(lhsx, e0, v);
      }
      if (INIT) {
        float b[4], re[4];
        unpack4(LD::q(rhs + e0), b);
#pragma unroll
        for (int j = 0; j < 4; ++j) re[j] = ct::fsub(b[j], v[j]);
        st4(out, e0, re);  // r
        st4(p, e0, re);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          acc[0] += (double)re[j] * (double)re[j];
          acc[1] += (double)b[j] * (double)b[j];
        }
      } else {
        st4(out, e0, v);  // Ap
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[0] += (double)qc[j] * (double)v[j];
      }
    }
  } else {
  for (size_t e = (size_t)blockIdx.x * NT + threadIdx.x; e < N; e += (size_t)gridDim.x * NT) {
    float v;
    if (cached) {
      v = LD::s(lhsx + e);
    } else {
      float a = LD::s(adj + e);
      for (int k = 1; k < nsplit; ++k) a = ct::fadd(a, LD::s(adj + (size_t)k * N + e));
      int c[ND];
      coords<ND>(e, sh, c);
      const float g = dtd_at<ND>(q, c, e, sh);
      v = ct::fmul(tp.rho, g);
      for (int t = 1; t < tp.ng; ++t) v = ct::fadd(v, ct::fmul(tp.rho, g));
      v = ct::fadd(v, ct::fmul(tp.c, a));
      if (INIT) lhsx[e] = v;
    }
    if (INIT) {
      const float b = LD::s(rhs + e);
      const float re = ct::fsub(b, v);
      out[e] = re;  // r
      p[e] = re;
      acc[0] += (double)re * (double)re;
      acc[1] += (double)b * (double)b;
    } else {
      out[e] = v;  // Ap
      acc[0] += (double)LD::s(q + e) * (double)v;
    }
  }
  }
}

// lhs(q) = sum_i rho D^T D q + c A^T A q, from the adjoint output (or its
// view splits).  INIT (q = x): r = rhs - lhs(x), p = r and the CG start
// scalars; lhs(x) is stored in lhsx, or read from it while x is unchanged
// (slots[S_XCLEAN]); before the CG scalars are reset the last block writes
// the previous iteration's itstat record.  PAP: Ap = lhs(q) and <q, Ap>.  In
// a graph with a conditional CG loop, INIT sets the loop condition.
template <int ND, bool INIT>
__global__ void __launch_bounds__(NT)
    k_lhs_finish(const float* __restrict__ adj, int nsplit, const float* __restrict__ q, Shape3 sh,
                 size_t N, TermParams tp, float* __restrict__ out, const float* __restrict__ rhs,
                 float* __restrict__ p, float* __restrict__ lhsx, double* __restrict__ slots,
                 double* __restrict__ cg, double tol, double atol, int maxiter,
                 double* __restrict__ partials, unsigned int* __restrict__ ticket,
                 cudaGraphConditionalHandle cond, int use_cond, int vec, RecParams rp) {
  ct::grid_dep_wait();  // before any global access (dependent launch)
  ct::grid_dep_trigger();
  if (!INIT && cg[CT_CG_DONE] != 0.0) return;
  const bool cached = INIT && slots[S_XCLEAN] != 0.0;
  double acc[2] = {0.0, 0.0};
  lhs_pass<ND, INIT, LdPlain>(adj, nsplit, q, sh, N, tp, out, rhs, p, lhsx, cached, vec, acc);
  double tot[2];
  if (ct::grid_sumk_last<NT, 2>(acc, partials, ticket, tot)) {
    if (INIT) {
      write_record(rp, slots);
      const double bn = sqrt(tot[1]);
      const double thr = fmax(tol * bn, atol);
      cg[CT_CG_NUM] = tot[0];
      cg[CT_CG_PAP] = 0.0;
      cg[CT_CG_ALPHA] = 0.0;
      cg[CT_CG_BETA] = 0.0;
      cg[CT_CG_BNORM] = bn;
      cg[CT_CG_TOL2] = thr * thr;
      cg[CT_CG_ITERS] = 0.0;
      cg[CT_CG_MAXITER] = (double)maxiter;
      cg[CT_CG_RAN] = 0.0;
      const bool done = maxiter <= 0 || !(tot[0] > thr * thr);
      cg[CT_CG_DONE] = done ? 1.0 : 0.0;
      slots[S_XCLEAN] = 1.0;
      if (use_cond) cudaGraphSetConditional(cond, done ? 0u : 1u);
    } else {
      cg[CT_CG_PAP] = tot[0];
    }
  }
}

// prox of one g term over the ND difference components of one element
// (L21Norm._prox / L1Norm.prox, scico/functional/_norm.py; threshold
// lam/rho in float32, _functional.py:198).
template <int ND>
__device__ __forceinline__ void prox_nd(int kind, float thr, const float (&v)[ND], float (&z)[ND]) {
  if (kind == 0) {  // L2,1 over the difference components
    float s2 = ct::fmul(v[0], v[0]);
#pragma unroll
    for (int k = 1; k < ND; ++k) s2 = ct::fadd(s2, ct::fmul(v[k], v[k]));
    const float len = __fsqrt_rn(s2);
    float nl = ct::fsub(len, thr);
    nl = ct::fmul(0.5f, ct::fadd(nl, fabsf(nl)));
#pragma unroll
    for (int k = 0; k < ND; ++k) z[k] = ct::fmul(nl, len != 0.0f ? __fdiv_rn(v[k], len) : 0.0f);
  } else {  // L1
#pragma unroll
    for (int k = 0; k < ND; ++k) {
      float t = ct::fsub(fabsf(v[k]), thr);
      t = ct::fmul(0.5f, ct::fadd(t, fabsf(t)));
      const float sg = v[k] > 0.0f ? 1.0f : (v[k] < 0.0f ? -1.0f : (v[k] == 0.0f ? 0.0f : v[k]));
      z[k] = ct::fmul(sg, t);
    }
  }
}

// z/u update of one element from its differences d (k_zu's body).
// zi, ui: the state read; z, u, dz: where the new state goes (the same
// arrays for the in-place update).
template <int ND, class LD = LdPlain>
__device__ __forceinline__ void zu_el(const float (&d)[ND], const float* zi, const float* ui, float* z, float* u,
                                      float* dz, size_t e, size_t N, const TermParams& tp, ct::KSum (&acc)[3]) {
  for (int t = 0; t < tp.ng; ++t) {
    const size_t o = (size_t)t * ND * N;
    float zo[ND], v[ND], zn[ND];
#pragma unroll
    for (int k = 0; k < ND; ++k) {
      zo[k] = LD::s(zi + o + k * N + e);
      float ck = d[k];
      if (tp.alpha != 1.0f) {
        const float om = ct::fsub(1.0f, tp.alpha);
        ck = ct::fadd(ct::fmul(tp.alpha, d[k]), ct::fmul(om, zo[k]));
      }
      v[k] = ct::fadd(ck, LD::s(ui + o + k * N + e));
    }
    prox_nd<ND>(tp.kind[t], tp.thr[t], v, zn);
    float pr = 0.0f;
#pragma unroll
    for (int k = 0; k < ND; ++k) {
      z[o + k * N + e] = zn[k];
      u[o + k * N + e] = ct::fsub(v[k], zn[k]);
      dz[o + k * N + e] = ct::fsub(zn[k], zo[k]);
      const float pk = ct::fsub(d[k], zn[k]);
      pr = k == 0 ? ct::fmul(pk, pk) : ct::fadd(pr, ct::fmul(pk, pk));
    }
    acc[0].add(ct::fmul(tp.rho, pr));
    if (tp.kind[t] == 0) {
      float s2 = ct::fmul(zn[0], zn[0]);
#pragma unroll
      for (int k = 1; k < ND; ++k) s2 = ct::fadd(s2, ct::fmul(zn[k], zn[k]));
      acc[1].add(__fsqrt_rn(s2));
    } else {
      float a1 = fabsf(zn[0]);
#pragma unroll
      for (int k = 1; k < ND; ++k) a1 = ct::fadd(a1, fabsf(zn[k]));
      acc[2].add(a1);
    }
  }
}

// z/u update of the quad at e0: the state arrays move in 128-bit loads and
// stores, the arithmetic is zu_el's per element, elements in order.
template <int ND, class LD = LdPlain>
__device__ __forceinline__ void zu_quad(const float (&d)[ND][4], const float* zi, const float* ui, float* z,
                                        float* u, float* dz, size_t e0, size_t N, const TermParams& tp,
                                        ct::KSum (&acc)[3]) {
  for (int t = 0; t < tp.ng; ++t) {
    const size_t o = (size_t)t * ND * N;
    float zo[ND][4], uo[ND][4];
#pragma unroll
    for (int k = 0; k < ND; ++k) {
      unpack4(LD::q(zi + o + k * N + e0), zo[k]);
      unpack4(LD::q(ui + o + k * N + e0), uo[k]);
    }
    float zn4[ND][4], un4[ND][4], dz4[ND][4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      float v[ND], zn[ND];
#pragma unroll
      for (int k = 0; k < ND; ++k) {
        float ck = d[k][j];
        if (tp.alpha != 1.0f) {
          const float om = ct::fsub(1.0f, tp.alpha);
          ck = ct::fadd(ct::fmul(tp.alpha, d[k][j]), ct::fmul(om, zo[k][j]));
        }
        v[k] = ct::fadd(ck, uo[k][j]);
      }
      prox_nd<ND>(tp.kind[t], tp.thr[t], v, zn);
      float pr = 0.0f;
#pragma unroll
      for (int k = 0; k < ND; ++k) {
        zn4[k][j] = zn[k];
        un4[k][j] = ct::fsub(v[k], zn[k]);
        dz4[k][j] = ct::fsub(zn[k], zo[k][j]);
        const float pk = ct::fsub(d[k][j], zn[k]);
        pr = k == 0 ? ct::fmul(pk, pk) : ct::fadd(pr, ct::fmul(pk, pk));
      }
      acc[0].add(ct::fmul(tp.rho, pr));
      if (tp.kind[t] == 0) {
        float s2 = ct::fmul(zn[0], zn[0]);
#pragma unroll
        for (int k = 1; k < ND; ++k) s2 = ct::fadd(s2, ct::fmul(zn[k], zn[k]));
        acc[1].add(__fsqrt_rn(s2));
      } else {
        float a1 = fabsf(zn[0]);
#pragma unroll
        for (int k = 1; k < ND; ++k) a1 = ct::fadd(a1, fabsf(zn[k]));
        acc[2].add(a1);
      }
    }
#pragma unroll
    for (int k = 0; k < ND; ++k) {
      st4(z + o + k * N, e0, zn4[k]);
      st4(u + o + k * N, e0, un4[k]);
      st4(dz + o + k * N, e0, dz4[k]);
    }
  }
}

// k_zu's pass over the elements: z, u (and dz = z - z_old) of every term
// from D x; ks: this thread's shares of the primal residual and the g norms.
// x is not written while the pass runs.
template <int ND, class LD>
__device__ __forceinline__ void zu_pass(const float* __restrict__ x, const float* zi, const float* ui, float* z,
                                        float* u, float* dz, const Shape3& sh, size_t N, const TermParams& tp,
                                        int vec, ct::KSum (&ks)[3]) {
  if (vec) {
    for (size_t e0 = 4 * ((size_t)blockIdx.x * NT + threadIdx.x); e0 < N; e0 += 4 * (size_t)gridDim.x * NT) {
      int c[ND];
      coords<ND>(e0, sh, c);
      float xc[4], d[ND][4];
      unpack4(ld4(x, e0), xc);
      d_at4<ND>(x, xc, c, e0, sh, d);
      zu_quad<ND, LD>(d, zi, ui, z, u, dz, e0, N, tp, ks);
    }
  } else {
    for (size_t e = (size_t)blockIdx.x * NT + threadIdx.x; e < N; e += (size_t)gridDim.x * NT) {
      int c[ND];
      coords<ND>(e, sh, c);
      float d[ND];
      d_at<ND>(x, c, e, sh, d);
      zu_el<ND, LD>(d, zi, ui, z, u, dz, e, N, tp, ks);
    }
  }
}

// In the solve graph (use_loop != 0) the last block also ends the iteration:
// it counts it and keeps the graph's iteration loop (a conditional WHILE
// node) running while fewer than maxiter iterations have run.
template <int ND>
__global__ void __launch_bounds__(NT)
    k_zu(const float* __restrict__ x, float* __restrict__ z, float* __restrict__ u, float* __restrict__ dz,
         Shape3 sh, size_t N, TermParams tp, double* __restrict__ slots, double* __restrict__ partials,
         unsigned int* __restrict__ ticket, int vec, cudaGraphConditionalHandle loop, int use_loop,
         int maxiter) {
  ct::grid_dep_wait();  // before any global access (dependent launch)
  ct::grid_dep_trigger();
  if (slots[S_ZU_DONE] != 0.0) {  // uniform: the iterations of this call are complete
    if (use_loop && blockIdx.x == 0 && threadIdx.x == 0) cudaGraphSetConditional(loop, 0u);
    return;
  }
  ct::KSum ks[3];  // primal, g21, g1
  zu_pass<ND, LdPlain>(x, z, u, z, u, dz, sh, N, tp, vec, ks);
  double acc[3] = {ks[0].value(), ks[1].value(), ks[2].value()};
  double tot[3];
  if (ct::grid_sumk_last<NT, 3>(acc, partials, ticket, tot)) {
    slots[S_PRIMAL2] = tot[0];
    slots[S_G21] = tot[1];
    slots[S_G1] = tot[2];
    slots[S_HAVE_PREV] = 1.0;
    if (slots[S_CG + CT_CG_ITERS] > 0.0) slots[S_XCLEAN] = 0.0;  // CG moved x
    if (use_loop) {
      const double it = slots[S_ITER] + 1.0;
      slots[S_ITER] = it;
      cudaGraphSetConditional(loop, it < (double)maxiter ? 1u : 0u);
    }
  }
}

__global__ void k_reset_call(double* __restrict__ slots) {
  ct::grid_dep_wait();  // before any global access (dependent launch)
  ct::grid_dep_trigger();
  slots[S_REC] = 0.0;
  slots[S_HAVE_PREV] = 0.0;
  slots[S_XCLEAN] = 0.0;  // the caller may have changed x between calls
  slots[S_ITER] = 0.0;
  slots[S_ZU_DONE] = 0.0;
}

// ---------------------------------------------------------------------------
// Fast-forward CG start.  In the 512^2 / 360-view solve (lambda 0.005,
// rho 2, CG <= 10) the CG stopping test passes at the first step from
// about the 12th iteration on: x stops moving and each remaining
// iteration is only the z/u update, the next right-hand side and the CG
// start -- three reducing passes of microseconds each, which as separate
// graph nodes cost more in launches and reduction tails than in work.
// k_init_ffwd replaces k_lhs_finish<INIT> in the solve graph: a cooperative
// launch (every block resident) that runs the CG start and, for as long as
// CG would run no step, the following iterations, one grid barrier per
// iteration.  In one phase each thread computes, for its own elements, the
// iteration's rhs (from the neighbours' z, u, dz, made visible by the last
// barrier), the CG start, and the z/u update speculatively into the other
// of two state buffers; after the barrier every block reads the CG start's
// sums: if CG has a step to run, the speculative update is dropped and the
// kernel returns (the CG loop's condition set); otherwise it is committed
// (its statistics written) and the next phase reads the other buffer.  At
// exit the current state is copied back into the primary buffers if it is
// in the second.  Each pass is the separate kernel's own pass (the same
// per-thread elements, per-block partials and partial sums in the same
// order), so the iterates, the CG step counts and the itstat records are
// bit-identical to the separate kernels'.  It returns when CG has a step to
// run or when the call's last iteration is done (S_ZU_DONE: the z/u kernel
// that follows in the graph then only ends the loop).
// ---------------------------------------------------------------------------
constexpr int kErrBarrier = 8;  // error-word bit: a grid barrier wait ran out
// Partials of the fast-forward kernel: per block and phase the six sums
// [CG start ||r||^2, ||rhs||^2, dual residual, z/u primal, g21, g1], reduced
// over the block in one pass (each sum by the same tree as alone); two sets
// alternating by phase.
constexpr int kFfK = 6, kFfInit = 0, kFfDual = 2, kFfZu = 3, kFfSet = kFfK * NB;
// ... and those of the fused CG step (k_cg_step): <p, Ap> and <r, r> phases.
constexpr int kCgPart = 2 * kFfSet, kFfDoubles = kCgPart + 4 * NB;

// The state arrays (every term's z, u and dz) of this thread's elements,
// copied from the second buffers to the primary ones.
template <int ND>
__device__ __forceinline__ void copy_state(const float* z2, const float* u2, const float* dz2, float* z, float* u,
                                           float* dz, size_t N, int ng, int vec) {
  const float* src[3] = {z2, u2, dz2};
  float* dst[3] = {z, u, dz};
  for (int a = 0; a < 3; ++a) {
    for (int comp = 0; comp < ng * ND; ++comp) {
      const size_t o = (size_t)comp * N;
      if (vec) {
        for (size_t e0 = 4 * ((size_t)blockIdx.x * NT + threadIdx.x); e0 < N; e0 += 4 * (size_t)gridDim.x * NT)
          *reinterpret_cast<float4*>(dst[a] + o + e0) = LdL2::q(src[a] + o + e0);
      } else {
        for (size_t e = (size_t)blockIdx.x * NT + threadIdx.x; e < N; e += (size_t)gridDim.x * NT)
          dst[a][o + e] = LdL2::s(src[a] + o + e);
      }
    }
  }
}

template <int ND>
__global__ void __launch_bounds__(NT, 2)
    k_init_ffwd(const float* adj, int nsplit, const float* __restrict__ x, Shape3 sh, size_t N, TermParams tp,
                float* r, float* rhs, float* p, float* lhsx, const float* __restrict__ atyc, float* z, float* u,
                float* dz, float* z2, float* u2, float* dz2, double* slots, double* cg, double tol, double atol,
                int cg_maxiter, int maxiter, double* fpart, unsigned int* bar, cudaGraphConditionalHandle cond,
                int vec, RecParams rp, uint32_t max_polls, int* errflag) {
  ct::grid_dep_wait();  // before any global access (dependent launch)
  ct::grid_dep_trigger();
  using LDS = LdL2;  // state written by other blocks earlier in this launch
  __shared__ double dec_s[2];
  // A block whose barrier wait runs out hands over to the graph's CG loop
  // and returns: the solve's results are void (the error word says so), and
  // the fused CG step then ends the loop on its own failed barrier, so every
  // failure path of the solve graph runs in the poll-limit test.
  auto give_up = [&]() {
    if (threadIdx.x == 0) cudaGraphSetConditional(cond, 1u);
  };
  // read by every block before the first barrier; blocks write them only after it
  bool cached = slots[S_XCLEAN] != 0.0;
  int iter = (int)slots[S_ITER];
  const unsigned int last = gridDim.x - 1;
  int cur = 0;  // the current iteration's z, u, dz: 0 = primary buffers, 1 = second buffers
  for (unsigned int phase = 0;; ++phase) {
    double* fp = fpart + (phase & 1u) * kFfSet;
    const float* zc = cur ? z2 : z;
    const float* uc = cur ? u2 : u;
    const float* dzc = cur ? dz2 : dz;
    float* zn = cur ? z : z2;
    float* un = cur ? u : u2;
    float* dzn = cur ? dz : dz2;
    double v6[kFfK];
    v6[kFfDual] = 0.0;
    if (phase > 0) {  // the rhs (k_rhs); the first phase's came from the graph's k_rhs
      ct::KSum kd = rhs_pass<ND, LDS>(atyc, zc, uc, dzc, rhs, sh, N, tp, vec);
      v6[kFfDual] = kd.value();
    }
    // the CG start (k_lhs_finish<INIT>); rhs at the thread's own elements
    double acc[2] = {0.0, 0.0};
    lhs_pass<ND, true, LDS>(adj, nsplit, x, sh, N, tp, r, rhs, p, lhsx, cached, vec, acc);
    v6[kFfInit] = acc[0];
    v6[kFfInit + 1] = acc[1];
    // the z/u update (k_zu, x unchanged), valid if CG runs no step
    ct::KSum ks[3];
    zu_pass<ND, LDS>(x, zc, uc, zn, un, dzn, sh, N, tp, vec, ks);
    for (int k = 0; k < 3; ++k) v6[kFfZu + k] = ks[k].value();
    ct::block_partials<NT, kFfK>(v6, fp);
    if (!ct::grid_barrier(bar, (phase + 1) * gridDim.x, max_polls, errflag, kErrBarrier)) return give_up();
    double tot[2];
    ct::sum_partials<NT, 2>(fp + kFfInit, gridDim.x, tot, kFfK);
    if (threadIdx.x == 0) {
      dec_s[0] = tot[0];
      dec_s[1] = tot[1];
    }
    __syncthreads();
    const double bn = sqrt(dec_s[1]);
    const double thr = fmax(tol * bn, atol);
    const bool done = cg_maxiter <= 0 || !(dec_s[0] > thr * thr);
    if (blockIdx.x == 0) {
      if (phase > 0) {  // k_rhs's total, before the record that reads it
        double d[1];
        ct::sum_partials<NT, 1>(fp + kFfDual, gridDim.x, d, kFfK);
        if (threadIdx.x == 0) slots[S_DUAL2] = d[0];
      }
      if (threadIdx.x == 0) {
        write_record(rp, slots);
        cg[CT_CG_NUM] = dec_s[0];
        cg[CT_CG_PAP] = 0.0;
        cg[CT_CG_ALPHA] = 0.0;
        cg[CT_CG_BETA] = 0.0;
        cg[CT_CG_BNORM] = bn;
        cg[CT_CG_TOL2] = thr * thr;
        cg[CT_CG_ITERS] = 0.0;
        cg[CT_CG_MAXITER] = (double)cg_maxiter;
        cg[CT_CG_RAN] = 0.0;
        cg[CT_CG_DONE] = done ? 1.0 : 0.0;
        slots[S_XCLEAN] = 1.0;
        if (!done) cudaGraphSetConditional(cond, 1u);
      }
    }
    if (!done) {  // uniform: CG runs this iteration's steps in the graph; the update is dropped
      if (cur) copy_state<ND>(z2, u2, dz2, z, u, dz, N, tp.ng, vec);
      return;
    }
    ++iter;  // the update is committed (k_zu's last block)
    if (blockIdx.x == last) {
      double zt[3];
      ct::sum_partials<NT, 3>(fp + kFfZu, gridDim.x, zt, kFfK);
      if (threadIdx.x == 0) {
        slots[S_PRIMAL2] = zt[0];
        slots[S_G21] = zt[1];
        slots[S_G1] = zt[2];
        slots[S_HAVE_PREV] = 1.0;
        slots[S_ITER] = (double)iter;
        if (iter >= maxiter) slots[S_ZU_DONE] = 1.0;
      }
    }
    cur ^= 1;
    cached = true;
    if (iter >= maxiter) {
      if (cur) copy_state<ND>(z2, u2, dz2, z, u, dz, N, tp.ng, vec);
      return;
    }
  }
}

// ---------------------------------------------------------------------------
// Fused CG step of the solve graph: k_lhs_finish<PAP>, k_cg_update and
// k_cg_direction as one cooperative launch with two bounded grid barriers
// (after <p, Ap> and after <r, r>), the projections of p staying separate
// kernels before it.  vec / vec_update / vec_dir: each pass's quad flag as
// its separate kernel takes it (the stencil pass needs the last axis in
// quads, the vector passes only the flat length and alignment).  Each thread updates only its own elements in the
// three passes (the same element mapping in all three), so the barriers
// carry only the two sums; the passes and sums are the separate kernels'
// own, so the iterates are bit-identical.  The barrier counter grows by two
// grids per launch from 0 (reset by the iteration's k_rhs); bar[2] holds the
// next launch's base.
// ---------------------------------------------------------------------------
template <int ND>
__global__ void __launch_bounds__(NT, 2)
    k_cg_step(const float* adj, int nsplit, float* p, Shape3 sh, size_t N, TermParams tp, float* ap, float* x,
              float* r, double* cg, double* part, unsigned int* bar, cudaGraphConditionalHandle cond, int vec,
              int vec_update, int vec_dir, uint32_t max_polls, int* errflag) {
  ct::grid_dep_wait();  // before any global access (dependent launch)
  ct::grid_dep_trigger();
  __shared__ double sum_s;
  // read by every block before the first barrier; block 0 writes them only after the second
  const double num = cg[CT_CG_NUM], it0 = cg[CT_CG_ITERS];
  const double tol2 = cg[CT_CG_TOL2], maxit = cg[CT_CG_MAXITER];
  const unsigned int base = bar[2];
  if (cg[CT_CG_DONE] != 0.0) {  // uniform (the graph's CG loop only runs while not done)
    if (blockIdx.x == 0 && threadIdx.x == 0) cudaGraphSetConditional(cond, 0u);
    return;
  }
  // A block whose barrier wait runs out ends the graph's CG loop (the error
  // bit is set): the loop then cannot run on with a condition that no block
  // of this launch cleared.  The loop continues only where block 0 passed
  // both barriers, which also counts the step, so it ends by cg_maxiter.
  auto give_up = [&]() {
    if (threadIdx.x == 0) {
      cg[CT_CG_DONE] = 1.0;
      cudaGraphSetConditional(cond, 0u);
    }
  };
  // Ap = lhs(p) and <p, Ap> (k_lhs_finish<PAP>)
  double acc[2] = {0.0, 0.0};
  lhs_pass<ND, false, LdPlain>(adj, nsplit, p, sh, N, tp, ap, nullptr, nullptr, nullptr, false, vec, acc);
  ct::block_partials<NT, 2>(acc, part);
  if (!ct::grid_barrier(bar + 1, base + gridDim.x, max_polls, errflag, kErrBarrier)) return give_up();
  double t[2];
  ct::sum_partials<NT, 2>(part, gridDim.x, t);
  if (threadIdx.x == 0) sum_s = t[0];
  __syncthreads();
  const double pap = sum_s;
  const double alpha = num / pap;
  // x += alpha p; r -= alpha Ap; <r, r> (k_cg_update)
  double v2[2] = {ct::cg_update_pass(x, r, p, ap, N, (float)alpha, vec_update), 0.0};
  ct::block_partials<NT, 2>(v2, part + 2 * NB);
  if (!ct::grid_barrier(bar + 1, base + 2 * gridDim.x, max_polls, errflag, kErrBarrier)) return give_up();
  ct::sum_partials<NT, 2>(part + 2 * NB, gridDim.x, t);
  if (threadIdx.x == 0) sum_s = t[0];
  __syncthreads();
  const double trr = sum_s;
  const double beta = trr / num;
  const double it = it0 + 1.0;
  const bool done = !(trr > tol2) || it >= maxit;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    cg[CT_CG_PAP] = pap;
    cg[CT_CG_ALPHA] = alpha;
    cg[CT_CG_NUM] = trr;
    cg[CT_CG_BETA] = beta;
    cg[CT_CG_ITERS] = it;
    cg[CT_CG_RAN] = 0.0;  // the direction update runs in this launch
    if (done) cg[CT_CG_DONE] = 1.0;
    bar[2] = base + 2 * gridDim.x;
    cudaGraphSetConditional(cond, done ? 0u : 1u);
  }
  // p = r + beta p (k_cg_direction): the direction update still runs in the
  // step that finds CG done (reference order)
  ct::cg_direction_pass(p, r, N, (float)beta, vec_dir);
}

// ---------------------------------------------------------------------------

// Solver parameters common to the 2D and 3D descriptors.
struct Params {
  int maxiter, cg_maxiter;
  double cg_tol, cg_atol, lam_l21, lam_l1, rho, loss_scale, alpha;
  int use_graph;
};

template <class D>
Params params_of(const D* d) {
  return Params{d->maxiter, d->cg_maxiter, d->cg_tol,     d->cg_atol,
                d->lam_l21, d->lam_l1,     d->rho,        d->loss_scale,
                d->alpha,   d->use_graph};
}

// The forward/adjoint pair behind A: the 2D or the 3D projector.
struct Projector {
  int nd = 2;
  const ct_geom2d* g2 = nullptr;
  const ct_geom3d* g3 = nullptr;
  ct::Proj2dPlan p2{};
  ct::Proj3dPlan p3{};
  size_t fwd_bytes() const { return nd == 2 ? p2.fwd_bytes : p3.fwd_ws_bytes; }
  // split area to reserve: the largest any recorded 2D schedule may use
  size_t adj_ws_bytes() const { return nd == 2 ? p2.adj_ws_bytes : p3.adj_ws_bytes; }
  int nsplit() const { return nd == 2 ? p2.nsplit : p3.nsplit; }
  ct_status prepare() const { return nd == 2 ? ct::proj2d_prepare(p2) : ct::proj3d_prepare(g3, p3); }
  ct_status fwd(const float* img, float* sino, void* ws, cudaStream_t s, const double* skip,
                bool dependent = false) const {
    return nd == 2 ? ct::proj2d_fwd_launch(g2, p2, img, sino, 1, static_cast<float*>(ws), s, skip, dependent)
                   : ct::proj3d_fwd_launch(g3, p3, img, sino, ws, s, skip);
  }
  // dependent: the 2D adjoint may be launched as the dependent of its stream
  // predecessor, one of this library's kernels
  ct_status adj(const float* sino, float* out, float* part, cudaStream_t s, const double* skip,
                bool dependent = false) const {
    return nd == 2 ? ct::proj2d_adj_launch(g2, p2, sino, out, part, 1, s, skip, dependent)
                   : ct::proj3d_adj_launch(g3, p3, sino, out, part, s, skip);
  }
};

// One problem: descriptor bytes (for the graph cache key), parameters,
// image shape and projector.
struct Problem {
  const void* desc = nullptr;
  size_t desc_size = 0;
  Params prm{};
  Shape3 sh{};
  int nd = 2;
  size_t N = 0, S = 0;
  Projector proj;
};

Problem problem_of(const ct_admm_tv_desc* d) {
  Problem P;
  P.desc = d;
  P.desc_size = sizeof(*d);
  P.prm = params_of(d);
  P.nd = 2;
  P.sh.n[0] = d->geom.rows;
  P.sh.n[1] = d->geom.cols;
  P.sh.n[2] = 1;
  P.N = (size_t)d->geom.rows * d->geom.cols;
  P.S = (size_t)d->geom.n_views * d->geom.det_count;
  P.proj.nd = 2;
  P.proj.g2 = &d->geom;
  P.proj.p2 = ct::proj2d_plan(&d->geom, 1);
  return P;
}

Problem problem_of(const ct_admm_tv3d_desc* d) {
  Problem P;
  P.desc = d;
  P.desc_size = sizeof(*d);
  P.prm = params_of(d);
  P.nd = 3;
  for (int k = 0; k < 3; ++k) P.sh.n[k] = d->geom.shape[k];
  P.N = (size_t)d->geom.shape[0] * d->geom.shape[1] * d->geom.shape[2];
  P.S = (size_t)d->geom.n_views * d->geom.det_shape[0] * d->geom.det_shape[1];
  P.proj.nd = 3;
  P.proj.g3 = &d->geom;
  P.proj.p3 = ct::proj3d_plan(&d->geom, 1);
  return P;
}

struct Layout {
  int ng;
  size_t off_slots, off_red, off_atyc, off_rhs, off_r, off_p, off_ap, off_adj, off_sino, off_z, off_u,
      off_dz, off_fwd, off_adjpart, off_lhsx, off_sinox, off_ff, off_z2, off_u2, off_dz2, total;
};

Layout layout(const Problem& P) {
  Layout L;
  L.ng = (P.prm.lam_l21 != 0.0) + (P.prm.lam_l1 != 0.0);
  size_t o = 0;
  auto take = [&](size_t bytes) {
    const size_t at = o;
    o += ct::round_up(bytes, 256);
    return at;
  };
  const size_t zbytes = P.N * 4 * (size_t)P.nd * (size_t)(L.ng > 0 ? L.ng : 1);
  L.off_slots = take(S_COUNT * sizeof(double));
  L.off_red = take(ct::kReduceWorkspace);
  L.off_atyc = take(P.N * 4);
  L.off_rhs = take(P.N * 4);
  L.off_r = take(P.N * 4);
  L.off_p = take(P.N * 4);
  L.off_ap = take(P.N * 4);
  L.off_adj = take(P.N * 4);
  L.off_sino = take(P.S * 4);
  L.off_z = take(zbytes);
  L.off_u = take(zbytes);
  L.off_dz = take(zbytes);
  L.off_fwd = take(P.proj.fwd_bytes() > 0 ? P.proj.fwd_bytes() : 256);
  L.off_adjpart = take(P.proj.adj_ws_bytes() > 0 ? P.proj.adj_ws_bytes() : 256);
  L.off_lhsx = take(P.N * 4);
  L.off_sinox = take(P.S * 4);
  L.off_ff = take(256 + sizeof(double) * kFfDoubles);  // barrier counter, then the partials
  L.off_z2 = take(zbytes);  // the fast-forward kernel's second state buffers
  L.off_u2 = take(zbytes);
  L.off_dz2 = take(zbytes);
  L.total = o;
  return L;
}

ct_status check_params(const Params& p, const char* who) {
  if (p.maxiter < 0 || p.cg_maxiter < 0)
    return ct::fail(CT_ERR_INVALID_ARG, "%s: maxiter=%d cg_maxiter=%d", who, p.maxiter, p.cg_maxiter);
  if ((p.lam_l21 != 0.0) + (p.lam_l1 != 0.0) == 0)
    return ct::fail(CT_ERR_INVALID_ARG, "%s: at least one of lam_l21, lam_l1 must be non-zero", who);
  if (!(p.rho > 0.0)) return ct::fail(CT_ERR_INVALID_ARG, "%s: rho must be > 0", who);
  return CT_OK;
}

ct_status check_desc(const ct_admm_tv_desc* d, const char* who) {
  if (!d) return ct::fail(CT_ERR_INVALID_ARG, "%s: null descriptor", who);
  ct_status st = ct::proj2d_check(&d->geom, who);
  if (st != CT_OK) return st;
  return check_params(params_of(d), who);
}

ct_status check_desc(const ct_admm_tv3d_desc* d, const char* who) {
  if (!d) return ct::fail(CT_ERR_INVALID_ARG, "%s: null descriptor", who);
  ct_status st = ct::proj3d_check(&d->geom, who);
  if (st != CT_OK) return st;
  return check_params(params_of(d), who);
}

struct Ctx {
  Problem P;
  Layout L;
  char* ws;
  const float* y;
  float* x;
  double* itstat;
  TermParams tp;
  int vi;  // image-sized kernels take the quad path (last axis % 4 == 0, x 16-B aligned)
  int vs;  // sinogram-sized kernels take the quad path (size % 4 == 0, y 16-B aligned)
  template <class T>
  T* at(size_t off) const { return reinterpret_cast<T*>(ws + off); }
  double* slots() const { return at<double>(L.off_slots); }
  double* cg() const { return slots() + S_CG; }
  unsigned int* ticket() const { return at<unsigned int>(L.off_red); }
  double* partials() const { return reinterpret_cast<double*>(ws + L.off_red + 256); }
  unsigned int* ff_bar() const { return at<unsigned int>(L.off_ff); }
  double* ff_part() const { return reinterpret_cast<double*>(ws + L.off_ff + 256); }
  bool ffwd = false;  // the solve graph's CG start is k_init_ffwd
};

#define CT_TRY(expr)                 \
  do {                               \
    ct_status _st = (expr);          \
    if (_st != CT_OK) return _st;    \
  } while (0)

// Launch the ND instance of a templated kernel for the problem's dimension.
#define CT_LAUNCH_ND(nd, kernel, grid, block, stream, ...)                 \
  do {                                                                     \
    if ((nd) == 2)                                                         \
      kernel<2><<<(grid), (block), 0, (stream)>>>(__VA_ARGS__);            \
    else                                                                   \
      kernel<3><<<(grid), (block), 0, (stream)>>>(__VA_ARGS__);            \
  } while (0)

// Inside a solve every kernel follows one of this library's kernels: the
// solver's launches are dependent ones (launch_k in common.cuh).
ct_status project(const Ctx& c, const float* img, float* sino, cudaStream_t s, const double* skip) {
  return c.P.proj.fwd(img, sino, c.at<float>(c.L.off_fwd), s, skip, true);
}

// A^T of a sinogram into the adjoint buffer (or its view splits); returns
// the buffer to read.
const float* backproject(const Ctx& c, const float* sino, cudaStream_t s, const double* skip, ct_status& st,
                         bool dependent = false) {
  float* adj = c.at<float>(c.L.off_adj);
  float* part = c.at<float>(c.L.off_adjpart);
  st = c.P.proj.adj(sino, adj, part, s, skip, dependent);
  return c.P.proj.nsplit() > 1 ? part : adj;
}

RecParams rec_params(const Ctx& c) {
  return RecParams{c.itstat, c.P.prm.maxiter, c.P.prm.loss_scale, c.P.prm.lam_l21, c.P.prm.lam_l1};
}

// The phases of one ADMM iteration:
//   rhs   k_rhs (with dirty/use_dirty: sets the condition of the graph's
//         projection node)
//   proj  A x, ||A x - y||^2 and A^T (A x) -- each a no-op while x is
//         unchanged (in the solve graph the phase is a conditional IF node
//         that runs only when x changed)
//   init  k_lhs_finish<INIT>: the previous iteration's record, CG start;
//         cond/use_cond: the conditional handle of the graph's CG loop
//   CG    enqueue_cg_step per step
//   post  k_zu (with loop/use_loop: ends the graph's iteration)
ct_status enqueue_rhs(const Ctx& c, cudaStream_t s, cudaGraphConditionalHandle dirty, int use_dirty) {
  auto k = c.P.nd == 2 ? k_rhs<2> : k_rhs<3>;
  return ct::cuda_check(ct::launch_k(k, dim3(NB), dim3(NT), 0, s, true, (const float*)c.at<float>(c.L.off_atyc),
                                     (const float*)c.at<float>(c.L.off_z), (const float*)c.at<float>(c.L.off_u),
                                     (const float*)c.at<float>(c.L.off_dz), c.at<float>(c.L.off_rhs), c.P.sh, c.P.N,
                                     c.tp, c.slots(), c.partials(), c.ticket(), c.vi, dirty, use_dirty,
                                     (c.ffwd && use_dirty) ? c.ff_bar() : (unsigned int*)nullptr),
                        "k_rhs");
}

ct_status enqueue_proj(const Ctx& c, cudaStream_t s) {
  float* sinox = c.at<float>(c.L.off_sinox);
  const double* clean = c.slots() + S_XCLEAN;
  CT_TRY(project(c, c.x, sinox, s, clean));
  // resid2 and the adjoint follow kernels of this library: dependent launches
  CT_TRY(ct::cuda_check(ct::launch_k(k_resid2, dim3(NB), dim3(NT), 0, s, true, (const float*)sinox, c.y, c.P.S,
                                     c.slots(), c.partials(), c.ticket(), c.vs),
                        "k_resid2"));
  ct_status st;
  backproject(c, sinox, s, clean, st, true);
  return st;
}

ct_status enqueue_init(const Ctx& c, cudaStream_t s, cudaGraphConditionalHandle cond, int use_cond) {
  const size_t N = c.P.N;
  const float* adj = c.P.proj.nsplit() > 1 ? c.at<float>(c.L.off_adjpart) : c.at<float>(c.L.off_adj);
  float* r = c.at<float>(c.L.off_r);
  float* p = c.at<float>(c.L.off_p);
  float* rhs = c.at<float>(c.L.off_rhs);
  if (c.ffwd && use_cond) {
    // the fast-forward CG start: a cooperative launch (all NB blocks resident)
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(NB);
    cfg.blockDim = dim3(NT);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const uint32_t polls = std::min<uint32_t>(ct::proj2d_wait_polls(), 1u << 21);
    int* err = ct::proj2d_errflag_ptr();
    if (!err) return ct::fail(CT_ERR_CUDA, "k_init_ffwd: error-word address unavailable");
    auto kf = c.P.nd == 2 ? k_init_ffwd<2> : k_init_ffwd<3>;
    return ct::cuda_check(
        cudaLaunchKernelEx(&cfg, kf, adj, c.P.proj.nsplit(), (const float*)c.x, c.P.sh, N, c.tp, r, rhs, p,
                           c.at<float>(c.L.off_lhsx), (const float*)c.at<float>(c.L.off_atyc), c.at<float>(c.L.off_z),
                           c.at<float>(c.L.off_u), c.at<float>(c.L.off_dz), c.at<float>(c.L.off_z2),
                           c.at<float>(c.L.off_u2), c.at<float>(c.L.off_dz2), c.slots(), c.cg(), c.P.prm.cg_tol,
                           c.P.prm.cg_atol, c.P.prm.cg_maxiter, c.P.prm.maxiter, c.ff_part(), c.ff_bar(), cond, c.vi,
                           rec_params(c), polls, err),
        "k_init_ffwd");
  }
  auto k = c.P.nd == 2 ? k_lhs_finish<2, true> : k_lhs_finish<3, true>;
  return ct::cuda_check(ct::launch_k(k, dim3(NB), dim3(NT), 0, s, true, adj, c.P.proj.nsplit(), (const float*)c.x,
                                     c.P.sh, N, c.tp, r, (const float*)rhs, p, c.at<float>(c.L.off_lhsx), c.slots(),
                                     c.cg(), c.P.prm.cg_tol, c.P.prm.cg_atol, c.P.prm.cg_maxiter, c.partials(),
                                     c.ticket(), cond, use_cond, c.vi, rec_params(c)),
                        "k_lhs_finish<init>");
}

ct_status enqueue_cg_step(const Ctx& c, cudaStream_t s, cudaGraphConditionalHandle cond, int use_cond) {
  const size_t N = c.P.N;
  float* r = c.at<float>(c.L.off_r);
  float* p = c.at<float>(c.L.off_p);
  float* ap = c.at<float>(c.L.off_ap);
  float* sino = c.at<float>(c.L.off_sino);
  const double* done = c.cg() + CT_CG_DONE;
  CT_TRY(project(c, p, sino, s, done));
  // every kernel after the forward's first follows a kernel of this library:
  // dependent launches (launch_k in common.cuh)
  ct_status st;
  const float* adj = backproject(c, sino, s, done, st, true);
  CT_TRY(st);
  if (c.ffwd && use_cond) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(NB);
    cfg.blockDim = dim3(NT);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const uint32_t polls = std::min<uint32_t>(ct::proj2d_wait_polls(), 1u << 21);
    int* err = ct::proj2d_errflag_ptr();
    if (!err) return ct::fail(CT_ERR_CUDA, "k_cg_step: error-word address unavailable");
    auto kf = c.P.nd == 2 ? k_cg_step<2> : k_cg_step<3>;
    return ct::cuda_check(cudaLaunchKernelEx(&cfg, kf, adj, c.P.proj.nsplit(), p, c.P.sh, N, c.tp, ap, c.x, r,
                                             c.cg(), c.ff_part() + kCgPart, c.ff_bar(), cond, c.vi,
                                             ct::quad_ok(N, c.x, r, p, ap), ct::quad_ok(N, p, r), polls, err),
                          "k_cg_step");
  }
  float* nf = nullptr;
  const float* ncf = nullptr;
  auto lhs = c.P.nd == 2 ? k_lhs_finish<2, false> : k_lhs_finish<3, false>;
  CT_TRY(ct::cuda_check(ct::launch_k(lhs, dim3(NB), dim3(NT), 0, s, true, adj, c.P.proj.nsplit(), (const float*)p,
                                     c.P.sh, N, c.tp, ap, ncf, nf, nf, c.slots(), c.cg(), 0.0, 0.0,
                                     c.P.prm.cg_maxiter, c.partials(), c.ticket(), (cudaGraphConditionalHandle)0, 0,
                                     c.vi, RecParams{}),
                        "k_lhs_finish<pap>"));
  CT_TRY(ct::cg_update_launch(c.x, r, p, ap, N, c.cg(), c.ws + c.L.off_red, s, cond, use_cond, true));
  return ct::cg_direction_launch(p, r, N, c.cg(), c.ws + c.L.off_red, s, true);
}

ct_status enqueue_post(const Ctx& c, cudaStream_t s, cudaGraphConditionalHandle loop, int use_loop) {
  auto k = c.P.nd == 2 ? k_zu<2> : k_zu<3>;
  return ct::cuda_check(ct::launch_k(k, dim3(NB), dim3(NT), 0, s, true, (const float*)c.x, c.at<float>(c.L.off_z),
                                     c.at<float>(c.L.off_u), c.at<float>(c.L.off_dz), c.P.sh, c.P.N, c.tp,
                                     c.slots(), c.partials(), c.ticket(), c.vi, loop, use_loop, c.P.prm.maxiter),
                        "k_zu");
}

// One iteration as plain launches (no graph): cg_maxiter CG steps that turn
// into no-ops once CG has converged.
ct_status enqueue_iteration(const Ctx& c, cudaStream_t s) {
  CT_TRY(enqueue_rhs(c, s, 0, 0));
  CT_TRY(enqueue_proj(c, s));
  CT_TRY(enqueue_init(c, s, 0, 0));
  for (int it = 0; it < c.P.prm.cg_maxiter; ++it) CT_TRY(enqueue_cg_step(c, s, 0, 0));
  return enqueue_post(c, s, 0, 0);
}

// Statistics of the last iteration: dual residual (k_rhs), objective.
ct_status enqueue_epilogue(const Ctx& c, cudaStream_t s) {
  float* sinox = c.at<float>(c.L.off_sinox);
  CT_TRY(enqueue_rhs(c, s, 0, 0));
  CT_TRY(project(c, c.x, sinox, s, c.slots() + S_XCLEAN));
  CT_TRY(ct::cuda_check(ct::launch_k(k_resid2, dim3(NB), dim3(NT), 0, s, true, (const float*)sinox, c.y, c.P.S,
                                     c.slots(), c.partials(), c.ticket(), c.vs),
                        "k_resid2"));
  return ct::cuda_check(ct::launch_k(k_itstat_final, dim3(1), dim3(32), 0, s, true, rec_params(c), c.slots()),
                        "k_itstat_final");
}

// The fast-forward CG start (k_init_ffwd): on unless CTGPU_FFWD=0 or
// ct_set_solver_fast_forward(0); used where the device runs cooperative
// launches and all NB blocks of it fit at once.
std::atomic<int> g_ffwd{-1};

bool ffwd_enabled() {
  int v = g_ffwd.load(std::memory_order_relaxed);
  if (v < 0) {
    const char* e = getenv("CTGPU_FFWD");
    v = (e && e[0] == '0') ? 0 : 1;
    g_ffwd.store(v, std::memory_order_relaxed);
  }
  return v != 0;
}

bool ffwd_usable(int nd) {
  if (!ffwd_enabled()) return false;
  int dev = 0, coop = 0, nb = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return false;
  if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop) return false;
  int nc = 0;
  const cudaError_t e = nd == 2 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_init_ffwd<2>, NT, 0)
                                : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_init_ffwd<3>, NT, 0);
  const cudaError_t e2 = nd == 2 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nc, k_cg_step<2>, NT, 0)
                                 : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nc, k_cg_step<3>, NT, 0);
  if (e != cudaSuccess || e2 != cudaSuccess) {
    (void)cudaGetLastError();
    return false;
  }
  return std::min(nb, nc) * ct::sm_count() >= NB;
}

// Executable iteration graphs, one per problem (key: dimension, descriptor
// bytes and the state/data pointers), least recently used evicted.  One
// capture stream per device; graphs are launched on the solve's stream.
constexpr int kMaxGraphs = 256;

struct GraphEntry {
  std::vector<unsigned char> key;
  int device = -1;
  cudaGraphExec_t exec = nullptr;
  unsigned long long last_use = 0;
};

struct GraphCache {
  std::mutex m;
  GraphEntry e[kMaxGraphs];
  unsigned long long clock = 0;
  cudaStream_t capture[64] = {nullptr};
};
GraphCache g_cache;

void make_key(const Ctx& c, int32_t iter0, std::vector<unsigned char>& key) {
  auto put = [&](const void* p, size_t b) {
    const unsigned char* q = static_cast<const unsigned char*>(p);
    key.insert(key.end(), q, q + b);
  };
  const int fresh = iter0 == 0 ? 1 : 0;  // the solve starts from x (state initialised in the graph)
  put(&c.P.nd, sizeof(c.P.nd));
  put(&fresh, sizeof(fresh));
  put(c.P.desc, c.P.desc_size);
  if (c.P.nd == 2) {  // the projector's schedule (the autotuner may record a new one)
    put(&c.P.proj.p2.vpc, sizeof(int));
    put(&c.P.proj.p2.nsplit, sizeof(int));
  }
  const uint32_t polls = ct::proj2d_wait_polls();  // the wait limits captured in the graph
  put(&polls, sizeof(polls));
  const int ff = c.ffwd ? 1 : 0;
  put(&ff, sizeof(ff));
  put(&c.ws, sizeof(c.ws));
  put(&c.y, sizeof(c.y));
  put(&c.x, sizeof(c.x));
  put(&c.itstat, sizeof(c.itstat));
}

// Capture fn(stream) into `graph` after `deps`; the capture's last nodes
// (at most 8) are returned in `tail`.
template <class F>
ct_status capture_into(cudaStream_t cs, cudaGraph_t graph, const std::vector<cudaGraphNode_t>& deps,
                       std::vector<cudaGraphNode_t>& tail, F&& fn) {
  CT_TRY(ct::cuda_check(cudaStreamBeginCaptureToGraph(cs, graph, deps.empty() ? nullptr : deps.data(), nullptr,
                                                      deps.size(), cudaStreamCaptureModeThreadLocal),
                        "begin capture"));
  ct_status st = fn(cs);
  cudaStreamCaptureStatus cst;
  const cudaGraphNode_t* fr = nullptr;
  size_t nfr = 0;
  cudaError_t ce = cudaStreamGetCaptureInfo(cs, &cst, nullptr, nullptr, &fr, nullptr, &nfr);
  tail.clear();
  for (size_t k = 0; ce == cudaSuccess && k < nfr && k < 8; ++k) tail.push_back(fr[k]);
  cudaGraph_t out = nullptr;
  cudaError_t ce2 = cudaStreamEndCapture(cs, &out);
  CT_TRY(st);
  CT_TRY(ct::cuda_check(ce, "capture info"));
  CT_TRY(ct::cuda_check(ce2, "end capture"));
  if (nfr > 8) return ct::fail(CT_ERR_CUDA, "unexpected capture frontier of %zu nodes", nfr);
  return CT_OK;
}

// Conditional node of type `type` on `handle` after `deps` in `graph`; its
// body graph is returned in `body`.
ct_status add_conditional(cudaGraph_t graph, const std::vector<cudaGraphNode_t>& deps,
                          cudaGraphConditionalHandle handle, cudaGraphConditionalNodeType type,
                          cudaGraphNode_t& node, cudaGraph_t& body) {
  cudaGraphNodeParams np = {};
  np.type = cudaGraphNodeTypeConditional;
  np.conditional.handle = handle;
  np.conditional.type = type;
  np.conditional.size = 1;
  CT_TRY(ct::cuda_check(cudaGraphAddNode(&node, graph, deps.empty() ? nullptr : deps.data(), nullptr, deps.size(),
                                         &np),
                        "conditional node"));
  body = np.conditional.phGraph_out[0];
  return CT_OK;
}

// Append one whole solve to `graph`, independent of every other node:
// the state set-up (iter0 == 0) and k_reset_call, then the ADMM loop as a
// conditional WHILE node whose body is one iteration -- k_rhs, the
// projections of x as a conditional IF node (run when CG moved x), the CG
// start, the CG loop as a nested WHILE node (its start and every CG update
// set its condition on the device: run while CG has not converged), and the
// z/u update, whose last block counts the iteration and sets the loop's
// condition -- then the statistics epilogue.
ct_status append_solve(const Ctx& c, int32_t iter0, cudaStream_t cs, cudaGraph_t graph) {
  const Params& prm = c.P.prm;
  std::vector<cudaGraphNode_t> tail;
  CT_TRY(capture_into(cs, graph, {}, tail, [&](cudaStream_t s) -> ct_status {
    if (iter0 == 0) {
      CT_TRY(ct::cuda_check(cudaMemsetAsync(c.ws, 0, c.L.off_atyc, s), "memset state"));
      // A^T y, scaled by 2*scale (hoisted out of the loop: y is constant).
      CT_TRY(c.P.proj.adj(c.y, c.at<float>(c.L.off_adj), c.at<float>(c.L.off_adjpart), s, nullptr));
      const int ns = c.P.proj.nsplit();
      const float* src = ns > 1 ? c.at<float>(c.L.off_adjpart) : c.at<float>(c.L.off_adj);
      k_scale_splits<<<NB, NT, 0, s>>>(src, c.at<float>(c.L.off_atyc), c.P.N, ns, c.tp.c, c.vi);
      CT_TRY(ct::launch_check("k_scale_splits"));
      CT_LAUNCH_ND(c.P.nd, k_init_state, NB, NT, s, c.x, c.at<float>(c.L.off_z), c.at<float>(c.L.off_u),
                   c.at<float>(c.L.off_dz), c.P.sh, c.P.N, c.tp.ng, c.vi);
      CT_TRY(ct::launch_check("k_init_state"));
    }
    k_reset_call<<<1, 1, 0, s>>>(c.slots());
    return ct::launch_check("k_reset_call");
  }));
  if (prm.maxiter <= 0) return CT_OK;  // no iteration: no statistics either
  cudaGraphConditionalHandle loop = 0;
  CT_TRY(ct::cuda_check(cudaGraphConditionalHandleCreate(&loop, graph, 1, cudaGraphCondAssignDefault),
                        "loop handle"));
  cudaGraphNode_t lnode = nullptr;
  cudaGraph_t body = nullptr;
  CT_TRY(add_conditional(graph, tail, loop, cudaGraphCondTypeWhile, lnode, body));
  cudaGraphConditionalHandle dirty = 0, cg = 0;
  CT_TRY(ct::cuda_check(cudaGraphConditionalHandleCreate(&dirty, body, 0, cudaGraphCondAssignDefault),
                        "projection handle"));
  CT_TRY(ct::cuda_check(cudaGraphConditionalHandleCreate(&cg, body, 0, cudaGraphCondAssignDefault),
                        "CG handle"));
  std::vector<cudaGraphNode_t> nodes, unused;
  CT_TRY(capture_into(cs, body, {}, nodes, [&](cudaStream_t s) { return enqueue_rhs(c, s, dirty, 1); }));
  cudaGraphNode_t pnode = nullptr, cnode = nullptr;
  cudaGraph_t pbody = nullptr, cbody = nullptr;
  CT_TRY(add_conditional(body, nodes, dirty, cudaGraphCondTypeIf, pnode, pbody));
  CT_TRY(capture_into(cs, pbody, {}, unused, [&](cudaStream_t s) { return enqueue_proj(c, s); }));
  CT_TRY(capture_into(cs, body, {pnode}, nodes, [&](cudaStream_t s) { return enqueue_init(c, s, cg, 1); }));
  CT_TRY(add_conditional(body, nodes, cg, cudaGraphCondTypeWhile, cnode, cbody));
  CT_TRY(capture_into(cs, cbody, {}, unused, [&](cudaStream_t s) { return enqueue_cg_step(c, s, cg, 1); }));
  CT_TRY(capture_into(cs, body, {cnode}, unused, [&](cudaStream_t s) { return enqueue_post(c, s, loop, 1); }));
  tail.assign(1, lnode);
  std::vector<cudaGraphNode_t> end;
  return capture_into(cs, graph, tail, end, [&](cudaStream_t s) { return enqueue_epilogue(c, s); });
}

// The executable graph of one solve, or of a batch of solves (independent
// branches of one graph), built on first use and cached by the problems'
// keys.  Caller holds g_cache.m.
ct_status graph_for(const Ctx* cs, int n, int32_t iter0, cudaGraphExec_t& exec) {
  int dev = 0;
  CT_TRY(ct::cuda_check(cudaGetDevice(&dev), "cudaGetDevice"));
  if (dev < 0 || dev >= 64) return ct::fail(CT_ERR_UNSUPPORTED, "device %d", dev);
  if (!g_cache.capture[dev])
    CT_TRY(ct::cuda_check(cudaStreamCreateWithFlags(&g_cache.capture[dev], cudaStreamNonBlocking),
                          "capture stream"));
  // the fast-forward CG start only in a single solve's graph: cooperative
  // kernels of concurrent branches could not all be resident at once
  std::vector<Ctx> cx(cs, cs + n);
  for (Ctx& c : cx) c.ffwd = n == 1 && ffwd_usable(c.P.nd);
  std::vector<unsigned char> key;
  key.insert(key.end(), reinterpret_cast<const unsigned char*>(&n),
             reinterpret_cast<const unsigned char*>(&n) + sizeof(n));
  for (int k = 0; k < n; ++k) make_key(cx[k], iter0, key);
  GraphEntry* slot = nullptr;
  for (GraphEntry& e : g_cache.e) {
    if (e.exec && e.device == dev && e.key == key) {
      e.last_use = ++g_cache.clock;
      exec = e.exec;
      return CT_OK;
    }
    if (!slot || !e.exec || (slot->exec && e.last_use < slot->last_use)) slot = &e;
  }
  if (slot->exec) {
    cudaGraphExecDestroy(slot->exec);
    slot->exec = nullptr;
  }
  cudaGraph_t graph = nullptr;
  CT_TRY(ct::cuda_check(cudaGraphCreate(&graph, 0), "graph create"));
  ct_status st = CT_OK;
  for (int k = 0; k < n && st == CT_OK; ++k) st = append_solve(cx[k], iter0, g_cache.capture[dev], graph);
  if (st != CT_OK) {
    cudaGraphDestroy(graph);
    return st;
  }
  cudaError_t ce = cudaGraphInstantiate(&slot->exec, graph, 0);
  cudaGraphDestroy(graph);
  if (ce != cudaSuccess) slot->exec = nullptr;
  CT_TRY(ct::cuda_check(ce, "graph instantiate"));
  slot->key = std::move(key);
  slot->device = dev;
  slot->last_use = ++g_cache.clock;
  exec = slot->exec;
  return CT_OK;
}

// One launch of the cached graph of n solves on stream s.
ct_status run_graph(const Ctx* cs, int n, int32_t iter0, cudaStream_t s) {
  cudaGraphExec_t exec = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_cache.m);
    CT_TRY(graph_for(cs, n, iter0, exec));
  }
  return ct::cuda_check(cudaGraphLaunch(exec, s), "graph launch");
}

// Validate one problem and fill its solver context.
template <class D>
ct_status make_ctx(const D* d, const char* who, const float* y, float* x, double* itstat_dev,
                   void* workspace, size_t workspace_bytes, Ctx& c) {
  CT_TRY(check_desc(d, who));
  if (!y || !x) return ct::fail(CT_ERR_INVALID_ARG, "%s: null array", who);
  c.P = problem_of(d);
  c.L = layout(c.P);
  if (!workspace || workspace_bytes < c.L.total || !ct::aligned(workspace, 256))
    return ct::fail(CT_ERR_WORKSPACE, "%s: need %zu bytes (256-B aligned), got %zu", who, c.L.total,
                    workspace_bytes);
  c.ws = static_cast<char*>(workspace);
  c.y = y;
  c.x = x;
  c.itstat = itstat_dev;
  const Params& prm = c.P.prm;
  TermParams& tp = c.tp;
  tp.ng = 0;
  // The reference's prox parameter is (1/rho) * lam in float64, then float32.
  if (prm.lam_l21 != 0.0) {
    tp.kind[tp.ng] = 0;
    tp.thr[tp.ng] = (float)((1.0 / prm.rho) * prm.lam_l21);
    ++tp.ng;
  }
  if (prm.lam_l1 != 0.0) {
    tp.kind[tp.ng] = 1;
    tp.thr[tp.ng] = (float)((1.0 / prm.rho) * prm.lam_l1);
    ++tp.ng;
  }
  tp.rho = (float)prm.rho;
  tp.alpha = (float)prm.alpha;
  tp.c = (float)(2.0 * prm.loss_scale);
  c.vi = (c.P.sh.n[c.P.nd - 1] % 4 == 0 && ct::aligned(c.x, 16)) ? 1 : 0;
  c.vs = (c.P.S % 4 == 0 && ct::aligned(c.y, 16)) ? 1 : 0;
  return c.P.proj.prepare();
}

// Enqueue one solve on stream s.
ct_status run_solve(const Ctx& c, int32_t iter0, cudaStream_t s) {
  const Params& prm = c.P.prm;
  if (prm.use_graph) return run_graph(&c, 1, iter0, s);  // the whole solve: one graph launch
  if (iter0 == 0) {
    CT_TRY(ct::cuda_check(cudaMemsetAsync(c.ws, 0, c.L.off_atyc, s), "memset state"));
    // A^T y, scaled by 2*scale (hoisted out of the loop: y is constant).
    CT_TRY(c.P.proj.adj(c.y, c.at<float>(c.L.off_adj), c.at<float>(c.L.off_adjpart), s, nullptr));
    const int ns = c.P.proj.nsplit();
    const float* src = ns > 1 ? c.at<float>(c.L.off_adjpart) : c.at<float>(c.L.off_adj);
    k_scale_splits<<<NB, NT, 0, s>>>(src, c.at<float>(c.L.off_atyc), c.P.N, ns, c.tp.c, c.vi);
    CT_TRY(ct::launch_check("k_scale_splits"));
    CT_LAUNCH_ND(c.P.nd, k_init_state, NB, NT, s, c.x, c.at<float>(c.L.off_z), c.at<float>(c.L.off_u),
                 c.at<float>(c.L.off_dz), c.P.sh, c.P.N, c.tp.ng, c.vi);
    CT_TRY(ct::launch_check("k_init_state"));
  }
  k_reset_call<<<1, 1, 0, s>>>(c.slots());
  CT_TRY(ct::launch_check("k_reset_call"));
  if (prm.maxiter == 0) return CT_OK;
  for (int k = 0; k < prm.maxiter; ++k) CT_TRY(enqueue_iteration(c, s));
  return enqueue_epilogue(c, s);
}

// Solve for either descriptor kind.
template <class D>
ct_status solve(const D* d, const char* who, const float* y, float* x, double* itstat_dev, int32_t iter0,
                void* workspace, size_t workspace_bytes, ct_stream_t stream) {
  Ctx c;
  CT_TRY(make_ctx(d, who, y, x, itstat_dev, workspace, workspace_bytes, c));
  return run_solve(c, iter0, ct::as_stream(stream));
}

// Internal streams for concurrent solves (per device, created once) and the
// events that fork them from, and join them back to, the caller's stream.
constexpr int kMaxBatchStreams = 32;

struct StreamPool {
  std::mutex m;
  cudaStream_t s[64][kMaxBatchStreams] = {};
  cudaEvent_t fork[64] = {};
  cudaEvent_t join[64][kMaxBatchStreams] = {};
};
StreamPool g_pool;

// Estimated device work of one solve: projector interactions per ADMM
// iteration (at most cg_maxiter + 2 forward/adjoint pairs) plus the
// elementwise work, times the iterations.
double solve_cost(const Ctx& c) {
  const double inter = (double)c.P.N * (c.P.nd == 2 ? c.P.proj.g2->n_views : c.P.proj.g3->n_views);
  return (double)c.P.prm.maxiter * ((c.P.prm.cg_maxiter + 2) * 2.0 * inter + 40.0 * (double)c.P.N);
}

template <class D>
ct_status workspace_of(const D* d, const char* who, size_t* bytes) {
  CT_TRY(check_desc(d, who));
  if (!bytes) return ct::fail(CT_ERR_INVALID_ARG, "%s: null bytes", who);
  *bytes = layout(problem_of(d)).total;
  return CT_OK;
}

template <class D>
ct_status state_of(const D* d, const char* who, size_t* z_offset, size_t* u_offset, int32_t* n_terms) {
  CT_TRY(check_desc(d, who));
  const Layout L = layout(problem_of(d));
  if (z_offset) *z_offset = L.off_z;
  if (u_offset) *u_offset = L.off_u;
  if (n_terms) *n_terms = L.ng;
  return CT_OK;
}

}  // namespace

extern "C" {

void ct_set_solver_fast_forward(int32_t on) { g_ffwd.store(on ? 1 : 0, std::memory_order_relaxed); }

int32_t ct_solver_fast_forward(void) { return ffwd_usable(2) ? 1 : 0; }

ct_status ct_admm_tv_workspace(const ct_admm_tv_desc* d, size_t* bytes) {
  return workspace_of(d, "ct_admm_tv_workspace", bytes);
}

ct_status ct_admm_tv_state(const ct_admm_tv_desc* d, size_t* z_offset, size_t* u_offset,
                           int32_t* n_terms) {
  return state_of(d, "ct_admm_tv_state", z_offset, u_offset, n_terms);
}

ct_status ct_admm_tv_solve(const ct_admm_tv_desc* d, const float* y, float* x, double* itstat_dev,
                           int32_t iter0, void* workspace, size_t workspace_bytes, ct_stream_t stream) {
  return solve(d, "ct_admm_tv_solve", y, x, itstat_dev, iter0, workspace, workspace_bytes, stream);
}

ct_status ct_admm_tv_solve_batch(const ct_admm_tv_desc* descs, int32_t n, const float* const* y,
                                 float* const* x, double* const* itstat_dev, int32_t iter0,
                                 void* const* workspace, const size_t* workspace_bytes, int32_t n_streams,
                                 ct_stream_t stream) {
  const char* who = "ct_admm_tv_solve_batch";
  if (n < 0) return ct::fail(CT_ERR_INVALID_ARG, "%s: n=%d", who, n);
  if (n == 0) return CT_OK;
  if (!descs || !y || !x || !workspace || !workspace_bytes)
    return ct::fail(CT_ERR_INVALID_ARG, "%s: null array of per-scan arguments", who);
  if (n_streams < 0 || n_streams > kMaxBatchStreams)
    return ct::fail(CT_ERR_INVALID_ARG, "%s: n_streams=%d (0..%d)", who, n_streams, kMaxBatchStreams);
  std::vector<Ctx> cs((size_t)n);
  bool all_graph = true;
  for (int k = 0; k < n; ++k) {
    CT_TRY(make_ctx(&descs[k], who, y[k], x[k], itstat_dev ? itstat_dev[k] : nullptr, workspace[k],
                    workspace_bytes[k], cs[k]));
    all_graph = all_graph && cs[k].P.prm.use_graph;
  }
  // All scans in one launch: a graph whose n independent branches are the
  // whole solves (built once per set of problems and cached).
  if (all_graph) return run_graph(cs.data(), n, iter0, ct::as_stream(stream));
  // Plain launches: the scans on a pool of streams.
  const int ns = n_streams > 0 ? std::min(n_streams, n) : std::min(n, 16);
  // longest-processing-time-first assignment to the least-loaded stream
  std::vector<int> order((size_t)n);
  for (int k = 0; k < n; ++k) order[k] = k;
  std::vector<double> cost((size_t)n);
  for (int k = 0; k < n; ++k) cost[k] = solve_cost(cs[k]);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cost[a] > cost[b]; });
  std::vector<double> load((size_t)ns, 0.0);
  std::vector<int> lane((size_t)n);
  for (int k : order) {
    int best = 0;
    for (int q = 1; q < ns; ++q)
      if (load[q] < load[best]) best = q;
    lane[k] = best;
    load[best] += cost[k];
  }
  int dev = 0;
  CT_TRY(ct::cuda_check(cudaGetDevice(&dev), "cudaGetDevice"));
  if (dev < 0 || dev >= 64) return ct::fail(CT_ERR_UNSUPPORTED, "%s: device %d", who, dev);
  std::lock_guard<std::mutex> lock(g_pool.m);
  if (!g_pool.fork[dev]) {
    CT_TRY(ct::cuda_check(cudaEventCreateWithFlags(&g_pool.fork[dev], cudaEventDisableTiming), "event"));
    for (int q = 0; q < kMaxBatchStreams; ++q) {
      CT_TRY(ct::cuda_check(cudaStreamCreateWithFlags(&g_pool.s[dev][q], cudaStreamNonBlocking), "stream"));
      CT_TRY(ct::cuda_check(cudaEventCreateWithFlags(&g_pool.join[dev][q], cudaEventDisableTiming), "event"));
    }
  }
  cudaStream_t caller = ct::as_stream(stream);
  CT_TRY(ct::cuda_check(cudaEventRecord(g_pool.fork[dev], caller), "event record"));
  for (int q = 0; q < ns; ++q)
    CT_TRY(ct::cuda_check(cudaStreamWaitEvent(g_pool.s[dev][q], g_pool.fork[dev], 0), "stream wait"));
  // enqueue in assignment order so each stream starts with its longest scan
  for (int k : order) CT_TRY(run_solve(cs[k], iter0, g_pool.s[dev][lane[k]]));
  for (int q = 0; q < ns; ++q) {
    CT_TRY(ct::cuda_check(cudaEventRecord(g_pool.join[dev][q], g_pool.s[dev][q]), "event record"));
    CT_TRY(ct::cuda_check(cudaStreamWaitEvent(caller, g_pool.join[dev][q], 0), "stream wait"));
  }
  return CT_OK;
}

ct_status ct_admm_tv3d_workspace(const ct_admm_tv3d_desc* d, size_t* bytes) {
  return workspace_of(d, "ct_admm_tv3d_workspace", bytes);
}

ct_status ct_admm_tv3d_state(const ct_admm_tv3d_desc* d, size_t* z_offset, size_t* u_offset,
                             int32_t* n_terms) {
  return state_of(d, "ct_admm_tv3d_state", z_offset, u_offset, n_terms);
}

ct_status ct_admm_tv3d_solve(const ct_admm_tv3d_desc* d, const float* y, float* x, double* itstat_dev,
                             int32_t iter0, void* workspace, size_t workspace_bytes, ct_stream_t stream) {
  return solve(d, "ct_admm_tv3d_solve", y, x, itstat_dev, iter0, workspace, workspace_bytes, stream);
}

}  // extern "C"
