// Fused proximal ADMM for CT with TV, the CG-free split of the reference's
// ct_3d_tv_padmm example (scico/optimize/_padmm.py:349-363):
//
//   min_x  scale ||y - C x||^2 + lam ||D x||_{2,1}
//   as  min f(x) + g(z)  s.t.  A x + B z = 0,  f = 0,
//   A = (C; alpha D), B = -I, g = g0(z0) + g1(z1),
//   g0 = scale ||y - z0||^2, g1 = (lam / alpha) ||z1||_{2,1},
//
// C the 2D or 3D projector, D = FiniteDifference over all axes (append=0).
// One iteration:
//   x  <- x - (1/mu) A^T (2u - u_old)          (prox of f = 0 is the identity)
//   z  <- prox_{g/(rho nu)}(z + (1/nu)(A x - z + u))
//   u  <- u + A x - z
// with the primal residual ||A x - z|| and the (fast) dual residual
// ||z - z_old|| in float64.
//
// Launches per iteration: the adjoint projection of t0 = 2u0 - u0_old, the
// x-update (adds alpha D^T t1, t1 = 2u1 - u1_old, and the adjoint's view
// splits in order), the forward projection of x, then one fused z/u update
// per block; each z/u update also writes the next iteration's t = 2u - u_old,
// so u_old is never stored.  With use_graph the iteration is captured once
// into a CUDA graph (cached per problem) and replayed maxiter times.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "kernels.cuh"

namespace {

constexpr int NT = ct::kReduceThreads;
constexpr int NB = ct::kReduceBlocks;

enum Slot {
  P_PRIMAL2 = 0,  // sum of the sinogram block's ||A x - z||^2 (this iteration)
  P_DUAL2 = 1,    // the same for ||z - z_old||^2
  P_G0 = 2,       // g0(z0) = scale ||y - z0||^2
  P_ITER = 3,     // records written in this call
  P_COUNT = 8
};

struct Shape3 {
  int n[3];
};

struct Scal {
  float inv_mu, inv_nu, alpha;
  float c, c1;      // prox of g0: (c y + v) / c1, c = 2 scale / (rho nu), c1 = c + 1
  float thr;        // prox threshold of g1: (lam / alpha) / (rho nu)
  double scale;     // g0 = scale ||y - z0||^2
  double w1;        // g1 = w1 ||z1||_{2,1}, w1 = lam / alpha
};

template <int ND>
__device__ __forceinline__ void coords(size_t e, const Shape3& sh, int (&c)[ND]) {
  size_t r = e;
#pragma unroll
  for (int k = ND - 1; k >= 0; --k) {
    c[k] = (int)(r % (size_t)sh.n[k]);
    r /= (size_t)sh.n[k];
  }
}

template <int ND>
__device__ __forceinline__ size_t axis_stride(const Shape3& sh, int k) {
  size_t st = 1;
  for (int q = ND - 1; q > k; --q) st *= (size_t)sh.n[q];
  return st;
}

// Quad path (n[ND-1] % 4 == 0, every array 16-B aligned, N < 2^31): a
// thread takes four consecutive elements along the last axis with 128-bit
// loads and stores; the per-element arithmetic is the scalar path's, in the
// same order.
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
template <int ND>
__device__ __forceinline__ void coords32(uint32_t e, const Shape3& sh, int (&c)[ND]) {
  uint32_t r = e;
#pragma unroll
  for (int k = ND - 1; k >= 0; --k) {
    const uint32_t q = r / (uint32_t)sh.n[k];
    c[k] = (int)(r - q * (uint32_t)sh.n[k]);
    r = q;
  }
}

// x <- x - (1/mu) (A^T t)(e):  A^T t = C^T t0 + alpha D^T t1, the adjoint's
// view splits summed in order, D^T with the append=0 boundaries, axes in
// order (linop/_stack.py:71-72, _diff.py).
template <int ND>
__global__ void __launch_bounds__(NT)
    k_pd_x(float* __restrict__ x, const float* __restrict__ adj, int nsplit, const float* __restrict__ t1,
           Shape3 sh, size_t N, Scal s, int vec) {
  if (vec) {
    for (size_t e0 = 4 * ((size_t)blockIdx.x * NT + threadIdx.x); e0 < N; e0 += 4 * (size_t)gridDim.x * NT) {
      int c[ND];
      coords32<ND>((uint32_t)e0, sh, c);
      float ct[4], dt[4], xv[4];
      unpack4(ld4(adj, e0), ct);
      for (int q = 1; q < nsplit; ++q) {
        float v[4];
        unpack4(ld4(adj, (size_t)q * N + e0), v);
#pragma unroll
        for (int j = 0; j < 4; ++j) ct[j] = ct::fadd(ct[j], v[j]);
      }
#pragma unroll
      for (int k = 0; k < ND; ++k) {
        const float* tk = t1 + (size_t)k * N;
        float fc[4], lo[4], hi[4];
        unpack4(ld4(tk, e0), fc);
        if (k < ND - 1) {
          const size_t st = axis_stride<ND>(sh, k);
          if (c[k] >= 1) {
            unpack4(ld4(tk, e0 - st), lo);
          } else {
#pragma unroll
            for (int j = 0; j < 4; ++j) lo[j] = 0.0f;
          }
          const bool h = c[k] <= sh.n[k] - 2;
#pragma unroll
          for (int j = 0; j < 4; ++j) hi[j] = h ? fc[j] : 0.0f;
        } else {
          const int cl = c[ND - 1], nl = sh.n[ND - 1];
          lo[0] = cl >= 1 ? tk[e0 - 1] : 0.0f;
          lo[1] = fc[0];
          lo[2] = fc[1];
          lo[3] = fc[2];
#pragma unroll
          for (int j = 0; j < 4; ++j) hi[j] = cl + j <= nl - 2 ? fc[j] : 0.0f;
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) dt[j] = k == 0 ? ct::fsub(lo[j], hi[j]) : ct::fadd(dt[j], ct::fsub(lo[j], hi[j]));
      }
      unpack4(ld4(x, e0), xv);
#pragma unroll
      for (int j = 0; j < 4; ++j)
        xv[j] = ct::fsub(xv[j], ct::fmul(s.inv_mu, ct::fadd(ct[j], ct::fmul(s.alpha, dt[j]))));
      st4(x, e0, xv);
    }
    return;
  }
  for (size_t e = (size_t)blockIdx.x * NT + threadIdx.x; e < N; e += (size_t)gridDim.x * NT) {
    float ct = adj[e];
    for (int q = 1; q < nsplit; ++q) ct = ct::fadd(ct, adj[(size_t)q * N + e]);
    int c[ND];
    coords<ND>(e, sh, c);
    float dt = 0.0f;
#pragma unroll
    for (int k = 0; k < ND; ++k) {
      const size_t st = axis_stride<ND>(sh, k);
      const float* tk = t1 + (size_t)k * N;
      const float lo = c[k] >= 1 ? tk[e - st] : 0.0f;
      const float hi = c[k] <= sh.n[k] - 2 ? tk[e] : 0.0f;
      dt = k == 0 ? ct::fsub(lo, hi) : ct::fadd(dt, ct::fsub(lo, hi));
    }
    const float at = ct::fadd(ct, ct::fmul(s.alpha, dt));
    x[e] = ct::fsub(x[e], ct::fmul(s.inv_mu, at));
  }
}

// Sinogram block, one element: a = (C x)[e];  pz = z0 + (1/nu)((a - z0) + u0);
// z0' = (c y + pz) / (c + 1);  u0' = (u0 + a) - z0';  t0 = 2 u0' - u0.
__device__ __forceinline__ void zu0_elem(float a, float z, float u, float ye, const Scal& s, float& zn, float& un,
                                         float& tn, ct::KSum& prim, ct::KSum& dual, ct::KSum& g0) {
  const float pz = ct::fadd(z, ct::fmul(s.inv_nu, ct::fadd(ct::fsub(a, z), u)));
  zn = __fdiv_rn(ct::fadd(ct::fmul(s.c, ye), pz), s.c1);
  un = ct::fsub(ct::fadd(u, a), zn);
  tn = ct::fsub(ct::fmul(2.0f, un), u);
  const float r = ct::fsub(a, zn), d = ct::fsub(zn, z), q = ct::fsub(ye, zn);
  prim.add(ct::fmul(r, r));
  dual.add(ct::fmul(d, d));
  g0.add(ct::fmul(q, q));
}

__global__ void __launch_bounds__(NT)
    k_pd_zu0(const float* __restrict__ ax, const float* __restrict__ y, float* __restrict__ z0,
             float* __restrict__ u0, float* __restrict__ t0, size_t S, Scal s, double* __restrict__ slots,
             double* __restrict__ partials, unsigned int* __restrict__ ticket, int vec) {
  ct::KSum prim, dual, g0;
  if (vec) {
    for (size_t e0 = 4 * ((size_t)blockIdx.x * NT + threadIdx.x); e0 < S; e0 += 4 * (size_t)gridDim.x * NT) {
      float a[4], z[4], u[4], ye[4], zn[4], un[4], tn[4];
      unpack4(ld4(ax, e0), a);
      unpack4(ld4(z0, e0), z);
      unpack4(ld4(u0, e0), u);
      unpack4(ld4(y, e0), ye);
#pragma unroll
      for (int j = 0; j < 4; ++j) zu0_elem(a[j], z[j], u[j], ye[j], s, zn[j], un[j], tn[j], prim, dual, g0);
      st4(z0, e0, zn);
      st4(u0, e0, un);
      st4(t0, e0, tn);
    }
  } else {
    for (size_t e = (size_t)blockIdx.x * NT + threadIdx.x; e < S; e += (size_t)gridDim.x * NT) {
      float zn, un, tn;
      zu0_elem(ax[e], z0[e], u0[e], y[e], s, zn, un, tn, prim, dual, g0);
      z0[e] = zn;
      u0[e] = un;
      t0[e] = tn;
    }
  }
  double v[3] = {prim.value(), dual.value(), g0.value()}, out[3];
  if (ct::grid_reduce_last<NT, 3>(v, partials, ticket, out)) {
    slots[P_PRIMAL2] = out[0];
    slots[P_DUAL2] = out[1];
    slots[P_G0] = s.scale * out[2];
  }
}

// FD block, one element: ax_k = alpha (D x)_k;
// pz_k = z1_k + (1/nu)((ax_k - z1_k) + u1_k); z1' = L2,1 prox of pz with
// threshold thr (_norm.py:254-263); u1_k' = (u1_k + ax_k) - z1_k';
// t1_k = 2 u1_k' - u1_k.
template <int ND>
__device__ __forceinline__ void zu1_elem(const float (&ax)[ND], const float (&z)[ND], const float (&u)[ND],
                                         const Scal& s, float (&zn)[ND], float (&un)[ND], float (&tn)[ND],
                                         ct::KSum& prim, ct::KSum& dual, ct::KSum& g1) {
  float pz[ND];
  float ss = 0.0f;
#pragma unroll
  for (int k = 0; k < ND; ++k) {
    pz[k] = ct::fadd(z[k], ct::fmul(s.inv_nu, ct::fadd(ct::fsub(ax[k], z[k]), u[k])));
    ss = k == 0 ? ct::fmul(pz[k], pz[k]) : ct::fadd(ss, ct::fmul(pz[k], pz[k]));
  }
  const float len = __fsqrt_rn(ss);
  float nl = ct::fsub(len, s.thr);
  nl = ct::fmul(0.5f, ct::fadd(nl, fabsf(nl)));
  float zz = 0.0f;
#pragma unroll
  for (int k = 0; k < ND; ++k) {
    zn[k] = ct::fmul(nl, len != 0.0f ? __fdiv_rn(pz[k], len) : 0.0f);
    un[k] = ct::fsub(ct::fadd(u[k], ax[k]), zn[k]);
    tn[k] = ct::fsub(ct::fmul(2.0f, un[k]), u[k]);
    const float r = ct::fsub(ax[k], zn[k]), d = ct::fsub(zn[k], z[k]);
    prim.add(ct::fmul(r, r));
    dual.add(ct::fmul(d, d));
    zz = k == 0 ? ct::fmul(zn[k], zn[k]) : ct::fadd(zz, ct::fmul(zn[k], zn[k]));
  }
  g1.add(__fsqrt_rn(zz));
}

// FD block over the grid; the last block adds the sinogram block's sums and
// writes the iteration's record.
template <int ND>
__global__ void __launch_bounds__(NT)
    k_pd_zu1(const float* __restrict__ x, float* __restrict__ z1, float* __restrict__ u1, float* __restrict__ t1,
             Shape3 sh, size_t N, Scal s, double* __restrict__ itstat, int maxiter, double* __restrict__ slots,
             double* __restrict__ partials, unsigned int* __restrict__ ticket, int vec) {
  ct::KSum prim, dual, g1;
  if (vec) {
    for (size_t e0 = 4 * ((size_t)blockIdx.x * NT + threadIdx.x); e0 < N; e0 += 4 * (size_t)gridDim.x * NT) {
      int c[ND];
      coords32<ND>((uint32_t)e0, sh, c);
      float xc[4], ax[ND][4], z[ND][4], u[ND][4];
      unpack4(ld4(x, e0), xc);
#pragma unroll
      for (int k = 0; k < ND; ++k) {
        float nx[4];
        if (k < ND - 1) {
          if (c[k] <= sh.n[k] - 2) {
            unpack4(ld4(x, e0 + axis_stride<ND>(sh, k)), nx);
          } else {
#pragma unroll
            for (int j = 0; j < 4; ++j) nx[j] = xc[j];
          }
        } else {
          const int cl = c[ND - 1], nl = sh.n[ND - 1];
          nx[0] = cl <= nl - 2 ? xc[1] : xc[0];
          nx[1] = cl + 1 <= nl - 2 ? xc[2] : xc[1];
          nx[2] = cl + 2 <= nl - 2 ? xc[3] : xc[2];
          nx[3] = cl + 3 <= nl - 2 ? x[e0 + 4] : xc[3];
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) ax[k][j] = ct::fmul(s.alpha, ct::fsub(nx[j], xc[j]));
        unpack4(ld4(z1, (size_t)k * N + e0), z[k]);
        unpack4(ld4(u1, (size_t)k * N + e0), u[k]);
      }
      float zn[ND][4], un[ND][4], tn[ND][4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        float a1[ND], z1v[ND], u1v[ND], zo[ND], uo[ND], to[ND];
#pragma unroll
        for (int k = 0; k < ND; ++k) {
          a1[k] = ax[k][j];
          z1v[k] = z[k][j];
          u1v[k] = u[k][j];
        }
        zu1_elem<ND>(a1, z1v, u1v, s, zo, uo, to, prim, dual, g1);
#pragma unroll
        for (int k = 0; k < ND; ++k) {
          zn[k][j] = zo[k];
          un[k][j] = uo[k];
          tn[k][j] = to[k];
        }
      }
#pragma unroll
      for (int k = 0; k < ND; ++k) {
        st4(z1, (size_t)k * N + e0, zn[k]);
        st4(u1, (size_t)k * N + e0, un[k]);
        st4(t1, (size_t)k * N + e0, tn[k]);
      }
    }
  } else {
    for (size_t e = (size_t)blockIdx.x * NT + threadIdx.x; e < N; e += (size_t)gridDim.x * NT) {
      int c[ND];
      coords<ND>(e, sh, c);
      const float xc = x[e];
      float ax[ND], z[ND], u[ND], zn[ND], un[ND], tn[ND];
#pragma unroll
      for (int k = 0; k < ND; ++k) {
        const float xn = c[k] <= sh.n[k] - 2 ? x[e + axis_stride<ND>(sh, k)] : xc;
        ax[k] = ct::fmul(s.alpha, ct::fsub(xn, xc));
        z[k] = z1[(size_t)k * N + e];
        u[k] = u1[(size_t)k * N + e];
      }
      zu1_elem<ND>(ax, z, u, s, zn, un, tn, prim, dual, g1);
#pragma unroll
      for (int k = 0; k < ND; ++k) {
        z1[(size_t)k * N + e] = zn[k];
        u1[(size_t)k * N + e] = un[k];
        t1[(size_t)k * N + e] = tn[k];
      }
    }
  }
  double v[3] = {prim.value(), dual.value(), g1.value()}, out[3];
  if (ct::grid_reduce_last<NT, 3>(v, partials, ticket, out)) {
    const int it = (int)slots[P_ITER];
    if (itstat && it < maxiter) {
      itstat[3 * it] = slots[P_G0] + s.w1 * out[2];
      itstat[3 * it + 1] = sqrt(slots[P_PRIMAL2] + out[0]);
      itstat[3 * it + 2] = sqrt(slots[P_DUAL2] + out[1]);
    }
    slots[P_ITER] = (double)(it + 1);
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

#define CT_TRY(expr)              \
  do {                            \
    ct_status _st = (expr);       \
    if (_st != CT_OK) return _st; \
  } while (0)

struct Problem {
  int nd = 2;
  Shape3 sh{};
  size_t N = 0, S = 0;
  ct::Proj2dPlan p2{};
  ct::Proj3dPlan p3{};
  Scal sc{};
};

struct Layout {
  size_t off_slots, off_red, off_z0, off_u0, off_t0, off_z1, off_u1, off_t1, off_sinox, off_adj, off_part,
      off_fwd, total;
};

ct_status problem_of(const ct_padmm_tv_desc* d, const char* who, Problem& P) {
  if (!d) return ct::fail(CT_ERR_INVALID_ARG, "%s: null descriptor", who);
  if (d->nd != 2 && d->nd != 3) return ct::fail(CT_ERR_INVALID_ARG, "%s: nd=%d (2 or 3)", who, d->nd);
  if (d->maxiter < 0) return ct::fail(CT_ERR_INVALID_ARG, "%s: maxiter=%d", who, d->maxiter);
  if (!(d->rho > 0.0) || !(d->mu > 0.0) || !(d->nu > 0.0) || !(d->alpha != 0.0) || !(d->loss_scale > 0.0))
    return ct::fail(CT_ERR_INVALID_ARG, "%s: rho, mu, nu and loss_scale must be > 0 and alpha != 0", who);
  P.nd = d->nd;
  if (P.nd == 2) {
    CT_TRY(ct::proj2d_check(&d->geom2, who));
    P.sh.n[0] = d->geom2.rows;
    P.sh.n[1] = d->geom2.cols;
    P.sh.n[2] = 1;
    P.N = (size_t)d->geom2.rows * d->geom2.cols;
    P.S = (size_t)d->geom2.n_views * d->geom2.det_count;
    P.p2 = ct::proj2d_plan(&d->geom2, 1);
  } else {
    CT_TRY(ct::proj3d_check(&d->geom3, who));
    for (int k = 0; k < 3; ++k) P.sh.n[k] = d->geom3.shape[k];
    P.N = (size_t)d->geom3.shape[0] * d->geom3.shape[1] * d->geom3.shape[2];
    P.S = (size_t)d->geom3.n_views * d->geom3.det_shape[0] * d->geom3.det_shape[1];
    P.p3 = ct::proj3d_plan(&d->geom3, 1);
  }
  // the scalars as the reference forms them: Python floats (double) rounded
  // to float32 when they multiply float32 arrays
  const double lam_p = 1.0 / (d->rho * d->nu);
  const double c = 2.0 * d->loss_scale * lam_p;
  P.sc.inv_mu = (float)(1.0 / d->mu);
  P.sc.inv_nu = (float)(1.0 / d->nu);
  P.sc.alpha = (float)d->alpha;
  P.sc.c = (float)c;
  P.sc.c1 = (float)(c + 1.0);
  P.sc.thr = (float)((d->lam / d->alpha) * lam_p);
  P.sc.scale = d->loss_scale;
  P.sc.w1 = d->lam / d->alpha;
  return CT_OK;
}

size_t fwd_bytes(const Problem& P) { return P.nd == 2 ? P.p2.fwd_bytes : P.p3.fwd_ws_bytes; }
size_t adj_ws_bytes(const Problem& P) { return P.nd == 2 ? P.p2.adj_ws_bytes : P.p3.adj_ws_bytes; }
int nsplit(const Problem& P) { return P.nd == 2 ? P.p2.nsplit : P.p3.nsplit; }

Layout layout(const Problem& P) {
  Layout L;
  size_t o = 0;
  auto take = [&](size_t bytes) {
    const size_t at = o;
    o += ct::round_up(bytes > 0 ? bytes : 1, 256);
    return at;
  };
  const size_t M = (size_t)P.nd * P.N;
  L.off_slots = take(P_COUNT * sizeof(double));
  L.off_red = take(ct::kReduceWorkspace);
  L.off_z0 = take(P.S * 4);
  L.off_u0 = take(P.S * 4);
  L.off_t0 = take(P.S * 4);
  L.off_z1 = take(M * 4);
  L.off_u1 = take(M * 4);
  L.off_t1 = take(M * 4);
  L.off_sinox = take(P.S * 4);
  L.off_adj = take(P.N * 4);
  L.off_part = take(adj_ws_bytes(P));
  L.off_fwd = take(fwd_bytes(P));
  L.total = o;
  return L;
}

struct Ctx {
  const ct_padmm_tv_desc* d;
  Problem P;
  Layout L;
  char* ws;
  const float* y;
  float* x;
  double* itstat;
  template <class T>
  T* at(size_t off) const { return reinterpret_cast<T*>(ws + off); }
  double* slots() const { return at<double>(L.off_slots); }
  unsigned int* ticket() const { return at<unsigned int>(L.off_red); }
  double* partials() const { return reinterpret_cast<double*>(ws + L.off_red + 256); }
};

ct_status enqueue_iteration(const Ctx& c, cudaStream_t s) {
  const Problem& P = c.P;
  float* adj = c.at<float>(c.L.off_adj);
  float* part = c.at<float>(c.L.off_part);
  float* sinox = c.at<float>(c.L.off_sinox);
  // C^T t0
  if (P.nd == 2)
    CT_TRY(ct::proj2d_adj_launch(&c.d->geom2, P.p2, c.at<float>(c.L.off_t0), adj, part, 1, s, nullptr));
  else
    CT_TRY(ct::proj3d_adj_launch(&c.d->geom3, P.p3, c.at<float>(c.L.off_t0), adj, part, s, nullptr));
  const float* a = nsplit(P) > 1 ? part : adj;
  float* t1 = c.at<float>(c.L.off_t1);
  float* z1 = c.at<float>(c.L.off_z1);
  float* u1 = c.at<float>(c.L.off_u1);
  // quads along the last axis: its length a multiple of 4, 32-bit indices
  const bool rows4 = P.sh.n[P.nd - 1] % 4 == 0 && P.N < (size_t(1) << 31);
  const int vx = rows4 && ct::quad_ok(P.N, c.x, a, t1) ? 1 : 0;
  const int vz1 = rows4 && ct::quad_ok(P.N, c.x, z1, u1, t1) ? 1 : 0;
  if (P.nd == 2)
    k_pd_x<2><<<NB, NT, 0, s>>>(c.x, a, nsplit(P), t1, P.sh, P.N, P.sc, vx);
  else
    k_pd_x<3><<<NB, NT, 0, s>>>(c.x, a, nsplit(P), t1, P.sh, P.N, P.sc, vx);
  CT_TRY(ct::launch_check("k_pd_x"));
  // C x
  if (P.nd == 2)
    CT_TRY(ct::proj2d_fwd_launch(&c.d->geom2, P.p2, c.x, sinox, 1, c.at<float>(c.L.off_fwd), s, nullptr));
  else
    CT_TRY(ct::proj3d_fwd_launch(&c.d->geom3, P.p3, c.x, sinox, c.at<void>(c.L.off_fwd), s, nullptr));
  float* z0 = c.at<float>(c.L.off_z0);
  float* u0 = c.at<float>(c.L.off_u0);
  float* t0 = c.at<float>(c.L.off_t0);
  k_pd_zu0<<<NB, NT, 0, s>>>(sinox, c.y, z0, u0, t0, P.S, P.sc, c.slots(), c.partials(), c.ticket(),
                             ct::quad_ok(P.S, sinox, c.y, z0, u0, t0));
  CT_TRY(ct::launch_check("k_pd_zu0"));
  if (P.nd == 2)
    k_pd_zu1<2><<<NB, NT, 0, s>>>(c.x, z1, u1, t1, P.sh, P.N, P.sc, c.itstat, c.d->maxiter, c.slots(), c.partials(),
                                  c.ticket(), vz1);
  else
    k_pd_zu1<3><<<NB, NT, 0, s>>>(c.x, z1, u1, t1, P.sh, P.N, P.sc, c.itstat, c.d->maxiter, c.slots(), c.partials(),
                                  c.ticket(), vz1);
  return ct::launch_check("k_pd_zu1");
}

// Executable one-iteration graphs, keyed by the descriptor bytes, the
// projector schedule and wait limit and the state/data pointers; least
// recently used evicted.
constexpr int kMaxGraphs = 64;

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

std::vector<unsigned char> make_key(const Ctx& c) {
  std::vector<unsigned char> key;
  auto put = [&](const void* p, size_t b) {
    const unsigned char* q = static_cast<const unsigned char*>(p);
    key.insert(key.end(), q, q + b);
  };
  put(c.d, sizeof(*c.d));
  if (c.P.nd == 2) {
    put(&c.P.p2.vpc, sizeof(int));
    put(&c.P.p2.nsplit, sizeof(int));
    const uint32_t polls = ct::proj2d_wait_polls();
    put(&polls, sizeof(polls));
  } else {
    put(&c.P.p3.G, sizeof(int));
    put(&c.P.p3.nsplit, sizeof(int));
  }
  put(&c.ws, sizeof(c.ws));
  put(&c.y, sizeof(c.y));
  put(&c.x, sizeof(c.x));
  put(&c.itstat, sizeof(c.itstat));
  return key;
}

ct_status graph_for(const Ctx& c, cudaGraphExec_t& exec) {
  int dev = 0;
  CT_TRY(ct::cuda_check(cudaGetDevice(&dev), "cudaGetDevice"));
  if (dev < 0 || dev >= 64) return ct::fail(CT_ERR_UNSUPPORTED, "device %d", dev);
  std::lock_guard<std::mutex> lock(g_cache.m);
  if (!g_cache.capture[dev])
    CT_TRY(ct::cuda_check(cudaStreamCreateWithFlags(&g_cache.capture[dev], cudaStreamNonBlocking), "capture stream"));
  const std::vector<unsigned char> key = make_key(c);
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
  cudaStream_t cs = g_cache.capture[dev];
  CT_TRY(ct::cuda_check(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal), "begin capture"));
  ct_status st = enqueue_iteration(c, cs);
  cudaGraph_t graph = nullptr;
  const cudaError_t ce = cudaStreamEndCapture(cs, &graph);
  if (st != CT_OK) {
    if (graph) cudaGraphDestroy(graph);
    return st;
  }
  CT_TRY(ct::cuda_check(ce, "end capture"));
  const cudaError_t ie = cudaGraphInstantiate(&slot->exec, graph, 0);
  cudaGraphDestroy(graph);
  if (ie != cudaSuccess) slot->exec = nullptr;
  CT_TRY(ct::cuda_check(ie, "graph instantiate"));
  slot->key = key;
  slot->device = dev;
  slot->last_use = ++g_cache.clock;
  exec = slot->exec;
  return CT_OK;
}

ct_status make_ctx(const ct_padmm_tv_desc* d, const char* who, const float* y, float* x, double* itstat, void* ws,
                   size_t ws_bytes, Ctx& c) {
  c.d = d;
  CT_TRY(problem_of(d, who, c.P));
  if (!y || !x) return ct::fail(CT_ERR_INVALID_ARG, "%s: null array", who);
  c.L = layout(c.P);
  if (!ws || ws_bytes < c.L.total || !ct::aligned(ws, 256))
    return ct::fail(CT_ERR_WORKSPACE, "%s: need %zu bytes (256-B aligned), got %zu", who, c.L.total, ws_bytes);
  c.ws = static_cast<char*>(ws);
  c.y = y;
  c.x = x;
  c.itstat = itstat;
  return CT_OK;
}

}  // namespace

extern "C" {

ct_status ct_padmm_tv_workspace(const ct_padmm_tv_desc* d, size_t* bytes) {
  Problem P;
  CT_TRY(problem_of(d, "ct_padmm_tv_workspace", P));
  if (!bytes) return ct::fail(CT_ERR_INVALID_ARG, "ct_padmm_tv_workspace: null bytes");
  *bytes = layout(P).total;
  return CT_OK;
}

ct_status ct_padmm_tv_state(const ct_padmm_tv_desc* d, size_t* z0_offset, size_t* z1_offset, size_t* u0_offset,
                            size_t* u1_offset) {
  Problem P;
  CT_TRY(problem_of(d, "ct_padmm_tv_state", P));
  const Layout L = layout(P);
  if (z0_offset) *z0_offset = L.off_z0;
  if (z1_offset) *z1_offset = L.off_z1;
  if (u0_offset) *u0_offset = L.off_u0;
  if (u1_offset) *u1_offset = L.off_u1;
  return CT_OK;
}

ct_status ct_padmm_tv_solve(const ct_padmm_tv_desc* d, const float* y, float* x, double* itstat_dev, int32_t cont,
                            void* workspace, size_t workspace_bytes, ct_stream_t stream) {
  const char* who = "ct_padmm_tv_solve";
  Ctx c;
  CT_TRY(make_ctx(d, who, y, x, itstat_dev, workspace, workspace_bytes, c));
  cudaStream_t s = ct::as_stream(stream);
  if (c.P.nd == 2)
    CT_TRY(ct::proj2d_prepare(c.P.p2));
  else
    CT_TRY(ct::proj3d_prepare(&d->geom3, c.P.p3));
  if (!cont) {
    // z = u = u_old = 0 (t = 2u - u_old = 0) and a clean reduction ticket
    CT_TRY(ct::cuda_check(cudaMemsetAsync(c.ws, 0, c.L.off_sinox, s), "state init"));
  } else {
    CT_TRY(ct::cuda_check(cudaMemsetAsync(c.slots(), 0, P_COUNT * sizeof(double), s), "slots init"));
  }
  if (d->maxiter == 0) return CT_OK;
  if (!d->use_graph) {
    for (int it = 0; it < d->maxiter; ++it) CT_TRY(enqueue_iteration(c, s));
    return CT_OK;
  }
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  CT_TRY(ct::cuda_check(cudaStreamIsCapturing(s, &cap), "stream capture query"));
  if (cap != cudaStreamCaptureStatusNone) {  // inside a caller's capture: plain launches
    for (int it = 0; it < d->maxiter; ++it) CT_TRY(enqueue_iteration(c, s));
    return CT_OK;
  }
  cudaGraphExec_t exec = nullptr;
  CT_TRY(graph_for(c, exec));
  for (int it = 0; it < d->maxiter; ++it) CT_TRY(ct::cuda_check(cudaGraphLaunch(exec, s), "graph launch"));
  return CT_OK;
}

}  // extern "C"
