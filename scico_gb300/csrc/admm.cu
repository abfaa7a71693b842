// Fused ADMM-TV solver for 2D parallel-beam CT.
//
// Solves  min_x scale ||A x - y||^2 + lam21 ||D x||_{2,1} + lam1 ||D x||_1
// with scico's ADMM + LinearSubproblemSolver (scico/optimize/_admm.py:334-378,
// _admmaux.py:205-269, scico/solver.py:326-405), D = FiniteDifference over
// both axes with append=0 (stacked (2, rows, cols)).  One g_i per non-zero
// lambda, L2,1 first, each with its own z_i and u_i, all sharing D and rho.
//
// Per outer iteration (each kernel below is one launch; the whole iteration
// is captured once into a CUDA graph and replayed):
//   k_rhs         rhs = c A^T y + sum_i rho D^T(z_i - u_i); also the dual
//                 residual ||sum_i rho D^T(z_i - z_i_old)|| of the previous
//                 iteration
//   A x           forward projection of the current x, k_resid2 gives
//                 ||A x - y||^2 for the previous iteration's objective
//   k_itstat      writes the previous iteration's itstat record
//   A^T, k_lhs_finish<INIT>   lhs(x) = c A^T A x + rho D^T D x, r = rhs - lhs(x),
//                 p = r, CG scalars (num, ||b||, tolerance) in float64
//   CG loop       A p, A^T, k_lhs_finish<PAP> (Ap, <p,Ap>), CG update,
//                 direction.  In the graph the loop is a conditional WHILE
//                 node whose condition the device sets (CG start and each
//                 update), so it runs exactly the reference's number of CG
//                 iterations; without a graph, cg_maxiter copies are launched
//                 and become no-ops once CG has converged
//   k_zu          Dx, z_i = prox(Dx + u_i), u_i += Dx - z_i, primal residual
//                 and g_i(z_i) partial sums
// lhs(x) and A x are kept from the last CG start while x is unchanged (no CG
// step ran since): the deterministic kernels would recompute the same bits,
// so the projections of x are skipped then.
// The reference evaluates the itstat quantities with extra operator
// applications after each step; here they are fused into the kernels that
// already read the operands, and the x-dependent ones are taken from the
// next iteration's first projection of the same x (an epilogue covers the
// last iteration).
#include <math.h>
#include <string.h>

#include <mutex>

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

__device__ __forceinline__ int pix_i(size_t e, int C) { return (int)(e / (size_t)C); }

// D^T applied at (i, j) to a stacked (2, R, C) field f = a - b (b may be null).
__device__ __forceinline__ float dT_at(const float* __restrict__ a, const float* __restrict__ b,
                                       int i, int j, int R, int C) {
  const size_t N = (size_t)R * C;
  const size_t e = (size_t)i * C + j;
  auto f = [&](int comp, size_t idx) -> float {
    const float av = a[comp * N + idx];
    return b ? ct::fsub(av, b[comp * N + idx]) : av;
  };
  const float lo0 = i >= 1 ? f(0, e - C) : 0.0f;
  const float hi0 = i <= R - 2 ? f(0, e) : 0.0f;
  const float lo1 = j >= 1 ? f(1, e - 1) : 0.0f;
  const float hi1 = j <= C - 2 ? f(1, e) : 0.0f;
  return ct::fadd(ct::fsub(lo0, hi0), ct::fsub(lo1, hi1));
}

// (D^T D q) at (i, j), append=0 differences over both axes.
__device__ __forceinline__ float dtd_at(const float* __restrict__ q, int i, int j, int R, int C) {
  const size_t e = (size_t)i * C + j;
  const float qc = q[e];
  const float lo0 = i >= 1 ? ct::fsub(qc, q[e - C]) : 0.0f;
  const float hi0 = i <= R - 2 ? ct::fsub(q[e + C], qc) : 0.0f;
  const float lo1 = j >= 1 ? ct::fsub(qc, q[e - 1]) : 0.0f;
  const float hi1 = j <= C - 2 ? ct::fsub(q[e + 1], qc) : 0.0f;
  return ct::fadd(ct::fsub(lo0, hi0), ct::fsub(lo1, hi1));
}

// D x at (i, j): (x[i+1,j]-x[i,j], x[i,j+1]-x[i,j]); the appended last
// difference along an axis is x - x.
__device__ __forceinline__ void d_at(const float* __restrict__ x, int i, int j, int R, int C,
                                     float& d0, float& d1) {
  const size_t e = (size_t)i * C + j;
  const float xc = x[e];
  d0 = ct::fsub(i <= R - 2 ? x[e + C] : xc, xc);
  d1 = ct::fsub(j <= C - 2 ? x[e + 1] : xc, xc);
}

__global__ void __launch_bounds__(NT) k_init_state(const float* __restrict__ x, float* __restrict__ z,
                                                   float* __restrict__ u, float* __restrict__ dz,
                                                   int R, int C, int ng) {
  const size_t N = (size_t)R * C;
  for (size_t e = (size_t)blockIdx.x * NT + threadIdx.x; e < N; e += (size_t)gridDim.x * NT) {
    float d0, d1;
    d_at(x, pix_i(e, C), (int)(e % C), R, C, d0, d1);
    for (int t = 0; t < ng; ++t) {
      float* zt = z + (size_t)t * 2 * N;
      zt[e] = d0;
      zt[N + e] = d1;
      u[(size_t)t * 2 * N + e] = 0.0f;
      u[(size_t)t * 2 * N + N + e] = 0.0f;
      dz[(size_t)t * 2 * N + e] = 0.0f;
      dz[(size_t)t * 2 * N + N + e] = 0.0f;
    }
  }
}

// out = c * (sum of the adjoint split partials), plain (used once for A^T y).
__global__ void __launch_bounds__(NT) k_scale_splits(const float* __restrict__ src, float* __restrict__ out,
                                                     size_t n, int nsplit, float c) {
  for (size_t e = (size_t)blockIdx.x * NT + threadIdx.x; e < n; e += (size_t)gridDim.x * NT) {
    float s = src[e];
    for (int k = 1; k < nsplit; ++k) s = ct::fadd(s, src[(size_t)k * n + e]);
    out[e] = ct::fmul(c, s);
  }
}

__global__ void __launch_bounds__(NT)
    k_rhs(const float* __restrict__ atyc, const float* __restrict__ z, const float* __restrict__ u,
          const float* __restrict__ dz, float* __restrict__ rhs, int R, int C, TermParams tp,
          double* __restrict__ slots, double* __restrict__ partials, unsigned int* __restrict__ ticket) {
  const size_t N = (size_t)R * C;
  double acc[1] = {0.0};
  for (size_t e = (size_t)blockIdx.x * NT + threadIdx.x; e < N; e += (size_t)gridDim.x * NT) {
    const int i = pix_i(e, C), j = (int)(e % C);
    float val = atyc[e];
    float dv = 0.0f;
    for (int t = 0; t < tp.ng; ++t) {
      const size_t o = (size_t)t * 2 * N;
      val = ct::fadd(val, ct::fmul(tp.rho, dT_at(z + o, u + o, i, j, R, C)));
      const float w = ct::fmul(tp.rho, dT_at(dz + o, nullptr, i, j, R, C));
      dv = (t == 0) ? w : ct::fadd(dv, w);
    }
    rhs[e] = val;
    acc[0] += (double)dv * (double)dv;
  }
  double tot[1];
  if (ct::grid_sumk_last<NT, 1>(acc, partials, ticket, tot)) slots[S_DUAL2] = tot[0];
}

__global__ void __launch_bounds__(NT)
    k_resid2(const float* __restrict__ sino, const float* __restrict__ y, size_t n,
             double* __restrict__ slots, double* __restrict__ partials, unsigned int* __restrict__ ticket) {
  if (slots[S_XCLEAN] != 0.0) return;  // x unchanged: S_RESID2 is current
  double acc[1] = {0.0};
  for (size_t e = (size_t)blockIdx.x * NT + threadIdx.x; e < n; e += (size_t)gridDim.x * NT) {
    const float d = ct::fsub(y[e], sino[e]);
    acc[0] += (double)d * (double)d;
  }
  double tot[1];
  if (ct::grid_sumk_last<NT, 1>(acc, partials, ticket, tot)) slots[S_RESID2] = tot[0];
}

// Writes the itstat record of the previous iteration (if there is one).
__global__ void k_itstat(double* __restrict__ itstat, double* __restrict__ slots, int max_records,
                         double scale, double lam21, double lam1, int final_call) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  if (slots[S_HAVE_PREV] != 0.0) {
    const int rec = (int)slots[S_REC];
    if (itstat && rec < max_records) {
      double* o = itstat + (size_t)rec * CT_ITSTAT_FIELDS;
      const double* cg = slots + S_CG;
      o[CT_ITSTAT_OBJECTIVE] = scale * slots[S_RESID2] + lam21 * slots[S_G21] + lam1 * slots[S_G1];
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
  slots[S_HAVE_PREV] = final_call ? 0.0 : slots[S_HAVE_PREV];
}

// lhs(q) = sum_i rho D^T D q + c A^T A q, from the adjoint output (or its
// view splits).  INIT (q = x): r = rhs - lhs(x), p = r and the CG start
// scalars; lhs(x) is stored in lhsx, or read from it while x is unchanged
// (slots[S_XCLEAN]).  PAP: Ap = lhs(q) and <q, Ap>.  In a graph with a
// conditional CG loop, INIT sets the loop condition.
template <bool INIT>
__global__ void __launch_bounds__(NT)
    k_lhs_finish(const float* __restrict__ adj, int nsplit, const float* __restrict__ q, int R, int C,
                 TermParams tp, float* __restrict__ out, const float* __restrict__ rhs,
                 float* __restrict__ p, float* __restrict__ lhsx, double* __restrict__ slots,
                 double* __restrict__ cg, double tol, double atol, int maxiter,
                 double* __restrict__ partials, unsigned int* __restrict__ ticket,
                 cudaGraphConditionalHandle cond, int use_cond) {
  if (!INIT && cg[CT_CG_DONE] != 0.0) return;
  const bool cached = INIT && slots[S_XCLEAN] != 0.0;
  const size_t N = (size_t)R * C;
  double acc[2] = {0.0, 0.0};
  for (size_t e = (size_t)blockIdx.x * NT + threadIdx.x; e < N; e += (size_t)gridDim.x * NT) {
    float v;
    if (cached) {
      v = lhsx[e];
    } else {
      float a = adj[e];
      for (int k = 1; k < nsplit; ++k) a = ct::fadd(a, adj[(size_t)k * N + e]);
      const float g = dtd_at(q, pix_i(e, C), (int)(e % C), R, C);
      v = ct::fmul(tp.rho, g);
      for (int t = 1; t < tp.ng; ++t) v = ct::fadd(v, ct::fmul(tp.rho, g));
      v = ct::fadd(v, ct::fmul(tp.c, a));
      if (INIT) lhsx[e] = v;
    }
    if (INIT) {
      const float b = rhs[e];
      const float re = ct::fsub(b, v);
      out[e] = re;  // r
      p[e] = re;
      acc[0] += (double)re * (double)re;
      acc[1] += (double)b * (double)b;
    } else {
      out[e] = v;  // Ap
      acc[0] += (double)q[e] * (double)v;
    }
  }
  double tot[2];
  if (ct::grid_sumk_last<NT, 2>(acc, partials, ticket, tot)) {
    if (INIT) {
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

__device__ __forceinline__ void prox_pair(int kind, float thr, float v0, float v1, float& z0, float& z1) {
  if (kind == 0) {  // L2,1 over the two difference components
    const float len = __fsqrt_rn(ct::fadd(ct::fmul(v0, v0), ct::fmul(v1, v1)));
    float nl = ct::fsub(len, thr);
    nl = ct::fmul(0.5f, ct::fadd(nl, fabsf(nl)));
    z0 = ct::fmul(nl, len != 0.0f ? __fdiv_rn(v0, len) : 0.0f);
    z1 = ct::fmul(nl, len != 0.0f ? __fdiv_rn(v1, len) : 0.0f);
  } else {  // L1
    auto soft = [&](float v) {
      float t = ct::fsub(fabsf(v), thr);
      t = ct::fmul(0.5f, ct::fadd(t, fabsf(t)));
      const float sg = v > 0.0f ? 1.0f : (v < 0.0f ? -1.0f : (v == 0.0f ? 0.0f : v));
      return ct::fmul(sg, t);
    };
    z0 = soft(v0);
    z1 = soft(v1);
  }
}

__global__ void __launch_bounds__(NT)
    k_zu(const float* __restrict__ x, float* __restrict__ z, float* __restrict__ u, float* __restrict__ dz,
         int R, int C, TermParams tp, double* __restrict__ slots, double* __restrict__ partials,
         unsigned int* __restrict__ ticket) {
  const size_t N = (size_t)R * C;
  double acc[3] = {0.0, 0.0, 0.0};  // primal, g21, g1
  for (size_t e = (size_t)blockIdx.x * NT + threadIdx.x; e < N; e += (size_t)gridDim.x * NT) {
    float d0, d1;
    d_at(x, pix_i(e, C), (int)(e % C), R, C, d0, d1);
    for (int t = 0; t < tp.ng; ++t) {
      const size_t o = (size_t)t * 2 * N;
      const float zo0 = z[o + e], zo1 = z[o + N + e];
      float c0 = d0, c1 = d1;
      if (tp.alpha != 1.0f) {
        const float om = ct::fsub(1.0f, tp.alpha);
        c0 = ct::fadd(ct::fmul(tp.alpha, d0), ct::fmul(om, zo0));
        c1 = ct::fadd(ct::fmul(tp.alpha, d1), ct::fmul(om, zo1));
      }
      const float v0 = ct::fadd(c0, u[o + e]);
      const float v1 = ct::fadd(c1, u[o + N + e]);
      float z0, z1;
      prox_pair(tp.kind[t], tp.thr[t], v0, v1, z0, z1);
      z[o + e] = z0;
      z[o + N + e] = z1;
      u[o + e] = ct::fsub(v0, z0);
      u[o + N + e] = ct::fsub(v1, z1);
      dz[o + e] = ct::fsub(z0, zo0);
      dz[o + N + e] = ct::fsub(z1, zo1);
      const double p0 = (double)d0 - (double)z0, p1 = (double)d1 - (double)z1;
      acc[0] += (double)tp.rho * (p0 * p0 + p1 * p1);
      if (tp.kind[t] == 0)
        acc[1] += (double)__fsqrt_rn(ct::fadd(ct::fmul(z0, z0), ct::fmul(z1, z1)));
      else
        acc[2] += fabs((double)z0) + fabs((double)z1);
    }
  }
  double tot[3];
  if (ct::grid_sumk_last<NT, 3>(acc, partials, ticket, tot)) {
    slots[S_PRIMAL2] = tot[0];
    slots[S_G21] = tot[1];
    slots[S_G1] = tot[2];
    slots[S_HAVE_PREV] = 1.0;
    if (slots[S_CG + CT_CG_ITERS] > 0.0) slots[S_XCLEAN] = 0.0;  // CG moved x
  }
}

__global__ void k_reset_call(double* __restrict__ slots) {
  slots[S_REC] = 0.0;
  slots[S_HAVE_PREV] = 0.0;
  slots[S_XCLEAN] = 0.0;  // the caller may have changed x between calls
}

// ---------------------------------------------------------------------------

struct Layout {
  size_t N, S;
  int ng;
  ct::Proj2dPlan plan;
  size_t off_slots, off_red, off_atyc, off_rhs, off_r, off_p, off_ap, off_adj, off_sino, off_z, off_u,
      off_dz, off_fwd, off_adjpart, off_lhsx, off_sinox, total;
};

Layout layout(const ct_admm_tv_desc* d) {
  Layout L;
  const ct_geom2d* g = &d->geom;
  L.N = (size_t)g->rows * g->cols;
  L.S = (size_t)g->n_views * g->det_count;
  L.ng = (d->lam_l21 != 0.0) + (d->lam_l1 != 0.0);
  L.plan = ct::proj2d_plan(g, 1);
  size_t o = 0;
  auto take = [&](size_t bytes) {
    const size_t at = o;
    o += ct::round_up(bytes, 256);
    return at;
  };
  L.off_slots = take(S_COUNT * sizeof(double));
  L.off_red = take(ct::kReduceWorkspace);
  L.off_atyc = take(L.N * 4);
  L.off_rhs = take(L.N * 4);
  L.off_r = take(L.N * 4);
  L.off_p = take(L.N * 4);
  L.off_ap = take(L.N * 4);
  L.off_adj = take(L.N * 4);
  L.off_sino = take(L.S * 4);
  L.off_z = take(L.N * 8 * (size_t)(L.ng > 0 ? L.ng : 1));
  L.off_u = take(L.N * 8 * (size_t)(L.ng > 0 ? L.ng : 1));
  L.off_dz = take(L.N * 8 * (size_t)(L.ng > 0 ? L.ng : 1));
  L.off_fwd = take(L.plan.fwd_bytes);
  L.off_adjpart = take(L.plan.adj_bytes > 0 ? L.plan.adj_bytes : 256);
  L.off_lhsx = take(L.N * 4);
  L.off_sinox = take(L.S * 4);
  L.total = o;
  return L;
}

ct_status check_desc(const ct_admm_tv_desc* d, const char* who) {
  if (!d) return ct::fail(CT_ERR_INVALID_ARG, "%s: null descriptor", who);
  ct_status st = ct::proj2d_check(&d->geom, who);
  if (st != CT_OK) return st;
  if (d->maxiter < 0 || d->cg_maxiter < 0)
    return ct::fail(CT_ERR_INVALID_ARG, "%s: maxiter=%d cg_maxiter=%d", who, d->maxiter, d->cg_maxiter);
  if ((d->lam_l21 != 0.0) + (d->lam_l1 != 0.0) == 0)
    return ct::fail(CT_ERR_INVALID_ARG, "%s: at least one of lam_l21, lam_l1 must be non-zero", who);
  if (!(d->rho > 0.0)) return ct::fail(CT_ERR_INVALID_ARG, "%s: rho must be > 0", who);
  return CT_OK;
}

struct Ctx {
  const ct_admm_tv_desc* d;
  Layout L;
  char* ws;
  const float* y;
  float* x;
  double* itstat;
  TermParams tp;
  template <class T>
  T* at(size_t off) const { return reinterpret_cast<T*>(ws + off); }
  double* slots() const { return at<double>(L.off_slots); }
  double* cg() const { return slots() + S_CG; }
  unsigned int* ticket() const { return at<unsigned int>(L.off_red); }
  double* partials() const { return reinterpret_cast<double*>(ws + L.off_red + 256); }
};

#define CT_TRY(expr)                 \
  do {                               \
    ct_status _st = (expr);          \
    if (_st != CT_OK) return _st;    \
  } while (0)

ct_status project(const Ctx& c, const float* img, float* sino, cudaStream_t s, const double* skip) {
  return ct::proj2d_fwd_launch(&c.d->geom, c.L.plan, img, sino, 1, c.at<float>(c.L.off_fwd), s, skip);
}

// A^T of a sinogram into the adjoint buffer (or its view splits); returns
// the buffer to read.
const float* backproject(const Ctx& c, const float* sino, cudaStream_t s, const double* skip, ct_status& st) {
  float* adj = c.at<float>(c.L.off_adj);
  float* part = c.at<float>(c.L.off_adjpart);
  st = ct::proj2d_adj_launch(&c.d->geom, c.L.plan, sino, adj, part, 1, s, skip);
  return c.L.plan.nsplit > 1 ? part : adj;
}

// The three phases of one ADMM iteration.  cond/use_cond: the conditional
// handle of the graph's CG loop (use_cond = 0 outside such a graph).
ct_status enqueue_pre(const Ctx& c, cudaStream_t s, cudaGraphConditionalHandle cond, int use_cond) {
  const int R = c.d->geom.rows, C = c.d->geom.cols;
  float* r = c.at<float>(c.L.off_r);
  float* p = c.at<float>(c.L.off_p);
  float* rhs = c.at<float>(c.L.off_rhs);
  float* sinox = c.at<float>(c.L.off_sinox);
  const double* clean = c.slots() + S_XCLEAN;
  k_rhs<<<NB, NT, 0, s>>>(c.at<float>(c.L.off_atyc), c.at<float>(c.L.off_z), c.at<float>(c.L.off_u),
                          c.at<float>(c.L.off_dz), rhs, R, C, c.tp, c.slots(), c.partials(), c.ticket());
  CT_TRY(ct::launch_check("k_rhs"));
  CT_TRY(project(c, c.x, sinox, s, clean));
  k_resid2<<<NB, NT, 0, s>>>(sinox, c.y, c.L.S, c.slots(), c.partials(), c.ticket());
  CT_TRY(ct::launch_check("k_resid2"));
  k_itstat<<<1, 32, 0, s>>>(c.itstat, c.slots(), c.d->maxiter, c.d->loss_scale, c.d->lam_l21, c.d->lam_l1, 0);
  CT_TRY(ct::launch_check("k_itstat"));
  ct_status st;
  const float* adj = backproject(c, sinox, s, clean, st);
  CT_TRY(st);
  k_lhs_finish<true><<<NB, NT, 0, s>>>(adj, c.L.plan.nsplit, c.x, R, C, c.tp, r, rhs, p,
                                       c.at<float>(c.L.off_lhsx), c.slots(), c.cg(), c.d->cg_tol,
                                       c.d->cg_atol, c.d->cg_maxiter, c.partials(), c.ticket(), cond, use_cond);
  return ct::launch_check("k_lhs_finish<init>");
}

ct_status enqueue_cg_step(const Ctx& c, cudaStream_t s, cudaGraphConditionalHandle cond, int use_cond) {
  const int R = c.d->geom.rows, C = c.d->geom.cols;
  float* r = c.at<float>(c.L.off_r);
  float* p = c.at<float>(c.L.off_p);
  float* ap = c.at<float>(c.L.off_ap);
  float* sino = c.at<float>(c.L.off_sino);
  const double* done = c.cg() + CT_CG_DONE;
  CT_TRY(project(c, p, sino, s, done));
  ct_status st;
  const float* adj = backproject(c, sino, s, done, st);
  CT_TRY(st);
  k_lhs_finish<false><<<NB, NT, 0, s>>>(adj, c.L.plan.nsplit, p, R, C, c.tp, ap, nullptr, nullptr, nullptr,
                                        c.slots(), c.cg(), 0.0, 0.0, c.d->cg_maxiter, c.partials(), c.ticket(),
                                        0, 0);
  CT_TRY(ct::launch_check("k_lhs_finish<pap>"));
  CT_TRY(ct::cg_update_launch(c.x, r, p, ap, c.L.N, c.cg(), c.ws + c.L.off_red, s, cond, use_cond));
  return ct::cg_direction_launch(p, r, c.L.N, c.cg(), c.ws + c.L.off_red, s);
}

ct_status enqueue_post(const Ctx& c, cudaStream_t s) {
  const int R = c.d->geom.rows, C = c.d->geom.cols;
  k_zu<<<NB, NT, 0, s>>>(c.x, c.at<float>(c.L.off_z), c.at<float>(c.L.off_u), c.at<float>(c.L.off_dz), R, C,
                         c.tp, c.slots(), c.partials(), c.ticket());
  return ct::launch_check("k_zu");
}

// One iteration as plain launches (no graph): cg_maxiter CG steps that turn
// into no-ops once CG has converged.
ct_status enqueue_iteration(const Ctx& c, cudaStream_t s) {
  CT_TRY(enqueue_pre(c, s, 0, 0));
  for (int it = 0; it < c.d->cg_maxiter; ++it) CT_TRY(enqueue_cg_step(c, s, 0, 0));
  return enqueue_post(c, s);
}

// Statistics of the last iteration: dual residual (k_rhs), objective.
ct_status enqueue_epilogue(const Ctx& c, cudaStream_t s) {
  const int R = c.d->geom.rows, C = c.d->geom.cols;
  float* sinox = c.at<float>(c.L.off_sinox);
  k_rhs<<<NB, NT, 0, s>>>(c.at<float>(c.L.off_atyc), c.at<float>(c.L.off_z), c.at<float>(c.L.off_u),
                          c.at<float>(c.L.off_dz), c.at<float>(c.L.off_rhs), R, C, c.tp, c.slots(),
                          c.partials(), c.ticket());
  CT_TRY(ct::launch_check("k_rhs"));
  CT_TRY(project(c, c.x, sinox, s, c.slots() + S_XCLEAN));
  k_resid2<<<NB, NT, 0, s>>>(sinox, c.y, c.L.S, c.slots(), c.partials(), c.ticket());
  CT_TRY(ct::launch_check("k_resid2"));
  k_itstat<<<1, 32, 0, s>>>(c.itstat, c.slots(), c.d->maxiter, c.d->loss_scale, c.d->lam_l21, c.d->lam_l1, 1);
  return ct::launch_check("k_itstat");
}

// One cached executable graph of the iteration body (per process).
struct GraphCache {
  std::mutex m;
  unsigned char key[512];
  size_t key_len = 0;
  int device = -1;
  cudaGraphExec_t exec = nullptr;
  cudaStream_t cs = nullptr;
  cudaEvent_t ev_in = nullptr, ev_out = nullptr;
};
GraphCache g_cache;

size_t make_key(const Ctx& c, unsigned char* key) {
  size_t n = 0;
  auto put = [&](const void* p, size_t b) {
    memcpy(key + n, p, b);
    n += b;
  };
  put(c.d, sizeof(ct_admm_tv_desc));
  put(&c.ws, sizeof(c.ws));
  put(&c.y, sizeof(c.y));
  put(&c.x, sizeof(c.x));
  put(&c.itstat, sizeof(c.itstat));
  return n;
}

// The iteration graph: pre-phase kernels, then a conditional WHILE node
// whose body is one CG step (the CG start and every CG update set the
// condition on the device: run while CG has not converged), then the z/u
// update.  Each phase is stream-captured into its place in the graph.
ct_status build_iteration_graph(const Ctx& c, cudaStream_t cs, cudaGraph_t& graph) {
  CT_TRY(ct::cuda_check(cudaGraphCreate(&graph, 0), "graph create"));
  cudaGraphConditionalHandle cond = 0;
  CT_TRY(ct::cuda_check(cudaGraphConditionalHandleCreate(&cond, graph, 0, cudaGraphCondAssignDefault),
                        "conditional handle"));
  // pre phase
  CT_TRY(ct::cuda_check(cudaStreamBeginCaptureToGraph(cs, graph, nullptr, nullptr, 0,
                                                      cudaStreamCaptureModeThreadLocal),
                        "capture pre"));
  ct_status st = enqueue_pre(c, cs, cond, 1);
  cudaStreamCaptureStatus cst;
  const cudaGraphNode_t* deps = nullptr;
  size_t ndeps = 0;
  cudaError_t ce = cudaStreamGetCaptureInfo(cs, &cst, nullptr, nullptr, &deps, nullptr, &ndeps);
  cudaGraphNode_t pre_tail[8];
  const size_t npre = ndeps < 8 ? ndeps : 8;
  for (size_t k = 0; ce == cudaSuccess && k < npre; ++k) pre_tail[k] = deps[k];
  cudaGraph_t out = nullptr;
  cudaError_t ce2 = cudaStreamEndCapture(cs, &out);
  CT_TRY(st);
  CT_TRY(ct::cuda_check(ce, "capture info"));
  CT_TRY(ct::cuda_check(ce2, "end capture pre"));
  if (ndeps > 8) return ct::fail(CT_ERR_CUDA, "unexpected capture frontier of %zu nodes", ndeps);
  // conditional WHILE node for the CG loop
  cudaGraphNodeParams cp = {};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = cond;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  cudaGraphNode_t cnode = nullptr;
  CT_TRY(ct::cuda_check(cudaGraphAddNode(&cnode, graph, pre_tail, nullptr, npre, &cp), "conditional node"));
  cudaGraph_t body = cp.conditional.phGraph_out[0];
  CT_TRY(ct::cuda_check(cudaStreamBeginCaptureToGraph(cs, body, nullptr, nullptr, 0,
                                                      cudaStreamCaptureModeThreadLocal),
                        "capture body"));
  st = enqueue_cg_step(c, cs, cond, 1);
  ce2 = cudaStreamEndCapture(cs, &out);
  CT_TRY(st);
  CT_TRY(ct::cuda_check(ce2, "end capture body"));
  // post phase after the loop
  CT_TRY(ct::cuda_check(cudaStreamBeginCaptureToGraph(cs, graph, &cnode, nullptr, 1,
                                                      cudaStreamCaptureModeThreadLocal),
                        "capture post"));
  st = enqueue_post(c, cs);
  ce2 = cudaStreamEndCapture(cs, &out);
  CT_TRY(st);
  return ct::cuda_check(ce2, "end capture post");
}

ct_status run_graph(const Ctx& c, cudaStream_t caller) {
  std::lock_guard<std::mutex> lock(g_cache.m);
  int dev = 0;
  CT_TRY(ct::cuda_check(cudaGetDevice(&dev), "cudaGetDevice"));
  if (g_cache.device != dev) {
    if (g_cache.exec) cudaGraphExecDestroy(g_cache.exec);
    g_cache.exec = nullptr;
    g_cache.key_len = 0;
    CT_TRY(ct::cuda_check(cudaStreamCreateWithFlags(&g_cache.cs, cudaStreamNonBlocking), "stream"));
    CT_TRY(ct::cuda_check(cudaEventCreateWithFlags(&g_cache.ev_in, cudaEventDisableTiming), "event"));
    CT_TRY(ct::cuda_check(cudaEventCreateWithFlags(&g_cache.ev_out, cudaEventDisableTiming), "event"));
    g_cache.device = dev;
  }
  unsigned char key[512];
  const size_t kl = make_key(c, key);
  if (!g_cache.exec || kl != g_cache.key_len || memcmp(key, g_cache.key, kl) != 0) {
    if (g_cache.exec) {
      cudaGraphExecDestroy(g_cache.exec);
      g_cache.exec = nullptr;
    }
    cudaGraph_t graph = nullptr;
    ct_status st = build_iteration_graph(c, g_cache.cs, graph);
    if (st != CT_OK) {
      if (graph) cudaGraphDestroy(graph);
      return st;
    }
    cudaError_t ce = cudaGraphInstantiate(&g_cache.exec, graph, 0);
    cudaGraphDestroy(graph);
    CT_TRY(ct::cuda_check(ce, "graph instantiate"));
    memcpy(g_cache.key, key, kl);
    g_cache.key_len = kl;
  }
  CT_TRY(ct::cuda_check(cudaEventRecord(g_cache.ev_in, caller), "event record"));
  CT_TRY(ct::cuda_check(cudaStreamWaitEvent(g_cache.cs, g_cache.ev_in, 0), "stream wait"));
  for (int k = 0; k < c.d->maxiter; ++k)
    CT_TRY(ct::cuda_check(cudaGraphLaunch(g_cache.exec, g_cache.cs), "graph launch"));
  CT_TRY(ct::cuda_check(cudaEventRecord(g_cache.ev_out, g_cache.cs), "event record"));
  return ct::cuda_check(cudaStreamWaitEvent(caller, g_cache.ev_out, 0), "stream wait");
}

}  // namespace

extern "C" {

ct_status ct_admm_tv_workspace(const ct_admm_tv_desc* d, size_t* bytes) {
  CT_TRY(check_desc(d, "ct_admm_tv_workspace"));
  if (!bytes) return ct::fail(CT_ERR_INVALID_ARG, "ct_admm_tv_workspace: null bytes");
  *bytes = layout(d).total;
  return CT_OK;
}

ct_status ct_admm_tv_state(const ct_admm_tv_desc* d, size_t* z_offset, size_t* u_offset,
                           int32_t* n_terms) {
  CT_TRY(check_desc(d, "ct_admm_tv_state"));
  const Layout L = layout(d);
  if (z_offset) *z_offset = L.off_z;
  if (u_offset) *u_offset = L.off_u;
  if (n_terms) *n_terms = L.ng;
  return CT_OK;
}

ct_status ct_admm_tv_solve(const ct_admm_tv_desc* d, const float* y, float* x, double* itstat_dev,
                           int32_t iter0, void* workspace, size_t workspace_bytes, ct_stream_t stream) {
  CT_TRY(check_desc(d, "ct_admm_tv_solve"));
  if (!y || !x) return ct::fail(CT_ERR_INVALID_ARG, "ct_admm_tv_solve: null array");
  Ctx c;
  c.d = d;
  c.L = layout(d);
  if (!workspace || workspace_bytes < c.L.total || !ct::aligned(workspace, 256))
    return ct::fail(CT_ERR_WORKSPACE, "ct_admm_tv_solve: need %zu bytes (256-B aligned), got %zu",
                    c.L.total, workspace_bytes);
  c.ws = static_cast<char*>(workspace);
  c.y = y;
  c.x = x;
  c.itstat = itstat_dev;
  TermParams& tp = c.tp;
  tp.ng = 0;
  // The reference's prox parameter is (1/rho) * lam in float64, then float32.
  if (d->lam_l21 != 0.0) {
    tp.kind[tp.ng] = 0;
    tp.thr[tp.ng] = (float)((1.0 / d->rho) * d->lam_l21);
    ++tp.ng;
  }
  if (d->lam_l1 != 0.0) {
    tp.kind[tp.ng] = 1;
    tp.thr[tp.ng] = (float)((1.0 / d->rho) * d->lam_l1);
    ++tp.ng;
  }
  tp.rho = (float)d->rho;
  tp.alpha = (float)d->alpha;
  tp.c = (float)(2.0 * d->loss_scale);
  cudaStream_t s = ct::as_stream(stream);
  CT_TRY(ct::proj2d_prepare(c.L.plan));
  const int R = d->geom.rows, C = d->geom.cols;

  if (iter0 == 0) {
    CT_TRY(ct::cuda_check(cudaMemsetAsync(c.ws, 0, c.L.off_atyc, s), "memset state"));
    // A^T y, scaled by 2*scale (hoisted out of the loop: y is constant).
    CT_TRY(ct::proj2d_adj_launch(&d->geom, c.L.plan, y, c.at<float>(c.L.off_adj),
                                 c.at<float>(c.L.off_adjpart), 1, s, nullptr));
    const float* src = c.L.plan.nsplit > 1 ? c.at<float>(c.L.off_adjpart) : c.at<float>(c.L.off_adj);
    k_scale_splits<<<NB, NT, 0, s>>>(src, c.at<float>(c.L.off_atyc), c.L.N, c.L.plan.nsplit, tp.c);
    CT_TRY(ct::launch_check("k_scale_splits"));
    k_init_state<<<NB, NT, 0, s>>>(x, c.at<float>(c.L.off_z), c.at<float>(c.L.off_u),
                                   c.at<float>(c.L.off_dz), R, C, tp.ng);
    CT_TRY(ct::launch_check("k_init_state"));
  }
  k_reset_call<<<1, 1, 0, s>>>(c.slots());
  CT_TRY(ct::launch_check("k_reset_call"));
  if (d->maxiter == 0) return CT_OK;
  if (d->use_graph) {
    CT_TRY(run_graph(c, s));
  } else {
    for (int k = 0; k < d->maxiter; ++k) CT_TRY(enqueue_iteration(c, s));
  }
  return enqueue_epilogue(c, s);
}

}  // extern "C"
