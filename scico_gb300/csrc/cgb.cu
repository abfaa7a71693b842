// Unrolled fixed-iteration CG block of the MoDL network with a hand-written
// backward: scico.flax.inverse.cg_solver (scico/flax/inverse.py:113-158) on
// (s H^T H + lam I) x = b for nsys independent images sharing the 2D
// projector H (s = gram_scale, e.g. c^2 for a projector scaled by c), and the
// reverse-mode recurrence of its K steps.
//
// Forward step k (float32 vectors, float64 scalars, per system):
//   Ap_k = s H^T H p_k + lam p_k;  d_k = <p_k, Ap_k>;  a_k = num_k / d_k
//   x += a_k p_k;  r_{k+1} = r_k - a_k Ap_k;  num_{k+1} = <r_{k+1}, r_{k+1}>
//   b_k = num_{k+1} / num_k;  p_{k+1} = r_{k+1} + b_k p_k
// with r_0 = b - A x_0, p_0 = r_0.  The tape keeps p_k, Ap_k, r_k and the
// scalars; with recompute it keeps only the scalars, and the backward reruns
// the forward from the block's inputs (its checkpoint) into the workspace.
//
// Backward step k, adjoints xb, rb, pb (of p_{k+1}), numb (of num_{k+1}):
//   bb = <pb, p_k>;  numb' = numb + bb / num_k;  nk = -bb num_{k+1} / num_k^2
//   rb += pb + 2 numb' r_{k+1};  ab = <xb, p_k> - <rb, Ap_k>
//   nk += ab / d_k;  db = -ab num_k / d_k^2
//   Apb = -a_k rb + db p_k;  lamb += <Apb, p_k>
//   pb = b_k pb + a_k xb + db Ap_k + A Apb;  numb = nk
// then rb_0 = rb + pb + 2 numb r_0 is the gradient of b, xb - A rb_0 that of
// x_0 and -<rb_0, x_0> is added to lamb.  Reductions are deterministic
// (fixed per-system trees), no float atomics.
#include <math.h>

#include <algorithm>

#include "kernels.cuh"

namespace {

constexpr int NT = ct::kReduceThreads;

// Per-system scalar block (doubles): running values, then one record per step.
enum { C_NUM = 0, C_NUMB = 1, C_LAMB = 2, C_NK = 3, C_DB = 4, C_HEAD = 8, C_REC = 5 };
enum { R_NUM = 0, R_D = 1, R_A = 2, R_B = 3, R_NUMN = 4 };

struct Sys {
  int nsys, nb;
  size_t n;
  int stride;  // doubles per system in the scalar block
};

__device__ __forceinline__ double* sys_scal(double* scal, const Sys& s, int sy) { return scal + (size_t)sy * s.stride; }
__device__ __forceinline__ double* rec(double* scal, const Sys& s, int sy, int k) {
  return sys_scal(scal, s, sy) + C_HEAD + C_REC * k;
}

// Reduction of K (<= 4) sums over the blocks of one system (grid = (nb, nsys));
// true in thread 0 of the system's last block.
template <int K>
__device__ __forceinline__ bool sys_reduce(double (&v)[K], double* partials, unsigned int* tickets, const Sys& s,
                                           double (&out)[K]) {
  return ct::grid_reduce_last<NT, K>(v, partials + (size_t)blockIdx.y * 4 * s.nb, tickets + blockIdx.y, out);
}

#define FOR_SYS(e, s)                                                     \
  const int sy = blockIdx.y;                                              \
  const size_t base = (size_t)sy * (s).n;                                 \
  for (size_t e = base + (size_t)blockIdx.x * NT + threadIdx.x; e < base + (s).n; e += (size_t)(s).nb * NT)

__global__ void __launch_bounds__(NT)
    k_cgb_init(const float* __restrict__ b, const float* __restrict__ ax0, float* __restrict__ r0,
               float* __restrict__ p0, Sys s, double* __restrict__ scal, double* __restrict__ partials,
               unsigned int* __restrict__ tickets) {
  double nn = 0.0;
  FOR_SYS(e, s) {
    const float r = ax0 ? ct::fsub(b[e], ax0[e]) : b[e];
    r0[e] = r;
    p0[e] = r;
    nn += (double)r * (double)r;
  }
  double v[1] = {nn}, out[1];
  if (sys_reduce<1>(v, partials, tickets, s, out)) sys_scal(scal, s, sy)[C_NUM] = out[0];
}

// ax = gs t + lam x (t = H^T H x); ax may be t itself.
__global__ void __launch_bounds__(NT)
    k_cgb_axpy(const float* t, const float* __restrict__ x, float* ax, float gs, float lam, Sys s) {
  FOR_SYS(e, s) ax[e] = ct::fadd(ct::fmul(gs, t[e]), ct::fmul(lam, x[e]));
}

// Ap = gs t + lam p (t = H^T H p), d = <p, Ap>, a = num / d.
__global__ void __launch_bounds__(NT)
    k_cgb_ap(const float* __restrict__ t, const float* __restrict__ p, float* __restrict__ ap, float gs, float lam,
             int k, Sys s, double* __restrict__ scal, double* __restrict__ partials, unsigned int* __restrict__ tickets) {
  double d = 0.0;
  FOR_SYS(e, s) {
    const float pe = p[e];
    const float a = ct::fadd(ct::fmul(gs, t[e]), ct::fmul(lam, pe));
    ap[e] = a;
    d += (double)pe * (double)a;
  }
  double v[1] = {d}, out[1];
  if (sys_reduce<1>(v, partials, tickets, s, out)) {
    const double num = sys_scal(scal, s, sy)[C_NUM];
    double* r = rec(scal, s, sy, k);
    r[R_NUM] = num;
    r[R_D] = out[0];
    r[R_A] = num / out[0];
  }
}

// x += a p; r' = r - a Ap; num' = <r', r'>; b = num' / num.
__global__ void __launch_bounds__(NT)
    k_cgb_upd(float* __restrict__ x, const float* __restrict__ r, float* __restrict__ rn, const float* __restrict__ p,
              const float* __restrict__ ap, int k, Sys s, double* __restrict__ scal, double* __restrict__ partials,
              unsigned int* __restrict__ tickets) {
  const float a = (float)rec(scal, s, blockIdx.y, k)[R_A];
  double nn = 0.0;
  FOR_SYS(e, s) {
    x[e] = ct::fadd(x[e], ct::fmul(a, p[e]));
    const float v = ct::fsub(r[e], ct::fmul(a, ap[e]));
    rn[e] = v;
    nn += (double)v * (double)v;
  }
  double v[1] = {nn}, out[1];
  if (sys_reduce<1>(v, partials, tickets, s, out)) {
    double* rr = rec(scal, s, sy, k);
    rr[R_NUMN] = out[0];
    rr[R_B] = out[0] / rr[R_NUM];
    sys_scal(scal, s, sy)[C_NUM] = out[0];
  }
}

// p' = r' + b p.
__global__ void __launch_bounds__(NT)
    k_cgb_dir(const float* __restrict__ rn, const float* __restrict__ p, float* __restrict__ pn, int k, Sys s,
              double* __restrict__ scal) {
  const float bt = (float)rec(scal, s, blockIdx.y, k)[R_B];
  FOR_SYS(e, s) pn[e] = ct::fadd(rn[e], ct::fmul(bt, p[e]));
}

// The backward's running scalars (numb, lamb) start at zero.
__global__ void k_cgb_reset(double* __restrict__ scal, Sys s) {
  for (int sy = threadIdx.x; sy < s.nsys; sy += blockDim.x) {
    scal[(size_t)sy * s.stride + C_NUMB] = 0.0;
    scal[(size_t)sy * s.stride + C_LAMB] = 0.0;
  }
}

// pb += gs t + lam Apb (the A Apb term of the previous backward step, when
// t != null); then, for k >= 0: bb = <pb, p_k>, numb' = numb + bb / num_k,
// nk = -bb num_{k+1} / num_k^2.
__global__ void __launch_bounds__(NT)
    k_cgb_b1(float* __restrict__ pb, const float* __restrict__ t, const float* __restrict__ apb, float gs, float lam,
             const float* __restrict__ pk, int k, Sys s, double* __restrict__ scal, double* __restrict__ partials,
             unsigned int* __restrict__ tickets) {
  double bb = 0.0;
  FOR_SYS(e, s) {
    float v = pb[e];
    if (t) {
      v = ct::fadd(v, ct::fadd(ct::fmul(gs, t[e]), ct::fmul(lam, apb[e])));
      pb[e] = v;
    }
    if (k >= 0) bb += (double)v * (double)pk[e];
  }
  if (k < 0) return;  // uniform over the grid
  double v[1] = {bb}, out[1];
  if (sys_reduce<1>(v, partials, tickets, s, out)) {
    double* c = sys_scal(scal, s, sy);
    const double* r = rec(scal, s, sy, k);
    c[C_NUMB] += out[0] / r[R_NUM];
    c[C_NK] = -out[0] * r[R_NUMN] / (r[R_NUM] * r[R_NUM]);
  }
}

// rb += pb + 2 numb' r_{k+1};  ab = <xb, p_k> - <rb, Ap_k>;
// numb = nk + ab / d_k;  db = -ab num_k / d_k^2.
__global__ void __launch_bounds__(NT)
    k_cgb_b2(float* __restrict__ rb, const float* __restrict__ pb, const float* __restrict__ rn,
             const float* __restrict__ xb, const float* __restrict__ pk, const float* __restrict__ apk, int k, Sys s,
             double* __restrict__ scal, double* __restrict__ partials, unsigned int* __restrict__ tickets) {
  const float tn = (float)(2.0 * sys_scal(scal, s, blockIdx.y)[C_NUMB]);
  double s_xp = 0.0, s_ra = 0.0;
  FOR_SYS(e, s) {
    const float v = ct::fadd(ct::fadd(rb[e], pb[e]), ct::fmul(tn, rn[e]));
    rb[e] = v;
    s_xp += (double)xb[e] * (double)pk[e];
    s_ra += (double)v * (double)apk[e];
  }
  double v[2] = {s_xp, s_ra}, out[2];
  if (sys_reduce<2>(v, partials, tickets, s, out)) {
    double* c = sys_scal(scal, s, sy);
    const double* r = rec(scal, s, sy, k);
    const double ab = out[0] - out[1];
    c[C_NUMB] = c[C_NK] + ab / r[R_D];
    c[C_DB] = -ab * r[R_NUM] / (r[R_D] * r[R_D]);
  }
}

// Apb = -a_k rb + db p_k;  pb = b_k pb + a_k xb + db Ap_k;  lamb += <Apb, p_k>.
__global__ void __launch_bounds__(NT)
    k_cgb_b3(const float* __restrict__ rb, const float* __restrict__ xb, float* __restrict__ pb,
             float* __restrict__ apb, const float* __restrict__ pk, const float* __restrict__ apk, int k, Sys s,
             double* __restrict__ scal, double* __restrict__ partials, unsigned int* __restrict__ tickets) {
  const double* r = rec(scal, s, blockIdx.y, k);
  const float a = (float)r[R_A], bt = (float)r[R_B], db = (float)sys_scal(scal, s, blockIdx.y)[C_DB];
  double lb = 0.0;
  FOR_SYS(e, s) {
    const float p = pk[e];
    const float g = ct::fadd(ct::fmul(-a, rb[e]), ct::fmul(db, p));
    apb[e] = g;
    pb[e] = ct::fadd(ct::fadd(ct::fmul(bt, pb[e]), ct::fmul(a, xb[e])), ct::fmul(db, apk[e]));
    lb += (double)g * (double)p;
  }
  double v[1] = {lb}, out[1];
  if (sys_reduce<1>(v, partials, tickets, s, out)) sys_scal(scal, s, sy)[C_LAMB] += out[0];
}

// gb = rb + pb + 2 numb r_0 (the adjoint of r_0, which is that of b).
__global__ void __launch_bounds__(NT)
    k_cgb_rb0(const float* __restrict__ rb, const float* __restrict__ pb, const float* __restrict__ r0,
              float* __restrict__ gb, Sys s, double* __restrict__ scal) {
  const float tn = (float)(2.0 * sys_scal(scal, s, blockIdx.y)[C_NUMB]);
  FOR_SYS(e, s) gb[e] = ct::fadd(ct::fadd(rb[e], pb[e]), ct::fmul(tn, r0[e]));
}

// gx0 = xb - (gs t + lam gb) (t = H^T H gb, gx0 may be null);  lamb -= <gb, x0>.
__global__ void __launch_bounds__(NT)
    k_cgb_x0(const float* __restrict__ xb, const float* __restrict__ t, const float* __restrict__ gb,
             const float* __restrict__ x0, float* __restrict__ gx0, float gs, float lam, Sys s,
             double* __restrict__ scal, double* __restrict__ partials, unsigned int* __restrict__ tickets) {
  double lb = 0.0;
  FOR_SYS(e, s) {
    const float g = gb[e];
    if (gx0) gx0[e] = ct::fsub(xb[e], ct::fadd(ct::fmul(gs, t[e]), ct::fmul(lam, g)));
    lb += (double)g * (double)x0[e];
  }
  double v[1] = {lb}, out[1];
  if (sys_reduce<1>(v, partials, tickets, s, out)) sys_scal(scal, s, sy)[C_LAMB] -= out[0];
}

// glam = sum of the systems' lamb, in system order.
__global__ void k_cgb_lamsum(const double* __restrict__ scal, Sys s, double* __restrict__ glam) {
  double acc = 0.0;
  for (int sy = 0; sy < s.nsys; ++sy) acc += scal[(size_t)sy * s.stride + C_LAMB];
  *glam = acc;
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

#define CT_TRY(expr)              \
  do {                            \
    ct_status _st = (expr);       \
    if (_st != CT_OK) return _st; \
  } while (0)

struct Plan {
  Sys s;
  ct::Proj2dPlan p2;
  size_t vec;  // bytes of one batched vector
  size_t tape_vectors, tape_scal, tape_total;
  size_t ws_red, ws_proj, ws_sino, ws_tmp, ws_recompute, ws_total;
};

// Tape: P[K], AP[K], R[K+1] (none with recompute), then the scalars.
// Workspace: reduction area, projector scratch, sinogram, t and the
// backward's rb, pb, xb, apb, gb; with recompute also P, AP, R and x.
Plan plan_of(const ct_cg_block_desc* d) {
  Plan P;
  const size_t n = (size_t)d->geom.rows * d->geom.cols;
  const int K = d->maxiter;
  P.s.nsys = d->nsys;
  P.s.n = n;
  P.s.nb = (int)std::min<size_t>(64, std::max<size_t>(1, (n + 8 * NT - 1) / (8 * NT)));
  P.s.stride = C_HEAD + C_REC * K;
  P.p2 = ct::proj2d_plan(&d->geom, d->nsys);
  P.vec = ct::round_up((size_t)d->nsys * n * sizeof(float), 256);
  const size_t vectors = (size_t)(3 * K + 1) * P.vec;
  P.tape_vectors = d->recompute ? 0 : vectors;
  P.tape_scal = ct::round_up((size_t)d->nsys * P.s.stride * sizeof(double), 256);
  P.tape_total = P.tape_vectors + P.tape_scal;
  P.ws_red = ct::round_up((size_t)d->nsys * sizeof(unsigned int), 256) +
             ct::round_up((size_t)d->nsys * 4 * P.s.nb * sizeof(double), 256);
  P.ws_proj = ct::round_up(std::max<size_t>(std::max(P.p2.fwd_bytes, P.p2.adj_ws_bytes), 256), 256);
  P.ws_sino = ct::round_up((size_t)d->nsys * d->geom.n_views * d->geom.det_count * sizeof(float), 256);
  P.ws_tmp = 6 * P.vec;
  P.ws_recompute = d->recompute ? vectors + P.vec : 0;
  P.ws_total = P.ws_red + P.ws_proj + P.ws_sino + P.ws_tmp + P.ws_recompute;
  return P;
}

ct_status check(const ct_cg_block_desc* d, const char* who) {
  if (!d) return ct::fail(CT_ERR_INVALID_ARG, "%s: null descriptor", who);
  CT_TRY(ct::proj2d_check(&d->geom, who));
  if (d->nsys <= 0 || d->maxiter < 0)
    return ct::fail(CT_ERR_INVALID_ARG, "%s: nsys=%d maxiter=%d", who, d->nsys, d->maxiter);
  if (d->nsys > 65535) return ct::fail(CT_ERR_UNSUPPORTED, "%s: nsys=%d above 65535", who, d->nsys);
  return CT_OK;
}

struct Bufs {
  unsigned int* tickets;
  double* partials;
  float* proj_ws;
  float* sino;
  float *t, *rb, *pb, *xb, *apb, *gb;
  float *P, *AP, *R, *x;  // iterates: the tape's, or the workspace's with recompute
  double* scal;
};

Bufs bufs(const ct_cg_block_desc* d, const Plan& P, void* tape, void* ws, float* x_out) {
  Bufs B{};
  char* w = static_cast<char*>(ws);
  B.tickets = reinterpret_cast<unsigned int*>(w);
  B.partials = reinterpret_cast<double*>(w + ct::round_up((size_t)d->nsys * sizeof(unsigned int), 256));
  char* q = w + P.ws_red;
  B.proj_ws = reinterpret_cast<float*>(q);
  q += P.ws_proj;
  B.sino = reinterpret_cast<float*>(q);
  q += P.ws_sino;
  float* tmp[6];
  for (int i = 0; i < 6; ++i) tmp[i] = reinterpret_cast<float*>(q + i * P.vec);
  B.t = tmp[0];
  B.rb = tmp[1];
  B.pb = tmp[2];
  B.xb = tmp[3];
  B.apb = tmp[4];
  B.gb = tmp[5];
  q += P.ws_tmp;
  char* vec = d->recompute ? q : static_cast<char*>(tape);
  const int K = d->maxiter;
  B.P = reinterpret_cast<float*>(vec);
  B.AP = reinterpret_cast<float*>(vec + (size_t)K * P.vec);
  B.R = reinterpret_cast<float*>(vec + (size_t)2 * K * P.vec);
  B.x = d->recompute ? reinterpret_cast<float*>(vec + (size_t)(3 * K + 1) * P.vec) : x_out;
  B.scal = reinterpret_cast<double*>(static_cast<char*>(tape) + P.tape_vectors);
  return B;
}

float* at(float* base, const Plan& P, int k) {
  return reinterpret_cast<float*>(reinterpret_cast<char*>(base) + (size_t)k * P.vec);
}

// t = H^T H v for the batch (forward projection, then adjoint with its view
// splits summed in order).
ct_status gram(const ct_cg_block_desc* d, const Plan& P, const Bufs& B, const float* v, float* t, cudaStream_t s) {
  CT_TRY(ct::proj2d_fwd_launch(&d->geom, P.p2, v, B.sino, d->nsys, B.proj_ws, s, nullptr));
  CT_TRY(ct::proj2d_adj_launch(&d->geom, P.p2, B.sino, t, B.proj_ws, d->nsys, s, nullptr));
  if (P.p2.nsplit > 1) CT_TRY(ct::proj2d_sum_splits(B.proj_ws, t, (size_t)d->nsys * P.s.n, P.p2.nsplit, s));
  return CT_OK;
}

dim3 grid_of(const Plan& P) { return dim3((unsigned)P.s.nb, (unsigned)P.s.nsys, 1); }

ct_status forward(const ct_cg_block_desc* d, const Plan& P, const Bufs& B, const float* b, float lam,
                  const float* x0, cudaStream_t s) {
  const size_t nbytes = (size_t)d->nsys * P.s.n * sizeof(float);
  const float gs = d->gram_scale;
  const dim3 g = grid_of(P);
  const float* ax0 = nullptr;
  if (x0) {
    CT_TRY(ct::cuda_check(cudaMemcpyAsync(B.x, x0, nbytes, cudaMemcpyDeviceToDevice, s), "x0 copy"));
    CT_TRY(gram(d, P, B, x0, B.t, s));
    k_cgb_axpy<<<g, NT, 0, s>>>(B.t, x0, B.t, gs, lam, P.s);  // A x0, in place of t
    CT_TRY(ct::launch_check("k_cgb_axpy"));
    ax0 = B.t;
  } else {
    CT_TRY(ct::cuda_check(cudaMemsetAsync(B.x, 0, nbytes, s), "x0 zero"));
  }
  const int K = d->maxiter;
  k_cgb_init<<<g, NT, 0, s>>>(b, ax0, at(B.R, P, 0), K > 0 ? at(B.P, P, 0) : B.pb, P.s, B.scal, B.partials,
                              B.tickets);
  CT_TRY(ct::launch_check("k_cgb_init"));
  for (int k = 0; k < K; ++k) {
    float* pk = at(B.P, P, k);
    float* apk = at(B.AP, P, k);
    CT_TRY(gram(d, P, B, pk, B.t, s));
    k_cgb_ap<<<g, NT, 0, s>>>(B.t, pk, apk, gs, lam, k, P.s, B.scal, B.partials, B.tickets);
    CT_TRY(ct::launch_check("k_cgb_ap"));
    k_cgb_upd<<<g, NT, 0, s>>>(B.x, at(B.R, P, k), at(B.R, P, k + 1), pk, apk, k, P.s, B.scal, B.partials,
                               B.tickets);
    CT_TRY(ct::launch_check("k_cgb_upd"));
    if (k + 1 < K) {
      k_cgb_dir<<<g, NT, 0, s>>>(at(B.R, P, k + 1), pk, at(B.P, P, k + 1), k, P.s, B.scal);
      CT_TRY(ct::launch_check("k_cgb_dir"));
    }
  }
  return CT_OK;
}

ct_status buffers_check(const Plan& P, void* tape, size_t tape_bytes, void* ws, size_t ws_bytes, const char* who) {
  if (!tape || tape_bytes < P.tape_total || !ct::aligned(tape, 256))
    return ct::fail(CT_ERR_WORKSPACE, "%s: tape needs %zu bytes (256-B aligned), got %zu", who, P.tape_total,
                    tape_bytes);
  if (!ws || ws_bytes < P.ws_total || !ct::aligned(ws, 256))
    return ct::fail(CT_ERR_WORKSPACE, "%s: workspace needs %zu bytes (256-B aligned), got %zu", who, P.ws_total,
                    ws_bytes);
  return CT_OK;
}

}  // namespace

extern "C" {

ct_status ct_cg_block_workspace(const ct_cg_block_desc* d, size_t* tape_bytes, size_t* ws_bytes) {
  CT_TRY(check(d, "ct_cg_block_workspace"));
  const Plan P = plan_of(d);
  if (tape_bytes) *tape_bytes = P.tape_total;
  if (ws_bytes) *ws_bytes = P.ws_total;
  return CT_OK;
}

ct_status ct_cg_block_fwd(const ct_cg_block_desc* d, const float* b, float lam, const float* x0, float* x,
                          void* tape, size_t tape_bytes, void* workspace, size_t workspace_bytes,
                          ct_stream_t stream) {
  const char* who = "ct_cg_block_fwd";
  CT_TRY(check(d, who));
  if (!b || !x) return ct::fail(CT_ERR_INVALID_ARG, "%s: null array", who);
  const Plan P = plan_of(d);
  CT_TRY(buffers_check(P, tape, tape_bytes, workspace, workspace_bytes, who));
  CT_TRY(ct::proj2d_prepare(P.p2));
  cudaStream_t s = ct::as_stream(stream);
  CT_TRY(ct::cuda_check(cudaMemsetAsync(workspace, 0, P.ws_red, s), "reduction init"));
  const Bufs B = bufs(d, P, tape, workspace, x);
  CT_TRY(forward(d, P, B, b, lam, x0, s));
  if (d->recompute)
    CT_TRY(ct::cuda_check(
        cudaMemcpyAsync(x, B.x, (size_t)d->nsys * P.s.n * sizeof(float), cudaMemcpyDeviceToDevice, s), "x copy"));
  return CT_OK;
}

ct_status ct_cg_block_bwd(const ct_cg_block_desc* d, const float* gx, const float* b, float lam, const float* x0,
                          void* tape, size_t tape_bytes, float* gb, float* gx0, double* glam, void* workspace,
                          size_t workspace_bytes, ct_stream_t stream) {
  const char* who = "ct_cg_block_bwd";
  CT_TRY(check(d, who));
  if (!gx || !gb || !glam) return ct::fail(CT_ERR_INVALID_ARG, "%s: null array", who);
  if (d->recompute && !b) return ct::fail(CT_ERR_INVALID_ARG, "%s: recompute needs b", who);
  if (gx0 && !x0) return ct::fail(CT_ERR_INVALID_ARG, "%s: gx0 without x0", who);
  const Plan P = plan_of(d);
  CT_TRY(buffers_check(P, tape, tape_bytes, workspace, workspace_bytes, who));
  CT_TRY(ct::proj2d_prepare(P.p2));
  cudaStream_t s = ct::as_stream(stream);
  CT_TRY(ct::cuda_check(cudaMemsetAsync(workspace, 0, P.ws_red, s), "reduction init"));
  const Bufs B = bufs(d, P, tape, workspace, nullptr);
  if (d->recompute) CT_TRY(forward(d, P, B, b, lam, x0, s));  // the iterates from the block's inputs
  const size_t nbytes = (size_t)d->nsys * P.s.n * sizeof(float);
  const float gs = d->gram_scale;
  const dim3 g = grid_of(P);
  CT_TRY(ct::cuda_check(cudaMemcpyAsync(B.xb, gx, nbytes, cudaMemcpyDeviceToDevice, s), "xb init"));
  CT_TRY(ct::cuda_check(cudaMemsetAsync(B.rb, 0, nbytes, s), "rb init"));
  CT_TRY(ct::cuda_check(cudaMemsetAsync(B.pb, 0, nbytes, s), "pb init"));
  k_cgb_reset<<<1, 256, 0, s>>>(B.scal, P.s);
  CT_TRY(ct::launch_check("k_cgb_reset"));
  const int K = d->maxiter;
  bool pending = false;  // B.t holds H^T H apb of the previous backward step
  for (int k = K - 1; k >= 0; --k) {
    const float* pk = at(B.P, P, k);
    const float* apk = at(B.AP, P, k);
    k_cgb_b1<<<g, NT, 0, s>>>(B.pb, pending ? B.t : nullptr, B.apb, gs, lam, pk, k, P.s, B.scal, B.partials,
                              B.tickets);
    CT_TRY(ct::launch_check("k_cgb_b1"));
    k_cgb_b2<<<g, NT, 0, s>>>(B.rb, B.pb, at(B.R, P, k + 1), B.xb, pk, apk, k, P.s, B.scal, B.partials, B.tickets);
    CT_TRY(ct::launch_check("k_cgb_b2"));
    k_cgb_b3<<<g, NT, 0, s>>>(B.rb, B.xb, B.pb, B.apb, pk, apk, k, P.s, B.scal, B.partials, B.tickets);
    CT_TRY(ct::launch_check("k_cgb_b3"));
    CT_TRY(gram(d, P, B, B.apb, B.t, s));
    pending = true;
  }
  if (pending) {
    k_cgb_b1<<<g, NT, 0, s>>>(B.pb, B.t, B.apb, gs, lam, nullptr, -1, P.s, B.scal, B.partials, B.tickets);
    CT_TRY(ct::launch_check("k_cgb_b1"));
  }
  k_cgb_rb0<<<g, NT, 0, s>>>(B.rb, B.pb, at(B.R, P, 0), gb, P.s, B.scal);
  CT_TRY(ct::launch_check("k_cgb_rb0"));
  if (x0) {
    CT_TRY(gram(d, P, B, gb, B.t, s));
    k_cgb_x0<<<g, NT, 0, s>>>(B.xb, B.t, gb, x0, gx0, gs, lam, P.s, B.scal, B.partials, B.tickets);
    CT_TRY(ct::launch_check("k_cgb_x0"));
  }
  k_cgb_lamsum<<<1, 1, 0, s>>>(B.scal, P.s, glam);
  return ct::launch_check("k_cgb_lamsum");
}

}  // extern "C"
