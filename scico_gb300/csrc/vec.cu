// Deterministic float64 reductions and the CG vector steps of
// scico.solver.cg (scico/solver.py:378-400), with the stopping test kept on
// the device so that a fixed launch sequence reproduces the early exit.
#include "common.cuh"
#include "kernels.cuh"

namespace {

struct RedWs {
  unsigned int* ticket;
  double* partials;
};

ct_status red_ws(void* ws, size_t bytes, const char* who, RedWs& r) {
  if (!ws || bytes < ct::kReduceWorkspace || !ct::aligned(ws, 256))
    return ct::fail(CT_ERR_WORKSPACE, "%s: reduction workspace needs %zu bytes (256-B aligned)",
                    who, ct::kReduceWorkspace);
  r.ticket = static_cast<unsigned int*>(ws);
  r.partials = reinterpret_cast<double*>(static_cast<char*>(ws) + 256);
  return CT_OK;
}

// Two simultaneous float64 grid sums; the last block gets both totals.
template <int NT>
__device__ __forceinline__ bool grid_sum2_last(double a, double b, double* partials,
                                               unsigned int* ticket, double& ta, double& tb) {
  double v[2] = {a, b}, out[2];
  const bool last = ct::grid_reduce_last<NT, 2>(v, partials, ticket, out);
  if (last) {
    ta = out[0];
    tb = out[1];
  }
  return last;
}

constexpr int NT = ct::kReduceThreads;

__global__ void __launch_bounds__(NT)
    k_dot(const float* __restrict__ a, const float* __restrict__ b, size_t n,
          double* __restrict__ out, double* __restrict__ partials, unsigned int* __restrict__ ticket) {
  double acc = 0.0;
  for (size_t e = (size_t)blockIdx.x * NT + threadIdx.x; e < n; e += (size_t)gridDim.x * NT)
    acc += (double)a[e] * (double)b[e];
  double t0, t1;
  if (grid_sum2_last<NT>(acc, 0.0, partials, ticket, t0, t1)) *out = t0;
}

__global__ void __launch_bounds__(NT)
    k_cg_init(const float* __restrict__ b, const float* __restrict__ Ax, float* __restrict__ r,
              float* __restrict__ p, size_t n, double tol, double atol, int maxiter,
              double* __restrict__ s, double* __restrict__ partials, unsigned int* __restrict__ ticket) {
  double rr = 0.0, bb = 0.0;
  for (size_t e = (size_t)blockIdx.x * NT + threadIdx.x; e < n; e += (size_t)gridDim.x * NT) {
    const float be = b[e];
    const float re = ct::fsub(be, Ax[e]);
    r[e] = re;
    p[e] = re;
    rr += (double)re * (double)re;
    bb += (double)be * (double)be;
  }
  double trr, tbb;
  if (grid_sum2_last<NT>(rr, bb, partials, ticket, trr, tbb)) {
    const double bn = sqrt(tbb);
    const double thr = fmax(tol * bn, atol);
    s[CT_CG_NUM] = trr;
    s[CT_CG_PAP] = 0.0;
    s[CT_CG_ALPHA] = 0.0;
    s[CT_CG_BETA] = 0.0;
    s[CT_CG_BNORM] = bn;
    s[CT_CG_TOL2] = thr * thr;
    s[CT_CG_ITERS] = 0.0;
    s[CT_CG_MAXITER] = (double)maxiter;
    s[CT_CG_RAN] = 0.0;
    s[CT_CG_DONE] = (maxiter <= 0 || !(trr > thr * thr)) ? 1.0 : 0.0;
  }
}

// alpha = num/pAp; x += alpha p; r -= alpha Ap; num' = <r,r>.
// In a CUDA graph whose CG loop is a conditional WHILE node (use_cond != 0)
// the last block also sets the loop condition to "not DONE".
__global__ void __launch_bounds__(NT)
    k_cg_update(float* __restrict__ x, float* __restrict__ r, const float* __restrict__ p,
                const float* __restrict__ Ap, size_t n, double* __restrict__ s,
                double* __restrict__ partials, unsigned int* __restrict__ ticket,
                cudaGraphConditionalHandle cond, int use_cond) {
  if (s[CT_CG_DONE] != 0.0) {  // uniform over the grid
    if (use_cond && blockIdx.x == 0 && threadIdx.x == 0) cudaGraphSetConditional(cond, 0u);
    return;
  }
  const double alpha = s[CT_CG_NUM] / s[CT_CG_PAP];
  const float af = (float)alpha;
  double rr = 0.0;
  for (size_t e = (size_t)blockIdx.x * NT + threadIdx.x; e < n; e += (size_t)gridDim.x * NT) {
    const float pe = p[e];
    x[e] = ct::fadd(x[e], ct::fmul(af, pe));
    const float re = ct::fsub(r[e], ct::fmul(af, Ap[e]));
    r[e] = re;
    rr += (double)re * (double)re;
  }
  double trr, t1;
  if (grid_sum2_last<NT>(rr, 0.0, partials, ticket, trr, t1)) {
    const double num_old = s[CT_CG_NUM];
    s[CT_CG_ALPHA] = alpha;
    s[CT_CG_NUM] = trr;
    s[CT_CG_BETA] = trr / num_old;
    const double it = s[CT_CG_ITERS] + 1.0;
    s[CT_CG_ITERS] = it;
    // The direction update still runs for this iteration (reference order);
    // DONE takes effect from the next update on.
    s[CT_CG_RAN] = 1.0;
    const bool done = !(trr > s[CT_CG_TOL2]) || it >= s[CT_CG_MAXITER];
    if (done) s[CT_CG_DONE] = 1.0;
    if (use_cond) cudaGraphSetConditional(cond, done ? 0u : 1u);
  }
}

// p = r + beta p, only when the preceding update ran.  Every block reads
// the marker when it starts; the last block to finish (ticket in the second
// word of the reduction workspace) clears it, after all blocks have read it.
__global__ void k_cg_direction(float* __restrict__ p, const float* __restrict__ r, size_t n,
                               double* __restrict__ s, unsigned int* __restrict__ ticket) {
  if (s[CT_CG_RAN] == 0.0) return;  // uniform over the grid
  const float bf = (float)s[CT_CG_BETA];
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n;
       e += (size_t)gridDim.x * blockDim.x)
    p[e] = ct::fadd(r[e], ct::fmul(bf, p[e]));
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(ticket, 1u) == gridDim.x - 1) {
      s[CT_CG_RAN] = 0.0;
      *ticket = 0u;
    }
  }
}

}  // namespace

extern "C" {

ct_status ct_dot(const float* a, const float* b, int64_t n, double* out_dev, void* workspace,
                 size_t workspace_bytes, ct_stream_t stream) {
  if (!a || !b || !out_dev) return ct::fail(CT_ERR_INVALID_ARG, "ct_dot: null pointer");
  if (n < 0) return ct::fail(CT_ERR_INVALID_ARG, "ct_dot: n=%lld", (long long)n);
  RedWs w;
  ct_status st = red_ws(workspace, workspace_bytes, "ct_dot", w);
  if (st != CT_OK) return st;
  k_dot<<<ct::kReduceBlocks, NT, 0, ct::as_stream(stream)>>>(a, b, (size_t)n, out_dev, w.partials,
                                                            w.ticket);
  return ct::launch_check("k_dot");
}

ct_status ct_cg_init(const float* b, const float* Ax, float* r, float* p, int64_t n, double tol,
                     double atol, int32_t maxiter, double* scalars, void* workspace,
                     size_t workspace_bytes, ct_stream_t stream) {
  if (!b || !Ax || !r || !p || !scalars)
    return ct::fail(CT_ERR_INVALID_ARG, "ct_cg_init: null pointer");
  if (n < 0) return ct::fail(CT_ERR_INVALID_ARG, "ct_cg_init: n=%lld", (long long)n);
  RedWs w;
  ct_status st = red_ws(workspace, workspace_bytes, "ct_cg_init", w);
  if (st != CT_OK) return st;
  k_cg_init<<<ct::kReduceBlocks, NT, 0, ct::as_stream(stream)>>>(
      b, Ax, r, p, (size_t)n, tol, atol, maxiter, scalars, w.partials, w.ticket);
  return ct::launch_check("k_cg_init");
}

ct_status ct_cg_update(float* x, float* r, const float* p, const float* Ap, int64_t n,
                       double* scalars, void* workspace, size_t workspace_bytes,
                       ct_stream_t stream) {
  if (!x || !r || !p || !Ap || !scalars)
    return ct::fail(CT_ERR_INVALID_ARG, "ct_cg_update: null pointer");
  RedWs w;
  ct_status st = red_ws(workspace, workspace_bytes, "ct_cg_update", w);
  if (st != CT_OK) return st;
  k_cg_update<<<ct::kReduceBlocks, NT, 0, ct::as_stream(stream)>>>(x, r, p, Ap, (size_t)n, scalars,
                                                                  w.partials, w.ticket, 0, 0);
  return ct::launch_check("k_cg_update");
}

ct_status ct_cg_direction(float* p, const float* r, int64_t n, double* scalars, void* workspace,
                          size_t workspace_bytes, ct_stream_t stream) {
  if (!p || !r || !scalars) return ct::fail(CT_ERR_INVALID_ARG, "ct_cg_direction: null pointer");
  RedWs w;
  ct_status st = red_ws(workspace, workspace_bytes, "ct_cg_direction", w);
  if (st != CT_OK) return st;
  return ct::cg_direction_launch(p, r, (size_t)n, scalars, workspace, ct::as_stream(stream));
}

}  // extern "C"


namespace ct {

ct_status cg_update_launch(float* x, float* r, const float* p, const float* Ap, size_t n,
                           double* scalars, void* red_ws, cudaStream_t s, cudaGraphConditionalHandle cond,
                           int use_cond) {
  unsigned int* ticket = static_cast<unsigned int*>(red_ws);
  double* partials = reinterpret_cast<double*>(static_cast<char*>(red_ws) + 256);
  k_cg_update<<<kReduceBlocks, NT, 0, s>>>(x, r, p, Ap, n, scalars, partials, ticket, cond, use_cond);
  return launch_check("k_cg_update");
}

ct_status cg_direction_launch(float* p, const float* r, size_t n, double* scalars, void* red_ws,
                              cudaStream_t s) {
  unsigned int* ticket2 = static_cast<unsigned int*>(red_ws) + 1;
  k_cg_direction<<<kReduceBlocks, NT, 0, s>>>(p, r, n, scalars, ticket2);
  return launch_check("k_cg_direction");
}

}  // namespace ct
