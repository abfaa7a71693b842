// Deterministic float64 reductions and the CG vector steps of
// scico.solver.cg (scico/solver.py:378-400), with the stopping test kept on
// the device so that a fixed launch sequence reproduces the early exit.
#include "cgpass.cuh"
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

// Quad path: with n % 4 == 0 and every array 16-B aligned a thread moves
// four consecutive elements per 128-bit access, two quads per loop step so
// that more loads are in flight; per element the arithmetic is the scalar
// code's.
__device__ __forceinline__ float4 ld4(const float* __restrict__ p, size_t e) {
  return *reinterpret_cast<const float4*>(p + e);
}
__device__ __forceinline__ void st4(float* __restrict__ p, size_t e, float4 v) {
  *reinterpret_cast<float4*>(p + e) = v;
}
__device__ __forceinline__ float at4(const float4& v, int j) {
  return j == 0 ? v.x : (j == 1 ? v.y : (j == 2 ? v.z : v.w));
}

__global__ void __launch_bounds__(NT)
    k_dot(const float* __restrict__ a, const float* __restrict__ b, size_t n,
          double* __restrict__ out, double* __restrict__ partials, unsigned int* __restrict__ ticket,
          int vec) {
  double acc = 0.0;
  if (vec) {
    const size_t stride = 4 * (size_t)gridDim.x * NT;
    for (size_t e0 = 4 * ((size_t)blockIdx.x * NT + threadIdx.x); e0 < n; e0 += 2 * stride) {
      const bool two = e0 + stride < n;
      const float4 a0 = ld4(a, e0), b0 = ld4(b, e0);
      float4 a1 = a0, b1 = b0;
      if (two) {
        a1 = ld4(a, e0 + stride);
        b1 = ld4(b, e0 + stride);
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) acc += (double)at4(a0, j) * (double)at4(b0, j);
      if (two) {
#pragma unroll
        for (int j = 0; j < 4; ++j) acc += (double)at4(a1, j) * (double)at4(b1, j);
      }
    }
  } else {
    for (size_t e = (size_t)blockIdx.x * NT + threadIdx.x; e < n; e += (size_t)gridDim.x * NT)
      acc += (double)a[e] * (double)b[e];
  }
  double t0, t1;
  if (grid_sum2_last<NT>(acc, 0.0, partials, ticket, t0, t1)) *out = t0;
}

__global__ void __launch_bounds__(NT)
    k_cg_init(const float* __restrict__ b, const float* __restrict__ Ax, float* __restrict__ r,
              float* __restrict__ p, size_t n, double tol, double atol, int maxiter,
              double* __restrict__ s, double* __restrict__ partials, unsigned int* __restrict__ ticket,
              int vec) {
  double rr = 0.0, bb = 0.0;
  if (vec) {
    for (size_t e0 = 4 * ((size_t)blockIdx.x * NT + threadIdx.x); e0 < n; e0 += 4 * (size_t)gridDim.x * NT) {
      const float4 b4 = ld4(b, e0), a4 = ld4(Ax, e0);
      float re[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const float be = at4(b4, j);
        re[j] = ct::fsub(be, at4(a4, j));
        rr += (double)re[j] * (double)re[j];
        bb += (double)be * (double)be;
      }
      const float4 r4 = make_float4(re[0], re[1], re[2], re[3]);
      st4(r, e0, r4);
      st4(p, e0, r4);
    }
  } else {
    for (size_t e = (size_t)blockIdx.x * NT + threadIdx.x; e < n; e += (size_t)gridDim.x * NT) {
      const float be = b[e];
      const float re = ct::fsub(be, Ax[e]);
      r[e] = re;
      p[e] = re;
      rr += (double)re * (double)re;
      bb += (double)be * (double)be;
    }
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
                cudaGraphConditionalHandle cond, int use_cond, int vec) {
  ct::grid_dep_wait();  // before any global access (dependent launch)
  ct::grid_dep_trigger();
  if (s[CT_CG_DONE] != 0.0) {  // uniform over the grid
    if (use_cond && blockIdx.x == 0 && threadIdx.x == 0) cudaGraphSetConditional(cond, 0u);
    return;
  }
  // one float64 division per block (float64 runs at a small fraction of
  // the float32 rate on this GPU), shared through shared memory
  __shared__ double alpha_s;
  if (threadIdx.x == 0) alpha_s = s[CT_CG_NUM] / s[CT_CG_PAP];
  __syncthreads();
  const double alpha = alpha_s;
  const float af = (float)alpha;
  const double rr = ct::cg_update_pass(x, r, p, Ap, n, af, vec);
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
                               double* __restrict__ s, unsigned int* __restrict__ ticket, int vec) {
  ct::grid_dep_wait();  // before any global access (dependent launch)
  ct::grid_dep_trigger();
  if (s[CT_CG_RAN] == 0.0) return;  // uniform over the grid
  const float bf = (float)s[CT_CG_BETA];
  ct::cg_direction_pass(p, r, n, bf, vec);
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
  RedWs w{};
  ct_status st = red_ws(workspace, workspace_bytes, "ct_dot", w);
  if (st != CT_OK) return st;
  const int vec = ct::quad_ok((size_t)n, a, b);
  k_dot<<<ct::kReduceBlocks, NT, 0, ct::as_stream(stream)>>>(a, b, (size_t)n, out_dev, w.partials,
                                                            w.ticket, vec);
  return ct::launch_check("k_dot");
}

ct_status ct_cg_init(const float* b, const float* Ax, float* r, float* p, int64_t n, double tol,
                     double atol, int32_t maxiter, double* scalars, void* workspace,
                     size_t workspace_bytes, ct_stream_t stream) {
  if (!b || !Ax || !r || !p || !scalars)
    return ct::fail(CT_ERR_INVALID_ARG, "ct_cg_init: null pointer");
  if (n < 0) return ct::fail(CT_ERR_INVALID_ARG, "ct_cg_init: n=%lld", (long long)n);
  RedWs w{};
  ct_status st = red_ws(workspace, workspace_bytes, "ct_cg_init", w);
  if (st != CT_OK) return st;
  const int vec = ct::quad_ok((size_t)n, b, Ax, r, p);
  k_cg_init<<<ct::kReduceBlocks, NT, 0, ct::as_stream(stream)>>>(
      b, Ax, r, p, (size_t)n, tol, atol, maxiter, scalars, w.partials, w.ticket, vec);
  return ct::launch_check("k_cg_init");
}

ct_status ct_cg_update(float* x, float* r, const float* p, const float* Ap, int64_t n,
                       double* scalars, void* workspace, size_t workspace_bytes,
                       ct_stream_t stream) {
  if (!x || !r || !p || !Ap || !scalars)
    return ct::fail(CT_ERR_INVALID_ARG, "ct_cg_update: null pointer");
  RedWs w{};
  ct_status st = red_ws(workspace, workspace_bytes, "ct_cg_update", w);
  if (st != CT_OK) return st;
  const int vec = ct::quad_ok((size_t)n, x, r, p, Ap);
  k_cg_update<<<ct::kReduceBlocks, NT, 0, ct::as_stream(stream)>>>(x, r, p, Ap, (size_t)n, scalars,
                                                                  w.partials, w.ticket, 0, 0, vec);
  return ct::launch_check("k_cg_update");
}

ct_status ct_cg_direction(float* p, const float* r, int64_t n, double* scalars, void* workspace,
                          size_t workspace_bytes, ct_stream_t stream) {
  if (!p || !r || !scalars) return ct::fail(CT_ERR_INVALID_ARG, "ct_cg_direction: null pointer");
  RedWs w{};
  ct_status st = red_ws(workspace, workspace_bytes, "ct_cg_direction", w);
  if (st != CT_OK) return st;
  return ct::cg_direction_launch(p, r, (size_t)n, scalars, workspace, ct::as_stream(stream));
}

}  // extern "C"


namespace ct {

ct_status cg_update_launch(float* x, float* r, const float* p, const float* Ap, size_t n,
                           double* scalars, void* red_ws, cudaStream_t s, cudaGraphConditionalHandle cond,
                           int use_cond, bool dependent) {
  unsigned int* ticket = static_cast<unsigned int*>(red_ws);
  double* partials = reinterpret_cast<double*>(static_cast<char*>(red_ws) + 256);
  return cuda_check(launch_k(k_cg_update, dim3(kReduceBlocks), dim3(NT), 0, s, dependent, x, r, p, Ap, n, scalars,
                             partials, ticket, cond, use_cond, quad_ok(n, x, r, p, Ap)),
                    "k_cg_update");
}

ct_status cg_direction_launch(float* p, const float* r, size_t n, double* scalars, void* red_ws,
                              cudaStream_t s, bool dependent) {
  unsigned int* ticket2 = static_cast<unsigned int*>(red_ws) + 1;
  return cuda_check(launch_k(k_cg_direction, dim3(kReduceBlocks), dim3(NT), 0, s, dependent, p, r, n, scalars,
                             ticket2, quad_ok(n, p, r)),
                    "k_cg_direction");
}

}  // namespace ct
