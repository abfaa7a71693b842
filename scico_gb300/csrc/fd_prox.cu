// Finite differences (scico FiniteDifference), their adjoint, and the
// L2,1 / L1 proximal operators and norms (scico/functional/_norm.py).
#include <math.h>

#include <algorithm>

#include "common.cuh"

namespace {

struct FdBlock {
  int axis;    // differenced axis (0..2 of the 3-D padded shape)
  int M;       // output length along that axis
  size_t off;  // element offset of this block in the concatenated output
  size_t count;
};

struct FdParams {
  int n[3];  // padded 3-D input shape
  int nblocks;
  FdBlock blk[3];
  int prepend, append, circular;
  size_t in_count;   // elements of one input
  size_t out_count;  // elements of one output (all blocks)
};

ct_status make_fd(const ct_fd_desc* d, FdParams& p, const char* who) {
  if (!d) return ct::fail(CT_ERR_INVALID_ARG, "%s: null descriptor", who);
  if (d->ndim < 1 || d->ndim > 3) return ct::fail(CT_ERR_UNSUPPORTED, "%s: ndim=%d", who, d->ndim);
  if (d->naxes < 1 || d->naxes > d->ndim)
    return ct::fail(CT_ERR_INVALID_ARG, "%s: naxes=%d", who, d->naxes);
  if (d->prepend < -1 || d->prepend > 1 || d->append < -1 || d->append > 1)
    return ct::fail(CT_ERR_INVALID_ARG, "%s: prepend/append must be -1, 0 or 1", who);
  if (d->circular && (d->prepend != -1 || d->append != -1))
    return ct::fail(CT_ERR_INVALID_ARG, "%s: circular needs prepend = append = None", who);
  const int pad = 3 - d->ndim;
  for (int k = 0; k < 3; ++k) p.n[k] = 1;
  for (int k = 0; k < d->ndim; ++k) {
    if (d->shape[k] <= 0) return ct::fail(CT_ERR_SHAPE, "%s: shape[%d]=%d", who, k, d->shape[k]);
    p.n[pad + k] = d->shape[k];
  }
  p.prepend = d->prepend;
  p.append = d->append;
  p.circular = d->circular ? 1 : 0;
  p.nblocks = d->naxes;
  p.in_count = (size_t)p.n[0] * p.n[1] * p.n[2];
  size_t off = 0;
  for (int k = 0; k < d->naxes; ++k) {
    const int ax = d->axes[k];
    if (ax < 0 || ax >= d->ndim) return ct::fail(CT_ERR_INVALID_ARG, "%s: axis %d", who, ax);
    for (int q = 0; q < k; ++q)
      if (d->axes[q] == ax) return ct::fail(CT_ERR_INVALID_ARG, "%s: repeated axis %d", who, ax);
    const int a3 = pad + ax;
    const int n = p.n[a3];
    int M = p.circular ? n : n + (p.prepend >= 0) + (p.append >= 0) - 1;
    if (M < 0) M = 0;
    p.blk[k].axis = a3;
    p.blk[k].M = M;
    p.blk[k].off = off;
    p.blk[k].count = p.in_count / n * M;
    off += p.blk[k].count;
  }
  p.out_count = off;
  return CT_OK;
}

// Value of the extended line e (prepend/append applied) at position t.
__device__ __forceinline__ float fd_ext(const float* __restrict__ x, size_t stride, int n, int P,
                                        int prepend, int append, int t) {
  if (t < P) return prepend == 0 ? __ldg(x) : 0.0f;
  const int s = t - P;
  if (s < n) return __ldg(x + (size_t)s * stride);
  return append == 0 ? __ldg(x + (size_t)(n - 1) * stride) : 0.0f;
}

__global__ void k_fd_fwd(const float* __restrict__ x, float* __restrict__ out, FdParams p,
                         int batch) {
  const size_t total = p.out_count * batch;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (size_t)gridDim.x * blockDim.x) {
    const size_t bi = e / p.out_count;
    size_t r = e - bi * p.out_count;
    int k = 0;
    while (k + 1 < p.nblocks && r >= p.blk[k + 1].off) ++k;
    r -= p.blk[k].off;
    const FdBlock& B = p.blk[k];
    int dims[3] = {p.n[0], p.n[1], p.n[2]};
    dims[B.axis] = B.M;
    const int c2 = (int)(r % dims[2]);
    const size_t r1 = r / dims[2];
    const int c1 = (int)(r1 % dims[1]);
    const int c0 = (int)(r1 / dims[1]);
    int c[3] = {c0, c1, c2};
    const int m = c[B.axis];
    const int n = p.n[B.axis];
    size_t stride = 1;
    for (int q = 2; q > B.axis; --q) stride *= p.n[q];
    c[B.axis] = 0;
    const float* line = x + bi * p.in_count + ((size_t)c[0] * p.n[1] + c[1]) * p.n[2] + c[2];
    float v;
    if (p.circular) {
      const int m1 = (m + 1 == n) ? 0 : m + 1;
      v = ct::fsub(__ldg(line + (size_t)m1 * stride), __ldg(line + (size_t)m * stride));
    } else {
      const int P = p.prepend >= 0 ? 1 : 0;
      v = ct::fsub(fd_ext(line, stride, n, P, p.prepend, p.append, m + 1),
                   fd_ext(line, stride, n, P, p.prepend, p.append, m));
    }
    out[e] = v;
  }
}

// Adjoint, as jax.linear_transpose builds it from the forward's jnp.diff:
// extended-line position q gets the cotangent ce[q] = d[q-1] - d[q] (a term
// outside 0..M-1 is 0), and x[t] = sum over blocks (axis order) of the sum,
// in position order, of ce[q] over the run [qa, qb] of positions holding
// x[t] -- one position inside the line, two at an end copied by prepend=0 /
// append=0 (the float32 sum (d[0] - d[1]) - d[0] is not -d[1] in general).
__global__ void k_fd_adj(const float* __restrict__ d, float* __restrict__ x, FdParams p,
                         int batch) {
  const size_t total = p.in_count * batch;
  const int P = p.prepend >= 0 ? 1 : 0;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (size_t)gridDim.x * blockDim.x) {
    const size_t bi = e / p.in_count;
    const size_t r = e - bi * p.in_count;
    const int c2 = (int)(r % p.n[2]);
    const size_t r1 = r / p.n[2];
    const int c1 = (int)(r1 % p.n[1]);
    const int c0 = (int)(r1 / p.n[1]);
    float acc = 0.0f;
    for (int k = 0; k < p.nblocks; ++k) {
      const FdBlock& B = p.blk[k];
      int c[3] = {c0, c1, c2};
      const int t = c[B.axis];
      const int n = p.n[B.axis];
      int dims[3] = {p.n[0], p.n[1], p.n[2]};
      dims[B.axis] = B.M;
      size_t stride = 1;
      for (int q = 2; q > B.axis; --q) stride *= dims[q];
      c[B.axis] = 0;
      const float* line =
          d + bi * p.out_count + B.off + ((size_t)c[0] * dims[1] + c[1]) * dims[2] + c[2];
      float v;
      if (p.circular) {
        const int tm = (t == 0) ? n - 1 : t - 1;
        v = ct::fsub(__ldg(line + (size_t)tm * stride), __ldg(line + (size_t)t * stride));
      } else {
        const int qa = (p.prepend == 0 && t == 0) ? 0 : t + P;
        const int qb = (p.append == 0 && t == n - 1) ? n + P : t + P;
        auto ce = [&](int q) {
          const float lo = (q - 1 >= 0 && q - 1 < B.M) ? __ldg(line + (size_t)(q - 1) * stride) : 0.0f;
          const float hi = (q >= 0 && q < B.M) ? __ldg(line + (size_t)q * stride) : 0.0f;
          return ct::fsub(lo, hi);
        };
        v = ce(qa);
        for (int q = qa + 1; q <= qb; ++q) v = ct::fadd(v, ce(q));
      }
      acc = (k == 0) ? v : ct::fadd(acc, v);
    }
    x[e] = acc;
  }
}

// Single-level shift-invariant Haar transform over the descriptor's axes
// (HaarTransform / SingleAxisHaarTransform, scico/functional/_tvnorm.py:
// 458-538), output (naxes, 2, *shape) per batch item: for axis k,
// w[k][0] = r (x + x[next]) and w[k][1] = r (x[next] - x), x[next] the
// circularly next sample along the axis, r = float32(1/sqrt 2); every sum and
// product rounded on its own (the reference's separate float32 operations).
__global__ void k_haar_fwd(const float* __restrict__ x, float* __restrict__ w, FdParams p, float r,
                           int batch) {
  const size_t per = 2 * (size_t)p.nblocks * p.in_count;
  const size_t total = per * batch;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (size_t)gridDim.x * blockDim.x) {
    const size_t bi = e / per;
    size_t rem = e - bi * per;
    const int k = (int)(rem / (2 * p.in_count));
    rem -= (size_t)k * 2 * p.in_count;
    const int comp = (int)(rem / p.in_count);
    const size_t idx = rem - (size_t)comp * p.in_count;
    const int ax = p.blk[k].axis;
    const int c2 = (int)(idx % p.n[2]);
    const size_t r1 = idx / p.n[2];
    const int c[3] = {(int)(r1 / p.n[1]), (int)(r1 % p.n[1]), c2};
    size_t stride = 1;
    for (int q = 2; q > ax; --q) stride *= p.n[q];
    const float* xb = x + bi * p.in_count;
    const float xc = __ldg(xb + idx);
    const size_t in = c[ax] + 1 == p.n[ax] ? idx - (size_t)c[ax] * stride : idx + stride;
    const float xn = __ldg(xb + in);
    w[e] = comp == 0 ? ct::fmul(r, ct::fadd(xc, xn)) : ct::fmul(r, ct::fsub(xn, xc));
  }
}

// Its adjoint: x = sum over axes, in axis order, of
// r (lo + lo[prev]) + r (hi[prev] - hi), [prev] the circularly previous
// sample along the axis.
__global__ void k_haar_adj(const float* __restrict__ w, float* __restrict__ x, FdParams p, float r,
                           int batch) {
  const size_t total = p.in_count * batch;
  const size_t per = 2 * (size_t)p.nblocks * p.in_count;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (size_t)gridDim.x * blockDim.x) {
    const size_t bi = e / p.in_count;
    const size_t idx = e - bi * p.in_count;
    const int c2 = (int)(idx % p.n[2]);
    const size_t r1 = idx / p.n[2];
    const int c[3] = {(int)(r1 / p.n[1]), (int)(r1 % p.n[1]), c2};
    float acc = 0.0f;
    for (int k = 0; k < p.nblocks; ++k) {
      const int ax = p.blk[k].axis;
      size_t stride = 1;
      for (int q = 2; q > ax; --q) stride *= p.n[q];
      const size_t ip = c[ax] == 0 ? idx + (size_t)(p.n[ax] - 1) * stride : idx - stride;
      const float* lo = w + bi * per + (size_t)k * 2 * p.in_count;
      const float* hi = lo + p.in_count;
      const float t = ct::fadd(ct::fmul(r, ct::fadd(__ldg(lo + idx), __ldg(lo + ip))),
                               ct::fmul(r, ct::fsub(__ldg(hi + ip), __ldg(hi + idx))));
      acc = k == 0 ? t : ct::fadd(acc, t);
    }
    x[e] = acc;
  }
}

int grid_for(size_t n, int threads) {
  const size_t want = (n + threads - 1) / threads;
  const size_t cap = (size_t)ct::sm_count() * 16;
  return (int)std::max<size_t>(1, std::min(want, cap));
}

// L2,1 prox over the leading axis (L21Norm._prox, _norm.py:254-263):
// len = sqrt(sum_c v_c^2); dir = v/len (0 where len == 0);
// nl = len - lam; nl = 0.5 (nl + |nl|); out = nl * dir.
__global__ void k_l21_prox(const float* __restrict__ v, float* __restrict__ out, int ncomp,
                           size_t n, float lam) {
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n;
       e += (size_t)gridDim.x * blockDim.x) {
    float ss = 0.0f;
    for (int c = 0; c < ncomp; ++c) {
      const float x = v[(size_t)c * n + e];
      const float sq = ct::fmul(x, x);
      ss = (c == 0) ? sq : ct::fadd(ss, sq);
    }
    const float len = __fsqrt_rn(ss);
    float nl = ct::fsub(len, lam);
    nl = ct::fmul(0.5f, ct::fadd(nl, fabsf(nl)));
    for (int c = 0; c < ncomp; ++c) {
      const float x = v[(size_t)c * n + e];
      const float dir = (len != 0.0f) ? __fdiv_rn(x, len) : 0.0f;
      out[(size_t)c * n + e] = ct::fmul(nl, dir);
    }
  }
}

// L1 prox (L1Norm.prox, _norm.py:110-116): sign(v) * 0.5 (t + |t|), t = |v| - lam.
__global__ void k_l1_prox(const float* __restrict__ v, float* __restrict__ out, size_t n,
                          float lam) {
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n;
       e += (size_t)gridDim.x * blockDim.x) {
    const float x = v[e];
    float t = ct::fsub(fabsf(x), lam);
    t = ct::fmul(0.5f, ct::fadd(t, fabsf(t)));
    const float sg = (x > 0.0f) ? 1.0f : ((x < 0.0f) ? -1.0f : (x == 0.0f ? 0.0f : x));
    out[e] = ct::fmul(sg, t);
  }
}

// sum_e sqrt(sum_c v_c^2) (ncomp > 0) or sum_e |v_e| (ncomp == 0), float64.
__global__ void __launch_bounds__(ct::kReduceThreads)
    k_l21_norm(const float* __restrict__ v, int ncomp, size_t n, double* __restrict__ out,
               double* __restrict__ partials, unsigned int* __restrict__ ticket) {
  double acc = 0.0;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n;
       e += (size_t)gridDim.x * blockDim.x) {
    if (ncomp == 0) {
      acc += fabs((double)v[e]);
    } else {
      float ss = 0.0f;
      for (int c = 0; c < ncomp; ++c) {
        const float x = v[(size_t)c * n + e];
        const float sq = ct::fmul(x, x);
        ss = (c == 0) ? sq : ct::fadd(ss, sq);
      }
      acc += (double)__fsqrt_rn(ss);
    }
  }
  double part[1] = {acc}, tot[1];
  if (ct::grid_reduce_last<ct::kReduceThreads, 1>(part, partials, ticket, tot)) *out = tot[0];
}

}  // namespace

extern "C" {

ct_status ct_fd_out_count(const ct_fd_desc* d, int64_t* count) {
  FdParams p{};
  ct_status st = make_fd(d, p, "ct_fd_out_count");
  if (st != CT_OK) return st;
  if (!count) return ct::fail(CT_ERR_INVALID_ARG, "ct_fd_out_count: null count");
  *count = (int64_t)p.out_count;
  return CT_OK;
}

ct_status ct_fd_fwd(const ct_fd_desc* d, const float* x, float* out, int32_t batch,
                    ct_stream_t stream) {
  FdParams p{};
  ct_status st = make_fd(d, p, "ct_fd_fwd");
  if (st != CT_OK) return st;
  if (!x || !out) return ct::fail(CT_ERR_INVALID_ARG, "ct_fd_fwd: null array");
  if (batch <= 0) return ct::fail(CT_ERR_INVALID_ARG, "ct_fd_fwd: batch=%d", batch);
  const size_t total = p.out_count * batch;
  if (total == 0) return CT_OK;
  k_fd_fwd<<<grid_for(total, 256), 256, 0, ct::as_stream(stream)>>>(x, out, p, batch);
  return ct::launch_check("k_fd_fwd");
}

ct_status ct_fd_adj(const ct_fd_desc* d, const float* dx, float* x, int32_t batch,
                    ct_stream_t stream) {
  FdParams p{};
  ct_status st = make_fd(d, p, "ct_fd_adj");
  if (st != CT_OK) return st;
  if (!x || !dx) return ct::fail(CT_ERR_INVALID_ARG, "ct_fd_adj: null array");
  if (batch <= 0) return ct::fail(CT_ERR_INVALID_ARG, "ct_fd_adj: batch=%d", batch);
  const size_t total = p.in_count * batch;
  k_fd_adj<<<grid_for(total, 256), 256, 0, ct::as_stream(stream)>>>(dx, x, p, batch);
  return ct::launch_check("k_fd_adj");
}

ct_status ct_haar_fwd(const ct_fd_desc* d, const float* x, float* w, int32_t batch, ct_stream_t stream) {
  FdParams p{};
  ct_status st = make_fd(d, p, "ct_haar_fwd");
  if (st != CT_OK) return st;
  if (!x || !w) return ct::fail(CT_ERR_INVALID_ARG, "ct_haar_fwd: null array");
  if (batch <= 0) return ct::fail(CT_ERR_INVALID_ARG, "ct_haar_fwd: batch=%d", batch);
  const size_t total = 2 * (size_t)p.nblocks * p.in_count * batch;
  k_haar_fwd<<<grid_for(total, 256), 256, 0, ct::as_stream(stream)>>>(x, w, p, (float)(1.0 / sqrt(2.0)), batch);
  return ct::launch_check("k_haar_fwd");
}

ct_status ct_haar_adj(const ct_fd_desc* d, const float* w, float* x, int32_t batch, ct_stream_t stream) {
  FdParams p{};
  ct_status st = make_fd(d, p, "ct_haar_adj");
  if (st != CT_OK) return st;
  if (!x || !w) return ct::fail(CT_ERR_INVALID_ARG, "ct_haar_adj: null array");
  if (batch <= 0) return ct::fail(CT_ERR_INVALID_ARG, "ct_haar_adj: batch=%d", batch);
  const size_t total = p.in_count * batch;
  k_haar_adj<<<grid_for(total, 256), 256, 0, ct::as_stream(stream)>>>(w, x, p, (float)(1.0 / sqrt(2.0)), batch);
  return ct::launch_check("k_haar_adj");
}

ct_status ct_l21_prox(const float* v, float* out, int32_t ncomp, int64_t n, float lam,
                      ct_stream_t stream) {
  if (!v || !out) return ct::fail(CT_ERR_INVALID_ARG, "ct_l21_prox: null array");
  if (ncomp < 1 || n < 0)
    return ct::fail(CT_ERR_INVALID_ARG, "ct_l21_prox: ncomp=%d n=%lld", ncomp, (long long)n);
  if (n == 0) return CT_OK;
  k_l21_prox<<<grid_for((size_t)n, 256), 256, 0, ct::as_stream(stream)>>>(v, out, ncomp,
                                                                           (size_t)n, lam);
  return ct::launch_check("k_l21_prox");
}

ct_status ct_l1_prox(const float* v, float* out, int64_t n, float lam, ct_stream_t stream) {
  if (!v || !out) return ct::fail(CT_ERR_INVALID_ARG, "ct_l1_prox: null array");
  if (n < 0) return ct::fail(CT_ERR_INVALID_ARG, "ct_l1_prox: n=%lld", (long long)n);
  if (n == 0) return CT_OK;
  k_l1_prox<<<grid_for((size_t)n, 256), 256, 0, ct::as_stream(stream)>>>(v, out, (size_t)n, lam);
  return ct::launch_check("k_l1_prox");
}

ct_status ct_l21_norm(const float* v, int32_t ncomp, int64_t n, double* out_dev, void* workspace,
                      size_t workspace_bytes, ct_stream_t stream) {
  if (!v || !out_dev) return ct::fail(CT_ERR_INVALID_ARG, "ct_l21_norm: null pointer");
  if (ncomp < 0 || n < 0)
    return ct::fail(CT_ERR_INVALID_ARG, "ct_l21_norm: ncomp=%d n=%lld", ncomp, (long long)n);
  if (!workspace || workspace_bytes < ct::kReduceWorkspace || !ct::aligned(workspace, 256))
    return ct::fail(CT_ERR_WORKSPACE, "ct_l21_norm: need %zu bytes", ct::kReduceWorkspace);
  unsigned int* ticket = static_cast<unsigned int*>(workspace);
  double* partials = reinterpret_cast<double*>(static_cast<char*>(workspace) + 256);
  k_l21_norm<<<ct::kReduceBlocks, ct::kReduceThreads, 0, ct::as_stream(stream)>>>(
      v, ncomp, (size_t)n, out_dev, partials, ticket);
  return ct::launch_check("k_l21_norm");
}

}  // extern "C"
