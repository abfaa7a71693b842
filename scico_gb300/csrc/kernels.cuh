// Internal launchers shared between translation units of the ctgpu library.
#pragma once

#include "common.cuh"

namespace ct {

// ---- 2D projector (proj2d.cu) ---------------------------------------------
struct Proj2dPlan {
  int tiles_i, tiles_j, n_tiles, L, LS, view_groups;
  size_t fwd_bytes, fwd_smem;
  int adj_gx, adj_gy, nsplit, per_split;
  size_t adj_bytes;  // split partial images (0 when nsplit == 1)
};

ct_status proj2d_check(const ct_geom2d* g, const char* who);
Proj2dPlan proj2d_plan(const ct_geom2d* g, int batch);
// One-time per-process function attributes (large dynamic shared memory);
// must run before any stream capture.
ct_status proj2d_prepare(const Proj2dPlan& p);

// sino = A img.  `skip` (device, may be null): when *skip != 0 the kernels
// return immediately (used to freeze converged CG iterations in a graph).
ct_status proj2d_fwd_launch(const ct_geom2d* g, const Proj2dPlan& p, const float* img, float* sino,
                            int batch, float* part, cudaStream_t s, const double* skip);

// A^T sino.  With p.nsplit == 1 the result goes to `out`; otherwise split k
// of the views goes to part + k * batch*rows*cols and the caller sums them.
ct_status proj2d_adj_launch(const ct_geom2d* g, const Proj2dPlan& p, const float* sino, float* out,
                            float* part, int batch, cudaStream_t s, const double* skip);

// ---- CG vector steps (vec.cu) ----------------------------------------------
ct_status cg_update_launch(float* x, float* r, const float* p, const float* Ap, size_t n,
                           double* scalars, void* red_ws, cudaStream_t s);
ct_status cg_direction_launch(float* p, const float* r, size_t n, double* scalars, cudaStream_t s);

// ---- generic N-way float64 grid sum ------------------------------------------
// All threads call with their K partial values; returns true in thread 0 of
// the last block to finish, with `out` holding the K grid totals (block
// partials summed in block order).
template <int NT, int K>
__device__ __forceinline__ bool grid_sumk_last(double (&v)[K], double* partials,
                                               unsigned int* ticket, double (&out)[K]) {
  __shared__ double red[K][NT / 32];
  __shared__ bool is_last;
#pragma unroll
  for (int k = 0; k < K; ++k)
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) red[k][warp] = v[k];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) {
      double s = 0.0;
      for (int w = 0; w < NT / 32; ++w) s += red[k][w];
      partials[(size_t)K * blockIdx.x + k] = s;
    }
    __threadfence();
    is_last = (atomicAdd(ticket, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (!is_last || threadIdx.x != 0) return false;
  __threadfence();
  volatile double* vp = partials;
#pragma unroll
  for (int k = 0; k < K; ++k) out[k] = 0.0;
  for (unsigned int b = 0; b < gridDim.x; ++b) {
#pragma unroll
    for (int k = 0; k < K; ++k) out[k] += vp[(size_t)K * b + k];
  }
  *ticket = 0u;
  return true;
}

}  // namespace ct
