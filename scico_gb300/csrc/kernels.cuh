// Internal launchers shared between translation units of the ctgpu library.
#pragma once

#include "common.cuh"

namespace ct {

// ---- 2D projector (proj2d.cu) ---------------------------------------------
struct Proj2dPlan {
  // forward: 32-row x 256-column strips, views per CTA, bins per tile / strip
  int tiles_i, n_chunks, n_strips, L, LS, cspan, vpc, fwd_groups;
  size_t fwd_bytes, fwd_smem;
  // adjoint: 16x64 tiles, view splits, staged window length
  int adj_gx, adj_gy, nsplit, per_split, W;
  size_t adj_bytes;  // split partial images (0 when nsplit == 1)
  size_t adj_smem;
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
// cond/use_cond: in a graph with a conditional WHILE CG loop, the update sets
// the loop condition to "not converged".
ct_status cg_update_launch(float* x, float* r, const float* p, const float* Ap, size_t n,
                           double* scalars, void* red_ws, cudaStream_t s,
                           cudaGraphConditionalHandle cond = 0, int use_cond = 0);
ct_status cg_direction_launch(float* p, const float* r, size_t n, double* scalars, void* red_ws,
                              cudaStream_t s);

// ---- generic N-way float64 grid sum (see grid_reduce_last in common.cuh) ----
template <int NT, int K>
__device__ __forceinline__ bool grid_sumk_last(double (&v)[K], double* partials, unsigned int* ticket,
                                               double (&out)[K]) {
  return grid_reduce_last<NT, K>(v, partials, ticket, out);
}

}  // namespace ct
