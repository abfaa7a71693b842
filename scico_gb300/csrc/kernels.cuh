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
  size_t adj_bytes;     // split partial images of this plan (0 when nsplit == 1)
  size_t adj_ws_bytes;  // the same for the largest split count a schedule may pick
  size_t adj_smem;
};

// Launch schedule of the 2D projector: forward views per CTA and adjoint view
// splits (0 = the planner's default).  ct_proj2d_autotune measures candidates
// and records the fastest per geometry; proj2d_plan uses the recorded one.
struct Sched2d {
  int vpc = 0;
  int ns = 0;
};

ct_status proj2d_check(const ct_geom2d* g, const char* who);
Proj2dPlan proj2d_plan(const ct_geom2d* g, int batch);  // recorded schedule, else default
Proj2dPlan proj2d_plan_sched(const ct_geom2d* g, int batch, Sched2d s);
// Current poll limit of the forward's strip-copy wait (ct_set_wait_poll_limit).
uint32_t proj2d_wait_polls();
// Device address of the library's device error word (ct_proj2d_check).
int* proj2d_errflag_ptr();
// out[e] = sum over the adjoint's view splits (in split order) of part[k n + e].
ct_status proj2d_sum_splits(const float* part, float* out, size_t n, int nsplit, cudaStream_t s);
// One-time per-process function attributes (large dynamic shared memory);
// must run before any stream capture.
ct_status proj2d_prepare(const Proj2dPlan& p);

// sino = A img.  `skip` (device, may be null): when *skip != 0 the kernels
// return immediately (used to freeze converged CG iterations in a graph).
// dependent: the stream predecessor is one of this library's kernels, so the
// first kernel may be launched as its dependent (launch_k in common.cuh).
ct_status proj2d_fwd_launch(const ct_geom2d* g, const Proj2dPlan& p, const float* img, float* sino,
                            int batch, float* part, cudaStream_t s, const double* skip,
                            bool dependent = false);

// A^T sino.  With p.nsplit == 1 the result goes to `out`; otherwise split k
// of the views goes to part + k * batch*rows*cols and the caller sums them.
// dependent: the stream predecessor is one of this library's kernels, so the
// adjoint may be launched as its dependent (launch_k in common.cuh).
ct_status proj2d_adj_launch(const ct_geom2d* g, const Proj2dPlan& p, const float* sino, float* out,
                            float* part, int batch, cudaStream_t s, const double* skip,
                            bool dependent = false);

// ---- 3D projector (proj3d.cu) ---------------------------------------------
struct Proj3dPlan {
  // AXIS0 forward: slices padded to the CTA's 64, tiles, tile groups, views per CTA
  int Spad = 0, tiles_k = 0, n_tiles = 0, G = 1, vpc = 16;
  size_t fwd_smem = 0;
  // adjoint view splits (both kinds)
  int nsplit = 1, per_split = 0;
  size_t fwd_bytes = 0, adj_bytes = 0;
  // the same for the largest tile-group / split counts a schedule may use
  // (workspaces sized with these stay valid after ct_proj3d_autotune)
  size_t fwd_ws_bytes = 0, adj_ws_bytes = 0;
};

// Launch schedule of the 3D projector: AXIS0 forward tile groups and
// adjoint view splits (0 = the planner's default).
struct Sched3d {
  int G = 0;
  int ns = 0;
};

ct_status proj3d_check(const ct_geom3d* g, const char* who);
Proj3dPlan proj3d_plan(const ct_geom3d* g, int batch);  // recorded schedule, else default
Proj3dPlan proj3d_plan_sched(const ct_geom3d* g, Sched3d s);
// One-time per-process function attributes; must run before any stream capture.
ct_status proj3d_prepare(const ct_geom3d* g, const Proj3dPlan& p);
// proj = A vol for one volume; `ws` holds p.fwd_bytes.  `skip` as for 2D.
ct_status proj3d_fwd_launch(const ct_geom3d* g, const Proj3dPlan& p, const float* vol, float* proj,
                            void* ws, cudaStream_t s, const double* skip);
// A^T proj for one projection set.  With p.nsplit == 1 the result goes to
// `out`; otherwise view split k goes to part + k * (volume size) and the
// caller sums the splits in order.
ct_status proj3d_adj_launch(const ct_geom3d* g, const Proj3dPlan& p, const float* proj, float* out,
                            float* part, cudaStream_t s, const double* skip);

// ---- CG vector steps (vec.cu) ----------------------------------------------
// cond/use_cond: in a graph with a conditional WHILE CG loop, the update sets
// the loop condition to "not converged".
// dependent: launched as the dependent of the stream predecessor, which
// must be one of this library's kernels (launch_k in common.cuh).
ct_status cg_update_launch(float* x, float* r, const float* p, const float* Ap, size_t n,
                           double* scalars, void* red_ws, cudaStream_t s,
                           cudaGraphConditionalHandle cond = 0, int use_cond = 0, bool dependent = false);
ct_status cg_direction_launch(float* p, const float* r, size_t n, double* scalars, void* red_ws,
                              cudaStream_t s, bool dependent = false);

// ---- generic N-way float64 grid sum (see grid_reduce_last in common.cuh) ----
template <int NT, int K>
__device__ __forceinline__ bool grid_sumk_last(double (&v)[K], double* partials, unsigned int* ticket,
                                               double (&out)[K]) {
  return grid_reduce_last<NT, K>(v, partials, ticket, out);
}

}  // namespace ct
