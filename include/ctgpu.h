/*
 * ctgpu.h -- C ABI of the GB300 (sm_103a) CT reconstruction hot path.
 *
 * The library replaces the array kernels behind scico's parallel-beam CT
 * ADMM-TV path.  Every entry point takes plain pointers and sizes, enqueues
 * its work on the caller's CUDA stream and returns a ct_status; none of them
 * allocates device memory.  Scratch memory, where an operation needs it, is
 * a caller-provided workspace whose size is reported by a *_workspace query
 * (the way an XLA FFI handler gets a scratch buffer from XLA, or a torch
 * binding gets one from the caching allocator).
 *
 * Interfaces replaced (scico, path within the scico source tree):
 *   ct_proj2d_*   scico/linop/xray/_xray2d.py  XRayTransform2D
 *   ct_proj3d_*   scico/linop/xray/_xray3d.py  XRayTransform3D
 *   ct_fd_*       scico/linop/_diff.py         FiniteDifference (+ its adjoint)
 *   ct_l21_*      scico/functional/_norm.py    L21Norm, L1Norm
 *   ct_cg_ and ct_dot scico/solver.py          cg
 *   ct_admm_tv_*  scico/optimize/_admm.py + _admmaux.py  ADMM with
 *                 LinearSubproblemSolver on 0.5||Ax-y||^2 + sum_i lam_i g_i(Dx)
 *
 * Conventions: all arrays are C-order float32 on the device unless noted;
 * "batch" stacks independent problems that share one geometry along a new
 * leading axis.  Results are deterministic: no kernel uses floating-point
 * atomics, every reduction runs in a fixed order.
 */
#ifndef CTGPU_H
#define CTGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* A cudaStream_t, passed through unchanged (0 = legacy default stream). */
typedef void* ct_stream_t;

typedef enum ct_status {
  CT_OK = 0,
  CT_ERR_INVALID_ARG = 1, /* null pointer, bad enum, non-positive size     */
  CT_ERR_SHAPE = 2,       /* sizes that do not conform                     */
  CT_ERR_UNSUPPORTED = 3, /* valid request outside what the library covers */
  CT_ERR_CUDA = 4,        /* a CUDA runtime call or launch failed          */
  CT_ERR_TIMEOUT = 5,     /* a bounded device wait ran out                 */
  CT_ERR_NONFINITE = 6,   /* NaN/Inf met where the caller asked to stop    */
  CT_ERR_WORKSPACE = 7,   /* workspace missing, misaligned or too small    */
  CT_ERR_NO_DEVICE = 8    /* no usable CUDA device                         */
} ct_status;

/* Library identification and error text. */
const char* ct_version(void);
const char* ct_status_string(ct_status s);
/* Message of the last failing call on the calling host thread ("" if none). */
const char* ct_last_error(void);

/* ------------------------------------------------------------------------ */
/* 2D parallel-beam projector (XRayTransform2D)                             */
/* ------------------------------------------------------------------------ */

/* Floats per view in the per-view geometry table. */
#define CT_VIEW2D_STRIDE 8

/*
 * Fill the per-view geometry table on the HOST, in float32 arithmetic and in
 * the order of XRayTransform2D._calc_weights (scico/linop/xray/_xray2d.py:
 * 326-347): u = (cos a, sin a); Px0 = x0[0]u0 + x0[1]u1 - y0;
 * Pdx = (dx0 u0, dx1 u1); Pxmin = min of the 4 pixel-corner projections;
 * width = (max(|Pdx0+Pdx1|,|Pdx0-Pdx1|) + min(...)) / 2.
 * Row v of views_out = {Pxmin, Pdx0, Pdx1, width, 1/width, 0, 0, 0}.
 * Also returns (optional, may be NULL) the largest projected pixel width,
 * the quantity XRayTransform2D.__init__ warns about when > 1 (:96-106).
 */
ct_status ct_proj2d_views(const float* angles, int32_t n_views, float x0_0,
                          float x0_1, float dx0, float dx1, float y0,
                          float* views_out, float* max_width_out);

typedef struct ct_geom2d {
  int32_t rows;      /* image axis 0                                   */
  int32_t cols;      /* image axis 1                                   */
  int32_t n_views;   /* number of angles                               */
  int32_t det_count; /* detector bins                                  */
  const float* views; /* DEVICE pointer to the n_views x 8 view table  */
  float max_width;   /* max_width_out of ct_proj2d_views for the table */
} ct_geom2d;

/* Workspace bytes that ct_proj2d_fwd / ct_proj2d_adj need for `batch`. */
ct_status ct_proj2d_workspace(const ct_geom2d* g, int32_t batch,
                              size_t* fwd_bytes, size_t* adj_bytes);

/*
 * sino[b, v, :] = A img[b]   (XRayTransform2D.project, _xray2d.py:138-146,
 * _project :223-265).  img: batch x rows x cols, sino: batch x n_views x
 * det_count.  Tile-owned pixel-driven sweep: each CTA owns an image tile
 * and a run of views, bins of one tile are reduced in shared memory and the
 * per-tile partial bins are summed in a fixed order by a second pass.
 */
ct_status ct_proj2d_fwd(const ct_geom2d* g, const float* img, float* sino,
                        int32_t batch, void* workspace, size_t workspace_bytes,
                        ct_stream_t stream);

/*
 * Allocation-free variant of ct_proj2d_fwd, for callers that cannot
 * allocate device memory when they project (inside a stream capture they do
 * not own, in plugin hosts that give a custom call no allocator or scratch
 * buffer, in real-time loops that forbid allocation after start-up).  No
 * counterpart in the reference: scico's projector allocates through XLA.
 * The scratch is a fixed 16 MiB array in the library's device memory, held
 * by every GPU that loads the library until the process exits; projections
 * whose scratch (ct_proj2d_workspace's fwd_bytes) exceeds 16 MiB are
 * rejected with CT_ERR_UNSUPPORTED.  All calls share that array: calls that
 * overlap on the GPU (other streams, other host threads) race and must be
 * serialised by the caller.  Nothing in the array needs clearing between
 * calls.  The first call on a device looks up the array's address for that
 * device; make it before any stream capture.  Calls no cudaMalloc or cudaFree.
 */
ct_status ct_proj2d_fwd_noalloc(const ct_geom2d* g, const float* img,
                                float* sino, int32_t batch,
                                ct_stream_t stream);

/*
 * img[b] = A^T sino[b]  (XRayTransform2D.back_project, :148-156,
 * _back_project :267-306).  Pixel-driven gather with the forward's weights,
 * views summed in a fixed order, no atomics.
 */
ct_status ct_proj2d_adj(const ct_geom2d* g, const float* sino, float* img,
                        int32_t batch, void* workspace, size_t workspace_bytes,
                        ct_stream_t stream);

/*
 * Device-side checks.  The projector kernels never trap: a check that fails
 * on the device sets a bit of a per-device error word and skips the work it
 * guards (bit 0: a forward tile's bins exceed the plan; bit 1: a forward
 * strip copy did not complete within the wait's poll limit, and the CTA
 * wrote zeros for its bins; bit 2: an adjoint view window exceeds the plan).
 * No reference counterpart (scico's projector is XLA code without waits).
 *
 * ct_proj2d_check synchronises `stream`, then reads and clears the word:
 * CT_OK when it was 0, CT_ERR_TIMEOUT when bit 1 was set, else
 * CT_ERR_UNSUPPORTED; ct_last_error() names the bits.  ct_proj2d_errflag
 * and ct_proj3d_errflag return and clear the raw words (-1 if unreadable).
 *
 * ct_set_wait_poll_limit sets the number of mbarrier polls the forward's
 * strip-copy wait makes before it gives up (default 2^24, process-wide,
 * read when a call launches; a solver graph keeps the value current at
 * its capture).  0 makes every wait give up at once: failure-detection
 * tests use it to exercise the timeout path without a hung GPU.
 */
ct_status ct_proj2d_check(ct_stream_t stream);
/* (bit 3 of the word: a grid barrier wait of the solver's fast-forward
 * kernel ran out -- ct_set_solver_fast_forward; reported as CT_ERR_TIMEOUT) */
int ct_proj2d_errflag(void);
int ct_proj3d_errflag(void);
void ct_set_wait_poll_limit(uint32_t polls);
uint32_t ct_wait_poll_limit(void);

/*
 * Launch schedule of the 2D projector for one geometry and batch: views per
 * CTA of the forward and view splits of the adjoint.  No counterpart in the
 * reference (XLA picks its own launch shapes); the batched-scan workload asks
 * for schedules chosen by measurement.
 */
typedef struct ct_proj2d_schedule {
  int32_t views_per_cta; /* forward: views per CTA */
  int32_t adj_splits;    /* adjoint: view splits (partial images summed in order) */
  float fwd_us;          /* measured device time per forward call (0 if not measured) */
  float adj_us;          /* measured device time per adjoint call (0 if not measured) */
  int32_t tuned;         /* 1: recorded by ct_proj2d_autotune; 0: the planner's default */
} ct_proj2d_schedule;

/*
 * Autotuner: times the forward for each candidate views-per-CTA and the
 * adjoint (with its split sum) for the split counts 1, 2, 4, 8, ... on
 * `stream` with CUDA events (one untimed call, then `reps` timed calls
 * each), and records the fastest forward and, among adjoint timings within
 * 3 % of the fastest, the fewest splits (so the choice, which sets the
 * adjoint's summation order, does not flip between runs on noise) in a
 * process-wide table (guarded by a mutex) keyed by the geometry's sizes and
 * batch.  Every later call on that
 * geometry (ct_proj2d_fwd/adj, the fused solvers) uses the recorded
 * schedule; results change only in the adjoint's split summation order.
 * img and sino are scratch (overwritten); the workspace needs
 * max(fwd_bytes, adj_bytes) of ct_proj2d_workspace, whose adj_bytes already
 * covers every split count a schedule may pick, so workspaces sized before
 * tuning stay valid.  Blocks the host until the stream drains; not allowed
 * inside a stream capture (CT_ERR_INVALID_ARG).
 */
ct_status ct_proj2d_autotune(const ct_geom2d* g, int32_t batch, float* img,
                             float* sino, void* workspace, size_t workspace_bytes,
                             int32_t reps, ct_stream_t stream,
                             ct_proj2d_schedule* chosen);

/* The schedule ct_proj2d_fwd/adj use for this geometry and batch now. */
ct_status ct_proj2d_schedule_get(const ct_geom2d* g, int32_t batch,
                                 ct_proj2d_schedule* out);

/* Forget every recorded schedule (later calls use the planner's defaults). */
void ct_proj2d_schedule_clear(void);

/*
 * Ramp filter of XRayTransform2D.fbp (_xray2d.py:158-221): every row of
 * `sino` (n_rows rows of det_count samples, e.g. batch x n_views) convolved
 * with the Kak & Slaney eq. (61) ramp filter at tau = 1 and cropped to the
 * input's samples, as the reference's zero-padded FFT product does.  FBP is
 * then A^T of the filtered rows, masked and scaled (scico_gb300.linop).
 */
ct_status ct_fbp_filter(const float* sino, float* out, int32_t n_rows,
                        int32_t det_count, ct_stream_t stream);

/* ------------------------------------------------------------------------ */
/* 3D parallel-beam projector (XRayTransform3D)                             */
/* ------------------------------------------------------------------------ */

/* Floats per view in the table ct_proj3d_views writes: the (2,4) projection
 * matrix row-major (entries 0..7), the axis along which the ray direction
 * has its largest component (entry 8, as a float), three unused. */
#define CT_VIEW3D_STRIDE 12
/* uint16 entries per view in the walk-order table of CT_PROJ3D_AXIS0 (one
 * 16 x 16 pixel tile, entry = 16 * row + column). */
#define CT_PROJ3D_ORDER 256

/* Geometry kinds.  AXIS0: every view leaves volume axis 0 on detector rows
 * (M[0][1] = M[0][2] = M[1][0] = 0, |M[1][1]|, |M[1][2]| <= 1) and, in every
 * view, slice i lands on detector row i + row_offset with to_next = 0.5, so
 * only the ul/ll taps carry weight --
 * the rotation-about-axis-0 geometry of matrices_from_euler_angles(..., "X",
 * ...) with equal slice and detector-row counts or an even difference.
 * The AXIS0 kernels compute each column weight once per view and apply it to
 * every slice.  GENERAL: any other matrices. */
#define CT_PROJ3D_GENERAL 0
#define CT_PROJ3D_AXIS0 1

/*
 * Host: build the per-view tables of a geometry (XRayTransform3D.__init__
 * keeps the (V,2,4) matrices as float32, scico/linop/xray/_xray3d.py:80) and
 * classify it.  matrices: host (n_views,2,4) float32.  views_out: host
 * n_views*CT_VIEW3D_STRIDE floats.  order_out: host n_views*CT_PROJ3D_ORDER
 * uint16 (the AXIS0 walk order of a 16x16 pixel tile, ordered along the
 * detector), or NULL, in which case the kind is always GENERAL.
 * Fails with CT_ERR_UNSUPPORTED when a matrix has parallel rows (a view
 * that maps the volume onto a line).
 */
ct_status ct_proj3d_views(const float* matrices, int32_t n_views,
                          const int32_t* shape, const int32_t* det_shape,
                          float* views_out, uint16_t* order_out,
                          int32_t* kind_out, int32_t* row_offset_out);

typedef struct ct_geom3d {
  int32_t shape[3];        /* volume (n0, n1, n2), C order              */
  int32_t det_shape[2];    /* detector (rows, cols)                     */
  int32_t n_views;
  int32_t kind;            /* CT_PROJ3D_GENERAL or CT_PROJ3D_AXIS0      */
  int32_t row_offset;      /* AXIS0: detector row of slice i - i        */
  const float* views;      /* device, n_views*CT_VIEW3D_STRIDE          */
  const uint16_t* order;   /* device, n_views*CT_PROJ3D_ORDER (AXIS0)   */
} ct_geom3d;

/* Workspace bytes that ct_proj3d_fwd / ct_proj3d_adj need for `batch`. */
ct_status ct_proj3d_workspace(const ct_geom3d* g, int32_t batch,
                              size_t* fwd_bytes, size_t* adj_bytes);

/*
 * proj[b] = A vol[b]  (XRayTransform3D.project / _project / _project_single,
 * _xray3d.py:95-159; weights _calc_weights :206-266).  vol (batch, n0, n1, n2)
 * -> proj (batch, n_views, rows, cols).  The reference scatters four taps
 * per voxel with mode="drop"; here every detector pixel gathers its taps
 * (GENERAL) or each slice's column contributions are accumulated by one
 * owner in a fixed order (AXIS0): no atomics, deterministic.
 */
ct_status ct_proj3d_fwd(const ct_geom3d* g, const float* vol, float* proj,
                        int32_t batch, void* workspace, size_t workspace_bytes,
                        ct_stream_t stream);

/*
 * vol[b] = A^T proj[b]  (XRayTransform3D.back_project / _back_project /
 * _back_project_single, :161-204).  Voxel-driven gather with the forward's
 * weights, views summed in a fixed order.
 */
ct_status ct_proj3d_adj(const ct_geom3d* g, const float* proj, float* vol,
                        int32_t batch, void* workspace, size_t workspace_bytes,
                        ct_stream_t stream);

/*
 * Launch schedule of the 3D projector.  No reference counterpart: scico
 * runs the 3D projector through lax.map with a fixed view batch
 * (scico/linop/xray/_xray3d.py:110-139).
 */
typedef struct ct_proj3d_schedule {
  int32_t tile_groups; /* AXIS0 forward: tile groups (accumulators summed in group order) */
  int32_t adj_splits;  /* adjoint: view splits (partial volumes summed in order) */
  float fwd_us;        /* measured device time per forward call (0 if not measured) */
  float adj_us;        /* measured device time per adjoint call (0 if not measured) */
  int32_t tuned;       /* 1: recorded by ct_proj3d_autotune; 0: the planner's default */
} ct_proj3d_schedule;

/*
 * Autotuner of the 3D projector: times the AXIS0 forward for tile-group
 * counts 1..8 (GENERAL geometries have no forward schedule) and the adjoint
 * with its split sum for 1, 2 and 4 view splits, on `stream` with CUDA
 * events (one untimed call, then `reps` timed ones each), and records the
 * fastest forward and, among adjoint timings within 3 % of the fastest, the
 * fewest splits, in a process-wide table (mutex-guarded) keyed by the
 * geometry's sizes and kind.  Later calls on that geometry (ct_proj3d_fwd /
 * adj, the fused 3D solver) use the recorded schedule; results change only
 * in summation order.  `vol` and `proj` are scratch arrays of the
 * geometry's sizes (overwritten); the workspace must hold both sizes
 * ct_proj3d_workspace reports, which cover every schedule the tuner may
 * record.  Not inside a stream capture (CT_ERR_INVALID_ARG).
 */
ct_status ct_proj3d_autotune(const ct_geom3d* g, float* vol, float* proj,
                             void* workspace, size_t workspace_bytes,
                             int32_t reps, ct_stream_t stream,
                             ct_proj3d_schedule* chosen);

/* The schedule ct_proj3d_fwd/adj use for this geometry now. */
ct_status ct_proj3d_schedule_get(const ct_geom3d* g, ct_proj3d_schedule* out);

/* Forget every recorded 3D schedule (later calls use the planner's defaults). */
void ct_proj3d_schedule_clear(void);

/* ------------------------------------------------------------------------ */
/* Finite differences (FiniteDifference / SingleAxisFiniteDifference)       */
/* ------------------------------------------------------------------------ */

/* prepend/append: -1 = None, 0 or 1 as in scico/linop/_diff.py:157-225.  */
typedef struct ct_fd_desc {
  int32_t ndim;      /* 1, 2 or 3                                        */
  int32_t shape[3];  /* input shape (first ndim entries)                 */
  int32_t naxes;     /* number of differenced axes                       */
  int32_t axes[3];   /* the axes, in output-block order                  */
  int32_t prepend;   /* -1, 0, 1                                         */
  int32_t append;    /* -1, 0, 1                                         */
  int32_t circular;  /* 0 / 1 (then prepend = append = -1)               */
} ct_fd_desc;

/* Number of output elements: the blocks of every axis, concatenated in axis
 * order (when all blocks share one shape this is the (naxes, *shape) stack of
 * VerticalStack, scico/operator/_stack.py:87-88,126-129). */
ct_status ct_fd_out_count(const ct_fd_desc* d, int64_t* count);

/* out = D x   (SingleAxisFiniteDifference._eval, _diff.py:236-272). */
ct_status ct_fd_fwd(const ct_fd_desc* d, const float* x, float* out,
                    int32_t batch, ct_stream_t stream);

/* x = D^T out = sum_k D_k^T out_k  (adjoint of the above; the reference
 * derives it with jax.linear_transpose, scico/_core.py:140-153, summed per
 * block in scico/linop/_stack.py:71-72). */
ct_status ct_fd_adj(const ct_fd_desc* d, const float* dx, float* x,
                    int32_t batch, ct_stream_t stream);

/* w = HaarTransform(x): the single-level shift-invariant Haar transform of
 * the TV norms' prox over d->axes (HaarTransform / SingleAxisHaarTransform,
 * scico/functional/_tvnorm.py:458-538): for axis k, w[k][0] =
 * r (x + roll(x, -1)) and w[k][1] = r (roll(x, -1) - x), r = float32(1/sqrt 2),
 * w of shape (naxes, 2, *shape) per batch item.  Only d's ndim, shape, naxes
 * and axes are read. */
ct_status ct_haar_fwd(const ct_fd_desc* d, const float* x, float* w,
                      int32_t batch, ct_stream_t stream);

/* x = its adjoint: the sum over axes, in order, of r (lo + roll(lo, 1)) +
 * r (roll(hi, 1) - hi) (the transpose jax builds for the reference's
 * FiniteSum / circular FiniteDifference, summed per VerticalStack block). */
ct_status ct_haar_adj(const ct_fd_desc* d, const float* w, float* x,
                      int32_t batch, ct_stream_t stream);

/* ------------------------------------------------------------------------ */
/* Proximal operators and norms (scico/functional/_norm.py)                 */
/* ------------------------------------------------------------------------ */

/* out = prox_{lam ||.||_{2,1}}(v), l2 over the leading axis of ncomp
 * components each of n elements (L21Norm._prox with l2_axis=0, :254-263,
 * no_nan_divide scico/numpy/util.py:302-315). out may alias v. */
ct_status ct_l21_prox(const float* v, float* out, int32_t ncomp, int64_t n,
                      float lam, ct_stream_t stream);

/* out = sign(v) max(|v| - lam, 0)  (L1Norm.prox, _norm.py:84-117). */
ct_status ct_l1_prox(const float* v, float* out, int64_t n, float lam,
                     ct_stream_t stream);

/* *out_dev (float64, device) = sum_n sqrt(sum_c v[c,n]^2) (L21Norm.__call__,
 * :246-250) -- or, when ncomp == 0, sum |v| over n (L1Norm.__call__). */
ct_status ct_l21_norm(const float* v, int32_t ncomp, int64_t n,
                      double* out_dev, void* workspace, size_t workspace_bytes,
                      ct_stream_t stream);

/* ------------------------------------------------------------------------ */
/* Reductions and CG vector steps (scico/solver.py:326-405)                 */
/* ------------------------------------------------------------------------ */

/* Workspace bytes for one reduction (ct_dot, ct_l21_norm, ct_cg_*).  The
 * workspace must be zero-filled before its first use; every reduction leaves
 * it zero-filled again.  Reductions that share one workspace must not
 * overlap in time (issue them on one stream). */
size_t ct_reduce_workspace(void);

/* *out_dev (float64, device) = sum a[i] b[i], products and sums in float64,
 * fixed summation order. */
ct_status ct_dot(const float* a, const float* b, int64_t n, double* out_dev,
                 void* workspace, size_t workspace_bytes, ct_stream_t stream);

/* Device-resident CG scalars (float64), indices into a double[16]. */
#define CT_CG_NUM 0       /* <r, r>                                  */
#define CT_CG_PAP 1       /* <p, A p>                                */
#define CT_CG_ALPHA 2
#define CT_CG_BETA 3
#define CT_CG_BNORM 4     /* ||b||                                   */
#define CT_CG_TOL2 5      /* max(tol ||b||, atol)^2                  */
#define CT_CG_ITERS 6     /* iterations taken                        */
#define CT_CG_DONE 7      /* 1 once num <= TOL2 or ITERS == maxiter  */
#define CT_CG_MAXITER 8
#define CT_CG_RAN 9       /* 1 between an update that ran and its direction step */
#define CT_CG_NSCALARS 16

/*
 * CG x/r step: alpha = num / pAp; x += alpha p; r -= alpha Ap;
 * num' = <r, r>; beta = num'/num; ITERS += 1; DONE when num' <= TOL2 or
 * ITERS reaches MAXITER.  Skips all work if DONE is already set, so a fixed
 * number of launches (e.g. captured in a CUDA graph) reproduces the
 * reference's early exit.  scalars: device double[CT_CG_NSCALARS].
 */
ct_status ct_cg_update(float* x, float* r, const float* p, const float* Ap,
                       int64_t n, double* scalars, void* workspace,
                       size_t workspace_bytes, ct_stream_t stream);

/* p = r + beta p (skipped once DONE was set before the preceding update).
 * Uses the reduction workspace of the preceding ct_cg_update. */
ct_status ct_cg_direction(float* p, const float* r, int64_t n,
                          double* scalars, void* workspace,
                          size_t workspace_bytes, ct_stream_t stream);

/* CG start: r = b - Ax; p = r; NUM = <r,r>; BNORM = ||b||;
 * TOL2 = max(tol BNORM, atol)^2; ITERS = 0; DONE = (NUM <= TOL2) || maxiter==0. */
ct_status ct_cg_init(const float* b, const float* Ax, float* r, float* p,
                     int64_t n, double tol, double atol, int32_t maxiter,
                     double* scalars, void* workspace, size_t workspace_bytes,
                     ct_stream_t stream);

/* ------------------------------------------------------------------------ */
/* Fused ADMM-TV solver (2D, batches of 2D scans, 3D)                      */
/* ------------------------------------------------------------------------ */

/*
 * ADMM for  min_x 0.5 ||A x - y||^2 + lam_l21 ||D x||_{2,1} + lam_l1 ||D x||_1
 * with D = FiniteDifference(append=0) over both image axes, one g_i per
 * non-zero lam (L21 then L1, sharing D and rho), the x-update solved by CG
 * on (A^T A + rho_sum D^T D) x = A^T y + sum_i rho_i D^T (z_i - u_i)
 * (LinearSubproblemSolver, scico/optimize/_admmaux.py:205-269), and the
 * z/u updates of ADMM.step (scico/optimize/_admm.py:334-378).
 * Iteration statistics per outer iteration (ADMM itstat fields,
 * _admm.py:171-198): objective f(x)+sum g_i(z_i), primal residual,
 * dual residual, CG iterations, CG relative residual.
 */
typedef struct ct_admm_tv_desc {
  ct_geom2d geom;
  int32_t maxiter;      /* ADMM outer iterations                         */
  int32_t cg_maxiter;   /* CG cap per x-update                           */
  double cg_tol;        /* CG relative tolerance                         */
  double cg_atol;       /* CG absolute tolerance                         */
  double lam_l21;       /* weight of ||Dx||_{2,1} (0 = term absent)      */
  double lam_l1;        /* weight of ||Dx||_1     (0 = term absent)      */
  double rho;           /* ADMM penalty, same for every g_i              */
  double loss_scale;    /* SquaredL2Loss scale (0.5)                     */
  double alpha;         /* ADMM relaxation (1.0 = none)                  */
  int32_t use_graph;    /* 1 = the whole solve is one CUDA graph launch  */
} ct_admm_tv_desc;

/* Fields of one itstat record (double each). */
#define CT_ITSTAT_OBJECTIVE 0
#define CT_ITSTAT_PRIMAL 1
#define CT_ITSTAT_DUAL 2
#define CT_ITSTAT_CG_ITERS 3
#define CT_ITSTAT_CG_RELRES 4
#define CT_ITSTAT_FIELDS 8

ct_status ct_admm_tv_workspace(const ct_admm_tv_desc* d, size_t* bytes);

/* Byte offsets, inside the solver workspace, of the ADMM state arrays
 * z_list and u_list (ADMM._state_variable_names, _admm.py:200-205): each is
 * n_terms x 2 x rows x cols float32, term order L2,1 then L1.  n_terms may
 * be NULL. */
ct_status ct_admm_tv_state(const ct_admm_tv_desc* d, size_t* z_offset,
                           size_t* u_offset, int32_t* n_terms);

/*
 * Run d->maxiter ADMM iterations.  y: sinogram (n_views x det_count);
 * x: in = x0, out = final x (rows x cols); itstat_dev: device
 * double[maxiter * CT_ITSTAT_FIELDS] (may be NULL).  z/u state lives in the
 * workspace; call with iter0 == 0 to initialise z = D x0, u = 0 (ADMM.z_init /
 * u_init, _admm.py:297-332), or iter0 > 0 to continue from the workspace.
 */
ct_status ct_admm_tv_solve(const ct_admm_tv_desc* d, const float* y, float* x,
                           double* itstat_dev, int32_t iter0, void* workspace,
                           size_t workspace_bytes, ct_stream_t stream);

/*
 * Run n independent 2D solves concurrently, each exactly as
 * ct_admm_tv_solve would: scan k uses descs[k], y[k], x[k], itstat_dev[k]
 * (itstat_dev itself may be NULL) and its own workspace workspace[k] of
 * workspace_bytes[k] bytes (ct_admm_tv_workspace of descs[k]).  For many
 * scans of different sizes (no counterpart in the reference, whose scripts
 * solve one scan after another).  When every descs[k].use_graph is 1 the
 * whole batch is one CUDA graph launch on `stream`: n independent branches,
 * each a whole solve with its ADMM loop and CG loops as device-side
 * conditional nodes (the graph is built on first use and cached for the same
 * set of problems); n_streams is then unused.  Otherwise each scan runs with
 * plain launches on one of n_streams internal streams (0 = min(n, 16), at
 * most 32), scans assigned longest-estimated-first to the least-loaded
 * stream.  All work starts after prior work on `stream`, and `stream` waits
 * for all of it.
 */
ct_status ct_admm_tv_solve_batch(const ct_admm_tv_desc* descs, int32_t n,
                                 const float* const* y, float* const* x,
                                 double* const* itstat_dev, int32_t iter0,
                                 void* const* workspace,
                                 const size_t* workspace_bytes,
                                 int32_t n_streams, ct_stream_t stream);

/*
 * Fast-forward CG start of the solve graphs (ct_admm_tv_solve and
 * ct_admm_tv3d_solve with use_graph = 1; not the batch).  Once CG's
 * stopping test passes at its first step, x stops moving and an iteration
 * is only the z/u update, the next right-hand side and the CG start.  The
 * CG start is then one cooperative launch that runs such iterations back
 * to back, its blocks meeting at bounded grid barriers, and returns when CG
 * has a step to run or the call's iterations are done.  Results are
 * bit-identical with it on or off (same passes, same sums in the same
 * order).  A barrier wait that runs out (poll limit: the smaller of
 * ct_wait_poll_limit and 2^21) sets bit 3 of the device error word
 * (ct_proj2d_check reports CT_ERR_TIMEOUT).  On by default unless the
 * environment sets CTGPU_FFWD=0; used only where the device supports
 * cooperative launches and the kernels' 304 blocks fit at once.  The
 * setting is read when a solve graph is built (graphs are cached per
 * setting).  In the same graphs each CG step's vector work (lhs, update,
 * direction) is one cooperative launch with two bounded grid barriers.
 * ct_solver_fast_forward returns 1 when the setting is on and the current
 * device runs the kernels.
 */
void ct_set_solver_fast_forward(int32_t on);
int32_t ct_solver_fast_forward(void);

/*
 * The same solver for 3D parallel-beam CT (XRayTransform3D,
 * scico/linop/xray/_xray3d.py), as in scico's ct_3d_tv_* examples:
 * D = FiniteDifference(append=0) over the three volume axes, stacked
 * (3, n0, n1, n2); z_i/u_i are n_terms x 3 x n0 x n1 x n2.  Fields and
 * semantics as ct_admm_tv_desc.
 */
typedef struct ct_admm_tv3d_desc {
  ct_geom3d geom;
  int32_t maxiter;
  int32_t cg_maxiter;
  double cg_tol;
  double cg_atol;
  double lam_l21;
  double lam_l1;
  double rho;
  double loss_scale;
  double alpha;
  int32_t use_graph;
} ct_admm_tv3d_desc;

ct_status ct_admm_tv3d_workspace(const ct_admm_tv3d_desc* d, size_t* bytes);
ct_status ct_admm_tv3d_state(const ct_admm_tv3d_desc* d, size_t* z_offset,
                             size_t* u_offset, int32_t* n_terms);
/* y: projections (n_views x rows x cols); x: volume (n0 x n1 x n2). */
ct_status ct_admm_tv3d_solve(const ct_admm_tv3d_desc* d, const float* y, float* x,
                             double* itstat_dev, int32_t iter0, void* workspace,
                             size_t workspace_bytes, ct_stream_t stream);

/* ------------------------------------------------------------------------ */
/* Unrolled CG block of MoDL with a hand-written backward                   */
/* (scico.flax.inverse.cg_solver, scico/flax/inverse.py:113-158)            */
/* ------------------------------------------------------------------------ */

/*
 * maxiter steps of CG on (gram_scale H^T H + lam I) x = b for nsys images
 * sharing the 2D projector H, from x0 (or 0), float32 vectors and float64
 * per-image scalars (the fixed-iteration solver the MoDL network unrolls,
 * without a stopping test).  ct_cg_block_fwd records the iterates in a tape
 * (recompute = 0) or only the step scalars (recompute = 1: the backward
 * recomputes the iterates from the block's inputs b, lam, x0, its
 * checkpoint).  ct_cg_block_bwd runs the reverse recurrence of the steps
 * (the gradient of a loss through x) and returns the gradients of b, x0
 * (optional) and lam (summed over the images, one float64 on the device).
 * gram_scale is c^2 for a projector scaled by c.
 */
typedef struct ct_cg_block_desc {
  ct_geom2d geom;
  int32_t nsys;        /* images (batch)                                     */
  int32_t maxiter;     /* CG steps                                           */
  int32_t recompute;   /* 1: the backward recomputes the iterates            */
  float gram_scale;    /* A = gram_scale H^T H + lam I                        */
} ct_cg_block_desc;

ct_status ct_cg_block_workspace(const ct_cg_block_desc* d, size_t* tape_bytes,
                                size_t* workspace_bytes);
/* b, x0 (may be NULL: zero), x: nsys x rows x cols. */
ct_status ct_cg_block_fwd(const ct_cg_block_desc* d, const float* b, float lam,
                          const float* x0, float* x, void* tape, size_t tape_bytes,
                          void* workspace, size_t workspace_bytes,
                          ct_stream_t stream);
/* gx: gradient of the loss with respect to x; b is needed with recompute;
 * x0 as given to the forward (NULL: zero); gx0 may be NULL. */
ct_status ct_cg_block_bwd(const ct_cg_block_desc* d, const float* gx, const float* b,
                          float lam, const float* x0, void* tape, size_t tape_bytes,
                          float* gb, float* gx0, double* glam, void* workspace,
                          size_t workspace_bytes, ct_stream_t stream);

/* ------------------------------------------------------------------------ */
/* Fused proximal ADMM for CT-TV (ProximalADMM, scico/optimize/_padmm.py)    */
/* ------------------------------------------------------------------------ */

/*
 * The CG-free split of the reference's ct_3d_tv_padmm example
 * (examples/scripts/ct_3d_tv_padmm.py:96-120): f = 0,
 * A = VerticalStack((C, alpha D)), B = -I, c = 0,
 * g = SeparableFunctional((SquaredL2Loss(y, scale), (lam / alpha) L21Norm)),
 * C the 2D or 3D projector, D = FiniteDifference(append=0) over all axes.
 * Iteration (_padmm.py:349-363):
 *   x <- x - (1/mu) A^T(2u - u_old);  z <- prox_{g/(rho nu)}(z + (1/nu)(A x - z + u));
 *   u <- u + A x - z
 * in float32 with the reference's scalars rounded to float32, residuals in
 * float64.  itstat: maxiter x 3 doubles {objective g0(z0) + g1(z1),
 * primal ||A x - z||, dual ||z - z_old||}.
 */
typedef struct ct_padmm_tv_desc {
  int32_t nd;          /* 2: geom2 (XRayTransform2D); 3: geom3 (XRayTransform3D) */
  ct_geom2d geom2;
  ct_geom3d geom3;
  int32_t maxiter;     /* iterations per call                                    */
  double lam;          /* g1 = (lam / alpha) ||z1||_{2,1}                         */
  double alpha;        /* weight of D in A                                        */
  double rho, mu, nu;  /* penalty; mu > ||A||^2, nu > ||B||^2 = 1                 */
  double loss_scale;   /* g0 = loss_scale ||y - z0||^2 (0.5)                      */
  int32_t use_graph;   /* 1: one iteration captured once as a graph and replayed */
} ct_padmm_tv_desc;

ct_status ct_padmm_tv_workspace(const ct_padmm_tv_desc* d, size_t* bytes);
/* Byte offsets in the workspace of the state blocks z0 (sinogram-shaped),
 * z1 (nd x image), u0, u1 (float32). */
ct_status ct_padmm_tv_state(const ct_padmm_tv_desc* d, size_t* z0_offset,
                            size_t* z1_offset, size_t* u0_offset,
                            size_t* u1_offset);
/* cont = 0: start from z = u = u_old = 0 and the given x; 1: continue from
 * the workspace's state (x must be the previous call's result). */
ct_status ct_padmm_tv_solve(const ct_padmm_tv_desc* d, const float* y, float* x,
                            double* itstat_dev, int32_t cont, void* workspace,
                            size_t workspace_bytes, ct_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* CTGPU_H */
