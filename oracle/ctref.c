/*
 * ctref.c -- C/OpenMP restatement of scico's CT ADMM-TV path.
 * TEST INFRASTRUCTURE ONLY: the CPU baseline of bench.py and a mid-size
 * checker for the tests; the product never links it.
 *
 * Follows the same scico source lines as oracle/ctref.py, in float32
 * arithmetic (built with -ffp-contract=off, so every operation rounds as
 * written):
 *   projector     scico/linop/xray/_xray2d.py:308-351 (_calc_weights),
 *                 :223-265 (_project), :267-306 (_back_project)
 *   FD (append=0) scico/linop/_diff.py:236-272 and its transpose
 *   L2,1 prox     scico/functional/_norm.py:254-263
 *   CG            scico/solver.py:326-405 (float32 dot products)
 *   ADMM          scico/optimize/_admm.py:334-378 with
 *                 LinearSubproblemSolver (_admmaux.py:205-269) and the
 *                 itstat quantities (:210-295), as scico evaluates them:
 *                 every iteration recomputes A^T y, and the statistics
 *                 apply A, D and D^T again.
 * Threads: OpenMP over views (forward), over image rows (adjoint, FD,
 * vector ops); the thread count is the caller's choice.
 *
 * Built twice from this file: float32 (`real` = float, the reference's
 * default precision) and, with -DCTREF_F64, float64 throughout (`real` =
 * double: geometry, weights, sums and the solver, the restatement of an
 * x64 run of the reference).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifdef CTREF_F64
typedef double real;
#define SQRT sqrt
#define FABS fabs
#define FLOOR floor
#define CEIL ceil
#define FMIN fmin
#else
typedef float real;
#define SQRT sqrtf
#define FABS fabsf
#define FLOOR floorf
#define CEIL ceilf
#define FMIN fminf
#endif

typedef struct {
  int rows, cols, nv, det;
  const real* views; /* nv x 8: Pxmin, Pdx0, Pdx1, width, ... */
} ref_geom;

void ref_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#endif
}

int ref_get_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

static inline void weight_of(const real* v, int i, int j, int* key, real* w) {
  const real px = (v[0] + v[1] * (real)i) + v[2] * (real)j;
  const real fl = FLOOR(px);
  *key = (int)fl;
  const real dist = (real)1.0 - (px - fl);
  const real width = v[3];
  *w = (dist < width ? dist : width) / width;
}

/* 1: accumulate the projector sums in float64 and round once (the same
 * operator with different rounding: used to measure how sensitive a solve is
 * to float32 summation order). */
static int g_proj64 = 0;
void ref_set_proj64(int on) { g_proj64 = on; }

static void proj2d_fwd64(const ref_geom* g, const real* x, real* y) {
  const int R = g->rows, C = g->cols, D = g->det;
#pragma omp parallel
  {
    double* acc = (double*)malloc(sizeof(double) * (size_t)D);
#pragma omp for schedule(dynamic, 1)
    for (int a = 0; a < g->nv; ++a) {
      const real* v = g->views + 8 * (size_t)a;
      for (int b = 0; b < D; ++b) acc[b] = 0.0;
      for (int i = 0; i < R; ++i)
        for (int j = 0; j < C; ++j) {
          int k;
          real w;
          weight_of(v, i, j, &k, &w);
          const double xv = x[(size_t)i * C + j];
          if (k >= 0 && k < D) acc[k] += xv * w;
          if (k + 1 >= 0 && k + 1 < D) acc[k + 1] += xv * ((real)1.0 - w);
        }
      for (int b = 0; b < D; ++b) y[(size_t)a * D + b] = (real)acc[b];
    }
    free(acc);
  }
}

static void proj2d_adj64(const ref_geom* g, const real* y, real* x) {
  const int R = g->rows, C = g->cols, D = g->det;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < R; ++i)
    for (int j = 0; j < C; ++j) {
      double s = 0.0;
      for (int a = 0; a < g->nv; ++a) {
        const real* v = g->views + 8 * (size_t)a;
        int k;
        real w;
        weight_of(v, i, j, &k, &w);
        const real* ya = y + (size_t)a * D;
        if (k >= 0 && k < D) s += (double)ya[k] * w;
        if (k + 1 >= 0 && k + 1 < D) s += (double)ya[k + 1] * ((real)1.0 - w);
      }
      x[(size_t)i * C + j] = (real)s;
    }
}

/* y = A x: the two scatter-adds per view, in update order (:254-263). */
void ref_proj2d_fwd(const ref_geom* g, const real* x, real* y) {
  const int R = g->rows, C = g->cols, D = g->det;
  if (g_proj64) {
    proj2d_fwd64(g, x, y);
    return;
  }
#pragma omp parallel for schedule(dynamic, 1)
  for (int a = 0; a < g->nv; ++a) {
    const real* v = g->views + 8 * (size_t)a;
    real* ya = y + (size_t)a * D;
    for (int b = 0; b < D; ++b) ya[b] = (real)0.0;
    for (int pass = 0; pass < 2; ++pass)
      for (int i = 0; i < R; ++i)
        for (int j = 0; j < C; ++j) {
          int k;
          real w;
          weight_of(v, i, j, &k, &w);
          const int kk = k + pass;
          if (kk >= 0 && kk < D) ya[kk] += x[(size_t)i * C + j] * (pass ? (real)1.0 - w : w);
        }
  }
}

/* x = A^T y: masked gathers summed over views, then the two sums added
 * (:293-306). */
void ref_proj2d_adj(const ref_geom* g, const real* y, real* x) {
  const int R = g->rows, C = g->cols, D = g->det;
  if (g_proj64) {
    proj2d_adj64(g, y, x);
    return;
  }
#pragma omp parallel for schedule(static)
  for (int i = 0; i < R; ++i)
    for (int j = 0; j < C; ++j) {
      real s1 = (real)0.0, s2 = (real)0.0;
      for (int a = 0; a < g->nv; ++a) {
        const real* v = g->views + 8 * (size_t)a;
        int k;
        real w;
        weight_of(v, i, j, &k, &w);
        const real* ya = y + (size_t)a * D;
        if (k >= 0 && k < D) s1 += ya[k] * w;
        if (k + 1 >= 0 && k + 1 < D) s2 += ya[k + 1] * ((real)1.0 - w);
      }
      x[(size_t)i * C + j] = s1 + s2;
    }
}

/* d = D x over every axis of an nd-dimensional array (nd <= 3), append=0
 * (_diff.py:259-266): d_k[e] = x[e + s_k] - x[e], 0 on the last slice along
 * axis k; blocks stacked in axis order (operator/_stack.py:126-129). */
static void fd_fwd_nd(int nd, const int* n, const real* x, real* d) {
  size_t N = 1, st[3];
  for (int k = nd - 1; k >= 0; --k) {
    st[k] = N;
    N *= (size_t)n[k];
  }
#pragma omp parallel for schedule(static)
  for (size_t e = 0; e < N; ++e) {
    const real xc = x[e];
    for (int k = 0; k < nd; ++k) {
      const size_t ik = (e / st[k]) % (size_t)n[k];
      d[(size_t)k * N + e] = (ik + 1 < (size_t)n[k] ? x[e + st[k]] : xc) - xc;
    }
  }
}

/* x = D^T d: per axis lo - hi (d_k[e - s_k] where the index is >= 1, d_k[e]
 * where it is <= n_k - 2), the axes' terms summed in axis order. */
static void fd_adj_nd(int nd, const int* n, const real* d, real* x) {
  size_t N = 1, st[3];
  for (int k = nd - 1; k >= 0; --k) {
    st[k] = N;
    N *= (size_t)n[k];
  }
#pragma omp parallel for schedule(static)
  for (size_t e = 0; e < N; ++e) {
    real acc = (real)0.0;
    for (int k = 0; k < nd; ++k) {
      const size_t ik = (e / st[k]) % (size_t)n[k];
      const real* dk = d + (size_t)k * N;
      const real lo = ik >= 1 ? dk[e - st[k]] : (real)0.0, hi = ik + 2 <= (size_t)n[k] ? dk[e] : (real)0.0;
      acc = k == 0 ? (lo - hi) : acc + (lo - hi);
    }
    x[e] = acc;
  }
}

/* d = D x, (2, R, C), append=0. */
void ref_fd_fwd(int R, int C, const real* x, real* d) {
  const int n[2] = {R, C};
  fd_fwd_nd(2, n, x, d);
}

/* x = D^T d (blocks summed in axis order). */
void ref_fd_adj(int R, int C, const real* d, real* x) {
  const int n[2] = {R, C};
  fd_adj_nd(2, n, d, x);
}

/* L2,1 prox over the nd difference components (_norm.py:254-263 with
 * no_nan_divide, numpy/util.py:302-315): len = sqrt(sum v_k^2),
 * nl = 0.5 (len - thr + |len - thr|), z_k = nl v_k / len (0 where len = 0). */
static void l21_prox(int nd, size_t n, const real* v, real thr, real* z) {
#pragma omp parallel for schedule(static)
  for (size_t e = 0; e < n; ++e) {
    real ss = v[e] * v[e];
    for (int k = 1; k < nd; ++k) ss = ss + v[(size_t)k * n + e] * v[(size_t)k * n + e];
    const real len = SQRT(ss);
    real nl = len - thr;
    nl = (real)0.5 * (nl + FABS(nl));
    for (int k = 0; k < nd; ++k) z[(size_t)k * n + e] = nl * (len != (real)0.0 ? v[(size_t)k * n + e] / len : (real)0.0);
  }
}

/* L1 prox (_norm.py:110-116): sign(v) * 0.5 (|v| - thr + ||v| - thr|). */
static void l1_prox(size_t n, const real* v, real thr, real* z) {
#pragma omp parallel for schedule(static)
  for (size_t e = 0; e < n; ++e) {
    real t = FABS(v[e]) - thr;
    t = (real)0.5 * (t + FABS(t));
    z[e] = (v[e] > (real)0.0 ? (real)1.0 : (v[e] < (real)0.0 ? -(real)1.0 : (real)0.0)) * t;
  }
}

/* 0: float32 dot products as the reference computes them; 1: float64
 * products and sums (the GPU solver's precision policy). */
static int g_dot64 = 0;
void ref_set_dot64(int on) { g_dot64 = on; }

static double dotf(size_t n, const real* a, const real* b) {
  if (g_dot64) {
    double s = 0.0;
    for (size_t e = 0; e < n; ++e) s += (double)a[e] * (double)b[e];
    return s;
  }
  real s = (real)0.0;
  for (size_t e = 0; e < n; ++e) s += a[e] * b[e];
  return s;
}

static real as_f(double v) { return (real)v; }

static double dotd(size_t n, const real* a, const real* b) {
  double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
  for (size_t e = 0; e < n; ++e) s += (double)a[e] * (double)b[e];
  return s;
}

/* The linear operator of the data term and the image shape it acts on. */
typedef struct {
  void (*fwd)(const void* ctx, const real* x, real* y);
  void (*adj)(const void* ctx, const real* y, real* x);
  const void* ctx;
  int nd, n[3];
  size_t N, S; /* image and projection element counts */
} ref_ops;

/* g terms: kind 0 = L2,1 (over the nd difference components), 1 = L1. */
typedef struct {
  int nterms, kind[2];
  real lam[2];
} ref_terms;

typedef struct {
  const ref_ops* A;
  int nterms;
  real rho, c;
  real *t_sino, *t_img, *t_d;
} lhs_ctx;

/* lhs(v) = sum_i rho D^T D v + c A^T A v (_admmaux.py:222-229). */
static void lhs_apply(const lhs_ctx* L, const real* v, real* out) {
  const ref_ops* A = L->A;
  fd_fwd_nd(A->nd, A->n, v, L->t_d);
  fd_adj_nd(A->nd, A->n, L->t_d, out);
  A->fwd(A->ctx, v, L->t_sino);
  A->adj(A->ctx, L->t_sino, L->t_img);
  const real rho = L->rho, c = L->c;
  if (L->nterms == 1) {
#pragma omp parallel for schedule(static)
    for (size_t e = 0; e < A->N; ++e) out[e] = rho * out[e] + c * L->t_img[e];
  } else {
#pragma omp parallel for schedule(static)
    for (size_t e = 0; e < A->N; ++e) out[e] = (rho * out[e] + rho * out[e]) + c * L->t_img[e];
  }
}

/*
 * ADMM with LinearSubproblemSolver for scale ||y - A x||^2 + sum_i lam_i g_i(D x),
 * D = FiniteDifference(append=0) over all axes, one rho for every term, for
 * `maxiter` iterations from the state (x, z_i, u_i), which the caller owns
 * (z_i = D x0, u_i = 0 on the first call; z and u hold the terms' blocks one
 * after another, nd * N floats each).  itstat (may be NULL): maxiter x 5
 * doubles {objective, primal, dual, cg iters, cg relres}.  Returns 0, -1 when
 * out of memory.
 */
static int admm_core(const ref_ops* A, const ref_terms* T, const real* y, real rho, real scale, int maxiter,
                     int cg_maxiter, real cg_tol, real* x, real* z, real* u, double* itstat) {
  const size_t N = A->N, S = A->S, M = (size_t)A->nd * N;
  const int nt = T->nterms;
  real* buf = (real*)malloc(sizeof(real) * (6 * N + (2 + (size_t)nt) * M + 2 * S));
  if (!buf) return -1;
  real *rhs = buf, *r = buf + N, *p = buf + 2 * N, *ap = buf + 3 * N, *timg = buf + 4 * N, *aty = buf + 5 * N;
  real *td = buf + 6 * N, *v = td + M, *zold = v + M;
  real *tsino = zold + (size_t)nt * M, *tsino2 = tsino + S;
  lhs_ctx L = {A, nt, rho, (real)2.0 * scale, tsino, timg, td};
  const real c = (real)2.0 * scale;
  for (int it = 0; it < maxiter; ++it) {
    /* compute_rhs (:231-256): A^T y every iteration, then each term's
     * rho D^T (z_i - u_i) added in term order */
    A->adj(A->ctx, y, aty);
    for (size_t e = 0; e < N; ++e) rhs[e] = (real)0.0 + c * aty[e];
    for (int t = 0; t < nt; ++t) {
      for (size_t e = 0; e < M; ++e) td[e] = z[t * M + e] - u[t * M + e];
      fd_adj_nd(A->nd, A->n, td, timg);
      for (size_t e = 0; e < N; ++e) rhs[e] = rhs[e] + rho * timg[e];
    }
    /* cg (solver.py:378-400) */
    lhs_apply(&L, x, ap);
    /* float32 policy: every scalar rounds to float32 like the reference's.
     * bn = norm(b) (solver.py:380): float32 sqrt of the float32 sum, or the
     * float64 root of the float64 sum */
    const double bb = dotf(N, rhs, rhs);
    const double bn = g_dot64 ? sqrt(bb) : (double)SQRT(as_f(bb));
    for (size_t e = 0; e < N; ++e) {
      r[e] = rhs[e] - ap[e];
      p[e] = r[e];
    }
    double num = g_dot64 ? dotf(N, r, r) : (double)as_f(dotf(N, r, r));
    const double tol2 = g_dot64 ? (cg_tol * bn) * (cg_tol * bn)
                                : (double)(as_f(cg_tol * bn) * as_f(cg_tol * bn));
    int ii = 0;
    while (ii < cg_maxiter && num > tol2) {
      lhs_apply(&L, p, ap);
      const real alpha = g_dot64 ? as_f(num / dotf(N, p, ap)) : as_f(num) / as_f(dotf(N, p, ap));
      for (size_t e = 0; e < N; ++e) {
        x[e] = x[e] + alpha * p[e];
        r[e] = r[e] - alpha * ap[e];
      }
      const double num_old = num;
      num = g_dot64 ? dotf(N, r, r) : (double)as_f(dotf(N, r, r));
      const real beta = g_dot64 ? as_f(num / num_old) : as_f(num) / as_f(num_old);
      for (size_t e = 0; e < N; ++e) p[e] = r[e] + beta * p[e];
      ++ii;
    }
    /* z/u update (:364-378), per term: z_i = prox(D x + u_i, lam_i / rho),
     * u_i = (u_i + D x) - z_i */
    memcpy(zold, z, sizeof(real) * (size_t)nt * M);
    fd_fwd_nd(A->nd, A->n, x, td);
    for (int t = 0; t < nt; ++t) {
      real* zt = z + t * M;
      real* ut = u + t * M;
      const real thr = (real)((1.0 / (double)rho) * (double)T->lam[t]);
      for (size_t e = 0; e < M; ++e) v[e] = td[e] + ut[e];
      if (T->kind[t] == 0)
        l21_prox(A->nd, N, v, thr, zt);
      else
        l1_prox(M, v, thr, zt);
      for (size_t e = 0; e < M; ++e) ut[e] = (ut[e] + td[e]) - zt[e];
    }
    /* itstat: objective, primal and dual residuals (:210-295) */
    A->fwd(A->ctx, x, tsino2);
    double f = 0.0, gz = 0.0, prim = 0.0;
    for (size_t e = 0; e < S; ++e) {
      const double d = (double)y[e] - (double)tsino2[e];
      f += d * d;
    }
    double obj = scale * f;
    for (int t = 0; t < nt; ++t) {
      const real* zt = z + t * M;
      gz = 0.0;
      if (T->kind[t] == 0) {
        for (size_t e = 0; e < N; ++e) {
          double ss = 0.0;
          for (int k = 0; k < A->nd; ++k) ss += (double)zt[(size_t)k * N + e] * zt[(size_t)k * N + e];
          gz += sqrt(ss);
        }
      } else {
        for (size_t e = 0; e < M; ++e) gz += fabs((double)zt[e]);
      }
      obj += T->lam[t] * gz;
    }
    for (int t = 0; t < nt; ++t)
      for (size_t e = 0; e < M; ++e) prim += ((double)td[e] - z[t * M + e]) * ((double)td[e] - z[t * M + e]);
    for (size_t e = 0; e < N; ++e) rhs[e] = (real)0.0; /* rhs is free now: the dual residual sum */
    for (int t = 0; t < nt; ++t) {
      for (size_t e = 0; e < M; ++e) td[e] = z[t * M + e] - zold[t * M + e];
      fd_adj_nd(A->nd, A->n, td, timg);
      for (size_t e = 0; e < N; ++e) rhs[e] = t == 0 ? rho * timg[e] : rhs[e] + rho * timg[e];
    }
    const double dual = sqrt(dotd(N, rhs, rhs));
    if (itstat) {
      double* o = itstat + 5 * (size_t)it;
      o[0] = obj;
      o[1] = sqrt(rho * prim);
      o[2] = dual;
      o[3] = ii;
      o[4] = sqrt(num) / bn;
    }
  }
  free(buf);
  return 0;
}

static void ops2d_fwd(const void* ctx, const real* x, real* y) { ref_proj2d_fwd((const ref_geom*)ctx, x, y); }
static void ops2d_adj(const void* ctx, const real* y, real* x) { ref_proj2d_adj((const ref_geom*)ctx, y, x); }

/*
 * 2D ADMM-TV with one L2,1 term (the benchmark problem) for `maxiter`
 * iterations from the state (x, z, u); z, u are (2, R, C).
 */
int ref_admm_tv(const ref_geom* g, const real* y, real lam, real rho, real scale, int maxiter,
                int cg_maxiter, real cg_tol, real* x, real* z, real* u, double* itstat) {
  ref_ops A = {ops2d_fwd, ops2d_adj, g, 2, {g->rows, g->cols, 1}, (size_t)g->rows * g->cols,
               (size_t)g->nv * g->det};
  ref_terms T = {1, {0, 0}, {lam, (real)0.0}};
  return admm_core(&A, &T, y, rho, scale, maxiter, cg_maxiter, cg_tol, x, z, u, itstat);
}

/* ---------------------------------------------------------------------------
 * 3D projector (XRayTransform3D, scico/linop/xray/_xray3d.py:110-266), any
 * (2,4) matrices, the reference's float32 weights: Px_r = ((M[r][0] x0 +
 * M[r][1] x1) + M[r][2] x2) + M[r][3] at voxel centres, left = Px - 0.25,
 * t = min(ceil(left) - left, 0.5), ul = floor(left), four taps with
 * products of (t, 0.5 - t) times 4, zero off the detector.  The forward
 * runs views in parallel (each thread scatters into its own view), the
 * adjoint voxels in parallel (views summed in order).
 * ------------------------------------------------------------------------- */
static inline void taps3(const real* m, real x0, real x1, real x2, int* u0, int* u1, real w[4]) {
  const real p0 = ((m[0] * x0 + m[1] * x1) + m[2] * x2) + m[3];
  const real p1 = ((m[4] * x0 + m[5] * x1) + m[6] * x2) + m[7];
  const real l0 = p0 - (real)0.25, l1 = p1 - (real)0.25;
  const real t0 = FMIN(CEIL(l0) - l0, (real)0.5), t1 = FMIN(CEIL(l1) - l1, (real)0.5);
  const real s0 = (real)0.5 - t0, s1 = (real)0.5 - t1;
  *u0 = (int)FLOOR(l0);
  *u1 = (int)FLOOR(l1);
  w[0] = (t0 * t1) * (real)4.0; /* (u0,   u1)   */
  w[1] = (s0 * t1) * (real)4.0; /* (u0+1, u1)   */
  w[2] = (t0 * s1) * (real)4.0; /* (u0,   u1+1) */
  w[3] = (s0 * s1) * (real)4.0; /* (u0+1, u1+1) */
}

void ref_proj3d_fwd(const int* shape, const int* det, int nv, const real* mats, const real* x, real* y) {
  const int n0 = shape[0], n1 = shape[1], n2 = shape[2], R = det[0], C = det[1];
#pragma omp parallel for schedule(dynamic, 1)
  for (int v = 0; v < nv; ++v) {
    const real* m = mats + (size_t)v * 8;
    real* yv = y + (size_t)v * R * C;
    for (size_t e = 0; e < (size_t)R * C; ++e) yv[e] = (real)0.0;
    for (int i = 0; i < n0; ++i)
      for (int j = 0; j < n1; ++j)
        for (int k = 0; k < n2; ++k) {
          const real xv = x[((size_t)i * n1 + j) * n2 + k];
          int u0, u1;
          real w[4];
          taps3(m, (real)i + (real)0.5, (real)j + (real)0.5, (real)k + (real)0.5, &u0, &u1, w);
          for (int q = 0; q < 4; ++q) {
            const int r = u0 + (q & 1), c = u1 + (q >> 1);
            if (r >= 0 && r < R && c >= 0 && c < C) yv[(size_t)r * C + c] += w[q] * xv;
          }
        }
  }
}

void ref_proj3d_adj(const int* shape, const int* det, int nv, const real* mats, const real* y, real* x) {
  const int n0 = shape[0], n1 = shape[1], n2 = shape[2], R = det[0], C = det[1];
#pragma omp parallel for collapse(2) schedule(static)
  for (int i = 0; i < n0; ++i)
    for (int j = 0; j < n1; ++j)
      for (int k = 0; k < n2; ++k) {
        real acc = (real)0.0;
        for (int v = 0; v < nv; ++v) {
          int u0, u1;
          real w[4];
          taps3(mats + (size_t)v * 8, (real)i + (real)0.5, (real)j + (real)0.5, (real)k + (real)0.5, &u0, &u1, w);
          const real* yv = y + (size_t)v * R * C;
          for (int q = 0; q < 4; ++q) {
            const int r = u0 + (q & 1), c = u1 + (q >> 1);
            if (r >= 0 && r < R && c >= 0 && c < C) acc += yv[(size_t)r * C + c] * w[q];
          }
        }
        x[((size_t)i * n1 + j) * n2 + k] = acc;
      }
}

typedef struct {
  const int *shape, *det;
  int nv;
  const real* mats;
} geom3d_ctx;

static void ops3d_fwd(const void* ctx, const real* x, real* y) {
  const geom3d_ctx* g = (const geom3d_ctx*)ctx;
  ref_proj3d_fwd(g->shape, g->det, g->nv, g->mats, x, y);
}

static void ops3d_adj(const void* ctx, const real* y, real* x) {
  const geom3d_ctx* g = (const geom3d_ctx*)ctx;
  ref_proj3d_adj(g->shape, g->det, g->nv, g->mats, y, x);
}

/*
 * 3D ADMM-TV (the 3D benchmark problem): g = lam_l21 ||D x||_{2,1} (if
 * lam_l21 != 0) then lam_l1 ||D x||_1 (if lam_l1 != 0), both on the same
 * FiniteDifference, one rho, for `maxiter` iterations from the state
 * (x, z, u); z and u hold one (3, n0, n1, n2) block per term, in that order.
 */
int ref_admm_tv3d(const int* shape, const int* det, int nv, const real* mats, const real* y, real lam_l21,
                  real lam_l1, real rho, real scale, int maxiter, int cg_maxiter, real cg_tol, real* x,
                  real* z, real* u, double* itstat) {
  geom3d_ctx g = {shape, det, nv, mats};
  ref_ops A = {ops3d_fwd, ops3d_adj, &g, 3, {shape[0], shape[1], shape[2]},
               (size_t)shape[0] * shape[1] * shape[2], (size_t)nv * det[0] * det[1]};
  ref_terms T = {0, {0, 0}, {(real)0.0, (real)0.0}};
  if (lam_l21 != (real)0.0) {
    T.kind[T.nterms] = 0;
    T.lam[T.nterms++] = lam_l21;
  }
  if (lam_l1 != (real)0.0) {
    T.kind[T.nterms] = 1;
    T.lam[T.nterms++] = lam_l1;
  }
  if (T.nterms == 0) return -2;
  return admm_core(&A, &T, y, rho, scale, maxiter, cg_maxiter, cg_tol, x, z, u, itstat);
}
