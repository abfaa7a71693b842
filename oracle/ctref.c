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
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
  int rows, cols, nv, det;
  const float* views; /* nv x 8: Pxmin, Pdx0, Pdx1, width, ... */
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

static inline void weight_of(const float* v, int i, int j, int* key, float* w) {
  const float px = (v[0] + v[1] * (float)i) + v[2] * (float)j;
  const float fl = floorf(px);
  *key = (int)fl;
  const float dist = 1.0f - (px - fl);
  const float width = v[3];
  *w = (dist < width ? dist : width) / width;
}

/* 1: accumulate the projector sums in float64 and round once (the same
 * operator with different rounding: used to measure how sensitive a solve is
 * to float32 summation order). */
static int g_proj64 = 0;
void ref_set_proj64(int on) { g_proj64 = on; }

static void proj2d_fwd64(const ref_geom* g, const float* x, float* y) {
  const int R = g->rows, C = g->cols, D = g->det;
#pragma omp parallel
  {
    double* acc = (double*)malloc(sizeof(double) * (size_t)D);
#pragma omp for schedule(dynamic, 1)
    for (int a = 0; a < g->nv; ++a) {
      const float* v = g->views + 8 * (size_t)a;
      for (int b = 0; b < D; ++b) acc[b] = 0.0;
      for (int i = 0; i < R; ++i)
        for (int j = 0; j < C; ++j) {
          int k;
          float w;
          weight_of(v, i, j, &k, &w);
          const double xv = x[(size_t)i * C + j];
          if (k >= 0 && k < D) acc[k] += xv * w;
          if (k + 1 >= 0 && k + 1 < D) acc[k + 1] += xv * (1.0f - w);
        }
      for (int b = 0; b < D; ++b) y[(size_t)a * D + b] = (float)acc[b];
    }
    free(acc);
  }
}

static void proj2d_adj64(const ref_geom* g, const float* y, float* x) {
  const int R = g->rows, C = g->cols, D = g->det;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < R; ++i)
    for (int j = 0; j < C; ++j) {
      double s = 0.0;
      for (int a = 0; a < g->nv; ++a) {
        const float* v = g->views + 8 * (size_t)a;
        int k;
        float w;
        weight_of(v, i, j, &k, &w);
        const float* ya = y + (size_t)a * D;
        if (k >= 0 && k < D) s += (double)ya[k] * w;
        if (k + 1 >= 0 && k + 1 < D) s += (double)ya[k + 1] * (1.0f - w);
      }
      x[(size_t)i * C + j] = (float)s;
    }
}

/* y = A x: the two scatter-adds per view, in update order (:254-263). */
void ref_proj2d_fwd(const ref_geom* g, const float* x, float* y) {
  const int R = g->rows, C = g->cols, D = g->det;
  if (g_proj64) {
    proj2d_fwd64(g, x, y);
    return;
  }
#pragma omp parallel for schedule(dynamic, 1)
  for (int a = 0; a < g->nv; ++a) {
    const float* v = g->views + 8 * (size_t)a;
    float* ya = y + (size_t)a * D;
    for (int b = 0; b < D; ++b) ya[b] = 0.0f;
    for (int pass = 0; pass < 2; ++pass)
      for (int i = 0; i < R; ++i)
        for (int j = 0; j < C; ++j) {
          int k;
          float w;
          weight_of(v, i, j, &k, &w);
          const int kk = k + pass;
          if (kk >= 0 && kk < D) ya[kk] += x[(size_t)i * C + j] * (pass ? 1.0f - w : w);
        }
  }
}

/* x = A^T y: masked gathers summed over views, then the two sums added
 * (:293-306). */
void ref_proj2d_adj(const ref_geom* g, const float* y, float* x) {
  const int R = g->rows, C = g->cols, D = g->det;
  if (g_proj64) {
    proj2d_adj64(g, y, x);
    return;
  }
#pragma omp parallel for schedule(static)
  for (int i = 0; i < R; ++i)
    for (int j = 0; j < C; ++j) {
      float s1 = 0.0f, s2 = 0.0f;
      for (int a = 0; a < g->nv; ++a) {
        const float* v = g->views + 8 * (size_t)a;
        int k;
        float w;
        weight_of(v, i, j, &k, &w);
        const float* ya = y + (size_t)a * D;
        if (k >= 0 && k < D) s1 += ya[k] * w;
        if (k + 1 >= 0 && k + 1 < D) s2 += ya[k + 1] * (1.0f - w);
      }
      x[(size_t)i * C + j] = s1 + s2;
    }
}

/* d = D x, (2, R, C), append=0 (_diff.py:259-266). */
void ref_fd_fwd(int R, int C, const float* x, float* d) {
  const size_t N = (size_t)R * C;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < R; ++i)
    for (int j = 0; j < C; ++j) {
      const size_t e = (size_t)i * C + j;
      const float xc = x[e];
      d[e] = (i < R - 1 ? x[e + C] : xc) - xc;
      d[N + e] = (j < C - 1 ? x[e + 1] : xc) - xc;
    }
}

/* x = D^T d (blocks summed in axis order). */
void ref_fd_adj(int R, int C, const float* d, float* x) {
  const size_t N = (size_t)R * C;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < R; ++i)
    for (int j = 0; j < C; ++j) {
      const size_t e = (size_t)i * C + j;
      const float lo0 = i >= 1 ? d[e - C] : 0.0f, hi0 = i <= R - 2 ? d[e] : 0.0f;
      const float lo1 = j >= 1 ? d[N + e - 1] : 0.0f, hi1 = j <= C - 2 ? d[N + e] : 0.0f;
      x[e] = (lo0 - hi0) + (lo1 - hi1);
    }
}

static void l21_prox(size_t n, const float* v, float thr, float* z) {
#pragma omp parallel for schedule(static)
  for (size_t e = 0; e < n; ++e) {
    const float v0 = v[e], v1 = v[n + e];
    const float len = sqrtf(v0 * v0 + v1 * v1);
    float nl = len - thr;
    nl = 0.5f * (nl + fabsf(nl));
    z[e] = nl * (len != 0.0f ? v0 / len : 0.0f);
    z[n + e] = nl * (len != 0.0f ? v1 / len : 0.0f);
  }
}

/* 0: float32 dot products as the reference computes them; 1: float64
 * products and sums (the GPU solver's precision policy). */
static int g_dot64 = 0;
void ref_set_dot64(int on) { g_dot64 = on; }

static double dotf(size_t n, const float* a, const float* b) {
  if (g_dot64) {
    double s = 0.0;
    for (size_t e = 0; e < n; ++e) s += (double)a[e] * (double)b[e];
    return s;
  }
  float s = 0.0f;
  for (size_t e = 0; e < n; ++e) s += a[e] * b[e];
  return s;
}

static float as_f(double v) { return (float)v; }

static double dotd(size_t n, const float* a, const float* b) {
  double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
  for (size_t e = 0; e < n; ++e) s += (double)a[e] * (double)b[e];
  return s;
}

typedef struct {
  const ref_geom* g;
  float rho, c;
  float *t_sino, *t_img, *t_d;
} lhs_ctx;

/* lhs(v) = rho D^T D v + c A^T A v (_admmaux.py:222-229). */
static void lhs_apply(const lhs_ctx* L, const float* v, float* out) {
  const int R = L->g->rows, C = L->g->cols;
  const size_t N = (size_t)R * C;
  ref_fd_fwd(R, C, v, L->t_d);
  ref_fd_adj(R, C, L->t_d, out);
  ref_proj2d_fwd(L->g, v, L->t_sino);
  ref_proj2d_adj(L->g, L->t_sino, L->t_img);
#pragma omp parallel for schedule(static)
  for (size_t e = 0; e < N; ++e) out[e] = L->rho * out[e] + L->c * L->t_img[e];
}

/*
 * ADMM-TV (one L2,1 term) for `maxiter` iterations from the state (x, z, u),
 * which the caller owns (z = D x0, u = 0 on the first call).  itstat (may be
 * NULL): maxiter x 5 doubles {objective, primal, dual, cg iters, cg relres}.
 * Returns 0.
 */
int ref_admm_tv(const ref_geom* g, const float* y, float lam, float rho, float scale, int maxiter,
                int cg_maxiter, float cg_tol, float* x, float* z, float* u, double* itstat) {
  const int R = g->rows, C = g->cols;
  const size_t N = (size_t)R * C, S = (size_t)g->nv * g->det;
  float* buf = (float*)malloc(sizeof(float) * (10 * N + 2 * S));
  if (!buf) return -1;
  float *rhs = buf, *r = buf + N, *p = buf + 2 * N, *ap = buf + 3 * N, *timg = buf + 4 * N,
        *aty = buf + 5 * N, *td = buf + 6 * N, *zold = buf + 8 * N;
  float *tsino = buf + 10 * N, *tsino2 = buf + 10 * N + S;
  lhs_ctx L = {g, rho, 2.0f * scale, tsino, timg, td};
  const float c = 2.0f * scale;
  const float thr = (float)((1.0 / (double)rho) * (double)lam);
  for (int it = 0; it < maxiter; ++it) {
    /* compute_rhs (:231-256): A^T y every iteration */
    ref_proj2d_adj(g, y, aty);
    for (size_t e = 0; e < 2 * N; ++e) td[e] = z[e] - u[e];
    ref_fd_adj(R, C, td, rhs);
    for (size_t e = 0; e < N; ++e) rhs[e] = (0.0f + c * aty[e]) + rho * rhs[e];
    /* cg (solver.py:378-400) */
    lhs_apply(&L, x, ap);
    /* float32 policy: every scalar rounds to float32 like the reference's */
    const double bnd = sqrt(dotf(N, rhs, rhs));
    const double bn = g_dot64 ? bnd : (double)sqrtf(as_f(bnd));
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
      const float alpha = g_dot64 ? as_f(num / dotf(N, p, ap)) : as_f(num) / as_f(dotf(N, p, ap));
      for (size_t e = 0; e < N; ++e) {
        x[e] = x[e] + alpha * p[e];
        r[e] = r[e] - alpha * ap[e];
      }
      const double num_old = num;
      num = g_dot64 ? dotf(N, r, r) : (double)as_f(dotf(N, r, r));
      const float beta = g_dot64 ? as_f(num / num_old) : as_f(num) / as_f(num_old);
      for (size_t e = 0; e < N; ++e) p[e] = r[e] + beta * p[e];
      ++ii;
    }
    /* z/u update (:364-378) */
    memcpy(zold, z, sizeof(float) * 2 * N);
    ref_fd_fwd(R, C, x, td);
    for (size_t e = 0; e < 2 * N; ++e) td[e] = td[e] + u[e];
    l21_prox(N, td, thr, z);
    ref_fd_fwd(R, C, x, td);
    for (size_t e = 0; e < 2 * N; ++e) u[e] = (u[e] + td[e]) - z[e];
    /* itstat: objective, primal and dual residuals (:210-295) */
    ref_proj2d_fwd(g, x, tsino2);
    double f = 0.0, gz = 0.0, prim = 0.0;
    for (size_t e = 0; e < S; ++e) {
      const double d = (double)y[e] - (double)tsino2[e];
      f += d * d;
    }
    for (size_t e = 0; e < N; ++e) gz += sqrt((double)z[e] * z[e] + (double)z[N + e] * z[N + e]);
    ref_fd_fwd(R, C, x, td);
    for (size_t e = 0; e < 2 * N; ++e) prim += ((double)td[e] - z[e]) * ((double)td[e] - z[e]);
    for (size_t e = 0; e < 2 * N; ++e) td[e] = z[e] - zold[e];
    ref_fd_adj(R, C, td, timg);
    for (size_t e = 0; e < N; ++e) timg[e] *= rho;
    const double dual = sqrt(dotd(N, timg, timg));
    if (itstat) {
      double* o = itstat + 5 * (size_t)it;
      o[0] = scale * f + lam * gz;
      o[1] = sqrt(rho * prim);
      o[2] = dual;
      o[3] = ii;
      o[4] = sqrt(num) / bn;
    }
  }
  free(buf);
  return 0;
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
static inline void taps3(const float* m, float x0, float x1, float x2, int* u0, int* u1, float w[4]) {
  const float p0 = ((m[0] * x0 + m[1] * x1) + m[2] * x2) + m[3];
  const float p1 = ((m[4] * x0 + m[5] * x1) + m[6] * x2) + m[7];
  const float l0 = p0 - 0.25f, l1 = p1 - 0.25f;
  const float t0 = fminf(ceilf(l0) - l0, 0.5f), t1 = fminf(ceilf(l1) - l1, 0.5f);
  const float s0 = 0.5f - t0, s1 = 0.5f - t1;
  *u0 = (int)floorf(l0);
  *u1 = (int)floorf(l1);
  w[0] = (t0 * t1) * 4.0f; /* (u0,   u1)   */
  w[1] = (s0 * t1) * 4.0f; /* (u0+1, u1)   */
  w[2] = (t0 * s1) * 4.0f; /* (u0,   u1+1) */
  w[3] = (s0 * s1) * 4.0f; /* (u0+1, u1+1) */
}

void ref_proj3d_fwd(const int* shape, const int* det, int nv, const float* mats, const float* x, float* y) {
  const int n0 = shape[0], n1 = shape[1], n2 = shape[2], R = det[0], C = det[1];
#pragma omp parallel for schedule(dynamic, 1)
  for (int v = 0; v < nv; ++v) {
    const float* m = mats + (size_t)v * 8;
    float* yv = y + (size_t)v * R * C;
    for (size_t e = 0; e < (size_t)R * C; ++e) yv[e] = 0.0f;
    for (int i = 0; i < n0; ++i)
      for (int j = 0; j < n1; ++j)
        for (int k = 0; k < n2; ++k) {
          const float xv = x[((size_t)i * n1 + j) * n2 + k];
          int u0, u1;
          float w[4];
          taps3(m, (float)i + 0.5f, (float)j + 0.5f, (float)k + 0.5f, &u0, &u1, w);
          for (int q = 0; q < 4; ++q) {
            const int r = u0 + (q & 1), c = u1 + (q >> 1);
            if (r >= 0 && r < R && c >= 0 && c < C) yv[(size_t)r * C + c] += w[q] * xv;
          }
        }
  }
}

void ref_proj3d_adj(const int* shape, const int* det, int nv, const float* mats, const float* y, float* x) {
  const int n0 = shape[0], n1 = shape[1], n2 = shape[2], R = det[0], C = det[1];
#pragma omp parallel for collapse(2) schedule(static)
  for (int i = 0; i < n0; ++i)
    for (int j = 0; j < n1; ++j)
      for (int k = 0; k < n2; ++k) {
        float acc = 0.0f;
        for (int v = 0; v < nv; ++v) {
          int u0, u1;
          float w[4];
          taps3(mats + (size_t)v * 8, (float)i + 0.5f, (float)j + 0.5f, (float)k + 0.5f, &u0, &u1, w);
          const float* yv = y + (size_t)v * R * C;
          for (int q = 0; q < 4; ++q) {
            const int r = u0 + (q & 1), c = u1 + (q >> 1);
            if (r >= 0 && r < R && c >= 0 && c < C) acc += yv[(size_t)r * C + c] * w[q];
          }
        }
        x[((size_t)i * n1 + j) * n2 + k] = acc;
      }
}
