// Library identification, status/error text and host-side geometry tables.
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "common.cuh"

namespace ct {

static thread_local char g_last_error[512] = "";

ct_status fail(ct_status s, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
  return s;
}

ct_status cuda_check(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return CT_OK;
  return fail(CT_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

ct_status launch_check(const char* what) { return cuda_check(cudaGetLastError(), what); }

bool dependent_launch_enabled() {
  static const bool on = [] {
    const char* v = getenv("CTGPU_PDL");
    return !(v && v[0] == '0');
  }();
  return on;
}

int sm_count() {
  static int cached[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
  if (cached[dev] == 0) {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
      n = 152;
    cached[dev] = n;
  }
  return cached[dev];
}

}  // namespace ct

extern "C" {

const char* ct_version(void) { return "ctgpu 0.1.0 sm_103a"; }

const char* ct_status_string(ct_status s) {
  switch (s) {
    case CT_OK: return "ok";
    case CT_ERR_INVALID_ARG: return "invalid argument";
    case CT_ERR_SHAPE: return "shape mismatch";
    case CT_ERR_UNSUPPORTED: return "unsupported";
    case CT_ERR_CUDA: return "CUDA error";
    case CT_ERR_TIMEOUT: return "device wait timed out";
    case CT_ERR_NONFINITE: return "non-finite value";
    case CT_ERR_WORKSPACE: return "workspace too small or misaligned";
    case CT_ERR_NO_DEVICE: return "no CUDA device";
  }
  return "unknown status";
}

const char* ct_last_error(void) { return ct::g_last_error; }

size_t ct_reduce_workspace(void) { return ct::kReduceWorkspace; }

// Host float32 restatement of XRayTransform2D._calc_weights' per-view scalars
// (scico/linop/xray/_xray2d.py:326-347).  Built with -ffp-contract=off so
// every operation rounds to float32 exactly as written.  cos/sin are the
// correctly rounded float32 values of the float32 angle.
ct_status ct_proj2d_views(const float* angles, int32_t n_views, float x0_0, float x0_1,
                          float dx0, float dx1, float y0, float* views_out,
                          float* max_width_out) {
  if (!angles || !views_out) return ct::fail(CT_ERR_INVALID_ARG, "ct_proj2d_views: null pointer");
  if (n_views <= 0) return ct::fail(CT_ERR_INVALID_ARG, "ct_proj2d_views: n_views=%d", n_views);
  float max_width = 0.0f;
  for (int32_t v = 0; v < n_views; ++v) {
    const float a = angles[v];
    const float u0 = (float)cos((double)a);
    const float u1 = (float)sin((double)a);
    const float t0 = x0_0 * u0;
    const float t1 = x0_1 * u1;
    const float t01 = t0 + t1;
    const float px0 = t01 - y0;
    const float pd0 = dx0 * u0;
    const float pd1 = dx1 * u1;
    const float c1 = px0 + pd0;
    const float c2 = px0 + pd1;
    const float c3 = c1 + pd1;
    float pxmin = px0;
    if (c1 < pxmin) pxmin = c1;
    if (c2 < pxmin) pxmin = c2;
    if (c3 < pxmin) pxmin = c3;
    const float s = pd0 + pd1;
    const float d = pd0 - pd1;
    const float diag1 = fabsf(s);
    const float diag2 = fabsf(d);
    const float wmax = diag1 > diag2 ? diag1 : diag2;
    const float wmin = diag1 > diag2 ? diag2 : diag1;
    const float wsum = wmax + wmin;
    const float width = wsum / 2.0f;
    if (!(width > 0.0f) || !isfinite(width) || !isfinite(pxmin))
      return ct::fail(CT_ERR_INVALID_ARG, "ct_proj2d_views: degenerate view %d (width %g)", v,
                      (double)width);
    float* o = views_out + (size_t)v * CT_VIEW2D_STRIDE;
    o[0] = pxmin;
    o[1] = pd0;
    o[2] = pd1;
    o[3] = width;
    o[4] = 1.0f / width;
    o[5] = 0.0f;
    o[6] = 0.0f;
    o[7] = 0.0f;
    if (wmax > max_width) max_width = wmax;
  }
  if (max_width_out) *max_width_out = max_width;
  return CT_OK;
}

}  // extern "C"
