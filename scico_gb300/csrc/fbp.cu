// Ramp filter of XRayTransform2D.fbp (scico/linop/xray/_xray2d.py:158-221).
//
// Each sinogram row y[0..N) is convolved with the ramp filter of Kak &
// Slaney eq. (61) at tau = 1 -- h(0) = 1/4, h(n) = -1/(pi^2 n^2) for odd n,
// 0 for even n != 0, taps n = -(N-1)/2 .. N-1-(N-1)/2 -- and cropped to the N
// samples aligned with the input:  out[i] = sum_n h(n) y[i - n].  The
// reference evaluates this linear convolution with zero-padded FFTs of
// length 2N-1; here it is summed directly from a shared-memory copy of the
// row (only the centre and odd taps are non-zero), which is exact up to
// float32 rounding and deterministic.
#include <math.h>

#include "common.cuh"

namespace {

constexpr int kFbpThreads = 256;

__global__ void __launch_bounds__(kFbpThreads) k_fbp_rows(const float* __restrict__ y, float* __restrict__ out,
                                                          int N) {
  extern __shared__ float sm[];
  float* row = sm;          // [N]
  float* taps = sm + N;     // taps[m] = -1/(pi^2 m^2) at odd m (index m), m < N
  const float* src = y + (size_t)blockIdx.x * N;
  for (int i = threadIdx.x; i < N; i += kFbpThreads) {
    row[i] = src[i];
    const double m = (double)i;
    taps[i] = (i & 1) ? (float)(-1.0 / (m * m * 9.869604401089358)) : 0.0f;
  }
  __syncthreads();
  const int off = (N - 1) / 2;       // centre tap index
  const int hi = N - 1 - off;        // largest positive offset
  for (int i = threadIdx.x; i < N; i += kFbpThreads) {
    float acc = 0.25f * row[i];
    // n = +m uses y[i - m] (m <= hi); n = -m uses y[i + m] (m <= off)
    for (int m = 1; m <= hi || m <= off; m += 2) {
      const float t = taps[m];
      if (m <= hi && i - m >= 0) acc = fmaf(t, row[i - m], acc);
      if (m <= off && i + m < N) acc = fmaf(t, row[i + m], acc);
    }
    out[(size_t)blockIdx.x * N + i] = acc;
  }
}

}  // namespace

extern "C" {

ct_status ct_fbp_filter(const float* sino, float* out, int32_t n_rows, int32_t det_count,
                        ct_stream_t stream) {
  if (!sino || !out) return ct::fail(CT_ERR_INVALID_ARG, "ct_fbp_filter: null array");
  if (n_rows <= 0 || det_count <= 0)
    return ct::fail(CT_ERR_SHAPE, "ct_fbp_filter: n_rows=%d det_count=%d", n_rows, det_count);
  const size_t smem = 2 * sizeof(float) * (size_t)det_count;
  if (smem > 200u * 1024u)
    return ct::fail(CT_ERR_UNSUPPORTED, "ct_fbp_filter: det_count=%d above %d", det_count,
                    (int)(100u * 1024u / sizeof(float)));
  if (smem > 48u * 1024u) {
    ct_status st = ct::cuda_check(
        cudaFuncSetAttribute(k_fbp_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
        "k_fbp_rows smem attribute");
    if (st != CT_OK) return st;
  }
  k_fbp_rows<<<n_rows, kFbpThreads, smem, ct::as_stream(stream)>>>(sino, out, det_count);
  return ct::launch_check("k_fbp_rows");
}

}  // extern "C"
