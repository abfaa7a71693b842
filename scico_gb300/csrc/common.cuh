// Shared helpers of the ctgpu library: status/error recording, launch checks,
// exact float32 arithmetic helpers and the deterministic block reduction.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <utility>

#include "ctgpu.h"

namespace ct {

// Record `s` with a printf-style message for ct_last_error() and return it.
ct_status fail(ct_status s, const char* fmt, ...);
// Map a CUDA error to CT_ERR_CUDA (recording `what`), or CT_OK.
ct_status cuda_check(cudaError_t e, const char* what);
// cudaGetLastError() after a launch.
ct_status launch_check(const char* what);
// Number of SMs of the current device (cached per device).
int sm_count();

inline cudaStream_t as_stream(ct_stream_t s) { return reinterpret_cast<cudaStream_t>(s); }

// ---------------------------------------------------------------------------
// Programmatic dependent launch.  A kernel launched by launch_k with
// dependent = true may be scheduled while its stream predecessor -- always
// one of this library's kernels -- is still finishing, which hides the host
// launch latency between the back-to-back kernels of a CG step (the 512^2 /
// 360-view solve with plain launches: 34.4 -> 21.1 ms).  Every kernel that
// can be launched that way calls grid_dep_wait() before it touches global
// memory: it returns once the predecessor grid has completed and its writes
// are visible (at once for a normal launch), so the kernel sees exactly what
// stream order would give it.  grid_dep_trigger() then lets the kernel's own
// successor be scheduled.  While the stream is being captured into a CUDA
// graph the launch is a normal one: graph kernel nodes already follow one
// another without the host gap, and dependent edges measured no faster there
// (the same solve as one graph: 9.55 ms either way).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void grid_dep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void grid_dep_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// Dependent launches are on unless the environment sets CTGPU_PDL=0
// (read once per process).
bool dependent_launch_enabled();

template <typename... KArgs, typename... Args>
inline cudaError_t launch_k(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                            bool dependent, Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  bool dep = dependent && dependent_launch_enabled();
  if (dep) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cs) != cudaSuccess) {
      (void)cudaGetLastError();  // not an error of the launch: launch normally
      dep = false;
    } else if (cs != cudaStreamCaptureStatusNone) {
      dep = false;
    }
  }
  cfg.attrs = attr;
  cfg.numAttrs = dep ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

__host__ __device__ inline bool aligned(const void* p, size_t a) {
  return (reinterpret_cast<uintptr_t>(p) % a) == 0;
}

inline size_t round_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// 1 when n elements split into float4 quads and every array is 16-B
// aligned: the elementwise kernels then move 128 bits per access.
template <class... P>
inline int quad_ok(size_t n, const P*... ptrs) {
  return (n % 4 == 0 && (aligned(ptrs, 16) && ...)) ? 1 : 0;
}

// ---------------------------------------------------------------------------
// Exact float32 arithmetic.  The projector weights must be computed with the
// same IEEE operations, in the same order, as the reference's float32
// expressions, so the compiler may not contract a*b+c into an FMA there.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }

// Detector position of pixel (i, j) for one view:
// (Pxmin + Pdx0*i) + Pdx1*j, each operation rounded to float32
// (scico/linop/xray/_xray2d.py:331-335).
__device__ __forceinline__ float px2d(float pxmin, float pd0, float pd1, int i, int j) {
  return fadd(fadd(pxmin, fmul(pd0, (float)i)), fmul(pd1, (float)j));
}

// Boxcar weight of the lower of the two bins a pixel lands in:
// w = min(1 - (Px - floor(Px)), width) / width (:348-349).  `inv_width` is
// 1/width rounded to float32; the product differs from the quotient by at
// most one ulp, and w == 1 exactly whenever the footprint fits the bin.
__device__ __forceinline__ void boxcar2d(float px, float width, float inv_width,
                                         int& key, float& w) {
  const float fl = floorf(px);
  key = (int)fl;
  const float dist = fsub(1.0f, fsub(px, fl));
  w = dist < width ? fmul(dist, inv_width) : 1.0f;
}

// Compensated (Kahan) float32 running sum: a thread's partial sum of
// statistics terms (residual norms, objective terms), combined over the grid
// in float64.  The compensation keeps a partial sum of hundreds of float32
// terms within a few units of rounding, as a float64 accumulation would,
// without float64 arithmetic per element (the float64 pipe of this GPU runs
// at a small fraction of the float32 rate).  The CG dot products, which
// steer the iteration, stay float64 per element.
struct KSum {
  float s = 0.0f, c = 0.0f;
  __device__ __forceinline__ void add(float v) {
    const float y = __fsub_rn(v, c);
    const float t = __fadd_rn(s, y);
    c = __fsub_rn(__fsub_rn(t, s), y);
    s = t;
  }
  __device__ __forceinline__ double value() const { return (double)s - (double)c; }
};

// ---------------------------------------------------------------------------
// Deterministic float64 grid reduction of K simultaneous sums.  Every block
// reduces its threads' values (fixed shuffle tree, warps in order) and
// writes K partials to partials[K*blockIdx.x + k]; the last block to finish
// (integer ticket, so which block it is does not affect the value) sums the
// partials with all its threads in a fixed pattern.  The ticket is reset by
// that block, so the sequence can be replayed (e.g. inside a CUDA graph)
// without host involvement.  Returns true in thread 0 of the last block,
// with `out` holding the K totals.
// ---------------------------------------------------------------------------
template <int NT, int K>
__device__ __forceinline__ void block_reduce(double (&v)[K], double (*red)[NT / 32]) {
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
      v[k] = s;
    }
  }
  __syncthreads();
}

// The two halves of the grid reduction.  block_partials: the block's K
// partials (thread 0 writes them).  sum_partials: the K totals over the
// grid's partials, summed with all threads of one block in a fixed pattern;
// valid in thread 0.  The partials are read through L2 (other blocks wrote
// them).
template <int NT, int K>
__device__ __forceinline__ void block_partials(double (&v)[K], double* partials) {
  __shared__ double red[K][NT / 32];
  block_reduce<NT, K>(v, red);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) partials[(size_t)K * blockIdx.x + k] = v[k];
  }
}

// stride: doubles per block in `partials` (K when the block's partials are
// exactly these K sums; larger when they are K of a wider set).
template <int NT, int K>
__device__ __forceinline__ void sum_partials(const double* partials, unsigned int nblocks, double (&out)[K],
                                             unsigned int stride = K) {
  __shared__ double red[K][NT / 32];
  double acc[K];
#pragma unroll
  for (int k = 0; k < K; ++k) acc[k] = 0.0;
  for (unsigned int b = threadIdx.x; b < nblocks; b += NT) {
#pragma unroll
    for (int k = 0; k < K; ++k) acc[k] += __ldcg(partials + (size_t)stride * b + k);
  }
  block_reduce<NT, K>(acc, red);
#pragma unroll
  for (int k = 0; k < K; ++k) out[k] = acc[k];
}

template <int NT, int K>
__device__ __forceinline__ bool grid_reduce_last(double (&v)[K], double* partials, unsigned int* ticket,
                                                 double (&out)[K]) {
  __shared__ bool is_last;
  block_partials<NT, K>(v, partials);
  if (threadIdx.x == 0) {
    __threadfence();
    is_last = (atomicAdd(ticket, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (!is_last) return false;
  __threadfence();
  double acc[K];
  sum_partials<NT, K>(partials, gridDim.x, acc);
  if (threadIdx.x != 0) return false;
#pragma unroll
  for (int k = 0; k < K; ++k) out[k] = acc[k];
  *ticket = 0u;
  return true;
}

// Grid barrier of a cooperative launch (all blocks resident).  `count` is a
// counter that only grows during the launch (reset to 0 before it); the
// k-th barrier of the launch waits until it reaches k * gridDim.x.  The wait
// is bounded: after max_polls polls the block sets bit `err_bit` of *err and
// the barrier returns false, so a block that is never joined ends instead of
// hanging (the launch's results are then void and reported).
__device__ __forceinline__ unsigned int ld_acquire_gpu(const unsigned int* p) {
  unsigned int v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ bool grid_barrier(unsigned int* count, unsigned int target, uint32_t max_polls, int* err,
                                             int err_bit) {
  __shared__ int ok_s;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    __threadfence();
    asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(count) : "memory");
    uint32_t polls = 0;
    while (ld_acquire_gpu(count) < target) {
      if (++polls > max_polls) {
        ok = 0;
        atomicOr(err, err_bit);
        break;
      }
    }
    ok_s = ok;
  }
  __syncthreads();
  return ok_s != 0;
}

// Fixed grid size for reductions (independent of the device, so results are
// reproducible across GPUs).
constexpr int kReduceBlocks = 304;
constexpr int kReduceThreads = 256;
// Workspace layout of one reduction: ticket (256 B aligned) + partials for
// up to four simultaneous sums.
constexpr int kReduceMaxSums = 4;
constexpr size_t kReduceWorkspace = 256 + sizeof(double) * kReduceMaxSums * kReduceBlocks;

}  // namespace ct
