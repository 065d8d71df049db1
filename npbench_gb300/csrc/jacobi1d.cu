// 1D 3-point Jacobi time loop (polybench/jacobi_1d/jacobi_1d_numpy.py:4-8).
//
// Per interior point, in the reference's order:
//   dst[i] = 0.33333 * ((src[i-1] + src[i]) + src[i+1])
// for t in 1..TSTEPS-1: A -> B, then B -> A.
//
// The arrays are small (NPBench's presets go up to 34000 points), so a plain
// one-launch-per-half-sweep loop is bound by launch latency.  Instead each
// launch performs kSteps half-sweeps with temporal blocking: a CTA stages its
// segment of w points (one segment per SM, at least 32) plus kSteps halo
// points on each side into shared
// memory, runs the half-sweeps there (the valid region shrinks by one point
// per side and half-sweep, so every kept value is computed exactly as the
// reference computes it), and writes back its segment of both arrays: A
// holds the state after the launch's last half-sweep and B the one before,
// exactly what the reference leaves after the same number of half-sweeps.
// Points 0 and n-1 are never written, in either array.
#include "npbgb_common.cuh"

namespace npbgb {
namespace {

constexpr int kThreads = 256;
constexpr int kSteps = 32;            // half-sweeps per launch (even)

// w: points written per CTA, chosen per array so that the CTAs cover the SMs
// exactly (the arithmetic is bound by the small binary64 pipe, so an idle SM
// costs and so does an SM with a larger share).  The two staged copies live in
// dynamic shared memory, w + 2*kSteps points each.
template <typename T>
__global__ void __launch_bounds__(kThreads)
jacobi1d_block(T* __restrict__ a, T* __restrict__ b, int64_t n, int steps, int w) {
  pdl_begin();
  extern __shared__ __align__(16) unsigned char jac1_smem[];
  const int span = w + 2 * kSteps;  // staged points per CTA
  T* buf0 = reinterpret_cast<T*>(jac1_smem);
  T* buf1 = buf0 + span;
  const T k = T(0.33333);
  const int64_t seg = int64_t(blockIdx.x) * w;        // first written point - 1 (interior starts at 1)
  const int64_t base = 1 + seg - kSteps;              // global index of buf[.][0]
  // Stage A (state h) into buf0 and B into buf1; points outside [0, n) are unused.
  for (int q = threadIdx.x; q < span; q += kThreads) {
    const int64_t g = base + q;
    const bool in = g >= 0 && g < n;
    buf0[q] = in ? a[g] : T(0);
    buf1[q] = in ? b[g] : T(0);
  }
  __syncthreads();
  // Half-sweep s reads buf[s & 1] and writes buf[(s + 1) & 1] for local points
  // q in [s + 1, span - 1 - s) whose global index is an interior point.
  for (int s = 0; s < steps; ++s) {
    const T* src = (s & 1) ? buf1 : buf0;
    T* dst = (s & 1) ? buf0 : buf1;
    for (int q = s + 1 + threadIdx.x; q < span - 1 - s; q += kThreads) {
      const int64_t g = base + q;
      if (g >= 1 && g < n - 1) dst[q] = mul_rn(k, add_rn(add_rn(src[q - 1], src[q]), src[q + 1]));
    }
    __syncthreads();
  }
  // steps is even: buf0 holds the newest field (A) and buf1 the one before (B).
  for (int q = kSteps + threadIdx.x; q < kSteps + w; q += kThreads) {
    const int64_t g = base + q;
    if (g >= 1 && g < n - 1) {
      a[g] = buf0[q];
      b[g] = buf1[q];
    }
  }
}

template <typename T>
int32_t run(T* a, T* b, int64_t n, int32_t tsteps, cudaStream_t st) {
  if (tsteps <= 1 || n < 3) return NPBGB_OK;
  // One segment per SM: at least 32 points, and at most what keeps both
  // staged copies within the default 48 KB of dynamic shared memory (larger
  // arrays get more CTAs).
  const int64_t w_max = int64_t(48 * 1024 / (2 * sizeof(T))) - 2 * kSteps;
  int64_t w = cdiv(n - 2, sm_count());
  if (w < 32) w = 32;
  if (w > w_max) w = w_max;
  const int64_t blocks = cdiv(n - 2, w);
  if (blocks > 0x7fffffff) return set_error(NPBGB_ERR_ARG, "jacobi1d: extent too large");
  const size_t smem = 2 * size_t(w + 2 * kSteps) * sizeof(T);
  int64_t left = 2 * int64_t(tsteps - 1);  // half-sweeps, even
  cudaError_t e = cudaSuccess;
  while (left > 0 && e == cudaSuccess) {
    const int s = int(left < kSteps ? left : kSteps);
    e = launch_chained(jacobi1d_block<T>, dim3{unsigned(blocks)}, dim3{unsigned(kThreads)}, smem,
                       st, a, b, n, s, int(w));
    left -= s;
  }
  return cuda_status(e, "jacobi1d_block");
}

}  // namespace
}  // namespace npbgb

extern "C" int32_t npbgb_jacobi1d(void* A, void* B, int64_t n, int32_t tsteps, int32_t dtype,
                                  void* stream) {
  using namespace npbgb;
  if (n < 0) return set_error(NPBGB_ERR_ARG, "jacobi1d: negative extent");
  if (tsteps > 1 && n >= 3) {
    if (!A || !B) return set_error(NPBGB_ERR_ARG, "jacobi1d: null array");
    if (A == B) return set_error(NPBGB_ERR_ARG, "jacobi1d: A and B alias");
  }
  if (dtype == NPBGB_F64)
    return run<double>(static_cast<double*>(A), static_cast<double*>(B), n, tsteps, as_stream(stream));
  if (dtype == NPBGB_F32)
    return run<float>(static_cast<float*>(A), static_cast<float*>(B), n, tsteps, as_stream(stream));
  return set_error(NPBGB_ERR_DTYPE, "jacobi1d: dtype %d", dtype);
}
