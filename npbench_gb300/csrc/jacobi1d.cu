// 1D 3-point Jacobi time loop (polybench/jacobi_1d/jacobi_1d_numpy.py:4-8).
//
// Per interior point, in the reference's order:
//   dst[i] = 0.33333 * ((src[i-1] + src[i]) + src[i+1])
// for t in 1..TSTEPS-1: A -> B, then B -> A.
//
// The arrays are small (NPBench's presets go up to 34000 points), so a plain
// one-launch-per-half-sweep loop is bound by launch latency.  Instead each
// launch performs up to H half-sweeps with temporal blocking: a CTA stages its
// segment of w points plus H halo points on each side into shared memory, runs
// the half-sweeps there (the valid region shrinks by one point per side and
// half-sweep, so every kept value is computed exactly as the reference
// computes it), and writes back its segment of both arrays: A holds the state
// after the launch's last half-sweep and B the one before, exactly what the
// reference leaves after the same number of half-sweeps.  Points 0 and n-1
// are never written, in either array.
//
// The arithmetic runs on the small binary64 pipe and each half-sweep is one
// dependent chain per point followed by a CTA barrier, so the launch shape
// trades latency hiding (more CTAs per SM, one point per thread) against the
// redundant halo work (2H points per segment): NPBGB_CFG_JACOBI1D_CTAS (CTAs
// per SM) and NPBGB_CFG_JACOBI1D_DEPTH (H) choose it; the block has one thread
// per staged point, up to 1024.
#include "npbgb_common.cuh"

namespace npbgb {

extern int64_t g_cfg_jacobi1d_ctas;
extern int64_t g_cfg_jacobi1d_depth;
int64_t jacobi1d_effective_depth();
int64_t jacobi1d_effective_ctas();

namespace {

constexpr int kMaxThreads = 1024;
constexpr int kMaxDepth = 64;
// Measured on GB300 at N=32000, TSTEPS=4000 (ms per call): depth 16 / 32 / 48
// / 64 with one CTA per SM 3.72 / 3.19 / 3.13 / 3.18.  More CTAs per SM add
// halo work without gaining speed (2 per SM 3.62 without PDL).
constexpr int kDefaultDepth = 48, kDefaultCtas = 1;

template <typename T>
__global__ void __launch_bounds__(kMaxThreads)
jacobi1d_block(T* __restrict__ a, T* __restrict__ b, int64_t n, int steps, int w, int halo) {
  pdl_begin();
  extern __shared__ __align__(16) unsigned char jac1_smem[];
  const int span = w + 2 * halo;  // staged points per CTA
  T* buf0 = reinterpret_cast<T*>(jac1_smem);
  T* buf1 = buf0 + span;
  const T k = T(0.33333);
  const int64_t seg = int64_t(blockIdx.x) * w;        // first written point - 1 (interior starts at 1)
  const int64_t base = 1 + seg - halo;                // global index of buf[.][0]
  const int nt = int(blockDim.x);
  // Stage A (state h) into buf0 and B into buf1; points outside [0, n) are unused.
  for (int q = threadIdx.x; q < span; q += nt) {
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
    for (int q = s + 1 + threadIdx.x; q < span - 1 - s; q += nt) {
      const int64_t g = base + q;
      if (g >= 1 && g < n - 1) dst[q] = mul_rn(k, add_rn(add_rn(src[q - 1], src[q]), src[q + 1]));
    }
    __syncthreads();
  }
  // steps is even: buf0 holds the newest field (A) and buf1 the one before (B).
  for (int q = halo + threadIdx.x; q < halo + w; q += nt) {
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
  // H half-sweeps per launch (even) and H halo points per side; segments of w
  // points, ctas per SM, at least 32 points, and at most what keeps both
  // staged copies within the default 48 KB of dynamic shared memory (larger
  // arrays get more CTAs).
  const int halo = int(jacobi1d_effective_depth());
  const int ctas = int(jacobi1d_effective_ctas());
  const int64_t w_max = int64_t(48 * 1024 / (2 * sizeof(T))) - 2 * halo;
  int64_t w = cdiv(n - 2, int64_t(sm_count()) * ctas);
  if (w < 32) w = 32;
  if (w > w_max) w = w_max;
  const int64_t blocks = cdiv(n - 2, w);
  if (blocks > 0x7fffffff) return set_error(NPBGB_ERR_ARG, "jacobi1d: extent too large");
  const int64_t span = w + 2 * halo;
  int64_t threads = cdiv(span - 2, 32) * 32;  // one thread per point of the first half-sweep
  if (threads > kMaxThreads) threads = kMaxThreads;
  const size_t smem = 2 * size_t(span) * sizeof(T);
  int64_t left = 2 * int64_t(tsteps - 1);  // half-sweeps, even
  cudaError_t e = cudaSuccess;
  while (left > 0 && e == cudaSuccess) {
    const int s = int(left < halo ? left : halo);
    // With more CTAs than SMs, letting the next launch's CTAs become resident
    // early (PDL) measured 3x slower (10.5 against 3.6 ms at 2 per SM), so
    // those shapes launch in plain stream order.
    e = launch_chained_if(blocks <= sm_count(), jacobi1d_block<T>, dim3{unsigned(blocks)},
                          dim3{unsigned(threads)}, smem, st, a, b, n, s, int(w), halo);
    left -= s;
  }
  return cuda_status(e, "jacobi1d_block");
}

}  // namespace

int64_t jacobi1d_effective_depth() { return g_cfg_jacobi1d_depth > 0 ? g_cfg_jacobi1d_depth : kDefaultDepth; }
int64_t jacobi1d_effective_ctas() { return g_cfg_jacobi1d_ctas > 0 ? g_cfg_jacobi1d_ctas : kDefaultCtas; }

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
