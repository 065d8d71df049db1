// Arithmetic pipe throughput probes: the compute roofs the binary64 stencils
// are stated against.
//
// GB300's binary64 pipe retires far fewer operations per clock than its
// binary32 and integer pipes, so the binary64 kernels here are bound by
// arithmetic issue, not by HBM.  Each probe kernel runs kChains independent
// dependency chains of one instruction kind per thread, over enough CTAs to
// fill every SM, so the measured time is the pipe's throughput: operations
// per second = threads * kChains * iters / time.  The chains depend on a
// kernel argument, so nothing is folded at compile time, and a sink store
// keeps the results live.
#include "npbgb_common.cuh"

namespace npbgb {
namespace {

constexpr int kChains = 8;
constexpr int kProbeThreads = 256;

enum Op : int32_t {
  kDadd = 0,   // binary64 add (round to nearest)
  kDmul = 1,   // binary64 multiply
  kDfma = 2,   // binary64 fused multiply-add
  kFfma = 3,   // binary32 fused multiply-add
  kLop3 = 4,   // 32-bit three-input logic (integer ALU pipe)
  kIadd = 5,   // 32-bit add (integer ALU pipe)
  kImad = 6,   // 32-bit multiply-add
  kOps = 7
};

__device__ __forceinline__ uint32_t lop3(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t d;
  asm volatile("lop3.b32 %0, %1, %2, %3, 0x96;" : "=r"(d) : "r"(a), "r"(b), "r"(c));  // a^b^c
  return d;
}
__device__ __forceinline__ uint32_t iadd(uint32_t a, uint32_t b) {
  uint32_t d;
  asm volatile("add.u32 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b));
  return d;
}
__device__ __forceinline__ uint32_t imad(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t d;
  asm volatile("mad.lo.u32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
  return d;
}

template <int OP>
__global__ void __launch_bounds__(kProbeThreads) pipe_probe(int64_t iters, double seed,
                                                            double* sink) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  if constexpr (OP == kDadd || OP == kDmul || OP == kDfma) {
    double x[kChains];
    const double y = seed * 1e-9 + 1.0, z = seed * 1e-12;
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = seed + c + tid * 1e-6;
    for (int64_t i = 0; i < iters; ++i) {
#pragma unroll
      for (int c = 0; c < kChains; ++c) {
        if constexpr (OP == kDadd) x[c] = __dadd_rn(x[c], z);
        else if constexpr (OP == kDmul) x[c] = __dmul_rn(x[c], y);
        else x[c] = __fma_rn(x[c], y, z);
      }
    }
    double s = 0;
#pragma unroll
    for (int c = 0; c < kChains; ++c) s += x[c];
    if (s == 1234.5678) sink[tid] = s;
  } else if constexpr (OP == kFfma) {
    float x[kChains];
    const float y = float(seed) * 1e-9f + 1.0f, z = float(seed) * 1e-12f;
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = float(seed) + c + tid * 1e-6f;
    for (int64_t i = 0; i < iters; ++i) {
#pragma unroll
      for (int c = 0; c < kChains; ++c) x[c] = __fmaf_rn(x[c], y, z);
    }
    float s = 0;
#pragma unroll
    for (int c = 0; c < kChains; ++c) s += x[c];
    if (s == 1234.5678f) sink[tid] = s;
  } else {
    uint32_t x[kChains];
    const uint32_t y = static_cast<uint32_t>(seed) | 1u, z = static_cast<uint32_t>(seed) >> 3;
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = uint32_t(tid * 2654435761u + c);
    for (int64_t i = 0; i < iters; ++i) {
#pragma unroll
      for (int c = 0; c < kChains; ++c) {
        if constexpr (OP == kLop3) x[c] = lop3(x[c], y, z);
        else if constexpr (OP == kIadd) x[c] = iadd(x[c], y);
        else x[c] = imad(x[c], y, z);
      }
    }
    uint32_t s = 0;
#pragma unroll
    for (int c = 0; c < kChains; ++c) s ^= x[c];
    if (s == 0x12345678u) sink[tid] = double(s);
  }
}

using ProbeFn = void (*)(int64_t, double, double*);
const ProbeFn kProbes[kOps] = {pipe_probe<kDadd>, pipe_probe<kDmul>, pipe_probe<kDfma>,
                               pipe_probe<kFfma>, pipe_probe<kLop3>, pipe_probe<kIadd>,
                               pipe_probe<kImad>};

}  // namespace
}  // namespace npbgb

// Launches probe `op` (0 DADD, 1 DMUL, 2 DFMA, 3 FFMA, 4 LOP3, 5 IADD, 6 IMAD)
// with `ctas` CTAs of 256 threads, each thread running 8 chains of `iters`
// operations; the caller times it.  `sink` must hold ctas * 256
// doubles (written only in the impossible case that defeats dead-code removal).
extern "C" int32_t npbgb_probe_pipe(int32_t op, int64_t iters, int32_t ctas, void* sink,
                                    void* stream) {
  using namespace npbgb;
  if (op < 0 || op >= kOps) return set_error(NPBGB_ERR_ARG, "probe: op %d", op);
  if (iters < 1 || ctas < 1 || !sink) return set_error(NPBGB_ERR_ARG, "probe: iters, ctas, sink");
  kProbes[op]<<<dim3(unsigned(ctas)), dim3(kProbeThreads), 0, as_stream(stream)>>>(
      iters, 3.0 + op, static_cast<double*>(sink));
  NPBGB_CHECK_LAUNCH("probe");
  return NPBGB_OK;
}
