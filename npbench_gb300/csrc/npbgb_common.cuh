// Shared definitions for the libnpbgb CUDA sources (sm_103a only).
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <utility>

#include "../../include/npbgb.h"

namespace npbgb {

// Records a message for npbgb_last_error() and returns `code`.
int32_t set_error(int32_t code, const char* fmt, ...);

// Adds n to the count of kernels the library has put on a stream
// (NPBGB_CFG_LAUNCHES; a batch graph's kernels count at each replay, a launch
// recorded into a caller's graph once, when recorded) and returns the new count.
int64_t add_launches(int64_t n);

// Maps a CUDA error to a status, recording the CUDA message.
inline int32_t cuda_status(cudaError_t e, const char* where) {
  if (e == cudaSuccess) return NPBGB_OK;
  return set_error(NPBGB_ERR_CUDA, "%s: %s", where, cudaGetErrorString(e));
}

#define NPBGB_CHECK_LAUNCH(where)                                      \
  do {                                                                 \
    cudaError_t _e = cudaGetLastError();                               \
    if (_e != cudaSuccess) return ::npbgb::cuda_status(_e, where);     \
    ::npbgb::add_launches(1);                                          \
  } while (0)

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

inline int sm_count() {
  static int n = 0;
  if (n == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n <= 0) n = 152;
  }
  return n;
}

inline int64_t cdiv(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Correctly rounded IEEE operations with no contraction into FMA, so that each
// result is rounded exactly once per source operator, as NumPy's ufuncs do.
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }

// Packed binary32 pairs for Blackwell's f32x2 instructions
// (add/sub/mul.rn.f32x2: two IEEE round-to-nearest operations in one
// instruction, subnormals kept), so each element's result is bit-identical to
// the scalar __fadd_rn / __fsub_rn / __fmul_rn.  Element x is the low half.
struct F2 {
  uint64_t v;
};
__device__ __forceinline__ F2 f2(float a, float b) {
  F2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r.v) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ float f2x(F2 a) { return __uint_as_float(static_cast<uint32_t>(a.v)); }
__device__ __forceinline__ float f2y(F2 a) { return __uint_as_float(static_cast<uint32_t>(a.v >> 32)); }
__device__ __forceinline__ F2 add2(F2 a, F2 b) {
  F2 r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
  return r;
}
__device__ __forceinline__ F2 sub2(F2 a, F2 b) {
  F2 r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
  return r;
}
__device__ __forceinline__ F2 mul2(F2 a, F2 b) {
  F2 r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
  return r;
}
// Programmatic dependent launch (griddepcontrol, sm_90 and later).  Time loops
// issue one short kernel per half-sweep; launched with
// launch_chained(), the next kernel's CTAs are scheduled while the current
// grid drains instead of after it has finished.  Every chained kernel calls
// pdl_begin() first, before touching global memory: it lets its own dependent
// launch early, then waits until the preceding kernel has completed and its
// memory is visible (griddepcontrol.wait), so read-after-write and
// write-after-read between consecutive half-sweeps stay ordered.  Without a
// programmatic predecessor both instructions are no-ops.
__device__ __forceinline__ void pdl_begin() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
}

extern int64_t g_cfg_pdl;  // NPBGB_CFG_PDL

// Passes a launch's status through, counting the launch when it succeeded.
inline cudaError_t counted(cudaError_t e) {
  if (e == cudaSuccess) add_launches(1);
  return e;
}
extern int64_t g_cfg_hdiff_emu;  // NPBGB_CFG_HDIFF_EMU

// allow_pdl = false launches in plain stream order whatever NPBGB_CFG_PDL says
// (for launch shapes where early residency of the next grid measured slower).
template <typename... KArgs, typename... Args>
cudaError_t launch_chained_if(bool allow_pdl, void (*kernel)(KArgs...), dim3 grid, dim3 block,
                              size_t smem, cudaStream_t st, Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = (allow_pdl && g_cfg_pdl) ? 1 : 0;
  return counted(cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...));
}

template <typename... KArgs, typename... Args>
cudaError_t launch_chained(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem,
                           cudaStream_t st, Args&&... args) {
  return launch_chained_if(true, kernel, grid, block, smem, st, std::forward<Args>(args)...);
}

}  // namespace npbgb
